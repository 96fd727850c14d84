// Adjoint estimator of the energy gradient over the ansatz parameters
// (no reference counterpart: the reference evaluates the energy only).
//
// For a parameter a, the log-derivative of the Slater determinant of one
// spin is O_a = d ln det tilde_U / d a = tr(tilde_U^{-1} tilde_D_a), where
// tilde_D_a gathers the rows of D_a = dU/da at the occupied sites as tilde_U
// gathers U (src/MonteCarlo.jl:92-115).  With orthonormal orbitals
// tilde_U^{-1} = U^H W, so with M_a = D_a U^H (N x N, built once on the host)
//
//   O_a = sum_{R occupied} M_a[R, R] + sum_{R' empty} sum_l M_a[R_l, R'] W[R', l]
//
// (R_l = the site holding orbital l; W's rows at occupied sites are unit
// vectors).  That is (N - n) n multiply-adds per parameter and spin, read
// from the W the sweep keeps, so the adjoint needs no second factorisation.
//
// One CTA per walker computes E_L (complex, src/Hamiltonian.jl:762-778
// before its real part is taken) and O_a for both spins, and adds into the
// walker's FP64 sums: w, w E, w O_a, w conj(O_a) E, w conj(O_a) O_b with
// w = Z_mu for the reference acceptance rule (its chain samples |psi|^2 / Z_mu,
// src/MonteCarlo.jl:544-591, so the weight restores |psi|^2) and w = 1 for
// the Metropolis rule.
#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc_device.cuh"
#include "kvmc_internal.h"

namespace kvmc {

namespace {

constexpr int kGradThreads = 256;

template <typename S> struct Cx;  // the complex type a stored scalar widens to
template <> struct Cx<float> { using T = cf; };
template <> struct Cx<double> { using T = cd; };
template <> struct Cx<cf> { using T = cf; };
template <> struct Cx<cd> { using T = cd; };

__device__ __forceinline__ cf widen(float v) { return cf{v, 0.f}; }
__device__ __forceinline__ cd widen(double v) { return cd{v, 0.0}; }
__device__ __forceinline__ cf widen(cf v) { return v; }
__device__ __forceinline__ cd widen(cd v) { return v; }

// Block-wide sums of `n` doubles (n <= 2 + 2 * kMaxGradParams); every thread
// gets the results in out[].  red holds 32 * n doubles.
__device__ void block_sum_vec(double *v, int n, double *red, double *out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < n; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
        for (int k = 0; k < n; ++k) red[warp * n + k] = v[k];
    __syncthreads();
    if (warp == 0)
        for (int k = 0; k < n; ++k) {
            double s = lane < nw ? red[lane * n + k] : 0.0;
            s = warp_sum(s);
            if (lane == 0) out[k] = s;
        }
    __syncthreads();
}

template <typename S>
__global__ void __launch_bounds__(kGradThreads) grad_kernel(DevModel m, DevBatch b, GradModel g, int rule) {
    using C = typename Cx<S>::T;
    using R = typename Real<C>::T;
    const int w = blockIdx.x, N = m.n_sites, P = g.n_params;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    extern __shared__ __align__(16) unsigned char smem[];
    short *kup = reinterpret_cast<short *>(smem);
    short *kdn = kup + N;
    short *loc_up = kdn + N;          // site of orbital l
    short *loc_dn = loc_up + m.n_up;
    short *emp_up = loc_dn + m.n_dn;  // sites without an up spin, in site order
    short *emp_dn = emp_up + N;
    __shared__ double red[32 * (2 + 2 * kMaxGradParams)];
    __shared__ double tot[2 + 2 * kMaxGradParams];
    __shared__ int s_cnt[2];
    __shared__ double s_z;

    for (int s = tid; s < N; s += blockDim.x) {
        const short u = b.kappa_up[(size_t)w * N + s], d = b.kappa_dn[(size_t)w * N + s];
        kup[s] = u;
        kdn[s] = d;
        if (u > 0) loc_up[u - 1] = (short)s;
        if (d > 0) loc_dn[d - 1] = (short)s;
    }
    __syncthreads();
    if (warp < 2) {  // warp 0 lists the sites empty of up spins, warp 1 of down spins
        const short *kap = warp == 0 ? kup : kdn;
        short *emp = warp == 0 ? emp_up : emp_dn;
        int base = 0;
        for (int R0 = 0; R0 < N; R0 += 32) {
            const int Rr = R0 + lane;
            const bool e = Rr < N && kap[Rr] == 0;
            const unsigned bal = __ballot_sync(0xffffffffu, e);
            if (e) emp[base + __popc(bal & ((1u << lane) - 1u))] = (short)Rr;
            base += __popc(bal);
        }
        if (lane == 0) s_cnt[warp] = base;
    }
    __syncthreads();

    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    const S *Wu = reinterpret_cast<const S *>(g.W) + (size_t)w * wblock;
    const S *Wd = Wu + (size_t)N * m.ld_up;
    const S *MT = reinterpret_cast<const S *>(g.MT);  // [P][2][N][N], MT[a][s][R'][R] = M_a,s[R, R']
    const size_t NN = (size_t)N * N;

    // local energy (complex) and Z_mu
    C e{0, 0};
    double zc = 0.0;
    for (int k = tid; k < m.n_bonds; k += blockDim.x) {
        const short2 bd = m.bonds[k];
        const int i = bd.x, j = bd.y;
        const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
        e.x += ((ui != 0) == (uj != 0)) ? (R)0.25 : (R)-0.25;
        if (uj != 0 && di != 0) {
            const C p = cmul(widen(Wu[(size_t)i * m.ld_up + uj - 1]), widen(Wd[(size_t)j * m.ld_dn + di - 1]));
            e.x -= (R)0.5 * p.x;
            e.y -= (R)0.5 * p.y;
        }
        if (ui != 0 && dj != 0) {
            const C p = cmul(widen(Wu[(size_t)j * m.ld_up + ui - 1]), widen(Wd[(size_t)i * m.ld_dn + dj - 1]));
            e.x -= (R)0.5 * p.x;
            e.y -= (R)0.5 * p.y;
        }
        zc += ((ui != 0 && dj != 0) || (uj != 0 && di != 0)) ? 1.0 : 0.0;
    }
    // log-derivatives, both spins
    C acc[kMaxGradParams];
#pragma unroll
    for (int a = 0; a < kMaxGradParams; ++a) acc[a] = C{0, 0};
    for (int spin = 0; spin < 2; ++spin) {
        const int n = spin == 0 ? m.n_up : m.n_dn;
        const int ld = spin == 0 ? m.ld_up : m.ld_dn;
        const short *kap = spin == 0 ? kup : kdn;
        const short *loc = spin == 0 ? loc_up : loc_dn;
        const short *emp = spin == 0 ? emp_up : emp_dn;
        const S *Ws = spin == 0 ? Wu : Wd;
        const int ne = s_cnt[spin];
        // occupied diagonal
        for (int Rr = tid; Rr < N; Rr += blockDim.x) {
            if (kap[Rr] == 0) continue;
#pragma unroll
            for (int a = 0; a < kMaxGradParams; ++a) {
                if (a >= P) break;
                const C v = widen(MT[((size_t)a * 2 + spin) * NN + (size_t)Rr * N + Rr]);
                acc[a].x += v.x;
                acc[a].y += v.y;
            }
        }
        // empty rows of W: l runs fastest so the W reads are contiguous
        const int items = ne * n;
        for (int it = tid; it < items; it += blockDim.x) {
            const int r = it / n, l = it - r * n;
            const int Rp = emp[r];
            const C wv = widen(Ws[(size_t)Rp * ld + l]);
            const size_t off = (size_t)Rp * N + loc[l];
#pragma unroll
            for (int a = 0; a < kMaxGradParams; ++a) {
                if (a >= P) break;
                acc[a] = cfma(widen(MT[((size_t)a * 2 + spin) * NN + off]), wv, acc[a]);
            }
        }
    }
    double v[2 + 2 * kMaxGradParams + 1];
    v[0] = (double)e.x;
    v[1] = (double)e.y;
    for (int a = 0; a < P; ++a) {
        v[2 + 2 * a] = (double)acc[a].x;
        v[3 + 2 * a] = (double)acc[a].y;
    }
    const int nv = 2 + 2 * P;
    block_sum_vec(v, nv, red, tot);
    {
        const double z = block_sum(zc, red);
        if (tid == 0) s_z = z;
    }
    __syncthreads();
    if (tid == 0) {
        const double wt = rule == 0 ? s_z : 1.0;
        const double er = tot[0], ei = tot[1];
        double *sm = g.sums + (size_t)w * g.sum_stride;
        sm[0] += wt;
        sm[1] += wt * er;
        sm[2] += wt * ei;
        double *sO = sm + 3, *sOE = sO + 2 * P, *sOO = sOE + 2 * P;
        for (int a = 0; a < P; ++a) {
            const double oar = tot[2 + 2 * a], oai = tot[3 + 2 * a];
            sO[2 * a] += wt * oar;
            sO[2 * a + 1] += wt * oai;
            // conj(O_a) * E
            sOE[2 * a] += wt * (oar * er + oai * ei);
            sOE[2 * a + 1] += wt * (oar * ei - oai * er);
            for (int c = 0; c < P; ++c) {
                const double obr = tot[2 + 2 * c], obi = tot[3 + 2 * c];
                // conj(O_a) * O_b
                sOO[2 * (a * P + c)] += wt * (oar * obr + oai * obi);
                sOO[2 * (a * P + c) + 1] += wt * (oar * obi - oai * obr);
            }
        }
        if (g.out) {
            double *o = g.out + (size_t)w * (2 + 2 * P);
            for (int k = 0; k < 2 + 2 * P; ++k) o[k] = tot[k];
        }
    }
}

template <typename S>
cudaError_t launch_grad_t(const DevModel &m, const DevBatch &b, const GradModel &g, int rule, cudaStream_t stream) {
    const size_t sm = (size_t)(4 * m.n_sites + m.n_up + m.n_dn) * sizeof(short) + 16;
    grad_kernel<S><<<b.n_walkers, kGradThreads, sm, stream>>>(m, b, g, rule);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_grad(const DevModel &m, const DevBatch &b, const GradModel &g, bool mixed, bool complex_w, int rule,
                        cudaStream_t stream) {
    if (g.n_params < 1 || g.n_params > kMaxGradParams) return cudaErrorInvalidValue;
    if (complex_w) return mixed ? launch_grad_t<cf>(m, b, g, rule, stream) : launch_grad_t<cd>(m, b, g, rule, stream);
    return mixed ? launch_grad_t<float>(m, b, g, rule, stream) : launch_grad_t<double>(m, b, g, rule, stream);
}

}  // namespace kvmc
