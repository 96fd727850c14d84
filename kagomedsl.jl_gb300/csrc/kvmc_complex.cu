// Complex-orbital kernels of libkvmc (sm_103a): the path for a hopping matrix
// with Peierls phases (B != 0, src/Hamiltonian.jl:201-204, :325-327), where U,
// tilde_U and W are complex as in the reference (ComplexF64 throughout,
// src/Hamiltonian.jl:423-425, src/MonteCarlo.jl:181-182).
//
//   refresh_c_kernel   reevaluateW! / tilde_U   src/MonteCarlo.jl:55-115 (FP64 complex)
//   sweep_c_kernel     Carlo.sweep! + update_W! src/MonteCarlo.jl:460-607, :279-292
//                      (plain form: complex FP64 W; mixed form: complex FP32 W)
//   measure_c_kernel   getOL                    src/Hamiltonian.jl:762-778 (real part)
//   ratio_c_kernel, apply_moves_c_kernel: the API / test entry points
//
// The acceptance probability is |ratio|^2 = |W_up[K,l]|^2 |W_down[K',l']|^2
// (src/MonteCarlo.jl:581); the local energy is the real part of its sum.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc_device.cuh"
#include "kvmc_internal.h"

namespace kvmc {

template <typename O> __device__ __forceinline__ O to_out(cd v);
template <> __device__ __forceinline__ cd to_out<cd>(cd v) { return v; }
template <> __device__ __forceinline__ cf to_out<cf>(cd v) { return cf{(float)v.x, (float)v.y}; }

// ---------------------------------------------------------------------------
// Refresh: W = U * tilde_U^{-1}, complex FP64.  One CTA per (walker, spin);
// tilde_U is LU-factorised with partial pivoting in shared memory (n <= 112
// orbitals per spin fit; refresh_c_large_kernel below takes larger n), the
// rows at sites not holding this spin are solved one thread per row from a
// column-major FP64 scratch block.
// ---------------------------------------------------------------------------
constexpr int kThreadsC = 256;
constexpr int kMaxComplexOrbitals = 112;

template <typename OutC>
__global__ void __launch_bounds__(kThreadsC)
refresh_c_kernel(DevModel m, DevBatch b, int only_due, int track_drift) {
    const int w = blockIdx.x, spin = blockIdx.y;
    if (only_due && b.since[w] >= 0) return;
    if (spin == 0 && threadIdx.x == 0) atomicAdd(b.refresh_count, 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const cd *U = reinterpret_cast<const cd *>(spin == 0 ? m.U_up : m.U_dn);
    const short *kappa = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    OutC *W = (sizeof(OutC) == 16 ? reinterpret_cast<OutC *>(b.W64) : reinterpret_cast<OutC *>(b.W32)) +
              (size_t)w * wblock + (spin == 0 ? 0 : (size_t)N * m.ld_up);
    cd *Y = reinterpret_cast<cd *>(b.solve_scratch) + ((size_t)w * 2 + spin) * (b.solve_block / 2);

    extern __shared__ __align__(16) unsigned char smem[];
    const int lda = n + 1;
    cd *A = reinterpret_cast<cd *>(smem);
    cd *invd = A + (size_t)n * lda;
    double *red = reinterpret_cast<double *>(invd + n);
    int *perm = reinterpret_cast<int *>(red + 33);
    short *rows = reinterpret_cast<short *>(perm + n);
    __shared__ int s_piv, s_nrows;
    __shared__ double s_pmax;
    __shared__ cd s_dinv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;

    for (int e = tid; e < n * lda; e += nt) A[e] = cd{0.0, 0.0};
    __syncthreads();
    for (int R = warp; R < N; R += nt / 32) {
        const int l = kappa[R];
        if (l >= 1 && l <= n)
            for (int c = lane; c < n; c += 32) A[(size_t)(l - 1) * lda + c] = U[(size_t)R * n + c];
    }
    for (int i = tid; i < n; i += nt) perm[i] = i;
    __syncthreads();

    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            double best = -1.0;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                const double v = cabs1(A[(size_t)i * lda + k]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) {
                s_piv = bi;
                s_pmax = best;
                s_dinv = best > 0.0 ? cinv(A[(size_t)bi * lda + k]) : cd{0.0, 0.0};
            }
        }
        __syncthreads();
        if (!(s_pmax > 0.0)) {
            if (tid == 0) {
                atomicOr(&b.status[w], kStatusSingular);
                b.logdet[4 * w + spin] = -INFINITY;
                b.logdet[4 * w + 2 + spin] = -INFINITY;
            }
            return;
        }
        const int p = s_piv;
        if (p != k) {
            for (int j = tid; j < n; j += nt) {
                const cd a = A[(size_t)k * lda + j];
                A[(size_t)k * lda + j] = A[(size_t)p * lda + j];
                A[(size_t)p * lda + j] = a;
            }
            if (tid == 0) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
        }
        __syncthreads();
        const cd dinv = s_dinv;
        for (int i = k + 1 + tid; i < n; i += nt) A[(size_t)i * lda + k] = cmul(A[(size_t)i * lda + k], dinv);
        __syncthreads();
        for (int i = k + 1 + warp; i < n; i += nt / 32) {
            const cd aik = A[(size_t)i * lda + k];
            for (int j = k + 1 + lane; j < n; j += 32)
                A[(size_t)i * lda + j] = cfms(aik, A[(size_t)k * lda + j], A[(size_t)i * lda + j]);
        }
        __syncthreads();
    }
    double ld = 0.0, dmin = INFINITY, dmaxp = 0.0;
    for (int i = tid; i < n; i += nt) {
        const cd d = A[(size_t)i * lda + i];
        invd[i] = cinv(d);
        const double mag = hypot(d.x, d.y);
        ld += log(mag);
        dmin = fmin(dmin, mag);
        dmaxp = fmax(dmaxp, mag);
    }
    ld = block_sum(ld, red);
    dmin = -block_sum_max(-dmin, red);
    dmaxp = block_sum_max(dmaxp, red);
    if (tid == 0) {
        b.logdet[4 * w + spin] = ld;
        b.logdet[4 * w + 2 + spin] = log(dmin / dmaxp);
        s_nrows = 0;
    }
    // sites not holding this spin, in site order
    if (warp == 0) {
        int base = 0;
        for (int R0 = 0; R0 < N; R0 += 32) {
            const int R = R0 + lane;
            const bool un = R < N && kappa[R] == 0;
            const unsigned bal = __ballot_sync(0xffffffffu, un);
            if (un) rows[base + __popc(bal & ((1u << lane) - 1u))] = (short)R;
            base += __popc(bal);
        }
        if (lane == 0) s_nrows = base;
    }
    // unit rows at occupied sites, zero padding
    float dmax = 0.f;
    for (int R = warp; R < N; R += nt / 32) {
        const int l = kappa[R];
        OutC *wr = W + (size_t)R * ldw;
        if (l != 0) {
            for (int c = lane; c < ldw; c += 32) {
                const cd nv = cd{c == l - 1 ? 1.0 : 0.0, 0.0};
                if (track_drift) {
                    const OutC o = wr[c];
                    dmax = fmaxf(dmax, (float)(hypot((double)o.x - nv.x, (double)o.y) / (1.0 + hypot(nv.x, nv.y))));
                }
                wr[c] = to_out<OutC>(nv);
            }
        } else {
            for (int c = n + lane; c < ldw; c += 32) wr[c] = to_out<OutC>(cd{0.0, 0.0});
        }
    }
    __syncthreads();
    const int nrows = s_nrows;
    // w * tilde_U = u: forward with Uf, backward with unit L, then w[perm[i]] = v[i]
    for (int r = tid; r < nrows; r += nt) {
        const int R = rows[r];
        cd *y = Y + r;  // column-major: y[j * nrows]
        for (int j = 0; j < n; ++j) y[(size_t)j * nrows] = U[(size_t)R * n + j];
        for (int i = 0; i < n; ++i) {
            const cd yi = cmul(y[(size_t)i * nrows], invd[i]);
            y[(size_t)i * nrows] = yi;
            const cd *Ai = A + (size_t)i * lda;
            for (int j = i + 1; j < n; ++j) y[(size_t)j * nrows] = cfms(yi, Ai[j], y[(size_t)j * nrows]);
        }
        for (int j = n - 1; j > 0; --j) {
            const cd vj = y[(size_t)j * nrows];
            const cd *Aj = A + (size_t)j * lda;
            for (int i = 0; i < j; ++i) y[(size_t)i * nrows] = cfms(vj, Aj[i], y[(size_t)i * nrows]);
        }
        OutC *wr = W + (size_t)R * ldw;
        for (int i = 0; i < n; ++i) {
            const cd nv = y[(size_t)i * nrows];
            if (track_drift) {
                const OutC o = wr[perm[i]];
                dmax = fmaxf(dmax, (float)(hypot((double)o.x - nv.x, (double)o.y - nv.y) / (1.0 + hypot(nv.x, nv.y))));
            }
            wr[perm[i]] = to_out<OutC>(nv);
        }
    }
    if (track_drift) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
    }
}

size_t refresh_c_smem(const DevModel &m) {
    const int n = m.n_up > m.n_dn ? m.n_up : m.n_dn;
    return (size_t)n * (n + 1) * 16 + (size_t)n * 16 + 33 * 8 + (size_t)n * 4 + (size_t)m.n_sites * 2 + 32;
}

// ---------------------------------------------------------------------------
// Refresh beyond 112 orbitals per spin: the same W = U tilde_U^{-1} with
// tilde_U factorised in HBM (lu_scratch, n x n complex per walker-spin) by
// a blocked right-looking LU with partial pivoting whose rows never move
// (row i of the factors is A[perm[i]]): 16-column panels in shared memory,
// the trailing update A22 -= L21 U12 in 2 x 2 complex register tiles
// against 32-column slices of U12 staged in shared memory.  The rows at
// sites not holding this spin are then solved one thread per row as in
// refresh_c_kernel, reading the factors through perm.
// ---------------------------------------------------------------------------
constexpr int kPanelC = 16;
constexpr int kPanelLd = kPanelC + 1;

__device__ __forceinline__ bool lu_c_blocked(cd *A, int n, cd *Pn, cd *Ut, int *perm) {
    __shared__ int s_piv;
    __shared__ double s_pmax;
    __shared__ cd s_dinv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    for (int i = tid; i < n; i += nt) perm[i] = i;
    __syncthreads();
    for (int pb = 0; pb < n; pb += kPanelC) {
        const int nb = min(kPanelC, n - pb);
        const int rp = n - pb;
        for (int e = tid; e < rp * kPanelC; e += nt) {
            const int r = e / kPanelC, c = e - r * kPanelC;
            Pn[(size_t)r * kPanelLd + c] = c < nb ? A[(size_t)perm[pb + r] * n + pb + c] : cd{0.0, 0.0};
        }
        __syncthreads();
        for (int k = 0; k < nb; ++k) {
            if (warp == 0) {
                double best = -1.0;
                int bi = rp;
                for (int i = k + lane; i < rp; i += 32) {
                    const double v = cabs1(Pn[(size_t)i * kPanelLd + k]);
                    if (v > best) { best = v; bi = i; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
                if (lane == 0) {
                    s_piv = bi;
                    s_pmax = best;
                    s_dinv = best > 0.0 ? cinv(Pn[(size_t)bi * kPanelLd + k]) : cd{0.0, 0.0};
                }
            }
            __syncthreads();
            if (!(s_pmax > 0.0)) return false;
            const int p = s_piv;
            if (p != k) {
                for (int j = tid; j < kPanelC; j += nt) {
                    const cd a = Pn[(size_t)k * kPanelLd + j];
                    Pn[(size_t)k * kPanelLd + j] = Pn[(size_t)p * kPanelLd + j];
                    Pn[(size_t)p * kPanelLd + j] = a;
                }
                if (tid == 0) { const int t = perm[pb + k]; perm[pb + k] = perm[pb + p]; perm[pb + p] = t; }
            }
            __syncthreads();
            const cd dinv = s_dinv;
            for (int i = k + 1 + tid; i < rp; i += nt) {
                const cd l = cmul(Pn[(size_t)i * kPanelLd + k], dinv);
                Pn[(size_t)i * kPanelLd + k] = l;
                for (int j = k + 1; j < nb; ++j)
                    Pn[(size_t)i * kPanelLd + j] = cfms(l, Pn[(size_t)k * kPanelLd + j], Pn[(size_t)i * kPanelLd + j]);
            }
            __syncthreads();
        }
        for (int e = tid; e < rp * kPanelC; e += nt) {
            const int r = e / kPanelC, c = e - r * kPanelC;
            if (c < nb) A[(size_t)perm[pb + r] * n + pb + c] = Pn[(size_t)r * kPanelLd + c];
        }
        const int c0 = pb + nb;
        if (c0 < n) {
            // U12 = L11^{-1} A12, one column per thread (nb = kPanelC here);
            // each row is finished in place before the next reads it
            for (int c = c0 + tid; c < n; c += nt) {
                for (int i = 1; i < kPanelC; ++i) {
                    cd *xi = A + (size_t)perm[pb + i] * n + c;
                    cd acc = *xi;
                    for (int k = 0; k < i; ++k)
                        acc = cfms(Pn[(size_t)i * kPanelLd + k], A[(size_t)perm[pb + k] * n + c], acc);
                    *xi = acc;
                }
            }
            __syncthreads();
            // A22 -= L21 U12: 32-column slices of U12, 2 x 2 complex per thread
            const int tx = tid & 15, ty = tid >> 4, rstep = 2 * (nt >> 4);
            for (int cb = c0; cb < n; cb += 32) {
                const int ncol = min(32, n - cb);
                for (int e = tid; e < kPanelC * 32; e += nt) {
                    const int k = e >> 5, c = e & 31;
                    Ut[e] = c < ncol ? A[(size_t)perm[pb + k] * n + cb + c] : cd{0.0, 0.0};
                }
                __syncthreads();
                for (int rb = c0; rb < n; rb += rstep) {
                    cd acc[2][2] = {};
                    int rr[2];
#pragma unroll
                    for (int a = 0; a < 2; ++a) rr[a] = min(rb + 2 * ty + a, n - 1);
#pragma unroll 4
                    for (int k = 0; k < kPanelC; ++k) {
                        const cd l0 = Pn[(size_t)(rr[0] - pb) * kPanelLd + k], l1 = Pn[(size_t)(rr[1] - pb) * kPanelLd + k];
                        const cd u0 = Ut[k * 32 + 2 * tx], u1 = Ut[k * 32 + 2 * tx + 1];
                        acc[0][0] = cfma(l0, u0, acc[0][0]);
                        acc[0][1] = cfma(l0, u1, acc[0][1]);
                        acc[1][0] = cfma(l1, u0, acc[1][0]);
                        acc[1][1] = cfma(l1, u1, acc[1][1]);
                    }
#pragma unroll
                    for (int a = 0; a < 2; ++a) {
                        const int r = rb + 2 * ty + a;
                        if (r >= n) continue;
                        cd *Ar = A + (size_t)perm[r] * n;
#pragma unroll
                        for (int q = 0; q < 2; ++q) {
                            const int c = cb + 2 * tx + q;
                            if (c < n) {
                                const cd o = Ar[c];
                                Ar[c] = cd{o.x - acc[a][q].x, o.y - acc[a][q].y};
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
    return true;
}

template <typename OutC>
__global__ void __launch_bounds__(kThreadsC)
refresh_c_large_kernel(DevModel m, DevBatch b, int only_due, int track_drift) {
    const int w = blockIdx.x, spin = blockIdx.y;
    if (only_due && b.since[w] >= 0) return;
    if (spin == 0 && threadIdx.x == 0) atomicAdd(b.refresh_count, 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const cd *U = reinterpret_cast<const cd *>(spin == 0 ? m.U_up : m.U_dn);
    const short *kappa = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    OutC *W = (sizeof(OutC) == 16 ? reinterpret_cast<OutC *>(b.W64) : reinterpret_cast<OutC *>(b.W32)) +
              (size_t)w * wblock + (spin == 0 ? 0 : (size_t)N * m.ld_up);
    cd *Y = reinterpret_cast<cd *>(b.solve_scratch) + ((size_t)w * 2 + spin) * (b.solve_block / 2);
    cd *A = reinterpret_cast<cd *>(b.lu_scratch + ((size_t)w * 2 + spin) * b.lu_block);

    extern __shared__ __align__(16) unsigned char smem[];
    cd *Pn = reinterpret_cast<cd *>(smem);
    cd *Ut = Pn + (size_t)n * kPanelLd;
    cd *invd = Ut + kPanelC * 32;
    double *red = reinterpret_cast<double *>(invd + n);
    int *perm = reinterpret_cast<int *>(red + 33);
    short *rows = reinterpret_cast<short *>(perm + n);
    __shared__ int s_nrows;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;

    // tilde_U: row l = U at the site holding label l + 1 (rows of labels no
    // site holds stay zero: an exactly singular tilde_U)
    for (int e = tid; e < n * n; e += nt) A[e] = cd{0.0, 0.0};
    __syncthreads();
    for (int R = warp; R < N; R += nt / 32) {
        const int l = kappa[R];
        if (l >= 1 && l <= n)
            for (int c = lane; c < n; c += 32) A[(size_t)(l - 1) * n + c] = U[(size_t)R * n + c];
    }
    __syncthreads();
    if (!lu_c_blocked(A, n, Pn, Ut, perm)) {
        if (tid == 0) {
            atomicOr(&b.status[w], kStatusSingular);
            b.logdet[4 * w + spin] = -INFINITY;
            b.logdet[4 * w + 2 + spin] = -INFINITY;
        }
        return;
    }
    double ld = 0.0, dmin = INFINITY, dmaxp = 0.0;
    for (int i = tid; i < n; i += nt) {
        const cd d = A[(size_t)perm[i] * n + i];
        invd[i] = cinv(d);
        const double mag = hypot(d.x, d.y);
        ld += log(mag);
        dmin = fmin(dmin, mag);
        dmaxp = fmax(dmaxp, mag);
    }
    ld = block_sum(ld, red);
    dmin = -block_sum_max(-dmin, red);
    dmaxp = block_sum_max(dmaxp, red);
    if (tid == 0) {
        b.logdet[4 * w + spin] = ld;
        b.logdet[4 * w + 2 + spin] = log(dmin / dmaxp);
        s_nrows = 0;
    }
    // sites not holding this spin, in site order
    if (warp == 0) {
        int base = 0;
        for (int R0 = 0; R0 < N; R0 += 32) {
            const int R = R0 + lane;
            const bool un = R < N && kappa[R] == 0;
            const unsigned bal = __ballot_sync(0xffffffffu, un);
            if (un) rows[base + __popc(bal & ((1u << lane) - 1u))] = (short)R;
            base += __popc(bal);
        }
        if (lane == 0) s_nrows = base;
    }
    // unit rows at occupied sites, zero padding
    float dmax = 0.f;
    for (int R = warp; R < N; R += nt / 32) {
        const int l = kappa[R];
        OutC *wr = W + (size_t)R * ldw;
        if (l != 0) {
            for (int c = lane; c < ldw; c += 32) {
                const cd nv = cd{c == l - 1 ? 1.0 : 0.0, 0.0};
                if (track_drift) {
                    const OutC o = wr[c];
                    dmax = fmaxf(dmax, (float)(hypot((double)o.x - nv.x, (double)o.y) / (1.0 + hypot(nv.x, nv.y))));
                }
                wr[c] = to_out<OutC>(nv);
            }
        } else {
            for (int c = n + lane; c < ldw; c += 32) wr[c] = to_out<OutC>(cd{0.0, 0.0});
        }
    }
    __syncthreads();
    const int nrows = s_nrows;
    // w * tilde_U = u: forward with Uf, backward with unit L (row i of the
    // factors at A[perm[i]]), then w[perm[i]] = v[i]
    for (int r = tid; r < nrows; r += nt) {
        const int R = rows[r];
        cd *y = Y + r;  // column-major: y[j * nrows]
        for (int j = 0; j < n; ++j) y[(size_t)j * nrows] = U[(size_t)R * n + j];
        for (int i = 0; i < n; ++i) {
            const cd yi = cmul(y[(size_t)i * nrows], invd[i]);
            y[(size_t)i * nrows] = yi;
            const cd *Ai = A + (size_t)perm[i] * n;
            for (int j = i + 1; j < n; ++j) y[(size_t)j * nrows] = cfms(yi, Ai[j], y[(size_t)j * nrows]);
        }
        for (int j = n - 1; j > 0; --j) {
            const cd vj = y[(size_t)j * nrows];
            const cd *Aj = A + (size_t)perm[j] * n;
            for (int i = 0; i < j; ++i) y[(size_t)i * nrows] = cfms(vj, Aj[i], y[(size_t)i * nrows]);
        }
        OutC *wr = W + (size_t)R * ldw;
        for (int i = 0; i < n; ++i) {
            const cd nv = y[(size_t)i * nrows];
            if (track_drift) {
                const OutC o = wr[perm[i]];
                dmax = fmaxf(dmax, (float)(hypot((double)o.x - nv.x, (double)o.y - nv.y) / (1.0 + hypot(nv.x, nv.y))));
            }
            wr[perm[i]] = to_out<OutC>(nv);
        }
    }
    if (track_drift) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
    }
}

size_t refresh_c_large_smem(const DevModel &m) {
    const int n = m.n_up > m.n_dn ? m.n_up : m.n_dn;
    return (size_t)n * kPanelLd * 16 + (size_t)kPanelC * 32 * 16 + (size_t)n * 16 + 33 * 8 + (size_t)n * 4 +
           (size_t)m.n_sites * 2 + 32;
}

// ---------------------------------------------------------------------------
// Sweep with complex W (one walker per CTA, W in global memory).  The same
// proposal window as the real kernels; the acceptance uses
// a = |W_up[K,l]|^2 |W_down[K',l']|^2.
// ---------------------------------------------------------------------------
template <typename C>
struct CPtr {
    C *up, *dn;
    int ld_up, ld_dn;
    __device__ __forceinline__ C &U(int r, int c) const { return up[(size_t)r * ld_up + c]; }
    __device__ __forceinline__ C &D(int r, int c) const { return dn[(size_t)r * ld_dn + c]; }
};

__device__ __forceinline__ bool decide_a(double a, unsigned long long u53, int c, const Thr &T, int rule, bool &bad) {
    if (!isfinite(a)) { bad = true; return false; }
    const double r = r_of(u53);
    if (rule == 0) return a >= 1.0 ? (c < 0) : (r < T.d * a);
    return a >= 1.0 || r < a;
}

__device__ __forceinline__ bool decide_c(cd pu, cd pd, unsigned long long u53, int c, const Thr &T, int rule, bool &bad) {
    const double ratio_abs2 = cabs2(cmul(pu, pd));
    return decide_a(ratio_abs2, u53, c, T, rule, bad);
}

// FP32 complex: the FP32 test with the 1e-5 guard band, FP64 inside it
__device__ __forceinline__ bool decide_c(cf pu, cf pd, unsigned long long u53, int c, const Thr &T, int rule, bool &bad) {
    const cf rt = cmul(pu, pd);
    const float a = cabs2(rt);
    if (isnan(a)) { bad = true; return false; }
    constexpr float band = 1e-5f;
    if (a >= 1.f + band) return rule == 0 ? (c < 0) : true;
    if (a <= 1.f - band) {
        const float x = rule == 0 ? T.f * a : a;
        const float rf = r_f32(u53);
        if (rf < x * (1.f - band)) return true;
        if (rf > x * (1.f + band)) return false;
    }
    const cd r64 = cmul(cd{(double)pu.x, (double)pu.y}, cd{(double)pd.x, (double)pd.y});
    return decide_a(cabs2(r64), u53, c, T, rule, bad);
}

template <typename C>
__device__ double local_energy_c(const DevModel &m, const short *kup, const short *kdn, const CPtr<C> &W, double *red) {
    using R = typename Real<C>::T;
    R acc = 0;
    for (int e = threadIdx.x; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = m.bonds[e];
        const int i = bd.x, j = bd.y;
        const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
        acc += ((ui != 0) == (uj != 0)) ? (R)0.25 : (R)-0.25;
        if (uj != 0 && di != 0) acc -= (R)0.5 * cmul(W.U(i, uj - 1), W.D(j, di - 1)).x;
        if (ui != 0 && dj != 0) acc -= (R)0.5 * cmul(W.U(j, ui - 1), W.D(i, dj - 1)).x;
    }
    if constexpr (sizeof(R) == 4) return block_sum_f32(acc, red);
    else return block_sum(acc, red);
}

template <typename C>
__device__ void rank1_update_c(const CPtr<C> &W, int N, int Ku, int lu, int Kd, int ld, C *cu, C *ru, C *cdn, C *rd) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const C au = cinv(W.U(Ku, lu));
    const C ad = cinv(W.D(Kd, ld));
    for (int r = tid; r < N; r += nt) {
        const C a = cmul(W.U(r, lu), au), d = cmul(W.D(r, ld), ad);
        cu[r] = C{-a.x, -a.y};
        cdn[r] = C{-d.x, -d.y};
    }
    for (int c = tid; c < W.ld_up; c += nt) { C v = W.U(Ku, c); if (c == lu) v.x -= 1; ru[c] = v; }
    for (int c = tid; c < W.ld_dn; c += nt) { C v = W.D(Kd, c); if (c == ld) v.x -= 1; rd[c] = v; }
    __syncthreads();
    const int tot_up = N * W.ld_up, tot = tot_up + N * W.ld_dn;
    for (int e = tid; e < tot; e += nt) {
        const bool is_up = e < tot_up;
        const int ee = is_up ? e : e - tot_up;
        const int q = is_up ? W.ld_up : W.ld_dn;
        const int r = ee / q, c = ee - r * q;
        C *wp = (is_up ? W.up : W.dn) + (size_t)r * q + c;
        *wp = cfma(is_up ? cu[r] : cdn[r], is_up ? ru[c] : rd[c], *wp);
    }
    __syncthreads();
}

struct SweepCtlC {
    long long t, next_meas, next_ref;
    int since, zmu, state;
    int Ku, lu, Kd, ld;
    Thr thr;
    double red[33];
};

template <typename C>
__global__ void __launch_bounds__(256) sweep_c_kernel(DevModel m, DevBatch b, SweepParams p, int refresh_by_proposals,
                                                      int *active_count) {
    const int w = blockIdx.x, N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long t0 = b.t[w], tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);  // this launch's share
    const long long acc_left = b.acc_end[w] - b.accepted[w];
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        if (threadIdx.x == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ SweepCtlC ctl;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    C *gW = (sizeof(C) == 16 ? reinterpret_cast<C *>(b.W64) : reinterpret_cast<C *>(b.W32)) + (size_t)w * wblock;
    CPtr<C> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    C *cu = reinterpret_cast<C *>(smem);
    C *cdn = cu + N;
    C *ru = cdn + N;
    C *rd = ru + m.ld_up;
    short *kup = reinterpret_cast<short *>(rd + m.ld_dn);
    short *kdn = kup + N;
    for (int s = tid; s < N; s += blockDim.x) {
        kup[s] = b.kappa_up[(size_t)w * N + s];
        kdn[s] = b.kappa_dn[(size_t)w * N + s];
    }
    __syncthreads();
    double zc = 0.0;
    for (int e = tid; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = m.bonds[e];
        zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
    }
    zc = block_sum(zc, ctl.red);
    const int R = p.refresh_every, M = p.measure_every;
    if (tid == 0) {
        ctl.t = t0;
        ctl.since = b.since[w] < 0 ? 0 : b.since[w];
        ctl.zmu = (int)zc;
        ctl.next_meas = (t0 / M + 1) * M;
        ctl.next_ref = refresh_by_proposals ? (t0 / R + 1) * R : tend;
        make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
    }
    __syncthreads();
    long long acc_count = 0, n_meas = 0;
    double se = 0.0, se2 = 0.0;
    while (true) {
        if (warp == 0) {
            long long t = ctl.t;
            const int since = ctl.since;
            const long long stop = min(tend, ctl.next_ref);
            const long long next_meas = ctl.next_meas;
            const Thr thr = ctl.thr;
            int state = 2;
            while (true) {
                if (t >= stop || acc_count >= acc_left) break;
                if (!refresh_by_proposals && since >= R) break;
                const long long lim = min(stop, next_meas) - t;
                const int win = lim < 32 ? (int)lim : 32;
                bool acc = false, bad = false;
                int Ku = 0, lu = 0, Kd = 0, ld = 0;
                if (lane < win) {
                    unsigned long long u53;
                    int bi;
                    proposal_bits(p.seed, w, t + lane, m.n_bonds, u53, bi);
                    const int c = cmp_r_thr(u53, thr);
                    if (p.accept_rule != 0 || c <= 0) {
                        const short2 bd = m.bonds[bi];
                        const int i = bd.x, j = bd.y;
                        const int kui = kup[i], kuj = kup[j], kdi = kdn[i], kdj = kdn[j];
                        const bool f1 = kui != 0 && kdj != 0;
                        const bool f2 = kuj != 0 && kdi != 0;
                        if (f1 || f2) {
                            if (f1) { Ku = j; lu = kui - 1; Kd = i; ld = kdj - 1; }
                            else    { Ku = i; lu = kuj - 1; Kd = j; ld = kdi - 1; }
                            acc = decide_c(W.U(Ku, lu), W.D(Kd, ld), u53, c, thr, p.accept_rule, bad);
                        }
                    }
                }
                if (__any_sync(0xffffffffu, bad) && bad) atomicOr(&b.status[w], kStatusNonFinite);
                const unsigned mask = __ballot_sync(0xffffffffu, acc);
                if (mask) {
                    const int f = __ffs(mask) - 1;
                    if (lane == f) { ctl.Ku = Ku; ctl.lu = lu; ctl.Kd = Kd; ctl.ld = ld; }
                    t += f + 1;
                    state = 1;
                    break;
                }
                t += win;
                if (t == next_meas || t == ctl.next_ref) { state = 3; break; }
            }
            if (lane == 0) { ctl.t = t; ctl.state = state; }
        }
        __syncthreads();
        const int state = ctl.state;
        if (state == 2) break;
        if (state == 1) {
            const int Ku = ctl.Ku, lu = ctl.lu, Kd = ctl.Kd, ld = ctl.ld;
            rank1_update_c<C>(W, N, Ku, lu, Kd, ld, cu, ru, cdn, rd);
            if (tid == 0) {
                // the up spin moves Kd -> Ku, the down spin Ku -> Kd
                const int before = incident_antiparallel(m, kup, Ku, Kd);
                kup[Ku] = (short)(lu + 1); kup[Kd] = 0;
                kdn[Kd] = (short)(ld + 1); kdn[Ku] = 0;
                const int after = incident_antiparallel(m, kup, Ku, Kd);
                ctl.zmu += after - before;
                ctl.since += 1;
                make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
            }
            acc_count += 1;
            __syncthreads();
        }
        const long long t = ctl.t;
        if (t == ctl.next_meas) {
            const double e = local_energy_c<C>(m, kup, kdn, W, ctl.red);
            if (tid == 0) {
                se += e;
                se2 += e * e;
                n_meas += 1;
                ctl.next_meas += M;
            }
        }
        if (t == ctl.next_ref) break;
        __syncthreads();
    }
    __syncthreads();
    for (int s = tid; s < N; s += blockDim.x) {
        b.kappa_up[(size_t)w * N + s] = kup[s];
        b.kappa_dn[(size_t)w * N + s] = kdn[s];
    }
    if (tid == 0) {
        const long long t = ctl.t;
        b.t[w] = t;
        bool due;
        if (refresh_by_proposals) due = t == ctl.next_ref;
        else due = ctl.since >= R;
        b.since[w] = due ? -1 : ctl.since;
        b.accepted[w] += acc_count;
        b.proposals[w] += t - t0;
        b.sum_e[w] += se;
        b.sum_e2[w] += se2;
        b.n_meas[w] += n_meas;
        if (t < tend_all && acc_count < acc_left) atomicAdd(active_count, 1);
    }
}

// ---------------------------------------------------------------------------
// Mixed complex form with delayed updates (the real delayed kernel's scheme
// with complex FP32 entries): W stays in HBM, the factors P (N x K) and
// Q (ld x K) of the last m accepted moves sit in shared memory and
// W_eff = W - P Q^T; move m (pivot p = W_eff[K,l]) appends
// P[:,m] = W_eff[:,l] / p and Q[:,m] = W_eff[K,:] - e_l, and every K moves
// one pass applies W -= P Q^T.
// ---------------------------------------------------------------------------
template <int K>
struct CDelayed {
    cf *W, *P, *Q;
    int ld;
    // W_eff over the first m factor columns
    __device__ __forceinline__ cf eff(int r, int c, int m) const {
        cf v = W[(size_t)r * ld + c];
        const cf *pr = P + (size_t)r * K, *qc = Q + (size_t)c * K;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < m) v = cfms(pr[k], qc[k], v);
        return v;
    }
};

template <int K>
__device__ void cdelayed_flush(const CDelayed<K> &S, int N) {
    const int tot = N * S.ld;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        const int r = e / S.ld, c = e - r * S.ld;
        cf v = S.W[e];
        const cf *pr = S.P + (size_t)r * K, *qc = S.Q + (size_t)c * K;
#pragma unroll
        for (int k = 0; k < K; ++k) v = cfms(pr[k], qc[k], v);
        S.W[e] = v;
    }
}

template <int K>
__device__ void cdelayed_zero(const CDelayed<K> &S, int N) {
    for (int e = threadIdx.x; e < N * K; e += blockDim.x) S.P[e] = cf{0.f, 0.f};
    for (int e = threadIdx.x; e < S.ld * K; e += blockDim.x) S.Q[e] = cf{0.f, 0.f};
}

struct CDelayedCtl {
    long long t, next_meas;
    int since, zmu, state, m;
    int Ku, lu, Kd, ld;
    cf piv_u, piv_d;
    Thr thr;
    double red[33];
};

template <int K>
__global__ void __launch_bounds__(256, 2)
sweep_c_delayed_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count) {
    const int w = blockIdx.x, N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long t0 = b.t[w], tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);  // this launch's share
    const long long acc_left = b.acc_end[w] - b.accepted[w];
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        if (threadIdx.x == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CDelayedCtl ctl;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    cf *gW = reinterpret_cast<cf *>(b.W32) + (size_t)w * wblock;
    CDelayed<K> SU, SD;
    SU.W = gW;
    SU.ld = m.ld_up;
    SD.W = gW + (size_t)N * m.ld_up;
    SD.ld = m.ld_dn;
    unsigned char *cur = smem;
    SU.P = reinterpret_cast<cf *>(cur); cur += (size_t)N * K * sizeof(cf);
    SD.P = reinterpret_cast<cf *>(cur); cur += (size_t)N * K * sizeof(cf);
    SU.Q = reinterpret_cast<cf *>(cur); cur += (size_t)m.ld_up * K * sizeof(cf);
    SD.Q = reinterpret_cast<cf *>(cur); cur += (size_t)m.ld_dn * K * sizeof(cf);
    short *kup = reinterpret_cast<short *>(cur); cur += (size_t)N * sizeof(short);
    short *kdn = reinterpret_cast<short *>(cur);
    cdelayed_zero<K>(SU, N);
    cdelayed_zero<K>(SD, N);
    for (int s2 = tid; s2 < N; s2 += blockDim.x) {
        kup[s2] = b.kappa_up[(size_t)w * N + s2];
        kdn[s2] = b.kappa_dn[(size_t)w * N + s2];
    }
    __syncthreads();
    double zc = 0.0;
    for (int e = tid; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = m.bonds[e];
        zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
    }
    zc = block_sum(zc, ctl.red);
    const int R = p.refresh_every, M = p.measure_every;
    if (tid == 0) {
        ctl.t = t0;
        ctl.since = b.since[w] < 0 ? 0 : b.since[w];
        ctl.zmu = (int)zc;
        ctl.m = 0;
        ctl.next_meas = (t0 / M + 1) * M;
        make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
    }
    __syncthreads();
    long long acc_count = 0, n_meas = 0;
    double se = 0.0, se2 = 0.0;
    while (true) {
        const int mm = ctl.m;
        if (warp == 0) {
            long long t = ctl.t;
            const int since = ctl.since;
            const long long next_meas = ctl.next_meas;
            const Thr thr = ctl.thr;
            int state = 2;
            while (true) {
                if (t >= tend || since >= R || acc_count >= acc_left) break;
                const long long lim = min(tend, next_meas) - t;
                const int win = lim < 32 ? (int)lim : 32;
                bool acc = false, bad = false;
                int Ku = 0, lu = 0, Kd = 0, ld = 0;
                cf pu{0.f, 0.f}, pd{0.f, 0.f};
                if (lane < win) {
                    unsigned long long u53;
                    int bi;
                    proposal_bits(p.seed, w, t + lane, m.n_bonds, u53, bi);
                    const int c = cmp_r_thr(u53, thr);
                    if (p.accept_rule != 0 || c <= 0) {
                        const short2 bd = m.bonds[bi];
                        const int i = bd.x, j = bd.y;
                        const int kui = kup[i], kuj = kup[j], kdi = kdn[i], kdj = kdn[j];
                        const bool f1 = kui != 0 && kdj != 0;
                        const bool f2 = kuj != 0 && kdi != 0;
                        if (f1 || f2) {
                            if (f1) { Ku = j; lu = kui - 1; Kd = i; ld = kdj - 1; }
                            else    { Ku = i; lu = kuj - 1; Kd = j; ld = kdi - 1; }
                            pu = SU.eff(Ku, lu, mm);
                            pd = SD.eff(Kd, ld, mm);
                            acc = decide_c(pu, pd, u53, c, thr, p.accept_rule, bad);
                        }
                    }
                }
                if (__any_sync(0xffffffffu, bad) && bad) atomicOr(&b.status[w], kStatusNonFinite);
                const unsigned mask = __ballot_sync(0xffffffffu, acc);
                if (mask) {
                    const int f = __ffs(mask) - 1;
                    if (lane == f) {
                        ctl.Ku = Ku; ctl.lu = lu; ctl.Kd = Kd; ctl.ld = ld;
                        ctl.piv_u = pu; ctl.piv_d = pd;
                    }
                    t += f + 1;
                    state = 1;
                    break;
                }
                t += win;
                if (t == next_meas) { state = 3; break; }
            }
            if (lane == 0) { ctl.t = t; ctl.state = state; }
        }
        __syncthreads();
        const int state = ctl.state;
        if (state == 2) break;
        if (state == 1) {
            const int Ku = ctl.Ku, lu = ctl.lu, Kd = ctl.Kd, ld = ctl.ld;
            const cf ipu = cinv(ctl.piv_u), ipd = cinv(ctl.piv_d);
            const int tot = 2 * N + m.ld_up + m.ld_dn;
            for (int e = tid; e < tot; e += blockDim.x) {
                if (e < N) SU.P[(size_t)e * K + mm] = cmul(SU.eff(e, lu, mm), ipu);
                else if (e < 2 * N) SD.P[(size_t)(e - N) * K + mm] = cmul(SD.eff(e - N, ld, mm), ipd);
                else if (e < 2 * N + m.ld_up) {
                    const int c = e - 2 * N;
                    cf v = SU.eff(Ku, c, mm);
                    if (c == lu) v.x -= 1.f;
                    SU.Q[(size_t)c * K + mm] = v;
                } else {
                    const int c = e - 2 * N - m.ld_up;
                    cf v = SD.eff(Kd, c, mm);
                    if (c == ld) v.x -= 1.f;
                    SD.Q[(size_t)c * K + mm] = v;
                }
            }
            if (tid == 0) {
                // the up spin moves Kd -> Ku, the down spin Ku -> Kd
                const int before = incident_antiparallel(m, kup, Ku, Kd);
                kup[Ku] = (short)(lu + 1); kup[Kd] = 0;
                kdn[Kd] = (short)(ld + 1); kdn[Ku] = 0;
                const int after = incident_antiparallel(m, kup, Ku, Kd);
                ctl.zmu += after - before;
                ctl.since += 1;
                make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
            }
            acc_count += 1;
            __syncthreads();
            if (mm + 1 == K) {
                cdelayed_flush<K>(SU, N);
                cdelayed_flush<K>(SD, N);
                __syncthreads();
                cdelayed_zero<K>(SU, N);
                cdelayed_zero<K>(SD, N);
                if (tid == 0) ctl.m = 0;
            } else if (tid == 0) {
                ctl.m = mm + 1;
            }
            __syncthreads();
        }
        const long long t = ctl.t;
        if (t == ctl.next_meas) {
            const int mnow = ctl.m;
            float accE = 0.f;
            for (int e = tid; e < m.n_bonds; e += blockDim.x) {
                const short2 bd = m.bonds[e];
                const int i = bd.x, j = bd.y;
                const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
                accE += ((ui != 0) == (uj != 0)) ? 0.25f : -0.25f;
                if (uj != 0 && di != 0) accE -= 0.5f * cmul(SU.eff(i, uj - 1, mnow), SD.eff(j, di - 1, mnow)).x;
                if (ui != 0 && dj != 0) accE -= 0.5f * cmul(SU.eff(j, ui - 1, mnow), SD.eff(i, dj - 1, mnow)).x;
            }
            const double e = block_sum_f32(accE, ctl.red);
            if (tid == 0) {
                se += e;
                se2 += e * e;
                n_meas += 1;
                ctl.next_meas += M;
            }
        }
        __syncthreads();
    }
    __syncthreads();
    if (ctl.m > 0) {
        // flush only the columns written so far (the rest are zero)
        cdelayed_flush<K>(SU, N);
        cdelayed_flush<K>(SD, N);
        __syncthreads();
    }
    for (int s2 = tid; s2 < N; s2 += blockDim.x) {
        b.kappa_up[(size_t)w * N + s2] = kup[s2];
        b.kappa_dn[(size_t)w * N + s2] = kdn[s2];
    }
    if (tid == 0) {
        const long long t = ctl.t;
        b.t[w] = t;
        b.since[w] = ctl.since >= R ? -1 : ctl.since;
        b.accepted[w] += acc_count;
        b.proposals[w] += t - t0;
        b.sum_e[w] += se;
        b.sum_e2[w] += se2;
        b.n_meas[w] += n_meas;
        if (t < tend_all && acc_count < acc_left) atomicAdd(active_count, 1);
    }
}

// ---------------------------------------------------------------------------
// The pipelined form of the complex delayed sweep (the real
// sweep_pipe_kernel's scheme, kvmc_kernels.cu): warp 0 scans for the next
// accepted move while the other warps write the factor column of the last
// one, reading W_eff through that move's Sherman-Morrison correction
//   W_eff'(r, c) = W_eff(r, c) - W_eff(r, l) (W_eff(K, c) - [c == l]) / pivot
// over the complete columns only; one barrier per accepted move.  Z_mu
// changes come from per-site up-neighbour counts, the accepted move reaches
// the warp by shuffles, the thresholds sit in shared memory when they fit.
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ cf ceff_after(const CDelayed<K> &S, int r, int c, int mm, bool pend, int Kp, int lp,
                                         cf ipiv) {
    cf v = S.eff(r, c, mm);
    if (pend) {
        const cf a = S.eff(r, lp, mm);
        cf q = S.eff(Kp, c, mm);
        if (c == lp) q.x -= 1.f;
        v = cfms(cmul(a, ipiv), q, v);
    }
    return v;
}

struct CPipeMove {
    int Ku, lu, Kd, ld;
    cf piv_u, piv_d;
};

struct CPipeCtl {
    long long t, next_meas, acc;
    int since, zmu;
    int state2[2];
    CPipeMove mv[2];
    Thr thr;
    double red[33];
};

template <int K>
__global__ void __launch_bounds__(256, 2)
sweep_c_pipe_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count, int thr_in_smem) {
    const int w = blockIdx.x, N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long t0 = b.t[w], tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);  // this launch's share
    const long long acc_left = b.acc_end[w] - b.accepted[w];
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        if (threadIdx.x == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CPipeCtl ctl;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    cf *gW = reinterpret_cast<cf *>(b.W32) + (size_t)w * wblock;
    CDelayed<K> SU, SD;
    SU.W = gW;
    SU.ld = m.ld_up;
    SD.W = gW + (size_t)N * m.ld_up;
    SD.ld = m.ld_dn;
    unsigned char *cur = smem;
    SU.P = reinterpret_cast<cf *>(cur); cur += (size_t)N * K * sizeof(cf);
    SD.P = reinterpret_cast<cf *>(cur); cur += (size_t)N * K * sizeof(cf);
    SU.Q = reinterpret_cast<cf *>(cur); cur += (size_t)m.ld_up * K * sizeof(cf);
    SD.Q = reinterpret_cast<cf *>(cur); cur += (size_t)m.ld_dn * K * sizeof(cf);
    int *nbr_off = reinterpret_cast<int *>(cur); cur += (size_t)(N + 1) * sizeof(int);
    int *nu = reinterpret_cast<int *>(cur); cur += (size_t)N * sizeof(int);
    short2 *bonds = reinterpret_cast<short2 *>(cur); cur += (size_t)m.n_bonds * sizeof(short2);
    short *nbr = reinterpret_cast<short *>(cur); cur += (size_t)2 * m.n_bonds * sizeof(short);
    short *kup = reinterpret_cast<short *>(cur); cur += (size_t)N * sizeof(short);
    short *kdn = reinterpret_cast<short *>(cur); cur += (size_t)N * sizeof(short);
    ThrEntry *thr_s = reinterpret_cast<ThrEntry *>((reinterpret_cast<uintptr_t>(cur) + 15) & ~uintptr_t(15));
    const ThrEntry *thr_tab = thr_in_smem ? thr_s : m.thr_table;
    cdelayed_zero<K>(SU, N);
    cdelayed_zero<K>(SD, N);
    for (int e = tid; e < m.n_bonds; e += blockDim.x) bonds[e] = m.bonds[e];
    for (int e = tid; e < 2 * m.n_bonds; e += blockDim.x) nbr[e] = m.nbr[e];
    for (int e = tid; e <= N; e += blockDim.x) nbr_off[e] = m.nbr_off[e];
    if (thr_in_smem)
        for (int e = tid; e <= m.n_bonds; e += blockDim.x) thr_s[e] = m.thr_table[e];
    for (int s2 = tid; s2 < N; s2 += blockDim.x) {
        kup[s2] = b.kappa_up[(size_t)w * N + s2];
        kdn[s2] = b.kappa_dn[(size_t)w * N + s2];
    }
    __syncthreads();
    double zc = 0.0;
    for (int e = tid; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = bonds[e];
        zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
    }
    for (int s2 = tid; s2 < N; s2 += blockDim.x) {
        int c = 0;
        for (int e = nbr_off[s2]; e < nbr_off[s2 + 1]; ++e) c += kup[nbr[e]] != 0 ? 1 : 0;
        nu[s2] = c;
    }
    zc = block_sum(zc, ctl.red);
    const int R = p.refresh_every, M = p.measure_every;
    if (tid == 0) {
        ctl.t = t0;
        ctl.acc = 0;
        ctl.since = b.since[w] < 0 ? 0 : b.since[w];
        ctl.zmu = (int)zc;
        ctl.next_meas = (t0 / M + 1) * M;
        make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
    }
    __syncthreads();
    long long n_meas = 0;
    double se = 0.0, se2 = 0.0;
    // loop state kept by every thread alike: pend = a move accepted in the
    // previous phase whose factor column this phase writes, slot = its entry
    // in ctl.mv, mm = complete factor columns
    int pend = 0, slot = 0, mm = 0, it = 0;
    while (true) {
        if (warp == 0) {
            const CPipeMove pm = ctl.mv[slot];
            const cf ipu = pend ? cinv(pm.piv_u) : cf{0.f, 0.f}, ipd = pend ? cinv(pm.piv_d) : cf{0.f, 0.f};
            long long t = ctl.t;
            const long long acc = ctl.acc, next_meas = ctl.next_meas;
            const int since = ctl.since;
            const Thr thr = ctl.thr;
            int state = 2;
            CPipeMove nm{};
            while (true) {
                if (t == next_meas) { state = 3; break; }
                if (t >= tend || since >= R || acc >= acc_left) break;
                const long long lim = min(tend, next_meas) - t;
                const int win = lim < 32 ? (int)lim : 32;
                bool accd = false, bad = false;
                int Ku = 0, lu = 0, Kd = 0, ld = 0;
                cf pu{0.f, 0.f}, pd{0.f, 0.f};
                if (lane < win) {
                    unsigned long long u53;
                    int bi;
                    proposal_bits(p.seed, w, t + lane, m.n_bonds, u53, bi);
                    const short2 bd = bonds[bi];
                    const int c = cmp_r_thr(u53, thr);
                    if (p.accept_rule != 0 || c <= 0) {
                        const int i = bd.x, j = bd.y;
                        const int kui = kup[i], kuj = kup[j], kdi = kdn[i], kdj = kdn[j];
                        const bool f1 = kui != 0 && kdj != 0;
                        const bool f2 = kuj != 0 && kdi != 0;
                        if (f1 || f2) {
                            if (f1) { Ku = j; lu = kui - 1; Kd = i; ld = kdj - 1; }
                            else    { Ku = i; lu = kuj - 1; Kd = j; ld = kdi - 1; }
                            pu = ceff_after<K>(SU, Ku, lu, mm, pend, pm.Ku, pm.lu, ipu);
                            pd = ceff_after<K>(SD, Kd, ld, mm, pend, pm.Kd, pm.ld, ipd);
                            accd = decide_c(pu, pd, u53, c, thr, p.accept_rule, bad);
                        }
                    }
                }
                if (__any_sync(0xffffffffu, bad) && bad) atomicOr(&b.status[w], kStatusNonFinite);
                const unsigned mask = __ballot_sync(0xffffffffu, accd);
                if (mask) {
                    const int f = __ffs(mask) - 1;
                    nm.Ku = __shfl_sync(0xffffffffu, Ku, f);
                    nm.lu = __shfl_sync(0xffffffffu, lu, f);
                    nm.Kd = __shfl_sync(0xffffffffu, Kd, f);
                    nm.ld = __shfl_sync(0xffffffffu, ld, f);
                    nm.piv_u = cf{__shfl_sync(0xffffffffu, pu.x, f), __shfl_sync(0xffffffffu, pu.y, f)};
                    nm.piv_d = cf{__shfl_sync(0xffffffffu, pd.x, f), __shfl_sync(0xffffffffu, pd.y, f)};
                    t += f + 1;
                    state = 1;
                    break;
                }
                t += win;
            }
            if (state == 1) {
                // the up spin moves Kd -> Ku along their bond: Z_mu changes by
                // (deg Ku - 1 - 2 (nu[Ku] - 1)) + (2 nu[Kd] - (deg Kd - 1))
                const int bu = nbr_off[nm.Ku], du = nbr_off[nm.Ku + 1] - bu;
                const int bdn = nbr_off[nm.Kd], dd = nbr_off[nm.Kd + 1] - bdn;
                const int dz = du - dd + 2 - 2 * nu[nm.Ku] + 2 * nu[nm.Kd];
                __syncwarp();  // every lane has read nu before it changes
                for (int e = lane; e < du + dd; e += 32)
                    atomicAdd(&nu[e < du ? nbr[bu + e] : nbr[bdn + e - du]], e < du ? 1 : -1);
                if (lane == 0) {
                    ctl.mv[slot ^ 1] = nm;
                    kup[nm.Ku] = (short)(nm.lu + 1); kup[nm.Kd] = 0;
                    kdn[nm.Kd] = (short)(nm.ld + 1); kdn[nm.Ku] = 0;
                    ctl.zmu += dz;
                    make_thr(ctl.thr, thr_tab, ctl.zmu, p.accept_rule);
                    ctl.since += 1;
                    ctl.acc += 1;
                }
            }
            if (lane == 0) { ctl.t = t; ctl.state2[it & 1] = state; }
        } else if (pend) {
            // factor column mm of the pending move, over columns [0, mm)
            const CPipeMove pm = ctl.mv[slot];
            const cf ipu = cinv(pm.piv_u), ipd = cinv(pm.piv_d);
            const int tot = 2 * N + m.ld_up + m.ld_dn;
            const int nt = blockDim.x - 32, id = tid - 32;
            for (int e = id; e < tot; e += nt) {
                if (e < N) SU.P[(size_t)e * K + mm] = cmul(SU.eff(e, pm.lu, mm), ipu);
                else if (e < 2 * N) SD.P[(size_t)(e - N) * K + mm] = cmul(SD.eff(e - N, pm.ld, mm), ipd);
                else if (e < 2 * N + m.ld_up) {
                    const int c = e - 2 * N;
                    cf v = SU.eff(pm.Ku, c, mm);
                    if (c == pm.lu) v.x -= 1.f;
                    SU.Q[(size_t)c * K + mm] = v;
                } else {
                    const int c = e - 2 * N - m.ld_up;
                    cf v = SD.eff(pm.Kd, c, mm);
                    if (c == pm.ld) v.x -= 1.f;
                    SD.Q[(size_t)c * K + mm] = v;
                }
            }
        }
        __syncthreads();
        const int state = ctl.state2[it & 1];
        ++it;
        const int mnew = pend ? mm + 1 : mm;
        if (mnew == K) {
            cdelayed_flush<K>(SU, N);
            cdelayed_flush<K>(SD, N);
            __syncthreads();
            cdelayed_zero<K>(SU, N);
            cdelayed_zero<K>(SD, N);
            __syncthreads();
        }
        mm = mnew == K ? 0 : mnew;
        if (state == 1) slot ^= 1;
        pend = state == 1;
        if (state == 3) {
            float accE = 0.f;
            for (int e = tid; e < m.n_bonds; e += blockDim.x) {
                const short2 bd = bonds[e];
                const int i = bd.x, j = bd.y;
                const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
                accE += ((ui != 0) == (uj != 0)) ? 0.25f : -0.25f;
                if (uj != 0 && di != 0) accE -= 0.5f * cmul(SU.eff(i, uj - 1, mm), SD.eff(j, di - 1, mm)).x;
                if (ui != 0 && dj != 0) accE -= 0.5f * cmul(SU.eff(j, ui - 1, mm), SD.eff(i, dj - 1, mm)).x;
            }
            const double e = block_sum_f32(accE, ctl.red);
            if (tid == 0) {
                se += e;
                se2 += e * e;
                n_meas += 1;
                ctl.next_meas += M;
            }
        }
        __syncthreads();
        if (state == 2) break;
    }
    if (mm > 0) {
        // columns past mm are zero, so the full flush is exact
        cdelayed_flush<K>(SU, N);
        cdelayed_flush<K>(SD, N);
        __syncthreads();
    }
    for (int s2 = tid; s2 < N; s2 += blockDim.x) {
        b.kappa_up[(size_t)w * N + s2] = kup[s2];
        b.kappa_dn[(size_t)w * N + s2] = kdn[s2];
    }
    if (tid == 0) {
        const long long t = ctl.t;
        b.t[w] = t;
        b.since[w] = ctl.since >= R ? -1 : ctl.since;
        b.accepted[w] += ctl.acc;
        b.proposals[w] += t - t0;
        b.sum_e[w] += se;
        b.sum_e2[w] += se2;
        b.n_meas[w] += n_meas;
        if (t < tend_all && ctl.acc < acc_left) atomicAdd(active_count, 1);
    }
}

static size_t complex_pipe_smem(const DevModel &m, int K) {
    const size_t N = m.n_sites;
    size_t s = (size_t)(2 * N + m.ld_up + m.ld_dn) * K * sizeof(cf);
    s += (N + 1) * 4 + N * 4 + (size_t)m.n_bonds * 4 + (size_t)2 * m.n_bonds * 2 + 2 * N * 2;
    return (s + 15) / 16 * 16 + 16;  // the threshold table starts 16-byte aligned after this
}

template <int K>
static cudaError_t launch_c_pipe(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                 cudaStream_t stream) {
    size_t sm = complex_pipe_smem(m, K);
    const size_t thr_bytes = (size_t)(m.n_bonds + 1) * sizeof(ThrEntry);
    const size_t kSmemPerSM = 228 * 1024, kReserve = 1024 + 2048;  // per-CTA reserve and static shared data
    const int thr_in_smem = 2 * (sm + thr_bytes + kReserve) <= kSmemPerSM && sm + thr_bytes <= 227 * 1024;
    if (thr_in_smem) sm += thr_bytes;
    cudaError_t e = cudaFuncSetAttribute(sweep_c_pipe_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    sweep_c_pipe_kernel<K><<<b.n_walkers, 256, sm, stream>>>(m, b, p, active, thr_in_smem);
    return cudaGetLastError();
}

size_t complex_delayed_smem(const DevModel &m, int K) {
    return (size_t)(2 * m.n_sites + m.ld_up + m.ld_dn) * K * sizeof(cf) + (size_t)2 * m.n_sites * 2 + 16;
}

template <typename C>
size_t sweep_c_smem(const DevModel &m) {
    return (size_t)(2 * m.n_sites + m.ld_up + m.ld_dn) * sizeof(C) + (size_t)2 * m.n_sites * 2 + 16;
}

// ---- API / test entry points ------------------------------------------------
template <typename C>
__global__ void measure_c_kernel(DevModel m, DevBatch b) {
    const int w = blockIdx.x, N = m.n_sites;
    __shared__ double red[33];
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    C *gW = (sizeof(C) == 16 ? reinterpret_cast<C *>(b.W64) : reinterpret_cast<C *>(b.W32)) + (size_t)w * wblock;
    CPtr<C> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    const double e = local_energy_c<C>(m, b.kappa_up + (size_t)w * N, b.kappa_dn + (size_t)w * N, W, red);
    if (threadIdx.x == 0) b.energy_out[w] = e;
}

// complex ratios, interleaved (re, im) into out
template <typename C>
__global__ void ratio_c_kernel(DevModel m, DevBatch b, int n_moves, const int *moves, double *out) {
    const int w = blockIdx.x, N = m.n_sites;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    C *gW = (sizeof(C) == 16 ? reinterpret_cast<C *>(b.W64) : reinterpret_cast<C *>(b.W32)) + (size_t)w * wblock;
    CPtr<C> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    for (int k = threadIdx.x; k < n_moves; k += blockDim.x) {
        const int *mv = moves + ((size_t)w * n_moves + k) * 4;
        const C a = W.U(mv[0], mv[1] - 1), d = W.D(mv[2], mv[3] - 1);
        const cd r = cmul(cd{(double)a.x, (double)a.y}, cd{(double)d.x, (double)d.y});
        out[2 * ((size_t)w * n_moves + k)] = r.x;
        out[2 * ((size_t)w * n_moves + k) + 1] = r.y;
    }
}

template <typename C>
__global__ void apply_moves_c_kernel(DevModel m, DevBatch b, const int *moves) {
    const int w = blockIdx.x, N = m.n_sites;
    const int *mv = moves + (size_t)w * 5;
    const int flag = mv[0];
    if (flag == 0) return;
    const int i = mv[1], site = mv[2], l_up = mv[3], l_dn = mv[4];
    extern __shared__ __align__(16) unsigned char smem[];
    C *stg = reinterpret_cast<C *>(smem);
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    C *gW = (sizeof(C) == 16 ? reinterpret_cast<C *>(b.W64) : reinterpret_cast<C *>(b.W32)) + (size_t)w * wblock;
    CPtr<C> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    const int Ku = flag == 1 ? site : i;
    const int Kd = flag == 1 ? i : site;
    rank1_update_c<C>(W, N, Ku, l_up - 1, Kd, l_dn - 1, stg, stg + 2 * N, stg + N, stg + 2 * N + m.ld_up);
    if (threadIdx.x == 0) {
        short *ku = b.kappa_up + (size_t)w * N, *kd = b.kappa_dn + (size_t)w * N;
        if (flag == 1) { ku[i] = 0; ku[site] = (short)l_up; kd[i] = (short)l_dn; kd[site] = 0; }
        else { ku[i] = (short)l_up; ku[site] = 0; kd[i] = 0; kd[site] = (short)l_dn; }
    }
}

// ---- launchers ----------------------------------------------------------------
int complex_max_orbitals() { return kMaxComplexOrbitals; }

bool complex_refresh_needs_large(const DevModel &m) {
    return (m.n_up > m.n_dn ? m.n_up : m.n_dn) > kMaxComplexOrbitals;
}

size_t complex_refresh_smem(const DevModel &m) {
    return complex_refresh_needs_large(m) ? refresh_c_large_smem(m) : refresh_c_smem(m);
}

cudaError_t launch_refresh_c(const DevModel &m, const DevBatch &b, bool fp32_out, int only_due, int track_drift,
                             cudaStream_t stream) {
    const dim3 grid(b.n_walkers, 2);
    if (complex_refresh_needs_large(m)) {
        if (!b.lu_scratch) return cudaErrorInvalidValue;
        const size_t sm = refresh_c_large_smem(m);
        if (fp32_out) {
            cudaError_t e = cudaFuncSetAttribute(refresh_c_large_kernel<cf>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            refresh_c_large_kernel<cf><<<grid, kThreadsC, sm, stream>>>(m, b, only_due, track_drift);
        } else {
            cudaError_t e = cudaFuncSetAttribute(refresh_c_large_kernel<cd>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            refresh_c_large_kernel<cd><<<grid, kThreadsC, sm, stream>>>(m, b, only_due, track_drift);
        }
        return cudaGetLastError();
    }
    const size_t sm = refresh_c_smem(m);
    if (fp32_out) {
        cudaError_t e = cudaFuncSetAttribute(refresh_c_kernel<cf>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        refresh_c_kernel<cf><<<grid, kThreadsC, sm, stream>>>(m, b, only_due, track_drift);
    } else {
        cudaError_t e = cudaFuncSetAttribute(refresh_c_kernel<cd>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        refresh_c_kernel<cd><<<grid, kThreadsC, sm, stream>>>(m, b, only_due, track_drift);
    }
    return cudaGetLastError();
}

template <int K>
static cudaError_t launch_c_delayed(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                    cudaStream_t stream) {
    const size_t sm = complex_delayed_smem(m, K);
    cudaError_t e = cudaFuncSetAttribute(sweep_c_delayed_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    sweep_c_delayed_kernel<K><<<b.n_walkers, 256, sm, stream>>>(m, b, p, active);
    return cudaGetLastError();
}

cudaError_t launch_sweep_c(const DevModel &m, const DevBatch &b, const SweepParams &p, bool mixed, int *active,
                           cudaStream_t stream) {
    if (mixed && p.delay_k == 4)
        return p.pipeline ? launch_c_pipe<4>(m, b, p, active, stream) : launch_c_delayed<4>(m, b, p, active, stream);
    if (mixed && p.delay_k == 8)
        return p.pipeline ? launch_c_pipe<8>(m, b, p, active, stream) : launch_c_delayed<8>(m, b, p, active, stream);
    if (mixed) {
        const size_t sm = sweep_c_smem<cf>(m);
        sweep_c_kernel<cf><<<b.n_walkers, 256, sm, stream>>>(m, b, p, 0, active);
    } else {
        const size_t sm = sweep_c_smem<cd>(m);
        sweep_c_kernel<cd><<<b.n_walkers, 256, sm, stream>>>(m, b, p, 1, active);
    }
    return cudaGetLastError();
}

cudaError_t launch_measure_c(const DevModel &m, const DevBatch &b, bool fp32, cudaStream_t stream) {
    if (fp32) measure_c_kernel<cf><<<b.n_walkers, 256, 0, stream>>>(m, b);
    else measure_c_kernel<cd><<<b.n_walkers, 256, 0, stream>>>(m, b);
    return cudaGetLastError();
}

cudaError_t launch_eval_ratios_c(const DevModel &m, const DevBatch &b, bool fp32, int n_moves, const int *moves,
                                 double *out, cudaStream_t stream) {
    if (fp32) ratio_c_kernel<cf><<<b.n_walkers, 128, 0, stream>>>(m, b, n_moves, moves, out);
    else ratio_c_kernel<cd><<<b.n_walkers, 128, 0, stream>>>(m, b, n_moves, moves, out);
    return cudaGetLastError();
}

cudaError_t launch_apply_moves_c(const DevModel &m, const DevBatch &b, bool fp32, const int *moves,
                                 cudaStream_t stream) {
    const size_t elem = fp32 ? sizeof(cf) : sizeof(cd);
    const size_t sm = (size_t)(2 * m.n_sites + m.ld_up + m.ld_dn) * elem + 16;
    if (fp32) apply_moves_c_kernel<cf><<<b.n_walkers, 256, sm, stream>>>(m, b, moves);
    else apply_moves_c_kernel<cd><<<b.n_walkers, 256, sm, stream>>>(m, b, moves);
    return cudaGetLastError();
}

}  // namespace kvmc
