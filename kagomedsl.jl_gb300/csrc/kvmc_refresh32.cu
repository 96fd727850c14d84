// Periodic refresh of the FP32 W by mixed-precision iterative refinement.
//
// reevaluateW! (src/MonteCarlo.jl:55-66) rebuilds W = U tilde_U^{-1} to bound
// the rounding the rank-1 / rank-k updates accumulate.  The FP32 W the
// sweep keeps only needs that rebuild to FP32 accuracy, so instead of an
// FP64 LU and FP64 triangular solves (FP64 runs at 1/64 of the FP32 rate on
// this part) each non-trivial row y of W (y tilde_U = u for the sites that do
// not hold this spin) is computed as
//   1. y0 = u tilde_U^{-1} with an FP32 LU of tilde_U (partial pivoting) and
//      FP32 triangular solves: error ~ cond(tilde_U) * 2^-24;
//   2. r = u - y0 tilde_U with exact products (two-product via fmaf) and
//      compensated (double-float) sums: r to ~2^-44 relative to |u|;
//   3. y = y0 + r tilde_U^{-1} (FP32 solves again): error
//      ~ (cond * 2^-24)^2, below FP32 rounding for cond up to ~1e4.
// A row whose correction exceeds 1e-3 of the row gets a second pass (error
// ~ (cond * 2^-24)^3); a row still moving by more than 1e-4 after it flags
// the walker (kStatusRefine), and the FP64 refresh then rebuilds that
// walker's W.
// All arithmetic runs on the FP32 pipes.  The rows at sites holding the spin
// are exact unit rows.  The FP64 refresh (kvmc_kernels.cu) stays in use for
// starts and restored states (where log|det| and the pivot ratio are needed)
// and for more than 224 orbitals per spin.
#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc_device.cuh"
#include "kvmc_internal.h"
#include "kvmc_refine.cuh"

namespace kvmc {

namespace {

// 128 threads, four walker-spins per SM: the refinement gives each thread
// one row of W, and more rows in flight per SM hide its dependent chains.
constexpr int kThreads32 = 128;
constexpr int kBlocks32 = 4;
constexpr int kMaxN32 = 224;

// P A = L Uf in place (float), first maximal |pivot| wins; false when singular.
__device__ bool lu32(float *A, int lda, int n, int *perm, float *invd) {
    __shared__ int s_piv;
    __shared__ float s_pmax, s_dinv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            float best = -1.f;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                const float v = fabsf(A[(size_t)i * lda + k]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) {
                s_piv = bi;
                s_pmax = best;
                s_dinv = best > 0.f ? 1.f / A[(size_t)bi * lda + k] : 0.f;
            }
        }
        __syncthreads();
        if (!(s_pmax > 0.f)) return false;
        const int p = s_piv;
        if (p != k) {
            for (int j = tid; j < n; j += nt) {
                const float a = A[(size_t)k * lda + j];
                A[(size_t)k * lda + j] = A[(size_t)p * lda + j];
                A[(size_t)p * lda + j] = a;
            }
            if (tid == 0) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
        }
        __syncthreads();
        const float dinv = s_dinv;
        for (int i = k + 1 + tid; i < n; i += nt) A[(size_t)i * lda + k] *= dinv;
        __syncthreads();
        for (int i = k + 1 + warp; i < n; i += nt / 32) {
            const float aik = A[(size_t)i * lda + k];
            float *Ai = A + (size_t)i * lda;
            const float *Ak = A + (size_t)k * lda;
            for (int j = k + 1 + lane; j < n; j += 32) Ai[j] = fmaf(-aik, Ak[j], Ai[j]);
        }
        __syncthreads();
    }
    for (int i = tid; i < n; i += nt) invd[i] = 1.f / A[(size_t)i * lda + i];
    __syncthreads();
    return true;
}

__global__ void __launch_bounds__(kThreads32, kBlocks32)
refresh32_kernel(DevModel m, DevBatch b, int only_due, int track_drift) {
    const int w = blockIdx.x, spin = blockIdx.y;
    if (only_due && b.since[w] >= 0) return;
    if (spin == 0 && threadIdx.x == 0) atomicAdd(b.refresh_count, 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const float *Uh = spin == 0 ? m.U32_up_hi : m.U32_dn_hi;
    const float *Ul = spin == 0 ? m.U32_up_lo : m.U32_dn_lo;
    const short *kappa = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    // during a one-warp sweep call the rows go to the label-indexed blocks
    const bool cpt = b.compact != 0;
    float *W = cpt ? b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up)
                   : b.W32 + (size_t)w * wblock + (spin == 0 ? 0 : (size_t)N * m.ld_up);
    const short *krow = cpt ? (spin == 0 ? b.kappa_dn : b.kappa_up) + (size_t)w * N : nullptr;

    extern __shared__ __align__(16) unsigned char smem[];
    const int lda = n + 1;
    float *A = reinterpret_cast<float *>(smem);
    float *invd = A + (size_t)n * lda;
    int *perm = reinterpret_cast<int *>(invd + n);
    short *site_of = reinterpret_cast<short *>(perm + n);  // the site whose U row is row l of tilde_U
    short *rows = site_of + n;
    __shared__ int s_nrows;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;

    for (int e = tid; e < n * lda; e += nt) A[e] = 0.f;
    for (int i = tid; i < n; i += nt) { perm[i] = i; site_of[i] = -1; }
    __syncthreads();
    for (int R = warp; R < N; R += nt / 32) {
        const int l = kappa[R];
        if (l >= 1 && l <= n) {
            if (lane == 0) site_of[l - 1] = (short)R;
            for (int c = lane; c < n; c += 32) A[(size_t)(l - 1) * lda + c] = Uh[(size_t)R * n + c];
        }
    }
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
    __syncthreads();
    if (!lu32(A, lda, n, perm, invd)) {  // an exactly zero FP32 pivot: leave it to the FP64 refresh
        if (tid == 0) atomicOr(&b.status[w], kStatusRefine);
        return;
    }
    {
        // log|det tilde_U| and log(min|pivot| / max|pivot|) from the FP32 factors
        __shared__ double red[33];
        double ldet = 0.0, dmin = INFINITY, dmaxp = 0.0;
        for (int i = tid; i < n; i += nt) {
            const float d = fabsf(A[(size_t)i * lda + i]);
            ldet += (double)logf(d);
            dmin = fmin(dmin, (double)d);
            dmaxp = fmax(dmaxp, (double)d);
        }
        ldet = block_sum(ldet, red);
        dmin = -block_sum_max(-dmin, red);
        dmaxp = block_sum_max(dmaxp, red);
        if (tid == 0) {
            b.logdet[4 * w + spin] = ldet;
            b.logdet[4 * w + 2 + spin] = log(dmin / dmaxp);
        }
    }
    // unit rows at occupied sites, zero padding elsewhere (site-indexed W only)
    if (!cpt) {
        float dmax = 0.f;
        for (int R = warp; R < N; R += nt / 32) {
            const int l = kappa[R];
            float *wr = W + (size_t)R * ldw;
            if (l != 0) {
                for (int c = lane; c < ldw; c += 32) {
                    const float nv = (c == l - 1) ? 1.f : 0.f;
                    if (track_drift) dmax = fmaxf(dmax, fabsf(wr[c] - nv) / (1.f + fabsf(nv)));
                    wr[c] = nv;
                }
            } else {
                for (int c = n + lane; c < ldw; c += 32) wr[c] = 0.f;
            }
        }
        if (track_drift) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
            if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
        }
    }
    const int nrows = s_nrows;
    // scratch (the FP64 refresh's block, as floats): y0 then the correction,
    // each [n][nrows] column-major
    float *Y = reinterpret_cast<float *>(b.solve_scratch + ((size_t)w * 2 + spin) * b.solve_block);
    float dmax = 0.f;
    for (int r0 = 0; r0 < nrows; r0 += nt) {
        const int cnt = min(nt, nrows - r0);
        const int r = tid;
        if (r < cnt) {
            const int R = rows[r0 + r];
            if (!refine_row(A, lda, invd, perm, site_of, Uh, Ul, n, R, Y + (size_t)r0 * n * 2 + r, cnt,
                            W + (size_t)(krow ? krow[R] - 1 : R) * ldw, track_drift != 0, dmax))
                atomicOr(&b.status[w], kStatusRefine);
        }
    }
    if (track_drift) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
    }
}

}  // namespace

size_t refresh32_smem(const DevModel &m) {
    const size_t n = m.n_up > m.n_dn ? m.n_up : m.n_dn;
    return n * (n + 1) * 4 + n * 4 + n * 4 + n * 2 + (size_t)m.n_sites * 2 + 64;
}

bool refresh32_supported(const DevModel &m) {
    return (m.n_up > m.n_dn ? m.n_up : m.n_dn) <= kMaxN32;
}

__global__ void clear_status_bits_kernel(DevBatch b, int bits) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < b.n_walkers) b.status[w] &= ~bits;
}

// The per-call statistics of a sweep call in one CTA, every sum in a fixed
// order (thread t takes walkers t, t + 512, ...; then a fixed tree), so the
// result does not depend on scheduling.  out: [0] sum of sum_e, [1] of
// sum_e2, [2] of n_meas, [3] of accepted, [4] of proposals, [5] walkers with
// a status bit set, [6] the first of them (-1: none), [7] its status, [8] the
// largest drift, [9] walkers short of acc_end, [10] the first of them,
// [11], [12] the two refresh counters.
constexpr int kStatsThreads = 512;
__global__ void __launch_bounds__(kStatsThreads) call_stats_kernel(DevBatch b, double *out) {
    __shared__ double sd[kStatsThreads][2];
    __shared__ long long sl[kStatsThreads][5];
    __shared__ int sf[kStatsThreads][2];
    __shared__ float sm[kStatsThreads];
    const int t = threadIdx.x;
    double e = 0.0, e2 = 0.0;
    long long nm = 0, acc = 0, prop = 0, nbad = 0, nshort = 0;
    int fbad = 0x7fffffff, fshort = 0x7fffffff;
    float dr = 0.f;
    for (int w = t; w < b.n_walkers; w += kStatsThreads) {
        e += b.sum_e[w];
        e2 += b.sum_e2[w];
        nm += b.n_meas[w];
        acc += b.accepted[w];
        prop += b.proposals[w];
        if (b.status[w]) { ++nbad; fbad = min(fbad, w); }
        if (b.accepted[w] < b.acc_end[w]) { ++nshort; fshort = min(fshort, w); }
        dr = fmaxf(dr, b.drift[w]);
    }
    sd[t][0] = e; sd[t][1] = e2;
    sl[t][0] = nm; sl[t][1] = acc; sl[t][2] = prop; sl[t][3] = nbad; sl[t][4] = nshort;
    sf[t][0] = fbad; sf[t][1] = fshort;
    sm[t] = dr;
    __syncthreads();
    for (int h = kStatsThreads / 2; h > 0; h >>= 1) {
        if (t < h) {
            sd[t][0] += sd[t + h][0];
            sd[t][1] += sd[t + h][1];
            for (int q = 0; q < 5; ++q) sl[t][q] += sl[t + h][q];
            sf[t][0] = min(sf[t][0], sf[t + h][0]);
            sf[t][1] = min(sf[t][1], sf[t + h][1]);
            sm[t] = fmaxf(sm[t], sm[t + h]);
        }
        __syncthreads();
    }
    if (t == 0) {
        out[0] = sd[0][0];
        out[1] = sd[0][1];
        out[2] = (double)sl[0][0];
        out[3] = (double)sl[0][1];
        out[4] = (double)sl[0][2];
        out[5] = (double)sl[0][3];
        const int fb = sf[0][0] == 0x7fffffff ? -1 : sf[0][0];
        out[6] = fb;
        out[7] = fb >= 0 ? (double)b.status[fb] : 0.0;
        out[8] = sm[0];
        out[9] = (double)sl[0][4];
        out[10] = sf[0][1] == 0x7fffffff ? -1.0 : (double)sf[0][1];
        out[11] = (double)b.refresh_count[0];
        out[12] = (double)b.refresh_count[1];
    }
}

cudaError_t launch_call_stats(const DevBatch &b, double *out, cudaStream_t stream) {
    call_stats_kernel<<<1, kStatsThreads, 0, stream>>>(b, out);
    return cudaGetLastError();
}

// The label checks of kvmc_set_state and kvmc_init, one warp per walker:
// every label in range, every site holding exactly one spin, no label twice
// (one bitmap per spin in shared memory, `words` 32-bit words each).
// bad[w] = 1 for a walker that fails any of them.
__global__ void __launch_bounds__(32 * kLabelWarps) labels_check_kernel(const int32_t *ku, const int32_t *kd,
                                                                        int n_walkers, int N, int n_up, int n_dn,
                                                                        int words, int *bad) {
    extern __shared__ unsigned seen[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * kLabelWarps + warp;
    if (w >= n_walkers) return;
    unsigned *su = seen + (size_t)warp * 2 * words, *sd = su + words;
    for (int i = lane; i < 2 * words; i += 32) su[i] = 0u;
    __syncwarp();
    const int32_t *u = ku + (size_t)w * N, *d = kd + (size_t)w * N;
    bool ok = true;
    for (int s = lane; s < N; s += 32) {
        const int a = u[s], b = d[s];
        if (a < 0 || a > n_up || b < 0 || b > n_dn || (a != 0) == (b != 0)) {
            ok = false;
            continue;
        }
        const int l = a != 0 ? a : b;
        const unsigned bit = 1u << (l & 31);
        if (atomicOr((a != 0 ? su : sd) + (l >> 5), bit) & bit) ok = false;
    }
    ok = __all_sync(0xffffffffu, ok);
    if (lane == 0) bad[w] = ok ? 0 : 1;
}

// Both spins' labels between the caller's 32-bit layout and the walkers'
// 16-bit labels (to_short: ku, kd -> a, b; otherwise a, b -> ku, kd).
__global__ void labels_convert_kernel(int32_t *ku, int32_t *kd, short *a, short *b, size_t tot, int to_short) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
        if (to_short) {
            a[e] = (short)ku[e];
            b[e] = (short)kd[e];
        } else {
            ku[e] = a[e];
            kd[e] = b[e];
        }
    }
}

size_t labels_check_smem(int n_up, int n_dn) {
    const int words = (n_up > n_dn ? n_up : n_dn) / 32 + 1;
    return (size_t)kLabelWarps * 2 * words * sizeof(unsigned);
}

cudaError_t launch_labels_check(const int32_t *ku, const int32_t *kd, int n_walkers, int N, int n_up, int n_dn,
                                int *bad, cudaStream_t stream) {
    const int words = (n_up > n_dn ? n_up : n_dn) / 32 + 1;
    labels_check_kernel<<<(n_walkers + kLabelWarps - 1) / kLabelWarps, 32 * kLabelWarps,
                          labels_check_smem(n_up, n_dn), stream>>>(ku, kd, n_walkers, N, n_up, n_dn, words, bad);
    return cudaGetLastError();
}

cudaError_t launch_labels_convert(int32_t *ku, int32_t *kd, const DevBatch &b, int N, int to_short,
                                  cudaStream_t stream) {
    const size_t tot = (size_t)b.n_walkers * N;
    const size_t blocks = (tot + 255) / 256;
    labels_convert_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(ku, kd, b.kappa_up, b.kappa_dn,
                                                                                       tot, to_short);
    return cudaGetLastError();
}

cudaError_t launch_clear_status(const DevBatch &b, int bits, cudaStream_t stream) {
    clear_status_bits_kernel<<<(b.n_walkers + 255) / 256, 256, 0, stream>>>(b, bits);
    return cudaGetLastError();
}

cudaError_t launch_refresh32(const DevModel &m, const DevBatch &b, int only_due, int track_drift, cudaStream_t stream) {
    if (!refresh32_supported(m)) return launch_refresh32_large(m, b, only_due, track_drift, stream);
    const size_t sm = refresh32_smem(m);
    cudaError_t e = cudaFuncSetAttribute(refresh32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    refresh32_kernel<<<dim3(b.n_walkers, 2), kThreads32, sm, stream>>>(m, b, only_due, track_drift);
    return cudaGetLastError();
}

}  // namespace kvmc
