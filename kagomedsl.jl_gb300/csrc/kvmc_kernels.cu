// CUDA kernels of libkvmc (sm_103a).
//
// Reference counterparts (KagomeDSL.jl):
//   refresh_kernel      reevaluateW! + tilde_U      src/MonteCarlo.jl:55-115
//   sweep_kernel        Carlo.sweep! + Z + update_configurations! + update_W!
//                       src/MonteCarlo.jl:460-607, measure! :628-634,
//                       getOL src/Hamiltonian.jl:762-778
//   measure_kernel      getOL                       src/Hamiltonian.jl:762-778
//   ratio_kernel        the ratio of src/MonteCarlo.jl:576-580
//   apply_moves_kernel  update_configurations!      src/MonteCarlo.jl:497-511
//   init_random_kernel  seeded random starts (replaces the QR start of
//                       src/MonteCarlo.jl:326-357 for batches of walkers)
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

#include "kvmc.h"
#include "kvmc_device.cuh"
#include "kvmc_refine.cuh"
#include "kvmc_internal.h"

namespace kvmc {

// ---------------------------------------------------------------------------
// Refresh: W_sigma = U_sigma * tilde_U_sigma^{-1} in FP64.
// One CTA per (walker, spin).  tilde_U (row l = U[R,:] with kappa[R] == l) is
// LU-factorised with partial pivoting in shared memory; the rows of W at
// sites not holding this spin are solved one warp per row (w * tilde_U = u,
// forward with the upper factor, backward with the unit-lower factor, then
// the pivot permutation), the rows at occupied sites are unit rows.
// ---------------------------------------------------------------------------
constexpr int kRefreshThreads = 256;

// Rows of W at sites that do not hold this spin: w * tilde_U = u, one
// thread per row.  With P tilde_U = L Uf (row pivots perm): y Uf = u
// (forward), v L = y (backward, unit diagonal), w[perm[i]] = v[i].
// The rows live column-major in an FP64 scratch block (a warp's 32 rows
// form one coalesced segment per column); each thread solves its row in
// blocks of kSolveB columns held in registers, and applies a block to the
// remaining columns eight at a time (eight independent FMA chains).  The
// factor entries are the same for every thread (shared-memory broadcast),
// so no barrier is needed.
constexpr int kSolveB = 16;

template <typename OutT>
__device__ void solve_rows_blocked(const double *A, int lda, const double *invd, const int *perm, const double *U,
                                   int n, const short *rows, int n_rows, double *Y, OutT *Wout, int ldw,
                                   float *drift_slot, bool track_drift, const short *krow = nullptr) {
    const int r = threadIdx.x;
    float dmax = 0.f;
    if (r < n_rows) {
        const int ld = n_rows;
        const int R = rows[r];
        for (int j = 0; j < n; ++j) Y[(size_t)j * ld + r] = U[(size_t)R * n + j];
        // forward: y * Uf = u
        for (int jb = 0; jb < n; jb += kSolveB) {
            const int nb = min(kSolveB, n - jb);
            double yb[kSolveB];
#pragma unroll
            for (int q = 0; q < kSolveB; ++q) yb[q] = q < nb ? Y[(size_t)(jb + q) * ld + r] : 0.0;
#pragma unroll
            for (int ii = 0; ii < kSolveB; ++ii) {
                if (ii < nb) {
                    yb[ii] *= invd[jb + ii];
                    const double *Ai = A + (size_t)(jb + ii) * lda + jb;
#pragma unroll
                    for (int jj = ii + 1; jj < kSolveB; ++jj)
                        if (jj < nb) yb[jj] = fma(-yb[ii], Ai[jj], yb[jj]);
                }
            }
#pragma unroll
            for (int q = 0; q < kSolveB; ++q)
                if (q < nb) Y[(size_t)(jb + q) * ld + r] = yb[q];
            for (int j0 = jb + kSolveB; j0 < n; j0 += 8) {
                const int cnt = min(8, n - j0);
                double acc[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) acc[t] = t < cnt ? Y[(size_t)(j0 + t) * ld + r] : 0.0;
#pragma unroll
                for (int ii = 0; ii < kSolveB; ++ii) {
                    if (ii < nb) {
                        const double *Ai = A + (size_t)(jb + ii) * lda + j0;
#pragma unroll
                        for (int t = 0; t < 8; ++t)
                            if (t < cnt) acc[t] = fma(-yb[ii], Ai[t], acc[t]);
                    }
                }
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    if (t < cnt) Y[(size_t)(j0 + t) * ld + r] = acc[t];
            }
        }
        // backward: v * L = y (L unit lower, L[j][i] = A[j][i] for j > i)
        const int last = ((n - 1) / kSolveB) * kSolveB;
        for (int jb = last; jb >= 0; jb -= kSolveB) {
            const int nb = min(kSolveB, n - jb);
            double yb[kSolveB];
#pragma unroll
            for (int q = 0; q < kSolveB; ++q) yb[q] = q < nb ? Y[(size_t)(jb + q) * ld + r] : 0.0;
#pragma unroll
            for (int ii = kSolveB - 1; ii >= 0; --ii) {
                if (ii < nb) {
                    const double *Aj = A + (size_t)(jb + ii) * lda + jb;
#pragma unroll
                    for (int kk = 0; kk < ii; ++kk) yb[kk] = fma(-yb[ii], Aj[kk], yb[kk]);
                }
            }
#pragma unroll
            for (int q = 0; q < kSolveB; ++q)
                if (q < nb) Y[(size_t)(jb + q) * ld + r] = yb[q];
            for (int i0 = 0; i0 < jb; i0 += 8) {
                const int cnt = min(8, jb - i0);
                double acc[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) acc[t] = t < cnt ? Y[(size_t)(i0 + t) * ld + r] : 0.0;
#pragma unroll
                for (int ii = 0; ii < kSolveB; ++ii) {
                    if (ii < nb) {
                        const double *Aj = A + (size_t)(jb + ii) * lda + i0;
#pragma unroll
                        for (int t = 0; t < 8; ++t)
                            if (t < cnt) acc[t] = fma(-yb[ii], Aj[t], acc[t]);
                    }
                }
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    if (t < cnt) Y[(size_t)(i0 + t) * ld + r] = acc[t];
            }
        }
        // krow: the label-indexed blocks of the one-warp sweep (row = the other
        // spin's label at site R); null: site-indexed W
        OutT *wr = Wout + (size_t)(krow ? krow[R] - 1 : R) * ldw;
        for (int i = 0; i < n; ++i) {
            const OutT nv = (OutT)Y[(size_t)i * ld + r];
            if (track_drift) {
                const float o = (float)wr[perm[i]];
                dmax = fmaxf(dmax, fabsf(o - (float)nv) / (1.f + fabsf((float)nv)));
            }
            wr[perm[i]] = nv;
        }
    }
    if (track_drift) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if ((threadIdx.x & 31) == 0 && dmax > 0.f) atomic_max_nonneg(drift_slot, dmax);
    }
}

// tilde_U into A (row l = U[R,:] with kappa[R] == l; zero-filled first so a
// configuration missing a label is singular), perm = identity.  All threads.
template <typename KT>
__device__ void gather_tilde_u(double *A, int lda, int *perm, const double *U, const KT *kappa, int N, int n) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    for (int e = tid; e < n * lda; e += nt) A[e] = 0.0;
    __syncthreads();
    for (int R = warp; R < N; R += nt / 32) {
        const int l = (int)kappa[R];
        if (l >= 1 && l <= n) {
            const double *src = U + (size_t)R * n;
            double *dst = A + (size_t)(l - 1) * lda;
            for (int c = lane; c < n; c += 32) dst[c] = src[c];
        }
    }
    for (int i = tid; i < n; i += nt) perm[i] = i;
    __syncthreads();
}

// LU with partial pivoting of A in shared memory (first maximal |pivot|
// wins, as LAPACK i*amax): P A = L Uf in place, perm tracks the row
// pivots.  All threads; returns true when A is exactly singular.  Otherwise
// invd receives 1/Uf[i][i], logdet = log|det A| and log_ratio =
// log(min|Uf[i][i]| / max|Uf[i][i]|).
__device__ bool lu_factor_shared(double *A, int lda, int n, int *perm, double *invd, double *red, double &logdet,
                                 double &log_ratio) {
    __shared__ int s_piv;
    __shared__ double s_pmax, s_dinv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            double best = -1.0;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                const double v = fabs(A[(size_t)i * lda + k]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            // one lane divides (FP64 division is a long FP64 sequence on this part)
            if (lane == 0) {
                s_piv = bi;
                s_pmax = best;
                s_dinv = best > 0.0 ? 1.0 / A[(size_t)bi * lda + k] : 0.0;
            }
        }
        __syncthreads();
        const int p = s_piv;
        if (!(s_pmax > 0.0)) return true;  // exactly singular (or NaN): every thread sees it
        if (p != k) {
            for (int j = tid; j < n; j += nt) {
                const double a = A[(size_t)k * lda + j];
                A[(size_t)k * lda + j] = A[(size_t)p * lda + j];
                A[(size_t)p * lda + j] = a;
            }
            if (tid == 0) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
        }
        __syncthreads();
        const double dinv = s_dinv;
        for (int i = k + 1 + tid; i < n; i += nt) A[(size_t)i * lda + k] *= dinv;
        __syncthreads();
        // trailing update: warp rows, lane columns
        for (int i = k + 1 + warp; i < n; i += nt / 32) {
            const double aik = A[(size_t)i * lda + k];
            double *Ai = A + (size_t)i * lda;
            const double *Ak = A + (size_t)k * lda;
            for (int j = k + 1 + lane; j < n; j += 32) Ai[j] = fma(-aik, Ak[j], Ai[j]);
        }
        __syncthreads();
    }
    double ld = 0.0, dmin = INFINITY, dmaxp = 0.0;
    for (int i = tid; i < n; i += nt) {
        const double d = A[(size_t)i * lda + i];
        invd[i] = 1.0 / d;
        ld += log(fabs(d));
        dmin = fmin(dmin, fabs(d));
        dmaxp = fmax(dmaxp, fabs(d));
    }
    logdet = block_sum(ld, red);
    dmin = -block_sum_max(-dmin, red);
    dmaxp = block_sum_max(dmaxp, red);
    log_ratio = log(dmin / dmaxp);
    return false;
}

// Sites not holding this spin, in site order (warp 0 fills rows; every
// thread gets the count).
template <typename KT>
__device__ int collect_empty_rows(const KT *kappa, int N, short *rows) {
    __shared__ int s_nrows;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
    return s_nrows;
}

// Unit rows at occupied sites (W[R][kappa[R]-1] = 1), zero padding columns
// elsewhere.  All threads.
template <typename KT, typename OutT>
__device__ void write_unit_rows(const KT *kappa, int N, int n, OutT *W, int ldw, bool track_drift, float *drift_slot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nt = blockDim.x;
    for (int R = warp; R < N; R += nt / 32) {
        const int l = (int)kappa[R];
        OutT *wr = W + (size_t)R * ldw;
        if (l != 0) {
            float dmax = 0.f;
            for (int c = lane; c < ldw; c += 32) {
                const OutT nv = (OutT)((c == l - 1) ? 1.0 : 0.0);
                if (track_drift) dmax = fmaxf(dmax, fabsf((float)wr[c] - (float)nv) / (1.f + fabsf((float)nv)));
                wr[c] = nv;
            }
            if (track_drift) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
                if (lane == 0 && dmax > 0.f) atomic_max_nonneg(drift_slot, dmax);
            }
        } else {
            for (int c = n + lane; c < ldw; c += 32) wr[c] = (OutT)0;
        }
    }
}

template <typename OutT>
__global__ void __launch_bounds__(kRefreshThreads, 2)
refresh_kernel(DevModel m, DevBatch b, int only_due, int track_drift) {
    const int w = blockIdx.x;
    const int spin = blockIdx.y;
    if (only_due == 1 && b.since[w] >= 0) return;  // a negative `since` marks a refresh as due
    if (only_due == 2 && !(b.status[w] & kStatusRefine)) return;  // the FP32 refresh gave this walker up

    if (spin == 0 && threadIdx.x == 0) atomicAdd(b.refresh_count + (only_due == 2 ? 1 : 0), 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const double *U = spin == 0 ? m.U_up : m.U_dn;
    const short *kappa = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    // during a one-warp sweep call the FP32 rows go to the label-indexed blocks
    const bool cpt = sizeof(OutT) == 4 && b.compact;
    OutT *W = cpt ? (OutT *)(b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up))
                  : (sizeof(OutT) == 8 ? (OutT *)b.W64 : (OutT *)b.W32) + (size_t)w * wblock +
                        (spin == 0 ? 0 : (size_t)N * m.ld_up);
    const short *krow = cpt ? (spin == 0 ? b.kappa_dn : b.kappa_up) + (size_t)w * N : nullptr;

    extern __shared__ __align__(16) unsigned char smem[];
    const int lda = n + 1;  // odd stride: column reads hit distinct banks
    double *A = reinterpret_cast<double *>(smem);
    double *invd = A + (size_t)n * lda;
    double *red = invd + n;                       // 33 doubles
    int *perm = reinterpret_cast<int *>(red + 33);
    short *rows = reinterpret_cast<short *>(perm + n);
    // FP64 scratch for the solved rows, [n][rows] column-major, one block per (walker, spin)
    double *Y = b.solve_scratch + ((size_t)w * 2 + spin) * b.solve_block;

    gather_tilde_u(A, lda, perm, U, kappa, N, n);
    double logdet = 0.0, log_ratio = 0.0;
    if (lu_factor_shared(A, lda, n, perm, invd, red, logdet, log_ratio)) {
        if (threadIdx.x == 0) {
            atomicOr(&b.status[w], kStatusSingular);
            b.logdet[4 * w + spin] = -INFINITY;
            b.logdet[4 * w + 2 + spin] = -INFINITY;
        }
        return;
    }
    if (threadIdx.x == 0) {
        b.logdet[4 * w + spin] = logdet;
        b.logdet[4 * w + 2 + spin] = log_ratio;
    }
    const int nrows = collect_empty_rows(kappa, N, rows);
    if (!cpt) write_unit_rows(kappa, N, n, W, ldw, track_drift != 0, &b.drift[w]);
    for (int r0 = 0; r0 < nrows; r0 += blockDim.x) {
        const int cnt = min((int)blockDim.x, nrows - r0);
        solve_rows_blocked<OutT>(A, lda, invd, perm, U, n, rows + r0, cnt, Y + (size_t)r0 * n, W, ldw, &b.drift[w],
                                 track_drift != 0, krow);
    }
}

// ---------------------------------------------------------------------------
// Refresh for more than kSmemLuMaxN orbitals per spin: tilde_U no longer fits
// in shared memory, so it is factorised in place in an FP64 scratch block in
// HBM with a blocked right-looking LU (panel width kPanel, partial pivoting):
//   1. the n - pb by kPanel panel is factorised in shared memory,
//   2. its row swaps are applied to the columns outside the panel,
//   3. U12 = L11^{-1} A12 (unit lower triangular solve, one thread per column),
//   4. A22 -= L21 U12 (FP64 GEMM, 4 x 4 register tiles per thread).
// The factors then feed the same row solver as the shared-memory path.
// ---------------------------------------------------------------------------
constexpr int kPanel = 32;
constexpr int kSmemLuMaxN = 160;

// LT: the arithmetic of the LU.  double = the FP64 refresh; float = the LU of
// the FP32 refinement refresh (kvmc_refine.cuh), whose rows are then refined
// against the exact-product residual (mixed real form, OutT float).
template <typename LT, typename OutT>
__global__ void __launch_bounds__(kRefreshThreads)
refresh_large_kernel(DevModel m, DevBatch b, int only_due, int track_drift) {
    constexpr bool kF32 = sizeof(LT) == 4;
    const int w = blockIdx.x;
    const int spin = blockIdx.y;
    // FP64: the row solves run in refresh_large_rows_kernel when lu_perm is set;
    // this launch marks the walker-spin's LU as not (yet) done
    int *lu_flag = (!kF32 && b.lu_perm) ? b.lu_perm + ((size_t)w * 2 + spin) * (b.lu_aux_n + 1) + b.lu_aux_n : nullptr;
    if (lu_flag && threadIdx.x == 0) *lu_flag = 0;
    if (only_due == 1 && b.since[w] >= 0) return;
    if (only_due == 2 && !(b.status[w] & kStatusRefine)) return;
    if (spin == 0 && threadIdx.x == 0) atomicAdd(b.refresh_count + (only_due == 2 ? 1 : 0), 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const double *U = spin == 0 ? m.U_up : m.U_dn;
    const short *kappa = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    const bool cpt = sizeof(OutT) == 4 && b.compact;
    OutT *W = cpt ? (OutT *)(b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up))
                  : (sizeof(OutT) == 8 ? (OutT *)b.W64 : (OutT *)b.W32) + (size_t)w * wblock +
                        (spin == 0 ? 0 : (size_t)N * m.ld_up);
    const short *krow = cpt ? (spin == 0 ? b.kappa_dn : b.kappa_up) + (size_t)w * N : nullptr;
    LT *A = reinterpret_cast<LT *>(b.lu_scratch) + ((size_t)w * 2 + spin) * b.lu_block;  // n x n, lda = n
    double *Y = b.solve_scratch + ((size_t)w * 2 + spin) * b.solve_block;

    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int ldp = kPanel + 1;
    double *red = reinterpret_cast<double *>(smem);          // 33 doubles
    LT *Pn = reinterpret_cast<LT *>(red + 33);               // panel [n][ldp]
    LT *Ut = Pn + (size_t)n * ldp;                           // U12 tile [kPanel][64]
    LT *invd = Ut + kPanel * 64;
    int *perm = reinterpret_cast<int *>(invd + n);
    int *ipiv = perm + n;
    short *rows = reinterpret_cast<short *>(ipiv + n);
    short *site_of = rows + N;                               // FP32 path: the site holding each label
    __shared__ int s_piv;
    __shared__ LT s_pmax, s_dinv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;

    // gather tilde_U into A (zeroed first)
    for (size_t e = tid; e < (size_t)n * n; e += nt) A[e] = LT(0);
    __syncthreads();
    const float *Uh = spin == 0 ? m.U32_up_hi : m.U32_dn_hi;
    for (int R = warp; R < N; R += nt / 32) {
        const int l = kappa[R];
        if (l >= 1 && l <= n) {
            LT *dst = A + (size_t)(l - 1) * n;
            if constexpr (kF32) {
                const float *src = Uh + (size_t)R * n;
                for (int c = lane; c < n; c += 32) dst[c] = src[c];
            } else {
                const double *src = U + (size_t)R * n;
                for (int c = lane; c < n; c += 32) dst[c] = src[c];
            }
        }
    }
    for (int i = tid; i < n; i += nt) perm[i] = i;
    __syncthreads();

    bool singular = false;
    for (int pb = 0; pb < n && !singular; pb += kPanel) {
        const int nb = min(kPanel, n - pb);
        const int rp = n - pb;
        // 1. panel into shared memory
        for (int e = tid; e < rp * nb; e += nt) {
            const int r = e / nb, c = e - r * nb;
            Pn[(size_t)r * ldp + c] = A[(size_t)(pb + r) * n + pb + c];
        }
        __syncthreads();
        for (int k = 0; k < nb; ++k) {
            if (warp == 0) {
                LT best = LT(-1);
                int bi = rp;
                for (int i = k + lane; i < rp; i += 32) {
                    const LT v = fabs(Pn[(size_t)i * ldp + k]);
                    if (v > best) { best = v; bi = i; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const LT ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
                if (lane == 0) {
                    s_piv = bi;
                    s_pmax = best;
                    s_dinv = best > LT(0) ? LT(1) / Pn[(size_t)bi * ldp + k] : LT(0);
                    ipiv[pb + k] = pb + bi;
                }
            }
            __syncthreads();
            if (!(s_pmax > LT(0))) { singular = true; break; }
            const int p = s_piv;
            if (p != k)
                for (int j = tid; j < nb; j += nt) {
                    const LT a = Pn[(size_t)k * ldp + j];
                    Pn[(size_t)k * ldp + j] = Pn[(size_t)p * ldp + j];
                    Pn[(size_t)p * ldp + j] = a;
                }
            __syncthreads();
            const LT dinv = s_dinv;
            for (int i = k + 1 + tid; i < rp; i += nt) Pn[(size_t)i * ldp + k] *= dinv;
            __syncthreads();
            for (int e = tid; e < (rp - k - 1) * (nb - k - 1); e += nt) {
                const int i = k + 1 + e / (nb - k - 1), j = k + 1 + e % (nb - k - 1);
                Pn[(size_t)i * ldp + j] = fma(-Pn[(size_t)i * ldp + k], Pn[(size_t)k * ldp + j], Pn[(size_t)i * ldp + j]);
            }
            __syncthreads();
        }
        if (singular) break;
        // panel back to A
        for (int e = tid; e < rp * nb; e += nt) {
            const int r = e / nb, c = e - r * nb;
            A[(size_t)(pb + r) * n + pb + c] = Pn[(size_t)r * ldp + c];
        }
        // 2. the panel's row swaps on the other columns, in order
        for (int k = 0; k < nb; ++k) {
            const int r1 = pb + k, r2 = ipiv[pb + k];
            if (r1 != r2) {
                for (int c = tid; c < n; c += nt) {
                    if (c >= pb && c < pb + nb) continue;
                    const LT a = A[(size_t)r1 * n + c];
                    A[(size_t)r1 * n + c] = A[(size_t)r2 * n + c];
                    A[(size_t)r2 * n + c] = a;
                }
                if (tid == 0) { const int t = perm[r1]; perm[r1] = perm[r2]; perm[r2] = t; }
            }
            __syncthreads();
        }
        const int c0 = pb + nb;
        if (c0 < n) {
            // 3. U12 = L11^{-1} A12, one column per thread
            for (int c = c0 + tid; c < n; c += nt) {
                LT x[kPanel];
#pragma unroll
                for (int i = 0; i < kPanel; ++i) x[i] = i < nb ? A[(size_t)(pb + i) * n + c] : LT(0);
#pragma unroll
                for (int i = 1; i < kPanel; ++i) {
                    if (i < nb) {
                        LT acc = x[i];
#pragma unroll
                        for (int k = 0; k < i; ++k) acc = fma(-Pn[(size_t)i * ldp + k], x[k], acc);
                        x[i] = acc;
                    }
                }
#pragma unroll
                for (int i = 0; i < kPanel; ++i)
                    if (i < nb) A[(size_t)(pb + i) * n + c] = x[i];
            }
            __syncthreads();
            // 4. A22 -= L21 U12: 64-column tiles of U12 staged in shared memory,
            //    each thread a 4 x 4 tile (rows r0 + 4*ty + {0..3}, cols 4*tx + {0..3})
            const int tx = tid & 15, ty = tid >> 4;
            for (int cb = c0; cb < n; cb += 64) {
                const int ncol = min(64, n - cb);
                for (int e = tid; e < nb * 64; e += nt) {
                    const int k = e >> 6, c = e & 63;
                    Ut[e] = c < ncol ? A[(size_t)(pb + k) * n + cb + c] : LT(0);
                }
                __syncthreads();
                for (int rb = c0; rb < n; rb += 64) {
                    LT acc[4][4];
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[a][q] = LT(0);
                    for (int k = 0; k < nb; ++k) {
                        LT lv[4], uv[4];
#pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            const int r = rb + 4 * ty + a;
                            lv[a] = r < n ? Pn[(size_t)(r - pb) * ldp + k] : LT(0);
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q) uv[q] = Ut[k * 64 + 4 * tx + q];
#pragma unroll
                        for (int a = 0; a < 4; ++a)
#pragma unroll
                            for (int q = 0; q < 4; ++q) acc[a][q] = fma(lv[a], uv[q], acc[a][q]);
                    }
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int r = rb + 4 * ty + a;
                        if (r >= n) continue;
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int c = cb + 4 * tx + q;
                            if (c < n) A[(size_t)r * n + c] -= acc[a][q];
                        }
                    }
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
    if (singular) {
        if (threadIdx.x == 0) {
            if constexpr (kF32) {
                atomicOr(&b.status[w], kStatusRefine);  // an exactly zero FP32 pivot: the FP64 refresh decides
            } else {
                atomicOr(&b.status[w], kStatusSingular);
                b.logdet[4 * w + spin] = -INFINITY;
                b.logdet[4 * w + 2 + spin] = -INFINITY;
            }
        }
        return;
    }
    double ld = 0.0, dmin = INFINITY, dmaxp = 0.0;
    for (int i = tid; i < n; i += nt) {
        const double d = (double)A[(size_t)i * n + i];
        invd[i] = LT(1) / A[(size_t)i * n + i];
        ld += log(fabs(d));
        dmin = fmin(dmin, fabs(d));
        dmaxp = fmax(dmaxp, fabs(d));
    }
    ld = block_sum(ld, red);
    dmin = -block_sum_max(-dmin, red);
    dmaxp = block_sum_max(dmaxp, red);
    if (tid == 0) {
        b.logdet[4 * w + spin] = ld;
        b.logdet[4 * w + 2 + spin] = log(dmin / dmaxp);
    }
    const int nrows = collect_empty_rows(kappa, N, rows);
    if (!cpt) write_unit_rows(kappa, N, n, W, ldw, track_drift != 0, &b.drift[w]);
    if constexpr (kF32) {
        for (int i = tid; i < n; i += nt) site_of[i] = -1;
        __syncthreads();
        for (int R = tid; R < N; R += nt) {
            const int l = kappa[R];
            if (l >= 1 && l <= n) site_of[l - 1] = (short)R;
        }
        __syncthreads();
        const float *Ul = spin == 0 ? m.U32_up_lo : m.U32_dn_lo;
        float *Yf = reinterpret_cast<float *>(Y);
        float dmax = 0.f;
        for (int r0 = 0; r0 < nrows; r0 += blockDim.x) {
            const int cnt = min((int)blockDim.x, nrows - r0);
            if (tid < cnt) {
                const int R = rows[r0 + tid];
                if (!refine_row(A, n, invd, perm, site_of, Uh, Ul, n, R, Yf + (size_t)r0 * n * 2 + tid, cnt,
                                reinterpret_cast<float *>(W) + (size_t)(krow ? krow[R] - 1 : R) * ldw,
                                track_drift != 0, dmax))
                    atomicOr(&b.status[w], kStatusRefine);
            }
        }
        if (track_drift) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
            if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
        }
    } else if (lu_flag) {
        // the factors' 1/diag and pivot order for the row solves' launch
        double *gi = b.lu_invd + ((size_t)w * 2 + spin) * b.lu_aux_n;
        int *gp = b.lu_perm + ((size_t)w * 2 + spin) * (b.lu_aux_n + 1);
        for (int i = tid; i < n; i += nt) {
            gi[i] = (double)invd[i];
            gp[i] = perm[i];
        }
        if (tid == 0) *lu_flag = 1;
        (void)nrows;
        (void)Y;
    } else {
        for (int r0 = 0; r0 < nrows; r0 += blockDim.x) {
            const int cnt = min((int)blockDim.x, nrows - r0);
            solve_rows_blocked<OutT>(A, n, invd, perm, U, n, rows + r0, cnt, Y + (size_t)r0 * n, W, ldw, &b.drift[w],
                                     track_drift != 0, krow);
        }
    }
}

// The row solves of the FP64 refresh beyond kSmemLuMaxN orbitals, after
// refresh_large_kernel has factorised tilde_U: CTA z of (walker, spin)
// solves the rows z * kRowsThreads .. of the sites not holding the spin, one
// thread per row (solve_rows_blocked), so the N - n rows of one walker-spin
// spread over many SMs' FP64 pipes instead of one.
constexpr int kRowsThreads = 64;

template <typename OutT>
__global__ void __launch_bounds__(kRowsThreads) refresh_large_rows_kernel(DevModel m, DevBatch b, int track_drift) {
    const int w = blockIdx.x, spin = blockIdx.y;
    const size_t ws = (size_t)w * 2 + spin;
    const int *gp = b.lu_perm + ws * (b.lu_aux_n + 1);
    if (gp[b.lu_aux_n] != 1) return;
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int r0 = blockIdx.z * kRowsThreads;
    if (r0 >= N - n) return;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const double *U = spin == 0 ? m.U_up : m.U_dn;
    const short *kappa = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    const bool cpt = sizeof(OutT) == 4 && b.compact;
    OutT *W = cpt ? (OutT *)(b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up))
                  : (sizeof(OutT) == 8 ? (OutT *)b.W64 : (OutT *)b.W32) + (size_t)w * wblock +
                        (spin == 0 ? 0 : (size_t)N * m.ld_up);
    const short *krow = cpt ? (spin == 0 ? b.kappa_dn : b.kappa_up) + (size_t)w * N : nullptr;
    const double *A = b.lu_scratch + ws * b.lu_block;
    double *Y = b.solve_scratch + ws * b.solve_block;
    extern __shared__ __align__(16) unsigned char smem[];
    double *invd = reinterpret_cast<double *>(smem);
    int *perm = reinterpret_cast<int *>(invd + n);
    short *rows = reinterpret_cast<short *>(perm + n);
    const double *gi = b.lu_invd + ws * b.lu_aux_n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        invd[i] = gi[i];
        perm[i] = gp[i];
    }
    const int nrows = collect_empty_rows(kappa, N, rows);   // synchronises the block
    const int cnt = min(kRowsThreads, nrows - r0);
    if (cnt <= 0) return;
    solve_rows_blocked<OutT>(A, n, invd, perm, U, n, rows + r0, cnt, Y + (size_t)r0 * n, W, ldw, &b.drift[w],
                             track_drift != 0, krow);
}

size_t refresh_large_smem(const DevModel &m, size_t lt_bytes) {
    const int n = m.n_up > m.n_dn ? m.n_up : m.n_dn;
    return 33 * 8 + ((size_t)n * (kPanel + 1) + kPanel * 64 + (size_t)n) * lt_bytes + (size_t)n * 8 +
           (size_t)m.n_sites * 2 + (size_t)n * 2 + 16;
}

size_t refresh_large_smem(const DevModel &m) { return refresh_large_smem(m, 8); }

bool refresh_needs_large(const DevModel &m) { return (m.n_up > m.n_dn ? m.n_up : m.n_dn) > kSmemLuMaxN; }

size_t refresh_smem(const DevModel &m) {
    const int n = m.n_up > m.n_dn ? m.n_up : m.n_dn;
    return (size_t)n * (n + 1) * 8 + (size_t)n * 8 + 33 * 8 + (size_t)n * 4 + (size_t)m.n_sites * 2 + 16;
}

// FP64 scratch doubles per (walker, spin) for the solved rows.
size_t refresh_scratch_block(const DevModel &m) {
    const int n = m.n_up > m.n_dn ? m.n_up : m.n_dn;
    const int rows = m.n_sites - (m.n_up < m.n_dn ? m.n_up : m.n_dn);
    return (size_t)n * rows;
}

// ---------------------------------------------------------------------------
// Sweep: proposals of one walker per CTA.
//
// Warp 0 evaluates proposals t..t+31 of its walker at once against the
// current state; the first accepted lane is the next accepted move (all
// earlier lanes were rejected against exactly the state they would have seen
// one at a time, so the chain is the sequential one).  Then the whole CTA
// applies the Sherman-Morrison update to both W matrices.
//
// T = double, W in global memory: the plain FP64 form.
// T = float,  W staged in shared memory: the mixed form.
// ---------------------------------------------------------------------------
struct SweepCtl {
    long long t, tend, next_meas, next_ref;
    int since, zmu, state;
    int Ku, lu, Kd, ld;
    Thr thr;
    double red[33];
};

template <typename T>
struct WPtr {
    T *up, *dn;
    int ld_up, ld_dn;
    __device__ __forceinline__ T &U(int r, int c) const { return up[(size_t)r * ld_up + c]; }
    __device__ __forceinline__ T &D(int r, int c) const { return dn[(size_t)r * ld_dn + c]; }
};

// Local energy of the state (src/Hamiltonian.jl:593-778): the plain form
// sums in FP64 throughout; the FP32 form sums each thread's terms and each
// warp in FP32 and the warp partials in FP64.
template <typename T>
__device__ double local_energy(const DevModel &m, const short2 *bonds, const short *kup,
                               const short *kdn, const WPtr<T> &W, double *red) {
    T acc = 0;
    for (int e = threadIdx.x; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = bonds[e];
        const int i = bd.x, j = bd.y;
        const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
        acc += ((ui != 0) == (uj != 0)) ? (T)0.25 : (T)-0.25;
        if (uj != 0 && di != 0) acc -= (T)0.5 * W.U(i, uj - 1) * W.D(j, di - 1);
        if (ui != 0 && dj != 0) acc -= (T)0.5 * W.U(j, ui - 1) * W.D(i, dj - 1);
    }
    if constexpr (sizeof(T) == 4) return block_sum_f32(acc, red);
    else return block_sum(acc, red);
}

// Sherman-Morrison update of both spins (src/MonteCarlo.jl:279-292):
// W <- W - W[:,l] (W[K,:] - e_l) / W[K,l].  col/row staging buffers hold
// N + ld entries per spin.
template <typename T>
__device__ void rank1_update(const WPtr<T> &W, int N, int Ku, int lu, int Kd, int ld, T *stg_col_u,
                             T *stg_row_u, T *stg_col_d, T *stg_row_d) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const T au = (T)(-1.0) / W.U(Ku, lu);
    const T ad = (T)(-1.0) / W.D(Kd, ld);
    for (int r = tid; r < N; r += nt) {
        stg_col_u[r] = W.U(r, lu) * au;
        stg_col_d[r] = W.D(r, ld) * ad;
    }
    for (int c = tid; c < W.ld_up; c += nt) stg_row_u[c] = W.U(Ku, c) - (c == lu ? (T)1 : (T)0);
    for (int c = tid; c < W.ld_dn; c += nt) stg_row_d[c] = W.D(Kd, c) - (c == ld ? (T)1 : (T)0);
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
        const int q_up = W.ld_up >> 2, q_dn = W.ld_dn >> 2;
        const int tot_up = N * q_up, tot = tot_up + N * q_dn;
        for (int e = tid; e < tot; e += nt) {
            const bool is_up = e < tot_up;
            const int ee = is_up ? e : e - tot_up;
            const int q = is_up ? q_up : q_dn;
            const int r = ee / q, c4 = ee - r * q;
            float4 *wp = reinterpret_cast<float4 *>(is_up ? W.up : W.dn) + (size_t)r * q + c4;
            const float cv = is_up ? stg_col_u[r] : stg_col_d[r];
            const float4 rv = reinterpret_cast<const float4 *>(is_up ? stg_row_u : stg_row_d)[c4];
            float4 v = *wp;
            v.x = fmaf(cv, rv.x, v.x);
            v.y = fmaf(cv, rv.y, v.y);
            v.z = fmaf(cv, rv.z, v.z);
            v.w = fmaf(cv, rv.w, v.w);
            *wp = v;
        }
    } else {
        const int tot_up = N * W.ld_up, tot = tot_up + N * W.ld_dn;
        for (int e = tid; e < tot; e += nt) {
            const bool is_up = e < tot_up;
            const int ee = is_up ? e : e - tot_up;
            const int q = is_up ? W.ld_up : W.ld_dn;
            const int r = ee / q, c = ee - r * q;
            T *wp = (is_up ? W.up : W.dn) + (size_t)r * q + c;
            const T cv = is_up ? stg_col_u[r] : stg_col_d[r];
            const T rv = is_up ? stg_row_u[c] : stg_row_d[c];
            *wp = fma(cv, rv, *wp);
        }
    }
    __syncthreads();
}

template <typename T, bool kSmemW>
__global__ void sweep_kernel(DevModel m, DevBatch b, SweepParams p, int refresh_by_proposals,
                             int *active_count) {
    const int w = blockIdx.x;
    const int N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    const long long t0 = b.t[w];
    const long long tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);  // this launch's share
    const long long acc_left = b.acc_end[w] - b.accepted[w];  // accepted moves still wanted
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        // nothing to do; a refresh marked due has run since (stream order), clear the mark
        if (threadIdx.x == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }

    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ SweepCtl ctl;

    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    T *gW = (sizeof(T) == 8 ? (T *)b.W64 : (T *)b.W32) + (size_t)w * wblock;
    unsigned char *cur = smem;
    WPtr<T> W;
    W.ld_up = m.ld_up;
    W.ld_dn = m.ld_dn;
    if constexpr (kSmemW) {
        T *sW = reinterpret_cast<T *>(cur);
        const int nvec = (int)(wblock * sizeof(T) / 16);
        const float4 *src = reinterpret_cast<const float4 *>(gW);
        float4 *dst = reinterpret_cast<float4 *>(sW);
        for (int e = tid; e < nvec; e += blockDim.x) dst[e] = src[e];
        W.up = sW;
        W.dn = sW + (size_t)N * m.ld_up;
        cur += wblock * sizeof(T);
    } else {
        W.up = gW;
        W.dn = gW + (size_t)N * m.ld_up;
    }
    T *stg_col_u = reinterpret_cast<T *>(cur); cur += (size_t)N * sizeof(T);
    T *stg_col_d = reinterpret_cast<T *>(cur); cur += (size_t)N * sizeof(T);
    T *stg_row_u = reinterpret_cast<T *>(cur); cur += (size_t)m.ld_up * sizeof(T);
    T *stg_row_d = reinterpret_cast<T *>(cur); cur += (size_t)m.ld_dn * sizeof(T);
    short2 *bonds = reinterpret_cast<short2 *>(cur); cur += (size_t)m.n_bonds * sizeof(short2);
    short *kup = reinterpret_cast<short *>(cur); cur += (size_t)N * sizeof(short);
    short *kdn = reinterpret_cast<short *>(cur);

    for (int e = tid; e < m.n_bonds; e += blockDim.x) bonds[e] = m.bonds[e];
    for (int s = tid; s < N; s += blockDim.x) {
        kup[s] = b.kappa_up[(size_t)w * N + s];
        kdn[s] = b.kappa_dn[(size_t)w * N + s];
    }
    __syncthreads();
    // Z_mu (src/MonteCarlo.jl:460-474)
    double zc = 0.0;
    for (int e = tid; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = bonds[e];
        zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
    }
    zc = block_sum(zc, ctl.red);
    const int R = p.refresh_every;
    const int M = p.measure_every;
    if (tid == 0) {
        ctl.t = t0;
        ctl.tend = tend;
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
            int state = 2;  // 2 = stop, 1 = accepted move, 3 = measurement or refresh boundary
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
                        const short2 bd = bonds[bi];
                        const int i = bd.x, j = bd.y;
                        const int kui = kup[i], kuj = kup[j], kdi = kdn[i], kdj = kdn[j];
                        const bool f1 = kui != 0 && kdj != 0;
                        const bool f2 = kuj != 0 && kdi != 0;
                        if (f1 || f2) {
                            if (f1) { Ku = j; lu = kui - 1; Kd = i; ld = kdj - 1; }
                            else    { Ku = i; lu = kuj - 1; Kd = j; ld = kdi - 1; }
                            acc = decide(W.U(Ku, lu), W.D(Kd, ld), u53, c, thr, p.accept_rule, bad);
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
            rank1_update<T>(W, N, Ku, lu, Kd, ld, stg_col_u, stg_row_u, stg_col_d, stg_row_d);
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
            const double e = local_energy<T>(m, bonds, kup, kdn, W, ctl.red);
            if (tid == 0) {  // only thread 0 keeps the FP64 sums
                se += e;
                se2 += e * e;
                n_meas += 1;
                ctl.next_meas += M;
            }
        }
        if (t == ctl.next_ref) break;  // refresh boundary (plain form): hand over to the refresh kernel
        __syncthreads();
    }
    __syncthreads();

    // write back
    if constexpr (kSmemW) {
        const int nvec = (int)(wblock * sizeof(T) / 16);
        const float4 *src = reinterpret_cast<const float4 *>(W.up);
        float4 *dst = reinterpret_cast<float4 *>(gW);
        for (int e = tid; e < nvec; e += blockDim.x) dst[e] = src[e];
    }
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

template <typename T, bool kSmemW>
size_t sweep_smem_bytes(const DevModel &m) {
    const size_t wblock = (size_t)m.n_sites * (m.ld_up + m.ld_dn);
    size_t s = kSmemW ? wblock * sizeof(T) : 0;
    s += (size_t)(2 * m.n_sites + m.ld_up + m.ld_dn) * sizeof(T);
    s += (size_t)m.n_bonds * sizeof(short2);
    s += (size_t)2 * m.n_sites * sizeof(short) + 16;
    return s;
}

size_t mixed_sweep_smem(const DevModel &m) { return sweep_smem_bytes<float, true>(m); }

// ---------------------------------------------------------------------------
// Mixed form with delayed updates (McDaniel, Mihm, Sanderson, Kent 2017,
// "Delayed Slater determinant update algorithms for high efficiency quantum
// Monte Carlo", J. Chem. Phys. 147, 174107).
//
// W (FP32) stays fixed in shared memory while up to K accepted moves collect
// as a low-rank correction: W_eff = W - P Q^T, P: N x K, Q: ld x K (unused
// columns kept at zero).  Move m (pivot W_eff[K,l]) appends
//   P[:,m] = W_eff[:,l] / W_eff[K,l],   Q[:,m] = W_eff[K,:] - e_l,
// which is the Sherman-Morrison update of src/MonteCarlo.jl:279-292 in
// factored form.  Ratios and local energies read W_eff = W - P Q^T (a
// K-term dot per element); after K moves one register-tiled pass applies
// W -= P Q^T, touching each W element once per K moves instead of once per
// move.
// ---------------------------------------------------------------------------
template <int K>
struct DelayedSpin {
    float *W;   // [N][ld]
    float *P;   // [N][K]
    float *Q;   // [ld][K]
    int ld;
    __device__ __forceinline__ float dotPQ(int r, int c) const {
        const float4 *pr = reinterpret_cast<const float4 *>(P + (size_t)r * K);
        const float4 *qc = reinterpret_cast<const float4 *>(Q + (size_t)c * K);
        float acc0 = 0.f, acc1 = 0.f;  // two chains: the window waits on this latency
#pragma unroll
        for (int k = 0; k < K / 4; ++k) {
            const float4 a = pr[k], b = qc[k];
            acc0 = fmaf(a.x, b.x, acc0);
            acc1 = fmaf(a.y, b.y, acc1);
            acc0 = fmaf(a.z, b.z, acc0);
            acc1 = fmaf(a.w, b.w, acc1);
        }
        return acc0 + acc1;
    }
    __device__ __forceinline__ float eff(int r, int c) const { return W[(size_t)r * ld + c] - dotPQ(r, c); }
    // sum over the first m factor columns of P[r,k] Q[c,k]
    __device__ __forceinline__ float dot_lt(int r, int c, int m) const {
        const float4 *pr = reinterpret_cast<const float4 *>(P + (size_t)r * K);
        const float4 *qc = reinterpret_cast<const float4 *>(Q + (size_t)c * K);
        float acc0 = 0.f, acc1 = 0.f;
#pragma unroll
        for (int k = 0; k < K / 4; ++k) {
            const float4 a = pr[k], b = qc[k];
            acc0 = fmaf(4 * k + 0 < m ? a.x : 0.f, b.x, acc0);
            acc1 = fmaf(4 * k + 1 < m ? a.y : 0.f, b.y, acc1);
            acc0 = fmaf(4 * k + 2 < m ? a.z : 0.f, b.z, acc0);
            acc1 = fmaf(4 * k + 3 < m ? a.w : 0.f, b.w, acc1);
        }
        return acc0 + acc1;
    }
    // W_eff over the first m factor columns only (column m is being written)
    __device__ __forceinline__ float eff_lt(int r, int c, int m) const {
        const float4 *pr = reinterpret_cast<const float4 *>(P + (size_t)r * K);
        const float4 *qc = reinterpret_cast<const float4 *>(Q + (size_t)c * K);
        float acc0 = 0.f, acc1 = 0.f;
#pragma unroll
        for (int k = 0; k < K / 4; ++k) {
            const float4 a = pr[k], b = qc[k];
            acc0 = fmaf(4 * k + 0 < m ? a.x : 0.f, b.x, acc0);
            acc1 = fmaf(4 * k + 1 < m ? a.y : 0.f, b.y, acc1);
            acc0 = fmaf(4 * k + 2 < m ? a.z : 0.f, b.z, acc0);
            acc1 = fmaf(4 * k + 3 < m ? a.w : 0.f, b.w, acc1);
        }
        return W[(size_t)r * ld + c] - (acc0 + acc1);
    }
};

// W -= P Q^T over all threads; each thread keeps the Q slab of its four
// columns in registers and walks rows.  The rows of occupied sites should
// come out as exact unit rows (W[R][kappa[R]-1] = 1, zeros elsewhere); their
// largest deviation, the rounding accumulated since the last FP64 refresh,
// is folded into *dev (float bits, atomicMax).
// skip0 / skip1: rows whose configuration entry already describes a move W
// does not yet hold (their unit-row check is skipped); -1 for none.
// check = false skips the unit-row check: the deviation it reads stays in W,
// so a later flush's check still sees it.
template <int K>
__device__ void delayed_flush(const DelayedSpin<K> &S, int N, const short *kappa, int *dev, int skip0 = -1,
                              int skip1 = -1, bool check = true) {
    const int qc = S.ld >> 2;
    const int groups = blockDim.x / qc;
    const int t = threadIdx.x;
    if (t < groups * qc) {
        const int c4 = t % qc, rp = t / qc;
        float dmax = 0.f;
        float q[4][K];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 *qr = reinterpret_cast<const float4 *>(S.Q + (size_t)(4 * c4 + j) * K);
#pragma unroll
            for (int k = 0; k < K / 4; ++k) {
                const float4 v = qr[k];
                q[j][4 * k] = v.x; q[j][4 * k + 1] = v.y; q[j][4 * k + 2] = v.z; q[j][4 * k + 3] = v.w;
            }
        }
        // two rows per pass: eight independent FMA chains per thread
        for (int r = rp; r < N; r += 2 * groups) {
            const int r2 = r + groups;
            const bool two = r2 < N;
            const float4 *pr = reinterpret_cast<const float4 *>(S.P + (size_t)r * K);
            const float4 *pr2 = reinterpret_cast<const float4 *>(S.P + (size_t)(two ? r2 : r) * K);
            float p[K], p2[K];
#pragma unroll
            for (int k = 0; k < K / 4; ++k) {
                const float4 v = pr[k], v2 = pr2[k];
                p[4 * k] = v.x; p[4 * k + 1] = v.y; p[4 * k + 2] = v.z; p[4 * k + 3] = v.w;
                p2[4 * k] = v2.x; p2[4 * k + 1] = v2.y; p2[4 * k + 2] = v2.z; p2[4 * k + 3] = v2.w;
            }
            float4 *wp = reinterpret_cast<float4 *>(S.W + (size_t)r * S.ld) + c4;
            float4 *wp2 = reinterpret_cast<float4 *>(S.W + (size_t)(two ? r2 : r) * S.ld) + c4;
            float4 w = *wp, w2 = *wp2;
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                a0 = fmaf(p[k], q[0][k], a0);
                a1 = fmaf(p[k], q[1][k], a1);
                a2 = fmaf(p[k], q[2][k], a2);
                a3 = fmaf(p[k], q[3][k], a3);
                b0 = fmaf(p2[k], q[0][k], b0);
                b1 = fmaf(p2[k], q[1][k], b1);
                b2 = fmaf(p2[k], q[2][k], b2);
                b3 = fmaf(p2[k], q[3][k], b3);
            }
            w.x -= a0; w.y -= a1; w.z -= a2; w.w -= a3;
            *wp = w;
            const int c0 = 4 * c4;
            int l = (!check || r == skip0 || r == skip1) ? -1 : kappa[r] - 1;
            if (l >= 0) {
                const float d = fmaxf(fmaxf(fabsf(w.x - (c0 == l ? 1.f : 0.f)), fabsf(w.y - (c0 + 1 == l ? 1.f : 0.f))),
                                      fmaxf(fabsf(w.z - (c0 + 2 == l ? 1.f : 0.f)), fabsf(w.w - (c0 + 3 == l ? 1.f : 0.f))));
                dmax = fmaxf(dmax, d);
            }
            if (two) {
                w2.x -= b0; w2.y -= b1; w2.z -= b2; w2.w -= b3;
                *wp2 = w2;
                l = (!check || r2 == skip0 || r2 == skip1) ? -1 : kappa[r2] - 1;
                if (l >= 0) {
                    const float d = fmaxf(fmaxf(fabsf(w2.x - (c0 == l ? 1.f : 0.f)), fabsf(w2.y - (c0 + 1 == l ? 1.f : 0.f))),
                                          fmaxf(fabsf(w2.z - (c0 + 2 == l ? 1.f : 0.f)), fabsf(w2.w - (c0 + 3 == l ? 1.f : 0.f))));
                    dmax = fmaxf(dmax, d);
                }
            }
        }
        if (dmax > 0.f) atomicMax(dev, __float_as_int(dmax));
    }
}

// The same update with W in HBM: four rows' W words are loaded before any
// arithmetic so that each thread keeps four global loads in flight (the
// loop would otherwise wait one full memory latency per row), and P is read
// from shared memory per 4-wide k step instead of being held in registers.
template <int K>
__device__ void delayed_flush_stream(const DelayedSpin<K> &S, int N, const short *kappa, int *dev, int skip0 = -1,
                                     int skip1 = -1, bool check = true) {
    const int qc = S.ld >> 2;
    const int groups = blockDim.x / qc;
    const int t = threadIdx.x;
    if (t >= groups * qc) return;
    const int c4 = t % qc, rp = t / qc, c0 = 4 * c4;
    float q[4][K];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float4 *qr = reinterpret_cast<const float4 *>(S.Q + (size_t)(c0 + j) * K);
#pragma unroll
        for (int k = 0; k < K / 4; ++k) {
            const float4 v = qr[k];
            q[j][4 * k] = v.x; q[j][4 * k + 1] = v.y; q[j][4 * k + 2] = v.z; q[j][4 * k + 3] = v.w;
        }
    }
    float dmax = 0.f;
    for (int r0 = rp; r0 < N; r0 += 4 * groups) {
        float4 w[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = r0 + i * groups;
            if (r < N) w[i] = reinterpret_cast<const float4 *>(S.W + (size_t)r * S.ld)[c4];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = r0 + i * groups;
            if (r < N) {
                const float4 *pr = reinterpret_cast<const float4 *>(S.P + (size_t)r * K);
                float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
                for (int k4 = 0; k4 < K / 4; ++k4) {
                    const float4 v = pr[k4];
                    a0 = fmaf(v.x, q[0][4 * k4], a0); a1 = fmaf(v.x, q[1][4 * k4], a1);
                    a2 = fmaf(v.x, q[2][4 * k4], a2); a3 = fmaf(v.x, q[3][4 * k4], a3);
                    a0 = fmaf(v.y, q[0][4 * k4 + 1], a0); a1 = fmaf(v.y, q[1][4 * k4 + 1], a1);
                    a2 = fmaf(v.y, q[2][4 * k4 + 1], a2); a3 = fmaf(v.y, q[3][4 * k4 + 1], a3);
                    a0 = fmaf(v.z, q[0][4 * k4 + 2], a0); a1 = fmaf(v.z, q[1][4 * k4 + 2], a1);
                    a2 = fmaf(v.z, q[2][4 * k4 + 2], a2); a3 = fmaf(v.z, q[3][4 * k4 + 2], a3);
                    a0 = fmaf(v.w, q[0][4 * k4 + 3], a0); a1 = fmaf(v.w, q[1][4 * k4 + 3], a1);
                    a2 = fmaf(v.w, q[2][4 * k4 + 3], a2); a3 = fmaf(v.w, q[3][4 * k4 + 3], a3);
                }
                float4 x = w[i];
                x.x -= a0; x.y -= a1; x.z -= a2; x.w -= a3;
                reinterpret_cast<float4 *>(S.W + (size_t)r * S.ld)[c4] = x;
                const int l = (!check || r == skip0 || r == skip1) ? -1 : kappa[r] - 1;
                if (l >= 0) {
                    const float d = fmaxf(fmaxf(fabsf(x.x - (c0 == l ? 1.f : 0.f)), fabsf(x.y - (c0 + 1 == l ? 1.f : 0.f))),
                                          fmaxf(fabsf(x.z - (c0 + 2 == l ? 1.f : 0.f)), fabsf(x.w - (c0 + 3 == l ? 1.f : 0.f))));
                    dmax = fmaxf(dmax, d);
                }
            }
        }
    }
    if (dmax > 0.f) atomicMax(dev, __float_as_int(dmax));
}

// ---------------------------------------------------------------------------
// The rank-k flush W -= P Q^T on the tensor cores (tcgen05, kind::tf32),
// for W in HBM.  P (N x K) and Q (ld x K) are split into TF32 high and low
// parts (hi = x with the low 13 mantissa bits cleared, lo = x - hi, exact),
// and D = Ph Qh^T + Ph Ql^T + Pl Qh^T accumulates in TMEM in FP32: the
// product to FP32 accuracy (3xTF32).  Operand tiles sit in shared memory in
// the no-swizzle K-major layout, core matrices of 8 rows x 16 bytes:
// element (row, k) of a tile with kk columns at float index
// ((row/8) * (kk/4) + k/4) * 32 + (row%8) * 4 + k%4, so the leading-dimension
// offset (next 4 k) is 128 bytes and the stride offset (next 8 rows) is
// kk * 32 bytes.  One thread issues the MMAs of a 128-row tile of P against
// a chunk of up to 128 columns of Q and commits them to an mbarrier; every
// warp then reads its 32 TMEM lanes (rows) of D, half of the columns each,
// and updates its rows of W in place.
// ---------------------------------------------------------------------------
namespace tc {

constexpr int kTileM = 128;   // rows of P per MMA tile (TMEM lanes)
constexpr int kChunkN = 128;  // columns of Q per chunk (TMEM columns allocated)
constexpr int kMaxKK = 16;    // K padded to a multiple of 8
constexpr uint32_t kWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ int canon(int row, int k, int kk) {
    return ((row >> 3) * (kk >> 2) + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
}

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for this architecture; no swizzle, base offset 0
    return d;
}

// kind::tf32: FP32 accumulator, TF32 A and B, both K-major, M x N
__device__ __forceinline__ uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_u32(mbar)));
}

// bounded wait for the mbarrier phase with this parity; false when it gave up
__device__ __forceinline__ bool wait(uint64_t *mbar, uint32_t parity) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < kWaitLimit && !done; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(smem_u32(mbar)), "r"(parity));
    return done != 0;
}

__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }

__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    lo = x - hi;
}

// Per-CTA tensor-core state: TMEM columns, the commit barrier and its phase.
struct State {
    float *a_hi, *a_lo, *b_hi, *b_lo;  // operand tiles in shared memory
    uint64_t *mbar;
    uint32_t tmem;
    uint32_t phase;
};

// warp 0 allocates kChunkN TMEM columns; thread 0 initialises the barrier
__device__ void setup(State &st, uint32_t *tmem_slot) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(st.mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(tmem_slot)), "r"((uint32_t)kChunkN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    st.tmem = *tmem_slot;
    st.phase = 0;
}

__device__ void teardown(const State &st) {
    fence_before();
    __syncthreads();
    fence_after();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(st.tmem), "r"((uint32_t)kChunkN));
}

}  // namespace tc

template <int K>
__device__ void delayed_flush_tc(const DelayedSpin<K> &S, int N, const short *kappa, int *dev, tc::State &st,
                                 int *status, int skip0 = -1, int skip1 = -1) {
    constexpr int KK = (K + 7) / 8 * 8;
    static_assert(KK <= tc::kMaxKK, "delay depth beyond the operand tiles");
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    const int quarter = warp & 3, half = warp >> 2, halves = nwarps >> 2;  // lanes 32*quarter.. of TMEM
    const uint32_t lbo = 128, sbo = KK * 32;
    float dmax = 0.f;
    for (int c0 = 0; c0 < S.ld; c0 += tc::kChunkN) {
        const int nvalid = min(tc::kChunkN, S.ld - c0);
        const int nc = (nvalid + 15) / 16 * 16;
        for (int e = tid; e < nc * KK; e += nt) {
            const int row = e / KK, k = e - row * KK;
            const float x = (row < nvalid && k < K) ? S.Q[(size_t)(c0 + row) * K + k] : 0.f;
            float hi, lo;
            tc::split_tf32(x, hi, lo);
            st.b_hi[tc::canon(row, k, KK)] = hi;
            st.b_lo[tc::canon(row, k, KK)] = lo;
        }
        const uint32_t idesc = tc::idesc_tf32(tc::kTileM, nc);
        for (int r0 = 0; r0 < N; r0 += tc::kTileM) {
            for (int e = tid; e < tc::kTileM * KK; e += nt) {
                const int row = e / KK, k = e - row * KK;
                const float x = (r0 + row < N && k < K) ? S.P[(size_t)(r0 + row) * K + k] : 0.f;
                float hi, lo;
                tc::split_tf32(x, hi, lo);
                st.a_hi[tc::canon(row, k, KK)] = hi;
                st.a_lo[tc::canon(row, k, KK)] = lo;
            }
            asm volatile("fence.proxy.async.shared::cta;");
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (tid == 0) {
                const float *As[3] = {st.a_hi, st.a_hi, st.a_lo};
                const float *Bs[3] = {st.b_hi, st.b_lo, st.b_hi};
                uint32_t acc = 0;
#pragma unroll
                for (int s = 0; s < KK / 8; ++s) {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const uint64_t ad = tc::sdesc(tc::smem_u32(As[q]) + s * 2 * lbo, lbo, sbo);
                        const uint64_t bd = tc::sdesc(tc::smem_u32(Bs[q]) + s * 2 * lbo, lbo, sbo);
                        tc::mma(st.tmem, ad, bd, idesc, acc);
                        acc = 1;
                    }
                }
                tc::commit(st.mbar);
            }
            const bool ok = tc::wait(st.mbar, st.phase);
            st.phase ^= 1u;
            if (!ok && lane == 0) atomicOr(status, kStatusTimeout);
            tc::fence_after();
            // epilogue: row r0 + 32*quarter + lane, this warp's share of the chunk's columns
            const int r = r0 + 32 * quarter + lane;
            const int l = (r < N && r != skip0 && r != skip1) ? kappa[r] - 1 : -1;
            float *wr = S.W + (size_t)(r < N ? r : 0) * S.ld + c0;
            for (int cc = 8 * half; cc < nc; cc += 8 * halves) {
                float d[8];
                tc::ld8(st.tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)cc, d);
                if (r < N && ok) {
                    if (cc + 8 <= nvalid) {
                        float4 *p4 = reinterpret_cast<float4 *>(wr + cc);
                        float4 x0 = p4[0], x1 = p4[1];
                        x0.x -= d[0]; x0.y -= d[1]; x0.z -= d[2]; x0.w -= d[3];
                        x1.x -= d[4]; x1.y -= d[5]; x1.z -= d[6]; x1.w -= d[7];
                        p4[0] = x0;
                        p4[1] = x1;
                        if (l >= 0) {
                            const float v[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
                            for (int j = 0; j < 8; ++j)
                                dmax = fmaxf(dmax, fabsf(v[j] - (c0 + cc + j == l ? 1.f : 0.f)));
                        }
                    } else {
                        for (int j = 0; j < 8 && cc + j < nvalid; ++j) {
                            const float v = wr[cc + j] - d[j];
                            wr[cc + j] = v;
                            if (l >= 0) dmax = fmaxf(dmax, fabsf(v - (c0 + cc + j == l ? 1.f : 0.f)));
                        }
                    }
                }
            }
            tc::fence_before();
            __syncthreads();  // the next tile rewrites the operand tiles and TMEM
            tc::fence_after();
        }
    }
    if (dmax > 0.f) atomicMax(dev, __float_as_int(dmax));
}

size_t tc_flush_smem_bytes() { return (size_t)2 * (tc::kTileM + tc::kChunkN) * tc::kMaxKK * 4 + 128; }

template <int K>
__device__ void delayed_zero(const DelayedSpin<K> &S, int N) {
    float4 *p = reinterpret_cast<float4 *>(S.P);
    for (int e = threadIdx.x; e < N * K / 4; e += blockDim.x) p[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 *q = reinterpret_cast<float4 *>(S.Q);
    for (int e = threadIdx.x; e < S.ld * K / 4; e += blockDim.x) q[e] = make_float4(0.f, 0.f, 0.f, 0.f);
}

struct DelayedCtl {
    long long t, next_meas;
    long long cache_t;  // the draws below belong to proposals cache_t .. cache_t+31
    unsigned long long cache_u53[32];
    short2 cache_bond[32];  // the proposal's bond endpoints
    int since, zmu, state, m;
    int dev;  // float bits: unit-row deviation seen at the last flush
    int Ku, lu, Kd, ld;
    float piv_u, piv_d;
    Thr thr;
    double red[33];
};

// Local energy with W_eff (src/Hamiltonian.jl:593-778), FP64 sums.
template <int K>
__device__ double delayed_local_energy(const DevModel &m, const short2 *bonds, const short *kup, const short *kdn,
                                       const DelayedSpin<K> &U, const DelayedSpin<K> &D, double *red) {
    float acc = 0.f;
    for (int e = threadIdx.x; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = bonds[e];
        const int i = bd.x, j = bd.y;
        const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
        acc += ((ui != 0) == (uj != 0)) ? 0.25f : -0.25f;
        if (uj != 0 && di != 0) acc -= 0.5f * U.eff(i, uj - 1) * D.eff(j, di - 1);
        if (ui != 0 && dj != 0) acc -= 0.5f * U.eff(j, ui - 1) * D.eff(i, dj - 1);
    }
    return block_sum_f32(acc, red);
}

// kStream = false: W (FP32) is staged in shared memory for the launch.
// kStream = true: W stays in HBM and only P, Q and the walker's small state
// are on chip, so several walkers share an SM and hide each other's global
// latency; the flush then streams W through once per K moves.
// kThreads: 512 with W on chip (one walker per SM); 256 or 128 with W in
// HBM (two or four walkers per SM).
template <int K, bool kStream, int kThreads>
__global__ void __launch_bounds__(kThreads, 512 / kThreads)
sweep_delayed_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count) {
    const int w = blockIdx.x;
    const int N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long t0 = b.t[w];
    const long long tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);  // this launch's share
    const long long acc_left = b.acc_end[w] - b.accepted[w];  // accepted moves still wanted
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        // nothing to do; a refresh marked due has run since (stream order), clear the mark
        if (threadIdx.x == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }

    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ DelayedCtl ctl;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    float *gW = b.W32 + (size_t)w * wblock;
    unsigned char *cur = smem;
    DelayedSpin<K> SU, SD;
    if constexpr (kStream) {
        SU.W = gW;
    } else {
        SU.W = reinterpret_cast<float *>(cur);
        cur += wblock * sizeof(float);
    }
    SU.ld = m.ld_up;
    SD.W = SU.W + (size_t)N * m.ld_up;
    SD.ld = m.ld_dn;
    SU.P = reinterpret_cast<float *>(cur); cur += (size_t)N * K * sizeof(float);
    SD.P = reinterpret_cast<float *>(cur); cur += (size_t)N * K * sizeof(float);
    SU.Q = reinterpret_cast<float *>(cur); cur += (size_t)m.ld_up * K * sizeof(float);
    SD.Q = reinterpret_cast<float *>(cur); cur += (size_t)m.ld_dn * K * sizeof(float);
    int *nbr_off = reinterpret_cast<int *>(cur); cur += (size_t)(N + 1) * sizeof(int);
    short2 *bonds = reinterpret_cast<short2 *>(cur); cur += (size_t)m.n_bonds * sizeof(short2);
    short *nbr = reinterpret_cast<short *>(cur); cur += (size_t)2 * m.n_bonds * sizeof(short);
    short *kup = reinterpret_cast<short *>(cur); cur += (size_t)N * sizeof(short);
    short *kdn = reinterpret_cast<short *>(cur);

    if constexpr (!kStream) {
        const int nvec = (int)(wblock / 4);
        const float4 *src = reinterpret_cast<const float4 *>(gW);
        float4 *dst = reinterpret_cast<float4 *>(SU.W);
        for (int e = tid; e < nvec; e += blockDim.x) dst[e] = src[e];
    }
    delayed_zero<K>(SU, N);
    delayed_zero<K>(SD, N);
    for (int e = tid; e < m.n_bonds; e += blockDim.x) bonds[e] = m.bonds[e];
    for (int e = tid; e < 2 * m.n_bonds; e += blockDim.x) nbr[e] = m.nbr[e];
    for (int e = tid; e <= N; e += blockDim.x) nbr_off[e] = m.nbr_off[e];
    for (int s = tid; s < N; s += blockDim.x) {
        kup[s] = b.kappa_up[(size_t)w * N + s];
        kdn[s] = b.kappa_dn[(size_t)w * N + s];
    }
    __syncthreads();
    double zc = 0.0;
    for (int e = tid; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = bonds[e];
        zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
    }
    zc = block_sum(zc, ctl.red);
    const int R = p.refresh_every;
    const int M = p.measure_every;
    if (tid == 0) {
        ctl.t = t0;
        ctl.since = b.since[w] < 0 ? 0 : b.since[w];
        ctl.zmu = (int)zc;
        ctl.m = 0;
        ctl.dev = 0;
        ctl.cache_t = -1;
        ctl.next_meas = (t0 / M + 1) * M;
        make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
    }
    __syncthreads();

    long long acc_count = 0, n_meas = 0;
    double se = 0.0, se2 = 0.0;

    while (true) {
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
                float pu = 0.f, pd = 0.f;
                if (lane < win) {
                    unsigned long long u53;
                    short2 bd;
                    if (t == ctl.cache_t) {  // drawn ahead during the previous update
                        u53 = ctl.cache_u53[lane];
                        bd = ctl.cache_bond[lane];
                    } else {
                        int bi;
                        proposal_bits(p.seed, w, t + lane, m.n_bonds, u53, bi);
                        bd = bonds[bi];
                    }
                    const int c = cmp_r_thr(u53, thr);
                    if (p.accept_rule != 0 || c <= 0) {
                        const int i = bd.x, j = bd.y;
                        const int kui = kup[i], kuj = kup[j], kdi = kdn[i], kdj = kdn[j];
                        const bool f1 = kui != 0 && kdj != 0;
                        const bool f2 = kuj != 0 && kdi != 0;
                        if (f1 || f2) {
                            if (f1) { Ku = j; lu = kui - 1; Kd = i; ld = kdj - 1; }
                            else    { Ku = i; lu = kuj - 1; Kd = j; ld = kdi - 1; }
                            pu = SU.eff(Ku, lu);
                            pd = SD.eff(Kd, ld);
                            acc = decide(pu, pd, u53, c, thr, p.accept_rule, bad);
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
            const float ipu = 1.f / ctl.piv_u, ipd = 1.f / ctl.piv_d;
            const int mm = ctl.m;
            // new factor column mm, written in place: its entries read only the
            // columns before mm, so writers and readers never touch the same word
            const int tot = 2 * N + m.ld_up + m.ld_dn;
            if constexpr (kStream) {
                // W in HBM: each thread loads the W words of up to four of its
                // entries before any shared-memory store, so their latencies overlap
                for (int base = 0; base < tot; base += 4 * blockDim.x) {
                    float wv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = base + q * blockDim.x + tid;
                        wv[q] = 0.f;
                        if (e < N) wv[q] = SU.W[(size_t)e * SU.ld + lu];
                        else if (e < 2 * N) wv[q] = SD.W[(size_t)(e - N) * SD.ld + ld];
                        else if (e < 2 * N + m.ld_up) wv[q] = SU.W[(size_t)Ku * SU.ld + (e - 2 * N)];
                        else if (e < tot) wv[q] = SD.W[(size_t)Kd * SD.ld + (e - 2 * N - m.ld_up)];
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = base + q * blockDim.x + tid;
                        if (e < N) SU.P[(size_t)e * K + mm] = (wv[q] - SU.dot_lt(e, lu, mm)) * ipu;
                        else if (e < 2 * N) SD.P[(size_t)(e - N) * K + mm] = (wv[q] - SD.dot_lt(e - N, ld, mm)) * ipd;
                        else if (e < 2 * N + m.ld_up) {
                            const int c = e - 2 * N;
                            SU.Q[(size_t)c * K + mm] = wv[q] - SU.dot_lt(Ku, c, mm) - (c == lu ? 1.f : 0.f);
                        } else if (e < tot) {
                            const int c = e - 2 * N - m.ld_up;
                            SD.Q[(size_t)c * K + mm] = wv[q] - SD.dot_lt(Kd, c, mm) - (c == ld ? 1.f : 0.f);
                        }
                    }
                }
            } else {
                for (int e = tid; e < tot; e += blockDim.x) {
                    if (e < N) SU.P[(size_t)e * K + mm] = SU.eff_lt(e, lu, mm) * ipu;
                    else if (e < 2 * N) SD.P[(size_t)(e - N) * K + mm] = SD.eff_lt(e - N, ld, mm) * ipd;
                    else if (e < 2 * N + m.ld_up) {
                        const int c = e - 2 * N;
                        SU.Q[(size_t)c * K + mm] = SU.eff_lt(Ku, c, mm) - (c == lu ? 1.f : 0.f);
                    } else {
                        const int c = e - 2 * N - m.ld_up;
                        SD.Q[(size_t)c * K + mm] = SD.eff_lt(Kd, c, mm) - (c == ld ? 1.f : 0.f);
                    }
                }
            }
            if (warp == (blockDim.x >> 5) - 2) {
                // draws for the next window, which starts at ctl.t
                const long long tn = ctl.t;
                unsigned long long u53;
                int bi;
                proposal_bits(p.seed, w, tn + lane, m.n_bonds, u53, bi);
                ctl.cache_u53[lane] = u53;
                ctl.cache_bond[lane] = bonds[bi];
                __syncwarp();
                if (lane == 0) ctl.cache_t = tn;
            }
            if (warp == (blockDim.x >> 5) - 1) {
                // Z_mu change: the up spin moves Kd -> Ku, the down spin Ku -> Kd
                int dz = 0;
                for (int e = nbr_off[Ku] + lane; e < nbr_off[Ku + 1]; e += 32) {
                    const int k = nbr[e];
                    if (k != Kd) dz += kup[k] == 0 ? 1 : -1;
                }
                for (int e = nbr_off[Kd] + lane; e < nbr_off[Kd + 1]; e += 32) {
                    const int k = nbr[e];
                    if (k != Ku) dz += kup[k] != 0 ? 1 : -1;
                }
                dz = __reduce_add_sync(0xffffffffu, dz);
                __syncwarp();
                if (lane == 0) {   // nobody else reads kappa in this phase
                    ctl.zmu += dz;
                    ctl.since += 1;
                    make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
                    kup[Ku] = (short)(lu + 1); kup[Kd] = 0;
                    kdn[Kd] = (short)(ld + 1); kdn[Ku] = 0;
                }
            }
            acc_count += 1;
            __syncthreads();
            // every thread has read ctl.m for this move before the barrier above
            if (mm + 1 == K) {
                if constexpr (kStream) {
                    delayed_flush_stream<K>(SU, N, kup, &ctl.dev);
                    delayed_flush_stream<K>(SD, N, kdn, &ctl.dev);
                } else {
                    delayed_flush<K>(SU, N, kup, &ctl.dev);
                    delayed_flush<K>(SD, N, kdn, &ctl.dev);
                }
                __syncthreads();
                delayed_zero<K>(SU, N);
                delayed_zero<K>(SD, N);
                if (tid == 0) {
                    ctl.m = 0;
                    // adaptive refresh: rounding past the tolerance ends this walker's
                    // run here, so the FP64 refresh rebuilds W now
                    if (__int_as_float(ctl.dev) > p.drift_tol) ctl.since = R;
                    ctl.dev = 0;
                }
                __syncthreads();
            } else if (tid == 0) {
                ctl.m = mm + 1;  // read again only after the bottom barrier
            }
        }
        const long long t = ctl.t;
        if (t == ctl.next_meas) {
            const double e = delayed_local_energy<K>(m, bonds, kup, kdn, SU, SD, ctl.red);
            if (tid == 0) {  // only thread 0 keeps the FP64 sums
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
        if constexpr (kStream) {
            delayed_flush_stream<K>(SU, N, kup, &ctl.dev);
            delayed_flush_stream<K>(SD, N, kdn, &ctl.dev);
        } else {
            delayed_flush<K>(SU, N, kup, &ctl.dev);
            delayed_flush<K>(SD, N, kdn, &ctl.dev);
        }
        __syncthreads();
    }
    if constexpr (!kStream) {
        const int nvec = (int)(wblock / 4);
        const float4 *src = reinterpret_cast<const float4 *>(SU.W);
        float4 *dst = reinterpret_cast<float4 *>(gW);
        for (int e = tid; e < nvec; e += blockDim.x) dst[e] = src[e];
    }
    for (int s = tid; s < N; s += blockDim.x) {
        b.kappa_up[(size_t)w * N + s] = kup[s];
        b.kappa_dn[(size_t)w * N + s] = kdn[s];
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
// Pipelined delayed-update sweep: the same chain as sweep_delayed_kernel, but
// the scan for the next accepted move (warp 0) runs while the other warps
// write the factor column of the move accepted last.  The scan sees that
// pending move (K, l, pivot) through its Sherman-Morrison correction on top
// of the m complete factor columns,
//   W_eff'(r, c) = W_eff(r, c) - W_eff(r, l) (W_eff(K, c) - [c == l]) / pivot,
// every W_eff term over columns [0, m) only, which the writers do not touch.
// The configuration, Z_mu and threshold of an accepted move are applied after
// the flush that may follow, so the flush's unit-row check sees the sites W
// describes.
// ---------------------------------------------------------------------------
struct PendingMove {
    int Ku, lu, Kd, ld;
    float piv_u, piv_d;
};

struct PipeCtl {
    long long t, next_meas, acc;
    int since, zmu;
    int state2[2];
    int dev, dev2[2];
    PendingMove mv[2];
    Thr thr;
    double red[33];
};

template <int K>
__device__ __forceinline__ float eff_after(const DelayedSpin<K> &S, int r, int c, int mm, bool pend, int Kp, int lp,
                                           float ipiv) {
    float v = S.eff_lt(r, c, mm);
    if (pend) {
        const float a = S.eff_lt(r, lp, mm);
        const float q = S.eff_lt(Kp, c, mm) - (c == lp ? 1.f : 0.f);
        v = fmaf(-a * ipiv, q, v);
    }
    return v;
}

template <int K, bool kStream, int kThreads, bool kTC>
__device__ __forceinline__ void sweep_pipe_body(const DevModel &m, const DevBatch &b, const SweepParams &p,
                                                int *active_count, int thr_in_smem) {
    const int w = blockIdx.x;
    const int N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long t0 = b.t[w];
    const long long tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);  // this launch's share
    const long long acc_left = b.acc_end[w] - b.accepted[w];
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        if (threadIdx.x == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ PipeCtl ctl;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    float *gW = b.W32 + (size_t)w * wblock;
    unsigned char *cur = smem;
    DelayedSpin<K> SU, SD;
    if constexpr (kStream) {
        SU.W = gW;
    } else {
        SU.W = reinterpret_cast<float *>(cur);
        cur += wblock * sizeof(float);
    }
    SU.ld = m.ld_up;
    SD.W = SU.W + (size_t)N * m.ld_up;
    SD.ld = m.ld_dn;
    SU.P = reinterpret_cast<float *>(cur); cur += (size_t)N * K * sizeof(float);
    SD.P = reinterpret_cast<float *>(cur); cur += (size_t)N * K * sizeof(float);
    SU.Q = reinterpret_cast<float *>(cur); cur += (size_t)m.ld_up * K * sizeof(float);
    SD.Q = reinterpret_cast<float *>(cur); cur += (size_t)m.ld_dn * K * sizeof(float);
    int *nbr_off = reinterpret_cast<int *>(cur); cur += (size_t)(N + 1) * sizeof(int);
    short2 *bonds = reinterpret_cast<short2 *>(cur); cur += (size_t)m.n_bonds * sizeof(short2);
    short *nbr = reinterpret_cast<short *>(cur); cur += (size_t)2 * m.n_bonds * sizeof(short);
    short *kup = reinterpret_cast<short *>(cur); cur += (size_t)N * sizeof(short);
    short *kdn = reinterpret_cast<short *>(cur);
    // nu[s] = the number of neighbours of s that hold the up spin
    int *nu = reinterpret_cast<int *>((reinterpret_cast<uintptr_t>(kdn + N) + 3) & ~uintptr_t(3));
    // the acceptance thresholds, on chip when the launch found room for them
    ThrEntry *thr_s = reinterpret_cast<ThrEntry *>((reinterpret_cast<uintptr_t>(nu + N) + 15) & ~uintptr_t(15));
    const ThrEntry *thr_tab = thr_in_smem ? thr_s : m.thr_table;
    [[maybe_unused]] __shared__ __align__(8) uint64_t tc_mbar;
    [[maybe_unused]] __shared__ uint32_t tc_tmem_slot;
    [[maybe_unused]] tc::State tcs{};
    if constexpr (kTC) {
        cur = thr_in_smem ? reinterpret_cast<unsigned char *>(thr_s + m.n_bonds + 1)
                          : reinterpret_cast<unsigned char *>(nu + N);
        cur = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(cur) + 127) & ~uintptr_t(127));
        tcs.a_hi = reinterpret_cast<float *>(cur); cur += tc::kTileM * tc::kMaxKK * sizeof(float);
        tcs.a_lo = reinterpret_cast<float *>(cur); cur += tc::kTileM * tc::kMaxKK * sizeof(float);
        tcs.b_hi = reinterpret_cast<float *>(cur); cur += tc::kChunkN * tc::kMaxKK * sizeof(float);
        tcs.b_lo = reinterpret_cast<float *>(cur);
        tcs.mbar = &tc_mbar;
        tc::setup(tcs, &tc_tmem_slot);
    }

    if constexpr (!kStream) {
        const int nvec = (int)(wblock / 4);
        const float4 *src = reinterpret_cast<const float4 *>(gW);
        float4 *dst = reinterpret_cast<float4 *>(SU.W);
        for (int e = tid; e < nvec; e += blockDim.x) dst[e] = src[e];
    }
    delayed_zero<K>(SU, N);
    delayed_zero<K>(SD, N);
    for (int e = tid; e < m.n_bonds; e += blockDim.x) bonds[e] = m.bonds[e];
    for (int e = tid; e < 2 * m.n_bonds; e += blockDim.x) nbr[e] = m.nbr[e];
    for (int e = tid; e <= N; e += blockDim.x) nbr_off[e] = m.nbr_off[e];
    if (thr_in_smem)
        for (int e = tid; e <= m.n_bonds; e += blockDim.x) thr_s[e] = m.thr_table[e];
    for (int s = tid; s < N; s += blockDim.x) {
        kup[s] = b.kappa_up[(size_t)w * N + s];
        kdn[s] = b.kappa_dn[(size_t)w * N + s];
    }
    __syncthreads();
    double zc = 0.0;
    for (int e = tid; e < m.n_bonds; e += blockDim.x) {
        const short2 bd = bonds[e];
        zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
    }
    for (int s0 = tid; s0 < N; s0 += blockDim.x) {
        int c = 0;
        for (int e = nbr_off[s0]; e < nbr_off[s0 + 1]; ++e) c += kup[nbr[e]] != 0 ? 1 : 0;
        nu[s0] = c;
    }
    zc = block_sum(zc, ctl.red);
    const int R = p.refresh_every;
    const int M = p.measure_every;
    if (tid == 0) {
        ctl.t = t0;
        ctl.acc = 0;
        ctl.since = b.since[w] < 0 ? 0 : b.since[w];
        ctl.zmu = (int)zc;
        ctl.dev = 0;
        ctl.dev2[0] = ctl.dev2[1] = 0;
        ctl.next_meas = (t0 / M + 1) * M;
        make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
    }
    __syncthreads();

    long long n_meas = 0;
    double se = 0.0, se2 = 0.0;
    // the loop state below is kept by every thread alike (no broadcast needed):
    // pend = a move accepted in the previous phase whose factor column this
    // phase writes, slot = its entry in ctl.mv, mm = complete factor columns,
    // fp = flushes so far (their parity picks the drift slot)
    int pend = 0, slot = 0, mm = 0, fp = 0, it = 0;
    while (true) {
        if (warp == 0) {
            // scan for the next accepted move
            const PendingMove pm = ctl.mv[slot];
            const float ipu = pend ? 1.f / pm.piv_u : 0.f, ipd = pend ? 1.f / pm.piv_d : 0.f;
            long long t = ctl.t;
            const long long acc = ctl.acc, next_meas = ctl.next_meas;
            const int since = ctl.since;
            const Thr thr = ctl.thr;
            int state = 2;
            PendingMove nm{};
            while (true) {
                if (t == next_meas) { state = 3; break; }
                if (t >= tend || since >= R || acc >= acc_left) break;
                const long long lim = min(tend, next_meas) - t;
                const int win = lim < 32 ? (int)lim : 32;
                bool accd = false, bad = false;
                int Ku = 0, lu = 0, Kd = 0, ld = 0;
                float pu = 0.f, pd = 0.f;
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
                            pu = eff_after<K>(SU, Ku, lu, mm, pend, pm.Ku, pm.lu, ipu);
                            pd = eff_after<K>(SD, Kd, ld, mm, pend, pm.Kd, pm.ld, ipd);
                            accd = decide(pu, pd, u53, c, thr, p.accept_rule, bad);
                        }
                    }
                }
                if (__any_sync(0xffffffffu, bad) && bad) atomicOr(&b.status[w], kStatusNonFinite);
                const unsigned mask = __ballot_sync(0xffffffffu, accd);
                if (mask) {
                    const int f = __ffs(mask) - 1;
                    nm = PendingMove{__shfl_sync(0xffffffffu, Ku, f), __shfl_sync(0xffffffffu, lu, f),
                                     __shfl_sync(0xffffffffu, Kd, f), __shfl_sync(0xffffffffu, ld, f),
                                     __shfl_sync(0xffffffffu, pu, f), __shfl_sync(0xffffffffu, pd, f)};
                    t += f + 1;
                    state = 1;
                    break;
                }
                t += win;
            }
            if (state == 1) {
                // apply the move: Z_mu change (configuration before it), then the
                // configuration, the threshold and the counters.  Nobody else reads
                // the configuration in this phase; the flush that may follow skips
                // the unit-row check of the two rows the move changes.
                // the up spin moves Kd -> Ku along their bond (every site holds one
                // spin, bonds are unique): the bonds from Ku to its other up
                // neighbours turn parallel and the rest antiparallel, and the other
                // way round at Kd, so Z_mu changes by
                //   (deg Ku - 1 - 2 (nu[Ku] - 1)) + (2 nu[Kd] - (deg Kd - 1))
                const int bu = nbr_off[nm.Ku], du = nbr_off[nm.Ku + 1] - bu;
                const int bd = nbr_off[nm.Kd], dd = nbr_off[nm.Kd + 1] - bd;
                const int dz = du - dd + 2 - 2 * nu[nm.Ku] + 2 * nu[nm.Kd];
                __syncwarp();  // every lane has read nu before it changes
                for (int e = lane; e < du + dd; e += 32)
                    atomicAdd(&nu[e < du ? nbr[bu + e] : nbr[bd + e - du]], e < du ? 1 : -1);
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
            // the state word alternates between two slots: a slot is rewritten only
            // after every thread has passed the barrier that follows its last read
            if (lane == 0) { ctl.t = t; ctl.state2[it & 1] = state; }
        } else if (pend) {
            // factor column mm of the pending move, over columns [0, mm)
            const PendingMove pm = ctl.mv[slot];
            const float ipu = 1.f / pm.piv_u, ipd = 1.f / pm.piv_d;
            const int tot = 2 * N + m.ld_up + m.ld_dn;
            const int nt = blockDim.x - 32, id = tid - 32;
            if constexpr (kStream) {
                for (int base = 0; base < tot; base += 4 * nt) {
                    float wv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = base + q * nt + id;
                        wv[q] = 0.f;
                        if (e < N) wv[q] = SU.W[(size_t)e * SU.ld + pm.lu];
                        else if (e < 2 * N) wv[q] = SD.W[(size_t)(e - N) * SD.ld + pm.ld];
                        else if (e < 2 * N + m.ld_up) wv[q] = SU.W[(size_t)pm.Ku * SU.ld + (e - 2 * N)];
                        else if (e < tot) wv[q] = SD.W[(size_t)pm.Kd * SD.ld + (e - 2 * N - m.ld_up)];
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = base + q * nt + id;
                        if (e < N) SU.P[(size_t)e * K + mm] = (wv[q] - SU.dot_lt(e, pm.lu, mm)) * ipu;
                        else if (e < 2 * N) SD.P[(size_t)(e - N) * K + mm] = (wv[q] - SD.dot_lt(e - N, pm.ld, mm)) * ipd;
                        else if (e < 2 * N + m.ld_up) {
                            const int c = e - 2 * N;
                            SU.Q[(size_t)c * K + mm] = wv[q] - SU.dot_lt(pm.Ku, c, mm) - (c == pm.lu ? 1.f : 0.f);
                        } else if (e < tot) {
                            const int c = e - 2 * N - m.ld_up;
                            SD.Q[(size_t)c * K + mm] = wv[q] - SD.dot_lt(pm.Kd, c, mm) - (c == pm.ld ? 1.f : 0.f);
                        }
                    }
                }
            } else {
                for (int e = id; e < tot; e += nt) {
                    if (e < N) SU.P[(size_t)e * K + mm] = SU.eff_lt(e, pm.lu, mm) * ipu;
                    else if (e < 2 * N) SD.P[(size_t)(e - N) * K + mm] = SD.eff_lt(e - N, pm.ld, mm) * ipd;
                    else if (e < 2 * N + m.ld_up) {
                        const int c = e - 2 * N;
                        SU.Q[(size_t)c * K + mm] = SU.eff_lt(pm.Ku, c, mm) - (c == pm.lu ? 1.f : 0.f);
                    } else {
                        const int c = e - 2 * N - m.ld_up;
                        SD.Q[(size_t)c * K + mm] = SD.eff_lt(pm.Kd, c, mm) - (c == pm.ld ? 1.f : 0.f);
                    }
                }
            }
        }
        __syncthreads();
        const int state = ctl.state2[it & 1];
        ++it;
        const int mnew = pend ? mm + 1 : mm;
        if (mnew == K) {
            // rows of the move just accepted (not yet in W) skip the unit-row check
            int s0 = -1, s1 = -1;
            if (state == 1) { const PendingMove nm = ctl.mv[slot ^ 1]; s0 = nm.Ku; s1 = nm.Kd; }
            int *dev = &ctl.dev2[fp & 1];
            // the unit-row check on every fourth flush (a quarter of the flush's
            // work): the deviation accumulates in W, so it is seen at most three
            // flushes late; the flush at the end of a launch always checks
            const bool check = (fp & 3) == 0;
            if constexpr (kTC) {
                delayed_flush_tc<K>(SU, N, kup, dev, tcs, &b.status[w], s0, s1);
                delayed_flush_tc<K>(SD, N, kdn, dev, tcs, &b.status[w], s0, s1);
            } else if constexpr (kStream) {
                delayed_flush_stream<K>(SU, N, kup, dev, s0, s1, check);
                delayed_flush_stream<K>(SD, N, kdn, dev, s0, s1, check);
            } else {
                delayed_flush<K>(SU, N, kup, dev, s0, s1, check);
                delayed_flush<K>(SD, N, kdn, dev, s0, s1, check);
            }
            __syncthreads();
            delayed_zero<K>(SU, N);
            delayed_zero<K>(SD, N);
            if (tid == 0) {
                // adaptive refresh on rounding past the tolerance: when the moves
                // this call still asks of the walker are fewer than an interval, at
                // the end of the call (its counter then reaches R exactly with its
                // last move, so refreshes stay on call boundaries and no walker stops
                // mid-call), else now; a deviation past drift_severe (by default
                // max(100 tolerances, 1e-2): W losing its accuracy, as near a
                // singular configuration) refreshes now in any case.  The other drift slot is free again
                // (everybody read it a flush ago).
                const float dv = __int_as_float(*dev);
                if (dv > p.drift_tol) {
                    const long long rem = acc_left - ctl.acc;
                    const bool mild = dv <= p.drift_severe;
                    ctl.since = (rem < R && mild) ? max(ctl.since, (int)(R - rem)) : R;
                }
                ctl.dev2[(fp & 1) ^ 1] = 0;
            }
            __syncthreads();
            ++fp;
        }
        mm = mnew == K ? 0 : mnew;
        if (state == 1) slot ^= 1;
        pend = state == 1;
        if (state == 3) {
            const double e = delayed_local_energy<K>(m, bonds, kup, kdn, SU, SD, ctl.red);
            if (tid == 0) {
                se += e;
                se2 += e * e;
                n_meas += 1;
                ctl.next_meas += M;
            }
        }
        if (state == 2) break;
    }
    if (mm > 0) {
        if constexpr (kTC) {
            delayed_flush_tc<K>(SU, N, kup, &ctl.dev, tcs, &b.status[w]);
            delayed_flush_tc<K>(SD, N, kdn, &ctl.dev, tcs, &b.status[w]);
        } else if constexpr (kStream) {
            delayed_flush_stream<K>(SU, N, kup, &ctl.dev);
            delayed_flush_stream<K>(SD, N, kdn, &ctl.dev);
        } else {
            delayed_flush<K>(SU, N, kup, &ctl.dev);
            delayed_flush<K>(SD, N, kdn, &ctl.dev);
        }
        __syncthreads();
    }
    if constexpr (kTC) tc::teardown(tcs);
    if constexpr (!kStream) {
        const int nvec = (int)(wblock / 4);
        const float4 *src = reinterpret_cast<const float4 *>(SU.W);
        float4 *dst = reinterpret_cast<float4 *>(gW);
        for (int e = tid; e < nvec; e += blockDim.x) dst[e] = src[e];
    }
    for (int s = tid; s < N; s += blockDim.x) {
        b.kappa_up[(size_t)w * N + s] = kup[s];
        b.kappa_dn[(size_t)w * N + s] = kdn[s];
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

// Two register budgets for the same body: two (or four) CTAs of 256 (128)
// threads per SM, 128 registers a thread; and, where shared memory already
// limits the launch to one CTA per SM (W in HBM at N = 864, k = 16: 187 KB),
// without the cap, so nothing spills (72 bytes spilled at k = 16 under it).
template <int K, bool kStream, int kThreads, bool kTC>
__global__ void __launch_bounds__(kThreads, 512 / kThreads)
sweep_pipe_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count, int thr_in_smem) {
    sweep_pipe_body<K, kStream, kThreads, kTC>(m, b, p, active_count, thr_in_smem);
}

template <int K>
__global__ void __launch_bounds__(256, 1)
sweep_pipe_wide_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count, int thr_in_smem) {
    sweep_pipe_body<K, true, 256, false>(m, b, p, active_count, thr_in_smem);
}

size_t delayed_smem_bytes(const DevModel &m, int K, bool w_on_chip) {
    const size_t N = m.n_sites;
    size_t s = w_on_chip ? N * (m.ld_up + m.ld_dn) * 4 : 0;  // W
    s += 2 * N * K * 4 + (size_t)(m.ld_up + m.ld_dn) * K * 4;  // P, Q
    s += (N + 1) * 4 + (size_t)m.n_bonds * 4 + (size_t)2 * m.n_bonds * 2 + 2 * N * 2 + 16;
    s += N * 4 + 4;  // up-neighbour counts (pipelined kernel)
    return (s + 15) / 16 * 16;
}

// ---------------------------------------------------------------------------
// Small kernels used by the Carlo-facing API and the parity tests.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void measure_kernel(DevModel m, DevBatch b) {
    const int w = blockIdx.x, N = m.n_sites;
    __shared__ double red[33];
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    T *gW = (sizeof(T) == 8 ? (T *)b.W64 : (T *)b.W32) + (size_t)w * wblock;
    WPtr<T> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    const double e = local_energy<T>(m, m.bonds, b.kappa_up + (size_t)w * N, b.kappa_dn + (size_t)w * N, W, red);
    if (threadIdx.x == 0) b.energy_out[w] = e;
}

template <typename T>
__global__ void ratio_kernel(DevModel m, DevBatch b, int n_moves, const int *moves, double *out) {
    const int w = blockIdx.x, N = m.n_sites;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    T *gW = (sizeof(T) == 8 ? (T *)b.W64 : (T *)b.W32) + (size_t)w * wblock;
    WPtr<T> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    for (int k = threadIdx.x; k < n_moves; k += blockDim.x) {
        const int *mv = moves + ((size_t)w * n_moves + k) * 4;
        out[(size_t)w * n_moves + k] = (double)W.U(mv[0], mv[1] - 1) * (double)W.D(mv[2], mv[3] - 1);
    }
}

template <typename T>
__global__ void apply_moves_kernel(DevModel m, DevBatch b, const int *moves) {
    const int w = blockIdx.x, N = m.n_sites;
    const int *mv = moves + (size_t)w * 5;
    const int flag = mv[0];
    if (flag == 0) return;
    const int i = mv[1], site = mv[2], l_up = mv[3], l_dn = mv[4];
    extern __shared__ __align__(16) unsigned char smem[];
    T *stg = reinterpret_cast<T *>(smem);
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    T *gW = (sizeof(T) == 8 ? (T *)b.W64 : (T *)b.W32) + (size_t)w * wblock;
    WPtr<T> W{gW, gW + (size_t)N * m.ld_up, m.ld_up, m.ld_dn};
    // flag 1: K_up = site, K_down = i; flag 2: K_up = i, K_down = site
    const int Ku = flag == 1 ? site : i;
    const int Kd = flag == 1 ? i : site;
    rank1_update<T>(W, N, Ku, l_up - 1, Kd, l_dn - 1, stg, stg + 2 * N, stg + N, stg + 2 * N + m.ld_up);
    if (threadIdx.x == 0) {
        short *ku = b.kappa_up + (size_t)w * N, *kd = b.kappa_dn + (size_t)w * N;
        if (flag == 1) {
            ku[i] = 0; ku[site] = (short)l_up;
            kd[i] = (short)l_dn; kd[site] = 0;
        } else {
            ku[i] = (short)l_up; ku[site] = 0;
            kd[i] = 0; kd[site] = (short)l_dn;
        }
    }
}

// Seeded uniformly random start (Fisher-Yates over sites with Philox stream
// 1, counter (word block, attempt, walker)); labels in increasing site order.
__global__ void init_random_kernel(DevModel m, DevBatch b, unsigned long long seed, const int *attempt,
                                   const int *redo) {
    const int w = blockIdx.x, N = m.n_sites;
    if (!redo[w]) return;
    extern __shared__ __align__(16) unsigned char smem[];
    short *perm = reinterpret_cast<short *>(smem);
    short *up = perm + N;
    if (threadIdx.x == 0) {
        for (int s = 0; s < N; ++s) { perm[s] = (short)s; up[s] = 0; }
        unsigned words[4];
        int nw = 0, ctr = 0;
        const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
        for (int k = N - 1; k > 0; --k) {
            if (nw == 0) {
                const uint4 x = philox4x32_10(make_uint4((unsigned)ctr, (unsigned)attempt[w], (unsigned)w, 1u), key);
                words[0] = x.x; words[1] = x.y; words[2] = x.z; words[3] = x.w;
                nw = 4;
                ++ctr;
            }
            const unsigned u = words[4 - nw];
            --nw;
            const int j = (int)(((unsigned long long)u * (unsigned long long)(k + 1)) >> 32);
            const short tmp = perm[k]; perm[k] = perm[j]; perm[j] = tmp;
        }
        for (int q = 0; q < m.n_up; ++q) up[perm[q]] = 1;
        int lu = 0, ld = 0;
        short *ku = b.kappa_up + (size_t)w * N, *kd = b.kappa_dn + (size_t)w * N;
        for (int s = 0; s < N; ++s) {
            if (up[s]) { ku[s] = (short)(++lu); kd[s] = 0; }
            else       { ku[s] = 0; kd[s] = (short)(++ld); }
        }
        b.status[w] = 0;
    }
}

// Targets of one call: kvmc_sweep sets t_end = t + proposals (no accepted
// target); kvmc_advance sets acc_end = accepted + moves and allows
// kAdvanceProposalsPerMove proposals per move.
__global__ void set_tend_kernel(DevBatch b, long long proposals, long long moves) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < b.n_walkers) {
        // moves: a walker that cannot make them stops after its proposal allowance
        b.t_end[w] = b.t[w] + (proposals > 0 ? proposals : min(moves, 1ll << 40) * kAdvanceProposalsPerMove);
        b.acc_end[w] = moves > 0 ? b.accepted[w] + moves : 0x3fffffffffffffffll;
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t launch_set_tend(const DevBatch &b, long long proposals, long long moves, cudaStream_t stream) {
    set_tend_kernel<<<(b.n_walkers + 255) / 256, 256, 0, stream>>>(b, proposals, moves);
    return cudaGetLastError();
}

// The FP32 refinement refresh with the LU blocked in HBM (more orbitals than
// the shared-memory FP32 LU holds).
cudaError_t launch_refresh32_large(const DevModel &m, const DevBatch &b, int only_due, int track_drift,
                                   cudaStream_t stream) {
    const dim3 grid(b.n_walkers, 2);
    const size_t sm = refresh_large_smem(m, 4);
    cudaError_t e = cudaFuncSetAttribute(refresh_large_kernel<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sm);
    if (e != cudaSuccess) return e;
    refresh_large_kernel<float, float><<<grid, kRefreshThreads, sm, stream>>>(m, b, only_due, track_drift);
    return cudaGetLastError();
}

int max_smem_optin(int device) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    return v;
}

cudaError_t launch_refresh(const DevModel &m, const DevBatch &b, bool fp32_out, int only_due,
                           int track_drift, cudaStream_t stream) {
    const dim3 grid(b.n_walkers, 2);
    if (refresh_needs_large(m)) {
        const size_t sm = refresh_large_smem(m);
        const int nmax = m.n_up > m.n_dn ? m.n_up : m.n_dn;
        const int omax = m.n_sites - (m.n_up < m.n_dn ? m.n_up : m.n_dn);
        const dim3 rgrid(b.n_walkers, 2, (omax + kRowsThreads - 1) / kRowsThreads);
        const size_t rsm = (size_t)nmax * (8 + 4) + (size_t)m.n_sites * 2 + 16;
        if (fp32_out) {
            cudaError_t e = cudaFuncSetAttribute(refresh_large_kernel<double, float>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            refresh_large_kernel<double, float><<<grid, kRefreshThreads, sm, stream>>>(m, b, only_due, track_drift);
            if (b.lu_perm) refresh_large_rows_kernel<float><<<rgrid, kRowsThreads, rsm, stream>>>(m, b, track_drift);
        } else {
            cudaError_t e = cudaFuncSetAttribute(refresh_large_kernel<double, double>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            refresh_large_kernel<double, double><<<grid, kRefreshThreads, sm, stream>>>(m, b, only_due, track_drift);
            if (b.lu_perm) refresh_large_rows_kernel<double><<<rgrid, kRowsThreads, rsm, stream>>>(m, b, track_drift);
        }
        return cudaGetLastError();
    }
    const size_t sm = refresh_smem(m);
    if (fp32_out) {
        cudaError_t e = cudaFuncSetAttribute(refresh_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        refresh_kernel<float><<<grid, kRefreshThreads, sm, stream>>>(m, b, only_due, track_drift);
    } else {
        cudaError_t e = cudaFuncSetAttribute(refresh_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        refresh_kernel<double><<<grid, kRefreshThreads, sm, stream>>>(m, b, only_due, track_drift);
    }
    return cudaGetLastError();
}

template <typename T, bool kSmemW>
static cudaError_t launch_sweep_impl(const DevModel &m, const DevBatch &b, const SweepParams &p,
                                     int by_proposals, int *active, int threads, cudaStream_t stream) {
    const size_t sm = sweep_smem_bytes<T, kSmemW>(m);
    cudaError_t e = cudaFuncSetAttribute(sweep_kernel<T, kSmemW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    sweep_kernel<T, kSmemW><<<b.n_walkers, threads, sm, stream>>>(m, b, p, by_proposals, active);
    return cudaGetLastError();
}

template <int K, bool kStream, int kThreads>
static cudaError_t launch_delayed_t(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                    cudaStream_t stream) {
    const size_t sm = delayed_smem_bytes(m, K, !kStream);
    cudaError_t e = cudaFuncSetAttribute(sweep_delayed_kernel<K, kStream, kThreads>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    sweep_delayed_kernel<K, kStream, kThreads><<<b.n_walkers, kThreads, sm, stream>>>(m, b, p, active);
    return cudaGetLastError();
}

template <int K, bool kStream, int kThreads, bool kTC = false>
static cudaError_t launch_pipe_t(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                 cudaStream_t stream) {
    size_t sm = delayed_smem_bytes(m, K, !kStream) + (kTC ? tc_flush_smem_bytes() : 0);
    // the threshold table joins the CTA's shared memory when the walkers per
    // SM the launch shape is made for (512 threads per SM) still fit
    const size_t thr_bytes = 16 + (size_t)(m.n_bonds + 1) * sizeof(ThrEntry);
    const int per_sm = kStream ? 512 / kThreads : 1;
    const size_t kSmemPerSM = 228 * 1024, kReserve = 1024 + 2048;  // per-CTA reserve and static shared data
    const int thr_in_smem = per_sm * (sm + thr_bytes + kReserve) <= kSmemPerSM && sm + thr_bytes <= 227 * 1024;
    if (thr_in_smem) sm += thr_bytes;
    cudaError_t e = cudaFuncSetAttribute(sweep_pipe_kernel<K, kStream, kThreads, kTC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    if constexpr (kStream && kThreads == 256 && !kTC && K >= 12) {
        // the uncapped form where it keeps as many CTAs per SM
        e = cudaFuncSetAttribute(sweep_pipe_wide_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        int occ_wide = 0, occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_wide, sweep_pipe_wide_kernel<K>, kThreads, sm);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sweep_pipe_kernel<K, kStream, kThreads, kTC>,
                                                              kThreads, sm);
        if (e != cudaSuccess) return e;
        if (occ_wide >= occ && occ_wide > 0) {
            sweep_pipe_wide_kernel<K><<<b.n_walkers, kThreads, sm, stream>>>(m, b, p, active, thr_in_smem);
            return cudaGetLastError();
        }
    }
    sweep_pipe_kernel<K, kStream, kThreads, kTC><<<b.n_walkers, kThreads, sm, stream>>>(m, b, p, active, thr_in_smem);
    return cudaGetLastError();
}

template <int K, bool kStream>
static cudaError_t launch_delayed(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                  cudaStream_t stream) {
    if (p.pipeline) {
        if constexpr (!kStream) return launch_pipe_t<K, false, 512>(m, b, p, active, stream);
        if (p.tc_flush) {
            if (p.stream_threads == 128) return launch_pipe_t<K, true, 128, true>(m, b, p, active, stream);
            return launch_pipe_t<K, true, 256, true>(m, b, p, active, stream);
        }
        if (p.stream_threads == 128) return launch_pipe_t<K, true, 128>(m, b, p, active, stream);
        return launch_pipe_t<K, true, 256>(m, b, p, active, stream);
    }
    if constexpr (!kStream) return launch_delayed_t<K, false, 512>(m, b, p, active, stream);
    if (p.stream_threads == 128) return launch_delayed_t<K, true, 128>(m, b, p, active, stream);
    return launch_delayed_t<K, true, 256>(m, b, p, active, stream);
}

cudaError_t launch_sweep(const DevModel &m, const DevBatch &b, const SweepParams &p, bool mixed,
                         bool smem_w, int *active, cudaStream_t stream) {
    if (!mixed) return launch_sweep_impl<double, false>(m, b, p, 1, active, 256, stream);
    if (p.cluster > 0) return launch_sweep_cluster(m, b, p, active, stream);
    if (p.warp_walkers > 0) return launch_sweep_warp(m, b, p, active, stream);
    if (smem_w && p.delay_k == 4) return launch_delayed<4, false>(m, b, p, active, stream);
    if (smem_w && p.delay_k == 8) return launch_delayed<8, false>(m, b, p, active, stream);
    if (smem_w && p.delay_k == 12) return launch_delayed<12, false>(m, b, p, active, stream);
    if (smem_w && p.delay_k == 16) return launch_delayed<16, false>(m, b, p, active, stream);
    // W in HBM, delayed factors on chip
    if (!smem_w && p.delay_k == 4) return launch_delayed<4, true>(m, b, p, active, stream);
    if (!smem_w && p.delay_k == 8) return launch_delayed<8, true>(m, b, p, active, stream);
    if (!smem_w && p.delay_k == 12) return launch_delayed<12, true>(m, b, p, active, stream);
    if (!smem_w && p.delay_k == 16) return launch_delayed<16, true>(m, b, p, active, stream);
    if (smem_w) return launch_sweep_impl<float, true>(m, b, p, 0, active, 512, stream);
    return launch_sweep_impl<float, false>(m, b, p, 0, active, 512, stream);
}

cudaError_t launch_measure(const DevModel &m, const DevBatch &b, bool fp32, cudaStream_t stream) {
    if (fp32) measure_kernel<float><<<b.n_walkers, 256, 0, stream>>>(m, b);
    else measure_kernel<double><<<b.n_walkers, 256, 0, stream>>>(m, b);
    return cudaGetLastError();
}

cudaError_t launch_eval_ratios(const DevModel &m, const DevBatch &b, bool fp32, int n_moves, const int *moves,
                               double *out, cudaStream_t stream) {
    if (fp32) ratio_kernel<float><<<b.n_walkers, 128, 0, stream>>>(m, b, n_moves, moves, out);
    else ratio_kernel<double><<<b.n_walkers, 128, 0, stream>>>(m, b, n_moves, moves, out);
    return cudaGetLastError();
}

cudaError_t launch_apply_moves(const DevModel &m, const DevBatch &b, bool fp32, const int *moves,
                               cudaStream_t stream) {
    const size_t elem = fp32 ? 4 : 8;
    const size_t sm = (size_t)(2 * m.n_sites + m.ld_up + m.ld_dn) * elem + 16;
    if (fp32) {
        cudaError_t e = cudaFuncSetAttribute(apply_moves_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        apply_moves_kernel<float><<<b.n_walkers, 256, sm, stream>>>(m, b, moves);
    } else {
        cudaError_t e = cudaFuncSetAttribute(apply_moves_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        apply_moves_kernel<double><<<b.n_walkers, 256, sm, stream>>>(m, b, moves);
    }
    return cudaGetLastError();
}

cudaError_t launch_init_random(const DevModel &m, const DevBatch &b, unsigned long long seed, const int *attempt,
                               const int *redo, cudaStream_t stream) {
    const size_t sm = (size_t)2 * m.n_sites * sizeof(short) + 16;
    init_random_kernel<<<b.n_walkers, 32, sm, stream>>>(m, b, seed, attempt, redo);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Refresh with no device allocation (kvmc_refresh_static).
//
// For callers that cannot allocate device memory: code running where every
// byte of the GPU belongs to another allocator (a Julia CUDA.jl memory pool,
// a framework's caching allocator) or where cudaMalloc's implicit device
// synchronisation is not allowed in the middle of a Monte Carlo loop.  The
// caller passes its own device buffers for inputs and outputs; the FP64
// rows being solved live in the fixed array below, which the library
// reserves on every GPU that loads it, for as long as the process runs.
// ---------------------------------------------------------------------------
constexpr size_t kStaticScratchBytes = 8u << 20;  // 8 MiB per device
static __device__ __align__(256) double g_static_solve_scratch[kStaticScratchBytes / sizeof(double)];

__global__ void __launch_bounds__(kRefreshThreads, 2)
refresh_static_kernel(int N, int n, const double *U, const int *kappa, double *W, double *logdet, double *scratch) {
    const int item = blockIdx.x;
    const int *ki = kappa + (size_t)item * N;
    double *Wi = W + (size_t)item * N * n;
    double *Y = scratch + (size_t)item * n * (N - n);
    extern __shared__ __align__(16) unsigned char smem[];
    const int lda = n + 1;
    double *A = reinterpret_cast<double *>(smem);
    double *invd = A + (size_t)n * lda;
    double *red = invd + n;
    int *perm = reinterpret_cast<int *>(red + 33);
    short *rows = reinterpret_cast<short *>(perm + n);
    // exactly N - n empty sites, or this item's rows would not fit its scratch block
    const int nrows = collect_empty_rows(ki, N, rows);
    if (nrows != N - n) {
        if (threadIdx.x == 0 && logdet) logdet[item] = NAN;
        return;
    }
    gather_tilde_u(A, lda, perm, U, ki, N, n);
    double ld = 0.0, lr = 0.0;
    if (lu_factor_shared(A, lda, n, perm, invd, red, ld, lr)) {
        if (threadIdx.x == 0 && logdet) logdet[item] = -INFINITY;
        return;
    }
    if (threadIdx.x == 0 && logdet) logdet[item] = ld;
    write_unit_rows(ki, N, n, Wi, n, false, (float *)nullptr);
    for (int r0 = 0; r0 < nrows; r0 += blockDim.x) {
        const int cnt = min((int)blockDim.x, nrows - r0);
        solve_rows_blocked<double>(A, lda, invd, perm, U, n, rows + r0, cnt, Y + (size_t)r0 * n, Wi, n,
                                   (float *)nullptr, false);
    }
}

namespace {
constexpr int kMaxDevices = 64;
void *g_static_scratch_ptr[kMaxDevices] = {};
std::mutex g_static_setup_mu;

// With the caller's device current: the device address of the static array
// (its host-side name is only a stand-in) and the kernel's shared-memory
// opt-in.  Both belong to the device's current context, so a call outside
// stream capture resolves them again (cheap, and right after a device reset
// or a new primary context); a call under capture, where the runtime must
// not be asked for them, reuses what the last call outside capture on this
// device resolved.
cudaError_t static_scratch_setup(int device, cudaStream_t stream, void **ptr) {
    std::lock_guard<std::mutex> lock(g_static_setup_mu);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess) return e;
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_solve_scratch);
        if (e != cudaSuccess) return e;
        // the kernel's own static shared variables count against the opt-in limit
        const int max_dyn = max_smem_optin(device) - 1024;
        e = cudaFuncSetAttribute(refresh_static_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn);
        if (e != cudaSuccess) return e;
        g_static_scratch_ptr[device] = p;
    } else if (!g_static_scratch_ptr[device]) {
        return cudaErrorStreamCaptureUnsupported;  // never resolved outside capture on this device
    }
    *ptr = g_static_scratch_ptr[device];
    return cudaSuccess;
}
}  // namespace

}  // namespace kvmc

extern "C" KVMC_API int kvmc_refresh_static(int32_t n_sites, int32_t n_orb, int32_t batch, const double *U,
                                            const int32_t *kappa, double *W, double *logdet, void *stream) {
    using namespace kvmc;
    if (n_sites <= 0 || n_sites > 30000 || n_orb <= 0 || n_orb >= n_sites || batch < 0 || !U || !kappa || !W)
        return KVMC_ERR_ARGUMENT;
    if (n_orb > 160) return KVMC_ERR_UNSUPPORTED;
    if (batch == 0) return KVMC_OK;
    const size_t need = (size_t)batch * n_orb * (n_sites - n_orb) * sizeof(double);
    if (need > kStaticScratchBytes) return KVMC_ERR_ARGUMENT;  // batch * n_orb * (n_sites - n_orb) * 8 > 8 MiB
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return KVMC_ERR_NO_DEVICE;
    void *scratch = nullptr;
    if (static_scratch_setup(device, static_cast<cudaStream_t>(stream), &scratch) != cudaSuccess) return KVMC_ERR_CUDA;
    const size_t sm = (size_t)n_orb * (n_orb + 1) * 8 + (size_t)n_orb * 8 + 33 * 8 + (size_t)n_orb * 4 +
                      (size_t)n_sites * 2 + 16;
    if ((int)sm > max_smem_optin(device) - 1024) return KVMC_ERR_UNSUPPORTED;
    refresh_static_kernel<<<batch, kRefreshThreads, sm, static_cast<cudaStream_t>(stream)>>>(
        n_sites, n_orb, U, reinterpret_cast<const int *>(kappa), W, logdet, static_cast<double *>(scratch));
    return cudaGetLastError() == cudaSuccess ? KVMC_OK : KVMC_ERR_CUDA;
}
