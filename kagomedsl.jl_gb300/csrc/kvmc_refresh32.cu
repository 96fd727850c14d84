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

namespace kvmc {

namespace {

constexpr int kThreads32 = 256;
constexpr int kMaxN32 = 224;
constexpr int kCol = 8;  // columns per register block in the solves and the residual

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

// x tilde_U = x in place for one row held column-major at x[j * ld] (this
// thread's row): forward with Uf, backward with the unit L, in register
// blocks of kCol columns.  The result is in pivot order (x[i] for column
// perm[i] of W).
__device__ void solve_row32(const float *A, int lda, const float *invd, int n, float *x, int ld) {
    for (int jb = 0; jb < n; jb += kCol) {
        const int nb = min(kCol, n - jb);
        float yb[kCol];
#pragma unroll
        for (int q = 0; q < kCol; ++q) yb[q] = q < nb ? x[(size_t)(jb + q) * ld] : 0.f;
#pragma unroll
        for (int ii = 0; ii < kCol; ++ii) {
            if (ii < nb) {
                yb[ii] *= invd[jb + ii];
                const float *Ai = A + (size_t)(jb + ii) * lda + jb;
#pragma unroll
                for (int jj = ii + 1; jj < kCol; ++jj)
                    if (jj < nb) yb[jj] = fmaf(-yb[ii], Ai[jj], yb[jj]);
            }
        }
#pragma unroll
        for (int q = 0; q < kCol; ++q)
            if (q < nb) x[(size_t)(jb + q) * ld] = yb[q];
        for (int j0 = jb + kCol; j0 < n; j0 += kCol) {
            const int cnt = min(kCol, n - j0);
            float acc[kCol];
#pragma unroll
            for (int t = 0; t < kCol; ++t) acc[t] = t < cnt ? x[(size_t)(j0 + t) * ld] : 0.f;
#pragma unroll
            for (int ii = 0; ii < kCol; ++ii) {
                if (ii < nb) {
                    const float *Ai = A + (size_t)(jb + ii) * lda + j0;
#pragma unroll
                    for (int t = 0; t < kCol; ++t)
                        if (t < cnt) acc[t] = fmaf(-yb[ii], Ai[t], acc[t]);
                }
            }
#pragma unroll
            for (int t = 0; t < kCol; ++t)
                if (t < cnt) x[(size_t)(j0 + t) * ld] = acc[t];
        }
    }
    const int last = ((n - 1) / kCol) * kCol;
    for (int jb = last; jb >= 0; jb -= kCol) {
        const int nb = min(kCol, n - jb);
        float yb[kCol];
#pragma unroll
        for (int q = 0; q < kCol; ++q) yb[q] = q < nb ? x[(size_t)(jb + q) * ld] : 0.f;
#pragma unroll
        for (int ii = kCol - 1; ii >= 0; --ii) {
            if (ii < nb) {
                const float *Aj = A + (size_t)(jb + ii) * lda + jb;
#pragma unroll
                for (int kk = 0; kk < ii; ++kk) yb[kk] = fmaf(-yb[ii], Aj[kk], yb[kk]);
            }
        }
#pragma unroll
        for (int q = 0; q < kCol; ++q)
            if (q < nb) x[(size_t)(jb + q) * ld] = yb[q];
        for (int i0 = 0; i0 < jb; i0 += kCol) {
            const int cnt = min(kCol, jb - i0);
            float acc[kCol];
#pragma unroll
            for (int t = 0; t < kCol; ++t) acc[t] = t < cnt ? x[(size_t)(i0 + t) * ld] : 0.f;
#pragma unroll
            for (int ii = 0; ii < kCol; ++ii) {
                if (ii < nb) {
                    const float *Aj = A + (size_t)(jb + ii) * lda + i0;
#pragma unroll
                    for (int t = 0; t < kCol; ++t)
                        if (t < cnt) acc[t] = fmaf(-yb[ii], Aj[t], acc[t]);
                }
            }
#pragma unroll
            for (int t = 0; t < kCol; ++t)
                if (t < cnt) x[(size_t)(i0 + t) * ld] = acc[t];
        }
    }
}

// (hi, lo) += a * b with the product exact (a, b floats) and the sum compensated
__device__ __forceinline__ void df_fma(float a, float b, float &hi, float &lo) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float s = hi + p;
    const float bv = s - hi;
    const float err = (hi - (s - bv)) + (p - bv);
    hi = s;
    lo += err + e;
}

__global__ void __launch_bounds__(kThreads32, 2)
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
    float *W = b.W32 + (size_t)w * wblock + (spin == 0 ? 0 : (size_t)N * m.ld_up);

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
    // unit rows at occupied sites, zero padding elsewhere
    {
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
            float *y = Y + (size_t)r0 * n * 2 + r;       // this block's rows: y0 at [j * cnt], d after n * cnt
            float *d = y + (size_t)n * cnt;
            const float *uh_row = Uh + (size_t)R * n, *ul_row = Ul + (size_t)R * n;
            for (int j = 0; j < n; ++j) y[(size_t)j * cnt] = uh_row[j];
            solve_row32(A, lda, invd, n, y, cnt);        // y0, in pivot order: y[i] belongs to label perm[i]
            float ratio = 0.f;
            for (int pass = 0; pass < 2; ++pass) {
            // residual r_j = u_j - sum_i y[i] U[site holding label perm[i]][j]
            for (int j0 = 0; j0 < n; j0 += kCol) {
                const int cc = min(kCol, n - j0);
                float hi[kCol], lo[kCol];
#pragma unroll
                for (int t = 0; t < kCol; ++t) { hi[t] = 0.f; lo[t] = 0.f; }
                for (int i = 0; i < n; ++i) {
                    const float yi = y[(size_t)i * cnt];
                    const size_t base = (size_t)site_of[perm[i]] * n + j0;
#pragma unroll
                    for (int t = 0; t < kCol; ++t) {
                        if (t < cc) {
                            df_fma(yi, Uh[base + t], hi[t], lo[t]);
                            lo[t] = fmaf(yi, Ul[base + t], lo[t]);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < kCol; ++t)
                    if (t < cc) d[(size_t)(j0 + t) * cnt] = ((uh_row[j0 + t] - hi[t]) - lo[t]) + ul_row[j0 + t];
            }
            solve_row32(A, lda, invd, n, d, cnt);        // correction, in pivot order
            float dm = 0.f, ym = 0.f;
            for (int i = 0; i < n; ++i) {
                const float nv = y[(size_t)i * cnt] + d[(size_t)i * cnt];
                dm = fmaxf(dm, fabsf(d[(size_t)i * cnt]));
                ym = fmaxf(ym, fabsf(nv));
                y[(size_t)i * cnt] = nv;
            }
            ratio = dm / fmaxf(ym, 1e-30f);
            if (!(ratio > 1e-3f)) break;
            }
            if (!(ratio <= 1e-4f)) atomicOr(&b.status[w], kStatusRefine);
            float *wr = W + (size_t)R * ldw;
            for (int i = 0; i < n; ++i) {
                const float nv = y[(size_t)i * cnt];
                if (track_drift) dmax = fmaxf(dmax, fabsf(wr[perm[i]] - nv) / (1.f + fabsf(nv)));
                wr[perm[i]] = nv;
            }
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

cudaError_t launch_clear_status(const DevBatch &b, int bits, cudaStream_t stream) {
    clear_status_bits_kernel<<<(b.n_walkers + 255) / 256, 256, 0, stream>>>(b, bits);
    return cudaGetLastError();
}

cudaError_t launch_refresh32(const DevModel &m, const DevBatch &b, int only_due, int track_drift, cudaStream_t stream) {
    const size_t sm = refresh32_smem(m);
    cudaError_t e = cudaFuncSetAttribute(refresh32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    refresh32_kernel<<<dim3(b.n_walkers, 2), kThreads32, sm, stream>>>(m, b, only_due, track_drift);
    return cudaGetLastError();
}

}  // namespace kvmc
