// Per-row FP32 iterative refinement of W = U tilde_U^{-1}, shared by the
// shared-memory refresh (kvmc_refresh32.cu) and the blocked-LU refresh for
// large orbital counts (kvmc_kernels.cu).  The arithmetic is stated in
// kvmc_refresh32.cu.
#pragma once

#include <cuda_runtime.h>

namespace kvmc {

constexpr int kCol = 8;  // columns per register block in the solves and the residual

// x tilde_U = x in place for one row held column-major at x[j * ld] (this
// thread's row): forward with Uf, backward with the unit L, in register
// blocks of kCol columns.  The result is in pivot order (x[i] for column
// perm[i] of W).
static __device__ void solve_row32(const float *A, int lda, const float *invd, int n, float *x, int ld) {
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


// One non-trivial row of W: site R, the row u = U[R,:] held as FP32 (high,
// low) pairs Uh/Ul (row-major, n per row), the FP32 factors A (lda) with
// 1/diagonal invd and row pivots perm, site_of[l] = the site holding label
// l+1.  y (column-major with stride cnt, 2n entries: the solution, then the
// correction) is this row's scratch.  Writes W row wr (in label order) and
// folds its change into dmax.  Returns false when the row did not converge
// (the caller flags the walker for the FP64 refresh).
static __device__ bool refine_row(const float *A, int lda, const float *invd, const int *perm, const short *site_of,
                                  const float *Uh, const float *Ul, int n, int R, float *y, int cnt, float *wr,
                                  bool track_drift, float &dmax) {
    float *d = y + (size_t)n * cnt;
    const float *uh_row = Uh + (size_t)R * n, *ul_row = Ul + (size_t)R * n;
    for (int j = 0; j < n; ++j) y[(size_t)j * cnt] = uh_row[j];
    solve_row32(A, lda, invd, n, y, cnt);  // y0, in pivot order: y[i] belongs to label perm[i]
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
        solve_row32(A, lda, invd, n, d, cnt);  // correction, in pivot order
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
    for (int i = 0; i < n; ++i) {
        const float nv = y[(size_t)i * cnt];
        if (track_drift) dmax = fmaxf(dmax, fabsf(wr[perm[i]] - nv) / (1.f + fabsf(nv)));
        wr[perm[i]] = nv;
    }
    return ratio <= 1e-4f;
}

}  // namespace kvmc
