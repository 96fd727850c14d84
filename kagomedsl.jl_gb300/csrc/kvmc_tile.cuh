// Device functions of the tiled FP32 refresh (kvmc_refresh_tile.cu) that the
// refresh with its residual on the tensor cores (kvmc_refresh_oz.cu) shares:
// the blocked LU with implicit pivoting, the 32-row tile solves, the
// cp.async-pipelined GEMM-shaped chunk loop and the fixed-grid residual.
// Everything sits in an anonymous namespace, so each translation unit that
// includes it has its own copy.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc.h"
#include "kvmc_device.cuh"
#include "kvmc_internal.h"
#include "kvmc_refine.cuh"

namespace kvmc {

namespace {


constexpr int kTT = 256;                // threads per CTA
constexpr int kNW = kTT / 32;           // warps per CTA
constexpr int kPB = 32;        // LU panel width, column block of the solves and the residual
constexpr int kRT = 32;        // rows per tile of X
constexpr int kRW = kRT / kNW;  // rows of the tile each warp owns
constexpr int kLdc = kPB + 1;  // leading dimension of the staged block columns
constexpr int kMaxPasses = 4; // refinement passes per tile at most
constexpr int kCB = 64;        // columns per block of the GEMM-shaped loops
constexpr int kKC = 64;        // rows of G / tilde_U per staged chunk

__host__ __device__ inline int round4(int n) { return (n + 3) & ~3; }
__host__ __device__ inline int ld_tile(int n) { return round4(n); }

// Copies `rows` rows of up to 32 columns into shared memory: dst[k * ld + c]
// = src(k)[c] for c < nc, zero where src(k) is null or nc <= c < wc; columns
// from wc on are not written.  Each thread issues up to 8 global loads
// before its first store, so that their latencies overlap.
template <typename Src>
__device__ __forceinline__ void stage_rows32(float *dst, int ld, int rows, int nc, int wc, Src src) {
    constexpr int kB = 8;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int total = rows * 32;
    for (int e0 = tid; e0 < total; e0 += nt * kB) {
        float v[kB];
#pragma unroll
        for (int q = 0; q < kB; ++q) {
            const int e = e0 + q * nt;
            const int k = e >> 5, c = e & 31;
            const float *p = (e < total && c < nc) ? src(k) : nullptr;
            v[q] = p ? p[c] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < kB; ++q) {
            const int e = e0 + q * nt;
            if (e < total && (e & 31) < wc) dst[(e >> 5) * ld + (e & 31)] = v[q];
        }
    }
}

// 4-byte asynchronous copy global -> shared; ok = false writes a zero.
__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// stage_rows32 with every element's copy in flight at once (cp.async, 4
// bytes each, no registers held), for block columns read once per solve
// from HBM or L2: the CTA waits one memory latency per block column, not
// one per eight elements.  `any` is a valid global address for the copies
// that write a zero.  Ends with the copies landed and the CTA synchronised.
template <typename Src>
__device__ __forceinline__ void stage_rows32_async(float *dst, int ld, int rows, int nc, int wc, Src src,
                                                   const float *any) {
    const int total = rows * 32;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int k = e >> 5, c = e & 31;
        if (c >= wc) continue;
        const float *p = c < nc ? src(k) : nullptr;
        cp_async4(dst + (size_t)k * ld + c, p ? p + c : any, p != nullptr);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
}

// Shared-memory layout (byte offsets, each a multiple of 16).
struct TileSmem {
    size_t z, r, pn, ut, st, invd, perm, srow, site_of, site_oth, total;
};

__host__ __device__ inline TileSmem tile_smem_layout(int n, int n_oth) {
    auto al = [](size_t x) { return (x + 15) / 16 * 16; };
    TileSmem s{};
    const size_t tile = al((size_t)kRT * ld_tile(n) * 4);
    const size_t lu = al((size_t)n * kLdc * 4) + (size_t)kPB * 64 * 4;
    s.z = 0;
    s.r = tile;
    s.pn = 0;  // the LU's panel lives where the tiles will be
    s.ut = al((size_t)n * kLdc * 4);
    size_t o = 2 * tile > lu ? 2 * tile : lu;
    // the chunk double buffer (two buffers of high and low planes), or the
    // block column of tile_solve
    const size_t chunks = (size_t)2 * 2 * kKC * kCB * 4, bcol = (size_t)round4(n) * kLdc * 4;
    s.st = o; o = al(o + (chunks > bcol ? chunks : bcol));
    s.invd = o; o = al(o + (size_t)n * 4);
    s.perm = o; o = al(o + (size_t)n * 4);
    s.srow = o; o = al(o + (size_t)n * 4);
    s.site_of = o; o = al(o + (size_t)n * 2);
    s.site_oth = o; o = al(o + (size_t)n_oth * 2);
    s.total = o;
    return s;
}

// The LU of one staged panel (rp rows of Pn, nb <= 32 columns) with its rows
// in registers, one row per thread (rp <= kTT, blockDim.x == kTT): the pivot
// choice of the shared-memory form in lu_blocked (the largest |entry|, the
// first position among equals) and its operations in the same order, so the
// factors are the same bit for bit; two barriers per column in place of
// three, and the column update in registers.  A row stays with its thread;
// `pos` follows its position through the swaps, and the rows go back to Pn
// in pivot order at the end.  permp is the pivot order from the panel's
// first row on.  Returns false on an exactly zero pivot (every thread sees
// the same answer).
__device__ __noinline__ bool panel_lu_regs(float *Pn, int rp, int nb, int *permp) {
    __shared__ float s_val[kNW];
    __shared__ int s_pos[kNW];
    __shared__ float s_row[kPB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool mine = tid < rp;
    int pos = tid;
    float v[kPB];
#pragma unroll
    for (int j = 0; j < kPB; ++j) v[j] = mine ? Pn[(size_t)tid * kLdc + j] : 0.f;
#pragma unroll
    for (int k = 0; k < kPB; ++k) {
        if (k >= nb) break;
        float best = -1.f;
        int bi = rp;
        if (mine && pos >= k) {
            const float a = fabsf(v[k]);
            if (a > best) { best = a; bi = pos; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { s_val[warp] = best; s_pos[warp] = bi; }
        __syncthreads();
        best = s_val[0];
        bi = s_pos[0];
#pragma unroll
        for (int g = 1; g < kNW; ++g) {
            const float ob = s_val[g];
            const int oi = s_pos[g];
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (!(best > 0.f)) return false;
        if (mine && pos == bi) {
#pragma unroll
            for (int j = 0; j < kPB; ++j) s_row[j] = v[j];
        }
        if (mine) pos = pos == k ? bi : (pos == bi ? k : pos);
        if (tid == 0 && bi != k) { const int t = permp[k]; permp[k] = permp[bi]; permp[bi] = t; }
        __syncthreads();
        if (mine && pos > k) {
            const float dinv = 1.f / s_row[k];
            const float l = v[k] * dinv;
            v[k] = l;
#pragma unroll
            for (int j = k + 1; j < kPB; ++j)
                if (j < nb) v[j] = fmaf(-l, s_row[j], v[j]);
        }
    }
    if (mine) {
#pragma unroll
        for (int j = 0; j < kPB; ++j) Pn[(size_t)pos * kLdc + j] = v[j];
    }
    __syncthreads();
    return true;
}

// The LU of one staged panel in shared memory, for panels of any height:
// one warp finds the pivot (the largest |entry|, the first position among
// equals), the pivot row is swapped into place, and every thread updates
// rows below it.  permp is the pivot order from the panel's first row on.
// Returns false on an exactly zero pivot (every thread sees the same
// answer).
__device__ __forceinline__ bool panel_lu_smem(float *Pn, int rp, int nb, int *permp) {
    __shared__ int s_piv;
    __shared__ float s_pmax, s_dinv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    for (int k = 0; k < nb; ++k) {
        if (warp == 0) {
            float best = -1.f;
            int bi = rp;
            for (int i = k + lane; i < rp; i += 32) {
                const float v = fabsf(Pn[(size_t)i * kLdc + k]);
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
                s_dinv = best > 0.f ? 1.f / Pn[(size_t)bi * kLdc + k] : 0.f;
            }
        }
        __syncthreads();
        if (!(s_pmax > 0.f)) return false;
        const int p = s_piv;
        if (p != k) {
            for (int j = tid; j < kPB; j += nt) {
                const float a = Pn[(size_t)k * kLdc + j];
                Pn[(size_t)k * kLdc + j] = Pn[(size_t)p * kLdc + j];
                Pn[(size_t)p * kLdc + j] = a;
            }
            if (tid == 0) { const int t = permp[k]; permp[k] = permp[p]; permp[p] = t; }
        }
        __syncthreads();
        const float dinv = s_dinv;
        for (int i = k + 1 + tid; i < rp; i += nt) {
            const float l = Pn[(size_t)i * kLdc + k] * dinv;
            Pn[(size_t)i * kLdc + k] = l;
            for (int j = k + 1; j < nb; ++j)
                Pn[(size_t)i * kLdc + j] = fmaf(-l, Pn[(size_t)k * kLdc + j], Pn[(size_t)i * kLdc + j]);
        }
        __syncthreads();
    }
    return true;
}

// P A = L Uf of A (n x n, row-major, lda = n, global memory) in FP32 with
// partial pivoting (first maximal |pivot| wins).  Rows stay where they are:
// row i of the factors is A[perm[i]].  Returns false on an exactly zero
// pivot (every thread sees the same answer).
__device__ __forceinline__ bool lu_blocked(float *A, int n, float *Pn, float *Ut, float *invd, int *perm) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < n; i += nt) perm[i] = i;
    __syncthreads();
    for (int pb = 0; pb < n; pb += kPB) {
        const int nb = min(kPB, n - pb);
        const int rp = n - pb;
        stage_rows32(Pn, kLdc, rp, nb, 32, [&](int r) -> const float * { return A + (size_t)perm[pb + r] * n + pb; });
        __syncthreads();
        const bool ok = rp <= kTT && nt == kTT ? panel_lu_regs(Pn, rp, nb, perm + pb) : panel_lu_smem(Pn, rp, nb, perm + pb);
        if (!ok) return false;
        for (int e = tid; e < rp * kPB; e += nt) {
            const int r = e >> 5, c = e & 31;
            if (c < nb) A[(size_t)perm[pb + r] * n + pb + c] = Pn[(size_t)r * kLdc + c];
        }
        const int c0 = pb + nb;
        if (c0 < n) {
            // U12 = L11^{-1} A12, one column per thread (rows perm[pb .. pb + nb))
            for (int c = c0 + tid; c < n; c += nt) {
                float x[kPB];
#pragma unroll
                for (int i = 0; i < kPB; ++i) x[i] = i < nb ? A[(size_t)perm[pb + i] * n + c] : 0.f;
#pragma unroll
                for (int i = 1; i < kPB; ++i) {
                    float acc = x[i];
#pragma unroll
                    for (int k = 0; k < i; ++k) acc = fmaf(-Pn[(size_t)i * kLdc + k], x[k], acc);
                    x[i] = acc;
                }
#pragma unroll
                for (int i = 0; i < kPB; ++i)
                    if (i < nb) A[(size_t)perm[pb + i] * n + c] = x[i];
            }
            __syncthreads();
            // A22 -= L21 U12: 64-column tiles of U12 in shared memory, 4 x 4 per thread
            const int tx = tid & 15, ty = tid >> 4;
            for (int cb = c0; cb < n; cb += 64) {
                const int ncol = min(64, n - cb);
                for (int h = 0; h < 2; ++h)
                    stage_rows32(Ut + 32 * h, 64, kPB, ncol - 32 * h, 32, [&](int k) -> const float * {
                        return k < nb ? A + (size_t)perm[pb + k] * n + cb + 32 * h : nullptr;
                    });
                __syncthreads();
                for (int rb = c0; rb < n; rb += 4 * (kTT / 16)) {
                    // the A22 entries first, so that their loads overlap the products
                    float acc[4][4] = {}, old[4][4];
                    int rr[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        rr[a] = min(rb + 4 * ty + a, n - 1);
                        const float *Ar = A + (size_t)perm[rr[a]] * n;
#pragma unroll
                        for (int q = 0; q < 4; ++q) old[a][q] = Ar[min(cb + 4 * tx + q, n - 1)];
                    }
                    for (int k = 0; k < nb; ++k) {
                        float lv[4];
#pragma unroll
                        for (int a = 0; a < 4; ++a) lv[a] = Pn[(size_t)(rr[a] - pb) * kLdc + k];
                        const float4 uv = *reinterpret_cast<const float4 *>(Ut + k * 64 + 4 * tx);
#pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            acc[a][0] = fmaf(lv[a], uv.x, acc[a][0]);
                            acc[a][1] = fmaf(lv[a], uv.y, acc[a][1]);
                            acc[a][2] = fmaf(lv[a], uv.z, acc[a][2]);
                            acc[a][3] = fmaf(lv[a], uv.w, acc[a][3]);
                        }
                    }
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int r = rb + 4 * ty + a;
                        if (r >= n) continue;
                        float *Ar = A + (size_t)perm[r] * n;
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int c = cb + 4 * tx + q;
                            if (c < n) Ar[c] = old[a][q] - acc[a][q];
                        }
                    }
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < n; i += nt) invd[i] = 1.f / A[(size_t)perm[i] * n + i];
    __syncthreads();
    return true;
}

// Z := Z (L Uf)^{-1} for the tile (rows x n, leading dimension ldz): forward
// with Uf, backward with the unit lower L, in pivot order.  Warp g owns rows
// g, g + kNW, ...; lane = column within the block.  Uc stages one
// block column of the factors (the forward sweep from row j0 on).  Columns
// n .. round4(n) of Z are zero, and so are its columns left of j0 (a
// multiple of 32), which the forward sweep then skips.  The pivots'
// reciprocals of a block travel in a register of its lane and reach the
// serial part by shuffles.
__device__ __forceinline__ void tile_solve(const float *A, const int *perm, int n, const float *invd, float *Z, int ldz,
                                           int rows, float *Uc, int j0) {
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int n4 = round4(n);
    for (int jb = j0; jb < n; jb += kPB) {
        const int nb = min(kPB, n - jb);
        const int kr = jb + nb - j0;
        const float dl = lane < nb ? invd[jb + lane] : 0.f;
        __syncthreads();
        stage_rows32_async(Uc, kLdc, kr, nb, 32,
                           [&](int k) -> const float * { return A + (size_t)perm[j0 + k] * n + jb; }, A);
        float acc[kRW] = {};
        for (int k = j0; k < jb; k += 4) {
            const float *u = Uc + (size_t)(k - j0) * kLdc + lane;
            const float u0 = u[0], u1 = u[kLdc], u2 = u[2 * kLdc], u3 = u[3 * kLdc];
#pragma unroll
            for (int a = 0; a < kRW; ++a) {
                const float4 z = *reinterpret_cast<const float4 *>(Z + (size_t)(g + kNW * a) * ldz + k);
                acc[a] = fmaf(z.x, u0, acc[a]);
                acc[a] = fmaf(z.y, u1, acc[a]);
                acc[a] = fmaf(z.z, u2, acc[a]);
                acc[a] = fmaf(z.w, u3, acc[a]);
            }
        }
        float x[kRW];
#pragma unroll
        for (int a = 0; a < kRW; ++a) {
            const int r = g + kNW * a;
            x[a] = (r < rows && lane < nb) ? Z[(size_t)r * ldz + jb + lane] - acc[a] : 0.f;
        }
        for (int j = 0; j < nb; ++j) {
            const float uj = Uc[(jb - j0 + j) * kLdc + lane];
            const float dj = __shfl_sync(0xffffffffu, dl, j);
#pragma unroll
            for (int a = 0; a < kRW; ++a) {
                const float xj = __shfl_sync(0xffffffffu, x[a], j) * dj;
                x[a] = lane == j ? xj : (lane > j ? fmaf(-xj, uj, x[a]) : x[a]);
            }
        }
#pragma unroll
        for (int a = 0; a < kRW; ++a) {
            const int r = g + kNW * a;
            if (r < rows && lane < nb) Z[(size_t)r * ldz + jb + lane] = x[a];
        }
    }
    const int last = ((n - 1) / kPB) * kPB;
    for (int jb = last; jb >= 0; jb -= kPB) {
        const int nb = min(kPB, n - jb);
        const int kr = n4 - jb;
        __syncthreads();
        stage_rows32_async(
            Uc, kLdc, kr, nb, 32,
            [&](int k) -> const float * { return jb + k < n ? A + (size_t)perm[jb + k] * n + jb : nullptr; }, A);
        float acc[kRW] = {};
        for (int k = jb + kPB; k < n4; k += 4) {
            const float *u = Uc + (size_t)(k - jb) * kLdc + lane;
            const float u0 = u[0], u1 = u[kLdc], u2 = u[2 * kLdc], u3 = u[3 * kLdc];
#pragma unroll
            for (int a = 0; a < kRW; ++a) {
                const float4 z = *reinterpret_cast<const float4 *>(Z + (size_t)(g + kNW * a) * ldz + k);
                acc[a] = fmaf(z.x, u0, acc[a]);
                acc[a] = fmaf(z.y, u1, acc[a]);
                acc[a] = fmaf(z.z, u2, acc[a]);
                acc[a] = fmaf(z.w, u3, acc[a]);
            }
        }
        float x[kRW];
#pragma unroll
        for (int a = 0; a < kRW; ++a) {
            const int r = g + kNW * a;
            x[a] = (r < rows && lane < nb) ? Z[(size_t)r * ldz + jb + lane] - acc[a] : 0.f;
        }
        for (int j = nb - 1; j > 0; --j) {
            const float lj = Uc[j * kLdc + lane];
#pragma unroll
            for (int a = 0; a < kRW; ++a) {
                const float vj = __shfl_sync(0xffffffffu, x[a], j);
                if (lane < j) x[a] = fmaf(-vj, lj, x[a]);
            }
        }
#pragma unroll
        for (int a = 0; a < kRW; ++a) {
            const int r = g + kNW * a;
            if (r < rows && lane < nb) Z[(size_t)r * ldz + jb + lane] = x[a];
        }
    }
    __syncthreads();
}

// Chunk (k0 .. k0 + kKC) x (c0 .. c0 + kCB) of a matrix whose row k is
// row(k) (n columns), into buf (row stride kCB); zero outside n x n.
template <typename Row>
__device__ __forceinline__ void stage_chunk(float *buf, int n, int k0, int c0, Row row) {
    for (int e = threadIdx.x; e < kKC * kCB; e += kTT) {
        const int k = k0 + (e >> 6), c = c0 + (e & 63);
        const bool ok = k < n && c < n;
        const float *src = row(ok ? k : 0);
        cp_async4(buf + e, ok ? src + c : src, ok);
    }
}

// The loop both GEMM-shaped phases share: for each 64-column block, the
// k-chunks of the right operand are staged by cp.async into one half of
// the double buffer while the other half is multiplied.  body(buf, kc, kn)
// multiplies one staged chunk (kn rows); begin(cb) / end(cb) open and close
// a column block.  Thread (rg = tid / 16, cg = tid % 16) owns tile rows rg
// and rg + 16 and columns 4 cg .. 4 cg + 3 of the block.
template <int kPlanes, typename Stage, typename Begin, typename Body, typename End>
__device__ __forceinline__ void chunk_loop(int n, float *st, Stage stage, Begin begin, Body body, End end) {
    const int n4 = round4(n);
    const int ncb = (n + kCB - 1) / kCB, nkc = (n4 + kKC - 1) / kKC, S = ncb * nkc;
    constexpr int kBuf = kPlanes * kKC * kCB;
    __syncthreads();  // the buffer's previous users are done
    stage(st, 0, 0);
    cp_async_commit();
    for (int s = 0; s < S; ++s) {
        const int cbi = s / nkc, kci = s - cbi * nkc;
        if (s + 1 < S) {
            const int cn = (s + 1) / nkc, kn = (s + 1) - cn * nkc;
            stage(st + ((s + 1) & 1) * kBuf, kn * kKC, cn * kCB);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        if (kci == 0) begin(cbi * kCB);
        body(st + (s & 1) * kBuf, kci * kKC, min(kKC, n4 - kci * kKC));
        if (kci == nkc - 1) end(cbi * kCB);
        __syncthreads();  // this half is free for the chunk after next
    }
}

// Out = In G (mode 0) or Out += In G (mode 1) for the tile; G (n x n,
// row-major) in HBM.  Mode 1 returns, for the tile's first `rows` rows, the
// largest |In G| relative to the row's largest |Out| (infinite when a row
// is not finite); In and Out have leading dimension ldz.
__device__ __forceinline__ float tile_gemm(const float *G, int n, const float *In, float *Out, int ldz, int rows,
                                           int mode, float *st, double *red) {
    const int tid = threadIdx.x, rg = tid >> 4, cg = tid & 15;
    float acc[2][4];
    float dm[2] = {0.f, 0.f}, vm[2] = {0.f, 0.f};
    chunk_loop<1>(
        n, st,
        [&](float *buf, int k0, int c0) { stage_chunk(buf, n, k0, c0, [&](int k) { return G + (size_t)k * n; }); },
        [&](int) {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
        },
        [&](const float *buf, int kc, int kn) {
            const float *a0 = In + (size_t)rg * ldz + kc, *a1 = In + (size_t)(rg + 16) * ldz + kc;
            for (int kk = 0; kk < kn; kk += 4) {
                const float4 x0 = *reinterpret_cast<const float4 *>(a0 + kk);
                const float4 x1 = *reinterpret_cast<const float4 *>(a1 + kk);
                const float v0[4] = {x0.x, x0.y, x0.z, x0.w}, v1[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 u = *reinterpret_cast<const float4 *>(buf + (kk + q) * kCB + 4 * cg);
                    acc[0][0] = fmaf(v0[q], u.x, acc[0][0]);
                    acc[0][1] = fmaf(v0[q], u.y, acc[0][1]);
                    acc[0][2] = fmaf(v0[q], u.z, acc[0][2]);
                    acc[0][3] = fmaf(v0[q], u.w, acc[0][3]);
                    acc[1][0] = fmaf(v1[q], u.x, acc[1][0]);
                    acc[1][1] = fmaf(v1[q], u.y, acc[1][1]);
                    acc[1][2] = fmaf(v1[q], u.z, acc[1][2]);
                    acc[1][3] = fmaf(v1[q], u.w, acc[1][3]);
                }
            }
        },
        [&](int cb) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = rg + 16 * i;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = cb + 4 * cg + j;
                    if (c >= n) continue;
                    float *o = Out + (size_t)r * ldz + c;
                    if (mode == 0) {
                        *o = acc[i][j];
                    } else {
                        const float nv = *o + acc[i][j];
                        *o = nv;
                        if (r < rows) {
                            dm[i] = fmaxf(dm[i], isfinite(nv) ? fabsf(acc[i][j]) : INFINITY);
                            vm[i] = fmaxf(vm[i], fabsf(nv));
                        }
                    }
                }
            }
        });
    if (mode == 0) return 0.f;
    // per row over its 16 threads (lanes of one half-warp), then over the rows
    float q = 0.f;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            dm[i] = fmaxf(dm[i], __shfl_xor_sync(0xffffffffu, dm[i], o));
            vm[i] = fmaxf(vm[i], __shfl_xor_sync(0xffffffffu, vm[i], o));
        }
        const float qi = dm[i] / fmaxf(vm[i], 1e-30f);
        q = isnan(qi) ? INFINITY : fmaxf(q, qi);
    }
    return (float)block_sum_max((double)q, red);
}

// R = B - V M for the tile: row k of M is U at site srow[k], row r of B is U
// at site site_oth[b0 + r] (rows from `rows` on are zero).  U enters as FP32
// (high, low) pairs.
//
// The high-part products are summed without rounding error by splitting
// each on a fixed grid (the extraction step of Rump, Ogita and Oishi's
// accurate summation): for row r, sigma_r is a power of two with
// sum_k |v_k u_kc| <= sigma_r / 4, which 4 ||v_r||_2 max_c ||u_:c||_2
// bounds (cmax = the largest column norm of tilde_U).  Then t = fl(v u +
// sigma) lies in [3/4, 5/4] sigma, q = t - sigma is exact and a multiple
// of 2^-24 sigma, and every partial sum of the q stays below sigma / 2, so
// hi = sum q is exact.  The remainders fl(v u - q) (at most 2^-24 sigma)
// and the products with the low parts (2^-24 of the high ones) are summed
// in lo.  Six FP32 operations per product.
__device__ __forceinline__ void tile_residual(const float *Uh, const float *Ul, int n, const int *srow,
                                              const short *site_oth, int b0, int rows, const float *V, float *R,
                                              int ldz, float *st, float cmax) {
    const int tid = threadIdx.x, rg = tid >> 4, cg = tid & 15;
    float sg[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float *vr = V + (size_t)(rg + 16 * i) * ldz;
        float ss = 0.f;
        for (int c = cg; c < n; c += 16) ss = fmaf(vr[c], vr[c], ss);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        const float x = 4.f * sqrtf(ss) * cmax * 1.0001f;
        int e = 0;
        frexpf(x, &e);                               // x = m 2^e, m in [1/2, 1)
        sg[i] = x < INFINITY ? ldexpf(1.f, e) : x;   // a power of two >= x (0 for a zero row)
    }
    float hi[2][4], lo[2][4], bh[2][4], bl[2][4];
    constexpr int kPlane = kKC * kCB;
    chunk_loop<2>(
        n, st,
        [&](float *buf, int k0, int c0) {
            stage_chunk(buf, n, k0, c0, [&](int k) { return Uh + (size_t)srow[k] * n; });
            stage_chunk(buf + kPlane, n, k0, c0, [&](int k) { return Ul + (size_t)srow[k] * n; });
        },
        [&](int cb) {
            // this block's entries of B, loaded now so that they arrive during the block
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = rg + 16 * i;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = cb + 4 * cg + j;
                    const bool ok = r < rows && c < n;
                    const size_t src = ok ? (size_t)site_oth[b0 + r] * n + c : 0;
                    bh[i][j] = ok ? Uh[src] : 0.f;
                    bl[i][j] = ok ? Ul[src] : 0.f;
                    hi[i][j] = 0.f;
                    lo[i][j] = 0.f;
                }
            }
        },
        [&](const float *buf, int kc, int kn) {
            const float *a0 = V + (size_t)rg * ldz + kc, *a1 = V + (size_t)(rg + 16) * ldz + kc;
            for (int kk = 0; kk < kn; kk += 4) {
                const float4 x0 = *reinterpret_cast<const float4 *>(a0 + kk);
                const float4 x1 = *reinterpret_cast<const float4 *>(a1 + kk);
                const float v[2][4] = {{x0.x, x0.y, x0.z, x0.w}, {x1.x, x1.y, x1.z, x1.w}};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 uh4 = *reinterpret_cast<const float4 *>(buf + (kk + q) * kCB + 4 * cg);
                    const float4 ul4 = *reinterpret_cast<const float4 *>(buf + kPlane + (kk + q) * kCB + 4 * cg);
                    const float uh[4] = {uh4.x, uh4.y, uh4.z, uh4.w}, ul[4] = {ul4.x, ul4.y, ul4.z, ul4.w};
#pragma unroll
                    for (int i = 0; i < 2; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const float t = fmaf(v[i][q], uh[j], sg[i]);
                            const float qq = t - sg[i];
                            hi[i][j] += qq;
                            lo[i][j] += fmaf(v[i][q], uh[j], -qq);
                            lo[i][j] = fmaf(v[i][q], ul[j], lo[i][j]);
                        }
                }
            }
        },
        [&](int cb) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = rg + 16 * i;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = cb + 4 * cg + j;
                    if (c < n) R[(size_t)r * ldz + c] = r < rows ? ((bh[i][j] - hi[i][j]) - lo[i][j]) + bl[i][j] : 0.f;
                }
            }
        });
}

// Steps 1 and 2 of the tiled refresh for (walker w, spin), shared with the
// refresh whose residual runs on the tensor cores: the sites holding both
// spins' labels (site_of, site_oth), tilde_U's FP32 LU in A (blocked in HBM,
// rows never moved: row i of the factors is A[perm[i]]), srow[i] =
// site_of[perm[i]], log|det tilde_U| and log(min|pivot| / max|pivot|) into
// b.logdet, and (with_inverse) G = M^{-1} (n x n, row-major) at A + n*n,
// built in the tile Z with St as its block-column buffer.  Returns false,
// with kStatusRefine set on the walker, for an incomplete configuration or
// an exactly zero pivot (every thread sees the same answer).
__device__ bool tile_factor(const DevModel &m, const DevBatch &b, int w, int spin, float *A, float *Z, float *Pn,
                            float *Ut, float *St, float *invd, int *perm, int *srow, short *site_of,
                            short *site_oth, double *red, bool with_inverse = true) {
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int n_oth = N - n;
    const float *Uh = spin == 0 ? m.U32_up_hi : m.U32_dn_hi;
    const short *kown = (spin == 0 ? b.kappa_up : b.kappa_dn) + (size_t)w * N;
    const short *koth = (spin == 0 ? b.kappa_dn : b.kappa_up) + (size_t)w * N;
    __shared__ int s_bad;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x, nw = nt / 32;

    // the sites holding each label of both spins
    for (int i = tid; i < n; i += nt) site_of[i] = -1;
    for (int i = tid; i < n_oth; i += nt) site_oth[i] = -1;
    if (tid == 0) s_bad = 0;
    __syncthreads();
    for (int s = tid; s < N; s += nt) {
        const int lw = kown[s], lt = koth[s];
        if (lw >= 1 && lw <= n) site_of[lw - 1] = (short)s;
        else if (lt >= 1 && lt <= n_oth) site_oth[lt - 1] = (short)s;
    }
    __syncthreads();
    for (int i = tid; i < n; i += nt)
        if (site_of[i] < 0) s_bad = 1;
    for (int i = tid; i < n_oth; i += nt)
        if (site_oth[i] < 0) s_bad = 1;
    __syncthreads();
    if (s_bad) {  // not a complete configuration: the FP64 refresh decides
        if (tid == 0) atomicOr(&b.status[w], kStatusRefine);
        return false;
    }
    // tilde_U (high parts): row l = U at the site holding label l + 1
    for (int l = warp; l < n; l += nw) {
        const float *src = Uh + (size_t)site_of[l] * n;
        float *dst = A + (size_t)l * n;
        for (int c = lane; c < n; c += 32) dst[c] = src[c];
    }
    __syncthreads();
    if (!lu_blocked(A, n, Pn, Ut, invd, perm)) {
        if (tid == 0) atomicOr(&b.status[w], kStatusRefine);  // an exactly zero FP32 pivot
        return false;
    }
    for (int i = tid; i < n; i += nt) srow[i] = site_of[perm[i]];
    {
        // log|det tilde_U| and log(min|pivot| / max|pivot|) from the FP32 factors
        double ldet = 0.0, dmin = INFINITY, dmaxp = 0.0;
        for (int i = tid; i < n; i += nt) {
            const float d = fabsf(A[(size_t)perm[i] * n + i]);
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
    if (!with_inverse) return true;
    const int ldz = ld_tile(n);
    // G = M^{-1}, 32 identity rows at a time (pad columns n .. ldz stay zero)
    float *G = A + (size_t)n * n;
    for (int t0 = 0; t0 < n; t0 += kRT) {
        const int rows = min(kRT, n - t0);
        __syncthreads();
        for (int e = tid; e < kRT * ldz; e += nt) {
            const int r = e / ldz, c = e - r * ldz;
            Z[e] = (r < rows && c == t0 + r) ? 1.f : 0.f;
        }
        tile_solve(A, perm, n, invd, Z, ldz, rows, St, t0);
        for (int r = warp; r < rows; r += nw)
            for (int c = lane; c < n; c += 32) G[(size_t)(t0 + r) * n + c] = Z[(size_t)r * ldz + c];
    }
    return true;
}

}  // namespace

}  // namespace kvmc
