// The periodic refresh of the mixed real form with the GEMM-shaped work of
// its iterative refinement on the tensor cores (kvmc.h: KVMC_TUNE_REFRESH32 = 3).
//
// Reference counterpart: reevaluateW! with tilde_U (KagomeDSL.jl
// src/MonteCarlo.jl:55-115): W = U tilde_U^{-1}.  The algorithm is the tiled
// FP32 refinement of kvmc_refresh_tile.cu -- X tilde_U = B for the n_oth rows
// at the other spin's sites, V = B G with G = M^{-1} (M = P tilde_U), then
// passes of V += (B - V M) G -- split into batched kernels over every walker
// and spin at once, with both products per pass as tensor-core GEMMs:
//   oz_prep_kernel      one CTA per (walker, spin): site tables and the FP32
//                       LU as in the tiled refresh; the pivot order and the
//                       site tables to HBM; unit rows of W.
//   oz_inverse_kernel   G = M^{-1}, one CTA per 32 identity rows; G^T as
//                       three bf16 planes.
//   oz_gather_kernel    the digit planes of M^T for this configuration.
//   oz_bplanes_kernel   the first pass's R = B as three bf16 planes.
//   oz_corr_kernel      V += R G (the first pass: V = B G), tcgen05 + TMA.
//   oz_check_kernel     per 32-row tile: the convergence test of the tiled
//                       refresh, and the tile's rows out to W once it has
//                       converged or the passes are spent; the tiles still
//                       refining make the next pass's work lists.
//   then per pass (at most kOzPasses = 24; a pass works only on the tiles
//   still refining, so a slowly contracting tile gets more passes than the
//   tiled refresh's 4 before its walker is handed to the FP64 refresh):
//   oz_slice_kernel     V's rows split into four digit planes.
//   oz_residual_kernel  R = B - V M from the digit planes (tcgen05 + TMA),
//                       written as R's three bf16 planes.
//   oz_corr_kernel, oz_check_kernel as above.
//
// Error-free products (the splitting of Ozaki, Ogita, Oishi and Rump,
// "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer.
// Algorithms 59, 2012).  Every column j of U gets a scale 2^f_j above its
// largest entry over all sites, every row i of V a scale 2^e_i above its
// largest entry; the scaled values are written as signed digits d_0, d_1,
// ... with |d| <= 64 and weights 2^-6, 2^-13, 2^-20, ... (round to nearest
// at each step, so every digit fits 7 bits and is exact in bf16): seven
// digits for U (48 bits below its column's scale), four for V (27 bits).
// A digit product is an integer of at most 2^12; the digit pairs (s, t)
// with the same s + t = c share one FP32 accumulator in tensor memory
// (weight 2^-7c), at most four pairs per class, so a sum over k < n stays
// below 2^24 for n < 1024 and the accumulation is exact.  Pairs with
// s + t > 6 weigh at most 2^-49 of class 0 per product and are left out.
// The classes are combined by TwoSum in FP32, scaled by 2^(e_i + f_j - 12)
// and subtracted from B (U's FP32 high and low parts): R to the accuracy of
// the tiled refresh's fixed-grid residual, with 22 bf16 MMAs per k-step of
// 16 in place of six FP32 operations per product.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "kvmc_tile.cuh"

namespace kvmc {

namespace {

namespace oz {

constexpr int kBM = 128;  // rows of V per residual tile (TMEM lanes)
constexpr int kBN = 64;   // columns of R per residual tile (TMEM columns per class)
constexpr int kKS = 32;   // k per pipeline stage: two MMA k-steps of 16
constexpr int kStages = 3;
constexpr int kClasses = 7;  // weight classes c = s + t, 0..6
constexpr int kABytes = kOzVDigits * kBM * kKS * 2;   // V's planes of one stage
constexpr int kBBytes = kOzUDigits * kBN * kKS * 2;   // M^T's planes of one stage
constexpr int kStageBytes = kABytes + kBBytes;
constexpr int kSmem = kStages * kStageBytes + 1024;   // + alignment slack
constexpr uint32_t kTmemCols = 512;                   // kClasses * kBN = 448, rounded to a power of two
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kOzPasses = 24;
// Operand tiles in shared memory: plane p, k-group g (8 k), row r at byte
// ((p * (kKS / 8) + g) * rows + r) * 16: every 8 rows x 16 bytes is one
// core matrix of the no-swizzle K-major layout, adjacent along the rows 128
// bytes apart (stride offset), adjacent along k rows * 16 bytes apart
// (leading offset).  The TMA boxes below land in exactly this order.
constexpr uint32_t kLboA = kBM * 16, kLboB = kBN * 16, kSbo = 128;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version; no swizzle, base offset 0
    return d;
}

// kind::f16 with bf16 A and B (both K-major), FP32 accumulator, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bounded wait for the completion of the barrier's phase with this parity
__device__ __forceinline__ bool wait(uint64_t *bar, uint32_t parity) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < kWaitLimit && !done; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return done != 0;
}

// 5-d tiled TMA load into shared memory, completing on `bar`
__device__ __forceinline__ void tma_load5(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4,
                                          uint64_t *bar) {
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
                 :: "r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
                    "r"(c4), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 2^e as a float for the exponents the scales take; ldexpf outside the normal range
__device__ __forceinline__ float pow2(int e) {
    return (e >= -126 && e <= 127) ? __int_as_float((e + 127) << 23) : ldexpf(1.f, e);
}

// x = x0 + x1 + x2 with every part a bf16 (rounded to nearest in turn; each
// difference is exact in FP32, and three parts hold all 24 bits)
__device__ __forceinline__ void split3(float x, uint32_t &h0, uint32_t &h1, uint32_t &h2) {
    const __nv_bfloat16 a = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(a);
    const __nv_bfloat16 c = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(c);
    const __nv_bfloat16 e = __float2bfloat16_rn(r2);
    h0 = __bfloat16_as_ushort(a);
    h1 = __bfloat16_as_ushort(c);
    h2 = __bfloat16_as_ushort(e);
}

__device__ __forceinline__ uint4 pack8(const uint32_t (&h)[8]) {
    uint4 pk;
    pk.x = h[0] | (h[1] << 16);
    pk.y = h[2] | (h[3] << 16);
    pk.z = h[4] | (h[5] << 16);
    pk.w = h[6] | (h[7] << 16);
    return pk;
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

}  // namespace oz

// Device view of the per-walker buffers (kvmc_internal.h: OzRefresh).
struct OzView {
    int n_max, oth_max, ldz, kp, rows_v, rows_m, tiles, n_ws, groups;
    int *tile_list, *grp_list, *counts, *grp_flag;
    const uint16_t *ud0, *ud1;
    const int *fexp0, *fexp1;
    float *V;
    uint16_t *vd, *mt, *rd, *gd;
    int cn, rows_g;
    float *dmax, *vmax;
    int *vexp, *perm, *srow;
    float *invd;
    short *site_oth;
    float *dprev;
    int *done, *active;
};

OzView view_of(const OzRefresh &o) {
    OzView v;
    v.n_max = o.n_max; v.oth_max = o.oth_max; v.ldz = o.ldz; v.kp = o.kp;
    v.rows_v = o.rows_v; v.rows_m = o.rows_m; v.tiles = o.tiles; v.n_ws = o.n_ws; v.groups = o.groups;
    v.tile_list = o.tile_list; v.grp_list = o.grp_list; v.counts = o.counts; v.grp_flag = o.grp_flag;
    v.ud0 = o.ud[0]; v.ud1 = o.ud[1]; v.fexp0 = o.fexp[0]; v.fexp1 = o.fexp[1];
    v.V = o.V; v.rd = o.rd; v.gd = o.gd; v.cn = o.cn; v.rows_g = o.rows_g; v.dmax = o.dmax; v.vmax = o.vmax;
    v.vd = o.vd; v.mt = o.mt; v.vexp = o.vexp; v.perm = o.perm; v.srow = o.srow; v.invd = o.invd;
    v.site_oth = o.site_oth; v.dprev = o.dprev; v.done = o.done; v.active = o.active;
    return v;
}

// Shared memory of the LU step: the 32-column panel, the staged block of
// U12, the pivot order and the site tables (70 KB at n = 432, so that three
// CTAs share an SM; the launch bound keeps their registers to a third of
// the SM's too).
struct PrepSmem {
    size_t pn, ut, invd, perm, srow, site_of, site_oth, total;
};
__host__ __device__ inline PrepSmem prep_layout(int n, int n_oth) {
    auto al = [](size_t x) { return (x + 15) / 16 * 16; };
    PrepSmem s{};
    s.pn = 0;
    s.ut = al((size_t)n * kLdc * 4);
    s.invd = s.ut + (size_t)kPB * 64 * 4;
    s.perm = al(s.invd + (size_t)n * 4);
    s.srow = al(s.perm + (size_t)n * 4);
    s.site_of = al(s.srow + (size_t)n * 4);
    s.site_oth = al(s.site_of + (size_t)n * 2);
    s.total = al(s.site_oth + (size_t)n_oth * 2);
    return s;
}

// Step 1 of the tiled refresh (site tables, LU of tilde_U in HBM), its
// results to HBM for the batched kernels, and the unit rows of W.
__global__ void __launch_bounds__(kTT, 3) oz_prep_kernel(DevModel m, DevBatch b, OzView v, int only_due, int track_drift) {
    const int w = blockIdx.x, spin = blockIdx.y, ws = 2 * w + spin;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x, nw = nt / 32;
    if (only_due && b.since[w] >= 0) {
        if (tid == 0) v.active[ws] = 0;
        return;
    }
    if (spin == 0 && tid == 0) atomicAdd(b.refresh_count, 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int n_oth = N - n;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const bool cpt = b.compact != 0;
    float *Wout = cpt ? b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up)
                      : b.W32 + (size_t)w * N * (m.ld_up + m.ld_dn) + (spin == 0 ? 0 : (size_t)N * m.ld_up);
    float *A = reinterpret_cast<float *>(b.solve_scratch + ((size_t)w * 2 + spin) * b.solve_block);

    extern __shared__ __align__(16) unsigned char smem[];
    const PrepSmem L = prep_layout(n, n_oth);
    float *Pn = reinterpret_cast<float *>(smem + L.pn);
    float *Ut = reinterpret_cast<float *>(smem + L.ut);
    float *invd = reinterpret_cast<float *>(smem + L.invd);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    int *srow = reinterpret_cast<int *>(smem + L.srow);
    short *site_of = reinterpret_cast<short *>(smem + L.site_of);
    short *site_oth = reinterpret_cast<short *>(smem + L.site_oth);
    __shared__ double red[33];

    if (!tile_factor(m, b, w, spin, A, nullptr, Pn, Ut, nullptr, invd, perm, srow, site_of, site_oth, red, false)) {
        if (tid == 0) v.active[ws] = 0;
        return;
    }
    for (int i = tid; i < n; i += nt) {
        v.invd[(size_t)ws * v.n_max + i] = invd[i];
        v.perm[(size_t)ws * v.n_max + i] = perm[i];
        v.srow[(size_t)ws * v.n_max + i] = srow[i];
    }
    for (int i = tid; i < n_oth; i += nt) v.site_oth[(size_t)ws * v.oth_max + i] = site_oth[i];
    for (int g = tid; g < v.groups; g += nt) v.grp_flag[(size_t)ws * v.groups + g] = 0;
    for (int r = tid; r < v.rows_v; r += nt) {
        v.dmax[(size_t)ws * v.rows_v + r] = 0.f;
        v.vmax[(size_t)ws * v.rows_v + r] = 0.f;
    }
    for (int t = tid; t < v.tiles; t += nt) {
        v.dprev[(size_t)ws * v.tiles + t] = 1.f;
        v.done[(size_t)ws * v.tiles + t] = t * kRT < n_oth ? 0 : 1;
    }
    // unit rows at the sites holding this spin (site-indexed W only)
    float dmax = 0.f;
    if (!cpt) {
        for (int l = warp; l < n; l += nw) {
            float *wr = Wout + (size_t)site_of[l] * ldw;
            for (int c = lane; c < ldw; c += 32) {
                const float nv = c == l ? 1.f : 0.f;
                if (track_drift) dmax = fmaxf(dmax, fabsf(wr[c] - nv) / (1.f + fabsf(nv)));
                wr[c] = nv;
            }
        }
    }
    if (track_drift) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
    }
    if (tid == 0) v.active[ws] = 1;
}

// G = M^{-1} (row-major n x n after the LU in the walker-spin's scratch),
// rows t0 .. t0 + 31 from the identity rows, as in the tiled refresh.
// Shared memory of the inverse: the tile of identity rows and the staged
// block column of the factors (112 KB at n = 432: two CTAs per SM); the
// pivot order and 1 / diag(Uf) are read from HBM.
struct InverseSmem {
    size_t z, st, perm, total;
};
__host__ __device__ inline InverseSmem inverse_layout(int n) {
    auto al = [](size_t x) { return (x + 15) / 16 * 16; };
    InverseSmem s{};
    s.z = 0;
    s.st = al((size_t)kRT * ld_tile(n) * 4);
    s.perm = s.st + al((size_t)round4(n) * kLdc * 4);
    s.total = s.perm + al((size_t)n * 4);
    return s;
}

// One CTA per (walker-spin, 32 identity rows), the tiles of a walker-spin
// adjacent in the one-dimensional grid (x = tile + tiles * (2 w + spin)), so
// that the CTAs reading one walker-spin's factors run together and share
// them in L2 (512 walkers at 432 orbitals hold 764 MB of factors).
__global__ void __launch_bounds__(kTT) oz_inverse_kernel(DevModel m, DevBatch b, OzView v) {
    const int tiles = (v.n_max + kRT - 1) / kRT;
    const int ws = blockIdx.x / tiles, w = ws >> 1, spin = ws & 1;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int t0 = (blockIdx.x - ws * tiles) * kRT;
    if (!v.active[ws] || t0 >= n) return;
    const int rows = min(kRT, n - t0), ldz = ld_tile(n);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x, nw = nt / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    const InverseSmem L = inverse_layout(n);
    float *Z = reinterpret_cast<float *>(smem + L.z);
    float *St = reinterpret_cast<float *>(smem + L.st);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    const float *invd = v.invd + (size_t)ws * v.n_max;
    float *A = reinterpret_cast<float *>(b.solve_scratch + ((size_t)w * 2 + spin) * b.solve_block);
    for (int i = tid; i < n; i += nt) perm[i] = v.perm[(size_t)ws * v.n_max + i];
    for (int e = tid; e < kRT * ldz; e += nt) {
        const int r = e / ldz, c = e - r * ldz;
        Z[e] = (r < rows && c == t0 + r) ? 1.f : 0.f;
    }
    __syncthreads();
    tile_solve(A, perm, n, invd, Z, ldz, rows, St, t0);
    // G^T's three bf16 planes for the correction GEMM: plane p, k-group g,
    // row j holds part p of G[8 g + q][j], q = 0..7 (k = G's row)
    const size_t gplane = (size_t)(v.kp / 8) * v.rows_g * 8;
    uint16_t *gdst = v.gd + (size_t)ws * 3 * gplane;
    const int ng = (rows + 7) / 8;
    for (int e = tid; e < ng * n; e += nt) {
        const int gl = e / n, j = e - gl * n;
        uint32_t h[3][8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int r = 8 * gl + q;
            oz::split3(r < rows ? Z[(size_t)r * ldz + j] : 0.f, h[0][q], h[1][q], h[2][q]);
        }
        const size_t at = ((size_t)(t0 / 8 + gl) * v.rows_g + j) * 8;
#pragma unroll
        for (int p = 0; p < 3; ++p) *reinterpret_cast<uint4 *>(gdst + p * gplane + at) = oz::pack8(h[p]);
    }
    (void)warp; (void)lane; (void)nw;
}

// The first pass's R = B (U's high parts at the other spin's sites) as the
// three bf16 planes the correction GEMM reads: one CTA per 32-row tile.
__global__ void __launch_bounds__(256) oz_bplanes_kernel(DevModel m, OzView v) {
    const int w = blockIdx.x, spin = blockIdx.y, tt = blockIdx.z, ws = 2 * w + spin;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int n_oth = m.n_sites - n;
    const int b0 = tt * kRT;
    if (!v.active[ws] || b0 >= n_oth) return;
    const int rows = min(kRT, n_oth - b0);
    const float *Uh = spin == 0 ? m.U32_up_hi : m.U32_dn_hi;
    const short *so = v.site_oth + (size_t)ws * v.oth_max + b0;
    const size_t rplane = (size_t)(v.kp / 8) * v.rows_v * 8;
    uint16_t *dst = v.rd + (size_t)ws * 3 * rplane;
    const int groups = (n + 7) / 8;
    for (int e = threadIdx.x; e < groups * kRT; e += blockDim.x) {
        const int r = e & (kRT - 1), g = e / kRT;
        if (r >= rows) continue;
        const float *src = Uh + (size_t)so[r] * n;
        uint32_t h[3][8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = 8 * g + q;
            oz::split3(k < n ? src[k] : 0.f, h[0][q], h[1][q], h[2][q]);
        }
        const size_t at = ((size_t)g * v.rows_v + b0 + r) * 8;
#pragma unroll
        for (int p = 0; p < 3; ++p) *reinterpret_cast<uint4 *>(dst + p * rplane + at) = oz::pack8(h[p]);
    }
}

// M^T's digit planes: plane t, k-group g, row j holds digit t of
// U[srow[8 g + q]][j] for q = 0..7 (zero beyond n, where nothing writes).
__global__ void __launch_bounds__(256) oz_gather_kernel(DevModel m, OzView v) {
    const int w = blockIdx.x, spin = blockIdx.y, t = blockIdx.z, ws = 2 * w + spin;
    if (!v.active[ws]) return;
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    __shared__ int srow[1024];
    for (int i = threadIdx.x; i < n; i += blockDim.x) srow[i] = v.srow[(size_t)ws * v.n_max + i];
    __syncthreads();
    const uint16_t *ud = (spin == 0 ? v.ud0 : v.ud1) + (size_t)t * N * n;
    uint16_t *dst = v.mt + ((size_t)ws * kOzUDigits + t) * (size_t)(v.kp / 8) * v.rows_m * 8;
    const int groups = (n + 7) / 8;
    for (int e = threadIdx.x; e < groups * n; e += blockDim.x) {
        const int g = e / n, j = e - g * n;
        uint16_t d[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = 8 * g + q;
            d[q] = k < n ? ud[(size_t)srow[k] * n + j] : (uint16_t)0;
        }
        uint4 pk;
        pk.x = d[0] | ((uint32_t)d[1] << 16);
        pk.y = d[2] | ((uint32_t)d[3] << 16);
        pk.z = d[4] | ((uint32_t)d[5] << 16);
        pk.w = d[6] | ((uint32_t)d[7] << 16);
        *reinterpret_cast<uint4 *>(dst + ((size_t)g * v.rows_m + j) * 8) = pk;
    }
}

// V's digit planes for the 32-row tiles of the pass's list: row i is scaled
// by 2^-e_i (2^e_i above its largest entry), then split into kOzVDigits
// digits.  One CTA per listed tile, in a grid-stride loop over the list.
__global__ void __launch_bounds__(256) oz_slice_kernel(DevModel m, OzView v, int cur) {
    const int count = v.counts[2 * cur];
    const int *list = v.tile_list + (size_t)cur * v.n_ws * v.tiles;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ int s_e[kRT];
    for (int it = blockIdx.x; it < count; it += gridDim.x) {
        const int item = list[it], ws = item / v.tiles, tt = item - ws * v.tiles, spin = ws & 1;
        const int n = spin == 0 ? m.n_up : m.n_dn;
        const int n_oth = m.n_sites - n;
        const int b0 = tt * kRT;
        const int rows = min(kRT, n_oth - b0);
        const float *Vw = v.V + ((size_t)ws * v.rows_v + b0) * v.ldz;
        for (int r = warp; r < kRT; r += 8) {
            float mx = 0.f;
            if (r < rows)
                for (int c = lane; c < n; c += 32) mx = fmaxf(mx, fabsf(Vw[(size_t)r * v.ldz + c]));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) {
                int e = 0;
                if (mx > 0.f && mx < INFINITY) frexpf(mx, &e);   // mx < 2^e
                s_e[r] = e;
                if (r < rows) v.vexp[(size_t)ws * v.rows_v + b0 + r] = e;
            }
        }
        __syncthreads();
        const int groups = (n + 7) / 8;
        const size_t plane = (size_t)(v.kp / 8) * v.rows_v * 8;
        uint16_t *dst = v.vd + (size_t)ws * kOzVDigits * plane;
        for (int e = tid; e < groups * kRT; e += blockDim.x) {
            const int r = e & (kRT - 1), g = e / kRT;
            if (r >= rows) continue;
            const float sc = oz::pow2(6 - s_e[r]);
            float y[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int k = 8 * g + q;
                y[q] = k < n ? Vw[(size_t)r * v.ldz + k] * sc : 0.f;   // |y| < 64, exact
            }
#pragma unroll
            for (int s = 0; s < kOzVDigits; ++s) {
                uint32_t h[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float d = rintf(y[q]);                   // |d| <= 64
                    h[q] = __float_as_uint(d) >> 16;               // exact in bf16
                    y[q] = (y[q] - d) * 128.f;                     // exact; |y| <= 64
                }
                uint4 pk;
                pk.x = h[0] | (h[1] << 16);
                pk.y = h[2] | (h[3] << 16);
                pk.z = h[4] | (h[5] << 16);
                pk.w = h[6] | (h[7] << 16);
                *reinterpret_cast<uint4 *>(dst + s * plane + ((size_t)g * v.rows_v + b0 + r) * 8) = pk;
            }
        }
        __syncthreads();
    }
}

// R = B - V M.  Persistent: one CTA per SM walks the units of the pass --
// (walker-spin, 128-row group, 64-column tile) for every group in the
// list -- in steps of the grid.  Warp 4's first lane loads the digit planes
// stage by stage with TMA, up to three stages ahead and across units; warp
// 5's first lane issues the 22 MMAs of each k-step into the seven class
// accumulators, and before a unit's first MMA waits until warps 0-3 have
// read the previous unit's classes out of tensor memory; warps 0-3 (TMEM
// lanes 0-127, the group's rows) combine the classes and subtract them from
// B, whose entries they fetch ahead.  Every wait is bounded; one that gives
// up stops the CTA, whose units' walkers are then marked kStatusTimeout.
constexpr int kResThreads = 192;

__global__ void __launch_bounds__(kResThreads, 1)
oz_residual_kernel(DevModel m, DevBatch b, OzView v, int cur, const __grid_constant__ CUtensorMap tmv,
                   const __grid_constant__ CUtensorMap tmm) {
    using namespace oz;
    const int ngrp = v.counts[2 * cur + 1];
    const int ctiles = v.rows_m / kBN;
    const int units = ngrp * ctiles;
    if ((int)blockIdx.x >= units) return;
    const int *glist = v.grp_list + (size_t)cur * v.n_ws * v.groups;

    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done_bar, tfree_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int s_fail;
    __shared__ int s_issued;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            bar_init(&full[s], 1);
            bar_init(&empty[s], 1);
        }
        bar_init(&done_bar, 1);
        bar_init(&tfree_bar, 4);   // one arrival per epilogue warp
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
        s_issued = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    // unit u -> (walker-spin, first row, first column, orbitals, other rows); false: nothing to do
    auto unit = [&](int u, int &item, int &ws, int &r0, int &c0, int &n, int &n_oth) {
        const int gi = u / ctiles, ct = u - gi * ctiles;
        item = glist[gi];
        ws = item / v.groups;
        r0 = (item - ws * v.groups) * kBM;
        c0 = ct * kBN;
        n = (ws & 1) == 0 ? m.n_up : m.n_dn;
        n_oth = m.n_sites - n;
        return c0 < n && r0 < n_oth;
    };

    if (warp == 4) {
        if (lane == 0) {
            int gch = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < units && !stop && !s_fail; u += gridDim.x) {
                int item, ws, r0, c0, n, n_oth;
                if (!unit(u, item, ws, r0, c0, n, n_oth)) continue;
                if (c0 == 0) v.grp_flag[item] = 0;   // the next pass's correction may list the group again
                const int nch = (n + kKS - 1) / kKS;
                for (int ch = 0; ch < nch; ++ch, ++gch) {
                    const int s = gch % kStages;
                    if (gch >= kStages && !wait(&empty[s], ((gch / kStages) - 1) & 1)) {
                        s_fail = 1;
                        stop = true;
                        break;
                    }
                    expect_tx(&full[s], kStageBytes);
                    unsigned char *st = sm + (size_t)s * kStageBytes;
                    tma_load5(st, &tmv, 0, r0, ch * (kKS / 8), 0, ws, &full[s]);
                    tma_load5(st + kABytes, &tmm, 0, c0, ch * (kKS / 8), 0, ws, &full[s]);
                }
            }
            s_issued = gch;
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(kBM, kBN);
            int gch = 0, k = 0;
            for (int u = blockIdx.x; u < units && !s_fail; u += gridDim.x) {
                int item, ws, r0, c0, n, n_oth;
                if (!unit(u, item, ws, r0, c0, n, n_oth)) continue;
                if (k > 0 && !wait(&tfree_bar, (k - 1) & 1)) {
                    s_fail = 1;
                    break;
                }
                fence_after();
                const int nch = (n + kKS - 1) / kKS;
                bool ok = true;
                for (int ch = 0; ch < nch; ++ch, ++gch) {
                    const int s = gch % kStages;
                    if (!wait(&full[s], (gch / kStages) & 1)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t a0 = smem_u32(sm + (size_t)s * kStageBytes), b0 = a0 + kABytes;
#pragma unroll
                    for (int q = 0; q < kKS / 16; ++q) {
#pragma unroll
                        for (int c = 0; c < kClasses; ++c) {
#pragma unroll
                            for (int sa = 0; sa < kOzVDigits; ++sa) {
                                const int tb = c - sa;
                                if (tb < 0 || tb >= kOzUDigits) continue;
                                const uint64_t ad = sdesc(a0 + sa * (kBM * kKS * 2) + q * 2 * kLboA, kLboA, kSbo);
                                const uint64_t bd = sdesc(b0 + tb * (kBN * kKS * 2) + q * 2 * kLboB, kLboB, kSbo);
                                mma(tmem + (uint32_t)(c * kBN), ad, bd, idesc, (ch > 0 || q > 0 || sa > 0) ? 1u : 0u);
                            }
                        }
                    }
                    commit(&empty[s]);   // the stage is free once these MMAs have read it
                }
                commit(&done_bar);       // always, so that the epilogue's wait ends
                ++k;
                if (!ok) {
                    s_fail = 1;
                    break;
                }
            }
        }
        __syncwarp();
    } else {
        // epilogue: warp g reads TMEM lanes 32 g .. 32 g + 31, rows r0 + 32 g + lane
        const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16);
        int k = 0;
        for (int u = blockIdx.x; u < units; u += gridDim.x) {
            int item, ws, r0, c0, n, n_oth;
            if (!unit(u, item, ws, r0, c0, n, n_oth)) continue;
            const int spin = ws & 1;
            const int i = r0 + 32 * warp + lane;
            const bool row_ok = i < n_oth;
            const int *fexp = spin == 0 ? v.fexp0 : v.fexp1;
            const float *Uh = spin == 0 ? m.U32_up_hi : m.U32_dn_hi;
            const float *Ul = spin == 0 ? m.U32_up_lo : m.U32_dn_lo;
            const int site = row_ok ? v.site_oth[(size_t)ws * v.oth_max + i] : 0;
            const float sc_i = row_ok ? pow2(v.vexp[(size_t)ws * v.rows_v + i] - 12) : 0.f;
            const float *bh = Uh + (size_t)site * n, *bl = Ul + (size_t)site * n;
            const size_t rplane = (size_t)(v.kp / 8) * v.rows_v * 8;
            uint16_t *rdst = v.rd + (size_t)ws * 3 * rplane + (size_t)(row_ok ? i : 0) * 8;
            float ph[8], pl[8];   // B's next eight entries, fetched ahead
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const bool ok = row_ok && c0 + q < n;
                ph[q] = ok ? bh[c0 + q] : 0.f;
                pl[q] = ok ? bl[c0 + q] : 0.f;
            }
            if (!wait(&done_bar, k & 1)) {
                s_fail = 1;
                break;
            }
            fence_after();
            const bool good = !s_fail;
            for (int cc = 0; cc < kBN; cc += 8) {
                float d[kClasses][8];
#pragma unroll
                for (int c = 0; c < kClasses; ++c) ld8(tl + (uint32_t)(c * kBN + cc), d[c]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                float ch_[8], cl_[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    ch_[q] = ph[q];
                    cl_[q] = pl[q];
                }
                if (cc + 8 < kBN) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int j = c0 + cc + 8 + q;
                        const bool ok = row_ok && j < n;
                        ph[q] = ok ? bh[j] : 0.f;
                        pl[q] = ok ? bl[j] : 0.f;
                    }
                }
                if (!(row_ok && good) || c0 + cc >= n) continue;
                // R's entries c0 + cc .. + 7 (zero from n on) as the correction's k-group (c0 + cc) / 8
                uint32_t h[3][8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int j = c0 + cc + q;
                    float r = 0.f;
                    if (j < n) {
                        float h1, e1, h2, e2;
                        two_sum(d[0][q], d[1][q] * 0x1p-7f, h1, e1);
                        two_sum(h1, d[2][q] * 0x1p-14f, h2, e2);
                        const float t = fmaf(d[6][q], 0x1p-42f,
                                             fmaf(d[5][q], 0x1p-35f, fmaf(d[4][q], 0x1p-28f, d[3][q] * 0x1p-21f)));
                        const float lo = (e1 + e2) + t;
                        const float s = sc_i * pow2(fexp[j]);
                        r = ((ch_[q] - h2 * s) - lo * s) + cl_[q];
                    }
                    split3(r, h[0][q], h[1][q], h[2][q]);
                }
                const size_t at = (size_t)((c0 + cc) / 8) * v.rows_v * 8;
#pragma unroll
                for (int p = 0; p < 3; ++p) *reinterpret_cast<uint4 *>(rdst + p * rplane + at) = pack8(h[p]);
            }
            fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(&tfree_bar)) : "memory");
            ++k;
        }
    }

    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
        // copies still in flight after a wait gave up: wait for them, bounded
        const int issued = s_issued;
        for (int s = 0; s < kStages && s < issued; ++s) {
            const int last = s + ((issued - 1 - s) / kStages) * kStages;
            wait(&full[s], (last / kStages) & 1);
        }
        if (s_fail)
            for (int u = blockIdx.x; u < units; u += gridDim.x) {
                int item, ws, r0, c0, n, n_oth;
                unit(u, item, ws, r0, c0, n, n_oth);
                atomicOr(&b.status[ws >> 1], kStatusTimeout);
            }
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTmemCols));
}


// V += R G on the tensor cores.  R and G^T are three bf16 planes each
// (x = x0 + x1 + x2 exactly); the six products with a + b <= 2 accumulate in
// one FP32 accumulator, the three left out weigh 2^-24 of the product or
// less, so the correction has FP32 accuracy, which the refinement needs (its
// contraction factor grows by the correction's relative error times
// cond(tilde_U)).  Persistent like the residual: units (walker-spin, 128-row
// group, cn-column tile) of the pass's group list -- every group on the
// first pass -- with the accumulator double-buffered in tensor memory, so the
// MMAs of one unit run while warps 0-3 add the previous one into V and keep
// each row's largest |R G| and |V| for the convergence test.
constexpr int kCorrStages = 3;
constexpr int kCorrABytes = 3 * oz::kBM * oz::kKS * 2;
__host__ __device__ inline int corr_stage_bytes(int cn) { return kCorrABytes + 3 * cn * oz::kKS * 2; }
__host__ __device__ inline int corr_smem(int cn) { return kCorrStages * corr_stage_bytes(cn) + 1024; }

__global__ void __launch_bounds__(kResThreads, 1)
oz_corr_kernel(DevModel m, DevBatch b, OzView v, int first, int cur, const __grid_constant__ CUtensorMap tmr,
               const __grid_constant__ CUtensorMap tmg) {
    using namespace oz;
    const int cn = v.cn;
    const int ctiles = v.rows_g / cn;
    const int ngrp = first ? v.n_ws * v.groups : v.counts[2 * cur + 1];
    const int units = ngrp * ctiles;
    if ((int)blockIdx.x >= units) return;
    const int *glist = v.grp_list + (size_t)cur * v.n_ws * v.groups;
    const int stage_bytes = corr_stage_bytes(cn);
    const uint32_t lbo_b = (uint32_t)cn * 16;

    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[kCorrStages], empty[kCorrStages], done_bar[2], tfree_bar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int s_fail;
    __shared__ int s_issued;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < kCorrStages; ++s) {
            bar_init(&full[s], 1);
            bar_init(&empty[s], 1);
        }
        for (int q = 0; q < 2; ++q) {
            bar_init(&done_bar[q], 1);
            bar_init(&tfree_bar[q], 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
        s_issued = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    auto unit = [&](int u, int &ws, int &r0, int &c0, int &n, int &n_oth) {
        const int gi = u / ctiles, ct = u - gi * ctiles;
        const int item = first ? gi : glist[gi];
        ws = item / v.groups;
        r0 = (item - ws * v.groups) * kBM;
        c0 = ct * cn;
        n = (ws & 1) == 0 ? m.n_up : m.n_dn;
        n_oth = m.n_sites - n;
        return (!first || v.active[ws]) && c0 < n && r0 < n_oth;
    };

    if (warp == 4) {
        if (lane == 0) {
            int gch = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < units && !stop && !s_fail; u += gridDim.x) {
                int ws, r0, c0, n, n_oth;
                if (!unit(u, ws, r0, c0, n, n_oth)) continue;
                const int nch = (n + kKS - 1) / kKS;
                for (int ch = 0; ch < nch; ++ch, ++gch) {
                    const int s = gch % kCorrStages;
                    if (gch >= kCorrStages && !wait(&empty[s], ((gch / kCorrStages) - 1) & 1)) {
                        s_fail = 1;
                        stop = true;
                        break;
                    }
                    expect_tx(&full[s], (uint32_t)stage_bytes);
                    unsigned char *st = sm + (size_t)s * stage_bytes;
                    tma_load5(st, &tmr, 0, r0, ch * (kKS / 8), 0, ws, &full[s]);
                    tma_load5(st + kCorrABytes, &tmg, 0, c0, ch * (kKS / 8), 0, ws, &full[s]);
                }
            }
            s_issued = gch;
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(kBM, cn);
            int gch = 0, k = 0;
            for (int u = blockIdx.x; u < units && !s_fail; u += gridDim.x) {
                int ws, r0, c0, n, n_oth;
                if (!unit(u, ws, r0, c0, n, n_oth)) continue;
                const int bf = k & 1, use = k >> 1;
                if (use > 0 && !wait(&tfree_bar[bf], (use - 1) & 1)) {
                    s_fail = 1;
                    break;
                }
                fence_after();
                const uint32_t acc_addr = tmem + (uint32_t)(bf * 256);
                const int nch = (n + kKS - 1) / kKS;
                bool ok = true;
                for (int ch = 0; ch < nch; ++ch, ++gch) {
                    const int s = gch % kCorrStages;
                    if (!wait(&full[s], (gch / kCorrStages) & 1)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t a0 = smem_u32(sm + (size_t)s * stage_bytes), b0 = a0 + kCorrABytes;
#pragma unroll
                    for (int q = 0; q < kKS / 16; ++q) {
#pragma unroll
                        for (int pr = 0; pr < 6; ++pr) {
                            const int pa = pr < 3 ? (pr == 2 ? 1 : 0) : (pr == 5 ? 2 : pr == 4 ? 1 : 0);
                            const int pb = pr < 3 ? (pr == 1 ? 1 : 0) : (pr == 3 ? 2 : pr == 4 ? 1 : 0);
                            const uint64_t ad = sdesc(a0 + pa * (kBM * kKS * 2) + q * 2 * kLboA, kLboA, kSbo);
                            const uint64_t bd = sdesc(b0 + pb * (cn * kKS * 2) + q * 2 * lbo_b, lbo_b, kSbo);
                            mma(acc_addr, ad, bd, idesc, (ch > 0 || q > 0 || pr > 0) ? 1u : 0u);
                        }
                    }
                    commit(&empty[s]);
                }
                commit(&done_bar[bf]);
                ++k;
                if (!ok) {
                    s_fail = 1;
                    break;
                }
            }
        }
        __syncwarp();
    } else {
        int k = 0;
        for (int u = blockIdx.x; u < units; u += gridDim.x) {
            int ws, r0, c0, n, n_oth;
            if (!unit(u, ws, r0, c0, n, n_oth)) continue;
            const int bf = k & 1, use = k >> 1;
            const int i = r0 + 32 * warp + lane;
            const bool row_ok = i < n_oth && !v.done[(size_t)ws * v.tiles + i / kRT];
            float *Vrow = v.V + ((size_t)ws * v.rows_v + (row_ok ? i : 0)) * v.ldz;
            if (!wait(&done_bar[bf], use & 1)) {
                s_fail = 1;
                break;
            }
            fence_after();
            const bool good = row_ok && !s_fail;
            const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(bf * 256);
            float dm = 0.f, vm = 0.f;
            for (int cc = 0; cc < cn; cc += 16) {
                float d0[8], d1[8];
                ld8(tl + (uint32_t)cc, d0);
                ld8(tl + (uint32_t)(cc + 8), d1);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (!good) continue;
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int j = c0 + cc + q;
                    if (j >= n) break;
                    const float dv = q < 8 ? d0[q] : d1[q - 8];
                    const float nv = (first ? 0.f : Vrow[j]) + dv;
                    Vrow[j] = nv;
                    dm = fmaxf(dm, isfinite(nv) ? fabsf(dv) : INFINITY);
                    vm = fmaxf(vm, fabsf(nv));
                }
            }
            if (good) {
                atomic_max_nonneg(&v.dmax[(size_t)ws * v.rows_v + i], dm);
                atomic_max_nonneg(&v.vmax[(size_t)ws * v.rows_v + i], vm);
            }
            fence_before();
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(&tfree_bar[bf])) : "memory");
            ++k;
        }
    }

    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
        const int issued = s_issued;
        for (int s = 0; s < kCorrStages && s < issued; ++s) {
            const int last = s + ((issued - 1 - s) / kCorrStages) * kCorrStages;
            wait(&full[s], (last / kCorrStages) & 1);
        }
        if (s_fail)
            for (int u = blockIdx.x; u < units; u += gridDim.x) {
                int ws, r0, c0, n, n_oth;
                unit(u, ws, r0, c0, n, n_oth);
                atomicOr(&b.status[ws >> 1], kStatusTimeout);
            }
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTmemCols));
}

// The convergence test of one 32-row tile after a correction (as in the
// tiled refresh: d = the largest |R G| relative to its row's largest |V|,
// est = d^2 / d_prev), and its rows out to W when it has converged or the
// passes are spent; a tile still refining goes on the next pass's list
// (nxt), and its 128-row group on the next group list unless it is there
// already.  The first pass's d is 1, so it ends no tile.
__device__ __forceinline__ void check_tile(const DevModel &m, const DevBatch &b, const OzView &v, int item, int first,
                                           int last, int nxt, int track_drift, int *s_fin) {
    const int ws = item / v.tiles, tt = item - ws * v.tiles, w = ws >> 1, spin = ws & 1;
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int n_oth = N - n;
    const int b0 = tt * kRT;
    if (!v.active[ws] || b0 >= n_oth || v.done[item]) return;
    const int rows = min(kRT, n_oth - b0);
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x / 32;
    if (warp == 0) {
        float q = 0.f;
        if (lane < rows) {
            const size_t r = (size_t)ws * v.rows_v + b0 + lane;
            const float qi = v.dmax[r] / fmaxf(v.vmax[r], 1e-30f);
            q = isnan(qi) ? INFINITY : qi;
            v.dmax[r] = 0.f;
            v.vmax[r] = 0.f;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q = fmaxf(q, __shfl_xor_sync(0xffffffffu, q, o));
        if (lane == 0) {
            const float d = q, dprev = v.dprev[item];
            const float est = d < dprev ? d * d / dprev : INFINITY;   // a correction that grows: diverging
            v.dprev[item] = d;
            const int fin = !first && (!(est > 1e-6f) || last);
            *s_fin = fin;
            if (fin) {
                v.done[item] = 1;
                if (!(est <= 1e-5f)) atomicOr(&b.status[w], kStatusRefine);
            } else {
                v.tile_list[(size_t)nxt * v.n_ws * v.tiles + atomicAdd(&v.counts[2 * nxt], 1)] = item;
                const int g = ws * v.groups + b0 / oz::kBM;
                if (atomicExch(&v.grp_flag[g], 1) == 0)
                    v.grp_list[(size_t)nxt * v.n_ws * v.groups + atomicAdd(&v.counts[2 * nxt + 1], 1)] = g;
            }
        }
    }
    __syncthreads();
    if (!*s_fin) return;
    // the tile's rows out, in label order: X[:, perm[i]] = V[:, i]
    const bool cpt = b.compact != 0;
    float *Wout = cpt ? b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up)
                      : b.W32 + (size_t)w * N * (m.ld_up + m.ld_dn) + (spin == 0 ? 0 : (size_t)N * m.ld_up);
    const int *perm = v.perm + (size_t)ws * v.n_max;
    const short *site_oth = v.site_oth + (size_t)ws * v.oth_max;
    const float *Vw = v.V + ((size_t)ws * v.rows_v + b0) * v.ldz;
    float dmax = 0.f;
    for (int r = warp; r < rows; r += nw) {
        float *wr = Wout + (size_t)(cpt ? b0 + r : site_oth[b0 + r]) * ldw;
        for (int i = lane; i < n; i += 32) {
            const float nv = Vw[(size_t)r * v.ldz + i];
            const int p = perm[i];
            if (track_drift) dmax = fmaxf(dmax, fabsf(wr[p] - nv) / (1.f + fabsf(nv)));
            wr[p] = nv;
        }
        if (!cpt)
            for (int c = n + lane; c < ldw; c += 32) wr[c] = 0.f;
    }
    if (track_drift) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0 && dmax > 0.f) atomic_max_nonneg(&b.drift[w], dmax);
    }
}

// first != 0: every tile of every walker-spin; else the tiles of list `cur`;
// a grid-stride loop either way.
__global__ void __launch_bounds__(256) oz_check_kernel(DevModel m, DevBatch b, OzView v, int first, int last,
                                                       int cur, int track_drift) {
    __shared__ int s_fin;
    const int nxt = cur ^ 1;
    const int count = first ? v.n_ws * v.tiles : v.counts[2 * cur];
    const int *list = v.tile_list + (size_t)cur * v.n_ws * v.tiles;
    for (int it = blockIdx.x; it < count; it += gridDim.x) {
        check_tile(m, b, v, first ? it : list[it], first, last, nxt, track_drift, &s_fin);
        __syncthreads();
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// planes of [groups = kp/8][rows][8] bf16 per (walker-spin, plane); box =
// all planes of one stage (kKS / 8 groups) and `box_rows` rows
cudaError_t encode_planes(void *map, void *base, int rows, int kp, int planes, int ws_count, int box_rows) {
    EncodeTiled fn = encode_fn();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t dims[5] = {8, (cuuint64_t)rows, (cuuint64_t)(kp / 8), (cuuint64_t)planes, (cuuint64_t)ws_count};
    const cuuint64_t strides[4] = {16, (cuuint64_t)rows * 16, (cuuint64_t)(kp / 8) * rows * 16,
                                   (cuuint64_t)planes * (kp / 8) * rows * 16};
    const cuuint32_t box[5] = {8, (cuuint32_t)box_rows, (cuuint32_t)(oz::kKS / 8), (cuuint32_t)planes, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = fn(reinterpret_cast<CUtensorMap *>(map), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, base, dims,
                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct OzDims {
    int n_max, oth_max, ldz, kp, rows_v, rows_m, tiles, cn, rows_g;
};
OzDims oz_dims(const DevModel &m) {
    OzDims d;
    d.n_max = std::max(m.n_up, m.n_dn);
    d.oth_max = m.n_sites - std::min(m.n_up, m.n_dn);
    d.ldz = (d.n_max + 3) & ~3;
    d.kp = (d.n_max + oz::kKS - 1) / oz::kKS * oz::kKS;
    d.rows_v = (d.oth_max + oz::kBM - 1) / oz::kBM * oz::kBM;
    d.rows_m = (d.n_max + oz::kBN - 1) / oz::kBN * oz::kBN;
    d.tiles = (d.oth_max + kRT - 1) / kRT;
    // the correction's column tiles: as few as fit 256 TMEM columns, equal widths, multiples of 16
    const int nt = (d.n_max + 255) / 256;
    d.cn = ((d.n_max + nt - 1) / nt + 15) / 16 * 16;
    d.rows_g = nt * d.cn;
    return d;
}

// byte offsets of the per-walker-spin buffers inside one allocation
struct OzOffsets {
    size_t V, rd, gd, dmax, vmax, invd, vd, mt, vexp, perm, srow, site_oth, dprev, done, active, tile_list, grp_list, counts, grp_flag,
        total;
};
OzOffsets oz_offsets(const OzDims &d, int n_walkers) {
    const size_t S = (size_t)2 * n_walkers;
    OzOffsets o{};
    size_t p = 0;
    auto take = [&](size_t bytes) {
        const size_t at = p;
        p = align256(p + bytes);
        return at;
    };
    o.V = take(S * d.rows_v * d.ldz * 4);
    o.rd = take(S * 3 * (size_t)d.kp * d.rows_v * 2);
    o.gd = take(S * 3 * (size_t)d.kp * d.rows_g * 2);
    o.dmax = take(S * d.rows_v * 4);
    o.invd = take(S * d.n_max * 4);
    o.vmax = take(S * d.rows_v * 4);
    o.vd = take(S * kOzVDigits * (size_t)d.kp * d.rows_v * 2);
    o.mt = take(S * kOzUDigits * (size_t)d.kp * d.rows_m * 2);
    o.vexp = take(S * d.rows_v * 4);
    o.perm = take(S * d.n_max * 4);
    o.srow = take(S * d.n_max * 4);
    o.site_oth = take(S * d.oth_max * 2);
    o.dprev = take(S * d.tiles * 4);
    o.done = take(S * d.tiles * 4);
    o.active = take(S * 4);
    o.tile_list = take(2 * S * d.tiles * 4);
    o.grp_list = take(2 * S * (d.rows_v / oz::kBM) * 4);
    o.counts = take(4 * 4);
    o.grp_flag = take(S * (d.rows_v / oz::kBM) * 4);
    o.total = p;
    return o;
}

}  // namespace

size_t oz_scratch_bytes(const DevModel &m, int n_walkers) { return oz_offsets(oz_dims(m), n_walkers).total; }

bool oz_supported(const DevModel &m, int optin) {
    const OzDims d = oz_dims(m);
    if (!m.U32_up_hi || d.n_max >= 1024 || 2 * d.n_max > 65535) return false;   // the exact-accumulation bound
    const size_t need = std::max({prep_layout(d.n_max, d.oth_max).total, (size_t)oz::kSmem, (size_t)corr_smem(d.cn),
                                  inverse_layout(d.n_max).total});
    return need + 1024 <= (size_t)optin;
}

void oz_digits_host(const double *U, int N, int n, uint16_t *ud, int *fexp) {
    for (int j = 0; j < n; ++j) {
        double cm = 0.0;
        for (int s = 0; s < N; ++s) cm = std::max(cm, std::fabs(U[(size_t)s * n + j]));
        int e = 0;
        if (cm > 0.0) std::frexp(cm, &e);   // cm < 2^e
        fexp[j] = e;
        for (int s = 0; s < N; ++s) {
            double y = std::ldexp(U[(size_t)s * n + j], 6 - e);   // |y| < 64
            for (int t = 0; t < kOzUDigits; ++t) {
                const double dg = std::nearbyint(y);              // |dg| <= 64
                const float f = (float)dg;
                uint32_t bits;
                std::memcpy(&bits, &f, 4);
                ud[((size_t)t * N + s) * n + j] = (uint16_t)(bits >> 16);   // exact in bf16
                y = (y - dg) * 128.0;                              // exact; |y| <= 64
            }
        }
    }
}

cudaError_t oz_setup(const DevModel &m, int n_walkers, void *scratch, OzRefresh &oz) {
    const OzDims d = oz_dims(m);
    const OzOffsets o = oz_offsets(d, n_walkers);
    unsigned char *base = static_cast<unsigned char *>(scratch);
    oz.n_max = d.n_max; oz.oth_max = d.oth_max; oz.ldz = d.ldz; oz.kp = d.kp;
    oz.rows_v = d.rows_v; oz.rows_m = d.rows_m; oz.tiles = d.tiles;
    oz.V = reinterpret_cast<float *>(base + o.V);
    oz.rd = reinterpret_cast<uint16_t *>(base + o.rd);
    oz.gd = reinterpret_cast<uint16_t *>(base + o.gd);
    oz.dmax = reinterpret_cast<float *>(base + o.dmax);
    oz.invd = reinterpret_cast<float *>(base + o.invd);
    oz.vmax = reinterpret_cast<float *>(base + o.vmax);
    oz.cn = d.cn;
    oz.rows_g = d.rows_g;
    oz.vd = reinterpret_cast<uint16_t *>(base + o.vd);
    oz.mt = reinterpret_cast<uint16_t *>(base + o.mt);
    oz.vexp = reinterpret_cast<int *>(base + o.vexp);
    oz.perm = reinterpret_cast<int *>(base + o.perm);
    oz.srow = reinterpret_cast<int *>(base + o.srow);
    oz.site_oth = reinterpret_cast<short *>(base + o.site_oth);
    oz.dprev = reinterpret_cast<float *>(base + o.dprev);
    oz.done = reinterpret_cast<int *>(base + o.done);
    oz.active = reinterpret_cast<int *>(base + o.active);
    oz.n_ws = 2 * n_walkers;
    oz.groups = d.rows_v / oz::kBM;
    oz.tile_list = reinterpret_cast<int *>(base + o.tile_list);
    oz.grp_list = reinterpret_cast<int *>(base + o.grp_list);
    oz.counts = reinterpret_cast<int *>(base + o.counts);
    oz.grp_flag = reinterpret_cast<int *>(base + o.grp_flag);
    cudaError_t e = encode_planes(oz.tmap_v, oz.vd, d.rows_v, d.kp, kOzVDigits, 2 * n_walkers, oz::kBM);
    if (e == cudaSuccess) e = encode_planes(oz.tmap_m, oz.mt, d.rows_m, d.kp, kOzUDigits, 2 * n_walkers, oz::kBN);
    if (e == cudaSuccess) e = encode_planes(oz.tmap_r, oz.rd, d.rows_v, d.kp, 3, 2 * n_walkers, oz::kBM);
    if (e == cudaSuccess) e = encode_planes(oz.tmap_g, oz.gd, d.rows_g, d.kp, 3, 2 * n_walkers, d.cn);
    return e;
}

cudaError_t launch_refresh_oz(const DevModel &m, const DevBatch &b, const OzRefresh &oz, int only_due,
                              int track_drift, int device, cudaStream_t stream) {
    if (!m.U32_up_hi || !b.solve_scratch || !oz.V) return cudaErrorInvalidValue;
    const OzView v = view_of(oz);
    const int W = b.n_walkers;
    const size_t sm_prep = std::max(prep_layout(m.n_up, m.n_dn).total, prep_layout(m.n_dn, m.n_up).total);
    cudaError_t e = cudaFuncSetAttribute(oz_prep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_prep);
    if (e != cudaSuccess) return e;
    oz_prep_kernel<<<dim3(W, 2), kTT, sm_prep, stream>>>(m, b, v, only_due, track_drift);
    const size_t sm_inv = inverse_layout(oz.n_max).total;
    if ((e = cudaFuncSetAttribute(oz_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_inv)))
        return e;
    oz_inverse_kernel<<<W * 2 * ((oz.n_max + kRT - 1) / kRT), kTT, sm_inv, stream>>>(m, b, v);
    oz_gather_kernel<<<dim3(W, 2, kOzUDigits), 256, 0, stream>>>(m, v);
    oz_bplanes_kernel<<<dim3(W, 2, oz.tiles), 256, 0, stream>>>(m, v);
    if ((e = cudaFuncSetAttribute(oz_residual_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, oz::kSmem)))
        return e;
    const int sm_corr = corr_smem(oz.cn);
    if ((e = cudaFuncSetAttribute(oz_corr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_corr))) return e;
    CUtensorMap tmv, tmm, tmr, tmg;
    std::memcpy(&tmv, oz.tmap_v, sizeof tmv);
    std::memcpy(&tmm, oz.tmap_m, sizeof tmm);
    std::memcpy(&tmr, oz.tmap_r, sizeof tmr);
    std::memcpy(&tmg, oz.tmap_g, sizeof tmg);
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device))) return e;
    // the first pass (V = B G) lists every tile still refining in list 1; pass
    // p works on list p & 1 and fills the other, whose counters are cleared first
    if ((e = cudaMemsetAsync(oz.counts, 0, 4 * sizeof(int), stream))) return e;
    oz_corr_kernel<<<sms, kResThreads, sm_corr, stream>>>(m, b, v, 1, 0, tmr, tmg);
    oz_check_kernel<<<4 * sms, 256, 0, stream>>>(m, b, v, 1, 0, 0, track_drift);
    for (int pass = 1; pass <= oz::kOzPasses; ++pass) {
        const int cur = pass & 1, nxt = cur ^ 1;
        oz_slice_kernel<<<4 * sms, 256, 0, stream>>>(m, v, cur);
        oz_residual_kernel<<<sms, kResThreads, oz::kSmem, stream>>>(m, b, v, cur, tmv, tmm);
        oz_corr_kernel<<<sms, kResThreads, sm_corr, stream>>>(m, b, v, 0, cur, tmr, tmg);
        if ((e = cudaMemsetAsync(oz.counts + 2 * nxt, 0, 2 * sizeof(int), stream))) return e;
        oz_check_kernel<<<4 * sms, 256, 0, stream>>>(m, b, v, 0, pass == oz::kOzPasses, cur, track_drift);
    }
    return cudaGetLastError();
}

}  // namespace kvmc
