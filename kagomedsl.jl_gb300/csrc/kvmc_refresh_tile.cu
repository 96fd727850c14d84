// The periodic refresh of the mixed real form with tiled triangular solves
// (kvmc.h: KVMC_TUNE_REFRESH32 = 2).
//
// Reference counterpart: reevaluateW! with tilde_U (KagomeDSL.jl
// src/MonteCarlo.jl:55-115): W = U tilde_U^{-1}.  Only the rows of W at the
// sites of the other spin are computed (the rest are unit rows); stacked as
// the n_oth x n matrix X (row b = the site holding the other spin's label
// b+1) they solve X tilde_U = B, B the rows of U at those sites.
//
// One CTA per (walker, spin), everything in FP32 (no FP64 operation but the
// log|det| sum):
//   1. tilde_U (FP32 high parts of U) gathered into an n x n block in HBM and
//      factorised there by a blocked right-looking LU with partial pivoting,
//      rows never moved (the pivot order is an index, perm): 32-column panels
//      in shared memory, the trailing update as 4 x 4 register tiles.
//      M = P tilde_U = L Uf with row i of M = tilde_U[perm[i]].
//   2. G = M^{-1} (n x n, HBM) from identity rows in tiles of 32: forward
//      with Uf (column blocks of 32 ascending: a GEMM update from the
//      finished columns against the staged block column of Uf, then the
//      32 x 32 triangle, one lane per column and the rows interleaved; the
//      blocks left of the tile's diagonal are zero and skipped), then
//      backward with the unit lower L.
//   3. X in tiles of 32 rows held in shared memory: V = B G, then iterative
//      refinement V += (B - V M) G, X[:, perm[i]] = V[:, i].  The residual
//      B - V M takes U as FP32 (high, low) pairs and sums the high-part
//      products without rounding error on a fixed grid (tile_residual).
//      With d_k the largest correction of pass k relative to its row's
//      largest entry, the error left is about d_k^2 / d_{k-1} (it contracts
//      by a factor near cond(tilde_U) 2^-24 per pass, d_0 = 1); passes run
//      until that is below 1e-6, at most 4.  A tile left above 1e-5 (or
//      whose correction grew) flags the walker (kStatusRefine) and the FP64
//      refresh redoes it.
// Every pass is then two GEMM-shaped loops over 64 x 64 chunks of G or of
// tilde_U, staged by cp.async into a double buffer while the previous chunk
// is multiplied: 2 rows x 4 columns per thread, no serial dependency.
#include "kvmc_tile.cuh"

namespace kvmc {

namespace {

__global__ void __launch_bounds__(kTT) refresh_tile_kernel(DevModel m, DevBatch b, int only_due, int track_drift) {
    const int w = blockIdx.x, spin = blockIdx.y;
    if (only_due && b.since[w] >= 0) return;
    if (spin == 0 && threadIdx.x == 0) atomicAdd(b.refresh_count, 1ull);
    const int N = m.n_sites;
    const int n = spin == 0 ? m.n_up : m.n_dn;
    const int n_oth = N - n;
    const int ldw = spin == 0 ? m.ld_up : m.ld_dn;
    const float *Uh = spin == 0 ? m.U32_up_hi : m.U32_dn_hi;
    const float *Ul = spin == 0 ? m.U32_up_lo : m.U32_dn_lo;
    // during a one-warp sweep call the rows go to the label-indexed blocks
    const bool cpt = b.compact != 0;
    float *Wout = cpt ? b.G32 + (size_t)w * b.g_block + (spin == 0 ? 0 : (size_t)m.n_dn * m.ld_up)
                      : b.W32 + (size_t)w * N * (m.ld_up + m.ld_dn) + (spin == 0 ? 0 : (size_t)N * m.ld_up);
    // tilde_U's factors and G: the FP64 refresh's row scratch (n x rows doubles >= 2 n x n floats)
    float *A = reinterpret_cast<float *>(b.solve_scratch + ((size_t)w * 2 + spin) * b.solve_block);

    extern __shared__ __align__(16) unsigned char smem[];
    const TileSmem L = tile_smem_layout(n, n_oth);
    float *Z = reinterpret_cast<float *>(smem + L.z);
    float *Rt = reinterpret_cast<float *>(smem + L.r);
    float *Pn = reinterpret_cast<float *>(smem + L.pn);
    float *Ut = reinterpret_cast<float *>(smem + L.ut);
    float *St = reinterpret_cast<float *>(smem + L.st);
    float *invd = reinterpret_cast<float *>(smem + L.invd);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    int *srow = reinterpret_cast<int *>(smem + L.srow);
    short *site_of = reinterpret_cast<short *>(smem + L.site_of);
    short *site_oth = reinterpret_cast<short *>(smem + L.site_oth);
    __shared__ double red[33];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x, nw = nt / 32;

    if (!tile_factor(m, b, w, spin, A, Z, Pn, Ut, St, invd, perm, srow, site_of, site_oth, red)) return;
    const int ldz = ld_tile(n);
    float *G = A + (size_t)n * n;
    // the largest column norm of tilde_U, for the residual's summation grid
    __shared__ float s_cmax;
    {
        float cm = 0.f;
        for (int c = tid; c < n; c += nt) {
            float ss = 0.f;
#pragma unroll 8
            for (int l = 0; l < n; ++l) {
                const float u = Uh[(size_t)site_of[l] * n + c];
                ss = fmaf(u, u, ss);
            }
            cm = fmaxf(cm, ss);
        }
        const float cm2 = (float)block_sum_max((double)cm, red);
        if (tid == 0) s_cmax = sqrtf(cm2);
        __syncthreads();
    }
    const float cmax = s_cmax;
    for (int e = tid; e < kRT * (ldz - n); e += nt) {
        const int r = e / (ldz - n), c = n + e % (ldz - n);
        Rt[(size_t)r * ldz + c] = 0.f;
    }
    float dmax = 0.f;
    bool converged = true;
    for (int b0 = 0; b0 < n_oth; b0 += kRT) {
        const int rows = min(kRT, n_oth - b0);
        __syncthreads();
        // B (high parts) into the residual tile, then V = B G
        for (int cb = 0; cb < n; cb += 32)
            stage_rows32(Rt + cb, ldz, kRT, min(32, n - cb), min(32, n - cb), [&](int r) -> const float * {
                return r < rows ? Uh + (size_t)site_oth[b0 + r] * n + cb : nullptr;
            });
        tile_gemm(G, n, Rt, Z, ldz, rows, 0, St, red);
        // passes until the error left, estimated as d_k^2 / d_{k-1} from the
        // relative corrections d_k, is below 1e-6; at most kMaxPasses
        float est = 1.f, dprev = 1.f;
        for (int pass = 0; pass < kMaxPasses; ++pass) {
            tile_residual(Uh, Ul, n, srow, site_oth, b0, rows, Z, Rt, ldz, St, cmax);
            const float d = tile_gemm(G, n, Rt, Z, ldz, rows, 1, St, red);  // V += R G
            est = d < dprev ? d * d / dprev : INFINITY;  // a correction that grows: diverging
            dprev = d;
            if (!(est > 1e-6f)) break;
        }
        if (!(est <= 1e-5f)) converged = false;
        // the tile's rows out, in label order: X[:, perm[i]] = V[:, i]
        for (int r = warp; r < rows; r += nw) {
            float *wr = Wout + (size_t)(cpt ? b0 + r : site_oth[b0 + r]) * ldw;
            for (int i = lane; i < n; i += 32) {
                const float nv = Z[(size_t)r * ldz + i];
                if (track_drift) dmax = fmaxf(dmax, fabsf(wr[perm[i]] - nv) / (1.f + fabsf(nv)));
                wr[perm[i]] = nv;
            }
            if (!cpt)
                for (int c = n + lane; c < ldw; c += 32) wr[c] = 0.f;
        }
    }
    // unit rows at the sites holding this spin (site-indexed W only)
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
    if (!converged && tid == 0) atomicOr(&b.status[w], kStatusRefine);
}

}  // namespace

size_t refresh_tile_smem(const DevModel &m) {
    const TileSmem a = tile_smem_layout(m.n_up, m.n_dn), c = tile_smem_layout(m.n_dn, m.n_up);
    return std::max(a.total, c.total) + 64;
}

cudaError_t launch_refresh_tile(const DevModel &m, const DevBatch &b, int only_due, int track_drift,
                                cudaStream_t stream) {
    if (!m.U32_up_hi || !b.solve_scratch) return cudaErrorInvalidValue;
    const size_t sm = refresh_tile_smem(m);
    cudaError_t e = cudaFuncSetAttribute(refresh_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    refresh_tile_kernel<<<dim3(b.n_walkers, 2), kTT, sm, stream>>>(m, b, only_due, track_drift);
    return cudaGetLastError();
}

}  // namespace kvmc
