// Device helpers shared by the real (kvmc_kernels.cu) and complex
// (kvmc_complex.cu) kernels of libkvmc: the Philox proposal stream, block
// reductions and the exact acceptance-threshold test.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc_internal.h"

namespace kvmc {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11): counter-based, so proposal t of
// walker w is the same draw however the proposals are split across launches.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned hi0 = __umulhi(0xD2511F53u, c.x);
        const unsigned lo0 = 0xD2511F53u * c.x;
        const unsigned hi1 = __umulhi(0xCD9E8D57u, c.z);
        const unsigned lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        if (r < 9) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
    }
    return c;
}

// Proposal t of walker w: r uniform in [0,1) (53 bits) and a bond index.
__device__ __forceinline__ void proposal_draw(unsigned long long seed, int walker, long long t,
                                              int n_bonds, double &r, int &bond) {
    const unsigned long long ut = (unsigned long long)t;
    const uint4 x = philox4x32_10(make_uint4((unsigned)ut, (unsigned)(ut >> 32), (unsigned)walker, 0u),
                                  make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const unsigned long long u53 = ((unsigned long long)(x.x >> 5) << 26) | (x.y >> 6);
    r = (double)u53 * (1.0 / 9007199254740992.0);
    bond = (int)(((unsigned long long)x.z * (unsigned long long)(unsigned)n_bonds) >> 32);
}

// The same draw as raw bits: u53 (r = u53 * 2^-53) and the bond index.
__device__ __forceinline__ void proposal_bits(unsigned long long seed, int walker, long long t, int n_bonds,
                                              unsigned long long &u53, int &bond) {
    const unsigned long long ut = (unsigned long long)t;
    const uint4 x = philox4x32_10(make_uint4((unsigned)ut, (unsigned)(ut >> 32), (unsigned)walker, 0u),
                                  make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    u53 = ((unsigned long long)(x.x >> 5) << 26) | (x.y >> 6);
    bond = (int)(((unsigned long long)x.z * (unsigned long long)(unsigned)n_bonds) >> 32);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide FP64 sum; every thread gets the result.  `red` holds >= 33 doubles.
static __device__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double s = lane < nw ? red[lane] : 0.0;
        s = warp_sum(s);
        if (lane == 0) red[32] = s;
    }
    __syncthreads();
    return red[32];
}

// Block-wide FP64 max; every thread gets the result.
static __device__ double block_sum_max(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double s = lane < nw ? red[lane] : -INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
        if (lane == 0) red[32] = s;
    }
    __syncthreads();
    return red[32];
}

__device__ __forceinline__ void atomic_max_nonneg(float *addr, float v) {
    atomicMax(reinterpret_cast<int *>(addr), __float_as_int(v));
}

// ---------------------------------------------------------------------------
// Acceptance decisions without FP64 on the common path.
//
// The reference rejects when r > Z_mu/Z_max (src/MonteCarlo.jl:546-550),
// then accepts when |ratio|^2 >= 1 and r < Z_mu/Z_max, or when
// r < (Z_mu/Z_max) |ratio|^2 (:581-591), all in FP64 with one uniform r.
// Here r = u53 * 2^-53 exactly, thr = fl(Z_mu/Z_max) is encoded once per
// change of Z_mu as m * 2^(k-53), and "r vs thr" becomes an exact integer
// comparison.  The second test runs in FP32 with a relative guard band of
// 1e-5 (FP32 carries ~1e-7); only a lane inside the band recomputes it in
// FP64, so every decision equals the FP64 one while the FP64 pipe (1/64 of
// the FP32 rate on GB300) is almost never issued.
// ---------------------------------------------------------------------------
struct Thr {
    double d;              // fl(zmu / n_bonds), or 1 for the Metropolis rule
    float f;
    unsigned long long m;  // thr = m * 2^(k - 53); m = 0 encodes thr = 0
    int k;
};

// thr for the current Z_mu: a lookup in the table the host filled with
// fl(z / n_bonds) for every z (an FP64 division on the device would sit on
// the critical path of every accepted move).
__device__ __forceinline__ void make_thr(Thr &T, const ThrEntry *table, int zmu, int rule) {
    const ThrEntry e = table[rule == 0 ? zmu : 0];
    T.d = rule == 0 ? e.d : 1.0;
    T.f = rule == 0 ? e.f : 1.f;
    T.m = rule == 0 ? e.m : (1ull << 52);
    T.k = rule == 0 ? e.k : 1;
}

// sign(r - thr) for r = u53 * 2^-53, exact.  thr >= 1/n_bonds keeps -k <= 11.
__device__ __forceinline__ int cmp_r_thr(unsigned long long u53, const Thr &T) {
    if (T.m == 0) return u53 > 0 ? 1 : 0;
    unsigned long long L = u53, Rr = T.m;
    if (T.k >= 0) Rr <<= T.k;
    else L <<= -T.k;
    return L > Rr ? 1 : (L < Rr ? -1 : 0);
}

__device__ __forceinline__ double r_of(unsigned long long u53) { return (double)u53 * (1.0 / 9007199254740992.0); }

// r in FP32 to ~1e-7 relative (two 32-bit conversions, no FP64)
__device__ __forceinline__ float r_f32(unsigned long long u53) {
    return (float)(unsigned)(u53 >> 21) * 2.3283064365386963e-10f + (float)(unsigned)(u53 & 0x1FFFFF) * 1.1102230246251565e-16f;
}

// FP64 decision from the two ratio factors (the plain form's rule, and the
// mixed form's fallback inside the guard band)
__device__ __forceinline__ bool decide_f64(double pu, double pd, unsigned long long u53, int c, const Thr &T, int rule,
                                           bool &bad) {
    const double ratio = pu * pd;
    const double a = ratio * ratio;
    if (!isfinite(a)) { bad = true; return false; }
    const double r = r_of(u53);
    if (rule == 0) return a >= 1.0 ? (c < 0) : (r < T.d * a);
    return a >= 1.0 || r < a;
}

__device__ __forceinline__ bool decide(double pu, double pd, unsigned long long u53, int c, const Thr &T, int rule,
                                       bool &bad) {
    return decide_f64(pu, pd, u53, c, T, rule, bad);
}

__device__ __forceinline__ bool decide(float pu, float pd, unsigned long long u53, int c, const Thr &T, int rule,
                                       bool &bad) {
    const float rt = pu * pd;
    const float a = rt * rt;
    if (isnan(a)) { bad = true; return false; }
    constexpr float band = 1e-5f;
    if (a >= 1.f + band) return rule == 0 ? (c < 0) : true;   // includes a = inf
    if (a <= 1.f - band) {
        const float x = rule == 0 ? T.f * a : a;
        const float rf = r_f32(u53);
        if (rf < x * (1.f - band)) return true;
        if (rf > x * (1.f + band)) return false;
    }
    return decide_f64((double)pu, (double)pd, u53, c, T, rule, bad);
}

// Block sum of FP32 partials into FP64: FP32 within each warp, FP64 across
// the warps (only warp 0 touches the FP64 pipe).  red holds >= 33 doubles.
static __device__ double block_sum_f32(float v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    float *redf = reinterpret_cast<float *>(red);
    __syncthreads();
    if (lane == 0) redf[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double s = lane < nw ? (double)redf[lane] : 0.0;
        s = warp_sum(s);
        if (lane == 0) red[32] = s;
    }
    __syncthreads();
    return red[32];
}

// Antiparallel bonds touching sites a or b (each bond counted once).
static __device__ int incident_antiparallel(const DevModel &m, const short *kup, int a, int bsite) {
    int c = 0;
    for (int e = m.nbr_off[a]; e < m.nbr_off[a + 1]; ++e) {
        const int k = m.nbr[e];
        c += ((kup[a] != 0) != (kup[k] != 0));
    }
    for (int e = m.nbr_off[bsite]; e < m.nbr_off[bsite + 1]; ++e) {
        const int k = m.nbr[e];
        if (k == a) continue;
        c += ((kup[bsite] != 0) != (kup[k] != 0));
    }
    return c;
}

// ---- complex scalars -------------------------------------------------------
struct __align__(16) cd { double x, y; };
struct __align__(8) cf { float x, y; };

template <typename C> struct Real;
template <> struct Real<cd> { using T = double; };
template <> struct Real<cf> { using T = float; };

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// c - a * b
template <typename C> __device__ __forceinline__ C cfms(C a, C b, C c) {
    return C{fma(-a.x, b.x, fma(a.y, b.y, c.x)), fma(-a.x, b.y, fma(-a.y, b.x, c.y))};
}
// c + a * b
template <typename C> __device__ __forceinline__ C cfma(C a, C b, C c) {
    return C{fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))};
}
template <typename C> __device__ __forceinline__ C cinv(C a) {
    const auto d = a.x * a.x + a.y * a.y;
    return C{a.x / d, -a.y / d};
}
template <typename C> __device__ __forceinline__ typename Real<C>::T cabs2(C a) { return a.x * a.x + a.y * a.y; }
// LAPACK's pivot magnitude for complex matrices, |re| + |im|
__device__ __forceinline__ double cabs1(cd a) { return fabs(a.x) + fabs(a.y); }

}  // namespace kvmc
