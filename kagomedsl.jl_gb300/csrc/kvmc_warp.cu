// One warp per walker: the mixed real form's sweep with W held as its
// non-trivial block, indexed by orbital labels (kvmc.h: KVMC_TUNE_WARP_WALKERS).
//
// Reference counterparts (KagomeDSL.jl): Carlo.sweep! with Z and the
// Z_mu-weighted acceptance (src/MonteCarlo.jl:460-607), update_W! / geru!
// (:279-292) applied as delayed rank-k updates, getOL (src/Hamiltonian.jl:762-778)
// at the measure! cadence (src/MonteCarlo.jl:628-634).
//
// Every site holds exactly one spin (n_up + n_down = N).  Row R of W_up is
// the unit row e_a when site R holds the up spin of label a, so only the
// rows at the n_down sites that hold a down spin carry information.  Indexing
// those rows by the down spin's label b gives the compact block
//     G_up[b][a] = W_up[site of down label b][a]       (n_down x n_up)
// and likewise G_dn[a][b] = W_dn[site of up label a][b] (n_up x n_down).
// An exchange moves up label a from site i to site j and down label b from j
// to i; its ratio is G_up[b][a] * G_dn[a][b], and the Sherman-Morrison
// update becomes, with piv = G_up[b][a],
//     G_up' = G_up - p q^T,  p = (G_up[:, a] + e_b) / piv,  q = G_up[b, :] - e_a
// (row b now describes site i, where label b sits after the move), and the
// same with the roles of the spins exchanged for G_dn.  No row moves, so the
// labels are the only bookkeeping.  Against the site-indexed form this halves
// the multiply-adds and the bytes of every flush.
//
// Delayed updates: G_eff = G - P Q^T with up to K pending moves; P, Q and the
// configuration live in shared memory (about 15 KB per walker at N = 216,
// K = 8), so a CTA holds up to 14 walkers, one per warp.  Each warp runs its
// own serial chain; the SM's other warps fill its latency.  G lives in
// HBM/L2; the first sweep call converts the handle's site-indexed W into G,
// which then stays the state from call to call (the refreshes write G), and
// the calls that read or write the site-indexed W convert it back.  The G
// blocks of the walkers in flight should
// fit in L2 (7 walkers per SM at N = 216: 99 MB): with more walkers in
// flight the flushes stream from HBM and each chain slows down more than
// the extra walkers gain.
//
// Accuracy guard: FP32 loses accuracy while W carries large entries (a
// configuration close to a node of the wave function): rounding at the scale
// of max|W| stays behind as W shrinks again.  The kernel tracks the largest
// |G_eff| entry of the column and row every accepted move reads; once that has
// exceeded cond_hi since the walker's last refresh and the move's entries are
// back below cond_lo, the walker stops for a refresh.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc.h"
#include "kvmc_device.cuh"
#include "kvmc_internal.h"

namespace kvmc {

namespace {

template <int K>
struct CSpin {
    float *G;        // global [n_oth][ldg]: row = other spin's label, column = own label
    float *P;        // shared [n_oth][K]
    float *Q;        // shared [ldg][K] (rows beyond n_own stay zero)
    int ldg, n_oth, n_own;
    // sum over the K factor columns of P[r][k] Q[c][k] (pending columns beyond
    // the current count are zero)
    __device__ __forceinline__ float pq(int r, int c) const {
        const float4 *pr = reinterpret_cast<const float4 *>(P + (size_t)r * K);
        const float4 *qc = reinterpret_cast<const float4 *>(Q + (size_t)c * K);
        float a0 = 0.f, a1 = 0.f;
#pragma unroll
        for (int k = 0; k < K / 4; ++k) {
            const float4 x = pr[k], y = qc[k];
            a0 = fmaf(x.x, y.x, a0);
            a1 = fmaf(x.y, y.y, a1);
            a0 = fmaf(x.z, y.z, a0);
            a1 = fmaf(x.w, y.w, a1);
        }
        return a0 + a1;
    }
    __device__ __forceinline__ float eff(int r, int c) const { return G[(size_t)r * ldg + c] - pq(r, c); }
};

// The factor columns of an accepted move, for both spins at once.  For a
// spin, s = the other spin's label whose row is replaced, l = the own label
// that moves (up: s = b, l = a; down: s = a, l = b):
//   P[r][m] = (G_eff[r][l] + [r == s]) / piv,   Q[c][m] = G_eff[s][c] - [c == l]
// The two entries that read P[s][m] / Q[l][m] themselves (r == s, c == l)
// are written by the caller after a __syncwarp, so that every dot here sees
// column m still zero.  Each round issues four loads per lane for each spin
// before any arithmetic, so the two spins' L2 round trips overlap.  Returns
// the largest |G_eff| entry the lane read.
template <int K>
__device__ __forceinline__ float column_write(const CSpin<K> &A, int sa, int la, float ipa, const CSpin<K> &B,
                                               int sb, int lb, float ipb, int m, int lane) {
    const int ta = A.n_oth + A.n_own, tb = B.n_oth + B.n_own;
    const int tot = ta > tb ? ta : tb;
    float mx = 0.f;
    for (int base = 0; base < tot; base += 128) {
        float wa[4], wb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = base + 32 * q + lane;
            wa[q] = 0.f;
            if (e < A.n_oth) wa[q] = A.G[(size_t)e * A.ldg + la];
            else if (e < ta) wa[q] = A.G[(size_t)sa * A.ldg + (e - A.n_oth)];
            wb[q] = 0.f;
            if (e < B.n_oth) wb[q] = B.G[(size_t)e * B.ldg + lb];
            else if (e < tb) wb[q] = B.G[(size_t)sb * B.ldg + (e - B.n_oth)];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = base + 32 * q + lane;
            if (e < A.n_oth) {
                const float v = wa[q] - A.pq(e, la);
                mx = fmaxf(mx, fabsf(v));
                if (e != sa) A.P[(size_t)e * K + m] = v * ipa;
            } else if (e < ta) {
                const int c = e - A.n_oth;
                const float v = wa[q] - A.pq(sa, c);
                mx = fmaxf(mx, fabsf(v));
                if (c != la) A.Q[(size_t)c * K + m] = v;
            }
            if (e < B.n_oth) {
                const float v = wb[q] - B.pq(e, lb);
                mx = fmaxf(mx, fabsf(v));
                if (e != sb) B.P[(size_t)e * K + m] = v * ipb;
            } else if (e < tb) {
                const int c = e - B.n_oth;
                const float v = wb[q] - B.pq(sb, c);
                mx = fmaxf(mx, fabsf(v));
                if (c != lb) B.Q[(size_t)c * K + m] = v;
            }
        }
    }
    return mx;
}

// G -= P Q^T.  Lane = a group of four columns (Q of those columns held in
// registers); rows streamed kRows at a time, all their loads in flight
// before the arithmetic.
template <int K, int kRows>
__device__ void warp_flush(const CSpin<K> &S, int lane) {
    const int q4 = S.ldg >> 2;
    for (int c4 = lane; c4 < q4; c4 += 32) {
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
        for (int r0 = 0; r0 < S.n_oth; r0 += kRows) {
            float4 g[kRows];
#pragma unroll
            for (int i = 0; i < kRows; ++i)
                if (r0 + i < S.n_oth) g[i] = reinterpret_cast<const float4 *>(S.G + (size_t)(r0 + i) * S.ldg)[c4];
#pragma unroll
            for (int i = 0; i < kRows; ++i) {
                if (r0 + i < S.n_oth) {
                    const float4 *pr = reinterpret_cast<const float4 *>(S.P + (size_t)(r0 + i) * K);
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
                    float4 x = g[i];
                    x.x -= a0; x.y -= a1; x.z -= a2; x.w -= a3;
                    reinterpret_cast<float4 *>(S.G + (size_t)(r0 + i) * S.ldg)[c4] = x;
                }
            }
        }
    }
}

template <int K>
__device__ __forceinline__ void zero_factors(const CSpin<K> &S, int lane) {
    float4 *p = reinterpret_cast<float4 *>(S.P);
    for (int e = lane; e < S.n_oth * K / 4; e += 32) p[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 *q = reinterpret_cast<float4 *>(S.Q);
    for (int e = lane; e < S.ldg * K / 4; e += 32) q[e] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// the four columns 4 c4 .. 4 c4 + 3 of a unit row whose 1 sits at offset o from the first
__device__ __forceinline__ float4 unit4(int o) {
    return make_float4(o == 0 ? 1.f : 0.f, o == 1 ? 1.f : 0.f, o == 2 ? 1.f : 0.f, o == 3 ? 1.f : 0.f);
}

__device__ __forceinline__ float warp_max_nonneg(float v) {
    return __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(v)));
}

}  // namespace

// Shared memory: the CTA's bond tables, then one region per warp.
size_t warp_cta_smem(const DevModel &m) {
    size_t s = (size_t)m.n_bonds * sizeof(short2) + (size_t)2 * m.n_bonds * sizeof(short);
    s = (s + 15) / 16 * 16;
    s += (size_t)(m.n_sites + 1) * sizeof(int);
    return (s + 15) / 16 * 16;
}

size_t warp_walker_smem(const DevModel &m, int K) {
    size_t s = (size_t)(m.n_dn + m.ld_up + m.n_up + m.ld_dn) * K * sizeof(float);  // P, Q of both spins
    s += (size_t)m.n_sites * sizeof(int);     // up-neighbour counts
    s += (size_t)m.n_sites * sizeof(short);   // signed labels
    return (s + 15) / 16 * 16;
}

size_t warp_compact_block(const DevModel &m) {
    return (size_t)m.n_dn * m.ld_up + (size_t)m.n_up * m.ld_dn;
}

// At most 14 walkers per CTA at 128 registers per thread: each SM
// sub-partition then holds four of the walkers' warps.
constexpr int kWarpMaxWalkers = 14;

template <int K, int kRows>
__device__ __forceinline__ void sweep_warp_body(const DevModel &m, const DevBatch &b, const SweepParams &p,
                                                int *active_count, size_t cta_bytes, size_t walker_bytes) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int N = m.n_sites, nb = m.n_bonds;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    short2 *bonds = reinterpret_cast<short2 *>(smem);
    short *nbr = reinterpret_cast<short *>(bonds + nb);
    int *nbr_off = reinterpret_cast<int *>(smem + ((nb * sizeof(short2) + 2 * nb * sizeof(short) + 15) / 16 * 16));
    for (int e = threadIdx.x; e < nb; e += blockDim.x) bonds[e] = m.bonds[e];
    for (int e = threadIdx.x; e < 2 * nb; e += blockDim.x) nbr[e] = m.nbr[e];
    for (int e = threadIdx.x; e <= N; e += blockDim.x) nbr_off[e] = m.nbr_off[e];
    __syncthreads();

    const int w = blockIdx.x * nwarps + wl;
    if (w >= b.n_walkers) return;
    const long long t0 = b.t[w];
    const long long tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);
    const long long acc_left = b.acc_end[w] - b.accepted[w];
    const int since0 = b.since[w];
    if (t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop)) {
        // nothing to do; a refresh marked due has run since (stream order): clear
        // the mark and the guard's record of the W it replaced
        if (lane == 0 && since0 < 0) {
            b.since[w] = 0;
            b.cond_max[w] = 0.f;
        }
        return;
    }

    unsigned char *mine = smem + cta_bytes + (size_t)wl * walker_bytes;
    const int nu_ = m.n_up, nd_ = m.n_dn;
    CSpin<K> SU, SD;
    SU.P = reinterpret_cast<float *>(mine);
    SU.Q = SU.P + (size_t)nd_ * K;
    SD.P = SU.Q + (size_t)m.ld_up * K;
    SD.Q = SD.P + (size_t)nu_ * K;
    int *nup = reinterpret_cast<int *>(SD.Q + (size_t)m.ld_dn * K);
    short *lab = reinterpret_cast<short *>(nup + N);
    SU.ldg = m.ld_up; SU.n_oth = nd_; SU.n_own = nu_;
    SD.ldg = m.ld_dn; SD.n_oth = nu_; SD.n_own = nd_;
    SU.G = b.G32 + (size_t)w * b.g_block;
    SD.G = SU.G + (size_t)nd_ * m.ld_up;

    // configuration: +a for up label a, -b for down label b
    for (int s = lane; s < N; s += 32) {
        const int ku = b.kappa_up[(size_t)w * N + s], kd = b.kappa_dn[(size_t)w * N + s];
        lab[s] = (short)(ku != 0 ? ku : -kd);
    }
    zero_factors<K>(SU, lane);
    zero_factors<K>(SD, lane);
    __syncwarp();
    // Z_mu and the up-neighbour counts
    int zl = 0;
    for (int e = lane; e < nb; e += 32) {
        const short2 bd = bonds[e];
        zl += (lab[bd.x] > 0) != (lab[bd.y] > 0);
    }
    for (int s = lane; s < N; s += 32) {
        int c = 0;
        for (int e = nbr_off[s]; e < nbr_off[s + 1]; ++e) c += lab[nbr[e]] > 0;
        nup[s] = c;
    }
    int zmu = __reduce_add_sync(0xffffffffu, zl);
    __syncwarp();

    const int R = p.refresh_every, M = p.measure_every;
    long long t = t0, acc = 0, next_meas = (t0 / M + 1) * M;
    int since = since0 < 0 ? 0 : since0;
    // the largest |G_eff| entry seen since the walker's last refresh
    float cmax = since0 < 0 ? 0.f : b.cond_max[w];
    Thr thr;
    make_thr(thr, m.thr_table, zmu, p.accept_rule);
    double se = 0.0, se2 = 0.0;
    long long n_meas = 0;
    int mm = 0;
    bool bad_walker = false;

    while (true) {
        if (t == next_meas) {
            // local energy (getOL): SzSz over the bonds, -1/2 ratio per antiparallel bond;
            // four bonds per lane at a time, their G entries loaded before the sums
            __syncwarp();
            float el = 0.f;
            for (int e0 = lane; e0 < nb; e0 += 128) {
                float gu[4], gd[4];
                int ai[4], bi4[4], kind[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int e = e0 + 32 * q;
                    kind[q] = -1;
                    gu[q] = gd[q] = 0.f;
                    ai[q] = bi4[q] = 0;
                    if (e < nb) {
                        const short2 bd = bonds[e];
                        const int li = lab[bd.x], lj = lab[bd.y];
                        if ((li > 0) == (lj > 0)) {
                            kind[q] = 0;
                        } else {
                            kind[q] = 1;
                            ai[q] = (li > 0 ? li : lj) - 1;
                            bi4[q] = (li > 0 ? -lj : -li) - 1;
                            gu[q] = SU.G[(size_t)bi4[q] * SU.ldg + ai[q]];
                            gd[q] = SD.G[(size_t)ai[q] * SD.ldg + bi4[q]];
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (kind[q] == 0)
                        el += 0.25f;
                    else if (kind[q] == 1)
                        el = fmaf(-0.5f * (gu[q] - SU.pq(bi4[q], ai[q])), gd[q] - SD.pq(ai[q], bi4[q]), el - 0.25f);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) el += __shfl_xor_sync(0xffffffffu, el, o);
            se += (double)el;
            se2 += (double)el * (double)el;
            n_meas += 1;
            next_meas += M;
            continue;
        }
        if (t >= tend || since >= R || acc >= acc_left || bad_walker) break;
        const long long lim = min(tend, next_meas) - t;
        const int win = lim < 32 ? (int)lim : 32;
        bool accd = false, bad = false;
        int a = 0, bl = 0, Ku = 0, Kd = 0;
        float pu = 0.f, pd = 0.f;
        if (lane < win) {
            unsigned long long u53;
            int bi;
            proposal_bits(p.seed, w, t + lane, nb, u53, bi);
            const int c = cmp_r_thr(u53, thr);
            if (p.accept_rule != 0 || c <= 0) {
                const short2 bd = bonds[bi];
                const int li = lab[bd.x], lj = lab[bd.y];
                if ((li > 0) != (lj > 0)) {
                    // the up spin at the up site moves to the down site (Ku), the down spin the other way (Kd)
                    if (li > 0) { a = li - 1; bl = -lj - 1; Ku = bd.y; Kd = bd.x; }
                    else        { a = lj - 1; bl = -li - 1; Ku = bd.x; Kd = bd.y; }
                    pu = SU.eff(bl, a);
                    pd = SD.eff(a, bl);
                    accd = decide(pu, pd, u53, c, thr, p.accept_rule, bad);
                }
            }
        }
        if (__any_sync(0xffffffffu, bad)) {
            // a non-finite ratio: the walker stops here and the call reports it
            if (lane == 0) atomicOr(&b.status[w], kStatusNonFinite);
            bad_walker = true;
            break;
        }
        const unsigned mask = __ballot_sync(0xffffffffu, accd);
        if (!mask) {
            t += win;
            continue;
        }
        const int f = __ffs(mask) - 1;
        a = __shfl_sync(0xffffffffu, a, f);
        bl = __shfl_sync(0xffffffffu, bl, f);
        Ku = __shfl_sync(0xffffffffu, Ku, f);
        Kd = __shfl_sync(0xffffffffu, Kd, f);
        pu = __shfl_sync(0xffffffffu, pu, f);
        pd = __shfl_sync(0xffffffffu, pd, f);
        t += f + 1;
        // factor columns mm of both spins (from the configuration before the move)
        const float ipu = 1.f / pu, ipd = 1.f / pd;
        float mx = column_write<K>(SU, bl, a, ipu, SD, a, bl, ipd, mm, lane);
        // Z_mu change from the up-neighbour counts (configuration before the move)
        const int bu = nbr_off[Ku], du = nbr_off[Ku + 1] - bu;
        const int bd0 = nbr_off[Kd], dd = nbr_off[Kd + 1] - bd0;
        const int dz = du - dd + 2 - 2 * nup[Ku] + 2 * nup[Kd];
        __syncwarp();  // every dot of the column write and every count read is done
        if (lane == 0) {
            SU.P[(size_t)bl * K + mm] = (pu + 1.f) * ipu;
            SU.Q[(size_t)a * K + mm] = pu - 1.f;
            SD.P[(size_t)a * K + mm] = (pd + 1.f) * ipd;
            SD.Q[(size_t)bl * K + mm] = pd - 1.f;
            lab[Ku] = (short)(a + 1);
            lab[Kd] = (short)(-(bl + 1));
        }
        for (int e = lane; e < du + dd; e += 32)
            atomicAdd(&nup[e < du ? nbr[bu + e] : nbr[bd0 + e - du]], e < du ? 1 : -1);
        zmu += dz;
        make_thr(thr, m.thr_table, zmu, p.accept_rule);
        since += 1;
        acc += 1;
        mm += 1;
        // accuracy guard
        mx = warp_max_nonneg(mx);
        cmax = fmaxf(cmax, mx);
        if (p.cond_hi > 0.f && cmax > p.cond_hi && mx < p.cond_lo) {
            // refresh when the moves this launch still owes are done (the end of
            // the call, or of its segment) if they are fewer than an interval,
            // so that refreshes stay on launch boundaries; else at once
            const long long rem = acc_left - acc;
            since = rem < R ? max(since, R - (int)rem) : R;
        }
        __syncwarp();
        if (mm == K) {
            warp_flush<K, kRows>(SU, lane);
            warp_flush<K, kRows>(SD, lane);
            __syncwarp();
            zero_factors<K>(SU, lane);
            zero_factors<K>(SD, lane);
            __syncwarp();
            mm = 0;
        }
    }
    if (mm > 0) {
        warp_flush<K, kRows>(SU, lane);
        warp_flush<K, kRows>(SD, lane);
    }
    __syncwarp();
    for (int s = lane; s < N; s += 32) {
        const int l = lab[s];
        b.kappa_up[(size_t)w * N + s] = (short)(l > 0 ? l : 0);
        b.kappa_dn[(size_t)w * N + s] = (short)(l < 0 ? -l : 0);
    }
    if (lane == 0) {
        b.t[w] = t;
        b.since[w] = since >= R ? -1 : since;
        b.cond_max[w] = cmax;
        b.accepted[w] += acc;
        b.proposals[w] += t - t0;
        b.sum_e[w] += se;
        b.sum_e2[w] += se2;
        b.n_meas[w] += n_meas;
        if (t < tend_all && acc < acc_left && !bad_walker) atomicAdd(active_count, 1);
    }
}

// Up to 14 walkers per CTA: 128 registers per thread, so that four warps
// fit on each SM sub-partition; the flush streams four rows at a time.
template <int K>
__global__ void __maxnreg__(128)
sweep_warp_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count, size_t cta_bytes, size_t walker_bytes) {
    sweep_warp_body<K, 4>(m, b, p, active_count, cta_bytes, walker_bytes);
}

// Up to 8 walkers per CTA, without the register cap: where shared memory
// allows one CTA per SM anyway, the registers of up to 256 threads are free,
// and the chain's loads stay in flight without spills (at N = 216, K = 12:
// 227 registers against 128 with 24 bytes spilled, and 11% faster).
constexpr int kWarpWideWalkers = 8;
template <int K>
__global__ void __launch_bounds__(32 * kWarpWideWalkers, 1)
sweep_warp_wide_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count, size_t cta_bytes,
                       size_t walker_bytes) {
    sweep_warp_body<K, 4>(m, b, p, active_count, cta_bytes, walker_bytes);
}

// Site-indexed W -> the label-indexed blocks (and back), one warp per walker.
// A handle in one-warp mode converts before its first sweep call, and back
// only for a call that reads or writes the site-indexed W.
__global__ void __launch_bounds__(128)
warp_to_compact_kernel(DevModel m, DevBatch b) {
    const int lane = threadIdx.x & 31, w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= b.n_walkers) return;
    const int N = m.n_sites, nd_ = m.n_dn;
    const short *ku = b.kappa_up + (size_t)w * N, *kd = b.kappa_dn + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    const float *Wu = b.W32 + (size_t)w * wblock;
    const float *Wd = Wu + (size_t)N * m.ld_up;
    float *G = b.G32 + (size_t)w * b.g_block;
    const int qu = m.ld_up >> 2, qd = m.ld_dn >> 2, qm = max(qu, qd);
    const int tot = N * qm;
    const int dn_off = (int)(((size_t)nd_ * m.ld_up) / 4);
    for (int e0 = 0; e0 < tot; e0 += 128) {
        float4 v[4];
        int dst[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = e0 + 32 * q + lane;
            dst[q] = -1;
            if (e < tot) {
                const int s = e / qm, c4 = e - s * qm;
                const int lu = ku[s], ld = kd[s];
                if (lu == 0 && ld > 0 && c4 < qu) {
                    v[q] = reinterpret_cast<const float4 *>(Wu + (size_t)s * m.ld_up)[c4];
                    dst[q] = (ld - 1) * qu + c4;
                } else if (lu > 0 && c4 < qd) {
                    v[q] = reinterpret_cast<const float4 *>(Wd + (size_t)s * m.ld_dn)[c4];
                    dst[q] = dn_off + (lu - 1) * qd + c4;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (dst[q] >= 0) reinterpret_cast<float4 *>(G)[dst[q]] = v[q];
    }
}

__global__ void __launch_bounds__(128)
warp_from_compact_kernel(DevModel m, DevBatch b) {
    const int lane = threadIdx.x & 31, w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= b.n_walkers) return;
    const int N = m.n_sites, nd_ = m.n_dn;
    const short *ku = b.kappa_up + (size_t)w * N, *kd = b.kappa_dn + (size_t)w * N;
    const size_t wblock = (size_t)N * (m.ld_up + m.ld_dn);
    float *Wu = b.W32 + (size_t)w * wblock;
    float *Wd = Wu + (size_t)N * m.ld_up;
    const float4 *Gv = reinterpret_cast<const float4 *>(b.G32 + (size_t)w * b.g_block);
    const int qu = m.ld_up >> 2, qd = m.ld_dn >> 2, qm = max(qu, qd);
    const int tot = N * qm;
    const int dn_off = (int)(((size_t)nd_ * m.ld_up) / 4);
    for (int e0 = 0; e0 < tot; e0 += 128) {
        float4 vu[4], vd[4];
        int s_[4], c_[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = e0 + 32 * q + lane;
            s_[q] = -1;
            c_[q] = 0;
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            vu[q] = z;
            vd[q] = z;
            if (e < tot) {
                const int s = e / qm, c4 = e - s * qm;
                const int lu = ku[s], ld = kd[s];
                s_[q] = s;
                c_[q] = c4;
                if (lu == 0) {
                    if (c4 < qu && ld > 0) vu[q] = Gv[(ld - 1) * qu + c4];
                    if (c4 < qd) vd[q] = unit4(ld - 1 - 4 * c4);
                } else {
                    if (c4 < qd) vd[q] = Gv[dn_off + (lu - 1) * qd + c4];
                    if (c4 < qu) vu[q] = unit4(lu - 1 - 4 * c4);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (s_[q] < 0) continue;
            if (c_[q] < qu) reinterpret_cast<float4 *>(Wu + (size_t)s_[q] * m.ld_up)[c_[q]] = vu[q];
            if (c_[q] < qd) reinterpret_cast<float4 *>(Wd + (size_t)s_[q] * m.ld_dn)[c_[q]] = vd[q];
        }
    }
}

cudaError_t launch_warp_convert(const DevModel &m, const DevBatch &b, bool to_compact, cudaStream_t stream) {
    if (!b.G32) return cudaErrorInvalidValue;
    const int grid = (b.n_walkers + 3) / 4;
    if (to_compact) warp_to_compact_kernel<<<grid, 128, 0, stream>>>(m, b);
    else warp_from_compact_kernel<<<grid, 128, 0, stream>>>(m, b);
    return cudaGetLastError();
}

int warp_walkers_max(const DevModel &m, int K, int optin) {
    const size_t cta = warp_cta_smem(m), per = warp_walker_smem(m, K);
    if (cta + per > (size_t)optin) return 0;
    return (int)std::min<size_t>(kWarpMaxWalkers, ((size_t)optin - cta) / per);
}

template <int K>
static cudaError_t launch_warp_t(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                 cudaStream_t stream) {
    const int wpb = p.warp_walkers;
    const size_t cta = warp_cta_smem(m), per = warp_walker_smem(m, K);
    const size_t sm = cta + (size_t)wpb * per;
    const int grid = (b.n_walkers + wpb - 1) / wpb;
    cudaError_t e = cudaFuncSetAttribute(sweep_warp_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    // shared memory no larger than the CTAs the launch can hold per SM need,
    // so that the rest of the SM's 256 KB stays L1, where the window's and the
    // column writes' G loads hit
    auto carve_for = [&](auto kernel, size_t smem) -> cudaError_t {
        cudaError_t r = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        int ctas = 0;
        if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, kernel, 32 * wpb, smem);
        if (r != cudaSuccess) return r;
        const size_t need = (size_t)std::max(ctas, 1) * (smem + 1024);
        const int carve = (int)std::min<size_t>(100, (need * 100 + 228 * 1024 - 1) / (228 * 1024));
        return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carve);
    };
    if ((e = carve_for(sweep_warp_kernel<K>, sm))) return e;
    if (K >= 8 && wpb <= kWarpWideWalkers) {
        // the register-rich kernel where it keeps as many CTAs per SM as the
        // capped one (shared memory already limits them: N = 216, 7 walkers
        // per CTA, one CTA per SM); not where its registers would halve them
        // (N = 96, 4 walkers per CTA)
        e = cudaFuncSetAttribute(sweep_warp_wide_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        if ((e = carve_for(sweep_warp_wide_kernel<K>, sm))) return e;
        int occ_wide = 0, occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_wide, sweep_warp_wide_kernel<K>, 32 * wpb, sm);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sweep_warp_kernel<K>, 32 * wpb, sm);
        if (e != cudaSuccess) return e;
        if (occ_wide >= occ && occ_wide > 0) {
            sweep_warp_wide_kernel<K><<<grid, 32 * wpb, sm, stream>>>(m, b, p, active, cta, per);
            return cudaGetLastError();
        }
    }
    sweep_warp_kernel<K><<<grid, 32 * wpb, sm, stream>>>(m, b, p, active, cta, per);
    return cudaGetLastError();
}

cudaError_t launch_sweep_warp(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                              cudaStream_t stream) {
    if (p.warp_walkers < 1 || p.warp_walkers > kWarpMaxWalkers || !b.G32 || !b.cond_max) return cudaErrorInvalidValue;
    switch (p.delay_k) {
        case 4: return launch_warp_t<4>(m, b, p, active, stream);
        case 8: return launch_warp_t<8>(m, b, p, active, stream);
        case 12: return launch_warp_t<12>(m, b, p, active, stream);
        case 16: return launch_warp_t<16>(m, b, p, active, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace kvmc
