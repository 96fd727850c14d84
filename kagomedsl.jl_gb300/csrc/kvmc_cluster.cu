// The mixed real form's rank-1 sweep with W split over a thread-block
// cluster in distributed shared memory (kvmc.h: KVMC_TUNE_CLUSTER).
//
// Reference counterpart: Carlo.sweep! with update_W! (KagomeDSL.jl
// src/MonteCarlo.jl:538-607, :279-292) and the measurement getOL
// (src/Hamiltonian.jl:762-778), as sweep_kernel<float> computes them.
//
// One cluster of C CTAs per walker.  CTA j keeps rows [j rp, (j+1) rp) of
// W_up and W_down (rp = ceil(N / C)) in its shared memory, so a W too large
// for one SM (N = 384: 590 KB) stays on chip.  Per proposal window:
//   1. CTA 0, warp 0, tests proposals t .. t+31 as sweep_kernel does; the two
//      W entries of a proposal are read from the CTA holding their rows
//      (ld.shared::cluster through map_shared_rank).
//   2. CTA 0 writes the outcome into every CTA's mailbox; cluster barrier.
//   3. On an accepted move every CTA reads the pivot rows W_up[Ku,:] and
//      W_down[Kd,:] from their owners; cluster barrier; every CTA updates its
//      own rows (W <- W - W[:,l] (W[K,:] - e_l) / W[K,l], the same FP32
//      operations as sweep_kernel<float>); CTA 0 updates kappa and Z_mu.
//   4. Cluster barrier; CTA 0 measures E_L when the cadence asks, reading W
//      entries from their owners.
// Every CTA passes the same barriers: the control flow after a barrier
// depends only on the mailbox, which CTA 0 wrote before it.
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "kvmc_device.cuh"
#include "kvmc_internal.h"

namespace cg = cooperative_groups;

namespace kvmc {

namespace {

constexpr int kClusterThreads = 256;

struct ClusterCtl {
    long long t, next_meas;
    int since, zmu, state;
    int Ku, lu, Kd, ld;
    Thr thr;
    double red[33];
};

struct Mailbox {
    long long t;
    int state;  // 1 = accepted move, 2 = stop, 3 = measurement boundary
    int Ku, lu, Kd, ld;
};

__host__ __device__ inline int rows_per_cta(int N, int C) { return (N + C - 1) / C; }

// Shared memory per CTA: its rows of both W blocks, the staged pivot rows and
// column factors, bonds and the configuration (the last two used by CTA 0).
__host__ __device__ inline size_t cluster_smem(const DevModel &m, int C) {
    const size_t rp = (size_t)rows_per_cta(m.n_sites, C);
    size_t s = rp * (m.ld_up + m.ld_dn) * 4;          // W rows
    s += (size_t)(m.ld_up + m.ld_dn) * 4;             // pivot rows
    s += 2 * rp * 4;                                   // column factors
    s += (size_t)m.n_bonds * 4;                        // bonds (short2)
    s += (size_t)2 * m.n_sites * 2 + 16;               // kappa up, down
    return (s + 15) / 16 * 16;
}

template <int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(kClusterThreads)
sweep_cluster_kernel(DevModel m, DevBatch b, SweepParams p, int *active_count) {
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int w = blockIdx.x / C;
    const int N = m.n_sites;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    const int rp = rows_per_cta(N, C);
    const int r0 = rank * rp;
    const int rows_here = max(0, min(rp, N - r0));
    const int ldu = m.ld_up, ldd = m.ld_dn;

    // every CTA reads the walker's progress before any CTA changes it
    const long long t0 = b.t[w];
    const long long tend_all = b.t_end[w];
    const long long tend = min(tend_all, t0 + kLaunchProposals);
    const long long acc_left = b.acc_end[w] - b.accepted[w];
    const bool idle = t0 >= tend || acc_left <= 0 || (b.status[w] & kStatusStop);
    cl.sync();
    if (idle) {
        if (rank == 0 && tid == 0 && b.since[w] < 0) b.since[w] = 0;
        return;
    }

    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Mailbox mbox;
    __shared__ ClusterCtl ctl;
    float *Wu = reinterpret_cast<float *>(smem);
    float *Wd = Wu + (size_t)rp * ldu;
    float *row_u = Wd + (size_t)rp * ldd;
    float *row_d = row_u + ldu;
    float *col_u = row_d + ldd;
    float *col_d = col_u + rp;
    short2 *bonds = reinterpret_cast<short2 *>(col_d + rp);
    short *kup = reinterpret_cast<short *>(bonds + m.n_bonds);
    short *kdn = kup + N;

    // this CTA's rows of W (FP32, site-indexed)
    const float *gW = b.W32 + (size_t)w * N * (ldu + ldd);
    for (int e = tid; e < rows_here * ldu; e += nt) Wu[e] = gW[(size_t)r0 * ldu + e];
    for (int e = tid; e < rows_here * ldd; e += nt) Wd[e] = gW[(size_t)N * ldu + (size_t)r0 * ldd + e];
    // entry (r, c) of either block, in the shared memory of the CTA holding row r
    auto wu_at = [&](int r, int c) -> float * {
        const int o = r / rp;
        return cl.map_shared_rank(Wu, o) + (size_t)(r - o * rp) * ldu + c;
    };
    auto wd_at = [&](int r, int c) -> float * {
        const int o = r / rp;
        return cl.map_shared_rank(Wd, o) + (size_t)(r - o * rp) * ldd + c;
    };

    const int R = p.refresh_every;
    const int M = p.measure_every;
    if (rank == 0) {
        for (int e = tid; e < m.n_bonds; e += nt) bonds[e] = m.bonds[e];
        for (int s = tid; s < N; s += nt) {
            kup[s] = b.kappa_up[(size_t)w * N + s];
            kdn[s] = b.kappa_dn[(size_t)w * N + s];
        }
        __syncthreads();
        double zc = 0.0;
        for (int e = tid; e < m.n_bonds; e += nt) {
            const short2 bd = bonds[e];
            zc += ((kup[bd.x] != 0 && kdn[bd.y] != 0) || (kup[bd.y] != 0 && kdn[bd.x] != 0)) ? 1.0 : 0.0;
        }
        zc = block_sum(zc, ctl.red);
        if (tid == 0) {
            ctl.t = t0;
            ctl.since = b.since[w] < 0 ? 0 : b.since[w];
            ctl.zmu = (int)zc;
            ctl.next_meas = (t0 / M + 1) * M;
            make_thr(ctl.thr, m.thr_table, ctl.zmu, p.accept_rule);
        }
    }
    // W rows in place in every CTA before anyone reads them remotely
    cl.sync();

    long long acc_count = 0, n_meas = 0;
    double se = 0.0, se2 = 0.0;
    while (true) {
        if (rank == 0) {
            if (warp == 0) {
                long long t = ctl.t;
                const int since = ctl.since;
                const long long next_meas = ctl.next_meas;
                const Thr thr = ctl.thr;
                int state = 2;
                while (true) {
                    if (t >= tend || acc_count >= acc_left || since >= R) break;
                    const long long lim = min(tend, next_meas) - t;
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
                                acc = decide(*wu_at(Ku, lu), *wd_at(Kd, ld), u53, c, thr, p.accept_rule, bad);
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
                    if (t == next_meas) { state = 3; break; }
                }
                if (lane == 0) { ctl.t = t; ctl.state = state; }
            }
            __syncthreads();
            if (tid < C) {
                Mailbox *mb = cl.map_shared_rank(&mbox, tid);
                mb->t = ctl.t;
                mb->state = ctl.state;
                mb->Ku = ctl.Ku; mb->lu = ctl.lu; mb->Kd = ctl.Kd; mb->ld = ctl.ld;
            }
        }
        cl.sync();
        const int state = mbox.state;
        if (state == 2) break;
        if (state == 1) {
            const int Ku = mbox.Ku, lu = mbox.lu, Kd = mbox.Kd, ld = mbox.ld;
            // the pivot rows from their owners, as sweep_kernel's staging
            const float au = -1.0f / *wu_at(Ku, lu);
            const float ad = -1.0f / *wd_at(Kd, ld);
            for (int c = tid; c < ldu; c += nt) row_u[c] = *wu_at(Ku, c) - (c == lu ? 1.f : 0.f);
            for (int c = tid; c < ldd; c += nt) row_d[c] = *wd_at(Kd, c) - (c == ld ? 1.f : 0.f);
            for (int r = tid; r < rows_here; r += nt) {
                col_u[r] = Wu[(size_t)r * ldu + lu] * au;
                col_d[r] = Wd[(size_t)r * ldd + ld] * ad;
            }
            // every CTA holds its copies before any row changes
            cl.sync();
            const int qu = ldu >> 2, qd = ldd >> 2;
            const int tot_u = rows_here * qu, tot = tot_u + rows_here * qd;
            for (int e = tid; e < tot; e += nt) {
                const bool is_up = e < tot_u;
                const int ee = is_up ? e : e - tot_u;
                const int q = is_up ? qu : qd;
                const int r = ee / q, c4 = ee - r * q;
                float4 *wp = reinterpret_cast<float4 *>(is_up ? Wu : Wd) + (size_t)r * q + c4;
                const float cv = is_up ? col_u[r] : col_d[r];
                const float4 rv = reinterpret_cast<const float4 *>(is_up ? row_u : row_d)[c4];
                float4 v = *wp;
                v.x = fmaf(cv, rv.x, v.x);
                v.y = fmaf(cv, rv.y, v.y);
                v.z = fmaf(cv, rv.z, v.z);
                v.w = fmaf(cv, rv.w, v.w);
                *wp = v;
            }
            if (rank == 0 && tid == 0) {
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
        }
        // every row updated before the next window or measurement reads it
        cl.sync();
        if (rank == 0 && mbox.t == ctl.next_meas) {
            // E_L (src/Hamiltonian.jl:593-778), W entries read from their owners
            float accf = 0.f;
            for (int e = tid; e < m.n_bonds; e += nt) {
                const short2 bd = bonds[e];
                const int i = bd.x, j = bd.y;
                const int ui = kup[i], uj = kup[j], di = kdn[i], dj = kdn[j];
                accf += ((ui != 0) == (uj != 0)) ? 0.25f : -0.25f;
                if (uj != 0 && di != 0) accf -= 0.5f * *wu_at(i, uj - 1) * *wd_at(j, di - 1);
                if (ui != 0 && dj != 0) accf -= 0.5f * *wu_at(j, ui - 1) * *wd_at(i, dj - 1);
            }
            const double e = block_sum_f32(accf, ctl.red);
            if (tid == 0) {
                se += e;
                se2 += e * e;
                n_meas += 1;
                ctl.next_meas += M;
            }
            __syncthreads();
        }
    }
    // write back this CTA's rows; CTA 0 the configuration and counters
    float *gWo = b.W32 + (size_t)w * N * (ldu + ldd);
    for (int e = tid; e < rows_here * ldu; e += nt) gWo[(size_t)r0 * ldu + e] = Wu[e];
    for (int e = tid; e < rows_here * ldd; e += nt) gWo[(size_t)N * ldu + (size_t)r0 * ldd + e] = Wd[e];
    if (rank == 0) {
        for (int s = tid; s < N; s += nt) {
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
    // no CTA leaves while another may still read its shared memory
    cl.sync();
}

template <int C>
cudaError_t launch_cluster_t(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                             cudaStream_t stream) {
    const size_t sm = cluster_smem(m, C);
    cudaError_t e = cudaFuncSetAttribute(sweep_cluster_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    sweep_cluster_kernel<C><<<b.n_walkers * C, kClusterThreads, sm, stream>>>(m, b, p, active);
    return cudaGetLastError();
}

}  // namespace

size_t sweep_cluster_smem(const DevModel &m, int cluster) { return cluster_smem(m, cluster); }

cudaError_t launch_sweep_cluster(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                 cudaStream_t stream) {
    if (p.cluster == 2) return launch_cluster_t<2>(m, b, p, active, stream);
    if (p.cluster == 4) return launch_cluster_t<4>(m, b, p, active, stream);
    return cudaErrorInvalidValue;
}

}  // namespace kvmc
