// Internal interface between the host side of libkvmc (kvmc_api.cpp) and its
// CUDA kernels (kvmc_kernels.cu).  Not part of the public C ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace kvmc {

// The acceptance threshold fl(z / n_bonds) for one Z_mu = z, also encoded
// exactly as m * 2^(k - 53) (m = 0 encodes 0).  Filled on the host.
struct ThrEntry {
    double d;
    unsigned long long m;
    float f;
    int k;
};

// Device view of the model, shared by every walker.
struct DevModel {
    int n_sites;         // N
    int n_up, n_dn;      // orbitals per spin; n_up + n_dn == N
    int ld_up, ld_dn;    // padded row strides of W (multiples of 4)
    int n_bonds;
    const short2 *bonds; // [n_bonds] 0-based (i, j)
    const int *nbr_off;  // [N+1] CSR adjacency built from the bond list
    const short *nbr;    // [2*n_bonds]
    const double *U_up;  // row-major [N][n_up]
    const double *U_dn;  // row-major [N][n_dn]
    const ThrEntry *thr_table;  // [n_bonds + 1]
    // mixed real form: U as FP32 (high, low) pairs, hi = fl32(U), lo = fl32(U - hi),
    // row-major like U_up / U_dn (the FP32 refresh's residual); null otherwise
    const float *U32_up_hi, *U32_up_lo, *U32_dn_hi, *U32_dn_lo;
};

// Device view of the batch state.
struct DevBatch {
    int n_walkers;
    short *kappa_up;       // [W][N]  0 = empty, 1..n = label
    short *kappa_dn;       // [W][N]
    double *W64;           // plain form: [W][N*(ld_up+ld_dn)] (up block then down block)
    float *W32;            // mixed form: same layout in FP32
    long long *t;          // [W] proposals made (Philox counter)
    long long *t_end;      // [W] target counter for the running kvmc_sweep
    long long *acc_end;    // [W] target accepted count for the running kvmc_advance
    int *since;            // [W] accepted moves since the last refresh
    double *sum_e;         // [W]
    double *sum_e2;        // [W]
    long long *n_meas;     // [W]
    long long *accepted;   // [W]
    long long *proposals;  // [W]
    int *status;           // [W] bit flags (kStatus*)
    double *logdet;        // [W][4] from the last refresh: log|det| up, down,
                           // log(min|pivot|/max|pivot|) up, down
    float *drift;          // [W] max |W32_old - W64_new| at the last refresh
    double *energy_out;    // [W] scratch for kvmc_measure
    unsigned long long *refresh_count;  // [2] walker refreshes performed; FP32 refreshes redone in FP64
    double *solve_scratch; // FP64 rows being solved by the refresh: [W][2][solve_block]
    size_t solve_block;    // doubles per (walker, spin)
    double *lu_scratch;    // more than 160 orbitals: tilde_U factorised in HBM, [W][2][lu_block]
    size_t lu_block;       // doubles per (walker, spin), 0 when unused
    // real orbitals beyond 160: the FP64 LU's 1/diag [W][2][lu_aux_n] and pivot
    // order [W][2][lu_aux_n + 1] (the last entry: 1 when the LU succeeded), read
    // by the row solves that run in a separate launch; null when unused
    double *lu_invd;
    int *lu_perm;
    int lu_aux_n;
    // one-warp-per-walker sweep (kvmc_warp.cu): W's non-trivial rows indexed by
    // the other spin's label, [W][g_block] (null until that sweep is enabled)
    float *G32;
    size_t g_block;        // floats per walker: n_dn * ld_up + n_up * ld_dn
    float *cond_max;       // [W] largest |W| entry the warp sweep saw since the walker's last refresh
    int compact;           // 1 while a one-warp sweep call runs: FP32 refreshes write G32, not W32
};

enum : int {
    kStatusSingular = 1,
    kStatusNonFinite = 2,
    kStatusTimeout = 4,   // a bounded wait on the tensor cores gave up
    kStatusRefine = 8,    // the FP32 refresh did not converge: the FP64 refresh redoes the walker
};
// A walker stops with one of these set: its chain cannot continue.
constexpr int kStatusStop = kStatusSingular | kStatusNonFinite | kStatusTimeout;
// Proposals one sweep launch makes per walker at most, so that every launch
// ends in bounded time, a walker that can no longer accept a move included.
constexpr long long kLaunchProposals = 1ll << 18;
// kvmc_advance gives a walker at most this many proposals per requested
// accepted move (the typical rate is below ten).
constexpr long long kAdvanceProposalsPerMove = 1ll << 16;


struct SweepParams {
    unsigned long long seed;
    int accept_rule;      // 0 reference, 1 metropolis
    int refresh_every;    // mixed: accepted moves between refreshes
    int measure_every;    // proposals between energy samples
    int delay_k;          // mixed form: delayed-update depth (4, 8, 12, 16), else rank-1
    float drift_tol;      // delayed form: unit-row deviation that triggers an early refresh
    float drift_severe;   // delayed form: a deviation past this refreshes at once even within a call
    int stream_threads;   // W in HBM: threads per walker's CTA (128 or 256)
    int pipeline;         // delayed form: scan for the next move while the last one's factor column is written
    int tc_flush;         // W in HBM: rank-k flush on the tensor cores (tcgen05, 3xTF32)
    int refresh32;        // mixed real form: FP32 refresh by iterative refinement (1 per row, 2 tiled)
    int warp_walkers;     // mixed real form: > 0 = one warp per walker, this many walkers per CTA (kvmc_warp.cu)
    float cond_hi, cond_lo;  // warp sweep's accuracy guard (0 = off), see kvmc_warp.cu
    int cluster;          // mixed real form, rank-1: W split over a cluster of this many CTAs (0 = off)
};

// Launchers.  All enqueue on `stream` and return the launch error.
// only_due: 1 = refresh only walkers whose `since` is negative (marked due
// by the sweep kernel); 2 = only walkers flagged kStatusRefine.
// track_drift: record max |W_old - W_new| per walker.
cudaError_t launch_refresh(const DevModel &m, const DevBatch &b, bool fp32_out,
                           int only_due, int track_drift, cudaStream_t stream);
// mixed=false: plain FP64 form (W in global memory, refresh every
// p.refresh_every proposals).  mixed=true: FP32 form, refresh every
// p.refresh_every accepted moves; W staged in shared memory when smem_w,
// else kept in HBM (delayed updates when p.delay_k > 1, rank-1 in place
// otherwise).  active (device int) counts walkers left short of t_end.
cudaError_t launch_sweep(const DevModel &m, const DevBatch &b, const SweepParams &p,
                         bool mixed, bool smem_w, int *active, cudaStream_t stream);
cudaError_t launch_measure(const DevModel &m, const DevBatch &b, bool fp32, cudaStream_t stream);
cudaError_t launch_eval_ratios(const DevModel &m, const DevBatch &b, bool fp32, int n_moves,
                               const int *moves, double *out, cudaStream_t stream);
cudaError_t launch_apply_moves(const DevModel &m, const DevBatch &b, bool fp32,
                               const int *moves, cudaStream_t stream);
cudaError_t launch_set_tend(const DevBatch &b, long long proposals, long long moves, cudaStream_t stream);
cudaError_t launch_init_random(const DevModel &m, const DevBatch &b, unsigned long long seed,
                               const int *attempt, const int *redo, cudaStream_t stream);

// Shared-memory bytes the mixed sweep kernel needs for this model (0 if it
// cannot hold both W matrices on one SM).
size_t mixed_sweep_smem(const DevModel &m);
// Shared memory of the delayed-update sweep: with W on chip, or with W in
// HBM (only P, Q and the walker's small state on chip).
size_t delayed_smem_bytes(const DevModel &m, int K, bool w_on_chip);
// FP32 refresh by iterative refinement (kvmc_refresh32.cu), mixed real form:
// LU in shared memory up to 224 orbitals per spin, blocked in HBM beyond.  Walkers it could not converge carry
// kStatusRefine; launch_refresh with only_due == 2 redoes exactly those.
size_t refresh32_smem(const DevModel &m);
bool refresh32_supported(const DevModel &m);
cudaError_t launch_refresh32(const DevModel &m, const DevBatch &b, int only_due, int track_drift, cudaStream_t stream);
// more than 224 orbitals: the same refinement on an FP32 LU blocked in HBM (kvmc_kernels.cu)
cudaError_t launch_refresh32_large(const DevModel &m, const DevBatch &b, int only_due, int track_drift,
                                   cudaStream_t stream);
size_t refresh_large_smem(const DevModel &m, size_t lt_bytes);
// The same refinement with tiled solves and residual, one CTA per walker-spin
// (kvmc_refresh_tile.cu): only_due 0 or 1 as for launch_refresh32.
size_t refresh_tile_smem(const DevModel &m);
cudaError_t launch_refresh_tile(const DevModel &m, const DevBatch &b, int only_due, int track_drift,
                                cudaStream_t stream);
cudaError_t launch_clear_status(const DevBatch &b, int bits, cudaStream_t stream);
// Labels from and to the caller's 32-bit arrays (kvmc_refresh32.cu): the
// checks of kvmc_set_state per walker into bad[] (one warp per walker,
// labels_check_smem bytes of shared memory), and the conversion to or from
// the walkers' 16-bit labels.
constexpr int kLabelWarps = 8;
size_t labels_check_smem(int n_up, int n_dn);
cudaError_t launch_labels_check(const int32_t *ku, const int32_t *kd, int n_walkers, int N, int n_up, int n_dn,
                                int *bad, cudaStream_t stream);
cudaError_t launch_labels_convert(int32_t *ku, int32_t *kd, const DevBatch &b, int N, int to_short,
                                  cudaStream_t stream);
// The sums a sweep call reports, reduced on the device (kvmc_refresh32.cu):
// kCallStats doubles at `out`, laid out as call_stats_kernel documents.
constexpr int kCallStats = 16;
cudaError_t launch_call_stats(const DevBatch &b, double *out, cudaStream_t stream);

// The tiled refresh with its residual B - V M on the tensor cores
// (kvmc_refresh_oz.cu, KVMC_TUNE_REFRESH32 = 3).  U is split once per model
// into seven bf16 digit planes on a per-column fixed-point grid, V into four
// per row at every pass; the digit products are exact integer sums in FP32
// TMEM accumulators, one per weight class.  The buffers belong to the handle.
constexpr int kOzUDigits = 7;   // digit planes of U (48 bits below its column's scale)
constexpr int kOzVDigits = 4;   // digit planes of V (27 bits below its row's scale)
struct OzRefresh {
    int n_max, oth_max;          // max over the spins of n and of N - n
    int ldz;                     // row stride of V and R (floats): round4(n_max)
    int kp;                      // K (orbitals) padded to a multiple of 32
    int rows_v, rows_m;          // rows of the V planes (multiple of 128) and of M^T (multiple of 64)
    int tiles;                   // 32-row tiles of X per (walker, spin): ceil(oth_max / 32)
    const uint16_t *ud[2];       // per spin: U's digits, [kOzUDigits][N][n] bf16 bits, row-major by site
    const int *fexp[2];          // per spin: column scale exponents, [n]
    float *V;                    // [W*2][rows_v][ldz]
    uint16_t *vd;                // [W*2][kOzVDigits][kp/8][rows_v][8] bf16 bits
    uint16_t *mt;                // [W*2][kOzUDigits][kp/8][rows_m][8] bf16 bits: M^T's digits
    int cn, rows_g;              // columns of V per correction tile; rows of the G^T planes (multiple of cn)
    uint16_t *rd;                // [W*2][3][kp/8][rows_v][8] bf16 bits: R = r0 + r1 + r2
    uint16_t *gd;                // [W*2][3][kp/8][rows_g][8] bf16 bits: G^T = g0 + g1 + g2
    float *dmax, *vmax;          // [W*2][rows_v]: per row, max |R G| and max |V| of the pass
    int *vexp;                   // [W*2][rows_v] row scale exponents of V
    int *perm, *srow;            // [W*2][n_max] pivot order and the site of M's row i
    float *invd;                 // [W*2][n_max] 1 / diag of the LU's upper factor, in pivot order
    short *site_oth;             // [W*2][oth_max]
    float *dprev;                // [W*2][tiles] the last relative correction per tile
    int *done, *active;          // [W*2][tiles], [W*2]
    int n_ws;                    // walker-spins: 2 W
    int groups;                  // 128-row groups of the residual per (walker, spin): rows_v / 128
    int *tile_list, *grp_list;   // [2][W*2*tiles], [2][W*2*groups]: work of a pass (ping-pong)
    int *counts;                 // [4]: tiles and groups in list 0, tiles and groups in list 1
    int *grp_flag;               // [W*2*groups]: the group is in the next pass's list
    alignas(64) unsigned char tmap_v[128], tmap_m[128];   // CUtensorMap of vd and mt
    alignas(64) unsigned char tmap_r[128], tmap_g[128];   // CUtensorMap of rd and gd
};
size_t oz_scratch_bytes(const DevModel &m, int n_walkers);
bool oz_supported(const DevModel &m, int optin);
// U's digits for one spin on the host: `ud` receives kOzUDigits planes of
// N x n bf16 bits, `fexp` the n column exponents.
void oz_digits_host(const double *U, int N, int n, uint16_t *ud, int *fexp);
// Lays out the per-walker buffers in `scratch` (oz_scratch_bytes, zeroed by
// the caller) and encodes the tensor maps; ud / fexp must be set already.
cudaError_t oz_setup(const DevModel &m, int n_walkers, void *scratch, OzRefresh &oz);
cudaError_t launch_refresh_oz(const DevModel &m, const DevBatch &b, const OzRefresh &oz, int only_due,
                              int track_drift, int device, cudaStream_t stream);

// One warp per walker with W's non-trivial rows indexed by labels (kvmc_warp.cu).
size_t warp_cta_smem(const DevModel &m);
size_t warp_walker_smem(const DevModel &m, int K);
size_t warp_compact_block(const DevModel &m);
int warp_walkers_max(const DevModel &m, int K, int optin);
// W32 -> G32 (to_compact) or back, every walker; kvmc_warp.cu
cudaError_t launch_warp_convert(const DevModel &m, const DevBatch &b, bool to_compact, cudaStream_t stream);
cudaError_t launch_sweep_warp(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                              cudaStream_t stream);
// W's rows split over a thread-block cluster in distributed shared memory (kvmc_cluster.cu)
size_t sweep_cluster_smem(const DevModel &m, int cluster);
cudaError_t launch_sweep_cluster(const DevModel &m, const DevBatch &b, const SweepParams &p, int *active,
                                 cudaStream_t stream);

// Extra shared memory of the tensor-core flush (its operand tiles).
size_t tc_flush_smem_bytes();
size_t refresh_smem(const DevModel &m);
size_t refresh_scratch_block(const DevModel &m);
size_t refresh_large_smem(const DevModel &m);
bool refresh_needs_large(const DevModel &m);
int max_smem_optin(int device);

// Adjoint gradient estimator (kvmc_grad.cu).
constexpr int kMaxGradParams = 8;
struct GradModel {
    int n_params;
    const void *MT;     // [P][2][N][N] of the working scalar: MT[a][s][R'][R] = (dU_a,s U_s^H)[R, R']
    const void *W;      // the handle's W (W64 or W32)
    double *sums;       // [n_walkers][sum_stride], see kvmc_grad_sums
    size_t sum_stride;
    double *out;        // [n_walkers][2 + 2P]: E_L (re, im), then O_a (re, im); may be null
};
cudaError_t launch_grad(const DevModel &m, const DevBatch &b, const GradModel &g, bool mixed, bool complex_w, int rule,
                        cudaStream_t stream);

// Complex orbitals (kvmc_complex.cu).  U_up / U_dn then point at interleaved
// (re, im) pairs, W64 / W32 at complex FP64 / FP32 pairs, and solve_block
// counts doubles (two per complex entry).
int complex_max_orbitals();   // the shared-memory complex refresh's limit
bool complex_refresh_needs_large(const DevModel &m);   // beyond it: tilde_U factorised in HBM (lu_scratch)
size_t complex_delayed_smem(const DevModel &m, int K);   // mixed complex form, W in HBM
size_t complex_refresh_smem(const DevModel &m);
cudaError_t launch_refresh_c(const DevModel &m, const DevBatch &b, bool fp32_out, int only_due, int track_drift,
                             cudaStream_t stream);
cudaError_t launch_sweep_c(const DevModel &m, const DevBatch &b, const SweepParams &p, bool mixed, int *active,
                           cudaStream_t stream);
cudaError_t launch_measure_c(const DevModel &m, const DevBatch &b, bool fp32, cudaStream_t stream);
cudaError_t launch_eval_ratios_c(const DevModel &m, const DevBatch &b, bool fp32, int n_moves, const int *moves,
                                 double *out, cudaStream_t stream);
cudaError_t launch_apply_moves_c(const DevModel &m, const DevBatch &b, bool fp32, const int *moves,
                                 cudaStream_t stream);

}  // namespace kvmc
