/*
 * kvmc.h -- C ABI of libkvmc, the GB300 (sm_103a) variational Monte Carlo
 * engine for Gutzwiller-projected parton states of the kagome Heisenberg
 * model.  It drops in for the hot path of KagomeDSL.jl: the Monte Carlo
 * driver callbacks (init!, sweep!, measure!, checkpoint I/O) and the
 * lattice / hopping-matrix constructors.
 *
 * Conventions
 *  - Every function returns int status: KVMC_OK (0) or a kvmc_status code;
 *    kvmc_last_error() gives the message.  No function aborts the process.
 *  - Site indices are 0-based.  Configuration vectors ("kappa") keep the
 *    reference's values: 0 = site empty for that spin, 1..n = orbital label
 *    (src/MonteCarlo.jl:92-135), so a Julia Vector{Int} passes through after
 *    conversion to Int32 only.
 *  - Orbital matrices U are column-major (Julia layout), n_sites x n.
 *  - A handle owns all device memory it uses; calls on one handle are
 *    synchronous with respect to the host and a handle is not thread-safe.
 *  - Per-walker arrays are walker-major: [n_walkers][n_sites].
 */
#ifndef KVMC_H
#define KVMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define KVMC_API __attribute__((visibility("default")))
#else
#define KVMC_API
#endif

#define KVMC_ABI_VERSION 4

enum kvmc_status {
    KVMC_OK = 0,
    KVMC_ERR_ARGUMENT = 1,  /* ArgumentError / AssertionError / DimensionMismatch */
    KVMC_ERR_BOUNDS = 2,    /* BoundsError */
    KVMC_ERR_SINGULAR = 3,  /* singular tilde_U (SingularException, singular init) */
    KVMC_ERR_CUDA = 4,      /* CUDA runtime failure */
    KVMC_ERR_NUMERIC = 5,   /* non-finite ratio or W detected by a kernel */
    KVMC_ERR_NO_DEVICE = 6, /* no usable sm_103 device */
    KVMC_ERR_UNSUPPORTED = 7
};

enum kvmc_precision {
    KVMC_PLAIN_FP64 = 0, /* reference algorithm: FP64 W, rank-1 per accepted move,
                            refresh every refresh_interval proposals */
    KVMC_MIXED_FP32 = 1  /* FP32 W resident in shared memory, FP64 refresh every
                            refresh_interval accepted moves, FP64 energy sums */
};

/* Where the mixed form keeps each walker's FP32 W.  On chip, one walker
 * owns an SM's shared memory for its launch (fits up to N = 216).  In HBM,
 * only the delayed-update factors P, Q are on chip, so several walkers share
 * an SM, and the rank-k flush streams W through once per k moves. */
enum kvmc_w_placement {
    KVMC_W_AUTO = 0,    /* on chip when it fits, else HBM */
    KVMC_W_ON_CHIP = 1,
    KVMC_W_HBM = 2
};

enum kvmc_accept {
    KVMC_ACCEPT_REFERENCE = 0, /* src/MonteCarlo.jl:544-591: stationary law |psi|^2/Z_mu */
    KVMC_ACCEPT_METROPOLIS = 1 /* uniform bond + min(1,|ratio|^2): stationary law |psi|^2 */
};

/* ---- lattice and hopping matrix (host FP64) ---------------------------- */

typedef struct {
    int32_t n1, n2;     /* DoubleKagome repetitions, n1 even (src/Lattice.jl:68-92) */
    int32_t pbc[2];     /* periodic along a1, a2 */
    int32_t antipbc[2]; /* antiperiodic along a1, a2 (requires pbc) */
    double t;           /* triangle side parameter, 1.0 in the reference */
} kvmc_lattice_desc;

/* One hopping table entry.  In-cell tables (src/Hamiltonian.jl:219-235) use
 * label1, label2 only; inter-cell tables (src/Hamiltonian.jl:250-261) also
 * use the cell offset (dx, dy).  Labels are 1..6 as in the reference. */
typedef struct {
    int32_t label1, label2, dx, dy;
    double amplitude;
} kvmc_link;

/* Number of sites n1*n2*3 (src/Lattice.jl:97).  Replaces ns(lat). */
KVMC_API int kvmc_lattice_sites(const kvmc_lattice_desc *lat, int32_t *n_sites);

/* Spinon hopping matrix H = -(T + T^dagger) with Peierls phase and
 * (anti)periodic images.  Replaces Hmat (src/Hamiltonian.jl:308-354) with
 * get_boundary_shifts / apply_boundary_conditions! (:99-207).
 * link_in / link_inter may be NULL for the reference's pi-flux tables.
 * H receives 2*N*N doubles: column-major, (re, im) interleaved. */
KVMC_API int kvmc_hopping_matrix(const kvmc_lattice_desc *lat,
                        const kvmc_link *link_in, int32_t n_link_in,
                        const kvmc_link *link_inter, int32_t n_link_inter,
                        double B, double *H);

/* Bond list: upper-triangular nonzeros of H in column-major order, 0-based
 * (i < j).  Replaces get_nn (src/Hamiltonian.jl:447-451).  Pass bonds=NULL to
 * query the count. */
KVMC_API int kvmc_bonds_from_hopping(int32_t n_sites, const double *H, int32_t *n_bonds,
                            int32_t *bonds);

/* Extended mean-field ansatz with three real variational parameters
 * params = {t2, m, theta}.  No reference counterpart: the reference has the
 * pi-flux hopping only; this is the parameterised family whose energy
 * gradient the adjoint entry points below measure.  On top of the pi-flux H
 * of kvmc_hopping_matrix (same tables, boundary conditions and field B):
 *   theta: each nearest-neighbour hop i->j is multiplied by
 *          exp(i*theta*s_ij/3), s_ij = +1 when i->j runs counter-clockwise
 *          around its triangle; every triangle then carries flux theta and
 *          every hexagon pi - 2*theta;
 *   t2, m: second-neighbour hops i->k (the two ends of a bent path i->j->k
 *          around a hexagon corner, |r_k - r_i| = sqrt(3) t) get
 *          H_ik += -(t2 + i*m*nu_ijk) * g_ijk, where g_ijk = sign(H0_ij H0_jk)
 *          carries the pi-flux gauge of the path and nu_ijk = +1 (-1) for a
 *          left (right) turn at j: a chiral mass of opposite sign on the two
 *          orientations.  Second-neighbour hops carry no Peierls phase.
 * H: 2*N*N doubles as kvmc_hopping_matrix.  dH (may be NULL): 3 matrices
 * dH/dt2, dH/dm, dH/dtheta in the same layout, 6*N*N doubles.  The
 * Heisenberg bonds stay the nearest-neighbour ones: take them from
 * kvmc_bonds_from_hopping on the params = 0 matrix. */
KVMC_API int kvmc_ansatz_hopping(const kvmc_lattice_desc *lat,
                        const kvmc_link *link_in, int32_t n_link_in,
                        const kvmc_link *link_inter, int32_t n_link_inter,
                        double B, const double *params, double *H, double *dH);

/* ---- batched Monte Carlo state ----------------------------------------- */

typedef struct {
    int32_t n_sites;
    int32_t n_up, n_down;  /* n_up + n_down == n_sites (one spinon per site) */
    int32_t n_bonds;
    const int32_t *bonds;  /* [n_bonds][2], 0-based, as kvmc_bonds_from_hopping */
    const double *U_up;    /* column-major n_sites x n_up (real parts of the orbitals) */
    const double *U_down;  /* column-major n_sites x n_down */
    /* Imaginary parts, same layout; both NULL for real orbitals (B = 0).  A
     * non-NULL pointer makes the handle complex, as the reference's
     * ComplexF64 W for B != 0 (src/Hamiltonian.jl:201-204, :325-327).  A
     * complex handle refreshes W in FP64, tilde_U factorised in shared
     * memory up to 112 orbitals per spin and blocked in HBM beyond; its
     * mixed form takes delay_k 1 (rank-1), 4 or 8 (W in HBM). */
    const double *U_up_imag;
    const double *U_down_imag;
} kvmc_model_desc;

typedef struct {
    int32_t n_walkers;
    int32_t precision;        /* enum kvmc_precision */
    int32_t accept_rule;      /* enum kvmc_accept */
    int32_t refresh_interval; /* plain: proposals, mixed: accepted moves; 0 = default
                                 (plain: min(n_up,n_down) as src/MonteCarlo.jl:594-595) */
    int32_t measure_interval; /* proposals between local-energy samples; 0 = min(n_up,n_down)
                                 (src/MonteCarlo.jl:628-634) */
    int32_t delay_k;          /* mixed form: delayed-update depth; 0 = the largest of
                                 16, 12, 8, 4 whose working set fits in shared memory,
                                 1 = a rank-1 update per accepted move */
    int32_t device;           /* CUDA device ordinal */
    uint64_t seed;            /* Philox4x32-10 key for proposals and seeded starts */
    int32_t w_placement;      /* mixed form, enum kvmc_w_placement */
} kvmc_batch_desc;

typedef struct kvmc_handle kvmc_handle;

/* Replaces MC(params) (src/MonteCarlo.jl:165-185, :209-234): uploads the
 * orbitals and bonds and allocates every walker's state on the device. */
KVMC_API int kvmc_create(const kvmc_model_desc *model, const kvmc_batch_desc *batch,
                kvmc_handle **out);
KVMC_API int kvmc_destroy(kvmc_handle *h);

/* Message of the last failure on h (or of the last failed kvmc_create when
 * h is NULL). */
KVMC_API int kvmc_last_error(const kvmc_handle *h, char *buf, size_t len);

/* Replaces Carlo.init! (src/MonteCarlo.jl:435-441) and
 * find_initial_configuration! (:382-410).  With kappa_up == NULL every
 * walker draws a seeded uniformly random configuration, redrawn until
 * tilde_U is regular for both spins (min|pivot|/max|pivot| of its partially
 * pivoted LU above 1e-8); otherwise the given configurations
 * ([n_walkers][n_sites]) are validated and used.  Seeded starts build W
 * in FP64; given configurations are rebuilt like kvmc_set_state.  attempts
 * (may be NULL) receives the draws each walker needed.
 * Returns KVMC_ERR_SINGULAR if a given configuration is singular. */
KVMC_API int kvmc_init(kvmc_handle *h, const int32_t *kappa_up, const int32_t *kappa_down,
              int32_t *attempts);

typedef struct {
    int64_t proposals;    /* proposals made by all walkers in the call */
    int64_t accepted;     /* accepted moves of all walkers in the call */
    int64_t measurements; /* local-energy samples taken in the call */
    double sum_energy;    /* sum of those samples (FP64) */
    double sum_energy2;   /* sum of their squares */
    int64_t refreshes;    /* walker W refreshes performed */
    double max_drift;     /* mixed: max |W_fp32 - W_fp64 fresh| seen at a refresh */
    int32_t bad_walkers;  /* walkers whose status word is nonzero */
    int32_t launches;     /* kernels launched by the call */
    int64_t fp64_redos;   /* refreshes the FP32 refinement handed to the FP64 refresh */
} kvmc_sweep_stats;

/* Replaces Carlo.sweep! (src/MonteCarlo.jl:538-607) plus the cadenced
 * Carlo.measure! (:628-634): every walker makes exactly
 * proposals_per_walker exchange proposals, refreshing W and sampling the
 * local energy at the configured intervals.  stats may be NULL. */
KVMC_API int kvmc_sweep(kvmc_handle *h, int64_t proposals_per_walker, kvmc_sweep_stats *stats);

/* Like kvmc_sweep, but every walker runs until it has made
 * moves_per_walker more accepted moves (the measurement and refresh
 * cadences are unchanged).  Equal accepted work per walker keeps the
 * batch's launches balanced.  A walker gets at most 65536 proposals per
 * requested move; one that cannot make its moves within them (a
 * configuration no proposal leaves) ends the call with KVMC_ERR_NUMERIC,
 * the other walkers' moves made.  Walkers flagged singular or non-finite
 * stop at once, and the call reports them. */
KVMC_API int kvmc_advance(kvmc_handle *h, int64_t moves_per_walker, kvmc_sweep_stats *stats);

/* Local energy of every walker's current state (getOL,
 * src/Hamiltonian.jl:762-778), FP64 result: local_energy[n_walkers]. */
KVMC_API int kvmc_measure(kvmc_handle *h, double *local_energy);

/* Determinant ratios W_up[K_up, l_up] * W_down[K_down, l_down] for given
 * moves, read from the device W (src/MonteCarlo.jl:576-580).
 * moves: [n_walkers][n_moves][4] = {K_up, l_up, K_down, l_down}, sites
 * 0-based, labels 1-based; ratios: [n_walkers][n_moves], or
 * [n_walkers][n_moves][2] as (re, im) for a complex handle. */
KVMC_API int kvmc_eval_ratios(kvmc_handle *h, int32_t n_moves, const int32_t *moves,
                     double *ratios);

/* Applies one exchange per walker through the device update path
 * (update_configurations!, src/MonteCarlo.jl:497-511 with update_W!,
 * :279-292).  moves: [n_walkers][5] = {flag, i, site, l_up, l_down};
 * flag 1 or 2 as in the reference, 0 = leave the walker unchanged; sites
 * 0-based, labels 1-based. */
KVMC_API int kvmc_apply_moves(kvmc_handle *h, const int32_t *moves);

/* Rebuilds every walker's W from its configuration in FP64
 * (reevaluateW!, src/MonteCarlo.jl:55-66). */
KVMC_API int kvmc_refresh(kvmc_handle *h);

/* Checkpoint state (write_checkpoint / read_checkpoint!,
 * src/MonteCarlo.jl:715-755): configurations plus the per-walker proposal
 * counter (the position in the Philox stream).  set_state rebuilds W.
 * Any pointer may be NULL to skip that field (set_state: counters NULL
 * keeps the current counters).  kvmc_set_state rebuilds W: in FP64, or for
 * the mixed real form with KVMC_TUNE_REFRESH32 by FP32 refinement.  A label
 * out of range (KVMC_ERR_BOUNDS), a label used twice or a site empty or
 * doubly occupied (KVMC_ERR_ARGUMENT) in any walker leaves every walker's
 * state as it was; the error names the first such walker and site. */
KVMC_API int kvmc_get_state(kvmc_handle *h, int32_t *kappa_up, int32_t *kappa_down,
                   int64_t *counters);
KVMC_API int kvmc_set_state(kvmc_handle *h, const int32_t *kappa_up, const int32_t *kappa_down,
                   const int64_t *counters);

/* Copies W to the host as FP64, row-major [n_walkers][n_sites][n]; a
 * complex handle writes [n_walkers][n_sites][n][2] as (re, im). */
KVMC_API int kvmc_get_w(kvmc_handle *h, double *W_up, double *W_down);

/* Per-walker accumulators since creation or the last kvmc_reset_stats:
 * sums of E_L and E_L^2, sample counts, accepted moves, proposals, status
 * words.  Any pointer may be NULL. */
KVMC_API int kvmc_walker_stats(kvmc_handle *h, double *sum_e, double *sum_e2, int64_t *n_meas,
                      int64_t *accepted, int64_t *proposals, int32_t *status);
KVMC_API int kvmc_reset_stats(kvmc_handle *h);

/* Each walker's largest relative W drift, max |W_fp32 - W_fp64| / (1 + |W_fp64|),
 * seen by the refreshes of the last kvmc_sweep / kvmc_advance call (0 when
 * the walker was not refreshed).  drift: [n_walkers]. */
KVMC_API int kvmc_walker_drift(kvmc_handle *h, float *drift);

/* Mixed form with delayed updates: after a flush of the K pending moves
 * (every fourth flush in the pipelined form) the rows of W at occupied
 * sites, which are exact unit rows in exact arithmetic, are compared with
 * their exact values; a walker whose largest deviation exceeds tol is
 * refreshed before its refresh_interval accepted moves are up: at the end of
 * the kvmc_advance call when the moves it still owes that call are fewer
 * than refresh_interval (so refreshes stay on call boundaries) and the
 * deviation is below max(100 tol, 1e-2), otherwise at once.  Default 1e-4. */
KVMC_API int kvmc_set_drift_tolerance(kvmc_handle *h, double tol);

/* Device-side timing of the kernels launched by kvmc_sweep, measured with
 * CUDA events on the handle's stream (enable before the calls to time).
 * kind: 0 = sweep kernel, 1 = refresh kernel, 2 = adjoint kernel
 * (kvmc_measure_grad).  Totals since enabling. */
KVMC_API int kvmc_enable_timing(kvmc_handle *h, int32_t on);
KVMC_API int kvmc_kernel_time(kvmc_handle *h, int32_t kind, double *total_ms, int64_t *launches);

/* Launch-shape knobs the autotuner sets (kagomevmc.autotune):
 *   KVMC_TUNE_STREAM_THREADS: threads per walker's CTA when W is in HBM,
 *   128 (four walkers per SM) or 256 (two walkers per SM, the default).
 *   KVMC_TUNE_PIPELINE: 1 = with delayed updates, one warp scans for the next
 *   accepted move while the others write the factor column of the last one
 *   (the scan applies that move as a Sherman-Morrison correction), the
 *   default; 0 = the two phases one after the other.
 *   KVMC_TUNE_TC_FLUSH: 1 = with W in HBM, the rank-k flush W -= P Q^T runs
 *   on the tensor cores (tcgen05, TF32 operands split in high and low parts,
 *   three products accumulated in FP32 in tensor memory); 0 = FP32 FMA.
 *   KVMC_TUNE_REFRESH32: 1 = the periodic refresh of the FP32 W runs as
 *   iterative refinement on the FP32 pipes (FP32 LU and solves, residual
 *   with exact products and compensated sums), walkers that do not converge
 *   falling back to the FP64 refresh; 2 = the same refinement with the
 *   solves and the residual in tiles of 32 rows, one CTA per walker and
 *   spin; 3 = the same refinement batched over all walkers with both
 *   products of each pass on the tensor cores -- the residual B - V M from
 *   exact bf16 digit products (V and U split on fixed-point grids, integer
 *   sums in FP32 tensor memory), the correction V += R G from three bf16
 *   parts of each factor -- with up to 12 passes; the handle then holds
 *   about 90 * n^2 bytes more per walker (16 MB at 432 orbitals per spin;
 *   fewer than 1024 orbitals per spin);
 *   0 = FP64 LU and solves.  It also
 *   rebuilds W in kvmc_set_state and kvmc_init with given configurations
 *   (log|det| then from the FP32 factors); seeded starts and kvmc_refresh
 *   always use FP64.  The default for the mixed real form is 1 below 96
 *   orbitals per spin, 2 from 96 on (while the tiles fit in shared memory)
 *   and 3 from 192 on; 0 for the other forms.
 *   KVMC_TUNE_WARP_WALKERS: 0 = one CTA per walker (the kernels above);
 *   1..14 = one warp per walker, this many walkers per CTA (mixed real form
 *   with delay_k 4..16).  Each warp keeps only W's non-trivial rows -- the
 *   rows at the sites of the other spin, indexed by that spin's label --
 *   so a flush touches half of W; the handle then holds an extra
 *   n_walkers * 2 * n_up * n_down floats for them.
 *   KVMC_TUNE_COND_HI, KVMC_TUNE_COND_LO: the one-warp sweep's accuracy
 *   guard.  FP32 W loses accuracy while it carries large entries (near a
 *   node of the wave function) and shows it once they shrink again: a walker
 *   whose largest |W| entry read by its moves has exceeded COND_HI since its
 *   last refresh is refreshed when a move's entries are all below COND_LO --
 *   at the end of the kvmc_advance call (or of its segment) when the moves it
 *   still owes are fewer than refresh_interval, else at once.  0 turns the
 *   guard off (the default).
 *   KVMC_TUNE_SEGMENT: one-warp mode: kvmc_advance runs its moves in
 *   segments of this many accepted moves per walker, so a refresh the guard
 *   asks for waits at most one segment; 0 = the whole call (the default).
 *   KVMC_TUNE_DRIFT_SEVERE: one CTA per walker with delayed updates: a
 *   unit-row deviation past the drift tolerance refreshes the walker at the
 *   end of the kvmc_advance call when its remaining moves fit in an
 *   interval, unless it is past the severe threshold, which refreshes at
 *   once.  value > 0 sets that threshold to value tolerances; 0 (the
 *   default) to max(100 tolerances, 1e-2).
 *   KVMC_TUNE_CLUSTER: 0 (the default) or 2 / 4 = the mixed real form with
 *   rank-1 updates (delay_k 1) keeps W on chip split over a thread-block
 *   cluster of that many CTAs per walker (rows by site blocks in each CTA's
 *   shared memory, read by the others over distributed shared memory). */
enum kvmc_tuning { KVMC_TUNE_STREAM_THREADS = 1, KVMC_TUNE_PIPELINE = 2, KVMC_TUNE_TC_FLUSH = 3,
                   KVMC_TUNE_REFRESH32 = 4, KVMC_TUNE_WARP_WALKERS = 5, KVMC_TUNE_COND_HI = 6,
                   KVMC_TUNE_COND_LO = 7, KVMC_TUNE_SEGMENT = 8, KVMC_TUNE_DRIFT_SEVERE = 9,
                   KVMC_TUNE_CLUSTER = 10 };
KVMC_API int kvmc_set_tuning(kvmc_handle *h, int32_t key, int32_t value);

/* The settings a handle resolved at creation: refresh and measurement
 * intervals, delayed-update depth, and whether W is staged on chip. */
KVMC_API int kvmc_get_config(kvmc_handle *h, int32_t *refresh_interval, int32_t *measure_interval,
                             int32_t *delay_k, int32_t *w_on_chip);

/* Device time of everything the handle enqueues between a call with
 * start=1 and a call with start=0 (CUDA events on the handle's stream);
 * the second call waits for the stream and returns the milliseconds. */
KVMC_API int kvmc_region_timer(kvmc_handle *h, int32_t start, double *ms);

/* Refresh that allocates nothing.  No counterpart in the reference.  It
 * computes W = U * tilde_U^{-1} in FP64, one configuration per batch item,
 * for callers that cannot allocate device memory: code whose GPU memory is
 * owned by another allocator (a Julia CUDA.jl pool, a framework's caching
 * allocator) or that must not trigger cudaMalloc's device synchronisation
 * inside its Monte Carlo loop.
 *
 * Inputs and outputs are the caller's device buffers:
 *   U       [n_sites][n_orb] FP64, row-major (row R = orbital amplitudes at site R)
 *   kappa   [batch][n_sites] int32, 0 or 1..n_orb, exactly n_orb nonzero
 *   W       [batch][n_sites][n_orb] FP64 out, row-major
 *   logdet  [batch] FP64 out (may be NULL): log|det tilde_U|; -inf when
 *           tilde_U is singular (a repeated or out-of-range label makes it
 *           so), NaN when kappa does not have n_orb occupied sites.  In both
 *           cases W of that item is left untouched.
 * The rows being solved use a fixed 8 MiB array inside the library, held by
 * every GPU that loads it until the process exits; a call needs
 * batch * n_orb * (n_sites - n_orb) * 8 <= 8 MiB (KVMC_ERR_ARGUMENT
 * otherwise) and n_orb <= 160 (KVMC_ERR_UNSUPPORTED).  No call allocates:
 * no cudaMalloc, cudaFree or allocating library routine.
 * A call outside stream capture resolves the array's device address and
 * the kernel's shared-memory limit for the current device's context; a call
 * under capture reuses what the last call outside capture on that device
 * resolved, so make one call on each device before capturing.  The kernel
 * is enqueued on `stream` (a cudaStream_t, NULL for the legacy default
 * stream) on the current device and the call returns without waiting.
 * Every call shares the one array, so calls that overlap on the GPU
 * (different streams, or the same buffers in flight) race: the caller must
 * serialise them.  The array keeps the last call's contents; nothing in it
 * needs to start at zero, since every element a call reads it first writes. */
KVMC_API int kvmc_refresh_static(int32_t n_sites, int32_t n_orb, int32_t batch, const double *U,
                                 const int32_t *kappa, double *W, double *logdet, void *stream);

/* ---- groups: walkers of different lattice sizes in one graph launch -----
 * No reference counterpart (the reference runs one chain per Carlo task).
 * A group advances several handles -- typically one per lattice size, each
 * with its own delayed-update depth and refresh interval -- together: one
 * captured CUDA graph forks into every handle's stream, runs its
 * (sweep, refresh) launches concurrently with the others, and joins.  The
 * graph is captured on the first call and reused while the handles' settings
 * do not change.  Handles keep working on their own between group calls. */
typedef struct kvmc_group kvmc_group;
KVMC_API int kvmc_group_create(kvmc_handle *const *handles, int32_t n, kvmc_group **out);
KVMC_API int kvmc_group_destroy(kvmc_group *g);
/* Every walker of every handle makes moves_per_walker more accepted moves.
 * stats: [n] per-handle statistics (may be NULL); ms: device time of the
 * graph launches (may be NULL). */
KVMC_API int kvmc_group_advance(kvmc_group *g, int64_t moves_per_walker, kvmc_sweep_stats *stats, double *ms);
KVMC_API int kvmc_group_last_error(const kvmc_group *g, char *buf, size_t len);

/* ---- adjoint gradient over ansatz parameters ---------------------------
 * No reference counterpart (the reference measures the energy only).  For P
 * real parameters a with orbital derivatives dU_a = dU/da (from first-order
 * eigenvector perturbation of kvmc_ansatz_hopping's H and dH, computed on the
 * host), the estimator takes per configuration the log-derivatives
 * O_a = d ln psi / d a = sum_spin tr(tilde_U^{-1} tilde_dU_a) and the complex
 * local energy E_L, and accumulates per walker the weighted sums from which
 *   dE/da  = 2 Re( <conj(O_a) E_L> - conj(<O_a>) <E_L> )
 *   S_ab   = Re( <conj(O_a) O_b> - conj(<O_a>) <O_b> )   (the SR matrix)
 * follow, <.> under |psi|^2: the weight is Z_mu for the reference acceptance
 * rule (whose chain samples |psi|^2 / Z_mu) and 1 for the Metropolis rule. */

/* dU_up: [n_params] column-major n_sites x n_up matrices (dU_up_imag the
 * imaginary parts, NULL when real); likewise dU_down.  1 <= n_params <= 8.
 * Resets the gradient sums. */
KVMC_API int kvmc_set_log_derivatives(kvmc_handle *h, int32_t n_params,
                             const double *dU_up, const double *dU_up_imag,
                             const double *dU_down, const double *dU_down_imag);

/* One adjoint evaluation at every walker's current configuration (run it
 * between kvmc_sweep calls, e.g. once per n-proposal sweep), added into the
 * sums.  Optional outputs: local_energy [n_walkers][2] (re, im) and
 * log_derivative [n_walkers][n_params][2]. */
KVMC_API int kvmc_measure_grad(kvmc_handle *h, double *local_energy, double *log_derivative);

/* Per-walker sums, [n_walkers][L] with L = 3 + 4P + 2P^2: sum w, sum w E_L
 * (re, im), sum w O_a (re, im)[P], sum w conj(O_a) E_L (re, im)[P],
 * sum w conj(O_a) O_b (re, im)[P][P].  Zeroed by kvmc_reset_stats. */
KVMC_API int kvmc_grad_sums(kvmc_handle *h, double *sums);

/* log|det tilde_U| per spin from the last refresh, [n_walkers][2] (up,
 * down): with kvmc_set_state it gives |psi'(x) / psi(x)|^2 between two
 * ansatz points on the same configurations (correlated sampling). */
KVMC_API int kvmc_walker_logdet(kvmc_handle *h, double *logdet);

/* Library version / build facts: abi version, compiled arch (e.g. 1030). */
KVMC_API int kvmc_version(int32_t *abi, int32_t *arch);

/* Name of CUDA device `device` (NUL-terminated, truncated to len) and its
 * SM count (sm_count may be NULL).  No reference counterpart: the tuning
 * cache is keyed by the chip its settings were measured on.
 * KVMC_ERR_NO_DEVICE when the device does not exist. */
KVMC_API int kvmc_device_name(int32_t device, char *buf, size_t len, int32_t *sm_count);

#ifdef __cplusplus
}
#endif

#endif /* KVMC_H */
