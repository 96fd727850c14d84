// Host side of libkvmc: the C ABI declared in include/kvmc.h.
//
// Handle lifecycle, argument validation with the reference's error classes,
// the FP64 hopping-matrix builder, and the launch loop that drives the CUDA
// kernels of kvmc_kernels.cu on one stream per handle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "kvmc.h"
#include "kvmc_internal.h"

using kvmc::DevBatch;
using kvmc::DevModel;

namespace {

thread_local std::string g_last_error;

int fail_global(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace

struct kvmc_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    kvmc_model_desc model{};
    kvmc_batch_desc batch{};
    int n_sites = 0, n_up = 0, n_dn = 0, ld_up = 0, ld_dn = 0, n_bonds = 0, n_walkers = 0;
    bool mixed = false;
    bool cplx = false;  // complex orbitals and W (B != 0)
    bool smem_w = false;
    int refresh_every = 0;
    int measure_every = 0;
    int delay_k = 1;  // mixed form: 1 = rank-1 updates, 4/8/12/16 = delayed-update depth
    float drift_tol = 1e-4f;  // delayed form: early refresh past this unit-row deviation
    int drift_severe = 0;     // > 0: immediate refresh past this many tolerances; 0: max(100 tol, 1e-2)
    int cluster = 0;          // mixed real form, rank-1: W split over a cluster of 2 or 4 CTAs
    int stream_threads = 256;  // W in HBM: threads per walker
    int pipeline = 1;          // delayed form: pipelined scan / factor-column write
    int tc_flush = 0;          // W in HBM: rank-k flush on the tensor cores
    int refresh32 = 0;         // mixed real form: periodic refresh by FP32 iterative refinement, 1 per row, 2 tiled, 3 tiled with the residual on the tensor cores
    kvmc::OzRefresh oz{};      // buffers of refresh32 = 3 (allocated when it is first chosen)
    bool oz_ready = false;
    int warp_walkers = 0;      // mixed real form: > 0 = one warp per walker, walkers per CTA
    float cond_hi = 0.f, cond_lo = 0.f;  // the warp sweep's accuracy guard (0 = off)
    int64_t segment = 0;       // one-warp mode: kvmc_advance in segments of this many moves (0 = whole call)
    std::string err;

    DevModel dm{};
    DevBatch db{};
    // owned device buffers (freed in destroy)
    std::vector<void *> allocs;
    int *d_active = nullptr;
    int *d_attempt = nullptr;
    int *d_redo = nullptr;
    double *d_stats = nullptr;  // two sets of kCallStats: a sweep call's start and end
    double *h_stats = nullptr;  // pinned copy of d_stats
    int32_t *d_labels = nullptr;  // both spins' labels in the caller's 32-bit layout (2 x walkers x sites)
    int *d_bad = nullptr;         // per walker: the device label check failed
    int *h_bad = nullptr;         // pinned copy of d_bad
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;

    // timing: per-launch event pairs recorded without host syncs, read after
    // the call's final synchronisation
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_used;  // (kind, first event index)
    cudaEvent_t region[2] = {nullptr, nullptr};
    double t_ms[3] = {0, 0, 0};
    long long t_launch[3] = {0, 0, 0};

    // orbitals kept on the host (row-major, (re, im) pairs when complex) for
    // the adjoint set-up, and the adjoint's device buffers
    std::vector<double> U_up_host, U_dn_host;
    int n_params = 0;
    void *d_MT = nullptr;
    double *d_gsums = nullptr;
    double *d_gout = nullptr;
    size_t gsum_stride = 0;

    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        g_last_error = buf;
        return code;
    }
    int cuda(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return KVMC_OK;
        return fail(KVMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
    template <typename T>
    int alloc(T **p, size_t count) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T) > 0 ? count * sizeof(T) : 16);
        if (e != cudaSuccess) return cuda(e, "cudaMalloc");
        allocs.push_back(q);
        *p = static_cast<T *>(q);
        return KVMC_OK;
    }
    int scratch(size_t bytes, void **p) {
        if (bytes > scratch_bytes) {
            if (d_scratch) cudaFree(d_scratch);
            d_scratch = nullptr;
            cudaError_t e = cudaMalloc(&d_scratch, bytes);
            if (e != cudaSuccess) { scratch_bytes = 0; return cuda(e, "cudaMalloc(scratch)"); }
            scratch_bytes = bytes;
        }
        *p = d_scratch;
        return KVMC_OK;
    }
};

#define KV_TRY(expr)                 \
    do {                             \
        int _rc = (expr);            \
        if (_rc != KVMC_OK) return _rc; \
    } while (0)

namespace {

int set_device(kvmc_handle *h) { return h->cuda(cudaSetDevice(h->device), "cudaSetDevice"); }

// kappa validation: every site holds exactly one spinon, labels are a
// permutation of 1..n per spin (src/Hamiltonian.jl:548-564, src/MonteCarlo.jl:92-115).
// One walker's labels: in range, every site holding exactly one spin, no
// label twice.  seen_u / seen_d (n_up + 1, n_dn + 1 entries) hold the last
// walker that used each label, so one pair of tables serves all walkers.
int validate_kappa(kvmc_handle *h, const int32_t *ku, const int32_t *kd, int walker, int *seen_u, int *seen_d) {
    const int N = h->n_sites;
    for (int s = 0; s < N; ++s) {
        const int a = ku[s], b = kd[s];
        if (a < 0 || a > h->n_up || b < 0 || b > h->n_dn)
            return h->fail(KVMC_ERR_BOUNDS, "walker %d site %d: label out of range (kappa_up=%d kappa_down=%d)", walker, s, a, b);
        if ((a != 0) == (b != 0))
            return h->fail(KVMC_ERR_ARGUMENT, "walker %d site %d is %s", walker, s, a != 0 ? "doubly occupied" : "unoccupied");
        if (a != 0) {
            if (seen_u[a] == walker) return h->fail(KVMC_ERR_ARGUMENT, "walker %d: up label %d repeated", walker, a);
            seen_u[a] = walker;
        } else {
            if (seen_d[b] == walker) return h->fail(KVMC_ERR_ARGUMENT, "walker %d: down label %d repeated", walker, b);
            seen_d[b] = walker;
        }
    }
    return KVMC_OK;
}

// Copies every walker's labels to the device, checks them there (one warp
// per walker) and only then converts them into the walkers' 16-bit labels:
// nothing of the walkers' state changes when a walker is invalid.  The
// first invalid walker is checked again on the host, whose check names the
// site and the label.  Beyond 48 KB of label bitmaps per CTA (more than
// about 6000 orbitals per spin) the host checks every walker.
int upload_kappa(kvmc_handle *h, const int32_t *ku, const int32_t *kd) {
    const int N = h->n_sites, Wk = h->n_walkers;
    const size_t tot = (size_t)Wk * N;
    int32_t *du = h->d_labels, *dd = h->d_labels + tot;
    KV_TRY(h->cuda(cudaMemcpyAsync(du, ku, tot * 4, cudaMemcpyHostToDevice, h->stream), "upload kappa"));
    KV_TRY(h->cuda(cudaMemcpyAsync(dd, kd, tot * 4, cudaMemcpyHostToDevice, h->stream), "upload kappa"));
    std::vector<int> seen_u(h->n_up + 1, -1), seen_d(h->n_dn + 1, -1);
    if (kvmc::labels_check_smem(h->n_up, h->n_dn) > 48 * 1024) {
        for (int w = 0; w < Wk; ++w)
            KV_TRY(validate_kappa(h, ku + (size_t)w * N, kd + (size_t)w * N, w, seen_u.data(), seen_d.data()));
    } else {
        KV_TRY(h->cuda(kvmc::launch_labels_check(du, dd, Wk, N, h->n_up, h->n_dn, h->d_bad, h->stream), "label check"));
        KV_TRY(h->cuda(cudaMemcpyAsync(h->h_bad, h->d_bad, (size_t)Wk * sizeof(int), cudaMemcpyDeviceToHost, h->stream),
                       "label check"));
        KV_TRY(h->cuda(cudaStreamSynchronize(h->stream), "label check"));
        for (int w = 0; w < Wk; ++w)
            if (h->h_bad[w]) {
                KV_TRY(validate_kappa(h, ku + (size_t)w * N, kd + (size_t)w * N, w, seen_u.data(), seen_d.data()));
                return h->fail(KVMC_ERR_ARGUMENT, "walker %d: invalid labels", w);
            }
    }
    return h->cuda(kvmc::launch_labels_convert(du, dd, h->db, N, 1, h->stream), "upload kappa");
}

// The FP32 refresh by iterative refinement: one thread per row (1) or tiled (2)
cudaError_t refresh32_launch(kvmc_handle *h, int only_due, int track_drift) {
    if (h->refresh32 == 3)
        return kvmc::launch_refresh_oz(h->dm, h->db, h->oz, only_due, track_drift, h->device, h->stream);
    return h->refresh32 == 2 ? kvmc::launch_refresh_tile(h->dm, h->db, only_due, track_drift, h->stream)
                             : kvmc::launch_refresh32(h->dm, h->db, only_due, track_drift, h->stream);
}

// The buffers of the refresh with its residual on the tensor cores: U's digit
// planes for both spins (computed here from the host copy of U) and the
// per-walker planes, matrices and tile states, zeroed once.
int oz_prepare(kvmc_handle *h) {
    if (h->oz_ready) return KVMC_OK;
    KV_TRY(set_device(h));
    const int N = h->n_sites;
    const int ns[2] = {h->n_up, h->n_dn};
    const std::vector<double> *U[2] = {&h->U_up_host, &h->U_dn_host};
    for (int s = 0; s < 2; ++s) {
        if (U[s]->size() != (size_t)N * ns[s]) return h->fail(KVMC_ERR_UNSUPPORTED, "no host copy of the orbitals");
        std::vector<uint16_t> ud((size_t)kvmc::kOzUDigits * N * ns[s]);
        std::vector<int> fe(ns[s]);
        kvmc::oz_digits_host(U[s]->data(), N, ns[s], ud.data(), fe.data());
        uint16_t *d_ud = nullptr;
        int *d_fe = nullptr;
        KV_TRY(h->alloc(&d_ud, ud.size()));
        KV_TRY(h->alloc(&d_fe, fe.size()));
        KV_TRY(h->cuda(cudaMemcpy(d_ud, ud.data(), ud.size() * 2, cudaMemcpyHostToDevice), "upload U digits"));
        KV_TRY(h->cuda(cudaMemcpy(d_fe, fe.data(), fe.size() * 4, cudaMemcpyHostToDevice), "upload U digits"));
        h->oz.ud[s] = d_ud;
        h->oz.fexp[s] = d_fe;
    }
    const size_t bytes = kvmc::oz_scratch_bytes(h->dm, h->n_walkers);
    unsigned char *scr = nullptr;
    KV_TRY(h->alloc(&scr, bytes));
    KV_TRY(h->cuda(cudaMemset(scr, 0, bytes), "clear refresh buffers"));
    KV_TRY(h->cuda(kvmc::oz_setup(h->dm, h->n_walkers, scr, h->oz), "tensor maps of the refresh"));
    h->oz_ready = true;
    return KVMC_OK;
}

// The real and the complex kernels behind one call each
cudaError_t refresh_launch(kvmc_handle *h, int only_due, int track_drift) {
    if (h->cplx) return kvmc::launch_refresh_c(h->dm, h->db, h->mixed, only_due, track_drift, h->stream);
    if (h->refresh32 && only_due == 1) {
        // FP32 refresh by iterative refinement; the walkers it gives up on are
        // rebuilt by the FP64 refresh, then their flag is cleared
        cudaError_t e = refresh32_launch(h, 1, track_drift);
        if (e == cudaSuccess) e = kvmc::launch_refresh(h->dm, h->db, true, 2, 0, h->stream);
        if (e == cudaSuccess) e = kvmc::launch_clear_status(h->db, kvmc::kStatusRefine, h->stream);
        return e;
    }
    return kvmc::launch_refresh(h->dm, h->db, h->mixed, only_due, track_drift, h->stream);
}

cudaError_t sweep_launch(kvmc_handle *h, const kvmc::SweepParams &p) {
    if (h->cplx) return kvmc::launch_sweep_c(h->dm, h->db, p, h->mixed, h->d_active, h->stream);
    return kvmc::launch_sweep(h->dm, h->db, p, h->mixed, h->smem_w, h->d_active, h->stream);
}

// Rebuilds every walker's W.  allow32: with the FP32 refinement refresh
// enabled, use it (FP64 for the walkers it flags); otherwise FP64 throughout.
int full_refresh(kvmc_handle *h, bool track_drift, bool allow32 = true) {
    h->db.compact = 0;  // W32 is rebuilt for every walker
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.drift, 0, sizeof(float) * h->n_walkers, h->stream), "memset"));
    if (allow32 && h->refresh32 && !h->cplx) {
        KV_TRY(h->cuda(refresh32_launch(h, 0, track_drift ? 1 : 0), "refresh launch"));
        KV_TRY(h->cuda(kvmc::launch_refresh(h->dm, h->db, true, 2, 0, h->stream), "refresh launch"));
        KV_TRY(h->cuda(kvmc::launch_clear_status(h->db, kvmc::kStatusRefine, h->stream), "refresh launch"));
    } else {
        KV_TRY(h->cuda(refresh_launch(h, 0, track_drift ? 1 : 0), "refresh launch"));
    }
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.since, 0, sizeof(int) * h->n_walkers, h->stream), "memset"));
    if (h->db.cond_max)
        KV_TRY(h->cuda(cudaMemsetAsync(h->db.cond_max, 0, sizeof(float) * h->n_walkers, h->stream), "memset"));
    return h->cuda(cudaStreamSynchronize(h->stream), "refresh");
}

// The error for nb walkers with a status set, the first of them walker
// `first` with status `code`.
int status_error(kvmc_handle *h, int nb, int first, int code) {
    if (nb) {
        if (code & kvmc::kStatusSingular)
            return h->fail(KVMC_ERR_SINGULAR, "%d walker(s) have a singular tilde_U (first: walker %d)", nb, first);
        if (code & kvmc::kStatusTimeout)
            return h->fail(KVMC_ERR_CUDA, "%d walker(s): a tensor-core wait timed out (first: walker %d)", nb, first);
        return h->fail(KVMC_ERR_NUMERIC, "%d walker(s) produced a non-finite ratio (first: walker %d)", nb, first);
    }
    return KVMC_OK;
}

int check_status(kvmc_handle *h, int *bad) {
    std::vector<int> st(h->n_walkers);
    KV_TRY(h->cuda(cudaMemcpy(st.data(), h->db.status, sizeof(int) * h->n_walkers, cudaMemcpyDeviceToHost), "status"));
    int nb = 0, first = -1, code = 0;
    for (int w = 0; w < h->n_walkers; ++w)
        if (st[w]) { ++nb; if (first < 0) { first = w; code = st[w]; } }
    if (bad) *bad = nb;
    if (nb) {
        if (code & kvmc::kStatusSingular)
            return h->fail(KVMC_ERR_SINGULAR, "%d walker(s) have a singular tilde_U (first: walker %d)", nb, first);
        if (code & kvmc::kStatusTimeout)
            return h->fail(KVMC_ERR_CUDA, "%d walker(s): a tensor-core wait timed out (first: walker %d)", nb, first);
        return h->fail(KVMC_ERR_NUMERIC, "%d walker(s) produced a non-finite ratio (first: walker %d)", nb, first);
    }
    return KVMC_OK;
}

struct Vec2 { double x, y; };

}  // namespace

// ===========================================================================
// Lattice and hopping matrix (host FP64)
// ===========================================================================

extern "C" int kvmc_lattice_sites(const kvmc_lattice_desc *lat, int32_t *n_sites) {
    if (!lat || !n_sites) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    if (lat->n1 % 2 != 0) return fail_global(KVMC_ERR_ARGUMENT, "n1 must be even in DoubleKagome");
    if (lat->n1 <= 0 || lat->n2 <= 0) return fail_global(KVMC_ERR_ARGUMENT, "n1, n2 must be positive");
    *n_sites = lat->n1 * lat->n2 * 3;
    return KVMC_OK;
}

namespace {

// Default tables: src/Hamiltonian.jl:219-235 and :250-261.
const kvmc_link kPiLinkIn[] = {
    {1, 2, 0, 0, 1}, {1, 3, 0, 0, 1}, {2, 3, 0, 0, 1}, {2, 4, 0, 0, -1}, {4, 6, 0, 0, 1},
    {4, 5, 0, 0, 1}, {5, 6, 0, 0, 1}, {2, 1, 0, 0, 1}, {3, 1, 0, 0, 1}, {3, 2, 0, 0, 1},
    {4, 2, 0, 0, -1}, {6, 4, 0, 0, 1}, {5, 4, 0, 0, 1}, {6, 5, 0, 0, 1}};
const kvmc_link kPiLinkInter[] = {
    {3, 5, -1, 1, -1}, {3, 1, 0, 1, -1}, {6, 2, 0, 1, -1}, {6, 4, 0, 1, 1}, {5, 1, 1, 0, 1},
    {1, 5, -1, 0, 1}, {1, 3, 0, -1, -1}, {2, 6, 0, -1, -1}, {4, 6, 0, -1, 1}, {5, 3, 1, -1, -1}};

struct LatticeGeom {
    int n1h, n2;
    Vec2 a1, a2, r[6];
    bool pbc1, pbc2, anti1, anti2;
    // src/Hamiltonian.jl:28-38 (s 1-based)
    Vec2 uc(int s) const {
        const int u = (s - 1) / 6;
        const double k1 = (double)(u % n1h), k2 = (double)(u / n1h);
        return {k1 * a1.x + k2 * a2.x, k1 * a1.y + k2 * a2.y};
    }
    // src/Hamiltonian.jl:279-283
    Vec2 site(int s) const {
        const Vec2 u = uc(s);
        const Vec2 d = r[(s - 1) % 6];
        return {u.x + d.x, u.y + d.y};
    }
};

LatticeGeom make_geom(const kvmc_lattice_desc *lat) {
    // src/Lattice.jl:68-92
    LatticeGeom g;
    const double t = lat->t, a = 2 * t;
    g.n1h = lat->n1 / 2;
    g.n2 = lat->n2;
    g.a1 = {2 * a, 0.0};
    g.a2 = {0.5 * a, 0.5 * std::sqrt(3.0) * a};
    g.r[0] = {0.0, 0.0};
    g.r[1] = {0.25 * g.a1.x, 0.25 * g.a1.y};
    g.r[2] = {0.5 * g.a2.x, 0.5 * g.a2.y};
    g.r[3] = {0.5 * g.a1.x, 0.5 * g.a1.y};
    g.r[4] = {0.75 * g.a1.x, 0.75 * g.a1.y};
    g.r[5] = {2.5 * t, 0.5 * std::sqrt(3.0) * t};
    g.pbc1 = lat->pbc[0] != 0;
    g.pbc2 = lat->pbc[1] != 0;
    g.anti1 = lat->antipbc[0] != 0;
    g.anti2 = lat->antipbc[1] != 0;
    return g;
}

std::complex<double> peierls(double B, Vec2 r1, Vec2 r2) {
    // src/Hamiltonian.jl:201-202, :325-326
    const double phase = (B / 2) * (r1.x + r2.x) * (r2.y - r1.y);
    return {std::cos(phase), std::sin(phase)};
}

}  // namespace

extern "C" int kvmc_hopping_matrix(const kvmc_lattice_desc *lat, const kvmc_link *link_in, int32_t n_link_in,
                                   const kvmc_link *link_inter, int32_t n_link_inter, double B, double *H) {
    int32_t N = 0;
    int rc = kvmc_lattice_sites(lat, &N);
    if (rc) return rc;
    if (!H) return fail_global(KVMC_ERR_ARGUMENT, "null H");
    for (int d = 0; d < 2; ++d)
        if (lat->antipbc[d] && !lat->pbc[d])
            return fail_global(KVMC_ERR_ARGUMENT,
                               "Invalid boundary conditions in %s direction: Cannot have antiperiodic boundary "
                               "conditions without periodic boundary conditions",
                               d == 0 ? "first" : "second");
    if (!link_in) { link_in = kPiLinkIn; n_link_in = (int32_t)(sizeof kPiLinkIn / sizeof kPiLinkIn[0]); }
    if (!link_inter) { link_inter = kPiLinkInter; n_link_inter = (int32_t)(sizeof kPiLinkInter / sizeof kPiLinkInter[0]); }
    std::map<std::pair<int, int>, double> lin;
    std::map<std::tuple<int, int, int, int>, double> linter;
    for (int e = 0; e < n_link_in; ++e) {
        const auto &k = link_in[e];
        if (k.label1 < 1 || k.label1 > 6 || k.label2 < 1 || k.label2 > 6)
            return fail_global(KVMC_ERR_ARGUMENT, "link_in entry %d: labels must be 1..6", e);
        if (!lin.emplace(std::make_pair(k.label1, k.label2), k.amplitude).second)
            return fail_global(KVMC_ERR_ARGUMENT, "link_in entry %d repeats a key", e);
    }
    for (int e = 0; e < n_link_inter; ++e) {
        const auto &k = link_inter[e];
        if (k.label1 < 1 || k.label1 > 6 || k.label2 < 1 || k.label2 > 6)
            return fail_global(KVMC_ERR_ARGUMENT, "link_inter entry %d: labels must be 1..6", e);
        if (!linter.emplace(std::make_tuple(k.label1, k.label2, k.dx, k.dy), k.amplitude).second)
            return fail_global(KVMC_ERR_ARGUMENT, "link_inter entry %d repeats a key", e);
    }
    const LatticeGeom g = make_geom(lat);
    const int ncell = lat->n1 * lat->n2 / 2;
    std::vector<std::complex<double>> T((size_t)N * N);
    auto at = [&](int s1, int s2) -> std::complex<double> & { return T[(size_t)(s1 - 1) + (size_t)(s2 - 1) * N]; };
    // in-cell (src/Hamiltonian.jl:316-330)
    for (int c = 1; c <= ncell; ++c)
        for (int s1 = (c - 1) * 6 + 1; s1 <= c * 6; ++s1)
            for (int s2 = s1 + 1; s2 <= c * 6; ++s2) {
                auto it = lin.find({(s1 - 1) % 6 + 1, (s2 - 1) % 6 + 1});
                if (it != lin.end()) at(s1, s2) = it->second * peierls(B, g.site(s1), g.site(s2));
            }
    // Inter-cell (src/Hamiltonian.jl:333-343 with :99-153, :177-207).  The
    // reference visits every cell pair and, per site pair, every image shift
    // (O(N^2)); here every (cell, inter-cell link, image) triple names its one
    // partner cell directly (O(N)).  For a pair (s1 < s2) in cells (c1, c2),
    // the reference tries the plain cell offset d first and then d + image
    // for the images (ix, iy) in order; a link key (l1, l2, dx, dy) matches
    // when that candidate equals (dx, dy), i.e. when c2 = c1 + (dx, dy) - image.
    // Each entry's contributions are summed in the reference's candidate
    // order, from the same floating-point expressions, so T is bit-identical.
    {
        struct Contrib { size_t entry; int pos; std::complex<double> v; };
        std::vector<Contrib> contrib;
        const int sx[3] = {-g.n1h, 0, g.n1h}, sy[3] = {-g.n2, 0, g.n2};
        for (int c1 = 1; c1 <= ncell; ++c1) {
            const int k1 = (c1 - 1) % g.n1h, k2 = (c1 - 1) / g.n1h;
            for (const auto &kv : linter) {
                const int l1 = std::get<0>(kv.first), l2 = std::get<1>(kv.first);
                const int qdx = std::get<2>(kv.first), qdy = std::get<3>(kv.first);
                // candidate positions: 0 = the plain offset, then the images in (ix, iy) order
                int pos = 0;
                for (int img = -1; img < 9; ++img) {
                    int ix = 1, iy = 1;
                    double sign = 1.0;
                    if (img >= 0) {
                        ix = img / 3;
                        iy = img % 3;
                        if (!(g.pbc1 || g.pbc2)) break;
                        if (!g.pbc1 && ix != 1) continue;
                        if (!g.pbc2 && iy != 1) continue;
                        if (ix == 1 && iy == 1) continue;
                        ++pos;
                        if (g.anti1 && sx[ix] != 0) sign *= -1.0;
                        if (g.anti2 && sy[iy] != 0) sign *= -1.0;
                    }
                    const int k1b = k1 + qdx - sx[ix], k2b = k2 + qdy - sy[iy];
                    if (k1b < 0 || k1b >= g.n1h || k2b < 0 || k2b >= g.n2) continue;
                    const int c2 = k2b * g.n1h + k1b + 1;
                    if (c2 <= c1) continue;  // s1 < s2 in different cells means c1 < c2
                    const int s1 = (c1 - 1) * 6 + l1, s2 = (c2 - 1) * 6 + l2;
                    const Vec2 u1 = g.uc(s1), u2 = g.uc(s2);
                    const Vec2 r1 = g.site(s1);
                    const Vec2 s2c = g.site(s2);
                    const Vec2 dr2 = {s2c.x - u2.x, s2c.y - u2.y};
                    Vec2 ruc2 = {u1.x + qdx * g.a1.x, u1.y + qdx * g.a1.y};
                    ruc2 = {ruc2.x + qdy * g.a2.x, ruc2.y + qdy * g.a2.y};
                    const Vec2 r2 = {ruc2.x + dr2.x, ruc2.y + dr2.y};
                    contrib.push_back({(size_t)(s1 - 1) + (size_t)(s2 - 1) * N, img < 0 ? 0 : pos,
                                       (sign * kv.second) * peierls(B, r1, r2)});
                }
            }
        }
        std::stable_sort(contrib.begin(), contrib.end(), [](const Contrib &x, const Contrib &y) {
            return x.entry != y.entry ? x.entry < y.entry : x.pos < y.pos;
        });
        for (const auto &c : contrib) T[c.entry] += c.v;
    }
    // H = -(T + T^dagger), column-major interleaved
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            const std::complex<double> v = -(T[(size_t)i + (size_t)j * N] + std::conj(T[(size_t)j + (size_t)i * N]));
            H[2 * ((size_t)i + (size_t)j * N)] = v.real();
            H[2 * ((size_t)i + (size_t)j * N) + 1] = v.imag();
        }
    return KVMC_OK;
}

extern "C" int kvmc_bonds_from_hopping(int32_t n_sites, const double *H, int32_t *n_bonds, int32_t *bonds) {
    if (!H || !n_bonds || n_sites <= 0) return fail_global(KVMC_ERR_ARGUMENT, "bad argument");
    int32_t c = 0;
    for (int j = 0; j < n_sites; ++j)
        for (int i = 0; i <= j; ++i) {
            const size_t e = 2 * ((size_t)i + (size_t)j * n_sites);
            if (H[e] != 0.0 || H[e + 1] != 0.0) {
                if (bonds) { bonds[2 * c] = i; bonds[2 * c + 1] = j; }
                ++c;
            }
        }
    *n_bonds = c;
    return KVMC_OK;
}

// Extended ansatz: the pi-flux H with a triangle flux theta and second-
// neighbour hops t2 + i*m*nu (the parameterisation is stated in kvmc.h).
// Geometry comes from the site coordinates (src/Hamiltonian.jl:279-283) and
// the minimum image over the periodic directions.
extern "C" int kvmc_ansatz_hopping(const kvmc_lattice_desc *lat, const kvmc_link *link_in, int32_t n_link_in,
                                   const kvmc_link *link_inter, int32_t n_link_inter, double B, const double *params,
                                   double *H, double *dH) {
    if (!lat || !params || !H) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    int32_t N = 0;
    if (int rc = kvmc_lattice_sites(lat, &N)) return rc;
    const double t2 = params[0], mch = params[1], theta = params[2];
    if (!std::isfinite(t2) || !std::isfinite(mch) || !std::isfinite(theta))
        return fail_global(KVMC_ERR_ARGUMENT, "ansatz parameters must be finite");
    std::vector<double> H0(2 * (size_t)N * N), Hpi(2 * (size_t)N * N);
    if (int rc = kvmc_hopping_matrix(lat, link_in, n_link_in, link_inter, n_link_inter, B, H0.data())) return rc;
    if (int rc = kvmc_hopping_matrix(lat, link_in, n_link_in, link_inter, n_link_inter, 0.0, Hpi.data())) return rc;
    using cplx = std::complex<double>;
    auto ix = [N](int i, int j) { return (size_t)i + (size_t)j * N; };
    const LatticeGeom g = make_geom(lat);
    const Vec2 L1 = {g.n1h * g.a1.x, g.n1h * g.a1.y}, L2 = {g.n2 * g.a2.x, g.n2 * g.a2.y};
    std::vector<Vec2> pos(N);
    for (int s = 0; s < N; ++s) pos[s] = g.site(s + 1);
    const double t = lat->t, tol = 1e-9 * t * t;
    // displacements r_j - r_i over the images at squared length want; n = how many
    auto disp = [&](int i, int j, double want, Vec2 &d) {
        int n = 0;
        for (int p = -1; p <= 1; ++p) {
            if (p != 0 && !g.pbc1) continue;
            for (int q = -1; q <= 1; ++q) {
                if (q != 0 && !g.pbc2) continue;
                const Vec2 e = {pos[j].x - pos[i].x + p * L1.x + q * L2.x, pos[j].y - pos[i].y + p * L1.y + q * L2.y};
                if (std::fabs(e.x * e.x + e.y * e.y - want) <= tol) { d = e; ++n; }
            }
        }
        return n;
    };
    // nearest neighbours: the nonzeros of the pi-flux H, each at one image
    std::vector<std::vector<int>> nbr(N);
    std::vector<std::vector<Vec2>> dnb(N);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            if (i == j || (Hpi[2 * ix(i, j)] == 0.0 && Hpi[2 * ix(i, j) + 1] == 0.0)) continue;
            Vec2 d{};
            const int n = disp(i, j, t * t, d);
            if (n != 1)
                return fail_global(KVMC_ERR_ARGUMENT,
                                   "lattice too small for the extended ansatz: sites %d and %d are %s", i, j,
                                   n == 0 ? "not at nearest-neighbour distance" : "neighbours through several images");
            nbr[i].push_back(j);
            dnb[i].push_back(d);
        }
    auto cross = [](Vec2 a, Vec2 b) { return a.x * b.y - a.y * b.x; };
    std::vector<cplx> Hx((size_t)N * N), dT2((size_t)N * N), dM((size_t)N * N), dTh((size_t)N * N);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) Hx[ix(i, j)] = cplx(H0[2 * ix(i, j)], H0[2 * ix(i, j) + 1]);
    // theta: orientation of each nearest-neighbour hop in its triangle
    for (int i = 0; i < N; ++i)
        for (size_t a = 0; a < nbr[i].size(); ++a) {
            const int j = nbr[i][a];
            const Vec2 dij = dnb[i][a];
            int found = 0;
            double s = 0.0;
            for (size_t b = 0; b < nbr[j].size(); ++b) {
                const Vec2 djk = dnb[j][b];
                const Vec2 dik = {dij.x + djk.x, dij.y + djk.y};
                if (nbr[j][b] == i || std::fabs(dik.x * dik.x + dik.y * dik.y - t * t) > tol) continue;
                s = cross(dij, djk) > 0 ? 1.0 : -1.0;
                ++found;
            }
            if (found != 1)
                return fail_global(KVMC_ERR_ARGUMENT, "bond (%d, %d) does not close exactly one triangle", i, j);
            const cplx ph(std::cos(theta * s / 3.0), std::sin(theta * s / 3.0));
            Hx[ix(i, j)] *= ph;
            dTh[ix(i, j)] = Hx[ix(i, j)] * cplx(0.0, s / 3.0);
        }
    // second neighbours: bent paths i -> j -> k around a hexagon corner
    for (int j = 0; j < N; ++j)
        for (size_t a = 0; a < nbr[j].size(); ++a)
            for (size_t b = 0; b < nbr[j].size(); ++b) {
                if (a == b) continue;
                const int i = nbr[j][a], k = nbr[j][b];
                // r_j - r_i is minus the displacement from j to i
                const Vec2 dij = {-dnb[j][a].x, -dnb[j][a].y}, djk = dnb[j][b];
                const Vec2 dik = {dij.x + djk.x, dij.y + djk.y};
                if (std::fabs(dik.x * dik.x + dik.y * dik.y - 3 * t * t) > tol) continue;
                const double gij = Hpi[2 * ix(i, j)], gjk = Hpi[2 * ix(j, k)];
                const double gs = (gij * gjk) > 0 ? 1.0 : -1.0;
                const double nu = cross(dij, djk) > 0 ? 1.0 : -1.0;
                Hx[ix(i, k)] += -cplx(t2, mch * nu) * gs;
                dT2[ix(i, k)] += -gs;
                dM[ix(i, k)] += cplx(0.0, -nu * gs);
            }
    for (size_t e = 0; e < (size_t)N * N; ++e) {
        H[2 * e] = Hx[e].real();
        H[2 * e + 1] = Hx[e].imag();
        if (dH) {
            const cplx *src[3] = {&dT2[e], &dM[e], &dTh[e]};
            for (int q = 0; q < 3; ++q) {
                dH[2 * ((size_t)q * N * N + e)] = src[q]->real();
                dH[2 * ((size_t)q * N * N + e) + 1] = src[q]->imag();
            }
        }
    }
    return KVMC_OK;
}

// ===========================================================================
// Handle
// ===========================================================================

extern "C" int kvmc_version(int32_t *abi, int32_t *arch) {
    if (abi) *abi = KVMC_ABI_VERSION;
    if (arch) *arch = 1030;
    return KVMC_OK;
}

extern "C" int kvmc_device_name(int32_t device, char *buf, size_t len, int32_t *sm_count) {
    if (!buf || len == 0) return fail_global(KVMC_ERR_ARGUMENT, "kvmc_device_name: buf must hold at least one byte");
    buf[0] = 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
        return fail_global(KVMC_ERR_NO_DEVICE, "kvmc_device_name: no CUDA device %d", device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return fail_global(KVMC_ERR_CUDA, "kvmc_device_name: cudaGetDeviceProperties failed");
    snprintf(buf, len, "%s", prop.name);
    if (sm_count) *sm_count = prop.multiProcessorCount;
    return KVMC_OK;
}

extern "C" int kvmc_last_error(const kvmc_handle *h, char *buf, size_t len) {
    if (!buf || len == 0) return KVMC_ERR_ARGUMENT;
    const std::string &s = h ? h->err : g_last_error;
    snprintf(buf, len, "%s", s.c_str());
    return KVMC_OK;
}

extern "C" int kvmc_destroy(kvmc_handle *h) {
    if (!h) return KVMC_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void *p : h->allocs) cudaFree(p);
    if (h->d_scratch) cudaFree(h->d_scratch);
    if (h->d_MT) cudaFree(h->d_MT);
    if (h->d_gsums) cudaFree(h->d_gsums);
    if (h->d_gout) cudaFree(h->d_gout);
    if (h->h_stats) cudaFreeHost(h->h_stats);
    if (h->h_bad) cudaFreeHost(h->h_bad);
    for (auto &e : h->ev_pool) cudaEventDestroy(e);
    for (auto &e : h->region)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return KVMC_OK;
}

extern "C" int kvmc_create(const kvmc_model_desc *model, const kvmc_batch_desc *batch, kvmc_handle **out) {
    if (!model || !batch || !out) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    const int N = model->n_sites, nu = model->n_up, nd = model->n_down, nb = model->n_bonds;
    if (N <= 0 || N > 30000) return fail_global(KVMC_ERR_ARGUMENT, "n_sites must be in 1..30000");
    if (nu <= 0 || nd <= 0 || nu + nd != N)
        return fail_global(KVMC_ERR_ARGUMENT, "n_up + n_down must equal n_sites with both positive (got %d + %d vs %d)", nu, nd, N);
    if (nb <= 0 || !model->bonds) return fail_global(KVMC_ERR_ARGUMENT, "empty bond list");
    if (!model->U_up || !model->U_down) return fail_global(KVMC_ERR_ARGUMENT, "null orbitals");
    for (int e = 0; e < nb; ++e) {
        const int i = model->bonds[2 * e], j = model->bonds[2 * e + 1];
        if (i < 0 || j < 0 || i >= N || j >= N) return fail_global(KVMC_ERR_BOUNDS, "bond %d (%d,%d) out of range", e, i, j);
        if (i == j) return fail_global(KVMC_ERR_ARGUMENT, "bond %d joins site %d to itself", e, i);
    }
    {
        // Z_mu counts bonds; the sweep updates it from neighbour counts, which
        // needs every bond once
        std::vector<std::pair<int, int>> pairs(nb);
        for (int e = 0; e < nb; ++e) {
            const int i = model->bonds[2 * e], j = model->bonds[2 * e + 1];
            pairs[e] = {std::min(i, j), std::max(i, j)};
        }
        std::sort(pairs.begin(), pairs.end());
        for (int e = 1; e < nb; ++e)
            if (pairs[e] == pairs[e - 1])
                return fail_global(KVMC_ERR_ARGUMENT, "bond (%d,%d) appears more than once", pairs[e].first,
                                   pairs[e].second);
    }
    if (batch->n_walkers <= 0) return fail_global(KVMC_ERR_ARGUMENT, "n_walkers must be positive");
    if (batch->precision != KVMC_PLAIN_FP64 && batch->precision != KVMC_MIXED_FP32)
        return fail_global(KVMC_ERR_ARGUMENT, "unknown precision %d", batch->precision);
    if (batch->accept_rule != KVMC_ACCEPT_REFERENCE && batch->accept_rule != KVMC_ACCEPT_METROPOLIS)
        return fail_global(KVMC_ERR_ARGUMENT, "unknown accept rule %d", batch->accept_rule);
    if (batch->refresh_interval < 0 || batch->measure_interval < 0)
        return fail_global(KVMC_ERR_ARGUMENT, "intervals must be >= 0");
    if (std::max(nu, nd) > 2048)
        return fail_global(KVMC_ERR_UNSUPPORTED, "more than 2048 orbitals per spin is not supported by this build");

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail_global(KVMC_ERR_NO_DEVICE, "no CUDA device");
    }
    if (batch->device < 0 || batch->device >= ndev) return fail_global(KVMC_ERR_NO_DEVICE, "device %d not present", batch->device);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, batch->device);
    if (prop.major * 10 + prop.minor != 103)
        return fail_global(KVMC_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a", batch->device, prop.major, prop.minor);

    kvmc_handle *h = new kvmc_handle();
    h->device = batch->device;
    h->model = *model;
    h->batch = *batch;
    h->n_sites = N; h->n_up = nu; h->n_dn = nd; h->n_bonds = nb; h->n_walkers = batch->n_walkers;
    h->ld_up = (nu + 3) / 4 * 4;
    h->ld_dn = (nd + 3) / 4 * 4;
    h->mixed = batch->precision == KVMC_MIXED_FP32;
    h->cplx = model->U_up_imag != nullptr || model->U_down_imag != nullptr;
    const int nocc = std::min(nu, nd);
    h->measure_every = batch->measure_interval > 0 ? batch->measure_interval : nocc;
    if (h->mixed) h->refresh_every = batch->refresh_interval > 0 ? batch->refresh_interval : 128;
    else h->refresh_every = batch->refresh_interval > 0 ? batch->refresh_interval : nocc;

    auto bail = [&](int rc) { g_last_error = h->err; kvmc_destroy(h); return rc; };
    if (int rc = set_device(h)) return bail(rc);
    if (int rc = h->cuda(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream")) return bail(rc);

    DevModel &m = h->dm;
    m.n_sites = N; m.n_up = nu; m.n_dn = nd; m.ld_up = h->ld_up; m.ld_dn = h->ld_dn; m.n_bonds = nb;
    // orbitals row-major; complex ones as interleaved (re, im)
    const size_t cw = h->cplx ? 2 : 1;
    std::vector<double> Uu((size_t)N * nu * cw), Ud((size_t)N * nd * cw);
    for (int r = 0; r < N; ++r) {
        for (int c = 0; c < nu; ++c) {
            const size_t src = (size_t)r + (size_t)c * N, dst = ((size_t)r * nu + c) * cw;
            Uu[dst] = model->U_up[src];
            if (h->cplx) Uu[dst + 1] = model->U_up_imag ? model->U_up_imag[src] : 0.0;
        }
        for (int c = 0; c < nd; ++c) {
            const size_t src = (size_t)r + (size_t)c * N, dst = ((size_t)r * nd + c) * cw;
            Ud[dst] = model->U_down[src];
            if (h->cplx) Ud[dst + 1] = model->U_down_imag ? model->U_down_imag[src] : 0.0;
        }
    }
    // bonds and adjacency
    std::vector<short2> bonds(nb);
    std::vector<int> deg(N + 1, 0);
    for (int e = 0; e < nb; ++e) {
        bonds[e] = make_short2((short)model->bonds[2 * e], (short)model->bonds[2 * e + 1]);
        deg[model->bonds[2 * e]]++;
        deg[model->bonds[2 * e + 1]]++;
    }
    std::vector<int> off(N + 1, 0);
    for (int s = 0; s < N; ++s) off[s + 1] = off[s] + deg[s];
    std::vector<short> nbr(2 * (size_t)nb);
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int e = 0; e < nb; ++e) {
        const int i = model->bonds[2 * e], j = model->bonds[2 * e + 1];
        nbr[fill[i]++] = (short)j;
        nbr[fill[j]++] = (short)i;
    }
    double *dUu = nullptr, *dUd = nullptr;
    short2 *dB = nullptr;
    int *dOff = nullptr;
    short *dNbr = nullptr;
    int rc = KVMC_OK;
    if ((rc = h->alloc(&dUu, Uu.size())) || (rc = h->alloc(&dUd, Ud.size())) || (rc = h->alloc(&dB, nb)) ||
        (rc = h->alloc(&dOff, N + 1)) || (rc = h->alloc(&dNbr, nbr.size())))
        return bail(rc);
    cudaMemcpy(dUu, Uu.data(), Uu.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dUd, Ud.data(), Ud.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, bonds.data(), nb * sizeof(short2), cudaMemcpyHostToDevice);
    cudaMemcpy(dOff, off.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(dNbr, nbr.data(), nbr.size() * sizeof(short), cudaMemcpyHostToDevice);
    m.U_up = dUu; m.U_dn = dUd; m.bonds = dB; m.nbr_off = dOff; m.nbr = dNbr;
    m.U32_up_hi = m.U32_up_lo = m.U32_dn_hi = m.U32_dn_lo = nullptr;
    if (h->mixed && !h->cplx) {
        // FP32 (high, low) pairs of U for the FP32 refresh's residual
        std::vector<float> hu[4];
        const std::vector<double> *src[2] = {&Uu, &Ud};
        for (int s2 = 0; s2 < 2; ++s2) {
            hu[2 * s2].resize(src[s2]->size());
            hu[2 * s2 + 1].resize(src[s2]->size());
            for (size_t e = 0; e < src[s2]->size(); ++e) {
                const double v = (*src[s2])[e];
                const float hi = (float)v;
                hu[2 * s2][e] = hi;
                hu[2 * s2 + 1][e] = (float)(v - (double)hi);
            }
        }
        float *d32[4];
        for (int q = 0; q < 4; ++q) {
            if ((rc = h->alloc(&d32[q], hu[q].size()))) return bail(rc);
            cudaMemcpy(d32[q], hu[q].data(), hu[q].size() * 4, cudaMemcpyHostToDevice);
        }
        m.U32_up_hi = d32[0]; m.U32_up_lo = d32[1]; m.U32_dn_hi = d32[2]; m.U32_dn_lo = d32[3];
    }
    h->U_up_host = std::move(Uu);
    h->U_dn_host = std::move(Ud);
    // thresholds fl(z / n_bonds) for z = 0..n_bonds, with their exact binary form
    std::vector<kvmc::ThrEntry> thr(nb + 1);
    for (int z = 0; z <= nb; ++z) {
        kvmc::ThrEntry &e = thr[z];
        e.d = (double)z / (double)nb;
        e.f = (float)e.d;
        if (z == 0) { e.m = 0; e.k = 0; continue; }
        unsigned long long bits;
        std::memcpy(&bits, &e.d, 8);
        e.m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        e.k = (int)((bits >> 52) & 0x7ff) - 1075 + 53;
    }
    kvmc::ThrEntry *dThr = nullptr;
    if ((rc = h->alloc(&dThr, thr.size()))) return bail(rc);
    cudaMemcpy(dThr, thr.data(), thr.size() * sizeof(kvmc::ThrEntry), cudaMemcpyHostToDevice);
    m.thr_table = dThr;

    DevBatch &b = h->db;
    const int Wk = h->n_walkers;
    b.n_walkers = Wk;
    const size_t wblock = (size_t)N * (h->ld_up + h->ld_dn) * cw;  // W64/W32 elements per walker
    b.W64 = nullptr;
    b.W32 = nullptr;
    if (h->mixed) rc = h->alloc(&b.W32, wblock * Wk);
    else rc = h->alloc(&b.W64, wblock * Wk);
    if (rc) return bail(rc);
    if ((rc = h->alloc(&b.kappa_up, (size_t)Wk * N)) || (rc = h->alloc(&b.kappa_dn, (size_t)Wk * N)) ||
        (rc = h->alloc(&b.t, Wk)) || (rc = h->alloc(&b.t_end, Wk)) || (rc = h->alloc(&b.acc_end, Wk)) ||
        (rc = h->alloc(&b.since, Wk)) ||
        (rc = h->alloc(&b.sum_e, Wk)) || (rc = h->alloc(&b.sum_e2, Wk)) || (rc = h->alloc(&b.n_meas, Wk)) ||
        (rc = h->alloc(&b.accepted, Wk)) || (rc = h->alloc(&b.proposals, Wk)) || (rc = h->alloc(&b.status, Wk)) ||
        (rc = h->alloc(&b.logdet, 4 * (size_t)Wk)) || (rc = h->alloc(&b.drift, Wk)) ||
        (rc = h->alloc(&b.energy_out, Wk)) || (rc = h->alloc(&b.refresh_count, 2)) || (rc = h->alloc(&h->d_active, 1)) ||
        (rc = h->alloc(&h->d_attempt, Wk)) || (rc = h->alloc(&h->d_redo, Wk)) ||
        (rc = h->alloc(&h->d_stats, 2 * kvmc::kCallStats)))
        return bail(rc);
    if ((rc = h->cuda(cudaMallocHost(reinterpret_cast<void **>(&h->h_stats), 2 * kvmc::kCallStats * sizeof(double)),
                      "cudaMallocHost")))
        return bail(rc);
    if ((rc = h->alloc(&h->d_labels, 2 * (size_t)Wk * m.n_sites)) || (rc = h->alloc(&h->d_bad, Wk)))
        return bail(rc);
    if ((rc = h->cuda(cudaMallocHost(reinterpret_cast<void **>(&h->h_bad), (size_t)Wk * sizeof(int)),
                      "cudaMallocHost")))
        return bail(rc);
    b.solve_block = kvmc::refresh_scratch_block(m) * cw;
    if ((rc = h->alloc(&b.solve_scratch, b.solve_block * 2 * (size_t)Wk))) return bail(rc);
    b.lu_block = 0;
    b.lu_scratch = nullptr;
    b.lu_invd = nullptr;
    b.lu_perm = nullptr;
    b.lu_aux_n = 0;
    b.G32 = nullptr;
    b.g_block = 0;
    b.cond_max = nullptr;
    if (h->mixed && (rc = h->alloc(&b.cond_max, Wk))) return bail(rc);
    if (b.cond_max) cudaMemset(b.cond_max, 0, Wk * sizeof(float));
    if (!h->cplx && kvmc::refresh_needs_large(m)) {
        const size_t nmax = (size_t)std::max(nu, nd);
        b.lu_block = nmax * nmax;
        if ((rc = h->alloc(&b.lu_scratch, b.lu_block * 2 * (size_t)Wk))) return bail(rc);
        // the FP64 refresh's row solves run as a separate launch over many CTAs
        b.lu_aux_n = (int)nmax;
        if ((rc = h->alloc(&b.lu_invd, nmax * 2 * (size_t)Wk)) ||
            (rc = h->alloc(&b.lu_perm, (nmax + 1) * 2 * (size_t)Wk)))
            return bail(rc);
        cudaMemset(b.lu_perm, 0, (nmax + 1) * 2 * (size_t)Wk * sizeof(int));
    } else if (h->cplx && kvmc::complex_refresh_needs_large(m)) {
        // complex tilde_U factorised in HBM: n x n complex = 2 n^2 doubles per walker-spin
        const size_t nmax = (size_t)std::max(nu, nd);
        b.lu_block = 2 * nmax * nmax;
        if ((rc = h->alloc(&b.lu_scratch, b.lu_block * 2 * (size_t)Wk))) return bail(rc);
    }
    if (h->mixed) cudaMemset(b.W32, 0, wblock * Wk * sizeof(float));
    else cudaMemset(b.W64, 0, wblock * Wk * sizeof(double));
    cudaMemset(b.kappa_up, 0, (size_t)Wk * N * 2);
    cudaMemset(b.kappa_dn, 0, (size_t)Wk * N * 2);
    cudaMemset(b.t, 0, Wk * 8);
    cudaMemset(b.t_end, 0, Wk * 8);
    cudaMemset(b.acc_end, 0, Wk * 8);
    cudaMemset(b.since, 0, Wk * 4);
    cudaMemset(b.status, 0, Wk * 4);
    cudaMemset(b.drift, 0, Wk * 4);
    cudaMemset(b.refresh_count, 0, 16);
    if (int e = kvmc_reset_stats(h)) return bail(e);
    // shared-memory capacity decides whether the FP32 W can be staged on chip
    const int optin = kvmc::max_smem_optin(h->device);
    const size_t rsm = h->cplx ? kvmc::complex_refresh_smem(m)
                               : kvmc::refresh_needs_large(m) ? kvmc::refresh_large_smem(m) : kvmc::refresh_smem(m);
    if ((size_t)optin < rsm + 1024)
        return bail(h->fail(KVMC_ERR_UNSUPPORTED, "refresh needs %zu B shared memory, device offers %d", rsm, optin));
    // where the mixed form keeps W: on chip when it fits (or when asked), else in HBM
    const int place = batch->w_placement;
    if (place < KVMC_W_AUTO || place > KVMC_W_HBM)
        return bail(h->fail(KVMC_ERR_ARGUMENT, "w_placement must be 0, 1 or 2 (got %d)", place));
    const bool fits = h->mixed && !h->cplx && kvmc::mixed_sweep_smem(m) <= (size_t)optin;
    if (place == KVMC_W_ON_CHIP && !fits)
        return bail(h->fail(KVMC_ERR_UNSUPPORTED, "W cannot be kept on chip for this model and precision"));
    h->smem_w = fits && place != KVMC_W_HBM;
    // the FP32 refresh by iterative refinement is the faster periodic refresh of
    // the mixed real form on GB300: one thread per row below 96 orbitals per spin
    // (measured at 27 and 48), in tiles of 32 rows from 96 on (measured at 108,
    // 192 and 432: 1.4x, 3.5x and 2.1x the FP64 refresh) while its tiles fit in
    // shared memory, and from 192 on with its residual and correction products
    // on the tensor cores (measured at 432: 142 against 236 ms for two
    // refreshes of 512 walkers; at 192: 8.8 against 9.7 ms; at 108 as fast as
    // the tiled form), else the FP64 refresh
    if (h->mixed && !h->cplx) {
        const int nmax = std::max(nu, nd);
        if (nmax < 96) h->refresh32 = kvmc::refresh32_supported(m) ? 1 : 0;
        else h->refresh32 = kvmc::refresh_tile_smem(m) + 1024 <= (size_t)optin ? 2 : 0;
        if (nmax >= 192 && kvmc::oz_supported(m, optin)) {
            if (int rc2 = oz_prepare(h)) return bail(rc2);
            h->refresh32 = 3;
        }
    } else {
        h->refresh32 = 0;
    }
    if (h->cplx) {
        // complex orbitals: rank-1 (plain form, or delay_k 1) or delayed updates of depth 4 / 8 with W in HBM
        const int want = batch->delay_k;
        if (want != 0 && want != 1 && want != 4 && want != 8)
            return bail(h->fail(KVMC_ERR_UNSUPPORTED, "complex orbitals: delay_k must be 0, 1, 4 or 8 (got %d)", want));
        h->delay_k = 1;
        if (h->mixed && want != 1) {
            const int k = want == 0 ? 8 : want;
            if (kvmc::complex_delayed_smem(m, k) + 1024 <= (size_t)optin) h->delay_k = k;
            else if (want != 0)
                return bail(h->fail(KVMC_ERR_UNSUPPORTED, "complex delay_k=%d needs %zu B shared memory", k,
                                    kvmc::complex_delayed_smem(m, k)));
        }
    }
    // delayed-update depth: 0 = the largest depth whose working set fits on chip
    // (W with P and Q when W is on chip; P and Q alone when W is in HBM)
    const size_t budget = (size_t)optin - 1024;  // leave room for the kernel's static shared memory
    if (h->mixed && !h->cplx) {
        const int want = batch->delay_k;
        const bool on = h->smem_w;
        // the flush gives each thread four columns: the HBM form (256 threads) needs ld <= 1024
        const bool can_delay = on || std::max(h->ld_up, h->ld_dn) <= 1024;
        if (want == 0) {
            h->delay_k = 1;
            for (int k : {16, 12, 8, 4})
                if (can_delay && kvmc::delayed_smem_bytes(m, k, on) <= budget) { h->delay_k = k; break; }
        } else if (want == 1) {
            h->delay_k = 1;
        } else if ((want == 4 || want == 8 || want == 12 || want == 16) && !can_delay) {
            return bail(h->fail(KVMC_ERR_UNSUPPORTED, "delayed updates with W in HBM support at most 1024 orbitals per spin"));
        } else if (want == 4 || want == 8 || want == 12 || want == 16) {
            if (kvmc::delayed_smem_bytes(m, want, on) > budget)
                return bail(h->fail(KVMC_ERR_UNSUPPORTED, "delay_k=%d needs %zu B shared memory (device offers %d)", want,
                                    kvmc::delayed_smem_bytes(m, want, on), optin));
            h->delay_k = want;
        } else {
            return bail(h->fail(KVMC_ERR_ARGUMENT, "delay_k must be 0, 1, 4, 8, 12 or 16 (got %d)", want));
        }
    }
    for (auto &e : h->region)
        if ((rc = h->cuda(cudaEventCreate(&e), "event"))) return bail(rc);
    if ((rc = h->cuda(cudaDeviceSynchronize(), "create"))) return bail(rc);
    *out = h;
    return KVMC_OK;
}

extern "C" int kvmc_reset_stats(kvmc_handle *h) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    const size_t Wk = h->n_walkers;
    auto &b = h->db;
    cudaMemsetAsync(b.sum_e, 0, Wk * 8, h->stream);
    cudaMemsetAsync(b.sum_e2, 0, Wk * 8, h->stream);
    cudaMemsetAsync(b.n_meas, 0, Wk * 8, h->stream);
    cudaMemsetAsync(b.accepted, 0, Wk * 8, h->stream);
    cudaMemsetAsync(b.proposals, 0, Wk * 8, h->stream);
    if (h->d_gsums) cudaMemsetAsync(h->d_gsums, 0, Wk * h->gsum_stride * 8, h->stream);
    return h->cuda(cudaStreamSynchronize(h->stream), "reset stats");
}

extern "C" int kvmc_init(kvmc_handle *h, const int32_t *kappa_up, const int32_t *kappa_down, int32_t *attempts) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    h->db.compact = 0;   // every walker's W32 is rebuilt below
    const int Wk = h->n_walkers;
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.t, 0, Wk * 8, h->stream), "memset"));
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.status, 0, Wk * 4, h->stream), "memset"));
    if (kappa_up || kappa_down) {
        if (!kappa_up || !kappa_down) return h->fail(KVMC_ERR_ARGUMENT, "give both kappa_up and kappa_down, or neither");
        KV_TRY(upload_kappa(h, kappa_up, kappa_down));
        KV_TRY(full_refresh(h, false));
        if (attempts) for (int w = 0; w < Wk; ++w) attempts[w] = 0;
        return check_status(h, nullptr);
    }
    // seeded random starts, redrawn while tilde_U is singular for either spin:
    // min|pivot| / max|pivot| of its partially pivoted LU at most 1e-8
    std::vector<int> att(Wk, 0), redo(Wk, 1);
    std::vector<double> ld(4 * (size_t)Wk);
    const double min_log_ratio = std::log(1e-8);
    const int max_attempts = 256;
    for (int round = 0; round < max_attempts; ++round) {
        KV_TRY(h->cuda(cudaMemcpyAsync(h->d_attempt, att.data(), Wk * 4, cudaMemcpyHostToDevice, h->stream), "upload"));
        KV_TRY(h->cuda(cudaMemcpyAsync(h->d_redo, redo.data(), Wk * 4, cudaMemcpyHostToDevice, h->stream), "upload"));
        KV_TRY(h->cuda(kvmc::launch_init_random(h->dm, h->db, h->batch.seed, h->d_attempt, h->d_redo, h->stream), "init launch"));
        // refresh only the walkers drawn this round (a negative `since` marks them)
        std::vector<int> mark(Wk);
        for (int w = 0; w < Wk; ++w) mark[w] = redo[w] ? -1 : 0;
        KV_TRY(h->cuda(cudaMemcpyAsync(h->db.since, mark.data(), Wk * 4, cudaMemcpyHostToDevice, h->stream), "upload"));
        // FP64 refresh: the start criterion reads the pivot ratio it records
        KV_TRY(h->cuda(h->cplx ? kvmc::launch_refresh_c(h->dm, h->db, h->mixed, 1, 0, h->stream)
                               : kvmc::launch_refresh(h->dm, h->db, h->mixed, 1, 0, h->stream),
                       "refresh launch"));
        KV_TRY(h->cuda(cudaStreamSynchronize(h->stream), "refresh"));
        KV_TRY(h->cuda(cudaMemcpy(ld.data(), h->db.logdet, ld.size() * 8, cudaMemcpyDeviceToHost), "logdet"));
        int left = 0;
        for (int w = 0; w < Wk; ++w) {
            if (!redo[w]) continue;
            const bool ok = ld[4 * w + 2] > min_log_ratio && ld[4 * w + 3] > min_log_ratio;
            if (ok) redo[w] = 0;
            else { ++att[w]; ++left; }
        }
        if (!left) break;
        if (round == max_attempts - 1)
            return h->fail(KVMC_ERR_SINGULAR, "%d walker(s) found no non-singular start in %d draws", left, max_attempts);
    }
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.status, 0, Wk * 4, h->stream), "memset"));
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.since, 0, Wk * 4, h->stream), "memset"));
    KV_TRY(h->cuda(cudaStreamSynchronize(h->stream), "init"));
    if (attempts) for (int w = 0; w < Wk; ++w) attempts[w] = att[w] + 1;
    return check_status(h, nullptr);
}

extern "C" int kvmc_enable_timing(kvmc_handle *h, int32_t on) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    h->timing = on != 0;
    for (int k = 0; k < 3; ++k) h->t_ms[k] = 0, h->t_launch[k] = 0;
    return KVMC_OK;
}

extern "C" int kvmc_region_timer(kvmc_handle *h, int32_t start, double *ms) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    if (start) return h->cuda(cudaEventRecord(h->region[0], h->stream), "event");
    KV_TRY(h->cuda(cudaEventRecord(h->region[1], h->stream), "event"));
    KV_TRY(h->cuda(cudaEventSynchronize(h->region[1]), "event"));
    float t = 0.f;
    KV_TRY(h->cuda(cudaEventElapsedTime(&t, h->region[0], h->region[1]), "event time"));
    if (ms) *ms = t;
    return KVMC_OK;
}

extern "C" int kvmc_get_config(kvmc_handle *h, int32_t *refresh_interval, int32_t *measure_interval,
                               int32_t *delay_k, int32_t *w_on_chip) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    if (refresh_interval) *refresh_interval = h->refresh_every;
    if (measure_interval) *measure_interval = h->measure_every;
    if (delay_k) *delay_k = h->mixed ? h->delay_k : 1;
    if (w_on_chip) *w_on_chip = h->smem_w ? 1 : 0;
    return KVMC_OK;
}

extern "C" int kvmc_kernel_time(kvmc_handle *h, int32_t kind, double *total_ms, int64_t *launches) {
    if (!h || kind < 0 || kind > 2) return fail_global(KVMC_ERR_ARGUMENT, "bad argument");
    if (total_ms) *total_ms = h->t_ms[kind];
    if (launches) *launches = h->t_launch[kind];
    return KVMC_OK;
}

namespace {

// One launch with optional event timing (kind 0 sweep, 1 refresh, 2 adjoint).  The
// events are only read by collect_timing() after the stream is synchronised.
template <typename F>
int timed(kvmc_handle *h, int kind, F &&launch, const char *what) {
    int first = -1;
    if (h->timing) {
        first = 0;
        for (const auto &u : h->ev_used) first = std::max(first, u.second + 2);
        while ((int)h->ev_pool.size() < first + 2) {
            cudaEvent_t e;
            KV_TRY(h->cuda(cudaEventCreate(&e), "event"));
            h->ev_pool.push_back(e);
        }
        KV_TRY(h->cuda(cudaEventRecord(h->ev_pool[first], h->stream), "event"));
    }
    KV_TRY(h->cuda(launch(), what));
    if (h->timing) {
        KV_TRY(h->cuda(cudaEventRecord(h->ev_pool[first + 1], h->stream), "event"));
        h->ev_used.push_back({kind, first});
    }
    return KVMC_OK;
}

int collect_timing(kvmc_handle *h) {
    for (const auto &u : h->ev_used) {
        float ms = 0.f;
        KV_TRY(h->cuda(cudaEventElapsedTime(&ms, h->ev_pool[u.second], h->ev_pool[u.second + 1]), "event time"));
        h->t_ms[u.first] += ms;
        h->t_launch[u.first] += 1;
    }
    h->ev_used.clear();
    return KVMC_OK;
}

}  // namespace

namespace {

kvmc::SweepParams sweep_params(const kvmc_handle *h) {
    kvmc::SweepParams p{};
    p.seed = h->batch.seed;
    p.accept_rule = h->batch.accept_rule;
    p.refresh_every = h->refresh_every;
    p.measure_every = h->measure_every;
    p.delay_k = h->delay_k;
    p.drift_tol = h->drift_tol;
    p.cluster = h->cluster;
    p.drift_severe = h->drift_severe > 0 ? (float)h->drift_severe * h->drift_tol : std::max(100.f * h->drift_tol, 1e-2f);
    p.stream_threads = h->stream_threads;
    p.pipeline = h->pipeline;
    p.tc_flush = h->tc_flush;
    p.refresh32 = h->refresh32;
    p.warp_walkers = h->warp_walkers;
    p.cond_hi = h->cond_hi;
    p.cond_lo = h->cond_lo;
    return p;
}

// The accounting around one kvmc_sweep / kvmc_advance call.
struct SweepCall {
    int launches = 1;
    int64_t moves = 0;      // kvmc_advance: accepted moves asked of every walker
    int64_t proposals = 0;  // kvmc_sweep: proposals asked of every walker
};

// The call's statistics come from two device reductions of the per-walker
// counters (call_stats_kernel), at its start and at its end, read back in one
// pinned copy at the end.
int sweep_begin(kvmc_handle *h, int64_t proposals_per_walker, int64_t moves_per_walker, bool stats, SweepCall &c) {
    KV_TRY(set_device(h));
    c.moves = proposals_per_walker > 0 ? 0 : moves_per_walker;
    c.proposals = proposals_per_walker;
    if (stats) KV_TRY(h->cuda(kvmc::launch_call_stats(h->db, h->d_stats, h->stream), "stats"));
    KV_TRY(h->cuda(kvmc::launch_set_tend(h->db, proposals_per_walker, moves_per_walker, h->stream), "set t_end"));
    return h->cuda(cudaMemsetAsync(h->db.drift, 0, sizeof(float) * h->n_walkers, h->stream), "memset");
}

// `pairs` (sweep, refresh) launches on the handle's stream; walkers that are
// done return at once.  d_active counts the walkers the last sweep left short.
int enqueue_pairs(kvmc_handle *h, const kvmc::SweepParams &p, int pairs, bool timed_launches) {
    for (int g = 0; g < pairs; ++g) {
        KV_TRY(h->cuda(cudaMemsetAsync(h->d_active, 0, sizeof(int), h->stream), "memset"));
        if (timed_launches) {
            KV_TRY(timed(h, 0, [&] { return sweep_launch(h, p); }, "sweep launch"));
            KV_TRY(timed(h, 1, [&] { return refresh_launch(h, 1, h->mixed ? 1 : 0); }, "refresh launch"));
        } else {
            KV_TRY(h->cuda(sweep_launch(h, p), "sweep launch"));
            KV_TRY(h->cuda(refresh_launch(h, 1, h->mixed ? 1 : 0), "refresh launch"));
        }
    }
    return KVMC_OK;
}

int sweep_end(kvmc_handle *h, kvmc_sweep_stats *stats, SweepCall &c) {
    constexpr int K = kvmc::kCallStats;
    KV_TRY(h->cuda(kvmc::launch_call_stats(h->db, h->d_stats + K, h->stream), "stats"));
    KV_TRY(h->cuda(cudaMemcpyAsync(h->h_stats, h->d_stats, 2 * K * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
                   "stats"));
    KV_TRY(h->cuda(cudaStreamSynchronize(h->stream), "stats"));
    const double *b0 = h->h_stats, *a = h->h_stats + K;
    const int bad = (int)a[5];
    KV_TRY(status_error(h, bad, (int)a[6], (int)a[7]));
    if (c.moves > 0 && a[9] > 0)
        // a walker that used its proposal allowance without making its moves
        return h->fail(KVMC_ERR_NUMERIC,
                       "%d walker(s) made fewer than %lld accepted moves within %lld proposals per move "
                       "(first: walker %d)", (int)a[9], (long long)c.moves, kvmc::kAdvanceProposalsPerMove, (int)a[10]);
    if (!stats) return KVMC_OK;
    std::memset(stats, 0, sizeof *stats);
    stats->proposals = (int64_t)(a[4] - b0[4]);
    stats->accepted = (int64_t)(a[3] - b0[3]);
    stats->measurements = (int64_t)(a[2] - b0[2]);
    stats->sum_energy = a[0] - b0[0];
    stats->sum_energy2 = a[1] - b0[1];
    stats->max_drift = a[8];
    stats->bad_walkers = bad;
    stats->launches = c.launches;
    stats->refreshes = (int64_t)(a[11] - b0[11]);
    stats->fp64_redos = (int64_t)(a[12] - b0[12]);
    return KVMC_OK;
}

bool warp_mode(const kvmc_handle *h) { return h->mixed && !h->cplx && h->warp_walkers > 0; }

// One-warp mode: the sweep and the refreshes work on the label-indexed
// blocks (the refreshes write the blocks while db.compact is set).  The first
// sweep call converts W32 to them; they then stay the state from call to call,
// and W32 is brought back (compact_end, w_current) only by the calls that read
// or write the site-indexed W.
int compact_begin(kvmc_handle *h) {
    if (!warp_mode(h) || h->db.compact) return KVMC_OK;
    KV_TRY(h->cuda(kvmc::launch_warp_convert(h->dm, h->db, true, h->stream), "to label-indexed W"));
    h->db.compact = 1;
    return KVMC_OK;
}

int compact_end(kvmc_handle *h) {
    if (!h->db.compact) return KVMC_OK;
    h->db.compact = 0;
    return h->cuda(kvmc::launch_warp_convert(h->dm, h->db, false, h->stream), "to site-indexed W");
}

// W32 current for a call that reads or writes it (and waits for the
// conversion, since some of those calls copy on the legacy stream)
int w_current(kvmc_handle *h) {
    if (!h->db.compact) return KVMC_OK;
    KV_TRY(compact_end(h));
    return h->cuda(cudaStreamSynchronize(h->stream), "to site-indexed W");
}

// Runs (sweep, refresh) pairs until every walker has reached its target.
int run_pairs(kvmc_handle *h, const kvmc::SweepParams &p, SweepCall &c) {
    // Between host checks the loop issues a group of (sweep, refresh) pairs.
    // A call of a proposal count that one launch covers usually ends with its
    // first pair (the walkers that stop for a refresh go on in the groups
    // after it), so its first group is one pair.
    const int group = h->mixed ? 4 : 8;
    const bool one_launch = c.moves == 0 && c.proposals <= kvmc::kLaunchProposals;
    for (int iter = 0;;) {
        const int g = (iter == 0 && one_launch) ? 1 : group;
        KV_TRY(enqueue_pairs(h, p, g, true));
        c.launches += 2 * g;
        iter += g;
        int active = 0;
        KV_TRY(h->cuda(cudaMemcpyAsync(&active, h->d_active, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "active"));
        KV_TRY(h->cuda(cudaStreamSynchronize(h->stream), "sweep"));
        KV_TRY(collect_timing(h));
        if (active == 0) break;
        if (iter > 100000000) return h->fail(KVMC_ERR_NUMERIC, "sweep made no progress");
    }
    return KVMC_OK;
}

int run_sweep(kvmc_handle *h, int64_t proposals_per_walker, int64_t moves_per_walker, kvmc_sweep_stats *stats) {
    SweepCall c;
    if (proposals_per_walker == 0 && moves_per_walker == 0) {
        KV_TRY(set_device(h));
        if (stats) std::memset(stats, 0, sizeof *stats);
        return KVMC_OK;
    }
    KV_TRY(sweep_begin(h, proposals_per_walker, moves_per_walker, stats != nullptr, c));
    const kvmc::SweepParams p = sweep_params(h);
    KV_TRY(compact_begin(h));
    int rc = KVMC_OK;
    if (moves_per_walker > 0 && warp_mode(h) && h->segment > 0 && h->segment < moves_per_walker) {
        // in segments of `segment` accepted moves per walker: a refresh the
        // accuracy guard asks for waits at most until the segment's end
        for (int64_t done = 0; done < moves_per_walker && rc == KVMC_OK; done += h->segment) {
            const int64_t seg = std::min<int64_t>(h->segment, moves_per_walker - done);
            rc = h->cuda(kvmc::launch_set_tend(h->db, 0, seg, h->stream), "set t_end");
            if (rc == KVMC_OK) rc = run_pairs(h, p, c);
        }
    } else {
        rc = run_pairs(h, p, c);
    }
    if (rc != KVMC_OK) return rc;
    return sweep_end(h, stats, c);
}

}  // namespace

extern "C" int kvmc_sweep(kvmc_handle *h, int64_t proposals_per_walker, kvmc_sweep_stats *stats) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    if (proposals_per_walker < 0) return h->fail(KVMC_ERR_ARGUMENT, "proposals_per_walker must be >= 0");
    return run_sweep(h, proposals_per_walker, 0, stats);
}

extern "C" int kvmc_advance(kvmc_handle *h, int64_t moves_per_walker, kvmc_sweep_stats *stats) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    if (moves_per_walker < 0) return h->fail(KVMC_ERR_ARGUMENT, "moves_per_walker must be >= 0");
    return run_sweep(h, 0, moves_per_walker, stats);
}

// ===========================================================================
// Groups: handles of different sizes advanced together by one CUDA graph
// ===========================================================================

struct kvmc_group {
    std::vector<kvmc_handle *> hs;
    int device = 0;
    cudaStream_t s0 = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> ready, join;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int> pairs;                  // (sweep, refresh) pairs per handle in the graph
    std::vector<kvmc::SweepParams> params;   // the parameters the graph was captured with
    int graph_launches = 0;                  // kernels in one graph launch
    std::string err;
    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        g_last_error = buf;
        return code;
    }
    int cuda(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return KVMC_OK;
        return fail(KVMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
};

extern "C" int kvmc_group_destroy(kvmc_group *g) {
    if (!g) return KVMC_OK;
    cudaSetDevice(g->device);
    if (g->s0) cudaStreamSynchronize(g->s0);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    for (auto e : g->ready) if (e) cudaEventDestroy(e);
    for (auto e : g->join) if (e) cudaEventDestroy(e);
    for (auto e : {g->fork, g->t0, g->t1}) if (e) cudaEventDestroy(e);
    if (g->s0) cudaStreamDestroy(g->s0);
    delete g;
    return KVMC_OK;
}

extern "C" int kvmc_group_create(kvmc_handle *const *handles, int32_t n, kvmc_group **out) {
    if (!handles || !out || n < 1 || n > 64) return fail_global(KVMC_ERR_ARGUMENT, "need 1..64 handles");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!handles[i]) return fail_global(KVMC_ERR_ARGUMENT, "handle %d is null", i);
        if (handles[i]->device != handles[0]->device)
            return fail_global(KVMC_ERR_ARGUMENT, "handles of a group must share one device");
        for (int j = 0; j < i; ++j)
            if (handles[j] == handles[i]) return fail_global(KVMC_ERR_ARGUMENT, "handle %d appears twice", i);
    }
    kvmc_group *g = new kvmc_group();
    g->hs.assign(handles, handles + n);
    g->device = handles[0]->device;
    auto bail = [&](int rc) { kvmc_group_destroy(g); return rc; };
    if (int rc = g->cuda(cudaSetDevice(g->device), "cudaSetDevice")) return bail(rc);
    if (int rc = g->cuda(cudaStreamCreateWithFlags(&g->s0, cudaStreamNonBlocking), "stream")) return bail(rc);
    g->ready.assign(n, nullptr);
    g->join.assign(n, nullptr);
    for (auto *e : {&g->fork, &g->t0, &g->t1})
        if (int rc = g->cuda(cudaEventCreate(e), "event")) return bail(rc);
    for (int i = 0; i < n; ++i) {
        if (int rc = g->cuda(cudaEventCreateWithFlags(&g->ready[i], cudaEventDisableTiming), "event")) return bail(rc);
        if (int rc = g->cuda(cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming), "event")) return bail(rc);
    }
    *out = g;
    return KVMC_OK;
}

namespace {

bool same_params(const kvmc::SweepParams &a, const kvmc::SweepParams &b) {
    return a.seed == b.seed && a.accept_rule == b.accept_rule && a.refresh_every == b.refresh_every &&
           a.measure_every == b.measure_every && a.delay_k == b.delay_k && a.drift_tol == b.drift_tol && a.drift_severe == b.drift_severe && a.cluster == b.cluster &&
           a.stream_threads == b.stream_threads && a.pipeline == b.pipeline && a.tc_flush == b.tc_flush &&
           a.refresh32 == b.refresh32 && a.warp_walkers == b.warp_walkers && a.cond_hi == b.cond_hi &&
           a.cond_lo == b.cond_lo;
}

// Captures one graph: from s0, every handle's stream runs its (sweep,
// refresh) pairs concurrently with the others, then s0 joins them all.
int group_capture(kvmc_group *g, const std::vector<int> &pairs) {
    std::vector<kvmc::SweepParams> params;
    for (auto *h : g->hs) params.push_back(sweep_params(h));
    bool same = g->exec && pairs == g->pairs;
    for (size_t i = 0; same && i < params.size(); ++i) same = same_params(params[i], g->params[i]);
    if (same) return KVMC_OK;
    if (g->exec) { cudaGraphExecDestroy(g->exec); g->exec = nullptr; }
    if (g->graph) { cudaGraphDestroy(g->graph); g->graph = nullptr; }
    KV_TRY(g->cuda(cudaStreamBeginCapture(g->s0, cudaStreamCaptureModeRelaxed), "begin capture"));
    int rc = g->cuda(cudaEventRecord(g->fork, g->s0), "event");
    int launches = 0;
    for (size_t i = 0; i < g->hs.size() && rc == KVMC_OK; ++i) {
        kvmc_handle *h = g->hs[i];
        rc = g->cuda(cudaStreamWaitEvent(h->stream, g->fork, 0), "wait");
        if (rc == KVMC_OK) {
            rc = enqueue_pairs(h, params[i], pairs[i], false);
            if (rc != KVMC_OK) g->err = h->err;
        }
        if (rc == KVMC_OK) rc = g->cuda(cudaEventRecord(g->join[i], h->stream), "event");
        if (rc == KVMC_OK) rc = g->cuda(cudaStreamWaitEvent(g->s0, g->join[i], 0), "wait");
        launches += 2 * pairs[i];
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(g->s0, &graph);
    if (rc != KVMC_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    KV_TRY(g->cuda(e, "end capture"));
    g->graph = graph;
    KV_TRY(g->cuda(cudaGraphInstantiate(&g->exec, g->graph, 0), "graph instantiate"));
    g->pairs = pairs;
    g->params = params;
    g->graph_launches = launches;
    return KVMC_OK;
}

}  // namespace

extern "C" int kvmc_group_advance(kvmc_group *g, int64_t moves_per_walker, kvmc_sweep_stats *stats, double *ms) {
    if (!g) return fail_global(KVMC_ERR_ARGUMENT, "null group");
    if (moves_per_walker < 0) return g->fail(KVMC_ERR_ARGUMENT, "moves_per_walker must be >= 0");
    KV_TRY(g->cuda(cudaSetDevice(g->device), "cudaSetDevice"));
    const size_t n = g->hs.size();
    std::vector<SweepCall> calls(n);
    std::vector<int> pairs(n);
    for (size_t i = 0; i < n; ++i) {
        kvmc_handle *h = g->hs[i];
        if (int rc = sweep_begin(h, 0, moves_per_walker, stats != nullptr, calls[i])) { g->err = h->err; return rc; }
        // one-warp handles: the graph's refreshes are captured writing the label-indexed blocks
        if (int rc = compact_begin(h)) { g->err = h->err; return rc; }
        // enough pairs for every walker to reach its target in one graph launch when no early refresh intervenes
        const int R = h->mixed ? std::max(h->refresh_every, 1) : 1;
        pairs[i] = h->mixed ? (int)std::min<int64_t>(64, moves_per_walker / R + 2) : 8;
    }
    KV_TRY(group_capture(g, pairs));
    // the graph runs after what each handle's stream already holds
    for (size_t i = 0; i < n; ++i) {
        KV_TRY(g->cuda(cudaEventRecord(g->ready[i], g->hs[i]->stream), "event"));
        KV_TRY(g->cuda(cudaStreamWaitEvent(g->s0, g->ready[i], 0), "wait"));
    }
    KV_TRY(g->cuda(cudaEventRecord(g->t0, g->s0), "event"));
    int launches = 0;
    for (int iter = 0;; ++iter) {
        KV_TRY(g->cuda(cudaGraphLaunch(g->exec, g->s0), "graph launch"));
        launches += g->graph_launches;
        KV_TRY(g->cuda(cudaStreamSynchronize(g->s0), "graph"));
        int any = 0;
        for (size_t i = 0; i < n; ++i) {
            int a = 0;
            KV_TRY(g->cuda(cudaMemcpy(&a, g->hs[i]->d_active, sizeof(int), cudaMemcpyDeviceToHost), "active"));
            any += a;
        }
        if (any == 0) break;
        if (iter > 1000000) return g->fail(KVMC_ERR_NUMERIC, "group advance made no progress");
    }
    KV_TRY(g->cuda(cudaEventRecord(g->t1, g->s0), "event"));
    KV_TRY(g->cuda(cudaEventSynchronize(g->t1), "event"));
    if (ms) {
        float t = 0.f;
        KV_TRY(g->cuda(cudaEventElapsedTime(&t, g->t0, g->t1), "event time"));
        *ms = t;
    }
    for (size_t i = 0; i < n; ++i)
        if (int rc = compact_end(g->hs[i])) { g->err = g->hs[i]->err; return rc; }
    for (size_t i = 0; i < n; ++i) {
        kvmc_handle *h = g->hs[i];
        calls[i].launches = launches;
        if (int rc = sweep_end(h, stats ? stats + i : nullptr, calls[i])) { g->err = h->err; return rc; }
    }
    return KVMC_OK;
}

extern "C" int kvmc_group_last_error(const kvmc_group *g, char *buf, size_t len) {
    if (!buf || len == 0) return KVMC_ERR_ARGUMENT;
    const std::string &e = g ? g->err : g_last_error;
    std::snprintf(buf, len, "%s", e.c_str());
    return KVMC_OK;
}

extern "C" int kvmc_measure(kvmc_handle *h, double *local_energy) {
    if (!h || !local_energy) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));
    KV_TRY(h->cuda(h->cplx ? kvmc::launch_measure_c(h->dm, h->db, h->mixed, h->stream)
                           : kvmc::launch_measure(h->dm, h->db, h->mixed, h->stream), "measure launch"));
    KV_TRY(h->cuda(cudaMemcpyAsync(local_energy, h->db.energy_out, sizeof(double) * h->n_walkers,
                                   cudaMemcpyDeviceToHost, h->stream), "measure"));
    return h->cuda(cudaStreamSynchronize(h->stream), "measure");
}

extern "C" int kvmc_eval_ratios(kvmc_handle *h, int32_t n_moves, const int32_t *moves, double *ratios) {
    if (!h || !moves || !ratios || n_moves <= 0) return fail_global(KVMC_ERR_ARGUMENT, "bad argument");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));
    const size_t cnt = (size_t)h->n_walkers * n_moves;
    for (size_t k = 0; k < cnt; ++k) {
        const int32_t *mv = moves + 4 * k;
        if (mv[0] < 0 || mv[0] >= h->n_sites || mv[2] < 0 || mv[2] >= h->n_sites || mv[1] < 1 || mv[1] > h->n_up ||
            mv[3] < 1 || mv[3] > h->n_dn)
            return h->fail(KVMC_ERR_BOUNDS, "move %zu out of range", k);
    }
    void *scr = nullptr;
    const size_t per = h->cplx ? 2 : 1;  // doubles per ratio
    KV_TRY(h->scratch(cnt * 4 * sizeof(int) + cnt * per * sizeof(double) + 256, &scr));
    int *d_moves = static_cast<int *>(scr);
    double *d_out = reinterpret_cast<double *>(static_cast<char *>(scr) + ((cnt * 16 + 255) / 256) * 256);
    KV_TRY(h->cuda(cudaMemcpyAsync(d_moves, moves, cnt * 16, cudaMemcpyHostToDevice, h->stream), "upload"));
    KV_TRY(h->cuda(h->cplx ? kvmc::launch_eval_ratios_c(h->dm, h->db, h->mixed, n_moves, d_moves, d_out, h->stream)
                           : kvmc::launch_eval_ratios(h->dm, h->db, h->mixed, n_moves, d_moves, d_out, h->stream),
                   "ratio launch"));
    KV_TRY(h->cuda(cudaMemcpyAsync(ratios, d_out, cnt * per * 8, cudaMemcpyDeviceToHost, h->stream), "ratios"));
    return h->cuda(cudaStreamSynchronize(h->stream), "ratios");
}

extern "C" int kvmc_apply_moves(kvmc_handle *h, const int32_t *moves) {
    if (!h || !moves) return fail_global(KVMC_ERR_ARGUMENT, "bad argument");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));
    for (int w = 0; w < h->n_walkers; ++w) {
        const int32_t *mv = moves + 5 * (size_t)w;
        if (mv[0] == 0) continue;
        if (mv[0] != 1 && mv[0] != 2) return h->fail(KVMC_ERR_ARGUMENT, "walker %d: flag must be 0, 1 or 2", w);
        if (mv[1] < 0 || mv[1] >= h->n_sites || mv[2] < 0 || mv[2] >= h->n_sites || mv[3] < 1 || mv[3] > h->n_up ||
            mv[4] < 1 || mv[4] > h->n_dn)
            return h->fail(KVMC_ERR_BOUNDS, "walker %d: move out of range", w);
    }
    void *scr = nullptr;
    KV_TRY(h->scratch((size_t)h->n_walkers * 5 * sizeof(int), &scr));
    KV_TRY(h->cuda(cudaMemcpyAsync(scr, moves, (size_t)h->n_walkers * 5 * sizeof(int), cudaMemcpyHostToDevice, h->stream), "upload"));
    KV_TRY(h->cuda(h->cplx ? kvmc::launch_apply_moves_c(h->dm, h->db, h->mixed, static_cast<int *>(scr), h->stream)
                           : kvmc::launch_apply_moves(h->dm, h->db, h->mixed, static_cast<int *>(scr), h->stream),
                   "move launch"));
    return h->cuda(cudaStreamSynchronize(h->stream), "apply moves");
}

extern "C" int kvmc_refresh(kvmc_handle *h) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.status, 0, h->n_walkers * 4, h->stream), "memset"));
    KV_TRY(full_refresh(h, h->mixed, false));   // kvmc_refresh: the FP64 rebuild
    return check_status(h, nullptr);
}

extern "C" int kvmc_get_state(kvmc_handle *h, int32_t *kappa_up, int32_t *kappa_down, int64_t *counters) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    const size_t tot = (size_t)h->n_walkers * h->n_sites;
    int32_t *du = h->d_labels, *dd = h->d_labels + tot;
    KV_TRY(h->cuda(kvmc::launch_labels_convert(du, dd, h->db, h->n_sites, 0, h->stream), "kappa"));
    if (kappa_up) KV_TRY(h->cuda(cudaMemcpyAsync(kappa_up, du, tot * 4, cudaMemcpyDeviceToHost, h->stream), "kappa"));
    if (kappa_down) KV_TRY(h->cuda(cudaMemcpyAsync(kappa_down, dd, tot * 4, cudaMemcpyDeviceToHost, h->stream), "kappa"));
    if (counters)
        KV_TRY(h->cuda(cudaMemcpyAsync(counters, h->db.t, h->n_walkers * 8, cudaMemcpyDeviceToHost, h->stream), "counters"));
    return h->cuda(cudaStreamSynchronize(h->stream), "kappa");
}

extern "C" int kvmc_set_state(kvmc_handle *h, const int32_t *kappa_up, const int32_t *kappa_down, const int64_t *counters) {
    if (!h || !kappa_up || !kappa_down) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    KV_TRY(set_device(h));
    if (counters)
        for (int w = 0; w < h->n_walkers; ++w)
            if (counters[w] < 0) return h->fail(KVMC_ERR_ARGUMENT, "negative counter for walker %d", w);
    KV_TRY(upload_kappa(h, kappa_up, kappa_down));
    if (counters)
        KV_TRY(h->cuda(cudaMemcpy(h->db.t, counters, h->n_walkers * 8, cudaMemcpyHostToDevice), "counters"));
    KV_TRY(h->cuda(cudaMemsetAsync(h->db.status, 0, h->n_walkers * 4, h->stream), "memset"));
    KV_TRY(full_refresh(h, false));
    return check_status(h, nullptr);
}

extern "C" int kvmc_get_w(kvmc_handle *h, double *W_up, double *W_down) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));
    const int N = h->n_sites;
    const size_t cw = h->cplx ? 2 : 1;  // doubles per entry
    const size_t wblock = (size_t)N * (h->ld_up + h->ld_dn) * cw;
    const size_t tot = wblock * h->n_walkers;
    std::vector<double> buf(tot);
    if (h->mixed) {
        std::vector<float> f(tot);
        KV_TRY(h->cuda(cudaMemcpy(f.data(), h->db.W32, tot * 4, cudaMemcpyDeviceToHost), "W"));
        for (size_t e = 0; e < tot; ++e) buf[e] = f[e];
    } else {
        KV_TRY(h->cuda(cudaMemcpy(buf.data(), h->db.W64, tot * 8, cudaMemcpyDeviceToHost), "W"));
    }
    for (int w = 0; w < h->n_walkers; ++w) {
        const double *base = buf.data() + (size_t)w * wblock;
        for (int r = 0; r < N; ++r) {
            if (W_up)
                for (size_t c = 0; c < h->n_up * cw; ++c)
                    W_up[((size_t)w * N + r) * h->n_up * cw + c] = base[(size_t)r * h->ld_up * cw + c];
            if (W_down)
                for (size_t c = 0; c < h->n_dn * cw; ++c)
                    W_down[((size_t)w * N + r) * h->n_dn * cw + c] =
                        base[((size_t)N * h->ld_up + (size_t)r * h->ld_dn) * cw + c];
        }
    }
    return KVMC_OK;
}

extern "C" int kvmc_set_tuning(kvmc_handle *h, int32_t key, int32_t value) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));   // a new launch shape may read W32
    if (key == KVMC_TUNE_STREAM_THREADS) {
        if (value != 128 && value != 256) return h->fail(KVMC_ERR_ARGUMENT, "stream threads must be 128 or 256");
        // the flush gives each thread four columns of one row group
        if (std::max(h->ld_up, h->ld_dn) > 4 * value)
            return h->fail(KVMC_ERR_ARGUMENT, "%d threads cannot flush %d columns", value, std::max(h->ld_up, h->ld_dn));
        h->stream_threads = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_CLUSTER) {
        if (value != 0 && value != 2 && value != 4) return h->fail(KVMC_ERR_ARGUMENT, "cluster size must be 0, 2 or 4");
        if (value > 0) {
            if (!h->mixed || h->cplx || h->delay_k != 1 || h->warp_walkers > 0)
                return h->fail(KVMC_ERR_UNSUPPORTED,
                               "the cluster sweep serves the mixed real form with rank-1 updates (delay_k 1)");
            const size_t need = kvmc::sweep_cluster_smem(h->dm, value);
            if (need + 1024 > (size_t)kvmc::max_smem_optin(h->device))
                return h->fail(KVMC_ERR_UNSUPPORTED, "a cluster of %d CTAs needs %zu B shared memory per CTA", value,
                               need);
        }
        h->cluster = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_DRIFT_SEVERE) {
        if (value < 0) return h->fail(KVMC_ERR_ARGUMENT, "the severe-drift factor must be >= 0");
        h->drift_severe = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_REFRESH32) {
        if (value < 0 || value > 3) return h->fail(KVMC_ERR_ARGUMENT, "refresh32 must be 0, 1, 2 or 3");
        if (value == 3) {
            if (!h->mixed || h->cplx)
                return h->fail(KVMC_ERR_UNSUPPORTED, "the FP32 refresh serves the mixed real form");
            if (!kvmc::oz_supported(h->dm, kvmc::max_smem_optin(h->device)))
                return h->fail(KVMC_ERR_UNSUPPORTED,
                               "the tensor-core residual serves fewer than 1024 orbitals per spin");
            KV_TRY(oz_prepare(h));
        }
        if (value == 2) {
            if (!h->mixed || h->cplx)
                return h->fail(KVMC_ERR_UNSUPPORTED, "the FP32 refresh serves the mixed real form");
            const size_t need = kvmc::refresh_tile_smem(h->dm);
            if (need + 1024 > (size_t)kvmc::max_smem_optin(h->device))
                return h->fail(KVMC_ERR_UNSUPPORTED, "the tiled FP32 refresh needs %zu B shared memory", need);
        }
        if (value == 1) {
            if (!h->mixed || h->cplx)
                return h->fail(KVMC_ERR_UNSUPPORTED, "the FP32 refresh serves the mixed real form");
            const size_t need = kvmc::refresh32_supported(h->dm) ? kvmc::refresh32_smem(h->dm)
                                                                 : kvmc::refresh_large_smem(h->dm, 4);
            if (need + 1024 > (size_t)kvmc::max_smem_optin(h->device))
                return h->fail(KVMC_ERR_UNSUPPORTED, "the FP32 refresh needs %zu B shared memory", need);
            if (!kvmc::refresh32_supported(h->dm) && !h->db.lu_scratch)
                return h->fail(KVMC_ERR_UNSUPPORTED, "no LU scratch for the blocked FP32 refresh");
        }
        h->refresh32 = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_TC_FLUSH) {
        if (value != 0 && value != 1) return h->fail(KVMC_ERR_ARGUMENT, "tensor-core flush must be 0 or 1");
        if (value == 1) {
            if (!h->mixed || h->cplx || h->smem_w || h->delay_k < 4)
                return h->fail(KVMC_ERR_UNSUPPORTED,
                               "the tensor-core flush serves the mixed real form with W in HBM and delayed updates");
            const size_t need = kvmc::delayed_smem_bytes(h->dm, h->delay_k, false) + kvmc::tc_flush_smem_bytes();
            if (need + 1024 > (size_t)kvmc::max_smem_optin(h->device))
                return h->fail(KVMC_ERR_UNSUPPORTED, "the tensor-core flush needs %zu B shared memory", need);
        }
        h->tc_flush = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_WARP_WALKERS) {
        if (value < 0 || value > 14) return h->fail(KVMC_ERR_ARGUMENT, "walkers per CTA must be 0..14");
        if (value > 0) {
            if (!h->mixed || h->cplx || h->delay_k < 4)
                return h->fail(KVMC_ERR_UNSUPPORTED,
                               "one warp per walker serves the mixed real form with delayed updates (delay_k 4..16)");
            const size_t need = kvmc::warp_cta_smem(h->dm) + (size_t)value * kvmc::warp_walker_smem(h->dm, h->delay_k);
            if (need + 1024 > (size_t)kvmc::max_smem_optin(h->device))
                return h->fail(KVMC_ERR_UNSUPPORTED, "%d walkers per CTA need %zu B shared memory (at most %d walkers)",
                               value, need,
                               kvmc::warp_walkers_max(h->dm, h->delay_k, kvmc::max_smem_optin(h->device) - 1024));
            if (!h->db.G32) {
                KV_TRY(set_device(h));
                h->db.g_block = kvmc::warp_compact_block(h->dm);
                KV_TRY(h->alloc(&h->db.G32, h->db.g_block * (size_t)h->n_walkers));
            }
        }
        h->warp_walkers = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_SEGMENT) {
        if (value < 0) return h->fail(KVMC_ERR_ARGUMENT, "segment must be >= 0");
        h->segment = value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_COND_HI || key == KVMC_TUNE_COND_LO) {
        if (value < 0) return h->fail(KVMC_ERR_ARGUMENT, "accuracy guard thresholds must be >= 0");
        (key == KVMC_TUNE_COND_HI ? h->cond_hi : h->cond_lo) = (float)value;
        return KVMC_OK;
    }
    if (key == KVMC_TUNE_PIPELINE) {
        if (value != 0 && value != 1) return h->fail(KVMC_ERR_ARGUMENT, "pipeline must be 0 or 1");
        h->pipeline = value;
        return KVMC_OK;
    }
    return h->fail(KVMC_ERR_ARGUMENT, "unknown tuning key %d", key);
}

extern "C" int kvmc_set_drift_tolerance(kvmc_handle *h, double tol) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    if (!(tol > 0.0)) return h->fail(KVMC_ERR_ARGUMENT, "drift tolerance must be positive");
    h->drift_tol = (float)tol;
    return KVMC_OK;
}

extern "C" int kvmc_walker_drift(kvmc_handle *h, float *drift) {
    if (!h || !drift) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    KV_TRY(set_device(h));
    return h->cuda(cudaMemcpy(drift, h->db.drift, sizeof(float) * h->n_walkers, cudaMemcpyDeviceToHost), "drift");
}

extern "C" int kvmc_walker_stats(kvmc_handle *h, double *sum_e, double *sum_e2, int64_t *n_meas, int64_t *accepted,
                                 int64_t *proposals, int32_t *status) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    KV_TRY(set_device(h));
    const size_t Wk = h->n_walkers;
    auto &b = h->db;
    if (sum_e) KV_TRY(h->cuda(cudaMemcpy(sum_e, b.sum_e, Wk * 8, cudaMemcpyDeviceToHost), "stats"));
    if (sum_e2) KV_TRY(h->cuda(cudaMemcpy(sum_e2, b.sum_e2, Wk * 8, cudaMemcpyDeviceToHost), "stats"));
    if (n_meas) KV_TRY(h->cuda(cudaMemcpy(n_meas, b.n_meas, Wk * 8, cudaMemcpyDeviceToHost), "stats"));
    if (accepted) KV_TRY(h->cuda(cudaMemcpy(accepted, b.accepted, Wk * 8, cudaMemcpyDeviceToHost), "stats"));
    if (proposals) KV_TRY(h->cuda(cudaMemcpy(proposals, b.proposals, Wk * 8, cudaMemcpyDeviceToHost), "stats"));
    if (status) KV_TRY(h->cuda(cudaMemcpy(status, b.status, Wk * 4, cudaMemcpyDeviceToHost), "stats"));
    return KVMC_OK;
}

// ===========================================================================
// Adjoint gradient estimator
// ===========================================================================

extern "C" int kvmc_set_log_derivatives(kvmc_handle *h, int32_t n_params, const double *dU_up,
                                        const double *dU_up_imag, const double *dU_down,
                                        const double *dU_down_imag) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    if (n_params < 1 || n_params > kvmc::kMaxGradParams)
        return h->fail(KVMC_ERR_ARGUMENT, "n_params must be in 1..%d (got %d)", kvmc::kMaxGradParams, n_params);
    if (!dU_up || !dU_down) return h->fail(KVMC_ERR_ARGUMENT, "null orbital derivatives");
    const int N = h->n_sites, P = n_params;
    if (!h->cplx) {
        for (int s = 0; s < 2; ++s) {
            const double *im = s == 0 ? dU_up_imag : dU_down_imag;
            const size_t cnt = (size_t)P * N * (s == 0 ? h->n_up : h->n_dn);
            if (im)
                for (size_t e = 0; e < cnt; ++e)
                    if (im[e] != 0.0)
                        return h->fail(KVMC_ERR_ARGUMENT, "complex orbital derivatives need a handle with complex orbitals");
        }
    }
    KV_TRY(set_device(h));
    // M_a,s = dU_a,s U_s^H in FP64, stored transposed: MT[a][s][R'][R] = M[R, R']
    const size_t NN = (size_t)N * N;
    std::vector<std::complex<double>> MT((size_t)P * 2 * NN);
    for (int s = 0; s < 2; ++s) {
        const int n = s == 0 ? h->n_up : h->n_dn;
        const std::vector<double> &Uh = s == 0 ? h->U_up_host : h->U_dn_host;
        const double *re = s == 0 ? dU_up : dU_down;
        const double *im = s == 0 ? dU_up_imag : dU_down_imag;
        std::vector<std::complex<double>> Ur((size_t)N * n), Dr((size_t)N * n);
        for (int R = 0; R < N; ++R)
            for (int c = 0; c < n; ++c)
                Ur[(size_t)R * n + c] = h->cplx ? std::complex<double>(Uh[2 * ((size_t)R * n + c)], -Uh[2 * ((size_t)R * n + c) + 1])
                                                : std::complex<double>(Uh[(size_t)R * n + c], 0.0);  // conj(U)
        for (int a = 0; a < P; ++a) {
            for (int R = 0; R < N; ++R)
                for (int c = 0; c < n; ++c) {
                    const size_t src = (size_t)a * N * n + (size_t)c * N + R;
                    Dr[(size_t)R * n + c] = std::complex<double>(re[src], im ? im[src] : 0.0);
                }
            std::complex<double> *dst = MT.data() + ((size_t)a * 2 + s) * NN;
            for (int R = 0; R < N; ++R) {
                const std::complex<double> *d = Dr.data() + (size_t)R * n;
                for (int Rp = 0; Rp < N; ++Rp) {
                    const std::complex<double> *u = Ur.data() + (size_t)Rp * n;
                    std::complex<double> acc = 0.0;
                    for (int c = 0; c < n; ++c) acc += d[c] * u[c];
                    dst[(size_t)Rp * N + R] = acc;
                }
            }
        }
    }
    // the working scalar of the handle: (complex) FP64 plain, (complex) FP32 mixed
    const size_t per = (h->cplx ? 2 : 1) * (h->mixed ? 4 : 8);
    std::vector<unsigned char> buf(MT.size() * per);
    for (size_t e = 0; e < MT.size(); ++e) {
        if (h->mixed) {
            float *f = reinterpret_cast<float *>(buf.data()) + e * (h->cplx ? 2 : 1);
            f[0] = (float)MT[e].real();
            if (h->cplx) f[1] = (float)MT[e].imag();
        } else {
            double *d = reinterpret_cast<double *>(buf.data()) + e * (h->cplx ? 2 : 1);
            d[0] = MT[e].real();
            if (h->cplx) d[1] = MT[e].imag();
        }
    }
    if (h->d_MT) { cudaFree(h->d_MT); h->d_MT = nullptr; }
    if (h->d_gsums) { cudaFree(h->d_gsums); h->d_gsums = nullptr; }
    if (h->d_gout) { cudaFree(h->d_gout); h->d_gout = nullptr; }
    h->n_params = 0;
    const size_t Wk = h->n_walkers;
    const size_t L = 3 + 4 * (size_t)P + 2 * (size_t)P * P;
    KV_TRY(h->cuda(cudaMalloc(&h->d_MT, buf.size()), "cudaMalloc"));
    KV_TRY(h->cuda(cudaMalloc(reinterpret_cast<void **>(&h->d_gsums), Wk * L * 8), "cudaMalloc"));
    KV_TRY(h->cuda(cudaMalloc(reinterpret_cast<void **>(&h->d_gout), Wk * (2 + 2 * (size_t)P) * 8), "cudaMalloc"));
    KV_TRY(h->cuda(cudaMemcpy(h->d_MT, buf.data(), buf.size(), cudaMemcpyHostToDevice), "upload"));
    KV_TRY(h->cuda(cudaMemset(h->d_gsums, 0, Wk * L * 8), "memset"));
    h->gsum_stride = L;
    h->n_params = P;
    return KVMC_OK;
}

extern "C" int kvmc_measure_grad(kvmc_handle *h, double *local_energy, double *log_derivative) {
    if (!h) return fail_global(KVMC_ERR_ARGUMENT, "null handle");
    if (h->n_params == 0) return h->fail(KVMC_ERR_ARGUMENT, "kvmc_set_log_derivatives has not been called");
    KV_TRY(set_device(h));
    KV_TRY(w_current(h));
    kvmc::GradModel g{};
    g.n_params = h->n_params;
    g.MT = h->d_MT;
    g.W = h->mixed ? static_cast<const void *>(h->db.W32) : static_cast<const void *>(h->db.W64);
    g.sums = h->d_gsums;
    g.sum_stride = h->gsum_stride;
    g.out = h->d_gout;
    KV_TRY(timed(h, 2, [&] { return kvmc::launch_grad(h->dm, h->db, g, h->mixed, h->cplx, h->batch.accept_rule, h->stream); },
                 "adjoint launch"));
    KV_TRY(h->cuda(cudaStreamSynchronize(h->stream), "adjoint"));
    KV_TRY(collect_timing(h));
    if (local_energy || log_derivative) {
        const size_t Wk = h->n_walkers, row = 2 + 2 * (size_t)h->n_params;
        std::vector<double> o(Wk * row);
        KV_TRY(h->cuda(cudaMemcpy(o.data(), h->d_gout, o.size() * 8, cudaMemcpyDeviceToHost), "adjoint"));
        for (size_t w = 0; w < Wk; ++w) {
            if (local_energy) { local_energy[2 * w] = o[w * row]; local_energy[2 * w + 1] = o[w * row + 1]; }
            if (log_derivative)
                for (size_t k = 0; k < row - 2; ++k) log_derivative[w * (row - 2) + k] = o[w * row + 2 + k];
        }
    }
    return KVMC_OK;
}

extern "C" int kvmc_grad_sums(kvmc_handle *h, double *sums) {
    if (!h || !sums) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    if (h->n_params == 0) return h->fail(KVMC_ERR_ARGUMENT, "kvmc_set_log_derivatives has not been called");
    KV_TRY(set_device(h));
    return h->cuda(cudaMemcpy(sums, h->d_gsums, (size_t)h->n_walkers * h->gsum_stride * 8, cudaMemcpyDeviceToHost),
                   "adjoint sums");
}

extern "C" int kvmc_walker_logdet(kvmc_handle *h, double *logdet) {
    if (!h || !logdet) return fail_global(KVMC_ERR_ARGUMENT, "null argument");
    KV_TRY(set_device(h));
    std::vector<double> ld(4 * (size_t)h->n_walkers);
    KV_TRY(h->cuda(cudaMemcpy(ld.data(), h->db.logdet, ld.size() * 8, cudaMemcpyDeviceToHost), "logdet"));
    for (int w = 0; w < h->n_walkers; ++w) {
        logdet[2 * w] = ld[4 * (size_t)w];
        logdet[2 * w + 1] = ld[4 * (size_t)w + 1];
    }
    return KVMC_OK;
}
