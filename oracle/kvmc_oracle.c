/*
 * kvmc_oracle.c -- C restatement of the KagomeDSL.jl Monte Carlo chain.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path and the timed CPU
 * baseline of bench.py.  Nothing in the product links or calls it.
 *
 * Compiled twice from this file: with -DKVO_COMPLEX the arithmetic is
 * complex double, as the reference's ComplexF64 W (src/MonteCarlo.jl:181-182,
 * src/Hamiltonian.jl:423-425); without it, real double (the B = 0 case).
 *
 * Restates, one chain at a time, single-threaded per chain as the reference
 * (MKL one thread, src/KagomeDSL.jl:9):
 *   kvo_refresh       reevaluateW! + tilde_U   src/MonteCarlo.jl:55-115
 *                     (LU with partial pivoting, tilde_U \ I, then U * inverse)
 *   kvo_update_W      update_W!                 src/MonteCarlo.jl:279-292
 *   kvo_local_energy  getOL                     src/Hamiltonian.jl:593-778
 *   kvo_run_chain     Carlo.sweep! + measure!   src/MonteCarlo.jl:460-634
 * The proposal stream is Philox4x32-10 (Salmon et al., SC'11), the same
 * definition the GPU path uses, keyed by (seed, walker, proposal index).
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef KVO_COMPLEX
#include <complex.h>
typedef double complex scal;
#define KVO_ABS(x) cabs(x)
#define KVO_ABS2(x) (creal(x) * creal(x) + cimag(x) * cimag(x))
#define KVO_RE(x) creal(x)
#else
typedef double scal;
#define KVO_ABS(x) fabs(x)
#define KVO_ABS2(x) ((x) * (x))
#define KVO_RE(x) (x)
#endif

/* ---- Philox4x32-10 ------------------------------------------------------ */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        if (r < 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
}

void kvo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    memcpy(out, ctr, 16);
    philox(out, key[0], key[1]);
}

static void draw(uint64_t seed, int walker, int64_t t, int nb, double *r, int *b) {
    uint32_t c[4] = {(uint32_t)(uint64_t)t, (uint32_t)((uint64_t)t >> 32), (uint32_t)walker, 0u};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t u53 = ((uint64_t)(c[0] >> 5) << 26) | (c[1] >> 6);
    *r = (double)u53 * (1.0 / 9007199254740992.0);
    *b = (int)(((uint64_t)c[2] * (uint64_t)(uint32_t)nb) >> 32);
}

/* ---- W algebra ---------------------------------------------------------- */

/* W = U * (tilde_U \ I); U row-major N x n, kappa values 0 / 1..n.
 * Returns 0, or 1 if tilde_U is exactly singular (the LAPACK info > 0 case). */
int kvo_refresh(int N, int n, const scal *U, const int32_t *kappa, scal *W, double *logdet) {
    scal *A = (scal *)calloc((size_t)n * n, sizeof(scal));
    scal *X = (scal *)calloc((size_t)n * n, sizeof(scal));
    int *piv = (int *)malloc(sizeof(int) * n);
    for (int R = 0; R < N; ++R)
        if (kappa[R] != 0) memcpy(A + (size_t)(kappa[R] - 1) * n, U + (size_t)R * n, sizeof(scal) * n);
    double ld = 0.0;
    int sing = 0;
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = KVO_ABS(A[(size_t)k * n + k]);
        for (int i = k + 1; i < n; ++i) {
            const double v = KVO_ABS(A[(size_t)i * n + k]);
            if (v > best) { best = v; p = i; }
        }
        piv[k] = p;
        if (best == 0.0) { sing = 1; break; }
        if (p != k)
            for (int j = 0; j < n; ++j) {
                scal tmp = A[(size_t)k * n + j];
                A[(size_t)k * n + j] = A[(size_t)p * n + j];
                A[(size_t)p * n + j] = tmp;
            }
        const scal d = A[(size_t)k * n + k];
        ld += log(KVO_ABS(d));
        const scal dinv = 1.0 / d;
        for (int i = k + 1; i < n; ++i) {
            scal *Ai = A + (size_t)i * n;
            const scal l = Ai[k] * dinv;
            Ai[k] = l;
            const scal *Ak = A + (size_t)k * n;
            for (int j = k + 1; j < n; ++j) Ai[j] -= l * Ak[j];
        }
    }
    if (!sing) {
        /* X = tilde_U \ I: apply the row swaps to I, then L and U solves */
        for (int i = 0; i < n; ++i) X[(size_t)i * n + i] = 1.0;
        for (int k = 0; k < n; ++k)
            if (piv[k] != k)
                for (int j = 0; j < n; ++j) {
                    scal tmp = X[(size_t)k * n + j];
                    X[(size_t)k * n + j] = X[(size_t)piv[k] * n + j];
                    X[(size_t)piv[k] * n + j] = tmp;
                }
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < i; ++k) {
                const scal l = A[(size_t)i * n + k];
                for (int j = 0; j < n; ++j) X[(size_t)i * n + j] -= l * X[(size_t)k * n + j];
            }
        for (int i = n - 1; i >= 0; --i) {
            for (int k = i + 1; k < n; ++k) {
                const scal u = A[(size_t)i * n + k];
                for (int j = 0; j < n; ++j) X[(size_t)i * n + j] -= u * X[(size_t)k * n + j];
            }
            const scal dinv = 1.0 / A[(size_t)i * n + i];
            for (int j = 0; j < n; ++j) X[(size_t)i * n + j] *= dinv;
        }
        /* W = U * X */
        for (int R = 0; R < N; ++R) {
            scal *wr = W + (size_t)R * n;
            for (int j = 0; j < n; ++j) wr[j] = 0.0;
            for (int k = 0; k < n; ++k) {
                const scal u = U[(size_t)R * n + k];
                const scal *xk = X + (size_t)k * n;
                for (int j = 0; j < n; ++j) wr[j] += u * xk[j];
            }
        }
    }
    if (logdet) *logdet = sing ? -INFINITY : ld;
    free(A); free(X); free(piv);
    return sing;
}

/* W <- W + alpha * W[:,l] (W[K,:] - e_l), alpha = -1/W[K,l]  (geru!, l, K 0-based) */
void kvo_update_W(int N, int n, scal *W, int l, int K, scal *col, scal *row) {
    for (int c = 0; c < n; ++c) row[c] = W[(size_t)K * n + c];
    row[l] -= 1.0;
    for (int r = 0; r < N; ++r) col[r] = W[(size_t)r * n + l];
    const scal alpha = -1.0 / W[(size_t)K * n + l];
    for (int c = 0; c < n; ++c) row[c] = alpha * row[c]; /* BLAS ger's temp = alpha * y(j) */
    for (int r = 0; r < N; ++r) {
        scal *wr = W + (size_t)r * n;
        const scal x = col[r];
        for (int c = 0; c < n; ++c) wr[c] += x * row[c];
    }
}

/* getOL: diag sum of Sz Sz plus -1/2 W_up * W_down per exchangeable bond orientation */
double kvo_local_energy(int nb, const int32_t *bonds, const int32_t *ku, const int32_t *kd, const scal *Wu, int nu,
                        const scal *Wd, int nd) {
    scal acc = 0.0;
    double diag = 0.0;
    for (int e = 0; e < nb; ++e) {
        const int i = bonds[2 * e], j = bonds[2 * e + 1];
        const int ui = ku[i] != 0, uj = ku[j] != 0;
        diag += (ui == uj) ? 0.25 : -0.25;
        if (uj && kd[i] != 0) acc -= 0.5 * Wu[(size_t)i * nu + ku[j] - 1] * Wd[(size_t)j * nd + kd[i] - 1];
        if (ui && kd[j] != 0) acc -= 0.5 * Wu[(size_t)j * nu + ku[i] - 1] * Wd[(size_t)i * nd + kd[j] - 1];
    }
    return diag + KVO_RE(acc);
}

static int zmu(int nb, const int32_t *bonds, const int32_t *ku, const int32_t *kd) {
    int c = 0;
    for (int e = 0; e < nb; ++e) {
        const int i = bonds[2 * e], j = bonds[2 * e + 1];
        if (ku[i] != 0 && kd[j] != 0) ++c;
        else if (ku[j] != 0 && kd[i] != 0) ++c;
    }
    return c;
}

typedef struct {
    int32_t n_sites, n_up, n_down, n_bonds;
    const int32_t *bonds; /* [nb][2] 0-based */
    const scal *U_up;     /* row-major */
    const scal *U_down;
} kvo_model;

typedef struct {
    int32_t *kappa_up, *kappa_down; /* [N] */
    scal *W_up, *W_down;            /* row-major N x n */
    int64_t t, accepted;
    double sum_e, sum_e2;
    int64_t n_meas;
    int32_t status;                 /* 1 singular refresh */
} kvo_chain;

/* Runs n_proposals proposals (src/MonteCarlo.jl:538-607).  After proposal t
 * (0-based) W is rebuilt when (t+1) % refresh_every == 0 and E_L is recorded
 * when (t+1) % measure_every == 0.  accept_rule 0: the reference's rule
 * (stationary |psi|^2 / Z_mu); 1: Metropolis on a uniform bond.  energies
 * (may be NULL) receives each E_L sample in order. */
int kvo_run_chain(const kvo_model *m, kvo_chain *c, uint64_t seed, int walker, int64_t n_proposals,
                  int refresh_every, int measure_every, int accept_rule, double *energies) {
    const int N = m->n_sites, nu = m->n_up, nd = m->n_down, nb = m->n_bonds;
    scal *col = (scal *)malloc(sizeof(scal) * N);
    scal *row = (scal *)malloc(sizeof(scal) * (nu > nd ? nu : nd));
    int64_t ne = 0;
    for (int64_t q = 0; q < n_proposals; ++q) {
        double r;
        int b;
        draw(seed, walker, c->t, nb, &r, &b);
        c->t += 1;
        double thr = 1.0;
        int proceed = 1;
        if (accept_rule == 0) {
            thr = (double)zmu(nb, m->bonds, c->kappa_up, c->kappa_down) / (double)nb;
            if (r > thr) proceed = 0;
        }
        if (proceed) {
            const int i = m->bonds[2 * b], site = m->bonds[2 * b + 1];
            const int f1 = c->kappa_up[i] != 0 && c->kappa_down[site] != 0;
            const int f2 = c->kappa_up[site] != 0 && c->kappa_down[i] != 0;
            if (f1 || f2) {
                const int flag = f1 ? 1 : 2;
                const int l_up = flag == 1 ? c->kappa_up[i] : c->kappa_up[site];
                const int l_dn = flag == 1 ? c->kappa_down[site] : c->kappa_down[i];
                const int Ku = flag == 1 ? site : i, Kd = flag == 1 ? i : site;
                const scal ratio = c->W_up[(size_t)Ku * nu + l_up - 1] * c->W_down[(size_t)Kd * nd + l_dn - 1];
                const double a = KVO_ABS2(ratio);
                int ok;
                if (accept_rule == 0) ok = (a >= 1.0 && r < thr) || (a < 1.0 && r < thr * a);
                else ok = a >= 1.0 || r < a;
                if (ok) {
                    kvo_update_W(N, nu, c->W_up, l_up - 1, Ku, col, row);
                    kvo_update_W(N, nd, c->W_down, l_dn - 1, Kd, col, row);
                    if (flag == 1) {
                        c->kappa_up[i] = 0; c->kappa_up[site] = l_up;
                        c->kappa_down[i] = l_dn; c->kappa_down[site] = 0;
                    } else {
                        c->kappa_up[i] = l_up; c->kappa_up[site] = 0;
                        c->kappa_down[i] = 0; c->kappa_down[site] = l_dn;
                    }
                    c->accepted += 1;
                }
            }
        }
        if (refresh_every > 0 && c->t % refresh_every == 0) {
            double ld;
            if (kvo_refresh(N, nu, m->U_up, c->kappa_up, c->W_up, &ld) ||
                kvo_refresh(N, nd, m->U_down, c->kappa_down, c->W_down, &ld)) {
                c->status = 1;
                break;
            }
        }
        if (measure_every > 0 && c->t % measure_every == 0) {
            const double e = kvo_local_energy(nb, m->bonds, c->kappa_up, c->kappa_down, c->W_up, nu, c->W_down, nd);
            c->sum_e += e;
            c->sum_e2 += e * e;
            c->n_meas += 1;
            if (energies) energies[ne] = e;
            ++ne;
        }
    }
    free(col);
    free(row);
    return c->status;
}

/* ---- many chains on host threads (the CPU baseline) -------------------- */
typedef struct {
    const kvo_model *m;
    kvo_chain *chains;
    int first, count;
    uint64_t seed;
    int64_t n_proposals;
    int refresh_every, measure_every, accept_rule;
} kvo_job;

static void *worker(void *arg) {
    kvo_job *j = (kvo_job *)arg;
    for (int k = 0; k < j->count; ++k)
        kvo_run_chain(j->m, &j->chains[j->first + k], j->seed, j->first + k, j->n_proposals, j->refresh_every,
                      j->measure_every, j->accept_rule, NULL);
    return NULL;
}

/* Runs chains[0..n_chains) for n_proposals each on n_threads threads (one
 * chain per thread at a time).  Returns wall seconds. */
double kvo_run_chains(const kvo_model *m, kvo_chain *chains, int n_chains, uint64_t seed, int64_t n_proposals,
                      int refresh_every, int measure_every, int accept_rule, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_chains) n_threads = n_chains;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
    kvo_job *jobs = (kvo_job *)malloc(sizeof(kvo_job) * n_threads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int first = 0;
    for (int k = 0; k < n_threads; ++k) {
        const int cnt = n_chains / n_threads + (k < n_chains % n_threads ? 1 : 0);
        jobs[k] = (kvo_job){m, chains, first, cnt, seed, n_proposals, refresh_every, measure_every, accept_rule};
        first += cnt;
        pthread_create(&th[k], NULL, worker, &jobs[k]);
    }
    for (int k = 0; k < n_threads; ++k) pthread_join(th[k], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    free(jobs);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

size_t kvo_scalar_size(void) { return sizeof(scal); }
