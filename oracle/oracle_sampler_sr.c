/*
 * oracle/oracle_sampler_sr.c -- CPU restatement: samplers, SR solvers, exact
 * diagonalisation.  TEST INFRASTRUCTURE ONLY (see nqs_oracle.h).
 */
#include "nqs_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Upstream xorshift64 single-chain sampler, src/nqs/nqs_sampler.c     */
/* ------------------------------------------------------------------ */

static uint64_t xs_next(uint64_t *s) {                            /* :31-38 */
    uint64_t x = *s;
    x ^= x << 13; x ^= x >> 7; x ^= x << 17;
    *s = x;
    return x;
}

typedef struct {
    const or_amp_t *amp;
    int N;
    int *cur, *prop;
    double cur_la;
    uint64_t rng;
    long acc, pro;
} xs_sampler_t;

static void xs_step(xs_sampler_t *s) {                            /* :86-117 */
    int site = (int)(xs_next(&s->rng) % (uint64_t)s->N);
    memcpy(s->prop, s->cur, sizeof(int) * (size_t)s->N);
    s->prop[site] = -s->prop[site];
    double pl, pa;
    oracle_log_amp_batch(s->amp, s->prop, 1, &pl, &pa);
    double lr = 2.0 * (pl - s->cur_la);
    int accept;
    if (lr >= 0.0) accept = 1;
    else {
        double u = (double)(xs_next(&s->rng) >> 11) * (1.0 / 9007199254740992.0);
        accept = (log(u) < lr);
    }
    s->pro++;
    if (accept) {
        s->acc++;
        int *t = s->cur; s->cur = s->prop; s->prop = t;
        s->cur_la = pl;
    }
}

int oracle_xorshift_sampler(const or_amp_t *amp, int N, unsigned seed,
                            int n_therm, int n_decor, int n, int *out,
                            double *out_acceptance) {
    xs_sampler_t s;
    s.amp = amp; s.N = N;
    s.cur = malloc(sizeof(int) * (size_t)N);
    s.prop = malloc(sizeof(int) * (size_t)N);
    s.rng = seed ? (uint64_t)seed : 0x9E3779B97F4A7C15ULL;        /* :62-63 */
    s.acc = s.pro = 0;
    for (int i = 0; i < N; i++) s.cur[i] = (xs_next(&s.rng) & 1) ? 1 : -1;   /* :70-72 */
    double a;
    oracle_log_amp_batch(amp, s.cur, 1, &s.cur_la, &a);
    for (int t = 0; t < n_therm; t++) xs_step(&s);                /* :119-124 */
    int d = n_decor > 0 ? n_decor : 1;                             /* :126-133 */
    for (int b = 0; b < n; b++) {
        for (int t = 0; t < d; t++) xs_step(&s);
        memcpy(out + (size_t)b * N, s.cur, sizeof(int) * (size_t)N);
    }
    if (out_acceptance) *out_acceptance = s.pro ? (double)s.acc / (double)s.pro : 0.0;
    free(s.cur); free(s.prop);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Multi-chain Philox sampler (extension).                            */
/* Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw,       */
/* "Parallel random numbers: as easy as 1, 2, 3" (SC'11).             */
/* ------------------------------------------------------------------ */

void oracle_philox4x32(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void chain_rand(uint64_t seed, int chain, uint64_t ctr, uint32_t stream, uint32_t r[4]) {
    uint32_t c[4] = {(uint32_t)chain, (uint32_t)ctr, (uint32_t)(ctr >> 32), stream};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    oracle_philox4x32(c, k, r);
}

int oracle_chain_init(const or_chain_opts_t *o, int N, uint64_t *bits) {
    if (N > 64) return -1;
    for (int c = 0; c < o->num_chains; c++) {
        uint32_t r[4];
        if (o->n_down < 0) {
            chain_rand(o->seed, c, 0, 1, r);
            uint64_t b = (uint64_t)r[0] | ((uint64_t)r[1] << 32);
            bits[c] = N == 64 ? b : (b & ((1ULL << N) - 1));
        } else {
            int a[64];
            for (int i = 0; i < N; i++) a[i] = i < o->n_down ? 1 : 0;
            for (int i = N - 1; i >= 1; i--) {                     /* Fisher-Yates */
                chain_rand(o->seed, c, (uint64_t)i, 1, r);
                int j = (int)(((uint64_t)r[0] * (uint64_t)(i + 1)) >> 32);
                int t = a[i]; a[i] = a[j]; a[j] = t;
            }
            uint64_t b = 0;
            for (int i = 0; i < N; i++) if (a[i]) b |= 1ULL << i;
            bits[c] = b;
        }
    }
    return 0;
}

static void bits_to_spins(uint64_t b, int N, int *s) {
    for (int i = 0; i < N; i++) s[i] = ((b >> i) & 1) ? -1 : 1;
}

int oracle_chain_run(const or_chain_opts_t *o, const or_amp_t *amp, const or_ham_t *h,
                     uint64_t *bits, uint64_t *move_counter, int skip,
                     int n_spc, int decor, int *out, long *accepted, long *proposed) {
    int N = amp->base.N, C = o->num_chains;
    int bd[4096];
    int nb = 0;
    if (o->move == 1) {
        nb = oracle_bonds(h, bd, 2048);
        if (nb <= 0) return -1;
    }
    int *s = malloc(sizeof(int) * (size_t)N);
    long acc = 0, pro = 0;
    uint64_t m0 = *move_counter;
    int per = decor > 0 ? decor : 1;
    for (int c = 0; c < C; c++) {
        uint64_t b = bits[c], m = m0;
        bits_to_spins(b, N, s);
        double la, ar;
        oracle_log_amp_batch(amp, s, 1, &la, &ar);
        int total = skip + n_spc * per;
        for (int t = 0; t < total; t++, m++) {
            uint32_t r[4];
            chain_rand(o->seed, c, m, 0, r);
            uint64_t nbits;
            pro++;
            if (o->move == 1) {
                int k = (int)(((uint64_t)r[0] * (uint64_t)nb) >> 32);
                int u = bd[2 * k], v = bd[2 * k + 1];
                if (((b >> u) & 1) == ((b >> v) & 1)) goto record;
                nbits = b ^ (1ULL << u) ^ (1ULL << v);
            } else {
                int site = (int)(((uint64_t)r[0] * (uint64_t)N) >> 32);
                nbits = b ^ (1ULL << site);
            }
            {
                bits_to_spins(nbits, N, s);
                double pl, pa;
                oracle_log_amp_batch(amp, s, 1, &pl, &pa);
                double lr = 2.0 * (pl - la);
                int accept = 1;
                if (!(lr >= 0.0)) {
                    uint64_t u53 = (((uint64_t)r[2] << 32) | r[3]) >> 11;
                    double u = (double)u53 * (1.0 / 9007199254740992.0);
                    accept = (log(u) < lr);
                }
                if (accept) { acc++; b = nbits; la = pl; }
            }
        record:
            if (t >= skip && ((t - skip + 1) % per) == 0 && out) {
                int k = (t - skip + 1) / per - 1;
                bits_to_spins(b, N, out + ((size_t)k * C + c) * N);
            }
        }
        bits[c] = b;
    }
    *move_counter = m0 + (uint64_t)(skip + n_spc * per);
    if (accepted) *accepted += acc;
    if (proposed) *proposed += pro;
    free(s);
    return 0;
}

/* ------------------------------------------------------------------ */
/* SR solvers on a fixed batch                                         */
/* ------------------------------------------------------------------ */

static double vdot(const double *a, const double *b, long n) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

static int batch_grads(const or_amp_t *amp, int grad_mode, const int *batch, int Ns,
                       double *g) {
    if (grad_mode == 1) return oracle_symproj_gradient_batch(amp, batch, Ns, g);
    return oracle_gradient_batch(&amp->base, batch, Ns, g);
}

/* In-place lower Cholesky, src/nqs/nqs_optimizer.c:1026-1043. */
static int chol_lower(double *A, int n) {
    for (int j = 0; j < n; j++) {
        double d = A[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
        if (!(d > 0.0)) return -1;
        double L = sqrt(d);
        A[(size_t)j * n + j] = L;
        double inv = 1.0 / L;
        for (int i = j + 1; i < n; i++) {
            double s = A[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
            A[(size_t)i * n + j] = s * inv;
        }
    }
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) A[(size_t)i * n + j] = 0.0;
    return 0;
}

/* L L^T x = b, src/nqs/nqs_optimizer.c:1046-1061. */
static void chol_solve(const double *L, int n, const double *b, double *x) {
    double *z = malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) {
        double s = b[i];
        for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * z[k];
        z[i] = s / L[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = z[i];
        for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * x[k];
        x[i] = s / L[(size_t)i * n + i];
    }
    free(z);
}

int oracle_minsr_step(const or_ham_t *h, const or_amp_t *amp, int grad_mode,
                      const int *batch, int Ns, double shift, double lr,
                      double *params, long P, double *out_E, double *out_delta,
                      or_step_info_t *info) {
    double *E = malloc(sizeof(double) * (size_t)Ns);
    double *g = malloc(sizeof(double) * (size_t)Ns * P);
    double *gm = calloc((size_t)P, sizeof(double));
    double *d = calloc((size_t)P, sizeof(double));
    double *eps = malloc(sizeof(double) * (size_t)Ns);
    double *T = malloc(sizeof(double) * (size_t)Ns * Ns);
    double *y = calloc((size_t)Ns, sizeof(double));
    if (!E || !g || !gm || !d || !eps || !T || !y) return -1;
    oracle_local_energy_batch(h, amp, batch, Ns, E, NULL);       /* :1091 */
    if (batch_grads(amp, grad_mode, batch, Ns, g)) return -1;       /* :1093-1098 */
    double em = 0.0, esq = 0.0;                                    /* :1101-1107 */
    for (int i = 0; i < Ns; i++) { em += E[i]; esq += E[i] * E[i]; }
    em /= (double)Ns; esq /= (double)Ns;
    for (long k = 0; k < P; k++) {                                 /* :1109-1113 */
        double s = 0.0;
        for (int i = 0; i < Ns; i++) s += g[(size_t)i * P + k];
        gm[k] = s / (double)Ns;
    }
    for (int i = 0; i < Ns; i++) eps[i] = E[i] - em;
    for (int i = 0; i < Ns; i++)                                   /* :1123-1126 */
        for (long k = 0; k < P; k++) g[(size_t)i * P + k] -= gm[k];
    double inv = 1.0 / (double)Ns;
    for (int i = 0; i < Ns; i++) {                                 /* :1134-1146 */
        for (int j = 0; j <= i; j++) {
            double s = 0.0;
            const double *gi = g + (size_t)i * P, *gj = g + (size_t)j * P;
            for (long k = 0; k < P; k++) s += gi[k] * gj[k];
            double t = s * inv;
            T[(size_t)i * Ns + j] = t;
            T[(size_t)j * Ns + i] = t;
        }
        T[(size_t)i * Ns + i] += shift;
    }
    int conv = 0;                                                  /* :1150-1170 */
    int rc = chol_lower(T, Ns);
    if (rc != 0) {
        for (int i = 0; i < Ns; i++) T[(size_t)i * Ns + i] += 1e-6;
        rc = chol_lower(T, Ns);
    }
    if (rc == 0) { chol_solve(T, Ns, eps, y); conv = 1; }
    else memset(y, 0, sizeof(double) * (size_t)Ns);
    for (long k = 0; k < P; k++) {                                 /* :1172-1177 */
        double s = 0.0;
        for (int i = 0; i < Ns; i++) s += g[(size_t)i * P + k] * y[i];
        d[k] = s * inv;
    }
    for (long k = 0; k < P; k++) params[k] += -lr * d[k];          /* :1180 */
    if (info) {
        info->mean_energy = em;
        info->variance_energy = esq - em * em;
        info->update_norm = sqrt(vdot(d, d, P)) * lr;
        info->cg_iterations = 0;
        info->converged = conv;
    }
    if (out_E) memcpy(out_E, E, sizeof(double) * (size_t)Ns);
    if (out_delta) memcpy(out_delta, d, sizeof(double) * (size_t)P);
    free(E); free(g); free(gm); free(d); free(eps); free(T); free(y);
    return 0;
}

/* (S + eps I) v, src/nqs/nqs_optimizer.c:44-80 */
static void qgt_apply(const double *O, long Ns, long P, const double *gm, double eps,
                      const double *v, double *out, double *u) {
    for (long i = 0; i < Ns; i++) {
        u[i] = 0.0;
        for (long k = 0; k < P; k++) u[i] += O[i * P + k] * v[k];
    }
    double um = 0.0;
    for (long i = 0; i < Ns; i++) um += u[i];
    um /= (double)Ns;
    for (long k = 0; k < P; k++) {
        double s = 0.0;
        for (long i = 0; i < Ns; i++) s += O[i * P + k] * u[i];
        out[k] = (s / (double)Ns) - gm[k] * um;
        out[k] += eps * v[k];
    }
}

int oracle_cgsr_step(const or_ham_t *h, const or_amp_t *amp, int grad_mode,
                     const int *batch, int Ns, double shift, double lr,
                     int max_iters, double tol, double *params, long P,
                     double *out_E, double *out_delta, or_step_info_t *info) {
    double *E = malloc(sizeof(double) * (size_t)Ns);
    double *g = malloc(sizeof(double) * (size_t)Ns * P);
    double *gm = calloc((size_t)P, sizeof(double));
    double *F = calloc((size_t)P, sizeof(double));
    double *d = calloc((size_t)P, sizeof(double));
    double *r = malloc(sizeof(double) * (size_t)P), *p = malloc(sizeof(double) * (size_t)P);
    double *Ap = malloc(sizeof(double) * (size_t)P), *u = malloc(sizeof(double) * (size_t)Ns);
    oracle_local_energy_batch(h, amp, batch, Ns, E, NULL);       /* :185-186 */
    if (batch_grads(amp, grad_mode, batch, Ns, g)) return -1;
    double em = 0.0, esq = 0.0;                                    /* :196-204 */
    for (int i = 0; i < Ns; i++) { em += E[i]; esq += E[i] * E[i]; }
    em /= (double)Ns; esq /= (double)Ns;
    for (long k = 0; k < P; k++) {                                 /* :206-216 */
        double sg = 0.0, sge = 0.0;
        for (int i = 0; i < Ns; i++) {
            double x = g[(size_t)i * P + k];
            sg += x; sge += x * E[i];
        }
        gm[k] = sg / (double)Ns;
        F[k] = (sge / (double)Ns) - gm[k] * em;
    }
    /* cg_solve, :84-139 */
    memcpy(r, F, sizeof(double) * (size_t)P);
    memcpy(p, r, sizeof(double) * (size_t)P);
    double rs_old = vdot(r, r, P), rs0 = rs_old;
    int it, conv = 0;
    for (it = 0; it < max_iters; it++) {
        qgt_apply(g, Ns, P, gm, shift, p, Ap, u);
        double pAp = vdot(p, Ap, P);
        if (!(fabs(pAp) >= 1e-30)) break;
        double alpha = rs_old / pAp;
        for (long k = 0; k < P; k++) d[k] += alpha * p[k];
        for (long k = 0; k < P; k++) r[k] += -alpha * Ap[k];
        double rs_new = vdot(r, r, P);
        if (rs_new <= tol * tol * rs0) { conv = 1; it++; break; }
        double beta = rs_new / rs_old;
        for (long k = 0; k < P; k++) p[k] = r[k] + beta * p[k];
        rs_old = rs_new;
    }
    for (long k = 0; k < P; k++) params[k] += -lr * d[k];          /* :227 */
    if (info) {
        info->mean_energy = em;
        info->variance_energy = esq - em * em;
        info->update_norm = sqrt(vdot(d, d, P)) * fabs(lr);
        info->cg_iterations = it;
        info->converged = conv;
    }
    if (out_E) memcpy(out_E, E, sizeof(double) * (size_t)Ns);
    if (out_delta) memcpy(out_delta, d, sizeof(double) * (size_t)P);
    free(E); free(g); free(gm); free(F); free(d); free(r); free(p); free(Ap); free(u);
    return 0;
}

/* Holomorphic SR: the step of src/nqs/nqs_optimizer.c:415-524 on a given
 * batch.  G v (qgt_complex_apply, :317-356) and the CG (cg_solve_complex,
 * :358-401) as upstream. */
static void qgt_complex_apply(const double *R, const double *I, long Ns, long P, const double *Rm,
                              const double *Im, double eps, const double *v, double *out,
                              double *uR, double *uI) {
    for (long i = 0; i < Ns; i++) {
        double sR = 0.0, sI = 0.0;
        for (long k = 0; k < P; k++) {
            sR += R[i * P + k] * v[k];
            sI += I[i * P + k] * v[k];
        }
        uR[i] = sR; uI[i] = sI;
    }
    double mR = 0.0, mI = 0.0;
    for (long i = 0; i < Ns; i++) { mR += uR[i]; mI += uI[i]; }
    mR /= (double)Ns; mI /= (double)Ns;
    for (long k = 0; k < P; k++) {
        double aR = 0.0, aI = 0.0;
        for (long i = 0; i < Ns; i++) {
            aR += R[i * P + k] * uR[i];
            aI += I[i * P + k] * uI[i];
        }
        out[k] = 2.0 * ((aR + aI) / (double)Ns - Rm[k] * mR - Im[k] * mI) + eps * v[k];
    }
}

/* The holomorphic family on one batch: mode 0 holomorphic SR (src/nqs/nqs_optimizer.c:415-524),
 * 1 excited-state SR (the penalty of :600-658 on top of mode 0; ref and mu used), 2 the
 * real-time tVMC force with theta += dt delta (:888-993; lr carries -dt). */
static int holo_family_step(const or_ham_t *h, const or_amp_t *amp, const or_amp_t *ref, double mu, int mode,
                            int grad_sym, const int *batch, int Ns, double shift, double lr, int max_iters,
                            double tol, double *params, long P, double *out_E, double *out_delta,
                            or_step_info_t *info);

int oracle_holo_step(const or_ham_t *h, const or_amp_t *amp, const int *batch, int Ns,
                     double shift, double lr, int max_iters, double tol,
                     double *params, long P, double *out_E, double *out_delta, or_step_info_t *info) {
    return holo_family_step(h, amp, NULL, 0.0, 0, 0, batch, Ns, shift, lr, max_iters, tol, params, P, out_E,
                            out_delta, info);
}

int oracle_holo_step_grad(const or_ham_t *h, const or_amp_t *amp, int grad_sym, const int *batch, int Ns,
                          double shift, double lr, int max_iters, double tol, double *params, long P,
                          double *out_E, double *out_delta, or_step_info_t *info) {
    return holo_family_step(h, amp, NULL, 0.0, 0, grad_sym, batch, Ns, shift, lr, max_iters, tol, params, P,
                            out_E, out_delta, info);
}

int oracle_excited_step(const or_ham_t *h, const or_amp_t *amp, const or_amp_t *ref, double mu,
                        const int *batch, int Ns, double shift, double lr, int max_iters, double tol,
                        double *params, long P, double *out_E, double *out_delta, or_step_info_t *info) {
    return holo_family_step(h, amp, ref, mu, 1, 0, batch, Ns, shift, lr, max_iters, tol, params, P, out_E,
                            out_delta, info);
}

int oracle_tvmc_step(const or_ham_t *h, const or_amp_t *amp, const int *batch, int Ns, double shift,
                     double dt, int max_iters, double tol, double *params, long P, double *out_E,
                     double *out_delta, or_step_info_t *info) {
    return holo_family_step(h, amp, NULL, 0.0, 2, 0, batch, Ns, shift, -dt, max_iters, tol, params, P, out_E,
                            out_delta, info);
}

static int holo_family_step(const or_ham_t *h, const or_amp_t *amp, const or_amp_t *ref, double mu, int mode,
                            int grad_sym, const int *batch, int Ns, double shift, double lr, int max_iters,
                            double tol, double *params, long P, double *out_E, double *out_delta,
                            or_step_info_t *info) {
    double *Er = malloc(sizeof(double) * (size_t)Ns), *Ei = malloc(sizeof(double) * (size_t)Ns);
    double *R = malloc(sizeof(double) * (size_t)Ns * P), *I = malloc(sizeof(double) * (size_t)Ns * P);
    double *Rm = calloc((size_t)P, sizeof(double)), *Im = calloc((size_t)P, sizeof(double));
    double *F = calloc((size_t)P, sizeof(double)), *d = calloc((size_t)P, sizeof(double));
    double *r = malloc(sizeof(double) * (size_t)P), *p = malloc(sizeof(double) * (size_t)P);
    double *Ap = malloc(sizeof(double) * (size_t)P);
    double *uR = malloc(sizeof(double) * (size_t)Ns), *uI = malloc(sizeof(double) * (size_t)Ns);
    oracle_local_energy_batch(h, amp, batch, Ns, Er, Ei);               /* :455-456 */
    if (grad_sym ? oracle_symproj_gradient_complex_batch(amp, batch, Ns, R, I)
                 : oracle_gradient_complex_batch(&amp->base, batch, Ns, R, I)) return -1;   /* :458-469 */
    double erm = 0.0, eim = 0.0, ersq = 0.0;                           /* :471-481 */
    for (int i = 0; i < Ns; i++) { erm += Er[i]; eim += Ei[i]; ersq += Er[i] * Er[i]; }
    erm /= (double)Ns; eim /= (double)Ns; ersq /= (double)Ns;
    double erm_f = erm, eim_f = eim;                  /* the means the force uses */
    if (mode == 1) {                                  /* :600-658: penalty mu r conj(<r>) */
        double *rr = malloc(sizeof(double) * (size_t)Ns), *ri = malloc(sizeof(double) * (size_t)Ns);
        double *la = malloc(sizeof(double) * (size_t)Ns), *ar = malloc(sizeof(double) * (size_t)Ns);
        double *lb = malloc(sizeof(double) * (size_t)Ns), *br = malloc(sizeof(double) * (size_t)Ns);
        oracle_log_amp_batch(amp, batch, Ns, la, ar);
        oracle_log_amp_batch(ref, batch, Ns, lb, br);
        double Rr = 0.0, Ri = 0.0;
        for (int i = 0; i < Ns; i++) {
            double dl = lb[i] - la[i];
            if (dl > 10.0) dl = 10.0;
            if (dl < -10.0) dl = -10.0;
            double m = exp(dl), th = br[i] - ar[i];
            rr[i] = m * cos(th);
            ri[i] = m * sin(th);
            Rr += rr[i];
            Ri += ri[i];
        }
        Rr /= (double)Ns;
        Ri /= (double)Ns;
        for (int i = 0; i < Ns; i++) {
            Er[i] += mu * (rr[i] * Rr + ri[i] * Ri);
            Ei[i] += mu * (ri[i] * Rr - rr[i] * Ri);
        }
        erm_f = erm + mu * (Rr * Rr + Ri * Ri);
        eim_f = eim + mu * (Ri * Rr - Rr * Ri);
        free(rr); free(ri); free(la); free(ar); free(lb); free(br);
    }
    for (long k = 0; k < P; k++) {                                     /* :483-498 */
        double sR = 0.0, sI = 0.0, sRe = 0.0, sIe = 0.0, sRi = 0.0, sIr = 0.0;
        for (int i = 0; i < Ns; i++) {
            double rk = R[(size_t)i * P + k], ik = I[(size_t)i * P + k];
            sR += rk; sI += ik; sRe += rk * Er[i]; sIe += ik * Ei[i];
            sRi += rk * Ei[i]; sIr += ik * Er[i];
        }
        Rm[k] = sR / (double)Ns;
        Im[k] = sI / (double)Ns;
        if (mode == 2)                                                 /* :929-941 */
            F[k] = 2.0 * ((sRi - sIr) / (double)Ns - Rm[k] * eim + Im[k] * erm);
        else
            F[k] = 2.0 * ((sRe + sIe) / (double)Ns - Rm[k] * erm_f - Im[k] * eim_f);
    }
    memcpy(r, F, sizeof(double) * (size_t)P);                          /* cg_solve_complex */
    memcpy(p, r, sizeof(double) * (size_t)P);
    double rs_old = vdot(r, r, P), rs0 = rs_old;
    int it, conv = 0;
    for (it = 0; it < max_iters; it++) {
        qgt_complex_apply(R, I, Ns, P, Rm, Im, shift, p, Ap, uR, uI);
        double pAp = vdot(p, Ap, P);
        if (!(fabs(pAp) >= 1e-30)) break;
        double alpha = rs_old / pAp;
        for (long k = 0; k < P; k++) d[k] += alpha * p[k];
        for (long k = 0; k < P; k++) r[k] += -alpha * Ap[k];
        double rs_new = vdot(r, r, P);
        if (rs_new <= tol * tol * rs0) { conv = 1; it++; break; }
        double beta = rs_new / rs_old;
        for (long k = 0; k < P; k++) p[k] = r[k] + beta * p[k];
        rs_old = rs_new;
    }
    for (long k = 0; k < P; k++) params[k] += -lr * d[k];             /* :503 */
    if (info) {
        info->mean_energy = erm;
        info->variance_energy = ersq - erm * erm;
        info->update_norm = sqrt(vdot(d, d, P)) * fabs(lr);
        info->cg_iterations = it;
        info->converged = conv;
    }
    if (out_E) memcpy(out_E, Er, sizeof(double) * (size_t)Ns);
    if (out_delta) memcpy(out_delta, d, sizeof(double) * (size_t)P);
    free(Er); free(Ei); free(R); free(I); free(Rm); free(Im); free(F); free(d);
    free(r); free(p); free(Ap); free(uR); free(uI);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Exact ground-state energy                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    const or_ham_t *h;
    int N, nb, nd;
    int bd[2048], dd[2048];
    int n_down;                /* < 0: full basis */
    long dim;
    uint64_t *states;          /* sector basis, ascending */
    long *binom;               /* (N+1) x (N+1) */
} ed_t;

static long ed_rank(const ed_t *e, uint64_t s) {
    if (e->n_down < 0) return (long)s;
    /* combinatorial number system: rank = sum_k C(p_k, k+1) over set bits p_0<p_1<... */
    long r = 0;
    int k = 0;
    for (int p = 0; p < e->N; p++)
        if ((s >> p) & 1) { k++; r += e->binom[p * (e->N + 1) + k]; }
    return r;
}

static void ed_matvec(const ed_t *e, const double *in, double *out) {
    const or_ham_t *h = e->h;
    for (long r = 0; r < e->dim; r++) {
        uint64_t s = e->n_down < 0 ? (uint64_t)r : e->states[r];
        double y = 0.0;
        if (h->ham == OR_TFIM) {
            double dg = 0.0;
            for (int b = 0; b < e->nb; b++) {
                int su = ((s >> e->bd[2 * b]) & 1) ? -1 : 1, sv = ((s >> e->bd[2 * b + 1]) & 1) ? -1 : 1;
                dg += -h->J * (double)(su * sv);
            }
            y = dg * in[r];
            for (int i = 0; i < e->N; i++) y += -h->Gamma * in[ed_rank(e, s ^ (1ULL << i))];
        } else {
            double Jxy = h->J, Jz = (h->ham == OR_XXZ) ? h->Jz : h->J;
            double dg = 0.0;
            for (int pass = 0; pass < 2; pass++) {
                const int *B = pass ? e->dd : e->bd;
                int n = pass ? e->nd : e->nb;
                double jx = pass ? h->J2 : Jxy, jz = pass ? h->J2 : Jz;
                for (int b = 0; b < n; b++) {
                    int u = B[2 * b], v = B[2 * b + 1];
                    int su = ((s >> u) & 1) ? -1 : 1, sv = ((s >> v) & 1) ? -1 : 1;
                    dg += 0.25 * jz * (double)(su * sv);
                    if (su != sv) y += 0.5 * jx * in[ed_rank(e, s ^ (1ULL << u) ^ (1ULL << v))];
                }
            }
            y += dg * in[r];
        }
        out[r] = y;
    }
}

/* smallest eigenvalue of the symmetric tridiagonal (a, b) by Sturm bisection */
static double tri_min_eig(const double *a, const double *b, int k) {
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < k; i++) {
        double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < k ? fabs(b[i]) : 0.0);
        if (a[i] - r < lo) lo = a[i] - r;
        if (a[i] + r > hi) hi = a[i] + r;
    }
    for (int it = 0; it < 200; it++) {
        double mid = 0.5 * (lo + hi);
        int cnt = 0;
        double q = 1.0;
        for (int i = 0; i < k; i++) {
            q = a[i] - mid - (i > 0 ? b[i - 1] * b[i - 1] / q : 0.0);
            if (q == 0.0) q = 1e-300;
            if (q < 0.0) cnt++;
        }
        if (cnt >= 1) hi = mid; else lo = mid;
    }
    return 0.5 * (lo + hi);
}

int oracle_exact_energy(const or_ham_t *h, int n_down, int max_iters, double tol,
                        double *out_e0) {
    ed_t *e = calloc(1, sizeof(ed_t));
    e->h = h;
    e->N = oracle_num_sites(h);
    if (e->N > 40) { free(e); return -1; }
    if (h->ham == OR_KAGOME) e->nb = oracle_bonds(h, e->bd, 1024);
    else {
        e->nb = square_bonds_public(h->size_x, h->size_y, h->pbc, e->bd);
        if (h->ham == OR_J1J2) e->nd = diag_bonds_public(h->size_x, h->size_y, h->pbc, e->dd);
    }
    e->n_down = h->ham == OR_TFIM ? -1 : n_down;
    int N = e->N;
    if (e->n_down < 0) e->dim = 1L << N;
    else {
        e->binom = calloc((size_t)(N + 1) * (N + 1), sizeof(long));
        for (int n = 0; n <= N; n++) {
            e->binom[n * (N + 1)] = 1;
            for (int k = 1; k <= n; k++)
                e->binom[n * (N + 1) + k] = e->binom[(n - 1) * (N + 1) + k - 1] +
                                            (k <= n - 1 ? e->binom[(n - 1) * (N + 1) + k] : 0);
        }
        e->dim = e->binom[N * (N + 1) + e->n_down];
        e->states = malloc(sizeof(uint64_t) * (size_t)e->dim);
        long c = 0;
        /* enumerate popcount-k states in ascending order (Gosper's hack) */
        uint64_t s = e->n_down ? ((1ULL << e->n_down) - 1) : 0;
        while (c < e->dim) {
            e->states[c++] = s;
            if (e->n_down == 0) break;
            uint64_t lo = s & (~s + 1), rr = s + lo;
            s = (((rr ^ s) >> 2) / lo) | rr;
        }
    }
    long dim = e->dim;
    int K = max_iters < dim ? max_iters : (int)dim;
    double *V = malloc(sizeof(double) * (size_t)dim * (K + 1));
    double *w = malloc(sizeof(double) * (size_t)dim);
    double *al = calloc((size_t)K + 1, sizeof(double)), *be = calloc((size_t)K + 1, sizeof(double));
    if (!V || !w) return -1;
    uint64_t st = 0x2545F4914F6CDD1DULL;
    double nrm = 0.0;
    for (long i = 0; i < dim; i++) {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        V[i] = (double)(st >> 11) / 9007199254740992.0 - 0.5;
        nrm += V[i] * V[i];
    }
    nrm = sqrt(nrm);
    for (long i = 0; i < dim; i++) V[i] /= nrm;
    double prev = 1e300, ev = 0.0;
    int k;
    for (k = 0; k < K; k++) {
        double *v = V + (size_t)k * dim;
        ed_matvec(e, v, w);
        al[k] = vdot(w, v, dim);
        for (int pass = 0; pass < 2; pass++)                        /* full re-orthogonalisation */
            for (int j = 0; j <= k; j++) {
                double c = vdot(w, V + (size_t)j * dim, dim);
                for (long i = 0; i < dim; i++) w[i] -= c * V[(size_t)j * dim + i];
            }
        double b = sqrt(vdot(w, w, dim));
        be[k] = b;
        ev = tri_min_eig(al, be, k + 1);
        if (fabs(ev - prev) < tol || b < 1e-12) { k++; break; }
        prev = ev;
        for (long i = 0; i < dim; i++) V[(size_t)(k + 1) * dim + i] = w[i] / b;
    }
    *out_e0 = ev;
    free(V); free(w); free(al); free(be); free(e->states); free(e->binom); free(e);
    return 0;
}
