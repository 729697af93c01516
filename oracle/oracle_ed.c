/*
 * oracle/oracle_ed.c -- CPU FP64 restatement of the exact-diagonalisation path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; see nqs_oracle.h).  Plain sequential loops in
 * the reference's own order:
 *   the kagome Heisenberg matvec          src/nqs/nqs_lanczos.c:380-432
 *   the sector projector (direct form)    src/nqs/nqs_symproj.c:786-852
 *   the memory-lean projecting Lanczos    src/mps/lanczos.c:824-960
 *   and its eigenvector replay            src/mps/lanczos.c:972-1119
 *   the NQS state on the full basis and its variational energy
 *                                         src/nqs/nqs_lanczos.c:65-149, 151-321, 434-455
 * The tridiagonal eigenproblem is solved here by Sturm bisection (the lowest value) and
 * a dense cyclic Jacobi sweep (the eigenvector) instead of upstream's QL; both give the
 * lowest pair to rounding.
 */
#include "nqs_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static int kg(int cx, int cy, int sub, int Ly) { return 3 * (cx * Ly + cy) + sub; }

/* Bond list of the kagome cluster in the loop order of src/nqs/nqs_lanczos.c:386-431. */
static int kagome_bond_list(int Lx, int Ly, int pbc, int (*bd)[2]) {
    int nb = 0;
    for (int cx = 0; cx < Lx; cx++)
        for (int cy = 0; cy < Ly; cy++) {
            int A = kg(cx, cy, 0, Ly), B = kg(cx, cy, 1, Ly), Cc = kg(cx, cy, 2, Ly);
            bd[nb][0] = A; bd[nb++][1] = B;
            bd[nb][0] = A; bd[nb++][1] = Cc;
            bd[nb][0] = B; bd[nb++][1] = Cc;
            int cxm, cym;
            if (pbc) {
                cxm = (cx - 1 + Lx) % Lx;
                cym = (cy - 1 + Ly) % Ly;
            } else if (cx == 0 || cy == 0) {
                continue;
            } else {
                cxm = cx - 1;
                cym = cy - 1;
            }
            int Bm = kg(cxm, cy, 1, Ly), Cm = kg(cx, cym, 2, Ly);
            bd[nb][0] = A;  bd[nb++][1] = Bm;
            bd[nb][0] = A;  bd[nb++][1] = Cm;
            bd[nb][0] = Bm; bd[nb++][1] = Cm;
        }
    return nb;
}

/* y(s) = E_diag(s) x(s) + sum over antiparallel bonds of (J/2) x(s with both spins flipped),
 * E_diag(s) = (J/4) sum_b s_u s_v: the diagonal first, then the bonds in loop order. */
void oracle_kagome_heis_matvec_range(int Lx, int Ly, double J, int pbc, const double *in, double *out,
                                     long s0, long s1) {
    int bd[6 * 64][2];
    int nb = kagome_bond_list(Lx, Ly, pbc, bd);
    for (long s = s0; s < s1; s++) {
        double diag = 0.0;
        for (int b = 0; b < nb; b++) {
            int su = ((s >> bd[b][0]) & 1) ? -1 : 1, sv = ((s >> bd[b][1]) & 1) ? -1 : 1;
            diag += 0.25 * J * (double)(su * sv);
        }
        double y = diag * in[s];
        for (int b = 0; b < nb; b++) {
            int u = bd[b][0], v = bd[b][1];
            if ((((s >> u) ^ (s >> v)) & 1) != 0) y += 0.5 * J * in[s ^ (1L << u) ^ (1L << v)];
        }
        out[s] = y;
    }
}

void oracle_kagome_heis_matvec(int Lx, int Ly, double J, int pbc, const double *in, double *out) {
    oracle_kagome_heis_matvec_range(Lx, Ly, J, pbc, in, out, 0, 1L << (3 * Lx * Ly));
}

void oracle_sector_project_range(const double *psi, double *out, int N, int G, const int *perm,
                                 const double *chars, long s0, long s1) {
    for (long s = s0; s < s1; s++) {
        double acc = 0.0;
        for (int g = 0; g < G; g++) {
            long src = 0;
            for (int i = 0; i < N; i++) src |= ((s >> perm[(size_t)g * N + i]) & 1L) << i;
            acc += chars[g] * psi[src];
        }
        out[s - s0] = acc / (double)G;
    }
}

void oracle_sector_project(double *psi, int N, int G, const int *perm, const double *chars) {
    long dim = 1L << N;
    double *out = calloc((size_t)dim, sizeof(double));
    oracle_sector_project_range(psi, out, N, G, perm, chars, 0, dim);
    memcpy(psi, out, sizeof(double) * (size_t)dim);
    free(out);
}

static void xorshift_fill(double *v, long dim, uint64_t x) {
    for (long i = 0; i < dim; i++) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        v[i] = (double)(x >> 11) / 9007199254740992.0 - 0.5;
    }
}

void oracle_lanczos_seed(int N, int alternate, double *out) {
    long dim = 1L << N;
    xorshift_fill(out, dim, (alternate ? 0xBEEFBABEULL : 0xA5A5A5A5A5A5A5A5ULL) ^ (uint64_t)dim);
}

static double ed_dot(const double *a, const double *b, long n) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

static double tri_lowest(const double *a, const double *b, int k) {
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < k; i++) {
        double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < k ? fabs(b[i]) : 0.0);
        if (a[i] - r < lo) lo = a[i] - r;
        if (a[i] + r > hi) hi = a[i] + r;
    }
    for (int it = 0; it < 300; it++) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        int cnt = 0;
        double q = 1.0;
        for (int i = 0; i < k; i++) {
            q = a[i] - mid - (i > 0 ? b[i - 1] * b[i - 1] / q : 0.0);
            if (q == 0.0) q = -1e-300;
            if (q < 0.0) cnt++;
        }
        if (cnt >= 1) hi = mid; else lo = mid;
    }
    return 0.5 * (lo + hi);
}

/* Lowest eigenpair of the k x k tridiagonal by cyclic Jacobi rotations on the dense matrix. */
static double tri_lowest_vector(const double *a, const double *b, int k, double *z) {
    double *A = calloc((size_t)k * k, sizeof(double)), *V = calloc((size_t)k * k, sizeof(double));
    for (int i = 0; i < k; i++) {
        A[i * k + i] = a[i];
        if (i + 1 < k) A[i * k + i + 1] = A[(i + 1) * k + i] = b[i];
        V[i * k + i] = 1.0;
    }
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int p = 0; p < k; p++)
            for (int q = p + 1; q < k; q++) off += A[p * k + q] * A[p * k + q];
        if (off < 1e-30) break;
        for (int p = 0; p < k; p++)
            for (int q = p + 1; q < k; q++) {
                double apq = A[p * k + q];
                if (fabs(apq) < 1e-300) continue;
                double theta = (A[q * k + q] - A[p * k + p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < k; r++) {
                    double arp = A[r * k + p], arq = A[r * k + q];
                    A[r * k + p] = c * arp - s * arq;
                    A[r * k + q] = s * arp + c * arq;
                }
                for (int r = 0; r < k; r++) {
                    double apr = A[p * k + r], aqr = A[q * k + r];
                    A[p * k + r] = c * apr - s * aqr;
                    A[q * k + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < k; r++) {
                    double vrp = V[r * k + p], vrq = V[r * k + q];
                    V[r * k + p] = c * vrp - s * vrq;
                    V[r * k + q] = s * vrp + c * vrq;
                }
            }
    }
    int idx = 0;
    for (int i = 1; i < k; i++)
        if (A[i * k + i] < A[idx * k + idx]) idx = i;
    double lam = A[idx * k + idx];
    for (int i = 0; i < k; i++) z[i] = V[i * k + idx];
    free(A);
    free(V);
    return lam;
}

int oracle_lanczos_lean_kagome(int Lx, int Ly, double J, int pbc, const int *perm, const double *chars, int G,
                               int max_iters, double tol, double *out_e, double *out_vec, or_lanczos_info_t *info) {
    int N = 3 * Lx * Ly;
    if (N <= 0 || N > 24 || max_iters <= 0) return -1;
    long dim = 1L << N;
    if (max_iters > dim) max_iters = (int)dim;
    double *vc = calloc((size_t)dim, sizeof(double)), *vp = calloc((size_t)dim, sizeof(double));
    double *w = calloc((size_t)dim, sizeof(double)), *seed = calloc((size_t)dim, sizeof(double));
    double *al = calloc((size_t)max_iters + 1, sizeof(double)), *be = calloc((size_t)max_iters + 2, sizeof(double));
    xorshift_fill(seed, dim, 0xA5A5A5A5A5A5A5A5ULL ^ (uint64_t)dim);
    oracle_sector_project(seed, N, G, perm, chars);
    double n = sqrt(ed_dot(seed, seed, dim));
    if (n < 1e-14) {
        xorshift_fill(seed, dim, 0xBEEFBABEULL ^ (uint64_t)dim);
        oracle_sector_project(seed, N, G, perm, chars);
        n = sqrt(ed_dot(seed, seed, dim));
    }
    if (n > 0) for (long i = 0; i < dim; i++) seed[i] /= n;
    memcpy(vc, seed, sizeof(double) * (size_t)dim);
    double lambda = 0.0, prev = 0.0;
    int K = 0, conv = 0;
    for (int k = 0; k < max_iters; k++) {
        oracle_kagome_heis_matvec(Lx, Ly, J, pbc, vc, w);
        al[k] = ed_dot(vc, w, dim);
        for (long i = 0; i < dim; i++) w[i] -= al[k] * vc[i];
        if (k > 0) for (long i = 0; i < dim; i++) w[i] -= be[k] * vp[i];
        oracle_sector_project(w, N, G, perm, chars);
        be[k + 1] = sqrt(ed_dot(w, w, dim));
        K = k + 1;
        if (be[k + 1] < 1e-14) break;
        prev = lambda;
        lambda = tri_lowest(al, be + 1, K);
        if (k > 5 && fabs(lambda - prev) < tol) { conv = 1; break; }
        memcpy(vp, vc, sizeof(double) * (size_t)dim);
        double inv = 1.0 / be[k + 1];
        for (long i = 0; i < dim; i++) vc[i] = w[i] * inv;
    }
    double lam = lambda;
    if (out_vec) {
        double *z = calloc((size_t)K, sizeof(double));
        lam = tri_lowest_vector(al, be + 1, K, z);
        memset(out_vec, 0, sizeof(double) * (size_t)dim);
        memcpy(vc, seed, sizeof(double) * (size_t)dim);
        for (long i = 0; i < dim; i++) out_vec[i] += z[0] * vc[i];
        for (int k = 0; k + 1 < K; k++) {
            oracle_kagome_heis_matvec(Lx, Ly, J, pbc, vc, w);
            for (long i = 0; i < dim; i++) w[i] -= al[k] * vc[i];
            if (k > 0) for (long i = 0; i < dim; i++) w[i] -= be[k] * vp[i];
            oracle_sector_project(w, N, G, perm, chars);
            if (be[k + 1] < 1e-14) break;
            memcpy(vp, vc, sizeof(double) * (size_t)dim);
            double inv = 1.0 / be[k + 1];
            for (long i = 0; i < dim; i++) vc[i] = w[i] * inv;
            for (long i = 0; i < dim; i++) out_vec[i] += z[k + 1] * vc[i];
        }
        double en = sqrt(ed_dot(out_vec, out_vec, dim));
        if (en > 0) for (long i = 0; i < dim; i++) out_vec[i] *= 1.0 / en;
        conv = (K >= 6 && fabs(lam - prev) < tol);
        free(z);
    }
    *out_e = lam;
    if (info) {
        info->iterations = K;
        info->converged = conv;
        info->residual = out_vec ? (K >= 2 ? fabs(lam - prev) : 0.0) : (K > 0 ? fabs(lam - prev) : 0.0);
        for (int i = 0; i < K && i < OR_LZ_MAX; i++) info->alpha[i] = al[i];
        for (int i = 0; i <= K && i < OR_LZ_MAX + 1; i++) info->beta[i] = be[i];
    }
    free(vc); free(vp); free(w); free(seed); free(al); free(be);
    return 0;
}


/* psi(s) = cos(arg) exp(log|psi| - max), normalised, over the 2^N basis states (bit i of s
 * = 1 <-> spin -1), src/nqs/nqs_lanczos.c:65-106. */
int oracle_materialise(const or_amp_t *amp, int N, double *psi) {
    if (N <= 0 || N > 24) return -1;
    long dim = 1L << N;
    int *spins = malloc(sizeof(int) * (size_t)N);
    double *lp = malloc(sizeof(double) * (size_t)dim), *ag = malloc(sizeof(double) * (size_t)dim);
    double mx = -INFINITY;
    for (long s = 0; s < dim; s++) {
        for (int i = 0; i < N; i++) spins[i] = ((s >> i) & 1) ? -1 : 1;
        oracle_log_amp_batch(amp, spins, 1, &lp[s], &ag[s]);
        if (lp[s] > mx) mx = lp[s];
    }
    double n2 = 0.0;
    for (long s = 0; s < dim; s++) {
        psi[s] = cos(ag[s]) * exp(lp[s] - mx);
        n2 += psi[s] * psi[s];
    }
    double inv = n2 > 0 ? 1.0 / sqrt(n2) : 1.0;
    for (long s = 0; s < dim; s++) psi[s] *= inv;
    free(spins); free(lp); free(ag);
    return 0;
}

/* H x on the full basis of an open Lx x Ly square lattice: kind 0 TFIM
 * -J sum s_i s_j - Gamma sum sigma^x (src/nqs/nqs_lanczos.c:151-184), kind 1 XXZ with
 * J/4 Jz diagonal and J/2 flips (:226-281). */
void oracle_square_matvec(int kind, int Lx, int Ly, double J, double X, const double *in, double *out) {
    int N = Lx * Ly;
    long dim = 1L << N;
    for (long s = 0; s < dim; s++) {
        double e = 0.0;
        for (int x = 0; x < Lx; x++)
            for (int y = 0; y < Ly; y++) {
                int a = x * Ly + y, sa = ((s >> a) & 1) ? -1 : 1;
                int nb[2], k = 0;
                if (x + 1 < Lx) nb[k++] = (x + 1) * Ly + y;
                if (y + 1 < Ly) nb[k++] = x * Ly + y + 1;
                for (int q = 0; q < k; q++) {
                    int sb = ((s >> nb[q]) & 1) ? -1 : 1;
                    e += kind == 0 ? -J * (double)(sa * sb) : 0.25 * X * (double)(sa * sb);
                }
            }
        double y = e * in[s];
        if (kind == 0) {
            for (int i = 0; i < N; i++) y += -X * in[s ^ (1L << i)];
        } else {
            for (int x = 0; x < Lx; x++)
                for (int yy = 0; yy < Ly; yy++) {
                    int a = x * Ly + yy, sa = ((s >> a) & 1) ? -1 : 1;
                    int nb[2], k = 0;
                    if (x + 1 < Lx) nb[k++] = (x + 1) * Ly + yy;
                    if (yy + 1 < Ly) nb[k++] = x * Ly + yy + 1;
                    for (int q = 0; q < k; q++) {
                        int sb = ((s >> nb[q]) & 1) ? -1 : 1;
                        if (sa == -sb) y += 0.5 * J * in[s ^ (1L << a) ^ (1L << nb[q])];
                    }
                }
        }
        out[s] = y;
    }
}

/* <psi|H|psi> / <psi|psi> of the materialised NQS state: ham 0 TFIM (X = Gamma), 1 XXZ
 * (X = Jz) on the open square lattice, 6 kagome Heisenberg (Lx, Ly cells; X unused, pbc)
 * (src/nqs/nqs_lanczos.c:188-224, 283-321, 434-455). */
int oracle_variational_energy(const or_amp_t *amp, int ham, int Lx, int Ly, double J, double X, int pbc,
                              double *out_e) {
    int N = ham == 6 ? 3 * Lx * Ly : Lx * Ly;
    if (N > 24) return -1;
    long dim = 1L << N;
    double *psi = malloc(sizeof(double) * (size_t)dim), *hp = malloc(sizeof(double) * (size_t)dim);
    if (oracle_materialise(amp, N, psi)) { free(psi); free(hp); return -1; }
    if (ham == 6) oracle_kagome_heis_matvec(Lx, Ly, J, pbc, psi, hp);
    else oracle_square_matvec(ham == 0 ? 0 : 1, Lx, Ly, J, X, psi, hp);
    double num = 0.0, den = 0.0;
    for (long s = 0; s < dim; s++) { num += psi[s] * hp[s]; den += psi[s] * psi[s]; }
    *out_e = num / den;
    free(psi); free(hp);
    return 0;
}
