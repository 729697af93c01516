/*
 * oracle/nqs_oracle.c -- CPU FP64 restatement: ansatz, wrappers, local energy.
 *
 * TEST INFRASTRUCTURE ONLY (see nqs_oracle.h).  Loops keep the upstream
 * summation order so that, built with the same flags on the same machine,
 * results agree with the upstream library bit for bit.
 */
#include "nqs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* Parameter layout and initialisation                                 */
/* ------------------------------------------------------------------ */

long oracle_num_params(int kind, int N, int M) {
    long n = N, m = M;
    switch (kind) {
        case OR_MF:   return n;
        case OR_RBM:  return n + m + m * n;                       /* src/nqs/nqs_ansatz.c:88 */
        case OR_CRBM: return 2 * (n + m + m * n);                 /* src/nqs/nqs_ansatz.c:223 */
        case OR_MLP:  return m * n + m + m * m + m + 2 * m + 2;   /* extension */
        case OR_VIT:  return 3 * m + m * m + n + 1;                /* :113-130, m = d */
        case OR_VITC: return 6 * m + 2 * m * m + n + 2;            /* :155-172 */
        default:      return -1;
    }
}

/* xorshift64 uniform and Box-Muller normal used for initialisation,
 * src/nqs/nqs_ansatz.c:47-61. */
static double xs_uniform(uint64_t *s) {
    uint64_t x = *s;
    x ^= x << 13; x ^= x >> 7; x ^= x << 17;
    *s = x;
    return (double)(x >> 11) / 9007199254740992.0;
}
static double xs_gauss(uint64_t *s) {
    double u1 = xs_uniform(s);
    double u2 = xs_uniform(s);
    if (u1 < 1e-15) u1 = 1e-15;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

int oracle_ansatz_init(int kind, int N, int M, double scale, unsigned seed,
                       double *p) {
    if (N <= 0 || !p) return -1;
    uint64_t st = seed ? (uint64_t)seed : 0xDEADBEEFCAFEBABEULL;   /* :73-75 */
    if (scale <= 0.0) scale = 0.01;
    if (kind == OR_MF) {                                          /* :77-87 */
        for (int i = 0; i < N; i++) p[i] = 0.01 * (xs_uniform(&st) - 0.5);
        return 0;
    }
    if (kind == OR_RBM || kind == OR_CRBM) {                      /* :89-110, :219-247 */
        long Pr = (long)N + M + (long)M * N;
        double wstd = scale / sqrt((double)N);
        for (int i = 0; i < N; i++) p[i] = scale * (xs_uniform(&st) - 0.5);
        for (int h = 0; h < M; h++) p[N + h] = scale * (xs_uniform(&st) - 0.5);
        for (long k = 0; k < (long)M * N; k++) p[N + M + k] = wstd * xs_gauss(&st);
        if (kind == OR_CRBM) {
            double is = 0.1 * scale, iw = is / sqrt((double)N);
            for (int i = 0; i < N; i++) p[Pr + i] = is * (xs_uniform(&st) - 0.5);
            for (int h = 0; h < M; h++) p[Pr + N + h] = is * (xs_uniform(&st) - 0.5);
            for (long k = 0; k < (long)M * N; k++) p[Pr + N + M + k] = iw * xs_gauss(&st);
        }
        return 0;
    }
    if (kind == OR_VIT || kind == OR_VITC) {                      /* :131-151, :173-214 (M = d) */
        int d = M;
        double vs = scale / sqrt((double)d), is = 0.1 * scale;
        if (kind == OR_VIT) {
            for (int i = 0; i < d; i++) p[i] = scale * xs_gauss(&st);
            for (int i = 0; i < d; i++) p[d + i] = scale * (xs_uniform(&st) - 0.5);
            for (long k = 0; k < (long)d * d; k++) p[2L * d + k] = vs * xs_gauss(&st);
            long ao = 2L * d + (long)d * d;
            for (int k = 0; k < N; k++) p[ao + k] = scale * (xs_uniform(&st) - 0.5);
            for (int i = 0; i < d; i++) p[ao + N + i] = scale * (xs_uniform(&st) - 0.5);
            p[ao + N + d] = 0.0;
        } else {
            for (int i = 0; i < d; i++) p[i] = scale * xs_gauss(&st);
            for (int i = 0; i < d; i++) p[d + i] = is * xs_gauss(&st);
            for (int i = 0; i < d; i++) p[2 * d + i] = scale * (xs_uniform(&st) - 0.5);
            for (int i = 0; i < d; i++) p[3 * d + i] = is * (xs_uniform(&st) - 0.5);
            long vr = 4L * d, vi = vr + (long)d * d, ao = vi + (long)d * d;
            for (long k = 0; k < (long)d * d; k++) p[vr + k] = vs * xs_gauss(&st);
            for (long k = 0; k < (long)d * d; k++) p[vi + k] = 0.1 * vs * xs_gauss(&st);
            for (int k = 0; k < N; k++) p[ao + k] = scale * (xs_uniform(&st) - 0.5);
            for (int i = 0; i < d; i++) p[ao + N + i] = scale * (xs_uniform(&st) - 0.5);
            for (int i = 0; i < d; i++) p[ao + N + d + i] = is * (xs_uniform(&st) - 0.5);
            p[ao + N + 2 * d] = 0.0;
            p[ao + N + 2 * d + 1] = 0.0;
        }
        return 0;
    }
    if (kind == OR_MLP) {
        /* Extension: Xavier-normal weights drawn in layout order from the same
         * xorshift/Box-Muller stream, biases zero. */
        long P = oracle_num_params(kind, N, M);
        memset(p, 0, (size_t)P * sizeof(double));
        long o = 0;
        double s1 = sqrt(2.0 / (double)(N + M));
        for (long k = 0; k < (long)M * N; k++) p[o + k] = s1 * xs_gauss(&st);
        o += (long)M * N + M;
        double s2 = sqrt(2.0 / (double)(M + M));
        for (long k = 0; k < (long)M * M; k++) p[o + k] = s2 * xs_gauss(&st);
        o += (long)M * M + M;
        double s3 = sqrt(2.0 / (double)(M + 1));
        for (long k = 0; k < 2L * M; k++) p[o + k] = s3 * xs_gauss(&st);
        return 0;
    }
    return -1;
}

/* ------------------------------------------------------------------ */
/* Base log-amplitudes                                                 */
/* ------------------------------------------------------------------ */

/* Factored-attention ViT, src/nqs/nqs_ansatz.c:357-473 (real) and :571-729 (complex), in
 * upstream's loop order on the complex form (imaginary parts 0 for the real ViT):
 * e_i = w s_i + b, v_i = V e_i, P_ij = softmax_j a[(i-j) mod N], o_i = sum_j P_ij v_j,
 * log psi = sum_i W . o_i + b_out. */
typedef struct {
    int N, d;
    const double *wR, *wI, *bR, *bI, *VR, *VI, *attn, *WR, *WI;
    double boR, boI;
    double *eR, *eI, *vR, *vI, *P, *oR, *oI;   /* scratch */
} vit_t;

static void vit_bind(const or_ansatz_t *a, vit_t *v) {
    int N = a->N, d = a->M;
    const double *p = a->params;
    v->N = N;
    v->d = d;
    if (a->kind == OR_VITC) {
        v->wR = p; v->wI = p + d; v->bR = p + 2 * d; v->bI = p + 3 * d;
        v->VR = p + 4 * d; v->VI = v->VR + (long)d * d; v->attn = v->VI + (long)d * d;
        v->WR = v->attn + N; v->WI = v->WR + d; v->boR = v->WI[d]; v->boI = v->WI[d + 1];
    } else {
        v->wR = p; v->wI = NULL; v->bR = p + d; v->bI = NULL;
        v->VR = p + 2 * d; v->VI = NULL; v->attn = v->VR + (long)d * d;
        v->WR = v->attn + N; v->WI = NULL; v->boR = v->WR[d]; v->boI = 0.0;
    }
    size_t nd = (size_t)N * d;
    v->eR = calloc(nd, sizeof(double)); v->eI = calloc(nd, sizeof(double));
    v->vR = calloc(nd, sizeof(double)); v->vI = calloc(nd, sizeof(double));
    v->P = calloc((size_t)N * N, sizeof(double));
    v->oR = calloc(nd, sizeof(double)); v->oI = calloc(nd, sizeof(double));
}

static void vit_free(vit_t *v) {
    free(v->eR); free(v->eI); free(v->vR); free(v->vI); free(v->P); free(v->oR); free(v->oI);
}

#define VI_(arr, k) ((arr) ? (arr)[k] : 0.0)

static void vit_forward(vit_t *v, const int *s, double *la, double *ar) {
    int N = v->N, d = v->d;
    for (int i = 0; i < N; i++)
        for (int k = 0; k < d; k++) {
            v->eR[i * d + k] = v->wR[k] * (double)s[i] + v->bR[k];
            v->eI[i * d + k] = VI_(v->wI, k) * (double)s[i] + VI_(v->bI, k);
        }
    for (int i = 0; i < N; i++)
        for (int k = 0; k < d; k++) {
            double sr = 0.0, si = 0.0;
            for (int l = 0; l < d; l++) {
                double vrr = v->VR[k * d + l], vii = VI_(v->VI, k * d + l);
                double er = v->eR[i * d + l], ei = v->eI[i * d + l];
                sr += vrr * er - vii * ei;
                si += vrr * ei + vii * er;
            }
            v->vR[i * d + k] = sr;
            v->vI[i * d + k] = si;
        }
    for (int i = 0; i < N; i++) {
        double mx = -1e300;
        for (int j = 0; j < N; j++) {
            double S = v->attn[((i - j) % N + N) % N];
            if (S > mx) mx = S;
        }
        double Z = 0.0;
        for (int j = 0; j < N; j++) {
            double e = exp(v->attn[((i - j) % N + N) % N] - mx);
            v->P[i * N + j] = e;
            Z += e;
        }
        double iz = 1.0 / Z;
        for (int j = 0; j < N; j++) v->P[i * N + j] *= iz;
    }
    for (int i = 0; i < N; i++)
        for (int k = 0; k < d; k++) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < N; j++) {
                sr += v->P[i * N + j] * v->vR[j * d + k];
                si += v->P[i * N + j] * v->vI[j * d + k];
            }
            v->oR[i * d + k] = sr;
            v->oI[i * d + k] = si;
        }
    double l = v->boR, g = v->boI;
    for (int i = 0; i < N; i++)
        for (int k = 0; k < d; k++) {
            double orr = v->oR[i * d + k], oii = v->oI[i * d + k];
            l += v->WR[k] * orr - VI_(v->WI, k) * oii;
            g += v->WR[k] * oii + VI_(v->WI, k) * orr;
        }
    *la = l;
    *ar = g;
}

/* Holomorphic derivatives z_k = d log psi / d(complex weight), src/nqs/nqs_ansatz.c:1104-1256,
 * written into the real-projected row (mode 1: Re z for real parts, -Im z for imaginary
 * parts; the real ViT's gradient, :475-567) or the holomorphic pair (mode 2). */
static void vit_gradient(const or_ansatz_t *a, const int *s, int mode, double *re, double *im) {
    vit_t v;
    vit_bind(a, &v);
    int N = v.N, d = v.d;
    const int cx = a->kind == OR_VITC;
    double la, ar;
    vit_forward(&v, s, &la, &ar);
    long P = oracle_num_params(a->kind, N, d);
    memset(re, 0, sizeof(double) * (size_t)P);
    if (im) memset(im, 0, sizeof(double) * (size_t)P);
    double *sp = calloc((size_t)N, sizeof(double)), *WvR = calloc((size_t)N, sizeof(double));
    double *WvI = calloc((size_t)N, sizeof(double)), *WoR = calloc((size_t)N, sizeof(double));
    double *WoI = calloc((size_t)N, sizeof(double)), *ga_r = calloc((size_t)N, sizeof(double));
    double *ga_i = calloc((size_t)N, sizeof(double));
    double *evR = calloc((size_t)d, sizeof(double)), *evI = calloc((size_t)d, sizeof(double));
    double *alR = calloc((size_t)d, sizeof(double)), *alI = calloc((size_t)d, sizeof(double));
    double *sWR = calloc((size_t)d, sizeof(double)), *sWI = calloc((size_t)d, sizeof(double));
    for (int k = 0; k < d; k++)
        for (int i = 0; i < N; i++) { sWR[k] += v.oR[i * d + k]; sWI[k] += v.oI[i * d + k]; }
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) sp[j] += v.P[i * N + j];
    for (int j = 0; j < N; j++)
        for (int k = 0; k < d; k++) {
            double vr = v.vR[j * d + k], vi = v.vI[j * d + k];
            WvR[j] += v.WR[k] * vr - VI_(v.WI, k) * vi;
            WvI[j] += v.WR[k] * vi + VI_(v.WI, k) * vr;
        }
    for (int i = 0; i < N; i++)
        for (int k = 0; k < d; k++) {
            double orr = v.oR[i * d + k], oii = v.oI[i * d + k];
            WoR[i] += v.WR[k] * orr - VI_(v.WI, k) * oii;
            WoI[i] += v.WR[k] * oii + VI_(v.WI, k) * orr;
        }
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) {
            int rel = ((i - j) % N + N) % N;
            ga_r[rel] += v.P[i * N + j] * (WvR[j] - WoR[i]);
            ga_i[rel] += v.P[i * N + j] * (WvI[j] - WoI[i]);
        }
    for (int j = 0; j < N; j++)
        for (int l = 0; l < d; l++) { evR[l] += sp[j] * v.eR[j * d + l]; evI[l] += sp[j] * v.eI[j * d + l]; }
    for (int l = 0; l < d; l++)
        for (int k = 0; k < d; k++) {
            alR[l] += v.VR[k * d + l] * v.WR[k] - VI_(v.VI, k * d + l) * VI_(v.WI, k);
            alI[l] += v.VR[k * d + l] * VI_(v.WI, k) + VI_(v.VI, k * d + l) * v.WR[k];
        }
    double sps = 0.0, spp = 0.0;
    for (int j = 0; j < N; j++) { sps += sp[j] * (double)s[j]; spp += sp[j]; }
    /* (re, im) of z at the real slot kR and the imaginary slot kI (kI < 0: real parameter) */
    #define PUT(kR, kI, zr, zi) do {                                              \
        if (mode == 2) {                                                           \
            re[kR] = (zr); im[kR] = (zi);                                          \
            if ((kI) >= 0) { re[kI] = -(zi); im[kI] = (zr); }                      \
        } else {                                                                   \
            re[kR] = (zr);                                                         \
            if ((kI) >= 0) re[kI] = -(zi);                                         \
        }                                                                          \
    } while (0)
    long o_w = 0, o_wI = cx ? d : -1, o_b = cx ? 2L * d : d, o_bI = cx ? 3L * d : -1;
    long o_V = cx ? 4L * d : 2L * d, o_VI = cx ? o_V + (long)d * d : -1;
    long o_a = cx ? 4L * d + 2L * d * d : 2L * d + (long)d * d;
    long o_W = o_a + N, o_WI = cx ? o_W + d : -1, o_bo = cx ? o_W + 2L * d : o_W + d;
    for (int l = 0; l < d; l++) {
        PUT(o_w + l, o_wI < 0 ? -1 : o_wI + l, sps * alR[l], sps * alI[l]);
        PUT(o_b + l, o_bI < 0 ? -1 : o_bI + l, spp * alR[l], spp * alI[l]);
    }
    for (int k = 0; k < d; k++)
        for (int l = 0; l < d; l++) {
            double zr = v.WR[k] * evR[l] - VI_(v.WI, k) * evI[l];
            double zi = v.WR[k] * evI[l] + VI_(v.WI, k) * evR[l];
            long q = (long)k * d + l;
            PUT(o_V + q, o_VI < 0 ? -1 : o_VI + q, zr, zi);
        }
    for (int r = 0; r < N; r++) PUT(o_a + r, -1, ga_r[r], ga_i[r]);
    for (int k = 0; k < d; k++) PUT(o_W + k, o_WI < 0 ? -1 : o_WI + k, sWR[k], sWI[k]);
    PUT(o_bo, cx ? o_bo + 1 : -1, 1.0, 0.0);
    #undef PUT
    free(sp); free(WvR); free(WvI); free(WoR); free(WoI); free(ga_r); free(ga_i);
    free(evR); free(evI); free(alR); free(alI); free(sWR); free(sWI);
    vit_free(&v);
}

/* complex log(2 cosh z), the stable form of src/nqs/nqs_ansatz.c:309-318 */
static void clogcosh(double x, double y, double *la, double *ar) {
    double ax = fabs(x);
    double e = exp(-2.0 * ax);
    double re = (1.0 + e) * cos(y);
    double im = (x >= 0.0 ? 1.0 : -1.0) * (1.0 - e) * sin(y);
    double mag = hypot(re, im);
    *la = ax + (mag > 0 ? log(mag) : -1e300);
    *ar = atan2(im, re);
}

static void mlp_forward(const or_ansatz_t *a, const int *s, double *h1, double *h2,
                        double *la, double *ar) {
    int N = a->N, M = a->M;
    const double *W1 = a->params, *b1 = W1 + (long)M * N;
    const double *W2 = b1 + M, *b2 = W2 + (long)M * M;
    const double *wr = b2 + M, *wi = wr + M;
    double cr = wi[M], ci = wi[M + 1];
    for (int k = 0; k < M; k++) {
        double x = b1[k];
        for (int i = 0; i < N; i++) x += W1[(long)k * N + i] * (double)s[i];
        h1[k] = tanh(x);
    }
    for (int j = 0; j < M; j++) {
        double x = b2[j];
        for (int k = 0; k < M; k++) x += W2[(long)j * M + k] * h1[k];
        h2[j] = tanh(x);
    }
    double r = cr, im = ci;
    for (int j = 0; j < M; j++) { r += wr[j] * h2[j]; im += wi[j] * h2[j]; }
    *la = r; *ar = im;
}

static void base_log_amp(const or_ansatz_t *a, const int *s, double *la, double *ar) {
    int N = a->N, M = a->M;
    const double *p = a->params;
    if (a->kind == OR_RBM) {                                       /* :277-294 */
        double acc = 0.0;
        for (int i = 0; i < N; i++) acc += p[i] * (double)s[i];
        for (int h = 0; h < M; h++) {
            double x = p[N + h];
            const double *W = p + N + M + (long)h * N;
            for (int i = 0; i < N; i++) x += W[i] * (double)s[i];
            double ax = fabs(x);
            acc += ax + log1p(exp(-2.0 * ax));
        }
        *la = acc; *ar = 0.0;
    } else if (a->kind == OR_CRBM) {                               /* :320-355 */
        long Pr = (long)N + M + (long)M * N;
        double l = 0.0, g = 0.0;
        for (int i = 0; i < N; i++) {
            l += p[i] * (double)s[i];
            g += p[Pr + i] * (double)s[i];
        }
        for (int h = 0; h < M; h++) {
            double xr = p[N + h], xi = p[Pr + N + h];
            const double *WR = p + N + M + (long)h * N;
            const double *WI = p + Pr + N + M + (long)h * N;
            for (int i = 0; i < N; i++) {
                xr += WR[i] * (double)s[i];
                xi += WI[i] * (double)s[i];
            }
            double t1, t2;
            clogcosh(xr, xi, &t1, &t2);
            l += t1; g += t2;
        }
        *la = l; *ar = g;
    } else if (a->kind == OR_MLP) {
        double *h1 = malloc(sizeof(double) * 2 * (size_t)M);
        mlp_forward(a, s, h1, h1 + M, la, ar);
        free(h1);
    } else if (a->kind == OR_VIT || a->kind == OR_VITC) {
        vit_t v;
        vit_bind(a, &v);
        vit_forward(&v, s, la, ar);
        vit_free(&v);
    } else {                                                       /* :265-270 */
        double acc = 0.0;
        for (int i = 0; i < N; i++) acc += p[i] * (double)s[i];
        *la = acc; *ar = 0.0;
    }
}

int oracle_marshall_parity(const int *spins, int size_x, int size_y) {
    int n = 0;                                                     /* src/nqs/nqs_marshall.c:16-27 */
    for (int x = 0; x < size_x; x++)
        for (int y = 0; y < size_y; y++)
            if (((x + y) & 1) == 0 && spins[x * size_y + y] < 0) n++;
    return n & 1;
}

/* Evaluate the program from layer k inward. */
static void amp_eval(const or_amp_t *amp, int k, const int *s, double *la, double *ar) {
    if (k >= amp->n_layers) { base_log_amp(&amp->base, s, la, ar); return; }
    const or_layer_t *L = &amp->layers[k];
    int N = amp->base.N;
    if (L->type == OR_LAYER_MARSHALL) {                            /* src/nqs/nqs_marshall.c:29-40 */
        double a0, g0;
        amp_eval(amp, k + 1, s, &a0, &g0);
        int par = oracle_marshall_parity(s, L->size_x, L->size_y);
        *la = a0;
        *ar = g0 + (par ? M_PI : 0.0);
        return;
    }
    /* symproj, src/nqs/nqs_symproj.c:31-80 */
    int G = L->G;
    int *sh = malloc(sizeof(int) * (size_t)N);
    double *lp = malloc(sizeof(double) * (size_t)G);
    double *cs = malloc(sizeof(double) * (size_t)G);
    double mx = -1e300;
    for (int g = 0; g < G; g++) {
        for (int i = 0; i < N; i++) sh[i] = s[L->perm[(size_t)g * N + i]];
        double l, a;
        amp_eval(amp, k + 1, sh, &l, &a);
        lp[g] = l;
        cs[g] = L->chars[g] * cos(a);
        if (l > mx) mx = l;
    }
    double sum = 0.0;
    for (int g = 0; g < G; g++) sum += cs[g] * exp(lp[g] - mx);
    double as = fabs(sum);
    if (as > 0.0) {
        *la = log(as) + mx - 0.5 * log((double)G);
        *ar = (sum < 0.0) ? M_PI : 0.0;
    } else {
        *la = -1e300;
        *ar = 0.0;
    }
    free(sh); free(lp); free(cs);
}

void oracle_log_amp_batch(const or_amp_t *amp, const int *spins, int B,
                          double *out_la, double *out_arg) {
    int N = amp->base.N;
    for (int b = 0; b < B; b++) {
        double l, a;
        amp_eval(amp, 0, spins + (size_t)b * N, &l, &a);
        if (out_la) out_la[b] = l;
        if (out_arg) out_arg[b] = a;
    }
}

/* ------------------------------------------------------------------ */
/* Gradients                                                           */
/* ------------------------------------------------------------------ */

/* tanh(xr + i xi) through sinh/cosh, src/nqs/nqs_ansatz.c:961-972 */
static void or_ctanh(double xr, double xi, double *tr, double *ti) {
    double cxr = cosh(xr), sxr = sinh(xr);
    double cy = cos(xi), sy = sin(xi);
    double nr = sxr * cy, ni = cxr * sy;
    double dr = cxr * cy, di = sxr * sy;
    double den = dr * dr + di * di;
    if (den < 1e-300) den = 1e-300;
    *tr = (nr * dr + ni * di) / den;
    *ti = (ni * dr - nr * di) / den;
}

static void crbm_theta(const or_ansatz_t *a, const int *s, int h, double *xr, double *xi) {
    int N = a->N, M = a->M;
    long Pr = (long)N + M + (long)M * N;
    const double *p = a->params;
    double r = p[N + h], im = p[Pr + N + h];
    const double *WR = p + N + M + (long)h * N, *WI = p + Pr + N + M + (long)h * N;
    for (int i = 0; i < N; i++) { r += WR[i] * (double)s[i]; im += WI[i] * (double)s[i]; }
    *xr = r; *xi = im;
}

static void mlp_backprop(const or_ansatz_t *a, const int *s, const double *head,
                         double *out) {
    /* d(head . h2)/d(theta) for the layers below the head; `out` is the full
     * parameter vector (head slots are filled by the caller). */
    int N = a->N, M = a->M;
    const double *W2 = a->params + (long)M * N + M;
    double *h1 = malloc(sizeof(double) * 4 * (size_t)M);
    double *h2 = h1 + M, *d2 = h2 + M, *d1 = d2 + M;
    double la, ar;
    mlp_forward(a, s, h1, h2, &la, &ar);
    long o_b1 = (long)M * N, o_W2 = o_b1 + M, o_b2 = o_W2 + (long)M * M;
    for (int j = 0; j < M; j++) d2[j] = head[j] * (1.0 - h2[j] * h2[j]);
    for (int k = 0; k < M; k++) {
        double t = 0.0;
        for (int j = 0; j < M; j++) t += W2[(long)j * M + k] * d2[j];
        d1[k] = t * (1.0 - h1[k] * h1[k]);
    }
    for (int j = 0; j < M; j++) {
        out[o_b2 + j] = d2[j];
        for (int k = 0; k < M; k++) out[o_W2 + (long)j * M + k] = d2[j] * h1[k];
    }
    for (int k = 0; k < M; k++) {
        out[o_b1 + k] = d1[k];
        for (int i = 0; i < N; i++) out[(long)k * N + i] = d1[k] * (double)s[i];
    }
    free(h1);
}

static void mlp_h2(const or_ansatz_t *a, const int *s, double *h2) {
    double *h1 = malloc(sizeof(double) * (size_t)a->M);
    double la, ar;
    mlp_forward(a, s, h1, h2, &la, &ar);
    free(h1);
}

static int grad_one(const or_ansatz_t *a, const int *s, double *out) {
    int N = a->N, M = a->M;
    if (a->kind == OR_RBM) {                                       /* :885-911 */
        const double *p = a->params;
        for (int i = 0; i < N; i++) out[i] = (double)s[i];
        for (int h = 0; h < M; h++) {
            double x = p[N + h];
            const double *W = p + N + M + (long)h * N;
            for (int i = 0; i < N; i++) x += W[i] * (double)s[i];
            out[N + h] = tanh(x);
        }
        for (int h = 0; h < M; h++)
            for (int i = 0; i < N; i++)
                out[N + M + (long)h * N + i] = out[N + h] * (double)s[i];
        return 0;
    }
    if (a->kind == OR_CRBM) {                                      /* :933-995 */
        long Pr = (long)N + M + (long)M * N;
        for (int i = 0; i < N; i++) { out[i] = (double)s[i]; out[Pr + i] = 0.0; }
        for (int h = 0; h < M; h++) {
            double xr, xi, tr, ti;
            crbm_theta(a, s, h, &xr, &xi);
            or_ctanh(xr, xi, &tr, &ti);
            out[N + h] = tr;
            out[Pr + N + h] = -ti;
            for (int i = 0; i < N; i++) {
                out[N + M + (long)h * N + i] = tr * (double)s[i];
                out[Pr + N + M + (long)h * N + i] = -ti * (double)s[i];
            }
        }
        return 0;
    }
    if (a->kind == OR_MLP) {
        long P = oracle_num_params(OR_MLP, N, M);
        const double *wr = a->params + (long)M * N + M + (long)M * M + M;
        mlp_backprop(a, s, wr, out);
        double *h2 = out + (long)M * N + M + (long)M * M + M;     /* w_re slots */
        mlp_h2(a, s, h2);
        for (int j = 0; j < M; j++) out[P - 2 - M + j] = 0.0;     /* w_im: no effect on log|psi| */
        out[P - 2] = 1.0;
        out[P - 1] = 0.0;
        return 0;
    }
    if (a->kind == OR_VIT || a->kind == OR_VITC) {                /* :475-567, :732-843 */
        vit_gradient(a, s, 1, out, NULL);
        return 0;
    }
    for (int i = 0; i < N; i++) out[i] = (double)s[i];            /* :875-879 */
    return 0;
}

int oracle_gradient_batch(const or_ansatz_t *a, const int *spins, int B, double *out) {
    long P = oracle_num_params(a->kind, a->N, a->M);
    for (int b = 0; b < B; b++)
        if (grad_one(a, spins + (size_t)b * a->N, out + (size_t)b * P)) return -1;
    return 0;
}

static int grad_complex_one(const or_ansatz_t *a, const int *s, double *re, double *im) {
    int N = a->N, M = a->M;
    long P = oracle_num_params(a->kind, N, M);
    if (a->kind == OR_CRBM) {                                      /* :1025-1091 */
        long Pr = (long)N + M + (long)M * N;
        for (int i = 0; i < N; i++) {
            re[i] = (double)s[i]; im[i] = 0.0;
            re[Pr + i] = 0.0;     im[Pr + i] = (double)s[i];
        }
        for (int h = 0; h < M; h++) {
            double xr, xi, tr, ti;
            crbm_theta(a, s, h, &xr, &xi);
            or_ctanh(xr, xi, &tr, &ti);
            re[N + h] = tr;       im[N + h] = ti;
            re[Pr + N + h] = -ti; im[Pr + N + h] = tr;
            for (int i = 0; i < N; i++) {
                double si = (double)s[i];
                re[N + M + (long)h * N + i] = tr * si;
                im[N + M + (long)h * N + i] = ti * si;
                re[Pr + N + M + (long)h * N + i] = -ti * si;
                im[Pr + N + M + (long)h * N + i] = tr * si;
            }
        }
        return 0;
    }
    if (a->kind == OR_MLP) {
        const double *wr = a->params + (long)M * N + M + (long)M * M + M;
        const double *wi = wr + M;
        mlp_backprop(a, s, wr, re);
        mlp_backprop(a, s, wi, im);
        double *h2 = malloc(sizeof(double) * (size_t)M);
        mlp_h2(a, s, h2);
        long o_wr = (long)M * N + M + (long)M * M + M, o_wi = o_wr + M;
        for (int j = 0; j < M; j++) {
            re[o_wr + j] = h2[j]; im[o_wr + j] = 0.0;
            re[o_wi + j] = 0.0;   im[o_wi + j] = h2[j];
        }
        re[P - 2] = 1.0; im[P - 2] = 0.0;
        re[P - 1] = 0.0; im[P - 1] = 1.0;
        free(h2);
        return 0;
    }
    if (a->kind == OR_VITC) {                                      /* :1104-1256 */
        vit_gradient(a, s, 2, re, im);
        return 0;
    }
    int rc = grad_one(a, s, re);                                   /* :1268-1272 */
    for (long k = 0; k < P; k++) im[k] = 0.0;
    return rc;
}

int oracle_gradient_complex_batch(const or_ansatz_t *a, const int *spins, int B,
                                  double *out_re, double *out_im) {
    long P = oracle_num_params(a->kind, a->N, a->M);
    for (int b = 0; b < B; b++)
        if (grad_complex_one(a, spins + (size_t)b * a->N, out_re + (size_t)b * P,
                             out_im + (size_t)b * P)) return -1;
    return 0;
}

/* Symmetry-projected gradient, src/nqs/nqs_symproj.c:82-155. */
int oracle_symproj_gradient_batch(const or_amp_t *amp, const int *spins, int B,
                                  double *out) {
    int k = -1;
    for (int l = 0; l < amp->n_layers; l++)
        if (amp->layers[l].type == OR_LAYER_SYMPROJ) { k = l; break; }
    if (k < 0) return -1;
    const or_layer_t *L = &amp->layers[k];
    int N = amp->base.N, G = L->G;
    long P = oracle_num_params(amp->base.kind, N, amp->base.M);
    int *sh = malloc(sizeof(int) * (size_t)G * N);
    double *lp = malloc(sizeof(double) * (size_t)G);
    double *cs = malloc(sizeof(double) * (size_t)G);
    double *ct = malloc(sizeof(double) * (size_t)G);
    double *tmp = malloc(sizeof(double) * (size_t)P);
    for (int b = 0; b < B; b++) {
        const int *s = spins + (size_t)b * N;
        double *o = out + (size_t)b * P;
        double mx = -1e300;
        for (int g = 0; g < G; g++) {
            for (int i = 0; i < N; i++) sh[(size_t)g * N + i] = s[L->perm[(size_t)g * N + i]];
            double l, a;
            amp_eval(amp, k + 1, sh + (size_t)g * N, &l, &a);
            lp[g] = l;
            cs[g] = L->chars[g] * cos(a);
            if (l > mx) mx = l;
        }
        double den = 0.0;
        for (int g = 0; g < G; g++) { ct[g] = cs[g] * exp(lp[g] - mx); den += ct[g]; }
        memset(o, 0, (size_t)P * sizeof(double));
        if (den == 0.0) continue;
        for (int g = 0; g < G; g++) {
            double w = ct[g] / den;
            if (w == 0.0) continue;
            grad_one(&amp->base, sh + (size_t)g * N, tmp);
            for (long q = 0; q < P; q++) o[q] += w * tmp[q];
        }
    }
    free(sh); free(lp); free(cs); free(ct); free(tmp);
    return 0;
}

/* Complex symmetry-projected gradient, src/nqs/nqs_symproj.c:157-261: complex weights
 * w_g = c_g / sum c, c_g = chi_g e^{lp_g - max} (cos arg_g + i sin arg_g), times the
 * holomorphic gradient of the base ansatz at g s. */
int oracle_symproj_gradient_complex_batch(const or_amp_t *amp, const int *spins, int B,
                                          double *out_re, double *out_im) {
    int k = -1;
    for (int l = 0; l < amp->n_layers; l++)
        if (amp->layers[l].type == OR_LAYER_SYMPROJ) { k = l; break; }
    if (k < 0) return -1;
    const or_layer_t *L = &amp->layers[k];
    int N = amp->base.N, G = L->G;
    long P = oracle_num_params(amp->base.kind, N, amp->base.M);
    int *sh = malloc(sizeof(int) * (size_t)G * N);
    double *lp = malloc(sizeof(double) * (size_t)G), *ag = malloc(sizeof(double) * (size_t)G);
    double *cr = malloc(sizeof(double) * (size_t)G), *ci = malloc(sizeof(double) * (size_t)G);
    double *tr = malloc(sizeof(double) * (size_t)P), *ti = malloc(sizeof(double) * (size_t)P);
    for (int b = 0; b < B; b++) {
        const int *s = spins + (size_t)b * N;
        double *ore = out_re + (size_t)b * P, *oim = out_im + (size_t)b * P;
        double mx = -1e300;
        for (int g = 0; g < G; g++) {
            for (int i = 0; i < N; i++) sh[(size_t)g * N + i] = s[L->perm[(size_t)g * N + i]];
            amp_eval(amp, k + 1, sh + (size_t)g * N, &lp[g], &ag[g]);
            if (lp[g] > mx) mx = lp[g];
        }
        double dr = 0.0, di = 0.0;
        for (int g = 0; g < G; g++) {
            double m = L->chars[g] * exp(lp[g] - mx);
            cr[g] = m * cos(ag[g]);
            ci[g] = m * sin(ag[g]);
            dr += cr[g];
            di += ci[g];
        }
        memset(ore, 0, (size_t)P * sizeof(double));
        memset(oim, 0, (size_t)P * sizeof(double));
        double d2 = dr * dr + di * di;
        if (d2 == 0.0) continue;
        for (int g = 0; g < G; g++) {
            double wr = (cr[g] * dr + ci[g] * di) / d2, wi = (ci[g] * dr - cr[g] * di) / d2;
            if (wr == 0.0 && wi == 0.0) continue;
            if (oracle_gradient_complex_batch(&amp->base, sh + (size_t)g * N, 1, tr, ti)) return -1;
            for (long q = 0; q < P; q++) {
                ore[q] += wr * tr[q] - wi * ti[q];
                oim[q] += wr * ti[q] + wi * tr[q];
            }
        }
    }
    free(sh); free(lp); free(ag); free(cr); free(ci); free(tr); free(ti);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Local energies                                                      */
/* ------------------------------------------------------------------ */

int oracle_num_sites(const or_ham_t *h) {
    return h->ham == OR_KAGOME ? 3 * h->size_x * h->size_y : h->size_x * h->size_y;
}

/* Nearest-neighbour bonds of a square / chain lattice in the upstream
 * enumeration order (src/nqs/nqs_gradient.c:98-107): for x, for y, the +x
 * bond then the +y bond.  With pbc (extension) the +x / +y neighbours wrap
 * whenever the extent exceeds 1. */
static int square_bonds(int Lx, int Ly, int pbc, int *bd) {
    int n = 0;
    for (int x = 0; x < Lx; x++)
        for (int y = 0; y < Ly; y++) {
            int a = x * Ly + y;
            if (x + 1 < Lx) { bd[2 * n] = a; bd[2 * n + 1] = (x + 1) * Ly + y; n++; }
            else if (pbc && Lx > 1) { bd[2 * n] = a; bd[2 * n + 1] = y; n++; }
            if (y + 1 < Ly) { bd[2 * n] = a; bd[2 * n + 1] = x * Ly + y + 1; n++; }
            else if (pbc && Ly > 1) { bd[2 * n] = a; bd[2 * n + 1] = x * Ly; n++; }
        }
    return n;
}

/* J1-J2 diagonal bonds, src/nqs/nqs_gradient.c:146-159 (+ periodic wrap). */
static int diag_bonds(int Lx, int Ly, int pbc, int *bd) {
    int n = 0;
    int xe = pbc && Lx > 1 ? Lx : Lx - 1, ye = pbc && Ly > 1 ? Ly : Ly - 1;
    for (int x = 0; x < xe; x++)
        for (int y = 0; y < ye; y++) {
            int x1 = (x + 1) % Lx, y1 = (y + 1) % Ly;
            bd[2 * n] = x * Ly + y;   bd[2 * n + 1] = x1 * Ly + y1; n++;
            bd[2 * n] = x * Ly + y1;  bd[2 * n + 1] = x1 * Ly + y;  n++;
        }
    return n;
}

/* Kagome bonds, src/nqs/nqs_gradient.c:374-445: per cell the up-triangle
 * (A-B, A-C, B-C) then the down-triangle anchored at A. */
static int kagome_bonds(int Lx, int Ly, int pbc, int *bd) {
    int n = 0;
#define KS(cx, cy, sub) (3 * ((cx) * Ly + (cy)) + (sub))
    for (int cx = 0; cx < Lx; cx++)
        for (int cy = 0; cy < Ly; cy++) {
            int A = KS(cx, cy, 0), B = KS(cx, cy, 1), C = KS(cx, cy, 2);
            int up[3][2] = {{A, B}, {A, C}, {B, C}};
            for (int b = 0; b < 3; b++) { bd[2 * n] = up[b][0]; bd[2 * n + 1] = up[b][1]; n++; }
            int cxm, cym;
            if (pbc) { cxm = (cx - 1 + Lx) % Lx; cym = (cy - 1 + Ly) % Ly; }
            else { if (cx == 0 || cy == 0) continue; cxm = cx - 1; cym = cy - 1; }
            int Bm = KS(cxm, cy, 1), Cm = KS(cx, cym, 2);
            int dn[3][2] = {{A, Bm}, {A, Cm}, {Bm, Cm}};
            for (int b = 0; b < 3; b++) { bd[2 * n] = dn[b][0]; bd[2 * n + 1] = dn[b][1]; n++; }
        }
#undef KS
    return n;
}

int square_bonds_public(int Lx, int Ly, int pbc, int *bd) { return square_bonds(Lx, Ly, pbc, bd); }
int diag_bonds_public(int Lx, int Ly, int pbc, int *bd) { return diag_bonds(Lx, Ly, pbc, bd); }

int oracle_bonds(const or_ham_t *h, int *bonds, int cap) {
    int tmp[4096];
    int n;
    if (h->ham == OR_KAGOME) n = kagome_bonds(h->size_x, h->size_y, h->kagome_pbc, tmp);
    else n = square_bonds(h->size_x, h->size_y, h->pbc, tmp);
    if (n > cap) return -1;
    memcpy(bonds, tmp, sizeof(int) * 2 * (size_t)n);
    return n;
}

/* psi(s')/psi(s), src/nqs/nqs_gradient.c:24-45 */
static void ratio(const or_amp_t *amp, const int *sn, double la0, double ar0,
                  double *re, double *im) {
    double l, a;
    amp_eval(amp, 0, sn, &l, &a);
    double mag = exp(l - la0), d = a - ar0;
    *re = mag * cos(d);
    *im = mag * sin(d);
}

/* Heisenberg-type bond sum: diag += 0.25 Jz s_u s_v; off += 0.5 Jxy ratio on
 * antiparallel bonds (src/nqs/nqs_gradient.c:87-139, :374-445). */
static void bond_sum(const or_amp_t *amp, const int *s, int *scr, int N,
                     const int *bd, int nb, double Jxy, double Jz,
                     double la0, double ar0,
                     double *diag, double *ore, double *oim) {
    (void)N;
    for (int b = 0; b < nb; b++) {
        int u = bd[2 * b], v = bd[2 * b + 1];
        int su = s[u], sv = s[v];
        *diag += 0.25 * Jz * (double)(su * sv);
        if (su != sv) {
            scr[u] = -su; scr[v] = -sv;
            double r, i;
            ratio(amp, scr, la0, ar0, &r, &i);
            scr[u] = su; scr[v] = sv;
            *ore += 0.5 * Jxy * r;
            *oim += 0.5 * Jxy * i;
        }
    }
}

static void eloc_one(const or_ham_t *h, const or_amp_t *amp, const int *s,
                     double *ore_out, double *oim_out) {
    int N = oracle_num_sites(h);
    int *bd = malloc(sizeof(int) * 8192);
    int *scr = malloc(sizeof(int) * (size_t)N);
    memcpy(scr, s, sizeof(int) * (size_t)N);
    double la0, ar0;
    amp_eval(amp, 0, s, &la0, &ar0);                               /* :461 */
    double re = 0.0, im = 0.0;
    if (h->ham == OR_TFIM) {                                       /* :50-82 */
        int nb = square_bonds(h->size_x, h->size_y, h->pbc, bd);
        double diag = 0.0;
        for (int b = 0; b < nb; b++)
            diag += -h->J * (double)(s[bd[2 * b]] * s[bd[2 * b + 1]]);
        double ore = 0.0, oim = 0.0;
        for (int i = 0; i < N; i++) {
            scr[i] = -scr[i];
            double r, q;
            ratio(amp, scr, la0, ar0, &r, &q);
            ore += -h->Gamma * r;
            oim += -h->Gamma * q;
            scr[i] = -scr[i];
        }
        re = diag + ore; im = oim;
    } else if (h->ham == OR_HEIS || h->ham == OR_XXZ || h->ham == OR_J1J2) {
        double Jxy = h->J, Jz = (h->ham == OR_XXZ) ? h->Jz : h->J;
        int nb = square_bonds(h->size_x, h->size_y, h->pbc, bd);
        double diag = 0.0, ore = 0.0, oim = 0.0;
        bond_sum(amp, s, scr, N, bd, nb, Jxy, Jz, la0, ar0, &diag, &ore, &oim);
        re = diag + ore; im = oim;
        if (h->ham == OR_J1J2) {                                   /* :188-205 */
            int nd = diag_bonds(h->size_x, h->size_y, h->pbc, bd);
            double d2 = 0.0, r2 = 0.0, i2 = 0.0;
            bond_sum(amp, s, scr, N, bd, nd, h->J2, h->J2, la0, ar0, &d2, &r2, &i2);
            re = re + d2 + r2;
            im = im + i2;
        }
    } else if (h->ham == OR_KAGOME) {                              /* :374-445 */
        int nb = kagome_bonds(h->size_x, h->size_y, h->kagome_pbc, bd);
        double diag = 0.0, ore = 0.0, oim = 0.0;
        bond_sum(amp, s, scr, N, bd, nb, h->J, h->J, la0, ar0, &diag, &ore, &oim);
        re = diag + ore; im = oim;
    }
    *ore_out = re;
    *oim_out = im;
    free(bd); free(scr);
}

void oracle_local_energy_batch(const or_ham_t *h, const or_amp_t *amp,
                               const int *spins, int B, double *out_re,
                               double *out_im) {
    int N = oracle_num_sites(h);
    for (int b = 0; b < B; b++) {
        double re, im;
        eloc_one(h, amp, spins + (size_t)b * N, &re, &im);
        out_re[b] = re;
        if (out_im) out_im[b] = im;
    }
}
