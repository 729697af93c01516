// Ansatz handle, amplitude-program builder, log-amplitude and Jacobian kernels.
#include <math.h>
#include <stdlib.h>

#include "nqs_amp.cuh"

namespace nqs {

// ---------------------------------------------------------------- parameters

static long num_params_of(int kind, int N, int M) {
    long n = N, m = M;
    switch (kind) {
        case KIND_MF: return n;                                   // src/nqs/nqs_ansatz.c:77-87
        case KIND_RBM: return n + m + m * n;                      // :88
        case KIND_CRBM: return 2 * (n + m + m * n);               // :223
        case KIND_MLP: return m * n + m + m * m + m + 2 * m + 2;  // GPU extension
        case KIND_VIT: return 3 * m + m * m + n + 1;              // :113-130 (m = d)
        case KIND_VITC: return 6 * m + 2 * m * m + n + 2;         // :155-172
        default: return -1;
    }
}

// Initial parameters: the upstream xorshift64 stream and Box-Muller draws
// (src/nqs/nqs_ansatz.c:47-61, :65-252), so a given config yields the same
// starting point as upstream.  Host-side set-up, run once per handle.
static double xs_uniform(uint64_t *s) {
    uint64_t x = *s;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *s = x;
    return (double)(x >> 11) / 9007199254740992.0;
}

static double xs_gauss(uint64_t *s) {
    double u1 = xs_uniform(s), u2 = xs_uniform(s);
    if (u1 < 1e-15) u1 = 1e-15;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
}

static void init_params(const nqs_config_t *cfg, int kind, int N, int M, double *p) {
    uint64_t st = cfg->rng_seed ? (uint64_t)cfg->rng_seed : 0xDEADBEEFCAFEBABEull;
    double scale = cfg->rbm_init_scale > 0.0 ? cfg->rbm_init_scale : 0.01;
    if (kind == KIND_MF) {
        for (int i = 0; i < N; i++) p[i] = 0.01 * (xs_uniform(&st) - 0.5);
        return;
    }
    if (kind == KIND_VIT) {                                // src/nqs/nqs_ansatz.c:131-151 (M = d)
        const int d = M;
        const double vs = scale / sqrt((double)d);
        for (int i = 0; i < d; i++) p[i] = scale * xs_gauss(&st);
        for (int i = 0; i < d; i++) p[d + i] = scale * (xs_uniform(&st) - 0.5);
        for (long k = 0; k < (long)d * d; k++) p[2L * d + k] = vs * xs_gauss(&st);
        const long ao = 2L * d + (long)d * d;
        for (long k = 0; k < N; k++) p[ao + k] = scale * (xs_uniform(&st) - 0.5);
        for (int i = 0; i < d; i++) p[ao + N + i] = scale * (xs_uniform(&st) - 0.5);
        p[ao + N + d] = 0.0;
        return;
    }
    if (kind == KIND_VITC) {                               // :173-214
        const int d = M;
        const double vs = scale / sqrt((double)d), is = 0.1 * scale;
        for (int i = 0; i < d; i++) p[i] = scale * xs_gauss(&st);
        for (int i = 0; i < d; i++) p[d + i] = is * xs_gauss(&st);
        for (int i = 0; i < d; i++) p[2 * d + i] = scale * (xs_uniform(&st) - 0.5);
        for (int i = 0; i < d; i++) p[3 * d + i] = is * (xs_uniform(&st) - 0.5);
        const long vr = 4L * d, vi = vr + (long)d * d, ao = vi + (long)d * d;
        for (long k = 0; k < (long)d * d; k++) p[vr + k] = vs * xs_gauss(&st);
        for (long k = 0; k < (long)d * d; k++) p[vi + k] = 0.1 * vs * xs_gauss(&st);
        for (long k = 0; k < N; k++) p[ao + k] = scale * (xs_uniform(&st) - 0.5);
        for (int i = 0; i < d; i++) p[ao + N + i] = scale * (xs_uniform(&st) - 0.5);
        for (int i = 0; i < d; i++) p[ao + N + d + i] = is * (xs_uniform(&st) - 0.5);
        p[ao + N + 2 * d] = 0.0;
        p[ao + N + 2 * d + 1] = 0.0;
        return;
    }
    if (kind == KIND_RBM || kind == KIND_CRBM) {
        long Pr = (long)N + M + (long)M * N;
        double wstd = scale / sqrt((double)N);
        for (int i = 0; i < N; i++) p[i] = scale * (xs_uniform(&st) - 0.5);
        for (int h = 0; h < M; h++) p[N + h] = scale * (xs_uniform(&st) - 0.5);
        for (long k = 0; k < (long)M * N; k++) p[N + M + k] = wstd * xs_gauss(&st);
        if (kind == KIND_CRBM) {
            double is = 0.1 * scale, iw = is / sqrt((double)N);
            for (int i = 0; i < N; i++) p[Pr + i] = is * (xs_uniform(&st) - 0.5);
            for (int h = 0; h < M; h++) p[Pr + N + h] = is * (xs_uniform(&st) - 0.5);
            for (long k = 0; k < (long)M * N; k++) p[Pr + N + M + k] = iw * xs_gauss(&st);
        }
        return;
    }
    // deep MLP: Xavier-normal weights in layout order, zero biases
    long P = num_params_of(kind, N, M);
    memset(p, 0, sizeof(double) * (size_t)P);
    long o = 0;
    double s1 = sqrt(2.0 / (double)(N + M));
    for (long k = 0; k < (long)M * N; k++) p[o + k] = s1 * xs_gauss(&st);
    o += (long)M * N + M;
    double s2 = sqrt(2.0 / (double)(M + M));
    for (long k = 0; k < (long)M * M; k++) p[o + k] = s2 * xs_gauss(&st);
    o += (long)M * M + M;
    double s3 = sqrt(2.0 / (double)(M + 1));
    for (long k = 0; k < 2L * M; k++) p[o + k] = s3 * xs_gauss(&st);
}

// Transposed weight copies: RBM/cRBM W[h][i] -> wt[i][h]; MLP W1 -> W1^T, W2 -> W2^T.
// RBM / cRBM also get the FP32 tables of the mixed-precision estimator:
// f32 = [W^T | cosh(2 W^T) | sinh(2 W^T)] ([N][M] each), a [N], b [M], complex.
__global__ void k_derive(DevAnsatz a, double *wtr, double *wti, float2 *f32, double *cs64) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int N = a.N, M = a.M;
    if (a.kind == KIND_RBM || a.kind == KIND_CRBM) {
        if (t >= (long)M * N) return;
        const bool cx = a.kind == KIND_CRBM;
        const long Pr = crbm_pr(a), NM = (long)N * M;
        int h = (int)(t / N), i = (int)(t % N);
        const double x = a.p[N + M + t], y = cx ? a.p[Pr + N + M + t] : 0.0;
        wtr[(long)i * M + h] = x;
        if (cx) wti[(long)i * M + h] = y;
        double s2y, c2y;
        sincos(2.0 * y, &s2y, &c2y);
        const double c2x = cosh(2.0 * x), s2x = sinh(2.0 * x);
        f32[(long)i * M + h] = make_float2((float)x, (float)y);
        f32[NM + (long)i * M + h] = make_float2((float)(c2x * c2y), (float)(s2x * s2y));
        f32[2 * NM + (long)i * M + h] = make_float2((float)(s2x * c2y), (float)(c2x * s2y));
        if (cs64) {
            const long q = (long)i * M + h;
            cs64[q] = c2x * c2y;                 // cosh(2 W) = cosh 2x cos 2y + i sinh 2x sin 2y
            cs64[NM + q] = s2x * s2y;
            cs64[2 * NM + q] = s2x * c2y;        // sinh(2 W) = sinh 2x cos 2y + i cosh 2x sin 2y
            cs64[3 * NM + q] = c2x * s2y;
        }
        if (t < N) f32[3 * NM + t] = make_float2((float)a.p[t], cx ? (float)a.p[Pr + t] : 0.f);
        if (t < M) f32[3 * NM + N + t] = make_float2((float)a.p[N + t], cx ? (float)a.p[Pr + N + t] : 0.f);
    } else if (a.kind == KIND_MLP) {
        long nW1 = (long)M * N;
        float *m = (float *)f32;
        const int MP = mlp32_pitch(M);
        float *w2t = m + nW1, *w2 = w2t + (long)M * MP, *vec = w2 + (long)M * MP;
        if (t < nW1) {
            int k = (int)(t / N), i = (int)(t % N);
            wtr[(long)i * M + k] = a.p[t];
            m[(long)i * M + k] = (float)a.p[t];
        } else if (t < nW1 + (long)M * MP) {
            long u = t - nW1;
            int r = (int)(u / MP), c = (int)(u % MP);           // row r, padded column c
            if (c < M) {
                const double w_rc = a.p[nW1 + M + (long)r * M + c];   // W2[r][c]
                wti[(long)c * M + r] = w_rc;
                w2[(long)r * MP + c] = (float)w_rc;
                w2t[(long)c * MP + r] = (float)w_rc;
            } else {
                w2[(long)r * MP + c] = 0.f;
                w2t[(long)r * MP + c] = 0.f;
            }
        }
        if (t < M) {
            const double *b1 = a.p + nW1, *b2 = b1 + M + (long)M * M, *wr = b2 + M, *wi = wr + M;
            vec[t] = (float)b1[t];
            vec[M + t] = (float)b2[t];
            vec[2 * M + t] = (float)wr[t];
            vec[3 * M + t] = (float)wi[t];
            if (t < 2) vec[4 * M + t] = (float)wi[M + t];
        }
    }
}

// ViT tables (one block): softmax weights, attention column sums, u = V^T W_out and the
// products the configuration-dependent terms need (layout VitTab).  Complex parameters
// are read from the complex ViT's layout; the real ViT has zero imaginary parts.
__global__ void k_vit_tables(DevAnsatz a, double *t) {
    const int N = a.N, d = a.M, tid = threadIdx.x;
    const VitTab T = vit_tab(N, d);
    const bool cx = a.kind == KIND_VITC;
    // offsets of the (re, im) blocks
    const long wR = 0, wI = cx ? d : -1, bR = cx ? 2L * d : d, bI = cx ? 3L * d : -1;
    const long VR = cx ? 4L * d : 2L * d, VI = cx ? VR + (long)d * d : -1;
    const long at = cx ? 4L * d + 2L * d * d : 2L * d + (long)d * d;
    const long WR = at + N, WI = cx ? WR + d : -1, boR = cx ? WR + 2L * d : WR + d, boI = cx ? boR + 1 : -1;
    const double *p = a.p;
    auto im = [&](long off, long k) { return off < 0 ? 0.0 : p[off + k]; };
    __shared__ double s_max, s_invz;
    if (tid == 0) {                                        // src/nqs/nqs_ansatz.c:431-447
        double mx = -1e300;
        for (int r = 0; r < N; r++) mx = fmax(mx, p[at + r]);
        double z = 0.0;
        for (int r = 0; r < N; r++) z += exp(p[at + r] - mx);
        s_max = mx;
        s_invz = 1.0 / z;
    }
    __syncthreads();
    for (int r = tid; r < N; r += blockDim.x) t[T.f + r] = exp(p[at + r] - s_max) * s_invz;
    for (int l = tid; l < d; l += blockDim.x) {
        t[T.w + 2 * l] = p[wR + l];
        t[T.w + 2 * l + 1] = im(wI, l);
        t[T.b + 2 * l] = p[bR + l];
        t[T.b + 2 * l + 1] = im(bI, l);
        t[T.W + 2 * l] = p[WR + l];
        t[T.W + 2 * l + 1] = im(WI, l);
    }
    __syncthreads();
    for (int j = tid; j < N; j += blockDim.x) {            // s_pred[j] = sum_i P_ij
        double sp = 0.0;
        for (int i = 0; i < N; i++) sp += t[T.f + ((i - j) % N + N) % N];
        t[T.sp + j] = sp;
    }
    for (int l = tid; l < d; l += blockDim.x) {            // u_l = sum_k W_k V_kl
        double ur = 0.0, ui = 0.0;
        for (int k = 0; k < d; k++) {
            const double vr = p[VR + (long)k * d + l], vi = im(VI, (long)k * d + l);
            const double Wr = p[WR + k], Wi = im(WI, k);
            ur += vr * Wr - vi * Wi;
            ui += vr * Wi + vi * Wr;
        }
        t[T.u + 2 * l] = ur;
        t[T.u + 2 * l + 1] = ui;
    }
    for (int k = tid; k < d; k += blockDim.x) {            // (V w)_k, (V b)_k
        double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
        for (int l = 0; l < d; l++) {
            const double vr = p[VR + (long)k * d + l], vi = im(VI, (long)k * d + l);
            const double xr = p[wR + l], xi = im(wI, l), yr = p[bR + l], yi = im(bI, l);
            ar += vr * xr - vi * xi;
            ai += vr * xi + vi * xr;
            br += vr * yr - vi * yi;
            bi += vr * yi + vi * yr;
        }
        t[T.vw + 2 * k] = ar;
        t[T.vw + 2 * k + 1] = ai;
        t[T.vb + 2 * k] = br;
        t[T.vb + 2 * k + 1] = bi;
    }
    __syncthreads();
    if (tid == 0) {
        double bs = 0.0, c1r = 0.0, c1i = 0.0, c0r = 0.0, c0i = 0.0;
        for (int j = 0; j < N; j++) bs += t[T.sp + j];
        for (int l = 0; l < d; l++) {
            const double ur = t[T.u + 2 * l], ui = t[T.u + 2 * l + 1];
            const double xr = t[T.w + 2 * l], xi = t[T.w + 2 * l + 1], yr = t[T.b + 2 * l], yi = t[T.b + 2 * l + 1];
            c1r += ur * xr - ui * xi;
            c1i += ur * xi + ui * xr;
            c0r += ur * yr - ui * yi;
            c0i += ur * yi + ui * yr;
        }
        t[T.bsum] = bs;
        t[T.bout] = p[boR];
        t[T.bout + 1] = im(boI, 0);
        t[T.c1] = c1r;
        t[T.c1 + 1] = c1i;
        t[T.c0] = c0r;
        t[T.c0 + 1] = c0i;
    }
}

DevAnsatz ansatz_dev(const Ansatz *a) {
    DevAnsatz d;
    d.kind = a->kind;
    d.N = a->N;
    d.M = a->M;
    d.P = a->P;
    d.p = a->d_params.p;
    d.wtr = a->d_wtr.p;
    d.wti = a->d_wti.p;
    const bool rbm = a->kind == KIND_RBM || a->kind == KIND_CRBM;
    const long NM = (long)a->N * a->M;
    d.w32 = rbm ? a->d_f32.p : nullptr;
    d.ch32 = rbm ? a->d_f32.p + NM : nullptr;
    d.sh32 = rbm ? a->d_f32.p + 2 * NM : nullptr;
    d.a32 = rbm ? a->d_f32.p + 3 * NM : nullptr;
    d.b32 = rbm ? a->d_f32.p + 3 * NM + a->N : nullptr;
    d.m32 = a->kind == KIND_MLP ? (const float *)a->d_f32.p : nullptr;
    d.cs64 = rbm ? a->d_cs64.p : nullptr;
    return d;
}

bool ansatz_refresh_derived(Ansatz *a) {
    if (a->kind == KIND_MF) return true;
    if (is_vit(a->kind)) {
        NQS_LAUNCH("derive_vit_tables");
        k_vit_tables<<<1, 256, 0, ctx().stream>>>(ansatz_dev(a), a->d_wtr.p);
        return NQS_CUDA(cudaGetLastError());
    }
    long work = a->kind == KIND_MLP ? (long)a->M * a->N + (long)a->M * mlp32_pitch(a->M) : (long)a->M * a->N;
    NQS_LAUNCH("derive_weights");
    // 64-thread blocks: the tables' FP64 cosh / sinh / sincos are FP64-pipe work (2 FMAs per
    // clock per SM on this GPU), so the weights are spread over as many SMs as they fill
    k_derive<<<(unsigned)((work + 63) / 64), 64, 0, ctx().stream>>>(ansatz_dev(a), a->d_wtr.p,
                                                                     a->d_wti.p, a->d_f32.p, a->d_cs64.p);
    return NQS_CUDA(cudaGetLastError());
}

bool ansatz_sync(Ansatz *a, bool force) {
    size_t bytes = sizeof(double) * (size_t)a->P;
    bool same = a->dev_valid && memcmp(a->h_params, a->h_shadow, bytes) == 0;
    if (same && !force) return true;
    if (!NQS_CUDA(cudaMemcpyAsync(a->d_params.p, a->h_params, bytes, cudaMemcpyHostToDevice,
                                  ctx().stream)))
        return false;
    if (same) return true;
    memcpy(a->h_shadow, a->h_params, bytes);
    a->dev_valid = true;
    return ansatz_refresh_derived(a);
}

bool ansatz_pull(Ansatz *a) {
    size_t bytes = sizeof(double) * (size_t)a->P;
    if (!NQS_CUDA(cudaMemcpyAsync(a->h_params, a->d_params.p, bytes, cudaMemcpyDeviceToHost,
                                  ctx().stream)))
        return false;
    if (!NQS_CUDA(cudaStreamSynchronize(ctx().stream))) return false;
    memcpy(a->h_shadow, a->h_params, bytes);
    return true;
}

// ---------------------------------------------------------------- program builder

struct PermEntry {
    std::vector<int> perm;
    std::vector<double> chars;
    DevBuf<int> d_perm;
    DevBuf<double> d_chars;
};
static std::map<const void *, PermEntry *> g_perm_cache;

static bool stage_perm(const nqs_symproj_wrapper_t *w, const int **dp, const double **dc) {
    size_t np = (size_t)w->num_group_elements * w->num_sites;
    PermEntry *&e = g_perm_cache[(const void *)w->perm];
    if (!e) e = new PermEntry();
    bool same = e->perm.size() == np && e->chars.size() == (size_t)w->num_group_elements &&
                memcmp(e->perm.data(), w->perm, np * sizeof(int)) == 0 &&
                memcmp(e->chars.data(), w->characters, sizeof(double) * w->num_group_elements) == 0;
    if (!same) {
        for (size_t k = 0; k < np; k++)
            if (w->perm[k] < 0 || w->perm[k] >= w->num_sites) {
                set_error("symproj permutation entry %d out of range", w->perm[k]);
                return false;
            }
        e->perm.assign(w->perm, w->perm + np);
        e->chars.assign(w->characters, w->characters + w->num_group_elements);
        if (!e->d_perm.ensure(np) || !e->d_chars.ensure((size_t)w->num_group_elements)) return false;
        if (!NQS_CUDA(cudaMemcpy(e->d_perm.p, w->perm, np * sizeof(int), cudaMemcpyHostToDevice)))
            return false;
        if (!NQS_CUDA(cudaMemcpy(e->d_chars.p, w->characters, sizeof(double) * w->num_group_elements,
                                 cudaMemcpyHostToDevice)))
            return false;
    }
    *dp = e->d_perm.p;
    *dc = e->d_chars.p;
    return true;
}

// Square-lattice translation table of upstream src/nqs/nqs_translation.c:37-50:
// row g = tx * Ly + ty, entry x * Ly + y = ((x + tx) mod Lx) * Ly + (y + ty) mod Ly.
static const std::vector<int> *translation_table(int Lx, int Ly) {
    static std::map<std::pair<int, int>, std::vector<int>> tabs;
    std::vector<int> &t = tabs[{Lx, Ly}];
    if (t.empty()) {
        const int N = Lx * Ly;
        t.resize((size_t)N * N);
        for (int tx = 0; tx < Lx; tx++)
            for (int ty = 0; ty < Ly; ty++)
                for (int x = 0; x < Lx; x++)
                    for (int y = 0; y < Ly; y++)
                        t[(size_t)(tx * Ly + ty) * N + x * Ly + y] = ((x + tx) % Lx) * Ly + (y + ty) % Ly;
    }
    return &t;
}

static uint64_t marshall_mask(int sx, int sy, int N) {
    uint64_t m = 0;
    for (int x = 0; x < sx; x++)
        for (int y = 0; y < sy; y++)
            if (((x + y) & 1) == 0) {
                int idx = x * sy + y;
                if (idx < N && idx < 64) m |= 1ull << idx;
            }
    return m;
}

bool build_amp(nqs_log_amp_fn_t fn, void *user, int num_sites, DevAmp *out, Ansatz **base) {
    memset(out, 0, sizeof(*out));
    // Walk the wrapper chain from the outside in.
    int layers_type[8];
    const void *layers_user[8];
    int nl = 0;
    while (true) {
        if (fn == nqs_ansatz_log_amp) break;
        if (nl >= 8) {
            set_error("amplitude wrapper chain too deep");
            return false;
        }
        if (fn == nqs_marshall_log_amp) {
            auto *w = (const nqs_marshall_wrapper_t *)user;
            if (!w) { set_error("NULL Marshall wrapper"); return false; }
            layers_type[nl] = 1;
            layers_user[nl++] = w;
            fn = w->base_log_amp;
            user = w->base_user;
        } else if (fn == nqs_translation_log_amp) {
            auto *w = (const nqs_translation_wrapper_t *)user;
            if (!w || w->size_x <= 0 || w->size_y <= 0) {
                set_error("invalid translation wrapper");
                return false;
            }
            layers_type[nl] = 3;
            layers_user[nl++] = w;
            fn = w->base_log_amp;
            user = w->base_user;
        } else if (fn == nqs_symproj_log_amp) {
            auto *w = (const nqs_symproj_wrapper_t *)user;
            if (!w || !w->perm || !w->characters || w->num_group_elements <= 0) {
                set_error("invalid symproj wrapper");
                return false;
            }
            layers_type[nl] = 2;
            layers_user[nl++] = w;
            fn = w->base_log_amp;
            user = w->base_user;
        } else {
            set_error("log_amp callback %p is not one of this library's amplitude programs "
                      "(nqs_ansatz_log_amp, nqs_marshall_log_amp, nqs_symproj_log_amp); "
                      "host callbacks are not evaluated",
                      (void *)fn);
            return false;
        }
    }
    Ansatz *a = (Ansatz *)user;
    if (!a) { set_error("NULL ansatz"); return false; }
    if (a->N != num_sites) {
        set_error("num_sites %d does not match the ansatz (%d)", num_sites, a->N);
        return false;
    }
    if (!ansatz_sync(a)) return false;
    out->a = ansatz_dev(a);
    int seen_sym = 0;
    int outer_tmp = 0, inner_tmp = 0;
    uint64_t outer_m[8], inner_m[8];
    for (int k = 0; k < nl; k++) {
        if (layers_type[k] == 1) {
            auto *w = (const nqs_marshall_wrapper_t *)layers_user[k];
            uint64_t m = marshall_mask(w->size_x, w->size_y, num_sites);
            if (seen_sym) inner_m[inner_tmp++] = m;
            else outer_m[outer_tmp++] = m;
        } else {
            if (seen_sym) {
                set_error("nested symmetry projections are not supported");
                return false;
            }
            seen_sym = 1;
            nqs_symproj_wrapper_t tw;
            auto *w = (const nqs_symproj_wrapper_t *)layers_user[k];
            if (layers_type[k] == 3) {                 // translations as a symmetry projection
                auto *t = (const nqs_translation_wrapper_t *)layers_user[k];
                const std::vector<int> *tab = translation_table(t->size_x, t->size_y);
                static const std::vector<double> ones(64, 1.0);
                tw = nqs_symproj_wrapper_t{nullptr, nullptr, t->size_x * t->size_y, t->size_x * t->size_y,
                                           tab->data(), ones.data()};
                w = &tw;
            }
            if (w->num_sites != num_sites) {
                set_error("symproj num_sites %d != %d", w->num_sites, num_sites);
                return false;
            }
            out->G = w->num_group_elements;
            if (!stage_perm(w, &out->perm, &out->chars)) return false;
        }
    }
    if (outer_tmp > 3 || inner_tmp > 3) {
        set_error("more than three Marshall layers");
        return false;
    }
    out->n_outer = outer_tmp;
    out->n_inner = inner_tmp;
    for (int k = 0; k < outer_tmp; k++) out->outer_mask[k] = outer_m[k];
    for (int k = 0; k < inner_tmp; k++) out->inner_mask[k] = inner_m[k];
    if (base) *base = a;
    return true;
}

// ---------------------------------------------------------------- kernels

constexpr int kWarpsPerBlock = 4;

static int scratch_per_warp(const DevAnsatz &a) {
    return a.kind == KIND_MLP ? 4 * a.M : 2 * a.M;   // doubles
}

__global__ void k_log_amp(DevAmp A, const uint64_t *__restrict__ bits, int B, double *la,
                          double *ar) {
    extern __shared__ double sm[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int b = blockIdx.x * kWarpsPerBlock + warp;
    double *scr = sm + warp * (A.a.kind == KIND_MLP ? 4 * A.a.M : 2 * A.a.M);
    if (b >= B) return;
    double l, a;
    warp_amp_eval(A, bits[b], l, a, scr);
    if (lane == 0) {
        if (la) la[b] = l;
        if (ar) ar[b] = a;
    }
}

bool launch_log_amp(const DevAmp &A, const uint64_t *bits, int B, double *la, double *ar) {
    size_t smem = sizeof(double) * (size_t)scratch_per_warp(A.a) * kWarpsPerBlock;
    NQS_LAUNCH("log_amp");
    k_log_amp<<<(B + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, smem, ctx().stream>>>(
        A, bits, B, la, ar);
    return NQS_CUDA(cudaGetLastError());
}

// Writes alpha * d log psi / d theta of configuration `bits` into row `o`
// (accumulating when acc).  mode 1: real projection (src/nqs/nqs_ansatz.c:885-995);
// mode 2: holomorphic pair (o = Re, oi = Im; :1025-1091), where the weight may be
// complex, alpha + i alpha_im (MF / RBM / complex RBM).  `t` is a per-warp scratch of
// 2*M doubles (4*M for the MLP).
__device__ void warp_grad_row(const DevAnsatz &a, uint64_t bits, int mode, double *o, double *oi,
                              double alpha, bool acc, double *t, double alpha_im = 0.0) {
    int lane = threadIdx.x & 31;
    const int N = a.N, M = a.M;
    auto put = [&](double *row, long k, double v) {
        if (acc) row[k] += alpha * v;
        else row[k] = alpha * v;
    };
    // (alpha + i alpha_im)(re + i im) into (o, oi)
    auto put2 = [&](long k, double re, double im) {
        const double vr = alpha * re - alpha_im * im, vi = alpha * im + alpha_im * re;
        if (acc) {
            o[k] += vr;
            oi[k] += vi;
        } else {
            o[k] = vr;
            oi[k] = vi;
        }
    };
    if (a.kind == KIND_MF) {
        for (int i = lane; i < N; i += 32) {
            if (mode == 2) put2(i, (double)spin_of(bits, i), 0.0);
            else put(o, i, (double)spin_of(bits, i));
        }
        return;
    }
    if (is_vit(a.kind)) {
        // src/nqs/nqs_ansatz.c:475-567 (real), :732-843 (real projection of the complex ViT),
        // :1104-1256 (holomorphic): with A = sum_j s_pred_j s_j, B = sum_j s_pred_j,
        // S = sum_j s_j every complex derivative z is a table entry times A or B:
        // w_emb: A u, b_emb: B u, V_kl: W_k (w_l A + b_l B), attention r:
        // f_r (c1 (S - A) + c0 (N - B)), W_out_k: (V w)_k A + (V b)_k B, b_out: 1.
        const VitTab T = vit_tab(N, M);
        const double *tb = a.wtr;
        const int d = M;
        const bool cx = a.kind == KIND_VITC;
        double S;
        const double A = vit_spin_sum(a, bits, &S), B = tb[T.bsum];
        const double gs_r = tb[T.c1] * (S - A) + tb[T.c0] * ((double)N - B);
        const double gs_i = tb[T.c1 + 1] * (S - A) + tb[T.c0 + 1] * ((double)N - B);
        const long nblk = 3L * d + (long)d * d + N + 1;     // complex derivatives
        // block order of the real ViT layout: w_emb, b_emb, V, attention, W_out, b_out
        for (long q = lane; q < nblk; q += 32) {
            double zr, zi;
            long blk_off;                                    // index of the block start in q
            bool real_param = false;
            if (q < d) {
                zr = A * tb[T.u + 2 * q];
                zi = A * tb[T.u + 2 * q + 1];
                blk_off = 0;
            } else if (q < 2L * d) {
                const long l = q - d;
                zr = B * tb[T.u + 2 * l];
                zi = B * tb[T.u + 2 * l + 1];
                blk_off = 1;
            } else if (q < 2L * d + (long)d * d) {
                const long kl = q - 2L * d, k = kl / d, l = kl % d;
                const double er = tb[T.w + 2 * l] * A + tb[T.b + 2 * l] * B;
                const double ei = tb[T.w + 2 * l + 1] * A + tb[T.b + 2 * l + 1] * B;
                const double Wr = tb[T.W + 2 * k], Wi = tb[T.W + 2 * k + 1];
                zr = Wr * er - Wi * ei;
                zi = Wr * ei + Wi * er;
                blk_off = 2;
            } else if (q < 2L * d + (long)d * d + N) {
                const long r = q - 2L * d - (long)d * d;
                zr = tb[T.f + r] * gs_r;
                zi = tb[T.f + r] * gs_i;
                real_param = true;
                blk_off = 3;
            } else if (q < 3L * d + (long)d * d + N) {
                const long k = q - 2L * d - (long)d * d - N;
                zr = tb[T.vw + 2 * k] * A + tb[T.vb + 2 * k] * B;
                zi = tb[T.vw + 2 * k + 1] * A + tb[T.vb + 2 * k + 1] * B;
                blk_off = 4;
            } else {
                zr = 1.0;
                zi = 0.0;
                blk_off = 5;
            }
            if (!cx) {                                       // real ViT: same index q
                if (mode == 2) put2(q, zr, 0.0);
                else put(o, q, zr);
                continue;
            }
            // complex ViT: (re, im) parameter pairs at their own offsets
            long iR, iI;
            if (blk_off == 0) { iR = q; iI = d + q; }
            else if (blk_off == 1) { iR = 2L * d + (q - d); iI = 3L * d + (q - d); }
            else if (blk_off == 2) { iR = 4L * d + (q - 2L * d); iI = iR + (long)d * d; }
            else if (blk_off == 3) { iR = 4L * d + 2L * d * d + (q - 2L * d - (long)d * d); iI = -1; }
            else if (blk_off == 4) {
                const long k = q - 2L * d - (long)d * d - N;
                iR = 4L * d + 2L * d * d + N + k;
                iI = iR + d;
            } else { iR = 6L * d + 2L * d * d + N; iI = iR + 1; }
            if (mode == 2) {
                put2(iR, zr, zi);
                if (!real_param) put2(iI, -zi, zr);
            } else {
                put(o, iR, zr);
                if (!real_param) put(o, iI, -zi);
            }
        }
        __syncwarp();
        return;
    }
    if (a.kind == KIND_MLP) {
        // back-propagation through the two tanh layers (extension)
        double *h1 = t, *h2 = t + M, *d2 = t + 2 * M, *d1 = t + 3 * M;
        const double *b1 = a.p + (long)M * N, *W2 = b1 + M, *b2 = W2 + (long)M * M;
        const double *wr = b2 + M, *wi = wr + M;
        for (int k = lane; k < M; k += 32) {
            double z = b1[k];
            for (int i = 0; i < N; i++) z += a.wtr[(long)i * M + k] * (double)spin_of(bits, i);
            h1[k] = tanh(z);
        }
        __syncwarp();
        for (int j = lane; j < M; j += 32) {
            double z = b2[j];
            for (int k = 0; k < M; k++) z += a.wti[(long)k * M + j] * h1[k];
            h2[j] = tanh(z);
        }
        __syncwarp();
        long o_b1 = (long)M * N, o_W2 = o_b1 + M, o_b2 = o_W2 + (long)M * M, o_wr = o_b2 + M;
        for (int pass = 0; pass < (mode == 2 ? 2 : 1); pass++) {
            double *row = pass ? oi : o;
            const double *head = pass ? wi : wr;
            for (int j = lane; j < M; j += 32) d2[j] = head[j] * (1.0 - h2[j] * h2[j]);
            __syncwarp();
            for (int k = lane; k < M; k += 32) {
                double s = 0.0;
                for (int j = 0; j < M; j++) s += W2[(long)j * M + k] * d2[j];
                d1[k] = s * (1.0 - h1[k] * h1[k]);
            }
            __syncwarp();
            for (long q = lane; q < (long)M * N; q += 32) {
                int k = (int)(q / N), i = (int)(q % N);
                put(row, q, d1[k] * (double)spin_of(bits, i));
            }
            for (int k = lane; k < M; k += 32) put(row, o_b1 + k, d1[k]);
            for (long q = lane; q < (long)M * M; q += 32) {
                int j = (int)(q / M), k = (int)(q % M);
                put(row, o_W2 + q, d2[j] * h1[k]);
            }
            for (int j = lane; j < M; j += 32) {
                put(row, o_b2 + j, d2[j]);
                put(row, o_wr + j, pass == 0 ? h2[j] : 0.0);
                put(row, o_wr + M + j, pass == 0 ? 0.0 : h2[j]);
            }
            if (lane == 0) {
                put(row, o_wr + 2 * M, pass == 0 ? 1.0 : 0.0);
                put(row, o_wr + 2 * M + 1, pass == 0 ? 0.0 : 1.0);
            }
            __syncwarp();
        }
        return;
    }
    // RBM / complex RBM: tanh of every hidden pre-activation into t[]
    double *tr = t, *ti = t + M;
    for (int h = lane; h < M; h += 32) {
        double xr, xi;
        rbm_theta(a, bits, h, xr, xi);
        if (a.kind == KIND_RBM) {
            tr[h] = tanh(xr);
            ti[h] = 0.0;
        } else {
            double r, i;
            ctanh_d(xr, xi, r, i);
            tr[h] = r;
            ti[h] = i;
        }
    }
    __syncwarp();
    if (a.kind == KIND_RBM) {
        for (long k = lane; k < a.P; k += 32) {
            double v;
            if (k < N) v = (double)spin_of(bits, (int)k);
            else if (k < N + M) v = tr[k - N];
            else {
                long q = k - N - M;
                v = tr[q / N] * (double)spin_of(bits, (int)(q % N));
            }
            if (mode == 2) put2(k, v, 0.0);
            else put(o, k, v);
        }
        __syncwarp();
        return;
    }
    long Pr = crbm_pr(a);
    for (long k = lane; k < Pr; k += 32) {
        double sr, si;   // (re, im) of d log psi / d theta_R; d/d theta_I = i * that
        if (k < N) {
            sr = (double)spin_of(bits, (int)k);
            si = 0.0;
        } else if (k < N + M) {
            sr = tr[k - N];
            si = ti[k - N];
        } else {
            long q = k - N - M;
            double s = (double)spin_of(bits, (int)(q % N));
            sr = tr[q / N] * s;
            si = ti[q / N] * s;
        }
        if (mode == 2) {
            put2(k, sr, si);
            put2(Pr + k, -si, sr);
        } else {
            put(o, k, sr);
            // real projection: d log|psi| / d theta_I = -Im(...), and 0 for the visible block
            put(o, Pr + k, k < N ? 0.0 : -si);
        }
    }
    __syncwarp();
}

__global__ void k_gradient(DevAnsatz a, const uint64_t *__restrict__ bits, int B, int mode, double *O,
                           double *Oi) {
    extern __shared__ double sm[];
    int warp = threadIdx.x >> 5;
    int b = blockIdx.x * kWarpsPerBlock + warp;
    double *scr = sm + warp * (a.kind == KIND_MLP ? 4 * a.M : 2 * a.M);
    if (b >= B) return;
    warp_grad_row(a, bits[b], mode, O + (size_t)b * a.P, Oi ? Oi + (size_t)b * a.P : nullptr, 1.0,
                  false, scr);
}

// Symmetry-projected gradient, src/nqs/nqs_symproj.c:82-155: the weights
// w_g = chi_g cos(arg_g) e^{lp_g - max} / sum_g' (...) are formed first, then
// the G base gradients are accumulated into the row in ascending g.
__global__ void k_symproj_gradient(DevAmp A, const uint64_t *__restrict__ bits, int B, double *O,
                                   double *wbuf) {
    extern __shared__ double sm[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int b = blockIdx.x * kWarpsPerBlock + warp;
    double *scr = sm + warp * (A.a.kind == KIND_MLP ? 4 * A.a.M : 2 * A.a.M);
    if (b >= B) return;
    const int N = A.a.N, G = A.G;
    uint64_t s = bits[b];
    double *lp = wbuf + (size_t)b * 2 * G, *cs = lp + G;
    double mx = -1e300;
    for (int g = 0; g < G; g++) {
        uint64_t pb = permute_bits(s, A.perm + (long)g * N, N);
        double l, a;
        warp_base_eval(A.a, pb, l, a, scr);
        a = apply_marshall(a, pb, A.n_inner, A.inner_mask);
        if (lane == 0) {
            lp[g] = l;
            cs[g] = A.chars[g] * cos(a);
        }
        mx = fmax(mx, l);
    }
    __syncwarp();
    double den = 0.0;
    for (int g = 0; g < G; g++) den += cs[g] * exp(lp[g] - mx);
    double *row = O + (size_t)b * A.a.P;
    for (long k = lane; k < A.a.P; k += 32) row[k] = 0.0;
    __syncwarp();
    if (den == 0.0) return;
    for (int g = 0; g < G; g++) {
        double w = cs[g] * exp(lp[g] - mx) / den;
        if (w == 0.0) continue;
        uint64_t pb = permute_bits(s, A.perm + (long)g * N, N);
        warp_grad_row(A.a, pb, 1, row, nullptr, w, true, scr);
    }
}

// Complex symmetry-projected gradient, src/nqs/nqs_symproj.c:157-261: with
// c_g = chi_g e^{lp_g - max + i arg_g} and w_g = c_g / sum_g' c_g', the rows
// (Re, Im) = sum_g w_g d log psi_base(g s) / d theta (holomorphic base gradient).
__global__ void k_symproj_gradient_complex(DevAmp A, const uint64_t *__restrict__ bits, int B, double *O,
                                           double *Oi, double *wbuf) {
    extern __shared__ double sm[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int b = blockIdx.x * kWarpsPerBlock + warp;
    double *scr = sm + warp * 2 * A.a.M;
    if (b >= B) return;
    const int N = A.a.N, G = A.G;
    uint64_t s = bits[b];
    double *lp = wbuf + (size_t)b * 2 * G, *ag = lp + G;
    double mx = -1e300;
    for (int g = 0; g < G; g++) {
        uint64_t pb = permute_bits(s, A.perm + (long)g * N, N);
        double l, a;
        warp_base_eval(A.a, pb, l, a, scr);
        a = apply_marshall(a, pb, A.n_inner, A.inner_mask);
        if (lane == 0) {
            lp[g] = l;
            ag[g] = a;
        }
        mx = fmax(mx, l);
    }
    __syncwarp();
    double dr = 0.0, di = 0.0;
    for (int g = 0; g < G; g++) {
        double m = A.chars[g] * exp(lp[g] - mx), sn, cs;
        sincos(ag[g], &sn, &cs);
        dr += m * cs;
        di += m * sn;
    }
    double *row = O + (size_t)b * A.a.P, *rowi = Oi + (size_t)b * A.a.P;
    for (long k = lane; k < A.a.P; k += 32) {
        row[k] = 0.0;
        rowi[k] = 0.0;
    }
    __syncwarp();
    const double d2 = dr * dr + di * di;
    if (d2 == 0.0) return;
    for (int g = 0; g < G; g++) {
        double m = A.chars[g] * exp(lp[g] - mx), sn, cs;
        sincos(ag[g], &sn, &cs);
        const double cr = m * cs, ci = m * sn;
        const double wr = (cr * dr + ci * di) / d2, wi = (ci * dr - cr * di) / d2;
        if (wr == 0.0 && wi == 0.0) continue;
        uint64_t pb = permute_bits(s, A.perm + (long)g * N, N);
        warp_grad_row(A.a, pb, 2, row, rowi, wr, true, scr, wi);
    }
}

static DevBuf<double> g_symw;

bool launch_symproj_gradient_complex(const DevAmp &A, const uint64_t *bits, int B, double *O, double *Oi) {
    if (A.a.kind == KIND_MLP) {
        set_error("complex symmetry-projected gradient: MF, RBM and complex RBM base ansatze only");
        return false;
    }
    if (!g_symw.ensure((size_t)B * 2 * A.G)) return false;
    size_t smem = sizeof(double) * (size_t)scratch_per_warp(A.a) * kWarpsPerBlock;
    NQS_LAUNCH("symproj_gradient_complex");
    k_symproj_gradient_complex<<<(B + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, smem,
                                 ctx().stream>>>(A, bits, B, O, Oi, g_symw.p);
    return NQS_CUDA(cudaGetLastError());
}

bool launch_symproj_gradient(const DevAmp &A, const uint64_t *bits, int B, double *O) {
    if (!g_symw.ensure((size_t)B * 2 * A.G)) return false;
    size_t smem = sizeof(double) * (size_t)scratch_per_warp(A.a) * kWarpsPerBlock;
    NQS_LAUNCH("symproj_gradient");
    k_symproj_gradient<<<(B + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, smem,
                         ctx().stream>>>(A, bits, B, O, g_symw.p);
    return NQS_CUDA(cudaGetLastError());
}

bool launch_gradient(const DevAnsatz &a, const uint64_t *bits, int B, int mode, double *O,
                            double *Oi) {
    size_t smem = sizeof(double) * (size_t)scratch_per_warp(a) * kWarpsPerBlock;
    NQS_LAUNCH("gradient");
    k_gradient<<<(B + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, smem, ctx().stream>>>(
        a, bits, B, mode, O, Oi);
    return NQS_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------- apply update
__global__ void k_axpy(double *p, const double *__restrict__ d, double step, long n) {
    long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] += step * d[k];
}

static DevBuf<double> g_delta_stage;

}  // namespace nqs

using namespace nqs;

// ---------------------------------------------------------------- C ABI

extern "C" {

nqs_ansatz_t *nqs_ansatz_create(const nqs_config_t *cfg, int num_sites) {
    clear_error();
    if (!cfg || num_sites <= 0) return nullptr;
    int kind = (int)cfg->ansatz;
    if (kind != KIND_MF && kind != KIND_RBM && kind != KIND_CRBM && kind != KIND_MLP && !is_vit(kind)) {
        set_error("ansatz kind %d is not available in this build", kind);
        return nullptr;
    }
    if (num_sites > kMaxSites) {
        set_error("num_sites %d > %d", num_sites, kMaxSites);
        return nullptr;
    }
    if (!ensure_context()) return nullptr;
    int M = 0;
    if (kind == KIND_RBM || kind == KIND_CRBM)
        M = cfg->rbm_hidden_units > 0 ? cfg->rbm_hidden_units : 2 * num_sites;
    if (kind == KIND_MLP) {
        M = cfg->width > 0 ? cfg->width : 4 * num_sites;
        if (cfg->depth != 2) {
            set_error("deep MLP supports depth = 2 hidden layers (got %d)", cfg->depth);
            return nullptr;
        }
    }
    if (is_vit(kind)) M = cfg->width > 0 ? cfg->width : 4;     // src/nqs/nqs_ansatz.c:124 (d)
    if (M > 32 * kMaxJ) {
        set_error("hidden width %d > %d", M, 32 * kMaxJ);
        return nullptr;
    }
    Ansatz *a = new Ansatz();
    a->kind = kind;
    a->N = num_sites;
    a->M = M;
    a->P = num_params_of(kind, num_sites, M);
    size_t bytes = sizeof(double) * (size_t)a->P;
    if (!NQS_CUDA(cudaMallocHost(&a->h_params, bytes)) || !(a->h_shadow = (double *)malloc(bytes)) ||
        !a->d_params.ensure((size_t)a->P) ||
        !a->d_wtr.ensure(is_vit(kind) ? (size_t)vit_tab(num_sites, M).total
                                      : (size_t)num_sites * (M ? M : 1)) ||
        !a->d_wti.ensure(kind == KIND_MLP ? (size_t)M * M : (size_t)num_sites * (M ? M : 1)) ||
        !a->d_f32.ensure(kind == KIND_MLP ? (mlp32_floats(num_sites, M) + 1) / 2
                                          : 3 * (size_t)num_sites * (M ? M : 1) + num_sites + (M ? M : 1)) ||
        ((kind == KIND_RBM || kind == KIND_CRBM) && !a->d_cs64.ensure(4 * (size_t)num_sites * M))) {
        nqs_ansatz_free((nqs_ansatz_t *)a);
        return nullptr;
    }
    init_params(cfg, kind, num_sites, M, a->h_params);
    if (!ansatz_sync(a) || !NQS_CUDA(cudaStreamSynchronize(ctx().stream))) {
        nqs_ansatz_free((nqs_ansatz_t *)a);
        return nullptr;
    }
    return (nqs_ansatz_t *)a;
}

void nqs_ansatz_free(nqs_ansatz_t *h) {
    Ansatz *a = (Ansatz *)h;
    if (!a) return;
    if (a->h_params) cudaFreeHost(a->h_params);
    free(a->h_shadow);
    delete a;
}

long nqs_ansatz_num_params(const nqs_ansatz_t *h) { return h ? ((const Ansatz *)h)->P : 0; }

int nqs_ansatz_is_complex(const nqs_ansatz_t *h) {
    if (!h) return 0;
    int k = ((const Ansatz *)h)->kind;
    return (k == KIND_CRBM || k == KIND_MLP || k == KIND_VITC) ? 1 : 0;
}

double *nqs_ansatz_params_raw(nqs_ansatz_t *h) { return h ? ((Ansatz *)h)->h_params : nullptr; }

int nqs_ansatz_apply_update(nqs_ansatz_t *h, const double *delta, double step) {
    Ansatz *a = (Ansatz *)h;
    if (!a || !delta) return -1;
    if (!ensure_context() || !ansatz_sync(a)) return -1;
    if (!g_delta_stage.ensure((size_t)a->P)) return -1;
    Context &c = ctx();
    if (!NQS_CUDA(cudaMemcpyAsync(g_delta_stage.p, delta, sizeof(double) * a->P,
                                  cudaMemcpyHostToDevice, c.stream)))
        return -1;
    {
        NQS_LAUNCH("apply_update");
        k_axpy<<<(unsigned)((a->P + 255) / 256), 256, 0, c.stream>>>(a->d_params.p, g_delta_stage.p,
                                                                   step, a->P);
    }
    if (!NQS_CUDA(cudaGetLastError()) || !ansatz_refresh_derived(a) || !ansatz_pull(a)) return -1;
    return 0;
}

static int scalar_log_amp(nqs_log_amp_fn_t fn, const int *spins, int N, void *user, double *la,
                          double *ar) {
    if (!ensure_context()) return -1;
    DevAmp A;
    if (!build_amp(fn, user, N, &A, nullptr)) return -1;
    uint64_t *bits;
    if (!upload_spins(spins, 1, N, &bits)) return -1;
    static DevBuf<double> out;
    if (!out.ensure(2)) return -1;
    if (!launch_log_amp(A, bits, 1, out.p, out.p + 1)) return -1;
    double h[2];
    if (!NQS_CUDA(cudaMemcpyAsync(h, out.p, sizeof(h), cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return -1;
    *la = h[0];
    *ar = h[1];
    return 0;
}

void nqs_ansatz_log_amp(const int *spins, int num_sites, void *user, double *out_log_abs,
                        double *out_arg) {
    double la = 0.0, ar = 0.0;
    Ansatz *a = (Ansatz *)user;
    if (a && spins && num_sites == a->N) {                 // src/nqs/nqs_ansatz.c:851-872
        if (scalar_log_amp(nqs_ansatz_log_amp, spins, num_sites, user, &la, &ar) != 0) la = ar = 0.0;
    }
    if (out_log_abs) *out_log_abs = la;
    if (out_arg) *out_arg = ar;
}

void nqs_marshall_log_amp(const int *spins, int num_sites, void *user, double *out_log_abs,
                          double *out_arg) {
    double la = 0.0, ar = 0.0;
    if (user && spins) scalar_log_amp(nqs_marshall_log_amp, spins, num_sites, user, &la, &ar);
    if (out_log_abs) *out_log_abs = la;
    if (out_arg) *out_arg = ar;
}

void nqs_symproj_log_amp(const int *spins, int num_sites, void *user, double *out_log_abs,
                         double *out_arg) {
    double la = 0.0, ar = 0.0;
    auto *w = (nqs_symproj_wrapper_t *)user;
    if (w && spins && num_sites == w->num_sites)
        if (scalar_log_amp(nqs_symproj_log_amp, spins, num_sites, user, &la, &ar) != 0) la = ar = 0.0;
    if (out_log_abs) *out_log_abs = la;
    if (out_arg) *out_arg = ar;
}

int nqs_marshall_parity(const int *spins, int size_x, int size_y) {
    // src/nqs/nqs_marshall.c:16-27 (host utility; the device program uses a popcount)
    int n = 0;
    for (int x = 0; x < size_x; x++)
        for (int y = 0; y < size_y; y++)
            if (((x + y) & 1) == 0 && spins[x * size_y + y] < 0) n++;
    return n & 1;
}

int nqs_gpu_log_amp_batch(nqs_log_amp_fn_t fn, void *user, const int *spins, int B, int N,
                          double *out_la, double *out_ar) {
    clear_error();
    if (!spins || B <= 0 || !ensure_context()) return -1;
    DevAmp A;
    if (!build_amp(fn, user, N, &A, nullptr)) return -1;
    uint64_t *bits;
    if (!upload_spins(spins, B, N, &bits)) return -1;
    static DevBuf<double> out;
    if (!out.ensure(2 * (size_t)B)) return -1;
    if (!launch_log_amp(A, bits, B, out.p, out.p + B)) return -1;
    Context &c = ctx();
    if (out_la && !NQS_CUDA(cudaMemcpyAsync(out_la, out.p, sizeof(double) * B, cudaMemcpyDeviceToHost,
                                            c.stream)))
        return -1;
    if (out_ar && !NQS_CUDA(cudaMemcpyAsync(out_ar, out.p + B, sizeof(double) * B,
                                            cudaMemcpyDeviceToHost, c.stream)))
        return -1;
    return NQS_CUDA(cudaStreamSynchronize(c.stream)) ? 0 : -1;
}

int nqs_gpu_gradient_batch(nqs_ansatz_t *h, nqs_gradient_fn_t gfn, void *guser, const int *spins,
                           int B, int complex_out, double *out_re, double *out_im) {
    clear_error();
    Ansatz *a = (Ansatz *)h;
    if (!a || !spins || B <= 0 || !out_re || (complex_out && !out_im)) return -1;
    if (!ensure_context() || !ansatz_sync(a)) return -1;
    uint64_t *bits;
    if (!upload_spins(spins, B, a->N, &bits)) return -1;
    static DevBuf<double> O;
    if (!O.ensure((size_t)B * a->P * (complex_out ? 2 : 1))) return -1;
    if (gfn == nullptr) {
        if (!launch_gradient(ansatz_dev(a), bits, B, complex_out ? 2 : 1, O.p,
                             complex_out ? O.p + (size_t)B * a->P : nullptr))
            return -1;
    } else if (gfn == nqs_symproj_gradient && !complex_out) {
        DevAmp A;
        if (!build_amp(nqs_symproj_log_amp, guser, a->N, &A, nullptr)) return -1;
        if (!launch_symproj_gradient(A, bits, B, O.p)) return -1;
    } else if (gfn == nqs_translation_gradient && !complex_out) {
        DevAmp A;
        if (!build_amp(nqs_translation_log_amp, guser, a->N, &A, nullptr)) return -1;
        if (!launch_symproj_gradient(A, bits, B, O.p)) return -1;
    } else if ((void *)gfn == (void *)nqs_symproj_gradient_complex && complex_out) {
        DevAmp A;
        if (!build_amp(nqs_symproj_log_amp, guser, a->N, &A, nullptr)) return -1;
        if (!launch_symproj_gradient_complex(A, bits, B, O.p, O.p + (size_t)B * a->P)) return -1;
    } else {
        set_error("gradient callback is not supported on the GPU");
        return -1;
    }
    Context &c = ctx();
    size_t bytes = sizeof(double) * (size_t)B * a->P;
    if (!NQS_CUDA(cudaMemcpyAsync(out_re, O.p, bytes, cudaMemcpyDeviceToHost, c.stream))) return -1;
    if (complex_out &&
        !NQS_CUDA(cudaMemcpyAsync(out_im, O.p + (size_t)B * a->P, bytes, cudaMemcpyDeviceToHost, c.stream)))
        return -1;
    return NQS_CUDA(cudaStreamSynchronize(c.stream)) ? 0 : -1;
}

int nqs_ansatz_logpsi_gradient(nqs_ansatz_t *h, const int *spins, int num_sites, double *out) {
    Ansatz *a = (Ansatz *)h;
    if (!a || !spins || !out || num_sites != a->N) return -1;
    return nqs_gpu_gradient_batch(h, nullptr, nullptr, spins, 1, 0, out, nullptr);
}

int nqs_ansatz_logpsi_gradient_complex(nqs_ansatz_t *h, const int *spins, int num_sites, double *re,
                                       double *im) {
    Ansatz *a = (Ansatz *)h;
    if (!a || !spins || !re || !im || num_sites != a->N) return -1;
    return nqs_gpu_gradient_batch(h, nullptr, nullptr, spins, 1, 1, re, im);
}

void nqs_translation_log_amp(const int *spins, int num_sites, void *user, double *out_log_abs,
                             double *out_arg) {
    double la = 0.0, ar = 0.0;
    auto *w = (nqs_translation_wrapper_t *)user;
    if (w && spins && num_sites == w->size_x * w->size_y)
        if (scalar_log_amp(nqs_translation_log_amp, spins, num_sites, user, &la, &ar) != 0) la = ar = 0.0;
    if (out_log_abs) *out_log_abs = la;
    if (out_arg) *out_arg = ar;
}

int nqs_translation_gradient(void *grad_user, nqs_ansatz_t *h, const int *spins, int num_sites, double *out) {
    auto *w = (nqs_translation_wrapper_t *)grad_user;
    if (!w || !h || !spins || !out || num_sites != w->size_x * w->size_y) return -1;
    return nqs_gpu_gradient_batch(h, nqs_translation_gradient, grad_user, spins, 1, 0, out, nullptr);
}

int nqs_symproj_gradient_complex(void *grad_user, nqs_ansatz_t *h, const int *spins, int num_sites,
                                 double *out_re, double *out_im) {
    auto *w = (nqs_symproj_wrapper_t *)grad_user;
    if (!w || !h || !spins || !out_re || !out_im || num_sites != w->num_sites) return -1;
    return nqs_gpu_gradient_batch(h, (nqs_gradient_fn_t)(void *)nqs_symproj_gradient_complex, grad_user, spins, 1,
                                  1, out_re, out_im);
}

int nqs_symproj_gradient(void *grad_user, nqs_ansatz_t *h, const int *spins, int num_sites,
                         double *out) {
    auto *w = (nqs_symproj_wrapper_t *)grad_user;
    if (!w || !h || !spins || !out || num_sites != w->num_sites) return -1;
    return nqs_gpu_gradient_batch(h, nqs_symproj_gradient, grad_user, spins, 1, 0, out, nullptr);
}

// Kagome permutation tables: host-side set-up restating
// src/nqs/nqs_symproj.c:269-371 (translations, and translations x C2).
#define KG_SITE(cx, cy, sub, Ly) (3 * ((cx) * (Ly) + (cy)) + (sub))

int nqs_kagome_translation_perm(int Lx, int Ly, int **out_perm, int *out_G) {
    if (Lx <= 0 || Ly <= 0 || !out_perm || !out_G) return -1;
    int N = 3 * Lx * Ly, G = Lx * Ly;
    int *perm = (int *)malloc(sizeof(int) * (size_t)G * N);
    if (!perm) return -1;
    int g = 0;
    for (int tx = 0; tx < Lx; tx++)
        for (int ty = 0; ty < Ly; ty++, g++)
            for (int cx = 0; cx < Lx; cx++)
                for (int cy = 0; cy < Ly; cy++)
                    for (int sub = 0; sub < 3; sub++)
                        perm[(size_t)g * N + KG_SITE(cx, cy, sub, Ly)] =
                            KG_SITE((cx + tx) % Lx, (cy + ty) % Ly, sub, Ly);
    *out_perm = perm;
    *out_G = G;
    return 0;
}

int nqs_kagome_p2_perm(int Lx, int Ly, int **out_perm, double **out_chars, int *out_G) {
    if (Lx <= 0 || Ly <= 0 || !out_perm || !out_chars || !out_G) return -1;
    int N = 3 * Lx * Ly, G = 2 * Lx * Ly;
    int *perm = (int *)malloc(sizeof(int) * (size_t)G * N);
    double *chars = (double *)malloc(sizeof(double) * (size_t)G);
    if (!perm || !chars) {
        free(perm);
        free(chars);
        return -1;
    }
    int g = 0;
    for (int half = 0; half < 2; half++)
        for (int tx = 0; tx < Lx; tx++)
            for (int ty = 0; ty < Ly; ty++, g++) {
                for (int cx = 0; cx < Lx; cx++)
                    for (int cy = 0; cy < Ly; cy++)
                        for (int sub = 0; sub < 3; sub++) {
                            int xs, ys;
                            if (!half) {
                                xs = (cx + tx) % Lx;
                                ys = (cy + ty) % Ly;
                            } else {   // C2 through the A site: B -> -a1, C -> -a2
                                int dx = sub == 1 ? -1 : 0, dy = sub == 2 ? -1 : 0;
                                xs = ((-cx + dx + tx) % Lx + Lx) % Lx;
                                ys = ((-cy + dy + ty) % Ly + Ly) % Ly;
                            }
                            perm[(size_t)g * N + KG_SITE(cx, cy, sub, Ly)] = KG_SITE(xs, ys, sub, Ly);
                        }
                chars[g] = 1.0;
            }
    *out_perm = perm;
    *out_chars = chars;
    *out_G = G;
    return 0;
}

// p6m on the L x L kagome torus, restating src/nqs/nqs_symproj.c:618-776 in exact
// integer coordinates: a point is (u, v) in units of a1/2 and a2/2, so sites are the
// points with u or v even (A = (2cx, 2cy), B = A + (1, 0), C = A + (0, 1)) and (1, 1) is
// the hexagon centre the rotations turn about.  Row g = op * L^2 + tx * L + ty maps output
// site p to the source site R(-60 k) M^m (p - t): translation t = (2tx, 2ty); mirror
// y -> sqrt(3)/2 - y is (u, v) -> (u + v - 1, 2 - v); rotation by -60 degrees is
// (u, v) -> (u + v, -u).
static int p6m_source_site(int L, int op, int tx, int ty, int cx, int cy, int sub) {
    int u = 2 * cx + (sub == 1) - 2 * tx, v = 2 * cy + (sub == 2) - 2 * ty;
    if (op >= 6) {
        int nu = u + v - 1, nv = 2 - v;
        u = nu;
        v = nv;
    }
    u -= 1;
    v -= 1;
    for (int r = 0; r < op % 6; r++) {
        int nu = u + v, nv = -u;
        u = nu;
        v = nv;
    }
    u += 1;
    v += 1;
    int bu = u & 1, bv = v & 1;
    if (bu && bv) return -1;                          // a hexagon centre, not a site
    int s = bu ? 1 : (bv ? 2 : 0);
    int X = ((((u - bu) / 2) % L) + L) % L, Y = ((((v - bv) / 2) % L) + L) % L;
    return KG_SITE(X, Y, s, L);
}

// C_6v character of op (src/nqs/nqs_symproj.c:683-736): ops 1, 5 = C6; 2, 4 = C3; 3 = C2;
// mirrors with even rotation index are sigma_v, odd are sigma_d.  E irreps carry d_E = 2.
static double c6v_character(int op, int irrep) {
    bool mir = op >= 6;
    int k = op % 6;
    bool c6 = !mir && (k == 1 || k == 5), c3 = !mir && (k == 2 || k == 4), c2 = !mir && k == 3;
    bool sv = mir && k % 2 == 0, sd = mir && k % 2 == 1;
    switch (irrep) {
    case NQS_SYMPROJ_KAGOME_GAMMA_A1: return 1.0;
    case NQS_SYMPROJ_KAGOME_GAMMA_A2: return mir ? -1.0 : 1.0;
    case NQS_SYMPROJ_KAGOME_GAMMA_B1: return (c6 || c2 || sd) ? -1.0 : 1.0;
    case NQS_SYMPROJ_KAGOME_GAMMA_B2: return (c6 || c2 || sv) ? -1.0 : 1.0;
    case NQS_SYMPROJ_KAGOME_GAMMA_E1: return mir ? 0.0 : c6 ? 2.0 : c3 ? -2.0 : c2 ? -4.0 : 4.0;
    case NQS_SYMPROJ_KAGOME_GAMMA_E2: return mir ? 0.0 : (c6 || c3) ? -2.0 : 4.0;
    }
    return 1.0;
}

int nqs_kagome_p6m_perm_irrep(int L, nqs_symproj_kagome_irrep_t irrep, int **out_perm, double **out_chars,
                              int *out_G) {
    if (L <= 0 || !out_perm || !out_chars || !out_G || (int)irrep < 0 || (int)irrep > 5) return -1;
    int N = 3 * L * L, G = 12 * L * L;
    int *perm = (int *)malloc(sizeof(int) * (size_t)G * N);
    double *chars = (double *)malloc(sizeof(double) * (size_t)G);
    if (!perm || !chars) {
        free(perm);
        free(chars);
        return -1;
    }
    int g = 0;
    for (int op = 0; op < 12; op++)
        for (int tx = 0; tx < L; tx++)
            for (int ty = 0; ty < L; ty++, g++) {
                for (int cx = 0; cx < L; cx++)
                    for (int cy = 0; cy < L; cy++)
                        for (int sub = 0; sub < 3; sub++) {
                            int src = p6m_source_site(L, op, tx, ty, cx, cy, sub);
                            if (src < 0) {
                                free(perm);
                                free(chars);
                                return -1;
                            }
                            perm[(size_t)g * N + KG_SITE(cx, cy, sub, L)] = src;
                        }
                chars[g] = c6v_character(op, (int)irrep);
            }
    *out_perm = perm;
    *out_chars = chars;
    *out_G = G;
    return 0;
}

int nqs_kagome_p6m_perm(int L, int **out_perm, double **out_chars, int *out_G) {
    return nqs_kagome_p6m_perm_irrep(L, NQS_SYMPROJ_KAGOME_GAMMA_A1, out_perm, out_chars, out_G);
}

// Rotations about a fixed centre, then a translation (src/nqs/nqs_symproj.c:436-590), in
// exact integer coordinates of 1/S lattice vectors: site (cx, cy, sub) sits at
// (S cx + h [sub = 1], S cy + h [sub = 2]), h = S / 2; the source of output site p is
// R(-60 steps)(p - c) + c - S t, with R(-60)(u, v) = (u + v, -u).
static int rot_shift_source(int L, int S, int cu, int cv, int steps, int tx, int ty, int cx, int cy, int sub) {
    const int h = S / 2;
    int u = S * cx + (sub == 1 ? h : 0) - cu, v = S * cy + (sub == 2 ? h : 0) - cv;
    for (int r = 0; r < steps; r++) {
        int nu = u + v, nv = -u;
        u = nu;
        v = nv;
    }
    u += cu - S * tx;
    v += cv - S * ty;
    auto fdiv = [](int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); };
    const int qu = fdiv(u, h), qv = fdiv(v, h);
    if (qu * h != u || qv * h != v) return -1;         // not on the half-lattice
    const int bu = qu & 1, bv = qv & 1;
    if (bu && bv) return -1;                            // a hexagon centre
    const int X = ((fdiv(qu - bu, 2)) % L + L) % L, Y = ((fdiv(qv - bv, 2)) % L + L) % L;
    return KG_SITE(X, Y, bu ? 1 : (bv ? 2 : 0), L);
}

static int rot_group_perm(int L, int S, int cu, int cv, int nops, int step_per_op, int **out_perm, double **out_chars,
                          int *out_G) {
    if (L <= 0 || !out_perm || !out_chars || !out_G) return -1;
    const int N = 3 * L * L, G = nops * L * L;
    int *perm = (int *)malloc(sizeof(int) * (size_t)G * N);
    double *chars = (double *)malloc(sizeof(double) * (size_t)G);
    if (!perm || !chars) {
        free(perm);
        free(chars);
        return -1;
    }
    int g = 0;
    for (int k = 0; k < nops; k++)
        for (int tx = 0; tx < L; tx++)
            for (int ty = 0; ty < L; ty++, g++) {
                for (int cx = 0; cx < L; cx++)
                    for (int cy = 0; cy < L; cy++)
                        for (int sub = 0; sub < 3; sub++) {
                            int src = rot_shift_source(L, S, cu, cv, k * step_per_op, tx, ty, cx, cy, sub);
                            if (src < 0) {
                                free(perm);
                                free(chars);
                                return -1;
                            }
                            perm[(size_t)g * N + KG_SITE(cx, cy, sub, L)] = src;
                        }
                chars[g] = 1.0;
            }
    *out_perm = perm;
    *out_chars = chars;
    *out_G = G;
    return 0;
}

// C3 about the up-triangle centroid (a1 + a2)/6 = (1, 1) in sixths
int nqs_kagome_p3_perm(int L, int **out_perm, double **out_chars, int *out_G) {
    return rot_group_perm(L, 6, 1, 1, 3, 2, out_perm, out_chars, out_G);
}

// C6 about the hexagon centre (a1 + a2)/2 = (1, 1) in halves
int nqs_kagome_p6_perm(int L, int **out_perm, double **out_chars, int *out_G) {
    return rot_group_perm(L, 2, 1, 1, 6, 1, out_perm, out_chars, out_G);
}

}  // extern "C"
