// Local energies: bond tables, the fused local-estimator kernel and the
// nqs_local_energy* entry points.
//
// Fused estimator (RBM / complex RBM, any Marshall layers): one warp per
// sample.  Each lane computes theta_h for its hidden units once, caches
// log(2 cosh theta_h), and every connected configuration s' (single flip at u
// or pair flip (u, v)) costs one O(M) update
//     theta'_h = theta_h - 2 s_u W_hu [- 2 s_v W_hv]
// plus M complex log-cosh evaluations and one warp butterfly, instead of the
// upstream O(N M) recomputation per connected configuration
// (src/nqs/nqs_gradient.c:24-30).  The same theta feeds the Jacobian row.
#include <math.h>

#include "nqs_amp.cuh"

namespace nqs {

// ---------------------------------------------------------------- bond tables

// Square / chain nearest-neighbour bonds in the upstream enumeration order
// (src/nqs/nqs_gradient.c:60-67, :98-107): for x, for y, the +x bond then the
// +y bond.  Periodic mode wraps a neighbour whenever the extent exceeds 1.
static void square_bonds(int Lx, int Ly, int pbc, std::vector<int> &b) {
    for (int x = 0; x < Lx; x++)
        for (int y = 0; y < Ly; y++) {
            int a = x * Ly + y;
            if (x + 1 < Lx) { b.push_back(a); b.push_back((x + 1) * Ly + y); }
            else if (pbc && Lx > 1) { b.push_back(a); b.push_back(y); }
            if (y + 1 < Ly) { b.push_back(a); b.push_back(x * Ly + y + 1); }
            else if (pbc && Ly > 1) { b.push_back(a); b.push_back(x * Ly); }
        }
}

// J1-J2 next-nearest bonds, src/nqs/nqs_gradient.c:146-159: for each
// plaquette the (x,y)-(x+1,y+1) diagonal then the (x,y+1)-(x+1,y) one.
static void diagonal_bonds(int Lx, int Ly, int pbc, std::vector<int> &b) {
    int xe = (pbc && Lx > 1) ? Lx : Lx - 1, ye = (pbc && Ly > 1) ? Ly : Ly - 1;
    for (int x = 0; x < xe; x++)
        for (int y = 0; y < ye; y++) {
            int x1 = (x + 1) % Lx, y1 = (y + 1) % Ly;
            b.push_back(x * Ly + y); b.push_back(x1 * Ly + y1);
            b.push_back(x * Ly + y1); b.push_back(x1 * Ly + y);
        }
}

// Kagome bonds, src/nqs/nqs_gradient.c:374-445: per unit cell the up-triangle
// (A-B, A-C, B-C) then the down-triangle {A(cx,cy), B(cx-1,cy), C(cx,cy-1)},
// site 3*(cx*Ly+cy)+sub; open boundaries drop down-triangles at cx=0 or cy=0.
static void kagome_bonds(int Lx, int Ly, int pbc, std::vector<int> &b) {
    auto S = [&](int cx, int cy, int sub) { return 3 * (cx * Ly + cy) + sub; };
    for (int cx = 0; cx < Lx; cx++)
        for (int cy = 0; cy < Ly; cy++) {
            int A = S(cx, cy, 0), B = S(cx, cy, 1), C = S(cx, cy, 2);
            int up[6] = {A, B, A, C, B, C};
            b.insert(b.end(), up, up + 6);
            int cxm, cym;
            if (pbc) { cxm = (cx - 1 + Lx) % Lx; cym = (cy - 1 + Ly) % Ly; }
            else {
                if (cx == 0 || cy == 0) continue;
                cxm = cx - 1;
                cym = cy - 1;
            }
            int Bm = S(cxm, cy, 1), Cm = S(cx, cym, 2);
            int dn[6] = {A, Bm, A, Cm, Bm, Cm};
            b.insert(b.end(), dn, dn + 6);
        }
}

struct BondEntry {
    DevBuf<int> d;
    int n1 = 0, n2 = 0;
};
static std::map<std::string, BondEntry *> g_bonds;

bool hamiltonian_build(const nqs_config_t *cfg, int size_x, int size_y, DevHam *H) {
    memset(H, 0, sizeof(*H));
    int kind = (int)cfg->hamiltonian;
    int pbc = ctx().opts.square_pbc;
    if (size_x <= 0 || size_y <= 0) {
        set_error("invalid lattice %d x %d", size_x, size_y);
        return false;
    }
    std::vector<int> b1, b2;
    switch (kind) {
        case NQS_HAM_TFIM:
        case NQS_HAM_HEISENBERG:
        case NQS_HAM_XXZ:
            square_bonds(size_x, size_y, pbc, b1);
            break;
        case NQS_HAM_J1_J2:
            square_bonds(size_x, size_y, pbc, b1);
            diagonal_bonds(size_x, size_y, pbc, b2);
            break;
        case NQS_HAM_KAGOME_HEISENBERG:
            kagome_bonds(size_x, size_y, cfg->kagome_pbc, b1);
            pbc = cfg->kagome_pbc;
            break;
        default:
            set_error("Hamiltonian kind %d is not implemented on the GPU", kind);
            return false;
    }
    H->kind = kind;
    H->N = kind == NQS_HAM_KAGOME_HEISENBERG ? 3 * size_x * size_y : size_x * size_y;
    if (H->N > kMaxSites) {
        set_error("lattice has %d sites > %d", H->N, kMaxSites);
        return false;
    }
    char key[96];
    snprintf(key, sizeof(key), "%d:%d:%d:%d", kind, size_x, size_y, pbc);
    BondEntry *&e = g_bonds[key];
    if (!e) {
        e = new BondEntry();
        e->n1 = (int)b1.size() / 2;
        e->n2 = (int)b2.size() / 2;
        std::vector<int> all(b1);
        all.insert(all.end(), b2.begin(), b2.end());
        if (!e->d.ensure(all.size() + 2)) return false;
        if (!all.empty() &&
            !NQS_CUDA(cudaMemcpy(e->d.p, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice)))
            return false;
    }
    H->nb1 = e->n1;
    H->nb2 = e->n2;
    H->b1 = e->d.p;
    H->b2 = e->d.p + 2 * e->n1;
    H->J = cfg->j_coupling;
    H->J2 = cfg->j2_coupling;
    H->Jz = kind == NQS_HAM_XXZ ? cfg->j_z_coupling : cfg->j_coupling;
    H->Jxy = cfg->j_coupling;
    H->Gamma = cfg->transverse_field;
    return true;
}

// ---------------------------------------------------------------- kernels

constexpr int kWarps = 4;

// v * s_i for s_i = +-1 and -v: sign-bit flips on the integer pipe, exact
__device__ __forceinline__ double sflip(double v, uint64_t bits, int i) {
    return __longlong_as_double(__double_as_longlong(v) ^ (long long)(((bits >> i) & 1ull) << 63));
}
__device__ __forceinline__ double dneg(double v) {
    return __longlong_as_double(__double_as_longlong(v) ^ (long long)(1ull << 63));
}

// Jacobian row from precomputed tanh(theta) (tr, ti in shared memory);
// same layouts and values as warp_grad_row in nqs_ansatz.cu.  The weight block
// W[h][i] (entry N + M + h N + i) is swept with per-lane (h, i) counters and
// the products t_h s_i are sign flips, so the row costs stores, not FP64
// arithmetic or integer division.
__device__ void rbm_row_from_t(const DevAnsatz &a, uint64_t bits, int mode, double *o, double *oi,
                               const double *tr, const double *ti) {
    const int lane = threadIdx.x & 31;
    const int N = a.N, M = a.M;
    const bool cx = a.kind == KIND_CRBM;
    const long Pr = cx ? crbm_pr(a) : a.P;
    for (int k = lane; k < N; k += 32) {
        const double sr = sflip(1.0, bits, k);
        o[k] = sr;
        if (!cx) {
            if (mode == 2) oi[k] = 0.0;
        } else if (mode == 2) {
            oi[k] = 0.0;
            o[Pr + k] = -0.0;
            oi[Pr + k] = sr;
        } else {
            o[Pr + k] = 0.0;
        }
    }
    for (int h = lane; h < M; h += 32) {
        const long k = N + h;
        const double sr = tr[h], si = cx ? ti[h] : 0.0;
        o[k] = sr;
        if (!cx) {
            if (mode == 2) oi[k] = 0.0;
        } else if (mode == 2) {
            oi[k] = si;
            o[Pr + k] = dneg(si);
            oi[Pr + k] = sr;
        } else {
            o[Pr + k] = dneg(si);
        }
    }
    const long nw = (long)M * N, base = (long)N + M;
    int h = lane / N, i = lane % N;
    for (long e = lane; e < nw; e += 32) {
        const long k = base + e;
        const double sr = sflip(tr[h], bits, i);
        o[k] = sr;
        if (!cx) {
            if (mode == 2) oi[k] = 0.0;
        } else {
            const double si = sflip(ti[h], bits, i);
            if (mode == 2) {
                oi[k] = si;
                o[Pr + k] = dneg(si);
                oi[Pr + k] = sr;
            } else {
                o[Pr + k] = dneg(si);
            }
        }
        i += 32;
        while (i >= N) {
            i -= N;
            h++;
        }
    }
}

template <int J, bool CPLX>
__global__ void __launch_bounds__(32 * kWarps)
k_local_rbm(DevAmp A, DevHam H, const uint64_t *__restrict__ bits, int B, double *__restrict__ Er,
            double *__restrict__ Ei, double *__restrict__ O, double *__restrict__ Oi, int grad_mode,
            double *__restrict__ la_out) {
    extern __shared__ double sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarps + warp;
    if (b >= B) return;
    const DevAnsatz &a = A.a;
    const int N = a.N, M = a.M;
    const double *aR = a.p;
    const double *aI = a.p + crbm_pr(a);
    const uint64_t s = bits[b];

    double thr[J], thi[J], lr[J], li[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        int h = lane + 32 * j;
        thr[j] = thi[j] = lr[j] = li[j] = 0.0;
        if (h < M) {
            rbm_theta(a, s, h, thr[j], thi[j]);
            if (CPLX) clogcosh(thr[j], thi[j], lr[j], li[j]);
            else lr[j] = logcosh_r(thr[j]);
        }
    }
    const int par0 = marshall_count(A, s);

    // psi(s') / psi(s) for s' = s with sites u (and v >= 0) flipped
    auto ratio = [&](int u, int v, double &rre, double &rim) {
        const double su = (double)spin_of(s, u);
        const double sv = v >= 0 ? (double)spin_of(s, v) : 0.0;
        double dla = 0.0, dar = 0.0;
#pragma unroll
        for (int j = 0; j < J; j++) {
            int h = lane + 32 * j;
            if (h < M) {
                double xr = thr[j] - 2.0 * su * a.wtr[(long)u * M + h];
                double xi = thi[j];
                if (CPLX) xi -= 2.0 * su * a.wti[(long)u * M + h];
                if (v >= 0) {
                    xr -= 2.0 * sv * a.wtr[(long)v * M + h];
                    if (CPLX) xi -= 2.0 * sv * a.wti[(long)v * M + h];
                }
                if (CPLX) {
                    double l2, a2;
                    clogcosh(xr, xi, l2, a2);
                    dla += l2 - lr[j];
                    dar += a2 - li[j];
                } else {
                    dla += logcosh_r(xr) - lr[j];
                }
            }
        }
        dla = warp_sum(dla);
        if (CPLX) dar = warp_sum(dar);
        dla += -2.0 * su * aR[u];
        if (CPLX) dar += -2.0 * su * aI[u];
        uint64_t s2 = s ^ (1ull << u);
        if (v >= 0) {
            dla += -2.0 * sv * aR[v];
            if (CPLX) dar += -2.0 * sv * aI[v];
            s2 ^= 1ull << v;
        }
        dar += kPi * (double)(marshall_count(A, s2) - par0);
        double mag = exp(dla);
        double sn, cs;
        sincos(dar, &sn, &cs);
        rre = mag * cs;
        rim = mag * sn;
    };

    double e_re, e_im;
    if (H.kind == NQS_HAM_TFIM) {                        // src/nqs/nqs_gradient.c:50-82
        double diag = 0.0;
        for (int k = 0; k < H.nb1; k++)
            diag += -H.J * (double)(spin_of(s, H.b1[2 * k]) * spin_of(s, H.b1[2 * k + 1]));
        double ore = 0.0, oim = 0.0;
        for (int i = 0; i < N; i++) {
            double r, q;
            ratio(i, -1, r, q);
            ore += -H.Gamma * r;
            oim += -H.Gamma * q;
        }
        e_re = diag + ore;
        e_im = oim;
    } else {                                             // :87-139, :146-205, :374-445
        double diag = 0.0, ore = 0.0, oim = 0.0;
        for (int k = 0; k < H.nb1; k++) {
            int u = H.b1[2 * k], v = H.b1[2 * k + 1];
            int su = spin_of(s, u), sv = spin_of(s, v);
            diag += 0.25 * H.Jz * (double)(su * sv);
            if (su != sv) {
                double r, q;
                ratio(u, v, r, q);
                ore += 0.5 * H.Jxy * r;
                oim += 0.5 * H.Jxy * q;
            }
        }
        e_re = diag + ore;
        e_im = oim;
        if (H.nb2 > 0) {
            double d2 = 0.0, r2 = 0.0, i2 = 0.0;
            for (int k = 0; k < H.nb2; k++) {
                int u = H.b2[2 * k], v = H.b2[2 * k + 1];
                int su = spin_of(s, u), sv = spin_of(s, v);
                d2 += 0.25 * H.J2 * (double)(su * sv);
                if (su != sv) {
                    double r, q;
                    ratio(u, v, r, q);
                    r2 += 0.5 * H.J2 * r;
                    i2 += 0.5 * H.J2 * q;
                }
            }
            e_re = e_re + d2 + r2;
            e_im = e_im + i2;
        }
    }
    if (lane == 0) {
        if (Er) Er[b] = e_re;
        if (Ei) Ei[b] = e_im;
    }
    if (la_out) {
        double sr = 0.0;
#pragma unroll
        for (int j = 0; j < J; j++) sr += lr[j];
        double vr, vi;
        warp_visible(a, s, vr, vi);
        sr = vr + warp_sum(sr);
        if (lane == 0) la_out[b] = sr;
    }
    if (grad_mode) {
        double *tr = sm + warp * 2 * M, *ti = tr + M;
#pragma unroll
        for (int j = 0; j < J; j++) {
            int h = lane + 32 * j;
            if (h < M) {
                if (CPLX) ctanh_d(thr[j], thi[j], tr[h], ti[h]);
                else {
                    tr[h] = tanh(thr[j]);
                    ti[h] = 0.0;
                }
            }
        }
        __syncwarp();
        rbm_row_from_t(a, s, grad_mode, O + (size_t)b * a.P, Oi ? Oi + (size_t)b * a.P : nullptr, tr, ti);
    }
}

// ---------------------------------------------------------------- FP32 estimator
// Mixed-precision variant of k_local_rbm for the RBM / cRBM.  A flip of site u
// (and v) moves theta_h by delta_h = 2 s_u W_hu (+ 2 s_v W_hv), and
//   cosh(theta_h - delta_h) / cosh(theta_h) = cosh(delta_h) - tanh(theta_h) sinh(delta_h),
// so with t_h = tanh(theta_h) once per sample and cosh / sinh(2 W) tabulated
// once per step, the amplitude ratio of a connected configuration is a
// product of M complex factors (a few FP32 multiply-adds each) times the
// visible-bias exponential and the Marshall sign; no transcendental per
// hidden unit.  For a pair flip cosh / sinh(delta_u + delta_v) follow from the
// addition theorems.  Local energies are accumulated in FP32 and stored in FP64;
// the Jacobian row is written from the FP32 tanh values.

// tanh(x + i y) = (sinh 2x + i sin 2y) / (cosh 2x + cos 2y), with
// sinh / cosh from expm1 so that small |x| keeps its relative accuracy.
__device__ __forceinline__ float2 ctanh32(float x, float y) {
    if (fabsf(x) > 9.f) return make_float2(x > 0.f ? 1.f : -1.f, 0.f);   // |error| < 1e-7
    const float e = expm1f(2.f * x);
    const float ch = 1.f + e * e / (2.f * (1.f + e)), sh = 0.5f * (e + e / (1.f + e));
    float s2, c2;
    sincosf(2.f * y, &s2, &c2);
    const float den = ch + c2;
    return make_float2(sh / den, s2 / den);
}

__device__ __forceinline__ float2 cmul32(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// theta_h (FP32, ascending i) and t_h = tanh(theta_h) of hidden unit h.
template <bool CPLX>
__device__ __forceinline__ void rbm_theta32(const DevAnsatz &a, uint64_t s, int h, float2 &th, float2 &t) {
    float xr = a.b32[h].x, xi = a.b32[h].y;
    for (int i = 0; i < a.N; i++) {
        const float sp = (float)spin_of(s, i);
        const float2 w = a.w32[(long)i * a.M + h];
        xr = fmaf(sp, w.x, xr);
        if (CPLX) xi = fmaf(sp, w.y, xi);
    }
    th = make_float2(xr, CPLX ? xi : 0.f);
    t = CPLX ? ctanh32(xr, xi) : make_float2(tanhf(xr), 0.f);
}

// cosh(delta_h) - t_h sinh(delta_h) for the flip of u (and v >= 0).
template <bool CPLX>
__device__ __forceinline__ float2 flip_factor32(const DevAnsatz &a, int h, int u, float su, int v, float sv,
                                                float2 t) {
    const long M = a.M;
    float2 C = a.ch32[u * M + h], S = a.sh32[u * M + h];
    S.x *= su;
    S.y *= su;
    if (v >= 0) {
        const float2 Cv = a.ch32[v * M + h];
        float2 Sv = a.sh32[v * M + h];
        Sv.x *= sv;
        Sv.y *= sv;
        const float2 c1 = cmul32(C, Cv), c2 = cmul32(S, Sv), s1 = cmul32(S, Cv), s2 = cmul32(C, Sv);
        C = make_float2(c1.x + c2.x, c1.y + c2.y);
        S = make_float2(s1.x + s2.x, s1.y + s2.y);
    }
    if (!CPLX) return make_float2(C.x - t.x * S.x, 0.f);
    const float2 tS = cmul32(t, S);
    return make_float2(C.x - tS.x, C.y - tS.y);
}

template <int J, bool CPLX>
__global__ void __launch_bounds__(32 * kWarps)
k_local_rbm32(DevAmp A, DevHam H, const uint64_t *__restrict__ bits, int B, double *__restrict__ Er,
              double *__restrict__ Ei, double *__restrict__ O, double *__restrict__ Oi, int grad_mode) {
    extern __shared__ double sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarps + warp;
    if (b >= B) return;
    const DevAnsatz &a = A.a;
    const int N = a.N, M = a.M;
    const uint64_t s = bits[b];
    float2 th[J], tt[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int h = lane + 32 * j;
        th[j] = tt[j] = make_float2(0.f, 0.f);
        if (h < M) rbm_theta32<CPLX>(a, s, h, th[j], tt[j]);
    }
    const int par0 = marshall_count(A, s);

    // psi(s') / psi(s) for s' = s with sites u (and v >= 0) flipped
    auto ratio = [&](int u, int v, float &rre, float &rim) {
        const float su = (float)spin_of(s, u), sv = v >= 0 ? (float)spin_of(s, v) : 0.f;
        float2 p = make_float2(1.f, 0.f);
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int h = lane + 32 * j;
            if (h < M) p = cmul32(p, flip_factor32<CPLX>(a, h, u, su, v, sv, tt[j]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float2 q = make_float2(__shfl_xor_sync(0xffffffffu, p.x, o), __shfl_xor_sync(0xffffffffu, p.y, o));
            p = cmul32(p, q);
        }
        float dvr = -2.f * su * a.a32[u].x, dvi = -2.f * su * a.a32[u].y;
        uint64_t s2 = s ^ (1ull << u);
        if (v >= 0) {
            dvr -= 2.f * sv * a.a32[v].x;
            dvi -= 2.f * sv * a.a32[v].y;
            s2 ^= 1ull << v;
        }
        const float mag = expf(dvr);
        float sn = 0.f, cs = 1.f;
        if (CPLX) sincosf(dvi, &sn, &cs);
        float2 e = make_float2(mag * cs, mag * sn);
        if ((marshall_count(A, s2) - par0) & 1) e = make_float2(-e.x, -e.y);
        const float2 r = cmul32(p, e);
        rre = r.x;
        rim = r.y;
    };

    float e_re, e_im;
    if (H.kind == NQS_HAM_TFIM) {
        float diag = 0.f, ore = 0.f, oim = 0.f;
        for (int k = 0; k < H.nb1; k++)
            diag += -(float)H.J * (float)(spin_of(s, H.b1[2 * k]) * spin_of(s, H.b1[2 * k + 1]));
        for (int i = 0; i < N; i++) {
            float r, q;
            ratio(i, -1, r, q);
            ore += -(float)H.Gamma * r;
            oim += -(float)H.Gamma * q;
        }
        e_re = diag + ore;
        e_im = oim;
    } else {
        float diag = 0.f, ore = 0.f, oim = 0.f;
        for (int k = 0; k < H.nb1; k++) {
            const int u = H.b1[2 * k], v = H.b1[2 * k + 1];
            const int su = spin_of(s, u), sv = spin_of(s, v);
            diag += 0.25f * (float)H.Jz * (float)(su * sv);
            if (su != sv) {
                float r, q;
                ratio(u, v, r, q);
                ore += 0.5f * (float)H.Jxy * r;
                oim += 0.5f * (float)H.Jxy * q;
            }
        }
        e_re = diag + ore;
        e_im = oim;
        if (H.nb2 > 0) {
            float d2 = 0.f, r2 = 0.f, i2 = 0.f;
            for (int k = 0; k < H.nb2; k++) {
                const int u = H.b2[2 * k], v = H.b2[2 * k + 1];
                const int su = spin_of(s, u), sv = spin_of(s, v);
                d2 += 0.25f * (float)H.J2 * (float)(su * sv);
                if (su != sv) {
                    float r, q;
                    ratio(u, v, r, q);
                    r2 += 0.5f * (float)H.J2 * r;
                    i2 += 0.5f * (float)H.J2 * q;
                }
            }
            e_re = e_re + d2 + r2;
            e_im = e_im + i2;
        }
    }
    if (lane == 0) {
        if (Er) Er[b] = (double)e_re;
        if (Ei) Ei[b] = (double)e_im;
    }
    if (grad_mode) {
        double *tr = sm + warp * 2 * M, *ti = tr + M;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int h = lane + 32 * j;
            if (h < M) {
                tr[h] = (double)tt[j].x;
                ti[h] = (double)tt[j].y;
            }
        }
        __syncwarp();
        rbm_row_from_t(a, s, grad_mode, O + (size_t)b * a.P, Oi ? Oi + (size_t)b * a.P : nullptr, tr, ti);
    }
}

// Generic estimator: any program (symmetry projection, MLP).  Every connected
// configuration is evaluated from scratch, as upstream does.
__global__ void __launch_bounds__(32 * kWarps)
k_local_generic(DevAmp A, DevHam H, const uint64_t *__restrict__ bits, int B, double *Er, double *Ei,
                double *la_out) {
    extern __shared__ double sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarps + warp;
    if (b >= B) return;
    double *scr = sm + warp * 4 * A.a.M;
    const uint64_t s = bits[b];
    const int N = A.a.N;
    double la0, ar0;
    warp_amp_eval(A, s, la0, ar0, scr);
    auto ratio = [&](uint64_t s2, double &r, double &q) {
        double l, g;
        warp_amp_eval(A, s2, l, g, scr);
        double mag = exp(l - la0), sn, cs;
        sincos(g - ar0, &sn, &cs);
        r = mag * cs;
        q = mag * sn;
    };
    double e_re, e_im;
    if (H.kind == NQS_HAM_TFIM) {
        double diag = 0.0;
        for (int k = 0; k < H.nb1; k++)
            diag += -H.J * (double)(spin_of(s, H.b1[2 * k]) * spin_of(s, H.b1[2 * k + 1]));
        double ore = 0.0, oim = 0.0;
        for (int i = 0; i < N; i++) {
            double r, q;
            ratio(s ^ (1ull << i), r, q);
            ore += -H.Gamma * r;
            oim += -H.Gamma * q;
        }
        e_re = diag + ore;
        e_im = oim;
    } else {
        double diag = 0.0, ore = 0.0, oim = 0.0;
        for (int k = 0; k < H.nb1; k++) {
            int u = H.b1[2 * k], v = H.b1[2 * k + 1];
            int su = spin_of(s, u), sv = spin_of(s, v);
            diag += 0.25 * H.Jz * (double)(su * sv);
            if (su != sv) {
                double r, q;
                ratio(s ^ (1ull << u) ^ (1ull << v), r, q);
                ore += 0.5 * H.Jxy * r;
                oim += 0.5 * H.Jxy * q;
            }
        }
        e_re = diag + ore;
        e_im = oim;
        if (H.nb2 > 0) {
            double d2 = 0.0, r2 = 0.0, i2 = 0.0;
            for (int k = 0; k < H.nb2; k++) {
                int u = H.b2[2 * k], v = H.b2[2 * k + 1];
                int su = spin_of(s, u), sv = spin_of(s, v);
                d2 += 0.25 * H.J2 * (double)(su * sv);
                if (su != sv) {
                    double r, q;
                    ratio(s ^ (1ull << u) ^ (1ull << v), r, q);
                    r2 += 0.5 * H.J2 * r;
                    i2 += 0.5 * H.J2 * q;
                }
            }
            e_re = e_re + d2 + r2;
            e_im = e_im + i2;
        }
    }
    if (lane == 0) {
        if (Er) Er[b] = e_re;
        if (Ei) Ei[b] = e_im;
        if (la_out) la_out[b] = la0;
    }
}

// ---------------------------------------------------------------- FP32 MLP estimator
// Mixed-precision local energies and Jacobian rows of the 2-hidden-layer MLP:
// warp = sample.  A connected configuration changes the layer-1 pre-activations
// by one or two weight columns (O(M)); layer 2 is a full GEMV against W2^T in
// shared memory; ratios psi(s') / psi(s) = exp(d log|psi| + i d arg) in FP32.
// The Jacobian row (d log|psi| / d theta, the real projection) comes from FP32
// back-propagation and is stored in FP64.
constexpr int kMlpWarps = 16;

template <int MQ>
__global__ void __launch_bounds__(32 * kMlpWarps)
k_local_mlp32(DevAmp A, DevHam H, const uint64_t *__restrict__ bits, int B, double *__restrict__ Er,
              double *__restrict__ Ei, double *__restrict__ O) {
    extern __shared__ float fsm[];
    constexpr int MP = 32 * MQ;
    const DevAnsatz &a = A.a;
    const int N = a.N, M = a.M, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *w2t = fsm, *w2 = fsm + M * MP, *ws = fsm + 2 * M * MP + warp * 3 * MP;
    float *h1s = ws, *d2s = ws + MP, *d1s = ws + 2 * MP;
    {
        const float *g = a.m32 + (long)N * M;                  // W2^T then W2, both [M][MP]
        for (int e = threadIdx.x; e < 2 * M * MP; e += blockDim.x) fsm[e] = g[e];
    }
    __syncthreads();
    const int b = blockIdx.x * kMlpWarps + warp;
    if (b >= B) return;
    const uint64_t s = bits[b];
    float z1[MQ], h1[MQ], h2[MQ], la0, ar0;
    mlp32_z1<MQ>(a, s, z1);
    mlp32_forward<MQ>(a, w2t, z1, h1s, h1, h2, la0, ar0);
    const int par0 = marshall_count(A, s);

    auto ratio = [&](int u, int v, float &rre, float &rim) {
        float zp[MQ], g1[MQ], g2[MQ], la, ar;
        mlp32_z1_flip<MQ>(a, s, u, v, z1, zp);
        mlp32_forward<MQ>(a, w2t, zp, h1s, g1, g2, la, ar);
        uint64_t s2 = s ^ (1ull << u);
        if (v >= 0) s2 ^= 1ull << v;
        const float mag = expf(la - la0);
        float sn, cs;
        sincosf(ar - ar0, &sn, &cs);
        const float sg = ((marshall_count(A, s2) - par0) & 1) ? -1.f : 1.f;
        rre = sg * mag * cs;
        rim = sg * mag * sn;
    };

    float e_re = 0.f, e_im = 0.f;
    if (!Er && !Ei) {
        // Jacobian rows only (the local energies come from the tensor-core kernel)
    } else if (H.kind == NQS_HAM_TFIM) {
        for (int k = 0; k < H.nb1; k++)
            e_re += -(float)H.J * (float)(spin_of(s, H.b1[2 * k]) * spin_of(s, H.b1[2 * k + 1]));
        for (int i = 0; i < N; i++) {
            float r, q;
            ratio(i, -1, r, q);
            e_re += -(float)H.Gamma * r;
            e_im += -(float)H.Gamma * q;
        }
    } else {
        for (int g = 0; g < 2; g++) {
            const int nb = g ? H.nb2 : H.nb1;
            const int *bl = g ? H.b2 : H.b1;
            const float jz = g ? (float)H.J2 : (float)H.Jz, jxy = g ? (float)H.J2 : (float)H.Jxy;
            for (int k = 0; k < nb; k++) {
                const int u = bl[2 * k], v = bl[2 * k + 1];
                const int su = spin_of(s, u), sv = spin_of(s, v);
                e_re += 0.25f * jz * (float)(su * sv);
                if (su != sv) {
                    float r, q;
                    ratio(u, v, r, q);
                    e_re += 0.5f * jxy * r;
                    e_im += 0.5f * jxy * q;
                }
            }
        }
    }
    if (lane == 0) {
        if (Er) Er[b] = (double)e_re;
        if (Ei) Ei[b] = (double)e_im;
    }
    if (!O) return;
    // back-propagation of log|psi| = w_re . h2 + c_re
    const float *wr = a.m32 + (long)N * M + 2L * M * MP + 2 * M;
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        const int j = lane + 32 * q;
        d2s[j] = j < M ? wr[j] * (1.f - h2[q] * h2[q]) : 0.f;
        h1s[j] = h1[q];
    }
    __syncwarp();
    float d1[MQ];
#pragma unroll
    for (int q = 0; q < MQ; q++) d1[q] = 0.f;
    for (int j = 0; j < M; j++) {
        const float d = d2s[j];
        const float *row = w2 + j * MP + lane;
#pragma unroll
        for (int q = 0; q < MQ; q++) d1[q] = fmaf(row[32 * q], d, d1[q]);
    }
#pragma unroll
    for (int q = 0; q < MQ; q++) d1s[lane + 32 * q] = d1[q] * (1.f - h1[q] * h1[q]);
    __syncwarp();
    double *row = O + (size_t)b * a.P;
    const long oW2 = (long)M * N + M, ob2 = oW2 + (long)M * M, owr = ob2 + M;
    for (long q = lane; q < (long)M * N; q += 32) {
        const int k = (int)(q / N), i = (int)(q % N);
        row[q] = (double)(spin_of(s, i) > 0 ? d1s[k] : -d1s[k]);
    }
    for (int k = lane; k < M; k += 32) row[(long)M * N + k] = (double)d1s[k];
    for (long q = lane; q < (long)M * M; q += 32) {
        const int j = (int)(q / M), k = (int)(q % M);
        row[oW2 + q] = (double)(d2s[j] * h1s[k]);
    }
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        const int j = lane + 32 * q;
        if (j < M) {
            row[ob2 + j] = (double)d2s[j];
            row[owr + j] = (double)h2[q];
            row[owr + M + j] = 0.0;
        }
    }
    if (lane == 0) {
        row[owr + 2 * M] = 1.0;
        row[owr + 2 * M + 1] = 0.0;
    }
}

bool fp32_mlp_capable(const DevAmp &A) {
    return A.G == 0 && A.a.kind == KIND_MLP && A.a.m32 != nullptr && A.a.M <= 128 && A.a.N <= 64;
}

static bool launch_mlp32(const DevAmp &A, const DevHam &H, const uint64_t *bits, int B, double *Er, double *Ei,
                         double *O) {
    const int MQ = (A.a.M + 31) / 32, MP = 32 * MQ;
    const size_t smem = sizeof(float) * (2 * (size_t)A.a.M * MP + (size_t)kMlpWarps * 3 * MP);
    const dim3 grid((B + kMlpWarps - 1) / kMlpWarps), block(32 * kMlpWarps);
    cudaStream_t st = ctx().stream;
#define NQS_MCASE(QQ)                                                                                        \
    case QQ: {                                                                                               \
        static bool attr = false;                                                                            \
        if (!attr && !NQS_CUDA(cudaFuncSetAttribute(k_local_mlp32<QQ>,                                       \
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024))) \
            return false;                                                                                    \
        attr = true;                                                                                         \
        k_local_mlp32<QQ><<<grid, block, smem, st>>>(A, H, bits, B, Er, Ei, O);                              \
        break;                                                                                               \
    }
    switch (MQ) {
        NQS_MCASE(1) NQS_MCASE(2) NQS_MCASE(3) NQS_MCASE(4)
        default:
            set_error("MLP width %d unsupported by the FP32 estimator", A.a.M);
            return false;
    }
#undef NQS_MCASE
    return NQS_CUDA(cudaGetLastError());
}

template <int J, bool C>
static void launch_rbm(const DevAmp &A, const DevHam &H, const uint64_t *bits, int B, double *Er,
                       double *Ei, double *O, double *Oi, int gm, bool f32) {
    size_t smem = gm ? sizeof(double) * 2 * A.a.M * kWarps : 0;
    if (f32)
        k_local_rbm32<J, C><<<(B + kWarps - 1) / kWarps, 32 * kWarps, smem, ctx().stream>>>(A, H, bits, B, Er,
                                                                                          Ei, O, Oi, gm);
    else
        k_local_rbm<J, C><<<(B + kWarps - 1) / kWarps, 32 * kWarps, smem, ctx().stream>>>(A, H, bits, B, Er,
                                                                                        Ei, O, Oi, gm,
                                                                                        nullptr);
}

bool fp32_capable(const DevAmp &A) {
    return A.G == 0 && (A.a.kind == KIND_RBM || A.a.kind == KIND_CRBM) && A.a.w32 != nullptr;
}

bool launch_local_estimator(const DevAmp &A, const DevHam &H, const uint64_t *bits, int B, double *Er,
                            double *Ei, double *O, double *Oi, int grad_mode, bool fp32) {
    if (A.a.N != H.N) {
        set_error("ansatz has %d sites, lattice has %d", A.a.N, H.N);
        return false;
    }
    if (fp32 && fp32_mlp_capable(A) && grad_mode != 2) {
        if ((Er || Ei) && !ctx().opts.mlp_simt && mlp_tc_capable(A, H)) {
            // local energies with the second layer on the tensor cores; the Jacobian rows
            // (one back-propagation per sample) by the SIMT kernel
            {
                NQS_LAUNCH("local_energy_mlp_tc");
                if (!launch_mlp_eloc_tc(A, H, bits, B, Er, Ei)) return false;
            }
            if (!grad_mode) return true;
            NQS_LAUNCH("local_estimator_mlp32");
            return launch_mlp32(A, H, bits, B, nullptr, nullptr, O);
        }
        NQS_LAUNCH("local_estimator_mlp32");
        return launch_mlp32(A, H, bits, B, Er, Ei, grad_mode ? O : nullptr);
    }
    const bool fused = A.G == 0 && (A.a.kind == KIND_RBM || A.a.kind == KIND_CRBM);
    if (fused) {
        int J = (A.a.M + 31) / 32;
        bool c = A.a.kind == KIND_CRBM;
        const bool f32 = fp32 && fp32_capable(A);
        NQS_LAUNCH(f32 ? "local_estimator_fp32" : "local_estimator");
#define NQS_CASE(JJ)                                                                   \
    case JJ:                                                                           \
        if (c) launch_rbm<JJ, true>(A, H, bits, B, Er, Ei, O, Oi, grad_mode, f32);     \
        else launch_rbm<JJ, false>(A, H, bits, B, Er, Ei, O, Oi, grad_mode, f32);      \
        break;
        switch (J) {
            NQS_CASE(1) NQS_CASE(2) NQS_CASE(3) NQS_CASE(4) NQS_CASE(5) NQS_CASE(6) NQS_CASE(7) NQS_CASE(8)
            default:
                set_error("hidden width %d unsupported", A.a.M);
                return false;
        }
#undef NQS_CASE
        return NQS_CUDA(cudaGetLastError());
    }
    {
        size_t smem = sizeof(double) * 4 * (A.a.M ? A.a.M : 1) * kWarps;
        NQS_LAUNCH("local_generic");
        k_local_generic<<<(B + kWarps - 1) / kWarps, 32 * kWarps, smem, ctx().stream>>>(A, H, bits, B, Er,
                                                                                      Ei, nullptr);
        if (!NQS_CUDA(cudaGetLastError())) return false;
    }
    if (grad_mode) {
        if (A.G > 0) {
            if (grad_mode != 1) {
                set_error("holomorphic gradient through a symmetry projection is not implemented");
                return false;
            }
            return launch_symproj_gradient(A, bits, B, O);
        }
        return launch_gradient(A.a, bits, B, grad_mode, O, Oi);
    }
    return true;
}

}  // namespace nqs

using namespace nqs;

extern "C" {

int nqs_gpu_local_energy_batch(const nqs_config_t *cfg, int size_x, int size_y, const int *spins,
                               int B, nqs_log_amp_fn_t fn, void *user, double *out_re, double *out_im) {
    clear_error();
    if (!cfg || !spins || B <= 0 || !fn) {
        set_error("invalid arguments");
        return -1;
    }
    if (!ensure_context()) return -1;
    DevHam H;
    if (!hamiltonian_build(cfg, size_x, size_y, &H)) return -1;
    DevAmp A;
    if (!build_amp(fn, user, H.N, &A, nullptr)) return -1;
    uint64_t *bits;
    if (!upload_spins(spins, B, H.N, &bits)) return -1;
    static DevBuf<double> E;
    if (!E.ensure(2 * (size_t)B)) return -1;
    if (!launch_local_estimator(A, H, bits, B, E.p, E.p + B, nullptr, nullptr, 0)) return -1;
    Context &c = ctx();
    if (out_re && !NQS_CUDA(cudaMemcpyAsync(out_re, E.p, sizeof(double) * B, cudaMemcpyDeviceToHost,
                                            c.stream)))
        return -1;
    if (out_im && !NQS_CUDA(cudaMemcpyAsync(out_im, E.p + B, sizeof(double) * B, cudaMemcpyDeviceToHost,
                                            c.stream)))
        return -1;
    return NQS_CUDA(cudaStreamSynchronize(c.stream)) ? 0 : -1;
}

double nqs_local_energy(const nqs_config_t *cfg, int size_x, int size_y, const int *spins,
                        nqs_log_amp_fn_t fn, void *user) {
    if (!cfg || !spins || !fn) return 0.0;               // src/nqs/nqs_gradient.c:453
    double e = 0.0;
    if (nqs_gpu_local_energy_batch(cfg, size_x, size_y, spins, 1, fn, user, &e, nullptr) != 0) return NAN;
    return e;
}

void nqs_local_energy_batch(const nqs_config_t *cfg, int size_x, int size_y, const int *spins, int B,
                            nqs_log_amp_fn_t fn, void *user, double *out) {
    if (!cfg || !spins || !out || B <= 0) return;        // :900
    if (nqs_gpu_local_energy_batch(cfg, size_x, size_y, spins, B, fn, user, out, nullptr) != 0)
        for (int i = 0; i < B; i++) out[i] = NAN;
}

void nqs_local_energy_complex(const nqs_config_t *cfg, int size_x, int size_y, const int *spins,
                              nqs_log_amp_fn_t fn, void *user, double *re, double *im) {
    if (!cfg || !spins || !fn || !re || !im) {           // :800-804
        if (re) *re = 0;
        if (im) *im = 0;
        return;
    }
    if (nqs_gpu_local_energy_batch(cfg, size_x, size_y, spins, 1, fn, user, re, im) != 0) *re = *im = NAN;
}

void nqs_local_energy_batch_complex(const nqs_config_t *cfg, int size_x, int size_y, const int *spins,
                                    int B, nqs_log_amp_fn_t fn, void *user, double *re, double *im) {
    if (!cfg || !spins || !re || !im || B <= 0) return;
    if (nqs_gpu_local_energy_batch(cfg, size_x, size_y, spins, B, fn, user, re, im) != 0)
        for (int i = 0; i < B; i++) re[i] = im[i] = NAN;
}

}  // extern "C"
