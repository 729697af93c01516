// Metropolis sampler: one warp per Markov chain.
//
// A chain's state is its configuration (one uint64 in HBM); at the start of a
// launch the warp rebuilds theta_h = b_h + sum_i W_hi s_i in registers (lane =
// hidden unit) and then runs its proposals with O(M) incremental updates:
// a single flip at u or an exchange on bond (u, v) changes theta by one or two
// weight columns, the acceptance needs only Re log(2 cosh theta') (3 FP64
// transcendentals per hidden unit) and one warp butterfly.  Random numbers are
// computed redundantly by all lanes (xorshift64 state replicated in registers,
// or counter-based Philox4x32-10 keyed by (seed, chain) with counter = move
// index), so no lane ever waits on another for them.
//
// Compat mode (one chain, xorshift64) replays the upstream chain of
// src/nqs/nqs_sampler.c:86-117 proposal for proposal: same site choice
// (next % N), same draw order (a uniform is drawn only when the log-ratio is
// negative), same test log(u) < 2 (log|psi'| - log|psi|).
#include <math.h>

#include "nqs_amp.cuh"
#include "nqs_made.cuh"

namespace nqs {

struct Sampler {
    int N = 0, C = 1;
    nqs_config_t cfg{};
    nqs_gpu_options_t opts{};
    nqs_log_amp_fn_t fn = nullptr;
    void *user = nullptr;
    uint64_t move_counter = 0;
    DevBuf<uint64_t> d_bits, d_rng, d_samples;
    DevBuf<double> d_cla;                 // compat chain: upstream's cached log|psi|
    DevBuf<unsigned long long> d_counts;
    DevBuf<int> d_bonds, d_spins;
    int nb = 0;
    int *h_current = nullptr;        // pinned, N ints (next/current)
    Made *made = nullptr;            // learned proposal (optional)
};

bool sampler_run(Sampler *sm, int skip, int n_out, uint64_t *out, unsigned long long *move_dev = nullptr);

struct SampleArgs {
    int C, N;
    uint64_t *bits;
    uint64_t *rng;
    uint64_t seed;
    uint64_t move0;
    const unsigned long long *move_dev;   // when set, the first move index is read here (graph replay)
    int skip, decor, total;          // proposals: skip, then `total - skip` recorded in groups of decor
    uint64_t *out;
    int n_out;
    const int *bonds;
    int nb;
    unsigned long long *counts;
    double *cla;                     // compat chain: log|psi| the upstream sampler has cached (NaN: none yet)
};

__device__ __forceinline__ uint64_t xs_next(uint64_t &s) {   // src/nqs/nqs_sampler.c:31-38
    uint64_t x = s;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    s = x;
    return x;
}

// Shared proposal driver.  `delta(u, v, accept_fn)` evaluates the proposal.
// la0 = log|psi| of the chain's configuration at the current parameters.  The compat
// chain reproduces the upstream sampler's cache (src/nqs/nqs_sampler.c:74-75, 109-113):
// upstream compares every proposal with the log|psi| stored when the current
// configuration was accepted, which after a parameter update is the value at the old
// parameters until the next accepted move.  off = la0 - cached carries that difference
// into the acceptance until the first accept of the launch (off = 0 exactly when the
// parameters did not change); the cache is written back at the end.
template <int RNG, int MOVE, typename Eval, typename Commit>
__device__ __forceinline__ void run_chain(const SampleArgs &S, int c, uint64_t &s, Eval eval,
                                          Commit commit, unsigned long long &acc,
                                          unsigned long long &pro, double la0 = 0.0) {
    const int lane = threadIdx.x & 31;
    uint64_t st = RNG == NQS_GPU_RNG_XORSHIFT_COMPAT ? S.rng[c] : 0;
    const int per = S.decor > 0 ? S.decor : 1;
    const bool cached = RNG == NQS_GPU_RNG_XORSHIFT_COMPAT && S.cla != nullptr;
    double cache0 = cached ? S.cla[c] : 0.0;
    if (cached && isnan(cache0)) cache0 = la0;
    double off = cached ? la0 - cache0 : 0.0, cur = la0;
    bool moved = false;
    for (int t = 0; t < S.total; t++) {
        int u, v = -1;
        uint4 r = make_uint4(0, 0, 0, 0);
        if (RNG == NQS_GPU_RNG_XORSHIFT_COMPAT) {
            u = (int)(xs_next(st) % (uint64_t)S.N);
        } else {
            uint64_t m = S.move0 + (uint64_t)t;
            r = philox4x32(make_uint4((uint32_t)c, (uint32_t)m, (uint32_t)(m >> 32), 0u),
                           make_uint2((uint32_t)S.seed, (uint32_t)(S.seed >> 32)));
            if (MOVE == NQS_GPU_MOVE_EXCHANGE) {
                int k = (int)(((uint64_t)r.x * (uint64_t)S.nb) >> 32);
                u = S.bonds[2 * k];
                v = S.bonds[2 * k + 1];
            } else {
                u = (int)(((uint64_t)r.x * (uint64_t)S.N) >> 32);
            }
        }
        pro++;
        bool parallel = v >= 0 && (((s >> u) ^ (s >> v)) & 1ull) == 0;
        if (!parallel) {
            const double d = eval(u, v);
            double lr = 2.0 * (d + off);
            bool accept;
            if (lr >= 0.0) {
                accept = true;
            } else {
                double uni;
                if (RNG == NQS_GPU_RNG_XORSHIFT_COMPAT) {
                    uni = (double)(xs_next(st) >> 11) * (1.0 / 9007199254740992.0);
                } else {
                    uint64_t u53 = ((((uint64_t)r.z) << 32) | r.w) >> 11;
                    uni = (double)u53 * (1.0 / 9007199254740992.0);
                }
                accept = log(uni) < lr;
            }
            if (accept) {
                acc++;
                commit(u, v);
                s ^= 1ull << u;
                if (v >= 0) s ^= 1ull << v;
                cur += d;
                off = 0.0;
                moved = true;
            }
        }
        if (t >= S.skip && ((t - S.skip + 1) % per) == 0) {
            long idx = (long)((t - S.skip + 1) / per - 1) * S.C + c;
            if (idx < S.n_out && lane == 0) S.out[idx] = s;
        }
    }
    if (RNG == NQS_GPU_RNG_XORSHIFT_COMPAT && lane == 0) S.rng[c] = st;
    if (cached && lane == 0) S.cla[c] = moved ? cur : cache0;
}

constexpr int kSW = 4;   // warps (chains) per block

template <int J, bool CPLX, int RNG, int MOVE>
__global__ void __launch_bounds__(32 * kSW) k_sample_rbm(SampleArgs S, DevAmp A) {
    if (S.move_dev) S.move0 = *S.move_dev;
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * kSW + (threadIdx.x >> 5);
    if (c >= S.C) return;
    const DevAnsatz &a = A.a;
    const int M = a.M;
    const double *aR = a.p;
    uint64_t s = S.bits[c];
    double thr[J], thi[J], lr[J], nr[J], ni[J], nl[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        int h = lane + 32 * j;
        thr[j] = thi[j] = lr[j] = 0.0;
        if (h < M) {
            rbm_theta(a, s, h, thr[j], thi[j]);
            lr[j] = CPLX ? rlogcosh(thr[j], thi[j]) : logcosh_r(thr[j]);
        }
    }
    auto eval = [&](int u, int v) -> double {
        const double su = (double)spin_of(s, u);
        const double sv = v >= 0 ? (double)spin_of(s, v) : 0.0;
        double d = 0.0;
#pragma unroll
        for (int j = 0; j < J; j++) {
            int h = lane + 32 * j;
            nr[j] = thr[j];
            ni[j] = thi[j];
            nl[j] = lr[j];
            if (h < M) {
                nr[j] -= 2.0 * su * a.wtr[(long)u * M + h];
                if (CPLX) ni[j] -= 2.0 * su * a.wti[(long)u * M + h];
                if (v >= 0) {
                    nr[j] -= 2.0 * sv * a.wtr[(long)v * M + h];
                    if (CPLX) ni[j] -= 2.0 * sv * a.wti[(long)v * M + h];
                }
                nl[j] = CPLX ? rlogcosh(nr[j], ni[j]) : logcosh_r(nr[j]);
                d += nl[j] - lr[j];
            }
        }
        d = warp_sum(d) - 2.0 * su * aR[u];
        if (v >= 0) d -= 2.0 * sv * aR[v];
        return d;
    };
    auto commit = [&](int, int) {
#pragma unroll
        for (int j = 0; j < J; j++) {
            thr[j] = nr[j];
            thi[j] = ni[j];
            lr[j] = nl[j];
        }
    };
    double la0 = 0.0;
    if (RNG == NQS_GPU_RNG_XORSHIFT_COMPAT) {
        // log|psi| of the start configuration (Re of the visible term + hidden log-cosh)
#pragma unroll
        for (int j = 0; j < J; j++) la0 += lr[j];
        for (int i = lane; i < a.N; i += 32) la0 += aR[i] * (double)spin_of(s, i);
        la0 = warp_sum(la0);
    }
    unsigned long long acc = 0, pro = 0;
    run_chain<RNG, MOVE>(S, c, s, eval, commit, acc, pro, la0);
    if (lane == 0) {
        S.bits[c] = s;
        atomicAdd(&S.counts[0], acc);
        atomicAdd(&S.counts[1], pro);
    }
}

// ---------------------------------------------------------------- FP64 product-form chains
// Philox single-flip chains in FP64 without a transcendental per hidden unit: flipping
// site u moves theta_h by -2 s_u W_uh, and cosh(theta - d) / cosh(theta) = cosh d -
// tanh(theta) sinh d with cosh d = cosh(2 W_uh), sinh d = s_u sinh(2 W_uh) from the
// tables rebuilt after every update, so |psi(s') / psi(s)|^2 = exp(-4 s_u Re a_u)
// prod_h |cosh 2W_uh - s_u t_h sinh 2W_uh|^2 is a complex multiply-add per hidden unit
// and a warp product; t_h = tanh(theta_h) is recomputed for accepted moves only.  The
// acceptance is the log form's (ratio >= 1, else the uniform of the same Philox word below
// the ratio), so the chain is the same Markov chain.
__device__ __forceinline__ void ctanh64(double x, double y, double &tr, double &ti) {
    if (fabs(x) > 20.0) {                       // tanh(x + iy) -> sign(x) to double precision
        tr = x > 0.0 ? 1.0 : -1.0;
        ti = 0.0;
        return;
    }
    double s2, c2;
    sincos(2.0 * y, &s2, &c2);
    const double den = cosh(2.0 * x) + c2;
    tr = sinh(2.0 * x) / den;
    ti = s2 / den;
}

template <int J, bool CPLX>
__global__ void __launch_bounds__(32 * kSW) k_sample_rbm_prod(SampleArgs S, DevAmp A) {
    if (S.move_dev) S.move0 = *S.move_dev;
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * kSW + (threadIdx.x >> 5);
    if (c >= S.C) return;
    const DevAnsatz &a = A.a;
    const int M = a.M;
    const long NM = (long)a.N * M;
    const double *c2r = a.cs64, *c2i = c2r + NM, *s2r = c2i + NM, *s2i = s2r + NM;
    const double *aR = a.p;
    uint64_t s = S.bits[c];
    double thr[J], thi[J], tr[J], ti[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int h = lane + 32 * j;
        thr[j] = thi[j] = tr[j] = ti[j] = 0.0;
        if (h < M) {
            rbm_theta(a, s, h, thr[j], thi[j]);
            if (CPLX) ctanh64(thr[j], thi[j], tr[j], ti[j]);
            else tr[j] = tanh(thr[j]);
        }
    }
    const int per = S.decor > 0 ? S.decor : 1;
    unsigned long long acc = 0, pro = 0;
    for (int t = 0; t < S.total; t++) {
        const uint64_t m = S.move0 + (uint64_t)t;
        const uint4 r = philox4x32(make_uint4((uint32_t)c, (uint32_t)m, (uint32_t)(m >> 32), 0u),
                                   make_uint2((uint32_t)S.seed, (uint32_t)(S.seed >> 32)));
        const int u = (int)(((uint64_t)r.x * (uint64_t)S.N) >> 32);
        pro++;
        const double su = (double)spin_of(s, u);
        double q = 1.0;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int h = lane + 32 * j;
            if (h < M) {
                const long k = (long)u * M + h;
                const double sr = su * s2r[k];
                double fr = fma(-tr[j], sr, c2r[k]), fi = 0.0;
                if (CPLX) {
                    const double si = su * s2i[k];
                    fr = fma(ti[j], si, fr);                       // Re(c - t s)
                    fi = c2i[k] - fma(tr[j], si, ti[j] * sr);      // Im(c - t s)
                }
                q *= fr * fr + fi * fi;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q *= __shfl_xor_sync(0xffffffffu, q, o);
        const double R = q * exp(-4.0 * su * aR[u]);
        bool accept = R >= 1.0;
        if (!accept) {
            const uint64_t u53 = ((((uint64_t)r.z) << 32) | r.w) >> 11;
            accept = (double)u53 * (1.0 / 9007199254740992.0) < R;
        }
        if (accept) {
            acc++;
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int h = lane + 32 * j;
                if (h < M) {
                    thr[j] -= 2.0 * su * a.wtr[(long)u * M + h];
                    if (CPLX) {
                        thi[j] -= 2.0 * su * a.wti[(long)u * M + h];
                        ctanh64(thr[j], thi[j], tr[j], ti[j]);
                    } else {
                        tr[j] = tanh(thr[j]);
                    }
                }
            }
            s ^= 1ull << u;
        }
        if (t >= S.skip && ((t - S.skip + 1) % per) == 0) {
            const long idx = (long)((t - S.skip + 1) / per - 1) * S.C + c;
            if (idx < S.n_out && lane == 0) S.out[idx] = s;
        }
    }
    if (lane == 0) {
        S.bits[c] = s;
        atomicAdd(&S.counts[0], acc);
        atomicAdd(&S.counts[1], pro);
    }
}

// ---------------------------------------------------------------- FP32 chains
// Mixed-precision variant (Philox chains only).  The acceptance needs
// log|psi'/psi| = sum_h log|cosh(delta_h) - t_h sinh(delta_h)| + Re(visible
// change), with t_h = tanh(theta_h) kept per chain in FP32 and cosh / sinh of
// the weights tabulated once per step (one fast log per hidden unit and
// proposal instead of three FP64 transcendentals); an accepted move updates
// theta additively and recomputes t.  The uniform is drawn from the same
// Philox word as in the FP64 chain, as a 24-bit float.
template <int MOVE, bool LEARNED, typename Eval, typename Commit, typename Learned>
__device__ __forceinline__ void run_chain32(const SampleArgs &S, int c, uint64_t &s, Eval eval, Commit commit,
                                            Learned learned, uint32_t mix_thr, unsigned long long &acc,
                                            unsigned long long &pro, unsigned long long &lacc,
                                            unsigned long long &lpro) {
    const int lane = threadIdx.x & 31;
    const int per = S.decor > 0 ? S.decor : 1;
    for (int t = 0; t < S.total; t++) {
        int u, v = -1;
        const uint64_t m = S.move0 + (uint64_t)t;
        const uint4 r = philox4x32(make_uint4((uint32_t)c, (uint32_t)m, (uint32_t)(m >> 32), 0u),
                                   make_uint2((uint32_t)S.seed, (uint32_t)(S.seed >> 32)));
        pro++;
        if (LEARNED && r.y < mix_thr) {
            // learned proposal slot: the move kind depends on the random word
            // only, never on the state, so the mixture stays |psi|^2-invariant
            lpro++;
            if (learned(r)) {
                acc++;
                lacc++;
            }
        } else {
            if (MOVE == NQS_GPU_MOVE_EXCHANGE) {
                const int k = (int)(((uint64_t)r.x * (uint64_t)S.nb) >> 32);
                u = S.bonds[2 * k];
                v = S.bonds[2 * k + 1];
            } else {
                u = (int)(((uint64_t)r.x * (uint64_t)S.N) >> 32);
            }
            const bool parallel = v >= 0 && (((s >> u) ^ (s >> v)) & 1ull) == 0;
            if (!parallel) {
                const float lr = 2.f * eval(u, v);
                bool accept = lr >= 0.f;
                if (!accept) {
                    const float uni = ((float)(r.z >> 8) + 0.5f) * (1.f / 16777216.f);
                    accept = __logf(uni) < lr;
                }
                if (accept) {
                    acc++;
                    commit(u, v);
                    s ^= 1ull << u;
                    if (v >= 0) s ^= 1ull << v;
                }
            }
        }
        if (t >= S.skip && ((t - S.skip + 1) % per) == 0) {
            const long idx = (long)((t - S.skip + 1) / per - 1) * S.C + c;
            if (idx < S.n_out && lane == 0) S.out[idx] = s;
        }
    }
}

__device__ __forceinline__ float2 ctanh32s(float x, float y) {
    if (fabsf(x) > 9.f) return make_float2(x > 0.f ? 1.f : -1.f, 0.f);
    const float e = expm1f(2.f * x);
    const float ch = 1.f + e * e / (2.f * (1.f + e)), sh = 0.5f * (e + e / (1.f + e));
    float s2, c2;
    sincosf(2.f * y, &s2, &c2);
    const float den = ch + c2;
    return make_float2(sh / den, s2 / den);
}

template <int J, bool CPLX, int MOVE, bool LEARNED>
__global__ void __launch_bounds__(32 * kSW) k_sample_rbm32(SampleArgs S, DevAmp A, DevMade md) {
    if (S.move_dev) S.move0 = *S.move_dev;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.x * kSW + warp;
    const __nv_bfloat16 *Wsm = nullptr;
    float *h1 = nullptr, *h2 = nullptr;
    uint32_t mix_thr = 0;
    if (LEARNED) {
        // BF16 weights of the proposal model in shared memory for the log q of
        // the current configuration
        const long PM = made_off(md.N, md.H).total, wbytes = (PM * 2 + 15) / 16 * 16;
        __nv_bfloat16 *W = (__nv_bfloat16 *)smraw;
        for (long p = threadIdx.x; p < PM; p += blockDim.x) W[p] = md.w[p];
        __syncthreads();
        Wsm = W;
        h1 = (float *)(smraw + wbytes) + (size_t)warp * 2 * md.H;
        h2 = h1 + md.H;
        mix_thr = *md.active ? md.mix_thr : 0u;
    }
    if (c >= S.C) return;
    const DevAnsatz &a = A.a;
    const int M = a.M;
    const long Ml = M;
    uint64_t s = S.bits[c];
    float thr[J], thi[J], tr[J], ti[J], nr[J], ni[J];
    auto rebuild = [&]() {
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int h = lane + 32 * j;
            thr[j] = thi[j] = tr[j] = ti[j] = 0.f;
            if (h < M) {
                float xr = a.b32[h].x, xi = a.b32[h].y;
                for (int i = 0; i < a.N; i++) {
                    const float sp = (float)spin_of(s, i);
                    const float2 w = a.w32[(long)i * Ml + h];
                    xr = fmaf(sp, w.x, xr);
                    if (CPLX) xi = fmaf(sp, w.y, xi);
                }
                thr[j] = xr;
                thi[j] = CPLX ? xi : 0.f;
                if (CPLX) {
                    const float2 t = ctanh32s(xr, xi);
                    tr[j] = t.x;
                    ti[j] = t.y;
                } else {
                    tr[j] = tanhf(xr);
                }
            }
        }
    };
    rebuild();
    auto eval = [&](int u, int v) -> float {
        const float su = (float)spin_of(s, u), sv = v >= 0 ? (float)spin_of(s, v) : 0.f;
        float lg = 0.f;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int h = lane + 32 * j;
            nr[j] = thr[j];
            ni[j] = thi[j];
            if (h < M) {
                const float2 wu = a.w32[u * Ml + h];
                float2 C = a.ch32[u * Ml + h], Sh = a.sh32[u * Ml + h];
                Sh.x *= su;
                Sh.y *= su;
                nr[j] -= 2.f * su * wu.x;
                if (CPLX) ni[j] -= 2.f * su * wu.y;
                if (v >= 0) {
                    const float2 wv = a.w32[v * Ml + h], Cv = a.ch32[v * Ml + h];
                    float2 Sv = a.sh32[v * Ml + h];
                    Sv.x *= sv;
                    Sv.y *= sv;
                    nr[j] -= 2.f * sv * wv.x;
                    if (CPLX) ni[j] -= 2.f * sv * wv.y;
                    const float cr = C.x * Cv.x - C.y * Cv.y + Sh.x * Sv.x - Sh.y * Sv.y;
                    const float ci = C.x * Cv.y + C.y * Cv.x + Sh.x * Sv.y + Sh.y * Sv.x;
                    const float sr = Sh.x * Cv.x - Sh.y * Cv.y + C.x * Sv.x - C.y * Sv.y;
                    const float si = Sh.x * Cv.y + Sh.y * Cv.x + C.x * Sv.y + C.y * Sv.x;
                    C = make_float2(cr, ci);
                    Sh = make_float2(sr, si);
                }
                const float fr = C.x - (tr[j] * Sh.x - ti[j] * Sh.y);
                const float fi = CPLX ? C.y - (tr[j] * Sh.y + ti[j] * Sh.x) : 0.f;
                lg += 0.5f * __logf(fr * fr + fi * fi);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lg += __shfl_xor_sync(0xffffffffu, lg, o);
        lg -= 2.f * su * a.a32[u].x;
        if (v >= 0) lg -= 2.f * sv * a.a32[v].x;
        return lg;
    };
    bool dirty = true;          // log q of the current configuration not known
    float lq = 0.f;
    int used = 0;
    auto commit = [&](int, int) {
#pragma unroll
        for (int j = 0; j < J; j++) {
            thr[j] = nr[j];
            thi[j] = ni[j];
            if (lane + 32 * j < M) {
                if (CPLX) {
                    const float2 t = ctanh32s(nr[j], ni[j]);
                    tr[j] = t.x;
                    ti[j] = t.y;
                } else {
                    tr[j] = tanhf(nr[j]);
                }
            }
        }
        dirty = true;
    };
    // independent proposal s' ~ q from this chain's next pool entry, accepted
    // with min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s'))); an exhausted pool
    // leaves the state unchanged (a rejected move)
    auto learned = [&](const uint4 &r) -> bool {
        if (!LEARNED || used >= md.per_chain) return false;
        const long e = (long)c * md.per_chain + used;
        used++;
        const uint64_t x2 = md.pbits[e];
        if (x2 == s) return false;
        const float lq2 = md.plq[e], lp2 = md.plpsi[e];
        const float lp = rbm_logabs32<CPLX>(a, s);
        if (dirty) {
            lq = made_logq_warp(md, Wsm, s, h1, h2);
            dirty = false;
        }
        const float la = 2.f * (lp2 - lp) + lq - lq2;
        bool accept = la >= 0.f;
        if (!accept) {
            const float uni = ((float)(r.z >> 8) + 0.5f) * (1.f / 16777216.f);
            accept = __logf(uni) < la;
        }
        if (accept) {
            s = x2;
            lq = lq2;
            rebuild();
        }
        return accept;
    };
    unsigned long long acc = 0, pro = 0, lacc = 0, lpro = 0;
    run_chain32<MOVE, LEARNED>(S, c, s, eval, commit, learned, mix_thr, acc, pro, lacc, lpro);
    if (lane == 0) {
        S.bits[c] = s;
        atomicAdd(&S.counts[0], acc);
        atomicAdd(&S.counts[1], pro);
        if (LEARNED) {
            atomicAdd(&S.counts[2], lpro);
            atomicAdd(&S.counts[3], lacc);
        }
    }
}

// Any other program (symmetry projection, mean field, MLP): full evaluation of
// every proposal, as upstream.
template <int RNG, int MOVE>
__global__ void __launch_bounds__(32 * kSW) k_sample_generic(SampleArgs S, DevAmp A) {
    if (S.move_dev) S.move0 = *S.move_dev;
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.x * kSW + warp;
    if (c >= S.C) return;
    double *scr = sm + warp * 4 * (A.a.M ? A.a.M : 1);
    uint64_t s = S.bits[c];
    double la, ar, nla = 0.0;
    warp_amp_eval(A, s, la, ar, scr);
    auto eval = [&](int u, int v) -> double {
        uint64_t s2 = s ^ (1ull << u);
        if (v >= 0) s2 ^= 1ull << v;
        double g;
        warp_amp_eval(A, s2, nla, g, scr);
        return nla - la;
    };
    auto commit = [&](int, int) { la = nla; };
    unsigned long long acc = 0, pro = 0;
    run_chain<RNG, MOVE>(S, c, s, eval, commit, acc, pro, la);
    if (lane == 0) {
        S.bits[c] = s;
        atomicAdd(&S.counts[0], acc);
        atomicAdd(&S.counts[1], pro);
    }
}

// FP32 chains of the MLP (mixed precision): the warp keeps the layer-1
// pre-activations of its configuration in registers; a local proposal moves
// them by one or two weight columns and runs layer 2 against W2^T in shared
// memory.  With a learned proposal, its slots (chosen by the random word only)
// take the chain's next pool entry x' ~ q and accept with min(1, |psi(x')|^2
// q(s) / (|psi(s)|^2 q(x'))), both log|psi| evaluated from scratch so the ratio
// uses one function of the configuration.
template <int MOVE, int MQ, bool LEARNED>
__global__ void __launch_bounds__(32 * kSW) k_sample_mlp32(SampleArgs S, DevAmp A, DevMade md) {
    if (S.move_dev) S.move0 = *S.move_dev;
    extern __shared__ __align__(16) unsigned char smraw[];
    constexpr int MP = 32 * MQ;
    const DevAnsatz &a = A.a;
    const int M = a.M, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *w2t = (float *)smraw, *h1s = w2t + M * MP + warp * MP;
    {
        const float *g = a.m32 + (long)a.N * M;
        for (int e = threadIdx.x; e < M * MP; e += blockDim.x) w2t[e] = g[e];
    }
    const __nv_bfloat16 *Wsm = nullptr;
    float *mh1 = nullptr, *mh2 = nullptr;
    uint32_t mix_thr = 0;
    if (LEARNED) {
        unsigned char *mb = smraw + sizeof(float) * (size_t)(M * MP + kSW * MP);
        const long PM = made_off(md.N, md.H).total, wbytes = (PM * 2 + 15) / 16 * 16;
        __nv_bfloat16 *W = (__nv_bfloat16 *)mb;
        for (long p = threadIdx.x; p < PM; p += blockDim.x) W[p] = md.w[p];
        Wsm = W;
        mh1 = (float *)(mb + wbytes) + (size_t)warp * 2 * md.H;
        mh2 = mh1 + md.H;
        mix_thr = *md.active ? md.mix_thr : 0u;
    }
    __syncthreads();
    const int c = blockIdx.x * kSW + warp;
    if (c >= S.C) return;
    uint64_t s = S.bits[c];
    float z1[MQ], nz1[MQ], h1[MQ], h2[MQ], la, ar, nla = 0.f;
    auto rebuild = [&]() {
        mlp32_z1<MQ>(a, s, z1);
        mlp32_forward<MQ>(a, w2t, z1, h1s, h1, h2, la, ar);
    };
    rebuild();
    auto eval = [&](int u, int v) -> float {
        mlp32_z1_flip<MQ>(a, s, u, v, z1, nz1);
        float g;
        mlp32_forward<MQ>(a, w2t, nz1, h1s, h1, h2, nla, g);
        return nla - la;
    };
    bool dirty = true;          // log q of the current configuration not known
    float lq = 0.f;
    int used = 0;
    auto commit = [&](int, int) {
#pragma unroll
        for (int q = 0; q < MQ; q++) z1[q] = nz1[q];
        la = nla;
        dirty = true;
    };
    auto learned = [&](const uint4 &r) -> bool {
        if (!LEARNED || used >= md.per_chain) return false;
        const long e = (long)c * md.per_chain + used;
        used++;
        const uint64_t x2 = md.pbits[e];
        if (x2 == s) return false;
        const float lq2 = md.plq[e];
        float zs[MQ], g1[MQ], g2[MQ], lp, lp2, g;
        mlp32_z1<MQ>(a, s, zs);
        mlp32_forward<MQ>(a, w2t, zs, h1s, g1, g2, lp, g);
        mlp32_z1<MQ>(a, x2, zs);
        mlp32_forward<MQ>(a, w2t, zs, h1s, g1, g2, lp2, g);
        if (dirty) {
            lq = made_logq_warp(md, Wsm, s, mh1, mh2);
            dirty = false;
        }
        const float lr = 2.f * (lp2 - lp) + lq - lq2;
        bool accept = lr >= 0.f;
        if (!accept) {
            const float uni = ((float)(r.z >> 8) + 0.5f) * (1.f / 16777216.f);
            accept = __logf(uni) < lr;
        }
        if (accept) {
            s = x2;
            lq = lq2;
            rebuild();
        }
        return accept;
    };
    unsigned long long acc = 0, pro = 0, lacc = 0, lpro = 0;
    run_chain32<MOVE, LEARNED>(S, c, s, eval, commit, learned, mix_thr, acc, pro, lacc, lpro);
    if (lane == 0) {
        S.bits[c] = s;
        atomicAdd(&S.counts[0], acc);
        atomicAdd(&S.counts[1], pro);
        if (LEARNED) {
            atomicAdd(&S.counts[2], lpro);
            atomicAdd(&S.counts[3], lacc);
        }
    }
}

template <int MOVE>
static bool launch_mlp32_chains(const SampleArgs &S, const DevAmp &A, const DevMade &md, size_t made_smem,
                                dim3 grid, dim3 block, cudaStream_t st) {
    const int MQ = (A.a.M + 31) / 32, MP = 32 * MQ;
    const bool learned = md.per_chain > 0;
    const size_t smem = sizeof(float) * ((size_t)A.a.M * MP + (size_t)kSW * MP) + (learned ? made_smem : 0);
#define NQS_MCASE(QQ)                                                                                        \
    case QQ: {                                                                                               \
        static bool attr = false;                                                                            \
        if (!attr) {                                                                                         \
            if (!NQS_CUDA(cudaFuncSetAttribute(k_sample_mlp32<MOVE, QQ, false>,                              \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)) ||  \
                !NQS_CUDA(cudaFuncSetAttribute(k_sample_mlp32<MOVE, QQ, true>,                               \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)))    \
                return false;                                                                                \
            attr = true;                                                                                     \
        }                                                                                                    \
        if (learned) k_sample_mlp32<MOVE, QQ, true><<<grid, block, smem, st>>>(S, A, md);                    \
        else k_sample_mlp32<MOVE, QQ, false><<<grid, block, smem, st>>>(S, A, md);                           \
        break;                                                                                               \
    }
    switch (MQ) {
        NQS_MCASE(1) NQS_MCASE(2) NQS_MCASE(3) NQS_MCASE(4)
        default:
            set_error("MLP width %d unsupported by the FP32 chains", A.a.M);
            return false;
    }
#undef NQS_MCASE
    return NQS_CUDA(cudaGetLastError());
}

// Philox chain start: uniform bits, or a Fisher-Yates shuffle of n_down down
// spins (fixed-magnetisation sector).  One thread per chain.
// Device-side move counter of a replayed sampler launch.
__global__ void k_move_advance(unsigned long long *ctr, unsigned long long total) { *ctr += total; }

__global__ void k_chain_init(int C, int N, uint64_t seed, int n_down, uint64_t *bits) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    if (n_down < 0) {
        uint4 r = philox4x32(make_uint4((uint32_t)c, 0u, 0u, 1u), key);
        uint64_t b = (uint64_t)r.x | ((uint64_t)r.y << 32);
        bits[c] = N == 64 ? b : (b & ((1ull << N) - 1));
        return;
    }
    unsigned char arr[64];
    for (int i = 0; i < N; i++) arr[i] = i < n_down ? 1 : 0;
    for (int i = N - 1; i >= 1; i--) {
        uint4 r = philox4x32(make_uint4((uint32_t)c, (uint32_t)i, 0u, 1u), key);
        int j = (int)(((uint64_t)r.x * (uint64_t)(i + 1)) >> 32);
        unsigned char t = arr[i];
        arr[i] = arr[j];
        arr[j] = t;
    }
    uint64_t b = 0;
    for (int i = 0; i < N; i++)
        if (arr[i]) b |= 1ull << i;
    bits[c] = b;
}

template <int J, bool CX, int MOVE>
static void launch_rbm32(dim3 grid, dim3 block, cudaStream_t st, const SampleArgs &S, const DevAmp &A,
                         const DevMade &md, size_t smem) {
    if (md.per_chain > 0) {
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_sample_rbm32<J, CX, MOVE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024);
            attr = true;
        }
        k_sample_rbm32<J, CX, MOVE, true><<<grid, block, smem, st>>>(S, A, md);
    } else {
        k_sample_rbm32<J, CX, MOVE, false><<<grid, block, 0, st>>>(S, A, md);
    }
}

template <int RNG, int MOVE>
static bool dispatch(const SampleArgs &S, const DevAmp &A, bool f32, const DevMade &md, size_t smem) {
    dim3 grid((S.C + kSW - 1) / kSW), block(32 * kSW);
    cudaStream_t st = ctx().stream;
    const bool fused = A.G == 0 && (A.a.kind == KIND_RBM || A.a.kind == KIND_CRBM);
    if (f32 && RNG == NQS_GPU_RNG_PHILOX && fp32_mlp_capable(A)) {
        NQS_LAUNCH(md.per_chain > 0 ? "sampler_mlp32_learned" : "sampler_mlp32");
        return launch_mlp32_chains<MOVE>(S, A, md, smem, grid, block, st);
    }
    if (f32 && RNG == NQS_GPU_RNG_PHILOX && fp32_capable(A)) {
        const int J = (A.a.M + 31) / 32;
        const bool cx = A.a.kind == KIND_CRBM;
        NQS_LAUNCH(md.per_chain > 0 ? "sampler_fp32_learned" : "sampler_fp32");
#define NQS_FCASE(JJ)                                                             \
    case JJ:                                                                      \
        if (cx) launch_rbm32<JJ, true, MOVE>(grid, block, st, S, A, md, smem);    \
        else launch_rbm32<JJ, false, MOVE>(grid, block, st, S, A, md, smem);      \
        break;
        switch (J) {
            NQS_FCASE(1) NQS_FCASE(2) NQS_FCASE(3) NQS_FCASE(4) NQS_FCASE(5) NQS_FCASE(6) NQS_FCASE(7)
            NQS_FCASE(8)
            default:
                set_error("hidden width %d unsupported", A.a.M);
                return false;
        }
#undef NQS_FCASE
        return NQS_CUDA(cudaGetLastError());
    }
    if (fused && RNG == NQS_GPU_RNG_PHILOX && MOVE == NQS_GPU_MOVE_SINGLE_FLIP && A.a.cs64) {
        const int J = (A.a.M + 31) / 32;
        const bool cx = A.a.kind == KIND_CRBM;
        NQS_LAUNCH("sampler");
#define NQS_PCASE(JJ)                                                             \
    case JJ:                                                                      \
        if (cx) k_sample_rbm_prod<JJ, true><<<grid, block, 0, st>>>(S, A);        \
        else k_sample_rbm_prod<JJ, false><<<grid, block, 0, st>>>(S, A);          \
        break;
        switch (J) {
            NQS_PCASE(1) NQS_PCASE(2) NQS_PCASE(3) NQS_PCASE(4) NQS_PCASE(5) NQS_PCASE(6) NQS_PCASE(7)
            NQS_PCASE(8)
            default:
                set_error("hidden width %d unsupported", A.a.M);
                return false;
        }
#undef NQS_PCASE
        return NQS_CUDA(cudaGetLastError());
    }
    if (fused) {
        int J = (A.a.M + 31) / 32;
        bool cx = A.a.kind == KIND_CRBM;
        NQS_LAUNCH("sampler");
#define NQS_SCASE(JJ)                                                             \
    case JJ:                                                                      \
        if (cx) k_sample_rbm<JJ, true, RNG, MOVE><<<grid, block, 0, st>>>(S, A);  \
        else k_sample_rbm<JJ, false, RNG, MOVE><<<grid, block, 0, st>>>(S, A);    \
        break;
        switch (J) {
            NQS_SCASE(1) NQS_SCASE(2) NQS_SCASE(3) NQS_SCASE(4) NQS_SCASE(5) NQS_SCASE(6) NQS_SCASE(7)
            NQS_SCASE(8)
            default:
                set_error("hidden width %d unsupported", A.a.M);
                return false;
        }
#undef NQS_SCASE
    } else {
        size_t smem = sizeof(double) * 4 * (A.a.M ? A.a.M : 1) * kSW;
        NQS_LAUNCH("sampler_generic");
        k_sample_generic<RNG, MOVE><<<grid, block, smem, st>>>(S, A);
    }
    return NQS_CUDA(cudaGetLastError());
}

// Advance all chains: `skip` proposals, then record `n_out` samples
// (sample k of chain c at row k*C + c), `decor` proposals apart.
bool sampler_run(Sampler *sm, int skip, int n_out, uint64_t *out, unsigned long long *move_dev) {
    DevAmp A;
    if (!build_amp(sm->fn, sm->user, sm->N, &A, nullptr)) return false;
    int per = sm->cfg.num_decorrelate > 0 ? sm->cfg.num_decorrelate : 1;
    int n_spc = n_out > 0 ? (n_out + sm->C - 1) / sm->C : 0;
    SampleArgs S;
    S.C = sm->C;
    S.N = sm->N;
    S.bits = sm->d_bits.p;
    S.rng = sm->d_rng.p;
    S.cla = sm->opts.rng == NQS_GPU_RNG_XORSHIFT_COMPAT ? sm->d_cla.p : nullptr;
    S.seed = sm->cfg.rng_seed;
    S.move0 = sm->move_counter;
    S.move_dev = move_dev;
    S.skip = skip;
    S.decor = per;
    S.total = skip + n_spc * per;
    S.out = out;
    S.n_out = n_out;
    S.bonds = sm->d_bonds.p;
    S.nb = sm->nb;
    S.counts = sm->d_counts.p;
    if (S.total <= 0) return true;
    bool ok;
    const bool f32 = sm->opts.precision == NQS_GPU_PREC_MIXED && sm->opts.fp32_estimator;
    DevMade md{};
    size_t smem = 0;
    if (sm->made && f32 && sm->opts.rng == NQS_GPU_RNG_PHILOX && (fp32_capable(A) || fp32_mlp_capable(A))) {
        if (!made_prepare(sm->made, A, sm->C, S.total, sm->cfg.rng_seed ^ 0x9E3779B97F4A7C15ull, &md)) return false;
        smem = made_chain_smem(sm->made, kSW);
    }
    if (sm->opts.rng == NQS_GPU_RNG_XORSHIFT_COMPAT)
        ok = dispatch<NQS_GPU_RNG_XORSHIFT_COMPAT, NQS_GPU_MOVE_SINGLE_FLIP>(S, A, false, md, 0);
    else if (sm->opts.move == NQS_GPU_MOVE_EXCHANGE)
        ok = dispatch<NQS_GPU_RNG_PHILOX, NQS_GPU_MOVE_EXCHANGE>(S, A, f32, md, smem);
    else
        ok = dispatch<NQS_GPU_RNG_PHILOX, NQS_GPU_MOVE_SINGLE_FLIP>(S, A, f32, md, smem);
    sm->move_counter += (uint64_t)S.total;
    return ok;
}

// Moves per chain of a sampler_produce(sm, n) call.
int sampler_moves(const Sampler *sm, int n) {
    const int per = sm->cfg.num_decorrelate > 0 ? sm->cfg.num_decorrelate : 1;
    return (n + sm->C - 1) / sm->C * per;
}

// sampler_produce for a captured step: the first move index comes from the
// device counter move_dev, which the captured sequence advances; the host
// counter is advanced by sampler_host_advance() once per replay.  No learned
// proposal.
bool sampler_produce_dev(Sampler *sm, int n, uint64_t **d_out, unsigned long long *move_dev) {
    if (!sm->d_samples.ensure((size_t)n)) return false;
    const uint64_t host = sm->move_counter;
    if (!sampler_run(sm, 0, n, sm->d_samples.p, move_dev)) return false;
    sm->move_counter = host;
    k_move_advance<<<1, 1, 0, ctx().stream>>>(move_dev, (unsigned long long)sampler_moves(sm, n));
    // online training of the learned proposal (its counters are on the device,
    // so this is replayable from a graph)
    if (sm->made && !made_train(sm->made, sm->d_samples.p, n, sm->d_counts.p)) return false;
    *d_out = sm->d_samples.p;
    return NQS_CUDA(cudaGetLastError());
}

void sampler_host_advance(Sampler *sm, int n) { sm->move_counter += (uint64_t)sampler_moves(sm, n); }
uint64_t sampler_move_counter(const Sampler *sm) { return sm->move_counter; }
int sampler_chains(const Sampler *sm) { return sm->C; }
const unsigned long long *sampler_counts(const Sampler *sm) { return sm->d_counts.p; }
bool sampler_fp32(const Sampler *sm) {
    return sm->opts.precision == NQS_GPU_PREC_MIXED && sm->opts.fp32_estimator && sm->opts.rng == NQS_GPU_RNG_PHILOX;
}

bool sampler_produce(Sampler *sm, int n, uint64_t **d_out) {
    if (!sm->d_samples.ensure((size_t)n)) return false;
    if (!sampler_run(sm, 0, n, sm->d_samples.p)) return false;
    // online training of the learned proposal on the chains' own samples
    if (sm->made && !made_train(sm->made, sm->d_samples.p, n, sm->d_counts.p)) return false;
    *d_out = sm->d_samples.p;
    return true;
}

static void exchange_bonds(const nqs_gpu_options_t &o, int N, std::vector<int> &b) {
    if (o.lattice_kagome) {
        int Lx = o.lattice_x, Ly = o.lattice_y;
        auto S = [&](int cx, int cy, int sub) { return 3 * (cx * Ly + cy) + sub; };
        for (int cx = 0; cx < Lx; cx++)
            for (int cy = 0; cy < Ly; cy++) {
                int A = S(cx, cy, 0), B = S(cx, cy, 1), Cc = S(cx, cy, 2);
                int Bm = S((cx - 1 + Lx) % Lx, cy, 1), Cm = S(cx, (cy - 1 + Ly) % Ly, 2);
                int e[12] = {A, B, A, Cc, B, Cc, A, Bm, A, Cm, Bm, Cm};
                b.insert(b.end(), e, e + 12);
            }
        return;
    }
    int Lx = o.lattice_x > 0 ? o.lattice_x : N, Ly = o.lattice_x > 0 ? o.lattice_y : 1;
    int pbc = o.lattice_x > 0 ? o.square_pbc : 1;
    for (int x = 0; x < Lx; x++)
        for (int y = 0; y < Ly; y++) {
            int a = x * Ly + y;
            if (x + 1 < Lx) { b.push_back(a); b.push_back((x + 1) * Ly + y); }
            else if (pbc && Lx > 1) { b.push_back(a); b.push_back(y); }
            if (y + 1 < Ly) { b.push_back(a); b.push_back(x * Ly + y + 1); }
            else if (pbc && Ly > 1) { b.push_back(a); b.push_back(x * Ly); }
        }
}

}  // namespace nqs

using namespace nqs;

extern "C" {

nqs_sampler_t *nqs_sampler_create_gpu(int num_sites, const nqs_config_t *cfg,
                                      const nqs_gpu_options_t *opts, nqs_log_amp_fn_t fn,
                                      void *user) {
    clear_error();
    if (num_sites <= 0 || !cfg || !fn || !opts) return nullptr;   // src/nqs/nqs_sampler.c:54
    if (num_sites > kMaxSites) {
        set_error("num_sites %d > %d", num_sites, kMaxSites);
        return nullptr;
    }
    if (!ensure_context()) return nullptr;
    DevAmp A;
    if (!build_amp(fn, user, num_sites, &A, nullptr)) return nullptr;
    Sampler *s = new Sampler();
    s->N = num_sites;
    s->cfg = *cfg;
    s->opts = *opts;
    s->fn = fn;
    s->user = user;
    bool compat = opts->rng == NQS_GPU_RNG_XORSHIFT_COMPAT;
    s->C = compat ? 1 : (opts->num_chains > 0 ? opts->num_chains : 1);
    if (!compat && opts->move == NQS_GPU_MOVE_EXCHANGE) {
        std::vector<int> b;
        exchange_bonds(*opts, num_sites, b);
        for (int x : b)
            if (x < 0 || x >= num_sites) {
                set_error("exchange lattice does not match num_sites %d", num_sites);
                delete s;
                return nullptr;
            }
        s->nb = (int)b.size() / 2;
        if (s->nb == 0 || !s->d_bonds.ensure(b.size()) ||
            !NQS_CUDA(cudaMemcpy(s->d_bonds.p, b.data(), sizeof(int) * b.size(), cudaMemcpyHostToDevice))) {
            if (s->nb == 0) set_error("exchange moves need at least one bond");
            delete s;
            return nullptr;
        }
    }
    if (!s->d_bits.ensure((size_t)s->C) || !s->d_rng.ensure((size_t)s->C) || !s->d_counts.ensure(4) ||
        !NQS_CUDA(cudaMallocHost(&s->h_current, sizeof(int) * num_sites))) {
        delete s;
        return nullptr;
    }
    cudaStream_t st = ctx().stream;
    NQS_CUDA(cudaMemsetAsync(s->d_counts.p, 0, 4 * sizeof(unsigned long long), st));
    if (compat) {
        // upstream start: rng = seed (or a fixed constant), then one draw per site
        // (src/nqs/nqs_sampler.c:62-72); host-side set-up of the single chain
        uint64_t rng = cfg->rng_seed ? (uint64_t)cfg->rng_seed : 0x9E3779B97F4A7C15ull;
        uint64_t bits = 0;
        for (int i = 0; i < num_sites; i++) {
            uint64_t x = rng;
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            rng = x;
            if (!(x & 1)) bits |= 1ull << i;     // odd draw -> +1, even -> -1 (bit set)
        }
        uint64_t h[2] = {bits, rng};
        NQS_CUDA(cudaMemcpyAsync(s->d_bits.p, &h[0], 8, cudaMemcpyHostToDevice, st));
        NQS_CUDA(cudaMemcpyAsync(s->d_rng.p, &h[1], 8, cudaMemcpyHostToDevice, st));
        // the cache starts empty (NaN): the first launch stores log|psi| of the start
        // configuration at the parameters it sees, as upstream does at creation
        if (!s->d_cla.ensure(1) || !NQS_CUDA(cudaMemsetAsync(s->d_cla.p, 0xff, sizeof(double), st))) {
            delete s;
            return nullptr;
        }
    } else {
        NQS_LAUNCH("chain_init");
        k_chain_init<<<(s->C + 127) / 128, 128, 0, st>>>(s->C, num_sites, cfg->rng_seed,
                                                          opts->n_down, s->d_bits.p);
    }
    if (!NQS_CUDA(cudaStreamSynchronize(st))) {
        delete s;
        return nullptr;
    }
    return (nqs_sampler_t *)s;
}

nqs_sampler_t *nqs_sampler_create(int num_sites, const nqs_config_t *cfg, nqs_log_amp_fn_t fn,
                                  void *user) {
    if (!ensure_context()) return nullptr;
    nqs_gpu_options_t o = ctx().opts;
    return nqs_sampler_create_gpu(num_sites, cfg, &o, fn, user);
}

void nqs_sampler_free(nqs_sampler_t *h) {
    Sampler *s = (Sampler *)h;
    if (!s) return;
    if (s->h_current) cudaFreeHost(s->h_current);
    if (s->made) made_free(s->made);
    delete s;
}

void nqs_sampler_thermalize(nqs_sampler_t *h) {
    Sampler *s = (Sampler *)h;
    if (!s) return;
    if (!sampler_run(s, s->cfg.num_thermalize, 0, nullptr)) return;
    NQS_CUDA(cudaStreamSynchronize(ctx().stream));
}

static const int *fetch_chain0(Sampler *s) {
    if (!s->d_spins.ensure((size_t)s->N)) return nullptr;
    if (!launch_bits_to_spins(s->d_bits.p, 1, s->N, s->d_spins.p)) return nullptr;
    if (!NQS_CUDA(cudaMemcpyAsync(s->h_current, s->d_spins.p, sizeof(int) * s->N, cudaMemcpyDeviceToHost,
                                  ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return nullptr;
    return s->h_current;
}

const int *nqs_sampler_next(nqs_sampler_t *h) {
    Sampler *s = (Sampler *)h;
    if (!s) return nullptr;
    int per = s->cfg.num_decorrelate > 0 ? s->cfg.num_decorrelate : 1;
    if (!sampler_run(s, per, 0, nullptr)) return nullptr;
    return fetch_chain0(s);
}

int nqs_sampler_batch(nqs_sampler_t *h, int n, int *out) {
    Sampler *s = (Sampler *)h;
    if (!s || !out || n <= 0) return -1;                 // src/nqs/nqs_sampler.c:136
    uint64_t *d;
    if (!sampler_produce(s, n, &d)) return -1;
    if (!s->d_spins.ensure((size_t)n * s->N)) return -1;
    if (!launch_bits_to_spins(d, n, s->N, s->d_spins.p)) return -1;
    if (!NQS_CUDA(cudaMemcpyAsync(out, s->d_spins.p, sizeof(int) * (size_t)n * s->N,
                                  cudaMemcpyDeviceToHost, ctx().stream)))
        return -1;
    return NQS_CUDA(cudaStreamSynchronize(ctx().stream)) ? 0 : -1;
}

double nqs_sampler_acceptance_ratio(const nqs_sampler_t *h) {
    const Sampler *s = (const Sampler *)h;
    if (!s) return 0.0;
    unsigned long long c[2] = {0, 0};
    if (!NQS_CUDA(cudaMemcpyAsync(c, s->d_counts.p, sizeof(c), cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return 0.0;
    return c[1] ? (double)c[0] / (double)c[1] : 0.0;
}

const int *nqs_sampler_current(const nqs_sampler_t *h) {
    return h ? fetch_chain0((Sampler *)h) : nullptr;
}

int nqs_sampler_num_sites(const nqs_sampler_t *h) { return h ? ((const Sampler *)h)->N : 0; }

int nqs_sampler_num_chains(const nqs_sampler_t *h) { return h ? ((const Sampler *)h)->C : 0; }

// ---------------------------------------------------------------- learned proposal
nqs_gpu_made_options_t nqs_gpu_made_options_default(void) {
    nqs_gpu_made_options_t o;
    memset(&o, 0, sizeof(o));
    o.hidden = 64;
    o.train_iters = 1;
    o.train_batch = 1024;
    o.mix = 0.5;
    o.learning_rate = 3e-3;
    o.min_acceptance = 0.01;
    o.seed = 20260214ull;
    return o;
}

int nqs_sampler_set_learned_proposal(nqs_sampler_t *h, const nqs_gpu_made_options_t *o) {
    clear_error();
    Sampler *s = (Sampler *)h;
    if (!s) return -1;
    if (s->made) {
        made_free(s->made);
        s->made = nullptr;
    }
    if (!o) return 0;
    if (s->opts.rng != NQS_GPU_RNG_PHILOX || s->opts.precision != NQS_GPU_PREC_MIXED || !s->opts.fp32_estimator) {
        set_error("learned proposal needs Philox chains and the MIXED precision mode with fp32_estimator = 1");
        return -1;
    }
    DevAmp A;
    if (!build_amp(s->fn, s->user, s->N, &A, nullptr)) return -1;
    if (!fp32_capable(A) && !fp32_mlp_capable(A)) {
        set_error("learned proposal needs an RBM / cRBM or MLP program without symmetry projection");
        return -1;
    }
    const int n_ones = s->opts.move == NQS_GPU_MOVE_EXCHANGE && s->opts.n_down >= 0 ? s->opts.n_down : -1;
    s->made = made_create(s->N, n_ones, *o);
    return s->made ? 0 : -1;
}

int nqs_sampler_learned_stats(const nqs_sampler_t *h, nqs_gpu_made_stats_t *out) {
    const Sampler *s = (const Sampler *)h;
    if (!s || !out || !s->made) return -1;
    return made_stats_read(s->made, out) ? 0 : -1;
}

long nqs_gpu_made_num_params(const nqs_sampler_t *h) {
    const Sampler *s = (const Sampler *)h;
    return s && s->made ? made_num_params(s->made) : 0;
}

int nqs_gpu_made_get_weights(const nqs_sampler_t *h, float *out) {
    const Sampler *s = (const Sampler *)h;
    if (!s || !s->made || !out) return -1;
    return made_get(s->made, out) ? 0 : -1;
}

int nqs_gpu_made_set_weights(nqs_sampler_t *h, const float *in) {
    Sampler *s = (Sampler *)h;
    if (!s || !s->made || !in) return -1;
    return made_set(s->made, in) ? 0 : -1;
}

int nqs_gpu_made_log_prob(const nqs_sampler_t *h, const int *spins, int batch, double *out) {
    clear_error();
    const Sampler *s = (const Sampler *)h;
    if (!s || !s->made || !spins || !out || batch <= 0) return -1;
    uint64_t *bits;
    static DevBuf<float> lq;
    if (!upload_spins(spins, batch, s->N, &bits) || !lq.ensure((size_t)batch) || !made_logq(s->made, bits, batch, lq.p))
        return -1;
    std::vector<float> h_((size_t)batch);
    if (!NQS_CUDA(cudaMemcpyAsync(h_.data(), lq.p, sizeof(float) * batch, cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return -1;
    for (int b = 0; b < batch; b++) out[b] = h_[b];
    return 0;
}

int nqs_gpu_made_nll_grad(nqs_sampler_t *h, const int *spins, int batch, float *out_grad, double *out_nll) {
    clear_error();
    Sampler *s = (Sampler *)h;
    if (!s || !s->made || !spins || !out_grad || batch <= 0) return -1;
    uint64_t *bits;
    if (!upload_spins(spins, batch, s->N, &bits)) return -1;
    return made_grad(s->made, bits, batch, out_grad, out_nll) ? 0 : -1;
}

int nqs_gpu_made_sample(nqs_sampler_t *h, int count, int *out_spins, double *out_logq) {
    clear_error();
    Sampler *s = (Sampler *)h;
    if (!s || !s->made || !out_spins || count <= 0) return -1;
    DevAmp A;
    if (!build_amp(s->fn, s->user, s->N, &A, nullptr)) return -1;
    const uint64_t *bits;
    const float *lq;
    if (!made_sample(s->made, A, count, s->cfg.rng_seed ^ 0x5EEDull, &bits, &lq)) return -1;
    if (!s->d_spins.ensure((size_t)count * s->N) || !launch_bits_to_spins(bits, count, s->N, s->d_spins.p)) return -1;
    std::vector<float> h_((size_t)count);
    if (!NQS_CUDA(cudaMemcpyAsync(out_spins, s->d_spins.p, sizeof(int) * (size_t)count * s->N, cudaMemcpyDeviceToHost,
                                  ctx().stream)) ||
        !NQS_CUDA(cudaMemcpyAsync(h_.data(), lq, sizeof(float) * count, cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return -1;
    if (out_logq)
        for (int b = 0; b < count; b++) out_logq[b] = h_[b];
    return 0;
}

}  // extern "C"
