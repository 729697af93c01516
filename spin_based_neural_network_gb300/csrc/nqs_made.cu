// Learned proposal (MADE) kernels and optimiser state; the model is described
// in nqs_made.cuh.
//
//   pool      every learned proposal of a sampler launch is drawn up front,
//             one warp per proposal (the autoregressive draw is sequential over
//             the sites but independent across proposals): bits, log q and the
//             FP32 log|psi| of the RBM, consumed by the chains in order;
//   grad      mean NLL gradient of the batch the chains produced, one warp per
//             slice of samples accumulating into its own shared-memory copy of
//             the gradient (no atomics: deterministic), BF16 weights read from
//             shared memory with transposed copies of W2 / W3 for the backward
//             pass;
//   adam      per-parameter reduction over the warp partials, masks, Adam on
//             the FP32 masters and the BF16 copy the next launch samples from;
//   stats     mean NLL, learned-proposal acceptance of the last batch, and the
//             fallback: below `min_acceptance` the next batches use local moves
//             only, with a probe every 8 batches.
#include <math.h>
#include <string.h>

#include <vector>

#include "nqs_amp.cuh"
#include "nqs_made.cuh"

namespace nqs {

struct Made {
    int N = 0, H = 0, n_ones = -1;
    long PM = 0;
    nqs_gpu_made_options_t opt{};
    DevBuf<float> master, m1, v1, partials, nllp, plq, plpsi;
    DevBuf<__nv_bfloat16> wb;
    DevBuf<uint64_t> pbits;
    DevBuf<int> active;
    DevBuf<double> stats;            // [0] mean NLL of the last batch [1] proposals [2] accepted
                                     // [3] probe countdown [4] prev proposals [5] prev accepted
    // device counters ([0] pool draws, [1] Adam steps), so that a sampler
    // launch replayed from a CUDA graph still draws a fresh pool and applies the
    // right bias corrections
    DevBuf<unsigned> ctr;
};

__global__ void k_made_count(unsigned *c) { *c += 1u; }

static inline uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_made_publish(const float *master, __nv_bfloat16 *wb, long PM, int N, int H) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < PM) wb[p] = __float2bfloat16(made_kept(p, N, H) ? master[p] : 0.f);
}

// ---------------------------------------------------------------- proposal pool
// One thread per proposal: the hidden-1 pre-activations live in registers
// (H is a template parameter), the weights in shared memory are read as
// broadcasts (every thread of a warp reads the same entry), and the running
// logits of the outputs sit in a shared-memory column per thread.  At site i
// the hidden-2 units of degree i (all of x_<i drawn) are formed and added to
// the logits of the outputs >= i in the order made_logq_warp uses, so the
// pool's log q equals the teacher-forced log q of the same configuration.
// made_h2 of one thread: W2n = W2 with unit-major rows (W2n[k][j] = W2t[j][k]),
// read 8 weights per 16-byte load; same products and partial sums as made_h2.
__device__ __forceinline__ void bf8(const __nv_bfloat16 *p, float (&w)[8]) {
    const uint4 v = *(const uint4 *)p;
    const uint32_t u[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        w[2 * q] = __uint_as_float(u[q] << 16);
        w[2 * q + 1] = __uint_as_float(u[q] & 0xFFFF0000u);
    }
}

template <int H>
__device__ __forceinline__ float made_h2_reg(const __nv_bfloat16 *W, const __nv_bfloat16 *W2n, const MadeOff &o,
                                             int k, const float (&a1)[H]) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
    for (int j = 0; j < H; j += 8) {
        float w[8];
        bf8(W2n + (long)k * H + j, w);
        s0 = fmaf(w[0], fmaxf(a1[j], 0.f), s0);
        s1 = fmaf(w[1], fmaxf(a1[j + 1], 0.f), s1);
        s2 = fmaf(w[2], fmaxf(a1[j + 2], 0.f), s2);
        s3 = fmaf(w[3], fmaxf(a1[j + 3], 0.f), s3);
        s0 = fmaf(w[4], fmaxf(a1[j + 4], 0.f), s0);
        s1 = fmaf(w[5], fmaxf(a1[j + 5], 0.f), s1);
        s2 = fmaf(w[6], fmaxf(a1[j + 6], 0.f), s2);
        s3 = fmaf(w[7], fmaxf(a1[j + 7], 0.f), s3);
    }
    return fmaxf(bf(W, o.b2 + k) + ((s0 + s1) + (s2 + s3)), 0.f);
}

constexpr int POOL_T = 128;

template <int H, bool CPLX>
__global__ void __launch_bounds__(POOL_T, 3) k_made_pool(DevMade m, DevAmp A, long total, uint64_t seed,
                                                      const unsigned *__restrict__ launch_ctr,
                                                      uint64_t *pbits, float *plq, float *plpsi) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (*m.active == 0) return;
    const uint32_t launch = *launch_ctr;
    const int N = m.N, tid = threadIdx.x;
    const MadeOff o = made_off(N, H);
    __nv_bfloat16 *W = (__nv_bfloat16 *)smraw;
    const long wbytes = (o.total * 2 + 15) / 16 * 16;
    __nv_bfloat16 *W2n = (__nv_bfloat16 *)(smraw + wbytes);                      // [H][H]
    float *Ls = (float *)(smraw + wbytes + (long)H * H * 2);                     // [N][POOL_T]
    float *Ps = Ls + (long)N * POOL_T;                                           // [32][POOL_T]
    for (long p = tid; p < o.total; p += POOL_T) W[p] = m.w[p];
    for (long p = tid; p < (long)H * H; p += POOL_T) W2n[(p % H) * H + p / H] = m.w[o.w2 + p];
    __syncthreads();
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    for (long e = (long)blockIdx.x * POOL_T + tid; e < total; e += (long)gridDim.x * POOL_T) {
        float a1[H];
#pragma unroll
        for (int k = 0; k < H; k++) a1[k] = bf(W, o.b1 + k);
        for (int i = 0; i < N; i++) Ls[i * POOL_T + tid] = 0.f;
        uint64_t x = 0;
        int ones = 0;
        float lq = 0.f;
        uint4 r = make_uint4(0, 0, 0, 0);
        for (int i = 0; i < N; i++) {
            if ((i & 3) == 0)
                r = philox4x32(make_uint4((uint32_t)e, (uint32_t)(e >> 32) ^ (launch << 8), (uint32_t)(i >> 2), 2u),
                               key);
            if (i >= 1) {
                const int k1 = made_first(i + 1, N, H);
                for (int k = made_first(i, N, H); k < k1; k++) {
                    const float h2 = made_h2_reg<H>(W, W2n, o, k, a1);
                    for (int io = i; io < N; io++)
                        Ls[io * POOL_T + tid] = fmaf(bf(W, o.w3 + (long)k * N + io), h2, Ls[io * POOL_T + tid]);
                }
            }
            const float l = Ls[i * POOL_T + tid] + bf(W, o.b3 + i);
            const int f = made_forced(i, ones, N, m.n_ones);
            int xi;
            if (f >= 0) {
                xi = f;
            } else {
                const uint32_t wd = (i & 3) == 0 ? r.x : (i & 3) == 1 ? r.y : (i & 3) == 2 ? r.z : r.w;
                const float u = ((float)(wd >> 8) + 0.5f) * (1.f / 16777216.f);
                xi = u < 1.f / (1.f + expf(-l)) ? 1 : 0;
                lq += xi ? log_sigmoid(l) : log_sigmoid(-l);
            }
            if (xi) {
                x |= 1ull << i;
                ones++;
#pragma unroll
                for (int k = 0; k < H; k += 8) {                  // masked entries are 0
                    float w[8];
                    bf8(W + o.w1 + (long)i * H + k, w);
#pragma unroll
                    for (int q = 0; q < 8; q++) a1[k + q] += w[q];
                }
            }
        }
        // log|psi(x)| of the RBM in FP32: the 32 lane partials of rbm_logabs32
        // combined in its XOR-butterfly order, so the chains' warp evaluation of
        // the same configuration gives the same number
        const DevAnsatz &a = A.a;
        if (a.kind != KIND_RBM && a.kind != KIND_CRBM) {    // MLP: the chain evaluates log|psi| itself
            pbits[e] = x;
            plq[e] = lq;
            plpsi[e] = 0.f;
            continue;
        }
        for (int l = 0; l < 32; l++) {
            float acc = 0.f;
            for (int h = l; h < a.M; h += 32) {
                float xr = a.b32[h].x, xim = a.b32[h].y;
                for (int i = 0; i < a.N; i++) {
                    const float sp = (x >> i) & 1ull ? -1.f : 1.f;
                    const float2 w = a.w32[(long)i * a.M + h];
                    xr = fmaf(sp, w.x, xr);
                    if (CPLX) xim = fmaf(sp, w.y, xim);
                }
                const float ax = fabsf(xr), ee = expf(-2.f * ax);
                acc += CPLX ? ax + 0.5f * log1pf(ee * (2.f * cosf(2.f * xim) + ee)) : ax + log1pf(ee);
            }
            for (int i = l; i < a.N; i += 32) acc += ((x >> i) & 1ull ? -1.f : 1.f) * a.a32[i].x;
            Ps[l * POOL_T + tid] = acc;
        }
        for (int off = 16; off > 0; off >>= 1)
            for (int l = 0; l < off; l++)
                Ps[l * POOL_T + tid] = Ps[l * POOL_T + tid] + Ps[(l + off) * POOL_T + tid];
        const float lp = Ps[tid];
        pbits[e] = x;
        plq[e] = lq;
        plpsi[e] = lp;
    }
}

// ---------------------------------------------------------------- training
__host__ __device__ inline long made_grad_floats(int N, int H) { return made_off(N, H).total + 5L * H + 64; }

__host__ __device__ inline long made_grad_smem(int N, int H, int warps) {
    const MadeOff o = made_off(N, H);
    const long wb = (o.total * 2 + 15) / 16 * 16, tb = ((long)H * H * 2 + (long)N * H * 2 + 15) / 16 * 16;
    return wb + tb + (long)warps * made_grad_floats(N, H) * 4;
}

__global__ void k_made_grad(DevMade m, const uint64_t *__restrict__ bits, int B, int per_warp, float *partials,
                            float *nllp) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int N = m.N, H = m.H, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const MadeOff o = made_off(N, H);
    const long PM = o.total;
    __nv_bfloat16 *W = (__nv_bfloat16 *)smraw;
    const long wbytes = (PM * 2 + 15) / 16 * 16;
    __nv_bfloat16 *W2n = (__nv_bfloat16 *)(smraw + wbytes);       // W2[k][j]
    __nv_bfloat16 *W3n = W2n + (long)H * H;                         // W3[i][k]
    const long tbytes = ((long)H * H * 2 + (long)N * H * 2 + 15) / 16 * 16;
    float *g = (float *)(smraw + wbytes + tbytes) + (size_t)warp * made_grad_floats(N, H);
    float *a1 = g + PM, *h1 = a1 + H, *a2 = h1 + H, *h2 = a2 + H, *da2 = h2 + H, *dl = da2 + H;
    for (long p = threadIdx.x; p < PM; p += blockDim.x) W[p] = m.w[p];
    __syncthreads();
    for (long p = threadIdx.x; p < (long)H * H; p += blockDim.x) W2n[(p % H) * H + p / H] = W[o.w2 + p];
    for (long p = threadIdx.x; p < (long)H * N; p += blockDim.x) W3n[(p % N) * H + p / N] = W[o.w3 + p];
    for (long p = lane; p < PM; p += 32) g[p] = 0.f;
    __syncthreads();
    const int gw = blockIdx.x * nwb + warp;
    float nll = 0.f;
    const int s0 = gw * per_warp, s1 = min(B, s0 + per_warp);
    for (int s = s0; s < s1; s++) {
        const uint64_t x = bits[s];
        for (int k = lane; k < H; k += 32) {
            float a = bf(W, o.b1 + k);
            for (int i = 0; i < N; i++)
                if ((x >> i) & 1ull) a += bf(W, o.w1 + (long)i * H + k);
            a1[k] = a;
            h1[k] = fmaxf(a, 0.f);
        }
        __syncwarp();
        for (int k = lane; k < H; k += 32) h2[k] = made_h2(W, o, H, k, h1, &a2[k]);
        __syncwarp();
        // outputs: dl_i = d NLL / d logit_i = sigmoid(l_i) - x_i on the free sites
        for (int i = lane; i < N; i += 32) {
            float l = bf(W, o.b3 + i);
            for (int k = 0; k < H; k++) l = fmaf(bf(W, o.w3 + (long)k * N + i), h2[k], l);
            const int f = made_forced(i, __popcll(x & ((1ull << i) - 1ull)), N, m.n_ones);
            float d = 0.f;
            if (f < 0) {
                const int xi = (int)((x >> i) & 1ull);
                nll -= xi ? log_sigmoid(l) : log_sigmoid(-l);
                d = 1.f / (1.f + expf(-l)) - (float)xi;
            }
            dl[i] = d;
            g[o.b3 + i] += d;
            for (int k = 0; k < H; k++) g[o.w3 + (long)k * N + i] += d * h2[k];
        }
        __syncwarp();
        for (int k = lane; k < H; k += 32) {
            float dh = 0.f;
            for (int i = 0; i < N; i++) dh = fmaf(__bfloat162float(W3n[(long)i * H + k]), dl[i], dh);
            const float d2 = a2[k] > 0.f ? dh : 0.f;
            da2[k] = d2;
            g[o.b2 + k] += d2;
            for (int j = 0; j < H; j++) g[o.w2 + (long)j * H + k] += h1[j] * d2;
        }
        __syncwarp();
        for (int j = lane; j < H; j += 32) {
            float dh = 0.f;
            for (int k = 0; k < H; k++) dh = fmaf(__bfloat162float(W2n[(long)k * H + j]), da2[k], dh);
            const float d1 = a1[j] > 0.f ? dh : 0.f;
            g[o.b1 + j] += d1;
            for (int i = 0; i < N; i++)
                if ((x >> i) & 1ull) g[o.w1 + (long)i * H + j] += d1;
        }
        __syncwarp();
    }
    nll = warp_sumf(nll);
    float *dst = partials + (size_t)gw * PM;
    for (long p = lane; p < PM; p += 32) dst[p] = g[p];
    if (lane == 0) nllp[gw] = nll;
}

// Sum of the warp partials (fixed order) / B, masked; with lr > 0 an Adam step
// on the masters and a new BF16 copy, else the gradient itself into `out`.
__global__ void k_made_adam(float *w, float *m1, float *v1, const float *__restrict__ partials, int nw, long PM,
                            int N, int H, float inv_b, float lr, const unsigned *__restrict__ t_ctr,
                            __nv_bfloat16 *wb, float *out) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= PM) return;
    const float tt = (float)(*t_ctr + 1u);                   // this Adam step
    const float bc1 = 1.f - powf(0.9f, tt), bc2 = 1.f - powf(0.999f, tt);
    float g = 0.f;
    for (int q = 0; q < nw; q++) g += partials[(size_t)q * PM + p];
    g = made_kept(p, N, H) ? g * inv_b : 0.f;
    if (out) {
        out[p] = g;
        return;
    }
    if (!made_kept(p, N, H)) {
        wb[p] = __float2bfloat16(0.f);
        return;
    }
    const float mm = 0.9f * m1[p] + 0.1f * g, vv = 0.999f * v1[p] + 0.001f * g * g;
    m1[p] = mm;
    v1[p] = vv;
    const float nwv = w[p] - lr * (mm / bc1) / (sqrtf(vv / bc2) + 1e-8f);
    w[p] = nwv;
    wb[p] = __float2bfloat16(nwv);
}

// Mean NLL and the fallback decision from the sampler's counters (2: learned
// proposals, 3: accepted).
__global__ void k_made_stats(const float *nllp, int nw, int B, double *stats, const unsigned long long *counts,
                             int *active, double min_acc) {
    double s = 0.0;
    for (int q = threadIdx.x; q < nw; q += 32) s += (double)nllp[q];
    s = warp_sum(s);
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (nw > 0) stats[0] = s / (double)B;
    const double p = (double)counts[2], a = (double)counts[3];
    const double dp = p - stats[4], da = a - stats[5];
    stats[1] = p;
    stats[2] = a;
    stats[4] = p;
    stats[5] = a;
    if (*active) {
        if (dp > 0.0 && da / dp < min_acc) {
            *active = 0;
            stats[3] = 8.0;
        }
    } else {
        stats[3] -= 1.0;
        if (stats[3] <= 0.0) *active = 1;                      // probe again
    }
}

// ---------------------------------------------------------------- host side
Made *made_create(int N, int n_ones, const nqs_gpu_made_options_t &opt) {
    if (N < 2 || N > 64 || opt.hidden < 32 || opt.hidden > MADE_MAX_H || opt.hidden % 32 != 0) {
        set_error("learned proposal: need 2 <= N <= 64 and hidden a multiple of 32 up to %d", MADE_MAX_H);
        return nullptr;
    }
    if (!(opt.mix >= 0.0 && opt.mix <= 1.0) || opt.train_iters < 0 || !(opt.learning_rate >= 0.0)) {
        set_error("learned proposal: invalid mix / train_iters / learning_rate");
        return nullptr;
    }
    const int H = opt.hidden;
    if (made_grad_smem(N, H, 1) > 200 * 1024) {
        set_error("learned proposal: N = %d, hidden = %d exceeds the shared-memory budget", N, H);
        return nullptr;
    }
    Made *m = new Made();
    m->N = N;
    m->H = H;
    m->n_ones = n_ones;
    m->opt = opt;
    const MadeOff o = made_off(N, H);
    m->PM = o.total;
    std::vector<float> w((size_t)o.total, 0.f);
    uint64_t st = opt.seed ^ 0x4D414445ull;
    auto uni = [&](float a) { return (float)(((double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0) * a; };
    // Glorot-uniform on the kept entries, zero biases
    const float a1 = sqrtf(6.f / (float)(N + H)), a2 = sqrtf(6.f / (float)(2 * H)), a3 = sqrtf(6.f / (float)(H + N));
    for (long p = 0; p < o.total; p++) {
        if (!made_kept(p, N, H)) continue;
        if (p < o.b1) w[p] = uni(a1);
        else if (p >= o.w2 && p < o.b2) w[p] = uni(a2);
        else if (p >= o.w3 && p < o.b3) w[p] = uni(a3);
    }
    cudaStream_t s = ctx().stream;
    double zs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int one = 1;
    if (!m->master.ensure(o.total) || !m->m1.ensure(o.total) || !m->v1.ensure(o.total) || !m->wb.ensure(o.total) ||
        !m->active.ensure(1) || !m->stats.ensure(8) || !m->ctr.ensure(2) ||
        !NQS_CUDA(cudaMemsetAsync(m->ctr.p, 0, 2 * sizeof(unsigned), s)) ||
        !NQS_CUDA(cudaMemcpyAsync(m->master.p, w.data(), sizeof(float) * o.total, cudaMemcpyHostToDevice, s)) ||
        !NQS_CUDA(cudaMemsetAsync(m->m1.p, 0, sizeof(float) * o.total, s)) ||
        !NQS_CUDA(cudaMemsetAsync(m->v1.p, 0, sizeof(float) * o.total, s)) ||
        !NQS_CUDA(cudaMemcpyAsync(m->active.p, &one, sizeof(int), cudaMemcpyHostToDevice, s)) ||
        !NQS_CUDA(cudaMemcpyAsync(m->stats.p, zs, sizeof(zs), cudaMemcpyHostToDevice, s))) {
        delete m;
        return nullptr;
    }
    k_made_publish<<<(unsigned)((o.total + 255) / 256), 256, 0, s>>>(m->master.p, m->wb.p, o.total, N, H);
    if (!NQS_CUDA(cudaGetLastError()) || !NQS_CUDA(cudaStreamSynchronize(s))) {
        delete m;
        return nullptr;
    }
    return m;
}

void made_free(Made *m) { delete m; }

long made_num_params(const Made *m) { return m->PM; }

DevMade made_view(const Made *m) {
    DevMade d{};
    d.N = m->N;
    d.H = m->H;
    d.n_ones = m->n_ones;
    d.w = m->wb.p;
    d.active = m->active.p;
    d.per_chain = 0;
    d.mix_thr = 0;
    return d;
}

size_t made_chain_smem(const Made *m, int warps) {
    const long wbytes = (m->PM * 2 + 15) / 16 * 16;
    return (size_t)(wbytes + (long)warps * 2 * m->H * 4);
}

static size_t pool_smem(const Made *m) {
    const long wbytes = (m->PM * 2 + 15) / 16 * 16;
    return (size_t)(wbytes + (long)m->H * m->H * 2 + (long)(m->N + 32) * POOL_T * 4);
}

template <int H>
static void pool_kernel(const Made *m, unsigned grid, size_t smem, const DevMade &d, const DevAmp &A, long count,
                        uint64_t seed, float *plq, float *plpsi, uint64_t *pbits) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_made_pool<H, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_made_pool<H, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    if (A.a.kind == KIND_CRBM)
        k_made_pool<H, true><<<grid, POOL_T, smem, ctx().stream>>>(d, A, count, seed, m->ctr.p, pbits, plq, plpsi);
    else
        k_made_pool<H, false><<<grid, POOL_T, smem, ctx().stream>>>(d, A, count, seed, m->ctr.p, pbits, plq, plpsi);
    k_made_count<<<1, 1, 0, ctx().stream>>>(m->ctr.p);
}

// Draw `count` proposals into the pool (count = chains x per_chain).
static bool pool_launch(Made *m, const DevAmp &A, long count, uint64_t seed, DevMade &d) {
    if (!m->pbits.ensure((size_t)count) || !m->plq.ensure((size_t)count) || !m->plpsi.ensure((size_t)count))
        return false;
    d.pbits = m->pbits.p;
    d.plq = m->plq.p;
    d.plpsi = m->plpsi.p;
    const size_t smem = pool_smem(m);
    const long blocks = (count + POOL_T - 1) / POOL_T;
    const unsigned grid = (unsigned)(blocks < (long)ctx().sm_count * 8 ? blocks : (long)ctx().sm_count * 8);
    NQS_LAUNCH("made_pool");
    switch (m->H) {
        case 32: pool_kernel<32>(m, grid, smem, d, A, count, seed, m->plq.p, m->plpsi.p, m->pbits.p); break;
        case 64: pool_kernel<64>(m, grid, smem, d, A, count, seed, m->plq.p, m->plpsi.p, m->pbits.p); break;
        case 96: pool_kernel<96>(m, grid, smem, d, A, count, seed, m->plq.p, m->plpsi.p, m->pbits.p); break;
        default: pool_kernel<128>(m, grid, smem, d, A, count, seed, m->plq.p, m->plpsi.p, m->pbits.p); break;
    }
    return NQS_CUDA(cudaGetLastError());
}

bool made_prepare(Made *m, const DevAmp &A, int C, int total_moves, uint64_t seed, DevMade *out) {
    DevMade d = made_view(m);
    const double mix = m->opt.mix;
    if (mix <= 0.0 || total_moves <= 0) {
        *out = d;
        return true;
    }
    // learned slots per chain ~ Binomial(total_moves, mix): the pool holds the
    // mean + 4 standard deviations + 2 (a chain that runs out rejects)
    const double mean = (double)total_moves * mix, sd = sqrt(mean * (1.0 - mix));
    const int per = (int)ceil(mean + 4.0 * sd) + 2;
    if (!pool_launch(m, A, (long)C * per, seed, d)) return false;
    d.per_chain = per;
    d.mix_thr = mix >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(mix * 4294967296.0);
    *out = d;
    return true;
}

bool made_sample(Made *m, const DevAmp &A, long count, uint64_t seed, const uint64_t **bits, const float **lq) {
    DevMade d = made_view(m);
    const int one = 1;
    if (!NQS_CUDA(cudaMemcpyAsync(m->active.p, &one, sizeof(int), cudaMemcpyHostToDevice, ctx().stream)))
        return false;
    if (!pool_launch(m, A, count, seed, d)) return false;
    *bits = m->pbits.p;
    *lq = m->plq.p;
    return true;
}

// Gradient partials of the batch: returns the number of warp partials.
static int grad_launch(Made *m, const uint64_t *bits, int B) {
    const int N = m->N, H = m->H;
    const int warps_per_block = made_grad_smem(N, H, 2) <= 200 * 1024 ? 2 : 1;
    int nw = B < 256 ? B : 256;
    nw = (nw + warps_per_block - 1) / warps_per_block * warps_per_block;
    const int per = (B + nw - 1) / nw;
    if (!m->partials.ensure((size_t)nw * m->PM) || !m->nllp.ensure((size_t)nw)) return -1;
    const size_t smem = (size_t)made_grad_smem(N, H, warps_per_block);
    static bool attr = false;
    if (!attr) {
        if (!NQS_CUDA(cudaFuncSetAttribute(k_made_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)))
            return -1;
        attr = true;
    }
    NQS_LAUNCH("made_grad");
    k_made_grad<<<nw / warps_per_block, 32 * warps_per_block, smem, ctx().stream>>>(made_view(m), bits, B, per,
                                                                                     m->partials.p, m->nllp.p);
    return NQS_CUDA(cudaGetLastError()) ? nw : -1;
}

bool made_train(Made *m, const uint64_t *bits, int B, const unsigned long long *counts) {
    if (B <= 0) return true;
    // train on the first train_batch rows: with the sampler's layout (sample k
    // of chain c at row k C + c) these are the latest states of distinct chains
    if (m->opt.train_batch > 0 && B > m->opt.train_batch) B = m->opt.train_batch;
    cudaStream_t s = ctx().stream;
    int nw = 0;
    for (int it = 0; it < m->opt.train_iters; it++) {
        nw = grad_launch(m, bits, B);
        if (nw < 0) return false;
        NQS_LAUNCH("made_adam");
        k_made_adam<<<(unsigned)((m->PM + 255) / 256), 256, 0, s>>>(m->master.p, m->m1.p, m->v1.p, m->partials.p, nw,
                                                                   m->PM, m->N, m->H, 1.f / (float)B,
                                                                   (float)m->opt.learning_rate, m->ctr.p + 1, m->wb.p,
                                                                   nullptr);
        k_made_count<<<1, 1, 0, s>>>(m->ctr.p + 1);
    }
    {
        // nw = 0 (no training): acceptance bookkeeping and fallback only
        NQS_LAUNCH("made_stats");
        k_made_stats<<<1, 32, 0, s>>>(m->nllp.p, nw, B, m->stats.p, counts, m->active.p, m->opt.min_acceptance);
    }
    return NQS_CUDA(cudaGetLastError());
}

bool made_stats_read(const Made *m, nqs_gpu_made_stats_t *out) {
    double h[8];
    int act = 0;
    unsigned ctr[2] = {0, 0};
    if (!NQS_CUDA(cudaMemcpyAsync(h, m->stats.p, sizeof(h), cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaMemcpyAsync(ctr, m->ctr.p, sizeof(ctr), cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaMemcpyAsync(&act, m->active.p, sizeof(int), cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return false;
    out->nll = h[0];
    out->proposals = h[1];
    out->accepted = h[2];
    out->active = act;
    out->train_steps = (int)ctr[1];
    return true;
}

bool made_get(const Made *m, float *out) {
    return NQS_CUDA(cudaMemcpyAsync(out, m->master.p, sizeof(float) * m->PM, cudaMemcpyDeviceToHost, ctx().stream)) &&
           NQS_CUDA(cudaStreamSynchronize(ctx().stream));
}

bool made_set(Made *m, const float *in) {
    cudaStream_t s = ctx().stream;
    std::vector<float> w(in, in + m->PM);
    for (long p = 0; p < m->PM; p++)
        if (!made_kept(p, m->N, m->H)) w[p] = 0.f;
    if (!NQS_CUDA(cudaMemcpyAsync(m->master.p, w.data(), sizeof(float) * m->PM, cudaMemcpyHostToDevice, s)))
        return false;
    k_made_publish<<<(unsigned)((m->PM + 255) / 256), 256, 0, s>>>(m->master.p, m->wb.p, m->PM, m->N, m->H);
    return NQS_CUDA(cudaGetLastError()) && NQS_CUDA(cudaStreamSynchronize(s));
}

__global__ void k_made_logq_batch(DevMade m, const uint64_t *bits, int B, float *out) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *h1 = (float *)smraw + (size_t)warp * 2 * m.H, *h2 = h1 + m.H;
    const int b = blockIdx.x * (blockDim.x >> 5) + warp;
    if (b >= B) return;
    const float lq = made_logq_warp(m, m.w, bits[b], h1, h2);
    if (lane == 0) out[b] = lq;
}

bool made_logq(const Made *m, const uint64_t *bits, int B, float *out) {
    NQS_LAUNCH("made_logq");
    k_made_logq_batch<<<(B + 3) / 4, 128, 4 * 2 * m->H * sizeof(float), ctx().stream>>>(made_view(m), bits, B, out);
    return NQS_CUDA(cudaGetLastError());
}

bool made_grad(Made *m, const uint64_t *bits, int B, float *out_grad, double *out_nll) {
    const int nw = grad_launch(m, bits, B);
    if (nw < 0) return false;
    static DevBuf<float> g;
    if (!g.ensure((size_t)m->PM)) return false;
    k_made_adam<<<(unsigned)((m->PM + 255) / 256), 256, 0, ctx().stream>>>(
        m->master.p, m->m1.p, m->v1.p, m->partials.p, nw, m->PM, m->N, m->H, 1.f / (float)B, 0.f, m->ctr.p + 1, m->wb.p,
        g.p);
    std::vector<float> nl((size_t)nw);
    if (!NQS_CUDA(cudaMemcpyAsync(out_grad, g.p, sizeof(float) * m->PM, cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaMemcpyAsync(nl.data(), m->nllp.p, sizeof(float) * nw, cudaMemcpyDeviceToHost, ctx().stream)) ||
        !NQS_CUDA(cudaStreamSynchronize(ctx().stream)))
        return false;
    double s = 0.0;
    for (float v : nl) s += v;
    if (out_nll) *out_nll = s / (double)B;
    return true;
}

}  // namespace nqs
