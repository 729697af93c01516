// Learned Metropolis proposal: a masked autoregressive MLP (MADE; Germain,
// Gregor, Murray, Larochelle, ICML 2015) over the N spins, trained online on
// the chains' own samples.
//
//   h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), p(x_i = 1 | x_<i) = sigmoid(W3 h2 + b3)_i
//
// x_i = 1 marks a down spin (the bit convention of the configurations).  Unit
// k of either hidden layer has degree m(k) = 1 + floor(k (N - 1) / H), so the
// units of one degree are contiguous; the masks keep
// W1[k][i] for m(k) >= i + 1, W2[k][j] for m(k) >= m(j) and W3[i][k] for
// i + 1 > m(k), so output i sees only x_<i.  With a fixed number of down spins
// (exchange moves conserve it) a site whose value is already determined by the
// count is forced and contributes nothing to log q, so q is normalised over
// the sector.  Weights are BF16 (FP32 accumulation); the optimiser keeps FP32
// masters.
//
// Parameter layout (FP32 masters and BF16 copies alike), laid out so that the
// lane-parallel loops read consecutive addresses:
//   W1t[i][k] (N x H), b1[k], W2t[j][k] (H x H, W2t[j][k] = W2[k][j]), b2[k],
//   W3t[k][i] (H x N, W3t[k][i] = W3[i][k]), b3[i].
#pragma once
#include <cuda_bf16.h>

#include "nqs_internal.cuh"

namespace nqs {

constexpr int MADE_MAX_H = 128;

struct MadeOff {
    long w1, b1, w2, b2, w3, b3, total;
};

__host__ __device__ inline MadeOff made_off(int N, int H) {
    MadeOff o;
    o.w1 = 0;
    o.b1 = (long)N * H;
    o.w2 = o.b1 + H;
    o.b2 = o.w2 + (long)H * H;
    o.w3 = o.b2 + H;
    o.b3 = o.w3 + (long)H * N;
    o.total = o.b3 + N;
    return o;
}

__host__ __device__ inline int made_degree(int k, int N, int H) { return 1 + (k * (N - 1)) / H; }

// first unit of degree d (d = 1 .. N; made_first(N) = H)
__host__ __device__ inline int made_first(int d, int N, int H) { return ((d - 1) * H + N - 2) / (N - 1); }

// Whether parameter p of the layout is kept by the masks.
__host__ __device__ inline bool made_kept(long p, int N, int H) {
    const MadeOff o = made_off(N, H);
    if (p < o.b1) return made_degree((int)(p % H), N, H) >= (int)(p / H) + 1;            // W1t[i][k]
    if (p >= o.w2 && p < o.b2) {
        const long q = p - o.w2;
        return made_degree((int)(q % H), N, H) >= made_degree((int)(q / H), N, H);     // W2t[j][k]
    }
    if (p >= o.w3 && p < o.b3) {
        const long q = p - o.w3;
        return (int)(q % N) + 1 > made_degree((int)(q / N), N, H);                     // W3t[k][i]
    }
    return true;                                                                       // biases
}

// Device view of a sampler's learned proposal.
struct DevMade {
    int N, H;
    int n_ones;                   // down spins of the sector, -1 = unconstrained
    const __nv_bfloat16 *w;       // BF16 weights (global)
    const uint64_t *pbits;        // proposal pool [C][per_chain]
    const float *plq, *plpsi;     // log q and log|psi| of the pool entries
    int per_chain;                // pool entries per chain, 0 = learned proposal off
    uint32_t mix_thr;             // a move is a learned proposal when its Philox word y < mix_thr
    const int *active;            // device flag written by the optimiser (fallback)
};

// -1: site i is free; 0 / 1: the sector forces this value (ones_before down
// spins among x_<i).
__device__ __forceinline__ int made_forced(int i, int ones_before, int N, int n_ones) {
    if (n_ones < 0) return -1;
    const int need = n_ones - ones_before, rem = N - i;
    if (need <= 0) return 0;
    if (need >= rem) return 1;
    return -1;
}

__device__ __forceinline__ float log_sigmoid(float l) {
    return l >= 0.f ? -log1pf(expf(-l)) : l - log1pf(expf(l));
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float bf(const __nv_bfloat16 *p, long i) { return __bfloat162float(p[i]); }

// Building blocks shared by the autoregressive sampler, the teacher-forced
// log q and the chains, written once so that all of them round identically
// (q(x) is the same FP32 number whichever path computes it).  Lanes own
// hidden units k = lane + 32 q and outputs i = lane + 32 q.

// h2_k = relu(b2_k + sum_j W2t[j][k] h1_j), four interleaved partial sums
__device__ __forceinline__ float made_h2(const __nv_bfloat16 *W, const MadeOff &o, int H, int k, const float *h1,
                                         float *a2_out = nullptr) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    const __nv_bfloat16 *w = W + o.w2 + k;
#pragma unroll 4
    for (int j = 0; j < H; j += 4) {
        s0 = fmaf(__bfloat162float(w[(long)j * H]), h1[j], s0);
        s1 = fmaf(__bfloat162float(w[(long)(j + 1) * H]), h1[j + 1], s1);
        s2 = fmaf(__bfloat162float(w[(long)(j + 2) * H]), h1[j + 2], s2);
        s3 = fmaf(__bfloat162float(w[(long)(j + 3) * H]), h1[j + 3], s3);
    }
    const float a = bf(W, o.b2 + k) + ((s0 + s1) + (s2 + s3));
    if (a2_out) *a2_out = a;
    return fmaxf(a, 0.f);
}

// Contribution of the hidden-2 units of degree d (contiguous, ascending k) to
// the running logit of output i.
__device__ __forceinline__ float made_logit_add(const __nv_bfloat16 *W, const MadeOff &o, int N, int H, int d, int i,
                                                const float *h2, float L) {
    const int k1 = made_first(d + 1, N, H);
    for (int k = made_first(d, N, H); k < k1; k++) L = fmaf(bf(W, o.w3 + (long)k * N + i), h2[k], L);
    return L;
}

// log q(x) with teacher forcing, one warp.  W: BF16 weights (shared or global),
// h1 / h2: per-warp scratch of H floats each.  The logit of output i sums the
// hidden-2 units degree by degree (d = 1 .. i), the order in which the
// autoregressive sampler finalises them, and log q adds the free sites in
// ascending order.
__device__ __forceinline__ float made_logq_warp(const DevMade &m, const __nv_bfloat16 *W, uint64_t x, float *h1,
                                                float *h2) {
    const int lane = threadIdx.x & 31, N = m.N, H = m.H;
    const MadeOff o = made_off(N, H);
    for (int k = lane; k < H; k += 32) {
        float a = bf(W, o.b1 + k);
        for (int i = 0; i < N; i++)
            if ((x >> i) & 1ull) a += bf(W, o.w1 + (long)i * H + k);
        h1[k] = fmaxf(a, 0.f);
    }
    __syncwarp();
    for (int k = lane; k < H; k += 32) h2[k] = made_h2(W, o, H, k, h1);
    __syncwarp();
    float term[2] = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int i = lane + 32 * q;
        if (i < N) {
            float L = 0.f;
            for (int d = 1; d <= i && d < N; d++) L = made_logit_add(W, o, N, H, d, i, h2, L);
            const float l = L + bf(W, o.b3 + i);
            const int xi = (int)((x >> i) & 1ull);
            if (made_forced(i, __popcll(x & ((1ull << i) - 1ull)), N, m.n_ones) < 0)
                term[q] = xi ? log_sigmoid(l) : log_sigmoid(-l);
        }
    }
    float lq = 0.f;
    for (int i = 0; i < N; i++) lq += __shfl_sync(0xffffffffu, i < 32 ? term[0] : term[1], i & 31);
    __syncwarp();
    return lq;
}

// log|psi(x)| of the RBM / cRBM in FP32, one warp: Re(sum_i a_i s_i) +
// sum_h log|2 cosh theta_h| with log|2 cosh(x + iy)| = |x| + 0.5 log1p(e (2 cos 2y + e)),
// e = exp(-2|x|).
template <bool CPLX>
__device__ __forceinline__ float rbm_logabs32(const DevAnsatz &a, uint64_t s) {
    const int lane = threadIdx.x & 31;
    float acc = 0.f;
    for (int h = lane; h < a.M; h += 32) {
        float xr = a.b32[h].x, xi = a.b32[h].y;
        for (int i = 0; i < a.N; i++) {
            const float sp = (s >> i) & 1ull ? -1.f : 1.f;
            const float2 w = a.w32[(long)i * a.M + h];
            xr = fmaf(sp, w.x, xr);
            if (CPLX) xi = fmaf(sp, w.y, xi);
        }
        const float ax = fabsf(xr), e = expf(-2.f * ax);
        acc += CPLX ? ax + 0.5f * log1pf(e * (2.f * cosf(2.f * xi) + e)) : ax + log1pf(e);
    }
    for (int i = lane; i < a.N; i += 32) acc += ((s >> i) & 1ull ? -1.f : 1.f) * a.a32[i].x;
    return warp_sumf(acc);
}

// ---------------------------------------------------------------- host interface (nqs_made.cu)
struct Made;
Made *made_create(int N, int n_ones, const nqs_gpu_made_options_t &opt);
void made_free(Made *m);
long made_num_params(const Made *m);
DevMade made_view(const Made *m);
// dynamic shared memory of a chain block with `warps` warps (BF16 weights + scratch)
size_t made_chain_smem(const Made *m, int warps);
// draw the pool for a launch of C chains x total_moves moves; fills the device view
bool made_prepare(Made *m, const DevAmp &A, int C, int total_moves, uint64_t seed, DevMade *out);
// `count` independent draws from q (diagnostic)
bool made_sample(Made *m, const DevAmp &A, long count, uint64_t seed, const uint64_t **bits, const float **lq);
// train_iters Adam iterations on a produced batch, then statistics / fallback
bool made_train(Made *m, const uint64_t *bits, int B, const unsigned long long *counts);
bool made_stats_read(const Made *m, nqs_gpu_made_stats_t *out);
bool made_get(const Made *m, float *out);
bool made_set(Made *m, const float *in);
bool made_logq(const Made *m, const uint64_t *bits, int B, float *out);
bool made_grad(Made *m, const uint64_t *bits, int B, float *out_grad, double *out_nll);

}  // namespace nqs
