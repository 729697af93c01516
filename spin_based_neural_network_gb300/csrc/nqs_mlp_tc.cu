// nqs_mlp_tc.cu -- local energies of the MLP ansatz with its second layer on the
// 5th-generation tensor cores.
//
// E_loc(s) = diag(s) + sum_{s'} H_{s s'} psi(s') / psi(s) needs the MLP forward pass of
// every connected configuration s' (54 per sample on the kagome 3 x 3 torus).  Its
// layer 1 is a two-column update of the sample's own pre-activations; its layer 2 is a
// dense (configurations x width) x (width x width) product, the GEMM-shaped part:
//
//   tile       128 rows = a few samples x (1 + their connected candidates), one CTA;
//   layer 1    SIMT: z1(s) per sample, z1(s') = z1(s) - 2 s_u W1[:, u] - 2 s_v W1[:, v]
//              (the FP32 order of the SIMT estimator), h1 = tanh(z1), written as TF32
//              hi / lo words in the 128-byte-swizzle K-major layout;
//   layer 2    tcgen05.mma.kind::tf32, M = 128 rows, N = width rounded up to 16,
//              K = width in 32-wide chunks, three passes (hi hi + hi lo + lo hi) into a
//              TMEM accumulator; W2 is split into hi / lo while it is staged (two
//              buffers, the next chunk staged while the tensor cores run the current);
//   epilogue   tcgen05.ld, h2 = tanh(acc + b2), (log|psi|, arg) = (w_re, w_im) . h2 +
//              (c_re, c_im) per row; then a warp per sample sums the ratios.
//
// The Jacobian rows (one back-propagation per sample) stay in k_local_mlp32.
// Upstream has no MLP ansatz; the local-energy formulas follow
// src/nqs/nqs_gradient.c:50-139 (TFIM, XXZ / Heisenberg) and :374-445 (kagome).
#include <math.h>

#include "nqs_amp.cuh"
#include "nqs_tc.cuh"

namespace nqs {
namespace {

constexpr int ML_ROWS = 128;                         // MMA M: configurations per tile
constexpr int ML_THREADS = 256;
constexpr int ML_MAX_SPT = 16;                       // samples per tile at most
constexpr int ML_CHUNK = ML_ROWS * 128;              // bytes of one 32-float K chunk of A (16 KB)
constexpr int ML_A_BYTES = 4 * ML_CHUNK;             // A hi (or lo): K padded to 128
constexpr int ML_B_MAX = 128 * 128;                  // bytes of one B operand chunk at N = 128

struct MlTile {
    int RS;             // rows per sample: the sample itself + its candidates
    int SPT;            // samples per tile
    int NP;             // N of the MMA: width rounded up to 16
    int KC;             // 32-wide K chunks
};

// Candidate kc >= 1 of a sample: a site (TFIM) or a bond of group 1 then group 2.
__device__ __forceinline__ void ml_candidate(const DevHam &H, int kc, int &u, int &v) {
    u = v = -1;
    if (kc <= 0) return;
    const int q = kc - 1;
    if (H.kind == NQS_HAM_TFIM) {
        u = q;
    } else if (q < H.nb1) {
        u = H.b1[2 * q];
        v = H.b1[2 * q + 1];
    } else {
        u = H.b2[2 * (q - H.nb1)];
        v = H.b2[2 * (q - H.nb1) + 1];
    }
}

// Byte offset of element (row r, k) of a K-major operand in 32-float chunks of `rows`
// rows, 128-byte swizzle: row r at r * 128 B of chunk k / 32, its 16-byte unit
// (k % 32) / 4 at position unit ^ (r % 8).
__device__ __forceinline__ uint32_t sw128_off(int r, int k, int rows) {
    const int c = k >> 5, w = k & 31;
    return (uint32_t)(c * rows * 128 + r * 128 + ((((w >> 2) ^ (r & 7))) << 4) + ((w & 3) << 2));
}

// Shared memory (dynamic, 1024-aligned): A hi, A lo (4 K chunks x 128 rows x 128 B each),
// two B buffers (hi, lo: one 32-wide K chunk of W2, N rows), the samples' z1, the head
// partials and the per-row (log|psi|, arg).
constexpr size_t ML_SMEM = 2 * (size_t)ML_A_BYTES + 4 * (size_t)ML_B_MAX + (ML_MAX_SPT * 128 + 6 * 128) * 4 + 1024;

__global__ void __launch_bounds__(ML_THREADS, 1)
k_local_mlp_tc(DevAmp A, DevHam H, const uint64_t *__restrict__ bits, int B, MlTile T, double *__restrict__ Er,
               double *__restrict__ Ei, int *err) {
    extern __shared__ __align__(1024) unsigned char ml_raw[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t slot;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t raw = smem_u32(ml_raw);
    unsigned char *sm = ml_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t sA = smem_u32(sm), sB = sA + 2 * ML_A_BYTES;
    unsigned char *gB = sm + 2 * ML_A_BYTES;
    float *z1s = (float *)(sm + 2 * ML_A_BYTES + 4 * ML_B_MAX);
    float *part = z1s + ML_MAX_SPT * 128;                // re (2 halves), im (2 halves) x 128 rows
    float *la = part + 4 * 128, *ar = la + 128;
    const DevAnsatz &a = A.a;
    const int N = a.N, M = a.M, MP = mlp32_pitch(M);
    const float *W1t = a.m32, *w2 = a.m32 + (long)N * M + (long)M * MP;
    const float *vec = a.m32 + (long)N * M + 2L * M * MP;
    const float *b1 = vec, *b2 = vec + M, *wr = vec + 2 * M, *wi = vec + 3 * M;
    const int s0 = blockIdx.x * T.SPT;

    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&slot)),
                     "r"(128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = slot;

    // layer-1 pre-activations of the tile's samples (the FP32 order of mlp32_z1)
    for (int e = tid; e < T.SPT * M; e += ML_THREADS) {
        const int p = e / M, j = e % M, b = s0 + p;
        if (b < B) {
            const uint64_t s = bits[b];
            float z = b1[j];
            for (int i = 0; i < N; i++) z = fmaf((float)spin_of(s, i), W1t[(long)i * M + j], z);
            z1s[p * 128 + j] = z;
        }
    }
    __syncthreads();
    // A = h1 of the tile's rows (mlp32_z1_flip's order), TF32 hi / lo: two threads per row
    {
        const int r = tid >> 1, k0 = (tid & 1) * 64;
        const int p = r / T.RS, kc = r % T.RS, b = s0 + p;
        const bool valid = p < T.SPT && b < B;
        int u = -1, v = -1;
        uint64_t s = 0;
        if (valid) {
            s = bits[b];
            ml_candidate(H, kc, u, v);
        }
        const float su = u >= 0 ? -2.f * (float)spin_of(s, u) : 0.f, sv = v >= 0 ? -2.f * (float)spin_of(s, v) : 0.f;
        for (int kk = 0; kk < 64; kk++) {
            const int k = k0 + kk;
            if (k >= 32 * T.KC) break;
            float x = 0.f;
            if (valid && k < M) {
                float z = z1s[p * 128 + k];
                if (u >= 0) z = fmaf(su, W1t[(long)u * M + k], z);
                if (v >= 0) z = fmaf(sv, W1t[(long)v * M + k], z);
                x = tanhf(z);
            }
            const float hi = tf32_rna(x), lo = tf32_rna(x - hi);
            const uint32_t off = sw128_off(r, k, ML_ROWS);
            *(float *)(sm + off) = hi;
            *(float *)(sm + ML_A_BYTES + off) = lo;
        }
    }
    // B = W2 rows (output unit j, K = input unit k), chunk q split into TF32 hi / lo while staged
    auto stage_b = [&](int q, int buf) {
        unsigned char *hb = gB + buf * 2 * ML_B_MAX;
        for (int e = tid; e < T.NP * 32; e += ML_THREADS) {
            const int j = e >> 5, k = 32 * q + (e & 31);
            const float x = (j < M && k < M) ? w2[(long)j * MP + k] : 0.f;
            const float hi = tf32_rna(x), lo = tf32_rna(x - hi);
            const uint32_t off = sw128_off(j, e & 31, T.NP);
            *(float *)(hb + off) = hi;
            *(float *)(hb + ML_B_MAX + off) = lo;
        }
    };
    // M = 128, N = NP, FP32 accumulate, TF32 operands, both K-major
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(T.NP >> 3) << 17) |
                           ((uint32_t)(ML_ROWS >> 4) << 24);
    uint32_t cnt[2] = {0u, 0u};
    bool ok = true;
    stage_b(0, 0);
    for (int q = 0; q < T.KC; q++) {
        const int bq = q & 1;
        fence_proxy_async();                             // generic-proxy stores -> tensor-core reads
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t bb = sB + bq * 2 * ML_B_MAX;
#pragma unroll
            for (int pass = 0; pass < 3; pass++) {       // hi hi, hi lo, lo hi
                const uint32_t ao = sA + (pass == 2 ? ML_A_BYTES : 0) + q * ML_CHUNK;
                const uint32_t bo = bb + (pass == 1 ? ML_B_MAX : 0);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    umma_tf32(tmem, sw128_desc(ao + k * 32), sw128_desc(bo + k * 32), idesc,
                              (q | pass | k) ? 1u : 0u);
            }
            umma_commit(&mbar[bq]);
        }
        cnt[bq]++;
        if (q + 1 < T.KC) {
            const int nb = (q + 1) & 1;
            // the buffer being refilled was read by the MMAs of chunk q - 1
            if (q >= 1 && !__syncthreads_and(mbar_wait(&mbar[nb], (cnt[nb] - 1) & 1, err))) {
                ok = false;
                break;
            }
            stage_b(q + 1, nb);
        }
    }
    if (ok) {
        const int lb = (T.KC - 1) & 1;
        bool done = mbar_wait(&mbar[lb], (cnt[lb] - 1) & 1, err);
        if (T.KC > 1) done = done && mbar_wait(&mbar[lb ^ 1], (cnt[lb ^ 1] - 1) & 1, err);
        ok = __syncthreads_and(done);
    }
    tc_fence_after();
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. (its rows), columns 64 (w / 4) ..;
    // h2 = tanh(acc + b2) and the two head sums of its half of the columns
    {
        const int h = warp >> 2, row = 32 * (warp & 3) + lane;
        float re = 0.f, im = 0.f;
        if (ok) {
            for (int cc = 0; cc < 2; cc++) {
                const int col = 64 * h + 32 * cc;
                if (col < T.NP) {                        // warp-uniform
                    float v[32];
                    tmem_ld32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col, v);
#pragma unroll
                    for (int t = 0; t < 32; t++) {
                        const int j = col + t;
                        if (j < M) {
                            const float h2 = tanhf(v[t] + b2[j]);
                            re = fmaf(wr[j], h2, re);
                            im = fmaf(wi[j], h2, im);
                        }
                    }
                }
            }
        }
        part[h * 128 + row] = re;
        part[256 + h * 128 + row] = im;
    }
    tc_fence_before();
    __syncthreads();
    if (tid < ML_ROWS) {
        la[tid] = part[tid] + part[128 + tid] + vec[4 * M];
        ar[tid] = part[256 + tid] + part[384 + tid] + vec[4 * M + 1];
    }
    __syncthreads();
    // local energies: a warp per sample, lanes over its candidates (k_local_mlp32's terms)
    for (int p = warp; p < T.SPT; p += ML_THREADS / 32) {
        const int b = s0 + p;
        if (b >= B) break;
        const uint64_t s = bits[b];
        const int par0 = marshall_count(A, s);
        const float la0 = la[p * T.RS], ar0 = ar[p * T.RS];
        float e_re = 0.f, e_im = 0.f;
        if (H.kind == NQS_HAM_TFIM)
            for (int k = lane; k < H.nb1; k += 32)
                e_re += -(float)H.J * (float)(spin_of(s, H.b1[2 * k]) * spin_of(s, H.b1[2 * k + 1]));
        for (int kc = 1 + lane; kc < T.RS; kc += 32) {
            int u, v;
            ml_candidate(H, kc, u, v);
            const int r = p * T.RS + kc;
            float jxy;
            if (H.kind == NQS_HAM_TFIM) {
                jxy = -2.f * (float)H.Gamma;             // the ratio's factor below is jxy / 2 = -Gamma
            } else {
                const bool g2 = kc - 1 >= H.nb1;
                const float jz = g2 ? (float)H.J2 : (float)H.Jz;
                jxy = g2 ? (float)H.J2 : (float)H.Jxy;
                e_re += 0.25f * jz * (float)(spin_of(s, u) * spin_of(s, v));
                if (spin_of(s, u) == spin_of(s, v)) continue;
            }
            uint64_t s2 = s ^ (1ull << u);
            if (v >= 0) s2 ^= 1ull << v;
            const float mag = expf(la[r] - la0);
            float sn, cs;
            sincosf(ar[r] - ar0, &sn, &cs);
            const float sg = ((marshall_count(A, s2) - par0) & 1) ? -1.f : 1.f;
            e_re += 0.5f * jxy * sg * mag * cs;
            e_im += 0.5f * jxy * sg * mag * sn;
        }
        e_re = warp_sum_f(e_re);
        e_im = warp_sum_f(e_im);
        if (lane == 0) {
            if (Er) Er[b] = ok ? (double)e_re : nan("");
            if (Ei) Ei[b] = ok ? (double)e_im : nan("");
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
}

int ml_candidates(const DevAmp &A, const DevHam &H) { return H.kind == NQS_HAM_TFIM ? A.a.N : H.nb1 + H.nb2; }

}  // namespace

// The tensor-core layer applies to the MLP program without a symmetry projection, width
// <= 128 (N of one MMA, one TMEM allocation), and a sample with its candidates within one
// 128-row tile.
bool mlp_tc_capable(const DevAmp &A, const DevHam &H) {
    return A.G == 0 && A.a.kind == KIND_MLP && A.a.m32 != nullptr && A.a.M <= 128 && A.a.N <= 64 &&
           1 + ml_candidates(A, H) <= ML_ROWS;
}

// Local energies (FP32, stored as doubles) of B configurations through the tensor-core
// layer; Er / Ei may be NULL.
bool launch_mlp_eloc_tc(const DevAmp &A, const DevHam &H, const uint64_t *bits, int B, double *Er, double *Ei) {
    MlTile T;
    T.RS = 1 + ml_candidates(A, H);
    T.SPT = ML_ROWS / T.RS < ML_MAX_SPT ? ML_ROWS / T.RS : ML_MAX_SPT;
    T.NP = (A.a.M + 15) / 16 * 16;
    T.KC = (A.a.M + 31) / 32;
    static bool attr = false;
    if (!attr) {
        if (!NQS_CUDA(cudaFuncSetAttribute(k_local_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)ML_SMEM)))
            return false;
        attr = true;
    }
    static DevBuf<int> err;
    cudaStream_t st = ctx().stream;
    if (!err.ensure(1) || !NQS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st))) return false;
    const int grid = (B + T.SPT - 1) / T.SPT;
    k_local_mlp_tc<<<grid, ML_THREADS, ML_SMEM, st>>>(A, H, bits, B, T, Er, Ei, err.p);
    return NQS_CUDA(cudaGetLastError());
}

}  // namespace nqs
