// Mixed-precision MinSR solve: tensor-core Gram, FP32 factor, FP64 refinement.
//
//   1. centre O in FP64 (in place) and split it into two TF32 words,
//      O_c = hi + lo (hi = tf32(O_c), lo = tf32(O_c - hi));
//   2. T = (hi hi^T + hi lo^T + lo hi^T) / N_s + shift I on the 5th-generation
//      tensor cores: tcgen05.mma kind::tf32 issued by one thread, operands
//      staged by TMA (cp.async.bulk.tensor, 128-byte swizzle) in a 3-stage
//      mbarrier ring, FP32 accumulator in TMEM read back with tcgen05.ld;
//      only the lower-triangular 128 x 128 tiles are computed;
//   3. FP32 blocked Cholesky T = L L^T and the explicit inverse X = L^{-1}, so
//      every solve with the factor is two GEMVs (X and X^T, 33.5 MB at
//      N_s = 4096, resident in the 129 MB L2);
//   4. iterative refinement in FP64 against the exact operator
//      A y = O_c (O_c^T y) / N_s + shift y (two FP64 passes over O_c):
//      y <- y + X^T X (eps - A y).
// The FP32 factor of the TF32x3 Gram keeps the refinement contraction well
// below 1 for cond(A) up to ~1e6; the achieved relative residual is returned.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <math.h>

#include "nqs_amp.cuh"

namespace nqs {

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after ~2^24 polls with back-off (seconds), raises the
// kernel's error flag and reports failure instead of spinning forever.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
    for (uint32_t it = 0; it < (1u << 24); it++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*((volatile int *)err)) return false;
        if (it > 32) __nanosleep(64);
    }
    atomicExch(err, 1);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile stored in the
// canonical 128-byte-swizzle layout (rows of 128 B, 8-row atoms 1024 B apart).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);        // start address
    d |= (uint64_t)1 << 16;                           // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                           // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                           // swizzle: 128 B
    return d;
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
        ::"r"(tmem_d), "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 32 consecutive TMEM columns -> 32 registers per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// ---------------------------------------------------------------- split
// O_c = O - <O> (FP64, in place) and its TF32 hi / lo words in the padded
// operand arrays (row pitch ldp floats; the pads stay zero).
__global__ void k_center_split(double *O, int Ns, long P, const double *__restrict__ gm, float *hi, float *lo,
                               long ldp) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, tot = (size_t)Ns * P;
    for (; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        size_t i = t / P, k = t % P;
        double x = O[t] - gm[k];
        O[t] = x;
        float h = tf32_rna((float)x);
        float l = tf32_rna((float)(x - (double)h));
        hi[i * ldp + k] = h;
        lo[i * ldp + k] = l;
    }
}

// ---------------------------------------------------------------- tensor-core Gram
constexpr int TC_M = 128, TC_N = 128, TC_K = 32;      // tile; K per stage = 128 B of FP32
constexpr int TC_STAGES = 3;
constexpr int TC_STAGE_BYTES = (TC_M + TC_N) * TC_K * 4;
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 + 256;

struct GramTcArgs {
    int kt_per_seg;       // K tiles per segment
    int nseg;             // passes: 1 = hi hi^T, 3 = hi hi^T + hi lo^T + lo hi^T
    float scale, shift;
    float *C;             // [n][n] lower triangle written
    int n;
    int *err;
};

__global__ void __launch_bounds__(128, 1)
k_gram_tf32_tc(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
               GramTcArgs g) {
    extern __shared__ uint8_t smem_raw[];
    uint32_t base = smem_u32(smem_raw);
    uint32_t pad = ((base + 1023u) & ~1023u) - base;
    uint8_t *sm = smem_raw + pad;
    uint64_t *full = (uint64_t *)(sm + TC_STAGES * TC_STAGE_BYTES);
    uint64_t *empty = full + TC_STAGES;
    uint64_t *done = empty + TC_STAGES;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int bi, bj;
    {
        int t = blockIdx.x;
        int r = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
        while ((r + 1) * (r + 2) / 2 <= t) r++;
        while (r * (r + 1) / 2 > t) r--;
        bi = r;
        bj = t - r * (r + 1) / 2;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(TC_N) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int total = g.kt_per_seg * g.nseg;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int it = 0; it < total && ok; it++) {
            int s = it % TC_STAGES, u = it / TC_STAGES;
            if (u > 0) ok = mbar_wait(&empty[s], (u - 1) & 1, g.err);
            if (!ok) break;
            int seg = it / g.kt_per_seg, kt = it - seg * g.kt_per_seg;
            const CUtensorMap *ma = seg == 2 ? &map_lo : &map_hi;   // segments: (hi,hi) (hi,lo) (lo,hi)
            const CUtensorMap *mb = seg == 1 ? &map_lo : &map_hi;
            uint8_t *sa = sm + s * TC_STAGE_BYTES;
            uint8_t *sb = sa + TC_M * TC_K * 4;
            mbar_expect_tx(&full[s], TC_STAGE_BYTES);
            tma_load_2d(sa, ma, &full[s], kt * TC_K, bi * TC_M);
            tma_load_2d(sb, mb, &full[s], kt * TC_K, bj * TC_N);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: M = N = 128, K = 8 per instruction, 4 per stage
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);
        for (int it = 0; it < total && ok; it++) {
            int s = it % TC_STAGES, u = it / TC_STAGES;
            ok = mbar_wait(&full[s], u & 1, g.err);
            if (!ok) break;
            tc_fence_after();
            uint32_t sa = smem_u32(sm + s * TC_STAGE_BYTES);
            uint32_t sb = sa + TC_M * TC_K * 4;
#pragma unroll
            for (int k = 0; k < TC_K / 8; k++)
                umma_tf32(tmem, sw128_desc(sa + k * 32), sw128_desc(sb + k * 32), idesc,
                          (it > 0 || k > 0) ? 1u : 0u);
            umma_commit(&empty[s]);
        }
        umma_commit(done);
    }
    __syncwarp();
    // epilogue: warp w owns TMEM lanes (rows) 32w .. 32w+31
    bool ready = mbar_wait(done, 0, g.err);
    tc_fence_after();
    if (ready) {
        const int row = bi * TC_M + warp * 32 + lane;
        for (int c = 0; c < TC_N / 32; c++) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
            int col0 = bj * TC_N + c * 32;
            if (row < g.n) {
                float *dst = g.C + (size_t)row * g.n;
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    int col = col0 + j;
                    if (col <= row && col < g.n) dst[col] = v[j] * g.scale + (col == row ? g.shift : 0.f);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N) : "memory");
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static bool make_map(CUtensorMap *m, const float *ptr, long rows, long cols_pad) {
    if (!g_encode) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return false;
        }
        g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    cuuint64_t dims[2] = {(cuuint64_t)cols_pad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols_pad * 4};
    cuuint32_t box[2] = {TC_K, TC_M};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)ptr, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return false;
    }
    return true;
}

// ---------------------------------------------------------------- FP32 Cholesky
constexpr int NB32 = 32, TG32 = 64, KC32 = 16;

__global__ void k_potrf_diag32(float *A, int n, int k0, int kb, int *status) {
    if (status[0] >= 0) return;
    __shared__ float L[NB32][NB32 + 1];
    __shared__ int fail;
    int tx = threadIdx.x, ty = threadIdx.y;
    if (tx < kb && ty < kb && tx <= ty) L[ty][tx] = A[(size_t)(k0 + ty) * n + k0 + tx];
    if (tx == 0 && ty == 0) fail = -1;
    __syncthreads();
    for (int j = 0; j < kb; j++) {
        if (tx == 0 && ty == 0) {
            float d = L[j][j];
            if (!(d > 0.f)) fail = j;
            else L[j][j] = sqrtf(d);
        }
        __syncthreads();
        if (fail >= 0) break;
        if (tx == 0 && ty > j && ty < kb) L[ty][j] = L[ty][j] / L[j][j];
        __syncthreads();
        if (ty > j && ty < kb && tx > j && tx <= ty) L[ty][tx] -= L[ty][j] * L[tx][j];
        __syncthreads();
    }
    if (fail >= 0) {
        if (tx == 0 && ty == 0) status[0] = k0 + fail;
        return;
    }
    if (tx < kb && ty < kb && tx <= ty) A[(size_t)(k0 + ty) * n + k0 + tx] = L[ty][tx];
}

__global__ void k_trsm_panel32(float *A, int n, int k0, int kb, int row0, const int *status) {
    if (status[0] >= 0) return;
    __shared__ float L[NB32][NB32 + 1];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        int r = e / kb, c = e % kb;
        L[r][c] = c <= r ? A[(size_t)(k0 + r) * n + k0 + c] : 0.f;
    }
    __syncthreads();
    int i = row0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x[NB32];
    float *row = A + (size_t)i * n + k0;
#pragma unroll
    for (int j = 0; j < NB32; j++) x[j] = j < kb ? row[j] : 0.f;
#pragma unroll
    for (int j = 0; j < NB32; j++) {
        if (j < kb) {
            float s = x[j];
#pragma unroll
            for (int m = 0; m < j; m++) s -= x[m] * L[j][m];
            x[j] = s / L[j][j];
        }
    }
#pragma unroll
    for (int j = 0; j < NB32; j++)
        if (j < kb) row[j] = x[j];
}

__device__ __forceinline__ void tri_tile32(int t, int &bi, int &bj) {
    int r = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= t) r++;
    while (r * (r + 1) / 2 > t) r--;
    bi = r;
    bj = t - r * (r + 1) / 2;
}

// A[i][j] -= sum_m L[i][k0+m] L[j][k0+m] over the lower trailing tiles.
__global__ void __launch_bounds__(256) k_syrk_update32(float *A, int n, int k0, int kb, int k1, const int *status) {
    if (status[0] >= 0) return;
    __shared__ float As[NB32][TG32 + 1], Bs[NB32][TG32 + 1];
    int bi, bj;
    tri_tile32(blockIdx.x, bi, bj);
    int r0 = k1 + bi * TG32, c0 = k1 + bj * TG32;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int e = tid; e < TG32 * NB32; e += 256) {
        int rr = e / NB32, cc = e % NB32;
        int ra = r0 + rr, rb = c0 + rr;
        As[cc][rr] = (ra < n && cc < kb) ? A[(size_t)ra * n + k0 + cc] : 0.f;
        Bs[cc][rr] = (rb < n && cc < kb) ? A[(size_t)rb * n + k0 + cc] : 0.f;
    }
    __syncthreads();
    float acc[4][4] = {};
#pragma unroll 8
    for (int c = 0; c < NB32; c++) {
        float av[4], bv[4];
#pragma unroll
        for (int m = 0; m < 4; m++) av[m] = As[c][ty + 16 * m];
#pragma unroll
        for (int q = 0; q < 4; q++) bv[q] = Bs[c][tx + 16 * q];
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[m][q] = fmaf(av[m], bv[q], acc[m][q]);
    }
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int i = r0 + ty + 16 * m, j = c0 + tx + 16 * q;
            if (i < n && j <= i) A[(size_t)i * n + j] -= acc[m][q];
        }
}

// ---------------------------------------------------------------- FP32 triangular inverse
// X = L^{-1} by block columns from the last to the first (blocked TRTRI):
//   X_jj = inv(L_jj);  X[j+b:, j:j+b] = -(X[j+b:, j+b:] L[j+b:, j:j+b]) X_jj.
__global__ void k_trtri_diag32(const float *L, float *X, int n, int k0, int kb) {
    // one warp: lane c inverts column c of the kb x kb lower block by forward substitution
    __shared__ float Ls[NB32][NB32 + 1];
    int lane = threadIdx.x;
    for (int e = lane; e < kb * kb; e += 32) {
        int r = e / kb, c = e % kb;
        Ls[r][c] = c <= r ? L[(size_t)(k0 + r) * n + k0 + c] : 0.f;
    }
    __syncwarp();
    if (lane < kb) {
        float x[NB32];
#pragma unroll
        for (int r = 0; r < NB32; r++) {
            if (r < kb) {
                float s = (r == lane) ? 1.f : 0.f;
#pragma unroll
                for (int m = 0; m < r; m++) s -= Ls[r][m] * x[m];
                x[r] = r < lane ? 0.f : s / Ls[r][r];
            }
        }
#pragma unroll
        for (int r = 0; r < NB32; r++)
            if (r < kb) X[(size_t)(k0 + r) * n + k0 + lane] = x[r];
    }
}

// W[i][c] = sum_{k=k1}^{i} X[i][k] L[k][k0+c] for rows i in [k1, n), then
// X[i][k0+c] = -sum_m W[i][m] X_jj[m][c].  One block per 64 rows.
__global__ void __launch_bounds__(256) k_trtri_panel32(const float *L, float *X, int n, int k0, int kb, int k1) {
    __shared__ float Xs[KC32][TG32 + 1];
    __shared__ float Ls[KC32][NB32 + 1];
    __shared__ float Xd[NB32][NB32 + 1];
    __shared__ float W[TG32][NB32 + 1];
    const int tid = threadIdx.x;
    const int r0 = k1 + blockIdx.x * TG32;
    const int tr = tid >> 2;            // row within the tile (64 rows, 4 threads each)
    const int tc = (tid & 3) * 8;       // 8 columns per thread
    float acc[8] = {};
    int rmax = min(r0 + TG32, n);
    for (int kk = k1; kk < rmax; kk += KC32) {
        for (int e = tid; e < TG32 * KC32; e += 256) {
            int rr = e / KC32, cc = e % KC32;
            int i = r0 + rr, k = kk + cc;
            Xs[cc][rr] = (i < n && k <= i && k < n) ? X[(size_t)i * n + k] : 0.f;
        }
        for (int e = tid; e < KC32 * NB32; e += 256) {
            int rr = e / NB32, cc = e % NB32;
            int k = kk + rr;
            Ls[rr][cc] = (k < n && cc < kb) ? L[(size_t)k * n + k0 + cc] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < KC32; c++) {
            float xv = Xs[c][tr];
#pragma unroll
            for (int q = 0; q < 8; q++) acc[q] = fmaf(xv, Ls[c][tc + q], acc[q]);
        }
        __syncthreads();
    }
    for (int e = tid; e < NB32 * NB32; e += 256) {
        int r = e / NB32, c = e % NB32;
        Xd[r][c] = (r < kb && c < kb && c <= r) ? X[(size_t)(k0 + r) * n + k0 + c] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) W[tr][tc + q] = acc[q];
    __syncthreads();
    int i = r0 + tr;
    if (i < n) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            int c = tc + q;
            if (c < kb) {
                float s = 0.f;
                for (int m = c; m < kb; m++) s += W[tr][m] * Xd[m][c];
                X[(size_t)i * n + k0 + c] = -s;
            }
        }
    }
}

// ---------------------------------------------------------------- GEMVs
// w = X v (X lower triangular FP32, v FP64): warp per row.
__global__ void k_trmv_lower(const float *__restrict__ X, int n, const double *__restrict__ v, double *w) {
    int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    const float *xr = X + (size_t)row * n;
    double s = 0.0;
    for (int k = lane; k <= row; k += 32) s += (double)xr[k] * v[k];
    s = warp_sum(s);
    if (lane == 0) w[row] = s;
}

// y = X^T w: y_k = sum_{i >= k} X[i][k] w_i, 32 columns x 8 row groups per block.
__global__ void k_trmv_lower_t(const float *__restrict__ X, int n, const double *__restrict__ w, double *y,
                               double *add_to) {
    __shared__ double a[8][33];
    int k = blockIdx.x * 32 + threadIdx.x;
    double s = 0.0;
    if (k < n)
        for (int i = k + threadIdx.y; i < n; i += 8) s += (double)X[(size_t)i * n + k] * w[i];
    a[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && k < n) {
        double S = 0.0;
        for (int q = 0; q < 8; q++) S += a[q][threadIdx.x];
        if (add_to) add_to[k] += S;
        else y[k] = S;
    }
}

// u = O_c^T y (FP64, 32 columns x 8 row groups per block)
__global__ void k_ct_dot(const double *__restrict__ O, int Ns, long P, const double *__restrict__ y, double *u) {
    __shared__ double a[8][33];
    long k = (long)blockIdx.x * 32 + threadIdx.x;
    double s = 0.0;
    if (k < P)
        for (int i = threadIdx.y; i < Ns; i += 8) s += O[(size_t)i * P + k] * y[i];
    a[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && k < P) {
        double S = 0.0;
        for (int q = 0; q < 8; q++) S += a[q][threadIdx.x];
        u[k] = S;
    }
}

// r_i = eps_i - (O_c u)_i / Ns - shift y_i  (warp per row), |r|^2 and |eps|^2 partials
__global__ void k_residual(const double *__restrict__ O, int Ns, long P, const double *__restrict__ u,
                           const double *__restrict__ y, const double *__restrict__ eps, double shift,
                           double *r) {
    int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= Ns) return;
    const double *o = O + (size_t)row * P;
    double s = 0.0;
    for (long k = lane; k < P; k += 32) s += o[k] * u[k];
    s = warp_sum(s);
    if (lane == 0) r[row] = eps[row] - s / (double)Ns - shift * y[row];
}

__global__ void k_norms(const double *__restrict__ r, const double *__restrict__ e, int n, double *out) {
    __shared__ double a[1024], b[1024];
    double s = 0.0, t = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s += r[i] * r[i];
        t += e[i] * e[i];
    }
    a[threadIdx.x] = s;
    b[threadIdx.x] = t;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            a[threadIdx.x] += a[threadIdx.x + o];
            b[threadIdx.x] += b[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = a[0];
        out[1] = b[0];
    }
}

// ---------------------------------------------------------------- driver
struct MixedWs {
    DevBuf<float> hi, lo, T, X;
    DevBuf<double> w, u, r, nrm;
    DevBuf<int> status;
    int ns_pad = 0;
    long p_pad = 0;
};
static MixedWs g_mx;

bool minsr_mixed_solve(double *O, const double *gm, const double *eps, int Ns, long P, double shift, int sweeps,
                       int passes, double *y, double *out_resid, int *out_fail) {
    cudaStream_t st = ctx().stream;
    MixedWs &w = g_mx;
    const int ns_pad = (Ns + TC_M - 1) / TC_M * TC_M;
    const long p_pad = (P + TC_K - 1) / TC_K * TC_K;
    if (ns_pad != w.ns_pad || p_pad != w.p_pad) {
        if (!w.hi.ensure((size_t)ns_pad * p_pad) || !w.lo.ensure((size_t)ns_pad * p_pad)) return false;
        if (!NQS_CUDA(cudaMemsetAsync(w.hi.p, 0, sizeof(float) * ns_pad * p_pad, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.lo.p, 0, sizeof(float) * ns_pad * p_pad, st)))
            return false;
        w.ns_pad = ns_pad;
        w.p_pad = p_pad;
    }
    if (!w.T.ensure((size_t)Ns * Ns) || !w.X.ensure((size_t)Ns * Ns) || !w.w.ensure(Ns) || !w.u.ensure(P) ||
        !w.r.ensure(Ns) || !w.nrm.ensure(2) || !w.status.ensure(2))
        return false;
    NQS_CUDA(cudaMemsetAsync(w.status.p, 0xff, 2 * sizeof(int), st));
    {
        NQS_LAUNCH("center_split");
        k_center_split<<<ctx().sm_count * 8, 256, 0, st>>>(O, Ns, P, gm, w.hi.p, w.lo.p, p_pad);
    }
    // tensor-core Gram
    CUtensorMap mh, ml;
    if (!make_map(&mh, w.hi.p, ns_pad, p_pad) || !make_map(&ml, w.lo.p, ns_pad, p_pad)) return false;
    static DevBuf<int> err;
    if (!err.ensure(1)) return false;
    NQS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    GramTcArgs g;
    g.kt_per_seg = (int)(p_pad / TC_K);
    g.nseg = passes >= 3 ? 3 : 1;
    g.scale = (float)(1.0 / (double)Ns);
    g.shift = (float)shift;
    g.C = w.T.p;
    g.n = Ns;
    g.err = err.p;
    int nt = ns_pad / TC_M;
    {
        static bool attr = false;
        if (!attr) {
            if (!NQS_CUDA(cudaFuncSetAttribute(k_gram_tf32_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               TC_SMEM)))
                return false;
            attr = true;
        }
        NQS_LAUNCH("gram_tc");
        k_gram_tf32_tc<<<nt * (nt + 1) / 2, 128, TC_SMEM, st>>>(mh, ml, g);
    }
    if (!NQS_CUDA(cudaGetLastError())) return false;
    // FP32 Cholesky
    for (int k0 = 0; k0 < Ns; k0 += NB32) {
        int kb = Ns - k0 < NB32 ? Ns - k0 : NB32;
        {
            NQS_LAUNCH("chol32_diag");
            k_potrf_diag32<<<1, dim3(32, 32), 0, st>>>(w.T.p, Ns, k0, kb, w.status.p);
        }
        int k1 = k0 + kb, rest = Ns - k1;
        if (rest <= 0) break;
        {
            NQS_LAUNCH("chol32_panel");
            k_trsm_panel32<<<(rest + 127) / 128, 128, 0, st>>>(w.T.p, Ns, k0, kb, k1, w.status.p);
        }
        int ntt = (rest + TG32 - 1) / TG32;
        {
            NQS_LAUNCH("chol32_syrk");
            k_syrk_update32<<<ntt * (ntt + 1) / 2, 256, 0, st>>>(w.T.p, Ns, k0, kb, k1, w.status.p);
        }
    }
    int fail = -1, ierr = 0;
    if (!NQS_CUDA(cudaMemcpyAsync(&fail, w.status.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(&ierr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return false;
    if (ierr) {
        set_error("tensor-core Gram timed out waiting on its pipeline");
        return false;
    }
    *out_fail = fail;
    if (fail >= 0) return true;
    // X = L^{-1}
    for (int k0 = ((Ns - 1) / NB32) * NB32; k0 >= 0; k0 -= NB32) {
        int kb = Ns - k0 < NB32 ? Ns - k0 : NB32;
        {
            NQS_LAUNCH("trtri32_diag");
            k_trtri_diag32<<<1, 32, 0, st>>>(w.T.p, w.X.p, Ns, k0, kb);
        }
        int k1 = k0 + kb;
        if (k1 < Ns) {
            NQS_LAUNCH("trtri32_panel");
            k_trtri_panel32<<<(Ns - k1 + TG32 - 1) / TG32, 256, 0, st>>>(w.T.p, w.X.p, Ns, k0, kb, k1);
        }
    }
    // y = X^T X eps, then refinement sweeps against the FP64 operator
    dim3 cb(32, 8);
    unsigned gridN = (unsigned)((Ns + 31) / 32), gridP = (unsigned)((P + 31) / 32);
    unsigned rowsN = (unsigned)((Ns * 32 + 255) / 256);
    {
        NQS_LAUNCH("solve_gemv");
        k_trmv_lower<<<rowsN, 256, 0, st>>>(w.X.p, Ns, eps, w.w.p);
        k_trmv_lower_t<<<gridN, cb, 0, st>>>(w.X.p, Ns, w.w.p, y, nullptr);
    }
    for (int s = 0; s < sweeps; s++) {
        {
            NQS_LAUNCH("refine_residual");
            k_ct_dot<<<gridP, cb, 0, st>>>(O, Ns, P, y, w.u.p);
            k_residual<<<rowsN, 256, 0, st>>>(O, Ns, P, w.u.p, y, eps, shift, w.r.p);
        }
        {
            NQS_LAUNCH("solve_gemv");
            k_trmv_lower<<<rowsN, 256, 0, st>>>(w.X.p, Ns, w.r.p, w.w.p);
            k_trmv_lower_t<<<gridN, cb, 0, st>>>(w.X.p, Ns, w.w.p, nullptr, y);
        }
    }
    {
        NQS_LAUNCH("refine_residual");
        k_ct_dot<<<gridP, cb, 0, st>>>(O, Ns, P, y, w.u.p);
        k_residual<<<rowsN, 256, 0, st>>>(O, Ns, P, w.u.p, y, eps, shift, w.r.p);
        k_norms<<<1, 1024, 0, st>>>(w.r.p, eps, Ns, w.nrm.p);
    }
    double h[2];
    if (!NQS_CUDA(cudaMemcpyAsync(h, w.nrm.p, sizeof(h), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return false;
    *out_resid = h[1] > 0 ? sqrt(h[0] / h[1]) : 0.0;
    return NQS_CUDA(cudaGetLastError());
}

}  // namespace nqs

using namespace nqs;

extern "C" {

// Diagnostic: the tensor-core Gram alone on a host matrix O [Ns][P] (FP64,
// used as given, i.e. already centred): T_out [Ns][Ns] (lower triangle) =
// scale * (hi hi^T [+ hi lo^T + lo hi^T]).
int nqs_gpu_gram_tc(const double *O_host, int Ns, long P, int passes, double scale, float *T_out) {
    clear_error();
    if (!O_host || !T_out || Ns <= 0 || P <= 0) return -1;
    if (!ensure_context()) return -1;
    cudaStream_t st = ctx().stream;
    static DevBuf<double> dO, dz;
    if (!dO.ensure((size_t)Ns * P) || !dz.ensure((size_t)P)) return -1;
    if (!NQS_CUDA(cudaMemcpyAsync(dO.p, O_host, sizeof(double) * Ns * P, cudaMemcpyHostToDevice, st)) ||
        !NQS_CUDA(cudaMemsetAsync(dz.p, 0, sizeof(double) * P, st)))
        return -1;
    MixedWs &w = g_mx;
    const int ns_pad = (Ns + TC_M - 1) / TC_M * TC_M;
    const long p_pad = (P + TC_K - 1) / TC_K * TC_K;
    if (ns_pad != w.ns_pad || p_pad != w.p_pad) {
        if (!w.hi.ensure((size_t)ns_pad * p_pad) || !w.lo.ensure((size_t)ns_pad * p_pad)) return -1;
        NQS_CUDA(cudaMemsetAsync(w.hi.p, 0, sizeof(float) * ns_pad * p_pad, st));
        NQS_CUDA(cudaMemsetAsync(w.lo.p, 0, sizeof(float) * ns_pad * p_pad, st));
        w.ns_pad = ns_pad;
        w.p_pad = p_pad;
    }
    if (!w.T.ensure((size_t)Ns * Ns)) return -1;
    k_center_split<<<ctx().sm_count * 8, 256, 0, st>>>(dO.p, Ns, P, dz.p, w.hi.p, w.lo.p, p_pad);
    CUtensorMap mh, ml;
    if (!make_map(&mh, w.hi.p, ns_pad, p_pad) || !make_map(&ml, w.lo.p, ns_pad, p_pad)) return -1;
    static DevBuf<int> err;
    if (!err.ensure(1)) return -1;
    NQS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    GramTcArgs g;
    g.kt_per_seg = (int)(p_pad / TC_K);
    g.nseg = passes >= 3 ? 3 : 1;
    g.scale = (float)scale;
    g.shift = 0.f;
    g.C = w.T.p;
    g.n = Ns;
    g.err = err.p;
    if (!NQS_CUDA(cudaFuncSetAttribute(k_gram_tf32_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM)))
        return -1;
    int nt = ns_pad / TC_M;
    {
        NQS_LAUNCH("gram_tc");
        k_gram_tf32_tc<<<nt * (nt + 1) / 2, 128, TC_SMEM, st>>>(mh, ml, g);
    }
    int ierr = 0;
    if (!NQS_CUDA(cudaGetLastError()) ||
        !NQS_CUDA(cudaMemcpyAsync(T_out, w.T.p, sizeof(float) * (size_t)Ns * Ns, cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(&ierr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return -1;
    if (ierr) {
        set_error("tensor-core Gram timed out waiting on its pipeline");
        return -1;
    }
    return 0;
}

}  // extern "C"
