// Mixed-precision MinSR solve: tensor-core Gram, FP32 factor, FP64 refinement.
//
//   1. centre O in FP64 (in place) and split it into two TF32 words,
//      O_c = hi + lo (hi = tf32(O_c), lo = tf32(O_c - hi)), and in parameter
//      space also into two FP32 words (double-float) for the CG operator;
//   2. T = (hi hi^T + hi lo^T + lo hi^T) / N_s + shift I on the 5th-generation
//      tensor cores: tcgen05.mma kind::tf32 issued by one thread, the hi and lo
//      words of both row blocks staged by TMA (cp.async.bulk.tensor, 128-byte
//      swizzle) in a 3-stage mbarrier ring, the three products into one FP32
//      accumulator in TMEM read back with tcgen05.ld; only the lower-triangular
//      128 x 128 tiles are computed (K split in three when they are few);
//   3. FP32 blocked Cholesky T = L L^T with 64- or 128-wide diagonal blocks
//      (pipelined behind one CTA's chain of diagonal blocks) and the explicit
//      inverse L^{-1} built beside it, so each triangular solve is a GEMV;
//   4. FP64-accurate preconditioned CG with M = L L^T against the exact
//      operator A y = O_c (O_c^T y) / N_s + shift y (FP64, or double-float
//      words on the FP32 pipe in parameter space), to |r| / |rhs| <= 1e-10.
// When N_p < N_s the same update is solved in parameter space instead (the
// push-through identity O^T (O O^T / N_s + s)^{-1} = (O^T O / N_s + s)^{-1} O^T):
// the Gram is O_c^T O_c / N_s (N_p x N_p), the right-hand side O_c^T eps / N_s,
// and the CG operator A d = O_c^T (O_c d) / N_s + shift d.
// The achieved relative residual is returned.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <math.h>

#include "nqs_amp.cuh"
#include "nqs_tc.cuh"

namespace nqs {

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
        const float xf = (float)x;                  // x - xf (2^-24 relative) is below the split's 2^-21
        float h = tf32_rna(xf);
        float l = tf32_rna(xf - h);
        hi[i * ldp + k] = h;
        lo[i * ldp + k] = l;
    }
}

// ---------------------------------------------------------------- tensor-core Gram
constexpr int TC_M = 128, TC_N = 128, TC_K = 32;      // tile; K per stage = 128 B of FP32
static_assert(TC_M == TC_N, "operand tiles of both sides share one layout");
constexpr int TC_STAGES = 3;
constexpr int TC_TILE_BYTES = TC_M * TC_K * 4;       // one operand tile of one K stage (16 KB)
constexpr int TC_STAGE_BYTES = 4 * TC_TILE_BYTES;    // rows i: hi, lo; rows j: hi, lo
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 + 256;

struct GramTcArgs {
    int kt_total;         // K tiles of the whole reduction
    int kt_per_seg;       // K tiles per CTA: kt_total, or a third of it in a split launch
    int nseg;             // products: 1 = hi hi^T, 3 = hi hi^T + hi lo^T + lo hi^T
    float scale, shift;
    float *C;             // [n][n] lower triangle written
    int n;
    int *err;
    int split;            // 1: blockIdx.y = K segment, raw partial sums into C + segment * n * n
};

// One 128 x 128 lower-triangular tile of hi hi^T (+ hi lo^T + lo hi^T) per CTA.  Each K stage
// brings the hi and lo words of both row blocks once (one pair when the tile is diagonal) and
// all products of the stage accumulate into one FP32 TMEM accumulator.
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
    const int kt0 = g.split ? (int)blockIdx.y * g.kt_per_seg : 0;
    const int total = max(0, min(g.kt_total, kt0 + g.kt_per_seg) - kt0);
    const bool three = g.nseg >= 3, diag = bi == bj;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // TMA producer: stage layout [rows i hi][rows i lo][rows j hi][rows j lo]
        const uint32_t tx = (uint32_t)TC_TILE_BYTES * (three ? 2u : 1u) * (diag ? 1u : 2u);
        for (int it = 0; it < total && ok; it++) {
            int s = it % TC_STAGES, u = it / TC_STAGES;
            if (u > 0) ok = mbar_wait(&empty[s], (u - 1) & 1, g.err);
            if (!ok) break;
            const int kc = (kt0 + it) * TC_K;
            uint8_t *sa = sm + s * TC_STAGE_BYTES;
            mbar_expect_tx(&full[s], tx);
            tma_load_2d(sa, &map_hi, &full[s], kc, bi * TC_M);
            if (three) tma_load_2d(sa + TC_TILE_BYTES, &map_lo, &full[s], kc, bi * TC_M);
            if (!diag) {
                tma_load_2d(sa + 2 * TC_TILE_BYTES, &map_hi, &full[s], kc, bj * TC_N);
                if (three) tma_load_2d(sa + 3 * TC_TILE_BYTES, &map_lo, &full[s], kc, bj * TC_N);
            }
        }
    } else if (warp == 1 && lane == 0 && total > 0) {
        // MMA issuer: M = N = 128, K = 8 per instruction, 4 per stage and product
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);
        for (int it = 0; it < total && ok; it++) {
            int s = it % TC_STAGES, u = it / TC_STAGES;
            ok = mbar_wait(&full[s], u & 1, g.err);
            if (!ok) break;
            tc_fence_after();
            const uint32_t ah = smem_u32(sm + s * TC_STAGE_BYTES), al = ah + TC_TILE_BYTES;
            const uint32_t bh = diag ? ah : ah + 2 * TC_TILE_BYTES, bl = diag ? al : ah + 3 * TC_TILE_BYTES;
#pragma unroll
            for (int k = 0; k < TC_K / 8; k++)
                umma_tf32(tmem, sw128_desc(ah + k * 32), sw128_desc(bh + k * 32), idesc,
                          (it > 0 || k > 0) ? 1u : 0u);
            if (three) {
#pragma unroll
                for (int k = 0; k < TC_K / 8; k++) {
                    umma_tf32(tmem, sw128_desc(ah + k * 32), sw128_desc(bl + k * 32), idesc, 1u);
                    umma_tf32(tmem, sw128_desc(al + k * 32), sw128_desc(bh + k * 32), idesc, 1u);
                }
            }
            umma_commit(&empty[s]);
        }
        umma_commit(done);
    }
    __syncwarp();
    // epilogue: warp w owns TMEM lanes (rows) 32w .. 32w+31; an empty K segment writes zeros
    bool ready = total > 0 ? mbar_wait(done, 0, g.err) : true;
    tc_fence_after();
    if (ready) {
        const int row = bi * TC_M + warp * 32 + lane;
        for (int c = 0; c < TC_N / 32; c++) {
            float v[32];
            if (total > 0) {
                tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
            } else {
#pragma unroll
                for (int j = 0; j < 32; j++) v[j] = 0.f;
            }
            int col0 = bj * TC_N + c * 32;
            if (row < g.n && g.split) {
                float *dst = g.C + (size_t)blockIdx.y * g.n * g.n + (size_t)row * g.n;
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int col = col0 + j;
                    if (col <= row && col < g.n) dst[col] = v[j];
                }
            } else if (row < g.n) {
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

// T = scale ((P0 + P1) + P2) + shift I on the lower triangle, from the three
// K-segment partial Grams of a split launch (rows dealt to the blocks, columns c <= r to
// the threads).
__global__ void k_gram_sum(const float *__restrict__ Pp, int n, float scale, float shift, float *T) {
    const size_t nn = (size_t)n * n;
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const size_t e0 = (size_t)r * n;
        for (int c = threadIdx.x; c <= r; c += blockDim.x) {
            const size_t e = e0 + c;
            T[e] = ((Pp[e] + Pp[nn + e]) + Pp[2 * nn + e]) * scale + (r == c ? shift : 0.f);
        }
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

// ---------------------------------------------------------------- double-float arithmetic
// The FP64 pipe of this GPU issues two FMAs per clock per SM, the FP32 pipe 128: sums that
// need FP64 accuracy over many terms run on the FP32 pipe as unevaluated pairs hi + lo
// (a 48-bit significand).  df_fma: s += a b with the exact product of the high words from
// an FMA (Dekker's two-product), the cross terms a_hi b_lo + a_lo b_hi in FP32 (a_lo b_lo,
// 2^-48 relative, is dropped), and the sum by Knuth's two-sum with its rounding error
// carried in lo.  df_add: s += b, renormalised.  Explicit _rn intrinsics keep the compiler
// from contracting or reordering the error terms.
__device__ __forceinline__ void df_fma(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = __fadd_rn(sh, p);
    const float bb = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}
__device__ __forceinline__ void df_add(float &sh, float &sl, float bh, float bl) {
    const float t = __fadd_rn(sh, bh);
    const float bb = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(bh, bb));
    const float lo = __fadd_rn(err, __fadd_rn(sl, bl));
    sh = __fadd_rn(t, lo);
    sl = __fsub_rn(lo, __fsub_rn(sh, t));
}
// x as two FP32 words h + l, h = x truncated to 24 significant bits and l = the remainder
// rounded to FP32 (|x - h - l| <= 2^-48 |x|), built from the bits of x on the integer and FP32
// pipes for 2^-113 <= |x| < 2^78; other values (zero included) go through FP64 conversions.
// The FP64 pipe of this GPU is 1/64 of the FP32 pipe, and conversions from FP64 run on it.
__device__ __forceinline__ void split_f64_words(double x, float &h, float &l) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7FF);
    if (E >= 910 && E <= 1100) {
        const unsigned sg = (unsigned)(b >> 63) << 31;
        const unsigned long long M = b & ((1ull << 52) - 1);
        h = __uint_as_float(sg | ((unsigned)(E - 896) << 23) | (unsigned)(M >> 29));
        const float sc = __uint_as_float((unsigned)(E - 908) << 23);          // 2^(E - 1075 + 40)
        const float r = __fmul_rn(__fmul_rn(__uint2float_rn((unsigned)(M & 0x1FFFFFFFull)), sc), 0x1p-40f);
        l = __uint_as_float(__float_as_uint(r) | sg);
    } else {
        h = __double2float_rn(x);
        l = __double2float_rn(x - (double)h);
    }
}

// The parameter-space operator runs in double-float when N_p is a multiple of 4 (float4
// rows) and at most 2048 (two four-column groups per thread).
__host__ __device__ inline bool df_words_ok(long P) { return (P & 3) == 0 && P <= 8 * 256; }
// Rows per chunk of the double-float operator: one chunk per SM at full grid, at least 8.
static int df_chunk_rows(int Ns) { return std::max(8, (Ns + ctx().sm_count - 1) / ctx().sm_count); }

// ---------------------------------------------------------------- FP32 factor, inverse and refinement
// One cooperative launch (one CTA per SM, all co-resident) runs everything
// after the Gram:
//   factor   for each BD-column block k (BD = 64 or 128): the owner CTA factors the
//            diagonal block in shared memory and inverts it (X_kk = L_kk^{-1}); every
//            CTA forms 64 x 64 tiles of the panel U_k = X_kk A_k^T (stored as L^T in
//            the unused upper triangle of T), then 128 x 128 tensor-core tiles of the
//            trailing update A -= U_k^T U_k (lower triangle), while the owner updates
//            and factors the next diagonal block (look-ahead); with 64-wide blocks on
//            four CTAs or more the owner runs a whole step ahead of the others, bound to
//            them by flags instead of grid barriers (the pipelined factor in fr_body);
//   inverse  L^{-1} beside the factor, by block rows: in the panel phase of step k
//            row block k of X = L^{-1} is X_kk R_k (R = I - L X over the eliminated
//            columns, accumulated in Li), in the trailing phase the rows below take
//            R -= L_{:,k} X_k on the tensor cores; L^{-1} is kept row-major (Li) and
//            transposed (LiT) so both triangular solves are row GEMVs;
//   refine   preconditioned CG on the exact operator (two passes over O_c per product:
//            double-float arithmetic on the FP32 pipe in parameter space, FP64 otherwise),
//            preconditioner L^{-T} L^{-1} in FP32.
// Phases are separated by a grid barrier on a monotonic arrival counter with a bounded
// spin budget; on timeout it raises *err and every CTA leaves at its next barrier.
// Data written by other CTAs is read with L1-bypassing loads.
constexpr int BT = 128;                              // shared-memory tile of the diagonal block
// Diagonal block width BD (a template parameter of the factor; chosen per
// system): 64 below BD_SWITCH, where the sequential chain of diagonal blocks
// dominates, 128 above, where wider tensor-core K and half the block steps pay.
constexpr int BD_SMALL = 64, BD_LARGE = 128, BD_SWITCH = 4096;
static_assert(BD_SMALL % 64 == 0 && BD_LARGE <= BT, "diagonal blocks are multiples of the 64-wide GEMM tile");
constexpr int PS_THREADS = 256;
constexpr int DF_G = 9;           // four-column groups per lane in flight in a row dot of the operator
constexpr int DF_SEGS = 4;        // row segments of a chunk at most in the operator's column sums
constexpr int PS_SMEM = 2 * BT * (BT + 1) * 4;       // two 128 x 129 float tiles
constexpr int GT = 64, GKC = 32;                     // GEMM tile and K chunk
constexpr int RCH = 64;                              // rows per partial column sum

struct TileSmem {
    float a[GKC][GT + 1];
    float b[GKC][GT + 1];
};

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Polls a grid barrier waits before it gives up (raising *err = 2).  A device variable so
// that graph replays read the current value; nqs_gpu_set_barrier_budget() lowers it for
// the tests of the timeout path.
__device__ unsigned g_barrier_budget = 1u << 24;

// A monotonic arrival counter (bar[0], cleared at every launch): the arrival that returns
// old belongs to barrier instance old / count, which is passed once the counter reaches
// (old / count + 1) * count, so no reset and no second word is needed (a CTA can only
// arrive at the next instance after all arrivals of this one).  Ordering: the block
// barrier, then an acq_rel fence at GPU scope around the relaxed atomic and the polls.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err, unsigned count) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned budget = *(volatile unsigned *)&g_barrier_budget;
        unsigned old;
        asm volatile("fence.acq_rel.gpu;\n\tatom.relaxed.gpu.global.add.u32 %0, [%1], 1;"
                     : "=r"(old) : "l"(bar) : "memory");
        const unsigned target = (old / count + 1u) * count;
        uint32_t it = 0;
        for (;;) {
            unsigned cur;
            asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(bar) : "memory");
            if ((int)(cur - target) >= 0) break;
            if (++it > budget) {
                atomicExch(err, 2);
                break;
            }
            if ((it & 31) == 0) {                       // the error word every 32nd poll only
                if (*((volatile int *)err)) break;
                if (it > 256) __nanosleep(32);
            }
        }
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        s_ok = *((volatile int *)err) == 0;
    }
    __syncthreads();
    return s_ok != 0;                                 // one answer for the whole CTA
}

// Factor the 128 x 128 block in S (rows >= bs padded with the identity) in four
// 32-column sub-panels and leave the inverses of the four diagonal 32 x 32
// factors in the matching diagonal blocks of X.  The 32 x 32 factor and its
// inverse run in one warp's registers; the panel below it and the update of the
// rest of the block use the whole CTA.  Returns the first failing column or -1.
template <int BD>
__device__ int block_chol(float (*S)[BT + 1], float (*X)[BT + 1], int bs, int *s_flag, float *tmp) {
    constexpr int NSUB = BD / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int e = tid; e < BD * BD; e += PS_THREADS) X[e / BD][e % BD] = 0.f;
    for (int sb = 0; sb < NSUB; sb++) {
        const int c0 = sb * 32;
        if (warp == 0) {
            // right-looking, lane = row in registers; the scaled column j is
            // broadcast through shared memory (a shuffle per entry is ~3x slower)
            // Lane = row; column j of L is broadcast by shuffles.  Branch-free:
            // every lane updates its whole row, and the entries right of a lane's
            // diagonal (zero on entry) become scratch that nothing reads (lane i's
            // row[c], c > i, is only broadcast at steps j = c > i, which read lanes
            // c' > j only).  A non-positive pivot records the first failing column
            // and continues on a unit pivot; the block is discarded then.  (With
            // a per-entry `c <= lane` guard this loop ran ~4x slower.)
            float row[32];
#pragma unroll
            for (int c = 0; c < 32; c++) row[c] = S[c0 + lane][c0 + c];
            int fail = -1;
            float dinv = 0.f;                                  // lane j keeps 1 / L_jj
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const float d = __shfl_sync(0xffffffffu, row[j], j);
                const bool ok = d > 0.f;
                fail = (fail < 0 && !ok) ? j : fail;
                const float inv = rsqrtf(ok ? d : 1.f);
                row[j] *= inv;                                 // lane j: d / sqrt(d) = L_jj
                dinv = lane == j ? inv : dinv;
                const float lrj = row[j];                     // L[lane][j]
#pragma unroll
                for (int c = j + 1; c < 32; c++) row[c] = fmaf(-lrj, __shfl_sync(0xffffffffu, lrj, c), row[c]);
            }
#pragma unroll
            for (int c = 0; c < 32; c++)
                if (c <= lane) S[c0 + lane][c0 + c] = row[c];
            if (lane == 0) *s_flag = (fail >= 0 && c0 + fail < bs) ? c0 + fail : -1;
            __syncwarp();
            if (fail < 0) {
                // X_s = L_s^{-1} by forward substitution, lane = column
                float x[32];
#pragma unroll
                for (int rr = 0; rr < 32; rr++) {
                    const float di = __shfl_sync(0xffffffffu, dinv, rr);
                    float s0 = (rr == lane) ? 1.f : 0.f, s1 = 0.f;
#pragma unroll
                    for (int m = 0; m < rr; m += 2) {
                        s0 -= S[c0 + rr][c0 + m] * x[m];
                        if (m + 1 < rr) s1 -= S[c0 + rr][c0 + m + 1] * x[m + 1];
                    }
                    x[rr] = rr < lane ? 0.f : (s0 + s1) * di;
                }
#pragma unroll
                for (int rr = 0; rr < 32; rr++) X[c0 + rr][c0 + lane] = x[rr];
            }
        }
        __syncthreads();
        if (*s_flag >= 0) return *s_flag;
        const int t0 = c0 + 32, nr = BD - t0;
        if (nr == 0) break;
        // rows below the sub-panel: L[r][c0+j] = sum_m A[r][c0+m] X_s[j][m]
        for (int w = tid; w < nr * 8; w += PS_THREADS) {
            const int r = t0 + w / 8, j0 = (w % 8) * 4;
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 8
            for (int m = 0; m < 32; m++) {
                float av = S[r][c0 + m];
                a0 += av * X[c0 + j0][c0 + m];
                a1 += av * X[c0 + j0 + 1][c0 + m];
                a2 += av * X[c0 + j0 + 2][c0 + m];
                a3 += av * X[c0 + j0 + 3][c0 + m];
            }
            tmp[w * 4 + 0] = a0;
            tmp[w * 4 + 1] = a1;
            tmp[w * 4 + 2] = a2;
            tmp[w * 4 + 3] = a3;
        }
        __syncthreads();
        for (int w = tid; w < nr * 8; w += PS_THREADS) {
            const int r = t0 + w / 8, j0 = (w % 8) * 4;
#pragma unroll
            for (int q = 0; q < 4; q++) S[r][c0 + j0 + q] = tmp[w * 4 + q];
        }
        __syncthreads();
        // rest of the block: S[i][j] -= sum_m L[i][c0+m] L[j][c0+m], 4 x 4 outputs
        // per thread on rows / columns strided by nr / 4
        const int q = nr / 4;
        for (int e = tid; e < q * q; e += PS_THREADS) {
            const int ti = e / q, tj = e % q;
            float acc[4][4] = {};
#pragma unroll 4
            for (int m = 0; m < 32; m++) {
                float av[4], bv[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    av[u] = S[t0 + ti + q * u][c0 + m];
                    bv[u] = S[t0 + tj + q * u][c0 + m];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const int i = t0 + ti + q * u, j = t0 + tj + q * v;
                    if (j <= i) S[i][j] -= acc[u][v];
                }
        }
        __syncthreads();
    }
    return -1;
}

// The 64 x 64 diagonal block, Cholesky and X = L^{-1} in one right-looking sweep over
// four-column panels with the block in registers: thread (w, l) = (tid / 32, tid % 32)
// holds rows i = w + 8u (u < 8) and columns c = l + 32v (v < 2) of S and of
// R = I - L X (forward substitution of L X = I, right-looking).  At panel j0 the owners
// publish the four pivot columns S[i][j0 .. j0+3] (i >= j0) and rows j0 .. j0+3 of R into
// shared memory (double-buffered: one block barrier per panel); every thread factors the
// 4 x 4 pivot block P = Lp Lp^T and inverts Lp (Ip = Lp^{-1}) itself, then
//   l_i = Ip S[i][j0..j0+3]^T (i > j0 + 3; lane 4u + q forms component q of its warp's row
//         w + 8u and the warp exchanges them by shuffles),
//   l_c = Ip S[c][j0..j0+3]^T (c > j0 + 3), x_c = Ip R[j0..j0+3][c] (c <= j0 + 3),
//   S_ic -= l_i . l_c, R_ic -= l_i . x_c, and rows j0 .. j0+3 of R become rows of X.
// Entries above the diagonal of S take values nothing reads.  S (rows >= bs padded with
// the identity) is read once; X (zeros above the diagonal) is written to X.  Returns the
// first non-positive pivot column below bs or -1 (the sweep goes on with a unit pivot; the
// caller discards the block).  buf: 1024 floats.
__device__ int block_chol_inv64(const float (*S)[BT + 1], float (*X)[BT + 1], int bs, float *buf) {
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    float s[8][2], r[8][2];
#pragma unroll
    for (int u = 0; u < 8; u++)
#pragma unroll
        for (int v = 0; v < 2; v++) {
            const int i = w + 8 * u, c = l + 32 * v;
            s[u][v] = S[i][c];
            r[u][v] = i == c ? 1.f : 0.f;
        }
    int fail = -1;
    const int lu = l >> 2, lq = l & 3;                       // this lane's (row, component) of l_i
#pragma unroll
    for (int jv = 0; jv < 2; jv++)
        for (int jj0 = 0; jj0 < 32; jj0 += 4) {
            const int j0 = 32 * jv + jj0, w0 = j0 & 7, ju = j0 >> 3;
            float *cb = buf + ((j0 >> 2) & 1) * 512, *rb = cb + 256;   // cb[q * 64 + i], rb[a * 64 + c]
            {
                const int q = l - jj0;
                if (q >= 0 && q < 4) {
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        if (w + 8 * u >= j0) cb[q * 64 + w + 8 * u] = s[u][jv];
                }
                const int a = w - w0;
                if (a >= 0 && a < 4) {
#pragma unroll
                    for (int v = 0; v < 2; v++) {
                        float x = 0.f;
#pragma unroll
                        for (int u = 0; u < 8; u++) x = u == ju ? r[u][v] : x;
                        if (l + 32 * v <= j0 + 3) rb[a * 64 + l + 32 * v] = x;
                    }
                }
            }
            __syncthreads();
            // the pivot block, its factor Lp and Ip = Lp^{-1} (every thread)
            float P[4][4], Lp[4][4], Ip[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b <= a; b++) P[a][b] = cb[b * 64 + j0 + a];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                float d = P[a][a];
#pragma unroll
                for (int b = 0; b < a; b++) d = fmaf(-Lp[a][b], Lp[a][b], d);
                const bool ok = d > 0.f;
                if (!ok && fail < 0 && j0 + a < bs) fail = j0 + a;
                const float inv = rsqrtf(ok ? d : 1.f);
                Lp[a][a] = (ok ? d : 1.f) * inv;
                Ip[a][a] = inv;
#pragma unroll
                for (int e = a + 1; e < 4; e++) {
                    float t = P[e][a];
#pragma unroll
                    for (int b = 0; b < a; b++) t = fmaf(-Lp[e][b], Lp[a][b], t);
                    Lp[e][a] = t * inv;
                }
            }
#pragma unroll
            for (int e = 1; e < 4; e++)
#pragma unroll
                for (int a = 0; a < e; a++) {
                    float t = 0.f;
#pragma unroll
                    for (int b = a; b < e; b++) t = fmaf(Lp[e][b], Ip[b][a], t);
                    Ip[e][a] = -Ip[e][e] * t;
                }
            // l_i: lane (lu, lq) forms component lq of row w + 8 lu; the warp gathers them by
            // shuffles below, for the rows still below the panel only (a warp-uniform test)
            float z = 0.f;
            {
                const int i = w + 8 * lu;
                if (i > j0 + 3) {
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        float ip = 0.f;
#pragma unroll
                        for (int q = 0; q < 4; q++) ip = (q == lq && b <= q) ? Ip[q][b] : ip;
                        z = fmaf(ip, cb[b * 64 + i], z);
                    }
                }
            }
            // l_c (columns below the panel) and x_c (columns up to it): in the first half
            // (jv = 0) columns 32.. are all below the panel, in the second columns ..31 all
            // above it, so those halves are known at compile time
            float lc[2][4], xc[2][4];
#pragma unroll
            for (int v = 0; v < 2; v++) {
                const int c = l + 32 * v;
                const bool below = v > jv || (v == jv && c > j0 + 3);
                float y[4];
#pragma unroll
                for (int b = 0; b < 4; b++) y[b] = below ? cb[b * 64 + c] : rb[b * 64 + c];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    float t = 0.f;
#pragma unroll
                    for (int b = 0; b <= q; b++) t = fmaf(Ip[q][b], y[b], t);
                    lc[v][q] = below ? t : 0.f;
                    xc[v][q] = below ? 0.f : t;
                }
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                if (w + 8 * u <= j0 + 3) continue;          // rows done (warp-uniform)
                float li[4];
#pragma unroll
                for (int q = 0; q < 4; q++) li[q] = __shfl_sync(0xffffffffu, z, 4 * u + q);
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    if (v >= jv) {                          // S: columns that can lie below the panel
                        float ds = 0.f;
#pragma unroll
                        for (int q = 0; q < 4; q++) ds = fmaf(li[q], lc[v][q], ds);
                        s[u][v] -= ds;
                    }
                    if (v <= jv) {                          // R: columns that can lie up to the panel
                        float dr = 0.f;
#pragma unroll
                        for (int q = 0; q < 4; q++) dr = fmaf(li[q], xc[v][q], dr);
                        r[u][v] -= dr;
                    }
                }
            }
            {
                const int a = w - w0;                        // rows j0 .. j0+3 of R become rows of X
                if (a >= 0 && a < 4) {
#pragma unroll
                    for (int v = 0; v <= jv; v++) {
                        float x = 0.f;
#pragma unroll
                        for (int q = 0; q < 4; q++) x = q == a ? xc[v][q] : x;
#pragma unroll
                        for (int u = 0; u < 8; u++) r[u][v] = u == ju ? x : r[u][v];
                    }
                }
            }
        }
#pragma unroll
    for (int u = 0; u < 8; u++)
#pragma unroll
        for (int v = 0; v < 2; v++) X[w + 8 * u][l + 32 * v] = r[u][v];
    __syncthreads();
    return fail;
}

// Off-diagonal 32-blocks of X = L^{-1} inside the 128-block (the diagonal
// 32-blocks are already in X): for d = 1..3, X_ba = -X_bb (sum_{m=a}^{b-1}
// L_bm X_ma), b = a + d, all pairs of one block diagonal computed by the CTA,
// 4 x 4 outputs per thread (rows and columns strided by 8).
template <int BD>
__device__ void block_inv(float (*S)[BT + 1], float (*X)[BT + 1], float *tmp) {
    constexpr int NSUB = BD / 32;
    const int tid = threadIdx.x, r8 = (tid >> 3) & 7, c8 = tid & 7;
    for (int d = 1; d < NSUB; d++) {
        const int pairs = NSUB - d;
        for (int w = tid; w < pairs * 64; w += PS_THREADS) {
            const int pa = w >> 6, ob = (pa + d) * 32, oa = pa * 32;
            float acc[4][4] = {};
#pragma unroll 4
            for (int m = oa; m < ob; m++) {
                float sv[4], xv[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    sv[u] = S[ob + r8 + 8 * u][m];
                    xv[u] = X[m][oa + c8 + 8 * u];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = fmaf(sv[u], xv[v], acc[u][v]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) tmp[pa * 1024 + (r8 + 8 * u) * 32 + c8 + 8 * v] = acc[u][v];
        }
        __syncthreads();
        for (int w = tid; w < pairs * 64; w += PS_THREADS) {
            const int pa = w >> 6, ob = (pa + d) * 32, oa = pa * 32;
            float acc[4][4] = {};
#pragma unroll 4
            for (int m = 0; m < 32; m++) {              // X_bb is lower triangular (zeros above)
                float xv[4], tv[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    xv[u] = X[ob + r8 + 8 * u][ob + m];
                    tv[u] = tmp[pa * 1024 + m * 32 + c8 + 8 * u];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = fmaf(xv[u], tv[v], acc[u][v]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) X[ob + r8 + 8 * u][oa + c8 + 8 * v] = -acc[u][v];
        }
        __syncthreads();
    }
}

// GEMM tile: acc[u][v] += sum_{m in [kb, ke)} A(r0 + ty + 16u, m) B(c0 + tx + 16v, m)
// (tx = tid % 16, ty = tid / 16).  An operand is row-major in its row index
// (RM: X(x, m) at p[x * ld + m]) or in the K index (KM: X(x, m) at p[m * ld + x]);
// rows at or beyond xlim read as zero.  K chunks of 32 go through shared memory
// with the next chunk prefetched in registers.
template <bool KM>
__device__ __forceinline__ void tile_fetch(float (&v)[8], const float *p, long ld, int x0, int xlim, int m0, int ke) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int e = threadIdx.x + PS_THREADS * q;
        const int m = KM ? (e >> 6) : (e & 31), x = KM ? (e & 63) : (e >> 5);
        const int gm = m0 + m, gx = x0 + x;
        v[q] = (gm < ke && gx < xlim) ? __ldcg(p + (KM ? (size_t)gm * ld + gx : (size_t)gx * ld + gm)) : 0.f;
    }
}

template <bool KM>
__device__ __forceinline__ void tile_put(float (*s)[GT + 1], const float (&v)[8]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int e = threadIdx.x + PS_THREADS * q;
        const int m = KM ? (e >> 6) : (e & 31), x = KM ? (e & 63) : (e >> 5);
        s[m][x] = v[q];
    }
}

template <bool AKM, bool BKM>
__device__ void gemm64(float (&acc)[4][4], const float *A, long lda, int r0, int rlim, const float *B, long ldb,
                       int c0, int clim, int kb, int ke, TileSmem &S) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    if (kb >= ke) return;
    float va[8], vb[8];
    tile_fetch<AKM>(va, A, lda, r0, rlim, kb, ke);
    tile_fetch<BKM>(vb, B, ldb, c0, clim, kb, ke);
    for (int k = kb; k < ke; k += GKC) {
        __syncthreads();
        tile_put<AKM>(S.a, va);
        tile_put<BKM>(S.b, vb);
        __syncthreads();
        if (k + GKC < ke) {
            tile_fetch<AKM>(va, A, lda, r0, rlim, k + GKC, ke);
            tile_fetch<BKM>(vb, B, ldb, c0, clim, k + GKC, ke);
        }
#pragma unroll 8
        for (int m = 0; m < GKC; m++) {
            float a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                a[u] = S.a[m][ty + 16 * u];
                b[u] = S.b[m][tx + 16 * u];
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void tri_tile(int t, int &bi, int &bj) {
    int r = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((r + 1) * (r + 2) / 2 <= t) r++;
    while (r * (r + 1) / 2 > t) r--;
    bi = r;
    bj = t - r * (r + 1) / 2;
}

// Partial column sums upart[ch][k] = sum_{i in chunk ch} O[i][k] v[i] (RCH rows
// per chunk).  Even N_p: one warp per (chunk, 64 columns), double2 loads, 16
// rows in flight per lane; odd N_p: one warp per (chunk, 32 columns).
__device__ __forceinline__ void colsum_partial(const double *O, int Ns, long P, const double *v, double *upart,
                                               int gwarp, int gwarps, int lane) {
    const int nch = (Ns + RCH - 1) / RCH;
    if ((P & 1) == 0) {
        const long P2 = P >> 1, ncg = (P2 + 31) / 32;
        const double2 *O2 = (const double2 *)O;
        for (long w = gwarp; w < (long)nch * ncg; w += gwarps) {
            const int ch = (int)(w / ncg);
            const long k2 = (w % ncg) * 32 + lane;
            const int i0 = ch * RCH, i1 = min(Ns, i0 + RCH);
            double ax = 0.0, ay = 0.0, bx = 0.0, by = 0.0;
            if (k2 < P2) {
                int i = i0;
                for (; i + 15 < i1; i += 16) {
                    double2 o[16];
#pragma unroll
                    for (int q = 0; q < 16; q++) o[q] = O2[(size_t)(i + q) * P2 + k2];
#pragma unroll
                    for (int q = 0; q < 16; q += 2) {
                        const double v0 = __ldcg(v + i + q), v1 = __ldcg(v + i + q + 1);
                        ax += o[q].x * v0;
                        ay += o[q].y * v0;
                        bx += o[q + 1].x * v1;
                        by += o[q + 1].y * v1;
                    }
                }
                for (; i < i1; i++) {
                    const double2 o = O2[(size_t)i * P2 + k2];
                    const double vi = __ldcg(v + i);
                    ax += o.x * vi;
                    ay += o.y * vi;
                }
                upart[(size_t)ch * P + 2 * k2] = ax + bx;
                upart[(size_t)ch * P + 2 * k2 + 1] = ay + by;
            }
        }
        return;
    }
    const long ncg = (P + 31) / 32;
    for (long w = gwarp; w < (long)nch * ncg; w += gwarps) {
        const int ch = (int)(w / ncg);
        const long k = (w % ncg) * 32 + lane;
        const int i0 = ch * RCH, i1 = min(Ns, i0 + RCH);
        double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (k < P) {
            int i = i0;
            for (; i + 7 < i1; i += 8) {
#pragma unroll
                for (int q = 0; q < 8; q++) acc[q] += O[(size_t)(i + q) * P + k] * __ldcg(v + i + q);
            }
            for (; i < i1; i++) acc[0] += O[(size_t)i * P + k] * __ldcg(v + i);
            upart[(size_t)ch * P + k] = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
        }
    }
}

__device__ __forceinline__ double colsum_reduce(const double *upart, int Ns, long P, long k, int lane) {
    const int nch = (Ns + RCH - 1) / RCH;
    double acc = 0.0;
    for (int ch = lane; ch < nch; ch += 32) acc += __ldcg(upart + (size_t)ch * P + k);
    return warp_sum(acc);
}

// o . v for one row of O (N_p doubles), one warp.  v is either in shared
// memory or (GV) in global memory written by other CTAs (L1-bypassing loads).
template <bool GV>
__device__ __forceinline__ double ldv(const double *p) { return GV ? __ldcg(p) : *p; }
template <bool GV>
__device__ __forceinline__ double2 ldv2(const double2 *p) { return GV ? __ldcg(p) : *p; }

template <bool GV>
__device__ __forceinline__ double rowdot(const double *o, long P, const double *v, int lane) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if ((P & 1) == 0) {                                  // rows 16-byte aligned: double2 loads
        const double2 *o2 = (const double2 *)o, *v2 = (const double2 *)v;
        const long P2 = P >> 1;
        long k = lane;
        for (; k + 224 < P2; k += 256) {
            double2 x[8];
#pragma unroll
            for (int q = 0; q < 8; q++) x[q] = o2[k + 32 * q];
#pragma unroll
            for (int q = 0; q < 8; q += 2) {
                const double2 y0 = ldv2<GV>(v2 + k + 32 * q), y1 = ldv2<GV>(v2 + k + 32 * q + 32);
                a0 += x[q].x * y0.x;
                a1 += x[q].y * y0.y;
                a2 += x[q + 1].x * y1.x;
                a3 += x[q + 1].y * y1.y;
            }
        }
        for (; k < P2; k += 32) {
            const double2 x0 = o2[k], y0 = ldv2<GV>(v2 + k);
            a0 += x0.x * y0.x;
            a1 += x0.y * y0.y;
        }
    } else {
        long k = lane;
        for (; k + 96 < P; k += 128) {
            a0 += o[k] * ldv<GV>(v + k);
            a1 += o[k + 32] * ldv<GV>(v + k + 32);
            a2 += o[k + 64] * ldv<GV>(v + k + 64);
            a3 += o[k + 96] * ldv<GV>(v + k + 96);
        }
        for (; k < P; k += 32) a0 += o[k] * ldv<GV>(v + k);
    }
    return warp_sum((a0 + a1) + (a2 + a3));
}

// Stage the N_p-vector v (written by other CTAs) in shared memory when it fits
// (the caller has passed a barrier since the last use of psm); returns where to
// read it.
__device__ __forceinline__ const double *stage_vec(const double *v, long P, double *smem, long cap) {
    if (P > cap) return v;
    for (long k = threadIdx.x; k < P; k += PS_THREADS) smem[k] = __ldcg(v + k);
    __syncthreads();
    return smem;
}

// sum over the float4 groups [g0, g1) of row . v, one warp, result in every lane
__device__ __forceinline__ float dot4_range(const float *row, const float *v, int g0, int g1, int lane) {
    const float4 *r4 = (const float4 *)row, *v4 = (const float4 *)v;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int g = g0 + lane;
    for (; g + 96 < g1; g += 128) {
        const float4 x0 = __ldcg(r4 + g), x1 = __ldcg(r4 + g + 32), x2 = __ldcg(r4 + g + 64),
                     x3 = __ldcg(r4 + g + 96);
        const float4 y0 = __ldcg(v4 + g), y1 = __ldcg(v4 + g + 32), y2 = __ldcg(v4 + g + 64),
                     y3 = __ldcg(v4 + g + 96);
        s0 += (x0.x * y0.x + x0.y * y0.y) + (x0.z * y0.z + x0.w * y0.w);
        s1 += (x1.x * y1.x + x1.y * y1.y) + (x1.z * y1.z + x1.w * y1.w);
        s2 += (x2.x * y2.x + x2.y * y2.y) + (x2.z * y2.z + x2.w * y2.w);
        s3 += (x3.x * y3.x + x3.y * y3.y) + (x3.z * y3.z + x3.w * y3.w);
    }
    for (; g < g1; g += 32) {
        const float4 x0 = __ldcg(r4 + g), y0 = __ldcg(v4 + g);
        s0 += (x0.x * y0.x + x0.y * y0.y) + (x0.z * y0.z + x0.w * y0.w);
    }
    float t = (s0 + s1) + (s2 + s3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// The same with v in shared memory.
__device__ __forceinline__ float dot4_range_sv(const float *row, const float *v, int g0, int g1, int lane) {
    const float4 *r4 = (const float4 *)row, *v4 = (const float4 *)v;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int g = g0 + lane;
    for (; g + 96 < g1; g += 128) {
        const float4 x0 = __ldcg(r4 + g), x1 = __ldcg(r4 + g + 32), x2 = __ldcg(r4 + g + 64),
                     x3 = __ldcg(r4 + g + 96);
        const float4 y0 = v4[g], y1 = v4[g + 32], y2 = v4[g + 64], y3 = v4[g + 96];
        s0 += (x0.x * y0.x + x0.y * y0.y) + (x0.z * y0.z + x0.w * y0.w);
        s1 += (x1.x * y1.x + x1.y * y1.y) + (x1.z * y1.z + x1.w * y1.w);
        s2 += (x2.x * y2.x + x2.y * y2.y) + (x2.z * y2.z + x2.w * y2.w);
        s3 += (x3.x * y3.x + x3.y * y3.y) + (x3.z * y3.z + x3.w * y3.w);
    }
    for (; g < g1; g += 32) {
        const float4 x0 = __ldcg(r4 + g), y0 = v4[g];
        s0 += (x0.x * y0.x + x0.y * y0.y) + (x0.z * y0.z + x0.w * y0.w);
    }
    float t = (s0 + s1) + (s2 + s3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// a . b and a . c over [0, n), computed by every CTA in the same fixed order (four
// thread-strided partial sums with their loads issued together, a warp butterfly, then
// the warps in order), so that all CTAs hold the same values whatever the grid size.
template <bool TWO>
__device__ __forceinline__ double2 dot_all2(const double *a, const double *b, const double *c, int n, double *red) {
    double s[4] = {0.0, 0.0, 0.0, 0.0}, t[4] = {0.0, 0.0, 0.0, 0.0};
    int i = threadIdx.x;
    for (; i + 3 * PS_THREADS < n; i += 4 * PS_THREADS) {
        double av[4], bv[4], cv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            av[q] = __ldcg(a + i + q * PS_THREADS);
            bv[q] = __ldcg(b + i + q * PS_THREADS);
            cv[q] = TWO ? __ldcg(c + i + q * PS_THREADS) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            s[q] += av[q] * bv[q];
            if (TWO) t[q] += av[q] * cv[q];
        }
    }
    for (; i < n; i += PS_THREADS) {
        const double ai = __ldcg(a + i);
        s[0] += ai * __ldcg(b + i);
        if (TWO) t[0] += ai * __ldcg(c + i);
    }
    double x = warp_sum((s[0] + s[1]) + (s[2] + s[3])), y = TWO ? warp_sum((t[0] + t[1]) + (t[2] + t[3])) : 0.0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = x;
        if (TWO) red[PS_THREADS / 32 + (threadIdx.x >> 5)] = y;
    }
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
#pragma unroll
    for (int w = 0; w < PS_THREADS / 32; w++) {
        r.x += red[w];
        if (TWO) r.y += red[PS_THREADS / 32 + w];
    }
    return r;
}
__device__ __forceinline__ double dot_all(const double *a, const double *b, int n, double *red) {
    return dot_all2<false>(a, b, nullptr, n, red).x;
}

// ---- tensor-core trailing update.  The panel phase stores U^T split into TF32
// hi / lo words, K contiguous ([row][BD]); a 128 x 128 tile of the trailing
// matrix is then C = U_i^T U_j over K = BD in three tcgen05.mma.kind::tf32
// passes (hi hi, hi lo, lo hi) accumulated in TMEM, with the operands staged by
// cp.async straight into the 128-byte-swizzle layout (double-buffered 32-wide K
// chunks) and the tile subtracted through shared memory with coalesced
// accesses.
constexpr int TT = 128;                              // trailing tile
constexpr int TT_CHUNK_BYTES = TT * 32 * 4;          // one operand, one 32-wide K chunk (16 KB)
constexpr int TT_STAGE_BYTES = 4 * TT_CHUNK_BYTES;   // A hi, A lo, B hi, B lo

// rows R0 .. R0+127, K columns 32q .. 32q+31 of X ([row][BD]) -> the SW128
// K-major tile at sbase (1024-byte aligned): row m at m * 128 B, its 16-byte
// chunk c at chunk position c ^ (m % 8)
template <int BD>
__device__ __forceinline__ void stage_sw128(uint32_t sbase, const float *X, int R0, int q) {
    for (int e = threadIdx.x; e < TT * 8; e += PS_THREADS) {
        const int m = e >> 3, c = e & 7;
        cp_async16(sbase + m * 128 + ((c ^ (m & 7)) << 4), X + (size_t)(R0 + m) * BD + q * 32 + c * 4);
    }
}

struct TcState {
    uint8_t *sm;          // 2 stages of TT_STAGE_BYTES, 1024-byte aligned (also the epilogue tile)
    uint64_t *mbar;       // [2] MMA completion per stage
    uint32_t cnt[2];      // commits issued per stage (mbarrier phase tracking)
    uint32_t tmem;        // 128 TMEM columns (128 x 128 FP32 accumulator)
    int *err;
};

// One 128 x 128 tile of a rank-BD update, C = A_i B_j^T over K = BD with the operands
// rows R0 .. R0 + 127 of (ah, al) and C0 .. C0 + 127 of (bh, bl) ([row][BD] TF32 hi / lo).
// Trailing mode (lim == 0): T[i][j] -= C for j <= i < n (row pitch n), except the entries
// with i, j < skip (the next diagonal block, updated by its owner).  Inverse mode
// (lim > 0): T[i][j] -= C for i < n, j < lim (row pitch ldt), where the columns j >= skip
// take their first update (T = -C, nothing read).  Returns false when a bounded wait gave
// up (err raised).
template <int BD>
__device__ bool trailing_tile_tc(TcState &ts, const float *ah, const float *al, const float *bh, const float *bl,
                                 float *T, int n, int ldt, int R0, int C0, int skip, int lim) {
    constexpr int NQ = BD / 32;
    const int tid = threadIdx.x;
    const uint32_t s0 = smem_u32(ts.sm);
    auto stage = [&](int q, int b) {
        const uint32_t sb = s0 + b * TT_STAGE_BYTES;
        stage_sw128<BD>(sb, ah, R0, q);
        stage_sw128<BD>(sb + TT_CHUNK_BYTES, al, R0, q);
        stage_sw128<BD>(sb + 2 * TT_CHUNK_BYTES, bh, C0, q);
        stage_sw128<BD>(sb + 3 * TT_CHUNK_BYTES, bl, C0, q);
        cp_async_commit();
    };
    // M = N = 128, FP32 accumulate, TF32 operands, both K-major
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TT >> 3) << 17) | ((uint32_t)(TT >> 4) << 24);
    stage(0, 0);
    for (int q = 0; q < NQ; q++) {
        const int b = q & 1;
        cp_async_wait_all();
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t sb = s0 + b * TT_STAGE_BYTES;
#pragma unroll
            for (int pass = 0; pass < 3; pass++) {
                const uint32_t sa = sb + (pass == 2 ? TT_CHUNK_BYTES : 0);                       // A hi, hi, lo
                const uint32_t sbb = sb + 2 * TT_CHUNK_BYTES + (pass == 1 ? TT_CHUNK_BYTES : 0);  // B hi, lo, hi
#pragma unroll
                for (int k = 0; k < 4; k++)
                    umma_tf32(ts.tmem, sw128_desc(sa + k * 32), sw128_desc(sbb + k * 32), idesc,
                              (q | pass | k) ? 1u : 0u);
            }
            umma_commit(&ts.mbar[b]);
        }
        ts.cnt[b]++;
        if (q + 1 < NQ) {
            const int nb = (q + 1) & 1;
            // the stage being refilled was read by the MMAs of chunk q - 1
            if (q >= 1 && !__syncthreads_and(mbar_wait(&ts.mbar[nb], (ts.cnt[nb] - 1) & 1, ts.err))) return false;
            stage(q + 1, nb);
        }
    }
    const int lb = (NQ - 1) & 1;
    bool done = mbar_wait(&ts.mbar[lb], (ts.cnt[lb] - 1) & 1, ts.err);
    if (NQ > 1) done = done && mbar_wait(&ts.mbar[lb ^ 1], (ts.cnt[lb ^ 1] - 1) & 1, ts.err);
    if (!__syncthreads_and(done)) return false;             // uniform over the CTA
    tc_fence_after();
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .., columns 64 (w / 4) .. + 63
    // into a shared tile of pitch EP (16-byte rows: conflict-free 128-bit
    // accesses), then the tile is subtracted from T with coalesced accesses
    constexpr int EP = TT + 4;
    float *ep = (float *)ts.sm;
    {
        const int warp = tid >> 5, lane = tid & 31, row = 32 * (warp & 3) + lane;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int col = 64 * (warp >> 2) + 32 * h;
            float v[32];
            tmem_ld32(ts.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col, v);
#pragma unroll
            for (int j = 0; j < 32; j += 4)
                *(float4 *)&ep[row * EP + col + j] = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (lim > 0) {
        // inverse mode: ldt, lim and skip are multiples of 4, so no float4 group straddles them
        float4 v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int e4 = tid + q * PS_THREADS, i = R0 + (e4 >> 5), j = C0 + 4 * (e4 & 31);
            v[q] = (i < n && j < lim && j < skip) ? __ldcg((const float4 *)&T[(size_t)i * ldt + j])
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int e4 = tid + q * PS_THREADS, r = e4 >> 5, c = 4 * (e4 & 31), i = R0 + r, j = C0 + c;
            if (i < n && j < lim) {
                const float4 d = *(const float4 *)&ep[r * EP + c];
                *(float4 *)&T[(size_t)i * ldt + j] = make_float4(v[q].x - d.x, v[q].y - d.y, v[q].z - d.z, v[q].w - d.w);
            }
        }
    } else if ((n & 3) == 0) {
        // 16 float4 per thread, all loads before the stores
        float4 v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int e4 = tid + q * PS_THREADS, i = R0 + (e4 >> 5), j = C0 + 4 * (e4 & 31);
            v[q] = (i < n && j <= i) ? __ldcg((const float4 *)&T[(size_t)i * n + j]) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int e4 = tid + q * PS_THREADS, r = e4 >> 5, c = 4 * (e4 & 31), i = R0 + r, j = C0 + c;
            if (i < n && j <= i && !(i < skip && j < skip)) {   // skip is a multiple of 4 here
                const float4 d = *(const float4 *)&ep[r * EP + c];
                float4 o = make_float4(v[q].x - d.x, v[q].y - d.y, v[q].z - d.z, v[q].w - d.w);
                if (j + 3 <= i) {
                    *(float4 *)&T[(size_t)i * n + j] = o;
                } else {                                    // the diagonal crosses this group
                    float *t = &T[(size_t)i * n + j];
                    t[0] = o.x;
                    if (j + 1 <= i) t[1] = o.y;
                    if (j + 2 <= i) t[2] = o.z;
                }
            }
        }
    } else {
        // 32 independent loads in flight per thread before the stores (a load after
        // a store to the same array is not hoisted)
        for (int e0 = tid; e0 < TT * TT; e0 += 32 * PS_THREADS) {
            float v[32];
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const int e = e0 + q * PS_THREADS, i = R0 + e / TT, j = C0 + e % TT;
                v[q] = (i < n && j <= i) ? __ldcg(&T[(size_t)i * n + j]) : 0.f;
            }
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const int e = e0 + q * PS_THREADS, i = R0 + e / TT, j = C0 + e % TT;
                if (i < n && j <= i && !(i < skip && j < skip)) T[(size_t)i * n + j] = v[q] - ep[(e / TT) * EP + e % TT];
            }
        }
    }
    __syncthreads();
    return true;
}

// Order from which the preconditioner is applied by blocked substitution
// instead of through an explicit L^{-1}.
constexpr int BLOCKED_SOLVE_MIN = 4608;

// Relative residual |r| / |rhs| at which the CG refinement stops.
constexpr double CG_RTOL = 1e-10;

struct FrArgs {
    float *T;           // [n][n] Gram + shift (lower) on entry; U = L^T in the upper triangle after
    float *Li, *LiT;    // [n][ldl] L^{-1} (lower; R while it is built) and its transpose; pad columns are zero
    int n;              // order of the system
    int ldl;            // row pitch of Li / LiT (n rounded up to 32)
    int space;          // 0: samples (n = N_s, unknown y), 1: parameters (n = N_p, unknown delta)
    const double *O;    // centred Jacobian [N_s][N_p]
    int Ns;
    long P;
    const double *eps;  // [N_s] centred local energies
    double shift;
    double *x;          // [n] solution
    double *rhs, *r;    // [n] right-hand side and residual
    double *r2;         // [n] the residual's second buffer (the double-float CG alternates them)
    double *u, *upart;  // intermediate vector, partial column sums ([chunks][N_p])
    double *p, *q, *z;  // [n] CG direction, operator times direction, preconditioned residual
    float *rf, *zf;     // [n] FP32 right-hand side and half-solve
    float *uh, *ul;     // [n + 128][bd] TF32 hi / lo words of the current panel U^T (K contiguous; pad rows zero)
    float *xh, *xl;     // [n + 128][bd] TF32 hi / lo words of X^T over the current block row of X = L^{-1}
    const float *oh, *ol;  // [N_s][N_p] O_c as double-float words (FP32 hi + lo), or null
    int df_rows;        // rows per chunk of the double-float operator (from N_s and the SM count only)
    int bd;             // diagonal block width (BD_SMALL or BD_LARGE)
    double *nrm;        // [3] |r|^2, |rhs|^2, CG iterations run
    int sweeps;         // maximum CG iterations
    int *status;        // [0] first failing column or -1
    unsigned *bar;      // [0] grid barrier arrivals, [1..3] owner / worker flags (X, U, T), [4] worker barrier
    int *err;
    unsigned long long *tm;   // [8] phase nanoseconds: [0..6] CTA 0's view, [7] owners' block work
};

// The solve of one system by the CTAs bx = 0 .. G-1 of a cooperative launch
// (all co-resident): the whole grid for a single system, a slice of it when a
// batch of systems shares one launch.
template <int BD>
__device__ __forceinline__ void fr_body(const FrArgs &a, const int bx, const int G, TcState &ts) {
    extern __shared__ float psm[];
    float (*S0)[BT + 1] = (float (*)[BT + 1])psm;
    float (*S1)[BT + 1] = (float (*)[BT + 1])(psm + BT * (BT + 1));
    TileSmem &TS = *(TileSmem *)psm;
    float (*ST)[GT + 1] = (float (*)[GT + 1])psm;           // 64 x 65 staging tile
    const int n = a.n, ldl = a.ldl, tid = threadIdx.x;
    const int lane = tid & 31, tx = tid & 15, ty = tid >> 4;
    const int gtid = bx * PS_THREADS + tid, gthreads = G * PS_THREADS;
    const int gwarp = bx * (PS_THREADS / 32) + (tid >> 5), gwarps = G * (PS_THREADS / 32);
    const int nb = (n + BD - 1) / BD;
    __shared__ int s_flag;
    __shared__ float tmpb[3 * 1024];
    unsigned long long tacc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const bool timing = a.tm != nullptr && bx == 0 && tid == 0;
    unsigned long long tstart = timing ? gtimer() : 0, tprev = tstart;
#define NQS_PHASE(k)                                  \
    if (timing) {                                     \
        unsigned long long now_ = gtimer();           \
        if ((k) >= 0) tacc[(k) < 0 ? 0 : (k)] += now_ - tprev; \
        tprev = now_;                                 \
    }

    // ---------------- factor
    // Diagonal block kb: its owner CTA loads it, factors and inverts it in
    // shared memory and stores X_kk in Li / LiT (a breakdown goes to status[0]).
    // With BD = 64 and pk0 >= 0 the block is first updated by the previous step's
    // panel rows pk0 .. pk0 + pbs - 1 of T (U = L^T): D -= U^T U, one 64 x 64 SIMT tile
    // whose result is subtracted as the block is loaded (the block of T itself is dead
    // after its factor, so it is not written back).
    auto factor_diag = [&](int kb, int pk0, int pbs) {
        const int k0 = kb * BD, bs = min(BD, n - k0);
        const unsigned long long t_own = tid == 0 ? gtimer() : 0;
        int f;
        if (BD == 64) {
            float acc[4][4] = {};
            if (pk0 >= 0) {
                const float *U = a.T + (size_t)pk0 * n;
                gemm64<true, true>(acc, U, n, k0, k0 + bs, U, n, k0, k0 + bs, 0, pbs, TS);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const int rr = ty + 16 * u, cc = tx + 16 * v;
                    const bool in = rr < bs && cc <= rr;
                    S0[rr][cc] = in ? __ldcg(&a.T[(size_t)(k0 + rr) * n + k0 + cc]) - acc[u][v]
                                    : (rr == cc ? 1.f : 0.f);
                }
            __syncthreads();
            f = block_chol_inv64(S0, S1, bs, tmpb);
        } else {
            for (int e0 = 0; e0 < BD * BD; e0 += 8 * PS_THREADS) {
                float v[8];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int e = e0 + tid + q * PS_THREADS, rr = e / BD, cc = e % BD;
                    const bool in = e < BD * BD && rr < bs && cc <= rr;
                    v[q] = in ? __ldcg(&a.T[(size_t)(k0 + rr) * n + k0 + cc]) : (rr == cc ? 1.f : 0.f);
                }
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int e = e0 + tid + q * PS_THREADS;
                    if (e < BD * BD) S0[e / BD][e % BD] = v[q];
                }
            }
            __syncthreads();
            f = block_chol<BD>(S0, S1, bs, &s_flag, tmpb);
            if (f < 0) block_inv<BD>(S0, S1, tmpb);
        }
        if (f >= 0) {
            if (tid == 0) {
                a.status[0] = k0 + f;
                __threadfence();
            }
        } else {
            for (int e = tid; e < BD * BD; e += PS_THREADS) {
                const int rr = e / BD, q = e % BD;
                if (rr < bs && q < bs) {
                    a.Li[(size_t)(k0 + rr) * ldl + k0 + q] = S1[rr][q];
                    a.LiT[(size_t)(k0 + rr) * ldl + k0 + q] = S1[q][rr];
                }
            }
        }
        __syncthreads();                                    // S0 / S1 are reused as GEMM staging
        if (tid == 0 && a.tm) atomicAdd(a.tm + 7, gtimer() - t_own);
    };
    // Large systems skip the explicit L^{-1} (n^3 / 3 flops) and apply the
    // preconditioner by blocked substitution (one grid barrier per diagonal
    // block and direction); below BLOCKED_SOLVE_MIN the inverse is cheaper than
    // those barriers over the CG iterations.
    const bool blocked = n >= BLOCKED_SOLVE_MIN;
    // X = L^{-1} is built beside the factor (forward substitution of L X = I, right-looking
    // by block columns): R = I - sum_{p < kb} L_{:,p} X_{p,:} accumulates in the lower
    // off-diagonal blocks of Li.  In the panel phase of step kb block row kb of X is
    // finalised, X_kb,c = X_kk R_kb,c (c < k0), written over R, transposed into LiT and split
    // into xh / xl; in the trailing phase the rows below are updated, R_i,c -= L_i,kb X_kb,c
    // (c < k1), by 128 x 128 tensor-core tiles beside the trailing tiles of the factor.
    // Task t of the block row: column tile t (64 wide) of X_kb, all its rows by one CTA (the
    // product reads the whole column tile of R before any of it is overwritten), t < k0 / 64;
    // then (with_x) the copy of X_kk^T into xh / xl.
    auto xrow_tasks = [&](int k0, bool with_x) { return k0 / GT + (with_x ? 1 : 0); };
    auto xrow_tile = [&](int k0, int bs, bool with_x, int t) {
        constexpr int NRT = BD / GT;
        if (t < k0 / GT) {
            const int c0 = t * GT;
            float acc[NRT][4][4] = {};
#pragma unroll
            for (int rt = 0; rt < NRT; rt++)
                if (rt * GT < bs)
                    gemm64<false, true>(acc[rt], a.Li + (size_t)k0 * ldl + k0, ldl, rt * GT, bs, a.Li + (size_t)k0 * ldl,
                                        ldl, c0, k0, 0, bs, TS);
#pragma unroll
            for (int rt = 0; rt < NRT; rt++) {
                const int r0 = rt * GT;
                if (r0 >= bs) break;
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const int r = r0 + ty + 16 * u, c = c0 + tx + 16 * v;
                        if (r < bs) a.Li[(size_t)(k0 + r) * ldl + c] = acc[rt][u][v];
                        ST[ty + 16 * u][tx + 16 * v] = acc[rt][u][v];
                    }
                __syncthreads();
                for (int e = tid; e < GT * GT; e += PS_THREADS) {
                    const int cc = e / GT, rr = e % GT, r = r0 + rr, c = c0 + cc;
                    if (r < bs) {
                        const float x = ST[rr][cc];
                        a.LiT[(size_t)c * ldl + k0 + r] = x;
                        if (with_x) {
                            const float h = tf32_rna(x);
                            a.xh[(size_t)c * BD + r] = h;
                            a.xl[(size_t)c * BD + r] = tf32_rna(x - h);
                        }
                    }
                }
                __syncthreads();
            }
        } else {
            for (int e = tid; e < BD * BD; e += PS_THREADS) {
                const int cc = e / BD, rr = e % BD;
                if (cc < bs) {
                    const float x = rr < bs ? __ldcg(&a.LiT[(size_t)(k0 + cc) * ldl + k0 + rr]) : 0.f, h = tf32_rna(x);
                    a.xh[(size_t)(k0 + cc) * BD + rr] = h;
                    a.xl[(size_t)(k0 + cc) * BD + rr] = tf32_rna(x - h);
                }
            }
        }
    };
    // Look-ahead: the diagonal block of step kb + 1 is updated and factored by CTA 0 during
    // the trailing phase of step kb (64 x 64 SIMT tiles of U_kb^T U_kb over its lower
    // triangle, then factor_diag), while the other CTAs update the trailing tiles, the
    // first of which leaves that block's entries to CTA 0.  So each step has two grid
    // barriers (after the panel and after the trailing update) and the block's factor runs
    // beside the trailing tiles instead of in a phase of its own.
    // Panel tile: U[k0 + c][r] = sum_m X_kk[c][m] A[r][k0 + m], columns c0 .. c0 + 63 of the
    // block, rows r0 .. r0 + 63, into the upper triangle of T and split into (uhk, ulk).
    auto panel_tile = [&](int k0, int bs, int c0, int r0, float *uhk, float *ulk) {
        float acc[4][4] = {};
        gemm64<false, false>(acc, a.Li + (size_t)k0 * ldl + k0, ldl, c0, bs, a.T + k0, n, r0, n, 0, min(bs, c0 + GT),
                             TS);
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const int c = c0 + ty + 16 * u, r = r0 + tx + 16 * v;
                if (c < bs && r < n) a.T[(size_t)(k0 + c) * n + r] = acc[u][v];
                ST[ty + 16 * u][tx + 16 * v] = acc[u][v];
            }
        __syncthreads();
        // U^T split into TF32 hi / lo, rows r (K = panel column contiguous)
        for (int e = tid; e < GT * GT; e += PS_THREADS) {
            const int rr = e / GT, cc = e % GT, r = r0 + rr, c = c0 + cc;
            if (c < bs && r < n) {
                const float x = ST[cc][rr], h = tf32_rna(x);
                uhk[(size_t)r * BD + c] = h;
                ulk[(size_t)r * BD + c] = tf32_rna(x - h);
            }
        }
        __syncthreads();
    };
    // Flags between the owner CTA and the others (monotonic words of bar[], cleared at every
    // launch): flag_set publishes after the whole CTA's writes (block barrier, then an
    // acq_rel fence at GPU scope before the store); flag_wait polls with the grid barrier's
    // bounded budget and gives up on an error or a broken factor (status set).
    auto flag_set = [&](unsigned *f, unsigned v) {
        __syncthreads();
        if (tid == 0) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            atomicExch(f, v);
        }
    };
    auto flag_wait = [&](const unsigned *f, unsigned target) -> bool {
        __shared__ int s_fok;
        __syncthreads();
        if (tid == 0) {
            const unsigned budget = *(volatile unsigned *)&g_barrier_budget;
            int ok = 1;
            for (uint32_t it = 0;; it++) {
                unsigned cur;
                asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(f) : "memory");
                if ((int)(cur - target) >= 0) break;
                if (it + 1 > budget) {
                    atomicExch(a.err, 2);
                    ok = 0;
                    break;
                }
                if ((it & 31) == 31) {
                    if (*((volatile int *)a.err)) {
                        ok = 0;
                        break;
                    }
                    if (it > 256) __nanosleep(32);
                }
            }
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            s_fok = ok && *((volatile int *)a.err) == 0 && *((volatile int *)a.status) < 0;
        }
        __syncthreads();
        return s_fok != 0;
    };
    // The owner's step kb of the pipelined factor (BD = 64), with X_kk in S1 from the previous
    // factor: the block A = T[k1 .. k1 + bs1)[k0 .. k1) is staged in shared memory (SA, the
    // unused rows between S0 and S1) while the next diagonal block D is prefetched into
    // registers; U = X_kk A^T (64 x bs1, both operands in shared memory) goes to the upper
    // triangle of T and to (uhk, ulk) and stays in S0; flag U; D -= U^T U from shared memory;
    // then D is factored and inverted into S1 (X of block kb + 1) and stored to Li / LiT.
    float (*SA)[BT + 1] = (float (*)[BT + 1])(psm + 64 * (BT + 1));
    auto owner_step = [&](int kb, float *uhk, float *ulk, unsigned *fl_u) -> bool {
        const int k0 = kb * BD, k1 = k0 + BD, bs1 = min(BD, n - k1);
        const unsigned long long t_own = tid == 0 ? gtimer() : 0;
        float dv[4][4];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const int rr = ty + 16 * u, cc = tx + 16 * v;
                dv[u][v] = (rr < bs1 && cc <= rr) ? __ldcg(&a.T[(size_t)(k1 + rr) * n + k1 + cc]) : 0.f;
            }
        for (int e = tid; e < BD * BD; e += PS_THREADS) {
            const int rr = e / BD, m = e % BD;
            SA[rr][m] = rr < bs1 ? __ldcg(&a.T[(size_t)(k1 + rr) * n + k0 + m]) : 0.f;
        }
        __syncthreads();
        {
            // U[c][r] = sum_m X[c][m] A[r][m]: thread (ty, tx) owns c = ty + 16u, r = tx + 16v
            float acc[4][4] = {};
#pragma unroll 8
            for (int m = 0; m < BD; m++) {
                float xa[4], av[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    xa[u] = S1[ty + 16 * u][m];
                    av[u] = SA[tx + 16 * u][m];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = fmaf(xa[u], av[v], acc[u][v]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const int c = ty + 16 * u, r = tx + 16 * v;
                    S0[c][r] = r < bs1 ? acc[u][v] : 0.f;
                    if (r < bs1) a.T[(size_t)(k0 + c) * n + k1 + r] = acc[u][v];
                }
        }
        __syncthreads();
        for (int e = tid; e < BD * BD; e += PS_THREADS) {
            const int rr = e / BD, c = e % BD;
            if (rr < bs1) {
                const float x = S0[c][rr], h = tf32_rna(x);
                uhk[(size_t)(k1 + rr) * BD + c] = h;
                ulk[(size_t)(k1 + rr) * BD + c] = tf32_rna(x - h);
            }
        }
        flag_set(fl_u, kb + 1);
        {
            // D[i][j] -= sum_c U[c][i] U[c][j] (i = ty + 16u, j = tx + 16v), lower triangle
            float acc[4][4] = {};
#pragma unroll 8
            for (int c = 0; c < BD; c++) {
                float ui[4], uj[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    ui[u] = S0[c][ty + 16 * u];
                    uj[u] = S0[c][tx + 16 * u];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = fmaf(ui[u], uj[v], acc[u][v]);
            }
            __syncthreads();                                // S0 is overwritten with the updated block
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const int rr = ty + 16 * u, cc = tx + 16 * v;
                    S0[rr][cc] = (rr < bs1 && cc <= rr) ? dv[u][v] - acc[u][v] : (rr == cc ? 1.f : 0.f);
                }
        }
        __syncthreads();
        const int f = block_chol_inv64(S0, S1, bs1, tmpb);
        if (f >= 0) {
            if (tid == 0) {
                a.status[0] = k1 + f;
                __threadfence();
            }
        } else {
            for (int e = tid; e < BD * BD; e += PS_THREADS) {
                const int rr = e / BD, q = e % BD;
                if (rr < bs1 && q < bs1) {
                    a.Li[(size_t)(k1 + rr) * ldl + k1 + q] = S1[rr][q];
                    a.LiT[(size_t)(k1 + rr) * ldl + k1 + q] = S1[q][rr];
                }
            }
        }
        __syncthreads();
        if (tid == 0 && a.tm) atomicAdd(a.tm + 7, gtimer() - t_own);
        return f < 0;
    };
    // Pipelined factor (64-wide blocks, four CTAs or more): CTA 0, the owner, runs one step
    // ahead of the others.  At step kb it waits until the trailing tile 0 of step kb - 1 is
    // done (flag T), forms the panel tile of the rows of block kb + 1 itself (the critical
    // one; flag U), then updates and factors the next diagonal block (flag X).  The other
    // CTAs, the workers, wait for X_kb (flag X), form the rest of the panel and block row kb
    // of L^{-1}, pass a barrier among themselves, wait for the critical tile (flag U) and
    // run the trailing and inverse tiles; the worker with trailing tile 0 raises flag T.  So
    // the chain of diagonal blocks is the owner's alone and no grid barrier lies on it.  The
    // split U^T alternates between two buffers by step, as the owner writes step kb + 1's
    // critical tile while the workers still read step kb's.
    const bool piped = BD == 64 && G >= 4 && nb > 1;
    if (piped) {
        unsigned *fl_x = a.bar + 1, *fl_u = a.bar + 2, *fl_t = a.bar + 3, *wbar = a.bar + 4;
        const size_t ubuf = (size_t)(n + TT) * BD;
        if (bx == 0) {
            factor_diag(0, -1, 0);
            flag_set(fl_x, 1);
            NQS_PHASE(0);
            for (int kb = 0; kb < nb; kb++) {
                const int k0 = kb * BD, bs = min(BD, n - k0), k1 = k0 + bs, rest = n - k1;
                if (rest <= 0 || __ldcg(a.status) >= 0) break;
                if (kb > 0 && !flag_wait(fl_t, kb)) return;
                NQS_PHASE(1);
                owner_step(kb, a.uh + (kb & 1) * ubuf, a.ul + (kb & 1) * ubuf, fl_u);
                flag_set(fl_x, kb + 2);                     // also wakes the workers after a breakdown
                NQS_PHASE(2);
            }
        } else {
            const int wid = bx - 1, W = G - 1;
            for (int kb = 0; kb < nb; kb++) {
                const int k0 = kb * BD, bs = min(BD, n - k0), k1 = k0 + bs, rest = n - k1;
                if (rest <= 0) break;
                if (!flag_wait(fl_x, kb + 1)) return;
                float *uhk = a.uh + (kb & 1) * ubuf, *ulk = a.ul + (kb & 1) * ubuf;
                {
                    const int npt = (rest + GT - 1) / GT - 1;   // panel row tiles after the critical one
                    const int ntasks = npt + (blocked ? 0 : xrow_tasks(k0, true));
                    for (int t = wid; t < ntasks; t += W) {
                        if (t >= npt) xrow_tile(k0, bs, true, t - npt);
                        else panel_tile(k0, bs, 0, k1 + (t + 1) * GT, uhk, ulk);
                    }
                }
                if (!grid_barrier(wbar, a.err, W)) return;
                if (!flag_wait(fl_u, kb + 1)) return;
                {
                    const int bs1 = min(BD, rest);
                    const int ntt = (rest + TT - 1) / TT, ntiles = ntt * (ntt + 1) / 2;
                    const int ncr = blocked ? 0 : (k1 + TT - 1) / TT, nall = ntiles + ntt * ncr;
                    for (int t = wid; t < nall; t += W) {
                        bool ok;
                        if (t < ntiles) {
                            int bi, bj;
                            tri_tile(t, bi, bj);
                            ok = trailing_tile_tc<BD>(ts, uhk, ulk, uhk, ulk, a.T, n, n, k1 + bi * TT, k1 + bj * TT,
                                                      t == 0 ? k1 + bs1 : 0, 0);
                            if (ok && t == 0) flag_set(fl_t, kb + 1);
                        } else {
                            const int tr = t - ntiles;
                            ok = trailing_tile_tc<BD>(ts, uhk, ulk, a.xh, a.xl, a.Li, n, ldl, k1 + (tr / ncr) * TT,
                                                      (tr % ncr) * TT, k0, k1);
                        }
                        if (!ok) return;
                    }
                }
                if (!grid_barrier(wbar, a.err, W)) return;
            }
            if (!flag_wait(fl_x, nb)) return;               // the last diagonal block (or a breakdown)
        }
        if (__ldcg(a.status) >= 0) return;                  // broken factor: every CTA leaves here
        if (!grid_barrier(a.bar, a.err, G)) return;
    } else {
        if (bx == 0) factor_diag(0, -1, 0);
        if (!grid_barrier(a.bar, a.err, G)) return;
        if (__ldcg(a.status) >= 0) return;                      // broken factor: every CTA leaves here
        NQS_PHASE(0);
        for (int kb = 0; kb < nb; kb++) {
            const int k0 = kb * BD, bs = min(BD, n - k0), k1 = k0 + bs, rest = n - k1;
            if (rest <= 0) break;
            // panel: U[k0 + c][r] = sum_m X_kk[c][m] A[r][k0 + m] for r >= k1; block row kb of X
            {
                constexpr int NCT = (BD + GT - 1) / GT;          // column tiles of the panel
                const int ntr = (rest + GT - 1) / GT, npt = NCT * ntr;
                const int ntasks = npt + (blocked ? 0 : xrow_tasks(k0, true));
                for (int t = bx; t < ntasks; t += G) {
                    if (t >= npt) {
                        xrow_tile(k0, bs, true, t - npt);
                        continue;
                    }
                    const int c0 = (t % NCT) * GT, r0 = k1 + (t / NCT) * GT;
                    if (c0 >= bs) continue;
                    panel_tile(k0, bs, c0, r0, a.uh, a.ul);
                }
            }
            if (!grid_barrier(a.bar, a.err, G)) return;
            NQS_PHASE(1);
            // trailing update, with the next diagonal block updated and factored by CTA 0, and
            // the update of R by block row kb of X
            {
                const int bs1 = min(BD, rest);                  // order of the next diagonal block
                if (bx == 0 && BD == 64) {
                    factor_diag(kb + 1, k0, bs);                // the update fused into the block's load
                } else if (bx == 0) {
                    // D -= U_kb^T U_kb on the lower 64 x 64 tiles of the next diagonal block, FP32
                    // from U (= L^T, the upper triangle rows k0 .. k0 + bs - 1 of T)
                    const float *U = a.T + (size_t)k0 * n;
                    for (int ti = 0; ti * GT < bs1; ti++)
                        for (int tj = 0; tj <= ti; tj++) {
                            float acc[4][4] = {};
                            gemm64<true, true>(acc, U, n, k1 + ti * GT, k1 + bs1, U, n, k1 + tj * GT, k1 + bs1, 0, bs, TS);
    #pragma unroll
                            for (int u = 0; u < 4; u++)
    #pragma unroll
                                for (int v = 0; v < 4; v++) {
                                    const int i = k1 + ti * GT + ty + 16 * u, j = k1 + tj * GT + tx + 16 * v;
                                    if (i < k1 + bs1 && j <= i) a.T[(size_t)i * n + j] -= acc[u][v];
                                }
                            __syncthreads();
                        }
                    factor_diag(kb + 1, -1, 0);
                }
                const int ntt = (rest + TT - 1) / TT, ntiles = ntt * (ntt + 1) / 2;
                const int ncr = blocked ? 0 : (k1 + TT - 1) / TT, nall = ntiles + ntt * ncr;
                const int t0 = G > 1 ? bx - 1 : 0, dt = G > 1 ? G - 1 : 1;
                for (int t = t0; t >= 0 && t < nall; t += dt) {
                    bool ok;
                    if (t < ntiles) {
                        int bi, bj;
                        tri_tile(t, bi, bj);
                        ok = trailing_tile_tc<BD>(ts, a.uh, a.ul, a.uh, a.ul, a.T, n, n, k1 + bi * TT, k1 + bj * TT,
                                                  t == 0 ? k1 + bs1 : 0, 0);
                    } else {
                        const int tr = t - ntiles;
                        ok = trailing_tile_tc<BD>(ts, a.uh, a.ul, a.xh, a.xl, a.Li, n, ldl, k1 + (tr / ncr) * TT,
                                                  (tr % ncr) * TT, k0, k1);
                    }
                    if (!ok) return;
                }
            }
            if (!grid_barrier(a.bar, a.err, G)) return;
            if (__ldcg(a.status) >= 0) return;                  // broken factor: every CTA leaves here
            NQS_PHASE(2);
        }
    }
    // ---------------- the last block row of L^{-1}
    if (!blocked && nb > 1) {
        const int k0 = (nb - 1) * BD, bs = n - k0;
        for (int t = bx; t < xrow_tasks(k0, false); t += G) xrow_tile(k0, bs, false, t);
        if (!grid_barrier(a.bar, a.err, G)) return;
    }
    NQS_PHASE(3);

    const int Ns = a.Ns;
    const long P = a.P;
    // ---------------- the parameter-space operator in double-float arithmetic
    // q = O_c^T (O_c v) / N_s + shift v, or the right-hand side O_c^T eps / N_s, from the
    // double-float words of O_c (oh + ol) with v split likewise (vh + vl).  The rows of O_c
    // are cut into chunks of DF_ROWS, dealt to the CTAs in turn: a warp forms u_i = o_i . v
    // for one row of the chunk at a time (double-float butterfly over the lanes), then the
    // threads accumulate sum_i u_i o_i over segments of the chunk's rows for four-column
    // groups (eight rows' loads in flight) and the segments are added in double-float; after
    // one grid barrier the chunks' partial column sums are summed in FP64 in a fixed order
    // (eight columns per CTA, 32 slots of chunks per column, five loads in flight).
    // The chunking does not depend on the grid size (a.df_rows comes from N_s and the SM
    // count), so a system solved by a slice of a batch launch gets the same bits as by the
    // whole grid, and at full grid every CTA has one chunk.
    const int DF_ROWS = a.df_rows;
    __shared__ double redc[PS_THREADS / 32][32];
    const int ndc = (Ns + DF_ROWS - 1) / DF_ROWS;
    const bool df_op = a.space == 1 && a.oh != nullptr && df_words_ok(P) && DF_ROWS > 0 &&
                       8 * P + 8 * (long)DF_ROWS + 8 * (long)DF_SEGS * P <= PS_SMEM;
    // With zs set, v is the CG direction formed on the fly by every CTA, v = zs (pold null) or
    // zs + beta pold, and written to pnew by one CTA per 256 entries (so no grid barrier
    // publishes it first).
    auto op_df = [&](const double *v, double *q, bool rhs_mode, const double *zs = nullptr,
                     const double *pold = nullptr, double beta = 0.0, double *pnew = nullptr) -> bool {
        const int warp = tid >> 5;
        float *vh = psm, *vl = vh + P, *uh = vl + P, *ul = uh + DF_ROWS;
        const long P4 = P >> 2;
        if (!rhs_mode) {
            for (long k = tid; k < P; k += PS_THREADS) {
                double x;
                if (zs) {
                    x = pold ? __fma_rn(beta, __ldcg(pold + k), __ldcg(zs + k)) : __ldcg(zs + k);
                    if (bx == (int)((k / PS_THREADS) % G)) pnew[k] = x;
                } else {
                    x = __ldcg(v + k);
                }
                split_f64_words(x, vh[k], vl[k]);
            }
        }
        __syncthreads();
        const float4 *oh4 = (const float4 *)a.oh, *ol4 = (const float4 *)a.ol;
        const float4 *vh4 = (const float4 *)vh, *vl4 = (const float4 *)vl;
        float2 *cs = (float2 *)(ul + DF_ROWS);          // per row segment: column sums (hi, lo)
        for (int ch = bx; ch < ndc; ch += G) {
            const int i0 = ch * DF_ROWS, nr = min(Ns, i0 + DF_ROWS) - i0;
            if (rhs_mode) {
                for (int r = tid; r < nr; r += PS_THREADS) split_f64_words(__ldcg(a.eps + i0 + r), uh[r], ul[r]);
            } else {
                for (int r = warp; r < nr; r += PS_THREADS / 32) {
                    const size_t rb = (size_t)(i0 + r) * P4;
                    float sh0 = 0.f, sl0 = 0.f, sh1 = 0.f, sl1 = 0.f;
                    for (long g0 = lane; g0 < P4; g0 += 32 * DF_G) {
                        // DF_G groups' loads in flight per lane before their products (a whole
                        // row of up to 32 DF_G groups in one batch)
                        float4 xh[DF_G], xl[DF_G];
#pragma unroll
                        for (int t = 0; t < DF_G; t++) {
                            const long g = g0 + 32 * t;
                            xh[t] = g < P4 ? __ldcg(oh4 + rb + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                            xl[t] = g < P4 ? __ldcg(ol4 + rb + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                        }
#pragma unroll
                        for (int t = 0; t < DF_G; t++) {
                            const long g = g0 + 32 * t;
                            if (g < P4) {
                                const float4 yh = vh4[g], yl = vl4[g];
                                df_fma(sh0, sl0, xh[t].x, xl[t].x, yh.x, yl.x);
                                df_fma(sh1, sl1, xh[t].y, xl[t].y, yh.y, yl.y);
                                df_fma(sh0, sl0, xh[t].z, xl[t].z, yh.z, yl.z);
                                df_fma(sh1, sl1, xh[t].w, xl[t].w, yh.w, yl.w);
                            }
                        }
                    }
                    df_add(sh0, sl0, sh1, sl1);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
                        df_add(sh0, sl0, __shfl_xor_sync(0xffffffffu, sh0, o), __shfl_xor_sync(0xffffffffu, sl0, o));
                    if (lane == 0) {
                        uh[r] = sh0;
                        ul[r] = sl0;
                    }
                }
            }
            __syncthreads();
            // sum_i u_i o_i over the chunk: items (four-column group g, row segment h), with the
            // number of segments H chosen from P and the chunk's rows only, so that the threads'
            // rounds times each item's batches of eight rows is least (P = 1120, 27 rows: four
            // segments of seven rows, five rounds of one batch)
            int H = 1;
            {
                long best = 0;
                for (int hh = 1; hh <= DF_SEGS; hh++) {
                    const long cost = (P4 * hh + PS_THREADS - 1) / PS_THREADS * (((nr + hh - 1) / hh + 7) / 8);
                    if (hh == 1 || cost < best) {
                        best = cost;
                        H = hh;
                    }
                }
            }
            const int seg = (nr + H - 1) / H;
            for (long it = tid; it < P4 * H; it += PS_THREADS) {
                const long g = it % P4;
                const int h = (int)(it / P4), r1 = min(nr, (h + 1) * seg);
                float chh[4] = {0.f, 0.f, 0.f, 0.f}, cll[4] = {0.f, 0.f, 0.f, 0.f};
                for (int r = h * seg; r < r1; r += 8) {
                    const int cnt = min(8, r1 - r);
                    float4 xh[8], xl[8];
#pragma unroll
                    for (int t = 0; t < 8; t++) {
                        xh[t] = t < cnt ? __ldcg(oh4 + (size_t)(i0 + r + t) * P4 + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                        xl[t] = t < cnt ? __ldcg(ol4 + (size_t)(i0 + r + t) * P4 + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                    for (int t = 0; t < 8; t++) {
                        if (t < cnt) {
                            const float wh = uh[r + t], wl = ul[r + t];
                            df_fma(chh[0], cll[0], xh[t].x, xl[t].x, wh, wl);
                            df_fma(chh[1], cll[1], xh[t].y, xl[t].y, wh, wl);
                            df_fma(chh[2], cll[2], xh[t].z, xl[t].z, wh, wl);
                            df_fma(chh[3], cll[3], xh[t].w, xl[t].w, wh, wl);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 4; c++) cs[(size_t)h * P + 4 * g + c] = make_float2(chh[c], cll[c]);
            }
            __syncthreads();
            for (long k = tid; k < P; k += PS_THREADS) {
                float sh = cs[k].x, sl = cs[k].y;
                for (int h = 1; h < H; h++) df_add(sh, sl, cs[(size_t)h * P + k].x, cs[(size_t)h * P + k].y);
                a.upart[(size_t)ch * P + k] = (double)sh + (double)sl;
            }
            __syncthreads();                                // uh / ul / cs are refilled for the next chunk
        }
        if (!grid_barrier(a.bar, a.err, G)) return false;
        // the chunks' partials, summed in FP64 for eight columns per CTA: thread (warp, lane)
        // takes column 8 cg + (lane & 7) of chunks s, s + 32, ... (s = 4 warp + lane / 8, five
        // loads in flight), then warp 0 adds the 32 slots of each column in a fixed order
        const long nc8 = (P + 7) / 8;
        for (long cg = bx; cg < nc8; cg += G) {
            const long k = cg * 8 + (lane & 7);
            const int s0 = warp * 4 + (lane >> 3);
            double acc = 0.0;
            if (k < P) {
                for (int b0 = s0; b0 < ndc; b0 += 32 * 5) {
                    double t5[5];
#pragma unroll
                    for (int j = 0; j < 5; j++) {
                        const int b = b0 + 32 * j;
                        t5[j] = b < ndc ? __ldcg(a.upart + (size_t)b * P + k) : 0.0;
                    }
                    acc += (t5[0] + t5[1]) + ((t5[2] + t5[3]) + t5[4]);
                }
            }
            redc[warp][lane] = acc;
            __syncthreads();
            if (warp == 0) {
                // lane: column lane & 7, slots 4 w + lane / 8 for w = 0..7; then across the four
                double t = 0.0;
#pragma unroll
                for (int w = 0; w < PS_THREADS / 32; w++) t += redc[w][lane];
                t += __shfl_xor_sync(0xffffffffu, t, 8);
                t += __shfl_xor_sync(0xffffffffu, t, 16);
                const long kk = cg * 8 + lane;
                if (lane < 8 && kk < P) {
                    t /= (double)Ns;
                    if (rhs_mode) {
                        q[kk] = t;
                        a.rf[kk] = (float)t;
                    } else {
                        q[kk] = t + a.shift * __ldcg((zs ? pnew : v) + kk);
                    }
                }
            }
            __syncthreads();
        }
        return grid_barrier(a.bar, a.err, G);
    };

    // ---------------- right-hand side
    if (df_op) {
        if (!op_df(nullptr, a.rhs, true)) return;
    } else if (a.space == 1) {
        colsum_partial(a.O, Ns, P, a.eps, a.upart, gwarp, gwarps, lane);
        if (!grid_barrier(a.bar, a.err, G)) return;
        for (long k = gwarp; k < P; k += gwarps) {
            const double s = colsum_reduce(a.upart, Ns, P, k, lane) / (double)Ns;
            if (lane == 0) {
                a.rhs[k] = s;
                a.rf[k] = (float)s;
            }
        }
        if (!grid_barrier(a.bar, a.err, G)) return;
    } else {
        for (int i = gtid; i < n; i += gthreads) {
            a.rhs[i] = a.eps[i];
            a.rf[i] = (float)a.eps[i];
        }
        if (!grid_barrier(a.bar, a.err, G)) return;
    }
    NQS_PHASE(5);

    // ---------------- preconditioned conjugate gradients in FP64 on the exact
    // operator, preconditioner M = L L^T from the FP32 factor.  Unlike plain
    // iterative refinement this still converges when cond(A) * eps_fp32 is not
    // small.  Scalars come from dot_all, so every CTA takes the same branches.
    // M^{-1} v with rf = float(v): zf = L^{-1} rf, out = L^{-T} zf (row i of
    // L^{-1} reads the 4-aligned groups up to i; the entries right of the
    // diagonal inside a group are the zeros of the diagonal block).
    __shared__ float vk[BD], yk[BD];
    auto precond = [&](double *out) -> bool {
        if (blocked) {
            const int warp = tid >> 5;
            constexpr int RL = BD / 32;
            // yk[t] = sum_c X[t][c] vk[c] over the diagonal block (rows of X at
            // xb + t * ldl; the zeros of the triangle are read too), a warp
            // taking 4 rows at a time with all their loads issued first
            auto diag_gemv = [&](const float *xb, int bs) {
                for (int c = bs + tid; c < BD; c += PS_THREADS) vk[c] = 0.f;
                __syncthreads();
                for (int t0 = 4 * warp; t0 < bs; t0 += 4 * (PS_THREADS / 32)) {
                    float xv[4][RL];
#pragma unroll
                    for (int h = 0; h < 4; h++)
#pragma unroll
                        for (int q = 0; q < RL; q++) {
                            const int t = t0 + h, c = lane + 32 * q;
                            xv[h][q] = (t < bs && c < bs) ? __ldcg(xb + (size_t)t * ldl + c) : 0.f;
                        }
#pragma unroll
                    for (int h = 0; h < 4; h++) {
                        float sacc = 0.f;
#pragma unroll
                        for (int q = 0; q < RL; q++) sacc = fmaf(xv[h][q], vk[lane + 32 * q], sacc);
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
                        if (lane == 0 && t0 + h < bs) yk[t0 + h] = sacc;
                    }
                }
                for (int t = bs + tid; t < BD; t += PS_THREADS) yk[t] = 0.f;   // read (times 0) past a partial block
                __syncthreads();
            };
            // forward, L y = rf (rf is the working vector): y_k = X_kk w_k, then
            // w_i -= sum_c L[i][k0 + c] y_k[c] = sum_c U[k0 + c][i] y_k[c] below the block
            for (int kb = 0; kb < nb; kb++) {
                const int k0 = kb * BD, bs = min(BD, n - k0), k1 = k0 + bs;
                for (int c = tid; c < bs; c += PS_THREADS) vk[c] = __ldcg(a.rf + k0 + c);
                diag_gemv(a.Li + (size_t)k0 * ldl + k0, bs);      // X_kk (lower triangle)
                if (bx == 0)
                    for (int c = tid; c < bs; c += PS_THREADS) a.zf[k0 + c] = yk[c];
                for (int i = k1 + gtid; i < n; i += gthreads) {
                    // 32 loads in flight per round (coalesced over i)
                    const float *u = a.T + (size_t)k0 * n + i;
                    float sacc = 0.f;
                    for (int c0 = 0; c0 < bs; c0 += 32) {
                        float uv[32];
#pragma unroll
                        for (int q = 0; q < 32; q++) uv[q] = c0 + q < bs ? __ldcg(u + (size_t)(c0 + q) * n) : 0.f;
#pragma unroll
                        for (int q = 0; q < 32; q++) sacc = fmaf(uv[q], yk[min(c0 + q, BD - 1)], sacc);
                    }
                    a.rf[i] = __ldcg(a.rf + i) - sacc;
                }
                if (!grid_barrier(a.bar, a.err, G)) return false;
            }
            // backward, L^T z = y (zf is the working vector): z_k = X_kk^T v_k, then
            // v_i -= sum_r L[k0 + r][i] z_k[r] = sum_r U[i][k0 + r] z_k[r] above the block
            for (int kb = nb - 1; kb >= 0; kb--) {
                const int k0 = kb * BD, bs = min(BD, n - k0);
                for (int c = tid; c < bs; c += PS_THREADS) vk[c] = __ldcg(a.zf + k0 + c);
                diag_gemv(a.LiT + (size_t)k0 * ldl + k0, bs);     // X_kk^T (upper triangle)
                if (bx == 0)
                    for (int c = tid; c < bs; c += PS_THREADS) out[k0 + c] = (double)yk[c];
                // a warp takes 4 rows at a time, all BD / 32 loads per row issued first
                for (int i0 = 4 * gwarp; i0 < k0; i0 += 4 * gwarps) {
                    float uv[4][RL];
#pragma unroll
                    for (int h = 0; h < 4; h++)
#pragma unroll
                        for (int q = 0; q < RL; q++) {
                            const int r = lane + 32 * q;
                            uv[h][q] = (i0 + h < k0 && r < bs) ? __ldcg(a.T + (size_t)(i0 + h) * n + k0 + r) : 0.f;
                        }
#pragma unroll
                    for (int h = 0; h < 4; h++) {
                        float sacc = 0.f;
#pragma unroll
                        for (int q = 0; q < RL; q++) sacc = fmaf(uv[h][q], yk[lane + 32 * q], sacc);
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
                        if (lane == 0 && i0 + h < k0) a.zf[i0 + h] = __ldcg(a.zf + i0 + h) - sacc;
                    }
                }
                if (!grid_barrier(a.bar, a.err, G)) return false;
            }
            return true;
        }
        for (int i = gwarp; i < n; i += gwarps) {
            const float t = dot4_range(a.Li + (size_t)i * ldl, a.rf, 0, (i >> 2) + 1, lane);
            if (lane == 0) a.zf[i] = t;
        }
        if (!grid_barrier(a.bar, a.err, G)) return false;
        for (int j = gwarp; j < n; j += gwarps) {
            const float t = dot4_range(a.LiT + (size_t)j * ldl, a.zf, j >> 2, ldl >> 2, lane);
            if (lane == 0) out[j] = (double)t;
        }
        return grid_barrier(a.bar, a.err, G);
    };
    // q = A v: O_c (O_c^T v) / N_s + shift v (samples) or O_c^T (O_c v) / N_s + shift v (parameters)
    auto apply_op = [&](const double *v, double *q) -> bool {
        if (df_op) return op_df(v, q, false);
        if (a.space == 0) {
            colsum_partial(a.O, Ns, P, v, a.upart, gwarp, gwarps, lane);
            if (!grid_barrier(a.bar, a.err, G)) return false;
            for (long k = gwarp; k < P; k += gwarps) {
                const double sk = colsum_reduce(a.upart, Ns, P, k, lane);
                if (lane == 0) a.u[k] = sk;
            }
            if (!grid_barrier(a.bar, a.err, G)) return false;
            const double *us = stage_vec(a.u, P, (double *)psm, PS_SMEM / 8);
            for (int i = gwarp; i < Ns; i += gwarps) {
                const double d = us == a.u ? rowdot<true>(a.O + (size_t)i * P, P, us, lane)
                                           : rowdot<false>(a.O + (size_t)i * P, P, us, lane);
                if (lane == 0) q[i] = d / (double)Ns + a.shift * __ldcg(v + i);
            }
        } else {
            const double *vs = stage_vec(v, P, (double *)psm, PS_SMEM / 8);
            for (int i = gwarp; i < Ns; i += gwarps) {
                const double d = vs == v ? rowdot<true>(a.O + (size_t)i * P, P, vs, lane)
                                         : rowdot<false>(a.O + (size_t)i * P, P, vs, lane);
                if (lane == 0) a.u[i] = d;
            }
            if (!grid_barrier(a.bar, a.err, G)) return false;
            colsum_partial(a.O, Ns, P, a.u, a.upart, gwarp, gwarps, lane);
            if (!grid_barrier(a.bar, a.err, G)) return false;
            for (long k = gwarp; k < P; k += gwarps) {
                const double sk = colsum_reduce(a.upart, Ns, P, k, lane);
                if (lane == 0) q[k] = sk / (double)Ns + a.shift * __ldcg(v + k);
            }
        }
        return grid_barrier(a.bar, a.err, G);
    };
    __shared__ double red[2 * (PS_THREADS / 32)];
    // The double-float operator with L^{-1} (n < 4608): CG with two grid barriers fewer per
    // iteration.  The direction p is formed inside the operator (op_df), and the
    // preconditioner stages float(r - alpha q) in shared memory itself (precond_from), so
    // the residual update needs no barrier before it; p and r alternate between two
    // buffers, as the update of one and the reads of the other overlap.
    auto precond_from = [&](const double *rs, const double *qs, double alpha, double *out) -> bool {
        float *rfs = psm;
        for (int j = tid; j < ldl; j += PS_THREADS)
            rfs[j] = j < n ? (float)(qs ? __fma_rn(-alpha, __ldcg(qs + j), __ldcg(rs + j)) : __ldcg(rs + j)) : 0.f;
        __syncthreads();
        for (int i = gwarp; i < n; i += gwarps) {
            const float t = dot4_range_sv(a.Li + (size_t)i * ldl, rfs, 0, (i >> 2) + 1, lane);
            if (lane == 0) a.zf[i] = t;
        }
        if (!grid_barrier(a.bar, a.err, G)) return false;
        for (int j = gwarp; j < n; j += gwarps) {
            const float t = dot4_range(a.LiT + (size_t)j * ldl, a.zf, j >> 2, ldl >> 2, lane);
            if (lane == 0) out[j] = (double)t;
        }
        return grid_barrier(a.bar, a.err, G);
    };
    if (df_op && !blocked) {
        if (!precond_from(a.rhs, nullptr, 0.0, a.x)) return;     // x0 = M^{-1} rhs
        NQS_PHASE(4);
        if (!op_df(a.x, a.q, false)) return;
        NQS_PHASE(5);
        for (int i = gtid; i < n; i += gthreads) a.r[i] = __fma_rn(-1.0, __ldcg(a.q + i), __ldcg(a.rhs + i));
        if (!precond_from(a.rhs, a.q, 1.0, a.z)) return;
        NQS_PHASE(4);
        const double bb = dot_all(a.rhs, a.rhs, n, red);
        const double2 zr0 = dot_all2<true>(a.r, a.z, a.r, n, red);
        double rho = zr0.x, rr = zr0.y, beta = 0.0;
        double *rc = a.r, *rn = a.r2, *pc = a.p, *pn = a.u;
        int it = 0;
        for (; it < a.sweeps && rr > CG_RTOL * CG_RTOL * bb && rho > 0.0; it++) {
            if (!op_df(nullptr, a.q, false, a.z, it == 0 ? nullptr : pc, beta, pn)) return;
            NQS_PHASE(5);
            const double pq = dot_all(pn, a.q, n, red);
            if (!(pq > 0.0)) break;
            const double alpha = rho / pq;
            for (int i = gtid; i < n; i += gthreads) {
                a.x[i] = __fma_rn(alpha, __ldcg(pn + i), __ldcg(a.x + i));
                rn[i] = __fma_rn(-alpha, __ldcg(a.q + i), __ldcg(rc + i));
            }
            NQS_PHASE(-1);
            if (!precond_from(rc, a.q, alpha, a.z)) return;
            NQS_PHASE(4);
            const double2 zr = dot_all2<true>(rn, a.z, rn, n, red);
            beta = zr.x / rho;
            rho = zr.x;
            rr = zr.y;
            double *t = rc;
            rc = rn;
            rn = t;
            t = pc;
            pc = pn;
            pn = t;
        }
        if (bx == 0 && tid == 0) {
            a.nrm[0] = rr;
            a.nrm[1] = bb;
            a.nrm[2] = (double)it;
        }
        if (timing) {
            tacc[6] = gtimer() - tstart;
            for (int k = 0; k < 7; k++) a.tm[k] = tacc[k];
        }
        return;
    }
    if (!precond(a.x)) return;                          // x0 = M^{-1} rhs
    NQS_PHASE(4);
    // phase 5: the operator (and the right-hand side above); the vector updates, the dots
    // and their barriers are left out of every slot (total minus the slots)
    if (!apply_op(a.x, a.q)) return;
    NQS_PHASE(5);
    for (int i = gtid; i < n; i += gthreads) {
        const double ri = __ldcg(a.rhs + i) - __ldcg(a.q + i);
        a.r[i] = ri;
        a.rf[i] = (float)ri;
    }
    if (!grid_barrier(a.bar, a.err, G)) return;
    NQS_PHASE(-1);
    if (!precond(a.z)) return;
    NQS_PHASE(4);
    const double bb = dot_all(a.rhs, a.rhs, n, red);
    const double2 zr0 = dot_all2<true>(a.r, a.z, a.r, n, red);
    double rho = zr0.x, rr = zr0.y, beta = 0.0;
    int it = 0;
    for (; it < a.sweeps && rr > CG_RTOL * CG_RTOL * bb && rho > 0.0; it++) {
        for (int i = gtid; i < n; i += gthreads)
            a.p[i] = it == 0 ? __ldcg(a.z + i) : __ldcg(a.z + i) + beta * __ldcg(a.p + i);
        if (!grid_barrier(a.bar, a.err, G)) return;
        NQS_PHASE(-1);
        if (!apply_op(a.p, a.q)) return;
        NQS_PHASE(5);
        const double pq = dot_all(a.p, a.q, n, red);
        if (!(pq > 0.0)) break;
        const double alpha = rho / pq;
        for (int i = gtid; i < n; i += gthreads) {
            a.x[i] = __ldcg(a.x + i) + alpha * __ldcg(a.p + i);
            const double ri = __ldcg(a.r + i) - alpha * __ldcg(a.q + i);
            a.r[i] = ri;
            a.rf[i] = (float)ri;
        }
        if (!grid_barrier(a.bar, a.err, G)) return;
        NQS_PHASE(-1);
        if (!precond(a.z)) return;
        NQS_PHASE(4);
        const double2 zr = dot_all2<true>(a.r, a.z, a.r, n, red);
        const double rho1 = zr.x;
        rr = zr.y;
        beta = rho1 / rho;
        rho = rho1;
    }
    if (bx == 0 && tid == 0) {
        a.nrm[0] = rr;
        a.nrm[1] = bb;
        a.nrm[2] = (double)it;
    }
    if (timing) {
        tacc[6] = gtimer() - tstart;
        for (int k = 0; k < 7; k++) a.tm[k] = tacc[k];     // [7]: summed by the block owners
    }
#undef NQS_PHASE
}

// Per-CTA setup of the tensor-core state: two mbarriers, 128 TMEM columns
// (released again after the body, whichever way it returned).
__device__ __forceinline__ void tc_setup(TcState &ts, uint64_t *mbar, uint32_t *slot, int *err) {
    extern __shared__ float psm[];
    const uint32_t base = smem_u32(psm);
    ts.sm = (uint8_t *)psm + (((base + 1023u) & ~1023u) - base);
    ts.mbar = mbar;
    ts.cnt[0] = ts.cnt[1] = 0;
    ts.err = err;
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(TT)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    ts.tmem = *slot;
}

__device__ __forceinline__ void tc_teardown(const TcState &ts) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(ts.tmem), "r"(TT) : "memory");
}

__global__ void __launch_bounds__(PS_THREADS, 1) k_factor_refine(FrArgs a) {
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t slot;
    TcState ts;
    tc_setup(ts, mbar, &slot, a.err);
    if (a.bd == BD_LARGE) fr_body<BD_LARGE>(a, blockIdx.x, gridDim.x, ts);
    else fr_body<BD_SMALL>(a, blockIdx.x, gridDim.x, ts);
    tc_teardown(ts);
}

// A batch of independent systems in one cooperative launch: system i owns the
// CTAs [cta0[i], cta0[i] + nctas[i]) and has its own barrier, status and error
// words; cta_sys maps a CTA to its system.
__global__ void __launch_bounds__(PS_THREADS, 1) k_factor_refine_batch(const FrArgs *__restrict__ sys,
                                                                       const int *__restrict__ cta_sys,
                                                                       const int *__restrict__ cta0,
                                                                       const int *__restrict__ nctas) {
    const int i = cta_sys[blockIdx.x];
    const FrArgs a = sys[i];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t slot;
    TcState ts;
    tc_setup(ts, mbar, &slot, a.err);
    if (a.bd == BD_LARGE) fr_body<BD_LARGE>(a, blockIdx.x - cta0[i], nctas[i], ts);
    else fr_body<BD_SMALL>(a, blockIdx.x - cta0[i], nctas[i], ts);
    tc_teardown(ts);
}

// ---------------------------------------------------------------- driver
struct MixedWs {
    DevBuf<float> hi, lo, T, Tp, Li, LiT, rf, zf, uh, ul, xh, xl, oh, ol;
    DevBuf<double> rhs, r, r2, u, upart, nrm, p, q, z;
    DevBuf<unsigned> bar;
    DevBuf<int> status;
    DevBuf<unsigned long long> tm;
    long rows_pad = 0, k_pad = 0;     // operand layout of hi / lo
    int space = -1;
    int n = 0;                        // order of the last system (pad columns of Li zeroed for it)
};
static MixedWs g_mx;

struct MixedPlan {
    bool split;       // tensor-core Gram with one CTA per (tile, third of K)
    int space;        // 0 samples, 1 parameters
    int n;            // order of the solved system
    long rows_pad;    // Gram operand rows (n padded to TC_M)
    long k_pad;       // Gram operand K (the other dimension padded to TC_K)
};

static MixedPlan plan_mixed(int Ns, long P, int space_opt, int passes) {
    MixedPlan p;
    p.space = space_opt == 1 ? 0 : space_opt == 2 ? 1 : ((long)Ns > P ? 1 : 0);
    const long rows = p.space ? P : Ns, k = p.space ? Ns : P;
    p.n = (int)rows;
    p.rows_pad = (rows + TC_M - 1) / TC_M * TC_M;
    p.k_pad = (k + TC_K - 1) / TC_K * TC_K;
    const long nt = p.rows_pad / TC_M;
    p.split = nt * (nt + 1) / 2 < ctx().sm_count;       // fewer tiles than SMs: split K in three
    return p;
}

// Param-space operand: hi[k][i] = tf32(O_c[i][k]) (row pitch ldn), via 32 x 32
// shared-memory transposes; O is centred in place as in k_center_split.
__global__ void k_center_split_t(double *O, int Ns, long P, const double *__restrict__ gm, float *hi, float *lo,
                                 long ldn, float *oh, float *ol) {
    __shared__ float th[32][33], tl[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
    const long tk = (P + 31) / 32, ti = (Ns + 31) / 32;
    for (long t = blockIdx.x; t < tk * ti; t += gridDim.x) {
        const long i0 = (t / tk) * 32, k0 = (t % tk) * 32;
        for (int r = ty; r < 32; r += 8) {
            const long i = i0 + r, k = k0 + tx;
            float h = 0.f, l = 0.f;
            if (i < Ns && k < P) {
                const double x = O[i * P + k] - gm[k];
                O[i * P + k] = x;
                float xh, xl;
                split_f64_words(x, xh, xl);
                h = tf32_rna(xh);
                l = tf32_rna(xh - h);
                if (oh) {                                   // the double-float words of O_c
                    oh[i * P + k] = xh;
                    ol[i * P + k] = xl;
                }
            }
            th[r][tx] = h;
            tl[r][tx] = l;
        }
        __syncthreads();
        for (int r = ty; r < 32; r += 8) {
            const long k = k0 + r, i = i0 + tx;
            if (k < P && i < Ns) {
                hi[k * ldn + i] = th[tx][r];
                lo[k * ldn + i] = tl[tx][r];
            }
        }
        __syncthreads();
    }
}

// Enqueue the whole mixed solve with no host synchronisation: centring and
// split, tensor-core Gram, then the cooperative factor / inverse / refinement
// kernel.  A broken factor is reported through status[0].
// Front of the mixed solve: status words, centring and TF32 split, tensor-core Gram.
static void enqueue_front(MixedWs &w, const MixedPlan &pl, double *O, const double *gm, int Ns, long P, double shift,
                          int passes, const CUtensorMap &mh, const CUtensorMap &ml, int *err, cudaStream_t st,
                          bool with_split = true) {
    cudaMemsetAsync(w.status.p, 0xff, 2 * sizeof(int), st);
    cudaMemsetAsync(err, 0, sizeof(int), st);
    if (!with_split) {
    } else if (pl.space == 0) {
        NQS_LAUNCH("center_split");
        k_center_split<<<ctx().sm_count * 8, 256, 0, st>>>(O, Ns, P, gm, w.hi.p, w.lo.p, pl.k_pad);
    } else {
        NQS_LAUNCH("center_split_t");
        const bool df = df_words_ok(P) && w.oh.n >= (size_t)Ns * P;
        k_center_split_t<<<ctx().sm_count * 8, dim3(32, 8), 0, st>>>(O, Ns, P, gm, w.hi.p, w.lo.p, pl.k_pad,
                                                                    df ? w.oh.p : nullptr, df ? w.ol.p : nullptr);
    }
    GramTcArgs g;
    g.kt_total = (int)(pl.k_pad / TC_K);
    g.kt_per_seg = pl.split ? (g.kt_total + 2) / 3 : g.kt_total;
    g.nseg = passes >= 3 ? 3 : 1;
    g.scale = (float)(1.0 / (double)Ns);
    g.shift = (float)shift;
    g.C = w.T.p;
    g.n = pl.n;
    g.err = err;
    const int nt = (int)(pl.rows_pad / TC_M);
    g.split = pl.split ? 1 : 0;
    if (pl.split) {
        // few lower-triangular tiles (parameter space): one CTA per tile and third of K
        g.C = w.Tp.p;
        {
            NQS_LAUNCH("gram_tc");
            k_gram_tf32_tc<<<dim3(nt * (nt + 1) / 2, 3), 128, TC_SMEM, st>>>(mh, ml, g);
        }
        NQS_LAUNCH("gram_sum");
        k_gram_sum<<<std::min(pl.n, 65535), 256, 0, st>>>(w.Tp.p, pl.n, g.scale, g.shift, w.T.p);
    } else {
        NQS_LAUNCH("gram_tc");
        k_gram_tf32_tc<<<nt * (nt + 1) / 2, 128, TC_SMEM, st>>>(mh, ml, g);
    }
}

static FrArgs make_frargs(MixedWs &w, const MixedPlan &pl, double *O, const double *eps, int Ns, long P, double shift,
                          int sweeps, double *x, int *err) {
    FrArgs fa;
    fa.T = w.T.p;
    fa.Li = w.Li.p;
    fa.LiT = w.LiT.p;
    fa.n = pl.n;
    fa.ldl = (pl.n + 31) / 32 * 32;
    fa.space = pl.space;
    fa.O = O;
    fa.Ns = Ns;
    fa.P = P;
    fa.eps = eps;
    fa.shift = shift;
    fa.x = x;
    fa.rhs = w.rhs.p;
    fa.r = w.r.p;
    fa.r2 = w.r2.p;
    fa.u = w.u.p;
    fa.upart = w.upart.p;
    fa.p = w.p.p;
    fa.q = w.q.p;
    fa.z = w.z.p;
    fa.rf = w.rf.p;
    fa.uh = w.uh.p;
    fa.ul = w.ul.p;
    fa.xh = w.xh.p;
    fa.xl = w.xl.p;
    const bool df = pl.space == 1 && df_words_ok(P) && w.oh.n >= (size_t)Ns * P;
    fa.oh = df ? w.oh.p : nullptr;
    fa.ol = df ? w.ol.p : nullptr;
    fa.df_rows = df_chunk_rows(Ns);
    fa.bd = pl.n >= BD_SWITCH ? BD_LARGE : BD_SMALL;
    fa.zf = w.zf.p;
    fa.nrm = w.nrm.p;
    fa.sweeps = sweeps;
    fa.status = w.status.p;
    fa.bar = w.bar.p;
    fa.err = err;
    fa.tm = w.tm.p;
    return fa;
}

// Zeroed words and vectors the factor / refinement kernel expects.
static void enqueue_fr_clear(MixedWs &w, const FrArgs &fa, cudaStream_t st) {
    cudaMemsetAsync(w.bar.p, 0, 8 * sizeof(unsigned), st);
    cudaMemsetAsync(w.tm.p, 0, 8 * sizeof(unsigned long long), st);
    cudaMemsetAsync(w.rf.p, 0, sizeof(float) * fa.ldl, st);
    cudaMemsetAsync(w.zf.p, 0, sizeof(float) * fa.ldl, st);
}

static void enqueue_mixed(const MixedPlan &pl, double *O, const double *gm, const double *eps, int Ns, long P,
                          double shift, int sweeps, int passes, double *x, const CUtensorMap &mh,
                          const CUtensorMap &ml, int *err, cudaStream_t st) {
    MixedWs &w = g_mx;
    enqueue_front(w, pl, O, gm, Ns, P, shift, passes, mh, ml, err, st);
    const FrArgs fa = make_frargs(w, pl, O, eps, Ns, P, shift, sweeps, x, err);
    enqueue_fr_clear(w, fa, st);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)ctx().sm_count);
    lc.blockDim = dim3(PS_THREADS);
    lc.dynamicSmemBytes = PS_SMEM;
    lc.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    {
        NQS_LAUNCH("factor_refine");
        cudaLaunchKernelEx(&lc, k_factor_refine, fa);
    }
}

// Buffers of a workspace for plan pl; *moved reports reallocation.
static bool prepare_ws(MixedWs &w, const MixedPlan &pl, int Ns, long P, cudaStream_t st, bool *moved) {
    const int n = pl.n;
    if (pl.rows_pad != w.rows_pad || pl.k_pad != w.k_pad || pl.space != w.space) {
        const size_t ne = (size_t)pl.rows_pad * pl.k_pad;
        if (!w.hi.ensure(ne) || !w.lo.ensure(ne)) return false;
        if (!NQS_CUDA(cudaMemsetAsync(w.hi.p, 0, sizeof(float) * ne, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.lo.p, 0, sizeof(float) * ne, st)))
            return false;
        w.rows_pad = pl.rows_pad;
        w.k_pad = pl.k_pad;
        w.space = pl.space;
        *moved = true;
    }
    const long big = (long)Ns > P ? (long)Ns : P;
    const void *before[23] = {w.T.p, w.Li.p, w.LiT.p, w.rf.p, w.zf.p, w.rhs.p, w.r.p, w.u.p, w.upart.p,
                              w.nrm.p, w.bar.p, w.tm.p, w.Tp.p, w.p.p, w.q.p, w.z.p, w.uh.p, w.ul.p, w.xh.p, w.xl.p,
                              w.oh.p, w.ol.p, w.r2.p};
    const int ldl = (n + 31) / 32 * 32;
    // split U^T: a trailing tile starting at row k1 + 128 bi reaches row n + 126 at most; pad rows read as zero.
    // Sized for the wide diagonal block so a batch's autotuner can pick either width.
    const size_t nu = (size_t)(n + TT) * BD_LARGE;
    if (!w.T.ensure((size_t)n * n) || !w.Li.ensure((size_t)n * ldl) || !w.LiT.ensure((size_t)n * ldl) ||
        !w.rf.ensure(ldl) || !w.zf.ensure(ldl) || !w.rhs.ensure(n) || !w.r.ensure(n) || !w.r2.ensure(n) ||
        !w.u.ensure(big) ||
        !w.p.ensure(n) || !w.q.ensure(n) || !w.z.ensure(n) || !w.uh.ensure(nu) || !w.ul.ensure(nu) ||
        !w.xh.ensure(nu) || !w.xl.ensure(nu) ||
        (pl.space == 1 && df_words_ok(P) && (!w.oh.ensure((size_t)Ns * P) || !w.ol.ensure((size_t)Ns * P))) ||
        !w.upart.ensure((size_t)std::max((Ns + 31) / 32, (Ns + df_chunk_rows(Ns) - 1) / df_chunk_rows(Ns)) * P) ||
        !w.nrm.ensure(3) ||
        !w.status.ensure(2) ||
        !w.bar.ensure(8) || !w.tm.ensure(8) || (pl.split && !w.Tp.ensure(3 * (size_t)n * n)))
        return false;
    const void *after[23] = {w.T.p, w.Li.p, w.LiT.p, w.rf.p, w.zf.p, w.rhs.p, w.r.p, w.u.p, w.upart.p,
                             w.nrm.p, w.bar.p, w.tm.p, w.Tp.p, w.p.p, w.q.p, w.z.p, w.uh.p, w.ul.p, w.xh.p, w.xl.p,
                             w.oh.p, w.ol.p, w.r2.p};
    for (int i = 0; i < 23; i++) *moved |= before[i] != after[i];
    if (*moved || w.n != n) {
        // the pad columns of L^{-1} are read (as zeros) by the vectorised solves,
        // the pad rows of the split U^T and X^T by the tensor-core tiles
        if (!NQS_CUDA(cudaMemsetAsync(w.Li.p, 0, sizeof(float) * (size_t)n * ldl, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.LiT.p, 0, sizeof(float) * (size_t)n * ldl, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.uh.p, 0, sizeof(float) * w.uh.n, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.ul.p, 0, sizeof(float) * w.ul.n, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.xh.p, 0, sizeof(float) * w.xh.n, st)) ||
            !NQS_CUDA(cudaMemsetAsync(w.xl.p, 0, sizeof(float) * w.xl.n, st)))
            return false;
        w.n = n;
        *moved = true;
    }
    return true;
}

static bool ensure_attrs() {
    static bool attr = false;
    if (attr) return true;
    if (!NQS_CUDA(cudaFuncSetAttribute(k_gram_tf32_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM)) ||
        !NQS_CUDA(cudaFuncSetAttribute(k_factor_refine, cudaFuncAttributeMaxDynamicSharedMemorySize, PS_SMEM)) ||
        !NQS_CUDA(cudaFuncSetAttribute(k_factor_refine_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, PS_SMEM)))
        return false;
    int per_sm = 0;
    if (!NQS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_factor_refine, PS_THREADS, PS_SMEM)))
        return false;
    if (per_sm < 1) {
        set_error("factor / refinement kernel does not fit on an SM");
        return false;
    }
    attr = true;
    return true;
}

// The launch sequence above is fixed for given buffers and sizes: it is
// captured once into a CUDA graph and replayed every step.  Per-kernel
// profiling runs the sequence uncaptured.
struct MixedGraph {
    cudaGraphExec_t exec = nullptr;
    const void *key[5] = {};
    int Ns = 0, sweeps = -1, passes = -1, space = -1;
    long P = 0;
    double shift = 0.0;
    long kernels = 0;
};
static MixedGraph g_mgraph;

bool minsr_mixed_solve(double *O, const double *gm, const double *eps, int Ns, long P, double shift, int sweeps,
                       int passes, int space_opt, double *y, double *delta, bool *param_space, double *out_resid,
                       int *out_fail, const MixedAfterLaunch &after_launch) {
    Context &c = ctx();
    cudaStream_t st = c.stream;
    MixedWs &w = g_mx;
    const MixedPlan pl = plan_mixed(Ns, P, space_opt, passes);
    bool moved = false;
    if (!prepare_ws(w, pl, Ns, P, st, &moved)) return false;
    static DevBuf<int> err;
    if (!err.ensure(1) || !ensure_attrs()) return false;
    CUtensorMap mh, ml;
    if (!make_map(&mh, w.hi.p, pl.rows_pad, pl.k_pad) || !make_map(&ml, w.lo.p, pl.rows_pad, pl.k_pad))
        return false;
    double *x = pl.space ? delta : y;

    if (c.profiling) {
        enqueue_mixed(pl, O, gm, eps, Ns, P, shift, sweeps, passes, x, mh, ml, err.p, st);
    } else {
        MixedGraph &Gr = g_mgraph;
        const void *key[5] = {O, gm, eps, x, w.hi.p};
        bool same = Gr.exec && !moved && Gr.Ns == Ns && Gr.P == P && Gr.sweeps == sweeps &&
                    Gr.passes == passes && Gr.shift == shift && Gr.space == pl.space;
        for (int i = 0; i < 5 && same; i++) same = Gr.key[i] == key[i];
        if (!same) {
            if (Gr.exec) cudaGraphExecDestroy(Gr.exec);
            Gr.exec = nullptr;
            cudaGraph_t graph;
            const long l0 = c.launches;
            if (!NQS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal))) return false;
            enqueue_mixed(pl, O, gm, eps, Ns, P, shift, sweeps, passes, x, mh, ml, err.p, st);
            if (!NQS_CUDA(cudaStreamEndCapture(st, &graph))) return false;
            Gr.kernels = c.launches - l0;
            c.launches = l0;
            const bool ok = NQS_CUDA(cudaGraphInstantiate(&Gr.exec, graph, 0));
            cudaGraphDestroy(graph);
            if (!ok) {
                Gr.exec = nullptr;
                return false;
            }
            for (int i = 0; i < 5; i++) Gr.key[i] = key[i];
            Gr.Ns = Ns;
            Gr.P = P;
            Gr.sweeps = sweeps;
            Gr.passes = passes;
            Gr.shift = shift;
            Gr.space = pl.space;
        }
        if (!NQS_CUDA(cudaGraphLaunch(Gr.exec, st))) return false;
        c.launches += Gr.kernels;
    }
    if (after_launch && !after_launch(w.status.p, err.p, w.nrm.p, pl.space == 1)) return false;
    int hs[2] = {-1, 0};
    double h[3] = {0.0, 0.0, 0.0};
    unsigned long long tns[8] = {};
    if (!NQS_CUDA(cudaMemcpyAsync(&hs[0], w.status.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(tns, w.tm.p, sizeof(tns), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(&hs[1], err.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(h, w.nrm.p, sizeof(h), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return false;
    if (hs[1]) {
        set_error(hs[1] == 2 ? "mixed solve: grid barrier timed out"
                             : "tensor-core Gram timed out waiting on its pipeline");
        return false;
    }
    *param_space = pl.space == 1;
    *out_resid = h[1] > 0 ? sqrt(h[0] / h[1]) : 0.0;
    // a factor too inaccurate for the CG to reach the residual bound counts as
    // a breakdown (the caller solves the step in FP64)
    *out_fail = hs[0] >= 0 ? hs[0] : (*out_resid > MIXED_RESID_MAX || !(*out_resid == *out_resid)) ? pl.n : -1;
    step_stats().refine_sweeps = (int)h[2];
    for (int k = 0; k < 8; k++) step_stats().phase_us[k] = 1e-3 * (double)tns[k];
    return NQS_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------- CG-SR
// The CG solve of (S + eps I) d = F with S v = O^T (O v) / N_s - <O> (<O> . v)
// (src/nqs/nqs_optimizer.c:44-139: qgt_apply, cg_solve) as one cooperative
// launch: every iteration is the operator (rows, partial column sums, column
// reduce) and the vector updates separated by bounded grid barriers, with the
// scalars from dot_all so every CTA takes the same branches.  Upstream
// semantics: d0 = 0, r0 = p0 = F; stop when r.r <= tol^2 r0.r0 (converged) or
// |p.Ap| < 1e-30 (Krylov breakdown, unconverged) or after max_iters.  With a
// second matrix O2 (the imaginary part I of a complex O = R + i I) the operator
// is the holomorphic one, G v = fac [(R^T R v + I^T I v) / N_s - <R> (<R>.v)
// - <I> (<I>.v)] + eps v (src/nqs/nqs_optimizer.c:317-356, fac = 2).
struct CgArgs {
    const double *O;      // [N_s][N_p] (uncentred)
    int Ns;
    long P;
    const double *F, *gm; // force, column means
    const double *O2, *gm2;   // optional second matrix and its column means
    double fac;               // operator factor (1 real, 2 holomorphic)
    double eps, tol;
    int max_iters;
    double *d, *r, *p, *Ap, *u, *upart, *u2, *upart2;
    double *scal;         // S_RS, S_RS0, S_PAP
    int *status;          // I_DONE, I_ITERS, I_CONV
    unsigned *bar;
    int *err;
};

__global__ void __launch_bounds__(PS_THREADS, 1) k_cg_sr(CgArgs a) {
    __shared__ double red[PS_THREADS / 32];
    const int G = gridDim.x, bx = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    const int gtid = bx * PS_THREADS + tid, gthreads = G * PS_THREADS;
    const int gwarp = bx * (PS_THREADS / 32) + (tid >> 5), gwarps = G * (PS_THREADS / 32);
    const long P = a.P;
    const int Ns = a.Ns, np = (int)P;
    for (long k = gtid; k < P; k += gthreads) {
        a.d[k] = 0.0;
        a.r[k] = a.F[k];
        a.p[k] = a.F[k];
    }
    const double rs0 = dot_all(a.F, a.F, np, red);
    double rs = rs0;
    int it = 0, done = 0, conv = 0;
    double pap_last = 0.0;
    if (!grid_barrier(a.bar, a.err, G)) return;
    for (; it < a.max_iters; it++) {
        // u = O p (and u2 = O2 p)
        for (int i = gwarp; i < Ns; i += gwarps) {
            const double v = rowdot<true>(a.O + (size_t)i * P, P, a.p, lane);
            if (lane == 0) a.u[i] = v;
            if (a.O2) {
                const double v2 = rowdot<true>(a.O2 + (size_t)i * P, P, a.p, lane);
                if (lane == 0) a.u2[i] = v2;
            }
        }
        if (!grid_barrier(a.bar, a.err, G)) return;
        colsum_partial(a.O, Ns, P, a.u, a.upart, gwarp, gwarps, lane);
        if (a.O2) colsum_partial(a.O2, Ns, P, a.u2, a.upart2, gwarp, gwarps, lane);
        // <u>, <u2> (the same in every CTA)
        auto mean_all = [&](const double *v) {
            double sacc = 0.0;
            for (int i = tid; i < Ns; i += PS_THREADS) sacc += __ldcg(v + i);
            sacc = warp_sum(sacc);
            __syncthreads();
            if (lane == 0) red[tid >> 5] = sacc;
            __syncthreads();
            double m = 0.0;
            for (int w = 0; w < PS_THREADS / 32; w++) m += red[w];
            return m / (double)Ns;
        };
        const double um = mean_all(a.u), um2 = a.O2 ? mean_all(a.u2) : 0.0;
        if (!grid_barrier(a.bar, a.err, G)) return;
        for (long k = gwarp; k < P; k += gwarps) {
            double sk = colsum_reduce(a.upart, Ns, P, k, lane);
            if (a.O2) {
                const double sk2 = colsum_reduce(a.upart2, Ns, P, k, lane);
                if (lane == 0)
                    a.Ap[k] = a.fac * ((sk + sk2) / (double)Ns - __ldcg(a.gm + k) * um - __ldcg(a.gm2 + k) * um2) +
                              a.eps * __ldcg(a.p + k);
            } else if (lane == 0) {
                a.Ap[k] = sk / (double)Ns - __ldcg(a.gm + k) * um + a.eps * __ldcg(a.p + k);
            }
        }
        if (!grid_barrier(a.bar, a.err, G)) return;
        const double pap = dot_all(a.p, a.Ap, np, red);
        if (!(fabs(pap) >= 1e-30)) {                    // Krylov breakdown: stop, unconverged
            done = 1;
            pap_last = pap;
            break;
        }
        const double alpha = rs / pap;
        for (long k = gtid; k < P; k += gthreads) {
            a.d[k] = __ldcg(a.d + k) + alpha * __ldcg(a.p + k);
            a.r[k] = __ldcg(a.r + k) - alpha * __ldcg(a.Ap + k);
        }
        if (!grid_barrier(a.bar, a.err, G)) return;
        const double rs_new = dot_all(a.r, a.r, np, red);
        if (rs_new <= a.tol * a.tol * rs0) {
            done = 1;
            conv = 1;
            it++;
            break;
        }
        const double beta = rs_new / rs;
        for (long k = gtid; k < P; k += gthreads) a.p[k] = __ldcg(a.r + k) + beta * __ldcg(a.p + k);
        rs = rs_new;
        if (!grid_barrier(a.bar, a.err, G)) return;
    }
    if (bx == 0 && tid == 0) {
        a.scal[S_RS] = rs;
        a.scal[S_RS0] = rs0;
        a.scal[S_PAP] = pap_last;
        a.status[I_DONE] = done;
        a.status[I_CONV] = conv;
        a.status[I_ITERS] = it;
    }
}

bool cg_sr_solve(const double *O, int Ns, long P, const double *F, const double *gm, double eps, double tol,
                 int max_iters, double *d, double *scal, int *status, const double *O2, const double *gm2,
                 double fac) {
    Context &c = ctx();
    cudaStream_t st = c.stream;
    static DevBuf<double> r, p, Ap, u, upart, u2, upart2;
    static DevBuf<unsigned> bar;
    static DevBuf<int> err;
    if (!r.ensure(P) || !p.ensure(P) || !Ap.ensure(P) || !u.ensure(Ns) ||
        !upart.ensure((size_t)((Ns + RCH - 1) / RCH) * P) || !bar.ensure(2) || !err.ensure(1) ||
        (O2 && (!u2.ensure(Ns) || !upart2.ensure((size_t)((Ns + RCH - 1) / RCH) * P))))
        return false;
    if (!NQS_CUDA(cudaMemsetAsync(bar.p, 0, 2 * sizeof(unsigned), st)) ||
        !NQS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st)))
        return false;
    CgArgs a{O,   Ns,  P,   F,    gm,      O2,   gm2,      fac,  eps,   tol,   max_iters, d,
             r.p, p.p, Ap.p, u.p, upart.p, u2.p, upart2.p, scal, status, bar.p, err.p};
    int per_sm = 0;
    if (!NQS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_sr, PS_THREADS, 0))) return false;
    if (per_sm < 1) {
        set_error("CG kernel does not fit on an SM");
        return false;
    }
    // one CTA per 256 KB of Jacobian (at least 8, at most one per SM): a small system
    // (the 1-D TFIM chain: 1024 x 288, 2.4 MB) then synchronises 10 CTAs instead of 152 at
    // its five grid barriers per iteration; the dot products run in every CTA in a fixed
    // order and the column sums are reduced over fixed row chunks, so the result does not
    // depend on the grid size
    const double jac_bytes = 8.0 * (double)Ns * (double)P * (O2 ? 2.0 : 1.0);
    const int grid = std::max(8, std::min(c.sm_count, (int)std::ceil(jac_bytes / (256.0 * 1024.0))));
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3(PS_THREADS);
    lc.dynamicSmemBytes = 0;
    lc.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    {
        NQS_LAUNCH("cg_sr");
        if (!NQS_CUDA(cudaLaunchKernelEx(&lc, k_cg_sr, a))) return false;
    }
    int herr = 0;
    if (!NQS_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return false;
    if (herr) {
        set_error("CG-SR solve: grid barrier timed out");
        return false;
    }
    return true;
}

// ---------------------------------------------------------------- batches of systems
// One system of a batch: its own workspace, tensor maps, status and error words.
struct MixedSys {
    MixedWs w;
    MixedPlan pl{};
    DevBuf<int> err;
    CUtensorMap mh, ml;
    FrArgs fa{};
    double *O = nullptr;
    const double *gm = nullptr;
    int Ns = 0, passes = 3;
    long P = 0;
    double shift = 0.0;
};

MixedSys *mixed_sys_create() { return new MixedSys(); }
void mixed_sys_free(MixedSys *m) { delete m; }

bool mixed_sys_prepare(MixedSys *m, double *O, const double *gm, const double *eps, int Ns, long P, double shift,
                       int sweeps, int passes, int space_opt, double *y, double *delta) {
    cudaStream_t st = ctx().stream;
    m->pl = plan_mixed(Ns, P, space_opt, passes);
    bool moved = false;
    if (!prepare_ws(m->w, m->pl, Ns, P, st, &moved) || !m->err.ensure(1) || !ensure_attrs()) return false;
    if (!make_map(&m->mh, m->w.hi.p, m->pl.rows_pad, m->pl.k_pad) ||
        !make_map(&m->ml, m->w.lo.p, m->pl.rows_pad, m->pl.k_pad))
        return false;
    m->O = O;
    m->gm = gm;
    m->Ns = Ns;
    m->P = P;
    m->shift = shift;
    m->passes = passes;
    m->fa = make_frargs(m->w, m->pl, O, eps, Ns, P, shift, sweeps, m->pl.space ? delta : y, m->err.p);
    m->fa.tm = nullptr;
    return true;
}

// Status words, centring + split (unless the operands are already split), Gram,
// and the cleared words of the factor kernel.
void mixed_sys_front(MixedSys *m, cudaStream_t st, bool with_split) {
    enqueue_front(m->w, m->pl, m->O, m->gm, m->Ns, m->P, m->shift, m->passes, m->mh, m->ml, m->err.p, st, with_split);
    enqueue_fr_clear(m->w, m->fa, st);
}

bool mixed_sys_param_space(const MixedSys *m) { return m->pl.space == 1; }
int mixed_bd_default() { return BD_SWITCH; }
int mixed_sys_order(const MixedSys *m) { return m->pl.n; }
const int *mixed_sys_status(const MixedSys *m) { return m->w.status.p; }
const int *mixed_sys_err(const MixedSys *m) { return m->err.p; }
const double *mixed_sys_nrm(const MixedSys *m) { return m->w.nrm.p; }

struct MixedBatch {
    DevBuf<FrArgs> sys;
    DevBuf<int> cta_sys, cta0, nctas;
    int total = 0, count = 0;
};

// CTAs that can be co-resident for the batched kernel.
int mixed_batch_capacity() {
    if (!ensure_attrs()) return 0;
    int per_sm = 0;
    if (!NQS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_factor_refine_batch, PS_THREADS, PS_SMEM)))
        return 0;
    return per_sm * ctx().sm_count;
}

// bd_from: systems of order >= bd_from factor with 128-wide diagonal blocks, the others
// with 64-wide ones (a tile shape the batch autotuner chooses).
MixedBatch *mixed_batch_create(MixedSys *const *sys, int count, const int *ctas, int bd_from) {
    std::vector<FrArgs> fa((size_t)count);
    std::vector<int> c0((size_t)count), nc((size_t)count), map;
    for (int i = 0; i < count; i++) {
        fa[i] = sys[i]->fa;
        fa[i].bd = sys[i]->pl.n >= bd_from ? BD_LARGE : BD_SMALL;
        c0[i] = (int)map.size();
        nc[i] = ctas[i] > 0 ? ctas[i] : 1;
        for (int k = 0; k < nc[i]; k++) map.push_back(i);
    }
    const int cap = mixed_batch_capacity();
    if ((int)map.size() > cap) {
        set_error("batched solve needs %d co-resident CTAs, the device holds %d", (int)map.size(), cap);
        return nullptr;
    }
    MixedBatch *b = new MixedBatch();
    b->total = (int)map.size();
    b->count = count;
    if (!b->sys.ensure(count) || !b->cta_sys.ensure(map.size()) || !b->cta0.ensure(count) || !b->nctas.ensure(count) ||
        !NQS_CUDA(cudaMemcpy(b->sys.p, fa.data(), sizeof(FrArgs) * count, cudaMemcpyHostToDevice)) ||
        !NQS_CUDA(cudaMemcpy(b->cta_sys.p, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice)) ||
        !NQS_CUDA(cudaMemcpy(b->cta0.p, c0.data(), sizeof(int) * count, cudaMemcpyHostToDevice)) ||
        !NQS_CUDA(cudaMemcpy(b->nctas.p, nc.data(), sizeof(int) * count, cudaMemcpyHostToDevice))) {
        delete b;
        return nullptr;
    }
    return b;
}

void mixed_batch_free(MixedBatch *b) { delete b; }

// Factor, inverse and refinement of every system of the batch in one
// cooperative launch.
bool mixed_batch_launch(MixedBatch *b, cudaStream_t st) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)b->total);
    lc.blockDim = dim3(PS_THREADS);
    lc.dynamicSmemBytes = PS_SMEM;
    lc.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    NQS_LAUNCH("factor_refine_batch");
    const FrArgs *s = b->sys.p;
    const int *m = b->cta_sys.p, *c0 = b->cta0.p, *nc = b->nctas.p;
    return NQS_CUDA(cudaLaunchKernelEx(&lc, k_factor_refine_batch, s, m, c0, nc));
}

}  // namespace nqs

using namespace nqs;

extern "C" {

// Diagnostic: the tensor-core Gram alone on a host matrix O [Ns][P] (FP64,
// used as given, i.e. already centred): T_out [Ns][Ns] (lower triangle) =
// scale * (hi hi^T [+ hi lo^T + lo hi^T]).
int nqs_gpu_set_barrier_budget(unsigned polls) {
    clear_error();
    if (!ensure_context()) return -1;
    const unsigned v = polls ? polls : (1u << 24);
    cudaStream_t st = ctx().stream;
    return NQS_CUDA(cudaMemcpyToSymbolAsync(g_barrier_budget, &v, sizeof(v), 0, cudaMemcpyHostToDevice, st)) &&
                   NQS_CUDA(cudaStreamSynchronize(st))
               ? 0
               : -1;
}

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
    if (ns_pad != w.rows_pad || p_pad != w.k_pad || w.space != 0) {
        if (!w.hi.ensure((size_t)ns_pad * p_pad) || !w.lo.ensure((size_t)ns_pad * p_pad)) return -1;
        NQS_CUDA(cudaMemsetAsync(w.hi.p, 0, sizeof(float) * ns_pad * p_pad, st));
        NQS_CUDA(cudaMemsetAsync(w.lo.p, 0, sizeof(float) * ns_pad * p_pad, st));
        w.rows_pad = ns_pad;
        w.k_pad = p_pad;
        w.space = 0;
    }
    if (!w.T.ensure((size_t)Ns * Ns)) return -1;
    k_center_split<<<ctx().sm_count * 8, 256, 0, st>>>(dO.p, Ns, P, dz.p, w.hi.p, w.lo.p, p_pad);
    CUtensorMap mh, ml;
    if (!make_map(&mh, w.hi.p, ns_pad, p_pad) || !make_map(&ml, w.lo.p, ns_pad, p_pad)) return -1;
    static DevBuf<int> err;
    if (!err.ensure(1)) return -1;
    NQS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    GramTcArgs g;
    g.kt_total = (int)(p_pad / TC_K);
    g.kt_per_seg = g.kt_total;
    g.nseg = passes >= 3 ? 3 : 1;
    g.scale = (float)scale;
    g.shift = 0.f;
    g.C = w.T.p;
    g.n = Ns;
    g.err = err.p;
    g.split = 0;
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
