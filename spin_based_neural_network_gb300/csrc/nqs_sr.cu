// Stochastic reconfiguration on the GPU: MinSR (sample-space Gram + Cholesky)
// and CG-SR (matrix-free QGT), FP64.
//
// Pipeline of one MinSR step (src/nqs/nqs_optimizer.c:1063-1194), every stage
// a kernel on the library stream, no host round trip until the step info:
//   sampler -> fused local estimator (E_loc + Jacobian row O_i)
//   -> energy statistics (compensated) and eps_i = E_i - <E>
//   -> column means <O_k>, centring O_c = O - <O>
//   -> T = O_c O_c^T / N_s + shift I (lower triangle, 64x64 tiles)
//   -> blocked right-looking Cholesky (32-wide panels: diagonal-block factor,
//      panel triangular solve, trailing SYRK update), status word on device
//   -> forward / backward blocked triangular solves
//   -> delta = O_c^T y / N_s, theta -= lr delta, ||delta||.
#include <algorithm>
#include <cuda.h>
#include <math.h>

#include "nqs_amp.cuh"

namespace nqs {

struct Sampler;
bool sampler_produce(Sampler *s, int n, uint64_t **d_out);

// ---------------------------------------------------------------- workspace
struct Workspace {
    DevBuf<double> E, Ei, eps, O, gm, T, T0, y, z, delta, scal, F, r, p, Ap, u, part, y64, d64, es;
    DevBuf<double> Oi, gm2, F2, scal2, eps2, es2;     // holomorphic SR: imaginary halves
    DevBuf<double> la, ar, la_ref, ar_ref, aug;       // excited-state SR: amplitude ratios, augmented means
    DevBuf<double> theta0, kacc;                      // Heun tVMC: parameter snapshot, averaged slope
    DevBuf<int> status;
    DevBuf<uint64_t> batch_bits;
};
static Workspace g_ws;


// ---------------------------------------------------------------- statistics
// Neumaier-compensated sums of E and E^2 (one block), then eps_i = E_i - <E>.
__global__ void k_energy_stats(const double *__restrict__ E, int n, double *scal, double *eps) {
    __shared__ double ss[1024], sc[1024], qs[1024], qc[1024];
    int t = threadIdx.x;
    double s = 0.0, c = 0.0, q = 0.0, qcc = 0.0;
    for (int i = t; i < n; i += blockDim.x) {
        double x = E[i], tt = s + x;
        c += fabs(s) >= fabs(x) ? (s - tt) + x : (x - tt) + s;
        s = tt;
        double x2 = x * x, t2 = q + x2;
        qcc += fabs(q) >= fabs(x2) ? (q - t2) + x2 : (x2 - t2) + q;
        q = t2;
    }
    ss[t] = s; sc[t] = c; qs[t] = q; qc[t] = qcc;
    __syncthreads();
    // pairwise tree over the (sum, compensation) pairs: each merge is an exact
    // TwoSum of the sums plus the two compensations
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (t < o) {
            double a = ss[t], b = ss[t + o], tt = a + b, bb = tt - a;
            double e = (a - (tt - bb)) + (b - bb);
            ss[t] = tt;
            sc[t] = sc[t] + sc[t + o] + e;
            double a2 = qs[t], b2 = qs[t + o], t2 = a2 + b2, b3 = t2 - a2;
            double e2 = (a2 - (t2 - b3)) + (b2 - b3);
            qs[t] = t2;
            qc[t] = qc[t] + qc[t + o] + e2;
        }
        __syncthreads();
    }
    __shared__ double mean;
    if (t == 0) {
        mean = (ss[0] + sc[0]) / (double)n;
        scal[S_EMEAN] = mean;
        scal[S_ESQ] = (qs[0] + qc[0]) / (double)n;
    }
    __syncthreads();
    if (eps)
        for (int i = t; i < n; i += blockDim.x) eps[i] = E[i] - mean;
}

// ---- multi-block statistics.  GB300's FP64 rate is ~2 FMA / clock / SM, so
// the compensated sums and the lag products are spread over blocks of
// ES_CHUNK samples; the last block to finish (an atomic ticket) merges the
// partials in block order, so results do not depend on scheduling.
constexpr int ES_THREADS = 256, ES_CHUNK = 256, ES_LAGS = 16;

static int es_blocks(int n) { return (n + ES_CHUNK - 1) / ES_CHUNK; }

// doubles of scratch enqueue_energy_stats needs for n samples: 2 words of
// tickets (zero on first use) followed by the block partials
size_t energy_scratch_doubles(int n) { return (size_t)es_blocks(n) * (4 + ES_LAGS + 1) + 2; }

__device__ __forceinline__ void two_sum_merge(double &s, double &c, double s2, double c2) {
    const double t = s + s2, bb = t - s;
    c = c + c2 + ((s - (t - bb)) + (s2 - bb));
    s = t;
}

// Sums of E and E^2 with Neumaier compensation per thread, merged by exact
// TwoSum trees; the last block merges the block partials in order and writes
// <E>, <E^2>.
__global__ void __launch_bounds__(ES_THREADS) k_energy_mb(const double *__restrict__ E, int n, double *part,
                                                         unsigned *ticket, double *scal) {
    __shared__ double ss[ES_THREADS], sc[ES_THREADS], qs[ES_THREADS], qc[ES_THREADS];
    __shared__ bool last;
    const int t = threadIdx.x, i0 = blockIdx.x * ES_CHUNK, i1 = min(n, i0 + ES_CHUNK);
    double s = 0.0, c = 0.0, q = 0.0, qcc = 0.0;
    for (int i = i0 + t; i < i1; i += ES_THREADS) {
        const double x = E[i], tt = s + x;
        c += fabs(s) >= fabs(x) ? (s - tt) + x : (x - tt) + s;
        s = tt;
        const double x2 = x * x, t2 = q + x2;
        qcc += fabs(q) >= fabs(x2) ? (q - t2) + x2 : (x2 - t2) + q;
        q = t2;
    }
    ss[t] = s;
    sc[t] = c;
    qs[t] = q;
    qc[t] = qcc;
    __syncthreads();
    for (int o = ES_THREADS / 2; o > 0; o >>= 1) {
        if (t < o) {
            two_sum_merge(ss[t], sc[t], ss[t + o], sc[t + o]);
            two_sum_merge(qs[t], qc[t], qs[t + o], qc[t + o]);
        }
        __syncthreads();
    }
    if (t == 0) {
        double *p = part + (size_t)blockIdx.x * 4;
        p[0] = ss[0];
        p[1] = sc[0];
        p[2] = qs[0];
        p[3] = qc[0];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the block partials, a tile of ES_THREADS blocks at a time, merged by a TwoSum tree over
    // the tile (its depth, not the block count, is the chain of dependent FP64 operations),
    // and the tiles by thread 0 in order
    double S = 0.0, Sc = 0.0, Q = 0.0, Qc = 0.0;
    for (int b0 = 0; b0 < (int)gridDim.x; b0 += ES_THREADS) {
        const int nb = min(ES_THREADS, (int)gridDim.x - b0);
        int w = 1;
        while (w < nb) w <<= 1;
        if (t < w) {
            const bool in = t < nb;
            ss[t] = in ? __ldcg(part + (size_t)(b0 + t) * 4 + 0) : 0.0;
            sc[t] = in ? __ldcg(part + (size_t)(b0 + t) * 4 + 1) : 0.0;
            qs[t] = in ? __ldcg(part + (size_t)(b0 + t) * 4 + 2) : 0.0;
            qc[t] = in ? __ldcg(part + (size_t)(b0 + t) * 4 + 3) : 0.0;
        }
        __syncthreads();
        for (int o = w / 2; o > 0; o >>= 1) {
            if (t < o) {
                two_sum_merge(ss[t], sc[t], ss[t + o], sc[t + o]);
                two_sum_merge(qs[t], qc[t], qs[t + o], qc[t + o]);
            }
            __syncthreads();
        }
        if (t == 0) {
            two_sum_merge(S, Sc, ss[0], sc[0]);
            two_sum_merge(Q, Qc, qs[0], qc[0]);
        }
        __syncthreads();
    }
    if (t != 0) return;
    scal[S_EMEAN] = (S + Sc) / (double)n;
    scal[S_ESQ] = (Q + Qc) / (double)n;
    *ticket = 0;
}

// eps_i = E_i - <E> for every sample, and the lag sums of the integrated
// autocorrelation time of E_loc over C chains whose samples sit at rows
// k * C + c (k = 0 .. K-1): gamma(t) = sum_e eps_e eps_{e + tC} over e < (K - t) C,
// t <= ES_LAGS, as block partials; the last block sums them in block order and
// applies the self-consistent window: tau(M) = 1 + 2 sum_{t=1}^{M} gamma(t) /
// gamma(0) with the smallest M >= 5 tau(M) (Sokal; the automatic window of
// emcee), continuing past ES_LAGS itself (up to 512) when the window is wider.
// ESS = K C / tau.
__global__ void __launch_bounds__(ES_THREADS) k_ess_mb(const double *__restrict__ E, int Ns, int C, double *gpart,
                                                      unsigned *ticket, double *scal, double *eps) {
    __shared__ double red[ES_THREADS / 32][ES_LAGS + 1];
    __shared__ bool last;
    const int t0 = threadIdx.x, lane = t0 & 31, w = t0 >> 5;
    const double mean = scal[S_EMEAN];
    const int i0 = blockIdx.x * ES_CHUNK, i1 = min(Ns, i0 + ES_CHUNK);
    for (int i = i0 + t0; i < i1; i += ES_THREADS) eps[i] = E[i] - mean;
    const int K = C > 0 ? Ns / C : 0, n = K * C;
    const int maxlag = K - 1 < 512 ? K - 1 : 512, T1 = maxlag < ES_LAGS ? maxlag : ES_LAGS;
    if (K < 2) {
        if (blockIdx.x == 0 && t0 == 0) {
            scal[S_TAU] = 1.0;
            scal[S_ESS] = (double)Ns;
        }
        return;
    }
    double g[ES_LAGS + 1];
#pragma unroll
    for (int t = 0; t <= ES_LAGS; t++) g[t] = 0.0;
    for (int e = i0 + t0; e < min(i1, n); e += ES_THREADS) {
        const double a = E[e] - mean;
#pragma unroll
        for (int t = 0; t <= ES_LAGS; t++)
            if (t <= T1 && e < (K - t) * C) g[t] += a * (E[e + t * C] - mean);
    }
    // block sums of the lag products through shared memory (an FP64 butterfly per lag costs
    // 16 cycles per warp add on this GPU's FP64 pipe): thread (lag, seg) sums 32 threads'
    // products, then one thread per lag sums the eight segments, both in a fixed order
    __shared__ double gs[ES_LAGS + 1][ES_THREADS + 1];
#pragma unroll
    for (int t = 0; t <= ES_LAGS; t++) gs[t][t0] = g[t];
    __syncthreads();
    if (t0 < (ES_LAGS + 1) * 8) {
        const int lag = t0 >> 3, seg = t0 & 7;
        double v4[4] = {0.0, 0.0, 0.0, 0.0};          // four chains of eight adds
#pragma unroll
        for (int q = 0; q < 32; q++) v4[q & 3] += gs[lag][32 * seg + q];
        red[seg][lag] = (v4[0] + v4[1]) + (v4[2] + v4[3]);
    }
    __syncthreads();
    if (t0 <= ES_LAGS) {
        double v = 0.0;
        for (int q = 0; q < ES_THREADS / 32; q++) v += red[q][t0];
        gpart[(size_t)blockIdx.x * (ES_LAGS + 1) + t0] = v;
    }
    __threadfence();
    __syncthreads();
    if (t0 == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // gamma(t) in block order; the window over t <= T1
    // the block partials loaded by the whole block (a tile of blocks at a time, into gs),
    // summed per lag in block order
    __shared__ double gam[ES_LAGS + 1];
    {
        constexpr int TB = ES_THREADS;                       // blocks per tile: gs holds [lag][block]
        double v = 0.0;
        for (int b0 = 0; b0 < (int)gridDim.x; b0 += TB) {
            const int nb = min(TB, (int)gridDim.x - b0);
            for (int e = t0; e < nb * (ES_LAGS + 1); e += ES_THREADS) {
                const int b = e / (ES_LAGS + 1), lag = e % (ES_LAGS + 1);
                gs[lag][b] = __ldcg(gpart + (size_t)(b0 + b) * (ES_LAGS + 1) + lag);
            }
            __syncthreads();
            if (t0 <= T1) {
                double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;   // four chains, then in order
                int b = 0;
                for (; b + 3 < nb; b += 4) {
                    v0 += gs[t0][b];
                    v1 += gs[t0][b + 1];
                    v2 += gs[t0][b + 2];
                    v3 += gs[t0][b + 3];
                }
                for (; b < nb; b++) v0 += gs[t0][b];
                v += (v0 + v1) + (v2 + v3);
            }
            __syncthreads();
        }
        if (t0 <= T1) gam[t0] = v / (double)((K - t0) * C);
    }
    __syncthreads();
    __shared__ double s_tau;
    __shared__ int s_done;
    if (t0 == 0) {
        double tau = 1.0;
        int done = 0;
        const double g0 = gam[0];
        if (!(g0 > 0.0)) {
            done = 1;
        } else {
            const double r2 = 2.0 / g0;                 // one division for the whole window
            for (int t = 1; t <= T1; t++) {
                tau += gam[t] * r2;
                if ((double)t >= 5.0 * tau) {
                    done = 1;
                    break;
                }
            }
        }
        s_tau = tau;
        s_done = done || T1 == maxlag;
        *ticket = 0;
    }
    __syncthreads();
    double tau = s_tau;
    if (!s_done) {
        // wide window: further lags by this block (eps of every block is written)
        const double g0 = gam[0];
        for (int t = T1 + 1; t <= maxlag; t++) {
            double v = 0.0;
            const int m = (K - t) * C;
            for (int e = t0; e < m; e += ES_THREADS) v += (E[e] - mean) * (E[e + t * C] - mean);
            v = warp_sum(v);
            __syncthreads();
            if (lane == 0) red[w][0] = v;
            __syncthreads();
            double gt = 0.0;
            for (int q = 0; q < ES_THREADS / 32; q++) gt += red[q][0];
            tau += 2.0 * (gt / (double)m) / g0;
            if ((double)t >= 5.0 * tau) break;
        }
    }
    if (t0 == 0) {
        if (!(tau > 0.0)) tau = 1.0;
        scal[S_TAU] = tau;
        scal[S_ESS] = (double)n / tau;
    }
}

// Column sums of O (and of O_ik E_i for CG-SR): 32 columns x 8 row groups per
// block, coalesced along the row.
__global__ void k_col_stats(const double *__restrict__ O, int Ns, long P, const double *__restrict__ E,
                            const double *__restrict__ scal, double *gm, double *F) {
    __shared__ double a[8][33], b[8][33];
    long k = (long)blockIdx.x * 32 + threadIdx.x;
    double s = 0.0, se = 0.0;
    if (k < P)
        for (int i = threadIdx.y; i < Ns; i += 8) {
            double g = O[(size_t)i * P + k];
            s += g;
            if (F) se += g * E[i];
        }
    a[threadIdx.y][threadIdx.x] = s;
    b[threadIdx.y][threadIdx.x] = se;
    __syncthreads();
    if (threadIdx.y == 0 && k < P) {
        double S = 0.0, SE = 0.0;
        for (int y = 0; y < 8; y++) {
            S += a[y][threadIdx.x];
            SE += b[y][threadIdx.x];
        }
        double m = S / (double)Ns;
        gm[k] = m;
        if (F) F[k] = SE / (double)Ns - m * scal[S_EMEAN];     // src/nqs/nqs_optimizer.c:213-215
    }
}

// The same statistics over a 2-D grid: partial column sums over row chunks
// (32 columns x 8 row groups per block), then a fixed-order sum over the
// chunks (deterministic).  With tickets (one zeroed word per column group), the
// last block of each column group to finish (an atomic ticket; no block waits for
// another) sums the chunks' partials itself and writes the means (and F), so that no
// second kernel is needed; it sets the ticket back to zero.
__global__ void k_col_part(const double *__restrict__ O, int Ns, long P, const double *__restrict__ E, int rows_per,
                           double *part, unsigned *tickets, const double *__restrict__ scal, double *gm, double *F) {
    __shared__ double a[8][33], b[8][33];
    __shared__ bool last;
    const long k = (long)blockIdx.x * 32 + threadIdx.x;
    const int r0 = blockIdx.y * rows_per, r1 = min(Ns, r0 + rows_per);
    // four rows' loads in flight per thread, four partial sums merged in a fixed order
    double s[4] = {0.0, 0.0, 0.0, 0.0}, se[4] = {0.0, 0.0, 0.0, 0.0};
    if (k < P) {
        int i = r0 + threadIdx.y;
        for (; i + 24 < r1; i += 32) {
            double g[4];
#pragma unroll
            for (int h = 0; h < 4; h++) g[h] = O[(size_t)(i + 8 * h) * P + k];
#pragma unroll
            for (int h = 0; h < 4; h++) {
                s[h] += g[h];
                if (E) se[h] += g[h] * E[i + 8 * h];
            }
        }
        for (; i < r1; i += 8) {
            const double g = O[(size_t)i * P + k];
            s[0] += g;
            if (E) se[0] += g * E[i];
        }
    }
    a[threadIdx.y][threadIdx.x] = (s[0] + s[1]) + (s[2] + s[3]);
    b[threadIdx.y][threadIdx.x] = (se[0] + se[1]) + (se[2] + se[3]);
    __syncthreads();
    if (threadIdx.y == 0 && k < P) {
        double S = 0.0, SE = 0.0;
        for (int y = 0; y < 8; y++) {
            S += a[y][threadIdx.x];
            SE += b[y][threadIdx.x];
        }
        part[(size_t)blockIdx.y * 2 * P + k] = S;
        part[(size_t)blockIdx.y * 2 * P + P + k] = SE;
    }
    if (!tickets) return;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) last = atomicAdd(tickets + blockIdx.x, 1u) == gridDim.y - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // thread (x, y) sums chunks y, y + 8, ... of column k; the eight sums are added in order of y
    const int nchunk = (int)gridDim.y;
    double S = 0.0, SE = 0.0;
    if (k < P) {
        for (int c = threadIdx.y; c < nchunk; c += 8) {
            S += __ldcg(part + (size_t)c * 2 * P + k);
            SE += __ldcg(part + (size_t)c * 2 * P + P + k);
        }
    }
    a[threadIdx.y][threadIdx.x] = S;
    b[threadIdx.y][threadIdx.x] = SE;
    __syncthreads();
    if (threadIdx.y == 0 && k < P) {
        double St = 0.0, SEt = 0.0;
        for (int y = 0; y < 8; y++) {
            St += a[y][threadIdx.x];
            SEt += b[y][threadIdx.x];
        }
        const double m = St / (double)Ns;
        gm[k] = m;
        if (F) F[k] = SEt / (double)Ns - m * scal[S_EMEAN];     // src/nqs/nqs_optimizer.c:213-215
    }
    if (threadIdx.x == 0 && threadIdx.y == 0) tickets[blockIdx.x] = 0;
}

__global__ void k_col_fin(const double *__restrict__ part, int nchunk, int Ns, long P, const double *__restrict__ scal,
                          double *gm, double *F) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    // eight chunks' loads in flight, summed in chunk order
    double S = 0.0, SE = 0.0;
    int c = 0;
    for (; c + 7 < nchunk; c += 8) {
        double ps[8], pe[8];
#pragma unroll
        for (int h = 0; h < 8; h++) {
            ps[h] = part[(size_t)(c + h) * 2 * P + k];
            pe[h] = part[(size_t)(c + h) * 2 * P + P + k];
        }
#pragma unroll
        for (int h = 0; h < 8; h++) {
            S += ps[h];
            SE += pe[h];
        }
    }
    for (; c < nchunk; c++) {
        S += part[(size_t)c * 2 * P + k];
        SE += part[(size_t)c * 2 * P + P + k];
    }
    const double m = S / (double)Ns;
    gm[k] = m;
    if (F) F[k] = SE / (double)Ns - m * scal[S_EMEAN];     // src/nqs/nqs_optimizer.c:213-215
}

__global__ void k_center(double *O, int Ns, long P, const double *__restrict__ gm) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, tot = (size_t)Ns * P;
    for (; t < tot; t += (size_t)gridDim.x * blockDim.x) O[t] -= gm[t % P];
}

// ---------------------------------------------------------------- FP64 Gram
// T[i][j] = scale * sum_k A[i][k] A[j][k] (+ shift on the diagonal) for the
// lower-triangular 64x64 tiles; 256 threads, 4x4 register blocking.
constexpr int TG = 64, KC = 16;

__device__ __forceinline__ void tri_tile(int t, int &bi, int &bj) {
    int r = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= t) r++;
    while (r * (r + 1) / 2 > t) r--;
    bi = r;
    bj = t - r * (r + 1) / 2;
}

// Shared tile product: acc[m][n] += sum_k A[r0+ty+16m][k] * B[c0+tx+16n][k] over k in [k0,k1).
__device__ __forceinline__ void tile_mma_fp64(const double *__restrict__ A, long lda,
                                              const double *__restrict__ Bm, long ldb, int rows_a,
                                              int rows_b, int r0, int c0, int k0, int k1,
                                              double (*As)[TG + 1], double (*Bs)[TG + 1],
                                              double acc[4][4]) {
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int kk = k0; kk < k1; kk += KC) {
        for (int e = tid; e < TG * KC; e += 256) {
            int rr = e / KC, cc = e % KC;
            int k = kk + cc;
            int ra = r0 + rr, rb = c0 + rr;
            As[cc][rr] = (ra < rows_a && k < k1) ? A[(size_t)ra * lda + k] : 0.0;
            Bs[cc][rr] = (rb < rows_b && k < k1) ? Bm[(size_t)rb * ldb + k] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < KC; c++) {
            double av[4], bv[4];
#pragma unroll
            for (int m = 0; m < 4; m++) av[m] = As[c][ty + 16 * m];
#pragma unroll
            for (int n = 0; n < 4; n++) bv[n] = Bs[c][tx + 16 * n];
#pragma unroll
            for (int m = 0; m < 4; m++)
#pragma unroll
                for (int n = 0; n < 4; n++) acc[m][n] = fma(av[m], bv[n], acc[m][n]);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_gram_fp64(const double *__restrict__ O, int Ns, long P,
                                                   double scale, double shift, double *T) {
    __shared__ double As[KC][TG + 1], Bs[KC][TG + 1];
    int bi, bj;
    tri_tile(blockIdx.x, bi, bj);
    double acc[4][4] = {};
    tile_mma_fp64(O, P, O, P, Ns, Ns, bi * TG, bj * TG, 0, (int)P, As, Bs, acc);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) {
            int i = bi * TG + ty + 16 * m, j = bj * TG + tx + 16 * n;
            if (i < Ns && j <= i) T[(size_t)i * Ns + j] = acc[m][n] * scale + (i == j ? shift : 0.0);
        }
}

// ---------------------------------------------------------------- Cholesky
constexpr int NB = 32;

// Factor the kb x kb diagonal block at k0 in shared memory (column by column,
// the pivot test of src/nqs/nqs_optimizer.c:1029-1031); first failing column
// goes to status[I_FAIL].
__global__ void k_potrf_diag(double *A, int n, int k0, int kb, int *status) {
    if (status[I_FAIL] >= 0) return;
    __shared__ double L[NB][NB + 1];
    __shared__ int fail;
    int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 32
    if (tx < kb && ty < kb && tx <= ty) L[ty][tx] = A[(size_t)(k0 + ty) * n + k0 + tx];
    if (tx == 0 && ty == 0) fail = -1;
    __syncthreads();
    for (int j = 0; j < kb; j++) {
        if (tx == 0 && ty == 0) {
            double d = L[j][j];
            if (!(d > 0.0)) fail = j;
            else L[j][j] = sqrt(d);
        }
        __syncthreads();
        if (fail >= 0) break;
        if (tx == 0 && ty > j && ty < kb) L[ty][j] = L[ty][j] * (1.0 / L[j][j]);
        __syncthreads();
        if (ty > j && ty < kb && tx > j && tx <= ty) L[ty][tx] -= L[ty][j] * L[tx][j];
        __syncthreads();
    }
    if (fail >= 0) {
        // keep the columns finished before the failing one (they define the
        // state the upstream retry works on)
        if (tx < fail && ty < kb && tx <= ty) A[(size_t)(k0 + ty) * n + k0 + tx] = L[ty][tx];
        if (tx == 0 && ty == 0) status[I_FAIL] = k0 + fail;
        return;
    }
    if (tx < kb && ty < kb && tx <= ty) A[(size_t)(k0 + ty) * n + k0 + tx] = L[ty][tx];
}

// Rows below the block: L[i][k0:k0+ncol] = A[i][k0:k0+ncol] L_kk^{-T}, one
// thread per row (forward substitution with the reciprocal pivot, as upstream).
__global__ void k_trsm_panel(double *A, int n, int k0, int kb, int ncol, int row0, const int *status,
                             int ignore_status) {
    if (!ignore_status && status[I_FAIL] >= 0) return;
    __shared__ double L[NB][NB + 1];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        int r = e / kb, c = e % kb;
        L[r][c] = c <= r ? A[(size_t)(k0 + r) * n + k0 + c] : 0.0;
    }
    __syncthreads();
    int i = row0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x[NB];
    double *row = A + (size_t)i * n + k0;
#pragma unroll
    for (int j = 0; j < NB; j++) x[j] = j < ncol ? row[j] : 0.0;
#pragma unroll
    for (int j = 0; j < NB; j++) {
        if (j < ncol) {
            double s = x[j];
            for (int m = 0; m < j; m++) s -= x[m] * L[j][m];
            x[j] = s * (1.0 / L[j][j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NB; j++)
        if (j < ncol) row[j] = x[j];
}

// Trailing update A[i][j] -= sum_m L[i][k0+m] L[j][k0+m] for k1 <= j <= i < n.
__global__ void __launch_bounds__(256) k_syrk_update(double *A, int n, int k0, int kb, int k1,
                                                     const int *status) {
    if (status[I_FAIL] >= 0) return;
    __shared__ double As[KC][TG + 1], Bs[KC][TG + 1];
    int bi, bj;
    tri_tile(blockIdx.x, bi, bj);
    int r0 = k1 + bi * TG, c0 = k1 + bj * TG;
    double acc[4][4] = {};
    tile_mma_fp64(A + k0, n, A + k0, n, n, n, r0, c0, 0, kb, As, Bs, acc);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int i = r0 + ty + 16 * m, j = c0 + tx + 16 * q;
            if (i < n && j <= i) A[(size_t)i * n + j] -= acc[m][q];
        }
}

static bool cholesky_fp64(double *T, int n, int *status) {
    cudaStream_t st = ctx().stream;
    for (int k0 = 0; k0 < n; k0 += NB) {
        int kb = n - k0 < NB ? n - k0 : NB;
        {
            NQS_LAUNCH("chol_diag");
            k_potrf_diag<<<1, dim3(32, 32), 0, st>>>(T, n, k0, kb, status);
        }
        int k1 = k0 + kb, rest = n - k1;
        if (rest <= 0) break;
        {
            NQS_LAUNCH("chol_panel");
            k_trsm_panel<<<(rest + 127) / 128, 128, 0, st>>>(T, n, k0, kb, kb, k1, status, 0);
        }
        int nt = (rest + TG - 1) / TG;
        {
            NQS_LAUNCH("chol_syrk");
            k_syrk_update<<<nt * (nt + 1) / 2, 256, 0, st>>>(T, n, k0, kb, k1, status);
        }
    }
    return NQS_CUDA(cudaGetLastError());
}

// The upstream retry (src/nqs/nqs_optimizer.c:1156-1160) re-factors the matrix
// as the failed column-by-column factorisation left it: columns c < j hold L
// (every row), columns >= j hold the original T.  Rebuild exactly that state
// from the partially factored T and a pristine copy T0, then add 1e-6.
__global__ void k_quirk_restore(double *T, const double *__restrict__ T0, int n, int j) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, tot = (size_t)n * n;
    for (; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        int r = (int)(t / n), c = (int)(t % n);
        if (c > r) continue;
        if (c >= j) T[t] = T0[t];
        if (r == c) T[t] += 1e-6;
    }
}

// ---------------------------------------------------------------- triangular solves
// Forward L z = b, block by block.  Every CTA re-solves the 32x32 diagonal
// block with a warp (lane = row) and then updates its rows of the right-hand
// side; CTA 0 stores the block of the solution.
__global__ void k_trsv_fwd(const double *__restrict__ L, int n, int k0, int kb, double *rhs, double *x) {
    __shared__ double xs[NB];
    int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
        double v = lane < kb ? rhs[k0 + lane] : 0.0;
        for (int j = 0; j < kb; j++) {
            double xj = __shfl_sync(0xffffffffu, v, j) / L[(size_t)(k0 + j) * n + k0 + j];
            if (lane == j) v = xj;
            if (lane > j && lane < kb) v -= L[(size_t)(k0 + lane) * n + k0 + j] * xj;
        }
        if (lane < kb) xs[lane] = v;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x < kb) x[k0 + threadIdx.x] = xs[threadIdx.x];
    int i = k0 + kb + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        double s = 0.0;
        const double *row = L + (size_t)i * n + k0;
        for (int m = 0; m < kb; m++) s += row[m] * xs[m];
        rhs[i] -= s;
    }
}

// Backward L^T y = z, last block first; the update reads row-block k of L.
__global__ void k_trsv_bwd(const double *__restrict__ L, int n, int k0, int kb, double *rhs, double *x) {
    __shared__ double xs[NB];
    int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
        double v = lane < kb ? rhs[k0 + lane] : 0.0;
        for (int j = kb - 1; j >= 0; j--) {
            double xj = __shfl_sync(0xffffffffu, v, j) / L[(size_t)(k0 + j) * n + k0 + j];
            if (lane == j) v = xj;
            if (lane < j) v -= L[(size_t)(k0 + j) * n + k0 + lane] * xj;
        }
        if (lane < kb) xs[lane] = v;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x < kb) x[k0 + threadIdx.x] = xs[threadIdx.x];
    int jcol = blockIdx.x * blockDim.x + threadIdx.x;
    if (jcol < k0) {
        double s = 0.0;
        for (int m = 0; m < kb; m++) s += L[(size_t)(k0 + m) * n + jcol] * xs[m];
        rhs[jcol] -= s;
    }
}

static bool cholesky_solve(const double *L, int n, const double *b, double *z, double *y) {
    cudaStream_t st = ctx().stream;
    if (!NQS_CUDA(cudaMemcpyAsync(z, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st))) return false;
    for (int k0 = 0; k0 < n; k0 += NB) {
        int kb = n - k0 < NB ? n - k0 : NB;
        int rest = n - k0 - kb;
        NQS_LAUNCH("trsv_fwd");
        k_trsv_fwd<<<rest > 0 ? (rest + 127) / 128 : 1, 128, 0, st>>>(L, n, k0, kb, z, y);
    }
    // y now holds the forward solution; reuse it as the right-hand side
    if (!NQS_CUDA(cudaMemcpyAsync(z, y, sizeof(double) * n, cudaMemcpyDeviceToDevice, st))) return false;
    int last = ((n - 1) / NB) * NB;
    for (int k0 = last; k0 >= 0; k0 -= NB) {
        int kb = n - k0 < NB ? n - k0 : NB;
        NQS_LAUNCH("trsv_bwd");
        k_trsv_bwd<<<k0 > 0 ? (k0 + 127) / 128 : 1, 128, 0, st>>>(L, n, k0, kb, z, y);
    }
    return NQS_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------- update
// delta_k = scale * sum_i O[i][k] y_i (same blocking as k_col_stats).
__global__ void k_col_dot(const double *__restrict__ O, int Ns, long P, const double *__restrict__ y,
                          double scale, double *out) {
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
        out[k] = S * scale;
    }
}

// theta -= lr * delta and ||delta||^2 (one block, deterministic order).
__global__ void k_apply(double *params, const double *__restrict__ delta, long P, double lr, double *scal,
                        const int *status, int zero_on_fail) {
    __shared__ double red[1024];
    bool zero = zero_on_fail && status[I_FAIL2] >= 0;
    double s = 0.0;
    for (long k = threadIdx.x; k < P; k += blockDim.x) {
        double d = zero ? 0.0 : delta[k];
        params[k] += -lr * d;
        s += d * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) scal[S_NORM2] = red[0];
}

// ---------------------------------------------------------------- the step

struct StepIn {
    const nqs_config_t *cfg;
    int size_x, size_y;
    Ansatz *ansatz;
    Sampler *sampler;                  // or NULL with a host batch
    const int *host_batch;
    int Ns;
    nqs_log_amp_fn_t fn;
    void *user;
    nqs_gradient_fn_t gfn;
    void *guser;
    // 0 CG-SR, 1 MinSR, 2 holomorphic SR (CG on the complex QGT), 3 excited-state SR (2 with
    // the orthogonality penalty), 4 real-time tVMC force (same metric), 5 holomorphic MinSR
    // (the holomorphic system solved as MinSR on the stacked real and imaginary parts)
    int minsr;
    nqs_holomorphic_gradient_fn_t hgfn;
    void *hguser;
    nqs_log_amp_fn_t ref_fn;           // excited-state SR: the reference wavefunction
    void *ref_user;
    double mu;                         //   and the penalty strength
    int custom_scale;                  // 1: params += scale * delta (tVMC), else -= lr * delta
    double scale;
    int no_apply;                      // 1: leave delta in the workspace, parameters unchanged
};

// F = 2 (F_R + sign F_I): the holomorphic force (sign +1, src/nqs/nqs_optimizer.c:471-498)
// and the real-time force (sign -1 with the energy halves swapped, :929-941)
__global__ void k_holo_force(double *F, const double *__restrict__ F2, long P, double sign) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < P; k += (long)gridDim.x * blockDim.x)
        F[k] = 2.0 * (F[k] + sign * F2[k]);
}

// Excited-state penalty (src/nqs/nqs_optimizer.c:600-658): r_i = psi_ref / psi at sample i
// with the log-modulus difference clamped to +-10, <r> over the batch, then
// E_i += mu r_i conj(<r>) and the augmented means
// <E_re> + mu |<r>|^2, <E_im> + mu (<r_im><r_re> - <r_re><r_im>) into aug[S_EMEAN] and
// aug[16 + S_EMEAN].  One block; the sums run in a fixed order.
__global__ void k_excited_augment(double *Er, double *Ei, const double *__restrict__ la,
                                  const double *__restrict__ ar, const double *__restrict__ lr,
                                  const double *__restrict__ arr, int Ns, double mu, const double *scal,
                                  const double *scal2, double *aug) {
    __shared__ double sr[1024], si[1024];
    const double cap = 10.0;
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < Ns; i += blockDim.x) {
        double d = fmin(fmax(lr[i] - la[i], -cap), cap), m = exp(d), th = arr[i] - ar[i];
        a += m * cos(th);
        b += m * sin(th);
    }
    sr[threadIdx.x] = a;
    si[threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sr[threadIdx.x] += sr[threadIdx.x + o];
            si[threadIdx.x] += si[threadIdx.x + o];
        }
        __syncthreads();
    }
    const double Rr = sr[0] / (double)Ns, Ri = si[0] / (double)Ns;
    for (int i = threadIdx.x; i < Ns; i += blockDim.x) {
        double d = fmin(fmax(lr[i] - la[i], -cap), cap), m = exp(d), th = arr[i] - ar[i];
        const double rr = m * cos(th), ri = m * sin(th);
        Er[i] += mu * (rr * Rr + ri * Ri);
        Ei[i] += mu * (ri * Rr - rr * Ri);
    }
    if (threadIdx.x == 0) {
        aug[S_EMEAN] = scal[S_EMEAN] + mu * (Rr * Rr + Ri * Ri);
        aug[16 + S_EMEAN] = scal2[S_EMEAN] + mu * (Ri * Rr - Rr * Ri);
    }
}

// k1 <- (k1 + k2) / 2 (Heun's averaged slope, src/nqs/nqs_optimizer.c:864)
__global__ void k_heun_average(double *k1, const double *__restrict__ k2, long P) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < P; k += (long)gridDim.x * blockDim.x)
        k1[k] = 0.5 * (k1[k] + k2[k]);
}

// Column means of O (and the CG-SR force F when E != NULL) over a 2-D grid of
// about four blocks per SM.
static int col_chunks(int Ns, long P, int *rows_per) {
    const int gx = (int)((P + 31) / 32);
    int rb = (4 * ctx().sm_count + gx - 1) / gx;
    rb = rb < 1 ? 1 : rb > (Ns + 63) / 64 ? (Ns + 63) / 64 : rb;
    *rows_per = (Ns + rb - 1) / rb;
    return (Ns + *rows_per - 1) / *rows_per;
}

// Doubles of partial sums col_stats needs (callers that run concurrently pass
// their own buffer).
long col_stats_scratch(int Ns, long P) {
    int rp;
    return (long)col_chunks(Ns, P, &rp) * 2 * P;
}

static bool col_stats(const double *O, int Ns, long P, const double *E, const double *scal, double *gm, double *F,
                      double *part_buf = nullptr) {
    static DevBuf<double> part;
    int rows_per;
    const int gx = (int)((P + 31) / 32), rb = col_chunks(Ns, P, &rows_per);
    const bool own_part = part_buf == nullptr;
    if (!part_buf) {
        if (!part.ensure((size_t)rb * 2 * P)) return false;
        part_buf = part.p;
    }
    cudaStream_t st = ctx().stream;
    // the library's own stream finishes the sums in the partial kernel (tickets zeroed when
    // allocated and reset by the kernel); callers with their own scratch run the two kernels
    static DevBuf<unsigned> tickets;
    unsigned *tk = nullptr;
    if (own_part) {
        const size_t n0 = tickets.p ? tickets.n : 0;
        if (!tickets.ensure((size_t)gx)) return false;
        if (tickets.n != n0 && !NQS_CUDA(cudaMemsetAsync(tickets.p, 0, sizeof(unsigned) * tickets.n, st)))
            return false;
        tk = tickets.p;
    }
    k_col_part<<<dim3((unsigned)gx, (unsigned)rb), dim3(32, 8), 0, st>>>(O, Ns, P, E, rows_per, part_buf, tk, scal,
                                                                         gm, F);
    if (!tk) {
        NQS_LAUNCH("col_sum");
        k_col_fin<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(part_buf, rb, Ns, P, scal, gm, F);
    }
    return NQS_CUDA(cudaGetLastError());
}

// Scratch for enqueue_energy_stats, zeroed when (re)allocated.
static bool ensure_energy_scratch(DevBuf<double> &b, int Ns) {
    const size_t nd = energy_scratch_doubles(Ns), n0 = b.p ? b.n : 0;
    if (!b.ensure(nd)) return false;
    // a new allocation starts zeroed (the ticket words, at its start, stay zero between calls)
    if (b.n != n0 && !NQS_CUDA(cudaMemsetAsync(b.p, 0, sizeof(double) * b.n, ctx().stream))) return false;
    return true;
}

bool enqueue_energy_stats(const double *E, int Ns, int chains, double *scal, double *eps, double *scratch) {
    cudaStream_t st = ctx().stream;
    const int G = es_blocks(Ns);
    unsigned *tickets = (unsigned *)scratch;
    double *part = scratch + 2, *gpart = part + (size_t)G * 4;
    {
        NQS_LAUNCH("energy_stats");
        k_energy_mb<<<G, ES_THREADS, 0, st>>>(E, Ns, part, tickets, scal);
    }
    {
        NQS_LAUNCH("ess");
        k_ess_mb<<<G, ES_THREADS, 0, st>>>(E, Ns, chains, gpart, tickets + 1, scal, eps);
    }
    return NQS_CUDA(cudaGetLastError());
}

bool enqueue_col_means(const double *O, int Ns, long P, const double *scal, double *gm, double *part) {
    NQS_LAUNCH("col_mean");
    return col_stats(O, Ns, P, nullptr, scal, gm, nullptr, part);
}

bool enqueue_col_dot(const double *O, int Ns, long P, const double *y, double scale, double *out) {
    dim3 cb(32, 8), cg((unsigned)((P + 31) / 32));
    NQS_LAUNCH("delta");
    k_col_dot<<<cg, cb, 0, ctx().stream>>>(O, Ns, P, y, scale, out);
    return NQS_CUDA(cudaGetLastError());
}

// FP64 factorisation and solve of (O O^T / N_s + shift I) y = eps on the
// centred O [N_s][N_p], with the upstream retry semantics on a Cholesky
// breakdown (src/nqs/nqs_optimizer.c:1148-1170): the retry adds 1e-6 to the
// diagonal of the partially overwritten matrix; a second breakdown sets the
// update to 0.  Writes y [N_s] and *conv (1 when solved).  Uses the shared
// workspace; returns 0 on success, -1 on a CUDA error.
int minsr_fp64_solve(const double *O, const double *eps, int Ns, long P, double shift, double *y_out, int *conv) {
    Workspace &w = g_ws;
    Context &c = ctx();
    cudaStream_t st = c.stream;
    *conv = 0;
    if (!w.T.ensure((size_t)Ns * Ns) || !w.z.ensure(Ns) || !w.status.ensure(16)) return -1;
    int nt = (Ns + TG - 1) / TG;
    NQS_CUDA(cudaMemsetAsync(w.status.p, 0xff, sizeof(int) * 16, st));
    {
        NQS_LAUNCH("gram_fp64");
        k_gram_fp64<<<nt * (nt + 1) / 2, 256, 0, st>>>(O, Ns, P, 1.0 / (double)Ns, shift, w.T.p);
    }
    if (!cholesky_fp64(w.T.p, Ns, w.status.p)) return -1;
    int fail = -1;
    if (!NQS_CUDA(cudaMemcpyAsync(&fail, w.status.p + I_FAIL, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return -1;
    step_stats().chol_fail_col = fail;
    step_stats().chol_retry = 0;
    int fail2 = -1;
    if (fail >= 0) {
        // upstream retry on the partially overwritten matrix (+1e-6)
        step_stats().chol_retry = 1;
        if (!w.T0.ensure((size_t)Ns * Ns)) return -1;
        {
            NQS_LAUNCH("gram_fp64");
            k_gram_fp64<<<nt * (nt + 1) / 2, 256, 0, st>>>(O, Ns, P, 1.0 / (double)Ns, shift, w.T0.p);
        }
        int k0 = (fail / NB) * NB, kb = Ns - k0 < NB ? Ns - k0 : NB;
        if (fail > k0 && k0 + kb < Ns) {
            NQS_LAUNCH("chol_panel");
            k_trsm_panel<<<(Ns - k0 - kb + 127) / 128, 128, 0, st>>>(w.T.p, Ns, k0, kb, fail - k0, k0 + kb,
                                                                    w.status.p, 1);
        }
        {
            NQS_LAUNCH("chol_restore");
            k_quirk_restore<<<c.sm_count * 8, 256, 0, st>>>(w.T.p, w.T0.p, Ns, fail);
        }
        NQS_CUDA(cudaMemsetAsync(w.status.p + I_FAIL, 0xff, sizeof(int), st));
        if (!cholesky_fp64(w.T.p, Ns, w.status.p)) return -1;
        if (!NQS_CUDA(cudaMemcpyAsync(&fail2, w.status.p + I_FAIL, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaStreamSynchronize(st)))
            return -1;
    }
    if (fail2 < 0) {
        if (!cholesky_solve(w.T.p, Ns, eps, w.z.p, y_out)) return -1;
        *conv = 1;
    } else {
        fprintf(stderr, "nqs_sr_step_minsr: Cholesky breakdown after retry; increase "
                        "sr_diag_shift or num_samples. Update set to 0.\n");
        NQS_CUDA(cudaMemsetAsync(y_out, 0, sizeof(double) * Ns, st));
    }
    return 0;
}

// ---------------------------------------------------------------- FP64 parameter-space solve
// Column Gram of the centred Jacobian, S[i][j] = sum_r O[r][i] O[r][j] over the
// lower-triangular 64x64 tiles of the N_p x N_p matrix.  The sample dimension is
// split over blockIdx.y so that small N_p still fills the GPU; split s writes
// part[s][i][j], and k_gram_cols_sum adds the splits in a fixed order
// (deterministic).  With one split the tile is written straight into S as
// scale * sum + shift on the diagonal.  Rows of O are read along the parameter
// index (one 512-byte segment per tile row and sample).
__global__ void __launch_bounds__(256) k_gram_cols_fp64(const double *__restrict__ O, int Ns, long P, int rows_per,
                                                        double scale, double shift, double *out) {
    __shared__ double As[KC][TG + 1], Bs[KC][TG + 1];
    int bi, bj;
    tri_tile(blockIdx.x, bi, bj);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const long r0 = (long)bi * TG, c0 = (long)bj * TG;
    const int s0 = blockIdx.y * rows_per, s1 = min(Ns, s0 + rows_per);
    double acc[4][4] = {};
    for (int ss = s0; ss < s1; ss += KC) {
        for (int e = tid; e < TG * KC; e += 256) {
            const int rr = e % TG, cc = e / TG, r = ss + cc;
            const long ia = r0 + rr, ib = c0 + rr;
            As[cc][rr] = (r < s1 && ia < P) ? O[(size_t)r * P + ia] : 0.0;
            Bs[cc][rr] = (r < s1 && ib < P) ? O[(size_t)r * P + ib] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < KC; c++) {
            double av[4], bv[4];
#pragma unroll
            for (int m = 0; m < 4; m++) av[m] = As[c][ty + 16 * m];
#pragma unroll
            for (int n = 0; n < 4; n++) bv[n] = Bs[c][tx + 16 * n];
#pragma unroll
            for (int m = 0; m < 4; m++)
#pragma unroll
                for (int n = 0; n < 4; n++) acc[m][n] = fma(av[m], bv[n], acc[m][n]);
        }
        __syncthreads();
    }
    const bool direct = gridDim.y == 1;
    double *dst = out + (direct ? 0 : (size_t)blockIdx.y * P * P);
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const long i = r0 + ty + 16 * m, j = c0 + tx + 16 * n;
            if (i < P && j <= i)
                dst[(size_t)i * P + j] = direct ? acc[m][n] * scale + (i == j ? shift : 0.0) : acc[m][n];
        }
}

// S[i][j] = scale * sum_s part[s][i][j] (+ shift on the diagonal), lower triangle.
__global__ void k_gram_cols_sum(const double *__restrict__ part, int nsplit, long P, double scale, double shift,
                                double *S) {
    const size_t tot = (size_t)P * P;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const long i = (long)(t / P), j = (long)(t % P);
        if (j > i) continue;
        double v = 0.0;
        for (int q = 0; q < nsplit; q++) v += part[(size_t)q * tot + t];
        S[t] = v * scale + (i == j ? shift : 0.0);
    }
}

// Splits of the sample dimension for the column Gram: enough CTAs for about
// eight per SM, at least 256 samples per split, and the partial sums within
// 64 M doubles (512 MB).
static int gram_cols_splits(int Ns, long P) {
    const long nt = (P + TG - 1) / TG, tiles = nt * (nt + 1) / 2;
    long want = (8L * ctx().sm_count + tiles - 1) / tiles;
    want = std::min<long>(want, std::max(1, Ns / 256));
    while (want > 1 && want * P * P > (64L << 20)) want--;
    return (int)std::max<long>(1, want);
}

// S = O_c^T O_c / N_s + shift I into w.T (lower triangle) from the centred O.
static bool gram_cols(const double *O, int Ns, long P, double shift) {
    Workspace &w = g_ws;
    cudaStream_t st = ctx().stream;
    const int ns = gram_cols_splits(Ns, P);
    const int rows_per = (Ns + ns - 1) / ns;
    const long nt = (P + TG - 1) / TG;
    if (!w.T.ensure((size_t)P * P)) return false;
    if (ns > 1 && !w.T0.ensure((size_t)ns * P * P)) return false;
    {
        NQS_LAUNCH("gram_cols_fp64");
        k_gram_cols_fp64<<<dim3((unsigned)(nt * (nt + 1) / 2), (unsigned)ns), 256, 0, st>>>(
            O, Ns, P, rows_per, 1.0 / (double)Ns, shift, ns > 1 ? w.T0.p : w.T.p);
    }
    if (ns > 1) {
        NQS_LAUNCH("gram_cols_sum");
        k_gram_cols_sum<<<ctx().sm_count * 8, 256, 0, st>>>(w.T0.p, ns, P, 1.0 / (double)Ns, shift, w.T.p);
    }
    return NQS_CUDA(cudaGetLastError());
}

// The FP64 MinSR update in parameter space (push-through identity):
// (O_c^T O_c / N_s + shift I) delta = O_c^T eps / N_s on the centred O [N_s][N_p].
// Same FP64 blocked Cholesky and triangular solves as the sample-space path; a
// failed factorisation is retried once with the shift raised by 1e-6 (the
// upstream retry adds 1e-6 to its diagonal too), then delta = 0 and *conv = 0.
// Writes delta [N_p]; returns 0 on success, -1 on a CUDA error.
int minsr_fp64_params(const double *O, const double *eps, int Ns, long P, double shift, double *delta, int *conv) {
    Workspace &w = g_ws;
    cudaStream_t st = ctx().stream;
    *conv = 0;
    if (!w.z.ensure(P) || !w.r.ensure(P) || !w.status.ensure(16)) return -1;
    // right-hand side b = O_c^T eps / N_s
    if (!enqueue_col_dot(O, Ns, P, eps, 1.0 / (double)Ns, w.r.p)) return -1;
    int fail = -1;
    step_stats().chol_retry = 0;
    for (int attempt = 0; attempt < 2; attempt++) {
        if (!gram_cols(O, Ns, P, shift + (attempt ? 1e-6 : 0.0))) return -1;
        NQS_CUDA(cudaMemsetAsync(w.status.p, 0xff, sizeof(int) * 16, st));
        if (!cholesky_fp64(w.T.p, (int)P, w.status.p)) return -1;
        if (!NQS_CUDA(cudaMemcpyAsync(&fail, w.status.p + I_FAIL, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaStreamSynchronize(st)))
            return -1;
        if (attempt == 0) step_stats().chol_fail_col = fail;
        if (fail < 0) break;
        step_stats().chol_retry = 1;
    }
    if (fail >= 0) {
        fprintf(stderr, "nqs_sr_step_minsr: Cholesky breakdown after retry; increase "
                        "sr_diag_shift or num_samples. Update set to 0.\n");
        return NQS_CUDA(cudaMemsetAsync(delta, 0, sizeof(double) * P, st)) ? 0 : -1;
    }
    if (!cholesky_solve(w.T.p, (int)P, w.r.p, w.z.p, delta)) return -1;
    *conv = 1;
    return 0;
}

// The FP64 MinSR update delta = O^T y / N_s of one system whose mixed solve
// broke down (FP32 pivot <= 0), on its centred O and eps.
int minsr_fp64_delta(const double *O, const double *eps, int Ns, long P, double shift, double *delta, int *conv) {
    Workspace &w = g_ws;
    if (!w.y.ensure(Ns)) return -1;
    if (minsr_fp64_solve(O, eps, Ns, P, shift, w.y.p, conv) != 0) return -1;
    return enqueue_col_dot(O, Ns, P, w.y.p, 1.0 / (double)Ns, delta) ? 0 : -1;
}

static int sr_step_impl(const StepIn &in, nqs_sr_step_info_t *info, double *out_E, double *out_delta) {
    clear_error();
    const nqs_config_t *cfg = in.cfg;
    Ansatz *a = in.ansatz;
    if (!ensure_context()) return -1;
    if (!ansatz_sync(a, true)) return -1;
    Context &c = ctx();
    cudaStream_t st = c.stream;
    long launches0 = c.launches;
    const int Ns = in.Ns;
    const long P = a->P;
    if (Ns <= 0 || P <= 0) {
        set_error("num_samples and num_params must be positive");
        return -1;
    }
    DevHam H;
    if (!hamiltonian_build(cfg, in.size_x, in.size_y, &H)) return -1;
    nqs_log_amp_fn_t fn = in.fn ? in.fn : nqs_ansatz_log_amp;   // src/nqs/nqs_optimizer.c:159
    void *user = in.fn ? in.user : (void *)a;
    DevAmp A;
    Ansatz *base = nullptr;
    if (!build_amp(fn, user, H.N, &A, &base)) return -1;
    if (base != a) {
        set_error("the log_amp program does not wrap the ansatz being optimised");
        return -1;
    }
    DevAmp Ag;   // program whose gradient fills O
    int grad_sym = 0;
    if (in.gfn == nullptr) {
        Ag = A;
        Ag.G = 0;
        Ag.n_outer = Ag.n_inner = 0;
    } else if (in.gfn == nqs_symproj_gradient) {
        if (!build_amp(nqs_symproj_log_amp, in.guser, H.N, &Ag, nullptr)) return -1;
        grad_sym = 1;
    } else if (in.gfn == nqs_translation_gradient) {
        if (!build_amp(nqs_translation_log_amp, in.guser, H.N, &Ag, nullptr)) return -1;
        grad_sym = 1;
    } else {
        set_error("gradient callback is not supported on the GPU (NULL, nqs_symproj_gradient or "
                  "nqs_translation_gradient)");
        return -1;
    }
    const bool holo = in.minsr >= 2, excited = in.minsr == 3, realtime = in.minsr == 4, hm = in.minsr == 5;
    if (excited && !in.ref_fn) {
        set_error("excited-state SR needs the reference log-amplitude");
        return -1;
    }
    // holomorphic gradient: NULL = the base ansatz's (src/nqs/nqs_optimizer.c:458-469), or the
    // symmetry-projected one (nqs_symproj_gradient_complex with its wrapper)
    const bool hg_sym = holo && (void *)in.hgfn == (void *)nqs_symproj_gradient_complex;
    if (holo && in.hgfn && !hg_sym) {
        set_error("holomorphic gradient callback is not supported on the GPU (NULL or nqs_symproj_gradient_complex)");
        return -1;
    }
    DevAmp Ahg;
    if (hg_sym) {
        Ansatz *hbase = nullptr;
        if (!build_amp(nqs_symproj_log_amp, in.hguser, H.N, &Ahg, &hbase)) return -1;
        if (hbase != a) {
            set_error("the gradient's symmetry wrapper does not wrap the ansatz being optimised");
            return -1;
        }
    }
    Workspace &w = g_ws;
    // holomorphic MinSR keeps R and I as one stacked [2 N_s][N_p] matrix and the centred
    // energies as one stacked [2 N_s] vector (the rows of its MinSR system)
    const int rows = hm ? 2 * Ns : Ns;
    if (!w.E.ensure(Ns) || !w.Ei.ensure(Ns) || !w.eps.ensure(rows) || !w.O.ensure((size_t)rows * P) ||
        !w.gm.ensure(P) || !w.delta.ensure(P) || !w.scal.ensure(16) || !w.status.ensure(16))
        return -1;
    if (holo && ((!hm && (!w.Oi.ensure((size_t)Ns * P) || !w.eps2.ensure(Ns))) || !w.gm2.ensure(P) ||
                 !w.F2.ensure(P) || !w.scal2.ensure(16)))
        return -1;
    double *const Oi = hm ? w.O.p + (size_t)Ns * P : w.Oi.p;
    double *const eps2 = hm ? w.eps.p + Ns : w.eps2.p;
    DevAmp Aref;
    if (excited && (!build_amp(in.ref_fn, in.ref_user, H.N, &Aref, nullptr) || !w.la.ensure(Ns) ||
                    !w.ar.ensure(Ns) || !w.la_ref.ensure(Ns) || !w.ar_ref.ensure(Ns) || !w.aug.ensure(32)))
        return -1;
    // 1. samples
    uint64_t *bits = nullptr;
    if (in.sampler) {
        if (!sampler_produce(in.sampler, Ns, &bits)) return -1;
    } else {
        if (!upload_spins(in.host_batch, Ns, H.N, &bits)) return -1;
    }
    // holomorphic MinSR: G + eps I = 4 (O_s^T O_s / (2 N_s) + eps / 4 I) with O_s = [R_c; I_c] and
    // F = 4 O_s^T [e_re; e_im] / (2 N_s), so delta is the MinSR update of the stacked rows
    // with the shift divided by 4
    const double shift = hm ? 0.25 * cfg->sr_diag_shift : cfg->sr_diag_shift;
    auto fp64_solve = [&](double *y_out, int *conv) -> int {
        return minsr_fp64_solve(w.O.p, w.eps.p, rows, P, shift, y_out, conv);
    };
    const bool mixed = c.opts.precision == NQS_GPU_PREC_MIXED;
    const bool fp32est = mixed && c.opts.fp32_estimator && !grad_sym && !holo && (fp32_capable(A) || fp32_mlp_capable(A));
    nqs_gpu_step_stats_t &ss = step_stats();
    ss.energy_rel_err = -1.0;
    double e64 = 0.0;
    bool have64 = false;
    if (in.minsr == 1 && fp32est && c.opts.mixed_check) {
        // reference for the check: the FP64 estimator, statistics and FP64
        // MinSR solve on the same samples
        if (!w.T.ensure((size_t)Ns * Ns) || !w.y.ensure(Ns) || !w.z.ensure(Ns) || !w.y64.ensure(Ns) ||
            !w.d64.ensure(P))
            return -1;
        if (!launch_local_estimator(A, H, bits, Ns, w.E.p, w.Ei.p, w.O.p, nullptr, 1, false)) return -1;
        dim3 cb0(32, 8), cg0((unsigned)((P + 31) / 32));
        k_energy_stats<<<1, 1024, 0, st>>>(w.E.p, Ns, w.scal.p, w.eps.p);
        if (!col_stats(w.O.p, Ns, P, nullptr, w.scal.p, w.gm.p, nullptr)) return -1;
        k_center<<<c.sm_count * 8, 256, 0, st>>>(w.O.p, Ns, P, w.gm.p);
        int conv64 = 0;
        if (fp64_solve(w.y64.p, &conv64) != 0) return -1;
        k_col_dot<<<cg0, cb0, 0, st>>>(w.O.p, Ns, P, w.y64.p, 1.0 / (double)Ns, w.d64.p);
        if (!NQS_CUDA(cudaMemcpyAsync(&e64, w.scal.p + S_EMEAN, sizeof(double), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaStreamSynchronize(st)))
            return -1;
        have64 = true;
    }
    // 2. local energies + Jacobian rows (fused when the program allows); the
    // holomorphic step takes the complex gradient of the base ansatz
    // (nqs_ansatz_logpsi_gradient_complex, src/nqs/nqs_optimizer.c:458-469)
    bool fused_grad = !grad_sym && A.G == 0;
    if (holo && A.G == 0 && !hg_sym) {
        if (!launch_local_estimator(A, H, bits, Ns, w.E.p, w.Ei.p, w.O.p, Oi, 2, false)) return -1;
    } else if (holo) {
        if (!launch_local_estimator(A, H, bits, Ns, w.E.p, w.Ei.p, nullptr, nullptr, 0, false)) return -1;
        if (hg_sym ? !launch_symproj_gradient_complex(Ahg, bits, Ns, w.O.p, Oi)
                   : !launch_gradient(A.a, bits, Ns, 2, w.O.p, Oi))
            return -1;
    } else if (!launch_local_estimator(A, H, bits, Ns, w.E.p, w.Ei.p, fused_grad ? w.O.p : nullptr, nullptr,
                                       fused_grad ? 1 : 0, fp32est)) {
        return -1;
    }
    if (!fused_grad && !holo) {
        if (grad_sym) {
            if (!launch_symproj_gradient(Ag, bits, Ns, w.O.p)) return -1;
        } else if (!launch_gradient(Ag.a, bits, Ns, 1, w.O.p, nullptr)) {
            return -1;
        }
    }
    // 3. statistics
    {
        const int chains = in.sampler ? nqs_sampler_num_chains((nqs_sampler_t *)in.sampler) : 0;
        if (!ensure_energy_scratch(w.es, Ns) || !enqueue_energy_stats(w.E.p, Ns, chains, w.scal.p, w.eps.p, w.es.p))
            return -1;
        // <E_im> for the holomorphic force
        if (holo && (!ensure_energy_scratch(w.es2, Ns) ||
                     !enqueue_energy_stats(w.Ei.p, Ns, 0, w.scal2.p, eps2, w.es2.p)))
            return -1;
        // excited-state SR: the physical statistics stay in scal for the step info; the force
        // takes the augmented local energies and means
        if (excited) {
            if (!launch_log_amp(A, bits, Ns, w.la.p, w.ar.p) || !launch_log_amp(Aref, bits, Ns, w.la_ref.p, w.ar_ref.p))
                return -1;
            NQS_LAUNCH("excited_penalty");
            k_excited_augment<<<1, 1024, 0, st>>>(w.E.p, w.Ei.p, w.la.p, w.ar.p, w.la_ref.p, w.ar_ref.p, Ns, in.mu,
                                                  w.scal.p, w.scal2.p, w.aug.p);
        }
    }
    NQS_CUDA(cudaMemsetAsync(w.status.p, 0xff, sizeof(int) * 16, st));   // all -1
    dim3 cb(32, 8), cg((unsigned)((P + 31) / 32));
    int converged = 0, cg_iters = 0;
    bool applied = false;             // update and derived tables already enqueued
    if (in.minsr == 1 || hm) {
        if (!w.T.ensure((size_t)rows * rows) || !w.y.ensure(rows) || !w.z.ensure(rows)) return -1;
        {
            NQS_LAUNCH("col_mean");
            if (!col_stats(w.O.p, Ns, P, nullptr, w.scal.p, w.gm.p, nullptr)) return -1;
        }
        if (hm) {
            // centre each half with its own column means; the stacked matrix then has zero
            // means for the solvers below
            NQS_LAUNCH("center");
            if (!col_stats(Oi, Ns, P, nullptr, w.scal2.p, w.gm2.p, nullptr)) return -1;
            k_center<<<c.sm_count * 8, 256, 0, st>>>(w.O.p, Ns, P, w.gm.p);
            k_center<<<c.sm_count * 8, 256, 0, st>>>(Oi, Ns, P, w.gm2.p);
            if (!NQS_CUDA(cudaMemsetAsync(w.gm.p, 0, sizeof(double) * P, st))) return -1;
        }
        ss.refine_residual = 0.0;
        ss.refine_sweeps = 0;
        ss.mixed_fallback = 0;
        ss.delta_rel_err = -1.0;
        bool solved = false, have_delta = false;
        if (mixed) {
            // centring happens inside the split kernel of the mixed solve.  In parameter space
            // the update and the derived tables are enqueued behind the solve before the host
            // waits for it, with the update taken as zero on the device when the solve broke
            // down (the FP64 solve below then applies its own)
            double resid = 0.0;
            int f32 = -1;
            bool pre = false;
            const double lr_pre = in.custom_scale ? -in.scale : cfg->learning_rate;
            auto after = [&](const int *mst, const int *merr, const double *mnrm, bool pspace) -> bool {
                if (in.no_apply || hm || !pspace) return true;
                if (!enqueue_gated_apply(a->d_params.p, w.delta.p, P, lr_pre, w.scal.p, mst, merr, mnrm) ||
                    !ansatz_refresh_derived(a))
                    return false;
                pre = true;
                return true;
            };
            if (!minsr_mixed_solve(w.O.p, w.gm.p, w.eps.p, rows, P, shift, c.opts.refine_sweeps,
                                   c.opts.gram_passes, c.opts.mixed_space, w.y.p, w.delta.p, &have_delta,
                                   &resid, &f32, after))
                return -1;
            ss.refine_residual = resid;
            if (f32 < 0) {
                solved = true;
                converged = 1;
                ss.chol_fail_col = -1;
                ss.chol_retry = 0;
                applied = pre;
            } else {
                ss.mixed_fallback = 1;          // FP32 factor failed: solve this step in FP64
                have_delta = false;
                if (hm && P < rows) {
                    // holomorphic MinSR: the stacked sample space (2 N_s) is the larger system;
                    // the FP64 solve takes the parameter-space one (no upstream retry order to keep)
                    if (minsr_fp64_params(w.O.p, w.eps.p, rows, P, shift, w.delta.p, &converged) != 0) return -1;
                    solved = have_delta = true;
                }
            }
        } else {
            if (!hm) {
                NQS_LAUNCH("center");
                k_center<<<c.sm_count * 8, 256, 0, st>>>(w.O.p, Ns, P, w.gm.p);
            }
            const int fs = c.opts.fp64_space;
            if (fs == NQS_GPU_SPACE_PARAMETERS || (fs == NQS_GPU_SPACE_SMALLER && P < rows)) {
                // push-through form: the N_p x N_p system gives delta directly
                if (minsr_fp64_params(w.O.p, w.eps.p, rows, P, shift, w.delta.p, &converged) != 0) return -1;
                solved = have_delta = true;
            }
        }
        if (!solved && fp64_solve(w.y.p, &converged) != 0) return -1;
        if (!have_delta) {
            NQS_LAUNCH("delta");
            k_col_dot<<<cg, cb, 0, st>>>(w.O.p, rows, P, w.y.p, 1.0 / (double)rows, w.delta.p);
        }
        if (mixed && solved && c.opts.mixed_check && !hm) {
            // the FP64 solve on the same centred Jacobian (or, with the FP32
            // estimator, the whole FP64 step computed above), for the
            // delta-theta error
            if (!have64) {
                if (!w.y64.ensure(Ns) || !w.d64.ensure(P)) return -1;
                int conv64 = 0;
                if (fp64_solve(w.y64.p, &conv64) != 0) return -1;
                k_col_dot<<<cg, cb, 0, st>>>(w.O.p, Ns, P, w.y64.p, 1.0 / (double)Ns, w.d64.p);
            } else {
                double em = 0.0;
                if (!NQS_CUDA(cudaMemcpyAsync(&em, w.scal.p + S_EMEAN, sizeof(double), cudaMemcpyDeviceToHost, st)) ||
                    !NQS_CUDA(cudaStreamSynchronize(st)))
                    return -1;
                ss.energy_rel_err = fabs(em - e64) / fmax(fabs(e64), 1e-300);
            }
            std::vector<double> a((size_t)P), b((size_t)P);
            if (!NQS_CUDA(cudaMemcpyAsync(a.data(), w.delta.p, sizeof(double) * P, cudaMemcpyDeviceToHost, st)) ||
                !NQS_CUDA(cudaMemcpyAsync(b.data(), w.d64.p, sizeof(double) * P, cudaMemcpyDeviceToHost, st)) ||
                !NQS_CUDA(cudaStreamSynchronize(st)))
                return -1;
            double num = 0.0, den = 0.0;
            for (long k = 0; k < P; k++) {
                num += (a[k] - b[k]) * (a[k] - b[k]);
                den += b[k] * b[k];
            }
            ss.delta_rel_err = den > 0 ? sqrt(num / den) : 0.0;
        }
    } else {
        if (!w.F.ensure(P) || !w.r.ensure(P) || !w.p.ensure(P) || !w.Ap.ensure(P) || !w.u.ensure(Ns))
            return -1;
        {
            NQS_LAUNCH("col_stats");
            if (realtime) {
                // F = 2 [(R^T E_im - I^T E_re) / N_s - <R><E_im> + <I><E_re>]
                if (!col_stats(w.O.p, Ns, P, w.Ei.p, w.scal2.p, w.gm.p, w.F.p) ||
                    !col_stats(w.Oi.p, Ns, P, w.E.p, w.scal.p, w.gm2.p, w.F2.p))
                    return -1;
                k_holo_force<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(w.F.p, w.F2.p, P, -1.0);
            } else {
                const double *m_re = excited ? w.aug.p : w.scal.p, *m_im = excited ? w.aug.p + 16 : w.scal2.p;
                if (!col_stats(w.O.p, Ns, P, w.E.p, m_re, w.gm.p, w.F.p)) return -1;
                if (holo) {
                    // <I>, (I^T E_im) / N_s - <I> <E_im>; then F = 2 (F_R + F_I)
                    if (!col_stats(w.Oi.p, Ns, P, w.Ei.p, m_im, w.gm2.p, w.F2.p)) return -1;
                    k_holo_force<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(w.F.p, w.F2.p, P, 1.0);
                }
            }
        }
        const int maxit = cfg->sr_cg_max_iters;
        // the whole CG (all iterations) in one cooperative launch
        if (!cg_sr_solve(w.O.p, Ns, P, w.F.p, w.gm.p, cfg->sr_diag_shift, cfg->sr_cg_tol, maxit, w.delta.p, w.scal.p,
                         w.status.p, holo ? w.Oi.p : nullptr, holo ? w.gm2.p : nullptr, holo ? 2.0 : 1.0))
            return -1;
        int h[16];
        double hs[16];
        if (!NQS_CUDA(cudaMemcpyAsync(h, w.status.p, sizeof(h), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaStreamSynchronize(st)))
            return -1;
        converged = h[I_CONV] == 1;
        cg_iters = h[I_DONE] == 1 ? h[I_ITERS] : maxit;
        if (h[I_DONE] == 1 && !converged)
            fprintf(stderr, "nqs_sr cg_solve: Krylov breakdown at iter=%d, pAp=%.3e. Returning "
                            "unconverged partial step.\n", h[I_ITERS], hs[S_PAP]);
    }
    // 4. update: theta -= lr delta, or theta += scale delta for tVMC (already enqueued behind a
    // mixed parameter-space solve that succeeded)
    const double lr_eff = in.custom_scale ? -in.scale : cfg->learning_rate;
    if (!in.no_apply && !applied) {
        NQS_LAUNCH("apply_update");
        k_apply<<<1, 1024, 0, st>>>(a->d_params.p, w.delta.p, P, lr_eff, w.scal.p, w.status.p, 0);
    }
    if (!NQS_CUDA(cudaGetLastError()) || (!applied && !ansatz_refresh_derived(a))) return -1;
    double hs[16];
    if (out_E && !NQS_CUDA(cudaMemcpyAsync(out_E, w.E.p, sizeof(double) * Ns, cudaMemcpyDeviceToHost, st)))
        return -1;
    if (out_delta && !NQS_CUDA(cudaMemcpyAsync(out_delta, w.delta.p, sizeof(double) * P,
                                               cudaMemcpyDeviceToHost, st)))
        return -1;
    if (!NQS_CUDA(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, st)) || !ansatz_pull(a))
        return -1;
    step_stats().gpu_launches = (int)(c.launches - launches0);
    step_stats().tau_int = hs[S_TAU];
    step_stats().ess = hs[S_ESS];
    if (info) {
        info->mean_energy = hs[S_EMEAN];
        info->variance_energy = hs[S_ESQ] - hs[S_EMEAN] * hs[S_EMEAN];
        info->update_norm = in.no_apply ? 0.0 : sqrt(hs[S_NORM2]) * fabs(lr_eff);
        info->acceptance_ratio = in.sampler ? nqs_sampler_acceptance_ratio((nqs_sampler_t *)in.sampler) : 0.0;
        info->cg_iterations = (in.minsr == 1 || hm) ? 0 : cg_iters;
        info->converged = converged;
    }
    return 0;
}

}  // namespace nqs

using namespace nqs;

extern "C" {

// Diagnostic: the step's ESS estimator on a host series (energies in the
// sampler's layout, sample k of chain c at row k * num_chains + c).
int nqs_gpu_ess(const double *energies, int num_samples, int num_chains, double *out_tau, double *out_ess) {
    clear_error();
    if (!energies || num_samples <= 0 || num_chains <= 0) {
        set_error("invalid arguments");
        return -1;
    }
    if (!ensure_context()) return -1;
    cudaStream_t st = ctx().stream;
    static DevBuf<double> dE, deps, dscal, des;
    if (!dE.ensure(num_samples) || !deps.ensure(num_samples) || !dscal.ensure(16) ||
        !ensure_energy_scratch(des, num_samples))
        return -1;
    double hs[16];
    if (!NQS_CUDA(cudaMemcpyAsync(dE.p, energies, sizeof(double) * num_samples, cudaMemcpyHostToDevice, st)))
        return -1;
    if (!enqueue_energy_stats(dE.p, num_samples, num_chains, dscal.p, deps.p, des.p) ||
        !NQS_CUDA(cudaGetLastError()) ||
        !NQS_CUDA(cudaMemcpyAsync(hs, dscal.p, sizeof(hs), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return -1;
    if (out_tau) *out_tau = hs[S_TAU];
    if (out_ess) *out_ess = hs[S_ESS];
    return 0;
}

static int step_common(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *ansatz, nqs_sampler_t *sampler,
                       nqs_log_amp_fn_t fn, void *user, nqs_gradient_fn_t gfn, void *guser, int minsr,
                       nqs_sr_step_info_t *info) {
    if (!cfg || !ansatz || !sampler) return -1;          // src/nqs/nqs_optimizer.c:150
    StepIn in{cfg, sx, sy, (Ansatz *)ansatz, (Sampler *)sampler, nullptr, cfg->num_samples,
              fn, user, gfn, guser, minsr};
    if (nqs_sampler_num_sites(sampler) != ((Ansatz *)ansatz)->N) {
        set_error("sampler and ansatz disagree on num_sites");
        return -1;
    }
    return sr_step_impl(in, info, nullptr, nullptr);
}

int nqs_sr_step_custom_full(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                            nqs_log_amp_fn_t fn, void *user, nqs_gradient_fn_t gfn, void *guser,
                            nqs_sr_step_info_t *info) {
    return step_common(cfg, sx, sy, a, s, fn, user, gfn, guser, 0, info);
}

int nqs_sr_step_custom(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                       nqs_log_amp_fn_t fn, void *user, nqs_sr_step_info_t *info) {
    return nqs_sr_step_custom_full(cfg, sx, sy, a, s, fn, user, nullptr, nullptr, info);
}

int nqs_sr_step(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                nqs_sr_step_info_t *info) {
    return nqs_sr_step_custom_full(cfg, sx, sy, a, s, nullptr, nullptr, nullptr, nullptr, info);
}

int nqs_sr_run_custom_full(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                           nqs_log_amp_fn_t fn, void *user, nqs_gradient_fn_t gfn, void *guser,
                           double *trace) {
    if (!cfg || !a || !s) return -1;                     // src/nqs/nqs_optimizer.c:264-284
    nqs_sampler_thermalize(s);
    for (int it = 0; it < cfg->num_iterations; it++) {
        nqs_sr_step_info_t info;
        int rc = nqs_sr_step_custom_full(cfg, sx, sy, a, s, fn, user, gfn, guser, &info);
        if (rc != 0) return rc;
        if (trace) trace[it] = info.mean_energy;
    }
    return 0;
}

int nqs_sr_run_custom(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                      nqs_log_amp_fn_t fn, void *user, double *trace) {
    return nqs_sr_run_custom_full(cfg, sx, sy, a, s, fn, user, nullptr, nullptr, trace);
}

int nqs_sr_run(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s, double *trace) {
    return nqs_sr_run_custom(cfg, sx, sy, a, s, nullptr, nullptr, trace);
}

// Holomorphic SR (src/nqs/nqs_optimizer.c:307-558): CG on the complex QGT
// G = 2 Re{<O* O> - <O*><O>} with the complex local energies.
int nqs_sr_step_holomorphic_full(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                                 nqs_log_amp_fn_t fn, void *user, nqs_holomorphic_gradient_fn_t gfn, void *guser,
                                 nqs_sr_step_info_t *info) {
    if (!cfg || !a || !s) return -1;
    StepIn in{cfg, sx, sy, (Ansatz *)a, (Sampler *)s, nullptr, cfg->num_samples, fn, user, nullptr, nullptr, 2,
              gfn, guser};
    if (nqs_sampler_num_sites(s) != ((Ansatz *)a)->N) {
        set_error("sampler and ansatz disagree on num_sites");
        return -1;
    }
    return sr_step_impl(in, info, nullptr, nullptr);
}

int nqs_sr_step_holomorphic(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                            nqs_log_amp_fn_t fn, void *user, nqs_sr_step_info_t *info) {
    return nqs_sr_step_holomorphic_full(cfg, sx, sy, a, s, fn, user, nullptr, nullptr, info);
}

int nqs_sr_run_holomorphic_full(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                                nqs_log_amp_fn_t fn, void *user, nqs_holomorphic_gradient_fn_t gfn, void *guser,
                                double *trace) {
    if (!cfg || !a || !s) return -1;
    nqs_sampler_thermalize(s);
    for (int it = 0; it < cfg->num_iterations; it++) {
        nqs_sr_step_info_t info;
        int rc = nqs_sr_step_holomorphic_full(cfg, sx, sy, a, s, fn, user, gfn, guser, &info);
        if (rc != 0) return rc;
        if (trace) trace[it] = info.mean_energy;
    }
    return 0;
}

int nqs_sr_run_holomorphic(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                           nqs_log_amp_fn_t fn, void *user, double *trace) {
    return nqs_sr_run_holomorphic_full(cfg, sx, sy, a, s, fn, user, nullptr, nullptr, trace);
}

int nqs_sr_step_minsr_full(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                           nqs_log_amp_fn_t fn, void *user, nqs_gradient_fn_t gfn, void *guser,
                           nqs_sr_step_info_t *info) {
    return step_common(cfg, sx, sy, a, s, fn, user, gfn, guser, 1, info);
}

int nqs_sr_run_minsr(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                     nqs_log_amp_fn_t fn, void *user, double *trace) {
    if (!cfg || !a || !s) return -1;                     // src/nqs/nqs_optimizer.c:1196-1214
    nqs_sampler_thermalize(s);
    for (int it = 0; it < cfg->num_iterations; it++) {
        nqs_sr_step_info_t info;
        int rc = nqs_sr_step_minsr_full(cfg, sx, sy, a, s, fn, user, nullptr, nullptr, &info);
        if (rc != 0) return rc;
        if (trace) trace[it] = info.mean_energy;
    }
    return 0;
}

int nqs_sr_step_minsr_holomorphic_full(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a,
                                       nqs_sampler_t *s, nqs_log_amp_fn_t fn, void *user,
                                       nqs_holomorphic_gradient_fn_t gfn, void *guser, nqs_sr_step_info_t *info) {
    if (!cfg || !a || !s) return -1;
    StepIn in{cfg, sx, sy, (Ansatz *)a, (Sampler *)s, nullptr, cfg->num_samples, fn, user, nullptr, nullptr, 5,
              gfn, guser};
    if (nqs_sampler_num_sites(s) != ((Ansatz *)a)->N) {
        set_error("sampler and ansatz disagree on num_sites");
        return -1;
    }
    return sr_step_impl(in, info, nullptr, nullptr);
}

int nqs_sr_run_minsr_holomorphic(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                                 nqs_log_amp_fn_t fn, void *user, double *trace) {
    if (!cfg || !a || !s) return -1;
    nqs_sampler_thermalize(s);
    for (int it = 0; it < cfg->num_iterations; it++) {
        nqs_sr_step_info_t info;
        int rc = nqs_sr_step_minsr_holomorphic_full(cfg, sx, sy, a, s, fn, user, nullptr, nullptr, &info);
        if (rc != 0) return rc;
        if (trace) trace[it] = info.mean_energy;
    }
    return 0;
}

int nqs_gpu_sr_step_batch(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_log_amp_fn_t fn,
                          void *user, nqs_gradient_fn_t gfn, void *guser, const int *batch, int Ns, int minsr,
                          nqs_sr_step_info_t *info, double *out_E, double *out_delta) {
    if (!cfg || !a || !batch || Ns <= 0) return -1;
    if (minsr < 0 || minsr > 5 || minsr == 3 || minsr == 4) {
        set_error("nqs_gpu_sr_step_batch: minsr must be 0 (CG-SR), 1 (MinSR), 2 (holomorphic SR) or 5 "
                  "(holomorphic MinSR)");
        return -1;
    }
    StepIn in{cfg, sx, sy, (Ansatz *)a, nullptr, batch, Ns, fn, user, gfn, guser, minsr};
    if ((minsr == 2 || minsr == 5) && gfn) {     // holomorphic: the callback is a holomorphic gradient
        in.hgfn = (nqs_holomorphic_gradient_fn_t)(void *)gfn;
        in.hguser = guser;
        in.gfn = nullptr;
        in.guser = nullptr;
    }
    return sr_step_impl(in, info, out_E, out_delta);
}

int nqs_gpu_sr_step_batch_excited(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_log_amp_fn_t fn,
                                  void *user, nqs_log_amp_fn_t ref_fn, void *ref_user, double mu, const int *batch,
                                  int Ns, nqs_sr_step_info_t *info, double *out_E, double *out_delta) {
    if (!cfg || !a || !batch || Ns <= 0 || !ref_fn) return -1;
    StepIn in{cfg, sx, sy, (Ansatz *)a, nullptr, batch, Ns, fn, user, nullptr, nullptr, 3, nullptr, nullptr,
              ref_fn, ref_user, mu, 0, 0.0, 0};
    return sr_step_impl(in, info, out_E, out_delta);
}

int nqs_gpu_tvmc_step_batch(const nqs_config_t *cfg, double dt, int sx, int sy, nqs_ansatz_t *a,
                            nqs_log_amp_fn_t fn, void *user, const int *batch, int Ns, nqs_sr_step_info_t *info,
                            double *out_E, double *out_delta) {
    if (!cfg || !a || !batch || Ns <= 0) return -1;
    StepIn in{cfg, sx, sy, (Ansatz *)a, nullptr, batch, Ns, fn, user, nullptr, nullptr, 4, nullptr, nullptr,
              nullptr, nullptr, 0.0, 1, dt, 0};
    return sr_step_impl(in, info, out_E, out_delta);
}

// Excited-state SR, src/nqs/nqs_optimizer.c:562-742: the holomorphic step with the
// orthogonality penalty mu r(s) conj(<r>) added to the local energies for the force; the
// step info reports the physical energy.
int nqs_sr_step_excited(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                        nqs_log_amp_fn_t fn, void *user, nqs_log_amp_fn_t ref_fn, void *ref_user, double mu,
                        nqs_sr_step_info_t *info) {
    if (!cfg || !a || !s || !ref_fn) return -1;
    StepIn in{cfg, sx, sy, (Ansatz *)a, (Sampler *)s, nullptr, cfg->num_samples, fn, user, nullptr, nullptr, 3,
              nullptr, nullptr, ref_fn, ref_user, mu, 0, 0.0, 0};
    if (nqs_sampler_num_sites(s) != ((Ansatz *)a)->N) {
        set_error("sampler and ansatz disagree on num_sites");
        return -1;
    }
    return sr_step_impl(in, info, nullptr, nullptr);
}

int nqs_sr_run_excited(const nqs_config_t *cfg, int sx, int sy, nqs_ansatz_t *a, nqs_sampler_t *s,
                       nqs_log_amp_fn_t fn, void *user, nqs_log_amp_fn_t ref_fn, void *ref_user, double mu,
                       double *trace) {
    if (!cfg || !a || !s || !ref_fn) return -1;        // src/nqs/nqs_optimizer.c:725-742
    nqs_sampler_thermalize(s);
    for (int it = 0; it < cfg->num_iterations; it++) {
        nqs_sr_step_info_t info;
        int rc = nqs_sr_step_excited(cfg, sx, sy, a, s, fn, user, ref_fn, ref_user, mu, &info);
        if (rc != 0) return rc;
        if (trace) trace[it] = info.mean_energy;
    }
    return 0;
}

// Real-time tVMC, forward Euler (src/nqs/nqs_optimizer.c:888-993): Re(S) delta = Im(F)
// on the holomorphic metric, theta += dt delta.
int nqs_tvmc_step_real_time(const nqs_config_t *cfg, double dt, int sx, int sy, nqs_ansatz_t *a,
                            nqs_sampler_t *s, nqs_log_amp_fn_t fn, void *user, nqs_sr_step_info_t *info) {
    if (!cfg || !a || !s) return -1;
    StepIn in{cfg, sx, sy, (Ansatz *)a, (Sampler *)s, nullptr, cfg->num_samples, fn, user, nullptr, nullptr, 4,
              nullptr, nullptr, nullptr, nullptr, 0.0, 1, dt, 0};
    if (nqs_sampler_num_sites(s) != ((Ansatz *)a)->N) {
        set_error("sampler and ansatz disagree on num_sites");
        return -1;
    }
    return sr_step_impl(in, info, nullptr, nullptr);
}

// Real-time tVMC, Heun (src/nqs/nqs_optimizer.c:815-886): k1 at theta, k2 at theta + dt k1
// (a second sampling), theta += dt (k1 + k2) / 2.  The snapshot, probe and average stay on
// the device.
int nqs_tvmc_step_heun(const nqs_config_t *cfg, double dt, int sx, int sy, nqs_ansatz_t *ah, nqs_sampler_t *s,
                       nqs_log_amp_fn_t fn, void *user, nqs_sr_step_info_t *info) {
    if (!cfg || !ah || !s) return -1;
    Ansatz *a = (Ansatz *)ah;
    if (nqs_sampler_num_sites(s) != a->N) {
        set_error("sampler and ansatz disagree on num_sites");
        return -1;
    }
    StepIn in{cfg, sx, sy, a, (Sampler *)s, nullptr, cfg->num_samples, fn, user, nullptr, nullptr, 4,
              nullptr, nullptr, nullptr, nullptr, 0.0, 1, dt, 1};
    nqs_sr_step_info_t i1{}, i2{};
    if (sr_step_impl(in, &i1, nullptr, nullptr) != 0) return -1;      // k1 in the workspace, theta unchanged
    Workspace &w = g_ws;
    const long P = a->P;
    cudaStream_t st = ctx().stream;
    if (!w.theta0.ensure(P) || !w.kacc.ensure(P) ||
        !NQS_CUDA(cudaMemcpyAsync(w.theta0.p, a->d_params.p, sizeof(double) * P, cudaMemcpyDeviceToDevice, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(w.kacc.p, w.delta.p, sizeof(double) * P, cudaMemcpyDeviceToDevice, st)))
        return -1;
    k_apply<<<1, 1024, 0, st>>>(a->d_params.p, w.kacc.p, P, -dt, w.scal.p, w.status.p, 0);   // theta0 + dt k1
    // the probe parameters go to the host mirror too: every step starts by uploading the
    // mirror (callers may edit the parameters in place through nqs_ansatz_params_raw)
    if (!NQS_CUDA(cudaGetLastError()) || !ansatz_refresh_derived(a) || !ansatz_pull(a)) return -1;
    const int rc2 = sr_step_impl(in, &i2, nullptr, nullptr);                                  // k2
    if (!NQS_CUDA(cudaMemcpyAsync(a->d_params.p, w.theta0.p, sizeof(double) * P, cudaMemcpyDeviceToDevice, st)))
        return -1;
    if (rc2 == 0) {
        k_heun_average<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(w.kacc.p, w.delta.p, P);
        k_apply<<<1, 1024, 0, st>>>(a->d_params.p, w.kacc.p, P, -dt, w.scal.p, w.status.p, 0);
    }
    double norm2 = 0.0;
    if (!NQS_CUDA(cudaGetLastError()) || !ansatz_refresh_derived(a) ||
        !NQS_CUDA(cudaMemcpyAsync(&norm2, w.scal.p + S_NORM2, sizeof(double), cudaMemcpyDeviceToHost, st)) ||
        !ansatz_pull(a))
        return -1;
    if (rc2 != 0) return rc2;
    if (info) {
        info->mean_energy = i1.mean_energy;
        info->variance_energy = i1.variance_energy;
        info->update_norm = sqrt(norm2) * fabs(dt);
        info->acceptance_ratio = nqs_sampler_acceptance_ratio(s);
        info->cg_iterations = i1.cg_iterations + i2.cg_iterations;
        info->converged = i1.converged && i2.converged;
    }
    return 0;
}

}  // extern "C"

// ====================================================================== no-allocation MinSR solve
//
// nqs_gpu_minsr_solve_noalloc solves the MinSR system for a Jacobian and local
// energies that the caller already holds in device memory, without allocating
// any device memory.  It is for callers that cannot call cudaMalloc: a host
// framework that owns (and has pre-reserved) all device memory, so that a
// stray cudaMalloc from a plug-in can fail or fragment its pool, or a
// latency-critical loop that must not enter the driver's allocator.  All of
// its scratch lives in one statically sized device array below, which every
// GPU that loads this library holds until the process exits.
namespace nqs {

constexpr int kNoAllocMaxSamples = 1024;     // T is N_s x N_s doubles (8 MiB at the limit)
constexpr long kNoAllocMaxParams = 16384;
constexpr size_t kNoAllocScratchDoubles = (size_t)kNoAllocMaxSamples * kNoAllocMaxSamples  // T
                                          + (size_t)kNoAllocMaxParams                       // <O_k>
                                          + 3 * (size_t)kNoAllocMaxSamples                  // eps, y, z
                                          + 16                                              // scalars
                                          + 16;                                             // status words

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Gram of the centred Jacobian with the centring done while staging tiles:
// T[i][j] = scale * sum_k (O[i][k] - m_k)(O[j][k] - m_k) (+ shift on the
// diagonal), lower triangle.  The caller's O is only read.
__global__ void __launch_bounds__(256) k_gram_fp64_centred(const double *__restrict__ O, int Ns, long P,
                                                           const double *__restrict__ m, double scale,
                                                           double shift, double *T) {
    __shared__ double As[KC][TG + 1], Bs[KC][TG + 1];
    int bi, bj;
    tri_tile(blockIdx.x, bi, bj);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int r0 = bi * TG, c0 = bj * TG;
    double acc[4][4] = {};
    for (long kk = 0; kk < P; kk += KC) {
        for (int e = tid; e < TG * KC; e += 256) {
            int rr = e / KC, cc = e % KC;
            long k = kk + cc;
            int ra = r0 + rr, rb = c0 + rr;
            As[cc][rr] = (ra < Ns && k < P) ? O[(size_t)ra * P + k] - m[k] : 0.0;
            Bs[cc][rr] = (rb < Ns && k < P) ? O[(size_t)rb * P + k] - m[k] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < KC; c++) {
            double av[4], bv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) av[q] = As[c][ty + 16 * q];
#pragma unroll
            for (int q = 0; q < 4; q++) bv[q] = Bs[c][tx + 16 * q];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            int i = r0 + ty + 16 * a, j = c0 + tx + 16 * b;
            if (i < Ns && j <= i) T[(size_t)i * Ns + j] = acc[a][b] * scale + (i == j ? shift : 0.0);
        }
}

// delta_k = scale * sum_i (O[i][k] - m_k) y_i  (status[I_FAIL] >= 0 -> 0).
__global__ void k_col_dot_centred(const double *__restrict__ O, int Ns, long P, const double *__restrict__ m,
                                  const double *__restrict__ y, double scale, const int *status,
                                  double *out) {
    __shared__ double a[8][33];
    long k = (long)blockIdx.x * 32 + threadIdx.x;
    double s = 0.0;
    if (k < P)
        for (int i = threadIdx.y; i < Ns; i += 8) s += (O[(size_t)i * P + k] - m[k]) * y[i];
    a[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && k < P) {
        double S = 0.0;
        for (int q = 0; q < 8; q++) S += a[q][threadIdx.x];
        out[k] = status[I_FAIL] >= 0 ? 0.0 : S * scale;
    }
}

// ||delta||^2 into scal[S_NORM2] (one block).
__global__ void k_norm2(const double *__restrict__ d, long P, double *scal) {
    __shared__ double red[1024];
    double s = 0.0;
    for (long k = threadIdx.x; k < P; k += blockDim.x) s += d[k] * d[k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) scal[S_NORM2] = red[0];
}

// Device address of the scratch array, looked up once per device and context.
// The address belongs to the context that loaded this module: after a
// cudaDeviceReset the device gets a new primary context (and a new copy of the
// array), so the cached address is looked up again when the current context's
// unique id (cuCtxGetId: unique for the life of the process, unlike the handle
// value, which a re-created primary context may reuse) differs from the one it
// was taken in.
static double *g_noalloc_ptr[64];
static unsigned long long g_noalloc_ctx[64];
static std::mutex g_noalloc_mu;

// Driver entry points, looked up through the runtime (the library does not link the
// driver library, so it loads on hosts without one).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

static bool driver_fn(const char *name, int version, void **fn) {
    cudaDriverEntryPointQueryResult q;
    *fn = nullptr;
    return cudaGetDriverEntryPointByVersion(name, fn, version, cudaEnableDefault, &q) == cudaSuccess &&
           q == cudaDriverEntryPointSuccess && *fn;
}

// The unique id of the context current on this thread (0 when there is none).
static unsigned long long current_context_id(int dev) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current && !driver_fn("cuCtxGetCurrent", 4000, (void **)&get_current)) return 0;
    if (!get_id && !driver_fn("cuCtxGetId", 12000, (void **)&get_id)) return 0;
    CUcontext cur = nullptr;
    if (get_current(&cur) == CUDA_SUCCESS && !cur) {
        // no context current on this thread yet: make the device's primary context
        // current (cudaSetDevice initialises it)
        if (cudaSetDevice(dev) != cudaSuccess || get_current(&cur) != CUDA_SUCCESS) cur = nullptr;
    }
    unsigned long long id = 0;
    if (!cur || get_id(cur, &id) != CUDA_SUCCESS) return 0;
    return id;
}

static double *noalloc_scratch(int dev) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return nullptr;
    }
    const unsigned long long id = current_context_id(dev);
    if (!id) {
        set_error("nqs_gpu_minsr_solve_noalloc: no current CUDA context on device %d", dev);
        return nullptr;
    }
    if (!g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != id) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("cudaGetSymbolAddress(g_noalloc_scratch) failed: %s", cudaGetErrorString(e));
            return nullptr;
        }
        g_noalloc_ptr[dev] = (double *)p;
        g_noalloc_ctx[dev] = id;
    }
    return g_noalloc_ptr[dev];
}

}  // namespace nqs

extern "C" {

// See nqs_gpu.h.  Same factorisation and solve as the MinSR step (blocked FP64
// Cholesky, blocked triangular solves); the upstream +1e-6 retry is not run
// here (it needs a second N_s x N_s copy): a failed factorisation returns
// delta = 0 with out_info->converged = 0.
int nqs_gpu_minsr_solve_noalloc(const double *d_O, const double *d_E, int Ns, long P, double shift,
                                double *d_delta, nqs_sr_step_info_t *out_info, void *stream_ptr) {
    clear_error();
    if (!d_O || !d_E || !d_delta || Ns <= 0 || P <= 0) {
        set_error("nqs_gpu_minsr_solve_noalloc: NULL buffer or non-positive size");
        return -1;
    }
    if (Ns > kNoAllocMaxSamples || P > kNoAllocMaxParams) {
        set_error("nqs_gpu_minsr_solve_noalloc: N_s = %d, N_p = %ld exceed the static scratch limits "
                  "(N_s <= %d, N_p <= %ld)", Ns, P, kNoAllocMaxSamples, kNoAllocMaxParams);
        return -1;
    }
    int dev = 0;
    if (!NQS_CUDA(cudaGetDevice(&dev))) return -1;
    double *base = noalloc_scratch(dev);
    if (!base) return -1;
    cudaStream_t st = (cudaStream_t)stream_ptr;
    double *T = base;
    double *gm = T + (size_t)kNoAllocMaxSamples * kNoAllocMaxSamples;
    double *eps = gm + kNoAllocMaxParams;
    double *y = eps + kNoAllocMaxSamples;
    double *z = y + kNoAllocMaxSamples;
    double *scal = z + kNoAllocMaxSamples;
    int *status = (int *)(scal + 16);
    // the array keeps the previous call's contents: reset what must start fresh
    if (!NQS_CUDA(cudaMemsetAsync(scal, 0, 16 * sizeof(double), st)) ||
        !NQS_CUDA(cudaMemsetAsync(status, 0xff, 16 * sizeof(int), st)))
        return -1;
    k_energy_stats<<<1, 1024, 0, st>>>(d_E, Ns, scal, eps);
    dim3 cb(32, 8), cg((unsigned)((P + 31) / 32));
    k_col_stats<<<cg, cb, 0, st>>>(d_O, Ns, P, nullptr, scal, gm, nullptr);
    int nt = (Ns + TG - 1) / TG;
    k_gram_fp64_centred<<<nt * (nt + 1) / 2, 256, 0, st>>>(d_O, Ns, P, gm, 1.0 / (double)Ns, shift, T);
    for (int k0 = 0; k0 < Ns; k0 += NB) {
        int kb = Ns - k0 < NB ? Ns - k0 : NB;
        k_potrf_diag<<<1, dim3(32, 32), 0, st>>>(T, Ns, k0, kb, status);
        int k1 = k0 + kb, rest = Ns - k1;
        if (rest <= 0) break;
        k_trsm_panel<<<(rest + 127) / 128, 128, 0, st>>>(T, Ns, k0, kb, kb, k1, status, 0);
        int ntt = (rest + TG - 1) / TG;
        k_syrk_update<<<ntt * (ntt + 1) / 2, 256, 0, st>>>(T, Ns, k0, kb, k1, status);
    }
    // forward and backward substitution (skipped work is harmless: delta is
    // zeroed below when the factorisation failed)
    if (!NQS_CUDA(cudaMemcpyAsync(z, eps, sizeof(double) * Ns, cudaMemcpyDeviceToDevice, st))) return -1;
    for (int k0 = 0; k0 < Ns; k0 += NB) {
        int kb = Ns - k0 < NB ? Ns - k0 : NB, rest = Ns - k0 - kb;
        k_trsv_fwd<<<rest > 0 ? (rest + 127) / 128 : 1, 128, 0, st>>>(T, Ns, k0, kb, z, y);
    }
    if (!NQS_CUDA(cudaMemcpyAsync(z, y, sizeof(double) * Ns, cudaMemcpyDeviceToDevice, st))) return -1;
    for (int k0 = ((Ns - 1) / NB) * NB; k0 >= 0; k0 -= NB) {
        int kb = Ns - k0 < NB ? Ns - k0 : NB;
        k_trsv_bwd<<<k0 > 0 ? (k0 + 127) / 128 : 1, 128, 0, st>>>(T, Ns, k0, kb, z, y);
    }
    k_col_dot_centred<<<cg, cb, 0, st>>>(d_O, Ns, P, gm, y, 1.0 / (double)Ns, status, d_delta);
    k_norm2<<<1, 1024, 0, st>>>(d_delta, P, scal);
    if (!NQS_CUDA(cudaGetLastError())) return -1;
    double hs[16];
    int hst[16];
    if (!NQS_CUDA(cudaMemcpyAsync(hs, scal, sizeof(hs), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaMemcpyAsync(hst, status, sizeof(hst), cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return -1;
    if (out_info) {
        out_info->mean_energy = hs[S_EMEAN];
        out_info->variance_energy = hs[S_ESQ] - hs[S_EMEAN] * hs[S_EMEAN];
        out_info->update_norm = sqrt(hs[S_NORM2]);
        out_info->acceptance_ratio = 0.0;
        out_info->cg_iterations = 0;
        out_info->converged = hst[I_FAIL] < 0 ? 1 : 0;
    }
    return 0;
}

}  // extern "C"
