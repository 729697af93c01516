// Warp-cooperative evaluation of the device amplitude program.
//
// One warp evaluates one configuration: lanes own hidden units (h = lane +
// 32 j), so a hidden pre-activation theta_h = b_h + sum_i W_hi s_i is summed
// by one lane in the upstream order (ascending i; s_i = +-1 makes every
// product exact, so theta is bit-identical to upstream), the weight column of
// site i is one coalesced load across the warp, and the sum over hidden units
// is a 5-step XOR butterfly that leaves the same value in every lane.
#pragma once
#include "nqs_internal.cuh"

namespace nqs {

__device__ __forceinline__ long crbm_pr(const DevAnsatz &a) {
    return (long)a.N + a.M + (long)a.M * a.N;
}

// Visible-bias term sum_i a_i s_i (real and imaginary parts).
__device__ __forceinline__ void warp_visible(const DevAnsatz &a, uint64_t bits, double &vr, double &vi) {
    int lane = threadIdx.x & 31;
    double r = 0.0, im = 0.0;
    if (a.kind != KIND_MLP) {
        long Pr = a.kind == KIND_CRBM ? crbm_pr(a) : 0;
        for (int i = lane; i < a.N; i += 32) {
            double s = (double)spin_of(bits, i);
            r += a.p[i] * s;
            if (a.kind == KIND_CRBM) im += a.p[Pr + i] * s;
        }
    }
    vr = warp_sum(r);
    vi = warp_sum(im);
}

// theta_h of the RBM / complex RBM, summed in the upstream order.
__device__ __forceinline__ void rbm_theta(const DevAnsatz &a, uint64_t bits, int h, double &xr,
                                          double &xi) {
    long Pr = crbm_pr(a);
    xr = a.p[a.N + h];
    xi = a.kind == KIND_CRBM ? a.p[Pr + a.N + h] : 0.0;
    for (int i = 0; i < a.N; i++) {
        double s = (double)spin_of(bits, i);
        xr += a.wtr[(long)i * a.M + h] * s;
        if (a.kind == KIND_CRBM) xi += a.wti[(long)i * a.M + h] * s;
    }
}

// Deep MLP forward pass; `h1` is a per-warp scratch of M doubles.
__device__ __forceinline__ void warp_mlp_eval(const DevAnsatz &a, uint64_t bits, double &la, double &ar,
                                              double *h1) {
    int lane = threadIdx.x & 31;
    const int N = a.N, M = a.M;
    const double *b1 = a.p + (long)M * N;
    const double *b2 = b1 + M + (long)M * M;
    const double *wr = b2 + M, *wi = wr + M;
    for (int k = lane; k < M; k += 32) {
        double z = b1[k];
        for (int i = 0; i < N; i++) z += a.wtr[(long)i * M + k] * (double)spin_of(bits, i);
        h1[k] = tanh(z);
    }
    __syncwarp();
    double r = 0.0, im = 0.0;
    for (int j = lane; j < M; j += 32) {
        double z = b2[j];
        for (int k = 0; k < M; k++) z += a.wti[(long)k * M + j] * h1[k];
        double h2 = tanh(z);
        r += wr[j] * h2;
        im += wi[j] * h2;
    }
    __syncwarp();
    la = warp_sum(r) + wi[M];
    ar = warp_sum(im) + wi[M + 1];
}

// ---- FP32 MLP (mixed precision).  Lane l owns hidden units l + 32 q, q < MQ.
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// layer-1 pre-activations z1 = W1 s + b1 (ascending i)
template <int MQ>
__device__ __forceinline__ void mlp32_z1(const DevAnsatz &a, uint64_t s, float (&z1)[MQ]) {
    const int lane = threadIdx.x & 31, M = a.M, N = a.N;
    const float *b1 = a.m32 + (long)N * M + 2L * M * mlp32_pitch(M);
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        const int k = lane + 32 * q;
        float z = k < M ? b1[k] : 0.f;
        if (k < M)
            for (int i = 0; i < N; i++) z = fmaf((float)spin_of(s, i), a.m32[(long)i * M + k], z);
        z1[q] = z;
    }
}

// z1 after flipping site u (and v >= 0): z1 - 2 s_u W1[:, u] - 2 s_v W1[:, v]
template <int MQ>
__device__ __forceinline__ void mlp32_z1_flip(const DevAnsatz &a, uint64_t s, int u, int v, const float (&z1)[MQ],
                                              float (&out)[MQ]) {
    const int lane = threadIdx.x & 31, M = a.M;
    const float su = -2.f * (float)spin_of(s, u), sv = v >= 0 ? -2.f * (float)spin_of(s, v) : 0.f;
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        const int k = lane + 32 * q;
        float z = z1[q];
        if (k < M) {
            z = fmaf(su, a.m32[(long)u * M + k], z);
            if (v >= 0) z = fmaf(sv, a.m32[(long)v * M + k], z);
        }
        out[q] = z;
    }
}

// h1 = tanh(z1) (to the warp's shared row h1s and h1), h2 = tanh(W2 h1 + b2)
// with W2^T rows from shared memory (pitch MQ * 32), log|psi| and arg; every
// lane returns the same la / ar
template <int MQ>
__device__ __forceinline__ void mlp32_forward(const DevAnsatz &a, const float *w2t, const float (&z1)[MQ],
                                              float *h1s, float (&h1)[MQ], float (&h2)[MQ], float &la, float &ar) {
    const int lane = threadIdx.x & 31, M = a.M;
    constexpr int MP = 32 * MQ;
    const float *vec = a.m32 + (long)a.N * M + 2L * M * MP;
    const float *b2 = vec + M, *wr = vec + 2 * M, *wi = vec + 3 * M;
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        h1[q] = lane + 32 * q < M ? tanhf(z1[q]) : 0.f;
        h1s[lane + 32 * q] = h1[q];
    }
    __syncwarp();
    float z[MQ];
#pragma unroll
    for (int q = 0; q < MQ; q++) z[q] = lane + 32 * q < M ? b2[lane + 32 * q] : 0.f;
    for (int k = 0; k < M; k++) {
        const float h = h1s[k];
        const float *row = w2t + k * MP + lane;
#pragma unroll
        for (int q = 0; q < MQ; q++) z[q] = fmaf(row[32 * q], h, z[q]);
    }
    float r = 0.f, im = 0.f;
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        const int j = lane + 32 * q;
        h2[q] = j < M ? tanhf(z[q]) : 0.f;
        if (j < M) {
            r = fmaf(wr[j], h2[q], r);
            im = fmaf(wi[j], h2[q], im);
        }
    }
    la = warp_sum_f(r) + vec[4 * M];
    ar = warp_sum_f(im) + vec[4 * M + 1];
    __syncwarp();
}

// Factored-attention ViT (src/nqs/nqs_ansatz.c:357-473, :571-729).  Its attention scores
// depend on the parameters only, so with the tables of k_derive
// log psi = b_out + sum_j s_pred_j W_out.V e_j = b_out + c1 A + c0 B, A = sum_j s_pred_j s_j,
// B = sum_j s_pred_j: one warp sum per configuration.  Returns A (all lanes).
__device__ __forceinline__ double vit_spin_sum(const DevAnsatz &a, uint64_t bits, double *S = nullptr) {
    int lane = threadIdx.x & 31;
    double A = 0.0, s1 = 0.0;
    for (int j = lane; j < a.N; j += 32) {
        const double sj = (double)spin_of(bits, j);
        A = fma(a.wtr[j], sj, A);
        s1 += sj;
    }
    if (S) *S = warp_sum(s1);
    return warp_sum(A);
}

__device__ __forceinline__ void warp_vit_eval(const DevAnsatz &a, uint64_t bits, double &la, double &ar) {
    const VitTab T = vit_tab(a.N, a.M);
    const double *t = a.wtr;
    const double A = vit_spin_sum(a, bits), B = t[T.bsum];
    la = t[T.bout] + t[T.c1] * A + t[T.c0] * B;
    ar = t[T.bout + 1] + t[T.c1 + 1] * A + t[T.c0 + 1] * B;
}

// log psi of the base ansatz (all lanes return the same value).
__device__ __forceinline__ void warp_base_eval(const DevAnsatz &a, uint64_t bits, double &la, double &ar,
                                               double *scratch) {
    int lane = threadIdx.x & 31;
    if (a.kind == KIND_MLP) {
        warp_mlp_eval(a, bits, la, ar, scratch);
        return;
    }
    if (is_vit(a.kind)) {
        warp_vit_eval(a, bits, la, ar);
        return;
    }
    double vr, vi;
    warp_visible(a, bits, vr, vi);
    double hr = 0.0, hi = 0.0;
    if (a.kind == KIND_RBM || a.kind == KIND_CRBM) {
        for (int h = lane; h < a.M; h += 32) {
            double xr, xi;
            rbm_theta(a, bits, h, xr, xi);
            if (a.kind == KIND_RBM) {
                hr += logcosh_r(xr);
            } else {
                double t1, t2;
                clogcosh(xr, xi, t1, t2);
                hr += t1;
                hi += t2;
            }
        }
    }
    la = vr + warp_sum(hr);
    ar = vi + warp_sum(hi);
}

// (g.s)_i = s_{perm_g[i]} as a bit permutation (two ballots for N <= 64).
__device__ __forceinline__ uint64_t permute_bits(uint64_t bits, const int *perm_g, int N) {
    int lane = threadIdx.x & 31;
    int i0 = lane, i1 = lane + 32;
    bool b0 = i0 < N && ((bits >> perm_g[i0]) & 1ull);
    bool b1 = i1 < N && ((bits >> perm_g[i1]) & 1ull);
    uint32_t lo = __ballot_sync(0xffffffffu, b0);
    uint32_t hi = __ballot_sync(0xffffffffu, b1);
    return (uint64_t)lo | ((uint64_t)hi << 32);
}

// Marshall layers (src/nqs/nqs_marshall.c:29-40): arg += pi for odd parity,
// innermost layer first.
__device__ __forceinline__ double apply_marshall(double ar, uint64_t bits, int n, const uint64_t *masks) {
    for (int m = n - 1; m >= 0; m--) ar = ar + ((__popcll(bits & masks[m]) & 1) ? kPi : 0.0);
    return ar;
}

// Full program: outer Marshall o symproj o inner Marshall o base.
__device__ __forceinline__ void warp_amp_eval(const DevAmp &A, uint64_t bits, double &la, double &ar,
                                              double *scratch) {
    if (A.G == 0) {
        warp_base_eval(A.a, bits, la, ar, scratch);
    } else {
        // src/nqs/nqs_symproj.c:31-80 with an online log-sum-exp over g
        const int N = A.a.N;
        double mx = -1e300, sum = 0.0;
        for (int g = 0; g < A.G; g++) {
            uint64_t pb = permute_bits(bits, A.perm + (long)g * N, N);
            double l, a;
            warp_base_eval(A.a, pb, l, a, scratch);
            a = apply_marshall(a, pb, A.n_inner, A.inner_mask);
            double c = A.chars[g] * cos(a);
            if (l > mx) {
                sum = sum * exp(mx - l) + c;
                mx = l;
            } else {
                sum += c * exp(l - mx);
            }
        }
        double as = fabs(sum);
        if (as > 0.0) {
            la = log(as) + mx - 0.5 * log((double)A.G);
            ar = sum < 0.0 ? kPi : 0.0;
        } else {
            la = -1e300;
            ar = 0.0;
        }
    }
    ar = apply_marshall(ar, bits, A.n_outer, A.outer_mask);
}

// Parity count of all Marshall layers of a projection-free program.
__device__ __forceinline__ int marshall_count(const DevAmp &A, uint64_t bits) {
    int c = 0;
    for (int m = 0; m < A.n_outer; m++) c += __popcll(bits & A.outer_mask[m]) & 1;
    return c;
}

}  // namespace nqs
