// Internal declarations shared by the translation units of libnqs_gb300.so.
//
// Data layout in HBM (one GPU, one stream):
//   * parameters: FP64 in the upstream layout (src/nqs/nqs_ansatz.c:39-41,
//     :219-247) plus derived copies transposed to [site][hidden] so that a warp
//     whose lanes own hidden units reads one weight column with one coalesced
//     256-byte load per flipped site;
//   * configurations: one uint64 per configuration, bit i = 1 <-> spin -1
//     (the basis convention of src/nqs/nqs_lanczos.c:16-20), N <= 64;
//   * Jacobian O: FP64 row-major [N_s][N_p] exactly as the upstream optimiser
//     (src/nqs/nqs_optimizer.c:164), so that the row and column sweeps of the
//     solvers are unit-stride.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

extern "C" {
#include "nqs/nqs_config.h"
#include "nqs/nqs_ansatz.h"
#include "nqs/nqs_sampler.h"
#include "nqs/nqs_gradient.h"
#include "nqs/nqs_translation.h"
#include "nqs/nqs_optimizer.h"
#include "nqs/nqs_marshall.h"
#include "nqs/nqs_symproj.h"
#include "nqs/nqs_gpu.h"
}

namespace nqs {

constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxSites = 64;
constexpr int kMaxJ = 8;           // hidden units per lane -> M <= 256

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
void clear_error();
bool cuda_ok(cudaError_t e, const char *what);
#define NQS_CUDA(call) ::nqs::cuda_ok((call), #call)

// ---------------------------------------------------------------- context
struct ProfEvent {
    const char *name;
    cudaEvent_t a, b;
};

struct Context {
    bool initialised = false;
    bool usable = false;
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    nqs_gpu_options_t opts{};
    std::mutex mu;
    bool profiling = false;
    std::vector<ProfEvent> prof_pending;
    std::map<std::string, std::pair<long, double>> prof_done;
    long launches = 0;
};
Context &ctx();
bool ensure_context();              // false (and error set) when no usable device

// Bracket a launch with profiling events when enabled and count it.
struct LaunchScope {
    ProfEvent ev{};
    bool on;
    explicit LaunchScope(const char *name);
    ~LaunchScope();
};
#define NQS_LAUNCH(name) ::nqs::LaunchScope _nqs_ls_##__LINE__(name)

// ---------------------------------------------------------------- device buffers
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    bool ensure(size_t count) {
        if (count <= n && p) return true;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (count == 0) count = 1;
        if (!NQS_CUDA(cudaMalloc(&p, count * sizeof(T)))) return false;
        n = count;
        return true;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
};

// ---------------------------------------------------------------- device program
enum : int { KIND_MF = 0, KIND_VIT = 2, KIND_RBM = 5, KIND_CRBM = 6, KIND_VITC = 7, KIND_MLP = NQS_GPU_ANSATZ_MLP };

// Factored-attention ViT tables (doubles, derived from the parameters after every
// update; complex quantities as (re, im) pairs, imaginary parts 0 for the real ViT):
// column sums s_pred[N] of the attention matrix, softmax weights f[N]
// (P_ij = f[(i - j) mod N]), sum_j s_pred_j, b_out, c1 = u.w_emb, c0 = u.b_emb with
// u = V^T W_out, then u, V w_emb, V b_emb, w_emb, b_emb, W_out [d] each.
struct VitTab {
    int sp, f, bsum, bout, c1, c0, u, vw, vb, w, b, W, total;
};
__host__ __device__ inline VitTab vit_tab(int N, int d) {
    VitTab t;
    t.sp = 0;
    t.f = N;
    t.bsum = 2 * N;
    t.bout = t.bsum + 1;
    t.c1 = t.bout + 2;
    t.c0 = t.c1 + 2;
    t.u = t.c0 + 2;
    t.vw = t.u + 2 * d;
    t.vb = t.vw + 2 * d;
    t.w = t.vb + 2 * d;
    t.b = t.w + 2 * d;
    t.W = t.b + 2 * d;
    t.total = t.W + 2 * d;
    return t;
}
__host__ __device__ inline bool is_vit(int kind) { return kind == KIND_VIT || kind == KIND_VITC; }

// Padded row pitch of the MLP's FP32 W2 tables and the floats of its FP32 tables.
__host__ __device__ inline int mlp32_pitch(int M) { return (M + 31) / 32 * 32; }
inline size_t mlp32_floats(int N, int M) { return (size_t)N * M + 2 * (size_t)M * mlp32_pitch(M) + 4 * (size_t)M + 2; }

struct DevAnsatz {
    int kind, N, M;
    long P;
    const double *p;     // device params, upstream layout
    const double *wtr;   // [N][M] real weights transposed (RBM, cRBM); MLP: W1^T; ViT: VitTab tables
    const double *wti;   // [N][M] imaginary weights transposed (cRBM); MLP: W2^T [M][M]
    // FP32 tables of the RBM / cRBM (complex, imaginary part 0 for the RBM),
    // rebuilt with the transposed copies: W^T [N][M], cosh(2 W^T), sinh(2 W^T)
    // [N][M], visible bias [N], hidden bias [M]
    const float2 *w32, *ch32, *sh32, *a32, *b32;
    // FP32 tables of the MLP (floats): W1^T [N][M], then W2^T and W2 as [M][MP]
    // rows padded with zeros to MP = 32 ceil(M / 32), then b1, b2, w_re, w_im
    // [M], c_re, c_im
    const float *m32;
    // FP64 tables of the RBM / cRBM for the product-form FP64 chains: cosh(2 W^T) (re, im)
    // then sinh(2 W^T) (re, im), each [N][M]
    const double *cs64;
};

struct DevAmp {
    DevAnsatz a;
    int n_outer;                 // Marshall layers outside the projection
    uint64_t outer_mask[3];
    int G;                       // symmetry projection group size, 0 = none
    const int *perm;             // [G][N] device
    const double *chars;         // [G] device
    int n_inner;                 // Marshall layers inside the projection
    uint64_t inner_mask[3];
};

// Hamiltonian as bond groups (built on the host from the lattice, in the
// upstream enumeration order; see hamiltonian_build()).
struct DevHam {
    int kind;           // NQS_HAM_*
    int N;
    int nb1, nb2;       // bond counts: group 1 (NN / kagome), group 2 (J1-J2 diagonals)
    const int *b1;      // [nb1][2] device
    const int *b2;      // [nb2][2] device
    double J, J2, Jz, Jxy, Gamma;
};

// ---------------------------------------------------------------- host objects
struct Ansatz {
    int kind, N, M;
    long P;
    double *h_params = nullptr;     // pinned host mirror (returned by params_raw)
    double *h_shadow = nullptr;     // last value known to be on the device
    DevBuf<double> d_params, d_wtr, d_wti;
    DevBuf<float2> d_f32;           // RBM / cRBM / MLP FP32 tables (see DevAnsatz)
    DevBuf<double> d_cs64;          // RBM / cRBM FP64 cosh / sinh(2 W^T) tables (see DevAnsatz)
    bool dev_valid = false;
};

// Upload the host mirror when it changed (or always with force: the SR steps
// take the mirror as the step's input).
bool ansatz_sync(Ansatz *a, bool force = false);
bool ansatz_refresh_derived(Ansatz *a);      // rebuild transposed copies (device)
bool ansatz_pull(Ansatz *a);                 // device -> host mirror
DevAnsatz ansatz_dev(const Ansatz *a);

// Resolve a (log_amp, user) callback pair into a device program.
bool build_amp(nqs_log_amp_fn_t fn, void *user, int num_sites, DevAmp *out, Ansatz **base);
bool hamiltonian_build(const nqs_config_t *cfg, int size_x, int size_y, DevHam *out);

// configurations: host int +-1 [B][N] <-> device bits
bool upload_spins(const int *spins, int B, int N, uint64_t **d_bits);
uint64_t pack_spins(const int *s, int N);

// kernels exported across translation units
bool launch_log_amp(const DevAmp &A, const uint64_t *bits, int B, double *la, double *ar);
bool launch_local_estimator(const DevAmp &A, const DevHam &H, const uint64_t *bits, int B,
                            double *E_re, double *E_im, double *O, double *O_im, int grad_mode,
                            bool fp32 = false);
// True when the FP32 estimator / sampler can run this program (RBM or cRBM
// with Marshall layers, no symmetry projection).
bool fp32_capable(const DevAmp &A);        // RBM / cRBM FP32 product-form tables
bool fp32_mlp_capable(const DevAmp &A);    // MLP with width <= 128 and FP32 tables
bool launch_gradient(const DevAnsatz &a, const uint64_t *bits, int B, int mode, double *O, double *Oi);
bool launch_symproj_gradient(const DevAmp &A, const uint64_t *bits, int B, double *O);
bool launch_symproj_gradient_complex(const DevAmp &A, const uint64_t *bits, int B, double *O, double *Oi);
bool launch_bits_to_spins(const uint64_t *bits, int B, int N, int *out);

// CG-SR solve (S + eps I) d = F in one cooperative launch (upstream cg_solve
// semantics); writes d, scal[S_RS, S_RS0, S_PAP], status[I_DONE, I_ITERS, I_CONV].
bool cg_sr_solve(const double *O, int Ns, long P, const double *F, const double *gm, double eps, double tol,
                 int max_iters, double *d, double *scal, int *status, const double *O2 = nullptr,
                 const double *gm2 = nullptr, double fac = 1.0);

// Relative residual |r| / |rhs| above which a mixed solve counts as broken down
// and the step is solved again in FP64.
constexpr double MIXED_RESID_MAX = 1e-6;

// Mixed-precision MinSR solve (nqs_mixed.cu): centres O in place and solves in
// sample space, (O_c O_c^T / N_s + shift I) y = eps (writes y), or in parameter
// space, (O_c^T O_c / N_s + shift I) delta = O_c^T eps / N_s (writes delta and
// sets *param_space); space_opt 0 picks the smaller system, 1 samples, 2
// parameters.  *out_fail >= 0 when the FP32 factor broke down.
// after_launch, when given, is called once the solve is enqueued and before the host waits for
// it, with the solve's status word, error word and residual norms (device pointers) and
// whether it solves in parameter space, so that a caller can enqueue work that depends on
// the solve without a host round trip.
using MixedAfterLaunch = std::function<bool(const int *status, const int *err, const double *nrm, bool param_space)>;
bool minsr_mixed_solve(double *O, const double *gm, const double *eps, int Ns, long P, double shift, int sweeps,
                       int passes, int space_opt, double *y, double *delta, bool *param_space, double *out_resid,
                       int *out_fail, const MixedAfterLaunch &after_launch = nullptr);

// theta -= lr delta and ||delta||^2 into scal[S_NORM2] on the library stream, with delta
// taken as zero when the mixed solve broke down (a non-positive FP32 pivot in status[0], or
// |r| / |rhs| above MIXED_RESID_MAX from nrm) or its kernels raised the error word
// (nqs_batch.cu).
bool enqueue_gated_apply(double *params, const double *delta, long P, double lr, double *scal, const int *mstatus,
                         const int *merr, const double *mnrm);

// Device scalar block of an SR step (doubles): [0] e_mean [1] e_sq_mean
// [2] ||delta||^2 [3] rs [4] rs0 [5] pAp [6] alpha [7] u mean [8] tau_int
// [9] ESS; status ints: [0] chol fail column (-1 ok) [1] cg done flag [2] cg
// iterations [3] cg converged [4] retry ran [5] failure after the retry.
enum { S_EMEAN = 0, S_ESQ = 1, S_NORM2 = 2, S_RS = 3, S_RS0 = 4, S_PAP = 5, S_ALPHA = 6, S_UMEAN = 7,
       S_TAU = 8, S_ESS = 9 };
enum { I_FAIL = 0, I_DONE = 1, I_ITERS = 2, I_CONV = 3, I_RETRY = 4, I_FAIL2 = 5 };

// Batches of mixed solves (nqs_mixed.cu): one system per instance, the
// factor / inverse / refinement of all of them in one cooperative launch.
struct MixedSys;
struct MixedBatch;
MixedSys *mixed_sys_create();
void mixed_sys_free(MixedSys *m);
bool mixed_sys_prepare(MixedSys *m, double *O, const double *gm, const double *eps, int Ns, long P, double shift,
                       int sweeps, int passes, int space_opt, double *y, double *delta);
void mixed_sys_front(MixedSys *m, cudaStream_t st, bool with_split);
bool mixed_sys_param_space(const MixedSys *m);
int mixed_sys_order(const MixedSys *m);
const int *mixed_sys_status(const MixedSys *m);
const int *mixed_sys_err(const MixedSys *m);
const double *mixed_sys_nrm(const MixedSys *m);
int mixed_batch_capacity();
MixedBatch *mixed_batch_create(MixedSys *const *sys, int count, const int *ctas, int bd_from);
// MLP local energies with the second layer on the tensor cores (nqs_mlp_tc.cu)
bool mlp_tc_capable(const DevAmp &A, const DevHam &H);
bool launch_mlp_eloc_tc(const DevAmp &A, const DevHam &H, const uint64_t *bits, int B, double *Er, double *Ei);
int mixed_bd_default();
void mixed_batch_free(MixedBatch *b);
bool mixed_batch_launch(MixedBatch *b, cudaStream_t st);

// Stream-only pieces of the SR step (nqs_sr.cu), for captured sequences.
// <E>, <E^2> (scal), eps = E - <E>, tau_int and ESS (scal) over multiple
// blocks; scratch holds energy_scratch_doubles(Ns) doubles, zero before its
// first use (its tickets return to zero after each call).
size_t energy_scratch_doubles(int Ns);
bool enqueue_energy_stats(const double *E, int Ns, int chains, double *scal, double *eps, double *scratch);
bool enqueue_col_means(const double *O, int Ns, long P, const double *scal, double *gm, double *part);
long col_stats_scratch(int Ns, long P);
bool enqueue_col_dot(const double *O, int Ns, long P, const double *y, double scale, double *out);
// FP64 MinSR solve (upstream retry semantics) on a centred O; and the update
// delta = O^T y / N_s from it.  Return 0 / -1 (CUDA error).
int minsr_fp64_solve(const double *O, const double *eps, int Ns, long P, double shift, double *y, int *conv);
int minsr_fp64_delta(const double *O, const double *eps, int Ns, long P, double shift, double *delta, int *conv);

// thread-local statistics of the last SR step
nqs_gpu_step_stats_t &step_stats();

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;   // XOR butterfly: every lane ends with the bitwise-identical sum
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int spin_of(uint64_t bits, int i) {
    return 1 - 2 * (int)((bits >> i) & 1ull);
}

// log(2 cosh z) for z = x + i y in the overflow-safe form used upstream
// (src/nqs/nqs_ansatz.c:309-318): with e = exp(-2|x|),
//   2 cosh z = e^{|x|} ((1 + e) cos y + i sgn(x) (1 - e) sin y).
__device__ __forceinline__ void clogcosh(double x, double y, double &la, double &ar) {
    double ax = fabs(x);
    double e = exp(-2.0 * ax);
    double sy, cy;
    sincos(y, &sy, &cy);
    double re = (1.0 + e) * cy;
    double im = (x >= 0.0 ? 1.0 : -1.0) * (1.0 - e) * sy;
    double mag = hypot(re, im);
    la = ax + (mag > 0.0 ? log(mag) : -1e300);
    ar = atan2(im, re);
}

// Re log(2 cosh z) only: |x| + 0.5 log(1 + 2 e cos 2y + e^2), e = exp(-2|x|).
__device__ __forceinline__ double rlogcosh(double x, double y) {
    double ax = fabs(x);
    double e = exp(-2.0 * ax);
    return ax + 0.5 * log1p(e * (2.0 * cos(2.0 * y) + e));
}

// Real log(2 cosh x), src/nqs/nqs_ansatz.c:291.
__device__ __forceinline__ double logcosh_r(double x) {
    double ax = fabs(x);
    return ax + log1p(exp(-2.0 * ax));
}

// tanh(x + i y) through sinh / cosh, the formula of src/nqs/nqs_ansatz.c:961-972.
__device__ __forceinline__ void ctanh_d(double x, double y, double &tr, double &ti) {
    double cxr = cosh(x), sxr = sinh(x);
    double sy, cy;
    sincos(y, &sy, &cy);
    double nr = sxr * cy, ni = cxr * sy;
    double dr = cxr * cy, di = sxr * sy;
    double den = dr * dr + di * di;
    if (den < 1e-300) den = 1e-300;
    tr = (nr * dr + ni * di) / den;
    ti = (ni * dr - nr * di) / den;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), computed redundantly by
// every lane of a warp so that a chain's random numbers need no shuffles.
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        uint4 n;
        n.x = hi1 ^ c.y ^ k.x;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k.y;
        n.w = lo0;
        c = n;
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

}  // namespace nqs
