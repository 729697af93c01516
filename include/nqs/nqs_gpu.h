/*
 * include/nqs/nqs_gpu.h -- GPU-only extensions of the NQS C API.
 *
 * None of these entry points exists upstream; they add what the upstream
 * nqs_config_t (whose layout is frozen) cannot express: many-chain Philox
 * sampling with exchange moves and a fixed-magnetisation start, periodic
 * square lattices, the precision mode of the SR solve, batched device entry
 * points on caller-supplied configurations ("replay" of identical batches),
 * the deep MLP ansatz, and per-kernel timing.
 */
#ifndef NQS_GPU_H
#define NQS_GPU_H

#include "nqs_config.h"
#include "nqs_ansatz.h"
#include "nqs_sampler.h"
#include "nqs_optimizer.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 2-hidden-layer tanh MLP, N -> width -> width -> (Re, Im) head.  Parameter
 * layout: W1[width][N], b1[width], W2[width][width], b2[width], w_re[width],
 * w_im[width], c_re, c_im.  Selected through nqs_config_t.ansatz. */
#define NQS_GPU_ANSATZ_MLP 100

#define NQS_GPU_SPACE_AUTO       0
#define NQS_GPU_SPACE_SAMPLES    1
#define NQS_GPU_SPACE_PARAMETERS 2
#define NQS_GPU_SPACE_SMALLER    3   /* fp64_space: whichever system is smaller */

typedef enum {
    NQS_GPU_RNG_XORSHIFT_COMPAT = 0,  /* upstream single chain, same sequence */
    NQS_GPU_RNG_PHILOX          = 1   /* num_chains chains, Philox4x32-10 */
} nqs_gpu_rng_t;

typedef enum {
    NQS_GPU_MOVE_SINGLE_FLIP = 0,
    NQS_GPU_MOVE_EXCHANGE    = 1      /* swap the spins of a random bond */
} nqs_gpu_move_t;

typedef enum {
    NQS_GPU_PREC_FP64  = 0,           /* every stage in FP64 (parity path) */
    NQS_GPU_PREC_MIXED = 1            /* tensor-core Gram, FP64 refinement */
} nqs_gpu_precision_t;

typedef struct {
    int num_chains;      /* Philox chains (one warp each); compat mode uses 1 */
    int rng;             /* nqs_gpu_rng_t */
    int move;            /* nqs_gpu_move_t (exchange needs rng = PHILOX) */
    int n_down;          /* >= 0: start each chain with this many down spins */
    int square_pbc;      /* 1: periodic chain / square lattices */
    int precision;       /* nqs_gpu_precision_t for MinSR */
    int refine_sweeps;   /* MIXED: maximum FP64 preconditioned-CG iterations of the solve (stops at |r|/|rhs| <= 1e-10) */
    int gram_passes;     /* MIXED: 1 = single TF32 pass, 3 = split (hi/lo) passes */
    int mixed_space;     /* MIXED: system solved, 0 = the smaller one, 1 = sample space
                          * (N_s x N_s, O O^T), 2 = parameter space (N_p x N_p, O^T O);
                          * both give the same delta (push-through identity) */
    int lattice_x;       /* exchange moves: lattice whose nearest-neighbour bonds */
    int lattice_y;       /*   are swapped (0 x 0 = periodic ring of N sites)      */
    int lattice_kagome;  /*   1: kagome cells, bonds of kagome_pbc = 1          */
    int mixed_check;     /* MIXED: also solve in FP64 on the same samples and
                          * report the delta-theta error (step stats) */
    int fp32_estimator;  /* MIXED: RBM / cRBM local energies, Jacobian rows and
                          * Metropolis acceptance in FP32 (product form of the
                          * amplitude ratios); with mixed_check the FP64
                          * estimator is rerun on the same samples */
    int fp64_space;      /* FP64 MinSR: system solved.  0 or NQS_GPU_SPACE_SAMPLES = the
                          * N_s x N_s sample-space system in the upstream order (the
                          * parity default); NQS_GPU_SPACE_PARAMETERS = the N_p x N_p
                          * parameter-space system (O_c^T O_c / N_s + shift I) delta =
                          * O_c^T eps / N_s, the same delta by the push-through identity;
                          * NQS_GPU_SPACE_SMALLER = parameters when N_p < N_s.  A failed
                          * parameter-space factorisation is retried once with the shift
                          * raised by 1e-6, then delta = 0 and converged = 0 */
    int mlp_simt;        /* MIXED, MLP ansatz: 1 = the second layer of the local energies'
                          * connected configurations as SIMT GEMVs; 0 (default) = on the
                          * tensor cores (tcgen05 TF32, three hi / lo passes, FP32 accumulate) */
} nqs_gpu_options_t;

/* Defaults: compat sampler, single flips, open lattices, FP64. */
nqs_gpu_options_t nqs_gpu_options_default(void);
/* Process-wide options read by nqs_sampler_create and every step call. */
int nqs_gpu_set_options(const nqs_gpu_options_t *opts);
int nqs_gpu_get_options(nqs_gpu_options_t *opts);

/* Sampler with explicit options (upstream nqs_sampler_create + options). */
nqs_sampler_t *nqs_sampler_create_gpu(int num_sites, const nqs_config_t *cfg,
                                      const nqs_gpu_options_t *opts,
                                      nqs_log_amp_fn_t log_amp, void *log_amp_user);
/* Number of chains the sampler runs. */
int nqs_sampler_num_chains(const nqs_sampler_t *s);

/* ---- learned proposal ---------------------------------------------------
 * A masked autoregressive MLP q(s) (MADE: 2 hidden layers, BF16 weights, FP32
 * accumulation) trained online by Adam on every batch the sampler produces
 * (maximum likelihood of the chains' own samples).  A move is a draw from q
 * with probability `mix` (an independent proposal accepted with
 * min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s')))), else the sampler's local move;
 * the mixture keeps |psi|^2 invariant.  When the learned proposals' acceptance
 * on a batch falls below `min_acceptance` the next batches use local moves only,
 * with a probe every 8 batches.  With a fixed magnetisation (n_down >= 0 and
 * exchange moves) q is normalised over that sector.  Needs Philox chains, the
 * MIXED precision mode with fp32_estimator = 1 and an RBM / cRBM program. */
typedef struct {
    int hidden;               /* width of both hidden layers: multiple of 32, <= 128 (64) */
    int train_iters;          /* Adam iterations per produced batch (1) */
    int train_batch;          /* samples of each batch it trains on, 0 = all (1024) */
    double mix;               /* probability that a move is a learned proposal (0.5) */
    double learning_rate;     /* Adam step (3e-3) */
    double min_acceptance;    /* fallback threshold (0.01) */
    unsigned long long seed;  /* weight initialisation and proposal streams */
} nqs_gpu_made_options_t;

typedef struct {
    double proposals;         /* learned proposals made so far */
    double accepted;          /* of which accepted */
    double nll;               /* mean negative log-likelihood of the last trained batch */
    int active;               /* 0 while the fallback (local moves only) is in force */
    int train_steps;          /* Adam steps taken */
} nqs_gpu_made_stats_t;

nqs_gpu_made_options_t nqs_gpu_made_options_default(void);
/* Attach (opts != NULL) or remove (NULL) the learned proposal of a sampler. */
int nqs_sampler_set_learned_proposal(nqs_sampler_t *s, const nqs_gpu_made_options_t *opts);
int nqs_sampler_learned_stats(const nqs_sampler_t *s, nqs_gpu_made_stats_t *out);
/* Diagnostics of the attached model: parameter count, FP32 master weights in
 * the layout W1t[N][H], b1[H], W2t[H][H], b2[H], W3t[H][N], b3[N] (transposed
 * weights; masked entries read 0 and are forced to 0 on set), log q of
 * configurations, the mean NLL gradient of a batch (masked), and draws from q. */
long nqs_gpu_made_num_params(const nqs_sampler_t *s);
int nqs_gpu_made_get_weights(const nqs_sampler_t *s, float *out);
int nqs_gpu_made_set_weights(nqs_sampler_t *s, const float *in);
int nqs_gpu_made_log_prob(const nqs_sampler_t *s, const int *spins, int batch, double *out_logq);
int nqs_gpu_made_nll_grad(nqs_sampler_t *s, const int *spins, int batch, float *out_grad, double *out_nll);
int nqs_gpu_made_sample(nqs_sampler_t *s, int count, int *out_spins, double *out_logq);

/* ---- batches of independent problems -------------------------------------
 * `count` independent VMC problems (each its own Hamiltonian, lattice, ansatz
 * and sampler; sizes may differ) advanced together: nqs_gpu_batch_step runs one
 * MinSR step of every instance.  Precision: the MIXED mode with the FP32
 * estimator; each sampler must be a Philox sampler created in that mode and
 * each program an RBM / cRBM (with Marshall layers) of the instance's ansatz.
 * The refinement sweeps, Gram passes and solve space are taken from the process
 * options at creation.  The factor / inverse / refinement of all instances run
 * in ONE cooperative launch whose CTAs are split between the instances by an
 * autotuner on the first step, which also picks the factor's tile shape (the
 * diagonal block width, 64 or 128, by instance order) (nqs_gpu_batch_ctas reports
 * the split, nqs_gpu_batch_block_widths the widths, nqs_gpu_batch_tune_ms the
 * candidates' times: every CTA split for each width rule); from the second step the whole
 * batch step is one CUDA graph replayed per step.  An instance whose FP32
 * factor breaks down is solved again in FP64 on the same samples after the
 * graph (as nqs_sr_step_minsr_full does in the MIXED mode);
 * nqs_gpu_batch_fallbacks counts those instance steps.
 * The samplers advance as in nqs_sampler_batch, with their learned proposal
 * when one is attached (pool draws, training and fallback are replayable from
 * the graph).  infos (optional) receives count step infos. */
typedef struct {
    const nqs_config_t *cfg;      /* Hamiltonian, couplings, num_samples, shift, learning rate */
    int size_x, size_y;           /* lattice */
    nqs_ansatz_t *ansatz;
    nqs_sampler_t *sampler;
    nqs_log_amp_fn_t log_amp;     /* NULL: nqs_ansatz_log_amp of the ansatz */
    void *log_amp_user;
} nqs_gpu_instance_t;
typedef struct nqs_gpu_batch nqs_gpu_batch_t;
nqs_gpu_batch_t *nqs_gpu_batch_create(const nqs_gpu_instance_t *instances, int count);
int nqs_gpu_batch_step(nqs_gpu_batch_t *b, nqs_sr_step_info_t *infos);
int nqs_gpu_batch_ctas(const nqs_gpu_batch_t *b, int *out_ctas);
int nqs_gpu_batch_tune_ms(const nqs_gpu_batch_t *b, double *out_ms, int cap);
/* The factor's diagonal block width (64 or 128) the autotuner chose for each instance. */
int nqs_gpu_batch_block_widths(const nqs_gpu_batch_t *b, int *out_bd);
long nqs_gpu_batch_fallbacks(const nqs_gpu_batch_t *b);
void nqs_gpu_batch_free(nqs_gpu_batch_t *b);

/* Human-readable reason of the last failure on this thread ("" if none). */
const char *nqs_gpu_last_error(void);
/* Device name and SM count of the device in use; 0 on success. */
int nqs_gpu_device_info(char *name, int name_len, int *sm_count);
/* The cudaStream_t every kernel of this library is launched on. */
void *nqs_gpu_stream(void);
int nqs_gpu_synchronize(void);

/* Batched entry points on caller-supplied configurations (host int +-1,
 * row-major [B][N]).  0 on success, -1 on failure. */
int nqs_gpu_log_amp_batch(nqs_log_amp_fn_t log_amp, void *user,
                          const int *spins, int batch, int num_sites,
                          double *out_log_abs, double *out_arg);
int nqs_gpu_local_energy_batch(const nqs_config_t *cfg, int size_x, int size_y,
                               const int *spins, int batch,
                               nqs_log_amp_fn_t log_amp, void *user,
                               double *out_re, double *out_im);
/* O[b][k] = d log|psi| / d theta_k (complex_out = 0) or the holomorphic pair
 * (complex_out = 1, out_im used) for the base ansatz, or the symmetry-
 * projected gradient when gradient_fn = nqs_symproj_gradient. */
int nqs_gpu_gradient_batch(nqs_ansatz_t *a, nqs_gradient_fn_t gradient_fn,
                           void *grad_user, const int *spins, int batch,
                           int complex_out, double *out_re, double *out_im);

/* One SR step on a caller-supplied batch (no sampling): the parity entry
 * points.  `minsr` = 1 runs MinSR, 0 runs CG-SR, 2 holomorphic SR, 5 holomorphic
 * MinSR (for 2 and 5 gradient_fn, when set, is the holomorphic gradient:
 * nqs_symproj_gradient_complex).  Optional outputs: out_energies[batch],
 * out_delta[num_params]. */
int nqs_gpu_sr_step_batch(const nqs_config_t *cfg, int size_x, int size_y,
                          nqs_ansatz_t *ansatz,
                          nqs_log_amp_fn_t log_amp_fn, void *log_amp_user,
                          nqs_gradient_fn_t gradient_fn, void *grad_user,
                          const int *batch, int num_samples, int minsr,
                          nqs_sr_step_info_t *out_info,
                          double *out_energies, double *out_delta);

/* Holomorphic MinSR (no upstream counterpart): the linear system of the upstream
 * holomorphic SR step (nqs_sr_step_holomorphic_full, src/nqs/nqs_optimizer.c:415-524:
 * G = 2 Re[<O* O> - <O*><O>] + shift I, F = 2 Re[<O* E_loc> - <O*><E_loc>], theta -= lr delta)
 * solved by MinSR instead of CG.  With O = R + i I for the real parameters,
 * G = (2 / N_s)(R_c^T R_c + I_c^T I_c) + shift I and F = (2 / N_s)(R_c^T e_re + I_c^T e_im),
 * which is the MinSR system of the stacked real matrix [R_c; I_c] (2 N_s rows) and the
 * stacked centred energies [e_re; e_im] with the shift divided by 4; the update equals the
 * converged holomorphic CG-SR update on the same samples.  It optimises complex ansaetze
 * (complex RBM, the complex-output MLP) through both the phase and the modulus, where the
 * upstream MinSR (real parts only) drops the phase.  Precision and solve space follow
 * the process options (FP64: fp64_space; MIXED: tensor-core Gram of the stacked rows).
 * grad_fn: NULL (the base ansatz's holomorphic gradient) or nqs_symproj_gradient_complex. */
int nqs_sr_step_minsr_holomorphic_full(const nqs_config_t *cfg, int size_x, int size_y,
                                       nqs_ansatz_t *ansatz, nqs_sampler_t *sampler,
                                       nqs_log_amp_fn_t log_amp_fn, void *log_amp_user,
                                       nqs_holomorphic_gradient_fn_t grad_fn, void *grad_user,
                                       nqs_sr_step_info_t *out_info);
/* cfg->num_iterations steps after thermalising the sampler; out_energy_trace (optional)
 * receives each step's mean energy, as nqs_sr_run_minsr. */
int nqs_sr_run_minsr_holomorphic(const nqs_config_t *cfg, int size_x, int size_y,
                                 nqs_ansatz_t *ansatz, nqs_sampler_t *sampler,
                                 nqs_log_amp_fn_t log_amp_fn, void *log_amp_user,
                                 double *out_energy_trace);

/* The excited-state SR step (nqs_sr_step_excited) and the Euler tVMC step
 * (nqs_tvmc_step_real_time) on a caller-supplied batch: the parity entry points. */
int nqs_gpu_sr_step_batch_excited(const nqs_config_t *cfg, int size_x, int size_y,
                                  nqs_ansatz_t *ansatz,
                                  nqs_log_amp_fn_t log_amp_fn, void *log_amp_user,
                                  nqs_log_amp_fn_t ref_log_amp_fn, void *ref_log_amp_user,
                                  double penalty_mu, const int *batch, int num_samples,
                                  nqs_sr_step_info_t *out_info,
                                  double *out_energies, double *out_delta);
int nqs_gpu_tvmc_step_batch(const nqs_config_t *cfg, double dt, int size_x, int size_y,
                            nqs_ansatz_t *ansatz,
                            nqs_log_amp_fn_t log_amp_fn, void *log_amp_user,
                            const int *batch, int num_samples,
                            nqs_sr_step_info_t *out_info,
                            double *out_energies, double *out_delta);

/* MinSR solve that allocates no device memory.  It has no counterpart in the
 * upstream library.
 *
 * For callers that cannot call cudaMalloc: a host framework that has reserved
 * (pre-allocated) the device memory for its own pool, so that an allocation
 * made by a plug-in fails or fragments that pool, or a latency-critical loop
 * that must stay out of the driver's allocator.  The caller passes device
 * buffers: the Jacobian d_O [num_samples][num_params] (FP64, row-major, not
 * centred, only read), the local energies d_E [num_samples] and the output
 * d_delta [num_params].  The routine centres O, forms T = O_c O_c^T / N_s +
 * diag_shift I, factors it (FP64 Cholesky), solves (T) y = E - <E> and writes
 * delta = O_c^T y / N_s, the same arithmetic as the MinSR step.  A failed
 * factorisation gives delta = 0 and out_info->converged = 0 (the upstream
 * +1e-6 retry would need a second N_s x N_s copy and is not run here).
 * out_info (host, optional) receives <E>, Var(E), ||delta|| (update_norm,
 * without a learning rate) and converged.  Runs on `stream` (a cudaStream_t;
 * NULL = the legacy default stream) and returns after the result is ready.
 *
 * Limits: num_samples <= 1024 and num_params <= 16384; larger sizes are
 * rejected with -1 and a message in nqs_gpu_last_error().  All scratch
 * (the 1024 x 1024 Gram matrix, vectors, status words: about 8.5 MB) is one
 * statically sized device array that every GPU which loads this library's
 * device code keeps until the process exits.  With CUDA's lazy module loading
 * (the default) that code, and the array with it, is loaded onto a device the
 * first time this routine runs there, not when the library is loaded: a caller
 * that reserves the rest of the device memory for its own pool should make one
 * warm-up call first (or set CUDA_MODULE_LOADING=EAGER), so the array is
 * already in place when the pool takes the remainder.  The first call on a
 * device (and the first after a cudaDeviceReset, which gives the device a new
 * context and a new copy of the array) looks up that array's device address
 * (cudaGetSymbolAddress) with the device current.  Every call blocks the host
 * until its result is ready (it synchronises `stream` and copies the status and
 * info to host memory), so it is never called on a stream that is being captured
 * into a graph.  Every call reuses the same array and it keeps the last
 * call's contents, so calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller. */
int nqs_gpu_minsr_solve_noalloc(const double *d_O, const double *d_E,
                                int num_samples, long num_params, double diag_shift,
                                double *d_delta, nqs_sr_step_info_t *out_info,
                                void *stream);

/* Diagnostic: the tensor-core (tcgen05, TF32) Gram used by the MIXED MinSR
 * path, alone.  O_host [num_samples][num_params] FP64 is taken as already
 * centred; T_out [num_samples][num_samples] receives the lower triangle of
 * scale * (hi hi^T) (passes = 1) or scale * (hi hi^T + hi lo^T + lo hi^T)
 * (passes = 3) where O = hi + lo is split into two TF32 words. */
int nqs_gpu_gram_tc(const double *O_host, int num_samples, long num_params, int passes,
                    double scale, float *T_out);

/* Diagnostic: the SR step's effective-sample-size estimator on a host series
 * `energies` laid out as the sampler writes a batch (sample k of chain c at
 * row k * num_chains + c).  tau = 1 + 2 sum_{t=1}^{M} rho(t), rho pooled over
 * the chains, M the smallest window with M >= 5 tau(M) (Sokal); ESS =
 * (complete rows x num_chains) / tau.  Fewer than two samples per chain give
 * tau = 1. */
int nqs_gpu_ess(const double *energies, int num_samples, int num_chains, double *out_tau, double *out_ess);

/* Test hook: the number of polls a grid-wide barrier of the cooperative solve kernels
 * (mixed MinSR factor / refinement, CG-SR, batches) waits before it gives up; 0 restores
 * the default (2^24).  A barrier that gives up raises the kernel's error word, every CTA
 * leaves at its next barrier (releasing its tensor memory), and the step returns -1 with
 * "grid barrier timed out" in nqs_gpu_last_error(); the next call starts from cleared
 * barrier and error words. */
int nqs_gpu_set_barrier_budget(unsigned polls);

/* Statistics of the last SR step on this thread. */
typedef struct {
    double tau_int;          /* integrated autocorrelation time of E_loc (see nqs_gpu_ess) */
    double ess;              /* effective sample size of the step's batch */
    double refine_residual;  /* MIXED: relative residual after refinement */
    int    refine_sweeps;    /* CG iterations used */
    int    chol_retry;       /* 1 if the +1e-6 retry ran */
    int    chol_fail_col;    /* first failing column or -1 */
    int    gpu_launches;     /* kernels launched by the step */
    double delta_rel_err;    /* MIXED with mixed_check: ||d - d_fp64|| / ||d_fp64|| */
    int    mixed_fallback;   /* 1 if the FP32 factor failed and FP64 solved the step */
    int    pad_;
    /* MIXED: microseconds spent in the phases of the cooperative factor /
     * inverse / CG kernel (seen from CTA 0): [0] the first diagonal block; with the
     * pipelined factor (64-wide blocks, four CTAs or more) [1] CTA 0 waiting for the
     * other CTAs and [2] CTA 0's own chain of diagonal-block steps, otherwise [1] panels
     * and [2] trailing updates (each with the next diagonal block's update and factor by
     * CTA 0 beside the trailing tiles); [3] the last block row of L^{-1} (or the whole
     * inverse); [4] preconditioner applications, [5] right-hand side and operator
     * products, [6] total (the CG vector updates and dot products are the rest of it);
     * [7] the time CTA 0 spent on its diagonal-block steps (summed over the blocks) */
    double phase_us[8];
    /* MIXED with mixed_check and fp32_estimator: |<E> - <E>_fp64| / |<E>_fp64|
     * on the same samples (-1 when not measured) */
    double energy_rel_err;
} nqs_gpu_step_stats_t;
int nqs_gpu_last_step_stats(nqs_gpu_step_stats_t *out);

/* Per-kernel CUDA-event timing.  While enabled every launch is bracketed by
 * events on the library stream; nqs_gpu_profile_read() returns, for up to
 * `cap` kernels, their name, launch count and summed milliseconds. */
int nqs_gpu_profile_enable(int on);
int nqs_gpu_profile_reset(void);
int nqs_gpu_profile_read(int cap, char names[][48], int *counts, double *ms);
/* Kernels launched by this library since the last nqs_gpu_profile_reset(). */
long nqs_gpu_launch_count(void);

/* CUDA events on the library stream, for timing from the host:
 * nqs_gpu_event_record() creates and records one; nqs_gpu_event_elapsed_ms()
 * waits for `end` and returns the milliseconds between the two. */
void *nqs_gpu_event_record(void);
double nqs_gpu_event_elapsed_ms(void *start, void *end);
void nqs_gpu_event_destroy(void *event);

#ifdef __cplusplus
}
#endif

#endif /* NQS_GPU_H */
