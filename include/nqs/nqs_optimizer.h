/*
 * include/nqs/nqs_optimizer.h -- stochastic reconfiguration (CG-SR, MinSR).
 *
 * Drop-in for upstream include/nqs/nqs_optimizer.h:35-323 (real-projected SR
 * and MinSR).  One step = sample -> local energies -> Jacobian O_k -> solve
 * -> parameter update, all on the GPU; only the step info and the parameter
 * mirror come back to the host.  The upstream semantics are kept: real-
 * projected gradients for complex ansatze, the real local energy, variance
 * <E^2> - <E>^2, update_norm = ||delta|| * lr, the one-shot +1e-6 Cholesky
 * retry and delta = 0 on a second failure.
 */
#ifndef NQS_OPTIMIZER_H
#define NQS_OPTIMIZER_H

#include "nqs_config.h"
#include "nqs_ansatz.h"
#include "nqs_sampler.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-step diagnostics, upstream include/nqs/nqs_optimizer.h:35-42. */
typedef struct {
    double mean_energy;
    double variance_energy;
    double update_norm;
    double acceptance_ratio;
    int    cg_iterations;
    int    converged;
} nqs_sr_step_info_t;

/* Replaces upstream nqs_sr_step (include/nqs/nqs_optimizer.h:47). */
int nqs_sr_step(const nqs_config_t *cfg,
                int size_x, int size_y,
                nqs_ansatz_t *ansatz,
                nqs_sampler_t *sampler,
                nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run (include/nqs/nqs_optimizer.h:58). */
int nqs_sr_run(const nqs_config_t *cfg,
               int size_x, int size_y,
               nqs_ansatz_t *ansatz,
               nqs_sampler_t *sampler,
               double *out_energy_trace);

/* Upstream gradient callback (include/nqs/nqs_optimizer.h:69-72).  Accepted
 * values: NULL (base ansatz gradient) or nqs_symproj_gradient with its
 * nqs_symproj_wrapper_t; anything else fails the step. */
typedef int (*nqs_gradient_fn_t)(void *grad_user,
                                  nqs_ansatz_t *ansatz,
                                  const int *spins, int num_sites,
                                  double *out_grad);

/* Replaces upstream nqs_sr_step_custom (include/nqs/nqs_optimizer.h:78). */
int nqs_sr_step_custom(const nqs_config_t *cfg,
                       int size_x, int size_y,
                       nqs_ansatz_t *ansatz,
                       nqs_sampler_t *sampler,
                       nqs_log_amp_fn_t log_amp_fn,
                       void *log_amp_user,
                       nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run_custom (include/nqs/nqs_optimizer.h:86). */
int nqs_sr_run_custom(const nqs_config_t *cfg,
                      int size_x, int size_y,
                      nqs_ansatz_t *ansatz,
                      nqs_sampler_t *sampler,
                      nqs_log_amp_fn_t log_amp_fn,
                      void *log_amp_user,
                      double *out_energy_trace);

/* Replaces upstream nqs_sr_step_custom_full (include/nqs/nqs_optimizer.h:97):
 * CG-SR with the matrix-free QGT product. */
int nqs_sr_step_custom_full(const nqs_config_t *cfg,
                             int size_x, int size_y,
                             nqs_ansatz_t *ansatz,
                             nqs_sampler_t *sampler,
                             nqs_log_amp_fn_t log_amp_fn,
                             void *log_amp_user,
                             nqs_gradient_fn_t gradient_fn,
                             void *grad_user,
                             nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run_custom_full (include/nqs/nqs_optimizer.h:107). */
int nqs_sr_run_custom_full(const nqs_config_t *cfg,
                            int size_x, int size_y,
                            nqs_ansatz_t *ansatz,
                            nqs_sampler_t *sampler,
                            nqs_log_amp_fn_t log_amp_fn,
                            void *log_amp_user,
                            nqs_gradient_fn_t gradient_fn,
                            void *grad_user,
                            double *out_energy_trace);

/* Replaces upstream nqs_sr_step_minsr_full (include/nqs/nqs_optimizer.h:307):
 * MinSR through the N_s x N_s sample-space Gram matrix. */
int nqs_sr_step_minsr_full(const nqs_config_t *cfg,
                            int size_x, int size_y,
                            nqs_ansatz_t *ansatz,
                            nqs_sampler_t *sampler,
                            nqs_log_amp_fn_t log_amp_fn,
                            void *log_amp_user,
                            nqs_gradient_fn_t gradient_fn,
                            void *grad_user,
                            nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run_minsr (include/nqs/nqs_optimizer.h:317). */
int nqs_sr_run_minsr(const nqs_config_t *cfg,
                      int size_x, int size_y,
                      nqs_ansatz_t *ansatz,
                      nqs_sampler_t *sampler,
                      nqs_log_amp_fn_t log_amp_fn,
                      void *log_amp_user,
                      double *out_energy_trace);

/* Holomorphic-gradient callback (upstream include/nqs/nqs_optimizer.h:155-159).
 * The GPU step accepts NULL only (the base ansatz's complex gradient). */
typedef int (*nqs_holomorphic_gradient_fn_t)(void *grad_user,
                                              nqs_ansatz_t *ansatz,
                                              const int *spins, int num_sites,
                                              double *out_re,
                                              double *out_im);

/* Replaces upstream nqs_sr_step_holomorphic (include/nqs/nqs_optimizer.h:135):
 * CG on the complex QGT G = 2 Re{<O* O> - <O*><O>} with complex local energies. */
int nqs_sr_step_holomorphic(const nqs_config_t *cfg,
                             int size_x, int size_y,
                             nqs_ansatz_t *ansatz,
                             nqs_sampler_t *sampler,
                             nqs_log_amp_fn_t log_amp_fn,
                             void *log_amp_user,
                             nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run_holomorphic (include/nqs/nqs_optimizer.h:143). */
int nqs_sr_run_holomorphic(const nqs_config_t *cfg,
                            int size_x, int size_y,
                            nqs_ansatz_t *ansatz,
                            nqs_sampler_t *sampler,
                            nqs_log_amp_fn_t log_amp_fn,
                            void *log_amp_user,
                            double *out_energy_trace);

/* Replaces upstream nqs_sr_step_holomorphic_full (include/nqs/nqs_optimizer.h:168). */
int nqs_sr_step_holomorphic_full(const nqs_config_t *cfg,
                                  int size_x, int size_y,
                                  nqs_ansatz_t *ansatz,
                                  nqs_sampler_t *sampler,
                                  nqs_log_amp_fn_t log_amp_fn,
                                  void *log_amp_user,
                                  nqs_holomorphic_gradient_fn_t grad_fn,
                                  void *grad_user,
                                  nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run_holomorphic_full (include/nqs/nqs_optimizer.h:178). */
int nqs_sr_run_holomorphic_full(const nqs_config_t *cfg,
                                 int size_x, int size_y,
                                 nqs_ansatz_t *ansatz,
                                 nqs_sampler_t *sampler,
                                 nqs_log_amp_fn_t log_amp_fn,
                                 void *log_amp_user,
                                 nqs_holomorphic_gradient_fn_t grad_fn,
                                 void *grad_user,
                                 double *out_energy_trace);

/* Replaces upstream nqs_tvmc_step_real_time (include/nqs/nqs_optimizer.h:206-212;
 * src/nqs/nqs_optimizer.c:888-993): Re(S) delta = Im(F) with
 * F_k = 2 [Cov(R_k, E_im) - Cov(I_k, E_re)] on the holomorphic metric, CG as in
 * nqs_sr_step_holomorphic, theta += dt delta (forward Euler).  update_norm uses |dt|. */
int nqs_tvmc_step_real_time(const nqs_config_t *cfg, double dt,
                             int size_x, int size_y,
                             nqs_ansatz_t *ansatz,
                             nqs_sampler_t *sampler,
                             nqs_log_amp_fn_t log_amp_fn,
                             void *log_amp_user,
                             nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_step_excited (include/nqs/nqs_optimizer.h:242-251;
 * src/nqs/nqs_optimizer.c:562-723): holomorphic SR with the local energies augmented by
 * penalty_mu r(s) conj(<r>), r = psi_ref / psi (log-modulus difference clamped to +-10);
 * mean_energy reports the physical energy. */
int nqs_sr_step_excited(const nqs_config_t *cfg,
                         int size_x, int size_y,
                         nqs_ansatz_t *ansatz,
                         nqs_sampler_t *sampler,
                         nqs_log_amp_fn_t log_amp_fn,
                         void *log_amp_user,
                         nqs_log_amp_fn_t ref_log_amp_fn,
                         void *ref_log_amp_user,
                         double penalty_mu,
                         nqs_sr_step_info_t *out_info);

/* Replaces upstream nqs_sr_run_excited (include/nqs/nqs_optimizer.h:253-262). */
int nqs_sr_run_excited(const nqs_config_t *cfg,
                        int size_x, int size_y,
                        nqs_ansatz_t *ansatz,
                        nqs_sampler_t *sampler,
                        nqs_log_amp_fn_t log_amp_fn,
                        void *log_amp_user,
                        nqs_log_amp_fn_t ref_log_amp_fn,
                        void *ref_log_amp_user,
                        double penalty_mu,
                        double *out_energy_trace);

/* Replaces upstream nqs_tvmc_step_heun (include/nqs/nqs_optimizer.h:267-273;
 * src/nqs/nqs_optimizer.c:815-886): k1 = delta(theta), k2 = delta(theta + dt k1) from a
 * second sampling, theta += dt (k1 + k2) / 2; mean / variance from the first evaluation,
 * cg_iterations summed, converged if both solves converged. */
int nqs_tvmc_step_heun(const nqs_config_t *cfg, double dt,
                        int size_x, int size_y,
                        nqs_ansatz_t *ansatz,
                        nqs_sampler_t *sampler,
                        nqs_log_amp_fn_t log_amp_fn,
                        void *log_amp_user,
                        nqs_sr_step_info_t *out_info);

#ifdef __cplusplus
}
#endif

#endif /* NQS_OPTIMIZER_H */
