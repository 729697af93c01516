/*
 * include/nqs/nqs_ansatz.h -- wavefunction ansatz handle (GPU-resident).
 *
 * Drop-in for upstream include/nqs/nqs_ansatz.h:28-82.  The handle owns the
 * parameters in HBM plus a host mirror in the upstream layout; every entry
 * point keeps the upstream meaning, argument order and return codes.
 */
#ifndef NQS_ANSATZ_H
#define NQS_ANSATZ_H

#include <stddef.h>
#include "nqs_config.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nqs_ansatz nqs_ansatz_t;

/* Replaces upstream nqs_ansatz_create (include/nqs/nqs_ansatz.h:34).
 * Initial parameters equal the upstream ones for the same config (same
 * xorshift64 / Box-Muller stream).  NULL for kinds this build lacks, when no
 * CUDA device is usable, or on allocation failure. */
nqs_ansatz_t *nqs_ansatz_create(const nqs_config_t *cfg, int num_sites);

/* Replaces upstream nqs_ansatz_free (include/nqs/nqs_ansatz.h:36). */
void nqs_ansatz_free(nqs_ansatz_t *a);

/* Replaces upstream nqs_ansatz_num_params (include/nqs/nqs_ansatz.h:39). */
long nqs_ansatz_num_params(const nqs_ansatz_t *a);

/* Replaces upstream nqs_ansatz_log_amp (include/nqs/nqs_ansatz.h:43).  One
 * configuration, evaluated on the GPU.  Writes zeros on bad arguments, as
 * upstream does.  Passing this function as an nqs_log_amp_fn_t to the
 * sampler / local-energy / SR entry points selects the fused device program;
 * the scalar call itself exists for drop-in callers. */
void nqs_ansatz_log_amp(const int *spins, int num_sites,
                        void *ansatz_user,
                        double *out_log_abs,
                        double *out_arg);

/* Replaces upstream nqs_ansatz_logpsi_gradient (include/nqs/nqs_ansatz.h:57):
 * d log|psi| / d theta (real projection for complex ansatze). 0 on success. */
int nqs_ansatz_logpsi_gradient(nqs_ansatz_t *a,
                               const int *spins, int num_sites,
                               double *out_grad);

/* Replaces upstream nqs_ansatz_logpsi_gradient_complex
 * (include/nqs/nqs_ansatz.h:65): Re and Im of d log psi / d theta. */
int nqs_ansatz_logpsi_gradient_complex(nqs_ansatz_t *a,
                                        const int *spins, int num_sites,
                                        double *out_re, double *out_im);

/* Replaces upstream nqs_ansatz_is_complex (include/nqs/nqs_ansatz.h:72). */
int nqs_ansatz_is_complex(const nqs_ansatz_t *a);

/* Replaces upstream nqs_ansatz_apply_update (include/nqs/nqs_ansatz.h:76):
 * params <- params + step * delta. */
int nqs_ansatz_apply_update(nqs_ansatz_t *a,
                            const double *delta, double step);

/* Replaces upstream nqs_ansatz_params_raw (include/nqs/nqs_ansatz.h:82).
 * Returns the host mirror.  Writes through this pointer are seen by the next
 * call into the library (the mirror is compared with the device copy at
 * every entry point and re-uploaded when it differs). */
double *nqs_ansatz_params_raw(nqs_ansatz_t *a);

#ifdef __cplusplus
}
#endif

#endif /* NQS_ANSATZ_H */
