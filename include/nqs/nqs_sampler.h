/*
 * include/nqs/nqs_sampler.h -- Metropolis sampler over spin configurations.
 *
 * Drop-in for upstream include/nqs/nqs_sampler.h:20-75.  With the default
 * GPU options the sampler reproduces the upstream single-chain xorshift64
 * Markov chain sample for sample (one warp runs the chain with incremental
 * theta updates).  With nqs_gpu_options_t.rng = NQS_GPU_RNG_PHILOX the same
 * handle runs thousands of chains, one warp each, with Philox4x32-10 and
 * single-flip or nearest-neighbour exchange moves (nqs_gpu.h).
 */
#ifndef NQS_SAMPLER_H
#define NQS_SAMPLER_H

#include <stddef.h>
#include "nqs_config.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nqs_sampler nqs_sampler_t;

/* Upstream callback type (include/nqs/nqs_sampler.h:35-37).  The GPU entry
 * points accept the callbacks this library exports (nqs_ansatz_log_amp,
 * nqs_marshall_log_amp, nqs_symproj_log_amp) and compile them, with their
 * user structs, into a device amplitude program.  Any other callback is
 * rejected (the call fails and nqs_gpu_last_error() says why): host code is
 * never called per configuration. */
typedef void (*nqs_log_amp_fn_t)(const int *spins, int num_sites,
                                 void *user,
                                 double *out_re, double *out_im);

/* Replaces upstream nqs_sampler_create (include/nqs/nqs_sampler.h:42). */
nqs_sampler_t *nqs_sampler_create(int num_sites,
                                  const nqs_config_t *cfg,
                                  nqs_log_amp_fn_t log_amp,
                                  void *log_amp_user);

/* Replaces upstream nqs_sampler_free (include/nqs/nqs_sampler.h:47). */
void nqs_sampler_free(nqs_sampler_t *s);

/* Replaces upstream nqs_sampler_thermalize (include/nqs/nqs_sampler.h:51):
 * cfg->num_thermalize proposals on every chain. */
void nqs_sampler_thermalize(nqs_sampler_t *s);

/* Replaces upstream nqs_sampler_next (include/nqs/nqs_sampler.h:56): advances
 * chain 0 by cfg->num_decorrelate proposals; the pointer is owned by the
 * sampler and valid until the next call. */
const int *nqs_sampler_next(nqs_sampler_t *s);

/* Replaces upstream nqs_sampler_batch (include/nqs/nqs_sampler.h:61):
 * n configurations into out[n * num_sites].  With C chains, row k*C + c is
 * the k-th sample of chain c.  0 on success. */
int nqs_sampler_batch(nqs_sampler_t *s, int n, int *out);

/* Replaces upstream nqs_sampler_acceptance_ratio (include/nqs/nqs_sampler.h:64). */
double nqs_sampler_acceptance_ratio(const nqs_sampler_t *s);

/* Replaces upstream nqs_sampler_current (include/nqs/nqs_sampler.h:67): the
 * current configuration of chain 0. */
const int *nqs_sampler_current(const nqs_sampler_t *s);

/* Replaces upstream nqs_sampler_num_sites (include/nqs/nqs_sampler.h:75). */
int nqs_sampler_num_sites(const nqs_sampler_t *s);

#ifdef __cplusplus
}
#endif

#endif /* NQS_SAMPLER_H */
