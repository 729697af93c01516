/*
 * include/nqs/nqs_marshall.h -- Marshall sign rule wrapper.
 *
 * Drop-in for upstream include/nqs/nqs_marshall.h:35-52.  On the GPU the
 * wrapper becomes a popcount of (down spins & sublattice-A mask) fused into
 * the amplitude program.
 */
#ifndef NQS_MARSHALL_H
#define NQS_MARSHALL_H

#include "nqs_sampler.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Upstream wrapper struct, include/nqs/nqs_marshall.h:35-40. */
typedef struct {
    nqs_log_amp_fn_t base_log_amp;
    void            *base_user;
    int              size_x;
    int              size_y;
} nqs_marshall_wrapper_t;

/* Replaces upstream nqs_marshall_parity (include/nqs/nqs_marshall.h:45):
 * parity of the number of down spins on sublattice A ((x + y) even). */
int nqs_marshall_parity(const int *spins, int size_x, int size_y);

/* Replaces upstream nqs_marshall_log_amp (include/nqs/nqs_marshall.h:49). */
void nqs_marshall_log_amp(const int *spins, int num_sites,
                           void *user,
                           double *out_log_abs,
                           double *out_arg);

#ifdef __cplusplus
}
#endif

#endif /* NQS_MARSHALL_H */
