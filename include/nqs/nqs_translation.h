/*
 * include/nqs/nqs_translation.h -- translation-symmetric projection of a square / chain
 * lattice ansatz (drop-in for upstream include/nqs/nqs_translation.h).
 *
 * psi_T(s) = |G|^{-1/2} sum_{(tx,ty)} psi(T_(tx,ty) s), G = size_x size_y, evaluated on the
 * device as the symmetry-projection program with the square translation table
 * (perm[g][x*Ly + y] = ((x+tx) mod Lx) * Ly + (y+ty) mod Ly, g = tx*Ly + ty, characters 1),
 * the same sums as upstream src/nqs/nqs_translation.c:23-145.
 */
#ifndef NQS_TRANSLATION_H
#define NQS_TRANSLATION_H

#include "nqs_sampler.h"
#include "nqs_ansatz.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Upstream wrapper struct. */
typedef struct {
    nqs_log_amp_fn_t base_log_amp;
    void            *base_user;
    int              size_x;
    int              size_y;   /* 1 for chains */
} nqs_translation_wrapper_t;

/* Replaces upstream nqs_translation_log_amp (src/nqs/nqs_translation.c:23-75). */
void nqs_translation_log_amp(const int *spins, int num_sites,
                              void *user,
                              double *out_log_abs,
                              double *out_arg);

/* Replaces upstream nqs_translation_gradient (src/nqs/nqs_translation.c:77-145). */
int nqs_translation_gradient(void *grad_user,
                              nqs_ansatz_t *ansatz,
                              const int *spins, int num_sites,
                              double *out_grad);

#ifdef __cplusplus
}
#endif

#endif /* NQS_TRANSLATION_H */
