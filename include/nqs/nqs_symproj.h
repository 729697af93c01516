/*
 * include/nqs/nqs_symproj.h -- finite-group symmetry projection wrapper.
 *
 * Drop-in for upstream include/nqs/nqs_symproj.h:39-120.  On the GPU the
 * permutation table is staged in device memory once per wrapper and the G
 * permuted configurations are produced as bit permutations inside the
 * amplitude program.
 */
#ifndef NQS_SYMPROJ_H
#define NQS_SYMPROJ_H

#include "nqs_sampler.h"
#include "nqs_ansatz.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Upstream wrapper struct, include/nqs/nqs_symproj.h:39-47. */
typedef struct {
    nqs_log_amp_fn_t base_log_amp;
    void            *base_user;
    int              num_sites;
    int              num_group_elements;
    const int       *perm;               /* [|G| * N], perm[g*N+i] = pi_g(i) */
    const double    *characters;         /* [|G|] */
} nqs_symproj_wrapper_t;

/* Replaces upstream nqs_symproj_log_amp (include/nqs/nqs_symproj.h:49). */
void nqs_symproj_log_amp(const int *spins, int num_sites,
                         void *user,
                         double *out_log_abs, double *out_arg);

/* Replaces upstream nqs_symproj_gradient (include/nqs/nqs_symproj.h:55). */
int nqs_symproj_gradient(void *grad_user,
                         nqs_ansatz_t *ansatz,
                         const int *spins, int num_sites,
                         double *out_grad);

/* Replaces upstream nqs_kagome_translation_perm (include/nqs/nqs_symproj.h:92).
 * Host-side table builder; *out_perm is malloc'd, the caller frees it. */
int nqs_kagome_translation_perm(int Lx, int Ly,
                                int **out_perm,
                                int *out_num_elements);

/* Replaces upstream nqs_kagome_p2_perm (include/nqs/nqs_symproj.h:107). */
int nqs_kagome_p2_perm(int Lx, int Ly,
                        int **out_perm,
                        double **out_characters,
                        int *out_num_elements);

#ifdef __cplusplus
}
#endif

#endif /* NQS_SYMPROJ_H */
