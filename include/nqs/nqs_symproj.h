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

/* Replaces upstream nqs_symproj_gradient_complex (include/nqs/nqs_symproj.h:69;
 * src/nqs/nqs_symproj.c:157-261): the
 * holomorphic gradient of the projected amplitude, sum_g w_g d log psi_base(g s) / d theta
 * with complex weights w_g = chi_g psi_base(g s) / sum_g' chi_g' psi_base(g' s).  Usable as
 * the nqs_holomorphic_gradient_fn_t of nqs_sr_step_holomorphic_full with the wrapper as
 * grad_user.  Base ansatz: mean-field, RBM or complex RBM. */
int nqs_symproj_gradient_complex(void *grad_user,
                                  nqs_ansatz_t *ansatz,
                                  const int *spins, int num_sites,
                                  double *out_grad_re,
                                  double *out_grad_im);

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

/* Replaces upstream nqs_kagome_p3_perm (include/nqs/nqs_symproj.h:129-133,
 * src/nqs/nqs_symproj.c:436-523): |G| = 3 L^2, g = k L^2 + tx L + ty, the rotation by
 * 120 k degrees about the centroid of the up triangle of cell (0,0) followed by the
 * translation (tx, ty); characters 1. */
int nqs_kagome_p3_perm(int L,
                        int **out_perm,
                        double **out_characters,
                        int *out_num_elements);

/* Replaces upstream nqs_kagome_p6_perm (include/nqs/nqs_symproj.h:156-160,
 * src/nqs/nqs_symproj.c:525-590): |G| = 6 L^2, the rotation by 60 k degrees about the
 * hexagon centre (a1 + a2)/2 followed by the translation; characters 1. */
int nqs_kagome_p6_perm(int L,
                        int **out_perm,
                        double **out_characters,
                        int *out_num_elements);

/* Upstream nqs_symproj_kagome_irrep_t (include/nqs/nqs_symproj.h:193-200): the C_6v
 * irreps at Gamma.  For E_1 / E_2 the characters carry the factor d_E = 2. */
typedef enum {
    NQS_SYMPROJ_KAGOME_GAMMA_A1 = 0,
    NQS_SYMPROJ_KAGOME_GAMMA_A2 = 1,
    NQS_SYMPROJ_KAGOME_GAMMA_B1 = 2,
    NQS_SYMPROJ_KAGOME_GAMMA_B2 = 3,
    NQS_SYMPROJ_KAGOME_GAMMA_E1 = 4,
    NQS_SYMPROJ_KAGOME_GAMMA_E2 = 5
} nqs_symproj_kagome_irrep_t;

/* Replaces upstream nqs_kagome_p6m_perm_irrep (include/nqs/nqs_symproj.h:225-229,
 * src/nqs/nqs_symproj.c:738-776): the |G| = 12 L^2 p6m table of the L x L kagome torus,
 * g = op * L^2 + tx * L + ty, op 0..5 = rotation by 60 op degrees about a hexagon
 * centre, op 6..11 = the horizontal mirror after that rotation; characters = the
 * C_6v character of op for the named irrep (translations carry +1 at Gamma).
 * Built in exact integer half-lattice coordinates.  Host only; caller frees both. */
int nqs_kagome_p6m_perm_irrep(int L,
                               nqs_symproj_kagome_irrep_t irrep_name,
                               int **out_perm,
                               double **out_characters,
                               int *out_num_elements);

/* Replaces upstream nqs_kagome_p6m_perm (include/nqs/nqs_symproj.h:178-181): A_1. */
int nqs_kagome_p6m_perm(int L,
                         int **out_perm,
                         double **out_characters,
                         int *out_num_elements);

/* Replaces upstream nqs_kagome_p6m_project_inplace (include/nqs/nqs_symproj.h:247-250,
 * src/nqs/nqs_symproj.c:786-852): psi <- (1/G) sum_g chi(g) T(g) psi on a host array of
 * 2^N doubles, computed on the device (copy in, project, copy out).  Failures leave psi
 * unchanged and set nqs_gpu_last_error. */
void nqs_kagome_p6m_project_inplace(double *psi, int N, int G,
                                     const int *perm,
                                     const double *characters);

#ifdef __cplusplus
}
#endif

#endif /* NQS_SYMPROJ_H */
