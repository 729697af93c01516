/*
 * include/nqs/nqs_lanczos.h -- exact diagonalisation on the device.
 *
 * The memory-lean projecting Lanczos of the kagome Heisenberg model over the full
 * 2^N basis (N = 3 Lx Ly <= 30), with the symmetry-sector projector
 * (1/|G|) sum_g chi(g) T(g) applied to every Krylov vector.  Every vector lives in
 * HBM (four vectors of 2^N doubles, five with the eigenvector); the host keeps only
 * the tridiagonal coefficients.
 *
 * Upstream interfaces replaced (names, arguments and return codes are the same):
 *   nqs_lanczos_e0_kagome_heisenberg_projected_lean        include/nqs/nqs_lanczos.h:192-197
 *   nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec include/nqs/nqs_lanczos.h:202-208
 *   lanczos_result_t                                       include/mps/lanczos.h:37-42
 */
#ifndef NQS_LANCZOS_H
#define NQS_LANCZOS_H

#ifdef __cplusplus
extern "C" {
#endif

#ifndef NQS_LANCZOS_RESULT_DEFINED
#define NQS_LANCZOS_RESULT_DEFINED
typedef struct {
    double eigenvalue;       /* smallest Ritz value found */
    int    iterations;       /* Krylov steps used */
    int    converged;        /* 1 when the Ritz value moved by less than tol */
    double residual_norm;    /* |lambda_k - lambda_{k-1}| at exit */
} lanczos_result_t;
#endif

/* Replaces upstream nqs_lanczos_e0_kagome_heisenberg_projected_lean
 * (src/nqs/nqs_lanczos.c:629-647 over src/mps/lanczos.c:824-960).  Seed: the upstream
 * xorshift sequence from 0xA5A5A5A5A5A5A5A5 ^ 2^N (bit-identical), projected and
 * normalised; three-term recurrence with the projector after each matvec; stops when
 * beta < 1e-14 or, after step 5, when the lowest Ritz value moves by less than tol.
 * (perm, characters, G): the sector, perm[g*N + i] = site whose spin lands on site i.
 * Returns 0, or -1 on invalid arguments / device failure (nqs_gpu_last_error). */
int nqs_lanczos_e0_kagome_heisenberg_projected_lean(
    int Lx_cells, int Ly_cells, double J, int pbc,
    const int *perm, const double *characters, int G,
    int max_iters, double tol,
    double *out_eigenvalue,
    lanczos_result_t *out_result);

/* Replaces upstream nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec
 * (src/nqs/nqs_lanczos.c:651-672 over src/mps/lanczos.c:972-1119): the same first pass,
 * then the lowest eigenvector of the K x K tridiagonal and a replay of the recurrence
 * that accumulates the Ritz vector on the device.  out_eigenvector: host array of 2^N
 * doubles, unit norm (its overall sign is arbitrary, as upstream). */
int nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec(
    int Lx_cells, int Ly_cells, double J, int pbc,
    const int *perm, const double *characters, int G,
    int max_iters, double tol,
    double *out_eigenvalue,
    double *out_eigenvector,
    lanczos_result_t *out_result);

/* GB300 addition, the magnetisation-sector form of the lean projecting Lanczos that the
 * upstream sector drivers run over the library's building blocks
 * (scripts/research_kagome_sz_spatial.c:96-121, 196-240; scripts/research_kagome_spin_gap.c:
 * 22-36, 118-145).  Their projector first zeroes every amplitude whose number of down spins
 * (set bits) differs from `popcount`, then applies the spatial projection (perm, characters,
 * G; the identity group G = 1 for the Sz sector alone).  Here that filter runs inside every
 * matvec and projection pass, so states outside the sector are written as zero without being
 * evaluated (H and the permutations keep the popcount).  popcount = -1: no filter.
 * seed_state = 0: the seed of nqs_lanczos_e0_kagome_heisenberg_projected_lean; otherwise the
 * drivers' seed protocol: u_i - 1/2 from xorshift64 (13, 7, 17) started at seed_state,
 * projected and normalised, then handed to the lean Lanczos as its initial vector, which
 * projects and normalises it again (the drivers use 0xA5A5A5A5A5A5A5A5 ^ 2^N for the Sz
 * sectors and 0xC3C3C3C3C3C3C3C3 ^ 2^N ^ (irrep index * 0x9E3779B97F4A7C15) with a p6m
 * irrep).  out_eigenvector (host, 2^N doubles) may be NULL.  Returns 0 or -1. */
int nqs_gpu_lanczos_e0_kagome_sz_projected_lean(
    int Lx_cells, int Ly_cells, double J, int pbc,
    const int *perm, const double *characters, int G,
    int popcount, unsigned long long seed_state,
    int max_iters, double tol,
    double *out_eigenvalue,
    double *out_eigenvector,
    lanczos_result_t *out_result);

/* ---- device-resident building blocks (GB300 additions) ---------------------------
 * Pointers marked d_ are device pointers of 2^N doubles. */

/* y = H x for H = J sum_<ij> S_i.S_j on the kagome bonds of src/nqs/nqs_lanczos.c:380-432
 * (up triangles always, down triangles with PBC or away from the open edges). */
int nqs_gpu_kagome_heis_matvec(int Lx_cells, int Ly_cells, double J, int pbc,
                               const double *d_in, double *d_out);

/* d_out = (1/G) sum_g characters[g] T(g) d_in (d_out may equal d_in).  When the
 * characters are multiplicative on the group the sum runs as up to four passes over a
 * chain of subgroups and coset representatives (G = R1 H1, H1 = R2 H2, ...; |H_k| + sum
 * |R_k| gathers per state), else as one pass of |G| gathers. */
int nqs_gpu_sector_project(int N, int G, const int *perm, const double *characters,
                           const double *d_in, double *d_out);

/* The Lanczos seed before projection: d_out[i] = u_i - 1/2, u_i the (i+1)-th output of
 * xorshift64 (13, 7, 17) from 0xA5A5A5A5A5A5A5A5 ^ 2^N (alternate = 0) or from
 * 0xBEEFBABE ^ 2^N (alternate = 1), scaled by 2^-53 after >> 11. */
int nqs_gpu_lanczos_seed(int N, int alternate, double *d_out);

/* Tridiagonal coefficients of the last Lanczos run: alpha[0..K-1] and beta[0..K]
 * (beta[0] = 0); at most cap entries of alpha and cap + 1 of beta are written (beta holds
 * cap + 1 doubles).  Returns K. */
int nqs_gpu_lanczos_last_coeffs(int cap, double *alpha, double *beta);

/* Host-side plan of the sector projector (no device needed): *out_passes = 1 (direct) to
 * 4; sizes[0..passes-1] (4 ints) = elements per pass; elems (G ints) = the group indices
 * of pass 0, then pass 1, ...  Pass 0 sums over the innermost subgroup H_k, each later
 * pass over coset representatives of the previous group in the next larger one, so that
 * the product of the passes' sums runs over every g of G exactly once. */
int nqs_ed_projector_plan(int N, int G, const int *perm, const double *characters,
                          int *out_passes, int *sizes, int *elems);

#ifdef __cplusplus
}
#endif

#endif /* NQS_LANCZOS_H */
