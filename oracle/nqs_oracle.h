/*
 * oracle/nqs_oracle.h -- CPU FP64 restatement of the NQS VMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is loaded by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline and
 * reference legs.  The product (libnqs_gb300.so) never links, loads or calls
 * it.  Every function names the upstream file:line it restates (paths are
 * relative to the upstream project root of tsotchke/spin_based_neural_network
 * v0.5.0).  Extensions that the upstream project does not have (periodic
 * square lattices, exchange moves, the deep MLP, multi-chain Philox sampling,
 * sector Lanczos) are written from their published definitions and say so.
 *
 * Conventions shared with the product:
 *   spins are int32 +-1, site index x*size_y + y (src/nqs/nqs_gradient.c:15-17),
 *   kagome site 3*(cx*Ly+cy)+sub (src/nqs/nqs_gradient.c:389),
 *   basis bit = 1 <-> spin -1 (src/nqs/nqs_lanczos.c:16-20).
 */
#ifndef NQS_ORACLE_H
#define NQS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Ansatz kinds: upstream values (include/nqs/nqs_config.h:25-45) + the deep MLP
 * extension (value 100, same as the product's NQS_GPU_ANSATZ_MLP). */
enum { OR_MF = 0, OR_VIT = 2, OR_RBM = 5, OR_CRBM = 6, OR_VITC = 7, OR_MLP = 100 };
/* Hamiltonian kinds: upstream values (include/nqs/nqs_config.h:58-79). */
enum { OR_TFIM = 0, OR_HEIS = 1, OR_J1J2 = 2, OR_XXZ = 4, OR_KAGOME = 6 };

typedef struct {
    int kind;        /* OR_* ansatz kind */
    int N;           /* sites */
    int M;           /* hidden units (RBM/cRBM) or hidden width (MLP) */
    int depth;       /* MLP hidden layers (only 2 supported) */
    const double *params;
} or_ansatz_t;

/* Wrapper layers, outermost first (mirrors the product's amplitude program). */
enum { OR_LAYER_MARSHALL = 1, OR_LAYER_SYMPROJ = 2 };
typedef struct {
    int type;
    int size_x, size_y;           /* Marshall */
    int G;                        /* symproj */
    const int *perm;              /* [G*N] */
    const double *chars;          /* [G] */
} or_layer_t;

typedef struct {
    or_ansatz_t base;
    int n_layers;
    or_layer_t layers[4];
} or_amp_t;

typedef struct {
    int ham;                 /* OR_* Hamiltonian */
    int size_x, size_y;      /* lattice (kagome: cells) */
    int pbc;                 /* square/chain PBC (extension); kagome uses kagome_pbc */
    int kagome_pbc;
    double J, J2, Jz, Gamma;
} or_ham_t;

long oracle_num_params(int kind, int N, int M);
/* Parameter initialisation, src/nqs/nqs_ansatz.c:65-252 (MF/RBM/cRBM) and the
 * MLP extension (Xavier-normal weights, zero biases). */
int oracle_ansatz_init(int kind, int N, int M, double scale, unsigned seed,
                       double *params);

void oracle_log_amp_batch(const or_amp_t *amp, const int *spins, int B,
                          double *out_la, double *out_arg);
/* Real-projected gradient (nqs_ansatz_logpsi_gradient, src/nqs/nqs_ansatz.c:997). */
int oracle_gradient_batch(const or_ansatz_t *a, const int *spins, int B, double *out);
/* Holomorphic gradient (src/nqs/nqs_ansatz.c:1258-1273). */
int oracle_gradient_complex_batch(const or_ansatz_t *a, const int *spins, int B,
                                  double *out_re, double *out_im);
/* Symmetry-projected gradient (src/nqs/nqs_symproj.c:82-155); the layer list of
 * `amp` must hold exactly one symproj layer (optionally with Marshall layers
 * beneath it, which only shift arg). */
int oracle_symproj_gradient_batch(const or_amp_t *amp, const int *spins, int B,
                                  double *out);
int oracle_marshall_parity(const int *spins, int size_x, int size_y);

/* Local energies, src/nqs/nqs_gradient.c:447-491 (real) and :495-892 (complex). */
void oracle_local_energy_batch(const or_ham_t *h, const or_amp_t *amp,
                               const int *spins, int B, double *out_re,
                               double *out_im /* may be NULL: real path */);
int oracle_num_sites(const or_ham_t *h);
/* Bond list used by the exchange move and the Heisenberg-type kernels.  Returns
 * the number of (u,v) pairs written to `bonds` (capacity `cap`). */
int oracle_bonds(const or_ham_t *h, int *bonds, int cap);

/* Square / chain nearest-neighbour bonds and J1-J2 diagonal bonds. */
int square_bonds_public(int Lx, int Ly, int pbc, int *bd);
int diag_bonds_public(int Lx, int Ly, int pbc, int *bd);

/* Upstream single-chain xorshift64 sampler, src/nqs/nqs_sampler.c:24-157.
 * Runs `n_therm` proposals, then `n` samples `n_decor` proposals apart. */
typedef struct {
    uint64_t rng;
    long accepted, proposed;
} or_xs_state_t;
int oracle_xorshift_sampler(const or_amp_t *amp, int N, unsigned seed,
                            int n_therm, int n_decor, int n, int *out,
                            double *out_acceptance);

/* Multi-chain Philox sampler (extension; the product's chain algorithm). */
typedef struct {
    uint64_t seed;
    int num_chains;
    int move;            /* 0 single flip, 1 nearest-neighbour exchange */
    int n_down;          /* >= 0: start in the sector with this many down spins */
} or_chain_opts_t;
void oracle_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
int oracle_chain_init(const or_chain_opts_t *o, int N, uint64_t *spins_bits);
/* Advance every chain by `moves` proposals starting at move counter
 * `move_base`; records a sample every `decor` moves after `skip` moves.
 * Samples are stored time-major: sample k of chain c at row k*C + c. */
int oracle_chain_run(const or_chain_opts_t *o, const or_amp_t *amp, const or_ham_t *h,
                     uint64_t *spins_bits, uint64_t *move_counter, int skip,
                     int n_samples_per_chain, int decor, int *out,
                     long *accepted, long *proposed);

/* Per-step SR solvers on a given batch, restating the upstream solvers with
 * the sampler replaced by the supplied batch:
 *   MinSR  src/nqs/nqs_optimizer.c:1063-1194
 *   CG-SR  src/nqs/nqs_optimizer.c:141-241 (qgt_apply :44-80, cg_solve :84-139) */
typedef struct {
    double mean_energy, variance_energy, update_norm;
    int cg_iterations, converged;
} or_step_info_t;
int oracle_minsr_step(const or_ham_t *h, const or_amp_t *amp, int grad_mode,
                      const int *batch, int Ns, double shift, double lr,
                      double *params_inout, long P, double *out_energies,
                      double *out_delta, or_step_info_t *info);
int oracle_cgsr_step(const or_ham_t *h, const or_amp_t *amp, int grad_mode,
                     const int *batch, int Ns, double shift, double lr,
                     int max_iters, double tol, double *params_inout, long P,
                     double *out_energies, double *out_delta, or_step_info_t *info);
/* Holomorphic SR, src/nqs/nqs_optimizer.c:415-524 (qgt_complex_apply :317-356,
 * cg_solve_complex :358-401): complex local energies, complex gradient of the
 * base ansatz, F = 2 [(R^T E_re + I^T E_im) / N_s - <R> <E_re> - <I> <E_im>],
 * CG on G v = 2 [(R^T R v + I^T I v) / N_s - <R> <R.v> - <I> <I.v>] + eps v. */
int oracle_holo_step(const or_ham_t *h, const or_amp_t *amp, const int *batch, int Ns,
                     double shift, double lr, int max_iters, double tol,
                     double *params_inout, long P, double *out_energies,
                     double *out_delta, or_step_info_t *info);

/* Complex symmetry-projected gradient (src/nqs/nqs_symproj.c:157-261) of the amplitude's
 * symproj layer: rows of Re and Im. */
int oracle_symproj_gradient_complex_batch(const or_amp_t *amp, const int *spins, int B,
                                          double *out_re, double *out_im);
/* Holomorphic SR with the gradient from the symproj layer (grad_sym = 1,
 * nqs_symproj_gradient_complex as the holomorphic gradient callback) or the base ansatz
 * (grad_sym = 0, as oracle_holo_step). */
int oracle_holo_step_grad(const or_ham_t *h, const or_amp_t *amp, int grad_sym, const int *batch, int Ns,
                          double shift, double lr, int max_iters, double tol, double *params_inout, long P,
                          double *out_energies, double *out_delta, or_step_info_t *info);

/* Excited-state SR, src/nqs/nqs_optimizer.c:562-723: the holomorphic step with
 * E_loc += mu r conj(<r>), r = psi_ref / psi (log-modulus difference clamped to +-10), the
 * force's means <E_re> + mu |<r>|^2 and <E_im> + mu (<r_im><r_re> - <r_re><r_im>); the
 * step info reports the physical energy; out_E the augmented local energies. */
int oracle_excited_step(const or_ham_t *h, const or_amp_t *amp, const or_amp_t *ref, double mu,
                        const int *batch, int Ns, double shift, double lr, int max_iters, double tol,
                        double *params_inout, long P, double *out_energies, double *out_delta,
                        or_step_info_t *info);
/* Real-time tVMC, forward Euler, src/nqs/nqs_optimizer.c:888-993: F_k = 2 [(R^T E_im -
 * I^T E_re) / N_s - <R><E_im> + <I><E_re>], CG on the holomorphic QGT, theta += dt delta. */
int oracle_tvmc_step(const or_ham_t *h, const or_amp_t *amp, const int *batch, int Ns, double shift,
                     double dt, int max_iters, double tol, double *params_inout, long P,
                     double *out_energies, double *out_delta, or_step_info_t *info);

/* Exact ground-state energy by Lanczos with full re-orthogonalisation (the
 * upstream src/mps/lanczos.c:119-303 scheme) over either the full 2^N basis
 * (n_down < 0) or the fixed-magnetisation sector with n_down down spins
 * (extension: sector basis ranked by the combinatorial number system). */
int oracle_exact_energy(const or_ham_t *h, int n_down, int max_iters, double tol,
                        double *out_e0);

/* ---- exact diagonalisation (oracle_ed.c) ---------------------------------------- */
#define OR_LZ_MAX 512
typedef struct {
    int iterations, converged;
    double residual;
    double alpha[OR_LZ_MAX], beta[OR_LZ_MAX + 1];
} or_lanczos_info_t;

/* Kagome Heisenberg H x over the full 2^N basis, src/nqs/nqs_lanczos.c:380-432. */
void oracle_kagome_heis_matvec(int Lx, int Ly, double J, int pbc, const double *in, double *out);
/* The same for the states s0 <= s < s1 only (out indexed by s). */
void oracle_kagome_heis_matvec_range(int Lx, int Ly, double J, int pbc, const double *in, double *out,
                                     long s0, long s1);
/* psi <- (1/G) sum_g chi(g) T(g) psi, bit i of T(g)'s source = bit perm[g][i],
 * src/nqs/nqs_symproj.c:786-852 (direct gather form). */
void oracle_sector_project(double *psi, int N, int G, const int *perm, const double *chars);
/* Out-of-place projector for the states s0 <= s < s1 (out[s - s0]). */
void oracle_sector_project_range(const double *psi, double *out, int N, int G, const int *perm,
                                 const double *chars, long s0, long s1);
/* The lean Lanczos seed before projection, src/mps/lanczos.c:864-880. */
void oracle_lanczos_seed(int N, int alternate, double *out);
/* Memory-lean projecting Lanczos for the kagome Heisenberg sector E_0, src/mps/lanczos.c:824-960,
 * with the eigenvector replay of :972-1119 when out_vec is not NULL.  N <= 24. */
int oracle_lanczos_lean_kagome(int Lx, int Ly, double J, int pbc, const int *perm, const double *chars, int G,
                               int max_iters, double tol, double *out_e, double *out_vec, or_lanczos_info_t *info);

/* The NQS state on the full basis (2^N doubles, N <= 24), src/nqs/nqs_lanczos.c:65-106. */
int oracle_materialise(const or_amp_t *amp, int N, double *psi);
/* Open square lattice H x: kind 0 TFIM (X = Gamma), 1 XXZ (X = Jz), src/nqs/nqs_lanczos.c:151-281. */
void oracle_square_matvec(int kind, int Lx, int Ly, double J, double X, const double *in, double *out);
/* Variational energy of the materialised state: ham 0 TFIM, 1 XXZ, 6 kagome Heisenberg,
 * src/nqs/nqs_lanczos.c:188-224, 283-321, 434-455. */
int oracle_variational_energy(const or_amp_t *amp, int ham, int Lx, int Ly, double J, double X, int pbc,
                              double *out_e);

#ifdef __cplusplus
}
#endif
#endif
