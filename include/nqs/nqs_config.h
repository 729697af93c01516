/*
 * include/nqs/nqs_config.h -- run configuration of the NQS VMC step.
 *
 * Drop-in for upstream include/nqs/nqs_config.h (tsotchke/spin_based_neural_network
 * v0.5.0).  The enums and nqs_config_t keep the upstream values and the
 * upstream field order byte for byte (upstream :25-120) so that a caller's
 * struct can be passed unchanged; nqs_config_defaults() returns the upstream
 * defaults (upstream :123-152).  GPU-only knobs live in nqs_gpu_options_t
 * (nqs_gpu.h) so this layout never changes.
 */
#ifndef NQS_CONFIG_H
#define NQS_CONFIG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Ansatz families (upstream :25-45).  Implemented on the GPU: LEGACY_MLP (the
 * mean-field product state), RBM, COMPLEX_RBM, and the GPU-only deep MLP
 * NQS_GPU_ANSATZ_MLP declared in nqs_gpu.h. */
typedef enum {
    NQS_ANSATZ_LEGACY_MLP   = 0,
    NQS_ANSATZ_VIT          = 1,
    NQS_ANSATZ_FACTORED_VIT = 2,
    NQS_ANSATZ_AUTOREGRESSIVE = 3,
    NQS_ANSATZ_KAN          = 4,
    NQS_ANSATZ_RBM          = 5,
    NQS_ANSATZ_COMPLEX_RBM  = 6,
    NQS_ANSATZ_FACTORED_VIT_COMPLEX = 7
} nqs_ansatz_kind_t;

/* Symmetry flags (upstream :48-55). */
typedef enum {
    NQS_SYM_NONE             = 0,
    NQS_SYM_TRANSLATION      = 1 << 0,
    NQS_SYM_SPIN_FLIP        = 1 << 1,
    NQS_SYM_U1               = 1 << 2,
    NQS_SYM_POINT_GROUP      = 1 << 3,
    NQS_SYM_SU2              = 1 << 4
} nqs_symmetry_flags_t;

/* Hamiltonians (upstream :58-79).  Implemented on the GPU: TFIM, HEISENBERG,
 * J1_J2, XXZ, KAGOME_HEISENBERG.  The Kitaev kinds are not part of this build
 * and make the local-energy entry points fail (see nqs_gpu_last_error()). */
typedef enum {
    NQS_HAM_TFIM             = 0,
    NQS_HAM_HEISENBERG       = 1,
    NQS_HAM_J1_J2            = 2,
    NQS_HAM_KITAEV_HONEYCOMB = 3,
    NQS_HAM_XXZ              = 4,
    NQS_HAM_KITAEV_HEISENBERG = 5,
    NQS_HAM_KAGOME_HEISENBERG = 6
} nqs_hamiltonian_kind_t;

typedef struct {
    /* Ansatz */
    nqs_ansatz_kind_t    ansatz;
    int                   patch_size;
    int                   depth;             /* deep-MLP hidden layers */
    int                   width;             /* deep-MLP hidden width */
    int                   heads;
    int                   rbm_hidden_units;  /* M; 0 selects 2*N */
    double                rbm_init_scale;
    nqs_symmetry_flags_t  symmetries;

    /* Hamiltonian */
    nqs_hamiltonian_kind_t hamiltonian;
    double                 j_coupling;       /* J (J1; XXZ: Jxy) */
    double                 j2_coupling;      /* J2 of J1-J2 */
    double                 j_z_coupling;     /* Jz of XXZ */
    double                 transverse_field; /* Gamma of TFIM */
    double                 kh_K;
    double                 kh_J;
    int                    kagome_pbc;

    /* Sampling */
    int     num_samples;
    int     num_thermalize;
    int     num_decorrelate;
    int     cluster_moves;
    unsigned rng_seed;

    /* Optimisation */
    int     num_iterations;
    double  learning_rate;
    double  sr_diag_shift;
    int     sr_cg_max_iters;
    double  sr_cg_tol;
} nqs_config_t;

static inline nqs_config_t nqs_config_defaults(void) {
    nqs_config_t c;
    c.ansatz            = NQS_ANSATZ_LEGACY_MLP;
    c.patch_size        = 1;
    c.depth             = 3;
    c.width             = 128;
    c.heads             = 4;
    c.rbm_hidden_units  = 0;
    c.rbm_init_scale    = 0.01;
    c.symmetries        = (nqs_symmetry_flags_t)(NQS_SYM_SPIN_FLIP | NQS_SYM_TRANSLATION);
    c.hamiltonian       = NQS_HAM_TFIM;
    c.j_coupling        = 1.0;
    c.j2_coupling       = 0.0;
    c.j_z_coupling      = 1.0;
    c.transverse_field  = 1.0;
    c.kh_K              = 1.0;
    c.kh_J              = 0.0;
    c.kagome_pbc        = 1;
    c.num_samples       = 1024;
    c.num_thermalize    = 256;
    c.num_decorrelate   = 4;
    c.cluster_moves     = 0;
    c.rng_seed          = 0xC0FFEEu;
    c.num_iterations    = 200;
    c.learning_rate     = 1e-2;
    c.sr_diag_shift     = 1e-3;
    c.sr_cg_max_iters   = 100;
    c.sr_cg_tol         = 1e-6;
    return c;
}

#ifdef __cplusplus
}
#endif

#endif /* NQS_CONFIG_H */
