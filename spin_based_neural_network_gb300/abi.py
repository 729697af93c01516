"""ctypes mirrors of the C structs in include/nqs/*.h.

The layouts are those of the upstream C11 headers (upstream
include/nqs/nqs_config.h:82-120, include/nqs/nqs_optimizer.h:35-42,
include/nqs/nqs_marshall.h:35-40, include/nqs/nqs_symproj.h:39-47) so that one
struct instance can be handed both to this library and to any other build of
the same API.  Importing this module loads no shared library.
"""
import ctypes as C

# nqs_ansatz_kind_t (upstream include/nqs/nqs_config.h:25-45) + GPU extension
ANSATZ_LEGACY_MLP = 0
ANSATZ_RBM = 5
ANSATZ_COMPLEX_RBM = 6
ANSATZ_FACTORED_VIT = 2       # factored-attention ViT, real amplitude
ANSATZ_FACTORED_VIT_COMPLEX = 7
ANSATZ_GPU_MLP = 100          # 2-hidden-layer tanh MLP with a complex head (extension)

# nqs_hamiltonian_kind_t (upstream include/nqs/nqs_config.h:58-79)
HAM_TFIM = 0
HAM_HEISENBERG = 1
HAM_J1_J2 = 2
HAM_XXZ = 4
HAM_KAGOME_HEISENBERG = 6

SYM_SPIN_FLIP = 1 << 1
SYM_TRANSLATION = 1 << 0


class NqsConfig(C.Structure):
    _fields_ = [
        ("ansatz", C.c_int), ("patch_size", C.c_int), ("depth", C.c_int),
        ("width", C.c_int), ("heads", C.c_int), ("rbm_hidden_units", C.c_int),
        ("rbm_init_scale", C.c_double), ("symmetries", C.c_int),
        ("hamiltonian", C.c_int), ("j_coupling", C.c_double),
        ("j2_coupling", C.c_double), ("j_z_coupling", C.c_double),
        ("transverse_field", C.c_double), ("kh_K", C.c_double), ("kh_J", C.c_double),
        ("kagome_pbc", C.c_int), ("num_samples", C.c_int),
        ("num_thermalize", C.c_int), ("num_decorrelate", C.c_int),
        ("cluster_moves", C.c_int), ("rng_seed", C.c_uint),
        ("num_iterations", C.c_int), ("learning_rate", C.c_double),
        ("sr_diag_shift", C.c_double), ("sr_cg_max_iters", C.c_int),
        ("sr_cg_tol", C.c_double),
    ]


def config_defaults(**kw):
    """nqs_config_defaults() (upstream include/nqs/nqs_config.h:123-152)."""
    c = NqsConfig()
    c.ansatz = ANSATZ_LEGACY_MLP
    c.patch_size = 1
    c.depth = 3
    c.width = 128
    c.heads = 4
    c.rbm_hidden_units = 0
    c.rbm_init_scale = 0.01
    c.symmetries = SYM_SPIN_FLIP | SYM_TRANSLATION
    c.hamiltonian = HAM_TFIM
    c.j_coupling = 1.0
    c.j2_coupling = 0.0
    c.j_z_coupling = 1.0
    c.transverse_field = 1.0
    c.kh_K = 1.0
    c.kh_J = 0.0
    c.kagome_pbc = 1
    c.num_samples = 1024
    c.num_thermalize = 256
    c.num_decorrelate = 4
    c.cluster_moves = 0
    c.rng_seed = 0xC0FFEE
    c.num_iterations = 200
    c.learning_rate = 1e-2
    c.sr_diag_shift = 1e-3
    c.sr_cg_max_iters = 100
    c.sr_cg_tol = 1e-6
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError(k)
        setattr(c, k, v)
    return c


class StepInfo(C.Structure):
    """nqs_sr_step_info_t (upstream include/nqs/nqs_optimizer.h:35-42)."""
    _fields_ = [
        ("mean_energy", C.c_double), ("variance_energy", C.c_double),
        ("update_norm", C.c_double), ("acceptance_ratio", C.c_double),
        ("cg_iterations", C.c_int), ("converged", C.c_int),
    ]


LOG_AMP_FN = C.CFUNCTYPE(None, C.POINTER(C.c_int), C.c_int, C.c_void_p,
                         C.POINTER(C.c_double), C.POINTER(C.c_double))
GRAD_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_int,
                      C.POINTER(C.c_double))


class MarshallWrapper(C.Structure):
    """nqs_marshall_wrapper_t (upstream include/nqs/nqs_marshall.h:35-40)."""
    _fields_ = [("base_log_amp", C.c_void_p), ("base_user", C.c_void_p),
                ("size_x", C.c_int), ("size_y", C.c_int)]


class TranslationWrapper(C.Structure):
    """nqs_translation_wrapper_t (upstream include/nqs/nqs_translation.h)."""
    _fields_ = [("base_log_amp", C.c_void_p), ("base_user", C.c_void_p),
                ("size_x", C.c_int), ("size_y", C.c_int)]


class SymprojWrapper(C.Structure):
    """nqs_symproj_wrapper_t (upstream include/nqs/nqs_symproj.h:39-47)."""
    _fields_ = [("base_log_amp", C.c_void_p), ("base_user", C.c_void_p),
                ("num_sites", C.c_int), ("num_group_elements", C.c_int),
                ("perm", C.POINTER(C.c_int)), ("characters", C.POINTER(C.c_double))]


# GPU extension options (include/nqs/nqs_gpu.h, nqs_gpu_options_t)
MOVE_SINGLE_FLIP = 0
MOVE_EXCHANGE = 1
RNG_XORSHIFT_COMPAT = 0      # upstream single chain, bit-identical sequence
RNG_PHILOX = 1               # many chains, counter-based Philox4x32-10
PREC_FP64 = 0                # plain FP64 path
PREC_MIXED = 1               # tensor-core Gram + FP64 iterative refinement
SPACE_AUTO = 0               # mixed MinSR: solve the smaller of the two systems
SPACE_SAMPLES = 1            # N_s x N_s (O O^T)
SPACE_PARAMETERS = 2         # N_p x N_p (O^T O)
SPACE_SMALLER = 3            # fp64_space: whichever system is smaller


class GpuOptions(C.Structure):
    """nqs_gpu_options_t (include/nqs/nqs_gpu.h)."""
    _fields_ = [
        ("num_chains", C.c_int),
        ("rng", C.c_int),
        ("move", C.c_int),
        ("n_down", C.c_int),
        ("square_pbc", C.c_int),
        ("precision", C.c_int),
        ("refine_sweeps", C.c_int),
        ("gram_passes", C.c_int),
        ("mixed_space", C.c_int),
        ("lattice_x", C.c_int),
        ("lattice_y", C.c_int),
        ("lattice_kagome", C.c_int),
        ("mixed_check", C.c_int),
        ("fp32_estimator", C.c_int),
        ("fp64_space", C.c_int),
        ("mlp_simt", C.c_int),
    ]


class MadeOptions(C.Structure):
    """nqs_gpu_made_options_t (include/nqs/nqs_gpu.h)."""
    _fields_ = [("hidden", C.c_int), ("train_iters", C.c_int), ("train_batch", C.c_int), ("mix", C.c_double),
                ("learning_rate", C.c_double), ("min_acceptance", C.c_double), ("seed", C.c_ulonglong)]


class MadeStats(C.Structure):
    """nqs_gpu_made_stats_t (include/nqs/nqs_gpu.h)."""
    _fields_ = [("proposals", C.c_double), ("accepted", C.c_double), ("nll", C.c_double),
                ("active", C.c_int), ("train_steps", C.c_int)]


class Instance(C.Structure):
    """nqs_gpu_instance_t (include/nqs/nqs_gpu.h)."""
    _fields_ = [("cfg", C.POINTER(NqsConfig)), ("size_x", C.c_int), ("size_y", C.c_int), ("ansatz", C.c_void_p),
                ("sampler", C.c_void_p), ("log_amp", C.c_void_p), ("log_amp_user", C.c_void_p)]


class LanczosResult(C.Structure):
    """lanczos_result_t (include/nqs/nqs_lanczos.h; upstream include/mps/lanczos.h:37-42)."""
    _fields_ = [("eigenvalue", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("residual_norm", C.c_double)]
