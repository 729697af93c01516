"""Thin Python mirror of the C API in include/nqs/*.h.

Names, argument meaning and error behaviour follow the upstream C entry points
(upstream include/nqs/nqs_ansatz.h, nqs_sampler.h, nqs_gradient.h,
nqs_optimizer.h, nqs_marshall.h, nqs_symproj.h); every call goes straight to
libnqs_gb300.so.  Failures raise NqsError carrying nqs_gpu_last_error().
"""
import ctypes as C

import numpy as np

from . import abi, lib

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)
VP = C.c_void_p


class NqsError(RuntimeError):
    pass


def _declare(L):
    cfgp = C.POINTER(abi.NqsConfig)
    optp = C.POINTER(abi.GpuOptions)
    infop = C.POINTER(abi.StepInfo)
    sig = {
        "nqs_ansatz_create": (VP, [cfgp, C.c_int]),
        "nqs_ansatz_free": (None, [VP]),
        "nqs_ansatz_num_params": (C.c_long, [VP]),
        "nqs_ansatz_log_amp": (None, [IP, C.c_int, VP, DP, DP]),
        "nqs_ansatz_logpsi_gradient": (C.c_int, [VP, IP, C.c_int, DP]),
        "nqs_ansatz_logpsi_gradient_complex": (C.c_int, [VP, IP, C.c_int, DP, DP]),
        "nqs_ansatz_is_complex": (C.c_int, [VP]),
        "nqs_ansatz_apply_update": (C.c_int, [VP, DP, C.c_double]),
        "nqs_ansatz_params_raw": (DP, [VP]),
        "nqs_sampler_create": (VP, [C.c_int, cfgp, VP, VP]),
        "nqs_sampler_create_gpu": (VP, [C.c_int, cfgp, optp, VP, VP]),
        "nqs_sampler_free": (None, [VP]),
        "nqs_sampler_thermalize": (None, [VP]),
        "nqs_sampler_next": (IP, [VP]),
        "nqs_sampler_batch": (C.c_int, [VP, C.c_int, IP]),
        "nqs_sampler_acceptance_ratio": (C.c_double, [VP]),
        "nqs_sampler_current": (IP, [VP]),
        "nqs_sampler_num_sites": (C.c_int, [VP]),
        "nqs_sampler_num_chains": (C.c_int, [VP]),
        "nqs_local_energy": (C.c_double, [cfgp, C.c_int, C.c_int, IP, VP, VP]),
        "nqs_local_energy_batch": (None, [cfgp, C.c_int, C.c_int, IP, C.c_int, VP, VP, DP]),
        "nqs_local_energy_complex": (None, [cfgp, C.c_int, C.c_int, IP, VP, VP, DP, DP]),
        "nqs_local_energy_batch_complex": (None, [cfgp, C.c_int, C.c_int, IP, C.c_int, VP, VP, DP, DP]),
        "nqs_sr_step": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, infop]),
        "nqs_sr_run": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, DP]),
        "nqs_sr_step_custom": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, infop]),
        "nqs_sr_run_custom": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, DP]),
        "nqs_sr_step_custom_full": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, infop]),
        "nqs_sr_run_custom_full": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, DP]),
        "nqs_sr_step_holomorphic_full": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, infop]),
        "nqs_sr_run_holomorphic": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, DP]),
        "nqs_sr_step_excited": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, C.c_double, infop]),
        "nqs_sr_run_excited": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, C.c_double, DP]),
        "nqs_tvmc_step_real_time": (C.c_int, [cfgp, C.c_double, C.c_int, C.c_int, VP, VP, VP, VP, infop]),
        "nqs_tvmc_step_heun": (C.c_int, [cfgp, C.c_double, C.c_int, C.c_int, VP, VP, VP, VP, infop]),
        "nqs_gpu_sr_step_batch_excited": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, C.c_double, IP,
                                                    C.c_int, infop, DP, DP]),
        "nqs_gpu_tvmc_step_batch": (C.c_int, [cfgp, C.c_double, C.c_int, C.c_int, VP, VP, VP, IP, C.c_int, infop,
                                              DP, DP]),
        "nqs_sr_step_minsr_full": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, infop]),
        "nqs_sr_run_minsr": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, DP]),
        "nqs_gpu_set_barrier_budget": (C.c_int, [C.c_uint]),
        "nqs_sr_step_minsr_holomorphic_full": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP, infop]),
        "nqs_sr_run_minsr_holomorphic": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, DP]),
        "nqs_marshall_parity": (C.c_int, [IP, C.c_int, C.c_int]),
        "nqs_marshall_log_amp": (None, [IP, C.c_int, VP, DP, DP]),
        "nqs_symproj_log_amp": (None, [IP, C.c_int, VP, DP, DP]),
        "nqs_symproj_gradient": (C.c_int, [VP, VP, IP, C.c_int, DP]),
        "nqs_symproj_gradient_complex": (C.c_int, [VP, VP, IP, C.c_int, DP, DP]),
        "nqs_translation_log_amp": (None, [IP, C.c_int, VP, DP, DP]),
        "nqs_translation_gradient": (C.c_int, [VP, VP, IP, C.c_int, DP]),
        "nqs_kagome_p3_perm": (C.c_int, [C.c_int, C.POINTER(IP), C.POINTER(DP), IP]),
        "nqs_kagome_p6_perm": (C.c_int, [C.c_int, C.POINTER(IP), C.POINTER(DP), IP]),
        "nqs_kagome_translation_perm": (C.c_int, [C.c_int, C.c_int, C.POINTER(IP), IP]),
        "nqs_kagome_p2_perm": (C.c_int, [C.c_int, C.c_int, C.POINTER(IP), C.POINTER(DP), IP]),
        "nqs_kagome_p6m_perm_irrep": (C.c_int, [C.c_int, C.c_int, C.POINTER(IP), C.POINTER(DP), IP]),
        "nqs_kagome_p6m_project_inplace": (None, [DP, C.c_int, C.c_int, IP, DP]),
        "nqs_lanczos_e0_kagome_heisenberg_projected_lean": (
            C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, IP, DP, C.c_int, C.c_int, C.c_double, DP,
                      C.POINTER(abi.LanczosResult)]),
        "nqs_gpu_lanczos_e0_kagome_sz_projected_lean": (
            C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, IP, DP, C.c_int, C.c_int, C.c_ulonglong, C.c_int,
                      C.c_double, DP, DP, C.POINTER(abi.LanczosResult)]),
        "nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec": (
            C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, IP, DP, C.c_int, C.c_int, C.c_double, DP, DP,
                      C.POINTER(abi.LanczosResult)]),
        "nqs_gpu_kagome_heis_matvec": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, VP, VP]),
        "nqs_gpu_sector_project": (C.c_int, [C.c_int, C.c_int, IP, DP, VP, VP]),
        "nqs_gpu_lanczos_seed": (C.c_int, [C.c_int, C.c_int, VP]),
        "nqs_gpu_lanczos_last_coeffs": (C.c_int, [C.c_int, DP, DP]),
        "nqs_ed_projector_plan": (C.c_int, [C.c_int, C.c_int, IP, DP, IP, IP, IP]),
        "nqs_gpu_options_default": (abi.GpuOptions, []),
        "nqs_gpu_set_options": (C.c_int, [optp]),
        "nqs_gpu_get_options": (C.c_int, [optp]),
        "nqs_gpu_last_error": (C.c_char_p, []),
        "nqs_gpu_device_info": (C.c_int, [C.c_char_p, C.c_int, IP]),
        "nqs_gpu_stream": (VP, []),
        "nqs_gpu_synchronize": (C.c_int, []),
        "nqs_gpu_log_amp_batch": (C.c_int, [VP, VP, IP, C.c_int, C.c_int, DP, DP]),
        "nqs_gpu_local_energy_batch": (C.c_int, [cfgp, C.c_int, C.c_int, IP, C.c_int, VP, VP, DP, DP]),
        "nqs_gpu_gradient_batch": (C.c_int, [VP, VP, VP, IP, C.c_int, C.c_int, DP, DP]),
        "nqs_gpu_sr_step_batch": (C.c_int, [cfgp, C.c_int, C.c_int, VP, VP, VP, VP, VP, IP, C.c_int,
                                            C.c_int, infop, DP, DP]),
        "nqs_gpu_last_step_stats": (C.c_int, [VP]),
        "nqs_gpu_profile_enable": (C.c_int, [C.c_int]),
        "nqs_gpu_profile_reset": (C.c_int, []),
        "nqs_gpu_profile_read": (C.c_int, [C.c_int, VP, IP, DP]),
        "nqs_gpu_launch_count": (C.c_long, []),
        "nqs_gpu_event_record": (VP, []),
        "nqs_gpu_event_elapsed_ms": (C.c_double, [VP, VP]),
        "nqs_gpu_event_destroy": (None, [VP]),
        "nqs_gpu_minsr_solve_noalloc": (C.c_int, [VP, VP, C.c_int, C.c_long, C.c_double, VP, infop, VP]),
        "nqs_gpu_gram_tc": (C.c_int, [DP, C.c_int, C.c_long, C.c_int, C.c_double, C.POINTER(C.c_float)]),
        "nqs_gpu_ess": (C.c_int, [DP, C.c_int, C.c_int, DP, DP]),
        "nqs_gpu_batch_create": (C.c_void_p, [C.POINTER(abi.Instance), C.c_int]),
        "nqs_gpu_batch_step": (C.c_int, [C.c_void_p, C.POINTER(abi.StepInfo)]),
        "nqs_gpu_batch_ctas": (C.c_int, [C.c_void_p, IP]),
        "nqs_gpu_batch_tune_ms": (C.c_int, [C.c_void_p, DP, C.c_int]),
        "nqs_gpu_batch_block_widths": (C.c_int, [C.c_void_p, IP]),
        "nqs_gpu_batch_free": (None, [C.c_void_p]),
        "nqs_gpu_batch_fallbacks": (C.c_long, [C.c_void_p]),
        "nqs_gpu_made_options_default": (abi.MadeOptions, []),
        "nqs_sampler_set_learned_proposal": (C.c_int, [C.c_void_p, C.POINTER(abi.MadeOptions)]),
        "nqs_sampler_learned_stats": (C.c_int, [C.c_void_p, C.POINTER(abi.MadeStats)]),
        "nqs_gpu_made_num_params": (C.c_long, [C.c_void_p]),
        "nqs_gpu_made_get_weights": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "nqs_gpu_made_set_weights": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "nqs_gpu_made_log_prob": (C.c_int, [C.c_void_p, IP, C.c_int, DP]),
        "nqs_gpu_made_nll_grad": (C.c_int, [C.c_void_p, IP, C.c_int, C.POINTER(C.c_float), DP]),
        "nqs_gpu_made_sample": (C.c_int, [C.c_void_p, C.c_int, IP, DP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def fn(name):
    """Address of an exported amplitude / gradient callback (e.g.
    'nqs_ansatz_log_amp'), usable as an nqs_log_amp_fn_t argument."""
    return C.cast(getattr(lib(), name), C.c_void_p).value


def last_error():
    return lib().nqs_gpu_last_error().decode()


def _check(rc, what):
    if rc != 0:
        raise NqsError("%s failed: %s" % (what, last_error()))


def _ip(a):
    return a.ctypes.data_as(IP)


def _dp(a):
    return a.ctypes.data_as(DP)


def spins_array(spins, N=None):
    s = np.ascontiguousarray(spins, dtype=np.int32)
    if s.ndim == 1:
        s = s.reshape(1, -1)
    if N is not None and s.shape[1] != N:
        raise ValueError("expected %d sites, got %d" % (N, s.shape[1]))
    return s


def set_options(**kw):
    o = lib().nqs_gpu_options_default()
    for k, v in kw.items():
        setattr(o, k, v)
    _check(lib().nqs_gpu_set_options(C.byref(o)), "nqs_gpu_set_options")
    return o


def options(**kw):
    o = lib().nqs_gpu_options_default()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Ansatz:
    """nqs_ansatz_t (upstream include/nqs/nqs_ansatz.h:28-82)."""

    def __init__(self, cfg, num_sites):
        self.cfg = cfg
        self.h = lib().nqs_ansatz_create(C.byref(cfg), num_sites)
        if not self.h:
            raise NqsError("nqs_ansatz_create failed: " + last_error())
        self.N = num_sites
        self.P = lib().nqs_ansatz_num_params(self.h)

    def free(self):
        if self.h:
            lib().nqs_ansatz_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def params(self):
        """numpy view of the host mirror (nqs_ansatz_params_raw); writes are
        picked up by the next library call."""
        return np.ctypeslib.as_array(lib().nqs_ansatz_params_raw(self.h), shape=(self.P,))

    @property
    def user(self):
        return self.h

    log_amp_fn = property(lambda self: fn("nqs_ansatz_log_amp"))

    def is_complex(self):
        return bool(lib().nqs_ansatz_is_complex(self.h))

    def log_amp(self, spins):
        s = spins_array(spins, self.N)[0]
        la, ar = C.c_double(), C.c_double()
        lib().nqs_ansatz_log_amp(_ip(s), self.N, self.h, C.byref(la), C.byref(ar))
        return la.value, ar.value

    def gradient(self, spins, complex_out=False):
        s = spins_array(spins, self.N)
        B = s.shape[0]
        re = np.zeros((B, self.P))
        im = np.zeros((B, self.P)) if complex_out else None
        _check(lib().nqs_gpu_gradient_batch(self.h, None, None, _ip(s), B, int(complex_out), _dp(re),
                                            _dp(im) if complex_out else None), "gradient")
        return (re, im) if complex_out else re

    def apply_update(self, delta, step):
        d = np.ascontiguousarray(delta, dtype=np.float64)
        _check(lib().nqs_ansatz_apply_update(self.h, _dp(d), step), "nqs_ansatz_apply_update")


class Marshall:
    """nqs_marshall_wrapper_t around another program."""

    def __init__(self, base_fn, base_user, size_x, size_y):
        self.s = abi.MarshallWrapper(base_fn, base_user, size_x, size_y)
        self.log_amp_fn = fn("nqs_marshall_log_amp")

    @property
    def user(self):
        return C.addressof(self.s)


class Symproj:
    """nqs_symproj_wrapper_t; keeps the permutation and character arrays alive."""

    def __init__(self, base_fn, base_user, num_sites, perm, chars):
        self.perm = np.ascontiguousarray(perm, dtype=np.int32).ravel()
        self.chars = np.ascontiguousarray(chars, dtype=np.float64)
        self.s = abi.SymprojWrapper(base_fn, base_user, num_sites, len(self.chars), _ip(self.perm),
                                    _dp(self.chars))
        self.log_amp_fn = fn("nqs_symproj_log_amp")
        self.gradient_fn = fn("nqs_symproj_gradient")
        self.gradient_complex_fn = fn("nqs_symproj_gradient_complex")

    @property
    def user(self):
        return C.addressof(self.s)


class Translation:
    """nqs_translation_wrapper_t: the translation-symmetric projection of a square or chain
    lattice amplitude (upstream include/nqs/nqs_translation.h)."""

    def __init__(self, base_fn, base_user, size_x, size_y):
        self.s = abi.TranslationWrapper(base_fn, base_user, size_x, size_y)
        self.log_amp_fn = fn("nqs_translation_log_amp")
        self.gradient_fn = fn("nqs_translation_gradient")

    @property
    def user(self):
        return C.addressof(self.s)


P6M_IRREPS = {"A1": 0, "A2": 1, "B1": 2, "B2": 3, "E1": 4, "E2": 5}


def kagome_perm(Lx, Ly, group="p2", irrep="A1"):
    """(perm [G, N], characters [G]) of a kagome symmetry group: "p2", "translations", or
    on an L x L torus "p3", "p6", "p6m" (irrep one of A1 A2 B1 B2 E1 E2 for p6m)."""
    p = IP()
    G = C.c_int()
    if group in ("p3", "p6"):
        if Lx != Ly:
            raise NqsError(group + " needs an L x L torus")
        ch = DP()
        f = lib().nqs_kagome_p3_perm if group == "p3" else lib().nqs_kagome_p6_perm
        _check(f(Lx, C.byref(p), C.byref(ch), C.byref(G)), group + " perm")
        chars = np.ctypeslib.as_array(ch, shape=(G.value,)).copy()
    elif group == "p6m":
        if Lx != Ly:
            raise NqsError("p6m needs an L x L torus")
        ch = DP()
        _check(lib().nqs_kagome_p6m_perm_irrep(Lx, P6M_IRREPS[irrep], C.byref(p), C.byref(ch), C.byref(G)),
               "p6m perm")
        chars = np.ctypeslib.as_array(ch, shape=(G.value,)).copy()
    elif group == "p2":
        ch = DP()
        _check(lib().nqs_kagome_p2_perm(Lx, Ly, C.byref(p), C.byref(ch), C.byref(G)), "p2 perm")
        chars = np.ctypeslib.as_array(ch, shape=(G.value,)).copy()
    else:
        _check(lib().nqs_kagome_translation_perm(Lx, Ly, C.byref(p), C.byref(G)), "translation perm")
        chars = np.ones(G.value)
    N = 3 * Lx * Ly
    perm = np.ctypeslib.as_array(p, shape=(G.value * N,)).copy().reshape(G.value, N)
    return perm, chars


def log_amp_batch(log_amp_fn, user, spins):
    s = spins_array(spins)
    B, N = s.shape
    la, ar = np.zeros(B), np.zeros(B)
    _check(lib().nqs_gpu_log_amp_batch(log_amp_fn, user, _ip(s), B, N, _dp(la), _dp(ar)), "log_amp_batch")
    return la, ar


def local_energy_batch(cfg, size_x, size_y, spins, log_amp_fn, user, complex_out=False):
    s = spins_array(spins)
    B = s.shape[0]
    re, im = np.zeros(B), np.zeros(B)
    _check(lib().nqs_gpu_local_energy_batch(C.byref(cfg), size_x, size_y, _ip(s), B, log_amp_fn, user,
                                            _dp(re), _dp(im)), "local_energy_batch")
    return (re, im) if complex_out else re


def symproj_gradient_complex_batch(ansatz, sym, spins):
    """nqs_symproj_gradient_complex over a batch: (Re, Im) rows [B, P]."""
    s = spins_array(spins, ansatz.N)
    B = s.shape[0]
    re, im = np.zeros((B, ansatz.P)), np.zeros((B, ansatz.P))
    _check(lib().nqs_gpu_gradient_batch(ansatz.h, sym.gradient_complex_fn, sym.user, _ip(s), B, 1, _dp(re),
                                        _dp(im)), "symproj complex gradient")
    return re, im


def symproj_gradient_batch(ansatz, sym, spins):
    s = spins_array(spins, ansatz.N)
    B = s.shape[0]
    out = np.zeros((B, ansatz.P))
    _check(lib().nqs_gpu_gradient_batch(ansatz.h, sym.gradient_fn, sym.user, _ip(s), B, 0, _dp(out), None),
           "symproj gradient")
    return out


class Sampler:
    """nqs_sampler_t (upstream include/nqs/nqs_sampler.h:20-75)."""

    def __init__(self, num_sites, cfg, log_amp_fn, user, opts=None):
        self.cfg = cfg
        if opts is None:
            self.h = lib().nqs_sampler_create(num_sites, C.byref(cfg), log_amp_fn, user)
        else:
            self.h = lib().nqs_sampler_create_gpu(num_sites, C.byref(cfg), C.byref(opts), log_amp_fn, user)
        if not self.h:
            raise NqsError("nqs_sampler_create failed: " + last_error())
        self.N = num_sites

    def free(self):
        if self.h:
            lib().nqs_sampler_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def thermalize(self):
        lib().nqs_sampler_thermalize(self.h)

    def batch(self, n):
        out = np.zeros((n, self.N), dtype=np.int32)
        _check(lib().nqs_sampler_batch(self.h, n, _ip(out)), "nqs_sampler_batch")
        return out

    def next(self):
        p = lib().nqs_sampler_next(self.h)
        return np.ctypeslib.as_array(p, shape=(self.N,)).copy()

    def current(self):
        p = lib().nqs_sampler_current(self.h)
        return np.ctypeslib.as_array(p, shape=(self.N,)).copy()

    def acceptance_ratio(self):
        return lib().nqs_sampler_acceptance_ratio(self.h)

    @property
    def num_chains(self):
        return lib().nqs_sampler_num_chains(self.h)


def sr_step_minsr(cfg, size_x, size_y, ansatz, sampler, log_amp_fn=None, user=None, grad_fn=None,
                  grad_user=None):
    info = abi.StepInfo()
    _check(lib().nqs_sr_step_minsr_full(C.byref(cfg), size_x, size_y, ansatz.h, sampler.h, log_amp_fn, user,
                                        grad_fn, grad_user, C.byref(info)), "nqs_sr_step_minsr_full")
    return info


def sr_step_holomorphic(cfg, size_x, size_y, ansatz, sampler, log_amp_fn=None, user=None, grad_fn=None,
                        grad_user=None):
    """nqs_sr_step_holomorphic_full (upstream include/nqs/nqs_optimizer.h:168); grad_fn is
    NULL (the base ansatz's holomorphic gradient) or nqs_symproj_gradient_complex."""
    info = abi.StepInfo()
    _check(lib().nqs_sr_step_holomorphic_full(C.byref(cfg), size_x, size_y, ansatz.h, sampler.h, log_amp_fn, user,
                                              grad_fn, grad_user, C.byref(info)), "nqs_sr_step_holomorphic_full")
    return info


def sr_step_minsr_holomorphic(cfg, size_x, size_y, ansatz, sampler, log_amp_fn=None, user=None, grad_fn=None,
                              grad_user=None):
    """nqs_sr_step_minsr_holomorphic_full: the holomorphic SR system solved by MinSR."""
    info = abi.StepInfo()
    _check(lib().nqs_sr_step_minsr_holomorphic_full(C.byref(cfg), size_x, size_y, ansatz.h, sampler.h, log_amp_fn,
                                                    user, grad_fn, grad_user, C.byref(info)),
           "nqs_sr_step_minsr_holomorphic_full")
    return info


def sr_step_cg(cfg, size_x, size_y, ansatz, sampler, log_amp_fn=None, user=None, grad_fn=None,
               grad_user=None):
    info = abi.StepInfo()
    _check(lib().nqs_sr_step_custom_full(C.byref(cfg), size_x, size_y, ansatz.h, sampler.h, log_amp_fn, user,
                                         grad_fn, grad_user, C.byref(info)), "nqs_sr_step_custom_full")
    return info


def sr_step_batch(cfg, size_x, size_y, ansatz, batch, minsr=True, log_amp_fn=None, user=None, grad_fn=None,
                  grad_user=None):
    """One SR step on a caller-supplied batch; returns (info, energies, delta).
    minsr: True / 1 MinSR, False / 0 CG-SR, 2 holomorphic SR, 5 holomorphic MinSR."""
    s = spins_array(batch, ansatz.N)
    Ns = s.shape[0]
    E, d = np.zeros(Ns), np.zeros(ansatz.P)
    info = abi.StepInfo()
    _check(lib().nqs_gpu_sr_step_batch(C.byref(cfg), size_x, size_y, ansatz.h, log_amp_fn, user, grad_fn,
                                       grad_user, _ip(s), Ns, int(minsr), C.byref(info), _dp(E), _dp(d)),
           "nqs_gpu_sr_step_batch")
    return info, E, d


def sr_step_excited(cfg, size_x, size_y, ansatz, sampler, ref_log_amp_fn, ref_user, mu, log_amp_fn=None,
                    user=None):
    """nqs_sr_step_excited (upstream include/nqs/nqs_optimizer.h:242): holomorphic SR with
    the orthogonality penalty against the reference wavefunction."""
    info = abi.StepInfo()
    _check(lib().nqs_sr_step_excited(C.byref(cfg), size_x, size_y, ansatz.h, sampler.h, log_amp_fn, user,
                                     ref_log_amp_fn, ref_user, mu, C.byref(info)), "nqs_sr_step_excited")
    return info


def tvmc_step(cfg, dt, size_x, size_y, ansatz, sampler, log_amp_fn=None, user=None, heun=False):
    """nqs_tvmc_step_real_time (forward Euler) or nqs_tvmc_step_heun (upstream
    include/nqs/nqs_optimizer.h:206, :267)."""
    info = abi.StepInfo()
    f = lib().nqs_tvmc_step_heun if heun else lib().nqs_tvmc_step_real_time
    _check(f(C.byref(cfg), dt, size_x, size_y, ansatz.h, sampler.h, log_amp_fn, user, C.byref(info)),
           "tvmc step")
    return info


def excited_step_batch(cfg, size_x, size_y, ansatz, batch, ref_log_amp_fn, ref_user, mu, log_amp_fn=None,
                       user=None):
    """Excited-state SR on a caller-supplied batch; returns (info, augmented energies, delta)."""
    s = spins_array(batch, ansatz.N)
    Ns = s.shape[0]
    E, d = np.zeros(Ns), np.zeros(ansatz.P)
    info = abi.StepInfo()
    _check(lib().nqs_gpu_sr_step_batch_excited(C.byref(cfg), size_x, size_y, ansatz.h, log_amp_fn, user,
                                               ref_log_amp_fn, ref_user, mu, _ip(s), Ns, C.byref(info), _dp(E),
                                               _dp(d)), "nqs_gpu_sr_step_batch_excited")
    return info, E, d


def tvmc_step_batch(cfg, dt, size_x, size_y, ansatz, batch, log_amp_fn=None, user=None):
    """Forward-Euler real-time tVMC step on a caller-supplied batch; returns (info, energies, delta)."""
    s = spins_array(batch, ansatz.N)
    Ns = s.shape[0]
    E, d = np.zeros(Ns), np.zeros(ansatz.P)
    info = abi.StepInfo()
    _check(lib().nqs_gpu_tvmc_step_batch(C.byref(cfg), dt, size_x, size_y, ansatz.h, log_amp_fn, user, _ip(s), Ns,
                                         C.byref(info), _dp(E), _dp(d)), "nqs_gpu_tvmc_step_batch")
    return info, E, d


class StepStats(C.Structure):
    _fields_ = [("tau_int", C.c_double), ("ess", C.c_double), ("refine_residual", C.c_double),
                ("refine_sweeps", C.c_int), ("chol_retry", C.c_int), ("chol_fail_col", C.c_int),
                ("gpu_launches", C.c_int), ("delta_rel_err", C.c_double), ("mixed_fallback", C.c_int),
                ("pad_", C.c_int), ("phase_us", C.c_double * 8), ("energy_rel_err", C.c_double)]


def last_step_stats():
    s = StepStats()
    lib().nqs_gpu_last_step_stats(C.byref(s))
    return s


def profile(on):
    lib().nqs_gpu_profile_enable(int(on))


def profile_reset():
    lib().nqs_gpu_profile_reset()


def profile_read(cap=64):
    names = (C.c_char * 48 * cap)()
    counts = (C.c_int * cap)()
    ms = (C.c_double * cap)()
    n = lib().nqs_gpu_profile_read(cap, C.cast(names, VP), counts, ms)
    return {bytes(names[i]).split(b"\0")[0].decode(): (counts[i], ms[i]) for i in range(n)}


def launch_count():
    return lib().nqs_gpu_launch_count()


def ess(energies, num_chains):
    """(tau_int, ESS) of a batch laid out as the sampler writes it."""
    e = np.ascontiguousarray(energies, dtype=np.float64)
    tau, n = C.c_double(), C.c_double()
    _check(lib().nqs_gpu_ess(_dp(e), len(e), num_chains, C.byref(tau), C.byref(n)), "nqs_gpu_ess")
    return tau.value, n.value


class LearnedProposal:
    """The learned (MADE) proposal attached to a Sampler (nqs_sampler_set_learned_proposal)."""

    def __init__(self, sampler, **kw):
        o = lib().nqs_gpu_made_options_default()
        for k, v in kw.items():
            setattr(o, k, v)
        _check(lib().nqs_sampler_set_learned_proposal(sampler.h, C.byref(o)), "nqs_sampler_set_learned_proposal")
        self.s = sampler
        self.opts = o

    def detach(self):
        _check(lib().nqs_sampler_set_learned_proposal(self.s.h, None), "nqs_sampler_set_learned_proposal")

    def stats(self):
        st = abi.MadeStats()
        _check(lib().nqs_sampler_learned_stats(self.s.h, C.byref(st)), "nqs_sampler_learned_stats")
        return st

    def num_params(self):
        return lib().nqs_gpu_made_num_params(self.s.h)

    def weights(self):
        w = np.zeros(self.num_params(), np.float32)
        _check(lib().nqs_gpu_made_get_weights(self.s.h, w.ctypes.data_as(C.POINTER(C.c_float))), "made_get_weights")
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _check(lib().nqs_gpu_made_set_weights(self.s.h, w.ctypes.data_as(C.POINTER(C.c_float))), "made_set_weights")

    def log_prob(self, spins):
        s = spins_array(spins)
        out = np.zeros(s.shape[0])
        _check(lib().nqs_gpu_made_log_prob(self.s.h, _ip(s), s.shape[0], _dp(out)), "made_log_prob")
        return out

    def nll_grad(self, spins):
        s = spins_array(spins)
        g = np.zeros(self.num_params(), np.float32)
        nll = C.c_double()
        _check(lib().nqs_gpu_made_nll_grad(self.s.h, _ip(s), s.shape[0], g.ctypes.data_as(C.POINTER(C.c_float)),
                                          C.byref(nll)), "made_nll_grad")
        return g, nll.value

    def sample(self, count):
        out = np.zeros((count, self.s.N), np.int32)
        lq = np.zeros(count)
        _check(lib().nqs_gpu_made_sample(self.s.h, count, _ip(out), _dp(lq)), "made_sample")
        return out, lq


class Batch:
    """A batch of independent problems stepped together (nqs_gpu_batch_*).
    items: (cfg, size_x, size_y, Ansatz, Sampler, log_amp_fn or None, user)."""

    def __init__(self, items):
        self.items = list(items)           # keeps the configs and objects alive
        arr = (abi.Instance * len(self.items))()
        for i, (cfg, sx, sy, a, s, fn, user) in enumerate(self.items):
            arr[i].cfg = C.pointer(cfg)
            arr[i].size_x, arr[i].size_y = sx, sy
            arr[i].ansatz, arr[i].sampler = a.h, s.h
            arr[i].log_amp = fn
            arr[i].log_amp_user = user
        self._arr = arr
        self.h = lib().nqs_gpu_batch_create(arr, len(self.items))
        if not self.h:
            raise NqsError("nqs_gpu_batch_create failed: " + last_error())

    def step(self):
        infos = (abi.StepInfo * len(self.items))()
        _check(lib().nqs_gpu_batch_step(self.h, infos), "nqs_gpu_batch_step")
        return list(infos)

    def ctas(self):
        out = (C.c_int * len(self.items))()
        _check(lib().nqs_gpu_batch_ctas(self.h, out), "nqs_gpu_batch_ctas")
        return list(out)

    def tune_ms(self):
        out = (C.c_double * 96)()
        n = lib().nqs_gpu_batch_tune_ms(self.h, out, 96)
        return list(out)[:max(n, 0)]

    def block_widths(self):
        """Diagonal block width (64 / 128) of each instance's factor, as autotuned."""
        out = np.zeros(len(self.items), dtype=np.int32)
        _check(lib().nqs_gpu_batch_block_widths(self.h, _ip(out)), "nqs_gpu_batch_block_widths")
        return out.tolist()

    def fallbacks(self):
        """Instance steps whose FP32 factor broke down and were solved in FP64."""
        return int(lib().nqs_gpu_batch_fallbacks(self.h))

    def free(self):
        if getattr(self, "h", None):
            lib().nqs_gpu_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------- exact diagonalisation

def _perm_args(perm, chars):
    perm = np.ascontiguousarray(perm, dtype=np.int32).reshape(-1)
    chars = np.ascontiguousarray(chars, dtype=np.float64).reshape(-1)
    return perm, chars


def lanczos_e0_kagome_lean(Lx, Ly, J, pbc, perm, chars, max_iters=100, tol=1e-9, eigvec=False):
    """Memory-lean projecting Lanczos of the kagome Heisenberg sector (perm, chars) on the
    device: nqs_lanczos_e0_kagome_heisenberg_projected_lean[_eigvec].  Returns
    (E0, eigenvector or None, {"iterations", "converged", "residual_norm"})."""
    perm, chars = _perm_args(perm, chars)
    e = C.c_double()
    r = abi.LanczosResult()
    vec = None
    if eigvec:
        vec = np.zeros(1 << (3 * Lx * Ly))
        rc = lib().nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec(
            Lx, Ly, J, pbc, _ip(perm), _dp(chars), len(chars), max_iters, tol, C.byref(e), _dp(vec), C.byref(r))
    else:
        rc = lib().nqs_lanczos_e0_kagome_heisenberg_projected_lean(
            Lx, Ly, J, pbc, _ip(perm), _dp(chars), len(chars), max_iters, tol, C.byref(e), C.byref(r))
    _check(rc, "lean Lanczos")
    return e.value, vec, {"iterations": r.iterations, "converged": r.converged, "residual_norm": r.residual_norm}


def sz_seed_state(N, irrep_index=None):
    """The xorshift64 start state of the upstream sector drivers' seeds: 0xA5A5A5A5A5A5A5A5 ^ 2^N
    for a magnetisation sector alone, 0xC3C3C3C3C3C3C3C3 ^ 2^N ^ (irrep index * 0x9E3779B97F4A7C15)
    with a p6m irrep (index in A1 A2 B1 B2 E1 E2 order)."""
    dim = 1 << N
    if irrep_index is None:
        return (0xA5A5A5A5A5A5A5A5 ^ dim) & 0xFFFFFFFFFFFFFFFF
    return (0xC3C3C3C3C3C3C3C3 ^ dim ^ ((irrep_index * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)) \
        & 0xFFFFFFFFFFFFFFFF


def lanczos_e0_kagome_sz(Lx, Ly, J, pbc, perm, chars, popcount, seed_state=0, max_iters=200, tol=1e-10,
                         eigvec=False):
    """Magnetisation-sector lean Lanczos (nqs_gpu_lanczos_e0_kagome_sz_projected_lean): the states
    with `popcount` down spins, projected on the sector (perm, chars); seed_state as
    sz_seed_state() for the upstream sector drivers' seeds, 0 for the library seed.  Returns
    (E0, eigenvector or None, {"iterations", "converged", "residual_norm"})."""
    perm, chars = _perm_args(perm, chars)
    e = C.c_double()
    r = abi.LanczosResult()
    vec = np.zeros(1 << (3 * Lx * Ly)) if eigvec else None
    rc = lib().nqs_gpu_lanczos_e0_kagome_sz_projected_lean(
        Lx, Ly, J, pbc, _ip(perm), _dp(chars), len(chars), popcount, seed_state, max_iters, tol, C.byref(e),
        _dp(vec) if eigvec else None, C.byref(r))
    _check(rc, "sector Lanczos")
    return e.value, vec, {"iterations": r.iterations, "converged": r.converged, "residual_norm": r.residual_norm}


def lanczos_last_coeffs(cap=4096):
    """(alpha[K], beta[K+1]) of the last Lanczos run (beta[0] = 0)."""
    a, b = np.zeros(cap), np.zeros(cap + 1)
    K = lib().nqs_gpu_lanczos_last_coeffs(cap, _dp(a), _dp(b))
    K = min(K, cap)
    return a[:K].copy(), b[:K + 1].copy()


def sector_project_host(psi, N, perm, chars):
    """nqs_kagome_p6m_project_inplace on a copy of psi (host array of 2^N doubles)."""
    perm, chars = _perm_args(perm, chars)
    out = np.array(psi, dtype=np.float64, copy=True)
    lib().nqs_kagome_p6m_project_inplace(_dp(out), N, len(chars), _ip(perm), _dp(chars))
    err = last_error()
    if err:
        raise NqsError("sector projection failed: " + err)
    return out


def gpu_sector_project(N, perm, chars, d_in, d_out):
    """Device-pointer projector (d_out may equal d_in)."""
    perm, chars = _perm_args(perm, chars)
    _check(lib().nqs_gpu_sector_project(N, len(chars), _ip(perm), _dp(chars), d_in, d_out), "sector projection")


def gpu_kagome_heis_matvec(Lx, Ly, J, pbc, d_in, d_out):
    _check(lib().nqs_gpu_kagome_heis_matvec(Lx, Ly, J, pbc, d_in, d_out), "kagome matvec")


def gpu_lanczos_seed(N, alternate, d_out):
    _check(lib().nqs_gpu_lanczos_seed(N, alternate, d_out), "Lanczos seed")


def projector_plan(N, perm, chars):
    """(passes, [sizes], element order) of the device sector projector (host only)."""
    perm, chars = _perm_args(perm, chars)
    G = len(chars)
    npass = C.c_int()
    sizes = (C.c_int * 4)()
    elems = np.zeros(G, dtype=np.int32)
    _check(lib().nqs_ed_projector_plan(N, G, _ip(perm), _dp(chars), C.byref(npass), sizes, _ip(elems)),
           "projector plan")
    sz = [sizes[i] for i in range(npass.value)]
    return npass.value, sz, elems[:sum(sz)].copy()
