"""ctypes bindings of the CPU oracle (oracle/liboracle.so) for tests.

Test infrastructure: the oracle is the checker.  Only tests/, the smoke check and
bench.py's CPU legs load it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libnqs_ref.so")

OR_MF, OR_RBM, OR_CRBM, OR_MLP = 0, 5, 6, 100
OR_TFIM, OR_HEIS, OR_J1J2, OR_XXZ, OR_KAGOME = 0, 1, 2, 4, 6
LAYER_MARSHALL, LAYER_SYMPROJ = 1, 2

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)


class OrAnsatz(C.Structure):
    _fields_ = [("kind", C.c_int), ("N", C.c_int), ("M", C.c_int), ("depth", C.c_int),
                ("params", DP)]


class OrLayer(C.Structure):
    _fields_ = [("type", C.c_int), ("size_x", C.c_int), ("size_y", C.c_int), ("G", C.c_int),
                ("perm", IP), ("chars", DP)]


class OrAmp(C.Structure):
    _fields_ = [("base", OrAnsatz), ("n_layers", C.c_int), ("layers", OrLayer * 4)]


class OrHam(C.Structure):
    _fields_ = [("ham", C.c_int), ("size_x", C.c_int), ("size_y", C.c_int), ("pbc", C.c_int),
                ("kagome_pbc", C.c_int), ("J", C.c_double), ("J2", C.c_double),
                ("Jz", C.c_double), ("Gamma", C.c_double)]


class OrStepInfo(C.Structure):
    _fields_ = [("mean_energy", C.c_double), ("variance_energy", C.c_double),
                ("update_norm", C.c_double), ("cg_iterations", C.c_int), ("converged", C.c_int)]


class OrChainOpts(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("num_chains", C.c_int), ("move", C.c_int),
                ("n_down", C.c_int)]


def build_oracle(force=False):
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("nqs_oracle.c", "oracle_sampler_sr.c", "oracle_ed.c")]
    if not force and os.path.exists(ORACLE_SO) and all(
            os.path.getmtime(ORACLE_SO) >= os.path.getmtime(s) for s in srcs):
        return ORACLE_SO
    subprocess.check_call(["gcc", "-std=c11", "-D_GNU_SOURCE", "-O2", "-fPIC", "-shared",
                           "-o", ORACLE_SO] + srcs + ["-lm"])
    return ORACLE_SO


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build_oracle())
        L = _LIB
        L.oracle_num_params.restype = C.c_long
        L.oracle_num_params.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oracle_ansatz_init.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint, DP]
        L.oracle_log_amp_batch.argtypes = [C.POINTER(OrAmp), IP, C.c_int, DP, DP]
        L.oracle_gradient_batch.argtypes = [C.POINTER(OrAnsatz), IP, C.c_int, DP]
        L.oracle_gradient_complex_batch.argtypes = [C.POINTER(OrAnsatz), IP, C.c_int, DP, DP]
        L.oracle_symproj_gradient_batch.argtypes = [C.POINTER(OrAmp), IP, C.c_int, DP]
        L.oracle_marshall_parity.argtypes = [IP, C.c_int, C.c_int]
        L.oracle_local_energy_batch.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), IP, C.c_int,
                                                DP, DP]
        L.oracle_bonds.argtypes = [C.POINTER(OrHam), IP, C.c_int]
        L.oracle_xorshift_sampler.argtypes = [C.POINTER(OrAmp), C.c_int, C.c_uint, C.c_int,
                                              C.c_int, C.c_int, IP, DP]
        L.oracle_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32)]
        L.oracle_chain_init.argtypes = [C.POINTER(OrChainOpts), C.c_int, C.POINTER(C.c_uint64)]
        L.oracle_chain_run.argtypes = [C.POINTER(OrChainOpts), C.POINTER(OrAmp), C.POINTER(OrHam),
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int,
                                       C.c_int, C.c_int, IP, C.POINTER(C.c_long),
                                       C.POINTER(C.c_long)]
        L.oracle_minsr_step.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), C.c_int, IP, C.c_int,
                                        C.c_double, C.c_double, DP, C.c_long, DP, DP,
                                        C.POINTER(OrStepInfo)]
        L.oracle_cgsr_step.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), C.c_int, IP, C.c_int,
                                       C.c_double, C.c_double, C.c_int, C.c_double, DP, C.c_long,
                                       DP, DP, C.POINTER(OrStepInfo)]
        L.oracle_holo_step.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), IP, C.c_int, C.c_double, C.c_double,
                                       C.c_int, C.c_double, DP, C.c_long, DP, DP, C.POINTER(OrStepInfo)]
        L.oracle_holo_step_grad.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), C.c_int, IP, C.c_int, C.c_double,
                                            C.c_double, C.c_int, C.c_double, DP, C.c_long, DP, DP,
                                            C.POINTER(OrStepInfo)]
        L.oracle_excited_step.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), C.POINTER(OrAmp), C.c_double, IP,
                                          C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, DP, C.c_long,
                                          DP, DP, C.POINTER(OrStepInfo)]
        L.oracle_tvmc_step.argtypes = [C.POINTER(OrHam), C.POINTER(OrAmp), IP, C.c_int, C.c_double, C.c_double,
                                       C.c_int, C.c_double, DP, C.c_long, DP, DP, C.POINTER(OrStepInfo)]
        L.oracle_exact_energy.argtypes = [C.POINTER(OrHam), C.c_int, C.c_int, C.c_double, DP]
    return _LIB


def dp(a):
    return a.ctypes.data_as(DP)


def ip(a):
    return a.ctypes.data_as(IP)


class Amp:
    """Keeps the numpy buffers an OrAmp points into alive."""

    def __init__(self, kind, N, M, params, layers=()):
        self.params = np.ascontiguousarray(params, dtype=np.float64)
        self._keep = []
        self.s = OrAmp()
        self.s.base = OrAnsatz(kind, N, M, 2, dp(self.params))
        self.s.n_layers = len(layers)
        for k, L in enumerate(layers):
            if L[0] == "marshall":
                self.s.layers[k] = OrLayer(LAYER_MARSHALL, L[1], L[2], 0, None, None)
            else:
                perm = np.ascontiguousarray(L[1], dtype=np.int32)
                chars = np.ascontiguousarray(L[2], dtype=np.float64)
                self._keep += [perm, chars]
                self.s.layers[k] = OrLayer(LAYER_SYMPROJ, 0, 0, len(chars), ip(perm), dp(chars))

    @property
    def N(self):
        return self.s.base.N

    def ref(self):
        return C.byref(self.s)


def num_params(kind, N, M):
    return lib().oracle_num_params(kind, N, M)


def init_params(kind, N, M, scale=0.01, seed=0xC0FFEE):
    P = num_params(kind, N, M)
    p = np.zeros(P)
    assert lib().oracle_ansatz_init(kind, N, M, scale, seed, dp(p)) == 0
    return p


def log_amp(amp, spins):
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    B = spins.shape[0]
    la, ar = np.zeros(B), np.zeros(B)
    lib().oracle_log_amp_batch(amp.ref(), ip(spins), B, dp(la), dp(ar))
    return la, ar


def gradient(amp, spins):
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    B = spins.shape[0]
    P = num_params(amp.s.base.kind, amp.N, amp.s.base.M)
    out = np.zeros((B, P))
    assert lib().oracle_gradient_batch(C.byref(amp.s.base), ip(spins), B, dp(out)) == 0
    return out


def gradient_complex(amp, spins):
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    B = spins.shape[0]
    P = num_params(amp.s.base.kind, amp.N, amp.s.base.M)
    re, im = np.zeros((B, P)), np.zeros((B, P))
    assert lib().oracle_gradient_complex_batch(C.byref(amp.s.base), ip(spins), B, dp(re),
                                               dp(im)) == 0
    return re, im


def symproj_gradient(amp, spins):
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    B = spins.shape[0]
    P = num_params(amp.s.base.kind, amp.N, amp.s.base.M)
    out = np.zeros((B, P))
    assert lib().oracle_symproj_gradient_batch(amp.ref(), ip(spins), B, dp(out)) == 0
    return out


def ham(kind, Lx, Ly, pbc=0, kagome_pbc=1, J=1.0, J2=0.0, Jz=1.0, Gamma=1.0):
    return OrHam(kind, Lx, Ly, pbc, kagome_pbc, J, J2, Jz, Gamma)


def local_energy(h, amp, spins, complex_out=False):
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    B = spins.shape[0]
    re, im = np.zeros(B), np.zeros(B)
    lib().oracle_local_energy_batch(C.byref(h), amp.ref(), ip(spins), B, dp(re), dp(im))
    return (re, im) if complex_out else re


def bonds(h):
    out = np.zeros(4096, dtype=np.int32)
    n = lib().oracle_bonds(C.byref(h), ip(out), 2048)
    return out[:2 * n].reshape(n, 2)


def xorshift_sampler(amp, seed, n_therm, n_decor, n):
    N = amp.N
    out = np.zeros((n, N), dtype=np.int32)
    acc = C.c_double()
    lib().oracle_xorshift_sampler(amp.ref(), N, seed, n_therm, n_decor, n, ip(out), C.byref(acc))
    return out, acc.value


def chain_sampler(amp, h, seed, chains, move, n_down, therm, n_spc, decor):
    N = amp.N
    o = OrChainOpts(seed, chains, move, n_down)
    bits = np.zeros(chains, dtype=np.uint64)
    assert lib().oracle_chain_init(C.byref(o), N, bits.ctypes.data_as(C.POINTER(C.c_uint64))) == 0
    mc = C.c_uint64(0)
    out = np.zeros((n_spc * chains, N), dtype=np.int32)
    acc, pro = C.c_long(0), C.c_long(0)
    assert lib().oracle_chain_run(C.byref(o), amp.ref(), C.byref(h),
                                  bits.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(mc),
                                  therm, n_spc, decor, ip(out), C.byref(acc), C.byref(pro)) == 0
    return out, bits, acc.value, pro.value


def minsr_step(h, amp, batch, shift, lr, grad_mode=0):
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    Ns = batch.shape[0]
    P = len(amp.params)
    E, d = np.zeros(Ns), np.zeros(P)
    info = OrStepInfo()
    assert lib().oracle_minsr_step(C.byref(h), amp.ref(), grad_mode, ip(batch), Ns, shift, lr,
                                   dp(amp.params), P, dp(E), dp(d), C.byref(info)) == 0
    return E, d, info


def cgsr_step(h, amp, batch, shift, lr, max_iters, tol, grad_mode=0):
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    Ns = batch.shape[0]
    P = len(amp.params)
    E, d = np.zeros(Ns), np.zeros(P)
    info = OrStepInfo()
    assert lib().oracle_cgsr_step(C.byref(h), amp.ref(), grad_mode, ip(batch), Ns, shift, lr,
                                  max_iters, tol, dp(amp.params), P, dp(E), dp(d),
                                  C.byref(info)) == 0
    return E, d, info


def holo_step(h, amp, batch, shift, lr, max_iters, tol):
    """Holomorphic SR on a batch (src/nqs/nqs_optimizer.c:415-524)."""
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    Ns = batch.shape[0]
    P = len(amp.params)
    E, d = np.zeros(Ns), np.zeros(P)
    info = OrStepInfo()
    assert lib().oracle_holo_step(C.byref(h), amp.ref(), ip(batch), Ns, shift, lr, max_iters, tol,
                                  dp(amp.params), P, dp(E), dp(d), C.byref(info)) == 0
    return E, d, info


def symproj_gradient_complex(amp, spins):
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    B = spins.shape[0]
    P = num_params(amp.s.base.kind, amp.N, amp.s.base.M)
    re, im = np.zeros((B, P)), np.zeros((B, P))
    assert lib().oracle_symproj_gradient_complex_batch(amp.ref(), ip(spins), B, dp(re), dp(im)) == 0
    return re, im


def holo_step_sym(h, amp, batch, shift, lr, max_iters, tol):
    """Holomorphic SR with nqs_symproj_gradient_complex as the gradient (the amplitude's
    symproj layer)."""
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    Ns = batch.shape[0]
    P = len(amp.params)
    E, d = np.zeros(Ns), np.zeros(P)
    info = OrStepInfo()
    assert lib().oracle_holo_step_grad(C.byref(h), amp.ref(), 1, ip(batch), Ns, shift, lr, max_iters, tol,
                                       dp(amp.params), P, dp(E), dp(d), C.byref(info)) == 0
    return E, d, info


def excited_step(h, amp, ref, mu, batch, shift, lr, max_iters, tol):
    """Excited-state SR on a batch (src/nqs/nqs_optimizer.c:562-723); returns the
    augmented local energies, the update and the info."""
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    Ns = batch.shape[0]
    P = len(amp.params)
    E, d = np.zeros(Ns), np.zeros(P)
    info = OrStepInfo()
    assert lib().oracle_excited_step(C.byref(h), amp.ref(), ref.ref(), mu, ip(batch), Ns, shift, lr, max_iters,
                                     tol, dp(amp.params), P, dp(E), dp(d), C.byref(info)) == 0
    return E, d, info


def tvmc_step(h, amp, batch, shift, dt, max_iters, tol):
    """Forward-Euler real-time tVMC step on a batch (src/nqs/nqs_optimizer.c:888-993)."""
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    Ns = batch.shape[0]
    P = len(amp.params)
    E, d = np.zeros(Ns), np.zeros(P)
    info = OrStepInfo()
    assert lib().oracle_tvmc_step(C.byref(h), amp.ref(), ip(batch), Ns, shift, dt, max_iters, tol,
                                  dp(amp.params), P, dp(E), dp(d), C.byref(info)) == 0
    return E, d, info


def exact_energy(h, n_down=-1, max_iters=300, tol=1e-12):
    e = C.c_double()
    assert lib().oracle_exact_energy(C.byref(h), n_down, max_iters, tol, C.byref(e)) == 0
    return e.value


class OrLanczosInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("residual", C.c_double),
                ("alpha", C.c_double * 512), ("beta", C.c_double * 513)]


def kagome_matvec(Lx, Ly, J, pbc, x):
    """H x on the full 2^N basis (src/nqs/nqs_lanczos.c:380-432)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().oracle_kagome_heis_matvec(Lx, Ly, C.c_double(J), pbc, dp(x), dp(y))
    return y


def sector_project(psi, N, perm, chars):
    """(1/G) sum_g chi(g) T(g) psi (src/nqs/nqs_symproj.c:786-852)."""
    out = np.array(psi, dtype=np.float64, copy=True)
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    chars = np.ascontiguousarray(chars, dtype=np.float64)
    lib().oracle_sector_project(dp(out), N, len(chars), ip(perm), dp(chars))
    return out


def lanczos_seed(N, alternate=0):
    out = np.zeros(1 << N)
    lib().oracle_lanczos_seed(N, alternate, dp(out))
    return out


def lanczos_lean_kagome(Lx, Ly, J, pbc, perm, chars, max_iters, tol, eigvec=False):
    """Memory-lean projecting Lanczos (src/mps/lanczos.c:824-960, :972-1119)."""
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    chars = np.ascontiguousarray(chars, dtype=np.float64)
    e = C.c_double()
    vec = np.zeros(1 << (3 * Lx * Ly)) if eigvec else None
    info = OrLanczosInfo()
    assert lib().oracle_lanczos_lean_kagome(Lx, Ly, C.c_double(J), pbc, ip(perm), dp(chars), len(chars),
                                            max_iters, C.c_double(tol), C.byref(e),
                                            dp(vec) if eigvec else None, C.byref(info)) == 0
    return e.value, vec, info


def ed_iteration_sample(Lx, Ly, perm, chars, x, count):
    """Seconds for the oracle's matvec and direct projector over the first `count` states
    (single thread): the CPU baseline's bounded sample of one Lanczos iteration."""
    import time
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    chars = np.ascontiguousarray(chars, dtype=np.float64)
    N = 3 * Lx * Ly
    y = np.zeros(1 << N)
    t = np.zeros(count)
    t0 = time.perf_counter()
    lib().oracle_kagome_heis_matvec_range(Lx, Ly, C.c_double(1.0), 1, dp(x), dp(y), C.c_long(0), C.c_long(count))
    t1 = time.perf_counter()
    lib().oracle_sector_project_range(dp(x), dp(t), N, len(chars), ip(perm), dp(chars), C.c_long(0),
                                      C.c_long(count))
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1


def materialise(amp, N):
    """The NQS state on the full basis (src/nqs/nqs_lanczos.c:65-106)."""
    psi = np.zeros(1 << N)
    assert lib().oracle_materialise(amp.ref(), N, dp(psi)) == 0
    return psi


def variational_energy(amp, ham, Lx, Ly, J, X, pbc=0):
    """<psi|H|psi>/<psi|psi> of the materialised state: ham 0 TFIM (X = Gamma), 1 XXZ
    (X = Jz), 6 kagome Heisenberg (src/nqs/nqs_lanczos.c:188-224, 283-321, 434-455)."""
    e = C.c_double()
    assert lib().oracle_variational_energy(amp.ref(), ham, Lx, Ly, C.c_double(J), C.c_double(X), pbc,
                                           C.byref(e)) == 0
    return e.value
