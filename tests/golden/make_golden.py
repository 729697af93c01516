"""Generate golden vectors from the upstream reference library itself.

Runs here only (it needs oracle/_ref/libnqs_ref.so, built from the upstream
sources by `make -C oracle`).  The outputs are small .npz fixtures committed
under tests/golden/; the GPU machine reads only those.

Each fixture records the upstream call that produced it (function names are
those of the upstream C API, include/nqs/*.h).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from spin_based_neural_network_gb300 import abi  # noqa: E402

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)


def load_ref():
    so = os.path.join(ROOT, "oracle", "_ref", "libnqs_ref.so")
    if not os.path.exists(so):
        raise SystemExit("build the reference first: make -C oracle")
    L = C.CDLL(so)
    L.nqs_ansatz_create.restype = C.c_void_p
    L.nqs_ansatz_create.argtypes = [C.POINTER(abi.NqsConfig), C.c_int]
    L.nqs_ansatz_free.argtypes = [C.c_void_p]
    L.nqs_ansatz_num_params.restype = C.c_long
    L.nqs_ansatz_num_params.argtypes = [C.c_void_p]
    L.nqs_ansatz_params_raw.restype = DP
    L.nqs_ansatz_params_raw.argtypes = [C.c_void_p]
    L.nqs_ansatz_log_amp.argtypes = [IP, C.c_int, C.c_void_p, DP, DP]
    L.nqs_ansatz_logpsi_gradient.argtypes = [C.c_void_p, IP, C.c_int, DP]
    L.nqs_ansatz_logpsi_gradient_complex.argtypes = [C.c_void_p, IP, C.c_int, DP, DP]
    L.nqs_local_energy_batch.argtypes = [C.POINTER(abi.NqsConfig), C.c_int, C.c_int, IP, C.c_int,
                                         C.c_void_p, C.c_void_p, DP]
    L.nqs_local_energy_batch_complex.argtypes = [C.POINTER(abi.NqsConfig), C.c_int, C.c_int, IP,
                                                 C.c_int, C.c_void_p, C.c_void_p, DP, DP]
    L.nqs_sampler_create.restype = C.c_void_p
    L.nqs_sampler_create.argtypes = [C.c_int, C.POINTER(abi.NqsConfig), C.c_void_p, C.c_void_p]
    L.nqs_sampler_free.argtypes = [C.c_void_p]
    L.nqs_sampler_thermalize.argtypes = [C.c_void_p]
    L.nqs_sampler_batch.argtypes = [C.c_void_p, C.c_int, IP]
    L.nqs_sampler_acceptance_ratio.restype = C.c_double
    L.nqs_sampler_acceptance_ratio.argtypes = [C.c_void_p]
    L.nqs_sr_step_minsr_full.argtypes = [C.POINTER(abi.NqsConfig), C.c_int, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.POINTER(abi.StepInfo)]
    L.nqs_sr_step_custom_full.argtypes = L.nqs_sr_step_minsr_full.argtypes
    L.nqs_symproj_gradient.argtypes = [C.c_void_p, C.c_void_p, IP, C.c_int, DP]
    L.nqs_kagome_p2_perm.argtypes = [C.c_int, C.c_int, C.POINTER(IP), C.POINTER(DP),
                                     C.POINTER(C.c_int)]
    L.nqs_kagome_translation_perm.argtypes = [C.c_int, C.c_int, C.POINTER(IP), C.POINTER(C.c_int)]
    L.nqs_lanczos_refine_tfim.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                          C.c_int, C.c_double, DP, DP, C.c_void_p]
    L.nqs_lanczos_refine_heisenberg.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double,
                                                C.c_double, C.c_int, C.c_double, DP, DP,
                                                C.c_void_p]
    return L


def fnptr(L, name):
    return C.cast(getattr(L, name), C.c_void_p).value


def params_of(L, a):
    P = L.nqs_ansatz_num_params(a)
    return np.ctypeslib.as_array(L.nqs_ansatz_params_raw(a), shape=(P,)).copy()


def rand_spins(rng, B, N):
    return np.where(rng.random((B, N)) < 0.5, 1, -1).astype(np.int32)


def gen_ansatz(L, out):
    """nqs_ansatz_create + nqs_ansatz_log_amp + gradients (real and holomorphic)."""
    rng = np.random.default_rng(1234)
    cases = [("mf", abi.ANSATZ_LEGACY_MLP, 9, 0, 0.01, 7),
             ("rbm", abi.ANSATZ_RBM, 16, 16, 0.01, 0xC0FFEE),
             ("rbm_big", abi.ANSATZ_RBM, 16, 32, 0.5, 11),
             ("crbm", abi.ANSATZ_COMPLEX_RBM, 16, 32, 0.01, 0xC0FFEE),
             ("crbm_big", abi.ANSATZ_COMPLEX_RBM, 12, 24, 0.8, 99)]
    for name, kind, N, M, scale, seed in cases:
        cfg = abi.config_defaults(ansatz=kind, rbm_hidden_units=M, rbm_init_scale=scale,
                                  rng_seed=seed)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p = params_of(L, a)
        P = len(p)
        spins = rand_spins(rng, 64, N)
        la, ar = np.zeros(64), np.zeros(64)
        g = np.zeros((64, P))
        gr, gi = np.zeros((64, P)), np.zeros((64, P))
        for b in range(64):
            s = spins[b].ctypes.data_as(IP)
            L.nqs_ansatz_log_amp(s, N, a, C.byref(C.c_double.from_buffer(la, 8 * b)),
                                 C.byref(C.c_double.from_buffer(ar, 8 * b)))
            L.nqs_ansatz_logpsi_gradient(a, s, N, g[b].ctypes.data_as(DP))
            L.nqs_ansatz_logpsi_gradient_complex(a, s, N, gr[b].ctypes.data_as(DP),
                                                 gi[b].ctypes.data_as(DP))
        out["ansatz_" + name] = dict(kind=kind, N=N, M=M, scale=scale, seed=seed, params=p,
                                     spins=spins, la=la, arg=ar, grad=g, grad_re=gr, grad_im=gi)
        L.nqs_ansatz_free(a)


def gen_local_energy(L, out):
    """nqs_local_energy_batch / _complex through nqs_ansatz_log_amp and nqs_marshall_log_amp."""
    rng = np.random.default_rng(99)
    cases = [("tfim_3x3_rbm", abi.HAM_TFIM, 3, 3, abi.ANSATZ_RBM, 18, 0.5, dict(transverse_field=0.7)),
             ("tfim_16x1_rbm", abi.HAM_TFIM, 16, 1, abi.ANSATZ_RBM, 16, 0.5, {}),
             ("heis_4x4_crbm_marshall", abi.HAM_HEISENBERG, 4, 4, abi.ANSATZ_COMPLEX_RBM, 32, 0.5, {}),
             ("xxz_4x3_crbm", abi.HAM_XXZ, 4, 3, abi.ANSATZ_COMPLEX_RBM, 24, 0.5,
              dict(j_z_coupling=1.7, j_coupling=0.8)),
             ("j1j2_4x4_crbm", abi.HAM_J1_J2, 4, 4, abi.ANSATZ_COMPLEX_RBM, 16, 0.5,
              dict(j2_coupling=0.5)),
             ("kagome_2x2_pbc_crbm", abi.HAM_KAGOME_HEISENBERG, 2, 2, abi.ANSATZ_COMPLEX_RBM, 24,
              0.5, dict(kagome_pbc=1)),
             ("kagome_2x2_obc_rbm", abi.HAM_KAGOME_HEISENBERG, 2, 2, abi.ANSATZ_RBM, 12, 0.5,
              dict(kagome_pbc=0)),
             ("kagome_3x3_pbc_crbm", abi.HAM_KAGOME_HEISENBERG, 3, 3, abi.ANSATZ_COMPLEX_RBM, 54,
              0.3, dict(kagome_pbc=1))]
    for name, ham, Lx, Ly, kind, M, scale, extra in cases:
        N = 3 * Lx * Ly if ham == abi.HAM_KAGOME_HEISENBERG else Lx * Ly
        cfg = abi.config_defaults(ansatz=kind, rbm_hidden_units=M, rbm_init_scale=scale,
                                  hamiltonian=ham, rng_seed=2024, **extra)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p = params_of(L, a)
        spins = rand_spins(rng, 48, N)
        marshall = name.endswith("marshall")
        if marshall:
            w = abi.MarshallWrapper(fnptr(L, "nqs_ansatz_log_amp"), a, Lx, Ly)
            fn, user = fnptr(L, "nqs_marshall_log_amp"), C.addressof(w)
        else:
            fn, user = fnptr(L, "nqs_ansatz_log_amp"), a
        E = np.zeros(48)
        Er, Ei = np.zeros(48), np.zeros(48)
        L.nqs_local_energy_batch(C.byref(cfg), Lx, Ly, spins.ctypes.data_as(IP), 48, fn, user,
                                 E.ctypes.data_as(DP))
        L.nqs_local_energy_batch_complex(C.byref(cfg), Lx, Ly, spins.ctypes.data_as(IP), 48, fn,
                                         user, Er.ctypes.data_as(DP), Ei.ctypes.data_as(DP))
        out["eloc_" + name] = dict(ham=ham, Lx=Lx, Ly=Ly, kind=kind, M=M, N=N, marshall=int(marshall),
                                   J=cfg.j_coupling, J2=cfg.j2_coupling, Jz=cfg.j_z_coupling,
                                   Gamma=cfg.transverse_field, kagome_pbc=cfg.kagome_pbc,
                                   params=p, spins=spins, E=E, E_re=Er, E_im=Ei)
        L.nqs_ansatz_free(a)


def gen_sampler(L, out):
    """nqs_sampler_create + thermalize + batch (single-chain xorshift64)."""
    cases = [("rbm16", abi.ANSATZ_RBM, 16, 16, 0.5, 77, 64, 3, 200),
             ("crbm16_marshall", abi.ANSATZ_COMPLEX_RBM, 16, 32, 0.4, 5, 128, 4, 256)]
    for name, kind, N, M, scale, seed, therm, decor, n in cases:
        cfg = abi.config_defaults(ansatz=kind, rbm_hidden_units=M, rbm_init_scale=scale,
                                  rng_seed=seed, num_thermalize=therm, num_decorrelate=decor)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p = params_of(L, a)
        keep = None
        if name.endswith("marshall"):
            keep = abi.MarshallWrapper(fnptr(L, "nqs_ansatz_log_amp"), a, 4, 4)
            fn, user = fnptr(L, "nqs_marshall_log_amp"), C.addressof(keep)
        else:
            fn, user = fnptr(L, "nqs_ansatz_log_amp"), a
        s = L.nqs_sampler_create(N, C.byref(cfg), fn, user)
        L.nqs_sampler_thermalize(s)
        batch = np.zeros((n, N), dtype=np.int32)
        L.nqs_sampler_batch(s, n, batch.ctypes.data_as(IP))
        acc = L.nqs_sampler_acceptance_ratio(s)
        out["sampler_" + name] = dict(kind=kind, N=N, M=M, seed=seed, therm=therm, decor=decor,
                                      params=p, batch=batch, acceptance=acc,
                                      marshall=int(keep is not None))
        L.nqs_sampler_free(s)
        L.nqs_ansatz_free(a)


def gen_sr(L, out):
    """One nqs_sr_step_minsr_full / nqs_sr_step_custom_full step.  A twin sampler
    with the same seed, thermalised and batched, reproduces the batch the step
    consumes (the sampler is a deterministic function of seed and amplitudes)."""
    cases = [("minsr_tfim_rbm", "minsr", abi.HAM_TFIM, 4, 4, abi.ANSATZ_RBM, 16, 256, 1e-3, 0.01),
             ("minsr_heis_crbm_marshall", "minsr", abi.HAM_HEISENBERG, 4, 4,
              abi.ANSATZ_COMPLEX_RBM, 32, 512, 1e-4, 0.005),
             ("cg_tfim_rbm", "cg", abi.HAM_TFIM, 4, 4, abi.ANSATZ_RBM, 16, 256, 1e-3, 0.01),
             ("cg_j1j2_crbm", "cg", abi.HAM_J1_J2, 3, 4, abi.ANSATZ_COMPLEX_RBM, 24, 256, 1e-3,
              0.01)]
    for name, solver, ham, Lx, Ly, kind, M, Ns, shift, lr in cases:
        N = Lx * Ly
        cfg = abi.config_defaults(ansatz=kind, rbm_hidden_units=M, rbm_init_scale=0.3,
                                  hamiltonian=ham, rng_seed=31337, num_samples=Ns,
                                  num_thermalize=64, num_decorrelate=2, sr_diag_shift=shift,
                                  learning_rate=lr, j2_coupling=0.4, transverse_field=0.9)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p0 = params_of(L, a)
        keep = None
        if name.endswith("marshall"):
            keep = abi.MarshallWrapper(fnptr(L, "nqs_ansatz_log_amp"), a, Lx, Ly)
            fn, user = fnptr(L, "nqs_marshall_log_amp"), C.addressof(keep)
        else:
            fn, user = fnptr(L, "nqs_ansatz_log_amp"), a
        twin = L.nqs_sampler_create(N, C.byref(cfg), fn, user)
        L.nqs_sampler_thermalize(twin)
        batch = np.zeros((Ns, N), dtype=np.int32)
        L.nqs_sampler_batch(twin, Ns, batch.ctypes.data_as(IP))
        s = L.nqs_sampler_create(N, C.byref(cfg), fn, user)
        L.nqs_sampler_thermalize(s)
        info = abi.StepInfo()
        step = L.nqs_sr_step_minsr_full if solver == "minsr" else L.nqs_sr_step_custom_full
        rc = step(C.byref(cfg), Lx, Ly, a, s, fn, user, None, None, C.byref(info))
        assert rc == 0
        p1 = params_of(L, a)
        out["sr_" + name] = dict(solver=solver, ham=ham, Lx=Lx, Ly=Ly, kind=kind, M=M, N=N,
                                 Ns=Ns, shift=shift, lr=lr, J=cfg.j_coupling, J2=cfg.j2_coupling,
                                 Gamma=cfg.transverse_field, cg_max=cfg.sr_cg_max_iters,
                                 cg_tol=cfg.sr_cg_tol, marshall=int(keep is not None),
                                 params0=p0, params1=p1, batch=batch,
                                 info=np.array([info.mean_energy, info.variance_energy,
                                                info.update_norm, info.acceptance_ratio,
                                                info.cg_iterations, info.converged]))
        L.nqs_sampler_free(s)
        L.nqs_sampler_free(twin)
        L.nqs_ansatz_free(a)


def gen_symproj(L, out):
    """nqs_symproj_log_amp / nqs_symproj_gradient with kagome p2 and translation groups."""
    rng = np.random.default_rng(5)
    for name, builder in (("p2", "p2"), ("trans", "trans")):
        Lx = Ly = 2
        N = 12
        cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=12,
                                  rbm_init_scale=0.6, rng_seed=4242)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p = params_of(L, a)
        perm = IP()
        G = C.c_int()
        if builder == "p2":
            chars = DP()
            assert L.nqs_kagome_p2_perm(Lx, Ly, C.byref(perm), C.byref(chars), C.byref(G)) == 0
            ch = np.ctypeslib.as_array(chars, shape=(G.value,)).copy()
        else:
            assert L.nqs_kagome_translation_perm(Lx, Ly, C.byref(perm), C.byref(G)) == 0
            ch = np.ones(G.value)
        pm = np.ctypeslib.as_array(perm, shape=(G.value * N,)).copy().astype(np.int32)
        pm_c = np.ascontiguousarray(pm)
        ch_c = np.ascontiguousarray(ch)
        w = abi.SymprojWrapper(fnptr(L, "nqs_ansatz_log_amp"), a, N, G.value,
                               pm_c.ctypes.data_as(IP), ch_c.ctypes.data_as(DP))
        spins = rand_spins(rng, 32, N)
        la, ar = np.zeros(32), np.zeros(32)
        P = len(p)
        g = np.zeros((32, P))
        sym_fn = C.CFUNCTYPE(None, IP, C.c_int, C.c_void_p, DP, DP)(
            fnptr(L, "nqs_symproj_log_amp"))
        for b in range(32):
            sp = spins[b].ctypes.data_as(IP)
            lb, ab = C.c_double(), C.c_double()
            sym_fn(sp, N, C.addressof(w), C.byref(lb), C.byref(ab))
            la[b], ar[b] = lb.value, ab.value
            L.nqs_symproj_gradient(C.addressof(w), a, sp, N, g[b].ctypes.data_as(DP))
        out["symproj_" + name] = dict(N=N, M=12, kind=abi.ANSATZ_COMPLEX_RBM, G=G.value,
                                      perm=pm, chars=ch, params=p, spins=spins, la=la, arg=ar,
                                      grad=g)
        L.nqs_ansatz_free(a)


def gen_exact(L, out):
    """nqs_lanczos_refine_tfim / _heisenberg (OBC, full basis)."""
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=4)
    rows = []
    for (kind, Lx, Ly, J, X) in [("tfim", 3, 3, 1.0, 0.8), ("tfim", 4, 3, 1.0, 1.0),
                                 ("heis", 2, 4, 1.0, 1.0), ("heis", 3, 3, 1.0, 0.6)]:
        a = L.nqs_ansatz_create(C.byref(cfg), Lx * Ly)
        ev = C.c_double()
        res = (C.c_double * 4)()          # lanczos_result_t (upstream include/mps/lanczos.h:37-42)
        if kind == "tfim":
            rc = L.nqs_lanczos_refine_tfim(a, Lx, Ly, J, X, 300, 1e-12, C.byref(ev), None,
                                           C.byref(res))
        else:
            rc = L.nqs_lanczos_refine_heisenberg(a, Lx, Ly, J, X, 300, 1e-12, C.byref(ev), None,
                                                 C.byref(res))
        assert rc == 0
        rows.append([0 if kind == "tfim" else 1, Lx, Ly, J, X, ev.value])
        L.nqs_ansatz_free(a)
    out["exact_obc"] = dict(rows=np.array(rows))


def main():
    L = load_ref()
    out = {}
    gen_ansatz(L, out)
    gen_local_energy(L, out)
    gen_sampler(L, out)
    gen_sr(L, out)
    gen_symproj(L, out)
    gen_exact(L, out)
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print("wrote", len(out), "fixtures")


if __name__ == "__main__":
    main()
