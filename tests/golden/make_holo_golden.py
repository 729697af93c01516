"""Golden vectors for the holomorphic SR family, written by the upstream library itself.

Drives oracle/_ref/libnqs_ref.so (built from the upstream sources by
`make -C oracle REF=<upstream checkout>`) through its public API:

  nqs_sr_step_holomorphic_full   (src/nqs/nqs_optimizer.c:415-524), with the base
                                  ansatz's gradient and with nqs_symproj_gradient_complex
  nqs_sr_step_excited            (src/nqs/nqs_optimizer.c:562-723)
  nqs_tvmc_step_real_time        (src/nqs/nqs_optimizer.c:895-993)
  nqs_tvmc_step_heun             (src/nqs/nqs_optimizer.c:830-886)

Each fixture holds the initial and final parameters, the step info and the
batches the step consumed.  The batches come from twin samplers: the upstream
sampler is a deterministic function of its seed and of the amplitudes it sees,
so a second sampler created with the same seed, thermalised and batched, yields
the batch the step drew.  Heun samples twice: its second batch is drawn at the
probe parameters theta + dt k1, which a twin ansatz reaches by one Euler step
(the same call Heun makes for k1); the twin sampler's next batch is then the
second batch.  CG is capped at a few iterations (or driven to a 1e-13
residual on a well-conditioned system) so that the 1e-10 parity bar on the
update is meaningful: a capped CG amplifies summation-order differences only
slightly, a converged one not at all.  Two 5-iteration runs (nqs_sr_run_minsr,
nqs_sr_run_holomorphic) record energy traces and final parameters.

Runs here only; writes tests/golden/{holo,excited,tvmc,run}_*.npz.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from spin_based_neural_network_gb300 import abi  # noqa: E402
from make_golden import DP, IP, fnptr, load_ref, params_of  # noqa: E402

HOLO_GRAD_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, IP, C.c_int, DP, DP)


def declare(L):
    step = [C.POINTER(abi.NqsConfig), C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqs_sr_step_holomorphic_full.argtypes = step + [C.c_void_p, C.c_void_p, C.POINTER(abi.StepInfo)]
    L.nqs_sr_step_excited.argtypes = step + [C.c_void_p, C.c_void_p, C.c_double, C.POINTER(abi.StepInfo)]
    tv = [C.POINTER(abi.NqsConfig), C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
          C.c_void_p, C.POINTER(abi.StepInfo)]
    L.nqs_tvmc_step_real_time.argtypes = tv
    L.nqs_tvmc_step_heun.argtypes = tv


def info_row(info):
    return np.array([info.mean_energy, info.variance_energy, info.update_norm, info.acceptance_ratio,
                     info.cg_iterations, info.converged])


class Problem:
    """An upstream ansatz, its amplitude callback (plain, Marshall or a symmetry
    projection) and samplers on it."""

    def __init__(self, L, cfg, N, Lx, Ly, wrap=None, group=None):
        self.L, self.cfg, self.N = L, cfg, N
        self.a = L.nqs_ansatz_create(C.byref(cfg), N)
        self.keep = []
        self.fn, self.user = fnptr(L, "nqs_ansatz_log_amp"), self.a
        self.perm = self.chars = None
        if wrap == "marshall":
            w = abi.MarshallWrapper(self.fn, self.a, Lx, Ly)
            self.keep.append(w)
            self.fn, self.user = fnptr(L, "nqs_marshall_log_amp"), C.addressof(w)
        elif wrap == "symproj":
            perm, chars, G = IP(), DP(), C.c_int()
            assert L.nqs_kagome_p2_perm(Lx, Ly, C.byref(perm), C.byref(chars), C.byref(G)) == 0
            self.perm = np.ascontiguousarray(np.ctypeslib.as_array(perm, shape=(G.value * N,)).astype(np.int32))
            self.chars = np.ascontiguousarray(np.ctypeslib.as_array(chars, shape=(G.value,)).copy())
            w = abi.SymprojWrapper(self.fn, self.a, N, G.value, self.perm.ctypes.data_as(IP),
                                   self.chars.ctypes.data_as(DP))
            self.keep.append(w)
            self.fn, self.user = fnptr(L, "nqs_symproj_log_amp"), C.addressof(w)

    def sampler(self):
        s = self.L.nqs_sampler_create(self.N, C.byref(self.cfg), self.fn, self.user)
        self.L.nqs_sampler_thermalize(s)
        return s

    def batch(self, s, n):
        out = np.zeros((n, self.N), dtype=np.int32)
        self.L.nqs_sampler_batch(s, n, out.ctypes.data_as(IP))
        return out

    def params(self):
        return params_of(self.L, self.a)

    def free(self, *samplers):
        for s in samplers:
            self.L.nqs_sampler_free(s)
        self.L.nqs_ansatz_free(self.a)


def make_cfg(kind, M, ham, Ns, shift, lr, cg_max, cg_tol, seed, **kw):
    return abi.config_defaults(ansatz=kind, rbm_hidden_units=M, rbm_init_scale=0.3, hamiltonian=ham,
                               rng_seed=seed, num_samples=Ns, num_thermalize=64, num_decorrelate=2,
                               sr_diag_shift=shift, learning_rate=lr, sr_cg_max_iters=cg_max, sr_cg_tol=cg_tol,
                               **kw)


def common(cfg, N, Lx, Ly, kind, M, ham, wrap):
    return dict(N=N, Lx=Lx, Ly=Ly, kind=kind, M=M, ham=ham, J=cfg.j_coupling, J2=cfg.j2_coupling,
                Jz=cfg.j_z_coupling, Gamma=cfg.transverse_field, kagome_pbc=cfg.kagome_pbc,
                Ns=cfg.num_samples, shift=cfg.sr_diag_shift, lr=cfg.learning_rate, cg_max=cfg.sr_cg_max_iters,
                cg_tol=cfg.sr_cg_tol, seed=cfg.rng_seed, therm=cfg.num_thermalize, decor=cfg.num_decorrelate,
                init_scale=cfg.rbm_init_scale, wrap=wrap or "")


def gen_holo(L, out):
    """nqs_sr_step_holomorphic_full: complex RBM on the open 4x4 Heisenberg lattice with the
    Marshall sign (CG capped at 10), a TFIM chain driven to convergence, and the p2-projected
    complex RBM on the periodic 2x2 kagome lattice with nqs_symproj_gradient_complex."""
    cases = [
        ("holo_heis_crbm_marshall", abi.HAM_HEISENBERG, 4, 4, 16, abi.ANSATZ_COMPLEX_RBM, 16, "marshall",
         dict(Ns=512, shift=1e-3, lr=0.01, cg_max=10, cg_tol=1e-6), {}, False),
        ("holo_tfim_crbm_converged", abi.HAM_TFIM, 8, 1, 8, abi.ANSATZ_COMPLEX_RBM, 8, None,
         dict(Ns=1024, shift=1e-2, lr=0.02, cg_max=3000, cg_tol=1e-13), dict(transverse_field=0.8), False),
        ("holo_kagome2x2_p2_symproj", abi.HAM_KAGOME_HEISENBERG, 2, 2, 12, abi.ANSATZ_COMPLEX_RBM, 12, "symproj",
         dict(Ns=256, shift=1e-2, lr=0.01, cg_max=10, cg_tol=1e-6), dict(kagome_pbc=1), True),
    ]
    for name, ham, Lx, Ly, N, kind, M, wrap, sr, extra, sym_grad in cases:
        cfg = make_cfg(kind, M, ham, sr["Ns"], sr["shift"], sr["lr"], sr["cg_max"], sr["cg_tol"], 31337, **extra)
        pb = Problem(L, cfg, N, Lx, Ly, wrap)
        twin = Problem(L, cfg, N, Lx, Ly, wrap)
        tws = twin.sampler()
        batch = twin.batch(tws, sr["Ns"])
        p0 = pb.params()
        s = pb.sampler()
        info = abi.StepInfo()
        gfn, guser = (fnptr(L, "nqs_symproj_gradient_complex"), pb.user) if sym_grad else (None, None)
        assert L.nqs_sr_step_holomorphic_full(C.byref(cfg), Lx, Ly, pb.a, s, pb.fn, pb.user, gfn, guser,
                                              C.byref(info)) == 0
        d = common(cfg, N, Lx, Ly, kind, M, ham, wrap)
        d.update(params0=p0, params1=pb.params(), batch=batch, info=info_row(info), sym_grad=int(sym_grad))
        if pb.perm is not None:
            d.update(perm=pb.perm, chars=pb.chars)
        out[name] = d
        pb.free(s)
        twin.free(tws)


def gen_excited(L, out):
    """nqs_sr_step_excited: complex RBM on a TFIM chain against a reference complex RBM from
    another seed, penalty mu = 0.7; CG capped at 10 and driven to convergence."""
    N, M = 8, 8
    for name, cg_max, cg_tol, Ns in (("excited_tfim_crbm", 10, 1e-6, 512),
                                      ("excited_tfim_crbm_converged", 3000, 1e-13, 1024)):
        cfg = make_cfg(abi.ANSATZ_COMPLEX_RBM, M, abi.HAM_TFIM, Ns, 1e-2, 0.02, cg_max, cg_tol, 4242,
                       transverse_field=0.9)
        ref_cfg = make_cfg(abi.ANSATZ_COMPLEX_RBM, M, abi.HAM_TFIM, Ns, 1e-2, 0.02, cg_max, cg_tol, 777,
                           transverse_field=0.9)
        ref = Problem(L, ref_cfg, N, N, 1)
        pb = Problem(L, cfg, N, N, 1)
        twin = Problem(L, cfg, N, N, 1)
        tws = twin.sampler()
        batch = twin.batch(tws, Ns)
        p0 = pb.params()
        s = pb.sampler()
        info = abi.StepInfo()
        mu = 0.7
        assert L.nqs_sr_step_excited(C.byref(cfg), N, 1, pb.a, s, pb.fn, pb.user, ref.fn, ref.user, mu,
                                     C.byref(info)) == 0
        d = common(cfg, N, N, 1, abi.ANSATZ_COMPLEX_RBM, M, abi.HAM_TFIM, None)
        d.update(params0=p0, params1=pb.params(), params_ref=ref.params(), ref_seed=777, mu=mu, batch=batch,
                 info=info_row(info))
        out[name] = d
        pb.free(s)
        twin.free(tws)
        ref.free()


def gen_tvmc(L, out):
    """nqs_tvmc_step_real_time (forward Euler) and nqs_tvmc_step_heun on a TFIM chain with a
    complex RBM, dt = 0.01, CG capped at 10 iterations."""
    N, M, Ns, dt = 8, 8, 512, 0.01
    for name, heun in (("tvmc_euler_tfim_crbm", False), ("tvmc_heun_tfim_crbm", True)):
        cfg = make_cfg(abi.ANSATZ_COMPLEX_RBM, M, abi.HAM_TFIM, Ns, 1e-2, 0.0, 10, 1e-6, 9001,
                       transverse_field=1.1)
        pb = Problem(L, cfg, N, N, 1)
        first = Problem(L, cfg, N, N, 1)          # yields the first batch
        fs = first.sampler()
        batch1 = first.batch(fs, Ns)
        p0 = pb.params()
        s = pb.sampler()
        info = abi.StepInfo()
        f = L.nqs_tvmc_step_heun if heun else L.nqs_tvmc_step_real_time
        assert f(C.byref(cfg), dt, N, 1, pb.a, s, pb.fn, pb.user, C.byref(info)) == 0
        d = common(cfg, N, N, 1, abi.ANSATZ_COMPLEX_RBM, M, abi.HAM_TFIM, None)
        d.update(params0=p0, params1=pb.params(), dt=dt, heun=int(heun), batch=batch1, info=info_row(info))
        if heun:
            # the probe: one Euler step from theta (Heun's k1 call), then the next batch
            probe = Problem(L, cfg, N, N, 1)
            ps = probe.sampler()
            pinfo = abi.StepInfo()
            assert L.nqs_tvmc_step_real_time(C.byref(cfg), dt, N, 1, probe.a, ps, probe.fn, probe.user,
                                             C.byref(pinfo)) == 0
            d.update(batch2=probe.batch(ps, Ns), params_probe=probe.params())
            probe.free(ps)
        out[name] = d
        pb.free(s)
        first.free(fs)


def gen_runs(L, out):
    """nqs_sr_run_minsr and nqs_sr_run_holomorphic over 5 iterations with the upstream sampler:
    the energy trace and the final parameters.  After each update the upstream sampler keeps
    the log|psi| it cached at the old parameters until its next accepted move, so a run checks
    that the compat chain reproduces that across steps."""
    run = [C.POINTER(abi.NqsConfig), C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
           C.POINTER(C.c_double)]
    L.nqs_sr_run_minsr.argtypes = run
    L.nqs_sr_run_holomorphic.argtypes = run
    cases = [("run_minsr_heis_crbm_marshall", "minsr", abi.HAM_HEISENBERG, 4, 4, abi.ANSATZ_COMPLEX_RBM, 16,
              dict(Ns=256, shift=1e-3, lr=0.01, cg_max=100, cg_tol=1e-6)),
             ("run_holo_tfim_crbm", "holo", abi.HAM_TFIM, 8, 1, abi.ANSATZ_COMPLEX_RBM, 8,
              dict(Ns=256, shift=1e-2, lr=0.02, cg_max=10, cg_tol=1e-6))]
    for name, solver, ham, Lx, Ly, kind, M, sr in cases:
        cfg = make_cfg(kind, M, ham, sr["Ns"], sr["shift"], sr["lr"], sr["cg_max"], sr["cg_tol"], 2718,
                       transverse_field=0.9)
        cfg.num_iterations = 5
        wrap = "marshall" if ham == abi.HAM_HEISENBERG else None
        pb = Problem(L, cfg, Lx * Ly, Lx, Ly, wrap)
        p0 = pb.params()
        s = L.nqs_sampler_create(pb.N, C.byref(cfg), pb.fn, pb.user)   # the run thermalises it
        trace = np.zeros(5)
        f = L.nqs_sr_run_minsr if solver == "minsr" else L.nqs_sr_run_holomorphic
        assert f(C.byref(cfg), Lx, Ly, pb.a, s, pb.fn, pb.user, trace.ctypes.data_as(DP)) == 0
        d = common(cfg, Lx * Ly, Lx, Ly, kind, M, ham, wrap)
        d.update(params0=p0, params1=pb.params(), trace=trace, solver=solver, iterations=5,
                 acceptance=L.nqs_sampler_acceptance_ratio(s))
        out[name] = d
        pb.free(s)


def main():
    L = load_ref()
    declare(L)
    out = {}
    gen_holo(L, out)
    gen_excited(L, out)
    gen_tvmc(L, out)
    gen_runs(L, out)
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, "info", d.get("info", d.get("trace")))
    print("wrote", len(out), "fixtures")


if __name__ == "__main__":
    main()
