"""The holomorphic SR family on the GPU against the upstream library's own outputs.

Fixtures (tests/golden/make_holo_golden.py) were written by the upstream
nqs_sr_step_holomorphic_full, nqs_sr_step_excited, nqs_tvmc_step_real_time and
nqs_tvmc_step_heun (src/nqs/nqs_optimizer.c:415-524, 562-723, 830-993) with the
upstream sampler.  Two checks per fixture, both through the C ABI:

* identical batch: the batch the upstream step drew, replayed through the
  batched entry points (nqs_gpu_sr_step_batch with minsr = 2,
  nqs_gpu_sr_step_batch_excited, nqs_gpu_tvmc_step_batch);
* drop-in: the library's own step function with the compat sampler created
  from the same seed, which replays the upstream Markov chain, so the whole
  call (sampling, estimator, gradient, CG, update) lands on the upstream
  parameters.

Bars: mean energy 1e-12 relative, parameter update 1e-10 relative (2-norm);
CG is capped at 10 iterations or converged to 1e-13, so these bars hold.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12
TOL_DELTA = 1e-10
HOLO = ["holo_heis_crbm_marshall", "holo_tfim_crbm_converged", "holo_kagome2x2_p2_symproj"]
EXCITED = ["excited_tfim_crbm", "excited_tfim_crbm_converged"]


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    N.set_options()                      # compat sampler, open lattices, FP64
    return N


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def fixture_cfg(d, **over):
    from spin_based_neural_network_gb300 import abi
    kw = dict(ansatz=int(d["kind"]), rbm_hidden_units=int(d["M"]), rbm_init_scale=float(d["init_scale"]),
              hamiltonian=int(d["ham"]), j_coupling=float(d["J"]), j2_coupling=float(d["J2"]),
              j_z_coupling=float(d["Jz"]), transverse_field=float(d["Gamma"]), kagome_pbc=int(d["kagome_pbc"]),
              rng_seed=int(d["seed"]), num_samples=int(d["Ns"]), num_thermalize=int(d["therm"]),
              num_decorrelate=int(d["decor"]), sr_diag_shift=float(d["shift"]), learning_rate=float(d["lr"]),
              sr_cg_max_iters=int(d["cg_max"]), sr_cg_tol=float(d["cg_tol"]))
    kw.update(over)
    return abi.config_defaults(**kw)


class Problem:
    """The library's ansatz for a fixture (initialised from the fixture's seed, which
    must reproduce the upstream parameters bit for bit) and its amplitude program."""

    def __init__(self, nqs, d, seed=None, params=None):
        self.cfg = fixture_cfg(d, **({} if seed is None else {"rng_seed": seed}))
        self.a = nqs.Ansatz(self.cfg, int(d["N"]))
        if params is not None:
            assert np.array_equal(self.a.params, params)
        self.fn, self.user = self.a.log_amp_fn, self.a.user
        self.gfn = self.guser = None
        wrap = str(d["wrap"])
        if wrap == "marshall":
            self.w = nqs.Marshall(self.fn, self.user, int(d["Lx"]), int(d["Ly"]))
            self.fn, self.user = self.w.log_amp_fn, self.w.user
        elif wrap == "symproj":
            self.w = nqs.Symproj(self.fn, self.user, int(d["N"]), d["perm"], d["chars"])
            self.fn, self.user = self.w.log_amp_fn, self.w.user
            if int(d.get("sym_grad", 0)):
                self.gfn, self.guser = self.w.gradient_complex_fn, self.w.user


def check(d, info, params, E=None):
    ref = d["info"]
    step = d["params1"] - d["params0"]
    assert np.linalg.norm((params - d["params0"]) - step) <= TOL_DELTA * np.linalg.norm(step)
    assert info.mean_energy == pytest.approx(ref[0], rel=TOL)
    assert info.variance_energy == pytest.approx(ref[1], rel=1e-9, abs=1e-12)
    assert info.update_norm == pytest.approx(ref[2], rel=TOL_DELTA)
    assert info.converged == int(ref[5])
    if int(ref[5]) and int(d["cg_max"]) > int(ref[4]):
        # converged to 1e-13: the last iterations sit at the rounding level, where the
        # summation order moves the crossing of the threshold by an iteration or two
        assert abs(info.cg_iterations - int(ref[4])) <= 3
    else:
        assert info.cg_iterations == int(ref[4])


@pytest.mark.parametrize("name", HOLO)
def test_holomorphic_on_upstream_batch(nqs, name):
    d = load(name)
    pb = Problem(nqs, d, params=d["params0"])
    info, E, delta = nqs.sr_step_batch(pb.cfg, int(d["Lx"]), int(d["Ly"]), pb.a, d["batch"], minsr=2,
                                       log_amp_fn=pb.fn, user=pb.user, grad_fn=pb.gfn, grad_user=pb.guser)
    check(d, info, pb.a.params)


@pytest.mark.parametrize("name", HOLO)
def test_holomorphic_dropin_step(nqs, name):
    d = load(name)
    pb = Problem(nqs, d, params=d["params0"])
    s = nqs.Sampler(int(d["N"]), pb.cfg, pb.fn, pb.user)
    s.thermalize()
    info = nqs.sr_step_holomorphic(pb.cfg, int(d["Lx"]), int(d["Ly"]), pb.a, s, pb.fn, pb.user, pb.gfn, pb.guser)
    check(d, info, pb.a.params)
    assert info.acceptance_ratio == pytest.approx(float(d["info"][3]), abs=0)


@pytest.mark.parametrize("name", EXCITED)
def test_excited_on_upstream_batch(nqs, name):
    d = load(name)
    pb = Problem(nqs, d, params=d["params0"])
    ref = Problem(nqs, d, seed=int(d["ref_seed"]), params=d["params_ref"])
    info, E, delta = nqs.excited_step_batch(pb.cfg, int(d["Lx"]), int(d["Ly"]), pb.a, d["batch"], ref.fn, ref.user,
                                            float(d["mu"]), log_amp_fn=pb.fn, user=pb.user)
    check(d, info, pb.a.params)


@pytest.mark.parametrize("name", EXCITED)
def test_excited_dropin_step(nqs, name):
    d = load(name)
    pb = Problem(nqs, d, params=d["params0"])
    ref = Problem(nqs, d, seed=int(d["ref_seed"]), params=d["params_ref"])
    s = nqs.Sampler(int(d["N"]), pb.cfg, pb.fn, pb.user)
    s.thermalize()
    info = nqs.sr_step_excited(pb.cfg, int(d["Lx"]), int(d["Ly"]), pb.a, s, ref.fn, ref.user, float(d["mu"]),
                               pb.fn, pb.user)
    check(d, info, pb.a.params)


def test_tvmc_euler_on_upstream_batch(nqs):
    d = load("tvmc_euler_tfim_crbm")
    pb = Problem(nqs, d, params=d["params0"])
    info, E, delta = nqs.tvmc_step_batch(pb.cfg, float(d["dt"]), int(d["Lx"]), int(d["Ly"]), pb.a, d["batch"],
                                         pb.fn, pb.user)
    check(d, info, pb.a.params)


def test_tvmc_heun_on_upstream_batches(nqs):
    """Heun from two Euler forces on the upstream step's two batches: k1 at theta on the
    first, k2 at the probe theta + dt k1 on the second, theta + dt (k1 + k2) / 2."""
    d = load("tvmc_heun_tfim_crbm")
    dt = float(d["dt"])
    pb = Problem(nqs, d, params=d["params0"])
    Lx, Ly = int(d["Lx"]), int(d["Ly"])
    i1, _, k1 = nqs.tvmc_step_batch(pb.cfg, dt, Lx, Ly, pb.a, d["batch"], pb.fn, pb.user)
    probe = pb.a.params.copy()
    assert np.linalg.norm(probe - d["params_probe"]) <= TOL * np.linalg.norm(d["params_probe"])
    i2, _, k2 = nqs.tvmc_step_batch(pb.cfg, dt, Lx, Ly, pb.a, d["batch2"], pb.fn, pb.user)
    final = d["params0"] + dt * (0.5 * (k1 + k2))
    step = d["params1"] - d["params0"]
    assert np.linalg.norm((final - d["params0"]) - step) <= TOL_DELTA * np.linalg.norm(step)
    assert i1.mean_energy == pytest.approx(float(d["info"][0]), rel=TOL)
    assert i1.cg_iterations + i2.cg_iterations == int(d["info"][4])


@pytest.mark.parametrize("name,heun", [("tvmc_euler_tfim_crbm", False), ("tvmc_heun_tfim_crbm", True)])
def test_tvmc_dropin_step(nqs, name, heun):
    d = load(name)
    pb = Problem(nqs, d, params=d["params0"])
    s = nqs.Sampler(int(d["N"]), pb.cfg, pb.fn, pb.user)
    s.thermalize()
    info = nqs.tvmc_step(pb.cfg, float(d["dt"]), int(d["Lx"]), int(d["Ly"]), pb.a, s, pb.fn, pb.user, heun=heun)
    check(d, info, pb.a.params)
    assert info.acceptance_ratio == pytest.approx(float(d["info"][3]), abs=0)


@pytest.mark.parametrize("name", ["run_minsr_heis_crbm_marshall", "run_holo_tfim_crbm"])
def test_run_with_compat_sampler_matches_upstream(nqs, name):
    """Five iterations of nqs_sr_run_minsr / nqs_sr_run_holomorphic with the compat sampler
    against the upstream run: energy trace and final parameters.  Between iterations the
    upstream sampler compares proposals with the log|psi| it cached at the previous
    parameters until its next accepted move; the compat chain must do the same for the
    runs to draw the same samples."""
    import ctypes as C
    d = load(name)
    pb = Problem(nqs, d, params=d["params0"])
    pb.cfg.num_iterations = int(d["iterations"])
    s = nqs.Sampler(int(d["N"]), pb.cfg, pb.fn, pb.user)
    trace = np.zeros(int(d["iterations"]))
    f = nqs.lib().nqs_sr_run_minsr if str(d["solver"]) == "minsr" else nqs.lib().nqs_sr_run_holomorphic
    rc = f(C.byref(pb.cfg), int(d["Lx"]), int(d["Ly"]), pb.a.h, s.h, pb.fn, pb.user,
           trace.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0, nqs.last_error()
    np.testing.assert_allclose(trace, d["trace"], rtol=1e-11, atol=0)
    step = d["params1"] - d["params0"]
    assert np.linalg.norm((pb.a.params - d["params0"]) - step) <= 1e-9 * np.linalg.norm(step)
    assert s.acceptance_ratio() == pytest.approx(float(d["acceptance"]), abs=0)


# ------------------------------------------------------------------ holomorphic MinSR
# nqs_sr_step_minsr_holomorphic_full solves the upstream holomorphic SR system by MinSR on
# the stacked rows [R_c; I_c].  Its update must equal the converged holomorphic CG-SR update
# of the oracle (pinned above against nqs_sr_step_holomorphic_full) on the same batch.

def _holo_minsr_case(nqs, Ns, M=16, seed=2718):
    import oracle_lib as O
    from spin_based_neural_network_gb300 import abi
    Lx = Ly = 4
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, rbm_init_scale=0.3, rng_seed=seed,
                              hamiltonian=abi.HAM_HEISENBERG, sr_diag_shift=1e-2, learning_rate=0.01,
                              sr_cg_max_iters=2000, sr_cg_tol=1e-13)
    a = nqs.Ansatz(cfg, 16)
    m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    rng = np.random.default_rng(Ns + seed)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(Ns)])
    amp = O.Amp(O.OR_CRBM, 16, M, a.params.copy(), [("marshall", Lx, Ly)])
    Eo, do, io = O.holo_step(O.ham(O.OR_HEIS, Lx, Ly, pbc=1), amp, batch, cfg.sr_diag_shift, cfg.learning_rate,
                             cfg.sr_cg_max_iters, cfg.sr_cg_tol)
    assert io.converged == 1
    return cfg, a, m, batch, Eo, do, io


@pytest.mark.parametrize("Ns,prec,space,bar", [(512, "fp64", "samples", 1e-9), (512, "fp64", "parameters", 1e-9),
                                               (256, "fp64", "parameters", 1e-9), (512, "mixed", "auto", 1e-6)])
def test_holomorphic_minsr_equals_converged_holomorphic_sr(nqs, Ns, prec, space, bar):
    """Complex RBM (N_p = 576) on the 4x4 Heisenberg torus with the Marshall sign: 2 N_s = 1024
    or 512 stacked rows, sample- or parameter-space solve, FP64 or the mixed path."""
    from spin_based_neural_network_gb300 import abi
    cfg, a, m, batch, Eo, do, io = _holo_minsr_case(nqs, Ns)
    opts = dict(square_pbc=1)
    if prec == "mixed":
        opts.update(precision=abi.PREC_MIXED, refine_sweeps=20)
    else:
        opts.update(fp64_space=abi.SPACE_PARAMETERS if space == "parameters" else 0)
    nqs.set_options(**opts)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, 4, 4, a, batch, minsr=5, log_amp_fn=m.log_amp_fn, user=m.user)
    finally:
        nqs.set_options()
    assert info.converged == 1 and info.cg_iterations == 0
    assert np.max(np.abs(E - Eo) / np.maximum(np.abs(Eo), 1.0)) < TOL
    assert info.mean_energy == pytest.approx(io.mean_energy, rel=TOL)
    assert np.linalg.norm(delta - do) <= bar * np.linalg.norm(do)


def test_holomorphic_minsr_of_a_real_rbm_is_minsr_at_half_shift(nqs):
    """For a real RBM the imaginary rows vanish, so the holomorphic system is 2 R_c^T R_c / N_s
    + shift I and its update equals the MinSR update with shift / 2."""
    from spin_based_neural_network_gb300 import abi
    N, M = 16, 16
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=M, rbm_init_scale=0.3, rng_seed=5,
                              hamiltonian=abi.HAM_TFIM, transverse_field=0.9, sr_diag_shift=2e-3, learning_rate=0.01)
    rng = np.random.default_rng(9)
    batch = np.where(rng.random((384, N)) < 0.5, 1, -1).astype(np.int32)
    a1 = nqs.Ansatz(cfg, N)
    i1, E1, d1 = nqs.sr_step_batch(cfg, 4, 4, a1, batch, minsr=5)
    cfg2 = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=M, rbm_init_scale=0.3, rng_seed=5,
                               hamiltonian=abi.HAM_TFIM, transverse_field=0.9, sr_diag_shift=1e-3, learning_rate=0.01)
    a2 = nqs.Ansatz(cfg2, N)
    i2, E2, d2 = nqs.sr_step_batch(cfg2, 4, 4, a2, batch, minsr=1)
    assert np.array_equal(E1, E2)
    assert np.linalg.norm(d1 - d2) <= 1e-10 * np.linalg.norm(d2)


def test_holomorphic_minsr_step_with_sampler(nqs):
    """The sampled step (nqs_sr_step_minsr_holomorphic_full) lowers the energy of the complex
    RBM on the 4x4 Heisenberg torus over a short run (nqs_sr_run_minsr_holomorphic)."""
    import ctypes as C
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=16, rbm_init_scale=0.05, rng_seed=9,
                              hamiltonian=abi.HAM_HEISENBERG, num_samples=1024, num_iterations=40,
                              sr_diag_shift=1e-3, learning_rate=0.02)
    a = nqs.Ansatz(cfg, 16)
    m = nqs.Marshall(a.log_amp_fn, a.user, 4, 4)
    o = nqs.options(num_chains=256, rng=abi.RNG_PHILOX, move=abi.MOVE_EXCHANGE, n_down=8, lattice_x=4, lattice_y=4,
                    square_pbc=1)
    nqs.set_options(square_pbc=1)
    try:
        s = nqs.Sampler(16, cfg, m.log_amp_fn, m.user, o)
        trace = np.zeros(40)
        rc = nqs.lib().nqs_sr_run_minsr_holomorphic(C.byref(cfg), 4, 4, a.h, s.h, m.log_amp_fn, m.user,
                                                    trace.ctypes.data_as(C.POINTER(C.c_double)))
    finally:
        nqs.set_options()
    assert rc == 0 and np.all(np.isfinite(trace))
    assert np.mean(trace[-5:]) < np.mean(trace[:5]) - 0.5
