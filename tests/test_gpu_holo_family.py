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
