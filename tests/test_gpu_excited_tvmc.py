"""Excited-state SR and real-time tVMC on the GPU (through the C ABI).

Parity: one step on a caller-supplied batch against the oracle restatement
(oracle_excited_step, oracle_tvmc_step; pinned against dense solves in
tests/test_oracle_pin.py): energies to 1e-12, delta-theta to 1e-10 relative.  Physics:
the upstream unit tests' checks (tests/test_nqs_excited.c, tests/test_nqs_tvmc.c) on the
same models and settings.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu
TOL = 1e-12
TOL_DELTA = 1e-10


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    N.set_options()
    return N


def rel(a, b, floor=1.0):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def crbm(nqs, N, M, scale, seed, **kw):
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, rbm_init_scale=scale,
                              rng_seed=seed, **kw)
    return cfg, nqs.Ansatz(cfg, N)


@pytest.mark.parametrize("mu,iters,tol", [(0.5, 12, 1e-6), (2.0, 600, 1e-13)])
def test_excited_step_against_oracle(nqs, mu, iters, tol):
    """Excited-state SR on a batch: complex RBM on the 4x4 Heisenberg torus with the
    Marshall sign, reference = a second complex RBM with the Marshall sign."""
    from spin_based_neural_network_gb300 import abi
    Lx = Ly = 4
    N, M = 16, 16
    _, a = crbm(nqs, N, M, 0.3, 2718)
    _, b = crbm(nqs, N, M, 0.3, 3141)
    p0, pref = a.params.copy(), b.params.copy()
    m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    mr = nqs.Marshall(b.log_amp_fn, b.user, Lx, Ly)
    rng = np.random.default_rng(int(mu * 10) + 3)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(1024)])
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, hamiltonian=1,
                              sr_diag_shift=1e-2, learning_rate=0.02, sr_cg_max_iters=iters, sr_cg_tol=tol)
    nqs.set_options(square_pbc=1)
    try:
        info, E, delta = nqs.excited_step_batch(cfg, Lx, Ly, a, batch, mr.log_amp_fn, mr.user, mu,
                                                log_amp_fn=m.log_amp_fn, user=m.user)
    finally:
        nqs.set_options()
    amp = O.Amp(O.OR_CRBM, N, M, p0.copy(), [("marshall", Lx, Ly)])
    ref = O.Amp(O.OR_CRBM, N, M, pref.copy(), [("marshall", Lx, Ly)])
    Eo, do, io = O.excited_step(O.ham(O.OR_HEIS, Lx, Ly, pbc=1), amp, ref, mu, batch, 1e-2, 0.02, iters, tol)
    assert rel(E, Eo) < TOL                                       # augmented local energies
    assert info.mean_energy == pytest.approx(io.mean_energy, abs=1e-12)   # physical energy
    assert np.linalg.norm(delta - do) <= TOL_DELTA * np.linalg.norm(do)
    assert rel(a.params, amp.params) < TOL
    assert info.converged == io.converged


@pytest.mark.parametrize("dt,iters,tol", [(0.01, 10, 1e-6), (-0.05, 600, 1e-13)])
def test_tvmc_step_against_oracle(nqs, dt, iters, tol):
    """Forward-Euler real-time tVMC on a batch: complex RBM, 1-D TFIM N = 12 (open)."""
    from spin_based_neural_network_gb300 import abi
    N, M = 12, 12
    _, a = crbm(nqs, N, M, 0.2, 77)
    p0 = a.params.copy()
    rng = np.random.default_rng(abs(int(dt * 100)) + 1)
    batch = rng.choice(np.array([-1, 1], np.int32), size=(768, N))
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, hamiltonian=0,
                              transverse_field=0.9, sr_diag_shift=1e-3, sr_cg_max_iters=iters, sr_cg_tol=tol)
    info, E, delta = nqs.tvmc_step_batch(cfg, dt, N, 1, a, batch)
    amp = O.Amp(O.OR_CRBM, N, M, p0.copy())
    Eo, do, io = O.tvmc_step(O.ham(O.OR_TFIM, N, 1, Gamma=0.9), amp, batch, 1e-3, dt, iters, tol)
    assert rel(E, Eo) < TOL
    assert np.linalg.norm(delta - do) <= TOL_DELTA * np.linalg.norm(do)
    assert rel(a.params, amp.params) < TOL
    assert info.update_norm == pytest.approx(io.update_norm, rel=TOL_DELTA)
    assert info.converged == io.converged


def heis2_cfg(nqs, iters, seed):
    """The upstream excited-state test's model: 2-site Heisenberg, complex RBM M = 8
    (tests/test_nqs_excited.c:28-44)."""
    from spin_based_neural_network_gb300 import abi
    return abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=8, rbm_init_scale=0.05,
                               hamiltonian=1, j_coupling=1.0, num_samples=512, num_thermalize=256,
                               num_decorrelate=2, num_iterations=iters, learning_rate=0.04, sr_diag_shift=1e-2,
                               sr_cg_max_iters=80, sr_cg_tol=1e-7, rng_seed=seed)


def run_trace(nqs, fnname, cfg, a, s, *extra):
    trace = np.zeros(cfg.num_iterations)
    rc = getattr(nqs.lib(), fnname)(C.byref(cfg), 2, 1, a.h, s.h, a.log_amp_fn, a.user, *extra,
                                    trace.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    return trace


def test_excited_zero_penalty_replays_holomorphic_run(nqs):
    """mu = 0: the same sampler stream and the same updates as nqs_sr_run_holomorphic, so
    the energy traces agree exactly (upstream tests/test_nqs_excited.c:48-105 asks for the
    tail means to agree within 0.05)."""
    cfg = heis2_cfg(nqs, 200, 0x2222)
    a_h = nqs.Ansatz(cfg, 2)
    s_h = nqs.Sampler(2, cfg, a_h.log_amp_fn, a_h.user)
    t_h = run_trace(nqs, "nqs_sr_run_holomorphic", cfg, a_h, s_h)
    ref = nqs.Ansatz(heis2_cfg(nqs, 0, 0xEB1), 2)
    a_e = nqs.Ansatz(cfg, 2)
    s_e = nqs.Sampler(2, cfg, a_e.log_amp_fn, a_e.user)
    t_e = run_trace(nqs, "nqs_sr_run_excited", cfg, a_e, s_e, ref.log_amp_fn, ref.user, C.c_double(0.0))
    assert np.all(np.isfinite(t_h))
    assert np.array_equal(t_h, t_e)
    assert abs(t_h[-20:].mean() - t_e[-20:].mean()) < 0.05


def test_excited_penalty_drives_energy_above_ground_state(nqs):
    """2-site Heisenberg (E0 = -0.75, E1 = +0.25): a reference pretrained to the singlet,
    then excited SR with penalty 5 ends at least 0.5 above it and below +0.7 (upstream
    tests/test_nqs_excited.c:107-175)."""
    cfg_ref = heis2_cfg(nqs, 400, 0x2222)
    a_ref = nqs.Ansatz(cfg_ref, 2)
    s_ref = nqs.Sampler(2, cfg_ref, a_ref.log_amp_fn, a_ref.user)
    t_ref = run_trace(nqs, "nqs_sr_run_holomorphic", cfg_ref, a_ref, s_ref)
    E_ref = t_ref[-20:].mean()
    cfg = heis2_cfg(nqs, 400, 0xEB3)
    cfg.learning_rate = 0.03
    cfg.sr_diag_shift = 5e-3
    a = nqs.Ansatz(cfg, 2)
    s = nqs.Sampler(2, cfg, a.log_amp_fn, a.user)
    t = run_trace(nqs, "nqs_sr_run_excited", cfg, a, s, a_ref.log_amp_fn, a_ref.user, C.c_double(5.0))
    E_exc = t[-20:].mean()
    assert np.all(np.isfinite(t))
    assert E_ref < -0.4
    assert E_ref + 0.5 < E_exc < 0.7


def tfim4_cfg(seed, samples=2048, lr=0.01):
    """The upstream tVMC tests' model: 4-site TFIM, J = h = 1, complex RBM M = 8
    (tests/test_nqs_tvmc.c:49-70)."""
    from spin_based_neural_network_gb300 import abi
    return abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=8, rbm_init_scale=0.08,
                               hamiltonian=0, j_coupling=1.0, transverse_field=1.0, num_samples=samples,
                               num_thermalize=512, num_decorrelate=2, sr_diag_shift=1e-3, sr_cg_max_iters=40,
                               sr_cg_tol=1e-6, rng_seed=seed, learning_rate=lr)


def measured_energy(nqs, cfg, a, s):
    c = type(cfg).from_buffer_copy(cfg)
    c.num_samples = 4096
    return np.mean([nqs.tvmc_step(c, 0.0, 4, 1, a, s).mean_energy for _ in range(4)])


@pytest.mark.parametrize("heun,dt,steps", [(False, 0.01, 20), (False, 0.02, 15), (True, 0.02, 15)])
def test_tvmc_conserves_energy(nqs, heun, dt, steps):
    """Unitary evolution conserves <H>: |E(T) - E(0)| < 0.5 after T = 0.2-0.3 with Euler
    and with Heun (upstream tests/test_nqs_tvmc.c:49-94, :154-227)."""
    cfg = tfim4_cfg(0xA1A1 if dt == 0.01 else 0xC3C3)
    a = nqs.Ansatz(cfg, 4)
    s = nqs.Sampler(4, cfg, a.log_amp_fn, a.user)
    s.thermalize()
    e0 = measured_energy(nqs, cfg, a, s)
    p0 = a.params.copy()
    for _ in range(steps):
        info = nqs.tvmc_step(cfg, dt, 4, 1, a, s, heun=heun)
        assert np.isfinite(info.mean_energy) and info.update_norm >= 0.0
    e1 = measured_energy(nqs, cfg, a, s)
    assert np.isfinite(e1) and abs(e1 - e0) < 0.5
    assert np.linalg.norm(a.params - p0) > 0.0


def test_real_time_differs_from_imaginary_time(nqs):
    """Holomorphic SR descends to the ground state (E0 = -4.75) while the real-time
    evolution stays near the initial energy (upstream tests/test_nqs_tvmc.c:96-144)."""
    cfg = tfim4_cfg(0xB2B2, samples=1024, lr=0.05)
    cfg.sr_diag_shift = 1e-2
    a_im, a_rt = nqs.Ansatz(cfg, 4), nqs.Ansatz(cfg, 4)
    s_im = nqs.Sampler(4, cfg, a_im.log_amp_fn, a_im.user)
    s_rt = nqs.Sampler(4, cfg, a_rt.log_amp_fn, a_rt.user)
    s_im.thermalize()
    s_rt.thermalize()
    for _ in range(25):
        e_im = nqs.sr_step_holomorphic(cfg, 4, 1, a_im, s_im, a_im.log_amp_fn, a_im.user).mean_energy
        e_rt = nqs.tvmc_step(cfg, 0.01, 4, 1, a_rt, s_rt).mean_energy
    assert e_im < e_rt - 0.5 and e_im < -1.5


def test_null_arguments_return_error(nqs):
    """Null configuration / ansatz / sampler / reference: -1 (upstream
    tests/test_nqs_tvmc.c:146-153)."""
    L = nqs.lib()
    cfg = tfim4_cfg(1, samples=32)
    a = nqs.Ansatz(cfg, 4)
    s = nqs.Sampler(4, cfg, a.log_amp_fn, a.user)
    assert L.nqs_tvmc_step_real_time(None, 0.01, 4, 1, a.h, s.h, None, None, None) == -1
    assert L.nqs_tvmc_step_heun(C.byref(cfg), 0.01, 4, 1, None, s.h, None, None, None) == -1
    assert L.nqs_sr_step_excited(C.byref(cfg), 4, 1, a.h, s.h, None, None, None, None, 1.0, None) == -1
