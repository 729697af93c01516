"""The allocation-free MinSR solve (nqs_gpu_minsr_solve_noalloc) against the
regular MinSR entry point.

nqs_gpu_minsr_solve_noalloc exists for callers that cannot call cudaMalloc
(a framework that has pre-reserved the device memory for its own pool, or a
loop that must stay out of the driver's allocator); it keeps its scratch in a
static device array.  These tests feed it the Jacobian and local energies of a
batch, in device buffers owned by the caller (torch tensors here), and check
that its update equals the one nqs_gpu_sr_step_batch computes for the same
batch, to the 1e-10 relative bar of the other delta-theta tests, on two calls
in a row (the second with a different batch size, so stale scratch from the
first call would show).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_DELTA = 1e-10


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import abi, nqs
    nqs.set_options(square_pbc=1)
    yield torch, abi, nqs
    nqs.set_options()


def existing_and_noalloc(torch, abi, nqs, Ns, seed):
    Lx = Ly = 4
    N = 16
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=32, rbm_init_scale=0.3,
                              hamiltonian=abi.HAM_HEISENBERG, rng_seed=seed, sr_diag_shift=1e-3,
                              learning_rate=0.01)
    a = nqs.Ansatz(cfg, N)
    m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    rng = np.random.default_rng(seed)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(Ns)])
    # inputs of the solve, computed at the current parameters
    O = a.gradient(batch)
    E = nqs.local_energy_batch(cfg, Lx, Ly, batch, m.log_amp_fn, m.user)
    # the regular entry point (allocates its workspace, applies the update)
    info_ref, E_ref, delta_ref = nqs.sr_step_batch(cfg, Lx, Ly, a, batch, minsr=True,
                                                   log_amp_fn=m.log_amp_fn, user=m.user)
    assert np.array_equal(E, E_ref)
    # the allocation-free entry point on caller-owned device buffers
    dO = torch.from_numpy(O).cuda()
    dE = torch.from_numpy(E).cuda()
    dd = torch.full((a.P,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    info = abi.StepInfo()
    rc = nqs.lib().nqs_gpu_minsr_solve_noalloc(dO.data_ptr(), dE.data_ptr(), Ns, a.P, cfg.sr_diag_shift,
                                               dd.data_ptr(), C.byref(info), None)
    assert rc == 0, nqs.last_error()
    delta = dd.cpu().numpy()
    return delta, info, delta_ref, info_ref, cfg.learning_rate


def test_noalloc_matches_existing_entry_point_twice(env):
    torch, abi, nqs = env
    for Ns, seed in ((512, 101), (384, 202)):
        delta, info, delta_ref, info_ref, lr = existing_and_noalloc(torch, abi, nqs, Ns, seed)
        assert np.all(np.isfinite(delta))
        assert np.linalg.norm(delta - delta_ref) <= TOL_DELTA * np.linalg.norm(delta_ref)
        assert info.converged == info_ref.converged == 1
        assert info.mean_energy == pytest.approx(info_ref.mean_energy, rel=1e-12)
        assert info.variance_energy == pytest.approx(info_ref.variance_energy, rel=1e-9)
        assert info.update_norm * lr == pytest.approx(info_ref.update_norm, rel=TOL_DELTA)


def test_noalloc_rejects_sizes_beyond_its_scratch(env):
    torch, abi, nqs = env
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = nqs.lib().nqs_gpu_minsr_solve_noalloc(d.data_ptr(), d.data_ptr(), 2048, 8, 1e-3, d.data_ptr(),
                                               None, None)
    assert rc == -1
    assert "exceed the static scratch limits" in nqs.last_error()
