"""The allocation-free MinSR solve (nqs_gpu_minsr_solve_noalloc) against the
regular MinSR entry point.

nqs_gpu_minsr_solve_noalloc exists for callers that cannot call cudaMalloc
(a framework that has pre-reserved the device memory for its own pool, or a
loop that must stay out of the driver's allocator); it keeps its scratch in a
static device array.  These tests feed it the Jacobian and local energies of a
batch, in device buffers owned by the caller (torch tensors here), and check
that its update equals the one nqs_gpu_sr_step_batch computes for the same
batch, to the 1e-10 relative bar of the other delta-theta tests, on calls in a
row with different shapes (so stale scratch from an earlier call would show):
tile-aligned sizes, sizes that leave partial tiles (N_s = 1000, N_p = 270 and
474, not multiples of the 64-wide Gram tile, the 32-wide factor block or 16),
and N_s at its 1024 limit.  Every call after the first must leave the device's
free memory unchanged (nothing allocated).  This file is collected last on
purpose.
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


def existing_and_noalloc(torch, abi, nqs, Ns, seed, M=32, free_bytes=None):
    """The regular step's update and the allocation-free solve's on the same batch.  With
    free_bytes (a list), the device's free memory just before and just after the
    allocation-free call is appended to it."""
    Lx = Ly = 4
    N = 16
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, rbm_init_scale=0.3,
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
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    info = abi.StepInfo()
    rc = nqs.lib().nqs_gpu_minsr_solve_noalloc(dO.data_ptr(), dE.data_ptr(), Ns, a.P, cfg.sr_diag_shift,
                                               dd.data_ptr(), C.byref(info), None)
    assert rc == 0, nqs.last_error()
    if free_bytes is not None:
        torch.cuda.synchronize()
        free_bytes.append(torch.cuda.mem_get_info()[0])
    delta = dd.cpu().numpy()
    return delta, info, delta_ref, info_ref, cfg.learning_rate


def test_noalloc_matches_existing_entry_point_twice(env):
    torch, abi, nqs = env
    # (N_s, seed, hidden units M): N_p = 2 (16 + M + 16 M) = 1120, 1120, 270, 474
    for Ns, seed, M in ((512, 101, 32), (384, 202, 32), (1000, 303, 7), (1024, 404, 13)):
        delta, info, delta_ref, info_ref, lr = existing_and_noalloc(torch, abi, nqs, Ns, seed, M)
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


def test_noalloc_call_allocates_no_device_memory(env):
    """After a warm-up call (which loads the library's device code and with it the static
    scratch), further calls leave cudaMemGetInfo's free memory unchanged."""
    torch, abi, nqs = env
    existing_and_noalloc(torch, abi, nqs, 256, 505, 16)
    free_bytes = []
    for Ns, seed in ((640, 606), (1000, 707)):
        existing_and_noalloc(torch, abi, nqs, Ns, seed, 16, free_bytes)
    assert free_bytes[0] == free_bytes[1] and free_bytes[2] == free_bytes[3], free_bytes
