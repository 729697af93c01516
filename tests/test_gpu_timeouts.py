"""The bounded-wait paths of the cooperative solve kernels, exercised on purpose.

Every grid-wide barrier of the mixed MinSR factor / refinement kernel and of the CG-SR
kernel, and every flag wait between the pipelined factor's first CTA and the others, polls a
bounded number of times (nqs_gpu_set_barrier_budget; 2^24 by default) and then raises the
kernel's error word instead of waiting on.  These tests lower the budget to
one poll, so the CTAs that reach a barrier first give up while the others are still on
their way: the step must return -1 with "grid barrier timed out", leave the parameters
untouched, and the next call, with the default budget again, must succeed and give the
same update as before (the barrier and error words are cleared at every launch).  Nothing
faults or hangs: the waits end by themselves and every CTA leaves through the code path
that releases its tensor memory.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    yield N
    N.lib().nqs_gpu_set_barrier_budget(0)
    N.set_options()


def problem(nqs, Ns=2048, seed=77):
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=32, rbm_init_scale=0.3, rng_seed=seed,
                              hamiltonian=abi.HAM_HEISENBERG, sr_diag_shift=1e-3, learning_rate=0.01,
                              sr_cg_max_iters=50, sr_cg_tol=1e-10)
    a = nqs.Ansatz(cfg, 16)
    m = nqs.Marshall(a.log_amp_fn, a.user, 4, 4)
    rng = np.random.default_rng(seed)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(Ns)])
    return cfg, a, m, batch


@pytest.mark.parametrize("solver", ["mixed_minsr", "cg_sr"])
def test_barrier_timeout_returns_an_error_and_the_next_call_succeeds(nqs, solver):
    from spin_based_neural_network_gb300 import abi
    if solver == "mixed_minsr":
        nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=5)
        minsr = True
    else:
        nqs.set_options(square_pbc=1)
        minsr = False
    try:
        cfg, a, m, batch = problem(nqs)
        p0 = a.params.copy()
        info, E, d_ok = nqs.sr_step_batch(cfg, 4, 4, a, batch, minsr=minsr, log_amp_fn=m.log_amp_fn, user=m.user)
        a.params[:] = p0
        assert nqs.lib().nqs_gpu_set_barrier_budget(1) == 0
        try:
            with pytest.raises(nqs.NqsError):
                nqs.sr_step_batch(cfg, 4, 4, a, batch, minsr=minsr, log_amp_fn=m.log_amp_fn, user=m.user)
            assert "grid barrier timed out" in nqs.last_error()
        finally:
            assert nqs.lib().nqs_gpu_set_barrier_budget(0) == 0
        assert np.array_equal(a.params, p0)                     # a failed step leaves theta alone
        info2, E2, d2 = nqs.sr_step_batch(cfg, 4, 4, a, batch, minsr=minsr, log_amp_fn=m.log_amp_fn, user=m.user)
        assert info2.converged == info.converged and info2.cg_iterations == info.cg_iterations
        assert np.array_equal(E2, E)
        assert np.linalg.norm(d2 - d_ok) <= 1e-12 * np.linalg.norm(d_ok)
    finally:
        nqs.set_options()
