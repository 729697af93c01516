"""Mixed-precision MinSR: tensor-core (tcgen05, TF32) Gram and FP32 factor with
FP64 iterative refinement, checked against FP64 references.

Bars: the 3-pass split Gram (hi hi^T + hi lo^T + lo hi^T) reproduces the FP64
Gram to 4e-5 of its largest entry (single pass TF32: 5e-3); after refinement the
MinSR update matches the FP64 oracle's on the same samples to 1e-8 relative
(the refinement residual is reported by the step), whether the solve runs in
sample space (N_s x N_s) or in parameter space (N_p x N_p, the push-through
form of the same update)."""
import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    N.set_options()
    return N


def gram_tc(nqs, Om, passes, scale):
    import ctypes as C
    Om = np.ascontiguousarray(Om, dtype=np.float64)
    Ns, P = Om.shape
    T = np.zeros((Ns, Ns), dtype=np.float32)
    rc = nqs.lib().nqs_gpu_gram_tc(Om.ctypes.data_as(nqs.DP), Ns, P, passes, scale,
                                   T.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0, nqs.last_error()
    return T


@pytest.mark.parametrize("Ns,P", [(128, 32), (500, 300), (4096, 1120)])
def test_gram_tc_against_fp64(nqs, Ns, P):
    rng = np.random.default_rng(Ns + P)
    Om = rng.normal(size=(Ns, P))
    Om[:, : P // 4] = np.sign(Om[:, : P // 4])          # +-1 columns like the visible block
    ref = np.tril(Om @ Om.T) / Ns
    scale = np.max(np.abs(ref))
    T3 = np.tril(gram_tc(nqs, Om, 3, 1.0 / Ns).astype(np.float64))
    # the split removes the TF32 input rounding; what remains is the tensor
    # core's FP32 accumulation over K (measured 4e-6 at K = 3 x 320 and 1.6e-5
    # at K = 3 x 1120 relative to the largest entry)
    assert np.max(np.abs(T3 - ref)) <= 4e-5 * scale
    T1 = np.tril(gram_tc(nqs, Om, 1, 1.0 / Ns).astype(np.float64))
    err1 = np.max(np.abs(T1 - ref))
    assert err1 <= 5e-3 * scale and err1 > np.max(np.abs(T3 - ref))


def minsr_mixed(nqs, sweeps, check=0, space=0, Ns=4096):
    from spin_based_neural_network_gb300 import abi
    Lx = Ly = 4
    N, M = 16, 32
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, rbm_init_scale=0.3,
                              hamiltonian=1, rng_seed=4242, sr_diag_shift=1e-4, learning_rate=0.005)
    a = nqs.Ansatz(cfg, N)
    p0 = a.params.copy()
    m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    rng = np.random.default_rng(11)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(Ns)])
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=sweeps, gram_passes=3,
                    mixed_check=check, mixed_space=space)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, Lx, Ly, a, batch, minsr=True, log_amp_fn=m.log_amp_fn,
                                           user=m.user)
        stats = nqs.last_step_stats()
    finally:
        nqs.set_options()
    amp = O.Amp(O.OR_CRBM, N, M, p0.copy(), [("marshall", Lx, Ly)])
    Eo, do, io = O.minsr_step(O.ham(O.OR_HEIS, Lx, Ly, pbc=1), amp, batch, 1e-4, 0.005)
    return info, E, delta, stats, Eo, do, io


# (N_s, space, sweeps): 4096 > N_p = 1120 picks parameter space, 512 < N_p picks
# samples; sweeps = maximum CG iterations.  The N_p x N_p system keeps the
# small-eigenvalue directions that the sample-space update projects out through
# O_c^T, so it converges more slowly and gets more iterations.
@pytest.mark.parametrize("Ns,space,sweeps", [(4096, 0, 8), (4096, 1, 3), (512, 0, 3), (512, 2, 3)])
def test_mixed_minsr_against_fp64_oracle(nqs, Ns, space, sweeps):
    info, E, delta, stats, Eo, do, io = minsr_mixed(nqs, sweeps=sweeps, check=1, space=space, Ns=Ns)
    assert info.converged == 1 and stats.mixed_fallback == 0
    assert np.max(np.abs(E - Eo) / np.maximum(np.abs(Eo), 1.0)) < 1e-12
    err = np.linalg.norm(delta - do) / np.linalg.norm(do)
    assert stats.refine_residual < 1e-8
    assert err < 1e-8
    assert 0 <= stats.delta_rel_err < 1e-8          # the step's own FP64 cross-check


@pytest.mark.parametrize("space", [1, 2])
def test_refinement_contracts(nqs, space):
    """More CG iterations, smaller residual: the preconditioned CG converges."""
    r = [minsr_mixed(nqs, sweeps=s, space=space)[3].refine_residual for s in (0, 1, 2)]
    assert r[1] < r[0] and r[2] < r[1]


def test_phase_times_reported(nqs):
    stats = minsr_mixed(nqs, sweeps=2)[3]
    ph = list(stats.phase_us)
    assert ph[6] > 0 and all(p >= 0 for p in ph[:6]) and sum(ph[:6]) <= ph[6] * 1.01


def test_mixed_blocked_substitution_large(nqs):
    """Systems of order >= 4608 apply the preconditioner by blocked substitution
    instead of an explicit L^{-1}: a 5120 x 5120 sample-space solve (N_s = 5120 >
    N_p, forced sample space) against the FP64 step on the same samples (the
    step's own check, FP64 estimator so the error is the solve's alone)."""
    from spin_based_neural_network_gb300 import abi
    Lx = Ly = 4
    N, M = 16, 32
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, rbm_init_scale=0.3,
                              hamiltonian=1, rng_seed=77, sr_diag_shift=1e-3, learning_rate=0.005)
    a = nqs.Ansatz(cfg, N)
    m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    rng = np.random.default_rng(5)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(5120)])
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=8, gram_passes=3, mixed_check=1,
                    mixed_space=abi.SPACE_SAMPLES)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, Lx, Ly, a, batch, minsr=True, log_amp_fn=m.log_amp_fn, user=m.user)
        st = nqs.last_step_stats()
    finally:
        nqs.set_options()
    assert info.converged == 1 and st.mixed_fallback == 0
    assert st.refine_residual < 1e-8
    assert 0 <= st.delta_rel_err < 1e-7
    assert st.phase_us[3] < 1.0               # no explicit triangular inverse (microseconds)


@pytest.mark.parametrize("fp32_estimator", [0, 1])
def test_pipelined_factor_breakdown_falls_back_to_fp64(nqs, fp32_estimator):
    """A negative diagonal shift breaks the FP32 factor of the 1120 x 1120 parameter-space
    system, which runs the pipelined factor (64-wide blocks on every SM): CTA 0 records the
    failing column and raises its flag, the other CTAs leave at their next wait, and the step
    is solved again in FP64, which breaks down as well (upstream retry semantics: update 0,
    converged 0), as the FP64 step on the same samples does.  Nothing waits out a budget:
    the call returns normally and the next regular step converges."""
    from spin_based_neural_network_gb300 import abi
    Lx = Ly = 4
    N, M = 16, 32
    def make(shift):
        cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M, rbm_init_scale=0.3,
                                  hamiltonian=1, rng_seed=4242, sr_diag_shift=shift, learning_rate=0.005)
        a = nqs.Ansatz(cfg, N)
        return cfg, a, nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    rng = np.random.default_rng(12)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(4096)])
    cfg, a, m = make(-2.0)
    p0 = a.params.copy()
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=3, gram_passes=3,
                    fp32_estimator=fp32_estimator, mixed_space=abi.SPACE_PARAMETERS)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, Lx, Ly, a, batch, minsr=True, log_amp_fn=m.log_amp_fn,
                                           user=m.user)
        st = nqs.last_step_stats()
    finally:
        nqs.set_options()
    assert st.mixed_fallback == 1
    assert info.converged == 0 and info.update_norm == 0.0
    assert np.array_equal(a.params, p0)
    cfg2, a2, m2 = make(-2.0)
    nqs.set_options(square_pbc=1, fp32_estimator=0)
    try:
        info2, E2, delta2 = nqs.sr_step_batch(cfg2, Lx, Ly, a2, batch, minsr=True, log_amp_fn=m2.log_amp_fn,
                                              user=m2.user)
    finally:
        nqs.set_options()
    assert info2.converged == 0 and info2.update_norm == 0.0
    # the next regular step (positive shift) runs the pipelined factor normally
    cfg3, a3, m3 = make(1e-4)
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=3, gram_passes=3,
                    fp32_estimator=fp32_estimator, mixed_space=abi.SPACE_PARAMETERS)
    try:
        info3, E3, delta3 = nqs.sr_step_batch(cfg3, Lx, Ly, a3, batch, minsr=True, log_amp_fn=m3.log_amp_fn,
                                              user=m3.user)
        st3 = nqs.last_step_stats()
    finally:
        nqs.set_options()
    assert info3.converged == 1 and st3.mixed_fallback == 0 and st3.refine_residual < 1e-8
