"""Batches of independent problems (nqs_gpu_batch_*): uneven instances stepped
together, with all solves in one cooperative launch and, from the second step,
the whole batch step replayed as a CUDA graph, give the same energies and the
same parameters as the same instances stepped one by one through
nqs_sr_step_minsr_full with the same options.  Every tile and reduction of the
solve is computed in the same order whichever CTAs of the launch own it, so the
agreement bar is 1e-12 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    return N


# (hamiltonian, Lx, Ly, hidden, complex, samples, chains, couplings)
CASES = [
    ("tfim", 12, 1, 12, False, 512, 128, dict(j_coupling=1.0, transverse_field=0.8)),
    ("xxz", 4, 4, 32, False, 1024, 256, dict(j_coupling=1.0, j_z_coupling=1.6)),
    ("heis", 20, 1, 20, True, 2048, 512, dict(j_coupling=1.0)),
    ("tfim", 2, 8, 64, False, 512, 128, dict(j_coupling=1.0, transverse_field=1.3)),   # N_p > N_s: sample space
]


def build(nqs, abi, case, seed):
    ham, Lx, Ly, M, cx, Ns, C, kw = case
    N = Lx * Ly
    hk = {"tfim": 0, "heis": 1, "xxz": 4}[ham]
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM if cx else abi.ANSATZ_RBM, rbm_hidden_units=M,
                              rbm_init_scale=0.2, hamiltonian=hk, rng_seed=seed, num_samples=Ns,
                              num_thermalize=64, num_decorrelate=N, sr_diag_shift=1e-3, learning_rate=0.02, **kw)
    a = nqs.Ansatz(cfg, N)
    fn, user = None, None
    if ham != "tfim":
        m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
        fn, user, keep = m.log_amp_fn, m.user, m
    else:
        keep = None
    o = nqs.options(num_chains=C, rng=abi.RNG_PHILOX,
                    move=abi.MOVE_EXCHANGE if ham != "tfim" else abi.MOVE_SINGLE_FLIP,
                    n_down=N // 2 if ham != "tfim" else -1, lattice_x=Lx, lattice_y=Ly, square_pbc=1,
                    precision=abi.PREC_MIXED, fp32_estimator=1)
    s = nqs.Sampler(N, cfg, fn if fn else a.log_amp_fn, user if user else a.user, o)
    s.thermalize()
    return dict(cfg=cfg, a=a, s=s, fn=fn, user=user, keep=keep, Lx=Lx, Ly=Ly)


def test_batch_matches_single_steps(nqs):
    from spin_based_neural_network_gb300 import abi
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, fp32_estimator=1, refine_sweeps=5, gram_passes=3)
    try:
        bat = [build(nqs, abi, c, 100 + i) for i, c in enumerate(CASES)]
        ref = [build(nqs, abi, c, 100 + i) for i, c in enumerate(CASES)]
        B = nqs.Batch([(b["cfg"], b["Lx"], b["Ly"], b["a"], b["s"], b["fn"], b["user"]) for b in bat])
        for step in range(4):
            infos = B.step()
            for i, r in enumerate(ref):
                info = nqs.sr_step_minsr(r["cfg"], r["Lx"], r["Ly"], r["a"], r["s"],
                                         r["fn"] if r["fn"] else r["a"].log_amp_fn,
                                         r["user"] if r["user"] else r["a"].user)
                assert infos[i].converged == 1
                assert infos[i].mean_energy == pytest.approx(info.mean_energy, rel=1e-12, abs=1e-12), (step, i)
                assert infos[i].update_norm == pytest.approx(info.update_norm, rel=1e-10), (step, i)
                pb, pr = bat[i]["a"].params, r["a"].params
                assert np.max(np.abs(pb - pr)) <= 1e-12 * max(1.0, np.max(np.abs(pr))), (step, i)
        ctas = B.ctas()
        assert len(ctas) == len(CASES) and min(ctas) >= 1
        assert len(B.tune_ms()) >= 2
        B.free()
    finally:
        nqs.set_options()


def test_batch_rejects_fp64_sampler(nqs):
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=8, hamiltonian=0, num_samples=256)
    a = nqs.Ansatz(cfg, 8)
    o = nqs.options(num_chains=32, rng=abi.RNG_PHILOX, lattice_x=8, lattice_y=1)
    s = nqs.Sampler(8, cfg, a.log_amp_fn, a.user, o)
    with pytest.raises(nqs.NqsError):
        nqs.Batch([(cfg, 8, 1, a, s, None, None)])


def test_batch_fp32_breakdown_falls_back_to_fp64(nqs):
    """A negative diagonal shift makes the first pivot negative: the FP32 factor
    of every instance breaks down inside the graph, the batch re-solves each in
    FP64 afterwards (upstream retry semantics: breakdown again, update 0,
    converged 0), exactly as the single-system MIXED step does."""
    from spin_based_neural_network_gb300 import abi
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, fp32_estimator=1, refine_sweeps=5, gram_passes=3)
    cases = CASES[:2]
    try:
        bat = [build(nqs, abi, c, 300 + i) for i, c in enumerate(cases)]
        ref = [build(nqs, abi, c, 300 + i) for i, c in enumerate(cases)]
        for b in bat + ref:
            b["cfg"].sr_diag_shift = -2.0
        B = nqs.Batch([(b["cfg"], b["Lx"], b["Ly"], b["a"], b["s"], b["fn"], b["user"]) for b in bat])
        p0 = [b["a"].params.copy() for b in bat]
        for step in range(3):
            infos = B.step()
            for i, r in enumerate(ref):
                info = nqs.sr_step_minsr(r["cfg"], r["Lx"], r["Ly"], r["a"], r["s"],
                                         r["fn"] if r["fn"] else r["a"].log_amp_fn,
                                         r["user"] if r["user"] else r["a"].user)
                assert infos[i].converged == info.converged == 0
                assert infos[i].update_norm == info.update_norm == 0.0
                assert infos[i].mean_energy == pytest.approx(info.mean_energy, rel=1e-12, abs=1e-12)
                assert np.array_equal(bat[i]["a"].params, p0[i])
                assert np.array_equal(r["a"].params, p0[i])
        assert B.fallbacks() == 3 * len(cases)
        B.free()
    finally:
        nqs.set_options()


def test_batch_with_learned_proposals_matches_single_steps(nqs):
    """Learned proposals attached to the instances' samplers: the pool draws,
    training and fallback run inside the batch graph (device counters), and the
    batch still equals the same instances stepped one by one."""
    from spin_based_neural_network_gb300 import abi
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, fp32_estimator=1, refine_sweeps=5, gram_passes=3)
    cases = CASES[:2]
    try:
        bat = [build(nqs, abi, c, 500 + i) for i, c in enumerate(cases)]
        ref = [build(nqs, abi, c, 500 + i) for i, c in enumerate(cases)]
        lps = [nqs.LearnedProposal(b["s"], hidden=32, mix=0.5) for b in bat + ref]
        B = nqs.Batch([(b["cfg"], b["Lx"], b["Ly"], b["a"], b["s"], b["fn"], b["user"]) for b in bat])
        for step in range(4):
            infos = B.step()
            for i, r in enumerate(ref):
                info = nqs.sr_step_minsr(r["cfg"], r["Lx"], r["Ly"], r["a"], r["s"],
                                         r["fn"] if r["fn"] else r["a"].log_amp_fn,
                                         r["user"] if r["user"] else r["a"].user)
                assert infos[i].mean_energy == pytest.approx(info.mean_energy, rel=1e-12, abs=1e-12), (step, i)
                pb, pr = bat[i]["a"].params, r["a"].params
                assert np.max(np.abs(pb - pr)) <= 1e-12 * max(1.0, np.max(np.abs(pr))), (step, i)
        for lp in lps[:len(cases)]:
            st = lp.stats()
            assert st.proposals > 0 and st.accepted > 0 and st.train_steps >= 4
        B.free()
    finally:
        nqs.set_options()
