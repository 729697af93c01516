"""Learned Metropolis proposal (masked autoregressive MLP, BF16 weights) against
the numpy restatement in made_ref.py, and the exactness of the Markov chain
that mixes it with local moves.

Bars: log q to 1e-4 (FP32 accumulation over <= 64 hidden units) and the NLL
gradient to 1e-4 of its largest entry against numpy on the same BF16 weights;
q normalised over the sector to 1e-4; draws from q follow q (total variation
below 0.015 with 200k draws over 70 states); the chain with learned proposals
samples |psi|^2 (total variation against the exact distribution below 0.02);
online training lowers the NLL; a proposal that is never accepted trips the
fallback to local moves."""
import itertools

import numpy as np
import pytest

import made_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    N.set_options()
    return N


def ring_sampler(nqs, N, n_down, chains=256, exchange=True, seed=5, M=None):
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=M or N, rbm_init_scale=0.6,
                              hamiltonian=1, rng_seed=seed, num_decorrelate=2)
    a = nqs.Ansatz(cfg, N)
    o = nqs.options(num_chains=chains, rng=abi.RNG_PHILOX,
                    move=abi.MOVE_EXCHANGE if exchange else abi.MOVE_SINGLE_FLIP,
                    n_down=n_down, lattice_x=N, lattice_y=1, square_pbc=1, precision=abi.PREC_MIXED,
                    fp32_estimator=1)
    s = nqs.Sampler(N, cfg, a.log_amp_fn, a.user, o)
    return cfg, a, s


def all_configs(N, n_down):
    x = np.array(list(itertools.product([0, 1], repeat=N)))
    if n_down >= 0:
        x = x[x.sum(1) == n_down]
    return x, (1 - 2 * x).astype(np.int32)


@pytest.mark.parametrize("n_down,exchange", [(5, True), (-1, False)])
def test_log_prob_matches_numpy_and_normalises(nqs, n_down, exchange):
    N, H = 10, 32
    cfg, a, s = ring_sampler(nqs, N, n_down, exchange=exchange)
    lp = nqs.LearnedProposal(s, hidden=H)
    rng = np.random.default_rng(1)
    w = (rng.normal(size=lp.num_params()) * 0.4).astype(np.float32)
    lp.set_weights(w)
    w_back = lp.weights()
    assert np.all(w_back[~R.mask_vector(N, H)] == 0)
    x, spins = all_configs(N, n_down if exchange else -1)
    got = lp.log_prob(spins)
    ref = R.logq(w_back, x, N, H, n_down if exchange else -1)
    assert np.max(np.abs(got - ref)) < 1e-4
    assert abs(np.exp(got).sum() - 1.0) < 1e-4


def test_nll_gradient_matches_numpy(nqs):
    N, H = 12, 64
    cfg, a, s = ring_sampler(nqs, N, 6)
    lp = nqs.LearnedProposal(s, hidden=H)
    rng = np.random.default_rng(2)
    lp.set_weights((rng.normal(size=lp.num_params()) * 0.3).astype(np.float32))
    w = lp.weights()
    x = np.array([rng.permutation([1] * 6 + [0] * 6) for _ in range(777)])
    g, nll = lp.nll_grad((1 - 2 * x).astype(np.int32))
    nll_ref, g_ref = R.nll_grad(w, x, N, H, 6)
    assert nll == pytest.approx(nll_ref, rel=1e-5)
    assert np.max(np.abs(g - g_ref)) <= 1e-4 * np.max(np.abs(g_ref))
    assert np.all(g[~R.mask_vector(N, H)] == 0)


def test_draws_follow_q(nqs):
    N, n_down = 8, 4
    cfg, a, s = ring_sampler(nqs, N, n_down)
    lp = nqs.LearnedProposal(s, hidden=32)
    rng = np.random.default_rng(3)
    lp.set_weights((rng.normal(size=lp.num_params()) * 0.5).astype(np.float32))
    spins, lq = lp.sample(200000)
    x = (spins < 0).astype(int)
    assert np.all(x.sum(1) == n_down)
    # the pool's log q is the teacher-forced log q of the same configuration
    assert np.max(np.abs(lq[:2000] - lp.log_prob(spins[:2000]))) < 1e-5
    allx, alls = all_configs(N, n_down)
    q = np.exp(lp.log_prob(alls))
    idx = {tuple(r): i for i, r in enumerate(allx)}
    counts = np.zeros(len(allx))
    for r in map(tuple, x):
        counts[idx[r]] += 1
    tv = 0.5 * np.abs(counts / counts.sum() - q).sum()
    assert tv < 0.015, tv


def exact_distribution(nqs, a, alls):
    la, _ = nqs.log_amp_batch(a.log_amp_fn, a.user, alls)
    p = np.exp(2 * (la - la.max()))
    return p / p.sum()


def chain_tv(nqs, s, a, alls, allx, batches=6, per=8192):
    idx = {tuple(r): i for i, r in enumerate(allx)}
    counts = np.zeros(len(allx))
    s.thermalize()
    for _ in range(batches):
        b = s.batch(per)
        for r in map(tuple, (b < 0).astype(int)):
            counts[idx[r]] += 1
    p = exact_distribution(nqs, a, alls)
    return 0.5 * np.abs(counts / counts.sum() - p).sum()


def test_learned_chain_samples_psi_squared(nqs):
    N, n_down = 8, 4
    cfg, a, s = ring_sampler(nqs, N, n_down, chains=512)
    lp = nqs.LearnedProposal(s, hidden=32, mix=0.5, train_iters=4, learning_rate=1e-2)
    allx, alls = all_configs(N, n_down)
    tv = chain_tv(nqs, s, a, alls, allx)
    st = lp.stats()
    assert st.proposals > 0 and st.accepted > 0 and st.train_steps > 0
    assert tv < 0.02, tv


def test_training_lowers_nll(nqs):
    N, n_down = 12, 6
    cfg, a, s = ring_sampler(nqs, N, n_down, chains=512)
    lp = nqs.LearnedProposal(s, hidden=64, mix=0.5, train_iters=4, learning_rate=1e-2)
    s.thermalize()
    nll = []
    for _ in range(12):
        s.batch(4096)
        nll.append(lp.stats().nll)
    assert nll[-1] < nll[0] - 0.05, nll
    st = lp.stats()
    assert st.accepted / st.proposals > 0.05


def test_fallback_when_never_accepted(nqs):
    """Weights that put all mass far from |psi|^2 are still exact (the chain
    keeps sampling |psi|^2) and trip the fallback to local moves."""
    N, n_down = 8, 4
    cfg, a, s = ring_sampler(nqs, N, n_down, chains=256)
    lp = nqs.LearnedProposal(s, hidden=32, mix=0.5, train_iters=0, min_acceptance=0.9)
    w = np.zeros(lp.num_params(), np.float32)
    lp.set_weights(w)
    s.thermalize()
    s.batch(2048)
    s.batch(2048)
    assert lp.stats().active == 0


def test_learned_mlp_chain_samples_psi_squared(nqs):
    """The learned proposal on the FP32 MLP chains (log|psi| of both states from
    scratch in the chain, the pool carrying only x' and log q(x')) keeps the
    chain exact: total variation against |psi|^2 below 0.02."""
    from spin_based_neural_network_gb300 import abi
    N, n_down = 8, 4
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_GPU_MLP, width=16, depth=2, hamiltonian=1, rng_seed=21,
                              num_decorrelate=2)
    a = nqs.Ansatz(cfg, N)
    a.params[:] = a.params * 3.0                 # a less uniform |psi|^2
    o = nqs.options(num_chains=512, rng=abi.RNG_PHILOX, move=abi.MOVE_EXCHANGE, n_down=n_down, lattice_x=N,
                    lattice_y=1, square_pbc=1, precision=abi.PREC_MIXED, fp32_estimator=1)
    s = nqs.Sampler(N, cfg, a.log_amp_fn, a.user, o)
    lp = nqs.LearnedProposal(s, hidden=32, mix=0.5, train_iters=4, learning_rate=1e-2)
    allx, alls = all_configs(N, n_down)
    tv = chain_tv(nqs, s, a, alls, allx)
    st = lp.stats()
    assert st.proposals > 0 and st.accepted > 0 and st.train_steps > 0
    assert tv < 0.02, tv
