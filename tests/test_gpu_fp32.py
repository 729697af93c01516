"""Mixed-precision estimator and sampler: the FP32 product form of the RBM /
cRBM amplitude ratios (cosh(theta - d) / cosh(theta) = cosh d - tanh(theta)
sinh d) against the FP64 oracle and the FP64 GPU path.

Bars: local energies within 2e-5 of the largest |E_loc| (FP32 rounding of a
sum of ~16 ratios); the step's own end-to-end check (the FP64 estimator and
FP64 MinSR rerun on the same samples) reports the energy and delta-theta
errors; FP32 and FP64 chains draw the same Philox words, so they take the same
decisions except where |log u - 2 log|psi'/psi|| falls below the FP32
rounding, and nearly all chains end in the same configuration."""
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


def heis_case(abi, Ns, seed=11):
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=32, rbm_init_scale=0.3,
                              hamiltonian=1, rng_seed=4242, sr_diag_shift=1e-4, learning_rate=0.005)
    rng = np.random.default_rng(seed)
    batch = np.stack([rng.permutation(np.array([1, -1] * 8, np.int32)) for _ in range(Ns)])
    return cfg, batch


def test_fp32_step_against_fp64(nqs):
    from spin_based_neural_network_gb300 import abi
    Lx = Ly = 4
    cfg, batch = heis_case(abi, 2048)
    a = nqs.Ansatz(cfg, 16)
    p0 = a.params.copy()
    m = nqs.Marshall(a.log_amp_fn, a.user, Lx, Ly)
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=8, gram_passes=3, mixed_check=1,
                    fp32_estimator=1)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, Lx, Ly, a, batch, minsr=True, log_amp_fn=m.log_amp_fn,
                                           user=m.user)
        st = nqs.last_step_stats()
    finally:
        nqs.set_options()
    amp = O.Amp(O.OR_CRBM, 16, 32, p0.copy(), [("marshall", Lx, Ly)])
    Eo, do, io = O.minsr_step(O.ham(O.OR_HEIS, Lx, Ly, pbc=1), amp, batch, 1e-4, 0.005)
    assert info.converged == 1
    assert np.max(np.abs(E - Eo)) <= 2e-5 * np.max(np.abs(Eo))
    assert abs(info.mean_energy - io.mean_energy) <= 1e-6 * abs(io.mean_energy)
    assert 0 <= st.energy_rel_err <= 1e-6
    err = np.linalg.norm(delta - do) / np.linalg.norm(do)
    print("fp32 estimator: energy rel err %.2e, delta err vs oracle %.2e (step's own check %.2e)"
          % (st.energy_rel_err, err, st.delta_rel_err))
    assert err < 1e-3 and 0 <= st.delta_rel_err < 1e-3
    # the step's own check and the oracle see the same error
    assert st.delta_rel_err == pytest.approx(err, rel=0.05, abs=1e-9)


def test_fp32_real_rbm_tfim_energies(nqs):
    from spin_based_neural_network_gb300 import abi
    N = 16
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=16, rbm_init_scale=0.2, hamiltonian=0,
                              j_coupling=1.0, transverse_field=1.0, rng_seed=7, sr_diag_shift=1e-3,
                              learning_rate=0.01)
    rng = np.random.default_rng(3)
    batch = rng.choice(np.array([-1, 1], np.int32), size=(512, N))
    a = nqs.Ansatz(cfg, N)
    p0 = a.params.copy()
    nqs.set_options(square_pbc=1, precision=abi.PREC_MIXED, refine_sweeps=8, fp32_estimator=1)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, N, 1, a, batch, minsr=True)
    finally:
        nqs.set_options()
    amp = O.Amp(O.OR_RBM, N, 16, p0.copy(), [])
    Eo, do, io = O.minsr_step(O.ham(O.OR_TFIM, N, 1, pbc=1, J=1.0, Gamma=1.0), amp, batch, 1e-3, 0.01)
    assert np.max(np.abs(E - Eo)) <= 2e-5 * np.max(np.abs(Eo))


@pytest.mark.parametrize("kind", ["crbm_exchange", "rbm_flip"])
def test_fp32_chains_follow_fp64_chains(nqs, kind):
    from spin_based_neural_network_gb300 import abi
    if kind == "crbm_exchange":
        N, Lx, Ly = 16, 4, 4
        cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=32, rbm_init_scale=0.3,
                                  hamiltonian=1, rng_seed=99)
        move, n_down = abi.MOVE_EXCHANGE, 8
    else:
        N, Lx, Ly = 16, 16, 1
        cfg = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=16, rbm_init_scale=0.3,
                                  hamiltonian=0, rng_seed=99)
        move, n_down = abi.MOVE_SINGLE_FLIP, -1
    a = nqs.Ansatz(cfg, N)
    chains = 128

    def run(prec, f32):
        o = nqs.options(num_chains=chains, rng=abi.RNG_PHILOX, move=move, n_down=n_down, lattice_x=Lx,
                        lattice_y=Ly, square_pbc=1, precision=prec, fp32_estimator=f32)
        s = nqs.Sampler(N, cfg, a.log_amp_fn, a.user, o)
        s.thermalize()
        out = s.batch(chains * 8)
        return out, s.acceptance_ratio()

    b64, acc64 = run(abi.PREC_FP64, 0)
    b32, acc32 = run(abi.PREC_MIXED, 1)
    same = np.mean(np.all(b64 == b32, axis=1))
    assert same >= 0.9, same
    assert abs(acc64 - acc32) <= 0.02


# ---- the 2-hidden-layer MLP (extension): FP32 forward from incrementally
# updated layer-1 pre-activations, FP32 back-propagation for the Jacobian.

def mlp_kagome_case(nqs, abi, width, Ns, seed=5):
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_GPU_MLP, width=width, depth=2, hamiltonian=abi.HAM_KAGOME_HEISENBERG,
                              kagome_pbc=1, j_coupling=1.0, rng_seed=seed, sr_diag_shift=1e-3, learning_rate=0.01)
    a = nqs.Ansatz(cfg, 12)
    rng = np.random.default_rng(seed)
    batch = np.stack([rng.permutation(np.array([1, -1] * 6, np.int32)) for _ in range(Ns)])
    return cfg, a, batch


@pytest.mark.parametrize("width", [24, 40, 108])
def test_fp32_mlp_kagome_step_against_oracle(nqs, width):
    """Kagome 2x2 PBC (N = 12) with the MLP: FP32 local energies within 2e-5 of
    max|E_loc| of the FP64 oracle, delta-theta within 1e-3 (FP32 Jacobian), and
    the step's own FP64 cross-check agreeing."""
    from spin_based_neural_network_gb300 import abi
    cfg, a, batch = mlp_kagome_case(nqs, abi, width, 1024)
    p0 = a.params.copy()
    nqs.set_options(precision=abi.PREC_MIXED, refine_sweeps=8, gram_passes=3, mixed_check=1, fp32_estimator=1)
    try:
        info, E, delta = nqs.sr_step_batch(cfg, 2, 2, a, batch, minsr=True)
        st = nqs.last_step_stats()
    finally:
        nqs.set_options()
    amp = O.Amp(O.OR_MLP, 12, width, p0.copy(), [])
    Eo, do, io = O.minsr_step(O.ham(O.OR_KAGOME, 2, 2, kagome_pbc=1), amp, batch, 1e-3, 0.01)
    assert info.converged == 1
    assert np.max(np.abs(E - Eo)) <= 2e-5 * np.max(np.abs(Eo))
    assert 0 <= st.energy_rel_err <= 1e-5
    err = np.linalg.norm(delta - do) / np.linalg.norm(do)
    assert err < 1e-3 and 0 <= st.delta_rel_err < 1e-3


def test_fp32_mlp_chains_follow_fp64_chains(nqs):
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_GPU_MLP, width=40, depth=2, hamiltonian=abi.HAM_KAGOME_HEISENBERG,
                              kagome_pbc=1, rng_seed=17)
    a = nqs.Ansatz(cfg, 12)
    chains = 128

    def run(prec, f32):
        o = nqs.options(num_chains=chains, rng=abi.RNG_PHILOX, move=abi.MOVE_EXCHANGE, n_down=6, lattice_x=2,
                        lattice_y=2, lattice_kagome=1, precision=prec, fp32_estimator=f32)
        s = nqs.Sampler(12, cfg, a.log_amp_fn, a.user, o)
        s.thermalize()
        return s.batch(chains * 8), s.acceptance_ratio()

    b64, acc64 = run(abi.PREC_FP64, 0)
    b32, acc32 = run(abi.PREC_MIXED, 1)
    assert np.all(b32.sum(axis=1) == 0)                  # Sz = 0 kept
    same = np.mean(np.all(b64 == b32, axis=1))
    assert same >= 0.9, same
    assert abs(acc64 - acc32) <= 0.02


@pytest.mark.parametrize("ham,L,width", [("kagome", 3, 108), ("kagome", 2, 24), ("tfim", 16, 40)])
def test_mlp_tensor_core_layer_local_energies(nqs, ham, L, width):
    """The MLP local energies with the second layer on the tensor cores (tcgen05 TF32, three
    hi / lo passes; the default in the mixed mode) against the SIMT layer (mlp_simt = 1) and
    the FP64 oracle on the same batch: kagome 3x3 at width 108 (55 rows per sample, two
    samples per 128-row tile), kagome 2x2 at width 24 (one K chunk), and a TFIM chain of 16
    sites (single-site candidates).  Bar: 2e-5 of max|E_loc|, the FP32 estimator's."""
    from spin_based_neural_network_gb300 import abi
    if ham == "kagome":
        N, Lx, Ly, h = 3 * L * L, L, L, abi.HAM_KAGOME_HEISENBERG
        oh = O.ham(O.OR_KAGOME, L, L, kagome_pbc=1)
    else:
        N, Lx, Ly, h = L, L, 1, abi.HAM_TFIM
        oh = O.ham(O.OR_TFIM, L, 1, Gamma=0.8)
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_GPU_MLP, width=width, depth=2, hamiltonian=h, kagome_pbc=1,
                              transverse_field=0.8, j_coupling=1.0, rng_seed=11, sr_diag_shift=1e-3,
                              learning_rate=0.01)
    a = nqs.Ansatz(cfg, N)
    p0 = a.params.copy()
    rng = np.random.default_rng(N + width)
    batch = np.where(rng.random((1000, N)) < 0.5, 1, -1).astype(np.int32)
    E = {}
    for simt in (0, 1):
        a.params[:] = p0
        nqs.set_options(precision=abi.PREC_MIXED, refine_sweeps=8, fp32_estimator=1, mlp_simt=simt)
        try:
            info, E[simt], _ = nqs.sr_step_batch(cfg, Lx, Ly, a, batch, minsr=True)
        finally:
            nqs.set_options()
        assert np.all(np.isfinite(E[simt]))
    Eo = O.local_energy(oh, O.Amp(O.OR_MLP, N, width, p0.copy(), []), batch)
    scale = np.max(np.abs(Eo))
    assert np.max(np.abs(E[0] - Eo)) <= 2e-5 * scale
    assert np.max(np.abs(E[1] - Eo)) <= 2e-5 * scale
    assert np.max(np.abs(E[0] - E[1])) <= 2e-5 * scale
