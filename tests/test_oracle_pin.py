"""Pin the CPU oracle against golden vectors produced by the upstream library.

The fixtures under tests/golden/ were written by tests/golden/make_golden.py,
which drives the upstream C library itself.  The oracle follows the upstream
loop order, so agreement is expected to the last few ulps (1e-13 relative).
"""
import glob
import os

import numpy as np
import pytest

import oracle_lib as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def rel(a, b, floor=1.0):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


@pytest.mark.parametrize("name", ["mf", "rbm", "rbm_big", "crbm", "crbm_big"])
def test_ansatz_init_logamp_gradients(name):
    d = load("ansatz_" + name)
    kind, N, M = int(d["kind"]), int(d["N"]), int(d["M"])
    p = O.init_params(kind, N, M, float(d["scale"]), int(d["seed"]))
    assert np.array_equal(p, d["params"])                       # bit-exact initialisation
    amp = O.Amp(kind, N, M, p)
    la, ar = O.log_amp(amp, d["spins"])
    assert rel(la, d["la"]) < 1e-13
    assert rel(ar, d["arg"]) < 1e-13
    assert rel(O.gradient(amp, d["spins"]), d["grad"]) < 1e-13
    gr, gi = O.gradient_complex(amp, d["spins"])
    assert rel(gr, d["grad_re"]) < 1e-13 and rel(gi, d["grad_im"]) < 1e-13


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "eloc_*.npz"))))
def test_local_energy(path):
    d = dict(np.load(path))
    layers = [("marshall", int(d["Lx"]), int(d["Ly"]))] if int(d["marshall"]) else []
    amp = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params"], layers)
    h = O.ham(int(d["ham"]), int(d["Lx"]), int(d["Ly"]), 0, int(d["kagome_pbc"]),
              float(d["J"]), float(d["J2"]), float(d["Jz"]), float(d["Gamma"]))
    re, im = O.local_energy(h, amp, d["spins"], complex_out=True)
    assert rel(re, d["E"]) < 1e-12
    assert rel(re, d["E_re"]) < 1e-12
    assert rel(im, d["E_im"]) < 1e-12


@pytest.mark.parametrize("name", ["rbm16", "crbm16_marshall"])
def test_xorshift_sampler_sequence(name):
    d = load("sampler_" + name)
    layers = [("marshall", 4, 4)] if int(d["marshall"]) else []
    amp = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params"], layers)
    out, acc = O.xorshift_sampler(amp, int(d["seed"]), int(d["therm"]), int(d["decor"]),
                                  d["batch"].shape[0])
    assert np.array_equal(out, d["batch"])                        # identical Markov chain
    assert acc == pytest.approx(float(d["acceptance"]), abs=0)


@pytest.mark.parametrize("name", ["minsr_tfim_rbm", "minsr_heis_crbm_marshall", "cg_tfim_rbm",
                                  "cg_j1j2_crbm"])
def test_sr_step_on_reference_batch(name):
    d = load("sr_" + name)
    layers = [("marshall", int(d["Lx"]), int(d["Ly"]))] if int(d["marshall"]) else []
    amp = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params0"].copy(), layers)
    h = O.ham(int(d["ham"]), int(d["Lx"]), int(d["Ly"]), 0, 1, float(d["J"]), float(d["J2"]),
              1.0, float(d["Gamma"]))
    if str(d["solver"]) == "minsr":
        E, delta, info = O.minsr_step(h, amp, d["batch"], float(d["shift"]), float(d["lr"]))
    else:
        E, delta, info = O.cgsr_step(h, amp, d["batch"], float(d["shift"]), float(d["lr"]),
                                     int(d["cg_max"]), float(d["cg_tol"]))
    ref = d["info"]
    assert info.mean_energy == pytest.approx(ref[0], rel=1e-12)
    assert info.variance_energy == pytest.approx(ref[1], rel=1e-9)
    assert info.update_norm == pytest.approx(ref[2], rel=1e-10)
    assert info.cg_iterations == int(ref[4]) and info.converged == int(ref[5])
    step = d["params1"] - d["params0"]
    assert np.linalg.norm((amp.params - d["params0"]) - step) <= 1e-10 * np.linalg.norm(step)


@pytest.mark.parametrize("name", ["p2", "trans"])
def test_symproj(name):
    d = load("symproj_" + name)
    amp = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params"],
                [("symproj", d["perm"], d["chars"])])
    la, ar = O.log_amp(amp, d["spins"])
    assert rel(la, d["la"]) < 1e-13
    assert np.array_equal(ar, d["arg"])
    assert rel(O.symproj_gradient(amp, d["spins"]), d["grad"]) < 1e-12


def test_exact_energies_obc():
    d = load("exact_obc")
    for kind, Lx, Ly, J, X, e0 in d["rows"]:
        if int(kind) == 0:
            h = O.ham(O.OR_TFIM, int(Lx), int(Ly), 0, 1, J, 0.0, 1.0, X)
            e = O.exact_energy(h, -1)
        else:
            h = O.ham(O.OR_XXZ, int(Lx), int(Ly), 0, 1, J, 0.0, X, 0.0)
            e = min(O.exact_energy(h, nd) for nd in range(int(Lx * Ly) + 1))
        assert e == pytest.approx(e0, abs=1e-8)


def test_known_answers():
    """Closed-form values from the upstream unit tests (test_nqs.c:110-156,
    test_nqs_kagome.c:52-141, test_nqs_lanczos.c:163,259, test_nqs_kspace_ed.c:47,61)."""
    mf0 = O.Amp(O.OR_MF, 9, 0, np.zeros(9))
    allup = np.ones((1, 9), np.int32)
    neel = np.array([[1, -1, 1, -1, 1, -1, 1, -1, 1]], np.int32)
    assert O.local_energy(O.ham(O.OR_TFIM, 3, 3, Gamma=0.0), mf0, allup)[0] == pytest.approx(-12.0, abs=1e-12)
    assert O.local_energy(O.ham(O.OR_HEIS, 3, 3), mf0, neel)[0] == pytest.approx(3.0, abs=1e-12)
    assert O.local_energy(O.ham(O.OR_J1J2, 3, 3, J2=0.0), mf0, neel)[0] == pytest.approx(3.0, abs=1e-12)
    mf12 = O.Amp(O.OR_MF, 12, 0, np.zeros(12))
    k_all = np.ones((1, 12), np.int32)
    assert O.local_energy(O.ham(O.OR_KAGOME, 2, 2, kagome_pbc=1), mf12, k_all)[0] == pytest.approx(6.0)
    assert O.local_energy(O.ham(O.OR_KAGOME, 2, 2, kagome_pbc=0), mf12, k_all)[0] == pytest.approx(3.75)
    mf3 = O.Amp(O.OR_MF, 3, 0, np.array([0.1, 0.2, 0.3]))
    e = O.local_energy(O.ham(O.OR_KAGOME, 1, 1, kagome_pbc=1), mf3, np.array([[1, -1, 1]], np.int32))
    assert e[0] == pytest.approx(-0.5 + 2 * np.cosh(0.2), abs=1e-12)
    # Heisenberg chains (OBC N=4, N=8) and rings (PBC N=4, N=6)
    assert O.exact_energy(O.ham(O.OR_HEIS, 4, 1), 2) == pytest.approx(-1.616025, abs=1e-6)
    assert O.exact_energy(O.ham(O.OR_HEIS, 8, 1), 4) == pytest.approx(-3.37493260, abs=1e-7)
    assert O.exact_energy(O.ham(O.OR_HEIS, 4, 1, pbc=1), 2) == pytest.approx(-2.0, abs=1e-10)
    assert O.exact_energy(O.ham(O.OR_HEIS, 6, 1, pbc=1), 3) == pytest.approx(-2.802775637732, abs=1e-9)
    # kagome 2x2 PBC, Sz=0 sector (upstream spin_gap_L2_Sz0.json:2-3)
    assert O.exact_energy(O.ham(O.OR_KAGOME, 2, 2, kagome_pbc=1), 6) == pytest.approx(
        -5.444875216941, abs=1e-9)
    assert O.exact_energy(O.ham(O.OR_KAGOME, 2, 2, kagome_pbc=1), 5) == pytest.approx(
        -5.062206850707, abs=1e-9)


def test_marshall_parity_tables():
    """upstream tests/test_nqs_marshall.c:25-55"""
    P = lambda s, x, y: O.lib().oracle_marshall_parity(O.ip(np.array(s, np.int32)), x, y)
    assert [P(s, 2, 1) for s in ([1, 1], [-1, 1], [1, -1], [-1, -1])] == [0, 1, 0, 1]
    assert P([1, -1, -1, 1], 2, 2) == 0 and P([-1, 1, 1, -1], 2, 2) == 0
    assert P([-1, -1, -1, 1], 2, 2) == 1


def test_philox_known_answer():
    """Philox4x32-10 known-answer vectors published with Random123 (kat_vectors):
    counter=0,key=0 and counter=all-ones,key=all-ones."""
    import ctypes as C
    out = (C.c_uint32 * 4)()
    O.lib().oracle_philox4x32((C.c_uint32 * 4)(0, 0, 0, 0), (C.c_uint32 * 2)(0, 0), out)
    assert list(out) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    m = 0xFFFFFFFF
    O.lib().oracle_philox4x32((C.c_uint32 * 4)(m, m, m, m), (C.c_uint32 * 2)(m, m), out)
    assert list(out) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def test_exact_energy_fixture():
    """tests/golden/exact_energies.json (bench's |dE/N| target) against closed
    forms: the critical TFIM ring, E0 = -2 / sin(pi / 2N) (even-parity sector of
    the free-fermion solution), and the 4x4 Heisenberg torus, -11.2284832084."""
    import json
    import math
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "exact_energies.json")) as f:
        ex = json.load(f)
    assert ex["tfim_chain16_pbc_h1"]["E0"] == pytest.approx(-2.0 / math.sin(math.pi / 32), abs=1e-9)
    assert ex["heisenberg_4x4_pbc_sz0"]["E0"] == pytest.approx(-11.2284832084, abs=1e-9)


def test_holomorphic_step_reduces_to_cg_sr_for_a_real_rbm():
    """Holomorphic SR restated from src/nqs/nqs_optimizer.c:415-524: for a real
    ansatz the imaginary parts vanish, G = 2 S and F = 2 F_real, so the step
    with shift 2 eps equals CG-SR with shift eps (converged solves)."""
    N, M = 8, 8
    p = O.init_params(O.OR_RBM, N, M, 0.3, 11)
    rng = np.random.default_rng(4)
    batch = rng.choice(np.array([-1, 1], np.int32), size=(256, N))
    h = O.ham(O.OR_TFIM, N, 1, Gamma=0.7)
    Eh, dh, ih = O.holo_step(h, O.Amp(O.OR_RBM, N, M, p.copy()), batch, 2e-3, 0.01, 1000, 1e-12)
    Ec, dc, ic = O.cgsr_step(h, O.Amp(O.OR_RBM, N, M, p.copy()), batch, 1e-3, 0.01, 1000, 1e-12)
    assert ih.converged == 1 and ic.converged == 1
    assert np.array_equal(Eh, Ec)
    assert np.linalg.norm(dh - dc) <= 1e-8 * np.linalg.norm(dc)


def _holo_dense(R, I, Er, Ei, erm, eim, shift, realtime=False):
    """Dense restatement of the holomorphic family's linear system: G = 2 [(R^T R + I^T I)/N_s
    - <R><R>^T - <I><I>^T] + eps 1 and the force of src/nqs/nqs_optimizer.c:483-498 (or
    :929-941 for the real-time force)."""
    Ns = R.shape[0]
    Rm, Im = R.mean(0), I.mean(0)
    G = 2.0 * ((R.T @ R + I.T @ I) / Ns - np.outer(Rm, Rm) - np.outer(Im, Im)) + shift * np.eye(R.shape[1])
    if realtime:
        F = 2.0 * ((R.T @ Ei - I.T @ Er) / Ns - Rm * eim + Im * erm)
    else:
        F = 2.0 * ((R.T @ Er + I.T @ Ei) / Ns - Rm * erm - Im * eim)
    return np.linalg.solve(G, F)


def _holo_case():
    N, M = 8, 6
    p = O.init_params(O.OR_CRBM, N, M, 0.3, 21)
    pref = O.init_params(O.OR_CRBM, N, M, 0.3, 22)
    rng = np.random.default_rng(5)
    batch = rng.choice(np.array([-1, 1], np.int32), size=(192, N))
    return N, M, p, pref, batch, O.ham(O.OR_TFIM, N, 1, Gamma=0.8)


def test_excited_step_with_zero_penalty_is_holomorphic_sr():
    """Excited-state SR restated from src/nqs/nqs_optimizer.c:562-723: with mu = 0 the local
    energies and the force's means are unchanged, so the step is the holomorphic step bit
    for bit (the upstream unit test checks the same equivalence on energy traces)."""
    N, M, p, pref, batch, h = _holo_case()
    Eh, dh, ih = O.holo_step(h, O.Amp(O.OR_CRBM, N, M, p.copy()), batch, 1e-2, 0.02, 50, 1e-10)
    Ee, de, ie = O.excited_step(h, O.Amp(O.OR_CRBM, N, M, p.copy()), O.Amp(O.OR_CRBM, N, M, pref.copy()), 0.0,
                                batch, 1e-2, 0.02, 50, 1e-10)
    assert np.array_equal(Eh, Ee) and np.array_equal(dh, de)
    assert ih.mean_energy == ie.mean_energy and ih.cg_iterations == ie.cg_iterations


def test_excited_step_matches_dense_penalised_solve():
    """The penalty mu r conj(<r>) (r = psi_ref / psi, log-modulus difference clamped at 10)
    and the augmented means, checked against a dense solve of the same system."""
    N, M, p, pref, batch, h = _holo_case()
    mu = 0.7
    amp, ref = O.Amp(O.OR_CRBM, N, M, p.copy()), O.Amp(O.OR_CRBM, N, M, pref.copy())
    Er, Ei = O.local_energy(h, amp, batch, complex_out=True)
    la, ar = O.log_amp(amp, batch)
    lb, br = O.log_amp(ref, batch)
    r = np.exp(np.clip(lb - la, -10, 10)) * np.exp(1j * (br - ar))
    rm = r.mean()
    Eaug = Er + 1j * Ei + mu * r * np.conj(rm)
    R, I = O.gradient_complex(amp, batch)
    want = _holo_dense(R, I, Eaug.real, Eaug.imag, Er.mean() + mu * abs(rm) ** 2, Ei.mean(), 1e-2)
    Ee, de, ie = O.excited_step(h, amp, ref, mu, batch, 1e-2, 0.02, 2000, 1e-13)
    assert ie.converged == 1
    np.testing.assert_allclose(Ee, Eaug.real, rtol=0, atol=1e-12)
    assert np.linalg.norm(de - want) <= 1e-8 * np.linalg.norm(want)
    assert ie.mean_energy == pytest.approx(Er.mean(), abs=1e-12)       # the physical energy


def test_tvmc_step_matches_dense_real_time_solve():
    """Real-time tVMC (src/nqs/nqs_optimizer.c:888-993): Re(S) delta = Im(F) on the
    holomorphic metric and theta += dt delta, against a dense solve."""
    N, M, p, _, batch, h = _holo_case()
    amp = O.Amp(O.OR_CRBM, N, M, p.copy())
    Er, Ei = O.local_energy(h, amp, batch, complex_out=True)
    R, I = O.gradient_complex(amp, batch)
    want = _holo_dense(R, I, Er, Ei, Er.mean(), Ei.mean(), 1e-2, realtime=True)
    dt = 0.01
    Et, dtv, it = O.tvmc_step(h, amp, batch, 1e-2, dt, 2000, 1e-13)
    assert it.converged == 1
    assert np.linalg.norm(dtv - want) <= 1e-8 * np.linalg.norm(want)
    np.testing.assert_allclose(amp.params, p + dt * dtv, rtol=0, atol=1e-15)
    assert it.update_norm == pytest.approx(np.linalg.norm(dtv) * dt, rel=1e-12)


@pytest.mark.parametrize("name", ["p2", "trans"])
def test_symproj_gradient_complex_matches_upstream(name):
    """oracle_symproj_gradient_complex_batch restates src/nqs/nqs_symproj.c:157-261; the
    fixture is the upstream function's output on the symproj_{p2,trans} cases."""
    d = load("symproj_" + name)
    g = load("symproj_complex")
    amp = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params"], [("symproj", d["perm"], d["chars"])])
    re, im = O.symproj_gradient_complex(amp, d["spins"])
    assert rel(re, g[name + "_re"]) < 1e-12 and rel(im, g[name + "_im"]) < 1e-12
    # its real part is the real-projected symmetric gradient only for real amplitudes; the
    # imaginary part is non-trivial for the complex RBM
    assert np.abs(im).max() > 1e-3


def test_holo_step_with_symproj_gradient_identity():
    """With the trivial group (identity only, character 1) the projected gradient is the
    base gradient, so the holomorphic step with nqs_symproj_gradient_complex equals the
    plain holomorphic step."""
    N, M = 8, 6
    p = O.init_params(O.OR_CRBM, N, M, 0.3, 31)
    rng = np.random.default_rng(9)
    batch = rng.choice(np.array([-1, 1], np.int32), size=(128, N))
    h = O.ham(O.OR_TFIM, N, 1, Gamma=0.6)
    perm = np.arange(N, dtype=np.int32)
    a1 = O.Amp(O.OR_CRBM, N, M, p.copy(), [("symproj", perm, np.ones(1))])
    a2 = O.Amp(O.OR_CRBM, N, M, p.copy(), [("symproj", perm, np.ones(1))])
    E1, d1, _ = O.holo_step_sym(h, a1, batch, 1e-2, 0.01, 40, 1e-10)
    E2, d2, _ = O.holo_step(h, a2, batch, 1e-2, 0.01, 40, 1e-10)
    assert np.array_equal(E1, E2)
    assert np.linalg.norm(d1 - d2) <= 1e-13 * np.linalg.norm(d2)


def _vit_cases():
    g = np.load(os.path.join(GOLD, "ansatz_vit.npz"))
    names = sorted({k.split("__")[0] for k in g.files})
    return {n: {k.split("__")[1]: g[k] for k in g.files if k.startswith(n + "__")} for n in names}


@pytest.mark.parametrize("name", sorted(_vit_cases()))
def test_oracle_vit_matches_upstream(name):
    """The oracle's factored-attention ViT (src/nqs/nqs_ansatz.c:113-215, 357-844,
    1093-1256 in upstream's loop order) against the upstream library's outputs
    (tests/golden/ansatz_vit.npz): initialisation bit for bit, log-amplitudes, both
    gradients and the local energies."""
    from spin_based_neural_network_gb300 import abi
    d = _vit_cases()[name]
    kind, N, w = int(d["kind"]), int(d["N"]), int(d["d"])
    scale = float(d["scale"]) if float(d["scale"]) > 0 else abi.config_defaults().rbm_init_scale
    assert np.array_equal(O.init_params(kind, N, w, scale, int(d["seed"])), d["params0"])
    amp = O.Amp(kind, N, w, d["params"].copy())
    la, ar = O.log_amp(amp, d["spins"])
    assert rel(la, d["la"]) < 1e-13 and np.max(np.abs(ar - d["arg"])) < 1e-13
    assert rel(O.gradient(amp, d["spins"]), d["grad"]) < 1e-13
    gr, gi = O.gradient_complex(amp, d["spins"])
    assert rel(gr, d["grad_re"]) < 1e-13 and rel(gi, d["grad_im"]) < 1e-13
    h = O.ham(int(d["ham"]), int(d["Lx"]), int(d["Ly"]), Gamma=0.8)
    er, ei = O.local_energy(h, amp, d["spins"], complex_out=True)
    assert rel(er, d["eloc_re"]) < 1e-12 and rel(ei, d["eloc_im"]) < 1e-12


# ------------------------------------------------------------------ holomorphic SR family
# Fixtures written by tests/golden/make_holo_golden.py from the upstream library's own
# nqs_sr_step_holomorphic_full, nqs_sr_step_excited, nqs_tvmc_step_real_time and
# nqs_tvmc_step_heun (src/nqs/nqs_optimizer.c:415-524, 562-723, 830-993); the batches are
# the ones the upstream steps drew.  CG is capped at 10 iterations or converged to 1e-13,
# so the update is held to 1e-10.

HOLO_FIXTURES = ["holo_heis_crbm_marshall", "holo_tfim_crbm_converged", "holo_kagome2x2_p2_symproj"]


def holo_problem(d):
    """Oracle amplitude and Hamiltonian of a holomorphic-family fixture."""
    wrap = str(d["wrap"])
    layers = []
    if wrap == "marshall":
        layers = [("marshall", int(d["Lx"]), int(d["Ly"]))]
    elif wrap == "symproj":
        layers = [("symproj", d["perm"], d["chars"])]
    amp = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params0"].copy(), layers)
    h = O.ham(int(d["ham"]), int(d["Lx"]), int(d["Ly"]), 0, int(d["kagome_pbc"]), float(d["J"]), float(d["J2"]),
              float(d["Jz"]), float(d["Gamma"]))
    return amp, h


def check_step(info, d, amp, tol=1e-10):
    ref = d["info"]
    assert info.mean_energy == pytest.approx(ref[0], rel=1e-12)
    assert info.variance_energy == pytest.approx(ref[1], rel=1e-9)
    assert info.update_norm == pytest.approx(ref[2], rel=tol)
    assert info.cg_iterations == int(ref[4]) and info.converged == int(ref[5])
    step = d["params1"] - d["params0"]
    assert np.linalg.norm((amp.params - d["params0"]) - step) <= tol * np.linalg.norm(step)


@pytest.mark.parametrize("name", HOLO_FIXTURES)
def test_holomorphic_step_against_upstream(name):
    d = load(name)
    amp, h = holo_problem(d)
    args = (h, amp, d["batch"], float(d["shift"]), float(d["lr"]), int(d["cg_max"]), float(d["cg_tol"]))
    E, delta, info = O.holo_step_sym(*args) if int(d["sym_grad"]) else O.holo_step(*args)
    check_step(info, d, amp)


@pytest.mark.parametrize("name", ["excited_tfim_crbm", "excited_tfim_crbm_converged"])
def test_excited_step_against_upstream(name):
    d = load(name)
    amp, h = holo_problem(d)
    ref = O.Amp(int(d["kind"]), int(d["N"]), int(d["M"]), d["params_ref"].copy())
    E, delta, info = O.excited_step(h, amp, ref, float(d["mu"]), d["batch"], float(d["shift"]), float(d["lr"]),
                                    int(d["cg_max"]), float(d["cg_tol"]))
    check_step(info, d, amp)


def test_tvmc_euler_against_upstream():
    d = load("tvmc_euler_tfim_crbm")
    amp, h = holo_problem(d)
    E, delta, info = O.tvmc_step(h, amp, d["batch"], float(d["shift"]), float(d["dt"]), int(d["cg_max"]),
                                 float(d["cg_tol"]))
    check_step(info, d, amp)


def test_tvmc_heun_against_upstream():
    """Heun = two Euler forces (k1 on the first batch at theta, k2 on the second batch at the
    probe theta + dt k1), theta + dt (k1 + k2) / 2."""
    d = load("tvmc_heun_tfim_crbm")
    amp, h = holo_problem(d)
    dt = float(d["dt"])
    shift, cmax, ctol = float(d["shift"]), int(d["cg_max"]), float(d["cg_tol"])
    E1, k1, i1 = O.tvmc_step(h, amp, d["batch"], shift, dt, cmax, ctol)
    probe = amp.params.copy()
    assert np.linalg.norm(probe - d["params_probe"]) <= 1e-12 * np.linalg.norm(d["params_probe"])
    E2, k2, i2 = O.tvmc_step(h, amp, d["batch2"], shift, dt, cmax, ctol)
    final = d["params0"] + dt * (0.5 * (k1 + k2))
    step = d["params1"] - d["params0"]
    assert np.linalg.norm((final - d["params0"]) - step) <= 1e-10 * np.linalg.norm(step)
    ref = d["info"]
    assert i1.mean_energy == pytest.approx(ref[0], rel=1e-12)
    assert i1.cg_iterations + i2.cg_iterations == int(ref[4])
    assert np.linalg.norm(0.5 * (k1 + k2)) * dt == pytest.approx(ref[2], rel=1e-10)


def test_batch_exact_tfim_chains_match_free_fermions():
    """The TFIM chain instances of the multi-instance fixture (periodic, J = 1, N up to 24)
    against the free-fermion closed form of H = -sum s_i s_{i+1} - h sum sigma^x_i:
    E0 = -sum_{n=0}^{N-1} sqrt(1 + h^2 - 2 h cos(pi (2n + 1) / N)) (Jordan-Wigner, even parity
    sector; h = 1 gives the -2 / sin(pi / 2N) of the critical ring)."""
    import json
    with open(os.path.join(GOLD, "batch_exact_energies.json")) as f:
        rec = json.load(f)
    checked = 0
    for v in rec.values():
        sp = v["spec"]
        if sp["kind"] != "tfim" or sp["Ly"] != 1:
            continue
        N, h = sp["N"], sp["h"]
        k = np.pi * (2 * np.arange(N) + 1) / N
        e0 = -np.sum(np.sqrt(1.0 + h * h - 2.0 * h * np.cos(k)))
        assert v["E0"] == pytest.approx(e0, rel=1e-10, abs=1e-10), (sp, v["E0"], e0)
        checked += 1
    assert checked >= 5
