"""Factored-attention ViT ansatz (real and complex) on the GPU against outputs of the
upstream library (tests/golden/ansatz_vit.npz, written by tests/golden/make_vit_golden.py
from the reference compiled out of its own sources): parameter initialisation bit for bit,
log-amplitudes, real-projected and holomorphic gradients to 1e-12, local energies through
the ViT to 1e-12; and the upstream unit tests' checks (tests/test_nqs_vit.c: parameter
counts, finite-difference gradients, SR descent on the 2x2 TFIM).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    N.set_options()
    return N


def cases():
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ansatz_vit.npz"))
    names = sorted({k.split("__")[0] for k in g.files})
    return {n: {k.split("__")[1]: g[k] for k in g.files if k.startswith(n + "__")} for n in names}


CASES = cases()


def rel(a, b, floor=1.0):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def make(nqs, g, set_params=True):
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=int(g["kind"]), width=int(g["d"]), rng_seed=int(g["seed"]),
                              hamiltonian=int(g["ham"]), transverse_field=0.8)
    if float(g["scale"]) > 0:
        cfg.rbm_init_scale = float(g["scale"])
    a = nqs.Ansatz(cfg, int(g["N"]))
    init = a.params.copy()
    if set_params:
        a.params[:] = g["params"]
    return cfg, a, init


@pytest.mark.parametrize("name", sorted(CASES))
def test_vit_against_reference(nqs, name):
    g = CASES[name]
    cfg, a, init = make(nqs, g)
    assert a.P == int(g["P"])
    assert np.array_equal(init, g["params0"])                       # upstream initialisation
    assert nqs.lib().nqs_ansatz_is_complex(a.h) == (1 if int(g["kind"]) == 7 else 0)
    la, ar = nqs.log_amp_batch(a.log_amp_fn, a.user, g["spins"])
    assert rel(la, g["la"]) < TOL and np.max(np.abs(ar - g["arg"])) < TOL
    P = a.P
    B = len(g["spins"])
    re, im = np.zeros((B, P)), np.zeros((B, P))
    s = np.ascontiguousarray(g["spins"], dtype=np.int32)
    L = nqs.lib()
    assert L.nqs_gpu_gradient_batch(a.h, None, None, s.ctypes.data_as(nqs.IP), B, 0,
                                    re.ctypes.data_as(nqs.DP), None) == 0
    assert rel(re, g["grad"]) < TOL
    assert L.nqs_gpu_gradient_batch(a.h, None, None, s.ctypes.data_as(nqs.IP), B, 1,
                                    re.ctypes.data_as(nqs.DP), im.ctypes.data_as(nqs.DP)) == 0
    assert rel(re, g["grad_re"]) < TOL and rel(im, g["grad_im"]) < TOL
    er, ei = nqs.local_energy_batch(cfg, int(g["Lx"]), int(g["Ly"]), g["spins"], a.log_amp_fn, a.user,
                                    complex_out=True)
    assert rel(er, g["eloc_re"]) < TOL and rel(ei, g["eloc_im"]) < TOL


def test_vit_parameter_counts(nqs):
    """P = 3 d + d^2 + N + 1 (real), 6 d + 2 d^2 + N + 2 (complex); upstream
    tests/test_nqs_vit.c:23-34, :150-162."""
    from spin_based_neural_network_gb300 import abi
    for kind, want in ((abi.ANSATZ_FACTORED_VIT, 35), (abi.ANSATZ_FACTORED_VIT_COMPLEX, 64)):
        a = nqs.Ansatz(abi.config_defaults(ansatz=kind, width=4, rng_seed=0xCAFEFACE), 6)
        assert a.P == want


@pytest.mark.parametrize("name", ["vit_n8_d6", "vitc_n8_d6"])
def test_vit_gradient_matches_finite_difference(nqs, name):
    """Central differences of the device log-amplitude (upstream tests/test_nqs_vit.c:73-106,
    :184-262): real projection d log|psi|, and d arg psi for the holomorphic imaginary part."""
    g = CASES[name]
    _, a, _ = make(nqs, g)
    s = np.ascontiguousarray(g["spins"][:3], dtype=np.int32)
    P, B, h = a.P, len(s), 1e-5
    L = nqs.lib()
    re, im = np.zeros((B, P)), np.zeros((B, P))
    assert L.nqs_gpu_gradient_batch(a.h, None, None, s.ctypes.data_as(nqs.IP), B, 1,
                                    re.ctypes.data_as(nqs.DP), im.ctypes.data_as(nqs.DP)) == 0
    p0 = a.params.copy()
    fd_re, fd_im = np.zeros((B, P)), np.zeros((B, P))
    for k in range(P):
        a.params[:] = p0
        a.params[k] += h
        lp, ap = nqs.log_amp_batch(a.log_amp_fn, a.user, s)
        a.params[:] = p0
        a.params[k] -= h
        lm, am = nqs.log_amp_batch(a.log_amp_fn, a.user, s)
        fd_re[:, k] = (lp - lm) / (2 * h)
        fd_im[:, k] = (ap - am) / (2 * h)
    a.params[:] = p0
    assert np.max(np.abs(fd_re - re)) < 1e-7
    assert np.max(np.abs(fd_im - im)) < 1e-7


def test_vit_descends_on_tfim_2x2(nqs):
    """CG-SR with the real ViT on the 2x2 TFIM: training does not blow up and the tail is
    not above the head by more than 0.5 (upstream tests/test_nqs_vit.c:108-148)."""
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_FACTORED_VIT, width=4, hamiltonian=abi.HAM_TFIM, j_coupling=1.0,
                              transverse_field=1.0, num_samples=256, num_thermalize=128, num_decorrelate=2,
                              num_iterations=30, learning_rate=5e-2, sr_diag_shift=1e-2, sr_cg_max_iters=40,
                              rng_seed=0xBA5E5EED)
    a = nqs.Ansatz(cfg, 4)
    s = nqs.Sampler(4, cfg, a.log_amp_fn, a.user)
    trace = np.zeros(30)
    assert nqs.lib().nqs_sr_run(C.byref(cfg), 2, 2, a.h, s.h, trace.ctypes.data_as(nqs.DP)) == 0
    assert np.all(np.isfinite(trace))
    assert trace[-5:].mean() < trace[:5].mean() + 0.5


def test_complex_vit_holomorphic_run(nqs):
    """Holomorphic SR drives the complex ViT on the 2x2 TFIM without blowing up."""
    from spin_based_neural_network_gb300 import abi
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_FACTORED_VIT_COMPLEX, width=4, rbm_init_scale=0.1,
                              hamiltonian=abi.HAM_TFIM, transverse_field=1.0, num_samples=512,
                              num_iterations=30, learning_rate=5e-2, sr_diag_shift=1e-2, sr_cg_max_iters=40,
                              rng_seed=7)
    a = nqs.Ansatz(cfg, 4)
    s = nqs.Sampler(4, cfg, a.log_amp_fn, a.user)
    trace = np.zeros(30)
    assert nqs.lib().nqs_sr_run_holomorphic(C.byref(cfg), 2, 2, a.h, s.h, a.log_amp_fn, a.user,
                                           trace.ctypes.data_as(nqs.DP)) == 0
    assert np.all(np.isfinite(trace))
    assert trace[-5:].mean() < trace[:5].mean() + 0.5
