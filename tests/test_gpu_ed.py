"""Exact-diagonalisation path on the GPU: the seed, the kagome matvec, the sector projector
and the memory-lean projecting Lanczos against the oracle and against outputs of the
upstream library (tests/golden/kagome_lean_ed.json, kagome_ed_vectors.npz), and the
kagome 3 x 3 sector spectrum (2^27 states) against the upstream recorded run.

Tolerances: the device sums in a different order from the reference, so vectors agree to
1e-13 (absolute, unit-scale entries) and Ritz values to 1e-11 on the small clusters;
at 2^27 states and 80-100 Krylov steps the lowest Ritz value agrees with the upstream
recorded run to 1e-8 and with the independent sector ED to 5e-9.
"""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from spin_based_neural_network_gb300 import nqs

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ED = json.load(open(os.path.join(GOLD, "kagome_lean_ed.json")))
VEC = dict(np.load(os.path.join(GOLD, "kagome_ed_vectors.npz")))
IRREPS = ["A1", "A2", "B1", "B2", "E1", "E2"]


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def group(case):
    if case["group"] == "p6m":
        return nqs.kagome_perm(case["Lx"], case["Ly"], "p6m", IRREPS[case["irrep"]])
    if case["group"] == "translations":
        return nqs.kagome_perm(case["Lx"], case["Ly"], "translations")
    N = 3 * case["Lx"] * case["Ly"]
    return np.arange(N, dtype=np.int32).reshape(1, N), np.ones(1)


def dev(torch, a):
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    torch.cuda.synchronize()                 # the library runs on its own stream
    return t


def sync(torch):
    assert nqs.lib().nqs_gpu_synchronize() == 0
    torch.cuda.synchronize()


@pytest.mark.parametrize("N", [10, 12, 18, 21])
@pytest.mark.parametrize("alt", [0, 1])
def test_seed_bit_exact(torch, N, alt):
    d = torch.zeros(1 << N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    nqs.gpu_lanczos_seed(N, alt, d.data_ptr())
    sync(torch)
    assert np.array_equal(d.cpu().numpy(), O.lanczos_seed(N, alt))


@pytest.mark.parametrize("geom", [(2, 2, 1), (2, 2, 0), (2, 3, 1), (1, 5, 1)])
def test_matvec_matches_oracle(torch, geom):
    Lx, Ly, pbc = geom
    N = 3 * Lx * Ly
    x = np.random.default_rng(N + pbc).standard_normal(1 << N)
    dy = torch.empty(1 << N, dtype=torch.float64, device="cuda")
    dx = dev(torch, x)
    nqs.gpu_kagome_heis_matvec(Lx, Ly, 0.75, pbc, dx.data_ptr(), dy.data_ptr())
    sync(torch)
    want = O.kagome_matvec(Lx, Ly, 0.75, pbc, x)
    np.testing.assert_allclose(dy.cpu().numpy(), want, rtol=0, atol=1e-13 * np.abs(want).max())


@pytest.mark.parametrize("irrep", ["A1", "B1", "E1"])
def test_project_inplace_matches_upstream(irrep):
    perm, chars = nqs.kagome_perm(2, 2, "p6m", irrep)
    got = nqs.sector_project_host(VEC["project_in"], 12, perm, chars)
    np.testing.assert_allclose(got, VEC["project_out_" + irrep], rtol=0, atol=1e-13)


@pytest.mark.parametrize("spec", [(2, "p6m", "B2"), (2, "p6m", "E2"), (2, "translations", None)])
def test_device_projector_in_and_out_of_place(torch, spec):
    L, grp, irrep = spec
    Lx, Ly = (L, L) if grp == "p6m" else (2, 3)
    perm, chars = nqs.kagome_perm(Lx, Ly, grp, irrep or "A1")
    N = perm.shape[1]
    x = np.random.default_rng(11).standard_normal(1 << N)
    want = O.sector_project(x, N, perm, chars)
    dy = torch.empty(1 << N, dtype=torch.float64, device="cuda")
    dx = dev(torch, x)
    nqs.gpu_sector_project(N, perm, chars, dx.data_ptr(), dy.data_ptr())
    nqs.gpu_sector_project(N, perm, chars, dx.data_ptr(), dx.data_ptr())
    sync(torch)
    np.testing.assert_allclose(dy.cpu().numpy(), want, rtol=0, atol=1e-13)
    np.testing.assert_allclose(dx.cpu().numpy(), want, rtol=0, atol=1e-13)
    # idempotent: P P x = P x
    nqs.gpu_sector_project(N, perm, chars, dy.data_ptr(), dx.data_ptr())
    sync(torch)
    np.testing.assert_allclose(dx.cpu().numpy(), want, rtol=0, atol=1e-13)


@pytest.mark.parametrize("case", ED["cases"], ids=lambda c: c["name"])
def test_lean_lanczos_matches_upstream(case):
    perm, chars = group(case)
    iters = case.get("max_iters", ED["max_iters"])
    e, _, res = nqs.lanczos_e0_kagome_lean(case["Lx"], case["Ly"], 1.0, case["pbc"], perm, chars, iters,
                                           ED["tol"])
    assert abs(e - case["E0"]) < 1e-11
    assert abs(res["iterations"] - case["iterations"]) <= 1
    assert res["converged"] == case["converged"]
    # the tridiagonal follows the oracle's (same seed, same recurrence)
    a, b = nqs.lanczos_last_coeffs()
    if case["Lx"] * case["Ly"] <= 4:
        eo, _, info = O.lanczos_lean_kagome(case["Lx"], case["Ly"], 1.0, case["pbc"], perm, chars, iters, ED["tol"])
        k = min(8, len(a), info.iterations)
        np.testing.assert_allclose(a[:k], np.array(info.alpha[:k]), rtol=0, atol=1e-12)
        np.testing.assert_allclose(b[1:k + 1], np.array(info.beta[1:k + 1]), rtol=0, atol=1e-12)


def test_lean_eigvec_matches_upstream():
    perm, chars = nqs.kagome_perm(2, 2, "p6m", "B1")
    e, vec, res = nqs.lanczos_e0_kagome_lean(2, 2, 1.0, 1, perm, chars, ED["max_iters"], ED["tol"], eigvec=True)
    ref = ED["eigvec_2x2_B1"]
    assert abs(e - ref["E0"]) < 1e-11
    assert res["iterations"] == ref["iterations"] and res["converged"] == ref["converged"]
    assert abs(np.linalg.norm(vec) - 1.0) < 1e-12
    assert abs(abs(vec @ VEC["eigvec_2x2_B1"]) - 1.0) < 1e-10
    hv = O.kagome_matvec(2, 2, 1.0, 1, vec)
    assert np.linalg.norm(hv - e * vec) < 1e-6
    # in the sector: P v = v
    np.testing.assert_allclose(O.sector_project(vec, 12, perm, chars), vec, rtol=0, atol=1e-12)


def test_lean_rejects_invalid_arguments():
    perm, chars = nqs.kagome_perm(2, 2, "p6m", "A1")
    with pytest.raises(nqs.NqsError):
        nqs.lanczos_e0_kagome_lean(4, 3, 1.0, 1, perm, chars, 10, 1e-9)          # N = 36 > 30
    bad = perm.copy()
    bad[5, 3] = bad[5, 4]                                                         # not a permutation
    with pytest.raises(nqs.NqsError):
        nqs.lanczos_e0_kagome_lean(2, 2, 1.0, 1, bad, chars, 10, 1e-9)


@pytest.mark.parametrize("irrep", ["A1", "B1"])
def test_kagome_3x3_sector_spectrum(irrep):
    """The upstream research run (2^27 states, max_iters 100, tol 1e-9): E0 to 1e-8 of the
    recorded value and 5e-9 of the independent sector ED; iteration count within 3."""
    rec = ED["kagome_3x3_recorded"]
    want = rec["sectors"][irrep]
    perm, chars = nqs.kagome_perm(3, 3, "p6m", irrep)
    e, _, res = nqs.lanczos_e0_kagome_lean(3, 3, 1.0, 1, perm, chars, rec["max_iters"], rec["tol"])
    assert abs(e - want["E0"]) < 1e-8
    assert abs(e - want["independent_ED"]) < 5e-9
    assert abs(res["iterations"] - want["iters"]) <= 3
    assert res["converged"] == int(want["converged"])
