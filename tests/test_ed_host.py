"""Exact-diagonalisation path, CPU side: the p6m tables of the product, the projector's
subgroup factorisation, and the oracle pinned against outputs of the upstream library
(tests/golden/kagome_lean_ed.json and kagome_ed_vectors.npz, written by
tests/golden/make_ed_golden.py from the reference compiled out of its own sources).
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from spin_based_neural_network_gb300 import nqs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ED = json.load(open(os.path.join(GOLD, "kagome_lean_ed.json")))
VEC = dict(np.load(os.path.join(GOLD, "kagome_ed_vectors.npz")))
IRREPS = ["A1", "A2", "B1", "B2", "E1", "E2"]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def group(case):
    if case["group"] == "p6m":
        return nqs.kagome_perm(case["Lx"], case["Ly"], "p6m", IRREPS[case["irrep"]])
    if case["group"] == "translations":
        return nqs.kagome_perm(case["Lx"], case["Ly"], "translations")
    N = 3 * case["Lx"] * case["Ly"]
    return np.arange(N, dtype=np.int32).reshape(1, N), np.ones(1)


def bit_permute(perm_row, s):
    out = np.zeros_like(s)
    for i, j in enumerate(perm_row):
        out |= ((s >> int(j)) & 1) << i
    return out


@pytest.mark.parametrize("L", [2, 3])
@pytest.mark.parametrize("irrep", IRREPS)
def test_p6m_tables_match_upstream(L, irrep):
    perm, chars = nqs.kagome_perm(L, L, "p6m", irrep)
    want = ED["perm_digests"]["p6m_L%d_%s" % (L, irrep)]
    assert perm.shape == (12 * L * L, 3 * L * L)
    assert digest(perm.astype(np.int32).reshape(-1)) == want["perm_int32"]
    assert digest(chars.astype(np.float64)) == want["chars_f64"]


@pytest.mark.parametrize("spec", [(2, "p6m", "A1"), (2, "p6m", "B2"), (2, "p6m", "E1"),
                                  (3, "p6m", "A1"), (3, "p6m", "E2"), (2, "translations", None)])
def test_projector_plan_reproduces_direct_sum(spec):
    L, grp, irrep = spec
    Lx, Ly = (L, L) if grp == "p6m" else (2, 3)
    perm, chars = nqs.kagome_perm(Lx, Ly, grp, irrep or "A1")
    N, G = perm.shape[1], len(chars)
    passes, sizes, elems = nqs.projector_plan(N, perm, chars)
    assert len(elems) == sum(sizes) and elems.min() >= 0 and elems.max() < G
    if irrep in ("E1", "E2"):                           # traces of a 2-D irrep do not factor;
        assert passes == 1 and sizes == [int(np.count_nonzero(chars))]   # chi = 0 is dropped
    else:
        assert passes >= 2 and int(np.prod(sizes)) == G and sum(sizes) < G
    if L == 3 and grp == "p6m":
        assert sum(sizes) == (18 if passes > 1 else 54)     # 3 + 3 + 12; E irreps: 54 non-zero characters
        return
    dim = 1 << N
    s = np.arange(dim, dtype=np.int64)
    x = np.random.default_rng(7).standard_normal(dim)
    direct = sum(chars[g] * x[bit_permute(perm[g], s)] for g in range(G)) / G
    if passes > 1:
        t, off = x, 0
        for sz in sizes:
            t = sum(chars[e] * t[bit_permute(perm[e], s)] for e in elems[off:off + sz])
            off += sz
        assert np.max(np.abs(t / G - direct)) < 1e-13
    # the oracle's direct form is the reference's projector (bit-identical on 2 x 2)
    if grp == "p6m" and irrep in ("A1", "E1"):
        np.testing.assert_allclose(O.sector_project(x, N, perm, chars), direct, rtol=0, atol=1e-14)


def test_projector_plan_rejects_bad_tables():
    perm = np.tile(np.arange(12, dtype=np.int32), (2, 1))
    perm[1, 3] = 4                                       # not a permutation
    with pytest.raises(nqs.NqsError):
        nqs.projector_plan(12, perm, np.ones(2))


@pytest.mark.parametrize("irrep", ["A1", "B1", "E1"])
def test_oracle_projector_matches_upstream(irrep):
    perm, chars = nqs.kagome_perm(2, 2, "p6m", irrep)
    got = O.sector_project(VEC["project_in"], 12, perm, chars)
    np.testing.assert_allclose(got, VEC["project_out_" + irrep], rtol=0, atol=1e-15)


def test_oracle_seed_is_upstream_xorshift():
    N = 10
    x = (0xA5A5A5A5A5A5A5A5 ^ (1 << N)) & (2 ** 64 - 1)
    want = []
    for _ in range(1 << N):
        x ^= (x << 13) & (2 ** 64 - 1)
        x ^= x >> 7
        x ^= (x << 17) & (2 ** 64 - 1)
        want.append((x >> 11) / 9007199254740992.0 - 0.5)
    assert np.array_equal(O.lanczos_seed(N), np.array(want))


@pytest.mark.parametrize("case", [c for c in ED["cases"] if c["Lx"] * c["Ly"] <= 4], ids=lambda c: c["name"])
def test_oracle_lean_lanczos_matches_upstream(case):
    perm, chars = group(case)
    e, _, info = O.lanczos_lean_kagome(case["Lx"], case["Ly"], 1.0, case["pbc"], perm, chars,
                                       case.get("max_iters", ED["max_iters"]), ED["tol"])
    assert abs(e - case["E0"]) < 1e-11
    assert info.iterations == case["iterations"]
    assert info.converged == case["converged"]


def test_oracle_lean_eigvec_matches_upstream():
    perm, chars = nqs.kagome_perm(2, 2, "p6m", "B1")
    e, vec, info = O.lanczos_lean_kagome(2, 2, 1.0, 1, perm, chars, ED["max_iters"], ED["tol"], eigvec=True)
    ref = ED["eigvec_2x2_B1"]
    assert abs(e - ref["E0"]) < 1e-11 and info.iterations == ref["iterations"]
    assert abs(abs(vec @ VEC["eigvec_2x2_B1"]) - 1.0) < 1e-10
    # H v = E v: the Ritz vector is the sector ground state
    hv = O.kagome_matvec(2, 2, 1.0, 1, vec)
    assert np.linalg.norm(hv - e * vec) < 1e-6


def test_recorded_3x3_sector_spectrum_is_consistent():
    rec = ED["kagome_3x3_recorded"]["sectors"]
    assert rec["A1"]["E0"] < rec["A2"]["E0"] < rec["B2"]["E0"]      # A1 is the global ground state
    for s in rec.values():
        assert abs(s["E0"] - s["independent_ED"]) < 5e-9


@pytest.mark.parametrize("group", ["p3", "p6"])
@pytest.mark.parametrize("L", [2, 3])
def test_p3_p6_tables_match_upstream(group, L):
    """nqs_kagome_p3_perm / nqs_kagome_p6_perm (rotation about the up-triangle centroid /
    the hexagon centre, then translation) equal upstream's tables
    (tests/golden/translation.npz, from the reference)."""
    g = np.load(os.path.join(GOLD, "translation.npz"))
    perm, chars = nqs.kagome_perm(L, L, group)
    assert np.array_equal(perm.astype(np.int32).reshape(-1), g["%s_L%d__perm" % (group, L)])
    assert np.array_equal(chars, g["%s_L%d__chars" % (group, L)])


@pytest.mark.parametrize("name", ["tfim_3x3_rbm", "xxz_4x3_crbm", "heis_2x4_rbm", "kagome_2x2_pbc_rbm"])
def test_oracle_dense_ed_matches_upstream(name):
    """The oracle's materialised NQS state and variational energies against upstream
    nqs_materialise_state / nqs_exact_energy_* (tests/golden/dense_ed.npz)."""
    g = np.load(os.path.join(GOLD, "dense_ed.npz"))
    d = {k.split("__")[1]: g[k] for k in g.files if k.startswith(name + "__")}
    N = int(d["N"])
    amp = O.Amp(int(d["kind"]), N, N, d["params"].copy())
    e = O.variational_energy(amp, int(d["ham"]), int(d["Lx"]), int(d["Ly"]), float(d["J"]), float(d["X"]),
                             int(d["pbc"]))
    assert abs(e - float(d["energy"])) < 1e-12 * max(1.0, abs(float(d["energy"])))
    if "psi" in d:
        np.testing.assert_allclose(O.materialise(amp, N), d["psi"], rtol=0, atol=1e-14)
