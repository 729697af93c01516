"""Golden vectors for the exact-diagonalisation path (memory-lean projecting Lanczos).

Generated by running the upstream reference itself, compiled from its sources by
oracle/Makefile into oracle/_ref/libnqs_ref.so:
  nqs_kagome_p6m_perm_irrep                                (src/nqs/nqs_symproj.c:738-776)
  nqs_kagome_translation_perm                              (src/nqs/nqs_symproj.c:269-301)
  nqs_lanczos_e0_kagome_heisenberg_projected_lean[_eigvec] (src/nqs/nqs_lanczos.c:629-672)
  nqs_kagome_p6m_project_inplace                           (src/nqs/nqs_symproj.c:786-852)
plus the upstream recorded 3 x 3 sector spectrum
(benchmarks/results/nqs/kagome_3x3_e0_sector_spectrum.json, 2^27 states, which the
reference needs ~2.8-3.6 ks per sector for on 14 threads).

Writes tests/golden/kagome_lean_ed.json and tests/golden/kagome_ed_vectors.npz.
Run: python tests/golden/make_ed_golden.py  (needs oracle/_ref built from the reference)
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libnqs_ref.so")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from link_upstream_tests import default_reference  # noqa: E402

REF_SRC = default_reference()   # $NQS_REFERENCE_SRC or the checkout oracle/_ref was built from
IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)


class LanczosResult(C.Structure):
    _fields_ = [("eigenvalue", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("residual_norm", C.c_double)]


def p6m(ref, L, irrep):
    p, ch, G = IP(), DP(), C.c_int()
    assert ref.nqs_kagome_p6m_perm_irrep(L, irrep, C.byref(p), C.byref(ch), C.byref(G)) == 0
    N = 3 * L * L
    return (np.ctypeslib.as_array(p, (G.value * N,)).copy(),
            np.ctypeslib.as_array(ch, (G.value,)).copy())


def translations(ref, Lx, Ly):
    p, G = IP(), C.c_int()
    assert ref.nqs_kagome_translation_perm(Lx, Ly, C.byref(p), C.byref(G)) == 0
    return np.ctypeslib.as_array(p, (G.value * 3 * Lx * Ly,)).copy(), np.ones(G.value)


def lean(ref, Lx, Ly, pbc, perm, chars, iters, tol, eigvec=False):
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    chars = np.ascontiguousarray(chars, dtype=np.float64)
    e, r = C.c_double(), LanczosResult()
    args = [Lx, Ly, C.c_double(1.0), pbc, perm.ctypes.data_as(IP), chars.ctypes.data_as(DP), len(chars),
            iters, C.c_double(tol), C.byref(e)]
    vec = None
    if eigvec:
        vec = np.zeros(1 << (3 * Lx * Ly))
        rc = ref.nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec(*args, vec.ctypes.data_as(DP), C.byref(r))
    else:
        rc = ref.nqs_lanczos_e0_kagome_heisenberg_projected_lean(*args, C.byref(r))
    assert rc == 0
    return {"E0": e.value, "iterations": r.iterations, "converged": r.converged,
            "residual_norm": r.residual_norm}, vec


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    ref = C.CDLL(REF_SO)
    names = ["A1", "A2", "B1", "B2", "E1", "E2"]
    out = {"source": "upstream reference compiled from its sources (oracle/_ref); J = 1",
           "tol": 1e-12, "max_iters": 200, "cases": [], "perm_digests": {}}
    vectors = {}
    for L in (2, 3):
        for i, nm in enumerate(names):
            perm, chars = p6m(ref, L, i)
            out["perm_digests"]["p6m_L%d_%s" % (L, nm)] = {"perm_int32": digest(perm.astype(np.int32)),
                                                         "chars_f64": digest(chars.astype(np.float64))}
    for i, nm in enumerate(names):
        perm, chars = p6m(ref, 2, i)
        res, _ = lean(ref, 2, 2, 1, perm, chars, 200, 1e-12)
        out["cases"].append({"name": "kagome_2x2_pbc_p6m_" + nm, "Lx": 2, "Ly": 2, "pbc": 1,
                             "group": "p6m", "irrep": i, **res})
    perm, chars = translations(ref, 2, 3)
    res, _ = lean(ref, 2, 3, 1, perm, chars, 200, 1e-12)
    out["cases"].append({"name": "kagome_2x3_pbc_translations", "Lx": 2, "Ly": 3, "pbc": 1,
                         "group": "translations", "irrep": 0, **res})
    res, _ = lean(ref, 2, 2, 0, np.arange(12), np.ones(1), 300, 1e-12)
    out["cases"].append({"name": "kagome_2x2_obc_trivial", "Lx": 2, "Ly": 2, "pbc": 0, "group": "trivial",
                         "irrep": 0, "max_iters": 300, **res})
    # eigenvector of the 2 x 2 B1 sector, and a projected random vector
    perm, chars = p6m(ref, 2, 2)
    res, vec = lean(ref, 2, 2, 1, perm, chars, 200, 1e-12, eigvec=True)
    out["eigvec_2x2_B1"] = res
    vectors["eigvec_2x2_B1"] = vec
    x = np.random.default_rng(2024).standard_normal(4096)
    vectors["project_in"] = x.copy()
    for i in (0, 2, 4):
        perm, chars = p6m(ref, 2, i)
        y = x.copy()
        ref.nqs_kagome_p6m_project_inplace(y.ctypes.data_as(DP), 12, len(chars), perm.ctypes.data_as(IP),
                                           chars.ctypes.data_as(DP))
        vectors["project_out_%s" % names[i]] = y
    rec = json.load(open(os.path.join(REF_SRC, "benchmarks", "results", "nqs",
                                      "kagome_3x3_e0_sector_spectrum.json")))
    out["kagome_3x3_recorded"] = {
        "source": "benchmarks/results/nqs/kagome_3x3_e0_sector_spectrum.json (upstream run, 14 threads)",
        "max_iters": rec["method"]["lanczos_max_iters"], "tol": rec["method"]["lanczos_tol"],
        "sectors": {s["irrep"].replace("_", ""): {"E0": s["E_0"], "iters": s["iters"],
                                                 "converged": bool(s["converged"]),
                                                 "independent_ED": s["libirrep_ED_reference"],
                                                 "wall_seconds": s["wall_seconds"]} for s in rec["sectors"]}}
    with open(os.path.join(HERE, "kagome_lean_ed.json"), "w") as f:
        json.dump(out, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "kagome_ed_vectors.npz"), **vectors)
    print(json.dumps(out["cases"], indent=1))
    print(out["kagome_3x3_recorded"])


if __name__ == "__main__":
    main()
