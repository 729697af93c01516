"""Golden vectors for the magnetisation-sector lean Lanczos, from the upstream library itself.

The upstream sector drivers (scripts/research_kagome_spin_gap.c, research_kagome_sz_spatial.c)
run the library's lanczos_smallest_projected_lean (src/mps/lanczos.c:824-960) with a
projector that zeroes every amplitude whose popcount (number of down spins) differs from
the target and then, for a spatial sector, applies nqs_kagome_p6m_project_inplace
(src/nqs/nqs_symproj.c:786-852).  Their seed is xorshift64 u - 1/2 from a driver-specific
state (0xA5A5A5A5A5A5A5A5 ^ 2^N for the Sz sectors alone, 0xC3C3C3C3C3C3C3C3 ^ 2^N ^
irrep * 0x9E3779B97F4A7C15 with a p6m irrep), projected and normalised (times 1/sqrt of
the squared norm), then handed to the Lanczos as its initial vector.

This script runs that protocol on the periodic 2 x 2 kagome torus (N = 12) through the
compiled upstream library (oracle/_ref/libnqs_ref.so): the library's lean Lanczos and
p6m projector, with the drivers' matvec (the same Hamiltonian as the library's
kagome_heis_matvec, src/nqs/nqs_lanczos.c:380-432) and projector restated as ctypes
callbacks.  It records E0, the iteration count and the first tridiagonal coefficients
of each sector, plus the recorded 2 x 2 spin-gap runs and the recorded 3 x 3
(Sz = 1/2, Gamma, E2) run from the upstream results (benchmarks/results/nqs/full_analysis/).

Writes tests/golden/kagome_sz_ed.json.  Runs here only (needs the built reference).
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from link_upstream_tests import default_reference  # noqa: E402

IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
MATVEC = C.CFUNCTYPE(None, DP, DP, C.c_long, C.c_void_p)
PROJECT = C.CFUNCTYPE(None, DP, C.c_long, C.c_void_p)
IRREPS = ["A1", "A2", "B1", "B2", "E1", "E2"]


class LanczosResult(C.Structure):
    _fields_ = [("eigenvalue", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("residual_norm", C.c_double)]


def load():
    so = os.path.join(ROOT, "oracle", "_ref", "libnqs_ref.so")
    if not os.path.exists(so):
        raise SystemExit("build the reference first: make -C oracle REF=<upstream checkout>")
    L = C.CDLL(so)
    L.lanczos_smallest_projected_lean.argtypes = [MATVEC, C.c_void_p, C.c_long, C.c_int, C.c_double, DP, PROJECT,
                                                  C.c_void_p, DP, C.POINTER(LanczosResult)]
    L.nqs_kagome_p6m_perm_irrep.argtypes = [C.c_int, C.c_int, C.POINTER(IP), C.POINTER(DP), IP]
    L.nqs_kagome_p6m_project_inplace.argtypes = [DP, C.c_int, C.c_int, IP, DP]
    return L


def kagome_bonds(L):
    """Up- and down-triangle bonds of the periodic L x L kagome torus in the drivers' order."""
    up, dn = [], []
    for cx in range(L):
        for cy in range(L):
            A, B, Cc = 3 * (cx * L + cy), 3 * (cx * L + cy) + 1, 3 * (cx * L + cy) + 2
            cxm, cym = (cx - 1 + L) % L, (cy - 1 + L) % L
            Bm, Cm = 3 * (cxm * L + cy) + 1, 3 * (cx * L + cym) + 2
            up += [(A, B), (A, Cc), (B, Cc)]
            dn += [(A, Bm), (A, Cm), (Bm, Cm)]
    return up + dn


def make_matvec(L, J=1.0):
    N = 3 * L * L
    dim = 1 << N
    s = np.arange(dim, dtype=np.int64)
    spin = 1 - 2 * ((s[:, None] >> np.arange(N)) & 1)            # +1 up, -1 down
    bonds = kagome_bonds(L)
    diag = 0.25 * J * sum(spin[:, u] * spin[:, v] for u, v in bonds)
    flips = [(spin[:, u] != spin[:, v], s ^ (1 << u) ^ (1 << v)) for u, v in bonds]

    def mv(xin, xout, n, ud):
        x = np.ctypeslib.as_array(xin, shape=(dim,))
        y = diag * x
        for anti, partner in flips:
            y = y + np.where(anti, 0.5 * J * x[partner], 0.0)
        np.ctypeslib.as_array(xout, shape=(dim,))[:] = y
    return MATVEC(mv)


def make_project(Lib, N, popcount, perm=None, chars=None):
    dim = 1 << N
    keep = np.array([bin(i).count("1") == popcount for i in range(dim)])

    def pr(vec, n, ud):
        v = np.ctypeslib.as_array(vec, shape=(dim,))
        v[~keep] = 0.0
        if perm is not None:
            Lib.nqs_kagome_p6m_project_inplace(vec, N, len(chars), perm.ctypes.data_as(IP), chars.ctypes.data_as(DP))
    return PROJECT(pr)


def xorshift_seed(state, dim):
    out = np.empty(dim)
    x = state
    M = 0xFFFFFFFFFFFFFFFF
    for i in range(dim):
        x ^= (x << 13) & M
        x ^= x >> 7
        x ^= (x << 17) & M
        out[i] = (x >> 11) / 9007199254740992.0 - 0.5
    return out


def run(Lib, L, popcount, irrep=None, max_iters=200, tol=1e-10):
    N = 3 * L * L
    dim = 1 << N
    perm = chars = None
    if irrep is not None:
        p, ch, G = IP(), DP(), C.c_int()
        assert Lib.nqs_kagome_p6m_perm_irrep(L, IRREPS.index(irrep), C.byref(p), C.byref(ch), C.byref(G)) == 0
        perm = np.ctypeslib.as_array(p, (G.value * N,)).copy().astype(np.int32)
        chars = np.ctypeslib.as_array(ch, (G.value,)).copy()
        state = (0xC3C3C3C3C3C3C3C3 ^ dim ^ ((IRREPS.index(irrep) * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF))
    else:
        state = 0xA5A5A5A5A5A5A5A5 ^ dim
    mv = make_matvec(L)
    pr = make_project(Lib, N, popcount, perm, chars)
    seed = xorshift_seed(state, dim)
    pr(seed.ctypes.data_as(DP), dim, None)
    n2 = float(np.sum(seed * seed))
    seed *= 1.0 / np.sqrt(n2)
    e, res = C.c_double(), LanczosResult()
    assert Lib.lanczos_smallest_projected_lean(mv, None, dim, max_iters, tol, seed.ctypes.data_as(DP), pr, None,
                                               C.byref(e), C.byref(res)) == 0
    return {"L": L, "N": N, "popcount": popcount, "irrep": irrep, "seed_state": state, "max_iters": max_iters,
            "tol": tol, "E0": e.value, "iterations": res.iterations, "converged": res.converged}


def main():
    Lib = load()
    out = {"runs": []}
    for pc in (6, 5):
        out["runs"].append(run(Lib, 2, pc))
    for irrep in ("A1", "B1", "E2"):
        out["runs"].append(run(Lib, 2, 6, irrep))
    ref = default_reference()
    rec = {}
    base = os.path.join(ref, "benchmarks", "results", "nqs", "full_analysis") if ref else None
    for name in ("spin_gap_L2_Sz0", "spin_gap_L2_Sz1", "L3_ir5_E2_sz1"):
        path = os.path.join(base, name + ".json") if base else None
        if path and os.path.exists(path):
            with open(path) as f:
                rec[name] = json.load(f)
    out["recorded_upstream_runs"] = rec
    with open(os.path.join(HERE, "kagome_sz_ed.json"), "w") as f:
        json.dump(out, f, indent=1)
    for r in out["runs"]:
        print(r)
    print("recorded:", {k: v.get("lanczos") for k, v in rec.items()})


if __name__ == "__main__":
    main()
