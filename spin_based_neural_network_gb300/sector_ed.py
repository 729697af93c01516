"""Sector ground-state energy of the kagome Heisenberg model by the device's memory-lean
projecting Lanczos (the job of the upstream driver scripts/research_kagome_3x3_e0.c).

    python -m spin_based_neural_network_gb300.sector_ed --L 3 --irrep A1
    python -m spin_based_neural_network_gb300.sector_ed --Lx 2 --Ly 4 --group translations

Prints one JSON line: E0, iterations, converged, residual and the wall time.
"""
import argparse
import json
import time

from . import nqs


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--L", type=int, default=None, help="L x L torus (sets --Lx and --Ly)")
    ap.add_argument("--Lx", type=int, default=3)
    ap.add_argument("--Ly", type=int, default=3)
    ap.add_argument("--group", default="p6m", choices=["p6m", "translations", "p2"])
    ap.add_argument("--irrep", default="A1", choices=sorted(nqs.P6M_IRREPS))
    ap.add_argument("--J", type=float, default=1.0)
    ap.add_argument("--obc", action="store_true", help="open boundaries (default periodic)")
    ap.add_argument("--max-iters", type=int, default=100)
    ap.add_argument("--tol", type=float, default=1e-9)
    a = ap.parse_args(argv)
    Lx, Ly = (a.L, a.L) if a.L else (a.Lx, a.Ly)
    perm, chars = nqs.kagome_perm(Lx, Ly, a.group, a.irrep)
    t0 = time.perf_counter()
    e, _, res = nqs.lanczos_e0_kagome_lean(Lx, Ly, a.J, 0 if a.obc else 1, perm, chars, a.max_iters, a.tol)
    wall = time.perf_counter() - t0
    print(json.dumps({"Lx": Lx, "Ly": Ly, "sites": 3 * Lx * Ly, "group": a.group, "irrep": a.irrep,
                      "group_order": len(chars), "E0": e, "E0_per_site": e / (3 * Lx * Ly), **res,
                      "wall_s": wall}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
