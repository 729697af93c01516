"""Exact ground-state energies of the multi-instance workload's instances with
N <= 24 (bench.py: batch_instances), for its energy-error check.

Computed by the oracle's Lanczos (full reorthogonalisation; TFIM on the full
basis, XXZ in the Sz = 0 sector), pinned against the upstream Lanczos results
in tests/test_oracle_pin.py.  Writes tests/golden/batch_exact_energies.json;
bench.py reads only that file.

Entries already in the file are kept; the missing ones are computed in two worker
processes (the N = 24 TFIM instances hold 2^24 x 161 Krylov vectors, ~22 GB each).

Run: python tests/golden/make_batch_exact.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle_lib as O  # noqa: E402
import bench  # noqa: E402


def solve(item):
    i, sp = item
    t0 = time.time()
    if sp["kind"] == "tfim":
        h = O.ham(O.OR_TFIM, sp["Lx"], sp["Ly"], pbc=1, J=1.0, Gamma=sp["h"])
        nd = -1
    else:
        h = O.ham(O.OR_XXZ, sp["Lx"], sp["Ly"], pbc=1, J=1.0, Jz=sp["delta"])
        nd = sp["N"] // 2
    e = O.exact_energy(h, n_down=nd, max_iters=160, tol=1e-12)
    print(i, sp["kind"], sp["N"], sp["Lx"], sp["Ly"], e / sp["N"], "%.1fs" % (time.time() - t0), flush=True)
    return str(i), {"E0": e, "E0_per_site": e / sp["N"], "spec": sp}


def main(max_n=24, workers=2):
    import multiprocessing as mp
    path = os.path.join(HERE, "batch_exact_energies.json")
    out = {}
    if os.path.exists(path):
        with open(path) as f:
            out = json.load(f)
    todo = [(i, sp) for i, sp in enumerate(bench.batch_instances()) if sp["N"] <= max_n and str(i) not in out]
    with mp.get_context("spawn").Pool(workers) as pool:
        for k, v in pool.imap_unordered(solve, todo):
            out[k] = v
            with open(path, "w") as f:
                json.dump(dict(sorted(out.items(), key=lambda kv: int(kv[0]))), f, indent=1)


if __name__ == "__main__":
    main()
