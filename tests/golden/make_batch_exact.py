"""Exact ground-state energies of the multi-instance workload's instances with
N <= 20 (bench.py: batch_instances), for its energy-error check.

Computed by the oracle's Lanczos (full reorthogonalisation; TFIM on the full
basis, XXZ in the Sz = 0 sector), pinned against the upstream Lanczos results
in tests/test_oracle_pin.py.  Writes tests/golden/batch_exact_energies.json;
bench.py reads only that file.

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


def main(max_n=20):
    out = {}
    for i, sp in enumerate(bench.batch_instances()):
        if sp["N"] > max_n:
            continue
        t0 = time.time()
        if sp["kind"] == "tfim":
            h = O.ham(O.OR_TFIM, sp["Lx"], sp["Ly"], pbc=1, J=1.0, Gamma=sp["h"])
            nd = -1
        else:
            h = O.ham(O.OR_XXZ, sp["Lx"], sp["Ly"], pbc=1, J=1.0, Jz=sp["delta"])
            nd = sp["N"] // 2
        e = O.exact_energy(h, n_down=nd, max_iters=160, tol=1e-12)
        out[str(i)] = {"E0": e, "E0_per_site": e / sp["N"], "spec": sp}
        print(i, sp["kind"], sp["N"], sp["Lx"], sp["Ly"], e / sp["N"], "%.1fs" % (time.time() - t0), flush=True)
    with open(os.path.join(HERE, "batch_exact_energies.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
