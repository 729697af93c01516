"""Exact ground-state energies of the benchmark Hamiltonians, for the
"energy error vs Lanczos" measurement.

Computed by the oracle's sector Lanczos (oracle/oracle_sampler_sr.c,
oracle_exact_energy: full reorthogonalisation, magnetisation sector basis
ranked by the combinadic), whose restatement is pinned against the upstream
nqs_lanczos_refine_* results in tests/test_oracle_pin.py.  Writes
tests/golden/exact_energies.json; bench.py reads only that file.

Run: python tests/golden/make_exact.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle_lib as O  # noqa: E402

CASES = {
    # name: (hamiltonian, Lx, Ly, pbc, couplings, n_down)
    "heisenberg_4x4_pbc_sz0": (O.OR_HEIS, 4, 4, 1, {}, 8),
    "tfim_chain16_pbc_h1": (O.OR_TFIM, 16, 1, 1, {"J": 1.0, "Gamma": 1.0}, -1),
    "heisenberg_ring16_pbc_sz0": (O.OR_HEIS, 16, 1, 1, {}, 8),
}


def main():
    out = {}
    for name, (kind, lx, ly, pbc, kw, nd) in CASES.items():
        e = O.exact_energy(O.ham(kind, lx, ly, pbc=pbc, **kw), n_down=nd, max_iters=400, tol=1e-13)
        n = lx * ly
        out[name] = {"E0": e, "E0_per_site": e / n, "sites": n, "n_down": nd,
                     "method": "oracle sector Lanczos (full reorthogonalisation)"}
        print(name, e, e / n)
    with open(os.path.join(HERE, "exact_energies.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
