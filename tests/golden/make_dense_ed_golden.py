"""Golden vectors for the materialised NQS state and its variational energies.

Runs upstream nqs_materialise_state and nqs_exact_energy_{tfim,heisenberg,kagome_heisenberg}
(src/nqs/nqs_lanczos.c:65-149, 188-224, 283-321, 434-455) from the reference compiled out of
its own sources (oracle/_ref/libnqs_ref.so).  Writes tests/golden/dense_ed.npz.
Run: python tests/golden/make_dense_ed_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402
from spin_based_neural_network_gb300 import abi  # noqa: E402

IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
CASES = [  # name, ansatz, Lx, Ly, ham, J, X, pbc
    ("tfim_3x3_rbm", abi.ANSATZ_RBM, 3, 3, 0, 1.0, 0.7, 0),
    ("xxz_4x3_crbm", abi.ANSATZ_COMPLEX_RBM, 4, 3, 1, 0.8, 1.4, 0),
    ("heis_2x4_rbm", abi.ANSATZ_RBM, 2, 4, 1, 1.0, 1.0, 0),
    ("kagome_2x2_pbc_rbm", abi.ANSATZ_RBM, 2, 2, 6, 1.0, 0.0, 1),
]


def main():
    L = MG.load_ref()
    L.nqs_exact_energy_tfim.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, DP]
    L.nqs_exact_energy_heisenberg.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, DP]
    L.nqs_exact_energy_kagome_heisenberg.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, DP]
    L.nqs_materialise_state.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(DP), C.POINTER(C.c_long)]
    out = {}
    for name, kind, Lx, Ly, ham, J, X, pbc in CASES:
        N = 3 * Lx * Ly if ham == 6 else Lx * Ly
        cfg = abi.config_defaults(ansatz=kind, rbm_hidden_units=N, rbm_init_scale=0.5, rng_seed=909)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p = MG.params_of(L, a)
        e = C.c_double()
        if ham == 0:
            assert L.nqs_exact_energy_tfim(a, Lx, Ly, J, X, C.byref(e)) == 0
        elif ham == 1:
            assert L.nqs_exact_energy_heisenberg(a, Lx, Ly, J, X, C.byref(e)) == 0
        else:
            assert L.nqs_exact_energy_kagome_heisenberg(a, Lx, Ly, J, pbc, C.byref(e)) == 0
        rec = dict(kind=kind, N=N, Lx=Lx, Ly=Ly, ham=ham, J=J, X=X, pbc=pbc, params=p, energy=e.value)
        if ham != 6:
            ptr, dim = DP(), C.c_long()
            assert L.nqs_materialise_state(a, Lx, Ly, C.byref(ptr), C.byref(dim)) == 0
            rec["psi"] = np.ctypeslib.as_array(ptr, (dim.value,)).copy()
        out[name] = rec
        L.nqs_ansatz_free(a)
    flat = {"%s__%s" % (c, k): np.asarray(v) for c, dd in out.items() for k, v in dd.items()}
    np.savez_compressed(os.path.join(HERE, "dense_ed.npz"), **flat)
    print({k: v["energy"] for k, v in out.items()})


if __name__ == "__main__":
    main()
