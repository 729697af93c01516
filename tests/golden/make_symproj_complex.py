"""Golden vectors for the complex symmetry-projected gradient.

Runs the upstream nqs_symproj_gradient_complex (src/nqs/nqs_symproj.c:157-261), from the
reference compiled out of its own sources into oracle/_ref/libnqs_ref.so, on the same
complex RBMs, groups and spins as tests/golden/symproj_{p2,trans}.npz (written by
make_golden.py), and stores the (Re, Im) gradient rows in symproj_complex.npz.
Run: python tests/golden/make_symproj_complex.py
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


def main():
    L = MG.load_ref()
    L.nqs_symproj_gradient_complex.argtypes = [C.c_void_p, C.c_void_p, IP, C.c_int, DP, DP]
    out = {}
    for name in ("p2", "trans"):
        d = dict(np.load(os.path.join(HERE, "symproj_%s.npz" % name)))
        N, G = int(d["N"]), int(d["G"])
        cfg = abi.config_defaults(ansatz=abi.ANSATZ_COMPLEX_RBM, rbm_hidden_units=int(d["M"]))
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        P = L.nqs_ansatz_num_params(a)
        raw = np.ctypeslib.as_array(L.nqs_ansatz_params_raw(a), shape=(P,))
        raw[:] = d["params"]                              # the fixture's parameters, in place
        p = raw
        pm = np.ascontiguousarray(d["perm"], dtype=np.int32)
        ch = np.ascontiguousarray(d["chars"], dtype=np.float64)
        w = abi.SymprojWrapper(MG.fnptr(L, "nqs_ansatz_log_amp"), a, N, G, pm.ctypes.data_as(IP),
                               ch.ctypes.data_as(DP))
        spins = np.ascontiguousarray(d["spins"], dtype=np.int32)
        P = len(p)
        gr, gi = np.zeros((len(spins), P)), np.zeros((len(spins), P))
        for b in range(len(spins)):
            assert L.nqs_symproj_gradient_complex(C.addressof(w), a, spins[b].ctypes.data_as(IP), N,
                                                  gr[b].ctypes.data_as(DP), gi[b].ctypes.data_as(DP)) == 0
        out[name + "_re"], out[name + "_im"] = gr, gi
        L.nqs_ansatz_free(a)
    np.savez_compressed(os.path.join(HERE, "symproj_complex.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
