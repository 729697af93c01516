"""Golden vectors for the factored-attention ViT ansatz (real and complex).

Runs the upstream library, compiled from its own sources into oracle/_ref/libnqs_ref.so:
nqs_ansatz_create (parameter initialisation, src/nqs/nqs_ansatz.c:113-215),
nqs_ansatz_log_amp (:357-473, :571-729), nqs_ansatz_logpsi_gradient (:475-567, :732-843),
nqs_ansatz_logpsi_gradient_complex (:1093-1256) and nqs_local_energy_batch[_complex] with
the ViT log-amplitude (TFIM chain and Heisenberg 4x2).  Writes tests/golden/ansatz_vit.npz.
Run: python tests/golden/make_vit_golden.py
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
CASES = [  # name, kind, N, d, scale, seed, hamiltonian, Lx, Ly
    ("vit_n6_d4", abi.ANSATZ_FACTORED_VIT, 6, 4, 0.0, 0xCAFEFACE, abi.HAM_TFIM, 6, 1),
    ("vitc_n6_d4", abi.ANSATZ_FACTORED_VIT_COMPLEX, 6, 4, 0.0, 0xCAFEBABE, abi.HAM_TFIM, 6, 1),
    ("vit_n8_d6", abi.ANSATZ_FACTORED_VIT, 8, 6, 0.6, 77, abi.HAM_HEISENBERG, 4, 2),
    ("vitc_n8_d6", abi.ANSATZ_FACTORED_VIT_COMPLEX, 8, 6, 0.6, 78, abi.HAM_HEISENBERG, 4, 2),
    ("vitc_n16_d8", abi.ANSATZ_FACTORED_VIT_COMPLEX, 16, 8, 0.4, 79, abi.HAM_TFIM, 16, 1),
]


def main():
    L = MG.load_ref()
    rng = np.random.default_rng(123)
    out = {}
    for name, kind, N, d, scale, seed, ham, Lx, Ly in CASES:
        cfg = abi.config_defaults(ansatz=kind, width=d, rng_seed=seed, hamiltonian=ham, transverse_field=0.8)
        if scale > 0:
            cfg.rbm_init_scale = scale
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        assert a
        P = L.nqs_ansatz_num_params(a)
        params0 = MG.params_of(L, a)
        if scale == 0.0:                      # also check a larger, non-trivial point
            raw = np.ctypeslib.as_array(L.nqs_ansatz_params_raw(a), shape=(P,))
            raw[:] = params0 + 0.4 * rng.standard_normal(P)
        params = MG.params_of(L, a)
        spins = MG.rand_spins(rng, 40, N)
        la, ar = np.zeros(40), np.zeros(40)
        g = np.zeros((40, P))
        gr, gi = np.zeros((40, P)), np.zeros((40, P))
        for b in range(40):
            sp = spins[b].ctypes.data_as(IP)
            l, t = C.c_double(), C.c_double()
            L.nqs_ansatz_log_amp(sp, N, a, C.byref(l), C.byref(t))
            la[b], ar[b] = l.value, t.value
            assert L.nqs_ansatz_logpsi_gradient(a, sp, N, g[b].ctypes.data_as(DP)) == 0
            assert L.nqs_ansatz_logpsi_gradient_complex(a, sp, N, gr[b].ctypes.data_as(DP),
                                                         gi[b].ctypes.data_as(DP)) == 0
        er, ei = np.zeros(40), np.zeros(40)
        L.nqs_local_energy_batch_complex(C.byref(cfg), Lx, Ly, spins.ctypes.data_as(IP), 40,
                                         MG.fnptr(L, "nqs_ansatz_log_amp"), a, er.ctypes.data_as(DP),
                                         ei.ctypes.data_as(DP))
        out[name] = dict(kind=kind, N=N, d=d, scale=scale, seed=seed, ham=ham, Lx=Lx, Ly=Ly, P=P,
                         params0=params0, params=params, spins=spins, la=la, arg=ar, grad=g, grad_re=gr,
                         grad_im=gi, eloc_re=er, eloc_im=ei)
        L.nqs_ansatz_free(a)
    flat = {"%s__%s" % (c, k): np.asarray(v) for c, dd in out.items() for k, v in dd.items()}
    np.savez_compressed(os.path.join(HERE, "ansatz_vit.npz"), **flat)
    print(list(out))


if __name__ == "__main__":
    main()
