"""Golden vectors for the translation projector and the kagome p3 / p6 tables.

Runs the upstream nqs_translation_log_amp / nqs_translation_gradient
(src/nqs/nqs_translation.c:23-145) and nqs_kagome_p3_perm / nqs_kagome_p6_perm
(src/nqs/nqs_symproj.c:436-590) from the reference compiled out of its own sources
(oracle/_ref/libnqs_ref.so).  Writes tests/golden/translation.npz.
Run: python tests/golden/make_translation_golden.py
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
    L.nqs_translation_gradient.argtypes = [C.c_void_p, C.c_void_p, IP, C.c_int, DP]
    fn_t = C.CFUNCTYPE(None, IP, C.c_int, C.c_void_p, DP, DP)(MG.fnptr(L, "nqs_translation_log_amp"))
    rng = np.random.default_rng(31)
    out = {}
    for name, kind, Lx, Ly, marshall in (("rbm_4x3", abi.ANSATZ_RBM, 4, 3, False),
                                         ("crbm_4x4_marshall", abi.ANSATZ_COMPLEX_RBM, 4, 4, True),
                                         ("rbm_chain8", abi.ANSATZ_RBM, 8, 1, False)):
        N = Lx * Ly
        cfg = abi.config_defaults(ansatz=kind, rbm_hidden_units=N, rbm_init_scale=0.5, rng_seed=606)
        a = L.nqs_ansatz_create(C.byref(cfg), N)
        p = MG.params_of(L, a)
        keep = []
        if marshall:
            m = abi.MarshallWrapper(MG.fnptr(L, "nqs_ansatz_log_amp"), a, Lx, Ly)
            keep.append(m)
            base_fn, base_user = MG.fnptr(L, "nqs_marshall_log_amp"), C.addressof(m)
        else:
            base_fn, base_user = MG.fnptr(L, "nqs_ansatz_log_amp"), a
        w = abi.TranslationWrapper(base_fn, base_user, Lx, Ly)
        spins = MG.rand_spins(rng, 24, N)
        la, ar = np.zeros(24), np.zeros(24)
        g = np.zeros((24, len(p)))
        for b in range(24):
            sp = spins[b].ctypes.data_as(IP)
            l, t = C.c_double(), C.c_double()
            fn_t(sp, N, C.addressof(w), C.byref(l), C.byref(t))
            la[b], ar[b] = l.value, t.value
            assert L.nqs_translation_gradient(C.addressof(w), a, sp, N, g[b].ctypes.data_as(DP)) == 0
        out[name] = dict(kind=kind, Lx=Lx, Ly=Ly, marshall=int(marshall), params=p, spins=spins, la=la, arg=ar,
                         grad=g)
        L.nqs_ansatz_free(a)
    for fname in ("p3", "p6"):
        f = getattr(L, "nqs_kagome_%s_perm" % fname)
        for Lc in (2, 3):
            pp, ch, G = IP(), DP(), C.c_int()
            assert f(Lc, C.byref(pp), C.byref(ch), C.byref(G)) == 0
            out["%s_L%d" % (fname, Lc)] = dict(
                perm=np.ctypeslib.as_array(pp, (G.value * 3 * Lc * Lc,)).copy().astype(np.int32),
                chars=np.ctypeslib.as_array(ch, (G.value,)).copy())
    flat = {"%s__%s" % (c, k): np.asarray(v) for c, dd in out.items() for k, v in dd.items()}
    np.savez_compressed(os.path.join(HERE, "translation.npz"), **flat)
    print(list(out))


if __name__ == "__main__":
    main()
