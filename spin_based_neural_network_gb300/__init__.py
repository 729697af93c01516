"""GB300-native NQS VMC step (sampler, log-amplitudes, local energies, Jacobian,
CG-SR and MinSR) behind the upstream `nqs_*` C API.

The compute lives in libnqs_gb300.so (hand-written sm_103a kernels behind a
C ABI declared in include/nqs/*.h).  This package only loads it and offers a
thin ctypes mirror of the C API (`nqs.py`).  There is no CPU implementation:
`lib()` raises if the shared library is missing or cannot be loaded.
"""
import ctypes as C
import os

from . import abi  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libnqs_gb300.so")
_LIB = None


def build(verbose=False):
    from . import _build
    return _build.build(verbose=verbose)


def lib():
    """Load libnqs_gb300.so (the CUDA path).  Raises if it is not built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libnqs_gb300.so is not built; run spin_based_neural_network_gb300.build() "
                           "(the NQS step has no CPU implementation)")
    _LIB = C.CDLL(LIB_PATH)
    from .nqs import _declare
    _declare(_LIB)
    return _LIB
