"""The upstream NQS unit tests compile against include/ and link against libnqs_gb300.so
unchanged (oracle/link_upstream_tests.py).  Needs the upstream sources and the built
library; skipped where either is absent."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# upstream test files whose every symbol the drop-in provides
LINKING = ["test_nqs", "test_nqs_complex_rbm", "test_nqs_convergence", "test_nqs_excited",
           "test_nqs_holomorphic_sr", "test_nqs_kagome", "test_nqs_kitaev", "test_nqs_kspace_ed",
           "test_nqs_marshall", "test_nqs_minsr", "test_nqs_rbm", "test_nqs_sector_projected",
           "test_nqs_symproj", "test_nqs_translation", "test_nqs_tvmc", "test_nqs_vit"]


def test_upstream_nqs_tests_link_against_the_drop_in():
    import link_upstream_tests as LU
    ref = LU.default_reference()
    if not ref or not os.path.isdir(os.path.join(ref, "tests")):
        pytest.skip("upstream sources not present")
    if not os.path.exists(os.path.join(LU.LIBDIR, "libnqs_gb300.so")):
        pytest.skip("library not built")
    res = LU.check(ref)
    bad = {k: v for k, v in res.items() if k in LINKING and v != "links"}
    assert not bad, bad
