"""Host-side arithmetic of bench.py (no GPU): the algorithmic work behind the roofline
figures, the workload description both arms print, and the ncu summaries the roofline's
traffic figures are read from."""
import os

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_algorithmic_work_of_the_headline_shape():
    Ns, P = bench.NS, 2 * (bench.N_SITES + bench.M_HIDDEN + bench.N_SITES * bench.M_HIDDEN)
    assert P == 1120
    w = bench.algorithmic_work(Ns, P)
    # FP64 Gram of the sample-space system: lower triangle with the diagonal, 2 flops per FMA
    assert w["gram_fp64"] == (Ns * (Ns + 1) * P, "fp64")
    # tensor-core Gram of the smaller (parameter-space) system, three TF32 products
    assert w["gram_tc"][0] == 3 * P * (P + 1) * Ns
    assert w["gram_tc"][0] == pytest.approx(15.4e9, rel=1e-2)
    # FP32 Cholesky + triangular inverse, then (sweeps + 1) operator and preconditioner passes
    n = min(Ns, P)
    want = 2 * n ** 3 / 3 + (bench.SWEEPS + 1) * (2 * n * n + 4 * Ns * P)
    assert w["factor_refine"] == (pytest.approx(want), "fp32")
    # SYRK trailing updates of the 32-wide FP64 panels: sum over panels of rest (rest + 1) x 32
    syrk = sum((Ns - k0 - 32) * (Ns - k0 - 31) * 32 for k0 in range(0, Ns, 32))
    assert w["chol_syrk"] == (syrk, "fp64")


def test_algorithmic_work_picks_the_smaller_system():
    # sample space when N_s < N_p (the J1-J2 shape): n = N_s, K = N_p
    w = bench.algorithmic_work(8192, 10728)
    assert w["gram_tc"][0] == 3 * 8192 * 8193 * 10728


def test_headline_config_names_the_workload():
    c = bench.headline_config(1)
    assert c["workload"] == "heisenberg_4x4_pbc_crbm_alpha2_ns4096_minsr"
    assert c["num_samples"] == c["chains"] * 4 == 4096
    assert c["num_params"] == 1120 and c["parallelism"] == "replicas x1"
    assert bench.headline_config(2)["parallelism"] == "replicas x2"


def test_roofline_traffic_comes_from_committed_profiles():
    for name, (traffic, src) in bench.NCU_TRAFFIC.items():
        path = os.path.join(ROOT, src)
        assert os.path.isfile(path), src
        text = open(path).read()
        assert "dram__bytes_read.sum" in text and "dram__bytes_write.sum" in text
        # the figure in bench.py is the profile's read + write bytes
        assert traffic > 0
        assert name in bench.LIMITERS


def test_reference_arm_kind_is_the_port():
    assert bench.reference_kind() == "port"
    h = bench.host_cpu()
    assert h["nproc"] >= 1 and h["cpu_model"]
