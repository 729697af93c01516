"""Effective sample size of the SR step (nqs_gpu_ess): the GPU estimator
against a numpy restatement of the same windowed estimator, and against the
known integrated autocorrelation time of AR(1) chains, tau = (1 + phi) / (1 - phi)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nqs():
    import spin_based_neural_network_gb300 as pkg
    pkg.build()
    from spin_based_neural_network_gb300 import nqs as N
    return N


def tau_numpy(E, C):
    """tau = 1 + 2 sum_{t<=M} rho(t), rho pooled over chains (rows k*C + c),
    M the smallest window with M >= 5 tau(M); lags capped at 512."""
    K = len(E) // C
    if K < 2:
        return 1.0
    x = E[:K * C].reshape(K, C) - np.mean(E)
    g0 = np.mean(x * x)
    tau = 1.0
    for t in range(1, min(K - 1, 512) + 1):
        tau += 2.0 * np.mean(x[:K - t] * x[t:]) / g0
        if t >= 5.0 * tau:
            break
    return tau


def ar1(rng, K, C, phi):
    x = np.zeros((K, C))
    x[0] = rng.normal(size=C) / np.sqrt(1 - phi * phi)
    for k in range(1, K):
        x[k] = phi * x[k - 1] + rng.normal(size=C)
    return (x - 3.0).reshape(-1)          # sample k of chain c at row k * C + c


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.8])
def test_ess_matches_numpy_and_ar1(nqs, phi):
    rng = np.random.default_rng(7)
    K, C = 256, 64
    E = ar1(rng, K, C, phi)
    tau, n = nqs.ess(E, C)
    ref = tau_numpy(E, C)
    assert tau == pytest.approx(ref, rel=1e-10)
    assert n == pytest.approx(K * C / ref, rel=1e-10)
    exact = (1 + phi) / (1 - phi)
    assert tau == pytest.approx(exact, rel=0.15)


def test_ess_short_chains(nqs):
    E = np.arange(100, dtype=np.float64)
    assert nqs.ess(E, 100) == (1.0, 100.0)      # one sample per chain: no lag available
