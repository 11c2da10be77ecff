"""Golden vectors (tests/golden/mmh_golden.npz, made by tests/golden/make_golden.py
with the CPU oracle): the oracle must keep reproducing them bit for bit, and
the GPU library must reproduce them through its C ABI -- bit for bit where no
FFT is involved, within 1e-10 relative for the spectral outputs."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mmh_golden.npz")
TOL_SPECTRAL = 1e-10


@pytest.fixture(scope="module")
def g():
    with np.load(GOLDEN) as z:
        return {k: (np.asfortranarray(z[k]) if z[k].ndim else z[k][()]) for k in z.files}


def _u(rho):
    n = rho.shape[0]
    u = np.zeros((5, n, n, n), order="F")
    u[0] = rho
    return u


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_oracle_reproduces_golden(oracle, g):
    assert np.array_equal(oracle.metric(g["metric_def"], g["metric_rho"], 1.0), g["metric_coef"])
    coef = oracle.metric(g["relax_def"], g["relax_rho"], 1.0)
    phi = g["relax_phi0"].copy(order="F")
    resid, rinf = oracle.relax(phi, g["relax_rhs"], coef, 1.0, 4, 19)
    assert np.array_equal(phi, g["relax_phi"]) and np.array_equal(resid, g["relax_resid"])
    assert rinf == g["relax_rinf"]
    d1, u1, defp, _, _ = oracle.iteration(g["iter_def0"], _u(g["iter_rho0"]))
    assert np.array_equal(defp, g["iter_defp"]) and np.array_equal(d1, g["iter_def1"])
    assert np.array_equal(u1[0], g["iter_rho1"])
    assert np.array_equal(oracle.gradient(g["spec_def"]), g["spec_grad"])
    assert np.array_equal(oracle.delta(g["spec_def"]), g["spec_delta"])


@pytest.mark.gpu
def test_gpu_reproduces_golden(mmh, g):
    with mmh.Context(8) as ctx:
        assert np.array_equal(ctx.metric(g["metric_def"], g["metric_rho"], 1.0), g["metric_coef"])
        phi = g["relax_phi0"].copy(order="F")
        resid, rinf = ctx.relax(phi, g["relax_rhs"], g["relax_def"], g["relax_rho"], 1.0, 4, 19)
        assert np.array_equal(phi, g["relax_phi"]) and np.array_equal(resid, g["relax_resid"])
        assert rinf == g["relax_rinf"]
        n = 8
        grad = np.zeros((n, n, n, 3), order="F")
        delta = np.zeros((n, n, n), order="F")
        ctx.scalar2gradient(g["spec_def"], grad, (n, n, n))
        ctx.defp2delta(g["spec_def"], delta, (n, n, n))
        assert _rel(grad, g["spec_grad"]) <= TOL_SPECTRAL
        assert _rel(delta, g["spec_delta"]) <= TOL_SPECTRAL
    n = 16
    u = _u(g["iter_rho0"])
    defpot = g["iter_def0"].copy(order="F")
    defp = np.zeros((n, n, n), order="F")
    with mmh.Context(n) as ctx:
        ctx.calcdefp(defp, None, None, defpot, u)
        defpot = np.asfortranarray(defpot + defp)
        ctx.relaxing(u, defpot, defp)
    assert np.array_equal(defp, g["iter_defp"])
    assert np.array_equal(defpot, g["iter_def1"])
    assert np.array_equal(u[0], g["iter_rho1"])
