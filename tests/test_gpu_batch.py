"""Batched independent reconstructions (mmh_batch_run) through the C ABI.

Every problem of a batch must give exactly the results of the same problem
run alone in a fresh context, whatever the mix of sizes and the number of
concurrent workers; a failing problem reports its own status without
stopping the others.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(fields, sizes, seed0):
    rng = np.random.default_rng(seed0)
    return [fields.lognormal_density(n, sigma=float(rng.uniform(0.5, 1.0)), ns=float(rng.uniform(-2.0, -1.0)),
                                     seed=seed0 + i) for i, n in enumerate(sizes)]


@pytest.mark.parametrize("workers", [1, 3])
def test_batch_matches_single_runs(mmh, fields, workers):
    sizes = [16, 32, 64, 32, 16, 64]
    rhos = _fields(fields, sizes, 500)
    niter = 2
    got = mmh.batch_run(rhos, niter, workers=workers, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL, tol=1e-8)
    for rho, g in zip(rhos, got):
        assert g["status"] == 0
        ref = mmh.reconstruct(rho, niter, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL, tol=1e-8)
        assert np.array_equal(g["def"], ref["def"])
        assert np.array_equal(g["grad"], ref["grad"])
        assert np.array_equal(g["delta"], ref["delta"])
        assert g["vcycles"] == ref["diag"]["vcycles"]


def test_batch_fp64_matches_single_runs(mmh, fields):
    rhos = _fields(fields, [32, 16], 700)
    got = mmh.batch_run(rhos, 1, workers=2, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-10)
    for rho, g in zip(rhos, got):
        ref = mmh.reconstruct(rho, 1, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-10)
        assert np.array_equal(g["def"], ref["def"])


def test_batch_reports_a_bad_problem_and_runs_the_rest(mmh, fields):
    good = fields.lognormal_density(16, sigma=0.5, seed=5)
    bad = np.asfortranarray(np.ones((12, 12, 12)))  # not a power of two
    with pytest.raises(mmh.MMHError):
        mmh.batch_run([good, bad, good], 1, workers=2)
    out = mmh.batch_run([good, bad, good], 1, workers=2, check=False)
    assert [o["status"] for o in out] == [0, -3, 0]  # MMH_ERR_NOTPOW2 for the 12^3 grid
    assert np.array_equal(out[0]["def"], out[2]["def"])
