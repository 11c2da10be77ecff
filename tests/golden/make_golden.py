"""Regenerate tests/golden/mmh_golden.npz: small seeded cases of the path with
the CPU oracle's results, so later changes of the oracle or of the GPU code
are checked against fixed bits.  Inputs are stored too (the test does not
depend on numpy reproducing the field generator bit for bit on another
machine).  The reference's own Fortran cannot be compiled here, so these
vectors pin the restatement, not the reference itself.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "moving-mesh-reconstruction_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import fields  # noqa: E402
import oracle  # noqa: E402
from conftest import smooth_field  # noqa: E402


def make():
    g = {}
    # cbajraw metric, 8^3
    n = 8
    g["metric_def"] = smooth_field(n, 0.3, 101)
    g["metric_rho"] = fields.lognormal_density(n, sigma=1.0, seed=102)
    g["metric_coef"] = oracle.metric(g["metric_def"], g["metric_rho"], 1.0)
    # relax (r1lax plane schedule, two chunks of 2), 8^3, nrelax 4, iresidopt 3
    rng = np.random.default_rng(103)
    g["relax_def"] = smooth_field(n, 0.1, 104)
    g["relax_rho"] = fields.lognormal_density(n, sigma=1.0, seed=105)
    g["relax_rhs"] = np.asfortranarray(rng.standard_normal((n, n, n)))
    g["relax_phi0"] = np.asfortranarray(rng.standard_normal((n, n, n)))
    coef = oracle.metric(g["relax_def"], g["relax_rho"], 1.0)
    phi = g["relax_phi0"].copy(order="F")
    resid, rinf = oracle.relax(phi, g["relax_rhs"], coef, 1.0, 4, 19)
    g["relax_phi"], g["relax_resid"], g["relax_rinf"] = phi, resid, np.array(rinf)
    # one deformation iteration (calcdefp with the reference schedule,
    # def += defp, relaxing), 16^3; u(2:5) = 0 is not stored
    n = 16
    defpot, u = fields.initial_state(n, sigma=1.0, seed=106)
    defpot = smooth_field(n, 0.05, 107)
    g["iter_def0"], g["iter_rho0"] = defpot, np.asfortranarray(u[0])
    d1, u1, defp, masks, diag = oracle.iteration(defpot, u)
    assert diag["ncompress"] == 0  # no FFT correction: the GPU must give the same bits
    assert not u1[1:].any()
    g["iter_defp"], g["iter_def1"], g["iter_rho1"] = defp, d1, np.asfortranarray(u1[0])
    # spectral outputs of a deformation potential, 8^3
    n = 8
    g["spec_def"] = smooth_field(n, 0.2, 108)
    g["spec_grad"] = oracle.gradient(g["spec_def"])
    g["spec_delta"] = oracle.delta(g["spec_def"])
    return g


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "mmh_golden.npz"), **make())
    print("wrote", os.path.join(HERE, "mmh_golden.npz"))
