"""Whole deformation iterations (mmh/main.f90:90-110) and the spectral outputs
(mmh/main.f90:131-179) on the GPU against the CPU oracle, field by field.

* FP64 form: the limiter's trigger masks (limiter.f90:335-370, 523-529) are
  bit-identical in every iteration; def and the density are bit-identical
  until the final compression test first limits a cell, and within 1e-10
  relative after that (its FFT Poisson correction is cuFFT against the
  oracle's own FFT); the spectral outputs are within 1e-10.
  - C1 as configured: 64^3, sigma_lnrho 1.0, V(2,2) cycles to 1e-10,
    10 iterations, limiter on.
  - The reference's own schedule (one V-cycle of 4*NG/n sweeps per level per
    iteration, mgtemplate.f90): C2 at 256^3 over 20 iterations at the largest
    stable field strength (sigma 0.5), 128^3 over 20 iterations (sigma 0.75),
    and runs where the compression limiter fires in the last iterations
    (128^3 sigma 1.0, 256^3 sigma 0.75; the field is then going unstable, as
    the reference's own algorithm does on it).
* Mixed form (the benchmark's): FP32 V-cycles inside the float-float outer
  loop, solves to 1e-8, relaxing with FP32 fluxes, against the FP64 oracle
  solved to 1e-11 after 10 iterations; the bound on each field is stated
  below and the measured errors are printed.
"""
import numpy as np
import pytest

from recon_parity import any_fft_correction, field_errors, rel, run_side_by_side

pytestmark = pytest.mark.gpu

TOL_SPECTRAL = 1e-10

# Mixed form (solves to 1e-8, FP32 V-cycles, float-float outer residual,
# relaxing with FP32 fluxes and an FP64 update) against the FP64 oracle
# converged to 1e-11, after 10 iterations: max |difference| / max |oracle|
# per field.  Measured on one GB300 (64^3 and 128^3, sigma 0.5 and 1.0): def
# 9.2e-10, density 5.0e-8, displacement 3.1e-9, reconstructed density 8.5e-9.
# The density carries the FP32 rounding of relaxing's fluxes (about 6e-9 of
# it per step); def, which integrates the solves, stays near the tolerance.
# The FP64 GPU form solved to the same 1e-8 differs from the oracle by up to
# 2.4e-10.
MIXED_BOUND = {"def": 5e-9, "rho": 2e-7, "grad": 2e-8, "delta": 5e-8}


def _check_fp64(res):
    for r in res["records"]:
        assert r["mask_mismatch"] == {"expand": 0, "compress1": 0, "compress2": 0}, r
        assert r["nexpand"][0] == r["nexpand"][1] and r["ncompress"][0] == r["ncompress"][1], r
    err = field_errors(res)
    # Once an unstable run's density has blown up (|rho| ~ 1e17 in the 256^3,
    # sigma 0.75 run's last iteration), relaxing's minmod branches turn the
    # spectral correction's 1e-16 differences in defp into visible density
    # differences; def, the masks and the outputs still agree.
    physical = np.abs(res["rho"][0]).max() < 1e3
    if any_fft_correction(res):
        assert err["def"] <= TOL_SPECTRAL, err
        assert err["rho"] <= TOL_SPECTRAL or not physical, err
    else:
        assert err["def"] == 0.0 and err["rho"] == 0.0, err
    assert err["grad"] <= TOL_SPECTRAL and err["delta"] <= TOL_SPECTRAL, err
    return err


def test_c1_vcycle_schedule_64cube(mmh, oracle, fields):
    """C1: 64^3, sigma_lnrho 1.0, FP64, V(2,2) cycles to relative residual
    1e-10, 10 deformation iterations, limiter on."""
    n, niter = 64, 10
    defpot, u = fields.initial_state(n, sigma=1.0, seed=1000)
    res = run_side_by_side(
        mmh, oracle, defpot, u, niter,
        gpu_kw=dict(precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_VCYCLE, nu1=2, nu2=2, tol=1e-10, max_cycles=200),
        oracle_kw=dict(sched=oracle.SCHED_VCYCLE, nu1=2, nu2=2, tol=1e-10, maxcyc=200, colour8=True))
    for r in res["records"]:
        assert r["vcycles"][0] == r["vcycles"][1], r
    err = _check_fp64(res)
    print("C1 64^3 errors", err)


@pytest.mark.parametrize("n,sigma,niter", [(128, 0.75, 20), (128, 1.0, 10), (256, 0.5, 20), (256, 0.75, 11)])
def test_reference_schedule(mmh, oracle, fields, n, sigma, niter):
    """The reference's schedule (mgN: one V-cycle, 4*NG/n sweeps per level)
    over whole iterations.  256^3 at sigma_lnrho 0.5 over 20 iterations is C2
    at the largest field strength the reference algorithm stays stable for on
    that grid (0.6 turns the density negative after 8 iterations, C2's 1.5
    after one; test_instability.py); 0.75 over 11 iterations runs into the
    compression limiter (thousands of cells in the last one) as the field
    goes unstable."""
    defpot, u = fields.initial_state(n, sigma=sigma, seed=1000)
    res = run_side_by_side(mmh, oracle, defpot, u, niter, gpu_kw=dict(precision=mmh.MMH_FP64),
                           oracle_kw=dict(sched=oracle.SCHED_REF))
    err = _check_fp64(res)
    if sigma >= 0.75 and niter < 20:
        # the compression limiter and its FFT Poisson correction took part
        assert any_fft_correction(res)
        assert sum(r["mask_count"]["compress2"] for r in res["records"]) > 0
    print(f"REF {n}^3 sigma {sigma} x{niter}: errors {err}; masks {[r['mask_count'] for r in res['records']]}; "
          f"oracle {res['t_oracle']:.1f} s, GPU {res['t_gpu']:.1f} s")


@pytest.mark.parametrize("n,sigma", [(64, 0.5), (64, 1.0), (128, 0.5)])
def test_mixed_reconstruction_vs_fp64_oracle(mmh, oracle, fields, n, sigma):
    """The timed form (MMH_MIXED + MMH_SCHED_TOL, solves to 1e-8) over 10
    iterations plus the outputs, against the FP64 oracle (tolerance schedule
    converged to 1e-11): every field within its stated bound.  The FP64 GPU
    form at the same tolerance is measured beside it (its error is that of
    the tolerance alone)."""
    niter = 10
    defpot, u = fields.initial_state(n, sigma=sigma, seed=1000)
    okw = dict(sched=oracle.SCHED_TOL, tol=1e-11, maxcyc=300, colour8=True)
    res = run_side_by_side(mmh, oracle, defpot, u, niter, masks=False,
                           gpu_kw=dict(precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL, tol=1e-8,
                                       max_cycles=200), oracle_kw=okw)
    err = field_errors(res)
    ref = {k: res[k][0] for k in ("def", "rho", "grad", "delta")}
    # FP64 GPU form at the same tolerance, against the same oracle fields
    r64 = mmh.reconstruct(u[0].copy(order="F"), niter, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-8,
                          max_cycles=200)
    err64 = {"def": rel(r64["def"], ref["def"]), "rho": rel(r64["u"][0], ref["rho"]),
             "grad": rel(r64["grad"], ref["grad"]), "delta": rel(r64["delta"], ref["delta"])}
    print(f"mixed {n}^3 sigma {sigma}: mixed vs oracle {err}; FP64 GPU (tol 1e-8) vs oracle {err64}")
    print("limiter counts (oracle, GPU):", [(r["nexpand"], r["ncompress"]) for r in res["records"]])
    for k, b in MIXED_BOUND.items():
        assert err[k] <= b, (k, err[k], b)
