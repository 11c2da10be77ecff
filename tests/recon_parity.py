"""Whole-reconstruction parity helpers shared by the GPU tests and the C2 record
script: deformation iterations (mmh/main.f90:90-110) run side by side on the
GPU (through the C ABI) and on the CPU oracle, compared iteration by
iteration (limiter trigger masks, counts) and field by field at the end
(def, density, and the spectral displacement and density outputs of
mmh/main.f90:131-179).

The oracle is the checker here, never the thing measured.
"""
import time

import numpy as np


def rel(a, b):
    """max |a - b| / max |b| (NaN-aware: matching NaN positions count as equal)."""
    a = np.asarray(a)
    b = np.asarray(b)
    na, nb = np.isnan(a), np.isnan(b)
    if na.any() or nb.any():
        if not np.array_equal(na, nb):
            return np.inf
        a, b = a[~na], b[~nb]
        if a.size == 0:
            return 0.0
    den = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / max(den, 1e-300))


def run_side_by_side(mmh, oracle, defpot, u, niter, gpu_kw, oracle_kw, masks=True, outputs=True, log=None):
    """niter iterations from (defpot, u) on both sides.  gpu_kw: mmh.Context
    settings; oracle_kw: oracle.iteration settings (sched, tol, ...).
    Returns a dict with per-iteration records and final fields of both sides."""
    n = defpot.shape[0]
    recs = []
    d_o, u_o = defpot, u
    t_gpu = t_orc = 0.0
    with mmh.Context(n, **gpu_kw) as ctx:
        if masks:
            ctx.keep_masks(True)
        ctx.load(defpot, u)
        for it in range(niter):
            t = time.perf_counter()
            dg = ctx.iterate(1)
            mg = ctx.masks() if masks else None
            t_gpu += time.perf_counter() - t
            t = time.perf_counter()
            d_o, u_o, _, mo, do_ = oracle.iteration(d_o, u_o, **oracle_kw)
            t_orc += time.perf_counter() - t
            r = {"it": it, "nexpand": (do_["nexpand"], dg["nexpand"]), "ncompress": (do_["ncompress"], dg["ncompress"]),
                 "vcycles": (do_["vcycles"], dg["vcycles"]), "umin": float(np.nanmin(u_o[0])) if np.isfinite(u_o[0]).any() else float("nan")}
            if masks:
                r["mask_mismatch"] = {k: int(np.count_nonzero(mo[k] != mg[k])) for k in ("expand", "compress1", "compress2")}
                r["mask_count"] = {k: int(mo[k].sum()) for k in ("expand", "compress1", "compress2")}
            recs.append(r)
            if log:
                log(r)
        def_g = np.zeros((n, n, n), order="F")
        u_g = np.zeros((u.shape[0], n, n, n), order="F")
        ctx.store(def_g, u_g)
        out = {"records": recs, "def": (d_o, def_g), "rho": (u_o[0], u_g[0]), "t_gpu": t_gpu, "t_oracle": t_orc}
        if outputs:
            grad_g = np.zeros((n, n, n, 3), order="F")
            delta_g = np.zeros((n, n, n), order="F")
            ctx.outputs(grad_g, delta_g)
            out["grad"] = (oracle.gradient(d_o), grad_g)
            out["delta"] = (oracle.delta(d_o), delta_g)
    return out


def field_errors(res):
    """Max relative difference per field (GPU against oracle)."""
    return {k: rel(res[k][1], res[k][0]) for k in ("def", "rho", "grad", "delta") if k in res}


def any_fft_correction(res):
    """True once the oracle's final compression test limited a cell (the FFT
    Poisson correction then ran, and results agree within the spectral
    tolerance instead of bit for bit)."""
    return any(r["ncompress"][0] > 0 for r in res["records"])
