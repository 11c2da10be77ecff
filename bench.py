#!/usr/bin/env python
"""MMH reconstruction benchmark on GB300: prints ONE JSON line.

Workload (the headline configuration): a 512^3 periodic lognormal density
(sigma_lnrho = 0.5, P(k) ~ k^-1.5, Gaussian-smoothed at 2 cells, seeded;
larger sigma makes the reference algorithm itself unstable at this size),
20 mesh-deformation iterations (calcdefp, def += defp, relaxing), every
multigrid solve run to ||r||_inf / ||rhs||_inf <= 1e-8 (the outer residual in
float-float, about 48 significant bits), followed by the spectral
displacement and density outputs.  One "step"
is one such reconstruction; the metric is seconds per reconstruction.

  value   : mixed form (FP32 V-cycles in a float-float defect-correction loop), input
            density resident in HBM, CUDA events on the library's stream,
            kernel timing hooks off (the production configuration).
  e2e     : the same through the C ABI with host buffers: H2D of the density
            from pinned memory, D2H of def, the displacement and the density
            outputs, all inside the timed region.
  fp64    : the plain FP64 GPU form of the same workload, for the mixed/FP64
            ratio the metric asks for; `errors` gives the mixed form's
            per-field difference from it.
  roofline: the dominant kernel's launches on the finest level, timed one by
            one with CUDA events in a separate reconstruction after the timed
            ones (achieved = algorithmic bytes / device time) against the
            measured HBM copy bandwidth.
  cpu_baseline: the CPU oracle (FP64, all host threads) on complete work: one
            whole deformation iteration and the outputs of a 256^3 instance,
            scaled to the reconstruction.

--batch and --adjoint print the batched-realisation line and the adjoint
line (the density gradient of a band-power loss at 256^3) instead.

Multi-GPU: independent reconstructions, one per rank (replicas; the path has
no exchange step).  --impl reference times the CPU restatement of the
reference (the Fortran reference has no compiler on this image).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = "moving-mesh-reconstruction_gb300"
for p in (ROOT, os.path.join(ROOT, PKG), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "s per 512³ reconstruction to residual 1e-8: mixed vs FP64 GPU; stencil HBM GB/s"
UNIT = "s/reconstruction"
# Algorithmic words per processed cell (the minimum one pass must move).  A
# Gauss-Seidel sweep must read phi, rhs and the 6 metric coefficients of every
# cell and write phi: 9 words per updated cell.  The residual reads phi, rhs
# and the 6 coefficients and writes r: 9 words per cell.
ALG_WORDS = {"gs": 9, "residual": 9}
# Words per updated cell the current kernel itself moves: one launch of the
# fused plane kernel (or of the strips marching in y) updates the planes of
# one parity and also reads phi and coefficients 3, 5, 6 of the other
# parity's planes (4 more words per updated cell).
KERNEL_WORDS = {"gs": 13, "residual": 9}
# (TX, TY) of the FP32 Gauss-Seidel shapes: 0-3 tiles, 4-5 strips marching in y
GS_SHAPES = [(32, 16), (64, 8), (16, 32), (32, 8), (64, 128), (64, 256)]
KERNEL_NAME = {"gs32": "k_gs_plane<float,32,16>", "gs64": "k_gs_plane<double,32,8>",
               "res64": "k_residual<double>", "res32": "k_residual<float>"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--niter", type=int, default=20)
    ap.add_argument("--sigma", type=float, default=0.5)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--max-cycles", type=int, default=200)
    ap.add_argument("--nu1", type=int, default=1, help="pre-smoothing sweeps of the preconditioner's V-cycle")
    ap.add_argument("--nu2", type=int, default=1, help="post-smoothing sweeps")
    ap.add_argument("--fp64-steps", type=int, default=1, help="timed FP64 reconstructions (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-sample", default="auto", choices=["auto", "none"])
    ap.add_argument("--cpu-n", type=int, default=256, help="grid of the CPU sample's complete iteration")
    ap.add_argument("--profile", default="gs32", choices=["gs32", "gs64", "res64", "res32", "none"])
    ap.add_argument("--roofline-steps", type=int, default=1,
                    help="reconstructions run after the timed ones with the profiled kernel's launches timed")
    ap.add_argument("--errors", type=int, default=1, help="report the mixed form's per-field error vs the FP64 form")
    ap.add_argument("--batch", action="store_true",
                    help="batched-realisations workload (mmh_batch_run) instead of the headline reconstruction")
    ap.add_argument("--adjoint", action="store_true",
                    help="print the C5 adjoint line instead (256^3 density gradient of a band-power loss)")
    ap.add_argument("--adj-n", type=int, default=256)
    ap.add_argument("--adj-tol", type=float, default=1e-10)
    ap.add_argument("--batch-workers", type=int, default=8)
    ap.add_argument("--batch-niter", type=int, default=4)
    ap.add_argument("--relax-case", type=int, default=0,
                    help="instead of the benchmark: two FP32 Gauss-Seidel sweeps (mmh_relax_f64 on a mixed "
                         "context) on an N^3 grid, the small case of the committed ncu captures of the sweep kernel")
    ap.add_argument("--gs-shape", type=int, default=-1,
                    help="pin the FP32 Gauss-Seidel shape (0-3 tiles, 4-5 strips); -1: the library times them")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = list(self.rows)

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        smax = [num(r[1]) for r in rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[4 + q].lower() == "active"})
        pw = [num(r[2]) for r in rows if num(r[2]) is not None]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows), "power_w": statistics.median(pw) if pw else None}


# ---------------------------------------------------------------------------
# CPU oracle sample (test infrastructure timed as the baseline)
# ---------------------------------------------------------------------------
def _oracle_outputs_seconds(oracle, d):
    t = time.perf_counter()
    oracle.gradient(d)
    oracle.delta(d)
    return time.perf_counter() - t


def cpu_sample(n_full, niter, sigma, seed, tol, n_sample=256, nu=(1, 1)):
    """Time the oracle (FP64, tolerance schedule as the GPU runs it, 8-colour
    order, all host threads) on complete work: one whole deformation
    iteration (calcdefp with its solve run to tol, def += defp, relaxing) of
    an n_sample^3 instance of the workload (same recipe, sigma and seed), and
    the spectral outputs of its def.  Nothing is modelled inside the sample:
    it is the path's full work for one iteration.  It is scaled to one
    n_full^3 reconstruction by the cell count (n_full/n_sample)^3 and by the
    niter iterations; the solves' iteration counts at n_full are within a few
    of n_sample's."""
    import oracle
    import fields
    threads = oracle.threads(0)
    defpot, u = fields.initial_state(n_sample, sigma=sigma, seed=seed)
    kw = dict(sched=oracle.SCHED_TOL, tol=tol, maxcyc=500, colour8=True, nu1=nu[0], nu2=nu[1])
    t = time.perf_counter()
    d, _, _, _, diag = oracle.iteration(defpot, u, **kw)
    t_it = time.perf_counter() - t
    t_out = _oracle_outputs_seconds(oracle, d)
    scale = (n_full / n_sample) ** 3
    value = scale * (niter * t_it + t_out)
    return {
        "value": value, "unit": UNIT, "cores": threads, "kind": "port",
        "sample": (f"oracle FP64 (tolerance schedule to {tol:g}, {threads} threads): one complete deformation "
                   f"iteration of the {n_sample}^3 instance ({t_it:.2f} s, {diag['vcycles']} PCG iterations) and its "
                   f"spectral outputs ({t_out:.2f} s), scaled by {niter} iterations and by the cell count "
                   f"({n_full}/{n_sample})^3 = {scale:g}"),
        "sample_seconds": t_it + t_out,
        "reference_schedule_fp32": reference_schedule_sample(n_full, niter, sigma, seed, n_sample),
    }


def reference_schedule_sample(n_full, niter, sigma, seed, n_sample=256):
    """The reference's own algorithm in its own precision, for context: the
    oracle in FP32 with the reference schedule (one V-cycle per iteration,
    4*NG/n sweeps per level, NG the sample's grid), one complete deformation
    iteration and the outputs of the n_sample^3 instance, scaled like the
    main sample.  Its solves are not run to the tolerance: this is what the
    Fortran (FP32 default reals, mmh/Makefile:9) computes per iteration, not
    the same work as the timed reconstruction."""
    import oracle
    import fields
    defpot, u = fields.initial_state(n_sample, sigma=sigma, seed=seed, dtype=np.float32)
    t = time.perf_counter()
    d, _, _, _, diag = oracle.iteration(defpot, u, sched=oracle.SCHED_REF)
    t_it = time.perf_counter() - t
    t_out = _oracle_outputs_seconds(oracle, d)
    scale = (n_full / n_sample) ** 3
    return {"value": scale * (niter * t_it + t_out), "unit": UNIT,
            "sample": (f"oracle FP32, reference schedule (one V-cycle of 4*NG/n sweeps per level, NG = {n_sample}): one "
                       f"iteration of the {n_sample}^3 instance ({t_it:.2f} s, relative residual after it "
                       f"{diag['resid_rel']:.2g}) and its outputs ({t_out:.2f} s), scaled as above")}


def reference_arm(args):
    """--impl reference: the CPU restatement of the reference path on all the
    host cores (rank 0 only; the Fortran reference has no compiler here).
    Each step is one complete deformation iteration (calcdefp with its solve
    run to tol, def += defp, relaxing) of a cpu_n^3 instance of the workload,
    each step continuing the previous one's state; the warm-up steps are the
    first iterations.  The spectral outputs of the final def are timed once.
    value = (niter * median step + outputs) * (n / cpu_n)^3 seconds per n^3
    reconstruction."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    import fields
    threads = oracle.threads(0)
    m = args.cpu_n or 256
    defpot, u = fields.initial_state(m, sigma=args.sigma, seed=args.seed)
    kw = dict(sched=oracle.SCHED_TOL, tol=args.tol, maxcyc=500, colour8=True, nu1=args.nu1, nu2=args.nu2)
    for _ in range(args.warmup):
        defpot, u, _, _, _ = oracle.iteration(defpot, u, **kw)
    times = []
    t0 = time.perf_counter()
    for _ in range(max(args.steps, 1)):
        t = time.perf_counter()
        defpot, u, _, _, diag = oracle.iteration(defpot, u, **kw)
        times.append(time.perf_counter() - t)
    t_out = _oracle_outputs_seconds(oracle, defpot)
    wall = time.perf_counter() - t0
    scale = (args.n / m) ** 3
    v = scale * (args.niter * statistics.median(times) + t_out)
    sample = (f"oracle FP64 (tolerance schedule to {args.tol:g}, {threads} threads): complete deformation "
              f"iterations of the {m}^3 instance, one per step (median {statistics.median(times):.2f} s, last solve "
              f"{diag['vcycles']} PCG iterations), spectral outputs {t_out:.2f} s; scaled by {args.niter} iterations "
              f"and by the cell count ({args.n}/{m})^3 = {scale:g}")
    ref32 = reference_schedule_sample(args.n, args.niter, args.sigma, args.seed, m)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * wall / max(args.steps, 1), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "reference_schedule_fp32": ref32},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the Fortran reference cannot be compiled here (no Fortran compiler); the CPU restatement "
                "in oracle/ stands in for it",
    }
    print(json.dumps(line))
    return 0


def replica_seed(base, rank):
    """Each rank reconstructs its own realisation (replicas; no data exchange)."""
    return base + rank


def max_over_ranks(value, device=None):
    """Max of a per-rank number over all ranks (the job's time is the slowest rank's)."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def workload_config(args):
    return {
        "workload": f"{args.n}^3 lognormal density, sigma_lnrho={args.sigma}, P(k)~k^-1.5, smoothed at 2 cells, "
                    f"seed {args.seed}; {args.niter} deformation iterations; each multigrid solve by flexible CG "
                    f"preconditioned with one V({args.nu1},{args.nu2}) cycle to ||r||inf/||rhs||inf<={args.tol:g} (outer residual in "
                    f"float-float, about 48 bits); "
                    f"spectral displacement and density outputs",
        "n": args.n, "iterations": args.niter, "tol": args.tol, "sigma_lnrho": args.sigma,
        "sigma_note": "sigma_lnrho=1.5 (and >=0.75) makes the reference algorithm itself unstable at 512^3 "
                      "(mesh increments of several cells per step in deep voids violate relaxing's CFL limit; "
                      "CPU restatement and GPU agree); 0.5 is the largest value stable for 20 iterations",
        "precision": "mixed (FP32 V-cycles and relaxing fluxes; float-float outer residual and finest metric; FP64 "
                     "limiter decisions, relaxing update, exact 4^3 coarsest solve and FFTs)",
        "l2": "inputs larger than L2 (one 512^3 FP64 field is 1 GiB vs 129 MB L2)",
        "parallelism": f"replicas x{args.gpus}",
    }


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_from_profiles(kernel):
    """Per-cell DRAM traffic of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic_per_cell.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel:
                return float(parts[1])
    except OSError:
        pass
    return None


def batch_arm(args):
    """Batched realisations: 96 independent reconstructions, 32 each of 64^3,
    128^3 and 256^3, sigma_lnrho ~ U[0.4, 0.7] (stronger fields make the
    reference algorithm itself unstable at 256^3), spectral index ~ U[-2, -1]
    (seeded), batch_niter deformation iterations each with every solve to
    tol, outputs to host memory.  Aggregate cells/s (sum n^3 * iterations over
    the wall time) of mmh_batch_run with batch_workers workers against the
    same problems run one after another (one worker, contexts reused)."""
    __import__("importlib").import_module(PKG)
    import mmh
    import fields
    rng = np.random.default_rng(args.seed)
    sizes = [64] * 32 + [128] * 32 + [256] * 32
    rhos = [fields.lognormal_density(n, sigma=float(rng.uniform(0.4, 0.7)), ns=float(rng.uniform(-2.0, -1.0)),
                                     seed=args.seed + i) for i, n in enumerate(sizes)]
    cells = sum(n ** 3 for n in sizes) * args.batch_niter
    kw = dict(precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL, tol=args.tol, max_cycles=args.max_cycles,
              nu1=args.nu1, nu2=args.nu2)
    mmh.batch_run(rhos[:3] + rhos[32:35] + rhos[64:67], 1, workers=args.batch_workers, **kw)  # warm-up
    res = {}
    for label, w in (("batch", args.batch_workers), ("loop", 1)):
        t = time.perf_counter()
        out = mmh.batch_run(rhos, args.batch_niter, workers=w, **kw)
        res[label] = time.perf_counter() - t
        bad = [o["status"] for o in out if o["status"] not in (0, mmh.MMH_ERR_DIVERGED)]
        assert not bad, bad
    line = {
        "metric": "aggregate cells/s, 96 batched reconstructions (32 each of 64^3, 128^3, 256^3)",
        "value": cells / res["batch"], "unit": "cells/s", "higher_is_better": True, "n_gpus": 1,
        "loop_value": cells / res["loop"], "speedup_vs_loop": res["loop"] / res["batch"],
        "seconds": res, "workers": args.batch_workers, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"96 lognormal fields, sigma_lnrho~U[0.4,0.7], n_s~U[-2,-1], seeds {args.seed}+i; "
                               f"{args.batch_niter} deformation iterations each, solves to {args.tol:g}; outputs to "
                               f"host", "note": "C4's sigma up to 2.0 makes the reference algorithm itself unstable (at "
                                           "256^3 sigma_lnrho 0.96 already gives negative densities after one iteration)"},
    }
    print(json.dumps(line))
    return 0


def adjoint_arm(args):
    """C5: the gradient of a band-power loss of the reconstructed density with
    respect to the input density.  adj_n^3 lognormal field (sigma_lnrho), 20
    deformation iterations (niter) with the forward states kept every 4, loss
    sum_b w_b P_b over 16 log-spaced |k| bands with seeded weights; its seed
    d loss / d delta is formed on the host from one forward run before the
    timed region.  One step = one mmh_iterate_adjoint_f64 call (checkpointed
    forward pass + reverse sweep), wall clock around the synchronous call;
    the forward reconstruction alone is timed the same way for the ratio.
    Mixed form, and the FP64 form with the gradients' difference."""
    __import__("importlib").import_module(PKG)
    import mmh
    import fields
    n, niter, every = args.adj_n, args.niter, 4
    rho = fields.lognormal_density(n, sigma=args.sigma, seed=args.seed)
    u = np.zeros((5, n, n, n), order="F")
    u[0] = rho
    z = np.zeros((n, n, n), order="F")
    k = np.fft.fftfreq(n, d=1.0 / n)
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    band = np.searchsorted(np.logspace(0.0, np.log10(np.sqrt(3.0) * n / 2 + 1e-9), 17), kk, side="right") - 1
    wb = np.random.default_rng(args.seed + 1).uniform(0.5, 1.5, 16)
    W = np.where((band >= 0) & (band < 16), wb[np.clip(band, 0, 15)], 0.0)
    out, grads = {}, {}
    for name, prec in (("mixed", mmh.MMH_MIXED), ("fp64", mmh.MMH_FP64)):
        if name == "fp64" and args.fp64_steps <= 0:
            continue
        with mmh.Context(n, precision=prec, schedule=mmh.MMH_SCHED_TOL, tol=args.adj_tol,
                         max_cycles=args.max_cycles, nu1=args.nu1, nu2=args.nu2) as ctx:
            def forward():
                ctx.load(z, u)
                ctx.iterate(niter)
                delta = np.zeros((n, n, n), order="F")
                ctx.outputs(None, delta)
                return delta
            forward()  # warm-up
            t = time.perf_counter()
            delta = forward()
            t_fwd = time.perf_counter() - t
            F = np.fft.fftn(delta)
            seed = np.asfortranarray(2.0 * np.real(np.fft.ifftn(W * F)))
            loss = float(np.sum(W * np.abs(F) ** 2)) / n ** 3
            times = []
            for _ in range(max(1, args.steps)):
                ctx.load(z, u)
                t = time.perf_counter()
                g, _, d = ctx.iterate_adjoint(niter, wdelta=seed, checkpoint_every=every)
                times.append(time.perf_counter() - t)
            grads[name] = g
            out[name] = {"gradient_s": statistics.median(times), "forward_s": t_fwd,
                         "ratio": statistics.median(times) / t_fwd, "loss": loss}
    line = {
        "metric": f"s per {n}^3 density gradient of a 16-band power loss (20 iterations, checkpoints every 4)",
        "value": out["mixed"]["gradient_s"], "unit": "s/gradient", "higher_is_better": False, "n_gpus": 1,
        "steps": max(1, args.steps), "warmup": 1, "mixed": out["mixed"], "fp64": out.get("fp64"),
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"{n}^3 lognormal density, sigma_lnrho {args.sigma}, seed {args.seed}; {niter} "
                               f"deformation iterations, solves to {args.adj_tol:g}; loss over 16 log-spaced |k| "
                               f"bands of the reconstructed density", "timing": "wall clock around the host call"},
    }
    if "fp64" in grads:
        line["mixed_vs_fp64_gradient"] = float(np.abs(grads["mixed"] - grads["fp64"]).max()
                                               / np.abs(grads["fp64"]).max())
    print(json.dumps(line))
    return 0


def relax_case(n, mmh, fields):
    """Two FP32 sweeps and the residual norm on an n^3 grid (a smooth deformation
    potential of amplitude 0.05, a lognormal density with sigma 0.5, random phi
    and rhs): one small, quick launch sequence of the sweep kernel to profile."""
    g = np.log(fields.lognormal_density(n, sigma=1.0, ns=-2.0, seed=7))
    defpot = np.asfortranarray((g - g.mean()) * 0.05)
    rho = fields.lognormal_density(n, sigma=0.5, seed=8)
    rng = np.random.default_rng(9)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi = np.asfortranarray(rng.standard_normal((n, n, n)))
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        _, rinf = ctx.relax(phi, rhs, defpot, rho, 1.0, 2, 18)
    print(json.dumps({"case": "relax", "n": n, "sweeps": 2, "rinf": rinf}))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.batch:
        return batch_arm(args)
    if args.adjoint:
        return adjoint_arm(args)

    import torch
    __import__("importlib").import_module(PKG)
    import mmh
    import fields

    mmh.gs_tile_pin(args.gs_shape)
    if args.relax_case > 0:
        return relax_case(args.relax_case, mmh, fields)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n
    n3 = n ** 3
    seed = replica_seed(args.seed, rank)

    rho_np = fields.lognormal_density(n, sigma=args.sigma, seed=seed)
    rho_dev = torch.from_numpy(rho_np.ravel(order="F")).to(dev)
    grad_dev = torch.empty(3 * n3, dtype=torch.float64, device=dev)
    delta_dev = torch.empty(n3, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def barrier():
        if dist:
            tdist.barrier()
        torch.cuda.synchronize()

    def make_ctx(precision):
        return mmh.Context(n, precision=precision, schedule=mmh.MMH_SCHED_TOL, tol=args.tol,
                           max_cycles=args.max_cycles, nu1=args.nu1, nu2=args.nu2, device=local,
                           stream=stream.cuda_stream)

    def recon(ctx):
        ctx.load_dev(None, rho_dev.data_ptr())
        d = ctx.iterate(args.niter)
        ctx.outputs_dev(grad_dev.data_ptr(), delta_dev.data_ptr())
        return d

    def timed(ctx, steps, profile_kind=None):
        barrier()
        launches0 = mmh.launch_count()
        if profile_kind:
            mmh.profile_start(profile_kind)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        diags = []
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                diags.append(recon(ctx))
            e1.record(stream)
        e1.synchronize()
        prof = mmh.profile_stop() if profile_kind else None
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1) / steps, dev)
        return ms, diags, mmh.launch_count() - launches0, prof

    # ---- mixed (headline value): timing hooks off, graph replay on ----
    ctx = make_ctx(mmh.MMH_MIXED)
    for _ in range(args.warmup):
        recon(ctx)
        ctx.sync()
    clocks = ClockSampler(local)
    clocks.start()
    ms_mixed, diags, launches, _ = timed(ctx, args.steps)
    clk = clocks.stop()

    # ---- roofline pass: one more reconstruction with the dominant kernel's
    # launches on the finest level timed one by one (hooks armed: the
    # preconditioner then runs launch by launch, not from its graph) ----
    kinds = {"gs32": mmh.K_GS | mmh.K_F32, "gs64": mmh.K_GS, "res64": mmh.K_RESIDUAL,
             "res32": mmh.K_RESIDUAL | mmh.K_F32, "none": None}
    pk = kinds[args.profile]
    prof = None
    if pk is not None and args.roofline_steps > 0:
        pk |= mmh.K_AT(n)  # the finest grid level only: the launches that dominate the step
        ms_prof, _, _, prof = timed(ctx, args.roofline_steps, pk)

    # mixed results kept for the error against the FP64 form
    keep = {}
    if args.fp64_steps > 0 and args.errors:
        keep["grad"] = grad_dev.clone()
        keep["delta"] = delta_dev.clone()
        keep["def"] = np.zeros((n, n, n), order="F")
        keep["rho"] = np.zeros((1, n, n, n), order="F")
        ctx.store(keep["def"], keep["rho"])

    # ---- e2e through the C ABI with host buffers ----
    rho_host = torch.from_numpy(rho_np.ravel(order="F").copy()).pin_memory()
    def_host = torch.empty(n3, dtype=torch.float64).pin_memory()
    grad_host = torch.empty(3 * n3, dtype=torch.float64).pin_memory()
    delta_host = torch.empty(n3, dtype=torch.float64).pin_memory()

    def as_np(t, shape):  # Fortran-ordered numpy view of pinned host memory
        return t.numpy().reshape(shape, order="F")

    u1 = as_np(rho_host, (1, n, n, n))
    defh = as_np(def_host, (n, n, n))
    gradh = as_np(grad_host, (n, n, n, 3))
    deltah = as_np(delta_host, (n, n, n))
    e2e_ms = None
    e2e_clk = None
    if args.e2e_steps > 0:
        e2e_clocks = ClockSampler(local)
        e2e_clocks.start()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(args.e2e_steps):
                ctx.load(None, u1)
                ctx.iterate(args.niter)
                ctx.outputs(gradh, deltah)
                ctx.store(defh, None)
            e1.record(stream)
        e1.synchronize()
        barrier()
        e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.e2e_steps, dev)
        e2e_clk = e2e_clocks.stop()
    ctx.close()

    # ---- FP64 form ----
    fp64 = None
    errors = None
    if args.fp64_steps > 0:
        c64 = make_ctx(mmh.MMH_FP64)
        recon(c64)
        c64.sync()
        ms64, d64, _, _ = timed(c64, args.fp64_steps)
        fp64 = {"value": ms64 / 1000.0, "unit": UNIT, "vcycles_last_solve": d64[-1]["vcycles"],
                "resid_rel_last_solve": d64[-1]["resid_rel"], "steps": args.fp64_steps, "warmup": 1}
        if keep:
            # the mixed form's fields against the FP64 form's, both solved to
            # tol: max |mixed - FP64| / max |FP64| per field
            f_def = np.zeros((n, n, n), order="F")
            f_rho = np.zeros((1, n, n, n), order="F")
            c64.store(f_def, f_rho)

            def rel_dev(a, b):
                return float((a - b).abs().max() / b.abs().max())

            errors = {"vs": f"FP64 GPU form of the same workload (solves to {args.tol:g})",
                      "def": float(np.abs(keep["def"] - f_def).max() / np.abs(f_def).max()),
                      "rho": float(np.abs(keep["rho"] - f_rho).max() / np.abs(f_rho).max()),
                      "displacement": rel_dev(keep["grad"], grad_dev),
                      "delta": rel_dev(keep["delta"], delta_dev)}
        c64.close()

    if rank != 0:
        if dist:
            tdist.destroy_process_group()
        return 0

    # roofline of the profiled kernel
    hbm, peak_src = peaks()
    roofline = None
    if prof and prof[0] > 0:
        nl, pms, cells = prof
        word = 4 if args.profile.endswith("32") else 8
        kname = args.profile
        unit = "gs" if kname.startswith("gs") else "residual"
        alg_bytes = cells * ALG_WORDS[unit] * word
        achieved = alg_bytes / (pms / 1000.0) / 1e9
        kern_bytes = cells * KERNEL_WORDS[unit] * word
        kernel = KERNEL_NAME[kname]
        if kname == "gs32":
            # the pinned shape, or the one the library kept for this grid
            tile = GS_SHAPES[args.gs_shape] if args.gs_shape >= 0 else mmh.gs_tile(n)
            if tile:
                kernel = (f"k_gs_strip<{tile[1] // 2}>" if tile[0] == 64 and tile[1] >= 32
                          else f"k_gs_plane<float,{tile[0]},{tile[1]}>")
        tr = traffic_from_profiles(kernel)
        roofline = {"kernel": f"{kernel} on the {n}^3 level",
                    "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                    "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else peak_src,
                    "alg_words_per_cell": ALG_WORDS[unit],
                    "traffic": (tr * cells / nl) if tr else None,
                    "alg_bytes_per_launch": alg_bytes / nl, "launches": nl,
                    "avg_launch_ms": pms / nl, "share_of_step": (pms / args.roofline_steps) / ms_prof,
                    "kernel_words_per_cell": KERNEL_WORDS[unit],
                    "frac_kernel_words": kern_bytes / (pms / 1000.0) / 1e9 / hbm,
                    "pass": f"{args.roofline_steps} reconstruction(s) after the timed ones, every launch of the "
                            f"kernel on the {n}^3 level timed with CUDA events on its stream"}

    cpu = None
    if args.cpu_sample != "none" and not dist:
        cpu = cpu_sample(n, args.niter, args.sigma, args.seed, args.tol, n_sample=args.cpu_n, nu=(args.nu1, args.nu2))
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "reference_schedule_fp32")}

    value = ms_mixed / 1000.0 / world  # whole-job seconds per reconstruction (replicas)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "config": workload_config(args),
        "e2e": {"value": (e2e_ms / 1000.0 / world) if e2e_ms else None, "unit": UNIT,
                "h2d_bytes_per_step": 8 * n3, "d2h_bytes_per_step": 8 * 5 * n3, "clocks": e2e_clk},
        "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
        "fp64": fp64, "mixed_vs_fp64_speedup": (fp64["value"] / (ms_mixed / 1000.0)) if fp64 else None,
        "errors": errors,
        "solve": {"vcycles_last": diags[-1]["vcycles"], "resid_rel_last": diags[-1]["resid_rel"],
                  "ncompress_last": diags[-1]["ncompress"], "guards_last": diags[-1]["guards"]},
        "cells_per_s": n3 * args.niter * world / (ms_mixed / 1000.0),
        "gs_tiles": {str(m): mmh.gs_tile(m) for m in (512, 256, 128, 64) if m <= n},
    }
    print(json.dumps(line))
    if dist:
        tdist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
