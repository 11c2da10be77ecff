"""Adjoint of a whole reconstruction (no counterpart in the reference):
mmh_iterate_adjoint_f64 against central finite differences of the forward
iterations (mmh/main.f90:83-179 through mmh_iterate and mmh_outputs_f64), and
the same gradient behind a torch.autograd.Function (test harness only) for a
banded power-spectrum loss of the reconstructed density.

The forward map is piecewise smooth (limiter, cflkeuler and minmod branches),
so the finite-difference steps are small (1e-7 of the direction's maximum)
and the solves tight (1e-13) to keep the differences on one smooth piece and
above the solver's noise."""
import numpy as np
import pytest

from conftest import smooth_field

N, TOL = 16, 1e-13


def _forward(ctx, rho, niter, n):
    z = np.zeros((n, n, n), order="F")
    ctx.load(z, _u(rho))
    ctx.iterate(niter)
    d = np.zeros((n, n, n), order="F")
    ctx.store(d, None)
    delta = np.zeros((n, n, n), order="F")
    ctx.outputs(None, delta)
    return d, delta


def _u(rho):
    n = rho.shape[0]
    u = np.zeros((5, n, n, n), order="F")
    u[0] = rho
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("niter,every", [(4, 2), (5, 2)])
def test_iterate_adjoint_matches_finite_differences(mmh, fields, niter, every):
    n = N
    rho = fields.lognormal_density(n, sigma=0.6, seed=61)
    rng = np.random.default_rng(62)
    wdef = np.asfortranarray(rng.standard_normal((n, n, n)))
    wdelta = np.asfortranarray(rng.standard_normal((n, n, n)))
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=TOL, max_cycles=400) as ctx:
        def_ref, _ = _forward(ctx, rho, niter, n)
        ctx.load(np.zeros((n, n, n), order="F"), _u(rho))
        grho, gdef, d = ctx.iterate_adjoint(niter, wdef=wdef, wdelta=wdelta, checkpoint_every=every)
        assert d["ncompress"] == 0
        # the state after the adjoint is the forward's final state
        after = np.zeros((n, n, n), order="F")
        ctx.store(after, None)
        assert np.array_equal(after, def_ref)

        def J(r):
            dN, delta = _forward(ctx, r, niter, n)
            return float(np.sum(wdef * dN) + np.sum(wdelta * delta))

        for q in range(2):
            v = smooth_field(n, 1.0, 70 + q)
            h = 1e-7 / np.abs(v).max()
            fd = (J(rho + h * v) - J(rho - h * v)) / (2 * h)
            ad = float(np.sum(grho * v))
            print(f"niter {niter}: fd {fd:.12e} adjoint {ad:.12e} rel {abs(fd - ad) / abs(ad):.2e}")
            assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def _band_loss(torch, delta, weights, n):
    """sum_b w_b P_b: P_b the power of delta in the b-th of 16 log-spaced |k|
    bands between 1 and sqrt(3) n / 2 (k = 0 excluded)."""
    k = torch.fft.fftfreq(n, d=1.0 / n, dtype=torch.float64)
    kk = torch.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    edges = torch.logspace(0.0, float(np.log10(np.sqrt(3.0) * n / 2 + 1e-9)), 17, dtype=torch.float64)
    band = torch.bucketize(kk, edges, right=True) - 1  # 0..15 inside, -1 for k = 0
    power = torch.abs(torch.fft.fftn(delta)) ** 2 / n ** 3
    wk = torch.where(band >= 0, weights[band.clamp(0, 15)], torch.zeros_like(kk))
    return torch.sum(wk * power)


@pytest.mark.gpu
def test_autograd_function_band_power_gradient(mmh, fields):
    torch = pytest.importorskip("torch")
    n, niter, every = N, 4, 2
    rho0 = fields.lognormal_density(n, sigma=0.6, seed=81)
    weights = torch.from_numpy(np.random.default_rng(82).uniform(0.5, 1.5, 16))

    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=TOL, max_cycles=400) as ctx:

        class Reconstruct(torch.autograd.Function):
            """delta_rec(rho_0) through the library; backward by its adjoint."""

            @staticmethod
            def forward(fc, rho):
                r = np.asfortranarray(rho.detach().numpy())
                fc.r = r
                _, delta = _forward(ctx, r, niter, n)
                return torch.from_numpy(delta)

            @staticmethod
            def backward(fc, gdelta):
                ctx.load(np.zeros((n, n, n), order="F"), _u(fc.r))
                g, _, _ = ctx.iterate_adjoint(niter, wdelta=np.asfortranarray(gdelta.numpy()), checkpoint_every=every)
                return torch.from_numpy(g)

        rho = torch.from_numpy(rho0.copy(order="F")).requires_grad_(True)
        loss = _band_loss(torch, Reconstruct.apply(rho), weights, n)
        loss.backward()
        grad = rho.grad.numpy()

        def L(r):
            _, delta = _forward(ctx, r, niter, n)
            return float(_band_loss(torch, torch.from_numpy(delta), weights, n))

        for q in range(2):
            v = smooth_field(n, 1.0, 90 + q)
            h = 1e-7 / np.abs(v).max()
            fd = (L(rho0 + h * v) - L(rho0 - h * v)) / (2 * h)
            ad = float(np.sum(grad * v))
            print(f"band loss: fd {fd:.12e} adjoint {ad:.12e} rel {abs(fd - ad) / abs(ad):.2e}")
            assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


@pytest.mark.gpu
def test_iterate_adjoint_mixed_matches_fp64(mmh, fields):
    """The mixed form's gradient (FP32 inner solves, FP64 residual to tol)
    against the FP64 form's on the same reconstruction."""
    n, niter = N, 4
    rho = fields.lognormal_density(n, sigma=0.6, seed=63)
    wdelta = np.asfortranarray(np.random.default_rng(64).standard_normal((n, n, n)))
    g = {}
    for prec in (mmh.MMH_FP64, mmh.MMH_MIXED):
        with mmh.Context(n, precision=prec, schedule=mmh.MMH_SCHED_TOL, tol=1e-12, max_cycles=400) as ctx:
            ctx.load(np.zeros((n, n, n), order="F"), _u(rho))
            g[prec], _, _ = ctx.iterate_adjoint(niter, wdelta=wdelta, checkpoint_every=3)
    err = np.abs(g[mmh.MMH_MIXED] - g[mmh.MMH_FP64]).max() / np.abs(g[mmh.MMH_FP64]).max()
    print(f"mixed vs FP64 gradient: {err:.2e}")
    assert err <= 1e-8


@pytest.mark.gpu
def test_iterate_adjoint_with_the_compression_limiter_firing(mmh, fields):
    """Three iterations from a def with a compressing bump (centre curvature
    -0.95): the final compression test limits cells, and its FFT Poisson
    correction enters the reconstruction; the density gradient of
    J = sum wdef * def_N against central differences."""
    n, niter, every = 32, 3, 2
    rho = fields.lognormal_density(n, sigma=0.4, seed=91)
    x = np.arange(n) - n / 2
    r2 = x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2
    def0 = np.asfortranarray(0.95 * 9.0 * np.exp(-r2 / 18.0))
    wdef = np.asfortranarray(np.random.default_rng(92).standard_normal((n, n, n)))
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=TOL, max_cycles=400) as ctx:
        ctx.load(def0, _u(rho))
        d = ctx.iterate(1)
        assert d["ncompress"] > 0
        ctx.load(def0, _u(rho))
        grho, _, _ = ctx.iterate_adjoint(niter, wdef=wdef, checkpoint_every=every)

        def J(r):
            ctx.load(def0, _u(r))
            ctx.iterate(niter)
            dN = np.zeros((n, n, n), order="F")
            ctx.store(dN, None)
            return float(np.sum(wdef * dN))

        for q in range(2):
            v = smooth_field(n, 1.0, 93 + q)
            h = 1e-7 / np.abs(v).max()
            fd = (J(rho + h * v) - J(rho - h * v)) / (2 * h)
            ad = float(np.sum(grho * v))
            scale = float(np.sum(np.abs(grho * v)))
            print(f"limited reconstruction: fd {fd:.12e} adjoint {ad:.12e} rel {abs(fd - ad) / abs(ad):.2e} "
                  f"of sum {abs(fd - ad) / scale:.2e}")
            assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-3 * scale), (fd, ad)
