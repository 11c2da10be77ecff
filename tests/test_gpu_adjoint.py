"""calcdefp adjoint (no counterpart in the reference): the density and def
gradients of J = sum(w * defp) from mmh_calcdefp_adjoint_f64 against central
finite differences of J through mmh_calcdefp_f64 on the same inputs.

The limiter's branch choices are frozen in the adjoint, so each case checks,
on the CPU, that the finite-difference steps stay clear of every branch edge:
the +-1/dtaumesh flux clamps and the density clip at |1 - rho| = 2 (density
steps), the expansion mask det > 10 (def steps)."""
import numpy as np
import pytest

from conftest import smooth_field


def _s3(a):
    """The 27-point smoother (mmh/limiter.f90:677-781): [1,2,1]/4 along each axis."""
    for ax in range(3):
        a = 0.25 * np.roll(a, 1, ax) + 0.5 * a + 0.25 * np.roll(a, -1, ax)
    return a


def _max_hessian(g):
    d2 = [np.roll(g, 1, ax) - 2 * g + np.roll(g, -1, ax) for ax in range(3)]
    return max(np.abs(x).max() for x in d2)


def _det(d):
    """det(I + Hess(def)) as the metric computes it (gauss1.f90:1107-1210)."""
    r = np.roll
    a11 = 1 + r(d, -1, 0) - 2 * d + r(d, 1, 0)
    a22 = 1 + r(d, -1, 1) - 2 * d + r(d, 1, 1)
    a33 = 1 + r(d, -1, 2) - 2 * d + r(d, 1, 2)

    def cross(p, q):
        return 0.25 * (r(r(d, -1, p), -1, q) - r(r(d, 1, p), -1, q) - r(r(d, -1, p), 1, q) + r(r(d, 1, p), 1, q))

    a12, a23, a13 = cross(0, 1), cross(1, 2), cross(0, 2)
    return a11 * a22 * a33 + 2 * a12 * a13 * a23 - a13 * a13 * a22 - a11 * a23 * a23 - a12 * a12 * a33


def _bump(n, kappa, width):
    """-A exp(-r^2 / 2 width^2) at the box centre: centre curvature kappa (an
    expanding region, det > 10 for kappa > 1.16), rim curvature >= -0.45 kappa."""
    x = np.arange(n) - n / 2
    r2 = x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2
    return np.asfortranarray(-kappa * width * width * np.exp(-r2 / (2.0 * width * width)))


def _gap_threshold(t, lo=0.55, hi=0.85):
    """A flux-clamp level 1/dtaumesh in the widest gap of sorted |t| between
    quantiles lo and hi (some cells clamped, none near the edge)."""
    s = np.sort(np.abs(t).ravel())
    a, b = int(lo * s.size), int(hi * s.size)
    q = a + int(np.argmax(np.diff(s[a:b])))
    return 0.5 * (s[q] + s[q + 1]), 0.5 * (s[q + 1] - s[q])


CASES = {
    # 16^3, gentle def, clamps and the density clip active
    "clamps": dict(n=16, sigma=0.6, seed=31, kind="smooth", clamp=True),
    # 32^3, an expanding bump: expansion mask active, strongly curved metric
    "expansion": dict(n=32, sigma=0.4, seed=57, kind="bump", clamp=False),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_calcdefp_adjoint_matches_finite_differences(mmh, fields, case):
    p = CASES[case]
    n, dtold = p["n"], 0.5
    rho = fields.lognormal_density(n, sigma=p["sigma"], seed=p["seed"])
    if p["kind"] == "bump":
        defpot = _bump(n, kappa=1.3, width=3.0)
    else:
        g = smooth_field(n, 1.0, p["seed"] + 1)
        defpot = np.asfortranarray(g * (0.3 / _max_hessian(g)))
    rng = np.random.default_rng(p["seed"] + 2)
    w = _s3(rng.standard_normal((n, n, n)))
    w = np.asfortranarray(w - w.mean())
    dirs = [np.asfortranarray(_s3(rng.standard_normal((n, n, n)))) for _ in range(2)]
    ddirs = []
    for q in range(2):
        v = smooth_field(n, 1.0, p["seed"] + 10 + q)
        ddirs.append(np.asfortranarray(v / _max_hessian(v)))
    h = 1e-4

    # pass-1 input S^3 g (limiter.f90:153-166) and the branch edges
    t = _s3(_s3(_s3(np.clip(1.0 - rho, -2.0, 2.0) / 30.0 / dtold)))
    dt_max = max(h * np.abs(_s3(_s3(_s3(v)))).max() / 30.0 / dtold for v in dirs)
    if p["clamp"]:
        level, margin = _gap_threshold(t)
        assert margin > 20 * dt_max, (margin, dt_max)
        dtaumesh = 1.0 / level
        assert (np.abs(t) > level).sum() > 0
    else:
        dtaumesh = 1e-6
    edge = np.abs(np.abs(1.0 - rho) - 2.0).min()
    assert edge > 20 * h * max(np.abs(v).max() for v in dirs)
    if p["clamp"]:
        assert (np.abs(1.0 - rho) > 2.0).sum() > 0  # the clip is exercised
    det = _det(defpot)
    for v in ddirs:
        for sgn in (-1, 1):
            assert np.array_equal(det > 10.0, _det(defpot + sgn * 20 * h * v) > 10.0)

    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-13, max_cycles=400) as ctx:
        grho, gdef, d = ctx.calcdefp_adjoint(defpot, rho, w, dtold, dtaumesh, nfluid=1)
        assert d["ncompress"] == 0
        if p["kind"] == "bump":
            assert d["nexpand"] > 0

        def J(dp, r):
            defp = np.zeros((n, n, n), order="F")
            ctx.calcdefp(defp, None, None, np.asfortranarray(dp), np.asfortranarray(r), dtold, dtaumesh, nfluid=1)
            return float(np.sum(w * defp))

        for name, g, vs in (("rho", grho, dirs), ("def", gdef, ddirs)):
            for v in vs:
                if name == "rho":
                    fd = (J(defpot, rho + h * v) - J(defpot, rho - h * v)) / (2 * h)
                else:
                    fd = (J(defpot + h * v, rho) - J(defpot - h * v, rho)) / (2 * h)
                ad = float(np.sum(g * v))
                scale = float(np.sum(np.abs(g * v)))
                print(f"{case} d/d{name}: fd {fd:.12e} adjoint {ad:.12e} rel {abs(fd - ad) / abs(ad):.2e}")
                assert abs(fd - ad) <= 1e-7 * max(abs(ad), 1e-3 * scale), (name, fd, ad)


@pytest.mark.gpu
def test_calcdefp_adjoint_needs_a_solving_schedule(mmh, fields):
    n = 16
    rho = fields.lognormal_density(n, sigma=0.5, seed=3)
    z = np.zeros((n, n, n), order="F")
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_REF) as ctx:
        with pytest.raises(mmh.MMHError) as e:
            ctx.calcdefp_adjoint(z, rho, z, 1.0, 1.0, nfluid=1)
        assert e.value.code == mmh.MMH_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_relaxing_adjoint_matches_finite_differences(mmh, fields):
    """relaxing adjoint against central differences of relaxing.f90's density
    update, on the state of the first deformation iteration (def = defp =
    calcdefp's increment from def = 0, as main.f90:95-101 calls them)."""
    n, dt = 16, 1.0
    rho = fields.lognormal_density(n, sigma=0.6, seed=21)
    z = np.zeros((n, n, n), order="F")
    rng = np.random.default_rng(22)
    w = np.asfortranarray(_s3(rng.standard_normal((n, n, n))))
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-12) as ctx:
        defp = np.zeros((n, n, n), order="F")
        ctx.calcdefp(defp, None, None, z, rho, 1.0, 1.0, nfluid=1)
        defpot = defp.copy(order="F")
        gu, gdef, gdefp = ctx.relaxing_adjoint(rho, defpot, defp, w, dt, nfluidcmp=1)

        def J(r, dpot, dp):
            u = np.asfortranarray(r.copy())
            ctx.relaxing(u, np.asfortranarray(dpot), np.asfortranarray(dp), 1.0, dt, nfluidcmp=1)
            return float(np.sum(w * u))

        amp = np.abs(defp).max()
        checks = []
        for q in range(2):
            checks.append(("rho", gu, np.asfortranarray(_s3(rng.standard_normal((n, n, n))))))
            checks.append(("def", gdef, smooth_field(n, amp, 40 + q)))
            checks.append(("defp", gdefp, smooth_field(n, amp, 50 + q)))
        # The map is piecewise smooth (cflkeuler's maximum and the minmod
        # branches switch at kinks; at 16^3 some lie ~1e-5 away in these
        # directions), so the steps are small enough to stay on one piece.
        for name, g, v in checks:
            h = 1e-7 / max(np.abs(v).max(), 1e-300)
            args_p = [rho, defpot, defp]
            args_m = [rho, defpot, defp]
            k = ("rho", "def", "defp").index(name)
            args_p[k] = args_p[k] + h * v
            args_m[k] = args_m[k] - h * v
            fd = (J(*args_p) - J(*args_m)) / (2 * h)
            ad = float(np.sum(g * v))
            # bound relative to the summed per-cell contributions: in some def
            # directions the derivative is a cancellation of many cells and
            # the differences' round-off (~1e-14 / h) dominates |ad|
            scale = float(np.sum(np.abs(g * v)))
            print(f"relaxing d/d{name}: fd {fd:.12e} adjoint {ad:.12e} rel {abs(fd - ad) / abs(ad):.2e} "
                  f"of sum {abs(fd - ad) / scale:.2e}")
            assert abs(fd - ad) <= 1e-6 * max(abs(ad), scale), (name, fd, ad)


@pytest.mark.gpu
def test_calcdefp_adjoint_through_the_compression_correction(mmh, fields):
    """A compressing region (a bump in def with centre curvature -0.95, so the
    smallest eigenvalue of C = I + Hess(def) + dtold Hess(defp) falls below
    1/cmpmax = 0.1): the final compression test limits cells and its FFT
    Poisson correction (limiter.f90:425-597) enters defp.  The adjoint through
    it (mask frozen, d lambda_min / dC = v v^T, the correction's operator
    symmetric) against central differences; the masks of all three limiter
    tests are checked unchanged at the perturbed inputs."""
    n, dtold, dtaumesh, h = 32, 1.0, 1.0, 1e-5
    rho = fields.lognormal_density(n, sigma=0.4, seed=71)
    defpot = _bump(n, kappa=-0.95, width=3.0)
    rng = np.random.default_rng(72)
    w = _s3(rng.standard_normal((n, n, n)))
    w = np.asfortranarray(w - w.mean())
    dirs = [np.asfortranarray(_s3(rng.standard_normal((n, n, n)))) for _ in range(2)]
    ddirs = []
    for q in range(2):
        v = smooth_field(n, 1.0, 80 + q)
        ddirs.append(np.asfortranarray(v / _max_hessian(v)))
    edge = np.abs(np.abs(1.0 - rho) - 2.0).min()
    assert edge > 20 * h * max(np.abs(v).max() for v in dirs)
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-13, max_cycles=400) as ctx:
        grho, gdef, d = ctx.calcdefp_adjoint(defpot, rho, w, dtold, dtaumesh, nfluid=1)
        assert d["ncompress"] > 0
        ctx.keep_masks(True)

        def J(dp, r):
            defp = np.zeros((n, n, n), order="F")
            ctx.calcdefp(defp, None, None, np.asfortranarray(dp), np.asfortranarray(r), dtold, dtaumesh, nfluid=1)
            return float(np.sum(w * defp)), ctx.masks()

        _, m0 = J(defpot, rho)
        assert m0["compress2"].sum() > 0
        for name, g, vs in (("rho", grho, dirs), ("def", gdef, ddirs)):
            for v in vs:
                if name == "rho":
                    (jp, mp), (jm, mm) = J(defpot, rho + h * v), J(defpot, rho - h * v)
                else:
                    (jp, mp), (jm, mm) = J(defpot + h * v, rho), J(defpot - h * v, rho)
                for key in m0:
                    assert np.array_equal(mp[key], m0[key]) and np.array_equal(mm[key], m0[key]), (name, key)
                fd = (jp - jm) / (2 * h)
                ad = float(np.sum(g * v))
                scale = float(np.sum(np.abs(g * v)))
                print(f"compression correction d/d{name}: fd {fd:.12e} adjoint {ad:.12e} "
                      f"rel {abs(fd - ad) / abs(ad):.2e} of sum {abs(fd - ad) / scale:.2e}")
                assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-3 * scale), (name, fd, ad)
