"""The mixed form's own FP64 kernels against the oracle, one by one.

In an MMH_MIXED context the drop-in entry points run the kernels mmh_iterate
runs in that form, which are not bit-matched to the reference:
* the metric (cbajraw, mmh/gauss1.f90:1107-1210) takes rho_bar/det once and
  six products instead of six divisions: each coefficient within 4 ulp;
* nsmooth (mmh/limiter.f90:677-781) runs as three axis passes of
  [1/4, 1/2, 1/4] instead of the 27-point sum: within 1e-15 of max |a|;
* relaxing (mmh/relaxing.f90:21-1139) forms its fluxes in FP32 and the
  update in FP64: the density within 5e-8 relative after one step (an FP32
  restatement in numpy gives 6e-9 at 32^3 for a step that moves the density
  by 0.2).
* the float-float metric of the outer residual (k_metric_ff) within
  1e-13 + 2^-44 max|def| of the largest coefficient;
* the limiter's pass 1 and final compression test screen cells in FP32 and
  evaluate in FP64 only where a decision is close: fluxes, masks and defplim
  identical to the FP64 form's.
The float-float outer residual (k_residual_ff) is checked against an FP64
recomputation in test_gpu_parity.py::test_multigrid_mixed_float_float_outer_loop.
"""
import numpy as np
import pytest

from conftest import smooth_field

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


@pytest.mark.parametrize("n", [16, 32, 64])
def test_mixed_metric_one_division(mmh, oracle, fields, n):
    defpot = smooth_field(n, 0.3, 11 + n)
    rho = fields.lognormal_density(n, sigma=1.0, seed=12 + n)
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        for dx in (1.0, 2.0):
            g = ctx.metric(defpot, rho, dx)
            o = oracle.metric(defpot, rho, dx)
            assert np.all(np.abs(g - o) <= 4 * EPS * np.abs(o)), np.abs(g - o).max()


def _det_numpy(defpot, dx):
    """det(I + Hess(def)) with the reference's central differences, FP64 numpy."""
    d = defpot
    r = lambda a, s, ax: np.roll(a, -s, axis=ax)
    di2 = 1.0 / (dx * dx)
    hxx = (r(d, 1, 0) - 2 * d + r(d, -1, 0)) * di2
    hyy = (r(d, 1, 1) - 2 * d + r(d, -1, 1)) * di2
    hzz = (r(d, 1, 2) - 2 * d + r(d, -1, 2)) * di2
    hxy = (r(r(d, 1, 0), 1, 1) - r(r(d, -1, 0), 1, 1) - r(r(d, 1, 0), -1, 1) + r(r(d, -1, 0), -1, 1)) * di2 * 0.25
    hyz = (r(r(d, 1, 1), 1, 2) - r(r(d, 1, 1), -1, 2) - r(r(d, -1, 1), 1, 2) + r(r(d, -1, 1), -1, 2)) * di2 * 0.25
    hxz = (r(r(d, 1, 0), 1, 2) - r(r(d, -1, 0), 1, 2) - r(r(d, 1, 0), -1, 2) + r(r(d, -1, 0), -1, 2)) * di2 * 0.25
    a11, a22, a33 = 1 + hxx, 1 + hyy, 1 + hzz
    return a11 * (a22 * a33 - hyz * hyz) + hxy * (hxz * hyz - hxy * a33) + hxz * (hxy * hyz - hxz * a22)


@pytest.mark.parametrize("n", [16, 32, 64])
def test_mixed_metric_float_float(mmh, oracle, fields, n):
    """The mixed form's float-float metric (k_metric_ff: inputs split into
    float pairs from their bit patterns, everything on the FP32 pipes)
    against the oracle's FP64 metric.  A pair holds a double to 2^-48 of its
    magnitude, so a Hessian entry (differences of four samples of def) is
    within ~2^-46 max|def| / dx^2: every coefficient must be within
    1e-13 + 2^-44 max|def| of the largest coefficient, and det likewise of
    max |det|.  A deformation potential offset by 300 shows that term."""
    for amp, off in ((0.3, 0.0), (0.3, 300.0)):
        defpot = np.asfortranarray(smooth_field(n, amp, 21 + n) + off)
        rho = fields.lognormal_density(n, sigma=1.0, seed=22 + n)
        with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
            for dx in (1.0, 2.0):
                g, det = ctx.metric_ff(defpot, rho, dx)
                o = oracle.metric(defpot, rho, dx)
                err = np.abs(g - o).max() / np.abs(o).max()
                dn = _det_numpy(defpot, dx)
                derr = np.abs(det - dn).max() / np.abs(dn).max()
                bound = 1e-13 + 2.0 ** -44 * np.abs(defpot).max()
                print(f"metric_ff {n}^3 offset {off} dx {dx}: coefficients {err:.2e}, det {derr:.2e} "
                      f"(bound {bound:.1e})")
                assert err <= bound and derr <= bound, (err, derr, bound)
    with mmh.Context(n, precision=mmh.MMH_FP64) as ctx:
        with pytest.raises(mmh.MMHError):
            ctx.metric_ff(defpot, rho, 1.0)


@pytest.mark.parametrize("n,amp,off", [(16, 2.0, 0.0), (32, 4.0, 0.0), (32, 4.0, 300.0), (64, 3.0, 0.0)])
def test_mixed_limiter_pass1_same_decisions(mmh, oracle, fields, n, amp, off):
    """The mixed form's pass 1 (every cell screened in FP32 from truncated
    samples with a bounded error, FP64 only where a decision is close)
    against the oracle: the flux and both trigger masks bit-identical, the
    expansion count equal; the det extrema and rho2, which come from the
    float-float det, within 1e-12.  The offset puts the samples far above
    their differences, which widens the screen's margin."""
    defpot = np.asfortranarray(smooth_field(n, amp, 77) + off)
    _, u = fields.initial_state(n, sigma=1.0, seed=78)
    rho = np.asfortranarray(u[0])
    tmp0 = np.asfortranarray(np.random.default_rng(n).standard_normal((n, n, n)) * 0.05)
    to, mxo, mco, do = oracle.limiter_pass1(tmp0, defpot, u)
    tg = tmp0.copy(order="F")
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        mxg, mcg, dg = ctx.limiter_pass1(tg, defpot, rho)
    print(f"pass 1 {n}^3 amp {amp} offset {off}: expand {int(mxo.sum())}, compress {int(mco.sum())}; "
          f"det max {dg['detmax']} vs {do['detmax']}, rho2 {dg['rho2']} vs {do['rho2']}")
    assert np.array_equal(mxo, mxg) and np.array_equal(mco, mcg)
    assert np.array_equal(to, tg)
    assert do["nexpand"] == dg["nexpand"]
    for key in ("detmax", "detmin", "rho2"):
        assert abs(dg[key] - do[key]) <= 1e-12 * abs(do[key]), key
    assert mco.sum() > 0


@pytest.mark.parametrize("n,amp,off", [(16, 2.0, 0.0), (32, 4.0, 0.0), (32, 4.0, 300.0), (64, 3.0, 0.0)])
def test_mixed_limiter_mask_same_decisions(mmh, oracle, n, amp, off):
    """The mixed form's final compression test (FP32 screen, FP64 for the
    cells that may matter) against the FP64 form: defplim and the mask
    bit-identical, the count and the largest compression equal; the mask
    also equals the oracle's."""
    defpot = np.asfortranarray(smooth_field(n, amp, 91) + off)
    defp = smooth_field(n, amp * 0.3, 92)
    _, mo, do = oracle.limiter_mask(defpot, defp)
    with mmh.Context(n) as ctx:
        l64, m64, d64 = ctx.limiter_mask(defpot, defp)
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        lm, mm, dm = ctx.limiter_mask(defpot, defp)
    print(f"mask {n}^3 amp {amp} offset {off}: limited {int(mm.sum())}, cmax {dm['cmax']}")
    assert np.array_equal(m64, mm) and np.array_equal(mo, mm)
    assert np.array_equal(l64, lm)
    assert d64["ncompress"] == dm["ncompress"] == do["ncompress"] and dm["ncompress"] > 0
    assert d64["cmax"] == dm["cmax"]


@pytest.mark.parametrize("n", [16, 32, 64])
def test_mixed_nsmooth_axis_passes(mmh, oracle, n):
    a = np.asfortranarray(np.random.default_rng(n).standard_normal((n, n, n)))
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        g = a.copy(order="F")
        ctx.nsmooth(g)
    o = oracle.nsmooth(a)
    assert np.abs(g - o).max() <= 1e-15 * np.abs(a).max()


@pytest.mark.parametrize("n", [16, 32, 64])
def test_mixed_relaxing_fp32_fluxes(mmh, oracle, fields, n):
    defpot = smooth_field(n, 0.3, 8)
    defp = smooth_field(n, 0.05, 9)
    _, u = fields.initial_state(n, sigma=1.0, seed=10)
    uo = oracle.relaxing(u, defpot, defp)
    ug = u.copy(order="F")
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        ctx.relaxing(ug, defpot, defp)
    err = np.abs(ug[0] - uo[0]).max() / np.abs(uo[0]).max()
    print(f"mixed relaxing {n}^3: {err:.2e}")
    assert err <= 5e-8
    assert np.all(ug[1:] == 0)


@pytest.mark.parametrize("n,nrelax,iopt", [(64, 1, 18), (64, 3, 18), (128, 2, 18), (256, 2, 18), (32, 2, 18),
                                           (128, 2, 19)])
def test_mixed_relax_fp32_sweeps(mmh, oracle, fields, n, nrelax, iopt):
    """The mixed form's FP32 Gauss-Seidel sweeps (one launch per whole sweep
    from 64^3 up) against the oracle's FP64 relax in the reference's plane
    order: every cell within 1e-5 of max |phi| (FP32 rounding), the residual
    norm within 1e-4 relative."""
    defpot = smooth_field(n, 0.05, 5 + n)
    rho = fields.lognormal_density(n, sigma=0.5, seed=6 + n)
    rng = np.random.default_rng(n + nrelax)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi0 = np.asfortranarray(rng.standard_normal((n, n, n)))
    coef = oracle.metric(defpot, rho, 1.0)
    a = phi0.copy(order="F")
    ro, rio = oracle.relax(a, rhs, coef, 1.0, nrelax, iopt, colour8=True)
    b = phi0.copy(order="F")
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        rg, rig = ctx.relax(b, rhs, defpot, rho, 1.0, nrelax, iopt)
    err = np.abs(b - a).max() / np.abs(a).max()
    print(f"FP32 relax {n}^3 x{nrelax}: phi {err:.2e}, rinf {rio:.6e} vs {rig:.6e}")
    assert err <= 1e-5
    assert abs(rig - rio) <= 1e-4 * rio
    if iopt % 8 == 3:
        assert np.abs(rg - ro).max() <= 1e-4 * np.abs(ro).max()


SHAPES = [(32, 16), (64, 8), (16, 32), (32, 8), (64, 128), (64, 256)]


@pytest.mark.parametrize("n", [64, 128, 256])
def test_fp32_sweep_tile_shapes_agree_bit_for_bit(mmh, oracle, fields, n):
    """The tile shapes of the FP32 plane kernel and the strips marching in y
    (shapes 4-6) compute the same bits, each pinned in turn: two sweeps with
    their residual norm (relax), and a whole mixed solve, whose V-cycles run
    the first sweep of every level from zero with the zero-field variants.
    Left to itself, the library times the shapes on a grid's first sweeps and
    reports the one it keeps."""
    nrelax = 2
    defpot = smooth_field(n, 0.05, 7)
    _, u = fields.initial_state(n, sigma=0.5, seed=8)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(9)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi0 = np.asfortranarray(rng.standard_normal((n, n, n)))
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    out = []
    nfit = 0
    try:
        with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL, tol=1e-8, max_cycles=200) as ctx:
            for shape, (tx, ty) in enumerate(SHAPES):
                fits = n >= tx + 8 and n >= ty + 8 if shape < 4 else (n // 2) % (ty // 2) == 0
                if not fits:
                    continue
                nfit += 1
                mmh.gs_tile_pin(shape)
                b = phi0.copy(order="F")
                _, rinf = ctx.relax(b, rhs, defpot, rho, 1.0, nrelax, 18)
                ug = np.zeros((n, n, n), order="F")
                rg = rhs0.copy(order="F")
                d = ctx.multigrid(ug, rg, defpot, u, 1.0, n, n, n, 5)
                out.append((shape, b, rinf, ug, d["vcycles"]))
            mmh.gs_tile_pin(-1)
    finally:
        mmh.gs_tile_pin(-1)
    assert len(out) == nfit >= 2
    for shape, b, rinf, ug, cyc in out[1:]:
        assert np.array_equal(b, out[0][1]), shape
        assert rinf == out[0][2], shape
        assert np.array_equal(ug, out[0][3]), shape
        assert cyc == out[0][4], shape
    print(f"{n}^3: {len(out)} shapes agree; solve {out[0][4]} cycles")


def test_fp32_tile_shape_kept_after_timing(mmh, fields):
    """With no shape pinned, the first sweep on a grid times the shapes that
    fit and keeps one of them."""
    n = 128
    defpot = smooth_field(n, 0.05, 7)
    rho = fields.lognormal_density(n, sigma=0.5, seed=8)
    rng = np.random.default_rng(9)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    b = np.asfortranarray(rng.standard_normal((n, n, n)))
    mmh.gs_tile_pin(-1)
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL) as ctx:
        ctx.relax(b, rhs, defpot, rho, 1.0, 2, 18)
        chosen = mmh.gs_tile(n)
    print("tile kept for 128^3:", chosen)
    assert chosen in SHAPES


@pytest.mark.parametrize("n", [64, 128])
def test_fp32_stencil_marching_agrees_bit_for_bit(mmh, fields, n):
    """The marching FP32 residual / operator stencil (a CTA walks 8 planes of
    its tile column and copies the next plane while computing one) gives the
    bits of the one-plane-per-CTA kernel, each pinned in turn: a relax with
    its residual norm and restricted residual (iresidopt 3), and a whole
    mixed solve (V-cycle residuals and the conjugate-gradient operator)."""
    defpot = smooth_field(n, 0.05, 17)
    _, u = fields.initial_state(n, sigma=0.5, seed=18)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(19)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi0 = np.asfortranarray(rng.standard_normal((n, n, n)))
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    out = {}
    try:
        with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_TOL, tol=1e-8, max_cycles=200) as ctx:
            for kind in (0, 1):
                mmh.stencil_pin(kind)
                b = phi0.copy(order="F")
                resid, rinf = ctx.relax(b, rhs, defpot, rho, 1.0, 2, 19)
                ug = np.zeros((n, n, n), order="F")
                rg = rhs0.copy(order="F")
                d = ctx.multigrid(ug, rg, defpot, u, 1.0, n, n, n, 5)
                out[kind] = (b, resid, rinf, ug, d["vcycles"], d["resid_rel"])
    finally:
        mmh.stencil_pin(-1)
    print(f"{n}^3: solve {out[1][4]} cycles to {out[1][5]:.2e}")
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
