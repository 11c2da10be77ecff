"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

FP64 form: every kernel that involves no libm transcendental and no FFT is
required to reproduce the oracle bit for bit (the oracle restates the
reference's arithmetic; the GPU evaluates the same operations in the same
order without FMA contraction, and the reference's plane schedule is executed
in its equivalent 8-colour order).  Spectral results (cuFFT against the
oracle's own FFT) are compared with a relative tolerance of 1e-10, the bound
the reference path is held to in FP64 mode.
"""
import numpy as np
import pytest

from conftest import smooth_field

pytestmark = pytest.mark.gpu

TOL_SPECTRAL = 1e-10


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def case(fields, n, seed, sigma=1.0, amp=0.05):
    defpot, u = fields.initial_state(n, sigma=sigma, seed=seed)
    if amp:
        defpot = smooth_field(n, amp, seed + 100)
    return defpot, u


@pytest.mark.parametrize("n", [8, 16, 32])
def test_metric_bitexact(mmh, oracle, fields, n):
    defpot, u = case(fields, n, 11)
    rho = np.asfortranarray(u[0])
    with mmh.Context(n) as ctx:
        for dx in (1.0, 2.0):
            g = ctx.metric(defpot, rho, dx)
            o = oracle.metric(defpot, rho, dx)
            assert np.array_equal(g, o)


@pytest.mark.parametrize("n,nrelax,iopt", [(8, 2, 19), (16, 4, 19), (32, 4, 19), (32, 8, 19), (16, 3, 18),
                                           (32, 1, 19), (16, 16, 19), (4, 32, 18), (16, 0, 19), (64, 4, 19),
                                           (64, 2, 18), (128, 4, 19)])
def test_relax_bitexact(mmh, oracle, fields, n, nrelax, iopt):
    """relax(): the literal r1lax plane schedule of the oracle vs the GPU's 8-colour sweeps."""
    defpot, u = case(fields, n, 5 + n)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(n + nrelax)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi0 = np.asfortranarray(rng.standard_normal((n, n, n)))
    coef = oracle.metric(defpot, rho, 1.0)
    a = phi0.copy(order="F")
    ro, rio = oracle.relax(a, rhs, coef, 1.0, nrelax, iopt, colour8=False)
    b = phi0.copy(order="F")
    with mmh.Context(max(n, 8)) as ctx:
        rg, rig = ctx.relax(b, rhs, defpot, rho, 1.0, nrelax, iopt)
    assert np.array_equal(a, b)
    assert rio == rig
    if iopt % 8 == 3:
        assert np.array_equal(ro, rg)


@pytest.mark.parametrize("n", [8, 16, 32])
def test_small_ops_bitexact(mmh, oracle, fields, n):
    rng = np.random.default_rng(n)
    a = np.asfortranarray(rng.standard_normal((n, n, n)))
    h = np.asfortranarray(rng.standard_normal((n // 2,) * 3))
    defpot, u = case(fields, n, 3)
    with mmh.Context(n) as ctx:
        assert np.array_equal(ctx.restrict(a), oracle.restrict(a))
        x = a.copy(order="F"); y = a.copy(order="F")
        ctx.inject(x, h); oracle.prolong_add(y, h)
        assert np.array_equal(x, y)
        x = a.copy(order="F")
        ctx.nsmooth(x)
        assert np.array_equal(x, oracle.nsmooth(a))
        x = a.copy(order="F"); y = a.copy(order="F")
        ctx.zerosum(x); oracle.zerosum(y)
        assert np.array_equal(x, y)
        x = a.copy(order="F"); y = a.copy(order="F")
        ctx.rgzerosum(x, defpot, 1.0); oracle.rgzerosum(y, defpot, 1.0)
        assert np.array_equal(x, y)


@pytest.mark.parametrize("n", [8, 16, 32, 64, 128])
def test_multigrid_ref_bitexact(mmh, oracle, fields, n):
    """multigrid(...) with the reference schedule (one V-cycle, 4*NG/n sweeps)."""
    defpot, u = case(fields, n, 21, sigma=1.5)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(n)
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    uo = np.zeros((n, n, n), order="F"); ro = rhs0.copy(order="F")
    rc, do = oracle.multigrid(uo, ro, defpot, rho, 1.0, sched=oracle.SCHED_REF)
    ug = np.zeros((n, n, n), order="F"); rg = rhs0.copy(order="F")
    with mmh.Context(n) as ctx:
        dg = ctx.multigrid(ug, rg, defpot, u, 1.0, n, n, n, 5)
    assert np.array_equal(ro, rg)
    assert np.array_equal(uo, ug)
    assert do["relaxerr"] == dg["relaxerr"] and do["r1"] == dg["r1"]
    assert do["guards"] == dg["guards"]


def test_multigrid_subgrid_entry(mmh, oracle, fields):
    """multigrid called on a grid smaller than NG (mgN with nrelax = 4*NG/n)."""
    NG, n = 32, 16
    defpot, u = case(fields, n, 23, sigma=1.0)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(3)
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    import ctypes as C
    ug = np.zeros((n, n, n), order="F"); rg = rhs0.copy(order="F")
    with mmh.Context(NG) as ctx:
        ctx.multigrid(ug, rg, defpot, u, 2.0, n, n, n, 5)
    exp_u = np.zeros((n, n, n), order="F"); exp_r = rhs0.copy(order="F")
    rc = oracle.lib().orc_multigrid_ng_d(oracle._p(exp_u), oracle._p(exp_r), oracle._p(defpot), oracle._p(rho), n,
                                         NG, C.c_double(2.0))
    assert rc == 0
    assert np.array_equal(exp_r, rg)
    assert np.array_equal(exp_u, ug)


@pytest.mark.parametrize("n,sched", [(16, 1), (32, 1), (64, 1), (16, 2), (32, 2)])
def test_multigrid_tol_fp64_bitexact(mmh, oracle, fields, n, sched):
    """Tolerance schedules in FP64: flexible PCG (sched 1) and repeated V-cycles
    (sched 2) reproduce the oracle bit for bit, iteration count included."""
    defpot, u = case(fields, n, 31, sigma=1.5)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(n + 1)
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    uo = np.zeros((n, n, n), order="F"); ro = rhs0.copy(order="F")
    rc, do = oracle.multigrid(uo, ro, defpot, rho, 1.0, sched=sched, tol=1e-10, maxcyc=200, colour8=True)
    ug = np.zeros((n, n, n), order="F"); rg = rhs0.copy(order="F")
    with mmh.Context(n, schedule=sched, tol=1e-10, max_cycles=200) as ctx:
        dg = ctx.multigrid(ug, rg, defpot, u, 1.0, n, n, n, 5)
    assert do["resid_rel"] <= 1e-10 and dg["resid_rel"] <= 1e-10
    assert do["vcycles"] == dg["vcycles"]
    assert np.array_equal(uo, ug)
    assert do["resid_rel"] == dg["resid_rel"]


@pytest.mark.parametrize("n,sched", [(16, 1), (32, 1), (64, 1), (32, 2)])
def test_multigrid_mixed_converges(mmh, oracle, fields, n, sched):
    """Mixed form: FP32 V-cycles inside FP64 PCG (sched 1) or an FP64
    defect-correction loop (sched 2) reach the FP64 tolerance, and the
    potential agrees with the converged FP64 oracle."""
    defpot, u = case(fields, n, 41, sigma=1.5)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(n + 2)
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    uo = np.zeros((n, n, n), order="F"); ro = rhs0.copy(order="F")
    oracle.multigrid(uo, ro, defpot, rho, 1.0, sched=1, tol=1e-12, maxcyc=300, colour8=True)
    ug = np.zeros((n, n, n), order="F"); rg = rhs0.copy(order="F")
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=sched, tol=1e-12, max_cycles=300) as ctx:
        dg = ctx.multigrid(ug, rg, defpot, u, 1.0, n, n, n, 5)
    assert dg["resid_rel"] <= 1e-12
    assert rel(ug, uo) <= 1e-9


@pytest.mark.parametrize("n", [32, 64, 128])
def test_multigrid_mixed_float_float_outer_loop(mmh, oracle, fields, n):
    """Mixed form at a tolerance the float-float outer residual serves
    (>= 1e-10): the solve reaches it, the residual it reports agrees with an
    FP64 recomputation of rhs - L[u] from the oracle, and the potential
    agrees with the converged FP64 oracle to the accuracy the tolerance
    allows."""
    defpot, u = case(fields, n, 43, sigma=1.5)
    rho = np.asfortranarray(u[0])
    rng = np.random.default_rng(n + 5)
    rhs0 = np.asfortranarray(rng.standard_normal((n, n, n)) * 0.01)
    uo = np.zeros((n, n, n), order="F"); ro = rhs0.copy(order="F")
    oracle.multigrid(uo, ro, defpot, rho, 1.0, sched=1, tol=1e-12, maxcyc=300, colour8=True)
    ug = np.zeros((n, n, n), order="F"); rg = rhs0.copy(order="F")
    with mmh.Context(n, precision=mmh.MMH_MIXED, schedule=1, tol=1e-10, max_cycles=300) as ctx:
        dg = ctx.multigrid(ug, rg, defpot, u, 1.0, n, n, n, 5)
    assert dg["resid_rel"] <= 1e-10
    r64 = oracle.residual(ug, rg, oracle.metric(defpot, rho))
    rel64 = np.abs(r64).max() / np.abs(rg).max()
    assert abs(rel64 - dg["resid_rel"]) <= 1e-12
    assert rel(ug, uo) <= 1e-7


@pytest.mark.parametrize("precision", ["MMH_MIXED", "MMH_FP64"])
def test_graph_replay_matches_direct_launches(mmh, fields, precision):
    """The preconditioner cycle replayed from a CUDA graph gives the same bits
    as launched kernel by kernel (the timing hooks force direct launches)."""
    n = 64
    rho = fields.lognormal_density(n, sigma=0.5, seed=91)
    out = []
    for direct in (False, True):
        with mmh.Context(n, precision=getattr(mmh, precision), schedule=mmh.MMH_SCHED_TOL, tol=1e-9) as ctx:
            ctx.load(None, rho.reshape((1, n, n, n), order="F"))
            if direct:
                mmh.profile_start(mmh.K_GS)
            launches = mmh.launch_count()
            d = ctx.iterate(2)
            launches = mmh.launch_count() - launches
            if direct:
                mmh.profile_stop()
            got = np.zeros((n, n, n), order="F")
            ctx.store(got, None)
        out.append((got, d["vcycles"], launches))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]
    assert out[0][2] == out[1][2]  # replays count the kernels they run


@pytest.mark.parametrize("n,amp", [(16, 4.0), (32, 2.0), (32, 8.0)])
def test_limiter_pass1_masks(mmh, oracle, fields, n, amp):
    """Pass-1 flux limiter: flux field and both trigger masks identical."""
    defpot = smooth_field(n, amp, 77)
    _, u = fields.initial_state(n, sigma=1.0, seed=78)
    rho = np.asfortranarray(u[0])
    tmp0 = np.asfortranarray(np.random.default_rng(n).standard_normal((n, n, n)) * 0.05)
    to, mxo, mco, do = oracle.limiter_pass1(tmp0, defpot, u)
    tg = tmp0.copy(order="F")
    with mmh.Context(n) as ctx:
        mxg, mcg, dg = ctx.limiter_pass1(tg, defpot, rho)
    assert np.array_equal(mxo, mxg) and np.array_equal(mco, mcg)
    assert np.array_equal(to, tg)
    assert do["nexpand"] == dg["nexpand"]
    assert do["detmax"] == dg["detmax"] and do["detmin"] == dg["detmin"]
    assert mco.sum() > 0


@pytest.mark.parametrize("n,amp", [(16, 2.0), (32, 4.0)])
def test_limiter_mask_and_poisson(mmh, oracle, fields, n, amp):
    defpot = smooth_field(n, amp, 91)
    defp = smooth_field(n, amp * 0.3, 92)
    lo, mo, do = oracle.limiter_mask(defpot, defp)
    with mmh.Context(n) as ctx:
        lg, mg, dg = ctx.limiter_mask(defpot, defp)
        assert np.array_equal(mo, mg)
        assert do["ncompress"] == dg["ncompress"] and do["ncompress"] > 0
        assert rel(lg, lo) <= 1e-13
        pg = defp.copy(order="F")
        ctx.limiter_poisson(pg, lo)
    po = oracle.limiter_poisson(defp, lo)
    assert rel(pg - defp, po - defp) <= TOL_SPECTRAL


@pytest.mark.parametrize("n", [8, 16, 32])
def test_spectral_outputs(mmh, oracle, fields, n):
    defpot = smooth_field(n, 0.3, 5)
    go = oracle.gradient(defpot)
    do = oracle.delta(defpot)
    gg = np.zeros((n, n, n, 3), order="F")
    dg = np.zeros((n, n, n), order="F")
    with mmh.Context(n) as ctx:
        ctx.scalar2gradient(defpot, gg, (n, n, n))
        ctx.defp2delta(defpot, dg, (n, n, n))
    assert rel(gg, go) <= TOL_SPECTRAL
    assert rel(dg, do) <= TOL_SPECTRAL


@pytest.mark.parametrize("n", [16, 32])
def test_relaxing_bitexact(mmh, oracle, fields, n):
    defpot = smooth_field(n, 0.3, 8)
    defp = smooth_field(n, 0.05, 9)
    _, u = fields.initial_state(n, sigma=1.0, seed=10)
    uo = oracle.relaxing(u, defpot, defp)
    ug = u.copy(order="F")
    with mmh.Context(n) as ctx:
        ctx.relaxing(ug, defpot, defp)
    assert np.array_equal(uo, ug)
    assert np.all(ug[1:] == 0)


@pytest.mark.parametrize("n", [16, 32])
def test_relaxing_degenerate_cells(mmh, oracle, fields, n):
    """Cells with zero density and a tangled metric take the relaxing
    kernels' general paths (0/x by division, the full sound-speed expression,
    minmod with NaN operands): the density has the oracle's bits, NaN where
    the reference produces NaN.  (The reference's momentum and energy turn
    NaN next to an empty cell, 0/0 in its velocity; the GPU carries only the
    density and leaves u(2:5) at zero.)"""
    defpot = smooth_field(n, 3.0, 18)  # strong deformation: tangled cells, det <= 0
    defp = smooth_field(n, 0.05, 19)
    _, u = fields.initial_state(n, sigma=1.0, seed=20)
    rng = np.random.default_rng(n)
    flat = u[0].reshape(-1, order="F")
    flat[rng.choice(flat.size, 12, replace=False)] = 0.0  # empty cells
    u[0] = flat.reshape((n, n, n), order="F")
    uo = oracle.relaxing(u, defpot, defp)
    ug = u.copy(order="F")
    with mmh.Context(n) as ctx:
        ctx.relaxing(ug, defpot, defp)
    assert np.array_equal(uo[0], ug[0], equal_nan=True)
    assert np.isnan(uo[0]).any()  # the degenerate cells did reach the general paths
    assert np.all(ug[1:] == 0)


@pytest.mark.parametrize("n,sigma,amp", [(16, 1.0, 0.05), (32, 1.5, 0.3), (16, 1.0, 2.0), (32, 1.5, 2.0)])
def test_calcdefp_ref(mmh, oracle, fields, n, sigma, amp):
    """calcdefp (reference schedule): bit-exact without the FFT correction,
    within 1e-10 with it."""
    defpot, u = case(fields, n, 51, sigma=sigma, amp=amp)
    do_, masks, diag_o, rc = oracle.calcdefp(defpot, u)
    dg = np.zeros((n, n, n), order="F")
    with mmh.Context(n) as ctx:
        diag_g = ctx.calcdefp(dg, None, None, defpot, u)
    assert diag_o["nexpand"] == diag_g["nexpand"]
    assert diag_o["ncompress"] == diag_g["ncompress"]
    if diag_o["ncompress"] == 0:
        assert np.array_equal(do_, dg)
    else:
        assert rel(dg, do_) <= TOL_SPECTRAL


@pytest.mark.parametrize("n,niter", [(16, 3), (32, 3), (64, 2)])
def test_iterations_ref(mmh, oracle, fields, n, niter):
    """Whole deformation iterations (calcdefp, def += defp, relaxing) on a
    field the reference algorithm handles stably (sigma_lnrho = 1)."""
    defpot, u = fields.initial_state(n, sigma=1.0, seed=61)
    do_, uo = defpot, u
    for _ in range(niter):
        do_, uo, _, _, _ = oracle.iteration(do_, uo, sched=oracle.SCHED_REF)
    with mmh.Context(n) as ctx:
        ctx.load(defpot, u)
        ctx.iterate(niter)
        dg = np.zeros((n, n, n), order="F")
        ug = np.zeros((5, n, n, n), order="F")
        ctx.store(dg, ug)
    assert rel(dg, do_) <= 1e-10
    assert rel(ug[0], uo[0]) <= 1e-10


def test_errors(mmh, fields):
    n = 16
    with mmh.Context(n) as ctx:
        a = np.zeros((n, n, n), order="F")
        ub = np.zeros((5, n, n, n), order="F")
        ub[0] = 1
        with pytest.raises(mmh.MMHError) as e:
            ctx.multigrid(a, a.copy(order="F"), a, ub, 1.0, n, n, 8, 5)
        assert e.value.code == -2
        with pytest.raises(mmh.MMHError) as e:
            ctx.multigrid(a, a.copy(order="F"), a, ub, 1.0, n, n, n, 5, nred=2)
        assert e.value.code == -1
        with pytest.raises(mmh.MMHError) as e:
            ctx.multigrid(a, a.copy(order="F"), a, ub, 1.0, n, n, n, 5, iopt=1)
        assert e.value.code == -1
        ub[2, 3, 3, 3] = 0.5
        with pytest.raises(mmh.MMHError) as e:
            ctx.relaxing(ub, a, a)
        assert e.value.code == -7
    with pytest.raises(mmh.MMHError) as e:
        mmh.Context(24)
    assert e.value.code == -3
    with pytest.raises(mmh.MMHError) as e:
        mmh.Context(16, precision=mmh.MMH_MIXED, schedule=mmh.MMH_SCHED_REF)
    assert e.value.code == -1


def test_injected_failures(mmh, fields):
    """Failures made on the host, never on the GPU: a NaN seeded into the
    density, a deformation potential whose determinants leave the exact-sum
    range, a solve allowed too few cycles.  Each call returns its status and
    the context stays usable."""
    n = 16
    rho = fields.lognormal_density(n, sigma=0.5, seed=5)
    z = np.zeros((n, n, n), order="F")
    defp = np.zeros((n, n, n), order="F")
    failed = (mmh.MMH_ERR_NAN, mmh.MMH_ERR_RANGE)
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-10, max_cycles=200) as ctx:
        bad = rho.copy(order="F")
        bad[3, 4, 5] = np.nan
        with pytest.raises(mmh.MMHError) as e:
            ctx.calcdefp(defp, None, None, z, bad, 1.0, 1.0, nfluid=1)
        assert e.value.code in failed
        spike = np.zeros((n, n, n), order="F")
        spike[7, 7, 7] = 1e12
        with pytest.raises(mmh.MMHError) as e:
            ctx.calcdefp(defp, None, None, spike, rho, 1.0, 1.0, nfluid=1)
        assert e.value.code in failed
        d = ctx.calcdefp(defp, None, None, z, rho, 1.0, 1.0, nfluid=1)
        assert d["status"] == 0 and np.isfinite(defp).all()
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_TOL, tol=1e-14, max_cycles=2) as ctx:
        d = ctx.calcdefp(defp, None, None, z, rho, 1.0, 1.0, nfluid=1)
        assert d["status"] == mmh.MMH_ERR_DIVERGED
