"""Known-answer tests that pin the CPU oracle (no GPU needed).

The reference ships no golden vectors and its self-tests do not compile, so
the oracle is pinned by analytic cases: the flat-metric Laplacian, cosine
deformations with closed-form Hessians, the separable smoothing filter,
eigenvalues against numpy.linalg.eigvalsh, the spectral derivative of a sine,
conservation of mass by the relaxing update, and the reference's own
test3d point-source problem (mmh/gauss1.f90:1573-1608) solved to convergence.
"""
import math

import numpy as np
import pytest

from conftest import smooth_field


def flat_case(n):
    return np.zeros((n, n, n), order="F"), np.ones((n, n, n), order="F")


def laplacian_solve_fft(rhs):
    """Exact periodic solution of the 7-point Laplacian (zero mean)."""
    n = rhs.shape[0]
    k = 2 * np.pi * np.fft.fftfreq(n)
    lam = (2 * np.cos(k)[:, None, None] + 2 * np.cos(k)[None, :, None] + 2 * np.cos(k)[None, None, :] - 6)
    R = np.fft.fftn(rhs)
    lam[0, 0, 0] = 1
    U = R / lam
    U[0, 0, 0] = 0
    return np.real(np.fft.ifftn(U))


@pytest.mark.parametrize("n", [8, 16])
def test_flat_metric_is_identity(oracle, n):
    d, r = flat_case(n)
    coef = oracle.metric(d, r, 1.0)
    exp = np.zeros_like(coef)
    exp[..., 0] = exp[..., 3] = exp[..., 5] = 1.0
    assert np.array_equal(coef, exp)


@pytest.mark.parametrize("n,axis", [(16, 0), (16, 1), (32, 2)])
def test_metric_cosine_deformation(oracle, n, axis):
    """def = A cos(2 pi x_a / n): A = I + Hess(def) is diagonal with a known entry."""
    A = 3.0
    x = np.arange(n)
    c = A * np.cos(2 * np.pi * x / n)
    shape = [1, 1, 1]
    shape[axis] = n
    d = np.asfortranarray(np.broadcast_to(c.reshape(shape), (n, n, n)))
    rho = np.ones((n, n, n), order="F")
    coef = oracle.metric(d, rho, 1.0)
    hxx = A * (np.cos(2 * np.pi * (x + 1) / n) - 2 * np.cos(2 * np.pi * x / n) + np.cos(2 * np.pi * (x - 1) / n))
    a = (1 + hxx).reshape(shape)
    a = np.broadcast_to(a, (n, n, n))
    diag_idx = {0: 0, 1: 3, 2: 5}
    for ax in range(3):
        exp = 1 / a if ax == axis else np.ones((n, n, n))
        np.testing.assert_allclose(coef[..., diag_idx[ax]], exp, rtol=1e-13)
    for off in (1, 2, 4):  # cross differences cancel up to rounding
        assert np.abs(coef[..., off]).max() <= 1e-15


@pytest.mark.parametrize("n", [8, 16])
def test_nsmooth_is_separable_filter(oracle, n):
    a = np.asfortranarray(np.random.default_rng(n).standard_normal((n, n, n)))
    exp = a
    for ax in range(3):
        exp = 0.25 * np.roll(exp, 1, ax) + 0.5 * exp + 0.25 * np.roll(exp, -1, ax)
    np.testing.assert_allclose(oracle.nsmooth(a), exp, rtol=0, atol=1e-14)


@pytest.mark.parametrize("n", [8, 16])
def test_restrict_prolong_constants(oracle, n):
    c = np.full((n, n, n), 1.25, order="F")
    assert np.all(oracle.restrict(c) == 1.25)
    u = np.zeros((n, n, n), order="F")
    oracle.prolong_add(u, np.full((n // 2,) * 3, 0.5, order="F"))
    assert np.all(u == 0.5)
    # coincident fine points take the coarse value exactly
    h = np.asfortranarray(np.random.default_rng(1).integers(-8, 8, (n // 2,) * 3).astype(np.float64))
    u = np.zeros((n, n, n), order="F")
    oracle.prolong_add(u, h)
    assert np.array_equal(u[::2, ::2, ::2], h)


def test_fixed_point_sum_exact_and_order_free(oracle):
    rng = np.random.default_rng(5)
    a = rng.standard_normal(100000) * 10.0 ** rng.integers(-6, 6, 100000)
    s1 = oracle.fxsum(a)
    s2 = oracle.fxsum(a[rng.permutation(a.size)])
    assert s1 == s2
    assert abs(s1 - math.fsum(a)) <= 1e-14 * np.abs(a).sum() + a.size * 2.0 ** -64


@pytest.mark.parametrize("n", [8, 16])
def test_zerosum_and_rgzerosum(oracle, n):
    a = np.asfortranarray(np.random.default_rng(n).standard_normal((n, n, n)) + 3.0)
    oracle.zerosum(a)
    assert abs(a.mean()) < 1e-15
    d = smooth_field(n, 0.2, 9)
    b = np.asfortranarray(np.random.default_rng(n + 1).standard_normal((n, n, n)))
    oracle.rgzerosum(b, d, 1.0)
    assert abs(b.sum()) < 1e-11 * n ** 3


@pytest.mark.parametrize("n", [8, 16, 32])
def test_flat_laplacian_solution(oracle, n):
    """def = 0, rho = 1: the operator is the 7-point Laplacian; the converged
    tolerance-schedule solution equals the FFT solution."""
    d, r = flat_case(n)
    rhs = np.asfortranarray(np.random.default_rng(n).standard_normal((n, n, n)))
    rhs -= rhs.mean()
    exact = laplacian_solve_fft(rhs)
    u = np.zeros((n, n, n), order="F")
    rc, diag = oracle.multigrid(u, rhs.copy(order="F"), d, r, 1.0, sched=oracle.SCHED_TOL, tol=1e-12, maxcyc=100)
    assert diag["resid_rel"] <= 1e-12
    np.testing.assert_allclose(u, exact - exact.mean(), rtol=0, atol=1e-10 * np.abs(exact).max())


def test_point_source_problem(oracle):
    """The reference's test3d problem (gauss1.f90:1573-1608): rhs(1,1,1) = n^3,
    zerosum, 4 sweeps; then solved to convergence against the FFT Green's function."""
    n = 16
    d, r = flat_case(n)
    rhs = np.zeros((n, n, n), order="F")
    rhs[0, 0, 0] = n ** 3
    oracle.zerosum(rhs)
    coef = oracle.metric(d, r, 1.0)
    phi = np.zeros((n, n, n), order="F")
    _, rinf4 = oracle.relax(phi, rhs, coef, 1.0, 4, 3)
    assert 0 < rinf4 < n ** 3
    u = np.zeros((n, n, n), order="F")
    rc, diag = oracle.multigrid(u, rhs.copy(order="F"), d, r, 1.0, sched=oracle.SCHED_TOL, tol=1e-12, maxcyc=200)
    exact = laplacian_solve_fft(rhs)
    np.testing.assert_allclose(u, exact - exact.mean(), rtol=0, atol=1e-9 * np.abs(exact).max())


def test_vcycle_reduces_residual(oracle, fields):
    n = 32
    d = smooth_field(n, 0.3, 3)
    rho = fields.lognormal_density(n, sigma=1.0, seed=4)
    rhs = np.asfortranarray(smooth_field(n, 0.01, 5))
    u = np.zeros((n, n, n), order="F")
    r = rhs.copy(order="F")
    rc, diag = oracle.multigrid(u, r, d, rho, 1.0, sched=oracle.SCHED_TOL, tol=1e-10, maxcyc=100)
    assert diag["resid_rel"] <= 1e-10
    assert diag["vcycles"] < 100


@pytest.mark.parametrize("seed", [1, 2])
def test_compression_eigenvalue(oracle, seed):
    """tlim = 3*(1/10 - lambda_min(I + Hess def)) where positive, against eigvalsh."""
    n = 16
    d = smooth_field(n, 3.0, seed)
    dp = np.zeros((n, n, n), order="F")
    lim, mask, diag = oracle.limiter_mask(d, dp)
    r = lambda a, s, ax: np.roll(a, -s, ax)
    hxx = r(d, 1, 0) - 2 * d + r(d, -1, 0)
    hyy = r(d, 1, 1) - 2 * d + r(d, -1, 1)
    hzz = r(d, 1, 2) - 2 * d + r(d, -1, 2)
    hxy = (r(r(d, 1, 0), 1, 1) - r(r(d, -1, 0), 1, 1) - r(r(d, 1, 0), -1, 1) + r(r(d, -1, 0), -1, 1)) / 4
    hyz = (r(r(d, 1, 1), 1, 2) - r(r(d, 1, 1), -1, 2) - r(r(d, -1, 1), 1, 2) + r(r(d, -1, 1), -1, 2)) / 4
    hxz = (r(r(d, 1, 0), 1, 2) - r(r(d, -1, 0), 1, 2) - r(r(d, 1, 0), -1, 2) + r(r(d, -1, 0), -1, 2)) / 4
    C = np.empty((n, n, n, 3, 3))
    C[..., 0, 0], C[..., 1, 1], C[..., 2, 2] = 1 + hxx, 1 + hyy, 1 + hzz
    C[..., 0, 1] = C[..., 1, 0] = hxy
    C[..., 1, 2] = C[..., 2, 1] = hyz
    C[..., 0, 2] = C[..., 2, 0] = hxz
    lmin = np.linalg.eigvalsh(C)[..., 0]
    exp_mask = lmin < 0.1
    clear = np.abs(lmin - 0.1) > 1e-10
    assert exp_mask.sum() > 0
    assert np.array_equal(mask.astype(bool)[clear], exp_mask[clear])
    sel = exp_mask & clear
    np.testing.assert_allclose(lim[sel], 3 * (0.1 - lmin[sel]), rtol=0, atol=1e-10)
    assert diag["ncompress"] == int(mask.sum())


def test_spectral_gradient_sign_and_delta(oracle):
    """scalar2gradient returns -d/dx (NR's exp(+i) forward transform);
    defp2delta returns -Laplacian, both spectrally exact on a sine."""
    n = 16
    x = np.arange(n)
    k = 2 * np.pi / n
    f = np.sin(k * x)
    d = np.asfortranarray(np.broadcast_to(f[:, None, None], (n, n, n)))
    g = oracle.gradient(d)
    np.testing.assert_allclose(g[..., 0], -k * np.cos(k * x)[:, None, None] * np.ones((n, n, n)), atol=1e-13)
    assert np.abs(g[..., 1]).max() < 1e-13 and np.abs(g[..., 2]).max() < 1e-13
    dl = oracle.delta(d)
    np.testing.assert_allclose(dl, k * k * d, atol=1e-13)


def _nr_real_inverse_loop(X):
    """Emulation of the packed-real inverse transform as the reference runs it
    (recipes12.f90:100-132 with isign = -1): the in-place pair loop over
    i1 = 1..n/4+1 and all i2, i3, then an unnormalised exp(-i) complex
    transform of the n/2 x n x n packed array.  X has shape (n/2+1, n, n)."""
    n = X.shape[1]
    M = n // 2
    data = X[:M].copy()           # rdata(i1,i2,i3)
    speq = X[M].copy()            # speq(i2,i3)
    theta = -2 * np.pi / n
    for i3 in range(n):
        j3 = 0 if i3 == 0 else n - i3
        for i1 in range(M // 2 + 1):
            j1 = (M - i1) % M if i1 else 0
            w = np.exp(1j * theta * i1)
            for i2 in range(n):
                j2 = 0 if i2 == 0 else n - i2
                if i1 == 0:
                    h1 = 0.5 * (data[0, i2, i3] + np.conj(speq[j2, j3]))
                    h2 = 0.5j * (data[0, i2, i3] - np.conj(speq[j2, j3]))
                    data[0, i2, i3] = h1 + h2
                    speq[j2, j3] = np.conj(h1 - h2)
                else:
                    h1 = 0.5 * (data[i1, i2, i3] + np.conj(data[j1, j2, j3]))
                    h2 = 0.5j * (data[i1, i2, i3] - np.conj(data[j1, j2, j3]))
                    data[i1, i2, i3] = h1 + w * h2
                    data[j1, j2, j3] = np.conj(h1 - w * h2)
    z = np.fft.fftn(data.transpose(2, 1, 0)).transpose(2, 1, 0)  # exp(-i), unnormalised
    out = np.empty((n, n, n))
    out[0::2] = z.real
    out[1::2] = z.imag
    return out


def test_rlft3_semantics(oracle):
    """Forward transform = exp(+i) spectrum; the inverse of non-Hermitian data
    (as the spectral gradient produces on the Nyquist planes) matches the
    reference's in-place packed algorithm."""
    n = 8
    x = np.asfortranarray(np.random.default_rng(3).standard_normal((n, n, n)))
    X = oracle.rlft3_fwd(x)
    ref = np.conj(np.fft.rfftn(x.transpose(2, 1, 0)).transpose(2, 1, 0))
    np.testing.assert_allclose(X, ref, atol=1e-12)
    np.testing.assert_allclose(oracle.rlft3_inv(X), x * n ** 3 / 2, atol=1e-10)
    Y = np.asfortranarray(np.random.default_rng(4).standard_normal((n // 2 + 1, n, n))
                          + 1j * np.random.default_rng(5).standard_normal((n // 2 + 1, n, n)))
    np.testing.assert_allclose(oracle.rlft3_inv(Y), _nr_real_inverse_loop(Y), atol=1e-10)


@pytest.mark.parametrize("n", [16, 32])
def test_relaxing_conserves_mass(oracle, fields, n):
    d = smooth_field(n, 0.3, 8)
    dp = smooth_field(n, 0.05, 9)
    _, u = fields.initial_state(n, sigma=1.0, seed=10)
    u2 = oracle.relaxing(u, d, dp)
    assert abs(u2[0].sum() - u[0].sum()) <= 1e-12 * u[0].sum()
    assert np.all(u2[1:] == 0)
    assert np.abs(u2[0] - u[0]).max() > 0


def test_float_and_double_agree(oracle, fields):
    n = 16
    d, u = fields.initial_state(n, sigma=1.0, seed=12)
    dp64, _, diag64, _ = oracle.calcdefp(d, u)
    dp32, _, diag32, _ = oracle.calcdefp(d.astype(np.float32), u.astype(np.float32))
    assert np.abs(dp32 - dp64).max() <= 1e-4 * np.abs(dp64).max()
