"""Binned power spectra in the bins of the reference's Fisher inputs
(mmh/calcfisherinfo.f90).  The program that wrote those spectrum files is not
in the reference; its bins follow from the bins calcfisherinfo.f90:60 skips
at 128^3 (2, 3, 4, 6, 8, 12 of 48): those are exactly the bins without a mode
when 48 bins are log-spaced in |k| from 1 to n/2 fundamental modes, edges
included below, the edges of bins 4, 8 and 12 falling on |k| = sqrt(2), 2,
sqrt(8).  The GPU spectra are checked against a numpy restatement."""
import numpy as np
import pytest

SKIPPED_AT_128 = {2, 3, 4, 6, 8, 12}  # calcfisherinfo.f90:60, 1-based


def np_edges2(n, nbins):
    """Squared edges (n/2)^(2i/nbins), exact where they are powers of two."""
    m = int(np.log2(n // 2))
    out = []
    for i in range(nbins + 1):
        num = 2 * m * i
        out.append(float(2 ** (num // nbins)) if num % nbins == 0 else 2.0 ** (num / nbins))
    return np.array(out)


def np_spectrum(a, b=None, nbins=48):
    n = a.shape[0]
    A = np.fft.fftn(a)
    P = np.real(A * np.conj(np.fft.fftn(b))) if b is not None else np.abs(A) ** 2
    k = np.fft.fftfreq(n, d=1.0 / n)
    K2 = (k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2).round().astype(np.int64)
    e2 = np_edges2(n, nbins)
    ok = (K2 > 0) & (K2 >= e2[0]) & (K2 < e2[-1])
    idx = np.searchsorted(e2, K2[ok], side="right") - 1
    cnt = np.bincount(idx, minlength=nbins)
    psum = np.bincount(idx, weights=P[ok] / n ** 3, minlength=nbins)
    ksum = np.bincount(idx, weights=np.sqrt(K2[ok]), minlength=nbins)
    with np.errstate(invalid="ignore", divide="ignore"):
        return ksum / cnt, psum / cnt, cnt


def test_bins_reproduce_the_skipped_fisher_bins():
    n = 128
    k = np.fft.fftfreq(n, d=1.0 / n)
    K2 = np.unique((k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2).round().astype(np.int64))
    e2 = np_edges2(n, 48)
    K2 = K2[(K2 > 0) & (K2 < e2[-1])]
    filled = set(np.searchsorted(e2, K2, side="right"))  # 1-based bin of each |k|^2
    assert set(range(1, 49)) - filled == SKIPPED_AT_128


@pytest.mark.gpu
@pytest.mark.parametrize("n", [32, 64, 128])
def test_power_spectrum_matches_numpy(mmh, fields, n):
    rho = fields.lognormal_density(n, sigma=0.7, seed=400 + n)
    other = fields.lognormal_density(n, sigma=0.7, seed=500 + n)
    a = np.asfortranarray(rho - 1.0)
    b = np.asfortranarray(0.5 * (rho - 1.0) + (other - 1.0))
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_REF) as ctx:
        for second in (None, b):
            k, p, m = ctx.power_spectrum(a, second)
            kr, pr, mr = np_spectrum(a, second)
            assert np.array_equal(m, mr)
            full = mr > 0
            np.testing.assert_allclose(k[full], kr[full], rtol=1e-12)  # numpy sums sequentially
            np.testing.assert_allclose(p[full], pr[full], rtol=1e-11, atol=1e-14 * np.abs(pr[full]).max())
            assert np.all(p[~full] == 0)
        if n == 128:
            assert {q + 1 for q in range(48) if m[q] == 0} == SKIPPED_AT_128


def test_spectrum_file_layout(mmh, tmp_path):
    """write_spectrum gives what calcfisherinfo.f90:41-49 reads list-directed
    into tmp(:, 1:2, 1:48): per bin the k then the power, whitespace-separated,
    read back exactly."""
    k = np.logspace(0, np.log10(64), 48)
    p = np.random.default_rng(3).uniform(0, 1e4, 48)
    path = str(tmp_path / "ps48bins_128_2.txt")
    mmh.write_spectrum(path, k, p)
    flat = np.array(open(path).read().split(), dtype=np.float64)
    assert flat.size == 96
    # Fortran column-major fill of a (2, 48) array: k_1, P_1, k_2, P_2, ...
    got = flat.reshape((2, 48), order="F")
    assert np.array_equal(got[0], k) and np.array_equal(got[1], p)
