"""After the path: mmh/column_density.f90 and gridfigure.f90:41-120.  The
oracle (oracle/prep_oracle.cpp) is checked against a known answer (def = 0:
the column is the mean of its planes) and against a plain-Python restatement
that builds gridfigure's node-grid halo literally with CSHIFT (np.roll); the
GPU must equal the oracle bit for bit."""
import numpy as np
import pytest

f32 = np.float32


def _exact_sum(a):
    s = sum(int(np.ldexp(np.float64(x), 64)) for x in a.ravel(order="F"))
    hi, lo = s >> 64, s & ((1 << 64) - 1)
    return np.float64(hi) + np.float64(lo) * np.float64(5.42101086242752217e-20)


def _norm(den):
    ng = den.shape[0]
    sf = f32(_exact_sum(den))
    return (den / sf * f32(ng ** 3)).astype(f32)


def _column(den, i, j, kk1, kk2):
    ng = den.shape[0]
    D = lambda k: den[i - 1, j - 1, (k - 1) % ng]  # noqa: E731
    nk1, nk2 = int(np.floor(kk1)) + 1, int(np.floor(kk2)) + 1
    r1 = f32(f32(nk1) - kk1)
    r2 = f32(f32(kk2 - f32(nk2)) + f32(1))
    s1 = s2 = f32(0)
    for k in range(nk1 + 1, nk2):
        s1 = f32(s1 + D(k))
    for k in range(nk2, nk1 + 1):
        s2 = f32(s2 + D(k))
    t = f32(f32(r1 * D(nk1)) + s1)
    t = f32(t + f32(r2 * D(nk2)))
    return f32(t - s2)


def _faces(dz, i, j, k1, k2, ng):
    jm, im, k1m = (j - 2) % ng + 1, (i - 2) % ng + 1, (k1 - 2) % ng + 1
    a = f32(f32(dz(im, jm, k1m) + dz(i, jm, k1m)) + dz(im, j, k1m))
    a = f32(a + dz(i, j, k1m))
    kk1 = f32(f32(k1 - 1) + f32(a / f32(4)))
    b = f32(f32(dz(im, jm, k2) + dz(i, jm, k2)) + dz(im, j, k2))
    b = f32(b + dz(i, j, k2))
    kk2 = f32(f32(k2) + f32(b / f32(4)))
    return kk1, kk2


def py_column_density(den, d, nplot):
    ng = den.shape[0]
    den = _norm(den)

    def dz(i, j, k):
        F = lambda a, b, c: d[a - 1, b - 1, c - 1]  # noqa: E731
        ip, jp, kp = i % ng + 1, j % ng + 1, k % ng + 1
        v = f32(F(i, j, kp) + F(ip, j, kp))
        for t, sgn in ((F(i, jp, kp), 1), (F(ip, jp, kp), 1), (F(i, j, k), -1), (F(ip, j, k), -1),
                       (F(i, jp, k), -1), (F(ip, jp, k), -1)):
            v = f32(v + t) if sgn > 0 else f32(v - t)
        return f32(v / f32(4))

    k1 = ng // 2
    proj = np.zeros((ng, ng), dtype=f32, order="F")
    for j in range(1, ng + 1):
        for i in range(1, ng + 1):
            kk1, kk2 = _faces(dz, i, j, k1, k1 + nplot - 1, ng)
            proj[i - 1, j - 1] = f32(_column(den, i, j, kk1, kk2) / f32(nplot))
    return proj


def py_gridfigure(d, den):
    nf, ng = d.shape[0], den.shape[0]
    ratio, m = ng // nf, nf + 1
    den = _norm(den)
    td = np.zeros((3, m, m, m), dtype=f32)  # tmp_dsp(3, 0:nf, 0:nf, 0:nf)
    cf = f32(f32(f32(ratio) * f32(1)) / f32(4))
    F = lambda a, b, c: d[a - 1, b - 1, c - 1]  # noqa: E731
    for k in range(1, nf + 1):
        for j in range(1, nf + 1):
            for i in range(1, nf + 1):
                ip, jp, kp = i % nf + 1, j % nf + 1, k % nf + 1
                terms = [
                    [F(ip, j, k), -F(i, j, k), F(ip, jp, k), -F(i, jp, k), F(ip, j, kp), -F(i, j, kp), F(ip, jp, kp),
                     -F(i, jp, kp)],
                    [F(i, jp, k), -F(i, j, k), F(ip, jp, k), -F(ip, j, k), F(i, jp, kp), -F(i, j, kp), F(ip, jp, kp),
                     -F(ip, j, kp)],
                    [F(i, j, kp), -F(i, j, k), F(ip, j, kp), -F(ip, j, k), F(i, jp, kp), -F(i, jp, k), F(ip, jp, kp),
                     -F(ip, jp, k)]]
                for c in range(3):
                    v = f32(terms[c][0] + terms[c][1])
                    for t in terms[c][2:]:
                        v = f32(v + t)
                    td[c, i, j, k] = f32(cf * v)
    tmp = np.roll(np.roll(np.roll(td, 1, 1), 1, 2), 1, 3)  # cshift(..., -1) along dims 2, 3, 4
    td[:, 0, 1:, 1:] = tmp[:, 0, 1:, 1:]
    td[:, 1:, :, 0] = tmp[:, 1:, :, 0]
    td[:, 1:, 0, 1:] = tmp[:, 1:, 0, 1:]

    def disp(c, i, j, k):
        ib, jb, kb = (f32(f32(v % ratio) / f32(ratio)) for v in (i, j, k))
        ip, jp, kp = (int(np.floor(f32(f32(v) / f32(ratio)))) + 1 for v in (i, j, k))
        i1, j1, k1 = (1 if v == nf + 1 else v for v in (ip, jp, kp))
        w = [(ip - 1, jp - 1, kp - 1, ib * jb * kb), (i1, jp - 1, kp - 1, (1 - ib) * jb * kb),
             (ip - 1, j1, kp - 1, ib * (1 - jb) * kb), (ip - 1, jp - 1, k1, ib * jb * (1 - kb)),
             (i1, j1, kp - 1, (1 - ib) * (1 - jb) * kb), (i1, jp - 1, k1, (1 - ib) * jb * (1 - kb)),
             (ip - 1, j1, k1, ib * (1 - jb) * (1 - kb)), (i1, j1, k1, (1 - ib) * (1 - jb) * (1 - kb))]
        s = f32(0)
        for a, b, e, p in w:
            s = f32(s + f32(td[c, a, b, e] * f32(p)))
        return s

    k1 = ng // 2
    proj = np.zeros((ng, ng), dtype=f32, order="F")
    for j in range(1, ng + 1):
        for i in range(1, ng + 1):
            kk1, kk2 = _faces(lambda a, b, e: disp(2, a, b, e), i, j, k1, k1, ng)
            proj[i - 1, j - 1] = _column(den, i, j, kk1, kk2)
    proj2 = np.zeros((2, nf, nf), dtype=f32, order="F")
    for b in range(1, nf + 1):
        for a in range(1, nf + 1):
            idx = (ratio * a, ratio * b, ng // 2)
            for c in range(2):
                proj2[c, a - 1, b - 1] = f32(f32(f32(idx[c]) + f32(0.5)) + disp(c, *idx))
    return proj2, proj


def _fields(seed, ng, nf, amp):
    rng = np.random.default_rng(seed)
    den = rng.uniform(0.2, 3.0, (ng, ng, ng)).astype(f32)
    d = (amp * rng.standard_normal((nf, nf, nf))).astype(f32)
    return np.asfortranarray(den), np.asfortranarray(d)


def test_column_density_known_answer(oracle):
    ng, nplot = 16, 4
    den, _ = _fields(1, ng, ng, 0.0)
    proj = oracle.column_density(den, np.zeros((ng, ng, ng), dtype=f32, order="F"), nplot)
    ref = _norm(den)[:, :, ng // 2 - 1: ng // 2 - 1 + nplot].astype(np.float64).mean(axis=2)
    np.testing.assert_allclose(proj, ref, rtol=2e-6)


@pytest.mark.parametrize("amp", [0.3, 3.0])
def test_column_density_oracle_matches_python(oracle, amp):
    den, d = _fields(2, 8, 8, amp)
    assert np.array_equal(oracle.column_density(den, d, 3), py_column_density(den, d, 3))


@pytest.mark.parametrize("nf,ng,amp", [(4, 8, 0.4), (4, 16, 2.0)])
def test_gridfigure_oracle_matches_python(oracle, nf, ng, amp):
    den, d = _fields(3, ng, nf, amp)
    p2, p = oracle.gridfigure(d, den)
    q2, q = py_gridfigure(d, den)
    assert np.array_equal(p2, q2)
    assert np.array_equal(p, q)


@pytest.mark.gpu
@pytest.mark.parametrize("ng,nf,amp", [(32, 32, 0.5), (64, 64, 4.0), (32, 8, 1.0), (64, 16, 6.0)])
def test_gpu_post_matches_oracle(mmh, oracle, ng, nf, amp):
    den, d = _fields(ng + nf, ng, nf, amp)
    if nf == ng:
        for nplot in (1, 4):
            assert np.array_equal(mmh.column_density(den, d, nplot), oracle.column_density(den, d, nplot))
    p2, p = oracle.gridfigure(d, den)
    g2, g = mmh.gridfigure(d, den)
    assert np.array_equal(g2, p2)
    assert np.array_equal(g, p)
