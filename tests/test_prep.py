"""Input preparation (the step before the path): haloden.f90's particle
density assignment and from1024to512.f90's coarsening.  The oracle
(oracle/prep_oracle.cpp) is checked against a pure-Python restatement on small
hand-built cases, including distance ties, and the GPU against the oracle:
the unnormalised density and the cells per particle bit for bit, the
normalised density within one 4-byte ulp (the oracle sums in sequential
real(8) as the reference does, the GPU exactly)."""
import numpy as np
import pytest


def py_haloden(x, nf, ng):
    """haloden.f90:87-182 in plain Python (small cases only): raw density and wp."""
    f32 = np.float32
    np_ = x.shape[1]
    xp = np.zeros((3, np_), dtype=f32)
    for p in range(np_):
        for a in range(3):
            v = f32(np.fmod(f32(x[a, p]), f32(nf)))
            if v != 0 and (v < 0) != (nf < 0):
                v = f32(v + f32(nf))
            xp[a, p] = f32(f32(v * f32(ng)) / f32(nf))
    cells = {}
    home = []
    for p in range(np_):
        c = tuple(int(np.floor(xp[a, p])) for a in range(3))
        cells.setdefault(c, []).append(p)
        home.append(c)
    wp = [1] * np_
    owner = {}
    h = f32(ng // 2)
    for k in range(ng):
        for j in range(ng):
            for i in range(ng):
                if (i, j, k) in cells:
                    continue
                g = (f32(i + 1) - f32(0.5), f32(j + 1) - f32(0.5), f32(k + 1) - f32(0.5))
                best, r2min, r = None, f32(1000 * ng * ng), 0
                while best is None:
                    r += 1
                    for dk in range(-r, r + 1):
                        for dj in range(-r, r + 1):
                            for di in range(-r, r + 1):
                                c = ((i + di) % ng, (j + dj) % ng, (k + dk) % ng)
                                for p in reversed(cells.get(c, [])):  # linked list: newest first
                                    d = []
                                    for a in range(3):
                                        v = f32(f32(xp[a, p] - g[a]) + h)
                                        m = f32(np.fmod(v, f32(ng)))
                                        if m != 0 and m < 0:
                                            m = f32(m + f32(ng))
                                        d.append(f32(m - h))
                                    r2 = f32(f32(d[0] * d[0]) + f32(d[1] * d[1]))
                                    r2 = f32(r2 + f32(d[2] * d[2]))
                                    if r2 < r2min:
                                        r2min, best = r2, p
                owner[(i, j, k)] = best
                wp[best] += 1
    raw = np.zeros((ng, ng, ng), dtype=f32, order="F")
    for p in range(np_):
        c = home[p]
        raw[c] = f32(raw[c] + f32(f32(1.0) / f32(wp[p])))
    for c, p in owner.items():
        raw[c] = f32(raw[c] + f32(f32(1.0) / f32(wp[p])))
    return raw, np.array(wp, dtype=np.int32)


def clustered(rng, np_, nf, blobs=4, spread=2.0):
    centres = rng.uniform(0, nf, (3, blobs))
    pick = rng.integers(0, blobs, np_)
    return (centres[:, pick] + rng.normal(0, spread, (3, np_))).astype(np.float32)


CASES = {
    # one particle: every cell is its own
    "single": (np.array([[1.3], [2.7], [0.2]], dtype=np.float32), 4, 4),
    # two particles on cell centres: the cells between them are distance ties
    "ties": (np.array([[0.5, 2.5], [0.5, 0.5], [0.5, 0.5]], dtype=np.float32), 4, 4),
    # lattice with a hole, positions outside [0, nf) wrapped
    "lattice": (np.array([[x, y, z] for x in (0.5, 3.5, 5.5) for y in (1.0, 4.0) for z in (-0.5, 6.5)],
                         dtype=np.float32).T, 8, 8),
    # clustered, fine cells twice the grid
    "clustered": (clustered(np.random.default_rng(5), 40, 16, blobs=2, spread=1.5), 16, 8),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_matches_python_restatement(oracle, case):
    x, nf, ng = CASES[case]
    den, raw, wp = oracle.haloden(x, nf, ng)
    raw_py, wp_py = py_haloden(x, nf, ng)
    assert np.array_equal(wp, wp_py)
    assert np.array_equal(raw, raw_py)
    assert raw.min() > 0 and abs(float(raw.sum(dtype=np.float64)) - x.shape[1]) < 1e-5 * x.shape[1]
    assert abs(float(den.mean(dtype=np.float64)) - 1.0) < 1e-6
    if case == "single":
        assert wp[0] == ng ** 3 and np.all(den == 1.0)


def test_oracle_coarsen(oracle):
    rng = np.random.default_rng(9)
    a = rng.uniform(0.1, 3.0, (16, 16, 16)).astype(np.float32)
    a = np.asfortranarray(a)
    c = oracle.coarsen(a, 2)
    blocks = a.reshape(4, 4, 4, 4, 4, 4, order="F").sum(axis=(0, 2, 4), dtype=np.float64)
    ref = blocks / blocks.sum() * 4 ** 3
    assert c.shape == (4, 4, 4)
    np.testing.assert_allclose(c, ref, rtol=3e-7)


def _ulp_diff(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    return int(np.abs(ia - ib).max())


@pytest.mark.gpu
@pytest.mark.parametrize("kind,np_,nf,ng", [("uniform", 3000, 64, 32), ("clustered", 20000, 128, 64),
                                            ("clustered", 4000, 64, 64)] + [(c, 0, 0, 0) for c in sorted(CASES)])
def test_gpu_haloden_matches_oracle(mmh, oracle, kind, np_, nf, ng):
    rng = np.random.default_rng(np_ + ng)
    if kind in CASES:
        x, nf, ng = CASES[kind]
    elif kind == "uniform":
        x = rng.uniform(-nf, 2 * nf, (3, np_)).astype(np.float32)
    else:
        x = clustered(rng, np_, nf, blobs=6, spread=nf / 20)
    den_o, raw_o, wp_o = oracle.haloden(x, nf, ng)
    den_g, raw_g, wp_g = mmh.haloden(x, nf, ng)
    assert np.array_equal(wp_g, wp_o)
    assert np.array_equal(raw_g, raw_o)
    assert _ulp_diff(den_g, den_o) <= 1
    c_o = oracle.coarsen(den_o, 1)
    c_g = mmh.coarsen(den_o, 1)
    assert _ulp_diff(c_g, c_o) <= 1


@pytest.mark.gpu
def test_gpu_haloden_search_radius_cap(mmh):
    """A void whose centre is more than 64 shells (cube shells, the search's
    own radius) from every particle: the search stops at its radius cap and
    the call reports MMH_ERR_RANGE."""
    ng = 144
    c = np.arange(ng, dtype=np.float32) + 0.5
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    cheb = np.maximum(np.maximum(np.abs(X - ng / 2), np.abs(Y - ng / 2)), np.abs(Z - ng / 2))
    keep = cheb > 66.5
    x = np.stack([X[keep], Y[keep], Z[keep]]).astype(np.float32)
    with pytest.raises(mmh.MMHError) as e:
        mmh.haloden(x, ng, ng)
    assert e.value.code == -8  # MMH_ERR_RANGE
