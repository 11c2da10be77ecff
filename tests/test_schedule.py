"""The reference's plane schedule (r1lax, mmh/gauss1.f90:208-499) and the
8-colour order the GPU executes (no GPU needed).

The literal schedule relaxes planes in a pyramid/wavefront order.  Tracking
read/write conflicts shows that its dependency levels are exactly nrelax
repetitions of (all odd planes, all even planes), that every residual is
taken after the last relaxation of the planes it reads, and that the
full-weighting accumulation adds the lower-plane part first for every coarse
plane except plane nrelax+1.  These tests check those facts and that both
orders give bit-identical results in the oracle.
"""
import numpy as np
import pytest

from conftest import smooth_field


def levels(trace, na3):
    nb = lambda p, d: (p - 1 + d) % na3 + 1
    last_w, last_r, last_c, out = {}, {}, {}, []
    for op in trace:
        if op > 0:
            reads, writes, cw = {nb(op, -1), op, nb(op, 1)}, {op}, set()
        else:
            ki = -op
            reads = {nb(ki - 1, d) for d in (-1, 0, 1)} | {nb(ki, d) for d in (-1, 0, 1)}
            writes, cw = set(), set()
        lv = max([last_w.get(p, 0) for p in reads] + [max(last_w.get(p, 0), last_r.get(p, 0)) for p in writes] + [0])
        lv += 1
        for p in reads:
            last_r[p] = max(last_r.get(p, 0), lv)
        for p in writes:
            last_w[p] = lv
        out.append((op, lv))
    return out


@pytest.mark.parametrize("na3,nrelax", [(4, 1), (8, 2), (16, 3), (16, 4), (32, 4), (64, 2), (256, 4)])
def test_schedule_is_odd_even_planes(oracle, na3, nrelax):
    tr = oracle.r1lax_trace(na3, nrelax, 0)
    assert sorted(tr) == sorted(list(range(1, na3 + 1)) * nrelax)
    lv = levels(tr, na3)
    by = {}
    for op, l in lv:
        by.setdefault(l, set()).add(op)
    assert len(by) == 2 * nrelax
    for l, planes in by.items():
        parity = 1 if l % 2 == 1 else 0  # odd levels: odd (1-based) planes
        assert planes == {p for p in range(1, na3 + 1) if p % 2 == parity}


@pytest.mark.parametrize("na3,nrelax", [(8, 1), (8, 2), (16, 3), (32, 4), (128, 4)])
def test_residuals_after_final_relaxation(oracle, na3, nrelax):
    tr = oracle.r1lax_trace(na3, nrelax, 3)
    nb = lambda p, d: (p - 1 + d) % na3 + 1
    crs = [i for i, op in enumerate(tr) if op < 0]
    assert sorted(-tr[i] for i in crs) == list(range(2, na3 + 1, 2))
    for i in crs:
        ki = -tr[i]
        reads = {nb(ki - 1, d) for d in (-1, 0, 1)} | {nb(ki, d) for d in (-1, 0, 1)}
        assert not [op for op in tr[i + 1:] if op > 0 and op in reads]
    # accumulation order: own-plane part first only for coarse plane nrelax+1
    nc = na3 // 2
    first = {}
    for i in crs:
        ki = -tr[i]
        first.setdefault(ki // 2, "own")
        first.setdefault(ki // 2 % nc + 1, "lower")
    assert [c for c, f in first.items() if f == "own"] == [nrelax + 1]


@pytest.mark.parametrize("n,nrelax,iopt", [(8, 2, 19), (16, 3, 19), (32, 4, 19), (16, 8, 19), (16, 0, 19)])
def test_literal_and_colour8_bit_identical(oracle, fields, n, nrelax, iopt):
    d = smooth_field(n, 0.1, n)
    rho = fields.lognormal_density(n, sigma=1.0, seed=n + 1)
    coef = oracle.metric(d, rho, 1.0)
    rng = np.random.default_rng(nrelax)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi = np.asfortranarray(rng.standard_normal((n, n, n)))
    a, b = phi.copy(order="F"), phi.copy(order="F")
    ra, ia = oracle.relax(a, rhs, coef, 1.0, nrelax, iopt, colour8=False)
    rb, ib = oracle.relax(b, rhs, coef, 1.0, nrelax, iopt, colour8=True)
    assert np.array_equal(a, b) and np.array_equal(ra, rb) and ia == ib


@pytest.mark.parametrize("n", [16, 32])
def test_multigrid_literal_and_colour8(oracle, fields, n):
    d = smooth_field(n, 0.1, 2)
    rho = fields.lognormal_density(n, sigma=1.5, seed=3)
    rhs = np.asfortranarray(smooth_field(n, 0.01, 4))
    out = []
    for c8 in (False, True):
        u = np.zeros((n, n, n), order="F")
        oracle.multigrid(u, rhs.copy(order="F"), d, rho, 1.0, sched=oracle.SCHED_REF, colour8=c8)
        out.append(u)
    assert np.array_equal(out[0], out[1])
