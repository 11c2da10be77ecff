"""The wavefront schedule of the FP32 strip Gauss-Seidel kernel (k_gs_strip), on the CPU.

A CTA of k_gs_strip owns a 64-cell strip of one plane and LY sub-rows (sub-row r
holds cell rows 2r and 2r+1).  The colours (io, jo) of a plane run in the order
(0,0), (0,1), (1,0), (1,1); at step s colour q updates sub-row s - lag[q],
lag = (0, 2, 3, 5), over the rows and sub-cells that later colours read:
colours (0, *) sub-cells 0..32, (1, *) 0..31; rows Y0-1..Y0+LY+1, Y0-1..Y0+LY,
Y0..Y0+LY and Y0..Y0+LY-1.  Shared memory holds a ring of 8 sub-rows; step s
reads sub-rows s-5..s, stores sub-row s+1 and writes back sub-row s-6.

This test restates that schedule in numpy (each step's updates applied
together, as the GPU runs them between two barriers) and checks:
  * the result equals a plain colour-by-colour half sweep;
  * no update reads a value another update of its step writes;
  * every read finds its sub-row in its ring slot, and no staged sub-row
    overwrites one still in use.
The GPU kernel itself is checked bit for bit against the tile kernel in
tests/test_gpu_mixed_kernels.py.
"""
import numpy as np
import pytest

LAG = (0, 2, 3, 5)
R = 8  # ring slots


def _op(P, Km, Kp, f, k, rhs, y, x, n):
    """19-point update of cell (x, y) of plane k (the reference's operand order)."""
    xp, xm, yp, ym = (x + 1) % n, (x - 1) % n, (y + 1) % n, (y - 1) % n
    kp, km = (k + 1) % n, (k - 1) % n
    b11p = (f[0][k][y, xp] + f[0][k][y, x]) * 0.5
    b11m = (f[0][k][y, xm] + f[0][k][y, x]) * 0.5
    b22p = (f[3][k][yp, x] + f[3][k][y, x]) * 0.5
    b22m = (f[3][k][ym, x] + f[3][k][y, x]) * 0.5
    b33p = (f[5][kp][y, x] + f[5][k][y, x]) * 0.5
    b33m = (f[5][km][y, x] + f[5][k][y, x]) * 0.5
    tdiag = -(b11p + b11m + b22p + b22m + b33p + b33m)
    t1 = b11p * P[y, xp] + b11m * P[y, xm] + b22p * P[yp, x] + b22m * P[ym, x] + b33p * Kp[y, x] + b33m * Km[y, x]
    t2 = ((P[yp, xp] - P[yp, xm]) * f[1][k][yp, x] - (P[ym, xp] - P[ym, xm]) * f[1][k][ym, x]
          + (P[yp, xp] - P[ym, xp]) * f[1][k][y, xp] - (P[yp, xm] - P[ym, xm]) * f[1][k][y, xm]
          + (Kp[yp, x] - Kp[ym, x]) * f[4][kp][y, x] - (Km[yp, x] - Km[ym, x]) * f[4][km][y, x]
          + (Kp[yp, x] - Km[yp, x]) * f[4][k][yp, x] - (Kp[ym, x] - Km[ym, x]) * f[4][k][ym, x]
          + (Kp[y, xp] - Kp[y, xm]) * f[2][kp][y, x] - (Km[y, xp] - Km[y, xm]) * f[2][km][y, x]
          + (Kp[y, xp] - Km[y, xp]) * f[2][k][y, xp] - (Kp[y, xm] - Km[y, xm]) * f[2][k][y, xm]) * 0.25
    return (rhs[k][y, x] - t1 - t2) / tdiag


def _reference_plane(phi, nbr, coef, rhs, k, n):
    P = phi[k].copy()
    for io in (0, 1):
        for jo in (0, 1):
            ys = np.arange(jo, n, 2)[:, None]
            xs = np.arange(io, n, 2)[None, :]
            P[ys, xs] = _op(P, nbr[(k - 1) % n], nbr[(k + 1) % n], coef, k, rhs, ys, xs, n)
    return P


def _strip_plane(phi, nbr, coef, rhs, k, n, LY):
    """All strips and segments of plane k by the wavefront schedule."""
    m = n // 2
    out = np.full((n, n), np.nan)
    for x0 in range(0, n, 64):
        for Y0 in range(0, m, LY):
            P = phi[k].copy()  # this CTA's view: old values, then its own updates
            rlo = (Y0 - 1, Y0 - 1, Y0, Y0)
            rhi = (Y0 + LY + 1, Y0 + LY, Y0 + LY, Y0 + LY - 1)
            owner = {}
            for r in range(Y0 - 2, Y0):
                owner[r % R] = r
            for s in range(Y0 - 1, Y0 + LY + 6):
                writes = []
                for q in range(4):
                    io, jo = q >> 1, q & 1
                    r = s - LAG[q]
                    if not rlo[q] <= r <= rhi[q]:
                        continue
                    for dy in (-1, 0, 1):  # the sub-rows this colour row reads must be in their slots
                        rr = (2 * r + jo + dy) // 2
                        assert owner.get(rr % R) == rr, ("read of a sub-row not in its slot", s, q, rr)
                    y = (2 * r + jo) % n
                    xs = (x0 + 2 * np.arange(33 if io == 0 else 32) + io) % n
                    writes.append((y, xs, _op(P, nbr[(k - 1) % n], nbr[(k + 1) % n], coef, k, rhs, y, xs, n)))
                for y, xs, v in writes:  # the step's updates land together, after its reads
                    P[y, xs] = v
                rb = s - 6
                if Y0 <= rb < Y0 + LY:
                    assert owner.get(rb % R) == rb
                    for jo in (0, 1):
                        out[2 * rb + jo, x0:x0 + 64] = P[2 * rb + jo, x0:x0 + 64]
                if s + 1 <= Y0 + LY + 1:
                    prev = owner.get((s + 1) % R)
                    assert prev is None or prev <= s - 7, ("staging overwrites a sub-row in use", s, prev)
                    owner[(s + 1) % R] = s + 1
    return out


def _same_step_conflicts(LY):
    """Cells one update of a step writes that another update of that step reads."""
    bad = 0
    Y0 = LY
    for s in range(Y0 - 1, Y0 + LY + 6):
        w, rd = {}, {}
        for q in range(4):
            io, jo = q >> 1, q & 1
            r = s - LAG[q]
            lo = Y0 - 1 if q < 2 else Y0
            hi = (Y0 + LY + 1, Y0 + LY, Y0 + LY, Y0 + LY - 1)[q]
            if not lo <= r <= hi:
                continue
            for sx in range(33 if io == 0 else 32):
                y, x = 2 * r + jo, 2 * sx + io
                w[(y, x)] = (q, sx)
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        rd.setdefault((y + dy, x + dx), set()).add((q, sx))
        for cell, upd in w.items():
            bad += len(rd.get(cell, set()) - {upd})
    return bad


@pytest.mark.parametrize("LY", [8, 16, 32, 64])
def test_no_update_reads_what_its_step_writes(LY):
    assert _same_step_conflicts(LY) == 0


@pytest.mark.parametrize("LY", [8, 16])
def test_wavefront_equals_colour_sweep(LY):
    n = 64
    rng = np.random.default_rng(LY)
    phi = rng.standard_normal((n, n, n))
    nbr = rng.standard_normal((n, n, n))
    rhs = rng.standard_normal((n, n, n))
    coef = 1.0 + 0.3 * rng.random((6, n, n, n))
    coef[[1, 2, 4]] *= 0.1
    for k in (0, 1, n - 1):
        a = _reference_plane(phi, nbr, coef, rhs, k, n)
        b = _strip_plane(phi, nbr, coef, rhs, k, n, LY)
        assert np.array_equal(a, b), k
