"""The prolongation's block form, on the CPU.

inject (mgutil.f90:38-71) adds to fine cell (i, j, k) the 8-term average
(H(ibl,jbl,kbl) + H(ibl,jbl,kbh) + H(ibl,jbh,kbl) + H(ibl,jbh,kbh) +
 H(ibh,jbh,kbl) + H(ibh,jbh,kbh) + H(ibh,jbl,kbl) + H(ibh,jbl,kbh)) / 8,
ibl = i/2, ibh = (i+1)/2 wrapped.  The GPU kernel (k_prolong_add_blk) runs one
thread per coarse cell and writes its 2 x 2 x 2 fine block from the 8 coarse
values h[a][b][d] = uh(ci + a x, cj + b y, ck + d z).  This test restates both
forms in numpy and checks that they give the same bits and that every fine cell
is written exactly once.  The GPU kernel is checked bit for bit against the
oracle in the FP64 multigrid tests (tests/test_gpu_parity.py).
"""
import numpy as np
import pytest


def _per_fine_cell(u, uh, n):
    nh = n // 2
    out = u.copy()
    i = np.arange(n)
    lo = i >> 1
    hi = ((i + 1) >> 1) % nh
    for k in range(n):
        for j in range(n):
            H = lambda a, b, c: uh[c, b, a]  # noqa: E731  arrays are [k][j][i]
            out[k, j] = u[k, j] + (H(lo, lo[j], lo[k]) + H(lo, lo[j], hi[k]) + H(lo, hi[j], lo[k])
                                   + H(lo, hi[j], hi[k]) + H(hi, hi[j], lo[k]) + H(hi, hi[j], hi[k])
                                   + H(hi, lo[j], lo[k]) + H(hi, lo[j], hi[k])) * 0.125
    return out


def _per_coarse_cell(u, uh, n):
    nh = n // 2
    out = u.copy()
    written = np.zeros(u.shape, dtype=int)
    for ck in range(nh):
        for cj in range(nh):
            for ci in range(nh):
                ih, jh, kh = (ci, (ci + 1) % nh), (cj, (cj + 1) % nh), (ck, (ck + 1) % nh)
                h = [[[uh[kh[d], jh[b], ih[a]] for d in range(2)] for b in range(2)] for a in range(2)]
                for z in range(2):
                    for y in range(2):
                        k, j, i = 2 * ck + z, 2 * cj + y, 2 * ci
                        out[k, j, i] = out[k, j, i] + (h[0][0][0] + h[0][0][z] + h[0][y][0] + h[0][y][z]
                                                       + h[0][y][0] + h[0][y][z] + h[0][0][0] + h[0][0][z]) * 0.125
                        out[k, j, i + 1] = out[k, j, i + 1] + (h[0][0][0] + h[0][0][z] + h[0][y][0] + h[0][y][z]
                                                               + h[1][y][0] + h[1][y][z] + h[1][0][0]
                                                               + h[1][0][z]) * 0.125
                        written[k, j, i] += 1
                        written[k, j, i + 1] += 1
    assert (written == 1).all()
    return out


@pytest.mark.parametrize("n", [4, 8, 16])
def test_block_prolongation_equals_per_cell(n):
    rng = np.random.default_rng(n)
    u = rng.standard_normal((n, n, n))
    uh = rng.standard_normal((n // 2,) * 3)
    assert np.array_equal(_per_fine_cell(u, uh, n), _per_coarse_cell(u, uh, n))
