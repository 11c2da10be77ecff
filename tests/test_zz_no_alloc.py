"""Allocation-free relax (mmh_relax_noalloc_f64) through the C ABI.

The entry point serves callers that cannot let the library allocate device
memory: they pass every input and output in their own device buffers and the
library works in a fixed scratch array it holds for the process lifetime.
This file checks it against the allocating entry point (mmh_relax_f64) on two
calls in a row -- the second call must not see anything the first one left in
the shared scratch -- and that grids above the scratch limit are rejected.
It is collected last so that a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import smooth_field

pytestmark = pytest.mark.gpu


def _case(fields, n, seed):
    rho = fields.lognormal_density(n, sigma=1.0, seed=seed)
    defpot = smooth_field(n, 0.05, seed + 1)
    rng = np.random.default_rng(seed)
    rhs = np.asfortranarray(rng.standard_normal((n, n, n)))
    phi = np.asfortranarray(rng.standard_normal((n, n, n)))
    return defpot, rho, rhs, phi


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to("cuda")


@pytest.mark.parametrize("n,nrelax,iopt", [(16, 4, 18), (64, 3, 18), (64, 2, 16), (32, 5, 18)])
def test_noalloc_matches_allocating_relax(mmh, fields, n, nrelax, iopt):
    torch = pytest.importorskip("torch")
    lib = mmh.lib()
    with mmh.Context(n) as ctx:
        for call in range(2):
            defpot, rho, rhs, phi = _case(fields, n, 100 + 10 * n + call)
            expect = phi.copy(order="F")
            _, rinf_expect = ctx.relax(expect, rhs, defpot, rho, 1.0, nrelax, iopt)
            d_def, d_rho, d_rhs, d_arr = (_dev(torch, a) for a in (defpot, rho, rhs, phi))
            torch.cuda.synchronize()
            rinf = C.c_double(-1.0)
            rc = lib.mmh_relax_noalloc_f64(C.c_void_p(d_def.data_ptr()), C.c_void_p(d_rho.data_ptr()),
                                           C.c_void_p(d_arr.data_ptr()), C.c_void_p(d_rhs.data_ptr()),
                                           C.c_double(1.0), n, nrelax, iopt, C.byref(rinf), None)
            assert rc == 0, mmh.strerror(rc)
            got = d_arr.cpu().numpy().reshape((n, n, n), order="F")
            assert np.array_equal(got, expect)
            assert rinf.value == (rinf_expect if iopt % 8 == 2 else 0.0)


def test_noalloc_rejects_grids_above_its_scratch(mmh):
    torch = pytest.importorskip("torch")
    lib = mmh.lib()
    n = 128
    buf = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    rinf = C.c_double(0.0)
    p = C.c_void_p(buf.data_ptr())
    rc = lib.mmh_relax_noalloc_f64(p, p, p, p, C.c_double(1.0), n, 1, 18, C.byref(rinf), None)
    assert rc == -10
    lib.mmh_strerror.restype = C.c_char_p
    assert b"n <= 64" in lib.mmh_strerror(rc)


@pytest.mark.parametrize("iopt", [274, 19, 17, -2])
def test_noalloc_rejects_what_the_allocating_relax_rejects(mmh, iopt):
    """iresidopt values mmh_relax_f64 refuses (above 256, or a residual mode
    that needs the coarse resid array this entry point does not take) are
    refused here too, before any work."""
    torch = pytest.importorskip("torch")
    lib = mmh.lib()
    n = 16
    buf = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    rinf = C.c_double(0.0)
    p = C.c_void_p(buf.data_ptr())
    rc = lib.mmh_relax_noalloc_f64(p, p, p, p, C.c_double(1.0), n, 1, iopt, C.byref(rinf), None)
    assert rc == -1  # MMH_ERR_ARG
