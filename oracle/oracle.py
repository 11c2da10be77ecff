"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle (oracle/mmh_oracle.cpp) restates the MMH reconstruction hot path of
pandaPQY/Moving-Mesh-reconstruction loop for loop.  Only the tests, the smoke
check and bench.py's CPU-baseline leg use this module; the product never does.

PARITY UNPINNED: the reference has no golden vectors and cannot be built here
(Fortran, no compiler); the oracle is pinned by analytic known-answer tests.

Arrays follow the Fortran layout: numpy arrays in Fortran order, a[i, j, k]
is the reference's a(i+1, j+1, k+1); u has shape (nf, n, n, n).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmmh_oracle.so")
_lib = None

# reference schedule / PCG to tolerance / repeated V-cycles to tolerance
SCHED_REF = 0
SCHED_TOL = 1
SCHED_VCYCLE = 2


class Diag(C.Structure):
    _fields_ = [
        ("r1", C.c_double), ("relaxerr", C.c_double), ("rhsnorm", C.c_double), ("resid_rel", C.c_double),
        ("vcycles", C.c_int), ("guards", C.c_int), ("bad", C.c_int), ("pad", C.c_int),
        ("nexpand", C.c_longlong), ("ncompress", C.c_longlong),
        ("cmax", C.c_double), ("detmin", C.c_double), ("detmax", C.c_double),
        ("fluxmax", C.c_double), ("fluxmin", C.c_double), ("rho2", C.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


def build():
    """Compile the oracle shared library (make in oracle/)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(_HERE, f) for f in ("mmh_oracle.cpp", "prep_oracle.cpp")]
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(map(os.path.getmtime, srcs)):
            build()
        _lib = C.CDLL(_LIB_PATH)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f(a, dtype):
    a = np.asarray(a)
    if a.dtype != dtype or not a.flags.f_contiguous:
        a = np.asfortranarray(a, dtype=dtype)
    return a


def _sfx(dtype):
    return "d" if np.dtype(dtype) == np.float64 else "f"


def _scalar(dtype, v):
    return C.c_double(v) if np.dtype(dtype) == np.float64 else C.c_float(v)


def threads(t=0):
    return lib().orc_threads(int(t))


def metric(defpot, rho, dx=1.0):
    """rho_bar * cof(A)/det for every cell, shape (6, n, n, n) -- cbajraw."""
    dt = defpot.dtype
    n = defpot.shape[0]
    d = _f(defpot, dt)
    r = _f(rho, dt)
    coef = np.zeros((n, n, n, 6), dtype=dt, order="F")
    getattr(lib(), "orc_metric_" + _sfx(dt))(_p(d), _p(r), n, _scalar(dt, dx), _p(coef))
    return coef


def relax(arr, rhs, coef, dx, nrelax, iopt, colour8=False):
    """relax(arr, resid, rhs, ...): returns (resid_half, rinf); arr updated in place."""
    dt = arr.dtype
    n = arr.shape[0]
    assert arr.flags.f_contiguous
    rhs = _f(rhs, dt)
    resid = np.zeros((n // 2, n // 2, n // 2), dtype=dt, order="F")
    rinf = np.zeros(1, dtype=dt)
    getattr(lib(), "orc_relax_" + _sfx(dt))(_p(arr), _p(resid), _p(rhs), _p(coef), n, _scalar(dt, dx),
                                             int(nrelax), int(iopt), int(colour8), _p(rinf))
    return resid, float(rinf[0])


def residual(phi, rhs, coef, dx=1.0):
    dt = phi.dtype
    n = phi.shape[0]
    r = np.zeros((n, n, n), dtype=dt, order="F")
    getattr(lib(), "orc_residual_" + _sfx(dt))(_p(_f(phi, dt)), _p(_f(rhs, dt)), _p(coef), n, _scalar(dt, dx), _p(r))
    return r


def restrict(fine):
    dt = fine.dtype
    n = fine.shape[0]
    c = np.zeros((n // 2,) * 3, dtype=dt, order="F")
    getattr(lib(), "orc_restrict_" + _sfx(dt))(_p(_f(fine, dt)), n, _p(c))
    return c


def prolong_add(u, uh):
    assert u.flags.f_contiguous
    getattr(lib(), "orc_prolong_add_" + _sfx(u.dtype))(_p(u), _p(_f(uh, u.dtype)), u.shape[0])


def nsmooth(a):
    a = np.array(a, order="F", copy=True)
    getattr(lib(), "orc_nsmooth_" + _sfx(a.dtype))(_p(a), a.shape[0])
    return a


def zerosum(a):
    assert a.flags.f_contiguous
    return getattr(lib(), "orc_zerosum_" + _sfx(a.dtype))(_p(a), a.shape[0])


def rgzerosum(a, defpot, dx=1.0):
    assert a.flags.f_contiguous
    return getattr(lib(), "orc_rgzerosum_" + _sfx(a.dtype))(_p(a), _p(_f(defpot, a.dtype)), a.shape[0],
                                                             _scalar(a.dtype, dx))


def fxsum(a):
    a = np.ascontiguousarray(a)
    fn = getattr(lib(), "orc_fxsum_" + _sfx(a.dtype))
    fn.restype = C.c_double
    return fn(_p(a), C.c_longlong(a.size))


def _flags(sched, colour8, precond_guards):
    """bit 0: 8-colour order; bit 1: no divergence guards (the PCG preconditioner's default)."""
    f = 1 if colour8 else 0
    if sched == SCHED_TOL and not precond_guards:
        f |= 2
    return f


def multigrid(u, rhs, defpot, rho, dx=1.0, sched=SCHED_REF, nu1=2, nu2=2, tol=1e-10, maxcyc=50, colour8=False,
              precond_guards=False):
    """multigrid(u, rhs, defpot, ubig, dx, ...) with iopt=2; u and rhs updated in place."""
    dt = u.dtype
    assert u.flags.f_contiguous and rhs.flags.f_contiguous and rhs.dtype == dt
    d = Diag()
    rc = getattr(lib(), "orc_multigrid_" + _sfx(dt))(
        _p(u), _p(rhs), _p(_f(defpot, dt)), _p(_f(rho, dt)), u.shape[0], _scalar(dt, dx), int(sched), int(nu1),
        int(nu2), C.c_double(tol), int(maxcyc), _flags(sched, colour8, precond_guards), C.byref(d))
    return rc, d.as_dict()


def limiter_pass1(tmp, defpot, u, dtold=1.0, dtaumesh=1.0):
    dt = tmp.dtype
    n = tmp.shape[0]
    tmp = np.array(tmp, order="F", copy=True)
    u = _f(u, dt)
    mx = np.zeros((n, n, n), dtype=np.uint8, order="F")
    mc = np.zeros((n, n, n), dtype=np.uint8, order="F")
    d = Diag()
    getattr(lib(), "orc_limiter_pass1_" + _sfx(dt))(_p(tmp), _p(_f(defpot, dt)), _p(u), u.shape[0], n,
                                                     _scalar(dt, dtold), _scalar(dt, dtaumesh), _p(mx), _p(mc),
                                                     C.byref(d))
    return tmp, mx, mc, d.as_dict()


def limiter_mask(defpot, defp, dtold=1.0):
    dt = defpot.dtype
    n = defpot.shape[0]
    lim = np.zeros((n, n, n), dtype=dt, order="F")
    m = np.zeros((n, n, n), dtype=np.uint8, order="F")
    d = Diag()
    getattr(lib(), "orc_limiter_mask_" + _sfx(dt))(_p(lim), _p(_f(defpot, dt)), _p(_f(defp, dt)), n,
                                                    _scalar(dt, dtold), _p(m), C.byref(d))
    return lim, m, d.as_dict()


def limiter_poisson(defp, defplim):
    defp = np.array(defp, order="F", copy=True)
    getattr(lib(), "orc_limiter_poisson_" + _sfx(defp.dtype))(_p(defp), _p(_f(defplim, defp.dtype)), defp.shape[0])
    return defp


def gradient(defpot):
    """scalar2gradient: shape (n, n, n, 3)."""
    dt = defpot.dtype
    n = defpot.shape[0]
    out = np.zeros((n, n, n, 3), dtype=dt, order="F")
    getattr(lib(), "orc_gradient_" + _sfx(dt))(_p(_f(defpot, dt)), _p(out), n)
    return out


def delta(defpot):
    """defp2delta."""
    dt = defpot.dtype
    n = defpot.shape[0]
    out = np.zeros((n, n, n), dtype=dt, order="F")
    getattr(lib(), "orc_delta_" + _sfx(dt))(_p(_f(defpot, dt)), _p(out), n)
    return out


def relaxing(u, defpot, defp, dt_=1.0):
    """relaxing(u, def, defp, cmax, dt, nfluid): returns the updated u (nf, n, n, n)."""
    dt = defpot.dtype
    u = np.array(u, dtype=dt, order="F", copy=True)
    nf = u.shape[0]
    getattr(lib(), "orc_relaxing_" + _sfx(dt))(_p(u), _p(_f(defpot, dt)), _p(_f(defp, dt)), u.shape[1], nf,
                                                _scalar(dt, dt_))
    return u


def calcdefp(defpot, u, dtold=1.0, dtaumesh=1.0, sched=SCHED_REF, nu1=2, nu2=2, tol=1e-10, maxcyc=50,
             colour8=False, precond_guards=False):
    """calcdefp(defp, tmp, tmp2, def, u, dtold, dtaumesh, nfluid): returns (defp, masks, diag)."""
    dt = defpot.dtype
    n = defpot.shape[0]
    u = _f(u, dt)
    defp = np.zeros((n, n, n), dtype=dt, order="F")
    m = [np.zeros((n, n, n), dtype=np.uint8, order="F") for _ in range(3)]
    d = Diag()
    rc = getattr(lib(), "orc_calcdefp_" + _sfx(dt))(
        _p(defp), _p(_f(defpot, dt)), _p(u), u.shape[0], n, _scalar(dt, dtold), _scalar(dt, dtaumesh), int(sched),
        int(nu1), int(nu2), C.c_double(tol), int(maxcyc), _flags(sched, colour8, precond_guards), _p(m[0]),
        _p(m[1]), _p(m[2]), C.byref(d))
    return defp, {"expand": m[0], "compress1": m[1], "compress2": m[2]}, d.as_dict(), rc


def iteration(defpot, u, sched=SCHED_REF, **kw):
    """One deformation iteration of main.f90:95-101: calcdefp, def += defp, relaxing."""
    defp, masks, diag, rc = calcdefp(defpot, u, sched=sched, **kw)
    defpot = np.asfortranarray(defpot + defp)
    u = relaxing(u, defpot, defp)
    return defpot, u, defp, masks, diag


def rlft3_fwd(x):
    """NR-semantics forward real FFT (exp(+i)): complex array (n/2+1, n, n)."""
    n = x.shape[0]
    x = _f(x, np.float64)
    out = np.zeros((n // 2 + 1, n, n), dtype=np.complex128, order="F")
    lib().orc_rlft3_fwd(_p(x), n, _p(out))
    return out


def rlft3_inv(X):
    """NR-semantics inverse (unnormalised, N^3/2 times the data)."""
    n = X.shape[1]
    X = np.asfortranarray(X, dtype=np.complex128)
    out = np.zeros((n, n, n), dtype=np.float64, order="F")
    lib().orc_rlft3_inv(_p(X), n, _p(out))
    return out


def r1lax_trace(na3, nrelax, iopt):
    cap = 64 * na3 + 64
    buf = (C.c_int * cap)()
    cnt = lib().orc_r1lax_trace(int(na3), int(nrelax), int(iopt), buf, cap)
    return list(buf[:cnt])


def haloden(x, nf, ng):
    """haloden.f90:87-189: x (3, np) float32 positions in fine-cell units.
    Returns (den, raw, wp): the normalised and raw ng^3 densities (Fortran
    order, float32) and the cells per particle."""
    x = np.asarray(x, dtype=np.float32)
    np_ = x.shape[1]
    xc = np.ascontiguousarray(x.T)  # component fastest, as xp(3, np)
    den = np.zeros((ng, ng, ng), dtype=np.float32, order="F")
    raw = np.zeros_like(den, order="F")
    wp = np.zeros(np_, dtype=np.int32)
    L = lib()
    L.orc_haloden.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    rc = L.orc_haloden(_p(xc), np_, nf, ng, _p(den), _p(raw), _p(wp))
    if rc != 0:
        raise ValueError("orc_haloden failed")
    return den, raw, wp


def coarsen(den, ncoarse=1):
    """from1024to512.f90: ncoarse 2x2x2 halvings, normalised to mean 1."""
    den = np.asfortranarray(den, dtype=np.float32)
    ng = den.shape[0]
    nf = ng >> ncoarse
    out = np.zeros((nf, nf, nf), dtype=np.float32, order="F")
    L = lib()
    L.orc_coarsen.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.orc_coarsen(_p(den), ng, ncoarse, _p(out))
    return out


def column_density(den, defpot, nplot=4):
    """mmh/column_density.f90: (ng, ng) column density."""
    den = np.asfortranarray(den, dtype=np.float32)
    defpot = np.asfortranarray(defpot, dtype=np.float32)
    ng = den.shape[0]
    proj = np.zeros((ng, ng), dtype=np.float32, order="F")
    L = lib()
    L.orc_column_density.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.orc_column_density(_p(den), _p(defpot), ng, nplot, _p(proj))
    return proj


def gridfigure(defpot, den):
    """gridfigure.f90:41-120: (proj2 (2, nf, nf), proj (ng, ng))."""
    defpot = np.asfortranarray(defpot, dtype=np.float32)
    den = np.asfortranarray(den, dtype=np.float32)
    nf, ng = defpot.shape[0], den.shape[0]
    proj2 = np.zeros((2, nf, nf), dtype=np.float32, order="F")
    proj = np.zeros((ng, ng), dtype=np.float32, order="F")
    L = lib()
    L.orc_gridfigure.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.orc_gridfigure(_p(defpot), nf, _p(den), ng, _p(proj2), _p(proj))
    return proj2, proj
