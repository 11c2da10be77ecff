"""Python mirror of the reference's Fortran interface for the MMH hot path.

Each function keeps the name, argument order and meaning of the Fortran
subroutine it replaces (mmh/limiter.f90 calcdefp, mmh/multigrid.f90 multigrid,
mmh/relaxing.f90 relaxing, mmh/gradient.f90 scalar2gradient,
mmh/reconstruct.f90 defp2delta, mmh/gauss1.f90 relax/zerosum/rgzerosum,
mmh/mgutil.f90 restrict/inject) and calls the CUDA library through its C ABI
(include/mmh.h).  Arrays are numpy arrays in Fortran order; the Fortran
convention of updating arguments in place is kept.  Where the Fortran stops
the program (write + stop/pause), these functions raise MMHError.

There is no CPU fallback: the library must be built (build.py) and a CUDA
device must be present, otherwise loading fails loudly.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmmh_gb300.so")

MMH_FP64 = 0
MMH_MIXED = 1
MMH_SCHED_REF = 0
MMH_SCHED_TOL = 1      # flexible CG, one V-cycle per iteration as preconditioner
MMH_SCHED_VCYCLE = 2   # plain repeated V-cycles

MMH_OK = 0
MMH_ERR_NAN = -5
MMH_ERR_DIVERGED = -6
MMH_ERR_UNSUPPORTED = -7
MMH_ERR_RANGE = -8

# every entry point of include/mmh.h
EXPORTS = (
    "mmh_config_default", "mmh_create", "mmh_destroy", "mmh_strerror", "mmh_sync", "mmh_launch_count",
    "mmh_calcdefp", "mmh_calcdefp_f64", "mmh_multigrid", "mmh_multigrid_f64", "mmh_relaxing", "mmh_relaxing_f64",
    "mmh_scalar2gradient", "mmh_scalar2gradient_f64", "mmh_defp2delta", "mmh_defp2delta_f64",
    "mmh_relax_f64", "mmh_metric_f64", "mmh_metric_ff_f64", "mmh_restrict_f64", "mmh_inject_f64", "mmh_zerosum_f64",
    "mmh_rgzerosum_f64", "mmh_nsmooth_f64", "mmh_limiter_pass1_f64", "mmh_limiter_mask_f64",
    "mmh_limiter_poisson_f64", "mmh_load_f64", "mmh_load_dev", "mmh_iterate", "mmh_store_f64",
    "mmh_outputs_f64", "mmh_outputs_dev", "mmh_state_dev", "mmh_profile_start", "mmh_profile_stop",
    "mmh_relax_noalloc_f64", "mmh_batch_run", "mmh_calcdefp_adjoint_f64",
    "mmh_relaxing_adjoint_f64", "mmh_iterate_adjoint_f64", "mmh_state_stats",
    "mmh_power_spectrum_f64", "mmh_haloden", "mmh_coarsen",
    "mmh_column_density", "mmh_gridfigure", "mmh_keep_masks", "mmh_masks", "mmh_gs_tile_pin", "mmh_gs_tile", "mmh_stencil_pin",
)

# kernel kinds for the timing hooks
K_GS, K_RESIDUAL, K_RESTRICT_RESID, K_METRIC, K_SMOOTH, K_PROLONG, K_RESTRICT = 1, 2, 3, 4, 5, 6, 7
K_F32 = 256


def K_AT(n):
    """Grid filter for profile_start: time only the launches on the n^3 level."""
    return int(n) << 12


def write_spectrum(path, k, p):
    """One bin per line, "k P(k)": the layout calcfisherinfo.f90:41-49 reads
    (list-directed, tmp(:, 1, bin) = k, tmp(:, 2, bin) = P)."""
    with open(path, "w") as f:
        for kv, pv in zip(k, p):
            f.write(f"{kv:.16e} {pv:.16e}\n")


def haloden(x, nf, ng):
    """Particle density assignment (haloden.f90) on the GPU: x (3, np) float32
    positions in fine-cell units.  Returns (den, raw, wp)."""
    xc = np.ascontiguousarray(np.asarray(x, dtype=np.float32).T)  # component fastest
    np_ = xc.shape[0]
    den = np.zeros((ng, ng, ng), dtype=np.float32, order="F")
    raw = np.zeros_like(den, order="F")
    wp = np.zeros(np_, dtype=np.int32)
    L = lib()
    L.mmh_haloden.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    _chk(L.mmh_haloden(_p(xc), np_, int(nf), int(ng), _p(den), _p(raw), _p(wp)), "haloden")
    return den, raw, wp


def coarsen(den, ncoarse=1):
    """from1024to512.f90's coarsening on the GPU: ncoarse 2x2x2 halvings, mean 1."""
    den = np.asfortranarray(den, dtype=np.float32)
    ng = den.shape[0]
    nc = ng >> ncoarse
    out = np.zeros((nc, nc, nc), dtype=np.float32, order="F")
    _chk(lib().mmh_coarsen(_p(den), int(ng), int(ncoarse), _p(out)), "coarsen")
    return out


def column_density(den, defpot, nplot=4):
    """mmh/column_density.f90 on the GPU: (ng, ng) column density."""
    den = np.asfortranarray(den, dtype=np.float32)
    defpot = np.asfortranarray(defpot, dtype=np.float32)
    ng = den.shape[0]
    proj = np.zeros((ng, ng), dtype=np.float32, order="F")
    _chk(lib().mmh_column_density(_p(den), _p(defpot), int(ng), int(nplot), _p(proj)), "column_density")
    return proj


def gridfigure(defpot, den):
    """gridfigure.f90:41-120 on the GPU: (proj2 (2, nf, nf), proj (ng, ng))."""
    defpot = np.asfortranarray(defpot, dtype=np.float32)
    den = np.asfortranarray(den, dtype=np.float32)
    nf, ng = defpot.shape[0], den.shape[0]
    proj2 = np.zeros((2, nf, nf), dtype=np.float32, order="F")
    proj = np.zeros((ng, ng), dtype=np.float32, order="F")
    _chk(lib().mmh_gridfigure(_p(defpot), int(nf), _p(den), int(ng), _p(proj2), _p(proj)), "gridfigure")
    return proj2, proj


class MMHError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__(f"{what}: {strerror(code)} ({code})" if what else f"{strerror(code)} ({code})")


class Stats(C.Structure):
    _fields_ = [("def_mean", C.c_double), ("def_sigma", C.c_double), ("defp_sigma", C.c_double),
                ("rho_mean", C.c_double), ("rho_sigma", C.c_double), ("rho_min", C.c_double),
                ("rho_max", C.c_double), ("rho_negative", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Config(C.Structure):
    _fields_ = [("n", C.c_int), ("precision", C.c_int), ("schedule", C.c_int), ("nu1", C.c_int), ("nu2", C.c_int),
                ("max_cycles", C.c_int), ("tol", C.c_double), ("device", C.c_int), ("stream", C.c_void_p),
                ("precond_guards", C.c_int)]


class Diag(C.Structure):
    _fields_ = [
        ("r1", C.c_double), ("relaxerr", C.c_double), ("rhsnorm", C.c_double), ("resid_rel", C.c_double),
        ("vcycles", C.c_int), ("guards", C.c_int), ("status", C.c_int), ("pad", C.c_int),
        ("nexpand", C.c_longlong), ("ncompress", C.c_longlong),
        ("cmax", C.c_double), ("detmin", C.c_double), ("detmax", C.c_double),
        ("fluxmax", C.c_double), ("fluxmin", C.c_double), ("rho2", C.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class Problem(C.Structure):
    _fields_ = [("n", C.c_int), ("niter", C.c_int), ("rho", C.c_void_p), ("def_", C.c_void_p),
                ("grad", C.c_void_p), ("delta", C.c_void_p), ("status", C.c_int), ("vcycles", C.c_int)]


_lib = None


def lib():
    """Load libmmh_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"libmmh_gb300.so not built ({LIB_PATH}); run build.py / __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        L.mmh_strerror.restype = C.c_char_p
        L.mmh_launch_count.restype = C.c_ulonglong
        _lib = L
    return _lib


def strerror(code):
    try:
        return lib().mmh_strerror(int(code)).decode()
    except OSError:
        return f"error {code}"


def launch_count():
    return int(lib().mmh_launch_count())


def gs_tile_pin(shape):
    """Pin the FP32 plane Gauss-Seidel tile shape (0..3: tiles; 4..5: strips
    marching in y) for every grid; -1 returns to timing the shapes per grid
    size."""
    _chk(lib().mmh_gs_tile_pin(int(shape)), "gs_tile_pin")


def stencil_pin(kind):
    """FP32 residual/operator stencil: -1 default (marching from 64^3 up), 0
    one plane per CTA, 1 marching."""
    _chk(lib().mmh_stencil_pin(int(kind)), "stencil_pin")


def gs_tile(n):
    """(TX, TY) of the FP32 plane Gauss-Seidel tile in use for grid n, or None."""
    tx, ty = C.c_int(), C.c_int()
    return (tx.value, ty.value) if lib().mmh_gs_tile(int(n), C.byref(tx), C.byref(ty)) == MMH_OK else None


def profile_start(kind):
    """Arm CUDA-event timing of every launch of one kernel kind."""
    _chk(lib().mmh_profile_start(int(kind)), "profile_start")


def profile_stop():
    """Returns (launches, total device ms, cells processed) since profile_start."""
    n, ms, cells = C.c_int(), C.c_double(), C.c_longlong()
    _chk(lib().mmh_profile_stop(C.byref(n), C.byref(ms), C.byref(cells)), "profile_stop")
    return n.value, ms.value, cells.value


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _chk(rc, what, allow_diverged=False):
    if rc != MMH_OK and not (allow_diverged and rc == MMH_ERR_DIVERGED):
        raise MMHError(rc, what)
    return rc


def _farr(a, dtype):
    if not (isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.f_contiguous):
        raise TypeError(f"expected a Fortran-ordered {np.dtype(dtype).name} array")
    return a


def _sfx(dtype):
    return "_f64" if np.dtype(dtype) == np.float64 else ""


def _sc(dtype, v):
    return C.c_double(v) if np.dtype(dtype) == np.float64 else C.c_float(v)


class Context:
    """Device state for one grid size NG (the Fortran's compile-time NG)."""

    def __init__(self, n, precision=MMH_FP64, schedule=MMH_SCHED_REF, nu1=2, nu2=2, tol=1e-10, max_cycles=200,
                 device=0, stream=None, precond_guards=False):
        L = lib()
        cfg = Config()
        L.mmh_config_default(C.byref(cfg), int(n))
        cfg.precision, cfg.schedule = int(precision), int(schedule)
        cfg.nu1, cfg.nu2, cfg.tol, cfg.max_cycles, cfg.device = int(nu1), int(nu2), float(tol), int(max_cycles), int(device)
        cfg.stream = stream
        cfg.precond_guards = int(bool(precond_guards))
        self.cfg = cfg
        self.n = int(n)
        self._h = C.c_void_p()
        _chk(L.mmh_create(C.byref(self._h), C.byref(cfg)), "mmh_create")

    def close(self):
        if self._h:
            lib().mmh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # ---- drop-ins ---------------------------------------------------------
    def calcdefp(self, defp, tmp, tmp2, defpot, u, dtold1=1.0, dtaumesh=1.0, nfluid=5):
        """calcdefp(defp,tmp,tmp2,def,u,dtold1,dtaumesh,nfluid)  (mmh/limiter.f90:17)."""
        dt = defp.dtype
        for a in (defp, defpot, u):
            _farr(a, dt)
        d = Diag()
        fn = getattr(lib(), "mmh_calcdefp" + _sfx(dt))
        rc = fn(self._h, _p(defp), _p(tmp), _p(tmp2), _p(defpot), _p(u), _sc(dt, dtold1), _sc(dt, dtaumesh),
                int(nfluid), C.byref(d))
        _chk(rc, "calcdefp", allow_diverged=True)
        return d.as_dict()

    def calcdefp_adjoint(self, defpot, u, w, dtold1=1.0, dtaumesh=1.0, nfluid=5):
        """Gradients of sum(w * defp) with respect to the density and to defpot
        for the defp that calcdefp(..., defpot, u, dtold1, dtaumesh, nfluid)
        computes, with the limiter branches frozen.  Returns (grho, gdef, diag)."""
        for a in (defpot, u, w):
            _farr(a, np.float64)
        grho = np.zeros(defpot.shape, dtype=np.float64, order="F")
        gdef = np.zeros(defpot.shape, dtype=np.float64, order="F")
        d = Diag()
        _chk(lib().mmh_calcdefp_adjoint_f64(self._h, _p(defpot), _p(u), int(nfluid), C.c_double(dtold1),
                                            C.c_double(dtaumesh), _p(w), _p(grho), _p(gdef), C.byref(d)),
             "calcdefp_adjoint")
        return grho, gdef, d.as_dict()

    def relaxing_adjoint(self, u, defpot, defp, w, dt=1.0, nfluidcmp=5):
        """Gradients of sum(w * u'[density]) for u' = relaxing(u, defpot, defp,
        dt) with the minmod slopes frozen.  Returns (gu, gdef, gdefp)."""
        for a in (u, defpot, defp, w):
            _farr(a, np.float64)
        g = [np.zeros(defpot.shape, dtype=np.float64, order="F") for _ in range(3)]
        _chk(lib().mmh_relaxing_adjoint_f64(self._h, _p(u), _p(defpot), _p(defp), C.c_double(dt), int(nfluidcmp),
                                            _p(w), _p(g[0]), _p(g[1]), _p(g[2])), "relaxing_adjoint")
        return tuple(g)

    def iterate_adjoint(self, niter, wdef=None, wdelta=None, checkpoint_every=4):
        """niter iterations from the loaded state, then the gradients of
        sum(wdef * def_N) + sum(wdelta * defp2delta(def_N)) with respect to the
        loaded density and def.  Returns (grho, gdef, diag)."""
        for a in (wdef, wdelta):
            if a is not None:
                _farr(a, np.float64)
        shape = (self.n,) * 3
        grho = np.zeros(shape, dtype=np.float64, order="F")
        gdef = np.zeros(shape, dtype=np.float64, order="F")
        d = Diag()
        _chk(lib().mmh_iterate_adjoint_f64(self._h, int(niter), int(checkpoint_every), _p(wdef), _p(wdelta),
                                           _p(grho), _p(gdef), C.byref(d)), "iterate_adjoint")
        return grho, gdef, d.as_dict()

    def multigrid(self, u, rhs, defpot, ubig, dx, nx, ny, nz, nu, nred=1, iopt=2):
        """multigrid(u,rhs,defpot,ubig,dx,nx,ny,nz,nu,nred,iopt)  (mmh/multigrid.f90:16)."""
        dt = u.dtype
        for a in (u, rhs, defpot, ubig):
            _farr(a, dt)
        d = Diag()
        fn = getattr(lib(), "mmh_multigrid" + _sfx(dt))
        rc = fn(self._h, _p(u), _p(rhs), _p(defpot), _p(ubig), _sc(dt, dx), int(nx), int(ny), int(nz), int(nu),
                int(nred), int(iopt), C.byref(d))
        _chk(rc, "multigrid", allow_diverged=True)
        return d.as_dict()

    def relaxing(self, u, defpot, defp, cmax=1.0, dt=1.0, nfluidcmp=5):
        """relaxing(u,def,defp,cmax,dt,nfluidcmp)  (mmh/relaxing.f90:21)."""
        ty = u.dtype
        for a in (u, defpot, defp):
            _farr(a, ty)
        fn = getattr(lib(), "mmh_relaxing" + _sfx(ty))
        _chk(fn(self._h, _p(u), _p(defpot), _p(defp), _sc(ty, cmax), _sc(ty, dt), int(nfluidcmp)), "relaxing")

    def scalar2gradient(self, indata, outdata, nn):
        """scalar2gradient(indata,outdata,nn)  (mmh/gradient.f90:1)."""
        dt = indata.dtype
        _farr(indata, dt), _farr(outdata, dt)
        nn = (C.c_int * 3)(*[int(x) for x in nn])
        fn = getattr(lib(), "mmh_scalar2gradient" + _sfx(dt))
        _chk(fn(self._h, _p(indata), _p(outdata), nn), "scalar2gradient")

    def defp2delta(self, indata, outdata, nn):
        """defp2delta(indata,outdata,nn)  (mmh/reconstruct.f90:1)."""
        dt = indata.dtype
        _farr(indata, dt), _farr(outdata, dt)
        nn = (C.c_int * 3)(*[int(x) for x in nn])
        fn = getattr(lib(), "mmh_defp2delta" + _sfx(dt))
        _chk(fn(self._h, _p(indata), _p(outdata), nn), "defp2delta")

    # ---- reference subroutines on the path (FP64) -------------------------
    def relax(self, arr, rhs, deformpot, rho, dx, nrelax, iopt):
        """relax(arr,resid,rhs,deformpot,u,rinf,dx,n,n,n,1,nrelax,iopt): returns (resid, rinf)."""
        n = arr.shape[0]
        for a in (arr, rhs, deformpot, rho):
            _farr(a, np.float64)
        resid = np.zeros((n // 2,) * 3, dtype=np.float64, order="F")
        rinf = C.c_double(0)
        _chk(lib().mmh_relax_f64(self._h, _p(arr), _p(resid), _p(rhs), _p(deformpot), _p(rho), C.byref(rinf),
                                 C.c_double(dx), n, int(nrelax), int(iopt)), "relax")
        return resid, rinf.value

    def metric(self, deformpot, rho, dx=1.0):
        n = deformpot.shape[0]
        coef = np.zeros((n, n, n, 6), dtype=np.float64, order="F")
        _chk(lib().mmh_metric_f64(self._h, _p(_farr(deformpot, np.float64)), _p(_farr(rho, np.float64)),
                                  C.c_double(dx), n, _p(coef)), "metric")
        return coef

    def metric_ff(self, deformpot, rho, dx=1.0):
        """The mixed form's float-float metric (mmh_metric_ff_f64): (coef, det)."""
        n = deformpot.shape[0]
        coef = np.zeros((n, n, n, 6), dtype=np.float64, order="F")
        det = np.zeros((n, n, n), dtype=np.float64, order="F")
        _chk(lib().mmh_metric_ff_f64(self._h, _p(_farr(deformpot, np.float64)), _p(_farr(rho, np.float64)),
                                     C.c_double(dx), n, _p(coef), _p(det)), "metric_ff")
        return coef, det

    def restrict(self, u):
        n = u.shape[0]
        uh = np.zeros((n // 2,) * 3, dtype=np.float64, order="F")
        _chk(lib().mmh_restrict_f64(self._h, _p(_farr(u, np.float64)), n, _p(uh)), "restrict")
        return uh

    def inject(self, u, uhalf):
        _chk(lib().mmh_inject_f64(self._h, _p(_farr(u, np.float64)), _p(_farr(uhalf, np.float64)), u.shape[0]),
             "inject")

    def zerosum(self, arr):
        _chk(lib().mmh_zerosum_f64(self._h, _p(_farr(arr, np.float64)), arr.shape[0]), "zerosum")

    def rgzerosum(self, arr, defpot, dx=1.0):
        _chk(lib().mmh_rgzerosum_f64(self._h, _p(_farr(arr, np.float64)), _p(_farr(defpot, np.float64)),
                                     C.c_double(dx), arr.shape[0]), "rgzerosum")

    def nsmooth(self, a):
        _chk(lib().mmh_nsmooth_f64(self._h, _p(_farr(a, np.float64)), a.shape[0]), "nsmooth")

    def limiter_pass1(self, tmp, defpot, rho, dtold=1.0, dtaumesh=1.0):
        n = tmp.shape[0]
        mx = np.zeros((n, n, n), dtype=np.uint8, order="F")
        mc = np.zeros((n, n, n), dtype=np.uint8, order="F")
        d = Diag()
        _chk(lib().mmh_limiter_pass1_f64(self._h, _p(_farr(tmp, np.float64)), _p(_farr(defpot, np.float64)),
                                         _p(_farr(rho, np.float64)), n, C.c_double(dtold), C.c_double(dtaumesh),
                                         _p(mx), _p(mc), C.byref(d)), "limiter_pass1")
        return mx, mc, d.as_dict()

    def limiter_mask(self, defpot, defp, dtold=1.0):
        n = defpot.shape[0]
        lim = np.zeros((n, n, n), dtype=np.float64, order="F")
        m = np.zeros((n, n, n), dtype=np.uint8, order="F")
        d = Diag()
        _chk(lib().mmh_limiter_mask_f64(self._h, _p(lim), _p(_farr(defpot, np.float64)), _p(_farr(defp, np.float64)),
                                        n, C.c_double(dtold), _p(m), C.byref(d)), "limiter_mask")
        return lim, m, d.as_dict()

    def limiter_poisson(self, defp, defplim):
        _chk(lib().mmh_limiter_poisson_f64(self._h, _p(_farr(defp, np.float64)), _p(_farr(defplim, np.float64)),
                                           defp.shape[0]), "limiter_poisson")

    # ---- device-resident reconstruction ----------------------------------
    def load(self, defpot, u):
        u = _farr(u, np.float64)
        _chk(lib().mmh_load_f64(self._h, _p(defpot), _p(u), u.shape[0]), "load")

    def load_dev(self, d_def, d_rho):
        _chk(lib().mmh_load_dev(self._h, C.c_void_p(d_def) if d_def else None, C.c_void_p(d_rho)), "load_dev")

    def iterate(self, niter=1):
        d = Diag()
        _chk(lib().mmh_iterate(self._h, int(niter), C.byref(d)), "iterate", allow_diverged=True)
        return d.as_dict()

    def power_spectrum(self, a, b=None, nbins=48):
        """Binned (cross) power spectrum of n^3 fields (mmh_power_spectrum_f64):
        returns (kmean in fundamental units, power, modes) per bin."""
        for x in (a, b):
            if x is not None:
                _farr(x, np.float64)
        k = np.zeros(nbins)
        p = np.zeros(nbins)
        m = np.zeros(nbins, dtype=np.int64)
        _chk(lib().mmh_power_spectrum_f64(self._h, _p(a), _p(b), int(nbins), _p(k), _p(p), _p(m)), "power_spectrum")
        return k, p, m

    def keep_masks(self, on=True):
        """Arm (or disarm) keeping the limiter masks of every calcdefp."""
        _chk(lib().mmh_keep_masks(self._h, int(bool(on))), "keep_masks")

    def masks(self):
        """Limiter masks of the last calcdefp: dict of expand, compress1,
        compress2 (uint8, Fortran order), as the oracle's calcdefp returns them."""
        shape = (self.n,) * 3
        m = [np.zeros(shape, dtype=np.uint8, order="F") for _ in range(3)]
        _chk(lib().mmh_masks(self._h, _p(m[0]), _p(m[1]), _p(m[2])), "masks")
        return {"expand": m[0], "compress1": m[1], "compress2": m[2]}

    def stats(self):
        """main.f90's iteration diagnostics of the resident state (mmh_state_stats)."""
        st = Stats()
        _chk(lib().mmh_state_stats(self._h, C.byref(st)), "state_stats")
        return st.as_dict()

    def store(self, defpot=None, u=None):
        nf = u.shape[0] if u is not None else 5
        _chk(lib().mmh_store_f64(self._h, _p(defpot), _p(u), nf), "store")

    def outputs(self, grad=None, delta=None):
        _chk(lib().mmh_outputs_f64(self._h, _p(grad), _p(delta)), "outputs")

    def outputs_dev(self, d_grad, d_delta):
        """Spectral outputs into device buffers (integer device addresses)."""
        _chk(lib().mmh_outputs_dev(self._h, C.c_void_p(d_grad) if d_grad else None,
                                   C.c_void_p(d_delta) if d_delta else None), "outputs_dev")

    def state_dev(self):
        a, b, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _chk(lib().mmh_state_dev(self._h, C.byref(a), C.byref(b), C.byref(c)), "state_dev")
        return a.value, b.value, c.value

    def sync(self):
        _chk(lib().mmh_sync(self._h), "sync")


def reconstruct(rho, niter, precision=MMH_FP64, schedule=MMH_SCHED_REF, tol=1e-10, outputs=True, **kw):
    """mmh/main.f90:83-179 on one density field: niter deformation iterations
    from def = 0, then the spectral displacement and density outputs."""
    n = rho.shape[0]
    with Context(n, precision=precision, schedule=schedule, tol=tol, **kw) as ctx:
        u = np.zeros((5, n, n, n), dtype=np.float64, order="F")
        u[0] = rho
        ctx.load(None, u)
        diag = ctx.iterate(niter)
        defpot = np.zeros((n, n, n), dtype=np.float64, order="F")
        ctx.store(defpot, u)
        res = {"def": defpot, "u": u, "diag": diag}
        if outputs:
            grad = np.zeros((n, n, n, 3), dtype=np.float64, order="F")
            delta = np.zeros((n, n, n), dtype=np.float64, order="F")
            ctx.outputs(grad, delta)
            res["grad"], res["delta"] = grad, delta
        return res


def batch_run(rhos, niter, workers=4, precision=MMH_MIXED, schedule=MMH_SCHED_TOL, tol=1e-8, max_cycles=200,
              outputs=True, device=0, check=True, **kw):
    """mmh_batch_run: independent reconstructions of the densities `rhos`
    (Fortran-ordered float64 cubes, any mix of power-of-two sizes) on
    `workers` concurrent host workers.  Returns one dict per problem with
    def, grad, delta (None when outputs=False), status and vcycles; raises
    MMHError on a failed problem unless check=False."""
    L = lib()
    cfg = Config()
    L.mmh_config_default(C.byref(cfg), 8)
    cfg.precision, cfg.schedule, cfg.tol, cfg.max_cycles, cfg.device = (int(precision), int(schedule), float(tol),
                                                                       int(max_cycles), int(device))
    for k, v in kw.items():
        setattr(cfg, k, v)
    probs = (Problem * len(rhos))()
    keep = []
    for i, r in enumerate(rhos):
        r = _farr(r, np.float64)
        n = r.shape[0]
        d = np.zeros((n, n, n), order="F")
        g = np.zeros((n, n, n, 3), order="F") if outputs else None
        de = np.zeros((n, n, n), order="F") if outputs else None
        keep.append((r, d, g, de))
        probs[i] = Problem(n, int(niter), r.ctypes.data, d.ctypes.data, None if g is None else g.ctypes.data,
                           None if de is None else de.ctypes.data, 0, 0)
    rc = L.mmh_batch_run(C.byref(cfg), probs, len(rhos), int(workers))
    out = [{"def": k[1], "grad": k[2], "delta": k[3], "status": probs[i].status, "vcycles": probs[i].vcycles}
           for i, k in enumerate(keep)]
    if check and rc not in (MMH_OK, MMH_ERR_DIVERGED):
        raise MMHError(rc, "batch_run")
    return out

