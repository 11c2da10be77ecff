/*
 * mmh.h -- C ABI of the GB300 (sm_103a) MMH reconstruction library.
 *
 * Drop-in replacement for the hot path of pandaPQY/Moving-Mesh-reconstruction
 * (Fortran 90, directory mmh/): the curvilinear multigrid solve, the
 * grid-compression limiter, the relaxing-TVD density update and the spectral
 * outputs.  Each drop-in entry point below replaces one Fortran subroutine and
 * keeps its argument meaning; arrays are the caller's, in the Fortran layout
 * (column-major, a(i,j,k) at a[(i-1) + n*((j-1) + n*(k-1))], u(nf,n,n,n)
 * component-fastest), periodic in all three directions.
 *
 * Differences from the Fortran calling convention:
 *   - every call takes a context created by mmh_create (device buffers, FFT
 *     plans, stream, configuration) instead of compile-time NG and COMMON state;
 *   - errors are returned as negative codes (mmh_strerror) instead of
 *     write + stop/pause; nothing exits the process;
 *   - diagnostics the Fortran prints are returned in an mmh_diag struct.
 *
 * A context is not thread-safe; use one context per host thread / stream.
 */
#ifndef MMH_H
#define MMH_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MMH_OK 0
#define MMH_ERR_ARG (-1)         /* bad argument (null pointer, nred != 1, iopt != 2, ...) */
#define MMH_ERR_SIZE (-2)        /* grid not a cube / size out of range / size mismatch with context */
#define MMH_ERR_NOTPOW2 (-3)     /* grid size not a power of two */
#define MMH_ERR_CUDA (-4)        /* CUDA runtime or cuFFT failure */
#define MMH_ERR_NAN (-5)         /* NaN or Inf detected in a residual or sum */
#define MMH_ERR_DIVERGED (-6)    /* tolerance schedule hit max_cycles without reaching tol */
#define MMH_ERR_UNSUPPORTED (-7) /* e.g. relaxing with nonzero momentum/energy components */
#define MMH_ERR_RANGE (-8)       /* a summed value is outside the exact-sum range |x| < 2^32 */
#define MMH_ERR_NOMEM (-9)       /* device allocation failed */
#define MMH_ERR_TOO_LARGE (-10)  /* grid larger than an allocation-free entry point's fixed scratch */

/* precision forms */
#define MMH_FP64 0  /* everything in FP64 (bit-identical to the CPU restatement) */
#define MMH_MIXED 1 /* FP32 inner V-cycles inside a defect-correction loop whose residual is
                       float-float (MMH_SCHED_TOL with tol >= 1e-10) or FP64 (otherwise);
                       relaxing with FP32 fluxes and an FP64 update */

/* multigrid schedules */
#define MMH_SCHED_REF 0    /* reference: one V-cycle, 4*NG/n sweeps per level (mgtemplate.f90) */
#define MMH_SCHED_TOL 1    /* flexible CG preconditioned by one V(nu1,nu2) cycle per iteration,
                              until ||r||_inf <= tol*||rhs||_inf */
#define MMH_SCHED_VCYCLE 2 /* plain V(nu1,nu2) cycles until ||r||_inf <= tol*||rhs||_inf (MMH_MIXED:
                              FP32 cycles in an FP64 defect-correction loop) */

typedef struct mmh_ctx mmh_ctx;

typedef struct mmh_config {
  int n;          /* NG: top-level grid size, power of two, 8..1024 (mmh/dimen.f90:1) */
  int precision;  /* MMH_FP64 or MMH_MIXED (MMH_MIXED needs MMH_SCHED_TOL or MMH_SCHED_VCYCLE) */
  int schedule;   /* MMH_SCHED_REF, MMH_SCHED_TOL or MMH_SCHED_VCYCLE */
  int nu1, nu2;   /* pre/post Gauss-Seidel sweeps per level, tolerance schedule */
  int max_cycles; /* V-cycle / outer-iteration cap, tolerance schedule */
  double tol;     /* relative max-norm residual target, tolerance schedule */
  int device;     /* CUDA device ordinal */
  void* stream;   /* cudaStream_t to run on; NULL: the context creates its own */
  int precond_guards; /* MMH_SCHED_TOL: apply the coarse-level divergence guards inside the
                         preconditioner V-cycle (default 0: the preconditioner stays linear) */
} mmh_config;

/* Diagnostics: the quantities the Fortran prints (mg64.f90:43-45,
 * limiter.f90:657-667, main.f90:97-105). */
typedef struct mmh_diag {
  double r1;        /* top-level max-norm residual after pre-smoothing (last cycle) */
  double relaxerr;  /* top-level max-norm residual after post-smoothing (last cycle) */
  double rhsnorm;   /* max |rhs| after rgzerosum */
  double resid_rel; /* final ||r||_inf/||rhs||_inf (FP64 residual in MMH_MIXED) */
  int vcycles;      /* V-cycles / PCG iterations / outer corrections run in the last solve */
  int guards;       /* coarse-level corrections discarded by the divergence guard */
  int status;       /* status of the call */
  int pad;
  long long nexpand;   /* cells hit by the expansion limiter (pass 1) */
  long long ncompress; /* cells hit by the compression limiter (second test) */
  double cmax, detmin, detmax, fluxmax, fluxmin, rho2;
} mmh_diag;

/* ---- context ----------------------------------------------------------- */
void mmh_config_default(mmh_config* cfg, int n);
int mmh_create(mmh_ctx** ctx, const mmh_config* cfg);
int mmh_destroy(mmh_ctx* ctx);
const char* mmh_strerror(int code);
int mmh_sync(mmh_ctx* ctx);
/* number of kernels this library has launched in the process (all contexts) */
unsigned long long mmh_launch_count(void);

/* ---- drop-ins for the Fortran subroutines (host arrays, default real) ---- */

/* calcdefp(defp,tmp,tmp2,def,u,dtold1,dtaumesh,nfluid)       mmh/limiter.f90:17
 * defp(n,n,n) out; tmp(n,n,n) and tmp2(n+2,n,n) are scratch as in the
 * reference (tmp(1..3,1,1) return rho2, xlum, temp; tmp2 is not written);
 * u(nfluid,n,n,n) with u(2:nfluid) == 0 (state at rest, as main.f90 sets it). */
int mmh_calcdefp(mmh_ctx* ctx, float* defp, float* tmp, float* tmp2, const float* def, const float* u, float dtold1,
                 float dtaumesh, int nfluid, mmh_diag* diag);
int mmh_calcdefp_f64(mmh_ctx* ctx, double* defp, double* tmp, double* tmp2, const double* def, const double* u,
                     double dtold1, double dtaumesh, int nfluid, mmh_diag* diag);

/* multigrid(u,rhs,defpot,ubig,dx,nx,ny,nz,nu,nred,iopt)    mmh/multigrid.f90:16
 * u in/out, rhs in/out (rgzerosum is applied in place), iopt must be 2
 * (potential-flow solver), nred must be 1, nx = ny = nz <= NG. */
int mmh_multigrid(mmh_ctx* ctx, float* u, float* rhs, const float* defpot, const float* ubig, float dx, int nx,
                  int ny, int nz, int nu, int nred, int iopt, mmh_diag* diag);
int mmh_multigrid_f64(mmh_ctx* ctx, double* u, double* rhs, const double* defpot, const double* ubig, double dx,
                      int nx, int ny, int nz, int nu, int nred, int iopt, mmh_diag* diag);

/* relaxing(u,def,defp,cmax,dt,nfluidcmp)                     mmh/relaxing.f90:21
 * u(nfluidcmp,n,n,n) in/out; components 2..nfluidcmp must be zero
 * (MMH_ERR_UNSUPPORTED otherwise); cmax is unused, as in the reference. */
int mmh_relaxing(mmh_ctx* ctx, float* u, const float* def, const float* defp, float cmax, float dt, int nfluidcmp);
int mmh_relaxing_f64(mmh_ctx* ctx, double* u, const double* def, const double* defp, double cmax, double dt,
                     int nfluidcmp);

/* scalar2gradient(indata,outdata,nn)                         mmh/gradient.f90:1
 * outdata(n,n,n,3) = F^-1[i k_a F[indata]] with the reference's FFT sign
 * convention (= minus the spectral gradient). */
int mmh_scalar2gradient(mmh_ctx* ctx, const float* indata, float* outdata, const int* nn);
int mmh_scalar2gradient_f64(mmh_ctx* ctx, const double* indata, double* outdata, const int* nn);

/* defp2delta(indata,outdata,nn)                              mmh/reconstruct.f90:1
 * outdata = F^-1[|k|^2 F[indata]] (= minus the spectral Laplacian). */
int mmh_defp2delta(mmh_ctx* ctx, const float* indata, float* outdata, const int* nn);
int mmh_defp2delta_f64(mmh_ctx* ctx, const double* indata, double* outdata, const int* nn);

/* ---- reference subroutines on the path (FP64 host arrays) ------------- */
/* Each computes in the context's precision form: in an MMH_MIXED context
 * mmh_metric_f64 takes one division per cell, mmh_nsmooth_f64 runs three axis
 * passes, mmh_relaxing_f64 one reciprocal per division site and
 * mmh_relax_f64 runs the FP32 Gauss-Seidel sweeps and FP32 residual of the
 * V-cycle on FP32 copies of its arrays (the kernels mmh_iterate runs in that
 * form; not bit-matched to the reference).  mmh_limiter_pass1_f64 and
 * mmh_limiter_mask_f64 give the FP64 form's decisions, fluxes and defplim in
 * both forms (the mixed form screens cells in FP32 and evaluates in FP64 only
 * where a decision is close); in the mixed form pass 1's det extrema and rho2
 * come from the float-float det (not bit-matched). */
/* relax(arr,resid,rhs,deformpot,u,rinf,dx,n,n,n,1,nrelax,iopt)  gauss1.f90:64
 * iopt = 8*isolver + iresidopt with isolver = 2; resid((n/2)^3) is written
 * when iresidopt is 1 or 3. */
int mmh_relax_f64(mmh_ctx* ctx, double* arr, double* resid, const double* rhs, const double* deformpot,
                  const double* rho, double* rinf, double dx, int n, int nrelax, int iopt);
/* cbajraw for every plane: coef(n,n,n,6) = rho_bar*cof(A)/det    gauss1.f90:1027 */
int mmh_metric_f64(mmh_ctx* ctx, const double* deformpot, const double* rho, double dx, int n, double* coef);
/* The mixed form's float-float metric (the coefficients of its outer
 * residual, about 48 significant bits): coef(n,n,n,6) as hi + lo rounded to
 * FP64, det(n,n,n) (may be NULL) = det(A) before the tangle fallback.  dx a
 * power of two; an MMH_MIXED context only (else MMH_ERR_UNSUPPORTED). */
int mmh_metric_ff_f64(mmh_ctx* ctx, const double* deformpot, const double* rho, double dx, int n, double* coef,
                      double* det);
int mmh_restrict_f64(mmh_ctx* ctx, const double* u, int n, double* uhalf);       /* mgutil.f90:74 */
int mmh_inject_f64(mmh_ctx* ctx, double* u, const double* uhalf, int n);         /* mgutil.f90:38 */
int mmh_zerosum_f64(mmh_ctx* ctx, double* arr, int n);                           /* gauss1.f90:1420 */
int mmh_rgzerosum_f64(mmh_ctx* ctx, double* arr, const double* def, double dx, int n); /* gauss1.f90:1219 */
int mmh_nsmooth_f64(mmh_ctx* ctx, double* a, int n);                             /* limiter.f90:677 */
/* pass-1 flux limiter on tmp (in place), density-only state: limiter.f90:175-381.
 * maskx / maskc (nullable, n^3 bytes) receive the expansion and compression masks. */
int mmh_limiter_pass1_f64(mmh_ctx* ctx, double* tmp, const double* def, const double* rho, int n, double dtold,
                          double dtaumesh, unsigned char* maskx, unsigned char* maskc, mmh_diag* diag);
/* compression test: defplim = tlim where tlim > 0 else 0: limiter.f90:425-533 */
int mmh_limiter_mask_f64(mmh_ctx* ctx, double* defplim, const double* def, const double* defp, int n, double dtold,
                         unsigned char* mask, mmh_diag* diag);
/* FFT Poisson correction defp += solve(defplim): limiter.f90:535-597 */
int mmh_limiter_poisson_f64(mmh_ctx* ctx, double* defp, const double* defplim, int n);

/* ---- device-resident reconstruction (mmh/main.f90:83-179) -------------- */
/* Load the state (host arrays): def(n,n,n) (NULL: zero) and u(nfluid,n,n,n). */
int mmh_load_f64(mmh_ctx* ctx, const double* def, const double* u, int nfluid);
/* Same from device memory: def (NULL: zero) and the density u(1,:,:,:) as n^3. */
int mmh_load_dev(mmh_ctx* ctx, const double* d_def, const double* d_rho);
/* niter deformation iterations: calcdefp, def = def + defp, relaxing. */
int mmh_iterate(mmh_ctx* ctx, int niter, mmh_diag* diag);
/* Copy the state back to the host (either pointer may be NULL). */
int mmh_store_f64(mmh_ctx* ctx, double* def, double* u, int nfluid);
/* Spectral outputs of the current def to the host: grad(n,n,n,3), delta(n,n,n)
 * (either may be NULL).  mmh/main.f90:131-179 */
int mmh_outputs_f64(mmh_ctx* ctx, double* grad, double* delta);
/* Same to device memory: d_grad (3 n^3 doubles), d_delta (n^3 doubles). */
int mmh_outputs_dev(mmh_ctx* ctx, double* d_grad, double* d_delta);
/* Device pointers of the resident state (n^3 doubles each). */
int mmh_state_dev(mmh_ctx* ctx, double** d_def, double** d_rho, double** d_defp);

/* The diagnostics main.f90 prints each iteration (main.f90:97-105) and at the
 * end (main.f90:115-117), from the resident state after mmh_iterate: the mean
 * and sqrt(mean square) of def and of the last increment defp, the mean of
 * the density, sqrt(mean (rho-1)^2), its extrema and the count of cells with
 * rho < 0.  The sums are exact (rounded once); NaN when a term is outside
 * |x| < 2^32. */
typedef struct mmh_stats {
  double def_mean, def_sigma, defp_sigma;
  double rho_mean, rho_sigma, rho_min, rho_max;
  long long rho_negative;
} mmh_stats;
int mmh_state_stats(mmh_ctx* ctx, mmh_stats* stats);

/* The limiter's trigger masks of the last calcdefp run on the context
 * (mmh_calcdefp*, mmh_iterate), for checking them against the reference's:
 * expand and compress1 are pass 1's expansion and compression triggers
 * (limiter.f90:335-370, the flux cell km of the tested plane), compress2 the
 * final compression test's (limiter.f90:523-529); n^3 bytes each in the
 * Fortran layout, 1 where the limiter acted; any pointer may be NULL.  The
 * reference keeps no masks (it counts them, limiter.f90:657-667).  Keeping
 * them is armed by mmh_keep_masks(ctx, 1), which costs 3 n^3 bytes of device
 * memory; mmh_masks returns MMH_ERR_ARG while it is not armed. */
int mmh_keep_masks(mmh_ctx* ctx, int on);
int mmh_masks(mmh_ctx* ctx, unsigned char* expand, unsigned char* compress1, unsigned char* compress2);

/* Binned power spectrum of a (n^3, host) -- or the cross spectrum with b (NULL:
 * auto) -- in the bins of the reference's Fisher inputs: nbins (<= 128) bins
 * log-spaced in |k| from 1 to n/2 fundamental modes, bin i holding
 * (n/2)^(i/nbins) <= |k| < (n/2)^((i+1)/nbins) (calcfisherinfo.f90 reads 48 of
 * them and skips the six that hold no mode at 128^3).  power[i] = mean over
 * the bin's modes of |A(k)|^2 / n^3 (Re(A conj(B)) / n^3), A the unnormalised
 * DFT (so unit white noise has power 1); kmean[i] = their mean |k| in
 * fundamental units (the bin's geometric centre, power 0, when it is empty);
 * modes[i] (may be NULL) their number.  Exact sums, independent of order. */
int mmh_power_spectrum_f64(mmh_ctx* ctx, const double* a, const double* b, int nbins, double* kmean, double* power,
                           long long* modes);

/* ---- input preparation (the reference's haloden.f90, from1024to512.f90) -- */
/* Particle density assignment of haloden.f90:87-189: x(3,np) particle
 * positions in fine-cell units (x, y, z fastest; nf fine cells per dimension,
 * wrapped periodically), the ng^3 density (Fortran order, 4-byte reals) with
 * every particle's cell counting it and every empty cell given to the nearest
 * particle of the first non-empty cube shell around it, each particle's unit
 * mass shared equally by its cells, normalised to mean 1.  raw (ng^3, may be
 * NULL) receives the density before normalisation, wp (np, may be NULL) the
 * cells of each particle.  ng <= 1024, np < 2^31.  MMH_ERR_RANGE when a
 * position falls outside the grid after the wrap, or when an empty cell has
 * no particle within 64 cells (the search's cost grows as the cube of that
 * distance; the reference would keep searching).  No context: the call
 * allocates and frees its own device memory on the current device. */
int mmh_haloden(const float* x, long long np, int nf, int ng, float* den, float* raw, int* wp);
/* from1024to512.f90: ncoarse halvings of an ng^3 density by 2x2x2 block sums,
 * then scaled to mean 1 (the sum taken exactly, then rounded to 4 bytes). */
int mmh_coarsen(const float* den, int ng, int ncoarse, float* out);

/* ---- after the path (mmh/column_density.f90, gridfigure.f90) ----------- */
/* Column density of mmh/column_density.f90: den and def (ng^3, Fortran order,
 * 4-byte reals) -> proj (ng^2): den scaled to mean 1, the z displacement
 * dspz of def, and for each column the density between the displaced faces
 * of cells ng/2 and ng/2+nplot-1 with fractional end cells, divided by nplot.
 * Cells outside 1..ng wrap periodically (the reference reads past the array
 * there); faces more than 4 ng cells apart give MMH_ERR_RANGE.  The sum that
 * scales den is exact, rounded once. */
int mmh_column_density(const float* den, const float* def, int ng, int nplot, float* proj);
/* gridfigure.f90:41-120: the displacement of a coarse def (nf^3) on the
 * reference's (0:nf)^3 node grid with its halo, interpolated to the fine
 * cells of an ng^3 density (ng a multiple of nf); proj2 (2, nf, nf) receives
 * the new x, y positions of every (ng/nf)-th cell of plane ng/2, proj (ng^2)
 * the column density of plane ng/2 (either may be NULL).  A node index nf+1
 * (fine cells i = ng, read past the array by the reference) wraps to 1. */
int mmh_gridfigure(const float* def, int nf, const float* den, int ng, float* proj2, float* proj);

/* ---- batched realisations (no single call in the reference) ------------ */
/* One independent reconstruction of mmh/main.f90:83-179: density rho (n^3,
 * Fortran order, host), def = 0, niter deformation iterations, then the
 * outputs; def/grad/delta are host outputs (each may be NULL: not copied). */
typedef struct mmh_problem {
  int n;             /* grid size: power of two, 8..1024 */
  int niter;         /* deformation iterations */
  const double* rho; /* n^3 density */
  double* def;       /* n^3 deformation potential out */
  double* grad;      /* 3 n^3 displacement out (scalar2gradient) */
  double* delta;     /* n^3 density out (defp2delta) */
  int status;        /* out: MMH_OK, or the error of this problem */
  int vcycles;       /* out: V-cycles / PCG iterations of its last solve */
} mmh_problem;
/* Run count problems with the settings of cfg (cfg->n is ignored: each problem
 * has its own) on `workers` concurrent host threads, each with its own CUDA
 * stream and one context per grid size, reused across that worker's problems
 * (largest problems first).  Results are those of running each problem alone.
 * Returns MMH_OK, or the first failing problem's status (all problems run). */
int mmh_batch_run(const mmh_config* cfg, mmh_problem* probs, int count, int workers);

/* ---- allocation-free relax (no counterpart in the reference) ----------- */
/* For callers that cannot let a library allocate device memory (a driver that
 * hands out every buffer from its own pool, or one that must not allocate in a
 * time-critical loop).  Same work as mmh_relax_f64 with iresidopt 0 or 2 --
 * metric, nrelax Gauss-Seidel sweeps, max-norm residual into *rinf -- on
 * device pointers, with no context and no allocation: the scratch (metric,
 * sweep buffer, reduction word) is a fixed device array of the library sized
 * for n <= MMH_NOALLOC_MAX_N (7*64^3+2 doubles, about 14.7 MB, held on every
 * GPU that loads the library until the process exits).  Larger grids return
 * MMH_ERR_TOO_LARGE.  The first call on a device looks up the array's device
 * address; make that first call before any stream capture.  All calls on one
 * device share that device's array, so calls that overlap on the same GPU
 * (concurrent streams or host threads) race and must be serialised by the
 * caller; each device has its own copy.  iopt is bounded as in mmh_relax_f64.
 * The call synchronises `stream` (a cudaStream_t, NULL for the default
 * stream). */
#define MMH_NOALLOC_MAX_N 64
int mmh_relax_noalloc_f64(const double* d_deformpot, const double* d_rho, double* d_arr, const double* d_rhs,
                          double dx, int n, int nrelax, int iopt, double* rinf, void* stream);

/* ---- calcdefp adjoint (no counterpart in the reference) ----------------- */
/* grho(n,n,n) = dJ/d rho and gdef(n,n,n) = dJ/d def (either may be NULL) for
 * J = sum w*defp, defp the increment that mmh_calcdefp_f64 computes from the
 * same def and u (u(2:nfluid) == 0), with the limiter's branch choices
 * (expansion and compression masks, flux clamps, the density clip, the
 * metric's tangle fallback) frozen where this forward pass took them.  defp
 * is defined up to a constant, so w counts through its deviation from its
 * mean.  Where the final compression test limits cells, the gradient runs
 * through its FFT Poisson correction with the mask frozen (the smallest
 * eigenvalue's derivative v v^T; a repeated smallest eigenvalue has none).
 * Needs a solving schedule (MMH_SCHED_TOL or MMH_SCHED_VCYCLE; MMH_SCHED_REF
 * gives MMH_ERR_UNSUPPORTED).  The diag is that of the forward pass; vcycles
 * adds the adjoint solve's. */
int mmh_calcdefp_adjoint_f64(mmh_ctx* ctx, const double* def, const double* u, int nfluid, double dtold1,
                             double dtaumesh, const double* w, double* grho, double* gdef, mmh_diag* diag);

/* gu(n,n,n) = dJ/d rho, gdef = dJ/d def, gdefp = dJ/d defp (the last two may
 * be NULL) for J = sum w*u'(1,:,:,:), u' the density that mmh_relaxing_f64
 * computes from the same u, def, defp and dt (u(2:nfluidcmp) == 0), with the
 * minmod slopes and the cflkeuler maximum frozen where this forward pass took
 * them.  Assumes a finite non-zero density and det in every cell. */
int mmh_relaxing_adjoint_f64(mmh_ctx* ctx, const double* u, const double* def, const double* defp, double dt,
                             int nfluidcmp, const double* w, double* gu, double* gdef, double* gdefp);

/* Adjoint of a whole reconstruction: niter deformation iterations of
 * mmh_iterate from the loaded state (def_0, rho_0), then grho = dJ/d rho_0 and
 * gdef = dJ/d def_0 (NULL: not returned) for
 *   J = sum wdef*def_N + sum wdelta*delta,  delta = defp2delta(def_N),
 * (wdef, wdelta: n^3 host arrays, NULL: zero), the limiter and slope-limiter
 * branches frozen as above.  The forward states are kept every
 * checkpoint_every iterations and the others recomputed as the adjoint walks
 * back.  Needs a solving schedule; the state ends as after mmh_iterate(niter)
 * (after an error it is the failing step's: reload before reuse). */
int mmh_iterate_adjoint_f64(mmh_ctx* ctx, int niter, int checkpoint_every, const double* wdef, const double* wdelta,
                            double* grho, double* gdef, mmh_diag* diag);

/* ---- Gauss-Seidel tile tuning (no counterpart in the reference) -------- */
/* The FP32 plane Gauss-Seidel kernel (the mixed form's smoother on grids of
 * 64^3 and up) has four tile shapes (TX x TY cells: 0 = 32x16, 1 = 64x8,
 * 2 = 16x32, 3 = 32x8) and two strip lengths of the kernel that marches a
 * 64-cell strip along y with the four colours as a wavefront (4 = 64x128,
 * 5 = 64x256).  All of them compute the same bits; the first sweep on
 * a grid size and device outside a stream capture times those that fit (three
 * half sweeps each, phi untouched) and keeps the fastest.  mmh_gs_tile_pin
 * pins one shape for every grid instead (-1: back to timing); mmh_gs_tile
 * reports the shape in use for grid n on the current device (MMH_ERR_ARG when
 * none has been chosen yet). */
int mmh_gs_tile_pin(int shape);
/* The FP32 residual and operator stencil of the mixed form's V-cycles and
 * conjugate gradients: from 64^3 up a CTA marches through 8 planes of its
 * tile column, keeping a ring of planes in shared memory and copying the next
 * plane while it computes one (the default, kind -1 or 1); kind 0 pins one
 * plane per CTA.  Both compute the same bits. */
int mmh_stencil_pin(int kind);
int mmh_gs_tile(int n, int* tx, int* ty);

/* ---- kernel timing (no counterpart in the reference) -------------------- */
/* Arm CUDA-event timing of one kernel kind (MMH_K_* | MMH_K_F32 for the FP32
 * instantiation) on the stream it is launched on; mmh_profile_stop returns the
 * number of launches timed, their summed device time in ms and the number of
 * cells they processed (cells updated, for the Gauss-Seidel colour kernel).
 * The event pool grows with the launches timed; mmh_profile_stop returns
 * MMH_ERR_NOMEM (with the figures of the launches it did time) when a launch
 * went untimed because no event could be created.  While armed, the
 * preconditioner cycle runs launch by launch instead of from its CUDA graph. */
#define MMH_K_GS 1
#define MMH_K_RESIDUAL 2
#define MMH_K_RESTRICT_RESID 3
#define MMH_K_METRIC 4
#define MMH_K_SMOOTH 5
#define MMH_K_PROLONG 6
#define MMH_K_RESTRICT 7
#define MMH_K_F32 256
/* OR-ed into the kind: time only the launches on the n^3 grid level. */
#define MMH_K_AT(n) ((n) << 12)
int mmh_profile_start(int kind);
int mmh_profile_stop(int* launches, double* ms, long long* cells);

#ifdef __cplusplus
}
#endif
#endif /* MMH_H */
