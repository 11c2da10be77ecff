// Host side of the MMH library: context, multigrid V-cycles (reference and
// tolerance schedules, FP64 and mixed precision), calcdefp, relaxing, spectral
// outputs, and the C ABI declared in include/mmh.h.
#include <cufft.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "../../include/mmh.h"
#include "mmh_internal.h"
#include "mmh_phys.cuh"

using namespace mmh;

namespace {

struct Scal {
  unsigned long long acc[4][2];  // fixed-point accumulators
  double mean, ratio;            // zerosum mean, rgzerosum dfact (unrounded)
  int bad;                       // |x| >= 2^32 or NaN in a sum, or non-zero momentum components
  int uflag;                     // usum flag (1: skip zerosum)
  unsigned long long r1bits[16], errbits[16];
  unsigned long long rhsbits, resbits;
  int gflag[16];
  int guards;
  int pad;
  PcgDev pcg;
  LimDev lim;
};

struct Err {
  int code = MMH_OK;
};

#define CK(x)                                                                   \
  do {                                                                          \
    cudaError_t e_ = (x);                                                       \
    if (e_ != cudaSuccess) {                                                    \
      fprintf(stderr, "mmh: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return MMH_ERR_CUDA;                                                      \
    }                                                                           \
  } while (0)

#define CKF(x)                                                                  \
  do {                                                                          \
    cufftResult r_ = (x);                                                       \
    if (r_ != CUFFT_SUCCESS) {                                                  \
      fprintf(stderr, "mmh: cuFFT error %d at %s:%d\n", (int)r_, __FILE__, __LINE__); \
      return MMH_ERR_CUDA;                                                      \
    }                                                                           \
  } while (0)

#define RET(x)                         \
  do {                                 \
    int rc_ = (x);                     \
    if (rc_ != MMH_OK) return rc_;     \
  } while (0)

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// NVTX range over one stage of the path (calcdefp, multigrid, relaxing,
// spectral outputs, adjoint) for profilers; free when none is attached.
struct Stage {
  explicit Stage(const char* name) { nvtxRangePushA(name); }
  ~Stage() { nvtxRangePop(); }
};
int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

// Coarse plane whose own-plane residual part is accumulated first: the size of
// the last r1lax chunk of relax() (gauss1.f90:134-157).
int special_plane(int nrelax, int n) {
  int nrmax = std::min(4, std::max(1, n / 4));
  if (nrelax > nrmax) {
    int left = nrelax % nrmax;
    return left ? left : nrmax;
  }
  return nrelax;
}

template <class T>
struct Hier {
  std::vector<T*> u, rhs, coef, r;
};

}  // namespace

struct mmh_ctx {
  mmh_config cfg;
  int n = 0, nlev = 0;
  i64 n3 = 0;
  std::vector<int> nl;
  cudaStream_t s = nullptr;
  bool own_stream = false;
  // resident FP64 state
  double *def = nullptr, *rho = nullptr, *scr = nullptr, *defplim = nullptr, *det = nullptr;
  // FP64 hierarchy; level 0 u = defp, rhs = tmp
  Hier<double> h64;
  std::vector<double*> defl, rhol;
  // FP32 hierarchy (mixed)
  Hier<float> h32;
  // flexible PCG vectors (solution, right-hand side, search direction, L p);
  // FP32 correction, right-hand side and directions of the mixed inner solve
  double *px = nullptr, *pb = nullptr, *pp = nullptr, *pq = nullptr;
  float *pe32 = nullptr, *pb32 = nullptr, *pp32 = nullptr, *pq32 = nullptr;
  // relaxing
  double *baj = nullptr, *cc = nullptr, *vt = nullptr, *u1 = nullptr, *gface = nullptr;
  // spectral
  void *Xc = nullptr, *Z = nullptr;
  double* spectab = nullptr;
  double* dotpart = nullptr;  // block sums of the fast FP32 dot products  // twiddle and cosine tables of the spectral kernels
  cufftHandle pd2z = 0, pz2z = 0;
  bool plans = false;
  Scal* sc = nullptr;   // device
  Scal* hsc = nullptr;  // pinned host mirror
  // CUDA graphs of the preconditioner cycle per precision (0 FP64, 1 FP32) and
  // entry level, with the number of library kernels one replay runs
  cudaGraphExec_t pgraph[2][16] = {};
  unsigned long long pgraph_launches[2][16] = {};
  bool pgraph_seen[2][16] = {};
  bool graphs = true;
  std::vector<void*> allocs;
  int last_status = MMH_OK;
  // limiter masks of the last calcdefp (expansion, pass-1 compression, final
  // compression test; n^3 bytes each), kept once mmh_keep_masks armed them
  uint8_t* masks = nullptr;
  bool keep_masks = false;
  // mixed form: inverse of the coarsest (4^3) level's operator, formed with
  // each metric (64 x 64 FP64)
  double* coarse_inv = nullptr;
  // the finest solve level's FP64 coefficient buffer holds float-float pairs
  bool coef_ff = false;
  // the finest metric of the resident def is built (calcdefp's mixed pass 1
  // reads its det); the next multigrid call at level 0 uses it as it is
  bool levels_ready = false;
  // the next solve starts from a zero guess (calcdefp zeroes defp before it)
  bool u_zero = false;
  uint8_t* mask(int q) { return keep_masks ? masks + q * n3 : nullptr; }

  double* defp() { return h64.u[0]; }
  double* tmp() { return h64.rhs[0]; }

  template <class T>
  int alloc(T** p, i64 count) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * (size_t)count) != cudaSuccess) return MMH_ERR_NOMEM;
    allocs.push_back(q);
    *p = (T*)q;
    return MMH_OK;
  }
};

namespace {

// ---------------------------------------------------------------------------
// small building blocks
// ---------------------------------------------------------------------------
template <class T>
int zerosum(mmh_ctx* c, T* a, i64 count) {
  CK(cudaMemsetAsync(c->sc->acc[0], 0, 16, c->s));
  launch_fxsum<T>(a, count, c->sc->acc[0], &c->sc->bad, c->s);
  launch_fx_mean(c->sc->acc[0], (double)count, &c->sc->mean, c->s);
  launch_sub_mean<T>(a, count, &c->sc->mean, c->s);
  return MMH_OK;
}

// rgzerosum(arr, def, dx) at level l (FP64)
int rgzerosum(mmh_ctx* c, double* arr, const double* def, int n, double dx, bool have_det = false) {
  i64 n3 = (i64)n * n * n;
  if (!have_det) launch_det<double>(def, n, dx, c->det, c->s);
  CK(cudaMemsetAsync(c->sc->acc[0], 0, 32, c->s));
  launch_fxsum<double>(c->det, n3, c->sc->acc[0], &c->sc->bad, c->s);
  launch_fxsum<double>(arr, n3, c->sc->acc[1], &c->sc->bad, c->s);
  launch_fx_ratio(c->sc->acc[1], c->sc->acc[0], &c->sc->ratio, c->s);
  launch_sub_dfact<double>(arr, c->det, n3, &c->sc->ratio, c->s);
  return MMH_OK;
}

// usum + conditional zerosum at the multigrid entry (multigrid.f90:41-46)
template <class T>
int usum_zerosum(mmh_ctx* c, T* u, i64 count) {
  CK(cudaMemsetAsync(c->sc->acc[2], 0, 16, c->s));
  launch_fxsum<T>(u, count, c->sc->acc[2], &c->sc->bad, c->s);
  launch_usum_flag<T>(c->sc->acc[2], &c->sc->uflag, c->s);
  launch_fx_mean(c->sc->acc[2], (double)count, &c->sc->mean, c->s);
  launch_sub_mean_unless<T>(u, count, &c->sc->mean, &c->sc->uflag, c->s);
  return MMH_OK;
}

template <class T>
Hier<T>& hier(mmh_ctx* c);
template <>
Hier<double>& hier<double>(mmh_ctx* c) { return c->h64; }
template <>
Hier<float>& hier<float>(mmh_ctx* c) { return c->h32; }

// relax(): nrelax 8-colour sweeps, then residual (mode 3: full weighting into
// rhs[l+1] and max norm; mode 2: max norm only; mode 0: none) into *maxslot.
// zero_init: H.u[l] holds no field yet; the sweeps start from zero.
template <class T>
int relax_level(mmh_ctx* c, int l, int nrelax, int mode, unsigned long long* maxslot, bool zero_init = false) {
  Hier<T>& H = hier<T>(c);
  int n = c->nl[l];
  T dx = T(double(1 << l));
  launch_gs_sweeps<T>(H.u[l], H.rhs[l], H.coef[l], n, dx, nrelax, H.r[l], c->s, zero_init);
  if (mode == 0) return MMH_OK;
  CK(cudaMemsetAsync(maxslot, 0, 8, c->s));
  launch_residual<T>(H.u[l], H.rhs[l], H.coef[l], n, dx, mode == 3 ? H.r[l] : (T*)nullptr, nullptr, maxslot, c->s);
  if (mode == 3) launch_restrict_resid<T>(H.r[l], n, special_plane(nrelax, n), H.rhs[l + 1], c->s);
  return MMH_OK;
}

// post-relaxation step of a level: divergence guard or zerosum
template <class T>
int guard_or_zerosum(mmh_ctx* c, int l, double margin, double floor_, bool guard) {
  Hier<T>& H = hier<T>(c);
  int n = c->nl[l];
  i64 n3 = (i64)n * n * n;
  // The mixed form's FP32 preconditioner keeps the constants its levels
  // carry: they lie in the operator's null space (every row's coefficients
  // sum to zero), so they change neither the PCG's residuals nor its dot
  // products with them, and the outer loop removes the solution's mean.
  if (!guard && std::is_same<T, float>::value && c->cfg.schedule == MMH_SCHED_TOL) return MMH_OK;
  if (!guard) return zerosum<T>(c, H.u[l], n3);
  launch_guard(&c->sc->r1bits[l], &c->sc->errbits[l], margin, floor_, &c->sc->gflag[l], &c->sc->guards, c->s);
  CK(cudaMemsetAsync(c->sc->acc[3], 0, 16, c->s));
  launch_fxsum<T>(H.u[l], n3, c->sc->acc[3], &c->sc->bad, c->s);
  launch_fx_mean(c->sc->acc[3], (double)n3, &c->sc->mean, c->s);
  launch_sub_mean_unless<T>(H.u[l], n3, &c->sc->mean, &c->sc->gflag[l], c->s);
  launch_zero_if<T>(H.u[l], n3, &c->sc->gflag[l], c->s);
  return MMH_OK;
}

int vcycle_fp64(mmh_ctx* c, int l);

// One V-cycle at level l (mgtemplate.f90:6-84; mg4 at multigrid.f90:94-121).
// u_zero: the level's correction starts from zero (H.u[l] is not yet set);
// the FP32 cycle then skips zeroing it where its first sweep runs from zero.
template <class T>
int vcycle(mmh_ctx* c, int l, bool u_zero = false) {
  Hier<T>& H = hier<T>(c);
  int n = c->nl[l];
  bool ref = c->cfg.schedule == MMH_SCHED_REF;
  bool at_ng = (n == c->n);
  bool guard = !at_ng && (c->cfg.schedule != MMH_SCHED_TOL || c->cfg.precond_guards);
  // the post-relaxation residual norms feed the guards and the reference's
  // diagnostics only; the preconditioner of the tolerance schedule without
  // guards skips them
  const int post = (guard || c->cfg.schedule != MMH_SCHED_TOL) ? 2 : 0;
  const bool zfirst = u_zero && std::is_same<T, float>::value && n > 4;
  if (u_zero && !zfirst && !(n == 4 && std::is_same<T, float>::value && c->coarse_inv && !guard))
    launch_fill<T>(H.u[l], (i64)n * n * n, T(0), c->s);
  if (n == 4) {
    if constexpr (std::is_same<T, float>::value) {
      Hier<float>& F = c->h32;
      if (c->coarse_inv && !guard) {
        // exact FP64 solve with the level's inverse (zero-mean result)
        launch_coarse_apply(F.rhs[l], c->coarse_inv, F.u[l], c->s);
        return MMH_OK;
      }
      // coarsest grid solved in FP64 by the reference's sweeps
      i64 n3 = 64;
      launch_f2d(F.rhs[l], c->h64.rhs[l], n3, c->s);
      launch_f2d(F.u[l], c->h64.u[l], n3, c->s);
      RET(vcycle_fp64(c, l));
      launch_d2f(c->h64.u[l], F.u[l], n3, c->s);
      return MMH_OK;
    } else {
      RET(relax_level<T>(c, l, 32, post, &c->sc->r1bits[l]));
      RET(relax_level<T>(c, l, 32, post, &c->sc->errbits[l]));
      return guard_or_zerosum<T>(c, l, 1.001, 1.e-5, guard);
    }
  }
  int nrelax = ref ? 4 * c->n / n : c->cfg.nu1;
  int nrelax2 = ref ? 4 * c->n / n : c->cfg.nu2;
  RET(relax_level<T>(c, l, nrelax, 3, &c->sc->r1bits[l], zfirst));
  RET(vcycle<T>(c, l + 1, true));
  launch_prolong_add<T>(H.u[l], H.u[l + 1], n, c->s);
  RET(relax_level<T>(c, l, nrelax2, post, &c->sc->errbits[l]));
  return guard_or_zerosum<T>(c, l, 1.0, -HUGE_VAL, guard);
}

int vcycle_fp64(mmh_ctx* c, int l) { return vcycle<double>(c, l); }

double bits_to_double(unsigned long long b) {
  double d;
  std::memcpy(&d, &b, 8);
  return d;
}

int pull_scal(mmh_ctx* c) {
  CK(cudaMemcpyAsync(c->hsc, c->sc, sizeof(Scal), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return MMH_OK;
}

// Smallest tolerance the float-float outer residual of the mixed form
// serves: its rounding is ~1e-12 of max|rhs| (terms of ~n/(2 pi) |rhs|, ~2^-45
// each); tighter tolerances take the FP64 residual.
const double kFFTolMin = 1e-10;

// Whether the mixed form's finest-level coefficients of this solve are kept
// as float-float pairs (the tolerance schedule above kFFTolMin).
bool ff_outer(const mmh_ctx* c) {
  return c->cfg.precision == MMH_MIXED && c->cfg.schedule == MMH_SCHED_TOL && c->cfg.tol >= kFFTolMin;
}

// Build the coarse geometry (restricted def and density) and the metric of
// every level from l0 down (FP64; FP32 copies for the mixed form, whose
// finest level's metric is formed as float-float pairs when its outer loop
// keeps them).
int build_levels(mmh_ctx* c, int l0) {
  for (int l = l0 + 1; l < c->nlev; ++l) {
    launch_restrict27<double>(c->defl[l - 1], c->nl[l - 1], c->defl[l], c->s);
    launch_restrict27<double>(c->rhol[l - 1], c->nl[l - 1], c->rhol[l], c->s);
  }
  c->coef_ff = false;
  for (int l = l0; l < c->nlev; ++l) {
    int n = c->nl[l];
    // (a solve on the coarsest level itself keeps FP64 coefficients: its exact
    // coarse solve is formed from them)
    if (l == l0 && l0 < c->nlev - 1 && ff_outer(c)) {
      launch_metric_ff(c->defl[l], c->rhol[l], n, double(1 << l), c->h64.coef[l], c->h32.coef[l], c->det, c->s);
      c->coef_ff = true;
      continue;
    }
    launch_metric<double>(c->defl[l], c->rhol[l], n, double(1 << l), c->h64.coef[l], c->s,
                          c->cfg.precision == MMH_MIXED);
    if (c->cfg.precision == MMH_MIXED) launch_d2f(c->h64.coef[l], c->h32.coef[l], 6 * (i64)n * n * n, c->s);
  }
  if (c->coarse_inv && c->nl[c->nlev - 1] == 4)
    launch_coarse_inverse(c->h64.coef[c->nlev - 1], double(1 << (c->nlev - 1)), c->coarse_inv, c->s);
  return MMH_OK;
}

// One preconditioner application z = V(r) on the precision-T hierarchy:
// r in H.rhs[l0], z to H.u[l0], max|z| into zbits.
template <class T>
int precond(mmh_ctx* c, int l0, unsigned long long* zbits) {
  Hier<T>& H = hier<T>(c);
  int n = c->nl[l0];
  i64 n3 = (i64)n * n * n;
  RET(vcycle<T>(c, l0, true));
  CK(cudaMemsetAsync(zbits, 0, 8, c->s));
  launch_absmax<T>(H.u[l0], n3, zbits, c->s);
  return MMH_OK;
}

// The preconditioner cycle runs tens of launches with no host
// synchronisation, so after one direct run (which also performs the one-time
// kernel attribute setup) it is captured into a CUDA graph and replayed: one
// launch per application instead of one per kernel.  Direct runs stay when
// the kernel timing hooks are armed (they time launches one by one) or when a
// capture fails.
template <class T>
int precond_replay(mmh_ctx* c, int l0, unsigned long long* zbits) {
  const int ti = std::is_same<T, float>::value ? 1 : 0;
  if (!c->graphs || l0 >= 16 || prof_armed()) return precond<T>(c, l0, zbits);
  cudaGraphExec_t& ex = c->pgraph[ti][l0];
  if (!ex) {
    if (!c->pgraph_seen[ti][l0]) {
      c->pgraph_seen[ti][l0] = true;
      return precond<T>(c, l0, zbits);
    }
    const unsigned long long before = launch_count();
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      c->graphs = false;
      return precond<T>(c, l0, zbits);
    }
    int rc = precond<T>(c, l0, zbits);
    cudaError_t e = cudaStreamEndCapture(c->s, &g);
    if (rc == MMH_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
      cudaGraphDestroy(g);
      c->pgraph_launches[ti][l0] = launch_count() - before;  // counted once, for the first replay
      CK(cudaGraphLaunch(ex, c->s));
      return MMH_OK;
    }
    if (g) cudaGraphDestroy(g);
    ex = nullptr;
    cudaGetLastError();
    c->graphs = false;
    return precond<T>(c, l0, zbits);
  }
  CK(cudaGraphLaunch(ex, c->s));
  count_launch((int)c->pgraph_launches[ti][l0]);
  return MMH_OK;
}

// Flexible preconditioned conjugate gradients on L x = b at level l0 in
// precision T, one V-cycle per iteration as preconditioner, until
// max|r| <= tol * bn (recurrence residual) or maxit iterations.  The
// residual lives in H.rhs[l0] (the preconditioner's right-hand side) and the
// preconditioned residual in H.u[l0].  Dot products are exact (FP64 scalars).
// Dot product of the PCG in precision T: exact and order-free in FP64 (the
// oracle's bits), fast and deterministic in FP32 (the mixed inner solve).
template <class T>
void pcg_dot(mmh_ctx* c, const T* a, const T* b, i64 n3, const unsigned long long* abits,
             const unsigned long long* bbits, unsigned long long* acc) {
  if constexpr (std::is_same<T, float>::value)
    launch_dot_fast(a, b, n3, abits, bbits, acc, c->dotpart, c->s);
  else
    launch_dot<T>(a, b, n3, abits, bbits, acc, c->s);
}

// x0_bmax >= 0: x is zero and H.rhs[l0] already holds b, whose max |b| is
// x0_bmax (the initial residual is b itself: no stencil pass).
template <class T>
int pcg_core(mmh_ctx* c, int l0, double dx, T* x, const T* b, T* p, T* q, double bn, double tol, int maxit,
             int* iters, double* rel_out, double* r0_out, double x0_bmax = -1.0) {
  Hier<T>& H = hier<T>(c);
  int n = c->nl[l0];
  i64 n3 = (i64)n * n * n;
  PcgDev* P = &c->sc->pcg;
  T* r = H.rhs[l0];
  T* z = H.u[l0];
  CK(cudaMemsetAsync(P, 0, sizeof(PcgDev), c->s));
  double rmax0 = x0_bmax;
  if (x0_bmax >= 0.0) {
    unsigned long long bits = 0;
    std::memcpy(&bits, &x0_bmax, 8);
    launch_set_u64(&P->rbits, bits, c->s);
  } else {
    launch_residual<T>(x, b, H.coef[l0], n, (T)dx, r, nullptr, &P->rbits, c->s);
    RET(pull_scal(c));
    rmax0 = bits_to_double(c->hsc->pcg.rbits);
  }
  double rel = rmax0 / bn;
  *r0_out = rmax0;
  int it = 0;
  int status = MMH_OK;
  if (rel > tol) {
    RET(precond_replay<T>(c, l0, &P->zbits));
    CK(cudaMemcpyAsync(p, z, sizeof(T) * n3, cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(&P->pbits, &P->zbits, 8, cudaMemcpyDeviceToDevice, c->s));
    pcg_dot<T>(c, r, z, n3, &P->rbits, &P->zbits, P->acc[0]);
    launch_pcg_scalar(P, 0, c->s);
    for (it = 1;; ++it) {
      CK(cudaMemsetAsync(&P->qbits, 0, 8, c->s));
      launch_apply<T>(p, H.coef[l0], n, (T)dx, q, &P->qbits, c->s);
      CK(cudaMemsetAsync(P->acc[1], 0, 16, c->s));
      pcg_dot<T>(c, p, q, n3, &P->pbits, &P->qbits, P->acc[1]);
      launch_pcg_scalar(P, 1, c->s);
      CK(cudaMemsetAsync(&P->rbits, 0, 8, c->s));
      launch_pcg_update<T>(x, r, p, q, n3, &P->alpha, &P->rbits, c->s);
      RET(pull_scal(c));
      rel = bits_to_double(c->hsc->pcg.rbits) / bn;
      if (!(rel == rel) || rel <= tol) break;
      if (it >= maxit) {
        status = MMH_ERR_DIVERGED;
        break;
      }
      RET(precond_replay<T>(c, l0, &P->zbits));
      CK(cudaMemsetAsync(P->acc[0], 0, 16, c->s));
      CK(cudaMemsetAsync(P->acc[2], 0, 16, c->s));
      pcg_dot<T>(c, z, q, n3, &P->zbits, &P->qbits, P->acc[2]);
      pcg_dot<T>(c, r, z, n3, &P->rbits, &P->zbits, P->acc[0]);
      launch_pcg_scalar(P, 2, c->s);
      CK(cudaMemsetAsync(&P->pbits, 0, 8, c->s));
      launch_pcg_pupdate<T>(p, z, n3, &P->beta, &P->pbits, c->s);
    }
  }
  *iters = it;
  *rel_out = rel;
  if (!(rel == rel)) return MMH_ERR_NAN;
  return status;
}

// FP64 true residual of x against b at level l0: max|b - L x| (also copied
// to FP32 in r32 when given).  The mixed form evaluates it with fused
// multiply-adds; the FP64 form keeps the reference's separate roundings.
int true_residual(mmh_ctx* c, int l0, double dx, const double* x, const double* b, float* r32, double* rmax) {
  int n = c->nl[l0];
  CK(cudaMemsetAsync(&c->sc->resbits, 0, 8, c->s));
  if (c->cfg.precision == MMH_MIXED)
    launch_residual_fma(x, b, c->h64.coef[l0], n, dx, r32, &c->sc->resbits, c->s);
  else
    launch_residual<double>(x, b, c->h64.coef[l0], n, dx, nullptr, r32, &c->sc->resbits, c->s);
  RET(pull_scal(c));
  *rmax = bits_to_double(c->hsc->resbits);
  return MMH_OK;
}

// Solve L x = b to tol (MMH_SCHED_TOL).  MMH_FP64: flexible PCG in FP64.
// MMH_MIXED: defect correction -- outer residual at FP64-class accuracy
// (float-float for tol >= kFFTolMin, FP64 below), inner FP32 flexible PCG
// (FP32 V-cycle preconditioner) on the correction to a relative 1e-3, update
// of the outer solution -- until the outer residual meets tol.
const double kInnerTol = 1e-3;
const int kInnerMax = 60;

// the same from the float-float outer solution and coefficients (mixed form)
int true_residual_ff(mmh_ctx* c, int l0, double dx, const double* x, const double* b, float* r32, double* rmax) {
  CK(cudaMemsetAsync(&c->sc->resbits, 0, 8, c->s));
  launch_residual_ff(x, b, c->h64.coef[l0], c->nl[l0], dx, r32, &c->sc->resbits, c->s);
  RET(pull_scal(c));
  *rmax = bits_to_double(c->hsc->resbits);
  return MMH_OK;
}

int pcg_level(mmh_ctx* c, int l0, double dx, double rn, int* iters, double* rel_out, double* r1_out) {
  int n = c->nl[l0];
  i64 n3 = (i64)n * n * n;
  double* u = c->h64.u[l0];
  double* rhs = c->h64.rhs[l0];
  CK(cudaMemcpyAsync(c->pb, rhs, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  CK(cudaMemcpyAsync(c->px, u, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  int status = MMH_OK, total = 0;
  double rel = 0.0, rt = 0.0;
  if (c->cfg.precision == MMH_FP64) {
    int it = 0;
    double r0 = 0.0;
    status = pcg_core<double>(c, l0, dx, c->px, c->pb, c->pp, c->pq, rn, c->cfg.tol, c->cfg.max_cycles, &it, &rel,
                              &r0);
    if (status != MMH_OK && status != MMH_ERR_DIVERGED) return status;
    total = it;
    *r1_out = r0;
  } else {
    // For tol >= kFFTolMin the outer solution and the fine coefficients are
    // carried as float-float pairs in their own buffers (the FP32 copy of the
    // coefficients is already made): the outer residual then runs on the FP32
    // pipes at ~48-bit accuracy (k_residual_ff).  Tighter tolerances keep the
    // FP64 residual of an FP64 solution.
    const bool ff = c->cfg.tol >= kFFTolMin;
    if (ff) {
      if (!c->coef_ff) launch_ff_split(c->h64.coef[l0], 6 * n3, c->s);
      c->coef_ff = true;
      launch_ff_split(c->px, n3, c->s);
    }
    auto outer_residual = [&](float* r32, double* r) {
      return ff ? true_residual_ff(c, l0, dx, c->px, c->pb, r32, r) : true_residual(c, l0, dx, c->px, c->pb, r32, r);
    };
    // A solve from a zero guess (calcdefp's) starts from the residual b itself.
    const bool x0 = c->u_zero && ff;
    c->u_zero = false;
    double rmax = 0.0;
    for (int outer = 0;; ++outer) {
      // the outer residual in FP32 is the inner solve's right-hand side and
      // initial residual (its correction starts from zero)
      if (outer == 0 && x0) {
        CK(cudaMemsetAsync(&c->sc->resbits, 0, 8, c->s));
        launch_ff_rhs32(c->pb, n3, c->h32.rhs[l0], &c->sc->resbits, c->s);
        RET(pull_scal(c));
        rmax = bits_to_double(c->hsc->resbits);
      } else {
        RET(outer_residual(c->h32.rhs[l0], &rmax));
      }
      rel = rmax / rn;
      if (outer == 0) *r1_out = rmax;
      if (!(rel == rel)) return MMH_ERR_NAN;
      if (rel <= c->cfg.tol) break;
      if (total >= c->cfg.max_cycles) {
        status = MMH_ERR_DIVERGED;
        break;
      }
      launch_fill<float>(c->pe32, n3, 0.0f, c->s);
      int it = 0;
      double rin = 0.0, r0 = 0.0;
      // the inner solve reduces the residual by kInnerTol, or only as far as
      // the outer tolerance still needs (with a margin) when that is less
      const double inner_tol = std::max(kInnerTol, 0.3 * c->cfg.tol * rn / rmax);
      int st = pcg_core<float>(c, l0, dx, c->pe32, c->pb32, c->pp32, c->pq32, rmax, inner_tol, kInnerMax, &it, &rin,
                               &r0, rmax);
      if (st != MMH_OK && st != MMH_ERR_DIVERGED) return st;
      total += it;
      if (ff)
        launch_ff_add_f(c->px, c->pe32, n3, c->s);
      else
        launch_add_f2d(c->px, c->pe32, n3, c->s);
    }
    if (ff) {
      // zero mean (the exact sum of all hi and lo parts), back to FP64.  The
      // operator annihilates constants (each row's coefficients sum to zero),
      // so the residual reported is the last outer residual.
      CK(cudaMemsetAsync(c->sc->acc[0], 0, 16, c->s));
      launch_fxsum<float>(reinterpret_cast<const float*>(c->px), 2 * n3, c->sc->acc[0], &c->sc->bad, c->s);
      launch_fx_mean(c->sc->acc[0], (double)n3, &c->sc->mean, c->s);
      launch_ff_sub_mean(c->px, &c->sc->mean, n3, c->s);
      rt = rmax;
      launch_ff_join(c->px, n3, c->s);
    }
  }
  if (c->cfg.precision == MMH_FP64 || c->cfg.tol < kFFTolMin) {
    // zero mean, true residual
    RET(zerosum<double>(c, c->px, n3));
    RET(true_residual(c, l0, dx, c->px, c->pb, nullptr, &rt));
  }
  CK(cudaMemcpyAsync(u, c->px, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  CK(cudaMemcpyAsync(rhs, c->pb, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  *rel_out = rt / rn;
  *iters = total;
  if (!(rt == rt)) return MMH_ERR_NAN;
  if (status == MMH_ERR_DIVERGED && *rel_out <= c->cfg.tol) status = MMH_OK;
  return status;
}

// multigrid(u, rhs, defpot, ubig, dx, ...) at level l0: u = h64.u[l0],
// rhs = h64.rhs[l0], defpot = defl[l0], density = rhol[l0] already in place.
int multigrid_level(mmh_ctx* c, int l0, double dx, mmh_diag* d) {
  Stage stage_("mmh multigrid");
  int n = c->nl[l0];
  i64 n3 = (i64)n * n * n;
  CK(cudaMemsetAsync(c->sc, 0, offsetof(Scal, lim), c->s));
  // The mixed form's float-float metric also gives det(A) for rgzerosum, so
  // the metric goes first there (it does not depend on rhs or u).
  const bool det_from_metric = ff_outer(c) && l0 < c->nlev - 1 && dx == double(1 << l0);
  const bool ready = c->levels_ready && l0 == 0;
  c->levels_ready = false;
  if (det_from_metric && !ready) RET(build_levels(c, l0));
  RET(rgzerosum(c, c->h64.rhs[l0], c->defl[l0], n, dx, det_from_metric));
  RET(usum_zerosum<double>(c, c->h64.u[l0], n3));
  launch_absmax<double>(c->h64.rhs[l0], n3, &c->sc->rhsbits, c->s);
  if (!det_from_metric) RET(build_levels(c, l0));
  int cycles = 0;
  double rn = 0.0, rel = 0.0;
  int status = MMH_OK;
  if (c->cfg.schedule == MMH_SCHED_REF) {
    RET(vcycle<double>(c, l0));
    cycles = 1;
    RET(pull_scal(c));
    rn = bits_to_double(c->hsc->rhsbits);
    rel = rn > 0 ? bits_to_double(c->hsc->errbits[l0]) / rn : 0.0;
  } else if (c->cfg.schedule == MMH_SCHED_TOL) {
    RET(pull_scal(c));
    rn = bits_to_double(c->hsc->rhsbits);
    if (rn > 0) {
      double r1 = 0.0;
      status = pcg_level(c, l0, dx, rn, &cycles, &rel, &r1);
      if (status != MMH_OK && status != MMH_ERR_DIVERGED) return status;
      if (d) d->r1 = r1;
    }
    RET(pull_scal(c));
    if (c->hsc->bad) status = MMH_ERR_RANGE;
    if (d) {
      d->relaxerr = rel * rn;
      d->rhsnorm = rn;
      d->resid_rel = rel;
      d->vcycles = cycles;
      d->guards = c->hsc->guards;
      d->status = status;
    }
    return status;
  } else if (c->cfg.precision == MMH_FP64) {
    RET(pull_scal(c));
    rn = bits_to_double(c->hsc->rhsbits);
    if (rn > 0) {
      for (cycles = 0; cycles < c->cfg.max_cycles;) {
        RET(vcycle<double>(c, l0));
        cycles++;
        RET(pull_scal(c));
        rel = bits_to_double(c->hsc->errbits[l0]) / rn;
        if (!(rel == rel)) break;
        if (rel <= c->cfg.tol) break;
      }
      if (rel > c->cfg.tol && rel == rel) status = MMH_ERR_DIVERGED;
    }
  } else {
    // mixed: FP64 residual / FP32 V-cycle defect correction
    RET(pull_scal(c));
    rn = bits_to_double(c->hsc->rhsbits);
    Hier<float>& F = c->h32;
    if (rn > 0) {
      for (cycles = 0;; ) {
        CK(cudaMemsetAsync(&c->sc->resbits, 0, 8, c->s));
        launch_residual_fma(c->h64.u[l0], c->h64.rhs[l0], c->h64.coef[l0], n, dx, F.rhs[l0], &c->sc->resbits, c->s);
        RET(pull_scal(c));
        rel = bits_to_double(c->hsc->resbits) / rn;
        if (!(rel == rel) || rel <= c->cfg.tol) break;
        if (cycles >= c->cfg.max_cycles) {
          status = MMH_ERR_DIVERGED;
          break;
        }
        launch_fill<float>(F.u[l0], n3, 0.0f, c->s);
        RET(vcycle<float>(c, l0));
        launch_add_f2d(c->h64.u[l0], F.u[l0], n3, c->s);
        RET(zerosum<double>(c, c->h64.u[l0], n3));
        cycles++;
      }
    }
  }
  RET(pull_scal(c));
  if (!(rel == rel)) status = MMH_ERR_NAN;
  if (c->hsc->bad) status = MMH_ERR_RANGE;
  if (d) {
    d->r1 = bits_to_double(c->hsc->r1bits[l0]);
    d->relaxerr = bits_to_double(c->hsc->errbits[l0]);
    d->rhsnorm = rn;
    d->resid_rel = rel;
    d->vcycles = cycles;
    d->guards = c->hsc->guards;
    d->status = status;
  }
  return status;
}

double ord_to_double(unsigned long long u) {
  unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
  return bits_to_double(b);
}

double fx_host(const unsigned long long* acc) {
  __int128 s = (__int128)(((unsigned __int128)acc[1] << 64) | (unsigned __int128)acc[0]);
  bool neg = s < 0;
  unsigned __int128 a = neg ? (unsigned __int128)(-s) : (unsigned __int128)s;
  double r = (double)(unsigned long long)(a >> 64) + (double)(unsigned long long)a * 5.42101086242752217e-20;
  return neg ? -r : r;
}

void lim_to_diag(const LimDev& L, mmh_diag* d) {
  if (!d) return;
  d->nexpand = (long long)L.nexpand;
  d->ncompress = (long long)L.ncompress;
  d->cmax = ord_to_double(L.cmax);
  d->detmin = ord_to_double(L.detmin);
  d->detmax = ord_to_double(L.detmax);
  d->fluxmax = ord_to_double(L.fluxmax);
  d->fluxmin = ord_to_double(L.fluxmin);
  // rho2 is a printed diagnostic only; terms outside the exact-sum range make it NaN
  d->rho2 = L.flag ? NAN : fx_host(L.rho2);
}

int make_plans(mmh_ctx* c) {
  if (c->plans) return MMH_OK;
  int n = c->n;
  CKF(cufftPlan3d(&c->pd2z, n, n, n, CUFFT_D2Z));
  CKF(cufftPlan3d(&c->pz2z, n, n, n / 2, CUFFT_Z2Z));
  CKF(cufftSetStream(c->pd2z, c->s));
  CKF(cufftSetStream(c->pz2z, c->s));
  RET(c->alloc(&c->spectab, 2 * (i64)n));
  launch_spec_tables(c->spectab, n, c->s);
  c->plans = true;
  return MMH_OK;
}

// FFT Poisson correction: defp += F^-1[F[defplim]/akernel] * 2/n^3, skipped on
// the device when no cell was limited (limiter.f90:535-597).
int limiter_poisson(mmh_ctx* c, double* defp, const double* defplim) {
  RET(make_plans(c));
  CKF(cufftExecD2Z(c->pd2z, (cufftDoubleReal*)defplim, (cufftDoubleComplex*)c->Xc));
  launch_spec_pack(c->Xc, c->n, 4, c->Z, &c->sc->lim, c->spectab, c->s);
  CKF(cufftExecZ2Z(c->pz2z, (cufftDoubleComplex*)c->Z, (cufftDoubleComplex*)c->Z, CUFFT_FORWARD));
  launch_spec_unpack(c->Z, c->n, defp, 1, 1, &c->sc->lim, c->s);
  return MMH_OK;
}

// nsmooth of calcdefp: the reference's 27-point sum in the FP64 form; three
// axis passes in the mixed form (same operator, other rounding), which
// overwrite `in` (every source calcdefp smooths is dead afterwards).
void smooth_step(mmh_ctx* c, double* in, double* out) {
  if (c->cfg.precision == MMH_MIXED)
    launch_smooth_sep(in, c->n, out, c->s);
  else
    launch_smooth27<double>(in, c->n, out, c->s);
}

// calcdefp on the resident state: defp (= h64.u[0]) from def and rho.
int calcdefp_dev(mmh_ctx* c, double dtold, double dtaumesh, uint8_t* mx, uint8_t* mc1, uint8_t* mc2, mmh_diag* d) {
  Stage stage_("mmh calcdefp");
  int n = c->n;
  i64 n3 = c->n3;
  if (dtold < 1.e-8) dtold = 1.0;
  double* tmp = c->tmp();
  double* defp = c->defp();
  launch_calcdefp_rhs(tmp, c->rho, n, dtold, c->cfg.precision == MMH_MIXED, c->s);
  smooth_step(c, tmp, c->scr);
  smooth_step(c, c->scr, tmp);
  smooth_step(c, tmp, c->scr);
  launch_lim_reset(&c->sc->lim, c->s);
  c->levels_ready = false;
  if (ff_outer(c) && c->nlev > 1) {
    // The float-float metric of def (which calcdefp does not change) is
    // built first: pass 1 screens its expansion test with its det.
    RET(build_levels(c, 0));
    c->levels_ready = true;
    launch_limiter_pass1_mixed(c->scr, c->def, c->rho, c->det, n, dtold, dtaumesh, &c->sc->lim, mx, mc1, c->s);
  } else {
    launch_limiter_pass1(c->scr, c->def, c->rho, n, dtold, dtaumesh, &c->sc->lim, mx, mc1, c->s);
  }
  smooth_step(c, c->scr, tmp);
  launch_fill<double>(defp, n3, 0.0, c->s);
  c->u_zero = true;
  int st = multigrid_level(c, 0, 1.0, d);
  c->u_zero = false;
  if (st != MMH_OK && st != MMH_ERR_DIVERGED) return st;
  smooth_step(c, defp, c->scr);
  smooth_step(c, c->scr, defp);
  if (c->cfg.precision == MMH_MIXED)
    launch_limiter_mask_mixed(c->defplim, c->def, defp, n, dtold, &c->sc->lim, mc2, c->s);
  else
    launch_limiter_mask(c->defplim, c->def, defp, n, dtold, &c->sc->lim, mc2, c->s);
  // The FFT Poisson correction adds F^-1[F[defplim]/kernel], which is zero
  // when no cell was limited: its transforms run only when one was.
  RET(pull_scal(c));
  if (c->hsc->lim.ncompress) {
    RET(limiter_poisson(c, defp, c->defplim));
    RET(pull_scal(c));
  }
  lim_to_diag(c->hsc->lim, d);
  return st;
}

// relaxing(u, def, defp, cmax, dt, 5) on the resident density.
int relaxing_dev(mmh_ctx* c, double dt) {
  Stage stage_("mmh relaxing");
  int n = c->n;
  if (c->cfg.precision == MMH_MIXED) {
    // FP32 fluxes, FP64 update (the relaxing buffers hold the FP32 scratch)
    launch_relax32(c->rho, c->def, c->defp(), n, dt, reinterpret_cast<float4*>(c->baj), reinterpret_cast<float*>(c->cc),
                   reinterpret_cast<float*>(c->u1), c->s);
    return MMH_OK;
  }
  launch_relax_stage1(c->rho, c->def, c->defp(), n, c->baj, c->cc, c->vt, c->s);
  launch_relax_dpv(c->vt, c->cc, n, c->rho, dt / 2.0, c->u1, c->gface, c->s);
  launch_relax_flux(c->u1, c->defp(), c->baj, c->cc, n, c->vt, c->s);
  launch_relax_dpv(c->vt, c->cc, n, c->rho, dt, c->rho, c->gface, c->s);
  return MMH_OK;
}

// spectral outputs of src into host/device buffers (grad: 3 planes of n^3)
int spectral_outputs(mmh_ctx* c, const double* src, double* d_grad, double* d_delta) {
  Stage stage_("mmh spectral outputs");
  RET(make_plans(c));
  CKF(cufftExecD2Z(c->pd2z, (cufftDoubleReal*)src, (cufftDoubleComplex*)c->Xc));
  for (int ax = 0; ax < 3 && d_grad; ++ax) {
    launch_spec_pack(c->Xc, c->n, ax, c->Z, &c->sc->lim, c->spectab, c->s);
    CKF(cufftExecZ2Z(c->pz2z, (cufftDoubleComplex*)c->Z, (cufftDoubleComplex*)c->Z, CUFFT_FORWARD));
    launch_spec_unpack(c->Z, c->n, d_grad + ax * c->n3, 1, 0, &c->sc->lim, c->s);
  }
  if (d_delta) {
    launch_spec_pack(c->Xc, c->n, 3, c->Z, &c->sc->lim, c->spectab, c->s);
    CKF(cufftExecZ2Z(c->pz2z, (cufftDoubleComplex*)c->Z, (cufftDoubleComplex*)c->Z, CUFFT_FORWARD));
    launch_spec_unpack(c->Z, c->n, d_delta, 1, 0, &c->sc->lim, c->s);
  }
  return MMH_OK;
}

// Device scratch of one call, released on the context's stream at scope exit.
struct DevTemp {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevTemp() {
    if (p) cudaFreeAsync(p, s);
  }
};

// What the calcdefp adjoint needs from its forward pass: the pass-1 input
// S^3 g, the expansion and compression masks (2 n^3 bytes), the solution
// before the last two smoothings and the rgzerosum ratio sum(b) / sum(det).
struct CalcKeep {
  double* pre;
  double* uf;
  uint8_t* mk;   // 3 n^3 bytes: pass 1's expansion and compression masks, the final test's mask
  double* ratio;
  long long* ncompress;  // host, may be null: cells the final compression test limited
};

// calcdefp_dev on the resident def and rho, keeping what the adjoint needs.
int calcdefp_fwd_keep(mmh_ctx* c, double dtold, double dtaumesh, const CalcKeep& kp, mmh_diag* d) {
  int n = c->n;
  i64 n3 = c->n3;
  if (dtold < 1.e-8) dtold = 1.0;
  double* tmp = c->tmp();
  double* defp = c->defp();
  launch_calcdefp_rhs(tmp, c->rho, n, dtold, c->cfg.precision == MMH_MIXED, c->s);
  smooth_step(c, tmp, c->scr);
  smooth_step(c, c->scr, tmp);
  smooth_step(c, tmp, c->scr);
  CK(cudaMemcpyAsync(kp.pre, c->scr, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  launch_lim_reset(&c->sc->lim, c->s);
  launch_limiter_pass1(c->scr, c->def, c->rho, n, dtold, dtaumesh, &c->sc->lim, kp.mk, kp.mk + n3, c->s);
  smooth_step(c, c->scr, tmp);
  launch_fill<double>(defp, n3, 0.0, c->s);
  c->u_zero = true;
  int st = multigrid_level(c, 0, 1.0, d);
  c->u_zero = false;
  if (st != MMH_OK) return st;
  CK(cudaMemcpyAsync(kp.ratio, &c->sc->ratio, sizeof(double), cudaMemcpyDeviceToDevice, c->s));
  CK(cudaMemcpyAsync(kp.uf, defp, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  smooth_step(c, defp, c->scr);
  smooth_step(c, c->scr, defp);
  launch_limiter_mask(c->defplim, c->def, defp, n, dtold, &c->sc->lim, kp.mk + 2 * n3, c->s);
  RET(pull_scal(c));
  if (c->hsc->lim.ncompress) {
    RET(limiter_poisson(c, defp, c->defplim));
    RET(pull_scal(c));
  }
  if (kp.ncompress) *kp.ncompress = (long long)c->hsc->lim.ncompress;
  lim_to_diag(c->hsc->lim, d);
  return MMH_OK;
}

// The adjoint half: gradients of J = w^T defp with respect to the density
// and to def (grho, gdef: device n^3, either may be null) on the resident
// def and rho of the forward pass kp was kept from.  scratch: 8 n^3.
//   dJ/drho = g' . S^3 (D . S y) - B27( sum_f C_f G_f(lam, u) ),
//   dJ/ddef = Hess^T( d/dA [ - sum_f urg G_f C_f(A) - r y det(A) ] ),
// y = P^T lam = lam - (det^T lam) / sum det, L lam = S^2 w - mean (L symmetric).
int calcdefp_adj_core(mmh_ctx* c, double dtold, double dtaumesh, const CalcKeep& kp, const double* w, double* grho,
                      double* gdef, double* scratch, mmh_diag* da) {
  int n = c->n;
  i64 n3 = c->n3;
  if (dtold < 1.e-8) dtold = 1.0;
  double* cf = scratch;    // C_f or the adjoint of A; 6 n^3
  double* y = cf + 6 * n3;
  double* z = y + n3;
  double* tmp = c->tmp();
  double* defp = c->defp();
  launch_smooth27<double>(w, n, c->scr, c->s);
  launch_smooth27<double>(c->scr, n, tmp, c->s);
  RET(zerosum<double>(c, tmp, n3));
  launch_fill<double>(defp, n3, 0.0, c->s);
  c->u_zero = true;
  int st = multigrid_level(c, 0, 1.0, da);
  c->u_zero = false;
  if (st != MMH_OK) return st;
  const double* lam = defp;
  launch_det<double>(c->def, n, 1.0, c->det, c->s);
  launch_adj_mul(c->det, lam, y, n3, c->s);
  CK(cudaMemsetAsync(c->sc->acc[0], 0, 32, c->s));
  launch_fxsum<double>(c->det, n3, c->sc->acc[0], &c->sc->bad, c->s);
  launch_fxsum<double>(y, n3, c->sc->acc[1], &c->sc->bad, c->s);
  launch_fx_ratio(c->sc->acc[1], c->sc->acc[0], &c->sc->ratio, c->s);
  CK(cudaMemcpyAsync(y, lam, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  launch_sub_mean<double>(y, n3, &c->sc->ratio, c->s);
  if (gdef) {
    launch_box27(c->rho, n, z, c->s);
    launch_adj_metric(c->def, lam, kp.uf, z, y, kp.ratio, n, cf, c->s);
    launch_adj_hess(cf, n, gdef, 0, c->s);
  }
  if (grho) {
    launch_smooth27<double>(y, n, c->scr, c->s);
    launch_adj_pass1(c->scr, kp.pre, kp.mk, kp.mk + n3, dtaumesh, n3, c->s);
    launch_smooth27<double>(c->scr, n, y, c->s);
    launch_smooth27<double>(y, n, c->scr, c->s);
    launch_smooth27<double>(c->scr, n, y, c->s);
    launch_adj_rhs(y, c->rho, dtold, n3, c->s);
    launch_fill<double>(z, n3, 1.0, c->s);
    launch_metric<double>(c->def, z, n, 1.0, cf, c->s);
    launch_adj_contract(lam, kp.uf, cf, n, c->scr, c->s);
    launch_box27(c->scr, n, z, c->s);
    launch_adj_sub(y, z, grho, n3, c->s);
  }
  RET(pull_scal(c));
  if (c->hsc->bad) return MMH_ERR_RANGE;
  return MMH_OK;
}

// calcdefp_adj_core for a forward pass whose final compression test limited
// cells: defp = defp_s + P(mask . tlim(C)), C = I + dtold Hess(defp_s) +
// Hess(def), defp_s = S^2 uf, P the FFT Poisson correction (a real even
// Fourier multiplier, so P^T = P).  With abar = dJ/dC (k_adj_limiter) for the
// seed g = mask . P w, the seed of defp_s is w + dtold Hess^T(abar) and def
// receives Hess^T(abar) directly.  scratch: 10 n^3 (the core's 8 first).
int calcdefp_adj_full(mmh_ctx* c, double dtold, double dtaumesh, const CalcKeep& kp, bool limited, const double* w,
                      double* grho, double* gdef, double* scratch, mmh_diag* da) {
  if (!limited) return calcdefp_adj_core(c, dtold, dtaumesh, kp, w, grho, gdef, scratch, da);
  const int n = c->n;
  const i64 n3 = c->n3;
  if (dtold < 1.e-8) dtold = 1.0;
  double* abar = scratch;        // 6 n^3
  double* pw = scratch + 6 * n3;
  double* ds = scratch + 7 * n3;
  double* wl = scratch + 8 * n3;  // smoothing scratch, then the seed of defp_s
  double* gl = scratch + 9 * n3;
  // P w (the correction's transforms run whenever the count is non-zero)
  CK(cudaMemsetAsync(&c->sc->lim.ncompress, 1, sizeof(c->sc->lim.ncompress), c->s));
  launch_fill<double>(pw, n3, 0.0, c->s);
  RET(limiter_poisson(c, pw, w));
  // defp_s = S^2 uf, smoothed as the forward pass smoothed it
  CK(cudaMemcpyAsync(ds, kp.uf, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  smooth_step(c, ds, wl);
  smooth_step(c, wl, ds);
  launch_adj_limiter(c->def, ds, pw, kp.mk + 2 * n3, n, dtold, abar, c->s);
  launch_adj_hess(abar, n, gl, 0, c->s);
  launch_adj_axpy(w, dtold, gl, wl, n3, c->s);
  RET(calcdefp_adj_core(c, dtold, dtaumesh, kp, wl, grho, gdef, scratch, da));
  if (gdef) launch_add(gdef, gl, n3, c->s);
  return MMH_OK;
}

// Gradients of J = w^T defp with respect to the density and to def for one
// calcdefp increment on the resident def and rho (no counterpart in the
// reference), the limiter's branch choices those of this forward pass.  w
// (device, n^3) is read; grho and gdef (device, n^3, either may be null)
// receive the gradients.  defp is defined up to a constant, so the gradients
// are those of w minus its mean.
int calcdefp_adjoint_dev(mmh_ctx* c, double dtold, double dtaumesh, const double* w, double* grho, double* gdef,
                         mmh_diag* d) {
  if (c->cfg.schedule == MMH_SCHED_REF) return MMH_ERR_UNSUPPORTED;  // one V-cycle is no solve
  i64 n3 = c->n3;
  DevTemp buf;
  buf.s = c->s;
  if (cudaMallocAsync(&buf.p, sizeof(double) * (12 * n3 + 1) + 3 * n3, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
  double* scratch = (double*)buf.p;  // 10 n^3
  long long nc = 0;
  CalcKeep kp;
  kp.pre = scratch + 10 * n3;
  kp.uf = kp.pre + n3;
  kp.ratio = kp.uf + n3;
  kp.mk = (uint8_t*)(kp.ratio + 1);
  kp.ncompress = &nc;
  RET(calcdefp_fwd_keep(c, dtold, dtaumesh, kp, d));
  mmh_diag da{};
  RET(calcdefp_adj_full(c, dtold, dtaumesh, kp, nc > 0, w, grho, gdef, scratch, &da));
  if (d) d->vcycles += da.vcycles;
  return MMH_OK;
}

// Gradients of J = ubar^T u' for u' = relaxing(u, def, defp, dt) on the
// resident rho, def and defp (no counterpart in the reference), with the
// minmod slopes and the cflkeuler maximum frozen where the forward pass took
// them: gu, gdef, gdefp (device, n^3; gdef and gdefp may be null) receive the
// gradients with respect to the density, def and defp.  ubar (device) is read.
// The forward buffers are relaxing_dev's (the context's shared scratch);
// `scratch` (15 n^3, null: allocated here) holds the rest.
int relaxing_adjoint_dev(mmh_ctx* c, double dt, const double* ubar, double* gu, double* gdef, double* gdefp,
                         double* scratch) {
  int n = c->n;
  i64 n3 = c->n3;
  DevTemp buf;
  buf.s = c->s;
  if (!scratch) {
    if (cudaMallocAsync(&buf.p, sizeof(double) * 15 * n3, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
    scratch = (double*)buf.p;
  }
  double* sd0 = c->vt;            // half sums and differences at u (6 planes)
  double* sd1 = scratch;          // ... at the half step (6 planes)
  double* alpha = sd1 + 6 * n3;   // 3 planes
  double* alphabar = alpha + 3 * n3;
  double* cbar = alphabar + 3 * n3;
  double* u1bar = cbar + n3;
  double* xbar = u1bar + n3;
  double* defp = c->defp();
  // forward pass (relaxing_dev) with both stages' half sums kept
  const bool fast = c->cfg.precision == MMH_MIXED;  // as relaxing_dev
  launch_relax_stage1(c->rho, c->def, defp, n, c->baj, c->cc, sd0, c->s, fast);
  launch_adj_alpha(c->baj, defp, c->cc, n, alpha, c->s);
  launch_relax_dpv(sd0, c->cc, n, c->rho, dt / 2.0, c->u1, c->gface, c->s);
  launch_relax_flux(c->u1, defp, c->baj, c->cc, n, sd1, c->s, fast);
  // stage 2 (u' = u - dt R(u1)), then stage 1 (u1 = u - dt/2 R(u))
  CK(cudaMemsetAsync(alphabar, 0, sizeof(double) * 4 * n3, c->s));
  launch_adj_dpv(sd1, c->cc, alpha, c->u1, ubar, -dt, n, u1bar, alphabar, cbar, c->s);
  launch_adj_dpv(sd0, c->cc, alpha, c->rho, u1bar, -dt / 2.0, n, xbar, alphabar, cbar, c->s);
  CK(cudaMemcpyAsync(gu, ubar, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->s));
  launch_add(gu, u1bar, n3, c->s);
  launch_add(gu, xbar, n3, c->s);
  // the flux ratios and speeds back to def and defp (sd0 and sd1 are free)
  double* abar = sd0;
  double* pdbar = sd1;
  launch_adj_relax_geom(c->def, defp, c->cc, alphabar, cbar, n, abar, pdbar, c->s);
  if (gdef) launch_adj_hess(abar, n, gdef, 0, c->s);
  if (gdefp) launch_adj_grad_t(pdbar, n, gdefp, 0, c->s);
  CK(cudaGetLastError());
  return MMH_OK;
}

// niter deformation iterations of mmh_iterate on the resident (def_0, rho_0)
// followed by their adjoint (no counterpart in the reference): for
// J = wdef^T def_N + wdelta^T defp2delta(def_N), grho = dJ/d rho_0 and
// gdef = dJ/d def_0 (device, n^3; wdef, wdelta, gdef may be null).  The
// forward states are kept every `every` iterations and the iterations between
// two of them recomputed, segment by segment, as the adjoint walks back.  The
// resident state ends as (def_N, rho_N); the defp buffer is scratch.
int iterate_adjoint_dev(mmh_ctx* c, int niter, int every, const double* wdef, const double* wdelta, double* grho,
                        double* gdef, mmh_diag* d) {
  Stage stage_("mmh adjoint");
  if (c->cfg.schedule == MMH_SCHED_REF) return MMH_ERR_UNSUPPORTED;
  if (niter < 0 || every < 1) return MMH_ERR_ARG;
  const i64 n3 = c->n3;
  const size_t f = sizeof(double) * (size_t)n3;
  const int ncp = niter > 0 ? (niter + every - 1) / every : 0;
  const int seg = std::min(every, std::max(niter, 1));
  DevTemp buf;
  buf.s = c->s;
  // checkpoints (def, rho) | per segment iteration: def, rho, defp and the
  // calcdefp forward's pre, uf | final state | rhobar, rhobar_next, defbar,
  // four gradient parts | adjoint scratch (15: relaxing's, or calcdefp's 8) |
  // segment ratios and masks
  const i64 words = (2 * (i64)ncp + 5 * (i64)seg + 2 + 7 + 15) * n3 + seg + (3 * (i64)seg * n3 + 7) / 8;
  if (cudaMallocAsync(&buf.p, sizeof(double) * words, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
  double* ckpt = (double*)buf.p;
  double* segst = ckpt + 2 * (i64)ncp * n3;
  double* fin = segst + 5 * (i64)seg * n3;
  double* rbar = fin + 2 * n3;
  double* rbar2 = rbar + n3;
  double* dbar = rbar2 + n3;
  double* ga = dbar + n3;
  double* gb = ga + n3;
  double* gc = gb + n3;
  double* gd = gc + n3;
  double* scratch = gd + n3;
  double* ratios = scratch + 15 * n3;
  uint8_t* masks = (uint8_t*)(ratios + seg);
  double* defp = c->defp();
  std::vector<long long> limited(seg, 0);  // cells each segment iteration's final test limited
  auto keep = [&](int q) {
    CalcKeep kp;
    double* sk = segst + 5 * (i64)q * n3;
    kp.pre = sk + 3 * n3;
    kp.uf = sk + 4 * n3;
    kp.ratio = ratios + q;
    kp.mk = masks + 3 * (i64)q * n3;
    kp.ncompress = &limited[q];
    return kp;
  };
  // forward pass with checkpoints
  for (int k = 0; k < niter; ++k) {
    if (k % every == 0) {
      CK(cudaMemcpyAsync(ckpt + 2 * (i64)(k / every) * n3, c->def, f, cudaMemcpyDeviceToDevice, c->s));
      CK(cudaMemcpyAsync(ckpt + (2 * (i64)(k / every) + 1) * n3, c->rho, f, cudaMemcpyDeviceToDevice, c->s));
    }
    mmh_diag dd{};
    int st = calcdefp_dev(c, 1.0, 1.0, nullptr, nullptr, nullptr, &dd);
    if (st != MMH_OK) return st;
    launch_add(c->def, defp, n3, c->s);
    RET(relaxing_dev(c, 1.0));
    if (d) *d = dd;
  }
  CK(cudaMemcpyAsync(fin, c->def, f, cudaMemcpyDeviceToDevice, c->s));
  CK(cudaMemcpyAsync(fin + n3, c->rho, f, cudaMemcpyDeviceToDevice, c->s));
  // seeds: defbar_N = wdef + defp2delta(wdelta) (defp2delta is symmetric)
  launch_fill<double>(rbar, n3, 0.0, c->s);
  if (wdelta) {
    RET(spectral_outputs(c, wdelta, nullptr, dbar));
    if (wdef) launch_add(dbar, wdef, n3, c->s);
  } else if (wdef) {
    CK(cudaMemcpyAsync(dbar, wdef, f, cudaMemcpyDeviceToDevice, c->s));
  } else {
    launch_fill<double>(dbar, n3, 0.0, c->s);
  }
  for (int s = ncp - 1; s >= 0; --s) {
    const int k0 = s * every, k1 = std::min(k0 + every, niter);
    // recompute the segment, keeping each iteration's state and calcdefp data
    CK(cudaMemcpyAsync(c->def, ckpt + 2 * (i64)s * n3, f, cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(c->rho, ckpt + (2 * (i64)s + 1) * n3, f, cudaMemcpyDeviceToDevice, c->s));
    for (int k = k0; k < k1; ++k) {
      double* sk = segst + 5 * (i64)(k - k0) * n3;
      CK(cudaMemcpyAsync(sk, c->def, f, cudaMemcpyDeviceToDevice, c->s));
      CK(cudaMemcpyAsync(sk + n3, c->rho, f, cudaMemcpyDeviceToDevice, c->s));
      RET(calcdefp_fwd_keep(c, 1.0, 1.0, keep(k - k0), nullptr));
      CK(cudaMemcpyAsync(sk + 2 * n3, defp, f, cudaMemcpyDeviceToDevice, c->s));
      if (k + 1 < k1) {
        launch_add(c->def, defp, n3, c->s);
        RET(relaxing_dev(c, 1.0));
      }
    }
    for (int k = k1 - 1; k >= k0; --k) {
      const double* sk = segst + 5 * (i64)(k - k0) * n3;
      // relaxing: rho_{k+1} = relaxing(rho_k, def_{k+1}, defp_k)
      CK(cudaMemcpyAsync(c->def, sk, f, cudaMemcpyDeviceToDevice, c->s));
      launch_add(c->def, sk + 2 * n3, n3, c->s);
      CK(cudaMemcpyAsync(c->rho, sk + n3, f, cudaMemcpyDeviceToDevice, c->s));
      CK(cudaMemcpyAsync(defp, sk + 2 * n3, f, cudaMemcpyDeviceToDevice, c->s));
      RET(relaxing_adjoint_dev(c, 1.0, rbar, rbar2, ga, gb, scratch));
      std::swap(rbar, rbar2);
      // def_{k+1} = def_k + defp_k: defbar_k = defbar_{k+1} + relaxing's part,
      // defpbar_k = the same + relaxing's defp part
      launch_add(dbar, ga, n3, c->s);
      launch_add(gb, dbar, n3, c->s);
      // calcdefp: defp_k = calcdefp(def_k, rho_k)
      CK(cudaMemcpyAsync(c->def, sk, f, cudaMemcpyDeviceToDevice, c->s));
      RET(calcdefp_adj_full(c, 1.0, 1.0, keep(k - k0), limited[k - k0] > 0, gb, gc, gd, scratch, nullptr));
      launch_add(rbar, gc, n3, c->s);
      launch_add(dbar, gd, n3, c->s);
    }
  }
  CK(cudaMemcpyAsync(grho, rbar, f, cudaMemcpyDeviceToDevice, c->s));
  if (gdef) CK(cudaMemcpyAsync(gdef, dbar, f, cudaMemcpyDeviceToDevice, c->s));
  CK(cudaMemcpyAsync(c->def, fin, f, cudaMemcpyDeviceToDevice, c->s));
  CK(cudaMemcpyAsync(c->rho, fin + n3, f, cudaMemcpyDeviceToDevice, c->s));
  CK(cudaStreamSynchronize(c->s));
  CK(cudaGetLastError());
  return MMH_OK;
}

int check_cube(mmh_ctx* c, int nx, int ny, int nz) {
  if (nx != ny || ny != nz) return MMH_ERR_SIZE;
  if (!is_pow2(nx)) return MMH_ERR_NOTPOW2;
  if (nx < 4 || nx > c->n) return MMH_ERR_SIZE;
  return MMH_OK;
}

// host <-> device helpers with element conversion
template <class H>
int upload(mmh_ctx* c, const H* src, double* dst, i64 count) {
  if (std::is_same<H, double>::value) {
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice, c->s));
  } else {
    float* tmpf = nullptr;
    CK(cudaMallocAsync((void**)&tmpf, sizeof(float) * count, c->s));
    CK(cudaMemcpyAsync(tmpf, src, sizeof(float) * count, cudaMemcpyHostToDevice, c->s));
    launch_f2d(tmpf, dst, count, c->s);
    CK(cudaFreeAsync(tmpf, c->s));
  }
  return MMH_OK;
}
template <class H>
int download(mmh_ctx* c, const double* src, H* dst, i64 count) {
  if (std::is_same<H, double>::value) {
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost, c->s));
  } else {
    float* tmpf = nullptr;
    CK(cudaMallocAsync((void**)&tmpf, sizeof(float) * count, c->s));
    launch_d2f(src, tmpf, count, c->s);
    CK(cudaMemcpyAsync(dst, tmpf, sizeof(float) * count, cudaMemcpyDeviceToHost, c->s));
    CK(cudaFreeAsync(tmpf, c->s));
  }
  CK(cudaStreamSynchronize(c->s));
  return MMH_OK;
}

// density of u(nf,n^3) into dst; MMH_ERR_UNSUPPORTED if u(2:nf) is not zero
template <class H>
int upload_density(mmh_ctx* c, const H* u, int nf, i64 n3, double* dst) {
  if (nf < 1 || nf > 5) return MMH_ERR_ARG;
  if (nf == 1 && std::is_same<H, double>::value) {
    CK(cudaMemcpyAsync(dst, u, sizeof(double) * n3, cudaMemcpyHostToDevice, c->s));
    return MMH_OK;
  }
  // staged in the finest-level coefficient planes (6 n^3 doubles), which hold
  // nothing between solves
  H* tmpu = reinterpret_cast<H*>(c->h64.coef[0]);
  CK(cudaMemcpyAsync(tmpu, u, sizeof(H) * n3 * nf, cudaMemcpyHostToDevice, c->s));
  CK(cudaMemsetAsync(&c->sc->bad, 0, sizeof(int), c->s));
  if (std::is_same<H, double>::value)
    launch_extract_density_d((const double*)tmpu, nf, n3, dst, &c->sc->bad, c->s);
  else
    launch_extract_density_f((const float*)tmpu, nf, n3, dst, &c->sc->bad, c->s);
  RET(pull_scal(c));
  if (c->hsc->bad) return MMH_ERR_UNSUPPORTED;
  return MMH_OK;
}

// write the density back into component 1 of the host u(nf,n^3)
template <class H>
int download_density(mmh_ctx* c, const double* rho, H* u, int nf, i64 n3) {
  std::vector<H> tmp(n3);
  RET(download(c, rho, tmp.data(), n3));
  for (i64 q = 0; q < n3; ++q) u[q * nf] = tmp[q];
  return MMH_OK;
}

template <class H>
int calcdefp_host(mmh_ctx* c, H* defp, H* tmp, H* tmp2, const H* def, const H* u, double dtold, double dtaumesh,
                  int nfluid, mmh_diag* d) {
  (void)tmp2;
  if (!c || !defp || !def || !u) return MMH_ERR_ARG;
  RET(upload(c, def, c->def, c->n3));
  RET(upload_density(c, u, nfluid, c->n3, c->rho));
  mmh_diag dd{};
  int st = calcdefp_dev(c, dtold, dtaumesh, c->mask(0), c->mask(1), c->mask(2), &dd);
  if (st != MMH_OK && st != MMH_ERR_DIVERGED) return st;
  RET(download(c, c->defp(), defp, c->n3));
  if (tmp) {
    // tmp is scratch in the reference; it returns rho2, xlum, temp in its first
    // three elements and the (inert) cold-region marker 1 elsewhere.
    for (i64 q = 0; q < c->n3; ++q) tmp[q] = H(1);
    tmp[0] = H(dd.rho2);
    if (c->n3 > 2) { tmp[1] = H(0); tmp[2] = H(0); }
  }
  dd.status = st;
  if (d) *d = dd;
  return st;
}

template <class H>
int multigrid_host(mmh_ctx* c, H* u, H* rhs, const H* defpot, const H* ubig, double dx, int nx, int ny, int nz, int nu,
                   int nred, int iopt, mmh_diag* d) {
  if (!c || !u || !rhs || !defpot || !ubig) return MMH_ERR_ARG;
  RET(check_cube(c, nx, ny, nz));
  if (nred != 1 || iopt != 2) return MMH_ERR_ARG;
  int l0 = ilog2(c->n / nx);
  i64 n3 = (i64)nx * nx * nx;
  RET(upload(c, u, c->h64.u[l0], n3));
  RET(upload(c, rhs, c->h64.rhs[l0], n3));
  RET(upload(c, defpot, c->defl[l0], n3));
  RET(upload_density(c, ubig, nu, n3, c->rhol[l0]));
  mmh_diag dd{};
  int st = multigrid_level(c, l0, dx, &dd);
  if (st != MMH_OK && st != MMH_ERR_DIVERGED) return st;
  RET(download(c, c->h64.u[l0], u, n3));
  RET(download(c, c->h64.rhs[l0], rhs, n3));
  if (d) *d = dd;
  return st;
}

template <class H>
int relaxing_host(mmh_ctx* c, H* u, const H* def, const H* defp, double dt, int nf) {
  if (!c || !u || !def || !defp) return MMH_ERR_ARG;
  RET(upload(c, def, c->def, c->n3));
  RET(upload(c, defp, c->defp(), c->n3));
  RET(upload_density(c, u, nf, c->n3, c->rho));
  RET(relaxing_dev(c, dt));
  RET(download_density(c, c->rho, u, nf, c->n3));
  return MMH_OK;
}

template <class H>
int spectral_host(mmh_ctx* c, const H* in, H* out, const int* nn, bool grad) {
  if (!c || !in || !out || !nn) return MMH_ERR_ARG;
  if (nn[0] != c->n || nn[1] != c->n || nn[2] != c->n) return MMH_ERR_SIZE;
  RET(upload(c, in, c->scr, c->n3));
  double* o = c->h64.coef[0];  // staging: holds nothing between solves
  int st = spectral_outputs(c, c->scr, grad ? o : nullptr, grad ? nullptr : o);
  if (st == MMH_OK) st = download(c, o, out, c->n3 * (grad ? 3 : 1));
  return st;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

void mmh_config_default(mmh_config* cfg, int n) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->n = n;
  cfg->precision = MMH_FP64;
  cfg->schedule = MMH_SCHED_REF;
  cfg->nu1 = 2;
  cfg->nu2 = 2;
  cfg->max_cycles = 200;
  cfg->tol = 1e-10;
  cfg->device = 0;
  cfg->stream = nullptr;
  cfg->precond_guards = 0;
}

const char* mmh_strerror(int code) {
  switch (code) {
    case MMH_OK: return "ok";
    case MMH_ERR_ARG: return "invalid argument";
    case MMH_ERR_SIZE: return "grid must be a cube no larger than the context size";
    case MMH_ERR_NOTPOW2: return "grid size must be a power of two";
    case MMH_ERR_CUDA: return "CUDA or cuFFT failure";
    case MMH_ERR_NAN: return "NaN or Inf in a residual";
    case MMH_ERR_DIVERGED: return "tolerance not reached within max_cycles";
    case MMH_ERR_UNSUPPORTED: return "unsupported input (nonzero momentum/energy components)";
    case MMH_ERR_RANGE: return "value outside the exact-sum range";
    case MMH_ERR_NOMEM: return "device allocation failed";
    case MMH_ERR_TOO_LARGE: return "grid larger than the fixed scratch of the allocation-free entry point (n <= 64)";
    default: return "unknown error";
  }
}

unsigned long long mmh_launch_count(void) { return mmh::launch_count(); }

int mmh_profile_start(int kind) { return mmh::prof_start(kind) == 0 ? MMH_OK : MMH_ERR_CUDA; }
int mmh_profile_stop(int* launches, double* ms, long long* cells) {
  int r = mmh::prof_stop(launches, ms, cells);
  // r == 1: launches went untimed (no event could be created for them)
  return r < 0 ? MMH_ERR_CUDA : (r > 0 ? MMH_ERR_NOMEM : MMH_OK);
}

int mmh_destroy(mmh_ctx* c) {
  if (!c) return MMH_OK;
  if (c->s) cudaStreamSynchronize(c->s);
  if (c->plans) {
    cufftDestroy(c->pd2z);
    cufftDestroy(c->pz2z);
  }
  for (auto& row : c->pgraph)
    for (cudaGraphExec_t& ex : row)
      if (ex) cudaGraphExecDestroy(ex);
  for (void* p : c->allocs) cudaFree(p);
  if (c->hsc) cudaFreeHost(c->hsc);
  if (c->own_stream && c->s) cudaStreamDestroy(c->s);
  delete c;
  return MMH_OK;
}

int mmh_create(mmh_ctx** out, const mmh_config* cfg) {
  if (!out || !cfg) return MMH_ERR_ARG;
  *out = nullptr;
  int n = cfg->n;
  if (!is_pow2(n)) return MMH_ERR_NOTPOW2;
  if (n < 8 || n > 1024) return MMH_ERR_SIZE;
  if (cfg->precision != MMH_FP64 && cfg->precision != MMH_MIXED) return MMH_ERR_ARG;
  if (cfg->schedule != MMH_SCHED_REF && cfg->schedule != MMH_SCHED_TOL && cfg->schedule != MMH_SCHED_VCYCLE)
    return MMH_ERR_ARG;
  if (cfg->precision == MMH_MIXED && cfg->schedule == MMH_SCHED_REF) return MMH_ERR_ARG;
  if (cfg->schedule != MMH_SCHED_REF && (cfg->nu1 < 1 || cfg->nu2 < 1 || cfg->max_cycles < 1)) return MMH_ERR_ARG;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return MMH_ERR_CUDA;
  mmh_ctx* c = new (std::nothrow) mmh_ctx();
  if (!c) return MMH_ERR_NOMEM;
  c->cfg = *cfg;
  c->n = n;
  c->n3 = (i64)n * n * n;
  for (int m = n; m >= 4; m >>= 1) c->nl.push_back(m);
  c->nlev = (int)c->nl.size();
  if (cfg->stream) {
    c->s = (cudaStream_t)cfg->stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return MMH_ERR_CUDA;
    }
    c->own_stream = true;
  }
  int rc = MMH_OK;
  auto A = [&](auto** p, i64 count) {
    if (rc == MMH_OK) rc = c->alloc(p, count);
  };
  i64 n3 = c->n3;
  // Scratch that is dead while relaxing runs (finest-level multigrid scratch,
  // limiter and spectral buffers, PCG vectors) shares one allocation with the
  // relaxing buffers, which are dead whenever that scratch is in use: this
  // takes 18 fields off the footprint (1024^3 fits on one GPU).
  struct Piece {
    void** p;
    size_t bytes;
  };
  std::vector<Piece> shared;
  auto S = [&](auto** p, i64 count) { shared.push_back({(void**)p, sizeof(**p) * (size_t)count}); };
  A(&c->def, n3);
  A(&c->rho, n3);
  S(&c->scr, n3);
  S(&c->defplim, n3);
  S(&c->det, n3);
  c->h64.u.resize(c->nlev);
  c->h64.rhs.resize(c->nlev);
  c->h64.coef.resize(c->nlev);
  c->h64.r.resize(c->nlev);
  c->defl.resize(c->nlev);
  c->rhol.resize(c->nlev);
  for (int l = 0; l < c->nlev; ++l) {
    i64 m3 = (i64)c->nl[l] * c->nl[l] * c->nl[l];
    A(&c->h64.u[l], m3);
    A(&c->h64.rhs[l], m3);
    if (l == 0) {
      S(&c->h64.coef[l], 6 * m3);
      S(&c->h64.r[l], m3);
      c->defl[0] = c->def;
      c->rhol[0] = c->rho;
    } else {
      A(&c->h64.coef[l], 6 * m3);
      A(&c->h64.r[l], m3);
      A(&c->defl[l], m3);
      A(&c->rhol[l], m3);
    }
  }
  if (cfg->precision == MMH_MIXED) {
    c->h32.u.resize(c->nlev);
    c->h32.rhs.resize(c->nlev);
    c->h32.coef.resize(c->nlev);
    c->h32.r.resize(c->nlev);
    for (int l = 0; l < c->nlev; ++l) {
      i64 m3 = (i64)c->nl[l] * c->nl[l] * c->nl[l];
      if (l == 0) {
        S(&c->h32.u[l], m3);
        S(&c->h32.rhs[l], m3);
        S(&c->h32.coef[l], 6 * m3);
        S(&c->h32.r[l], m3);
      } else {
        A(&c->h32.u[l], m3);
        A(&c->h32.rhs[l], m3);
        A(&c->h32.coef[l], 6 * m3);
        A(&c->h32.r[l], m3);
      }
    }
  }
  if (cfg->precision == MMH_MIXED && c->nl[c->nlev - 1] == 4) A(&c->coarse_inv, 64 * 64);
  if (cfg->schedule == MMH_SCHED_TOL) {
    S(&c->px, n3);
    S(&c->pb, n3);
    if (cfg->precision == MMH_FP64) {
      S(&c->pp, n3);
      S(&c->pq, n3);
    } else {
      S(&c->pe32, n3);
      S(&c->pb32, n3);
      S(&c->pp32, n3);
      S(&c->pq32, n3);
    }
  }
  S((double**)&c->Xc, 2 * (i64)(n / 2 + 1) * n * n);
  S((double**)&c->Z, 2 * (i64)(n / 2) * n * n);
  {
    const size_t align = 256;
    size_t total = 0;
    for (const Piece& q : shared) total += (q.bytes + align - 1) / align * align;
    const size_t relax_bytes = sizeof(double) * 18 * (size_t)n3;  // baj 7, cc 1, sd 6, faces 3, u1 1
    double* arena = nullptr;
    A(&arena, (i64)((std::max(total, relax_bytes) + sizeof(double) - 1) / sizeof(double)));
    if (rc == MMH_OK) {
      char* at = reinterpret_cast<char*>(arena);
      for (const Piece& q : shared) {
        *q.p = at;
        at += (q.bytes + align - 1) / align * align;
      }
      c->baj = arena;
      c->cc = arena + 7 * n3;
      c->vt = arena + 8 * n3;  // half sums and differences of the relaxing fluxes
      c->gface = arena + 14 * n3;
      c->u1 = arena + 17 * n3;
    }
  }
  if (cfg->precision == MMH_MIXED) A(&c->dotpart, kDotBlocks);
  A(&c->sc, 1);
  if (rc == MMH_OK && cudaMallocHost((void**)&c->hsc, sizeof(Scal)) != cudaSuccess) rc = MMH_ERR_NOMEM;
  if (rc == MMH_OK && cudaMemsetAsync(c->sc, 0, sizeof(Scal), c->s) != cudaSuccess) rc = MMH_ERR_CUDA;
  if (rc == MMH_OK) {
    for (int l = 0; l < c->nlev && rc == MMH_OK; ++l) {
      i64 m3 = (i64)c->nl[l] * c->nl[l] * c->nl[l];
      if (cudaMemsetAsync(c->h64.u[l], 0, sizeof(double) * m3, c->s) != cudaSuccess) rc = MMH_ERR_CUDA;
    }
    if (cudaMemsetAsync(c->def, 0, sizeof(double) * n3, c->s) != cudaSuccess) rc = MMH_ERR_CUDA;
  }
  if (rc == MMH_OK && cudaStreamSynchronize(c->s) != cudaSuccess) rc = MMH_ERR_CUDA;
  if (rc != MMH_OK) {
    mmh_destroy(c);
    return rc;
  }
  *out = c;
  return MMH_OK;
}

int mmh_sync(mmh_ctx* c) {
  if (!c) return MMH_ERR_ARG;
  CK(cudaStreamSynchronize(c->s));
  CK(cudaGetLastError());
  return MMH_OK;
}

int mmh_calcdefp(mmh_ctx* c, float* defp, float* tmp, float* tmp2, const float* def, const float* u, float dtold1,
                 float dtaumesh, int nfluid, mmh_diag* d) {
  return calcdefp_host<float>(c, defp, tmp, tmp2, def, u, dtold1, dtaumesh, nfluid, d);
}
int mmh_calcdefp_f64(mmh_ctx* c, double* defp, double* tmp, double* tmp2, const double* def, const double* u,
                     double dtold1, double dtaumesh, int nfluid, mmh_diag* d) {
  return calcdefp_host<double>(c, defp, tmp, tmp2, def, u, dtold1, dtaumesh, nfluid, d);
}
int mmh_calcdefp_adjoint_f64(mmh_ctx* c, const double* def, const double* u, int nfluid, double dtold1,
                             double dtaumesh, const double* w, double* grho, double* gdef, mmh_diag* d) {
  if (!c || !def || !u || !w || (!grho && !gdef)) return MMH_ERR_ARG;
  i64 n3 = c->n3;
  RET(upload(c, def, c->def, n3));
  RET(upload_density(c, u, nfluid, n3, c->rho));
  DevTemp buf;
  buf.s = c->s;
  if (cudaMallocAsync(&buf.p, sizeof(double) * 3 * n3, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
  double* dw = (double*)buf.p;
  RET(upload(c, w, dw, n3));
  mmh_diag dd{};
  int st = calcdefp_adjoint_dev(c, dtold1, dtaumesh, dw, grho ? dw + n3 : nullptr, gdef ? dw + 2 * n3 : nullptr, &dd);
  dd.status = st;
  if (d) *d = dd;
  RET(st);
  if (grho) RET(download(c, dw + n3, grho, n3));
  if (gdef) RET(download(c, dw + 2 * n3, gdef, n3));
  return MMH_OK;
}
int mmh_relaxing_adjoint_f64(mmh_ctx* c, const double* u, const double* def, const double* defp, double dt,
                             int nfluidcmp, const double* w, double* gu, double* gdef, double* gdefp) {
  if (!c || !u || !def || !defp || !w || !gu) return MMH_ERR_ARG;
  i64 n3 = c->n3;
  RET(upload(c, def, c->def, n3));
  RET(upload(c, defp, c->defp(), n3));
  RET(upload_density(c, u, nfluidcmp, n3, c->rho));
  DevTemp buf;
  buf.s = c->s;
  if (cudaMallocAsync(&buf.p, sizeof(double) * 4 * n3, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
  double* dw = (double*)buf.p;
  RET(upload(c, w, dw, n3));
  RET(relaxing_adjoint_dev(c, dt, dw, dw + n3, gdef ? dw + 2 * n3 : nullptr, gdefp ? dw + 3 * n3 : nullptr, nullptr));
  RET(download(c, dw + n3, gu, n3));
  if (gdef) RET(download(c, dw + 2 * n3, gdef, n3));
  if (gdefp) RET(download(c, dw + 3 * n3, gdefp, n3));
  return MMH_OK;
}
int mmh_iterate_adjoint_f64(mmh_ctx* c, int niter, int checkpoint_every, const double* wdef, const double* wdelta,
                            double* grho, double* gdef, mmh_diag* d) {
  if (!c || !grho) return MMH_ERR_ARG;
  i64 n3 = c->n3;
  DevTemp buf;
  buf.s = c->s;
  if (cudaMallocAsync(&buf.p, sizeof(double) * 4 * n3, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
  double* dw = (double*)buf.p;
  if (wdef) RET(upload(c, wdef, dw, n3));
  if (wdelta) RET(upload(c, wdelta, dw + n3, n3));
  mmh_diag dd{};
  int st = iterate_adjoint_dev(c, niter, checkpoint_every, wdef ? dw : nullptr, wdelta ? dw + n3 : nullptr, dw + 2 * n3,
                               gdef ? dw + 3 * n3 : nullptr, &dd);
  dd.status = st;
  if (d) *d = dd;
  RET(st);
  RET(download(c, dw + 2 * n3, grho, n3));
  if (gdef) RET(download(c, dw + 3 * n3, gdef, n3));
  return MMH_OK;
}
int mmh_gs_tile_pin(int shape) {
  if (shape < -1 || shape >= mmh::kGsShapes) return MMH_ERR_ARG;
  mmh::gs_tile_override.store(shape);
  return MMH_OK;
}

int mmh_stencil_pin(int kind) {
  if (kind < -1 || kind > 1) return MMH_ERR_ARG;
  mmh::stencil_march_pin.store(kind);
  return MMH_OK;
}

int mmh_gs_tile(int n, int* tx, int* ty) {
  if (!tx || !ty) return MMH_ERR_ARG;
  *tx = *ty = 0;
  return mmh::gs_tile_chosen(n, tx, ty) >= 0 ? MMH_OK : MMH_ERR_ARG;
}

int mmh_keep_masks(mmh_ctx* c, int on) {
  if (!c) return MMH_ERR_ARG;
  if (on && !c->masks) {
    RET(c->alloc(&c->masks, 3 * c->n3));
    CK(cudaMemsetAsync(c->masks, 0, (size_t)(3 * c->n3), c->s));
  }
  c->keep_masks = on != 0;
  return MMH_OK;
}

int mmh_masks(mmh_ctx* c, unsigned char* expand, unsigned char* compress1, unsigned char* compress2) {
  if (!c || !c->keep_masks) return MMH_ERR_ARG;
  unsigned char* out[3] = {expand, compress1, compress2};
  for (int q = 0; q < 3; ++q)
    if (out[q]) CK(cudaMemcpyAsync(out[q], c->masks + q * c->n3, (size_t)c->n3, cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return MMH_OK;
}

int mmh_state_stats(mmh_ctx* c, mmh_stats* out) {
  if (!c || !out) return MMH_ERR_ARG;
  StatsDev* st = nullptr;
  CK(cudaMallocAsync((void**)&st, sizeof(StatsDev), c->s));
  CK(cudaMemsetAsync(st, 0, sizeof(StatsDev), c->s));
  CK(cudaMemsetAsync(&st->rmin, 0xff, sizeof(unsigned long long), c->s));
  launch_state_stats(c->def, c->defp(), c->rho, c->n3, st, c->s);
  StatsDev h;
  CK(cudaMemcpyAsync(&h, st, sizeof(StatsDev), cudaMemcpyDeviceToHost, c->s));
  CK(cudaFreeAsync(st, c->s));
  CK(cudaStreamSynchronize(c->s));
  const double n3 = (double)c->n3;
  double sum[5];
  for (int q = 0; q < 5; ++q) sum[q] = h.flag ? NAN : fx_host(h.acc[q]);
  out->def_mean = sum[0] / n3;
  out->def_sigma = std::sqrt(sum[1] / n3);
  out->defp_sigma = std::sqrt(sum[2] / n3);
  out->rho_mean = sum[3] / n3;
  out->rho_sigma = std::sqrt(sum[4] / n3);
  out->rho_min = ord_to_double(h.rmin);
  out->rho_max = ord_to_double(h.rmax);
  out->rho_negative = (long long)h.nneg;
  return MMH_OK;
}
int mmh_power_spectrum_f64(mmh_ctx* c, const double* a, const double* b, int nbins, double* kmean, double* power,
                           long long* modes) {
  if (!c || !a || !kmean || !power || nbins < 1 || nbins > kPowMaxBins) return MMH_ERR_ARG;
  const int n = c->n;
  const i64 n3 = c->n3, nc = (i64)(n / 2 + 1) * n * n;
  RET(make_plans(c));
  // squared bin edges (n/2)^(2i/nbins): exact where the exponent makes a power of two
  int m = 0;
  while ((2 << m) < n) ++m;  // n/2 = 2^m
  std::vector<double> e2(nbins + 1);
  for (int i = 0; i <= nbins; ++i) {
    const int num = 2 * m * i;
    e2[i] = num % nbins == 0 ? std::ldexp(1.0, num / nbins) : std::exp2((double)num / nbins);
  }
  DevTemp buf;
  buf.s = c->s;
  const size_t bytes = sizeof(double) * (b ? 2 * nc : 0) + sizeof(double) * (nbins + 1) + sizeof(PowDev);
  if (cudaMallocAsync(&buf.p, bytes, c->s) != cudaSuccess) return MMH_ERR_NOMEM;
  double* Bc = (double*)buf.p;
  double* de2 = Bc + (b ? 2 * nc : 0);
  PowDev* acc = (PowDev*)(de2 + nbins + 1);
  CK(cudaMemcpyAsync(de2, e2.data(), sizeof(double) * (nbins + 1), cudaMemcpyHostToDevice, c->s));
  CK(cudaMemsetAsync(acc, 0, sizeof(PowDev), c->s));
  RET(upload(c, a, c->scr, n3));
  CKF(cufftExecD2Z(c->pd2z, (cufftDoubleReal*)c->scr, (cufftDoubleComplex*)c->Xc));
  if (b) {
    RET(upload(c, b, c->scr, n3));
    CKF(cufftExecD2Z(c->pd2z, (cufftDoubleReal*)c->scr, (cufftDoubleComplex*)Bc));
  }
  launch_power_bins(c->Xc, b ? Bc : nullptr, n, nbins, de2, 1.0 / (double)n3, acc, c->s);
  PowDev h;
  CK(cudaMemcpyAsync(&h, acc, sizeof(PowDev), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  if (h.flag) return MMH_ERR_RANGE;
  for (int q = 0; q < nbins; ++q) {
    const double cnt = (double)h.cnt[q];
    kmean[q] = h.cnt[q] ? fx_host(h.k[q]) / cnt : std::sqrt(std::sqrt(e2[q] * e2[q + 1]));
    power[q] = h.cnt[q] ? fx_host(h.p[q]) / cnt : 0.0;
    if (modes) modes[q] = (long long)h.cnt[q];
  }
  return MMH_OK;
}
int mmh_multigrid(mmh_ctx* c, float* u, float* rhs, const float* defpot, const float* ubig, float dx, int nx, int ny,
                  int nz, int nu, int nred, int iopt, mmh_diag* d) {
  return multigrid_host<float>(c, u, rhs, defpot, ubig, dx, nx, ny, nz, nu, nred, iopt, d);
}
int mmh_multigrid_f64(mmh_ctx* c, double* u, double* rhs, const double* defpot, const double* ubig, double dx, int nx,
                      int ny, int nz, int nu, int nred, int iopt, mmh_diag* d) {
  return multigrid_host<double>(c, u, rhs, defpot, ubig, dx, nx, ny, nz, nu, nred, iopt, d);
}
int mmh_relaxing(mmh_ctx* c, float* u, const float* def, const float* defp, float cmax, float dt, int nfluidcmp) {
  (void)cmax;
  return relaxing_host<float>(c, u, def, defp, dt, nfluidcmp);
}
int mmh_relaxing_f64(mmh_ctx* c, double* u, const double* def, const double* defp, double cmax, double dt,
                     int nfluidcmp) {
  (void)cmax;
  return relaxing_host<double>(c, u, def, defp, dt, nfluidcmp);
}
int mmh_scalar2gradient(mmh_ctx* c, const float* in, float* out, const int* nn) {
  return spectral_host<float>(c, in, out, nn, true);
}
int mmh_scalar2gradient_f64(mmh_ctx* c, const double* in, double* out, const int* nn) {
  return spectral_host<double>(c, in, out, nn, true);
}
int mmh_defp2delta(mmh_ctx* c, const float* in, float* out, const int* nn) {
  return spectral_host<float>(c, in, out, nn, false);
}
int mmh_defp2delta_f64(mmh_ctx* c, const double* in, double* out, const int* nn) {
  return spectral_host<double>(c, in, out, nn, false);
}

int mmh_relax_f64(mmh_ctx* c, double* arr, double* resid, const double* rhs, const double* deformpot,
                  const double* rho, double* rinf, double dx, int n, int nrelax, int iopt) {
  if (!c || !arr || !rhs || !deformpot || !rho || !rinf) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  int ir = iopt % 8;
  if (iopt < 0 || iopt > 256 || (iopt / 8) % 8 != 2 || nrelax < 0) return MMH_ERR_ARG;
  if ((ir == 1 || ir == 3) && (!resid || n < 8)) return MMH_ERR_ARG;
  if (ir != 0 && ir != 2 && ir != 3) return MMH_ERR_ARG;
  int l = ilog2(c->n / n);
  i64 n3 = (i64)n * n * n;
  RET(upload(c, arr, c->h64.u[l], n3));
  RET(upload(c, rhs, c->h64.rhs[l], n3));
  RET(upload(c, deformpot, c->defl[l], n3));
  RET(upload(c, rho, c->rhol[l], n3));
  if (c->cfg.precision == MMH_MIXED) {
    // the mixed form's smoother: FP32 sweeps (and FP32 residual) on FP32
    // copies of phi, rhs and the coefficients, as inside its V-cycles
    Hier<float>& F = c->h32;
    launch_metric<double>(c->defl[l], c->rhol[l], n, dx, c->h64.coef[l], c->s, true);
    launch_d2f(c->h64.coef[l], F.coef[l], 6 * n3, c->s);
    launch_d2f(c->h64.u[l], F.u[l], n3, c->s);
    launch_d2f(c->h64.rhs[l], F.rhs[l], n3, c->s);
    launch_gs_sweeps<float>(F.u[l], F.rhs[l], F.coef[l], n, (float)dx, nrelax, F.r[l], c->s);
    CK(cudaMemsetAsync(c->sc->errbits, 0, 8, c->s));
    if (ir != 0) {
      launch_residual<float>(F.u[l], F.rhs[l], F.coef[l], n, (float)dx, ir == 3 ? F.r[l] : nullptr, nullptr,
                             c->sc->errbits, c->s);
      if (ir == 3) {
        launch_restrict_resid<float>(F.r[l], n, special_plane(nrelax, n), F.rhs[l + 1], c->s);
        launch_f2d(F.rhs[l + 1], c->scr, n3 / 8, c->s);
      }
    }
    launch_f2d(F.u[l], c->h64.u[l], n3, c->s);
    RET(pull_scal(c));
    *rinf = ir >= 2 ? bits_to_double(c->hsc->errbits[0]) : 0.0;
    RET(download(c, c->h64.u[l], arr, n3));
    if (ir == 3) RET(download(c, c->scr, resid, n3 / 8));
    return MMH_OK;
  }
  launch_metric<double>(c->defl[l], c->rhol[l], n, dx, c->h64.coef[l], c->s);
  launch_gs_sweeps<double>(c->h64.u[l], c->h64.rhs[l], c->h64.coef[l], n, dx, nrelax, c->h64.r[l], c->s);
  CK(cudaMemsetAsync(c->sc->errbits, 0, 8, c->s));
  if (ir != 0) {
    launch_residual<double>(c->h64.u[l], c->h64.rhs[l], c->h64.coef[l], n, dx, ir == 3 ? c->h64.r[l] : nullptr,
                            nullptr, c->sc->errbits, c->s);
    if (ir == 3) launch_restrict_resid<double>(c->h64.r[l], n, special_plane(nrelax, n), c->scr, c->s);
  }
  RET(pull_scal(c));
  *rinf = ir >= 2 ? bits_to_double(c->hsc->errbits[0]) : 0.0;
  RET(download(c, c->h64.u[l], arr, n3));
  if (ir == 3) RET(download(c, c->scr, resid, n3 / 8));
  return MMH_OK;
}

int mmh_metric_f64(mmh_ctx* c, const double* deformpot, const double* rho, double dx, int n, double* coef) {
  if (!c || !deformpot || !rho || !coef) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  int l = ilog2(c->n / n);
  i64 n3 = (i64)n * n * n;
  RET(upload(c, deformpot, c->defl[l], n3));
  RET(upload(c, rho, c->rhol[l], n3));
  // the context's form: the reference's six divisions (FP64) or one (mixed)
  launch_metric<double>(c->defl[l], c->rhol[l], n, dx, c->h64.coef[l], c->s, c->cfg.precision == MMH_MIXED);
  return download(c, c->h64.coef[l], coef, 6 * n3);
}

int mmh_metric_ff_f64(mmh_ctx* c, const double* deformpot, const double* rho, double dx, int n, double* coef,
                      double* det) {
  if (!c || !deformpot || !rho || !coef) return MMH_ERR_ARG;
  if (c->cfg.precision != MMH_MIXED) return MMH_ERR_UNSUPPORTED;
  RET(check_cube(c, n, n, n));
  if (n < 4 || dx <= 0.0 || std::ldexp(1.0, std::ilogb(dx)) != dx) return MMH_ERR_ARG;
  int l = ilog2(c->n / n);
  i64 n3 = (i64)n * n * n;
  RET(upload(c, deformpot, c->defl[l], n3));
  RET(upload(c, rho, c->rhol[l], n3));
  launch_metric_ff(c->defl[l], c->rhol[l], n, dx, c->h64.coef[l], c->h32.coef[l], det ? c->det : nullptr, c->s);
  launch_ff_join(c->h64.coef[l], 6 * n3, c->s);
  c->coef_ff = false;
  if (det) RET(download(c, c->det, det, n3));
  return download(c, c->h64.coef[l], coef, 6 * n3);
}

int mmh_restrict_f64(mmh_ctx* c, const double* u, int n, double* uhalf) {
  if (!c || !u || !uhalf) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  if (n < 8) return MMH_ERR_SIZE;
  i64 n3 = (i64)n * n * n;
  RET(upload(c, u, c->scr, n3));
  launch_restrict27<double>(c->scr, n, c->det, c->s);
  return download(c, c->det, uhalf, n3 / 8);
}

int mmh_inject_f64(mmh_ctx* c, double* u, const double* uhalf, int n) {
  if (!c || !u || !uhalf) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  if (n < 8) return MMH_ERR_SIZE;
  i64 n3 = (i64)n * n * n;
  RET(upload(c, u, c->scr, n3));
  RET(upload(c, uhalf, c->det, n3 / 8));
  launch_prolong_add<double>(c->scr, c->det, n, c->s);
  return download(c, c->scr, u, n3);
}

int mmh_zerosum_f64(mmh_ctx* c, double* arr, int n) {
  if (!c || !arr) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  i64 n3 = (i64)n * n * n;
  RET(upload(c, arr, c->scr, n3));
  CK(cudaMemsetAsync(&c->sc->bad, 0, sizeof(int), c->s));
  RET(zerosum<double>(c, c->scr, n3));
  RET(download(c, c->scr, arr, n3));
  RET(pull_scal(c));
  return c->hsc->bad ? MMH_ERR_RANGE : MMH_OK;
}

int mmh_rgzerosum_f64(mmh_ctx* c, double* arr, const double* def, double dx, int n) {
  if (!c || !arr || !def) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  i64 n3 = (i64)n * n * n;
  int l = ilog2(c->n / n);
  RET(upload(c, arr, c->scr, n3));
  RET(upload(c, def, c->defl[l], n3));
  CK(cudaMemsetAsync(&c->sc->bad, 0, sizeof(int), c->s));
  RET(rgzerosum(c, c->scr, c->defl[l], n, dx));
  RET(download(c, c->scr, arr, n3));
  RET(pull_scal(c));
  return c->hsc->bad ? MMH_ERR_RANGE : MMH_OK;
}

int mmh_nsmooth_f64(mmh_ctx* c, double* a, int n) {
  if (!c || !a) return MMH_ERR_ARG;
  RET(check_cube(c, n, n, n));
  i64 n3 = (i64)n * n * n;
  RET(upload(c, a, c->scr, n3));
  // the context's form: the 27-point sum (FP64) or three axis passes (mixed)
  if (c->cfg.precision == MMH_MIXED)
    launch_smooth_sep(c->scr, n, c->det, c->s);
  else
    launch_smooth27<double>(c->scr, n, c->det, c->s);
  return download(c, c->det, a, n3);
}

int mmh_limiter_pass1_f64(mmh_ctx* c, double* tmp, const double* def, const double* rho, int n, double dtold,
                          double dtaumesh, unsigned char* maskx, unsigned char* maskc, mmh_diag* d) {
  if (!c || !tmp || !def || !rho) return MMH_ERR_ARG;
  if (n != c->n) return MMH_ERR_SIZE;
  i64 n3 = c->n3;
  RET(upload(c, tmp, c->scr, n3));
  RET(upload(c, def, c->def, n3));
  RET(upload(c, rho, c->rho, n3));
  uint8_t* dm = nullptr;
  CK(cudaMallocAsync((void**)&dm, 2 * n3, c->s));
  launch_lim_reset(&c->sc->lim, c->s);
  if (c->cfg.precision == MMH_MIXED) {
    // the mixed form screens with the float-float metric's det (the metric
    // of level 0 is rebuilt by the next solve)
    launch_metric_ff(c->def, c->rho, n, 1.0, c->h64.coef[0], c->h32.coef[0], c->det, c->s);
    c->coef_ff = true;
    c->levels_ready = false;
    launch_limiter_pass1_mixed(c->scr, c->def, c->rho, c->det, n, dtold, dtaumesh, &c->sc->lim, dm, dm + n3, c->s);
  } else {
    launch_limiter_pass1(c->scr, c->def, c->rho, n, dtold, dtaumesh, &c->sc->lim, dm, dm + n3, c->s);
  }
  RET(download(c, c->scr, tmp, n3));
  if (maskx) CK(cudaMemcpyAsync(maskx, dm, n3, cudaMemcpyDeviceToHost, c->s));
  if (maskc) CK(cudaMemcpyAsync(maskc, dm + n3, n3, cudaMemcpyDeviceToHost, c->s));
  CK(cudaFreeAsync(dm, c->s));
  RET(pull_scal(c));
  lim_to_diag(c->hsc->lim, d);
  return MMH_OK;
}

int mmh_limiter_mask_f64(mmh_ctx* c, double* defplim, const double* def, const double* defp, int n, double dtold,
                         unsigned char* mask, mmh_diag* d) {
  if (!c || !defplim || !def || !defp) return MMH_ERR_ARG;
  if (n != c->n) return MMH_ERR_SIZE;
  i64 n3 = c->n3;
  RET(upload(c, def, c->def, n3));
  RET(upload(c, defp, c->scr, n3));
  uint8_t* dm = nullptr;
  CK(cudaMallocAsync((void**)&dm, n3, c->s));
  launch_lim_reset(&c->sc->lim, c->s);
  if (c->cfg.precision == MMH_MIXED)
    launch_limiter_mask_mixed(c->defplim, c->def, c->scr, n, dtold, &c->sc->lim, dm, c->s);
  else
    launch_limiter_mask(c->defplim, c->def, c->scr, n, dtold, &c->sc->lim, dm, c->s);
  RET(download(c, c->defplim, defplim, n3));
  if (mask) CK(cudaMemcpyAsync(mask, dm, n3, cudaMemcpyDeviceToHost, c->s));
  CK(cudaFreeAsync(dm, c->s));
  RET(pull_scal(c));
  lim_to_diag(c->hsc->lim, d);
  return MMH_OK;
}

int mmh_limiter_poisson_f64(mmh_ctx* c, double* defp, const double* defplim, int n) {
  if (!c || !defp || !defplim) return MMH_ERR_ARG;
  if (n != c->n) return MMH_ERR_SIZE;
  i64 n3 = c->n3;
  RET(upload(c, defp, c->scr, n3));
  RET(upload(c, defplim, c->defplim, n3));
  // force the correction on: the caller asks for it explicitly
  launch_lim_reset(&c->sc->lim, c->s);
  unsigned long long one = 1;
  CK(cudaMemcpyAsync(&c->sc->lim.ncompress, &one, sizeof(one), cudaMemcpyHostToDevice, c->s));
  RET(limiter_poisson(c, c->scr, c->defplim));
  return download(c, c->scr, defp, n3);
}

int mmh_load_f64(mmh_ctx* c, const double* def, const double* u, int nfluid) {
  if (!c || !u) return MMH_ERR_ARG;
  if (def) RET(upload(c, def, c->def, c->n3));
  else CK(cudaMemsetAsync(c->def, 0, sizeof(double) * c->n3, c->s));
  return upload_density(c, u, nfluid, c->n3, c->rho);
}

int mmh_load_dev(mmh_ctx* c, const double* d_def, const double* d_rho) {
  if (!c || !d_rho) return MMH_ERR_ARG;
  if (d_def) CK(cudaMemcpyAsync(c->def, d_def, sizeof(double) * c->n3, cudaMemcpyDeviceToDevice, c->s));
  else CK(cudaMemsetAsync(c->def, 0, sizeof(double) * c->n3, c->s));
  CK(cudaMemcpyAsync(c->rho, d_rho, sizeof(double) * c->n3, cudaMemcpyDeviceToDevice, c->s));
  return MMH_OK;
}

int mmh_iterate(mmh_ctx* c, int niter, mmh_diag* d) {
  if (!c || niter < 0) return MMH_ERR_ARG;
  int st = MMH_OK;
  for (int it = 0; it < niter; ++it) {
    mmh_diag dd{};
    st = calcdefp_dev(c, 1.0, 1.0, c->mask(0), c->mask(1), c->mask(2), &dd);
    if (st != MMH_OK && st != MMH_ERR_DIVERGED) return st;
    launch_add(c->def, c->defp(), c->n3, c->s);
    RET(relaxing_dev(c, 1.0));
    dd.status = st;
    if (d) *d = dd;
  }
  CK(cudaStreamSynchronize(c->s));
  CK(cudaGetLastError());
  return st;
}

int mmh_store_f64(mmh_ctx* c, double* def, double* u, int nfluid) {
  if (!c) return MMH_ERR_ARG;
  if (def) RET(download(c, c->def, def, c->n3));
  if (u) {
    if (nfluid < 1 || nfluid > 5) return MMH_ERR_ARG;
    RET(download_density(c, c->rho, u, nfluid, c->n3));
  }
  return MMH_OK;
}

int mmh_outputs_f64(mmh_ctx* c, double* grad, double* delta) {
  if (!c) return MMH_ERR_ARG;
  // staged in the finest-level coefficient planes (6 n^3 doubles), which hold
  // nothing between solves and are not used by the spectral transforms
  double* o = c->h64.coef[0];
  int st = spectral_outputs(c, c->def, grad ? o : nullptr, delta ? o + 3 * c->n3 : nullptr);
  if (st == MMH_OK && grad) st = download(c, o, grad, 3 * c->n3);
  if (st == MMH_OK && delta) st = download(c, o + 3 * c->n3, delta, c->n3);
  return st;
}

int mmh_outputs_dev(mmh_ctx* c, double* d_grad, double* d_delta) {
  if (!c) return MMH_ERR_ARG;
  RET(spectral_outputs(c, c->def, d_grad, d_delta));
  return MMH_OK;
}

int mmh_state_dev(mmh_ctx* c, double** d_def, double** d_rho, double** d_defp) {
  if (!c) return MMH_ERR_ARG;
  if (d_def) *d_def = c->def;
  if (d_rho) *d_rho = c->rho;
  if (d_defp) *d_defp = c->defp();
  return MMH_OK;
}

}  // extern "C"
