// FP64 kernels of the MMH hot path.  Compiled with --fmad=false: every
// expression rounds as written, so results match the CPU restatement bit for
// bit (except where a libm function -- acos, cos -- is involved).
#include <algorithm>
#include <atomic>
#include <vector>

#include "mmh_ff.cuh"
#include "mmh_launch.cuh"
#include "mmh_pcg.cuh"
#include "mmh_phys.cuh"

namespace mmh {

static std::atomic<unsigned long long> g_launches{0};
void count_launch(int k) { g_launches.fetch_add((unsigned long long)k, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(); }

// ---------------------------------------------------------------------------
// kernel timing hooks
// ---------------------------------------------------------------------------
namespace {
struct Prof {
  int kind = 0;
  std::vector<cudaEvent_t> ev;
  int used = 0, dropped = 0;
  long long cells = 0;
};
Prof g_prof;
}  // namespace

bool prof_armed() { return g_prof.kind != 0; }

// Events are created in chunks as launches are timed (the pool grows with the
// launch count: a 512^3 reconstruction times ~2400 finest-level launches).
static bool prof_grow() {
  const size_t have = g_prof.ev.size();
  g_prof.ev.resize(have + 2 * 4096);
  for (size_t q = have; q < g_prof.ev.size(); ++q)
    if (cudaEventCreate(&g_prof.ev[q]) != cudaSuccess) {
      g_prof.ev.resize(q);
      g_prof.ev.resize(q & ~(size_t)1);
      return false;
    }
  return true;
}

int prof_start(int kind) {
  if (g_prof.ev.empty() && !prof_grow()) return -1;
  g_prof.kind = kind;
  g_prof.used = 0;
  g_prof.dropped = 0;
  g_prof.cells = 0;
  return 0;
}

// The armed kind may carry a grid filter in bits 12 and up (MMH_K_AT(n)):
// then only launches on that grid are timed.
static bool prof_match(int kind, int n) {
  if (g_prof.kind == 0 || kind != (g_prof.kind & 0xfff)) return false;
  const int at = g_prof.kind >> 12;
  return at == 0 || at == n;
}

void prof_begin(int kind, cudaStream_t s, i64 cells, int n) {
  if (!prof_match(kind, n)) return;
  if (g_prof.used >= (int)g_prof.ev.size() / 2 && !prof_grow()) {
    g_prof.dropped++;
    return;
  }
  cudaEventRecord(g_prof.ev[2 * g_prof.used], s);
  g_prof.cells += cells;
}

void prof_end(int kind, cudaStream_t s, int n) {
  if (!prof_match(kind, n)) return;
  if (g_prof.used >= (int)g_prof.ev.size() / 2) return;
  cudaEventRecord(g_prof.ev[2 * g_prof.used + 1], s);
  g_prof.used++;
}

int prof_stop(int* launches, double* ms, long long* cells) {
  double tot = 0.0;
  for (int q = 0; q < g_prof.used; ++q) {
    float m = 0.f;
    if (cudaEventSynchronize(g_prof.ev[2 * q + 1]) != cudaSuccess) return -1;
    if (cudaEventElapsedTime(&m, g_prof.ev[2 * q], g_prof.ev[2 * q + 1]) != cudaSuccess) return -1;
    tot += m;
  }
  if (launches) *launches = g_prof.used;
  if (ms) *ms = tot;
  if (cells) *cells = g_prof.cells;
  g_prof.kind = 0;
  return g_prof.dropped ? 1 : 0;
}

MMH_INSTANTIATE(double)

// ---------------------------------------------------------------------------
// scalar helpers
// ---------------------------------------------------------------------------
__global__ void k_fx_mean(const unsigned long long* acc, double count, double* out) {
  *out = fx_to(acc[0], acc[1]) / count;
}
__global__ void k_fx_ratio(const unsigned long long* num, const unsigned long long* den, double* out) {
  *out = fx_to(num[0], num[1]) / fx_to(den[0], den[1]);
}
void launch_fx_mean(const unsigned long long* acc, double count, double* out, cudaStream_t s) {
  k_fx_mean<<<1, 1, 0, s>>>(acc, count, out);
  count_launch();
}
void launch_fx_ratio(const unsigned long long* num, const unsigned long long* den, double* out, cudaStream_t s) {
  k_fx_ratio<<<1, 1, 0, s>>>(num, den, out);
  count_launch();
}

__global__ void k_guard(const unsigned long long* r1bits, const unsigned long long* errbits, double margin,
                        double floor_, int* flag, int* guards) {
  double r1 = __longlong_as_double((long long)*r1bits);
  double err = __longlong_as_double((long long)*errbits);
  int g = (err > r1 * margin && r1 > floor_) ? 1 : 0;
  *flag = g;
  if (g) *guards += 1;
}
void launch_guard(const unsigned long long* r1bits, const unsigned long long* errbits, double margin, double floor_,
                  int* flag, int* guards, cudaStream_t s) {
  k_guard<<<1, 1, 0, s>>>(r1bits, errbits, margin, floor_, flag, guards);
  count_launch();
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) b[t] = (float)a[t];
}
__global__ void k_f2d(const float* __restrict__ a, double* __restrict__ b, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) b[t] = (double)a[t];
}
__global__ void k_add_f2d(double* __restrict__ a, const float* __restrict__ b, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) a[t] = a[t] + (double)b[t];
}
__global__ void k_add(double* __restrict__ a, const double* __restrict__ b, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) a[t] = a[t] + b[t];
}
void launch_d2f(const double* a, float* b, i64 count, cudaStream_t s) {
  k_d2f<<<grid_of(count, kBlock), kBlock, 0, s>>>(a, b, count);
  count_launch();
}
void launch_f2d(const float* a, double* b, i64 count, cudaStream_t s) {
  k_f2d<<<grid_of(count, kBlock), kBlock, 0, s>>>(a, b, count);
  count_launch();
}
// ---------------------------------------------------------------------------
// Exact solve of the coarsest level (4^3 = 64 cells) in the mixed form's
// preconditioner, in FP64.  The level's operator L (the 19-point stencil of
// relaxplane, gauss1.f90:950-980, on the restricted metric) is singular with
// the constants as its null space and symmetric negative semi-definite, so
// A = L - beta 1 1^T (beta = mean |L_ii| / 64) is negative definite and
// z = A^-1 (r - mean r) is the zero-mean solution of L z = r - mean r: what
// the reference's 32 + 32 Gauss-Seidel sweeps and zerosum of mg4
// (multigrid.f90:94-121) converge to.  M = A^-1 is formed once per metric.
// ---------------------------------------------------------------------------
constexpr int kCoarseN = 64;
// L column by column (the operator applied to unit vectors, so it is exactly
// the smoother's operator), then an in-place Gauss-Jordan inversion (no
// pivoting: -A is symmetric positive definite).  One CTA of 256 threads.
__global__ void __launch_bounds__(256) k_coarse_inverse(const double* __restrict__ coef, double di2,
                                                        double* __restrict__ M) {
  constexpr int N = kCoarseN;
  __shared__ double A[N][N];
  __shared__ double e[N];
  __shared__ double colp[N];
  __shared__ double piv_s;
  const int tid = threadIdx.x;
  for (int j = 0; j < N; ++j) {
    if (tid < N) e[tid] = tid == j ? 1.0 : 0.0;
    __syncthreads();
    if (tid < N) {
      int i, jj, k;
      cell_of(tid, 4, i, jj, k);
      double tdiag, t1, t2;
      op_terms(e, coef, 4, (i64)N, i, jj, k, tdiag, t1, t2);
      A[tid][j] = (t1 + t2 + tdiag * e[tid]) * di2;
    }
    __syncthreads();
  }
  if (tid == 0) {
    double d = 0.0;
    for (int i = 0; i < N; ++i) d += fabs(A[i][i]);
    piv_s = d / N / N;  // beta
  }
  __syncthreads();
  const double beta = piv_s;
  for (int q = tid; q < N * N; q += blockDim.x) A[q / N][q % N] -= beta;
  __syncthreads();
  for (int p = 0; p < N; ++p) {
    if (tid < N) colp[tid] = A[tid][p];
    if (tid == 0) piv_s = 1.0 / A[p][p];
    __syncthreads();
    const double ip = piv_s;
    if (tid < N) A[p][tid] = (tid == p ? 1.0 : A[p][tid]) * ip;
    __syncthreads();
    for (int q = tid; q < N * N; q += blockDim.x) {
      const int i = q / N, j = q % N;
      if (i != p) A[i][j] = (j == p ? 0.0 : A[i][j]) - colp[i] * A[p][j];
    }
    __syncthreads();
  }
  for (int q = tid; q < N * N; q += blockDim.x) M[q] = A[q / N][q % N];
}

// z = M (r - mean r) on the 64 cells: one CTA of 64 threads, FP64 sums.
__global__ void __launch_bounds__(64) k_coarse_apply(const float* __restrict__ r, const double* __restrict__ M,
                                                     float* __restrict__ z) {
  constexpr int N = kCoarseN;
  __shared__ double b[N];
  __shared__ double wsum[2];
  const int tid = threadIdx.x;
  double v = (double)r[tid];
  double sv = v;
  for (int d = 16; d > 0; d >>= 1) sv += __shfl_down_sync(0xffffffffu, sv, d);
  if ((tid & 31) == 0) wsum[tid >> 5] = sv;
  __syncthreads();
  b[tid] = v - (wsum[0] + wsum[1]) / N;
  __syncthreads();
  double acc = 0.0;
#pragma unroll 8
  for (int j = 0; j < N; ++j) acc += M[tid * N + j] * b[j];
  z[tid] = (float)acc;
}

void launch_coarse_inverse(const double* coef, double dx, double* M, cudaStream_t s) {
  k_coarse_inverse<<<1, 256, 0, s>>>(coef, 1.0 / (dx * dx), M);
  count_launch();
}
void launch_coarse_apply(const float* r, const double* M, float* z, cudaStream_t s) {
  k_coarse_apply<<<1, kCoarseN, 0, s>>>(r, M, z);
  count_launch();
}

void launch_add_f2d(double* a, const float* b, i64 count, cudaStream_t s) {
  k_add_f2d<<<grid_of(count, kBlock), kBlock, 0, s>>>(a, b, count);
  count_launch();
}
void launch_add(double* a, const double* b, i64 count, cudaStream_t s) {
  k_add<<<grid_of(count, kBlock), kBlock, 0, s>>>(a, b, count);
  count_launch();
}

// ---------------------------------------------------------------------------
// calcdefp right-hand side and limiter
// ---------------------------------------------------------------------------
// tmp = clamp(1 - rho, +-2) / 30 / dtold (limiter.f90:153-166).  The mixed
// form multiplies by 1 / (30 dtold) instead of dividing twice (an FP64
// division is some ten FP64-pipe operations): within 2 ulp.
template <bool MIXED>
__global__ void k_calcdefp_rhs(double* __restrict__ tmp, const double* __restrict__ rho, i64 n3, double dtold,
                               double rcp) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  double t1 = 1.0 - rho[t];
  const double xhigh = 2.0;
  if (fabs(t1) > xhigh) t1 = t1 >= 0.0 ? xhigh : -xhigh;
  tmp[t] = MIXED ? t1 * rcp : t1 / 30.0 / dtold;
}
void launch_calcdefp_rhs(double* tmp, const double* rho, int n, double dtold, bool mixed, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  if (mixed)
    k_calcdefp_rhs<true><<<grid_of(n3, kBlock), kBlock, 0, s>>>(tmp, rho, n3, dtold, 1.0 / (30.0 * dtold));
  else
    k_calcdefp_rhs<false><<<grid_of(n3, kBlock), kBlock, 0, s>>>(tmp, rho, n3, dtold, 0.0);
  count_launch();
}

// Block reduction of a uint64: op 0 = sum, 1 = max, 2 = min.  Result valid in
// thread 0; every thread of the block must call it.
__device__ __forceinline__ unsigned long long block_u64(unsigned long long v, unsigned long long* buf, int op) {
  for (int d = 16; d > 0; d >>= 1) {
    unsigned long long o = __shfl_down_sync(0xffffffffu, v, d);
    v = op == 0 ? v + o : (op == 1 ? (o > v ? o : v) : (o < v ? o : v));
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) buf[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = buf[0];
    for (int q = 1; q < nw; ++q) {
      unsigned long long o = buf[q];
      v = op == 0 ? v + o : (op == 1 ? (o > v ? o : v) : (o < v ? o : v));
    }
  }
  return v;
}

// Pass 1 of the limiter at one cell in FP64 (limiter.f90:268-372), the
// reference's order: det from the Hessian of def, rho^2/det for rho2, the
// expansion clamp (det > 10), the compression test, the flux clamps.
struct Pass1Cell {
  double eflux, det;
  __int128 r2;
  bool bad;
  uint8_t mx, mc;
};
__device__ __forceinline__ Pass1Cell pass1_cell_fp64(const double* __restrict__ tmp, const double* __restrict__ def,
                                                     const double* __restrict__ rho, int n, i64 t, double dtold,
                                                     double dtaumesh, double cmpmaxglobal) {
  Pass1Cell o;
  int i, j, km;
  cell_of(t, n, i, j, km);
  int k = wp(km, n);
  LimM m = lim_hess_det(def, n, i, j, k);
  o.det = m.det;
  double rl = rho[t];
  double q = rl * rl / o.det;
  o.bad = false;
  o.r2 = 0;
  if (!(fabs(q) < 4294967296.0)) o.bad = true;
  else o.r2 = fx_of(q);
  // momentum-flux divergence of a state at rest is zero (u(2:4) = 0)
  double eflux = 0.0 + tmp[t];
  o.mx = 0;
  o.mc = 0;
  const double densinit = 1.0;
  if (o.det > 10.0 * densinit) {
    eflux = -2.0 * fabs(eflux);
    o.mx = 1;
  }
  // Only the sign of tlim is used here.  When the Gershgorin lower bound of
  // the smallest eigenvalue of C = I + Hess(def) exceeds 1/cmpmax by a wide
  // margin, tlim < 0 for certain and the trigonometric evaluation is skipped.
  double c11 = 1.0 + m.phixx, c22 = 1.0 + m.phiyy, c33 = 1.0 + m.phizz;
  double g = fmin(fmin(c11 - fabs(m.phixy) - fabs(m.phixz), c22 - fabs(m.phixy) - fabs(m.phiyz)),
                  c33 - fabs(m.phixz) - fabs(m.phiyz));
  double cmpmax = cmpmaxglobal * 1.0;
  if (!(g > 1.0 / cmpmax + 1e-6)) {
    double compression = compression_of(c11, m.phixy, m.phixz, c22, m.phiyz, c33);
    double tlim = 3.0 * (1.0 / cmpmax - 1.0 / compression) / dtold;
    if (tlim > 0.0) {
      eflux = fmax(0.0, eflux);
      o.mc = 1;
    }
  }
  eflux = fmin(1.0 / dtaumesh, eflux);
  eflux = fmax(-1.0 / dtaumesh, eflux);
  o.eflux = eflux;
  return o;
}

// The statistics of pass 1: one block reduction and one atomic per block and
// statistic.  Every thread of the block calls it.
__device__ __forceinline__ void pass1_commit(LimDev* st, unsigned long long nexp, unsigned long long dmax,
                                             unsigned long long dmin, unsigned long long fmx, unsigned long long fmn,
                                             bool bad, __int128 r2, unsigned long long* s_buf) {
  unsigned long long v;
  v = block_u64(nexp, s_buf, 0);
  if (threadIdx.x == 0 && v) atomicAdd(&st->nexpand, v);
  v = block_u64(dmax, s_buf, 1);
  if (threadIdx.x == 0) atomicMax(&st->detmax, v);
  v = block_u64(dmin, s_buf, 2);
  if (threadIdx.x == 0) atomicMin(&st->detmin, v);
  v = block_u64(fmx, s_buf, 1);
  if (threadIdx.x == 0) atomicMax(&st->fluxmax, v);
  v = block_u64(fmn, s_buf, 2);
  if (threadIdx.x == 0) atomicMin(&st->fluxmin, v);
  if (bad) atomicOr(&st->flag, 2);
  fx_block_commit(r2, st->rho2);
}

__global__ void k_limiter_pass1(double* __restrict__ tmp, const double* __restrict__ def,
                                const double* __restrict__ rho, int n, double dtold, double dtaumesh,
                                double cmpmaxglobal, LimDev* st, uint8_t* __restrict__ maskx,
                                uint8_t* __restrict__ maskc) {
  __shared__ unsigned long long s_buf[32];
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  __int128 r2 = 0;
  bool bad = false;
  unsigned long long nexp = 0;
  unsigned long long dmax = ord_of(0.0), dmin = ord_of(1.0), fmx = ord_of(0.0), fmn = ord_of(0.0);
  if (t < n3) {
    const Pass1Cell o = pass1_cell_fp64(tmp, def, rho, n, t, dtold, dtaumesh, cmpmaxglobal);
    tmp[t] = o.eflux;
    r2 = o.r2;
    bad = o.bad;
    nexp = o.mx;
    dmax = dmin = ord_of(o.det);
    fmx = ord_of(fmax(0.0, o.eflux * dtold));
    fmn = ord_of(fmin(0.0, o.eflux * dtold));
    if (maskx) maskx[t] = o.mx;
    if (maskc) maskc[t] = o.mc;
  }
  pass1_commit(st, nexp, dmax, dmin, fmx, fmn, bad, r2, s_buf);
}

// Pass 1 in the mixed form: the same decisions and fluxes as the FP64 pass,
// with FP64 arithmetic only where a decision is close.  Every cell is first
// screened in FP32 from its def samples truncated to floats (bit operations):
// each sample is within 2^-23 |x| + 2^-126 of its double, so every entry of
// C = I + Hess(def) is within E = 2^-18 max|sample| + 2^-20 (1 + sum |C_ij|)
// of the FP64 one (about 4x the worst case of truncation and rounding), and
// the Gershgorin bound g within 3E.  A cell with g - 3E above the FP64
// shortcut's threshold skips the compression test in the FP64 pass too, so
// its mc is 0; a cell whose float-float det(A) (detff, from the metric of the
// same def: within 2^-40 (1 + max|sample|) (1 + sum|C_ij|)^2 of the FP64 det)
// is that far from 10 has the FP64 expansion decision.  Cells where either
// decision is close take pass1_cell_fp64, compacted so whole warps evaluate
// it.  The flux is the FP64 pass's: the clamps only select values, -2|e| is
// exact.  The statistics of the screened cells come from detff (det min and
// max) and rho^2 / det in float-float (rho2): not bit-matched.
__global__ void __launch_bounds__(256) k_limiter_pass1_mixed(double* __restrict__ tmp, const double* __restrict__ def,
                                                             const double* __restrict__ rho,
                                                             const double* __restrict__ detff, int n, double dtold,
                                                             double dtaumesh, double lim, double cmpmaxglobal,
                                                             float gthr,
                                                             LimDev* st, uint8_t* __restrict__ maskx,
                                                             uint8_t* __restrict__ maskc) {
  __shared__ unsigned long long s_buf[32];
  __shared__ int s_list[256];
  __shared__ int s_cnt;
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  __int128 r2 = 0;
  bool bad = false;
  unsigned long long nexp = 0;
  unsigned long long dmax = ord_of(0.0), dmin = ord_of(1.0), fmx = ord_of(0.0), fmn = ord_of(0.0);
  const unsigned long long oL = ord_of(lim), onL = ord_of(-lim);  // lim = 1 / dtaumesh
  if (t < n3) {
    int i, j, km;
    cell_of(t, n, i, j, km);
    const int k = wp(km, n);
    const int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), kq = wm(k, n);
    bool ok = true;
    float M = 0.0f;
    auto S = [&](int x, int y, int z) {
      float f;
      ok = f32_trunc_bits(def[IDX(x, y, z, n)], f) && ok;
      M = fmaxf(M, fabsf(f));
      return f;
    };
    const float c0 = S(i, j, k);
    const float hxx = (S(ip, j, k) - c0) + (S(im, j, k) - c0);
    const float hyy = (S(i, jp, k) - c0) + (S(i, jm, k) - c0);
    const float hzz = (S(i, j, kp) - c0) + (S(i, j, kq) - c0);
    const float hxy = ((S(ip, jp, k) - S(im, jp, k)) - (S(ip, jm, k) - S(im, jm, k))) * 0.25f;
    const float hyz = ((S(i, jp, kp) - S(i, jp, kq)) - (S(i, jm, kp) - S(i, jm, kq))) * 0.25f;
    const float hxz = ((S(ip, j, kp) - S(im, j, kp)) - (S(ip, j, kq) - S(im, j, kq))) * 0.25f;
    const float c11 = 1.0f + hxx, c22 = 1.0f + hyy, c33 = 1.0f + hzz;
    const float sc = 1.0f + fabsf(c11) + fabsf(c22) + fabsf(c33) + 2.0f * (fabsf(hxy) + fabsf(hyz) + fabsf(hxz));
    const float E = 3.814697265625e-6f * M + 9.5367431640625e-7f * sc;  // 2^-18 M + 2^-20 sc
    const float g = fminf(fminf(c11 - fabsf(hxy) - fabsf(hxz), c22 - fabsf(hxy) - fabsf(hyz)),
                          c33 - fabsf(hxz) - fabsf(hyz));
    const bool gsure = g - 3.0f * E > gthr;
    // pass 1 evaluates the metric at (i, j, k = km + 1) for the cell (i, j, km)
    const double det = detff[IDX(i, j, k, n)];
    float d32;
    ok = f32_trunc_bits(det, d32) && ok;
    const float Ed = 9.094947017729282e-13f * (1.0f + M) * sc * sc + 4.76837158203125e-6f * (1.0f + fabsf(d32));
    const bool dsure = fabsf(d32 - 10.0f) > Ed;  // 2^-40 (1+M) sc^2 + 2^-21 (1 + |det|)
    if (ok && gsure && dsure) {
      const uint8_t mx = d32 > 10.0f;
      // 0.0 + e: -0 becomes +0, everything else is kept
      unsigned long long eb = (unsigned long long)__double_as_longlong(tmp[t]);
      if (eb == 0x8000000000000000ull) eb = 0;
      double e = __longlong_as_double((long long)eb);
      if (mx) e = -2.0 * fabs(e);
      // fmin(1/dtaumesh, e), then fmax(-1/dtaumesh, .): a NaN flux becomes 1/dtaumesh
      const unsigned long long ebits = (unsigned long long)__double_as_longlong(e);
      const bool nan = ((ebits >> 52) & 0x7ffull) == 0x7ffull && (ebits & 0xfffffffffffffull);
      unsigned long long oe = ord_of(e);
      if (nan || oe > oL) oe = oL;
      if (oe < onL) oe = onL;
      e = from_ord(oe);
      tmp[t] = e;
      if (maskx) maskx[t] = mx;
      if (maskc) maskc[t] = 0;
      nexp = mx;
      dmax = dmin = ord_of(det);
      const double ed = dtold == 1.0 ? e : e * dtold;
      const unsigned long long oed = ord_of(ed);
      fmx = oed > ord_of(0.0) ? oed : ord_of(0.0);
      fmn = oed < ord_of(0.0) ? oed : ord_of(0.0);
      // rho^2 / det in float-float, into the exact fixed-point sum
      const FF rl = ff_of_bits(rho[t]);
      const FF qq = ff_div(ff_mul(rl, rl), ff_of_bits(det));
      if (!(fabsf(qq.hi) < 4294967296.0f)) bad = true;
      else r2 = fx_of_f(qq.hi) + fx_of_f(qq.lo);
    } else {
      s_list[atomicAdd(&s_cnt, 1)] = threadIdx.x;
    }
  }
  __syncthreads();
  const int ncand = s_cnt;
  for (int q = threadIdx.x; q < ncand; q += blockDim.x) {
    const i64 tt = (i64)blockIdx.x * blockDim.x + s_list[q];
    const Pass1Cell o = pass1_cell_fp64(tmp, def, rho, n, tt, dtold, dtaumesh, cmpmaxglobal);
    tmp[tt] = o.eflux;
    if (maskx) maskx[tt] = o.mx;
    if (maskc) maskc[tt] = o.mc;
    nexp += o.mx;
    const unsigned long long od = ord_of(o.det);
    dmax = od > dmax ? od : dmax;
    dmin = od < dmin ? od : dmin;
    const unsigned long long ox = ord_of(fmax(0.0, o.eflux * dtold)), on = ord_of(fmin(0.0, o.eflux * dtold));
    fmx = ox > fmx ? ox : fmx;
    fmn = on < fmn ? on : fmn;
    bad = bad || o.bad;
    r2 += o.r2;
  }
  pass1_commit(st, nexp, dmax, dmin, fmx, fmn, bad, r2, s_buf);
}

void launch_limiter_pass1(double* tmp, const double* def, const double* rho, int n, double dtold, double dtaumesh,
                          LimDev* st, uint8_t* maskx, uint8_t* maskc, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_limiter_pass1<<<grid_of(n3, kBlock), kBlock, 0, s>>>(tmp, def, rho, n, dtold, dtaumesh, 10.0, st, maskx, maskc);
  count_launch();
}
void launch_limiter_pass1_mixed(double* tmp, const double* def, const double* rho, const double* detff, int n,
                                double dtold, double dtaumesh, LimDev* st, uint8_t* maskx, uint8_t* maskc,
                                cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  // a float at or above the FP64 shortcut's threshold 1/cmpmax + 1e-6
  const double thr = 1.0 / 10.0 + 1e-6;
  float gthr = (float)thr;
  if ((double)gthr < thr) gthr = nextafterf(gthr, 1.0f);
  k_limiter_pass1_mixed<<<grid_of(n3, kBlock), kBlock, 0, s>>>(tmp, def, rho, detff, n, dtold, dtaumesh,
                                                               1.0 / dtaumesh, 10.0, gthr, st, maskx, maskc);
  count_launch();
}

// Bounds of the smallest eigenvalue that compression_of computes, from the
// values it computes first (mu = trace/3, am): every root r_i = am*cos(.)
// lies in [-am, am], so min_i (r_i + mu) >= mu - am = lo.  The root through
// theta + 2pi/3 has cos <= -1/2, so the minimum is <= mu - am/2 < hi.  The
// bounds come from FP32 arithmetic on the FP64 entries rounded once, widened
// by 1e-5 (|mu| + am): FP32 rounding moves mu and am by a few 1e-7 of
// |mu| + am, so lo stays below and hi above the FP64 formula's smallest
// eigenvalue.  They only decide which cells may skip the exact FP64 test; the
// cells that take it, and therefore every output, are unchanged.
__device__ __forceinline__ void compression_bounds_f(float c11, float c12, float c13, float c22, float c23, float c33,
                                                     float& lo, float& hi) {
  const float mu = (c11 + c22 + c33) * (1.0f / 3.0f);
  const float d11 = c11 - mu, d22 = c22 - mu;
  const float a = d11 * d11 + c12 * c12 + c13 * c13 + d11 * d22 + d22 * d22 + c23 * c23;
  const float am = 2.0f * sqrtf(fabsf(a) * (1.0f / 3.0f));
  const float margin = 1e-5f * (fabsf(mu) + am) + 1e-30f;
  lo = mu - am - margin;
  hi = (mu - 0.49f * am) + margin;
}
__device__ __forceinline__ void compression_bounds32(const double* c, double& lo, double& hi) {
  float l, h;
  compression_bounds_f((float)c[0], (float)c[1], (float)c[2], (float)c[3], (float)c[4], (float)c[5], l, h);
  lo = (double)l;
  hi = (double)h;
}

// C = I + Hess(def + dtold defp) at cell t in FP64, the reference's order
// (limiter.f90:498-520): c = (C11, C12, C13, C22, C23, C33).
__device__ __forceinline__ void mask_c64(const double* __restrict__ def, const double* __restrict__ defp, int n, i64 t,
                                         double dtold, double* c) {
  int i, j, k;
  cell_of(t, n, i, j, k);
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
#define P_(x, y, z) defp[IDX(x, y, z, n)]
#define D_(x, y, z) def[IDX(x, y, z, n)]
  double phixx = (P_(ip, j, k) - 2.0 * P_(i, j, k) + P_(im, j, k)) * dtold;
  double phiyy = (P_(i, jp, k) - 2.0 * P_(i, j, k) + P_(i, jm, k)) * dtold;
  double phizz = (P_(i, j, kp) - 2.0 * P_(i, j, k) + P_(i, j, km)) * dtold;
  double phixy = (P_(ip, jp, k) - P_(im, jp, k) - P_(ip, jm, k) + P_(im, jm, k)) * 0.25 * dtold;
  double phiyz = (P_(i, jp, kp) - P_(i, jp, km) - P_(i, jm, kp) + P_(i, jm, km)) * 0.25 * dtold;
  double phixz = (P_(ip, j, kp) - P_(im, j, kp) - P_(ip, j, km) + P_(im, j, km)) * 0.25 * dtold;
  phixx = phixx + (D_(ip, j, k) - 2.0 * D_(i, j, k) + D_(im, j, k));
  phiyy = phiyy + (D_(i, jp, k) - 2.0 * D_(i, j, k) + D_(i, jm, k));
  phizz = phizz + (D_(i, j, kp) - 2.0 * D_(i, j, k) + D_(i, j, km));
  phixy = phixy + (D_(ip, jp, k) - D_(im, jp, k) - D_(ip, jm, k) + D_(im, jm, k)) * 0.25;
  phiyz = phiyz + (D_(i, jp, kp) - D_(i, jp, km) - D_(i, jm, kp) + D_(i, jm, km)) * 0.25;
  phixz = phixz + (D_(ip, j, kp) - D_(im, j, kp) - D_(ip, j, km) + D_(im, j, km)) * 0.25;
#undef P_
#undef D_
  c[0] = 1.0 + phixx; c[1] = phixy; c[2] = phixz; c[3] = 1.0 + phiyy; c[4] = phiyz; c[5] = 1.0 + phizz;
}

// Final compression test (limiter.f90:498-533): defplim = tlim where tlim > 0,
// the count of such cells, and cmax = max compression.  The trigonometric
// evaluation is exact only where it can matter.  A cell with lo > 1/cmpmax
// has tlim < 0 for certain.  Such a cell can be skipped for cmax too when its
// upper bound 1/lo is below the compression of a cell that is evaluated: the
// block's cell with the smallest hi, or any cell already folded into the
// global maximum.  The cells left are compacted so whole warps evaluate them.
__global__ void __launch_bounds__(256) k_limiter_mask(double* __restrict__ defplim, const double* __restrict__ def,
                                                      const double* __restrict__ defp, int n, double dtold,
                                                      double cmpmaxglobal, LimDev* st, uint8_t* __restrict__ mask) {
  __shared__ double s_c[6][256];
  __shared__ int s_list[256];
  __shared__ int s_cnt;
  __shared__ unsigned long long s_buf[32];
  __shared__ unsigned long long s_lam;
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (threadIdx.x == 0) s_cnt = 0;
  const double cmpmax = cmpmaxglobal * 1.0;
  double c[6] = {0, 0, 0, 0, 0, 0};
  double lo = 0.0, hi = 0.0;
  if (t < n3) {
    mask_c64(def, defp, n, t, dtold, c);
    compression_bounds32(c, lo, hi);
  }
  const bool pd = t < n3 && lo > 0.0;
  // smallest upper bound of the block's positive definite cells
  unsigned long long lam = block_u64(pd ? ord_of(hi) : ord_of(INFINITY), s_buf, 2);
  if (threadIdx.x == 0) s_lam = lam;
  __syncthreads();
  const double lam_b = from_ord(s_lam);
  // the largest compression folded in so far (exact values of evaluated cells)
  const double tg = from_ord(*(volatile unsigned long long*)&st->cmax);
  const double lam_g = tg > 0.0 ? (1.0 / tg) * (1.0 + 1e-15) : INFINITY;
  const bool skip = pd && dtold > 0.0 && lo > (1.0 / cmpmax) * (1.0 + 1e-12) && (lo > lam_b || lo >= lam_g);
  if (t < n3) {
    if (skip) {
      defplim[t] = 0.0;
      if (mask) mask[t] = 0;
    } else {
      int pos = atomicAdd(&s_cnt, 1);
      s_list[pos] = threadIdx.x;
#pragma unroll
      for (int q = 0; q < 6; ++q) s_c[q][pos] = c[q];
    }
  }
  __syncthreads();
  unsigned long long cnt = 0, cm = ord_of(0.0);
  const int ncand = s_cnt;
  for (int q = threadIdx.x; q < ncand; q += blockDim.x) {
    const i64 tt = (i64)blockIdx.x * blockDim.x + s_list[q];
    double compression = compression_of(s_c[0][q], s_c[1][q], s_c[2][q], s_c[3][q], s_c[4][q], s_c[5][q]);
    double tlim = 3.0 * (1.0 / cmpmax - 1.0 / compression) / dtold;
    unsigned long long o = ord_of(fmax(0.0, compression));
    cm = o > cm ? o : cm;
    double v = 0.0;
    uint8_t mk = 0;
    if (tlim > 0.0) {
      cnt += 1;
      v = tlim;
      mk = 1;
    }
    defplim[tt] = v;
    if (mask) mask[tt] = mk;
  }
  unsigned long long r = block_u64(cnt, s_buf, 0);
  if (threadIdx.x == 0 && r) atomicAdd(&st->ncompress, r);
  r = block_u64(cm, s_buf, 1);
  if (threadIdx.x == 0) atomicMax(&st->cmax, r);
}

void launch_limiter_mask(double* defplim, const double* def, const double* defp, int n, double dtold, LimDev* st,
                         uint8_t* mask, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_limiter_mask<<<grid_of(n3, kBlock), kBlock, 0, s>>>(defplim, def, defp, n, dtold, 10.0, st, mask);
  count_launch();
}

// The final compression test in the mixed form: the same outputs as
// k_limiter_mask, with FP64 arithmetic only for the cells that may matter.
// The bounds lo and hi come from C in FP32, formed from the samples of def
// and defp truncated to floats (bit operations): every entry is within E =
// 2^-18 (max|def sample| + |dtold| max|defp sample|) + 2^-20 (1 + sum|C_ij|)
// of the FP64 one (about 4x the worst case of truncation and rounding), so
// the smallest eigenvalue within 3E, by which lo and hi are widened.  The
// cells that are not skipped form C in FP64 (mask_c64) after compaction.
// inv_tight = (1/cmpmax)(1 + 1e-12), formed on the host.
__global__ void __launch_bounds__(256) k_limiter_mask_mixed(double* __restrict__ defplim,
                                                            const double* __restrict__ def,
                                                            const double* __restrict__ defp, int n, double dtold,
                                                            double cmpmaxglobal, double inv_tight, LimDev* st,
                                                            uint8_t* __restrict__ mask) {
  __shared__ int s_list[256];
  __shared__ int s_cnt;
  __shared__ unsigned long long s_buf[32];
  __shared__ unsigned long long s_lam;
  __shared__ double s_lam_g;
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (threadIdx.x == 0) {
    s_cnt = 0;
    // the largest compression folded in so far (exact values of evaluated cells)
    const double tg = from_ord(*(volatile unsigned long long*)&st->cmax);
    s_lam_g = tg > 0.0 ? (1.0 / tg) * (1.0 + 1e-15) : INFINITY;
  }
  const double cmpmax = cmpmaxglobal * 1.0;
  const float dtf = (float)dtold;
  float lo = 0.0f, hi = 0.0f;
  bool ok = true;
  if (t < n3) {
    int i, j, k;
    cell_of(t, n, i, j, k);
    const int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
    float Md = 0.0f, Mp = 0.0f;
    auto D = [&](int x, int y, int z) {
      float f;
      ok = f32_trunc_bits(def[IDX(x, y, z, n)], f) && ok;
      Md = fmaxf(Md, fabsf(f));
      return f;
    };
    auto P = [&](int x, int y, int z) {
      float f;
      ok = f32_trunc_bits(defp[IDX(x, y, z, n)], f) && ok;
      Mp = fmaxf(Mp, fabsf(f));
      return f;
    };
    const float pc = P(i, j, k), dc = D(i, j, k);
    const float pxx = ((P(ip, j, k) - pc) + (P(im, j, k) - pc)) * dtf;
    const float pyy = ((P(i, jp, k) - pc) + (P(i, jm, k) - pc)) * dtf;
    const float pzz = ((P(i, j, kp) - pc) + (P(i, j, km) - pc)) * dtf;
    const float pxy = ((P(ip, jp, k) - P(im, jp, k)) - (P(ip, jm, k) - P(im, jm, k))) * 0.25f * dtf;
    const float pyz = ((P(i, jp, kp) - P(i, jp, km)) - (P(i, jm, kp) - P(i, jm, km))) * 0.25f * dtf;
    const float pxz = ((P(ip, j, kp) - P(im, j, kp)) - (P(ip, j, km) - P(im, j, km))) * 0.25f * dtf;
    const float c11 = 1.0f + (pxx + ((D(ip, j, k) - dc) + (D(im, j, k) - dc)));
    const float c22 = 1.0f + (pyy + ((D(i, jp, k) - dc) + (D(i, jm, k) - dc)));
    const float c33 = 1.0f + (pzz + ((D(i, j, kp) - dc) + (D(i, j, km) - dc)));
    const float c12 = pxy + ((D(ip, jp, k) - D(im, jp, k)) - (D(ip, jm, k) - D(im, jm, k))) * 0.25f;
    const float c23 = pyz + ((D(i, jp, kp) - D(i, jp, km)) - (D(i, jm, kp) - D(i, jm, km))) * 0.25f;
    const float c13 = pxz + ((D(ip, j, kp) - D(im, j, kp)) - (D(ip, j, km) - D(im, j, km))) * 0.25f;
    const float sc = 1.0f + fabsf(c11) + fabsf(c22) + fabsf(c33) + 2.0f * (fabsf(c12) + fabsf(c23) + fabsf(c13));
    const float E = 3.814697265625e-6f * (Md + fabsf(dtf) * Mp) + 9.5367431640625e-7f * sc;  // 2^-18, 2^-20
    compression_bounds_f(c11, c12, c13, c22, c23, c33, lo, hi);
    lo -= 3.0f * E;
    hi += 3.0f * E;
  }
  const bool pd = t < n3 && ok && lo > 0.0f;
  // smallest upper bound of the block's positive definite cells
  unsigned long long lam = block_u64(pd ? ord_of((double)hi) : ord_of(INFINITY), s_buf, 2);
  if (threadIdx.x == 0) s_lam = lam;
  __syncthreads();
  const double lam_b = from_ord(s_lam), lam_g = s_lam_g, lod = (double)lo;
  const bool skip = pd && dtold > 0.0 && lod > inv_tight && (lod > lam_b || lod >= lam_g);
  if (t < n3) {
    if (skip) {
      defplim[t] = 0.0;
      if (mask) mask[t] = 0;
    } else {
      s_list[atomicAdd(&s_cnt, 1)] = threadIdx.x;
    }
  }
  __syncthreads();
  unsigned long long cnt = 0, cm = ord_of(0.0);
  const int ncand = s_cnt;
  for (int q = threadIdx.x; q < ncand; q += blockDim.x) {
    const i64 tt = (i64)blockIdx.x * blockDim.x + s_list[q];
    double c[6];
    mask_c64(def, defp, n, tt, dtold, c);
    double compression = compression_of(c[0], c[1], c[2], c[3], c[4], c[5]);
    double tlim = 3.0 * (1.0 / cmpmax - 1.0 / compression) / dtold;
    unsigned long long o = ord_of(fmax(0.0, compression));
    cm = o > cm ? o : cm;
    double v = 0.0;
    uint8_t mk = 0;
    if (tlim > 0.0) {
      cnt += 1;
      v = tlim;
      mk = 1;
    }
    defplim[tt] = v;
    if (mask) mask[tt] = mk;
  }
  unsigned long long r = block_u64(cnt, s_buf, 0);
  if (threadIdx.x == 0 && r) atomicAdd(&st->ncompress, r);
  r = block_u64(cm, s_buf, 1);
  if (threadIdx.x == 0) atomicMax(&st->cmax, r);
}
void launch_limiter_mask_mixed(double* defplim, const double* def, const double* defp, int n, double dtold, LimDev* st,
                               uint8_t* mask, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_limiter_mask_mixed<<<grid_of(n3, kBlock), kBlock, 0, s>>>(defplim, def, defp, n, dtold, 10.0,
                                                              (1.0 / 10.0) * (1.0 + 1e-12), st, mask);
  count_launch();
}

__global__ void k_lim_reset(LimDev* st) {
  st->nexpand = 0;
  st->ncompress = 0;
  st->detmax = ord_of(0.0);
  st->detmin = ord_of(1.0);
  st->fluxmax = ord_of(0.0);
  st->fluxmin = ord_of(0.0);
  st->cmax = ord_of(0.0);
  st->rho2[0] = 0;
  st->rho2[1] = 0;
  st->flag = 0;
}
// Diagnostics of main.f90's iteration loop (main.f90:97-105, 115-117, 181-182):
// exact sums of def, def^2, defp^2, rho and (rho-1)^2, the extrema of rho and
// the count of rho < 0.  st is zeroed by the caller except rmin (all ones).
__global__ void k_state_stats(const double* __restrict__ def, const double* __restrict__ defp,
                              const double* __restrict__ rho, i64 n3, StatsDev* st) {
  __int128 s[5] = {0, 0, 0, 0, 0};
  bool bad = false;
  unsigned long long neg = 0, omin = ~0ull, omax = 0;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < n3; t += (i64)gridDim.x * blockDim.x) {
    double d = def[t], p = defp[t], r = rho[t];
    double v[5] = {d, d * d, p * p, r, (r - 1.0) * (r - 1.0)};
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      if (!(fabs(v[q]) < 4294967296.0)) bad = true;
      else s[q] += fx_of(v[q]);
    }
    if (r < 0.0) ++neg;
    unsigned long long o = ord_of(r);
    omin = o < omin ? o : omin;
    omax = o > omax ? o : omax;
  }
  __shared__ unsigned long long s_buf[32];
  unsigned long long v;
  v = block_u64(neg, s_buf, 0);
  if (threadIdx.x == 0 && v) atomicAdd(&st->nneg, v);
  v = block_u64(omin, s_buf, 2);
  if (threadIdx.x == 0) atomicMin(&st->rmin, v);
  v = block_u64(omax, s_buf, 1);
  if (threadIdx.x == 0) atomicMax(&st->rmax, v);
  if (bad) atomicOr(&st->flag, 1);
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    __syncthreads();
    fx_block_commit(s[q], st->acc[q]);
  }
}
void launch_state_stats(const double* def, const double* defp, const double* rho, i64 n3, StatsDev* st,
                        cudaStream_t s) {
  i64 blocks = std::min<i64>((n3 + kBlock - 1) / kBlock, 152 * 8);
  k_state_stats<<<(unsigned)blocks, kBlock, 0, s>>>(def, defp, rho, n3, st);
  count_launch();
}

// Binned power spectrum of the half spectrum A (cuFFT D2Z layout, (n/2+1) x n
// x n, x fastest): |A|^2 (or Re(A conj(B))) * scale over the modes of each
// |k| bin.  Bin b holds e2[b] <= |k|^2 < e2[b+1] (squared edges, exact where
// an edge is a power of two); half-spectrum modes with 0 < kx < n/2 stand for
// two modes.  Per-block fixed-point histograms in shared memory, committed
// with 128-bit carries: the sums are exact and independent of order.
__device__ __forceinline__ void fx_atomic_add(unsigned long long* acc, __int128 v) {
  unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)((unsigned __int128)v >> 64);
  unsigned long long old = atomicAdd(&acc[0], lo);
  atomicAdd(&acc[1], hi + ((old + lo < old) ? 1ull : 0ull));
}
__global__ void __launch_bounds__(256) k_power_bins(const double2* __restrict__ A, const double2* __restrict__ B,
                                                    int n, int nb, const double* __restrict__ e2, double scale,
                                                    PowDev* acc) {
  __shared__ unsigned long long sp[kPowMaxBins][2], sk[kPowMaxBins][2], sc[kPowMaxBins];
  __shared__ double se2[kPowMaxBins + 1];
  for (int q = threadIdx.x; q < kPowMaxBins; q += blockDim.x) {
    sp[q][0] = sp[q][1] = sk[q][0] = sk[q][1] = sc[q] = 0ull;
  }
  for (int q = threadIdx.x; q <= nb; q += blockDim.x) se2[q] = e2[q];
  __syncthreads();
  const int nh = n / 2 + 1;
  const i64 tot = (i64)nh * n * n;
  bool bad = false;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (i64)gridDim.x * blockDim.x) {
    int i = (int)(t % nh);
    i64 r = t / nh;
    int j = (int)(r % n), k = (int)(r / n);
    long long ky = j <= n / 2 ? j : j - n, kz = k <= n / 2 ? k : k - n;
    long long K2 = (long long)i * i + ky * ky + kz * kz;
    double kk2 = (double)K2;
    if (K2 == 0 || kk2 < se2[0] || !(kk2 < se2[nb])) continue;
    int lo = 0, hi = nb - 1;  // the largest b with se2[b] <= kk2
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (se2[mid] <= kk2) lo = mid;
      else hi = mid - 1;
    }
    const double w = (i == 0 || 2 * i == n) ? 1.0 : 2.0;
    double2 a = A[t];
    double p = B ? (a.x * B[t].x + a.y * B[t].y) : (a.x * a.x + a.y * a.y);
    double pv = w * (p * scale), kv = w * sqrt(kk2);
    if (!(fabs(pv) < 4294967296.0) || !(kv < 4294967296.0)) {
      bad = true;
      continue;
    }
    fx_atomic_add(sp[lo], fx_of(pv));
    fx_atomic_add(sk[lo], fx_of(kv));
    atomicAdd(&sc[lo], (unsigned long long)w);
  }
  if (bad) atomicOr(&acc->flag, 1);
  __syncthreads();
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    if (sc[q] == 0) continue;
    __int128 vp = (__int128)(((unsigned __int128)sp[q][1] << 64) | (unsigned __int128)sp[q][0]);
    __int128 vk = (__int128)(((unsigned __int128)sk[q][1] << 64) | (unsigned __int128)sk[q][0]);
    fx_atomic_add(acc->p[q], vp);
    fx_atomic_add(acc->k[q], vk);
    atomicAdd(&acc->cnt[q], sc[q]);
  }
}
void launch_power_bins(const void* A, const void* B, int n, int nb, const double* e2, double scale, PowDev* acc,
                       cudaStream_t s) {
  i64 tot = (i64)(n / 2 + 1) * n * n;
  i64 blocks = std::min<i64>((tot + 255) / 256, 152 * 4);
  k_power_bins<<<(unsigned)blocks, 256, 0, s>>>((const double2*)A, (const double2*)B, n, nb, e2, scale, acc);
  count_launch();
}

// ---------------------------------------------------------------------------
// Float-float kernels of the mixed form (arithmetic in mmh_ff.cuh).  The
// outer residual is formed from neighbour differences, r = rhs - sum_f b_f
// (phi_nb - phi_c) - cross terms, so its terms are ~ n/(2 pi) |rhs| and its
// error ~ 1e-12 |rhs| -- far below the outer loop's tolerance -- while every
// product and sum runs on the FP32 pipes (the FP64 form of this kernel is
// bound by the FP64 rate).
// ---------------------------------------------------------------------------
// The mixed form's finest-level metric (cbajraw, gauss1.f90:1107-1210) in
// float-float, for the outer residual: rho_bar * cof(A) / det as (hi, lo)
// pairs in `coef` (six planes of n^3 pairs, the layout k_ff_split makes) and
// the hi parts, the FP32 V-cycle's coefficients, in coef32.  Every input is
// split into a float-float pair from its bit pattern (ff_of_bits), and the
// whole metric runs on the FP32 and integer pipes: the Hessian of def from
// neighbour differences (ff_diff), A, its cofactors and determinant,
// rho_bar / det and the six products in float-float, the 27-cell density sum
// by compensated summation (TwoSum of the high parts, Ogita-Rump-Oishi Sum2;
// the densities are non-negative, so its error is ~2^-48 of the sum).  A
// pair holds its double to 2^-48, so a Hessian entry carries ~2^-46 max|def|
// / dx^2 and the coefficients about 48 significant bits otherwise.  det <=
// 1e-5 takes the reference's fallback (unit cofactors, det = 1).  di2 =
// 1/dx^2 is a power of two.
__global__ void __launch_bounds__(256) k_metric_ff(const double* __restrict__ def, const double* __restrict__ rho,
                                                   int n, float di2, float2* __restrict__ coef,
                                                   float* __restrict__ coef32, double* __restrict__ det_out) {
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  const int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
#define D_(x, y, z) ff_of_bits(def[IDX(x, y, z, n)])
  const FF c = ff_of_bits(def[t]);
  const FF pxx = ff_scale(ff_add(ff_diff(D_(ip, j, k), c), ff_diff(D_(im, j, k), c)), di2);
  const FF pyy = ff_scale(ff_add(ff_diff(D_(i, jp, k), c), ff_diff(D_(i, jm, k), c)), di2);
  const FF pzz = ff_scale(ff_add(ff_diff(D_(i, j, kp), c), ff_diff(D_(i, j, km), c)), di2);
  const float q = 0.25f * di2;
  const FF pxy = ff_scale(ff_sub(ff_diff(D_(ip, jp, k), D_(im, jp, k)), ff_diff(D_(ip, jm, k), D_(im, jm, k))), q);
  const FF pyz = ff_scale(ff_sub(ff_diff(D_(i, jp, kp), D_(i, jp, km)), ff_diff(D_(i, jm, kp), D_(i, jm, km))), q);
  const FF pxz = ff_scale(ff_sub(ff_diff(D_(ip, j, kp), D_(im, j, kp)), ff_diff(D_(ip, j, km), D_(im, j, km))), q);
#undef D_
  const FF one = {1.0f, 0.0f};
  const FF a11 = ff_add(one, pxx), a22 = ff_add(one, pyy), a33 = ff_add(one, pzz);
  const FF a12 = pxy, a13 = pxz, a23 = pyz;
  FF b[6];
  b[0] = ff_sub(ff_mul(a22, a33), ff_mul(a23, a23));
  b[1] = ff_sub(ff_mul(a13, a23), ff_mul(a12, a33));
  b[2] = ff_sub(ff_mul(a12, a23), ff_mul(a13, a22));
  b[3] = ff_sub(ff_mul(a11, a33), ff_mul(a13, a13));
  b[4] = ff_sub(ff_mul(a12, a13), ff_mul(a11, a23));
  b[5] = ff_sub(ff_mul(a11, a22), ff_mul(a12, a12));
  FF det = ff_add(ff_add(ff_mul(a11, b[0]), ff_mul(a12, b[1])), ff_mul(a13, b[2]));
  // det(A) itself (before the tangle fallback) for rgzerosum
  if (det_out) det_out[t] = (double)det.hi + (double)det.lo;
  if (det.hi + det.lo <= 1.e-5f) {
    b[0] = one; b[1] = {0.0f, 0.0f}; b[2] = {0.0f, 0.0f}; b[3] = one; b[4] = {0.0f, 0.0f}; b[5] = one;
    det = one;
  }
  const int is[3] = {im, i, ip}, js[3] = {jm, j, jp}, ks[3] = {km, k, kp};
  float sh = 0.0f, se = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const FF v = ff_of_bits(rho[IDX(is[a], js[bb], ks[d], n)]);
        const FF s2 = ff_two_sum(sh, v.hi);
        sh = s2.hi;
        se = se + (s2.lo + v.lo);
      }
  const FF urg = ff_quick(sh, se);
  // 1/27 as a float-float constant
  const double r27 = 1.0 / 27.0;
  const float r27h = (float)r27;
  const FF w = ff_div(ff_mul(urg, {r27h, (float)(r27 - (double)r27h)}), det);
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const FF cf = ff_mul(w, b[f]);
    coef[(i64)f * n3 + t] = make_float2(cf.hi, cf.lo);
    coef32[(i64)f * n3 + t] = cf.hi;
  }
}

void launch_metric_ff(const double* def, const double* rho, int n, double dx, double* coef, float* coef32,
                      double* det, cudaStream_t s) {
  const i64 n3 = (i64)n * n * n;
  prof_begin(KK_METRIC, s, n3, n);
  k_metric_ff<<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, rho, n, (float)(1.0 / (dx * dx)), reinterpret_cast<float2*>(coef),
                                                     coef32, det);
  prof_end(KK_METRIC, s, n);
  count_launch();
}

// in place: doubles -> (hi, lo) pairs in the same 8 bytes, and back
__global__ void k_ff_split(double* __restrict__ a, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  FF v = ff_of_bits(a[t]);
  reinterpret_cast<float2*>(a)[t] = make_float2(v.hi, v.lo);
}
__global__ void k_ff_join(double* __restrict__ a, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  float2 v = reinterpret_cast<const float2*>(a)[t];
  a[t] = (double)v.x + (double)v.y;
}
// x += e (float) ; x -= mean (double)
__global__ void k_ff_add_f(float2* __restrict__ x, const float* __restrict__ e, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  float2 v = x[t];
  FF r = ff_add({v.x, v.y}, {e[t], 0.0f});
  x[t] = make_float2(r.hi, r.lo);
}
__global__ void k_ff_sub_mean(float2* __restrict__ x, const double* __restrict__ mean, i64 count) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  float2 v = x[t];
  FF r = ff_sub({v.x, v.y}, ff_of_bits(*mean));
  x[t] = make_float2(r.hi, r.lo);
}

// r = rhs - L[phi] * di2 in float-float: phi and the six coefficient planes
// as (hi, lo) pairs, rhs in FP64; r32 (may be null) = r rounded to float,
// max |r| into maxbits (from the high parts: within 2^-24 of itself).
__global__ void __launch_bounds__(256) k_residual_ff(const float2* __restrict__ phi, const double* __restrict__ rhs,
                                                     const float2* __restrict__ coef, int n, float di2,
                                                     float* __restrict__ r32, unsigned long long* maxbits) {
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (t < n3) {
    int i, j, k;
    cell_of(t, n, i, j, k);
    const int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
    auto P = [&](int a, int b, int c) {
      float2 v = __ldg(phi + IDX(a, b, c, n));
      return FF{v.x, v.y};
    };
    auto C = [&](int f, int a, int b, int c) {
      float2 v = __ldg(coef + (i64)f * n3 + IDX(a, b, c, n));
      return FF{v.x, v.y};
    };
    const FF pc = P(i, j, k);
    // face terms: b_f (phi_nb - phi_c), b_f the mean of the two cells' coefficients
    const FF f1c = C(0, i, j, k), f4c = C(3, i, j, k), f6c = C(5, i, j, k);
    FF L = ff_mul(ff_scale(ff_add(C(0, ip, j, k), f1c), 0.5f), ff_sub(P(ip, j, k), pc));
    L = ff_add(L, ff_mul(ff_scale(ff_add(C(0, im, j, k), f1c), 0.5f), ff_sub(P(im, j, k), pc)));
    L = ff_add(L, ff_mul(ff_scale(ff_add(C(3, i, jp, k), f4c), 0.5f), ff_sub(P(i, jp, k), pc)));
    L = ff_add(L, ff_mul(ff_scale(ff_add(C(3, i, jm, k), f4c), 0.5f), ff_sub(P(i, jm, k), pc)));
    L = ff_add(L, ff_mul(ff_scale(ff_add(C(5, i, j, kp), f6c), 0.5f), ff_sub(P(i, j, kp), pc)));
    L = ff_add(L, ff_mul(ff_scale(ff_add(C(5, i, j, km), f6c), 0.5f), ff_sub(P(i, j, km), pc)));
    // cross terms (relaxplane's t2)
    const FF ppk = P(ip, jp, k), mpk = P(im, jp, k), pmk = P(ip, jm, k), mmk = P(im, jm, k);
    const FF jpkp = P(i, jp, kp), jmkp = P(i, jm, kp), jpkm = P(i, jp, km), jmkm = P(i, jm, km);
    const FF ipkp = P(ip, j, kp), imkp = P(im, j, kp), ipkm = P(ip, j, km), imkm = P(im, j, km);
    FF x = ff_mul(ff_sub(ppk, mpk), C(1, i, jp, k));
    x = ff_sub(x, ff_mul(ff_sub(pmk, mmk), C(1, i, jm, k)));
    x = ff_add(x, ff_mul(ff_sub(ppk, pmk), C(1, ip, j, k)));
    x = ff_sub(x, ff_mul(ff_sub(mpk, mmk), C(1, im, j, k)));
    x = ff_add(x, ff_mul(ff_sub(jpkp, jmkp), C(4, i, j, kp)));
    x = ff_sub(x, ff_mul(ff_sub(jpkm, jmkm), C(4, i, j, km)));
    x = ff_add(x, ff_mul(ff_sub(jpkp, jpkm), C(4, i, jp, k)));
    x = ff_sub(x, ff_mul(ff_sub(jmkp, jmkm), C(4, i, jm, k)));
    x = ff_add(x, ff_mul(ff_sub(ipkp, imkp), C(2, i, j, kp)));
    x = ff_sub(x, ff_mul(ff_sub(ipkm, imkm), C(2, i, j, km)));
    x = ff_add(x, ff_mul(ff_sub(ipkp, ipkm), C(2, ip, j, k)));
    x = ff_sub(x, ff_mul(ff_sub(imkp, imkm), C(2, im, j, k)));
    L = ff_add(L, ff_scale(x, 0.25f));
    const FF r = ff_sub(ff_of_bits(rhs[t]), ff_scale(L, di2));
    if (r32) r32[t] = r.hi;
    m = fabsf(r.hi);
  }
  if (maxbits) block_max_commit(m, maxbits);
}

// The outer residual of a zero guess, b itself, as the inner solve's FP32
// right-hand side: what k_residual_ff gives for phi = 0 (b split into a
// float-float pair and rounded, hi + lo), with max |r| into maxbits.
__global__ void k_ff_rhs32(const double* __restrict__ b, i64 count, float* __restrict__ r32,
                           unsigned long long* maxbits) {
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (t < count) {
    const FF v = ff_of_bits(b[t]);
    const float r = __fadd_rn(v.hi, v.lo);
    r32[t] = r;
    m = fabsf(r);
  }
  block_max_commit(m, maxbits);
}
void launch_ff_rhs32(const double* b, i64 count, float* r32, unsigned long long* maxbits, cudaStream_t s) {
  k_ff_rhs32<<<grid_of(count, kBlock), kBlock, 0, s>>>(b, count, r32, maxbits);
  count_launch();
}
__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }
void launch_set_u64(unsigned long long* p, unsigned long long v, cudaStream_t s) {
  k_set_u64<<<1, 1, 0, s>>>(p, v);
  count_launch();
}

void launch_ff_split(double* a, i64 count, cudaStream_t s) {
  k_ff_split<<<grid_of(count, kBlock), kBlock, 0, s>>>(a, count);
  count_launch();
}
void launch_ff_join(double* a, i64 count, cudaStream_t s) {
  k_ff_join<<<grid_of(count, kBlock), kBlock, 0, s>>>(a, count);
  count_launch();
}
void launch_ff_add_f(double* x, const float* e, i64 count, cudaStream_t s) {
  k_ff_add_f<<<grid_of(count, kBlock), kBlock, 0, s>>>(reinterpret_cast<float2*>(x), e, count);
  count_launch();
}
void launch_ff_sub_mean(double* x, const double* mean, i64 count, cudaStream_t s) {
  k_ff_sub_mean<<<grid_of(count, kBlock), kBlock, 0, s>>>(reinterpret_cast<float2*>(x), mean, count);
  count_launch();
}
void launch_residual_ff(const double* phi, const double* rhs, const double* coef, int n, double dx, float* r32,
                        unsigned long long* maxbits, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  prof_begin(KK_RESIDUAL, s, n3, n);
  k_residual_ff<<<grid_of(n3, kBlock), kBlock, 0, s>>>(reinterpret_cast<const float2*>(phi), rhs,
                                                       reinterpret_cast<const float2*>(coef), n,
                                                       (float)(1.0 / (dx * dx)), r32, maxbits);
  prof_end(KK_RESIDUAL, s, n);
  count_launch();
}

// One axis of the smoother [1/4, 1/2, 1/4] (the 27-point nsmooth of
// limiter.f90:677-781 is its product over the three axes), periodic, as a
// pass without its weights: out = in[-1] + in[+1] + 2 in (one add and one fused multiply-add; 2 in is exact).  The
// last pass applies the three passes' weights, 1/64, at once.  Scaling by a
// power of two is exact and commutes with rounding, so the result has the
// bits of three passes of (in[-1] + in[+1]) / 4 + in / 2.
template <bool LAST>
__global__ void k_smooth_axis(const double* __restrict__ in, int n, int axis, double* __restrict__ out) {
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int c[3];
  cell_of(t, n, c[0], c[1], c[2]);
  const i64 stride = axis == 0 ? 1 : (axis == 1 ? (i64)n : (i64)n * n);
  const i64 lo = c[axis] == 0 ? t + (i64)(n - 1) * stride : t - stride;
  const i64 hi = c[axis] == n - 1 ? t - (i64)(n - 1) * stride : t + stride;
  const double v = __fma_rn(2.0, in[t], in[lo] + in[hi]);
  out[t] = LAST ? v * 0.015625 : v;
}
// The 27-point smoother as three axis passes (the mixed form's nsmooth:
// the same operator, other rounding): in -> out -> in -> out; in is
// overwritten.
void launch_smooth_sep(double* in, int n, double* out, cudaStream_t s) {
  const i64 n3 = (i64)n * n * n;
  k_smooth_axis<false><<<grid_of(n3, kBlock), kBlock, 0, s>>>(in, n, 0, out);
  k_smooth_axis<false><<<grid_of(n3, kBlock), kBlock, 0, s>>>(out, n, 1, in);
  k_smooth_axis<true><<<grid_of(n3, kBlock), kBlock, 0, s>>>(in, n, 2, out);
  count_launch(3);
}

void launch_lim_reset(LimDev* st, cudaStream_t s) {
  k_lim_reset<<<1, 1, 0, s>>>(st);
  count_launch();
}

// ---------------------------------------------------------------------------
// Spectral kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 spec_mode(double2 x, int kx, int ky, int kz, int n, int mode, const double* ctab) {
  const double pi = 3.14159265358979323846264338328;
  double re = x.x, im = x.y;
  if (mode <= 2) {
    // cmp * cmplx(0,kk) / n * 2 * pi  (gradient.f90:21,43,65)
    double kk;
    if (mode == 0) kk = (double)kx;
    else if (mode == 1) kk = (ky + 1 <= n / 2 + 1) ? (double)ky : (double)(ky - n);
    else kk = (kz + 1 <= n / 2 + 1) ? (double)kz : (double)(kz - n);
    double r2 = re * 0.0 - im * kk;
    double i2 = re * kk + im * 0.0;
    r2 = r2 * (1.0 / n) * 2. * pi;  // n is a power of two: exact reciprocal
    i2 = i2 * (1.0 / n) * 2. * pi;
    return make_double2(r2, i2);
  } else if (mode == 3) {
    // *(k1^2 + k2^2 + k3^2)  (reconstruct.f90:88-110)
    double k3 = (kz + 1 <= n / 2 + 1) ? (double)kz : (double)(kz - n);
    k3 = k3 * (1.0 / n) * 2. * pi;
    double k2 = (ky + 1 <= n / 2 + 1) ? (double)ky : (double)(ky - n);
    k2 = k2 * (1.0 / n) * 2. * pi;
    double k1 = (double)kx;
    k1 = k1 * (1.0 / n) * 2. * pi;
    double f = k1 * k1 + k2 * k2 + k3 * k3;
    return make_double2(re * f, im * f);
  } else {
    // / (2cos kx + 2cos ky + 2cos kz - 6), DC real part zeroed (limiter.f90:561-576);
    // ctab[k] = cos(2 pi k / n), the reference's angles (ky + 1 - 1. is ky exactly)
    double akernel = 2 * ctab[kx] + 2 * ctab[ky] + 2 * ctab[kz] - 6;
    if (fabs(akernel) < 1e-10) akernel = 1;
    double r2 = re / akernel, i2 = im / akernel;
    if (kx == 0 && ky == 0 && kz == 0) r2 = 0.0;
    return make_double2(r2, i2);
  }
}

// Tables of the spectral kernels, computed once per context with the same
// expressions the kernels used: tab[2kx], tab[2kx+1] = cos, sin(-2 pi kx / n)
// for kx < n/2 (the packing twiddle), tab[n + k] = cos(2 pi k / n).
__global__ void k_spec_tables(double* tab, int n) {
  const double pi = 3.14159265358979323846264338328;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  if (k < n / 2) {
    double th = -2.0 * pi * k / n;
    tab[2 * k] = cos(th);
    tab[2 * k + 1] = sin(th);
  }
  tab[n + k] = cos(2 * pi * k / n);
}
void launch_spec_tables(double* tab, int n, cudaStream_t s) {
  k_spec_tables<<<grid_of(n, kBlock), kBlock, 0, s>>>(tab, n);
  count_launch();
}

__global__ void k_spec_pack(const double2* __restrict__ Xc, int n, int mode, double2* __restrict__ Z,
                            const LimDev* st, const double* __restrict__ tab) {
  if (mode == 4 && st->ncompress == 0) return;
  int M = n / 2, H = M + 1;
  i64 tot = (i64)M * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tot) return;
  const int lgm = __ffs(M) - 1, lgn = lgm + 1;  // n is a power of two
  int kx = (int)t & (M - 1);
  int ky = (int)(t >> lgm) & (n - 1), kz = (int)(t >> (lgm + lgn));
  int kx2 = M - kx, ky2 = (n - ky) & (n - 1), kz2 = (n - kz) & (n - 1);
  // X_NR(k) = conj(Xc(k)) : spectrum with exp(+2 pi i k.x / n)
  double2 a = Xc[kx + (i64)H * (ky + (i64)n * kz)];
  double2 b = Xc[kx2 + (i64)H * (ky2 + (i64)n * kz2)];
  const double* ctab = tab + n;
  double2 A = spec_mode(make_double2(a.x, -a.y), kx, ky, kz, n, mode, ctab);
  double2 B = spec_mode(make_double2(b.x, -b.y), kx2, ky2, kz2, n, mode, ctab);
  B.y = -B.y;  // conj
  double wr = tab[2 * kx], wi = tab[2 * kx + 1];
  double sr = A.x + B.x, si = A.y + B.y;
  double dr = A.x - B.x, di = A.y - B.y;
  double wdr = wr * dr - wi * di, wdi = wr * di + wi * dr;
  // 0.5*(A+B) + 0.5 i w (A-B)
  Z[t] = make_double2(0.5 * sr - 0.5 * wdi, 0.5 * si + 0.5 * wdr);
}

void launch_spec_pack(const void* Xc, int n, int mode, void* Z, const LimDev* st, const double* tab, cudaStream_t s) {
  i64 tot = (i64)(n / 2) * n * n;
  k_spec_pack<<<grid_of(tot, kBlock), kBlock, 0, s>>>((const double2*)Xc, n, mode, (double2*)Z, st, tab);
  count_launch();
}

__global__ void k_spec_unpack(const double2* __restrict__ z, int n, double* __restrict__ out, int stride_out, int add,
                              const LimDev* st) {
  if (add && st->ncompress == 0) return;
  i64 tot = (i64)(n / 2) * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tot) return;
  double2 v = z[t];
  const double rn = 1.0 / n;  // n is a power of two: exact reciprocal
  double a = v.x * 2. * rn * rn * rn;
  double b = v.y * 2. * rn * rn * rn;
  i64 o0 = 2 * t, o1 = 2 * t + 1;
  if (add) {
    out[o0] = out[o0] + a;
    out[o1] = out[o1] + b;
  } else {
    out[o0 * stride_out] = a;
    out[o1 * stride_out] = b;
  }
}

void launch_spec_unpack(const void* z, int n, double* out, int stride_out, int add, const LimDev* st, cudaStream_t s) {
  i64 tot = (i64)(n / 2) * n * n;
  k_spec_unpack<<<grid_of(tot, kBlock), kBlock, 0, s>>>((const double2*)z, n, out, stride_out, add, st);
  count_launch();
}

// ---------------------------------------------------------------------------
// relaxing-TVD, density component (relaxing.f90).  u(2:5) = 0, so the Euler
// flux of the density is the zero momentum and the pressure vanishes; the
// results are those of the reference's operations on those zero components.
// FP64 arithmetic dominates these kernels, so each keeps only the operations
// whose result is not already known exactly.
// ---------------------------------------------------------------------------

// 0.0 / d with IEEE semantics: a signed zero for finite non-zero and infinite
// d, the division itself (NaN) only for zero or NaN d.
__device__ __forceinline__ double zdiv(double d) { return (d == d && d != 0.0) ? copysign(0.0, d) : 0.0 / d; }
// biased binary exponent: 0 for zero and subnormals, 2047 for inf and NaN
__device__ __forceinline__ int bexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }
// MIN/MAX as the restatement evaluates them (std::min / std::max: a
// comparison and a select), so NaN arguments propagate the same way.
__device__ __forceinline__ double ref_min(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double ref_max(double a, double b) { return (a < b) ? b : a; }

// dpv (relaxing.f90:269-496) forms, at every stencil point along axis a, the
// flux w_a = v_a / c divided by the freezing speed and then only the half sums
// (u + w_a)/2 and half differences (u - w_a)/2.  Those six values per cell
// are computed once here: sd[a] = (u + w_a)/2, sd[3 + a] = (u - w_a)/2.
__device__ __forceinline__ void store_sd(double* __restrict__ sd, i64 n3, i64 t, double u0, double wx, double wy,
                                         double wz) {
  sd[0 * n3 + t] = (u0 + wx) * 0.5;
  sd[1 * n3 + t] = (u0 + wy) * 0.5;
  sd[2 * n3 + t] = (u0 + wz) * 0.5;
  sd[3 * n3 + t] = (u0 - wx) * 0.5;
  sd[4 * n3 + t] = (u0 - wy) * 0.5;
  sd[5 * n3 + t] = (u0 - wz) * 0.5;
}

// stage 1: calcbaj + cflkeuler + flux of u at every cell.
// baj: 7 planes (b11,b12,b13,b22,b23,b33,det); cc: freezing speed; sd: the
// half sums and differences of store_sd.
// FastDiv (the mixed form, which is not bit-matched): each cell's divisions
// by det, by det again and by c become one reciprocal each and products.
template <bool FastDiv>
__global__ void k_relax_stage1(const double* __restrict__ rho, const double* __restrict__ def,
                               const double* __restrict__ defp, int n, double* __restrict__ baj,
                               double* __restrict__ cc, double* __restrict__ sd) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  const double gamma = 5. / 3.;
  LimM m = lim_metric<FastDiv>(def, n, i, j, k);
  baj[0 * n3 + t] = m.b11;
  baj[1 * n3 + t] = m.b12;
  baj[2 * n3 + t] = m.b13;
  baj[3 * n3 + t] = m.b22;
  baj[4 * n3 + t] = m.b23;
  baj[5 * n3 + t] = m.b33;
  baj[6 * n3 + t] = m.det;
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  double dxp = defp[IDX(ip, j, k, n)], dxm = defp[IDX(im, j, k, n)];
  double dyp = defp[IDX(i, jp, k, n)], dym = defp[IDX(i, jm, k, n)];
  double dzp = defp[IDX(i, j, kp, n)], dzm = defp[IDX(i, j, km, n)];
  double u0 = rho[t];
  double c;
  // cflkeuler (relaxing.f90:1097-1135)
  {
    double pdx = (dxp - dxm) * 0.5, pdy = (dyp - dym) * 0.5, pdz = (dzp - dzm) * 0.5;
    double det = m.det;
    double vx = zdiv(u0), vy = vx, vz = vx;
    double v1 = vx - pdx, v2 = vy - pdy, v3 = vz - pdz;
    double vv1 = m.b11 * v1 + m.b12 * v2 + m.b13 * v3;
    double vv2 = m.b12 * v1 + m.b22 * v2 + m.b23 * v3;
    double vv3 = m.b13 * v1 + m.b23 * v2 + m.b33 * v3;
    // With u0 and det finite and non-zero, u0/det finite and non-zero and every
    // b finite below 2^500, the kinetic and internal energies are signed
    // zeros, so the sound speed cs is +0, cs*sqrt(...) is +0 and each bound is
    // |vv|: the same bits as the full expression, which runs otherwise.
    const int eu = bexp(u0), ed = bexp(det);
    const int eb = max(max(max(bexp(m.b11), bexp(m.b12)), max(bexp(m.b13), bexp(m.b22))), max(bexp(m.b23), bexp(m.b33)));
    if (eu >= 1 && eu <= 2046 && ed >= 1 && ed <= 2046 && abs(eu - ed) <= 1000 && eb <= 1523) {
      c = ref_max(ref_max(fabs(vv1), fabs(vv2)), fabs(vv3));
    } else {
      double rhoc = u0 / det;
      double kin = rhoc * (vx * vx + vy * vy + vz * vz) * 0.5;
      double edn = zdiv(det) - kin;
      double pressure = (gamma - 1.0) * edn;
      double cs = sqrt(gamma * fabs(pressure / rhoc));
      double blim1 = cs * sqrt(m.b11 * m.b11 + m.b12 * m.b12 + m.b13 * m.b13) + fabs(vv1);
      double blim2 = cs * sqrt(m.b12 * m.b12 + m.b22 * m.b22 + m.b23 * m.b23) + fabs(vv2);
      double blim3 = cs * sqrt(m.b13 * m.b13 + m.b23 * m.b23 + m.b33 * m.b33) + fabs(vv3);
      c = ref_max(ref_max(blim1, blim2), blim3);
    }
    cc[t] = c;
  }
  // flux (relaxing.f90:970-988) of the density
  {
    double rg = m.det;
    double mx = zdiv(rg), my = mx, mz = mx;
    double pdxg, pdyg, pdzg;
    if (FastDiv) {
      const double rr = 1.0 / rg;
      pdxg = (dxp - dxm) * 0.5 * rr;
      pdyg = (dyp - dym) * 0.5 * rr;
      pdzg = (dzp - dzm) * 0.5 * rr;
    } else {
      pdxg = (dxp - dxm) * 0.5 / rg;
      pdyg = (dyp - dym) * 0.5 / rg;
      pdzg = (dzp - dzm) * 0.5 / rg;
    }
    double b11 = m.b11 * rg, b12 = m.b12 * rg, b13 = m.b13 * rg, b22 = m.b22 * rg, b23 = m.b23 * rg, b33 = m.b33 * rg;
    double vtt1 = mx - u0 * pdxg;
    double vtt2 = my - u0 * pdyg;
    double vtt3 = mz - u0 * pdzg;
    if (FastDiv) {
      const double rc = 1.0 / c;
      store_sd(sd, n3, t, u0, (b11 * vtt1 + b12 * vtt2 + b13 * vtt3) * rc, (b12 * vtt1 + b22 * vtt2 + b23 * vtt3) * rc,
               (b13 * vtt1 + b23 * vtt2 + b33 * vtt3) * rc);
    } else {
      store_sd(sd, n3, t, u0, (b11 * vtt1 + b12 * vtt2 + b13 * vtt3) / c, (b12 * vtt1 + b22 * vtt2 + b23 * vtt3) / c,
               (b13 * vtt1 + b23 * vtt2 + b33 * vtt3) / c);
    }
  }
}

void launch_relax_stage1(const double* rho, const double* def, const double* defp, int n, double* baj, double* cc,
                         double* sd, cudaStream_t s, bool fast_div) {
  i64 n3 = (i64)n * n * n;
  if (fast_div)
    k_relax_stage1<true><<<grid_of(n3, kBlock), kBlock, 0, s>>>(rho, def, defp, n, baj, cc, sd);
  else
    k_relax_stage1<false><<<grid_of(n3, kBlock), kBlock, 0, s>>>(rho, def, defp, n, baj, cc, sd);
  count_launch();
}

// flux of the half-step state u1 with the metric of stage 1 (relaxing.f90:
// 970-988), as the half sums and differences of store_sd.
template <bool FastDiv>
__global__ void k_relax_flux(const double* __restrict__ u1, const double* __restrict__ defp,
                             const double* __restrict__ baj, const double* __restrict__ cc, int n,
                             double* __restrict__ sd) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  double rg = baj[6 * n3 + t];
  double u0 = u1[t];
  double c = cc[t];
  double mx = zdiv(rg), my = mx, mz = mx;
  double pdxg, pdyg, pdzg;
  if (FastDiv) {
    const double rr = 1.0 / rg;
    pdxg = (defp[IDX(ip, j, k, n)] - defp[IDX(im, j, k, n)]) * 0.5 * rr;
    pdyg = (defp[IDX(i, jp, k, n)] - defp[IDX(i, jm, k, n)]) * 0.5 * rr;
    pdzg = (defp[IDX(i, j, kp, n)] - defp[IDX(i, j, km, n)]) * 0.5 * rr;
  } else {
    pdxg = (defp[IDX(ip, j, k, n)] - defp[IDX(im, j, k, n)]) * 0.5 / rg;
    pdyg = (defp[IDX(i, jp, k, n)] - defp[IDX(i, jm, k, n)]) * 0.5 / rg;
    pdzg = (defp[IDX(i, j, kp, n)] - defp[IDX(i, j, km, n)]) * 0.5 / rg;
  }
  double b11 = baj[0 * n3 + t] * rg, b12 = baj[1 * n3 + t] * rg, b13 = baj[2 * n3 + t] * rg;
  double b22 = baj[3 * n3 + t] * rg, b23 = baj[4 * n3 + t] * rg, b33 = baj[5 * n3 + t] * rg;
  double vtt1 = mx - u0 * pdxg;
  double vtt2 = my - u0 * pdyg;
  double vtt3 = mz - u0 * pdzg;
  if (FastDiv) {
    const double rc = 1.0 / c;
    store_sd(sd, n3, t, u0, (b11 * vtt1 + b12 * vtt2 + b13 * vtt3) * rc, (b12 * vtt1 + b22 * vtt2 + b23 * vtt3) * rc,
             (b13 * vtt1 + b23 * vtt2 + b33 * vtt3) * rc);
  } else {
    store_sd(sd, n3, t, u0, (b11 * vtt1 + b12 * vtt2 + b13 * vtt3) / c, (b12 * vtt1 + b22 * vtt2 + b23 * vtt3) / c,
             (b13 * vtt1 + b23 * vtt2 + b33 * vtt3) / c);
  }
}

void launch_relax_flux(const double* u1, const double* defp, const double* baj, const double* cc, int n, double* sd,
                       cudaStream_t s, bool fast_div) {
  i64 n3 = (i64)n * n * n;
  if (fast_div)
    k_relax_flux<true><<<grid_of(n3, kBlock), kBlock, 0, s>>>(u1, defp, baj, cc, n, sd);
  else
    k_relax_flux<false><<<grid_of(n3, kBlock), kBlock, 0, s>>>(u1, defp, baj, cc, n, sd);
  count_launch();
}

__device__ __forceinline__ double fsign1(double a) { return a >= 0.0 ? 1.0 : -1.0; }
// minmod of relaxing.f90 with wslopelim = 1.5, wbee = 1:
//   mm = min(1.5*lo, 1*hi + 0*lo), result (sign(a) + sign(b)) * mm / 2.
// For finite lo, 1*hi + 0*lo is hi; for mm below 2^1023, (+-2)*mm/2 is +-mm
// and 0*mm/2 is +0.  Those cases skip the multiplications; the others run
// the expression as written.
__device__ __forceinline__ double minmod(double a, double b) {
  const double wslopelim = 1.5, wbee = 1.0;
  const unsigned long long inf_bits = 0x7FF0000000000000ull;
  const unsigned long long ax = abs_bits(a), ay = abs_bits(b);
  double lo, hi, mm;
  if (ax <= inf_bits && ay <= inf_bits) {
    // Without a NaN operand (an integer test of the bits) the magnitudes
    // |a|, |b| and 1.5*lo are non-negative, and non-negative doubles order
    // like their bit patterns: min, max and the comparison with hi are
    // integer compare-and-selects with the bits fmin/fmax would return, and
    // a >= 0.0 is a test of the sign bit (-0 included).
    const unsigned long long lob = ax <= ay ? ax : ay, hib = ax <= ay ? ay : ax;
    lo = __longlong_as_double((long long)lob);
    hi = __longlong_as_double((long long)hib);
    if (lob < inf_bits) {
      const double l15 = wslopelim * lo;  // finite or +inf
      mm = abs_bits(l15) <= hib ? l15 : hi;
    } else {
      mm = fmin(wslopelim * lo, wbee * hi + (1.0 - wbee) * lo);
    }
    if (bexp(mm) < 2046) {
      const bool pa = (__double_as_longlong(a) >= 0) || ax == 0, pb = (__double_as_longlong(b) >= 0) || ay == 0;
      return pa != pb ? 0.0 : (pa ? mm : -mm);
    }
    return (fsign1(a) + fsign1(b)) * mm * 0.5;
  }
  // a NaN operand: the restatement's compare-and-select decides which value
  // propagates
  double x = fabs(a), y = fabs(b);
  lo = ref_min(x, y);
  hi = ref_max(x, y);
  mm = bexp(lo) < 2047 ? ref_min(wslopelim * lo, hi) : ref_min(wslopelim * lo, wbee * hi + (1.0 - wbee) * lo);
  if (bexp(mm) < 2046) {
    const bool pa = a >= 0.0, pb = b >= 0.0;
    return pa != pb ? 0.0 : (pa ? mm : -mm);
  }
  return (fsign1(a) + fsign1(b)) * mm * 0.5;
}
// x * 0.5 with the same bits: a normal x whose half is normal (biased
// exponent 2..2046) loses one from its exponent field; zeros, subnormals,
// the smallest normals, inf and NaN take the multiplication.
__device__ __forceinline__ double half_of(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  return (e >= 2u && e <= 2046u) ? __longlong_as_double((long long)(b - (1ull << 52))) : x * 0.5;
}
// wphalf (relaxing.f90) from the half sums s = (u+w)/2 at the cells -1, 0, +1
// and the half differences d = (u-w)/2 at the cells 0, +1, +2 of the face.
__device__ __forceinline__ double wphalf_sd(double sm, double s0, double sp, double d0, double dp, double dpp) {
  double a = s0;
  double b = dp;
  double da = sp - a;
  double dam = a - sm;
  double ap = a + half_of(minmod(dam, da));
  double db = dpp - b;
  double dbm = b - d0;
  double bp = b - half_of(minmod(db, dbm));
  return ap - bp;
}

// Face fluxes of dpv (relaxing.f90:269-496): g_a[cell] is the flux through
// the upper face of the cell along axis a, (c(+1) + c(0))/2 * wphalf over the
// cells -1, 0, +1, +2 of that axis.  dpv takes the difference of the upper
// and the lower face of each cell; the lower face is the upper face of the
// neighbour below, computed from the same operands in the same order, so each
// face is evaluated once here instead of once from each side.
__global__ void k_relax_faces(const double* __restrict__ sd, const double* __restrict__ cc, int n,
                              double* __restrict__ g) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  const double c0 = cc[t];
  {
    int im = wm(i, n), ip = wp(i, n), ipp = wp(ip, n);
    i64 a = IDX(im, j, k, n), b = IDX(ip, j, k, n), d = IDX(ipp, j, k, n);
    const double* S = sd;
    const double* D = sd + 3 * n3;
    double fl = wphalf_sd(S[a], S[t], S[b], D[t], D[b], D[d]);
    g[t] = half_of(cc[b] + c0) * fl;
  }
  {
    int jm = wm(j, n), jp = wp(j, n), jpp = wp(jp, n);
    i64 a = IDX(i, jm, k, n), b = IDX(i, jp, k, n), d = IDX(i, jpp, k, n);
    const double* S = sd + n3;
    const double* D = sd + 4 * n3;
    double fl = wphalf_sd(S[a], S[t], S[b], D[t], D[b], D[d]);
    g[n3 + t] = half_of(cc[b] + c0) * fl;
  }
  {
    int km = wm(k, n), kp = wp(k, n), kpp = wp(kp, n);
    i64 a = IDX(i, j, km, n), b = IDX(i, j, kp, n), d = IDX(i, j, kpp, n);
    const double* S = sd + 2 * n3;
    const double* D = sd + 5 * n3;
    double fl = wphalf_sd(S[a], S[t], S[b], D[t], D[b], D[d]);
    g[2 * n3 + t] = half_of(cc[b] + c0) * fl;
  }
}

// dpv residual from the face fluxes, in the reference's order (z, then x,
// then y), and out = ubase - res*dt.
__global__ void k_relax_div(const double* __restrict__ g, int n, const double* __restrict__ ubase, double dt,
                            double* __restrict__ out) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  double r = g[2 * n3 + t] - g[2 * n3 + IDX(i, j, wm(k, n), n)];
  r = r + g[t] - g[IDX(wm(i, n), j, k, n)];
  r = r + g[n3 + t] - g[n3 + IDX(i, wm(j, n), k, n)];
  out[t] = ubase[t] - r * dt;
}

void launch_relax_dpv(const double* sd, const double* cc, int n, const double* ubase, double dt, double* out,
                      double* gface, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_relax_faces<<<grid_of(n3, kBlock), kBlock, 0, s>>>(sd, cc, n, gface);
  count_launch();
  k_relax_div<<<grid_of(n3, kBlock), kBlock, 0, s>>>(gface, n, ubase, dt, out);
  count_launch();
}

template <class U>
__global__ void k_extract_density(const U* __restrict__ u, int nf, i64 n3, double* __restrict__ rho, int* flag) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  rho[t] = (double)u[(i64)nf * t];
  bool nz = false;
  for (int c = 1; c < nf; ++c) nz = nz || (u[(i64)nf * t + c] != U(0));
  if (nz) atomicOr(flag, 1);
}
void launch_extract_density_f(const float* u, int nf, i64 n3, double* rho, int* flag, cudaStream_t s) {
  k_extract_density<float><<<grid_of(n3, kBlock), kBlock, 0, s>>>(u, nf, n3, rho, flag);
  count_launch();
}
void launch_extract_density_d(const double* u, int nf, i64 n3, double* rho, int* flag, cudaStream_t s) {
  k_extract_density<double><<<grid_of(n3, kBlock), kBlock, 0, s>>>(u, nf, n3, rho, flag);
  count_launch();
}

}  // namespace mmh


// ---------------------------------------------------------------------------
// Krylov scalars (flexible PCG): dot products from the exact accumulators.
// ---------------------------------------------------------------------------
namespace mmh {

MMH_INSTANTIATE_PCG(double)

__device__ __forceinline__ double fx_unscale(const unsigned long long* acc, int E) {
  __int128 s = (__int128)(((unsigned __int128)acc[1] << 64) | (unsigned __int128)acc[0]);
  bool neg = s < 0;
  unsigned __int128 a = neg ? (unsigned __int128)(-s) : (unsigned __int128)s;
  double r = __dadd_rn(scalbn(__ull2double_rn((unsigned long long)(a >> 64)), E - 32),
                       scalbn(__ull2double_rn((unsigned long long)a), E - 96));
  return neg ? -r : r;
}

__device__ __forceinline__ double dot_value(const unsigned long long* acc, const unsigned long long* abits,
                                            const unsigned long long* bbits) {
  double ma = bits_d(abits), mb = bits_d(bbits);
  if (!(ma > 0.0) || !(mb > 0.0)) return 0.0;
  return fx_unscale(acc, ilogb(ma) + ilogb(mb) + 2);
}

// stage 0: rz = dot(r,z) ; 1: alpha = rz / dot(p,q) ;
// 2: beta = -(alpha*dot(z,q))/rz, rz = dot(r,z)
__global__ void k_pcg_scalar(PcgDev* s, int stage) {
  if (stage == 0) {
    s->rz = dot_value(s->acc[0], &s->rbits, &s->zbits);
  } else if (stage == 1) {
    s->pq = dot_value(s->acc[1], &s->pbits, &s->qbits);
    s->alpha = s->rz / s->pq;
  } else {
    double zq = dot_value(s->acc[2], &s->zbits, &s->qbits);
    double rznew = dot_value(s->acc[0], &s->rbits, &s->zbits);
    s->beta = -(s->alpha * zq) / s->rz;
    s->rz = rznew;
  }
}

void launch_pcg_scalar(PcgDev* st, int stage, cudaStream_t s) {
  k_pcg_scalar<<<1, 1, 0, s>>>(st, stage);
  count_launch();
}

}  // namespace mmh
