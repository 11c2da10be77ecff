// FP64 kernels of the calcdefp adjoint (no counterpart in the reference):
// the transposed pieces of one calcdefp increment (mmh/limiter.f90:17-600)
// with the mesh potential fixed and the limiter's branch choices frozen.
//
// Forward map, restated:  g = clip(1 - rho, +-2) / 30 / dtold,
//   t = S^3 g,  e = pass1(t) (branches frozen),  b = P S e,
//   L(rho) u = b  (u zero mean),  defp = S^2 u,
// with S the 27-point smoother (symmetric), P b = b - det (sum b / sum det)
// (rgzerosum), L the 19-point curvilinear operator with coefficients
// coef_f = rhobar * C_f, rhobar the 27-cell box mean of rho and C_f the
// cofactor over det of I + Hess(def) (cbajraw).  L is symmetric.  For
// J = w^T defp the gradient is
//   dJ/drho = g' . S^3 (D . S (P^T lam)) - B27( sum_f C_f G_f(lam, u) ),
// where L lam = S^2 w - mean, D the frozen pass-1 derivative, B27 the box
// mean and G_f the bilinear form of coefficient f (k_adj_contract).
#include "mmh_launch.cuh"

namespace mmh {

// D . y: the derivative of the pass-1 flux limiter (limiter.f90:175-381,
// density-only state) at its input t, with the expansion and compression
// branches the forward pass took.
__global__ void k_adj_pass1(double* __restrict__ y, const double* __restrict__ t, const uint8_t* __restrict__ maskx,
                            const uint8_t* __restrict__ maskc, double dtaumesh, i64 n3) {
  i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  double e = 0.0 + t[q];
  double dd = 1.0;
  if (maskx[q]) {  // eflux = -2 |eflux|
    dd = e > 0.0 ? -2.0 : (e < 0.0 ? 2.0 : 0.0);
    e = -2.0 * fabs(e);
  }
  if (maskc[q]) {  // eflux = max(0, eflux)
    if (!(e > 0.0)) dd = 0.0;
    e = fmax(0.0, e);
  }
  if (e > 1.0 / dtaumesh || e < -1.0 / dtaumesh) dd = 0.0;  // the +-1/dtaumesh clamps
  y[q] = y[q] * dd;
}

// g'(rho) . y for g = clip(1 - rho, +-2) / 30 / dtold (limiter.f90:153-166)
__global__ void k_adj_rhs(double* __restrict__ y, const double* __restrict__ rho, double dtold, i64 n3) {
  i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  double t1 = 1.0 - rho[q];
  y[q] = fabs(t1) > 2.0 ? 0.0 : -(y[q] / 30.0 / dtold);
}

// out = sum_f C_f G_f with G_f(e) the factor of coef_f(e) in lam^T L[coef] u:
// face terms (b11, b22, b33 pair neighbours through the half sums of
// relaxplane, gauss1.f90:950-980) and cross terms (b12, b13, b23 of the
// four-point differences).
__global__ void k_adj_contract(const double* __restrict__ lam, const double* __restrict__ u,
                               const double* __restrict__ cf, int n, double* __restrict__ out) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  i64 xp = IDX(wp(i, n), j, k, n), xm = IDX(wm(i, n), j, k, n);
  i64 yp = IDX(i, wp(j, n), k, n), ym = IDX(i, wm(j, n), k, n);
  i64 zp = IDX(i, j, wp(k, n), n), zm = IDX(i, j, wm(k, n), n);
  double lc = lam[t], uc = u[t];
  double lxp = lam[xp], lxm = lam[xm], lyp = lam[yp], lym = lam[ym], lzp = lam[zp], lzm = lam[zm];
  double uxp = u[xp], uxm = u[xm], uyp = u[yp], uym = u[ym], uzp = u[zp], uzm = u[zm];
  double g11 = 0.5 * ((lc - lxp) * (uxp - uc) + (lc - lxm) * (uxm - uc));
  double g22 = 0.5 * ((lc - lyp) * (uyp - uc) + (lc - lym) * (uym - uc));
  double g33 = 0.5 * ((lc - lzp) * (uzp - uc) + (lc - lzm) * (uzm - uc));
  double g12 = 0.25 * ((lym - lyp) * (uxp - uxm) + (lxm - lxp) * (uyp - uym));
  double g13 = 0.25 * ((lzm - lzp) * (uxp - uxm) + (lxm - lxp) * (uzp - uzm));
  double g23 = 0.25 * ((lzm - lzp) * (uyp - uym) + (lym - lyp) * (uzp - uzm));
  out[t] = cf[t] * g11 + cf[n3 + t] * g12 + cf[2 * n3 + t] * g13 + cf[3 * n3 + t] * g22 + cf[4 * n3 + t] * g23 +
           cf[5 * n3 + t] * g33;
}

// 27-cell box mean (the density average of cbajraw, gauss1.f90:1185-1194);
// symmetric, so it is its own transpose.
__global__ void k_box27(const double* __restrict__ in, int n, double* __restrict__ out) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  const int is[3] = {wm(i, n), i, wp(i, n)}, js[3] = {wm(j, n), j, wp(j, n)}, ks[3] = {wm(k, n), k, wp(k, n)};
  double s = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int d = 0; d < 3; ++d) s += in[IDX(is[a], js[b], ks[d], n)];
  out[t] = s / 27.0;
}

// out = a * b (op 1) or a - b (op 0), elementwise
__global__ void k_adj_pair(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                           int op, i64 n3) {
  i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  out[q] = op ? a[q] * b[q] : a[q] - b[q];
}

void launch_adj_pass1(double* y, const double* t, const uint8_t* maskx, const uint8_t* maskc, double dtaumesh,
                      i64 n3, cudaStream_t s) {
  k_adj_pass1<<<grid_of(n3, kBlock), kBlock, 0, s>>>(y, t, maskx, maskc, dtaumesh, n3);
  count_launch();
}
void launch_adj_rhs(double* y, const double* rho, double dtold, i64 n3, cudaStream_t s) {
  k_adj_rhs<<<grid_of(n3, kBlock), kBlock, 0, s>>>(y, rho, dtold, n3);
  count_launch();
}
void launch_adj_contract(const double* lam, const double* u, const double* cf, int n, double* out, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_contract<<<grid_of(n3, kBlock), kBlock, 0, s>>>(lam, u, cf, n, out);
  count_launch();
}
void launch_box27(const double* in, int n, double* out, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_box27<<<grid_of(n3, kBlock), kBlock, 0, s>>>(in, n, out);
  count_launch();
}
void launch_adj_mul(const double* a, const double* b, double* out, i64 n3, cudaStream_t s) {
  k_adj_pair<<<grid_of(n3, kBlock), kBlock, 0, s>>>(a, b, out, 1, n3);
  count_launch();
}
void launch_adj_sub(const double* a, const double* b, double* out, i64 n3, cudaStream_t s) {
  k_adj_pair<<<grid_of(n3, kBlock), kBlock, 0, s>>>(a, b, out, 0, n3);
  count_launch();
}

}  // namespace mmh
