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

// Gradient with respect to the entries of A = I + Hess(def) of
//   - sum_f urg G_f C_f(A)   (the operator path, C_f = cof_f / det with the
//                              tangle fallback det <= 1e-5 of cbajraw)
//   - r y det(A)             (rgzerosum: P b = b - det r, r = sum b / sum det)
// abar: 6 planes (a11, a12, a13, a22, a23, a33).
__global__ void k_adj_metric(const double* __restrict__ def, const double* __restrict__ lam,
                             const double* __restrict__ u, const double* __restrict__ urg,
                             const double* __restrict__ y, const double* __restrict__ rptr, int n,
                             double* __restrict__ abar) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  double c = def[t];
  double a11 = 1.0 + (def[IDX(ip, j, k, n)] - 2.0 * c + def[IDX(im, j, k, n)]);
  double a22 = 1.0 + (def[IDX(i, jp, k, n)] - 2.0 * c + def[IDX(i, jm, k, n)]);
  double a33 = 1.0 + (def[IDX(i, j, kp, n)] - 2.0 * c + def[IDX(i, j, km, n)]);
  double a12 = (def[IDX(ip, jp, k, n)] - def[IDX(im, jp, k, n)] - def[IDX(ip, jm, k, n)] + def[IDX(im, jm, k, n)]) * 0.25;
  double a23 = (def[IDX(i, jp, kp, n)] - def[IDX(i, jp, km, n)] - def[IDX(i, jm, kp, n)] + def[IDX(i, jm, km, n)]) * 0.25;
  double a13 = (def[IDX(ip, j, kp, n)] - def[IDX(im, j, kp, n)] - def[IDX(ip, j, km, n)] + def[IDX(im, j, km, n)]) * 0.25;
  double det = a11 * a22 * a33 + 2.0 * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33;
  double b11 = a22 * a33 - a23 * a23, b12 = a13 * a23 - a12 * a33, b13 = a12 * a23 - a13 * a22;
  double b22 = a11 * a33 - a13 * a13, b23 = a12 * a13 - a11 * a23, b33 = a11 * a22 - a12 * a12;
  // adjoint of det (rgzerosum): -r y
  double detb = -(*rptr) * y[t];
  double c11 = 0.0, c12 = 0.0, c13 = 0.0, c22 = 0.0, c23 = 0.0, c33 = 0.0;
  if (det > 1.e-5) {
    i64 xp = IDX(ip, j, k, n), xm = IDX(im, j, k, n), yp = IDX(i, jp, k, n), ym = IDX(i, jm, k, n);
    i64 zp = IDX(i, j, kp, n), zm = IDX(i, j, km, n);
    double lc = lam[t], uc = u[t];
    double lxp = lam[xp], lxm = lam[xm], lyp = lam[yp], lym = lam[ym], lzp = lam[zp], lzm = lam[zm];
    double uxp = u[xp], uxm = u[xm], uyp = u[yp], uym = u[ym], uzp = u[zp], uzm = u[zm];
    double w = -urg[t];
    // adjoint of C_f: -urg G_f, then of cof_f / det
    double g11 = w * 0.5 * ((lc - lxp) * (uxp - uc) + (lc - lxm) * (uxm - uc)) / det;
    double g22 = w * 0.5 * ((lc - lyp) * (uyp - uc) + (lc - lym) * (uym - uc)) / det;
    double g33 = w * 0.5 * ((lc - lzp) * (uzp - uc) + (lc - lzm) * (uzm - uc)) / det;
    double g12 = w * 0.25 * ((lym - lyp) * (uxp - uxm) + (lxm - lxp) * (uyp - uym)) / det;
    double g13 = w * 0.25 * ((lzm - lzp) * (uxp - uxm) + (lxm - lxp) * (uzp - uzm)) / det;
    double g23 = w * 0.25 * ((lzm - lzp) * (uyp - uym) + (lym - lyp) * (uzp - uzm)) / det;
    detb -= (g11 * b11 + g12 * b12 + g13 * b13 + g22 * b22 + g23 * b23 + g33 * b33) / det;
    c11 = g11; c12 = g12; c13 = g13; c22 = g22; c23 = g23; c33 = g33;
  }
  // d det / d a and d cof / d a (symmetric A: a12 stands for both off-diagonal entries)
  abar[t] = detb * b11 + c22 * a33 - c23 * a23 + c33 * a22;
  abar[n3 + t] = 2.0 * detb * b12 - c12 * a33 + c13 * a23 + c23 * a13 - 2.0 * c33 * a12;
  abar[2 * n3 + t] = 2.0 * detb * b13 + c12 * a23 - c13 * a22 - 2.0 * c22 * a13 + c23 * a12;
  abar[3 * n3 + t] = detb * b22 + c11 * a33 - c13 * a13 + c33 * a11;
  abar[4 * n3 + t] = 2.0 * detb * b23 - 2.0 * c11 * a23 + c12 * a13 + c13 * a12 - c23 * a11;
  abar[5 * n3 + t] = detb * b33 + c11 * a22 - c12 * a12 + c22 * a11;
}

// out (+)= Hess^T abar: the second differences of the metric are symmetric
// stencils, so the transpose applies the same stencils to the abar planes.
__global__ void k_adj_hess(const double* __restrict__ abar, int n, double* __restrict__ out, int add) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  const double *A11 = abar, *A12 = abar + n3, *A13 = abar + 2 * n3, *A22 = abar + 3 * n3, *A23 = abar + 4 * n3,
               *A33 = abar + 5 * n3;
  double r = (A11[IDX(ip, j, k, n)] - 2.0 * A11[t] + A11[IDX(im, j, k, n)]) +
             (A22[IDX(i, jp, k, n)] - 2.0 * A22[t] + A22[IDX(i, jm, k, n)]) +
             (A33[IDX(i, j, kp, n)] - 2.0 * A33[t] + A33[IDX(i, j, km, n)]) +
             0.25 * (A12[IDX(ip, jp, k, n)] - A12[IDX(im, jp, k, n)] - A12[IDX(ip, jm, k, n)] + A12[IDX(im, jm, k, n)]) +
             0.25 * (A23[IDX(i, jp, kp, n)] - A23[IDX(i, jp, km, n)] - A23[IDX(i, jm, kp, n)] + A23[IDX(i, jm, km, n)]) +
             0.25 * (A13[IDX(ip, j, kp, n)] - A13[IDX(im, j, kp, n)] - A13[IDX(ip, j, km, n)] + A13[IDX(im, j, km, n)]);
  out[t] = add ? out[t] + r : r;
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

void launch_adj_metric(const double* def, const double* lam, const double* u, const double* urg, const double* y,
                       const double* rptr, int n, double* abar, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_metric<<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, lam, u, urg, y, rptr, n, abar);
  count_launch();
}
void launch_adj_hess(const double* abar, int n, double* out, int add, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_hess<<<grid_of(n3, kBlock), kBlock, 0, s>>>(abar, n, out, add);
  count_launch();
}

}  // namespace mmh
