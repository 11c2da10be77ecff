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
#include "mmh_phys.cuh"

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

// Adjoint of A = I + Hess(def) (6 planes a11, a12, a13, a22, a23, a33; a12
// stands for both off-diagonal entries) from the adjoint detb of det(A) and
// the adjoints c_f of the cofactors cof_f(A).
__device__ __forceinline__ void adj_cofdet(double a11, double a12, double a13, double a22, double a23, double a33,
                                           double b11, double b12, double b13, double b22, double b23, double b33,
                                           double detb, double c11, double c12, double c13, double c22, double c23,
                                           double c33, double* __restrict__ abar, i64 t, i64 n3) {
  abar[t] = detb * b11 + c22 * a33 - c23 * a23 + c33 * a22;
  abar[n3 + t] = 2.0 * detb * b12 - c12 * a33 + c13 * a23 + c23 * a13 - 2.0 * c33 * a12;
  abar[2 * n3 + t] = 2.0 * detb * b13 + c12 * a23 - c13 * a22 - 2.0 * c22 * a13 + c23 * a12;
  abar[3 * n3 + t] = detb * b22 + c11 * a33 - c13 * a13 + c33 * a11;
  abar[4 * n3 + t] = 2.0 * detb * b23 - 2.0 * c11 * a23 + c12 * a13 + c13 * a12 - c23 * a11;
  abar[5 * n3 + t] = detb * b33 + c11 * a22 - c12 * a12 + c22 * a11;
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
  adj_cofdet(a11, a12, a13, a22, a23, a33, b11, b12, b13, b22, b23, b33, detb, c11, c12, c13, c22, c23, c33, abar,
             t, n3);
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

// Adjoint of the final compression test's correction (limiter.f90:425-597)
// with its mask frozen.  On a limited cell defplim = tlim =
// 3 (1/cmpmax - lambda_min(C)) / dtold, C = I + dtold Hess(defp_s) +
// Hess(def) (as k_limiter_mask forms it), and for a simple smallest
// eigenvalue d lambda_min / dC = v v^T, v its unit eigenvector (the cross
// product of two rows of C - lambda_min I).  With g = mask . P w (P the
// symmetric FFT Poisson operator), abar = dJ/dC for J = sum g defplim:
// abar = -3 g / dtold (v1^2, 2 v1 v2, 2 v1 v3, v2^2, 2 v2 v3, v3^2), the
// off-diagonal entries counting both places they occupy in C.
__global__ void k_adj_limiter(const double* __restrict__ def, const double* __restrict__ defps,
                              const double* __restrict__ pw, const uint8_t* __restrict__ mask, int n, double dtold,
                              double* __restrict__ abar) {
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  double a[6] = {0, 0, 0, 0, 0, 0};
  if (mask[t]) {
    int i, j, k;
    cell_of(t, n, i, j, k);
    const int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
#define P_(x, y, z) defps[IDX(x, y, z, n)]
#define D_(x, y, z) def[IDX(x, y, z, n)]
    double pxx = (P_(ip, j, k) - 2.0 * P_(i, j, k) + P_(im, j, k)) * dtold;
    double pyy = (P_(i, jp, k) - 2.0 * P_(i, j, k) + P_(i, jm, k)) * dtold;
    double pzz = (P_(i, j, kp) - 2.0 * P_(i, j, k) + P_(i, j, km)) * dtold;
    double pxy = (P_(ip, jp, k) - P_(im, jp, k) - P_(ip, jm, k) + P_(im, jm, k)) * 0.25 * dtold;
    double pyz = (P_(i, jp, kp) - P_(i, jp, km) - P_(i, jm, kp) + P_(i, jm, km)) * 0.25 * dtold;
    double pxz = (P_(ip, j, kp) - P_(im, j, kp) - P_(ip, j, km) + P_(im, j, km)) * 0.25 * dtold;
    pxx = pxx + (D_(ip, j, k) - 2.0 * D_(i, j, k) + D_(im, j, k));
    pyy = pyy + (D_(i, jp, k) - 2.0 * D_(i, j, k) + D_(i, jm, k));
    pzz = pzz + (D_(i, j, kp) - 2.0 * D_(i, j, k) + D_(i, j, km));
    pxy = pxy + (D_(ip, jp, k) - D_(im, jp, k) - D_(ip, jm, k) + D_(im, jm, k)) * 0.25;
    pyz = pyz + (D_(i, jp, kp) - D_(i, jp, km) - D_(i, jm, kp) + D_(i, jm, km)) * 0.25;
    pxz = pxz + (D_(ip, j, kp) - D_(im, j, kp) - D_(ip, j, km) + D_(im, j, km)) * 0.25;
#undef P_
#undef D_
    const double c11 = 1.0 + pxx, c22 = 1.0 + pyy, c33 = 1.0 + pzz, c12 = pxy, c13 = pxz, c23 = pyz;
    // smallest eigenvalue (the trigonometric formula of the compression test)
    const double pi = 3.14159265358979323846264338328;
    const double mu = (c11 + c22 + c33) / 3.0;
    const double d11 = c11 - mu, d22 = c22 - mu;
    double aa = -(d11 * d11 + c12 * c12 + c13 * c13 + d11 * d22 + d22 * d22 + c23 * c23);
    const double bb = -d11 * (c12 * c12) + d11 * d11 * d22 - c12 * c12 * d22 + c13 * c13 * d22 + d11 * (d22 * d22) -
                      2.0 * c12 * c13 * c23 + d11 * (c23 * c23);
    if (fabs(aa) < 1.e-20) aa = 1.e-20;
    const double am = 2.0 * sqrt(fabs(-aa) / 3.0);
    const double th = acos(fmax(-1.0, fmin(1.0, 3.0 * bb / aa / am))) / 3.0;
    const double lam = fmin(fmin(am * cos(th), am * cos(th + 2.0 * pi / 3.0)), am * cos(th + 4.0 * pi / 3.0)) + mu;
    // eigenvector: the longest cross product of two rows of C - lam I
    const double r1[3] = {c11 - lam, c12, c13}, r2[3] = {c12, c22 - lam, c23}, r3[3] = {c13, c23, c33 - lam};
    auto cross = [](const double* x, const double* y, double* z) {
      z[0] = x[1] * y[2] - x[2] * y[1];
      z[1] = x[2] * y[0] - x[0] * y[2];
      z[2] = x[0] * y[1] - x[1] * y[0];
    };
    double v[3], w2[3], w3[3];
    cross(r1, r2, v);
    cross(r1, r3, w2);
    cross(r2, r3, w3);
    double nv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double n2 = w2[0] * w2[0] + w2[1] * w2[1] + w2[2] * w2[2];
    const double n3v = w3[0] * w3[0] + w3[1] * w3[1] + w3[2] * w3[2];
    if (n2 > nv) { v[0] = w2[0]; v[1] = w2[1]; v[2] = w2[2]; nv = n2; }
    if (n3v > nv) { v[0] = w3[0]; v[1] = w3[1]; v[2] = w3[2]; nv = n3v; }
    if (nv > 0.0) {
      const double rn = 1.0 / sqrt(nv);
      v[0] *= rn; v[1] *= rn; v[2] *= rn;
      const double sc = -3.0 * pw[t] / dtold;
      a[0] = sc * v[0] * v[0];
      a[1] = sc * 2.0 * v[0] * v[1];
      a[2] = sc * 2.0 * v[0] * v[2];
      a[3] = sc * v[1] * v[1];
      a[4] = sc * 2.0 * v[1] * v[2];
      a[5] = sc * v[2] * v[2];
    }
  }
#pragma unroll
  for (int q = 0; q < 6; ++q) abar[q * n3 + t] = a[q];
}

// out = a + s * b
__global__ void k_adj_axpy(const double* __restrict__ a, double s, const double* __restrict__ b,
                           double* __restrict__ out, i64 n3) {
  i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  out[q] = a[q] + s * b[q];
}

// out = a * b (op 1) or a - b (op 0), elementwise
__global__ void k_adj_pair(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                           int op, i64 n3) {
  i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  out[q] = op ? a[q] * b[q] : a[q] - b[q];
}

// ---------------------------------------------------------------------------
// relaxing adjoint (relaxing.f90, density-only state at rest)
//
// Forward map, restated: per cell the flux ratios alpha_a = vv_a / c with
// vv = b (0 - grad defp), b = cof/det of I + Hess(def), c = max_a |vv_a|
// (cflkeuler, the branch of a finite non-zero density and det); the half sums
// S_a = x (1 + alpha_a) / 2 and differences D_a = x (1 - alpha_a) / 2; the
// face flux F_a(f) = (c(f) + c(f+a)) / 2 * wphalf(S_a, D_a) with the minmod
// slopes; R(x) = sum_a F_a(e) - F_a(e-a).  TVD RK2: x1 = u - dt/2 R(u),
// u' = u - dt R(x1), both stages with the alpha and c of u's stage.
// ---------------------------------------------------------------------------

// minmod with wslopelim 1.5 (relaxing.f90): value and the partial
// derivatives in a and b on the branch it takes.
__device__ __forceinline__ double mm_branch(double a, double b, double& da, double& db) {
  double x = fabs(a), y = fabs(b);
  da = 0.0;
  db = 0.0;
  if ((a >= 0.0) != (b >= 0.0)) return 0.0;
  double s = a >= 0.0 ? 1.0 : -1.0;
  double lo = fmin(x, y), hi = fmax(x, y);
  if (1.5 * lo <= hi) {
    if (x <= y) da = 1.5; else db = 1.5;
    return s * 1.5 * lo;
  }
  if (x >= y) da = 1.0; else db = 1.0;
  return s * hi;
}

// Face f -> fp along one axis (cells fm, f, fp, fpp): the adjoints P of the
// six half sums and differences it reads and Q of each of its two speeds,
// for the output adjoint rbar scaled by `scale`.
struct FaceAdj {
  double p0, p1, p2, p3, p4, p5, q;
};
__device__ __forceinline__ FaceAdj face_adj(const double* __restrict__ S, const double* __restrict__ D,
                                            const double* __restrict__ cc, const double* __restrict__ rbar,
                                            double scale, i64 fm, i64 f, i64 fp, i64 fpp) {
  double sm = S[fm], s0 = S[f], sp = S[fp], d0 = D[f], dp = D[fp], dpp = D[fpp];
  double mu1, mu2, nu1, nu2;
  double ma = mm_branch(s0 - sm, sp - s0, mu1, mu2);
  double mb = mm_branch(dpp - dp, dp - d0, nu1, nu2);
  double wph = (s0 + ma * 0.5) - (dp - mb * 0.5);
  double fb = scale * (rbar[f] - rbar[fp]);
  double wb = fb * (cc[fp] + cc[f]) * 0.5;
  FaceAdj r;
  r.p0 = wb * (-0.5 * mu1);
  r.p1 = wb * (1.0 + 0.5 * mu1 - 0.5 * mu2);
  r.p2 = wb * (0.5 * mu2);
  r.p3 = -wb * (1.0 + 0.5 * nu1 - 0.5 * nu2);
  r.p4 = wb * (0.5 * nu1);
  r.p5 = -wb * (0.5 * nu2);
  r.q = fb * wph * 0.5;
  return r;
}

// flux ratios alpha_a = vv_a / c of stage 1 (3 planes)
__global__ void k_adj_alpha(const double* __restrict__ baj, const double* __restrict__ defp,
                            const double* __restrict__ cc, int n, double* __restrict__ alpha) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  double v1 = 0.0 - (defp[IDX(wp(i, n), j, k, n)] - defp[IDX(wm(i, n), j, k, n)]) * 0.5;
  double v2 = 0.0 - (defp[IDX(i, wp(j, n), k, n)] - defp[IDX(i, wm(j, n), k, n)]) * 0.5;
  double v3 = 0.0 - (defp[IDX(i, j, wp(k, n), n)] - defp[IDX(i, j, wm(k, n), n)]) * 0.5;
  double b11 = baj[t], b12 = baj[n3 + t], b13 = baj[2 * n3 + t], b22 = baj[3 * n3 + t], b23 = baj[4 * n3 + t],
         b33 = baj[5 * n3 + t];
  double c = cc[t];
  alpha[t] = (b11 * v1 + b12 * v2 + b13 * v3) / c;
  alpha[n3 + t] = (b12 * v1 + b22 * v2 + b23 * v3) / c;
  alpha[2 * n3 + t] = (b13 * v1 + b23 * v2 + b33 * v3) / c;
}

// Adjoint of one dpv evaluation x -> scale * R(x) against rbar: xbar = the
// state adjoint (written), alphabar and cbar accumulated.  sd holds the half
// sums and differences of x as the forward pass formed them (their minmod
// branches are the forward's).
__global__ void k_adj_dpv(const double* __restrict__ sd, const double* __restrict__ cc,
                          const double* __restrict__ alpha, const double* __restrict__ x,
                          const double* __restrict__ rbar, double scale, int n, double* __restrict__ xbar,
                          double* __restrict__ alphabar, double* __restrict__ cbar) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int ijk[3];
  cell_of(t, n, ijk[0], ijk[1], ijk[2]);
  double xb = 0.0, cb = 0.0;
  const double xe = x[t];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    // cells e-3a .. e+3a along axis a
    i64 at[7];
#pragma unroll
    for (int o = -3; o <= 3; ++o) {
      int c3[3] = {ijk[0], ijk[1], ijk[2]};
      int v = c3[a] + o;
      v = v < 0 ? v + n : (v >= n ? v - n : v);
      c3[a] = v;
      at[o + 3] = IDX(c3[0], c3[1], c3[2], n);
    }
    const double* S = sd + a * n3;
    const double* D = sd + (3 + a) * n3;
    FaceAdj up = face_adj(S, D, cc, rbar, scale, at[3], at[4], at[5], at[6]);  // face e+a
    FaceAdj f0 = face_adj(S, D, cc, rbar, scale, at[2], at[3], at[4], at[5]);  // face e
    FaceAdj m1 = face_adj(S, D, cc, rbar, scale, at[1], at[2], at[3], at[4]);  // face e-a
    FaceAdj m2 = face_adj(S, D, cc, rbar, scale, at[0], at[1], at[2], at[3]);  // face e-2a
    double sb = up.p0 + f0.p1 + m1.p2;
    double db = f0.p5 + m1.p3 + m2.p4;
    cb += f0.q + m1.q;
    double al = alpha[a * n3 + t];
    xb += sb * (1.0 + al) * 0.5 + db * (1.0 - al) * 0.5;
    alphabar[a * n3 + t] += (sb - db) * xe * 0.5;
  }
  xbar[t] = xb;
  cbar[t] += cb;
}

// From alphabar and cbar to the adjoints of A = I + Hess(def) (6 planes) and
// of the centred differences pd_a = (defp(e+a) - defp(e-a)) / 2 (3 planes).
__global__ void k_adj_relax_geom(const double* __restrict__ def, const double* __restrict__ defp,
                                 const double* __restrict__ cc, const double* __restrict__ alphabar,
                                 const double* __restrict__ cbar, int n, double* __restrict__ abar,
                                 double* __restrict__ pdbar) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  LimM m = lim_metric(def, n, i, j, k);
  double pd1 = (defp[IDX(wp(i, n), j, k, n)] - defp[IDX(wm(i, n), j, k, n)]) * 0.5;
  double pd2 = (defp[IDX(i, wp(j, n), k, n)] - defp[IDX(i, wm(j, n), k, n)]) * 0.5;
  double pd3 = (defp[IDX(i, j, wp(k, n), n)] - defp[IDX(i, j, wm(k, n), n)]) * 0.5;
  double v1 = 0.0 - pd1, v2 = 0.0 - pd2, v3 = 0.0 - pd3;
  double vv[3] = {m.b11 * v1 + m.b12 * v2 + m.b13 * v3, m.b12 * v1 + m.b22 * v2 + m.b23 * v3,
                  m.b13 * v1 + m.b23 * v2 + m.b33 * v3};
  // the maximum cflkeuler takes: max(max(|vv1|, |vv2|), |vv3|), first on ties
  int as = fabs(vv[0]) < fabs(vv[1]) ? 1 : 0;
  as = fabs(vv[as]) < fabs(vv[2]) ? 2 : as;
  double c = cc[t];
  double ab[3] = {alphabar[t], alphabar[n3 + t], alphabar[2 * n3 + t]};
  // alpha_a = vv_a / c, c = |vv_as|
  double cb = cbar[t] - (ab[0] * vv[0] + ab[1] * vv[1] + ab[2] * vv[2]) / (c * c);
  double vb[3] = {ab[0] / c, ab[1] / c, ab[2] / c};
  vb[as] += cb * (vv[as] > 0.0 ? 1.0 : (vv[as] < 0.0 ? -1.0 : 0.0));
  // vv = b v, v = -pd; b = cof / det
  double g11 = vb[0] * v1, g22 = vb[1] * v2, g33 = vb[2] * v3;
  double g12 = vb[0] * v2 + vb[1] * v1, g13 = vb[0] * v3 + vb[2] * v1, g23 = vb[1] * v3 + vb[2] * v2;
  pdbar[t] = -(m.b11 * vb[0] + m.b12 * vb[1] + m.b13 * vb[2]);
  pdbar[n3 + t] = -(m.b12 * vb[0] + m.b22 * vb[1] + m.b23 * vb[2]);
  pdbar[2 * n3 + t] = -(m.b13 * vb[0] + m.b23 * vb[1] + m.b33 * vb[2]);
  double a11 = 1.0 + m.phixx, a22 = 1.0 + m.phiyy, a33 = 1.0 + m.phizz, a12 = m.phixy, a13 = m.phixz, a23 = m.phiyz;
  double det = m.det;
  double c11 = a22 * a33 - a23 * a23, c12 = a13 * a23 - a12 * a33, c13 = a12 * a23 - a13 * a22;
  double c22 = a11 * a33 - a13 * a13, c23 = a12 * a13 - a11 * a23, c33 = a11 * a22 - a12 * a12;
  g11 /= det; g12 /= det; g13 /= det; g22 /= det; g23 /= det; g33 /= det;
  double detb = -(g11 * c11 + g12 * c12 + g13 * c13 + g22 * c22 + g23 * c23 + g33 * c33) / det;
  adj_cofdet(a11, a12, a13, a22, a23, a33, c11, c12, c13, c22, c23, c33, detb, g11, g12, g13, g22, g23, g33, abar,
             t, n3);
}

// out (+)= the transpose of the centred differences pd_a of defp
__global__ void k_adj_grad_t(const double* __restrict__ pdbar, int n, double* __restrict__ out, int add) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  double r = (pdbar[IDX(wm(i, n), j, k, n)] - pdbar[IDX(wp(i, n), j, k, n)]) * 0.5 +
             (pdbar[n3 + IDX(i, wm(j, n), k, n)] - pdbar[n3 + IDX(i, wp(j, n), k, n)]) * 0.5 +
             (pdbar[2 * n3 + IDX(i, j, wm(k, n), n)] - pdbar[2 * n3 + IDX(i, j, wp(k, n), n)]) * 0.5;
  out[t] = add ? out[t] + r : r;
}

void launch_adj_alpha(const double* baj, const double* defp, const double* cc, int n, double* alpha, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_alpha<<<grid_of(n3, kBlock), kBlock, 0, s>>>(baj, defp, cc, n, alpha);
  count_launch();
}
void launch_adj_dpv(const double* sd, const double* cc, const double* alpha, const double* x, const double* rbar,
                    double scale, int n, double* xbar, double* alphabar, double* cbar, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_dpv<<<grid_of(n3, kBlock), kBlock, 0, s>>>(sd, cc, alpha, x, rbar, scale, n, xbar, alphabar, cbar);
  count_launch();
}
void launch_adj_relax_geom(const double* def, const double* defp, const double* cc, const double* alphabar,
                           const double* cbar, int n, double* abar, double* pdbar, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_relax_geom<<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, defp, cc, alphabar, cbar, n, abar, pdbar);
  count_launch();
}
void launch_adj_grad_t(const double* pdbar, int n, double* out, int add, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_grad_t<<<grid_of(n3, kBlock), kBlock, 0, s>>>(pdbar, n, out, add);
  count_launch();
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
void launch_adj_limiter(const double* def, const double* defps, const double* pw, const uint8_t* mask, int n,
                        double dtold, double* abar, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_limiter<<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, defps, pw, mask, n, dtold, abar);
  count_launch();
}
void launch_adj_axpy(const double* a, double sc, const double* b, double* out, i64 n3, cudaStream_t s) {
  k_adj_axpy<<<grid_of(n3, kBlock), kBlock, 0, s>>>(a, sc, b, out, n3);
  count_launch();
}

void launch_adj_hess(const double* abar, int n, double* out, int add, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  k_adj_hess<<<grid_of(n3, kBlock), kBlock, 0, s>>>(abar, n, out, add);
  count_launch();
}

}  // namespace mmh
