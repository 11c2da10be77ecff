// MMH reconstruction hot path -- limiter, spectral and relaxing kernels (FP64).
//
// Grid-compression limiter (mmh/limiter.f90), spectral outputs and the FFT
// Poisson correction (mmh/gradient.f90, mmh/reconstruct.f90, limiter.f90:535-597)
// and the relaxing-TVD density update (mmh/relaxing.f90).  Operand order
// follows the reference; the translation unit is compiled with --fmad=false.
#pragma once
#include "mmh_kernels.cuh"

namespace mmh {

// Limiter metric: cof(A)/det and det of A = I + Hess(def) at unit spacing
// (limiter.f90:268-286, relaxing.f90:876-901).
struct LimM {
  double b11, b12, b13, b22, b23, b33, det;
  double phixx, phiyy, phizz, phixy, phiyz, phixz;
};

// FastDiv (the mixed form, which is not bit-matched): the six divisions by
// det become one reciprocal and six multiplications.
template <bool FastDiv = false>
__device__ __forceinline__ LimM lim_metric(const double* __restrict__ def, int n, int i, int j, int k) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  LimM m;
  double c = def[IDX(i, j, k, n)];
  m.phixx = (def[IDX(ip, j, k, n)] - 2.0 * c + def[IDX(im, j, k, n)]);
  m.phiyy = (def[IDX(i, jp, k, n)] - 2.0 * c + def[IDX(i, jm, k, n)]);
  m.phizz = (def[IDX(i, j, kp, n)] - 2.0 * c + def[IDX(i, j, km, n)]);
  m.phixy = (def[IDX(ip, jp, k, n)] - def[IDX(im, jp, k, n)] - def[IDX(ip, jm, k, n)] + def[IDX(im, jm, k, n)]) * 0.25;
  m.phiyz = (def[IDX(i, jp, kp, n)] - def[IDX(i, jp, km, n)] - def[IDX(i, jm, kp, n)] + def[IDX(i, jm, km, n)]) * 0.25;
  m.phixz = (def[IDX(ip, j, kp, n)] - def[IDX(im, j, kp, n)] - def[IDX(ip, j, km, n)] + def[IDX(im, j, km, n)]) * 0.25;
  double a11 = 1.0 + m.phixx, a12 = m.phixy, a13 = m.phixz, a22 = 1.0 + m.phiyy, a23 = m.phiyz, a33 = 1.0 + m.phizz;
  double det = a11 * a22 * a33 + 2.0 * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33;
  m.det = det;
  if (FastDiv) {
    const double r = 1.0 / det;
    m.b11 = (a22 * a33 - a23 * a23) * r;
    m.b12 = (a13 * a23 - a12 * a33) * r;
    m.b13 = (a12 * a23 - a13 * a22) * r;
    m.b22 = (a11 * a33 - a13 * a13) * r;
    m.b23 = (a12 * a13 - a11 * a23) * r;
    m.b33 = (a11 * a22 - a12 * a12) * r;
  } else {
    m.b11 = (a22 * a33 - a23 * a23) / det;
    m.b12 = (a13 * a23 - a12 * a33) / det;
    m.b13 = (a12 * a23 - a13 * a22) / det;
    m.b22 = (a11 * a33 - a13 * a13) / det;
    m.b23 = (a12 * a13 - a11 * a23) / det;
    m.b33 = (a11 * a22 - a12 * a12) / det;
  }
  return m;
}

// The Hessian entries and det of lim_metric alone, by the same operations
// (the same bits), without the cofactors and their divisions.
__device__ __forceinline__ LimM lim_hess_det(const double* __restrict__ def, int n, int i, int j, int k) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  LimM m;
  double c = def[IDX(i, j, k, n)];
  m.phixx = (def[IDX(ip, j, k, n)] - 2.0 * c + def[IDX(im, j, k, n)]);
  m.phiyy = (def[IDX(i, jp, k, n)] - 2.0 * c + def[IDX(i, jm, k, n)]);
  m.phizz = (def[IDX(i, j, kp, n)] - 2.0 * c + def[IDX(i, j, km, n)]);
  m.phixy = (def[IDX(ip, jp, k, n)] - def[IDX(im, jp, k, n)] - def[IDX(ip, jm, k, n)] + def[IDX(im, jm, k, n)]) * 0.25;
  m.phiyz = (def[IDX(i, jp, kp, n)] - def[IDX(i, jp, km, n)] - def[IDX(i, jm, kp, n)] + def[IDX(i, jm, km, n)]) * 0.25;
  m.phixz = (def[IDX(ip, j, kp, n)] - def[IDX(im, j, kp, n)] - def[IDX(ip, j, km, n)] + def[IDX(im, j, km, n)]) * 0.25;
  double a11 = 1.0 + m.phixx, a12 = m.phixy, a13 = m.phixz, a22 = 1.0 + m.phiyy, a23 = m.phiyz, a33 = 1.0 + m.phizz;
  m.det = a11 * a22 * a33 + 2.0 * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33;
  m.b11 = m.b12 = m.b13 = m.b22 = m.b23 = m.b33 = 0.0;
  return m;
}

// 1/(smallest eigenvalue) of the symmetric matrix C by the trigonometric
// cubic-root formula (limiter.f90:346-358 and 459-471).
__device__ __forceinline__ double compression_of(double c11, double c12, double c13, double c22, double c23,
                                                 double c33) {
  const double pi = 3.14159265358979323846264338328;
  double trace = c11 + c22 + c33;
  double d11 = c11 - trace / 3.0;
  double d22 = c22 - trace / 3.0;
  double a = -(d11 * d11 + c12 * c12 + c13 * c13 + d11 * d22 + d22 * d22 + c23 * c23);
  double b = -d11 * (c12 * c12) + d11 * d11 * d22 - c12 * c12 * d22 + c13 * c13 * d22 + d11 * (d22 * d22) -
             2.0 * c12 * c13 * c23 + d11 * (c23 * c23);
  if (fabs(a) < 1.e-20) a = 1.e-20;
  double am = 2.0 * sqrt(fabs(-a) / 3.0);
  double theta = acos(fmax(-1.0, fmin(1.0, 3.0 * b / a / am))) / 3.0;
  double r1 = am * cos(theta);
  double r2 = am * cos(theta + 2.0 * pi / 3.0);
  double r3 = am * cos(theta + 4.0 * pi / 3.0);
  return 1.0 / fmin(fmin(r1 + trace / 3.0, r2 + trace / 3.0), r3 + trace / 3.0);
}

// Limiter statistics block in device memory.
struct LimDev {
  unsigned long long nexpand, ncompress;
  unsigned long long detmax, detmin, fluxmax, fluxmin, cmax;  // ord_of() encoded
  unsigned long long rho2[2];                                  // fixed-point sum
  int flag;
  int pad;
};

// Pass-1 flux limiter for a density-only state (u(2:5) = 0, so the
// momentum-flux divergence is zero): limiter.f90:238-381.  The flux of cell
// (i,j,km) is tested with the metric of plane k = km+1.
__global__ void k_limiter_pass1(double* __restrict__ tmp, const double* __restrict__ def,
                                const double* __restrict__ rho, int n, double dtold, double dtaumesh,
                                double cmpmaxglobal, LimDev* st, uint8_t* __restrict__ maskx,
                                uint8_t* __restrict__ maskc);

// Compression test on I + dtold*Hess(defp) + Hess(def) (limiter.f90:425-533).
__global__ void k_limiter_mask(double* __restrict__ defplim, const double* __restrict__ def,
                               const double* __restrict__ defp, int n, double dtold, double cmpmaxglobal, LimDev* st,
                               uint8_t* __restrict__ mask);

// calcdefp RHS: tmp = clip(1 - rho, +-2)/30/dtold (limiter.f90:134-169)
__global__ void k_calcdefp_rhs(double* __restrict__ tmp, const double* __restrict__ rho, i64 n3, double dtold);

// Spectral stage 1: from the e^{-i} half spectrum Xc = D2Z(x), build the packed
// complex input Z' of the reference's inverse real FFT applied to
// mode(X_NR), X_NR = conj(Xc) the e^{+i} spectrum.  mode: 0,1,2 = gradient
// along x,y,z; 3 = |k|^2 (defp2delta); 4 = division by the 7-point Laplacian
// symbol (limiter.f90:561-576).
__global__ void k_spec_pack(const double2* __restrict__ Xc, int n, int mode, double2* __restrict__ Z,
                            const LimDev* st);
// Spectral stage 2: x = 2/n^3 * (real samples held pairwise by z); add != 0
// adds into out (defp += defplim) and is skipped when no cell was limited.
__global__ void k_spec_unpack(const double2* __restrict__ z, int n, double* __restrict__ out, int stride_out,
                              int add, const LimDev* st);

// relaxing-TVD (relaxing.f90) for the density component.
__global__ void k_relax_stage1(const double* __restrict__ rho, const double* __restrict__ def,
                               const double* __restrict__ defp, int n, double* __restrict__ baj,
                               double* __restrict__ cc, double* __restrict__ vt);
__global__ void k_relax_flux(const double* __restrict__ u1, const double* __restrict__ defp,
                             const double* __restrict__ baj, int n, double* __restrict__ vt);
__global__ void k_relax_dpv(const double* __restrict__ u, const double* __restrict__ vt,
                            const double* __restrict__ cc, int n, const double* __restrict__ ubase, double dt,
                            double* __restrict__ out);

}  // namespace mmh
