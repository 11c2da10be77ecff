// relaxing (mmh/relaxing.f90:21-1139) for the mixed form: the density's
// relaxing-TVD RK2 step with the fluxes in FP32 and the update in FP64.
//
// With u(2:5) = 0 (main.f90:57) the step moves only the density, with the
// mesh velocity -A^-1 grad defp.  At every cell the metric gives
//   vv = cof(A)/det . (-grad defp),  c = max_a |vv_a|  (cflkeuler's freezing
//   speed for a state at rest),  alpha_a = vv_a / c,
// and the flux of a state u along axis a is carried by the half sums and
// differences u (1 +- alpha_a) / 2 (relaxing.f90:970-988).  The face flux is
// (c + c_next)/2 times wphalf over the four cells of the face (minmod slopes
// with wslopelim = 1.5, relaxing.f90:514-541), and
//   u1 = u - dt/2 R(u),  u' = u - dt R(u1)   (relaxing.f90:200-212),
// c and the metric from the pre-step state in both stages.
//
// Precision: the second differences of def and the central differences of
// defp are formed from float-float splits of the FP64 samples (their operands
// are O(n) larger than the differences; the splits keep 48 bits) and rounded
// once to FP32; the metric, speeds, flux ratios and
// face fluxes are FP32; u' = u - dt R is formed in FP64.  R is small against u
// (a few per cent per step), so the FP32 rounding of R moves u by ~1e-8 of
// itself per step.  Cells where the reference's state is degenerate (zero or
// non-finite density or det) get a NaN speed, as the reference's 0/0 does.
#include <cuda_runtime.h>

#include "mmh_ff.cuh"
#include "mmh_kernels.cuh"

namespace mmh {
namespace {

// comparisons and selects, so a NaN operand propagates as in the reference's
// MIN / MAX restatement
__device__ __forceinline__ float rmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float rmax(float a, float b) { return (a < b) ? b : a; }

// minmod of relaxing.f90 (wslopelim = 1.5, wbee = 1): (sign a + sign b)/2
// times min(1.5 min(|a|,|b|), max(|a|,|b|)), Fortran sign(1, -0) = +1.
__device__ __forceinline__ float minmod32(float a, float b) {
  const float x = fabsf(a), y = fabsf(b);
  const float lo = rmin(x, y), hi = rmax(x, y);
  const float mm = rmin(1.5f * lo, hi);
  const bool pa = a >= 0.f, pb = b >= 0.f;
  return pa != pb ? 0.f : (pa ? mm : -mm);
}

// wphalf from the half sums s at the cells -1, 0, +1 and the half
// differences d at the cells 0, +1, +2 of a face
__device__ __forceinline__ float wphalf32(float sm, float s0, float sp, float d0, float dp, float dpp) {
  const float ap = s0 + 0.5f * minmod32(s0 - sm, sp - s0);
  const float bp = dp - 0.5f * minmod32(dpp - dp, dp - d0);
  return ap - bp;
}

// Geometry of the step at every cell: geo = (alpha_x, alpha_y, alpha_z, c),
// and the density rounded to FP32.
__global__ void __launch_bounds__(256) k_relax32_geom(const double* __restrict__ rho, const double* __restrict__ def,
                                                      const double* __restrict__ defp, int n,
                                                      float4* __restrict__ geo, float* __restrict__ uf) {
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  const int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  // second differences of def and central differences of defp from
  // float-float splits of the samples (integer and FP32 operations; FP64
  // runs at two operations per clock per SM on GB300), rounded once to FP32
#define D_(x, y, z) ff_of_bits(def[IDX(x, y, z, n)])
  const FF c0 = ff_of_bits(def[t]);
  const float pxx = ff_sum_f(ff_diff(D_(ip, j, k), c0), ff_diff(D_(im, j, k), c0));
  const float pyy = ff_sum_f(ff_diff(D_(i, jp, k), c0), ff_diff(D_(i, jm, k), c0));
  const float pzz = ff_sum_f(ff_diff(D_(i, j, kp), c0), ff_diff(D_(i, j, km), c0));
  const float pxy = ff_sum_f(ff_diff(D_(ip, jp, k), D_(im, jp, k)), ff_neg(ff_diff(D_(ip, jm, k), D_(im, jm, k)))) * 0.25f;
  const float pyz = ff_sum_f(ff_diff(D_(i, jp, kp), D_(i, jp, km)), ff_neg(ff_diff(D_(i, jm, kp), D_(i, jm, km)))) * 0.25f;
  const float pxz = ff_sum_f(ff_diff(D_(ip, j, kp), D_(im, j, kp)), ff_neg(ff_diff(D_(ip, j, km), D_(im, j, km)))) * 0.25f;
#undef D_
  const float a11 = 1.f + pxx, a12 = pxy, a13 = pxz, a22 = 1.f + pyy, a23 = pyz, a33 = 1.f + pzz;
  const float b11 = a22 * a33 - a23 * a23, b12 = a13 * a23 - a12 * a33, b13 = a12 * a23 - a13 * a22;
  const float b22 = a11 * a33 - a13 * a13, b23 = a12 * a13 - a11 * a23, b33 = a11 * a22 - a12 * a12;
  const float det = a11 * b11 + a12 * b12 + a13 * b13;
  // -grad defp (central differences)
#define P_(x, y, z) ff_of_bits(defp[IDX(x, y, z, n)])
  const float gx = ff_diff_f(P_(im, j, k), P_(ip, j, k)) * 0.5f;
  const float gy = ff_diff_f(P_(i, jm, k), P_(i, jp, k)) * 0.5f;
  const float gz = ff_diff_f(P_(i, j, km), P_(i, j, kp)) * 0.5f;
#undef P_
  const float rd = 1.f / det;
  const float v1 = (b11 * gx + b12 * gy + b13 * gz) * rd;
  const float v2 = (b12 * gx + b22 * gy + b23 * gz) * rd;
  const float v3 = (b13 * gx + b23 * gy + b33 * gz) * rd;
  const double u0 = rho[t];
  float c = rmax(rmax(fabsf(v1), fabsf(v2)), fabsf(v3));
  // u0 != 0 and finite, from its bits
  const unsigned long long ub = (unsigned long long)__double_as_longlong(u0);
  const bool u_ok = (ub << 1) != 0ull && ((ub >> 52) & 0x7ffull) != 0x7ffull;
  const bool sound = u_ok && det != 0.f && isfinite(det);
  if (!sound) c = __int_as_float(0x7fffffff);  // NaN
  const float rc = 1.f / c;
  geo[t] = make_float4(v1 * rc, v2 * rc, v3 * rc, c);
  uf[t] = (float)u0;
}

// One stage: R(u) from the FP32 state us and the geometry, then
// out = ubase - dt R in FP64 (out32: the result rounded to FP32 instead).
// Each face flux is formed by both cells that share it, from the same
// operands in the same order, so a face adds to one cell exactly what it
// takes from the other.
template <bool OUT32>
__global__ void __launch_bounds__(256) k_relax32_stage(const float* __restrict__ us, const float4* __restrict__ geo,
                                                       int n, const double* __restrict__ ubase, float dt,
                                                       double* __restrict__ out, float* __restrict__ out32) {
  const i64 n3 = (i64)n * n * n;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  const float4 g0 = geo[t];
  const float u0 = us[t];
  float r = 0.f;
  // axes in the reference's order of accumulation (z, then x, then y)
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int ax = q == 0 ? 2 : q - 1;
    i64 s1;
    int c, m2;
    if (ax == 0) { s1 = 1; c = i; }
    else if (ax == 1) { s1 = n; c = j; }
    else { s1 = (i64)n * n; c = k; }
    m2 = n;
    // cells -2 .. +2 along the axis (periodic)
    const i64 tm1 = c == 0 ? t + (i64)(m2 - 1) * s1 : t - s1;
    const i64 tp1 = c == m2 - 1 ? t - (i64)(m2 - 1) * s1 : t + s1;
    const int cm1 = c == 0 ? m2 - 1 : c - 1, cp1 = c == m2 - 1 ? 0 : c + 1;
    const i64 tm2 = cm1 == 0 ? tm1 + (i64)(m2 - 1) * s1 : tm1 - s1;
    const i64 tp2 = cp1 == m2 - 1 ? tp1 - (i64)(m2 - 1) * s1 : tp1 + s1;
    const float4 gm2 = geo[tm2], gm1 = geo[tm1], gp1 = geo[tp1], gp2 = geo[tp2];
    auto al = [ax](const float4& g) { return ax == 0 ? g.x : (ax == 1 ? g.y : g.z); };
    const float um2 = us[tm2], um1 = us[tm1], up1 = us[tp1], up2 = us[tp2];
    // half sums (s) and differences (d) of the five cells
    const float sm2 = (um2 + um2 * al(gm2)) * 0.5f, dm2 = (um2 - um2 * al(gm2)) * 0.5f;
    const float sm1 = (um1 + um1 * al(gm1)) * 0.5f, dm1 = (um1 - um1 * al(gm1)) * 0.5f;
    const float s0 = (u0 + u0 * al(g0)) * 0.5f, d0 = (u0 - u0 * al(g0)) * 0.5f;
    const float sp1 = (up1 + up1 * al(gp1)) * 0.5f, dp1 = (up1 - up1 * al(gp1)) * 0.5f;
    const float sp2 = (up2 + up2 * al(gp2)) * 0.5f, dp2 = (up2 - up2 * al(gp2)) * 0.5f;
    (void)sp2;
    (void)dm2;
    // upper face (cells 0 | +1) and lower face (cells -1 | 0)
    const float fu = (gp1.w + g0.w) * 0.5f * wphalf32(sm1, s0, sp1, d0, dp1, dp2);
    const float fl = (g0.w + gm1.w) * 0.5f * wphalf32(sm2, sm1, s0, dm1, d0, dp1);
    r += fu - fl;
  }
  const double v = ubase[t] - (double)(r * dt);
  if (OUT32)
    out32[t] = (float)v;
  else
    out[t] = v;
}

}  // namespace

// The mixed form's relaxing of the density rho (in place): geo (n^3 float4),
// uf0 and uf1 (n^3 floats each) are scratch.
void launch_relax32(double* rho, const double* def, const double* defp, int n, double dt, float4* geo, float* uf0,
                    float* uf1, cudaStream_t s) {
  const i64 n3 = (i64)n * n * n;
  const unsigned g = (unsigned)((n3 + 255) / 256);
  k_relax32_geom<<<g, 256, 0, s>>>(rho, def, defp, n, geo, uf0);
  k_relax32_stage<true><<<g, 256, 0, s>>>(uf0, geo, n, rho, (float)(dt / 2.0), nullptr, uf1);
  k_relax32_stage<false><<<g, 256, 0, s>>>(uf1, geo, n, rho, (float)dt, rho, nullptr);
  count_launch(3);
}

}  // namespace mmh
