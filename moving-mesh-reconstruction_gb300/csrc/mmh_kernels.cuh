// MMH reconstruction hot path -- CUDA kernels for sm_103a (GB300).
//
// Every kernel restates one routine of pandaPQY/Moving-Mesh-reconstruction
// (mmh/*.f90) with the reference's operand order.  The FP64 translation unit is
// compiled with --fmad=false, so the FP64 kernels round exactly like the CPU
// restatement and reproduce it bit for bit; the FP32 unit (mixed-precision
// inner V-cycle) keeps FMA contraction.
//
// Divisions by powers of two are written as multiplications by the exact
// reciprocal: both round the same exact quotient, so the bits are the same.
//
// Layout: a(i,j,k) of the Fortran arrays is a[i + n*(j + n*k)] (0-based),
// periodic in all three directions.  Metric coefficients are 6 planes of n^3
// (structure of arrays).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "mmh_internal.h"

namespace mmh {

typedef long long i64;

__device__ __forceinline__ int wp(int i, int n) { return i + 1 == n ? 0 : i + 1; }
__device__ __forceinline__ int wm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ i64 IDX(int i, int j, int k, int n) { return (i64)i + (i64)n * ((i64)j + (i64)n * (i64)k); }

template <class T> struct Vec16;
template <> struct Vec16<float> { typedef float4 type; };
template <> struct Vec16<double> { typedef double2 type; };

// (i, j, k) of cell t.  Grid sizes are powers of two (the library checks),
// which turns the index split into shifts; the division form stays for any
// other size.
__device__ __forceinline__ void cell_of(i64 t, int n, int& i, int& j, int& k) {
  if ((n & (n - 1)) == 0) {
    const int lg = __ffs(n) - 1;
    i = (int)t & (n - 1);
    j = (int)(t >> lg) & (n - 1);
    k = (int)(t >> (2 * lg));
    return;
  }
  i = (int)(t % n);
  i64 r = t / n;
  j = (int)(r % n);
  k = (int)(r / n);
}

// ---------------------------------------------------------------------------
// Reductions
// ---------------------------------------------------------------------------
// Exact 128-bit fixed-point sum (2^-64 resolution, |term| < 2^32), matching the
// oracle: sums do not depend on launch shape or order.
// trunc(x * 2^sh) as a 128-bit integer from the bits of x (integer operations
// only; valid for finite x with |x * 2^sh| < 2^126).
__device__ __forceinline__ __int128 fx_bits(double x, int sh) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int ex = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (ex == 0) {
    if (m == 0) return 0;
    ex = 1;
  } else {
    m |= (1ull << 52);
  }
  int s = ex - 1075 + sh;
  unsigned __int128 v;
  if (s >= 0) v = (unsigned __int128)m << s;
  else if (s > -64) v = (unsigned __int128)(m >> (-s));
  else v = 0;
  return (b >> 63) ? -(__int128)v : (__int128)v;
}
__device__ __forceinline__ __int128 fx_of(double x) { return fx_bits(x, 64); }
// trunc(x * 2^64) for a float, from its bits
__device__ __forceinline__ __int128 fx_of_f(float x) {
  const unsigned b = __float_as_uint(x);
  int ex = (int)((b >> 23) & 0xffu);
  unsigned m = b & 0x7fffffu;
  if (ex == 0) {
    if (m == 0) return 0;
    ex = 1;
  } else {
    m |= 0x800000u;
  }
  const int s = ex - 150 + 64;
  unsigned __int128 v;
  if (s >= 0) v = (unsigned __int128)m << s;
  else if (s > -32) v = (unsigned __int128)(m >> (-s));
  else v = 0;
  return (b >> 31) ? -(__int128)v : (__int128)v;
}
__device__ __forceinline__ double fx_to(unsigned long long lo, unsigned long long hi) {
  __int128 s = (__int128)(((unsigned __int128)hi << 64) | (unsigned __int128)lo);
  bool neg = s < 0;
  unsigned __int128 a = neg ? (unsigned __int128)(-s) : (unsigned __int128)s;
  unsigned long long h = (unsigned long long)(a >> 64), l = (unsigned long long)a;
  double r = __dadd_rn(__ull2double_rn(h), __dmul_rn(__ull2double_rn(l), 5.42101086242752217e-20));
  return neg ? -r : r;
}

__device__ __forceinline__ unsigned long long shfl_down_u64(unsigned long long v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}

// Block-wide reduction of a 128-bit accumulator, then two 64-bit atomics
// (two's-complement addition is order independent).  acc[0]=lo, acc[1]=hi.
__device__ __forceinline__ void fx_block_commit(__int128 v, unsigned long long* acc) {
  __shared__ unsigned long long s_lo[32], s_hi[32];
  unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)((unsigned __int128)v >> 64);
  for (int d = 16; d > 0; d >>= 1) {
    unsigned long long olo = shfl_down_u64(lo, d), ohi = shfl_down_u64(hi, d);
    unsigned long long nlo = lo + olo;
    hi = hi + ohi + (nlo < lo ? 1ull : 0ull);
    lo = nlo;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { s_lo[w] = lo; s_hi[w] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tl = 0, th = 0;
    int nw = (blockDim.x + 31) >> 5;
    for (int q = 0; q < nw; ++q) {
      unsigned long long nl = tl + s_lo[q];
      th = th + s_hi[q] + (nl < tl ? 1ull : 0ull);
      tl = nl;
    }
    unsigned long long old = atomicAdd(&acc[0], tl);
    unsigned long long carry = (old + tl < old) ? 1ull : 0ull;
    atomicAdd(&acc[1], th + carry);
  }
}

// order-preserving map of a double onto uint64 (for atomic min/max)
__device__ __forceinline__ unsigned long long ord_of(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ord(unsigned long long o) {
  unsigned long long b = (o >> 63) ? (o & 0x7FFFFFFFFFFFFFFFull) : ~o;
  return __longlong_as_double((long long)b);
}

__device__ __forceinline__ double warp_max(double v) {
  for (int d = 16; d > 0; d >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, d));
  return v;
}

// Block-wide max of non-negative values into *out (FP64 bits, atomicMax):
// the bit patterns of non-negative floating-point numbers are ordered like
// their values (NaN above inf), so the reduction is integer-only.
__device__ __forceinline__ void block_max_commit_bits(unsigned long long b, unsigned long long* out) {
  __shared__ unsigned long long s_m[32];
  for (int d = 16; d > 0; d >>= 1) {
    unsigned long long o = shfl_down_u64(b, d);
    b = o > b ? o : b;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) s_m[w] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0;
    int nw = (blockDim.x + 31) >> 5;
    for (int q = 0; q < nw; ++q) m = s_m[q] > m ? s_m[q] : m;
    atomicMax(out, m);
  }
}
__device__ __forceinline__ void block_max_commit(double v, unsigned long long* out) {
  block_max_commit_bits((unsigned long long)__double_as_longlong(v), out);
}
// FP32 values reduce as 32-bit patterns within the warp and are widened to
// FP64 once per warp (a widening is an FP64-pipe operation).
__device__ __forceinline__ void block_max_commit(float v, unsigned long long* out) {
  unsigned b = __float_as_uint(v);
  for (int d = 16; d > 0; d >>= 1) {
    unsigned o = __shfl_down_sync(0xffffffffu, b, d);
    b = o > b ? o : b;
  }
  unsigned long long w = 0;
  if ((threadIdx.x & 31) == 0) w = (unsigned long long)__double_as_longlong((double)__uint_as_float(b));
  block_max_commit_bits(w, out);
}
__device__ __forceinline__ unsigned abs_bits(float x) { return __float_as_uint(x) & 0x7FFFFFFFu; }
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ float from_bits(unsigned b) { return __uint_as_float(b); }
__device__ __forceinline__ double from_bits(unsigned long long b) { return __longlong_as_double((long long)b); }

// ---------------------------------------------------------------------------
// Curvilinear metric (cbajraw, mmh/gauss1.f90:1107-1210, non-lsquare branch)
// ---------------------------------------------------------------------------
// FastDiv (the mixed form, which is not bit-matched): urg/det once, then six
// multiplications instead of six divisions.
template <class T, bool FastDiv = false>
__global__ void k_metric(const T* __restrict__ def, const T* __restrict__ rho, int n, T di2, T* __restrict__ coef) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  T c = def[t];
  T phixx = (def[IDX(ip, j, k, n)] - T(2) * c + def[IDX(im, j, k, n)]) * di2;
  T phiyy = (def[IDX(i, jp, k, n)] - T(2) * c + def[IDX(i, jm, k, n)]) * di2;
  T phizz = (def[IDX(i, j, kp, n)] - T(2) * c + def[IDX(i, j, km, n)]) * di2;
  T phixy = (def[IDX(ip, jp, k, n)] - def[IDX(im, jp, k, n)] - def[IDX(ip, jm, k, n)] + def[IDX(im, jm, k, n)]) * di2 * T(0.25);
  T phiyz = (def[IDX(i, jp, kp, n)] - def[IDX(i, jp, km, n)] - def[IDX(i, jm, kp, n)] + def[IDX(i, jm, km, n)]) * di2 * T(0.25);
  T phixz = (def[IDX(ip, j, kp, n)] - def[IDX(im, j, kp, n)] - def[IDX(ip, j, km, n)] + def[IDX(im, j, km, n)]) * di2 * T(0.25);
  T a11 = T(1) + phixx, a12 = phixy, a13 = phixz, a22 = T(1) + phiyy, a23 = phiyz, a33 = T(1) + phizz;
  T det = a11 * a22 * a33 + T(2) * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33;
  T b11 = (a22 * a33 - a23 * a23);
  T b12 = (a13 * a23 - a12 * a33);
  T b13 = (a12 * a23 - a13 * a22);
  T b22 = (a11 * a33 - a13 * a13);
  T b23 = (a12 * a13 - a11 * a23);
  T b33 = (a11 * a22 - a12 * a12);
  if (det <= T(1.e-5)) {
    b11 = T(1); b12 = T(0); b13 = T(0); b22 = T(1); b23 = T(0); b33 = T(1); det = T(1);
  }
  const int is[3] = {im, i, ip}, js[3] = {jm, j, jp}, ks[3] = {km, k, kp};
  T urg = rho[IDX(im, jm, km, n)];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (a == 0 && b == 0 && d == 0) continue;
        urg = urg + rho[IDX(is[a], js[b], ks[d], n)];
      }
  urg = urg / T(27);
  if (FastDiv) {
    const T w = urg / det;
    coef[0 * n3 + t] = w * b11;
    coef[1 * n3 + t] = w * b12;
    coef[2 * n3 + t] = w * b13;
    coef[3 * n3 + t] = w * b22;
    coef[4 * n3 + t] = w * b23;
    coef[5 * n3 + t] = w * b33;
    return;
  }
  coef[0 * n3 + t] = urg * b11 / det;
  coef[1 * n3 + t] = urg * b12 / det;
  coef[2 * n3 + t] = urg * b13 / det;
  coef[3 * n3 + t] = urg * b22 / det;
  coef[4 * n3 + t] = urg * b23 / det;
  coef[5 * n3 + t] = urg * b33 / det;
}

// ---------------------------------------------------------------------------
// 19-point operator pieces (relaxplane gauss1.f90:950-980, calcresid :683-709)
// ---------------------------------------------------------------------------
// The 19 values of phi and 21 coefficient values one update reads.
template <class T>
struct Stencil {
  T c, ip, im, jp, jm, kp, km;                      // phi: centre and faces
  T ppk, mpk, pmk, mmk;                             // phi: in-plane edges (i+-1, j+-1, k)
  T jpkp, jmkp, jpkm, jmkm, ipkp, imkp, ipkm, imkm;  // phi: edges through k+-1
  T f1c, f1ip, f1im, f4c, f4jp, f4jm, f6c, f6kp, f6km;
  T f2jp, f2jm, f2ip, f2im, f5kp, f5km, f5jp, f5jm, f3kp, f3km, f3ip, f3im;
};

// tdiag, t1 (face terms) and t2 (cross terms) in the reference's operand order.
template <class T>
__device__ __forceinline__ void op_eval(const Stencil<T>& s, T& tdiag, T& t1, T& t2) {
  T b11p = (s.f1ip + s.f1c) * T(0.5);
  T b11m = (s.f1im + s.f1c) * T(0.5);
  T b22p = (s.f4jp + s.f4c) * T(0.5);
  T b22m = (s.f4jm + s.f4c) * T(0.5);
  T b33p = (s.f6kp + s.f6c) * T(0.5);
  T b33m = (s.f6km + s.f6c) * T(0.5);
  tdiag = -(b11p + b11m + b22p + b22m + b33p + b33m);
  t1 = (b11p * s.ip + b11m * s.im + b22p * s.jp + b22m * s.jm + b33p * s.kp + b33m * s.km);
  t2 = ((s.ppk - s.mpk) * s.f2jp
        - (s.pmk - s.mmk) * s.f2jm
        + (s.ppk - s.pmk) * s.f2ip
        - (s.mpk - s.mmk) * s.f2im
        + (s.jpkp - s.jmkp) * s.f5kp
        - (s.jpkm - s.jmkm) * s.f5km
        + (s.jpkp - s.jpkm) * s.f5jp
        - (s.jmkp - s.jmkm) * s.f5jm
        + (s.ipkp - s.imkp) * s.f3kp
        - (s.ipkm - s.imkm) * s.f3km
        + (s.ipkp - s.ipkm) * s.f3ip
        - (s.imkp - s.imkm) * s.f3im) * T(0.25);
}

// The Gauss-Seidel update's division: IEEE in FP64 (the oracle's bits); the
// fast reciprocal-based division in FP32 (the mixed form's smoother, which is
// not bit-matched; within 2 ulp).
__device__ __forceinline__ double gs_div(double a, double b) { return a / b; }
__device__ __forceinline__ float gs_div(float a, float b) { return __fdividef(a, b); }

// Gather the stencil of cell (i,j,k) from global memory.
template <class T>
__device__ __forceinline__ void op_terms(const T* __restrict__ phi, const T* __restrict__ coef, int n, i64 n3, int i,
                                         int j, int k, T& tdiag, T& t1, T& t2) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  const T* f1 = coef;
  const T* f2 = coef + n3;
  const T* f3 = coef + 2 * n3;
  const T* f4 = coef + 3 * n3;
  const T* f5 = coef + 4 * n3;
  const T* f6 = coef + 5 * n3;
  i64 c = IDX(i, j, k, n);
  i64 cip = IDX(ip, j, k, n), cim = IDX(im, j, k, n), cjp = IDX(i, jp, k, n), cjm = IDX(i, jm, k, n);
  i64 ckp = IDX(i, j, kp, n), ckm = IDX(i, j, km, n);
  Stencil<T> s;
  s.c = phi[c]; s.ip = phi[cip]; s.im = phi[cim]; s.jp = phi[cjp]; s.jm = phi[cjm]; s.kp = phi[ckp]; s.km = phi[ckm];
  s.ppk = phi[IDX(ip, jp, k, n)]; s.mpk = phi[IDX(im, jp, k, n)]; s.pmk = phi[IDX(ip, jm, k, n)];
  s.mmk = phi[IDX(im, jm, k, n)];
  s.jpkp = phi[IDX(i, jp, kp, n)]; s.jmkp = phi[IDX(i, jm, kp, n)]; s.jpkm = phi[IDX(i, jp, km, n)];
  s.jmkm = phi[IDX(i, jm, km, n)];
  s.ipkp = phi[IDX(ip, j, kp, n)]; s.imkp = phi[IDX(im, j, kp, n)]; s.ipkm = phi[IDX(ip, j, km, n)];
  s.imkm = phi[IDX(im, j, km, n)];
  s.f1c = f1[c]; s.f1ip = f1[cip]; s.f1im = f1[cim];
  s.f4c = f4[c]; s.f4jp = f4[cjp]; s.f4jm = f4[cjm];
  s.f6c = f6[c]; s.f6kp = f6[ckp]; s.f6km = f6[ckm];
  s.f2jp = f2[cjp]; s.f2jm = f2[cjm]; s.f2ip = f2[cip]; s.f2im = f2[cim];
  s.f5kp = f5[ckp]; s.f5km = f5[ckm]; s.f5jp = f5[cjp]; s.f5jm = f5[cjm];
  s.f3kp = f3[ckp]; s.f3km = f3[ckm]; s.f3ip = f3[cip]; s.f3im = f3[cim];
  op_eval(s, tdiag, t1, t2);
}

// One colour of the 8-colour Gauss-Seidel sweep: planes with k%2 == kpar,
// i%2 == io, j%2 == jo (0-based).  Sweep order kpar(0,1) x io(0,1) x jo(0,1)
// reproduces the reference's plane schedule (r1lax) exactly.
template <class T>
__global__ void k_gs_colour(T* __restrict__ phi, const T* __restrict__ rhs, const T* __restrict__ coef, int n, T dx2,
                            int kpar, int io, int jo) {
  int h = n >> 1;
  i64 tot = (i64)h * h * h;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tot) return;
  int ti = (int)(t % h);
  i64 r = t / h;
  int tj = (int)(r % h), tk = (int)(r / h);
  int i = 2 * ti + io, j = 2 * tj + jo, k = 2 * tk + kpar;
  i64 n3 = (i64)n * n * n;
  T tdiag, t1, t2;
  op_terms(phi, coef, n, n3, i, j, k, tdiag, t1, t2);
  i64 c = IDX(i, j, k, n);
  phi[c] = gs_div(rhs[c] * dx2 - t1 - t2, tdiag);
}

// nsweeps full 8-colour sweeps of a small grid (n <= 16) by one CTA: the
// colour phases are separated by block barriers instead of kernel launches.
template <class T>
__global__ void __launch_bounds__(512) k_gs_small(T* __restrict__ phi, const T* __restrict__ rhs,
                                                   const T* __restrict__ coef, int n, T dx2, int nsweeps) {
  const int h = n >> 1;
  const int tot = h * h * h;
  const i64 n3 = (i64)n * n * n;
  for (int sw = 0; sw < nsweeps; ++sw)
    for (int q = 0; q < 8; ++q) {
      const int kpar = q >> 2, io = (q >> 1) & 1, jo = q & 1;
      for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        int ti = t % h, tj = (t / h) % h, tk = t / (h * h);
        int i = 2 * ti + io, j = 2 * tj + jo, k = 2 * tk + kpar;
        T tdiag, t1, t2;
        op_terms(phi, coef, n, n3, i, j, k, tdiag, t1, t2);
        i64 c = IDX(i, j, k, n);
        phi[c] = gs_div(rhs[c] * dx2 - t1 - t2, tdiag);
      }
      __syncthreads();
    }
}

// The same sweeps with the whole grid held in shared memory (phi, rhs and the
// six coefficients: 8*n^3 words, n <= 8), read once and written back once; a
// colour phase then costs shared-memory latency instead of L2 latency.  Used
// for the coarsest levels, where one CTA runs tens of sweeps.
template <class T>
__global__ void __launch_bounds__(512) k_gs_small_sm(T* __restrict__ phi, const T* __restrict__ rhs,
                                                      const T* __restrict__ coef, int n, T dx2, int nsweeps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int h = n >> 1;
  const int tot = h * h * h;
  const int n3 = n * n * n;
  T* sp = reinterpret_cast<T*>(smem_raw);
  T* sr = sp + n3;
  T* sc = sr + n3;
  for (int e = threadIdx.x; e < n3; e += blockDim.x) {
    sp[e] = phi[e];
    sr[e] = rhs[e];
  }
  for (int e = threadIdx.x; e < 6 * n3; e += blockDim.x) sc[e] = coef[e];
  __syncthreads();
  for (int sw = 0; sw < nsweeps; ++sw)
    for (int q = 0; q < 8; ++q) {
      const int kpar = q >> 2, io = (q >> 1) & 1, jo = q & 1;
      for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        int ti = t % h, tj = (t / h) % h, tk = t / (h * h);
        int i = 2 * ti + io, j = 2 * tj + jo, k = 2 * tk + kpar;
        T tdiag, t1, t2;
        op_terms(sp, sc, n, (i64)n3, i, j, k, tdiag, t1, t2);
        i64 c = IDX(i, j, k, n);
        sp[c] = gs_div(sr[c] * dx2 - t1 - t2, tdiag);
      }
      __syncthreads();
    }
  for (int e = threadIdx.x; e < n3; e += blockDim.x) phi[e] = sp[e];
}

// Tile geometry of the fused plane kernel.  A tile holds TX x TY interior
// cells of one plane and a halo of HB = 4 cells: W x HT cells.  Colour
// q = 2*io + jo (x parity io, y parity jo) is applied on NXC = W/2 - 2 cells
// of each of its rows, x = XS(io) + 2m (XS = 4 for even x, 1 for odd x), and
// on the rows ys(q) = HB-2+q, ys(q)+2, ... (ny(q) = TY/2+3-q rows).  With the
// colours in the reference's order (io outer, jo inner), the later colours
// read updated cells of the earlier ones within one cell in x and within
// 3-q rows in y, so this region covers everything they read and the interior
// ends exactly as after the four global colour phases; the extra cells a
// colour computes beyond that are never read.  Row 0 of the tile is never
// read and is not loaded.
//
// Shared memory holds the fields read at neighbours (phi of planes P-1, P,
// P+1 and coefficients 1-5 of P) with the even rows first and the odd rows
// OFFB words after them, a pitch of Q words between two rows of one parity,
// and every row split into its even-x and its odd-x half (H2 words each).
// Cell m of row t of a colour then sits at word const + Q*t + m, and
// Q = NXC (mod 32) puts the words of any 32 consecutive cells of a colour in
// 32 different banks (16 different bank pairs for 8-byte words): a colour
// phase reads shared memory without bank conflicts.  Q, OFFB and H2 are
// even, so the cells x0, x0+2 of a 16-byte group are one aligned pair.  The
// fields read only at the cell itself (rhs, coefficient 6 of P, coefficients
// 3, 5, 6 of P-1 and P+1) are read from global memory by the thread that
// updates the cell.
template <class T, int TX, int TY>
struct GsGeom {
  static constexpr int HB = 4, W = TX + 2 * HB, HT = TY + 2 * HB, H2 = W / 2, NXC = H2 - 2;
  static constexpr int Q = NXC + 32 * ((W - NXC + 31) / 32);
  static constexpr int OFFB0 = (HT / 2) * Q;
  static constexpr int OFFB = OFFB0 + ((30 - OFFB0 % 32) + 32) % 32;  // first odd row (fewer store conflicts)
  static constexpr int SF = OFFB + (HT / 2) * Q;                       // words of one field
  static constexpr int NSF = 8;
  static constexpr int WORDS = NSF * SF;
  static __device__ __forceinline__ constexpr int XS(int io) { return io ? 1 : HB; }
  static __device__ __forceinline__ constexpr int ys(int q) { return HB - 2 + q; }
  static __device__ __forceinline__ constexpr int ny(int q) { return TY / 2 + 3 - q; }
  static __device__ __forceinline__ int word(int x, int y) {
    return (y & 1) * OFFB + (y >> 1) * Q + (x & 1) * H2 + (x >> 1);
  }
  static_assert(Q >= W && (Q - NXC) % 32 == 0 && Q % 2 == 0 && OFFB % 2 == 0, "row pitch");
  static_assert(HT % 2 == 0 && TX % 4 == 0 && HB == 4, "tile shape");
  static_assert(NXC * (TY / 2 + 3) <= 256, "one cell per thread and colour (256 threads)");
};

// Store one 16-byte group (cells x0..x0+VW-1 of tile row y) into a field at
// its word sw = word(x0, y); read one back.
__device__ __forceinline__ void gs_put(float* f, int sw, int h2, const float4& v) {
  *reinterpret_cast<float2*>(f + sw) = make_float2(v.x, v.z);
  *reinterpret_cast<float2*>(f + sw + h2) = make_float2(v.y, v.w);
}
__device__ __forceinline__ void gs_put(double* f, int sw, int h2, const double2& v) {
  f[sw] = v.x;
  f[sw + h2] = v.y;
}
__device__ __forceinline__ float4 gs_get(const float* f, int sw, int h2) {
  float2 e = *reinterpret_cast<const float2*>(f + sw);
  float2 o = *reinterpret_cast<const float2*>(f + sw + h2);
  return make_float4(e.x, o.x, e.y, o.y);
}
__device__ __forceinline__ double2 gs_get(const double* f, int sw, int h2) { return make_double2(f[sw], f[sw + h2]); }

// All four in-plane colours of one plane P (k%2 == kpar) for one tile (see
// GsGeom).  The half sweep reads its own planes from src, the neighbour planes
// P+-1 (not written during the half sweep) from nbr, and writes dst != src,
// so no tile can read a halo that another tile has already updated.  Needs
// n >= TX+8 and n >= TY+8.  The register budget of 4 CTAs per SM lets the
// compiler keep the tile's global loads in flight together.
// Z = 1: the planes being updated are zero (src is not read); Z = 2: the
// neighbour planes are zero too (nbr is not read either).  The first sweep
// from a zero field runs its half sweeps with Z = 2 and Z = 1, in place: no
// tile reads a plane that the half sweep writes.  A loaded zero and the
// constant zero give the same results.
template <class T, int TX, int TY, int Z = 0>
__global__ void __launch_bounds__(256, 4) k_gs_plane(const T* __restrict__ src, const T* __restrict__ nbr,
                                                     T* __restrict__ dst, const T* __restrict__ rhs,
                                                     const T* __restrict__ coef, int n, T dx2, int kpar) {
  typedef GsGeom<T, TX, TY> G;
  constexpr int HB = G::HB, W = G::W, HT = G::HT, H2 = G::H2, NXC = G::NXC, Q = G::Q, OFFB = G::OFFB;
  constexpr int SF = G::SF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const i64 n2 = (i64)n * n, n3 = n2 * n;
  const int i0 = blockIdx.x * TX - HB, j0 = blockIdx.y * TY - HB, k = 2 * blockIdx.z + kpar;
  const int kmn = wm(k, n), kpn = wp(k, n);
  // 16-byte loads: a row segment of the tile starts 16-byte aligned (i0 is a
  // multiple of 4 elements) and a 16-byte group never straddles the periodic
  // wrap (n is a multiple of the group), so each group is one aligned load.
  typedef typename Vec16<T>::type V;
  constexpr int VW = 16 / (int)sizeof(T), NV = W / VW, NVT = NV * (HT - 1);
  const V* vsrc = reinterpret_cast<const V*>(src);
  const V* vnbr = reinterpret_cast<const V*>(nbr);
  const V* vcoef = reinterpret_cast<const V*>(coef);
  const i64 nv3 = n3 / VW;
  const T* f3 = coef + 2 * n3;
  const T* f5 = coef + 4 * n3;
  const T* f6 = coef + 5 * n3;
  // The fields read only at the cell itself (rhs, coefficient 6 of P,
  // coefficients 3, 5, 6 of P+-1) of this thread's cell of colour q (at most
  // one cell per colour): colour 0's are requested before the tile loads and
  // colour q+1's while colour q computes, so their latency overlaps work.
  auto centre = [&](int q, T* o) {
    const int io = q >> 1;
    const int e = threadIdx.x;
    if (e >= NXC * G::ny(q)) return;
    const int m = e % NXC, t = e / NXC;
    int gi = i0 + G::XS(io) + 2 * m, gj = j0 + G::ys(q) + 2 * t;
    gi += (gi < 0) ? n : ((gi >= n) ? -n : 0);
    gj += (gj < 0) ? n : ((gj >= n) ? -n : 0);
    const i64 g = (i64)gi + (i64)n * gj;
    const i64 gt = g + n2 * k, gm = g + n2 * kmn, gp = g + n2 * kpn;
    o[0] = rhs[gt]; o[1] = f6[gt]; o[2] = f6[gm]; o[3] = f6[gp];
    o[4] = f3[gm]; o[5] = f5[gm]; o[6] = f3[gp]; o[7] = f5[gp];
  };
  T pre[8];
  centre(0, pre);
  for (int e = threadIdx.x; e < NVT; e += blockDim.x) {
    const int xv = e % NV, y = 1 + e / NV, x0 = xv * VW;
    int gi = i0 + x0, gj = j0 + y;
    gi += (gi < 0) ? n : ((gi >= n) ? -n : 0);
    gj += (gj < 0) ? n : ((gj >= n) ? -n : 0);
    const i64 b = (i64)gi + (i64)n * gj;
    const i64 cP = (b + n2 * k) / VW, cm = (b + n2 * kmn) / VW, cp = (b + n2 * kpn) / VW;
    V v[8];
    if (Z == 0) v[0] = vsrc[cP];
    else v[0] = V{};
    if (Z < 2) {
      v[1] = vnbr[cm];
      v[2] = vnbr[cp];
    }
#pragma unroll
    for (int f = 0; f < 5; ++f) v[3 + f] = vcoef[f * nv3 + cP];
    const int sw = G::word(x0, y);
#pragma unroll
    for (int f = 0; f < 8; ++f)
      if (Z < 2 || (f != 1 && f != 2)) gs_put(sm + f * SF, sw, H2, v[f]);
  }
  __syncthreads();
  T* sP = sm;
  const T* sKm = sm + 1 * SF;
  const T* sKp = sm + 2 * SF;
  const T* F1 = sm + 3 * SF;
  const T* F2 = sm + 4 * SF;
  const T* F3 = sm + 5 * SF;
  const T* F4 = sm + 6 * SF;
  const T* F5 = sm + 7 * SF;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    T cur[8];
#pragma unroll
    for (int z = 0; z < 8; ++z) cur[z] = pre[z];
    if (q < 3) centre(q + 1, pre);
    const int io = q >> 1, jo = q & 1;
    const int cnt = NXC * G::ny(q);
    // word offsets of the x+-1 and y+-1 neighbours (constant within a colour)
    const int oxp = io ? 1 - H2 : H2, oxm = io ? -H2 : H2 - 1;
    const int oyp = jo ? Q - OFFB : OFFB, oym = jo ? -OFFB : OFFB - Q;
    // one cell per thread: a colour has at most NXC * ny(0) <= 256 cells
    if (threadIdx.x < cnt) {
      const int e = threadIdx.x;
      const int m = e % NXC, t = e / NXC;
      const int x = G::XS(io) + 2 * m, y = G::ys(q) + 2 * t;
      const int c = G::word(x, y);
      const int cxp = c + oxp, cxm = c + oxm, cyp = c + oyp, cym = c + oym;
      Stencil<T> st;
      st.f6c = cur[1]; st.f6km = cur[2]; st.f6kp = cur[3];
      st.f3km = cur[4]; st.f5km = cur[5]; st.f3kp = cur[6]; st.f5kp = cur[7];
      const T r = cur[0];
      st.c = sP[c]; st.ip = sP[cxp]; st.im = sP[cxm]; st.jp = sP[cyp]; st.jm = sP[cym];
      st.ppk = sP[cxp + oyp]; st.mpk = sP[cxm + oyp]; st.pmk = sP[cxp + oym]; st.mmk = sP[cxm + oym];
      if (Z < 2) {
        st.kp = sKp[c]; st.km = sKm[c];
        st.jpkp = sKp[cyp]; st.jmkp = sKp[cym]; st.jpkm = sKm[cyp]; st.jmkm = sKm[cym];
        st.ipkp = sKp[cxp]; st.imkp = sKp[cxm]; st.ipkm = sKm[cxp]; st.imkm = sKm[cxm];
      } else {
        st.kp = st.km = st.jpkp = st.jmkp = st.jpkm = st.jmkm = st.ipkp = st.imkp = st.ipkm = st.imkm = T(0);
      }
      st.f1c = F1[c]; st.f1ip = F1[cxp]; st.f1im = F1[cxm];
      st.f4c = F4[c]; st.f4jp = F4[cyp]; st.f4jm = F4[cym];
      st.f2jp = F2[cyp]; st.f2jm = F2[cym]; st.f2ip = F2[cxp]; st.f2im = F2[cxm];
      st.f5jp = F5[cyp]; st.f5jm = F5[cym];
      st.f3ip = F3[cxp]; st.f3im = F3[cxm];
      T tdiag, t1, t2;
      op_eval(st, tdiag, t1, t2);
      sP[c] = gs_div(r * dx2 - t1 - t2, tdiag);
    }
    __syncthreads();
  }
  constexpr int NVI = TX / VW;
  V* vdst = reinterpret_cast<V*>(dst);
  for (int e = threadIdx.x; e < NVI * TY; e += blockDim.x) {
    const int x0 = HB + (e % NVI) * VW, y = HB + e / NVI;
    vdst[((i64)(i0 + x0) + (i64)n * (j0 + y) + n2 * k) / VW] = gs_get(sP, G::word(x0, y), H2);
  }
}

// cp.async helpers: 16-byte global -> shared copies that bypass registers
// (cp.async.cg: cached in L2 only), committed and waited for as groups.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// FP32 half sweep by strips marching in y (the same updates as k_gs_plane,
// operand for operand, so the same bits).  A CTA owns a strip of 64 cells in
// x and LY sub-rows (2 LY cell rows: sub-row r holds cell rows 2r and 2r+1) of
// one plane P of parity kpar.  Within a plane the four colours (io, jo) run in
// the order (0,0), (0,1), (1,0), (1,1); an update reads its 8 in-plane
// neighbours, and only the colours before it may have been updated.  So the
// colours can advance as a wavefront: at step s, colour q updates sub-row
// s - lag[q] with lag = (0, 2, 3, 5).  With those lags every value a colour
// reads is either final (an earlier colour's rows <= r + 1, finished at an
// earlier step) or still old (a later colour's rows >= r - 1, not reached yet),
// and no two updates of one step touch a value the other reads, so a step
// needs one barrier instead of four per tile, and the recomputed halo of a
// tile (a third of the updates for 32 x 16 tiles) shrinks to the strip's two
// ends and one extra column of the first two colours.
//   Shared memory keeps a ring of R sub-rows of the 8 fields read at
// neighbours (phi of P, P-1, P+1, coefficients 1-5 of P), each sub-row split
// into its four colours (sub-cells -2 .. 33: cells x0-4 .. x0+67), so a warp's
// 32 lanes read 32 consecutive words.  Step s reads sub-rows s-5 .. s, writes
// back sub-row s-6 (final since step s-1) and stores sub-row s+1 into the
// ring from 16-byte loads issued at the start of the step.  The fields read
// at the cell only (rhs, coefficient 6 of P, coefficients 3, 5, 6 of P+-1)
// are loaded one step ahead.  (Loading two sub-rows ahead in alternating
// register sets was slower: its registers allow 4 CTAs per SM instead of 5;
// so was a 64-register build for 6 CTAs per SM.)
// Warps 0-3 take colours 0-3 (sub-cells 0..31); warp 4 takes sub-cell 32 of
// colours 0 and 1 (x0+64, read by the last two colours at x0+63) and the
// write-back.
// Z as in k_gs_plane.  Needs n >= 64 and LY | n/2.
struct StripGeom {
  // the ring holds sub-rows s-6 .. s+1 at step s
  static constexpr int SW = 64, PITCH = 36, ROWW = 4 * PITCH, R = 8, FW = R * ROWW, NF = 8;
  static constexpr int WORDS = NF * FW, NT = 160, NSTAGE = NF * 2 * 18;
  // ring offset of sub-cell s (-2 <= s < 34) of colour (io, jo) in ring slot sl
  static __device__ __forceinline__ int at(int sl, int io, int jo, int s) {
    return sl * ROWW + (2 * jo + io) * PITCH + s + 2;
  }
  static __device__ __forceinline__ int slot(int r) { return r & (R - 1); }
};

// JO < 0: the colour's jo is the runtime value jo (one path for the two
// lanes of the last warp, which update colours (0,0) and (0,1) together).
template <int IO, int JO, int Z>
__device__ __forceinline__ float strip_update(const float* __restrict__ sm, int sl, int slm, int slp, int s,
                                              const float* cur, float dx2, int jo = JO) {
  typedef StripGeom G;
  const float* P = sm;
  const float* Km = sm + G::FW;
  const float* Kp = sm + 2 * G::FW;
  const float* F1 = sm + 3 * G::FW;
  const float* F2 = sm + 4 * G::FW;
  const float* F3 = sm + 5 * G::FW;
  const float* F4 = sm + 6 * G::FW;
  const float* F5 = sm + 7 * G::FW;
  // neighbours in x: the other io's sub-row; in y: the other jo's sub-row
  // (slots of rows r-1 / r for jo = 0, r / r+1 for jo = 1)
  const int J = JO >= 0 ? JO : jo;
  const int sy_p = J ? slp : sl, sy_m = J ? sl : slm;
  const int c = G::at(sl, IO, J, s);
  const int xp = G::at(sl, 1 - IO, J, IO ? s + 1 : s), xm = G::at(sl, 1 - IO, J, IO ? s : s - 1);
  const int yp = G::at(sy_p, IO, 1 - J, s), ym = G::at(sy_m, IO, 1 - J, s);
  const int ypxp = G::at(sy_p, 1 - IO, 1 - J, IO ? s + 1 : s);
  const int ypxm = G::at(sy_p, 1 - IO, 1 - J, IO ? s : s - 1);
  const int ymxp = G::at(sy_m, 1 - IO, 1 - J, IO ? s + 1 : s);
  const int ymxm = G::at(sy_m, 1 - IO, 1 - J, IO ? s : s - 1);
  Stencil<float> st;
  st.f6c = cur[1]; st.f6km = cur[2]; st.f6kp = cur[3];
  st.f3km = cur[4]; st.f5km = cur[5]; st.f3kp = cur[6]; st.f5kp = cur[7];
  st.c = P[c]; st.ip = P[xp]; st.im = P[xm]; st.jp = P[yp]; st.jm = P[ym];
  st.ppk = P[ypxp]; st.mpk = P[ypxm]; st.pmk = P[ymxp]; st.mmk = P[ymxm];
  if (Z < 2) {
    st.kp = Kp[c]; st.km = Km[c];
    st.jpkp = Kp[yp]; st.jmkp = Kp[ym]; st.jpkm = Km[yp]; st.jmkm = Km[ym];
    st.ipkp = Kp[xp]; st.imkp = Kp[xm]; st.ipkm = Km[xp]; st.imkm = Km[xm];
  } else {
    st.kp = st.km = st.jpkp = st.jmkp = st.jpkm = st.jmkm = st.ipkp = st.imkp = st.ipkm = st.imkm = 0.0f;
  }
  st.f1c = F1[c]; st.f1ip = F1[xp]; st.f1im = F1[xm];
  st.f4c = F4[c]; st.f4jp = F4[yp]; st.f4jm = F4[ym];
  st.f2jp = F2[yp]; st.f2jm = F2[ym]; st.f2ip = F2[xp]; st.f2im = F2[xm];
  st.f5jp = F5[yp]; st.f5jm = F5[ym];
  st.f3ip = F3[xp]; st.f3im = F3[xm];
  float tdiag, t1, t2;
  op_eval(st, tdiag, t1, t2);
  return gs_div(cur[0] * dx2 - t1 - t2, tdiag);
}

template <int LY, int Z>
__global__ void __launch_bounds__(160, 5) k_gs_strip(const float* __restrict__ src, const float* __restrict__ nbr,
                                                     float* __restrict__ dst, const float* __restrict__ rhs,
                                                     const float* __restrict__ coef, int n, float dx2, int kpar) {
  typedef StripGeom G;
  __shared__ __align__(16) float sm[G::WORDS];
  const int m = n >> 1;
  const i64 n2 = (i64)n * n, n3 = n2 * n;
  const int x0 = blockIdx.x * G::SW, Y0 = blockIdx.y * LY, k = 2 * blockIdx.z + kpar;
  const int kmn = wm(k, n), kpn = wp(k, n);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto wrow = [&](int r) { return r < 0 ? r + m : (r >= m ? r - m : r); };
  const int rlast = Y0 + LY + 1;  // last staged sub-row
  // ---- staging: item e of a sub-row is (field f, cell row jo, 16-byte group g);
  // a thread's items are the same in every sub-row, so their global column
  // pointers and shared offsets are formed once ----
  const float* gcol[2];
  int soff[2], gjo[2];
  bool gld[2], gst[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int e = tid + h * G::NT;
    const int f = e / 36, jo = (e / 18) & 1, g = e % 18;
    gst[h] = e < G::NSTAGE && !(Z == 2 && (f == 1 || f == 2));
    gld[h] = gst[h] && !(Z >= 1 && f == 0);
    int x = x0 - 4 + 4 * g;
    x += (x < 0) ? n : ((x >= n) ? -n : 0);
    const float* base = f == 0 ? src + n2 * k
                        : f == 1 ? nbr + n2 * kmn
                        : f == 2 ? nbr + n2 * kpn
                                 : coef + (i64)(f - 3) * n3 + n2 * k;
    gcol[h] = base + x;
    gjo[h] = jo;
    soff[h] = f * G::FW + G::at(0, 0, jo, 2 * g - 2);
  }
  auto stage_load = [&](int r, float4(&ld)[2]) {
    if (r > rlast) return;
    const i64 yb = (i64)n * (2 * wrow(r));
#pragma unroll
    for (int h = 0; h < 2; ++h)
      if (gld[h]) ld[h] = *reinterpret_cast<const float4*>(gcol[h] + yb + (gjo[h] ? n : 0));
  };
  auto stage_store = [&](int r, const float4(&ld)[2]) {
    if (r > rlast) return;
    const int so = G::slot(r) * G::ROWW;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!gst[h]) continue;
      const float4 v = (Z >= 1 && !gld[h]) ? make_float4(0.f, 0.f, 0.f, 0.f) : ld[h];
      float* row = sm + soff[h] + so;
      *reinterpret_cast<float2*>(row) = make_float2(v.x, v.z);
      *reinterpret_cast<float2*>(row + G::PITCH) = make_float2(v.y, v.w);
    }
  };
  // ---- this thread's cell: colour q, sub-cell sc ----
  const int q = warp < 4 ? warp : lane;
  const bool computes = warp < 4 || lane < 2;
  const int sc = warp < 4 ? lane : 32;
  const int io = q >> 1, jo = q & 1;
  const int lag = q == 0 ? 0 : (q == 1 ? 2 : (q == 2 ? 3 : 5));
  const int rlo = Y0 + (q < 2 ? -1 : 0), rhi = Y0 + (q == 0 ? LY + 1 : (q == 3 ? LY - 1 : LY));
  int xc = x0 + 2 * sc + io;
  xc -= (xc >= n) ? n : 0;
  // the 8 fields read at the cell of sub-row r (nothing outside the colour's rows),
  // from column pointers formed once
  const float* cr = rhs + (xc + n2 * k + (jo ? n : 0));
  const float* c6 = coef + (5 * n3 + xc + n2 * k + (jo ? n : 0));
  const float* c6m = coef + (5 * n3 + xc + n2 * kmn + (jo ? n : 0));
  const float* c6p = coef + (5 * n3 + xc + n2 * kpn + (jo ? n : 0));
  const i64 d3m = (i64)3 * n3;       // coefficient 6 -> 3
  const i64 d5 = n3;                 // coefficient 6 -> 5 is -n3
  auto centre = [&](int r, float(&o)[8]) {
    if (!computes || r < rlo || r > rhi) return;
    const i64 yb = (i64)n * (2 * wrow(r));
    o[0] = cr[yb]; o[1] = c6[yb]; o[2] = c6m[yb]; o[3] = c6p[yb];
    o[4] = c6m[yb - d3m]; o[5] = c6m[yb - d5]; o[6] = c6p[yb - d3m]; o[7] = c6p[yb - d5];
  };
  const int s0 = Y0 - 1, s1 = Y0 + LY + 5;
  float4 ld[2];
  float pre[8];
  // sub-rows Y0-2 and Y0-1 (read by the first step)
  stage_load(Y0 - 2, ld);
  stage_store(Y0 - 2, ld);
  stage_load(Y0 - 1, ld);
  stage_store(Y0 - 1, ld);
  centre(s0 - lag, pre);
  __syncthreads();
  // step s: the colour updates of step s with the cell fields in pre (then
  // refilled with those of the colour's next row), the write-back of sub-row
  // s-6, and sub-row s+1 loaded and stored
  for (int s = s0; s <= s1; ++s) {
    stage_load(s + 1, ld);
    const int r = s - lag;
    if (computes && r >= rlo && r <= rhi) {
      float cur[8];
#pragma unroll
      for (int z = 0; z < 8; ++z) cur[z] = pre[z];
      centre(r + 1, pre);
      const int sl = G::slot(r), slm = G::slot(r - 1), slp = G::slot(r + 1);
      float v;
      if (warp == 4) {
        v = strip_update<0, -1, Z>(sm, sl, slm, slp, sc, cur, dx2, jo);
      } else {
        switch (q) {
          case 0: v = strip_update<0, 0, Z>(sm, sl, slm, slp, sc, cur, dx2); break;
          case 1: v = strip_update<0, 1, Z>(sm, sl, slm, slp, sc, cur, dx2); break;
          case 2: v = strip_update<1, 0, Z>(sm, sl, slm, slp, sc, cur, dx2); break;
          default: v = strip_update<1, 1, Z>(sm, sl, slm, slp, sc, cur, dx2); break;
        }
      }
      sm[G::at(sl, io, jo, sc)] = v;
    } else if (r + 1 == rlo) {
      centre(rlo, pre);  // the colour starts at the next step
    }
    const int rb = s - 6;
    if (warp == 4 && rb >= Y0 && rb < Y0 + LY) {
      const int wj = lane >> 4, g = lane & 15, sl = G::slot(rb);
      const float2 a = *reinterpret_cast<const float2*>(sm + G::at(sl, 0, wj, 2 * g));
      const float2 b = *reinterpret_cast<const float2*>(sm + G::at(sl, 1, wj, 2 * g));
      const i64 o = (i64)(x0 + 4 * g) + (i64)n * (2 * wrow(rb) + wj) + n2 * k;
      *reinterpret_cast<float4*>(dst + o) = make_float4(a.x, b.x, a.y, b.y);
    }
    stage_store(s + 1, ld);
    __syncthreads();
  }
}

// Residual r = rhs - L[phi] on every cell (calcresid), max-norm into maxbits.
// r may be null; r32 (float copy of the residual) may be null.  Contract
// only names a separate instantiation: the translation unit that instantiates
// it decides whether multiply-adds are fused.
template <class T, bool Contract = false>
__global__ void k_residual(const T* __restrict__ phi, const T* __restrict__ rhs, const T* __restrict__ coef, int n,
                           T di2, T* __restrict__ r, float* __restrict__ r32, unsigned long long* maxbits) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  T m = T(0);
  if (t < n3) {
    int i, j, k;
    cell_of(t, n, i, j, k);
    T tdiag, t1, t2;
    op_terms(phi, coef, n, n3, i, j, k, tdiag, t1, t2);
    T tr = rhs[t] - (t1 + t2 + tdiag * phi[t]) * di2;
    if (r) r[t] = tr;
    if (r32) r32[t] = (float)tr;
    m = fabs(tr);
  }
  if (maxbits) block_max_commit(m, maxbits);
}

// The residual (MODE 0: r = rhs - L[phi], calcresid) or the operator (MODE 1:
// q = L[p]) of every cell of one TX x TY tile of one plane.  The fields the
// 19-point stencil reads at neighbours (phi of planes P-1, P, P+1 and
// coefficients 1-5 of P) are staged in shared memory, row-major with an x halo
// of 4 (aligned 16-byte loads) and a y halo of 1; the fields read only at the
// cell itself come straight from global memory.  A warp covers 32 consecutive
// cells of a row, so the shared reads are conflict-free and the global
// accesses coalesced.  Same arithmetic as k_residual / k_apply.  Needs
// n >= TX and n a multiple of TY.
template <class T, int MODE, bool Contract = false>
__global__ void __launch_bounds__(256) k_stencil_plane(const T* __restrict__ phi, const T* __restrict__ rhs,
                                                       const T* __restrict__ coef, int n, T di2, T* __restrict__ out,
                                                       float* __restrict__ out32, unsigned long long* maxbits) {
  constexpr int TX = 32, TY = 16, HX = 4, W = TX + 2 * HX, HT = TY + 2, S = W * HT;
  __shared__ __align__(16) T sm[8 * S];  // 0 phi(P), 1 phi(P-1), 2 phi(P+1), 3-7 f1..f5(P)
  const i64 n2 = (i64)n * n, n3 = n2 * n;
  const int i0 = blockIdx.x * TX - HX, j0 = blockIdx.y * TY - 1, k = blockIdx.z;
  const int kmn = wm(k, n), kpn = wp(k, n);
  typedef typename Vec16<T>::type V;
  constexpr int VW = 16 / (int)sizeof(T), NV = W / VW, NVT = NV * HT;
  const V* vphi = reinterpret_cast<const V*>(phi);
  const V* vcoef = reinterpret_cast<const V*>(coef);
  const i64 nv3 = n3 / VW;
  // the fields read only at the thread's own cells are requested first, so
  // their latency overlaps the tile loads
  constexpr int NCELL = TY / (256 / TX);
  const int tx = threadIdx.x % TX, ty0 = threadIdx.x / TX;
  const T* f3 = coef + 2 * n3;
  const T* f5 = coef + 4 * n3;
  const T* f6 = coef + 5 * n3;
  T c6[NCELL], c6p[NCELL], c6m[NCELL], c5p[NCELL], c5m[NCELL], c3p[NCELL], c3m[NCELL], cr[NCELL];
#pragma unroll
  for (int q = 0; q < NCELL; ++q) {
    const int ty = ty0 + q * (256 / TX);
    const i64 g = (i64)(blockIdx.x * TX + tx) + (i64)n * (blockIdx.y * TY + ty);
    const i64 gt = g + n2 * k, gm = g + n2 * kmn, gp = g + n2 * kpn;
    c6[q] = f6[gt]; c6p[q] = f6[gp]; c6m[q] = f6[gm];
    c5p[q] = f5[gp]; c5m[q] = f5[gm];
    c3p[q] = f3[gp]; c3m[q] = f3[gm];
    cr[q] = MODE == 0 ? rhs[gt] : T(0);
  }
  for (int e = threadIdx.x; e < NVT; e += blockDim.x) {
    const int xv = e % NV, y = e / NV, x0 = xv * VW;
    int gi = i0 + x0, gj = j0 + y;
    gi += (gi < 0) ? n : ((gi >= n) ? -n : 0);
    gj += (gj < 0) ? n : ((gj >= n) ? -n : 0);
    const i64 b = (i64)gi + (i64)n * gj;
    const i64 cP = (b + n2 * k) / VW, cm = (b + n2 * kmn) / VW, cp = (b + n2 * kpn) / VW;
    V v[8];
    v[0] = vphi[cP];
    v[1] = vphi[cm];
    v[2] = vphi[cp];
#pragma unroll
    for (int f = 0; f < 5; ++f) v[3 + f] = vcoef[f * nv3 + cP];
#pragma unroll
    for (int f = 0; f < 8; ++f) *reinterpret_cast<V*>(sm + f * S + y * W + x0) = v[f];
  }
  __syncthreads();
  const T* P = sm;
  const T* Km = sm + S;
  const T* Kp = sm + 2 * S;
  const T* F1 = sm + 3 * S;
  const T* F2 = sm + 4 * S;
  const T* F3 = sm + 5 * S;
  const T* F4 = sm + 6 * S;
  const T* F5 = sm + 7 * S;
  decltype(abs_bits(T(0))) mb = 0;
#pragma unroll
  for (int q = 0; q < NCELL; ++q) {
    const int ty = ty0 + q * (256 / TX);
    const int c = (1 + ty) * W + HX + tx;
    const i64 gt = (i64)(blockIdx.x * TX + tx) + (i64)n * (blockIdx.y * TY + ty) + n2 * k;
    Stencil<T> st;
    st.c = P[c]; st.ip = P[c + 1]; st.im = P[c - 1]; st.jp = P[c + W]; st.jm = P[c - W];
    st.kp = Kp[c]; st.km = Km[c];
    st.ppk = P[c + 1 + W]; st.mpk = P[c - 1 + W]; st.pmk = P[c + 1 - W]; st.mmk = P[c - 1 - W];
    st.jpkp = Kp[c + W]; st.jmkp = Kp[c - W]; st.jpkm = Km[c + W]; st.jmkm = Km[c - W];
    st.ipkp = Kp[c + 1]; st.imkp = Kp[c - 1]; st.ipkm = Km[c + 1]; st.imkm = Km[c - 1];
    st.f1c = F1[c]; st.f1ip = F1[c + 1]; st.f1im = F1[c - 1];
    st.f4c = F4[c]; st.f4jp = F4[c + W]; st.f4jm = F4[c - W];
    st.f2jp = F2[c + W]; st.f2jm = F2[c - W]; st.f2ip = F2[c + 1]; st.f2im = F2[c - 1];
    st.f5jp = F5[c + W]; st.f5jm = F5[c - W];
    st.f3ip = F3[c + 1]; st.f3im = F3[c - 1];
    st.f6c = c6[q]; st.f6kp = c6p[q]; st.f6km = c6m[q];
    st.f5kp = c5p[q]; st.f5km = c5m[q];
    st.f3kp = c3p[q]; st.f3km = c3m[q];
    T tdiag, t1, t2;
    op_eval(st, tdiag, t1, t2);
    T v;
    if (MODE == 0) {
      v = cr[q] - (t1 + t2 + tdiag * st.c) * di2;
      if (out32) out32[gt] = (float)v;
    } else {
      v = (t1 + t2 + tdiag * st.c) * di2;
    }
    if (out) out[gt] = v;
    const auto vb = abs_bits(v);
    mb = vb > mb ? vb : mb;
  }
  if (maxbits) block_max_commit(from_bits(mb), maxbits);
}

// The FP32 residual (MODE 0: r = rhs - L[phi]) or operator (MODE 1: q = L[p])
// of k_stencil_plane, with each CTA marching through KC consecutive planes of
// one 32 x 16 tile column instead of taking one plane.  Shared memory keeps
// a ring of four planes of phi and of coefficients 3, 5, 6 (the planes k-1,
// k, k+1 a plane reads, and k+2 in flight) and two of coefficients 1, 2, 4 and
// of rhs, so every plane of a field is fetched once per column instead of
// three times (phi) or twice (3, 5, 6), and the next plane's tiles are copied
// (cp.async) while the current one is computed.  Tiles of phi and of
// coefficients 1-5 carry a halo of 4 cells in x (aligned 16-byte copies) and
// 1 in y; coefficient 6 and rhs are read at the cell only.  The arithmetic is
// k_stencil_plane's, operand for operand.  Needs n >= 32 and KC | n.
constexpr int kMarchKC = 8;
struct MarchGeom {
  static constexpr int TX = 32, TY = 16, HX = 4, W = TX + 2 * HX, HT = TY + 2, S = W * HT, SI = TX * TY;
  // slots: phi 4, f3 4, f5 4, f1 2, f2 2, f4 2 halo tiles; f6 4, rhs 2 interior tiles
  static constexpr int PHI = 0, F3 = 4 * S, F5 = 8 * S, F1 = 12 * S, F2 = 14 * S, F4 = 16 * S, F6 = 18 * S,
                       RHS = 18 * S + 4 * SI, WORDS = 18 * S + 6 * SI;
};
template <int MODE>
__global__ void __launch_bounds__(256) k_stencil_march(const float* __restrict__ phi, const float* __restrict__ rhs,
                                                       const float* __restrict__ coef, int n, float di2,
                                                       float* __restrict__ out, unsigned long long* maxbits) {
  typedef MarchGeom G;
  constexpr int TX = G::TX, TY = G::TY, HX = G::HX, W = G::W, S = G::S, SI = G::SI, KC = kMarchKC;
  extern __shared__ __align__(16) float smf[];
  const i64 n2 = (i64)n * n, n3 = n2 * n;
  const int i0 = blockIdx.x * TX - HX, j0 = blockIdx.y * TY - 1, k0 = blockIdx.z * KC;
  const int e = threadIdx.x;
  // this thread's 16-byte group of a halo tile (e < 180) and of an interior tile (e < 128)
  const int hxv = e % (W / 4), hy = e / (W / 4);
  int gi = i0 + 4 * hxv, gj = j0 + hy;
  gi += (gi < 0) ? n : ((gi >= n) ? -n : 0);
  gj += (gj < 0) ? n : ((gj >= n) ? -n : 0);
  const i64 hoff = (i64)gi + (i64)n * gj;
  const int hdst = hy * W + 4 * hxv;
  const bool hl = e < (W / 4) * G::HT;
  const int ixv = e % (TX / 4), iy = (e / (TX / 4)) & (TY - 1);
  const i64 ioff = (i64)(blockIdx.x * TX + 4 * ixv) + (i64)n * (blockIdx.y * TY + iy);
  const int idst = iy * TX + 4 * ixv;
  const bool il = e < SI / 4;  // e < 128: coefficient 6; 128 <= e < 256: rhs
  const float* f1 = coef;
  const float* f2 = coef + n3;
  const float* f3 = coef + 2 * n3;
  const float* f4 = coef + 3 * n3;
  const float* f5 = coef + 4 * n3;
  const float* f6 = coef + 5 * n3;
  auto ring4 = [&](int kk) { return (kk - k0 + 1) & 3; };
  auto ring2 = [&](int kk) { return (kk - k0) & 1; };
  auto plane = [&](int kk) { return kk < 0 ? kk + n : (kk >= n ? kk - n : kk); };
  // copies of plane kk of a field with a halo tile / the interior tile
  auto halo = [&](const float* f, int kk, int slot) {
    if (hl) cp_async16(smf + slot + hdst, f + hoff + n2 * plane(kk));
  };
  auto f6_rhs = [&](int k6, int kr) {
    if (il) cp_async16(smf + G::F6 + ring4(k6) * SI + idst, f6 + ioff + n2 * plane(k6));
    else if (MODE == 0) cp_async16(smf + G::RHS + ring2(kr) * SI + idst, rhs + ioff + n2 * plane(kr));
  };
  // the planes the first plane of the column reads
#pragma unroll
  for (int d = -1; d <= 1; ++d) {
    halo(phi, k0 + d, G::PHI + ring4(k0 + d) * S);
    halo(f3, k0 + d, G::F3 + ring4(k0 + d) * S);
    halo(f5, k0 + d, G::F5 + ring4(k0 + d) * S);
    if (il) cp_async16(smf + G::F6 + ring4(k0 + d) * SI + idst, f6 + ioff + n2 * plane(k0 + d));
  }
  halo(f1, k0, G::F1);
  halo(f2, k0, G::F2);
  halo(f4, k0, G::F4);
  if (!il && MODE == 0) cp_async16(smf + G::RHS + idst, rhs + ioff + n2 * k0);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  const int tx = threadIdx.x % TX, ty0 = threadIdx.x / TX;
  constexpr int NCELL = TY / (256 / TX);
  decltype(abs_bits(0.0f)) mb = 0;
  for (int k = k0; k < k0 + KC; ++k) {
    if (k + 1 < k0 + KC) {
      // what plane k+1 adds: phi and coefficients 3, 5, 6 of k+2; 1, 2, 4 and rhs of k+1
      halo(phi, k + 2, G::PHI + ring4(k + 2) * S);
      halo(f3, k + 2, G::F3 + ring4(k + 2) * S);
      halo(f5, k + 2, G::F5 + ring4(k + 2) * S);
      halo(f1, k + 1, G::F1 + ring2(k + 1) * S);
      halo(f2, k + 1, G::F2 + ring2(k + 1) * S);
      halo(f4, k + 1, G::F4 + ring2(k + 1) * S);
      f6_rhs(k + 2, k + 1);
      cp_async_commit();
    }
    const float* P = smf + G::PHI + ring4(k) * S;
    const float* Km = smf + G::PHI + ring4(k - 1) * S;
    const float* Kp = smf + G::PHI + ring4(k + 1) * S;
    const float* F1 = smf + G::F1 + ring2(k) * S;
    const float* F2 = smf + G::F2 + ring2(k) * S;
    const float* F4 = smf + G::F4 + ring2(k) * S;
    const float* F3 = smf + G::F3 + ring4(k) * S;
    const float* F3m = smf + G::F3 + ring4(k - 1) * S;
    const float* F3p = smf + G::F3 + ring4(k + 1) * S;
    const float* F5 = smf + G::F5 + ring4(k) * S;
    const float* F5m = smf + G::F5 + ring4(k - 1) * S;
    const float* F5p = smf + G::F5 + ring4(k + 1) * S;
    const float* F6 = smf + G::F6 + ring4(k) * SI;
    const float* F6m = smf + G::F6 + ring4(k - 1) * SI;
    const float* F6p = smf + G::F6 + ring4(k + 1) * SI;
    const float* R = smf + G::RHS + ring2(k) * SI;
#pragma unroll
    for (int q = 0; q < NCELL; ++q) {
      const int ty = ty0 + q * (256 / TX);
      const int c = (1 + ty) * W + HX + tx, ci = ty * TX + tx;
      const i64 gt = (i64)(blockIdx.x * TX + tx) + (i64)n * (blockIdx.y * TY + ty) + n2 * k;
      Stencil<float> st;
      st.c = P[c]; st.ip = P[c + 1]; st.im = P[c - 1]; st.jp = P[c + W]; st.jm = P[c - W];
      st.kp = Kp[c]; st.km = Km[c];
      st.ppk = P[c + 1 + W]; st.mpk = P[c - 1 + W]; st.pmk = P[c + 1 - W]; st.mmk = P[c - 1 - W];
      st.jpkp = Kp[c + W]; st.jmkp = Kp[c - W]; st.jpkm = Km[c + W]; st.jmkm = Km[c - W];
      st.ipkp = Kp[c + 1]; st.imkp = Kp[c - 1]; st.ipkm = Km[c + 1]; st.imkm = Km[c - 1];
      st.f1c = F1[c]; st.f1ip = F1[c + 1]; st.f1im = F1[c - 1];
      st.f4c = F4[c]; st.f4jp = F4[c + W]; st.f4jm = F4[c - W];
      st.f2jp = F2[c + W]; st.f2jm = F2[c - W]; st.f2ip = F2[c + 1]; st.f2im = F2[c - 1];
      st.f5jp = F5[c + W]; st.f5jm = F5[c - W];
      st.f3ip = F3[c + 1]; st.f3im = F3[c - 1];
      st.f6c = F6[ci]; st.f6kp = F6p[ci]; st.f6km = F6m[ci];
      st.f5kp = F5p[c]; st.f5km = F5m[c];
      st.f3kp = F3p[c]; st.f3km = F3m[c];
      float tdiag, t1, t2;
      op_eval(st, tdiag, t1, t2);
      float v;
      if (MODE == 0)
        v = R[ci] - (t1 + t2 + tdiag * st.c) * di2;
      else
        v = (t1 + t2 + tdiag * st.c) * di2;
      if (out) out[gt] = v;
      const auto vb = abs_bits(v);
      mb = vb > mb ? vb : mb;
    }
    cp_async_wait_all();
    __syncthreads();
  }
  if (maxbits) block_max_commit(from_bits(mb), maxbits);
}

// Full-weighting restriction of the residual with the reference's
// accumulation order (calcresid gauss1.f90:819-859 as scheduled by r1lax):
// coarse plane `special` adds its own-plane part first, all others their
// lower-plane part first.
template <class T>
__global__ void k_restrict_resid(const T* __restrict__ r, int n, int special, T* __restrict__ coarse) {
  int nh = n >> 1;
  i64 tot = (i64)nh * nh * nh;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tot) return;
  int I, J, K;
  cell_of(t, nh, I, J, K);
  int ib = 2 * I, ibp = (ib + 1) % n, ibm = (ib + n - 1) % n;
  int jb = 2 * J, jbp = (jb + 1) % n, jbm = (jb + n - 1) % n;
  int kb = 2 * K, kbp = kb + 1, kl = (kb + n - 1) % n;
#define R_(x, y, z) r[IDX(x, y, z, n)]
  T lower_a = R_(ib, jb, kl) * T(0.0625);
  T lower_b = (R_(ibp, jb, kl) + R_(ibm, jb, kl) + R_(ib, jbp, kl) + R_(ib, jbm, kl)) * T(0.03125);
  T lower_c = (R_(ibp, jbp, kl) + R_(ibp, jbm, kl) + R_(ibm, jbp, kl) + R_(ibm, jbm, kl)) * T(0.015625);
  T main_a = R_(ib, jb, kb) * T(0.125);
  T main_b = (R_(ibp, jb, kb) + R_(ibm, jb, kb) + R_(ib, jbp, kb) + R_(ib, jbm, kb) + R_(ib, jb, kbp)) * T(0.0625);
  T main_c = (R_(ibp, jbp, kb) + R_(ibp, jbm, kb) + R_(ibm, jbp, kb) + R_(ibm, jbm, kb) + R_(ibp, jb, kbp) +
              R_(ibm, jb, kbp) + R_(ib, jbp, kbp) + R_(ib, jbm, kbp)) * T(0.03125);
  T main_d = (R_(ibp, jbp, kbp) + R_(ibp, jbm, kbp) + R_(ibm, jbp, kbp) + R_(ibm, jbm, kbp)) * T(0.015625);
#undef R_
  T acc = T(0);
  if (K == special) {
    acc = acc + main_a + main_b + main_c + main_d;
    acc = acc + lower_a + lower_b + lower_c;
  } else {
    acc = acc + lower_a + lower_b + lower_c;
    acc = acc + main_a + main_b + main_c + main_d;
  }
  coarse[t] = acc;
}

// 27-point full weighting [1/4,1/2,1/4]^3 (restrict mgutil.f90:74-118 at the
// odd fine points, nsmooth limiter.f90:677-781 at every point).
template <class T>
__device__ __forceinline__ T smooth27(const T* __restrict__ a, int n, int i, int j, int k) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
#define A_(x, y, z) a[IDX(x, y, z, n)]
  return A_(i, j, k) * T(0.125) +
         (A_(ip, j, k) + A_(im, j, k) + A_(i, jp, k) + A_(i, jm, k) + A_(i, j, kp) + A_(i, j, km)) * T(0.0625) +
         (A_(ip, jp, k) + A_(ip, jm, k) + A_(im, jp, k) + A_(im, jm, k) + A_(ip, j, kp) + A_(ip, j, km) +
          A_(im, j, kp) + A_(im, j, km) + A_(i, jp, kp) + A_(i, jp, km) + A_(i, jm, kp) + A_(i, jm, km)) * T(0.03125) +
         (A_(ip, jp, kp) + A_(ip, jp, km) + A_(ip, jm, kp) + A_(ip, jm, km) + A_(im, jp, kp) + A_(im, jp, km) +
          A_(im, jm, kp) + A_(im, jm, km)) * T(0.015625);
#undef A_
}

template <class T>
__global__ void k_restrict27(const T* __restrict__ fine, int n, T* __restrict__ coarse) {
  int nh = n >> 1;
  i64 tot = (i64)nh * nh * nh;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tot) return;
  int I, J, K;
  cell_of(t, nh, I, J, K);
  coarse[t] = smooth27(fine, n, 2 * I, 2 * J, 2 * K);
}

template <class T>
__global__ void k_smooth27(const T* __restrict__ in, int n, T* __restrict__ out) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  out[t] = smooth27(in, n, i, j, k);
}

// inject (mgutil.f90:38-71): u += trilinear prolongation of uh.  Fine cell
// (i, j, k) adds (H(ibl,jbl,kbl) + H(ibl,jbl,kbh) + H(ibl,jbh,kbl) +
// H(ibl,jbh,kbh) + H(ibh,jbh,kbl) + H(ibh,jbh,kbh) + H(ibh,jbl,kbl) +
// H(ibh,jbl,kbh)) * 1/8 with ibl = i/2, ibh = (i+1)/2 wrapped (the same for j,
// k), summed in that order.  One thread per coarse cell (ci, cj, ck) writes
// the 2 x 2 x 2 fine cells (2ci + x, 2cj + y, 2ck + z), whose ibl = ci and
// ibh = ci + x, so their terms are the coarse values h[a][b][d] =
// uh(ci + a x, cj + b y, ck + d z): the block reads the 8 coarse values once
// instead of 8 per fine cell, and each fine pair x = 0, 1 is one vector load
// and store.
template <class T>
__global__ void k_prolong_add_blk(T* __restrict__ u, const T* __restrict__ uh, int n) {
  typedef typename std::conditional<sizeof(T) == 4, float2, double2>::type V2;
  const int nh = n >> 1;
  const i64 nh3 = (i64)nh * nh * nh;
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nh3) return;
  int ci, cj, ck;
  cell_of(t, nh, ci, cj, ck);
  const int ch[2] = {ci, ci + 1 < nh ? ci + 1 : 0}, cjh[2] = {cj, cj + 1 < nh ? cj + 1 : 0},
            ckh[2] = {ck, ck + 1 < nh ? ck + 1 : 0};
  T h[2][2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int d = 0; d < 2; ++d) h[a][b][d] = uh[IDX(ch[a], cjh[b], ckh[d], nh)];
#pragma unroll
  for (int z = 0; z < 2; ++z)
#pragma unroll
    for (int y = 0; y < 2; ++y) {
      V2* p = reinterpret_cast<V2*>(u + IDX(2 * ci, 2 * cj + y, 2 * ck + z, n));
      V2 v = *p;
      v.x = v.x + (h[0][0][0] + h[0][0][z] + h[0][y][0] + h[0][y][z] + h[0][y][0] + h[0][y][z] + h[0][0][0] +
                   h[0][0][z]) * T(0.125);
      v.y = v.y + (h[0][0][0] + h[0][0][z] + h[0][y][0] + h[0][y][z] + h[1][y][0] + h[1][y][z] + h[1][0][0] +
                   h[1][0][z]) * T(0.125);
      *p = v;
    }
}

// Exact sum of a[0..count) into acc (lo, hi); flag |= 1 on a term out of range.
template <class T>
__global__ void k_fxsum(const T* __restrict__ a, i64 count, unsigned long long* acc, int* flag) {
  __int128 s = 0;
  bool bad = false;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (i64)gridDim.x * blockDim.x) {
    double x = (double)a[t];
    if (!(fabs(x) < 4294967296.0)) bad = true;
    else s += fx_of(x);
  }
  if (bad) atomicOr(flag, 1);
  fx_block_commit(s, acc);
}

// det of I + Hess(def)/dx^2 without the tangle fallback (rgzerosum gauss1.f90:1390-1402)
template <class T>
__global__ void k_det(const T* __restrict__ def, int n, T di2, T* __restrict__ det) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  int i, j, k;
  cell_of(t, n, i, j, k);
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  T c = def[t];
  T phixx = (def[IDX(ip, j, k, n)] - T(2) * c + def[IDX(im, j, k, n)]) * di2;
  T phiyy = (def[IDX(i, jp, k, n)] - T(2) * c + def[IDX(i, jm, k, n)]) * di2;
  T phizz = (def[IDX(i, j, kp, n)] - T(2) * c + def[IDX(i, j, km, n)]) * di2;
  T phixy = (def[IDX(ip, jp, k, n)] - def[IDX(im, jp, k, n)] - def[IDX(ip, jm, k, n)] + def[IDX(im, jm, k, n)]) * di2 * T(0.25);
  T phiyz = (def[IDX(i, jp, kp, n)] - def[IDX(i, jp, km, n)] - def[IDX(i, jm, kp, n)] + def[IDX(i, jm, km, n)]) * di2 * T(0.25);
  T phixz = (def[IDX(ip, j, kp, n)] - def[IDX(im, j, kp, n)] - def[IDX(ip, j, km, n)] + def[IDX(im, j, km, n)]) * di2 * T(0.25);
  T a11 = T(1) + phixx, a12 = phixy, a13 = phixz, a22 = T(1) + phiyy, a23 = phiyz, a33 = T(1) + phizz;
  det[t] = (a11 * a22 * a33 + T(2) * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33);
}

// scalars: sc[0] = zerosum mean, sc[1] = rgzerosum dfact, sc[2] = usum
__global__ void k_fx_mean(const unsigned long long* acc, double count, double* out);
__global__ void k_fx_ratio(const unsigned long long* num, const unsigned long long* den, double* out);

template <class T>
__global__ void k_sub_mean(T* __restrict__ a, i64 count, const double* __restrict__ mean) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  a[t] = (T)((double)a[t] - *mean);
}

// rhs = rhs - dfact * det, dfact rounded to T (rgzerosum)
template <class T>
__global__ void k_sub_dfact(T* __restrict__ a, const T* __restrict__ det, i64 count, const double* __restrict__ ratio) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  T dfact = (T)(*ratio);
  a[t] = a[t] - dfact * det[t];
}

template <class T>
__global__ void k_fill(T* __restrict__ a, i64 count, T v) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) a[t] = v;
}

// a = v where the guard flag is set, else untouched (device-side divergence guard)
template <class T>
__global__ void k_zero_if(T* __restrict__ a, i64 count, const int* __restrict__ flag) {
  if (*flag == 0) return;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) a[t] = T(0);
}
template <class T>
__global__ void k_sub_mean_unless(T* __restrict__ a, i64 count, const double* __restrict__ mean,
                                  const int* __restrict__ flag) {
  if (*flag != 0) return;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  a[t] = (T)((double)a[t] - *mean);
}

}  // namespace mmh
