// MMH reconstruction hot path -- CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// This file restates, loop for loop, the moving-mesh reconstruction hot path of
// pandaPQY/Moving-Mesh-reconstruction (Fortran 90 + OpenMP, directory mmh/).  It is
// the checker for the CUDA library: only the tests, the smoke check and the
// CPU-baseline leg of bench.py may load it.  The product never links it.
//
// PARITY UNPINNED: the reference ships no golden vectors, no recorded outputs and
// no working self-test (TESTMG, mmh/multigrid.f90:123-174, and TESTRELAX,
// mmh/gauss1.f90:1505-1608, are stale and do not compile), and no Fortran compiler
// exists in the build image, so the reference cannot be run.  This restatement is
// pinned instead by analytic known-answer tests (tests/test_oracle_kat.py) and by
// an internal equivalence check between the reference's literal plane schedule
// and the 8-colour order the GPU uses.
//
// Conventions
//  * Arrays are the Fortran arrays laid out column-major: a(i,j,k) (1-based) is
//    a[(i-1) + n*((j-1) + n*(k-1))].  u(nf,n,n,n) is component-fastest.
//  * Every floating-point expression keeps the reference's operand order
//    (Fortran left-to-right evaluation, parentheses as written, x**2 as x*x);
//    the file must be compiled with -ffp-contract=off so that no FMA is formed.
//  * T = double is the "FP64 mode" (promoted precision of the FP32 Fortran);
//    T = float mirrors the shipped FP32 arithmetic and serves as CPU baseline.
//  * Sums the reference accumulates in real(8) (zerosum, usum, rgzerosum) are
//    taken in 128-bit fixed point (2^-64 resolution): exact, so the result does
//    not depend on thread count or order.  The GPU library sums the same way.
//  * The reference's z-plane ring buffers (gauss1.f90:222-242, relaxing.f90:58-67,
//    limiter.f90:50) only save memory; every value they hold is recomputed here
//    on the full grid with the same formula, so the per-cell results are equal.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef int64_t i64;
typedef __int128 i128;
typedef unsigned __int128 u128;

inline int wp(int i, int n) { return i + 1 == n ? 0 : i + 1; }
inline int wm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
inline i64 ID(int i, int j, int k, int n) { return (i64)i + (i64)n * ((i64)j + (i64)n * (i64)k); }

// ---------------------------------------------------------------------------
// Exact fixed-point summation (stand-in for the real(8) accumulators).
// A term x (|x| < 2^32) maps to trunc(x * 2^64) as a signed 128-bit integer.
// ---------------------------------------------------------------------------
// trunc(x * 2^sh) as a 128-bit integer, from the bits of x (finite x,
// |x * 2^sh| < 2^126).
inline i128 fx_bits(double x, int sh) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  int ex = (int)((b >> 52) & 0x7FF);
  uint64_t m = b & 0xFFFFFFFFFFFFFull;
  if (ex == 0) {
    if (m == 0) return 0;
    ex = 1;
  } else {
    m |= (1ull << 52);
  }
  int s = ex - 1075 + sh;
  u128 v;
  if (s >= 0) v = (u128)m << s;
  else if (s > -64) v = (u128)(m >> (-s));
  else v = 0;
  return (b >> 63) ? -(i128)v : (i128)v;
}
inline i128 fx_of(double x) { return fx_bits(x, 64); }
inline double fx_to(i128 s) {
  bool neg = s < 0;
  u128 a = neg ? (u128)(-s) : (u128)s;
  uint64_t hi = (uint64_t)(a >> 64), lo = (uint64_t)a;
  double r = (double)hi + (double)lo * 5.42101086242752217e-20;  // hi + lo*2^-64
  return neg ? -r : r;
}
struct FxAcc {
  i128 s = 0;
  bool bad = false;
  inline void add(double x) {
    if (!(std::fabs(x) < 4294967296.0)) { bad = true; return; }
    s += fx_of(x);
  }
};

template <class T>
double fx_sum(const T* a, i64 n, bool* bad) {
  i128 tot = 0;
  bool b = false;
#pragma omp parallel
  {
    FxAcc acc;
#pragma omp for nowait
    for (i64 i = 0; i < n; ++i) acc.add((double)a[i]);
#pragma omp critical
    {
      tot += acc.s;
      b = b || acc.bad;
    }
  }
  if (bad) *bad = *bad || b;
  return fx_to(tot);
}

template <class T> inline T fsign1(T a) { return a >= T(0) ? T(1) : T(-1); }  // ifort sign(1.,a)

// ---------------------------------------------------------------------------
// Curvilinear metric rho_bar * cof(A)/det, non-lsquare branch of cbajraw
// (mmh/gauss1.f90:1107-1210).  coef layout: 6 planes of n^3 (SoA).
// ---------------------------------------------------------------------------
template <class T>
void metric_cell(const T* def, const T* rho, int n, T di2, int i, int j, int k, T* o) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  T c = def[ID(i, j, k, n)];
  T phixx = (def[ID(ip, j, k, n)] - T(2) * c + def[ID(im, j, k, n)]) * di2;
  T phiyy = (def[ID(i, jp, k, n)] - T(2) * c + def[ID(i, jm, k, n)]) * di2;
  T phizz = (def[ID(i, j, kp, n)] - T(2) * c + def[ID(i, j, km, n)]) * di2;
  T phixy = (def[ID(ip, jp, k, n)] - def[ID(im, jp, k, n)] - def[ID(ip, jm, k, n)] + def[ID(im, jm, k, n)]) * di2 / T(4);
  T phiyz = (def[ID(i, jp, kp, n)] - def[ID(i, jp, km, n)] - def[ID(i, jm, kp, n)] + def[ID(i, jm, km, n)]) * di2 / T(4);
  T phixz = (def[ID(ip, j, kp, n)] - def[ID(im, j, kp, n)] - def[ID(ip, j, km, n)] + def[ID(im, j, km, n)]) * di2 / T(4);
  T a11 = T(1) + phixx, a12 = phixy, a13 = phixz, a22 = T(1) + phiyy, a23 = phiyz, a33 = T(1) + phizz;
  T det = a11 * a22 * a33 + T(2) * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33;
  T b11 = (a22 * a33 - a23 * a23);
  T b12 = (a13 * a23 - a12 * a33);
  T b13 = (a12 * a23 - a13 * a22);
  T b22 = (a11 * a33 - a13 * a13);
  T b23 = (a12 * a13 - a11 * a23);
  T b33 = (a11 * a22 - a12 * a12);
  if (det <= T(1.e-5)) {  // tangled cell: identity metric (gauss1.f90:1162-1171)
    b11 = T(1); b12 = T(0); b13 = T(0); b22 = T(1); b23 = T(0); b33 = T(1); det = T(1);
  }
  const int is[3] = {im, i, ip}, js[3] = {jm, j, jp}, ks[3] = {km, k, kp};
  T urg = T(0);
  bool first = true;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int d = 0; d < 3; ++d) {
        T v = rho[ID(is[a], js[b], ks[d], n)];
        urg = first ? v : urg + v;
        first = false;
      }
  urg = urg / T(27);
  o[0] = urg * b11 / det;
  o[1] = urg * b12 / det;
  o[2] = urg * b13 / det;
  o[3] = urg * b22 / det;
  o[4] = urg * b23 / det;
  o[5] = urg * b33 / det;
}

template <class T>
void metric(const T* def, const T* rho, int n, T dx, T* coef) {
  i64 n3 = (i64)n * n * n;
  T di2 = T(1) / (dx * dx);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        T o[6];
        metric_cell(def, rho, n, di2, i, j, k, o);
        i64 id = ID(i, j, k, n);
        for (int c = 0; c < 6; ++c) coef[c * n3 + id] = o[c];
      }
}

// ---------------------------------------------------------------------------
// 19-point curvilinear operator pieces shared by relaxplane (gauss1.f90:950-980)
// and calcresid (gauss1.f90:683-709).
// ---------------------------------------------------------------------------
template <class T>
struct Op {
  const T* f[6];
  int n;
  i64 n3;
  Op(const T* coef, int n_) : n(n_), n3((i64)n_ * n_ * n_) {
    for (int c = 0; c < 6; ++c) f[c] = coef + c * n3;
  }
  // returns tdiag, t1, t2 for cell (i,j,k)
  inline void terms(const T* phi, int i, int j, int k, T& tdiag, T& t1, T& t2) const {
    int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
    const T *f1 = f[0], *f2 = f[1], *f3 = f[2], *f4 = f[3], *f5 = f[4], *f6 = f[5];
    i64 c = ID(i, j, k, n);
    T b11p = (f1[ID(ip, j, k, n)] + f1[c]) / T(2);
    T b11m = (f1[ID(im, j, k, n)] + f1[c]) / T(2);
    T b22p = (f4[ID(i, jp, k, n)] + f4[c]) / T(2);
    T b22m = (f4[ID(i, jm, k, n)] + f4[c]) / T(2);
    T b33p = (f6[ID(i, j, kp, n)] + f6[c]) / T(2);
    T b33m = (f6[ID(i, j, km, n)] + f6[c]) / T(2);
    tdiag = -(b11p + b11m + b22p + b22m + b33p + b33m);
    t1 = (b11p * phi[ID(ip, j, k, n)] + b11m * phi[ID(im, j, k, n)] + b22p * phi[ID(i, jp, k, n)] +
          b22m * phi[ID(i, jm, k, n)] + b33p * phi[ID(i, j, kp, n)] + b33m * phi[ID(i, j, km, n)]);
    t2 = ((phi[ID(ip, jp, k, n)] - phi[ID(im, jp, k, n)]) * f2[ID(i, jp, k, n)]
          - (phi[ID(ip, jm, k, n)] - phi[ID(im, jm, k, n)]) * f2[ID(i, jm, k, n)]
          + (phi[ID(ip, jp, k, n)] - phi[ID(ip, jm, k, n)]) * f2[ID(ip, j, k, n)]
          - (phi[ID(im, jp, k, n)] - phi[ID(im, jm, k, n)]) * f2[ID(im, j, k, n)]
          + (phi[ID(i, jp, kp, n)] - phi[ID(i, jm, kp, n)]) * f5[ID(i, j, kp, n)]
          - (phi[ID(i, jp, km, n)] - phi[ID(i, jm, km, n)]) * f5[ID(i, j, km, n)]
          + (phi[ID(i, jp, kp, n)] - phi[ID(i, jp, km, n)]) * f5[ID(i, jp, k, n)]
          - (phi[ID(i, jm, kp, n)] - phi[ID(i, jm, km, n)]) * f5[ID(i, jm, k, n)]
          + (phi[ID(ip, j, kp, n)] - phi[ID(im, j, kp, n)]) * f3[ID(i, j, kp, n)]
          - (phi[ID(ip, j, km, n)] - phi[ID(im, j, km, n)]) * f3[ID(i, j, km, n)]
          + (phi[ID(ip, j, kp, n)] - phi[ID(ip, j, km, n)]) * f3[ID(ip, j, k, n)]
          - (phi[ID(im, j, kp, n)] - phi[ID(im, j, km, n)]) * f3[ID(im, j, k, n)]) / T(4);
  }
};

// relaxplane: 4-colour in-plane Gauss-Seidel of plane k (gauss1.f90:866-991).
template <class T>
void relaxplane(T* phi, const Op<T>& op, const T* rhs, T dx, int k) {
  int n = op.n;
  T dx2 = dx * dx;
  for (int io = 0; io <= 1; ++io)
    for (int jo = 0; jo <= 1; ++jo) {
#pragma omp parallel for
      for (int j = jo; j < n; j += 2)
        for (int i = io; i < n; i += 2) {
          T tdiag, t1, t2;
          op.terms(phi, i, j, k, tdiag, t1, t2);
          i64 c = ID(i, j, k, n);
          phi[c] = (rhs[c] * dx2 - t1 - t2) / tdiag;
        }
    }
}

// Residual r = rhs - L[phi] of one cell (gauss1.f90:709).
template <class T>
inline T resid_cell(const T* phi, const Op<T>& op, const T* rhs, T di2, int i, int j, int k) {
  T tdiag, t1, t2;
  op.terms(phi, i, j, k, tdiag, t1, t2);
  i64 c = ID(i, j, k, op.n);
  return rhs[c] - (t1 + t2 + tdiag * phi[c]) * di2;
}

// calcresid (gauss1.f90:509-861): residual on fine planes ki-1, ki (1-based,
// ki even), max-norm into rinf, full-weighting accumulation into the coarse
// planes ki/2 and ki/2+1 of resid (literal accumulation order).
template <class T>
void calcresid(T* resid, const Op<T>& op, const T* phi, const T* rhs, T dx, int ki1, int iopt, T& rinf,
               std::vector<T>& rt) {
  int n = op.n;
  bool lresid = (iopt % 2) == 1;
  bool lnorminf = ((iopt / 2) % 2) == 1;
  T di2 = T(1) / (dx * dx);
  i64 n2 = (i64)n * n;
  rt.resize(2 * n2);
  T rmax = T(0);
  for (int ko = 1; ko <= 2; ++ko) {
    int k0 = ki1 - 2 + ko - 1;  // 0-based plane
    T loc = T(0);
#pragma omp parallel for reduction(max : loc)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        T tr = resid_cell(phi, op, rhs, di2, i, j, k0);
        loc = std::max(loc, std::fabs(tr));
        if (lresid) rt[(ko - 1) * n2 + (i64)i + (i64)n * j] = tr;
      }
    rmax = std::max(rmax, loc);
  }
  if (lnorminf) rinf = std::max(rinf, rmax);
  if (!lresid) return;
  int nh = n / 2;
  int k0 = ki1 / 2 - 1;
  int kp0 = (k0 + 1) % nh;
  auto RT = [&](int i, int j, int kb) { return rt[(kb)*n2 + (i64)i + (i64)n * j]; };
#pragma omp parallel for
  for (int J = 0; J < nh; ++J)
    for (int I = 0; I < nh; ++I) {
      int ib = 2 * I, ibp = (ib + 1) % n, ibm = (ib + n - 1) % n;
      int jb = 2 * J, jbp = (jb + 1) % n, jbm = (jb + n - 1) % n;
      const int kb = 0, kbp = 1;
      i64 c0 = ID(I, J, k0, nh), c1 = ID(I, J, kp0, nh);
      resid[c0] = resid[c0] + RT(ib, jb, kb) / T(8) +
                  (RT(ibp, jb, kb) + RT(ibm, jb, kb) + RT(ib, jbp, kb) + RT(ib, jbm, kb) + RT(ib, jb, kbp)) / T(16) +
                  (RT(ibp, jbp, kb) + RT(ibp, jbm, kb) + RT(ibm, jbp, kb) + RT(ibm, jbm, kb) + RT(ibp, jb, kbp) +
                   RT(ibm, jb, kbp) + RT(ib, jbp, kbp) + RT(ib, jbm, kbp)) / T(32) +
                  (RT(ibp, jbp, kbp) + RT(ibp, jbm, kbp) + RT(ibm, jbp, kbp) + RT(ibm, jbm, kbp)) / T(64);
      resid[c1] = resid[c1] + RT(ib, jb, kbp) / T(16) +
                  (RT(ibp, jb, kbp) + RT(ibm, jb, kbp) + RT(ib, jbp, kbp) + RT(ib, jbm, kbp)) / T(32) +
                  (RT(ibp, jbp, kbp) + RT(ibp, jbm, kbp) + RT(ibm, jbp, kbp) + RT(ibm, jbm, kbp)) / T(64);
    }
}

// r1lax (gauss1.f90:208-499): the reference's plane schedule, emitted in its
// literal order (initial pyramid, intermediate planes, wrap-around finale).
// Planes here are 1-based as in the Fortran.  The metric ring (calcbajxy) is
// replaced by the full precomputed metric held in op.
template <class T>
void r1lax(T* arr, T* resid, const T* rhs, const Op<T>& op, T& rinf, T dx, int nrelax, int iopt) {
  int na3 = op.n;
  int iresidopt = iopt % 8;
  rinf = T(0);
  if (iresidopt == 4) rinf = T(1.0e20);
  std::vector<T> rt;
  if (iresidopt == 1 || iresidopt == 3) {
    i64 nh3 = (i64)(na3 / 2) * (na3 / 2) * (na3 / 2);
    std::fill(resid, resid + nh3, T(0));
  }
  auto RP = [&](int k1) { relaxplane(arr, op, rhs, dx, k1 - 1); };
  auto CR = [&](int ki1) { calcresid(resid, op, arr, rhs, dx, ki1, iresidopt, rinf, rt); };
  auto md = [&](int a) { return ((a % na3) + na3) % na3; };
  if (nrelax == 0) {
    for (int k = 2; k <= na3; k += 2) CR(k);
    return;
  }
  RP(1);
  for (int ko = 2; ko <= (nrelax - 1) * 4 + 1; ko += 2) {
    int iclvls = (ko - 2) / 4;
    for (int ki = 0; ki <= iclvls; ++ki) {
      RP(md(ko - 2 * ki + 4 * na3) + 1);
      RP(md(ko - 2 * ki + 4 * na3 - 1) + 1);
    }
    if (ko % 4 == 0) RP(md(ko / 2) + 1);
  }
  for (int ko = (nrelax - 1) * 4 + 2; ko <= na3 - 1; ko += 2) {
    for (int ki = 1; ki <= nrelax * 2; ki += 2) {
      RP(ko - ki + 2);
      RP(ko - ki + 1);
    }
    if (iresidopt > 0 && ko > (nrelax - 1) * 4 + 2) CR(md(4 * na3 + ko - nrelax * 2 + 1) + 1);
  }
  int k = na3;
  RP(k);
  for (int ki = 2; ki <= nrelax; ++ki) {
    k = md(4 * na3 - 2 * ki + 2) + 1;
    RP(k);
    k = md(4 * na3 - 2 * ki + 1) + 1;
    RP(k);
  }
  if (iresidopt > 0) CR(md(4 * na3 - nrelax * 2 + 1) + 1);
  k = 3;
  for (int ko = 1; ko <= nrelax - 1; ++ko) {
    k = md(4 * na3 + 2 * ko + 2) + 1;
    for (int it = 1; it <= 2; ++it)
      for (int ki = 1; ki <= nrelax - ko; ++ki) {
        if (it != 2 || ki != 1) {
          k = md(4 * na3 + 2 * ko - 2 * ki + 2 * it - 2) + 1;
          RP(k);
        }
        k = md(4 * na3 + 2 * ko - 2 * ki + 2 * it - 3) + 1;
        RP(k);
      }
    if (iresidopt > 0) {
      CR(md(4 * na3 + 4 * ko - 2 * nrelax - 1) + 1);
      CR(md(4 * na3 + 4 * ko - 2 * nrelax + 1) + 1);
    }
  }
  if (iresidopt > 0) {
    k = md(k + 1) + 1;
    if (nrelax == 1) k = 2;
    CR(k);
  }
}

// The same sweeps in 8-colour order: nrelax x (all odd planes, all even planes),
// then the residual of every plane and the full-weighting restriction with the
// accumulation order the literal schedule produces (coarse plane nrelax+1 takes
// its own-plane part first, every other coarse plane its lower-plane part
// first).  This is the order the GPU library executes.
template <class T>
void r1lax_colour8(T* arr, T* resid, const T* rhs, const Op<T>& op, T& rinf, T dx, int nrelax, int iopt) {
  int n = op.n;
  int iresidopt = iopt % 8;
  rinf = T(0);
  for (int s = 0; s < nrelax; ++s)
    for (int par = 0; par <= 1; ++par) {
      T dx2 = dx * dx;
      for (int io = 0; io <= 1; ++io)
        for (int jo = 0; jo <= 1; ++jo) {
#pragma omp parallel for collapse(2)
          for (int k = par; k < n; k += 2)
            for (int j = jo; j < n; j += 2)
              for (int i = io; i < n; i += 2) {
                T tdiag, t1, t2;
                op.terms(arr, i, j, k, tdiag, t1, t2);
                i64 c = ID(i, j, k, n);
                arr[c] = (rhs[c] * dx2 - t1 - t2) / tdiag;
              }
        }
    }
  if (iresidopt == 0) return;
  bool lresid = (iresidopt % 2) == 1;
  T di2 = T(1) / (dx * dx);
  i64 n3 = (i64)n * n * n;
  std::vector<T> r(lresid ? n3 : 0);
  T rmax = T(0);
#pragma omp parallel for collapse(2) reduction(max : rmax)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        T tr = resid_cell(arr, op, rhs, di2, i, j, k);
        rmax = std::max(rmax, std::fabs(tr));
        if (lresid) r[ID(i, j, k, n)] = tr;
      }
  if ((iresidopt / 2) % 2 == 1) rinf = rmax;
  if (!lresid) return;
  int nh = n / 2;
  int special = nrelax;  // 0-based coarse plane whose own part comes first
  auto R = [&](int i, int j, int k) { return r[ID(i, j, k, n)]; };
#pragma omp parallel for collapse(2)
  for (int K = 0; K < nh; ++K)
    for (int J = 0; J < nh; ++J)
      for (int I = 0; I < nh; ++I) {
        int ib = 2 * I, ibp = (ib + 1) % n, ibm = (ib + n - 1) % n;
        int jb = 2 * J, jbp = (jb + 1) % n, jbm = (jb + n - 1) % n;
        int kb = 2 * K, kbp = kb + 1, kl = (kb + n - 1) % n;
        T acc = T(0);
        auto add_lower = [&](T a) {
          a = a + R(ib, jb, kl) / T(16) + (R(ibp, jb, kl) + R(ibm, jb, kl) + R(ib, jbp, kl) + R(ib, jbm, kl)) / T(32) +
              (R(ibp, jbp, kl) + R(ibp, jbm, kl) + R(ibm, jbp, kl) + R(ibm, jbm, kl)) / T(64);
          return a;
        };
        auto add_main = [&](T a) {
          a = a + R(ib, jb, kb) / T(8) +
              (R(ibp, jb, kb) + R(ibm, jb, kb) + R(ib, jbp, kb) + R(ib, jbm, kb) + R(ib, jb, kbp)) / T(16) +
              (R(ibp, jbp, kb) + R(ibp, jbm, kb) + R(ibm, jbp, kb) + R(ibm, jbm, kb) + R(ibp, jb, kbp) +
               R(ibm, jb, kbp) + R(ib, jbp, kbp) + R(ib, jbm, kbp)) / T(32) +
              (R(ibp, jbp, kbp) + R(ibp, jbm, kbp) + R(ibm, jbp, kbp) + R(ibm, jbm, kbp)) / T(64);
          return a;
        };
        if (K == special) acc = add_lower(add_main(acc));
        else acc = add_main(add_lower(acc));
        resid[ID(I, J, K, nh)] = acc;
      }
}

// relax (gauss1.f90:64-160): split nrelax into r1lax chunks of nrmax sweeps.
template <class T>
void relax(T* arr, T* resid, const T* rhs, const Op<T>& op, T& rinf, T dx, int nrelax, int iopt, bool colour8) {
  int na3 = op.n;
  int nrmax = std::min(4, std::max(1, na3 / 4));
  int nrmleft = nrelax % nrmax;
  auto R1 = [&](int nr, int io) {
    if (colour8) r1lax_colour8(arr, resid, rhs, op, rinf, dx, nr, io);
    else r1lax(arr, resid, rhs, op, rinf, dx, nr, io);
  };
  if (nrelax > nrmax) {
    int iiopt = iopt - iopt % 8;
    int itmax = nrelax / nrmax;
    for (int i = 1; i <= itmax; ++i) {
      if (i == itmax && nrmleft == 0) iiopt = iopt;
      R1(nrmax, iiopt);
    }
    if (nrmleft > 0) R1(nrmleft, iopt);
  } else {
    R1(nrelax, iopt);
  }
}

// restrict / restrictu (mgutil.f90:74-167): 27-point full weighting at the odd
// fine points; nsmooth (limiter.f90:677-781) is the same formula at every point.
template <class T>
inline T smooth27(const T* a, int n, int i, int j, int k) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  auto A = [&](int x, int y, int z) { return a[ID(x, y, z, n)]; };
  return A(i, j, k) / T(8) + (A(ip, j, k) + A(im, j, k) + A(i, jp, k) + A(i, jm, k) + A(i, j, kp) + A(i, j, km)) / T(16) +
         (A(ip, jp, k) + A(ip, jm, k) + A(im, jp, k) + A(im, jm, k) + A(ip, j, kp) + A(ip, j, km) + A(im, j, kp) +
          A(im, j, km) + A(i, jp, kp) + A(i, jp, km) + A(i, jm, kp) + A(i, jm, km)) / T(32) +
         (A(ip, jp, kp) + A(ip, jp, km) + A(ip, jm, kp) + A(ip, jm, km) + A(im, jp, kp) + A(im, jp, km) +
          A(im, jm, kp) + A(im, jm, km)) / T(64);
}

template <class T>
void restrict27(const T* fine, int n, T* coarse) {
  int nh = n / 2;
#pragma omp parallel for collapse(2)
  for (int k = 0; k < nh; ++k)
    for (int j = 0; j < nh; ++j)
      for (int i = 0; i < nh; ++i) coarse[ID(i, j, k, nh)] = smooth27(fine, n, 2 * i, 2 * j, 2 * k);
}

template <class T>
void nsmooth(T* a, int n) {
  i64 n3 = (i64)n * n * n;
  std::vector<T> v(n3);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) v[ID(i, j, k, n)] = smooth27(a, n, i, j, k);
  std::memcpy(a, v.data(), sizeof(T) * n3);
}

// inject (mgutil.f90:38-71): trilinear prolongation added to u.
template <class T>
void prolong_add(T* u, const T* uh, int n) {
  int nh = n / 2;
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        int ibl = i / 2, ibh = (i + 1) / 2, jbl = j / 2, jbh = (j + 1) / 2, kbl = k / 2, kbh = (k + 1) / 2;
        if (ibh >= nh) ibh = 0;
        if (jbh >= nh) jbh = 0;
        if (kbh >= nh) kbh = 0;
        auto H = [&](int x, int y, int z) { return uh[ID(x, y, z, nh)]; };
        i64 c = ID(i, j, k, n);
        u[c] = u[c] + (H(ibl, jbl, kbl) + H(ibl, jbl, kbh) + H(ibl, jbh, kbl) + H(ibl, jbh, kbh) + H(ibh, jbh, kbl) +
                       H(ibh, jbh, kbh) + H(ibh, jbl, kbl) + H(ibh, jbl, kbh)) / T(8);
      }
}

// zerosum (gauss1.f90:1420-1466): subtract the mean (real(8) mean).
template <class T>
void zerosum(T* a, int n, bool* bad) {
  i64 n3 = (i64)n * n * n;
  double s = fx_sum(a, n3, bad);
  s = s / (double)n3;
#pragma omp parallel for
  for (i64 i = 0; i < n3; ++i) a[i] = (T)((double)a[i] - s);
}

// det of I + Hess(def)/dx^2 without the tangle fallback (gauss1.f90:1390-1402).
template <class T>
inline T det_cell(const T* def, int n, T di2, int i, int j, int k) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  T c = def[ID(i, j, k, n)];
  T phixx = (def[ID(ip, j, k, n)] - T(2) * c + def[ID(im, j, k, n)]) * di2;
  T phiyy = (def[ID(i, jp, k, n)] - T(2) * c + def[ID(i, jm, k, n)]) * di2;
  T phizz = (def[ID(i, j, kp, n)] - T(2) * c + def[ID(i, j, km, n)]) * di2;
  T phixy = (def[ID(ip, jp, k, n)] - def[ID(im, jp, k, n)] - def[ID(ip, jm, k, n)] + def[ID(im, jm, k, n)]) * di2 / T(4);
  T phiyz = (def[ID(i, jp, kp, n)] - def[ID(i, jp, km, n)] - def[ID(i, jm, kp, n)] + def[ID(i, jm, km, n)]) * di2 / T(4);
  T phixz = (def[ID(ip, j, kp, n)] - def[ID(im, j, kp, n)] - def[ID(ip, j, km, n)] + def[ID(im, j, km, n)]) * di2 / T(4);
  T a11 = T(1) + phixx, a12 = phixy, a13 = phixz, a22 = T(1) + phiyy, a23 = phiyz, a33 = T(1) + phizz;
  return (a11 * a22 * a33 + T(2) * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33);
}

// rgzerosum (gauss1.f90:1219-1417): rhs -= (sum rhs / sum det) * det.
template <class T>
void rgzerosum(T* arr, const T* def, int n, T dx, bool* bad) {
  i64 n3 = (i64)n * n * n;
  T di2 = T(1) / (dx * dx);
  std::vector<T> det(n3);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) det[ID(i, j, k, n)] = det_cell(def, n, di2, i, j, k);
  double dsum = fx_sum(det.data(), n3, bad);
  double asum = fx_sum(arr, n3, bad);
  T dfact = (T)(asum / dsum);
#pragma omp parallel for
  for (i64 i = 0; i < n3; ++i) arr[i] = arr[i] - dfact * det[i];
}

// ---------------------------------------------------------------------------
// Multigrid (multigrid.f90:16-121, mgtemplate.f90:6-84).
// ---------------------------------------------------------------------------
struct MgCfg {
  int ng;          // NG: the top-level size (nrelax = 4*NG/n)
  int sched;       // 0 = reference schedule, 1 = PCG to tolerance, 2 = repeated V-cycles to tolerance
  int nu1, nu2;    // sweeps per level in the tolerance schedule
  double tol;      // relative max-norm residual target (tolerance schedule)
  int maxcyc;      // V-cycle cap (tolerance schedule)
  bool colour8;    // execute sweeps in 8-colour order instead of the literal schedule
  bool guards = true;  // divergence guards of the coarse levels (mgtemplate.f90:46-55)
};

struct MgStats {
  double r1 = 0, relaxerr = 0, rhsnorm = 0, resid_rel = 0;
  int vcycles = 0, guards = 0;
  bool bad = false;
};

template <class T>
void mg_level(T* u, T* rhs, const T* def, const T* rho, int n, T dx, const MgCfg& cfg, MgStats& st, bool top) {
  i64 n3 = (i64)n * n * n;
  std::vector<T> coef(6 * n3);
  metric(def, rho, n, dx, coef.data());
  Op<T> op(coef.data(), n);
  T r1 = 0, relaxerr = 0;
  if (n == 4) {
    // mg4 (multigrid.f90:94-121): 32 + 32 sweeps, guard with 1.001 margin.
    std::vector<T> dummy(8);
    relax(u, dummy.data(), rhs, op, r1, dx, 32, 2 * 8 + 2, cfg.colour8);
    relax(u, dummy.data(), rhs, op, relaxerr, dx, 32, 2 * 8 + 2, cfg.colour8);
    if (cfg.guards && n != cfg.ng && relaxerr > r1 * T(1.001) && r1 > T(1.E-5)) {
      std::fill(u, u + n3, T(0));
      st.guards++;
    } else {
      zerosum(u, n, &st.bad);
    }
    if (top) { st.r1 = r1; st.relaxerr = relaxerr; }
    return;
  }
  int nh = n / 2;
  i64 nh3 = (i64)nh * nh * nh;
  int nrelax = cfg.sched == 0 ? 4 * cfg.ng / n : cfg.nu1;
  int nrelax2 = cfg.sched == 0 ? 4 * cfg.ng / n : cfg.nu2;
  std::vector<T> rhshalf(nh3), defhalf(nh3), rhohalf(nh3), uhalf(nh3, T(0));
  relax(u, rhshalf.data(), rhs, op, r1, dx, nrelax, 2 * 8 + 3, cfg.colour8);
  restrict27(def, n, defhalf.data());
  restrict27(rho, n, rhohalf.data());
  mg_level(uhalf.data(), rhshalf.data(), defhalf.data(), rhohalf.data(), nh, dx * T(2), cfg, st, false);
  prolong_add(u, uhalf.data(), n);
  relax(u, rhshalf.data(), rhs, op, relaxerr, dx, nrelax2, 2 * 8 + 2, cfg.colour8);
  if (cfg.guards && n != cfg.ng && relaxerr > r1) {
    std::fill(u, u + n3, T(0));
    st.guards++;
  } else {
    zerosum(u, n, &st.bad);
  }
  if (top) { st.r1 = r1; st.relaxerr = relaxerr; }
}

// ---------------------------------------------------------------------------
// Exact, order-free dot product for the Krylov solver: each product a_i*b_i
// (rounded to double) is scaled by 2^(96-E) with 2^E > max|a| * max|b|,
// truncated to a 128-bit integer and summed exactly; the GPU does the same.
// ---------------------------------------------------------------------------
inline int dot_exp(double ma, double mb) { return std::ilogb(ma) + std::ilogb(mb) + 2; }
inline double fx_unscale(i128 s, int E) {
  bool neg = s < 0;
  u128 a = neg ? (u128)(-s) : (u128)s;
  double r = std::ldexp((double)(uint64_t)(a >> 64), E - 32) + std::ldexp((double)(uint64_t)a, E - 96);
  return neg ? -r : r;
}
template <class T>
double dot_exact(const T* a, const T* b, i64 n, double ma, double mb) {
  if (!(ma > 0) || !(mb > 0)) return 0.0;
  int E = dot_exp(ma, mb);
  i128 tot = 0;
#pragma omp parallel
  {
    i128 loc = 0;
#pragma omp for nowait
    for (i64 i = 0; i < n; ++i) loc += fx_bits((double)a[i] * (double)b[i], 96 - E);
#pragma omp critical
    tot += loc;
  }
  return fx_unscale(tot, E);
}
template <class T>
double absmax(const T* a, i64 n) {
  double m = 0.0;
#pragma omp parallel for reduction(max : m)
  for (i64 i = 0; i < n; ++i) m = std::max(m, (double)std::fabs(a[i]));
  return m;
}

// Flexible preconditioned conjugate gradients on L x = b, preconditioned by
// one V-cycle (mg_level from a zero guess).  L is symmetric and, for a regular
// mesh, negative definite on zero-mean fields; the Polak-Ribiere form of beta
// keeps the iteration stable when the preconditioner is not exactly linear
// (divergence guard, FP32 inner cycles on the GPU).
template <class T>
void pcg(T* x, const T* b, const T* def, const T* rho, int n, T dx, const MgCfg& cfg, MgStats& st, double rn) {
  i64 n3 = (i64)n * n * n;
  std::vector<T> coef(6 * n3), r(n3), z(n3), p(n3), q(n3);
  metric(def, rho, n, dx, coef.data());
  Op<T> op(coef.data(), n);
  T di2 = T(1) / (dx * dx);
  auto apply = [&](const T* v, T* out) {
#pragma omp parallel for collapse(2)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          T tdiag, t1, t2;
          op.terms(v, i, j, k, tdiag, t1, t2);
          i64 c = ID(i, j, k, n);
          out[c] = (t1 + t2 + tdiag * v[c]) * di2;
        }
  };
  auto precond = [&]() {
    std::fill(z.begin(), z.end(), T(0));
    MgStats sv;
    mg_level(z.data(), r.data(), def, rho, n, dx, cfg, sv, true);
    st.guards += sv.guards;
    st.bad = st.bad || sv.bad;
  };
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) r[ID(i, j, k, n)] = resid_cell(x, op, b, di2, i, j, k);
  double rmax = absmax(r.data(), n3);
  st.r1 = rmax;
  if (!(rmax / rn > cfg.tol)) {
    st.relaxerr = rmax;
    st.resid_rel = rmax / rn;
    return;
  }
  precond();
  double zmax = absmax(z.data(), n3);
  p = z;
  double pmax = zmax;
  double rz = dot_exact(r.data(), z.data(), n3, rmax, zmax);
  for (int it = 1; it <= cfg.maxcyc; ++it) {
    apply(p.data(), q.data());
    double qmax = absmax(q.data(), n3);
    double pq = dot_exact(p.data(), q.data(), n3, pmax, qmax);
    double alpha = rz / pq;
    T ta = (T)alpha;
#pragma omp parallel for
    for (i64 c = 0; c < n3; ++c) {
      x[c] = x[c] + ta * p[c];
      r[c] = r[c] - ta * q[c];
    }
    rmax = absmax(r.data(), n3);
    st.vcycles = it;
    if (!(rmax / rn > cfg.tol)) break;
    precond();
    zmax = absmax(z.data(), n3);
    double zq = dot_exact(z.data(), q.data(), n3, zmax, qmax);
    double rznew = dot_exact(r.data(), z.data(), n3, rmax, zmax);
    double beta = -(alpha * zq) / rz;
    rz = rznew;
    T tb = (T)beta;
#pragma omp parallel for
    for (i64 c = 0; c < n3; ++c) p[c] = z[c] + tb * p[c];
    pmax = absmax(p.data(), n3);
  }
  zerosum(x, n, &st.bad);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) r[ID(i, j, k, n)] = resid_cell(x, op, b, di2, i, j, k);
  rmax = absmax(r.data(), n3);
  st.relaxerr = rmax;
  st.resid_rel = rmax / rn;
}

// multigrid(u,rhs,defpot,ubig,dx,...) with iopt=2 (potential-flow solver).
// rho is ubig(1,:,:,:).  rhs is modified in place (rgzerosum), as in the reference.
template <class T>
void multigrid(T* u, T* rhs, const T* def, const T* rho, int n, T dx, const MgCfg& cfg, MgStats& st) {
  i64 n3 = (i64)n * n * n;
  rgzerosum(rhs, def, n, dx, &st.bad);
  T asum = (T)fx_sum(u, n3, &st.bad);
  if (asum > T(1.e-2)) zerosum(u, n, &st.bad);
  T rn = 0;
  for (i64 i = 0; i < n3; ++i) rn = std::max(rn, (T)std::fabs(rhs[i]));
  st.rhsnorm = rn;
  if (cfg.sched == 0) {
    mg_level(u, rhs, def, rho, n, dx, cfg, st, true);
    st.vcycles = 1;
    st.resid_rel = rn > 0 ? st.relaxerr / rn : 0;
    return;
  }
  st.vcycles = 0;
  if (rn == T(0)) return;
  if (cfg.sched == 1) {
    pcg(u, rhs, def, rho, n, dx, cfg, st, (double)rn);
    return;
  }
  // Repeated V-cycles until the post-smoothing max-norm residual on the
  // finest grid is below tol * max|rhs|.
  for (int c = 0; c < cfg.maxcyc; ++c) {
    mg_level(u, rhs, def, rho, n, dx, cfg, st, true);
    st.vcycles++;
    st.resid_rel = st.relaxerr / rn;
    if (st.resid_rel <= cfg.tol) break;
  }
}

// ---------------------------------------------------------------------------
// Eigenvalue-based compression measure (limiter.f90:346-359 and 459-472).
// ---------------------------------------------------------------------------
template <class T> struct Cst;
template <> struct Cst<double> { static double pi() { return 3.14159265358979323846264338328; } };
template <> struct Cst<float> { static float pi() { return 3.14159265358979323846264338328f; } };

template <class T>
inline T compression_of(T c11, T c12, T c13, T c22, T c23, T c33) {
  const T pi = Cst<T>::pi();
  T trace = c11 + c22 + c33;
  T d11 = c11 - trace / T(3);
  T d22 = c22 - trace / T(3);
  T a = -(d11 * d11 + c12 * c12 + c13 * c13 + d11 * d22 + d22 * d22 + c23 * c23);
  T b = -d11 * (c12 * c12) + d11 * d11 * d22 - c12 * c12 * d22 + c13 * c13 * d22 + d11 * (d22 * d22) -
        T(2) * c12 * c13 * c23 + d11 * (c23 * c23);
  if (std::fabs(a) < T(1.e-20)) a = T(1.e-20);
  T am = T(2) * std::sqrt(std::fabs(-a) / T(3));
  T theta = std::acos(std::max(T(-1), std::min(T(1), T(3) * b / a / am))) / T(3);
  T r1 = am * std::cos(theta);
  T r2 = am * std::cos(theta + T(2) * pi / T(3));
  T r3 = am * std::cos(theta + T(4) * pi / T(3));
  return T(1) / std::min(std::min(r1 + trace / T(3), r2 + trace / T(3)), r3 + trace / T(3));
}

// Limiter metric: cof(A)/det and det of A = I + Hess(def), unit spacing
// (limiter.f90:193-218, 268-286; relaxing.f90:876-901).
template <class T>
struct LimM {
  T b11, b12, b13, b22, b23, b33, det;
  T phixx, phiyy, phizz, phixy, phiyz, phixz;
};
template <class T>
inline LimM<T> lim_metric(const T* def, int n, int i, int j, int k) {
  int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
  LimM<T> m;
  T c = def[ID(i, j, k, n)];
  m.phixx = (def[ID(ip, j, k, n)] - T(2) * c + def[ID(im, j, k, n)]);
  m.phiyy = (def[ID(i, jp, k, n)] - T(2) * c + def[ID(i, jm, k, n)]);
  m.phizz = (def[ID(i, j, kp, n)] - T(2) * c + def[ID(i, j, km, n)]);
  m.phixy = (def[ID(ip, jp, k, n)] - def[ID(im, jp, k, n)] - def[ID(ip, jm, k, n)] + def[ID(im, jm, k, n)]) / T(4);
  m.phiyz = (def[ID(i, jp, kp, n)] - def[ID(i, jp, km, n)] - def[ID(i, jm, kp, n)] + def[ID(i, jm, km, n)]) / T(4);
  m.phixz = (def[ID(ip, j, kp, n)] - def[ID(im, j, kp, n)] - def[ID(ip, j, km, n)] + def[ID(im, j, km, n)]) / T(4);
  T a11 = T(1) + m.phixx, a12 = m.phixy, a13 = m.phixz, a22 = T(1) + m.phiyy, a23 = m.phiyz, a33 = T(1) + m.phizz;
  T det = a11 * a22 * a33 + T(2) * a12 * a13 * a23 - a13 * a13 * a22 - a11 * (a23 * a23) - a12 * a12 * a33;
  m.det = det;
  m.b11 = (a22 * a33 - a23 * a23) / det;
  m.b12 = (a13 * a23 - a12 * a33) / det;
  m.b13 = (a12 * a23 - a13 * a22) / det;
  m.b22 = (a11 * a33 - a13 * a13) / det;
  m.b23 = (a12 * a13 - a11 * a23) / det;
  m.b33 = (a11 * a22 - a12 * a12) / det;
  return m;
}

struct LimStats {
  long long nexpand = 0, ncompress = 0;
  double detmax = 0, detmin = 1, fluxmax = 0, fluxmin = 0, rho2 = 0, cmax = 0;
};

// Pass-1 flux limiter (limiter.f90:175-381).  u is u(nf,n,n,n).
// The flux of cell (i,j,km) is tested with the metric of plane k = km+1.
template <class T>
void limiter_pass1(T* tmp, const T* def, const T* u, int nf, int n, T dtold, T dtaumesh, T cmpmaxglobal,
                   LimStats& ls, uint8_t* maskx, uint8_t* maskc) {
  const T densinit = T(1);
  long long nexp = 0;
  T detmax = T(0), detmin = T(1), fluxmax = T(0), fluxmin = T(0);
  double rho2 = 0;
  auto U = [&](int c, int i, int j, int k) { return u[(i64)c + (i64)nf * ID(i, j, k, n)]; };
#pragma omp parallel for collapse(2) reduction(+ : nexp, rho2) reduction(max : detmax, fluxmax) \
    reduction(min : detmin, fluxmin)
  for (int km = 0; km < n; ++km)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        int k = wp(km, n), kmm = wm(km, n);
        int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n);
        LimM<T> m = lim_metric(def, n, i, j, k);
        T det = m.det;
        rho2 += (double)(U(0, i, j, km) * U(0, i, j, km) / det);
        T s1p = T(0), s2p = T(0), s3p = T(0), s1m = T(0), s2m = T(0), s3m = T(0);
        if (nf >= 4) {
          LimM<T> mxp = lim_metric(def, n, ip, j, km), myp = lim_metric(def, n, i, jp, km);
          LimM<T> mxm = lim_metric(def, n, im, j, km), mym = lim_metric(def, n, i, jm, km);
          LimM<T> mzm = lim_metric(def, n, i, j, kmm);
          s1p = (mxp.b11 * U(1, ip, j, km) + mxp.b12 * U(2, ip, j, km) + mxp.b13 * U(3, ip, j, km)) / U(0, ip, j, km);
          s2p = (myp.b12 * U(1, i, jp, km) + myp.b22 * U(2, i, jp, km) + myp.b23 * U(3, i, jp, km)) / U(0, i, jp, km);
          s3p = (m.b13 * U(1, i, j, k) + m.b23 * U(2, i, j, k) + m.b33 * U(3, i, j, k)) / U(0, i, j, k);
          s1m = (mxm.b11 * U(1, im, j, km) + mxm.b12 * U(2, im, j, km) + mxm.b13 * U(3, im, j, km)) / U(0, im, j, km);
          s2m = (mym.b12 * U(1, i, jm, km) + mym.b22 * U(2, i, jm, km) + mym.b23 * U(3, i, jm, km)) / U(0, i, jm, km);
          s3m = (mzm.b13 * U(1, i, j, kmm) + mzm.b23 * U(2, i, j, kmm) + mzm.b33 * U(3, i, j, kmm)) / U(0, i, j, kmm);
        }
        T eflux = (s1p + s2p + s3p - s1m - s2m - s3m) / T(2);
        i64 cm = ID(i, j, km, n);
        eflux = eflux + tmp[cm];
        uint8_t mx = 0, mc = 0;
        if (det > T(10) * densinit) {
          eflux = -T(2) * std::fabs(eflux);
          nexp++;
          mx = 1;
        }
        T c11 = T(1) + m.phixx, c12 = m.phixy, c13 = m.phixz, c22 = T(1) + m.phiyy, c23 = m.phiyz, c33 = T(1) + m.phizz;
        T compression = compression_of(c11, c12, c13, c22, c23, c33);
        T cmpmax = cmpmaxglobal * T(1);  // densinit**(-1./3.) with densinit = 1
        T tlim = T(3) * (T(1) / cmpmax - T(1) / compression) / dtold;
        if (tlim > T(0)) {
          eflux = std::max(T(0), eflux);
          mc = 1;
        }
        detmax = std::max(detmax, det);
        detmin = std::min(detmin, det);
        eflux = std::min(T(1) / dtaumesh, eflux);
        eflux = std::max(-T(1) / dtaumesh, eflux);
        tmp[cm] = eflux;
        fluxmax = std::max(fluxmax, eflux * dtold);
        fluxmin = std::min(fluxmin, eflux * dtold);
        if (maskx) maskx[cm] = mx;
        if (maskc) maskc[cm] = mc;
      }
  ls.nexpand = nexp;
  ls.detmax = detmax;
  ls.detmin = detmin;
  ls.fluxmax = fluxmax;
  ls.fluxmin = fluxmin;
  ls.rho2 = rho2;
}

// Compression test on I + dtold*Hess(defp) + Hess(def) (limiter.f90:425-533).
template <class T>
void limiter_mask(T* defplim, const T* def, const T* defp, int n, T dtold, T cmpmaxglobal, LimStats& ls,
                  uint8_t* mask) {
  long long nc = 0;
  T cmax = T(0);
#pragma omp parallel for collapse(2) reduction(+ : nc) reduction(max : cmax)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
        auto P = [&](int x, int y, int z) { return defp[ID(x, y, z, n)]; };
        auto D = [&](int x, int y, int z) { return def[ID(x, y, z, n)]; };
        T phixx = (P(ip, j, k) - T(2) * P(i, j, k) + P(im, j, k)) * dtold;
        T phiyy = (P(i, jp, k) - T(2) * P(i, j, k) + P(i, jm, k)) * dtold;
        T phizz = (P(i, j, kp) - T(2) * P(i, j, k) + P(i, j, km)) * dtold;
        T phixy = (P(ip, jp, k) - P(im, jp, k) - P(ip, jm, k) + P(im, jm, k)) / T(4) * dtold;
        T phiyz = (P(i, jp, kp) - P(i, jp, km) - P(i, jm, kp) + P(i, jm, km)) / T(4) * dtold;
        T phixz = (P(ip, j, kp) - P(im, j, kp) - P(ip, j, km) + P(im, j, km)) / T(4) * dtold;
        phixx = phixx + (D(ip, j, k) - T(2) * D(i, j, k) + D(im, j, k));
        phiyy = phiyy + (D(i, jp, k) - T(2) * D(i, j, k) + D(i, jm, k));
        phizz = phizz + (D(i, j, kp) - T(2) * D(i, j, k) + D(i, j, km));
        phixy = phixy + (D(ip, jp, k) - D(im, jp, k) - D(ip, jm, k) + D(im, jm, k)) / T(4);
        phiyz = phiyz + (D(i, jp, kp) - D(i, jp, km) - D(i, jm, kp) + D(i, jm, km)) / T(4);
        phixz = phixz + (D(ip, j, kp) - D(im, j, kp) - D(ip, j, km) + D(im, j, km)) / T(4);
        T compression = compression_of(T(1) + phixx, phixy, phixz, T(1) + phiyy, phiyz, T(1) + phizz);
        T cmpmax = cmpmaxglobal * T(1);
        T tlim = T(3) * (T(1) / cmpmax - T(1) / compression) / dtold;
        cmax = std::max(cmax, compression);
        i64 c = ID(i, j, k, n);
        defplim[c] = T(0);
        if (mask) mask[c] = 0;
        if (tlim > T(0)) {
          nc++;
          defplim[c] = tlim;
          if (mask) mask[c] = 1;
        }
      }
  ls.ncompress = nc;
  ls.cmax = cmax;
}

// ---------------------------------------------------------------------------
// Real 3-D FFT with the semantics of the reference's rlft3 (recipes12.f90:77-135):
// forward uses exp(+2 pi i k.x/N); output is (n+2) x n x n reals, kx = 0..n/2,
// Re/Im interleaved.  The inverse is unnormalised (returns N^3/2 times the
// data); for data that is not Hermitian on the kx = 0 and kx = n/2 planes it
// acts as the packed-real algorithm does: Z'(k,p) = (X(k,p) + X*(M-k,-p))/2 +
// i w(k) (X(k,p) - X*(M-k,-p))/2, w(k) = exp(-2 pi i k/N), followed by an
// unnormalised complex inverse transform of size (N/2) x N x N whose complex
// output holds the real samples pairwise.  The FFT itself is a project-written
// radix-2 transform (the Numerical Recipes source is not reused).
// ---------------------------------------------------------------------------
typedef std::complex<double> cd;

void fft1(cd* a, int n, i64 stride, int sign) {
  // iterative radix-2, in place, along a strided line
  std::vector<cd> tmp(n);
  for (int i = 0; i < n; ++i) tmp[i] = a[i * stride];
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(tmp[i], tmp[j]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    double ang = 2.0 * M_PI / len * sign;
    for (int i = 0; i < n; i += len)
      for (int q = 0; q < len / 2; ++q) {
        cd w(std::cos(ang * q), std::sin(ang * q));
        cd x = tmp[i + q], y = tmp[i + q + len / 2] * w;
        tmp[i + q] = x + y;
        tmp[i + q + len / 2] = x - y;
      }
  }
  for (int i = 0; i < n; ++i) a[i * stride] = tmp[i];
}

// complex 3-D FFT over (m, n, n), x fastest
void fft3c(cd* a, int m, int n, int sign) {
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) fft1(a + (i64)m * (j + (i64)n * k), m, 1, sign);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < m; ++i) fft1(a + i + (i64)m * n * k, n, m, sign);
#pragma omp parallel for collapse(2)
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) fft1(a + i + (i64)m * j, n, (i64)m * n, sign);
}

// forward: x (n^3 real) -> X ((n/2+1) x n x n complex)
void rlft3_fwd(const double* x, int n, cd* X) {
  int M = n / 2;
  std::vector<cd> z((i64)M * n * n);
  for (i64 q = 0; q < (i64)M * n * n; ++q) z[q] = cd(x[2 * q], x[2 * q + 1]);
  fft3c(z.data(), M, n, +1);
  int H = M + 1;
#pragma omp parallel for collapse(2)
  for (int kz = 0; kz < n; ++kz)
    for (int ky = 0; ky < n; ++ky)
      for (int kx = 0; kx <= M; ++kx) {
        int nky = (n - ky) % n, nkz = (n - kz) % n;
        cd Z = z[(kx % M) + (i64)M * (ky + (i64)n * kz)];
        cd Zc = std::conj(z[((M - kx) % M) + (i64)M * (nky + (i64)n * nkz)]);
        double th = 2.0 * M_PI * kx / n;
        cd w(std::cos(th), std::sin(th));
        cd h1 = 0.5 * (Z + Zc), h2 = cd(0, -0.5) * (Z - Zc);
        X[kx + (i64)H * (ky + (i64)n * kz)] = h1 + w * h2;
      }
}

// inverse: X ((n/2+1) x n x n complex) -> x (n^3 real), unnormalised (x N^3/2)
void rlft3_inv(const cd* X, int n, double* x) {
  int M = n / 2, H = M + 1;
  std::vector<cd> z((i64)M * n * n);
#pragma omp parallel for collapse(2)
  for (int kz = 0; kz < n; ++kz)
    for (int ky = 0; ky < n; ++ky)
      for (int kx = 0; kx < M; ++kx) {
        int nky = (n - ky) % n, nkz = (n - kz) % n;
        cd A = X[kx + (i64)H * (ky + (i64)n * kz)];
        cd B = std::conj(X[(M - kx) + (i64)H * (nky + (i64)n * nkz)]);
        double th = -2.0 * M_PI * kx / n;
        cd w(std::cos(th), std::sin(th));
        z[kx + (i64)M * (ky + (i64)n * kz)] = 0.5 * (A + B) + cd(0, 0.5) * w * (A - B);
      }
  fft3c(z.data(), M, n, -1);
  for (i64 q = 0; q < (i64)M * n * n; ++q) {
    x[2 * q] = z[q].real();
    x[2 * q + 1] = z[q].imag();
  }
}

// FFT Poisson correction of the compression limiter (limiter.f90:535-597).
template <class T>
void limiter_poisson(T* defp, const T* defplim, int n) {
  const double pi = 3.14159265358979323846264338328;
  i64 n3 = (i64)n * n * n;
  int H = n / 2 + 1;
  std::vector<double> x(n3);
  for (i64 q = 0; q < n3; ++q) x[q] = (double)defplim[q];
  std::vector<cd> X((i64)H * n * n);
  rlft3_fwd(x.data(), n, X.data());
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int ii = 0; ii < H; ++ii) {
        double xk = 2 * pi * ii / n;
        double yk = 2 * pi * (j + 1 - 1.) / n;
        double zk = 2 * pi * (k + 1 - 1.) / n;
        double akernel = 2 * std::cos(xk) + 2 * std::cos(yk) + 2 * std::cos(zk) - 6;
        if (std::fabs(akernel) < 1e-10) akernel = 1;
        cd& v = X[ii + (i64)H * (j + (i64)n * k)];
        v = cd(v.real() / akernel, v.imag() / akernel);
      }
  X[0] = cd(0.0, X[0].imag());
  rlft3_inv(X.data(), n, x.data());
  for (i64 q = 0; q < n3; ++q) {
    double v = x[q] * 2. / n / n / n;
    defp[q] = defp[q] + (T)v;
  }
}

// scalar2gradient (gradient.f90): out(:,:,:,a) = F^-1[i k_a F[def]] (= -d_a def).
template <class T>
void gradient(const T* in, T* out, int n) {
  const double pi = 3.14159265358979323846264338328;
  i64 n3 = (i64)n * n * n;
  int H = n / 2 + 1;
  std::vector<double> x(n3);
  for (i64 q = 0; q < n3; ++q) x[q] = (double)in[q];
  std::vector<cd> X0((i64)H * n * n), X((i64)H * n * n);
  rlft3_fwd(x.data(), n, X0.data());
  for (int ax = 0; ax < 3; ++ax) {
#pragma omp parallel for collapse(2)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < H; ++i) {
          double kk;
          if (ax == 0) kk = i;
          else if (ax == 1) kk = (j + 1 <= n / 2 + 1) ? j : j - n;
          else kk = (k + 1 <= n / 2 + 1) ? k : k - n;
          i64 q = i + (i64)H * (j + (i64)n * k);
          cd c = X0[q];
          // cmp * cmplx(0,kk) / n * 2 * pi
          double re = c.real() * 0.0 - c.imag() * kk;
          double im = c.real() * kk + c.imag() * 0.0;
          re = re / n * 2. * pi;
          im = im / n * 2. * pi;
          X[q] = cd(re, im);
        }
    rlft3_inv(X.data(), n, x.data());
    for (i64 q = 0; q < n3; ++q) out[(i64)ax * n3 + q] = (T)(x[q] * 2. / n / n / n);
  }
}

// defp2delta (reconstruct.f90): F^-1[|k|^2 F[def]] (= -Laplacian(def)).
template <class T>
void delta(const T* in, T* out, int n) {
  const double pi = 3.14159265358979323846264338328;
  i64 n3 = (i64)n * n * n;
  int H = n / 2 + 1;
  std::vector<double> x(n3);
  for (i64 q = 0; q < n3; ++q) x[q] = (double)in[q];
  std::vector<cd> X((i64)H * n * n);
  rlft3_fwd(x.data(), n, X.data());
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      double k3 = (k + 1 <= n / 2 + 1) ? k : k - n;
      k3 = k3 / n * 2. * pi;
      double k2 = (j + 1 <= n / 2 + 1) ? j : j - n;
      k2 = k2 / n * 2. * pi;
      for (int i = 0; i < H; ++i) {
        double k1 = i;
        k1 = k1 / n * 2. * pi;
        double f = k1 * k1 + k2 * k2 + k3 * k3;
        cd& v = X[i + (i64)H * (j + (i64)n * k)];
        v = cd(v.real() * f, v.imag() * f);
      }
    }
  rlft3_inv(X.data(), n, x.data());
  for (i64 q = 0; q < n3; ++q) out[q] = (T)(x[q] * 2. / n / n / n);
}

// ---------------------------------------------------------------------------
// relaxing (relaxing.f90:21-1139): relaxing-TVD RK2 update of u(5,n,n,n) in
// curvilinear coordinates.  Restated as full-grid stages: metric + freezing
// speed + flux of u, half step u1 = u - dt/2 R(u), flux of u1, full step
// u -= dt R(u1) with the freezing speed of u (the reference's plane pipeline
// computes the same per-cell values).
// ---------------------------------------------------------------------------
template <class T>
struct RelaxWork {
  std::vector<T> baj, c, vt, vtf, u1;
};

template <class T>
inline T minmod(T a, T b) {
  const T wslopelim = T(1.5), wbee = T(1);
  auto mm1 = [&](T x, T y) { return std::min(wslopelim * x, wbee * y + (T(1) - wbee) * x); };
  auto mm2 = [&](T x, T y) { return mm1(std::min(x, y), std::max(x, y)); };
  return (fsign1(a) + fsign1(b)) * mm2(std::fabs(a), std::fabs(b)) / T(2);
}

// relaxing-TVD half-cell flux (wphalfx/y/z): positions m, 0, p, pp
template <class T>
inline T wphalf(T um, T vm, T u0, T v0, T up, T vp, T upp, T vpp) {
  T a = (u0 + v0) / T(2);
  T b = (up - vp) / T(2);
  T da = (up + vp) / T(2) - a;
  T dam = a - (um + vm) / T(2);
  T ap = a + minmod(dam, da) / T(2);
  T db = (upp - vpp) / T(2) - b;
  T dbm = b - (u0 - v0) / T(2);
  T bp = b - minmod(db, dbm) / T(2);
  return ap - bp;
}

template <class T>
void relax_flux(const T* u, const T* defp, const T* baj, int n, int nf, T* vt) {
  // vt layout: [(dim*nf + l) * n3 + cell]
  i64 n3 = (i64)n * n * n;
  const T gamma = T(5.) / T(3.);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        i64 c = ID(i, j, k, n);
        int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
        T rg = baj[6 * n3 + c];
        T ul[5] = {T(0), T(0), T(0), T(0), T(0)};
        for (int l = 0; l < nf; ++l) ul[l] = u[(i64)l + (i64)nf * c];
        // fluxeuler (relaxing.f90:999-1063)
        T vt1[3][5];
        {
          T rho = ul[0] / rg, mx = ul[1] / rg, my = ul[2] / rg, mz = ul[3] / rg;
          T vx = mx / rho, vy = my / rho, vz = mz / rho;
          T engy = ul[4] / rg;
          T kinetic = rho * (vx * vx + vy * vy + vz * vz) / T(2);
          T pressure = (gamma - T(1)) * (engy - kinetic);
          pressure = std::max(T(0), pressure);
          T econv = engy + pressure;
          vt1[0][0] = mx; vt1[1][0] = my; vt1[2][0] = mz;
          vt1[0][1] = mx * vx + pressure; vt1[1][1] = mx * vy; vt1[2][1] = mx * vz;
          vt1[0][2] = my * vx; vt1[1][2] = my * vy + pressure; vt1[2][2] = my * vz;
          vt1[0][3] = mz * vx; vt1[1][3] = mz * vy; vt1[2][3] = mz * vz + pressure;
          vt1[0][4] = econv * vx; vt1[1][4] = econv * vy; vt1[2][4] = econv * vz;
        }
        T pdxg = (defp[ID(ip, j, k, n)] - defp[ID(im, j, k, n)]) / T(2) / rg;
        T pdyg = (defp[ID(i, jp, k, n)] - defp[ID(i, jm, k, n)]) / T(2) / rg;
        T pdzg = (defp[ID(i, j, kp, n)] - defp[ID(i, j, km, n)]) / T(2) / rg;
        T b11 = baj[0 * n3 + c] * rg, b12 = baj[1 * n3 + c] * rg, b13 = baj[2 * n3 + c] * rg;
        T b22 = baj[3 * n3 + c] * rg, b23 = baj[4 * n3 + c] * rg, b33 = baj[5 * n3 + c] * rg;
        for (int l = 0; l < nf; ++l) {
          T vtt1 = vt1[0][l] - ul[l] * pdxg;
          T vtt2 = vt1[1][l] - ul[l] * pdyg;
          T vtt3 = vt1[2][l] - ul[l] * pdzg;
          vt[(0 * nf + l) * n3 + c] = b11 * vtt1 + b12 * vtt2 + b13 * vtt3;
          vt[(1 * nf + l) * n3 + c] = b12 * vtt1 + b22 * vtt2 + b23 * vtt3;
          vt[(2 * nf + l) * n3 + c] = b13 * vtt1 + b23 * vtt2 + b33 * vtt3;
        }
      }
}

// dpv (relaxing.f90:269-496): res(l) of every cell.
template <class T>
void relax_dpv(const T* u, const T* vt, const T* cc, int n, int nf, T* res) {
  i64 n3 = (i64)n * n * n;
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        i64 c = ID(i, j, k, n);
        int kk[5], ii[5], jj[5];
        for (int l = 0; l < 5; ++l) {
          kk[l] = ((k + l - 2) % n + n) % n;
          ii[l] = ((i + l - 2) % n + n) % n;
          jj[l] = ((j + l - 2) % n + n) % n;
        }
        for (int l = 0; l < nf; ++l) {
          const T* vz = vt + (2 * nf + l) * n3;
          const T* vx = vt + (0 * nf + l) * n3;
          const T* vy = vt + (1 * nf + l) * n3;
          auto Uq = [&](int x, int y, int z) { return u[(i64)l + (i64)nf * ID(x, y, z, n)]; };
          // z sweep: vk(l) = vt(.,3)/c at planes k-2..k+2
          T uz[5], wz[5];
          for (int q = 0; q < 5; ++q) {
            i64 cq = ID(i, j, kk[q], n);
            uz[q] = Uq(i, j, kk[q]);
            wz[q] = vz[cq] / cc[cq];
          }
          T flz1 = wphalf(uz[0], wz[0], uz[1], wz[1], uz[2], wz[2], uz[3], wz[3]);
          T flz2 = wphalf(uz[1], wz[1], uz[2], wz[2], uz[3], wz[3], uz[4], wz[4]);
          T ck = cc[c], ckp = cc[ID(i, j, kk[3], n)], ckm = cc[ID(i, j, kk[1], n)];
          T r = (ckp + ck) / T(2) * flz2 - (ck + ckm) / T(2) * flz1;
          // x sweep
          T ux[5], wx[5];
          for (int q = 0; q < 5; ++q) {
            i64 cq = ID(ii[q], j, k, n);
            ux[q] = Uq(ii[q], j, k);
            wx[q] = vx[cq] / cc[cq];
          }
          T flx0 = wphalf(ux[1], wx[1], ux[2], wx[2], ux[3], wx[3], ux[4], wx[4]);  // flux at i+1/2
          T flxm = wphalf(ux[0], wx[0], ux[1], wx[1], ux[2], wx[2], ux[3], wx[3]);  // flux at i-1/2
          T cip = cc[ID(ii[3], j, k, n)], cim = cc[ID(ii[1], j, k, n)];
          T fp = (cip + ck) / T(2) * flx0;
          T fm = (ck + cim) / T(2) * flxm;
          r = r + fp - fm;
          // y sweep
          T uy[5], wy[5];
          for (int q = 0; q < 5; ++q) {
            i64 cq = ID(i, jj[q], k, n);
            uy[q] = Uq(i, jj[q], k);
            wy[q] = vy[cq] / cc[cq];
          }
          T fly0 = wphalf(uy[1], wy[1], uy[2], wy[2], uy[3], wy[3], uy[4], wy[4]);
          T flym = wphalf(uy[0], wy[0], uy[1], wy[1], uy[2], wy[2], uy[3], wy[3]);
          T cjp = cc[ID(i, jj[3], k, n)], cjm = cc[ID(i, jj[1], k, n)];
          r = r + (cjp + ck) / T(2) * fly0 - (ck + cjm) / T(2) * flym;
          res[(i64)l * n3 + c] = r;
        }
      }
}

template <class T>
void relaxing(T* u, const T* def, const T* defp, int n, int nf, T dt) {
  i64 n3 = (i64)n * n * n;
  const T gamma = T(5.) / T(3.);
  std::vector<T> baj(7 * n3), cc(n3), vt(3 * nf * n3), res(nf * n3), u1(nf * n3);
  // calcbaj (relaxing.f90:840-906) and cflkeuler (relaxing.f90:1067-1139)
#pragma omp parallel for collapse(2)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        i64 c = ID(i, j, k, n);
        LimM<T> m = lim_metric(def, n, i, j, k);
        baj[6 * n3 + c] = m.det;
        baj[0 * n3 + c] = m.b11; baj[1 * n3 + c] = m.b12; baj[2 * n3 + c] = m.b13;
        baj[3 * n3 + c] = m.b22; baj[4 * n3 + c] = m.b23; baj[5 * n3 + c] = m.b33;
        int ip = wp(i, n), im = wm(i, n), jp = wp(j, n), jm = wm(j, n), kp = wp(k, n), km = wm(k, n);
        T pdx = (defp[ID(ip, j, k, n)] - defp[ID(im, j, k, n)]) / T(2);
        T pdy = (defp[ID(i, jp, k, n)] - defp[ID(i, jm, k, n)]) / T(2);
        T pdz = (defp[ID(i, j, kp, n)] - defp[ID(i, j, km, n)]) / T(2);
        T b11 = m.b11, b12 = m.b12, b13 = m.b13, b22 = m.b22, b23 = m.b23, b33 = m.b33, det = m.det;
        T u0 = u[(i64)nf * c];
        T us[5] = {u0, T(0), T(0), T(0), T(0)};
        for (int l = 1; l < nf; ++l) us[l] = u[(i64)l + (i64)nf * c];
        T vx = us[1] / us[0], vy = us[2] / us[0], vz = us[3] / us[0];
        T rho = us[0] / det;
        T kin = rho * (vx * vx + vy * vy + vz * vz) / T(2);
        T ed = us[4] / det - kin;
        T pressure = (gamma - T(1)) * ed;
        T cs = std::sqrt(gamma * std::fabs(pressure / rho));
        T v1 = vx - pdx, v2 = vy - pdy, v3 = vz - pdz;
        T vv1 = b11 * v1 + b12 * v2 + b13 * v3;
        T vv2 = b12 * v1 + b22 * v2 + b23 * v3;
        T vv3 = b13 * v1 + b23 * v2 + b33 * v3;
        T blim1 = cs * std::sqrt(b11 * b11 + b12 * b12 + b13 * b13) + std::fabs(vv1);
        T blim2 = cs * std::sqrt(b12 * b12 + b22 * b22 + b23 * b23) + std::fabs(vv2);
        T blim3 = cs * std::sqrt(b13 * b13 + b23 * b23 + b33 * b33) + std::fabs(vv3);
        cc[c] = std::max(std::max(blim1, blim2), blim3);
      }
  relax_flux(u, defp, baj.data(), n, nf, vt.data());
  relax_dpv(u, vt.data(), cc.data(), n, nf, res.data());
  T dth = dt / T(2);
#pragma omp parallel for
  for (i64 c = 0; c < n3; ++c)
    for (int l = 0; l < nf; ++l) u1[(i64)l + (i64)nf * c] = u[(i64)l + (i64)nf * c] - res[(i64)l * n3 + c] * dth;
  relax_flux(u1.data(), defp, baj.data(), n, nf, vt.data());
  relax_dpv(u1.data(), vt.data(), cc.data(), n, nf, res.data());
#pragma omp parallel for
  for (i64 c = 0; c < n3; ++c)
    for (int l = 0; l < nf; ++l) u[(i64)l + (i64)nf * c] = u[(i64)l + (i64)nf * c] - res[(i64)l * n3 + c] * dt;
}

// ---------------------------------------------------------------------------
// calcdefp (limiter.f90:17-673).
// ---------------------------------------------------------------------------
template <class T>
void calcdefp(T* defp, const T* def, const T* u, int nf, int n, T dtold, T dtaumesh, const MgCfg& cfg, MgStats& ms,
              LimStats& ls, uint8_t* mask_exp, uint8_t* mask_c1, uint8_t* mask_c2) {
  i64 n3 = (i64)n * n * n;
  const T densinit = T(1);
  const T cmpmaxglobal = T(10);  // compressmax (main.f90:56)
  if (dtold < T(1.e-8)) dtold = T(1);
  std::vector<T> tmp(n3), rho(n3), defplim(n3);
  for (i64 c = 0; c < n3; ++c) rho[c] = u[(i64)nf * c];
#pragma omp parallel for
  for (i64 c = 0; c < n3; ++c) {
    T t1 = densinit - u[(i64)nf * c];
    T xhigh = T(2);
    if (std::fabs(t1) > xhigh) t1 = t1 >= T(0) ? xhigh : -xhigh;
    tmp[c] = t1 / T(30) / dtold;
  }
  for (int i = 0; i < 3; ++i) nsmooth(tmp.data(), n);
  limiter_pass1(tmp.data(), def, u, nf, n, dtold, dtaumesh, cmpmaxglobal, ls, mask_exp, mask_c1);
  nsmooth(tmp.data(), n);
  std::fill(defp, defp + n3, T(0));
  multigrid(defp, tmp.data(), def, rho.data(), n, T(1), cfg, ms);
  for (int i = 0; i < 2; ++i) nsmooth(defp, n);
  limiter_mask(defplim.data(), def, defp, n, dtold, cmpmaxglobal, ls, mask_c2);
  if (ls.ncompress > 0) limiter_poisson(defp, defplim.data(), n);
}

MgCfg make_cfg(int n, int sched, int nu1, int nu2, double tol, int maxcyc, int colour8) {
  MgCfg c;
  c.ng = n;
  c.sched = sched;
  c.nu1 = nu1;
  c.nu2 = nu2;
  c.tol = tol;
  c.maxcyc = maxcyc;
  c.colour8 = (colour8 & 1) != 0;
  c.guards = (colour8 & 2) == 0;  // bit 1 of the flags word switches the guards off
  return c;
}

}  // namespace

// ===========================================================================
// C entry points (ctypes).  Suffix _d = double, _f = float.
// ===========================================================================
extern "C" {

typedef struct orc_diag {
  double r1, relaxerr, rhsnorm, resid_rel;
  int vcycles, guards, bad, pad;
  long long nexpand, ncompress;
  double cmax, detmin, detmax, fluxmax, fluxmin, rho2;
} orc_diag;

int orc_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
  return omp_get_max_threads();
#else
  (void)t;
  return 1;
#endif
}

#define ORC_BOTH(X) X(double, d) X(float, f)

#define DEF_METRIC(T, S) \
  void orc_metric_##S(const T* def, const T* rho, int n, T dx, T* coef) { metric(def, rho, n, dx, coef); }
ORC_BOTH(DEF_METRIC)

#define DEF_RELAX(T, S)                                                                                      \
  void orc_relax_##S(T* arr, T* resid, const T* rhs, const T* coef, int n, T dx, int nrelax, int iopt,      \
                     int colour8, T* rinf) {                                                                 \
    Op<T> op(coef, n);                                                                                       \
    T r = 0;                                                                                                 \
    relax(arr, resid, rhs, op, r, dx, nrelax, iopt, colour8 != 0);                                          \
    *rinf = r;                                                                                               \
  }
ORC_BOTH(DEF_RELAX)

#define DEF_RESID(T, S)                                                                            \
  void orc_residual_##S(const T* phi, const T* rhs, const T* coef, int n, T dx, T* r) {           \
    Op<T> op(coef, n);                                                                             \
    T di2 = T(1) / (dx * dx);                                                                      \
    _Pragma("omp parallel for collapse(2)") for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) \
        for (int i = 0; i < n; ++i) r[ID(i, j, k, n)] = resid_cell(phi, op, rhs, di2, i, j, k);    \
  }
ORC_BOTH(DEF_RESID)

#define DEF_SMALL(T, S)                                                                              \
  void orc_restrict_##S(const T* fine, int n, T* coarse) { restrict27(fine, n, coarse); }           \
  void orc_prolong_add_##S(T* u, const T* uh, int n) { prolong_add(u, uh, n); }                     \
  void orc_nsmooth_##S(T* a, int n) { nsmooth(a, n); }                                               \
  int orc_zerosum_##S(T* a, int n) {                                                                 \
    bool bad = false;                                                                                \
    zerosum(a, n, &bad);                                                                             \
    return bad ? -1 : 0;                                                                             \
  }                                                                                                  \
  int orc_rgzerosum_##S(T* a, const T* def, int n, T dx) {                                           \
    bool bad = false;                                                                                \
    rgzerosum(a, def, n, dx, &bad);                                                                  \
    return bad ? -1 : 0;                                                                             \
  }                                                                                                  \
  double orc_fxsum_##S(const T* a, long long n) { return fx_sum(a, (i64)n, nullptr); }
ORC_BOTH(DEF_SMALL)

#define DEF_MG(T, S)                                                                                      \
  int orc_multigrid_##S(T* u, T* rhs, const T* def, const T* rho, int n, T dx, int sched, int nu1, int nu2, \
                        double tol, int maxcyc, int colour8, orc_diag* d) {                                 \
    MgCfg cfg = make_cfg(n, sched, nu1, nu2, tol, maxcyc, colour8);                                        \
    MgStats st;                                                                                              \
    multigrid(u, rhs, def, rho, n, dx, cfg, st);                                                            \
    if (d) {                                                                                                 \
      d->r1 = st.r1; d->relaxerr = st.relaxerr; d->rhsnorm = st.rhsnorm; d->resid_rel = st.resid_rel;       \
      d->vcycles = st.vcycles; d->guards = st.guards; d->bad = st.bad;                                      \
    }                                                                                                        \
    return st.bad ? -1 : 0;                                                                                  \
  }
ORC_BOTH(DEF_MG)

#define DEF_LIM(T, S)                                                                                       \
  void orc_limiter_pass1_##S(T* tmp, const T* def, const T* u, int nf, int n, T dtold, T dtaumesh,          \
                             uint8_t* maskx, uint8_t* maskc, orc_diag* d) {                                 \
    LimStats ls;                                                                                             \
    limiter_pass1(tmp, def, u, nf, n, dtold, dtaumesh, T(10), ls, maskx, maskc);                            \
    if (d) {                                                                                                 \
      d->nexpand = ls.nexpand; d->detmax = ls.detmax; d->detmin = ls.detmin;                                \
      d->fluxmax = ls.fluxmax; d->fluxmin = ls.fluxmin; d->rho2 = ls.rho2;                                  \
    }                                                                                                        \
  }                                                                                                          \
  void orc_limiter_mask_##S(T* defplim, const T* def, const T* defp, int n, T dtold, uint8_t* mask,         \
                            orc_diag* d) {                                                                   \
    LimStats ls;                                                                                             \
    limiter_mask(defplim, def, defp, n, dtold, T(10), ls, mask);                                            \
    if (d) { d->ncompress = ls.ncompress; d->cmax = ls.cmax; }                                              \
  }                                                                                                          \
  void orc_limiter_poisson_##S(T* defp, const T* defplim, int n) { limiter_poisson(defp, defplim, n); }     \
  void orc_gradient_##S(const T* in, T* out, int n) { gradient(in, out, n); }                               \
  void orc_delta_##S(const T* in, T* out, int n) { delta(in, out, n); }                                     \
  void orc_relaxing_##S(T* u, const T* def, const T* defp, int n, int nf, T dt) {                           \
    relaxing(u, def, defp, n, nf, dt);                                                                       \
  }                                                                                                          \
  int orc_calcdefp_##S(T* defp, const T* def, const T* u, int nf, int n, T dtold, T dtaumesh, int sched,     \
                       int nu1, int nu2, double tol, int maxcyc, int colour8, uint8_t* mexp, uint8_t* mc1,   \
                       uint8_t* mc2, orc_diag* d) {                                                          \
    MgCfg cfg = make_cfg(n, sched, nu1, nu2, tol, maxcyc, colour8);                                        \
    MgStats st;                                                                                              \
    LimStats ls;                                                                                             \
    calcdefp(defp, def, u, nf, n, dtold, dtaumesh, cfg, st, ls, mexp, mc1, mc2);                            \
    if (d) {                                                                                                 \
      d->r1 = st.r1; d->relaxerr = st.relaxerr; d->rhsnorm = st.rhsnorm; d->resid_rel = st.resid_rel;       \
      d->vcycles = st.vcycles; d->guards = st.guards; d->bad = st.bad;                                      \
      d->nexpand = ls.nexpand; d->ncompress = ls.ncompress; d->cmax = ls.cmax; d->detmax = ls.detmax;       \
      d->detmin = ls.detmin; d->fluxmax = ls.fluxmax; d->fluxmin = ls.fluxmin; d->rho2 = ls.rho2;           \
    }                                                                                                        \
    return st.bad ? -1 : 0;                                                                                  \
  }
ORC_BOTH(DEF_LIM)

// multigrid at size n inside a build whose top-level size is ng (reference schedule)
int orc_multigrid_ng_d(double* u, double* rhs, const double* def, const double* rho, int n, int ng, double dx) {
  MgCfg cfg = make_cfg(ng, 0, 2, 2, 1e-10, 1, 0);
  MgStats st;
  multigrid(u, rhs, def, rho, n, dx, cfg, st);
  return st.bad ? -1 : 0;
}

// raw NR-semantics transforms (double only), for tests
void orc_rlft3_fwd(const double* x, int n, double* Xri) {
  rlft3_fwd(x, n, reinterpret_cast<cd*>(Xri));
}
void orc_rlft3_inv(const double* Xri, int n, double* x) {
  rlft3_inv(reinterpret_cast<const cd*>(Xri), n, x);
}

// r1lax schedule trace: writes the 1-based plane of every relaxplane call
// (positive) and calcresid call (negative) in the literal order; returns count.
int orc_r1lax_trace(int na3, int nrelax, int iopt, int* out, int cap) {
  int cnt = 0;
  // re-run the literal emission with recording callbacks
  int iresidopt = iopt % 8;
  auto RP = [&](int k) { if (cnt < cap) out[cnt] = k; cnt++; };
  auto CR = [&](int k) { if (cnt < cap) out[cnt] = -k; cnt++; };
  auto md = [&](int a) { return ((a % na3) + na3) % na3; };
  if (nrelax == 0) {
    for (int k = 2; k <= na3; k += 2) CR(k);
    return cnt;
  }
  RP(1);
  for (int ko = 2; ko <= (nrelax - 1) * 4 + 1; ko += 2) {
    int iclvls = (ko - 2) / 4;
    for (int ki = 0; ki <= iclvls; ++ki) {
      RP(md(ko - 2 * ki + 4 * na3) + 1);
      RP(md(ko - 2 * ki + 4 * na3 - 1) + 1);
    }
    if (ko % 4 == 0) RP(md(ko / 2) + 1);
  }
  for (int ko = (nrelax - 1) * 4 + 2; ko <= na3 - 1; ko += 2) {
    for (int ki = 1; ki <= nrelax * 2; ki += 2) {
      RP(ko - ki + 2);
      RP(ko - ki + 1);
    }
    if (iresidopt > 0 && ko > (nrelax - 1) * 4 + 2) CR(md(4 * na3 + ko - nrelax * 2 + 1) + 1);
  }
  int k = na3;
  RP(k);
  for (int ki = 2; ki <= nrelax; ++ki) {
    k = md(4 * na3 - 2 * ki + 2) + 1;
    RP(k);
    k = md(4 * na3 - 2 * ki + 1) + 1;
    RP(k);
  }
  if (iresidopt > 0) CR(md(4 * na3 - nrelax * 2 + 1) + 1);
  k = 3;
  for (int ko = 1; ko <= nrelax - 1; ++ko) {
    k = md(4 * na3 + 2 * ko + 2) + 1;
    for (int it = 1; it <= 2; ++it)
      for (int ki = 1; ki <= nrelax - ko; ++ki) {
        if (it != 2 || ki != 1) {
          k = md(4 * na3 + 2 * ko - 2 * ki + 2 * it - 2) + 1;
          RP(k);
        }
        k = md(4 * na3 + 2 * ko - 2 * ki + 2 * it - 3) + 1;
        RP(k);
      }
    if (iresidopt > 0) {
      CR(md(4 * na3 + 4 * ko - 2 * nrelax - 1) + 1);
      CR(md(4 * na3 + 4 * ko - 2 * nrelax + 1) + 1);
    }
  }
  if (iresidopt > 0) {
    k = md(k + 1) + 1;
    if (nrelax == 1) k = 2;
    CR(k);
  }
  return cnt;
}

}  // extern "C"
