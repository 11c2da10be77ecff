// After the path: the column density of mmh/column_density.f90 and the
// displacement interpolation, new positions and column density of
// gridfigure.f90:41-120.  FP32 as the reference computes them, compiled with
// --fmad=false so every operation rounds as written; one thread per column
// (the displaced faces of column (i, j) need only the two planes around them,
// so no displacement field is stored).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "../../include/mmh.h"
#include "mmh_kernels.cuh"

namespace mmh {
namespace {

constexpr int kB = 256;
unsigned nblk(i64 count) { return (unsigned)((count + kB - 1) / kB); }

__device__ __forceinline__ int imod(int a, int p) {
  int r = a % p;
  return r < 0 ? r + p : r;
}

// exact sum of a float array (fixed point, 64 fractional bits)
__global__ void k_post_fsum(const float* __restrict__ a, i64 count, unsigned long long* acc, int* flag) {
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

// den / sum(den) * ng**3 in real(4), the sum exact and rounded once
struct Norm {
  const float* den;
  int ng;
  float sf, scale;
  __device__ __forceinline__ float at(int i, int j, int k) const {  // 1-based i, j; k wraps
    int kw = imod(k - 1, ng);
    return den[(i - 1) + (i64)ng * ((j - 1) + (i64)ng * kw)] / sf * scale;
  }
};

// column_density.f90:42-53: the column of (i, j) between the displaced faces
// kk1 and kk2 with fractional end cells (cells outside 1..ng wrap; the
// reference reads out of bounds there)
__device__ float column(const Norm& D, int i, int j, float kk1, float kk2, int* flag) {
  // faces more than 4 ng cells apart (displacements of several boxes) or not
  // finite: flagged, not summed
  if (!(fabsf(kk2 - kk1) <= 4.0f * (float)D.ng) || !(fabsf(kk1) < 1.0e9f)) {
    atomicOr(flag, 2);
    return 0.0f;
  }
  int nk1 = (int)floorf(kk1) + 1, nk2 = (int)floorf(kk2) + 1;
  float r1 = (float)nk1 - kk1;
  float r2 = kk2 - (float)nk2 + 1.0f;
  float s1 = 0.0f, s2 = 0.0f;
  for (int k = nk1 + 1; k <= nk2 - 1; ++k) s1 = s1 + D.at(i, j, k);
  for (int k = nk2; k <= nk1; ++k) s2 = s2 + D.at(i, j, k);
  float t = r1 * D.at(i, j, nk1) + s1;
  t = t + r2 * D.at(i, j, nk2);
  return t - s2;
}

// dspz of column_density.f90:29-37 at (i, j, k), 1-based
__device__ __forceinline__ float dspz(const float* __restrict__ def, int ng, int i, int j, int k) {
  auto F = [&](int a, int b, int c) { return def[(a - 1) + (i64)ng * ((b - 1) + (i64)ng * (c - 1))]; };
  int kp = k % ng + 1, jp = j % ng + 1, ip = i % ng + 1;
  float v = F(i, j, kp) + F(ip, j, kp);
  v = v + F(i, jp, kp);
  v = v + F(ip, jp, kp);
  v = v - F(i, j, k);
  v = v - F(ip, j, k);
  v = v - F(i, jp, k);
  v = v - F(ip, jp, k);
  return v / 4.0f;
}

__global__ void k_column_density(const float* __restrict__ den, const float* __restrict__ def, int ng, int nplot,
                                 const unsigned long long* acc, float* __restrict__ proj, int* flag) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)ng * ng) return;
  int i = (int)(t % ng) + 1, j = (int)(t / ng) + 1;
  Norm D{den, ng, (float)fx_to(acc[0], acc[1]), (float)(int)((i64)ng * ng * ng)};
  const int k1 = ng / 2, k2 = k1 + nplot - 1;
  int jm = imod(j - 2, ng) + 1, im = imod(i - 2, ng) + 1, k1m = imod(k1 - 2, ng) + 1;
  float a = dspz(def, ng, im, jm, k1m) + dspz(def, ng, i, jm, k1m);
  a = a + dspz(def, ng, im, j, k1m);
  a = a + dspz(def, ng, i, j, k1m);
  float kk1 = (float)(k1 - 1) + a / 4.0f;
  float b = dspz(def, ng, im, jm, k2) + dspz(def, ng, i, jm, k2);
  b = b + dspz(def, ng, im, j, k2);
  b = b + dspz(def, ng, i, j, k2);
  float kk2 = (float)k2 + b / 4.0f;
  proj[t] = column(D, i, j, kk1, kk2, flag) / (float)nplot;
}

// gridfigure.f90:46-56: the displacement of the coarse def at the nodes
// 1..nf of the (0:nf)^3 node grid (3 components fastest); index-0 planes 0
__global__ void k_grid_nodes(const float* __restrict__ def, int nf, float* __restrict__ T0) {
  const int m = nf + 1;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)m * m * m) return;
  int i = (int)(t % m), j = (int)((t / m) % m), k = (int)(t / ((i64)m * m));
  if (i == 0 || j == 0 || k == 0) {
    T0[3 * t] = T0[3 * t + 1] = T0[3 * t + 2] = 0.0f;
    return;
  }
  auto F = [&](int a, int b, int c) { return def[(a - 1) + (i64)nf * ((b - 1) + (i64)nf * (c - 1))]; };
  int ip = i % nf + 1, jp = j % nf + 1, kp = k % nf + 1;
  float x = F(ip, j, k) - F(i, j, k);
  x = x + F(ip, jp, k);
  x = x - F(i, jp, k);
  x = x + F(ip, j, kp);
  x = x - F(i, j, kp);
  x = x + F(ip, jp, kp);
  x = x - F(i, jp, kp);
  float y = F(i, jp, k) - F(i, j, k);
  y = y + F(ip, jp, k);
  y = y - F(ip, j, k);
  y = y + F(i, jp, kp);
  y = y - F(i, j, kp);
  y = y + F(ip, jp, kp);
  y = y - F(ip, j, kp);
  float z = F(i, j, kp) - F(i, j, k);
  z = z + F(ip, j, kp);
  z = z - F(ip, j, k);
  z = z + F(i, jp, kp);
  z = z - F(i, jp, k);
  z = z + F(ip, jp, kp);
  z = z - F(ip, jp, k);
  T0[3 * t] = x;
  T0[3 * t + 1] = y;
  T0[3 * t + 2] = z;
}

// scale by real(ratio)*1./4. and the halo of gridfigure.f90:58-64: tmp =
// cshift(tmp_dsp, -1) along the three node dimensions, copied into the
// index-0 planes
__global__ void k_grid_halo(const float* __restrict__ T0, int nf, float cf, float* __restrict__ TD) {
  const int m = nf + 1;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)m * m * m) return;
  int i = (int)(t % m), j = (int)((t / m) % m), k = (int)(t / ((i64)m * m));
  auto w = [&](int v) { return v < 0 ? v + m : v; };
  auto at = [&](int a, int b, int c) { return 3 * (a + (i64)m * (b + (i64)m * c)); };
  i64 src = at(i, j, k);
  if (i == 0 && j >= 1 && k >= 1) src = at(w(-1), j - 1, k - 1);
  else if (i >= 1 && k == 0) src = at(i - 1, w(j - 1), w(-1));
  else if (i >= 1 && j == 0 && k >= 1) src = at(i - 1, w(-1), k - 1);
  for (int c = 0; c < 3; ++c) {
    float v = T0[src + c];
    // index-0 planes of T0 hold 0 (never assigned in the reference)
    TD[3 * t + c] = cf * v;
  }
}

// displacement component c at fine cell (i, j, k), 1-based (gridfigure.f90:66-96)
__device__ float grid_disp(const float* __restrict__ TD, int nf, int ratio, int c, int i, int j, int k) {
  const int m = nf + 1;
  float ib = (float)(i % ratio) / (float)ratio, jb = (float)(j % ratio) / (float)ratio,
        kb = (float)(k % ratio) / (float)ratio;
  int ip = (int)floorf((float)i / (float)ratio) + 1 - (int)floorf(ib);
  int jp = (int)floorf((float)j / (float)ratio) + 1 - (int)floorf(jb);
  int kp = (int)floorf((float)k / (float)ratio) + 1 - (int)floorf(kb);
  int i0 = ip - 1, j0 = jp - 1, k0 = kp - 1;
  int i1 = ip == nf + 1 ? 1 : ip, j1 = jp == nf + 1 ? 1 : jp, k1 = kp == nf + 1 ? 1 : kp;
  auto T = [&](int a, int b, int d) { return TD[3 * (a + (i64)m * (b + (i64)m * d)) + c]; };
  float p111 = ib * jb * kb, p211 = (1.0f - ib) * jb * kb, p121 = ib * (1.0f - jb) * kb;
  float p112 = ib * jb * (1.0f - kb), p221 = (1.0f - ib) * (1.0f - jb) * kb, p212 = (1.0f - ib) * jb * (1.0f - kb);
  float p122 = ib * (1.0f - jb) * (1.0f - kb), p222 = (1.0f - ib) * (1.0f - jb) * (1.0f - kb);
  float d = 0.0f;
  d = d + T(i0, j0, k0) * p111;
  d = d + T(i1, j0, k0) * p211;
  d = d + T(i0, j1, k0) * p121;
  d = d + T(i0, j0, k1) * p112;
  d = d + T(i1, j1, k0) * p221;
  d = d + T(i1, j0, k1) * p212;
  d = d + T(i0, j1, k1) * p122;
  d = d + T(i1, j1, k1) * p222;
  return d;
}

__global__ void k_grid_column(const float* __restrict__ den, const float* __restrict__ TD, int nf, int ng,
                              const unsigned long long* acc, float* __restrict__ proj, int* flag) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)ng * ng) return;
  const int ratio = ng / nf;
  int i = (int)(t % ng) + 1, j = (int)(t / ng) + 1;
  Norm D{den, ng, (float)fx_to(acc[0], acc[1]), (float)(int)((i64)ng * ng * ng)};
  const int k1 = ng / 2, k2 = k1;
  int jm = imod(j - 2, ng) + 1, im = imod(i - 2, ng) + 1, k1m = imod(k1 - 2, ng) + 1;
  float a = grid_disp(TD, nf, ratio, 2, im, jm, k1m) + grid_disp(TD, nf, ratio, 2, i, jm, k1m);
  a = a + grid_disp(TD, nf, ratio, 2, im, j, k1m);
  a = a + grid_disp(TD, nf, ratio, 2, i, j, k1m);
  float kk1 = (float)(k1 - 1) + a / 4.0f;
  float b = grid_disp(TD, nf, ratio, 2, im, jm, k2) + grid_disp(TD, nf, ratio, 2, i, jm, k2);
  b = b + grid_disp(TD, nf, ratio, 2, im, j, k2);
  b = b + grid_disp(TD, nf, ratio, 2, i, j, k2);
  float kk2 = (float)k2 + b / 4.0f;
  proj[t] = column(D, i, j, kk1, kk2, flag) / 1.0f;
}

// proj2(1:2, a, b) = newposition(1:2, ratio*a, ratio*b, ng/2)
__global__ void k_grid_positions(const float* __restrict__ TD, int nf, int ng, float* __restrict__ proj2) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)nf * nf) return;
  const int ratio = ng / nf;
  int a = (int)(t % nf) + 1, b = (int)(t / nf) + 1;
  int idx[3] = {ratio * a, ratio * b, ng / 2};
  for (int c = 0; c < 2; ++c)
    proj2[2 * t + c] = ((float)idx[c] + 0.5f) + grid_disp(TD, nf, ratio, c, idx[0], idx[1], idx[2]);
}

struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
};

#define QK(x)                                                                                     \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess) {                                                                      \
      fprintf(stderr, "mmh: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return e_ == cudaErrorMemoryAllocation ? MMH_ERR_NOMEM : MMH_ERR_CUDA;                      \
    }                                                                                             \
  } while (0)

}  // namespace
}  // namespace mmh

using namespace mmh;

extern "C" {

int mmh_column_density(const float* den, const float* def, int ng, int nplot, float* proj) {
  if (!den || !def || !proj || ng < 2 || nplot < 1) return MMH_ERR_ARG;
  const i64 n3 = (i64)ng * ng * ng;
  Dev mem;
  QK(cudaMalloc(&mem.p, sizeof(float) * (2 * n3 + (i64)ng * ng) + 64));
  float* dden = (float*)mem.p;
  float* ddef = dden + n3;
  float* dproj = ddef + n3;
  unsigned long long* acc = (unsigned long long*)(((uintptr_t)(dproj + (i64)ng * ng) + 15) & ~(uintptr_t)15);
  int* flag = (int*)(acc + 2);
  QK(cudaMemcpy(dden, den, sizeof(float) * n3, cudaMemcpyHostToDevice));
  QK(cudaMemcpy(ddef, def, sizeof(float) * n3, cudaMemcpyHostToDevice));
  QK(cudaMemset(acc, 0, 24));
  k_post_fsum<<<(unsigned)std::min<i64>(nblk(n3), 152 * 8), kB>>>(dden, n3, acc, flag);
  k_column_density<<<nblk((i64)ng * ng), kB>>>(dden, ddef, ng, nplot, acc, dproj, flag);
  count_launch(2);
  QK(cudaGetLastError());
  int hflag = 0;
  QK(cudaMemcpy(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (hflag) return MMH_ERR_RANGE;
  QK(cudaMemcpy(proj, dproj, sizeof(float) * ng * ng, cudaMemcpyDeviceToHost));
  return MMH_OK;
}

int mmh_gridfigure(const float* def, int nf, const float* den, int ng, float* proj2, float* proj) {
  if (!def || !den || (!proj2 && !proj) || nf < 2 || ng < nf || ng % nf) return MMH_ERR_ARG;
  const i64 n3 = (i64)ng * ng * ng, m3 = (i64)(nf + 1) * (nf + 1) * (nf + 1), f3 = (i64)nf * nf * nf;
  Dev mem;
  QK(cudaMalloc(&mem.p, sizeof(float) * (n3 + f3 + 6 * m3 + (i64)ng * ng + 2 * (i64)nf * nf) + 64));
  float* dden = (float*)mem.p;
  float* ddef = dden + n3;
  float* T0 = ddef + f3;
  float* TD = T0 + 3 * m3;
  float* dproj = TD + 3 * m3;
  float* dproj2 = dproj + (i64)ng * ng;
  unsigned long long* acc = (unsigned long long*)(((uintptr_t)(dproj2 + 2 * (i64)nf * nf) + 15) & ~(uintptr_t)15);
  int* flag = (int*)(acc + 2);
  QK(cudaMemcpy(dden, den, sizeof(float) * n3, cudaMemcpyHostToDevice));
  QK(cudaMemcpy(ddef, def, sizeof(float) * f3, cudaMemcpyHostToDevice));
  QK(cudaMemset(acc, 0, 24));
  const int ratio = ng / nf;
  const float cf = (float)ratio * 1.0f / 4.0f;
  k_grid_nodes<<<nblk(m3), kB>>>(ddef, nf, T0);
  k_grid_halo<<<nblk(m3), kB>>>(T0, nf, cf, TD);
  k_post_fsum<<<(unsigned)std::min<i64>(nblk(n3), 152 * 8), kB>>>(dden, n3, acc, flag);
  k_grid_column<<<nblk((i64)ng * ng), kB>>>(dden, TD, nf, ng, acc, dproj, flag);
  k_grid_positions<<<nblk((i64)nf * nf), kB>>>(TD, nf, ng, dproj2);
  count_launch(5);
  QK(cudaGetLastError());
  int hflag = 0;
  QK(cudaMemcpy(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (hflag) return MMH_ERR_RANGE;
  if (proj) QK(cudaMemcpy(proj, dproj, sizeof(float) * ng * ng, cudaMemcpyDeviceToHost));
  if (proj2) QK(cudaMemcpy(proj2, dproj2, sizeof(float) * 2 * nf * nf, cudaMemcpyDeviceToHost));
  return MMH_OK;
}

}  // extern "C"
