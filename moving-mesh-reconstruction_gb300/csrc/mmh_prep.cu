// Input preparation on the GPU (the step before the path): haloden.f90's
// particle density assignment and from1024to512.f90's coarsening.  FP32 as
// the reference computes them, compiled with --fmad=false so every operation
// rounds as written.
//
// haloden.f90:87-189, restated:
//   xp = modulo(x, nf) * ng / nf; each particle's cell is floor(xp) + 1;
//   every empty cell is given to the particle nearest its centre among those
//   in the first cube shell (growing r) around it that holds any, the
//   reference's scan order deciding ties; a particle's unit mass is shared
//   equally (1/wp) by its own cell and the empty cells it was given; the
//   density is normalised to mean 1.
// The GPU form: one stable radix sort of (cell, particle) pairs gives each
// cell its particles in ascending index order (the reference's linked lists
// hold them in descending order, and its density loop adds them in ascending
// order); the empty-cell searches run one thread per cell; each cell sums its
// particles' shares in the reference's order.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/mmh.h"
#include "mmh_kernels.cuh"

namespace mmh {
namespace {

constexpr int kB = 256;
// largest search radius (cells) of an empty cell's nearest-particle search
constexpr int kHaloMaxRadius = 64;
unsigned blocks_of(i64 count) { return (unsigned)((count + kB - 1) / kB); }

// Fortran MODULO for reals: the exact remainder, moved into [0, p).
__device__ __forceinline__ float fmodulo(float a, float p) {
  float r = fmodf(a, p);
  if (r != 0.0f && ((r < 0.0f) != (p < 0.0f))) r = r + p;
  return r;
}

// positions to grid units and cells (haloden.f90:87-108)
__global__ void k_halo_cells(const float* __restrict__ x, i64 np, int nf, int ng, float* __restrict__ xp,
                             unsigned* __restrict__ cell, unsigned* __restrict__ ip_out, int* flag) {
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  int c[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float v = fmodulo(x[3 * p + a], (float)nf);
    v = v * (float)ng / (float)nf;
    xp[3 * p + a] = v;
    c[a] = (int)floorf(v);
  }
  bool ok = c[0] >= 0 && c[0] < ng && c[1] >= 0 && c[1] < ng && c[2] >= 0 && c[2] < ng;
  if (!ok) {
    atomicOr(flag, 1);
    c[0] = c[1] = c[2] = 0;
  }
  cell[p] = (unsigned)(c[0] + ng * (c[1] + ng * c[2]));
  ip_out[p] = (unsigned)p;
}

// first and one-past-last sorted position of each non-empty cell
__global__ void k_halo_bounds(const unsigned* __restrict__ key, i64 np, int* __restrict__ first,
                              int* __restrict__ last) {
  i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np) return;
  unsigned k = key[q];
  if (q == 0 || key[q - 1] != k) first[k] = (int)q;
  if (q == np - 1 || key[q + 1] != k) last[k] = (int)(q + 1);
}

// Each empty cell: the nearest particle of the first non-empty cube shell
// (haloden.f90:127-170).  Cells are scanned in the reference's order (k_s, j_s,
// i_s), each cell's particles in its linked-list order (descending index), and
// only a strictly smaller distance replaces the choice, so ties go as there.
// The shells grow to at most rmax cells; a cell with no particle within that
// radius sets flag bit 4 (the reference's search would go on, and so would
// its cost: (2r+1)^3 cells per empty cell).  Launched on cells [g0, g1).
__global__ void k_halo_search(const float* __restrict__ xp, const unsigned* __restrict__ order,
                              const int* __restrict__ first, const int* __restrict__ last, int ng, int rmax,
                              i64 g0, i64 g1, int* __restrict__ choice, int* __restrict__ wp, int* flag) {
  i64 g = g0 + (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= g1) return;
  if (first[g] >= 0) return;
  int i = (int)(g % ng), j = (int)((g / ng) % ng), k = (int)(g / ((i64)ng * ng));
  const float gx = (float)(i + 1) - 0.5f, gy = (float)(j + 1) - 0.5f, gz = (float)(k + 1) - 0.5f;
  const float h = (float)(ng / 2), fng = (float)ng;
  float r2min = (float)(1000 * ng * ng);
  int best = -1;
  for (int r = 1; r <= rmax && best < 0; ++r) {
    for (int dk = -r; dk <= r; ++dk)
      for (int dj = -r; dj <= r; ++dj)
        for (int di = -r; di <= r; ++di) {
          // cells inside the shell were empty at the previous radius
          if (dk > -r && dk < r && dj > -r && dj < r && di > -r && di < r) continue;
          int ii = ((i + di) % ng + ng) % ng, jj = ((j + dj) % ng + ng) % ng, kk = ((k + dk) % ng + ng) % ng;
          i64 c = ii + (i64)ng * (jj + (i64)ng * kk);
          int f = first[c];
          if (f < 0) continue;
          for (int q = last[c] - 1; q >= f; --q) {
            int p = (int)order[q];
            float d0 = fmodulo(xp[3 * p] - gx + h, fng) - h;
            float d1 = fmodulo(xp[3 * p + 1] - gy + h, fng) - h;
            float d2 = fmodulo(xp[3 * p + 2] - gz + h, fng) - h;
            float r2 = d0 * d0 + d1 * d1;
            r2 = r2 + d2 * d2;
            if (r2 < r2min) {
              r2min = r2;
              best = p;
            }
          }
        }
  }
  choice[g] = best;
  if (best >= 0) atomicAdd(&wp[best], 1);
  else atomicOr(flag, 4);
}

// the unnormalised density (haloden.f90:173-182): a cell's particles add
// 1/wp in ascending index order; an empty cell holds its particle's share
__global__ void k_halo_density(const unsigned* __restrict__ order, const int* __restrict__ first,
                               const int* __restrict__ last, const int* __restrict__ choice,
                               const int* __restrict__ wp, i64 ng3, float* __restrict__ raw) {
  i64 g = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng3) return;
  int f = first[g];
  float s = 0.0f;
  if (f >= 0) {
    for (int q = f; q < last[g]; ++q) s = s + 1.0f / (float)wp[order[q]];
  } else {
    int p = choice[g];
    s = p >= 0 ? 0.0f + 1.0f / (float)wp[p] : 0.0f;
  }
  raw[g] = s;
}

// exact sum of a float array (fixed point, 64 fractional bits)
__global__ void k_fsum(const float* __restrict__ a, i64 count, unsigned long long* acc, int* flag) {
  __int128 s = 0;
  bool bad = false;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (i64)gridDim.x * blockDim.x) {
    double x = (double)a[t];
    if (!(fabs(x) < 4294967296.0)) bad = true;
    else s += fx_of(x);
  }
  if (bad) atomicOr(flag, 2);
  fx_block_commit(s, acc);
}

// den = real(raw, 8) / sum * scale, rounded to real(4) (haloden.f90:189)
__global__ void k_halo_norm(const float* __restrict__ raw, i64 ng3, const unsigned long long* acc, double scale,
                            float* __restrict__ den) {
  i64 g = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng3) return;
  double s = fx_to(acc[0], acc[1]);
  den[g] = (float)((double)raw[g] / s * scale);
}

// one halving of from1024to512.f90's coarsen: the sum over the 2x2x2 block,
// first index fastest
__global__ void k_coarsen2(const float* __restrict__ a, int nf, float* __restrict__ b) {
  int h = nf / 2;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)h * h * h) return;
  int i = (int)(t % h), j = (int)((t / h) % h), k = (int)(t / ((i64)h * h));
  float s = 0.0f;
  for (int dk = 0; dk < 2; ++dk)
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) s = s + a[(2 * i + di) + (i64)nf * ((2 * j + dj) + (i64)nf * (2 * k + dk))];
  b[t] = s;
}

// out = a / sum * n^3 in real(4), the sum taken exactly and rounded to real(4)
__global__ void k_coarse_norm(const float* __restrict__ a, i64 n3, const unsigned long long* acc,
                              float* __restrict__ out) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  float sf = (float)fx_to(acc[0], acc[1]);
  out[t] = a[t] / sf * (float)n3;
}

__global__ void k_fill_int(int* __restrict__ a, i64 count, int v) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) a[t] = v;
}

struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
};

#define PK(x)                                                                                     \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess) {                                                                      \
      fprintf(stderr, "mmh: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return e_ == cudaErrorMemoryAllocation ? MMH_ERR_NOMEM : MMH_ERR_CUDA;                      \
    }                                                                                             \
  } while (0)

unsigned sum_blocks(i64 count) { return (unsigned)std::min<i64>((count + kB - 1) / kB, 152 * 8); }

// bump allocator over one device allocation (256-byte aligned pieces)
struct Carve {
  char* at;
  template <class T>
  T* take(i64 count) {
    T* r = (T*)at;
    at += ((size_t)count * sizeof(T) + 255) / 256 * 256;
    return r;
  }
};

}  // namespace
}  // namespace mmh

using namespace mmh;

extern "C" {

int mmh_haloden(const float* x, long long np, int nf, int ng, float* den, float* raw, int* wp) {
  if (!x || !den || np < 1 || nf < 1 || ng < 2 || ng > 1024) return MMH_ERR_ARG;
  if (np >= (1ll << 31)) return MMH_ERR_SIZE;
  const i64 ng3 = (i64)ng * ng * ng;
  int bits = 1;
  while ((1ll << bits) < ng3) ++bits;
  size_t sort_bytes = 0;
  PK(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (const unsigned*)nullptr, (unsigned*)nullptr,
                                     (const unsigned*)nullptr, (unsigned*)nullptr, (int)np, 0, bits));
  const size_t bytes = 256 * 16 + sizeof(float) * 6 * (size_t)np + sizeof(unsigned) * 4 * (size_t)np +
                       sizeof(int) * (size_t)np + sizeof(int) * 3 * (size_t)ng3 + sizeof(float) * 2 * (size_t)ng3 +
                       sort_bytes;
  Dev mem;
  PK(cudaMalloc(&mem.p, bytes));
  Carve cv{(char*)mem.p};
  float* dx = cv.take<float>(3 * np);
  float* xp = cv.take<float>(3 * np);
  unsigned* key = cv.take<unsigned>(np);
  unsigned* ips = cv.take<unsigned>(np);
  unsigned* skey = cv.take<unsigned>(np);
  unsigned* order = cv.take<unsigned>(np);
  int* dwp = cv.take<int>(np);
  int* first = cv.take<int>(ng3);
  int* last = cv.take<int>(ng3);
  int* choice = cv.take<int>(ng3);
  float* draw = cv.take<float>(ng3);
  float* dden = cv.take<float>(ng3);
  unsigned long long* acc = cv.take<unsigned long long>(2);
  int* flag = cv.take<int>(1);
  void* sort_tmp = cv.take<char>((i64)sort_bytes);
  PK(cudaMemcpy(dx, x, sizeof(float) * 3 * np, cudaMemcpyHostToDevice));
  PK(cudaMemset(first, 0xff, sizeof(int) * ng3));
  PK(cudaMemset(acc, 0, 16));
  PK(cudaMemset(flag, 0, sizeof(int)));
  k_halo_cells<<<blocks_of(np), kB>>>(dx, np, nf, ng, xp, key, ips, flag);
  count_launch();
  PK(cub::DeviceRadixSort::SortPairs(sort_tmp, sort_bytes, key, skey, ips, order, (int)np, 0, bits));
  k_halo_bounds<<<blocks_of(np), kB>>>(skey, np, first, last);
  k_fill_int<<<blocks_of(np), kB>>>(dwp, np, 1);
  // empty-cell searches in chunks, the flag read between them, so an input
  // whose voids exceed the radius cap ends after one chunk
  const int rmax = std::min(ng / 2 + 1, kHaloMaxRadius);
  const i64 chunk = (i64)1 << 20;
  for (i64 g0 = 0; g0 < ng3; g0 += chunk) {
    const i64 g1 = std::min(ng3, g0 + chunk);
    k_halo_search<<<blocks_of(g1 - g0), kB>>>(xp, order, first, last, ng, rmax, g0, g1, choice, dwp, flag);
    count_launch();
    int hf = 0;
    PK(cudaMemcpy(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (hf & 4) return MMH_ERR_RANGE;
  }
  k_halo_density<<<blocks_of(ng3), kB>>>(order, first, last, choice, dwp, ng3, draw);
  k_fsum<<<sum_blocks(ng3), kB>>>(draw, ng3, acc, flag);
  const double scale = (double)((float)ng * (float)ng * (float)ng);
  k_halo_norm<<<blocks_of(ng3), kB>>>(draw, ng3, acc, scale, dden);
  count_launch(5);
  PK(cudaGetLastError());
  int hflag = 0;
  PK(cudaMemcpy(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (hflag & 1) return MMH_ERR_RANGE;  // a position outside the grid after the wrap
  if (hflag & 2) return MMH_ERR_RANGE;
  PK(cudaMemcpy(den, dden, sizeof(float) * ng3, cudaMemcpyDeviceToHost));
  if (raw) PK(cudaMemcpy(raw, draw, sizeof(float) * ng3, cudaMemcpyDeviceToHost));
  if (wp) PK(cudaMemcpy(wp, dwp, sizeof(int) * np, cudaMemcpyDeviceToHost));
  return MMH_OK;
}

int mmh_coarsen(const float* den, int ng, int ncoarse, float* out) {
  if (!den || !out || ng < 2 || ncoarse < 0 || ncoarse > 10 || ((ng >> ncoarse) << ncoarse) != ng || (ng >> ncoarse) < 1)
    return MMH_ERR_ARG;
  const i64 ng3 = (i64)ng * ng * ng;
  const int nc = ng >> ncoarse;
  const i64 n3 = (i64)nc * nc * nc;
  Dev mem;
  PK(cudaMalloc(&mem.p, sizeof(float) * (ng3 + ng3 / 8 + 1 + n3) + 256 * 5));
  Carve cv{(char*)mem.p};
  float* a = cv.take<float>(ng3);
  float* b = cv.take<float>(ng3 / 8 + 1);
  float* res = cv.take<float>(n3);
  unsigned long long* acc = cv.take<unsigned long long>(2);
  int* flag = cv.take<int>(1);
  PK(cudaMemcpy(a, den, sizeof(float) * ng3, cudaMemcpyHostToDevice));
  PK(cudaMemset(acc, 0, 16));
  PK(cudaMemset(flag, 0, sizeof(int)));
  // halvings alternate between a and b (b holds any grid after the first)
  float* cur = a;
  int nf = ng;
  for (int c = 0; c < ncoarse; ++c) {
    float* nxt = (cur == a) ? b : a;
    const i64 h3 = (i64)(nf / 2) * (nf / 2) * (nf / 2);
    k_coarsen2<<<blocks_of(h3), kB>>>(cur, nf, nxt);
    cur = nxt;
    nf /= 2;
    count_launch();
  }
  k_fsum<<<sum_blocks(n3), kB>>>(cur, n3, acc, flag);
  k_coarse_norm<<<blocks_of(n3), kB>>>(cur, n3, acc, res);
  count_launch(2);
  PK(cudaGetLastError());
  int hflag = 0;
  PK(cudaMemcpy(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (hflag) return MMH_ERR_RANGE;
  PK(cudaMemcpy(out, res, sizeof(float) * n3, cudaMemcpyDeviceToHost));
  return MMH_OK;
}

}  // extern "C"
