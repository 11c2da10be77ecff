// FP32 kernels of the mixed-precision inner V-cycle (smoother, residual,
// restriction, prolongation, zero-mean).  FMA contraction stays enabled here.
#include <mutex>

#include "mmh_launch.cuh"
#include "mmh_pcg.cuh"

namespace mmh {

// Tile autotuning of the FP32 plane kernel (see gs_tile_choice), per device
// (up to 64) and grid size (2^0 .. 2^15).
static std::mutex g_tile_mu;
static signed char g_tile[64][16];
static bool g_tile_init = false;
std::atomic<int> gs_tile_override{-1};
std::atomic<int> stencil_march_pin{-1};

int gs_tile_choice(int n, const float* phi, const float* rhs, const float* coef, float dx2, float* scratch,
                   cudaStream_t s) {
  const int pin = gs_tile_override.load();
  if (pin >= 0 && pin < kGsShapes && gs_shape_fits(pin, n)) return pin;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  int lg = 0;
  while ((1 << lg) < n && lg < 15) ++lg;
  {
    std::lock_guard<std::mutex> lock(g_tile_mu);
    if (!g_tile_init) {
      for (auto& row : g_tile)
        for (auto& x : row) x = -1;
      g_tile_init = true;
    }
    if (g_tile[dev][lg] >= 0) return g_tile[dev][lg];
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return 0;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return 0;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return 0;
  }
  int best = 0;
  float best_ms = 0.f;
  for (int v = 0; v < kGsShapes; ++v) {
    if (!gs_shape_fits(v, n)) continue;
    gs_plane_half<float>(v, phi, phi, scratch, rhs, coef, n, dx2, 0, s);  // warm-up (attribute, caches)
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; ++r) gs_plane_half<float>(v, phi, phi, scratch, rhs, coef, n, dx2, 0, s);
    cudaEventRecord(e1, s);
    count_launch(4);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) continue;
    if (v == 0 || ms < best_ms) {
      best = v;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::lock_guard<std::mutex> lock(g_tile_mu);
  g_tile[dev][lg] = (signed char)best;
  return best;
}

int gs_tile_chosen(int n, int* tx, int* ty) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  int lg = 0;
  while ((1 << lg) < n && lg < 15) ++lg;
  std::lock_guard<std::mutex> lock(g_tile_mu);
  if (!g_tile_init || g_tile[dev][lg] < 0) return -1;
  const int v = g_tile[dev][lg];
  *tx = kGsShape[v].tx;
  *ty = kGsShape[v].ty;
  return v;
}

MMH_INSTANTIATE(float)
MMH_INSTANTIATE_PCG(float)

// Dot product of two FP32 vectors for the mixed form's inner solve, whose
// results are not bit-matched to the oracle: a fixed grid of kDotBlocks
// blocks, each thread summing its strided products in FP32 with four
// accumulators, each block reducing in a fixed pattern, and one block adding
// the block sums in FP64 in a fixed order -- deterministic, and bound by
// memory instead of by the integer work of the exact form.  The result is
// stored in the fixed-point form (same scale) the PCG scalar kernel reads.
__device__ __forceinline__ float block_sum_f32(float v, float* buf) {
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) buf[w] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += buf[q];
  return t;
}

__global__ void __launch_bounds__(256) k_dot_f32_part(const float* __restrict__ a, const float* __restrict__ b,
                                                      i64 count, double* __restrict__ part) {
  __shared__ float buf[32];
  const i64 stride = (i64)gridDim.x * blockDim.x;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  for (; t + 3 * stride < count; t += 4 * stride) {
    s0 += a[t] * b[t];
    s1 += a[t + stride] * b[t + stride];
    s2 += a[t + 2 * stride] * b[t + 2 * stride];
    s3 += a[t + 3 * stride] * b[t + 3 * stride];
  }
  for (; t < count; t += stride) s0 += a[t] * b[t];
  const float blk = block_sum_f32((s0 + s1) + (s2 + s3), buf);
  if (threadIdx.x == 0) part[blockIdx.x] = (double)blk;
}

__global__ void __launch_bounds__(256) k_dot_f32_final(const double* __restrict__ part, int nparts,
                                                       const unsigned long long* abits,
                                                       const unsigned long long* bbits, unsigned long long* acc) {
  __shared__ double buf[256];
  double s = 0.0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) s += part[q];
  buf[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) buf[threadIdx.x] += buf[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ma = bits_d(abits), mb = bits_d(bbits);
    __int128 v = 0;
    if (ma > 0.0 && mb > 0.0 && fabs(buf[0]) < INFINITY) v = fx_bits(buf[0], 96 - (ilogb(ma) + ilogb(mb) + 2));
    acc[0] = (unsigned long long)v;
    acc[1] = (unsigned long long)((unsigned __int128)v >> 64);
  }
}

void launch_dot_fast(const float* a, const float* b, i64 count, const unsigned long long* abits,
                            const unsigned long long* bbits, unsigned long long* acc, double* part, cudaStream_t s) {
  k_dot_f32_part<<<kDotBlocks, 256, 0, s>>>(a, b, count, part);
  k_dot_f32_final<<<1, 256, 0, s>>>(part, kDotBlocks, abits, bbits, acc);
  count_launch(2);
}

// FP64 residual with fused multiply-adds, for the outer loop of the mixed
// form (fewer FP64 operations; that form is not bit-matched to the oracle).
void launch_residual_fma(const double* phi, const double* rhs, const double* coef, int n, double dx, float* r32,
                         unsigned long long* maxbits, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  double di2 = 1.0 / (dx * dx);
  prof_begin(KK_RESIDUAL, s, n3, n);
  if (n >= 32)
    k_stencil_plane<double, 0, true><<<dim3(n / 32, n / 16, n), 256, 0, s>>>(phi, rhs, coef, n, di2, nullptr, r32,
                                                                             maxbits);
  else
    k_residual<double, true><<<grid_of(n3, kBlock), kBlock, 0, s>>>(phi, rhs, coef, n, di2, nullptr, r32, maxbits);
  prof_end(KK_RESIDUAL, s, n);
  count_launch();
}
}  // namespace mmh
