// Launcher templates for the multigrid kernels; each precision's translation
// unit includes this file and instantiates the launchers explicitly.
#pragma once
#include <atomic>
#include <type_traits>

#include "mmh_kernels.cuh"

namespace mmh {

static inline unsigned grid_of(i64 count, int block) { return (unsigned)((count + block - 1) / block); }
static const int kBlock = 256;

// Dynamic shared memory above the 48 KB default is an attribute of a kernel on
// one device: it is set on each device the library launches the kernel on,
// once per device (bit d of `done`).  A failure leaves the bit clear, and the
// launch that needs the attribute then fails and is reported by the entry
// point's launch-error check.
template <class K>
inline void smem_attr_once(K* kernel, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  const unsigned long long bit = 1ull << dev;
  if (done.load(std::memory_order_acquire) & bit) return;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess)
    done.fetch_or(bit, std::memory_order_acq_rel);
}

template <class T>
void launch_metric(const T* def, const T* rho, int n, T dx, T* coef, cudaStream_t s, bool fast_div) {
  i64 n3 = (i64)n * n * n;
  T di2 = T(1) / (dx * dx);
  prof_begin(kk<T>(KK_METRIC), s, n3, n);
  if (fast_div)
    k_metric<T, true><<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, rho, n, di2, coef);
  else
    k_metric<T, false><<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, rho, n, di2, coef);
  prof_end(kk<T>(KK_METRIC), s, n);
  count_launch();
}

// Tile shapes of the fused plane kernel.  Every shape updates every cell with
// the same operations in the same colour order, so the swept field is the
// same bit for bit whichever runs; the shapes differ in halo overhead, active
// threads per colour phase and shared memory.  Shapes 4-5 are the strips of
// 64 cells marching in y over 128 or 256 cell rows (k_gs_strip, LY = ty/2
// sub-rows).  FP32 levels try the shapes below once per grid size and device
// and keep the fastest (gs_tile_choice); FP64 levels keep (32, 8).
struct GsShape {
  int tx, ty;
};
constexpr GsShape kGsShape[kGsShapes] = {{32, 16}, {64, 8}, {16, 32}, {32, 8}, {64, 128}, {64, 256}};
constexpr int kGsFirstStrip = 4;

template <int LY, int Z>
void gs_strip_launch(const float* src, const float* nbr, float* dst, const float* rhs, const float* coef, int n,
                     float dx2, int kpar, cudaStream_t s) {
  k_gs_strip<LY, Z><<<dim3(n / StripGeom::SW, (n / 2) / LY, n / 2), StripGeom::NT, 0, s>>>(src, nbr, dst, rhs, coef,
                                                                                            n, dx2, kpar);
}

template <class T, int TX, int TY, int Z = 0>
void gs_plane_launch(const T* src, const T* nbr, T* dst, const T* rhs, const T* coef, int n, T dx2, int kpar,
                     cudaStream_t s) {
  const size_t smem = sizeof(T) * GsGeom<T, TX, TY>::WORDS;
  static std::atomic<unsigned long long> attr_done{0};
  smem_attr_once(k_gs_plane<T, TX, TY, Z>, (int)smem, attr_done);
  k_gs_plane<T, TX, TY, Z><<<dim3(n / TX, n / TY, n / 2), 256, smem, s>>>(src, nbr, dst, rhs, coef, n, dx2, kpar);
}

// one half sweep with tile shape v (FP64: always (32, 8))
// (the zero-field variants Z = 1, 2 exist for FP32 only)
template <class T, int Z = 0>
void gs_plane_half(int v, const T* src, const T* nbr, T* dst, const T* rhs, const T* coef, int n, T dx2, int kpar,
                   cudaStream_t s) {
  if constexpr (std::is_same<T, double>::value) {
    static_assert(Z == 0, "FP64 sweeps read their fields");
    (void)v;
    gs_plane_launch<T, 32, 8>(src, nbr, dst, rhs, coef, n, dx2, kpar, s);
  } else {
    switch (v) {
      case 1: gs_plane_launch<T, 64, 8, Z>(src, nbr, dst, rhs, coef, n, dx2, kpar, s); break;
      case 2: gs_plane_launch<T, 16, 32, Z>(src, nbr, dst, rhs, coef, n, dx2, kpar, s); break;
      case 3: gs_plane_launch<T, 32, 8, Z>(src, nbr, dst, rhs, coef, n, dx2, kpar, s); break;
      case 4: gs_strip_launch<64, Z>(src, nbr, dst, rhs, coef, n, dx2, kpar, s); break;
      case 5: gs_strip_launch<128, Z>(src, nbr, dst, rhs, coef, n, dx2, kpar, s); break;
      default: gs_plane_launch<T, 32, 16, Z>(src, nbr, dst, rhs, coef, n, dx2, kpar, s); break;
    }
  }
}

// the plane kernel needs n >= TX + 8 and n >= TY + 8; the strips n >= 64 and
// their LY sub-rows dividing the n/2 sub-rows of a plane
inline bool gs_shape_fits(int v, int n) {
  if (v >= kGsFirstStrip) return n >= 64 && (n / 2) % (kGsShape[v].ty / 2) == 0;
  return n >= kGsShape[v].tx + 8 && n >= kGsShape[v].ty + 8;
}

// Tile shape for an FP32 grid of size n on the current device: the one
// chosen before, else (outside a stream capture) each shape is timed on
// three half sweeps that read phi and write the sweep's scratch buffer
// (phi is left as it was), and the fastest is kept.  gs_tile_override >= 0
// pins a shape instead.
int gs_tile_choice(int n, const float* phi, const float* rhs, const float* coef, float dx2, float* scratch,
                   cudaStream_t s);

// nsweeps 8-colour Gauss-Seidel sweeps.  Grids of 64^3 and up run one fused
// launch per half sweep (all in-plane colours of every plane of one parity);
// smaller grids run one launch per colour.
// zero_init: phi holds no field yet and the sweeps start from zero (FP32
// grids of 64^3 and up run the first sweep in place without reading phi;
// elsewhere phi is zeroed first).
template <class T>
void launch_gs_sweeps(T* phi, const T* rhs, const T* coef, int n, T dx, int nsweeps, T* scratch, cudaStream_t s,
                      bool zero_init) {
  i64 h3 = (i64)(n / 2) * (n / 2) * (n / 2);
  T dx2 = dx * dx;
  int sw0 = 0;
  if (zero_init) {
    bool done = false;
    if constexpr (std::is_same<T, float>::value) {
      if (n >= 64 && nsweeps > 0) {
        const int v = gs_tile_choice(n, phi, rhs, coef, dx2, scratch, s);
        prof_begin(kk<T>(KK_GS), s, 4 * h3, n);
        gs_plane_half<T, 2>(v, phi, phi, phi, rhs, coef, n, dx2, 0, s);
        prof_end(kk<T>(KK_GS), s, n);
        prof_begin(kk<T>(KK_GS), s, 4 * h3, n);
        gs_plane_half<T, 1>(v, phi, phi, phi, rhs, coef, n, dx2, 1, s);
        prof_end(kk<T>(KK_GS), s, n);
        count_launch(2);
        sw0 = 1;
        done = true;
      }
    }
    if (!done) launch_fill<T>(phi, (i64)n * n * n, T(0), s);
  }
  if (n >= 64) {
    int v = 0;
    if constexpr (std::is_same<T, float>::value) {
      if (nsweeps > sw0) v = gs_tile_choice(n, phi, rhs, coef, dx2, scratch, s);
    }
    // double buffer: a sweep reads a and leaves the swept field in b
    T* a = phi;
    T* b = scratch;
    for (int sw = sw0; sw < nsweeps; ++sw) {
      for (int kpar = 0; kpar < 2; ++kpar) {
        prof_begin(kk<T>(KK_GS), s, 4 * h3, n);
        gs_plane_half<T>(v, a, kpar == 0 ? a : b, b, rhs, coef, n, dx2, kpar, s);
        prof_end(kk<T>(KK_GS), s, n);
        count_launch();
      }
      T* t = a;
      a = b;
      b = t;
    }
    if (a != phi) cudaMemcpyAsync(phi, a, sizeof(T) * (size_t)n * n * n, cudaMemcpyDeviceToDevice, s);
    return;
  }
  if (n <= 8) {
    if (nsweeps > 0) {
      prof_begin(kk<T>(KK_GS), s, h3 * 8 * nsweeps, n);
      // one thread per cell of a colour (8 at 4^3, 64 at 8^3), whole warps: the
      // colour phases' barriers then span one or two warps instead of 16
      const int nt = (int)std::max<i64>(32, (h3 + 31) / 32 * 32);
      k_gs_small_sm<T><<<1, nt, sizeof(T) * 8 * n * n * n, s>>>(phi, rhs, coef, n, dx2, nsweeps);
      prof_end(kk<T>(KK_GS), s, n);
      count_launch();
    }
    return;
  }
  if (n <= 16) {
    if (nsweeps > 0) {
      prof_begin(kk<T>(KK_GS), s, h3 * 8 * nsweeps, n);
      k_gs_small<T><<<1, 512, 0, s>>>(phi, rhs, coef, n, dx2, nsweeps);
      prof_end(kk<T>(KK_GS), s, n);
      count_launch();
    }
    return;
  }
  unsigned g = grid_of(h3, kBlock);
  for (int sw = 0; sw < nsweeps; ++sw)
    for (int kpar = 0; kpar < 2; ++kpar)
      for (int io = 0; io < 2; ++io)
        for (int jo = 0; jo < 2; ++jo) {
          prof_begin(kk<T>(KK_GS), s, h3, n);
          k_gs_colour<T><<<g, kBlock, 0, s>>>(phi, rhs, coef, n, dx2, kpar, io, jo);
          prof_end(kk<T>(KK_GS), s, n);
          count_launch();
        }
}

// The marching FP32 stencil (k_stencil_march) for grids of 64 and up, unless
// pinned to one plane per CTA (mmh_stencil_pin).
extern std::atomic<int> stencil_march_pin;
template <int MODE>
inline void launch_stencil_march(const float* phi, const float* rhs, const float* coef, int n, float di2, float* out,
                                 unsigned long long* maxbits, cudaStream_t s) {
  static std::atomic<unsigned long long> attr_done{0};
  const int smem = (int)(sizeof(float) * MarchGeom::WORDS);
  smem_attr_once(k_stencil_march<MODE>, smem, attr_done);
  k_stencil_march<MODE><<<dim3(n / MarchGeom::TX, n / MarchGeom::TY, n / kMarchKC), 256, smem, s>>>(
      phi, rhs, coef, n, di2, out, maxbits);
}
inline bool use_march(int n) { return n >= 64 && stencil_march_pin.load(std::memory_order_relaxed) != 0; }

template <class T>
void launch_residual(const T* phi, const T* rhs, const T* coef, int n, T dx, T* r, float* r32,
                     unsigned long long* maxbits, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  T di2 = T(1) / (dx * dx);
  prof_begin(kk<T>(KK_RESIDUAL), s, n3, n);
  bool done = false;
  if constexpr (std::is_same<T, float>::value) {
    if (use_march(n) && r32 == nullptr) {
      launch_stencil_march<0>(phi, rhs, coef, n, di2, r, maxbits, s);
      done = true;
    }
  }
  if (done) {
  } else if (n >= 32)
    k_stencil_plane<T, 0><<<dim3(n / 32, n / 16, n), 256, 0, s>>>(phi, rhs, coef, n, di2, r, r32, maxbits);
  else
    k_residual<T><<<grid_of(n3, kBlock), kBlock, 0, s>>>(phi, rhs, coef, n, di2, r, r32, maxbits);
  prof_end(kk<T>(KK_RESIDUAL), s, n);
  count_launch();
}

template <class T>
void launch_restrict_resid(const T* r, int n, int special, T* coarse, cudaStream_t s) {
  i64 h3 = (i64)(n / 2) * (n / 2) * (n / 2);
  prof_begin(kk<T>(KK_RESTRICT_RESID), s, h3, n);
  k_restrict_resid<T><<<grid_of(h3, kBlock), kBlock, 0, s>>>(r, n, special, coarse);
  prof_end(kk<T>(KK_RESTRICT_RESID), s, n);
  count_launch();
}

template <class T>
void launch_restrict27(const T* fine, int n, T* coarse, cudaStream_t s) {
  i64 h3 = (i64)(n / 2) * (n / 2) * (n / 2);
  prof_begin(kk<T>(KK_RESTRICT), s, h3, n);
  k_restrict27<T><<<grid_of(h3, kBlock), kBlock, 0, s>>>(fine, n, coarse);
  prof_end(kk<T>(KK_RESTRICT), s, n);
  count_launch();
}

template <class T>
void launch_smooth27(const T* in, int n, T* out, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  prof_begin(kk<T>(KK_SMOOTH), s, n3, n);
  k_smooth27<T><<<grid_of(n3, kBlock), kBlock, 0, s>>>(in, n, out);
  prof_end(kk<T>(KK_SMOOTH), s, n);
  count_launch();
}

template <class T>
void launch_prolong_add(T* u, const T* uh, int n, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  prof_begin(kk<T>(KK_PROLONG), s, n3, n);
  k_prolong_add_blk<T><<<grid_of((i64)(n / 2) * (n / 2) * (n / 2), kBlock), kBlock, 0, s>>>(u, uh, n);
  prof_end(kk<T>(KK_PROLONG), s, n);
  count_launch();
}

template <class T>
void launch_fxsum(const T* a, i64 count, unsigned long long* acc, int* flag, cudaStream_t s) {
  i64 blocks = (count + kBlock - 1) / kBlock;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_fxsum<T><<<(unsigned)blocks, kBlock, 0, s>>>(a, count, acc, flag);
  count_launch();
}

template <class T>
void launch_det(const T* def, int n, T dx, T* det, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  T di2 = T(1) / (dx * dx);
  k_det<T><<<grid_of(n3, kBlock), kBlock, 0, s>>>(def, n, di2, det);
  count_launch();
}

template <class T>
void launch_sub_mean(T* a, i64 count, const double* mean, cudaStream_t s) {
  k_sub_mean<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(a, count, mean);
  count_launch();
}

template <class T>
void launch_sub_dfact(T* a, const T* det, i64 count, const double* ratio, cudaStream_t s) {
  k_sub_dfact<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(a, det, count, ratio);
  count_launch();
}

template <class T>
void launch_fill(T* a, i64 count, T v, cudaStream_t s) {
  k_fill<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(a, count, v);
  count_launch();
}

template <class T>
__global__ void k_absmax(const T* __restrict__ a, i64 count, unsigned long long* maxbits) {
  decltype(abs_bits(T(0))) m = 0;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (i64)gridDim.x * blockDim.x) {
    auto v = abs_bits(a[t]);
    m = v > m ? v : m;
  }
  block_max_commit(from_bits(m), maxbits);
}

template <class T>
void launch_absmax(const T* a, i64 count, unsigned long long* maxbits, cudaStream_t s) {
  i64 blocks = (count + kBlock - 1) / kBlock;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_absmax<T><<<(unsigned)blocks, kBlock, 0, s>>>(a, count, maxbits);
  count_launch();
}

template <class T>
void launch_zero_if(T* a, i64 count, const int* flag, cudaStream_t s) {
  k_zero_if<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(a, count, flag);
  count_launch();
}

template <class T>
void launch_sub_mean_unless(T* a, i64 count, const double* mean, const int* flag, cudaStream_t s) {
  k_sub_mean_unless<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(a, count, mean, flag);
  count_launch();
}

template <class T>
__global__ void k_usum_flag(const unsigned long long* acc, int* flag) {
  T s = (T)fx_to(acc[0], acc[1]);
  *flag = (s > T(1.e-2)) ? 0 : 1;  // 0: run zerosum, 1: skip (flag semantics of k_sub_mean_unless)
}

template <class T>
void launch_usum_flag(const unsigned long long* acc, int* flag, cudaStream_t s) {
  k_usum_flag<T><<<1, 1, 0, s>>>(acc, flag);
  count_launch();
}

#define MMH_INSTANTIATE(T)                                                                                          \
  template void launch_metric<T>(const T*, const T*, int, T, T*, cudaStream_t, bool);                             \
  template void launch_gs_sweeps<T>(T*, const T*, const T*, int, T, int, T*, cudaStream_t, bool);                         \
  template void launch_residual<T>(const T*, const T*, const T*, int, T, T*, float*, unsigned long long*,          \
                                   cudaStream_t);                                                                   \
  template void launch_restrict_resid<T>(const T*, int, int, T*, cudaStream_t);                                   \
  template void launch_restrict27<T>(const T*, int, T*, cudaStream_t);                                            \
  template void launch_smooth27<T>(const T*, int, T*, cudaStream_t);                                              \
  template void launch_prolong_add<T>(T*, const T*, int, cudaStream_t);                                           \
  template void launch_fxsum<T>(const T*, i64, unsigned long long*, int*, cudaStream_t);                          \
  template void launch_det<T>(const T*, int, T, T*, cudaStream_t);                                                \
  template void launch_sub_mean<T>(T*, i64, const double*, cudaStream_t);                                         \
  template void launch_sub_dfact<T>(T*, const T*, i64, const double*, cudaStream_t);                              \
  template void launch_fill<T>(T*, i64, T, cudaStream_t);                                                         \
  template void launch_absmax<T>(const T*, i64, unsigned long long*, cudaStream_t);                               \
  template void launch_zero_if<T>(T*, i64, const int*, cudaStream_t);                                             \
  template void launch_sub_mean_unless<T>(T*, i64, const double*, const int*, cudaStream_t);                      \
  template void launch_usum_flag<T>(const unsigned long long*, int*, cudaStream_t);

}  // namespace mmh
