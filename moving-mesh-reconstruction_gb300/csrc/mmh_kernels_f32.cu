// FP32 kernels of the mixed-precision inner V-cycle (smoother, residual,
// restriction, prolongation, zero-mean).  FMA contraction stays enabled here.
#include "mmh_launch.cuh"
#include "mmh_pcg.cuh"

namespace mmh {
MMH_INSTANTIATE(float)
MMH_INSTANTIATE_PCG(float)

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
