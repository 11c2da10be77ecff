// FP32 kernels of the mixed-precision inner V-cycle (smoother, residual,
// restriction, prolongation, zero-mean).  FMA contraction stays enabled here.
#include "mmh_launch.cuh"
#include "mmh_pcg.cuh"

namespace mmh {
MMH_INSTANTIATE(float)
MMH_INSTANTIATE_PCG(float)
}  // namespace mmh
