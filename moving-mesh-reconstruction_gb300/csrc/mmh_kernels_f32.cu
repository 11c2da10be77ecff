// FP32 kernels of the mixed-precision inner V-cycle (smoother, residual,
// restriction, prolongation, zero-mean).  FMA contraction stays enabled here.
#include "mmh_launch.cuh"

namespace mmh {
MMH_INSTANTIATE(float)
}  // namespace mmh
