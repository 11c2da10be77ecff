// Allocation-free relax() on caller-owned device memory.
//
// Some callers cannot let a library allocate device memory: a driver that
// hands out every buffer from its own pool, or one that must not allocate
// inside a time-critical loop.  mmh_relax_noalloc_f64 serves them: the
// caller passes inputs and outputs in device memory, and the scratch the
// smoother needs (6 metric planes, the sweep double buffer and one reduction
// word) lives in the fixed array below, which every GPU that loads this
// library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mmh.h"
#include "mmh_internal.h"

using namespace mmh;

namespace {

constexpr int kMaxN = MMH_NOALLOC_MAX_N;
constexpr long long kMaxN3 = (long long)kMaxN * kMaxN * kMaxN;
// 6 metric planes + 1 sweep buffer of n^3 doubles, then one 8-byte reduction word
constexpr long long kScratchWords = 7 * kMaxN3 + 2;

static __device__ __align__(256) double g_scratch[kScratchWords];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
double* g_scratch_dev[kMaxDevices] = {nullptr};  // device address of g_scratch, per device

// Device address of the scratch array on the current device, looked up once
// per device with that device current (the host-side name of the array is not
// a device address).
int scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MMH_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess) return MMH_ERR_CUDA;
    g_scratch_dev[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_dev[dev];
  return MMH_OK;
}

}  // namespace

extern "C" int mmh_relax_noalloc_f64(const double* d_deformpot, const double* d_rho, double* d_arr,
                                     const double* d_rhs, double dx, int n, int nrelax, int iopt, double* rinf,
                                     void* stream) {
  if (!d_deformpot || !d_rho || !d_arr || !d_rhs) return MMH_ERR_ARG;
  if (n <= 0 || (n & (n - 1)) != 0) return MMH_ERR_NOTPOW2;
  if (n < 4) return MMH_ERR_SIZE;
  if (n > kMaxN) return MMH_ERR_TOO_LARGE;
  int ir = iopt % 8;
  // the same iresidopt bounds as mmh_relax_f64 (modes 1 and 3 need a resid
  // array this entry point does not take)
  if (iopt < 0 || iopt > 256 || (iopt / 8) % 8 != 2 || (ir != 0 && ir != 2) || nrelax < 0) return MMH_ERR_ARG;
  if (ir == 2 && !rinf) return MMH_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // an error left pending by earlier, unrelated work is not this call's
  cudaGetLastError();
  double* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != MMH_OK) return rc;
  const i64 n3 = (i64)n * n * n;
  double* coef = scratch;                 // 6 n^3: rho_bar * cof(A)/det
  double* buf = scratch + 6 * n3;         // n^3: Gauss-Seidel double buffer
  unsigned long long* maxw = reinterpret_cast<unsigned long long*>(scratch + 7 * kMaxN3);
  launch_metric<double>(d_deformpot, d_rho, n, dx, coef, s);
  launch_gs_sweeps<double>(d_arr, d_rhs, coef, n, dx, nrelax, buf, s);
  if (cudaGetLastError() != cudaSuccess) return MMH_ERR_CUDA;
  double v = 0.0;
  if (ir == 2) {
    // the word keeps the previous call's maximum: clear it first
    if (cudaMemsetAsync(maxw, 0, sizeof(unsigned long long), s) != cudaSuccess) return MMH_ERR_CUDA;
    launch_residual<double>(d_arr, d_rhs, coef, n, dx, nullptr, nullptr, maxw, s);
    if (cudaGetLastError() != cudaSuccess) return MMH_ERR_CUDA;
    unsigned long long bits = 0;
    if (cudaMemcpyAsync(&bits, maxw, sizeof(bits), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MMH_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MMH_ERR_CUDA;
    static_assert(sizeof(v) == sizeof(bits), "word size");
    memcpy(&v, &bits, sizeof(v));
  } else {
    if (cudaStreamSynchronize(s) != cudaSuccess) return MMH_ERR_CUDA;
  }
  if (rinf) *rinf = v;
  return MMH_OK;
}
