// Flexible preconditioned conjugate gradients: operator application, exact
// dot products and vector updates, templated on the vector precision.  Dot
// products are exact and order free: each product a_i*b_i (formed in FP64,
// exact for FP32 vectors) is scaled by 2^(96-E), 2^E > max|a|*max|b|,
// truncated to a 128-bit integer and summed with two 64-bit atomics.
#pragma once
#include "mmh_launch.cuh"

namespace mmh {

__device__ __forceinline__ double bits_d(const unsigned long long* b) { return __longlong_as_double((long long)*b); }

// q = L[p] = (t1 + t2 + tdiag*p) * di2, max|q| into qbits
template <class T>
__global__ void k_apply(const T* __restrict__ p, const T* __restrict__ coef, int n, T di2, T* __restrict__ q,
                        unsigned long long* qbits) {
  i64 n3 = (i64)n * n * n;
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  T m = T(0);
  if (t < n3) {
    int i, j, k;
    cell_of(t, n, i, j, k);
    T tdiag, t1, t2;
    op_terms(p, coef, n, n3, i, j, k, tdiag, t1, t2);
    T v = (t1 + t2 + tdiag * p[t]) * di2;
    q[t] = v;
    m = fabs(v);
  }
  block_max_commit(m, qbits);
}

// trunc(a*b * 2^sh) for FP32 a, b from their bits: the product of the 24-bit
// significands is exact in 64 bits, so this equals fx_bits of the (exact)
// FP64 product without any FP64 operation.
__device__ __forceinline__ __int128 fx_prod(float a, float b, int sh) {
  unsigned ua = __float_as_uint(a), ub = __float_as_uint(b);
  int ea = (int)((ua >> 23) & 0xFF), eb = (int)((ub >> 23) & 0xFF);
  unsigned ma = ua & 0x7FFFFFu, mb = ub & 0x7FFFFFu;
  if (ea) ma |= 0x800000u; else ea = 1;
  if (eb) mb |= 0x800000u; else eb = 1;
  unsigned long long m = (unsigned long long)ma * mb;
  int s = ea + eb - 300 + sh;
  unsigned __int128 v;
  if (s >= 0) v = (unsigned __int128)m << s;
  else if (s > -64) v = (unsigned __int128)(m >> (-s));
  else v = 0;
  return ((ua ^ ub) >> 31) ? -(__int128)v : (__int128)v;
}
__device__ __forceinline__ __int128 fx_prod(double a, double b, int sh) { return fx_bits(a * b, sh); }

template <class T>
__global__ void k_dot(const T* __restrict__ a, const T* __restrict__ b, i64 count, const unsigned long long* abits,
                      const unsigned long long* bbits, unsigned long long* acc) {
  double ma = bits_d(abits), mb = bits_d(bbits);
  __int128 s = 0;
  if (ma > 0.0 && mb > 0.0) {
    int E = ilogb(ma) + ilogb(mb) + 2;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (i64)gridDim.x * blockDim.x)
      s += fx_prod(a[t], b[t], 96 - E);
  }
  fx_block_commit(s, acc);
}

// x = x + alpha*p ; r = r - alpha*q ; max|r|
template <class T>
__global__ void k_pcg_update(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ q,
                             i64 count, const double* __restrict__ alpha, unsigned long long* rbits) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  T a = (T)*alpha;
  T m = T(0);
  if (t < count) {
    x[t] = x[t] + a * p[t];
    T v = r[t] - a * q[t];
    r[t] = v;
    m = fabs(v);
  }
  block_max_commit(m, rbits);
}

// p = z + beta*p ; max|p|
template <class T>
__global__ void k_pcg_pupdate(T* __restrict__ p, const T* __restrict__ z, i64 count, const double* __restrict__ beta,
                              unsigned long long* pbits) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  T b = (T)*beta;
  T m = T(0);
  if (t < count) {
    T v = z[t] + b * p[t];
    p[t] = v;
    m = fabs(v);
  }
  block_max_commit(m, pbits);
}

template <class T>
void launch_apply(const T* p, const T* coef, int n, T dx, T* q, unsigned long long* qbits, cudaStream_t s) {
  i64 n3 = (i64)n * n * n;
  prof_begin(kk<T>(KK_APPLY), s, n3, n);
  bool done = false;
  if constexpr (std::is_same<T, float>::value) {
    if (use_march(n)) {
      launch_stencil_march<1>(p, nullptr, coef, n, T(1) / (dx * dx), q, qbits, s);
      done = true;
    }
  }
  if (done) {
  } else if (n >= 32)
    k_stencil_plane<T, 1><<<dim3(n / 32, n / 16, n), 256, 0, s>>>(p, nullptr, coef, n, T(1) / (dx * dx), q, nullptr,
                                                                 qbits);
  else
    k_apply<T><<<grid_of(n3, kBlock), kBlock, 0, s>>>(p, coef, n, T(1) / (dx * dx), q, qbits);
  prof_end(kk<T>(KK_APPLY), s, n);
  count_launch();
}

template <class T>
void launch_dot(const T* a, const T* b, i64 count, const unsigned long long* abits, const unsigned long long* bbits,
                unsigned long long* acc, cudaStream_t s) {
  i64 blocks = (count + kBlock - 1) / kBlock;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_dot<T><<<(unsigned)blocks, kBlock, 0, s>>>(a, b, count, abits, bbits, acc);
  count_launch();
}

template <class T>
void launch_pcg_update(T* x, T* r, const T* p, const T* q, i64 count, const double* alpha, unsigned long long* rbits,
                       cudaStream_t s) {
  k_pcg_update<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(x, r, p, q, count, alpha, rbits);
  count_launch();
}

template <class T>
void launch_pcg_pupdate(T* p, const T* z, i64 count, const double* beta, unsigned long long* pbits, cudaStream_t s) {
  k_pcg_pupdate<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(p, z, count, beta, pbits);
  count_launch();
}

#define MMH_INSTANTIATE_PCG(T)                                                                                   \
  template void launch_apply<T>(const T*, const T*, int, T, T*, unsigned long long*, cudaStream_t);             \
  template void launch_dot<T>(const T*, const T*, i64, const unsigned long long*, const unsigned long long*,     \
                              unsigned long long*, cudaStream_t);                                                \
  template void launch_pcg_update<T>(T*, T*, const T*, const T*, i64, const double*, unsigned long long*,        \
                                     cudaStream_t);                                                              \
  template void launch_pcg_pupdate<T>(T*, const T*, i64, const double*, unsigned long long*, cudaStream_t);

}  // namespace mmh
