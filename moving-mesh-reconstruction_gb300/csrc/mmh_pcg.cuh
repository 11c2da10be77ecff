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

// The FP32 updates of the mixed form's inner solve over whole vectors of four:
// a fixed grid of at most 8 blocks per SM walks the vectors with 16-byte
// loads and commits one maximum per block (the elementwise results and the
// maximum are those of k_pcg_update / k_pcg_pupdate).  count % 4 == 0.
static __global__ void __launch_bounds__(256) k_pcg_update_v4(float4* __restrict__ x, float4* __restrict__ r,
                                                       const float4* __restrict__ p, const float4* __restrict__ q,
                                                       i64 count4, const double* __restrict__ alpha,
                                                       unsigned long long* rbits) {
  const float a = (float)*alpha;
  unsigned m = 0;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < count4; t += (i64)gridDim.x * blockDim.x) {
    float4 xv = x[t], rv = r[t];
    const float4 pv = p[t], qv = q[t];
    xv.x = xv.x + a * pv.x; xv.y = xv.y + a * pv.y; xv.z = xv.z + a * pv.z; xv.w = xv.w + a * pv.w;
    rv.x = rv.x - a * qv.x; rv.y = rv.y - a * qv.y; rv.z = rv.z - a * qv.z; rv.w = rv.w - a * qv.w;
    x[t] = xv;
    r[t] = rv;
    const unsigned b0 = __float_as_uint(fabsf(rv.x)), b1 = __float_as_uint(fabsf(rv.y));
    const unsigned b2 = __float_as_uint(fabsf(rv.z)), b3 = __float_as_uint(fabsf(rv.w));
    m = max(m, max(max(b0, b1), max(b2, b3)));
  }
  block_max_commit(__uint_as_float(m), rbits);
}
static __global__ void __launch_bounds__(256) k_pcg_pupdate_v4(float4* __restrict__ p, const float4* __restrict__ z,
                                                        i64 count4, const double* __restrict__ beta,
                                                        unsigned long long* pbits) {
  const float b = (float)*beta;
  unsigned m = 0;
  for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < count4; t += (i64)gridDim.x * blockDim.x) {
    float4 pv = p[t];
    const float4 zv = z[t];
    pv.x = zv.x + b * pv.x; pv.y = zv.y + b * pv.y; pv.z = zv.z + b * pv.z; pv.w = zv.w + b * pv.w;
    p[t] = pv;
    const unsigned b0 = __float_as_uint(fabsf(pv.x)), b1 = __float_as_uint(fabsf(pv.y));
    const unsigned b2 = __float_as_uint(fabsf(pv.z)), b3 = __float_as_uint(fabsf(pv.w));
    m = max(m, max(max(b0, b1), max(b2, b3)));
  }
  block_max_commit(__uint_as_float(m), pbits);
}

inline unsigned vec_blocks(i64 count4) {
  i64 b = (count4 + kBlock - 1) / kBlock;
  const i64 cap = 152 * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <class T>
void launch_pcg_update(T* x, T* r, const T* p, const T* q, i64 count, const double* alpha, unsigned long long* rbits,
                       cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    if (count % 4 == 0) {
      k_pcg_update_v4<<<vec_blocks(count / 4), kBlock, 0, s>>>(
          reinterpret_cast<float4*>(x), reinterpret_cast<float4*>(r), reinterpret_cast<const float4*>(p),
          reinterpret_cast<const float4*>(q), count / 4, alpha, rbits);
      count_launch();
      return;
    }
  }
  k_pcg_update<T><<<grid_of(count, kBlock), kBlock, 0, s>>>(x, r, p, q, count, alpha, rbits);
  count_launch();
}

template <class T>
void launch_pcg_pupdate(T* p, const T* z, i64 count, const double* beta, unsigned long long* pbits, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    if (count % 4 == 0) {
      k_pcg_pupdate_v4<<<vec_blocks(count / 4), kBlock, 0, s>>>(
          reinterpret_cast<float4*>(p), reinterpret_cast<const float4*>(z), count / 4, beta, pbits);
      count_launch();
      return;
    }
  }
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
