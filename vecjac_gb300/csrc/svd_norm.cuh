// The project's Euclidean column norm on one warp (in place of the BLAS xNRM2 that the
// reference's dnorm2_/znorm2_ call, src/dnorm2.c:12), with the bit helpers it shares with
// the SVD kernels. Device code that needs only vj_fp.cuh, threadIdx.x and the warp
// shuffles, so that a host harness can run it lane by lane.
#pragma once
#include "vj_fp.cuh"

namespace vj {

template <typename T> __device__ __forceinline__ T bitst(unsigned long long u)
{
  return fp<T>::val((typename fp<T>::U)u);
}
template <typename T> __device__ __forceinline__ unsigned long long absbits(T x)
{
  return (unsigned long long)(fp<T>::bits(x) & ~fp<T>::SIGN);
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v) ? w : v;
  }
  return v;
}

// The project's column norm (two-pass power-of-two scaling, 32 lanes, halving tree) for
// one warp; every lane returns the same value.
template <typename T> __device__ T warp_nrm2(const T *x, long long m)
{
  const int lane = threadIdx.x & 31;
  unsigned long long mx = 0ull;
  for (long long i = lane; i < m; i += 32) {
    const unsigned long long a = absbits(x[i]);
    mx = (a > mx) ? a : mx;
  }
  mx = warp_max_u64(mx);
  const T a = bitst<T>(mx);
  if (!visfinite(a))
    return visnan(a) ? fp<T>::qnan() : a;
  if (mx == 0ull)
    return (T)0;
  const int k = ilogb_(a);
  T acc = (T)0;
  for (long long i = lane; i < m; i += 32) {
    const T y = scale2(x[i], -k);
    acc = fp<T>::fma_(y, y, acc);
  }
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1)
    acc = acc + __shfl_down_sync(0xffffffffu, acc, w);
  acc = __shfl_sync(0xffffffffu, acc, 0);
  return scale2(fp<T>::sqrt_(acc), k);
}

}  // namespace vj
