// Interleaved <-> split-plane complex matrices: zsplit_/zmerge_ (FP64) and
// csplit_/cmerge_ (FP32), the conversions the reference's complex drivers run around
// zvjsvd_/cvjsvd_ (src/tzvjsvd.c:69,137,163): the SVD takes the real and imaginary parts
// as separate column-major planes, while files and most callers hold interleaved
// (re, im) pairs.
//
// Each thread moves one complex element per iteration (one 16-byte load or store of the
// interleaved pair for FP64, 8 bytes for FP32, and one element of each plane), over a
// grid that strides through the m x n elements column by column. The host-pointer forms
// stage column blocks through device memory on the library's two streams, so that the
// copies of one block overlap the kernel of the other.
#include <cfenv>
#include <cstdint>
#include <cuda_runtime.h>

#include "vj_host.h"

namespace vj {

template <typename T> struct cpx2;
template <> struct cpx2<double> { using V = double2; };
template <> struct cpx2<float> { using V = float2; };

// Ar(i, j) = Re A(i, j), Ai(i, j) = Im A(i, j)
template <typename T>
__global__ void __launch_bounds__(256) k_split(long long m, long long n, const typename cpx2<T>::V *__restrict__ A,
                                               long long ldA, T *__restrict__ Ar, long long ldAr, T *__restrict__ Ai,
                                               long long ldAi)
{
  const long long total = m * n;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long j = t / m, i = t - j * m;
    const typename cpx2<T>::V z = A[j * ldA + i];
    Ar[j * ldAr + i] = z.x;
    Ai[j * ldAi + i] = z.y;
  }
}

// A(i, j) = Ar(i, j) + i Ai(i, j)
template <typename T>
__global__ void __launch_bounds__(256) k_merge(long long m, long long n, const T *__restrict__ Ar, long long ldAr,
                                               const T *__restrict__ Ai, long long ldAi,
                                               typename cpx2<T>::V *__restrict__ A, long long ldA)
{
  const long long total = m * n;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long j = t / m, i = t - j * m;
    typename cpx2<T>::V z;
    z.x = Ar[j * ldAr + i];
    z.y = Ai[j * ldAi + i];
    A[j * ldA + i] = z;
  }
}

static unsigned grid_for(long long total)
{
  const long long cap = (long long)host::sm_count() * 8;
  long long g = (total + 255) / 256;
  if (g > cap)
    g = cap;
  return (unsigned)(g > 0 ? g : 1);
}

// The reference's argument checks (compiled in its debug builds, src/zsplit.c:6-27,
// src/zmerge.c:6-27), in its order: the rows in whole vectors (4 complex FP64 / 8 complex
// FP32 elements: -1), each leading dimension at least m and a multiple of the vector
// length (interleaved: that many complex elements; planes: 8 / 16 reals). Alignment is
// not needed by the GPU path; the device forms check the natural alignment of the
// element types instead, with the reference's codes for the array in question.
template <typename T>
static vj_fint check_args(long long m, long long ldA, long long ldP1, long long ldP2, bool merge)
{
  const long long cl = (sizeof(T) == 8) ? 4 : 8, pl = (sizeof(T) == 8) ? 8 : 16;
  if (m < 0 || (m % cl))
    return -1;
  if (merge) {
    if (ldP1 < m || (ldP1 % pl))
      return -4;
    if (ldP2 < m || (ldP2 % pl))
      return -6;
    if (ldA < m || (ldA % cl))
      return -8;
  }
  else {
    if (ldA < m || (ldA % cl))
      return -4;
    if (ldP1 < m || (ldP1 % pl))
      return -6;
    if (ldP2 < m || (ldP2 % pl))
      return -8;
  }
  return 0;
}

template <typename T>
static vj_fint split_dev(long long m, long long n, const T *A, long long ldA, T *Ar, long long ldAr, T *Ai,
                         long long ldAi, cudaStream_t s)
{
  const vj_fint r = check_args<T>(m, ldA, ldAr, ldAi, false);
  if (r)
    return r;
  if ((uintptr_t)A % (2 * sizeof(T)))
    return -3;
  if ((uintptr_t)Ar % sizeof(T))
    return -5;
  if ((uintptr_t)Ai % sizeof(T))
    return -7;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  if (n <= 0 || !m)
    return 1;
  k_split<T><<<grid_for(m * n), 256, 0, s>>>(m, n, reinterpret_cast<const typename cpx2<T>::V *>(A), ldA, Ar, ldAr,
                                              Ai, ldAi);
  return (cudaGetLastError() == cudaSuccess) ? 1 : VJ_ERR_CUDA;
}

template <typename T>
static vj_fint merge_dev(long long m, long long n, const T *Ar, long long ldAr, const T *Ai, long long ldAi, T *A,
                         long long ldA, cudaStream_t s)
{
  const vj_fint r = check_args<T>(m, ldA, ldAr, ldAi, true);
  if (r)
    return r;
  if ((uintptr_t)Ar % sizeof(T))
    return -3;
  if ((uintptr_t)Ai % sizeof(T))
    return -5;
  if ((uintptr_t)A % (2 * sizeof(T)))
    return -7;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  if (n <= 0 || !m)
    return 1;
  k_merge<T><<<grid_for(m * n), 256, 0, s>>>(m, n, Ar, ldAr, Ai, ldAi,
                                              reinterpret_cast<typename cpx2<T>::V *>(A), ldA);
  return (cudaGetLastError() == cudaSuccess) ? 1 : VJ_ERR_CUDA;
}

// Host-pointer forms: blocks of columns go through device buffers (about 256 MiB per
// block, two blocks in flight on the library's two streams). Synchronous, like the
// reference. The floating-point environment check comes first, as in the reference
// (IS_NOT_VFPENV, -9): the calling thread must round to nearest.
template <typename T>
static vj_fint convert_host(bool merge, long long m, long long n, const T *A_in, T *A_out, long long ldA,
                            const T *P1_in, T *P1_out, long long ld1, const T *P2_in, T *P2_out, long long ld2)
{
  if (fegetround() != FE_TONEAREST)
    return -9;
  const vj_fint r = check_args<T>(m, ldA, ld1, ld2, merge);
  if (r)
    return r;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  if (n <= 0 || !m)
    return 1;
  std::lock_guard<std::recursive_mutex> lk(host::host_call_lock());  // the device's staging buffers
  const size_t colb = (size_t)m * 4 * sizeof(T);  // one column: interleaved + two planes
  long long cols = (long long)(((size_t)256 << 20) / colb);
  if (cols < 1)
    cols = 1;
  if (cols > n)
    cols = n;
  const size_t plane = (size_t)m * cols * sizeof(T);
  const size_t slot = (4 * plane + 255u) & ~(size_t)255u;
  host::Staging &stg = host::staging();
  if (!stg.reserve(2 * slot))
    return VJ_ERR_NOMEM;
  cudaStream_t st[2];
  if (!host::streams2(st))
    return VJ_ERR_CUDA;
  const size_t esz = sizeof(T);
  for (long long j0 = 0, it = 0; j0 < n; j0 += cols, ++it) {
    const long long nc = (n - j0 < cols) ? (n - j0) : cols;
    const int b = (int)(it & 1);
    cudaStream_t s = st[b];
    T *dA = reinterpret_cast<T *>(stg.ptr + (size_t)b * slot);  // m x nc interleaved (2 m T per column)
    T *d1 = dA + 2 * (size_t)m * cols, *d2 = d1 + (size_t)m * cols;
    vj_fint kr;
    if (!merge) {
      if (cudaMemcpy2DAsync(dA, (size_t)m * 2 * esz, A_in + 2 * (size_t)j0 * ldA, (size_t)ldA * 2 * esz,
                            (size_t)m * 2 * esz, (size_t)nc, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      kr = split_dev<T>(m, nc, dA, m, d1, m, d2, m, s);
      if (kr < 0)
        return kr;
      if (cudaMemcpy2DAsync(P1_out + (size_t)j0 * ld1, (size_t)ld1 * esz, d1, (size_t)m * esz, (size_t)m * esz,
                            (size_t)nc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaMemcpy2DAsync(P2_out + (size_t)j0 * ld2, (size_t)ld2 * esz, d2, (size_t)m * esz, (size_t)m * esz,
                            (size_t)nc, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return VJ_ERR_CUDA;
    }
    else {
      if (cudaMemcpy2DAsync(d1, (size_t)m * esz, P1_in + (size_t)j0 * ld1, (size_t)ld1 * esz, (size_t)m * esz,
                            (size_t)nc, cudaMemcpyHostToDevice, s) != cudaSuccess ||
          cudaMemcpy2DAsync(d2, (size_t)m * esz, P2_in + (size_t)j0 * ld2, (size_t)ld2 * esz, (size_t)m * esz,
                            (size_t)nc, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      kr = merge_dev<T>(m, nc, d1, m, d2, m, dA, m, s);
      if (kr < 0)
        return kr;
      if (cudaMemcpy2DAsync(A_out + 2 * (size_t)j0 * ldA, (size_t)ldA * 2 * esz, dA, (size_t)m * 2 * esz,
                            (size_t)m * 2 * esz, (size_t)nc, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return VJ_ERR_CUDA;
    }
  }
  if (cudaStreamSynchronize(st[0]) != cudaSuccess || cudaStreamSynchronize(st[1]) != cudaSuccess)
    return VJ_ERR_CUDA;
  return 1;
}

}  // namespace vj

using namespace vj;

extern "C" {

vj_fint zsplit_(const vj_fnat m[1], const vj_fnat n[1], const double A[], const vj_fnat ldA[1], double Ar[],
                const vj_fnat ldAr[1], double Ai[], const vj_fnat ldAi[1])
{
  return convert_host<double>(false, (long long)*m, (long long)*n, A, nullptr, (long long)*ldA, nullptr, Ar,
                              (long long)*ldAr, nullptr, Ai, (long long)*ldAi);
}

vj_fint zmerge_(const vj_fnat m[1], const vj_fnat n[1], const double Ar[], const vj_fnat ldAr[1], const double Ai[],
                const vj_fnat ldAi[1], double A[], const vj_fnat ldA[1])
{
  return convert_host<double>(true, (long long)*m, (long long)*n, nullptr, A, (long long)*ldA, Ar, nullptr,
                              (long long)*ldAr, Ai, nullptr, (long long)*ldAi);
}

vj_fint csplit_(const vj_fnat m[1], const vj_fnat n[1], const float A[], const vj_fnat ldA[1], float Ar[],
                const vj_fnat ldAr[1], float Ai[], const vj_fnat ldAi[1])
{
  return convert_host<float>(false, (long long)*m, (long long)*n, A, nullptr, (long long)*ldA, nullptr, Ar,
                             (long long)*ldAr, nullptr, Ai, (long long)*ldAi);
}

vj_fint cmerge_(const vj_fnat m[1], const vj_fnat n[1], const float Ar[], const vj_fnat ldAr[1], const float Ai[],
                const vj_fnat ldAi[1], float A[], const vj_fnat ldA[1])
{
  return convert_host<float>(true, (long long)*m, (long long)*n, nullptr, A, (long long)*ldA, Ar, nullptr,
                             (long long)*ldAr, Ai, nullptr, (long long)*ldAi);
}

vj_fint vj_zsplit_dev(vj_fnat m, vj_fnat n, const double *A, vj_fnat ldA, double *Ar, vj_fnat ldAr, double *Ai,
                      vj_fnat ldAi, void *stream)
{
  return split_dev<double>((long long)m, (long long)n, A, (long long)ldA, Ar, (long long)ldAr, Ai, (long long)ldAi,
                           (cudaStream_t)stream);
}

vj_fint vj_zmerge_dev(vj_fnat m, vj_fnat n, const double *Ar, vj_fnat ldAr, const double *Ai, vj_fnat ldAi,
                      double *A, vj_fnat ldA, void *stream)
{
  return merge_dev<double>((long long)m, (long long)n, Ar, (long long)ldAr, Ai, (long long)ldAi, A, (long long)ldA,
                           (cudaStream_t)stream);
}

vj_fint vj_csplit_dev(vj_fnat m, vj_fnat n, const float *A, vj_fnat ldA, float *Ar, vj_fnat ldAr, float *Ai,
                      vj_fnat ldAi, void *stream)
{
  return split_dev<float>((long long)m, (long long)n, A, (long long)ldA, Ar, (long long)ldAr, Ai, (long long)ldAi,
                          (cudaStream_t)stream);
}

vj_fint vj_cmerge_dev(vj_fnat m, vj_fnat n, const float *Ar, vj_fnat ldAr, const float *Ai, vj_fnat ldAi, float *A,
                      vj_fnat ldA, void *stream)
{
  return merge_dev<float>((long long)m, (long long)n, Ar, (long long)ldAr, Ai, (long long)ldAi, A, (long long)ldA,
                          (cudaStream_t)stream);
}

}  // extern "C"
