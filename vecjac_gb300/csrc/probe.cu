// Peak arithmetic rate of the FMA pipes of the current GPU, measured: the denominator of
// the rooflines of the kernels that are bound by FP64 (the 2x2 EVD in FP64, the SVD's
// dot products) or FP32 arithmetic rather than by memory.
//
// Every thread runs 8 independent chains of fused multiply-adds (x <- x * a + b, with a
// and b chosen so that the values stay bounded), enough to cover the pipe latency; the
// grid fills every SM with 8 CTAs of 256 threads. The kernel is timed with CUDA events
// after a warm-up launch; the result is FMA operations (one per thread and instruction)
// per second. Nothing else runs on the stream meanwhile.
#include <cuda_runtime.h>

#include "vj_host.h"

namespace vj {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(int iters, T a, T b, T *out)
{
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c)
    x[c] = (T)(threadIdx.x + c) * (T)1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 8; ++c)
      x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c)
    s += x[c];
  // a store the compiler cannot drop (never taken for the launch's a and b)
  if (s == (T)-1.2345)
    out[blockIdx.x] = s;
}

template <typename T> static vj_fint fma_rate(double *ops_per_s, cudaStream_t s)
{
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const int blocks = host::sm_count() * 8, threads = 256;
  // FP64 runs ~60x slower than FP32 on this part: size each to a few milliseconds
  const int iters = (sizeof(T) == 8) ? 2048 : 65536;
  T *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  vj_fint r = VJ_ERR_CUDA;
  if (cudaMalloc(&out, (size_t)blocks * sizeof(T)) != cudaSuccess)
    return VJ_ERR_NOMEM;
  if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
    const T a = (T)0.999, b = (T)1e-3;
    k_fma_chains<T><<<blocks, threads, 0, s>>>(iters, a, b, out);
    float best = 0.f;
    bool ok = cudaGetLastError() == cudaSuccess;
    for (int rep = 0; ok && rep < 3; ++rep) {
      ok = cudaEventRecord(e0, s) == cudaSuccess;
      k_fma_chains<T><<<blocks, threads, 0, s>>>(iters, a, b, out);
      ok = ok && cudaGetLastError() == cudaSuccess && cudaEventRecord(e1, s) == cudaSuccess &&
           cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.f;
      ok = ok && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (ok && (best == 0.f || ms < best))
        best = ms;
    }
    if (ok && best > 0.f) {
      *ops_per_s = (double)blocks * threads * iters * 8.0 / (best * 1e-3);
      r = 0;
    }
  }
  if (e0)
    cudaEventDestroy(e0);
  if (e1)
    cudaEventDestroy(e1);
  cudaFree(out);
  return r;
}

}  // namespace vj

// fp64 != 0: DFMA; 0: FFMA. *ops_per_s receives thread-level FMA operations per second
// (2 flops each). Returns 0 or a VJ_ERR_* code.
extern "C" vj_fint vj_measure_fma_rate(int fp64, double *ops_per_s, void *stream)
{
  if (!ops_per_s)
    return VJ_ERR_ARG;
  return fp64 ? vj::fma_rate<double>(ops_per_s, (cudaStream_t)stream)
              : vj::fma_rate<float>(ops_per_s, (cudaStream_t)stream);
}
