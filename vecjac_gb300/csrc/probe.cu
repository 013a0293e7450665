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

// CH independent chains per thread; the lanes at or above `lanes` of every warp exit first
template <typename T, int CH>
__global__ void __launch_bounds__(256) k_fma_chains(int iters, int lanes, T a, T b, T *out)
{
  if ((int)(threadIdx.x & 31) >= lanes)
    return;
  T x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c)
    x[c] = (T)(threadIdx.x + c) * (T)1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c)
      x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c)
    s += x[c];
  // a store the compiler cannot drop (never taken for the launch's a and b)
  if (s == (T)-1.2345)
    out[blockIdx.x] = s;
}

// warps_per_sm warps on every SM (CTAs of up to 8 warps), `lanes` active lanes per warp,
// `chains` (8 or 1) FMA chains per lane: *ops_per_s = active-lane FMAs per second
template <typename T>
static vj_fint fma_rate(int warps_per_sm, int lanes, int chains, double *ops_per_s, cudaStream_t s)
{
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  if (warps_per_sm < 1 || warps_per_sm > 64 || (warps_per_sm > 8 && (warps_per_sm % 8)) || lanes < 1 || lanes > 32 ||
      (chains != 1 && chains != 8))
    return VJ_ERR_ARG;
  const int wpc = (warps_per_sm < 8) ? warps_per_sm : 8;
  const int blocks = host::sm_count() * (warps_per_sm / wpc), threads = 32 * wpc;
  // FP64 runs ~60x slower than FP32 on this part: size each to a few milliseconds
  const int iters = (sizeof(T) == 8) ? 2048 : 65536;
  T *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  vj_fint r = VJ_ERR_CUDA;
  if (cudaMalloc(&out, (size_t)blocks * sizeof(T)) != cudaSuccess)
    return VJ_ERR_NOMEM;
  if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
    const T a = (T)0.999, b = (T)1e-3;
    auto launch = [&]() {
      if (chains == 8)
        k_fma_chains<T, 8><<<blocks, threads, 0, s>>>(iters, lanes, a, b, out);
      else
        k_fma_chains<T, 1><<<blocks, threads, 0, s>>>(iters, lanes, a, b, out);
    };
    launch();
    float best = 0.f;
    bool ok = cudaGetLastError() == cudaSuccess;
    for (int rep = 0; ok && rep < 3; ++rep) {
      ok = cudaEventRecord(e0, s) == cudaSuccess;
      launch();
      ok = ok && cudaGetLastError() == cudaSuccess && cudaEventRecord(e1, s) == cudaSuccess &&
           cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.f;
      ok = ok && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (ok && (best == 0.f || ms < best))
        best = ms;
    }
    if (ok && best > 0.f) {
      *ops_per_s = (double)blocks * (threads / 32) * lanes * (double)iters * chains / (best * 1e-3);
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
// (2 flops each), with 64 warps of 8 chains on every SM. Returns 0 or a VJ_ERR_* code.
extern "C" vj_fint vj_measure_fma_rate(int fp64, double *ops_per_s, void *stream)
{
  if (!ops_per_s)
    return VJ_ERR_ARG;
  return fp64 ? vj::fma_rate<double>(64, 32, 8, ops_per_s, (cudaStream_t)stream)
              : vj::fma_rate<float>(64, 32, 8, ops_per_s, (cudaStream_t)stream);
}

// The same probe with warps_per_sm warps on every SM, `lanes` active lanes per warp and
// `chains` (8: independent, 1: one dependent chain per lane): the FMA pipe's throughput per
// warp instruction and per active lane, and its dependent latency
// (chains = 1: cycles per FMA = clock / (ops_per_s / (SMs x warps_per_sm x lanes))).
extern "C" vj_fint vj_measure_fma_shape(int fp64, int warps_per_sm, int lanes, int chains, double *ops_per_s,
                                        void *stream)
{
  if (!ops_per_s)
    return VJ_ERR_ARG;
  return fp64 ? vj::fma_rate<double>(warps_per_sm, lanes, chains, ops_per_s, (cudaStream_t)stream)
              : vj::fma_rate<float>(warps_per_sm, lanes, chains, ops_per_s, (cudaStream_t)stream);
}
