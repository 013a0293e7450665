// Host-side services shared by the entry points: device discovery, a growable device
// staging buffer for the host-pointer forms, and a pair of library-owned streams.
#pragma once
#include <mutex>
#include <cfenv>
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/vecjac_gb300.h"

namespace vj {
namespace host {

// Round-to-nearest for the host-side arithmetic of one call (tolerances, rescaling
// bounds), whatever rounding mode the caller's thread has; the caller's mode is restored.
struct NearestRounding {
  int saved;
  NearestRounding() : saved(fegetround())
  {
    if (saved != FE_TONEAREST)
      fesetround(FE_TONEAREST);
  }
  ~NearestRounding()
  {
    if (saved != FE_TONEAREST)
      fesetround(saved);
  }
  NearestRounding(const NearestRounding &) = delete;
  NearestRounding &operator=(const NearestRounding &) = delete;
};

// true when a CUDA device is usable (checked once; the current device is used)
bool gpu_ready();
// Library state is kept per device (the current device of each call): SM count, staging
// buffers, streams, the batch queue, the cuBLAS / cuSOLVER handles of the mixed SVD.
constexpr int MAX_DEVICES = 64;
int device_slot();
int sm_count();
// the device can read and write pageable host memory (and VJ_STAGED is not set)
bool pageable_access();
// p (NULL counts as true) is page-locked host memory (cudaHostAlloc / cudaHostRegister)
bool host_pinned(const void *p);

// device memory reused across host-API calls; grows on demand, never shrinks
struct Staging {
  char *ptr = nullptr;
  size_t size = 0;
  bool reserve(size_t bytes);
};
Staging &staging();
Staging &staging2();
// scratch of the mixed-precision SVD (its inner SVD calls use staging2)
Staging &staging3();

// the work-queue counter of the batched SVD (device memory, allocated on first use)
unsigned *batch_queue();

// two non-blocking streams owned by the library
bool streams2(cudaStream_t s[2]);

// Taken by the host-pointer entry points (dbjac2_ ... zsplit_ ...), which share the
// device's staging buffers: calls from several host threads run one at a time on a device,
// so those entry points are reentrant like the reference's. (Recursive: a host form may
// call another.)
std::recursive_mutex &host_call_lock();

// launch with programmatic stream serialisation (the kernel calls pdl_enter first)
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// per-sweep statistics of the last SVD (transformed pairs per sweep)
void trace_reset();
void trace_sweep(unsigned sweep, unsigned long long rotations);
// per-phase cycle counts (VJ_TRACE=1 in the environment enables their collection)
bool trace_enabled();
void trace_phases(const unsigned long long *cycles, int count);

// phase times (ms) of the last mixed-precision SVD, its number of FP32 launches and whether
// its FP32 stages ran as block sweeps on the tensor cores (1) or column-pair sweeps (0)
void mixed_phases_set(double fp32, double gemm, double fp64, double fin, double fp32_steps, double block);

// elements per chunk of a host-pointer 2x2 call (a multiple of `lanes`)
long long bjac2_chunk(long long n, size_t elem, bool cplx, int lanes);

}  // namespace host
}  // namespace vj
