// Parallel pivot-pair tables (pjs, src/pjs.c:9-67), generated on the GPU.
//
// VecJac obtains its tables from libpvn's pvn_cjs_init/next (src/pjs.c:3-5,28,37), which
// is not part of the reference checkout and has no pinned version; its exact tables
// therefore cannot be reproduced here. The tables below have the same shape and pair
// contract (row s holds n/2 disjoint pairs covering 0..n-1, p < q inside a pair, every
// pair appears once per sweep) and follow published parallel orderings:
//   id 2 (PJS_ME, n-1 steps): the round-robin ("circle") ordering of Brent and Luk (1985):
//        step s pairs s with n-1 and (s+k) mod (n-1) with (s-k) mod (n-1), k = 1..n/2-1;
//   id 4 (PJS_MM, n steps): the modulus ordering of Luk and Park (1989): step s pairs i
//        with (s-i) mod n; the two indices with 2i = s (mod n) of an even step are paired
//        with each other.
// One thread writes one pair; the table for n = 4096 (16 MiB at n-1 steps) takes one
// launch.
#include <cstdlib>

#include <cuda_runtime.h>

#include "pjs.cuh"
#include "vj_host.h"

namespace vj {

__global__ void k_pjs_rr(unsigned n, unsigned stp, unsigned *t)
{
  const unsigned half = n >> 1;
  const unsigned long long tot = (unsigned long long)stp * half;
  for (unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; w < tot;
       w += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned s = (unsigned)(w / half), k = (unsigned)(w % half);
    unsigned *r = t + (size_t)s * n + 2u * k;
    pair_rr(n, s, k, r[0], r[1]);
  }
}

__global__ void k_pjs_mod(unsigned n, unsigned stp, unsigned *t)
{
  const unsigned half = n >> 1;
  const unsigned long long tot = (unsigned long long)stp * half;
  for (unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; w < tot;
       w += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned s = (unsigned)(w / half), k = (unsigned)(w % half);
    unsigned *r = t + (size_t)s * n + 2u * k;
    pair_mod(n, s, k, r[0], r[1]);
  }
}

static vj_fint pjs_launch(long id, unsigned n, unsigned *table, cudaStream_t s)
{
  if (n <= 1u || (n & 1u))
    return -1;
  unsigned stp;
  if (id == 2l)
    stp = n - 1u;
  else if (id == 4l)
    stp = n;
  else
    return -1;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const unsigned long long tot = (unsigned long long)stp * (n >> 1);
  unsigned long long blocks = (tot + 255) / 256;
  const unsigned long long cap = (unsigned long long)host::sm_count() * 16ull;
  if (blocks > cap)
    blocks = cap;
  if (id == 2l)
    k_pjs_rr<<<(unsigned)blocks, 256, 0, s>>>(n, stp, table);
  else
    k_pjs_mod<<<(unsigned)blocks, 256, 0, s>>>(n, stp, table);
  return (cudaGetLastError() == cudaSuccess) ? (vj_fint)stp : VJ_ERR_CUDA;
}

}  // namespace vj

extern "C" {

vj_fint vj_pjs_dev(long id, unsigned n, unsigned *table, void *stream)
{
  return vj::pjs_launch(id, n, table, (cudaStream_t)stream);
}

unsigned *pjs(long id, unsigned n, unsigned stp[1])
{
  *stp = 0u;
  if (n <= 1u || (n & 1u) || (id != 2l && id != 4l))
    return nullptr;
  const unsigned st = (id == 2l) ? (n - 1u) : n;
  const size_t bytes = (size_t)st * n * sizeof(unsigned);
  unsigned *h = (unsigned *)malloc(bytes);
  if (!h)
    return nullptr;
  unsigned *d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    cudaGetLastError();
    free(h);
    return nullptr;
  }
  const vj_fint r = vj::pjs_launch(id, n, d, nullptr);
  const bool ok = (r > 0) && (cudaMemcpy(h, d, bytes, cudaMemcpyDeviceToHost) == cudaSuccess);
  cudaFree(d);
  if (!ok) {
    free(h);
    return nullptr;
  }
  *stp = st;
  return h;
}

}  // extern "C"
