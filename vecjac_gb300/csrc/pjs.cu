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

#include "vj_host.h"

namespace vj {

__global__ void k_pjs_rr(unsigned n, unsigned stp, unsigned *t)
{
  const unsigned half = n >> 1;
  const unsigned long long tot = (unsigned long long)stp * half;
  for (unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; w < tot;
       w += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned s = (unsigned)(w / half), k = (unsigned)(w % half);
    const unsigned N = n - 1u;
    unsigned a, b;
    if (!k) {
      a = s;
      b = N;
    }
    else {
      a = (s + k) % N;
      b = (s + N - k) % N;
    }
    unsigned *r = t + (size_t)s * n + 2u * k;
    r[0] = (a < b) ? a : b;
    r[1] = (a < b) ? b : a;
  }
}

// modulus ordering: the pairs (i, j), i < j, i + j = s (mod n), in increasing i, then the
// self-paired couple of an even step
__global__ void k_pjs_mod(unsigned n, unsigned stp, unsigned *t)
{
  const unsigned half = n >> 1;
  const unsigned long long tot = (unsigned long long)stp * half;
  for (unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; w < tot;
       w += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned s = (unsigned)(w / half), k = (unsigned)(w % half);
    unsigned *r = t + (size_t)s * n + 2u * k;
    // the i < j solutions of i + j = s (mod n) in increasing i: for odd s there are n/2 of
    // them; for even s, n/2 - 1 of them, followed by (s/2, s/2 + n/2)
    const bool even = !(s & 1u);
    // enumerate i = 0.. with j = (s - i) mod n, keeping i < j
    // count of valid i below a bound is computed in closed form: i valid iff i < j(i)
    // For i <= s: j = s - i, valid iff i < s - i  <=> 2i < s.
    // For i > s:  j = s + n - i, valid iff 2i < s + n.
    const unsigned c1 = (s + 1u) >> 1;                   // i in [0, ceil(s/2)) with 2i < s
    const unsigned lo2 = s + 1u, hi2 = (s + n + 1u) >> 1; // i in [s+1, ceil((s+n)/2))
    const unsigned c2 = (hi2 > lo2) ? (hi2 - lo2) : 0u;
    unsigned a, b;
    if (k < c1) {
      a = k;
      b = s - k;
    }
    else if (k < c1 + c2) {
      a = lo2 + (k - c1);
      b = s + n - a;
    }
    else {
      a = s >> 1;
      b = a + half;
      (void)even;
    }
    r[0] = a;
    r[1] = b;
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
