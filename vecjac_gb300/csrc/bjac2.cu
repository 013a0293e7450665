// Batched 2x2 Hermitian EVD: dbjac2_/zbjac2_/sbjac2_/cbjac2_ and the masked i-variants.
//
// The reference walks the SoA arrays in 8- (FP64) or 16-lane (FP32) AVX-512 vectors and
// stores one permutation word per vector (src/dbjac2.c:104-137). Here a quad of 4
// consecutive threads covers one such group: every thread moves 16 bytes per array
// per iteration (2 doubles or 4 floats, 128-bit streaming loads and stores), computes
// its lanes with vj::rjac2/cjac2, and the quad ORs its permutation bits into the
// group's word with two xor-shuffles. The grid is a multiple of the SM count and
// strides over the arrays, so every byte of HBM is touched exactly once.
#include <cfenv>
#include <cstdlib>
#include <cuda_runtime.h>

#include "jac2.cuh"
#include "vj_host.h"

namespace vj {

template <typename T> struct vec16;
template <> struct vec16<double> { using V = double2; static constexpr int N = 2; };
template <> struct vec16<float> { using V = float4; static constexpr int N = 4; };

template <typename T> __device__ __forceinline__ typename vec16<T>::V ld(const T *p, long long i)
{
  return __ldcs(reinterpret_cast<const typename vec16<T>::V *>(p) + i);
}
template <typename T> __device__ __forceinline__ void st(T *p, long long i, const typename vec16<T>::V &v)
{
  __stcs(reinterpret_cast<typename vec16<T>::V *>(p) + i, v);
}
template <typename T> __device__ __forceinline__ T &el(typename vec16<T>::V &v, int k)
{
  return reinterpret_cast<T *>(&v)[k];
}

// group of LANES elements = 4 threads x VN elements; LOWMASK of the i-variant
template <typename T> struct grp {
  static constexpr int VN = vec16<T>::N;
  static constexpr int LANES = 4 * VN;
  static constexpr unsigned LOW = (LANES == 8) ? 0xFFu : 0xFFFFu;
};

template <typename T, bool CPLX, int KIND, bool INTERNAL, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) k_bjac2(long long nvec, const T *__restrict__ a11, const T *__restrict__ a22,
                                               const T *__restrict__ a21r, const T *__restrict__ a21i,
                                               T *__restrict__ c, T *__restrict__ cat, T *__restrict__ sat,
                                               T *__restrict__ l1, T *__restrict__ l2, unsigned *__restrict__ p)
{
  using V = typename vec16<T>::V;
  constexpr int VN = grp<T>::VN;
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // warps iterate uniformly so that the full-mask shuffles are always legal
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nvec; base += stride) {
    const long long i = base + lane;
    const bool act = (i < nvec);
    const long long g = i >> 2;  // group (= p word) index
    bool work = act;
    unsigned pin = 0u;
    if (INTERNAL && act) {
      pin = p[g];
      work = (pin & grp<T>::LOW) != 0u;
    }
    unsigned bitsv = 0u;
    if (work) {
      V x1 = ld(a11, i), x2 = ld(a22, i), xr = ld(a21r, i), xi;
      if (CPLX)
        xi = ld(a21i, i);
      V vc, vat, vsat, vl1, vl2;
#pragma unroll
      for (int k = 0; k < VN; ++k) {
        unsigned b;
        if (CPLX)
          b = cjac2<T, KIND>(el<T>(x1, k), el<T>(x2, k), el<T>(xr, k), el<T>(xi, k), el<T>(vc, k), el<T>(vat, k),
                             el<T>(vsat, k), el<T>(vl1, k), el<T>(vl2, k));
        else
          b = rjac2<T, KIND>(el<T>(x1, k), el<T>(x2, k), el<T>(xr, k), el<T>(vc, k), el<T>(vat, k), el<T>(vl1, k),
                             el<T>(vl2, k));
        bitsv |= (b << k);
      }
      st(c, i, vc);
      st(cat, i, vat);
      if (CPLX)
        st(sat, i, vsat);
      st(l1, i, vl1);
      st(l2, i, vl2);
    }
    unsigned w = bitsv << (VN * (lane & 3));
    w |= __shfl_xor_sync(0xffffffffu, w, 1);
    w |= __shfl_xor_sync(0xffffffffu, w, 2);
    if (act && work && ((lane & 3) == 0))
      p[g] = (INTERNAL ? ((pin & ~grp<T>::LOW) | w) : w);
  }
}

template <typename T, bool CPLX, int KIND, bool INTERNAL>
static cudaError_t launch_kind(long long n, const T *a11, const T *a22, const T *a21r, const T *a21i, T *c, T *cat,
                               T *sat, T *l1, T *l2, unsigned *p, cudaStream_t s)
{
  const long long nvec = n / grp<T>::VN;
  if (nvec <= 0)
    return cudaSuccess;
  int blocks = host::sm_count() * 8;  // 8 CTAs of 256 threads per SM
  const long long need = (nvec + 255) / 256;
  if (need < blocks)
    blocks = (int)need;
  // FP64: registers capped for 4 resident CTAs per SM (a few bytes of spills; 2% faster than
  // 3 CTAs, measured on the 2^28 / 2^27 batches)
  if (sizeof(T) == 8)
    k_bjac2<T, CPLX, KIND, INTERNAL, 4><<<blocks, 256, 0, s>>>(nvec, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
  else
    k_bjac2<T, CPLX, KIND, INTERNAL><<<blocks, 256, 0, s>>>(nvec, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
  return cudaGetLastError();
}

// n signed as in the reference; internal selects the i-variant (secants for n < 0)
template <typename T, bool CPLX>
static vj_fint bjac2_dev(vj_fint n, int internal, const T *a11, const T *a22, const T *a21r, const T *a21i, T *c,
                         T *cat, T *sat, T *l1, T *l2, unsigned *p, cudaStream_t s)
{
  if (n % grp<T>::LANES)
    return -1;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const long long nn = (n < 0) ? -n : n;
  cudaError_t e;
  if (internal) {
    if (n < 0)
      e = launch_kind<T, CPLX, 2, true>(nn, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, s);
    else
      e = launch_kind<T, CPLX, 0, true>(nn, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, s);
  }
  else {
    if (n < 0)
      e = launch_kind<T, CPLX, 1, false>(nn, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, s);
    else
      e = launch_kind<T, CPLX, 0, false>(nn, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, s);
  }
  return (e == cudaSuccess) ? 1 : VJ_ERR_CUDA;
}

// Host-pointer form. Where the GPU can read pageable host memory the kernel reads the
// caller's inputs in place; otherwise chunks of the batch are staged through device
// buffers on two streams (copy in, compute, copy out), so that the copies of one chunk
// overlap the kernel of the other. VJ_STAGED=1 in the environment forces the staged form.
template <typename T, bool CPLX>
static vj_fint bjac2_host(vj_fint n, int internal, const T *a11, const T *a22, const T *a21r, const T *a21i, T *c,
                          T *cat, T *sat, T *l1, T *l2, unsigned *p)
{
  constexpr int LANES = grp<T>::LANES;
  // the reference's first check (IS_NOT_VFPENV, src/dbjac2.c:84, src/zbjac2.c:111): the
  // calling thread must round to nearest; -10 for real, -12 for complex data
  if (fegetround() != FE_TONEAREST)
    return CPLX ? -12 : -10;
  if (n % LANES)
    return -1;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const long long nn = (n < 0) ? -n : n;
  if (!nn)
    return 1;
  std::lock_guard<std::recursive_mutex> lk(host::host_call_lock());  // the device's staging buffers
  // On a GPU that reads pageable host memory coherently (Grace-Blackwell: NVLink-C2C with
  // address translation), the kernel reads the caller's inputs in place and writes its
  // outputs to device buffers, whose copies back to the caller's arrays overlap the
  // kernel of the next chunk. (GPU stores into pageable host memory are slower than the
  // copy engines, so outputs are not written in place.) The masked i-variant keeps the
  // caller's outputs for unprocessed groups and takes the fully staged path below.
  auto al16 = [](const void *q) { return q == nullptr || !((uintptr_t)q & 15u); };
  // Page-locked outputs as well: one launch reads the inputs and writes the outputs in
  // place over NVLink-C2C (both directions of the link at once, no copy-engine pass)
  const char *eo = getenv("VJ_E2E_OUT");
  if (!internal && host::pageable_access() && !(eo && *eo == 'c') && al16(a11) && al16(a22) && al16(a21r) &&
      al16(a21i) && al16(c) && al16(cat) && al16(sat) && al16(l1) && al16(l2) && host::host_pinned(c) &&
      host::host_pinned(cat) && host::host_pinned(sat) && host::host_pinned(l1) && host::host_pinned(l2) &&
      host::host_pinned(p)) {
    cudaStream_t st[2];
    if (!host::streams2(st))
      return VJ_ERR_CUDA;
    const vj_fint r = bjac2_dev<T, CPLX>(n, 0, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, st[0]);
    if (r < 0)
      return r;
    return (cudaStreamSynchronize(st[0]) == cudaSuccess) ? 1 : VJ_ERR_CUDA;
  }
  if (!internal && host::pageable_access() && al16(a11) && al16(a22) && al16(a21r) && al16(a21i)) {
    const long long chunk = host::bjac2_chunk(nn, sizeof(T), CPLX, LANES);
    const int nout = CPLX ? 5 : 4;
    T *hout[5] = {c, cat, CPLX ? sat : l1, CPLX ? l1 : l2, CPLX ? l2 : nullptr};
    const size_t per = (size_t)chunk * sizeof(T);
    const size_t pwords = (size_t)(chunk / LANES) * sizeof(unsigned);
    const size_t slot = ((nout * per + pwords) + 255u) & ~(size_t)255u;
    host::Staging &stg = host::staging();
    if (!stg.reserve(2 * slot))
      return VJ_ERR_NOMEM;
    cudaStream_t st[2];
    if (!host::streams2(st))
      return VJ_ERR_CUDA;
    auto copy_back = [&](int b, long long off, long long cnt) -> bool {
      char *base = stg.ptr + (size_t)b * slot;
      const size_t bytes = (size_t)cnt * sizeof(T);
      for (int k = 0; k < nout; ++k)
        if (cudaMemcpyAsync(hout[k] + off, base + k * per, bytes, cudaMemcpyDeviceToHost, st[b]) != cudaSuccess)
          return false;
      return cudaMemcpyAsync(p + off / LANES, base + nout * per, (size_t)(cnt / LANES) * sizeof(unsigned),
                             cudaMemcpyDeviceToHost, st[b]) == cudaSuccess;
    };
    long long prev_off = -1, prev_cnt = 0;
    int prev_b = 0;
    for (long long off = 0, it = 0; off < nn; off += chunk, ++it) {
      const long long cnt = (nn - off < chunk) ? (nn - off) : chunk;
      const int b = (int)(it & 1);
      char *base = stg.ptr + (size_t)b * slot;
      T *dout[5];
      for (int k = 0; k < nout; ++k)
        dout[k] = reinterpret_cast<T *>(base + k * per);
      unsigned *dp = reinterpret_cast<unsigned *>(base + nout * per);
      const vj_fint sn = (n < 0) ? -cnt : cnt;
      const vj_fint r = bjac2_dev<T, CPLX>(sn, 0, a11 + off, a22 + off, a21r + off, CPLX ? a21i + off : nullptr,
                                           dout[0], dout[1], CPLX ? dout[2] : nullptr, CPLX ? dout[3] : dout[2],
                                           CPLX ? dout[4] : dout[3], dp, st[b]);
      if (r < 0)
        return r;
      // while this chunk computes, copy the previous one back (its stream is in order)
      if (prev_off >= 0 && !copy_back(prev_b, prev_off, prev_cnt))
        return VJ_ERR_CUDA;
      prev_off = off;
      prev_cnt = cnt;
      prev_b = b;
    }
    if (prev_off >= 0 && !copy_back(prev_b, prev_off, prev_cnt))
      return VJ_ERR_CUDA;
    if (cudaStreamSynchronize(st[0]) != cudaSuccess || cudaStreamSynchronize(st[1]) != cudaSuccess)
      return VJ_ERR_CUDA;
    return 1;
  }
  const long long chunk = host::bjac2_chunk(nn, sizeof(T), CPLX, LANES);
  const int nin = CPLX ? 4 : 3, nout = CPLX ? 5 : 4;
  const T *hin[4] = {a11, a22, a21r, a21i};
  T *hout[5] = {c, cat, CPLX ? sat : l1, CPLX ? l1 : l2, CPLX ? l2 : nullptr};
  host::Staging &stg = host::staging();
  const size_t per = (size_t)chunk * sizeof(T);
  const size_t pwords = (size_t)(chunk / LANES) * sizeof(unsigned);
  const size_t slot = (((nin + nout) * per + pwords) + 255u) & ~(size_t)255u;
  if (!stg.reserve(2 * slot))
    return VJ_ERR_NOMEM;
  cudaStream_t st[2];
  if (!host::streams2(st))
    return VJ_ERR_CUDA;
  for (long long off = 0, it = 0; off < nn; off += chunk, ++it) {
    const long long cnt = (nn - off < chunk) ? (nn - off) : chunk;
    const int b = (int)(it & 1);
    cudaStream_t s = st[b];
    char *base = stg.ptr + (size_t)b * slot;
    T *din[4], *dout[5];
    for (int k = 0; k < nin; ++k)
      din[k] = reinterpret_cast<T *>(base + k * per);
    for (int k = 0; k < nout; ++k)
      dout[k] = reinterpret_cast<T *>(base + (nin + k) * per);
    unsigned *dp = reinterpret_cast<unsigned *>(base + (nin + nout) * per);
    const size_t bytes = (size_t)cnt * sizeof(T);
    const size_t pb = (size_t)(cnt / LANES) * sizeof(unsigned);
    for (int k = 0; k < nin; ++k)
      if (cudaMemcpyAsync(din[k], hin[k] + off, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return VJ_ERR_CUDA;
    if (internal) {
      if (cudaMemcpyAsync(dp, p + off / LANES, pb, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      // unprocessed groups keep the caller's outputs
      for (int k = 0; k < nout; ++k)
        if (cudaMemcpyAsync(dout[k], hout[k] + off, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
          return VJ_ERR_CUDA;
    }
    const vj_fint sn = (n < 0) ? -cnt : cnt;
    const vj_fint r = bjac2_dev<T, CPLX>(sn, internal, din[0], din[1], din[2], CPLX ? din[3] : nullptr, dout[0],
                                         dout[1], CPLX ? dout[2] : nullptr, CPLX ? dout[3] : dout[2],
                                         CPLX ? dout[4] : dout[3], dp, s);
    if (r < 0)
      return r;
    for (int k = 0; k < nout; ++k)
      if (cudaMemcpyAsync(hout[k] + off, dout[k], bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return VJ_ERR_CUDA;
    if (cudaMemcpyAsync(p + off / LANES, dp, pb, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return VJ_ERR_CUDA;
  }
  if (cudaStreamSynchronize(st[0]) != cudaSuccess || cudaStreamSynchronize(st[1]) != cudaSuccess)
    return VJ_ERR_CUDA;
  return 1;
}

}  // namespace vj

using namespace vj;

extern "C" {

vj_fint dbjac2_(const vj_fint n[1], const double a11[], const double a22[], const double a21[], double c[],
                double at[], double l1[], double l2[], unsigned p[])
{
  return bjac2_host<double, false>(*n, 0, a11, a22, a21, nullptr, c, at, nullptr, l1, l2, p);
}
vj_fint dbjac2i(const vj_fint n[1], const double a11[], const double a22[], const double a21[], double c[],
                double at[], double l1[], double l2[], unsigned p[])
{
  return bjac2_host<double, false>(*n, 1, a11, a22, a21, nullptr, c, at, nullptr, l1, l2, p);
}
vj_fint zbjac2_(const vj_fint n[1], const double a11[], const double a22[], const double a21r[], const double a21i[],
                double c[], double cat[], double sat[], double l1[], double l2[], unsigned p[])
{
  return bjac2_host<double, true>(*n, 0, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
}
vj_fint zbjac2i(const vj_fint n[1], const double a11[], const double a22[], const double a21r[], const double a21i[],
                double c[], double cat[], double sat[], double l1[], double l2[], unsigned p[])
{
  return bjac2_host<double, true>(*n, 1, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
}
vj_fint sbjac2_(const vj_fint n[1], const float a11[], const float a22[], const float a21[], float c[], float at[],
                float l1[], float l2[], unsigned p[])
{
  return bjac2_host<float, false>(*n, 0, a11, a22, a21, nullptr, c, at, nullptr, l1, l2, p);
}
vj_fint sbjac2i(const vj_fint n[1], const float a11[], const float a22[], const float a21[], float c[], float at[],
                float l1[], float l2[], unsigned p[])
{
  return bjac2_host<float, false>(*n, 1, a11, a22, a21, nullptr, c, at, nullptr, l1, l2, p);
}
vj_fint cbjac2_(const vj_fint n[1], const float a11[], const float a22[], const float a21r[], const float a21i[],
                float c[], float cat[], float sat[], float l1[], float l2[], unsigned p[])
{
  return bjac2_host<float, true>(*n, 0, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
}
vj_fint cbjac2i(const vj_fint n[1], const float a11[], const float a22[], const float a21r[], const float a21i[],
                float c[], float cat[], float sat[], float l1[], float l2[], unsigned p[])
{
  return bjac2_host<float, true>(*n, 1, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
}

vj_fint vj_dbjac2_dev(vj_fint n, int internal, const double *a11, const double *a22, const double *a21, double *c,
                      double *at, double *l1, double *l2, unsigned *p, void *stream)
{
  return bjac2_dev<double, false>(n, internal, a11, a22, a21, nullptr, c, at, nullptr, l1, l2, p,
                                  (cudaStream_t)stream);
}
vj_fint vj_zbjac2_dev(vj_fint n, int internal, const double *a11, const double *a22, const double *a21r,
                      const double *a21i, double *c, double *cat, double *sat, double *l1, double *l2, unsigned *p,
                      void *stream)
{
  return bjac2_dev<double, true>(n, internal, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, (cudaStream_t)stream);
}
vj_fint vj_sbjac2_dev(vj_fint n, int internal, const float *a11, const float *a22, const float *a21, float *c,
                      float *at, float *l1, float *l2, unsigned *p, void *stream)
{
  return bjac2_dev<float, false>(n, internal, a11, a22, a21, nullptr, c, at, nullptr, l1, l2, p,
                                 (cudaStream_t)stream);
}
vj_fint vj_cbjac2_dev(vj_fint n, int internal, const float *a11, const float *a22, const float *a21r,
                      const float *a21i, float *c, float *cat, float *sat, float *l1, float *l2, unsigned *p,
                      void *stream)
{
  return bjac2_dev<float, true>(n, internal, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p, (cudaStream_t)stream);
}

}  // extern "C"
