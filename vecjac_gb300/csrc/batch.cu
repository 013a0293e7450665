// Batched one-sided Jacobi SVD: thousands of independent matrices of uneven size in one
// persistent launch (real FP64 and FP32; every matrix with dvjsvd_'s / svjsvd_'s result).
//
// One CTA owns one matrix at a time and runs the reference driver on it literally
// (src/dvjsvd.c:78-638): setup and global prescale, then sweeps of pivot steps, each step
// being "norms of the changed columns (with the overflow retry) -> all scaled dot products
// -> error check -> classification -> all transformations -> max |G|, max |V| update", with
// __syncthreads between the phases. Matrices are handed out by an atomic work queue in the
// order the caller gives (largest first balances the tail); a matrix stops at its own
// convergence (its own sweep count, its own info entry), so uneven convergence does not
// hold the batch back. Pivot pairs are computed on the fly from the strategy's closed
// form (pjs.cuh), so no tables are stored. Matrix sizes: m >= n, n <= 512, and the
// reference's divisibility rules (the host wrapper pads with zero rows/columns).
#include <cuda_runtime.h>

#include "batch_core.cuh"

namespace vj {

// MINB: the register bound for MINB resident CTAs of 256 threads per SM (more, smaller
// CTAs when the caller launches fewer threads per CTA). The best bound depends on the
// batch (the autotuner of vecjac_gb300/batch.py searches it with the CTA size): on the
// 20,000-matrix FP32 batch 4 CTAs of 256 threads (64 registers) gave 1434 matrices/s,
// 3 (80 registers) 1221, 2 (128) 937.
template <typename T, int MINB>
__global__ void __launch_bounds__(256, MINB) k_batch(BatchArgs<T> a)
{
  __shared__ BatchShared<T> sh;
  __shared__ long long s_b;
  for (;;) {
    if (threadIdx.x == 0)
      s_b = (long long)atomicAdd(a.queue, 1u);
    __syncthreads();
    const long long bi = s_b;
    __syncthreads();
    if (bi >= a.count)
      return;
    const int b = a.order ? a.order[bi] : (int)bi;
    const long long r = svd_one<T>(a, sh, a.m[b], a.n[b], a.G + a.offG[b], a.V + a.offV[b], a.eS + a.offS[b],
                                   a.fS + a.offS[b]);
    if (threadIdx.x == 0)
      a.info[b] = r;
    __syncthreads();
  }
}

// default register bound: FP32 4 CTAs of 256 threads per SM, FP64 2 (118 registers; a
// bound of 3 spills)
template <typename T> constexpr int batch_occ_default() { return sizeof(T) == 4 ? 4 : 2; }

template <typename T, int MINB> static void *batch_kernel() { return reinterpret_cast<void *>(k_batch<T, MINB>); }

template <typename T>
static vj_fint batch_dev(vj_fint count, const long long *m, const long long *n, T *G, const long long *offG, T *V,
                         const long long *offV, T *eS, T *fS, const long long *offS, const int *order,
                         long strategy, unsigned swp, long long *info, int block, int occ, void *stream)
{
  if (count < 0 || (strategy != 2l && strategy != 4l))
    return VJ_ERR_ARG;
  if (!count)
    return 0;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  if (block != 64 && block != 128 && block != 256)
    block = 128;
  if (occ < 2 || occ > 6)
    occ = batch_occ_default<T>();
  cudaStream_t s = (cudaStream_t)stream;
  unsigned *queue = host::batch_queue();
  if (!queue)
    return VJ_ERR_NOMEM;
  if (cudaMemsetAsync(queue, 0, sizeof(unsigned), s) != cudaSuccess)
    return VJ_ERR_CUDA;
  BatchArgs<T> a;
  a.count = count;
  a.m = m; a.n = n; a.offG = offG; a.offV = offV; a.offS = offS; a.order = order;
  a.G = G; a.V = V; a.eS = eS; a.fS = fS; a.info = info; a.queue = queue;
  a.strategy = (int)strategy;
  a.swp = swp;
  void *k = (occ == 2)   ? batch_kernel<T, 2>()
            : (occ == 3) ? batch_kernel<T, 3>()
            : (occ == 4) ? batch_kernel<T, 4>()
            : (occ == 5) ? batch_kernel<T, 5>()
                         : batch_kernel<T, 6>();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  long long grid = (long long)host::sm_count() * per_sm;
  if (grid > count)
    grid = count;
  void *args[] = {&a};
  if (cudaLaunchKernel(k, dim3((unsigned)grid), dim3((unsigned)block), args, 0, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  return (cudaGetLastError() == cudaSuccess) ? 0 : VJ_ERR_CUDA;
}

}  // namespace vj

extern "C" {

vj_fint vj_dvjsvd_batch_dev(vj_fint count, const long long *m, const long long *n, double *G, const long long *offG,
                            double *V, const long long *offV, double *eS, double *fS, const long long *offS,
                            const int *order, long strategy, unsigned swp, long long *info, int block, void *stream)
{
  return vj::batch_dev<double>(count, m, n, G, offG, V, offV, eS, fS, offS, order, strategy, swp, info, block, 0,
                               stream);
}

vj_fint vj_svjsvd_batch_dev(vj_fint count, const long long *m, const long long *n, float *G, const long long *offG,
                            float *V, const long long *offV, float *eS, float *fS, const long long *offS,
                            const int *order, long strategy, unsigned swp, long long *info, int block, void *stream)
{
  return vj::batch_dev<float>(count, m, n, G, offG, V, offV, eS, fS, offS, order, strategy, swp, info, block, 0,
                              stream);
}

vj_fint vj_dvjsvd_batch_tuned_dev(vj_fint count, const long long *m, const long long *n, double *G,
                                  const long long *offG, double *V, const long long *offV, double *eS, double *fS,
                                  const long long *offS, const int *order, long strategy, unsigned swp,
                                  long long *info, int block, int occupancy, void *stream)
{
  return vj::batch_dev<double>(count, m, n, G, offG, V, offV, eS, fS, offS, order, strategy, swp, info, block,
                               occupancy, stream);
}

vj_fint vj_svjsvd_batch_tuned_dev(vj_fint count, const long long *m, const long long *n, float *G,
                                  const long long *offG, float *V, const long long *offV, float *eS, float *fS,
                                  const long long *offS, const int *order, long strategy, unsigned swp,
                                  long long *info, int block, int occupancy, void *stream)
{
  return vj::batch_dev<float>(count, m, n, G, offG, V, offV, eS, fS, offS, order, strategy, swp, info, block,
                              occupancy, stream);
}

}  // extern "C"
