// Adjoint (reverse-mode derivative) of the thin SVD A = U diag(s) V^T, batched.
//
// Given cotangents dS (n), dU (m x k: the first k columns of U) and dV (n x k: the first k
// columns of V), the cotangent of A is (Townsend, "Differentiating the singular value
// decomposition", 2016, eq. for the thin real SVD with m >= n, V square):
//   dA = U N V^T + dU_k S_k^{-1} V_k^T,
//   N  = diag(dS) + (F o (J - J^T)) S + S (F o (K - K^T)) - J S^{-1},
//   J  = U^T dU (n x k, zero-extended to n x n), K = V^T dV (n x k, zero-extended),
//   F_ij = 1 / (s_j^2 - s_i^2) for i != j, 0 on the diagonal.
// The difference s_j^2 - s_i^2 is formed as (s_j - s_i)(s_j + s_i) (no cancellation), and
// F is made gap-safe by Lorentzian broadening (Liao, Liu, Wang, Xiang, "Differentiable
// programming tensor networks", 2019): F = d / (d^2 + (g max(s_i, s_j)^2)^2), with g the
// caller's gap parameter; g = 0 keeps 1/d exactly and maps d = 0 (a degenerate pair) to 0.
// Columns with s_j = 0 contribute no 1/s_j terms.
//
// One CTA per matrix (a persistent grid strides over the batch). Everything a matrix
// needs is staged in shared memory with odd leading dimensions (conflict-free row and
// column walks); the two products are register-tiled (TM x TN per thread):
//   P = N V^T and Q = S_k^{-1} V_k^T, stacked as PQ ((n + k) x n),
//   dA = [U | dU] PQ (inner dimension n + k), written straight to global memory.
#include <cuda_runtime.h>

#include "vj_host.h"

namespace vj {

static __host__ __device__ __forceinline__ int odd_ld(int r)
{
  return r | 1;
}

// shared-memory elements of one matrix's working set
static __host__ __device__ __forceinline__ long long adj_elems(int m, int n, int k)
{
  const int lu = odd_ld(m), lv = odd_ld(n), lpq = odd_ld(n + k);
  return (long long)lu * (n + k) + (long long)lv * n + (long long)lv * k * 3 + (long long)lv * n +
         (long long)lpq * n + 2LL * n;
}

// C(r, c) = sum_l A(r, l) B(l, c) for r < R, c < Cn, l < L, with A(r, l) = A[r*ars + l*als],
// B(l, c) = B[l*bls + c*bcs]; rows of a thread's tile are strided by the row-group count so
// that neighbouring threads walk neighbouring rows. The store is done by `st(r, c, value)`.
template <typename T, int TM, int TN, typename Store>
__device__ __forceinline__ void cta_gemm(int R, int Cn, int L, const T *A, int ars, int als, const T *B, int bls,
                                         int bcs, Store st)
{
  const int RG = (R + TM - 1) / TM, CG = (Cn + TN - 1) / TN;
  for (int t = threadIdx.x; t < RG * CG; t += blockDim.x) {
    const int rb = t % RG, cb = t / RG;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j)
        acc[i][j] = (T)0;
    int rr[TM], cc[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int r = rb + i * RG;
      rr[i] = r < R ? r : R - 1;
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int c = cb * TN + j;
      cc[j] = c < Cn ? c : Cn - 1;
    }
    for (int l = 0; l < L; ++l) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i)
        a[i] = A[rr[i] * ars + l * als];
#pragma unroll
      for (int j = 0; j < TN; ++j)
        b[j] = B[l * bls + cc[j] * bcs];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j)
          acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j)
        if (rb + i * RG < R && cb * TN + j < Cn)
          st(rb + i * RG, cb * TN + j, acc[i][j]);
  }
}

template <typename T> struct AdjArgs {
  long long count;
  int m, n, k;
  const T *U, *S, *V, *dS, *dU, *dV;
  T *dA;
  T gap;
};

template <typename T> __global__ void __launch_bounds__(256) k_svd_adjoint(AdjArgs<T> a)
{
  extern __shared__ __align__(16) unsigned char adj_smem[];
  T *sm = reinterpret_cast<T *>(adj_smem);
  const int m = a.m, n = a.n, k = a.k;
  const int lu = odd_ld(m), lv = odd_ld(n), lpq = odd_ld(n + k);
  T *UD = sm;                            // m x (n + k): U then dU
  T *Vs = UD + (size_t)lu * (n + k);     // n x n
  T *dVs = Vs + (size_t)lv * n;          // n x k
  T *J = dVs + (size_t)lv * k;           // n x k
  T *K = J + (size_t)lv * k;             // n x k
  T *N = K + (size_t)lv * k;             // n x n
  T *PQ = N + (size_t)lv * n;            // (n + k) x n
  T *s = PQ + (size_t)lpq * n;           // n
  T *ds = s + n;                         // n
  for (long long b = blockIdx.x; b < a.count; b += gridDim.x) {
    const T *U = a.U + b * (long long)m * n, *V = a.V + b * (long long)n * n;
    const T *dU = a.dU + b * (long long)m * k, *dV = a.dV + b * (long long)n * k;
    for (int e = threadIdx.x; e < m * n; e += blockDim.x)
      UD[(e / m) * lu + e % m] = U[e];
    for (int e = threadIdx.x; e < m * k; e += blockDim.x)
      UD[(n + e / m) * lu + e % m] = dU[e];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x)
      Vs[(e / n) * lv + e % n] = V[e];
    for (int e = threadIdx.x; e < n * k; e += blockDim.x)
      dVs[(e / n) * lv + e % n] = dV[e];
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      s[e] = a.S[b * n + e];
      ds[e] = a.dS[b * n + e];
    }
    __syncthreads();
    // J = U^T dU, K = V^T dV (n x k each)
    cta_gemm<T, 2, 2>(n, k, m, UD, lu, 1, UD + (size_t)n * lu, 1, lu,
                      [&](int r, int c, T v) { J[c * lv + r] = v; });
    cta_gemm<T, 2, 2>(n, k, n, Vs, lv, 1, dVs, 1, lv, [&](int r, int c, T v) { K[c * lv + r] = v; });
    __syncthreads();
    // N (n x n)
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const T si = s[i], sj = s[j];
      T v;
      if (i == j) {
        v = ds[i];
        if (j < k && sj != (T)0)
          v -= J[j * lv + i] / sj;
      }
      else {
        const T jij = j < k ? J[j * lv + i] : (T)0, jji = i < k ? J[i * lv + j] : (T)0;
        const T kij = j < k ? K[j * lv + i] : (T)0, kji = i < k ? K[i * lv + j] : (T)0;
        const T d = (sj - si) * (sj + si);
        const T mx = si > sj ? si : sj;
        const T g = a.gap * mx * mx;
        const T den = d * d + g * g;
        const T F = den != (T)0 ? d / den : (T)0;
        v = F * ((jij - jji) * sj + si * (kij - kji));
        if (j < k && sj != (T)0)
          v -= jij / sj;
      }
      N[j * lv + i] = v;
    }
    // Q = S_k^{-1} V_k^T into rows n .. n+k-1 of PQ
    for (int e = threadIdx.x; e < k * n; e += blockDim.x) {
      const int j = e % k, l = e / k;
      const T sj = s[j];
      PQ[l * lpq + n + j] = sj != (T)0 ? Vs[j * lv + l] / sj : (T)0;
    }
    __syncthreads();
    // P = N V^T into rows 0 .. n-1 of PQ
    cta_gemm<T, 4, 2>(n, n, n, N, 1, lv, Vs, lv, 1, [&](int r, int c, T v) { PQ[c * lpq + r] = v; });
    __syncthreads();
    // dA = [U | dU] PQ
    T *dA = a.dA + b * (long long)m * n;
    cta_gemm<T, 4, 4>(m, n, n + k, UD, 1, lu, PQ, 1, lpq, [&](int r, int c, T v) { dA[(size_t)c * m + r] = v; });
    __syncthreads();
  }
}

template <typename T>
static vj_fint adjoint_dev(long long count, int m, int n, int k, const T *U, const T *S, const T *V, const T *dS,
                           const T *dU, const T *dV, T *dA, T gap, void *stream)
{
  if (count < 0 || m < n || n < 1 || k < 0 || k > n)
    return VJ_ERR_ARG;
  if (!count)
    return 0;
  if (!U || !S || !V || !dS || !dA || (k && (!dU || !dV)))
    return VJ_ERR_ARG;
  const size_t smem = (size_t)adj_elems(m, n, k) * sizeof(T);
  if (smem > 227 * 1024)
    return VJ_ERR_ARG;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  if (cudaFuncSetAttribute(k_svd_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return VJ_ERR_CUDA;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_svd_adjoint<T>, 256, smem) != cudaSuccess || occ < 1)
    return VJ_ERR_CUDA;
  long long grid = (long long)host::sm_count() * occ;
  if (grid > count)
    grid = count;
  AdjArgs<T> a{count, m, n, k, U, S, V, dS, dU, dV, dA, gap};
  k_svd_adjoint<T><<<(unsigned)grid, 256, smem, (cudaStream_t)stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : VJ_ERR_CUDA;
}

}  // namespace vj

extern "C" {

vj_fint vj_ssvd_adjoint_batch_dev(vj_fint count, vj_fnat m, vj_fnat n, vj_fnat k, const float *U, const float *S,
                                  const float *V, const float *dS, const float *dU, const float *dV, float *dA,
                                  float gap, void *stream)
{
  if (m > 65536 || n > 65536 || k > 65536)
    return VJ_ERR_ARG;
  return vj::adjoint_dev<float>(count, (int)m, (int)n, (int)k, U, S, V, dS, dU, dV, dA, gap, stream);
}

vj_fint vj_dsvd_adjoint_batch_dev(vj_fint count, vj_fnat m, vj_fnat n, vj_fnat k, const double *U, const double *S,
                                  const double *V, const double *dS, const double *dU, const double *dV, double *dA,
                                  double gap, void *stream)
{
  if (m > 65536 || n > 65536 || k > 65536)
    return VJ_ERR_ARG;
  return vj::adjoint_dev<double>(count, (int)m, (int)n, (int)k, U, S, V, dS, dU, dV, dA, gap, stream);
}

}  // extern "C"
