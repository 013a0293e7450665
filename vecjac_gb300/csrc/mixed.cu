// Mixed-precision one-sided Jacobi SVD: FP32 presweeps, FP64 finishing sweeps.
//
// GB300 runs FP32 arithmetic at about 70 times its FP64 rate, so most of the sweeps are
// done in FP32 and only the last ones in FP64:
//   1. A (FP64) is scaled by a power of two to max |a_ij| ~ 1 and rounded to FP32;
//   2. svjsvd_/cvjsvd_'s algorithm runs on it (V32 := I) until FP32 convergence;
//   3. V32 is widened to FP64 and made orthonormal to FP64 accuracy by two Newton-Schulz
//      polar steps, V <- V (3I - V^H V) / 2 (FP64 GEMMs; V32 is orthonormal to ~1e-6, so two
//      quadratically convergent steps reach rounding level);
//   4. G1 = A V (FP64 GEMM); its columns are orthogonal to the FP32 level;
//   5. dvjsvd_/zvjsvd_'s algorithm runs on G1 with V as the preset matrix (the reference's
//      iwork[0] != 0 mode, src/dvjsvd.c:88-96): a few FP64 sweeps finish the
//      factorisation, G1 R = U Sigma and V R = V_final, so A = U Sigma V_final^H with FP64
//      accuracy.
// The GEMMs are plain library GEMMs (cuBLAS DGEMM, four real products per complex one on
// the split planes).
#include <cmath>
#include <cstdio>
#include <cstring>

#include <cublas_v2.h>
#include <cuda_runtime.h>

#include "vj_fp.cuh"
#include "vj_host.h"

namespace vj {

// defined in jsvd.cu
template <typename T, bool CPLX>
vj_fint svd_dev_entry(vj_fnat m, vj_fnat n, T *G, vj_fnat ldG, T *Gi, vj_fnat ldGi, T *V, vj_fnat ldV, T *Vi,
                      vj_fnat ldVi, T *eS, T *fS, const unsigned *js, unsigned stp, unsigned swp, int preset,
                      cudaStream_t s);

__global__ void k_to_f32(const double *A, long long ld, long long rows, long long cols, int e, float *B)
{
  for (long long j = blockIdx.y; j < cols; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x)
      B[j * rows + i] = __double2float_rn(scale2(A[j * ld + i], e));
}

__global__ void k_to_f64(const float *A, long long n, double *B)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    B[i] = (double)A[i];
}

__global__ void k_copy(const double *A, long long ld, long long rows, long long cols, double *B)
{
  for (long long j = blockIdx.y; j < cols; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x)
      B[j * rows + i] = A[j * ld + i];
}

__global__ void k_absmax(const double *A, long long ld, long long rows, long long cols, unsigned long long *out)
{
  unsigned long long mx = 0ull;
  for (long long j = blockIdx.y; j < cols; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(A[j * ld + i]) & 0x7fffffffffffffffull;
      mx = (b > mx) ? b : mx;
    }
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = (w > mx) ? w : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx)
    atomicMax(out, mx);
}

static dim3 grid2(long long rows, long long cols)
{
  long long gx = (rows + 255) / 256;
  if (gx > 32)
    gx = 32;
  long long gy = cols < 65535 ? cols : 65535;
  return dim3((unsigned)gx, (unsigned)(gy > 0 ? gy : 1));
}

static cublasHandle_t cublas()
{
  static cublasHandle_t h = nullptr;
  if (!h && cublasCreate(&h) != CUBLAS_STATUS_SUCCESS)
    h = nullptr;
  return h;
}

// split-plane complex matrix: real and imaginary planes with their leading dimensions
struct Planes {
  double *re, *im;
  int ldr, ldi;
};

// C = op(A) B on split planes (op(A) = A or A^H; complex: four real products)
static bool zgemm(cublasHandle_t h, bool cplx, bool conjA, int m, int n, int k, Planes A, Planes B, Planes Cm)
{
  const cublasOperation_t op = conjA ? CUBLAS_OP_T : CUBLAS_OP_N;
  auto g = [&](const double *X, int ldx, const double *Y, int ldy, double a, double b, double *Z, int ldz) {
    return cublasDgemm(h, op, CUBLAS_OP_N, m, n, k, &a, X, ldx, Y, ldy, &b, Z, ldz) == CUBLAS_STATUS_SUCCESS;
  };
  if (!cplx)
    return g(A.re, A.ldr, B.re, B.ldr, 1.0, 0.0, Cm.re, Cm.ldr);
  // real part: Ar Br - Ai Bi, or Ar^T Br + Ai^T Bi for A^H
  const double sgn = conjA ? 1.0 : -1.0;
  bool ok = g(A.re, A.ldr, B.re, B.ldr, 1.0, 0.0, Cm.re, Cm.ldr) && g(A.im, A.ldi, B.im, B.ldi, sgn, 1.0, Cm.re, Cm.ldr);
  // imaginary part: Ar Bi + Ai Br, or Ar^T Bi - Ai^T Br for A^H
  ok = ok && g(A.re, A.ldr, B.im, B.ldi, 1.0, 0.0, Cm.im, Cm.ldi) && g(A.im, A.ldi, B.re, B.ldr, -sgn, 1.0, Cm.im, Cm.ldi);
  return ok;
}

template <bool CPLX>
static vj_fint mixed_dev(vj_fnat m_, vj_fnat n_, double *G, vj_fnat ldG, double *Gi, vj_fnat ldGi, double *V,
                         vj_fnat ldV, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                         unsigned stp, unsigned swp, cudaStream_t s, unsigned *sweeps32)
{
  const long long m = (long long)m_, n = (long long)n_;
  if (!n)
    return 0;
  if (m_ < n_ || (m % 16) || (n & 1) || ((n >> 1) % 16))  // the FP32 presweeps' shape rules
    return -1;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  cublasHandle_t h = cublas();
  if (!h)
    return VJ_ERR_CUDA;
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS)
    return VJ_ERR_CUDA;
  const int P = CPLX ? 2 : 1;
  // scratch: A32 (P m n), V32 (P n n), eS32/fS32 (2n) floats; A64 copy (P m n), T (P n n), W (P n n) doubles
  const size_t f32 = (size_t)P * m * n + (size_t)P * n * n + 2 * (size_t)n;
  const size_t f64 = (size_t)P * m * n + 2 * (size_t)P * n * n;
  host::Staging &stg = host::staging3();
  if (!stg.reserve(f32 * 4 + f64 * 8 + 1024))
    return VJ_ERR_NOMEM;
  float *A32 = reinterpret_cast<float *>(stg.ptr);
  float *V32 = A32 + (size_t)P * m * n;
  float *e32 = V32 + (size_t)P * n * n;
  float *f32p = e32 + n;
  double *A64 = reinterpret_cast<double *>(stg.ptr + ((f32 * 4 + 255) & ~(size_t)255));
  double *T = A64 + (size_t)P * m * n;
  double *W = T + (size_t)P * n * n;
  unsigned long long *cell = reinterpret_cast<unsigned long long *>(W + (size_t)P * n * n);
  // 1. scale to max |a| ~ 1 and round to FP32
  if (cudaMemsetAsync(cell, 0, 8, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  k_absmax<<<grid2(m, n), 256, 0, s>>>(G, (long long)ldG, m, n, cell);
  if (CPLX)
    k_absmax<<<grid2(m, n), 256, 0, s>>>(Gi, (long long)ldGi, m, n, cell);
  unsigned long long mb = 0;
  if (cudaMemcpyAsync(&mb, cell, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return VJ_ERR_CUDA;
  double amax;
  memcpy(&amax, &mb, 8);
  if (!(amax <= 1.7976931348623157e308))
    return CPLX ? -92 : -80;
  int e = 0;
  if (amax > 0.0) {
    (void)std::frexp(amax, &e);
    e = -e;
  }
  k_to_f32<<<grid2(m, n), 256, 0, s>>>(G, (long long)ldG, m, n, e, A32);
  if (CPLX)
    k_to_f32<<<grid2(m, n), 256, 0, s>>>(Gi, (long long)ldGi, m, n, e, A32 + (size_t)m * n);
  k_copy<<<grid2(m, n), 256, 0, s>>>(G, (long long)ldG, m, n, A64);
  if (CPLX)
    k_copy<<<grid2(m, n), 256, 0, s>>>(Gi, (long long)ldGi, m, n, A64 + (size_t)m * n);
  // 2. FP32 presweeps, V32 := I
  const vj_fint r32 = svd_dev_entry<float, CPLX>(m_, n_, A32, m_, CPLX ? A32 + (size_t)m * n : nullptr, m_, V32, n_,
                                                 CPLX ? V32 + (size_t)n * n : nullptr, n_, e32, f32p, js, stp, swp,
                                                 0, s);
  if (r32 < 0)
    return r32;
  if (sweeps32)
    *sweeps32 = (unsigned)r32;
  // 3. V (FP64, caller's buffer, leading dimension ldV) from V32; two Newton-Schulz steps
  for (int pl = 0; pl < P; ++pl) {
    double *Vd = pl ? Vi : V;
    const vj_fnat ldd = pl ? ldVi : ldV;
    k_to_f64<<<(unsigned)((n * n + 255) / 256 < 4096 ? (n * n + 255) / 256 : 4096), 256, 0, s>>>(
        V32 + (size_t)pl * n * n, n * n, W);
    if (cudaMemcpy2DAsync(Vd, ldd * 8, W, n * 8, n * 8, n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return VJ_ERR_CUDA;
  }
  const int ni = (int)n, mi = (int)m;
  const Planes Vp{V, Vi, (int)ldV, (int)(CPLX ? ldVi : ldV)};
  const Planes Tp{T, T + (size_t)n * n, ni, ni}, Wp{W, W + (size_t)n * n, ni, ni};
  for (int it = 0; it < 2; ++it) {
    // T = V^H V;  W = V T;  V = 1.5 V - 0.5 W
    if (!zgemm(h, CPLX, true, ni, ni, ni, Vp, Vp, Tp) || !zgemm(h, CPLX, false, ni, ni, ni, Vp, Tp, Wp))
      return VJ_ERR_CUDA;
    const double a15 = 1.5, am05 = -0.5;
    for (int pl = 0; pl < P; ++pl) {
      double *Vd = pl ? Vp.im : Vp.re;
      const int ldd = pl ? Vp.ldi : Vp.ldr;
      if (cublasDgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, ni, ni, &a15, Vd, ldd, &am05, pl ? Wp.im : Wp.re, ni, Vd, ldd) !=
          CUBLAS_STATUS_SUCCESS)
        return VJ_ERR_CUDA;
    }
  }
  // 4. G1 = A V (into the caller's G)
  const Planes Ap{A64, A64 + (size_t)m * n, mi, mi};
  const Planes Gp{G, Gi, (int)ldG, (int)(CPLX ? ldGi : ldG)};
  if (!zgemm(h, CPLX, false, mi, ni, ni, Ap, Vp, Gp))
    return VJ_ERR_CUDA;
  // 5. FP64 finishing sweeps with V preset
  return svd_dev_entry<double, CPLX>(m_, n_, G, ldG, Gi, ldGi, V, ldV, Vi, ldVi, eS, fS, js, stp, swp, 1, s);
}

}  // namespace vj

extern "C" {

vj_fint vj_dvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS,
                            double *fS, const unsigned *js, unsigned stp, unsigned swp, unsigned *sweeps32,
                            void *stream)
{
  return vj::mixed_dev<false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp,
                              (cudaStream_t)stream, sweeps32);
}

vj_fint vj_zvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *Gr, vj_fnat ldGr, double *Gi, vj_fnat ldGi, double *Vr,
                            vj_fnat ldVr, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                            unsigned stp, unsigned swp, unsigned *sweeps32, void *stream)
{
  return vj::mixed_dev<true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp,
                             (cudaStream_t)stream, sweeps32);
}

}  // extern "C"
