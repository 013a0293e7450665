// Mixed-precision one-sided Jacobi SVD: FP32 presweeps, FP64 finishing sweeps.
//
// GB300 runs FP32 arithmetic at about 70 times its FP64 rate, so most of the sweeps are
// done in FP32 and only the last ones in FP64. Starting from G_0 = A (FP64), V_0 = I, each
// preconditioning stage s = 1..S
//   1. rounds G_{s-1} (scaled by a power of two to max |g_ij| <= 1) to FP32;
//   2. runs FP32 one-sided Jacobi sweeps on it (k_presweep, Hestenes rotations from plain
//      FP32 dot products) from W := I until no pair exceeds the FP32 tolerance;
//   3. widens W to FP64 and makes it orthonormal to FP64 accuracy with two Newton-Schulz
//      polar steps, W <- W (3I - W^H W) / 2 (W is orthonormal to ~1e-5, and each step
//      squares the error);
//   4. forms G_s = G_{s-1} W and V_s = V_{s-1} W (FP64 GEMMs).
// FP32 rounding is relative to each element, so from the second stage on the FP32 sweeps
// see the columns of G_{s-1} to their own relative accuracy and resolve the directions of
// small singular values that the first stage (on A itself) could not. Finally
// dvjsvd_/zvjsvd_'s algorithm runs on G_S with V_S as the preset matrix (the reference's
// iwork[0] != 0 mode, src/dvjsvd.c:88-96, src/zvjsvd.c:100-110): G_S R = U Sigma and
// V_S R = V, so A = U Sigma V^H with the FP64 algorithm's accuracy, after a few FP64
// sweeps instead of a full run. The GEMMs are plain library GEMMs (cuBLAS DGEMM; four
// real products per complex one on the split planes).
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

template <typename T> __global__ void k_eye_p(T *V, long long ld, long long n, int diag)
{
  for (long long j = blockIdx.y; j < n; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
      V[j * ld + i] = (diag && i == j) ? (T)1 : (T)0;
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

// One pivot step of FP32 one-sided Jacobi on planar G (m x n, ld m) and W (n x n, ld n):
// CTA k takes pair (p, q) = row st of the pivot table, forms a = |g_p|^2, b = |g_q|^2,
// c = g_p^H g_q (FP32, per-thread partial sums and a block tree), and when
// |c| >= tol sqrt(a b) applies the unitary [[cs, sn e^{i phi}], [-sn e^{-i phi}, cs]]
// (c = |c| e^{i phi}; t = sn/cs the smaller root of t^2 + 2 zeta t - 1 = 0,
// zeta = (b - a) / (2|c|)) to columns p and q of G and W, which makes them orthogonal.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_presweep(int m, int n, float *Gr, float *Gi, float *Wr, float *Wi,
                                                  const unsigned *js, int st, float tol, unsigned *cnt)
{
  __shared__ float red[4][8];
  __shared__ float rot[4];
  const int k = blockIdx.x;
  const unsigned p = js[(size_t)st * n + 2 * k], q = js[(size_t)st * n + 2 * k + 1];
  float *gpr = Gr + (size_t)p * m, *gqr = Gr + (size_t)q * m;
  float *gpi = CPLX ? Gi + (size_t)p * m : nullptr, *gqi = CPLX ? Gi + (size_t)q * m : nullptr;
  float a = 0.f, b = 0.f, cr = 0.f, ci = 0.f;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const float xr = gpr[i], yr = gqr[i];
    a = fmaf(xr, xr, a);
    b = fmaf(yr, yr, b);
    cr = fmaf(xr, yr, cr);
    if (CPLX) {
      const float xi = gpi[i], yi = gqi[i];
      a = fmaf(xi, xi, a);
      b = fmaf(yi, yi, b);
      cr = fmaf(xi, yi, cr);
      ci = fmaf(xr, yi, ci);
      ci = fmaf(-xi, yr, ci);
    }
  }
  for (int o = 16; o >= 1; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    cr += __shfl_xor_sync(0xffffffffu, cr, o);
    ci += __shfl_xor_sync(0xffffffffu, ci, o);
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = a;
    red[1][w] = b;
    red[2][w] = cr;
    red[3][w] = ci;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = cr = ci = 0.f;
    for (int j = 0; j < nw; ++j) {
      a += red[0][j];
      b += red[1][j];
      cr += red[2][j];
      ci += red[3][j];
    }
    const float ac = hypotf(cr, ci);
    float cs = 1.f, snr = 0.f, sni = 0.f, go = 0.f;
    if (ac > 0.f && ac >= tol * sqrtf(a) * sqrtf(b)) {
      const float zeta = (b - a) / (2.f * ac);
      const float az = fabsf(zeta);
      const float t = (az > 1e18f) ? 0.5f / zeta : copysignf(1.f, zeta) / (az + sqrtf(fmaf(zeta, zeta, 1.f)));
      cs = 1.f / sqrtf(fmaf(t, t, 1.f));
      const float sn = t * cs;
      snr = sn * (cr / ac);
      sni = sn * (ci / ac);
      go = 1.f;
      atomicAdd(cnt, 1u);
    }
    rot[0] = cs;
    rot[1] = snr;
    rot[2] = sni;
    rot[3] = go;
  }
  __syncthreads();
  if (rot[3] == 0.f)
    return;
  const float cs = rot[0], snr = rot[1], sni = rot[2];
  auto apply = [&](float *xr_, float *xi_, float *yr_, float *yi_, int rows) {
    for (int i = threadIdx.x; i < rows; i += blockDim.x) {
      const float pr = xr_[i], qr = yr_[i];
      if (CPLX) {
        const float pi = xi_[i], qi = yi_[i];
        xr_[i] = cs * pr - (snr * qr + sni * qi);
        xi_[i] = cs * pi - (snr * qi - sni * qr);
        yr_[i] = (snr * pr - sni * pi) + cs * qr;
        yi_[i] = (snr * pi + sni * pr) + cs * qi;
      }
      else {
        xr_[i] = cs * pr - snr * qr;
        yr_[i] = snr * pr + cs * qr;
      }
    }
  };
  apply(gpr, gpi, gqr, gqi, m);
  apply(Wr + (size_t)p * n, CPLX ? Wi + (size_t)p * n : nullptr, Wr + (size_t)q * n,
        CPLX ? Wi + (size_t)q * n : nullptr, n);
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

static bool copy2d(double *dst, long long ldd, const double *src, long long lds, long long rows, long long cols,
                   cudaStream_t s)
{
  return cudaMemcpy2DAsync(dst, (size_t)ldd * 8, src, (size_t)lds * 8, (size_t)rows * 8, (size_t)cols,
                           cudaMemcpyDeviceToDevice, s) == cudaSuccess;
}

template <bool CPLX>
static vj_fint mixed_dev(vj_fnat m_, vj_fnat n_, double *G, vj_fnat ldG, double *Gi, vj_fnat ldGi, double *V,
                         vj_fnat ldV, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                         unsigned stp, unsigned swp, unsigned stages, cudaStream_t s, unsigned *sweeps32)
{
  const long long m = (long long)m_, n = (long long)n_;
  if (sweeps32)
    *sweeps32 = 0;
  if (!n)
    return 0;
  // the FP64 phase checks the reference's shape rules (src/dvjsvd.c:43-68) itself; they are
  // checked first here too, so that nothing runs on arguments that phase would reject
  if (m_ < n_ || (m % 8))
    return -1;
  if ((n & 1) || ((n >> 1) % 8))
    return -2;
  if (m > 0x3fffffffLL)
    return VJ_ERR_ARG;
  if (!stages)
    stages = 3;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  cublasHandle_t h = cublas();
  if (!h)
    return VJ_ERR_CUDA;
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS)
    return VJ_ERR_CUDA;
  const int P = CPLX ? 2 : 1;
  const size_t mn = (size_t)m * n, nn = (size_t)n * n;
  // scratch: G32 (P m n), W32 (P n n) floats; Gp (P m n), X, T, Y (P n n each) doubles; counters
  const size_t f32b = ((P * (mn + nn) * 4) + 255) & ~(size_t)255;
  const size_t f64b = P * (mn + 3 * nn) * 8;
  host::Staging &stg = host::staging3();
  if (!stg.reserve(f32b + f64b + 256))
    return VJ_ERR_NOMEM;
  float *G32 = reinterpret_cast<float *>(stg.ptr);
  float *W32 = G32 + P * mn;
  double *Gp = reinterpret_cast<double *>(stg.ptr + f32b);
  double *X = Gp + P * mn;
  double *T = X + P * nn;
  double *Y = T + P * nn;
  unsigned long long *cell = reinterpret_cast<unsigned long long *>(Y + P * nn);
  unsigned *cnt = reinterpret_cast<unsigned *>(cell + 1);
  const int ni = (int)n, mi = (int)m;
  const Planes Gpl{G, Gi, (int)ldG, (int)(CPLX ? ldGi : ldG)};
  const Planes Vpl{V, Vi, (int)ldV, (int)(CPLX ? ldVi : ldV)};
  const Planes Xp{X, X + nn, ni, ni}, Tp{T, T + nn, ni, ni}, Yp{Y, Y + nn, ni, ni};
  const Planes Gpp{Gp, Gp + mn, mi, mi};
  // sqrt(m)/2 units of FP32 roundoff (the reference's FP32 tolerance), at least 8 units
  const float tol = fmaxf(0.5f * sqrtf((float)m), 8.f) * 5.9604645e-8f;
  const unsigned maxsw = swp < 60u ? swp : 60u;
  unsigned total32 = 0;
  for (unsigned stage = 0; stage < stages; ++stage) {
    // 1. scale to max |g| in [1/2, 1) and round to FP32
    if (cudaMemsetAsync(cell, 0, 8, s) != cudaSuccess)
      return VJ_ERR_CUDA;
    k_absmax<<<grid2(m, n), 256, 0, s>>>(G, (long long)ldG, m, n, cell);
    if (CPLX)
      k_absmax<<<grid2(m, n), 256, 0, s>>>(Gi, (long long)ldGi, m, n, cell);
    unsigned long long mb = 0;
    if (cudaMemcpyAsync(&mb, cell, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return VJ_ERR_CUDA;
    double amax;
    memcpy(&amax, &mb, 8);
    if (!(amax <= 1.7976931348623157e308))
      return CPLX ? -92 : -80;
    if (amax == 0.0)
      break;
    int e = 0;
    (void)std::frexp(amax, &e);
    k_to_f32<<<grid2(m, n), 256, 0, s>>>(G, (long long)ldG, m, n, -e, G32);
    if (CPLX)
      k_to_f32<<<grid2(m, n), 256, 0, s>>>(Gi, (long long)ldGi, m, n, -e, G32 + mn);
    k_eye_p<float><<<grid2(n, n), 256, 0, s>>>(W32, n, n, 1);
    if (CPLX)
      k_eye_p<float><<<grid2(n, n), 256, 0, s>>>(W32 + nn, n, n, 0);
    // 2. FP32 sweeps until a sweep rotates nothing
    unsigned sw = 0;
    for (; sw < maxsw; ++sw) {
      if (cudaMemsetAsync(cnt, 0, 4, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      for (unsigned st = 0; st < stp; ++st)
        k_presweep<CPLX><<<(unsigned)(n / 2), 256, 0, s>>>(mi, ni, G32, CPLX ? G32 + mn : nullptr, W32,
                                                          CPLX ? W32 + nn : nullptr, js, (int)st, tol, cnt);
      unsigned hc = 0;
      if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&hc, cnt, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
      if (!hc)
        break;
    }
    total32 += sw;
    if (!sw)
      break;  // already orthogonal to the FP32 level: later stages would change nothing
    // 3. W (FP64) with two Newton-Schulz steps: Y = W^H W, T = W Y, W = 1.5 W - 0.5 T
    for (int pl = 0; pl < P; ++pl)
      k_to_f64<<<(unsigned)((nn + 255) / 256 < 4096 ? (nn + 255) / 256 : 4096), 256, 0, s>>>(
          W32 + pl * nn, (long long)nn, X + pl * nn);
    for (int it = 0; it < 2; ++it) {
      if (!zgemm(h, CPLX, true, ni, ni, ni, Xp, Xp, Yp) || !zgemm(h, CPLX, false, ni, ni, ni, Xp, Yp, Tp))
        return VJ_ERR_CUDA;
      const double a15 = 1.5, am05 = -0.5;
      for (int pl = 0; pl < P; ++pl)
        if (cublasDgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, ni, ni, &a15, X + pl * nn, ni, &am05, T + pl * nn, ni,
                        X + pl * nn, ni) != CUBLAS_STATUS_SUCCESS)
          return VJ_ERR_CUDA;
    }
    // 4. G <- G W, V <- V W (V_0 = I, so the first stage that rotates sets V = W)
    if (!copy2d(Gp, m, G, ldG, m, n, s) || (CPLX && !copy2d(Gp + mn, m, Gi, ldGi, m, n, s)))
      return VJ_ERR_CUDA;
    if (!zgemm(h, CPLX, false, mi, ni, ni, Gpp, Xp, Gpl))
      return VJ_ERR_CUDA;
    if (total32 == sw) {
      if (!copy2d(V, ldV, X, n, n, n, s) || (CPLX && !copy2d(Vi, ldVi, X + nn, n, n, n, s)))
        return VJ_ERR_CUDA;
    }
    else {
      if (!copy2d(T, n, V, ldV, n, n, s) || (CPLX && !copy2d(T + nn, n, Vi, ldVi, n, n, s)))
        return VJ_ERR_CUDA;
      if (!zgemm(h, CPLX, false, ni, ni, ni, Tp, Xp, Vpl))
        return VJ_ERR_CUDA;
    }
  }
  if (sweeps32)
    *sweeps32 = total32;
  if (!total32) {
    // nothing was rotated (zero matrix or columns already orthogonal): V := I
    k_eye_p<double><<<grid2(n, n), 256, 0, s>>>(V, (long long)ldV, n, 1);
    if (CPLX)
      k_eye_p<double><<<grid2(n, n), 256, 0, s>>>(Vi, (long long)ldVi, n, 0);
  }
  // 5. FP64 finishing sweeps with V preset
  return svd_dev_entry<double, CPLX>(m_, n_, G, ldG, Gi, ldGi, V, ldV, Vi, ldVi, eS, fS, js, stp, swp, 1, s);
}

}  // namespace vj

extern "C" {

vj_fint vj_dvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS,
                            double *fS, const unsigned *js, unsigned stp, unsigned swp, unsigned stages,
                            unsigned *sweeps32, void *stream)
{
  return vj::mixed_dev<false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp, stages,
                              (cudaStream_t)stream, sweeps32);
}

vj_fint vj_zvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *Gr, vj_fnat ldGr, double *Gi, vj_fnat ldGi, double *Vr,
                            vj_fnat ldVr, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                            unsigned stp, unsigned swp, unsigned stages, unsigned *sweeps32, void *stream)
{
  return vj::mixed_dev<true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, stages,
                             (cudaStream_t)stream, sweeps32);
}

}  // extern "C"
