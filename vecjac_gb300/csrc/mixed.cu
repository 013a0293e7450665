// Mixed-precision one-sided Jacobi SVD: FP32 presweeps, FP64 finishing sweeps.
//
// GB300 runs FP32 arithmetic at about 70 times its FP64 rate, so most of the sweeps are
// done in FP32 and only the last ones in FP64. Starting from G_0 = A (FP64), V_0 = I, each
// preconditioning stage s = 1..S
//   1. rounds G_{s-1} (scaled by a power of two to max |g_ij| <= 1) to FP32;
//   2. runs FP32 one-sided Jacobi sweeps on it from W := I until no pair exceeds the FP32
//      tolerance: block sweeps with split-BF16x3 tensor-core products (blockjac.cu) where
//      n is a whole number of block pairs, else column-pair Hestenes sweeps (k_presweep_reg
//      / k_presweep, rotations from plain FP32 dot products);
//   3. widens W to FP64 and makes it unitary to FP64 accuracy by a Cholesky QR with its
//      columns in ascending order of norm (cuSOLVER's Cholesky, a triangular solve);
//   4. forms G_s = G_{s-1} Q and V_s = V_{s-1} Q (FP64 GEMMs).
// FP32 rounding is relative to each element, so from the second stage on the FP32 sweeps
// see the columns of G_{s-1} to their own relative accuracy and resolve the directions of
// small singular values that the first stage (on A itself) could not. FP64 sweeps with
// plain dot products (the same step kernel in FP64, on G and V themselves, with a scale
// factor per column so that a rotation takes two FMAs per output, and the squared column
// norms tracked through the sweep so that a step forms only the inner product) then bring
// the columns to FP64 orthogonality. Finally dvjsvd_/zvjsvd_'s algorithm runs on G with V as
// the preset matrix (the reference's iwork[0] != 0 mode, src/dvjsvd.c:88-96,
// src/zvjsvd.c:100-110): G R = U Sigma and V R = V, so A = U Sigma V^H with the FP64
// algorithm's accuracy and convergence test; its first sweep is checked for every pair at
// once (jsvd.cu, k_confirm) and skipped when it would transform nothing. The FP64 GEMMs
// are plain library GEMMs (cuBLAS DGEMM; four or three real products per complex one on
// the split planes).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <cstring>
#include <algorithm>
#include <vector>

#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include "presweep.cuh"
#include "svd_core.cuh"
#include "vj_fp.cuh"
#include "vj_host.h"

namespace vj {

// defined in blockjac.cu: block sweeps with split-BF16x3 tensor-core products
bool block_sweeps_apply(bool cplx, long long m, long long n, long long ld);
size_t block_sweep_scratch(bool cplx, long long m, long long n, int inner);
long long block_sweep(bool cplx, int m, int n, float *Gr, float *Gi, long long ldg, float *Wr, float *Wi,
                      long long ldw, unsigned char *scratch, unsigned *stats, float tol, int inner, int terms,
                      cudaStream_t s, float *mu);

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

// Vector of 16 bytes: 4 floats or 2 doubles.
template <typename T> struct vec16;
template <> struct vec16<float> { using V = float4; static constexpr int E = 4; };
template <> struct vec16<double> { using V = double2; static constexpr int E = 2; };

// CTA-wide sums of a, b, cr, ci (up to 512 threads) into thread 0
template <typename T> __device__ void block_sum4(T &a, T &b, T &cr, T &ci, T (*red)[16])
{
  for (int o = 16; o >= 1; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    cr += __shfl_xor_sync(0xffffffffu, cr, o);
    ci += __shfl_xor_sync(0xffffffffu, ci, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = a;
    red[1][w] = b;
    red[2][w] = cr;
    red[3][w] = ci;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = cr = ci = 0;
    for (int j = 0; j < (int)(blockDim.x >> 5); ++j) {
      a += red[0][j];
      b += red[1][j];
      cr += red[2][j];
      ci += red[3][j];
    }
  }
}

// rotate columns (x, y); with swap the rotated y goes to x's place and the rotated x to y's
template <typename T, bool CPLX, bool SHRT>
__device__ void rot_cols_(int rows, T *xr, T *xi, T *yr, T *yi, const Rot<T> &c)
{
  T *dxr = c.swap ? yr : xr, *dxi = c.swap ? yi : xi, *dyr = c.swap ? xr : yr, *dyi = c.swap ? xi : yi;
  Rot<T> k = c;
  k.shrt = SHRT;  // a compile-time form inside the loop
  unscaled_form(k);
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    T pr = xr[i], qr = yr[i], pi = 0, qi = 0;
    if (CPLX) {
      pi = xi[i];
      qi = yi[i];
    }
    rot_elem<T, CPLX>(k, pr, pi, qr, qi);
    dxr[i] = pr;
    dyr[i] = qr;
    if (CPLX) {
      dxi[i] = pi;
      dyi[i] = qi;
    }
  }
}
template <typename T, bool CPLX>
__device__ void rot_cols(int rows, T *xr, T *xi, T *yr, T *yi, const Rot<T> &c)
{
  if (has_scales<T>() && c.shrt)
    rot_cols_<T, CPLX, true>(rows, xr, xi, yr, yi, c);
  else
    rot_cols_<T, CPLX, false>(rows, xr, xi, yr, yi, c);
}

// The same for the register kernels, U rows per thread loaded before any is stored: a
// store may alias a later load as far as the compiler knows, so the loop above waits for one
// memory round trip per row of the thread, which is most of a step at the small sizes the
// register kernels serve (U = 4 real / 2 complex: 1024 x 1024 real FP32 sweeps 92 -> 80 ms).
template <typename T, bool CPLX, bool SHRT, int U>
__device__ void rot_cols_batched_(int rows, T *xr, T *xi, T *yr, T *yi, const Rot<T> &c)
{
  T *dxr = c.swap ? yr : xr, *dxi = c.swap ? yi : xi, *dyr = c.swap ? xr : yr, *dyi = c.swap ? xi : yi;
  Rot<T> k = c;
  k.shrt = SHRT;
  unscaled_form(k);
  const int nt = (int)blockDim.x;
  for (int i0 = threadIdx.x; i0 < rows; i0 += U * nt) {
    T pr[U], qr[U], pi[U], qi[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * nt;
      pr[u] = qr[u] = pi[u] = qi[u] = (T)0;
      if (i < rows) {
        pr[u] = xr[i];
        qr[u] = yr[i];
        if (CPLX) {
          pi[u] = xi[i];
          qi[u] = yi[i];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * nt;
      if (i < rows) {
        rot_elem<T, CPLX>(k, pr[u], pi[u], qr[u], qi[u]);
        dxr[i] = pr[u];
        dyr[i] = qr[u];
        if (CPLX) {
          dxi[i] = pi[u];
          dyi[i] = qi[u];
        }
      }
    }
  }
}
template <typename T, bool CPLX, int U>
__device__ void rot_cols_batched(int rows, T *xr, T *xi, T *yr, T *yi, const Rot<T> &c)
{
  if (has_scales<T>() && c.shrt)
    rot_cols_batched_<T, CPLX, true, U>(rows, xr, xi, yr, yi, c);
  else
    rot_cols_batched_<T, CPLX, false, U>(rows, xr, xi, yr, yi, c);
}

// this thread's share of c = g_p^H g_q and, with NORMS, of |g_p|^2 and |g_q|^2
template <typename T, bool CPLX, bool NORMS>
__device__ __forceinline__ void pair_dots(int m, const T *gpr, const T *gqr, const T *gpi, const T *gqi, T &a, T &b,
                                          T &cr, T &ci)
{
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const T xr = gpr[i], yr = gqr[i];
    if (NORMS) {
      a = fma(xr, xr, a);
      b = fma(yr, yr, b);
    }
    cr = fma(xr, yr, cr);
    if (CPLX) {
      const T xi = gpi[i], yi = gqi[i];
      if (NORMS) {
        a = fma(xi, xi, a);
        b = fma(yi, yi, b);
      }
      cr = fma(xi, yi, cr);
      ci = fma(xr, yi, ci);
      ci = fma(-xi, yr, ci);
    }
  }
}
// One pivot step of one-sided Jacobi (Hestenes) with plain dot products, FP32 or FP64, on
// planar G (m x n) and W (n x n): CTA k takes pair (p, q) = row st of the pivot table,
// forms a = |g_p|^2, b = |g_q|^2, c = g_p^H g_q (per-thread partial sums and a block
// tree) and rotates columns p and q of G and W (hestenes, presweep.cuh). Any m; G is read
// twice. dsc, nrm: the column scales and tracked norms of the FP64 sweeps (Rot and
// tracked_norms, presweep.cuh), or nullptr.
template <typename T, bool CPLX>
__global__ void __launch_bounds__(256) k_presweep(int m, int n, T *Gr, long long ldr, T *Gi, long long ldi, T *Wr,
                                                  long long lwr, T *Wi, long long lwi, const unsigned *js, int st,
                                                  T tol, unsigned *cnt, T *dsc, T *nrm)
{
  __shared__ T red[4][16];
  __shared__ Rot<T> rs;
  pdl_enter();
  const int k = blockIdx.x;
  const unsigned p = js[(size_t)st * n + 2 * k], q = js[(size_t)st * n + 2 * k + 1];
  T *gpr = Gr + (size_t)p * ldr, *gqr = Gr + (size_t)q * ldr;
  T *gpi = CPLX ? Gi + (size_t)p * ldi : nullptr, *gqi = CPLX ? Gi + (size_t)q * ldi : nullptr;
  T nab[2];
  tracked_norms(nrm, p, q, nab);
  const bool norms = nab[0] < (T)0;
  T a = 0, b = 0, cr = 0, ci = 0;
  if (norms)
    pair_dots<T, CPLX, true>(m, gpr, gqr, gpi, gqi, a, b, cr, ci);
  else
    pair_dots<T, CPLX, false>(m, gpr, gqr, gpi, gqi, a, b, cr, ci);
  block_sum4(a, b, cr, ci, red);
  if (threadIdx.x == 0)
    pair_rotation(a, b, cr, ci, tol, cnt, dsc, p, q, &rs, nrm, nab);
  __syncthreads();
  const Rot<T> c = rs;
  if (!c.go)
    return;
  rot_cols<T, CPLX>(m, gpr, gpi, gqr, gqi, c);
  rot_cols<T, CPLX>(n, Wr + (size_t)p * lwr, CPLX ? Wi + (size_t)p * lwi : nullptr, Wr + (size_t)q * lwr,
                    CPLX ? Wi + (size_t)q * lwi : nullptr, c);
}

// the dot products of the register-resident column vectors of k_presweep_reg
template <typename T, bool CPLX, int R, bool NORMS, typename V>
__device__ __forceinline__ void reg_dots(const V (&xr)[R], const V (&yr)[R], const V (&xi)[R], const V (&yi)[R], T &a,
                                         T &b, T &cr, T &ci)
{
  constexpr int E = vec16<T>::E;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const T *X = reinterpret_cast<const T *>(&xr[r]), *Y = reinterpret_cast<const T *>(&yr[r]);
    const T *Xi = reinterpret_cast<const T *>(&xi[r]), *Yi = reinterpret_cast<const T *>(&yi[r]);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (NORMS) {
        a = fma(X[e], X[e], a);
        b = fma(Y[e], Y[e], b);
      }
      cr = fma(X[e], Y[e], cr);
      if (CPLX) {
        if (NORMS) {
          a = fma(Xi[e], Xi[e], a);
          b = fma(Yi[e], Yi[e], b);
        }
        cr = fma(Xi[e], Yi[e], cr);
        ci = fma(X[e], Yi[e], ci);
        ci = fma(-Xi[e], Y[e], ci);
      }
    }
  }
}

// the rotation of the register-resident column vectors of k_presweep_reg, written back
template <typename T, bool CPLX, int R, int NT, bool SHRT, typename V>
__device__ __forceinline__ void rot_regs(V (&xr)[R], V (&yr)[R], V (&xi)[R], V (&yi)[R], int mv, Rot<T> k, V *gpr,
                                         V *gqr, V *gpi, V *gqi)
{
  constexpr int E = vec16<T>::E;
  k.shrt = SHRT;
  unscaled_form(k);
  V *dpr = k.swap ? gqr : gpr, *dqr = k.swap ? gpr : gqr, *dpi = k.swap ? gqi : gpi, *dqi = k.swap ? gpi : gqi;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int i = threadIdx.x + r * NT;
    if (i < mv) {
      T *X = reinterpret_cast<T *>(&xr[r]), *Y = reinterpret_cast<T *>(&yr[r]);
      T *Xi = reinterpret_cast<T *>(&xi[r]), *Yi = reinterpret_cast<T *>(&yi[r]);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        T d0 = 0, d1 = 0;
        rot_elem<T, CPLX>(k, X[e], CPLX ? Xi[e] : d0, Y[e], CPLX ? Yi[e] : d1);
      }
      dpr[i] = xr[r];
      dqr[i] = yr[r];
      if (CPLX) {
        dpi[i] = xi[r];
        dqi[i] = yi[r];
      }
    }
  }
}

// resident CTAs per SM the FP64 register kernels are compiled for: a pivot step of a
// 1024-column matrix is 512 CTAs, one wave on 152 SMs at 4 per SM and two at 3 (at
// 1024 x 1024 real the FP64 sweeps took 61 ms with 4 per SM, 80 ms with 3); 0 (the FP32
// kernels) leaves the compiler's own register choice, as a bound without a minimum does
template <typename T, bool CPLX, int R, int NT> __host__ __device__ constexpr int presweep_min_ctas()
{
  return (sizeof(T) == 8 && NT == 256) ? ((CPLX && R == 2) ? 3 : 4) : 0;
}

// The same step with the two columns of G held in registers between the dot products and
// the rotation (one read and one write of G): thread t of NT owns the 16-byte vectors
// t + NT r, r < R, of each column, so m <= NT R E (E = 4 floats or 2 doubles per vector);
// m % E == 0 and 16-byte aligned columns.
// PW: W's two columns are loaded as 16-byte vectors with G's at the start, and rotated from
// registers (real FP32 data with 16-byte aligned columns of W); otherwise they are read
// after the rotation is known.
template <typename T, bool CPLX, int R, int NT, bool PW = false>
__global__ void __launch_bounds__(NT, presweep_min_ctas<T, CPLX, R, NT>()) k_presweep_reg(int m, int n, T *Gr, long long ldr, T *Gi, long long ldi,
                                                      T *Wr, long long lwr, T *Wi, long long lwi, const unsigned *js,
                                                      int st, T tol, unsigned *cnt, T *dsc, T *nrm)
{
  static_assert(!PW || (!CPLX && sizeof(T) == 4), "W prefetch: real FP32 data");
  using V = typename vec16<T>::V;
  constexpr int E = vec16<T>::E;
  __shared__ T red[4][16];
  __shared__ Rot<T> rs;
  pdl_enter();
  const int k = blockIdx.x;
  const unsigned p = js[(size_t)st * n + 2 * k], q = js[(size_t)st * n + 2 * k + 1];
  V *gpr = reinterpret_cast<V *>(Gr + (size_t)p * ldr), *gqr = reinterpret_cast<V *>(Gr + (size_t)q * ldr);
  V *gpi = CPLX ? reinterpret_cast<V *>(Gi + (size_t)p * ldi) : nullptr;
  V *gqi = CPLX ? reinterpret_cast<V *>(Gi + (size_t)q * ldi) : nullptr;
  const int mv = m / E;
  V xr[R], yr[R], xi[R], yi[R];
  T a = 0, b = 0, cr = 0, ci = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int i = threadIdx.x + r * NT;
    V z;
    T *zz = reinterpret_cast<T *>(&z);
#pragma unroll
    for (int e = 0; e < E; ++e)
      zz[e] = 0;
    xr[r] = (i < mv) ? gpr[i] : z;
    yr[r] = (i < mv) ? gqr[i] : z;
    if (CPLX) {
      xi[r] = (i < mv) ? gpi[i] : z;
      yi[r] = (i < mv) ? gqi[i] : z;
    }
  }
  // W's columns (n <= m rows, so R vectors per thread cover them)
  const int nv = n / E;
  V *wpr = reinterpret_cast<V *>(Wr + (size_t)p * lwr), *wqr = reinterpret_cast<V *>(Wr + (size_t)q * lwr);
  V wp[PW ? R : 1], wq[PW ? R : 1];
  if constexpr (PW) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + r * NT;
      V z;
      T *zz = reinterpret_cast<T *>(&z);
#pragma unroll
      for (int e = 0; e < E; ++e)
        zz[e] = 0;
      wp[r] = (i < nv) ? wpr[i] : z;
      wq[r] = (i < nv) ? wqr[i] : z;
    }
  }
  // (the tracked norms are read after the column loads were issued: their latencies overlap)
  T nab[2];
  tracked_norms(nrm, p, q, nab);
  const bool norms = nab[0] < (T)0;
  if (norms)
    reg_dots<T, CPLX, R, true>(xr, yr, xi, yi, a, b, cr, ci);
  else
    reg_dots<T, CPLX, R, false>(xr, yr, xi, yi, a, b, cr, ci);
  block_sum4(a, b, cr, ci, red);
  if (threadIdx.x == 0)
    pair_rotation(a, b, cr, ci, tol, cnt, dsc, p, q, &rs, nrm, nab);
  __syncthreads();
  const Rot<T> c = rs;
  if (!c.go)
    return;
  if (has_scales<T>() && c.shrt)
    rot_regs<T, CPLX, R, NT, true>(xr, yr, xi, yi, mv, c, gpr, gqr, gpi, gqi);
  else
    rot_regs<T, CPLX, R, NT, false>(xr, yr, xi, yi, mv, c, gpr, gqr, gpi, gqi);
  if constexpr (PW)
    rot_regs<T, CPLX, R, NT, false>(wp, wq, wp, wq, nv, c, wpr, wqr, wpr, wqr);
  else
    rot_cols_batched<T, CPLX, CPLX ? 2 : 4>(n, Wr + (size_t)p * lwr, CPLX ? Wi + (size_t)p * lwi : nullptr,
                                            Wr + (size_t)q * lwr, CPLX ? Wi + (size_t)q * lwi : nullptr, c);
}

static dim3 grid2(long long rows, long long cols)
{
  long long gx = (rows + 255) / 256;
  if (gx > 32)
    gx = 32;
  long long gy = cols < 65535 ? cols : 65535;
  return dim3((unsigned)gx, (unsigned)(gy > 0 ? gy : 1));
}

template <typename T> __global__ void k_fill(T *x, int n, T v)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = v;
}

// columns j of planar G (m x n) and W (n x n) times their scale dsc[j] (those != 1)
template <typename T, bool CPLX>
__global__ void k_apply_scales(int m, int n, T *Gr, long long ldr, T *Gi, long long ldi, T *Wr, long long lwr, T *Wi,
                               long long lwi, const T *dsc)
{
  for (int j = blockIdx.y; j < n; j += gridDim.y) {
    const T d = dsc[j];
    if (d == (T)1)
      continue;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)m + n;
         i += (long long)gridDim.x * blockDim.x) {
      const bool g = i < m;
      const long long r = g ? i : i - m;
      T *pr = g ? Gr + (size_t)j * ldr + r : Wr + (size_t)j * lwr + r;
      *pr *= d;
      if (CPLX) {
        T *pi = g ? Gi + (size_t)j * ldi + r : Wi + (size_t)j * lwi + r;
        *pi *= d;
      }
    }
  }
}

// one sweep of presweep steps (stp launches); returns the number of rotations or < 0, and
// in *mu the largest |cos| of a rotated pair. With dsc (n entries of scratch) the columns
// carry scales during the sweep (Rot, presweep.cuh), multiplied into G and W at its end; with nrm
// (n entries) the squared column norms are tracked through the sweep (tracked_norms).
template <typename T, bool CPLX>
static long long presweep(int m, int n, T *Gr, long long ldr, T *Gi, long long ldi, T *Wr, long long lwr, T *Wi,
                          long long lwi, const unsigned *js, unsigned stp, T tol, unsigned *cnt, cudaStream_t s,
                          float *mu, T *dsc = nullptr, T *nrm = nullptr)
{
  constexpr int E = vec16<T>::E;
  const bool al = !(m % E) && !((ldr * (long long)sizeof(T)) % 16) && !((uintptr_t)Gr % 16) &&
                  (!CPLX || (!((ldi * (long long)sizeof(T)) % 16) && !((uintptr_t)Gi % 16)));
  if (cudaMemsetAsync(cnt, 0, 8, s) != cudaSuccess)
    return -1;
  if (dsc)
    k_fill<T><<<(n + 255) / 256, 256, 0, s>>>(dsc, n, (T)1);
  if (nrm)
    k_fill<T><<<(n + 255) / 256, 256, 0, s>>>(nrm, n, (T)-1);
  const unsigned nb = (unsigned)(n / 2);
  const long long cap = 256LL * E;  // rows per register vector slot
  void (*k)(int, int, T *, long long, T *, long long, T *, long long, T *, long long, const unsigned *, int, T,
            unsigned *, T *, T *) = k_presweep<T, CPLX>;
  int nt = 256;
  // register-resident columns: up to 2 vectors per thread and plane with 256 threads, then
  // (FP32) 2 vectors with 512 threads; beyond that the FP64 kernel's register use would
  // leave too few CTAs per SM to keep the FP64 pipe busy, and the two-pass kernel is
  // faster (measured at 4096x2048)
  if (al && m <= cap)
    k = k_presweep_reg<T, CPLX, 1, 256>;
  else if (al && m <= 2 * cap)
    k = k_presweep_reg<T, CPLX, 2, 256>;
  else if (al && sizeof(T) == 4 && m <= 4 * cap) {
    k = k_presweep_reg<T, CPLX, 2, 512>;
    nt = 512;
  }
  // real FP32 with 16-byte aligned columns of W: the variant that loads W with G
  if constexpr (!CPLX && sizeof(T) == 4) {
    const bool alw = !(n % E) && !((lwr * (long long)sizeof(T)) % 16) && !((uintptr_t)Wr % 16);
    if (alw && al && m <= cap)
      k = k_presweep_reg<T, CPLX, 1, 256, true>;
    else if (alw && al && m <= 2 * cap)
      k = k_presweep_reg<T, CPLX, 2, 256, true>;
    else if (alw && al && m <= 4 * cap)
      k = k_presweep_reg<T, CPLX, 2, 512, true>;
  }
  for (unsigned st = 0; st < stp; ++st)
    if (host::launch_pdl(k, dim3(nb), dim3(nt), 0, s, m, n, Gr, ldr, Gi, ldi, Wr, lwr, Wi, lwi, js, (int)st, tol,
                         cnt, dsc, nrm) != cudaSuccess)
      return -1;
  if (dsc)
    k_apply_scales<T, CPLX><<<grid2(m + n, n), 256, 0, s>>>(m, n, Gr, ldr, Gi, ldi, Wr, lwr, Wi, lwi, dsc);
  unsigned hc[2] = {0u, 0u};
  if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(hc, cnt, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return -1;
  memcpy(mu, &hc[1], 4);
  return (long long)hc[0];
}

// squared 2-norms of the columns of planar G (one CTA per column)
template <bool CPLX>
__global__ void __launch_bounds__(256) k_colnorm2(int m, const double *Gr, long long ldr, const double *Gi,
                                                  long long ldi, double *out)
{
  __shared__ double red[8];
  const int j = blockIdx.x;
  double a = 0;
  for (int i = threadIdx.x; i < m; i += 256) {
    const double x = Gr[(size_t)j * ldr + i];
    a = fma(x, x, a);
    if (CPLX) {
      const double y = Gi[(size_t)j * ldi + i];
      a = fma(y, y, a);
    }
  }
  for (int o = 16; o >= 1; o >>= 1)
    a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0)
    red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    a = 0;
    for (int w = 0; w < 8; ++w)
      a += red[w];
    out[j] = a;
  }
}

// B[:, j] = A[:, perm[j]] (rows x n, B with leading dimension rows)
__global__ void k_gather_cols(int rows, int n, const double *A, long long lda, const int *perm, double *B)
{
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x)
      B[(size_t)j * rows + i] = A[(size_t)perm[j] * lda + i];
}

// library handles, one per device (created with that device current)
static cublasHandle_t cublas()
{
  static std::mutex mu;
  static cublasHandle_t hs[host::MAX_DEVICES] = {};
  std::lock_guard<std::mutex> lk(mu);
  cublasHandle_t &h = hs[host::device_slot()];
  if (!h && cublasCreate(&h) != CUBLAS_STATUS_SUCCESS)
    h = nullptr;
  return h;
}

static cusolverDnHandle_t cusolver()
{
  static std::mutex mu;
  static cusolverDnHandle_t hs[host::MAX_DEVICES] = {};
  std::lock_guard<std::mutex> lk(mu);
  cusolverDnHandle_t &h = hs[host::device_slot()];
  if (!h && cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS)
    h = nullptr;
  return h;
}

// squared 2-norms of the columns of planar FP32 G (one CTA per column): the order key of
// the orthonormalisation below
template <bool CPLX>
__global__ void __launch_bounds__(256) k_colnorm2_f32(int m, const float *Gr, const float *Gi, double *out)
{
  __shared__ double red[8];
  const int j = blockIdx.x;
  double a = 0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const double x = Gr[(size_t)j * m + i];
    a = fma(x, x, a);
    if (CPLX) {
      const double y = Gi[(size_t)j * m + i];
      a = fma(y, y, a);
    }
  }
  for (int o = 16; o >= 1; o >>= 1)
    a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0)
    red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    a = 0;
    for (int w = 0; w < 8; ++w)
      a += red[w];
    out[j] = a;
  }
}

// planar (re, im) n x n <-> interleaved complex n x n (both with leading dimension n)
__global__ void k_to_interleaved(const double *re, const double *im, long long nn, double2 *z)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x)
    z[i] = make_double2(re[i], im[i]);
}
__global__ void k_from_interleaved(const double2 *z, long long nn, double *re, double *im)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
    re[i] = z[i].x;
    im[i] = z[i].y;
  }
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

// T(r, c) = T(c, r) for r < c (fill the upper triangle of an n x n matrix from the lower)
__global__ void k_sym_lower(double *Tm, int n)
{
  for (int c = blockIdx.y; c < n; c += gridDim.y)
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < c; r += gridDim.x * blockDim.x)
      Tm[(size_t)c * n + r] = Tm[(size_t)r * n + c];
}

// D(r, c) = M(r, c) - M(c, r) (n x n)
__global__ void k_antisym(const double *M, int n, double *D)
{
  for (int c = blockIdx.y; c < n; c += gridDim.y)
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
      D[(size_t)c * n + r] = M[(size_t)c * n + r] - M[(size_t)r * n + c];
}

// 3M combination: Cr holds P1 = Ar Br, Ci holds P3 = (Ar + Ai)(Br + Bi), P2 = Ai Bi:
// Cr = P1 - P2, Ci = P3 - P1 - P2 (rows x cols, leading dimensions ldr / ldi / rows)
__global__ void k_combine3m(int rows, int cols, double *Cr, long long ldr, double *Ci, long long ldi, const double *P2)
{
  for (int c = blockIdx.y; c < cols; c += gridDim.y)
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
      const double p1 = Cr[(size_t)c * ldr + r], p2 = P2[(size_t)c * rows + r], p3 = Ci[(size_t)c * ldi + r];
      Cr[(size_t)c * ldr + r] = p1 - p2;
      Ci[(size_t)c * ldi + r] = (p3 - p1) - p2;
    }
}

// T = X^H X for an n x n split-plane X (leading dimension n): the real part by two
// symmetric rank-k updates (half a product each), the imaginary part from one product
// M = Xr^T Xi as M - M^T. tmp: n x n doubles.
static bool gram(cublasHandle_t h, bool cplx, int n, Planes X, Planes Tm, double *tmp, cudaStream_t s)
{
  const double one = 1.0, zero = 0.0;
  if (cublasDsyrk(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, n, n, &one, X.re, X.ldr, &zero, Tm.re, n) !=
      CUBLAS_STATUS_SUCCESS)
    return false;
  if (cplx) {
    if (cublasDsyrk(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, n, n, &one, X.im, X.ldi, &one, Tm.re, n) !=
            CUBLAS_STATUS_SUCCESS ||
        cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &one, X.re, X.ldr, X.im, X.ldi, &zero, tmp, n) !=
            CUBLAS_STATUS_SUCCESS)
      return false;
    k_antisym<<<grid2(n, n), 256, 0, s>>>(tmp, n, Tm.im);
  }
  k_sym_lower<<<grid2(n, n), 256, 0, s>>>(Tm.re, n);
  return cudaGetLastError() == cudaSuccess;
}

// C = A B for complex split planes with three real products (Gauss / 3M): P1 = Ar Br,
// P2 = Ai Bi, P3 = (Ar + Ai)(Br + Bi). Used for products of near-unitary n x n matrices
// (rotation accumulators), where its slightly larger error bound is harmless. tmp: room
// for m k + k n + m n doubles. Real data: one product.
static bool zgemm3m(cublasHandle_t h, bool cplx, int m, int n, int k, Planes A, Planes B, Planes Cm, double *tmp,
                    cudaStream_t s)
{
  const double one = 1.0, zero = 0.0;
  if (!cplx)
    return cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A.re, A.ldr, B.re, B.ldr, &zero, Cm.re, Cm.ldr) ==
           CUBLAS_STATUS_SUCCESS;
  double *As = tmp, *Bs = As + (size_t)m * k, *P2 = Bs + (size_t)k * n;
  bool ok = cublasDgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, m, k, &one, A.re, A.ldr, &one, A.im, A.ldi, As, m) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, k, n, &one, B.re, B.ldr, &one, B.im, B.ldi, Bs, k) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A.re, A.ldr, B.re, B.ldr, &zero, Cm.re, Cm.ldr) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A.im, A.ldi, B.im, B.ldi, &zero, P2, m) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, As, m, Bs, k, &zero, Cm.im, Cm.ldi) ==
                CUBLAS_STATUS_SUCCESS;
  if (!ok)
    return false;
  k_combine3m<<<grid2(m, n), 256, 0, s>>>(m, n, Cm.re, Cm.ldr, Cm.im, Cm.ldi, P2);
  return cudaGetLastError() == cudaSuccess;
}

// C = A B for complex split planes by 3M as above, with A's imaginary plane overwritten by
// Ar + Ai (A is a scratch copy) so that the temporaries are only P2 (m n) and Br + Bi (k n):
// tmp holds m n + k n doubles. For G := G Q (m x n by n x n): three products instead of four.
static bool zgemm3m_overwrite(cublasHandle_t h, int m, int n, int k, Planes A, Planes B, Planes Cm, double *tmp,
                              cudaStream_t s)
{
  const double one = 1.0, zero = 0.0;
  double *P2 = tmp, *Bs = tmp + (size_t)m * n;
  bool ok = cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A.im, A.ldi, B.im, B.ldi, &zero, P2, m) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, k, n, &one, B.re, B.ldr, &one, B.im, B.ldi, Bs, k) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, m, k, &one, A.re, A.ldr, &one, A.im, A.ldi, A.im, A.ldi) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A.re, A.ldr, B.re, B.ldr, &zero, Cm.re, Cm.ldr) ==
                CUBLAS_STATUS_SUCCESS &&
            cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A.im, A.ldi, Bs, k, &zero, Cm.im, Cm.ldi) ==
                CUBLAS_STATUS_SUCCESS;
  if (!ok)
    return false;
  k_combine3m<<<grid2(m, n), 256, 0, s>>>(m, n, Cm.re, Cm.ldr, Cm.im, Cm.ldi, P2);
  return cudaGetLastError() == cudaSuccess;
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
                         unsigned stp, unsigned swp, unsigned stages, cudaStream_t s, unsigned *presweeps)
{
  const host::NearestRounding rn;
  const long long m = (long long)m_, n = (long long)n_;
  if (presweeps)
    presweeps[0] = presweeps[1] = 0;
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
    stages = 2;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  cublasHandle_t h = cublas();
  if (!h)
    return VJ_ERR_CUDA;
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS)
    return VJ_ERR_CUDA;
  const int P = CPLX ? 2 : 1;
  const size_t mn = (size_t)m * n, nn = (size_t)n * n;
  // scratch: G32 (P m n), W32 (P n n) floats; Gp, X, T, Y (P n n each) doubles; counters
  const size_t f32b = ((P * (mn + nn) * 4) + 255) & ~(size_t)255;
  // Gp: the copy of G for G W (P m n doubles), earlier the temporaries of the 3M products
  // (3 n n doubles)
  const size_t gpn = ((size_t)P * mn > 3 * nn) ? (size_t)P * mn : 3 * nn;
  const size_t f64b = (gpn + P * 3 * nn) * 8;
  // FP32 stages: block sweeps on the tensor cores where the shape has whole blocks and at
  // least 16 block pairs per step (fewer pairs leave most SMs idle in the pair
  // eigenproblems: at 1024 x 1024 real the column-pair sweeps take 109 ms against 176 ms,
  // at 4096 x 2048 real the block sweeps 495 ms against 685 ms). VJ_BLOCK=0 in the
  // environment selects the column-pair sweeps, VJ_BLOCK=1 the block sweeps wherever the
  // shape allows; VJ_BLOCK_TERMS (6 or 3) the terms of the split products, VJ_BLOCK_INNER
  // the inner Jacobi sweeps per block pair.
  const char *eb = getenv("VJ_BLOCK");
  const bool blk = !(eb && *eb == '0') && block_sweeps_apply(CPLX, m, n, m) &&
                   ((eb && *eb == '1') || n >= (CPLX ? 1024 : 2048));
  const char *et = getenv("VJ_BLOCK_TERMS");
  const int terms = (et && atoi(et) == 3) ? 3 : 6;
  const char *ei = getenv("VJ_BLOCK_INNER");
  const int inner = (ei && atoi(ei) >= 1 && atoi(ei) <= 8) ? atoi(ei) : 1;
  const size_t blkb = blk ? ((block_sweep_scratch(CPLX, m, n, inner) + 255) & ~(size_t)255) : 0;
  host::Staging &stg = host::staging3();
  if (!stg.reserve(f32b + f64b + 256 + blkb))
    return VJ_ERR_NOMEM;
  unsigned char *bscr = reinterpret_cast<unsigned char *>(stg.ptr) + f32b + f64b + 256;
  float *G32 = reinterpret_cast<float *>(stg.ptr);
  float *W32 = G32 + P * mn;
  double *Gp = reinterpret_cast<double *>(stg.ptr + f32b);
  double *X = Gp + gpn;
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
  // the wall-clock time of each phase is kept for vj_last_mixed_phases (every phase ends
  // with a stream synchronisation, so host time is device time here); with VJ_TRACE=1 it
  // also goes to stderr
  const bool trace = host::trace_enabled();
  auto now = [] { return std::chrono::steady_clock::now(); };
  auto t0 = now();
  double ms32 = 0, msgemm = 0;
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
    // (a sweep whose rotated pairs were all within 4x the tolerance ends the stage without
    // a confirming sweep: the stage is a preconditioner, the next one finishes the work;
    // a stage that another one follows also ends once a sweep rotates fewer than half of
    // all possible pairs: the first stage works on A rounded to FP32, where the directions
    // of singular values below FP32 resolution are noise that the next stage resolves
    // properly, and its long tail of sweeps over them costs more than the next stage's
    // extra sweeps -- at 4096 x 2048 complex, 31 + 16 FP32 sweeps in 2.58 s against
    // 18 + 18 in 2.47 s)
    unsigned sw = 0;
    const float stop = 4.f * tol;
    const long long nbk = n / (CPLX ? 32 : 64), hw = CPLX ? 32 : 64;
    const double every = blk ? (double)(nbk - 1) * (double)(nbk / 2) * inner * (double)(2 * hw - 1) * (double)hw
                             : (double)stp * (double)(n / 2);
    for (; sw < maxsw; ++sw) {
      float mu = 0.f;
      const long long hc =
          blk ? block_sweep(CPLX, mi, ni, G32, CPLX ? G32 + mn : nullptr, m, W32, CPLX ? W32 + nn : nullptr, n, bscr,
                            cnt, tol, inner, terms, s, &mu)
              : presweep<float, CPLX>(mi, ni, G32, m, CPLX ? G32 + mn : nullptr, m, W32, n, CPLX ? W32 + nn : nullptr,
                                      n, js, stp, tol, cnt, s, &mu);
      if (hc < 0)
        return VJ_ERR_CUDA;
      if (trace)
        std::fprintf(stderr, "mixed SVD stage %u sweep %u: %lld rotations, max scaled |h_pq| %.3e\n", stage, sw, hc,
                     (double)mu);
      if (!hc)
        break;
      if (mu < stop || (stage + 1 < stages && 2.0 * (double)hc < every)) {
        ++sw;
        break;
      }
    }
    if (trace)
      std::fprintf(stderr, "mixed SVD stage %u: %u FP32 sweeps\n", stage, sw);
    total32 += sw;
    {
      const auto t1 = now();
      ms32 += std::chrono::duration<double, std::milli>(t1 - t0).count();
      t0 = t1;
    }
    if (!sw)
      break;  // already orthogonal to the FP32 level: later stages would change nothing
    // 3. W (FP64) made unitary by one Cholesky QR, Q = W R^-1 with R^H R = W^H W (a Gram
    //    product, cuSOLVER's Cholesky factorisation, a triangular solve): W^H W is within
    //    1e-4 of I after the FP32 stage, so one pass is unitary to FP64 accuracy, at about
    //    half the cost of the two Newton-Schulz steps that the same accuracy needs. W's
    //    columns go in ascending order of the norms of the FP32 G's columns first: R^-1 is
    //    upper triangular, so the correction mixes into each column of G Q only columns of
    //    smaller norm. (The first FP64 sweep below still meets scaled inner products of up
    //    to ~5e-3 at 4096 x 2048 complex with sigma down to 1e-8, and 2e-5 at 4096 x 2048 real
    //    with sigma down to 1e-6: the FP32 rounding of W's own entries couples large columns
    //    of G into small ones, which no orthonormalisation of W undoes; the descending order
    //    measured worse, 1e-2 and 1.5e-4, and one FP64 sweep more at 4096 x 2048 complex.)
    for (int pl = 0; pl < P; ++pl)
      k_to_f64<<<(unsigned)((nn + 255) / 256 < 4096 ? (nn + 255) / 256 : 4096), 256, 0, s>>>(
          W32 + pl * nn, (long long)nn, X + pl * nn);
    {
      double *nrm = Y;  // n entries of scratch, free until the Gram product below
      int *perm = reinterpret_cast<int *>(Y + n);
      k_colnorm2_f32<CPLX><<<(unsigned)n, 256, 0, s>>>(mi, G32, CPLX ? G32 + mn : nullptr, nrm);
      std::vector<double> hn((size_t)n);
      std::vector<int> hp((size_t)n);
      if (cudaMemcpyAsync(hn.data(), nrm, (size_t)n * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
      for (int j = 0; j < ni; ++j)
        hp[(size_t)j] = j;
      std::stable_sort(hp.begin(), hp.end(), [&](int x, int y) { return hn[(size_t)x] < hn[(size_t)y]; });
      if (cudaMemcpyAsync(perm, hp.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      // T := W with its columns permuted (the copy reads the host vector: wait for it)
      for (int pl = 0; pl < P; ++pl)
        k_gather_cols<<<grid2(n, n), 256, 0, s>>>(ni, ni, X + pl * nn, n, perm, T + pl * nn);
      if (cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
    }
    if (!gram(h, CPLX, ni, Tp, Yp, Gp, s))
      return VJ_ERR_CUDA;
    {
      cusolverDnHandle_t hs = cusolver();
      if (!hs || cusolverDnSetStream(hs, s) != CUSOLVER_STATUS_SUCCESS)
        return VJ_ERR_CUDA;
      int *info = reinterpret_cast<int *>(cell);
      static host::Staging wsps[host::MAX_DEVICES];  // the factorisation's workspace, per device
      host::Staging &wsp = wsps[host::device_slot()];
      const double one = 1.0;
      int lw = 0, hinfo = 0;
      if (!CPLX) {
        // R overwrites the upper triangle of Y; T := T R^-1
        if (cusolverDnDpotrf_bufferSize(hs, CUBLAS_FILL_MODE_UPPER, ni, Y, ni, &lw) != CUSOLVER_STATUS_SUCCESS ||
            !wsp.reserve((size_t)(lw > 0 ? lw : 1) * 8) ||
            cusolverDnDpotrf(hs, CUBLAS_FILL_MODE_UPPER, ni, Y, ni, reinterpret_cast<double *>(wsp.ptr), lw, info) !=
                CUSOLVER_STATUS_SUCCESS ||
            cublasDtrsm(h, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, ni, ni, &one,
                        Y, ni, T, ni) != CUBLAS_STATUS_SUCCESS)
          return VJ_ERR_CUDA;
      }
      else {
        // interleaved copies for the complex factorisation: Z = W^H W (in Gp), Xz = W (in Y)
        cuDoubleComplex *Z = reinterpret_cast<cuDoubleComplex *>(Gp);
        cuDoubleComplex *Xz = reinterpret_cast<cuDoubleComplex *>(Y);
        const unsigned g1 = (unsigned)((nn + 255) / 256 < 4096 ? (nn + 255) / 256 : 4096);
        k_to_interleaved<<<g1, 256, 0, s>>>(Y, Y + nn, (long long)nn, reinterpret_cast<double2 *>(Z));
        k_to_interleaved<<<g1, 256, 0, s>>>(T, T + nn, (long long)nn, reinterpret_cast<double2 *>(Xz));
        const cuDoubleComplex zone = make_cuDoubleComplex(1.0, 0.0);
        if (cusolverDnZpotrf_bufferSize(hs, CUBLAS_FILL_MODE_UPPER, ni, Z, ni, &lw) != CUSOLVER_STATUS_SUCCESS ||
            !wsp.reserve((size_t)(lw > 0 ? lw : 1) * 16) ||
            cusolverDnZpotrf(hs, CUBLAS_FILL_MODE_UPPER, ni, Z, ni, reinterpret_cast<cuDoubleComplex *>(wsp.ptr), lw,
                             info) != CUSOLVER_STATUS_SUCCESS ||
            cublasZtrsm(h, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, ni, ni, &zone,
                        Z, ni, Xz, ni) != CUBLAS_STATUS_SUCCESS)
          return VJ_ERR_CUDA;
        k_from_interleaved<<<g1, 256, 0, s>>>(reinterpret_cast<const double2 *>(Xz), (long long)nn, T, T + nn);
      }
      if (cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
      if (hinfo != 0)
        return VJ_ERR_CUDA;  // W^H W not positive definite: W was not near unitary
      // Q (in T) becomes the stage's transformation X
      for (int pl = 0; pl < P; ++pl)
        if (!copy2d(X + pl * nn, n, T + pl * nn, n, n, n, s))
          return VJ_ERR_CUDA;
      if (trace)
        std::fprintf(stderr, "mixed SVD stage %u: Cholesky QR of W\n", stage);
    }
    // 4. V <- V W (V_0 = I, so the first stage that rotates sets V = W), G <- G W
    if (total32 == sw) {
      if (!copy2d(V, ldV, X, n, n, n, s) || (CPLX && !copy2d(Vi, ldVi, X + nn, n, n, n, s)))
        return VJ_ERR_CUDA;
    }
    else {
      if (!copy2d(T, n, V, ldV, n, n, s) || (CPLX && !copy2d(T + nn, n, Vi, ldVi, n, n, s)))
        return VJ_ERR_CUDA;
      if (!zgemm3m(h, CPLX, ni, ni, ni, Tp, Xp, Vpl, Gp, s))
        return VJ_ERR_CUDA;
    }
    if (!copy2d(Gp, m, G, ldG, m, n, s) || (CPLX && !copy2d(Gp + mn, m, Gi, ldGi, m, n, s)))
      return VJ_ERR_CUDA;
    // complex G := G Q by 3M when its temporaries fit in the free T and Y scratch
    // (m n + n n <= 4 n n doubles), else by four real products
    if (CPLX && m <= 3 * n) {
      if (!zgemm3m_overwrite(h, mi, ni, ni, Gpp, Xp, Gpl, T, s))
        return VJ_ERR_CUDA;
    }
    else if (!zgemm(h, CPLX, false, mi, ni, ni, Gpp, Xp, Gpl))
      return VJ_ERR_CUDA;
    {
      if (cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
      const auto t1 = now();
      msgemm += std::chrono::duration<double, std::milli>(t1 - t0).count();
      t0 = t1;
    }
  }
  if (presweeps)
    presweeps[0] = total32;
  if (!total32) {
    // nothing was rotated (zero matrix or columns already orthogonal): V := I
    k_eye_p<double><<<grid2(n, n), 256, 0, s>>>(V, (long long)ldV, n, 1);
    if (CPLX)
      k_eye_p<double><<<grid2(n, n), 256, 0, s>>>(Vi, (long long)ldVi, n, 0);
  }
  // 5. FP64 sweeps with plain dot products on G and V themselves until no pair reaches half
  //    the reference's tolerance sqrt(m) eps / 2 (at most 20 sweeps): they take the columns from
  //    FP32 to FP64 orthogonality at a fraction of a reference sweep's cost (4 FP64
  //    operations per complex element of G for the inner product with tracked norms and 8
  //    for the rotation in the short form of Rot, instead of 68), so the reference's sweeps below
  //    have at most the last rotations to do and the convergence to confirm.
  if (total32) {
    // half the reference's tolerance: the plain dot product's rounding (a few eps) stays
    // well below it, and pairs the reference would still rotate are rotated here
    const double tol64 = 0.5 * std::sqrt((double)m) * 1.1102230246251565e-16;
    const unsigned maxsw64 = swp < 20u ? swp : 20u;
    unsigned sw64 = 0;
    // A sweep whose rotated pairs all had |cos| <= 1e-11 leaves off-diagonal terms of the
    // order of their squares (times n / relative gap), far below the tolerance: its
    // confirming sweep is skipped, the reference's sweep below confirms.
    for (; sw64 < maxsw64; ++sw64) {
      float mu = 0.f;
      // (column scales and tracked norms in Y, free scratch until the sort below)
      const long long hc = presweep<double, CPLX>(mi, ni, G, (long long)ldG, Gi, (long long)(CPLX ? ldGi : ldG), V,
                                                  (long long)ldV, Vi, (long long)(CPLX ? ldVi : ldV), js, stp, tol64,
                                                  cnt, s, &mu, Y, Y + n);
      if (hc < 0)
        return VJ_ERR_CUDA;
      if (trace)
        std::fprintf(stderr, "mixed SVD FP64 sweep %u: %lld rotations, max |cos| %.3e, %.1f ms since the phase began\n",
                     sw64, hc, (double)mu, std::chrono::duration<double, std::milli>(now() - t0).count());
      if (!hc)
        break;
      if (mu <= 1e-11f) {
        ++sw64;
        break;
      }
    }
    if (presweeps)
      presweeps[1] = sw64;
    // columns in descending order of their norms, the order the reference's sweeps keep
    // (src/dvjsvd.c:367-370): its sweeps then have no pair to reorder
    double *nrm = T;  // n entries of scratch
    int *perm = reinterpret_cast<int *>(T + n);
    k_colnorm2<CPLX><<<(unsigned)n, 256, 0, s>>>(mi, G, (long long)ldG, Gi, (long long)(CPLX ? ldGi : ldG), nrm);
    std::vector<double> hn((size_t)n);
    std::vector<int> hp((size_t)n);
    if (cudaMemcpyAsync(hn.data(), nrm, (size_t)n * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return VJ_ERR_CUDA;
    for (int j = 0; j < ni; ++j)
      hp[(size_t)j] = j;
    std::stable_sort(hp.begin(), hp.end(), [&](int x, int y) { return hn[(size_t)x] > hn[(size_t)y]; });
    bool moved = false;
    for (int j = 0; j < ni && !moved; ++j)
      moved = (hp[(size_t)j] != j);
    if (moved) {
      if (cudaMemcpyAsync(perm, hp.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      for (int pl = 0; pl < P; ++pl) {
        double *Gd = pl ? Gi : G, *Vd = pl ? Vi : V;
        const long long lg = pl ? (long long)ldGi : (long long)ldG, lv = pl ? (long long)ldVi : (long long)ldV;
        k_gather_cols<<<grid2(m, n), 256, 0, s>>>(mi, ni, Gd, lg, perm, Gp);
        k_gather_cols<<<grid2(n, n), 256, 0, s>>>(ni, ni, Vd, lv, perm, Y);
        if (!copy2d(Gd, lg, Gp, m, m, n, s) || !copy2d(Vd, lv, Y, n, n, n, s))
          return VJ_ERR_CUDA;
      }
      // the host vectors are read by the copy above: wait before they go out of scope
      if (cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
    }
  }
  double ms64 = 0;
  {
    const auto t1 = now();
    ms64 = std::chrono::duration<double, std::milli>(t1 - t0).count();
    t0 = t1;
  }
  // 6. FP64 finishing sweeps (the reference's algorithm) with V preset
  const vj_fint r = svd_dev_entry<double, CPLX>(m_, n_, G, ldG, Gi, ldGi, V, ldV, Vi, ldVi, eS, fS, js, stp, swp, 2, s);
  const double msfin = std::chrono::duration<double, std::milli>(now() - t0).count();
  // FP32 launches: 5 per block step (Gram, its reduction, the pair eigenproblems, R, the
  // rotation; n/b - 1 steps per block sweep), else 1 per pivot step
  const double steps32 = blk ? (double)total32 * (double)(n / (CPLX ? 32 : 64) - 1) * 5.0 : (double)total32 * stp;
  host::mixed_phases_set(ms32, msgemm, ms64, msfin, steps32, blk ? 1.0 : 0.0);
  if (trace)
    std::fprintf(stderr, "mixed SVD phases (ms): FP32 sweeps %.1f, Newton-Schulz + GEMMs %.1f, plain FP64 sweeps + sort %.1f, "
                 "finishing %.1f\n", ms32, msgemm, ms64, msfin);
  return r;
}

}  // namespace vj

extern "C" {

vj_fint vj_dvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS,
                            double *fS, const unsigned *js, unsigned stp, unsigned swp, unsigned stages,
                            unsigned *presweeps, void *stream)
{
  return vj::mixed_dev<false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp, stages,
                              (cudaStream_t)stream, presweeps);
}

vj_fint vj_zvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *Gr, vj_fnat ldGr, double *Gi, vj_fnat ldGi, double *Vr,
                            vj_fnat ldVr, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                            unsigned stp, unsigned swp, unsigned stages, unsigned *presweeps, void *stream)
{
  return vj::mixed_dev<true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, stages,
                             (cudaStream_t)stream, presweeps);
}

}  // extern "C"
