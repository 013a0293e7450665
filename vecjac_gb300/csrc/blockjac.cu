// Block one-sided Jacobi sweeps in FP32 with the block rotations on the tensor cores
// (split-BF16x3 products, FP32 accumulation): the FP32 stages of the mixed-precision SVD.
//
// The n columns of the FP32 matrix G (m x n, split real/imaginary planes) and of the
// rotation accumulator W (n x n) are cut into blocks of b columns (b = 64 real, 32
// complex, so that a block pair is 128 real columns: [G_I G_J], or [Re G_I Re G_J Im G_I
// Im G_J]). A block sweep visits every pair of blocks once in the round-robin order, n/b/2
// independent pairs per block step, and for each pair
//   1. k_gram:  S = X^T X, the real Gram matrix of the pair's 128 real columns X (128 x 128,
//      K = m, split over several CTAs), on the tensor cores (its symmetry halves the cross
//      terms of the split products), and k_gram_reduce: the sum over the K splits;
//   2. k_pair_evd: the Hermitian Gram matrix H = [G_I G_J]^H [G_I G_J] (from S), one cyclic
//      two-sided Jacobi sweep on H -- in exact arithmetic the rotations of one-sided Jacobi
//      on the pair's columns, from the same 2x2 Gram blocks, with the same threshold --
//      with its rotations logged, and the order of descending norms (the block form of the
//      scalar sweep's swap rule); k_build_r: the unitary R (2b x 2b) as the product of the
//      logged rotations, its columns in that order, and R's split image;
//   3. k_apply: [G_I G_J] := [G_I G_J] R and [W_I W_J] := [W_I W_J] R on the tensor cores
//      (the real 128 x 128 form of R for complex data: [[Re R, Im R], [-Im R, Re R]]).
// Each FP32 operand x is split into three BF16 terms x = h + m + l (exactly: 8 + 8 + 8
// significant bits) and a product is formed from the six terms h h, h m, m h, h l, m m,
// l h (the dropped ones are below 2^-24 relative), accumulated in FP32 in TMEM: the
// accuracy of an FP32 product at tensor-core speed. Operands are converted from FP32 to
// the split BF16 tiles by the CTA's threads (the A side) or copied by the bulk-copy TMA
// engine from the split image that k_build_r writes (the R side of k_apply).
#include <cuda_bf16.h>
#include <type_traits>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "svd_core.cuh"
#include "tc.cuh"
#include "vj_host.h"

namespace vj {
namespace bj {

constexpr int TILE = 128;                 // real columns of a block pair = rows of a GEMM tile
constexpr int KC = 64;                    // K elements of one operand stage
constexpr int LBO = 128;                  // bytes between core matrices adjacent in K
constexpr int SBO = (KC / 8) * 128;       // bytes between groups of 8 rows
constexpr int PLANE = TILE * KC * 2;      // bytes of one BF16 term of a 128 x 64 stage tile
constexpr uint32_t IDESC = tc::idesc_bf16<TILE, TILE>::value;
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz: a wait that long has failed

// terms of the split product, smallest first: (A term, B term), 0 = h, 1 = m, 2 = l
__constant__ int TA[6] = {2, 1, 0, 1, 0, 0};
__constant__ int TB[6] = {0, 1, 2, 0, 1, 0};

// byte offset of element (row r, k) in a K-major tile without swizzle
__device__ __forceinline__ int tile_off(int r, int k)
{
  return (r >> 3) * SBO + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2;
}

// x = h + m + l exactly, each a BF16 (for FP32 inputs of normal or zero magnitude), two
// values at a time: cvt.rn.bf16x2.f32 rounds a pair into one 32-bit word, and a BF16 back to
// FP32 is its bits shifted up by 16
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}
__device__ __forceinline__ void split3x2(float x0, float x1, uint32_t &h, uint32_t &m, uint32_t &l)
{
  h = pack_bf16x2(x0, x1);
  const float r0 = x0 - __uint_as_float(h << 16), r1 = x1 - __uint_as_float(h & 0xFFFF0000u);
  m = pack_bf16x2(r0, r1);
  const float s0 = r0 - __uint_as_float(m << 16), s1 = r1 - __uint_as_float(m & 0xFFFF0000u);
  l = pack_bf16x2(s0, s1);
}

// the three BF16 terms of 8 values, stored as 16 bytes each at p0, p0 + PLANE, p0 + 2 PLANE
__device__ __forceinline__ void store_split8(unsigned char *p0, const float (&v)[8])
{
  uint4 h, m, l;
  split3x2(v[0], v[1], h.x, m.x, l.x);
  split3x2(v[2], v[3], h.y, m.y, l.y);
  split3x2(v[4], v[5], h.z, m.z, l.z);
  split3x2(v[6], v[7], h.w, m.w, l.w);
  *reinterpret_cast<uint4 *>(p0) = h;
  *reinterpret_cast<uint4 *>(p0 + PLANE) = m;
  *reinterpret_cast<uint4 *>(p0 + 2 * PLANE) = l;
}

// planar FP32 matrix and the block layout of its columns
struct Cols {
  float *re, *im;  // im == nullptr for real data
  long long ld;
  int b;  // columns per block: 64 (real) or 32 (complex)
};

// real column c (0..127) of the block pair (I, J): complex data put the real parts of the
// pair's 2b columns first, then their imaginary parts
__device__ __forceinline__ float *pair_col(const Cols &X, int I, int J, int c)
{
  const bool cx = X.im != nullptr;
  const int h = cx ? (c & 63) : c;
  float *base = (cx && c >= 64) ? X.im : X.re;
  const int col = (h < X.b) ? (I * X.b + h) : (J * X.b + (h - X.b));
  return base + (long long)col * X.ld;
}

// block pair k of block step s of the round-robin ordering of nb blocks (I < J)
__device__ __forceinline__ void block_pair(int nb, int s, int k, int &I, int &J)
{
  const int N = nb - 1;
  int a, c;
  if (k == 0) {
    a = s;
    c = N;
  }
  else {
    a = (s + k) % N;
    c = (s + N - k) % N;
  }
  I = a < c ? a : c;
  J = a < c ? c : a;
}

// ---------------------------------------------------------------- Gram matrices
// CTA (pair, split): S_part = X[k0:k1]^T X[k0:k1] for the pair's 128 real columns, rows
// k0..k1 of this split. 128 threads: thread t converts real column t (the next chunk's 64
// values are loaded into registers while the current one is split and stored); thread 0
// issues the MMAs. Two operand stages (A = B: the Gram tile is its own B operand), 96 KiB.
template <int NT>
__global__ void __launch_bounds__(128) k_gram(Cols X, int m, int nb, int step, int ksplit, float *Spart,
                                               unsigned *err)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024u - (tc::saddr(smem_raw) & 1023u)) & 1023u);
  __shared__ unsigned long long bar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int pair = blockIdx.x / ksplit, ks = blockIdx.x % ksplit;
  int I, J;
  block_pair(nb, step, pair, I, J);
  const int nch_all = (m + KC - 1) / KC;
  const int per = (nch_all + ksplit - 1) / ksplit;
  const int c0 = ks * per;
  const int nch = (nch_all - c0 < per) ? ((nch_all - c0 > 0) ? nch_all - c0 : 0) : per;
  if (tid == 0) {
    tc::mbar_init1(&bar[0]);
    tc::mbar_init1(&bar[1]);
    tc::mbar_init_fence();
  }
  __syncwarp();
  if (warp == 0)
    tc::tmem_alloc(&tslot, 2 * TILE);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const float *col = pair_col(X, I, J, tid);
  // rows k0 .. k0 + 63 of this thread's column (zeros past m)
  auto load = [&](int it, float (&v)[KC]) {
    const int k0 = (c0 + it) * KC;
    if (k0 + KC <= m) {
#pragma unroll
      for (int g = 0; g < KC / 4; ++g) {
        const float4 a = *reinterpret_cast<const float4 *>(col + k0 + 4 * g);
        v[4 * g] = a.x;
        v[4 * g + 1] = a.y;
        v[4 * g + 2] = a.z;
        v[4 * g + 3] = a.w;
      }
    }
    else {
#pragma unroll
      for (int e = 0; e < KC; ++e)
        v[e] = (k0 + e < m) ? col[k0 + e] : 0.f;
    }
  };
  int issued = 0;  // chunks whose MMAs were issued
  // chunk it from the registers cur while chunk it + 1 loads into nxt; false (for the whole
  // CTA) when the wait for a stage gave up
  auto one = [&](int it, float (&cur)[KC], float (&nxt)[KC]) -> bool {
    const int s = it & 1;
    unsigned char *st = smem + s * 3 * PLANE;
    if (it + 1 < nch)
      load(it + 1, nxt);
    // the MMAs of chunk it - 2 have read stage s
    const bool w = (it >= 2) ? tc::mbar_wait(&bar[s], (uint32_t)(((it >> 1) - 1) & 1), WAIT_CYCLES) : true;
    if (!__syncthreads_and(w))
      return false;
#pragma unroll
    for (int g = 0; g < KC / 8; ++g) {
      const float(&v8)[8] = *reinterpret_cast<const float(*)[8]>(cur + 8 * g);
      store_split8(st + tile_off(tid, 8 * g), v8);
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      const uint32_t a0 = tc::saddr(st);
      // X^T X is symmetric and D_ts = D_st^T for D_st = X_s^T X_t: F = D_hh + D_mm and
      // E = D_hm + D_hl (six-term split) or F = D_hh, E = D_hm (three-term), so that
      // S = F + E + E^T with four (two) products instead of six (three)
#pragma unroll
      for (int kk = 0; kk < KC / 16; ++kk) {
        auto d = [&](int term) { return tc::sdesc(a0 + term * PLANE + kk * 2 * LBO, LBO, SBO); };
        const uint32_t first = (it > 0 || kk > 0) ? 1u : 0u;
        if (NT == 6) {
          tc::mma_bf16(tmem, d(1), d(1), IDESC, first);
          tc::mma_bf16(tmem, d(0), d(0), IDESC, 1u);
          tc::mma_bf16(tmem + TILE, d(0), d(2), IDESC, first);
          tc::mma_bf16(tmem + TILE, d(0), d(1), IDESC, 1u);
        }
        else {
          tc::mma_bf16(tmem, d(0), d(0), IDESC, first);
          tc::mma_bf16(tmem + TILE, d(0), d(1), IDESC, first);
        }
      }
      tc::commit(&bar[s]);
    }
    issued = it + 1;
    return true;
  };
  bool ok = true;
  {
    float va[KC], vb[KC];
    if (nch > 0)
      load(0, va);
    for (int it = 0; it < nch; it += 2) {
      if (!one(it, va, vb)) {
        ok = false;
        break;
      }
      if (it + 1 >= nch)
        break;
      if (!one(it + 1, vb, va)) {
        ok = false;
        break;
      }
    }
  }
  // every issued chunk complete (commits complete in order; a second bounded wait after a
  // failed one, so that no MMA is in flight when the TMEM is released)
  for (int rep = 0; rep < 2 && issued >= 1; ++rep) {
    bool w = tc::mbar_wait(&bar[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1), WAIT_CYCLES);
    if (issued >= 2)
      w = tc::mbar_wait(&bar[(issued - 2) & 1], (uint32_t)(((issued - 2) >> 1) & 1), WAIT_CYCLES) && w;
    if (w)
      break;
    ok = false;
  }
  tc::fence_after();
  __syncwarp();
  // F then E, row tid of each (TMEM lane tid)
  for (int mat = 0; mat < 2; ++mat) {
    float4 *out = reinterpret_cast<float4 *>(Spart + ((size_t)blockIdx.x * 2 + mat) * TILE * TILE +
                                             (size_t)tid * TILE);
    if (nch == 0) {
      for (int c = 0; c < TILE / 4; ++c)
        out[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    else {
#pragma unroll 1
      for (int c = 0; c < TILE; c += 32) {
        uint32_t r[32];
        tc::tmem_ld32(tmem + (uint32_t)(mat * TILE) + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
#pragma unroll
        for (int e = 0; e < 8; ++e)
          out[c / 4 + e] = make_float4(__uint_as_float(r[4 * e]), __uint_as_float(r[4 * e + 1]),
                                       __uint_as_float(r[4 * e + 2]), __uint_as_float(r[4 * e + 3]));
      }
    }
  }
  if (!ok)
    atomicOr(err, 1u);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  __syncwarp();
  if (warp == 0)
    tc::tmem_dealloc(tmem, 2 * TILE);
}

// ---------------------------------------------------------------- block rotations
// CTA (pair, q): the row tiles q, q + Q, q + 2Q, ... of the pair's 128 real columns of G
// (tiles 0..tg-1, 128 rows each) and of W (tiles tg..tg+tw-1): Y = X R, Y replacing X in
// place. R's split image (2 K stages x 3 terms of 128 x 64 BF16, 96 KiB) is copied in once
// by TMA; each tile of X is converted by the 256 threads (thread t: row t % 128, K half
// t / 128), multiplied into one of two TMEM accumulators, and written back while the next
// tile's product runs. Each CTA reads all of a tile before any of it is written, and the
// tiles of a pair are disjoint rows.
constexpr int APPLY_THREADS = 256;
template <int NT>
__global__ void __launch_bounds__(APPLY_THREADS) k_apply(Cols G, int m, Cols W, int n, int nb, int step, int tg,
                                                         int tw, int Q, const unsigned char *Rimg, unsigned *err)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024u - (tc::saddr(smem_raw) & 1023u)) & 1023u);
  unsigned char *Rs = smem, *As = smem + 6 * PLANE;  // R: [stage][term]; A: [stage][term]
  float **colG = reinterpret_cast<float **>(smem + 12 * PLANE), **colW = colG + TILE;  // the pair's columns
  __shared__ unsigned long long bar[2];  // 0: TMA of R, 1: MMA completion (one phase per tile)
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int pair = blockIdx.x / Q, q0 = blockIdx.x % Q;
  const int ntile = tg + tw;
  int I, J;
  block_pair(nb, step, pair, I, J);
  if (tid == 0) {
    tc::mbar_init1(&bar[0]);
    tc::mbar_init1(&bar[1]);
    tc::mbar_init_fence();
  }
  __syncwarp();
  if (warp == 0)
    tc::tmem_alloc(&tslot, 2 * TILE);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    mbar_expect_tx(&bar[0], 6u * PLANE);
    const unsigned char *src = Rimg + (size_t)pair * 6 * PLANE;
    tma_load_1d(Rs, src, 3u * PLANE, &bar[0]);
    tma_load_1d(Rs + 3 * PLANE, src + 3 * PLANE, 3u * PLANE, &bar[0]);
  }
  const int row = tid & (TILE - 1), half = tid >> 7;
  bool ok = true, rready = false;
  if (tid < TILE)
    colG[tid] = pair_col(G, I, J, tid);
  else
    colW[tid - TILE] = pair_col(W, I, J, tid - TILE);
  __syncthreads();
  auto tile_of = [&](int t, float **&X, int &rows, int &r0) {
    const bool onG = t < tg;
    X = onG ? colG : colW;
    rows = onG ? m : n;
    r0 = (onG ? t : t - tg) * TILE;
  };
  // write back tile t from TMEM buffer b: warp w reads lanes 32 (w % 4) .. + 31 (rows),
  // columns 64 (w / 4) .. + 63
  auto epilogue = [&](int t, int b) {
    float **X;
    int rows, r0;
    tile_of(t, X, rows, r0);
    const int r = r0 + 32 * (warp & 3) + (tid & 31);
#pragma unroll 1
    for (int c = 64 * (warp >> 2); c < 64 * (warp >> 2) + 64; c += 32) {
      uint32_t v[32];
      tc::tmem_ld32(tmem + (uint32_t)(b * TILE) + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)c, v);
      if (r < rows) {
#pragma unroll
        for (int e = 0; e < 32; ++e)
          X[c + e][r] = __uint_as_float(v[e]);
      }
    }
  };
  auto load_tile = [&](int t, float (&v)[KC]) {
    float **X;
    int rows, r0;
    tile_of(t, X, rows, r0);
    const int gr = r0 + row;
    const bool live = gr < rows;
#pragma unroll
    for (int e = 0; e < KC; ++e)
      v[e] = live ? X[half * KC + e][gr] : 0.f;
  };
  int done = 0;  // tiles whose MMAs were committed
  // tile t (the k-th of this CTA) from the registers cur, while the next tile's values load
  // into nxt; false (for the whole CTA) when a wait gave up
  auto one = [&](int t, int k, float (&cur)[KC], float (&nxt)[KC]) -> bool {
    // the previous tile's MMAs have read the A buffer
    if (k > 0) {
      const bool w = tc::mbar_wait(&bar[1], (uint32_t)((k - 1) & 1), WAIT_CYCLES);
      if (!__syncthreads_and(w))
        return false;
      tc::fence_after();
    }
    unsigned char *st = As + half * 3 * PLANE;
#pragma unroll
    for (int g = 0; g < KC / 8; ++g) {
      const float(&v8)[8] = *reinterpret_cast<const float(*)[8]>(cur + 8 * g);
      store_split8(st + tile_off(row, 8 * g), v8);
    }
    if (t + Q < ntile)
      load_tile(t + Q, nxt);  // in flight during this tile's product and the write-back below
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      if (!rready) {
        rready = tc::mbar_wait(&bar[0], 0u, WAIT_CYCLES);
        if (!rready)  // the copy did not arrive: wait once more so that it is not in flight at exit
          tc::mbar_wait(&bar[0], 0u, WAIT_CYCLES);
      }
      tc::fence_after();
      if (rready) {
        const uint32_t d = tmem + (uint32_t)((k & 1) * TILE);
#pragma unroll 1
        for (int s2 = 0; s2 < 2; ++s2) {
          const uint32_t a0 = tc::saddr(As + s2 * 3 * PLANE), b0 = tc::saddr(Rs + s2 * 3 * PLANE);
#pragma unroll
          for (int kk = 0; kk < KC / 16; ++kk)
#pragma unroll
            for (int tt = 6 - NT; tt < 6; ++tt) {
              const uint64_t ad = tc::sdesc(a0 + TA[tt] * PLANE + kk * 2 * LBO, LBO, SBO);
              const uint64_t bd = tc::sdesc(b0 + TB[tt] * PLANE + kk * 2 * LBO, LBO, SBO);
              tc::mma_bf16(d, ad, bd, IDESC, (s2 > 0 || kk > 0 || tt > 6 - NT) ? 1u : 0u);
            }
        }
      }
      tc::commit(&bar[1]);
    }
    done = k + 1;
    if (__syncthreads_or(tid == 0 && !rready))
      return false;
    // write back the previous tile while this one's product runs
    if (k > 0) {
      __syncwarp();
      epilogue(t - Q, (k - 1) & 1);
    }
    return true;
  };
  {
    float va[KC], vb[KC];
    if (q0 < ntile)
      load_tile(q0, va);
    for (int t = q0, k = 0; t < ntile; t += 2 * Q, k += 2) {
      if (!one(t, k, va, vb)) {
        ok = false;
        break;
      }
      if (t + Q >= ntile)
        break;
      if (!one(t + Q, k + 1, vb, va)) {
        ok = false;
        break;
      }
    }
  }
  // the last tile: its product complete, then written back
  if (done > 0) {
    bool w = tc::mbar_wait(&bar[1], (uint32_t)((done - 1) & 1), WAIT_CYCLES);
    if (!w)
      w = tc::mbar_wait(&bar[1], (uint32_t)((done - 1) & 1), WAIT_CYCLES);
    ok = __syncthreads_and(w && ok) != 0;
    tc::fence_after();
    __syncwarp();
    if (ok)
      epilogue(q0 + (done - 1) * Q, (done - 1) & 1);
  }
  if (!ok)
    atomicOr(err, 1u);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  __syncwarp();
  if (warp == 0)
    tc::tmem_dealloc(tmem, 2 * TILE);
}

// the split image of the real 128 x 128 rotation Rb (Rb[k][i], k = input column, i = output
// column) as k_apply's B operand: B[i][k] = Rb[k][i], stage k / 64, three BF16 terms.
// Thread layout: each (i, 8 consecutive k) chunk is one 16-byte store per term.
template <typename F>
__device__ __forceinline__ void write_rimg(unsigned char *img, F rb)
{
  for (int q = threadIdx.x; q < TILE * (TILE / 8); q += blockDim.x) {
    const int i = q % TILE, k8 = (q / TILE) * 8;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e)
      v[e] = rb(k8 + e, i);
    store_split8(img + (k8 / KC) * 3 * PLANE + tile_off(i, k8 % KC), v);
  }
}

// ---------------------------------------------------------------- Gram reduction
// S = sum over the K splits of F + E + E^T, tile by tile: CTA (pair, 32 x 32 tile (ti, tj))
// reads the tile (ti, tj) of every split's F and E and the tile (tj, ti) of its E through
// shared memory (coalesced rows; the transpose in shared memory), and writes S's tile.
__global__ void __launch_bounds__(256) k_gram_reduce(const float *Spart, int ksplit, float *S)
{
  __shared__ float et[32][33];
  const int pair = blockIdx.x >> 4, tile = blockIdx.x & 15, ti = tile >> 2, tj = tile & 3;
  const int x = threadIdx.x & 31, y0 = threadIdx.x >> 5;  // 8 rows of the tile per pass
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k = 0; k < ksplit; ++k) {
    const float *F = Spart + ((size_t)pair * ksplit + k) * 2 * TILE * TILE, *E = F + TILE * TILE;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int y = y0 + 8 * r;
      et[y][x] = E[(tj * 32 + y) * TILE + ti * 32 + x];  // row tj*32+y of E, columns of tile ti
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int y = y0 + 8 * r, i = ti * 32 + y, j = tj * 32 + x;
      acc[r] += F[i * TILE + j] + (E[i * TILE + j] + et[x][y]);
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
    S[(size_t)pair * TILE * TILE + (ti * 32 + y0 + 8 * r) * TILE + tj * 32 + x] = acc[r];
}

// ---------------------------------------------------------------- pair eigenproblems
// Rotation of one pair (p, q) of the Hermitian H from h_pp = a, h_qq = b, h_pq = c (the
// scalar sweep's formulas: zeta = (b - a) / (2|c|), t the smaller root of t^2 + 2 zeta t = 1,
// cs = 1 / sqrt(1 + t^2), s = t cs c / |c|), with fast approximate division and reciprocal
// square roots refined by one Newton step: these sweeps are a preconditioner, and the same
// rotation is applied to G and W, so a rotation a few ulps from unitary changes nothing
// but the accumulated W's orthogonality, which the FP64 orthonormalisation restores.
struct Rot {
  float c, sr, si, d1, d2, ac, sc;
  int go;
};
__device__ __forceinline__ float rsqrt_nr(float x)
{
  const float y = rsqrtf(x);
  return y * fmaf(-0.5f * x, y * y, 1.5f);
}
__device__ __forceinline__ Rot pair_rot(float ha, float hb, float cr, float ci, float tol)
{
  Rot r{1.f, 0.f, 0.f, ha, hb, 0.f, 0.f, 0};
  const float ar = fabsf(cr), ai = fabsf(ci);
  const float am = fmaxf(ar, ai), an = fminf(ar, ai);
  if (!(am > 0.f))
    return r;
  // (IEEE quotients: the entries of small columns' Gram blocks can be subnormal, where the
  // approximate division flushes to zero)
  const float qn = an / am;
  const float ac = am * (fmaf(qn, qn, 1.f) * rsqrt_nr(fmaf(qn, qn, 1.f)));  // |c|
  const float sc = sqrtf(ha) * sqrtf(hb);
  r.ac = ac;
  r.sc = sc;
  if (!(ac >= tol * sc))
    return r;
  const float zeta = (hb - ha) / (2.f * ac);
  const float az = fabsf(zeta);
  const float t = (az > 1e18f) ? 0.5f / zeta
                               : copysignf(1.f, zeta) / (az + fmaf(az, az, 1.f) * rsqrt_nr(fmaf(az, az, 1.f)));
  const float cs = rsqrt_nr(fmaf(t, t, 1.f));
  const float sn = t * cs;
  r.c = cs;
  r.sr = sn * (cr / ac);
  r.si = sn * (ci / ac);
  r.d1 = fmaf(-t, ac, ha);
  r.d2 = fmaf(t, ac, hb);
  r.go = 1;
  return r;
}

// One CTA (256 threads) per block pair: from the pair's Gram matrix S forms H (complex
// 64 x 64 from the real Gram of [Re | Im], or real 128 x 128), runs `sweeps` cyclic
// Jacobi sweeps on H, logs every step's rotations (rlog: sweeps (N - 1) steps x N/2
// records per pair) and the order of the final diagonal (rranks: descending, ties by
// index); k_build_r accumulates the rotations into R on more SMs.
// stats[0] += rotations, stats[1] = max over rotated pairs of |h_pq| / sqrt(h_pp h_qq)
// (as float bits).
// Layout: complex H as interleaved (re, im) pairs, one 64-bit shared-memory access per
// entry; each pair's rotation as one 16-byte record {c, Re s, Im s, p | q << 8 |
// active << 16}.
// Per Jacobi step: warp 0 (lane u: pair u, and u + 32 for real data) reads the step's
// pairs from H, writes their rotation records and, for the pairs it rotates, the new 2x2
// diagonal blocks of H (no other block touches them); after a barrier every thread updates
// off-diagonal 2x2 blocks (u, v), u < v, of H := J^H H J from a list; a second barrier
// ends the step.
constexpr int EVD_THREADS = 256;
template <bool CPLX>
__global__ void __launch_bounds__(EVD_THREADS) k_pair_evd(const float *Sred, int sweeps, float tol, float4 *rlog,
                                                          int *rranks, unsigned *stats)
{
  using E = typename std::conditional<CPLX, float2, float>::type;
  constexpr int N = CPLX ? 64 : 128;  // order of H
  constexpr int P = N / 2;             // pairs per Jacobi step
  constexpr int PL = P / 32;           // pairs per lane
  constexpr int LD = N + 1;
  constexpr int NO = P * (P - 1) / 2;  // off-diagonal blocks u < v
  extern __shared__ __align__(16) float fsm[];
  float4 *rot = reinterpret_cast<float4 *>(fsm);  // P records
  E *H = reinterpret_cast<E *>(rot + P);
  unsigned short *tri = reinterpret_cast<unsigned short *>(H + N * LD);  // NO entries: u << 8 | v
  int *rank = reinterpret_cast<int *>(tri + ((NO + 1) & ~1));
  __shared__ unsigned nrot_s, mu_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float *S0 = Sred + (size_t)blockIdx.x * TILE * TILE;
  if (tid == 0) {
    nrot_s = 0u;
    mu_s = 0u;
  }
  for (int q = tid; q < P * P; q += EVD_THREADS) {
    const int u = q / P, v = q % P;
    if (u < v)
      tri[u * P - u * (u + 1) / 2 + (v - u - 1)] = (unsigned short)((u << 8) | v);
  }
  float4 *lg = rlog + (size_t)blockIdx.x * sweeps * (N - 1) * P;
  // H from S; only the upper triangle of H is stored (an entry (i, j) with i > j is the
  // conjugate of the stored (j, i)), so that an update writes each entry once
  for (int q = tid; q < N * N; q += EVD_THREADS) {
    const int i = q / N, j = q % N;
    if (i > j)
      continue;
    auto S = [&](int a, int b) { return S0[a * TILE + b]; };
    if constexpr (CPLX) {
      const float hr = S(i, j) + S(64 + i, 64 + j);
      const float hi = (i == j) ? 0.f : (S(i, 64 + j) - S(64 + i, j));
      H[i * LD + j] = make_float2(hr, hi);
    }
    else
      H[i * LD + j] = S(i, j);
  }
  __syncthreads();
  auto re = [](const E &x) -> float {
    if constexpr (CPLX)
      return x.x;
    else
      return x;
  };
  auto cj = [](const E &x) -> E {
    if constexpr (CPLX)
      return make_float2(x.x, -x.y);
    else
      return x;
  };
  // entry (i, j), i != j, of the Hermitian H, and its store
  auto hget = [&](int i, int j) -> E { return (i < j) ? H[i * LD + j] : cj(H[j * LD + i]); };
  auto hput = [&](int i, int j, const E &x) {
    if (i < j)
      H[i * LD + j] = x;
    else
      H[j * LD + i] = cj(x);
  };
  unsigned nrot = 0u;
  float mu = 0.f;
  for (int sw = 0; sw < sweeps; ++sw)
    for (int stp = 0; stp < N - 1; ++stp) {
      // the step's pairs, their rotations and new diagonal blocks (warp 0; lane u: pairs
      // u, u + 32)
      if (warp == 0) {
#pragma unroll
        for (int h = 0; h < PL; ++h) {
          const int u = lane + 32 * h;
          int a, c;
          if (u == 0) {
            a = stp;
            c = N - 1;
          }
          else {
            a = stp + u;
            a -= (a >= N - 1) ? (N - 1) : 0;
            c = stp + (N - 1) - u;
            c -= (c >= N - 1) ? (N - 1) : 0;
          }
          // (the circle order's own orientation: the first indices of a step are consecutive
          // modulo N - 1, and so are the second ones, so that the row and column accesses of
          // the updates fall into distinct shared-memory banks)
          const int p = a, q = c;
          const E hpq = hget(p, q);
          float cr, ci = 0.f;
          if constexpr (CPLX) {
            cr = hpq.x;
            ci = hpq.y;
          }
          else
            cr = hpq;
          const Rot r = pair_rot(fmaxf(re(H[p * LD + p]), 0.f), fmaxf(re(H[q * LD + q]), 0.f), cr, ci, tol);
          const bool act = r.go && ((r.sr != 0.f) || (r.si != 0.f));
          const unsigned tag = (unsigned)p | ((unsigned)q << 8) | (act ? (1u << 16) : 0u);
          const float4 rec =
              act ? make_float4(r.c, r.sr, r.si, __uint_as_float(tag)) : make_float4(1.f, 0.f, 0.f, __uint_as_float(tag));
          rot[u] = rec;
          lg[(size_t)(sw * (N - 1) + stp) * P + u] = rec;
          if (act) {
            if constexpr (CPLX) {
              H[p * LD + p] = make_float2(r.d1, 0.f);
              H[q * LD + q] = make_float2(r.d2, 0.f);
              H[min(p, q) * LD + max(p, q)] = make_float2(0.f, 0.f);
            }
            else {
              H[p * LD + p] = r.d1;
              H[q * LD + q] = r.d2;
              H[min(p, q) * LD + max(p, q)] = 0.f;
            }
          }
          if (r.go) {
            ++nrot;
            mu = fmaxf(mu, (r.sc > 0.f) ? r.ac / r.sc : 1.f);
          }
        }
      }
      __syncthreads();
      // H := J^H H J, one off-diagonal 2x2 block (u, v) per item, the (v, u) block its
      // conjugate transpose (an inactive side is the identity)
      for (int it = tid; it < NO; it += EVD_THREADS) {
        const unsigned uv = tri[it];
        const float4 ru = rot[uv >> 8], rv = rot[uv & 255];
        const unsigned tu = __float_as_uint(ru.w), tv = __float_as_uint(rv.w);
        if (!((tu | tv) >> 16))
          continue;
        const int pu = tu & 255, qu = (tu >> 8) & 255, pv = tv & 255, qv = (tv >> 8) & 255;
        const float cu = ru.x, sur = ru.y, sui = ru.z;
        const float cv = rv.x, svr = rv.y, svi = rv.z;
        if constexpr (CPLX) {
          const float2 b00 = hget(pu, pv), b01 = hget(pu, qv), b10 = hget(qu, pv), b11 = hget(qu, qv);
          // C = B J_v: C[:,0] = cv B[:,0] - conj(s_v) B[:,1], C[:,1] = cv B[:,1] + s_v B[:,0]
          const float c00r = fmaf(cv, b00.x, -fmaf(svr, b01.x, svi * b01.y));
          const float c00i = fmaf(cv, b00.y, -fmaf(svr, b01.y, -(svi * b01.x)));
          const float c10r = fmaf(cv, b10.x, -fmaf(svr, b11.x, svi * b11.y));
          const float c10i = fmaf(cv, b10.y, -fmaf(svr, b11.y, -(svi * b11.x)));
          const float c01r = fmaf(cv, b01.x, fmaf(svr, b00.x, -(svi * b00.y)));
          const float c01i = fmaf(cv, b01.y, fmaf(svr, b00.y, svi * b00.x));
          const float c11r = fmaf(cv, b11.x, fmaf(svr, b10.x, -(svi * b10.y)));
          const float c11i = fmaf(cv, b11.y, fmaf(svr, b10.y, svi * b10.x));
          // B' = J_u^H C: row 0 = cu C[0,:] - s_u C[1,:], row 1 = cu C[1,:] + conj(s_u) C[0,:]
          const float n00r = fmaf(cu, c00r, -fmaf(sur, c10r, -(sui * c10i)));
          const float n00i = fmaf(cu, c00i, -fmaf(sur, c10i, sui * c10r));
          const float n01r = fmaf(cu, c01r, -fmaf(sur, c11r, -(sui * c11i)));
          const float n01i = fmaf(cu, c01i, -fmaf(sur, c11i, sui * c11r));
          const float n10r = fmaf(cu, c10r, fmaf(sur, c00r, sui * c00i));
          const float n10i = fmaf(cu, c10i, fmaf(sur, c00i, -(sui * c00r)));
          const float n11r = fmaf(cu, c11r, fmaf(sur, c01r, sui * c01i));
          const float n11i = fmaf(cu, c11i, fmaf(sur, c01i, -(sui * c01r)));
          hput(pu, pv, make_float2(n00r, n00i));
          hput(pu, qv, make_float2(n01r, n01i));
          hput(qu, pv, make_float2(n10r, n10i));
          hput(qu, qv, make_float2(n11r, n11i));
        }
        else {
          const float b00 = hget(pu, pv), b01 = hget(pu, qv), b10 = hget(qu, pv), b11 = hget(qu, qv);
          const float c00 = fmaf(cv, b00, -(svr * b01)), c10 = fmaf(cv, b10, -(svr * b11));
          const float c01 = fmaf(cv, b01, svr * b00), c11 = fmaf(cv, b11, svr * b10);
          const float n00 = fmaf(cu, c00, -(sur * c10)), n01 = fmaf(cu, c01, -(sur * c11));
          const float n10 = fmaf(cu, c10, sur * c00), n11 = fmaf(cu, c11, sur * c01);
          hput(pu, pv, n00);
          hput(pu, qv, n01);
          hput(qu, pv, n10);
          hput(qu, qv, n11);
        }
      }
      __syncthreads();
    }
  // descending order of the diagonal (ties by index): column rank[r] of R goes to place r
  // (a NaN sorts as -inf, so that the ranks stay a permutation)
  auto key = [&](int i) {
    const float d = re(H[i * LD + i]);
    return (d == d) ? d : -INFINITY;
  };
  for (int i = tid; i < N; i += EVD_THREADS) {
    const float d = key(i);
    int r = 0;
    for (int j = 0; j < N; ++j) {
      const float e = key(j);
      r += (e > d || (e == d && j < i)) ? 1 : 0;
    }
    rank[r] = i;
  }
  if (warp == 0) {
    if (nrot)
      atomicAdd(&nrot_s, nrot);
    if (mu > 0.f)
      atomicMax(&mu_s, __float_as_uint(mu));
  }
  __syncthreads();
  for (int i = tid; i < N; i += EVD_THREADS)
    rranks[(size_t)blockIdx.x * N + i] = rank[i];
  if (tid == 0) {
    if (nrot_s)
      atomicAdd(stats, nrot_s);
    if (mu_s)
      atomicMax(stats + 1, mu_s);
  }
}

// R := J_1 J_2 ... (the logged rotations of a pair's eigenproblem, in order) and R's split
// image for k_apply, with its columns in the order of rranks. BR_PARTS CTAs per pair, each
// a share of R's rows: every warp owns whole rows (in shared memory), so consecutive steps
// need only the warp's own synchronisation; lane v applies pair v's rotation (and v + 32's
// for real data) to the columns p_v, q_v of each of its rows. The records are staged in
// shared memory BR_CHUNK steps at a time.
constexpr int BR_THREADS = 256, BR_PARTS = 4;
template <bool CPLX> struct brc {
  static constexpr int N = CPLX ? 64 : 128, LD = N + 1, ROWS = N / BR_PARTS, CHUNK = CPLX ? 32 : 16;
};
template <bool CPLX> static size_t br_smem()
{
  using C = brc<CPLX>;
  return (size_t)C::ROWS * C::LD * (CPLX ? 8 : 4) + (size_t)C::CHUNK * (C::N / 2) * 16 + (size_t)C::N * 4;
}
template <bool CPLX>
__global__ void __launch_bounds__(BR_THREADS) k_build_r(const float4 *rlog, const int *rranks, int sweeps,
                                                        unsigned char *Rimg)
{
  using E = typename std::conditional<CPLX, float2, float>::type;
  using C = brc<CPLX>;
  constexpr int N = C::N, P = N / 2, PL = P / 32, LD = C::LD, ROWS = C::ROWS, CH = C::CHUNK;
  constexpr int NW = BR_THREADS / 32, RPW = ROWS / NW;  // rows per warp
  extern __shared__ __align__(16) float fsm[];
  E *R = reinterpret_cast<E *>(fsm);                      // ROWS x LD: rows r0 .. r0 + ROWS - 1
  float4 *lg = reinterpret_cast<float4 *>(R + ROWS * LD);  // CH steps x P records
  int *rank = reinterpret_cast<int *>(lg + CH * P);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int pair = blockIdx.x / BR_PARTS, r0 = (blockIdx.x % BR_PARTS) * ROWS;
  const int steps = sweeps * (N - 1);
  const float4 *src = rlog + (size_t)pair * steps * P;
  for (int i = tid; i < N; i += BR_THREADS)
    rank[i] = rranks[(size_t)pair * N + i];
  for (int q = tid; q < ROWS * N; q += BR_THREADS) {
    const int r = q / N, j = q % N;
    if constexpr (CPLX)
      R[r * LD + j] = make_float2((r0 + r == j) ? 1.f : 0.f, 0.f);
    else
      R[r * LD + j] = (r0 + r == j) ? 1.f : 0.f;
  }
  for (int c0 = 0; c0 < steps; c0 += CH) {
    const int nst = (steps - c0 < CH) ? (steps - c0) : CH;
    __syncthreads();  // the previous chunk's records are consumed
    for (int q = tid; q < nst * P; q += BR_THREADS)
      lg[q] = src[(size_t)c0 * P + q];
    __syncthreads();
    for (int st = 0; st < nst; ++st) {
#pragma unroll
      for (int h = 0; h < PL; ++h) {
        const float4 rv = lg[st * P + lane + 32 * h];
        const unsigned tv = __float_as_uint(rv.w);
        if (!(tv >> 16))
          continue;
        const int pv = tv & 255, qv = (tv >> 8) & 255;
        const float cv = rv.x, svr = rv.y, svi = rv.z;
#pragma unroll
        for (int i = 0; i < RPW; ++i) {
          const int r = warp * RPW + i;
          if constexpr (CPLX) {
            const float2 x = R[r * LD + pv], y = R[r * LD + qv];
            R[r * LD + pv] = make_float2(fmaf(cv, x.x, -fmaf(svr, y.x, svi * y.y)), fmaf(cv, x.y, -fmaf(svr, y.y, -(svi * y.x))));
            R[r * LD + qv] = make_float2(fmaf(cv, y.x, fmaf(svr, x.x, -(svi * x.y))), fmaf(cv, y.y, fmaf(svr, x.y, svi * x.x)));
          }
          else {
            const float x = R[r * LD + pv], y = R[r * LD + qv];
            R[r * LD + pv] = fmaf(cv, x, -(svr * y));
            R[r * LD + qv] = fmaf(cv, y, svr * x);
          }
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
  // the image: B[i][k] = Rb[k][i] for the rows k of Rb this CTA holds (real: R's rows
  // r0 ..; complex: Rb = [[Re R, Im R], [-Im R, Re R]], rows r0 .. and 64 + r0 ..), columns
  // i in rank order; 8 consecutive k per 16-byte store of each term (the layout of write_rimg)
  unsigned char *img = Rimg + (size_t)pair * 6 * PLANE;
  constexpr int NK8 = CPLX ? 2 * ROWS / 8 : ROWS / 8;
  for (int q = tid; q < TILE * NK8; q += BR_THREADS) {
    const int i = q % TILE, ci = q / TILE;
    int k8;
    if constexpr (CPLX)
      k8 = (ci < ROWS / 8) ? (r0 + 8 * ci) : (64 + r0 + 8 * (ci - ROWS / 8));
    else
      k8 = r0 + 8 * ci;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = k8 + e;
      if constexpr (CPLX) {
        const float2 x = R[((k & 63) - r0) * LD + rank[i & 63]];
        v[e] = (k < 64) ? ((i < 64) ? x.x : x.y) : ((i < 64) ? -x.y : x.x);
      }
      else
        v[e] = R[(k - r0) * LD + rank[i]];
    }
    store_split8(img + (k8 / KC) * 3 * PLANE + tile_off(i, k8 % KC), v);
  }
}

// the split image of caller-given real 128 x 128 rotations (pair k: R + k 128 128,
// column-major: R[k][i] at k + 128 i), for vj_block_apply_dev
__global__ void __launch_bounds__(256) k_rimg(const float *R, unsigned char *Rimg)
{
  const float *Rk = R + (size_t)blockIdx.x * TILE * TILE;
  write_rimg(Rimg + (size_t)blockIdx.x * 6 * PLANE, [&](int k, int i) { return Rk[k + TILE * i]; });
}

static size_t evd_smem(bool cplx)
{
  const int N = cplx ? 64 : 128, P = N / 2, LD = N + 1, NO = P * (P - 1) / 2;
  return (size_t)P * 16 + (size_t)N * LD * (cplx ? 8 : 4) + (size_t)((NO + 1) & ~1) * 2 + (size_t)N * 4;
}

constexpr size_t GRAM_SMEM = 2 * 3 * PLANE + 1024;
constexpr size_t APPLY_SMEM = 2 * 6 * PLANE + 2 * TILE * sizeof(float *) + 1024;  // R image, one A tile, columns

// ---------------------------------------------------------------- host side
struct Plan {
  int nb, npairs, ksplit, tg, tw, b, q;  // q: CTAs per pair of k_apply
  bool cplx;
};

static bool attrs_set(bool cplx)
{
  static int done[host::MAX_DEVICES][2] = {};  // kernel attributes are set per device
  int &d = done[host::device_slot()][cplx ? 1 : 0];
  if (!d) {
    bool ok = cudaFuncSetAttribute(k_gram<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRAM_SMEM) ==
                  cudaSuccess &&
              cudaFuncSetAttribute(k_gram<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRAM_SMEM) ==
                  cudaSuccess &&
              cudaFuncSetAttribute(k_apply<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)APPLY_SMEM) ==
                  cudaSuccess &&
              cudaFuncSetAttribute(k_apply<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)APPLY_SMEM) ==
                  cudaSuccess;
    ok = ok && (cplx ? cudaFuncSetAttribute(k_pair_evd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)evd_smem(true))
                     : cudaFuncSetAttribute(k_pair_evd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)evd_smem(false))) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return false;
    }
    d = 1;
  }
  return true;
}

static Plan plan(bool cplx, long long m, long long n)
{
  Plan p;
  p.cplx = cplx;
  p.b = cplx ? 32 : 64;
  p.nb = (int)(n / p.b);
  p.npairs = p.nb / 2;
  // split K so that the Gram grid covers every SM with its two resident CTAs
  const int sms = host::sm_count();
  const int nch = (int)((m + KC - 1) / KC);
  int ks = (2 * sms) / p.npairs;
  if (ks > nch)
    ks = nch;
  if (ks < 1)
    ks = 1;
  p.ksplit = ks;
  p.tg = (int)((m + TILE - 1) / TILE);
  p.tw = (int)((n + TILE - 1) / TILE);
  // k_apply: one CTA per SM (its shared memory), the pair's row tiles spread over q CTAs
  int q = sms / p.npairs;
  if (q > p.tg + p.tw)
    q = p.tg + p.tw;
  p.q = (q < 1) ? 1 : q;
  return p;
}

}  // namespace bj

// whether the block sweeps apply to an m x n FP32 problem: whole blocks in an even number
// (n a multiple of 128 real / 64 complex columns), 16-byte aligned columns
bool block_sweeps_apply(bool cplx, long long m, long long n, long long ld)
{
  const long long bw = cplx ? 64 : 128;
  return n >= bw && (n % bw) == 0 && (m % 4) == 0 && (ld % 4) == 0 && m <= (1LL << 30);
}

// Scratch bytes of block_sweep for an m x n problem.
// (the Gram partials and their sum, R's split images, the rotation logs of `inner` sweeps
// of the pair eigenproblems and their orders)
static size_t rlog_records(bool cplx, int npairs, int inner)
{
  const int N = cplx ? 64 : 128;
  return (size_t)npairs * inner * (N - 1) * (N / 2);
}
size_t block_sweep_scratch(bool cplx, long long m, long long n, int inner)
{
  const bj::Plan p = bj::plan(cplx, m, n);
  return (size_t)p.npairs * (p.ksplit * 2 + 1) * bj::TILE * bj::TILE * 4 + (size_t)p.npairs * 6 * bj::PLANE +
         rlog_records(cplx, p.npairs, inner) * 16 + (size_t)p.npairs * (cplx ? 64 : 128) * 4 + 256;
}

// One block sweep (nb - 1 block steps) on planar FP32 G (m x n) and W (n x n), both with
// the given leading dimensions. scratch: block_sweep_scratch bytes; stats: 4 device words
// (zeroed here; [0] rotations, [1] max scaled |h_pq| of a rotated pair as float bits, [2]
// error flag). terms: 6 (FP32-accurate products) or 3. Returns rotations, or -1 (launch
// failure or a kernel whose wait gave up).
long long block_sweep(bool cplx, int m, int n, float *Gr, float *Gi, long long ldg, float *Wr, float *Wi,
                      long long ldw, unsigned char *scratch, unsigned *stats, float tol, int inner, int terms,
                      cudaStream_t s, float *mu)
{
  using namespace bj;
  if (!attrs_set(cplx))
    return -1;
  const Plan p = plan(cplx, m, n);
  float *Spart = reinterpret_cast<float *>(scratch);
  float *Sred = Spart + (size_t)p.npairs * p.ksplit * 2 * TILE * TILE;
  unsigned char *Rimg = scratch + (size_t)p.npairs * (p.ksplit * 2 + 1) * TILE * TILE * 4;
  float4 *rlog = reinterpret_cast<float4 *>(Rimg + (size_t)p.npairs * 6 * PLANE);
  int *rranks = reinterpret_cast<int *>(rlog + rlog_records(cplx, p.npairs, inner));
  const Cols G{Gr, cplx ? Gi : nullptr, ldg, p.b}, W{Wr, cplx ? Wi : nullptr, ldw, p.b};
  if (cudaMemsetAsync(stats, 0, 16, s) != cudaSuccess)
    return -1;
  for (int step = 0; step < p.nb - 1; ++step) {
    if (terms == 3)
      k_gram<3><<<p.npairs * p.ksplit, 128, GRAM_SMEM, s>>>(G, m, p.nb, step, p.ksplit, Spart, stats + 2);
    else
      k_gram<6><<<p.npairs * p.ksplit, 128, GRAM_SMEM, s>>>(G, m, p.nb, step, p.ksplit, Spart, stats + 2);
    k_gram_reduce<<<p.npairs * 16, 256, 0, s>>>(Spart, p.ksplit, Sred);
    if (cplx) {
      k_pair_evd<true><<<p.npairs, EVD_THREADS, evd_smem(true), s>>>(Sred, inner, tol, rlog, rranks, stats);
      k_build_r<true><<<p.npairs * BR_PARTS, BR_THREADS, br_smem<true>(), s>>>(rlog, rranks, inner, Rimg);
    }
    else {
      k_pair_evd<false><<<p.npairs, EVD_THREADS, evd_smem(false), s>>>(Sred, inner, tol, rlog, rranks, stats);
      k_build_r<false><<<p.npairs * BR_PARTS, BR_THREADS, br_smem<false>(), s>>>(rlog, rranks, inner, Rimg);
    }
    if (terms == 3)
      k_apply<3><<<p.npairs * p.q, APPLY_THREADS, APPLY_SMEM, s>>>(G, m, W, n, p.nb, step, p.tg, p.tw, p.q, Rimg,
                                                                    stats + 2);
    else
      k_apply<6><<<p.npairs * p.q, APPLY_THREADS, APPLY_SMEM, s>>>(G, m, W, n, p.nb, step, p.tg, p.tw, p.q, Rimg,
                                                                    stats + 2);
  }
  unsigned hs[4] = {0u, 0u, 0u, 0u};
  if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(hs, stats, 16, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return -1;
  if (hs[2])
    return -1;
  std::memcpy(mu, &hs[1], 4);
  return (long long)hs[0];
}

}  // namespace vj

using namespace vj;

// ---------------------------------------------------------------- C ABI
// The block-sweep building blocks on their own (tests, and callers that drive their own
// block orderings). Real data: Gi, Wi NULL; complex: split planes.
static bool block_args(int cplx, vj_fnat m, vj_fnat n, vj_fnat ld)
{
  return block_sweeps_apply(cplx != 0, (long long)m, (long long)n, (long long)ld) && ld >= m;
}

extern "C" vj_fint vj_block_gram_dev(int cplx, vj_fnat m, vj_fnat n, const float *Gr, const float *Gi, vj_fnat ldG,
                                     int step, int terms, float *S, void *stream)
{
  using namespace vj::bj;
  if (!block_args(cplx, m, n, ldG) || (terms != 3 && terms != 6) || (cplx && !Gi))
    return VJ_ERR_ARG;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const Plan p = plan(cplx != 0, (long long)m, (long long)n);
  if (step < 0 || step >= p.nb - 1)
    return VJ_ERR_ARG;
  if (!attrs_set(cplx != 0))
    return VJ_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  float *Spart = nullptr;
  unsigned *err = nullptr;
  if (cudaMalloc(&Spart, (size_t)p.npairs * p.ksplit * 2 * TILE * TILE * 4) != cudaSuccess)
    return VJ_ERR_NOMEM;
  if (cudaMalloc(&err, 16) != cudaSuccess) {
    cudaFree(Spart);
    return VJ_ERR_NOMEM;
  }
  const Cols G{const_cast<float *>(Gr), cplx ? const_cast<float *>(Gi) : nullptr, (long long)ldG, p.b};
  bool ok = cudaMemsetAsync(err, 0, 16, s) == cudaSuccess;
  if (ok) {
    // the split partials, then S = their sum of F + E + E^T, pair by pair
    if (terms == 3)
      k_gram<3><<<p.npairs * p.ksplit, 128, GRAM_SMEM, s>>>(G, (int)m, p.nb, step, p.ksplit, Spart, err);
    else
      k_gram<6><<<p.npairs * p.ksplit, 128, GRAM_SMEM, s>>>(G, (int)m, p.nb, step, p.ksplit, Spart, err);
    k_gram_reduce<<<p.npairs * 16, 256, 0, s>>>(Spart, p.ksplit, S);
    ok = cudaGetLastError() == cudaSuccess;
  }
  unsigned he = 0;
  ok = ok && cudaMemcpyAsync(&he, err, 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaStreamSynchronize(s) == cudaSuccess && !he;
  cudaFree(Spart);
  cudaFree(err);
  return ok ? (vj_fint)p.npairs : VJ_ERR_CUDA;
}

extern "C" vj_fint vj_block_apply_dev(int cplx, vj_fnat m, vj_fnat n, float *Gr, float *Gi, vj_fnat ldG, float *Wr,
                                      float *Wi, vj_fnat ldW, int step, int terms, const float *R, void *stream)
{
  using namespace vj::bj;
  if (!block_args(cplx, m, n, ldG) || !block_args(cplx, n, n, ldW) || (terms != 3 && terms != 6) ||
      (cplx && (!Gi || !Wi)))
    return VJ_ERR_ARG;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const Plan p = plan(cplx != 0, (long long)m, (long long)n);
  if (step < 0 || step >= p.nb - 1)
    return VJ_ERR_ARG;
  if (!attrs_set(cplx != 0))
    return VJ_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char *img = nullptr;
  unsigned *err = nullptr;
  if (cudaMalloc(&img, (size_t)p.npairs * 6 * PLANE) != cudaSuccess)
    return VJ_ERR_NOMEM;
  if (cudaMalloc(&err, 16) != cudaSuccess) {
    cudaFree(img);
    return VJ_ERR_NOMEM;
  }
  const Cols G{Gr, cplx ? Gi : nullptr, (long long)ldG, p.b}, W{Wr, cplx ? Wi : nullptr, (long long)ldW, p.b};
  bool ok = cudaMemsetAsync(err, 0, 16, s) == cudaSuccess;
  if (ok) {
    k_rimg<<<p.npairs, 256, 0, s>>>(R, img);
    if (terms == 3)
      k_apply<3><<<p.npairs * p.q, APPLY_THREADS, APPLY_SMEM, s>>>(G, (int)m, W, (int)n, p.nb, step, p.tg, p.tw, p.q,
                                                                      img,
                                                                    err);
    else
      k_apply<6><<<p.npairs * p.q, APPLY_THREADS, APPLY_SMEM, s>>>(G, (int)m, W, (int)n, p.nb, step, p.tg, p.tw, p.q,
                                                                      img,
                                                                    err);
    ok = cudaGetLastError() == cudaSuccess;
  }
  unsigned he = 0;
  ok = ok && cudaMemcpyAsync(&he, err, 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaStreamSynchronize(s) == cudaSuccess && !he;
  cudaFree(img);
  cudaFree(err);
  return ok ? (vj_fint)p.npairs : VJ_ERR_CUDA;
}

extern "C" vj_fint vj_block_sweep_dev(int cplx, vj_fnat m, vj_fnat n, float *Gr, float *Gi, vj_fnat ldG, float *Wr,
                                      float *Wi, vj_fnat ldW, float tol, int inner, int terms, float *mu,
                                      void *stream)
{
  if (!block_args(cplx, m, n, ldG) || !block_args(cplx, n, n, ldW) || (terms != 3 && terms != 6) || inner < 1 ||
      (cplx && (!Gi || !Wi)))
    return VJ_ERR_ARG;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  unsigned char *scr = nullptr;
  unsigned *stats = nullptr;
  if (cudaMalloc(&scr, block_sweep_scratch(cplx != 0, (long long)m, (long long)n, inner)) != cudaSuccess)
    return VJ_ERR_NOMEM;
  if (cudaMalloc(&stats, 16) != cudaSuccess) {
    cudaFree(scr);
    return VJ_ERR_NOMEM;
  }
  float mu_ = 0.f;
  const long long r = block_sweep(cplx != 0, (int)m, (int)n, Gr, Gi, (long long)ldG, Wr, Wi, (long long)ldW, scr,
                                  stats, tol, inner, terms, (cudaStream_t)stream, &mu_);
  cudaFree(scr);
  cudaFree(stats);
  if (mu)
    *mu = mu_;
  return r < 0 ? VJ_ERR_CUDA : (vj_fint)r;
}
