// Command-line SVD drivers with the reference's interface, over the drop-in C ABI:
//
//   t?vjsvd.exe J M N BaseName
//
// replaces src/tdvjsvd.c, src/tzvjsvd.c, src/tsvjsvd.c, src/tcvjsvd.c and the parts of
// src/mtxio.c (open_ro_/open_wo_/resizef_/?read2_/?write2_/wwrite1_) and src/aalloc.c
// (?alloc2_) that they use. One source, compiled once per precision with VJ_CLI_KIND set
// to 'd', 'z', 's' or 'c'.
//
// Files (raw, column-major, no header; complex data interleaved re/im like C99 complex):
//   BaseName.G   input, M x N
//   BaseName.U2  U (the overwritten G), M x N      (U4 for J = 4)
//   BaseName.V2  V, N x N                          (V4 for J = 4)
//   BaseName.S2  sigma_j = fS_j 2^eS_j, N values of the reference's `wide` type (S4)
// The `wide` type is the reference's build choice (src/common.h:85-115): IEEE binary128
// (its default, WP=q) or, with VJ_WIDE=l in the environment, the x87 80-bit extended
// format in 16-byte slots (WP=l; the 6 padding bytes are written as zeros). Both are
// encoded here from the bits of (eS, fS), exactly, on any host.
//
// Standard output: one CSV line, as the reference's OpenMP build prints it:
//   real:    "BaseName",J,M,N,seconds,info
//   complex: "BaseName",J,M,N,split s,SVD s,info,merge V s,merge G s
// Exit codes follow the reference: 1 usage, 2 J (only 2 and 4) or pivot table, 3 M,
// 4 N (N <= M, N even, N/2 a multiple of 8 (FP64) or 16 (FP32)), 5 BaseName or reading
// G, 6-9 allocation, then one per failed output file (real: 10 S, 11 V, 12 U; complex:
// 10 S, 11-12 V, 13-14 U). Unlike the reference, a library-only failure of the SVD call
// (no usable GPU, a CUDA error: codes <= -100000) is reported on standard error after the
// CSV line and ends the program with exit code 15 before any output file is written.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "vecjac_gb300.h"

#ifndef VJ_CLI_KIND
#error VJ_CLI_KIND must be one of 'd', 'z', 's', 'c'
#endif

namespace {

constexpr char KIND = VJ_CLI_KIND;
constexpr bool CPLX = (KIND == 'z' || KIND == 'c');
constexpr bool FP64 = (KIND == 'd' || KIND == 'z');
using T = std::conditional<FP64, double, float>::type;
constexpr vj_fnat VL = FP64 ? 8u : 16u;  // lanes of the reference's vectors (VDL / VSL)
constexpr size_t ALIGN = 64u;            // the reference's VA

// strtoull with base detection; 0 for an empty string or trailing characters
// (src/common.c:26-31)
vj_fnat atoz(const char *s)
{
  char *e = nullptr;
  const vj_fnat z = (s && *s) ? (vj_fnat)strtoull(s, &e, 0) : 0u;
  return (e && *e) ? 0u : z;
}

std::string fname(const char *bn, const char *ex) { return std::string(bn) + "." + ex; }

int open_ro(const char *bn, const char *ex) { return open(fname(bn, ex).c_str(), O_RDONLY); }

int open_wo(const char *bn, const char *ex)
{
  return open(fname(bn, ex).c_str(), O_WRONLY | O_CREAT, S_IRUSR | S_IWUSR | S_IRGRP | S_IROTH);
}

bool resize(int fd, size_t sz) { return (ftruncate(fd, (off_t)sz) == 0) && (fsync(fd) == 0); }

// column j of an m x n matrix with leading dimension ld at file offset j m sizeof(E)
template <typename E> bool read_cols(int fd, vj_fnat m, vj_fnat n, E *A, vj_fnat ld)
{
  const size_t sz = (size_t)m * sizeof(E);
  for (vj_fnat j = 0; j < n; ++j)
    if (pread(fd, A + j * ld, sz, (off_t)(j * sz)) != (ssize_t)sz)
      return false;
  return true;
}

template <typename E> bool write_cols(int fd, vj_fnat m, vj_fnat n, const E *A, vj_fnat ld)
{
  const size_t sz = (size_t)m * sizeof(E);
  for (vj_fnat j = 0; j < n; ++j)
    if (pwrite(fd, A + j * ld, sz, (off_t)(j * sz)) != (ssize_t)sz)
      return false;
  return true;
}

template <typename E> E *alloc(size_t count)
{
  const size_t bytes = ((count * sizeof(E) + ALIGN - 1) / ALIGN) * ALIGN;
  void *p = aligned_alloc(ALIGN, bytes ? bytes : ALIGN);
  if (p)
    memset(p, 0, bytes ? bytes : ALIGN);
  return (E *)p;
}

// leading dimension: m rounded up to the vector length (src/aalloc.c dalloc2_/salloc2_)
vj_fnat lead(vj_fnat m) { return (m % VL) ? (m + (VL - m % VL)) : m; }

// f 2^e (f when e == 0) in the reference's wide type, 16 bytes little-endian. f and e come
// from the SVD: f a finite FP number (normally in [1, 2)), e integer-valued or -inf.
// Exact: f has at most 53 significant bits and both formats carry at least 64.
void wide_bytes(double f, double e, bool x87, unsigned char out[16])
{
  memset(out, 0, 16);
  // classes of scalb(f, e): 0 zero, 1 finite nonzero, 2 infinite, 3 NaN
  int cls;
  uint64_t M = 0;
  long long E = 0;
  const bool fin_e = std::isfinite(e);
  if (std::isnan(f) || std::isnan(e) || (fin_e && e != std::floor(e)) || (e > 0 && !fin_e && f == 0.0) ||
      (e < 0 && !fin_e && std::isinf(f)))
    cls = 3;
  else if (f == 0.0 || (e < 0 && !fin_e))
    cls = 0;
  else if (std::isinf(f) || !fin_e)
    cls = 2;
  else {
    int ef = 0;
    const double mf = std::frexp(std::fabs(f), &ef);  // [0.5, 1)
    M = (uint64_t)std::ldexp(mf, 53);                  // 53-bit integer, top bit set
    const double ec = std::fmax(-65536.0, std::fmin(65536.0, e));
    E = (long long)ef - 1 + (long long)ec;             // value = (M / 2^52) 2^E
    if (E > 16383)
      cls = 2;
    else if (E < -16382)
      cls = 0;  // below the normal range of both formats; unreachable from a double SVD
    else
      cls = 1;
  }
  const bool neg = (cls != 3) && std::signbit(f);
  const uint64_t sign = neg ? 1u : 0u;
  uint64_t lo = 0, hi = 0;
  if (x87) {
    // 64-bit significand with explicit integer bit, then sign and 15-bit exponent
    uint16_t se = (uint16_t)(sign << 15);
    if (cls == 1) {
      lo = M << 11;
      se |= (uint16_t)(E + 16383);
    }
    else if (cls == 2) {
      lo = 1ull << 63;
      se |= 0x7fff;
    }
    else if (cls == 3) {
      lo = 3ull << 62;  // quiet NaN
      se |= 0x7fff;
    }
    for (int k = 0; k < 8; ++k)
      out[k] = (unsigned char)(lo >> (8 * k));
    out[8] = (unsigned char)(se & 0xff);
    out[9] = (unsigned char)(se >> 8);
    return;
  }
  // binary128: sign, 15-bit exponent, 112-bit fraction (hidden integer bit)
  hi = sign << 63;
  if (cls == 1) {
    const uint64_t frac = M & ((1ull << 52) - 1u);  // 52 fraction bits -> bits 111..60
    hi |= ((uint64_t)(E + 16383) << 48) | (frac >> 4);
    lo = (frac & 0xfu) << 60;
  }
  else if (cls == 2)
    hi |= 0x7fffull << 48;
  else if (cls == 3)
    hi |= (0x7fffull << 48) | (1ull << 47);
  for (int k = 0; k < 8; ++k) {
    out[k] = (unsigned char)(lo >> (8 * k));
    out[8 + k] = (unsigned char)(hi >> (8 * k));
  }
}

double seconds_since(std::chrono::steady_clock::time_point t0)
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

vj_fint svd_call(vj_fnat m, vj_fnat n, T *Gr, vj_fnat ldGr, T *Gi, vj_fnat ldGi, T *Vr, vj_fnat ldVr, T *Vi,
                 vj_fnat ldVi, T *eS, T *fS, const unsigned *js, unsigned stp, unsigned swp, T *work,
                 unsigned *iwork)
{
#if VJ_CLI_KIND == 'd'
  (void)Gi, (void)ldGi, (void)Vi, (void)ldVi;
  return dvjsvd_(&m, &n, Gr, &ldGr, Vr, &ldVr, eS, fS, js, &stp, &swp, work, iwork);
#elif VJ_CLI_KIND == 's'
  (void)Gi, (void)ldGi, (void)Vi, (void)ldVi;
  return svjsvd_(&m, &n, Gr, &ldGr, Vr, &ldVr, eS, fS, js, &stp, &swp, work, iwork);
#elif VJ_CLI_KIND == 'z'
  return zvjsvd_(&m, &n, Gr, &ldGr, Gi, &ldGi, Vr, &ldVr, Vi, &ldVi, eS, fS, js, &stp, &swp, work, iwork);
#else
  return cvjsvd_(&m, &n, Gr, &ldGr, Gi, &ldGi, Vr, &ldVr, Vi, &ldVi, eS, fS, js, &stp, &swp, work, iwork);
#endif
}

// interleaved complex (re, im pairs, leading dimension ld in complex elements) <-> planes,
// through the library's zsplit_/zmerge_ (csplit_/cmerge_), as the reference's complex
// drivers call its own (src/tzvjsvd.c:69,137,163)
vj_fint split(vj_fnat m, vj_fnat n, const T *A, vj_fnat ld, T *Ar, T *Ai, vj_fnat ldp)
{
#if VJ_CLI_KIND == 'z'
  return zsplit_(&m, &n, A, &ld, Ar, &ldp, Ai, &ldp);
#elif VJ_CLI_KIND == 'c'
  return csplit_(&m, &n, A, &ld, Ar, &ldp, Ai, &ldp);
#else
  (void)m, (void)n, (void)A, (void)ld, (void)Ar, (void)Ai, (void)ldp;
  return -1;
#endif
}

vj_fint merge(vj_fnat m, vj_fnat n, const T *Ar, const T *Ai, vj_fnat ldp, T *A, vj_fnat ld)
{
#if VJ_CLI_KIND == 'z'
  return zmerge_(&m, &n, Ar, &ldp, Ai, &ldp, A, &ld);
#elif VJ_CLI_KIND == 'c'
  return cmerge_(&m, &n, Ar, &ldp, Ai, &ldp, A, &ld);
#else
  (void)m, (void)n, (void)Ar, (void)Ai, (void)ldp, (void)A, (void)ld;
  return -1;
#endif
}

// the whole file of a real (CPLX false: E = T) or complex (E = 2 T per element) matrix
bool write_matrix(const char *bn, const char *ex, vj_fnat m, vj_fnat n, const T *A, vj_fnat ld)
{
  const int fd = open_wo(bn, ex);
  if (fd < 0)
    return false;
  const size_t esz = sizeof(T) * (CPLX ? 2u : 1u);
  bool ok = resize(fd, (size_t)m * n * esz);
  if (ok) {
    if (CPLX) {
      struct C2 {
        T re, im;
      };
      ok = write_cols<C2>(fd, m, n, (const C2 *)A, ld);
    }
    else
      ok = write_cols<T>(fd, m, n, A, ld);
  }
  return (close(fd) == 0) && ok;
}

}  // namespace

int main(int argc, char *argv[])
{
  if (argc != 5) {
    (void)fprintf(stderr, "%s J M N BaseName\n", *argv);
    return 1;
  }
  const vj_fnat m = atoz(argv[2]);
  if (!m)
    return 3;
  const vj_fnat n = atoz(argv[3]);
  if (!n || n > m || (n & 1u) || ((n >> 1u) % VL))
    return 4;
  const long j = atol(argv[1]);
  if (j != 2l && j != 4l)
    return 2;
  unsigned stp = 0u;
  unsigned *const js = pjs(j, (unsigned)n, &stp);
  if (!js) {
    (void)fprintf(stderr, "%s: no pivot table (it is generated on the GPU)\n", *argv);
    return 2;
  }
  const char *const bn = argv[4];
  if (!*bn)
    return 5;
  const char *const tag = (j == 2l) ? "2" : "4";
  const int gd = open_ro(bn, "G");
  if (gd < 0)
    return 5;

  const vj_fnat ldG = lead(m), ldV = lead(n);
  T *const G = alloc<T>((size_t)ldG * n * (CPLX ? 2u : 1u));  // interleaved for complex data
  if (!G)
    return 6;
  bool rd;
  if (CPLX) {
    struct C2 {
      T re, im;
    };
    rd = read_cols<C2>(gd, m, n, (C2 *)G, ldG);
  }
  else
    rd = read_cols<T>(gd, m, n, G, ldG);
  if (!rd || close(gd))
    return 5;

  T *Gr = G, *Gi = nullptr, *Vr = nullptr, *Vi = nullptr;
  double ts = 0.0;
  if (CPLX) {
    Gr = alloc<T>((size_t)ldG * n);
    Gi = alloc<T>((size_t)ldG * n);
    if (!Gr || !Gi)
      return 6;
    const auto t0 = std::chrono::steady_clock::now();
    if (split(m, n, G, ldG, Gr, Gi, ldG) < 0)
      return 6;
    ts = seconds_since(t0);
  }
  Vr = alloc<T>((size_t)ldV * n);
  if (!Vr)
    return 7;
  if (CPLX) {
    Vi = alloc<T>((size_t)ldV * n);
    if (!Vi)
      return 7;
  }
  // eS, fS and work: 7 n (real) / 9 n (complex) elements, as the reference's drivers
  T *const w = alloc<T>((size_t)n * (CPLX ? 9u : 7u));
  if (!w)
    return 8;
  T *const eS = w, *const fS = w + n, *const work = w + 2 * n;
  unsigned *const iwork = alloc<unsigned>((size_t)(n / VL));
  if (!iwork)
    return 9;
  iwork[0] = 0u;  // V := I

  const unsigned swp = 999u;
  const auto t1 = std::chrono::steady_clock::now();
  const vj_fint o = svd_call(m, n, Gr, ldG, Gi, ldG, Vr, ldV, Vi, ldV, eS, fS, js, stp, swp, work, iwork);
  const double tj = seconds_since(t1);
  if (!CPLX) {
    (void)fprintf(stdout, "\"%s\",%1ld,%4llu,%4llu,%15.9f,%3lld\n", bn, j, (unsigned long long)m,
                  (unsigned long long)n, tj, (long long)o);
    (void)fflush(stdout);
  }
  if (o <= VJ_ERR_NO_GPU) {
    if (CPLX) {
      (void)fprintf(stdout, "\"%s\",%1ld,%4llu,%4llu,%15.9f,%15.9f,%3lld,%15.9f,%15.9f\n", bn, j,
                    (unsigned long long)m, (unsigned long long)n, ts, tj, (long long)o, 0.0, 0.0);
      (void)fflush(stdout);
    }
    (void)fprintf(stderr, "%s: the SVD failed in the library (%lld: %s)\n", *argv, (long long)o,
                  (o == VJ_ERR_NO_GPU) ? "no usable GPU" : (o == VJ_ERR_CUDA) ? "CUDA error" :
                  (o == VJ_ERR_NOMEM) ? "out of memory" : "bad argument");
    return 15;
  }
  free(iwork);

  // sigma in the wide type
  {
    const bool x87 = getenv("VJ_WIDE") && !strcmp(getenv("VJ_WIDE"), "l");
    unsigned char *const ws = alloc<unsigned char>((size_t)n * 16u);
    if (!ws)
      return 10;
    for (vj_fnat i = 0; i < n; ++i)
      wide_bytes((double)fS[i], (double)eS[i], x87, ws + 16u * i);
    const int sd = open_wo(bn, (std::string("S") + tag).c_str());
    if (sd < 0)
      return 10;
    const size_t sz = (size_t)n * 16u;
    const bool ok = resize(sd, sz) && (write(sd, ws, sz) == (ssize_t)sz);
    if (close(sd) || !ok)
      return 10;
    free(ws);
  }
  free(w);

  double tv = 0.0, tg = 0.0;
  if (CPLX) {
    T *const V = alloc<T>((size_t)ldV * n * 2u);
    if (!V)
      return 11;
    auto t2 = std::chrono::steady_clock::now();
    if (merge(n, n, Vr, Vi, ldV, V, ldV) < 0)
      return 11;
    tv = seconds_since(t2);
    if (!write_matrix(bn, (std::string("V") + tag).c_str(), n, n, V, ldV))
      return 12;
    free(V);
    t2 = std::chrono::steady_clock::now();
    if (merge(m, n, Gr, Gi, ldG, G, ldG) < 0)
      return 13;
    tg = seconds_since(t2);
    if (!write_matrix(bn, (std::string("U") + tag).c_str(), m, n, G, ldG))
      return 14;
    free(Vi);
    free(Gi);
    free(Gr);
    (void)fprintf(stdout, "\"%s\",%1ld,%4llu,%4llu,%15.9f,%15.9f,%3lld,%15.9f,%15.9f\n", bn, j,
                  (unsigned long long)m, (unsigned long long)n, ts, tj, (long long)o, tv, tg);
    (void)fflush(stdout);
  }
  else {
    if (!write_matrix(bn, (std::string("V") + tag).c_str(), n, n, Vr, ldV))
      return 11;
    if (!write_matrix(bn, (std::string("U") + tag).c_str(), m, n, G, ldG))
      return 12;
  }
  free(Vr);
  free(G);
  free(js);
  return EXIT_SUCCESS;
}
