// Accuracy drivers of the batched 2x2 EVD with the reference's interface, over the drop-in
// C ABI:
//
//   t?bjac2.exe filename lg(batch_size) #batches
//
// replaces src/tdbjac2.c, src/tzbjac2.c, src/tsbjac2.c, src/tcbjac2.c. One source, compiled
// once per precision with VJ_CLI_KIND set to 'd', 'z', 's' or 'c'.
//
// Input (the files of the reference's generator, src/gen2rand.c): raw arrays of the
// precision's real type, batch j at element offset j * 2^lg:
//   filename.f  a11,  filename.g  a22,  filename.h  a21 (real)  or  .r / .j  Re / Im a21,
//   filename.k  the first and  filename.l  the second exact eigenvalue.
// For each batch the driver calls ?bjac2_ with n = -2^lg (cosines and sines) and prints
//   "B","Ts","ORT","REN","RLN","RLX","RLM"
// B the batch, Ts the seconds of the call, then in `long double`:
//   ORT  max |c^2 + |s|^2 - 1|                               (orthogonality of U)
//   REN  max ||U diag(l1, l2) U^H - A||_F / ||A||_F           (relative residual)
//   RLN  max ||(L1, L2) - (l1, l2)|| / ||(l1, l2)||           (eigenvalues, sorted by |.|)
//   RLX  max relative error of the larger, RLM of the smaller |eigenvalue|
// printed as the reference prints long doubles: sign or blank, 21 fraction digits, a
// four-digit exponent (30 characters). The complex drivers also print, on standard
// error, the first element with the largest ORT and its data, as the reference's do.
// `long double` is the reference's `wide` of its WP=l build on x86 hosts (x87); on hosts
// whose long double is binary128 the metrics are evaluated in that format instead.
// Errors: usage or a batch size that is not a multiple of 8 (FP64) / 16 (FP32), or an
// input file that cannot be opened: a message and exit status 1; a short read: status 1.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include <fcntl.h>
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
using W = long double;
constexpr size_t VL = FP64 ? 8u : 16u;

size_t atoz(const char *s)
{
  char *e = nullptr;
  const size_t z = (s && *s) ? (size_t)strtoull(s, &e, 0) : 0u;
  return (e && *e) ? 0u : z;
}

// the reference's print form of a long double: "% .21LE" with the exponent widened to four
// digits, non-finite values left-aligned in 30 characters
std::string wfmt(W x)
{
  char b[64];
  if (!std::isfinite(x)) {
    snprintf(b, sizeof(b), "% LE", x);
    std::string s(b);
    s.resize(30, ' ');
    return s;
  }
  snprintf(b, sizeof(b), "% .21LE", x);
  std::string s(b);
  const size_t e = s.rfind('E');
  const std::string mant = s.substr(0, e + 2);  // up to and including the exponent sign
  const long ex = strtol(s.c_str() + e + 2, nullptr, 10);
  snprintf(b, sizeof(b), "%04ld", ex);
  return mant + b;
}

const W SQRT2 = std::sqrt((W)2);

W fro_r(W a11, W a22, W a21) { return std::hypot(std::hypot(a11, a22), SQRT2 * a21); }
W fro_c(W a11, W a22, W a21r, W a21i) { return std::hypot(std::hypot(a11, a22), SQRT2 * std::hypot(a21r, a21i)); }

// |c^2 + s^2 - 1| with the product c^2 rounded once and the rest fused
W orth(W c, W s) { return std::fabs(std::fma(s + (W)1, s - (W)1, c * c)); }

// the diagonal of U diag(l1, l2) U^H - A, through tan or cot of the angle (the smaller)
void diag_err(W a11, W a22, W c, W s, W l1, W l2, W &d11, W &d22)
{
  if (std::fabs(c) >= std::fabs(s)) {
    const W t = s / c, t2 = t * t, c2 = c * c;
    d11 = std::fma(std::fma(l2, t2, l1), c2, -a11);
    d22 = std::fma(std::fma(l1, t2, l2), c2, -a22);
  }
  else {
    const W g = c / s, g2 = g * g, s2 = s * s;
    d11 = std::fma(std::fma(l1, g2, l2), s2, -a11);
    d22 = std::fma(std::fma(l2, g2, l1), s2, -a22);
  }
}

W resid_r(W a11, W a22, W a21, W c, W s, W l1, W l2)
{
  W d11, d22;
  diag_err(a11, a22, c, s, l1, l2, d11, d22);
  const W d21 = std::fma(l1 - l2, c * s, -a21);
  return std::fmax(fro_r(d11, d22, d21) / fro_r(a11, a22, a21), (W)0);
}

W resid_c(W a11, W a22, W a21r, W a21i, W c, W sr, W si, W l1, W l2)
{
  const W s = std::hypot(sr, si);
  W d11, d22;
  diag_err(a11, a22, c, s, l1, l2, d11, d22);
  const W l = l1 - l2;
  const W d21r = std::fma(l, c * sr, -a21r), d21i = std::fma(l, c * si, -a21i);
  return std::fmax(fro_c(d11, d22, d21r, d21i) / fro_c(a11, a22, a21r, a21i), (W)0);
}

// computed (L1, L2) against exact (x1, x2), compared by magnitude; returns the relative
// error of the pair and sets those of the larger and of the smaller one
W eig_err(W L1, W L2, W x1, W x2, W &rel_big, W &rel_small)
{
  L1 = std::fabs(L1);
  L2 = std::fabs(L2);
  x1 = std::fabs(x1);
  x2 = std::fabs(x2);
  const W Ls = (L1 <= L2) ? L1 : L2, Lb = (L1 <= L2) ? L2 : L1;
  const W xs = (x1 <= x2) ? x1 : x2, xb = (x1 <= x2) ? x2 : x1;
  const W eb = (Lb <= xb) ? (xb - Lb) : (Lb - xb), es = (Ls <= xs) ? (xs - Ls) : (Ls - xs);
  rel_big = std::fmax(eb / xb, (W)0);
  rel_small = std::fmax(es / xs, (W)0);
  return std::fmax(std::hypot(eb, es) / std::hypot(xb, xs), (W)0);
}

vj_fint bjac2_call(vj_fint n, const T *a11, const T *a22, const T *a21r, const T *a21i, T *c, T *cat, T *sat,
                   T *l1, T *l2, unsigned *p)
{
#if VJ_CLI_KIND == 'd'
  (void)a21i, (void)sat;
  return dbjac2_(&n, a11, a22, a21r, c, cat, l1, l2, p);
#elif VJ_CLI_KIND == 's'
  (void)a21i, (void)sat;
  return sbjac2_(&n, a11, a22, a21r, c, cat, l1, l2, p);
#elif VJ_CLI_KIND == 'z'
  return zbjac2_(&n, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
#else
  return cbjac2_(&n, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
#endif
}

bool read_batch(int fd, T *dst, size_t n, size_t j)
{
  const size_t bytes = n * sizeof(T);
  return pread(fd, dst, bytes, (off_t)(j * bytes)) == (ssize_t)bytes;
}

}  // namespace

int main(int argc, char *argv[])
{
  if (argc != 4) {
    (void)fprintf(stderr, "%s filename lg(batch_size) #batches\n", *argv);
    return EXIT_FAILURE;
  }
  const size_t n = (size_t)1u << atoz(argv[2]);
  if (n % VL) {
    (void)fprintf(stderr, "batch_size has to be a multiple of %zu.\n", VL);
    return EXIT_FAILURE;
  }
  const size_t b = atoz(argv[3]);
  if (!b)
    return EXIT_SUCCESS;
  const std::string base(argv[1]);
  const char *names = CPLX ? "klfgrj" : "klfgh";
  int fd[6] = {-1, -1, -1, -1, -1, -1};
  for (int k = 0; names[k]; ++k) {
    const std::string fn = base + "." + names[k];
    fd[k] = open(fn.c_str(), O_RDONLY);
    if (fd[k] < 0) {
      (void)fprintf(stderr, "Cannot open %s for reading!\n", fn.c_str());
      return EXIT_FAILURE;
    }
  }
  const int fk = fd[0], fl = fd[1], ff = fd[2], fg = fd[3], fr = fd[4], fj = CPLX ? fd[5] : -1;
  std::vector<T> a11(n), a22(n), a21r(n), a21i(CPLX ? n : 0), c(n), cat(n), sat(CPLX ? n : 0), l1(n), l2(n), x1(n),
      x2(n);
  std::vector<unsigned> p(n / VL);
  (void)fprintf(stdout, "\"B\",\"Ts\",\"ORT\",\"REN\",\"RLN\",\"RLX\",\"RLM\"\n");
  (void)fflush(stdout);
  const int bw = (b <= 10u) ? 1 : (b <= 100u) ? 2 : (b <= 1000u) ? 3 : 0;
  for (size_t j = 0; j < b; ++j) {
    (void)fprintf(stdout, "%*zu", bw, j);
    (void)fflush(stdout);
    if (!read_batch(ff, a11.data(), n, j) || !read_batch(fg, a22.data(), n, j) || !read_batch(fr, a21r.data(), n, j) ||
        (CPLX && !read_batch(fj, a21i.data(), n, j)))
      return EXIT_FAILURE;
    (void)fprintf(stdout, ",");
    (void)fflush(stdout);
    const auto t0 = std::chrono::steady_clock::now();
    const vj_fint r = bjac2_call(-(vj_fint)n, a11.data(), a22.data(), a21r.data(), CPLX ? a21i.data() : nullptr,
                                 c.data(), cat.data(), CPLX ? sat.data() : nullptr, l1.data(), l2.data(), p.data());
    const double ts = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (r <= VJ_ERR_NO_GPU) {
      (void)fprintf(stderr, "%s: the 2x2 EVD failed in the library (%lld)\n", *argv, (long long)r);
      return EXIT_FAILURE;
    }
    (void)fprintf(stdout, "%15.9f,", ts);
    (void)fflush(stdout);
    W o = 0, re = 0;
    size_t ix = n;
    for (size_t i = 0; i < n; ++i) {
      const W oi = CPLX ? orth((W)c[i], std::hypot((W)cat[i], (W)sat[i])) : orth((W)c[i], (W)cat[i]);
      const W ri = CPLX ? resid_c(a11[i], a22[i], a21r[i], a21i[i], c[i], cat[i], sat[i], l1[i], l2[i])
                        : resid_r(a11[i], a22[i], a21r[i], c[i], cat[i], l1[i], l2[i]);
      // the maximum (NaN ignored) and the first element that attains it
      if (oi > o) {
        o = oi;
        ix = i;
      }
      else if (oi == o && ix == n)
        ix = i;
      re = std::fmax(re, ri);
    }
    (void)fprintf(stdout, "%s,%s", wfmt(o).c_str(), wfmt(re).c_str());
    (void)fflush(stdout);
    if (CPLX && ix < n)
      (void)fprintf(stderr, "%zu,%zu,%s;%s,%s,(%s,%s);%s,(%s,%s);%s,%s\n", j, ix, wfmt(o).c_str(),
                    wfmt(a11[ix]).c_str(), wfmt(a22[ix]).c_str(), wfmt(a21r[ix]).c_str(), wfmt(a21i[ix]).c_str(),
                    wfmt(c[ix]).c_str(), wfmt(cat[ix]).c_str(), wfmt(sat[ix]).c_str(), wfmt(l1[ix]).c_str(),
                    wfmt(l2[ix]).c_str());
    if (!read_batch(fk, x1.data(), n, j) || !read_batch(fl, x2.data(), n, j))
      return EXIT_FAILURE;
    (void)fprintf(stdout, ",");
    W rn = 0, rx = 0, rm = 0;
    for (size_t i = 0; i < n; ++i) {
      W big = 0, small = 0;
      rn = std::fmax(rn, eig_err(l1[i], l2[i], x1[i], x2[i], big, small));
      rx = std::fmax(rx, big);
      rm = std::fmax(rm, small);
    }
    (void)fprintf(stdout, "%s,%s,%s\n", wfmt(rn).c_str(), wfmt(rx).c_str(), wfmt(rm).c_str());
    (void)fflush(stdout);
  }
  for (int k = 0; k < 6; ++k)
    if (fd[k] >= 0)
      (void)close(fd[k]);
  return EXIT_SUCCESS;
}
