// Host harness for the pair rotation of the mixed SVD's plain-dot FP64 sweeps
// (vecjac_gb300/csrc/presweep.cuh: hestenes, pair_rot, rot_elem, tracked_norms,
// pair_rotation), compiled with g++ over tests/cuda_host_shim.h. Whole one-sided Jacobi
// sweeps are run on seeded matrices A = Q1 diag(sigma) Q2^T (or ^H) with the kernel's own
// pair arithmetic, serially over the pairs of each round-robin step, in two modes:
//   plain    no column scales, norms recomputed at every step (the unscaled form);
//   scaled   column scales with short-form rotations and tracked squared norms, the scales
//            applied to the columns at the end of each sweep (the FP64 sweeps' form).
// Output, one line per run:
//   mode sweeps max_rel_sigma_vs_exact orth_V_fro residual_rel short general tracked exact
// (short/general: rotations in each form; tracked/exact: steps that used tracked norms or
// recomputed them).
//
//   presweep_host KIND M N SPECTRUM SEED    KIND r|c; SPECTRUM graded|clustered|zerocols
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cuda_host_shim.h"

// the two atomics the pair code uses (one host thread: plain read-modify-write)
static inline unsigned atomicAdd(unsigned *p, unsigned v)
{
  const unsigned o = *p;
  *p = o + v;
  return o;
}
static inline unsigned atomicMax(unsigned *p, unsigned v)
{
  const unsigned o = *p;
  if (v > o)
    *p = v;
  return o;
}

#include "../vecjac_gb300/csrc/presweep.cuh"

static uint64_t g_s;
static double urand()
{
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return (double)(g_s >> 11) * (1.0 / 9007199254740992.0);
}
static double nrand()
{
  double u = urand(), v = urand();
  if (u < 1e-300)
    u = 1e-300;
  return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
}

// column-major complex matrix in planes (im empty for real data)
struct Mat {
  int r, c;
  std::vector<double> re, im;
  Mat(int r_, int c_, bool cx) : r(r_), c(c_), re((size_t)r_ * c_, 0.0), im(cx ? (size_t)r_ * c_ : 0, 0.0) {}
  double &R(int i, int j) { return re[(size_t)j * r + i]; }
  double &I(int i, int j) { return im[(size_t)j * r + i]; }
};

// orthonormal (unitary) columns by modified Gram-Schmidt, twice
static Mat haar(int r, int c, bool cx)
{
  Mat Q(r, c, cx);
  for (int j = 0; j < c; ++j)
    for (int i = 0; i < r; ++i) {
      Q.R(i, j) = nrand();
      if (cx)
        Q.I(i, j) = nrand();
    }
  for (int pass = 0; pass < 2; ++pass)
    for (int j = 0; j < c; ++j) {
      for (int k = 0; k < j; ++k) {
        double sr = 0, si = 0;  // <q_k, q_j> = q_k^H q_j
        for (int i = 0; i < r; ++i) {
          sr += Q.R(i, k) * Q.R(i, j) + (cx ? Q.I(i, k) * Q.I(i, j) : 0.0);
          si += cx ? (Q.R(i, k) * Q.I(i, j) - Q.I(i, k) * Q.R(i, j)) : 0.0;
        }
        for (int i = 0; i < r; ++i) {
          const double kr = Q.R(i, k), ki = cx ? Q.I(i, k) : 0.0;
          Q.R(i, j) -= sr * kr - si * ki;
          if (cx)
            Q.I(i, j) -= sr * ki + si * kr;
        }
      }
      double nn = 0;
      for (int i = 0; i < r; ++i)
        nn += Q.R(i, j) * Q.R(i, j) + (cx ? Q.I(i, j) * Q.I(i, j) : 0.0);
      nn = std::sqrt(nn);
      for (int i = 0; i < r; ++i) {
        Q.R(i, j) /= nn;
        if (cx)
          Q.I(i, j) /= nn;
      }
    }
  return Q;
}

struct Result {
  int sweeps;
  double rel_sigma, orth, resid;
  long nshort, ngeneral, ntracked, nexact;
};

static Result run(const Mat &A, const std::vector<double> &sig, bool cx, bool scaled)
{
  const int m = A.r, n = A.c;
  Mat G = A, W(n, n, cx);
  for (int j = 0; j < n; ++j)
    W.R(j, j) = 1.0;
  const double tol = 0.5 * std::sqrt((double)m) * 1.1102230246251565e-16;
  std::vector<double> dsc(n, 1.0), nrm(n, -1.0);
  std::vector<int> idx(n);
  Result res{};
  unsigned cnt[2];
  for (int sw = 0; sw < 40; ++sw) {
    for (int j = 0; j < n; ++j) {
      idx[j] = j;
      dsc[j] = 1.0;
      nrm[j] = -1.0;
    }
    cnt[0] = cnt[1] = 0u;
    for (int st = 0; st < n - 1; ++st) {
      for (int k = 0; k < n / 2; ++k) {
        int p = idx[k], q = idx[n - 1 - k];
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double nab[2];
        vj::tracked_norms(scaled ? nrm.data() : (double *)nullptr, (unsigned)p, (unsigned)q, nab);
        const bool norms = nab[0] < 0.0;
        double a = 0, b = 0, cr = 0, ci = 0;
        for (int i = 0; i < m; ++i) {
          const double xr = G.R(i, p), yr = G.R(i, q), xi = cx ? G.I(i, p) : 0.0, yi = cx ? G.I(i, q) : 0.0;
          if (norms) {
            a = std::fma(xr, xr, a);
            b = std::fma(yr, yr, b);
            if (cx) {
              a = std::fma(xi, xi, a);
              b = std::fma(yi, yi, b);
            }
          }
          cr = std::fma(xr, yr, cr);
          if (cx) {
            cr = std::fma(xi, yi, cr);
            ci = std::fma(xr, yi, ci);
            ci = std::fma(-xi, yr, ci);
          }
        }
        (norms ? res.nexact : res.ntracked)++;
        vj::Rot<double> r;
        vj::pair_rotation(a, b, cr, ci, tol, cnt, scaled ? dsc.data() : (double *)nullptr, (unsigned)p,
                          (unsigned)q, &r, scaled ? nrm.data() : (double *)nullptr, nab);
        if (!r.go)
          continue;
        (r.shrt ? res.nshort : res.ngeneral)++;
        auto rot2 = [&](Mat &X) {
          for (int i = 0; i < X.r; ++i) {
            double pr = X.R(i, p), qr = X.R(i, q), pi = cx ? X.I(i, p) : 0.0, qi = cx ? X.I(i, q) : 0.0;
            if (cx)
              vj::rot_elem<double, true>(r, pr, pi, qr, qi);
            else
              vj::rot_elem<double, false>(r, pr, pi, qr, qi);
            const int dp = r.swap ? q : p, dq = r.swap ? p : q;
            X.R(i, dp) = pr;
            X.R(i, dq) = qr;
            if (cx) {
              X.I(i, dp) = pi;
              X.I(i, dq) = qi;
            }
          }
        };
        rot2(G);
        rot2(W);
      }
      // round robin: keep the first index, rotate the others
      const int last = idx[n - 1];
      for (int j = n - 1; j > 1; --j)
        idx[j] = idx[j - 1];
      idx[1] = last;
    }
    if (scaled)
      for (int j = 0; j < n; ++j)
        if (dsc[j] != 1.0) {
          for (int i = 0; i < m; ++i) {
            G.R(i, j) *= dsc[j];
            if (cx)
              G.I(i, j) *= dsc[j];
          }
          for (int i = 0; i < n; ++i) {
            W.R(i, j) *= dsc[j];
            if (cx)
              W.I(i, j) *= dsc[j];
          }
        }
    res.sweeps = sw + 1;
    if (!cnt[0])
      break;
  }
  // sigma = column norms of G, sorted descending, against the construction
  std::vector<double> s(n);
  for (int j = 0; j < n; ++j) {
    double t = 0;
    for (int i = 0; i < m; ++i)
      t += G.R(i, j) * G.R(i, j) + (cx ? G.I(i, j) * G.I(i, j) : 0.0);
    s[j] = std::sqrt(t);
  }
  std::sort(s.begin(), s.end(), [](double x, double y) { return x > y; });
  res.rel_sigma = 0;
  for (int j = 0; j < n; ++j)
    if (sig[j] > 0)
      res.rel_sigma = std::max(res.rel_sigma, std::fabs(s[j] - sig[j]) / sig[j]);
    else
      res.rel_sigma = std::max(res.rel_sigma, s[j] / sig[0]);
  // ||W^H W - I||_F and max |A W - G| / max |A|
  double of = 0;
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) {
      double sr = 0, si = 0;
      for (int i = 0; i < n; ++i) {
        sr += W.R(i, j) * W.R(i, k) + (cx ? W.I(i, j) * W.I(i, k) : 0.0);
        si += cx ? (W.R(i, j) * W.I(i, k) - W.I(i, j) * W.R(i, k)) : 0.0;
      }
      sr -= (j == k) ? 1.0 : 0.0;
      of += sr * sr + si * si;
    }
  res.orth = std::sqrt(of);
  double amax = 0, rmax = 0;
  Mat &Am = const_cast<Mat &>(A);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      amax = std::max(amax, std::hypot(Am.R(i, j), cx ? Am.I(i, j) : 0.0));
      double sr = 0, si = 0;
      for (int k = 0; k < n; ++k) {
        const double ar = Am.R(i, k), ai = cx ? Am.I(i, k) : 0.0, wr = W.R(k, j), wi = cx ? W.I(k, j) : 0.0;
        sr += ar * wr - ai * wi;
        si += ar * wi + ai * wr;
      }
      rmax = std::max(rmax, std::hypot(sr - G.R(i, j), si - (cx ? G.I(i, j) : 0.0)));
    }
  res.resid = rmax / amax;
  return res;
}

int main(int argc, char **argv)
{
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s r|c M N graded|clustered|zerocols SEED\n", argv[0]);
    return 2;
  }
  const bool cx = argv[1][0] == 'c';
  const int m = std::atoi(argv[2]), n = std::atoi(argv[3]);
  const char *spec = argv[4];
  g_s = 0x9E3779B97F4A7C15ull ^ (uint64_t)std::atoll(argv[5]);
  std::vector<double> sig(n);
  for (int j = 0; j < n; ++j) {
    if (!std::strcmp(spec, "clustered"))
      sig[j] = (j < n / 2) ? 1.0 : 1.0 + 1e-9 * j;  // two clusters of (nearly) equal values
    else
      sig[j] = std::pow(10.0, -6.0 * urand());
    if (!std::strcmp(spec, "zerocols") && j >= n - 4)
      sig[j] = 0.0;  // rank n - 4
  }
  std::sort(sig.begin(), sig.end(), [](double x, double y) { return x > y; });
  const Mat U = haar(m, n, cx), V = haar(n, n, cx);
  Mat A(m, n, cx);  // U diag(sigma) V^H
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      double sr = 0, si = 0;
      for (int k = 0; k < n; ++k) {
        const double ur = U.re[(size_t)k * m + i] * sig[k], ui = cx ? U.im[(size_t)k * m + i] * sig[k] : 0.0;
        const double vr = V.re[(size_t)k * n + j], vi = cx ? -V.im[(size_t)k * n + j] : 0.0;  // conj(V)_{j,k}
        sr += ur * vr - ui * vi;
        si += ur * vi + ui * vr;
      }
      A.R(i, j) = sr;
      if (cx)
        A.I(i, j) = si;
    }
  for (int mode = 0; mode < 2; ++mode) {
    const Result r = run(A, sig, cx, mode == 1);
    std::printf("%s %d %.3e %.3e %.3e %ld %ld %ld %ld\n", mode ? "scaled" : "plain", r.sweeps, r.rel_sigma, r.orth,
                r.resid, r.nshort, r.ngeneral, r.ntracked, r.nexact);
  }
  return 0;
}
