// Host harness for the closed-form pivot pairs of vecjac_gb300/csrc/pjs.cuh, which the
// GPU table generator (pjs.cu) and the batched SVD kernel (batch.cu) evaluate on the
// device: compiled here with the header's __host__ __device__ functions as plain host
// code, every pair (n, step, k) for every even n up to NMAX is compared with the oracle's
// loop-built tables (vjo_pjs) and checked against the pair contract (each step a
// permutation of 0..n-1 read as pairs with p < q; every pair once per sweep, the modulus
// ordering's n/2 couples (i, i + n/2) twice).
//
//   pjs_host NMAX  ->  "n_checked mismatches contract_violations"
#include <cstdio>
#include <cstdlib>
#include <vector>

#define __host__
#define __device__
#define __forceinline__ inline
#include "../vecjac_gb300/csrc/pjs.cuh"

extern "C" unsigned *vjo_pjs(long id, unsigned n, unsigned *stp);

int main(int argc, char **argv)
{
  const unsigned NMAX = (argc > 1) ? (unsigned)atoi(argv[1]) : 1024u;
  long long bad = 0, contract = 0, checked = 0;
  for (long id : {2l, 4l})
    for (unsigned n = 2; n <= NMAX; n += 2) {
      unsigned stp = 0;
      unsigned *t = vjo_pjs(id, n, &stp);
      if (!t || stp != ((id == 2l) ? n - 1u : n)) {
        ++bad;
        continue;
      }
      std::vector<unsigned char> seen((size_t)n * n, 0);
      for (unsigned s = 0; s < stp; ++s) {
        std::vector<unsigned char> used(n, 0);
        for (unsigned k = 0; k < n / 2; ++k) {
          unsigned p, q;
          if (id == 2l)
            vj::pair_rr(n, s, k, p, q);
          else
            vj::pair_mod(n, s, k, p, q);
          bad += (p != t[(size_t)s * n + 2 * k]) || (q != t[(size_t)s * n + 2 * k + 1]);
          if (p >= q || q >= n || used[p] || used[q]) {
            ++contract;
            continue;
          }
          used[p] = used[q] = 1;
          ++seen[(size_t)p * n + q];
        }
      }
      // every pair at least once per sweep; the round-robin's n-1 steps hold each pair
      // exactly once, the modulus ordering's n steps hold the n/2 couples (i, i + n/2)
      // twice (once as the couple of an even step, once as a pair summing to i + n/2)
      long long pairs = 0, repeats = 0;
      for (size_t i = 0; i < seen.size(); ++i) {
        pairs += seen[i] ? 1 : 0;
        repeats += (seen[i] > 1) ? (seen[i] - 1) : 0;
      }
      contract += (pairs != (long long)n * (n - 1) / 2);
      contract += (repeats != ((id == 2l) ? 0 : (long long)n / 2));
      free(t);
      ++checked;
    }
  printf("%lld %lld %lld\n", checked, bad, contract);
  return 0;
}
