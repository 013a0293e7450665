// Closed forms of the two parallel pivot orderings (see pjs.cu): pair k of step s.
#pragma once

namespace vj {

// round-robin (Brent-Luk) ordering, n-1 steps: s with n-1, (s+k) mod (n-1) with (s-k) mod (n-1)
__host__ __device__ __forceinline__ void pair_rr(unsigned n, unsigned s, unsigned k, unsigned &p, unsigned &q)
{
  const unsigned N = n - 1u;
  unsigned a, b;
  if (!k) {
    a = s;
    b = N;
  }
  else {
    a = (s + k) % N;
    b = (s + N - k) % N;
  }
  p = (a < b) ? a : b;
  q = (a < b) ? b : a;
}

// modulus (Luk-Park) ordering, n steps: the pairs i < j with i + j = s (mod n) in
// increasing i, then (for even s) the couple s/2, s/2 + n/2
__host__ __device__ __forceinline__ void pair_mod(unsigned n, unsigned s, unsigned k, unsigned &p, unsigned &q)
{
  const unsigned half = n >> 1;
  const unsigned c1 = (s + 1u) >> 1;
  const unsigned lo2 = s + 1u, hi2 = (s + n + 1u) >> 1;
  const unsigned c2 = (hi2 > lo2) ? (hi2 - lo2) : 0u;
  if (k < c1) {
    p = k;
    q = s - k;
  }
  else if (k < c1 + c2) {
    p = lo2 + (k - c1);
    q = s + n - p;
  }
  else {
    p = s >> 1;
    q = p + half;
  }
}

}  // namespace vj
