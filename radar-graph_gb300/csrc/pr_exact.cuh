// Exact sums of FP64 PageRank contributions on the integer pipes.
//
// PR_F (PageRank.C:30-72) adds p_curr[s]/deg(s) into p_next[d] in double
// precision.  Here every contribution is that same IEEE quotient, and a
// vertex's incoming sum is formed EXACTLY as a 128-bit fixed-point integer
// (value * 2^124) and rounded to the nearest double once, so
//   - each rank is the correctly rounded sum of the reference's doubles
//     (the reference's own order-dependent FP64 additions differ from it by
//     their rounding errors only), and
//   - sums are independent of the order of the additions: results are
//     deterministic and identical in every schedule that pulls.
// Range: values in [0, 16).  Exactness: a double >= 2^-72 converts exactly;
// PageRank contributions are at least (0.15/n)/deg > 2^-72 for every graph
// with n, m < 2^32, so every sum is exact.  Smaller terms would be truncated
// below 2^-124.
//
// GB300 issues one FP64 instruction per 16 lane-operations of an integer
// instruction, so the per-edge additions stay on the integer pipes; the FP64
// work is per vertex (the quotient, the damping step, |p - p'|).
#pragma once

#include <math.h>
#include <stdint.h>

namespace rg {

constexpr int kPrFrac = 124;  // fraction bits of the fixed-point sums

struct alignas(16) U128 {
  unsigned long long lo, hi;
};

__host__ __device__ __forceinline__ void add128(U128& a, const U128& b) {
#ifdef __CUDA_ARCH__
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(a.lo), "+l"(a.hi) : "l"(b.lo), "l"(b.hi));
#else
  a.lo += b.lo;
  a.hi += b.hi + (a.lo < b.lo ? 1ull : 0ull);
#endif
}

__host__ __device__ __forceinline__ int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

__host__ __device__ __forceinline__ unsigned long long bits_of(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  __builtin_memcpy(&b, &x, 8);
  return b;
#endif
}

__host__ __device__ __forceinline__ double double_of(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  __builtin_memcpy(&x, &b, 8);
  return x;
#endif
}

// x in [0, 16) -> x * 2^124 as a 128-bit integer (exact for x >= 2^-72).
__host__ __device__ __forceinline__ U128 fx_from_double(double x) {
  const unsigned long long b = bits_of(x);
  const int e = (int)(b >> 52);  // the sign bit is 0
  if (e == 0) return U128{0ull, 0ull};
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - (1075 - kPrFrac);  // x = m * 2^(e - 1075)
  if (sh >= 64) return U128{0ull, m << (sh - 64)};
  if (sh > 0) return U128{m << sh, m >> (64 - sh)};
  if (sh > -64) return U128{m >> (-sh), 0ull};
  return U128{0ull, 0ull};
}

// s * 2^-124 rounded to the nearest double, ties to even.
__host__ __device__ __forceinline__ double fx_to_double(const U128& s) {
  int t;  // position of the leading one
  if (s.hi) t = 127 - clz64(s.hi);
  else if (s.lo) t = 63 - clz64(s.lo);
  else return 0.0;
  unsigned long long M;
  if (t <= 52) {
    M = s.lo << (52 - t);  // fits the mantissa: exact
  } else {
    const int k = t - 52;  // bits below the mantissa, 1..75
    M = k >= 64 ? (s.hi >> (k - 64)) : ((s.lo >> k) | (s.hi << (64 - k)));
    const int r = k - 1;  // the rounding bit
    const unsigned long long rbit = r >= 64 ? (s.hi >> (r - 64)) & 1ull : (s.lo >> r) & 1ull;
    bool sticky;
    if (r >= 64) sticky = s.lo != 0ull || (r > 64 && (s.hi & ((1ull << (r - 64)) - 1ull)) != 0ull);
    else sticky = r > 0 && (s.lo & ((1ull << r) - 1ull)) != 0ull;
    if (rbit && (sticky || (M & 1ull))) {
      M++;
      if (M == (1ull << 53)) {
        M >>= 1;
        t++;
      }
    }
  }
  const unsigned long long ex = (unsigned long long)(t - kPrFrac + 1023);
  return double_of((ex << 52) | (M & 0xFFFFFFFFFFFFFull));
}

// a / b rounded to nearest (the IEEE quotient) from y = RN(1/b), for a
// positive normal double a and a positive integer b held exactly as a double,
// with every intermediate value normal (PageRank: a = p' >= 0.15/n, b = a
// degree below 2^32).  Five FP64 operations instead of a division.
// Markstein's theorem (P. Markstein, IBM J. Res. Dev. 34(1), 1990): if y is
// the correctly rounded 1/b, q lies within one ulp of a/b and r = a - b*q is
// exact, then RN(q + r*y) = RN(a/b).  q0 = RN(a*y) lies within 1.5 ulp of
// a/b; one correction q1 = RN(q0 + RN(a - b*q0)*y) has error
// |q0 - a/b| * O(2^-52) before its single rounding, so q1 lies within
// 0.5 ulp + tiny < 1 ulp, its residual a - b*q1 is exactly representable
// (computed exactly by the FMA), and the second correction is the theorem's
// step.  tests/test_pr_exact_host.py compares it with IEEE division on
// random and adversarial samples.
__host__ __device__ __forceinline__ double div_by_recip(double a, double b, double y) {
  const double q0 = a * y;
  const double r0 = fma(-b, q0, a);
  const double q1 = fma(r0, y, q0);
  const double r1 = fma(-b, q1, a);
  return fma(r1, y, q1);
}

// The L1 threshold of PageRank.C:172 (epsilon = 1e-7, the double) scaled
// exactly: L1 < 1e-7  <=>  L1_fx < kPrEpsFx (both exact).
__host__ __device__ __forceinline__ U128 pr_eps_fx() { return fx_from_double(1e-7); }

__host__ __device__ __forceinline__ bool less128(const U128& a, const U128& b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

}  // namespace rg
