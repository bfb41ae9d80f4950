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
// GB300 issues FP64 at a small fraction of its integer rate, so the per-edge
// additions and the per-vertex quotient p/deg stay on the integer pipes; the
// FP64 work is the damping step and |p - p'|.
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

__host__ __device__ __forceinline__ int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

__host__ __device__ __forceinline__ unsigned long long mulhi64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

// The integer reciprocal of a degree d >= 3 that is not a power of two:
// R = floor(2^(63+l) / d) with 2^(l-1) < d < 2^l, so R lies in [2^63, 2^64).
// Long division in two 64-by-32-bit steps.
__host__ __device__ __forceinline__ unsigned long long recip_magic(uint32_t d) {
  const int l = 32 - clz32(d);
  const unsigned long long hi = 1ull << (31 + l);  // 2^(63+l) = hi * 2^32
  const unsigned long long q1 = hi / d, r1 = hi % d;
  return (q1 << 32) | ((r1 << 32) / d);
}

// a / d rounded to nearest, ties to even (the IEEE quotient), on the integer
// pipes: GB300 issues FP64 at a small fraction of its integer rate, and the
// FP64 route (a reciprocal and two Markstein correction steps, or a
// division) cost five or more FP64 operations per vertex.
//   a = Ma * 2^(E-1075), A = Ma * 2^11 in [2^63, 2^64), N = A * 2^(l-1):
//   a / d = (N / d) * 2^(E-1085-l), and N / d lies in (2^62, 2^64).
//   Q = mulhi(A, R) is floor(N / d) or one less (R undershoots 2^(63+l)/d by
//   less than one, so A*R/2^64 undershoots N/d by less than one); the
//   remainder N - Q*d is below 2d, so it is exact modulo 2^64 and one
//   comparison corrects Q.  The 53 leading bits of Q, its next bit and a
//   sticky bit (lower bits of Q or a nonzero remainder) round to nearest even.
// Preconditions: d >= 3 not a power of two, R = recip_magic(d), a a
// positive normal double with a >= 2^-990 (so the quotient is normal).
__host__ __device__ __forceinline__ double div_by_magic(double a, uint32_t d, unsigned long long R) {
  const unsigned long long b = bits_of(a);
  const int E = (int)(b >> 52);
  const unsigned long long A = ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11;
  const int l = 32 - clz32(d);
  unsigned long long Q = mulhi64(A, R);
  unsigned long long r = (A << (l - 1)) - Q * (unsigned long long)d;
  if (r >= d) {
    Q++;
    r -= d;
  }
  const int k = (Q >> 63) ? 11 : 10;  // bits of Q below the 53 kept
  unsigned long long M = Q >> k;
  const bool guard = (Q >> (k - 1)) & 1ull;
  const bool sticky = (Q & ((1ull << (k - 1)) - 1ull)) != 0ull || r != 0ull;
  unsigned long long ex = (unsigned long long)(E - 10 - l + k);  // biased exponent of M * 2^(k+E-1085-l)
  if (guard && (sticky || (M & 1ull))) {
    M++;
    if (M == (1ull << 53)) {
      M >>= 1;
      ex++;
    }
  }
  return double_of((ex << 52) | (M & 0xFFFFFFFFFFFFFull));
}

// p / deg(v), the IEEE quotient of PR_F (PageRank.C:48), by degree class: 0
// for no out-edges, an exact exponent shift for a power of two, else
// div_by_magic with R = recip_magic(d) (a >= 2^-990: PageRank values are at
// least 0.15/n).
__host__ __device__ __forceinline__ double deg_quotient(double a, uint32_t d, unsigned long long R) {
  if (d == 0) return 0.0;
  if ((d & (d - 1)) == 0) return double_of(bits_of(a) - ((unsigned long long)(31 - clz32(d)) << 52));
  return div_by_magic(a, d, R);
}

// The L1 threshold of PageRank.C:172 (epsilon = 1e-7, the double) scaled
// exactly: L1 < 1e-7  <=>  L1_fx < kPrEpsFx (both exact).
__host__ __device__ __forceinline__ U128 pr_eps_fx() { return fx_from_double(1e-7); }

__host__ __device__ __forceinline__ bool less128(const U128& a, const U128& b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

}  // namespace rg
