"""The PageRank arithmetic helpers (radar-graph_gb300/csrc/pr_exact.cuh)
compiled as host C++ and checked on the CPU:
  - fx_from_double / add128 / fx_to_double: a sum of doubles accumulated in
    128-bit fixed point and converted back equals the exactly computed sum
    correctly rounded (Python's Fraction -> float rounds to nearest even),
    including exact ties;
  - recip_magic: the integer reciprocal floor(2^(63+l) / d) equals the
    exact big-integer quotient;
  - deg_quotient / div_by_magic: the integer-pipe quotient by degree class
    equals IEEE division a / d for integer d (degrees), on random and
    adversarial samples (quotients at and next to representable values,
    exact ties, degrees next to powers of two)."""

import ctypes as C
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#define __host__
#define __device__
#define __forceinline__ inline
#include "pr_exact.cuh"
extern "C" double fx_sum(const double* x, long n) {
  rg::U128 a{0, 0};
  for (long i = 0; i < n; i++) rg::add128(a, rg::fx_from_double(x[i]));
  return rg::fx_to_double(a);
}
extern "C" long div_mismatches(const double* a, const unsigned* b, long n) {
  long bad = 0;
  for (long i = 0; i < n; i++) {
    const unsigned d = b[i];
    const unsigned long long R = (d & (d - 1)) ? rg::recip_magic(d) : 0ull;
    const double want = d ? a[i] / (double)d : 0.0;  // no out-edges: contribution 0
    bad += rg::deg_quotient(a[i], d, R) != want;
  }
  return bad;
}
extern "C" void magics(const unsigned* d, unsigned long long* out, long n) {
  for (long i = 0; i < n; i++) out[i] = rg::recip_magic(d[i]);
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("prx")
    (d / "t.cc").write_text(SRC)
    so = d / "t.so"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC",
                    "-I", os.path.join(ROOT, "radar-graph_gb300", "csrc"), str(d / "t.cc"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.fx_sum.restype = C.c_double
    L.fx_sum.argtypes = [C.c_void_p, C.c_long]
    L.div_mismatches.restype = C.c_long
    L.div_mismatches.argtypes = [C.c_void_p, C.c_void_p, C.c_long]
    L.magics.restype = None
    L.magics.argtypes = [C.c_void_p, C.c_void_p, C.c_long]
    return L


def test_fixed_point_sums_round_like_the_exact_sum(lib):
    rng = np.random.default_rng(1)
    for trial in range(3000):
        k = int(rng.integers(1, 40))
        kind = trial % 3
        if kind == 0:
            x = rng.random(k)
        elif kind == 1:
            x = rng.random(k) * 10.0 ** rng.integers(-20, 0, size=k)
        else:
            x = np.ldexp(rng.integers(1, 2 ** 53, size=k).astype(np.float64), rng.integers(-124, -53, size=k))
        x = x / max(1.0, float(x.sum()))
        assert lib.fx_sum(x.ctypes.data, len(x)) == float(sum(Fraction(float(v)) for v in x))
    for _ in range(500):  # exact ties: a + half an ulp of a
        m, e = int(rng.integers(2 ** 52, 2 ** 53)), int(rng.integers(-60, -1))
        a, h = np.ldexp(float(m), e - 52), np.ldexp(1.0, e - 53)
        x = np.array([a, h])
        assert lib.fx_sum(x.ctypes.data, 2) == float(Fraction(a) + Fraction(h))


def test_integer_reciprocal_is_exact(lib):
    rng = np.random.default_rng(3)
    d = np.concatenate([np.arange(3, 5000), rng.integers(3, 2 ** 32, 20000),
                        2 ** np.arange(2, 32) + 1, 2 ** np.arange(3, 33) - 1]).astype(np.uint64)
    d = d[(d & (d - 1)) != 0].astype(np.uint32)
    out = np.empty(len(d), np.uint64)
    lib.magics(d.ctypes.data, out.ctypes.data, len(d))
    for x, r in zip(d.tolist(), out.tolist()):
        assert r == (1 << (63 + x.bit_length())) // x


def test_integer_quotient_equals_ieee_division(lib):
    rng = np.random.default_rng(2)
    n = 2_000_000
    b = np.concatenate([rng.integers(0, 65, n // 4), rng.integers(1, 100_000, n // 4),
                        rng.integers(1, 2 ** 32, n // 4),
                        (2 ** rng.integers(0, 32, n // 4) + rng.integers(-1, 2, n // 4)).clip(1, 2 ** 32 - 1)])
    b = b.astype(np.uint32)
    a = np.ldexp(1.0 + rng.random(n), -rng.integers(-3, 60, n))
    near = rng.random(n) < 0.3  # a = b * q (+ one ulp): quotients at and next to representable values
    q = np.ldexp(1.0 + rng.random(n), -rng.integers(25, 65, n))
    t = b.astype(np.float64) * q
    a = np.where(near, np.where(rng.random(n) < 0.5, t, np.nextafter(t, 1.0)), a)
    a = np.where(a > 0, a, 1.0)
    assert lib.div_mismatches(a.ctypes.data, b.ctypes.data, n) == 0


def test_integer_quotient_next_to_midpoints(lib):
    # a = RN(d * mid) and its neighbours, mid halfway between two doubles:
    # a / d lies within a few ulps of a for tiny offsets from mid, so the
    # remainder alone decides the rounding direction
    rng = np.random.default_rng(4)
    rows_a, rows_b = [], []
    for _ in range(40000):
        d = int(rng.choice([3, 5, 7, 9, 11, 13, 15, 17, 25, 31, 33, 63, 65, 127, 1023, 65537, 2 ** 31 + 1,
                            2 ** 32 - 1, int(rng.integers(3, 2 ** 32))]))
        if d & (d - 1) == 0:
            d += 1
        mid = Fraction(2 * int(rng.integers(2 ** 52, 2 ** 53)) + 1, 2 ** int(rng.integers(40, 110)))
        a = float(mid * d)
        for x in (a, float(np.nextafter(a, 0.0)), float(np.nextafter(a, np.inf))):
            rows_a.append(x)
            rows_b.append(d)
    a = np.array(rows_a)
    b = np.array(rows_b, np.uint32)
    assert lib.div_mismatches(a.ctypes.data, b.ctypes.data, len(a)) == 0
