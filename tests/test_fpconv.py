"""The kernels' double <-> float conversions and comparisons done with integer operations
(relxill_gb300/csrc/relx_fpconv.cuh), compiled for the host and checked bit for bit against the
compiler's conversions: random bit patterns, every float denormal, values at and around the edges of
the float range and the rounding ties.  No GPU needed."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "relxill_gb300", "csrc", "relx_fpconv.cuh")

PROGRAM = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#define RELX_FPCONV_FN static inline
static inline unsigned int __float_as_uint(float f) { unsigned int u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned int u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline long long __double_as_longlong(double d) { long long u; std::memcpy(&u, &d, 8); return u; }
static inline double __longlong_as_double(long long u) { double d; std::memcpy(&d, &u, 8); return d; }
static inline int __clz(unsigned int x) { return x ? __builtin_clz(x) : 32; }
#include "relx_fpconv.cuh"
using namespace relx;
static long bad = 0, n = 0;
static void chk_d(double d) {
  const float a = d2f(d), b = (float) d;
  n++;
  if (std::memcmp(&a, &b, 4) != 0 && !(std::isnan(a) && std::isnan(b))) {
    if (bad < 5) std::printf("d2f %a -> %a, expected %a\n", d, a, b);
    bad++;
  }
}
static void chk_f(float f) {
  const double a = f2d(f), b = (double) f;
  n++;
  if (std::memcmp(&a, &b, 8) != 0 && !(std::isnan(a) && std::isnan(b))) {
    if (bad < 5) std::printf("f2d %a -> %a, expected %a\n", f, a, b);
    bad++;
  }
}
static void chk_cmp(double a, double b) {  // b > 0, a not NaN
  n++;
  if (dgt(a, b) != (a > b) || dge(a, b) != (a >= b)) {
    if (bad < 5) std::printf("compare %a %a\n", a, b);
    bad++;
  }
}
int main() {
  std::mt19937_64 g(2026);
  for (long i = 0; i < 4000000; i++) {
    const uint64_t u = g();
    double d;
    std::memcpy(&d, &u, 8);
    chk_d(d);
    const uint32_t v = (uint32_t) u;
    float f;
    std::memcpy(&f, &v, 4);
    chk_f(f);
  }
  for (int e = -160; e <= 130; e++)
    for (int k = -3; k <= 3; k++)
      for (int sg = 0; sg < 2; sg++) {
        const double base = std::ldexp(1.0, e), d = base * (1 + k * std::ldexp(1.0, -24));
        chk_d(sg ? -d : d);
        chk_d(std::nextafter(d, 0.0));
        chk_d(std::nextafter(d, 1e300));
        chk_d(base * (1 + std::ldexp(1.0, -24)));      // a tie, rounds to even
        chk_d(base * (1 + 3 * std::ldexp(1.0, -24)));  // a tie, rounds up
      }
  const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 3.4028235677973366e38, 3.4028234663852886e38, 1e300,
                            1e-300, 0.95, 5e-3};
  for (double d : special) chk_d(d);
  for (uint32_t v = 0; v < 0x800000u; v++) {  // every float denormal, both signs
    float f;
    std::memcpy(&f, &v, 4);
    chk_f(f);
    const uint32_t w = v | 0x80000000u;
    std::memcpy(&f, &w, 4);
    chk_f(f);
  }
  std::uniform_real_distribution<double> uni(-2000.0, 2000.0), pos(1e-6, 2000.0);
  for (long i = 0; i < 1000000; i++) {
    const double b = pos(g);
    chk_cmp(uni(g), b);
    chk_cmp(b, b);
    chk_cmp(std::nextafter(b, 0.0), b);
  }
  std::printf("checked %ld mismatches %ld\n", n, bad);
  return bad != 0;
}
"""


def test_integer_conversions_match_the_compiler():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "fpconv_test.cpp")
        exe = os.path.join(d, "fpconv_test")
        with open(src, "w") as f:
            f.write(PROGRAM)
        subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.dirname(HEADER), src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "mismatches 0" in r.stdout
