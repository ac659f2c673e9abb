"""Double-float primitives of the mixed implicit step (168861_gb300/csrc/ff.cuh), checked on
the CPU: the header is plain C++ outside nvcc, so a small program compiled with g++ runs the
same functions the kernel runs over seeded random values, against long double (64-bit
significand) arithmetic.

Bars: error-free transformations exact; the split of a double relative error <= 2^-46
(2^-23 below 2^-76, where the low part would be an FP32 subnormal); float -> double exact;
pair add / subtract within 2^-44 of the operands' magnitudes, pair products within 2^-44
of the product's."""
import os
import subprocess

from conftest import ROOT

PROG = r"""
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>
#include "ff.cuh"
using namespace nrt;
typedef long double LD;
static LD val(ff a) { return (LD)a.hi + (LD)a.lo; }
int main() {
  std::mt19937_64 g(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-90, 90);
  double worst_split = 0, worst_add = 0, worst_mul = 0, worst_mulf = 0, worst_addf = 0;
  long bad_two_sum = 0, bad_f2d = 0, bad_hi = 0, bad_norm = 0;
  for (int it = 0; it < 2000000; it++) {
    const double d = std::ldexp(u(g), ex(g));
    const ff s = ff_of(d);
    if (std::fabs(d) >= std::ldexp(1.0, -99)) {  // the split's range (smaller values give 0)
      const double e = (double)std::fabs((val(s) - (LD)d) / (LD)d);
      if (std::fabs(d) >= std::ldexp(1.0, -76)) {
        if (e > worst_split) worst_split = e;
      } else if (e > std::ldexp(1.0, -23)) {
        bad_hi++;
      }
      // hi is d truncated to 24 bits: d - hi exact in double, |d - hi| < ulp(hi)
      const double r = d - (double)s.hi;
      if (std::fabs(r) >= std::ldexp(std::fabs((double)s.hi), -23) || (r != 0 && std::signbit(r) != std::signbit(d))) bad_hi++;
    }
    const float a = (float)std::ldexp(u(g), ex(g) / 4), b = (float)std::ldexp(u(g), ex(g) / 4);
    const ff t = two_sum(a, b);
    if ((LD)t.hi + (LD)t.lo != (LD)a + (LD)b) bad_two_sum++;
    if (double_of(a) != (double)a) bad_f2d++;
    // pairs built from doubles of nearby and far magnitudes
    const ff x = ff_of(std::ldexp(u(g), ex(g) / 8)), y = ff_of(std::ldexp(u(g), ex(g) / 8));
    const ff z = ff_add(x, y);
    const LD ez = std::fabs(val(z) - (val(x) + val(y))) / (std::fabs(val(x)) + std::fabs(val(y)));
    if ((double)ez > worst_add) worst_add = (double)ez;
    if (std::fabs(z.lo) > std::ldexp(std::fabs(z.hi), -23)) bad_norm++;
    const ff zs = ff_sub(x, y);
    const LD es = std::fabs(val(zs) - (val(x) - val(y))) / (std::fabs(val(x)) + std::fabs(val(y)));
    if ((double)es > worst_add) worst_add = (double)es;
    const ff p = ff_mul(x, y);
    if (val(x) != 0 && val(y) != 0) {
      const LD ep = std::fabs((val(p) - val(x) * val(y)) / (val(x) * val(y)));
      if ((double)ep > worst_mul) worst_mul = (double)ep;
      const ff q = ff_mul_f(x, y.hi);
      const LD eq = std::fabs((val(q) - val(x) * (LD)y.hi) / (val(x) * (LD)y.hi));
      if ((double)eq > worst_mulf) worst_mulf = (double)eq;
    }
    const ff w = ff_add_f(x, y.hi);
    const LD ew = std::fabs(val(w) - (val(x) + (LD)y.hi)) / (std::fabs(val(x)) + std::fabs((LD)y.hi));
    if ((double)ew > worst_addf) worst_addf = (double)ew;
  }
  // add_ff is v + (hi + lo) in FP64
  const ff k = ff_of(1.2345e-3);
  const double v = -0.0651234567891234;
  const int add_ok = add_ff(v, k) == v + ((double)k.hi + (double)k.lo);
  std::printf("%.3e %.3e %.3e %.3e %.3e %ld %ld %ld %ld %d\n", worst_split, worst_add, worst_mul,
              worst_mulf, worst_addf, bad_two_sum, bad_f2d, bad_hi, bad_norm, add_ok);
  return 0;
}
"""


def test_double_float_primitives(tmp_path):
    src = tmp_path / "ff_check.cpp"
    src.write_text(PROG)
    exe = tmp_path / "ff_check"
    inc = os.path.join(ROOT, "168861_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", inc, str(src), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    split, add, mul, mulf, addf = (float(x) for x in out[:5])
    bad_two_sum, bad_f2d, bad_hi, bad_norm, add_ok = (int(x) for x in out[5:])
    assert bad_two_sum == 0 and bad_f2d == 0 and bad_hi == 0 and bad_norm == 0
    assert add_ok == 1
    assert split <= 2.0 ** -46, split
    assert add <= 2.0 ** -44, add
    assert addf <= 2.0 ** -44, addf
    assert mul <= 2.0 ** -44, mul
    assert mulf <= 2.0 ** -44, mulf


def test_double_float_header_has_no_fp64_conversion_in_splits():
    """The hot conversions work on bit patterns: ff_of and double_of fall back to the FP64
    conversion instruction only for values outside the range they split (Inf, NaN, huge)."""
    text = open(os.path.join(ROOT, "168861_gb300", "csrc", "ff.cuh")).read()
    body = text[text.index("NRT_HD ff ff_of(double d)"):text.index("NRT_HD double add_ff")]
    assert body.count("(float)d") == 1 and body.count("(double)f") == 1
