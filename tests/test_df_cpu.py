"""Double-float arithmetic of the FP64 form's assembly stage
(kqed_gb300/csrc/kqed_df.h), checked on the host against long double: sums
and products of random double-float operands over a wide exponent range have
relative error <= 2^-44 of the operands' magnitude, and the exact
conversions round-trip."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r'''
#include "kqed_df.h"
#include <cstdio>
#include <cstdlib>
#include <random>
using namespace kqed;
int main() {
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0), e(-20.0, 20.0);
  long double worst_add = 0, worst_mul = 0, worst_conv = 0;
  for (int i = 0; i < 200000; i++) {
    const double a = u(g) * std::exp2(e(g)), b = u(g) * std::exp2(e(g));
    const df A(a), B(b);
    const long double la = (long double)A.hi + A.lo, lb = (long double)B.hi + B.lo;
    worst_conv = std::max(worst_conv, std::fabs(la - a) / std::fabs((long double)a));
    const df S = A + B, P = A * B;
    const long double s = (long double)S.hi + S.lo, p = (long double)P.hi + P.lo;
    const long double es = std::fabs(s - (la + lb)) / (std::fabs(la) + std::fabs(lb));
    const long double ep = std::fabs(p - la * lb) / std::fabs(la * lb);
    worst_add = std::max(worst_add, es);
    worst_mul = std::max(worst_mul, ep);
  }
  std::printf("%.6Le %.6Le %.6Le\n", worst_conv, worst_add, worst_mul);
  return 0;
}
'''


def test_double_float_error_bounds(tmp_path):
    c = tmp_path / "df.cpp"
    c.write_text(PROG)
    exe = str(tmp_path / "df")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I",
                    os.path.join(ROOT, "kqed_gb300", "csrc"), "-o", exe, str(c)], check=True)
    conv, add, mul = (float(v) for v in
                      subprocess.run([exe], capture_output=True, text=True,
                                     check=True).stdout.split())
    assert conv <= 2.0 ** -47, conv
    assert add <= 2.0 ** -44, add
    assert mul <= 2.0 ** -44, mul
