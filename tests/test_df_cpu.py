"""Double-float arithmetic of the FP64 form's assembly stage
(kqed_gb300/csrc/kqed_df.h), checked on the host against long double: sums
products and fused multiply-adds of random double-float operands over a wide
exponent range have relative error <= 2^-44 of the operands' magnitude, the
exact conversions round-trip, and a Chebyshev (second kind) Clenshaw sum of
40 terms run in double-float -- the recurrence of the FP64 form's Chebyshev
sums, |x| <= 0.99 -- stays within 2^-40 of the sum of the terms'
magnitudes."""
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
  long double worst_add = 0, worst_mul = 0, worst_conv = 0, worst_fma = 0, worst_cl = 0;
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
    const double c = u(g) * std::exp2(e(g));
    const df C(c);
    const long double lc = (long double)C.hi + C.lo;
    const df F = fma(A, B, C);
    const long double f = (long double)F.hi + F.lo;
    worst_fma = std::max(worst_fma,
                         std::fabs(f - (la * lb + lc)) / (std::fabs(la * lb) + std::fabs(lc)));
  }
  /* b_k = 2x b_{k+1} - b_{k+2} + c_k, k = K-1..0; sum = b_0 = sum_k c_k U_k(x) */
  for (int i = 0; i < 20000; i++) {
    const int K = 40;
    const double x = 0.99 * u(g);
    const df twox(2.0 * x);
    df b1(0.0f, 0.0f), b2(0.0f, 0.0f);
    long double l1 = 0, l2 = 0, mag = 0;
    const long double ltwox = (long double)twox.hi + twox.lo;
    for (int k = K - 1; k >= 0; --k) {
      const df ck(u(g) * std::exp2(-0.25 * k));
      const long double lck = (long double)ck.hi + ck.lo;
      const df t = fma(twox, b1, ck - b2);
      b2 = b1; b1 = t;
      const long double lt = ltwox * l1 - l2 + lck;
      l2 = l1; l1 = lt;
      mag += std::fabs(lck) * (k + 1);
    }
    const long double got = (long double)b1.hi + b1.lo;
    worst_cl = std::max(worst_cl, std::fabs(got - l1) / mag);
  }
  std::printf("%.6Le %.6Le %.6Le %.6Le %.6Le\n", worst_conv, worst_add, worst_mul, worst_fma,
              worst_cl);
  return 0;
}
'''


def test_double_float_error_bounds(tmp_path):
    c = tmp_path / "df.cpp"
    c.write_text(PROG)
    exe = str(tmp_path / "df")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I",
                    os.path.join(ROOT, "kqed_gb300", "csrc"), "-o", exe, str(c)], check=True)
    conv, add, mul, fma, clen = (float(v) for v in
                      subprocess.run([exe], capture_output=True, text=True,
                                     check=True).stdout.split())
    assert conv <= 2.0 ** -47, conv
    assert add <= 2.0 ** -44, add
    assert mul <= 2.0 ** -44, mul
    assert fma <= 2.0 ** -44, fma
    assert clen <= 2.0 ** -40, clen
