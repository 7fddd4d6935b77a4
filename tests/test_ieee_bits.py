"""The bit-pattern comparisons and scalings of csrc/ieee_bits.h against the
compiler's own IEEE double comparisons and multiplies by 0.5 and 2.0, on the
host (the header is plain C++ too).

The reference-mode kernels use these predicates in place of FP64 compares,
and must return exactly what the FP64 compare returns, so the check runs
over every pair of special values (signed zeros, denormals, infinities,
quiet and signalling NaNs of either sign, the kernels' constants and their
neighbours) and a million random bit patterns."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "tissue-ablation-mc_gb300", "csrc")

DRIVER = r"""
#include "ieee_bits.h"
#include <cmath>
#include <cstdio>
#include <limits>
#include <random>
#include <vector>
using namespace tam::ieee;

static double from(uint64_t b) { double x; std::memcpy(&x, &b, sizeof x); return x; }
static long bad = 0;
static void check(bool got, bool want, const char *what, double a, double b)
{
    if (got != want && bad++ < 20)
        std::printf("MISMATCH %s a=%a (%016llx) b=%a\n", what, a, (unsigned long long)bits(a), b);
}
static void scaled(double x)
{
    // exact halving and doubling against the host's IEEE multiply (NaN: stays NaN)
    const double h = 0.5 * x, t = 2.0 * h;
    const double hh = half(x), tt = twice_half(x, hh);
    if (x != x) {
        check(hh != hh, true, "half nan", x, 0);
        check(tt != tt, true, "twice_half nan", x, 0);
    } else {
        check(bits(hh) == bits(h), true, "half", x, h);
        check(bits(tt) == bits(t), true, "twice_half", x, t);
    }
}
static void one(double x, const std::vector<double> &cs)
{
    scaled(x);
    check(is_nan(x), x != x, "is_nan", x, 0);
    check(is_zero(x), x == 0.0, "is_zero", x, 0);
    check(gt_zero(x), x > 0.0, "gt_zero", x, 0);
    check(ge_zero(x), x >= 0.0, "ge_zero", x, 0);
    check(lt_zero(x), x < 0.0, "lt_zero", x, 0);
    for (double c : cs) {
        check(lt(x, c), x < c, "lt", x, c);
        check(lt(c, x), c < x, "lt'", c, x);
        check(le(x, c), x <= c, "le", x, c);
        check(le(c, x), c <= x, "le'", c, x);
        check(eq(x, c), x == c, "eq", x, c);
        if (c > 0.0 && std::isfinite(c)) {
            check(ge_pos(x, bits(c)), x >= c, "ge_pos", x, c);
            check(lt_pos(x, bits(c)), x < c, "lt_pos", x, c);
        }
    }
}
int main()
{
    const double inf = std::numeric_limits<double>::infinity();
    std::vector<double> sp = {0.0, -0.0, 1.0, -1.0, 0.75, 0.53, 1.0, 1e4, 316.0, 373.0, 773.0, 300.0,
                              std::numeric_limits<double>::denorm_min(), -std::numeric_limits<double>::denorm_min(),
                              std::numeric_limits<double>::min(), std::numeric_limits<double>::max(),
                              -std::numeric_limits<double>::max(), inf, -inf,
                              from(0x7FF8000000000000ull), from(0xFFF8000000000000ull),
                              from(0x7FF0000000000001ull), from(0xFFF0000000000001ull),
                              from(0x7FFFFFFFFFFFFFFFull), from(0xFFFFFFFFFFFFFFFFull)};
    const size_t base = sp.size();
    for (size_t i = 0; i < base; ++i) {
        sp.push_back(std::nextafter(sp[i], inf));
        sp.push_back(std::nextafter(sp[i], -inf));
    }
    for (double x : sp) one(x, sp);
    std::mt19937_64 g(12345);
    std::vector<double> cs = {0.75, 0.53, 316.0, 373.0, 1e4, 5e-324, 1.7976931348623157e308, -0.0, 0.0, -316.0};
    for (int n = 0; n < 1000000; ++n) {
        const uint64_t r = g();
        // half the draws near the constants' exponents, half anywhere
        const uint64_t b = (n & 1) ? r : ((r & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1016 + (r >> 52) % 16) << 52));
        one(from(b), cs);
        // denormals and the two lowest binades, where halving rounds
        scaled(from((r & 0x800FFFFFFFFFFFFFull) | ((uint64_t)((r >> 52) % 3) << 52)));
        const double y = from(g());
        check(lt(from(b), y), from(b) < y, "lt r", from(b), y);
        check(eq(from(b), y), from(b) == y, "eq r", from(b), y);
    }
    std::printf("mismatches %ld\n", bad);
    return bad != 0;
}
"""


def test_bit_predicates_match_ieee_compares(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "ieee_check.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "ieee_check"
    # -O2 without fast-math: the compiler's double compares are IEEE
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "mismatches 0" in r.stdout, r.stdout
