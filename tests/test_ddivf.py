"""ddiv_f<D> and fdiv_c<D> (the double and the float quotient of a float by 3 or 5 through a
product and one remainder correction, used in the reference-rounded Horner steps and in the rules'
power-basis coefficients) return the correctly rounded quotient: every significand and sign at
exponents across the float range, plus zeros, subnormals, the largest float, infinities and NaN.
The exponents here stand for the rest (the correction is one fused operation at the quotient's
scale); a pass over all 2^32 floats was also run once for each."""
import os
import subprocess

from conftest import ROOT

PROG = r'''
#include <cstdio>
#include <cstring>
#include <cmath>
#include "vcu_integrands.h"
template <int D> static long check(float x) {
    const double q = vcu::ddiv_f<D>(x);
    volatile double dd = (double)D;
    const double r = (double)x / dd;
    if (std::isnan(r)) return std::isnan(q) ? 0 : 1;
    unsigned long long a, b;
    std::memcpy(&a, &q, 8);
    std::memcpy(&b, &r, 8);
    if (a != b) {
        std::printf("D=%d x=%a got %a want %a\n", D, x, q, r);
        return 1;
    }
    return 0;
}
template <int D> static long checkf(float x) {
    const float q = vcu::fdiv_c<D>(x);
    volatile float dd = (float)D;
    const float r = x / dd;
    if (std::isnan(r)) return std::isnan(q) ? 0 : 1;
    if (std::memcmp(&q, &r, 4) != 0) {
        std::printf("D=%d x=%a got %a want %a (float)\n", D, x, q, r);
        return 1;
    }
    return 0;
}
template <int D> static long sweep() {
    long bad = 0;
    const int exps[] = {-126, -100, -60, -1, 0, 1, 23, 60, 100, 127};
    for (int e : exps)
        for (unsigned m = 0; m < (1u << 23); ++m)
            for (unsigned s = 0; s < 2; ++s) {
                unsigned u = (s << 31) | ((unsigned)(e + 127) << 23) | m;
                float x;
                std::memcpy(&x, &u, 4);
                bad += check<D>(x) + checkf<D>(x);
            }
    for (unsigned u = 0; u < (1u << 16); ++u) {  /* zeros and subnormals */
        float x;
        unsigned v = u * 127u;
        std::memcpy(&x, &v, 4);
        bad += check<D>(x) + check<D>(-x) + checkf<D>(x) + checkf<D>(-x);
    }
    bad += check<D>(INFINITY) + check<D>(-INFINITY) + check<D>(NAN) + check<D>(3.4028235e38f) + check<D>(-0.0f);
    bad += checkf<D>(INFINITY) + checkf<D>(-INFINITY) + checkf<D>(NAN) + checkf<D>(3.4028235e38f) + checkf<D>(-0.0f);
    return bad;
}
int main() {
    const long bad = sweep<3>() + sweep<5>();
    std::printf("%ld\n", bad);
    return bad != 0;
}
'''


def test_double_division_of_floats_is_correctly_rounded(tmp_path):
    src = tmp_path / "ddivf.cc"
    src.write_text(PROG)
    exe = tmp_path / "ddivf"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
