"""vexp_nonpos (the exponential of the Gaussian bumps, whose argument is never positive) returns
vexp's bits for every argument x <= 0 and a NaN for a NaN.  This sweep takes one float pattern in
16 over the whole non-positive range, every pattern within 2^16 of the clamp at -87, of -0 and of
each k = rint(x log2e) boundary, and the special values; a pass over all 2^31 non-positive floats
and the NaNs was also run once."""
import os
import subprocess

from conftest import ROOT

PROG = r'''
#include <cstdio>
#include <cstring>
#include <cmath>
#include "vcu_integrands.h"
static long check(unsigned u) {
    float x;
    std::memcpy(&x, &u, 4);
    if (!(x <= 0.0f) && !std::isnan(x)) return 0;
    const float a = vcu::vexp(x), b = vcu::vexp_nonpos(x);
    if (std::isnan(a)) return std::isnan(b) ? 0 : 1;
    unsigned ua, ub;
    std::memcpy(&ua, &a, 4);
    std::memcpy(&ub, &b, 4);
    if (ua != ub) {
        std::printf("x=%a vexp %a vexp_nonpos %a\n", x, a, b);
        return 1;
    }
    return 0;
}
static long around(float c) {
    unsigned u;
    std::memcpy(&u, &c, 4);
    long bad = 0;
    for (unsigned d = 0; d < (1u << 16); ++d) bad += check(u + d) + check(u - d);
    return bad;
}
int main() {
    long bad = 0;
    for (unsigned long long v = 0x80000000ull; v < (1ull << 32); v += 16) bad += check((unsigned)v);
    bad += around(-87.0f) + around(-0.0f) + check(0u);
    for (int k = 0; k <= 126; ++k) bad += around(-((float)k + 0.5f) / 1.4426950216293335f);
    bad += check(0xff800000u) + check(0x7fc00000u) + check(0xffc00000u) + check(0x7f800001u);
    std::printf("%ld\n", bad);
    return bad != 0;
}
'''


def test_nonpositive_exponential_matches_vexp(tmp_path):
    src = tmp_path / "vexp.cc"
    src.write_text(PROG)
    exe = tmp_path / "vexp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
