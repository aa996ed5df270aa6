"""The FP32 emulation of the reference's double-promoted rule values (viltrum_gb300/csrc/vcu_refrule.h)
returns the reference's float for random node lines of many magnitudes, including constant lines
(error estimate exactly zero) and lines spanning several orders of magnitude."""
import os
import subprocess
import tempfile

from conftest import ROOT

PROG = r'''
#include <cstdio>
#include <cmath>
#include <random>
#include "vcu_refrule.h"
int main() {
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    std::uniform_int_distribution<int> ex(-30, 30), kind(0, 3);
    long bad5 = 0, bad3 = 0, n = 0;
    for (int t = 0; t < 2000000; ++t) {
        float p[5];
        const int k = kind(rng);
        const float scale = std::ldexp(1.0f, ex(rng));
        for (int i = 0; i < 5; ++i) {
            if (k == 0) p[i] = scale * u(rng);                                   /* random */
            else if (k == 1) p[i] = (i == 0) ? scale * u(rng) : p[0];            /* constant */
            else if (k == 2) p[i] = scale * (0.5f + 1e-6f * u(rng));             /* nearly constant */
            else p[i] = std::ldexp(u(rng), ex(rng) / 3);                         /* mixed magnitudes */
        }
        const float ref5 = (7.0 * p[0] + 32.0 * p[1] + 12.0 * p[2] + 32.0 * p[3] + 7.0 * p[4]) / 90.0;
        const float ref3 = (p[0] + 4.0 * p[1] + p[2]) / 6.0;
        if (vcu::RefRule<5>::scalar(p) != ref5) ++bad5;
        if (vcu::RefRule<3>::scalar(p) != ref3) ++bad3;
        ++n;
    }
    std::printf("%ld %ld %ld\n", n, bad5, bad3);
    return 0;
}
'''


def test_refrule_matches_reference_rounding():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "r.cc")
        exe = os.path.join(d, "r")
        open(src, "w").write(PROG)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                               "-I", os.path.join(ROOT, "viltrum_gb300", "csrc"), src, "-o", exe])
        n, bad5, bad3 = map(int, subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split())
        assert n == 2000000
        # only the reference's own double-rounding cases may differ (probability ~2^-29 per value)
        assert bad5 <= 2 and bad3 <= 2, (bad5, bad3)
