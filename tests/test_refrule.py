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


PROG_FAST = r'''
#include <cstdio>
#include <cmath>
#include <cstring>
#include <random>
#include "vcu_refrule.h"
/* ff_div without its common-case return: the candidate and remainder as ff_div forms them, then
 * the exact decision */
static float full(float h, float l, float D, float inv) {
    const float ah = vcu::vabs(h);
    const float q00 = (ah >= 8.077935669463161e-28f && ah <= 1.2379400392853803e27f) ? h * inv : h / D;
    const float q0 = std::fmaf(std::fmaf(-q00, D, h) + l, inv, q00);
    float s, e;
    vcu::two_sum(std::fmaf(-q0, D, h), l, s, e);
    return vcu::ff_div_decide(q0, s, e, D);
}
int main() {
    std::mt19937 rng(11);
    std::uniform_int_distribution<unsigned> mant(0, (1u << 23) - 1), sgn(0, 1);
    std::uniform_int_distribution<int> ex(-100, 100);
    std::uniform_real_distribution<double> off(-1.0, 1.0);
    const float Ds[2] = {6.0f, 90.0f}, invs[2] = {0.1666666716337204f, 0.011111111380159855f};
    long bad = 0, n = 0;
    for (int t = 0; t < 4000000; ++t) {
        const int k = t & 1;
        const float D = Ds[k], inv = invs[k];
        unsigned u = (sgn(rng) << 31) | ((unsigned)(ex(rng) + 127) << 23) | mant(rng);
        float q;
        std::memcpy(&q, &u, 4);
        const double ulp = std::ldexp(1.0, std::ilogb(q) - 23);
        /* the quotient a random offset away from q, or within 2^-18 ulp of a midpoint (the band
         * around it included) */
        const int mode = (t >> 1) % 6;
        double delta = off(rng);
        if (mode == 1) delta = 0.5 + std::ldexp(off(rng), -18);
        if (mode == 2) delta = -0.5 + std::ldexp(off(rng), -18);
        if (mode == 3) delta = (t & 2 ? 0.5 : -0.5) + std::ldexp(off(rng), -29);
        if (mode == 4) delta = (t & 2) ? 0.5 : -0.5;   /* exact ties */
        if (mode == 5) delta = 0.0;                    /* exact quotients (zeros among them) */
        if (mode == 5 && (t & 6) == 6) q = 0.0f;
        const double target = ((double)q + delta * ulp) * (double)D;
        const float h = (float)target;
        const float l = (float)(target - (double)h);
        const float a = vcu::ff_div(h, l, D, inv), b = full(h, l, D, inv);
        if (std::memcmp(&a, &b, 4) != 0) {
            if (bad < 5) std::printf("h=%a l=%a D=%g fast %a full %a\n", h, l, D, a, b);
            ++bad;
        }
        ++n;
    }
    std::printf("%ld %ld\n", n, bad);
    return 0;
}
'''


def test_ff_div_common_case_matches_exact_decision():
    """ff_div's early returns (remainder well inside the half gap, exact ties, exact quotients) give
    the exact decision's result, including quotients within 2^-18 and 2^-29 ulp of a rounding
    midpoint, on it, and zero."""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "f.cc")
        exe = os.path.join(d, "f")
        open(src, "w").write(PROG_FAST)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                               "-I", os.path.join(ROOT, "viltrum_gb300", "csrc"), src, "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
        n, bad = int(out[-2]), int(out[-1])
        assert n == 4000000 and bad == 0, " ".join(out)


PROG_INT01 = r'''
#include <cstdio>
#include <cmath>
#include <cstring>
#include <random>
#include "vcu_refrule.h"
/* the reference's double Horner steps at t = 1 for float coefficients, rounded once to float */
static float ref3(const float* c) {
    double r = (double)(c[2] * 1.0f) / 3.0 + (double)c[1] * 0.5;
    r = r * 1.0 + (double)c[0];
    return (float)(r * 1.0);
}
static float ref5(const float* c) {
    double r = (double)(c[4] * 1.0f) / 5.0 + (double)c[3] * 0.25;
    r = r * 1.0 + (double)c[2] / 3.0;
    r = r * 1.0 + (double)c[1] * 0.5;
    r = r * 1.0 + (double)c[0];
    return (float)(r * 1.0);
}
int main() {
    std::mt19937 rng(5);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    std::uniform_int_distribution<int> ex(-30, 30), deep(0, 44);
    long n[5] = {0}, fb[5] = {0}, bad = 0;
    for (int t = 0; t < 3000000; ++t) {
        const int mode = t % 5;
        float c[5];
        const float scale = std::ldexp(1.0f, ex(rng));
        for (int i = 0; i < 5; ++i) c[i] = scale * u(rng);
        if (mode == 1) /* mixed magnitudes */
            for (int i = 0; i < 5; ++i) c[i] = std::ldexp(u(rng), ex(rng));
        if (mode == 2) {
            /* the sum within 2^-44 .. 1 ulp of a midpoint of c0's floats (exact ties among them):
             * c1/2 is half an ulp of c0, the higher terms tiny */
            const float ulp = std::ldexp(1.0f, std::ilogb(c[0]) - 23);
            c[1] = (t & 8) ? ulp : -ulp;
            const float tiny = std::ldexp(ulp, -deep(rng));
            for (int i = 2; i < 5; ++i) c[i] = (t & 16) ? 0.0f : tiny * u(rng);
        }
        if (mode == 3) { /* cancellation: c0 nearly minus the rest */
            const double rest = (double)c[4] / 5.0 + (double)c[3] / 4.0 + (double)c[2] / 3.0 + (double)c[1] / 2.0;
            c[0] = (float)(-rest) * (1.0f + std::ldexp(u(rng), -deep(rng) / 2));
        }
        if (mode == 4) { /* zeros, infinities, NaN, out-of-range magnitudes */
            const int k = (t / 5) % 4;
            if (k == 0) for (int i = 0; i < 5; ++i) c[i] = 0.0f;
            if (k == 1) c[t % 5 < 2 ? 0 : 2] = INFINITY;
            if (k == 2) c[1] = NAN;
            if (k == 3) for (int i = 0; i < 5; ++i) c[i] = std::ldexp(c[i], (t & 32) ? 100 : -100);
        }
        for (int S = 3; S <= 5; S += 2) {
            float out = 0.0f;
            const bool ok = (S == 3) ? vcu::ref_integral01<3>(c, out) : vcu::ref_integral01<5>(c, out);
            const float want = (S == 3) ? ref3(c) : ref5(c);
            ++n[mode];
            if (!ok) { ++fb[mode]; continue; }
            if (std::memcmp(&out, &want, 4) != 0) {
                if (bad < 5) std::printf("S=%d c=%a %a %a %a %a got %a want %a\n", S, c[0], c[1], c[2], c[3], c[4], out, want);
                ++bad;
            }
        }
    }
    for (int m = 0; m < 5; ++m) std::printf("%ld %ld ", n[m], fb[m]);
    std::printf("%ld\n", bad);
    return 0;
}
'''


def test_integral01_certified_matches_reference_double():
    """ref_integral01 (the whole-interval integral of a rule's polynomial in FP32) returns the reference's
    double-Horner float whenever it certifies a result -- on random, mixed-magnitude, near-midpoint (down
    to 2^-44 ulp, exact ties), cancelling and special coefficients -- and declines rarely on ordinary
    ones (the caller then evaluates in double)."""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "i.cc")
        exe = os.path.join(d, "i")
        open(src, "w").write(PROG_INT01)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                               "-I", os.path.join(ROOT, "viltrum_gb300", "csrc"), src, "-o", exe])
        out = list(map(int, subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()))
        n, fb, bad = out[0:10:2], out[1:10:2], out[10]
        assert bad == 0, out
        assert fb[0] <= n[0] * 1e-4, out   # ordinary coefficients: certified (exact ties included)
        assert fb[1] <= n[1] * 1e-2, out   # terms 2^60 apart: ties the reference's doubles do not hold exactly
        assert fb[4] == n[4], out                                    # zeros and specials: always declined
        assert 0 < fb[2] < n[2] and 0 < fb[3] < n[3], out            # near-boundary cases: some of each
