/*
 * vcu_refrule.h -- Newton-Cotes rule values rounded exactly as the reference rounds them.
 * Host and device compile the same code (tests/test_refrule.py checks it on the host against
 * the reference's double-promoted expressions).
 */
#pragma once
#include "../../include/vcu_integrands.h"
#if !defined(__CUDACC__)
#include <cmath>
#include <cstring>
#endif

namespace vcu {

/* ---------------------------------------------------------------------------------------------
 * The rule VALUE as the reference computes it, used for the nested error estimate that decides
 * every split.  For float node values the reference evaluates e.g. Boole's
 *     (7.0*p0 + 32.0*p1 + 12.0*p2 + 32.0*p3 + 7.0*p4) / 90.0
 * in double and rounds once to float (rules.h:254-257): the products are exact, the double sum is
 * exact whenever the nodes span fewer than ~2^23 in magnitude, and the result is the float nearest
 * to sum/90.  ref_scalar() reproduces that on the FP32 pipe: the weighted sum is accumulated
 * error-free as a float-float pair (two-product / two-sum), then divided with a correctly rounded
 * FP32 division plus one residual correction.  It differs from the reference only where the
 * reference itself double-rounds (result within 2^-29 ulp of a float rounding boundary).
 * ref_rgb() is the same expression for the 3-channel value type, whose operators round every
 * step to float (oracle/vrgb.h semantics).
 * ------------------------------------------------------------------------------------------- */
VCU_HD void two_sum(float a, float b, float& s, float& e) {
    s = vadd(a, b);
    const float bb = vsub(s, a);
    e = vadd(vsub(a, vsub(s, bb)), vsub(b, bb));
}
VCU_HD void two_prod(float a, float b, float& p, float& e) {
    p = vmul(a, b);
    e = vfma(a, b, -p);
}
/* nextafter(x, +inf) / nextafter(x, -inf) for the finite quotients ff_div produces: one integer
 * step of the bit pattern (+/-0 go to the smallest subnormal; infinities and NaN are returned) */
VCU_HD float next_up(float x) {
    const uint32_t u = float_to_bits(x);
    if ((u & 0x7fffffffu) == 0u) return bits_to_float(1u);
    if ((u & 0x7f800000u) == 0x7f800000u) return (u == 0xff800000u) ? bits_to_float(0xff7fffffu) : x;
    return bits_to_float((u >> 31) ? u - 1u : u + 1u);
}
VCU_HD float next_down(float x) { return -next_up(-x); }
VCU_HD bool even_bits(float x) {
#if defined(__CUDA_ARCH__)
    return (__float_as_uint(x) & 1u) == 0u;
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return (u & 1u) == 0u;
#endif
}
/* The exact rounding decision of ff_div below for its candidate q0 and the exact remainder
 * R = s + e = h + l - q0*D: R/D beyond half the gap to a neighbour moves to it, exactly half (or
 * within the 2^-30-ulp band where the reference's intermediate double lands on the midpoint) ties
 * to even. */
VCU_HD float ff_div_decide(float q0, float s, float e, float D) {
    const float up = next_up(q0), dn = next_down(q0);
    const float tu = vmul(D, vmul(vsub(up, q0), 0.5f)); /* exact: D * half gap above */
    const float td = vmul(D, vmul(vsub(q0, dn), 0.5f)); /* exact: D * half gap below */
    const float band = vmul(tu, 9.313225746154785e-10f); /* 2^-30 of the half gap */
    /* distance of R above +tu and below -td, each as (float + small float) */
    const float du = vadd(vsub(s, tu), e);
    const float dd = vadd(vsub(-s, td), -e);
    if (vabs(du) <= band) return even_bits(q0) ? q0 : up;
    if (vabs(dd) <= band) return even_bits(q0) ? q0 : dn;
    if (du > 0.0f) return up;
    if (dd > 0.0f) return dn;
    return q0;
}
/* RN_f(RN_d((h + l) / D)) for the float-float pair (h, l) and a small positive integer D, as the
 * reference's "double sum / double constant, assigned to float" rounds it.  q0 (a corrected
 * RN(h/D)) is within one float of the result; the exact remainder R = h + l - q0*D (two_sum of the
 * exact fma residual and l) decides (ff_div_decide). */
VCU_HD float ff_div(float h, float l, float D, float inv_D /* RN(1/D) */) {
    /* q00 ~ h/D, then one approximate correction step brings q0 within one float of the result
     * (the exact decision does the rest).  For h = 0 or |h| in [2^-90, 2^90] the product by
     * RN(1/D) is close enough; outside that range (subnormal quotients, near overflow) a true
     * division. */
    const float ah = vabs(h);
    float q00 = vmul(h, inv_D);
    if (!((ah >= 8.077935669463161e-28f || ah == 0.0f) && ah <= 1.2379400392853803e27f)) q00 = vdiv(h, D);
    const float q0 = vfma(vadd(vfma(-q00, D, h), l), inv_D, q00);
    float s, e;
    two_sum(vfma(-q0, D, h), l, s, e);
    /* Common cases first, with ff_div_decide's results.  q0 normal, not a power of two (both
     * neighbours one ulp away, so the half gaps tu = td = D ulp / 2):
     *  - |s| below tu (1 - 2^-20), with |e| <= 2^-24 |s|: R/D is farther than 2^-21 ulp from either
     *    midpoint, outside the tie band: q0.  (The threshold RN(D (1 - 2^-20) / 2) ulp is within
     *    2^-24 of that bound.)
     *  - R = +-tu exactly (e = 0): an exact tie, to the even neighbour -- frequent for Simpson's
     *    (p0 + 4 p1 + p2) / 6, whose numerator often has one bit more than a multiple of 3.
     * Any q0 with R = 0 (s = e = 0): the quotient is exact. */
    const uint32_t u = float_to_bits(q0);
    const uint32_t ex = u & 0x7f800000u;
    if ((u & 0x007fffffu) != 0u && ex >= (25u << 23) && ex < (254u << 23)) {
        const float ulp = bits_to_float(ex - (23u << 23));
        const float as = vabs(s);
        if (as <= vmul(ulp, vmul(D, 0.49999952316284180f /* (1 - 2^-20) / 2 */))) return q0;
        if (e == 0.0f && as == vmul(vmul(D, 0.5f), ulp)) {
            if ((u & 1u) == 0u) return q0;
            return bits_to_float(((s > 0.0f) == (q0 > 0.0f)) ? u + 1u : u - 1u); /* the neighbour on R's side */
        }
    } else if (s == 0.0f && e == 0.0f) {
        return q0;
    }
    return ff_div_decide(q0, s, e, D);
}

/* (p0 + 4.0*p1 + p2)/6.0 and (7.0*p0 + 32.0*p1 + 12.0*p2 + 32.0*p3 + 7.0*p4)/90.0 as the reference
 * rounds them: error-free float-float sums, then ff_div */
VCU_HD float ref_simpson(float p0, float p1, float p2) {
    float h, e1, h2, e2;
    two_sum(p0, vmul(4.0f, p1), h, e1);
    two_sum(h, p2, h2, e2);
    return ff_div(h2, vadd(e1, e2), 6.0f, 0.1666666716337204f /* RN(1/6) */);
}
VCU_HD float ref_boole(float p0, float p1, float p2, float p3, float p4) {
    float h, l, ph, pl, e;
    two_prod(7.0f, p0, h, l);
    two_sum(h, vmul(32.0f, p1), h, e);
    l = vadd(l, e);
    two_prod(12.0f, p2, ph, pl);
    two_sum(h, ph, h, e);
    l = vadd(l, vadd(pl, e));
    two_sum(h, vmul(32.0f, p3), h, e);
    l = vadd(l, e);
    two_prod(7.0f, p4, ph, pl);
    two_sum(h, ph, h, e);
    l = vadd(l, vadd(pl, e));
    return ff_div(h, l, 90.0f, 0.011111111380159855f /* RN(1/90) */);
}

/* sum_k c[k] / (k + 1), the integral over [0, 1] of the power-basis polynomial c[0] + c[1] t + ... of
 * a rule of S nodes, as the reference rounds subrange(0, 1) for float coefficients: Horner steps in
 * double ("c[k]*t/(k+1.0)" a float product divided in double), the result rounded once to float
 * (rules.h:41-44, 96-100, 288-293; the antiderivative at 0 is a zero).  Here the terms are summed
 * error-free as a float-float pair (h, l), the divisions by 3 and 5 as the IEEE quotient plus its exact
 * remainder's share.  Two ways to the reference's float:
 *  - the reference's double value and h + l both lie within ~2^-44 T of the exact sum (T: the sum of
 *    the terms' magnitudes), so q = RN(h + l) is the reference's float whenever every value within
 *    E = 2^-40 T of h + l rounds to q (rounding is monotone: the two ends of that interval suffice);
 *  - where that fails because the sum sits on or next to a rounding boundary, the sum may be exact:
 *    every term a float (zero division remainders, exact halvings), so all are multiples of the
 *    smallest term's ulp u; with T < 2^51 u every double step of the reference is exact, and if l
 *    also carries the error terms exactly, RN(h + l) is the reference's float (ties to even alike).
 * Returns false otherwise -- a boundary within E of an inexact sum, a sum that cancels to below
 * ~2^-17 T, T outside [2^-60, 2^60] or not finite -- and the caller evaluates the reference's double
 * expression instead. */
VCU_HD bool ref_certify(float h, float l, float T, float& out) {
    const float q = vadd(h, l);
    const float r = vadd(vsub(h, q), l);
    const float E = vmul(T, 9.094947017729282e-13f); /* 2^-40 */
    if (vadd(q, vsub(r, E)) != q || vadd(q, vadd(r, E)) != q) return false;
    out = q;
    return true;
}
VCU_HD bool ref_in_range(float T) { /* 2^-60 <= T <= 2^60 (false for NaN) */
    return T >= 8.673617379884035e-19f && T <= 1.152921504606847e18f;
}
/* the exponent field of the smallest ulp among the non-zero terms (1 for subnormals; 255 if all are
 * zero), and whether T < 2^51 times that ulp */
VCU_HD bool ref_exact_span(const float* t, int n, float T) {
    uint32_t ef = 255u;
    for (int i = 0; i < n; ++i) {
        const uint32_t e = (float_to_bits(t[i]) >> 23) & 0xffu;
        if (float_to_bits(t[i]) << 1) ef = (e == 0u ? 1u : e) < ef ? (e == 0u ? 1u : e) : ef;
    }
    if (ef == 255u) return false; /* all zero: the signs of zeros are the double path's */
    /* u = 2^(ef - 150); 2^51 u = 2^(ef - 99) as a float: exponent field ef - 99 + 127 */
    const uint32_t bf = ef + 28u;
    if (bf >= 255u) return false;
    return T < bits_to_float(bf << 23);
}
template <int S> VCU_HD bool ref_integral01(const float* c, float& out);
template <> VCU_HD bool ref_integral01<3>(const float* c, float& out) {
    /* c2/3 + c1/2 + c0 */
    const float a = fdiv_c<3>(c[2]);
    const float ra = vfma(-a, 3.0f, c[2]); /* exact remainder */
    const float b = vmul(c[1], 0.5f);
    float s, e1, h, e2;
    two_sum(a, b, s, e1);
    two_sum(s, c[0], h, e2);
    const float T = vadd(vadd(vabs(a), vabs(b)), vabs(c[0]));
    if (!ref_in_range(T)) return false;
    if (ref_certify(h, vadd(vadd(vmul(ra, 0.3333333432674408f), e1), e2), T, out)) return true;
    float l, le;
    two_sum(e1, e2, l, le);
    const float terms[3] = {a, b, c[0]};
    if (ra != 0.0f || le != 0.0f || vmul(b, 2.0f) != c[1] || !ref_exact_span(terms, 3, T)) return false;
    out = vadd(h, l);
    return true;
}
template <> VCU_HD bool ref_integral01<5>(const float* c, float& out) {
    /* c4/5 + c3/4 + c2/3 + c1/2 + c0, summed in the reference's order */
    const float a5 = fdiv_c<5>(c[4]);
    const float r5 = vfma(-a5, 5.0f, c[4]);
    const float b4 = vmul(c[3], 0.25f);
    const float a3 = fdiv_c<3>(c[2]);
    const float r3 = vfma(-a3, 3.0f, c[2]);
    const float b2 = vmul(c[1], 0.5f);
    float s, e1, e2, e3, h, e4;
    two_sum(a5, b4, s, e1);
    two_sum(s, a3, s, e2);
    two_sum(s, b2, s, e3);
    two_sum(s, c[0], h, e4);
    const float T = vadd(vadd(vadd(vadd(vabs(a5), vabs(b4)), vabs(a3)), vabs(b2)), vabs(c[0]));
    if (!ref_in_range(T)) return false;
    const float l0 = vadd(vmul(r5, 0.20000000298023224f), vmul(r3, 0.3333333432674408f));
    if (ref_certify(h, vadd(vadd(vadd(vadd(l0, e1), e2), e3), e4), T, out)) return true;
    if (r5 != 0.0f || r3 != 0.0f || vmul(b4, 4.0f) != c[3] || vmul(b2, 2.0f) != c[1]) return false;
    float l, le1, le2, le3;
    two_sum(e1, e2, l, le1);
    two_sum(l, e3, l, le2);
    two_sum(l, e4, l, le3);
    const float terms[5] = {a5, b4, a3, b2, c[0]};
    if (le1 != 0.0f || le2 != 0.0f || le3 != 0.0f || !ref_exact_span(terms, 5, T)) return false;
    out = vadd(h, l);
    return true;
}

template <int S> struct RefRule;
template <> struct RefRule<2> { /* (p0+p1)/2.0: float sum, exact halving */
    static VCU_HD float scalar(const float* p) { return vmul(vadd(p[0], p[1]), 0.5f); }
    static VCU_HD float rgb(const float* p) { return vmul(vadd(p[0], p[1]), 0.5f); }
};
template <> struct RefRule<3> { /* (p0 + 4.0*p1 + p2)/6.0 */
    static VCU_HD float scalar(const float* p) { return ref_simpson(p[0], p[1], p[2]); }
    static VCU_HD float rgb(const float* p) {
        return vdiv(vadd(vadd(p[0], vmul(4.0f, p[1])), p[2]), 6.0f);
    }
};
template <> struct RefRule<5> { /* (7.0*p0 + 32.0*p1 + 12.0*p2 + 32.0*p3 + 7.0*p4)/90.0 */
    static VCU_HD float scalar(const float* p) { return ref_boole(p[0], p[1], p[2], p[3], p[4]); }
    static VCU_HD float rgb(const float* p) {
        const float s = vadd(vadd(vadd(vadd(vmul(7.0f, p[0]), vmul(32.0f, p[1])), vmul(12.0f, p[2])), vmul(32.0f, p[3])),
                             vmul(7.0f, p[4]));
        return vdiv(s, 90.0f);
    }
};

}  // namespace vcu
