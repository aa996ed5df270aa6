/*
 * vcu_rules.cuh -- Newton-Cotes rule arithmetic on the device, in FP32.
 *
 * The coefficient formulas and evaluation order follow src/newton-cotes/rules.h:9-319 (power-basis
 * coefficients in float, Horner at(), exact sub-range integral subrange()); every operation is an
 * explicitly rounded FP32 operation (vmul/vadd/vsub/vdiv), where the reference promotes the outer
 * Horner steps to double.
 *
 * Nested error (src/nested/nested.h:25-33): the error metric of the two rule values H(p), L(p)
 * decides every split, so the rule values are reproduced exactly as the reference rounds them
 * (RefRule below), without the FP64 pipe (GB300's FP64 rate is 1/64 of FP32).
 */
#pragma once
#include "../../include/vcu_integrands.h"
#include "vcu_refrule.h"

namespace vcu {

template <int S> struct Rule;

/* Divisions by the rules' constants: by 2 and 4 as the equal products (exact scalings), by 3 and 5
 * through fdiv_c (the IEEE quotient, see vcu_integrands.h).  subrange01() is subrange(0, 1, p):
 * the antiderivative at 1 with the products by 1 left out, minus the one at 0, which is a zero for
 * finite coefficients -- subtracting it changes at most the sign of a zero result -- so it is
 * evaluated only when the value at 1 is not finite.  subrange01 divides without fdiv_c's select of
 * the special operands (G = false): that differs from the IEEE quotient only by the sign of a zero
 * quotient and by NaN for an infinite operand, so a finite result differs at most in the sign of a
 * zero, and a non-finite one is recomputed with the selects. */
template <int D, bool G> __device__ __forceinline__ float div_c(float x) {
    if constexpr (G) {
        return fdiv_c<D>(x);
    } else {
        constexpr float inv = 1.0f / (float)D;
        const float q0 = vmul(x, inv);
        return vfma(vfma(-q0, (float)D, x), inv, q0);
    }
}
template <> struct Rule<2> { /* trapezoidal */
    static __device__ __forceinline__ float rule(const float* p) { return vmul(vadd(p[0], p[1]), 0.5f); }
    static __device__ __forceinline__ void coefficients(const float* p, float* c) {
        c[0] = p[0];
        c[1] = vsub(p[1], p[0]);
    }
    static __device__ __forceinline__ float horner_at(const float* c, float t) { return vadd(vmul(c[1], t), c[0]); }
    static __device__ __forceinline__ float at(float t, const float* p) {
        float c[2];
        coefficients(p, c);
        return horner_at(c, t);
    }
    static __device__ __forceinline__ float horner_int(const float* c, float t) {
        return vmul(vadd(vmul(vmul(c[1], t), 0.5f), c[0]), t);
    }
    static __device__ __forceinline__ float horner_int1(const float* c) { return vadd(vmul(c[1], 0.5f), c[0]); }
    static __device__ __forceinline__ float subrange(float a, float b, const float* p) {
        float c[2];
        coefficients(p, c);
        return vsub(horner_int(c, b), horner_int(c, a));
    }
    static __device__ __forceinline__ float subrange01(const float* p) {
        float c[2];
        coefficients(p, c);
        const float h1 = horner_int1(c);
        return isfinite(h1) ? h1 : vsub(h1, horner_int(c, 0.0f));
    }
};

template <> struct Rule<3> { /* simpson */
    static __device__ __forceinline__ float rule(const float* p) {
        return vdiv(vadd(vadd(p[0], vmul(4.0f, p[1])), p[2]), 6.0f);
    }
    static __device__ __forceinline__ void coefficients(const float* p, float* c) {
        c[0] = p[0];
        c[1] = vsub(vadd(vmul(-3.0f, p[0]), vmul(4.0f, p[1])), p[2]);
        c[2] = vadd(vsub(vmul(2.0f, p[0]), vmul(4.0f, p[1])), vmul(2.0f, p[2]));
    }
    static __device__ __forceinline__ float horner_at(const float* c, float t) {
        return vadd(vmul(vadd(vmul(c[2], t), c[1]), t), c[0]);
    }
    static __device__ __forceinline__ float at(float t, const float* p) {
        float c[3];
        coefficients(p, c);
        return horner_at(c, t);
    }
    static __device__ __forceinline__ float horner_int(const float* c, float t) {
        float r = vadd(fdiv_c<3>(vmul(c[2], t)), vmul(c[1], 0.5f));
        r = vadd(vmul(r, t), c[0]);
        return vmul(r, t);
    }
    template <bool G = true> static __device__ __forceinline__ float horner_int1(const float* c) {
        return vadd(vadd(div_c<3, G>(c[2]), vmul(c[1], 0.5f)), c[0]);
    }
    static __device__ __forceinline__ float subrange(float a, float b, const float* p) {
        float c[3];
        coefficients(p, c);
        return vsub(horner_int(c, b), horner_int(c, a));
    }
    static __device__ __noinline__ float subrange01_special(float p0, float p1, float p2) {
        const float p[3] = {p0, p1, p2};
        float c[3];
        coefficients(p, c);
        return vsub(horner_int1(c), horner_int(c, 0.0f));
    }
    static __device__ __forceinline__ float subrange01(const float* p) {
        float c[3];
        coefficients(p, c);
        const float h1 = horner_int1<false>(c);
        return isfinite(h1) ? h1 : subrange01_special(p[0], p[1], p[2]);
    }
};

template <> struct Rule<5> { /* boole */
    static __device__ __forceinline__ float rule(const float* p) {
        const float s = vadd(vadd(vmul(7.0f, vadd(p[0], p[4])), vmul(32.0f, vadd(p[1], p[3]))), vmul(12.0f, p[2]));
        return vdiv(s, 90.0f);
    }
    template <bool G = true> static __device__ __forceinline__ void coefficients(const float* p, float* c) {
        c[0] = p[0];
        c[1] = vsub(vadd(vsub(vadd(div_c<3, G>(vmul(-25.0f, p[0])), vmul(16.0f, p[1])), vmul(12.0f, p[2])),
                         div_c<3, G>(vmul(16.0f, p[3]))),
                    p[4]);
        c[2] = vadd(vsub(vadd(vsub(div_c<3, G>(vmul(70.0f, p[0])), div_c<3, G>(vmul(208.0f, p[1]))), vmul(76.0f, p[2])),
                         div_c<3, G>(vmul(112.0f, p[3]))),
                    div_c<3, G>(vmul(22.0f, p[4])));
        c[3] = vsub(vadd(vsub(vadd(div_c<3, G>(vmul(-80.0f, p[0])), vmul(96.0f, p[1])), vmul(128.0f, p[2])),
                         div_c<3, G>(vmul(224.0f, p[3]))),
                    vmul(16.0f, p[4]));
        c[4] = vadd(vsub(vadd(vsub(div_c<3, G>(vmul(32.0f, p[0])), div_c<3, G>(vmul(128.0f, p[1]))), vmul(64.0f, p[2])),
                         div_c<3, G>(vmul(128.0f, p[3]))),
                    div_c<3, G>(vmul(32.0f, p[4])));
    }
    static __device__ __forceinline__ float horner_at(const float* c, float t) {
        float r = vadd(vmul(c[4], t), c[3]);
        r = vadd(vmul(r, t), c[2]);
        r = vadd(vmul(r, t), c[1]);
        return vadd(vmul(r, t), c[0]);
    }
    static __device__ __forceinline__ float at(float t, const float* p) {
        float c[5];
        coefficients(p, c);
        return horner_at(c, t);
    }
    static __device__ __forceinline__ float horner_int(const float* c, float t) {
        float r = vadd(fdiv_c<5>(vmul(c[4], t)), vmul(c[3], 0.25f));
        r = vadd(vmul(r, t), fdiv_c<3>(c[2]));
        r = vadd(vmul(r, t), vmul(c[1], 0.5f));
        r = vadd(vmul(r, t), c[0]);
        return vmul(r, t);
    }
    template <bool G = true> static __device__ __forceinline__ float horner_int1(const float* c) {
        float r = vadd(div_c<5, G>(c[4]), vmul(c[3], 0.25f));
        r = vadd(r, div_c<3, G>(c[2]));
        r = vadd(r, vmul(c[1], 0.5f));
        return vadd(r, c[0]);
    }
    static __device__ __forceinline__ float subrange(float a, float b, const float* p) {
        float c[5];
        coefficients(p, c);
        return vsub(horner_int(c, b), horner_int(c, a));
    }
    static __device__ __noinline__ float subrange01_special(float p0, float p1, float p2, float p3, float p4) {
        const float p[5] = {p0, p1, p2, p3, p4};
        float c[5];
        coefficients(p, c);
        return vsub(horner_int1(c), horner_int(c, 0.0f));
    }
    static __device__ __forceinline__ float subrange01(const float* p) {
        float c[5];
        coefficients<false>(p, c);
        const float h1 = horner_int1<false>(c);
        return isfinite(h1) ? h1 : subrange01_special(p[0], p[1], p[2], p[3], p[4]);
    }
};

/* subrange() as the reference computes it for float nodes (rules.h:41-44, 96-100, 288-293): float
 * coefficients, then the Horner steps in double ("c[k]*b/5.0" is a float product divided in double)
 * and the difference of the two ends rounded once to float.  (Divisions by 2 and 4 are exact in
 * double, so they are written as the equal multiplications.)  Used where bin n region can be a short
 * piece of a large region (control variates), so the two Horner values nearly cancel. */
template <int S> __device__ __forceinline__ double horner_int_ref(const float* c, float t);
template <> __device__ __forceinline__ double horner_int_ref<2>(const float* c, float t) {
    double r = __dadd_rn(__dmul_rn((double)vmul(c[1], t), 0.5), (double)c[0]); /* /2.0 is exact */
    return __dmul_rn(r, (double)t);
}
template <> __device__ __forceinline__ double horner_int_ref<3>(const float* c, float t) {
    double r = __dadd_rn(ddiv_f<3>(vmul(c[2], t)), __dmul_rn((double)c[1], 0.5));
    r = __dadd_rn(__dmul_rn(r, (double)t), (double)c[0]);
    return __dmul_rn(r, (double)t);
}
template <> __device__ __forceinline__ double horner_int_ref<5>(const float* c, float t) {
    double r = __dadd_rn(ddiv_f<5>(vmul(c[4], t)), __dmul_rn((double)c[3], 0.25));
    r = __dadd_rn(__dmul_rn(r, (double)t), ddiv_f<3>(c[2]));
    r = __dadd_rn(__dmul_rn(r, (double)t), __dmul_rn((double)c[1], 0.5));
    r = __dadd_rn(__dmul_rn(r, (double)t), (double)c[0]);
    return __dmul_rn(r, (double)t);
}
template <int S> __device__ __forceinline__ float subrange_ref(float a, float b, const float* p) {
    float c[S];
    Rule<S>::coefficients(p, c);
    return __double2float_rn(__dsub_rn(horner_int_ref<S>(c, b), horner_int_ref<S>(c, a)));
}

/* error metrics (src/nested/error-metric.h): absolute |L-H|, relative |L-H|/max(|H|,|L|) unless
 * max(|H|,|L|) < min_val */
__device__ __forceinline__ float metric_value(int relative, float min_val, float H, float L) {
    const float ad = vabs(vsub(L, H));
    if (!relative) return ad;
    const float aH = vabs(H), aL = vabs(L);
    const float m = (aH < aL) ? aL : aH;
    return (m < min_val) ? ad : vdiv(ad, m);
}

/* exact node coordinate float(p*w + m) with p a dyadic fraction, computed as the reference does
 * it in double (src/newton-cotes/region.h:39-47) */
/* node positions in [0,1]: j/(S-1) and (2k+1)/(2(S-1)), as the reference computes them in double
 * (region.h:62-78, split.h:13-49); S-1 is a power of two for every rule, so the quotients are
 * exact products by a constant */
template <int S> __device__ __forceinline__ double node_pos(int j) {
    static_assert(S == 2 || S == 3 || S == 5, "S-1 must be a power of two");
    return (double)j * (1.0 / (double)(S - 1));
}
template <int S> __device__ __forceinline__ double mid_pos(int k) {
    static_assert(S == 2 || S == 3 || S == 5, "S-1 must be a power of two");
    return (double)(2 * k + 1) * (0.5 / (double)(S - 1));
}
__device__ __forceinline__ float node_coord(double p, float w, float m) {
    /* p has at most 3 significant bits, so p*w is exact in double and the fused form rounds
     * p*w + m once, as the reference's product-then-sum does */
    return __double2float_rn(__fma_rn(p, (double)w, (double)m));
}

/* std::max / std::min semantics: (a < b) ? b : a */
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }

}  // namespace vcu
