/*
 * vcu_pdf.cuh -- polynomial importance sampling of a Simpson region on the device.
 *
 * viltrum samples the residual of its control variates in proportion to the control variate itself
 * (src/newton-cotes/rules.h:102-248, src/newton-cotes/region.h:220-343): along each line of three
 * nodes the norms of the node values define a parabola, lifted so that its minimum on [0,1] is 0
 * (pdf_points); integrals of that parabola over [a,b] fold a region's nodes into marginals, its
 * value at a point folds them into the unnormalised density, and a coordinate is drawn by solving
 * cdf(t) = x, a cubic, in closed form (Cardano, or Viete's trigonometric form for three roots).
 *
 * The float steps round as the reference's float code does (explicit _rn operations; no
 * contraction), the double steps (the lift's vertex, the cdf's Horner steps, the cubic) run in
 * double; the cubic's pow/sqrt/acos/cos are CUDA's double-precision functions, so a drawn coordinate
 * can differ from the reference's in the last float bits.  Node values of a region are given as
 * their norms (sum of |channel|, norm.h:11-24), dimension 0 fastest.
 */
#pragma once

#include "vcu_rules.cuh"

namespace vcu {
namespace pdf3 {

__host__ __device__ constexpr int pow3(int e) { return e <= 0 ? 1 : 3 * pow3(e - 1); }

/* pdf_points (rules.h:104-145): |p| lifted by the parabola's minimum inside (0,1) when it dips below 0 */
__device__ __forceinline__ void points(const float* in, float* q) {
    q[0] = vabs(in[0]);
    q[1] = vabs(in[1]);
    q[2] = vabs(in[2]);
    float c[3];
    Rule<3>::coefficients(q, c);
    float ymin = 0.0f;
    if (c[2] > 0.0f) {
        const float tmin = __double2float_rn(__ddiv_rn((double)(-c[1]), __dmul_rn(2.0, (double)c[2])));
        if (tmin > 0.0f && tmin < 1.0f) {
            const float ytmin = vadd(vmul(vadd(vmul(c[2], tmin), c[1]), tmin), c[0]);
            if (ytmin < ymin) ymin = ytmin;
        }
    }
    q[0] = vsub(q[0], ymin);
    q[1] = vsub(q[1], ymin);
    q[2] = vsub(q[2], ymin);
}

/* pdf_integral_subrange over [a,b] of one line (rules.h:150-154) */
__device__ __forceinline__ float line_integral(float a, float b, const float* in) {
    float q[3];
    points(in, q);
    return subrange_ref<3>(a, b, q);
}

/* pdf_unnormalized at t of one line (rules.h:157-161) */
__device__ __forceinline__ float line_at(float t, const float* in) {
    float q[3];
    points(in, q);
    return Rule<3>::at(t, q);
}

/* cdf(t) of the lifted parabola (rules.h:176-180): float product, Horner steps in double */
__device__ __forceinline__ float cdf(float t, const float* c) {
    double r = __dadd_rn(ddiv_f<3>(vmul(c[2], t)), __dmul_rn((double)c[1], 0.5));
    r = __dadd_rn(__dmul_rn(r, (double)t), (double)c[0]);
    return __double2float_rn(__dmul_rn(r, (double)t));
}

__device__ __forceinline__ double cuberoot(double x) { return (x < 0) ? -pow(-x, 1.0 / 3.0) : pow(x, 1.0 / 3.0); }

/* the roots of cdf(t) = x in the reference's order (rules.h:182-225); returns how many */
static __device__ __noinline__ int inv_cdf(float x, const float* q, float* sol) {
    float co[3];
    Rule<3>::coefficients(q, co);
    double a = ddiv_f<3>(co[2]);
    double b = __dmul_rn((double)co[1], 0.5);
    float c = co[0];
    float d = -x;
    const double sum = __dadd_rn(__dadd_rn(__dadd_rn(a, b), (double)c), (double)d);
    a = __ddiv_rn(a, sum);
    b = __ddiv_rn(b, sum);
    c = __double2float_rn(__ddiv_rn((double)c, sum));
    d = __double2float_rn(__ddiv_rn((double)d, sum));
    int n = 0;
    if (fabs(a) < 1.e-3) {
        if (fabs(b) < 1.e-3) {
            if (fabsf(c) >= 1.e-3) sol[n++] = vdiv(-d, c);
        } else {
            const double disc = __dsub_rn((double)vmul(c, c), __dmul_rn(__dmul_rn(4.0, b), (double)d));
            if (disc >= 0) {
                const double sq = sqrt(disc), b2 = __dmul_rn(2.0, b);
                sol[n++] = __double2float_rn(__ddiv_rn(__dadd_rn((double)(-c), sq), b2));
                sol[n++] = __double2float_rn(__ddiv_rn(__dsub_rn((double)(-c), sq), b2));
            }
        }
    } else {
        const double a2 = pow(a, 2.0), a3 = pow(a, 3.0), b2 = pow(b, 2.0), b3 = pow(b, 3.0);
        const double p = __dsub_rn(__ddiv_rn((double)c, a), __ddiv_rn(b2, __dmul_rn(3.0, a2)));
        const double q3 = __dadd_rn(__dsub_rn(__ddiv_rn(__dmul_rn(2.0, b3), __dmul_rn(27.0, a3)),
                                              __ddiv_rn(__dmul_rn(b, (double)c), __dmul_rn(3.0, a2))),
                                    __ddiv_rn((double)d, a));
        const double sqr = __dadd_rn(pow(__ddiv_rn(q3, 2.0), 2.0), pow(__ddiv_rn(p, 3.0), 3.0));
        const double shift = __ddiv_rn(b, __dmul_rn(3.0, a));
        if (sqr >= 0.) {
            const double s = sqrt(sqr), h = __ddiv_rn(-q3, 2.0);
            sol[n++] = __double2float_rn(__dsub_rn(__dadd_rn(cuberoot(__dsub_rn(h, s)), cuberoot(__dadd_rn(h, s))), shift));
        } else {
            const double m = __dmul_rn(2.0, sqrt(__ddiv_rn(-p, 3.0)));
            const double th = acos(__dmul_rn(__ddiv_rn(__dmul_rn(3.0, q3), __dmul_rn(2.0, p)), sqrt(__ddiv_rn(-3.0, p))));
            for (int i = 0; i < 3; ++i) {
                const double ang = __dsub_rn(__dmul_rn(1.0 / 3.0, th), __ddiv_rn(__dmul_rn(2.0 * 3.141592653589793, (double)i), 3.0));
                sol[n++] = __double2float_rn(__dsub_rn(__dmul_rn(m, cos(ang)), shift));
            }
        }
    }
    return n;
}

/* a coordinate of [t0,t1] with density proportional to the lifted parabola of the line; uniform when
 * no root lies in the interval (rules.h:227-246) */
static __device__ __noinline__ float line_sample(float s, float t0, float t1, const float* in) {
    float q[3], c[3];
    points(in, q);
    Rule<3>::coefficients(q, c);
    const float x = vadd(vmul(s, cdf(t1, c)), vmul(vsub(1.0f, s), cdf(t0, c)));
    float sol[3];
    const int n = inv_cdf(x, q, sol);
    for (int i = 0; i < n; ++i) {
        float r = sol[i];
        if (r < t0 && (double)fabsf(vsub(t0, r)) < 1.e-5) r = t0;
        if (r > t1 && (double)fabsf(vsub(r, t1)) < 1.e-5) r = t1;
        if (r >= t0 && r <= t1 && !isnan(r)) return r;
    }
    return vadd(vmul(s, vsub(t1, t0)), t0);
}

/* fold dimension d of a k-dimensional 3^k array (dimension 0 fastest) into out[3^(k-1)].  Folding the
 * first (d = 0) or the last (d = k-1) dimension may be done in place (out == in): output J is written
 * after its line is read, and every line read later starts beyond J. */
template <class Fn> __device__ __forceinline__ void fold(const float* in, int k, int d, float* out, const Fn& fn) {
    const int outn = pow3(k - 1), sd = pow3(d);
#pragma unroll 1
    for (int J = 0; J < outn; ++J) {
        const int base = J % sd + (J / sd) * sd * 3;
        const float l[3] = {in[base], in[base + sd], in[base + 2 * sd]};
        out[J] = fn(l);
    }
}

/* Folds of a DIM-dimensional region's node norms N over bin n region, [A,B] in the region's unit
 * coordinates.  Each fold overwrites N. */
template <int DIM> struct Region {
    /* pdf_sub (region.h:267-283): integrals over [A_d,B_d], the last dimension first */
    static __device__ __noinline__ float integral(float* N, const float* A, const float* B) {
#pragma unroll 1
        for (int k = DIM; k >= 1; --k) {
            const int d = k - 1;
            fold(N, k, d, N, [&](const float* l) { return line_integral(A[d], B[d], l); });
        }
        return N[0];
    }
    /* pdf_at (region.h:293-307): the unnormalised density at P, the last dimension first */
    static __device__ __noinline__ float at(float* N, const float* P) {
#pragma unroll 1
        for (int k = DIM; k >= 1; --k) {
            const int d = k - 1;
            fold(N, k, d, N, [&](const float* l) { return line_at(P[d], l); });
        }
        return N[0];
    }
    /* sample_subrange_i / sample_marginal (region.h:220-257): the first remaining dimension from its
     * marginal (the others integrated over [A,B], last first, into M: 3^(DIM-1) floats), then the
     * density conditioned on it (dimension 0 of N folded at the drawn coordinate); sol in unit
     * coordinates */
    static __device__ __noinline__ void sample(float* N, float* M, const float* U, const float* A, const float* B,
                                               float* sol) {
#pragma unroll 1
        for (int off = 0; off < DIM; ++off) {
            const int k = DIM - off;
            if (k == 1) {
                sol[off] = line_sample(U[off], A[off], B[off], N);
                break;
            }
            {
                const int dd = off + k - 1;
                fold(N, k, k - 1, M, [&](const float* l) { return line_integral(A[dd], B[dd], l); });
            }
#pragma unroll 1
            for (int j = k - 1; j >= 2; --j) {
                const int dd = off + j - 1;
                fold(M, j, j - 1, M, [&](const float* l) { return line_integral(A[dd], B[dd], l); });
            }
            sol[off] = line_sample(U[off], A[off], B[off], M);
            const float t = sol[off];
            fold(N, k, 0, N, [&](const float* l) { return line_at(t, l); });
        }
    }
};

}  // namespace pdf3
}  // namespace vcu
