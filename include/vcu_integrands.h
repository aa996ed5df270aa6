/*
 * vcu_integrands.h -- built-in integrands of libviltrum_cuda, compiled identically for the host
 * (g++, -ffp-contract=off) and the device (nvcc).
 *
 * An integrand cannot cross a C ABI as code, so every integrand the library can run is a
 * trivially-copyable functor defined here and selected by a VCU_F_* tag (vcu_integrand::kind).
 * The functor is built on the host from a flat float parameter array and handed to the kernels
 * BY VALUE (a __grid_constant__ kernel parameter), exactly as viltrum passes its integrand
 * functor by const reference into Integrator::integrate (src/integrate.h:72-79).
 *
 * Every operation is spelled out with explicit rounding (vmul/vadd/vsub/vfma below): on the
 * device they map to the __f*_rn intrinsics, which the compiler never contracts; on the host
 * the file is compiled with -ffp-contract=off.  The transcendental functions are the
 * project's own (vexp, vsin, vcos: Cody-Waite range reduction + Taylor polynomials), not the
 * platform's, so a host evaluation and a device evaluation of the same point return the same
 * bits.  This is what lets the adaptive-quadrature split decisions of the GPU be compared
 * one-to-one with the CPU reference path.
 */
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define VCU_HD __host__ __device__ __forceinline__
#else
#define VCU_HD inline
#include <cmath>
#include <cstring>
#endif

namespace vcu {

/* ---------------------------------------------------------------- explicit-rounding ops */
VCU_HD float vmul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
VCU_HD float vadd(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
VCU_HD float vsub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
VCU_HD float vdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
VCU_HD float vfma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
VCU_HD float vrint(float a) {
#if defined(__CUDA_ARCH__)
    return rintf(a);
#else
    return std::rint(a);
#endif
}
VCU_HD float vabs(float a) {
#if defined(__CUDA_ARCH__)
    return fabsf(a);
#else
    return std::fabs(a);
#endif
}
/* RN_d(x / D) of a float x (D = 3 or 5, the divisors of the reference's double-promoted Horner
 * steps) without the double division routine: q0 = RN_d(x * RN_d(1/D)), then one correction by the
 * exact remainder, q = RN_d(q0 + (x - q0*D) * RN_d(1/D)) (the correction step of Markstein's
 * division; Brisebarre, Muller and Raina, IEEE Trans. Computers 53(8), 2004).  q equals the
 * correctly rounded quotient for every finite non-zero float x (checked over all 2^32 floats;
 * tests/test_ddivf.py re-checks every significand at several exponents); zeros, infinities and NaN
 * return q0, which is exact for them. */
template <int D> VCU_HD double ddiv_f(float xf) {
    static_assert(D == 3 || D == 5, "ddiv_f: divisor not checked");
    const double x = (double)xf;
    constexpr double inv = 1.0 / (double)D;
#if defined(__CUDA_ARCH__)
    const double q0 = __dmul_rn(x, inv);
    const double q = __fma_rn(__fma_rn(-q0, (double)D, x), inv, q0);
#else
    const double q0 = x * inv;
    const double q = std::fma(std::fma(-q0, (double)D, x), inv, q0);
#endif
    return (xf != 0.0f && vabs(xf) <= 3.4028234663852886e38f) ? q : q0;
}
/* RN(x / D) of a float x for D = 3 or 5 without the division routine: q0 = RN(x RN(1/D)), then the
 * same correction by the exact remainder as ddiv_f, in float.  q equals the IEEE quotient for every
 * finite non-zero float x (all 2^32 checked; tests/test_ddivf.py re-checks every significand at
 * several exponents); zeros, infinities and NaN return q0, which is the IEEE quotient for them. */
template <int D> VCU_HD float fdiv_c(float x) {
    static_assert(D == 3 || D == 5, "fdiv_c: divisor not checked");
    constexpr float inv = 1.0f / (float)D;
    const float q0 = vmul(x, inv);
    const float q = vfma(vfma(-q0, (float)D, x), inv, q0);
    return (x != 0.0f && vabs(x) <= 3.4028234663852886e38f) ? q : q0;
}
/* index of the lowest set bit of a non-zero mask */
VCU_HD int ctz64(uint64_t m) {
#if defined(__CUDA_ARCH__)
    return __ffsll((long long)m) - 1;
#else
    return __builtin_ctzll(m);
#endif
}
VCU_HD int ctz32(uint32_t m) {
#if defined(__CUDA_ARCH__)
    return __ffs((int)m) - 1;
#else
    return __builtin_ctz(m);
#endif
}
VCU_HD uint32_t float_to_bits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; std::memcpy(&u, &f, 4); return u;
#endif
}
VCU_HD float bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; std::memcpy(&f, &u, 4); return f;
#endif
}

/* ---------------------------------------------------------------- portable transcendentals
 * Constants are exact splits of ln 2 and pi/2 into float parts with 12 significant bits in
 * the high and middle parts (so k*hi and k*mid are exact for |k| < 2^12), and the Taylor
 * coefficients 1/n! rounded to float.  Both were computed from exact decimal arithmetic.   */
constexpr float kLog2e = 1.4426950216293335f;
constexpr float kLn2Hi = 0.693115234375f;
constexpr float kLn2Mi = 3.193318843841553e-05f;
constexpr float kLn2Lo = 1.2996506981721723e-08f;
constexpr float kTwoOverPi = 0.6366197466850281f;
constexpr float kPio2Hi = 1.5703125f;
constexpr float kPio2Mi = 0.0004837512969970703f;
constexpr float kPio2Lo = 7.549790126404332e-08f;
constexpr float kInvFact2 = 0.5f;
constexpr float kInvFact3 = 0.1666666716337204f;
constexpr float kInvFact4 = 0.0416666679084301f;
constexpr float kInvFact5 = 0.008333333767950535f;
constexpr float kInvFact6 = 0.0013888889225199819f;
constexpr float kInvFact7 = 0.00019841270113829523f;
constexpr float kInvFact8 = 2.4801587642286904e-05f;
constexpr float kInvFact9 = 2.7557318844628753e-06f;
constexpr float kInvFact10 = 2.755731998149713e-07f;

/* e^x: x = k ln2 + r, |r| <= ln2/2, e^r by its degree-7 Taylor polynomial (truncation error
 * < 6e-9 relative), times 2^k assembled in the exponent field.  Results below 2^-126 are
 * returned as 0 (no denormals), results above FLT_MAX as +inf.                              */
VCU_HD float vexp_core(float x) {
    /* k = rint(x log2e) by the 1.5*2^23 shift (exact round-to-nearest-even for |t| < 2^22);
     * the integer k is the difference of the two bit patterns, no float->int conversion */
    const float t = vadd(vmul(x, kLog2e), 12582912.0f);
    const float k = vsub(t, 12582912.0f);
    float r = vfma(-k, kLn2Hi, x);
    r = vfma(-k, kLn2Mi, r);
    r = vfma(-k, kLn2Lo, r);
    float p = kInvFact7;
    p = vfma(p, r, kInvFact6);
    p = vfma(p, r, kInvFact5);
    p = vfma(p, r, kInvFact4);
    p = vfma(p, r, kInvFact3);
    p = vfma(p, r, kInvFact2);
    p = vfma(p, r, 1.0f);
    p = vfma(p, r, 1.0f);
    /* k in [-126, 128] for the clamped argument: p * 2^k with 2^min(k,127) built in the exponent
     * field (p in [0.7, 1.42], so p * 2^127 is exact) and one more doubling for k = 128 */
    const int ki = (int)(float_to_bits(t) - 0x4B400000u);
    const float s = bits_to_float((uint32_t)((ki < 127 ? ki : 127) + 127) << 23);
    const float ps = vmul(p, s);
    return (ki > 127) ? vmul(ps, 2.0f) : ps;
}
/* branch-free: the core runs on the clamped argument and the special results are selected, so
 * that loops of exponentials (and two interleaved evaluations) compile without divergent branches */
VCU_HD float vexp(float x) {
    const float xc = (x > 88.5f) ? 88.5f : ((x > -87.0f) ? x : -87.0f);
    const float core = vexp_core(xc);
    return (x > -87.0f) ? ((x > 88.5f) ? bits_to_float(0x7f800000u) : core) : ((x != x) ? x : 0.0f);
}
/* vexp(x) for the arguments of a Gaussian bump, x <= 0 or NaN: the same bits (NaN for NaN), with
 * the clamps and the exponent assembly of the positive range left out.  The core runs on x itself:
 * for x <= -87 (where its value is meaningless) one select returns 0; a NaN propagates through the
 * polynomial.  For x in (-87, 0], k = rint(x log2e) lies in [-126, 0], so 2^k is (k + 127) << 23,
 * and bits(t) = 0x4B400000 + k has the low 9 bits of k: bits(t) << 23 is (k << 23) mod 2^32, one
 * multiply-add. */
VCU_HD float vexp_nonpos(float x) {
    const bool under = x <= -87.0f;
    const float xc = x;
    const float t = vadd(vmul(xc, kLog2e), 12582912.0f);
    const float k = vsub(t, 12582912.0f);
    float r = vfma(-k, kLn2Hi, xc);
    r = vfma(-k, kLn2Mi, r);
    r = vfma(-k, kLn2Lo, r);
    float p = kInvFact7;
    p = vfma(p, r, kInvFact6);
    p = vfma(p, r, kInvFact5);
    p = vfma(p, r, kInvFact4);
    p = vfma(p, r, kInvFact3);
    p = vfma(p, r, kInvFact2);
    p = vfma(p, r, 1.0f);
    p = vfma(p, r, 1.0f);
    const float s = bits_to_float(float_to_bits(t) * 8388608u + 0x3F800000u);
    const float ps = vmul(p, s);
    return under ? 0.0f : ps;
}

/* sin and cos of the reduced argument |r| <= pi/4 (Taylor to degree 9 and 10). */
VCU_HD float sin_kernel(float r) {
    const float r2 = vmul(r, r);
    float p = kInvFact9;
    p = vfma(p, r2, -kInvFact7);
    p = vfma(p, r2, kInvFact5);
    p = vfma(p, r2, -kInvFact3);
    p = vmul(p, r2);
    return vfma(p, r, r);
}
VCU_HD float cos_kernel(float r) {
    const float r2 = vmul(r, r);
    float p = -kInvFact10;
    p = vfma(p, r2, kInvFact8);
    p = vfma(p, r2, -kInvFact6);
    p = vfma(p, r2, kInvFact4);
    p = vfma(p, r2, -kInvFact2);
    return vfma(p, r2, 1.0f);
}
/* Quadrant reduction x = k pi/2 + r; accurate for |x| < 4000 (k*hi exact).                 */
VCU_HD float vsincos_q(float x, int add_quadrant) {
    const float k = vrint(vmul(x, kTwoOverPi));
    float r = vfma(-k, kPio2Hi, x);
    r = vfma(-k, kPio2Mi, r);
    r = vfma(-k, kPio2Lo, r);
    const int q = ((int)k + add_quadrant) & 3;
    const float s = (q & 1) ? cos_kernel(r) : sin_kernel(r);
    return (q & 2) ? -s : s;
}
VCU_HD float vsin(float x) { return vsincos_q(x, 0); }
VCU_HD float vcos(float x) { return vsincos_q(x, 1); }

/* ---------------------------------------------------------------- integrand tags */
enum IntegrandKind : int32_t {
    VCU_F_POLY2 = 1,          /* x^2 + y^2 on 2-D (main/doc/integrators.cc:6-11)                */
    VCU_F_SIN1 = 2,           /* sin(x) on 1-D (main/doc/montecarlo-1d.cc:6-12)                 */
    VCU_F_SPHERE3 = 3,        /* indicator x^2+y^2+z^2 <= 1 on 3-D (main/doc/integrands.cc:3-5)  */
    VCU_F_WAVE2 = 4,          /* sin(8x) e^-y + x^2 + y^2 on 2-D (per-bin Monte Carlo workload)   */
    VCU_F_SCENE2 = 5,         /* Gaussian bumps + hard-edged disks on 2-D                          */
    VCU_F_MOVING_SCENE3 = 6,  /* bumps + disks moving over t, RGB, on 3-D (x, y, t)                */
    VCU_F_HALFSPACE = 7,      /* prod_d e^{-a_d x_d} cos(b_d x_d) [n.x < c], 2..6-D                */
    VCU_F_OCCLUDED_SCENE5 = 8, /* SCENE2(x,y) times box visibility of a segment, 5-D               */
    VCU_F_WALK2 = 9           /* random walk over SCENE2 from (x,y): unbounded dimensions          */
};

constexpr int kMaxGauss = 64;
constexpr int kMaxDisk = 32;
constexpr int kMaxBox = 128;
constexpr int kMaxHalfspaceDim = 6;
#if defined(__CUDA_ARCH__)
#define VCU_UNROLL _Pragma("unroll")
#else
#define VCU_UNROLL
#endif

/* ---------------------------------------------------------------- functors
 * Each functor: static DIM (compile-time arity) and CH (value channels), a host-side
 * build(params, n) returning 0 on success, and operator()(const float* x, float* out).      */

struct Poly2 {
    static constexpr int DIM = 2, CH = 1;
    int32_t dummy;
    VCU_HD void operator()(const float* x, float* out) const {
        out[0] = vadd(vmul(x[0], x[0]), vmul(x[1], x[1]));
    }
};

struct Sin1 {
    static constexpr int DIM = 1, CH = 1;
    int32_t dummy;
    VCU_HD void operator()(const float* x, float* out) const { out[0] = vsin(x[0]); }
};

struct Sphere3 {
    static constexpr int DIM = 3, CH = 1;
    int32_t dummy;
    VCU_HD void operator()(const float* x, float* out) const {
        const float r2 = vadd(vadd(vmul(x[0], x[0]), vmul(x[1], x[1])), vmul(x[2], x[2]));
        out[0] = (r2 <= 1.0f) ? 1.0f : 0.0f;
    }
};

struct Wave2 {
    static constexpr int DIM = 2, CH = 1;
    int32_t dummy;
    VCU_HD void operator()(const float* x, float* out) const {
        float t = vmul(vsin(vmul(8.0f, x[0])), vexp(-x[1]));
        t = vadd(t, vmul(x[0], x[0]));
        out[0] = vadd(t, vmul(x[1], x[1]));
    }
};

/* Scene parameters (flat float array, as produced by viltrum_gb300.scenes):
 *   [0] n_gauss, [1] n_disk,
 *   n_gauss x (cx, cy, sigma, amplitude), n_disk x (cx, cy, radius, value)
 * The functor stores the exponent factor -1/(2 sigma^2) and the squared radius, computed once
 * here with explicit float rounding.                                                          */
struct Scene2 {
    static constexpr int DIM = 2, CH = 1;
    int32_t ng, nd;
    float g[kMaxGauss][4]; /* cx, cy, -1/(2 s^2), amplitude */
    float d[kMaxDisk][4];  /* cx, cy, r^2, value           */

    int build(const float* p, int n) {
        if (n < 2) return 1;
        ng = (int32_t)p[0];
        nd = (int32_t)p[1];
        if (ng < 0 || nd < 0 || ng > kMaxGauss || nd > kMaxDisk) return 1;
        if (n < 2 + 4 * ng + 4 * nd) return 1;
        const float* q = p + 2;
        for (int i = 0; i < ng; ++i, q += 4) {
            g[i][0] = q[0];
            g[i][1] = q[1];
            g[i][2] = vdiv(-0.5f, vmul(q[2], q[2]));
            g[i][3] = q[3];
        }
        for (int i = 0; i < nd; ++i, q += 4) {
            d[i][0] = q[0];
            d[i][1] = q[1];
            d[i][2] = vmul(q[2], q[2]);
            d[i][3] = q[3];
        }
        return 0;
    }
    VCU_HD float eval(float x, float y) const {
        float acc = 0.0f;
        for (int i = 0; i < ng; ++i) {
            const float dx = vsub(x, g[i][0]);
            const float dy = vsub(y, g[i][1]);
            const float r2 = vfma(dx, dx, vmul(dy, dy));
            acc = vfma(g[i][3], vexp_nonpos(vmul(r2, g[i][2])), acc);
        }
        for (int i = 0; i < nd; ++i) {
            const float dx = vsub(x, d[i][0]);
            const float dy = vsub(y, d[i][1]);
            const float r2 = vfma(dx, dx, vmul(dy, dy));
            acc = vadd(acc, (r2 <= d[i][2]) ? d[i][3] : 0.0f);
        }
        return acc;
    }
    VCU_HD void operator()(const float* x, float* out) const { out[0] = eval(x[0], x[1]); }
    /* The terms that can be non-zero somewhere in the box [lo, hi]: a bump whose exponent rounds to
     * -87 or below at every point of the box contributes exactly 0 (vexp returns 0 there and
     * fma(a, 0, acc) == acc, acc never being -0), as does a disk that misses the box.  The test is
     * conservative: the box grown by 1e-6 plus 1e-6 of each bound's magnitude (the evaluated points
     * may stray a few ulps outside the box of a bin) and a 1e-4 relative margin on the squared
     * distance, far above the rounding of the evaluation's own dx, dy, r^2 and product.  multi_cull() then sums
     * only the kept terms, in the same order, so its results equal multi()'s bit for bit. */
    struct Cull {
        uint64_t g;
        uint32_t d;
    };
    /* The same decision term by term, for callers that spread the terms over lanes: the grown box
     * (x0, y0, x1, y1), then term t of the mask's three 32-bit words (bumps 0-31, bumps 32-63,
     * disks 0-31; false past ng / nd) */
    static constexpr int kCullWords = 3, kCullBox = 4;
    VCU_HD void cull_prepare(const float* lo, const float* hi, float* box) const {
        auto grow = [](float v) { return vadd(1e-6f, vmul(v < 0.0f ? -v : v, 1e-6f)); };
        box[0] = vsub(lo[0], grow(lo[0]));
        box[1] = vsub(lo[1], grow(lo[1]));
        box[2] = vadd(hi[0], grow(hi[0]));
        box[3] = vadd(hi[1], grow(hi[1]));
    }
    VCU_HD bool cull_keep(int t, const float* box) const {
        auto dist2 = [&](float cx, float cy) {
            const float ex = vsub(box[0], cx), fx = vsub(cx, box[2]), ey = vsub(box[1], cy), fy = vsub(cy, box[3]);
            const float dx = ex > 0.0f ? ex : (fx > 0.0f ? fx : 0.0f);
            const float dy = ey > 0.0f ? ey : (fy > 0.0f ? fy : 0.0f);
            return vfma(dx, dx, vmul(dy, dy));
        };
        if (t < 64) {
            if (t >= ng) return false;
            return !(vmul(vmul(dist2(g[t][0], g[t][1]), -g[t][2]), 0.9999f) > 87.0f);
        }
        const int i = t - 64;
        if (i >= nd) return false;
        return !(vmul(dist2(d[i][0], d[i][1]), 0.9999f) > d[i][2]);
    }
    VCU_HD static Cull cull_from_words(const uint32_t* w) { return Cull{(uint64_t)w[0] | ((uint64_t)w[1] << 32), w[2]}; }
    VCU_HD Cull cull(const float* lo, const float* hi) const {
        float box[4];
        cull_prepare(lo, hi, box);
        uint32_t w[kCullWords] = {0u, 0u, 0u};
        for (int t = 0; t < 32 * kCullWords; ++t)
            if (cull_keep(t, box)) w[t >> 5] |= 1u << (t & 31);
        return cull_from_words(w);
    }
    template <int N> VCU_HD void multi_cull(const Cull& c, const float (*x)[DIM], float (*o)[CH]) const {
        float a[N];
        VCU_UNROLL
        for (int p = 0; p < N; ++p) a[p] = 0.0f;
        /* the kept bumps in index order, one 32-bit half of the mask after the other */
        for (int half = 0; half < 2; ++half) {
            uint32_t m = half ? (uint32_t)(c.g >> 32) : (uint32_t)c.g;
            const int base = 32 * half;
            while (m) {
                const int i = base + ctz32(m);
                m &= m - 1;
                const float gx0 = g[i][0], gy0 = g[i][1], gs0 = g[i][2], ga0 = g[i][3];
                if (m) { /* two kept bumps per step, independent exponentials, the sum in order */
                    const int j = base + ctz32(m);
                    m &= m - 1;
                    const float gx1 = g[j][0], gy1 = g[j][1], gs1 = g[j][2], ga1 = g[j][3];
                    float e0[N], e1[N];
                    VCU_UNROLL
                    for (int p = 0; p < N; ++p) {
                        const float dx0 = vsub(x[p][0], gx0), dy0 = vsub(x[p][1], gy0);
                        const float dx1 = vsub(x[p][0], gx1), dy1 = vsub(x[p][1], gy1);
                        e0[p] = vexp_nonpos(vmul(vfma(dx0, dx0, vmul(dy0, dy0)), gs0));
                        e1[p] = vexp_nonpos(vmul(vfma(dx1, dx1, vmul(dy1, dy1)), gs1));
                    }
                    VCU_UNROLL
                    for (int p = 0; p < N; ++p) a[p] = vfma(ga1, e1[p], vfma(ga0, e0[p], a[p]));
                } else {
                    VCU_UNROLL
                    for (int p = 0; p < N; ++p) {
                        const float dx = vsub(x[p][0], gx0), dy = vsub(x[p][1], gy0);
                        a[p] = vfma(ga0, vexp_nonpos(vmul(vfma(dx, dx, vmul(dy, dy)), gs0)), a[p]);
                    }
                }
            }
        }
        uint32_t dm = c.d;
        while (dm) {
            const int i = ctz32(dm);
            dm &= dm - 1;
            const float cx = d[i][0], cy = d[i][1], rr = d[i][2], dv = d[i][3];
            VCU_UNROLL
            for (int p = 0; p < N; ++p) {
                const float dx = vsub(x[p][0], cx), dy = vsub(x[p][1], cy);
                const float r2 = vfma(dx, dx, vmul(dy, dy));
                a[p] = vadd(a[p], (r2 <= rr) ? dv : 0.0f);
            }
        }
        VCU_UNROLL
        for (int p = 0; p < N; ++p) o[p][0] = a[p];
    }
    /* N points at once, each with exactly the arithmetic of eval(): N independent chains */
    template <int N> VCU_HD void multi(const float (*x)[DIM], float (*o)[CH]) const {
        float a[N];
        VCU_UNROLL
        for (int p = 0; p < N; ++p) a[p] = 0.0f;
        int i = 0;
        for (; i + 1 < ng; i += 2) {
            /* two bumps per step: their exponentials are independent chains; the sum keeps the order */
            const float gx0 = g[i][0], gy0 = g[i][1], gs0 = g[i][2], ga0 = g[i][3];
            const float gx1 = g[i + 1][0], gy1 = g[i + 1][1], gs1 = g[i + 1][2], ga1 = g[i + 1][3];
            float e0[N], e1[N];
            VCU_UNROLL
            for (int p = 0; p < N; ++p) {
                const float dx0 = vsub(x[p][0], gx0), dy0 = vsub(x[p][1], gy0);
                const float dx1 = vsub(x[p][0], gx1), dy1 = vsub(x[p][1], gy1);
                e0[p] = vexp_nonpos(vmul(vfma(dx0, dx0, vmul(dy0, dy0)), gs0));
                e1[p] = vexp_nonpos(vmul(vfma(dx1, dx1, vmul(dy1, dy1)), gs1));
            }
            VCU_UNROLL
            for (int p = 0; p < N; ++p) a[p] = vfma(ga1, e1[p], vfma(ga0, e0[p], a[p]));
        }
        for (; i < ng; ++i) {
            const float gx = g[i][0], gy = g[i][1], gs = g[i][2], ga = g[i][3];
            VCU_UNROLL
            for (int p = 0; p < N; ++p) {
                const float dx = vsub(x[p][0], gx), dy = vsub(x[p][1], gy);
                const float r2 = vfma(dx, dx, vmul(dy, dy));
                a[p] = vfma(ga, vexp_nonpos(vmul(r2, gs)), a[p]);
            }
        }
        for (int i = 0; i < nd; ++i) {
            const float cx = d[i][0], cy = d[i][1], rr = d[i][2], dv = d[i][3];
            VCU_UNROLL
            for (int p = 0; p < N; ++p) {
                const float dx = vsub(x[p][0], cx), dy = vsub(x[p][1], cy);
                const float r2 = vfma(dx, dx, vmul(dy, dy));
                a[p] = vadd(a[p], (r2 <= rr) ? dv : 0.0f);
            }
        }
        VCU_UNROLL
        for (int p = 0; p < N; ++p) o[p][0] = a[p];
    }
    VCU_HD void pair(const float* x0, const float* x1, float* o0, float* o1) const {
        const float x[2][2] = {{x0[0], x0[1]}, {x1[0], x1[1]}};
        float o[2][1];
        multi<2>(x, o);
        o0[0] = o[0][0];
        o1[0] = o[1][0];
    }
};

/* Moving scene, 3 channels, on (x, y, t):
 *   [0] n_gauss, [1] n_disk,
 *   n_gauss x (cx, cy, sigma, amplitude)                   -- static, grey
 *   n_disk  x (cx, cy, vx, vy, radius, r, g, b)            -- centre (cx + t vx, cy + t vy)
 */
struct MovingScene3 {
    static constexpr int DIM = 3, CH = 3;
    int32_t ng, nd;
    float g[kMaxGauss][4];
    float d[kMaxDisk][8]; /* cx, cy, vx, vy, r^2, r, g, b */

    int build(const float* p, int n) {
        if (n < 2) return 1;
        ng = (int32_t)p[0];
        nd = (int32_t)p[1];
        if (ng < 0 || nd < 0 || ng > kMaxGauss || nd > kMaxDisk) return 1;
        if (n < 2 + 4 * ng + 8 * nd) return 1;
        const float* q = p + 2;
        for (int i = 0; i < ng; ++i, q += 4) {
            g[i][0] = q[0];
            g[i][1] = q[1];
            g[i][2] = vdiv(-0.5f, vmul(q[2], q[2]));
            g[i][3] = q[3];
        }
        for (int i = 0; i < nd; ++i, q += 8) {
            d[i][0] = q[0];
            d[i][1] = q[1];
            d[i][2] = q[2];
            d[i][3] = q[3];
            d[i][4] = vmul(q[4], q[4]);
            d[i][5] = q[5];
            d[i][6] = q[6];
            d[i][7] = q[7];
        }
        return 0;
    }
    VCU_HD void operator()(const float* x, float* out) const {
        float grey = 0.0f;
        for (int i = 0; i < ng; ++i) {
            const float dx = vsub(x[0], g[i][0]);
            const float dy = vsub(x[1], g[i][1]);
            const float r2 = vfma(dx, dx, vmul(dy, dy));
            grey = vfma(g[i][3], vexp_nonpos(vmul(r2, g[i][2])), grey);
        }
        float c0 = grey, c1 = grey, c2 = grey;
        for (int i = 0; i < nd; ++i) {
            const float cx = vfma(x[2], d[i][2], d[i][0]);
            const float cy = vfma(x[2], d[i][3], d[i][1]);
            const float dx = vsub(x[0], cx);
            const float dy = vsub(x[1], cy);
            const float r2 = vfma(dx, dx, vmul(dy, dy));
            if (r2 <= d[i][4]) {
                c0 = vadd(c0, d[i][5]);
                c1 = vadd(c1, d[i][6]);
                c2 = vadd(c2, d[i][7]);
            }
        }
        out[0] = c0;
        out[1] = c1;
        out[2] = c2;
    }
    /* The terms that can be non-zero over the box [lo, hi] of (x, y, t): a bump as Scene2::cull
     * decides (static), a disk whose centre's path over [lo[2], hi[2]] -- the segment between its
     * centres at the two ends, the centre being monotone in t -- stays farther than its radius from the
     * box.  Same conservative margins as Scene2::cull (box grown by 1e-6 plus 1e-6 of each bound's
     * magnitude, 1e-4 relative on the squared distance).  eval_culled() then sums only the kept terms in
     * the same order, so it returns operator()'s bits at every point of the box (a skipped bump adds
     * fma(a, 0, grey) = grey, a skipped disk adds nothing). */
    struct CullBox {
        uint64_t g;
        uint32_t d;
    };
    VCU_HD CullBox cull_box(const float* lo, const float* hi) const {
        auto grow = [](float v) { return vadd(1e-6f, vmul(v < 0.0f ? -v : v, 1e-6f)); };
        const float x0 = vsub(lo[0], grow(lo[0])), y0 = vsub(lo[1], grow(lo[1]));
        const float x1 = vadd(hi[0], grow(hi[0])), y1 = vadd(hi[1], grow(hi[1]));
        auto gap = [](float a0, float a1, float b0, float b1) { /* distance between [a0,a1] and [b0,b1] */
            const float e = vsub(b0, a1), f = vsub(a0, b1);
            return e > 0.0f ? e : (f > 0.0f ? f : 0.0f);
        };
        CullBox c{0ull, 0u};
        for (int i = 0; i < ng; ++i) {
            const float dx = gap(x0, x1, g[i][0], g[i][0]), dy = gap(y0, y1, g[i][1], g[i][1]);
            if (!(vmul(vmul(vfma(dx, dx, vmul(dy, dy)), -g[i][2]), 0.9999f) > 87.0f)) c.g |= 1ull << i;
        }
        for (int i = 0; i < nd; ++i) {
            const float ca = vfma(lo[2], d[i][2], d[i][0]), cb = vfma(hi[2], d[i][2], d[i][0]);
            const float da = vfma(lo[2], d[i][3], d[i][1]), db = vfma(hi[2], d[i][3], d[i][1]);
            float sx0 = ca < cb ? ca : cb, sx1 = ca < cb ? cb : ca, sy0 = da < db ? da : db, sy1 = da < db ? db : da;
            sx0 = vsub(sx0, grow(sx0));
            sx1 = vadd(sx1, grow(sx1));
            sy0 = vsub(sy0, grow(sy0));
            sy1 = vadd(sy1, grow(sy1));
            const float dx = gap(x0, x1, sx0, sx1), dy = gap(y0, y1, sy0, sy1);
            if (!(vmul(vfma(dx, dx, vmul(dy, dy)), 0.9999f) > d[i][4])) c.d |= 1u << i;
        }
        return c;
    }
    VCU_HD void eval_culled(const CullBox& c, const float* x, float* out) const {
        float grey = 0.0f;
        uint64_t m = c.g;
        while (m) {
            const int i = ctz64(m);
            m &= m - 1;
            const float dx = vsub(x[0], g[i][0]);
            const float dy = vsub(x[1], g[i][1]);
            const float r2 = vfma(dx, dx, vmul(dy, dy));
            grey = vfma(g[i][3], vexp_nonpos(vmul(r2, g[i][2])), grey);
        }
        float c0 = grey, c1 = grey, c2 = grey;
        uint32_t dm = c.d;
        while (dm) {
            const int i = ctz32(dm);
            dm &= dm - 1;
            const float cx = vfma(x[2], d[i][2], d[i][0]);
            const float cy = vfma(x[2], d[i][3], d[i][1]);
            const float dx = vsub(x[0], cx);
            const float dy = vsub(x[1], cy);
            const float r2 = vfma(dx, dx, vmul(dy, dy));
            if (r2 <= d[i][4]) {
                c0 = vadd(c0, d[i][5]);
                c1 = vadd(c1, d[i][6]);
                c2 = vadd(c2, d[i][7]);
            }
        }
        out[0] = c0;
        out[1] = c1;
        out[2] = c2;
    }
    /* two points of the box at once: eval_culled's arithmetic for each, the kept terms' loops shared */
    VCU_HD void pair_culled(const CullBox& c, const float* x0, const float* x1, float* o0, float* o1) const {
        float g0 = 0.0f, g1 = 0.0f;
        uint64_t m = c.g;
        while (m) {
            const int i = ctz64(m);
            m &= m - 1;
            const float gx = g[i][0], gy = g[i][1], gs = g[i][2], ga = g[i][3];
            const float dx0 = vsub(x0[0], gx), dy0 = vsub(x0[1], gy);
            const float dx1 = vsub(x1[0], gx), dy1 = vsub(x1[1], gy);
            const float r0 = vfma(dx0, dx0, vmul(dy0, dy0));
            const float r1 = vfma(dx1, dx1, vmul(dy1, dy1));
            g0 = vfma(ga, vexp_nonpos(vmul(r0, gs)), g0);
            g1 = vfma(ga, vexp_nonpos(vmul(r1, gs)), g1);
        }
        float a0 = g0, a1 = g0, a2 = g0, b0 = g1, b1 = g1, b2 = g1;
        uint32_t dm = c.d;
        while (dm) {
            const int i = ctz32(dm);
            dm &= dm - 1;
            const float cx0 = vfma(x0[2], d[i][2], d[i][0]), cy0 = vfma(x0[2], d[i][3], d[i][1]);
            const float cx1 = vfma(x1[2], d[i][2], d[i][0]), cy1 = vfma(x1[2], d[i][3], d[i][1]);
            const float dx0 = vsub(x0[0], cx0), dy0 = vsub(x0[1], cy0);
            const float dx1 = vsub(x1[0], cx1), dy1 = vsub(x1[1], cy1);
            const float r0 = vfma(dx0, dx0, vmul(dy0, dy0));
            const float r1 = vfma(dx1, dx1, vmul(dy1, dy1));
            if (r0 <= d[i][4]) {
                a0 = vadd(a0, d[i][5]);
                a1 = vadd(a1, d[i][6]);
                a2 = vadd(a2, d[i][7]);
            }
            if (r1 <= d[i][4]) {
                b0 = vadd(b0, d[i][5]);
                b1 = vadd(b1, d[i][6]);
                b2 = vadd(b2, d[i][7]);
            }
        }
        o0[0] = a0;
        o0[1] = a1;
        o0[2] = a2;
        o1[0] = b0;
        o1[1] = b1;
        o1[2] = b2;
    }
    /* two points at once, each with exactly the arithmetic of operator() */
    VCU_HD void pair(const float* x0, const float* x1, float* o0, float* o1) const {
        float g0 = 0.0f, g1 = 0.0f;
        for (int i = 0; i < ng; ++i) {
            const float gx = g[i][0], gy = g[i][1], gs = g[i][2], ga = g[i][3];
            const float dx0 = vsub(x0[0], gx), dy0 = vsub(x0[1], gy);
            const float dx1 = vsub(x1[0], gx), dy1 = vsub(x1[1], gy);
            const float r0 = vfma(dx0, dx0, vmul(dy0, dy0));
            const float r1 = vfma(dx1, dx1, vmul(dy1, dy1));
            g0 = vfma(ga, vexp_nonpos(vmul(r0, gs)), g0);
            g1 = vfma(ga, vexp_nonpos(vmul(r1, gs)), g1);
        }
        float a0 = g0, a1 = g0, a2 = g0, b0 = g1, b1 = g1, b2 = g1;
        for (int i = 0; i < nd; ++i) {
            const float cx0 = vfma(x0[2], d[i][2], d[i][0]), cy0 = vfma(x0[2], d[i][3], d[i][1]);
            const float cx1 = vfma(x1[2], d[i][2], d[i][0]), cy1 = vfma(x1[2], d[i][3], d[i][1]);
            const float dx0 = vsub(x0[0], cx0), dy0 = vsub(x0[1], cy0);
            const float dx1 = vsub(x1[0], cx1), dy1 = vsub(x1[1], cy1);
            const float r0 = vfma(dx0, dx0, vmul(dy0, dy0));
            const float r1 = vfma(dx1, dx1, vmul(dy1, dy1));
            if (r0 <= d[i][4]) {
                a0 = vadd(a0, d[i][5]);
                a1 = vadd(a1, d[i][6]);
                a2 = vadd(a2, d[i][7]);
            }
            if (r1 <= d[i][4]) {
                b0 = vadd(b0, d[i][5]);
                b1 = vadd(b1, d[i][6]);
                b2 = vadd(b2, d[i][7]);
            }
        }
        o0[0] = a0;
        o0[1] = a1;
        o0[2] = a2;
        o1[0] = b0;
        o1[1] = b1;
        o1[2] = b2;
    }
};

/* Separable smooth product times a half-space indicator, dimension dim (2..6):
 *   [0] dim, [1..6] a_d, [7..12] b_d, [13..18] n_d, [19] c
 *   f(x) = prod_d e^{-a_d x_d} cos(b_d x_d)  if  sum_d n_d x_d < c,  else 0
 * The functor's DIM is the maximum; the kernels use dim() at run time for the arity.        */
struct Halfspace {
    static constexpr int DIM = kMaxHalfspaceDim, CH = 1;
    int32_t dim;
    float a[kMaxHalfspaceDim], b[kMaxHalfspaceDim], nrm[kMaxHalfspaceDim], c;

    int build(const float* p, int n) {
        if (n < 20) return 1;
        dim = (int32_t)p[0];
        if (dim < 1 || dim > kMaxHalfspaceDim) return 1;
        for (int i = 0; i < kMaxHalfspaceDim; ++i) {
            a[i] = p[1 + i];
            b[i] = p[7 + i];
            nrm[i] = p[13 + i];
        }
        c = p[19];
        return 0;
    }
    VCU_HD void operator()(const float* x, float* out) const {
        /* loops unrolled to the maximum arity and predicated, so that x[] stays in registers */
        float dot = 0.0f;
        VCU_UNROLL
        for (int i = 0; i < kMaxHalfspaceDim; ++i)
            if (i < dim) dot = vfma(nrm[i], x[i], dot);
        if (!(dot < c)) {
            out[0] = 0.0f;
            return;
        }
        float v = 1.0f;
        VCU_UNROLL
        for (int i = 0; i < kMaxHalfspaceDim; ++i)
            if (i < dim) v = vmul(v, vmul(vexp(-vmul(a[i], x[i])), vcos(vmul(b[i], x[i]))));
        out[0] = v;
    }
};

/* Scene2 on (x, y) times the visibility of the segment from (x, y, 0) to (u, v, h) with
 * h = 0.25 + 0.75 w, against axis-aligned boxes (slab test):
 *   scene parameters as Scene2, then [k] n_box, n_box x (cx, cy, cz, hx, hy, hz)            */
struct OccludedScene5 {
    static constexpr int DIM = 5, CH = 1;
    Scene2 scene;
    int32_t nb;
    float lo[kMaxBox][3], hi[kMaxBox][3];

    int build(const float* p, int n) {
        if (scene.build(p, n)) return 1;
        const int off = 2 + 4 * scene.ng + 4 * scene.nd;
        if (n < off + 1) return 1;
        nb = (int32_t)p[off];
        if (nb < 0 || nb > kMaxBox || n < off + 1 + 6 * nb) return 1;
        const float* q = p + off + 1;
        for (int i = 0; i < nb; ++i, q += 6)
            for (int k = 0; k < 3; ++k) {
                lo[i][k] = vsub(q[k], q[3 + k]);
                hi[i][k] = vadd(q[k], q[3 + k]);
            }
        return 0;
    }
    VCU_HD float visibility(const float* x) const {
        const float o[3] = {x[0], x[1], 0.0f};
        const float e[3] = {x[2], x[3], vfma(0.75f, x[4], 0.25f)};
        float dir[3], inv[3];
        for (int k = 0; k < 3; ++k) {
            dir[k] = vsub(e[k], o[k]);
            inv[k] = vdiv(1.0f, dir[k]);
        }
        for (int i = 0; i < nb; ++i) {
            float t0 = 0.0f, t1 = 1.0f;
            for (int k = 0; k < 3; ++k) {
                float ta = vmul(vsub(lo[i][k], o[k]), inv[k]);
                float tb = vmul(vsub(hi[i][k], o[k]), inv[k]);
                if (ta > tb) { const float s = ta; ta = tb; tb = s; }
                /* a NaN (0 * inf on a face) leaves the interval unchanged */
                t0 = (ta > t0) ? ta : t0;
                t1 = (tb < t1) ? tb : t1;
            }
            if (t0 <= t1) return 0.0f;
        }
        return 1.0f;
    }
    VCU_HD void operator()(const float* x, float* out) const {
        const float s = scene.eval(x[0], x[1]);
        out[0] = (s == 0.0f) ? 0.0f : vmul(s, visibility(x));
    }
    /* two points at once: the scene by Scene2::pair, then both segments against the boxes in one
     * loop that ends when both are blocked (each point's result is that of operator()) */
    VCU_HD void pair(const float* x0, const float* x1, float* o0, float* o1) const {
        float s[2];
        {
            const float a0[2] = {x0[0], x0[1]}, a1[2] = {x1[0], x1[1]};
            scene.pair(a0, a1, &s[0], &s[1]);
        }
        visible_pair(s, x0, x1, o0, o1);
    }
    /* The scene terms that can be non-zero over the box [lo, hi] (its first two coordinates:
     * Scene2::cull), and pair() evaluating only those: bit for bit pair()'s results for points whose
     * first two coordinates lie in the box. */
    using CullBox = Scene2::Cull;
    VCU_HD CullBox cull_box(const float* lo, const float* hi) const { return scene.cull(lo, hi); }
    VCU_HD void pair_culled(const CullBox& c, const float* x0, const float* x1, float* o0, float* o1) const {
        const float a[2][2] = {{x0[0], x0[1]}, {x1[0], x1[1]}};
        float so[2][1];
        scene.multi_cull<2>(c, a, so);
        const float s[2] = {so[0][0], so[1][0]};
        visible_pair(s, x0, x1, o0, o1);
    }
    /* scene values s times the visibility of the two points' segments; a point whose scene value is
     * 0 skips the boxes (its result is 0 either way, as operator() gives) */
    VCU_HD void visible_pair(const float* s, const float* x0, const float* x1, float* o0, float* o1) const {
        const float* xs[2] = {x0, x1};
        float o[2][3], inv[2][3];
        for (int p = 0; p < 2; ++p) {
            const float e[3] = {xs[p][2], xs[p][3], vfma(0.75f, xs[p][4], 0.25f)};
            o[p][0] = xs[p][0];
            o[p][1] = xs[p][1];
            o[p][2] = 0.0f;
            for (int k = 0; k < 3; ++k) inv[p][k] = vdiv(1.0f, vsub(e[k], o[p][k]));
        }
        bool blocked0 = s[0] == 0.0f, blocked1 = s[1] == 0.0f;
        for (int i = 0; i < nb && !(blocked0 && blocked1); ++i) {
            float t00 = 0.0f, t01 = 1.0f, t10 = 0.0f, t11 = 1.0f;
            for (int k = 0; k < 3; ++k) {
                float ta = vmul(vsub(lo[i][k], o[0][k]), inv[0][k]);
                float tb = vmul(vsub(hi[i][k], o[0][k]), inv[0][k]);
                if (ta > tb) { const float w = ta; ta = tb; tb = w; }
                t00 = (ta > t00) ? ta : t00;
                t01 = (tb < t01) ? tb : t01;
                float ua = vmul(vsub(lo[i][k], o[1][k]), inv[1][k]);
                float ub = vmul(vsub(hi[i][k], o[1][k]), inv[1][k]);
                if (ua > ub) { const float w = ua; ua = ub; ub = w; }
                t10 = (ua > t10) ? ua : t10;
                t11 = (ub < t11) ? ub : t11;
            }
            blocked0 = blocked0 || (t00 <= t01);
            blocked1 = blocked1 || (t10 <= t11);
        }
        o0[0] = (s[0] == 0.0f) ? 0.0f : vmul(s[0], blocked0 ? 0.0f : 1.0f);
        o1[0] = (s[1] == 0.0f) ? 0.0f : vmul(s[1], blocked1 ? 0.0f : 1.0f);
    }
};

/* ---------------------------------------------------------------- unbounded dimensions
 * Philox4x32-10 (Salmon et al., SC'11) on host and device alike: the stream of uniforms an
 * integrand of unbounded dimension draws after its first coordinates. */
VCU_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}
VCU_HD void philox_round(uint32_t* c, uint32_t k0, uint32_t k1) {
    const uint32_t h0 = mulhi32(0xD2511F53u, c[0]), l0 = 0xD2511F53u * c[0];
    const uint32_t h1 = mulhi32(0xCD9E8D57u, c[2]), l1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = h1 ^ c[1] ^ k0, n2 = h0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = l1;
    c[2] = n2;
    c[3] = l0;
}
VCU_HD void philox10(uint32_t* c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        philox_round(c, k0, k1);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

/* A random walk over the 2-D scene, an integrand of unbounded dimension (viltrum's
 * range_infinite / random_sequence integrands, src/range-infinite.h, src/monte-carlo/random-
 * sequence-*.h): coordinates 0-1 start the walk at (x, y) with the scene's value there; then each
 * bounce draws three more -- it continues with probability `keep` (weight *= albedo / keep), turns
 * by 2 pi u and moves u * step on the torus [0,1)^2, adding the weighted scene value -- for at most
 * `max_bounces` bounces.  walk() takes the coordinates from any source (a reference random
 * sequence, a device stream); operator() draws them from a Philox stream keyed by the point, so the
 * library's 2-D integrators see a function of (x, y). */
struct Walk2 {
    static constexpr int DIM = 2, CH = 1;
    static constexpr bool kUnbounded = true;
    Scene2 scene;
    float albedo, keep, step;
    int32_t max_bounces;
    uint32_t k0, k1; /* key of the coordinates after the first two */

    /* params: albedo, keep, step, max_bounces, key, then the scene's parameters */
    int build(const float* p, int n) {
        if (n < 5) return 1;
        albedo = p[0];
        keep = p[1];
        step = p[2];
        max_bounces = (int32_t)p[3];
        if (!(keep > 0.0f && keep <= 1.0f) || max_bounces < 0 || max_bounces > 4096) return 1;
        k0 = (uint32_t)p[4];
        k1 = 0x5EED0000u;
        return scene.build(p + 5, n - 5);
    }
    template <class Next> VCU_HD float walk(float x, float y, Next&& next) const {
        float v = scene.eval(x, y);
        float w = 1.0f;
        const float gain = vdiv(albedo, keep);
        for (int k = 0; k < max_bounces; ++k) {
            if (!(next() < keep)) break;
            w = vmul(w, gain);
            const float ang = vmul(next(), 6.2831854820251465f);
            const float len = vmul(next(), step);
            x = vfma(len, vcos(ang), x);
            y = vfma(len, vsin(ang), y);
            x = vsub(x, floorf(x));
            y = vsub(y, floorf(y));
            v = vfma(w, scene.eval(x, y), v);
        }
        return v;
    }
    /* the walk from (x, y) whose further coordinates are stream `idx` of the point */
    VCU_HD float sample(float x, float y, uint32_t idx) const {
        uint32_t c[4], blk = 0;
        int used = 4;
        auto next = [&]() {
            if (used == 4) {
                c[0] = float_to_bits(x);
                c[1] = float_to_bits(y);
                c[2] = idx;
                c[3] = blk++;
                philox10(c, k0, k1);
                used = 0;
            }
            return (float)(c[used++] >> 8) * 5.9604644775390625e-08f;
        };
        return walk(x, y, next);
    }
    VCU_HD void operator()(const float* x, float* out) const { out[0] = sample(x[0], x[1], 0u); }
};

}  // namespace vcu
