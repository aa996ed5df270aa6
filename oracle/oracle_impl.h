/*
 * oracle_impl.h -- the templates of the CPU restatement of viltrum's per-bin integration path
 * (see oracle.cc for what each part restates).  TEST INFRASTRUCTURE ONLY: included by oracle.cc
 * (liboracle.so) and by test programs that check the device path on integrands of their own.
 */
#pragma once
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <random>
#include <thread>
#include <tuple>
#include <vector>

#include "../include/vcu_integrands.h"
#include "vrgb.h"

namespace orc {

constexpr int ipow(int b, int e) { return e <= 0 ? 1 : b * ipow(b, e - 1); }

/* ------------------------------------------------------------------ value helpers */
template <class T> struct VT;
template <> struct VT<float> {
    static constexpr int CH = 1;
    static float from(const float* o) { return o[0]; }
    static void to(const float& v, float* o) { o[0] = v; }
};
template <> struct VT<vrgb> {
    static constexpr int CH = 3;
    static vrgb from(const float* o) { return vrgb(o[0], o[1], o[2]); }
    static void to(const vrgb& v, float* o) { o[0] = v.c[0]; o[1] = v.c[1]; o[2] = v.c[2]; }
};

/* ------------------------------------------------------------------ Range<float,DIM> */
template <int DIM> struct Range {
    std::array<float, DIM> a, b;
    float vol;
    Range() = default;
    Range(const std::array<float, DIM>& a_, const std::array<float, DIM>& b_) : a(a_), b(b_) {
        vol = 1.0f;
        for (int i = 0; i < DIM; ++i) vol *= (b[i] - a[i]);
    }
    float min(int i) const { return a[i]; }
    float max(int i) const { return b[i]; }
    float volume() const { return vol; }
    Range subrange_dimension(int d, float lo, float hi) const {
        auto na = a, nb = b;
        na[d] = lo;
        nb[d] = hi;
        return Range(na, nb);
    }
    bool empty() const {
        for (int i = 0; i < DIM; ++i)
            if (a[i] >= b[i]) return true;
        return false;
    }
    Range intersection(const Range& o) const {
        std::array<float, DIM> na, nb;
        for (int d = 0; d < DIM; ++d) {
            na[d] = std::max(a[d], o.a[d]);
            nb[d] = std::max(na[d], std::min(b[d], o.b[d]));
        }
        return Range(na, nb);
    }
    std::array<float, DIM> pos_in_range(const std::array<float, DIM>& p) const {
        std::array<float, DIM> r;
        for (int i = 0; i < DIM; ++i) {
            if (a[i] >= b[i]) r[i] = a[i];
            else r[i] = (p[i] - a[i]) / (b[i] - a[i]);
        }
        return r;
    }
};

/* ------------------------------------------------------------------ rules */
struct Trapezoidal {
    static constexpr int S = 2;
    template <class T> T rule(const T* p) const { return (p[0] + p[1]) / 2.0; }
    template <class T> void coefficients(const T* p, T* c) const {
        c[0] = p[0];
        c[1] = p[1] - p[0];
    }
    template <class T> T at(float t, const T* p) const {
        T c[2];
        coefficients(p, c);
        return c[1] * t + c[0];
    }
    template <class T> T subrange(float a, float b, const T* p) const {
        T c[2];
        coefficients(p, c);
        return (c[1] * b / 2.0 + c[0]) * b - (c[1] * a / 2.0 + c[0]) * a;
    }
};
struct Simpson {
    static constexpr int S = 3;
    template <class T> T rule(const T* p) const { return (p[0] + 4.0 * p[1] + p[2]) / 6.0; }
    template <class T> void coefficients(const T* p, T* c) const {
        c[0] = p[0];
        c[1] = -3 * p[0] + 4 * p[1] - p[2];
        c[2] = 2 * p[0] - 4 * p[1] + 2 * p[2];
    }
    template <class T> T at(float t, const T* p) const {
        T c[3];
        coefficients(p, c);
        return (c[2] * t + c[1]) * t + c[0];
    }
    template <class T> T subrange(float a, float b, const T* p) const {
        T c[3];
        coefficients(p, c);
        return ((c[2] * b / 3.0 + c[1] / 2.0) * b + c[0]) * b -
               ((c[2] * a / 3.0 + c[1] / 2.0) * a + c[0]) * a;
    }
};
struct Boole {
    static constexpr int S = 5;
    template <class T> T rule(const T* p) const {
        return (7.0 * p[0] + 32.0 * p[1] + 12.0 * p[2] + 32.0 * p[3] + 7.0 * p[4]) / 90.0;
    }
    template <class T> void coefficients(const T* p, T* c) const {
        c[0] = p[0];
        c[1] = -25 * p[0] / 3 + 16 * p[1] - 12 * p[2] + 16 * p[3] / 3 - p[4];
        c[2] = 70 * p[0] / 3 - 208 * p[1] / 3 + 76 * p[2] - 112 * p[3] / 3 + 22 * p[4] / 3;
        c[3] = -80 * p[0] / 3 + 96 * p[1] - 128 * p[2] + 224 * p[3] / 3 - 16 * p[4];
        c[4] = 32 * p[0] / 3 - 128 * p[1] / 3 + 64 * p[2] - 128 * p[3] / 3 + 32 * p[4] / 3;
    }
    template <class T> T at(float t, const T* p) const {
        T c[5];
        coefficients(p, c);
        return (((c[4] * t + c[3]) * t + c[2]) * t + c[1]) * t + c[0];
    }
    template <class T> T subrange(float a, float b, const T* p) const {
        T c[5];
        coefficients(p, c);
        return ((((c[4] * b / 5.0 + c[3] / 4.0) * b + c[2] / 3.0) * b + c[1] / 2.0) * b + c[0]) * b -
               ((((c[4] * a / 5.0 + c[3] / 4.0) * a + c[2] / 3.0) * a + c[1] / 2.0) * a + c[0]) * a;
    }
};

/* ------------------------------------------------------------------ metrics */
struct MetricAbs {
    float operator()(float a, float b) const { return std::abs(b - a); }
    float operator()(const vrgb& a, const vrgb& b) const {
        float s = (*this)(a.c[0], b.c[0]);
        s += (*this)(a.c[1], b.c[1]);
        s += (*this)(a.c[2], b.c[2]);
        return s;
    }
};
struct MetricRel {
    double min_val;
    float operator()(float a, float b) const {
        if (std::max(std::abs(a), std::abs(b)) < min_val) return std::abs(b - a);
        else return std::abs(b - a) / std::max(std::abs(a), std::abs(b));
    }
    float operator()(const vrgb& a, const vrgb& b) const {
        float s = (*this)(a.c[0], b.c[0]);
        s += (*this)(a.c[1], b.c[1]);
        s += (*this)(a.c[2], b.c[2]);
        return s;
    }
};
inline float norm_default(float v) { return std::abs(v); }
inline float norm_default(const vrgb& v) {
    float s = std::abs(v.c[0]);
    s += std::abs(v.c[1]);
    s += std::abs(v.c[2]);
    return s;
}

/* ------------------------------------------------------------------ Simpson's pdf (rules.h:102-248)
 * The polynomial importance sampling of the control variate: the parabola through the norms of the
 * three node values, lifted so its minimum on [0,1] is 0 (pdf_points), its integral, value, cdf and
 * an inverse cdf by the closed-form roots of the cubic (Cardano / Viete), in the reference's mix of
 * float and double arithmetic. */
struct SimpsonPdf {
    template <class T> static std::array<float, 3> points(const T* p) {
        std::array<float, 3> q;
        for (int i = 0; i < 3; ++i) q[i] = norm_default(p[i]);
        float cs[3];
        Simpson().coefficients(q.data(), cs);
        float ymin = 0;
        if (cs[2] > 0) {
            const float tmin = -cs[1] / (2.0 * cs[2]);
            if ((tmin > 0) && (tmin < 1)) {
                const float ytmin = (cs[2] * tmin + cs[1]) * tmin + cs[0];
                if (ytmin < ymin) ymin = ytmin;
            }
        }
        for (int i = 0; i < 3; ++i) q[i] -= ymin;
        return q;
    }
    static float integral(float t0, float t1, const std::array<float, 3>& ps) { return Simpson().subrange(t0, t1, ps.data()); }
    static float at(float t, const std::array<float, 3>& ps) { return Simpson().at(t, ps.data()); }
    static float cdf(float t, const std::array<float, 3>& ps) {
        float c[3];
        Simpson().coefficients(ps.data(), c);
        return ((c[2] * t / 3.0 + c[1] / 2.0) * t + c[0]) * t;
    }
    static double cuberoot(double x) { return (x < 0) ? (-1 * std::pow(-x, 1. / 3.)) : std::pow(x, 1. / 3.); }
    static std::vector<float> inv_cdf(float x, const std::array<float, 3>& pts) {
        std::vector<float> sol;
        float co[3];
        Simpson().coefficients(pts.data(), co);
        double a = co[2] / 3.;
        double b = co[1] / 2.;
        float c = co[0];
        float d = -x;
        const double sum = a + b + c + d;
        a /= sum;
        b /= sum;
        c /= sum;
        d /= sum;
        if (std::abs(a) < 1.e-3) {
            if (std::abs(b) < 1.e-3) {
                if (std::abs(c) >= 1.e-3) sol.push_back(-d / c);
            } else {
                const double disc = c * c - 4 * b * d;
                if (disc >= 0) {
                    sol.push_back((-c + std::sqrt(disc)) / (2 * b));
                    sol.push_back((-c - std::sqrt(disc)) / (2 * b));
                }
            }
        } else {
            const double p = c / a - std::pow(b, 2.) / (3. * std::pow(a, 2.));
            const double q = 2 * std::pow(b, 3.) / (27. * std::pow(a, 3.)) - b * c / (3. * std::pow(a, 2.)) + d / a;
            const double sqr = std::pow(q / 2., 2.) + std::pow(p / 3., 3.);
            if (sqr >= 0.) {
                sol.push_back(cuberoot(-q / 2. - std::sqrt(sqr)) + cuberoot(-q / 2. + std::sqrt(sqr)) - b / (3 * a));
            } else {
                for (int i = 0; i < 3; i++)
                    sol.push_back(2. * std::sqrt(-p / 3.) *
                                      std::cos(1. / 3. * std::acos(3. * q / (2. * p) * std::sqrt(-3. / p)) - 2. * M_PI * i / 3.) -
                                  b / (3. * a));
            }
        }
        return sol;
    }
    /* a point of [t0,t1] with density proportional to the lifted parabola; uniform when no root fits */
    template <class T> static float sample(float s, float t0, float t1, const T* p) {
        const auto ps = points(p);
        const float x = s * cdf(t1, ps) + (float(1) - s) * cdf(t0, ps);
        for (float r : inv_cdf(x, ps)) {
            if ((r < t0) && (std::abs(t0 - r) < 1.e-5)) r = t0;
            if ((r > t1) && (std::abs(r - t1) < 1.e-5)) r = t1;
            if ((r >= t0) && (r <= t1) && (!std::isnan(r))) return r;
        }
        return s * (t1 - t0) + t0;
    }
};

/* ------------------------------------------------------------------ nd folds */
template <int S, class U, class T, class Fn>
std::vector<U> fold(const std::vector<T>& in, int k, int d, const Fn& fn) {
    const int outn = ipow(S, k - 1);
    std::vector<U> out(outn);
    const int stride = ipow(S, d);
    for (int J = 0; J < outn; ++J) {
        int rem = J, base = 0;
        for (int e = 0; e < k; ++e) {
            if (e == d) continue;
            base += (rem % S) * ipow(S, e);
            rem /= S;
        }
        T line[S];
        for (int i = 0; i < S; ++i) line[i] = in[base + i * stride];
        out[J] = fn(line);
    }
    return out;
}
template <int S, class T, class Fn> T fold_all(std::vector<T> v, int k, const Fn& fn) {
    while (k > 0) {
        v = fold<S, T>(v, k, 0, fn);
        --k;
    }
    return v[0];
}

/* ------------------------------------------------------------------ region */
template <class H, class L, int DIM, class T> struct Region {
    static constexpr int S = H::S;
    static constexpr int N = ipow(S, DIM);
    static constexpr int DIMS = DIM;
    Range<DIM> range;
    std::vector<T> data;
    float err = 0.0f;
    int err_dim = 0;

    template <class F> T eval_mapped(const F& f, const std::array<double, DIM>& p) const {
        std::array<float, DIM> x;
        for (int i = 0; i < DIM; ++i) x[i] = p[i] * (range.max(i) - range.min(i)) + range.min(i);
        return f(x);
    }
    template <class F> void fill(const F& f) {
        data.resize(N);
        for (int idx = 0; idx < N; ++idx) {
            std::array<double, DIM> p;
            int rem = idx;
            for (int d = 0; d < DIM; ++d) {
                p[d] = double(rem % S) / double(S - 1);
                rem /= S;
            }
            data[idx] = eval_mapped(f, p);
        }
    }
    /* split into two children along dim (region.h:345-359, split.h:13-49) */
    template <class F> void split(const F& f, int dim, Region& c0, Region& c1) const {
        const int full = 2 * (S - 1) + 1;
        c0.data.assign(N, T());
        c1.data.assign(N, T());
        Region* ch[2] = {&c0, &c1};
        const int sd = ipow(S, dim);
        for (int i = 0; i < full; ++i) {
            int part = i / (S - 1);
            int position = i - part * (S - 1);
            const double v = double(i) / double(full - 1);
            if (part >= 2) {
                --part;
                position += (S - 1);
            }
            for (int J = 0; J < ipow(S, DIM - 1); ++J) {
                /* slice index J over the other dims (dim-0 fastest) */
                int rem = J, base = 0;
                std::array<double, DIM> p;
                for (int e = 0; e < DIM; ++e) {
                    if (e == dim) continue;
                    const int ie = rem % S;
                    rem /= S;
                    base += ie * ipow(S, e);
                    p[e] = double(ie) / double(S - 1);
                }
                p[dim] = v;
                T val;
                if ((i % 2) == 0) val = data[base + (i / 2) * sd];
                else val = eval_mapped(f, p);
                ch[part]->data[base + position * sd] = val;
                if (position == 0 && part > 0) c0.data[base + (S - 1) * sd] = val;
            }
        }
        std::array<float, DIM> mn = range.a, mx = range.b;
        const float d = (range.max(dim) - range.min(dim)) / (float(2));
        mx[dim] = range.min(dim) + d * 1;
        c0.range = Range<DIM>(mn, mx);
        mn[dim] = mx[dim];
        mx[dim] = range.max(dim);
        c1.range = Range<DIM>(mn, mx);
    }
    template <class M> float error(int dim, const M& metric) const {
        H h;
        L l;
        auto line_err = [&](const T* v) -> float {
            T plow[L::S];
            for (int i = 0; i < L::S; ++i) plow[i] = v[i * (H::S - 1) / (L::S - 1)];
            return metric(h.rule(v), l.rule(plow));
        };
        std::vector<float> e = fold<S, float>(data, DIM, dim, line_err);
        const float folded = fold_all<S>(e, DIM - 1, [&](const float* v) -> float { return h.rule(v); });
        return range.volume() * folded;
    }
    /* the whole region's error estimate, volume * (fold_all(H) - fold_all(low)) (region.h:422-426,
     * nested.h:17-24) */
    T error_total() const {
        H h;
        L l;
        const T hi = fold_all<S>(data, DIM, [&](const T* v) -> T { return h.rule(v); });
        const T lo = fold_all<S>(data, DIM, [&](const T* v) -> T {
            T plow[L::S];
            for (int i = 0; i < L::S; ++i) plow[i] = v[i * (H::S - 1) / (L::S - 1)];
            return l.rule(plow);
        });
        return range.volume() * (hi - lo);
    }
    /* integral over [a,b] (absolute coordinates), region.h:141-169 */
    T integral_subrange(const Range<DIM>& r) const {
        H h;
        const auto a = range.pos_in_range(r.a);
        const auto b = range.pos_in_range(r.b);
        std::vector<T> v = data;
        int k = DIM;
        while (k > 1) {
            const int d = k - 1;
            v = fold<S, T>(v, k, d, [&](const T* line) -> T { return h.subrange(a[d], b[d], line); });
            --k;
        }
        v = fold<S, T>(v, 1, 0, [&](const T* line) -> T { return h.subrange(a[0], b[0], line); });
        return range.volume() * v[0];
    }
    /* polynomial value at an absolute position, region.h:86-112 */
    T approximation_at(const std::array<float, DIM>& pos) const {
        H h;
        const auto p = range.pos_in_range(pos);
        std::vector<T> v = data;
        for (int k = DIM, d = 0; k >= 1; --k, ++d)
            v = fold<S, T>(v, k, 0, [&](const T* line) -> T { return h.at(p[d], line); });
        return v[0] * 1.0f;
    }
    /* Simpson regions only: the pdf integral over [a,b] folding from the last dimension
     * (region.h:267-290), the unnormalised pdf at a point (:296-311), the normalised pdf (:326-331) */
    template <class Line> float pdf_fold(const float* a, const float* b, const Line& line_fn) const {
        std::vector<float> v = fold<S, float>(data, DIM, DIM - 1, [&](const T* l) { return line_fn(DIM - 1, l); });
        for (int k = DIM - 1; k >= 1; --k)
            v = fold<S, float>(v, k, k - 1, [&](const float* l) { return line_fn(k - 1, l); });
        (void)a;
        (void)b;
        return v[0];
    }
    float pdf_integral_subrange(const Range<DIM>& r) const {
        const auto a = range.pos_in_range(r.a);
        const auto b = range.pos_in_range(r.b);
        return range.volume() * pdf_fold(a.data(), b.data(), [&](int d, const auto* l) {
                   return SimpsonPdf::integral(a[d], b[d], SimpsonPdf::points(l));
               });
    }
    float pdf_subrange(const std::array<float, DIM>& pos, const Range<DIM>& r) const {
        const auto p = range.pos_in_range(pos);
        const auto a = range.pos_in_range(r.a);
        const auto b = range.pos_in_range(r.b);
        const float at = pdf_fold(a.data(), b.data(), [&](int d, const auto* l) {
            return SimpsonPdf::at(p[d], SimpsonPdf::points(l));
        });
        return at / pdf_integral_subrange(r);
    }
    /* a point of bin n region drawn from the pdf: the marginal of the first remaining dimension (the
     * others integrated over [a,b], last first), sampled; then the pdf conditioned on it and the
     * next dimension (region.h:220-257) */
    template <class U>
    void sample_rec(const std::vector<U>& ma, int k, int off, const float* s, const float* a, const float* b,
                    float* sol) const {
        if (k == 1) {
            sol[off] = SimpsonPdf::sample(s[off], a[off], b[off], ma.data());
            return;
        }
        std::vector<float> m = fold<S, float>(ma, k, k - 1, [&](const U* l) {
            return SimpsonPdf::integral(a[off + k - 1], b[off + k - 1], SimpsonPdf::points(l));
        });
        for (int j = k - 1; j >= 2; --j)
            m = fold<S, float>(m, j, j - 1, [&](const float* l) {
                return SimpsonPdf::integral(a[off + j - 1], b[off + j - 1], SimpsonPdf::points(l));
            });
        sol[off] = SimpsonPdf::sample(s[off], a[off], b[off], m.data());
        const float t = sol[off];
        std::vector<float> c = fold<S, float>(ma, k, 0, [&](const U* l) { return SimpsonPdf::at(t, SimpsonPdf::points(l)); });
        sample_rec<float>(c, k - 1, off + 1, s, a, b, sol);
    }
    std::array<float, DIM> sample_subrange(const std::array<float, DIM>& s, const Range<DIM>& r) const {
        const auto a = range.pos_in_range(r.a);
        const auto b = range.pos_in_range(r.b);
        std::array<float, DIM> sol;
        sample_rec<T>(data, DIM, 0, s.data(), a.data(), b.data(), sol.data());
        std::array<float, DIM> x;
        for (int i = 0; i < DIM; ++i) x[i] = sol[i] * (range.max(i) - range.min(i)) + range.min(i);
        return x;
    }
};

/* heuristics (error-heuristic.h:10-47); returns (error, dim) */
template <class R, class M> std::tuple<float, int> heuristic(const R& r, const orc_nested& nc, const M& metric) {
    constexpr int DIM = R::DIMS;
    if (nc.heuristic == ORC_HEUR_DEFAULT) {
        float max_err = 0;
        int max_dim = 0;
        for (int d = 0; d < DIM; ++d) {
            const float err = r.error(d, metric);
            if (err > max_err) {
                max_err = err;
                max_dim = d;
            }
        }
        return std::tuple<float, int>(max_err, max_dim);
    }
    float max_err = r.error(0, metric);
    if ((r.range.max(0) - r.range.min(0)) < nc.min_size || std::isnan(r.range.max(0) - r.range.min(0)))
        max_err = 0;
    else max_err += nc.size_weight * std::abs(r.range.max(0) - r.range.min(0));
    int max_dim = 0;
    float err = max_err;
    for (int d = 1; d < DIM; ++d) {
        err = r.error(d, metric) + nc.size_weight * std::abs(r.range.max(d) - r.range.min(d));
        if ((r.range.max(d) - r.range.min(d)) < nc.min_size) err = 0;
        if (err >= max_err) {
            max_err = err;
            max_dim = d;
        }
    }
    return std::tuple<float, int>(max_err, max_dim);
}

/* adaptive heap generator (regions-generator-adaptive-heap.h:18-45) */
template <class H, class L, int DIM, class T, class F, class M>
std::vector<Region<H, L, DIM, T>> generate(const F& f, const Range<DIM>& range, uint64_t iterations,
                                           const orc_nested& nc, const M& metric, int32_t* trace) {
    using R = Region<H, L, DIM, T>;
    auto ordering = [](const R& a, const R& b) { return a.err < b.err; };
    R root;
    root.range = range;
    root.fill(f);
    std::tie(root.err, root.err_dim) = heuristic(root, nc, metric);
    std::vector<R> heap;
    heap.reserve(iterations + 1);
    heap.push_back(root);
    for (uint64_t i = 0; i < iterations; ++i) {
        R top = heap.front();
        R c[2];
        top.split(f, top.err_dim, c[0], c[1]);
        if (trace) {
            trace[2 * i] = top.err_dim;
            std::memcpy(&trace[2 * i + 1], &top.err, 4);
        }
        std::pop_heap(heap.begin(), heap.end(), ordering);
        heap.pop_back();
        for (int k = 0; k < 2; ++k) {
            std::tie(c[k].err, c[k].err_dim) = heuristic(c[k], nc, metric);
            heap.push_back(c[k]);
            std::push_heap(heap.begin(), heap.end(), ordering);
        }
    }
    return heap;
}

/* ------------------------------------------------------------------ integrand adaptor */
template <class Fun, int DIM, class T> struct Fn {
    const Fun* f;
    T operator()(const std::array<float, DIM>& x) const {
        float o[3];
        (*f)(x.data(), o);
        return VT<T>::from(o);
    }
};
template <class Fun, int DIM, class T> struct RecFn {
    const Fun* f;
    mutable float* rec;
    T operator()(const std::array<float, DIM>& x) const {
        if (rec) {
            for (int i = 0; i < DIM; ++i) *rec++ = x[i];
        }
        float o[3];
        (*f)(x.data(), o);
        return VT<T>::from(o);
    }
};

struct Problem {
    int dim, dimbins;
    const float *rmin, *rmax;
    const uint64_t* res;
    uint64_t nbins() const {
        uint64_t n = 1;
        for (int i = 0; i < dimbins; ++i) n *= res[i];
        return n;
    }
};

template <int DIM> Range<DIM> make_range(const Problem& p) {
    std::array<float, DIM> a, b;
    for (int i = 0; i < DIM; ++i) {
        a[i] = p.rmin[i];
        b[i] = p.rmax[i];
    }
    return Range<DIM>(a, b);
}
/* bin position (dim-0 fastest) */
inline void bin_pos(const Problem& p, uint64_t bin, std::array<uint64_t, 8>& pos) {
    for (int i = 0; i < p.dimbins; ++i) {
        pos[i] = bin % p.res[i];
        bin /= p.res[i];
    }
}
template <int DIM> Range<DIM> bin_subrange(const Problem& p, const Range<DIM>& range, const std::array<uint64_t, 8>& pos) {
    std::array<float, DIM> drange;
    for (int i = 0; i < p.dimbins; ++i) drange[i] = (range.max(i) - range.min(i)) / ((float)(p.res[i]));
    Range<DIM> sub = range;
    for (int i = 0; i < p.dimbins; ++i)
        sub = sub.subrange_dimension(i, range.min(i) + pos[i] * drange[i], range.min(i) + (pos[i] + 1) * drange[i]);
    return sub;
}

/* ------------------------------------------------------------------ per-bin Monte Carlo */
template <int DIM, class T, class Fun>
void per_bin_mc(const Fun& fun, const Problem& p, uint64_t spp, uint64_t seed, int flavour, float* out, float* points) {
    const auto range = make_range<DIM>(p);
    const uint64_t nb = p.nbins();
    uint64_t factor = 1;
    for (int i = 0; i < p.dimbins; ++i) factor *= p.res[i];
    RecFn<Fun, DIM, T> f{&fun, points};
    if (flavour == ORC_MC_PER_BIN_PARALLEL) {
        /* monte_carlo(spp, seed) is copied into the per-bin wrapper (copy ctor reseeds), then
         * copied once per bin in bin order (each copy reseeds from the prototype). */
        std::mt19937 first(seed);
        std::mt19937 proto(static_cast<std::size_t>(first()));
        std::vector<std::size_t> seeds(nb);
        for (uint64_t b = 0; b < nb; ++b) seeds[b] = std::size_t(proto());
        std::array<uint64_t, 8> pos;
        for (uint64_t b = 0; b < nb; ++b) {
            bin_pos(p, b, pos);
            const auto sub = bin_subrange<DIM>(p, range, pos);
            std::mt19937 rng(seeds[b]);
            T sol(0.0);
            const double fac = 1.0 * sub.volume() / double(spp);
            for (uint64_t s = 0; s < spp; ++s) {
                std::array<float, DIM> x;
                for (int i = 0; i < DIM; ++i) {
                    std::uniform_real_distribution<float> dis(sub.min(i), sub.max(i));
                    x[i] = dis(rng);
                }
                bool inside = true;
                for (int i = 0; (i < DIM) && inside; ++i) inside = (x[i] >= sub.min(i)) && (x[i] <= sub.max(i));
                if (inside) sol += f(x) * fac;
            }
            const T v = double(factor) * sol;
            VT<T>::to(v, out + b * VT<T>::CH);
        }
    } else {
        std::mt19937 rng(seed);
        const double fac = range.volume() / double(spp);
        std::vector<unsigned> seeds(nb);
        for (uint64_t b = 0; b < nb; ++b) seeds[b] = unsigned(rng());
        std::array<uint64_t, 8> pos;
        for (uint64_t b = 0; b < nb; ++b) {
            bin_pos(p, b, pos);
            const auto sub = bin_subrange<DIM>(p, range, pos);
            std::mt19937 local(seeds[b]);
            T acc = VT<T>::from(out + b * VT<T>::CH);
            for (uint64_t s = 0; s < spp; ++s) {
                std::array<float, DIM> x;
                for (int i = 0; i < DIM; ++i) {
                    std::uniform_real_distribution<float> dis(sub.min(i), sub.max(i));
                    x[i] = dis(local);
                }
                acc += f(x) * fac;
            }
            VT<T>::to(acc, out + b * VT<T>::CH);
        }
    }
}

/* ------------------------------------------------------------------ per-bin adaptive nested */
template <class H, class L, int DIM, class T, class Fun, class M>
void per_bin_nested_range(const Fun& fun, const Problem& p, const orc_nested& nc, const M& metric, uint64_t iters,
                          uint64_t b0, uint64_t b1, float* out, int32_t* trace) {
    const auto range = make_range<DIM>(p);
    uint64_t factor = 1;
    for (int i = 0; i < p.dimbins; ++i) factor *= p.res[i];
    Fn<Fun, DIM, T> f{&fun};
    std::array<uint64_t, 8> pos;
    for (uint64_t b = b0; b < b1; ++b) {
        bin_pos(p, b, pos);
        const auto sub = bin_subrange<DIM>(p, range, pos);
        auto regions = generate<H, L, DIM, T>(f, sub, iters, nc, metric, trace ? trace + 2 * iters * b : nullptr);
        /* RegionsIntegratorSequential with a single bin (resolution {1}) */
        T sol(0.0);
        const float drange0 = (sub.max(0) - sub.min(0)) / float(1);
        const Range<DIM> binrange = sub.subrange_dimension(0, sub.min(0) + 0 * drange0, sub.min(0) + 1 * drange0);
        for (const auto& r : regions) {
            const Range<DIM> rb = binrange.intersection(r.range);
            if (!rb.empty()) sol += double(1) * r.integral_subrange(rb);
        }
        const T v = double(factor) * sol;
        VT<T>::to(v, out + b * VT<T>::CH);
    }
}

/* ------------------------------------------------------------------ global adaptive into bins */
template <class H, class L, int DIM, class T, class Fun, class M>
void adaptive_global(const Fun& fun, const Problem& p, const orc_nested& nc, const M& metric, uint64_t iters,
                     float* out) {
    using R = Region<H, L, DIM, T>;
    const auto range = make_range<DIM>(p);
    Fn<Fun, DIM, T> f{&fun};
    const std::vector<R> regions = generate<H, L, DIM, T>(f, range, iters, nc, metric, nullptr);
    uint64_t factor = 1;
    for (int i = 0; i < p.dimbins; ++i) factor *= p.res[i];
    std::array<float, DIM> drange;
    for (int i = 0; i < p.dimbins; ++i) drange[i] = (range.max(i) - range.min(i)) / float(p.res[i]);
    for (const auto& r : regions) {
        /* pixels_in_region (region.h:454-463) */
        std::array<uint64_t, 8> st, en;
        for (int i = 0; i < p.dimbins; ++i) {
            st[i] = std::max(std::size_t(0),
                             std::size_t(float(p.res[i]) * (r.range.min(i) - range.min(i)) / (range.max(i) - range.min(i))));
            en[i] = std::max(std::size_t(st[i] + 1),
                             std::min(std::size_t(p.res[i]),
                                      std::size_t(0.99f + (float(p.res[i]) * (r.range.max(i) - range.min(i)) /
                                                           (range.max(i) - range.min(i))))));
        }
        std::array<uint64_t, 8> q = st;
        for (;;) {
            Range<DIM> binrange = range;
            uint64_t lin = 0, mul = 1;
            for (int i = 0; i < p.dimbins; ++i) {
                binrange = binrange.subrange_dimension(i, range.min(i) + q[i] * drange[i], range.min(i) + (q[i] + 1) * drange[i]);
                lin += q[i] * mul;
                mul *= p.res[i];
            }
            const Range<DIM> rb = binrange.intersection(r.range);
            if (!rb.empty()) {
                T v = VT<T>::from(out + lin * VT<T>::CH);
                v += double(factor) * r.integral_subrange(rb);
                VT<T>::to(v, out + lin * VT<T>::CH);
            }
            int i = 0;
            for (; i < p.dimbins; ++i) {
                if (++q[i] < en[i]) break;
                q[i] = st[i];
            }
            if (i == p.dimbins) break;
        }
    }
}

/* ------------------------------------------------------------------ tolerance-driven adaptive */
/* integrator_adaptive_tolerance (src/nested/integrator-adaptive-tolerance.h:9-56): depth first, a
 * region whose heuristic error is below the tolerance is integrated into the bins it overlaps, any
 * other is split along the heuristic's dimension and its two halves visited in order.  Returns the
 * number of leaves, or -1 when max_regions regions were built before the recursion closed. */
template <class H, class L, int DIM, class T, class Fun, class M>
int64_t adaptive_tolerance(const Fun& fun, const Problem& p, const orc_nested& nc, const M& metric, float tol,
                           uint64_t max_regions, float* out) {
    using R = Region<H, L, DIM, T>;
    const auto range = make_range<DIM>(p);
    Fn<Fun, DIM, T> f{&fun};
    uint64_t factor = 1;
    for (int i = 0; i < p.dimbins; ++i) factor *= p.res[i];
    std::array<float, DIM> drange;
    for (int i = 0; i < p.dimbins; ++i) drange[i] = (range.max(i) - range.min(i)) / float(p.res[i]);
    auto add_region = [&](const R& r) {
        std::array<uint64_t, 8> st, en;
        for (int i = 0; i < p.dimbins; ++i) {
            st[i] = std::max(std::size_t(0),
                             std::size_t(float(p.res[i]) * (r.range.min(i) - range.min(i)) / (range.max(i) - range.min(i))));
            en[i] = std::max(std::size_t(st[i] + 1),
                             std::min(std::size_t(p.res[i]),
                                      std::size_t(0.99f + (float(p.res[i]) * (r.range.max(i) - range.min(i)) /
                                                           (range.max(i) - range.min(i))))));
        }
        std::array<uint64_t, 8> q = st;
        for (;;) {
            Range<DIM> binrange = range;
            uint64_t lin = 0, mul = 1;
            for (int i = 0; i < p.dimbins; ++i) {
                binrange = binrange.subrange_dimension(i, range.min(i) + q[i] * drange[i], range.min(i) + (q[i] + 1) * drange[i]);
                lin += q[i] * mul;
                mul *= p.res[i];
            }
            const Range<DIM> rb = binrange.intersection(r.range);
            if (!rb.empty()) {
                T v = VT<T>::from(out + lin * VT<T>::CH);
                v += double(factor) * r.integral_subrange(rb);
                VT<T>::to(v, out + lin * VT<T>::CH);
            }
            int i = 0;
            for (; i < p.dimbins; ++i) {
                if (++q[i] < en[i]) break;
                q[i] = st[i];
            }
            if (i == p.dimbins) break;
        }
    };
    uint64_t built = 1;
    int64_t leaves = 0;
    R root;
    root.range = range;
    root.fill(f);
    /* explicit stack in visit order (the reference recurses) */
    std::vector<R> stack;
    stack.push_back(std::move(root));
    while (!stack.empty()) {
        R r = std::move(stack.back());
        stack.pop_back();
        float err;
        int dim;
        std::tie(err, dim) = heuristic(r, nc, metric);
        if (err < tol) {
            add_region(r);
            ++leaves;
        } else {
            if (built + 2 > max_regions) return -1;
            R c[2];
            r.split(f, dim, c[0], c[1]);
            built += 2;
            stack.push_back(std::move(c[1]));
            stack.push_back(std::move(c[0]));
        }
    }
    return leaves;
}

/* ------------------------------------------------------------------ single-value integrals */
/* monte_carlo(budget, seed) through integrate(I, f, range): one bin of resolution {1}, the
 * integrator's own std::mt19937(seed) (moved in, not reseeded), bins(pos) += f(x) * factor */
template <int DIM, class Fun>
float single_mc(const Fun& fun, const Range<DIM>& range, uint64_t budget, uint64_t seed) {
    Fn<Fun, DIM, float> f{&fun};
    std::mt19937 rng(seed);
    const double factor = double(1) * range.volume() / double(budget);
    float sol = 0.0f;
    for (uint64_t s = 0; s < budget; ++s) {
        std::array<float, DIM> x;
        for (int i = 0; i < DIM; ++i) {
            std::uniform_real_distribution<float> dis(range.min(i), range.max(i));
            x[i] = dis(rng);
        }
        bool inside = true;
        for (int i = 0; (i < DIM) && inside; ++i) inside = (x[i] >= range.min(i)) && (x[i] <= range.max(i));
        if (inside) sol += f(x) * factor;
    }
    return sol;
}

/* integrator_adaptive_iterations(nested(H,L), heuristic, iters) through integrate(I, f, range) */
template <class H, class L, int DIM, class Fun, class M>
float single_nested(const Fun& fun, const Range<DIM>& range, const orc_nested& nc, const M& metric, uint64_t iters) {
    Fn<Fun, DIM, float> f{&fun};
    auto regions = generate<H, L, DIM, float>(f, range, iters, nc, metric, nullptr);
    float sol = 0.0f;
    const float drange0 = (range.max(0) - range.min(0)) / float(1);
    const Range<DIM> binrange = range.subrange_dimension(0, range.min(0) + 0 * drange0, range.min(0) + 1 * drange0);
    for (const auto& r : regions) {
        const Range<DIM> rb = binrange.intersection(r.range);
        if (!rb.empty()) sol += double(1) * r.integral_subrange(rb);
    }
    return sol;
}

/* ------------------------------------------------------------------ control variates */
template <class T> struct CvOptimize {
    T sum_f, sum_app;
    std::size_t size = 0;
    double k_f = 0, k_app = 0, e_f = 0, e_ap = 0, e_ap2 = 0, e_fap = 0;
    explicit CvOptimize(const T& ini) : sum_f(ini), sum_app(ini) {}
    void push(const T& fs, const T& as) {
        if (size == 0) {
            k_f = norm_default(fs);
            k_app = norm_default(as);
        }
        e_f += (norm_default(fs) - k_f);
        e_ap += (norm_default(as) - k_app);
        e_ap2 += (norm_default(as) - k_app) * (norm_default(as) - k_app);
        e_fap += (norm_default(fs) - k_f) * (norm_default(as) - k_app);
        sum_f += fs;
        sum_app += as;
        ++size;
    }
    double covariance() const { return (e_fap - (e_f * e_ap) / double(size)) / double(size - 1); }
    double variance() const { return (e_ap2 - (e_ap * e_ap) / double(size)) / double(size - 1); }
    double alpha() const {
        if (size < 2) return 1.0;
        auto v = std::max(0.0, variance());
        if (v <= 0.0) return 1.0;
        auto c = std::min(v, std::max(0.0, covariance()));
        return c / v;
    }
    T integral(const T& approximation) const {
        if (size < 2) return approximation;
        auto a = alpha();
        return (sum_f - a * sum_app) / double(size) + a * approximation;
    }
};
template <class T> struct CvFixed {
    T sum;
    std::size_t size = 0;
    double alpha;
    CvFixed(double a, const T& ini) : sum(ini), alpha(a) {}
    void push(const T& fs, const T& as) {
        sum += fs - alpha * as;
        ++size;
    }
    T integral(const T& approximation) const {
        if (size == 0) return approximation;
        return sum / double(size) + alpha * approximation;
    }
};

template <class H, class L, int DIM, class T, class Fun, class M>
void control_variates(const Fun& fun, const Problem& p, const orc_nested& nc, const M& metric, uint64_t iters,
                      uint64_t spp, uint64_t seed, const orc_cv& cv, float* out, float* approx_out,
                      float* regions_out, float* replay_out) {
    const int weight = cv.weight, rr_mode = cv.rr, sampling = cv.sampling;
    const double alpha = cv.alpha;
    const int width = orc_replay_width(DIM, sampling);
    using R = Region<H, L, DIM, T>;
    const auto range = make_range<DIM>(p);
    Fn<Fun, DIM, T> f{&fun};
    const std::vector<R> regions = generate<H, L, DIM, T>(f, range, iters, nc, metric, nullptr);
    if (regions_out) {
        for (std::size_t k = 0; k < regions.size(); ++k)
            for (int d = 0; d < DIM; ++d) {
                regions_out[k * 2 * DIM + d] = regions[k].range.a[d];
                regions_out[k * 2 * DIM + DIM + d] = regions[k].range.b[d];
            }
    }
    const uint64_t nb = p.nbins();
    uint64_t factor = 1;
    for (int i = 0; i < p.dimbins; ++i) factor *= p.res[i];
    std::array<float, DIM> drange;
    for (int i = 0; i < p.dimbins; ++i) drange[i] = (range.max(i) - range.min(i)) / float(p.res[i]);
    /* stratification: each region appended to the lists of the bins pixels_in_region gives */
    std::vector<std::vector<const R*>> perbin(nb);
    for (const auto& r : regions) {
        std::array<uint64_t, 8> st, en;
        for (int i = 0; i < p.dimbins; ++i) {
            st[i] = std::max(std::size_t(0),
                             std::size_t(float(p.res[i]) * (r.range.min(i) - range.min(i)) / (range.max(i) - range.min(i))));
            en[i] = std::max(std::size_t(st[i] + 1),
                             std::min(std::size_t(p.res[i]),
                                      std::size_t(0.99f + (float(p.res[i]) * (r.range.max(i) - range.min(i)) /
                                                           (range.max(i) - range.min(i))))));
        }
        std::array<uint64_t, 8> q = st;
        for (;;) {
            uint64_t lin = 0, mul = 1;
            for (int i = 0; i < p.dimbins; ++i) {
                lin += q[i] * mul;
                mul *= p.res[i];
            }
            perbin[lin].push_back(&r);
            int i = 0;
            for (; i < p.dimbins; ++i) {
                if (++q[i] < en[i]) break;
                q[i] = st[i];
            }
            if (i == p.dimbins) break;
        }
    }
    std::mt19937 master(seed);
    std::vector<std::mt19937> rngs(nb);
    for (uint64_t b = 0; b < nb; ++b) rngs[b].seed(std::size_t(master()));
    std::array<uint64_t, 8> pos;
    for (uint64_t b = 0; b < nb; ++b) {
        bin_pos(p, b, pos);
        std::mt19937& rng = rngs[b];
        (void)rng(); /* monte_carlo_per_bin(rng,1) built for the Fubini split consumes one draw */
        Range<DIM> binrange = range;
        for (int i = 0; i < p.dimbins; ++i)
            binrange = binrange.subrange_dimension(i, range.min(i) + pos[i] * drange[i], range.min(i) + (pos[i] + 1) * drange[i]);
        const auto& list = perbin[b];
        std::vector<Range<DIM>> rr(list.size());
        T approximation(0);
        for (std::size_t i = 0; i < list.size(); ++i) {
            rr[i] = binrange.intersection(list[i]->range);
            if (!rr[i].empty()) approximation += double(factor) * list[i]->integral_subrange(rr[i]);
        }
        if (approx_out) VT<T>::to(approximation, approx_out + b * VT<T>::CH);
        float* rep = replay_out ? replay_out + b * spp * width : nullptr;
        /* region choice: uniform (region-russian-roulette.h:9-28), or proportional to the norm of
         * the control variate's integral over bin n region (:30-68) or of the region's error scaled
         * by the share of its volume in the bin (:70-108), with a floor of 1% of the mean weight */
        std::uniform_int_distribution<std::size_t> uniform(0, list.size() - 1);
        std::discrete_distribution<std::size_t> weighted;
        if (rr_mode != ORC_RR_UNIFORM) {
            std::vector<double> w(list.size());
            for (std::size_t i = 0; i < list.size(); ++i) {
                if (rr_mode == ORC_RR_INTEGRAL) w[i] = norm_default(list[i]->integral_subrange(rr[i]));
                else if (rr_mode == ORC_RR_ERROR)
                    w[i] = norm_default(list[i]->error_total()) * rr[i].volume() / list[i]->range.volume();
                else if constexpr (R::S == 3) w[i] = list[i]->pdf_integral_subrange(rr[i]); /* rr_pdf_region (:112-149) */
            }
            double sum = 0.0;
            for (double v : w) sum += v;
            if (sum <= 0.0)
                for (double& v : w) v = 1.0;
            else if (rr_mode == ORC_RR_PDF)
                for (double& v : w) v = std::max(v, cv.rr_factor * sum / double(w.size()));
            else
                for (double& v : w) v = std::max(v, 0.01 * sum / double(w.size()));
            weighted = std::discrete_distribution<std::size_t>(w.begin(), w.end());
        }
        auto choose = [&](std::size_t& chosen, double& rrfactor) {
            if (rr_mode == ORC_RR_UNIFORM) {
                chosen = uniform(rng);
                rrfactor = double(uniform.max() + 1);
            } else {
                chosen = weighted(rng);
                rrfactor = 1.0 / weighted.probabilities()[chosen];
            }
        };
        auto body = [&](auto& acc) {
            for (uint64_t s = 0; s < spp; ++s) {
                std::size_t chosen;
                double rrfactor;
                choose(chosen, rrfactor);
                const R* r = list[chosen];
                const Range<DIM>& rbr = rr[chosen];
                std::array<float, DIM> x, ximp{};
                float sfactor;
                int branch = 0;
                auto uniform_point = [&]() {
                    for (int i = 0; i < DIM; ++i) {
                        std::uniform_real_distribution<float> dis(rbr.min(i), rbr.max(i));
                        x[i] = dis(rng);
                    }
                    sfactor = rbr.volume();
                };
                if constexpr (R::S == 3) {
                    std::uniform_real_distribution<float> dis(0, 1);
                    std::array<float, DIM> u;
                    if (sampling == ORC_RS_IMPORTANCE) { /* region-sampling.h:22-43 */
                        if (rbr.volume() < 1.e-5) uniform_point();
                        else {
                            for (int i = 0; i < DIM; ++i) u[i] = dis(rng);
                            x = r->sample_subrange(u, rbr);
                            const float pdf = r->pdf_subrange(x, rbr);
                            sfactor = (pdf < 1.e-5) ? 0.0 : (1.0 / pdf);
                        }
                    } else if (sampling == ORC_RS_RUSSIAN_ROULETTE) { /* :47-81 */
                        for (int i = 0; i < DIM; ++i) u[i] = dis(rng);
                        const float pdf_importance = r->pdf_integral_subrange(rbr);
                        const float pdf_uniform = rbr.volume();
                        const float rr_sample = dis(rng);
                        float pdf = 0;
                        if (rr_sample < (pdf_importance / (pdf_importance + pdf_uniform))) {
                            x = r->sample_subrange(u, rbr);
                            pdf = r->pdf_subrange(x, rbr);
                            branch = 1;
                        } else {
                            for (int i = 0; i < DIM; ++i) x[i] = rbr.min(i) + u[i] * (rbr.max(i) - rbr.min(i));
                            pdf = float(1) / rbr.volume();
                        }
                        sfactor = (pdf < 1.e-10) ? 0.0 : (1.0 / pdf);
                    } else if (sampling == ORC_RS_MIS) { /* :84-135 */
                        for (int i = 0; i < DIM; ++i) u[i] = dis(rng);
                        x = r->sample_subrange(u, rbr);
                        ximp = x;
                        const float pdf_importance = r->pdf_subrange(x, rbr);
                        const float pdf_uniform = float(1) / rbr.volume();
                        float mis_importance = std::pow(pdf_importance, cv.mis_power);
                        float mis_uniform = std::pow(pdf_uniform, cv.mis_power);
                        float mis_sum = mis_importance + mis_uniform;
                        if (mis_importance < (cv.mis_cutoff * mis_sum)) {
                            mis_importance = 0;
                            mis_sum = mis_uniform;
                        }
                        if (mis_uniform < (cv.mis_cutoff * mis_sum)) {
                            mis_uniform = 0;
                            mis_sum = mis_importance;
                        }
                        const float p_rr_importance =
                            (pdf_importance > 1.e-10) ? (mis_importance / pdf_importance) : float(0);
                        const float p_rr_uniform = mis_uniform * rbr.volume();
                        const float p_rr_sum = p_rr_importance + p_rr_uniform;
                        sfactor = p_rr_sum / mis_sum;
                        const float rr_sample = dis(rng);
                        branch = 1;
                        if (rr_sample < (p_rr_uniform / p_rr_sum)) {
                            for (int i = 0; i < DIM; ++i) x[i] = rbr.min(i) + u[i] * (rbr.max(i) - rbr.min(i));
                            branch = 0;
                        }
                    } else {
                        uniform_point();
                    }
                } else {
                    uniform_point();
                }
                if (rep) {
                    float* rc = rep + s * width;
                    rc[0] = float(chosen);
                    for (int i = 0; i < DIM; ++i) rc[1 + i] = x[i];
                    if (sampling == ORC_RS_RUSSIAN_ROULETTE || sampling == ORC_RS_MIS) rc[1 + DIM] = float(branch);
                    if (sampling == ORC_RS_MIS)
                        for (int i = 0; i < DIM; ++i) rc[2 + DIM + i] = ximp[i];
                }
                const T fs = f(x) * double(factor) * rrfactor * sfactor;
                const T as = r->approximation_at(x) * double(factor) * rrfactor * sfactor;
                acc.push(fs, as);
            }
            VT<T>::to(acc.integral(approximation), out + b * VT<T>::CH);
        };
        if (weight == ORC_CV_FIXED) {
            CvFixed<T> acc(alpha, T(0));
            body(acc);
        } else {
            CvOptimize<T> acc{T(0)};
            body(acc);
        }
    }
}

/* ------------------------------------------------------------------ dispatch */
template <class Visitor> int with_integrand(int32_t kind, const float* params, int32_t n, int32_t dim, Visitor&& v) {
    switch (kind) {
    case vcu::VCU_F_POLY2: {
        if (dim != 2) return 2;
        vcu::Poly2 f{};
        return v(f, std::integral_constant<int, 2>{}, float{});
    }
    case vcu::VCU_F_SIN1: {
        if (dim != 1) return 2;
        vcu::Sin1 f{};
        return v(f, std::integral_constant<int, 1>{}, float{});
    }
    case vcu::VCU_F_SPHERE3: {
        if (dim != 3) return 2;
        vcu::Sphere3 f{};
        return v(f, std::integral_constant<int, 3>{}, float{});
    }
    case vcu::VCU_F_WAVE2: {
        if (dim != 2) return 2;
        vcu::Wave2 f{};
        return v(f, std::integral_constant<int, 2>{}, float{});
    }
    case vcu::VCU_F_SCENE2: {
        if (dim != 2) return 2;
        auto* f = new vcu::Scene2;
        if (f->build(params, n)) { delete f; return 3; }
        const int r = v(*f, std::integral_constant<int, 2>{}, float{});
        delete f;
        return r;
    }
    case vcu::VCU_F_MOVING_SCENE3: {
        if (dim != 3) return 2;
        auto* f = new vcu::MovingScene3;
        if (f->build(params, n)) { delete f; return 3; }
        const int r = v(*f, std::integral_constant<int, 3>{}, vrgb{});
        delete f;
        return r;
    }
    case vcu::VCU_F_HALFSPACE: {
        vcu::Halfspace f{};
        if (f.build(params, n) || f.dim != dim) return 3;
        switch (dim) {
        case 1: return v(f, std::integral_constant<int, 1>{}, float{});
        case 2: return v(f, std::integral_constant<int, 2>{}, float{});
        case 3: return v(f, std::integral_constant<int, 3>{}, float{});
        case 4: return v(f, std::integral_constant<int, 4>{}, float{});
        case 5: return v(f, std::integral_constant<int, 5>{}, float{});
        case 6: return v(f, std::integral_constant<int, 6>{}, float{});
        default: return 2;
        }
    }
    case vcu::VCU_F_WALK2: {
        if (dim != 2) return 2;
        auto* f = new vcu::Walk2;
        if (f->build(params, n)) { delete f; return 3; }
        const int r = v(*f, std::integral_constant<int, 2>{}, float{});
        delete f;
        return r;
    }
    case vcu::VCU_F_OCCLUDED_SCENE5: {
        if (dim != 5) return 2;
        auto* f = new vcu::OccludedScene5;
        if (f->build(params, n)) { delete f; return 3; }
        const int r = v(*f, std::integral_constant<int, 5>{}, float{});
        delete f;
        return r;
    }
    default: return 4;
    }
}

template <class Visitor> int with_rules(const orc_nested& nc, Visitor&& v) {
    if (nc.rule_hi == ORC_RULE_BOOLE && nc.rule_lo == ORC_RULE_SIMPSON) return v(Boole{}, Simpson{});
    if (nc.rule_hi == ORC_RULE_BOOLE && nc.rule_lo == ORC_RULE_TRAPEZOIDAL) return v(Boole{}, Trapezoidal{});
    if (nc.rule_hi == ORC_RULE_SIMPSON && nc.rule_lo == ORC_RULE_TRAPEZOIDAL) return v(Simpson{}, Trapezoidal{});
    return 5;
}

}  // namespace orc
