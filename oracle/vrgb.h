/*
 * vrgb.h -- the 3-channel value type used as viltrum's bin value type for RGB integrands.
 *
 * Test infrastructure (oracle): shared by the CPU restatement (oracle.cc) and by the driver
 * that runs the unmodified reference headers (ref_driver.cc), so both compute with the same
 * value-type semantics.  viltrum's rules and control-variate accumulators are templates over
 * the bin value type and need + - with itself, scaling by int/float/double, T(0), and
 * begin()/end() over channels (src/newton-cotes/rules.h:59-100, src/control-variates/norm.h:11-42,
 * src/nested/error-metric.h:61-73).  Every operation works per channel and rounds each result
 * to float once; a scale by double is computed in double and rounded to float.
 */
#pragma once
#include <array>
#include <cstddef>

struct vrgb {
    using value_type = float;
    float c[3];
    vrgb() : c{0.0f, 0.0f, 0.0f} {}
    explicit vrgb(double v) : c{float(v), float(v), float(v)} {}
    explicit vrgb(float v) : c{v, v, v} {}
    explicit vrgb(int v) : c{float(v), float(v), float(v)} {}
    vrgb(float a, float b, float d) : c{a, b, d} {}
    const float* begin() const { return c; }
    const float* end() const { return c + 3; }
    float* begin() { return c; }
    float* end() { return c + 3; }
    float& operator[](std::size_t i) { return c[i]; }
    const float& operator[](std::size_t i) const { return c[i]; }
    vrgb& operator+=(const vrgb& o) { for (int i = 0; i < 3; ++i) c[i] = c[i] + o.c[i]; return *this; }
    vrgb& operator-=(const vrgb& o) { for (int i = 0; i < 3; ++i) c[i] = c[i] - o.c[i]; return *this; }
    vrgb& operator=(double v) { for (int i = 0; i < 3; ++i) c[i] = float(v); return *this; }
};
inline vrgb operator+(const vrgb& a, const vrgb& b) { return vrgb(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]); }
inline vrgb operator-(const vrgb& a, const vrgb& b) { return vrgb(a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]); }
inline vrgb operator-(const vrgb& a) { return vrgb(-a.c[0], -a.c[1], -a.c[2]); }
inline vrgb operator*(const vrgb& a, float s) { return vrgb(a.c[0] * s, a.c[1] * s, a.c[2] * s); }
inline vrgb operator*(float s, const vrgb& a) { return a * s; }
inline vrgb operator*(const vrgb& a, int s) { return a * float(s); }
inline vrgb operator*(int s, const vrgb& a) { return a * float(s); }
inline vrgb operator*(const vrgb& a, std::size_t s) { return a * float(s); }
inline vrgb operator*(std::size_t s, const vrgb& a) { return a * float(s); }
inline vrgb operator*(const vrgb& a, double s) {
    return vrgb(float(double(a.c[0]) * s), float(double(a.c[1]) * s), float(double(a.c[2]) * s));
}
inline vrgb operator*(double s, const vrgb& a) { return a * s; }
inline vrgb operator/(const vrgb& a, float s) { return vrgb(a.c[0] / s, a.c[1] / s, a.c[2] / s); }
inline vrgb operator/(const vrgb& a, int s) { return a / float(s); }
inline vrgb operator/(const vrgb& a, double s) {
    return vrgb(float(double(a.c[0]) / s), float(double(a.c[1]) / s), float(double(a.c[2]) / s));
}
