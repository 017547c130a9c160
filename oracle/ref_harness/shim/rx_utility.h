/*
 * Test-infrastructure shim: stands in for the reference's missing
 * `rx_utility.h` (it is included by rx_kernel.h:18, rx_nnsearch.h:18 and
 * rx_sph_commons.h but is not part of the reference tree).  It supplies only
 * what the reference's CPU fluid functions use: a double-precision 3-vector
 * `Vec3`, `RXFunc::Max3`, and the constants RX_PI / RX_EPS / RX_FEQ_EPS.
 *
 * Written for this project; used only by oracle/ref_harness to compile the
 * reference's own CPU solver functions into oracle/_ref (the oracle's
 * reference pin).  Nothing in the product includes it.
 */
#ifndef FSPH_REF_SHIM_RX_UTILITY_H
#define FSPH_REF_SHIM_RX_UTILITY_H

#include <cassert>
#include <cmath>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>
#include <algorithm>
#include <bitset>

using namespace std;

#define RX_PI 3.14159265358979323846
#define RX_EPS 1.0e-8
#define RX_FEQ_EPS 1.0e-10

/* Vec3: the reference evaluates all per-pair geometry in double
 * (rx_nnsearch.h:657 draws it with glVertex3dv). */
class Vec3 {
public:
    double d[3];
    Vec3() { d[0] = d[1] = d[2] = 0.0; }
    explicit Vec3(double a) { d[0] = d[1] = d[2] = a; }
    Vec3(double a, double b, double c) { d[0] = a; d[1] = b; d[2] = c; }
    double &operator[](int i) { return d[i]; }
    const double &operator[](int i) const { return d[i]; }
    Vec3 &operator+=(const Vec3 &o) { d[0] += o.d[0]; d[1] += o.d[1]; d[2] += o.d[2]; return *this; }
    Vec3 &operator-=(const Vec3 &o) { d[0] -= o.d[0]; d[1] -= o.d[1]; d[2] -= o.d[2]; return *this; }
    Vec3 &operator*=(double s) { d[0] *= s; d[1] *= s; d[2] *= s; return *this; }
    Vec3 &operator/=(double s) { d[0] /= s; d[1] /= s; d[2] /= s; return *this; }
    Vec3 operator-() const { return Vec3(-d[0], -d[1], -d[2]); }
};
inline Vec3 operator+(const Vec3 &a, const Vec3 &b) { return Vec3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline Vec3 operator-(const Vec3 &a, const Vec3 &b) { return Vec3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline Vec3 operator-(const Vec3 &a, double s) { return Vec3(a[0] - s, a[1] - s, a[2] - s); }
inline Vec3 operator*(const Vec3 &a, double s) { return Vec3(a[0] * s, a[1] * s, a[2] * s); }
inline Vec3 operator*(double s, const Vec3 &a) { return Vec3(a[0] * s, a[1] * s, a[2] * s); }
/* element-wise product, as the reference's vector class (rx_sph_pbd.cpp:2045) */
inline Vec3 operator*(const Vec3 &a, const Vec3 &b) { return Vec3(a[0] * b[0], a[1] * b[1], a[2] * b[2]); }
inline Vec3 operator/(const Vec3 &a, double s) { return Vec3(a[0] / s, a[1] / s, a[2] / s); }
inline double norm2(const Vec3 &a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }
inline double norm(const Vec3 &a) { return sqrt(norm2(a)); }
inline double dot(const Vec3 &a, const Vec3 &b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline Vec3 cross(const Vec3 &a, const Vec3 &b) {
    return Vec3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline Vec3 Unit(const Vec3 &a) { double n = norm(a); return n > 0.0 ? a / n : a; }
inline std::ostream &operator<<(std::ostream &o, const Vec3 &a) {
    return o << "(" << a[0] << ", " << a[1] << ", " << a[2] << ")";
}

namespace RXFunc {
inline double Max3(const Vec3 &a) { return std::max(a[0], std::max(a[1], a[2])); }
}

#ifndef RXREAL
#define RXREAL float
#endif

#endif
