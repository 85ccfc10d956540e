// Test infrastructure (oracle): forward-mode dual number for exact
// Jacobian-vector products of the CPU restatement.  Replaces the role ADOL-C's
// adouble plays in the reference (src/common.h:55-58, src/solver/solver.cpp:72-90):
// the same templated residual code evaluated on Dual gives dR/dQ . v exactly.
#pragma once
#include <cmath>

struct Dual {
    double v, d;
    Dual() : v(0.0), d(0.0) {}
    Dual(double x) : v(x), d(0.0) {}
    Dual(double x, double dx) : v(x), d(dx) {}
    Dual& operator+=(const Dual& o) { v += o.v; d += o.d; return *this; }
    Dual& operator-=(const Dual& o) { v -= o.v; d -= o.d; return *this; }
    Dual& operator*=(const Dual& o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
    Dual& operator/=(const Dual& o) { double q = v / o.v; d = (d - q * o.d) / o.v; v = q; return *this; }
};
inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator+(Dual a, double b) { a.v += b; return a; }
inline Dual operator+(double b, Dual a) { a.v += b; return a; }
inline Dual operator-(Dual a, double b) { a.v -= b; return a; }
inline Dual operator-(double b, const Dual& a) { return Dual(b - a.v, -a.d); }
inline Dual operator*(Dual a, double b) { a.v *= b; a.d *= b; return a; }
inline Dual operator*(double b, Dual a) { a.v *= b; a.d *= b; return a; }
inline Dual operator/(Dual a, double b) { a.v /= b; a.d /= b; return a; }
inline Dual operator/(double b, const Dual& a) { double q = b / a.v; return Dual(q, -q * a.d / a.v); }
inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline bool operator<(const Dual& a, double b) { return a.v < b; }
inline bool operator>(const Dual& a, double b) { return a.v > b; }
inline bool operator<=(const Dual& a, double b) { return a.v <= b; }
inline bool operator>=(const Dual& a, double b) { return a.v >= b; }
inline Dual sqrt(const Dual& a) { double s = std::sqrt(a.v); return Dual(s, a.d / (2.0 * s)); }
inline Dual fabs(const Dual& a) { return a.v < 0.0 ? -a : a; }
inline Dual pow(const Dual& a, double e) {
    double p = std::pow(a.v, e);
    return Dual(p, a.v == 0.0 ? 0.0 : e * p / a.v * a.d);
}
inline double value(const Dual& a) { return a.v; }
inline double value(double a) { return a; }
