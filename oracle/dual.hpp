// Forward-mode dual number (value, one tangent) for the oracle compiled as
// C++ with ORC_DUAL: the same restatement of the step, differentiated
// exactly along one seeded direction.  Branches follow the values.  Test
// infrastructure.
#pragma once
#include <cmath>

struct real {
    double v, d;
    real() : v(0.0), d(0.0) {}
    real(double a) : v(a), d(0.0) {}
    real(double a, double b) : v(a), d(b) {}
};

#define R_VAL(x) ((x).v)

inline real operator+(real a, real b) { return real(a.v + b.v, a.d + b.d); }
inline real operator-(real a, real b) { return real(a.v - b.v, a.d - b.d); }
inline real operator*(real a, real b) { return real(a.v * b.v, a.d * b.v + a.v * b.d); }
inline real operator/(real a, real b) { return real(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline real operator-(real a) { return real(-a.v, -a.d); }
inline real operator+(real a, double b) { return real(a.v + b, a.d); }
inline real operator+(double a, real b) { return real(a + b.v, b.d); }
inline real operator-(real a, double b) { return real(a.v - b, a.d); }
inline real operator-(double a, real b) { return real(a - b.v, -b.d); }
inline real operator*(real a, double b) { return real(a.v * b, a.d * b); }
inline real operator*(double a, real b) { return real(a * b.v, a * b.d); }
inline real operator/(real a, double b) { return real(a.v / b, a.d / b); }
inline real operator/(double a, real b) { return real(a / b.v, -a * b.d / (b.v * b.v)); }
inline real &operator+=(real &a, real b) { return a = a + b; }
inline real &operator-=(real &a, real b) { return a = a - b; }
inline real &operator*=(real &a, real b) { return a = a * b; }
inline real &operator/=(real &a, real b) { return a = a / b; }

#define ORC_DUAL_CMP(OP)                                                      \
    inline bool operator OP(real a, real b) { return a.v OP b.v; }            \
    inline bool operator OP(real a, double b) { return a.v OP b; }            \
    inline bool operator OP(double a, real b) { return a OP b.v; }
ORC_DUAL_CMP(<)
ORC_DUAL_CMP(<=)
ORC_DUAL_CMP(>)
ORC_DUAL_CMP(>=)
ORC_DUAL_CMP(==)
ORC_DUAL_CMP(!=)
#undef ORC_DUAL_CMP

inline real sqrt(real a) {
    const double s = std::sqrt(a.v);
    return real(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
}
inline real exp(real a) {
    const double e = std::exp(a.v);
    return real(e, e * a.d);
}
inline real sin(real a) { return real(std::sin(a.v), std::cos(a.v) * a.d); }
inline real cos(real a) { return real(std::cos(a.v), -std::sin(a.v) * a.d); }
inline real pow(real a, double n) {
    const double p = std::pow(a.v, n);
    return real(p, a.v != 0.0 ? n * std::pow(a.v, n - 1.0) * a.d : 0.0);
}
inline real fabs(real a) { return a.v < 0.0 ? -a : a; }
inline real fmin(real a, real b) { return a.v <= b.v ? a : b; }
inline real fmin(real a, double b) { return a.v <= b ? a : real(b); }
inline real fmin(double a, real b) { return a <= b.v ? real(a) : b; }
