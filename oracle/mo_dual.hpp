// Test infrastructure only: the forward-mode (tangent-linear) number of the oracle's
// tangent build (MO_TANGENT).  A Dual carries a value v and its directional derivative d;
// v is computed by exactly the double operation the oracle's plain build performs, so the
// tangent build's values equal the plain build's bit for bit, and every branch (limiter,
// upwind choice, min / max) is decided on v as in the forward model.  d follows the
// derivative of the branch taken: the tangent-linear model of the piecewise-smooth stage.
#pragma once
#include <cmath>

namespace mo {

struct Dual {
    double v = 0.0, d = 0.0;
    Dual() = default;
    Dual(double x) : v(x), d(0.0) {}  // constants carry no derivative
    Dual(double x, double dx) : v(x), d(dx) {}
    Dual& operator+=(const Dual& b) { d = d + b.d; v = v + b.v; return *this; }
    Dual& operator-=(const Dual& b) { d = d - b.d; v = v - b.v; return *this; }
    Dual& operator*=(const Dual& b) { d = d * b.v + v * b.d; v = v * b.v; return *this; }
    Dual& operator/=(const Dual& b) {
        const double q = v / b.v;
        d = (d - q * b.d) / b.v;
        v = q;
        return *this;
    }
};

inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
inline Dual operator+(const Dual& a) { return a; }
inline Dual operator+(double a, const Dual& b) { return Dual(a) + b; }
inline Dual operator-(double a, const Dual& b) { return Dual(a) - b; }
inline Dual operator*(double a, const Dual& b) { return Dual(a * b.v, a * b.d); }
inline Dual operator/(double a, const Dual& b) { return Dual(a) / b; }
inline Dual operator+(const Dual& a, double b) { return a + Dual(b); }
inline Dual operator-(const Dual& a, double b) { return a - Dual(b); }
inline Dual operator*(const Dual& a, double b) { return Dual(a.v * b, a.d * b); }
inline Dual operator/(const Dual& a, double b) { return Dual(a.v / b, a.d / b); }

#define MO_DUAL_CMP(op)                                                            \
    inline bool operator op(const Dual& a, const Dual& b) { return a.v op b.v; } \
    inline bool operator op(const Dual& a, double b) { return a.v op b; }       \
    inline bool operator op(double a, const Dual& b) { return a op b.v; }
MO_DUAL_CMP(<)
MO_DUAL_CMP(>)
MO_DUAL_CMP(<=)
MO_DUAL_CMP(>=)
MO_DUAL_CMP(==)
MO_DUAL_CMP(!=)
#undef MO_DUAL_CMP

inline double value_of(const Dual& a) { return a.v; }
inline double tangent_of(const Dual& a) { return a.d; }

// |a|, copysign(a, b) (the sign of b decides, so b's derivative does not enter), sqrt
inline Dual fabs_r(const Dual& a) { return std::signbit(a.v) ? -a : a; }
inline Dual copysign_r(const Dual& a, const Dual& b) {
    const double r = std::copysign(a.v, b.v);
    return Dual(r, std::signbit(r) == std::signbit(a.v) ? a.d : -a.d);
}
inline Dual sqrt_r(const Dual& a) {
    const double r = std::sqrt(a.v);
    return Dual(r, r > 0.0 ? a.d / (2.0 * r) : 0.0);
}

}  // namespace mo
