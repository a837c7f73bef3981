// Test infrastructure only: an f64 forward-mode dual number for the CPU
// oracle of the AVBD step.  Only tests/, __graft_entry__.smoke() and the
// bench's CPU-baseline leg may load anything built from oracle/.
//
// Dual carries a value and DUAL_DIRS directional derivatives.  Running the
// oracle's Engine<Dual> with seeded tangents gives the exact derivative of
// the CPU step along those directions (for the branch pattern the values
// take), which is what the device adjoint is checked against.  The rules are
// the textbook ones: (uv)' = u'v + uv', (u/v)' = (u'v - uv')/v^2,
// sqrt' = 1/(2 sqrt), asin' = 1/sqrt(1 - x^2), atan2(y, x)' = (x y' - y x')/r^2;
// comparisons, min/max and clamps look at values only, so a selection
// passes the selected operand's tangent through.
#pragma once
#include <cmath>
#include <limits>
#include <type_traits>

#include "avbd_crmath.hpp"

namespace orc {

constexpr int DUAL_DIRS = 8;

// V: the value type.  DualT<double> differentiates the f64 step; DualT<float>
// keeps f32 values computed in the f32 engine's operation order (so its
// trajectory is the f32 one bit for bit) with f64 tangents.
template <class V> struct DualT {
    V v = V(0);
    double d[DUAL_DIRS] = {};

    DualT() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic<A>::value>>
    DualT(A a) : v(V(a)) {}

    explicit operator double() const { return double(v); }
    explicit operator float() const { return float(v); }

    DualT& operator+=(const DualT& o) { return *this = *this + o; }
    DualT& operator-=(const DualT& o) { return *this = *this - o; }
    DualT& operator*=(const DualT& o) { return *this = *this * o; }
    DualT& operator/=(const DualT& o) { return *this = *this / o; }

    friend DualT operator+(const DualT& a, const DualT& b) {
        DualT r;
        r.v = a.v + b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = a.d[i] + b.d[i];
        return r;
    }
    friend DualT operator-(const DualT& a, const DualT& b) {
        DualT r;
        r.v = a.v - b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = a.d[i] - b.d[i];
        return r;
    }
    friend DualT operator-(const DualT& a) {
        DualT r;
        r.v = -a.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = -a.d[i];
        return r;
    }
    friend DualT operator*(const DualT& a, const DualT& b) {
        DualT r;
        r.v = a.v * b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = a.d[i] * double(b.v) + double(a.v) * b.d[i];
        return r;
    }
    friend DualT operator/(const DualT& a, const DualT& b) {
        DualT r;
        r.v = a.v / b.v;
        double ib = 1.0 / double(b.v), q = double(a.v) * ib;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = (a.d[i] - q * b.d[i]) * ib;
        return r;
    }
    friend bool operator<(const DualT& a, const DualT& b) { return a.v < b.v; }
    friend bool operator<=(const DualT& a, const DualT& b) { return a.v <= b.v; }
    friend bool operator>(const DualT& a, const DualT& b) { return a.v > b.v; }
    friend bool operator>=(const DualT& a, const DualT& b) { return a.v >= b.v; }
    friend bool operator==(const DualT& a, const DualT& b) { return a.v == b.v; }
    friend bool operator!=(const DualT& a, const DualT& b) { return a.v != b.v; }
};
using Dual = DualT<double>;
using DualF = DualT<float>;

// f(a) with f' given: the chain rule on every direction
template <class V> inline DualT<V> dual_apply(const DualT<V>& a, V fv, double dfv) {
    DualT<V> r;
    r.v = fv;
    for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = dfv * a.d[i];
    return r;
}

// The value with the tangents dropped (a quantity held fixed by the
// derivative), and a value carrying another expression's tangents.
template <class T> inline T no_tangent(const T& x) { return x; }
template <class V> inline DualT<V> no_tangent(const DualT<V>& x) { return DualT<V>(x.v); }
template <class T> inline T value_with_tangent(const T& value, const T&) { return value; }
template <class V> inline DualT<V> value_with_tangent(const DualT<V>& value, const DualT<V>& tangent_of) {
    DualT<V> r = tangent_of;
    r.v = value.v;
    return r;
}
template <class T> struct is_dual : std::false_type {};
template <class V> struct is_dual<DualT<V>> : std::true_type {};

}  // namespace orc

namespace std {
template <class V> inline orc::DualT<V> sqrt(const orc::DualT<V>& a) {
    V s = std::sqrt(a.v);
    return orc::dual_apply(a, s, s > V(0) ? 0.5 / double(s) : 0.0);
}
template <class V> inline orc::DualT<V> fabs(const orc::DualT<V>& a) {
    return orc::dual_apply(a, std::fabs(a.v), a.v < V(0) ? -1.0 : 1.0);
}
template <class V> inline orc::DualT<V> abs(const orc::DualT<V>& a) { return fabs(a); }
// a step function: derivative zero
template <class V> inline orc::DualT<V> floor(const orc::DualT<V>& a) { return orc::dual_apply(a, std::floor(a.v), 0.0); }
template <class V> inline orc::DualT<V> fmin(const orc::DualT<V>& a, const orc::DualT<V>& b) {
    return (b.v < a.v || std::isnan(a.v)) ? b : a;
}
template <class V> inline orc::DualT<V> fmax(const orc::DualT<V>& a, const orc::DualT<V>& b) {
    return (b.v > a.v || std::isnan(a.v)) ? b : a;
}
template <class V> inline orc::DualT<V> copysign(const orc::DualT<V>& a, const orc::DualT<V>& b) {
    bool flip = std::signbit(a.v) != std::signbit(b.v);
    return flip ? -a : a;
}
template <class V> inline orc::DualT<V> fmod(const orc::DualT<V>& x, const orc::DualT<V>& m) {
    double q = std::trunc(double(x.v) / double(m.v));
    orc::DualT<V> r;
    r.v = std::fmod(x.v, m.v);
    for (int i = 0; i < orc::DUAL_DIRS; i++) r.d[i] = x.d[i] - q * m.d[i];
    return r;
}
template <class V> inline orc::DualT<V> sin(const orc::DualT<V>& a) {
    return orc::dual_apply(a, orc::osin(a.v), std::cos(double(a.v)));
}
template <class V> inline orc::DualT<V> cos(const orc::DualT<V>& a) {
    return orc::dual_apply(a, orc::ocos(a.v), -std::sin(double(a.v)));
}
template <class V> inline orc::DualT<V> asin(const orc::DualT<V>& a) {
    double c = 1.0 - double(a.v) * double(a.v);
    return orc::dual_apply(a, orc::oasin(a.v), c > 0.0 ? 1.0 / std::sqrt(c) : 0.0);
}
template <class V> inline orc::DualT<V> atan2(const orc::DualT<V>& y, const orc::DualT<V>& x) {
    orc::DualT<V> r;
    r.v = orc::oatan2(y.v, x.v);
    double xv = double(x.v), yv = double(y.v);
    double r2 = xv * xv + yv * yv;
    double k = r2 > 0.0 ? 1.0 / r2 : 0.0;
    for (int i = 0; i < orc::DUAL_DIRS; i++) r.d[i] = (xv * y.d[i] - yv * x.d[i]) * k;
    return r;
}
template <class V> inline bool isfinite(const orc::DualT<V>& a) { return std::isfinite(a.v); }
template <class V> inline bool isnan(const orc::DualT<V>& a) { return std::isnan(a.v); }
template <class V> inline bool signbit(const orc::DualT<V>& a) { return std::signbit(a.v); }

template <class V> class numeric_limits<orc::DualT<V>> {
public:
    static constexpr bool is_specialized = true;
    static orc::DualT<V> infinity() { return orc::DualT<V>(std::numeric_limits<V>::infinity()); }
    static orc::DualT<V> max() { return orc::DualT<V>(std::numeric_limits<V>::max()); }
    static orc::DualT<V> lowest() { return orc::DualT<V>(std::numeric_limits<V>::lowest()); }
    static orc::DualT<V> epsilon() { return orc::DualT<V>(std::numeric_limits<V>::epsilon()); }
};
}  // namespace std
