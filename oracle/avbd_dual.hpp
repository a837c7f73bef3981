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

namespace orc {

constexpr int DUAL_DIRS = 8;

struct Dual {
    double v = 0.0;
    double d[DUAL_DIRS] = {};

    Dual() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic<A>::value>>
    Dual(A a) : v(double(a)) {}

    explicit operator double() const { return v; }
    explicit operator float() const { return float(v); }

    Dual& operator+=(const Dual& o) { return *this = *this + o; }
    Dual& operator-=(const Dual& o) { return *this = *this - o; }
    Dual& operator*=(const Dual& o) { return *this = *this * o; }
    Dual& operator/=(const Dual& o) { return *this = *this / o; }

    friend Dual operator+(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v + b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = a.d[i] + b.d[i];
        return r;
    }
    friend Dual operator-(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v - b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = a.d[i] - b.d[i];
        return r;
    }
    friend Dual operator-(const Dual& a) {
        Dual r;
        r.v = -a.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = -a.d[i];
        return r;
    }
    friend Dual operator*(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v * b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
        return r;
    }
    friend Dual operator/(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v / b.v;
        double ib = 1.0 / b.v;
        for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
        return r;
    }
    friend bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    friend bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
    friend bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
};

// f(a) with f' given: the chain rule on every direction
inline Dual dual_apply(const Dual& a, double fv, double dfv) {
    Dual r;
    r.v = fv;
    for (int i = 0; i < DUAL_DIRS; i++) r.d[i] = dfv * a.d[i];
    return r;
}

// The value with the tangents dropped (a quantity held fixed by the
// derivative), and a value carrying another expression's tangents.
template <class T> inline T no_tangent(const T& x) { return x; }
inline Dual no_tangent(const Dual& x) { return Dual(x.v); }
template <class T> inline T value_with_tangent(const T& value, const T&) { return value; }
inline Dual value_with_tangent(const Dual& value, const Dual& tangent_of) {
    Dual r = tangent_of;
    r.v = value.v;
    return r;
}
template <class T> struct is_dual : std::false_type {};
template <> struct is_dual<Dual> : std::true_type {};

}  // namespace orc

namespace std {
inline orc::Dual sqrt(const orc::Dual& a) {
    double s = std::sqrt(a.v);
    return orc::dual_apply(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
inline orc::Dual fabs(const orc::Dual& a) { return orc::dual_apply(a, std::fabs(a.v), a.v < 0.0 ? -1.0 : 1.0); }
inline orc::Dual abs(const orc::Dual& a) { return fabs(a); }
inline orc::Dual fmin(const orc::Dual& a, const orc::Dual& b) { return (b.v < a.v || std::isnan(a.v)) ? b : a; }
inline orc::Dual fmax(const orc::Dual& a, const orc::Dual& b) { return (b.v > a.v || std::isnan(a.v)) ? b : a; }
inline orc::Dual copysign(const orc::Dual& a, const orc::Dual& b) {
    bool flip = std::signbit(a.v) != std::signbit(b.v);
    return flip ? -a : a;
}
inline orc::Dual fmod(const orc::Dual& x, const orc::Dual& m) {
    double q = std::trunc(x.v / m.v);
    orc::Dual r = x - orc::Dual(q) * m;
    r.v = std::fmod(x.v, m.v);
    return r;
}
inline orc::Dual sin(const orc::Dual& a) { return orc::dual_apply(a, std::sin(a.v), std::cos(a.v)); }
inline orc::Dual cos(const orc::Dual& a) { return orc::dual_apply(a, std::cos(a.v), -std::sin(a.v)); }
inline orc::Dual asin(const orc::Dual& a) {
    double c = 1.0 - a.v * a.v;
    return orc::dual_apply(a, std::asin(a.v), c > 0.0 ? 1.0 / std::sqrt(c) : 0.0);
}
inline orc::Dual atan2(const orc::Dual& y, const orc::Dual& x) {
    orc::Dual r;
    r.v = std::atan2(y.v, x.v);
    double r2 = x.v * x.v + y.v * y.v;
    double k = r2 > 0.0 ? 1.0 / r2 : 0.0;
    for (int i = 0; i < orc::DUAL_DIRS; i++) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) * k;
    return r;
}
inline bool isfinite(const orc::Dual& a) { return std::isfinite(a.v); }
inline bool isnan(const orc::Dual& a) { return std::isnan(a.v); }
inline bool signbit(const orc::Dual& a) { return std::signbit(a.v); }

template <> class numeric_limits<orc::Dual> {
public:
    static constexpr bool is_specialized = true;
    static orc::Dual infinity() { return orc::Dual(std::numeric_limits<double>::infinity()); }
    static orc::Dual max() { return orc::Dual(std::numeric_limits<double>::max()); }
    static orc::Dual lowest() { return orc::Dual(std::numeric_limits<double>::lowest()); }
    static orc::Dual epsilon() { return orc::Dual(std::numeric_limits<double>::epsilon()); }
};
}  // namespace std
