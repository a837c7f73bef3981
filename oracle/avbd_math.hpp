// Test infrastructure only: scalar vector/quaternion arithmetic for the CPU
// oracle of the AVBD step.  Only tests/, __graft_entry__.smoke() and the
// bench's CPU-baseline leg may load anything built from oracle/.
//
// The operation order follows glam 0.34.3 (Cargo.lock:1357-1358), the math
// crate the reference calls on every line of its AVBD path, so that the f32
// instantiation reproduces the reference's rounding:
//   Vec3::dot        (x*x' + y*y') + z*z'
//   Vec3::cross      (y*z' - y'*z, z*x' - z'*x, x*y' - x'*y)
//   Vec3::normalize  v * (1 / |v|);  normalize_or falls back unless the
//                    reciprocal is finite and positive
//   Quat * Vec3      v*(w*w - |b|^2) + b*(2 v.b) + (b x v)*(2w)
//   Quat * Quat      Hamilton product, component order of avbd/rows.rs:91-98
//   Mat3::from_quat  columns of the doubled-product form
// Compile without FMA contraction (-ffp-contract=off): the reference's Rust
// code never fuses.
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>

namespace orc {

template <class T> struct V3 {
    T x, y, z;
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline bool operator==(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T> inline bool operator!=(V3<T> a, V3<T> b) { return !(a == b); }
template <class T> inline T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> inline T len2(V3<T> a) { return dot(a, a); }
template <class T> inline T len(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) { return a * (T(1) / len(a)); }
template <class T> inline V3<T> normalize_or(V3<T> a, V3<T> f) {
    T r = T(1) / len(a);
    if (std::isfinite(r) && r > T(0)) return a * r;
    return f;
}
template <class T> inline V3<T> normalize_or_zero(V3<T> a) { return normalize_or(a, V3<T>{0, 0, 0}); }
template <class T> inline V3<T> vabs(V3<T> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
// Rust f32::min / f32::max (NaN-ignoring) are fmin / fmax.
template <class T> inline T fmn(T a, T b) { return std::fmin(a, b); }
template <class T> inline T fmx(T a, T b) { return std::fmax(a, b); }
template <class T> inline T fclamp(T x, T lo, T hi) {
    // Rust f32::clamp: x < lo -> lo, x > hi -> hi, NaN passes through.
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
template <class T> inline V3<T> vclamp(V3<T> v, V3<T> lo, V3<T> hi) {
    // glam Vec3::clamp = self.max(min).min(max)
    return {fmn(fmx(v.x, lo.x), hi.x), fmn(fmx(v.y, lo.y), hi.y), fmn(fmx(v.z, lo.z), hi.z)};
}
template <class T> inline T min_element(V3<T> v) { return fmn(v.x, fmn(v.y, v.z)); }
template <class T> inline T signum(T x) { return std::isnan(x) ? x : std::copysign(T(1), x); }

template <class T> inline V3<T> VX() { return {T(1), T(0), T(0)}; }
template <class T> inline V3<T> VY() { return {T(0), T(1), T(0)}; }
template <class T> inline V3<T> VZ() { return {T(0), T(0), T(1)}; }
template <class T> inline V3<T> VZERO() { return {T(0), T(0), T(0)}; }

template <class T> struct Qt {
    T x, y, z, w;
};
template <class T> inline Qt<T> qident() { return {T(0), T(0), T(0), T(1)}; }
template <class T> inline bool operator==(Qt<T> a, Qt<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }
template <class T> inline bool operator!=(Qt<T> a, Qt<T> b) { return !(a == b); }
template <class T> inline Qt<T> conj(Qt<T> q) { return {-q.x, -q.y, -q.z, q.w}; }
template <class T> inline Qt<T> qmul(Qt<T> a, Qt<T> b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w,
            a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
template <class T> inline V3<T> qrot(Qt<T> q, V3<T> v) {
    V3<T> b{q.x, q.y, q.z};
    T b2 = dot(b, b);
    return (v * (q.w * q.w - b2) + b * (dot(v, b) * T(2))) + cross(b, v) * (q.w * T(2));
}
template <class T> inline Qt<T> qnormalize(Qt<T> q) {
    // glam Vec4 length on aarch64 NEON: pairwise horizontal add.
    T l = std::sqrt((q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w));
    T r = T(1) / l;
    return {q.x * r, q.y * r, q.z * r, q.w * r};
}

template <class T> struct M3 {
    // row-major: m[row][col]
    T m[3][3];
};
// glam Mat3::from_quat; returns columns (x_axis, y_axis, z_axis).
template <class T> inline void mat3_from_quat(Qt<T> q, V3<T> cols[3]) {
    T x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    T xx = q.x * x2, xy = q.x * y2, xz = q.x * z2;
    T yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
    T wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    cols[0] = {T(1) - (yy + zz), xy + wz, xz - wy};
    cols[1] = {xy - wz, T(1) - (xx + zz), yz + wx};
    cols[2] = {xz + wy, yz - wx, T(1) - (xx + yy)};
}

}  // namespace orc
