// avbd_vec.cuh — scalar f32 vector / quaternion arithmetic for the AVBD kernels.
//
// The reference's AVBD step (crates/physics/src/avbd/*) does all its math
// through glam 0.34.3.  To make the GPU's integer decisions (pair sets,
// contact IDs, colours) identical to the reference on identical input, every
// helper here evaluates in glam's operation order and the translation units
// that decide integers are compiled with -fmad=false (no contraction):
//   dot          (x*x' + y*y') + z*z'
//   cross        (y*z' - y'*z, z*x' - z'*x, x*y' - x'*y)
//   normalize    v * (1/|v|); normalize_or keeps the fallback unless the
//                reciprocal is finite and > 0
//   q * v        v*(w*w - |b|^2) + b*(2 v.b) + (b x v)*(2w)
//   q * q        Hamilton product (avbd/rows.rs:91-98 component order)
//   |q|          (x*x + y*y) + (z*z + w*w)  (4-lane pairwise sum)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#define AVBD_HD __host__ __device__ __forceinline__

namespace avbd {

struct V3 {
    float x, y, z;
    AVBD_HD float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    AVBD_HD float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
AVBD_HD V3 mk(float x, float y, float z) { return V3{x, y, z}; }
AVBD_HD V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
AVBD_HD V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
AVBD_HD V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
AVBD_HD V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
AVBD_HD V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
AVBD_HD V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
AVBD_HD bool veq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
AVBD_HD float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
AVBD_HD V3 cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
AVBD_HD float len2(V3 a) { return dot(a, a); }
AVBD_HD float len(V3 a) { return sqrtf(dot(a, a)); }
AVBD_HD V3 normalize(V3 a) { return a * (1.0f / len(a)); }
AVBD_HD bool finitef(float x) { return isfinite(x); }
AVBD_HD V3 normalize_or(V3 a, V3 f) {
    float r = 1.0f / len(a);
    return (finitef(r) && r > 0.0f) ? a * r : f;
}
AVBD_HD V3 vabs(V3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
AVBD_HD float fclamp(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
AVBD_HD V3 vclamp(V3 v, V3 lo, V3 hi) {
    return {fminf(fmaxf(v.x, lo.x), hi.x), fminf(fmaxf(v.y, lo.y), hi.y), fminf(fmaxf(v.z, lo.z), hi.z)};
}
AVBD_HD float min_element(V3 v) { return fminf(v.x, fminf(v.y, v.z)); }
AVBD_HD float signumf(float x) { return isnan(x) ? x : copysignf(1.0f, x); }
AVBD_HD V3 VX() { return {1.0f, 0.0f, 0.0f}; }
AVBD_HD V3 VY() { return {0.0f, 1.0f, 0.0f}; }
AVBD_HD V3 VZ() { return {0.0f, 0.0f, 1.0f}; }
AVBD_HD V3 V0() { return {0.0f, 0.0f, 0.0f}; }

struct Q {
    float x, y, z, w;
};
AVBD_HD Q qid() { return {0.0f, 0.0f, 0.0f, 1.0f}; }
AVBD_HD bool qeq(Q a, Q b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }
AVBD_HD Q conj(Q q) { return {-q.x, -q.y, -q.z, q.w}; }
AVBD_HD Q qmul(Q a, Q b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
AVBD_HD V3 qrot(Q q, V3 v) {
    V3 b{q.x, q.y, q.z};
    float b2 = dot(b, b);
    return (v * (q.w * q.w - b2) + b * (dot(v, b) * 2.0f)) + cross(b, v) * (q.w * 2.0f);
}
AVBD_HD Q qnormalize(Q q) {
    float l = sqrtf((q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w));
    float r = 1.0f / l;
    return {q.x * r, q.y * r, q.z * r, q.w * r};
}
// Columns of the rotation matrix (glam Mat3::from_quat).
AVBD_HD void mat3_cols(Q q, V3 c[3]) {
    float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    float xx = q.x * x2, xy = q.x * y2, xz = q.x * z2;
    float yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
    float wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    c[0] = {1.0f - (yy + zz), xy + wz, xz - wy};
    c[1] = {xy - wz, 1.0f - (xx + zz), yz + wx};
    c[2] = {xz + wy, yz - wx, 1.0f - (xx + yy)};
}

AVBD_HD V3 ld3(float4 v) { return {v.x, v.y, v.z}; }
AVBD_HD Q ldq(float4 v) { return {v.x, v.y, v.z, v.w}; }
AVBD_HD float4 st3(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
AVBD_HD float4 stq(Q q) { return make_float4(q.x, q.y, q.z, q.w); }

// Order-preserving map of a float onto uint32 (for radix keys and atomicMin).
AVBD_HD uint32_t f2key(float f) {
#ifdef __CUDA_ARCH__
    uint32_t u = __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

}  // namespace avbd
