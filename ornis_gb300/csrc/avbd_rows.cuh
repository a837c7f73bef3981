// avbd_rows.cuh — per-row AVBD arithmetic shared by the primal and dual
// kernels: Taylor contact residuals, clamped contact forces, row stamps into
// the lower triangle of the per-body 6x6 system, and the dense LDL^T solve.
//
// Reference: crates/physics/src/avbd/rows.rs:110-191 (rotation helpers, limit
// state), :947-1111 (row_c, levers, contact_force, stamp rows),
// crates/physics/src/avbd/assembly.rs:25-69 (solve_6x6),
// crates/physics/src/avbd/joints_ext.rs:21-32 (gap_c0).
#pragma once
#include "avbd_crmath.cuh"
#include "avbd_world.cuh"

namespace avbd {

// Lower triangle of the symmetric 6x6 system, row-major: (i, j) with j <= i
// lives at i*(i+1)/2 + j.
struct Sys {
    float h[21];
    float r[6];
};
static __host__ __device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// sin, cos, asin and atan2 are the correctly rounded ones (avbd_crmath.cuh):
// the reference's libm results, identical on every device and host.
static __host__ __device__ __forceinline__ Q quat_integrate(Q q, V3 v) {  // rows.rs:110-119
    float theta = len(v);
    if (theta < NEAR_ZERO) return q;
    float s, c;
    crm::sincosf(HALF * theta, &s, &c);
    float k = s / theta;
    Q dq = qmul(Q{v.x * k, v.y * k, v.z * k, c}, q);
    return qnormalize(dq);
}
static __host__ __device__ __forceinline__ V3 quat_diff_vec(Q a, Q b) {  // rows.rs:128-146
    Q r = qmul(a, Q{-b.x, -b.y, -b.z, b.w});
    V3 xyz{r.x, r.y, r.z};
    if (r.w < 0.0f) xyz = -xyz;
    float s = fminf(len(xyz), 1.0f);
    if (s < NEAR_ZERO) return V0();
    return xyz * (2.0f * crm::asinf(s) / s);
}
static __host__ __device__ __forceinline__ float rem_euclid(float x, float m) {
    float r = fmodf(x, m);
    return r < 0.0f ? r + fabsf(m) : r;
}
static __host__ __device__ __forceinline__ float wrap_pi(float x) { return rem_euclid(x + PI_F, TAU_F) - PI_F; }
static __host__ __device__ __forceinline__ float quat_twist(Q q, V3 axis) {  // sequential_impulse/joints.rs:44-48
    float t = 2.0f * crm::atan2f(dot(V3{q.x, q.y, q.z}, axis), q.w);
    return rem_euclid(t + PI_F, TAU_F) - PI_F;
}
static __host__ __device__ __forceinline__ float hinge_twist(Q qa, Q qb, V3 axis) {  // :38-43
    return quat_twist(qmul(conj(qa), qb), axis);
}
static __host__ __device__ __forceinline__ int limit_state(float v, float lo, float hi, float slop) {  // rows.rs:156-164
    if (v <= lo + slop) return 1;
    if (v >= hi - slop) return 0;
    return -1;
}
static __host__ __device__ __forceinline__ int warm_limit_state(float v, float lo, float hi, float slop, float force) {  // rows.rs:156-183
    if (v <= lo + slop) return 1;
    if (v >= hi - slop) return 0;
    if (force < 0.0f) return 1;
    if (force > 0.0f) return 0;
    return -1;
}
static __host__ __device__ __forceinline__ float regularized_limit(float value, float initial, float bound, bool lower) {
    float old = initial - bound;
    float viol = lower ? fminf(old, 0.0f) : fmaxf(old, 0.0f);
    return value - bound - ALPHA * viol;
}
static __host__ __device__ __forceinline__ V3 tangent_t1(V3 n) {  // math.rs:152-160
    V3 axis = fabsf(n.x) < TANGENT_REF_AXIS_DOT ? VX() : VY();
    return normalize_or(cross(n, axis), VZ());
}
// math.rs:179-186: the wheel's axle made orthogonal to its suspension axis
static __host__ __device__ __forceinline__ V3 orthogonalize_axle(V3 s, V3 axle) {
    V3 a = axle - s * dot(axle, s);
    if (len2(a) < POS_CORRECTION_EPS) return tangent_t1(s);
    return normalize(a);
}
static __host__ __device__ __forceinline__ void world_inertia(V3 inertia, Q rot, float m[3][3]) {  // rows.rs:194-207
    V3 c[3];
    mat3_cols(rot, c);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            m[a][b] = c[0][a] * inertia.x * c[0][b] + c[1][a] * inertia.y * c[1][b] + c[2][a] * inertia.z * c[2][b];
}
static __host__ __device__ __forceinline__ void inverse_symmetric(const float m[3][3], V3 diag, float o[3][3]) {  // rows.rs:211-241
    float a = m[0][0], b = m[0][1], c = m[0][2], d = m[1][1], e = m[1][2], f = m[2][2];
    float det = a * (d * f - e * e) - b * (b * f - c * e) + c * (b * e - c * d);
    if (fabsf(det) < DEGENERATE_LEN2) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) o[i][j] = 0.0f;
        o[0][0] = diag.x > 0.0f ? 1.0f / diag.x : 0.0f;
        o[1][1] = diag.y > 0.0f ? 1.0f / diag.y : 0.0f;
        o[2][2] = diag.z > 0.0f ? 1.0f / diag.z : 0.0f;
        return;
    }
    float id = 1.0f / det;
    o[0][0] = (d * f - e * e) * id; o[0][1] = (c * e - b * f) * id; o[0][2] = (b * e - c * d) * id;
    o[1][0] = (c * e - b * f) * id; o[1][1] = (a * f - c * c) * id; o[1][2] = (b * c - a * e) * id;
    o[2][0] = (b * e - c * d) * id; o[2][1] = (b * c - a * e) * id; o[2][2] = (a * d - b * b) * id;
}
static __host__ __device__ __forceinline__ V3 mat3_vec(const float m[3][3], V3 v) {
    return {m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
            m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z};
}
static __host__ __device__ __forceinline__ bool row_live(float c, float f) { return fabsf(c) >= C_EPS || f != 0.0f; }

// stamp_row (rows.rs:1064-1092) restricted to the lower triangle.
static __host__ __device__ __forceinline__ void stamp_row(Sys& s, V3 axis, float pen, float f, V3 r, float sign) {
    V3 nn = sign * axis;
    V3 t = cross(r, nn);
    float n3[3] = {nn.x, nn.y, nn.z}, t3[3] = {t.x, t.y, t.z};
#pragma unroll
    for (int x = 0; x < 3; x++) {
#pragma unroll
        for (int y = 0; y <= x; y++) {
            s.h[tri(x, y)] += pen * (n3[x] * n3[y]);
            s.h[tri(3 + x, 3 + y)] += pen * (t3[x] * t3[y]);
        }
#pragma unroll
        for (int y = 0; y < 3; y++) s.h[tri(3 + x, y)] += pen * (n3[y] * t3[x]);
    }
    s.r[0] += f * nn.x; s.r[1] += f * nn.y; s.r[2] += f * nn.z;
    s.r[3] += f * t.x; s.r[4] += f * t.y; s.r[5] += f * t.z;
}
// Pure angular row (assembly.rs:637-647 and the limit rows).
static __host__ __device__ __forceinline__ void stamp_angular(Sys& s, V3 g, float pen, float f) {
    float g3[3] = {g.x, g.y, g.z};
#pragma unroll
    for (int x = 0; x < 3; x++)
#pragma unroll
        for (int y = 0; y <= x; y++) s.h[tri(3 + x, 3 + y)] += pen * (g3[x] * g3[y]);
    s.r[3] += f * g.x; s.r[4] += f * g.y; s.r[5] += f * g.z;
}

// Dense LDL^T without pivoting (assembly.rs:25-69), as a factorisation and
// a solve: l holds the strict lower triangle of L row-major ((i, j), j < i,
// at i*(i-1)/2 + j), dg the pivots.  Returns false on a breakdown pivot
// (<= 1e-12); the body then skips its update.
static __host__ __device__ __forceinline__ int stri(int i, int j) { return i * (i - 1) / 2 + j; }
static __host__ __device__ __forceinline__ bool ldl_factor(const float h[21], float l[15], float dg[6]) {
#pragma unroll
    for (int i = 0; i < 6; i++) {
#pragma unroll
        for (int j = 0; j <= i; j++) {
            float v = h[tri(i, j)];
#pragma unroll
            for (int k = 0; k < j; k++) v -= l[stri(i, k)] * dg[k] * l[stri(j, k)];
            if (i == j) {
                if (v <= DEGENERATE_LEN2) return false;
                dg[i] = v;
            } else {
                l[stri(i, j)] = v / dg[j];
            }
        }
    }
    return true;
}
// x = -(L D L^T)^-1 r
static __host__ __device__ __forceinline__ void ldl_solve(const float l[15], const float dg[6], const float r[6],
                                                          float x[6]) {
    float y[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
        float v = -r[i];
#pragma unroll
        for (int k = 0; k < i; k++) v -= l[stri(i, k)] * y[k];
        y[i] = v;
    }
    float z[6];
#pragma unroll
    for (int i = 0; i < 6; i++) z[i] = y[i] / dg[i];
#pragma unroll
    for (int i = 5; i >= 0; i--) {
        float v = z[i];
#pragma unroll
        for (int k = i + 1; k < 6; k++) v -= l[stri(k, i)] * x[k];
        x[i] = v;
    }
}
static __host__ __device__ __forceinline__ bool solve_6x6(const Sys& s, float x[6]) {
    float l[15], dg[6];
    if (!ldl_factor(s.h, l, dg)) return false;
    ldl_solve(l, dg, s.r, x);
    return true;
}

// contact_force (rows.rs:1032-1060): push-only normal, elliptical cone.
static __host__ __device__ __forceinline__ void contact_force(float cn, float4 pen, float4 lam, float ct0, float ct1, float2 mu,
                                              float f[3]) {
    float fnc = fminf(pen.x * cn + lam.x, 0.0f);
    float fr0 = pen.y * ct0 + lam.y, fr1 = pen.z * ct1 + lam.z;
    float b1 = fabsf(fnc) * mu.x, b2 = fabsf(fnc) * mu.y;
    if (b1 <= 0.0f || b2 <= 0.0f) {
        f[0] = fnc;
        f[1] = b1 <= 0.0f ? 0.0f : fclamp(fr0, -b1, b1);
        f[2] = b2 <= 0.0f ? 0.0f : fclamp(fr1, -b2, b2);
        return;
    }
    float sq = (fr0 / b1) * (fr0 / b1) + (fr1 / b2) * (fr1 / b2);
    float k = sq > 1.0f ? 1.0f / sqrtf(sq) : 1.0f;
    f[0] = fnc;
    f[1] = fr0 * k;
    f[2] = fr1 * k;
}

// Per-pair body context for the Taylor residual C = C0(1-alpha) + u.(dA - dB)
// (rows.rs:1006-1025): step displacement and rotation vector of both sides.
struct PairCtx {
    V3 n;
    float gap;
    float2 mu;
    uint32_t a, b, np;
    V3 pa, pb;
    Q qa, qb;
    V3 dxa, dxb;    // x - x0
    V3 dra, drb;    // quat_diff_vec(q, q0)
    V3 t1, t2;      // friction frame (touching pairs)
    bool sph_a, sph_b;
    float rad_a, rad_b;
    float mu_roll, mu_spin;  // max of the two bodies' rolling / torsion friction
    bool roll_a, roll_b;     // adjoint: the side's witness anchor rolls (a capsule not against a box)
};

static __host__ __device__ __forceinline__ float row_c_levers(const PairCtx& c, V3 u, float c0, V3 raw, V3 rbw) {
    V3 da = c.dxa + u * dot(cross(raw, u), c.dra);
    V3 db = c.dxb + u * dot(cross(rbw, u), c.drb);
    return c0 * (1.0f - ALPHA) + dot(u, da - db);
}
static __host__ __device__ __forceinline__ void contact_levers(const PairCtx& c, float4 ra, float4 rb, V3& raw, V3& rbw) {  // :963-973
    raw = c.sph_a ? -c.n * c.rad_a : qrot(c.qa, ld3(ra));
    rbw = c.sph_b ? c.n * c.rad_b : qrot(c.qb, ld3(rb));
}
static __host__ __device__ __forceinline__ void friction_levers(const PairCtx& c, V3 raw, V3 rbw, V3& raf, V3& rbf) {  // :987-996
    float sep = dot((c.pa + raw) - (c.pb + rbw), c.n);
    raf = raw - c.n * (sep * HALF);
    rbf = rbw + c.n * (sep * HALF);
}
// Step-start normal violation of a point (joints_ext.rs:21-32).  It depends on
// the step-start poses only, so it is evaluated once per substep and kept in
// the w lane of the point's lambda record.
static __host__ __device__ __forceinline__ float gap_c0(bool sphere_pair, float gap, V3 n, V3 pa0, Q qa0, V3 pb0, Q qb0,
                                               float4 ra, float4 rb) {
    if (sphere_pair) return gap + MARGIN;
    V3 pa = pa0 + qrot(qa0, ld3(ra));
    V3 pb = pb0 + qrot(qb0, ld3(rb));
    return dot(n, pa - pb) + MARGIN;
}

}  // namespace avbd
