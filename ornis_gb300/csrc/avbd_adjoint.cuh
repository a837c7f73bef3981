// avbd_adjoint.cuh — vector-Jacobian products of the AVBD step's arithmetic,
// for the adjoint (reverse-mode) kernels in avbd_adjoint.cu.
//
// Each *_bwd function takes the forward inputs and the adjoint of the
// forward output and ADDS the adjoints of the inputs to its reference
// arguments.  The forward functions are the ones in avbd_vec.cuh and
// avbd_rows.cuh (glam operation order, crates/physics/src/avbd/rows.rs);
// the derivatives below are the plain calculus of those formulas.
#pragma once
#include "avbd_rows.cuh"

namespace avbd {

AVBD_HD V3 vadd(V3 a, V3 b) { return a + b; }
AVBD_HD Q qadd(Q a, Q b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
AVBD_HD Q qscale(Q a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
AVBD_HD float qdot(Q a, Q b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
AVBD_HD Q Q0() { return {0.0f, 0.0f, 0.0f, 0.0f}; }

// y = qrot(q, v) = v (w^2 - b.b) + 2 b (v.b) + 2 w (b x v),  b = q.xyz
static __host__ __device__ __forceinline__ void qrot_bwd(Q q, V3 v, V3 g, Q& gq, V3& gv) {
    V3 b{q.x, q.y, q.z};
    float s = q.w * q.w - dot(b, b);
    gv = gv + g * s + b * (2.0f * dot(b, g)) + cross(g, b) * (2.0f * q.w);
    float vg = dot(v, g), vb = dot(v, b), bg = dot(b, g);
    V3 gb = b * (-2.0f * vg) + g * (2.0f * vb) + v * (2.0f * bg) + cross(v, g) * (2.0f * q.w);
    gq.x += gb.x;
    gq.y += gb.y;
    gq.z += gb.z;
    gq.w += dot(g, v * (2.0f * q.w) + cross(b, v) * 2.0f);
}
// p = a (x) b: ga = g (x) conj(b), gb = conj(a) (x) g
static __host__ __device__ __forceinline__ void qmul_bwd(Q a, Q b, Q g, Q& ga, Q& gb) {
    ga = qadd(ga, qmul(g, conj(b)));
    gb = qadd(gb, qmul(conj(a), g));
}
// n = q / |q|
static __host__ __device__ __forceinline__ Q qnormalize_bwd(Q q, Q g) {
    float l = sqrtf((q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w));
    float il = 1.0f / l;
    Q n = qscale(q, il);
    float ng = qdot(n, g);
    return {(g.x - n.x * ng) * il, (g.y - n.y * ng) * il, (g.z - n.z * ng) * il, (g.w - n.w * ng) * il};
}

// quat_integrate (rows.rs:110-119): out = normalize((v k, cos(t/2)) (x) q),
// t = |v|, k = sin(t/2)/t; the identity below NEAR_ZERO.
static __host__ __device__ __forceinline__ void quat_integrate_bwd(Q q, V3 v, Q g, Q& gq, V3& gv) {
    float t = len(v);
    if (t < NEAR_ZERO) {
        gq = qadd(gq, g);
        return;
    }
    float s, c;
    sincosf(HALF * t, &s, &c);
    float k = s / t;
    Q e{v.x * k, v.y * k, v.z * k, c};
    Q d = qmul(e, q);
    Q gd = qnormalize_bwd(d, g);
    Q ge = Q0();
    qmul_bwd(e, q, gd, ge, gq);
    // dk/dt / t: (t cos(t/2)/2 - sin(t/2)) / t^3, by its series for small t
    float kp;
    if (t < 1e-2f) {
        float t2 = t * t;
        kp = -1.0f / 24.0f + t2 / 960.0f;
    } else {
        kp = (t * c * HALF - s) / (t * t * t);
    }
    V3 gexyz{ge.x, ge.y, ge.z};
    gv = gv + gexyz * k + v * (dot(gexyz, v) * kp) - v * (ge.w * k * HALF);
}

// quat_diff_vec (rows.rs:128-146): r = a (x) conj(b); u = +-r.xyz (sign of
// r.w); s = min(|u|, 1); out = u * 2 asin(s)/s, zero below NEAR_ZERO.
static __host__ __device__ __forceinline__ void quat_diff_vec_bwd(Q a, Q b, V3 g, Q& ga, Q& gb) {
    Q r = qmul(a, conj(b));
    float sg = r.w < 0.0f ? -1.0f : 1.0f;
    V3 u{r.x * sg, r.y * sg, r.z * sg};
    float lu = len(u);
    float s = fminf(lu, 1.0f);
    if (s < NEAR_ZERO) return;
    V3 gu;
    if (lu >= 1.0f) {
        gu = g * (2.0f * asinf(1.0f));
    } else {
        float f = 2.0f * asinf(s) / s;
        // f'(s)/s = 2 (s/sqrt(1 - s^2) - asin(s)) / s^3, by its series for small s
        float fp;
        if (s < 1e-2f) fp = 2.0f / 3.0f + 0.6f * s * s;
        else fp = 2.0f * (s / sqrtf(1.0f - s * s) - asinf(s)) / (s * s * s);
        gu = g * f + u * (dot(g, u) * fp);
    }
    Q gr{gu.x * sg, gu.y * sg, gu.z * sg, 0.0f};
    Q gcb = Q0();
    qmul_bwd(a, conj(b), gr, ga, gcb);
    gb = qadd(gb, conj(gcb));
}

// Columns of the rotation matrix (glam Mat3::from_quat, avbd_vec.cuh
// mat3_cols): adjoint of the quaternion from the columns' adjoints.
static __host__ __device__ __forceinline__ void mat3_cols_bwd(Q q, const V3 gc[3], Q& gq) {
    float x = q.x, y = q.y, z = q.z, w = q.w;
    gq.x += 2.0f * (y * gc[0].y + z * gc[0].z + y * gc[1].x - 2.0f * x * gc[1].y + w * gc[1].z + z * gc[2].x -
                    w * gc[2].y - 2.0f * x * gc[2].z);
    gq.y += 2.0f * (-2.0f * y * gc[0].x + x * gc[0].y - w * gc[0].z + x * gc[1].x + z * gc[1].z + w * gc[2].x +
                    z * gc[2].y - 2.0f * y * gc[2].z);
    gq.z += 2.0f * (-2.0f * z * gc[0].x + w * gc[0].y + x * gc[0].z - w * gc[1].x - 2.0f * z * gc[1].y + y * gc[1].z +
                    x * gc[2].x + y * gc[2].y);
    gq.w += 2.0f * (z * gc[0].y - y * gc[0].z - z * gc[1].x + x * gc[1].z + y * gc[2].x - x * gc[2].y);
}
// psi = u^T Iw(q) v with Iw = sum_k I_k c_k c_k^T (rows.rs:194-207)
static __host__ __device__ __forceinline__ void world_inertia_bwd(V3 inertia, Q q, V3 u, V3 v, float scale, Q& gq) {
    V3 c[3];
    mat3_cols(q, c);
    float ik[3] = {inertia.x, inertia.y, inertia.z};
    V3 gc[3];
#pragma unroll
    for (int k = 0; k < 3; k++) gc[k] = (u * dot(c[k], v) + v * dot(u, c[k])) * (ik[k] * scale);
    mat3_cols_bwd(q, gc, gq);
}

// contact_force (rows.rs:1032-1060) adjoint.  gf: adjoints of the three
// force components; adds to gcn, gpen, glam, gct0/gct1, gmu.
static __host__ __device__ __forceinline__ void contact_force_bwd(float cn, float4 pen, float4 lam, float ct0, float ct1,
                                                         float2 mu, const float gf[3], float& gcn, float4& gpen,
                                                         float4& glam, float& gct0, float& gct1, float2& gmu) {
    float fn_raw = pen.x * cn + lam.x;
    float fnc = fminf(fn_raw, 0.0f);
    float fr0 = pen.y * ct0 + lam.y, fr1 = pen.z * ct1 + lam.z;
    float afn = fabsf(fnc);
    float b1 = afn * mu.x, b2 = afn * mu.y;
    float gfnc = gf[0], gfr0 = 0.0f, gfr1 = 0.0f, gb1 = 0.0f, gb2 = 0.0f;
    if (b1 <= 0.0f || b2 <= 0.0f) {
        if (b1 > 0.0f) {
            if (fr0 < -b1) gb1 -= gf[1];
            else if (fr0 > b1) gb1 += gf[1];
            else gfr0 += gf[1];
        }
        if (b2 > 0.0f) {
            if (fr1 < -b2) gb2 -= gf[2];
            else if (fr1 > b2) gb2 += gf[2];
            else gfr1 += gf[2];
        }
    } else {
        float q0 = fr0 / b1, q1 = fr1 / b2;
        float sq = q0 * q0 + q1 * q1;
        if (sq > 1.0f) {
            float k = 1.0f / sqrtf(sq);
            float gk = gf[1] * fr0 + gf[2] * fr1;
            gfr0 += gf[1] * k;
            gfr1 += gf[2] * k;
            float gsq = -0.5f * gk * k * k * k;
            gfr0 += gsq * 2.0f * q0 / b1;
            gfr1 += gsq * 2.0f * q1 / b2;
            gb1 += gsq * (-2.0f * q0 * q0 / b1);
            gb2 += gsq * (-2.0f * q1 * q1 / b2);
        } else {
            gfr0 += gf[1];
            gfr1 += gf[2];
        }
    }
    // b1 = |fnc| mu.x, b2 = |fnc| mu.y; fnc <= 0, so |fnc| = -fnc
    gmu.x += gb1 * afn;
    gmu.y += gb2 * afn;
    gfnc -= gb1 * mu.x + gb2 * mu.y;
    if (fn_raw < 0.0f) {
        gcn += pen.x * gfnc;
        gpen.x += cn * gfnc;
        glam.x += gfnc;
    }
    gct0 += pen.y * gfr0;
    gpen.y += ct0 * gfr0;
    glam.y += gfr0;
    gct1 += pen.z * gfr1;
    gpen.z += ct1 * gfr1;
    glam.z += gfr1;
}

// Per-pair kinematics as one body sees them, with the adjoints they collect.
struct PairGrad {
    V3 xa, xb;    // pose adjoints (position)
    Q qa, qb;     //                (orientation)
    V3 xa0, xb0;  // step-start pose adjoints
    Q qa0, qb0;
};
static __host__ __device__ __forceinline__ void pair_grad_zero(PairGrad& g) {
    g.xa = g.xb = g.xa0 = g.xb0 = V0();
    g.qa = g.qb = g.qa0 = g.qb0 = Q0();
}

// row_c_levers (rows.rs:1006-1025) adjoint, axis u held fixed:
// C = c0 (1 - alpha) + u.dxa - u.dxb + (u.u)(raw.(u x dra) - rbw.(u x drb)).
// dx = x - x0 and dr = quat_diff_vec(q, q0) are expanded into the poses.
static __host__ __device__ __forceinline__ void row_c_bwd(const PairCtx& c, const Q& qa0, const Q& qb0, V3 u, V3 raw, V3 rbw,
                                                 float gC, float& gc0, V3& graw, V3& grbw, PairGrad& pg) {
    gc0 += (1.0f - ALPHA) * gC;
    V3 gdxa = u * gC, gdxb = u * (-gC);
    float uu = dot(u, u);
    float gsa = uu * gC, gsb = -uu * gC;
    graw = graw + cross(u, c.dra) * gsa;
    grbw = grbw + cross(u, c.drb) * gsb;
    V3 gdra = cross(raw, u) * gsa, gdrb = cross(rbw, u) * gsb;
    pg.xa = pg.xa + gdxa;
    pg.xa0 = pg.xa0 - gdxa;
    pg.xb = pg.xb + gdxb;
    pg.xb0 = pg.xb0 - gdxb;
    quat_diff_vec_bwd(c.qa, qa0, gdra, pg.qa, pg.qa0);
    quat_diff_vec_bwd(c.qb, qb0, gdrb, pg.qb, pg.qb0);
}

}  // namespace avbd
