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

// ---- joints (assembly.rs:255-881 rows, joints_ext.rs:574-896 dual) ------------------
namespace avbd {

// One joint as a reversed body update sees it: its definition, the poses of
// both bodies (current and step start) and its warm state.
struct JDef {
    V3 la, lb, axa_l, axb_l;
    float ref;     // reference twist of the hinge
    bool revolute;
    float4 lim;    // lo, hi, has_limit (w unused)
};
struct JPose {
    V3 xa, xb, xa0, xb0;
    Q qa, qb, qa0, qb0;
};
struct JState {
    float4 laml, penl, lama, pena;
    float acc;  // the limit's accumulated force (j_lim.w)
};
AVBD_HD void jstate_zero(JState& s) {
    s.laml = s.penl = s.lama = s.pena = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    s.acc = 0.0f;
}
static __host__ __device__ __forceinline__ float f4get(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}
static __host__ __device__ __forceinline__ void f4add_at(float4& v, int k, float a) {
    if (k == 0) v.x += a;
    else if (k == 1) v.y += a;
    else if (k == 2) v.z += a;
    else v.w += a;
}

// A capsule's witness anchor (taken this substep, not kept from a stuck
// point, and not a box corner's projection) is the closest point of its
// rounded surface: segment point + s R0^T n in the body frame (s = -r on
// side A, +r on side B).  Held fixed as a material point instead, its
// lever would not roll with the body, and the linearised iteration of a
// capsule resting on its cap grows without bound; the anchor adjoint g
// therefore reaches the step-start orientation q0.
static __host__ __device__ __forceinline__ void rolling_anchor_bwd(Q q0, V3 n, float s, V3 g, Q& gq0) {
    Q gc = Q0();
    V3 dummy = V0();
    qrot_bwd(conj(q0), n, g * s, gc, dummy);
    gq0.x -= gc.x;
    gq0.y -= gc.y;
    gq0.z -= gc.z;
    gq0.w += gc.w;
}

// hinge_twist (sequential_impulse/joints.rs:38-48): 2 atan2(q.xyz . axis, q.w)
// of q = conj(qa) (x) qb, wrapped (the wrap is the identity almost everywhere).
// r2 = s^2 + w^2 = cos^2(swing / 2) of q's swing-twist split: as the hinge
// axes part by a half turn the twist angle loses its meaning and its
// derivative 2/r2 has no bound.  Past a swing of 120 degrees (r2 < 1/4) the
// angle is held fixed, as a contact frame is.
constexpr float TWIST_HELD_R2 = 0.25f;
static __host__ __device__ __forceinline__ void hinge_twist_bwd(Q qa, Q qb, V3 axis, float g, Q& gqa, Q& gqb) {
    Q q = qmul(conj(qa), qb);
    float s = dot(V3{q.x, q.y, q.z}, axis), w = q.w;
    float r2 = s * s + w * w;
    if (!(r2 >= TWIST_HELD_R2)) return;
    float k = 2.0f * g / r2;
    Q gq{axis.x * w * k, axis.y * w * k, axis.z * w * k, -s * k};
    Q gca = Q0();
    qmul_bwd(conj(qa), qb, gq, gca, gqb);
    gqa = qadd(gqa, conj(gca));
}
// tangent_t1 (math.rs:152-160): normalize(n x r) with r = X or Y by |n.x|;
// adds the adjoint of n.
static __host__ __device__ __forceinline__ void tangent_t1_bwd(V3 n, V3 gt, V3& gn) {
    V3 axis = fabsf(n.x) < TANGENT_REF_AXIS_DOT ? VX() : VY();
    V3 u = cross(n, axis);
    float l = len(u);
    if (!(l > 0.0f)) return;
    V3 t = u / l;
    V3 gu = (gt - t * dot(t, gt)) / l;
    gn = gn + cross(axis, gu);
}

// Adjoint of one stamped row for the solve's -d/ds [w.(rhs + H d)]
// (stamp_row and stamp_angular; see row_bwd in avbd_adjoint.cu).
static __host__ __device__ __forceinline__ void jrow_lin_bwd(V3 axis, float pen, float f, V3 r, float sign,
                                                             const float w6[6], const float d6[6], float& gf,
                                                             float& gpen, V3& gr) {
    V3 nn = sign * axis;
    V3 t = cross(r, nn);
    V3 wl{w6[0], w6[1], w6[2]}, wa{w6[3], w6[4], w6[5]};
    V3 dl{d6[0], d6[1], d6[2]}, da{d6[3], d6[4], d6[5]};
    float a = dot(nn, wl) + dot(t, wa);
    float dd = dot(nn, dl) + dot(t, da);
    gf -= a;
    gpen -= a * dd;
    V3 gja = -(wa * f + (wa * dd + da * a) * pen);
    gr = gr + cross(nn, gja);
}
static __host__ __device__ __forceinline__ void jrow_ang_bwd(V3 g, float pen, float f, const float w6[6],
                                                             const float d6[6], float& gf, float& gpen, V3& gg) {
    V3 wa{w6[3], w6[4], w6[5]}, da{d6[3], d6[4], d6[5]};
    float a = dot(g, wa), dd = dot(g, da);
    gf -= a;
    gpen -= a * dd;
    gg = gg - (wa * f + (wa * dd + da * a) * pen);
}

// The hinge frame of a joint at its step-start pose: t1, t2 from axa0.
static __host__ __device__ __forceinline__ void hinge_frame(V3 axa0, V3& t1, V3& t2) {
    t1 = tangent_t1(axa0);
    t2 = cross(t1, axa0);
}
// adjoint of (t1, t2) -> axa0
static __host__ __device__ __forceinline__ void hinge_frame_bwd(V3 axa0, V3 t1, V3 gt1, V3 gt2, V3& gaxa0) {
    // t2 = t1 x axa0
    gt1 = gt1 + cross(axa0, gt2);
    gaxa0 = gaxa0 + cross(gt2, t1);
    tangent_t1_bwd(axa0, gt1, gaxa0);
}

// The joint rows of one body (the forward stamp_joint of avbd_phase_solve.cu).
static __host__ __device__ __forceinline__ void joint_stamp(const JDef& d, const JPose& p, const JState& s, bool is_a,
                                                            Sys& sys) {
    float sign = is_a ? 1.0f : -1.0f;
    V3 pa = p.xa + qrot(p.qa, d.la), pb = p.xb + qrot(p.qb, d.lb);
    V3 pa0 = p.xa0 + qrot(p.qa0, d.la), pb0 = p.xb0 + qrot(p.qb0, d.lb);
    V3 live = pa - pb, c0v = pa0 - pb0;
    V3 lever = is_a ? qrot(p.qa, d.la) : qrot(p.qb, d.lb);
    float fl[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; k++) {
        V3 axis = V0();
        axis[k] = 1.0f;
        float cc = live[k] - ALPHA * c0v[k];
        float f = f4get(s.penl, k) * cc + f4get(s.laml, k);
        if (!row_live(cc, f)) continue;
        stamp_row(sys, axis, f4get(s.penl, k), f, lever, sign);
        fl[k] = f;
    }
    {
        V3 r = is_a ? qrot(p.qa, d.la) : -qrot(p.qb, d.lb);
        float rf = dot(r, V3{fl[0], fl[1], fl[2]});
        for (int y = 0; y < 3; y++) {
            V3 col = r * fl[y];
            col[y] -= rf;
            sys.h[tri(3 + y, 3 + y)] += len(col);
        }
    }
    if (!d.revolute) return;
    V3 axa = qrot(p.qa, d.axa_l), axb = qrot(p.qb, d.axb_l);
    V3 axa0 = qrot(p.qa0, d.axa_l), axb0 = qrot(p.qb0, d.axb_l);
    V3 t1, t2;
    hinge_frame(axa0, t1, t2);
    V3 ts[2] = {t1, t2};
    for (int li = 0; li < 2; li++) {
        float cc = dot(ts[li], axa - axb) - ALPHA * dot(ts[li], axa0 - axb0);
        float f = f4get(s.pena, li) * cc + f4get(s.lama, li);
        if (!row_live(cc, f)) continue;
        stamp_angular(sys, is_a ? cross(axa, ts[li]) : -cross(axb, ts[li]), f4get(s.pena, li), f);
    }
    if (d.lim.z != 0.0f) {
        V3 wa = normalize_or(axa, VZ());
        float angle = wrap_pi(hinge_twist(p.qa, p.qb, d.axa_l) - d.ref);
        int stt = warm_limit_state(angle, d.lim.x, d.lim.y, LIMIT_SLOP_ANG, s.acc);
        if (stt >= 0) {
            bool lower = stt == 1;
            float initial = wrap_pi(hinge_twist(p.qa0, p.qb0, d.axa_l) - d.ref);
            float cc = regularized_limit(angle, initial, lower ? d.lim.x : d.lim.y, lower);
            float f_raw = s.pena.z * cc + s.acc;
            float f = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
            if (row_live(cc, f)) stamp_angular(sys, is_a ? -wa : wa, s.pena.z, f);
        }
    }
}

// Adjoint of joint_stamp for the body on side is_a, given w = H^-1 d_bar and
// the step d of that body: adds the adjoints of both bodies' poses (g) and
// of the joint's warm state (gs).
static __host__ __device__ __forceinline__ void joint_stamp_bwd(const JDef& d, const JPose& p, const JState& s,
                                                                bool is_a, const float w6[6], const float d6[6],
                                                                PairGrad& g, JState& gs) {
    float sign = is_a ? 1.0f : -1.0f;
    V3 pa = p.xa + qrot(p.qa, d.la), pb = p.xb + qrot(p.qb, d.lb);
    V3 pa0 = p.xa0 + qrot(p.qa0, d.la), pb0 = p.xb0 + qrot(p.qb0, d.lb);
    V3 live = pa - pb, c0v = pa0 - pb0;
    V3 lever = is_a ? qrot(p.qa, d.la) : qrot(p.qb, d.lb);
    V3 glive = V0(), gc0v = V0(), glever = V0();
    float fl[3] = {0.0f, 0.0f, 0.0f}, cs[3] = {0.0f, 0.0f, 0.0f};
    bool liv[3] = {false, false, false};
    float gfl[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; k++) {
        float cc = live[k] - ALPHA * c0v[k];
        float f = f4get(s.penl, k) * cc + f4get(s.laml, k);
        cs[k] = cc;
        if (!row_live(cc, f)) continue;
        liv[k] = true;
        fl[k] = f;
        V3 axis = V0();
        axis[k] = 1.0f;
        float gpen = 0.0f;
        jrow_lin_bwd(axis, f4get(s.penl, k), f, lever, sign, w6, d6, gfl[k], gpen, glever);
        f4add_at(gs.penl, k, gpen);
    }
    {
        // geometric stiffness: H[3+y][3+y] += |col_y|, col_y = r fl_y - (r.fl) e_y
        V3 r = is_a ? qrot(p.qa, d.la) : -qrot(p.qb, d.lb);
        V3 flv{fl[0], fl[1], fl[2]};
        float rf = dot(r, flv);
        V3 gr = V0(), gflv = V0();
        for (int y = 0; y < 3; y++) {
            V3 col = r * fl[y];
            col[y] -= rf;
            float l = len(col);
            if (!(l > 0.0f)) continue;
            float c = -w6[3 + y] * d6[3 + y];
            V3 gcol = col * (c / l);
            // col[x] = r_x fl_y - rf delta_xy
            gr = gr + gcol * fl[y] - flv * gcol[y];
            gflv[y] += dot(gcol, r);
            gflv = gflv - r * gcol[y];
        }
        for (int k = 0; k < 3; k++) gfl[k] += gflv[k];
        V3 dummy = V0();
        if (is_a) qrot_bwd(p.qa, d.la, gr, g.qa, dummy);
        else qrot_bwd(p.qb, d.lb, -gr, g.qb, dummy);
    }
    for (int k = 0; k < 3; k++) {
        if (!liv[k]) continue;
        // f = pen c + lambda, c = live_k - alpha c0v_k
        float gc = f4get(s.penl, k) * gfl[k];
        f4add_at(gs.penl, k, cs[k] * gfl[k]);
        f4add_at(gs.laml, k, gfl[k]);
        glive[k] += gc;
        gc0v[k] -= ALPHA * gc;
    }
    {
        V3 dummy = V0();
        if (is_a) qrot_bwd(p.qa, d.la, glever, g.qa, dummy);
        else qrot_bwd(p.qb, d.lb, glever, g.qb, dummy);
        g.xa = g.xa + glive;
        qrot_bwd(p.qa, d.la, glive, g.qa, dummy);
        g.xb = g.xb - glive;
        qrot_bwd(p.qb, d.lb, -glive, g.qb, dummy);
        g.xa0 = g.xa0 + gc0v;
        qrot_bwd(p.qa0, d.la, gc0v, g.qa0, dummy);
        g.xb0 = g.xb0 - gc0v;
        qrot_bwd(p.qb0, d.lb, -gc0v, g.qb0, dummy);
    }
    if (!d.revolute) return;
    V3 axa = qrot(p.qa, d.axa_l), axb = qrot(p.qb, d.axb_l);
    V3 axa0 = qrot(p.qa0, d.axa_l), axb0 = qrot(p.qb0, d.axb_l);
    V3 t1, t2;
    hinge_frame(axa0, t1, t2);
    V3 ts[2] = {t1, t2};
    V3 gaxa = V0(), gaxb = V0(), gaxa0 = V0(), gaxb0 = V0(), gts[2] = {V0(), V0()};
    for (int li = 0; li < 2; li++) {
        float cc = dot(ts[li], axa - axb) - ALPHA * dot(ts[li], axa0 - axb0);
        float pen = f4get(s.pena, li);
        float f = pen * cc + f4get(s.lama, li);
        if (!row_live(cc, f)) continue;
        V3 gv = is_a ? cross(axa, ts[li]) : -cross(axb, ts[li]);
        float gf = 0.0f, gpen = 0.0f;
        V3 ggv = V0();
        jrow_ang_bwd(gv, pen, f, w6, d6, gf, gpen, ggv);
        if (is_a) {
            gaxa = gaxa + cross(ts[li], ggv);
            gts[li] = gts[li] + cross(ggv, axa);
        } else {
            gaxb = gaxb - cross(ts[li], ggv);
            gts[li] = gts[li] - cross(ggv, axb);
        }
        float gc = pen * gf;
        f4add_at(gs.pena, li, gpen + cc * gf);
        f4add_at(gs.lama, li, gf);
        gts[li] = gts[li] + ((axa - axb) - (axa0 - axb0) * ALPHA) * gc;
        gaxa = gaxa + ts[li] * gc;
        gaxb = gaxb - ts[li] * gc;
        gaxa0 = gaxa0 - ts[li] * (ALPHA * gc);
        gaxb0 = gaxb0 + ts[li] * (ALPHA * gc);
    }
    if (d.lim.z != 0.0f) {
        V3 wa = normalize_or(axa, VZ());
        float angle = wrap_pi(hinge_twist(p.qa, p.qb, d.axa_l) - d.ref);
        int stt = warm_limit_state(angle, d.lim.x, d.lim.y, LIMIT_SLOP_ANG, s.acc);
        if (stt >= 0) {
            bool lower = stt == 1;
            float bound = lower ? d.lim.x : d.lim.y;
            float initial = wrap_pi(hinge_twist(p.qa0, p.qb0, d.axa_l) - d.ref);
            float cc = regularized_limit(angle, initial, bound, lower);
            float f_raw = s.pena.z * cc + s.acc;
            float f = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
            if (row_live(cc, f)) {
                float gf = 0.0f, gpen = 0.0f;
                V3 gwv = V0();
                jrow_ang_bwd(is_a ? -wa : wa, s.pena.z, f, w6, d6, gf, gpen, gwv);
                gs.pena.z += gpen;
                V3 gwa = is_a ? -gwv : gwv;
                float la = len(axa);
                if (la > 0.0f) gaxa = gaxa + (gwa - wa * dot(wa, gwa)) / la;
                bool pass = lower ? f_raw < 0.0f : f_raw > 0.0f;
                if (pass) {
                    float gc = s.pena.z * gf;
                    gs.pena.z += cc * gf;
                    gs.acc += gf;
                    float old = initial - bound;
                    bool active = lower ? old < 0.0f : old > 0.0f;
                    hinge_twist_bwd(p.qa, p.qb, d.axa_l, gc, g.qa, g.qb);
                    if (active) hinge_twist_bwd(p.qa0, p.qb0, d.axa_l, -ALPHA * gc, g.qa0, g.qb0);
                }
            }
        }
    }
    hinge_frame_bwd(axa0, t1, gts[0], gts[1], gaxa0);
    V3 dummy = V0();
    qrot_bwd(p.qa, d.axa_l, gaxa, g.qa, dummy);
    qrot_bwd(p.qb, d.axb_l, gaxb, g.qb, dummy);
    qrot_bwd(p.qa0, d.axa_l, gaxa0, g.qa0, dummy);
    qrot_bwd(p.qb0, d.axb_l, gaxb0, g.qb0, dummy);
}

// The joint dual update (k_dual_joints) with finite stiffness K (0: hard).
static __host__ __device__ __forceinline__ void joint_dual(const JDef& d, const JPose& p, const JState& in, float K,
                                                           JState& out) {
    out = in;
    V3 pa = p.xa + qrot(p.qa, d.la), pb = p.xb + qrot(p.qb, d.lb);
    V3 pa0 = p.xa0 + qrot(p.qa0, d.la), pb0 = p.xb0 + qrot(p.qb0, d.lb);
    V3 live = pa - pb, c0v = pa0 - pb0;
    for (int k = 0; k < 3; k++) {
        float cc = live[k] - ALPHA * c0v[k];
        float pen = f4get(in.penl, k);
        if (K > 0.0f) {
            f4add_at(out.penl, k, K - pen);
            continue;
        }
        if (fabsf(cc) < C_EPS) continue;
        f4add_at(out.laml, k, pen * cc);
        f4add_at(out.penl, k, fminf(pen + BETA * fabsf(cc), PENALTY_MAX) - pen);
    }
    if (!d.revolute) return;
    V3 axa = qrot(p.qa, d.axa_l), axb = qrot(p.qb, d.axb_l);
    V3 axa0 = qrot(p.qa0, d.axa_l), axb0 = qrot(p.qb0, d.axb_l);
    V3 t1, t2;
    hinge_frame(axa0, t1, t2);
    V3 ts[2] = {t1, t2};
    for (int li = 0; li < 2; li++) {
        float cc = dot(ts[li], axa - axb) - ALPHA * dot(ts[li], axa0 - axb0);
        float pen = f4get(in.pena, li);
        if (K > 0.0f) {
            f4add_at(out.pena, li, K - pen);
            continue;
        }
        if (fabsf(cc) < C_EPS) continue;
        f4add_at(out.lama, li, pen * cc);
        f4add_at(out.pena, li, fminf(pen + BETA_ANG * fabsf(cc), PENALTY_MAX) - pen);
    }
    if (d.lim.z != 0.0f) {
        float angle = wrap_pi(hinge_twist(p.qa, p.qb, d.axa_l) - d.ref);
        int stt = warm_limit_state(angle, d.lim.x, d.lim.y, LIMIT_SLOP_ANG, in.acc);
        if (stt >= 0) {
            bool lower = stt == 1;
            float initial = wrap_pi(hinge_twist(p.qa0, p.qb0, d.axa_l) - d.ref);
            float cc = regularized_limit(angle, initial, lower ? d.lim.x : d.lim.y, lower);
            if (fabsf(cc) >= C_EPS) {
                float f = in.pena.z * cc + in.acc;
                out.acc = lower ? fminf(f, 0.0f) : fmaxf(f, 0.0f);
                out.pena.z = fminf(in.pena.z + BETA_ANG * fabsf(cc), LIM_PEN_MAX);
            }
        } else {
            out.acc = 0.0f;
        }
    }
}

// Adjoint of joint_dual: gout (adjoint of the state after) -> gin (before),
// the poses (g) and the stiffness (gK).
static __host__ __device__ __forceinline__ void joint_dual_bwd(const JDef& d, const JPose& p, const JState& in, float K,
                                                               const JState& gout, JState& gin, PairGrad& g,
                                                               float& gK) {
    gin = gout;
    V3 pa = p.xa + qrot(p.qa, d.la), pb = p.xb + qrot(p.qb, d.lb);
    V3 pa0 = p.xa0 + qrot(p.qa0, d.la), pb0 = p.xb0 + qrot(p.qb0, d.lb);
    V3 live = pa - pb, c0v = pa0 - pb0;
    V3 glive = V0(), gc0v = V0();
    for (int k = 0; k < 3; k++) {
        float cc = live[k] - ALPHA * c0v[k];
        float pen = f4get(in.penl, k);
        float gl = f4get(gout.laml, k), gp = f4get(gout.penl, k);
        if (K > 0.0f) {  // penalty := K (the pass-through copied into gin is undone)
            f4add_at(gin.penl, k, -gp);
            gK += gp;
            continue;
        }
        if (fabsf(cc) < C_EPS) continue;
        float gc = 0.0f;
        if (!(pen + BETA * fabsf(cc) < PENALTY_MAX)) f4add_at(gin.penl, k, -gp);
        else gc += BETA * copysignf(1.0f, cc) * gp;
        f4add_at(gin.penl, k, cc * gl);  // lambda += pen c
        gc += pen * gl;
        glive[k] += gc;
        gc0v[k] -= ALPHA * gc;
    }
    {
        V3 dummy = V0();
        g.xa = g.xa + glive;
        qrot_bwd(p.qa, d.la, glive, g.qa, dummy);
        g.xb = g.xb - glive;
        qrot_bwd(p.qb, d.lb, -glive, g.qb, dummy);
        g.xa0 = g.xa0 + gc0v;
        qrot_bwd(p.qa0, d.la, gc0v, g.qa0, dummy);
        g.xb0 = g.xb0 - gc0v;
        qrot_bwd(p.qb0, d.lb, -gc0v, g.qb0, dummy);
    }
    if (!d.revolute) return;
    V3 axa = qrot(p.qa, d.axa_l), axb = qrot(p.qb, d.axb_l);
    V3 axa0 = qrot(p.qa0, d.axa_l), axb0 = qrot(p.qb0, d.axb_l);
    V3 t1, t2;
    hinge_frame(axa0, t1, t2);
    V3 ts[2] = {t1, t2};
    V3 gaxa = V0(), gaxb = V0(), gaxa0 = V0(), gaxb0 = V0(), gts[2] = {V0(), V0()};
    for (int li = 0; li < 2; li++) {
        float cc = dot(ts[li], axa - axb) - ALPHA * dot(ts[li], axa0 - axb0);
        float pen = f4get(in.pena, li);
        float gl = f4get(gout.lama, li), gp = f4get(gout.pena, li);
        if (K > 0.0f) {
            f4add_at(gin.pena, li, -gp);
            gK += gp;
            continue;
        }
        if (fabsf(cc) < C_EPS) continue;
        float gc = 0.0f;
        if (!(pen + BETA_ANG * fabsf(cc) < PENALTY_MAX)) f4add_at(gin.pena, li, -gp);
        else gc += BETA_ANG * copysignf(1.0f, cc) * gp;
        f4add_at(gin.pena, li, cc * gl);
        gc += pen * gl;
        gts[li] = gts[li] + ((axa - axb) - (axa0 - axb0) * ALPHA) * gc;
        gaxa = gaxa + ts[li] * gc;
        gaxb = gaxb - ts[li] * gc;
        gaxa0 = gaxa0 - ts[li] * (ALPHA * gc);
        gaxb0 = gaxb0 + ts[li] * (ALPHA * gc);
    }
    if (d.lim.z != 0.0f) {
        float angle = wrap_pi(hinge_twist(p.qa, p.qb, d.axa_l) - d.ref);
        int stt = warm_limit_state(angle, d.lim.x, d.lim.y, LIMIT_SLOP_ANG, in.acc);
        if (stt >= 0) {
            bool lower = stt == 1;
            float bound = lower ? d.lim.x : d.lim.y;
            float initial = wrap_pi(hinge_twist(p.qa0, p.qb0, d.axa_l) - d.ref);
            float cc = regularized_limit(angle, initial, bound, lower);
            if (fabsf(cc) >= C_EPS) {
                float gacc = gout.acc, gp = gout.pena.z;
                gin.acc = 0.0f;  // overwritten
                gin.pena.z = 0.0f;
                float gc = 0.0f;
                float f = in.pena.z * cc + in.acc;
                if (lower ? f < 0.0f : f > 0.0f) {
                    gin.pena.z += cc * gacc;
                    gin.acc += gacc;
                    gc += in.pena.z * gacc;
                }
                if (in.pena.z + BETA_ANG * fabsf(cc) < LIM_PEN_MAX) {
                    gin.pena.z += gp;
                    gc += BETA_ANG * copysignf(1.0f, cc) * gp;
                }
                float old = initial - bound;
                bool active = lower ? old < 0.0f : old > 0.0f;
                hinge_twist_bwd(p.qa, p.qb, d.axa_l, gc, g.qa, g.qb);
                if (active) hinge_twist_bwd(p.qa0, p.qb0, d.axa_l, -ALPHA * gc, g.qa0, g.qb0);
            }
        } else {
            gin.acc = 0.0f;
        }
    }
    hinge_frame_bwd(axa0, t1, gts[0], gts[1], gaxa0);
    V3 dummy = V0();
    qrot_bwd(p.qa, d.axa_l, gaxa, g.qa, dummy);
    qrot_bwd(p.qb, d.axb_l, gaxb, g.qb, dummy);
    qrot_bwd(p.qa0, d.axa_l, gaxa0, g.qa0, dummy);
    qrot_bwd(p.qb0, d.axb_l, gaxb0, g.qb0, dummy);
}

}  // namespace avbd
