// avbd_phase_solve.cu — the AVBD iterations: per-colour primal block solves,
// the order-free dual update, then BDF1 velocities and sleep bookkeeping.
//
// Reference: crates/physics/src/avbd/assembly.rs:73-903 (solve_body),
// avbd/joints_ext.rs:464-919 (dual_update), avbd/mod.rs:1060-1142 (BDF1,
// sleep, driver baseline), avbd/sleep.rs:140-175.
#include "avbd_common.cuh"

// This file is compiled twice: the exact build (-fmad=false, IEEE divide and
// square root) reproduces the CPU oracle bit for bit with one thread per
// body; the fast build (-DAVBD_SOLVE_FAST: contracted multiply-adds,
// approximate divide and square root) stays within the 1e-5 pose tolerance
// and is what the benchmark runs.  Discovery is exact in both.
#ifdef AVBD_SOLVE_FAST
#define AVBD_SOLVE_NS fast
#else
#define AVBD_SOLVE_NS exact
#endif

namespace avbd {
namespace AVBD_SOLVE_NS {

static __device__ __forceinline__ void load_ctx(const DW& w, uint32_t p, PairCtx& c) {
    uint2 ab = w.p_ab[p];
    float4 n4 = w.p_n[p];
    c.a = ab.x;
    c.b = ab.y;
    c.n = ld3(n4);
    c.gap = n4.w;
    c.mu = w.p_mu[p];
    c.np = w.p_np[p];
    const float4* ka = w.kin + (size_t)c.a * 4;
    const float4* kb = w.kin + (size_t)c.b * 4;
    float4 a0 = ka[0], a1 = ka[1], a2 = ka[2], a3 = ka[3];
    float4 b0 = kb[0], b1 = kb[1], b2 = kb[2], b3 = kb[3];
    c.pa = ld3(a0);
    c.pb = ld3(b0);
    c.qa = ldq(a1);
    c.qb = ldq(b1);
    c.dxa = ld3(a2);
    c.dxb = ld3(b2);
    c.dra = ld3(a3);
    c.drb = ld3(b3);
    c.sph_a = info_shape(__float_as_uint(a2.w)) == AVBD_SHAPE_SPHERE;
    c.sph_b = info_shape(__float_as_uint(b2.w)) == AVBD_SHAPE_SPHERE;
    c.rad_a = a0.w;
    c.rad_b = b0.w;
    float4 ma = w.mat[c.a], mb = w.mat[c.b];
    c.mu_roll = fmaxf(ma.z, mb.z);
    c.mu_spin = fmaxf(ma.w, mb.w);
    if (c.gap <= 0.0f) {
        c.t1 = tangent_t1(c.n);
        c.t2 = cross(c.t1, c.n);
    }
}

// Rows of point k of pair p for the body on side is_a (assembly.rs:99-252).
static __device__ __forceinline__ void stamp_point(const DW& w, const PairCtx& c, uint32_t p, uint32_t k, bool is_a,
                                                   Sys& s) {
    uint32_t q = p * MAX_PTS + k;
    float4 ra = w.q_ra[q], rb = w.q_rb[q];
    float4 lam = w.q_lam[q];
    float sign = is_a ? 1.0f : -1.0f;
    bool touching = c.gap <= 0.0f;
    float c0 = touching ? lam.w : 0.0f;
    V3 rup, rlo;
    contact_levers(c, ra, rb, rup, rlo);
    float cn = row_c_levers(c, c.n, c0, rup, rlo);
    V3 r_side = is_a ? rup : rlo;
    if (!touching) {
        // separated damper, imminence-gated (assembly.rs:113-175)
        float approach = fmaxf(dot(ld3(w.vel[c.b]) - ld3(w.vel[c.a]), c.n), 0.0f);
        if (c.gap - approach * w.dt > 0.0f) return;
        if (fabsf(cn) >= C_EPS) {
            float npts = (float)max(c.np, 1u);
            float ka = is_dynamic(w, c.a) ? w.inv_mass[c.a] : 0.0f;
            float kb = is_dynamic(w, c.b) ? w.inv_mass[c.b] : 0.0f;
            float m_red = ka + kb > NEAR_ZERO ? 1.0f / (ka + kb) : 0.0f;
            if (m_red > 0.0f) {
                float pen_d = fminf(2.0f * m_red / (w.dt * w.dt) / npts, PENALTY_MAX);
                stamp_row(s, c.n, pen_d, fminf(pen_d * cn, 0.0f), r_side, sign);
            }
        }
        return;
    }
    const V3 t1 = c.t1, t2 = c.t2;
    V3 raf, rbf;
    friction_levers(c, rup, rlo, raf, rbf);
    V3 r_side_f = is_a ? raf : rbf;
    float ct1 = row_c_levers(c, t1, 0.0f, raf, rbf);
    float ct2 = row_c_levers(c, t2, 0.0f, raf, rbf);
    float4 pen = w.q_pen[q];
    float f[3];
    contact_force(cn, pen, lam, ct1, ct2, c.mu, f);
    if (row_live(cn, f[0])) stamp_row(s, c.n, pen.x, f[0], r_side, sign);
    if (row_live(ct1, f[1])) stamp_row(s, t1, pen.y, f[1], r_side_f, sign);
    if (row_live(ct2, f[2])) stamp_row(s, t2, pen.z, f[2], r_side_f, sign);
    const float mu_roll = c.mu_roll, mu_spin = c.mu_spin;
    if (mu_roll > 0.0f || mu_spin > 0.0f) {
        V3 wrel = c.dra - c.drb;
        float4 rl = w.q_roll[q];
        V3 rax[3] = {t1, t2, c.n};
        float murs[3] = {mu_roll, mu_roll, mu_spin};
        float rls[3] = {rl.x, rl.y, rl.z};
        for (int li = 0; li < 3; li++) {
            if (murs[li] <= 0.0f) continue;
            float cap = murs[li] * fabsf(f[0]);
            float fr = fclamp(ROLL_PEN * dot(wrel, rax[li]) + rls[li], -cap, cap);
            stamp_angular(s, is_a ? rax[li] : -rax[li], ROLL_PEN, fr);
        }
    }
}

// Joint rows for body h (assembly.rs:255-881): Ball, Revolute (and its
// limit), Prismatic (and its limit), Fixed, Distance, Rope, SixDof.
// ALL = false: the instantiation for worlds whose joints are all ball and
// revolute joints (the other kinds' rows would cost it registers).
// A gear's rows on body h, one of its coupled joints' bodies
// (assembly.rs:426-454 slides, :650-682 hinges): the shared force on the
// position-level row C = coord_a + ratio coord_b - constant, the slide
// sides first, then the hinge sides.
static __device__ __forceinline__ void stamp_gear(const DW& w, uint32_t j, uint32_t h, Sys& s) {
    const GearSide sd[2] = {gear_side(w, j, 0), gear_side(w, j, 1)};
    const float c = gear_error(w, j, sd[0], sd[1]);
    const float pen = w.j_pen_l[j].x;
    const float f = pen * c + w.j_lam_l[j].x;
    if (!row_live(c, f)) return;
    const float coef[2] = {1.0f, w.j_dref[j].x};
    for (int k = 0; k < 2; k++) {
        const GearSide& side = sd[k];
        if (side.angular || (h != side.a && h != side.b)) continue;
        stamp_row(s, side.axis, pen * coef[k] * coef[k], f * coef[k], h == side.a ? side.ra : side.rb,
                  h == side.a ? -1.0f : 1.0f);
    }
    for (int k = 0; k < 2; k++) {
        const GearSide& side = sd[k];
        if (!side.angular || (h != side.a && h != side.b)) continue;
        stamp_angular(s, h == side.a ? -side.axis : side.axis, pen * coef[k] * coef[k], f * coef[k]);
    }
}

template <bool ALL>
static __device__ __forceinline__ void stamp_joint(const DW& w, uint32_t j, uint32_t h, Sys& s) {
    uint2 ab = w.j_ab[j];
    const uint32_t kind = w.j_kind[j];
    if (ALL && kind == AVBD_JOINT_GEAR) {
        stamp_gear(w, j, h, s);
        return;
    }
    const bool k_pri = ALL && kind == AVBD_JOINT_PRISMATIC, k_six = ALL && kind == AVBD_JOINT_SIXDOF;
    const bool k_dist = ALL && (kind == AVBD_JOINT_DISTANCE || kind == AVBD_JOINT_ROPE);
    const bool k_spr = ALL && kind == AVBD_JOINT_SPRING, k_whl = ALL && kind == AVBD_JOINT_WHEEL;
    bool is_a = ab.x == h;
    float sign = is_a ? 1.0f : -1.0f;
    float lsign = is_a ? -1.0f : 1.0f;  // rows measured B minus A flip the gradient
    Q qa = ldq(w.rot[ab.x]), qb = ldq(w.rot[ab.y]);
    Q qa0 = ldq(w.rot0[ab.x]), qb0 = ldq(w.rot0[ab.y]);
    V3 la = ld3(w.j_la[j]), lb = ld3(w.j_lb[j]);
    V3 pa = ld3(w.pos[ab.x]) + qrot(qa, la), pb = ld3(w.pos[ab.y]) + qrot(qb, lb);
    V3 pa0 = ld3(w.pos0[ab.x]) + qrot(qa0, la), pb0 = ld3(w.pos0[ab.y]) + qrot(qb0, lb);
    V3 live = pa - pb, c0v = pa0 - pb0;
    float4 axa4 = w.j_axa[j];
    V3 axa_l = ld3(axa4), axb_l = ld3(w.j_axb[j]);
    V3 wa = normalize_or(qrot(qa, axa_l), VZ());
    float4 pl = w.j_pen_l[j], ll = w.j_lam_l[j], pa4 = w.j_pen_a[j], la4 = w.j_lam_a[j];
    float penl[3] = {pl.x, pl.y, pl.z}, laml[3] = {ll.x, ll.y, ll.z};
    float pena[3] = {pa4.x, pa4.y, pa4.z}, lama[3] = {la4.x, la4.y, la4.z};
    const bool fixed = ALL && kind == AVBD_JOINT_FIXED;
    const V3 dref = fixed || k_six ? ld3(w.j_dref[j]) : V0();
    const float4 ref = w.j_ref[j];
    V3 r_plain = is_a ? qrot(qa, la) : qrot(qb, lb);
    V3 fl = V0();
    // linear rows
    if (kind == AVBD_JOINT_BALL || kind == AVBD_JOINT_REVOLUTE || fixed) {
        // Ball/Revolute levers carry a zero offset in the weld-offset slot
        V3 lever = is_a ? qrot(qa, la + (fixed ? dref : V0())) : qrot(qb, lb);
        V3 lv = fixed ? live + qrot(qa, dref) : live;
        V3 iv = fixed ? c0v + qrot(qa0, dref) : c0v;
        for (int k = 0; k < 3; k++) {
            V3 axis = V0();
            axis[k] = 1.0f;
            float cc = lv[k] - ALPHA * iv[k];
            float f = penl[k] * cc + laml[k];
            if (!row_live(cc, f)) continue;
            stamp_row(s, axis, penl[k], f, lever, sign);
            fl[k] = f;
        }
    } else if (k_pri) {
        V3 u = tangent_t1(wa);
        V3 v = cross(u, wa);
        V3 axs[2] = {u, v};
        for (int li = 0; li < 2; li++) {
            float cc = dot(live - ALPHA * c0v, axs[li]);
            float f = penl[li] * cc + laml[li];
            if (!row_live(cc, f)) continue;
            stamp_row(s, axs[li], penl[li], f, r_plain, sign);
            fl = fl + axs[li] * f;
        }
    } else if (k_dist) {
        float ln = len(live);
        if (kind == AVBD_JOINT_DISTANCE || ln > ref.x) {
            V3 dir = ln > NEAR_ZERO ? live / ln : VY();
            float cc = (ln - ref.x) - ALPHA * (len(c0v) - ref.x);
            float f = penl[0] * cc + laml[0];
            if (row_live(cc, f)) {
                stamp_row(s, dir, penl[0], f, r_plain, sign);
                fl = dir * f;
            }
        }
    } else if (k_whl) {
        // two rows across the suspension axis and the suspension spring
        // along it (assembly.rs:521-581); a zero frequency makes the spring a
        // rigid row on slot 2
        V3 u = tangent_t1(wa);
        V3 v = cross(u, wa);
        V3 axs[2] = {u, v};
        for (int li = 0; li < 2; li++) {
            float cc = dot(live - ALPHA * c0v, axs[li]);
            float f = penl[li] * cc + laml[li];
            if (!row_live(cc, f)) continue;
            stamp_row(s, axs[li], penl[li], f, r_plain, sign);
            fl = fl + axs[li] * f;
        }
        const float4 susp = w.j_lim[j];  // frequency, damping ratio
        const float sv = dot(pb - pa, wa) - ref.x;
        const V3 wa0 = normalize_or(qrot(qa0, axa_l), VZ());
        if (susp.x > 0.0f) {
            const float ka = eff_inv_mass(w, ab.x), kb = eff_inv_mass(w, ab.y);
            const float m = ka + kb > NEAR_ZERO ? 1.0f / (ka + kb) : 0.0f;
            if (m > 0.0f) {
                const float omega = TAU_F * susp.x;
                const float stiff = m * omega * omega, dampc = 2.0f * m * susp.y * omega;
                const float s0 = dot(pb0 - pa0, wa0) - ref.x;
                stamp_row(s, wa, stiff, stiff * sv + dampc * (sv - s0) / w.dt, r_plain, lsign);
            }
        } else {
            const float cc = sv - ALPHA * (dot(pb0 - pa0, wa0) - ref.x);
            const float f = penl[2] * cc + laml[2];
            if (row_live(cc, f)) stamp_row(s, wa, penl[2], f, r_plain, lsign);
        }
    } else if (k_spr) {
        // position-level spring about the rest length (assembly.rs:363-425):
        // penalty from the stiffness, damping from the step delta, no dual
        const float ln = len(live);
        const V3 dir = ln > NEAR_ZERO ? live / ln : VY();
        const float sv = ln - ref.x, s0 = len(c0v) - ref.x;
        const float ka = eff_inv_mass(w, ab.x), kb = eff_inv_mass(w, ab.y);
        const float m = ka + kb > NEAR_ZERO ? 1.0f / (ka + kb) : 0.0f;
        if (m > 0.0f) {
            const float4 mo = w.j_axb[j];  // stiffness, damping, max_force, target_velocity
            const bool force = (w.j_cfg[j] >> 4) == AVBD_MODEL_FORCE;
            const float stiff = force ? mo.x : mo.x * m, dampc = force ? mo.y : mo.y * m;
            if (stiff > 0.0f) {
                stamp_row(s, dir, stiff, stiff * sv + dampc * (sv - s0) / w.dt, r_plain, sign);
            } else if (dampc > 0.0f) {  // a pure damper: the viscous row only
                stamp_row(s, dir, dampc / w.dt, dampc * (sv - s0) / w.dt, r_plain, sign);
            }
        }
    } else if (k_six) {
        const uint32_t cfg = w.j_cfg[j];
        const float4 sa0 = w.j_sacc[2 * (size_t)j];
        const float sacc[3] = {sa0.x, sa0.y, sa0.z};
        for (int i = 0; i < 3; i++) {
            const uint32_t c = axis_cfg(cfg, i);
            if (c == AVBD_AXIS_FREE) continue;
            V3 e = V0();
            e[i] = 1.0f;
            V3 dir = normalize_or(qrot(qa, e), e);
            if (c == AVBD_AXIS_LOCKED) {
                float cc = dot((pb - pa) - qrot(qa, dref), dir);
                float f = penl[i] * cc + laml[i];
                if (!row_live(cc, f)) continue;
                stamp_row(s, dir, penl[i], f, r_plain, lsign);
            } else {
                float2 win = axis_window(w, j, i);
                float sep = dot((pb - pa) - qrot(qa, dref), dir);
                int stt = warm_limit_state(sep, win.x, win.y, LIMIT_SLOP_LIN, sacc[i]);
                if (stt < 0) continue;
                bool lower = stt == 1;
                V3 axis0 = normalize_or(qrot(qa0, e), e);
                float initial = dot((pb0 - pa0) - qrot(qa0, dref), axis0);
                float cc = regularized_limit(sep, initial, lower ? win.x : win.y, lower);
                float f_raw = penl[i] * cc + sacc[i];
                float f = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
                if (!row_live(cc, f)) continue;
                stamp_row(s, dir, penl[i], f, r_plain, lsign);
            }
        }
    }
    {
        // geometric stiffness (rows.rs:69-88, assembly.rs:589-618)
        V3 r = is_a ? qrot(qa, la + (fixed ? dref : V0())) : -qrot(qb, lb);
        float arr[3] = {r.x, r.y, r.z};
        float hm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int k = 0; k < 3; k++) {
            float g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            g[0][0] = -arr[k];
            g[1][1] = -arr[k];
            g[2][2] = -arr[k];
            g[0][k] += arr[0];
            g[1][k] += arr[1];
            g[2][k] += arr[2];
            for (int x = 0; x < 3; x++)
                for (int y = 0; y < 3; y++) hm[x][y] += g[x][y] * fl[k];
        }
        s.h[tri(3, 3)] += len(V3{hm[0][0], hm[1][0], hm[2][0]});
        s.h[tri(4, 4)] += len(V3{hm[0][1], hm[1][1], hm[2][1]});
        s.h[tri(5, 5)] += len(V3{hm[0][2], hm[1][2], hm[2][2]});
    }
    // angular rows (a wheel's pair keys on its axle, in the weld-reference slots)
    if (kind == AVBD_JOINT_REVOLUTE || k_pri || k_whl) {
        const V3 hxa = k_whl ? ld3(w.j_dref[j]) : axa_l, hxb = k_whl ? ld3(w.j_qref[j]) : axb_l;
        V3 axa = qrot(qa, hxa), axb = qrot(qb, hxb);
        V3 axa0 = qrot(qa0, hxa), axb0 = qrot(qb0, hxb);
        V3 t1 = tangent_t1(axa0);
        V3 t2 = cross(t1, axa0);
        V3 ts[2] = {t1, t2};
        for (int li = 0; li < 2; li++) {
            float cc = dot(ts[li], axa - axb) - ALPHA * dot(ts[li], axa0 - axb0);
            float f = pena[li] * cc + lama[li];
            if (!row_live(cc, f)) continue;
            stamp_angular(s, is_a ? cross(axa, ts[li]) : -cross(axb, ts[li]), pena[li], f);
        }
    } else if (k_six) {
        const uint32_t cfg = w.j_cfg[j];
        const Q qref = ldq(w.j_qref[j]);
        const float4 sa0 = w.j_sacc[2 * (size_t)j], sa1 = w.j_sacc[2 * (size_t)j + 1];
        const float sacc[3] = {sa0.w, sa1.x, sa1.y};
        V3 diff = quat_diff_vec(qmul(conj(qa), qb), qref);
        for (int i = 0; i < 3; i++) {
            const uint32_t c = axis_cfg(cfg, 3 + i);
            if (c == AVBD_AXIS_FREE) continue;
            V3 e = V0();
            e[i] = 1.0f;
            V3 dir = normalize_or(qrot(qa, e), e);
            V3 g = is_a ? -dir : dir;
            if (c == AVBD_AXIS_LOCKED) {
                float cc = dot(diff, e);
                float f = pena[i] * cc + lama[i];
                if (!row_live(cc, f)) continue;
                stamp_angular(s, g, pena[i], f);
            } else {
                float2 win = axis_window(w, j, 3 + i);
                float travel = hinge_twist(qa, qb, e) - quat_twist(qref, e);
                int stt = warm_limit_state(travel, win.x, win.y, LIMIT_SLOP_ANG, sacc[i]);
                if (stt < 0) continue;
                bool lower = stt == 1;
                float initial = hinge_twist(qa0, qb0, e) - quat_twist(qref, e);
                float cc = regularized_limit(travel, initial, lower ? win.x : win.y, lower);
                float f_raw = pena[i] * cc + sacc[i];
                float f = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
                if (!row_live(cc, f)) continue;
                stamp_angular(s, g, pena[i], f);
            }
        }
    } else if (fixed) {
        const Q qref = ldq(w.j_qref[j]);
        V3 diff = quat_diff_vec(qmul(conj(qa), qb), qref);
        V3 diff0 = quat_diff_vec(qmul(conj(qa0), qb0), qref);
        for (int k = 0; k < 3; k++) {
            float cc = diff[k] - ALPHA * diff0[k];
            float f = pena[k] * cc + lama[k];
            if (!row_live(cc, f)) continue;
            V3 e = V0();
            e[k] = 1.0f;
            V3 dir = qrot(qa, e);
            stamp_angular(s, is_a ? -dir : dir, pena[k], f);
        }
    }
    // one-sided limit rows
    float4 lim = w.j_lim[j];
    if (lim.z != 0.0f && kind == AVBD_JOINT_REVOLUTE) {
        float refv = axa4.w;
        float angle = wrap_pi(hinge_twist(qa, qb, axa_l) - refv);
        int stt = warm_limit_state(angle, lim.x, lim.y, LIMIT_SLOP_ANG, lim.w);
        if (stt >= 0) {
            bool lower = stt == 1;
            float initial = wrap_pi(hinge_twist(qa0, qb0, axa_l) - refv);
            float cc = regularized_limit(angle, initial, lower ? lim.x : lim.y, lower);
            float f_raw = pa4.z * cc + lim.w;
            float f = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
            if (row_live(cc, f)) stamp_angular(s, is_a ? -wa : wa, pa4.z, f);
        }
    } else if (lim.z != 0.0f && k_pri) {
        float sv = dot(pb - pa, wa) - ref.x;
        int stt = warm_limit_state(sv, lim.x, lim.y, LIMIT_SLOP_LIN, ref.y);
        if (stt >= 0) {
            bool lower = stt == 1;
            V3 axis0 = normalize_or(qrot(qa0, axa_l), VZ());
            float initial = dot(pb0 - pa0, axis0) - ref.x;
            float cc = regularized_limit(sv, initial, lower ? lim.x : lim.y, lower);
            float f_raw = pl.z * cc + ref.y;
            float f = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
            if (row_live(cc, f)) stamp_row(s, wa, pl.z, f, r_plain, lsign);
        }
    }
}

// inertial block and rhs (assembly.rs:74-96)
static __device__ __forceinline__ void inertial_block(const DW& w, uint32_t h, Sys& s) {
    float dt2 = w.dt * w.dt;
    float im = is_dynamic(w, h) ? w.inv_mass[h] : 0.0f;
    float m_dt2 = 1.0f / im / dt2;
    float iw[3][3];
    Q q = ldq(w.rot[h]);
    world_inertia(ld3(w.inertia[h]), q, iw);
    for (int i = 0; i < 21; i++) s.h[i] = 0.0f;
    s.h[tri(0, 0)] = m_dt2;
    s.h[tri(1, 1)] = m_dt2;
    s.h[tri(2, 2)] = m_dt2;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b <= a; b++) s.h[tri(3 + a, 3 + b)] = iw[a][b] / dt2;
    V3 rl = m_dt2 * (ld3(w.pos[h]) - ld3(w.inertial[h]));
    s.r[0] = rl.x;
    s.r[1] = rl.y;
    s.r[2] = rl.z;
    V3 ra = mat3_vec(iw, quat_diff_vec(q, ldq(w.inertial_rot[h]))) / dt2;
    s.r[3] = ra.x;
    s.r[4] = ra.y;
    s.r[5] = ra.z;
}

static __device__ __forceinline__ void apply_solve(const DW& w, uint32_t h, const Sys& s) {
    float dx[6];
    if (solve_6x6(s, dx)) {
        V3 p = ld3(w.pos[h]) + V3{dx[0], dx[1], dx[2]};
        Q q = quat_integrate(ldq(w.rot[h]), V3{dx[3], dx[4], dx[5]});
        V3 dx = p - ld3(w.pos0[h]);
        V3 dr = quat_diff_vec(q, ldq(w.rot0[h]));
        w.pos[h] = st3(p, 0.0f);
        w.rot[h] = stq(q);
        float4* k = w.kin + (size_t)h * 4;
        k[0] = st3(p, w.shp[h].x);
        k[1] = stq(q);
        k[2] = st3(dx, __uint_as_float(w.info[h]));
        k[3] = st3(dr, 0.0f);
    } else {
        atomicAdd(&w.ctr[C_BREAKDOWN], 1u);  // breakdown: the body skips its update
    }
}

// One thread per body: rows accumulate in the reference's order (pairs in
// ascending index — B-side pairs precede A-side ones — then joints).
// JT: 0 for worlds without joints (the joint rows' code and registers stay
// out of the contact-only kernels), 1 with ball and revolute joints only,
// 2 with any joint kind.
template <int MINB, int JT>
__global__ void __launch_bounds__(128, MINB) k_primal_thread(DW w, int colour) {
    if (aborted_solve(w)) return;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c0 = w.col_cnt[colour], c1 = w.col_cnt[colour + 1];
    if (c0 + i >= c1) return;
    uint32_t h = w.col_list[c0 + i];
    Sys s;
    inertial_block(w, h, s);
    for (uint32_t k = w.offB[h]; k < w.offB[h + 1]; k++) {
        uint32_t p = w.listB[k];
        PairCtx c;
        load_ctx(w, p, c);
        for (uint32_t q = 0; q < c.np; q++) stamp_point(w, c, p, q, false, s);
    }
    for (uint32_t p = w.offA[h]; p < w.offA[h + 1]; p++) {
        PairCtx c;
        load_ctx(w, p, c);
        for (uint32_t q = 0; q < c.np; q++) stamp_point(w, c, p, q, true, s);
    }
    if (JT)
        for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1]; k++) stamp_joint<JT == 2>(w, w.jlist[k], h, s);
    apply_solve(w, h, s);
}

// L lanes per body: the body's incident pairs are dealt round-robin over the
// lanes, the partial systems are summed with shuffles, lane 0 adds the
// inertial block and the joints and solves.
template <int L, int JT>
__global__ void k_primal_lanes(DW w, int colour) {
    if (aborted_solve(w)) return;
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t i = gid / L;
    int lane = threadIdx.x % L;
    uint32_t c0 = w.col_cnt[colour], c1 = w.col_cnt[colour + 1];
    bool active = c0 + i < c1;
    uint32_t h = active ? w.col_list[c0 + i] : 0u;
    Sys s;
#pragma unroll
    for (int k = 0; k < 21; k++) s.h[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++) s.r[k] = 0.0f;
    if (active) {
        uint32_t nb = w.offB[h + 1] - w.offB[h], na = w.offA[h + 1] - w.offA[h];
        for (uint32_t e = lane; e < nb + na; e += L) {
            uint32_t p = e < nb ? w.listB[w.offB[h] + e] : w.offA[h] + (e - nb);
            PairCtx c;
            load_ctx(w, p, c);
            for (uint32_t q = 0; q < c.np; q++) stamp_point(w, c, p, q, e >= nb, s);
        }
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 21; k++) s.h[k] += __shfl_down_sync(0xffffffffu, s.h[k], o, L);
#pragma unroll
        for (int k = 0; k < 6; k++) s.r[k] += __shfl_down_sync(0xffffffffu, s.r[k], o, L);
    }
    if (!active || lane != 0) return;
    Sys t;
    inertial_block(w, h, t);
#pragma unroll
    for (int k = 0; k < 21; k++) t.h[k] += s.h[k];
#pragma unroll
    for (int k = 0; k < 6; k++) t.r[k] += s.r[k];
    if (JT)
        for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1]; k++) stamp_joint<JT == 2>(w, w.jlist[k], h, t);
    apply_solve(w, h, t);
}

// ---- split primal -------------------------------------------------------------------
// Per colour, phase 1 (k_side_rows) computes for every (pair, side) whose body
// has this colour the pair's rows for that body, summed over its points, and
// stores the 27 numbers in the incidence slot of that body; phase 2
// (k_side_solve) gives each body of the colour its inertial block plus its
// slots in incidence order (B-side pairs ascending, then A-side pairs
// ascending), then its joints, and solves.  Phase 1 has one thread per
// (pair, side) instead of one per body: several times more threads and short
// dependency chains, which is what the latency-bound per-body loop lacks once
// bodies touch many others.  Rows are summed per pair before they join the
// body's sum, so results equal the thread-per-body kernel's within rounding.
// Slots: body h owns [offA[h] + offB[h], offA[h+1] + offB[h+1]), B sides first;
// the A side of pair p is slot p + offB[a+1], the B side slot offA[b] + posB[p].
constexpr int SIDE_BLOCK = 256;
__global__ void k_side_count(DW w) {
    if (aborted_solve(w)) return;
    __shared__ uint32_t hist[MAX_COLOURS];
    for (int c = threadIdx.x; c < MAX_COLOURS; c += blockDim.x) hist[c] = 0;
    __syncthreads();
    const uint32_t n = n_pairs(w);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint2 ab = w.p_ab[p];
        int ca = w.colour[ab.x], cb = w.colour[ab.y];
        if (ca >= 0) atomicAdd(&hist[ca], 1u);
        if (cb >= 0) atomicAdd(&hist[cb], 1u);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < MAX_COLOURS; c += blockDim.x)
        if (hist[c]) atomicAdd(&w.side_cnt[MAX_COLOURS + 1 + c], hist[c]);
}
// one thread: list starts from the per-colour totals; cursors start there
__global__ void k_side_starts(DW w) {
    if (aborted_solve(w) || threadIdx.x != 0) return;
    uint32_t acc = 0;
    for (int c = 0; c < MAX_COLOURS; c++) {
        uint32_t t = w.side_cnt[MAX_COLOURS + 1 + c];
        w.side_cnt[c] = acc;
        w.side_cnt[MAX_COLOURS + 1 + c] = acc;
        acc += t;
    }
    w.side_cnt[MAX_COLOURS] = acc;
}
// Entries are placed with block-aggregated reservations, so a colour's list
// keeps roughly the pair order (neighbouring entries share bodies and point
// arrays: grouping entries by point count instead lost more in locality than
// it won in convergence); the exact order is irrelevant (each entry writes
// its own slot).
__global__ void k_side_place(DW w) {
    if (aborted_solve(w)) return;
    __shared__ uint32_t cnt[MAX_COLOURS], base[MAX_COLOURS];
    const uint32_t n = n_pairs(w);
    for (uint32_t p0 = blockIdx.x * blockDim.x; p0 < n; p0 += gridDim.x * blockDim.x) {
        for (int c = threadIdx.x; c < MAX_COLOURS; c += blockDim.x) cnt[c] = 0;
        __syncthreads();
        uint32_t p = p0 + threadIdx.x;
        int ca = -1, cb = -1;
        if (p < n) {
            uint2 ab = w.p_ab[p];
            ca = w.colour[ab.x];
            cb = w.colour[ab.y];
        }
        uint32_t ra = ca >= 0 ? atomicAdd(&cnt[ca], 1u) : 0u;
        uint32_t rb = cb >= 0 ? atomicAdd(&cnt[cb], 1u) : 0u;
        __syncthreads();
        for (int c = threadIdx.x; c < MAX_COLOURS; c += blockDim.x)
            base[c] = cnt[c] ? atomicAdd(&w.side_cnt[MAX_COLOURS + 1 + c], cnt[c]) : 0u;
        __syncthreads();
        if (ca >= 0) w.side_list[base[ca] + ra] = p * 2u + 1u;
        if (cb >= 0) w.side_list[base[cb] + rb] = p * 2u;
        __syncthreads();
    }
}

// The rows of pair p for its body on side side_a, summed over the pair's
// points in point order: 21 Hessian + 6 rhs numbers as 7 float4 at o.
static __device__ __forceinline__ void side_rows(const DW& w, uint32_t p, bool side_a, PairCtx& c, float4* o) {
    Sys s;
#pragma unroll
    for (int k = 0; k < 21; k++) s.h[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++) s.r[k] = 0.0f;
    for (uint32_t q = 0; q < c.np; q++) stamp_point(w, c, p, q, side_a, s);
    o[0] = make_float4(s.h[0], s.h[1], s.h[2], s.h[3]);
    o[1] = make_float4(s.h[4], s.h[5], s.h[6], s.h[7]);
    o[2] = make_float4(s.h[8], s.h[9], s.h[10], s.h[11]);
    o[3] = make_float4(s.h[12], s.h[13], s.h[14], s.h[15]);
    o[4] = make_float4(s.h[16], s.h[17], s.h[18], s.h[19]);
    o[5] = make_float4(s.h[20], s.r[0], s.r[1], s.r[2]);
    o[6] = make_float4(s.r[3], s.r[4], s.r[5], 0.0f);
}
// Add one incidence slot's 7 float4 to a body's system (k_side_solve's order).
static __device__ __forceinline__ void add_slot(Sys& s, const float4* o) {
    float4 v0 = o[0], v1 = o[1], v2 = o[2], v3 = o[3], v4 = o[4], v5 = o[5], v6 = o[6];
    s.h[0] += v0.x; s.h[1] += v0.y; s.h[2] += v0.z; s.h[3] += v0.w;
    s.h[4] += v1.x; s.h[5] += v1.y; s.h[6] += v1.z; s.h[7] += v1.w;
    s.h[8] += v2.x; s.h[9] += v2.y; s.h[10] += v2.z; s.h[11] += v2.w;
    s.h[12] += v3.x; s.h[13] += v3.y; s.h[14] += v3.z; s.h[15] += v3.w;
    s.h[16] += v4.x; s.h[17] += v4.y; s.h[18] += v4.z; s.h[19] += v4.w;
    s.h[20] += v5.x; s.r[0] += v5.y; s.r[1] += v5.z; s.r[2] += v5.w;
    s.r[3] += v6.x; s.r[4] += v6.y; s.r[5] += v6.z;
}
// Work lists are taken in chunks of one block (128 entries) whose entries are
// handed to the block's threads grouped by a small work class (the entry's
// loop length), so that the lanes of a warp run loops of the same length
// instead of idling behind the longest one.  The chunk keeps the list's
// locality; each entry writes only its own outputs, so which thread takes
// it changes no result.
constexpr int CHUNK = 128;
// Counting sort of the chunk's entries by class (0..MAX_PTS) into ent[].
// Every thread of the block calls it; returns the entries in the chunk.
static __device__ __forceinline__ uint32_t chunk_sort(uint32_t* cnt, uint32_t* ent, bool has, uint32_t e,
                                                      uint32_t cls, uint32_t n) {
    if (threadIdx.x <= MAX_PTS) cnt[threadIdx.x] = 0;
    __syncthreads();
    if (has) atomicAdd(&cnt[cls], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int k = 0; k <= MAX_PTS; k++) {
            uint32_t c = cnt[k];
            cnt[k] = acc;
            acc += c;
        }
    }
    __syncthreads();
    if (has) ent[atomicAdd(&cnt[cls], 1u)] = e;
    __syncthreads();
    return n;
}
__global__ void __launch_bounds__(CHUNK, 4) k_side_rows(DW w, int colour) {
    if (aborted_solve(w)) return;
    __shared__ uint32_t s_cnt[MAX_PTS + 1], s_ent[CHUNK];
    const uint32_t s0 = w.side_cnt[colour], s1 = w.side_cnt[colour + 1];
    for (uint32_t base = s0 + blockIdx.x * CHUNK; base < s1; base += gridDim.x * CHUNK) {
        const uint32_t i = base + threadIdx.x;
        const bool has = i < s1;
        uint32_t e = 0, cls = 0;
        if (has) {
            e = w.side_list[i];
            uint32_t p = e >> 1;
            cls = w.p_n[p].w <= 0.0f ? w.p_np[p] : 0u;  // separated pairs stamp at most a damper row
        }
        const uint32_t n = chunk_sort(s_cnt, s_ent, has, e, cls, min((uint32_t)CHUNK, s1 - base));
        if (threadIdx.x < n) {
            e = s_ent[threadIdx.x];
            uint32_t p = e >> 1;
            bool side_a = (e & 1u) != 0u;
            PairCtx c;
            load_ctx(w, p, c);
            uint32_t slot = side_a ? p + w.offB[c.a + 1] : w.offA[c.b] + w.posB[p];
            // a recording frame too small: the host reports it
            if (slot < w.contrib_slots) side_rows(w, p, side_a, c, w.contrib + (size_t)slot * 7);
        }
        __syncthreads();  // the chunk's entries are read before the next chunk is sorted
    }
}
template <int JT>
__global__ void __launch_bounds__(128) k_side_solve(DW w, int colour) {
    if (aborted_solve(w)) return;
    const uint32_t c0 = w.col_cnt[colour], c1 = w.col_cnt[colour + 1];
    for (uint32_t i = c0 + blockIdx.x * blockDim.x + threadIdx.x; i < c1; i += gridDim.x * blockDim.x) {
        uint32_t h = w.col_list[i];
        Sys s;
        inertial_block(w, h, s);
        const uint32_t k0 = w.offA[h] + w.offB[h], k1 = min(w.offA[h + 1] + w.offB[h + 1], w.contrib_slots);
        for (uint32_t k = k0; k < k1; k++) add_slot(s, w.contrib + (size_t)k * 7);
        if (JT)
            for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1]; k++) stamp_joint<JT == 2>(w, w.jlist[k], h, s);
        apply_solve(w, h, s);
    }
}

// ---- dual (joints_ext.rs:464-573 contacts, :574-896 Ball/Revolute) ----
// One thread per pair: the pair context is built once for all its points.
static __device__ __forceinline__ void dual_point(const DW& w, const PairCtx& c, V3 t1, V3 t2, uint32_t q) {
    float4 ra = w.q_ra[q], rb = w.q_rb[q];
    bool touching = c.gap <= 0.0f;
    float4 pen = w.q_pen[q], lam = w.q_lam[q];
    float c0 = touching ? lam.w : 0.0f;
    V3 raw, rbw;
    contact_levers(c, ra, rb, raw, rbw);
    float cn = row_c_levers(c, c.n, c0, raw, rbw);
    V3 raf, rbf;
    friction_levers(c, raw, rbw, raf, rbf);
    float ct1 = row_c_levers(c, t1, 0.0f, raf, rbf);
    float ct2 = row_c_levers(c, t2, 0.0f, raf, rbf);
    float f[3];
    contact_force(cn, pen, lam, ct1, ct2, c.mu, f);
    float bnd = fabsf(f[0]) * fmaxf(c.mu.x, c.mu.y);
    float fu0 = pen.y * ct1 + lam.y, fu1 = pen.z * ct2 + lam.z;
    bool stuck = sqrtf(fu0 * fu0 + fu1 * fu1) <= bnd && sqrtf(ct1 * ct1 + ct2 * ct2) < STICK_THRESH;
    float4 nl = lam, np4 = pen;
    if (touching && fabsf(cn) >= C_EPS) {
        nl.x = f[0];
        if (f[0] < 0.0f) np4.x = fminf(pen.x + BETA * fabsf(cn), PENALTY_MAX);
    }
    float b1 = fabsf(f[0]) * c.mu.x, b2 = fabsf(f[0]) * c.mu.y;
    float s_ell = (b1 > 0.0f && b2 > 0.0f) ? (fu0 / b1) * (fu0 / b1) + (fu1 / b2) * (fu1 / b2) : INFINITY;
    if (touching) {
        nl.y = f[1];
        nl.z = f[2];
        if (s_ell <= 1.0f) {
            if (fabsf(ct1) >= C_EPS) np4.y = fminf(pen.y + BETA * fabsf(ct1), PENALTY_MAX);
            if (fabsf(ct2) >= C_EPS) np4.z = fminf(pen.z + BETA * fabsf(ct2), PENALTY_MAX);
        }
    }
    w.q_lam[q] = nl;
    // penalties and the grip flag change in few iterations: store only changes
    if (np4.x != pen.x || np4.y != pen.y || np4.z != pen.z) w.q_pen[q] = np4;
    if (stuck != (rb.w != 0.0f)) reinterpret_cast<float*>(&w.q_rb[q])[3] = stuck ? 1.0f : 0.0f;
    const float mu_roll = c.mu_roll, mu_spin = c.mu_spin;
    if (touching && (mu_roll > 0.0f || mu_spin > 0.0f)) {
        V3 wrel = c.dra - c.drb;
        float lam_n = fabsf(nl.x);
        float4 rl = w.q_roll[q];
        float rls[3] = {rl.x, rl.y, rl.z};
        V3 rax[3] = {t1, t2, c.n};
        float murs[3] = {mu_roll, mu_roll, mu_spin};
        for (int li = 0; li < 3; li++) {
            if (murs[li] <= 0.0f) continue;
            float cap = murs[li] * lam_n;
            rls[li] = fclamp(ROLL_PEN * dot(wrel, rax[li]) + rls[li], -cap, cap);
        }
        w.q_roll[q] = make_float4(rls[0], rls[1], rls[2], 0.0f);
    }
}
static __device__ __forceinline__ void dual_pair(const DW& w, uint32_t p) {
    uint32_t np = w.p_np[p];
    if (np == 0) return;
    PairCtx c;
    load_ctx(w, p, c);
    V3 t1 = tangent_t1(c.n);  // the grip flag of separated points needs the frame too
    V3 t2 = cross(t1, c.n);
    for (uint32_t k = 0; k < np; k++) dual_point(w, c, t1, t2, p * MAX_PTS + k);
}
__global__ void __launch_bounds__(CHUNK) k_dual_pairs(DW w) {
    if (aborted_solve(w)) return;
    __shared__ uint32_t s_cnt[MAX_PTS + 1], s_ent[CHUNK];
    const uint32_t np = n_pairs(w);
    for (uint32_t base = blockIdx.x * CHUNK; base < np; base += gridDim.x * CHUNK) {
        const uint32_t p = base + threadIdx.x;
        const bool has = p < np;
        const uint32_t cls = has ? min(w.p_np[p], (uint32_t)MAX_PTS) : 0u;
        const uint32_t n = chunk_sort(s_cnt, s_ent, has, p, cls, min((uint32_t)CHUNK, np - base));
        if (threadIdx.x < n) dual_pair(w, s_ent[threadIdx.x]);
        __syncthreads();
    }
}
// joints_ext.rs:574-896: the joint rows' multipliers and penalties
static __device__ __forceinline__ float ramp(float pen, float c, float beta, float cap) {
    return fminf(pen + beta * fabsf(c), cap);
}
template <bool ALL>
static __device__ void dual_joint(const DW& w, uint32_t j) {
    uint2 ab = w.j_ab[j];
    const uint32_t kind = w.j_kind[j];
    if (ALL && kind == AVBD_JOINT_GEAR) {
        // reads only bodies and its own state: its place after every other
        // joint (joints_ext.rs:897-918) cannot change it; penalty capped
        // like a limit's
        const GearSide sa = gear_side(w, j, 0), sb = gear_side(w, j, 1);
        const float c = gear_error(w, j, sa, sb);
        if (fabsf(c) < C_EPS) return;
        float4 ll = w.j_lam_l[j], pl = w.j_pen_l[j];
        ll.x = ll.x + pl.x * c;
        pl.x = ramp(pl.x, c, BETA, LIM_PEN_MAX);
        w.j_lam_l[j] = ll;
        w.j_pen_l[j] = pl;
        return;
    }
    const bool k_pri = ALL && kind == AVBD_JOINT_PRISMATIC, k_six = ALL && kind == AVBD_JOINT_SIXDOF;
    Q qa = ldq(w.rot[ab.x]), qb = ldq(w.rot[ab.y]);
    Q qa0 = ldq(w.rot0[ab.x]), qb0 = ldq(w.rot0[ab.y]);
    V3 la = ld3(w.j_la[j]), lb = ld3(w.j_lb[j]);
    V3 pa = ld3(w.pos[ab.x]) + qrot(qa, la), pb = ld3(w.pos[ab.y]) + qrot(qb, lb);
    V3 pa0 = ld3(w.pos0[ab.x]) + qrot(qa0, la), pb0 = ld3(w.pos0[ab.y]) + qrot(qb0, lb);
    V3 live = pa - pb, c0v = pa0 - pb0;
    float4 ll = w.j_lam_l[j], pl = w.j_pen_l[j];
    float laml[3] = {ll.x, ll.y, ll.z}, penl[3] = {pl.x, pl.y, pl.z};
    float4 la4 = w.j_lam_a[j], pa4 = w.j_pen_a[j];
    float lama[3] = {la4.x, la4.y, la4.z}, pena[3] = {pa4.x, pa4.y, pa4.z};
    float4 ref = w.j_ref[j];
    // a soft joint (finite stiffness K) is a spring: penalty K, lambda zero,
    // for the anchor and hinge rows of ball and revolute joints; a hard one
    // is the reference's dual ascent
    const float K = w.joint_k;
    const bool soft = K > 0.0f && (kind == AVBD_JOINT_BALL || kind == AVBD_JOINT_REVOLUTE);
    const bool fixed = ALL && kind == AVBD_JOINT_FIXED;
    if (kind == AVBD_JOINT_BALL || kind == AVBD_JOINT_REVOLUTE || fixed) {
        const V3 dref = fixed ? ld3(w.j_dref[j]) : V0();
        V3 lv = fixed ? live + qrot(qa, dref) : live;
        V3 iv = fixed ? c0v + qrot(qa0, dref) : c0v;
        for (int k = 0; k < 3; k++) {
            float cc = lv[k] - ALPHA * iv[k];
            if (soft) {
                penl[k] = K;
            } else if (fabsf(cc) >= C_EPS) {
                laml[k] += penl[k] * cc;
                penl[k] = ramp(penl[k], cc, BETA, PENALTY_MAX);
            }
        }
    } else if (k_pri) {
        V3 wa = normalize_or(qrot(qa, ld3(w.j_axa[j])), VZ());
        V3 u = tangent_t1(wa);
        V3 v = cross(u, wa);
        V3 axs[2] = {u, v};
        for (int li = 0; li < 2; li++) {
            float cc = dot(live - ALPHA * c0v, axs[li]);
            if (fabsf(cc) >= C_EPS) {
                laml[li] += penl[li] * cc;
                penl[li] = ramp(penl[li], cc, BETA, PENALTY_MAX);
            }
        }
    } else if (ALL && kind == AVBD_JOINT_WHEEL) {
        // the rows across the suspension axis, and the rigid suspension row
        // when the frequency is zero (joints_ext.rs:738-764); a live spring
        // carries no dual state
        V3 wa = normalize_or(qrot(qa, ld3(w.j_axa[j])), VZ());
        V3 u = tangent_t1(wa);
        V3 v = cross(u, wa);
        V3 axs[2] = {u, v};
        for (int li = 0; li < 2; li++) {
            float cc = dot(live - ALPHA * c0v, axs[li]);
            if (fabsf(cc) >= C_EPS) {
                laml[li] += penl[li] * cc;
                penl[li] = ramp(penl[li], cc, BETA, PENALTY_MAX);
            }
        }
        if (w.j_lim[j].x <= 0.0f) {
            V3 wa0 = normalize_or(qrot(qa0, ld3(w.j_axa[j])), VZ());
            float cc = (-dot(live, wa) - ref.x) - ALPHA * (-dot(pa0 - pb0, wa0) - ref.x);
            if (fabsf(cc) >= C_EPS) {
                laml[2] += penl[2] * cc;
                penl[2] = ramp(penl[2], cc, BETA, LIM_PEN_MAX);
            }
        }
    } else if (ALL && kind == AVBD_JOINT_DISTANCE) {
        float cc = (len(live) - ref.x) - ALPHA * (len(c0v) - ref.x);
        if (fabsf(cc) >= C_EPS) {
            laml[0] += penl[0] * cc;
            penl[0] = ramp(penl[0], cc, BETA, PENALTY_MAX);
        }
    } else if (ALL && kind == AVBD_JOINT_ROPE) {
        float ln = len(live);
        if (ln > ref.x) {
            float cc = (ln - ref.x) - ALPHA * (len(c0v) - ref.x);
            if (fabsf(cc) >= C_EPS) {
                laml[0] = fmaxf(laml[0] + penl[0] * cc, 0.0f);
                penl[0] = ramp(penl[0], cc, BETA, LIM_PEN_MAX);
            }
        } else {
            laml[0] = 0.0f;
        }
    } else if (k_six) {
        const uint32_t cfg = w.j_cfg[j];
        const V3 dref = ld3(w.j_dref[j]);
        const Q qref = ldq(w.j_qref[j]);
        float4 sa0 = w.j_sacc[2 * (size_t)j], sa1 = w.j_sacc[2 * (size_t)j + 1];
        float sacc[6] = {sa0.x, sa0.y, sa0.z, sa0.w, sa1.x, sa1.y};
        for (int i = 0; i < 3; i++) {
            const uint32_t c = axis_cfg(cfg, i);
            if (c == AVBD_AXIS_FREE) continue;
            V3 e = V0();
            e[i] = 1.0f;
            V3 dir = normalize_or(qrot(qa, e), e);
            float sep = dot((pb - pa) - qrot(qa, dref), dir);
            if (c == AVBD_AXIS_LOCKED) {
                if (fabsf(sep) >= C_EPS) {
                    laml[i] += penl[i] * sep;
                    penl[i] = ramp(penl[i], sep, BETA, PENALTY_MAX);
                }
            } else {
                float2 win = axis_window(w, j, i);
                int stt = warm_limit_state(sep, win.x, win.y, LIMIT_SLOP_LIN, sacc[i]);
                if (stt >= 0) {
                    bool lower = stt == 1;
                    V3 axis0 = normalize_or(qrot(qa0, e), e);
                    float initial = dot((pb0 - pa0) - qrot(qa0, dref), axis0);
                    float cc = regularized_limit(sep, initial, lower ? win.x : win.y, lower);
                    if (fabsf(cc) >= C_EPS) {
                        float f = penl[i] * cc + sacc[i];
                        sacc[i] = lower ? fminf(f, 0.0f) : fmaxf(f, 0.0f);
                        penl[i] = ramp(penl[i], cc, BETA, LIM_PEN_MAX);
                    }
                } else {
                    sacc[i] = 0.0f;
                }
            }
        }
        V3 diff = quat_diff_vec(qmul(conj(qa), qb), qref);
        for (int i = 0; i < 3; i++) {
            const uint32_t c = axis_cfg(cfg, 3 + i);
            if (c == AVBD_AXIS_FREE) continue;
            V3 e = V0();
            e[i] = 1.0f;
            if (c == AVBD_AXIS_LOCKED) {
                float cc = dot(diff, e);
                if (fabsf(cc) >= C_EPS) {
                    lama[i] += pena[i] * cc;
                    pena[i] = ramp(pena[i], cc, BETA_ANG, PENALTY_MAX);
                }
            } else {
                float2 win = axis_window(w, j, 3 + i);
                float travel = hinge_twist(qa, qb, e) - quat_twist(qref, e);
                int stt = warm_limit_state(travel, win.x, win.y, LIMIT_SLOP_ANG, sacc[3 + i]);
                if (stt >= 0) {
                    bool lower = stt == 1;
                    float initial = hinge_twist(qa0, qb0, e) - quat_twist(qref, e);
                    float cc = regularized_limit(travel, initial, lower ? win.x : win.y, lower);
                    if (fabsf(cc) >= C_EPS) {
                        float f = pena[i] * cc + sacc[3 + i];
                        sacc[3 + i] = lower ? fminf(f, 0.0f) : fmaxf(f, 0.0f);
                        pena[i] = ramp(pena[i], cc, BETA_ANG, LIM_PEN_MAX);
                    }
                } else {
                    sacc[3 + i] = 0.0f;
                }
            }
        }
        w.j_sacc[2 * (size_t)j] = make_float4(sacc[0], sacc[1], sacc[2], sacc[3]);
        w.j_sacc[2 * (size_t)j + 1] = make_float4(sacc[4], sacc[5], 0.0f, 0.0f);
    }
    // angular equality rows (a wheel's keyed on its axle, joints_ext.rs:789-803)
    if (kind == AVBD_JOINT_REVOLUTE || k_pri || (ALL && kind == AVBD_JOINT_WHEEL)) {
        const bool whl = ALL && kind == AVBD_JOINT_WHEEL;
        V3 axa_l = whl ? ld3(w.j_dref[j]) : ld3(w.j_axa[j]), axb_l = whl ? ld3(w.j_qref[j]) : ld3(w.j_axb[j]);
        V3 axa = qrot(qa, axa_l), axb = qrot(qb, axb_l);
        V3 axa0 = qrot(qa0, axa_l), axb0 = qrot(qb0, axb_l);
        V3 t1 = tangent_t1(axa0);
        V3 t2 = cross(t1, axa0);
        V3 ts[2] = {t1, t2};
        for (int li = 0; li < 2; li++) {
            float cc = dot(ts[li], axa - axb) - ALPHA * dot(ts[li], axa0 - axb0);
            if (soft) {
                pena[li] = K;
                continue;
            }
            if (fabsf(cc) < C_EPS) continue;
            lama[li] = pena[li] * cc + lama[li];
            pena[li] = ramp(pena[li], cc, BETA_ANG, PENALTY_MAX);
        }
    } else if (fixed) {
        const Q qref = ldq(w.j_qref[j]);
        V3 diff = quat_diff_vec(qmul(conj(qa), qb), qref);
        V3 diff0 = quat_diff_vec(qmul(conj(qa0), qb0), qref);
        for (int k = 0; k < 3; k++) {
            float cc = diff[k] - ALPHA * diff0[k];
            if (fabsf(cc) < C_EPS) continue;
            lama[k] += pena[k] * cc;
            pena[k] = ramp(pena[k], cc, BETA_ANG, PENALTY_MAX);
        }
    }
    // one-sided limits
    float4 lim = w.j_lim[j];
    if (lim.z != 0.0f && kind == AVBD_JOINT_REVOLUTE) {
        V3 axa_l = ld3(w.j_axa[j]);
        float refv = w.j_axa[j].w;
        float angle = wrap_pi(hinge_twist(qa, qb, axa_l) - refv);
        int stt = warm_limit_state(angle, lim.x, lim.y, LIMIT_SLOP_ANG, lim.w);
        if (stt >= 0) {
            bool lower = stt == 1;
            float initial = wrap_pi(hinge_twist(qa0, qb0, axa_l) - refv);
            float cc = regularized_limit(angle, initial, lower ? lim.x : lim.y, lower);
            if (fabsf(cc) >= C_EPS) {
                float f = pena[2] * cc + lim.w;
                lim.w = lower ? fminf(f, 0.0f) : fmaxf(f, 0.0f);
                pena[2] = ramp(pena[2], cc, BETA_ANG, LIM_PEN_MAX);
            }
        } else {
            lim.w = 0.0f;
        }
        w.j_lim[j] = lim;
    } else if (lim.z != 0.0f && k_pri) {
        V3 axa_l = ld3(w.j_axa[j]);
        V3 wa = normalize_or(qrot(qa, axa_l), VZ());
        float sv = dot(pb - pa, wa) - ref.x;
        int stt = warm_limit_state(sv, lim.x, lim.y, LIMIT_SLOP_LIN, ref.y);
        if (stt >= 0) {
            bool lower = stt == 1;
            V3 axis0 = normalize_or(qrot(qa0, axa_l), VZ());
            float initial = dot(pb0 - pa0, axis0) - ref.x;
            float cc = regularized_limit(sv, initial, lower ? lim.x : lim.y, lower);
            if (fabsf(cc) >= C_EPS) {
                float f_raw = penl[2] * cc + ref.y;
                ref.y = lower ? fminf(f_raw, 0.0f) : fmaxf(f_raw, 0.0f);
                penl[2] = ramp(penl[2], cc, BETA, LIM_PEN_MAX);
            }
        } else {
            lim.w = 0.0f;
            ref.y = 0.0f;
        }
        w.j_lim[j] = lim;
        w.j_ref[j] = ref;
    }
    w.j_lam_l[j] = make_float4(laml[0], laml[1], laml[2], 0.0f);
    w.j_pen_l[j] = make_float4(penl[0], penl[1], penl[2], 0.0f);
    w.j_lam_a[j] = make_float4(lama[0], lama[1], lama[2], 0.0f);
    w.j_pen_a[j] = make_float4(pena[0], pena[1], pena[2], 0.0f);
}
template <bool ALL>
__global__ void k_dual_joints(DW w) {
    if (aborted_solve(w)) return;
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < (uint32_t)w.J) dual_joint<ALL>(w, j);
}

// ---- per-scene solve: one block walks a scene through every iteration ---------
// Scenes never interact, so a block can take one scene through all
// iterations of a substep — every colour's primal, then the scene's dual —
// with block barriers between the phases and no wait on any other block.
// The scene's data (its bodies' motion records, pairs and points) is touched
// iterations x (colours + 1) times within one block, so after the first
// touch it is served from L2 instead of being streamed from HBM once per
// launch.  Blocks take scenes from a queue in descending size order (the
// longest first), so the largest scenes do not finish last.
//
// Arithmetic is the split primal's: per (pair, side) the pair's rows summed
// over its points (one thread per item, staged in shared memory), then per
// body the inertial block, its items in incidence order and its joints, and
// the 6x6 solve (one owner thread per body); the dual per pair and per joint.
// Bodies of one colour share no pair or joint, so the order in which a
// colour's bodies are visited cannot change a result.

// In-place exclusive scan of a[0..n) (n <= SCENE_MAX_BODIES) by the block;
// a[n] receives the total.  Needs 32 words of scratch.
template <int BS>
static __device__ __forceinline__ void block_scan(uint32_t* a, uint32_t n, uint32_t* warp_tot) {
    const uint32_t per = (n + BS - 1) / BS;
    const uint32_t t = threadIdx.x, i0 = min(n, t * per), i1 = min(n, i0 + per);
    uint32_t sum = 0;
    for (uint32_t i = i0; i < i1; i++) sum += a[i];
    const uint32_t lane = t & 31u, wid = t >> 5;
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += v;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t v = lane < BS / 32 ? warp_tot[lane] : 0u, x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane < BS / 32) warp_tot[lane] = x - v;  // exclusive warp offsets
        if (lane == BS / 32 - 1) a[n] = x;          // the total (a[n] is past every thread's chunk)
    }
    __syncthreads();
    uint32_t run = warp_tot[wid] + inc - sum;
    for (uint32_t i = i0; i < i1; i++) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
}

template <int BS, int MINB, int JT>
__global__ void __launch_bounds__(BS, MINB) k_scene_solve(DW w) {
    if (aborted_solve(w)) return;
    __shared__ uint32_t s_list[SCENE_MAX_BODIES];      // swept bodies grouped by colour
    __shared__ uint32_t s_pref[SCENE_MAX_BODIES + 1];  // item offset of each list entry
    __shared__ uint32_t s_cstart[MAX_COLOURS + 1];
    __shared__ uint32_t s_cur[MAX_COLOURS];
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_scene;
    __shared__ int s_ncol;
    extern __shared__ float4 s_rows[];  // BS items x 7 float4
    const uint32_t tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_scene = atomicAdd(&w.ctr[C_SCENE_Q], 1u);
        __syncthreads();
        const uint32_t q = s_scene;
        if (q >= (uint32_t)w.S) return;
        const uint32_t sc = w.scene_order[q];
        const uint32_t b0 = w.scene_off[sc], b1 = w.scene_off[sc + 1];
        // colour lists of the scene's swept bodies
        for (uint32_t c = tid; c < MAX_COLOURS; c += BS) s_cur[c] = 0;
        if (tid == 0) s_ncol = 0;
        __syncthreads();
        for (uint32_t h = b0 + tid; h < b1; h += BS) {
            int c = w.colour[h];
            if (c >= 0 && c < MAX_COLOURS) {
                atomicAdd(&s_cur[c], 1u);
                atomicMax(&s_ncol, c + 1);
            }
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t acc = 0;
            for (int c = 0; c < s_ncol; c++) {
                s_cstart[c] = acc;
                acc += s_cur[c];
                s_cur[c] = s_cstart[c];
            }
            s_cstart[s_ncol] = acc;
        }
        __syncthreads();
        const int ncol = s_ncol;
        const uint32_t nlist = s_cstart[ncol];
        for (uint32_t h = b0 + tid; h < b1; h += BS) {
            int c = w.colour[h];
            if (c >= 0 && c < MAX_COLOURS) s_list[atomicAdd(&s_cur[c], 1u)] = h;
        }
        __syncthreads();
        for (uint32_t i = tid; i < nlist; i += BS) {
            uint32_t h = s_list[i];
            s_pref[i] = (w.offA[h + 1] - w.offA[h]) + (w.offB[h + 1] - w.offB[h]);
        }
        __syncthreads();
        block_scan<BS>(s_pref, nlist, s_warp);
        const uint32_t p0 = w.offA[b0], p1 = w.offA[b1];
        for (int it = 0; it < w.iterations; it++) {
            for (int c = 0; c < ncol; c++) {
                const uint32_t hi = s_cstart[c + 1];
                for (uint32_t i0 = s_cstart[c]; i0 < hi;) {
                    // a group: the next (up to) BS bodies of the colour, one
                    // owner thread each; their items are computed BS per round
                    const uint32_t base = s_pref[i0];
                    const uint32_t i1 = min(hi, i0 + BS);
                    const uint32_t nb = i1 - i0, nitems = s_pref[i1] - base;
                    Sys s;
                    uint32_t h = 0, my0 = 0, my1 = 0;
                    if (tid < nb) {
                        h = s_list[i0 + tid];
                        inertial_block(w, h, s);
                        my0 = s_pref[i0 + tid] - base;
                        my1 = s_pref[i0 + tid + 1] - base;
                    }
                    for (uint32_t r0 = 0; r0 < nitems; r0 += BS) {
                        const uint32_t g = r0 + tid;
                        if (g < nitems) {
                            // the body of item g: the last entry starting at or before it
                            int lo = (int)i0, up = (int)i1 - 1;
                            while (lo < up) {
                                int m = (lo + up + 1) >> 1;
                                if (s_pref[m] - base <= g) lo = m;
                                else up = m - 1;
                            }
                            const uint32_t hb = s_list[lo], k = g - (s_pref[lo] - base);
                            const uint32_t nB = w.offB[hb + 1] - w.offB[hb];
                            const bool side_a = k >= nB;
                            const uint32_t p = side_a ? w.offA[hb] + (k - nB) : w.listB[w.offB[hb] + k];
                            PairCtx cx;
                            load_ctx(w, p, cx);
                            side_rows(w, p, side_a, cx, s_rows + (size_t)tid * 7);
                        }
                        __syncthreads();
                        if (tid < nb) {
                            const uint32_t e1 = min(my1, r0 + BS);
                            for (uint32_t e = max(my0, r0); e < e1; e++) add_slot(s, s_rows + (size_t)(e - r0) * 7);
                        }
                        __syncthreads();
                    }
                    if (tid < nb) {
                        if (JT)
                            for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1]; k++) stamp_joint<JT == 2>(w, w.jlist[k], h, s);
                        apply_solve(w, h, s);
                    }
                    i0 = i1;
                }
                __syncthreads();  // this colour's poses before the next colour reads them
            }
            for (uint32_t p = p0 + tid; p < p1; p += BS) dual_pair(w, p);
            if (JT)
                for (uint32_t h = b0 + tid; h < b1; h += BS)
                    for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1]; k++) {
                        uint32_t j = w.jlist[k];
                        if (joint_dual_owner(w, j) == h) dual_joint<JT == 2>(w, j);
                    }
            __syncthreads();
        }
    }
}

template <int BS, int MINB, int JT>
static void scene_solve_launch(const DW& w, cudaStream_t st) {
    const size_t smem = (size_t)BS * 7 * sizeof(float4);
    static int grid[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // per device ordinal
    int dev = 0;
    cudaGetDevice(&dev);
    int& g = grid[dev & 7];
    if (!g) {
        cudaFuncSetAttribute(k_scene_solve<BS, MINB, JT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scene_solve<BS, MINB, JT>, BS, smem);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g = max(1, per_sm) * max(1, sms);
    }
    k_scene_solve<BS, MINB, JT><<<min(g, max(1, w.S)), BS, smem, st>>>(w);
}
template <int JT>
static void scene_solve_block(const DW& w, int block, cudaStream_t st) {
    switch (block) {
        case 128: scene_solve_launch<128, 4, JT>(w, st); break;
        case 512: scene_solve_launch<512, 1, JT>(w, st); break;
        default: scene_solve_launch<256, 2, JT>(w, st); break;
    }
}
void launch_scene_solve(const DW& w, const Tune& tune, cudaStream_t st) {
    cudaMemsetAsync(w.ctr + C_SCENE_Q, 0, sizeof(uint32_t), st);
    if (!w.J) scene_solve_block<0>(w, tune.primal_block, st);
    else if (!w.j_all) scene_solve_block<1>(w, tune.primal_block, st);
    else scene_solve_block<2>(w, tune.primal_block, st);
}

// The per-scene solve's fallback for a world with a scene above its limit is
// the split launch.
static inline int launch_lanes(const Tune& tune) { return tune.primal_lanes < 0 ? 0 : tune.primal_lanes; }
void launch_solve_prep(const DW& w, const Tune& tune, cudaStream_t st) {
    if (launch_lanes(tune) != 0) return;
    k_zero_u32<<<1, 256, 0, st>>>(w.side_cnt, 2 * MAX_COLOURS + 2);
    k_side_count<<<gsz(w.pair_cap, SIDE_BLOCK), SIDE_BLOCK, 0, st>>>(w);
    k_side_starts<<<1, 32, 0, st>>>(w);
    k_side_place<<<gsz(w.pair_cap, SIDE_BLOCK), SIDE_BLOCK, 0, st>>>(w);
}
template <int J>
static void primal_colour(const DW& w, const Tune& tune, int c, uint32_t max_bodies, cudaStream_t st) {
    int bs = tune.primal_block;
    switch (launch_lanes(tune)) {
        case 0:
            k_side_rows<<<gsz((size_t)w.pair_cap * 2, 128), 128, 0, st>>>(w, c);
            k_side_solve<J><<<gsz(max_bodies, 128), 128, 0, st>>>(w, c);
            break;
        case 1:
            // occupancy variants of the thread-per-body kernel: 4, 6 or 8
            // resident 128-thread blocks per SM (128, 80 or 64 registers)
            if (tune.primal_minb >= 8) k_primal_thread<8, J><<<nblk(max_bodies, bs), bs, 0, st>>>(w, c);
            else if (tune.primal_minb >= 6) k_primal_thread<6, J><<<nblk(max_bodies, bs), bs, 0, st>>>(w, c);
            else k_primal_thread<4, J><<<nblk(max_bodies, bs), bs, 0, st>>>(w, c);
            break;
        case 4: k_primal_lanes<4, J><<<nblk((size_t)max_bodies * 4, bs), bs, 0, st>>>(w, c); break;
        case 8: k_primal_lanes<8, J><<<nblk((size_t)max_bodies * 8, bs), bs, 0, st>>>(w, c); break;
        case 16: k_primal_lanes<16, J><<<nblk((size_t)max_bodies * 16, bs), bs, 0, st>>>(w, c); break;
        default: k_primal_lanes<32, J><<<nblk((size_t)max_bodies * 32, bs), bs, 0, st>>>(w, c); break;
    }
}
void launch_primal_colour(const DW& w, const Tune& tune, int c, uint32_t max_bodies, cudaStream_t st) {
    if (!w.J) primal_colour<0>(w, tune, c, max_bodies, st);
    else if (!w.j_all) primal_colour<1>(w, tune, c, max_bodies, st);
    else primal_colour<2>(w, tune, c, max_bodies, st);
}
void launch_dual(const DW& w, const Tune& tune, cudaStream_t st) {
    k_dual_pairs<<<gsz(w.pair_cap, 128), 128, 0, st>>>(w);
    if (w.J) {
        if (w.j_all) k_dual_joints<true><<<nblk(w.J, 128), 128, 0, st>>>(w);
        else k_dual_joints<false><<<nblk(w.J, 128), 128, 0, st>>>(w);
    }
}
void launch_iteration(const DW& w, const Tune& tune, int ncolours, cudaStream_t st) {
    for (int c = 0; c < ncolours; c++) AVBD_SOLVE_NS::launch_primal_colour(w, tune, c, (uint32_t)w.N, st);
    AVBD_SOLVE_NS::launch_dual(w, tune, st);
}

// ---- BDF1 + sleep + driver baseline (mod.rs:1060-1142) -------------------------
__global__ void k_bdf1(DW w) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N || !solved(w, h)) return;
    V3 p = ld3(w.pos[h]);
    w.vel[h] = st3((p - ld3(w.pos0[h])) / w.dt, 0.0f);
    Q q = ldq(w.rot[h]);
    V3 spin = quat_diff_vec(q, ldq(w.rot0[h]));
    w.angvel[h] = st3(len(spin) < SPIN_REST_EPS ? V0() : spin / w.dt, 0.0f);
    w.rot[h] = stq(qnormalize(q));
}
// flag bits for the sleep pass: 1 joint-ready, 2 supported, 4 freeze.  Every
// writer of a flag byte within one kernel changes the same bit the same way.
__global__ void k_ready_init(DW w) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < (uint32_t)w.N) w.flag[h] = 1;
}
__global__ void k_ready_joint(DW w) {
    if (aborted_solve(w)) return;
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (uint32_t)w.J) return;
    if (joint_driven(w, j) || joint_rest_error(w, j) > JOINT_REST_ERROR) {
        uint32_t m[4];
        const int nm = joint_members(w, j, m);
        for (int k = 0; k < nm; k++) w.flag[m[k]] &= (uint8_t)~1u;
    }
}
__global__ void k_ready_gather(DW w) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    int c = w.comp[h];
    if (c >= 0 && is_dynamic(w, h) && !(w.flag[h] & 1)) w.comp_flag[c] = 1;
}
__global__ void k_ready_scatter(DW w) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    int c = w.comp[h];
    if (c >= 0 && is_dynamic(w, h) && w.comp_flag[c]) w.flag[h] &= (uint8_t)~1u;
}
__global__ void k_support_joints(DW w) {
    if (aborted_solve(w)) return;
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (uint32_t)w.J) return;
    uint2 ab = w.j_ab[j];
    w.flag[ab.x] |= 2;
    w.flag[ab.y] |= 2;
}
static __device__ __forceinline__ void k_support_one(const DW& w, uint32_t p) {
    if (w.p_n[p].w <= 0.0f && w.p_np[p] > 0) {
        uint2 ab = w.p_ab[p];
        w.flag[ab.x] |= 2;
        w.flag[ab.y] |= 2;
    }
}
__global__ void k_support(DW w) {
    if (aborted_solve(w)) return;
    const uint32_t n = n_pairs(w);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        k_support_one(w, p);
}

__global__ void k_sleep_timer(DW w) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    uint8_t f = w.flag[h];
    bool freeze = w.asleep[h] != 0;
    if (solved(w, h)) {
        if (!(f & 2) || !(f & 1)) {
            w.sleep_timer[h] = 0.0f;
        } else if (len(ld3(w.vel[h])) < SLEEP_LIN && len(ld3(w.angvel[h])) < SLEEP_ANG) {
            float t = w.sleep_timer[h] + w.dt;
            w.sleep_timer[h] = t;
            freeze = t >= SLEEP_TIME;
        } else {
            w.sleep_timer[h] = 0.0f;
        }
    }
    w.flag[h] = freeze ? 4 : 0;
}
__global__ void k_freeze_gather(DW w) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    int c = w.comp[h];
    if (c >= 0 && is_dynamic(w, h) && !(w.flag[h] & 4)) w.comp_flag[c] = 1;
}
__global__ void k_freeze_apply(DW w, int sleep_on) {
    if (aborted_solve(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    if (sleep_on) {
        bool freeze = (w.flag[h] & 4) != 0;
        int c = w.comp[h];
        if (c >= 0 && is_dynamic(w, h) && w.comp_flag[c]) freeze = false;
        if (freeze && !w.asleep[h] && is_dynamic(w, h)) {  // sleep_staticify (body.rs:403-408)
            w.vel[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w.angvel[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w.inv_mass[h] = 0.0f;
            w.inertia[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w.asleep[h] = 1;
        }
        if (w.asleep[h]) agg_inc(&w.ctr[C_SLEEP]);
    }
    w.prev_pos[h] = w.pos[h];
    w.prev_rot[h] = w.rot[h];
}

void launch_finish_substep(const DW& w, cudaStream_t st) {
    unsigned gb = nblk(w.N, 256);
    k_bdf1<<<gb, 256, 0, st>>>(w);
    if (w.enable_sleep) {
        k_ready_init<<<gb, 256, 0, st>>>(w);
        if (w.J) {
            k_ready_joint<<<nblk(w.J, 128), 128, 0, st>>>(w);
            k_comp_clear<<<gb, 256, 0, st>>>(w);
            k_ready_gather<<<gb, 256, 0, st>>>(w);
            k_ready_scatter<<<gb, 256, 0, st>>>(w);
            k_support_joints<<<nblk(w.J, 128), 128, 0, st>>>(w);
        }
        k_support<<<gsz(w.pair_cap, 256), 256, 0, st>>>(w);
        k_sleep_timer<<<gb, 256, 0, st>>>(w);
        k_comp_clear<<<gb, 256, 0, st>>>(w);
        if (w.J) k_freeze_gather<<<gb, 256, 0, st>>>(w);
    }
    k_freeze_apply<<<gb, 256, 0, st>>>(w, w.enable_sleep);
}

}  // namespace AVBD_SOLVE_NS
}  // namespace avbd
