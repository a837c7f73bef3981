// avbd_adjoint.cu — reverse-mode (adjoint) kernels of one AVBD substep.
//
// The forward substep (crates/physics/src/avbd/mod.rs:980-1078: targets and
// warmstart decay, the primal/dual iterations of avbd/assembly.rs and
// avbd/joints_ext.rs, BDF1) is reversed with the contact set, the contact
// frames (normal, friction basis, local anchors) and the colouring held at
// the values the forward computed.  The step-start gap C0 stays a function
// of the step-start poses (joints_ext.rs:21-32, with the witnesses carried
// by the bodies for sphere pairs), the warm lambda / penalty state flows
// across substeps through the point inheritance of the discovery merge, and
// every clamp, cone and liveness test keeps the branch the forward took.
//
// Order of one substep's reverse:
//   k_adj_bdf          BDF1 velocities and the quaternion renormalisation
//   per iteration, last first:
//     k_adj_dual       the dual update of every point (4 lanes per pair);
//                      k_adj_dual_joints that of every joint
//     per colour, last first:
//       k_adj_solve    each body's block solve (thread per body)
//       k_adj_sides    its contact rows (4 lanes per pair side)
//   k_adj_c0           C0 and the warmstart decay (k_adj_decay_joints: joints')
//   k_adj_start        the inertial targets -> previous substep's state
//   k_adj_inherit      point adjoints -> the previous generation's points
//   k_adj_mu_scene     friction adjoint summed per scene
// A body's update x1 = x + d, q1 = integrate(q, d_ang), d = -H^-1 r, has the
// adjoint  s_bar = -(d(r + H d)/ds)^T H^-1 d_bar  for every input s; each
// stamped row contributes through its force, penalty and lever.
#include "avbd_common.cuh"
#include "avbd_adjoint.cuh"

namespace avbd {

static __device__ __forceinline__ size_t pslice(const DW& w, int s) { return (size_t)s * (size_t)w.N; }

// Pose slice in which body o is seen by a body of colour c during iteration
// it: bodies of lower colours have already moved in this iteration.
static __device__ __forceinline__ int seen_slice(const AdjFrame& f, uint32_t o, int c, int it) {
    int co = f.colour[o];
    return (co >= 0 && co < c) ? it + 1 : it;
}

static __device__ __forceinline__ void adj_ctx(const DW& w, const AdjFrame& f, uint32_t p, int sa, int sb, PairCtx& c,
                                               Q& qa0, Q& qb0) {
    uint2 ab = f.p_ab[p];
    float4 n4 = f.p_n[p];
    c.a = ab.x;
    c.b = ab.y;
    c.n = ld3(n4);
    c.gap = n4.w;
    c.mu = f.p_mu[p];
    c.np = f.p_np[p];
    c.pa = ld3(f.it_pos[pslice(w, sa) + c.a]);
    c.qa = ldq(f.it_rot[pslice(w, sa) + c.a]);
    c.pb = ld3(f.it_pos[pslice(w, sb) + c.b]);
    c.qb = ldq(f.it_rot[pslice(w, sb) + c.b]);
    qa0 = ldq(f.rot0[c.a]);
    qb0 = ldq(f.rot0[c.b]);
    c.dxa = c.pa - ld3(f.pos0[c.a]);
    c.dxb = c.pb - ld3(f.pos0[c.b]);
    c.dra = quat_diff_vec(c.qa, qa0);
    c.drb = quat_diff_vec(c.qb, qb0);
    const uint32_t sha = info_shape(w.info[c.a]), shb = info_shape(w.info[c.b]);
    c.sph_a = sha == AVBD_SHAPE_SPHERE;
    c.sph_b = shb == AVBD_SHAPE_SPHERE;
    c.roll_a = sha == AVBD_SHAPE_CAPSULE && shb != AVBD_SHAPE_BOX;
    c.roll_b = shb == AVBD_SHAPE_CAPSULE && sha != AVBD_SHAPE_BOX;
    c.rad_a = w.shp[c.a].x;
    c.rad_b = w.shp[c.b].x;
    c.mu_roll = 0.0f;
    c.mu_spin = 0.0f;
    c.t1 = tangent_t1(c.n);
    c.t2 = cross(c.t1, c.n);
}

// Separated-point damper gate and stiffness (assembly.rs:113-175); false when
// the point stamps nothing.
static __device__ __forceinline__ bool damper(const DW& w, const AdjFrame& f, const PairCtx& c, float cn, float& pen_d) {
    float approach = fmaxf(dot(ld3(f.vel[c.b]) - ld3(f.vel[c.a]), c.n), 0.0f);
    if (c.gap - approach * w.dt > 0.0f) return false;
    if (fabsf(cn) < C_EPS) return false;
    float npts = (float)max(c.np, 1u);
    float ka = is_dynamic(w, c.a) ? f.inv_mass[c.a] : 0.0f;
    float kb = is_dynamic(w, c.b) ? f.inv_mass[c.b] : 0.0f;
    float m_red = ka + kb > NEAR_ZERO ? 1.0f / (ka + kb) : 0.0f;
    if (!(m_red > 0.0f)) return false;
    pen_d = fminf(2.0f * m_red / (w.dt * w.dt) / npts, PENALTY_MAX);
    return true;
}

// One stamped row J = [s a; r x (s a)] with H += pen J J^T, rhs += f J: the
// seeds of s_bar = -d/ds [w.(rhs + H d)] for its force, penalty and lever.
static __device__ __forceinline__ void row_bwd(V3 axis, float pen, float fo, V3 r, float sign, const float w6[6],
                                               const float d6[6], float& gf, float& gpen, V3& gr) {
    V3 nn = sign * axis;
    V3 t = cross(r, nn);
    V3 wl{w6[0], w6[1], w6[2]}, wa{w6[3], w6[4], w6[5]};
    V3 dl{d6[0], d6[1], d6[2]}, da{d6[3], d6[4], d6[5]};
    float a = dot(nn, wl) + dot(t, wa);
    float dd = dot(nn, dl) + dot(t, da);
    gf -= a;
    gpen -= a * dd;
    V3 gja = -(wa * fo + (wa * dd + da * a) * pen);
    gr = gr + cross(nn, gja);
}

// friction_levers (rows.rs:987-996): sep = n.((pa + raw) - (pb + rbw)),
// raf = raw - n sep/2, rbf = rbw + n sep/2.
static __device__ __forceinline__ void friction_levers_bwd(const PairCtx& c, V3 graf, V3 grbf, V3& graw, V3& grbw,
                                                           PairGrad& pg) {
    float gsep = HALF * dot(c.n, grbf - graf);
    graw = graw + graf + c.n * gsep;
    grbw = grbw + grbf - c.n * gsep;
    pg.xa = pg.xa + c.n * gsep;
    pg.xb = pg.xb - c.n * gsep;
}
// contact_levers (rows.rs:963-973): a non-sphere lever is the anchor rotated
// by the body; a sphere's is fixed by the (frozen) normal.
static __device__ __forceinline__ void contact_levers_bwd(const PairCtx& c, Q qa0, Q qb0, float4 ra, float4 rb,
                                                          V3 graw, V3 grbw, PairGrad& pg) {
    V3 gla = V0(), glb = V0();
    if (!c.sph_a) qrot_bwd(c.qa, ld3(ra), graw, pg.qa, gla);
    if (!c.sph_b) qrot_bwd(c.qb, ld3(rb), grbw, pg.qb, glb);
    if (ra.w == 0.0f) {
        if (c.roll_a) rolling_anchor_bwd(qa0, c.n, -c.rad_a, gla, pg.qa0);
        if (c.roll_b) rolling_anchor_bwd(qb0, c.n, c.rad_b, glb, pg.qb0);
    }
}

// Adjoint of one point's rows in a block solve of the body on side is_a.
static __device__ __forceinline__ void adj_point_bwd(const DW& w, const AdjFrame& f, const PairCtx& c, Q qa0, Q qb0,
                                                     uint32_t q, bool is_a, float4 lam, float4 pen, const float w6[6],
                                                     const float d6[6], PairGrad& pg, float4& glam, float4& gpen,
                                                     float2& gmu) {
    float4 ra = f.q_ra[q], rb = f.q_rb[q];
    float sign = is_a ? 1.0f : -1.0f;
    bool touching = c.gap <= 0.0f;
    float c0 = touching ? lam.w : 0.0f;
    V3 rup, rlo;
    contact_levers(c, ra, rb, rup, rlo);
    float cn = row_c_levers(c, c.n, c0, rup, rlo);
    V3 graw = V0(), grbw = V0();
    float gcn = 0.0f, gc0 = 0.0f;
    if (!touching) {
        float pen_d;
        if (!damper(w, f, c, cn, pen_d)) return;
        float fd = fminf(pen_d * cn, 0.0f);
        float gf = 0.0f, gp = 0.0f;
        V3 gr = V0();
        row_bwd(c.n, pen_d, fd, is_a ? rup : rlo, sign, w6, d6, gf, gp, gr);
        if (pen_d * cn < 0.0f) gcn += pen_d * gf;
        if (is_a) graw = graw + gr;
        else grbw = grbw + gr;
    } else {
        V3 raf, rbf;
        friction_levers(c, rup, rlo, raf, rbf);
        float ct1 = row_c_levers(c, c.t1, 0.0f, raf, rbf);
        float ct2 = row_c_levers(c, c.t2, 0.0f, raf, rbf);
        float fo[3];
        contact_force(cn, pen, lam, ct1, ct2, c.mu, fo);
        float gf[3] = {0.0f, 0.0f, 0.0f};
        V3 gr = V0(), grf = V0();
        if (row_live(cn, fo[0])) row_bwd(c.n, pen.x, fo[0], is_a ? rup : rlo, sign, w6, d6, gf[0], gpen.x, gr);
        if (row_live(ct1, fo[1])) row_bwd(c.t1, pen.y, fo[1], is_a ? raf : rbf, sign, w6, d6, gf[1], gpen.y, grf);
        if (row_live(ct2, fo[2])) row_bwd(c.t2, pen.z, fo[2], is_a ? raf : rbf, sign, w6, d6, gf[2], gpen.z, grf);
        float gct1 = 0.0f, gct2 = 0.0f;
        contact_force_bwd(cn, pen, lam, ct1, ct2, c.mu, gf, gcn, gpen, glam, gct1, gct2, gmu);
        V3 graf = is_a ? grf : V0(), grbf = is_a ? V0() : grf;
        float unused = 0.0f;
        row_c_bwd(c, qa0, qb0, c.t1, raf, rbf, gct1, unused, graf, grbf, pg);
        row_c_bwd(c, qa0, qb0, c.t2, raf, rbf, gct2, unused, graf, grbf, pg);
        friction_levers_bwd(c, graf, grbf, graw, grbw, pg);
        if (is_a) graw = graw + gr;
        else grbw = grbw + gr;
    }
    row_c_bwd(c, qa0, qb0, c.n, rup, rlo, gcn, gc0, graw, grbw, pg);
    contact_levers_bwd(c, qa0, qb0, ra, rb, graw, grbw, pg);
    glam.w += gc0;
}

// inertial block (assembly.rs:74-96) with the frame's masses and targets
static __device__ __forceinline__ void adj_inertial(const DW& w, const AdjFrame& f, uint32_t h, V3 x, Q q, Sys& s) {
    float dt2 = w.dt * w.dt;
    float im = is_dynamic(w, h) ? f.inv_mass[h] : 0.0f;
    float m_dt2 = 1.0f / im / dt2;
    float iw[3][3];
    world_inertia(ld3(f.inertia[h]), q, iw);
    for (int i = 0; i < 21; i++) s.h[i] = 0.0f;
    s.h[tri(0, 0)] = m_dt2;
    s.h[tri(1, 1)] = m_dt2;
    s.h[tri(2, 2)] = m_dt2;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b <= a; b++) s.h[tri(3 + a, 3 + b)] = iw[a][b] / dt2;
    V3 rl = m_dt2 * (x - ld3(f.inertial[h]));
    s.r[0] = rl.x;
    s.r[1] = rl.y;
    s.r[2] = rl.z;
    V3 ra = mat3_vec(iw, quat_diff_vec(q, ldq(f.inertial_rot[h]))) / dt2;
    s.r[3] = ra.x;
    s.r[4] = ra.y;
    s.r[5] = ra.z;
}

static __device__ __forceinline__ float4* slot_of(const AdjFrame& f, const AdjState& A, uint32_t p, bool side_a,
                                                  uint2 ab) {
    uint32_t k = side_a ? p + f.offB[ab.x + 1] : f.offA[ab.y] + f.posB[p];
    return A.slot + (size_t)k * 4;
}
static __device__ __forceinline__ void slot_add(float4* s, V3 x, Q q, V3 x0, Q q0) {
    float4 a = s[0], b = s[1], c = s[2], d = s[3];
    s[0] = make_float4(a.x + x.x, a.y + x.y, a.z + x.z, 0.0f);
    s[1] = make_float4(b.x + q.x, b.y + q.y, b.z + q.z, b.w + q.w);
    s[2] = make_float4(c.x + x0.x, c.y + x0.y, c.z + x0.z, 0.0f);
    s[3] = make_float4(d.x + q0.x, d.y + q0.y, d.z + q0.z, d.w + q0.w);
}
// Sum a PairGrad and a float2 over the ADJ_LANES lanes of a group.
constexpr int ADJ_LANES = 4;
static __device__ __forceinline__ float lsum(float v) {
#pragma unroll
    for (int o = ADJ_LANES / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, ADJ_LANES);
    return v;
}
static __device__ __forceinline__ V3 lsum(V3 v) { return {lsum(v.x), lsum(v.y), lsum(v.z)}; }
static __device__ __forceinline__ Q lsum(Q v) { return {lsum(v.x), lsum(v.y), lsum(v.z), lsum(v.w)}; }
static __device__ __forceinline__ void lsum(PairGrad& g, float2& m) {
    g.xa = lsum(g.xa); g.xb = lsum(g.xb); g.xa0 = lsum(g.xa0); g.xb0 = lsum(g.xb0);
    g.qa = lsum(g.qa); g.qb = lsum(g.qb); g.qa0 = lsum(g.qa0); g.qb0 = lsum(g.qb0);
    m.x = lsum(m.x);
    m.y = lsum(m.y);
}
static __device__ __forceinline__ float4 f4add(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// ---- joints ----------------------------------------------------------------
static __device__ __forceinline__ const float4* jslice(const DW& w, const AdjFrame& f, int s) {
    return f.it_joint + (size_t)s * 5 * (size_t)w.J;
}
static __device__ __forceinline__ JDef jdef(const DW& w, uint32_t j) {
    JDef d;
    float4 axa = w.j_axa[j];
    d.la = ld3(w.j_la[j]);
    d.lb = ld3(w.j_lb[j]);
    d.axa_l = ld3(axa);
    d.axb_l = ld3(w.j_axb[j]);
    d.ref = axa.w;
    d.revolute = w.j_kind[j] == AVBD_JOINT_REVOLUTE;
    d.lim = w.j_lim[j];
    return d;
}
static __device__ __forceinline__ JState jstate(const DW& w, const AdjFrame& f, uint32_t j, int s) {
    const float4* b = jslice(w, f, s);
    const size_t J = (size_t)w.J;
    JState st;
    st.laml = b[j];
    st.penl = b[J + j];
    st.lama = b[2 * J + j];
    st.pena = b[3 * J + j];
    st.acc = b[4 * J + j].w;
    return st;
}
static __device__ __forceinline__ JPose jpose(const DW& w, const AdjFrame& f, uint2 ab, int sa, int sb) {
    JPose p;
    p.xa = ld3(f.it_pos[pslice(w, sa) + ab.x]);
    p.qa = ldq(f.it_rot[pslice(w, sa) + ab.x]);
    p.xb = ld3(f.it_pos[pslice(w, sb) + ab.y]);
    p.qb = ldq(f.it_rot[pslice(w, sb) + ab.y]);
    p.xa0 = ld3(f.pos0[ab.x]);
    p.qa0 = ldq(f.rot0[ab.x]);
    p.xb0 = ld3(f.pos0[ab.y]);
    p.qb0 = ldq(f.rot0[ab.y]);
    return p;
}
static __device__ __forceinline__ JState ajs_load(const AdjState& A, uint32_t j) {
    const float4* g = A.ajs + (size_t)j * 5;
    JState st;
    st.laml = g[0];
    st.penl = g[1];
    st.lama = g[2];
    st.pena = g[3];
    st.acc = g[4].w;
    return st;
}
static __device__ __forceinline__ void ajs_store(const AdjState& A, uint32_t j, const JState& st) {
    float4* g = A.ajs + (size_t)j * 5;
    g[0] = st.laml;
    g[1] = st.penl;
    g[2] = st.lama;
    g[3] = st.pena;
    g[4] = make_float4(0.0f, 0.0f, 0.0f, st.acc);
}
static __device__ __forceinline__ JState jstate_add(JState a, const JState& b) {
    a.laml = f4add(a.laml, b.laml);
    a.penl = f4add(a.penl, b.penl);
    a.lama = f4add(a.lama, b.lama);
    a.pena = f4add(a.pena, b.pena);
    a.acc += b.acc;
    return a;
}

// ---- BDF1 (mod.rs:1060-1078) --------------------------------------------------
__global__ void k_adj_bdf(DW w, AdjFrame f, AdjState A, int iters) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h == 0) *A.nlong = 0u;
    if (h >= (uint32_t)w.N) return;
    A.ay[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    A.aqt[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (f.colour[h] < 0) {  // not swept: its pose and velocities pass through the substep
        A.ax0[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        A.aq0[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    float dt = w.dt;
    V3 xk = ld3(f.it_pos[pslice(w, iters) + h]);
    Q qk = ldq(f.it_rot[pslice(w, iters) + h]);
    Q q0 = ldq(f.rot0[h]);
    (void)xk;
    V3 gv = ld3(A.av[h]), gw = ld3(A.aw[h]);
    if (f.asleep_end[h]) gv = gw = V0();  // frozen at the end of the substep: velocities zeroed
    V3 gx = ld3(A.ax[h]) + gv / dt;
    V3 gx0 = -(gv / dt);
    Q gq = qnormalize_bwd(qk, ldq(A.aq[h]));
    Q gq0 = Q0();
    V3 spin = quat_diff_vec(qk, q0);
    if (len(spin) >= SPIN_REST_EPS) quat_diff_vec_bwd(qk, q0, gw / dt, gq, gq0);
    A.ax[h] = st3(gx, 0.0f);
    A.aq[h] = stq(gq);
    A.ax0[h] = st3(gx0, 0.0f);
    A.aq0[h] = stq(gq0);
    A.av[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    A.aw[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// ---- dual update (joints_ext.rs:464-573), ADJ_LANES lanes per pair -------------
// Lane l of a pair's group takes points l, l + ADJ_LANES, ...; the pose and
// friction adjoints are summed over the group before lane 0 stores them.
__global__ void __launch_bounds__(128, 3) k_adj_dual(DW w, AdjFrame f, AdjState A, int it) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t p = gid / ADJ_LANES;
    const int lane = (int)(threadIdx.x % ADJ_LANES);
    const bool active = p < f.npairs && f.p_np[p] != 0 && f.p_n[p].w <= 0.0f;  // separated points keep lambda
    PairGrad pg;
    pair_grad_zero(pg);
    float2 gmu = make_float2(0.0f, 0.0f);
    PairCtx c;
    Q qa0 = Q0(), qb0 = Q0();
    if (active) {
        adj_ctx(w, f, p, it + 1, it + 1, c, qa0, qb0);
        for (uint32_t k = lane; k < c.np; k += ADJ_LANES) {
            uint32_t q = p * MAX_PTS + k;
            size_t qi = (size_t)it * f.qstride + q;
            float4 lam = f.it_lam[qi], pen = f.it_pen[qi];
            float4 gl = A.alam[q], gp = A.apen[q];
            float4 ra = f.q_ra[q], rb = f.q_rb[q];
            float c0 = lam.w;
            V3 raw, rbw;
            contact_levers(c, ra, rb, raw, rbw);
            float cn = row_c_levers(c, c.n, c0, raw, rbw);
            V3 raf, rbf;
            friction_levers(c, raw, rbw, raf, rbf);
            float ct1 = row_c_levers(c, c.t1, 0.0f, raf, rbf);
            float ct2 = row_c_levers(c, c.t2, 0.0f, raf, rbf);
            float fo[3];
            contact_force(cn, pen, lam, ct1, ct2, c.mu, fo);
            float fu0 = pen.y * ct1 + lam.y, fu1 = pen.z * ct2 + lam.z;
            float b1 = fabsf(fo[0]) * c.mu.x, b2 = fabsf(fo[0]) * c.mu.y;
            float s_ell = (b1 > 0.0f && b2 > 0.0f) ? (fu0 / b1) * (fu0 / b1) + (fu1 / b2) * (fu1 / b2) : INFINITY;
            float4 glo = make_float4(0.0f, 0.0f, 0.0f, gl.w), gpo = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            float gf[3] = {0.0f, 0.0f, 0.0f};
            float gcn = 0.0f, gct1 = 0.0f, gct2 = 0.0f;
            if (fabsf(cn) >= C_EPS) {
                gf[0] += gl.x;
                if (fo[0] < 0.0f) {
                    if (pen.x + BETA * fabsf(cn) < PENALTY_MAX) {
                        gpo.x += gp.x;
                        gcn += BETA * copysignf(1.0f, cn) * gp.x;
                    }
                } else {
                    gpo.x += gp.x;
                }
            } else {
                glo.x += gl.x;
                gpo.x += gp.x;
            }
            gf[1] += gl.y;
            gf[2] += gl.z;
            float cts[2] = {ct1, ct2}, pts[2] = {pen.y, pen.z}, gps[2] = {gp.y, gp.z};
            float gpt[2] = {0.0f, 0.0f}, gct[2] = {0.0f, 0.0f};
            for (int k2 = 0; k2 < 2; k2++) {
                if (s_ell <= 1.0f && fabsf(cts[k2]) >= C_EPS) {
                    if (pts[k2] + BETA * fabsf(cts[k2]) < PENALTY_MAX) {
                        gpt[k2] += gps[k2];
                        gct[k2] += BETA * copysignf(1.0f, cts[k2]) * gps[k2];
                    }
                } else {
                    gpt[k2] += gps[k2];
                }
            }
            gpo.y += gpt[0];
            gpo.z += gpt[1];
            gct1 += gct[0];
            gct2 += gct[1];
            contact_force_bwd(cn, pen, lam, ct1, ct2, c.mu, gf, gcn, gpo, glo, gct1, gct2, gmu);
            V3 graw = V0(), grbw = V0(), graf = V0(), grbf = V0();
            float gc0 = 0.0f, unused = 0.0f;
            row_c_bwd(c, qa0, qb0, c.t1, raf, rbf, gct1, unused, graf, grbf, pg);
            row_c_bwd(c, qa0, qb0, c.t2, raf, rbf, gct2, unused, graf, grbf, pg);
            friction_levers_bwd(c, graf, grbf, graw, grbw, pg);
            row_c_bwd(c, qa0, qb0, c.n, raw, rbw, gcn, gc0, graw, grbw, pg);
            contact_levers_bwd(c, qa0, qb0, ra, rb, graw, grbw, pg);
            glo.w += gc0;
            A.alam[q] = glo;
            A.apen[q] = gpo;
        }
    }
    lsum(pg, gmu);
    if (!active || lane != 0) return;
    uint2 ab = make_uint2(c.a, c.b);
    slot_add(slot_of(f, A, p, true, ab), pg.xa, pg.qa, pg.xa0, pg.qa0);
    slot_add(slot_of(f, A, p, false, ab), pg.xb, pg.qb, pg.xb0, pg.qb0);
    float2 m = A.amu[p];
    A.amu[p] = make_float2(m.x + gmu.x, m.y + gmu.y);
}

// ---- primal block solve of one colour (assembly.rs:73-903) --------------------
// Two passes per colour, like the forward's split primal.  k_adj_solve (one
// thread per body) rebuilds the body's system from its inertial block and
// the per-incidence row sums the recompute kept, solves for the step d and
// for w = H^-1 d_bar, and takes the inertial rows' adjoint; k_adj_sides (one
// thread per (pair, side)) takes the adjoint of that side's contact rows and
// leaves the results in the incidence slots of both bodies of the pair.
// JOINTS = false: a world without joints (the joint code would cost it
// registers and occupancy).
template <bool JOINTS>
__global__ void __launch_bounds__(128) k_adj_solve(DW w, AdjFrame f, AdjState A, int it, int colour) {
    const uint32_t c0 = f.col_cnt[colour], c1 = f.col_cnt[colour + 1];
    for (uint32_t i = c0 + blockIdx.x * blockDim.x + threadIdx.x; i < c1; i += gridDim.x * blockDim.x) {
        uint32_t h = f.col_list[i];
        V3 gx = ld3(A.ax[h]);
        Q gq = ldq(A.aq[h]);
        const uint32_t k0 = f.offA[h] + f.offB[h], k1 = f.offA[h + 1] + f.offB[h + 1];
        for (uint32_t k = k0; k < k1; k++) {
            float4* sl = A.slot + (size_t)k * 4;
            gx = gx + ld3(sl[0]);
            gq = qadd(gq, ldq(sl[1]));
            sl[0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            sl[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        const uint32_t j0 = JOINTS ? w.jofs[h] : 0u, j1 = JOINTS ? w.jofs[h + 1] : 0u;
        for (uint32_t k = j0; k < j1; k++) {
            uint32_t j = w.jlist[k];
            float4* sl = A.jslot + ((size_t)j * 2 + (w.j_ab[j].x == h ? 0u : 1u)) * 4;
            gx = gx + ld3(sl[0]);
            gq = qadd(gq, ldq(sl[1]));
            sl[0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            sl[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        V3 x = ld3(f.it_pos[pslice(w, it) + h]);
        Q q = ldq(f.it_rot[pslice(w, it) + h]);
        Sys s;
        adj_inertial(w, f, h, x, q, s);
        const float4* cb = f.it_contrib + (size_t)it * f.cstride;
        for (uint32_t k = k0; k < k1; k++) {  // incidence order, as the forward sums them
            const float4* o = cb + (size_t)k * 7;
            float4 v0 = o[0], v1 = o[1], v2 = o[2], v3 = o[3], v4 = o[4], v5 = o[5], v6 = o[6];
            s.h[0] += v0.x; s.h[1] += v0.y; s.h[2] += v0.z; s.h[3] += v0.w;
            s.h[4] += v1.x; s.h[5] += v1.y; s.h[6] += v1.z; s.h[7] += v1.w;
            s.h[8] += v2.x; s.h[9] += v2.y; s.h[10] += v2.z; s.h[11] += v2.w;
            s.h[12] += v3.x; s.h[13] += v3.y; s.h[14] += v3.z; s.h[15] += v3.w;
            s.h[16] += v4.x; s.h[17] += v4.y; s.h[18] += v4.z; s.h[19] += v4.w;
            s.h[20] += v5.x; s.r[0] += v5.y; s.r[1] += v5.z; s.r[2] += v5.w;
            s.r[3] += v6.x; s.r[4] += v6.y; s.r[5] += v6.z;
        }
        for (uint32_t k = j0; k < j1; k++) {  // joints after the contact rows, as the forward
            uint32_t j = w.jlist[k];
            uint2 ab = w.j_ab[j];
            bool is_a = ab.x == h;
            JPose jp = is_a ? jpose(w, f, ab, it, seen_slice(f, ab.y, colour, it))
                            : jpose(w, f, ab, seen_slice(f, ab.x, colour, it), it);
            joint_stamp(jdef(w, j), jp, jstate(w, f, j, it), is_a, s);
        }
        float4* wd = A.wd + (size_t)h * 3;
        float d6[6];
        if (!solve_6x6(s, d6)) {  // breakdown: the forward skipped the update
            A.ax[h] = st3(gx, 0.0f);
            A.aq[h] = stq(gq);
            wd[0] = wd[1] = wd[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        V3 dang{d6[3], d6[4], d6[5]};
        Q gqb = Q0();
        V3 gdang = V0();
        quat_integrate_bwd(q, dang, gq, gqb, gdang);
        Sys s2 = s;
        s2.r[0] = -gx.x;
        s2.r[1] = -gx.y;
        s2.r[2] = -gx.z;
        s2.r[3] = -gdang.x;
        s2.r[4] = -gdang.y;
        s2.r[5] = -gdang.z;
        float w6[6];
        solve_6x6(s2, w6);  // w = H^-1 d_bar
        // inertial rows: -d/ds [w.(rhs + H d)] of the mass and inertia blocks
        float dt2 = w.dt * w.dt;
        float m_dt2 = 1.0f / f.inv_mass[h] / dt2;
        V3 wl{w6[0], w6[1], w6[2]}, wa{w6[3], w6[4], w6[5]};
        V3 gxb = gx - wl * m_dt2;
        float4 ay = A.ay[h];
        A.ay[h] = make_float4(ay.x + wl.x * m_dt2, ay.y + wl.y * m_dt2, ay.z + wl.z * m_dt2, 0.0f);
        Q qt = ldq(f.inertial_rot[h]);
        V3 inr = ld3(f.inertia[h]);
        float iw[3][3];
        world_inertia(inr, q, iw);
        V3 th = quat_diff_vec(q, qt);
        V3 gth = mat3_vec(iw, wa) * (-1.0f / dt2);
        Q gqt = Q0();
        quat_diff_vec_bwd(q, qt, gth, gqb, gqt);
        world_inertia_bwd(inr, q, wa, th + dang, -1.0f / dt2, gqb);
        A.aqt[h] = f4add(A.aqt[h], stq(gqt));
        A.ax[h] = st3(gxb, 0.0f);
        A.aq[h] = stq(gqb);
        wd[0] = make_float4(w6[0], w6[1], w6[2], w6[3]);
        wd[1] = make_float4(w6[4], w6[5], d6[0], d6[1]);
        wd[2] = make_float4(d6[2], d6[3], d6[4], d6[5]);
    }
}

// The joint rows of the colour's bodies, one thread per (joint, side): the
// adjoint of the side's stamp with that body's w and d.  Both bodies'
// results go to the joint's slots; the side's own pose adjoint is gathered
// with the rest of its slots before the body's previous update.  The two
// bodies of a joint never share a colour, so one launch writes each joint's
// state adjoint once.
__global__ void __launch_bounds__(128) k_adj_joint_sides(DW w, AdjFrame f, AdjState A, int it, int colour) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < 2u * (uint32_t)w.J; e += gridDim.x * blockDim.x) {
        const uint32_t j = e >> 1;
        const bool is_a = (e & 1u) == 0u;
        const uint2 ab = w.j_ab[j];
        const uint32_t h = is_a ? ab.x : ab.y;
        if (f.colour[h] != colour) continue;
        const float4* wd = A.wd + (size_t)h * 3;
        const float4 x0 = wd[0], x1 = wd[1], x2 = wd[2];
        const float w6[6] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y};
        const float d6[6] = {x1.z, x1.w, x2.x, x2.y, x2.z, x2.w};
        JPose jp = is_a ? jpose(w, f, ab, it, seen_slice(f, ab.y, colour, it))
                        : jpose(w, f, ab, seen_slice(f, ab.x, colour, it), it);
        PairGrad pg;
        pair_grad_zero(pg);
        JState gs;
        jstate_zero(gs);
        joint_stamp_bwd(jdef(w, j), jp, jstate(w, f, j, it), is_a, w6, d6, pg, gs);
        ajs_store(A, j, jstate_add(ajs_load(A, j), gs));
        slot_add(A.jslot + ((size_t)j * 2) * 4, pg.xa, pg.qa, pg.xa0, pg.qa0);
        slot_add(A.jslot + ((size_t)j * 2 + 1u) * 4, pg.xb, pg.qb, pg.xb0, pg.qb0);
    }
}

__global__ void __launch_bounds__(128, 3) k_adj_sides(DW w, AdjFrame f, AdjState A, int it, int colour) {
    const uint32_t s0 = f.side_cnt[colour], s1 = f.side_cnt[colour + 1];
    const size_t qoff = (size_t)it * f.qstride;
    const uint32_t i = s0 + (blockIdx.x * blockDim.x + threadIdx.x) / ADJ_LANES;
    const int lane = (int)(threadIdx.x % ADJ_LANES);
    const bool active = i < s1;
    PairGrad pg;
    pair_grad_zero(pg);
    float2 gmu = make_float2(0.0f, 0.0f);
    uint32_t p = 0;
    uint2 ab = make_uint2(0u, 0u);
    if (active) {
        uint32_t e = f.side_list[i];
        p = e >> 1;
        bool is_a = (e & 1u) != 0u;
        ab = f.p_ab[p];
        uint32_t h = is_a ? ab.x : ab.y;
        const float4* wd = A.wd + (size_t)h * 3;
        float4 x0 = wd[0], x1 = wd[1], x2 = wd[2];
        const float w6[6] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y};
        const float d6[6] = {x1.z, x1.w, x2.x, x2.y, x2.z, x2.w};
        PairCtx c;
        Q qa0, qb0;
        if (is_a) adj_ctx(w, f, p, it, seen_slice(f, ab.y, colour, it), c, qa0, qb0);
        else adj_ctx(w, f, p, seen_slice(f, ab.x, colour, it), it, c, qa0, qb0);
        for (uint32_t k = lane; k < c.np; k += ADJ_LANES) {
            uint32_t q = p * MAX_PTS + k;
            float4 glam = make_float4(0.0f, 0.0f, 0.0f, 0.0f), gpen = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            adj_point_bwd(w, f, c, qa0, qb0, q, is_a, f.it_lam[qoff + q], f.it_pen[qoff + q], w6, d6, pg, glam, gpen,
                          gmu);
            A.alam[q] = f4add(A.alam[q], glam);
            A.apen[q] = f4add(A.apen[q], gpen);
        }
    }
    lsum(pg, gmu);
    if (!active || lane != 0) return;
    // the body's own adjoint (of its pose before this update) and its
    // partner's both wait in the slots until the next gather
    slot_add(slot_of(f, A, p, true, ab), pg.xa, pg.qa, pg.xa0, pg.qa0);
    slot_add(slot_of(f, A, p, false, ab), pg.xb, pg.qb, pg.xb0, pg.qb0);
    float2 m = A.amu[p];
    A.amu[p] = make_float2(m.x + gmu.x, m.y + gmu.y);
}

// ---- joint dual update (joints_ext.rs:574-896), one thread per joint -----------
__global__ void k_adj_dual_joints(DW w, AdjFrame f, AdjState A, int it) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (uint32_t)w.J) return;
    uint2 ab = w.j_ab[j];
    PairGrad pg;
    pair_grad_zero(pg);
    JState gin;
    float gk = 0.0f;
    joint_dual_bwd(jdef(w, j), jpose(w, f, ab, it + 1, it + 1), jstate(w, f, j, it), w.joint_k, ajs_load(A, j), gin,
                   pg, gk);
    ajs_store(A, j, gin);
    A.ajk[j] += gk;
    slot_add(A.jslot + (size_t)j * 8, pg.xa, pg.qa, pg.xa0, pg.qa0);
    slot_add(A.jslot + (size_t)j * 8 + 4, pg.xb, pg.qb, pg.xb0, pg.qb0);
}
// joint warmstart decay (mod.rs:1019-1040): lambda * alpha gamma; penalty
// clamp(p gamma), or the stiffness for the rows of a soft joint
__global__ void k_adj_decay_joints(DW w, AdjFrame f, AdjState A) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (uint32_t)w.J) return;
    const float ag = ALPHA * GAMMA, K = w.joint_k;
    JState g = ajs_load(A, j), s0 = jstate(w, f, j, 0);
    float gk = 0.0f;
    auto pen_bwd = [&](float after, float gp, bool soft) {
        if (soft && K > 0.0f) {
            gk += gp;
            return 0.0f;
        }
        return (after > PENALTY_MIN && after < PENALTY_MAX) ? gp * GAMMA : 0.0f;
    };
    g.laml = make_float4(g.laml.x * ag, g.laml.y * ag, g.laml.z * ag, 0.0f);
    g.lama = make_float4(g.lama.x * ag, g.lama.y * ag, g.lama.z * ag, 0.0f);
    g.penl = make_float4(pen_bwd(s0.penl.x, g.penl.x, true), pen_bwd(s0.penl.y, g.penl.y, true),
                         pen_bwd(s0.penl.z, g.penl.z, true), 0.0f);
    g.pena = make_float4(pen_bwd(s0.pena.x, g.pena.x, true), pen_bwd(s0.pena.y, g.pena.y, true),
                         pen_bwd(s0.pena.z, g.pena.z, false), 0.0f);
    ajs_store(A, j, g);
    A.ajk[j] += gk;
}

// ---- C0 and the warmstart decay (joints_ext.rs:21-32, mod.rs:1019-1040) -------
__global__ void k_adj_c0(DW w, AdjFrame f, AdjState A) {
    const float ag = ALPHA * GAMMA;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < f.npairs; p += gridDim.x * blockDim.x) {
        uint32_t np = f.p_np[p];
        if (np == 0) continue;
        uint2 ab = f.p_ab[p];
        float4 n4 = f.p_n[p];
        V3 n = ld3(n4);
        bool touching = n4.w <= 0.0f;
        bool sa = info_shape(w.info[ab.x]) == AVBD_SHAPE_SPHERE, sb = info_shape(w.info[ab.y]) == AVBD_SHAPE_SPHERE;
        Q qa0 = ldq(f.rot0[ab.x]), qb0 = ldq(f.rot0[ab.y]);
        PairGrad pg;
        pair_grad_zero(pg);
        for (uint32_t k = 0; k < np; k++) {
            uint32_t q = p * MAX_PTS + k;
            float4 gl = A.alam[q], gp = A.apen[q];
            if (touching && gl.w != 0.0f) {
                // C0 = n.(w_a - w_b) + margin with the witnesses carried by the bodies
                V3 g = n * gl.w;
                V3 dummy = V0();
                pg.xa0 = pg.xa0 + g;
                if (!sa) qrot_bwd(qa0, ld3(f.q_ra[q]), g, pg.qa0, dummy);
                pg.xb0 = pg.xb0 - g;
                if (!sb) qrot_bwd(qb0, ld3(f.q_rb[q]), -g, pg.qb0, dummy);
            }
            float4 pen0 = f.it_pen[q];  // slice 0: after the decay clamp
            auto keep = [](float v) { return v > PENALTY_MIN && v < PENALTY_MAX; };
            A.alam[q] = make_float4(gl.x * ag, gl.y * ag, gl.z * ag, 0.0f);
            A.apen[q] = make_float4(keep(pen0.x) ? gp.x * GAMMA : 0.0f, keep(pen0.y) ? gp.y * GAMMA : 0.0f,
                                    keep(pen0.z) ? gp.z * GAMMA : 0.0f, 0.0f);
        }
        slot_add(slot_of(f, A, p, true, ab), V0(), Q0(), pg.xa0, pg.qa0);
        slot_add(slot_of(f, A, p, false, ab), V0(), Q0(), pg.xb0, pg.qb0);
    }
}

// ---- inertial targets (mod.rs:993-1018) -> the previous substep's state --------
// The start of the substep: the pose adjoints gathered from every incidence
// slot are taken back through the targets (and a swept impact) to the
// previous substep's state.  A thread gathers up to START_SHORT slots; a
// body with more (a floor under many bodies) is listed for k_adj_start_long,
// whose block sums them in a fixed-shape tree.
constexpr uint32_t START_SHORT = 32;
static __device__ __forceinline__ void start_finish(const DW& w, const AdjFrame& f, const AdjState& A, uint32_t h,
                                                    V3 gx, Q gq, V3 gx0, Q gq0) {
    gx = gx + ld3(A.ax[h]);
    gq = qadd(gq, ldq(A.aq[h]));
    gx0 = gx0 + ld3(A.ax0[h]);
    gq0 = qadd(gq0, ldq(A.aq0[h]));
    if (w.J)
        for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1]; k++) {
            uint32_t j = w.jlist[k];
            const float4* s = A.jslot + ((size_t)j * 2 + (w.j_ab[j].x == h ? 0u : 1u)) * 4;
            gx = gx + ld3(s[0]);
            gq = qadd(gq, ldq(s[1]));
            gx0 = gx0 + ld3(s[2]);
            gq0 = qadd(gq0, ldq(s[3]));
        }
    if (f.colour[h] >= 0) {
        // the iterations started from the targets: x = y = x0 + v dt + g dt^2,
        // q = qt = integrate(q0, w dt)
        float dt = w.dt;
        V3 gy = ld3(A.ay[h]) + gx;
        Q gqt = qadd(ldq(A.aqt[h]), gq);
        gx0 = gx0 + gy;
        V3 gwd = V0();
        quat_integrate_bwd(ldq(f.rot0[h]), ld3(f.angvel[h]) * dt, gqt, gq0, gwd);
        V3 gv = gy * dt;
        if (f.ccd && f.ccd[2 * h + 1].y != 0.0f) {
            // a swept impact moved the body before the targets: x' = x + v dt
            // frac, v' = (I - bounce n n^T) v, time of impact and normal held
            // fixed like a contact frame
            float4 nb = f.ccd[2 * h];
            V3 n = ld3(nb);
            gv = gv - n * (nb.w * dot(n, gv)) + gx0 * f.ccd[2 * h + 1].x;
        }
        A.av[h] = st3(gv, 0.0f);
        A.aw[h] = st3(gwd * dt, 0.0f);
        A.ax[h] = st3(gx0, 0.0f);
        A.aq[h] = stq(gq0);
    } else {
        A.ax[h] = st3(gx + gx0, 0.0f);
        A.aq[h] = stq(qadd(gq, gq0));
    }
}
__global__ void k_adj_start(DW w, AdjFrame f, AdjState A) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    const uint32_t k0 = f.offA[h] + f.offB[h], k1 = f.offA[h + 1] + f.offB[h + 1];
    if (k1 - k0 > START_SHORT) {
        A.long_list[atomicAdd(A.nlong, 1u)] = h;
        return;
    }
    V3 gx = V0(), gx0 = V0();
    Q gq = Q0(), gq0 = Q0();
    for (uint32_t k = k0; k < k1; k++) {
        const float4* s = A.slot + (size_t)k * 4;
        gx = gx + ld3(s[0]);
        gq = qadd(gq, ldq(s[1]));
        gx0 = gx0 + ld3(s[2]);
        gq0 = qadd(gq0, ldq(s[3]));
    }
    start_finish(w, f, A, h, gx, gq, gx0, gq0);
}
__global__ void __launch_bounds__(256) k_adj_start_long(DW w, AdjFrame f, AdjState A) {
    __shared__ float4 part[4][256];
    const uint32_t nl = *A.nlong;
    for (uint32_t l = blockIdx.x; l < nl; l += gridDim.x) {
        const uint32_t h = A.long_list[l];
        const uint32_t k0 = f.offA[h] + f.offB[h], k1 = f.offA[h + 1] + f.offB[h + 1];
        float4 s0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), s1 = s0, s2 = s0, s3 = s0;
        for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            const float4* s = A.slot + (size_t)k * 4;
            s0 = f4add(s0, s[0]);
            s1 = f4add(s1, s[1]);
            s2 = f4add(s2, s[2]);
            s3 = f4add(s3, s[3]);
        }
        part[0][threadIdx.x] = s0;
        part[1][threadIdx.x] = s1;
        part[2][threadIdx.x] = s2;
        part[3][threadIdx.x] = s3;
        __syncthreads();
        for (uint32_t m = blockDim.x >> 1; m > 0; m >>= 1) {
            if (threadIdx.x < m)
                for (int c = 0; c < 4; c++) part[c][threadIdx.x] = f4add(part[c][threadIdx.x], part[c][threadIdx.x + m]);
            __syncthreads();
        }
        if (threadIdx.x == 0)
            start_finish(w, f, A, h, ld3(part[0][0]), ldq(part[1][0]), ld3(part[2][0]), ldq(part[3][0]));
        __syncthreads();
    }
}

// ---- warm-state inheritance of the discovery merge (rows.rs:831-904) -----------
// One thread per new pair: all new points that inherit from one old pair
// belong to the same new pair, so the sums need no atomics.
__global__ void k_adj_inherit(DW w, AdjFrame f, AdjState A) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < f.npairs; p += gridDim.x * blockDim.x) {
        int32_t o = f.p_old[p];
        if (o < 0) continue;
        uint32_t np = f.p_np[p];
        for (uint32_t k = 0; k < np; k++) {
            uint32_t q = p * MAX_PTS + k;
            int32_t m = f.q_matched[q];
            if (m < 0) continue;
            size_t oq = (size_t)o * MAX_PTS + (uint32_t)m;
            A.alam_old[oq] = f4add(A.alam_old[oq], A.alam[q]);
            A.apen_old[oq] = f4add(A.apen_old[oq], A.apen[q]);
        }
    }
}

// ---- friction coefficient adjoint per scene (pair mu = max of the bodies') -----
// One block per scene; the block's fixed-shape tree sum keeps the result the
// same from run to run.
__global__ void __launch_bounds__(256) k_adj_mu_scene(DW w, AdjFrame f, AdjState A) {
    const uint32_t s = blockIdx.x;
    uint32_t b0 = w.scene_off[s], b1 = w.scene_off[s + 1];
    // pairs are ordered by their A body: binary search the scene's range
    auto lower = [&](uint32_t key) {
        uint32_t lo = 0, hi = f.npairs;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (f.p_ab[mid].x < key) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    uint32_t p0 = lower(b0), p1 = lower(b1);
    float acc = 0.0f;
    for (uint32_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        float2 m = A.amu[p];
        acc += m.x + m.y;
    }
    __shared__ float part[256];
    part[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t k = blockDim.x >> 1; k > 0; k >>= 1) {
        if (threadIdx.x < k) part[threadIdx.x] += part[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.ascene_mu[s] += part[0];
}

// The largest magnitude among the body adjoints (pose, orientation,
// velocities) after a reversed substep, and the first body holding it; a
// non-finite component counts as infinite.  One block, fixed reduction order.
__global__ void __launch_bounds__(256) k_adj_trace(DW w, AdjState A, uint2* out) {
    __shared__ float mv[256];
    __shared__ uint32_t mb[256];
    float best = -1.0f;
    uint32_t bh = 0xffffffffu;
    for (uint32_t h = threadIdx.x; h < (uint32_t)w.N; h += blockDim.x) {
        const float4 v[4] = {A.ax[h], A.aq[h], A.av[h], A.aw[h]};
        float m = 0.0f;
        for (int i = 0; i < 4; i++) {
            const float c[4] = {v[i].x, v[i].y, v[i].z, v[i].w};
            for (int k = 0; k < 4; k++) m = isfinite(c[k]) ? fmaxf(m, fabsf(c[k])) : INFINITY;
        }
        if (m > best) {
            best = m;
            bh = h;
        }
    }
    mv[threadIdx.x] = best;
    mb[threadIdx.x] = bh;
    __syncthreads();
    for (uint32_t s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            float o = mv[threadIdx.x + s];
            uint32_t ob = mb[threadIdx.x + s];
            if (o > mv[threadIdx.x] || (o == mv[threadIdx.x] && ob < mb[threadIdx.x])) {
                mv[threadIdx.x] = o;
                mb[threadIdx.x] = ob;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = make_uint2(__float_as_uint(fmaxf(mv[0], 0.0f)), mb[0]);
}
void launch_adjoint_trace(const DW& w, const AdjState& A, uint2* out, cudaStream_t st) {
    k_adj_trace<<<1, 256, 0, st>>>(w, A, out);
}

void launch_adjoint_substep(const DW& w, const AdjFrame& f, const AdjState& A, int iters, cudaStream_t st) {
    unsigned gb = nblk(w.N, 256);
    unsigned gp = f.npairs ? nblk(f.npairs, 128) : 1u;
    unsigned gpl = f.npairs ? nblk((size_t)f.npairs * ADJ_LANES, 128) : 1u;
    unsigned gp2 = f.npairs ? nblk((size_t)f.npairs * 2 * ADJ_LANES, 128) : 1u;
    k_adj_bdf<<<gb, 256, 0, st>>>(w, f, A, iters);
    for (int it = iters - 1; it >= 0; it--) {
        k_adj_dual<<<gpl, 128, 0, st>>>(w, f, A, it);
        if (w.J) k_adj_dual_joints<<<nblk(w.J, 128), 128, 0, st>>>(w, f, A, it);
        for (int c = (int)f.ncol - 1; c >= 0; c--) {
            if (w.J) k_adj_solve<true><<<nblk(w.N, 128), 128, 0, st>>>(w, f, A, it, c);
            else k_adj_solve<false><<<nblk(w.N, 128), 128, 0, st>>>(w, f, A, it, c);
            k_adj_sides<<<gp2, 128, 0, st>>>(w, f, A, it, c);
            if (w.J) k_adj_joint_sides<<<nblk(2 * (size_t)w.J, 128), 128, 0, st>>>(w, f, A, it, c);
        }
    }
    k_adj_c0<<<gp, 128, 0, st>>>(w, f, A);
    if (w.J) k_adj_decay_joints<<<nblk(w.J, 128), 128, 0, st>>>(w, f, A);
    k_adj_start<<<gb, 256, 0, st>>>(w, f, A);
    k_adj_start_long<<<152, 256, 0, st>>>(w, f, A);
    k_adj_inherit<<<gp, 128, 0, st>>>(w, f, A);
    if (w.S > 0) k_adj_mu_scene<<<(unsigned)w.S, 256, 0, st>>>(w, f, A);
}

}  // namespace avbd
