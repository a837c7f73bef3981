// Central-difference checks of the joint rows' adjoint
// (ornis_gb300/csrc/avbd_adjoint.cuh), built and run on the host.
// joint_stamp_bwd against psi = w . (r + H d) of joint_stamp, and
// joint_dual_bwd against a random linear form of joint_dual's output, for
// ball and hinge joints with and without a twist limit, hard (k = 0) and
// soft (k = 55) rows, over every pose and warm-state input.  An input whose
// difference quotients at two step sizes disagree straddles a kink (a row
// switching on, a clamp) and is skipped.  Prints "<checks> checks,
// <failures> failures, <skipped> skipped at kinks" and exits 0; the Python
// test (tests/test_adjoint_fd_cpu.py) judges the counts.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "../../ornis_gb300/csrc/avbd_adjoint.cuh"
using namespace avbd;
static double frand() { return (double)rand() / RAND_MAX * 2.0 - 1.0; }
static int fails = 0, checks = 0, skipped = 0;
static void check(const char* name, double an, double fd, double scale) {
    checks++;
    double err = fabs(an - fd) / (1e-2 * scale + fabs(fd));
    if (err > 3e-2) { printf("FAIL %s: adjoint %.6g fd %.6g\n", name, an, fd); fails++; }
}
static Q rq() { Q q{(float)frand(), (float)frand(), (float)frand(), (float)frand()}; return qnormalize(q); }
static V3 rv(float s = 1) { return V3{(float)frand() * s, (float)frand() * s, (float)frand() * s}; }
static Q small_rot(Q base, float s) { return quat_integrate(base, rv(s)); }
static double psi(const JDef& d, const JPose& p, const JState& s, bool is_a, const float w6[6], const float d6[6]) {
    Sys sys;
    for (int i = 0; i < 21; i++) sys.h[i] = 0; for (int i = 0; i < 6; i++) sys.r[i] = 0;
    joint_stamp(d, p, s, is_a, sys);
    double acc = 0;
    for (int i = 0; i < 6; i++) {
        double hd = 0;
        for (int j = 0; j < 6; j++) hd += sys.h[i >= j ? tri(i, j) : tri(j, i)] * d6[j];
        acc += w6[i] * (sys.r[i] + hd);
    }
    return acc;
}
static double dual_scalar(const JDef& d, const JPose& p, const JState& s, float K, const JState& gout) {
    JState o; joint_dual(d, p, s, K, o);
    double a = 0;
    for (int k = 0; k < 4; k++) a += f4get(gout.laml, k) * f4get(o.laml, k) + f4get(gout.penl, k) * f4get(o.penl, k)
                                  + f4get(gout.lama, k) * f4get(o.lama, k) + f4get(gout.pena, k) * f4get(o.pena, k);
    return a + gout.acc * o.acc;
}
// pointers to every float input
struct In { const char* name; float* v; };
static int inputs(JPose& p, JState& s, In* out) {
    int n = 0;
    auto v3 = [&](const char* nm, V3& x) { out[n++] = {nm, &x.x}; out[n++] = {nm, &x.y}; out[n++] = {nm, &x.z}; };
    auto q4 = [&](const char* nm, Q& x) { out[n++] = {nm, &x.x}; out[n++] = {nm, &x.y}; out[n++] = {nm, &x.z}; out[n++] = {nm, &x.w}; };
    auto f4 = [&](const char* nm, float4& x) { out[n++] = {nm, &x.x}; out[n++] = {nm, &x.y}; out[n++] = {nm, &x.z}; };
    v3("xa", p.xa); v3("xb", p.xb); v3("xa0", p.xa0); v3("xb0", p.xb0);
    q4("qa", p.qa); q4("qb", p.qb); q4("qa0", p.qa0); q4("qb0", p.qb0);
    f4("laml", s.laml); f4("penl", s.penl); f4("lama", s.lama); f4("pena", s.pena);
    out[n++] = {"acc", &s.acc};
    return n;
}
static void grads(const PairGrad& g, const JState& gs, float* out) {
    int n = 0;
    auto v3 = [&](V3 x) { out[n++] = x.x; out[n++] = x.y; out[n++] = x.z; };
    auto q4 = [&](Q x) { out[n++] = x.x; out[n++] = x.y; out[n++] = x.z; out[n++] = x.w; };
    auto f4 = [&](float4 x) { out[n++] = x.x; out[n++] = x.y; out[n++] = x.z; };
    v3(g.xa); v3(g.xb); v3(g.xa0); v3(g.xb0); q4(g.qa); q4(g.qb); q4(g.qa0); q4(g.qb0);
    f4(gs.laml); f4(gs.penl); f4(gs.lama); f4(gs.pena); out[n++] = gs.acc;
}
int main() {
    srand(7);
    for (int trial = 0; trial < 60; trial++) {
        JDef d;
        d.la = rv(0.3f); d.lb = rv(0.3f);
        d.axa_l = normalize(rv()); d.axb_l = normalize(rv());
        d.ref = 0.1f * (float)frand();
        d.revolute = trial % 3 != 0;
        float twist_lo = -0.3f, twist_hi = 0.3f;
        d.lim = make_float4(twist_lo, twist_hi, (trial % 2) ? 1.0f : 0.0f, 0.0f);
        JPose p;
        p.qa0 = rq(); p.qb0 = small_rot(p.qa0, 0.6f);
        p.qa = small_rot(p.qa0, 0.05f); p.qb = small_rot(p.qb0, 0.05f);
        p.xa0 = rv(); p.xb0 = p.xa0 + qrot(p.qa0, d.la) - qrot(p.qb0, d.lb) + rv(0.01f);
        p.xa = p.xa0 + rv(0.02f); p.xb = p.xb0 + rv(0.02f);
        JState s;
        s.laml = make_float4(frand(), frand(), frand(), 0); s.penl = make_float4(50 + 20 * frand(), 60, 70, 0);
        s.lama = make_float4(frand(), frand(), 0, 0); s.pena = make_float4(40, 45 + 5 * frand(), 30, 0);
        s.acc = (trial % 4 == 1) ? -0.2f : ((trial % 4 == 2) ? 0.2f : 0.0f);
        bool is_a = trial % 2 == 0;
        {   // keep the limit's one-sided force away from its kink (finite differences straddle it)
            float angle = wrap_pi(hinge_twist(p.qa, p.qb, d.axa_l) - d.ref);
            float initial = wrap_pi(hinge_twist(p.qa0, p.qb0, d.axa_l) - d.ref);
            int stt = warm_limit_state(angle, d.lim.x, d.lim.y, LIMIT_SLOP_ANG, s.acc);
            if (d.revolute && d.lim.z != 0.0f && stt >= 0) {
                bool lower = stt == 1;
                float cc = regularized_limit(angle, initial, lower ? d.lim.x : d.lim.y, lower);
                if (fabsf(s.pena.z * cc + s.acc) < 0.05f) { printf("trial %d: limit force near its kink, skipped\n", trial); continue; }
            }
        }
        float w6[6], d6[6];
        for (int i = 0; i < 6; i++) { w6[i] = (float)frand(); d6[i] = 0.01f * (float)frand(); }
        // stamp
        PairGrad g; pair_grad_zero(g); JState gs; jstate_zero(gs);
        joint_stamp_bwd(d, p, s, is_a, w6, d6, g, gs);
        float an[64]; grads(g, gs, an);
        In in[64]; int n = inputs(p, s, in);
        double scale = 0; for (int i = 0; i < n; i++) scale = fmax(scale, fabs(an[i]));
        for (int i = 0; i < n; i++) {
            double fds[2];
            for (int e = 0; e < 2; e++) {
                float h = e ? 4e-4f : 2e-3f, v0 = *in[i].v;
                *in[i].v = v0 + h; double up = psi(d, p, s, is_a, w6, d6);
                *in[i].v = v0 - h; double dn = psi(d, p, s, is_a, w6, d6);
                *in[i].v = v0;
                fds[e] = -(up - dn) / (2 * h);
            }
            if (fabs(fds[0] - fds[1]) > 0.05 * (fabs(fds[1]) + 1e-2 * scale)) { skipped++; continue; }  // a kink
            char nm[64]; snprintf(nm, 64, "stamp[%d] %s#%d rev%d lim%d", trial, in[i].name, i, d.revolute, (int)d.lim.z);
            check(nm, an[i], fds[1], scale);
        }
        // dual
        for (float K : {0.0f, 55.0f}) {
            JState gout; gout.laml = make_float4(frand(), frand(), frand(), 0); gout.penl = make_float4(frand(), frand(), frand(), 0);
            gout.lama = make_float4(frand(), frand(), frand(), 0); gout.pena = make_float4(frand(), frand(), frand(), 0); gout.acc = (float)frand();
            PairGrad g2; pair_grad_zero(g2); JState gin; float gK = 0;
            joint_dual_bwd(d, p, s, K, gout, gin, g2, gK);
            float an2[64]; grads(g2, gin, an2);
            double sc2 = 0; for (int i = 0; i < n; i++) sc2 = fmax(sc2, fabs(an2[i]));
            for (int i = 0; i < n; i++) {
                double fds[2];
                for (int e = 0; e < 2; e++) {
                    float h = e ? 4e-4f : 2e-3f, v0 = *in[i].v;
                    *in[i].v = v0 + h; double up = dual_scalar(d, p, s, K, gout);
                    *in[i].v = v0 - h; double dn = dual_scalar(d, p, s, K, gout);
                    *in[i].v = v0;
                    fds[e] = (up - dn) / (2 * h);
                }
                if (fabs(fds[0] - fds[1]) > 0.05 * (fabs(fds[1]) + 1e-2 * sc2)) { skipped++; continue; }
                char nm[64]; snprintf(nm, 64, "dual[%d] K%g %s#%d", trial, K, in[i].name, i);
                check(nm, an2[i], fds[1], sc2);
            }
            if (K > 0) {
                float h = 1e-2f;
                double fd = (dual_scalar(d, p, s, K + h, gout) - dual_scalar(d, p, s, K - h, gout)) / (2 * h);
                check("dual dK", gK, fd, fmax(1.0, fabs(fd)));
            }
        }
    }
    printf("%d checks, %d failures, %d skipped at kinks\n", checks, fails, skipped);
    return 0;
}
