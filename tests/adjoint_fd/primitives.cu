// Central-difference checks of the adjoint's vector-Jacobian products
// (ornis_gb300/csrc/avbd_adjoint.cuh), built and run on the host: every
// VJP is compared with (f(x + h e_i) - f(x - h e_i)) / 2h of the forward
// function it reverses, contracted with a random output adjoint.  Prints
// "<checks> checks, <failures> failures" and exits 0; the Python test
// (tests/test_adjoint_fd_cpu.py) judges the counts.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "../../ornis_gb300/csrc/avbd_adjoint.cuh"
using namespace avbd;

static float frand() { return (float)rand() / RAND_MAX * 2.0f - 1.0f; }
static int fails = 0, checks = 0;
// Float central differences carry noise near 1e-4 (f32 rounding / 2h), so
// the relative error is taken against |fd| + 1e-2.
static void check(const char* name, double an, double fd) {
    checks++;
    double err = fabs(an - fd) / (1e-2 + fabs(fd));
    if (err > 3e-2) {
        printf("FAIL %s: adjoint %.6g fd %.6g\n", name, an, fd);
        fails++;
    }
}
static void check_zero(const char* name, double an) {
    checks++;
    if (an != 0.0) {
        printf("FAIL %s: adjoint %.6g, expected 0\n", name, an);
        fails++;
    }
}
static Q rq() { return qnormalize(Q{frand(), frand(), frand(), frand()}); }
static V3 rv() { return V3{frand(), frand(), frand()}; }
static float& qc(Q& q, int i) { return (&q.x)[i]; }

static void rotations(float h) {
    {  // qrot
        Q q = rq();
        V3 v = rv(), g = rv();
        Q gq = Q0();
        V3 gv = V0();
        qrot_bwd(q, v, g, gq, gv);
        for (int i = 0; i < 4; i++) {
            Q a = q, b = q;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("qrot q", qc(gq, i), (dot(g, qrot(a, v)) - dot(g, qrot(b, v))) / (2 * h));
        }
        for (int i = 0; i < 3; i++) {
            V3 a = v, b = v;
            a[i] += h;
            b[i] -= h;
            check("qrot v", gv[i], (dot(g, qrot(q, a)) - dot(g, qrot(q, b))) / (2 * h));
        }
    }
    {  // qnormalize
        Q q{frand(), frand(), frand(), frand()}, g{frand(), frand(), frand(), frand()};
        Q gq = qnormalize_bwd(q, g);
        for (int i = 0; i < 4; i++) {
            Q a = q, b = q;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("qnormalize", qc(gq, i), (qdot(g, qnormalize(a)) - qdot(g, qnormalize(b))) / (2 * h));
        }
    }
    for (float sc : {1.0f, 0.05f}) {  // quat_integrate, a large and a small turn
        Q q = rq(), g{frand(), frand(), frand(), frand()}, gq = Q0();
        V3 v = rv() * sc, gv = V0();
        quat_integrate_bwd(q, v, g, gq, gv);
        for (int i = 0; i < 4; i++) {
            Q a = q, b = q;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("quat_integrate q", qc(gq, i),
                  (qdot(g, quat_integrate(a, v)) - qdot(g, quat_integrate(b, v))) / (2 * h));
        }
        for (int i = 0; i < 3; i++) {
            V3 a = v, b = v;
            a[i] += h;
            b[i] -= h;
            check("quat_integrate v", gv[i], (qdot(g, quat_integrate(q, a)) - qdot(g, quat_integrate(q, b))) / (2 * h));
        }
    }
    for (int flip = 0; flip < 2; flip++)  // quat_diff_vec, both signs of the difference's w
        for (float sc : {1.0f, 0.05f}) {
            Q b = rq(), a = quat_integrate(b, rv() * sc), ga = Q0(), gb = Q0();
            if (flip) a = qscale(a, -1.0f);
            V3 g = rv();
            quat_diff_vec_bwd(a, b, g, ga, gb);
            const float hh = h * 0.1f;
            for (int i = 0; i < 4; i++) {
                Q x = a, y = a;
                qc(x, i) += hh;
                qc(y, i) -= hh;
                check("quat_diff_vec a", qc(ga, i), (dot(g, quat_diff_vec(x, b)) - dot(g, quat_diff_vec(y, b))) / (2 * hh));
                x = b;
                y = b;
                qc(x, i) += hh;
                qc(y, i) -= hh;
                check("quat_diff_vec b", qc(gb, i), (dot(g, quat_diff_vec(a, x)) - dot(g, quat_diff_vec(a, y))) / (2 * hh));
            }
        }
    {  // world inertia: psi = u . Iw(q) v
        Q q = rq(), gq = Q0();
        V3 I{1.0f + frand() * 0.5f, 1.2f, 0.7f}, u = rv(), v = rv();
        world_inertia_bwd(I, q, u, v, 1.0f, gq);
        auto psi = [&](Q qq) {
            float m[3][3];
            world_inertia(I, qq, m);
            return dot(u, mat3_vec(m, v));
        };
        for (int i = 0; i < 4; i++) {
            Q a = q, b = q;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("world_inertia", qc(gq, i), (psi(a) - psi(b)) / (2 * h));
        }
    }
}

static void contact_rows(float h) {
    for (int mode = 0; mode < 3; mode++) {  // inside the cone, on the cone, separating
        float cn = mode == 2 ? 0.3f : -0.5f + 0.2f * frand();
        float4 pen = make_float4(2.0f + frand(), 3.0f + frand(), 2.5f + frand(), 0.0f);
        float4 lam = make_float4(-0.2f + 0.1f * frand(), 0.1f * frand(), 0.1f * frand(), 0.0f);
        float ct0 = (mode == 1 ? 1.0f : 0.05f) * frand(), ct1 = (mode == 1 ? 1.0f : 0.05f) * frand();
        float2 mu = make_float2(0.6f, 0.5f);
        float g[3] = {frand(), frand(), frand()};
        float gcn = 0.0f, gct0 = 0.0f, gct1 = 0.0f;
        float4 gp = make_float4(0, 0, 0, 0), gl = make_float4(0, 0, 0, 0);
        float2 gmu = make_float2(0, 0);
        contact_force_bwd(cn, pen, lam, ct0, ct1, mu, g, gcn, gp, gl, gct0, gct1, gmu);
        auto F = [&](float c_, float4 p_, float4 l_, float a_, float b_, float2 m_) {
            float f[3];
            contact_force(c_, p_, l_, a_, b_, m_, f);
            return g[0] * f[0] + g[1] * f[1] + g[2] * f[2];
        };
        check("contact_force cn", gcn, (F(cn + h, pen, lam, ct0, ct1, mu) - F(cn - h, pen, lam, ct0, ct1, mu)) / (2 * h));
        check("contact_force ct0", gct0, (F(cn, pen, lam, ct0 + h, ct1, mu) - F(cn, pen, lam, ct0 - h, ct1, mu)) / (2 * h));
        check("contact_force ct1", gct1, (F(cn, pen, lam, ct0, ct1 + h, mu) - F(cn, pen, lam, ct0, ct1 - h, mu)) / (2 * h));
        for (int k = 0; k < 3; k++) {
            float4 p1 = pen, p2 = pen, l1 = lam, l2 = lam;
            f4add_at(p1, k, h);
            f4add_at(p2, k, -h);
            f4add_at(l1, k, h);
            f4add_at(l2, k, -h);
            check("contact_force pen", f4get(gp, k), (F(cn, p1, lam, ct0, ct1, mu) - F(cn, p2, lam, ct0, ct1, mu)) / (2 * h));
            check("contact_force lam", f4get(gl, k), (F(cn, pen, l1, ct0, ct1, mu) - F(cn, pen, l2, ct0, ct1, mu)) / (2 * h));
        }
        float2 m1 = mu, m2 = mu;
        m1.x += h;
        m2.x -= h;
        check("contact_force mu", gmu.x, (F(cn, pen, lam, ct0, ct1, m1) - F(cn, pen, lam, ct0, ct1, m2)) / (2 * h));
    }
    {  // the friction frame's first tangent
        V3 n = normalize_or(rv(), VY()), gt = rv(), gn = V0();
        tangent_t1_bwd(n, gt, gn);
        for (int i = 0; i < 3; i++) {
            V3 a = n, b = n;
            a[i] += h;
            b[i] -= h;
            check("tangent_t1", gn[i], (dot(gt, tangent_t1(a)) - dot(gt, tangent_t1(b))) / (2 * h));
        }
    }
    {  // a capsule's rolling witness anchor: s R0^T n (the segment point is constant)
        Q q0 = rq(), gq0 = Q0();
        V3 n = normalize_or(rv(), VY()), g = rv();
        float s = 0.05f + 0.1f * fabsf(frand());
        rolling_anchor_bwd(q0, n, s, g, gq0);
        auto A = [&](Q q) { return dot(g, qrot(conj(q), n) * s); };
        for (int i = 0; i < 4; i++) {
            Q a = q0, b = q0;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("rolling anchor", qc(gq0, i), (A(a) - A(b)) / (2 * h));
        }
    }
}

// The hinge twist: its derivative where the swing is under 120 degrees, and
// none (held) beyond.
static void hinge_twist_checks(float h) {
    V3 axis = normalize_or(rv(), VX());
    for (int held = 0; held < 2; held++) {
        Q qa = rq(), qb;
        for (;;) {  // a relative rotation whose swing is inside / outside the band
            qb = rq();
            Q q = qmul(conj(qa), qb);
            float s = dot(V3{q.x, q.y, q.z}, axis);
            float r2 = s * s + q.w * q.w;
            if (held ? r2 < 0.2f : (r2 > 0.3f && fabsf(hinge_twist(qa, qb, axis)) < 2.5f)) break;
        }
        float g = frand();
        Q gqa = Q0(), gqb = Q0();
        hinge_twist_bwd(qa, qb, axis, g, gqa, gqb);
        for (int i = 0; i < 4; i++) {
            if (held) {
                check_zero("hinge_twist held qa", qc(gqa, i));
                check_zero("hinge_twist held qb", qc(gqb, i));
                continue;
            }
            Q a = qa, b = qa;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("hinge_twist qa", qc(gqa, i), g * (hinge_twist(a, qb, axis) - hinge_twist(b, qb, axis)) / (2 * h));
            a = qb;
            b = qb;
            qc(a, i) += h;
            qc(b, i) -= h;
            check("hinge_twist qb", qc(gqb, i), g * (hinge_twist(qa, a, axis) - hinge_twist(qa, b, axis)) / (2 * h));
        }
    }
}

int main() {
    srand(3);
    const float h = 1e-3f;
    for (int trial = 0; trial < 40; trial++) {
        rotations(h);
        contact_rows(h);
        hinge_twist_checks(h);
    }
    printf("%d checks, %d failures\n", checks, fails);
    return 0;
}
