// avbd_shapes.cuh — narrowphase geometry on the device: signed surface
// distance with witness points for sphere / box / capsule / half-space pairs
// (analytic) and cylinder / cone / convex-hull pairs (GJK / EPA, avbd_gjk.cuh).
//
// Semantics follow the reference's analytic oracles one for one (citations to
// crates/physics/src/collision/): the pair set, the contact normal and the
// manifold anchors all derive from these values, so they must agree with the
// reference bit for bit on identical input (this translation unit is built
// with -fmad=false; see avbd_vec.cuh for the operation order).
#pragma once
#include <cfloat>

#include "avbd_world.cuh"

namespace avbd {

struct Dist {
    float dist;
    V3 pa, pb;
};
struct Shape {
    uint32_t kind;
    V3 p;  // params
    V3 pos;
    Q rot;
    const HullDesc* hull;  // AVBD_SHAPE_HULL only
};

static __device__ __forceinline__ V3 point_segment_closest(V3 p, V3 a, V3 b) {  // distance.rs:63-71
    V3 ab = b - a;
    float l2 = len2(ab);
    if (l2 < DEGENERATE_EPS) return a;
    float t = fclamp(dot(p - a, ab) / l2, 0.0f, 1.0f);
    return a + ab * t;
}

static __device__ __forceinline__ void seg_seg_closest(V3 a0, V3 a1, V3 b0, V3 b1, V3& oa, V3& ob) {  // distance.rs:75-113
    V3 d1 = a1 - a0, d2 = b1 - b0, r = a0 - b0;
    float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    if (a < DEGENERATE_EPS && e < DEGENERATE_EPS) { oa = a0; ob = b0; return; }
    if (a < DEGENERATE_EPS) {
        float t = fclamp(f / e, 0.0f, 1.0f);
        oa = a0; ob = b0 + d2 * t;
        return;
    }
    float c = dot(d1, r);
    if (e < DEGENERATE_EPS) {
        float t = fclamp(-c / a, 0.0f, 1.0f);
        oa = a0 + d1 * t; ob = b0;
        return;
    }
    float b = dot(d1, d2);
    float denom = a * e - b * b;
    float s = fabsf(denom) > DEGENERATE_EPS ? fclamp((b * f - c * e) / denom, 0.0f, 1.0f) : 0.0f;
    float t = e > DEGENERATE_EPS ? (b * s + f) / e : 0.0f;
    if (!(t >= 0.0f && t <= 1.0f)) {
        t = fclamp(t, 0.0f, 1.0f);
        s = fclamp((b * t - c) / a, 0.0f, 1.0f);
    }
    oa = a0 + d1 * s;
    ob = b0 + d2 * t;
}

static __device__ __forceinline__ V3 point_obb_closest(V3 p, V3 pos, V3 half, Q rot) {  // distance.rs:117-138
    V3 l = qrot(conj(rot), p - pos);
    V3 cl = vclamp(l, -half, half);
    V3 q;
    if (veq(cl, l)) {
        float dx = half.x - fabsf(l.x), dy = half.y - fabsf(l.y), dz = half.z - fabsf(l.z);
        q = l;
        if (dx <= dy && dx <= dz) q.x = copysignf(half.x, l.x);
        else if (dy <= dz) q.y = copysignf(half.y, l.y);
        else q.z = copysignf(half.z, l.z);
    } else {
        q = cl;
    }
    return pos + qrot(rot, q);
}

static __device__ __forceinline__ void obb_axes(V3 half, Q rot, V3& x, V3& y, V3& z) {
    x = qrot(rot, VX() * half.x);
    y = qrot(rot, VY() * half.y);
    z = qrot(rot, VZ() * half.z);
}
// corner i of an OBB in the reference's bit order (distance.rs:142-156):
// bit2 selects -x, bit1 -y, bit0 -z.
static __device__ __forceinline__ V3 obb_corner(V3 pos, V3 x, V3 y, V3 z, int i) {
    V3 c = (i & 4) ? pos - x : pos + x;
    c = (i & 2) ? c - y : c + y;
    c = (i & 1) ? c - z : c + z;
    return c;
}
static __constant__ const int8_t kObbEdges[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                                              {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};

static __device__ __forceinline__ Dist sphere_sphere(V3 pa, float ra, V3 pb, float rb) {  // distance.rs:180-189
    V3 d = pb - pa;
    float cd = len(d);
    V3 n = normalize_or(d, VX());
    return {cd - ra - rb, pa + n * ra, pb - n * rb};
}

static __device__ __forceinline__ Dist sphere_obb(V3 apos, float r, V3 bpos, Q brot, V3 half) {  // distance.rs:192-216
    V3 pb = point_obb_closest(apos, bpos, half, brot);
    V3 d = apos - pb;
    float core = len(d);
    V3 local = qrot(conj(brot), apos - bpos);
    V3 al = vabs(local);
    bool inside = al.x <= half.x && al.y <= half.y && al.z <= half.z;
    V3 n;
    if (inside) {
        V3 cl = half - al;
        V3 axis;
        if (cl.x <= cl.y && cl.x <= cl.z) axis = VX() * signumf(local.x);
        else if (cl.y <= cl.z) axis = VY() * signumf(local.y);
        else axis = VZ() * signumf(local.z);
        n = normalize_or(pb - apos, qrot(brot, axis));
    } else {
        n = normalize_or(d, VX());
    }
    return {inside ? -core - r : core - r, apos - n * r, pb};
}

static __device__ __forceinline__ Dist sphere_capsule(V3 apos, float r, V3 bpos, Q brot, float cr, float hh) {  // :219-230
    V3 axis = qrot(brot, VY());
    V3 s0 = bpos - axis * hh, s1 = bpos + axis * hh;
    V3 cb = point_segment_closest(apos, s0, s1);
    V3 d = apos - cb;
    float core = len(d);
    V3 n = normalize_or(d, VX());
    return {core - r - cr, apos - n * r, cb + n * cr};
}

static __device__ __forceinline__ Dist capsule_capsule(V3 apos, Q arot, float ra, float ha, V3 bpos, Q brot, float rb,
                                                float hb) {  // :233-245
    V3 axa = qrot(arot, VY()), axb = qrot(brot, VY());
    V3 a0 = apos - axa * ha, a1 = apos + axa * ha;
    V3 b0 = bpos - axb * hb, b1 = bpos + axb * hb;
    V3 ca, cb;
    seg_seg_closest(a0, a1, b0, b1, ca, cb);
    V3 d = cb - ca;
    float core = len(d);
    V3 n = normalize_or(d, VX());
    return {core - ra - rb, ca + n * ra, cb - n * rb};
}

// gjk.rs:68-186 (support point) for the path's shapes.
static __device__ __forceinline__ V3 support(const Shape& s, V3 dir) {
    switch (s.kind) {
        case AVBD_SHAPE_SPHERE:
            return s.pos + normalize_or(dir, VX()) * s.p.x;
        case AVBD_SHAPE_BOX: {
            V3 l = qrot(conj(s.rot), dir);
            V3 g{l.x >= 0.0f ? 1.0f : -1.0f, l.y >= 0.0f ? 1.0f : -1.0f, l.z >= 0.0f ? 1.0f : -1.0f};
            return s.pos + qrot(s.rot, V3{s.p.x * g.x, s.p.y * g.y, s.p.z * g.z});
        }
        case AVBD_SHAPE_CAPSULE: {
            V3 axis = qrot(s.rot, VY());
            V3 tip = (dot(dir, axis) >= 0.0f ? axis : -axis) * s.p.y;
            return s.pos + tip + normalize_or(dir, VX()) * s.p.x;
        }
        default:
            return s.pos;
    }
}

// distance_box.rs:21-50 — 15-axis SAT; returns the largest gap and its axis.
static __device__ __noinline__ float separating_axis(V3 apos, Q arot, V3 ha, V3 bpos, Q brot, V3 hb, V3& nout) {
    V3 aa[3], bb[3];
    mat3_cols(arot, aa);
    mat3_cols(brot, bb);
    V3 delta = bpos - apos;
    float best = -INFINITY;
    V3 bn = VY();
    for (int k = 0; k < 15; k++) {
        V3 n;
        if (k < 3) n = aa[k];
        else if (k < 6) n = bb[k - 3];
        else {
            int i = (k - 6) / 3, j = (k - 6) % 3;
            V3 c = cross(aa[i], bb[j]);
            n = len2(c) > DEGENERATE_EPS ? normalize(c) : V0();
        }
        if (veq(n, V0())) continue;
        float ea = ha.x * fabsf(dot(n, aa[0])) + ha.y * fabsf(dot(n, aa[1])) + ha.z * fabsf(dot(n, aa[2]));
        float eb = hb.x * fabsf(dot(n, bb[0])) + hb.y * fabsf(dot(n, bb[1])) + hb.z * fabsf(dot(n, bb[2]));
        float proj = dot(delta, n);
        float gap = fabsf(proj) - ea - eb;
        if (gap > best) {
            best = gap;
            bn = proj >= 0.0f ? n : -n;
        }
    }
    nout = bn;
    return best;
}

static __device__ __forceinline__ void support_face(V3 pos, Q rot, V3 half, V3 dir, V3& fpos, V3& ext) {  // :80-97
    V3 local = qrot(conj(rot), dir);
    V3 off = V0();
    ext = half;
    for (int i = 0; i < 3; i++) {
        if (fabsf(local[i]) > FACE_AXIS_EPS) {
            off[i] = signumf(local[i]) * half[i];
            ext[i] = 0.0f;
        }
    }
    fpos = pos + qrot(rot, off);
}

// For a box with collapsed extents (a support face, edge or corner of the
// penetration branch), corner i and corner i ^ bit coincide along a collapsed
// axis, and so do edges whose corners coincide.  A repeated feature gives the
// same squared distance as its first occurrence, which never strictly wins,
// so only first occurrences are tested: the result is the full loop's.
// Edge keep masks by collapse pattern (bit 4: x, 2: y, 1: z), kObbEdges order.
static __constant__ const uint16_t kEdgeKeep[8] = {0xfff, 0xf55, 0x5f3, 0x51, 0x33f, 0x15, 0x103, 0x1};
static __device__ __forceinline__ int collapsed(V3 h) {
    return (h.x == 0.0f ? 4 : 0) | (h.y == 0.0f ? 2 : 0) | (h.z == 0.0f ? 1 : 0);
}

// distance_box.rs:99-129 — closest corner/face and edge/edge features.
static __device__ __noinline__ Dist feature_distance(V3 apos, Q arot, V3 ha, V3 bpos, Q brot, V3 hb) {
    V3 ax, ay, az, bx, by, bz;
    obb_axes(ha, arot, ax, ay, az);
    obb_axes(hb, brot, bx, by, bz);
    const int ma = collapsed(ha), mb = collapsed(hb);
    const uint32_t ka = kEdgeKeep[ma], kb = kEdgeKeep[mb];
    Dist res{INFINITY, apos, bpos};
    float best = INFINITY;
    auto consider = [&](V3 x, V3 y) {
        float sq = len2(y - x);
        if (sq < best) {
            best = sq;
            res = {sqrtf(sq), x, y};
        }
    };
    for (int i = 0; i < 8; i++) {
        if (i & ma) continue;
        V3 c = obb_corner(apos, ax, ay, az, i);
        consider(c, point_obb_closest(c, bpos, hb, brot));
    }
    for (int i = 0; i < 8; i++) {
        if (i & mb) continue;
        V3 c = obb_corner(bpos, bx, by, bz, i);
        consider(point_obb_closest(c, apos, ha, arot), c);
    }
    for (int i = 0; i < 12; i++) {
        if (!((ka >> i) & 1u)) continue;
        V3 a0 = obb_corner(apos, ax, ay, az, kObbEdges[i][0]);
        V3 a1 = obb_corner(apos, ax, ay, az, kObbEdges[i][1]);
        for (int j = 0; j < 12; j++) {
            if (!((kb >> j) & 1u)) continue;
            V3 b0 = obb_corner(bpos, bx, by, bz, kObbEdges[j][0]);
            V3 b1 = obb_corner(bpos, bx, by, bz, kObbEdges[j][1]);
            V3 x, y;
            seg_seg_closest(a0, a1, b0, b1, x, y);
            consider(x, y);
        }
    }
    return res;
}

static __device__ __forceinline__ Dist box_box(V3 apos, Q arot, V3 ha, V3 bpos, Q brot, V3 hb, float* sat_gap) {  // :131-142
    V3 n;
    float gap = separating_axis(apos, arot, ha, bpos, brot, hb, n);
    if (sat_gap) *sat_gap = gap;
    if (gap > 0.0f) return feature_distance(apos, arot, ha, bpos, brot, hb);
    V3 fa, ea, fb, eb;
    support_face(apos, arot, ha, n, fa, ea);
    support_face(bpos, brot, hb, -n, fb, eb);
    Dist r = feature_distance(fa, arot, ea, fb, brot, eb);
    r.dist = gap;
    return r;
}


// distance_box.rs:146-190 — segment vs solid box, piecewise quadratic.
static __device__ __noinline__ void segment_box(V3 start, V3 end, V3 lo, V3 hi, V3& opoint, V3& oclosest, float& osq) {
    V3 delta = end - start;
    float cuts[8];
    int nc = 0;
    cuts[nc++] = 0.0f;
    cuts[nc++] = 1.0f;
    for (int i = 0; i < 3; i++) {
        if (fabsf(delta[i]) > DEGENERATE_EPS) {
            float t0 = (lo[i] - start[i]) / delta[i];
            if (t0 > 0.0f && t0 < 1.0f) cuts[nc++] = t0;
            float t1 = (hi[i] - start[i]) / delta[i];
            if (t1 > 0.0f && t1 < 1.0f) cuts[nc++] = t1;
        }
    }
    for (int i = 1; i < nc; i++)
        for (int k = i; k > 0 && cuts[k] < cuts[k - 1]; k--) {
            float t = cuts[k];
            cuts[k] = cuts[k - 1];
            cuts[k - 1] = t;
        }
    opoint = start;
    oclosest = vclamp(start, lo, hi);
    osq = INFINITY;
    for (int w = 0; w + 1 < nc; w++) {
        float r0 = cuts[w], r1 = cuts[w + 1];
        float middle = (r0 + r1) * HALF;
        V3 p = start + middle * delta;
        float num = 0.0f, den = 0.0f;
        for (int i = 0; i < 3; i++) {
            bool has = false;
            float bd = 0.0f;
            if (p[i] < lo[i]) { has = true; bd = lo[i]; }
            else if (p[i] > hi[i]) { has = true; bd = hi[i]; }
            if (has) {
                num += delta[i] * (start[i] - bd);
                den += delta[i] * delta[i];
            }
        }
        float stationary = den > 0.0f ? fclamp(-num / den, r0, r1) : middle;
        float ts[3] = {stationary, r0, r1};
        for (int k = 0; k < 3; k++) {
            V3 point = start + ts[k] * delta;
            V3 cl = vclamp(point, lo, hi);
            float sq = len2(point - cl);
            if (sq < osq) {
                opoint = point;
                oclosest = cl;
                osq = sq;
            }
        }
    }
}

static __device__ __forceinline__ void spine_penetration(V3 center, V3 axis, V3 half, float radius, float height, float& og,
                                                  V3& on) {  // distance_box.rs:240-265
    og = -INFINITY;
    on = VX();
    for (int e = 0; e < 3; e++) {
        V3 ev = e == 0 ? VX() : (e == 1 ? VY() : VZ());
        for (int k = 0; k < 2; k++) {
            V3 n = k == 0 ? ev : normalize_or(cross(axis, ev), V0());
            if (veq(n, V0())) continue;
            float proj = dot(center, n);
            float gap = fabsf(proj) - dot(half, vabs(n)) - height * fabsf(dot(axis, n)) - radius;
            if (gap > og) {
                og = gap;
                on = proj >= 0.0f ? n : -n;
            }
        }
    }
}

static __device__ __noinline__ Dist box_capsule(V3 apos, Q arot, V3 half, V3 bpos, Q brot, float radius,
                                         float height) {  // distance_box.rs:192-236
    Q inv = conj(arot);
    V3 center = qrot(inv, bpos - apos);
    V3 axis = qrot(inv, qrot(brot, VY()));
    V3 start = center - axis * height, end = center + axis * height;
    V3 core, surface;
    float sq;
    segment_box(start, end, -half, half, core, surface, sq);
    float distance;
    V3 normal;
    if (sq > DEGENERATE_EPS) {
        float l = sqrtf(sq);
        distance = l - radius;
        normal = (core - surface) / l;
    } else {
        float depth;
        V3 nrm;
        spine_penetration(center, axis, half, radius, height, depth, nrm);
        V3 lo = -half, hi = half;
        for (int i = 0; i < 3; i++) {
            if (fabsf(nrm[i]) > FACE_AXIS_EPS) {
                lo[i] = signumf(nrm[i]) * half[i];
                hi[i] = lo[i];
            }
        }
        float proj = dot(axis, nrm);
        V3 e0 = start, e1 = end;
        if (proj > SPINE_ALIGNMENT_EPS) e1 = start;
        else if (proj < -SPINE_ALIGNMENT_EPS) e0 = end;
        float dummy;
        segment_box(e0, e1, lo, hi, core, surface, dummy);
        distance = depth;
        normal = nrm;
    }
    return {distance, apos + qrot(arot, surface), apos + qrot(arot, core - normal * radius)};
}

#include "avbd_gjk.cuh"

static __device__ __forceinline__ Dist halfspace_distance(const Shape& h, const Shape& o, bool first) {  // distance.rs:607-642
    if (o.kind == AVBD_SHAPE_HALFSPACE) return first ? Dist{INFINITY, h.pos, o.pos} : Dist{INFINITY, o.pos, h.pos};
    V3 n = qrot(h.rot, h.p);
    V3 s = support_any(o, -n);
    float dist = dot(s - h.pos, n);
    Dist d{dist, s - n * dist, s};
    if (first) return d;
    return {d.dist, d.pb, d.pa};
}

// shape_distance (distance.rs:654-821).  For box-box pairs the SAT gap (the
// reference's signed gap, rows.rs:498-510) is returned through sat_gap.
static __device__ __noinline__ Dist shape_distance(const Shape& a, const Shape& b, float* sat_gap) {
    if (a.kind == AVBD_SHAPE_HALFSPACE) return halfspace_distance(a, b, true);
    if (b.kind == AVBD_SHAPE_HALFSPACE) return halfspace_distance(b, a, false);
    uint32_t sa = a.kind, sb = b.kind;
    if (gjk_shape(sa) || gjk_shape(sb)) return gjk_pair_distance(a, b);  // distance.rs:811-817
    if (sa == AVBD_SHAPE_SPHERE && sb == AVBD_SHAPE_SPHERE) return sphere_sphere(a.pos, a.p.x, b.pos, b.p.x);
    if (sa == AVBD_SHAPE_SPHERE && sb == AVBD_SHAPE_BOX) return sphere_obb(a.pos, a.p.x, b.pos, b.rot, b.p);
    if (sa == AVBD_SHAPE_BOX && sb == AVBD_SHAPE_SPHERE) {
        Dist d = sphere_obb(b.pos, b.p.x, a.pos, a.rot, a.p);
        return {d.dist, d.pb, d.pa};
    }
    if (sa == AVBD_SHAPE_SPHERE && sb == AVBD_SHAPE_CAPSULE)
        return sphere_capsule(a.pos, a.p.x, b.pos, b.rot, b.p.x, b.p.y);
    if (sa == AVBD_SHAPE_CAPSULE && sb == AVBD_SHAPE_SPHERE) {
        Dist d = sphere_capsule(b.pos, b.p.x, a.pos, a.rot, a.p.x, a.p.y);
        return {d.dist, d.pb, d.pa};
    }
    if (sa == AVBD_SHAPE_BOX && sb == AVBD_SHAPE_BOX) return box_box(a.pos, a.rot, a.p, b.pos, b.rot, b.p, sat_gap);
    if (sa == AVBD_SHAPE_BOX && sb == AVBD_SHAPE_CAPSULE)
        return box_capsule(a.pos, a.rot, a.p, b.pos, b.rot, b.p.x, b.p.y);
    if (sa == AVBD_SHAPE_CAPSULE && sb == AVBD_SHAPE_BOX) {
        Dist d = box_capsule(b.pos, b.rot, b.p, a.pos, a.rot, a.p.x, a.p.y);
        return {d.dist, d.pb, d.pa};
    }
    return capsule_capsule(a.pos, a.rot, a.p.x, a.p.y, b.pos, b.rot, b.p.x, b.p.y);
}

}  // namespace avbd
