// avbd_oracle.cpp — CPU restatement of the reference AVBD rigid-body step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the
// GB300 kernels in ornis_gb300/csrc.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may load the library built from it, and
// only as the checker or the timed CPU baseline — never as the product path.
//
// It restates, function by function, the AVBD engine of Ornis's physics
// crate (the reference is Rust and cannot be built here: no cargo/rustc).
// Citations are to crates/physics/src/... in the reference tree.
//
// Two sweep modes share all arithmetic:
//   Reference — the reference's exact semantics: pair vector kept in append +
//               swap_remove order (avbd/rows.rs:905-937), primal sweep in
//               reverse handle order (avbd/mod.rs:1052-1059).
//   Coloured  — the GPU's schedule: pairs kept in ascending (a, b) order and
//               the primal sweep run colour by colour over a greedy colouring
//               in hash-priority order (identical to the Jones-Plassmann
//               colouring the GPU computes).  Within a colour bodies are
//               independent, so the order inside a colour is immaterial.
// Scalar T = float (bit-level parity), double (the f64 error column) or Dual
// (f64 forward-mode derivatives for the adjoint checks, avbd_dual.hpp).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <set>
#include <thread>
#include <utility>
#include <vector>

#include "../include/ornis_avbd.h"
#include "avbd_dual.hpp"  // before the templates that call std:: math on T
#include "avbd_math.hpp"

namespace orc {

// sin, cos, asin, atan2 of the step: correctly rounded for f32 (the platform
// libm's results, avbd_crmath.hpp), std's for f64, the dual rules for duals
template <class V> inline DualT<V> osin(const DualT<V>& a) { return std::sin(a); }
template <class V> inline DualT<V> ocos(const DualT<V>& a) { return std::cos(a); }
template <class V> inline DualT<V> oasin(const DualT<V>& a) { return std::asin(a); }
template <class V> inline DualT<V> oatan2(const DualT<V>& y, const DualT<V>& x) { return std::atan2(y, x); }

// ---- constants (avbd/mod.rs:154-247, constants.rs:26-79) -------------------
struct K {
    static constexpr float ALPHA = 0.99f;
    static constexpr float GAMMA = 0.999f;
    static constexpr float BETA = 10000.0f;
    static constexpr float BETA_ANG = 100.0f;
    static constexpr float MARGIN = 0.01f;
    static constexpr float PENALTY_MIN = 1.0f;
    static constexpr float PENALTY_MAX = 1.0e10f;
    static constexpr float PENALTY_INIT = 1.0f;
    static constexpr float JOINT_PENALTY_INIT = 1.0f;
    static constexpr float GEN_MARGIN = 0.05f;
    static constexpr float EXPAND_SLOP = 0.005f;
    static constexpr float POINT_MATCH_DIST = 0.03f;
    static constexpr float LAMBDA_MATCH_DIST = 0.05f;
    static constexpr float C_EPS = 1e-7f;
    static constexpr float STICK_THRESH = 0.00001f;
    static constexpr float SLEEP_LIN = 0.15f;
    static constexpr float SLEEP_ANG = 0.15f;
    static constexpr float HALF = 0.5f;
    static constexpr float SLEEP_TIME = 0.5f;
    static constexpr float WAKE_IMPACT_SPEED = 0.5f;
    static constexpr float WAKE_PENETRATION = 0.01f;
    static constexpr float LIMIT_SLOP_ANG = 0.005f;
    static constexpr float LIMIT_SLOP_LIN = 0.002f;      // mod.rs:222
    static constexpr float MIN_EFFECTIVE_MASS = 1e-10f;  // constants.rs:16
    static constexpr float LIM_PEN_MAX = 1e4f;
    static constexpr float ROLL_PEN = 100.0f;
    static constexpr float MIN_TOI_DISP_LENGTH = 1e-9f;
    static constexpr float SPIN_REST_EPS = 1e-9f;
    static constexpr float CCD_BOUNCE_SPEED = 1.0f;
    static constexpr float CONTACT_BEGIN_SLOP = 0.005f;    // trigger.rs:68
    static constexpr float CONTACT_HIT_THRESHOLD = 1.0f;   // trigger.rs:63
    static constexpr float DEGENERATE_LEN2 = 1e-12f;
    static constexpr float POS_CORRECTION_EPS = 1e-6f;  // constants.rs:71
    static constexpr float NEAR_ZERO = 1e-9f;
    static constexpr float SHAPE_TOUCH = 1e-3f;
    static constexpr float AXIS_REST_LEN2 = 1e-16f;
    static constexpr float CCD_TRAVEL_GATE_FRACTION = 0.5f;
    static constexpr float DEGENERATE_EPS = 1e-12f;  // distance.rs:24, distance_box.rs:8
    static constexpr float FACE_AXIS_EPS = 1e-6f;
    static constexpr float SPINE_ALIGNMENT_EPS = 1e-6f;
    static constexpr float TANGENT_REF_AXIS_DOT = 0.9f;  // math.rs
    static constexpr float JOINT_REST_ERROR = 0.005f;    // avbd/sleep.rs:6
    static constexpr float PI = 3.14159265358979323846f;
    static constexpr float TAU = 6.28318530717958647692f;
};
static constexpr int MAX_POINTS = 8;
static constexpr int SPATIAL_DOF = 6;

template <class T> static inline T C(float v) { return T(v); }

// ---- shapes --------------------------------------------------------------------
// ConvexHull (collision/shape.rs:317-365): centroid-relative vertices and the
// triangle faces the reference builds for hulls of at most 64 vertices.
template <class T> struct Hull {
    std::vector<V3<T>> verts;
    std::vector<uint32_t> faces;  // 3 indices per face
    T bound = T(0), min_ext = T(0);
    V3<T> unit_inertia{};  // body-frame inertia per unit mass (ConvexHull::try_inertia)
};
// A part of a rounded or compound shape (Shape::Round's inner, a compound
// child with its Pose; collision/shape.rs:95-135, :144-230): a primitive, a
// border radius (0: not rounded) and its pose in the parent frame.
template <class T> struct Part {
    uint32_t shape;
    V3<T> sp;
    T radius;
    V3<T> pos;
    Qt<T> rot;
    const Hull<T>* hull;
};
// A rounded shape (one part, identity pose) or a compound (its children in
// order), with the measures the engine reads from it.
template <class T> struct ExtShape {
    bool compound = false;
    std::vector<Part<T>> parts;
    V3<T> unit_inertia{};
    T bound = T(0), min_dim = T(0);
};
// Heightfield (shape.rs:352-361): row-major heights, rows along +Z and cols
// along +X, spacing `cell`, and the sample range.
template <class T> struct HField {
    uint32_t rows = 0, cols = 0;
    T cell = T(0);
    std::vector<T> h;
    T y_min = T(0), y_max = T(0);
};
// One node of a mesh's median-split tree (BvhNode / BvhLink, shape.rs:411-455):
// a leaf owns order[a .. a+b), an inner node branches to nodes a and b.
template <class T> struct BNode {
    V3<T> lo, hi;
    bool leaf;
    uint32_t a, b;
};
// TriMesh (shape.rs:377-396): centroid-relative triangle hulls, their
// centroids, the tree and its permutation, the longest vertex, the
// shortest edge.
template <class T> struct TMesh {
    std::deque<Hull<T>> tris;
    std::vector<V3<T>> cent;
    std::vector<BNode<T>> nodes;
    std::vector<uint32_t> order;
    T bound = T(0), min_feature = T(0);
};
// bound (rows.rs:268-272: the longest vertex) and smallest extent
// (shape.rs:1468-1479) of a hull
template <class T> static void hull_measures(Hull<T>& h) {
    T b = T(0);
    V3<T> lo{std::numeric_limits<T>::infinity(), std::numeric_limits<T>::infinity(),
             std::numeric_limits<T>::infinity()};
    V3<T> hi = -lo;
    for (const V3<T>& v : h.verts) {
        b = std::fmax(b, len(v));
        lo = {std::fmin(lo.x, v.x), std::fmin(lo.y, v.y), std::fmin(lo.z, v.z)};
        hi = {std::fmax(hi.x, v.x), std::fmax(hi.y, v.y), std::fmax(hi.z, v.z)};
    }
    h.bound = b;
    h.min_ext = h.verts.empty() ? T(0) : std::fmax(min_element(hi - lo), T(0));
}
template <class T> struct Body {
    const Hull<T>* hull = nullptr;  // AVBD_SHAPE_HULL only
    const ExtShape<T>* ext = nullptr;  // AVBD_SHAPE_ROUND, AVBD_SHAPE_COMPOUND
    const HField<T>* hf = nullptr;     // AVBD_SHAPE_HEIGHTFIELD
    const TMesh<T>* mesh = nullptr;    // AVBD_SHAPE_TRIMESH
    V3<T> pos;
    Qt<T> rot;
    V3<T> vel, angvel, torque;
    T mass, inv_mass;
    V3<T> inertia;
    T restitution, friction, friction_t, rolling, torsion;
    uint32_t shape;
    V3<T> sp;  // shape params
    uint32_t layer, mask, type, flags;
    bool trigger() const { return (flags & AVBD_FLAG_TRIGGER) != 0; }
};

template <class T> struct ShapeRef {
    const Body<T>* body;  // shape + params
    uint32_t shape;
    V3<T> sp;
    V3<T> pos;
    Qt<T> rot;
    const Hull<T>* hull;
    const ExtShape<T>* ext;
    const HField<T>* hf;
    const TMesh<T>* mesh;
};
template <class T> static ShapeRef<T> sref(const Body<T>& b) {
    return {&b, b.shape, b.sp, b.pos, b.rot, b.hull, b.ext, b.hf, b.mesh};
}

template <class T> struct Dist {
    T dist;
    V3<T> pa, pb;
};

// Shape::inertia (collision/shape.rs:713-790) for the path's shapes.
template <class T> static V3<T> shape_inertia(uint32_t shape, V3<T> sp, T mass) {
    if (!(mass > T(0)) || !std::isfinite(mass)) return VZERO<T>();
    switch (shape) {
        case AVBD_SHAPE_SPHERE: {
            T r = sp.x;
            T v = C<T>(0.4f) * mass * r * r;
            return {v, v, v};
        }
        case AVBD_SHAPE_BOX: {
            V3<T> s = sp * T(2);
            T x = s.x * s.x, y = s.y * s.y, z = s.z * s.z;
            T k = mass / T(12);
            return {k * (y + z), k * (z + x), k * (x + y)};
        }
        case AVBD_SHAPE_CAPSULE: {
            T r = sp.x, h = sp.y;
            T iy = C<T>(0.5f) * mass * r * r;
            T ixz = C<T>(0.25f) * mass * (r * r) + (mass / T(3)) * h * r + C<T>(0.25f) * mass * h * h;
            return {ixz, iy, ixz};
        }
        case AVBD_SHAPE_CYLINDER: {  // shape.rs:780-790
            T r = sp.x, h = sp.y;
            T iy = C<T>(0.5f) * mass * r * r;
            T ixz = mass * (T(3) * r * r + T(4) * h * h) / T(12);
            return {ixz, iy, ixz};
        }
        case AVBD_SHAPE_CONE: {  // shape.rs:791-801
            T r = sp.x, h = sp.y;
            T iy = C<T>(0.3f) * mass * r * r;
            T ixz = mass * (T(3) * r * r + T(8) * h * h) / T(20);
            return {ixz, iy, ixz};
        }
        default:
            return VZERO<T>();
    }
}

// ---- collision/distance.rs ------------------------------------------------------
template <class T> static V3<T> point_segment_closest(V3<T> p, V3<T> a, V3<T> b) {  // :63-71
    V3<T> ab = b - a;
    T l2 = len2(ab);
    if (l2 < C<T>(K::DEGENERATE_EPS)) return a;
    T t = fclamp(dot(p - a, ab) / l2, T(0), T(1));
    return a + ab * t;
}

template <class T> static void seg_seg_closest(V3<T> a0, V3<T> a1, V3<T> b0, V3<T> b1, V3<T>& oa, V3<T>& ob) {  // :75-113
    const T E = C<T>(K::DEGENERATE_EPS);
    V3<T> d1 = a1 - a0, d2 = b1 - b0, r = a0 - b0;
    T a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    if (a < E && e < E) { oa = a0; ob = b0; return; }
    if (a < E) {
        T t = fclamp(f / e, T(0), T(1));
        oa = a0; ob = b0 + d2 * t;
        return;
    }
    T c = dot(d1, r);
    if (e < E) {
        T t = fclamp(-c / a, T(0), T(1));
        oa = a0 + d1 * t; ob = b0;
        return;
    }
    T b = dot(d1, d2);
    T denom = a * e - b * b;
    T s = std::fabs(denom) > E ? fclamp((b * f - c * e) / denom, T(0), T(1)) : T(0);
    T t = e > E ? (b * s + f) / e : T(0);
    if (!(t >= T(0) && t <= T(1))) {
        t = fclamp(t, T(0), T(1));
        s = fclamp((b * t - c) / a, T(0), T(1));
    }
    oa = a0 + d1 * s;
    ob = b0 + d2 * t;
}

template <class T> static V3<T> point_obb_closest(V3<T> p, V3<T> pos, V3<T> half, Qt<T> rot) {  // :117-138
    V3<T> l = qrot(conj(rot), p - pos);
    V3<T> cl = vclamp(l, -half, half);
    V3<T> q;
    if (cl == l) {
        T dx = half.x - std::fabs(l.x), dy = half.y - std::fabs(l.y), dz = half.z - std::fabs(l.z);
        q = l;
        if (dx <= dy && dx <= dz) q.x = std::copysign(half.x, l.x);
        else if (dy <= dz) q.y = std::copysign(half.y, l.y);
        else q.z = std::copysign(half.z, l.z);
    } else {
        q = cl;
    }
    return pos + qrot(rot, q);
}

template <class T> static void obb_corners(V3<T> pos, V3<T> half, Qt<T> rot, V3<T> c[8]) {  // :142-156
    V3<T> x = qrot(rot, VX<T>() * half.x);
    V3<T> y = qrot(rot, VY<T>() * half.y);
    V3<T> z = qrot(rot, VZ<T>() * half.z);
    c[0] = pos + x + y + z; c[1] = pos + x + y - z; c[2] = pos + x - y + z; c[3] = pos + x - y - z;
    c[4] = pos - x + y + z; c[5] = pos - x + y - z; c[6] = pos - x - y + z; c[7] = pos - x - y - z;
}
static const int OBB_EDGES[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                                     {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};

template <class T> static void capsule_segment(V3<T> pos, T hh, Qt<T> rot, V3<T>& s0, V3<T>& s1) {
    V3<T> axis = qrot(rot, VY<T>());
    s0 = pos - axis * hh;
    s1 = pos + axis * hh;
}

template <class T> static Dist<T> sphere_sphere(V3<T> pa, T ra, V3<T> pb, T rb) {  // :180-189
    V3<T> d = pb - pa;
    T cd = len(d);
    V3<T> n = normalize_or(d, VX<T>());
    return {cd - ra - rb, pa + n * ra, pb - n * rb};
}

template <class T> static Dist<T> sphere_obb(V3<T> apos, T r, V3<T> bpos, Qt<T> brot, V3<T> half) {  // :192-216
    V3<T> pb = point_obb_closest(apos, bpos, half, brot);
    V3<T> d = apos - pb;
    T core = len(d);
    V3<T> local = qrot(conj(brot), apos - bpos);
    V3<T> al = vabs(local);
    bool inside = al.x <= half.x && al.y <= half.y && al.z <= half.z;
    V3<T> n;
    if (inside) {
        V3<T> cl = half - al;
        V3<T> axis;
        if (cl.x <= cl.y && cl.x <= cl.z) axis = VX<T>() * signum(local.x);
        else if (cl.y <= cl.z) axis = VY<T>() * signum(local.y);
        else axis = VZ<T>() * signum(local.z);
        n = normalize_or(pb - apos, qrot(brot, axis));
    } else {
        n = normalize_or(d, VX<T>());
    }
    return {inside ? -core - r : core - r, apos - n * r, pb};
}

template <class T> static Dist<T> sphere_capsule(V3<T> apos, T r, V3<T> bpos, Qt<T> brot, T cr, T hh) {  // :219-230
    V3<T> s0, s1;
    capsule_segment(bpos, hh, brot, s0, s1);
    V3<T> cb = point_segment_closest(apos, s0, s1);
    V3<T> d = apos - cb;
    T core = len(d);
    V3<T> n = normalize_or(d, VX<T>());
    return {core - r - cr, apos - n * r, cb + n * cr};
}

template <class T> static Dist<T> capsule_capsule(V3<T> apos, Qt<T> arot, T ra, T ha, V3<T> bpos, Qt<T> brot, T rb, T hb) {  // :233-245
    V3<T> a0, a1, b0, b1, ca, cb;
    capsule_segment(apos, ha, arot, a0, a1);
    capsule_segment(bpos, hb, brot, b0, b1);
    seg_seg_closest(a0, a1, b0, b1, ca, cb);
    V3<T> d = cb - ca;
    T core = len(d);
    V3<T> n = normalize_or(d, VX<T>());
    return {core - ra - rb, ca + n * ra, cb - n * rb};
}

// gjk.rs:68-186 (support) for the path's shapes.
template <class T> static V3<T> support(uint32_t shape, V3<T> sp, V3<T> pos, Qt<T> rot, V3<T> dir) {
    switch (shape) {
        case AVBD_SHAPE_SPHERE:
            return pos + normalize_or(dir, VX<T>()) * sp.x;
        case AVBD_SHAPE_BOX: {
            V3<T> l = qrot(conj(rot), dir);
            V3<T> s{l.x >= T(0) ? T(1) : T(-1), l.y >= T(0) ? T(1) : T(-1), l.z >= T(0) ? T(1) : T(-1)};
            return pos + qrot(rot, V3<T>{sp.x * s.x, sp.y * s.y, sp.z * s.z});
        }
        case AVBD_SHAPE_CAPSULE: {
            V3<T> axis = qrot(rot, VY<T>());
            V3<T> tip = (dot(dir, axis) >= T(0) ? axis : -axis) * sp.y;
            return pos + tip + normalize_or(dir, VX<T>()) * sp.x;
        }
        default:
            return pos;
    }
}

// collision/distance_box.rs
template <class T> static void separating_axis(V3<T> apos, Qt<T> arot, V3<T> ha, V3<T> bpos, Qt<T> brot, V3<T> hb,
                                               T& gap_out, V3<T>& n_out) {  // :21-50
    V3<T> aa[3], bb[3];
    mat3_from_quat(arot, aa);
    mat3_from_quat(brot, bb);
    V3<T> axes[15];
    for (int i = 0; i < 3; i++) axes[i] = aa[i];
    for (int i = 0; i < 3; i++) axes[3 + i] = bb[i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            V3<T> c = cross(aa[i], bb[j]);
            axes[6 + 3 * i + j] = len2(c) > C<T>(K::DEGENERATE_EPS) ? normalize(c) : VZERO<T>();
        }
    V3<T> delta = bpos - apos;
    T best = -std::numeric_limits<T>::infinity();
    V3<T> bn = VY<T>();
    for (int k = 0; k < 15; k++) {
        V3<T> n = axes[k];
        if (n == VZERO<T>()) continue;
        T ea = ha.x * std::fabs(dot(n, aa[0])) + ha.y * std::fabs(dot(n, aa[1])) + ha.z * std::fabs(dot(n, aa[2]));
        T eb = hb.x * std::fabs(dot(n, bb[0])) + hb.y * std::fabs(dot(n, bb[1])) + hb.z * std::fabs(dot(n, bb[2]));
        T proj = dot(delta, n);
        T gap = std::fabs(proj) - ea - eb;
        if (gap > best) {
            best = gap;
            bn = proj >= T(0) ? n : -n;
        }
    }
    gap_out = best;
    n_out = bn;
}

template <class T> static T box_box_signed_gap(V3<T> apos, Qt<T> arot, V3<T> ha, V3<T> bpos, Qt<T> brot, V3<T> hb) {
    T g;
    V3<T> n;
    separating_axis(apos, arot, ha, bpos, brot, hb, g, n);
    return g;
}

template <class T> static void support_face(V3<T> pos, Qt<T> rot, V3<T> half, V3<T> dir, V3<T>& fpos, V3<T>& ext) {  // :80-97
    V3<T> local = qrot(conj(rot), dir);
    V3<T> off = VZERO<T>();
    ext = half;
    for (int i = 0; i < 3; i++) {
        if (std::fabs(local[i]) > C<T>(K::FACE_AXIS_EPS)) {
            off[i] = signum(local[i]) * half[i];
            ext[i] = T(0);
        }
    }
    fpos = pos + qrot(rot, off);
}

template <class T> static Dist<T> feature_distance(V3<T> apos, Qt<T> arot, V3<T> ha, V3<T> bpos, Qt<T> brot, V3<T> hb) {  // :99-129
    V3<T> ca[8], cb[8];
    obb_corners(apos, ha, arot, ca);
    obb_corners(bpos, hb, brot, cb);
    Dist<T> res{std::numeric_limits<T>::infinity(), apos, bpos};
    T best = std::numeric_limits<T>::infinity();
    auto consider = [&](V3<T> x, V3<T> y) {
        T sq = len2(y - x);
        if (sq < best) {
            best = sq;
            res = {std::sqrt(sq), x, y};
        }
    };
    for (int i = 0; i < 8; i++) consider(ca[i], point_obb_closest(ca[i], bpos, hb, brot));
    for (int i = 0; i < 8; i++) consider(point_obb_closest(cb[i], apos, ha, arot), cb[i]);
    for (int i = 0; i < 12; i++)
        for (int j = 0; j < 12; j++) {
            V3<T> x, y;
            seg_seg_closest(ca[OBB_EDGES[i][0]], ca[OBB_EDGES[i][1]], cb[OBB_EDGES[j][0]], cb[OBB_EDGES[j][1]], x, y);
            consider(x, y);
        }
    return res;
}

template <class T> static Dist<T> box_box(V3<T> apos, Qt<T> arot, V3<T> ha, V3<T> bpos, Qt<T> brot, V3<T> hb) {  // :131-142
    T gap;
    V3<T> n;
    separating_axis(apos, arot, ha, bpos, brot, hb, gap, n);
    if (gap > T(0)) return feature_distance(apos, arot, ha, bpos, brot, hb);
    V3<T> fa, ea, fb, eb;
    support_face(apos, arot, ha, n, fa, ea);
    support_face(bpos, brot, hb, -n, fb, eb);
    Dist<T> r = feature_distance(fa, arot, ea, fb, brot, eb);
    r.dist = gap;
    return r;
}

template <class T> static void segment_box(V3<T> start, V3<T> end, V3<T> lo, V3<T> hi, V3<T>& opoint, V3<T>& oclosest,
                                           T& osq) {  // :146-190
    V3<T> delta = end - start;
    T cuts[8];
    int nc = 0;
    cuts[nc++] = T(0);
    cuts[nc++] = T(1);
    for (int i = 0; i < 3; i++) {
        if (std::fabs(delta[i]) > C<T>(K::DEGENERATE_EPS)) {
            T bnds[2] = {lo[i], hi[i]};
            for (T bd : bnds) {
                T t = (bd - start[i]) / delta[i];
                if (t > T(0) && t < T(1)) cuts[nc++] = t;
            }
        }
    }
    for (int i = 1; i < nc; i++)  // ascending (f32::total_cmp on finite values)
        for (int k = i; k > 0 && cuts[k] < cuts[k - 1]; k--) std::swap(cuts[k], cuts[k - 1]);
    opoint = start;
    oclosest = vclamp(start, lo, hi);
    osq = std::numeric_limits<T>::infinity();
    for (int w = 0; w + 1 < nc; w++) {
        T r0 = cuts[w], r1 = cuts[w + 1];
        T middle = (r0 + r1) * C<T>(K::HALF);
        V3<T> p = start + middle * delta;
        T num = T(0), den = T(0);
        for (int i = 0; i < 3; i++) {
            bool has = false;
            T bd = T(0);
            if (p[i] < lo[i]) { has = true; bd = lo[i]; }
            else if (p[i] > hi[i]) { has = true; bd = hi[i]; }
            if (has) {
                num += delta[i] * (start[i] - bd);
                den += delta[i] * delta[i];
            }
        }
        T stationary = den > T(0) ? fclamp(-num / den, r0, r1) : middle;
        T ts[3] = {stationary, r0, r1};
        for (T t : ts) {
            V3<T> point = start + t * delta;
            V3<T> cl = vclamp(point, lo, hi);
            T sq = len2(point - cl);
            if (sq < osq) {
                opoint = point;
                oclosest = cl;
                osq = sq;
            }
        }
    }
}

template <class T> static void spine_penetration(V3<T> center, V3<T> axis, V3<T> half, T radius, T height, T& og,
                                                 V3<T>& on) {  // :240-265
    og = -std::numeric_limits<T>::infinity();
    on = VX<T>();
    V3<T> es[3] = {VX<T>(), VY<T>(), VZ<T>()};
    for (auto e : es) {
        V3<T> ns[2] = {e, normalize_or_zero(cross(axis, e))};
        for (auto n : ns) {
            if (n == VZERO<T>()) continue;
            T proj = dot(center, n);
            T gap = std::fabs(proj) - dot(half, vabs(n)) - height * std::fabs(dot(axis, n)) - radius;
            if (gap > og) {
                og = gap;
                on = proj >= T(0) ? n : -n;
            }
        }
    }
}

template <class T> static Dist<T> box_capsule(V3<T> apos, Qt<T> arot, V3<T> half, V3<T> bpos, Qt<T> brot, T radius,
                                              T height) {  // :192-236
    Qt<T> inv = conj(arot);
    V3<T> center = qrot(inv, bpos - apos);
    V3<T> axis = qrot(inv, qrot(brot, VY<T>()));
    V3<T> start = center - axis * height, end = center + axis * height;
    V3<T> core, surface;
    T sq;
    segment_box(start, end, -half, half, core, surface, sq);
    T distance;
    V3<T> normal;
    if (sq > C<T>(K::DEGENERATE_EPS)) {
        T l = std::sqrt(sq);
        distance = l - radius;
        normal = (core - surface) / l;
    } else {
        T depth;
        V3<T> nrm;
        spine_penetration(center, axis, half, radius, height, depth, nrm);
        V3<T> lo = -half, hi = half;
        for (int i = 0; i < 3; i++) {
            if (std::fabs(nrm[i]) > C<T>(K::FACE_AXIS_EPS)) {
                lo[i] = signum(nrm[i]) * half[i];
                hi[i] = lo[i];
            }
        }
        T proj = dot(axis, nrm);
        V3<T> e0, e1;
        if (proj > C<T>(K::SPINE_ALIGNMENT_EPS)) { e0 = start; e1 = start; }
        else if (proj < -C<T>(K::SPINE_ALIGNMENT_EPS)) { e0 = end; e1 = end; }
        else { e0 = start; e1 = end; }
        T dummy;
        segment_box(e0, e1, lo, hi, core, surface, dummy);
        distance = depth;
        normal = nrm;
    }
    return {distance, apos + qrot(arot, surface), apos + qrot(arot, core - normal * radius)};
}

#include "avbd_gjk.hpp"

template <class T> static Dist<T> halfspace_distance(V3<T> hpos, Qt<T> hrot, V3<T> ln, const ShapeRef<T>& o, bool first) {  // :607-642
    if (o.shape == AVBD_SHAPE_HALFSPACE) {
        T inf = std::numeric_limits<T>::infinity();
        return first ? Dist<T>{inf, hpos, o.pos} : Dist<T>{inf, o.pos, hpos};
    }
    V3<T> n = qrot(hrot, ln);
    V3<T> s = support_any(o, -n);
    T dist = dot(s - hpos, n);
    Dist<T> d{dist, s - n * dist, s};
    if (first) return d;
    return {d.dist, d.pb, d.pa};
}

// shape_distance (distance.rs:654-821) for sphere/box/capsule/half-space.
template <class T> static Dist<T> shape_distance(const ShapeRef<T>& a, const ShapeRef<T>& b) {
    if (a.shape == AVBD_SHAPE_HALFSPACE) return halfspace_distance(a.pos, a.rot, a.sp, b, true);
    if (b.shape == AVBD_SHAPE_HALFSPACE) return halfspace_distance(b.pos, b.rot, b.sp, a, false);
    uint32_t sa = a.shape, sb = b.shape;
    if (gjk_shape<T>(sa) || gjk_shape<T>(sb)) return gjk_pair_distance(a, b);  // distance.rs:811-817
    auto swap = [](Dist<T> d) { return Dist<T>{d.dist, d.pb, d.pa}; };
    if (sa == AVBD_SHAPE_SPHERE && sb == AVBD_SHAPE_SPHERE) return sphere_sphere(a.pos, a.sp.x, b.pos, b.sp.x);
    if (sa == AVBD_SHAPE_SPHERE && sb == AVBD_SHAPE_BOX) return sphere_obb(a.pos, a.sp.x, b.pos, b.rot, b.sp);
    if (sa == AVBD_SHAPE_BOX && sb == AVBD_SHAPE_SPHERE) return swap(sphere_obb(b.pos, b.sp.x, a.pos, a.rot, a.sp));
    if (sa == AVBD_SHAPE_SPHERE && sb == AVBD_SHAPE_CAPSULE)
        return sphere_capsule(a.pos, a.sp.x, b.pos, b.rot, b.sp.x, b.sp.y);
    if (sa == AVBD_SHAPE_CAPSULE && sb == AVBD_SHAPE_SPHERE)
        return swap(sphere_capsule(b.pos, b.sp.x, a.pos, a.rot, a.sp.x, a.sp.y));
    if (sa == AVBD_SHAPE_BOX && sb == AVBD_SHAPE_BOX) return box_box(a.pos, a.rot, a.sp, b.pos, b.rot, b.sp);
    if (sa == AVBD_SHAPE_BOX && sb == AVBD_SHAPE_CAPSULE)
        return box_capsule(a.pos, a.rot, a.sp, b.pos, b.rot, b.sp.x, b.sp.y);
    if (sa == AVBD_SHAPE_CAPSULE && sb == AVBD_SHAPE_BOX)
        return swap(box_capsule(b.pos, b.rot, b.sp, a.pos, a.rot, a.sp.x, a.sp.y));
    // capsule-capsule
    return capsule_capsule(a.pos, a.rot, a.sp.x, a.sp.y, b.pos, b.rot, b.sp.x, b.sp.y);
}

// Rounded-shape distance offset (distance.rs:519-545): the rounded surface
// sits `r` closer along the witness axis; an infinite distance stays.
template <class T> static Dist<T> round_offset(Dist<T> d, T r, bool first, V3<T> pos_a, V3<T> pos_b) {
    if (!std::isfinite(d.dist)) return d;
    V3<T> axis = d.pb - d.pa;
    if (len2(axis) <= C<T>(gjk::COINCIDENT_LEN2)) axis = pos_b - pos_a;
    V3<T> n = normalize_or(axis, VX<T>());
    if (first) return {d.dist - r, d.pa + n * r, d.pb};
    return {d.dist - r, d.pa, d.pb - n * r};
}
// Pose::world_rot (shape.rs:119-134): the child's rotation under its parent,
// normalized, or the parent's for a degenerate product.
template <class T> static Qt<T> pose_world_rot(Qt<T> parent, Qt<T> local) {
    Qt<T> q = qmul(parent, local);
    T l2 = (q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w);
    if (std::isfinite(q.x) && std::isfinite(q.y) && std::isfinite(q.z) && std::isfinite(q.w) &&
        l2 > C<T>(K::DEGENERATE_LEN2))
        return qnormalize(q);
    return parent;
}
template <class T> static Dist<T> shape_distance_any(const ShapeRef<T>& a, const ShapeRef<T>& b);
// Shape::aabb (shape.rs:619-680) of a primitive.
template <class T> static void prim_aabb(const ShapeRef<T>& s, V3<T>& lo, V3<T>& hi) {
    auto absv = [](V3<T> v) { return V3<T>{std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)}; };
    V3<T> r;
    switch (s.shape) {
        case AVBD_SHAPE_SPHERE: r = {s.sp.x, s.sp.x, s.sp.x}; break;
        case AVBD_SHAPE_BOX:
            r = (absv(qrot(s.rot, VX<T>())) * s.sp.x + absv(qrot(s.rot, VY<T>())) * s.sp.y) +
                absv(qrot(s.rot, VZ<T>())) * s.sp.z;
            break;
        case AVBD_SHAPE_HULL: {
            V3<T> mn{std::numeric_limits<T>::infinity(), std::numeric_limits<T>::infinity(),
                     std::numeric_limits<T>::infinity()};
            V3<T> mx = -mn;
            if (!s.hull || s.hull->verts.empty()) {
                lo = hi = s.pos;
                return;
            }
            for (const V3<T>& v : s.hull->verts) {
                V3<T> w = s.pos + qrot(s.rot, v);
                mn = {fmn(mn.x, w.x), fmn(mn.y, w.y), fmn(mn.z, w.z)};
                mx = {fmx(mx.x, w.x), fmx(mx.y, w.y), fmx(mx.z, w.z)};
            }
            lo = mn;
            hi = mx;
            return;
        }
        default: {  // capsule, cylinder, cone: the axis shell plus the radius
            V3<T> e = absv(qrot(s.rot, VY<T>())) * s.sp.y;
            r = {e.x + s.sp.x, e.y + s.sp.x, e.z + s.sp.x};
        }
    }
    lo = s.pos - r;
    hi = s.pos + r;
}
// The convex side's AABB corners in the frame of (pos, rot): their bounds.
template <class T> static void local_window(const ShapeRef<T>& convex, V3<T> pos, Qt<T> rot, V3<T>& lo, V3<T>& hi) {
    V3<T> amin, amax;
    prim_aabb(convex, amin, amax);
    const Qt<T> inv = conj(rot);
    lo = {std::numeric_limits<T>::infinity(), std::numeric_limits<T>::infinity(), std::numeric_limits<T>::infinity()};
    hi = -lo;
    for (int i = 0; i < 8; i++) {
        V3<T> corner{(i & 1) ? amax.x : amin.x, (i & 2) ? amax.y : amin.y, (i & 4) ? amax.z : amin.z};
        V3<T> l = qrot(inv, corner - pos);
        lo = {fmn(lo.x, l.x), fmn(lo.y, l.y), fmn(lo.z, l.z)};
        hi = {fmx(hi.x, l.x), fmx(hi.y, l.y), fmx(hi.z, l.z)};
    }
}
// heightfield_convex (distance.rs:246-350): the nearest of the overlapped
// columns, each a solid box from the lowest sample up to its height (a
// flat one a one-cell skirt); `first`: the terrain owns pa.
template <class T> static Dist<T> hf_convex(const ShapeRef<T>& t, const ShapeRef<T>& convex, bool first) {
    const HField<T>& hf = *t.hf;
    const T inf = std::numeric_limits<T>::infinity();
    V3<T> lo, hi;
    local_window(convex, t.pos, t.rot, lo, hi);
    const T half = C<T>(K::HALF);
    // the column index along x serves the rows too (distance.rs:299-303)
    auto col_at = [&](T x, uint32_t n) -> uint32_t {
        T f = std::floor(x / hf.cell + T(hf.cols - 1) * half);
        if (!(f > T(0))) return 0u;  // NaN and below zero clamp to 0
        return f >= T(n - 1) ? n - 1 : (uint32_t)(double)f;
    };
    const uint32_t c0 = col_at(lo.x, hf.cols), c1 = col_at(hi.x, hf.cols);
    const uint32_t r0 = col_at(lo.z, hf.rows), r1 = col_at(hi.z, hf.rows);
    const T x_origin = -T(hf.cols - 1) * half * hf.cell, z_origin = -T(hf.rows - 1) * half * hf.cell;
    bool have = false;
    Dist<T> best{};
    for (uint32_t row = r0; row <= r1; row++)
        for (uint32_t col = c0; col <= c1; col++) {
            const T h = hf.h[(size_t)row * hf.cols + col];
            const T y_low = h - hf.y_min >= C<T>(1e-4f) ? hf.y_min : h - fmx(hf.cell, C<T>(1e-3f));
            V3<T> mn{x_origin + T(col) * hf.cell, y_low, z_origin + T(row) * hf.cell};
            V3<T> mx{mn.x + hf.cell, fmx(h, y_low), mn.z + hf.cell};
            V3<T> center = (mn + mx) * half;
            V3<T> hl = (mx - mn) * half;
            hl = {fmx(hl.x, T(0)), fmx(hl.y, T(0)), fmx(hl.z, T(0))};
            ShapeRef<T> column{nullptr, AVBD_SHAPE_BOX, hl, t.pos + qrot(t.rot, center), t.rot, nullptr};
            Dist<T> d = shape_distance(column, convex);
            if (!have || d.dist < best.dist) {
                best = d;
                have = true;
            }
        }
    if (!have) return first ? Dist<T>{inf, t.pos, convex.pos} : Dist<T>{inf, convex.pos, t.pos};
    return first ? best : Dist<T>{best.dist, best.pb, best.pa};
}
// trimesh_convex (distance.rs:416-517): the nearest of the triangles whose
// tree boxes overlap the convex side's window, walked last-in-first-out; the
// winner's witnesses come back swapped when the mesh is the first shape and
// as found when it is the second (the reference's own order, kept).
template <class T> static Dist<T> mesh_convex(const ShapeRef<T>& m, const ShapeRef<T>& convex, bool first) {
    const TMesh<T>& mesh = *m.mesh;
    const T inf = std::numeric_limits<T>::infinity();
    const Dist<T> none = first ? Dist<T>{inf, m.pos, convex.pos} : Dist<T>{inf, convex.pos, m.pos};
    if (mesh.tris.empty()) return none;
    V3<T> lo, hi;
    local_window(convex, m.pos, m.rot, lo, hi);
    bool have = false;
    Dist<T> best{};
    uint32_t stack[64];
    size_t len = 1;
    stack[0] = 0;
    while (len > 0) {
        const uint32_t ni = stack[--len];
        if (ni >= mesh.nodes.size()) continue;
        const BNode<T>& node = mesh.nodes[ni];
        if (node.hi.x < lo.x || node.lo.x > hi.x || node.hi.y < lo.y || node.lo.y > hi.y || node.hi.z < lo.z ||
            node.lo.z > hi.z)
            continue;
        if (node.leaf) {
            const size_t end = std::min<size_t>((size_t)node.a + node.b, mesh.order.size());
            for (size_t o = node.a; o < end; o++) {
                const uint32_t tri = mesh.order[o];
                if (tri >= mesh.tris.size()) continue;
                ShapeRef<T> th{nullptr, AVBD_SHAPE_HULL, VZERO<T>(), m.pos + qrot(m.rot, mesh.cent[tri]), m.rot,
                               &mesh.tris[tri]};
                Dist<T> d = shape_distance(th, convex);
                if (!have || d.dist < best.dist) {
                    best = d;
                    have = true;
                }
            }
        } else {
            if (len + 2 > 64) break;  // depth guard: keep the best so far
            stack[len] = node.a;
            stack[len + 1] = node.b;
            len += 2;
        }
    }
    if (!have) return none;
    return first ? Dist<T>{best.dist, best.pb, best.pa} : best;
}
// shape_distance below the rounded and compound arms (distance.rs:706-745):
// half-spaces, terrain, meshes, then the primitive pairs.
template <class T> static Dist<T> shape_distance_leaf(const ShapeRef<T>& a, const ShapeRef<T>& b) {
    const T inf = std::numeric_limits<T>::infinity();
    if (a.shape == AVBD_SHAPE_HALFSPACE || b.shape == AVBD_SHAPE_HALFSPACE) return shape_distance(a, b);
    const bool ta = a.shape == AVBD_SHAPE_HEIGHTFIELD, tb = b.shape == AVBD_SHAPE_HEIGHTFIELD;
    const bool ma = a.shape == AVBD_SHAPE_TRIMESH, mb = b.shape == AVBD_SHAPE_TRIMESH;
    if ((ta && !a.hf) || (tb && !b.hf) || (ma && !a.mesh) || (mb && !b.mesh)) return {inf, a.pos, b.pos};
    // terrain against terrain or a mesh, mesh against mesh: separation
    if ((ta || ma) && (tb || mb)) return {inf, a.pos, b.pos};
    if (ta) return hf_convex(a, b, true);
    if (tb) return hf_convex(b, a, false);
    if (ma) return mesh_convex(a, b, true);
    if (mb) return mesh_convex(b, a, false);
    return shape_distance(a, b);
}
// compound_distance (distance.rs:550-599): the child that reports the
// smallest distance, children in order; `first`: the compound owns pa.
template <class T> static Dist<T> compound_distance(const ShapeRef<T>& c, const ShapeRef<T>& other, bool first) {
    bool have = false;
    Dist<T> best{};
    for (const Part<T>& part : c.ext->parts) {
        ShapeRef<T> child{nullptr, part.shape, part.sp, c.pos + qrot(c.rot, part.pos), pose_world_rot(c.rot, part.rot),
                          part.hull, nullptr};
        Dist<T> d = shape_distance_leaf(child, other);
        // a rounded child peels inside its own query (distance.rs:654-685)
        if (part.radius > T(0)) d = round_offset(d, part.radius, true, child.pos, other.pos);
        if (!have || d.dist < best.dist) {
            best = d;
            have = true;
        }
    }
    if (!have) return first ? Dist<T>{std::numeric_limits<T>::infinity(), c.pos, other.pos}
                            : Dist<T>{std::numeric_limits<T>::infinity(), other.pos, c.pos};
    return first ? best : Dist<T>{best.dist, best.pb, best.pa};
}
// shape_distance's wrapper arms (distance.rs:648-705): rounded shapes peel
// first (a's, then b's), then compounds expand; compound-vs-compound is
// separation.  Rounded inners and compound children are primitives here.
template <class T> static Dist<T> shape_distance_any(const ShapeRef<T>& a, const ShapeRef<T>& b) {
    const bool ext_a = a.shape == AVBD_SHAPE_ROUND || a.shape == AVBD_SHAPE_COMPOUND;
    const bool ext_b = b.shape == AVBD_SHAPE_ROUND || b.shape == AVBD_SHAPE_COMPOUND;
    if ((ext_a && !a.ext) || (ext_b && !b.ext)) return {std::numeric_limits<T>::infinity(), a.pos, b.pos};
    if (a.shape == AVBD_SHAPE_ROUND) {
        const Part<T>& in = a.ext->parts[0];
        ShapeRef<T> inner{nullptr, in.shape, in.sp, a.pos, a.rot, in.hull, nullptr};
        return round_offset(shape_distance_any(inner, b), in.radius, true, a.pos, b.pos);
    }
    if (b.shape == AVBD_SHAPE_ROUND) {
        const Part<T>& in = b.ext->parts[0];
        ShapeRef<T> inner{nullptr, in.shape, in.sp, b.pos, b.rot, in.hull, nullptr};
        return round_offset(shape_distance_any(a, inner), in.radius, false, a.pos, b.pos);
    }
    if (a.shape == AVBD_SHAPE_COMPOUND) {
        if (b.shape == AVBD_SHAPE_COMPOUND) return {std::numeric_limits<T>::infinity(), a.pos, b.pos};
        return compound_distance(a, b, true);
    }
    if (b.shape == AVBD_SHAPE_COMPOUND) return compound_distance(b, a, false);
    return shape_distance_leaf(a, b);
}

// ---- AVBD engine (avbd/*) ------------------------------------------------------
template <class T> struct Point {
    V3<T> ra, rb;
    T lam[3], pen[3];
    bool stuck;
    T roll_lam[3];
    int32_t matched;
    bool kept;  // anchors kept from a stuck point of the previous substep
};
template <class T> struct Pair {
    uint32_t a, b;
    V3<T> n;
    T mu[2];
    T gap;
    std::vector<Point<T>> points;
};
template <class T> struct Joint {  // AvbdJoint (avbd/mod.rs:327-402)
    uint32_t a, b, kind;
    V3<T> la, lb, ax_a, ax_b;
    // revolute reference twist, prismatic reference length, distance rest
    // length, rope maximum
    T ref_val;
    bool has_lim;
    T lo, hi;
    T acc_lim;   // revolute limit accumulator
    T lim_dual;  // prismatic limit force
    bool has_mot;
    T mot_speed, mot_max;
    Qt<T> q_ref;  // fixed / sixdof: qa^-1 qb at assembly
    V3<T> dref;   // fixed / sixdof: anchor separation in A's frame at assembly
    uint32_t six_cfg[6];
    T six_min[6], six_max[6];
    T sacc[6];
    // free motor (JointKind::Motor): velocity targets and budgets
    V3<T> mot_lin, mot_ang;
    T mot_force, mot_torque;
    // spring (JointKind::Spring): its JointMotor
    T spr_vel, spr_k, spr_c, spr_max;
    uint32_t spr_kind, spr_model;
    // wheel (JointKind::Wheel): spin axles, suspension frequency and damping ratio
    V3<T> bx_a, bx_b;
    T susp_hz, susp_zeta;
    // gear (JointKind::Gear): the coupled joints, the ratio, and the
    // coordinates at the last step start (gear_mem, avbd/mod.rs:373-383)
    uint32_t gb[2];
    T gratio;
    bool gmem_set;
    T graw[2], gcont[2];
    T lam_l[3], lam_a[3], pen_l[3], pen_a[3];
};

// One side of a gear (GearSide, avbd/mod.rs:304-317): the coupled joint's
// bodies, whether it turns (revolute) or slides (prismatic), its live world
// axis, the slide's anchor levers and its continuous coordinate.
template <class T> struct GearSide {
    uint32_t a, b;
    bool angular;
    V3<T> axis, ra, rb;
    T coord;
};

template <class T> static V3<T> tangent_t1(V3<T> n) {  // math.rs:152-160
    V3<T> axis = std::fabs(n.x) < C<T>(K::TANGENT_REF_AXIS_DOT) ? VX<T>() : VY<T>();
    return normalize_or(cross(n, axis), VZ<T>());
}
template <class T> static void tangent_basis(V3<T> n, V3<T>& t1, V3<T>& t2) {
    t1 = tangent_t1(n);
    t2 = cross(t1, n);
}
// math.rs:179-186: the axle made orthogonal to the suspension axis
template <class T> static V3<T> orthogonalize_axle(V3<T> s, V3<T> axle) {
    V3<T> a = axle - s * dot(axle, s);
    if (len2(a) < C<T>(K::POS_CORRECTION_EPS)) return tangent_t1(s);
    return normalize(a);
}

// avbd/rows.rs helpers
template <class T> static Qt<T> quat_integrate(Qt<T> q, V3<T> v) {  // :110-119
    T theta = len(v);
    if (theta < C<T>(K::NEAR_ZERO)) return q;
    T hth = C<T>(K::HALF) * theta;
    T s = osin(hth), c = ocos(hth);
    T k = s / theta;
    Qt<T> dq = qmul(Qt<T>{v.x * k, v.y * k, v.z * k, c}, q);
    return qnormalize(dq);
}
template <class T> static V3<T> quat_diff_vec(Qt<T> a, Qt<T> b) {  // :128-146
    Qt<T> r = qmul(a, Qt<T>{-b.x, -b.y, -b.z, b.w});
    V3<T> xyz{r.x, r.y, r.z};
    if (r.w < T(0)) xyz = -xyz;
    T s = fmn(len(xyz), T(1));
    if (s < C<T>(K::NEAR_ZERO)) return VZERO<T>();
    return xyz * (T(2) * oasin(s) / s);
}
template <class T> static T rem_euclid(T x, T m) {
    T r = std::fmod(x, m);
    return r < T(0) ? r + std::fabs(m) : r;
}
template <class T> static T wrap_pi(T x) { return rem_euclid(x + C<T>(K::PI), C<T>(K::TAU)) - C<T>(K::PI); }
template <class T> static T quat_twist(Qt<T> q, V3<T> axis) {  // sequential_impulse/joints.rs:44-48
    T t = T(2) * oatan2(dot(V3<T>{q.x, q.y, q.z}, axis), q.w);
    return rem_euclid(t + C<T>(K::PI), C<T>(K::TAU)) - C<T>(K::PI);
}
template <class T> static T hinge_twist(Qt<T> qa, Qt<T> qb, V3<T> axis) { return quat_twist(qmul(conj(qa), qb), axis); }

template <class T> static int limit_state(T v, T lo, T hi, T slop) {  // :156-164  (1 lower, 0 upper, -1 none)
    if (v <= lo + slop) return 1;
    if (v >= hi - slop) return 0;
    return -1;
}
template <class T> static int warm_limit_state(T v, T lo, T hi, T slop, T force) {  // :169-183
    int s = limit_state(v, lo, hi, slop);
    if (s >= 0) return s;
    if (force < T(0)) return 1;
    if (force > T(0)) return 0;
    return -1;
}
template <class T> static T regularized_limit(T value, T initial, T bound, bool lower) {  // :187-191
    T old = initial - bound;
    T viol = lower ? fmn(old, T(0)) : fmx(old, T(0));
    return value - bound - C<T>(K::ALPHA) * viol;
}

template <class T> static void world_inertia(V3<T> inertia, Qt<T> rot, T m[3][3]) {  // :194-207
    V3<T> cols[3];
    mat3_from_quat(rot, cols);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            T ca0 = cols[0][a], ca1 = cols[1][a], ca2 = cols[2][a];
            T cb0 = cols[0][b], cb1 = cols[1][b], cb2 = cols[2][b];
            m[a][b] = ca0 * inertia.x * cb0 + ca1 * inertia.y * cb1 + ca2 * inertia.z * cb2;
        }
}
template <class T> static void inverse_symmetric(const T m[3][3], V3<T> diag, T o[3][3]) {  // :211-241
    T a = m[0][0], b = m[0][1], c = m[0][2], d = m[1][1], e = m[1][2], f = m[2][2];
    T det = a * (d * f - e * e) - b * (b * f - c * e) + c * (b * e - c * d);
    if (std::fabs(det) < C<T>(K::DEGENERATE_LEN2)) {
        T ix = diag.x > T(0) ? T(1) / diag.x : T(0);
        T iy = diag.y > T(0) ? T(1) / diag.y : T(0);
        T iz = diag.z > T(0) ? T(1) / diag.z : T(0);
        T r[3][3] = {{ix, 0, 0}, {0, iy, 0}, {0, 0, iz}};
        std::memcpy(o, r, sizeof(r));
        return;
    }
    T id = T(1) / det;
    o[0][0] = (d * f - e * e) * id; o[0][1] = (c * e - b * f) * id; o[0][2] = (b * e - c * d) * id;
    o[1][0] = (c * e - b * f) * id; o[1][1] = (a * f - c * c) * id; o[1][2] = (b * c - a * e) * id;
    o[2][0] = (b * e - c * d) * id; o[2][1] = (b * c - a * e) * id; o[2][2] = (a * d - b * b) * id;
}
template <class T> static V3<T> mat3_vec(const T m[3][3], V3<T> v) {
    return {m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
            m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z};
}

template <class T> static T bound_radius(const Body<T>& b) {  // rows.rs:253-292
    switch (b.shape) {
        case AVBD_SHAPE_SPHERE: return b.sp.x;
        case AVBD_SHAPE_BOX: return len(b.sp);
        case AVBD_SHAPE_CAPSULE: return b.sp.y + b.sp.x;
        case AVBD_SHAPE_CYLINDER:
        case AVBD_SHAPE_CONE: return std::sqrt(b.sp.x * b.sp.x + b.sp.y * b.sp.y);
        case AVBD_SHAPE_HULL: return b.hull ? b.hull->bound : T(0);
        case AVBD_SHAPE_ROUND:
        case AVBD_SHAPE_COMPOUND: return b.ext ? b.ext->bound : T(0);
        default: return std::numeric_limits<T>::infinity();
    }
}
template <class T> static T shape_min_dimension(const Body<T>& b) {  // rows.rs:373-403
    switch (b.shape) {
        case AVBD_SHAPE_SPHERE: return b.sp.x;
        case AVBD_SHAPE_BOX: return min_element(b.sp);
        case AVBD_SHAPE_CAPSULE: return b.sp.x;
        case AVBD_SHAPE_CYLINDER: return fmn(b.sp.x, b.sp.y);
        case AVBD_SHAPE_CONE: return C<T>(K::HALF) * fmn(b.sp.x, b.sp.y);
        case AVBD_SHAPE_HULL: return C<T>(K::HALF) * (b.hull ? b.hull->min_ext : T(0));
        case AVBD_SHAPE_ROUND:
        case AVBD_SHAPE_COMPOUND: return b.ext ? b.ext->min_dim : std::numeric_limits<T>::infinity();
        case AVBD_SHAPE_HEIGHTFIELD: return C<T>(K::HALF) * (b.hf ? b.hf->cell : T(0));
        case AVBD_SHAPE_TRIMESH: return C<T>(K::HALF) * (b.mesh ? b.mesh->min_feature : T(0));
        default: return std::numeric_limits<T>::infinity();
    }
}
template <class T> static bool pair_allowed(const Body<T>& a, const Body<T>& b) {  // rows.rs:366-368
    return (a.layer & b.mask) != 0 && (b.layer & a.mask) != 0;
}
template <class T> static T eff_inv_mass(const Body<T>& b) { return b.type == AVBD_BODY_DYNAMIC ? b.inv_mass : T(0); }
template <class T> static bool row_live(T c, T f) { return std::fabs(c) >= C<T>(K::C_EPS) || f != T(0); }

template <class T> static void outer(V3<T> a, V3<T> b, T o[3][3]) {
    T av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) o[i][j] = av[i] * bv[j];
}
template <class T> static void stamp_row(T lhs[6][6], T rhs[6], V3<T> axis, T pen, T f, V3<T> r, T sign) {  // :1064-1092
    V3<T> nn = sign * axis;
    V3<T> t = cross(r, nn);
    T onn[3][3], ott[3][3], ont[3][3];
    outer(nn, nn, onn);
    outer(t, t, ott);
    outer(nn, t, ont);
    for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++) {
            lhs[x][y] += pen * onn[x][y];
            lhs[3 + x][3 + y] += pen * ott[x][y];
            lhs[x][3 + y] += pen * ont[x][y];
            lhs[3 + x][y] += pen * ont[y][x];
        }
    rhs[0] += f * nn.x; rhs[1] += f * nn.y; rhs[2] += f * nn.z;
    rhs[3] += f * t.x; rhs[4] += f * t.y; rhs[5] += f * t.z;
}
template <class T> static void stamp_angular(T lhs[6][6], T rhs[6], V3<T> g, T pen, T f) {
    T o[3][3];
    outer(g, g, o);
    for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++) lhs[3 + x][3 + y] += pen * o[x][y];
    rhs[3] += f * g.x; rhs[4] += f * g.y; rhs[5] += f * g.z;
}

// avbd/assembly.rs:25-69
template <class T> static bool solve_6x6(const T lhs[6][6], const T rhs[6], T x[6]) {
    T l[6][6] = {};
    T d[6] = {};
    for (int i = 0; i < 6; i++)
        for (int j = 0; j <= i; j++) {
            T s = lhs[i][j];
            for (int k = 0; k < j; k++) s -= l[i][k] * d[k] * l[j][k];
            if (i == j) {
                if (s <= C<T>(K::DEGENERATE_LEN2)) return false;
                d[i] = s;
                l[i][i] = T(1);
            } else {
                l[i][j] = s / d[j];
            }
        }
    T y[6], z[6];
    for (int i = 0; i < 6; i++) {
        T s = rhs[i];
        for (int k = 0; k < i; k++) s -= l[i][k] * y[k];
        y[i] = s;
    }
    for (int i = 0; i < 6; i++) z[i] = y[i] / d[i];
    for (int i = 5; i >= 0; i--) {
        T s = z[i];
        for (int k = i + 1; k < 6; k++) s -= l[k][i] * x[k];
        x[i] = s;
    }
    return true;
}

// Colouring priority hash (shared definition with the GPU colouring kernel).
static inline uint32_t colour_hash(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

enum Mode { REFERENCE = 0, COLOURED = 1 };

template <class T> struct Engine {
    AvbdParams prm;
    int mode = REFERENCE;
    int threads = 1;
    bool faithful_scan = false;  // true: solve_body scans every pair/joint (the reference's O(P) scan)
    // true: a pair's rows are summed on their own before they join the body's
    // system (the device's split primal, whose rounding this reproduces)
    bool split_sums = false;
    // Dual numbers only: hold each step's contact frames (normal, gap, local
    // anchors) fixed in the derivative, the device adjoint's convention; the
    // step-start gap keeps the derivative of n.(witness_a - witness_b) with
    // the witnesses carried by the bodies.
    bool freeze_frames = false;
    int freeze_bits = 7;
    // Finite joint stiffness (0: the reference's hard joints).  A soft joint
    // row is a spring of that stiffness: penalty = stiffness, lambda = 0.
    T joint_k = T(0);
    V3<T> gravity;
    T dt;
    std::vector<Body<T>> bodies;
    std::vector<Pair<T>> pairs;
    std::vector<Joint<T>> joints;
    std::vector<V3<T>> pos0, inertial, prev_pos;
    std::vector<Qt<T>> rot0, inertial_rot, prev_rot;
    std::vector<T> sleep_timer;
    std::vector<uint8_t> asleep;
    std::vector<int32_t> colour;
    T time_debt = T(0);
    uint64_t steps = 0, breakdowns = 0, ccd_hits = 0;
    uint64_t ncolours = 0;
    // adjacency (same order as the pair vector) for the non-faithful sweep
    std::vector<std::vector<uint32_t>> adj_pairs, adj_joints;
    // events (mod.rs:425-464 event state, :1606-1669 emit_events)
    using Key = std::pair<uint32_t, uint32_t>;
    std::set<Key> prev_touch, prev_trigger, trig_now;
    std::vector<AvbdContactEvent> cev;
    std::vector<AvbdTriggerEvent> tev;
    std::vector<V3<T>> pre_vel;
    std::vector<AvbdContactEvent> ccd_ev;  // this substep's swept hits (mod.rs:935-960)
    int emit_period = 0;                   // 0: the last substep of each step call emits

    bool solvable(uint32_t h) const { return bodies[h].type == AVBD_BODY_DYNAMIC && bodies[h].inv_mass > T(0); }

    void ensure_scratch() {  // mod.rs:1183-1200
        size_t n = bodies.size(), old = pos0.size();
        pos0.resize(n, VZERO<T>()); rot0.resize(n, qident<T>());
        inertial.resize(n, VZERO<T>()); inertial_rot.resize(n, qident<T>());
        sleep_timer.resize(n, T(0)); asleep.resize(n, 0);
        prev_pos.resize(n, VZERO<T>()); prev_rot.resize(n, qident<T>());
        colour.resize(n, -1);
        for (size_t h = std::min(old, n); h < n; h++) { prev_pos[h] = bodies[h].pos; prev_rot[h] = bodies[h].rot; }
    }

    void sleep_body(uint32_t h) {  // mod.rs:822-828, body.rs:403-408
        if (h >= asleep.size() || bodies[h].type != AVBD_BODY_DYNAMIC) return;
        Body<T>& b = bodies[h];
        b.vel = VZERO<T>(); b.angvel = VZERO<T>(); b.inv_mass = T(0); b.inertia = VZERO<T>();
        asleep[h] = 1;
    }
    void wake_body(uint32_t h) {  // mod.rs:833-842, body.rs:412-418
        if (h >= asleep.size() || !asleep[h]) return;
        asleep[h] = 0;
        sleep_timer[h] = T(0);
        Body<T>& b = bodies[h];
        if (b.type == AVBD_BODY_DYNAMIC) {
            T m = b.mass;
            b.inv_mass = (m > T(0)) ? T(1) / m : T(0);
            const bool by_unit = b.shape == AVBD_SHAPE_HULL || b.shape == AVBD_SHAPE_ROUND || b.shape == AVBD_SHAPE_COMPOUND;
            const V3<T> unit = b.shape == AVBD_SHAPE_HULL ? (b.hull ? b.hull->unit_inertia : VZERO<T>())
                                                          : (b.ext ? b.ext->unit_inertia : VZERO<T>());
            b.inertia = by_unit ? (m > T(0) && std::isfinite(m) ? unit * m : VZERO<T>()) : shape_inertia(b.shape, b.sp, m);
        }
    }
    std::deque<Hull<T>> hulls;  // stable addresses: bodies point at them
    std::deque<ExtShape<T>> exts;  // rounded and compound shapes, likewise
    std::deque<HField<T>> hfs;     // heightfields
    std::deque<TMesh<T>> meshes;   // triangle meshes
    void link_hull(Body<T>& b) {
        b.hull = nullptr;
        b.ext = nullptr;
        b.hf = nullptr;
        b.mesh = nullptr;
        double id = (double)b.sp.x;
        if (b.shape == AVBD_SHAPE_HEIGHTFIELD && id >= 0.0 && id < (double)hfs.size()) b.hf = &hfs[(size_t)id];
        if (b.shape == AVBD_SHAPE_TRIMESH && id >= 0.0 && id < (double)meshes.size()) b.mesh = &meshes[(size_t)id];
        if (b.shape == AVBD_SHAPE_HULL && id >= 0.0 && id < (double)hulls.size()) b.hull = &hulls[(size_t)id];
        if ((b.shape == AVBD_SHAPE_ROUND || b.shape == AVBD_SHAPE_COMPOUND) && id >= 0.0 && id < (double)exts.size() &&
            exts[(size_t)id].compound == (b.shape == AVBD_SHAPE_COMPOUND))
            b.ext = &exts[(size_t)id];
    }
    // Heightfield::new (shape.rs:1485-1505, invariants.rs:403-425)
    int add_hf(uint32_t rows, uint32_t cols, float cell, const float* heights, uint32_t& id) {
        if (rows == 0 || cols == 0 || !heights) return AVBD_ERR_INVALID_ARG;
        if (!std::isfinite(cell) || !(cell > 0.0f)) return AVBD_ERR_INVALID_ARG;
        HField<T> f;
        f.rows = rows;
        f.cols = cols;
        f.cell = T(cell);
        T lo = std::numeric_limits<T>::infinity(), hi = -lo;
        for (size_t i = 0; i < (size_t)rows * cols; i++) {
            if (!std::isfinite(heights[i])) return AVBD_ERR_NONFINITE;
            f.h.push_back(T(heights[i]));
            lo = fmn(lo, f.h.back());  // height_range (shape.rs:1571-1583)
            hi = fmx(hi, f.h.back());
        }
        f.y_min = lo;
        f.y_max = hi;
        id = (uint32_t)hfs.size();
        hfs.push_back(std::move(f));
        return AVBD_OK;
    }
    // TriMesh::build_bvh / split (shape.rs:1793-1890): median splits of the
    // longest axis over a stable centroid sort, leaves of up to 4 triangles.
    static uint32_t bvh_split(const std::vector<std::pair<V3<T>, V3<T>>>& bounds, const std::vector<V3<T>>& cent,
                              uint32_t* order, size_t n, uint32_t base, std::vector<BNode<T>>& nodes) {
        V3<T> lo{std::numeric_limits<T>::infinity(), std::numeric_limits<T>::infinity(),
                 std::numeric_limits<T>::infinity()};
        V3<T> hi = -lo;
        for (size_t i = 0; i < n; i++) {
            const auto& bb = bounds[order[i]];
            lo = {fmn(lo.x, bb.first.x), fmn(lo.y, bb.first.y), fmn(lo.z, bb.first.z)};
            hi = {fmx(hi.x, bb.second.x), fmx(hi.y, bb.second.y), fmx(hi.z, bb.second.z)};
        }
        const uint32_t here = (uint32_t)nodes.size();
        nodes.push_back(BNode<T>{lo, hi, true, 0u, 0u});
        if (n <= 4) {
            nodes[here].a = base;
            nodes[here].b = (uint32_t)n;
            return here;
        }
        const V3<T> e = hi - lo;
        const int axis = (e.x >= e.y && e.x >= e.z) ? 0 : (e.y >= e.z ? 1 : 2);
        std::stable_sort(order, order + n, [&](uint32_t x, uint32_t y) { return cent[x][axis] < cent[y][axis]; });
        const size_t mid = n / 2;
        if (cent[order[0]][axis] == cent[order[n - 1]][axis]) {  // all equal: a leaf
            nodes[here].a = base;
            nodes[here].b = (uint32_t)n;
            return here;
        }
        const uint32_t left = bvh_split(bounds, cent, order, mid, base, nodes);
        const uint32_t right = bvh_split(bounds, cent, order + mid, n - mid, base + (uint32_t)mid, nodes);
        nodes[here].leaf = false;
        nodes[here].a = left;
        nodes[here].b = right;
        return here;
    }
    // TriMesh::from_indexed / from_triangles (shape.rs:1646-1772)
    int add_mesh(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t& id) {
        if ((nv && !verts) || (nt && !idx)) return AVBD_ERR_INVALID_ARG;
        std::vector<V3<T>> vs(nv);
        for (uint32_t i = 0; i < nv; i++) {
            for (int k = 0; k < 3; k++)
                if (!std::isfinite(verts[3 * i + k])) return AVBD_ERR_NONFINITE;
            vs[i] = {T(verts[3 * i]), T(verts[3 * i + 1]), T(verts[3 * i + 2])};
        }
        TMesh<T> m;
        const T inf = std::numeric_limits<T>::infinity();
        m.min_feature = inf;
        for (uint32_t t = 0; t < nt; t++) {
            for (int k = 0; k < 3; k++)
                if (idx[3 * t + k] >= nv) return AVBD_ERR_INVALID_ARG;
            const V3<T> v[3] = {vs[idx[3 * t]], vs[idx[3 * t + 1]], vs[idx[3 * t + 2]]};
            if (len2(cross(v[1] - v[0], v[2] - v[0])) < C<T>(K::DEGENERATE_LEN2)) continue;  // a sliver
            const V3<T> ends[3][2] = {{v[0], v[1]}, {v[1], v[2]}, {v[2], v[0]}};
            for (const auto& e : ends) m.min_feature = fmn(m.min_feature, len(e[1] - e[0]));
            for (const V3<T>& p : v) m.bound = fmx(m.bound, len(p));
            const V3<T> c = (v[0] + v[1] + v[2]) / T(3);
            m.cent.push_back(c);
            // ConvexHull::from_vertices welds points closer than 1e-6
            // (shape.rs:1304-1325); a triangle that welds below three
            // points is refused here
            Hull<T> h;
            for (const V3<T>& p : v) {
                const V3<T> q = p - c;
                bool near = false;
                for (const V3<T>& w : h.verts) near = near || len2(w - q) < C<T>(1e-6f) * C<T>(1e-6f);
                if (!near) h.verts.push_back(q);
            }
            if (h.verts.size() != 3) return AVBD_ERR_INVALID_ARG;
            h.faces = {0u, 1u, 2u, 0u, 2u, 1u};  // both windings
            hull_measures(h);
            m.tris.push_back(std::move(h));
        }
        if (m.tris.empty()) m.min_feature = T(0);
        std::vector<std::pair<V3<T>, V3<T>>> bounds;
        for (size_t t = 0; t < m.tris.size(); t++) {
            V3<T> lo{inf, inf, inf}, hi = -lo;
            for (const V3<T>& q : m.tris[t].verts) {
                const V3<T> w = q + m.cent[t];
                lo = {fmn(lo.x, w.x), fmn(lo.y, w.y), fmn(lo.z, w.z)};
                hi = {fmx(hi.x, w.x), fmx(hi.y, w.y), fmx(hi.z, w.z)};
            }
            bounds.push_back({lo, hi});
        }
        m.order.resize(bounds.size());
        for (size_t i = 0; i < m.order.size(); i++) m.order[i] = (uint32_t)i;
        if (!m.order.empty()) bvh_split(bounds, m.cent, m.order.data(), m.order.size(), 0u, m.nodes);
        if (m.nodes.empty()) m.nodes.push_back(BNode<T>{VZERO<T>(), VZERO<T>(), true, 0u, 0u});
        id = (uint32_t)meshes.size();
        meshes.push_back(std::move(m));
        return AVBD_OK;
    }
    // rows.rs:253-292 and :373-403 for one part of a rounded or compound shape
    T part_bound(const Part<T>& p) const {
        T r;
        switch (p.shape) {
            case AVBD_SHAPE_SPHERE: r = p.sp.x; break;
            case AVBD_SHAPE_BOX: r = len(p.sp); break;
            case AVBD_SHAPE_CAPSULE: r = p.sp.y + p.sp.x; break;
            case AVBD_SHAPE_HULL: r = p.hull ? p.hull->bound : T(0); break;
            default: r = std::sqrt(p.sp.x * p.sp.x + p.sp.y * p.sp.y);  // cylinder, cone
        }
        return p.radius > T(0) ? r + fmx(p.radius, T(0)) : r;
    }
    T part_min_dim(const Part<T>& p) const {
        T m;
        switch (p.shape) {
            case AVBD_SHAPE_SPHERE: m = p.sp.x; break;
            case AVBD_SHAPE_BOX: m = min_element(p.sp); break;
            case AVBD_SHAPE_CAPSULE: m = p.sp.x; break;
            case AVBD_SHAPE_CYLINDER: m = fmn(p.sp.x, p.sp.y); break;
            case AVBD_SHAPE_CONE: m = C<T>(K::HALF) * fmn(p.sp.x, p.sp.y); break;
            default: m = C<T>(K::HALF) * (p.hull ? p.hull->min_ext : T(0));  // hull
        }
        return p.radius > T(0) ? fmn(m, fmx(p.radius, T(0)) * T(2)) : m;
    }
    // Shape::try_round / try_compound (shape.rs:556-575) over primitive parts
    int add_ext(bool compound, const AvbdShapePart* parts, uint32_t n, const float* unit_inertia, uint32_t& id) {
        if (!parts || !unit_inertia || n == 0 || (!compound && n != 1)) return AVBD_ERR_INVALID_ARG;
        ExtShape<T> e;
        e.compound = compound;
        for (uint32_t i = 0; i < n; i++) {
            const AvbdShapePart& q = parts[i];
            if (q.shape > AVBD_SHAPE_HULL || q.shape == AVBD_SHAPE_HALFSPACE) return AVBD_ERR_UNSUPPORTED;
            if (!compound && !(std::isfinite(q.border_radius) && q.border_radius > 0.0f)) return AVBD_ERR_INVALID_ARG;
            if (!std::isfinite(q.border_radius) || q.border_radius < 0.0f) return AVBD_ERR_INVALID_ARG;
            Part<T> p;
            p.shape = q.shape;
            p.sp = {T(q.params[0]), T(q.params[1]), T(q.params[2])};
            p.radius = T(q.border_radius);
            p.pos = {T(q.position[0]), T(q.position[1]), T(q.position[2])};
            p.rot = {T(q.orientation[0]), T(q.orientation[1]), T(q.orientation[2]), T(q.orientation[3])};
            p.hull = nullptr;
            if (q.shape == AVBD_SHAPE_HULL) {
                double hid = (double)q.params[0];
                if (!(hid >= 0.0 && hid < (double)hulls.size())) return AVBD_ERR_INVALID_ARG;
                p.hull = &hulls[(size_t)hid];
            }
            e.parts.push_back(p);
        }
        e.unit_inertia = {T(unit_inertia[0]), T(unit_inertia[1]), T(unit_inertia[2])};
        // rows.rs:279-290, :393-400
        if (compound) {
            e.bound = T(0);
            e.min_dim = std::numeric_limits<T>::infinity();
            for (const Part<T>& p : e.parts) {
                e.bound = fmx(e.bound, part_bound(p) + len(p.pos));
                e.min_dim = fmn(e.min_dim, part_min_dim(p));
            }
        } else {
            e.bound = part_bound(e.parts[0]);
            e.min_dim = part_min_dim(e.parts[0]);
        }
        id = (uint32_t)exts.size();
        exts.push_back(std::move(e));
        return AVBD_OK;
    }

    // ---- joints / sleep (avbd/sleep.rs) ----
    // ---- gears (joints_ext.rs:34-160) ----
    // A revolute joint's twist or a prismatic joint's slide from its assembly
    // reference (joints_ext.rs:37-51).
    T joint_coordinate(const Joint<T>& r) const {
        const Body<T>& a = bodies[r.a];
        const Body<T>& b = bodies[r.b];
        if (r.kind == AVBD_JOINT_REVOLUTE) return hinge_twist(a.rot, b.rot, r.ax_a) - r.ref_val;
        V3<T> wa = normalize_or(qrot(a.rot, r.ax_a), VZ<T>());
        V3<T> pa = a.pos + qrot(a.rot, r.la);
        V3<T> pb = b.pos + qrot(b.rot, r.lb);
        return dot(pb - pa, wa) - r.ref_val;
    }
    // Once per step: the coupled joints' raw coordinates, and the continuous
    // ones unwrapped across turns for hinges (joints_ext.rs:55-118).
    void update_gear_mem() {
        for (Joint<T>& g : joints) {
            if (g.kind != AVBD_JOINT_GEAR) continue;
            T raw[2];
            bool ang[2];
            for (int k = 0; k < 2; k++) {
                const Joint<T>& r = joints[g.gb[k]];
                raw[k] = joint_coordinate(r);
                ang[k] = r.kind == AVBD_JOINT_REVOLUTE;
            }
            for (int k = 0; k < 2; k++) {
                T cont = g.gmem_set && ang[k] ? g.gcont[k] + wrap_pi(raw[k] - g.graw[k]) : raw[k];
                g.graw[k] = raw[k];
                g.gcont[k] = cont;
            }
            g.gmem_set = true;
        }
    }
    // The live sides of a gear (joints_ext.rs:120-160).
    void gear_sides(const Joint<T>& g, GearSide<T> sd[2]) const {
        for (int k = 0; k < 2; k++) {
            const Joint<T>& r = joints[g.gb[k]];
            const Body<T>& ba = bodies[r.a];
            const Body<T>& bb = bodies[r.b];
            T raw = joint_coordinate(r);
            GearSide<T>& s = sd[k];
            s.a = r.a;
            s.b = r.b;
            s.angular = r.kind == AVBD_JOINT_REVOLUTE;
            s.axis = normalize_or(qrot(ba.rot, r.ax_a), VZ<T>());
            s.ra = s.angular ? VZERO<T>() : qrot(ba.rot, r.la);
            s.rb = s.angular ? VZERO<T>() : qrot(bb.rot, r.lb);
            s.coord = g.gmem_set && s.angular ? g.gcont[k] + wrap_pi(raw - g.graw[k]) : raw;
        }
    }
    T gear_error(const Joint<T>& g) const {  // C = coord_a + ratio coord_b - constant
        GearSide<T> sd[2];
        gear_sides(g, sd);
        return sd[0].coord + g.gratio * sd[1].coord - g.ref_val;
    }
    // The bodies a joint holds (sleep.rs:9-16): a gear's are its coupled
    // joints' bodies.
    void joint_members(const Joint<T>& j, uint32_t m[4]) const {
        if (j.kind == AVBD_JOINT_GEAR) {
            const Joint<T>& x = joints[j.gb[0]];
            const Joint<T>& y = joints[j.gb[1]];
            m[0] = x.a; m[1] = x.b; m[2] = y.a; m[3] = y.b;
        } else {
            m[0] = j.a; m[1] = j.b; m[2] = j.a; m[3] = j.b;
        }
    }

    T joint_rest_error(const Joint<T>& j) const {  // sleep.rs:30-105
        if (j.kind == AVBD_JOINT_GEAR) return std::fabs(gear_error(j));
        const Body<T>& a = bodies[j.a];
        const Body<T>& b = bodies[j.b];
        V3<T> delta = (b.pos + qrot(b.rot, j.lb)) - (a.pos + qrot(a.rot, j.la));
        V3<T> axis = qrot(a.rot, j.ax_a);
        switch (j.kind) {
            case AVBD_JOINT_BALL: return len(delta);
            case AVBD_JOINT_REVOLUTE: return fmx(len(delta), len(axis - qrot(b.rot, j.ax_b)));
            case AVBD_JOINT_FIXED:
            case AVBD_JOINT_MOTOR:  // a free motor: the assembly deviation (sleep.rs:76-82)
                return fmx(len(delta - qrot(a.rot, j.dref)), len(quat_diff_vec(qmul(conj(a.rot), b.rot), j.q_ref)));
            case AVBD_JOINT_DISTANCE:
            case AVBD_JOINT_SPRING: return std::fabs(len(delta) - j.ref_val);  // a spring: about its rest
            case AVBD_JOINT_ROPE: return fmx(len(delta) - j.ref_val, T(0));
            case AVBD_JOINT_PRISMATIC:
            case AVBD_JOINT_WHEEL: {
                V3<T> perp = delta - axis * dot(delta, axis);
                T e = len(perp);
                if (j.has_lim) {
                    T value = dot(delta, axis) - j.ref_val;
                    e = fmx(e, fmx(j.lo - value, value - j.hi));
                }
                if (j.kind == AVBD_JOINT_PRISMATIC) return fmx(e, len(axis - qrot(b.rot, j.ax_b)));
                e = fmx(e, len(qrot(a.rot, j.bx_a) - qrot(b.rot, j.bx_b)));
                if (j.susp_hz <= T(0)) e = fmx(e, std::fabs(dot(delta, axis) - j.ref_val));
                return e;
            }
            default: {  // sixdof (sleep.rs:86-103)
                V3<T> lin = qrot(conj(a.rot), delta) - j.dref;
                V3<T> ang = quat_diff_vec(qmul(conj(a.rot), b.rot), j.q_ref);
                T e = T(0);
                for (int i = 0; i < 3; i++) {
                    T vals[2] = {lin[i], ang[i]};
                    uint32_t cfg[2] = {j.six_cfg[i], j.six_cfg[3 + i]};
                    T los[2] = {j.six_min[i], j.six_min[3 + i]}, his[2] = {j.six_max[i], j.six_max[3 + i]};
                    for (int k = 0; k < 2; k++) {
                        T r = T(0);
                        if (cfg[k] == AVBD_AXIS_LOCKED) r = std::fabs(vals[k]);
                        else if (cfg[k] == AVBD_AXIS_LIMITED) r = fmx(fmx(los[k] - vals[k], vals[k] - his[k]), T(0));
                        e = fmx(e, r);
                    }
                }
                return e;
            }
        }
    }
    // joints_ext.rs:423-437: I_w^-1 wa of a solvable body, zero otherwise
    V3<T> ang_inv_wa(uint32_t h, V3<T> wa) const {
        if (!solvable(h)) return VZERO<T>();
        const Body<T>& b = bodies[h];
        T iw[3][3], inv[3][3];
        world_inertia(b.inertia, b.rot, iw);
        V3<T> dg{fmx(b.inertia.x, T(0)), fmx(b.inertia.y, T(0)), fmx(b.inertia.z, T(0))};
        inverse_symmetric(iw, dg, inv);
        return mat3_vec(inv, wa);
    }
    T eff_inv_mass(const Body<T>& b) const { return b.type == AVBD_BODY_DYNAMIC ? b.inv_mass : T(0); }  // rows.rs:406-412
    bool limit_violated(const Joint<T>& j) const {  // joints_ext.rs:441-462
        if (!j.has_lim) return false;
        const Body<T>& a = bodies[j.a];
        const Body<T>& b = bodies[j.b];
        if (j.kind == AVBD_JOINT_REVOLUTE) {
            T angle = wrap_pi(hinge_twist(a.rot, b.rot, j.ax_a) - j.ref_val);
            return limit_state(angle, j.lo, j.hi, C<T>(K::LIMIT_SLOP_ANG)) >= 0;
        }
        if (j.kind == AVBD_JOINT_PRISMATIC) {
            V3<T> wa = normalize_or(qrot(a.rot, j.ax_a), VZ<T>());
            V3<T> pa = a.pos + qrot(a.rot, j.la), pb = b.pos + qrot(b.rot, j.lb);
            return limit_state(dot(pb - pa, wa) - j.ref_val, j.lo, j.hi, C<T>(K::LIMIT_SLOP_LIN)) >= 0;
        }
        return false;
    }
    // JointMotor::velocity_impulse (joint.rs:1172-1177) with the spec motor's
    // velocity drive: the deadbeat rate correction, clamped to the budget
    T velocity_impulse(T rate_error, T inv_eff_mass, T max_force) const {
        if (!(dt > T(0)) || max_force <= T(0) || inv_eff_mass <= T(0)) return T(0);
        return fclamp(rate_error / inv_eff_mass, -max_force * dt, max_force * dt);
    }
    // motor_impulse (joints_ext.rs:237-383): revolute and prismatic velocity
    // motors, before the warm start, paused while a limit is violated
    // free_motor_impulse (joints_ext.rs:384-420): per world axis, the
    // deadbeat linear then angular drive of B relative to A
    void free_motor_impulse(Joint<T>& j) {
        Body<T>& a = bodies[j.a];
        Body<T>& b = bodies[j.b];
        const V3<T> axes[3] = {VX<T>(), VY<T>(), VZ<T>()};
        for (const V3<T>& axis : axes) {
            T v = dot(b.vel - a.vel, axis);
            T ka = eff_inv_mass(a), kb = eff_inv_mass(b);
            T dj = velocity_impulse(dot(j.mot_lin, axis) - v, ka + kb, j.mot_force);
            if (dj != T(0)) {
                if (solvable(j.a)) a.vel = a.vel + axis * (-dj * ka);
                if (solvable(j.b)) b.vel = b.vel + axis * (dj * kb);
            }
            T w = dot(b.angvel - a.angvel, axis);
            V3<T> ia = ang_inv_wa(j.a, axis), ib = ang_inv_wa(j.b, axis);
            T k = dot(ia, axis) + dot(ib, axis);
            T dw = velocity_impulse(dot(j.mot_ang, axis) - w, k, j.mot_torque);
            if (dw != T(0)) {
                if (solvable(j.a)) a.angvel = a.angvel + (-dw) * ia;
                if (solvable(j.b)) b.angvel = b.angvel + dw * ib;
            }
        }
    }
    void motor_impulse() {
        for (Joint<T>& j : joints) {
            if (j.kind == AVBD_JOINT_MOTOR) {  // free motors carry their drive inline
                free_motor_impulse(j);
                continue;
            }
            if (!j.has_mot || j.mot_max <= T(0) || limit_violated(j)) continue;
            Body<T>& a = bodies[j.a];
            Body<T>& b = bodies[j.b];
            V3<T> wa = normalize_or(qrot(a.rot, j.ax_a), VZ<T>());
            if (j.kind == AVBD_JOINT_REVOLUTE) {
                T w = dot(b.angvel - a.angvel, wa);
                V3<T> ia = ang_inv_wa(j.a, wa), ib = ang_inv_wa(j.b, wa);
                T k = dot(ia, wa) + dot(ib, wa);
                if (k < C<T>(K::MIN_EFFECTIVE_MASS)) continue;
                T dj = velocity_impulse(j.mot_speed - w, k, j.mot_max);
                if (solvable(j.a)) a.angvel = a.angvel + (-dj) * ia;
                if (solvable(j.b)) b.angvel = b.angvel + dj * ib;
            } else if (j.kind == AVBD_JOINT_PRISMATIC) {
                T v = dot(b.vel - a.vel, wa);
                T ka = eff_inv_mass(a), kb = eff_inv_mass(b);
                T k = ka + kb;
                if (k < C<T>(K::MIN_EFFECTIVE_MASS)) continue;
                T dj = velocity_impulse(j.mot_speed - v, k, j.mot_max);
                if (solvable(j.a)) a.vel = a.vel + (-dj) * ka * wa;
                if (solvable(j.b)) b.vel = b.vel + dj * kb * wa;
            } else if (j.kind == AVBD_JOINT_WHEEL) {  // spin about the axle (joints_ext.rs:337-371)
                V3<T> xa = normalize_or(qrot(a.rot, j.bx_a), VZ<T>());
                T w = dot(b.angvel - a.angvel, xa);
                V3<T> ia = ang_inv_wa(j.a, xa), ib = ang_inv_wa(j.b, xa);
                T k = dot(ia, xa) + dot(ib, xa);
                if (k < C<T>(K::MIN_EFFECTIVE_MASS)) continue;
                T dj = velocity_impulse(j.mot_speed - w, k, j.mot_max);
                if (solvable(j.a)) a.angvel = a.angvel + (-dj) * ia;
                if (solvable(j.b)) b.angvel = b.angvel + dj * ib;
            }
        }
    }
    // rope_impulse (joints_ext.rs:173-236): a stretched rope's separating
    // velocity removed through the pair's effective mass
    void rope_impulse() {
        for (Joint<T>& j : joints) {
            if (j.kind != AVBD_JOINT_ROPE) continue;
            Body<T>& a = bodies[j.a];
            Body<T>& b = bodies[j.b];
            V3<T> pa = a.pos + qrot(a.rot, j.la), pb = b.pos + qrot(b.rot, j.lb);
            V3<T> delta = pb - pa;
            T ln = len(delta);
            if (ln <= j.ref_val) continue;
            V3<T> nn = delta / ln;
            V3<T> ra = pa - a.pos, rb = pb - b.pos;
            T ka = eff_inv_mass(a), kb = eff_inv_mass(b);
            V3<T> ta = cross(ra, nn), tb = cross(rb, nn);
            T k = ka + kb + dot(ang_inv_wa(j.a, ta), ta) + dot(ang_inv_wa(j.b, tb), tb);
            if (k < C<T>(K::MIN_EFFECTIVE_MASS)) continue;
            V3<T> va = a.vel + cross(a.angvel, ra);
            V3<T> vb = b.vel + cross(b.angvel, rb);
            T vsep = dot(vb - va, nn);
            if (vsep <= T(0)) continue;
            T dj = -vsep / k;
            if (solvable(j.a)) {
                V3<T> ia = ang_inv_wa(j.a, ta);
                a.vel = a.vel - nn * (dj * ka);
                a.angvel = a.angvel - ia * dj;
            }
            if (solvable(j.b)) {
                V3<T> ib = ang_inv_wa(j.b, tb);
                b.vel = b.vel + nn * (dj * kb);
                b.angvel = b.angvel + ib * dj;
            }
        }
    }
    bool joint_driven(const Joint<T>& j) const {  // sleep.rs:18-28
        if (j.has_mot && j.mot_speed != T(0) && j.mot_max > T(0)) return true;
        // JointMotor::keeps_awake (joint.rs:1116-1126) of a spring
        if (j.kind == AVBD_JOINT_SPRING && j.spr_max > T(0) &&
            (j.spr_kind == AVBD_MOTOR_VELOCITY ? j.spr_vel != T(0) : (j.spr_k > T(0) || j.spr_vel != T(0))))
            return true;
        // MotorDrive::keeps_awake (joint.rs:474-477)
        if (j.kind == AVBD_JOINT_MOTOR && ((j.mot_force > T(0) && (j.mot_lin.x != T(0) || j.mot_lin.y != T(0) ||
                                                                   j.mot_lin.z != T(0))) ||
                                          (j.mot_torque > T(0) && (j.mot_ang.x != T(0) || j.mot_ang.y != T(0) ||
                                                                   j.mot_ang.z != T(0)))))
            return true;
        uint32_t m[4];
        joint_members(j, m);
        for (uint32_t h : m) {
            const Body<T>& b = bodies[h];
            if (b.type != AVBD_BODY_DYNAMIC && (b.pos != prev_pos[h] || b.rot != prev_rot[h])) return true;
        }
        return false;
    }
    void propagate_joint_flags(std::vector<uint8_t>& flags, uint8_t value) const {
        for (;;) {
            bool changed = false;
            for (const Joint<T>& j : joints) {
                uint32_t mem[4];
                joint_members(j, mem);
                bool any = false;
                for (uint32_t h : mem)
                    if (bodies[h].type == AVBD_BODY_DYNAMIC && flags[h] == value) any = true;
                if (any)
                    for (uint32_t h : mem)
                        if (bodies[h].type == AVBD_BODY_DYNAMIC && flags[h] != value) { flags[h] = value; changed = true; }
            }
            if (!changed) break;
        }
    }
    void wake_joint_motion() {
        size_t n = bodies.size();
        std::vector<uint8_t> awake(n);
        for (size_t h = 0; h < n; h++) {
            const Body<T>& b = bodies[h];
            awake[h] = b.type == AVBD_BODY_DYNAMIC &&
                       (!asleep[h] || b.vel != VZERO<T>() || b.angvel != VZERO<T>() || b.torque != VZERO<T>() ||
                        b.pos != prev_pos[h] || b.rot != prev_rot[h]);
        }
        for (const Joint<T>& j : joints) {
            if (joint_driven(j) || joint_rest_error(j) > C<T>(K::JOINT_REST_ERROR)) {
                uint32_t mem[4];
                joint_members(j, mem);
                for (uint32_t h : mem)
                    if (bodies[h].type == AVBD_BODY_DYNAMIC) awake[h] = 1;
            }
        }
        propagate_joint_flags(awake, 1);
        for (size_t h = 0; h < n; h++)
            if (awake[h] && asleep[h]) wake_body((uint32_t)h);
    }
    std::vector<uint8_t> joint_sleep_ready() const {
        std::vector<uint8_t> ready(bodies.size(), 1);
        for (const Joint<T>& j : joints)
            if (joint_driven(j) || joint_rest_error(j) > C<T>(K::JOINT_REST_ERROR)) {
                uint32_t mem[4];
                joint_members(j, mem);
                for (uint32_t h : mem) ready[h] = 0;
            }
        propagate_joint_flags(ready, 0);
        return ready;
    }

    // ---- pair discovery (avbd/rows.rs:432-756) ----
    struct Discovered {
        uint32_t ia, ib;
        bool trigger, exists;
        V3<T> normal;
        T mu[2];
        T sgn;
        std::vector<std::pair<V3<T>, V3<T>>> fresh;
        bool wake_vote;
    };
    // The reference scans the pair vector (rows.rs:546, :811).  The Coloured
    // schedule keeps the vector in (a, b) order, so there (the checker's
    // mode, not the timed reference order) a binary search finds the same
    // pair; pairs_sorted is set at the start of each discovery.
    bool pairs_sorted = false;
    const Pair<T>* find_pair(uint32_t ia, uint32_t ib) const {
        if (pairs_sorted) {
            size_t lo = 0, hi = pairs.size();
            while (lo < hi) {
                size_t m = (lo + hi) / 2;
                const Pair<T>& p = pairs[m];
                if (p.a < ia || (p.a == ia && p.b < ib)) lo = m + 1;
                else hi = m;
            }
            return lo < pairs.size() && pairs[lo].a == ia && pairs[lo].b == ib ? &pairs[lo] : nullptr;
        }
        for (const Pair<T>& p : pairs)
            if (p.a == ia && p.b == ib) return &p;
        return nullptr;
    }
    // rows.rs:434-474: joined bodies do not collide, except through weld-like
    // Fixed and SixDof joints (their contact is structural)
    static bool no_collide_kind(uint32_t k) {
        return k == AVBD_JOINT_BALL || k == AVBD_JOINT_REVOLUTE || k == AVBD_JOINT_PRISMATIC ||
               k == AVBD_JOINT_DISTANCE || k == AVBD_JOINT_ROPE || k == AVBD_JOINT_MOTOR || k == AVBD_JOINT_SPRING ||
               k == AVBD_JOINT_WHEEL;
    }

    bool discover_pair(uint32_t ia, uint32_t ib, Discovered& out) const {
        const Body<T>& a = bodies[ia];
        const Body<T>& b = bodies[ib];
        if (!pair_allowed(a, b)) return false;
        if (!a.trigger() && !b.trigger()) {
            for (const Joint<T>& j : joints)
                if (no_collide_kind(j.kind) && ((j.a == ia && j.b == ib) || (j.a == ib && j.b == ia))) return false;
        }
        T ra = bound_radius(a), rb = bound_radius(b);
        if (len(a.pos - b.pos) > ra + rb + C<T>(K::GEN_MARGIN)) return false;
        Dist<T> d = shape_distance_any(sref(a), sref(b));
        T sgn = (a.shape == AVBD_SHAPE_BOX && b.shape == AVBD_SHAPE_BOX)
                    ? box_box_signed_gap(a.pos, a.rot, a.sp, b.pos, b.rot, b.sp)
                    : d.dist;
        out.ia = ia; out.ib = ib;
        out.fresh.clear();
        if (a.trigger() || b.trigger()) {
            out.trigger = true; out.exists = false; out.normal = VY<T>(); out.mu[0] = out.mu[1] = T(0);
            out.sgn = sgn; out.wake_vote = false;
            return true;
        }
        out.trigger = false;
        const Pair<T>* stored = find_pair(ia, ib);
        // orient_contact_normal (rows.rs:303-333)
        V3<T> normal;
        if (a.shape == AVBD_SHAPE_HALFSPACE) normal = -qrot(a.rot, a.sp);
        else if (b.shape == AVBD_SHAPE_HALFSPACE) normal = qrot(b.rot, b.sp);
        else {
            V3<T> nm = d.pa - d.pb;
            if (d.dist < T(0)) nm = -nm;
            if (len2(nm) < C<T>(K::AXIS_REST_LEN2)) nm = a.pos - b.pos;
            nm = normalize_or(nm, VY<T>());
            if (stored) {
                if (dot(nm, stored->n) < T(0)) nm = -nm;
            } else if (dot(nm, a.pos - b.pos) < T(0)) {
                nm = -nm;
            }
            normal = nm;
        }
        bool exists = stored != nullptr;
        T approach = fmx(dot(b.vel - a.vel, normal), T(0));
        T reach = C<T>(K::GEN_MARGIN) + approach * dt;
        if (sgn > reach && !exists) return false;
        bool separated = sgn > reach;
        T mu = fmx(a.friction, b.friction);  // friction_frame, isotropic bodies
        out.mu[0] = fmx(mu, T(0));
        out.mu[1] = fmx(mu, T(0));
        T patch = fmn(ra, rb) + C<T>(K::MARGIN);
        V3<T> pp = (d.pa + d.pb) * C<T>(K::HALF);
        V3<T> pa_c = a.pos - normal * dot(a.pos - pp, normal);
        V3<T> pb_c = b.pos - normal * dot(b.pos - pp, normal);
        auto plane = [&](const Body<T>& body, V3<T> witness, T sign) -> T {
            if (body.shape == AVBD_SHAPE_BOX) {
                T extent = dot(vabs(qrot(conj(body.rot), normal)), body.sp);
                return dot(normal, body.pos) - sign * extent;
            }
            return dot(normal, witness);
        };
        T plane_a = plane(a, d.pa, T(1));
        T plane_b = plane(b, d.pb, T(-1));
        auto& fresh = out.fresh;
        auto dup = [&](V3<T> ral, V3<T> rbl) {
            for (auto& e : fresh)
                if (len(e.first - ral) < C<T>(K::POINT_MATCH_DIST) && len(e.second - rbl) < C<T>(K::POINT_MATCH_DIST))
                    return true;
            return false;
        };
        Qt<T> inv_a = conj(a.rot), inv_b = conj(b.rot);
        if (!separated) {
            struct Side { uint32_t h; V3<T> witness; T sign; V3<T> pc; };
            Side sides[2] = {{ia, d.pa, T(1), pa_c}, {ib, d.pb, T(-1), pb_c}};
            for (const Side& sd : sides) {
                const Body<T>& body = bodies[sd.h];
                if (body.shape != AVBD_SHAPE_BOX) continue;
                bool brk = false;
                for (int ix = 0; ix < 2 && !brk; ix++)
                    for (int iy = 0; iy < 2 && !brk; iy++)
                        for (int iz = 0; iz < 2 && !brk; iz++) {
                            T sx = ix ? T(1) : T(-1), sy = iy ? T(1) : T(-1), sz = iz ? T(1) : T(-1);
                            V3<T> corner{sx * body.sp.x, sy * body.sp.y, sz * body.sp.z};
                            V3<T> world = body.pos + qrot(body.rot, corner);
                            T along = dot(world - sd.witness, sd.sign * normal);
                            if (std::fabs(along) > C<T>(K::EXPAND_SLOP) + fmx(-sgn, T(0))) continue;
                            V3<T> rel = world - sd.pc;
                            V3<T> tang = rel - normal * dot(rel, normal);
                            if (len(tang) > patch) continue;
                            if ((int)fresh.size() >= MAX_POINTS) { brk = true; break; }
                            V3<T> pa, pb;
                            if (sd.h == ia) { pa = world; pb = world + normal * (plane_b - dot(normal, world)); }
                            else { pa = world + normal * (plane_a - dot(normal, world)); pb = world; }
                            V3<T> ral = qrot(inv_a, pa - a.pos), rbl = qrot(inv_b, pb - b.pos);
                            if (dup(ral, rbl)) continue;
                            fresh.push_back({ral, rbl});
                        }
            }
        }
        if (!separated && fresh.size() >= 2 && (int)fresh.size() < MAX_POINTS) {
            V3<T> mid = ra < rb ? pa_c : (rb < ra ? pb_c : (pa_c + pb_c) * C<T>(K::HALF));
            V3<T> pa = mid + normal * (plane_a - dot(normal, mid));
            V3<T> pb = mid + normal * (plane_b - dot(normal, mid));
            V3<T> ral = qrot(inv_a, pa - a.pos), rbl = qrot(inv_b, pb - b.pos);
            if (!dup(ral, rbl)) fresh.push_back({ral, rbl});
        }
        if (!separated && fresh.size() < 3) {
            V3<T> ral = qrot(inv_a, d.pa - a.pos), rbl = qrot(inv_b, d.pb - b.pos);
            if (!dup(ral, rbl)) fresh.push_back({ral, rbl});
        }
        bool wake_vote;
        if (exists) {
            wake_vote = (asleep[ia] || asleep[ib]) && sgn < -C<T>(K::WAKE_PENETRATION);
        } else {
            bool impact = sgn < -C<T>(K::WAKE_PENETRATION);
            if (!impact) {
                uint32_t ss[2] = {ia, ib}, oo[2] = {ib, ia};
                T sg[2] = {T(1), T(-1)};
                for (int k = 0; k < 2; k++) {
                    if (asleep[ss[k]]) {
                        T app = dot(bodies[oo[k]].vel - bodies[ss[k]].vel, sg[k] * normal);
                        if (app > C<T>(K::WAKE_IMPACT_SPEED)) { impact = true; break; }
                    }
                }
            }
            wake_vote = impact;
        }
        out.exists = exists; out.normal = normal; out.sgn = sgn; out.wake_vote = wake_vote;
        return true;
    }

    // generate_pairs (rows.rs:767-943)
    void generate_pairs() {
        uint32_t n = (uint32_t)bodies.size();
        pairs_sorted = mode == COLOURED;
        for (size_t k = 1; pairs_sorted && k < pairs.size(); k++)
            pairs_sorted = pairs[k - 1].a < pairs[k].a || (pairs[k - 1].a == pairs[k].a && pairs[k - 1].b < pairs[k].b);
        std::vector<Discovered> disc;
        if (threads > 1 && n > 256) {
            // Parallel over the first index, like the rayon split at rows.rs:769-782;
            // the sort below restores canonical order.
            int nt = threads;
            std::vector<std::vector<Discovered>> parts(nt);
            std::vector<std::thread> th;
            for (int t = 0; t < nt; t++)
                th.emplace_back([&, t]() {
                    Discovered d;
                    for (uint32_t ia = t; ia < n; ia += nt)
                        for (uint32_t ib = ia + 1; ib < n; ib++)
                            if (discover_pair(ia, ib, d)) parts[t].push_back(d);
                });
            for (auto& x : th) x.join();
            for (auto& p : parts)
                for (auto& d : p) disc.push_back(std::move(d));
        } else {
            Discovered d;
            for (uint32_t ia = 0; ia < n; ia++)
                for (uint32_t ib = ia + 1; ib < n; ib++)
                    if (discover_pair(ia, ib, d)) disc.push_back(d);
        }
        std::stable_sort(disc.begin(), disc.end(), [](const Discovered& x, const Discovered& y) {
            return x.ia != y.ia ? x.ia < y.ia : x.ib < y.ib;
        });
        std::vector<std::pair<uint32_t, uint32_t>> wake;
        auto make_points_fresh = [](const Discovered& d) {
            std::vector<Point<T>> pts;
            for (auto& f : d.fresh) {
                Point<T> p{};
                p.ra = f.first; p.rb = f.second;
                for (int k = 0; k < 3; k++) { p.lam[k] = T(0); p.pen[k] = C<T>(K::PENALTY_INIT); p.roll_lam[k] = T(0); }
                p.stuck = true;
                p.matched = -1;
                pts.push_back(p);
            }
            return pts;
        };
        auto merge_points = [&](const Pair<T>& old, const Discovered& d) {
            std::vector<Point<T>> next;
            bool touching = d.sgn <= T(0);
            bool smooth = bodies[d.ia].shape == AVBD_SHAPE_SPHERE || bodies[d.ib].shape == AVBD_SHAPE_SPHERE;
            for (auto& f : d.fresh) {
                int m = -1;
                for (size_t k = 0; k < old.points.size(); k++)
                    if (len(old.points[k].ra - f.first) < C<T>(K::LAMBDA_MATCH_DIST)) { m = (int)k; break; }
                Point<T> p{};
                if (m >= 0) {
                    const Point<T>& o = old.points[m];
                    if (o.stuck && touching && !smooth) { p.ra = o.ra; p.rb = o.rb; p.kept = true; }
                    else { p.ra = f.first; p.rb = f.second; }
                    for (int k = 0; k < 3; k++) { p.lam[k] = o.lam[k]; p.pen[k] = o.pen[k]; p.roll_lam[k] = o.roll_lam[k]; }
                    p.stuck = o.stuck;
                    p.matched = m;
                } else {
                    p.ra = f.first; p.rb = f.second;
                    for (int k = 0; k < 3; k++) { p.lam[k] = T(0); p.pen[k] = C<T>(K::PENALTY_INIT); p.roll_lam[k] = T(0); }
                    p.stuck = true;
                    p.matched = -1;
                }
                next.push_back(p);
            }
            return next;
        };
        // trigger overlaps of this substep (rows.rs:802-807)
        trig_now.clear();
        for (auto& d : disc)
            if (d.trigger && d.sgn <= T(0)) trig_now.insert({d.ia, d.ib});
        if (mode == REFERENCE) {
            std::vector<uint8_t> seen(pairs.size(), 0);
            for (auto& d : disc) {
                if (d.trigger) continue;
                if (d.exists) {
                    size_t idx = 0;
                    bool found = false;
                    for (; idx < pairs.size(); idx++)
                        if (pairs[idx].a == d.ia && pairs[idx].b == d.ib) { found = true; break; }
                    if (!found) continue;
                    seen[idx] = 1;
                    Pair<T>& p = pairs[idx];
                    p.n = d.normal; p.mu[0] = d.mu[0]; p.mu[1] = d.mu[1]; p.gap = d.sgn;
                    if (d.wake_vote) wake.push_back({d.ia, d.ib});
                    p.points = merge_points(p, d);
                } else {
                    seen.push_back(1);
                    if (d.wake_vote) wake.push_back({d.ia, d.ib});
                    Pair<T> p;
                    p.a = d.ia; p.b = d.ib; p.n = d.normal; p.mu[0] = d.mu[0]; p.mu[1] = d.mu[1]; p.gap = d.sgn;
                    p.points = make_points_fresh(d);
                    pairs.push_back(std::move(p));
                }
            }
            for (size_t idx = seen.size(); idx-- > 0;)
                if (!seen[idx]) {
                    pairs[idx] = std::move(pairs.back());
                    pairs.pop_back();
                }
        } else {
            // Coloured schedule: the pair vector is the discovered set in (a, b)
            // order.  Same per-pair merge, no swap_remove reordering.
            std::vector<Pair<T>> next;
            for (auto& d : disc) {
                if (d.trigger) continue;
                Pair<T> p;
                p.a = d.ia; p.b = d.ib; p.n = d.normal; p.mu[0] = d.mu[0]; p.mu[1] = d.mu[1]; p.gap = d.sgn;
                if (d.exists) {
                    const Pair<T>* old = find_pair(d.ia, d.ib);
                    if (!old) continue;
                    p.points = merge_points(*old, d);
                } else {
                    p.points = make_points_fresh(d);
                }
                if (d.wake_vote) wake.push_back({d.ia, d.ib});
                next.push_back(std::move(p));
            }
            pairs = std::move(next);
        }
        for (auto& w : wake) { wake_body(w.first); wake_body(w.second); }
        if (freeze_frames)
            for (auto& p : pairs) {
                if (freeze_bits & 1) p.n = {no_tangent(p.n.x), no_tangent(p.n.y), no_tangent(p.n.z)};
                p.gap = no_tangent(p.gap);
                if (freeze_bits & 8)
                    for (auto& pt : p.points)
                        for (int k = 0; k < 3; k++) { pt.lam[k] = no_tangent(pt.lam[k]); pt.pen[k] = no_tangent(pt.pen[k]); }
                if (freeze_bits & 16)
                    for (auto& pt : p.points)
                        for (int k = 0; k < 3; k++) pt.pen[k] = no_tangent(pt.pen[k]);
                if (freeze_bits & 4)
                for (auto& pt : p.points) {
                    pt.ra = {no_tangent(pt.ra.x), no_tangent(pt.ra.y), no_tangent(pt.ra.z)};
                    pt.rb = {no_tangent(pt.rb.x), no_tangent(pt.rb.y), no_tangent(pt.rb.z)};
                }
                if (freeze_bits & 4)
                    for (auto& pt : p.points) {
                        if (pt.kept) continue;
                        // a capsule's witness anchor rolls with the body: segment
                        // point + s R0^T n (s = -r on side A, +r on side B)
                        const Body<T>& A = bodies[p.a];
                        const Body<T>& B = bodies[p.b];
                        if (B.shape == AVBD_SHAPE_CAPSULE && A.shape != AVBD_SHAPE_BOX) {
                            V3<T> t = qrot(conj(B.rot), p.n) * B.sp.x;
                            pt.rb = {value_with_tangent(pt.rb.x, t.x), value_with_tangent(pt.rb.y, t.y),
                                     value_with_tangent(pt.rb.z, t.z)};
                        }
                        if (A.shape == AVBD_SHAPE_CAPSULE && B.shape != AVBD_SHAPE_BOX) {
                            V3<T> t = qrot(conj(A.rot), p.n) * (-A.sp.x);
                            pt.ra = {value_with_tangent(pt.ra.x, t.x), value_with_tangent(pt.ra.y, t.y),
                                     value_with_tangent(pt.ra.z, t.z)};
                        }
                    }
            }
    }

    // Hinge twist of a joint.  Under frozen frames the angle is held fixed
    // once the hinge axes part by more than 120 degrees (cos^2(swing/2) < 1/4),
    // where the twist stops being defined and its derivative has no bound.
    T twist(Qt<T> qa, Qt<T> qb, V3<T> axis) const {
        T t = hinge_twist(qa, qb, axis);
        if (!freeze_frames) return t;
        Qt<T> q = qmul(conj(qa), qb);
        T s = dot(V3<T>{q.x, q.y, q.z}, axis);
        return s * s + q.w * q.w < T(0.25) ? no_tangent(t) : t;
    }

    // ---- contact rows (rows.rs:947-1060, joints_ext.rs:21-32) ----
    V3<T> lever_a(const Body<T>& a, V3<T> n, const Point<T>& pt) const {
        return a.shape == AVBD_SHAPE_SPHERE ? -n * a.sp.x : qrot(a.rot, pt.ra);
    }
    V3<T> lever_b(const Body<T>& b, V3<T> n, const Point<T>& pt) const {
        return b.shape == AVBD_SHAPE_SPHERE ? n * b.sp.x : qrot(b.rot, pt.rb);
    }
    T gap_c0(const Pair<T>& p, const Point<T>& pt) const {
        const Body<T>& a = bodies[p.a];
        const Body<T>& b = bodies[p.b];
        if (a.shape == AVBD_SHAPE_SPHERE || b.shape == AVBD_SHAPE_SPHERE) {
            if (!freeze_frames) return p.gap + C<T>(K::MARGIN);
            // value from the narrowphase gap, derivative from the witnesses
            // (a sphere's witness is its centre minus radius along the normal)
            V3<T> wa = a.shape == AVBD_SHAPE_SPHERE ? pos0[p.a] - p.n * a.sp.x : pos0[p.a] + qrot(rot0[p.a], pt.ra);
            V3<T> wb = b.shape == AVBD_SHAPE_SPHERE ? pos0[p.b] + p.n * b.sp.x : pos0[p.b] + qrot(rot0[p.b], pt.rb);
            return value_with_tangent(p.gap + C<T>(K::MARGIN), dot(p.n, wa - wb));
        }
        V3<T> pa = pos0[p.a] + qrot(rot0[p.a], pt.ra);
        V3<T> pb = pos0[p.b] + qrot(rot0[p.b], pt.rb);
        return dot(p.n, pa - pb) + C<T>(K::MARGIN);
    }
    T row_c_levers(const Pair<T>& p, V3<T> u, T c0, V3<T> raw, V3<T> rbw) const {
        const Body<T>& a = bodies[p.a];
        const Body<T>& b = bodies[p.b];
        V3<T> da = a.pos - pos0[p.a] + u * dot(cross(raw, u), quat_diff_vec(a.rot, rot0[p.a]));
        V3<T> db = b.pos - pos0[p.b] + u * dot(cross(rbw, u), quat_diff_vec(b.rot, rot0[p.b]));
        return c0 * (T(1) - C<T>(K::ALPHA)) + dot(u, da - db);
    }
    void friction_levers(const Pair<T>& p, const Point<T>& pt, V3<T>& raf, V3<T>& rbf) const {
        const Body<T>& a = bodies[p.a];
        const Body<T>& b = bodies[p.b];
        V3<T> raw = lever_a(a, p.n, pt), rbw = lever_b(b, p.n, pt);
        T sep = dot((a.pos + raw) - (b.pos + rbw), p.n);
        raf = raw - p.n * (sep * C<T>(K::HALF));
        rbf = rbw + p.n * (sep * C<T>(K::HALF));
    }
    static void contact_force(T cn, const T pens[3], const T lam[3], T ct0, T ct1, const T mu[2], T f[3]) {
        T fnc = fmn(pens[0] * cn + lam[0], T(0));
        T fr0 = pens[1] * ct0 + lam[1], fr1 = pens[2] * ct1 + lam[2];
        T b1 = std::fabs(fnc) * mu[0], b2 = std::fabs(fnc) * mu[1];
        if (b1 <= T(0) || b2 <= T(0)) {
            f[0] = fnc;
            f[1] = b1 <= T(0) ? T(0) : fclamp(fr0, -b1, b1);
            f[2] = b2 <= T(0) ? T(0) : fclamp(fr1, -b2, b2);
            return;
        }
        T s = (fr0 / b1) * (fr0 / b1) + (fr1 / b2) * (fr1 / b2);
        T k = s > T(1) ? T(1) / std::sqrt(s) : T(1);
        f[0] = fnc; f[1] = fr0 * k; f[2] = fr1 * k;
    }

    void stamp_contacts_for(uint32_t h, uint32_t pi, T lhs[6][6], T rhs[6]) const {
        const Pair<T>& p = pairs[pi];
        bool is_a = p.a == h;
        T sign = is_a ? T(1) : T(-1);
        const Body<T>& A = bodies[p.a];
        const Body<T>& B = bodies[p.b];
        V3<T> n = p.n;
        for (size_t qi = 0; qi < p.points.size(); qi++) {
            const Point<T>& pt = p.points[qi];
            bool touching = p.gap <= T(0);
            T c0 = touching ? gap_c0(p, pt) : T(0);
            V3<T> rup = lever_a(A, n, pt), rlo = lever_b(B, n, pt);
            T cn = row_c_levers(p, n, c0, rup, rlo);
            V3<T> r_side = is_a ? rup : rlo;
            if (!touching) {
                T approach = fmx(dot(B.vel - A.vel, n), T(0));
                if (p.gap - approach * dt > T(0)) continue;
                if (std::fabs(cn) >= C<T>(K::C_EPS)) {
                    T npts = T(std::max<size_t>(p.points.size(), 1));
                    T ka = eff_inv_mass(A), kb = eff_inv_mass(B);
                    T m_red = ka + kb > C<T>(K::NEAR_ZERO) ? T(1) / (ka + kb) : T(0);
                    if (m_red > T(0)) {
                        T pen_d = fmn(T(2) * m_red / (dt * dt) / npts, C<T>(K::PENALTY_MAX));
                        T f_d = fmn(pen_d * cn, T(0));
                        stamp_row(lhs, rhs, n, pen_d, f_d, r_side, sign);
                    }
                }
                continue;
            }
            V3<T> t1 = tangent_t1(n);
            V3<T> t2 = cross(t1, n);
            V3<T> raf, rbf;
            friction_levers(p, pt, raf, rbf);
            V3<T> r_side_f = is_a ? raf : rbf;
            T ct1 = row_c_levers(p, t1, T(0), raf, rbf);
            T ct2 = row_c_levers(p, t2, T(0), raf, rbf);
            T f[3];
            contact_force(cn, pt.pen, pt.lam, ct1, ct2, p.mu, f);
            V3<T> axes[3] = {n, t1, t2};
            T cvs[3] = {cn, ct1, ct2};
            V3<T> rs[3] = {r_side, r_side_f, r_side_f};
            for (int row = 0; row < 3; row++) {
                if (!row_live(cvs[row], f[row])) continue;
                stamp_row(lhs, rhs, axes[row], pt.pen[row], f[row], rs[row], sign);
            }
            T mu_roll = fmx(A.rolling, B.rolling), mu_spin = fmx(A.torsion, B.torsion);
            if (mu_roll > T(0) || mu_spin > T(0)) {
                V3<T> wrel = quat_diff_vec(A.rot, rot0[p.a]) - quat_diff_vec(B.rot, rot0[p.b]);
                V3<T> rax[3] = {t1, t2, n};
                T murs[3] = {mu_roll, mu_roll, mu_spin};
                for (int li = 0; li < 3; li++) {
                    if (murs[li] <= T(0)) continue;
                    T c = dot(wrel, rax[li]);
                    T cap = murs[li] * std::fabs(f[0]);
                    T fr = fclamp(C<T>(K::ROLL_PEN) * c + pt.roll_lam[li], -cap, cap);
                    V3<T> g = is_a ? rax[li] : -rax[li];
                    T o[3][3];
                    outer(g, g, o);
                    for (int x = 0; x < 3; x++)
                        for (int y = 0; y < 3; y++) lhs[3 + x][3 + y] += C<T>(K::ROLL_PEN) * o[x][y];
                    rhs[3] += fr * g.x; rhs[4] += fr * g.y; rhs[5] += fr * g.z;
                }
            }
        }
    }

    // A gear's rows on body h, one of its coupled joints' bodies
    // (assembly.rs:426-454 slides, :650-682 hinges): the shared force on
    // the position-level row C = coord_a + ratio coord_b - constant, with
    // the slide sides first, then the hinge sides.
    void stamp_gear_for(uint32_t h, const Joint<T>& j, T lhs[6][6], T rhs[6]) const {
        GearSide<T> sd[2];
        gear_sides(j, sd);
        T c = sd[0].coord + j.gratio * sd[1].coord - j.ref_val;
        T f = j.pen_l[0] * c + j.lam_l[0];
        if (!row_live(c, f)) return;
        const T coef[2] = {T(1), j.gratio};
        for (int k = 0; k < 2; k++) {
            const GearSide<T>& side = sd[k];
            if (side.angular || (h != side.a && h != side.b)) continue;
            T lsign = h == side.a ? T(-1) : T(1);
            V3<T> r = h == side.a ? side.ra : side.rb;
            stamp_row(lhs, rhs, side.axis, j.pen_l[0] * coef[k] * coef[k], f * coef[k], r, lsign);
        }
        for (int k = 0; k < 2; k++) {
            const GearSide<T>& side = sd[k];
            if (!side.angular || (h != side.a && h != side.b)) continue;
            V3<T> g = h == side.a ? -side.axis : side.axis;
            stamp_angular(lhs, rhs, g, j.pen_l[0] * coef[k] * coef[k], f * coef[k]);
        }
    }

    void stamp_joint_for(uint32_t h, const Joint<T>& j, T lhs[6][6], T rhs[6]) const {  // assembly.rs:255-881
        if (j.kind == AVBD_JOINT_GEAR) return stamp_gear_for(h, j, lhs, rhs);
        bool is_a = j.a == h;
        T sign = is_a ? T(1) : T(-1);
        T lsign = is_a ? T(-1) : T(1);  // rows measured B minus A flip the gradient
        const Body<T>& a = bodies[j.a];
        const Body<T>& b = bodies[j.b];
        V3<T> pa = a.pos + qrot(a.rot, j.la);
        V3<T> pb = b.pos + qrot(b.rot, j.lb);
        V3<T> pa0 = pos0[j.a] + qrot(rot0[j.a], j.la);
        V3<T> pb0 = pos0[j.b] + qrot(rot0[j.b], j.lb);
        V3<T> live = pa - pb, c0v = pa0 - pb0;
        V3<T> wa = normalize_or(qrot(a.rot, j.ax_a), VZ<T>());
        const bool fixed = j.kind == AVBD_JOINT_FIXED;
        V3<T> r_plain = is_a ? qrot(a.rot, j.la) : qrot(b.rot, j.lb);
        V3<T> fl = VZERO<T>();
        // linear rows (assembly.rs:278-455)
        if (j.kind == AVBD_JOINT_BALL || j.kind == AVBD_JOINT_REVOLUTE || fixed) {
            for (int k = 0; k < 3; k++) {
                V3<T> axis = VZERO<T>();
                axis[k] = T(1);
                V3<T> lv = fixed ? live + qrot(a.rot, j.dref) : live;
                V3<T> iv = fixed ? c0v + qrot(rot0[j.a], j.dref) : c0v;
                T c = lv[k] - C<T>(K::ALPHA) * iv[k];
                T f = j.pen_l[k] * c + j.lam_l[k];
                if (!row_live(c, f)) continue;
                // Ball/Revolute levers add a zero offset (the Fixed weld's dref slot).
                V3<T> r_side = is_a ? qrot(a.rot, j.la + (fixed ? j.dref : VZERO<T>())) : qrot(b.rot, j.lb);
                stamp_row(lhs, rhs, axis, j.pen_l[k], f, r_side, sign);
                fl[k] = f;
            }
        } else if (j.kind == AVBD_JOINT_PRISMATIC) {
            V3<T> u, v;
            tangent_basis(wa, u, v);
            V3<T> axs[2] = {u, v};
            for (int li = 0; li < 2; li++) {
                T c = dot(live - C<T>(K::ALPHA) * c0v, axs[li]);
                T f = j.pen_l[li] * c + j.lam_l[li];
                if (!row_live(c, f)) continue;
                stamp_row(lhs, rhs, axs[li], j.pen_l[li], f, r_plain, sign);
                fl = fl + axs[li] * f;
            }
        } else if (j.kind == AVBD_JOINT_DISTANCE || j.kind == AVBD_JOINT_ROPE) {
            T ln = len(live);
            if (j.kind == AVBD_JOINT_DISTANCE || ln > j.ref_val) {
                V3<T> dir = ln > C<T>(K::NEAR_ZERO) ? live / ln : VY<T>();
                T c = (ln - j.ref_val) - C<T>(K::ALPHA) * (len(c0v) - j.ref_val);
                T f = j.pen_l[0] * c + j.lam_l[0];
                if (row_live(c, f)) {
                    stamp_row(lhs, rhs, dir, j.pen_l[0], f, r_plain, sign);
                    fl = dir * f;
                }
            }
        } else if (j.kind == AVBD_JOINT_WHEEL) {
            // two rows across the suspension axis and the suspension spring
            // along it (assembly.rs:521-581); a zero frequency makes the
            // spring a rigid row on slot 2
            V3<T> u, v;
            tangent_basis(wa, u, v);
            V3<T> axs[2] = {u, v};
            for (int li = 0; li < 2; li++) {
                T c = dot(live - C<T>(K::ALPHA) * c0v, axs[li]);
                T f = j.pen_l[li] * c + j.lam_l[li];
                if (!row_live(c, f)) continue;
                stamp_row(lhs, rhs, axs[li], j.pen_l[li], f, r_plain, sign);
                fl = fl + axs[li] * f;
            }
            T sv = dot(pb - pa, wa) - j.ref_val;
            V3<T> wa0 = normalize_or(qrot(rot0[j.a], j.ax_a), VZ<T>());
            if (j.susp_hz > T(0)) {
                T ka = eff_inv_mass(a), kb = eff_inv_mass(b);
                T m = ka + kb > C<T>(K::NEAR_ZERO) ? T(1) / (ka + kb) : T(0);
                if (m > T(0)) {
                    T omega = C<T>(K::TAU) * j.susp_hz;
                    T stiff = m * omega * omega;
                    T dampc = T(2) * m * j.susp_zeta * omega;
                    T s0 = dot(pb0 - pa0, wa0) - j.ref_val;
                    T f = stiff * sv + dampc * (sv - s0) / dt;
                    stamp_row(lhs, rhs, wa, stiff, f, r_plain, lsign);
                }
            } else {
                T c = sv - C<T>(K::ALPHA) * (dot(pb0 - pa0, wa0) - j.ref_val);
                T f = j.pen_l[2] * c + j.lam_l[2];
                if (row_live(c, f)) stamp_row(lhs, rhs, wa, j.pen_l[2], f, r_plain, lsign);
            }
        } else if (j.kind == AVBD_JOINT_SPRING) {
            // position-level spring about the rest length (assembly.rs:363-425):
            // penalty from the stiffness, damping from the step delta, no dual
            T ln = len(live);
            V3<T> dir = ln > C<T>(K::NEAR_ZERO) ? live / ln : VY<T>();
            T s = ln - j.ref_val;
            T s0 = len(c0v) - j.ref_val;
            T ka = eff_inv_mass(a), kb = eff_inv_mass(b);
            T m = ka + kb > C<T>(K::NEAR_ZERO) ? T(1) / (ka + kb) : T(0);
            if (m > T(0)) {
                T stiff = j.spr_model == AVBD_MODEL_FORCE ? j.spr_k : j.spr_k * m;
                T dampc = j.spr_model == AVBD_MODEL_FORCE ? j.spr_c : j.spr_c * m;
                if (stiff > T(0)) {
                    T f = stiff * s + dampc * (s - s0) / dt;
                    stamp_row(lhs, rhs, dir, stiff, f, r_plain, sign);
                } else if (dampc > T(0)) {  // a pure damper: the viscous row only
                    T pen_v = dampc / dt;
                    T f = dampc * (s - s0) / dt;
                    stamp_row(lhs, rhs, dir, pen_v, f, r_plain, sign);
                }
            }
        } else if (j.kind == AVBD_JOINT_SIXDOF) {
            for (int i = 0; i < 3; i++) {
                V3<T> e = VZERO<T>();
                e[i] = T(1);
                V3<T> dir = normalize_or(qrot(a.rot, e), e);
                if (j.six_cfg[i] == AVBD_AXIS_LOCKED) {
                    V3<T> evec = (pb - pa) - qrot(a.rot, j.dref);
                    T c = dot(evec, dir);
                    T f = j.pen_l[i] * c + j.lam_l[i];
                    if (!row_live(c, f)) continue;
                    stamp_row(lhs, rhs, dir, j.pen_l[i], f, r_plain, lsign);
                } else if (j.six_cfg[i] == AVBD_AXIS_LIMITED) {
                    T sep = dot((pb - pa) - qrot(a.rot, j.dref), dir);
                    int st = warm_limit_state(sep, j.six_min[i], j.six_max[i], C<T>(K::LIMIT_SLOP_LIN), j.sacc[i]);
                    if (st < 0) continue;
                    bool lower = st == 1;
                    V3<T> axis0 = normalize_or(qrot(rot0[j.a], e), e);
                    T initial = dot((pb0 - pa0) - qrot(rot0[j.a], j.dref), axis0);
                    T c = regularized_limit(sep, initial, lower ? j.six_min[i] : j.six_max[i], lower);
                    T f_raw = j.pen_l[i] * c + j.sacc[i];
                    T f = lower ? fmn(f_raw, T(0)) : fmx(f_raw, T(0));
                    if (!row_live(c, f)) continue;
                    stamp_row(lhs, rhs, dir, j.pen_l[i], f, r_plain, lsign);
                }
            }
        }
        {
            // geometric stiffness (rows.rs:69-88, assembly.rs:589-618)
            V3<T> r = is_a ? qrot(a.rot, j.la + (fixed ? j.dref : VZERO<T>())) : -qrot(b.rot, j.lb);
            T hm[3][3] = {};
            T arr[3] = {r.x, r.y, r.z};
            for (int k = 0; k < 3; k++) {
                T g[3][3] = {};
                g[0][0] = -arr[k]; g[1][1] = -arr[k]; g[2][2] = -arr[k];
                g[0][k] += arr[0]; g[1][k] += arr[1]; g[2][k] += arr[2];
                for (int x = 0; x < 3; x++)
                    for (int y = 0; y < 3; y++) hm[x][y] += g[x][y] * fl[k];
            }
            V3<T> hd{len(V3<T>{hm[0][0], hm[1][0], hm[2][0]}), len(V3<T>{hm[0][1], hm[1][1], hm[2][1]}),
                     len(V3<T>{hm[0][2], hm[1][2], hm[2][2]})};
            lhs[3][3] += hd.x; lhs[4][4] += hd.y; lhs[5][5] += hd.z;
        }
        // angular rows (assembly.rs:634-806); a wheel's pair keys on its axle
        if (j.kind == AVBD_JOINT_REVOLUTE || j.kind == AVBD_JOINT_PRISMATIC || j.kind == AVBD_JOINT_WHEEL) {
            const bool wheel = j.kind == AVBD_JOINT_WHEEL;
            const V3<T> hxa = wheel ? j.bx_a : j.ax_a, hxb = wheel ? j.bx_b : j.ax_b;
            V3<T> axa = qrot(a.rot, hxa), axb = qrot(b.rot, hxb);
            V3<T> axa0 = qrot(rot0[j.a], hxa), axb0 = qrot(rot0[j.b], hxb);
            V3<T> t1, t2;
            tangent_basis(axa0, t1, t2);
            V3<T> ts[2] = {t1, t2};
            for (int li = 0; li < 2; li++) {
                V3<T> t = ts[li];
                T c = dot(t, axa - axb) - C<T>(K::ALPHA) * dot(t, axa0 - axb0);
                T f = j.pen_a[li] * c + j.lam_a[li];
                if (!row_live(c, f)) continue;
                V3<T> g = is_a ? cross(axa, t) : -cross(axb, t);
                stamp_angular(lhs, rhs, g, j.pen_a[li], f);
            }
        } else if (j.kind == AVBD_JOINT_SIXDOF) {
            V3<T> diff = quat_diff_vec(qmul(conj(a.rot), b.rot), j.q_ref);
            for (int i = 0; i < 3; i++) {
                V3<T> e = VZERO<T>();
                e[i] = T(1);
                V3<T> dir = normalize_or(qrot(a.rot, e), e);
                V3<T> g = is_a ? -dir : dir;
                if (j.six_cfg[3 + i] == AVBD_AXIS_LOCKED) {
                    T c = dot(diff, e);
                    T f = j.pen_a[i] * c + j.lam_a[i];
                    if (!row_live(c, f)) continue;
                    stamp_angular(lhs, rhs, g, j.pen_a[i], f);
                } else if (j.six_cfg[3 + i] == AVBD_AXIS_LIMITED) {
                    T travel = twist(a.rot, b.rot, e) - quat_twist(j.q_ref, e);
                    int st = warm_limit_state(travel, j.six_min[3 + i], j.six_max[3 + i], C<T>(K::LIMIT_SLOP_ANG),
                                              j.sacc[3 + i]);
                    if (st < 0) continue;
                    bool lower = st == 1;
                    T initial = twist(rot0[j.a], rot0[j.b], e) - quat_twist(j.q_ref, e);
                    T c = regularized_limit(travel, initial, lower ? j.six_min[3 + i] : j.six_max[3 + i], lower);
                    T f_raw = j.pen_a[i] * c + j.sacc[3 + i];
                    T f = lower ? fmn(f_raw, T(0)) : fmx(f_raw, T(0));
                    if (!row_live(c, f)) continue;
                    stamp_angular(lhs, rhs, g, j.pen_a[i], f);
                }
            }
        } else if (fixed) {
            V3<T> diff = quat_diff_vec(qmul(conj(a.rot), b.rot), j.q_ref);
            V3<T> diff0 = quat_diff_vec(qmul(conj(rot0[j.a]), rot0[j.b]), j.q_ref);
            for (int k = 0; k < 3; k++) {
                T c = diff[k] - C<T>(K::ALPHA) * diff0[k];
                T f = j.pen_a[k] * c + j.lam_a[k];
                if (!row_live(c, f)) continue;
                V3<T> e = VZERO<T>();
                e[k] = T(1);
                V3<T> dir = qrot(a.rot, e);
                stamp_angular(lhs, rhs, is_a ? -dir : dir, j.pen_a[k], f);
            }
        }
        // one-sided limit rows (assembly.rs:807-881)
        if (j.has_lim && j.kind == AVBD_JOINT_REVOLUTE) {
            T angle = wrap_pi(twist(a.rot, b.rot, j.ax_a) - j.ref_val);
            int st = warm_limit_state(angle, j.lo, j.hi, C<T>(K::LIMIT_SLOP_ANG), j.acc_lim);
            if (st >= 0) {
                bool lower = st == 1;
                T initial = wrap_pi(twist(rot0[j.a], rot0[j.b], j.ax_a) - j.ref_val);
                T c = regularized_limit(angle, initial, lower ? j.lo : j.hi, lower);
                T f_raw = j.pen_a[2] * c + j.acc_lim;
                T f = lower ? fmn(f_raw, T(0)) : fmx(f_raw, T(0));
                if (row_live(c, f)) stamp_angular(lhs, rhs, is_a ? -wa : wa, j.pen_a[2], f);
            }
        } else if (j.has_lim && j.kind == AVBD_JOINT_PRISMATIC) {
            T sv = dot(pb - pa, wa) - j.ref_val;
            int st = warm_limit_state(sv, j.lo, j.hi, C<T>(K::LIMIT_SLOP_LIN), j.lim_dual);
            if (st >= 0) {
                bool lower = st == 1;
                V3<T> axis0 = normalize_or(qrot(rot0[j.a], j.ax_a), VZ<T>());
                T initial = dot(pb0 - pa0, axis0) - j.ref_val;
                T c = regularized_limit(sv, initial, lower ? j.lo : j.hi, lower);
                T f_raw = j.pen_l[2] * c + j.lim_dual;
                T f = lower ? fmn(f_raw, T(0)) : fmx(f_raw, T(0));
                if (row_live(c, f)) stamp_row(lhs, rhs, wa, j.pen_l[2], f, r_plain, lsign);
            }
        }
    }

    void solve_body(uint32_t h) {  // assembly.rs:73-903
        const Body<T>& bd = bodies[h];
        T dt2 = dt * dt;
        T m_dt2 = T(1) / eff_inv_mass(bd) / dt2;
        T iw[3][3];
        world_inertia(bd.inertia, bd.rot, iw);
        T lhs[6][6] = {};
        T rhs[6] = {};
        for (int i = 0; i < 3; i++) lhs[i][i] = m_dt2;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) lhs[3 + a][3 + b] = iw[a][b] / dt2;
        V3<T> rl = m_dt2 * (bd.pos - inertial[h]);
        rhs[0] = rl.x; rhs[1] = rl.y; rhs[2] = rl.z;
        V3<T> ra = mat3_vec(iw, quat_diff_vec(bd.rot, inertial_rot[h])) / dt2;
        rhs[3] = ra.x; rhs[4] = ra.y; rhs[5] = ra.z;
        if (faithful_scan) {
            for (uint32_t pi = 0; pi < pairs.size(); pi++)
                if (pairs[pi].a == h || pairs[pi].b == h) stamp_contacts_for(h, pi, lhs, rhs);
            for (const Joint<T>& j : joints)  // gears stamp on their coupled joints' bodies
                if (j.a == h || j.b == h || j.kind == AVBD_JOINT_GEAR) stamp_joint_for(h, j, lhs, rhs);
        } else if (split_sums) {
            for (uint32_t pi : adj_pairs[h]) {
                T lp[6][6] = {};
                T rp[6] = {};
                stamp_contacts_for(h, pi, lp, rp);
                for (int i = 0; i < 6; i++) {
                    for (int k = 0; k < 6; k++) lhs[i][k] += lp[i][k];
                    rhs[i] += rp[i];
                }
            }
            for (uint32_t ji : adj_joints[h]) stamp_joint_for(h, joints[ji], lhs, rhs);
        } else {
            for (uint32_t pi : adj_pairs[h]) stamp_contacts_for(h, pi, lhs, rhs);
            for (uint32_t ji : adj_joints[h]) stamp_joint_for(h, joints[ji], lhs, rhs);
        }
        T neg[6] = {-rhs[0], -rhs[1], -rhs[2], -rhs[3], -rhs[4], -rhs[5]};
        T dx[6];
        if (solve_6x6(lhs, neg, dx)) {
            Body<T>& b = bodies[h];
            b.pos = b.pos + V3<T>{dx[0], dx[1], dx[2]};
            b.rot = quat_integrate(b.rot, V3<T>{dx[3], dx[4], dx[5]});
        } else {
            breakdowns++;
        }
    }

    void dual_update() {  // joints_ext.rs:464-919
        for (Pair<T>& p : pairs) {
            V3<T> n = p.n;
            V3<T> t1 = tangent_t1(n);
            V3<T> t2 = cross(t1, n);
            const Body<T>& A = bodies[p.a];
            const Body<T>& B = bodies[p.b];
            for (size_t qi = 0; qi < p.points.size(); qi++) {
                Point<T>& pt = p.points[qi];
                bool touching = p.gap <= T(0);
                T c0 = touching ? gap_c0(p, pt) : T(0);
                T cn = row_c_levers(p, n, c0, lever_a(A, n, pt), lever_b(B, n, pt));
                V3<T> raf, rbf;
                friction_levers(p, pt, raf, rbf);
                T ct1 = row_c_levers(p, t1, T(0), raf, rbf);
                T ct2 = row_c_levers(p, t2, T(0), raf, rbf);
                T pen[3] = {pt.pen[0], pt.pen[1], pt.pen[2]};
                T lam[3] = {pt.lam[0], pt.lam[1], pt.lam[2]};
                T f[3];
                contact_force(cn, pen, lam, ct1, ct2, p.mu, f);
                {
                    T bnd = std::fabs(f[0]) * fmx(p.mu[0], p.mu[1]);
                    T fu0 = pen[1] * ct1 + lam[1], fu1 = pen[2] * ct2 + lam[2];
                    T fs = std::sqrt(fu0 * fu0 + fu1 * fu1);
                    pt.stuck = fs <= bnd && std::sqrt(ct1 * ct1 + ct2 * ct2) < C<T>(K::STICK_THRESH);
                }
                if (touching && std::fabs(cn) >= C<T>(K::C_EPS)) {
                    pt.lam[0] = f[0];
                    if (f[0] < T(0)) pt.pen[0] = fmn(pt.pen[0] + C<T>(K::BETA) * std::fabs(cn), C<T>(K::PENALTY_MAX));
                }
                T b1 = std::fabs(f[0]) * p.mu[0], b2 = std::fabs(f[0]) * p.mu[1];
                T fu0 = pen[1] * ct1 + lam[1], fu1 = pen[2] * ct2 + lam[2];
                T s_ell = (b1 > T(0) && b2 > T(0)) ? (fu0 / b1) * (fu0 / b1) + (fu1 / b2) * (fu1 / b2)
                                                   : std::numeric_limits<T>::infinity();
                if (touching) {
                    pt.lam[1] = f[1];
                    pt.lam[2] = f[2];
                    if (s_ell <= T(1)) {
                        if (std::fabs(ct1) >= C<T>(K::C_EPS)) pt.pen[1] = fmn(pt.pen[1] + C<T>(K::BETA) * std::fabs(ct1), C<T>(K::PENALTY_MAX));
                        if (std::fabs(ct2) >= C<T>(K::C_EPS)) pt.pen[2] = fmn(pt.pen[2] + C<T>(K::BETA) * std::fabs(ct2), C<T>(K::PENALTY_MAX));
                    }
                }
                T mu_roll = fmx(A.rolling, B.rolling), mu_spin = fmx(A.torsion, B.torsion);
                if (touching && (mu_roll > T(0) || mu_spin > T(0))) {
                    V3<T> wrel = quat_diff_vec(A.rot, rot0[p.a]) - quat_diff_vec(B.rot, rot0[p.b]);
                    T lam_n = std::fabs(pt.lam[0]);
                    T rl[3] = {pt.roll_lam[0], pt.roll_lam[1], pt.roll_lam[2]};
                    V3<T> rax[3] = {t1, t2, n};
                    T murs[3] = {mu_roll, mu_roll, mu_spin};
                    for (int li = 0; li < 3; li++) {
                        if (murs[li] <= T(0)) continue;
                        T c = dot(wrel, rax[li]);
                        T cap = murs[li] * lam_n;
                        pt.roll_lam[li] = fclamp(C<T>(K::ROLL_PEN) * c + rl[li], -cap, cap);
                    }
                }
            }
        }
        for (Joint<T>& j : joints)
            if (j.kind != AVBD_JOINT_GEAR) dual_joint(j);
        // gears after every other joint (joints_ext.rs:897-918), penalty
        // capped like a limit's
        for (Joint<T>& g : joints) {
            if (g.kind != AVBD_JOINT_GEAR) continue;
            T c = gear_error(g);
            if (std::fabs(c) < C<T>(K::C_EPS)) continue;
            g.lam_l[0] = g.lam_l[0] + g.pen_l[0] * c;
            g.pen_l[0] = fmn(g.pen_l[0] + C<T>(K::BETA) * std::fabs(c), C<T>(K::LIM_PEN_MAX));
        }
    }

    // joints_ext.rs:574-896: the joint rows' multipliers and penalties.
    void dual_joint(Joint<T>& j) {
        const Body<T>& a = bodies[j.a];
        const Body<T>& b = bodies[j.b];
        V3<T> pa = a.pos + qrot(a.rot, j.la);
        V3<T> pb = b.pos + qrot(b.rot, j.lb);
        V3<T> pa0 = pos0[j.a] + qrot(rot0[j.a], j.la);
        V3<T> pb0 = pos0[j.b] + qrot(rot0[j.b], j.lb);
        V3<T> live = pa - pb, c0v = pa0 - pb0;
        const T eps = C<T>(K::C_EPS);
        auto ramp = [](T pen, T c, float beta, float cap) { return fmn(pen + C<T>(beta) * std::fabs(c), C<T>(cap)); };
        // a finite joint stiffness makes the anchor and hinge rows of ball and
        // revolute joints springs (penalty k, no multiplier)
        const bool soft = joint_k > T(0) && (j.kind == AVBD_JOINT_BALL || j.kind == AVBD_JOINT_REVOLUTE);
        if (j.kind == AVBD_JOINT_BALL || j.kind == AVBD_JOINT_REVOLUTE || j.kind == AVBD_JOINT_FIXED) {
            const bool fixed = j.kind == AVBD_JOINT_FIXED;
            V3<T> lv = fixed ? live + qrot(a.rot, j.dref) : live;
            V3<T> iv = fixed ? c0v + qrot(rot0[j.a], j.dref) : c0v;
            for (int k = 0; k < 3; k++) {
                T c = lv[k] - C<T>(K::ALPHA) * iv[k];
                if (soft) {
                    j.pen_l[k] = joint_k;
                } else if (std::fabs(c) >= eps) {
                    j.lam_l[k] += j.pen_l[k] * c;
                    j.pen_l[k] = ramp(j.pen_l[k], c, K::BETA, K::PENALTY_MAX);
                }
            }
        } else if (j.kind == AVBD_JOINT_PRISMATIC) {
            V3<T> wa = normalize_or(qrot(a.rot, j.ax_a), VZ<T>());
            V3<T> u, v;
            tangent_basis(wa, u, v);
            V3<T> axs[2] = {u, v};
            for (int li = 0; li < 2; li++) {
                T c = dot(live - C<T>(K::ALPHA) * c0v, axs[li]);
                if (std::fabs(c) >= eps) {
                    j.lam_l[li] += j.pen_l[li] * c;
                    j.pen_l[li] = ramp(j.pen_l[li], c, K::BETA, K::PENALTY_MAX);
                }
            }
        } else if (j.kind == AVBD_JOINT_WHEEL) {
            // the rows across the suspension axis, and the rigid suspension
            // row when the frequency is zero (joints_ext.rs:738-764); a live
            // spring carries no dual state
            V3<T> wa = normalize_or(qrot(a.rot, j.ax_a), VZ<T>());
            V3<T> u, v;
            tangent_basis(wa, u, v);
            V3<T> axs[2] = {u, v};
            for (int li = 0; li < 2; li++) {
                T c = dot(live - C<T>(K::ALPHA) * c0v, axs[li]);
                if (std::fabs(c) >= eps) {
                    j.lam_l[li] += j.pen_l[li] * c;
                    j.pen_l[li] = ramp(j.pen_l[li], c, K::BETA, K::PENALTY_MAX);
                }
            }
            if (j.susp_hz <= T(0)) {
                V3<T> wa0 = normalize_or(qrot(rot0[j.a], j.ax_a), VZ<T>());
                T c = (-dot(live, wa) - j.ref_val) - C<T>(K::ALPHA) * (-dot(pa0 - pb0, wa0) - j.ref_val);
                if (std::fabs(c) >= eps) {
                    j.lam_l[2] += j.pen_l[2] * c;
                    j.pen_l[2] = ramp(j.pen_l[2], c, K::BETA, K::LIM_PEN_MAX);
                }
            }
        } else if (j.kind == AVBD_JOINT_DISTANCE) {
            T c = (len(live) - j.ref_val) - C<T>(K::ALPHA) * (len(c0v) - j.ref_val);
            if (std::fabs(c) >= eps) {
                j.lam_l[0] += j.pen_l[0] * c;
                j.pen_l[0] = ramp(j.pen_l[0], c, K::BETA, K::PENALTY_MAX);
            }
        } else if (j.kind == AVBD_JOINT_ROPE) {
            T ln = len(live);
            if (ln > j.ref_val) {
                T c = (ln - j.ref_val) - C<T>(K::ALPHA) * (len(c0v) - j.ref_val);
                if (std::fabs(c) >= eps) {
                    j.lam_l[0] = fmx(j.lam_l[0] + j.pen_l[0] * c, T(0));
                    j.pen_l[0] = ramp(j.pen_l[0], c, K::BETA, K::LIM_PEN_MAX);
                }
            } else {
                j.lam_l[0] = T(0);
            }
        } else if (j.kind == AVBD_JOINT_SIXDOF) {
            for (int i = 0; i < 3; i++) {
                V3<T> e = VZERO<T>();
                e[i] = T(1);
                V3<T> dir = normalize_or(qrot(a.rot, e), e);
                if (j.six_cfg[i] == AVBD_AXIS_LOCKED) {
                    T c = dot((pb - pa) - qrot(a.rot, j.dref), dir);
                    if (std::fabs(c) >= eps) {
                        j.lam_l[i] += j.pen_l[i] * c;
                        j.pen_l[i] = ramp(j.pen_l[i], c, K::BETA, K::PENALTY_MAX);
                    }
                } else if (j.six_cfg[i] == AVBD_AXIS_LIMITED) {
                    T sep = dot((pb - pa) - qrot(a.rot, j.dref), dir);
                    int st = warm_limit_state(sep, j.six_min[i], j.six_max[i], C<T>(K::LIMIT_SLOP_LIN), j.sacc[i]);
                    if (st >= 0) {
                        bool lower = st == 1;
                        V3<T> axis0 = normalize_or(qrot(rot0[j.a], e), e);
                        T initial = dot((pb0 - pa0) - qrot(rot0[j.a], j.dref), axis0);
                        T c = regularized_limit(sep, initial, lower ? j.six_min[i] : j.six_max[i], lower);
                        if (std::fabs(c) >= eps) {
                            T f = j.pen_l[i] * c + j.sacc[i];
                            j.sacc[i] = lower ? fmn(f, T(0)) : fmx(f, T(0));
                            j.pen_l[i] = ramp(j.pen_l[i], c, K::BETA, K::LIM_PEN_MAX);
                        }
                    } else {
                        j.sacc[i] = T(0);
                    }
                }
            }
            V3<T> diff = quat_diff_vec(qmul(conj(a.rot), b.rot), j.q_ref);
            for (int i = 0; i < 3; i++) {
                V3<T> e = VZERO<T>();
                e[i] = T(1);
                if (j.six_cfg[3 + i] == AVBD_AXIS_LOCKED) {
                    T c = dot(diff, e);
                    if (std::fabs(c) >= eps) {
                        j.lam_a[i] += j.pen_a[i] * c;
                        j.pen_a[i] = ramp(j.pen_a[i], c, K::BETA_ANG, K::PENALTY_MAX);
                    }
                } else if (j.six_cfg[3 + i] == AVBD_AXIS_LIMITED) {
                    T travel = twist(a.rot, b.rot, e) - quat_twist(j.q_ref, e);
                    int st = warm_limit_state(travel, j.six_min[3 + i], j.six_max[3 + i], C<T>(K::LIMIT_SLOP_ANG),
                                              j.sacc[3 + i]);
                    if (st >= 0) {
                        bool lower = st == 1;
                        T initial = twist(rot0[j.a], rot0[j.b], e) - quat_twist(j.q_ref, e);
                        T c = regularized_limit(travel, initial, lower ? j.six_min[3 + i] : j.six_max[3 + i], lower);
                        if (std::fabs(c) >= eps) {
                            T f = j.pen_a[i] * c + j.sacc[3 + i];
                            j.sacc[3 + i] = lower ? fmn(f, T(0)) : fmx(f, T(0));
                            j.pen_a[i] = ramp(j.pen_a[i], c, K::BETA_ANG, K::LIM_PEN_MAX);
                        }
                    } else {
                        j.sacc[3 + i] = T(0);
                    }
                }
            }
        }
        // angular equality rows (a wheel's keyed on its axle, joints_ext.rs:789-803)
        if (j.kind == AVBD_JOINT_REVOLUTE || j.kind == AVBD_JOINT_PRISMATIC || j.kind == AVBD_JOINT_WHEEL) {
            const bool wheel = j.kind == AVBD_JOINT_WHEEL;
            const V3<T> hxa = wheel ? j.bx_a : j.ax_a, hxb = wheel ? j.bx_b : j.ax_b;
            V3<T> axa = qrot(a.rot, hxa), axb = qrot(b.rot, hxb);
            V3<T> axa0 = qrot(rot0[j.a], hxa), axb0 = qrot(rot0[j.b], hxb);
            V3<T> t1, t2;
            tangent_basis(axa0, t1, t2);
            V3<T> ts[2] = {t1, t2};
            for (int li = 0; li < 2; li++) {
                T c = dot(ts[li], axa - axb) - C<T>(K::ALPHA) * dot(ts[li], axa0 - axb0);
                if (soft) {
                    j.pen_a[li] = joint_k;
                    continue;
                }
                if (std::fabs(c) < eps) continue;
                j.lam_a[li] = j.pen_a[li] * c + j.lam_a[li];
                j.pen_a[li] = ramp(j.pen_a[li], c, K::BETA_ANG, K::PENALTY_MAX);
            }
        } else if (j.kind == AVBD_JOINT_FIXED) {
            V3<T> diff = quat_diff_vec(qmul(conj(a.rot), b.rot), j.q_ref);
            V3<T> diff0 = quat_diff_vec(qmul(conj(rot0[j.a]), rot0[j.b]), j.q_ref);
            for (int k = 0; k < 3; k++) {
                T c = diff[k] - C<T>(K::ALPHA) * diff0[k];
                if (std::fabs(c) < eps) continue;
                j.lam_a[k] += j.pen_a[k] * c;
                j.pen_a[k] = ramp(j.pen_a[k], c, K::BETA_ANG, K::PENALTY_MAX);
            }
        }
        // one-sided limits
        if (j.has_lim && j.kind == AVBD_JOINT_REVOLUTE) {
            T angle = wrap_pi(twist(a.rot, b.rot, j.ax_a) - j.ref_val);
            int st = warm_limit_state(angle, j.lo, j.hi, C<T>(K::LIMIT_SLOP_ANG), j.acc_lim);
            if (st >= 0) {
                bool lower = st == 1;
                T initial = wrap_pi(twist(rot0[j.a], rot0[j.b], j.ax_a) - j.ref_val);
                T c = regularized_limit(angle, initial, lower ? j.lo : j.hi, lower);
                if (std::fabs(c) >= eps) {
                    T f = j.pen_a[2] * c + j.acc_lim;
                    j.acc_lim = lower ? fmn(f, T(0)) : fmx(f, T(0));
                    j.pen_a[2] = ramp(j.pen_a[2], c, K::BETA_ANG, K::LIM_PEN_MAX);
                }
            } else {
                j.acc_lim = T(0);
            }
        } else if (j.has_lim && j.kind == AVBD_JOINT_PRISMATIC) {
            V3<T> wa = normalize_or(qrot(a.rot, j.ax_a), VZ<T>());
            T sv = dot(pb - pa, wa) - j.ref_val;
            int st = warm_limit_state(sv, j.lo, j.hi, C<T>(K::LIMIT_SLOP_LIN), j.lim_dual);
            if (st >= 0) {
                bool lower = st == 1;
                V3<T> axis0 = normalize_or(qrot(rot0[j.a], j.ax_a), VZ<T>());
                T initial = dot(pb0 - pa0, axis0) - j.ref_val;
                T c = regularized_limit(sv, initial, lower ? j.lo : j.hi, lower);
                if (std::fabs(c) >= eps) {
                    T f_raw = j.pen_l[2] * c + j.lim_dual;
                    j.lim_dual = lower ? fmn(f_raw, T(0)) : fmx(f_raw, T(0));
                    j.pen_l[2] = ramp(j.pen_l[2], c, K::BETA, K::LIM_PEN_MAX);
                }
            } else {
                j.acc_lim = T(0);
                j.lim_dual = T(0);
            }
        }
    }

    // Greedy colouring in descending hash priority == the GPU's Jones-Plassmann colouring.
    void compute_colouring() {
        uint32_t n = (uint32_t)bodies.size();
        std::vector<std::vector<uint32_t>> nb(n);
        auto solved = [&](uint32_t h) { return solvable(h) && !asleep[h]; };
        for (const Pair<T>& p : pairs)
            if (!p.points.empty() && solved(p.a) && solved(p.b)) { nb[p.a].push_back(p.b); nb[p.b].push_back(p.a); }
        for (const Joint<T>& j : joints) {
            if (j.kind == AVBD_JOINT_GEAR) {  // a gear couples its coupled joints' bodies
                uint32_t m[4];
                joint_members(j, m);
                for (uint32_t x : m)
                    for (uint32_t y : m)
                        if (x != y && solved(x) && solved(y)) nb[x].push_back(y);
                continue;
            }
            if (solved(j.a) && solved(j.b)) { nb[j.a].push_back(j.b); nb[j.b].push_back(j.a); }
        }
        std::vector<uint32_t> order;
        for (uint32_t h = 0; h < n; h++) {
            colour[h] = -1;
            if (solved(h)) order.push_back(h);
        }
        auto prio_gt = [](uint32_t x, uint32_t y) {
            uint32_t hx = colour_hash(x), hy = colour_hash(y);
            return hx != hy ? hx > hy : x > y;
        };
        std::sort(order.begin(), order.end(), prio_gt);
        int32_t maxc = -1;
        std::vector<uint8_t> used;
        for (uint32_t h : order) {
            used.assign(nb[h].size() + 2, 0);
            for (uint32_t o : nb[h])
                if (colour[o] >= 0 && colour[o] < (int32_t)used.size()) used[colour[o]] = 1;
            int32_t c = 0;
            while (used[c]) c++;
            colour[h] = c;
            maxc = std::max(maxc, c);
        }
        ncolours = (uint64_t)(maxc + 1);
    }

    void build_adjacency() {
        size_t n = bodies.size();
        adj_pairs.assign(n, {});
        adj_joints.assign(n, {});
        for (uint32_t pi = 0; pi < pairs.size(); pi++) {
            adj_pairs[pairs[pi].a].push_back(pi);
            if (pairs[pi].b != pairs[pi].a) adj_pairs[pairs[pi].b].push_back(pi);
        }
        for (uint32_t ji = 0; ji < joints.size(); ji++) {
            if (joints[ji].kind == AVBD_JOINT_GEAR) {  // once on each of its coupled joints' bodies
                uint32_t m[4];
                joint_members(joints[ji], m);
                for (uint32_t h : m)
                    if (adj_joints[h].empty() || adj_joints[h].back() != ji) adj_joints[h].push_back(ji);
                continue;
            }
            adj_joints[joints[ji].a].push_back(ji);
            adj_joints[joints[ji].b].push_back(ji);
        }
        // adjacency lists are filled in ascending pair index: same order as
        // the reference's scan over the pair vector (assembly.rs:99-106).
        for (size_t h = 0; h < n; h++) std::sort(adj_pairs[h].begin(), adj_pairs[h].end());
    }

    // ---- CCD (mod.rs:882-978, distance.rs:841-893) ----
    void ccd_pass() {
        uint32_t n = (uint32_t)bodies.size();
        for (uint32_t h = 0; h < n; h++) {
            if (!solvable(h) || asleep[h] || bodies[h].trigger()) continue;
            V3<T> disp = bodies[h].vel * dt;
            if (len(disp) <= C<T>(K::CCD_TRAVEL_GATE_FRACTION) * shape_min_dimension(bodies[h])) continue;
            std::vector<uint32_t> joined;
            for (const Joint<T>& j : joints) {
                if (j.kind == AVBD_JOINT_GEAR) continue;  // a gear joins no bodies (mod.rs:903-906)
                if (j.a == h) joined.push_back(j.b);
                else if (j.b == h) joined.push_back(j.a);
            }
            T L = len(disp);
            if (L < C<T>(K::NEAR_ZERO)) continue;
            V3<T> dir = disp / L;
            bool have = false;
            T best_t = T(0);
            V3<T> best_n{}, best_p{};
            uint32_t best_h = 0;
            const Body<T>& mb = bodies[h];
            for (uint32_t o = 0; o < n; o++) {
                if (o == h || bodies[o].trigger() || !pair_allowed(bodies[h], bodies[o])) continue;
                if (std::find(joined.begin(), joined.end(), o) != joined.end()) continue;
                ShapeRef<T> tgt = sref(bodies[o]);
                T t = T(0);
                bool hit = false;
                V3<T> hn{}, hp{};
                for (int it = 0; it < 24; it++) {
                    ShapeRef<T> mv{&mb, mb.shape, mb.sp, mb.pos + dir * t, mb.rot, mb.hull, mb.ext, mb.hf, mb.mesh};
                    Dist<T> d = shape_distance_any(mv, tgt);
                    if (d.dist <= C<T>(K::SHAPE_TOUCH)) {
                        if (t > T(0)) { hit = true; hn = normalize_or(d.pa - d.pb, -dir); hp = d.pb; }
                        break;
                    }
                    t += d.dist - C<T>(K::SHAPE_TOUCH) * C<T>(K::HALF);
                    if (t >= L) break;
                }
                if (hit && (!have || t < best_t)) { have = true; best_t = t; best_n = hn; best_p = hp; best_h = o; }
            }
            if (!have) continue;
            ccd_hits++;
            {   // a swept impact is a hit event (mod.rs:946-960)
                T approach = -dot(pre_vel[h] - pre_vel[best_h], best_n);
                if (approach > C<T>(K::CONTACT_HIT_THRESHOLD)) {
                    AvbdContactEvent e{};
                    V3<T> nn = h < best_h ? -best_n : best_n;
                    e.body_a = std::min(h, best_h);
                    e.body_b = std::max(h, best_h);
                    e.kind = AVBD_CONTACT_HIT;
                    e.point[0] = (float)best_p.x; e.point[1] = (float)best_p.y; e.point[2] = (float)best_p.z;
                    e.normal[0] = (float)nn.x; e.normal[1] = (float)nn.y; e.normal[2] = (float)nn.z;
                    e.approach_speed = (float)approach;
                    ccd_ev.push_back(e);
                }
            }
            T l2 = fmx(L, C<T>(K::MIN_TOI_DISP_LENGTH));
            T frac = fclamp(best_t / l2, T(0), T(1));
            T e = fmn(bodies[h].restitution, bodies[best_h].restitution);
            if (freeze_frames) {  // the time of impact and its normal held fixed, as a contact frame
                frac = no_tangent(frac);
                best_n = {no_tangent(best_n.x), no_tangent(best_n.y), no_tangent(best_n.z)};
            }
            Body<T>& b = bodies[h];
            b.pos = b.pos + disp * frac;
            T vn = dot(b.vel, best_n);
            if (vn < T(0)) {
                T bounce = vn < -C<T>(K::CCD_BOUNCE_SPEED) ? T(1) + e : T(1);
                b.vel = b.vel - best_n * (bounce * vn);
            }
            wake_body(best_h);
            sleep_timer[h] = T(0);
        }
    }

    // ---- events (mod.rs:1606-1669) ----
    void emit_events() {
        // trigger transitions: symmetric difference in key order
        {
            auto i = trig_now.begin(), j = prev_trigger.begin();
            while (i != trig_now.end() || j != prev_trigger.end()) {
                if (j == prev_trigger.end() || (i != trig_now.end() && *i < *j)) {
                    tev.push_back(AvbdTriggerEvent{i->first, i->second, 1u});
                    ++i;
                } else if (i == trig_now.end() || *j < *i) {
                    tev.push_back(AvbdTriggerEvent{j->first, j->second, 0u});
                    ++j;
                } else {
                    ++i;
                    ++j;
                }
            }
            prev_trigger = trig_now;
        }
        std::set<Key> touch_now;
        std::vector<AvbdContactEvent> hits;
        for (const Pair<T>& p : pairs) {
            const Body<T>& a = bodies[p.a];
            const Body<T>& b = bodies[p.b];
            T deepest = T(0);
            V3<T> witness = (a.pos + b.pos) * C<T>(K::HALF);
            for (const Point<T>& pt : p.points) {
                V3<T> pa = a.pos + qrot(a.rot, pt.ra);
                V3<T> pb = b.pos + qrot(b.rot, pt.rb);
                T gap = dot(p.n, pa - pb);
                if (-gap > deepest) { deepest = -gap; witness = pa; }
            }
            if (deepest > C<T>(K::CONTACT_BEGIN_SLOP)) {
                touch_now.insert({p.a, p.b});
                if (!prev_touch.count({p.a, p.b})) {
                    T approach = -dot(pre_vel[p.a] - pre_vel[p.b], p.n);
                    if (approach > C<T>(K::CONTACT_HIT_THRESHOLD)) {
                        AvbdContactEvent e{};
                        e.body_a = p.a; e.body_b = p.b; e.kind = AVBD_CONTACT_HIT;
                        e.point[0] = (float)witness.x; e.point[1] = (float)witness.y; e.point[2] = (float)witness.z;
                        e.normal[0] = (float)-p.n.x; e.normal[1] = (float)-p.n.y; e.normal[2] = (float)-p.n.z;
                        e.approach_speed = (float)approach;
                        hits.push_back(e);
                    }
                }
            }
        }
        auto i = touch_now.begin(), j = prev_touch.begin();
        while (i != touch_now.end() || j != prev_touch.end()) {
            AvbdContactEvent e{};
            if (j == prev_touch.end() || (i != touch_now.end() && *i < *j)) {
                e.body_a = i->first; e.body_b = i->second; e.kind = AVBD_CONTACT_BEGIN;
                cev.push_back(e);
                ++i;
            } else if (i == touch_now.end() || *j < *i) {
                e.body_a = j->first; e.body_b = j->second; e.kind = AVBD_CONTACT_END;
                cev.push_back(e);
                ++j;
            } else {
                ++i;
                ++j;
            }
        }
        for (auto& e : hits) cev.push_back(e);
        prev_touch.swap(touch_now);
    }

    // ---- one fixed substep (mod.rs:846-1143); `emit`: the step's last substep ----
    void step_inner(bool emit = true) {
        ensure_scratch();
        wake_joint_motion();
        update_gear_mem();
        uint32_t n = (uint32_t)bodies.size();
        ccd_ev.clear();
        for (uint32_t h = 0; h < n; h++) {
            if (!solvable(h)) continue;
            Body<T>& b = bodies[h];
            T iw[3][3], inv[3][3];
            world_inertia(b.inertia, b.rot, iw);
            V3<T> dg{b.inertia.x > T(0) ? b.inertia.x : T(0), b.inertia.y > T(0) ? b.inertia.y : T(0),
                     b.inertia.z > T(0) ? b.inertia.z : T(0)};
            inverse_symmetric(iw, dg, inv);
            V3<T> tq = b.torque;
            b.torque = VZERO<T>();
            b.angvel = b.angvel + mat3_vec(inv, tq) * dt;
        }
        motor_impulse();
        rope_impulse();
        pre_vel.resize(n);
        for (uint32_t h = 0; h < n; h++) pre_vel[h] = bodies[h].vel;  // mod.rs:874-876
        if (prm.enable_ccd) ccd_pass();
        generate_pairs();
        wake_joint_motion();
        for (uint32_t h = 0; h < n; h++)
            if (asleep[h]) {
                const Body<T>& b = bodies[h];
                if (len(b.vel) > C<T>(K::SLEEP_LIN) || len(b.angvel) > C<T>(K::SLEEP_ANG)) wake_body(h);
            }
        for (uint32_t h = 0; h < n; h++) {
            if (bodies[h].type == AVBD_BODY_KINEMATIC) { pos0[h] = prev_pos[h]; rot0[h] = prev_rot[h]; }
            else { pos0[h] = bodies[h].pos; rot0[h] = bodies[h].rot; }
            if (!solvable(h)) { inertial[h] = bodies[h].pos; inertial_rot[h] = bodies[h].rot; continue; }
            const Body<T>& b = bodies[h];
            inertial[h] = b.pos + b.vel * dt + gravity * (dt * dt);
            inertial_rot[h] = quat_integrate(b.rot, b.angvel * dt);
        }
        const T ag = C<T>(K::ALPHA) * C<T>(K::GAMMA);
        for (Pair<T>& p : pairs)
            for (Point<T>& pt : p.points)
                for (int k = 0; k < 3; k++) {
                    pt.lam[k] *= ag;
                    pt.roll_lam[k] *= ag;
                    pt.pen[k] = fclamp(pt.pen[k] * C<T>(K::GAMMA), C<T>(K::PENALTY_MIN), C<T>(K::PENALTY_MAX));
                }
        for (Joint<T>& j : joints)
            for (int k = 0; k < 3; k++) {
                j.lam_l[k] *= ag;
                j.lam_a[k] *= ag;
                j.pen_l[k] = fclamp(j.pen_l[k] * C<T>(K::GAMMA), C<T>(K::PENALTY_MIN), C<T>(K::PENALTY_MAX));
                j.pen_a[k] = fclamp(j.pen_a[k] * C<T>(K::GAMMA), C<T>(K::PENALTY_MIN), C<T>(K::PENALTY_MAX));
                if (joint_k > T(0) && (j.kind == AVBD_JOINT_BALL || j.kind == AVBD_JOINT_REVOLUTE)) {
                    // soft rows: anchors and hinge alignment (not the limit)
                    j.pen_l[k] = joint_k;
                    if (k < 2) j.pen_a[k] = joint_k;
                }
            }
        for (uint32_t h = 0; h < n; h++) {
            if (!solvable(h) || asleep[h]) continue;
            bodies[h].pos = inertial[h];
            bodies[h].rot = inertial_rot[h];
        }
        if (!faithful_scan) build_adjacency();
        std::vector<std::vector<uint32_t>> by_colour;
        if (mode == COLOURED) {
            compute_colouring();
            by_colour.assign(ncolours, {});
            for (uint32_t h = 0; h < n; h++)
                if (colour[h] >= 0) by_colour[colour[h]].push_back(h);
        }
        for (int it = 0; it < prm.iterations; it++) {
            if (mode == COLOURED) {
                for (auto& group : by_colour)
                    for (uint32_t h : group) solve_body(h);
            } else {
                for (uint32_t h = n; h-- > 0;)
                    if (solvable(h) && !asleep[h]) solve_body(h);
            }
            dual_update();
        }
        for (uint32_t h = 0; h < n; h++) {
            if (!solvable(h) || asleep[h]) continue;
            Body<T>& b = bodies[h];
            b.vel = (b.pos - pos0[h]) / dt;
            V3<T> spin = quat_diff_vec(b.rot, rot0[h]);
            b.angvel = len(spin) < C<T>(K::SPIN_REST_EPS) ? VZERO<T>() : spin / dt;
            b.rot = qnormalize(b.rot);
        }
        if (prm.enable_sleep) {
            std::vector<uint8_t> supported(n, 0);
            for (const Pair<T>& p : pairs)
                if (p.gap <= T(0) && !p.points.empty()) { supported[p.a] = 1; supported[p.b] = 1; }
            for (const Joint<T>& j : joints) { supported[j.a] = 1; supported[j.b] = 1; }
            std::vector<uint8_t> ready = joint_sleep_ready();
            std::vector<uint8_t> freeze(asleep.begin(), asleep.end());
            for (uint32_t h = 0; h < n; h++) {
                if (!solvable(h) || asleep[h]) continue;
                if (!supported[h] || !ready[h]) { sleep_timer[h] = T(0); continue; }
                const Body<T>& b = bodies[h];
                if (len(b.vel) < C<T>(K::SLEEP_LIN) && len(b.angvel) < C<T>(K::SLEEP_ANG)) {
                    sleep_timer[h] += dt;
                    freeze[h] = sleep_timer[h] >= C<T>(K::SLEEP_TIME);
                } else {
                    sleep_timer[h] = T(0);
                }
            }
            propagate_joint_flags(freeze, 0);
            for (uint32_t h = 0; h < n; h++)
                if (freeze[h] && !asleep[h]) sleep_body(h);
        }
        {
            size_t ev_start = cev.size();
            if (emit) emit_events();
            // swept impacts not already reported as hits this substep (mod.rs:1126-1136)
            for (const AvbdContactEvent& e : ccd_ev) {
                bool dup = false;
                for (size_t i = ev_start; i < cev.size(); i++)
                    if (cev[i].body_a == e.body_a && cev[i].body_b == e.body_b && cev[i].kind == AVBD_CONTACT_HIT)
                        dup = true;
                if (!dup) cev.push_back(e);
            }
        }
        for (uint32_t h = 0; h < n; h++) { prev_pos[h] = bodies[h].pos; prev_rot[h] = bodies[h].rot; }
        steps++;
    }
    void step_fixed(int nsub) {
        for (int i = 0; i < nsub; i++)
            step_inner(emit_period > 0 ? (i + 1) % emit_period == 0 : i == nsub - 1);
    }

    void step(float host_dt) {  // mod.rs:1212-1235
        if (!std::isfinite(host_dt) || host_dt <= 0.0f) return;
        T sd = dt;
        time_debt = fmn(time_debt + T(host_dt), sd * T(prm.max_substeps));
        int k = 0;
        while (time_debt >= sd && k < prm.max_substeps) {
            time_debt -= sd;
            k++;
            step_inner(time_debt < sd || k == prm.max_substeps);
        }
    }

    // PhysicsEngine::remove_body (mod.rs:1241-1300): the last body moves into
    // the freed slot; pairs and joints of the removed body go, the others are
    // renumbered; handle-keyed event state is cleared or remapped; every
    // sleeper wakes.
    // retain_joints (mod.rs:766-784) with joint_remap (migration.rs:74-115):
    // a gear whose coupled joint goes goes too; the survivors move down and
    // gears follow their joints' new handles.
    void retain_joints(std::vector<uint8_t> gone) {
        for (bool changed = true; changed;) {
            changed = false;
            for (size_t i = 0; i < joints.size(); i++)
                if (!gone[i] && joints[i].kind == AVBD_JOINT_GEAR && (gone[joints[i].gb[0]] || gone[joints[i].gb[1]])) {
                    gone[i] = 1;
                    changed = true;
                }
        }
        std::vector<uint32_t> remap(joints.size(), 0);
        uint32_t next = 0;
        for (size_t i = 0; i < joints.size(); i++) remap[i] = gone[i] ? 0u : next++;
        std::vector<Joint<T>> kept;
        for (size_t i = 0; i < joints.size(); i++) {
            if (gone[i]) continue;
            Joint<T> j = joints[i];
            if (j.kind == AVBD_JOINT_GEAR) {
                j.gb[0] = remap[j.gb[0]];
                j.gb[1] = remap[j.gb[1]];
            }
            kept.push_back(j);
        }
        joints.swap(kept);
    }

    void remove_body(uint32_t hi) {
        if (hi >= bodies.size()) return;
        uint32_t last = (uint32_t)bodies.size() - 1;
        std::vector<Key> exited;
        for (const Key& k : prev_trigger)
            if (k.first == hi || k.second == hi) exited.push_back(k);
        std::sort(exited.begin(), exited.end());
        for (const Key& k : exited) tev.push_back(AvbdTriggerEvent{k.first, k.second, 0u});
        bodies[hi] = bodies[last];
        bodies.pop_back();
        auto map = [&](uint32_t h) { return h == last ? hi : h; };
        std::vector<Pair<T>> kept;
        for (Pair<T>& p : pairs) {
            if (p.a == hi || p.b == hi) continue;
            p.a = map(p.a);
            p.b = map(p.b);
            kept.push_back(std::move(p));
        }
        pairs.swap(kept);
        std::vector<uint8_t> gone(joints.size(), 0);
        for (size_t i = 0; i < joints.size(); i++) gone[i] = joints[i].a == hi || joints[i].b == hi;
        retain_joints(gone);
        for (Joint<T>& j : joints) {
            j.a = map(j.a);
            j.b = map(j.b);
        }
        prev_touch.clear();
        std::set<Key> remapped;
        for (const Key& k : prev_trigger) {
            if (k.first == hi || k.second == hi) continue;
            uint32_t a = map(k.first), b = map(k.second);
            remapped.insert({std::min(a, b), std::max(a, b)});
        }
        prev_trigger.swap(remapped);
        cev.clear();
        auto swap_remove = [&](auto& v) {
            if (hi < v.size()) {
                v[hi] = v.back();
                v.pop_back();
            }
        };
        swap_remove(sleep_timer);
        swap_remove(asleep);
        swap_remove(prev_pos);
        swap_remove(prev_rot);
        for (uint32_t h = 0; h < bodies.size(); h++) wake_body(h);
    }

    int add_joint(const AvbdJointDesc& d, uint32_t& handle) {  // mod.rs:1310-1529
        // validate_joint (migration.rs:160-330): anchors and axes finite, bounds ordered, motors finite
        auto finite3 = [](const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); };
        auto bounds_ok = [](float lo, float hi) { return std::isfinite(lo) && std::isfinite(hi) && lo <= hi; };
        if (d.kind > AVBD_JOINT_GEAR) return AVBD_ERR_UNSUPPORTED;
        const bool gear = d.kind == AVBD_JOINT_GEAR;
        if (gear && !std::isfinite(d.gear_ratio)) return AVBD_ERR_JOINT_NONFINITE;  // migration.rs:193-200
        if (!gear && d.kind != AVBD_JOINT_MOTOR && (!finite3(d.local_anchor_a) || !finite3(d.local_anchor_b)))
            return AVBD_ERR_JOINT_BAD_AXIS;
        if (d.kind == AVBD_JOINT_MOTOR) {  // migration.rs:331-356
            if (!finite3(d.motor_linear) || !finite3(d.motor_angular)) return AVBD_ERR_JOINT_NONFINITE;
            if (!(std::isfinite(d.motor_max_force) && d.motor_max_force >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
            if (!(std::isfinite(d.motor_max_torque) && d.motor_max_torque >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
            if (!(std::isfinite(d.motor_correction) && d.motor_correction >= 0.0f && d.motor_correction <= 1.0f))
                return AVBD_ERR_JOINT_BAD_BOUNDS;
        }
        const bool axial = d.kind == AVBD_JOINT_REVOLUTE || d.kind == AVBD_JOINT_PRISMATIC;
        if (axial) {
            if (!finite3(d.local_axis_a) || !finite3(d.local_axis_b)) return AVBD_ERR_JOINT_BAD_AXIS;
            if (d.has_limit && !bounds_ok(d.limit_min, d.limit_max)) return AVBD_ERR_JOINT_BAD_BOUNDS;
            if (d.has_motor && !(std::isfinite(d.motor_speed) && std::isfinite(d.motor_max) && d.motor_max >= 0.0f))
                return AVBD_ERR_JOINT_NONFINITE;
        }
        if (d.kind == AVBD_JOINT_WHEEL) {  // migration.rs:284-314
            if (!finite3(d.local_axis_a) || !finite3(d.local_axis_b) || !finite3(d.local_axle_a) ||
                !finite3(d.local_axle_b))
                return AVBD_ERR_JOINT_BAD_AXIS;
            if (!(std::isfinite(d.suspension_hz) && d.suspension_hz >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
            if (!(std::isfinite(d.suspension_damping) && d.suspension_damping >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
            if (d.has_motor && !(std::isfinite(d.motor_speed) && std::isfinite(d.motor_max) && d.motor_max >= 0.0f))
                return AVBD_ERR_JOINT_NONFINITE;
        }
        if (d.kind == AVBD_JOINT_SIXDOF)
            for (int k = 0; k < 6; k++) {
                if (d.axis_config[k] > AVBD_AXIS_LIMITED) return AVBD_ERR_INVALID_ARG;
                if (d.axis_config[k] == AVBD_AXIS_LIMITED && !bounds_ok(d.axis_min[k], d.axis_max[k]))
                    return AVBD_ERR_JOINT_BAD_BOUNDS;
            }
        if (d.kind == AVBD_JOINT_ROPE && !(std::isfinite(d.max_distance) && d.max_distance > 0.0f))
            return AVBD_ERR_JOINT_BAD_BOUNDS;
        if (d.kind == AVBD_JOINT_SPRING) {  // validate_motor (migration.rs:366-394)
            if (!std::isfinite(d.spring_rest) || !std::isfinite(d.spring_velocity)) return AVBD_ERR_JOINT_NONFINITE;
            for (float v : {d.spring_stiffness, d.spring_damping, d.spring_max_force})
                if (!(std::isfinite(v) && v >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
            if (d.spring_kind > AVBD_MOTOR_SERVO || d.spring_model > AVBD_MODEL_FORCE) return AVBD_ERR_INVALID_ARG;
        }
        wake_body(d.body_a);
        wake_body(d.body_b);
        if (d.body_a == d.body_b) return AVBD_ERR_JOINT_SELF;
        if (d.body_a >= bodies.size() || d.body_b >= bodies.size()) return AVBD_ERR_JOINT_HANDLES;
        Joint<T> j{};
        j.a = d.body_a; j.b = d.body_b; j.kind = d.kind;
        if (gear) {  // mod.rs:1329-1404: the coupled joints exist and are hinges or slides
            if (d.gear_joint_a >= joints.size() || d.gear_joint_b >= joints.size()) return AVBD_ERR_JOINT_UNKNOWN_REF;
            for (uint32_t r : {d.gear_joint_a, d.gear_joint_b})
                if (joints[r].kind != AVBD_JOINT_REVOLUTE && joints[r].kind != AVBD_JOINT_PRISMATIC)
                    return AVBD_ERR_UNSUPPORTED;
            j.la = j.lb = VZERO<T>();
            j.ax_a = j.ax_b = j.bx_a = j.bx_b = VX<T>();
            j.q_ref = Qt<T>{T(0), T(0), T(0), T(1)};
            j.dref = VZERO<T>();
            j.gb[0] = d.gear_joint_a;
            j.gb[1] = d.gear_joint_b;
            j.gratio = T(d.gear_ratio);
            j.ref_val = joint_coordinate(joints[j.gb[0]]) + j.gratio * joint_coordinate(joints[j.gb[1]]);
            j.gmem_set = false;
            for (int k = 0; k < 6; k++) j.sacc[k] = T(0);
            for (int k = 0; k < 3; k++) {
                j.lam_l[k] = j.lam_a[k] = T(0);
                j.pen_l[k] = j.pen_a[k] = C<T>(K::JOINT_PENALTY_INIT);
            }
            joints.push_back(j);
            handle = (uint32_t)(joints.size() - 1);
            return AVBD_OK;
        }
        j.la = {T(d.local_anchor_a[0]), T(d.local_anchor_a[1]), T(d.local_anchor_a[2])};
        j.lb = {T(d.local_anchor_b[0]), T(d.local_anchor_b[1]), T(d.local_anchor_b[2])};
        if (d.kind == AVBD_JOINT_MOTOR) j.la = j.lb = VZERO<T>();  // a free motor has no anchors
        j.ax_a = VX<T>(); j.ax_b = VX<T>();
        j.ref_val = T(0);
        j.q_ref = Qt<T>{T(0), T(0), T(0), T(1)};
        j.dref = VZERO<T>();
        // resolve_joint (joint.rs:1251-1400)
        const Body<T>& ba = bodies[j.a];
        const Body<T>& bb = bodies[j.b];
        if (axial) {
            V3<T> aa{T(d.local_axis_a[0]), T(d.local_axis_a[1]), T(d.local_axis_a[2])};
            V3<T> ab{T(d.local_axis_b[0]), T(d.local_axis_b[1]), T(d.local_axis_b[2])};
            if (len2(aa) < C<T>(K::DEGENERATE_LEN2) || len2(ab) < C<T>(K::DEGENERATE_LEN2)) return AVBD_ERR_JOINT_BAD_AXIS;
            j.ax_a = normalize_or(aa, VZ<T>());
            j.ax_b = normalize_or(ab, VZ<T>());
            if (d.kind == AVBD_JOINT_REVOLUTE) {
                j.ref_val = hinge_twist(ba.rot, bb.rot, j.ax_a);
            } else {
                V3<T> wa = normalize_or(qrot(ba.rot, j.ax_a), VZ<T>());
                V3<T> pa0 = ba.pos + qrot(ba.rot, j.la);
                V3<T> pb0 = bb.pos + qrot(bb.rot, j.lb);
                j.ref_val = dot(pb0 - pa0, wa);
            }
            j.has_lim = d.has_limit != 0;
            j.lo = T(d.limit_min);
            j.hi = T(d.limit_max);
            j.has_mot = d.has_motor != 0;
            j.mot_speed = T(d.motor_speed);
            j.mot_max = T(d.motor_max);
        } else if (d.kind == AVBD_JOINT_WHEEL) {  // joint.rs:1352-1379
            V3<T> sa{T(d.local_axis_a[0]), T(d.local_axis_a[1]), T(d.local_axis_a[2])};
            V3<T> sb{T(d.local_axis_b[0]), T(d.local_axis_b[1]), T(d.local_axis_b[2])};
            if (len2(sa) < C<T>(K::DEGENERATE_LEN2) || len2(sb) < C<T>(K::DEGENERATE_LEN2)) return AVBD_ERR_JOINT_BAD_AXIS;
            j.ax_a = normalize_or(sa, VY<T>());
            j.ax_b = normalize_or(sb, VY<T>());
            V3<T> xa{T(d.local_axle_a[0]), T(d.local_axle_a[1]), T(d.local_axle_a[2])};
            V3<T> xb{T(d.local_axle_b[0]), T(d.local_axle_b[1]), T(d.local_axle_b[2])};
            j.bx_a = orthogonalize_axle(j.ax_a, xa);
            j.bx_b = orthogonalize_axle(j.ax_b, xb);
            V3<T> wa = normalize_or(qrot(ba.rot, j.ax_a), VZ<T>());
            V3<T> pa0 = ba.pos + qrot(ba.rot, j.la);
            V3<T> pb0 = bb.pos + qrot(bb.rot, j.lb);
            j.ref_val = dot(pb0 - pa0, wa);
            j.has_mot = d.has_motor != 0;
            j.mot_speed = T(d.motor_speed);
            j.mot_max = T(d.motor_max);
            j.susp_hz = T(d.suspension_hz);
            j.susp_zeta = T(d.suspension_damping);
        } else if (d.kind == AVBD_JOINT_FIXED || d.kind == AVBD_JOINT_SIXDOF || d.kind == AVBD_JOINT_MOTOR) {
            // the assembly pose (a free motor's only for its rest residual)
            j.q_ref = qmul(conj(ba.rot), bb.rot);
            V3<T> ra = qrot(ba.rot, j.la), rb = qrot(bb.rot, j.lb);
            j.dref = qrot(conj(ba.rot), (bb.pos + rb) - (ba.pos + ra));
            for (int k = 0; k < 6; k++) {
                j.six_cfg[k] = d.kind == AVBD_JOINT_SIXDOF ? d.axis_config[k] : AVBD_AXIS_FREE;
                j.six_min[k] = T(d.axis_min[k]);
                j.six_max[k] = T(d.axis_max[k]);
            }
        } else if (d.kind == AVBD_JOINT_DISTANCE) {
            V3<T> ra = qrot(ba.rot, j.la), rb = qrot(bb.rot, j.lb);
            j.ref_val = len((bb.pos + rb) - (ba.pos + ra));
        } else if (d.kind == AVBD_JOINT_ROPE) {
            j.ref_val = T(d.max_distance);
        }
        j.mot_lin = {T(d.motor_linear[0]), T(d.motor_linear[1]), T(d.motor_linear[2])};
        j.mot_ang = {T(d.motor_angular[0]), T(d.motor_angular[1]), T(d.motor_angular[2])};
        j.mot_force = T(d.motor_max_force);
        j.mot_torque = T(d.motor_max_torque);
        if (d.kind != AVBD_JOINT_MOTOR) {
            j.mot_lin = j.mot_ang = VZERO<T>();
            j.mot_force = j.mot_torque = T(0);
        }
        if (d.kind == AVBD_JOINT_SPRING) {  // the rest length rides in the motor (mod.rs:1487-1493)
            j.ref_val = T(d.spring_rest);
            j.spr_vel = T(d.spring_velocity);
            j.spr_k = T(d.spring_stiffness);
            j.spr_c = T(d.spring_damping);
            j.spr_max = T(d.spring_max_force);
            j.spr_kind = d.spring_kind;
            j.spr_model = d.spring_model;
        }
        j.acc_lim = T(0);
        j.lim_dual = T(0);
        for (int k = 0; k < 6; k++) j.sacc[k] = T(0);
        for (int k = 0; k < 3; k++) {
            j.lam_l[k] = j.lam_a[k] = T(0);
            j.pen_l[k] = j.pen_a[k] = C<T>(K::JOINT_PENALTY_INIT);
        }
        joints.push_back(j);
        handle = (uint32_t)(joints.size() - 1);
        return AVBD_OK;
    }
};

template <class T> static Body<T> from_desc(const AvbdBody& s) {
    Body<T> b;
    b.pos = {T(s.position[0]), T(s.position[1]), T(s.position[2])};
    b.rot = {T(s.orientation[0]), T(s.orientation[1]), T(s.orientation[2]), T(s.orientation[3])};
    b.vel = {T(s.velocity[0]), T(s.velocity[1]), T(s.velocity[2])};
    b.angvel = {T(s.angular_velocity[0]), T(s.angular_velocity[1]), T(s.angular_velocity[2])};
    b.torque = {T(s.torque[0]), T(s.torque[1]), T(s.torque[2])};
    b.mass = T(s.mass); b.inv_mass = T(s.inv_mass);
    b.inertia = {T(s.inertia[0]), T(s.inertia[1]), T(s.inertia[2])};
    b.restitution = T(s.restitution); b.friction = T(s.friction); b.friction_t = T(s.friction_transverse);
    b.rolling = T(s.rolling_friction); b.torsion = T(s.torsion_friction);
    b.shape = s.shape;
    b.sp = {T(s.shape_params[0]), T(s.shape_params[1]), T(s.shape_params[2])};
    b.layer = s.collision_layer; b.mask = s.collision_mask; b.type = s.body_type; b.flags = s.flags;
    return b;
}
template <class T> static void to_desc(const Body<T>& b, AvbdBody& s) {
    s.position[0] = float(b.pos.x); s.position[1] = float(b.pos.y); s.position[2] = float(b.pos.z);
    s.orientation[0] = float(b.rot.x); s.orientation[1] = float(b.rot.y); s.orientation[2] = float(b.rot.z); s.orientation[3] = float(b.rot.w);
    s.velocity[0] = float(b.vel.x); s.velocity[1] = float(b.vel.y); s.velocity[2] = float(b.vel.z);
    s.angular_velocity[0] = float(b.angvel.x); s.angular_velocity[1] = float(b.angvel.y); s.angular_velocity[2] = float(b.angvel.z);
    s.torque[0] = float(b.torque.x); s.torque[1] = float(b.torque.y); s.torque[2] = float(b.torque.z);
    s.mass = float(b.mass); s.inv_mass = float(b.inv_mass);
    s.inertia[0] = float(b.inertia.x); s.inertia[1] = float(b.inertia.y); s.inertia[2] = float(b.inertia.z);
    s.restitution = float(b.restitution); s.friction = float(b.friction); s.friction_transverse = float(b.friction_t);
    s.rolling_friction = float(b.rolling); s.torsion_friction = float(b.torsion);
    s.shape = b.shape;
    s.shape_params[0] = float(b.sp.x); s.shape_params[1] = float(b.sp.y); s.shape_params[2] = float(b.sp.z);
    s.collision_layer = b.layer; s.collision_mask = b.mask; s.body_type = b.type; s.flags = b.flags;
}

struct OracleBase {
    virtual ~OracleBase() {}
};
template <class T> struct Oracle : OracleBase {
    Engine<T> e;
};

}  // namespace orc

// ---- C API for the tests (ctypes) ----------------------------------------------
using namespace orc;

struct OracleWorld {
    int dbl;  // 0 f32, 1 f64, 2 f64 dual numbers, 3 dual numbers with f32 values
    Engine<float>* f;
    Engine<double>* d;
    Engine<Dual>* g;
    Engine<DualF>* gf;
};

#define DISPATCH(w, ...)                                       \
    do {                                                       \
        if ((w)->dbl == 3) { auto& E = *(w)->gf; __VA_ARGS__; } \
        else if ((w)->dbl == 2) { auto& E = *(w)->g; __VA_ARGS__; } \
        else if ((w)->dbl) { auto& E = *(w)->d; __VA_ARGS__; } \
        else { auto& E = *(w)->f; __VA_ARGS__; }                \
    } while (0)
// the dual-number engines only
#define DISPATCH_DUAL(w, ...)                                  \
    do {                                                       \
        if ((w)->dbl == 3) { auto& E = *(w)->gf; __VA_ARGS__; } \
        else { auto& E = *(w)->g; __VA_ARGS__; }                \
    } while (0)

extern "C" {

// mode: 0 = Reference, 1 = Coloured.  use_double: 0 = f32, 1 = f64, 2 = f64
// dual numbers (forward-mode derivatives), 3 = dual numbers whose values are
// the f32 engine's (its trajectory bit for bit) with f64 tangents.
OracleWorld* oracle_world_create(const AvbdParams* p, int mode, int use_double, int threads) {
    OracleWorld* w = new OracleWorld{use_double, nullptr, nullptr, nullptr, nullptr};
    auto init = [&](auto& E) {
        using TT = std::remove_reference_t<decltype(E.dt)>;
        E.prm = *p;
        E.mode = mode;
        E.threads = threads;
        E.gravity = {TT(p->gravity[0]), TT(p->gravity[1]), TT(p->gravity[2])};
        E.dt = TT(p->step_dt);
    };
    if (use_double == 3) { w->gf = new Engine<DualF>(); init(*w->gf); }
    else if (use_double == 2) { w->g = new Engine<Dual>(); init(*w->g); }
    else if (use_double) { w->d = new Engine<double>(); init(*w->d); }
    else { w->f = new Engine<float>(); init(*w->f); }
    return w;
}
void oracle_world_destroy(OracleWorld* w) {
    if (!w) return;
    delete w->f;
    delete w->d;
    delete w->g;
    delete w->gf;
    delete w;
}
void oracle_set_faithful_scan(OracleWorld* w, int on) { DISPATCH(w, E.faithful_scan = on != 0); }
void oracle_set_split_sums(OracleWorld* w, int on) { DISPATCH(w, E.split_sums = on != 0); }
int oracle_add_bodies(OracleWorld* w, const AvbdBody* b, uint32_t n) {
    DISPATCH(w, {
        using TT = std::remove_reference_t<decltype(E.dt)>;
        for (uint32_t i = 0; i < n; i++) {
            E.bodies.push_back(from_desc<TT>(b[i]));
            E.link_hull(E.bodies.back());
        }
    });
    return AVBD_OK;
}
// A convex hull (centroid-relative vertices, triangle faces as 3 indices,
// body-frame inertia per unit mass); bodies of shape AVBD_SHAPE_HULL name it
// by index in shape_params[0].  Returns the index.
int oracle_add_heightfield(OracleWorld* w, uint32_t rows, uint32_t cols, float cell, const float* heights,
                           uint32_t* id) {
    int rc = 0;
    uint32_t out = 0;
    DISPATCH(w, rc = E.add_hf(rows, cols, cell, heights, out));
    if (id) *id = out;
    return rc;
}
int oracle_add_trimesh(OracleWorld* w, const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt,
                       uint32_t* id) {
    int rc = 0;
    uint32_t out = 0;
    DISPATCH(w, rc = E.add_mesh(verts, nv, tris, nt, out));
    if (id) *id = out;
    return rc;
}
// Shape::try_round / try_compound over primitive parts (shape.rs:556-575).
int oracle_add_ext(OracleWorld* w, int compound, const AvbdShapePart* parts, uint32_t n, const float* unit_inertia,
                   uint32_t* id) {
    int rc = 0;
    uint32_t out = 0;
    DISPATCH(w, rc = E.add_ext(compound != 0, parts, n, unit_inertia, out));
    if (id) *id = out;
    return rc;
}
uint32_t oracle_add_hull(OracleWorld* w, const float* verts, uint32_t nv, const uint32_t* faces, uint32_t nf,
                         const float* unit_inertia) {
    uint32_t id = 0;
    DISPATCH(w, {
        using TT = std::remove_reference_t<decltype(E.dt)>;
        Hull<TT> h;
        for (uint32_t i = 0; i < nv; i++) h.verts.push_back({TT(verts[3 * i]), TT(verts[3 * i + 1]), TT(verts[3 * i + 2])});
        h.faces.assign(faces, faces + 3 * nf);
        h.unit_inertia = {TT(unit_inertia[0]), TT(unit_inertia[1]), TT(unit_inertia[2])};
        hull_measures(h);
        id = (uint32_t)E.hulls.size();
        E.hulls.push_back(std::move(h));
    });
    return id;
}
// Test hooks: the raw GJK/EPA query (gjk.rs:589-638) and the full
// shape_distance between bodies ia and ib.  out = dist, normal[3] (GJK only),
// pa[3], pb[3].
void oracle_convex_distance(OracleWorld* w, uint32_t ia, uint32_t ib, float* out) {
    DISPATCH(w, {
        auto g = convex_distance(sref(E.bodies[ia]), sref(E.bodies[ib]));
        float v[10] = {(float)g.dist, (float)g.normal.x, (float)g.normal.y, (float)g.normal.z, (float)g.pa.x,
                       (float)g.pa.y, (float)g.pa.z, (float)g.pb.x, (float)g.pb.y, (float)g.pb.z};
        std::memcpy(out, v, sizeof(v));
    });
}
void oracle_shape_distance(OracleWorld* w, uint32_t ia, uint32_t ib, float* out) {
    DISPATCH(w, {
        auto d = shape_distance_any(sref(E.bodies[ia]), sref(E.bodies[ib]));
        float v[10] = {(float)d.dist, 0.0f, 0.0f, 0.0f, (float)d.pa.x, (float)d.pa.y, (float)d.pa.z,
                       (float)d.pb.x, (float)d.pb.y, (float)d.pb.z};
        std::memcpy(out, v, sizeof(v));
    });
}
int oracle_remove_body(OracleWorld* w, uint32_t handle) {
    DISPATCH(w, E.remove_body(handle));
    return AVBD_OK;
}
// PhysicsEngine::remove_joint (mod.rs:1531-1540): wake both, then retain.
int oracle_remove_joint(OracleWorld* w, uint32_t handle) {
    DISPATCH(w, {
        if (handle < E.joints.size()) {
            E.wake_body(E.joints[handle].a);
            E.wake_body(E.joints[handle].b);
            std::vector<uint8_t> gone(E.joints.size(), 0);
            gone[handle] = 1;
            E.retain_joints(gone);
        }
    });
    return AVBD_OK;
}
// PhysicsEngine::wake_body (mod.rs:1599-1601)
int oracle_wake_body(OracleWorld* w, uint32_t handle) {
    DISPATCH(w, E.wake_body(handle));
    return AVBD_OK;
}
int oracle_add_joint(OracleWorld* w, const AvbdJointDesc* d, uint32_t* handle) {
    int rc = 0;
    DISPATCH(w, rc = E.add_joint(*d, *handle));
    return rc;
}
int oracle_step(OracleWorld* w, float dt) {
    DISPATCH(w, E.step(dt));
    return AVBD_OK;
}
int oracle_step_fixed(OracleWorld* w, int32_t nsub) {
    DISPATCH(w, E.step_fixed(nsub));
    return AVBD_OK;
}
// Substeps per emitting step for step_fixed: 0 = only the last substep of a call.
int oracle_set_emit_period(OracleWorld* w, int32_t period) {
    DISPATCH(w, E.emit_period = period < 0 ? 0 : period);
    return AVBD_OK;
}
// Move up to `cap` queued events out (oldest first); returns how many were moved.
uint32_t oracle_drain_contact_events(OracleWorld* w, AvbdContactEvent* out, uint32_t cap) {
    uint32_t n = 0;
    DISPATCH(w, {
        n = (uint32_t)std::min<size_t>(cap, E.cev.size());
        std::copy(E.cev.begin(), E.cev.begin() + n, out);
        E.cev.erase(E.cev.begin(), E.cev.begin() + n);
    });
    return n;
}
uint32_t oracle_drain_trigger_events(OracleWorld* w, AvbdTriggerEvent* out, uint32_t cap) {
    uint32_t n = 0;
    DISPATCH(w, {
        n = (uint32_t)std::min<size_t>(cap, E.tev.size());
        std::copy(E.tev.begin(), E.tev.begin() + n, out);
        E.tev.erase(E.tev.begin(), E.tev.begin() + n);
    });
    return n;
}
uint32_t oracle_body_count(OracleWorld* w) {
    uint32_t n = 0;
    DISPATCH(w, n = (uint32_t)E.bodies.size());
    return n;
}
int oracle_get_bodies(OracleWorld* w, AvbdBody* out) {
    DISPATCH(w, for (size_t i = 0; i < E.bodies.size(); i++) to_desc(E.bodies[i], out[i]));
    return AVBD_OK;
}
// Full-precision body poses/velocities as doubles: 13 per body (pos, quat, vel, angvel).
int oracle_get_state13(OracleWorld* w, double* out) {
    DISPATCH(w, for (size_t i = 0; i < E.bodies.size(); i++) {
        auto& b = E.bodies[i];
        double v[13] = {double(b.pos.x), double(b.pos.y), double(b.pos.z), double(b.rot.x), double(b.rot.y),
                        double(b.rot.z), double(b.rot.w), double(b.vel.x), double(b.vel.y), double(b.vel.z),
                        double(b.angvel.x), double(b.angvel.y), double(b.angvel.z)};
        std::memcpy(out + 13 * i, v, sizeof(v));
    });
    return AVBD_OK;
}
// ---- dual-number worlds (use_double = 2 or 3): forward-mode derivatives -------
static bool is_dual_world(const OracleWorld* w) { return w && (w->dbl == 2 || w->dbl == 3); }
int oracle_dual_dirs() { return DUAL_DIRS; }
// Seed d(field[comp] of body)/d(direction dir) = value.  field: 0 position,
// 1 rotation (x, y, z, w), 2 velocity, 3 angular velocity, 4 friction (both
// friction coefficients; comp ignored).
int oracle_dual_seed(OracleWorld* w, uint32_t body, int field, int comp, int dir, double value) {
    if (!is_dual_world(w) || dir < 0 || dir >= DUAL_DIRS) return AVBD_ERR_INVALID_ARG;
    int rc = AVBD_OK;
    DISPATCH_DUAL(w, {
        if (body >= E.bodies.size()) {
            rc = AVBD_ERR_INVALID_ARG;
        } else {
            auto& b = E.bodies[body];
            double* f = nullptr;
            switch (field) {
                case 0: f = comp == 0 ? b.pos.x.d : comp == 1 ? b.pos.y.d : b.pos.z.d; break;
                case 1: f = comp == 0 ? b.rot.x.d : comp == 1 ? b.rot.y.d : comp == 2 ? b.rot.z.d : b.rot.w.d; break;
                case 2: f = comp == 0 ? b.vel.x.d : comp == 1 ? b.vel.y.d : b.vel.z.d; break;
                case 3: f = comp == 0 ? b.angvel.x.d : comp == 1 ? b.angvel.y.d : b.angvel.z.d; break;
                case 4:
                    b.friction.d[dir] = value;
                    b.friction_t.d[dir] = value;
                    break;
                default: rc = AVBD_ERR_INVALID_ARG;
            }
            if (f) f[dir] = value;
        }
    });
    return rc;
}
// Finite joint stiffness (0: hard joints, the reference's).
int oracle_set_joint_stiffness(OracleWorld* w, float k) {
    if (!w || !(k >= 0.0f)) return AVBD_ERR_INVALID_ARG;
    DISPATCH(w, {
        using TT = std::remove_reference_t<decltype(E.dt)>;
        E.joint_k = TT(k);
    });
    return AVBD_OK;
}
// d(joint stiffness)/d(direction dir) = value (dual worlds).
int oracle_dual_seed_joint_stiffness(OracleWorld* w, int dir, double value) {
    if (!is_dual_world(w) || dir < 0 || dir >= DUAL_DIRS) return AVBD_ERR_INVALID_ARG;
    DISPATCH_DUAL(w, E.joint_k.d[dir] = value);
    return AVBD_OK;
}
int oracle_dual_freeze_frames(OracleWorld* w, int on) {
    if (!is_dual_world(w)) return AVBD_ERR_INVALID_ARG;
    DISPATCH_DUAL(w, {
        E.freeze_frames = on != 0;
        E.freeze_bits = on;
    });
    return AVBD_OK;
}
// Tangents of the 13 state numbers of every body: out[(13 * body + k) * DUAL_DIRS + dir].
int oracle_dual_tangents(OracleWorld* w, double* out) {
    if (!is_dual_world(w)) return AVBD_ERR_INVALID_ARG;
    DISPATCH_DUAL(w, {
        for (size_t i = 0; i < E.bodies.size(); i++) {
            auto& b = E.bodies[i];
            const double* v[13] = {b.pos.x.d, b.pos.y.d, b.pos.z.d, b.rot.x.d, b.rot.y.d, b.rot.z.d, b.rot.w.d,
                                   b.vel.x.d, b.vel.y.d, b.vel.z.d, b.angvel.x.d, b.angvel.y.d, b.angvel.z.d};
            for (int k = 0; k < 13; k++)
                for (int d = 0; d < DUAL_DIRS; d++) out[(13 * i + k) * DUAL_DIRS + d] = v[k][d];
        }
    });
    return AVBD_OK;
}
int oracle_set_bodies(OracleWorld* w, const AvbdBody* in, uint32_t n) {
    DISPATCH(w, {
        using TT = std::remove_reference_t<decltype(E.dt)>;
        if (n != E.bodies.size()) return AVBD_ERR_INVALID_ARG;
        for (uint32_t i = 0; i < n; i++) {
            E.bodies[i] = from_desc<TT>(in[i]);
            E.link_hull(E.bodies[i]);
        }
    });
    return AVBD_OK;
}
uint32_t oracle_joint_count(OracleWorld* w) {
    uint32_t n = 0;
    DISPATCH(w, n = (uint32_t)E.joints.size());
    return n;
}
uint32_t oracle_pair_count(OracleWorld* w) {
    uint32_t n = 0;
    DISPATCH(w, n = (uint32_t)E.pairs.size());
    return n;
}
int oracle_export_state(OracleWorld* w, AvbdBody* bodies, AvbdBodyAux* aux, AvbdPairState* pairs,
                        AvbdPointState* points, AvbdJointState* joints) {
    DISPATCH(w, {
        E.ensure_scratch();
        for (size_t i = 0; i < E.bodies.size(); i++) {
            if (bodies) to_desc(E.bodies[i], bodies[i]);
            if (aux) {
                auto& x = aux[i];
                x.prev_position[0] = float(E.prev_pos[i].x); x.prev_position[1] = float(E.prev_pos[i].y); x.prev_position[2] = float(E.prev_pos[i].z);
                x.prev_orientation[0] = float(E.prev_rot[i].x); x.prev_orientation[1] = float(E.prev_rot[i].y);
                x.prev_orientation[2] = float(E.prev_rot[i].z); x.prev_orientation[3] = float(E.prev_rot[i].w);
                x.sleep_timer = float(E.sleep_timer[i]);
                x.asleep = E.asleep[i];
            }
        }
        for (size_t i = 0; i < E.pairs.size(); i++) {
            auto& p = E.pairs[i];
            if (pairs) {
                auto& s = pairs[i];
                s.a = p.a; s.b = p.b;
                s.normal[0] = float(p.n.x); s.normal[1] = float(p.n.y); s.normal[2] = float(p.n.z);
                s.mu[0] = float(p.mu[0]); s.mu[1] = float(p.mu[1]);
                s.gap = float(p.gap);
                s.npoints = (uint32_t)p.points.size();
            }
            if (points) {
                for (int k = 0; k < AVBD_MAX_POINTS; k++) {
                    AvbdPointState& q = points[i * AVBD_MAX_POINTS + k];
                    std::memset(&q, 0, sizeof(q));
                    q.matched = -1;
                    if (k >= (int)p.points.size()) continue;
                    auto& pt = p.points[k];
                    for (int c = 0; c < 3; c++) {
                        q.ra[c] = float(pt.ra[c]); q.rb[c] = float(pt.rb[c]);
                        q.lam[c] = float(pt.lam[c]); q.pen[c] = float(pt.pen[c]); q.roll_lam[c] = float(pt.roll_lam[c]);
                    }
                    q.stuck = pt.stuck;
                    q.matched = pt.matched;
                }
            }
        }
        if (joints)
            for (size_t i = 0; i < E.joints.size(); i++) {
                auto& j = E.joints[i];
                auto& s = joints[i];
                for (int c = 0; c < 3; c++) {
                    s.lam_l[c] = float(j.lam_l[c]); s.lam_a[c] = float(j.lam_a[c]);
                    s.pen_l[c] = float(j.pen_l[c]); s.pen_a[c] = float(j.pen_a[c]);
                }
                s.acc_lim = float(j.acc_lim);
                s.lim_dual = float(j.lim_dual);
                for (int c = 0; c < 6; c++) s.sacc[c] = float(j.sacc[c]);
                for (int c = 0; c < 2; c++) {
                    s.gear_raw[c] = j.kind == AVBD_JOINT_GEAR ? float(j.graw[c]) : 0.0f;
                    s.gear_cont[c] = j.kind == AVBD_JOINT_GEAR ? float(j.gcont[c]) : 0.0f;
                }
                s.gear_mem_set = j.kind == AVBD_JOINT_GEAR && j.gmem_set ? 1u : 0u;
            }
    });
    return AVBD_OK;
}
int oracle_import_state(OracleWorld* w, const AvbdBody* bodies, const AvbdBodyAux* aux, const AvbdPairState* pairs,
                        const AvbdPointState* points, uint32_t npairs, const AvbdJointState* joints) {
    DISPATCH(w, {
        using TT = std::remove_reference_t<decltype(E.dt)>;
        E.ensure_scratch();
        size_t n = E.bodies.size();
        for (size_t i = 0; i < n; i++) {
            if (bodies) {
                E.bodies[i] = from_desc<TT>(bodies[i]);
                E.link_hull(E.bodies[i]);
            }
            if (aux) {
                E.prev_pos[i] = {TT(aux[i].prev_position[0]), TT(aux[i].prev_position[1]), TT(aux[i].prev_position[2])};
                E.prev_rot[i] = {TT(aux[i].prev_orientation[0]), TT(aux[i].prev_orientation[1]),
                                 TT(aux[i].prev_orientation[2]), TT(aux[i].prev_orientation[3])};
                E.sleep_timer[i] = TT(aux[i].sleep_timer);
                E.asleep[i] = aux[i].asleep ? 1 : 0;
            }
        }
        if (pairs) {
            E.pairs.clear();
            for (uint32_t i = 0; i < npairs; i++) {
                Pair<TT> p;
                p.a = pairs[i].a; p.b = pairs[i].b;
                p.n = {TT(pairs[i].normal[0]), TT(pairs[i].normal[1]), TT(pairs[i].normal[2])};
                p.mu[0] = TT(pairs[i].mu[0]); p.mu[1] = TT(pairs[i].mu[1]);
                p.gap = TT(pairs[i].gap);
                for (uint32_t k = 0; k < pairs[i].npoints && k < AVBD_MAX_POINTS; k++) {
                    const AvbdPointState& q = points[i * AVBD_MAX_POINTS + k];
                    Point<TT> pt{};
                    for (int c = 0; c < 3; c++) {
                        pt.ra[c] = TT(q.ra[c]); pt.rb[c] = TT(q.rb[c]);
                        pt.lam[c] = TT(q.lam[c]); pt.pen[c] = TT(q.pen[c]); pt.roll_lam[c] = TT(q.roll_lam[c]);
                    }
                    pt.stuck = q.stuck != 0;
                    pt.matched = q.matched;
                    p.points.push_back(pt);
                }
                E.pairs.push_back(std::move(p));
            }
        }
        if (joints)
            for (size_t i = 0; i < E.joints.size(); i++) {
                auto& j = E.joints[i];
                for (int c = 0; c < 3; c++) {
                    j.lam_l[c] = TT(joints[i].lam_l[c]); j.lam_a[c] = TT(joints[i].lam_a[c]);
                    j.pen_l[c] = TT(joints[i].pen_l[c]); j.pen_a[c] = TT(joints[i].pen_a[c]);
                }
                j.acc_lim = TT(joints[i].acc_lim);
                j.lim_dual = TT(joints[i].lim_dual);
                for (int c = 0; c < 6; c++) j.sacc[c] = TT(joints[i].sacc[c]);
                if (j.kind == AVBD_JOINT_GEAR) {
                    for (int c = 0; c < 2; c++) {
                        j.graw[c] = TT(joints[i].gear_raw[c]);
                        j.gcont[c] = TT(joints[i].gear_cont[c]);
                    }
                    j.gmem_set = joints[i].gear_mem_set != 0;
                }
            }
    });
    return AVBD_OK;
}
int oracle_get_colours(OracleWorld* w, int32_t* out) {
    DISPATCH(w, for (size_t i = 0; i < E.bodies.size(); i++) out[i] = i < E.colour.size() ? E.colour[i] : -1);
    return AVBD_OK;
}
int oracle_get_counters(OracleWorld* w, AvbdCounters* c) {
    std::memset(c, 0, sizeof(*c));
    DISPATCH(w, {
        c->steps = E.steps;
        c->pairs = E.pairs.size();
        uint64_t pts = 0;
        for (auto& p : E.pairs) pts += p.points.size();
        c->points = pts;
        c->colours = E.ncolours;
        c->breakdowns = E.breakdowns;
        c->ccd_hits = E.ccd_hits;
        uint64_t sl = 0;
        for (auto s : E.asleep) sl += s;
        c->sleeping = sl;
    });
    return AVBD_OK;
}

// ---- row-level known-answer hooks (gpu_batches.rs:781-898) ----
void oracle_stamp_row(float* lhs36, float* rhs6, const float* axis, float pen, float f, const float* lever, float sign) {
    float lhs[6][6], rhs[6];
    std::memcpy(lhs, lhs36, sizeof(lhs));
    std::memcpy(rhs, rhs6, sizeof(rhs));
    stamp_row<float>(lhs, rhs, {axis[0], axis[1], axis[2]}, pen, f, {lever[0], lever[1], lever[2]}, sign);
    std::memcpy(lhs36, lhs, sizeof(lhs));
    std::memcpy(rhs6, rhs, sizeof(rhs));
}
int oracle_solve_6x6(const float* lhs36, const float* rhs6, float* x6) {
    float lhs[6][6];
    std::memcpy(lhs, lhs36, sizeof(lhs));
    bool ok = solve_6x6<float>(lhs, rhs6, x6);
    if (!ok)
        for (int i = 0; i < 6; i++) x6[i] = 0.0f;
    return ok ? 1 : 0;
}
void oracle_tangent_basis(const float* n, float* t1, float* t2) {
    V3<float> a, b;
    tangent_basis<float>({n[0], n[1], n[2]}, a, b);
    t1[0] = a.x; t1[1] = a.y; t1[2] = a.z;
    t2[0] = b.x; t2[1] = b.y; t2[2] = b.z;
}
void oracle_shape_inertia(uint32_t shape, const float* sp, float mass, float* out) {
    V3<float> r = shape_inertia<float>(shape, {sp[0], sp[1], sp[2]}, mass);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
uint32_t oracle_colour_hash(uint32_t x) { return colour_hash(x); }

// Unit-test hooks mirroring the reference's in-module tests
// (avbd/contact_tests.rs:38-96): pos0/rot0 = current poses, then one
// generate_pairs pass; gap_c0 of point qi of pair pi.
int oracle_generate_pairs(OracleWorld* w) {
    DISPATCH(w, {
        E.ensure_scratch();
        for (size_t h = 0; h < E.bodies.size(); h++) { E.pos0[h] = E.bodies[h].pos; E.rot0[h] = E.bodies[h].rot; }
        E.generate_pairs();
    });
    return AVBD_OK;
}
double oracle_gap_c0(OracleWorld* w, uint32_t pi, uint32_t qi) {
    double r = 0.0;
    DISPATCH(w, r = (double)E.gap_c0(E.pairs[pi], E.pairs[pi].points[qi]));
    return r;
}

// RigidBody constructors (body.rs:346-376, :470-576, :873-889): default
// materials per shape and the mass triple of Mass::from_kind
// (invariants.rs:175-199).
int oracle_body_new(uint32_t shape, const float* params, const float* position, float mass, AvbdBody* out) {
    std::memset(out, 0, sizeof(*out));
    float rest = 0.3f, fric = 0.5f;
    float sp[3] = {params[0], params[1], params[2]};
    if (shape == AVBD_SHAPE_SPHERE) { rest = 0.5f; fric = 0.3f; }
    else if (shape == AVBD_SHAPE_CAPSULE || shape == AVBD_SHAPE_CYLINDER) { rest = 0.4f; fric = 0.4f; }  // body.rs:580-591
    else if (shape == AVBD_SHAPE_CONE) { rest = 0.3f; fric = 0.5f; }  // body.rs:596-607
    else if (shape == AVBD_SHAPE_HALFSPACE) {
        if (mass > 0.0f && std::isfinite(mass)) return AVBD_ERR_INVALID_ARG;
        V3<float> nn = normalize_or(V3<float>{sp[0], sp[1], sp[2]}, VZERO<float>());
        if (nn == VZERO<float>()) return AVBD_ERR_INVALID_ARG;
        sp[0] = nn.x; sp[1] = nn.y; sp[2] = nn.z;
        rest = 0.3f; fric = 0.6f;
    } else if (shape != AVBD_SHAPE_BOX) {
        return AVBD_ERR_UNSUPPORTED;
    }
    bool free = mass > 0.0f && std::isfinite(mass);
    for (int i = 0; i < 3; i++) out->position[i] = position[i];
    out->orientation[3] = 1.0f;
    out->mass = free ? mass : 0.0f;
    out->inv_mass = free ? 1.0f / mass : 0.0f;
    V3<float> in = shape_inertia<float>(shape, {sp[0], sp[1], sp[2]}, free ? mass : 0.0f);
    out->inertia[0] = in.x; out->inertia[1] = in.y; out->inertia[2] = in.z;
    out->restitution = rest;
    out->friction = fric;
    out->friction_transverse = fric;
    out->shape = shape;
    for (int i = 0; i < 3; i++) out->shape_params[i] = sp[i];
    out->collision_layer = 1;
    out->collision_mask = 0xffffffffu;
    out->body_type = mass > 0.0f ? AVBD_BODY_DYNAMIC : AVBD_BODY_STATIC;
    out->flags = 0;
    return AVBD_OK;
}

}  // extern "C"
