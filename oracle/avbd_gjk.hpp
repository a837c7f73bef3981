// avbd_gjk.hpp — CPU restatement (oracle, test infrastructure only) of the
// reference's convex narrowphase for cylinders, cones and convex hulls:
// support functions (collision/gjk.rs:68-186), GJK separation (:200-356),
// simplex reduction (:358-458), EPA penetration (:460-587), the full query
// (:589-638), the witness re-seating pass (collision/distance.rs:364-421) and
// the closest-point queries it uses (collision/shape.rs:955-1215).
// Included by avbd_oracle.cpp after the analytic shape routines.
#pragma once

namespace gjk {
constexpr float DEGENERATE_EPS = 1e-12f;
constexpr float PROGRESS_EPS = 1e-6f;
constexpr float STALL_DIST = 1e-6f;
constexpr float TET_VOLUME_EPS = 1e-9f;
constexpr float EPA_VISIBLE_EPS = 1e-9f;
constexpr size_t EPA_MAX_VERTS = 128;
constexpr size_t EPA_MAX_FACES = 64;
constexpr float COINCIDENT_LEN2 = 1e-18f;
constexpr float NEAR_ZERO = 1e-9f;
constexpr float SHAPE_TOUCH = 1e-3f;
}  // namespace gjk

// support point of any convex shape of the path along world `dir`
template <class T> static V3<T> support_any(const ShapeRef<T>& s, V3<T> dir) {
    const V3<T> pos = s.pos;
    const Qt<T> rot = s.rot;
    switch (s.shape) {
        case AVBD_SHAPE_CYLINDER: {
            T radius = s.sp.x, hh = s.sp.y;
            V3<T> axis = qrot(rot, VY<T>());
            T along = dot(dir, axis);
            V3<T> cap = axis * (along >= T(0) ? hh : -hh);
            V3<T> radial = dir - axis * along;
            V3<T> rim = len2(radial) > C<T>(gjk::DEGENERATE_EPS) ? normalize(radial) * radius : VZERO<T>();
            return pos + cap + rim;
        }
        case AVBD_SHAPE_CONE: {
            T radius = s.sp.x, hh = s.sp.y;
            V3<T> axis = qrot(rot, VY<T>());
            V3<T> apex = pos + axis * hh;
            V3<T> base = pos - axis * hh;
            T along = dot(dir, axis);
            V3<T> radial = dir - axis * along;
            V3<T> rim = len2(radial) > C<T>(gjk::DEGENERATE_EPS) ? base + normalize(radial) * radius : base;
            return dot(dir, apex) >= dot(dir, rim) ? apex : rim;
        }
        case AVBD_SHAPE_HULL: {
            V3<T> best = pos;
            T best_d = -std::numeric_limits<T>::max();
            if (s.hull)
                for (const V3<T>& v : s.hull->verts) {
                    V3<T> w = pos + qrot(rot, v);
                    T d = dot(w, dir);
                    if (d > best_d) {
                        best_d = d;
                        best = w;
                    }
                }
            return best;
        }
        case AVBD_SHAPE_HEIGHTFIELD:
        case AVBD_SHAPE_TRIMESH:
            return pos;  // no support of its own (gjk.rs:141-155): its origin
        default:
            return support(s.shape, s.sp, pos, rot, dir);
    }
}

template <class T> struct SVert {
    V3<T> v, sa, sb;
};
template <class T> static SVert<T> minkowski(const ShapeRef<T>& a, const ShapeRef<T>& b, V3<T> dir) {
    V3<T> sa = support_any(a, dir);
    V3<T> sb = support_any(b, -dir);
    return {sa - sb, sa, sb};
}
template <class T> static V3<T> closest_segment(V3<T> p, V3<T> q, T& wp, T& wq) {
    V3<T> pq = q - p;
    T l2 = len2(pq);
    if (l2 < C<T>(gjk::COINCIDENT_LEN2)) {
        wp = T(1);
        wq = T(0);
        return p;
    }
    T t = fclamp(-dot(p, pq) / l2, T(0), T(1));
    wp = T(1) - t;
    wq = t;
    return p + pq * t;
}
// gjk.rs:220-265 (Ericson, Real-Time Collision Detection 5.1.5)
template <class T> static V3<T> closest_triangle(V3<T> a, V3<T> b, V3<T> c, T& wa, T& wb, T& wc) {
    V3<T> ab = b - a, ac = c - a, ap = -a;
    T d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= T(0) && d2 <= T(0)) { wa = T(1); wb = T(0); wc = T(0); return a; }
    V3<T> bp = -b;
    T d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= T(0) && d4 <= d3) { wa = T(0); wb = T(1); wc = T(0); return b; }
    T vc = d1 * d4 - d3 * d2;
    if (vc <= T(0) && d1 >= T(0) && d3 <= T(0)) {
        T v = d1 / (d1 - d3);
        wa = T(1) - v; wb = v; wc = T(0);
        return a + ab * v;
    }
    V3<T> cp = -c;
    T d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= T(0) && d5 <= d6) { wa = T(0); wb = T(0); wc = T(1); return c; }
    T vb = d5 * d2 - d1 * d6;
    if (vb <= T(0) && d2 >= T(0) && d6 <= T(0)) {
        T w = d2 / (d2 - d6);
        wa = T(1) - w; wb = T(0); wc = w;
        return a + ac * w;
    }
    T va = d3 * d6 - d5 * d4;
    if (va <= T(0) && (d4 - d3) >= T(0) && (d5 - d6) >= T(0)) {
        T w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        wa = T(0); wb = T(1) - w; wc = w;
        return b + (c - b) * w;
    }
    T denom = T(1) / (va + vb + vc);
    T v = vb * denom, w = vc * denom;
    wa = T(1) - v - w; wb = v; wc = w;
    return a + ab * v + ac * w;
}

// reduce_simplex / reduce_tetra (gjk.rs:358-458): closest point, keep mask,
// weights aligned with the input order; an enclosing tetrahedron keeps none.
template <class T> static V3<T> reduce_simplex(const SVert<T>* s, int n, bool keep[4], T w[4]) {
    for (int i = 0; i < 4; i++) { keep[i] = false; w[i] = T(0); }
    if (n == 1) { keep[0] = true; w[0] = T(1); return s[0].v; }
    if (n == 2) {
        V3<T> p = closest_segment(s[0].v, s[1].v, w[0], w[1]);
        keep[0] = w[0] > T(0); keep[1] = w[1] > T(0);
        return p;
    }
    if (n == 3) {
        V3<T> p = closest_triangle(s[0].v, s[1].v, s[2].v, w[0], w[1], w[2]);
        keep[0] = w[0] > T(0); keep[1] = w[1] > T(0); keep[2] = w[2] > T(0);
        return p;
    }
    V3<T> e1 = s[1].v - s[0].v, e2 = s[2].v - s[0].v, e3 = s[3].v - s[0].v;
    T vol = std::fabs(dot(e1, cross(e2, e3)));
    T scale = len(e1) * len(e2) * len(e3);
    bool have = false;
    V3<T> bp{};
    T bg = T(0), bw[4] = {T(0), T(0), T(0), T(0)};
    if (vol <= C<T>(gjk::TET_VOLUME_EPS) * fmx(scale, C<T>(gjk::COINCIDENT_LEN2))) {
        static const int F[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
        for (const auto& f : F) {
            T wa, wb, wc;
            V3<T> p = closest_triangle(s[f[0]].v, s[f[1]].v, s[f[2]].v, wa, wb, wc);
            T gap = len(p);
            if (!have || gap < bg) {
                have = true; bp = p; bg = gap;
                for (T& x : bw) x = T(0);
                bw[f[0]] = wa; bw[f[1]] = wb; bw[f[2]] = wc;
            }
        }
        for (int i = 0; i < 4; i++) { w[i] = bw[i]; keep[i] = bw[i] > T(0); }
        return bp;
    }
    static const int FF[4][4] = {{0, 1, 2, 3}, {0, 3, 1, 2}, {0, 2, 3, 1}, {1, 3, 2, 0}};
    for (const auto& f : FF) {
        T wa, wb, wc;
        V3<T> p = closest_triangle(s[f[0]].v, s[f[1]].v, s[f[2]].v, wa, wb, wc);
        T gap = len(p);
        if (!have || gap < bg) {
            have = true; bp = p; bg = gap;
            for (T& x : bw) x = T(0);
            bw[f[0]] = wa; bw[f[1]] = wb; bw[f[2]] = wc;
        }
    }
    bool inside = true;
    for (const auto& f : FF) {
        V3<T> nn = cross(s[f[1]].v - s[f[0]].v, s[f[2]].v - s[f[0]].v);
        if (dot(nn, s[f[3]].v - s[f[0]].v) > T(0)) nn = -nn;
        if (dot(nn, -s[f[0]].v) > T(0)) { inside = false; break; }
    }
    if (inside) return VZERO<T>();
    for (int i = 0; i < 4; i++) { w[i] = bw[i]; keep[i] = bw[i] > T(0); }
    return bp;
}

template <class T> struct GjkDist {
    T dist;
    V3<T> normal, pa, pb;
};
// gjk.rs:267-356: separation, or false when the origin is enclosed / touching
template <class T> static bool gjk_separated(const ShapeRef<T>& a, const ShapeRef<T>& b, GjkDist<T>& out) {
    V3<T> dir = a.pos - b.pos;
    if (len2(dir) < C<T>(gjk::COINCIDENT_LEN2)) dir = VX<T>();
    SVert<T> simplex[4];
    SVert<T> first = minkowski(a, b, dir);
    for (auto& v : simplex) v = first;
    int count = 1;
    T weights[4] = {T(1), T(0), T(0), T(0)};
    V3<T> closest = simplex[0].v;
    if (len2(closest) < C<T>(gjk::COINCIDENT_LEN2)) {
        out = {T(0), normalize_or(b.pos - a.pos, VY<T>()), simplex[0].sa, simplex[0].sb};
        return true;
    }
    auto blend = [&](GjkDist<T>& r) {
        V3<T> pa = VZERO<T>(), pb = VZERO<T>();
        for (int i = 0; i < count; i++) {
            pa = pa + simplex[i].sa * weights[i];
            pb = pb + simplex[i].sb * weights[i];
        }
        V3<T> delta = pa - pb;
        r = {len(delta), normalize_or(delta, normalize_or(b.pos - a.pos, VY<T>())), pa, pb};
        return len(delta);
    };
    for (int it = 0; it < 64; it++) {
        dir = -closest;
        SVert<T> w = minkowski(a, b, dir);
        if (dot(w.v, dir) - dot(closest, dir) <= C<T>(gjk::PROGRESS_EPS) * fmx(len2(closest), T(1))) {
            GjkDist<T> r;
            T d = blend(r);
            if (d <= C<T>(gjk::STALL_DIST)) return false;
            out = r;
            return true;
        }
        simplex[count] = w;
        count++;
        bool keep[4];
        T wts[4];
        V3<T> next = reduce_simplex(simplex, count, keep, wts);
        int nc = 0;
        for (int i = 0; i < 4; i++)
            if (keep[i]) {
                simplex[nc] = simplex[i];
                weights[nc] = wts[i];
                nc++;
            }
        count = nc;
        if (count == 0 || len2(next) <= C<T>(gjk::DEGENERATE_EPS)) return false;
        closest = next;
    }
    blend(out);
    return true;
}

// gjk.rs:460-587
template <class T> static void epa(const ShapeRef<T>& a, const ShapeRef<T>& b, const SVert<T> tet[4], T& depth,
                                   V3<T>& normal, V3<T>& pa, V3<T>& pb) {
    std::vector<SVert<T>> verts(tet, tet + 4);
    std::vector<std::array<size_t, 3>> faces = {{0, 2, 1}, {0, 3, 2}, {0, 1, 3}, {1, 2, 3}};
    auto fnorm = [&](const std::array<size_t, 3>& f) {
        return cross(verts[f[1]].v - verts[f[0]].v, verts[f[2]].v - verts[f[0]].v);
    };
    for (auto& f : faces) {
        V3<T> nn = fnorm(f);
        size_t apex = 0;
        bool found = false;
        for (size_t i = 0; i < verts.size(); i++)
            if (i != f[0] && i != f[1] && i != f[2]) { apex = i; found = true; break; }
        if (found && dot(nn, verts[apex].v - verts[f[0]].v) > T(0)) std::swap(f[1], f[2]);
    }
    depth = T(0);
    normal = VX<T>();
    pa = a.pos;
    pb = b.pos;
    const T fmax_ = std::numeric_limits<T>::max();
    for (int it = 0; it < 32; it++) {
        if (faces.empty() || faces.size() > gjk::EPA_MAX_FACES) break;
        size_t bi = 0;
        T bdist = fmax_;
        V3<T> bnormal = VX<T>();
        for (size_t i = 0; i < faces.size(); i++) {
            V3<T> nn = fnorm(faces[i]);
            T l = len(nn);
            if (l < C<T>(gjk::COINCIDENT_LEN2)) continue;
            nn = nn / l;
            T d = dot(nn, verts[faces[i][0]].v);
            if (d < bdist) { bdist = d; bnormal = nn; bi = i; }
        }
        SVert<T> w = minkowski(a, b, bnormal);
        if (dot(w.v, bnormal) - bdist <= C<T>(1e-6f) * fmx(bdist, T(1))) {
            const auto& f = faces[bi];
            T wa, wb, wc;
            closest_triangle(verts[f[0]].v, verts[f[1]].v, verts[f[2]].v, wa, wb, wc);
            pa = verts[f[0]].sa * wa + verts[f[1]].sa * wb + verts[f[2]].sa * wc;
            pb = verts[f[0]].sb * wa + verts[f[1]].sb * wb + verts[f[2]].sb * wc;
            depth = fmx(bdist, T(0));
            normal = bnormal;
            return;
        }
        std::vector<uint8_t> visible(faces.size(), 0);
        for (size_t i = 0; i < faces.size(); i++) {
            V3<T> nn = fnorm(faces[i]);
            T l = len(nn);
            if (l < C<T>(gjk::COINCIDENT_LEN2)) continue;
            if (dot(nn / l, w.v - verts[faces[i][0]].v) > C<T>(gjk::EPA_VISIBLE_EPS)) visible[i] = 1;
        }
        std::vector<std::pair<size_t, size_t>> edges, horizon;
        for (size_t i = 0; i < faces.size(); i++) {
            if (!visible[i]) continue;
            for (int e = 0; e < 3; e++) edges.push_back({faces[i][e], faces[i][(e + 1) % 3]});
        }
        for (const auto& e : edges) {
            size_t twin = 0;
            for (const auto& o : edges)
                if (o.first == e.second && o.second == e.first) twin++;
            if (twin == 0) horizon.push_back(e);
        }
        if (bdist < fmax_) {
            depth = fmx(bdist, T(0));
            normal = bnormal;
            pa = a.pos;
            pb = b.pos;
        }
        if (horizon.size() > faces.size()) break;
        std::vector<std::array<size_t, 3>> kept;
        for (size_t i = 0; i < faces.size(); i++)
            if (!visible[i]) kept.push_back(faces[i]);
        faces.swap(kept);
        size_t wi = verts.size();
        verts.push_back(w);
        for (const auto& e : horizon) faces.push_back({e.first, e.second, wi});
        V3<T> centroid = VZERO<T>();
        for (const auto& v : verts) centroid = centroid + v.v;
        centroid = centroid / T(verts.size());
        for (auto& f : faces) {
            V3<T> nn = fnorm(f);
            if (dot(nn, centroid - verts[f[0]].v) > T(0)) std::swap(f[1], f[2]);
        }
        if (verts.size() > gjk::EPA_MAX_VERTS) break;
    }
}

// gjk.rs:589-638
template <class T> static GjkDist<T> convex_distance(const ShapeRef<T>& a, const ShapeRef<T>& b) {
    GjkDist<T> sep;
    if (gjk_separated(a, b, sep)) return sep;
    const V3<T> dirs[6] = {VX<T>(), -VX<T>(), VY<T>(), -VY<T>(), VZ<T>(), -VZ<T>()};
    SVert<T> tet[4];
    SVert<T> x0 = minkowski(a, b, VX<T>());
    for (auto& t : tet) t = x0;
    int found = 0;
    for (const V3<T>& d : dirs) {
        SVert<T> w = minkowski(a, b, d);
        bool fresh = true;
        for (int i = 0; i < found; i++)
            if (!(len2(tet[i].v - w.v) > C<T>(gjk::DEGENERATE_EPS))) fresh = false;
        if (fresh && found < 4) tet[found++] = w;
        if (found == 4) break;
    }
    if (found < 4) return {T(0), normalize_or(b.pos - a.pos, VY<T>()), a.pos, b.pos};
    T depth;
    V3<T> normal, pa, pb;
    epa(a, b, tet, depth, normal, pa, pb);
    return {-depth, normal, pa, pb};
}

// Shape::closest_point (shape.rs:955-993) and its per-shape helpers.
template <class T> static V3<T> closest_point_local(const ShapeRef<T>& s, V3<T> p) {
    switch (s.shape) {
        case AVBD_SHAPE_SPHERE: return normalize_or(p, VX<T>()) * s.sp.x;
        case AVBD_SHAPE_BOX: {  // shape.rs:1098-1116
            V3<T> h = s.sp;
            V3<T> c = vclamp(p, -h, h);
            if (len2(c - p) > C<T>(gjk::COINCIDENT_LEN2)) return c;
            T dx = h.x - std::fabs(p.x), dy = h.y - std::fabs(p.y), dz = h.z - std::fabs(p.z);
            if (dx < dy && dx < dz) return {std::copysign(h.x, p.x), p.y, p.z};
            if (dy < dz) return {p.x, std::copysign(h.y, p.y), p.z};
            return {p.x, p.y, std::copysign(h.z, p.z)};
        }
        case AVBD_SHAPE_CAPSULE: {
            T core = fclamp(p.y, -s.sp.y, s.sp.y);
            V3<T> axis{T(0), core, T(0)};
            return axis + normalize_or(p - axis, VX<T>()) * s.sp.x;
        }
        case AVBD_SHAPE_CYLINDER: {  // shape.rs:1118-1153
            T radius = s.sp.x, hh = s.sp.y;
            T l = std::sqrt(p.x * p.x + p.z * p.z);
            V3<T> wall = l > C<T>(gjk::NEAR_ZERO)
                             ? V3<T>{p.x / l * radius, fclamp(p.y, -hh, hh), p.z / l * radius}
                             : V3<T>{radius, fclamp(p.y, -hh, hh), T(0)};
            T sc = l > C<T>(gjk::NEAR_ZERO) ? fmn(radius / l, T(1)) : T(0);
            V3<T> top{p.x * sc, hh, p.z * sc}, bottom{p.x * sc, -hh, p.z * sc};
            if (len2(p - wall) < len2(p - top) && len2(p - wall) < len2(p - bottom)) return wall;
            if (len2(p - top) < len2(p - bottom)) return top;
            return bottom;
        }
        case AVBD_SHAPE_CONE: {  // shape.rs:1155-1189
            T radius = s.sp.x, hh = s.sp.y;
            if (hh <= C<T>(gjk::NEAR_ZERO)) return {fclamp(p.x, -radius, radius), T(0), fclamp(p.z, -radius, radius)};
            T l = std::sqrt(p.x * p.x + p.z * p.z);
            T yc = fclamp(p.y, -hh, hh);
            T r_at = radius * (hh - yc) / (T(2) * hh);
            V3<T> wall = l > C<T>(gjk::NEAR_ZERO) ? V3<T>{p.x / l * r_at, yc, p.z / l * r_at} : V3<T>{r_at, yc, T(0)};
            T sc = l > C<T>(gjk::NEAR_ZERO) ? fmn(radius / l, T(1)) : T(0);
            V3<T> base{p.x * sc, -hh, p.z * sc}, apex{T(0), hh, T(0)};
            V3<T> best = wall;
            T bd = len2(p - wall);
            for (const V3<T>& c : {base, apex}) {
                T d = len2(p - c);
                if (d < bd) { best = c; bd = d; }
            }
            return best;
        }
        case AVBD_SHAPE_HULL: {  // shape.rs:1191-1215
            const Hull<T>* h = s.hull;
            if (!h || h->faces.empty()) {
                if (!h || h->verts.empty()) return VZERO<T>();
                V3<T> sum = VZERO<T>();
                for (const V3<T>& v : h->verts) sum = sum + v;
                return sum / T(h->verts.size());
            }
            V3<T> best = h->verts[h->faces[0]];
            T bd = len2(p - best);
            for (size_t f = 0; f + 2 < h->faces.size(); f += 3) {
                V3<T> a = h->verts[h->faces[f]], b = h->verts[h->faces[f + 1]], c = h->verts[h->faces[f + 2]];
                T wa, wb, wc;
                V3<T> q = closest_triangle(a - p, b - p, c - p, wa, wb, wc) + p;
                T d = len2(p - q);
                if (d < bd) { best = q; bd = d; }
            }
            return best;
        }
        default:
            return p;
    }
}
template <class T> static V3<T> closest_point_world(const ShapeRef<T>& s, V3<T> p) {
    V3<T> local = qrot(conj(s.rot), p - s.pos);
    return s.pos + qrot(s.rot, closest_point_local(s, local));
}

// distance.rs:364-421
template <class T> static Dist<T> refine_witnesses(const ShapeRef<T>& a, const ShapeRef<T>& b, T dist, V3<T> normal,
                                                   V3<T> pa, V3<T> pb) {
    if (!std::isfinite(dist)) return {dist, pa, pb};
    V3<T> n = len2(normal) > C<T>(gjk::COINCIDENT_LEN2) ? normalize(normal) : normalize_or(b.pos - a.pos, VY<T>());
    T depth = -dist;
    if (dist < C<T>(gjk::SHAPE_TOUCH)) {
        pa = a.pos;
        pb = b.pos;
    }
    for (int k = 0; k < 2; k++) {
        pb = closest_point_world(b, pa - n * depth);
        pa = closest_point_world(a, pb - n * depth);
        V3<T> axis = pb - pa;
        if (len2(axis) > C<T>(gjk::COINCIDENT_LEN2)) n = normalize(axis);
    }
    return {dist, pa, pb};
}

template <class T> static bool gjk_shape(uint32_t s) {
    return s == AVBD_SHAPE_CYLINDER || s == AVBD_SHAPE_CONE || s == AVBD_SHAPE_HULL;
}
template <class T> static Dist<T> gjk_pair_distance(const ShapeRef<T>& a, const ShapeRef<T>& b) {
    GjkDist<T> g = convex_distance(a, b);
    return refine_witnesses(a, b, g.dist, g.normal, g.pa, g.pb);
}
