// avbd_gjk.cuh — convex narrowphase for cylinders, cones and convex hulls:
// support functions (collision/gjk.rs:68-186), GJK separation (:200-356),
// simplex reduction (:358-458), EPA penetration (:460-587), the full query
// (:589-638), the witness re-seating pass (collision/distance.rs:364-421) and
// the closest-point queries it uses (collision/shape.rs:955-1215).
//
// One thread runs one query.  The EPA polytope lives in per-thread arrays
// bounded by the reference's own caps: at most 4 + 32 vertices (one per
// iteration) and 128 faces (64 at the top of an iteration plus a horizon no
// longer than the face list), so nothing is allocated.  Included by
// avbd_shapes.cuh; the arithmetic order follows the reference's so the exact
// build matches the CPU oracle.
// This header is included by avbd_shapes.cuh inside namespace avbd.
#pragma once

namespace gjk {
constexpr float DEGENERATE_EPS = 1e-12f;
constexpr float PROGRESS_EPS = 1e-6f;
constexpr float STALL_DIST = 1e-6f;
constexpr float TET_VOLUME_EPS = 1e-9f;
constexpr float EPA_VISIBLE_EPS = 1e-9f;
constexpr int EPA_MAX_VERTS = 128;
constexpr int EPA_MAX_FACES = 64;
constexpr int EPA_ITERS = 32;
constexpr int EPA_VERT_CAP = 4 + EPA_ITERS;
constexpr int EPA_FACE_CAP = 2 * EPA_MAX_FACES;
constexpr float COINCIDENT_LEN2 = 1e-18f;
constexpr float GJK_NEAR_ZERO = 1e-9f;
}  // namespace gjk

static __device__ __forceinline__ bool gjk_shape(uint32_t k) {
    return k == AVBD_SHAPE_CYLINDER || k == AVBD_SHAPE_CONE || k == AVBD_SHAPE_HULL;
}

// support point of the convex shapes that only this path handles
static __device__ __noinline__ V3 support_convex(const Shape& s, V3 dir) {
    if (s.kind == AVBD_SHAPE_CYLINDER) {
        V3 axis = qrot(s.rot, VY());
        float along = dot(dir, axis);
        V3 cap = axis * (along >= 0.0f ? s.p.y : -s.p.y);
        V3 radial = dir - axis * along;
        V3 rim = len2(radial) > gjk::DEGENERATE_EPS ? normalize(radial) * s.p.x : V0();
        return s.pos + cap + rim;
    }
    if (s.kind == AVBD_SHAPE_CONE) {
        V3 axis = qrot(s.rot, VY());
        V3 apex = s.pos + axis * s.p.y;
        V3 base = s.pos - axis * s.p.y;
        float along = dot(dir, axis);
        V3 radial = dir - axis * along;
        V3 rim = len2(radial) > gjk::DEGENERATE_EPS ? base + normalize(radial) * s.p.x : base;
        return dot(dir, apex) >= dot(dir, rim) ? apex : rim;
    }
    // hull: first maximum over the vertices in index order
    V3 best = s.pos;
    float best_d = -FLT_MAX;
    if (s.hull)
        for (uint32_t i = 0; i < s.hull->nv; i++) {
            V3 w = s.pos + qrot(s.rot, ld3(s.hull->v[i]));
            float d = dot(w, dir);
            if (d > best_d) {
                best_d = d;
                best = w;
            }
        }
    return best;
}
static __device__ __forceinline__ V3 support_any(const Shape& s, V3 dir) {
    // terrain and meshes have no support of their own (gjk.rs:141-155): the origin
    if (s.kind == AVBD_SHAPE_HEIGHTFIELD || s.kind == AVBD_SHAPE_TRIMESH) return s.pos;
    return gjk_shape(s.kind) ? support_convex(s, dir) : support(s, dir);
}

struct SVert {
    V3 v, sa, sb;
};
static __device__ __forceinline__ SVert minkowski(const Shape& a, const Shape& b, V3 dir) {
    V3 sa = support_any(a, dir);
    V3 sb = support_any(b, -dir);
    return {sa - sb, sa, sb};
}
static __device__ __forceinline__ V3 closest_segment0(V3 p, V3 q, float& wp, float& wq) {
    V3 pq = q - p;
    float l2 = len2(pq);
    if (l2 < gjk::COINCIDENT_LEN2) {
        wp = 1.0f;
        wq = 0.0f;
        return p;
    }
    float t = fclamp(-dot(p, pq) / l2, 0.0f, 1.0f);
    wp = 1.0f - t;
    wq = t;
    return p + pq * t;
}
// gjk.rs:220-265 (Ericson, Real-Time Collision Detection 5.1.5)
static __device__ __noinline__ V3 closest_triangle0(V3 a, V3 b, V3 c, float& wa, float& wb, float& wc) {
    V3 ab = b - a, ac = c - a, ap = -a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) { wa = 1.0f; wb = 0.0f; wc = 0.0f; return a; }
    V3 bp = -b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) { wa = 0.0f; wb = 1.0f; wc = 0.0f; return b; }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = d1 / (d1 - d3);
        wa = 1.0f - v; wb = v; wc = 0.0f;
        return a + ab * v;
    }
    V3 cp = -c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) { wa = 0.0f; wb = 0.0f; wc = 1.0f; return c; }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = d2 / (d2 - d6);
        wa = 1.0f - w; wb = 0.0f; wc = w;
        return a + ac * w;
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        wa = 0.0f; wb = 1.0f - w; wc = w;
        return b + (c - b) * w;
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    wa = 1.0f - v - w; wb = v; wc = w;
    return a + ab * v + ac * w;
}

// gjk.rs:358-458: closest point, keep mask and weights in input order; an
// enclosing tetrahedron keeps nothing
static __device__ __noinline__ V3 reduce_simplex(const SVert* s, int n, bool keep[4], float w[4]) {
    for (int i = 0; i < 4; i++) { keep[i] = false; w[i] = 0.0f; }
    if (n == 1) { keep[0] = true; w[0] = 1.0f; return s[0].v; }
    if (n == 2) {
        V3 p = closest_segment0(s[0].v, s[1].v, w[0], w[1]);
        keep[0] = w[0] > 0.0f; keep[1] = w[1] > 0.0f;
        return p;
    }
    if (n == 3) {
        V3 p = closest_triangle0(s[0].v, s[1].v, s[2].v, w[0], w[1], w[2]);
        keep[0] = w[0] > 0.0f; keep[1] = w[1] > 0.0f; keep[2] = w[2] > 0.0f;
        return p;
    }
    V3 e1 = s[1].v - s[0].v, e2 = s[2].v - s[0].v, e3 = s[3].v - s[0].v;
    float vol = fabsf(dot(e1, cross(e2, e3)));
    float scale = len(e1) * len(e2) * len(e3);
    const bool degenerate = vol <= gjk::TET_VOLUME_EPS * fmaxf(scale, gjk::COINCIDENT_LEN2);
    // faces (a, b, c, apex): flat tetrahedra test the plain triples
    const uint8_t FD[4][4] = {{0, 1, 2, 3}, {0, 1, 3, 2}, {0, 2, 3, 1}, {1, 2, 3, 0}};
    const uint8_t FF[4][4] = {{0, 1, 2, 3}, {0, 3, 1, 2}, {0, 2, 3, 1}, {1, 3, 2, 0}};
    bool have = false;
    V3 bp = V0();
    float bg = 0.0f, bw[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 4; k++) {
        const uint8_t* f = degenerate ? FD[k] : FF[k];
        float wa, wb, wc;
        V3 p = closest_triangle0(s[f[0]].v, s[f[1]].v, s[f[2]].v, wa, wb, wc);
        float gap = len(p);
        if (!have || gap < bg) {
            have = true;
            bp = p;
            bg = gap;
            bw[0] = bw[1] = bw[2] = bw[3] = 0.0f;
            bw[f[0]] = wa;
            bw[f[1]] = wb;
            bw[f[2]] = wc;
        }
    }
    if (!degenerate) {
        bool inside = true;
        for (int k = 0; k < 4; k++) {
            const uint8_t* f = FF[k];
            V3 nn = cross(s[f[1]].v - s[f[0]].v, s[f[2]].v - s[f[0]].v);
            if (dot(nn, s[f[3]].v - s[f[0]].v) > 0.0f) nn = -nn;
            if (dot(nn, -s[f[0]].v) > 0.0f) { inside = false; break; }
        }
        if (inside) return V0();
    }
    for (int i = 0; i < 4; i++) { w[i] = bw[i]; keep[i] = bw[i] > 0.0f; }
    return bp;
}

struct GjkDist {
    float dist;
    V3 normal, pa, pb;
};
// gjk.rs:267-356: separation; false when the origin is enclosed or touching
static __device__ __noinline__ bool gjk_separated(const Shape& a, const Shape& b, GjkDist& out) {
    V3 dir = a.pos - b.pos;
    if (len2(dir) < gjk::COINCIDENT_LEN2) dir = VX();
    SVert simplex[4];
    SVert first = minkowski(a, b, dir);
    for (int i = 0; i < 4; i++) simplex[i] = first;
    int count = 1;
    float weights[4] = {1.0f, 0.0f, 0.0f, 0.0f};
    V3 closest = simplex[0].v;
    if (len2(closest) < gjk::COINCIDENT_LEN2) {
        out = {0.0f, normalize_or(b.pos - a.pos, VY()), simplex[0].sa, simplex[0].sb};
        return true;
    }
    auto blend = [&](GjkDist& r) {
        V3 pa = V0(), pb = V0();
        for (int i = 0; i < count; i++) {
            pa = pa + simplex[i].sa * weights[i];
            pb = pb + simplex[i].sb * weights[i];
        }
        V3 delta = pa - pb;
        r = {len(delta), normalize_or(delta, normalize_or(b.pos - a.pos, VY())), pa, pb};
        return len(delta);
    };
    for (int it = 0; it < 64; it++) {
        dir = -closest;
        SVert w = minkowski(a, b, dir);
        if (dot(w.v, dir) - dot(closest, dir) <= gjk::PROGRESS_EPS * fmaxf(len2(closest), 1.0f)) {
            GjkDist r;
            float d = blend(r);
            if (d <= gjk::STALL_DIST) return false;
            out = r;
            return true;
        }
        simplex[count] = w;
        count++;
        bool keep[4];
        float wts[4];
        V3 next = reduce_simplex(simplex, count, keep, wts);
        int nc = 0;
        for (int i = 0; i < 4; i++)
            if (keep[i]) {
                simplex[nc] = simplex[i];
                weights[nc] = wts[i];
                nc++;
            }
        count = nc;
        if (count == 0 || len2(next) <= gjk::DEGENERATE_EPS) return false;
        closest = next;
    }
    blend(out);
    return true;
}

// gjk.rs:460-587
static __device__ __noinline__ void epa(const Shape& a, const Shape& b, const SVert* tet, float& depth, V3& normal,
                                        V3& pa, V3& pb) {
    SVert verts[gjk::EPA_VERT_CAP];
    uint8_t faces[gjk::EPA_FACE_CAP][3];
    uint8_t edges[3 * gjk::EPA_FACE_CAP][2];
    bool visible[gjk::EPA_FACE_CAP];
    int nv = 4, nf = 4;
    for (int i = 0; i < 4; i++) verts[i] = tet[i];
    const uint8_t init[4][3] = {{0, 2, 1}, {0, 3, 2}, {0, 1, 3}, {1, 2, 3}};
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) faces[i][k] = init[i][k];
    auto fnorm = [&](int i) {
        return cross(verts[faces[i][1]].v - verts[faces[i][0]].v, verts[faces[i][2]].v - verts[faces[i][0]].v);
    };
    for (int i = 0; i < nf; i++) {
        V3 nn = fnorm(i);
        int apex = -1;
        for (int k = 0; k < nv; k++)
            if (k != faces[i][0] && k != faces[i][1] && k != faces[i][2]) {
                apex = k;
                break;
            }
        if (apex >= 0 && dot(nn, verts[apex].v - verts[faces[i][0]].v) > 0.0f) {
            uint8_t t = faces[i][1];
            faces[i][1] = faces[i][2];
            faces[i][2] = t;
        }
    }
    depth = 0.0f;
    normal = VX();
    pa = a.pos;
    pb = b.pos;
    for (int it = 0; it < gjk::EPA_ITERS; it++) {
        if (nf == 0 || nf > gjk::EPA_MAX_FACES) break;
        int bi = 0;
        float bdist = FLT_MAX;
        V3 bnormal = VX();
        for (int i = 0; i < nf; i++) {
            V3 nn = fnorm(i);
            float l = len(nn);
            if (l < gjk::COINCIDENT_LEN2) continue;
            nn = nn / l;
            float d = dot(nn, verts[faces[i][0]].v);
            if (d < bdist) {
                bdist = d;
                bnormal = nn;
                bi = i;
            }
        }
        SVert w = minkowski(a, b, bnormal);
        if (dot(w.v, bnormal) - bdist <= 1e-6f * fmaxf(bdist, 1.0f)) {
            float wa, wb, wc;
            closest_triangle0(verts[faces[bi][0]].v, verts[faces[bi][1]].v, verts[faces[bi][2]].v, wa, wb, wc);
            pa = verts[faces[bi][0]].sa * wa + verts[faces[bi][1]].sa * wb + verts[faces[bi][2]].sa * wc;
            pb = verts[faces[bi][0]].sb * wa + verts[faces[bi][1]].sb * wb + verts[faces[bi][2]].sb * wc;
            depth = fmaxf(bdist, 0.0f);
            normal = bnormal;
            return;
        }
        for (int i = 0; i < nf; i++) {
            visible[i] = false;
            V3 nn = fnorm(i);
            float l = len(nn);
            if (l < gjk::COINCIDENT_LEN2) continue;
            if (dot(nn / l, w.v - verts[faces[i][0]].v) > gjk::EPA_VISIBLE_EPS) visible[i] = true;
        }
        int ne = 0;
        for (int i = 0; i < nf; i++) {
            if (!visible[i]) continue;
            for (int e = 0; e < 3; e++) {
                edges[ne][0] = faces[i][e];
                edges[ne][1] = faces[i][(e + 1) % 3];
                ne++;
            }
        }
        // horizon: directed edges without a reversed twin, in edge order
        uint8_t horizon[3 * gjk::EPA_FACE_CAP][2];
        int nh = 0;
        for (int e = 0; e < ne; e++) {
            bool twin = false;
            for (int o = 0; o < ne; o++)
                if (edges[o][0] == edges[e][1] && edges[o][1] == edges[e][0]) {
                    twin = true;
                    break;
                }
            if (!twin) {
                horizon[nh][0] = edges[e][0];
                horizon[nh][1] = edges[e][1];
                nh++;
            }
        }
        if (bdist < FLT_MAX) {
            depth = fmaxf(bdist, 0.0f);
            normal = bnormal;
            pa = a.pos;
            pb = b.pos;
        }
        if (nh > nf) break;
        int k = 0;
        for (int i = 0; i < nf; i++)
            if (!visible[i]) {
                faces[k][0] = faces[i][0];
                faces[k][1] = faces[i][1];
                faces[k][2] = faces[i][2];
                k++;
            }
        nf = k;
        if (nv >= gjk::EPA_VERT_CAP) break;  // unreachable: one vertex per iteration
        int wi = nv;
        verts[nv++] = w;
        for (int e = 0; e < nh && nf < gjk::EPA_FACE_CAP; e++) {
            faces[nf][0] = horizon[e][0];
            faces[nf][1] = horizon[e][1];
            faces[nf][2] = (uint8_t)wi;
            nf++;
        }
        V3 centroid = V0();
        for (int i = 0; i < nv; i++) centroid = centroid + verts[i].v;
        centroid = centroid / (float)nv;
        for (int i = 0; i < nf; i++) {
            V3 nn = fnorm(i);
            if (dot(nn, centroid - verts[faces[i][0]].v) > 0.0f) {
                uint8_t t = faces[i][1];
                faces[i][1] = faces[i][2];
                faces[i][2] = t;
            }
        }
        if (nv > gjk::EPA_MAX_VERTS) break;
    }
}

// gjk.rs:589-638
static __device__ __noinline__ GjkDist convex_distance(const Shape& a, const Shape& b) {
    GjkDist sep;
    if (gjk_separated(a, b, sep)) return sep;
    const V3 dirs[6] = {VX(), -VX(), VY(), -VY(), VZ(), -VZ()};
    SVert tet[4];
    SVert x0 = minkowski(a, b, VX());
    for (int i = 0; i < 4; i++) tet[i] = x0;
    int found = 0;
    for (int d = 0; d < 6; d++) {
        SVert w = minkowski(a, b, dirs[d]);
        bool fresh = true;
        for (int i = 0; i < found; i++)
            if (!(len2(tet[i].v - w.v) > gjk::DEGENERATE_EPS)) fresh = false;
        if (fresh && found < 4) tet[found++] = w;
        if (found == 4) break;
    }
    if (found < 4) return {0.0f, normalize_or(b.pos - a.pos, VY()), a.pos, b.pos};
    float depth;
    V3 normal, pa, pb;
    epa(a, b, tet, depth, normal, pa, pb);
    return {-depth, normal, pa, pb};
}

// Shape::closest_point (shape.rs:955-1215), in the shape's frame
static __device__ __noinline__ V3 closest_point_local(const Shape& s, V3 p) {
    switch (s.kind) {
        case AVBD_SHAPE_SPHERE: return normalize_or(p, VX()) * s.p.x;
        case AVBD_SHAPE_BOX: {
            V3 h = s.p;
            V3 c = vclamp(p, -h, h);
            if (len2(c - p) > gjk::COINCIDENT_LEN2) return c;
            float dx = h.x - fabsf(p.x), dy = h.y - fabsf(p.y), dz = h.z - fabsf(p.z);
            if (dx < dy && dx < dz) return V3{copysignf(h.x, p.x), p.y, p.z};
            if (dy < dz) return V3{p.x, copysignf(h.y, p.y), p.z};
            return V3{p.x, p.y, copysignf(h.z, p.z)};
        }
        case AVBD_SHAPE_CAPSULE: {
            float core = fclamp(p.y, -s.p.y, s.p.y);
            V3 axis{0.0f, core, 0.0f};
            return axis + normalize_or(p - axis, VX()) * s.p.x;
        }
        case AVBD_SHAPE_CYLINDER: {
            float radius = s.p.x, hh = s.p.y;
            float l = sqrtf(p.x * p.x + p.z * p.z);
            V3 wall = l > gjk::GJK_NEAR_ZERO ? V3{p.x / l * radius, fclamp(p.y, -hh, hh), p.z / l * radius}
                                           : V3{radius, fclamp(p.y, -hh, hh), 0.0f};
            float sc = l > gjk::GJK_NEAR_ZERO ? fminf(radius / l, 1.0f) : 0.0f;
            V3 top{p.x * sc, hh, p.z * sc}, bottom{p.x * sc, -hh, p.z * sc};
            if (len2(p - wall) < len2(p - top) && len2(p - wall) < len2(p - bottom)) return wall;
            if (len2(p - top) < len2(p - bottom)) return top;
            return bottom;
        }
        case AVBD_SHAPE_CONE: {
            float radius = s.p.x, hh = s.p.y;
            if (hh <= gjk::GJK_NEAR_ZERO) return V3{fclamp(p.x, -radius, radius), 0.0f, fclamp(p.z, -radius, radius)};
            float l = sqrtf(p.x * p.x + p.z * p.z);
            float yc = fclamp(p.y, -hh, hh);
            float r_at = radius * (hh - yc) / (2.0f * hh);
            V3 wall = l > gjk::GJK_NEAR_ZERO ? V3{p.x / l * r_at, yc, p.z / l * r_at} : V3{r_at, yc, 0.0f};
            float sc = l > gjk::GJK_NEAR_ZERO ? fminf(radius / l, 1.0f) : 0.0f;
            V3 base{p.x * sc, -hh, p.z * sc}, apex{0.0f, hh, 0.0f};
            V3 best = wall;
            float bd = len2(p - wall);
            float d = len2(p - base);
            if (d < bd) { best = base; bd = d; }
            d = len2(p - apex);
            if (d < bd) { best = apex; bd = d; }
            return best;
        }
        case AVBD_SHAPE_HULL: {
            const HullDesc* h = s.hull;
            if (!h || h->nf == 0) {
                if (!h || h->nv == 0) return V0();
                V3 sum = V0();
                for (uint32_t i = 0; i < h->nv; i++) sum = sum + ld3(h->v[i]);
                return sum / (float)h->nv;
            }
            V3 best = ld3(h->v[h->f[0]]);
            float bd = len2(p - best);
            for (uint32_t f = 0; f < h->nf; f++) {
                V3 a = ld3(h->v[h->f[3 * f]]), b = ld3(h->v[h->f[3 * f + 1]]), c = ld3(h->v[h->f[3 * f + 2]]);
                float wa, wb, wc;
                V3 q = closest_triangle0(a - p, b - p, c - p, wa, wb, wc) + p;
                float d = len2(p - q);
                if (d < bd) {
                    best = q;
                    bd = d;
                }
            }
            return best;
        }
        default:
            return p;
    }
}
static __device__ __forceinline__ V3 closest_point_world(const Shape& s, V3 p) {
    V3 local = qrot(conj(s.rot), p - s.pos);
    return s.pos + qrot(s.rot, closest_point_local(s, local));
}

// distance.rs:364-421
static __device__ __noinline__ Dist gjk_pair_distance(const Shape& a, const Shape& b) {
    GjkDist g = convex_distance(a, b);
    float dist = g.dist;
    V3 pa = g.pa, pb = g.pb;
    if (!isfinite(dist)) return {dist, pa, pb};
    V3 n = len2(g.normal) > gjk::COINCIDENT_LEN2 ? normalize(g.normal) : normalize_or(b.pos - a.pos, VY());
    float depth = -dist;
    if (dist < SHAPE_TOUCH) {
        pa = a.pos;
        pb = b.pos;
    }
    for (int k = 0; k < 2; k++) {
        pb = closest_point_world(b, pa - n * depth);
        pa = closest_point_world(a, pb - n * depth);
        V3 axis = pb - pa;
        if (len2(axis) > gjk::COINCIDENT_LEN2) n = normalize(axis);
    }
    return {dist, pa, pb};
}
