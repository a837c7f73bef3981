// avbd_common.cuh — small device helpers shared by the pipeline phases.
#pragma once
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "avbd_kernels.h"
#include "avbd_rows.cuh"
#include "avbd_shapes.cuh"

namespace avbd {

static inline unsigned nblk(size_t n, int b) { return (unsigned)((n + (size_t)b - 1) / (size_t)b); }
// Grid for kernels whose trip count lives on the device (grid-stride loops):
// enough resident blocks to fill the 152 SMs, never more than the capacity needs.
static inline unsigned gsz(size_t cap, int b) {
    unsigned g = nblk(cap, b);
    return g < 152u * 16u ? g : 152u * 16u;
}

// Warp-aggregated counters: the lanes that call together share one atomic, so
// a counter bumped by millions of threads (candidates, points) is not
// serialised at one L2 address.  Call from the lanes that add, in any branch.
static __device__ __forceinline__ uint32_t agg_inc(uint32_t* ctr) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(ctr, (uint32_t)g.size());
    return g.shfl(base, 0) + g.thread_rank();
}
// Same for a per-key counter arr[key]: lanes with equal keys share one atomic
// (a half-space is the A side of every candidate it has in its scene).
static __device__ __forceinline__ uint32_t agg_inc_at(uint32_t* arr, uint32_t key) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    cg::coalesced_group s = cg::labeled_partition(g, key);
    uint32_t base = 0;
    if (s.thread_rank() == 0) base = atomicAdd(&arr[key], (uint32_t)s.size());
    return s.shfl(base, 0) + s.thread_rank();
}
static __device__ __forceinline__ void agg_add(uint32_t* ctr, uint32_t v) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t s = cg::reduce(g, v, cg::plus<uint32_t>());
    if (g.thread_rank() == 0 && s) atomicAdd(ctr, s);
}

static __device__ __forceinline__ bool is_dynamic(const DW& w, uint32_t h) {
    return info_type(w.info[h]) == AVBD_BODY_DYNAMIC;
}
// AvbdEngine::solvable (mod.rs:1179-1181)
static __device__ __forceinline__ bool solvable(const DW& w, uint32_t h) {
    return info_type(w.info[h]) == AVBD_BODY_DYNAMIC && w.inv_mass[h] > 0.0f;
}
// swept by the primal: solvable and awake
static __device__ __forceinline__ bool solved(const DW& w, uint32_t h) { return solvable(w, h) && !w.asleep[h]; }
static __device__ __forceinline__ Shape shape_of(const DW& w, uint32_t h) {
    float4 sp = w.shp[h];
    uint32_t kind = info_shape(w.info[h]);
    const HullDesc* hull = nullptr;
    if (kind == AVBD_SHAPE_HULL) {
        uint32_t id = (uint32_t)sp.x;
        hull = id < w.nhulls ? &w.hulls[id] : nullptr;
    }
    return Shape{kind, V3{sp.x, sp.y, sp.z}, ld3(w.pos[h]), ldq(w.rot[h]), hull};
}

// ---- rounded and compound shapes, terrain, meshes (distance.rs:246-745) ----
static __device__ __forceinline__ bool ext_kind(uint32_t kind) {
    return kind == AVBD_SHAPE_ROUND || kind == AVBD_SHAPE_COMPOUND;
}
// shapes without a finite bound: paired with every body of their scene
static __host__ __device__ __forceinline__ bool unbounded_kind(uint32_t kind) {
    return kind == AVBD_SHAPE_HALFSPACE || kind == AVBD_SHAPE_HEIGHTFIELD || kind == AVBD_SHAPE_TRIMESH;
}
// Shape::aabb (shape.rs:619-680) of a primitive.
static __device__ __forceinline__ void prim_aabb(const Shape& s, V3& lo, V3& hi) {
    auto absv = [](V3 v) { return V3{fabsf(v.x), fabsf(v.y), fabsf(v.z)}; };
    V3 r;
    if (s.kind == AVBD_SHAPE_SPHERE) {
        r = V3{s.p.x, s.p.x, s.p.x};
    } else if (s.kind == AVBD_SHAPE_BOX) {
        r = (absv(qrot(s.rot, VX())) * s.p.x + absv(qrot(s.rot, VY())) * s.p.y) + absv(qrot(s.rot, VZ())) * s.p.z;
    } else if (s.kind == AVBD_SHAPE_HULL) {
        if (!s.hull || s.hull->nv == 0) {
            lo = hi = s.pos;
            return;
        }
        lo = V3{INFINITY, INFINITY, INFINITY};
        hi = V3{-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = 0; i < s.hull->nv; i++) {
            const V3 w = s.pos + qrot(s.rot, ld3(s.hull->v[i]));
            lo = V3{fminf(lo.x, w.x), fminf(lo.y, w.y), fminf(lo.z, w.z)};
            hi = V3{fmaxf(hi.x, w.x), fmaxf(hi.y, w.y), fmaxf(hi.z, w.z)};
        }
        return;
    } else {  // capsule, cylinder, cone: the axis shell plus the radius
        const V3 e = absv(qrot(s.rot, VY())) * s.p.y;
        r = V3{e.x + s.p.x, e.y + s.p.x, e.z + s.p.x};
    }
    lo = s.pos - r;
    hi = s.pos + r;
}
// The convex side's AABB corners in the frame (pos, rot): their bounds.
static __device__ __forceinline__ void local_window(const Shape& convex, V3 pos, Q rot, V3& lo, V3& hi) {
    V3 amin, amax;
    prim_aabb(convex, amin, amax);
    const Q inv = conj(rot);
    lo = V3{INFINITY, INFINITY, INFINITY};
    hi = V3{-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < 8; i++) {
        const V3 corner{(i & 1) ? amax.x : amin.x, (i & 2) ? amax.y : amin.y, (i & 4) ? amax.z : amin.z};
        const V3 l = qrot(inv, corner - pos);
        lo = V3{fminf(lo.x, l.x), fminf(lo.y, l.y), fminf(lo.z, l.z)};
        hi = V3{fmaxf(hi.x, l.x), fmaxf(hi.y, l.y), fmaxf(hi.z, l.z)};
    }
}
// heightfield_convex (distance.rs:246-350): the nearest overlapped column,
// each a solid box from the lowest sample up to its height (a flat one a
// one-cell skirt); `first`: the terrain owns pa.
static __device__ __noinline__ Dist hf_convex(const DW& w, const Shape& t, const Shape& convex, bool first) {
    const HfDesc hf = w.hfs[(uint32_t)t.p.x];
    V3 lo, hi;
    local_window(convex, t.pos, t.rot, lo, hi);
    // the column index along x serves the rows too (distance.rs:299-303)
    auto col_at = [&](float x, uint32_t n) -> uint32_t {
        const float f = floorf(x / hf.cell + (float)(hf.cols - 1) * HALF);
        if (!(f > 0.0f)) return 0u;
        return f >= (float)(n - 1) ? n - 1 : (uint32_t)f;
    };
    const uint32_t c0 = col_at(lo.x, hf.cols), c1 = col_at(hi.x, hf.cols);
    const uint32_t r0 = col_at(lo.z, hf.rows), r1 = col_at(hi.z, hf.rows);
    const float x_origin = -(float)(hf.cols - 1) * HALF * hf.cell, z_origin = -(float)(hf.rows - 1) * HALF * hf.cell;
    bool have = false;
    Dist best{INFINITY, t.pos, convex.pos};
    for (uint32_t row = r0; row <= r1; row++)
        for (uint32_t col = c0; col <= c1; col++) {
            const float h = hf.h[(size_t)row * hf.cols + col];
            const float y_low = h - hf.y_min >= 1e-4f ? hf.y_min : h - fmaxf(hf.cell, 1e-3f);
            const V3 mn{x_origin + (float)col * hf.cell, y_low, z_origin + (float)row * hf.cell};
            const V3 mx{mn.x + hf.cell, fmaxf(h, y_low), mn.z + hf.cell};
            const V3 center = (mn + mx) * HALF;
            V3 hl = (mx - mn) * HALF;
            hl = V3{fmaxf(hl.x, 0.0f), fmaxf(hl.y, 0.0f), fmaxf(hl.z, 0.0f)};
            const Shape column{AVBD_SHAPE_BOX, hl, t.pos + qrot(t.rot, center), t.rot, nullptr};
            const Dist d = shape_distance(column, convex, nullptr);
            if (!have || d.dist < best.dist) {
                best = d;
                have = true;
            }
        }
    if (!have) return first ? Dist{INFINITY, t.pos, convex.pos} : Dist{INFINITY, convex.pos, t.pos};
    return first ? best : Dist{best.dist, best.pb, best.pa};
}
// trimesh_convex (distance.rs:416-517): the nearest triangle whose tree
// boxes overlap the convex side's window, walked last-in-first-out; the
// winner's witnesses come back swapped when the mesh is the first shape and
// as found when it is the second (the reference's own order, kept).
static __device__ __noinline__ Dist mesh_convex(const DW& w, const Shape& m, const Shape& convex, bool first) {
    const MeshDesc mesh = w.meshes[(uint32_t)m.p.x];
    const Dist none = first ? Dist{INFINITY, m.pos, convex.pos} : Dist{INFINITY, convex.pos, m.pos};
    if (mesh.ntris == 0) return none;
    V3 lo, hi;
    local_window(convex, m.pos, m.rot, lo, hi);
    bool have = false;
    Dist best = none;
    uint32_t stack[64];
    uint32_t len = 1;
    stack[0] = 0;
    while (len > 0) {
        const uint32_t ni = stack[--len];
        if (ni >= mesh.nnodes) continue;
        const MeshNodeD node = mesh.nodes[ni];
        if (node.hi[0] < lo.x || node.lo[0] > hi.x || node.hi[1] < lo.y || node.lo[1] > hi.y || node.hi[2] < lo.z ||
            node.lo[2] > hi.z)
            continue;
        if (node.leaf) {
            const uint32_t end = min(node.a + node.b, mesh.norder);
            for (uint32_t o = node.a; o < end; o++) {
                const uint32_t tri = mesh.order[o];
                if (tri >= mesh.ntris) continue;
                const Shape th{AVBD_SHAPE_HULL, V0(), m.pos + qrot(m.rot, ld3(mesh.cent[tri])), m.rot, &mesh.tris[tri]};
                const Dist d = shape_distance(th, convex, nullptr);
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
    return first ? Dist{best.dist, best.pb, best.pa} : best;
}
// shape_distance below the rounded and compound arms (distance.rs:706-745):
// half-spaces, terrain, meshes, then the primitive pairs.
static __device__ __noinline__ Dist leaf_distance(const DW& w, const Shape& a, const Shape& b) {
    if (a.kind == AVBD_SHAPE_HALFSPACE || b.kind == AVBD_SHAPE_HALFSPACE) return shape_distance(a, b, nullptr);
    const bool ta = a.kind == AVBD_SHAPE_HEIGHTFIELD, tb = b.kind == AVBD_SHAPE_HEIGHTFIELD;
    const bool ma = a.kind == AVBD_SHAPE_TRIMESH, mb = b.kind == AVBD_SHAPE_TRIMESH;
    // terrain against terrain or a mesh, mesh against mesh: separation
    if ((ta || ma) && (tb || mb)) return Dist{INFINITY, a.pos, b.pos};
    if (ta) return hf_convex(w, a, b, true);
    if (tb) return hf_convex(w, b, a, false);
    if (ma) return mesh_convex(w, a, b, true);
    if (mb) return mesh_convex(w, b, a, false);
    return shape_distance(a, b, nullptr);
}
// The rounded surface sits r closer along the witness axis; an infinite
// distance stays (round_offset, distance.rs:519-545).
static __device__ __forceinline__ Dist round_offset(Dist d, float r, bool first, V3 pos_a, V3 pos_b) {
    if (!isfinite(d.dist)) return d;
    V3 axis = d.pb - d.pa;
    if (len2(axis) <= gjk::COINCIDENT_LEN2) axis = pos_b - pos_a;
    const V3 n = normalize_or(axis, VX());
    if (first) return {d.dist - r, d.pa + n * r, d.pb};
    return {d.dist - r, d.pa, d.pb - n * r};
}
// Pose::world_rot (shape.rs:119-134)
static __device__ __forceinline__ Q pose_world_rot(Q parent, Q local) {
    const Q q = qmul(parent, local);
    const float l2 = (q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w);
    if (isfinite(q.x) && isfinite(q.y) && isfinite(q.z) && isfinite(q.w) && l2 > 1e-12f) return qnormalize(q);
    return parent;
}
static __device__ __forceinline__ Shape part_shape(const PartDesc& pt, V3 pos, Q rot) {
    return Shape{pt.kind, V3{pt.p.x, pt.p.y, pt.p.z}, pos, rot, pt.hull};
}
// compound_distance (distance.rs:550-599): the part reporting the smallest
// distance, parts in order, each rounded part peeled inside its own query;
// `first`: the compound owns pa.
static __device__ __noinline__ Dist compound_distance(const DW& w, const Shape& c, const Shape& other, bool first) {
    const ExtDesc e = w.exts[(uint32_t)c.p.x];
    bool have = false;
    Dist best{INFINITY, c.pos, other.pos};
    for (uint32_t k = 0; k < e.count; k++) {
        const PartDesc pt = w.parts[e.first + k];
        const Shape child = part_shape(pt, c.pos + qrot(c.rot, ld3(pt.pos)), pose_world_rot(c.rot, ldq(pt.rot)));
        Dist d = leaf_distance(w, child, other);
        if (pt.p.w > 0.0f) d = round_offset(d, pt.p.w, true, child.pos, other.pos);
        if (!have || d.dist < best.dist) {
            best = d;
            have = true;
        }
    }
    if (!have) return first ? Dist{INFINITY, c.pos, other.pos} : Dist{INFINITY, other.pos, c.pos};
    return first ? best : Dist{best.dist, best.pb, best.pa};
}
// shape_distance with the wrapper arms (distance.rs:648-705): rounded shapes
// peel first (a's, then b's), then compounds expand; compound against
// compound is separation.  Rounded inners and compound parts are primitives.
static __device__ __noinline__ Dist ext_distance_wrapped(const DW& w, const Shape& a, const Shape& b) {
    Shape ia = a, ib = b;
    float ra = 0.0f, rb = 0.0f;
    if (a.kind == AVBD_SHAPE_ROUND) {
        const PartDesc pt = w.parts[w.exts[(uint32_t)a.p.x].first];
        ia = part_shape(pt, a.pos, a.rot);
        ra = pt.p.w;
    }
    if (b.kind == AVBD_SHAPE_ROUND) {
        const PartDesc pt = w.parts[w.exts[(uint32_t)b.p.x].first];
        ib = part_shape(pt, b.pos, b.rot);
        rb = pt.p.w;
    }
    Dist d;
    if (ia.kind == AVBD_SHAPE_COMPOUND && ib.kind == AVBD_SHAPE_COMPOUND) d = Dist{INFINITY, a.pos, b.pos};
    else if (ia.kind == AVBD_SHAPE_COMPOUND) d = compound_distance(w, ia, ib, true);
    else if (ib.kind == AVBD_SHAPE_COMPOUND) d = compound_distance(w, ib, ia, false);
    else d = leaf_distance(w, ia, ib);
    if (b.kind == AVBD_SHAPE_ROUND) d = round_offset(d, rb, false, a.pos, b.pos);
    if (a.kind == AVBD_SHAPE_ROUND) d = round_offset(d, ra, true, a.pos, b.pos);
    return d;
}
// Primitive pairs keep the direct call; the wrapper arms take the rest.
static __device__ __forceinline__ Dist ext_distance(const DW& w, const Shape& a, const Shape& b, float* sat_gap) {
    if (a.kind <= AVBD_SHAPE_HULL && b.kind <= AVBD_SHAPE_HULL) return shape_distance(a, b, sat_gap);
    return ext_distance_wrapped(w, a, b);
}
// rows.rs:366-368
static __device__ __forceinline__ bool pair_allowed(const DW& w, uint32_t a, uint32_t b) {
    uint2 fa = w.filter[a], fb = w.filter[b];
    return (fa.x & fb.y) != 0u && (fb.x & fa.y) != 0u;
}
// a joint links a and b (the swept cast skips every joined partner but a
// gear's, mod.rs:887-917)
static __device__ __forceinline__ bool jointed(const DW& w, uint32_t a, uint32_t b) {
    for (uint32_t k = w.jofs[a]; k < w.jofs[a + 1]; k++) {
        const uint32_t j = w.jlist[k];
        uint2 ab = w.j_ab[j];
        if (w.j_kind[j] == AVBD_JOINT_GEAR) continue;
        if ((ab.x == a && ab.y == b) || (ab.x == b && ab.y == a)) return true;
    }
    return false;
}
// a joint that turns contact off links a and b (rows.rs:434-474): every kind
// but the weld-like Fixed and SixDof, whose contact is structural
static __device__ __forceinline__ bool jointed_no_collide(const DW& w, uint32_t a, uint32_t b) {
    for (uint32_t k = w.jofs[a]; k < w.jofs[a + 1]; k++) {
        const uint32_t j = w.jlist[k];
        uint2 ab = w.j_ab[j];
        const uint32_t kind = w.j_kind[j];
        if (kind == AVBD_JOINT_FIXED || kind == AVBD_JOINT_SIXDOF || kind == AVBD_JOINT_GEAR) continue;
        if ((ab.x == a && ab.y == b) || (ab.x == b && ab.y == a)) return true;
    }
    return false;
}
static __device__ __forceinline__ float eff_inv_mass(const DW& w, uint32_t h) {  // rows.rs:406-412
    return is_dynamic(w, h) ? w.inv_mass[h] : 0.0f;
}
// mod.rs:833-842 with RigidBody::wake_restore (body.rs:412-418)
static __device__ __forceinline__ void wake_body(const DW& w, uint32_t h) {
    if (!w.asleep[h]) return;
    w.asleep[h] = 0;
    w.sleep_timer[h] = 0.0f;
    if (is_dynamic(w, h)) {
        w.inv_mass[h] = w.inv_mass_rest[h];
        w.inertia[h] = w.inertia_rest[h];
    }
}
// A candidate-buffer overflow aborts the rest of the substep (every later
// kernel returns at once) so the host can grow the buffers and replay it: the
// kernels that ran before the check (wake, torque, AABBs) are idempotent.
static __device__ __forceinline__ bool aborted(const DW& w) { return (w.ctr[C_ERR] & E_CAND_OVERFLOW) != 0u; }
// The iterations of a substep whose colouring needs more colours than the
// launched iteration covers are skipped; the host finishes that substep.
static __device__ __forceinline__ bool aborted_solve(const DW& w) {
    return (w.ctr[C_ERR] & (E_CAND_OVERFLOW | E_COLOUR_RANGE)) != 0u;
}
static __device__ __forceinline__ uint32_t n_cand(const DW& w) { return min(w.ctr[C_CAND], w.cand_cap); }
static __device__ __forceinline__ uint32_t n_pairs(const DW& w) { return w.offA[w.N]; }

// Index of the previous-generation pair (a, b), or -1.  The old B-side list
// of b (rebuilt every substep, untouched until this substep's incidence
// rebuild) holds its pairs in ascending pair index, i.e. ascending a, so a
// binary search finds (a, b) whatever the size of a's own A-side segment
// (a half-space is the A side of every pair in its scene).
static __device__ __forceinline__ int32_t find_old_pair(const DW& w, uint32_t a, uint32_t b) {
    uint32_t lo = w.offB[b], hi = w.offB[b + 1];
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t p = w.listB[mid];
        uint32_t v = w.o_ab[p].x;
        if (v == a) return (int32_t)p;
        if (v < a) lo = mid + 1;
        else hi = mid;
    }
    return -1;
}

// sixdof axis configuration word: 2 bits per axis (linear x y z, angular x y z)
static __host__ __device__ __forceinline__ uint32_t axis_cfg(uint32_t cfg, int axis) { return (cfg >> (2 * axis)) & 3u; }
// (min, max) of sixdof axis k
static __device__ __forceinline__ float2 axis_window(const DW& w, uint32_t j, int k) {
    float4 v = w.j_six[3 * (size_t)j + (k >> 1)];
    return (k & 1) ? make_float2(v.z, v.w) : make_float2(v.x, v.y);
}
// ---- gears (joints_ext.rs:34-160) ----
// One side of a gear (GearSide, avbd/mod.rs:304-317): the coupled joint's
// bodies, whether it turns (revolute) or slides (prismatic), its live world
// axis, the slide's anchor levers and its continuous coordinate.
struct GearSide {
    uint32_t a, b;
    bool angular;
    V3 axis, ra, rb;
    float coord;
};
// A revolute joint's twist or a prismatic joint's slide from its assembly
// reference (joints_ext.rs:37-51); the side's axis and levers on the way.
static __device__ __forceinline__ float joint_coordinate(const DW& w, uint32_t r, GearSide* s = nullptr) {
    const uint2 ab = w.j_ab[r];
    const Q qa = ldq(w.rot[ab.x]), qb = ldq(w.rot[ab.y]);
    const float4 axa4 = w.j_axa[r];
    const V3 axis = ld3(axa4);
    const bool angular = w.j_kind[r] == AVBD_JOINT_REVOLUTE;
    const V3 wa = normalize_or(qrot(qa, axis), VZ());
    float raw;
    V3 ra = V0(), rb = V0();
    if (angular) {
        raw = hinge_twist(qa, qb, axis) - axa4.w;
    } else {
        ra = qrot(qa, ld3(w.j_la[r]));
        rb = qrot(qb, ld3(w.j_lb[r]));
        const V3 pa = ld3(w.pos[ab.x]) + ra, pb = ld3(w.pos[ab.y]) + rb;
        raw = dot(pb - pa, wa) - w.j_ref[r].x;
    }
    if (s) {
        s->a = ab.x;
        s->b = ab.y;
        s->angular = angular;
        s->axis = wa;
        s->ra = ra;
        s->rb = rb;
    }
    return raw;
}
// Side k of gear g, its coordinate unwrapped across turns against the step
// start for a hinge (joints_ext.rs:120-160).
static __device__ __forceinline__ GearSide gear_side(const DW& w, uint32_t g, int k) {
    const uint2 gb = w.j_gb[g];
    GearSide s;
    const float raw = joint_coordinate(w, k ? gb.y : gb.x, &s);
    const float4 m = w.j_gmem[g];
    s.coord = w.j_gset[g] && s.angular ? (k ? m.w : m.z) + wrap_pi(raw - (k ? m.y : m.x)) : raw;
    return s;
}
// C = coordinate_a + ratio coordinate_b - constant
static __device__ __forceinline__ float gear_error(const DW& w, uint32_t g, const GearSide& sa, const GearSide& sb) {
    return sa.coord + w.j_dref[g].x * sb.coord - w.j_ref[g].x;
}
// The bodies a joint holds (sleep.rs:9-16), how many: a joint's two, a
// gear's coupled joints' four (a body may repeat).
static __device__ __forceinline__ int joint_members(const DW& w, uint32_t j, uint32_t m[4]) {
    if (w.j_kind[j] == AVBD_JOINT_GEAR) {
        const uint2 gb = w.j_gb[j];
        const uint2 x = w.j_ab[gb.x], y = w.j_ab[gb.y];
        m[0] = x.x; m[1] = x.y; m[2] = y.x; m[3] = y.y;
        return 4;
    }
    const uint2 ab = w.j_ab[j];
    m[0] = ab.x; m[1] = ab.y;
    return 2;
}

// The body whose walk over its joints updates a joint's multipliers in the
// per-scene solve: a joint's first body, a gear's first coupled body (a gear
// is listed only on its coupled joints' bodies).
static __device__ __forceinline__ uint32_t joint_dual_owner(const DW& w, uint32_t j) {
    return w.j_kind[j] == AVBD_JOINT_GEAR ? w.j_ab[w.j_gb[j].x].x : w.j_ab[j].x;
}

// sleep.rs:30-105: how far a joint is from its assembly pose
static __device__ __forceinline__ float joint_rest_error(const DW& w, uint32_t j) {
    if (w.j_kind[j] == AVBD_JOINT_GEAR) {
        const GearSide sa = gear_side(w, j, 0), sb = gear_side(w, j, 1);
        return fabsf(gear_error(w, j, sa, sb));
    }
    uint2 ab = w.j_ab[j];
    V3 pa = ld3(w.pos[ab.x]), pb = ld3(w.pos[ab.y]);
    Q qa = ldq(w.rot[ab.x]), qb = ldq(w.rot[ab.y]);
    V3 delta = (pb + qrot(qb, ld3(w.j_lb[j]))) - (pa + qrot(qa, ld3(w.j_la[j])));
    const uint32_t kind = w.j_kind[j];
    if (kind == AVBD_JOINT_BALL) return len(delta);
    V3 axis = qrot(qa, ld3(w.j_axa[j]));
    if (kind == AVBD_JOINT_REVOLUTE) return fmaxf(len(delta), len(axis - qrot(qb, ld3(w.j_axb[j]))));
    const float refv = w.j_ref[j].x;
    if (kind == AVBD_JOINT_FIXED || kind == AVBD_JOINT_MOTOR)  // a free motor: its assembly deviation
        return fmaxf(len(delta - qrot(qa, ld3(w.j_dref[j]))), len(quat_diff_vec(qmul(conj(qa), qb), ldq(w.j_qref[j]))));
    if (kind == AVBD_JOINT_DISTANCE || kind == AVBD_JOINT_SPRING) return fabsf(len(delta) - refv);
    if (kind == AVBD_JOINT_ROPE) return fmaxf(len(delta) - refv, 0.0f);
    if (kind == AVBD_JOINT_PRISMATIC) {
        float e = len(delta - axis * dot(delta, axis));
        float4 lim = w.j_lim[j];
        if (lim.z != 0.0f) {
            float value = dot(delta, axis) - refv;
            e = fmaxf(e, fmaxf(lim.x - value, value - lim.y));
        }
        return fmaxf(e, len(axis - qrot(qb, ld3(w.j_axb[j]))));
    }
    if (kind == AVBD_JOINT_WHEEL) {  // sleep.rs:54-70: axles in the weld-reference slots
        float e = len(delta - axis * dot(delta, axis));
        e = fmaxf(e, len(qrot(qa, ld3(w.j_dref[j])) - qrot(qb, ld3(w.j_qref[j]))));
        if (w.j_lim[j].x <= 0.0f) e = fmaxf(e, fabsf(dot(delta, axis) - refv));
        return e;
    }
    // sixdof (sleep.rs:86-103)
    V3 lin = qrot(conj(qa), delta) - ld3(w.j_dref[j]);
    V3 ang = quat_diff_vec(qmul(conj(qa), qb), ldq(w.j_qref[j]));
    const uint32_t cfg = w.j_cfg[j];
    float e = 0.0f;
    for (int i = 0; i < 3; i++) {
        float vals[2] = {lin[i], ang[i]};
        for (int k = 0; k < 2; k++) {
            const int axis_i = i + 3 * k;
            const uint32_t c = axis_cfg(cfg, axis_i);
            float r = 0.0f;
            if (c == AVBD_AXIS_LOCKED) {
                r = fabsf(vals[k]);
            } else if (c == AVBD_AXIS_LIMITED) {
                float2 win = axis_window(w, j, axis_i);
                r = fmaxf(fmaxf(win.x - vals[k], vals[k] - win.y), 0.0f);
            }
            e = fmaxf(e, r);
        }
    }
    return e;
}
// sleep.rs:18-27: a running motor, or a non-dynamic member moved by its driver
static __device__ __forceinline__ bool joint_driven(const DW& w, uint32_t j) {
    const float4 ref = w.j_ref[j];
    if (w.j_kind[j] == AVBD_JOINT_SPRING) {  // JointMotor::keeps_awake (joint.rs:1116-1126)
        const float4 m = w.j_axb[j];  // stiffness, damping, max_force, target_velocity
        const bool velocity_kind = (w.j_cfg[j] & 15u) == AVBD_MOTOR_VELOCITY;
        if (m.z > 0.0f && (velocity_kind ? m.w != 0.0f : (m.x > 0.0f || m.w != 0.0f))) return true;
    } else if (w.j_kind[j] == AVBD_JOINT_MOTOR) {  // MotorDrive::keeps_awake (joint.rs:474-477)
        const float4 lin = w.j_axa[j], ang = w.j_axb[j];
        if ((ref.z > 0.0f && (lin.x != 0.0f || lin.y != 0.0f || lin.z != 0.0f)) ||
            (ref.w > 0.0f && (ang.x != 0.0f || ang.y != 0.0f || ang.z != 0.0f)))
            return true;
    } else if (ref.z != 0.0f && ref.w > 0.0f) {
        return true;
    }
    uint32_t m[4];
    const int nm = joint_members(w, j, m);
    for (int k = 0; k < nm; k++) {
        uint32_t h = m[k];
        if (is_dynamic(w, h)) continue;
        float4 p = w.pos[h], pp = w.prev_pos[h], q = w.rot[h], pq = w.prev_rot[h];
        if (p.x != pp.x || p.y != pp.y || p.z != pp.z || q.x != pq.x || q.y != pq.y || q.z != pq.z || q.w != pq.w)
            return true;
    }
    return false;
}

static __global__ void k_zero_u32(uint32_t* p, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = 0u;
}
static __global__ void k_comp_clear(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < (uint32_t)w.N) w.comp_flag[h] = 0;
}

}  // namespace avbd
