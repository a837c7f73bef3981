// avbd_world.cu — the C ABI of include/ornis_avbd.h: world lifecycle, host
// model <-> device SoA, the substep driver, CUDA-graph replay and the state
// exchange used for checkpoints and parity checks.
//
// Host semantics mirror the reference's engine seam (crates/physics/src/
// engine.rs:24-133, avbd/mod.rs:1211-1602): dense handles in insertion order,
// the fixed-step accumulator of PhysicsEngine::step, JointError-style codes.
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "avbd_crmath.cuh"
#include "avbd_kernels.h"
#include "avbd_rows.cuh"

using namespace avbd;

namespace {

struct JointRec {
    uint32_t kind, a, b;
    float la[3], lb[3], axa[3], axb[3];
    float ref;   // revolute reference twist
    float refv;  // prismatic reference length, distance rest length, rope maximum
    int32_t has_lim;
    float lo, hi;
    float mot_speed, mot_max;  // velocity motor (mot_max 0: none)
    float qref[4], dref[3];    // fixed / sixdof / free-motor assembly references
    float mlin[3], mang[3];    // free motor: B-minus-A velocity targets (world frame)
    float mforce, mtorque;     // free motor budgets
    float spr[4];              // spring: stiffness, damping, max_force, target_velocity
    uint32_t spr_mode;         // spring: kind | model << 4
    float bxa[3], bxb[3];      // wheel: spin axles
    float susp[2];             // wheel: suspension frequency (Hz) and damping ratio
    uint32_t gb[2];            // gear: the coupled joints
    float gratio;              // gear: coordinate_a + gratio coordinate_b stays at ref
    uint32_t cfg;              // sixdof axis configuration, 2 bits per axis
    float six_min[6], six_max[6];
    AvbdJointState st;
};

// The bodies a joint holds, each once (sleep.rs:9-16): its two bodies, or
// for a gear the bodies of the two joints it couples.
int joint_members_host(const std::vector<JointRec>& js, uint32_t ji, uint32_t m[4]) {
    const JointRec& j = js[ji];
    if (j.kind != AVBD_JOINT_GEAR) {
        m[0] = j.a;
        m[1] = j.b;
        return 2;
    }
    const uint32_t c[4] = {js[j.gb[0]].a, js[j.gb[0]].b, js[j.gb[1]].a, js[j.gb[1]].b};
    int n = 0;
    for (uint32_t x : c) {
        bool seen = false;
        for (int k = 0; k < n; k++) seen = seen || m[k] == x;
        if (!seen) m[n++] = x;
    }
    return n;
}

struct Alloc {
    std::vector<void*> ptrs;
    template <class T> T* get(size_t n) {
        void* p = nullptr;
        if (n == 0) n = 1;
        if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, n * sizeof(T));
        ptrs.push_back(p);
        return (T*)p;
    }
    void release() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

struct PairBuf {
    uint2* ab;
    float4* n;
    float2* mu;
    uint32_t* np;
    float4 *ra, *rb, *lam, *pen, *roll;
    int32_t* matched;
    int32_t* old;  // previous-generation pair index (-1 new)
    uint32_t* offA;
};

// A convex hull as the host keeps it (ConvexHull, collision/shape.rs:317-365).
struct HostHull {
    std::vector<float4> v;
    std::vector<uint32_t> f;
    float unit_inertia[3];
    float bound, min_ext;
};

// A rounded shape (one part) or a compound as the host keeps it, with the
// measures the engine reads from it (rows.rs:279-290, :393-400).
struct HostExt {
    bool compound;
    std::vector<AvbdShapePart> parts;
    float unit_inertia[3];
    float bound, min_dim;
};

// A heightfield as registered, with its sample range (shape.rs:1571-1583).
struct HostHf {
    uint32_t rows, cols;
    float cell, y_min, y_max;
    std::vector<float> h;
};
// A triangle mesh: the registration's input (for snapshots), its
// centroid-relative triangle hulls, centroids, tree and permutation.
struct HostMesh {
    std::vector<float> verts;
    std::vector<uint32_t> tris_in;
    std::vector<HostHull> tris;
    std::vector<float4> cent;
    std::vector<MeshNodeD> nodes;
    std::vector<uint32_t> order;
    float bound, min_feature;
};

float shape_bound(uint32_t shape, const float* p, const std::vector<HostHull>& hulls,
                  const std::vector<HostExt>& exts) {  // rows.rs:253-292
    switch (shape) {
        case AVBD_SHAPE_ROUND:
        case AVBD_SHAPE_COMPOUND: {
            size_t id = (size_t)p[0];
            return id < exts.size() ? exts[id].bound : 0.0f;
        }
        case AVBD_SHAPE_SPHERE: return p[0];
        case AVBD_SHAPE_BOX: return std::sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]);
        case AVBD_SHAPE_CAPSULE: return p[1] + p[0];
        case AVBD_SHAPE_CYLINDER:
        case AVBD_SHAPE_CONE: return std::sqrt(p[0] * p[0] + p[1] * p[1]);
        case AVBD_SHAPE_HULL: {
            size_t id = (size_t)p[0];
            return id < hulls.size() ? hulls[id].bound : 0.0f;
        }
        default: return INFINITY;
    }
}
// Shape::inertia (collision/shape.rs:713-790)
void shape_inertia(uint32_t shape, const float* sp, float mass, float out[3]) {
    out[0] = out[1] = out[2] = 0.0f;
    if (!(mass > 0.0f) || !std::isfinite(mass)) return;
    if (shape == AVBD_SHAPE_SPHERE) {
        float v = 0.4f * mass * sp[0] * sp[0];
        out[0] = out[1] = out[2] = v;
    } else if (shape == AVBD_SHAPE_BOX) {
        float sx = sp[0] * 2.0f, sy = sp[1] * 2.0f, sz = sp[2] * 2.0f;
        float x = sx * sx, y = sy * sy, z = sz * sz;
        float k = mass / 12.0f;
        out[0] = k * (y + z);
        out[1] = k * (z + x);
        out[2] = k * (x + y);
    } else if (shape == AVBD_SHAPE_CAPSULE) {
        float r = sp[0], h = sp[1];
        float iy = 0.5f * mass * r * r;
        float ixz = 0.25f * mass * (r * r) + (mass / 3.0f) * h * r + 0.25f * mass * h * h;
        out[0] = ixz;
        out[1] = iy;
        out[2] = ixz;
    } else if (shape == AVBD_SHAPE_CYLINDER || shape == AVBD_SHAPE_CONE) {  // shape.rs:780-801
        float r = sp[0], h = sp[1];
        bool cyl = shape == AVBD_SHAPE_CYLINDER;
        float iy = (cyl ? 0.5f : 0.3f) * mass * r * r;
        float ixz = mass * (3.0f * r * r + (cyl ? 4.0f : 8.0f) * h * h) / (cyl ? 12.0f : 20.0f);
        out[0] = ixz;
        out[1] = iy;
        out[2] = ixz;
    }
}
// rest inertia of a body: its shape's, or the hull's per-unit-mass inertia times the mass
static void rest_inertia(const AvbdBody& b, float mass, const std::vector<HostHull>& hulls,
                         const std::vector<HostExt>& exts, float out[3]) {
    if (b.shape == AVBD_SHAPE_ROUND || b.shape == AVBD_SHAPE_COMPOUND) {
        size_t id = (size_t)b.shape_params[0];
        for (int k = 0; k < 3; k++)
            out[k] = (id < exts.size() && mass > 0.0f && std::isfinite(mass)) ? exts[id].unit_inertia[k] * mass : 0.0f;
        return;
    }
    if (b.shape != AVBD_SHAPE_HULL) {
        shape_inertia(b.shape, b.shape_params, mass, out);
        return;
    }
    size_t id = (size_t)b.shape_params[0];
    for (int k = 0; k < 3; k++)
        out[k] = (id < hulls.size() && mass > 0.0f && std::isfinite(mass)) ? hulls[id].unit_inertia[k] * mass : 0.0f;
}
float hinge_twist_host(const float qa[4], const float qb[4], const float ax[3]) {  // sequential_impulse/joints.rs:38-48
    // q = conj(qa) * qb (Hamilton product, avbd/rows.rs:91-98 order)
    float a0 = -qa[0], a1 = -qa[1], a2 = -qa[2], a3 = qa[3];
    float x = a3 * qb[0] + a0 * qb[3] + a1 * qb[2] - a2 * qb[1];
    float y = a3 * qb[1] - a0 * qb[2] + a1 * qb[3] + a2 * qb[0];
    float z = a3 * qb[2] + a0 * qb[1] - a1 * qb[0] + a2 * qb[3];
    float w = a3 * qb[3] - a0 * qb[0] - a1 * qb[1] - a2 * qb[2];
    float t = 2.0f * avbd::crm::atan2f((x * ax[0] + y * ax[1]) + z * ax[2], w);
    const float PI = 3.14159265358979323846f, TAU = 6.28318530717958647692f;
    float r = std::fmod(t + PI, TAU);
    if (r < 0.0f) r += std::fabs(TAU);
    return r - PI;
}

}  // namespace

namespace {
struct AdjTape;
void adj_free(AdjTape* t);
}  // namespace

struct AvbdWorld {
    AvbdParams prm;
    int device = 0;
    cudaStream_t st = nullptr;
    std::vector<uint32_t> scene_off{0};
    // host model (authoritative while host_valid)
    std::vector<AvbdBody> bodies;
    std::vector<AvbdBodyAux> aux;
    std::vector<AvbdPairState> pairs;
    std::vector<AvbdPointState> points;
    std::vector<JointRec> joints;
    bool host_valid = true;
    bool dev_valid = false;
    // device
    Alloc mem;
    DW w{};
    PairBuf pb[2]{};
    int cur = 0;  // pair buffer holding the current generation
    uint32_t n_alloc = 0, j_alloc = 0, cand_cap = 0;
    Tune tune;
    BroadphasePlan plan;
    uint32_t* d_small = nullptr;
    uint32_t* scan_tmp = nullptr;
    AvbdBody* d_stage = nullptr;
    uint32_t* h_ctr = nullptr;  // pinned copy of the device counters
    uint32_t ev_cap0 = 0;
    void* flush_buf = nullptr;  // L2 eviction scratch (avbd_world_flush_cache)
    AvbdCounters cum{};
    float time_debt = 0.0f;
    int last_ncol = 0;
    // graphs: one captured substep per pair-buffer parity, without and with events
    cudaGraphExec_t gexec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    // events: emitted on the last substep of each step call, or every
    // ev_period substeps of a fixed-step call; -1 turns them off
    int ev_period = 0;
    bool has_trig = false;
    Alloc evmem;  // the event queues: kept across reallocations of the world
    std::vector<HostHull> hulls;
    std::vector<HostExt> exts;  // rounded and compound shapes
    std::vector<HostHf> hfs;    // heightfields
    std::vector<HostMesh> meshes;  // triangle meshes
    Alloc hullmem;              // the hull, rounded, compound, terrain and mesh tables
    int graph_cols = 0;
    size_t graph_nodes = 0;       // kernel nodes in one captured substep (no events)
    size_t graph_nodes_emit = 0;  // ... in one that reports events
    uint64_t steps = 0;
    AdjTape* adj = nullptr;  // checkpoints of the last differentiable rollout
    uint64_t mem_gen = 0;    // bumped whenever the device arrays are (re)allocated or a launch setting changes
};

#define CK(x)                                    \
    do {                                         \
        cudaError_t e_ = (x);                    \
        if (e_ != cudaSuccess) {                 \
            fprintf(stderr, "ornis_avbd: %s: %s\n", #x, cudaGetErrorString(e_)); \
            return AVBD_ERR_DEVICE;              \
        }                                        \
    } while (0)

static void set_pair_ptrs(AvbdWorld* W) {
    PairBuf& c = W->pb[W->cur];
    PairBuf& o = W->pb[1 - W->cur];
    DW& w = W->w;
    w.p_ab = c.ab; w.p_n = c.n; w.p_mu = c.mu; w.p_np = c.np;
    w.q_ra = c.ra; w.q_rb = c.rb; w.q_lam = c.lam; w.q_pen = c.pen; w.q_roll = c.roll; w.q_matched = c.matched;
    w.p_old = c.old;
    w.offA = c.offA;
    w.o_ab = o.ab; w.o_n = o.n; w.o_np = o.np;
    w.oq_ra = o.ra; w.oq_rb = o.rb; w.oq_lam = o.lam; w.oq_pen = o.pen; w.oq_roll = o.roll;
    w.o_offA = o.offA;
}

// settings_changed: something a captured launch holds by value changed, so
// the recording graphs of a differentiable rollout are stale too.
static void free_graphs(AvbdWorld* W, bool settings_changed = true) {
    for (int i = 0; i < 2; i++)
        for (int e = 0; e < 2; e++)
            if (W->gexec[i][e]) {
                cudaGraphExecDestroy(W->gexec[i][e]);
                W->gexec[i][e] = nullptr;
            }
    if (settings_changed) W->mem_gen++;
}

// Capacities: candidates are bounded by the sweep-and-prune overlaps plus the
// half-space pairs; surviving pairs never outnumber candidates.
static uint32_t default_cand_cap(uint32_t n) { return 12u * n + 4096u; }

// The previous touch set (handle keyed, CSR by the higher handle) held on the
// device, read for a world of N bodies: bodies added since have no touches.
// Empty when the device holds none.
static void read_touch_set(AvbdWorld* W, uint32_t N, std::vector<uint32_t>& tof, std::vector<uint32_t>& tkeys) {
    tof.clear();
    tkeys.clear();
    if (!W->w.toff || !W->w.evs) return;
    uint32_t on = (uint32_t)W->w.N, par = 0;
    tof.resize(on + 1);
    cudaMemcpy(tof.data(), W->w.toff, (on + 1) * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&par, W->w.evs + EV_PAR, 4, cudaMemcpyDeviceToHost);
    tkeys.resize(tof[on]);
    if (!tkeys.empty())
        cudaMemcpy(tkeys.data(), (par & 1u) ? W->w.tk1 : W->w.tk0, tkeys.size() * 4, cudaMemcpyDeviceToHost);
    tof.resize(N + 1, tof[on]);
}

static int alloc_device(AvbdWorld* W, uint32_t N, uint32_t J, uint32_t cand_cap) {
    W->mem_gen++;
    // the previous touch set survives a reallocation
    std::vector<uint32_t> tof, tkeys;
    read_touch_set(W, N, tof, tkeys);
    W->mem.release();
    free_graphs(W);
    Alloc& m = W->mem;
    DW& w = W->w;
    const int sort_static = w.sort_static;  // settings of the world, not of the allocation
    const float joint_k = w.joint_k;
    w = DW{};
    w.sort_static = sort_static;
    w.joint_k = joint_k;
    uint32_t S = (uint32_t)W->scene_off.size() - 1;
    w.N = (int)N;
    w.S = (int)S;
    w.J = (int)J;
    w.cand_cap = cand_cap;
    w.pair_cap = cand_cap;
    w.scene_off = m.get<uint32_t>(S + 1);
    w.scene_of = m.get<uint32_t>(N);
    w.plane_off = m.get<uint32_t>(S + 1);
    w.plane_list = m.get<uint32_t>(N);
    w.pos = m.get<float4>(N); w.rot = m.get<float4>(N); w.vel = m.get<float4>(N);
    w.angvel = m.get<float4>(N); w.torque = m.get<float4>(N);
    w.pos0 = m.get<float4>(N); w.rot0 = m.get<float4>(N);
    w.inertial = m.get<float4>(N); w.inertial_rot = m.get<float4>(N);
    w.prev_pos = m.get<float4>(N); w.prev_rot = m.get<float4>(N);
    w.inertia = m.get<float4>(N); w.inertia_rest = m.get<float4>(N);
    w.kin = m.get<float4>((size_t)N * 4);
    w.mat = m.get<float4>(N); w.shp = m.get<float4>(N);
    w.inv_mass = m.get<float>(N); w.inv_mass_rest = m.get<float>(N); w.mass = m.get<float>(N);
    w.friction_t = m.get<float>(N); w.sleep_timer = m.get<float>(N);
    w.info = m.get<uint32_t>(N); w.asleep = m.get<uint32_t>(N);
    w.filter = m.get<uint2>(N);
    w.colour = m.get<int32_t>(N);
    w.comp = m.get<int32_t>(N);
    w.j_kind = m.get<uint32_t>(J); w.j_ab = m.get<uint2>(J);
    w.j_la = m.get<float4>(J); w.j_lb = m.get<float4>(J); w.j_axa = m.get<float4>(J); w.j_axb = m.get<float4>(J);
    w.j_lim = m.get<float4>(J);
    w.j_ref = m.get<float4>(J); w.j_dref = m.get<float4>(J); w.j_qref = m.get<float4>(J);
    w.j_cfg = m.get<uint32_t>(J); w.j_six = m.get<float4>(3 * (size_t)J); w.j_sacc = m.get<float4>(2 * (size_t)J);
    w.jimp_off = m.get<uint32_t>(S + 1);
    w.jimp_list = m.get<uint32_t>(J);
    w.j_lam_l = m.get<float4>(J); w.j_lam_a = m.get<float4>(J); w.j_pen_l = m.get<float4>(J); w.j_pen_a = m.get<float4>(J);
    w.j_gb = m.get<uint2>(J); w.j_gmem = m.get<float4>(J); w.j_gset = m.get<uint32_t>(J);
    w.jofs = m.get<uint32_t>(N + 1);
    w.jlist = m.get<uint32_t>(4 * (size_t)J);
    for (int b = 0; b < 2; b++) {
        PairBuf& p = W->pb[b];
        p.ab = m.get<uint2>(cand_cap); p.n = m.get<float4>(cand_cap); p.mu = m.get<float2>(cand_cap);
        p.np = m.get<uint32_t>(cand_cap);
        size_t q = (size_t)cand_cap * MAX_PTS;
        p.ra = m.get<float4>(q); p.rb = m.get<float4>(q); p.lam = m.get<float4>(q); p.pen = m.get<float4>(q);
        p.roll = m.get<float4>(q); p.matched = m.get<int32_t>(q);
        p.old = m.get<int32_t>(cand_cap);
        p.offA = m.get<uint32_t>(N + 1);
    }
    w.offB = m.get<uint32_t>(N + 1);
    w.listB = m.get<uint32_t>(cand_cap);
    w.posB = m.get<uint32_t>(cand_cap);
    w.side_list = m.get<uint32_t>((size_t)cand_cap * 2);
    w.side_cnt = m.get<uint32_t>(2 * MAX_COLOURS + 2);
    // the split primal's per-incidence partial systems (the per-scene solve
    // falls back to the split launches when a scene is above its limit)
    uint32_t max_scene = 0;
    for (uint32_t s = 0; s < S; s++) max_scene = std::max(max_scene, W->scene_off[s + 1] - W->scene_off[s]);
    w.max_scene = max_scene;
    const bool need_contrib = W->tune.primal_lanes == 0 ||
                              (W->tune.primal_lanes < 0 && max_scene > (uint32_t)SCENE_MAX_BODIES);
    w.contrib = need_contrib ? m.get<float4>((size_t)cand_cap * 2 * 7) : nullptr;
    w.contrib_slots = w.contrib ? (uint32_t)(cand_cap * 2) : 0u;
    w.cand = m.get<uint2>(cand_cap);
    w.keep = m.get<uint8_t>(cand_cap);
    w.cnt = m.get<uint32_t>(N + 1);
    w.cur = m.get<uint32_t>(N + 1);
    w.slot_c = m.get<uint32_t>(cand_cap);
    w.long_seg = m.get<uint32_t>(N);
    w.seg_key = m.get<unsigned long long>(cand_cap);
    w.boxlist = m.get<uint32_t>(cand_cap);
    w.clist = m.get<uint32_t>(cand_cap);
    w.bd_pa = m.get<float4>(cand_cap);
    w.bd_pb = m.get<float4>(cand_cap);
    w.aabb_lo = m.get<float4>(N); w.aabb_hi = m.get<float4>(N);
    // large-scene sort scratch
    uint32_t max_large = 0;
    std::vector<uint32_t> small;
    W->plan.large.clear();
    for (uint32_t s = 0; s < S; s++) {
        uint32_t n = W->scene_off[s + 1] - W->scene_off[s];
        if (n <= (uint32_t)W->tune.small_scene_max) small.push_back(s);
        else {
            W->plan.large.push_back({W->scene_off[s], W->scene_off[s + 1]});
            max_large = std::max(max_large, n);
        }
    }
    w.n_large_scenes = (int)W->plan.large.size();
    w.sort_key = m.get<uint32_t>(max_large);
    w.sort_idx = m.get<uint32_t>(max_large);
    W->plan.keys_alt = m.get<uint32_t>(max_large);
    W->plan.vals_alt = m.get<uint32_t>(max_large);
    W->plan.hist = m.get<uint32_t>(radix_hist_words(max_large));
    W->plan.rows = W->tune.sweep_rows;
    W->plan.row_key = m.get<uint32_t>(max_large);
    W->plan.ext = m.get<float>(W->plan.large.size());
    size_t scan_words = std::max({scan_tmp_words((size_t)N + 1), scan_tmp_words(radix_hist_words(max_large)),
                                  scan_tmp_words(radix_hist_words(N))});
    W->scan_tmp = m.get<uint32_t>(scan_words + 16);
    W->plan.scan_tmp = W->scan_tmp;
    W->d_small = m.get<uint32_t>(small.size());
    if (!small.empty())
        cudaMemcpy(W->d_small, small.data(), small.size() * 4, cudaMemcpyHostToDevice);
    {
        // the per-scene solve's queue: largest scenes first (ties by index)
        std::vector<uint32_t> order(S);
        for (uint32_t s = 0; s < S; s++) order[s] = s;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
            return W->scene_off[a + 1] - W->scene_off[a] > W->scene_off[b + 1] - W->scene_off[b];
        });
        uint32_t* d = m.get<uint32_t>(S);
        if (S) cudaMemcpy(d, order.data(), S * 4, cudaMemcpyHostToDevice);
        w.scene_order = d;
    }
    W->plan.small_scenes = W->d_small;
    W->plan.n_small = (int)small.size();
    w.fbody = m.get<uint32_t>(N);
    w.fcand = m.get<uint32_t>(cand_cap);
    w.fast = m.get<uint8_t>(N);
    w.ccd_best = m.get<unsigned long long>(N);
    w.ccd_deps = m.get<uint32_t>(N);
    w.ccd_state = m.get<uint8_t>(N);
    w.ccd_recompute = m.get<uint8_t>(N);
    if (W->prm.enable_ccd) {
        w.ccd_hit_cap = std::max(4096u, cand_cap / 4u);
        w.ccd_hit = m.get<float4>((size_t)w.ccd_hit_cap * 3);
        w.ccd_win = m.get<uint32_t>(N);
    }
    w.ccd_rec = W->prm.enable_ccd ? m.get<float4>(2 * N) : nullptr;
    w.flag = m.get<uint8_t>(N);
    w.comp_flag = m.get<uint32_t>(N);
    // events
    w.pre_vel = m.get<float4>(N);
    if (W->prm.enable_ccd) {
        w.ccd_ev_o = m.get<int32_t>(N);
        w.ccd_ev_p = m.get<float4>(N);
        w.ccd_ev_n = m.get<float4>(N);
    }
    w.t_flag = m.get<uint8_t>(cand_cap);
    w.t_wit = m.get<float4>(cand_cap);
    w.toff = m.get<uint32_t>(N + 1);
    w.tk0 = m.get<uint32_t>(cand_cap);
    w.tk1 = m.get<uint32_t>(cand_cap);
    w.ev_cbe = m.get<uint32_t>(N + 1);
    w.ev_ch = m.get<uint32_t>(N + 1);
    w.ev_cc = m.get<uint32_t>(N + 1);
    w.ev_ct = m.get<uint32_t>(N + 1);
    if (W->evmem.ptrs.empty()) {
        W->evmem.get<uint32_t>(EV_NUM);
        W->evmem.get<AvbdContactEvent>(std::max<uint32_t>(65536u, 2u * N));
        W->evmem.get<AvbdTriggerEvent>(65536u);
        W->evmem.get<unsigned long long>(TRIG_CAP);
        W->evmem.get<unsigned long long>(TRIG_CAP);
        W->ev_cap0 = std::max<uint32_t>(65536u, 2u * N);
    }
    if (W->evmem.ptrs.size() != 5) return AVBD_ERR_DEVICE;
    w.evs = (uint32_t*)W->evmem.ptrs[0];
    w.ev = (AvbdContactEvent*)W->evmem.ptrs[1];
    w.ev_cap = W->ev_cap0;
    w.tev = (AvbdTriggerEvent*)W->evmem.ptrs[2];
    w.tev_cap = 65536u;
    w.trig_now = (unsigned long long*)W->evmem.ptrs[3];
    w.trig_prev = (unsigned long long*)W->evmem.ptrs[4];
    if (!tof.empty()) {
        uint32_t par = 0;
        cudaMemcpy(&par, w.evs + EV_PAR, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(w.toff, tof.data(), (N + 1) * 4, cudaMemcpyHostToDevice);
        if (!tkeys.empty())
            cudaMemcpy((par & 1u) ? w.tk1 : w.tk0, tkeys.data(), tkeys.size() * 4, cudaMemcpyHostToDevice);
    }
    w.col_cnt = m.get<uint32_t>(2 * MAX_COLOURS + 2);
    w.col_list = m.get<uint32_t>(N);
    w.col_key = m.get<uint32_t>(N);
    w.col_key2 = m.get<uint32_t>(N);
    w.col_val = m.get<uint32_t>(N);
    w.col_hist = m.get<uint32_t>(radix_hist_words(N));
    w.ctr = m.get<uint32_t>(C_NUM);
    W->d_stage = m.get<AvbdBody>(N);
    for (void* p : m.ptrs)
        if (!p) return AVBD_ERR_DEVICE;
    if (!w.ctr || !W->d_stage) return AVBD_ERR_DEVICE;
    W->n_alloc = N;
    W->j_alloc = J;
    W->cand_cap = cand_cap;
    w.dt = W->prm.step_dt;
    w.gravity = V3{W->prm.gravity[0], W->prm.gravity[1], W->prm.gravity[2]};
    w.iterations = W->prm.iterations;
    w.enable_sleep = W->prm.enable_sleep;
    w.enable_ccd = W->prm.enable_ccd;
    w.max_cols = MAX_COLOURS;
    set_pair_ptrs(W);
    return AVBD_OK;
}

// ---- AoS <-> SoA kernels ----------------------------------------------------------
__global__ void k_bodies_in(DW w, const AvbdBody* in, uint32_t first, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const AvbdBody& b = in[i];
    uint32_t h = first + i;
    w.pos[h] = make_float4(b.position[0], b.position[1], b.position[2], 0.0f);
    w.rot[h] = make_float4(b.orientation[0], b.orientation[1], b.orientation[2], b.orientation[3]);
    w.vel[h] = make_float4(b.velocity[0], b.velocity[1], b.velocity[2], 0.0f);
    w.angvel[h] = make_float4(b.angular_velocity[0], b.angular_velocity[1], b.angular_velocity[2], 0.0f);
    w.torque[h] = make_float4(b.torque[0], b.torque[1], b.torque[2], 0.0f);
    w.mass[h] = b.mass;
    w.inv_mass[h] = b.inv_mass;
    w.inertia[h] = make_float4(b.inertia[0], b.inertia[1], b.inertia[2], 0.0f);
    w.mat[h] = make_float4(b.restitution, b.friction, b.rolling_friction, b.torsion_friction);
    w.friction_t[h] = b.friction_transverse;
    w.filter[h] = make_uint2(b.collision_layer, b.collision_mask);
}
__global__ void k_bodies_out(DW w, AvbdBody* out, uint32_t first, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    AvbdBody& b = out[i];
    uint32_t h = first + i;
    float4 p = w.pos[h], q = w.rot[h], v = w.vel[h], om = w.angvel[h], tq = w.torque[h], in = w.inertia[h];
    b.position[0] = p.x; b.position[1] = p.y; b.position[2] = p.z;
    b.orientation[0] = q.x; b.orientation[1] = q.y; b.orientation[2] = q.z; b.orientation[3] = q.w;
    b.velocity[0] = v.x; b.velocity[1] = v.y; b.velocity[2] = v.z;
    b.angular_velocity[0] = om.x; b.angular_velocity[1] = om.y; b.angular_velocity[2] = om.z;
    b.torque[0] = tq.x; b.torque[1] = tq.y; b.torque[2] = tq.z;
    b.mass = w.mass[h];
    b.inv_mass = w.inv_mass[h];
    b.inertia[0] = in.x; b.inertia[1] = in.y; b.inertia[2] = in.z;
    float4 m = w.mat[h];
    b.restitution = m.x; b.friction = m.y; b.rolling_friction = m.z; b.torsion_friction = m.w;
    b.friction_transverse = w.friction_t[h];
    uint32_t info = w.info[h];
    b.shape = info_shape(info);
    float4 sp = w.shp[h];
    b.shape_params[0] = sp.x; b.shape_params[1] = sp.y; b.shape_params[2] = sp.z;
    uint2 f = w.filter[h];
    b.collision_layer = f.x; b.collision_mask = f.y;
    b.body_type = info_type(info);
    b.flags = info_trigger(info) ? AVBD_FLAG_TRIGGER : 0u;
}

static bool body_finite(const AvbdBody& b) {
    const float* f = b.position;
    for (int i = 0; i < 16; i++)
        if (!std::isfinite(f[i])) return false;
    return std::isfinite(b.mass) && std::isfinite(b.inv_mass);
}

// Upload the whole host model: bodies, aux, joints, pairs.
static int upload_all(AvbdWorld* W) {
    uint32_t N = (uint32_t)W->bodies.size();
    uint32_t J = (uint32_t)W->joints.size();
    uint32_t S = (uint32_t)W->scene_off.size() - 1;
    if (N == 0) return AVBD_OK;
    uint32_t need = std::max(default_cand_cap(N), (uint32_t)W->pairs.size() + 1024u);
    {
        // terrain and meshes pair with every body of their scene (no bound)
        uint64_t extra = 0;
        for (uint32_t s = 0; s + 1 < (uint32_t)W->scene_off.size(); s++) {
            uint64_t t = 0;
            for (uint32_t h = W->scene_off[s]; h < W->scene_off[s + 1]; h++)
                t += W->bodies[h].shape == AVBD_SHAPE_HEIGHTFIELD || W->bodies[h].shape == AVBD_SHAPE_TRIMESH;
            extra += t * (W->scene_off[s + 1] - W->scene_off[s]);
        }
        need = (uint32_t)std::min<uint64_t>((uint64_t)need + extra, 0x7fffffffull);
    }
    if (N != W->n_alloc || J != W->j_alloc || need > W->cand_cap || !W->w.ctr) {
        uint32_t cap = std::max(need, W->cand_cap);
        int rc = alloc_device(W, N, J, cap);
        if (rc) return rc;
    }
    DW& w = W->w;
    cudaStream_t st = W->st;
    // convex hull tables (rebuilt on every full upload: hulls are few and small)
    W->hullmem.release();
    w.hulls = nullptr;
    w.nhulls = 0;
    if (!W->hulls.empty()) {
        size_t nv = 0, nf = 0;
        for (const HostHull& h : W->hulls) {
            nv += h.v.size();
            nf += h.f.size();
        }
        float4* dv = W->hullmem.get<float4>(nv);
        uint32_t* df = W->hullmem.get<uint32_t>(nf);
        HullDesc* dd = W->hullmem.get<HullDesc>(W->hulls.size());
        if (!dv || !df || !dd) return AVBD_ERR_DEVICE;
        std::vector<HullDesc> desc;
        size_t ov = 0, of = 0;
        for (const HostHull& h : W->hulls) {
            if (!h.v.empty()) CK(cudaMemcpy(dv + ov, h.v.data(), h.v.size() * 16, cudaMemcpyHostToDevice));
            if (!h.f.empty()) CK(cudaMemcpy(df + of, h.f.data(), h.f.size() * 4, cudaMemcpyHostToDevice));
            desc.push_back(HullDesc{dv + ov, df + of, (uint32_t)h.v.size(), (uint32_t)(h.f.size() / 3), h.bound,
                                    h.min_ext});
            ov += h.v.size();
            of += h.f.size();
        }
        CK(cudaMemcpy(dd, desc.data(), desc.size() * sizeof(HullDesc), cudaMemcpyHostToDevice));
        w.hulls = dd;
        w.nhulls = (uint32_t)desc.size();
    }
    // rounded and compound tables, after the hulls their parts point at
    w.exts = nullptr;
    w.parts = nullptr;
    w.nexts = 0;
    if (!W->exts.empty()) {
        size_t np = 0;
        for (const HostExt& e : W->exts) np += e.parts.size();
        ExtDesc* de = W->hullmem.get<ExtDesc>(W->exts.size());
        PartDesc* dp = W->hullmem.get<PartDesc>(np);
        if (!de || !dp) return AVBD_ERR_DEVICE;
        std::vector<ExtDesc> ed;
        std::vector<PartDesc> pd;
        for (const HostExt& e : W->exts) {
            ed.push_back(ExtDesc{(uint32_t)pd.size(), (uint32_t)e.parts.size(), e.compound ? 1u : 0u, e.min_dim});
            for (const AvbdShapePart& q : e.parts) {
                PartDesc d{};
                d.p = make_float4(q.params[0], q.params[1], q.params[2], q.border_radius);
                d.pos = make_float4(q.position[0], q.position[1], q.position[2], 0.0f);
                d.rot = make_float4(q.orientation[0], q.orientation[1], q.orientation[2], q.orientation[3]);
                d.kind = q.shape;
                d.hull = q.shape == AVBD_SHAPE_HULL ? w.hulls + (size_t)q.params[0] : nullptr;
                pd.push_back(d);
            }
        }
        CK(cudaMemcpy(de, ed.data(), ed.size() * sizeof(ExtDesc), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dp, pd.data(), pd.size() * sizeof(PartDesc), cudaMemcpyHostToDevice));
        w.exts = de;
        w.parts = dp;
        w.nexts = (uint32_t)ed.size();
    }
    w.hfs = nullptr;
    w.meshes = nullptr;
    w.nhfs = w.nmeshes = 0;
    if (!W->hfs.empty()) {
        std::vector<HfDesc> hd;
        for (const HostHf& f : W->hfs) {
            float* dh = W->hullmem.get<float>(f.h.size());
            if (!dh) return AVBD_ERR_DEVICE;
            CK(cudaMemcpy(dh, f.h.data(), f.h.size() * 4, cudaMemcpyHostToDevice));
            hd.push_back(HfDesc{dh, f.rows, f.cols, f.cell, f.y_min});
        }
        HfDesc* dd = W->hullmem.get<HfDesc>(hd.size());
        if (!dd) return AVBD_ERR_DEVICE;
        CK(cudaMemcpy(dd, hd.data(), hd.size() * sizeof(HfDesc), cudaMemcpyHostToDevice));
        w.hfs = dd;
        w.nhfs = (uint32_t)hd.size();
    }
    if (!W->meshes.empty()) {
        std::vector<MeshDesc> md;
        for (const HostMesh& m : W->meshes) {
            MeshDesc d{};
            d.ntris = (uint32_t)m.tris.size();
            d.nnodes = (uint32_t)m.nodes.size();
            d.norder = (uint32_t)m.order.size();
            d.min_feature = m.min_feature;
            std::vector<HullDesc> th;
            float4* dv = W->hullmem.get<float4>(3 * m.tris.size());
            uint32_t* df = W->hullmem.get<uint32_t>(6 * m.tris.size());
            HullDesc* dt = W->hullmem.get<HullDesc>(m.tris.size());
            float4* dc = W->hullmem.get<float4>(m.cent.size());
            MeshNodeD* dn = W->hullmem.get<MeshNodeD>(m.nodes.size());
            uint32_t* dord = W->hullmem.get<uint32_t>(m.order.size());
            if (!dv || !df || !dt || !dc || !dn || !dord) return AVBD_ERR_DEVICE;
            for (size_t t = 0; t < m.tris.size(); t++) {
                const HostHull& hh = m.tris[t];
                CK(cudaMemcpy(dv + 3 * t, hh.v.data(), 3 * 16, cudaMemcpyHostToDevice));
                CK(cudaMemcpy(df + 6 * t, hh.f.data(), 6 * 4, cudaMemcpyHostToDevice));
                th.push_back(HullDesc{dv + 3 * t, df + 6 * t, 3u, 2u, hh.bound, hh.min_ext});
            }
            if (!th.empty()) CK(cudaMemcpy(dt, th.data(), th.size() * sizeof(HullDesc), cudaMemcpyHostToDevice));
            if (!m.cent.empty()) CK(cudaMemcpy(dc, m.cent.data(), m.cent.size() * 16, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(dn, m.nodes.data(), m.nodes.size() * sizeof(MeshNodeD), cudaMemcpyHostToDevice));
            if (!m.order.empty()) CK(cudaMemcpy(dord, m.order.data(), m.order.size() * 4, cudaMemcpyHostToDevice));
            d.tris = dt;
            d.cent = dc;
            d.nodes = dn;
            d.order = dord;
            md.push_back(d);
        }
        MeshDesc* dd = W->hullmem.get<MeshDesc>(md.size());
        if (!dd) return AVBD_ERR_DEVICE;
        CK(cudaMemcpy(dd, md.data(), md.size() * sizeof(MeshDesc), cudaMemcpyHostToDevice));
        w.meshes = dd;
        w.nmeshes = (uint32_t)md.size();
    }
    for (uint32_t h = 0; h < N; h++) {
        const AvbdBody& b = W->bodies[h];
        if (b.shape > AVBD_SHAPE_TRIMESH) return AVBD_ERR_UNSUPPORTED;
        if (b.shape == AVBD_SHAPE_HEIGHTFIELD || b.shape == AVBD_SHAPE_TRIMESH) {
            // static colliders (shape.rs:181-192): no moving terrain or mesh
            if (b.body_type == AVBD_BODY_DYNAMIC) return AVBD_ERR_UNSUPPORTED;
            const size_t id = (size_t)b.shape_params[0];
            const size_t n = b.shape == AVBD_SHAPE_HEIGHTFIELD ? W->hfs.size() : W->meshes.size();
            if (!(b.shape_params[0] >= 0.0f && id < n)) return AVBD_ERR_INVALID_ARG;
        }
        if (b.shape == AVBD_SHAPE_HULL && !((size_t)b.shape_params[0] < W->hulls.size()))
            return AVBD_ERR_INVALID_ARG;  // names a hull that was never added
        if (b.shape == AVBD_SHAPE_ROUND || b.shape == AVBD_SHAPE_COMPOUND) {
            const size_t id = (size_t)b.shape_params[0];
            if (!(b.shape_params[0] >= 0.0f && id < W->exts.size()) ||
                W->exts[id].compound != (b.shape == AVBD_SHAPE_COMPOUND))
                return AVBD_ERR_INVALID_ARG;  // names no shape of its kind
        }
    }
    // static per-body data
    std::vector<uint32_t> scene_of(N), info(N);
    std::vector<float4> shp(N), inertia_rest(N);
    std::vector<float> inv_rest(N), timer(N);
    std::vector<uint32_t> asleep(N);
    std::vector<float4> prev_pos(N), prev_rot(N);
    std::vector<uint32_t> plane_off(S + 1, 0), plane_list;
    for (uint32_t s = 0; s < S; s++) {
        plane_off[s] = (uint32_t)plane_list.size();
        for (uint32_t h = W->scene_off[s]; h < W->scene_off[s + 1]; h++) {
            scene_of[h] = s;
            const uint32_t k = W->bodies[h].shape;  // half-spaces, terrain, meshes
            if (k == AVBD_SHAPE_HALFSPACE || k == AVBD_SHAPE_HEIGHTFIELD || k == AVBD_SHAPE_TRIMESH)
                plane_list.push_back(h);
        }
    }
    plane_off[S] = (uint32_t)plane_list.size();
    W->has_trig = false;
    for (uint32_t h = 0; h < N; h++) {
        const AvbdBody& b = W->bodies[h];
        if (b.flags & AVBD_FLAG_TRIGGER) W->has_trig = true;
        info[h] = (b.shape & 15u) | ((b.body_type & 3u) << 4) | ((b.flags & AVBD_FLAG_TRIGGER) ? 64u : 0u);
        shp[h] = make_float4(b.shape_params[0], b.shape_params[1], b.shape_params[2],
                             shape_bound(b.shape, b.shape_params, W->hulls, W->exts));
        float in[3];
        bool free_mass = b.mass > 0.0f && std::isfinite(b.mass);
        rest_inertia(b, free_mass ? b.mass : 0.0f, W->hulls, W->exts, in);
        inertia_rest[h] = make_float4(in[0], in[1], in[2], 0.0f);
        inv_rest[h] = free_mass ? 1.0f / b.mass : 0.0f;
        const AvbdBodyAux& a = W->aux[h];
        timer[h] = a.sleep_timer;
        asleep[h] = a.asleep;
        prev_pos[h] = make_float4(a.prev_position[0], a.prev_position[1], a.prev_position[2], 0.0f);
        prev_rot[h] = make_float4(a.prev_orientation[0], a.prev_orientation[1], a.prev_orientation[2], a.prev_orientation[3]);
    }
    // joints: adjacency (ascending joint index per body; a gear on each body
    // of its coupled joints) and components over the dynamic members of each
    // joint (sleep.rs:152-175)
    std::vector<uint32_t> jofs(N + 1, 0), jlist;
    {
        uint32_t m[4];
        for (uint32_t ji = 0; ji < J; ji++) {
            const int nm = joint_members_host(W->joints, ji, m);
            for (int k = 0; k < nm; k++) jofs[m[k] + 1]++;
        }
        for (uint32_t h = 0; h < N; h++) jofs[h + 1] += jofs[h];
        jlist.resize(jofs[N]);
        std::vector<uint32_t> curj(jofs.begin(), jofs.end() - 1);
        for (uint32_t ji = 0; ji < J; ji++) {
            const int nm = joint_members_host(W->joints, ji, m);
            for (int k = 0; k < nm; k++) jlist[curj[m[k]]++] = ji;
        }
    }
    std::vector<int32_t> parent(N);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int32_t x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    std::vector<uint8_t> in_joint(N, 0);
    for (uint32_t ji = 0; ji < J; ji++) {
        uint32_t m[4], d[4];
        const int nm = joint_members_host(W->joints, ji, m);
        int nd = 0;
        for (int k = 0; k < nm; k++)
            if (W->bodies[m[k]].body_type == AVBD_BODY_DYNAMIC) d[nd++] = m[k];
        if (nd < 2) continue;  // one dynamic member wakes or freezes only itself
        for (int k = 0; k < nd; k++) {
            in_joint[d[k]] = 1;
            int32_t ra = find((int32_t)d[k]), rb = find((int32_t)d[0]);
            if (ra != rb) parent[ra] = rb;
        }
    }
    std::vector<int32_t> comp(N, -1);
    for (uint32_t h = 0; h < N; h++)
        if (in_joint[h]) comp[h] = find((int32_t)h);
    std::vector<uint32_t> j_kind(J), j_cfg(J);
    std::vector<uint2> j_ab(J);
    std::vector<float4> j_la(J), j_lb(J), j_axa(J), j_axb(J), j_lim(J), jll(J), jla(J), jpl(J), jpa(J);
    std::vector<float4> j_ref(J), j_dref(J), j_qref(J), j_six(3 * (size_t)J), j_sacc(2 * (size_t)J);
    // joints with a motor or a rope, per scene in joint order
    std::vector<uint32_t> jimp_off(S + 1, 0), jimp_list;
    {
        std::vector<std::vector<uint32_t>> per(S);
        for (uint32_t i = 0; i < J; i++) {
            const JointRec& j = W->joints[i];
            if (j.mot_max > 0.0f || j.kind == AVBD_JOINT_ROPE || j.kind == AVBD_JOINT_MOTOR)
                per[scene_of[j.a]].push_back(i);
        }
        for (uint32_t sc = 0; sc < S; sc++) {
            jimp_off[sc] = (uint32_t)jimp_list.size();
            jimp_list.insert(jimp_list.end(), per[sc].begin(), per[sc].end());
        }
        jimp_off[S] = (uint32_t)jimp_list.size();
        w.n_imp = (int)jimp_list.size();
    }
    for (uint32_t i = 0; i < J; i++) {
        const JointRec& j = W->joints[i];
        j_kind[i] = j.kind;
        j_cfg[i] = j.cfg;
        j_lim[i] = make_float4(j.lo, j.hi, j.has_lim ? 1.0f : 0.0f, j.st.acc_lim);
        j_ref[i] = make_float4(j.refv, j.st.lim_dual, j.mot_speed, j.mot_max);
        j_dref[i] = make_float4(j.dref[0], j.dref[1], j.dref[2], 0.0f);
        j_qref[i] = make_float4(j.qref[0], j.qref[1], j.qref[2], j.qref[3]);
        for (int k = 0; k < 3; k++)
            j_six[3 * (size_t)i + k] = make_float4(j.six_min[2 * k], j.six_max[2 * k], j.six_min[2 * k + 1],
                                                   j.six_max[2 * k + 1]);
        j_sacc[2 * (size_t)i] = make_float4(j.st.sacc[0], j.st.sacc[1], j.st.sacc[2], j.st.sacc[3]);
        j_sacc[2 * (size_t)i + 1] = make_float4(j.st.sacc[4], j.st.sacc[5], 0.0f, 0.0f);
        j_ab[i] = make_uint2(j.a, j.b);
        j_la[i] = make_float4(j.la[0], j.la[1], j.la[2], 0.0f);
        j_lb[i] = make_float4(j.lb[0], j.lb[1], j.lb[2], 0.0f);
        j_axa[i] = make_float4(j.axa[0], j.axa[1], j.axa[2], j.ref);
        j_axb[i] = make_float4(j.axb[0], j.axb[1], j.axb[2], 0.0f);
        if (j.kind == AVBD_JOINT_MOTOR) {
            // a free motor has no axes: its targets ride in the axis slots and
            // its budgets in the motor slots of j_ref
            j_axa[i] = make_float4(j.mlin[0], j.mlin[1], j.mlin[2], 0.0f);
            j_axb[i] = make_float4(j.mang[0], j.mang[1], j.mang[2], 0.0f);
            j_ref[i] = make_float4(0.0f, 0.0f, j.mforce, j.mtorque);
        }
        if (j.kind == AVBD_JOINT_SPRING) {
            // a spring has no axes: its motor rides in the B-axis slot, its
            // kind and model in the configuration word
            j_axb[i] = make_float4(j.spr[0], j.spr[1], j.spr[2], j.spr[3]);
            j_cfg[i] = j.spr_mode;
        }
        if (j.kind == AVBD_JOINT_GEAR) {
            // a gear's ratio rides in the weld-offset slot, its constant in j_ref.x
            j_dref[i] = make_float4(j.gratio, 0.0f, 0.0f, 0.0f);
            j_ref[i] = make_float4(j.refv, 0.0f, 0.0f, 0.0f);
        }
        if (j.kind == AVBD_JOINT_WHEEL) {
            // a wheel's axles ride in the weld-reference slots, its suspension
            // in the limit slot (a wheel has no limit: has_limit stays 0)
            j_dref[i] = make_float4(j.bxa[0], j.bxa[1], j.bxa[2], 0.0f);
            j_qref[i] = make_float4(j.bxb[0], j.bxb[1], j.bxb[2], 0.0f);
            j_lim[i] = make_float4(j.susp[0], j.susp[1], 0.0f, j.st.acc_lim);
        }
        jll[i] = make_float4(j.st.lam_l[0], j.st.lam_l[1], j.st.lam_l[2], 0.0f);
        jla[i] = make_float4(j.st.lam_a[0], j.st.lam_a[1], j.st.lam_a[2], 0.0f);
        jpl[i] = make_float4(j.st.pen_l[0], j.st.pen_l[1], j.st.pen_l[2], 0.0f);
        jpa[i] = make_float4(j.st.pen_a[0], j.st.pen_a[1], j.st.pen_a[2], 0.0f);
    }
    // pairs: current generation, sorted by (a, b), CSR by a
    std::vector<uint32_t> order(W->pairs.size());
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const AvbdPairState &p = W->pairs[x], &q = W->pairs[y];
        return p.a != q.a ? p.a < q.a : p.b < q.b;
    });
    uint32_t P = (uint32_t)order.size();
    std::vector<uint2> pab(P);
    std::vector<float4> pn(P);
    std::vector<float2> pmu(P);
    std::vector<uint32_t> pnp(P), offA(N + 1, 0);
    std::vector<float4> qra((size_t)P * MAX_PTS), qrb((size_t)P * MAX_PTS), qlam((size_t)P * MAX_PTS),
        qpen((size_t)P * MAX_PTS), qroll((size_t)P * MAX_PTS);
    std::vector<int32_t> qm((size_t)P * MAX_PTS, -1);
    for (uint32_t i = 0; i < P; i++) {
        const AvbdPairState& s = W->pairs[order[i]];
        pab[i] = make_uint2(s.a, s.b);
        pn[i] = make_float4(s.normal[0], s.normal[1], s.normal[2], s.gap);
        pmu[i] = make_float2(s.mu[0], s.mu[1]);
        pnp[i] = std::min<uint32_t>(s.npoints, MAX_PTS);
        offA[s.a + 1]++;
        for (int k = 0; k < MAX_PTS; k++) {
            const AvbdPointState& q = W->points[(size_t)order[i] * MAX_PTS + k];
            size_t d = (size_t)i * MAX_PTS + k;
            qra[d] = make_float4(q.ra[0], q.ra[1], q.ra[2], 0.0f);
            qrb[d] = make_float4(q.rb[0], q.rb[1], q.rb[2], q.stuck ? 1.0f : 0.0f);
            qlam[d] = make_float4(q.lam[0], q.lam[1], q.lam[2], 0.0f);
            qpen[d] = make_float4(q.pen[0], q.pen[1], q.pen[2], 0.0f);
            qroll[d] = make_float4(q.roll_lam[0], q.roll_lam[1], q.roll_lam[2], 0.0f);
            qm[d] = q.matched;
        }
    }
    for (uint32_t h = 0; h < N; h++) offA[h + 1] += offA[h];
    // B-side incidence of the uploaded pairs (read by the next discovery's
    // old-pair lookup): per body, pair indices ascending
    std::vector<uint32_t> offB(N + 1, 0), listB(std::max<uint32_t>(P, 1));
    for (uint32_t i = 0; i < P; i++) offB[pab[i].y + 1]++;
    for (uint32_t h = 0; h < N; h++) offB[h + 1] += offB[h];
    {
        std::vector<uint32_t> cb(offB.begin(), offB.end() - 1);
        for (uint32_t i = 0; i < P; i++) listB[cb[pab[i].y]++] = i;
    }
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    up((void*)w.scene_off, W->scene_off.data(), (S + 1) * 4);
    up((void*)w.scene_of, scene_of.data(), N * 4);
    up((void*)w.plane_off, plane_off.data(), (S + 1) * 4);
    up((void*)w.plane_list, plane_list.data(), plane_list.size() * 4);
    up(w.info, info.data(), N * 4);
    up(w.shp, shp.data(), N * 16);
    up(w.inertia_rest, inertia_rest.data(), N * 16);
    up(w.inv_mass_rest, inv_rest.data(), N * 4);
    up(w.sleep_timer, timer.data(), N * 4);
    up(w.asleep, asleep.data(), N * 4);
    up(w.prev_pos, prev_pos.data(), N * 16);
    up(w.prev_rot, prev_rot.data(), N * 16);
    up(w.comp, comp.data(), N * 4);
    up((void*)w.jofs, jofs.data(), (N + 1) * 4);
    up((void*)w.jlist, jlist.data(), jlist.size() * 4);
    up(w.j_kind, j_kind.data(), J * 4);
    // the joint rows' kernels come in a ball-and-revolute instantiation
    w.j_all = 0;
    for (uint32_t k : j_kind) w.j_all |= (k != AVBD_JOINT_BALL && k != AVBD_JOINT_REVOLUTE) ? 1 : 0;
    {
        std::vector<uint2> gb(J, make_uint2(0u, 0u));
        std::vector<float4> gmem(J, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        std::vector<uint32_t> gset(J, 0u);
        w.n_gear = 0;
        for (uint32_t i = 0; i < J; i++) {
            const JointRec& j = W->joints[i];
            if (j.kind != AVBD_JOINT_GEAR) continue;
            w.n_gear++;
            gb[i] = make_uint2(j.gb[0], j.gb[1]);
            gmem[i] = make_float4(j.st.gear_raw[0], j.st.gear_raw[1], j.st.gear_cont[0], j.st.gear_cont[1]);
            gset[i] = j.st.gear_mem_set;
        }
        up(w.j_gb, gb.data(), J * 8);
        up(w.j_gmem, gmem.data(), J * 16);
        up(w.j_gset, gset.data(), J * 4);
    }
    up(w.j_ab, j_ab.data(), J * 8);
    up(w.j_la, j_la.data(), J * 16); up(w.j_lb, j_lb.data(), J * 16);
    up(w.j_axa, j_axa.data(), J * 16); up(w.j_axb, j_axb.data(), J * 16);
    up(w.j_lim, j_lim.data(), J * 16);
    up(w.j_ref, j_ref.data(), J * 16); up(w.j_dref, j_dref.data(), J * 16); up(w.j_qref, j_qref.data(), J * 16);
    up(w.j_cfg, j_cfg.data(), J * 4); up(w.j_six, j_six.data(), 3 * (size_t)J * 16);
    up(w.j_sacc, j_sacc.data(), 2 * (size_t)J * 16);
    up((void*)w.jimp_off, jimp_off.data(), (S + 1) * 4);
    up((void*)w.jimp_list, jimp_list.data(), jimp_list.size() * 4);
    up(w.j_lam_l, jll.data(), J * 16); up(w.j_lam_a, jla.data(), J * 16);
    up(w.j_pen_l, jpl.data(), J * 16); up(w.j_pen_a, jpa.data(), J * 16);
    up(w.p_ab, pab.data(), P * 8); up(w.p_n, pn.data(), P * 16); up(w.p_mu, pmu.data(), P * 8);
    up(w.p_np, pnp.data(), P * 4);
    up(w.q_ra, qra.data(), qra.size() * 16); up(w.q_rb, qrb.data(), qrb.size() * 16);
    up(w.q_lam, qlam.data(), qlam.size() * 16); up(w.q_pen, qpen.data(), qpen.size() * 16);
    up(w.q_roll, qroll.data(), qroll.size() * 16); up(w.q_matched, qm.data(), qm.size() * 4);
    up(w.offA, offA.data(), (N + 1) * 4);
    up(w.offB, offB.data(), (N + 1) * 4);
    up(w.listB, listB.data(), P * 4);
    up(W->d_stage, W->bodies.data(), N * sizeof(AvbdBody));
    k_bodies_in<<<(N + 255) / 256, 256, 0, st>>>(w, W->d_stage, 0, N);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    W->dev_valid = true;
    return AVBD_OK;
}

// Refresh the host model from the device.
static int download_all(AvbdWorld* W) {
    if (!W->dev_valid || W->host_valid) return AVBD_OK;
    DW& w = W->w;
    cudaStream_t st = W->st;
    uint32_t N = (uint32_t)w.N, J = (uint32_t)w.J;
    k_bodies_out<<<(N + 255) / 256, 256, 0, st>>>(w, W->d_stage, 0, N);
    W->bodies.resize(N);
    CK(cudaMemcpyAsync(W->bodies.data(), W->d_stage, N * sizeof(AvbdBody), cudaMemcpyDeviceToHost, st));
    std::vector<float4> pp(N), pr(N);
    std::vector<float> timer(N);
    std::vector<uint32_t> asleep(N);
    CK(cudaMemcpyAsync(pp.data(), w.prev_pos, N * 16, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(pr.data(), w.prev_rot, N * 16, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(timer.data(), w.sleep_timer, N * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(asleep.data(), w.asleep, N * 4, cudaMemcpyDeviceToHost, st));
    uint32_t P = 0;
    CK(cudaMemcpyAsync(&P, w.offA + N, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    W->aux.resize(N);
    for (uint32_t h = 0; h < N; h++) {
        AvbdBodyAux& a = W->aux[h];
        a.prev_position[0] = pp[h].x; a.prev_position[1] = pp[h].y; a.prev_position[2] = pp[h].z;
        a.prev_orientation[0] = pr[h].x; a.prev_orientation[1] = pr[h].y;
        a.prev_orientation[2] = pr[h].z; a.prev_orientation[3] = pr[h].w;
        a.sleep_timer = timer[h];
        a.asleep = asleep[h];
    }
    std::vector<uint2> pab(P);
    std::vector<float4> pn(P);
    std::vector<float2> pmu(P);
    std::vector<uint32_t> pnp(P);
    size_t Q = (size_t)P * MAX_PTS;
    std::vector<float4> qra(Q), qrb(Q), qlam(Q), qpen(Q), qroll(Q);
    std::vector<int32_t> qm(Q);
    if (P) {
        CK(cudaMemcpyAsync(pab.data(), w.p_ab, P * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(pn.data(), w.p_n, P * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(pmu.data(), w.p_mu, P * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(pnp.data(), w.p_np, P * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(qra.data(), w.q_ra, Q * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(qrb.data(), w.q_rb, Q * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(qlam.data(), w.q_lam, Q * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(qpen.data(), w.q_pen, Q * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(qroll.data(), w.q_roll, Q * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(qm.data(), w.q_matched, Q * 4, cudaMemcpyDeviceToHost, st));
    }
    std::vector<float4> jll(J), jla(J), jpl(J), jpa(J), jlim(J), jref(J), jsacc(2 * (size_t)J), jgmem(J);
    std::vector<uint32_t> jgset(J);
    if (J) {
        CK(cudaMemcpyAsync(jgmem.data(), w.j_gmem, J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jgset.data(), w.j_gset, J * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jref.data(), w.j_ref, J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jsacc.data(), w.j_sacc, 2 * (size_t)J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jll.data(), w.j_lam_l, J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jla.data(), w.j_lam_a, J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jpl.data(), w.j_pen_l, J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jpa.data(), w.j_pen_a, J * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(jlim.data(), w.j_lim, J * 16, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    W->pairs.resize(P);
    W->points.assign(Q, AvbdPointState{});
    for (uint32_t i = 0; i < P; i++) {
        AvbdPairState& s = W->pairs[i];
        s.a = pab[i].x; s.b = pab[i].y;
        s.normal[0] = pn[i].x; s.normal[1] = pn[i].y; s.normal[2] = pn[i].z;
        s.gap = pn[i].w;
        s.mu[0] = pmu[i].x; s.mu[1] = pmu[i].y;
        s.npoints = pnp[i];
        for (int k = 0; k < MAX_PTS; k++) {
            size_t d = (size_t)i * MAX_PTS + k;
            AvbdPointState& q = W->points[d];
            q.matched = -1;
            if ((uint32_t)k >= pnp[i]) continue;
            q.ra[0] = qra[d].x; q.ra[1] = qra[d].y; q.ra[2] = qra[d].z;
            q.rb[0] = qrb[d].x; q.rb[1] = qrb[d].y; q.rb[2] = qrb[d].z;
            q.stuck = qrb[d].w != 0.0f;
            q.lam[0] = qlam[d].x; q.lam[1] = qlam[d].y; q.lam[2] = qlam[d].z;
            q.pen[0] = qpen[d].x; q.pen[1] = qpen[d].y; q.pen[2] = qpen[d].z;
            q.roll_lam[0] = qroll[d].x; q.roll_lam[1] = qroll[d].y; q.roll_lam[2] = qroll[d].z;
            q.matched = qm[d];
        }
    }
    // The device keeps a static body's pairs in discovery order unless the
    // world sorts them (sort_static): the host model lists pairs in
    // ascending (a, b), whatever order the device holds.
    auto ab_less = [&](uint32_t x, uint32_t y) {
        const AvbdPairState &px = W->pairs[x], &py = W->pairs[y];
        return px.a != py.a ? px.a < py.a : px.b < py.b;
    };
    std::vector<uint32_t> perm(P);
    std::iota(perm.begin(), perm.end(), 0u);
    if (!std::is_sorted(perm.begin(), perm.end(), ab_less)) {
        std::sort(perm.begin(), perm.end(), ab_less);
        std::vector<AvbdPairState> sp(P);
        std::vector<AvbdPointState> sq(Q);
        for (uint32_t i = 0; i < P; i++) {
            sp[i] = W->pairs[perm[i]];
            std::memcpy(&sq[(size_t)i * MAX_PTS], &W->points[(size_t)perm[i] * MAX_PTS],
                        MAX_PTS * sizeof(AvbdPointState));
        }
        W->pairs.swap(sp);
        W->points.swap(sq);
    }
    for (uint32_t i = 0; i < J; i++) {
        AvbdJointState& s = W->joints[i].st;
        s.lam_l[0] = jll[i].x; s.lam_l[1] = jll[i].y; s.lam_l[2] = jll[i].z;
        s.lam_a[0] = jla[i].x; s.lam_a[1] = jla[i].y; s.lam_a[2] = jla[i].z;
        s.pen_l[0] = jpl[i].x; s.pen_l[1] = jpl[i].y; s.pen_l[2] = jpl[i].z;
        s.pen_a[0] = jpa[i].x; s.pen_a[1] = jpa[i].y; s.pen_a[2] = jpa[i].z;
        s.acc_lim = jlim[i].w;
        s.lim_dual = jref[i].y;
        const float4 s0 = jsacc[2 * (size_t)i], s1 = jsacc[2 * (size_t)i + 1];
        s.sacc[0] = s0.x; s.sacc[1] = s0.y; s.sacc[2] = s0.z; s.sacc[3] = s0.w; s.sacc[4] = s1.x; s.sacc[5] = s1.y;
        if (W->joints[i].kind == AVBD_JOINT_GEAR) {
            s.gear_raw[0] = jgmem[i].x; s.gear_raw[1] = jgmem[i].y;
            s.gear_cont[0] = jgmem[i].z; s.gear_cont[1] = jgmem[i].w;
            s.gear_mem_set = jgset[i];
        }
    }
    W->host_valid = true;
    return AVBD_OK;
}

static int ensure_device(AvbdWorld* W) {
    if (W->dev_valid && !W->host_valid) return AVBD_OK;
    if (W->dev_valid && W->host_valid) return AVBD_OK;
    return upload_all(W);
}
// The host model is about to change: make it current and mark the device stale.
static int host_edit(AvbdWorld* W) {
    int rc = download_all(W);
    W->dev_valid = false;
    W->host_valid = true;
    return rc;
}

// ---- substep driver ---------------------------------------------------------------
// Enqueue one substep up to and including the colouring (emit: the
// substep reports events, so discovery also collects trigger overlaps).
static void enqueue_front(AvbdWorld* W, bool emit) {
    cudaStream_t st = W->st;
    W->cur = 1 - W->cur;  // the previous generation becomes `old`
    set_pair_ptrs(W);
    const DW& w = W->w;
    launch_begin_substep(w, st);
    launch_wake_joint_motion(w, st);
    launch_gear_mem(w, st);
    launch_torque(w, st);
    launch_broadphase(w, W->plan, st);
    launch_ccd(w, st);
    launch_discovery(w, W->scan_tmp, st, emit && W->has_trig);
    launch_post_discovery(w, W->scan_tmp, st);
    launch_colouring(w, W->tune, W->scan_tmp, st);
}
static void enqueue_back(AvbdWorld* W, int ncol, bool emit) {
    const DW& w = W->w;
    if (use_scene_solve(w, W->tune)) {
        launch_scene_solve(w, W->tune, W->st);
    } else {
        launch_solve_prep(w, W->tune, W->st);
        for (int it = 0; it < w.iterations; it++) launch_iteration(w, W->tune, ncol, W->st);
    }
    launch_finish_substep(w, W->tune, W->st);
    if (W->ev_period >= 0) launch_events(w, emit, emit && W->has_trig, W->scan_tmp, W->st);
}

static int read_ctr(AvbdWorld* W) {
    CK(cudaMemcpyAsync(W->h_ctr, W->w.ctr, C_NUM * 4, cudaMemcpyDeviceToHost, W->st));
    CK(cudaStreamSynchronize(W->st));
    return AVBD_OK;
}

static int grow_candidates(AvbdWorld* W) {
    // keep the (valid) previous generation: round-trip through the host model
    W->host_valid = false;
    int rc = download_all(W);
    if (rc) return rc;
    uint32_t cap = W->cand_cap * 2u;
    rc = alloc_device(W, (uint32_t)W->bodies.size(), (uint32_t)W->joints.size(), cap);
    if (rc) return rc;
    W->dev_valid = false;
    return upload_all(W);
}

static void accumulate(AvbdWorld* W) {
    const uint32_t* c = W->h_ctr;
    W->cum.steps += 1;
    W->cum.pairs = c[C_PAIRS];
    W->cum.points = c[C_POINTS];
    W->cum.candidates = c[C_CAND];
    W->cum.colours = c[C_NCOL];
    W->cum.breakdowns = c[C_BREAKDOWN];
    W->cum.ccd_hits = c[C_CCD];
    W->cum.sleeping = c[C_SLEEP];
    W->cum.timeouts = c[C_TIMEOUT] + c[C_CCD_LEFT];
}

// One substep through plain launches (the host reads the colour count).
static int substep_plain(AvbdWorld* W, bool emit) {
    for (int attempt = 0; attempt < 8; attempt++) {
        enqueue_front(W, emit);
        CK(cudaGetLastError());
        int rc = read_ctr(W);
        if (rc) return rc;
        if (W->h_ctr[C_ERR] & E_CAND_OVERFLOW) {
            // nothing after the broadphase ran: undo the buffer flip, grow, replay
            W->cur = 1 - W->cur;
            set_pair_ptrs(W);
            CK(cudaMemsetAsync(W->w.ctr + C_ERR, 0, 4, W->st));
            rc = grow_candidates(W);
            if (rc) return rc;
            continue;
        }
        int ncol = (int)W->h_ctr[C_NCOL];
        W->last_ncol = ncol;
        enqueue_back(W, ncol, emit);
        CK(cudaGetLastError());
        rc = read_ctr(W);
        if (rc) return rc;
        accumulate(W);
        if (W->h_ctr[C_ERR] & E_COLOUR_OVERFLOW) return AVBD_ERR_CAPACITY;
        return AVBD_OK;
    }
    return AVBD_ERR_CAPACITY;
}

// ---- differentiable rollouts ----------------------------------------------------
// The forward records a device checkpoint of the whole step state every
// `every` steps.  The backward walks the segments last to first: it restores
// a segment's checkpoint, recomputes the segment with plain launches while
// copying each substep's frozen contact set, colouring and iterates into a
// frame, then runs the adjoint kernels over the frames in reverse.
namespace {

struct Snap {
    Alloc mem;
    int cur = 0;
    uint32_t P = 0;
    float4 *pos, *rot, *vel, *angvel, *torque, *prev_pos, *prev_rot, *inertia;
    float *inv_mass, *sleep_timer;
    uint32_t *asleep, *info;
    PairBuf pb{};
    uint32_t *offB, *listB, *posB;  // B-side incidence: the next discovery finds old pairs through it
    float4 *jll, *jla, *jpl, *jpa, *jlim;
};

struct AdjTape {
    int steps = 0, substeps = 0, every = 0;
    uint32_t N = 0, J = 0, S = 0, max_pairs = 0;
    std::vector<Snap*> ckpt;  // segment starts
    Snap* fin = nullptr;      // the state after the rollout
    Alloc fmem, smem;         // frames; adjoint state
    uint32_t pcap = 0;        // pairs a frame holds
    int nframes = 0;
    std::vector<AdjFrame> frames;
    std::vector<std::array<cudaGraphExec_t, 2>> rg;  // recording graphs per frame and parity
    int rg_cols = 0;
    uint64_t rg_key = 0;  // the world allocation (mem_gen) the graphs were captured against
    AdjState A{};
    float ms_recompute = 0.0f, ms_reverse = 0.0f;  // device time of the last backward
    std::vector<float> gk_scene;  // joint stiffness adjoint per scene, last backward
    uint2* d_trace = nullptr;     // per substep of the rollout: (max |body adjoint| bits, body)
    int trace_cap = 0;
    std::vector<uint2> trace;
};

void snap_free(Snap* s) {
    if (!s) return;
    s->mem.release();
    delete s;
}
void adj_free_graphs(AdjTape* t);
void adj_free(AdjTape* t) {
    if (!t) return;
    adj_free_graphs(t);
    for (Snap* s : t->ckpt) snap_free(s);
    snap_free(t->fin);
    t->fmem.release();
    t->smem.release();
    if (t->d_trace) cudaFree(t->d_trace);
    delete t;
}

#define D2D(dst, src, bytes) CK(cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyDeviceToDevice, st))

int snap_take(AvbdWorld* W, Snap** out) {
    DW& w = W->w;
    cudaStream_t st = W->st;
    const size_t N = (size_t)w.N, J = (size_t)w.J;
    uint32_t P = 0;
    CK(cudaMemcpyAsync(&P, w.offA + N, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    Snap* s = new Snap();
    Alloc& m = s->mem;
    s->cur = W->cur;
    s->P = P;
    const size_t Q = (size_t)P * MAX_PTS;
    s->pos = m.get<float4>(N); s->rot = m.get<float4>(N); s->vel = m.get<float4>(N); s->angvel = m.get<float4>(N);
    s->torque = m.get<float4>(N); s->prev_pos = m.get<float4>(N); s->prev_rot = m.get<float4>(N);
    s->inertia = m.get<float4>(N);
    s->inv_mass = m.get<float>(N); s->sleep_timer = m.get<float>(N);
    s->asleep = m.get<uint32_t>(N); s->info = m.get<uint32_t>(N);
    PairBuf& b = s->pb;
    b.ab = m.get<uint2>(P); b.n = m.get<float4>(P); b.mu = m.get<float2>(P); b.np = m.get<uint32_t>(P);
    b.old = m.get<int32_t>(P);
    b.ra = m.get<float4>(Q); b.rb = m.get<float4>(Q); b.lam = m.get<float4>(Q); b.pen = m.get<float4>(Q);
    b.roll = m.get<float4>(Q); b.matched = m.get<int32_t>(Q);
    b.offA = m.get<uint32_t>(N + 1);
    s->offB = m.get<uint32_t>(N + 1); s->listB = m.get<uint32_t>(P); s->posB = m.get<uint32_t>(P);
    s->jll = m.get<float4>(J); s->jla = m.get<float4>(J); s->jpl = m.get<float4>(J); s->jpa = m.get<float4>(J);
    s->jlim = m.get<float4>(J);
    if (!s->jlim || !b.offA) {
        snap_free(s);
        return AVBD_ERR_DEVICE;
    }
    D2D(s->pos, w.pos, N * 16); D2D(s->rot, w.rot, N * 16); D2D(s->vel, w.vel, N * 16);
    D2D(s->angvel, w.angvel, N * 16); D2D(s->torque, w.torque, N * 16); D2D(s->prev_pos, w.prev_pos, N * 16);
    D2D(s->prev_rot, w.prev_rot, N * 16); D2D(s->inertia, w.inertia, N * 16);
    D2D(s->inv_mass, w.inv_mass, N * 4); D2D(s->sleep_timer, w.sleep_timer, N * 4);
    D2D(s->asleep, w.asleep, N * 4); D2D(s->info, w.info, N * 4);
    if (P) {
        D2D(b.ab, w.p_ab, P * 8); D2D(b.n, w.p_n, P * 16); D2D(b.mu, w.p_mu, P * 8); D2D(b.np, w.p_np, P * 4);
        D2D(b.old, w.p_old, P * 4);
        D2D(b.ra, w.q_ra, Q * 16); D2D(b.rb, w.q_rb, Q * 16); D2D(b.lam, w.q_lam, Q * 16);
        D2D(b.pen, w.q_pen, Q * 16); D2D(b.roll, w.q_roll, Q * 16); D2D(b.matched, w.q_matched, Q * 4);
    }
    D2D(b.offA, w.offA, (N + 1) * 4);
    D2D(s->offB, w.offB, (N + 1) * 4);
    if (P) {
        D2D(s->listB, w.listB, P * 4);
        D2D(s->posB, w.posB, P * 4);
    }
    if (J) {
        D2D(s->jll, w.j_lam_l, J * 16); D2D(s->jla, w.j_lam_a, J * 16); D2D(s->jpl, w.j_pen_l, J * 16);
        D2D(s->jpa, w.j_pen_a, J * 16); D2D(s->jlim, w.j_lim, J * 16);
    }
    *out = s;
    return AVBD_OK;
}

int snap_restore(AvbdWorld* W, const Snap* s) {
    W->cur = s->cur;
    set_pair_ptrs(W);
    DW& w = W->w;
    cudaStream_t st = W->st;
    const size_t N = (size_t)w.N, J = (size_t)w.J, P = s->P, Q = P * MAX_PTS;
    const PairBuf& b = s->pb;
    D2D(w.pos, s->pos, N * 16); D2D(w.rot, s->rot, N * 16); D2D(w.vel, s->vel, N * 16);
    D2D(w.angvel, s->angvel, N * 16); D2D(w.torque, s->torque, N * 16); D2D(w.prev_pos, s->prev_pos, N * 16);
    D2D(w.prev_rot, s->prev_rot, N * 16); D2D(w.inertia, s->inertia, N * 16);
    D2D(w.inv_mass, s->inv_mass, N * 4); D2D(w.sleep_timer, s->sleep_timer, N * 4);
    D2D(w.asleep, s->asleep, N * 4); D2D(w.info, s->info, N * 4);
    if (P) {
        D2D(w.p_ab, b.ab, P * 8); D2D(w.p_n, b.n, P * 16); D2D(w.p_mu, b.mu, P * 8); D2D(w.p_np, b.np, P * 4);
        D2D(w.p_old, b.old, P * 4);
        D2D(w.q_ra, b.ra, Q * 16); D2D(w.q_rb, b.rb, Q * 16); D2D(w.q_lam, b.lam, Q * 16);
        D2D(w.q_pen, b.pen, Q * 16); D2D(w.q_roll, b.roll, Q * 16); D2D(w.q_matched, b.matched, Q * 4);
    }
    D2D(w.offA, b.offA, (N + 1) * 4);
    D2D(w.offB, s->offB, (N + 1) * 4);
    if (P) {
        D2D(w.listB, s->listB, P * 4);
        D2D(w.posB, s->posB, P * 4);
    }
    if (J) {
        D2D(w.j_lam_l, s->jll, J * 16); D2D(w.j_lam_a, s->jla, J * 16); D2D(w.j_pen_l, s->jpl, J * 16);
        D2D(w.j_pen_a, s->jpa, J * 16); D2D(w.j_lim, s->jlim, J * 16);
    }
    W->host_valid = false;
    W->dev_valid = true;
    return AVBD_OK;
}

// Frames for `n` substeps of up to `pcap` pairs, and the adjoint state.
int adj_storage(AvbdWorld* W, AdjTape* t, int n, uint32_t pcap) {
    if (t->nframes >= n && t->pcap >= pcap) return AVBD_OK;
    adj_free_graphs(t);  // they copy into the frames
    t->fmem.release();
    t->smem.release();
    t->frames.assign(n, AdjFrame{});
    t->nframes = n;
    t->pcap = pcap;
    const size_t N = (size_t)W->w.N, Pc = pcap, Qc = Pc * MAX_PTS;
    const int K = W->w.iterations;
    Alloc& m = t->fmem;
    for (AdjFrame& f : t->frames) {
        f.qstride = Qc;
        f.pos0 = m.get<float4>(N); f.rot0 = m.get<float4>(N); f.inertial = m.get<float4>(N);
        f.inertial_rot = m.get<float4>(N); f.vel = m.get<float4>(N); f.angvel = m.get<float4>(N);
        f.inertia = m.get<float4>(N); f.inv_mass = m.get<float>(N); f.asleep_end = m.get<uint32_t>(N);
        f.it_pos = m.get<float4>(N * (K + 1)); f.it_rot = m.get<float4>(N * (K + 1));
        f.colour = m.get<int32_t>(N); f.col_cnt = m.get<uint32_t>(MAX_COLOURS + 1); f.col_list = m.get<uint32_t>(N);
        f.offA = m.get<uint32_t>(N + 1); f.offB = m.get<uint32_t>(N + 1);
        f.listB = m.get<uint32_t>(Pc); f.posB = m.get<uint32_t>(Pc);
        f.p_ab = m.get<uint2>(Pc); f.p_n = m.get<float4>(Pc); f.p_mu = m.get<float2>(Pc);
        f.p_np = m.get<uint32_t>(Pc); f.p_old = m.get<int32_t>(Pc);
        f.q_ra = m.get<float4>(Qc); f.q_rb = m.get<float4>(Qc); f.q_matched = m.get<int32_t>(Qc);
        f.it_lam = m.get<float4>(Qc * (K + 1)); f.it_pen = m.get<float4>(Qc * (K + 1));
        f.side_list = m.get<uint32_t>(Pc * 2); f.side_cnt = m.get<uint32_t>(2 * MAX_COLOURS + 2);
        f.cstride = Pc * 2 * 7;
        f.it_contrib = m.get<float4>(f.cstride * K);
        f.it_joint = m.get<float4>((size_t)(K + 1) * 5 * W->w.J);
        f.ccd = W->w.ccd_rec ? m.get<float4>(N * 2) : nullptr;
        if (!f.it_contrib || !f.it_joint || (W->w.ccd_rec && !f.ccd)) return AVBD_ERR_DEVICE;
    }
    Alloc& a = t->smem;
    AdjState& A = t->A;
    A.ax = a.get<float4>(N); A.aq = a.get<float4>(N); A.av = a.get<float4>(N); A.aw = a.get<float4>(N);
    A.ax0 = a.get<float4>(N); A.aq0 = a.get<float4>(N); A.ay = a.get<float4>(N); A.aqt = a.get<float4>(N);
    A.slot = a.get<float4>(Pc * 2 * 4);
    A.alam = a.get<float4>(Qc); A.apen = a.get<float4>(Qc);
    A.alam_old = a.get<float4>(Qc); A.apen_old = a.get<float4>(Qc);
    A.amu = a.get<float2>(Pc);
    A.ascene_mu = a.get<float>(W->w.S);
    A.wd = a.get<float4>(N * 3);
    const size_t J = (size_t)W->w.J;
    A.jslot = a.get<float4>(J * 2 * 4);
    A.ajs = a.get<float4>(J * 5);
    A.ajk = a.get<float>(J);
    A.nlong = a.get<uint32_t>(1);
    A.long_list = a.get<uint32_t>(N);
    return (A.wd && A.ajk && A.long_list) ? AVBD_OK : AVBD_ERR_DEVICE;
}

// One substep with plain launches, its frame filled on the way.
// The joints' warm state into pose slice s of a frame.
int adj_copy_joints(AvbdWorld* W, AdjFrame& f, int slice) {
    cudaStream_t st = W->st;
    const DW& w = W->w;
    const size_t J = (size_t)w.J;
    if (!J) return AVBD_OK;
    float4* b = f.it_joint + (size_t)slice * 5 * J;
    D2D(b, w.j_lam_l, J * 16); D2D(b + J, w.j_pen_l, J * 16); D2D(b + 2 * J, w.j_lam_a, J * 16);
    D2D(b + 3 * J, w.j_pen_a, J * 16); D2D(b + 4 * J, w.j_lim, J * 16);
    return AVBD_OK;
}
// What the reverse reads of a substep, copied right after its front (the
// copies cover the frame's capacity, so that a captured graph replays them).
int adj_copy_front(AvbdWorld* W, AdjTape* t, AdjFrame& f) {
    cudaStream_t st = W->st;
    const DW& w = W->w;
    const size_t N = (size_t)w.N, P = std::min<size_t>(t->pcap, W->cand_cap), Q = P * MAX_PTS;
    D2D(f.pos0, w.pos0, N * 16); D2D(f.rot0, w.rot0, N * 16); D2D(f.inertial, w.inertial, N * 16);
    D2D(f.inertial_rot, w.inertial_rot, N * 16); D2D(f.vel, w.vel, N * 16); D2D(f.angvel, w.angvel, N * 16);
    D2D(f.inertia, w.inertia, N * 16); D2D(f.inv_mass, w.inv_mass, N * 4);
    D2D(f.colour, w.colour, N * 4); D2D(f.col_cnt, w.col_cnt, (MAX_COLOURS + 1) * 4); D2D(f.col_list, w.col_list, N * 4);
    D2D(f.offA, w.offA, (N + 1) * 4); D2D(f.offB, w.offB, (N + 1) * 4);
    D2D(f.it_pos, w.pos, N * 16); D2D(f.it_rot, w.rot, N * 16);
    D2D(f.listB, w.listB, P * 4); D2D(f.posB, w.posB, P * 4);
    D2D(f.p_ab, w.p_ab, P * 8); D2D(f.p_n, w.p_n, P * 16); D2D(f.p_mu, w.p_mu, P * 8);
    D2D(f.p_np, w.p_np, P * 4); D2D(f.p_old, w.p_old, P * 4);
    D2D(f.q_ra, w.q_ra, Q * 16); D2D(f.q_rb, w.q_rb, Q * 16); D2D(f.q_matched, w.q_matched, Q * 4);
    D2D(f.it_lam, w.q_lam, Q * 16); D2D(f.it_pen, w.q_pen, Q * 16);
    if (f.ccd) D2D(f.ccd, w.ccd_rec, N * 32);
    adj_copy_joints(W, f, 0);
    return AVBD_OK;
}
// The iterations and the finish of a substep for `cover` colours, with the
// split primal's row sums and every iterate copied into the frame.
int adj_back(AvbdWorld* W, AdjTape* t, AdjFrame& f, int cover) {
    cudaStream_t st = W->st;
    const DW& w = W->w;
    const size_t N = (size_t)w.N, P = std::min<size_t>(t->pcap, W->cand_cap), Q = P * MAX_PTS;
    launch_solve_prep(w, W->tune, st);
    D2D(f.side_cnt, w.side_cnt, (2 * MAX_COLOURS + 2) * 4);
    D2D(f.side_list, w.side_list, P * 2 * 4);
    for (int it = 0; it < w.iterations; it++) {
        // the split primal writes this iteration's row sums straight into the frame
        DW wi = w;
        wi.contrib = f.it_contrib + it * f.cstride;
        wi.contrib_slots = (uint32_t)(2 * P);
        for (int c = 0; c < cover; c++) launch_primal_colour(wi, W->tune, c, (uint32_t)w.N, st);
        D2D(f.it_pos + (it + 1) * N, w.pos, N * 16);
        D2D(f.it_rot + (it + 1) * N, w.rot, N * 16);
        launch_dual(w, W->tune, st);
        D2D(f.it_lam + (it + 1) * f.qstride, w.q_lam, Q * 16);
        D2D(f.it_pen + (it + 1) * f.qstride, w.q_pen, Q * 16);
        adj_copy_joints(W, f, it + 1);
    }
    launch_finish_substep(w, W->tune, st);
    D2D(f.asleep_end, w.asleep, N * 4);
    return AVBD_OK;
}

uint64_t adj_graph_key(const AvbdWorld* W) { return W->mem_gen; }

void adj_free_graphs(AdjTape* t) {
    for (auto& g : t->rg)
        for (auto& e : g)
            if (e) {
                cudaGraphExecDestroy(e);
                e = nullptr;
            }
    t->rg.clear();
}

// One captured recording substep per frame and pair-buffer parity.  The
// primal is captured for rg_cols colours; a substep that needs more is
// finished with plain launches.
int adj_capture(AvbdWorld* W, AdjTape* t) {
    adj_free_graphs(t);
    const int base = W->cur;
    t->rg_cols = std::max(W->graph_cols, std::max(W->last_ncol + 2, 4));
    t->rg.assign(t->frames.size(), {nullptr, nullptr});
    for (size_t k = 0; k < t->frames.size(); k++)
        for (int par = 0; par < 2; par++) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(W->st, cudaStreamCaptureModeThreadLocal));
            W->w.max_cols = t->rg_cols;
            enqueue_front(W, false);
            adj_copy_front(W, t, t->frames[k]);
            adj_back(W, t, t->frames[k], t->rg_cols);
            W->w.max_cols = MAX_COLOURS;
            CK(cudaStreamEndCapture(W->st, &g));
            cudaError_t e = cudaGraphInstantiate(&t->rg[k][W->cur], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                adj_free_graphs(t);
                W->cur = base;
                set_pair_ptrs(W);
                return AVBD_ERR_DEVICE;
            }
        }
    W->cur = base;  // each capture flipped the parity twice per frame
    set_pair_ptrs(W);
    t->rg_key = adj_graph_key(W);
    return AVBD_OK;
}

// Substep k of the segment being recomputed, its frame filled on the way:
// by graph replay when the recording graphs match the world, else plainly.
int adj_substep(AvbdWorld* W, AdjTape* t, int k) {
    cudaStream_t st = W->st;
    AdjFrame& f = t->frames[k];
    if (!t->rg.empty() && t->rg_key == adj_graph_key(W)) {
        const int next = 1 - W->cur;
        CK(cudaGraphLaunch(t->rg[k][next], st));
        W->cur = next;
        set_pair_ptrs(W);
        int rc = read_ctr(W);
        if (rc) return rc;
        if (!(W->h_ctr[C_ERR] & E_CAND_OVERFLOW)) {
            const uint32_t P = W->h_ctr[C_PAIRS], ncol = W->h_ctr[C_NCOL];
            if (P > t->pcap) return AVBD_ERR_CAPACITY;
            if (W->h_ctr[C_ERR] & E_COLOUR_RANGE) {
                // the graph's iterations were skipped: finish this substep plainly
                CK(cudaMemsetAsync(W->w.ctr + C_ERR, 0, 4, st));
                adj_back(W, t, f, (int)ncol);
                rc = read_ctr(W);
                if (rc) return rc;
            }
            W->last_ncol = (int)ncol;
            f.npairs = P;
            f.ncol = ncol;
            accumulate(W);
            if (W->h_ctr[C_ERR] & E_COLOUR_OVERFLOW) return AVBD_ERR_CAPACITY;
            return AVBD_OK;
        }
        // candidate overflow: nothing after the broadphase ran; undo the flip
        // and record this substep plainly after growing
        W->cur = 1 - W->cur;
        set_pair_ptrs(W);
        CK(cudaMemsetAsync(W->w.ctr + C_ERR, 0, 4, st));
        rc = grow_candidates(W);
        if (rc) return rc;
    }
    for (int attempt = 0;; attempt++) {
        if (attempt == 8) return AVBD_ERR_CAPACITY;
        enqueue_front(W, false);
        CK(cudaGetLastError());
        int rc = read_ctr(W);
        if (rc) return rc;
        if (!(W->h_ctr[C_ERR] & E_CAND_OVERFLOW)) break;
        W->cur = 1 - W->cur;
        set_pair_ptrs(W);
        CK(cudaMemsetAsync(W->w.ctr + C_ERR, 0, 4, st));
        rc = grow_candidates(W);
        if (rc) return rc;
    }
    const uint32_t P = W->h_ctr[C_PAIRS], ncol = W->h_ctr[C_NCOL];
    if (P > t->pcap) return AVBD_ERR_CAPACITY;
    W->last_ncol = (int)ncol;
    f.npairs = P;
    f.ncol = ncol;
    adj_copy_front(W, t, f);
    adj_back(W, t, f, (int)ncol);
    CK(cudaGetLastError());
    int rc = read_ctr(W);
    if (rc) return rc;
    accumulate(W);
    if (W->h_ctr[C_ERR] & E_COLOUR_OVERFLOW) return AVBD_ERR_CAPACITY;
    return AVBD_OK;
}

int adj_reverse(AvbdWorld* W, AdjTape* t, const AdjFrame& f) {
    cudaStream_t st = W->st;
    AdjState& A = t->A;
    const size_t Qc = (size_t)t->pcap * MAX_PTS;
    if (f.npairs) {
        CK(cudaMemsetAsync(A.slot, 0, (size_t)f.npairs * 2 * 4 * 16, st));
        CK(cudaMemsetAsync(A.amu, 0, (size_t)f.npairs * 8, st));
    }
    CK(cudaMemsetAsync(A.alam_old, 0, Qc * 16, st));
    CK(cudaMemsetAsync(A.apen_old, 0, Qc * 16, st));
    if (W->w.J) CK(cudaMemsetAsync(A.jslot, 0, (size_t)W->w.J * 2 * 4 * 16, st));
    launch_adjoint_substep(W->w, f, A, W->w.iterations, st);
    CK(cudaGetLastError());
    std::swap(A.alam, A.alam_old);
    std::swap(A.apen, A.apen_old);
    return AVBD_OK;
}

#undef D2D

}  // namespace

template <class T>
static int drain(AvbdWorld* W, int which, T* out, uint32_t cap, uint32_t* n) {
    if (!W || !n || (cap && !out)) return AVBD_ERR_INVALID_ARG;
    *n = 0;
    if (!W->w.evs) return AVBD_OK;
    cudaSetDevice(W->device);
    const int idx = which == 0 ? EV_N : EV_TN;
    uint32_t q = 0;
    CK(cudaStreamSynchronize(W->st));
    CK(cudaMemcpy(&q, W->w.evs + idx, 4, cudaMemcpyDeviceToHost));
    *n = q;
    if (q > cap) return AVBD_ERR_CAPACITY;  // nothing moved: call again with room for *n
    if (q) {
        const void* src = which == 0 ? (const void*)W->w.ev : (const void*)W->w.tev;
        CK(cudaMemcpy(out, src, (size_t)q * sizeof(T), cudaMemcpyDeviceToHost));
        CK(cudaMemset(W->w.evs + idx, 0, 4));
    }
    return AVBD_OK;
}

// The world's stream and pinned counters on `device`; the world is deleted
// when that fails.
static int open_device(AvbdWorld* W, int device) {
    W->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&W->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&W->h_ctr, C_NUM * 4) != cudaSuccess) {
        if (W->st) cudaStreamDestroy(W->st);
        delete W;
        return AVBD_ERR_DEVICE;
    }
    return AVBD_OK;
}

extern "C" {

int avbd_default_params(AvbdParams* p) {
    if (!p) return AVBD_ERR_INVALID_ARG;
    p->gravity[0] = 0.0f;
    p->gravity[1] = -9.81f;
    p->gravity[2] = 0.0f;
    p->step_dt = 1.0f / 60.0f;
    p->iterations = 10;
    p->max_substeps = 4;
    p->enable_sleep = 1;
    p->enable_ccd = 1;
    return AVBD_OK;
}

int avbd_world_create(const AvbdParams* params, int device, AvbdWorld** out) {
    if (!params || !out) return AVBD_ERR_INVALID_ARG;
    if (!(params->step_dt > 0.0f) || !std::isfinite(params->step_dt) || params->iterations < 0 ||
        params->max_substeps < 1)
        return AVBD_ERR_INVALID_ARG;
    AvbdWorld* W = new AvbdWorld();
    W->prm = *params;
    int rc = open_device(W, device);
    if (rc) return rc;
    W->scene_off = {0, 0};
    *out = W;
    return AVBD_OK;
}

int avbd_world_create_batch(const AvbdParams* params, int device, const AvbdBody* bodies, uint32_t n,
                            const uint32_t* scene_offsets, uint32_t nscenes, AvbdWorld** out) {
    if (!bodies || !scene_offsets || nscenes == 0 || scene_offsets[0] != 0 || scene_offsets[nscenes] != n)
        return AVBD_ERR_INVALID_ARG;
    for (uint32_t s = 0; s < nscenes; s++)
        if (scene_offsets[s + 1] < scene_offsets[s]) return AVBD_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; i++)
        if (!body_finite(bodies[i])) return AVBD_ERR_NONFINITE;
    int rc = avbd_world_create(params, device, out);
    if (rc) return rc;
    AvbdWorld* W = *out;
    W->scene_off.assign(scene_offsets, scene_offsets + nscenes + 1);
    W->bodies.assign(bodies, bodies + n);
    W->aux.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        AvbdBodyAux& a = W->aux[i];
        std::memcpy(a.prev_position, bodies[i].position, 12);
        std::memcpy(a.prev_orientation, bodies[i].orientation, 16);
        a.sleep_timer = 0.0f;
        a.asleep = 0;
    }
    return AVBD_OK;
}

int avbd_world_destroy(AvbdWorld* W) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    free_graphs(W);
    adj_free(W->adj);
    W->mem.release();
    W->evmem.release();
    W->hullmem.release();
    if (W->h_ctr) cudaFreeHost(W->h_ctr);
    if (W->flush_buf) cudaFree(W->flush_buf);
    if (W->st) cudaStreamDestroy(W->st);
    delete W;
    return AVBD_OK;
}

int avbd_world_add_bodies(AvbdWorld* W, const AvbdBody* bodies, uint32_t n, uint32_t* first_handle) {
    if (!W || (!bodies && n)) return AVBD_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; i++)
        if (!body_finite(bodies[i])) return AVBD_ERR_NONFINITE;
    cudaSetDevice(W->device);
    int rc = host_edit(W);
    if (rc) return rc;
    uint32_t first = (uint32_t)W->bodies.size();
    for (uint32_t i = 0; i < n; i++) {
        W->bodies.push_back(bodies[i]);
        AvbdBodyAux a{};
        std::memcpy(a.prev_position, bodies[i].position, 12);  // ensure_scratch (mod.rs:1193-1199)
        std::memcpy(a.prev_orientation, bodies[i].orientation, 16);
        W->aux.push_back(a);
    }
    W->scene_off.back() = (uint32_t)W->bodies.size();
    if (first_handle) *first_handle = first;
    return AVBD_OK;
}

// Shape::try_round / try_compound (collision/shape.rs:556-575) over
// primitive parts, with the bound and minimum dimension the engine reads
// (rows.rs:279-290, :393-400).
static int make_ext(const AvbdWorld* W, bool compound, const AvbdShapePart* parts, uint32_t n,
                    const float* unit_inertia, HostExt& e) {
    if (!W || !parts || !unit_inertia || n == 0 || (!compound && n != 1)) return AVBD_ERR_INVALID_ARG;
    e.compound = compound;
    auto len3 = [](const float* v) { return std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]); };
    auto part_bound = [&](const AvbdShapePart& p) {
        float r;
        switch (p.shape) {
            case AVBD_SHAPE_SPHERE: r = p.params[0]; break;
            case AVBD_SHAPE_BOX: r = len3(p.params); break;
            case AVBD_SHAPE_CAPSULE: r = p.params[1] + p.params[0]; break;
            case AVBD_SHAPE_HULL: r = W->hulls[(size_t)p.params[0]].bound; break;
            default: r = std::sqrt(p.params[0] * p.params[0] + p.params[1] * p.params[1]);  // cylinder, cone
        }
        return p.border_radius > 0.0f ? r + std::fmax(p.border_radius, 0.0f) : r;
    };
    auto part_min_dim = [&](const AvbdShapePart& p) {
        float m;
        switch (p.shape) {
            case AVBD_SHAPE_SPHERE: m = p.params[0]; break;
            case AVBD_SHAPE_BOX: m = std::fmin(p.params[0], std::fmin(p.params[1], p.params[2])); break;
            case AVBD_SHAPE_CAPSULE: m = p.params[0]; break;
            case AVBD_SHAPE_CYLINDER: m = std::fmin(p.params[0], p.params[1]); break;
            case AVBD_SHAPE_CONE: m = 0.5f * std::fmin(p.params[0], p.params[1]); break;
            default: m = 0.5f * W->hulls[(size_t)p.params[0]].min_ext;  // hull
        }
        return p.border_radius > 0.0f ? std::fmin(m, std::fmax(p.border_radius, 0.0f) * 2.0f) : m;
    };
    for (uint32_t i = 0; i < n; i++) {
        const AvbdShapePart& q = parts[i];
        if (q.shape > AVBD_SHAPE_HULL || q.shape == AVBD_SHAPE_HALFSPACE) return AVBD_ERR_UNSUPPORTED;
        if (!compound && !(std::isfinite(q.border_radius) && q.border_radius > 0.0f)) return AVBD_ERR_INVALID_ARG;
        if (!std::isfinite(q.border_radius) || q.border_radius < 0.0f) return AVBD_ERR_INVALID_ARG;
        if (q.shape == AVBD_SHAPE_HULL && !(q.params[0] >= 0.0f && (size_t)q.params[0] < W->hulls.size()))
            return AVBD_ERR_INVALID_ARG;
        e.parts.push_back(q);
    }
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(unit_inertia[k])) return AVBD_ERR_NONFINITE;
    std::memcpy(e.unit_inertia, unit_inertia, 12);
    if (compound) {
        e.bound = 0.0f;
        e.min_dim = INFINITY;
        for (const AvbdShapePart& p : e.parts) {
            e.bound = std::fmax(e.bound, part_bound(p) + len3(p.position));
            e.min_dim = std::fmin(e.min_dim, part_min_dim(p));
        }
    } else {
        e.bound = part_bound(e.parts[0]);
        e.min_dim = part_min_dim(e.parts[0]);
    }
    return AVBD_OK;
}
// Heightfield::new (shape.rs:1485-1505, invariants.rs:403-425) with its
// sample range (shape.rs:1571-1583).
static int make_hf(uint32_t rows, uint32_t cols, float cell, const float* heights, HostHf& f) {
    if (rows == 0 || cols == 0 || !heights || !std::isfinite(cell) || !(cell > 0.0f)) return AVBD_ERR_INVALID_ARG;
    if ((uint64_t)rows * cols > (1ull << 28)) return AVBD_ERR_INVALID_ARG;
    f.rows = rows;
    f.cols = cols;
    f.cell = cell;
    f.y_min = INFINITY;
    f.y_max = -INFINITY;
    f.h.assign(heights, heights + (size_t)rows * cols);
    for (float h : f.h) {
        if (!std::isfinite(h)) return AVBD_ERR_NONFINITE;
        f.y_min = std::fmin(f.y_min, h);
        f.y_max = std::fmax(f.y_max, h);
    }
    return AVBD_OK;
}
// TriMesh::build_bvh / split (shape.rs:1793-1890): median splits of the
// longest axis over a stable centroid sort, leaves of up to 4 triangles.
static uint32_t mesh_split(const std::vector<std::array<float, 6>>& bounds, const std::vector<float4>& cent,
                           uint32_t* order, size_t n, uint32_t base, std::vector<MeshNodeD>& nodes) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            lo[k] = std::fmin(lo[k], bounds[order[i]][k]);
            hi[k] = std::fmax(hi[k], bounds[order[i]][3 + k]);
        }
    const uint32_t here = (uint32_t)nodes.size();
    nodes.push_back(MeshNodeD{{lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}, 1u, base, (uint32_t)n});
    if (n <= 4) return here;
    const float e[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    const int axis = (e[0] >= e[1] && e[0] >= e[2]) ? 0 : (e[1] >= e[2] ? 1 : 2);
    auto key = [&](uint32_t t) { return axis == 0 ? cent[t].x : (axis == 1 ? cent[t].y : cent[t].z); };
    std::stable_sort(order, order + n, [&](uint32_t x, uint32_t y) { return key(x) < key(y); });
    if (key(order[0]) == key(order[n - 1])) return here;  // all equal: a leaf
    const size_t mid = n / 2;
    const uint32_t left = mesh_split(bounds, cent, order, mid, base, nodes);
    const uint32_t right = mesh_split(bounds, cent, order + mid, n - mid, base + (uint32_t)mid, nodes);
    nodes[here].leaf = 0u;
    nodes[here].a = left;
    nodes[here].b = right;
    return here;
}
// TriMesh::from_indexed / from_triangles (shape.rs:1646-1772): slivers
// dropped, each triangle a centroid-relative hull with both windings; a
// triangle whose corners weld below three points (ConvexHull::from_vertices
// welds closer than 1e-6, shape.rs:1304-1325) is refused.
static int make_mesh(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, HostMesh& m) {
    if ((nv && !verts) || (nt && !tris)) return AVBD_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < 3 * nv; i++)
        if (!std::isfinite(verts[i])) return AVBD_ERR_NONFINITE;
    m.verts.assign(verts, verts + 3 * (size_t)nv);
    m.tris_in.assign(tris, tris + 3 * (size_t)nt);
    using namespace avbd;
    auto vert = [&](uint32_t i) { return V3{verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]}; };
    m.bound = 0.0f;
    m.min_feature = INFINITY;
    for (uint32_t t = 0; t < nt; t++) {
        for (int k = 0; k < 3; k++)
            if (tris[3 * t + k] >= nv) return AVBD_ERR_INVALID_ARG;
        const V3 v[3] = {vert(tris[3 * t]), vert(tris[3 * t + 1]), vert(tris[3 * t + 2])};
        if (len2(cross(v[1] - v[0], v[2] - v[0])) < 1e-12f) continue;  // a sliver
        const V3 ends[3][2] = {{v[0], v[1]}, {v[1], v[2]}, {v[2], v[0]}};
        for (const auto& e : ends) m.min_feature = std::fmin(m.min_feature, len(e[1] - e[0]));
        for (const V3& p : v) m.bound = std::fmax(m.bound, len(p));
        const V3 c = (v[0] + v[1] + v[2]) / 3.0f;
        HostHull h;
        for (const V3& p : v) {
            const V3 q = p - c;
            bool near = false;
            for (const float4& w : h.v) near = near || len2(V3{w.x, w.y, w.z} - q) < 1e-6f * 1e-6f;
            if (!near) h.v.push_back(make_float4(q.x, q.y, q.z, 0.0f));
        }
        if (h.v.size() != 3) return AVBD_ERR_INVALID_ARG;
        h.f = {0u, 1u, 2u, 0u, 2u, 1u};
        h.unit_inertia[0] = h.unit_inertia[1] = h.unit_inertia[2] = 0.0f;
        // the hull measures (rows.rs:268-272, shape.rs:1468-1479)
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        h.bound = 0.0f;
        for (const float4& w : h.v) {
            const float p[3] = {w.x, w.y, w.z};
            h.bound = std::fmax(h.bound, std::sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]));
            for (int k = 0; k < 3; k++) {
                lo[k] = std::fmin(lo[k], p[k]);
                hi[k] = std::fmax(hi[k], p[k]);
            }
        }
        h.min_ext = std::fmax(std::fmin(hi[0] - lo[0], std::fmin(hi[1] - lo[1], hi[2] - lo[2])), 0.0f);
        m.cent.push_back(make_float4(c.x, c.y, c.z, 0.0f));
        m.tris.push_back(std::move(h));
    }
    if (m.tris.empty()) m.min_feature = 0.0f;
    std::vector<std::array<float, 6>> bounds;
    for (size_t t = 0; t < m.tris.size(); t++) {
        std::array<float, 6> b{INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        for (const float4& q : m.tris[t].v) {
            const float w[3] = {q.x + m.cent[t].x, q.y + m.cent[t].y, q.z + m.cent[t].z};
            for (int k = 0; k < 3; k++) {
                b[k] = std::fmin(b[k], w[k]);
                b[3 + k] = std::fmax(b[3 + k], w[k]);
            }
        }
        bounds.push_back(b);
    }
    m.order.resize(bounds.size());
    std::iota(m.order.begin(), m.order.end(), 0u);
    m.nodes.clear();
    if (!m.order.empty()) mesh_split(bounds, m.cent, m.order.data(), m.order.size(), 0u, m.nodes);
    if (m.nodes.empty()) m.nodes.push_back(MeshNodeD{{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, 1u, 0u, 0u});
    return AVBD_OK;
}
static int add_ext(AvbdWorld* W, bool compound, const AvbdShapePart* parts, uint32_t n, const float* unit_inertia,
                   uint32_t* id) {
    HostExt e;
    int rc = make_ext(W, compound, parts, n, unit_inertia, e);
    if (rc) return rc;
    rc = host_edit(W);  // the tables are rebuilt with the next full upload
    if (rc) return rc;
    if (id) *id = (uint32_t)W->exts.size();
    W->exts.push_back(std::move(e));
    return AVBD_OK;
}

// A convex hull shared by bodies of shape AVBD_SHAPE_HULL (ConvexHull,
// collision/shape.rs:317-365): the reference's centroid-relative vertices and
// triangle faces, and its inertia per unit mass (ConvexHull::try_inertia).
int avbd_world_add_round(AvbdWorld* W, const AvbdShapePart* inner, const float* unit_inertia, uint32_t* id) {
    return add_ext(W, false, inner, 1, unit_inertia, id);
}

int avbd_world_add_compound(AvbdWorld* W, const AvbdShapePart* parts, uint32_t n, const float* unit_inertia,
                            uint32_t* id) {
    return add_ext(W, true, parts, n, unit_inertia, id);
}

int avbd_world_add_heightfield(AvbdWorld* W, uint32_t rows, uint32_t cols, float cell, const float* heights,
                               uint32_t* id) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    HostHf f;
    int rc = make_hf(rows, cols, cell, heights, f);
    if (rc) return rc;
    cudaSetDevice(W->device);
    rc = host_edit(W);  // the tables are rebuilt with the next full upload
    if (rc) return rc;
    if (id) *id = (uint32_t)W->hfs.size();
    W->hfs.push_back(std::move(f));
    return AVBD_OK;
}

int avbd_world_add_trimesh(AvbdWorld* W, const float* verts, uint32_t nverts, const uint32_t* tris, uint32_t ntris,
                           uint32_t* id) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    HostMesh m;
    int rc = make_mesh(verts, nverts, tris, ntris, m);
    if (rc) return rc;
    cudaSetDevice(W->device);
    rc = host_edit(W);
    if (rc) return rc;
    if (id) *id = (uint32_t)W->meshes.size();
    W->meshes.push_back(std::move(m));
    return AVBD_OK;
}

int avbd_world_add_hull(AvbdWorld* W, const float* verts, uint32_t nv, const uint32_t* faces, uint32_t nf,
                        const float* unit_inertia, uint32_t* hull_id) {
    if (!W || !unit_inertia || (nv && !verts) || (nf && !faces)) return AVBD_ERR_INVALID_ARG;
    HostHull h;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    h.bound = 0.0f;
    for (uint32_t i = 0; i < nv; i++) {
        const float* p = verts + 3 * i;
        if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2])) return AVBD_ERR_NONFINITE;
        h.v.push_back(make_float4(p[0], p[1], p[2], 0.0f));
        h.bound = std::fmax(h.bound, std::sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]));
        for (int k = 0; k < 3; k++) {
            lo[k] = std::fmin(lo[k], p[k]);
            hi[k] = std::fmax(hi[k], p[k]);
        }
    }
    h.min_ext = nv ? std::fmax(std::fmin(hi[0] - lo[0], std::fmin(hi[1] - lo[1], hi[2] - lo[2])), 0.0f) : 0.0f;
    for (uint32_t i = 0; i < 3 * nf; i++) {
        if (faces[i] >= nv) return AVBD_ERR_INVALID_ARG;
        h.f.push_back(faces[i]);
    }
    for (int k = 0; k < 3; k++) {
        if (!std::isfinite(unit_inertia[k])) return AVBD_ERR_NONFINITE;
        h.unit_inertia[k] = unit_inertia[k];
    }
    cudaSetDevice(W->device);
    int rc = host_edit(W);  // the device tables are rebuilt at the next upload
    if (rc) return rc;
    if (hull_id) *hull_id = (uint32_t)W->hulls.size();
    W->hulls.push_back(std::move(h));
    return AVBD_OK;
}

// PhysicsEngine::remove_body (mod.rs:1241-1300) on a one-scene world.
// AvbdEngine::wake_body (mod.rs:833-842) with RigidBody::wake_restore
// (body.rs:412-418) on the host model: a sleeper's mass and inertia return.
// A revolute joint's twist or a prismatic joint's slide from its assembly
// reference (joints_ext.rs:37-51), from the host's body records.
static float joint_coordinate_host(const AvbdWorld* W, const JointRec& r) {
    using namespace avbd;
    const AvbdBody& ba = W->bodies[r.a];
    const AvbdBody& bb = W->bodies[r.b];
    const Q qa{ba.orientation[0], ba.orientation[1], ba.orientation[2], ba.orientation[3]};
    const Q qb{bb.orientation[0], bb.orientation[1], bb.orientation[2], bb.orientation[3]};
    const V3 axis{r.axa[0], r.axa[1], r.axa[2]};
    if (r.kind == AVBD_JOINT_REVOLUTE) return hinge_twist(qa, qb, axis) - r.ref;
    const V3 wa = normalize_or(qrot(qa, axis), VZ());
    const V3 pa = V3{ba.position[0], ba.position[1], ba.position[2]} + qrot(qa, V3{r.la[0], r.la[1], r.la[2]});
    const V3 pb = V3{bb.position[0], bb.position[1], bb.position[2]} + qrot(qb, V3{r.lb[0], r.lb[1], r.lb[2]});
    return dot(pb - pa, wa) - r.refv;
}

// retain_joints (mod.rs:766-784) with joint_remap (migration.rs:74-115):
// the joints marked gone go, a gear whose coupled joint goes goes too, the
// survivors move down and gears follow their joints' new handles.
static void retain_joints(AvbdWorld* W, std::vector<uint8_t> gone) {
    std::vector<JointRec>& js = W->joints;
    for (bool changed = true; changed;) {
        changed = false;
        for (size_t i = 0; i < js.size(); i++)
            if (!gone[i] && js[i].kind == AVBD_JOINT_GEAR && (gone[js[i].gb[0]] || gone[js[i].gb[1]])) {
                gone[i] = 1;
                changed = true;
            }
    }
    std::vector<uint32_t> remap(js.size(), 0u);
    uint32_t next = 0;
    for (size_t i = 0; i < js.size(); i++) remap[i] = gone[i] ? 0u : next++;
    std::vector<JointRec> kept;
    kept.reserve(next);
    for (size_t i = 0; i < js.size(); i++) {
        if (gone[i]) continue;
        JointRec j = js[i];
        if (j.kind == AVBD_JOINT_GEAR) {
            j.gb[0] = remap[j.gb[0]];
            j.gb[1] = remap[j.gb[1]];
        }
        kept.push_back(j);
    }
    js.swap(kept);
}

static void wake_host(AvbdWorld* W, uint32_t h) {
    AvbdBodyAux& a = W->aux[h];
    if (!a.asleep) return;
    a.asleep = 0;
    a.sleep_timer = 0.0f;
    AvbdBody& b = W->bodies[h];
    if (b.body_type == AVBD_BODY_DYNAMIC) {
        bool free_mass = b.mass > 0.0f && std::isfinite(b.mass);
        b.inv_mass = free_mass ? 1.0f / b.mass : 0.0f;
        rest_inertia(b, free_mass ? b.mass : 0.0f, W->hulls, W->exts, b.inertia);
    }
}

int avbd_world_remove_body(AvbdWorld* W, uint32_t hi) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    if (W->scene_off.size() != 2) return AVBD_ERR_UNSUPPORTED;
    cudaSetDevice(W->device);
    int rc = host_edit(W);
    if (rc) return rc;
    const uint32_t N = (uint32_t)W->bodies.size();
    if (hi >= N) return AVBD_OK;  // invalid handles are a no-op
    const uint32_t last = N - 1;
    auto map = [&](uint32_t h) { return h == last ? hi : h; };
    if (W->w.evs) {
        // device event state: trigger pairs of the removed body exit, the
        // others are renumbered; touches and queued contact events are cleared
        const DW& w = W->w;
        uint32_t e[EV_NUM];
        CK(cudaStreamSynchronize(W->st));
        CK(cudaMemcpy(e, w.evs, sizeof(e), cudaMemcpyDeviceToHost));
        std::vector<unsigned long long> prev(e[EV_TRIG_PREV]), keep;
        if (!prev.empty()) CK(cudaMemcpy(prev.data(), w.trig_prev, prev.size() * 8, cudaMemcpyDeviceToHost));
        std::vector<AvbdTriggerEvent> exits;
        for (unsigned long long k : prev) {
            uint32_t a = (uint32_t)(k & 0xffffffffu), b = (uint32_t)(k >> 32);
            if (a == hi || b == hi) {
                exits.push_back(AvbdTriggerEvent{a, b, 0u});
            } else {
                uint32_t x = map(a), y = map(b);
                keep.push_back(((unsigned long long)std::max(x, y) << 32) | std::min(x, y));
            }
        }
        std::sort(keep.begin(), keep.end());
        uint32_t q = e[EV_TN];
        for (const AvbdTriggerEvent& t : exits) {
            if (q < w.tev_cap) CK(cudaMemcpy(w.tev + q, &t, sizeof(t), cudaMemcpyHostToDevice));
            else e[EV_TDROP]++;
            q++;
        }
        e[EV_TN] = std::min(q, w.tev_cap);
        e[EV_TRIG_PREV] = (uint32_t)keep.size();
        e[EV_N] = 0;
        if (!keep.empty()) CK(cudaMemcpy(w.trig_prev, keep.data(), keep.size() * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(w.evs, e, sizeof(e), cudaMemcpyHostToDevice));
        CK(cudaMemset(w.toff, 0, ((size_t)w.N + 1) * 4));
    }
    W->bodies[hi] = W->bodies[last];
    W->bodies.pop_back();
    W->aux[hi] = W->aux[last];
    W->aux.pop_back();
    // pairs: a pair renumbered out of (a < b) order is never matched again by
    // the reference's discovery (it keeps (a, b) as they map): drop it now
    std::vector<AvbdPairState> pairs;
    std::vector<AvbdPointState> points;
    for (size_t i = 0; i < W->pairs.size(); i++) {
        AvbdPairState p = W->pairs[i];
        if (p.a == hi || p.b == hi) continue;
        p.a = map(p.a);
        p.b = map(p.b);
        if (p.a >= p.b) continue;
        pairs.push_back(p);
        for (int k = 0; k < MAX_PTS; k++) points.push_back(W->points[i * MAX_PTS + k]);
    }
    W->pairs.swap(pairs);
    W->points.swap(points);
    std::vector<uint8_t> gone(W->joints.size(), 0);
    for (size_t i = 0; i < W->joints.size(); i++) gone[i] = W->joints[i].a == hi || W->joints[i].b == hi;
    retain_joints(W, std::move(gone));
    for (JointRec& j : W->joints) {
        j.a = map(j.a);
        j.b = map(j.b);
    }
    // every sleeper wakes (mod.rs:1294-1296, body.rs:412-418)
    for (uint32_t h = 0; h < last; h++) wake_host(W, h);
    W->scene_off.back() = last;
    return AVBD_OK;
}

int avbd_world_remove_joint(AvbdWorld* W, uint32_t handle) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = host_edit(W);
    if (rc) return rc;
    if (handle >= W->joints.size()) return AVBD_OK;  // invalid handles are a no-op (mod.rs:1532)
    // both members wake, then the joint goes and later handles move down one
    // (mod.rs:1531-1540, retain_joints mod.rs:766-784)
    wake_host(W, W->joints[handle].a);
    wake_host(W, W->joints[handle].b);
    std::vector<uint8_t> gone(W->joints.size(), 0);
    gone[handle] = 1;
    retain_joints(W, std::move(gone));
    return AVBD_OK;
}

int avbd_world_wake_body(AvbdWorld* W, uint32_t handle) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = host_edit(W);
    if (rc) return rc;
    if (handle < W->bodies.size()) wake_host(W, handle);  // mod.rs:1599-1601, :833-842
    return AVBD_OK;
}

int avbd_world_add_joint(AvbdWorld* W, const AvbdJointDesc* d, uint32_t* handle) {
    if (!W || !d) return AVBD_ERR_INVALID_ARG;
    // validate_joint (migration.rs:160-330): anchors and axes finite, bounds
    // ordered, motor fields finite, a rope longer than zero
    auto finite3 = [](const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); };
    auto bounds_ok = [](float lo, float hi) { return std::isfinite(lo) && std::isfinite(hi) && lo <= hi; };
    if (d->kind > AVBD_JOINT_GEAR) return AVBD_ERR_UNSUPPORTED;
    const bool motor = d->kind == AVBD_JOINT_MOTOR, gear = d->kind == AVBD_JOINT_GEAR;
    // a gear is checked for its ratio alone (migration.rs:193-200)
    if (gear && !std::isfinite(d->gear_ratio)) return AVBD_ERR_JOINT_NONFINITE;
    // a free motor has no anchors (migration.rs:250-252); its drive is checked instead (:331-356)
    if (!motor && !gear && (!finite3(d->local_anchor_a) || !finite3(d->local_anchor_b))) return AVBD_ERR_JOINT_BAD_AXIS;
    if (motor) {
        if (!finite3(d->motor_linear) || !finite3(d->motor_angular)) return AVBD_ERR_JOINT_NONFINITE;
        if (!(std::isfinite(d->motor_max_force) && d->motor_max_force >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
        if (!(std::isfinite(d->motor_max_torque) && d->motor_max_torque >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
        if (!(std::isfinite(d->motor_correction) && d->motor_correction >= 0.0f && d->motor_correction <= 1.0f))
            return AVBD_ERR_JOINT_BAD_BOUNDS;
    }
    const bool axial = d->kind == AVBD_JOINT_REVOLUTE || d->kind == AVBD_JOINT_PRISMATIC;
    if (axial) {
        if (!finite3(d->local_axis_a) || !finite3(d->local_axis_b)) return AVBD_ERR_JOINT_BAD_AXIS;
        if (d->has_limit && !bounds_ok(d->limit_min, d->limit_max)) return AVBD_ERR_JOINT_BAD_BOUNDS;
        if (d->has_motor && !(std::isfinite(d->motor_speed) && std::isfinite(d->motor_max) && d->motor_max >= 0.0f))
            return AVBD_ERR_JOINT_NONFINITE;
    }
    if (d->kind == AVBD_JOINT_WHEEL) {  // migration.rs:284-314
        if (!finite3(d->local_axis_a) || !finite3(d->local_axis_b) || !finite3(d->local_axle_a) ||
            !finite3(d->local_axle_b))
            return AVBD_ERR_JOINT_BAD_AXIS;
        if (!(std::isfinite(d->suspension_hz) && d->suspension_hz >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
        if (!(std::isfinite(d->suspension_damping) && d->suspension_damping >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
        if (d->has_motor && !(std::isfinite(d->motor_speed) && std::isfinite(d->motor_max) && d->motor_max >= 0.0f))
            return AVBD_ERR_JOINT_NONFINITE;
    }
    if (d->kind == AVBD_JOINT_SIXDOF)
        for (int k = 0; k < 6; k++) {
            if (d->axis_config[k] > AVBD_AXIS_LIMITED) return AVBD_ERR_INVALID_ARG;
            if (d->axis_config[k] == AVBD_AXIS_LIMITED && !bounds_ok(d->axis_min[k], d->axis_max[k]))
                return AVBD_ERR_JOINT_BAD_BOUNDS;
        }
    if (d->kind == AVBD_JOINT_ROPE && !(std::isfinite(d->max_distance) && d->max_distance > 0.0f))
        return AVBD_ERR_JOINT_BAD_BOUNDS;
    if (d->kind == AVBD_JOINT_SPRING) {  // validate_motor (migration.rs:366-394)
        if (!std::isfinite(d->spring_rest) || !std::isfinite(d->spring_velocity)) return AVBD_ERR_JOINT_NONFINITE;
        for (float v : {d->spring_stiffness, d->spring_damping, d->spring_max_force})
            if (!(std::isfinite(v) && v >= 0.0f)) return AVBD_ERR_JOINT_NONFINITE;
        if (d->spring_kind > AVBD_MOTOR_SERVO || d->spring_model > AVBD_MODEL_FORCE) return AVBD_ERR_INVALID_ARG;
    }
    cudaSetDevice(W->device);
    int rc = host_edit(W);
    if (rc) return rc;
    uint32_t n = (uint32_t)W->bodies.size();
    // a new constraint wakes both members (mod.rs:1320-1321)
    for (uint32_t h : {d->body_a, d->body_b})
        if (h < n) wake_host(W, h);
    if (d->body_a == d->body_b) return AVBD_ERR_JOINT_SELF;
    if (d->body_a >= n || d->body_b >= n) return AVBD_ERR_JOINT_HANDLES;
    // both members must live in the same scene
    auto scene_of = [&](uint32_t h) {
        return (uint32_t)(std::upper_bound(W->scene_off.begin(), W->scene_off.end(), h) - W->scene_off.begin()) - 1;
    };
    if (scene_of(d->body_a) != scene_of(d->body_b)) return AVBD_ERR_JOINT_HANDLES;
    JointRec j{};
    j.kind = d->kind;
    j.a = d->body_a;
    j.b = d->body_b;
    if (gear) {
        // mod.rs:1329-1404: the coupled joints exist and are hinges or
        // slides; the constant is their coordinates' combination now
        const uint32_t ja = d->gear_joint_a, jb = d->gear_joint_b;
        if (ja >= W->joints.size() || jb >= W->joints.size()) return AVBD_ERR_JOINT_UNKNOWN_REF;
        for (uint32_t r : {ja, jb})
            if (W->joints[r].kind != AVBD_JOINT_REVOLUTE && W->joints[r].kind != AVBD_JOINT_PRISMATIC)
                return AVBD_ERR_UNSUPPORTED;
        // and all its bodies live in the gear's scene
        for (uint32_t r : {ja, jb})
            if (scene_of(W->joints[r].a) != scene_of(d->body_a)) return AVBD_ERR_JOINT_HANDLES;
        j.axa[0] = 1.0f; j.axb[0] = 1.0f;
        j.bxa[0] = 1.0f; j.bxb[0] = 1.0f;
        j.qref[3] = 1.0f;
        j.gb[0] = ja;
        j.gb[1] = jb;
        j.gratio = d->gear_ratio;
        j.refv = joint_coordinate_host(W, W->joints[ja]) + j.gratio * joint_coordinate_host(W, W->joints[jb]);
        for (int k = 0; k < 3; k++) {
            j.st.pen_l[k] = 1.0f;  // JOINT_PENALTY_INIT
            j.st.pen_a[k] = 1.0f;
        }
        W->joints.push_back(j);
        if (handle) *handle = (uint32_t)(W->joints.size() - 1);
        return AVBD_OK;
    }
    if (!motor) {
        std::memcpy(j.la, d->local_anchor_a, 12);
        std::memcpy(j.lb, d->local_anchor_b, 12);
    }
    j.axa[0] = 1.0f; j.axb[0] = 1.0f;
    j.qref[3] = 1.0f;
    // resolve_joint (joint.rs:1251-1400), in the reference's f32 operation order
    using namespace avbd;
    const AvbdBody& ba = W->bodies[j.a];
    const AvbdBody& bb = W->bodies[j.b];
    const Q qa{ba.orientation[0], ba.orientation[1], ba.orientation[2], ba.orientation[3]};
    const Q qb{bb.orientation[0], bb.orientation[1], bb.orientation[2], bb.orientation[3]};
    const V3 xa{ba.position[0], ba.position[1], ba.position[2]}, xb{bb.position[0], bb.position[1], bb.position[2]};
    const V3 la{j.la[0], j.la[1], j.la[2]}, lb{j.lb[0], j.lb[1], j.lb[2]};
    if (axial) {
        const float* aa = d->local_axis_a;
        const float* ab = d->local_axis_b;
        V3 va{aa[0], aa[1], aa[2]}, vb{ab[0], ab[1], ab[2]};
        if (len2(va) < 1e-12f || len2(vb) < 1e-12f) return AVBD_ERR_JOINT_BAD_AXIS;
        V3 na = normalize_or(va, VZ()), nb = normalize_or(vb, VZ());
        j.axa[0] = na.x; j.axa[1] = na.y; j.axa[2] = na.z;
        j.axb[0] = nb.x; j.axb[1] = nb.y; j.axb[2] = nb.z;
        if (d->kind == AVBD_JOINT_REVOLUTE) {
            j.ref = hinge_twist_host(ba.orientation, bb.orientation, j.axa);
        } else {
            V3 wa = normalize_or(qrot(qa, na), VZ());
            j.refv = dot((xb + qrot(qb, lb)) - (xa + qrot(qa, la)), wa);
        }
        j.has_lim = d->has_limit;
        j.lo = d->limit_min;
        j.hi = d->limit_max;
        if (d->has_motor) {
            j.mot_speed = d->motor_speed;
            j.mot_max = d->motor_max;
        }
    } else if (d->kind == AVBD_JOINT_WHEEL) {  // joint.rs:1352-1379
        const float* sa = d->local_axis_a;
        const float* sb = d->local_axis_b;
        V3 va{sa[0], sa[1], sa[2]}, vb{sb[0], sb[1], sb[2]};
        if (len2(va) < 1e-12f || len2(vb) < 1e-12f) return AVBD_ERR_JOINT_BAD_AXIS;
        V3 na = normalize_or(va, VY()), nb = normalize_or(vb, VY());
        j.axa[0] = na.x; j.axa[1] = na.y; j.axa[2] = na.z;
        j.axb[0] = nb.x; j.axb[1] = nb.y; j.axb[2] = nb.z;
        V3 axle_a = orthogonalize_axle(na, V3{d->local_axle_a[0], d->local_axle_a[1], d->local_axle_a[2]});
        V3 axle_b = orthogonalize_axle(nb, V3{d->local_axle_b[0], d->local_axle_b[1], d->local_axle_b[2]});
        j.bxa[0] = axle_a.x; j.bxa[1] = axle_a.y; j.bxa[2] = axle_a.z;
        j.bxb[0] = axle_b.x; j.bxb[1] = axle_b.y; j.bxb[2] = axle_b.z;
        V3 wa = normalize_or(qrot(qa, na), VZ());
        j.refv = dot((xb + qrot(qb, lb)) - (xa + qrot(qa, la)), wa);
        if (d->has_motor) {
            j.mot_speed = d->motor_speed;
            j.mot_max = d->motor_max;
        }
        j.susp[0] = d->suspension_hz;
        j.susp[1] = d->suspension_damping;
    } else if (d->kind == AVBD_JOINT_FIXED || d->kind == AVBD_JOINT_SIXDOF || motor) {
        // the assembly pose (a free motor's only for its rest residual)
        Q r = qmul(conj(qa), qb);
        j.qref[0] = r.x; j.qref[1] = r.y; j.qref[2] = r.z; j.qref[3] = r.w;
        V3 dr = qrot(conj(qa), (xb + qrot(qb, lb)) - (xa + qrot(qa, la)));
        j.dref[0] = dr.x; j.dref[1] = dr.y; j.dref[2] = dr.z;
        if (d->kind == AVBD_JOINT_SIXDOF)
            for (int k = 0; k < 6; k++) {
                j.cfg |= (d->axis_config[k] & 3u) << (2 * k);
                j.six_min[k] = d->axis_min[k];
                j.six_max[k] = d->axis_max[k];
            }
    } else if (d->kind == AVBD_JOINT_DISTANCE) {
        j.refv = len((xb + qrot(qb, lb)) - (xa + qrot(qa, la)));
    } else if (d->kind == AVBD_JOINT_ROPE) {
        j.refv = d->max_distance;
    }
    if (d->kind == AVBD_JOINT_SPRING) {  // the rest length rides in the motor (mod.rs:1487-1493)
        j.refv = d->spring_rest;
        j.spr[0] = d->spring_stiffness;
        j.spr[1] = d->spring_damping;
        j.spr[2] = d->spring_max_force;
        j.spr[3] = d->spring_velocity;
        j.spr_mode = d->spring_kind | (d->spring_model << 4);
    }
    if (motor) {
        std::memcpy(j.mlin, d->motor_linear, 12);
        std::memcpy(j.mang, d->motor_angular, 12);
        j.mforce = d->motor_max_force;
        j.mtorque = d->motor_max_torque;
    }
    for (int k = 0; k < 3; k++) {
        j.st.pen_l[k] = 1.0f;  // JOINT_PENALTY_INIT
        j.st.pen_a[k] = 1.0f;
    }
    W->joints.push_back(j);
    if (handle) *handle = (uint32_t)(W->joints.size() - 1);
    return AVBD_OK;
}

int avbd_world_body_count(const AvbdWorld* W, uint32_t* n) {
    if (!W || !n) return AVBD_ERR_INVALID_ARG;
    *n = W->host_valid ? (uint32_t)W->bodies.size() : (uint32_t)W->w.N;
    return AVBD_OK;
}
int avbd_world_scene_count(const AvbdWorld* W, uint32_t* n) {
    if (!W || !n) return AVBD_ERR_INVALID_ARG;
    *n = (uint32_t)W->scene_off.size() - 1;
    return AVBD_OK;
}

int avbd_world_get_bodies(AvbdWorld* W, uint32_t first, uint32_t n, AvbdBody* out) {
    if (!W || (!out && n)) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    if (W->host_valid) {
        if ((size_t)first + n > W->bodies.size()) return AVBD_ERR_INVALID_ARG;
        std::memcpy(out, W->bodies.data() + first, n * sizeof(AvbdBody));
        return AVBD_OK;
    }
    if ((size_t)first + n > (size_t)W->w.N) return AVBD_ERR_INVALID_ARG;
    if (n == 0) return AVBD_OK;
    k_bodies_out<<<(n + 255) / 256, 256, 0, W->st>>>(W->w, W->d_stage, first, n);
    CK(cudaMemcpyAsync(out, W->d_stage, n * sizeof(AvbdBody), cudaMemcpyDeviceToHost, W->st));
    CK(cudaStreamSynchronize(W->st));
    return AVBD_OK;
}

int avbd_world_set_bodies(AvbdWorld* W, uint32_t first, uint32_t n, const AvbdBody* in) {
    if (!W || (!in && n)) return AVBD_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; i++)
        if (!body_finite(in[i])) return AVBD_ERR_NONFINITE;
    cudaSetDevice(W->device);
    if (W->host_valid) {
        if ((size_t)first + n > W->bodies.size()) return AVBD_ERR_INVALID_ARG;
        for (uint32_t i = 0; i < n; i++) {
            const AvbdBody& o = W->bodies[first + i];
            if (o.shape != in[i].shape || o.body_type != in[i].body_type ||
                std::memcmp(o.shape_params, in[i].shape_params, 12) != 0 || o.flags != in[i].flags)
                W->dev_valid = false;  // static per-body data changed: full re-upload
        }
        std::memcpy(W->bodies.data() + first, in, n * sizeof(AvbdBody));
        if (W->dev_valid) {
            CK(cudaMemcpyAsync(W->d_stage, in, n * sizeof(AvbdBody), cudaMemcpyHostToDevice, W->st));
            k_bodies_in<<<(n + 255) / 256, 256, 0, W->st>>>(W->w, W->d_stage, first, n);
            CK(cudaStreamSynchronize(W->st));
        }
        return AVBD_OK;
    }
    if ((size_t)first + n > (size_t)W->w.N) return AVBD_ERR_INVALID_ARG;
    if (n == 0) return AVBD_OK;
    // device-resident: dynamic fields only (shape, type and flags are fixed
    // after creation on this path)
    CK(cudaMemcpyAsync(W->d_stage, in, n * sizeof(AvbdBody), cudaMemcpyHostToDevice, W->st));
    k_bodies_in<<<(n + 255) / 256, 256, 0, W->st>>>(W->w, W->d_stage, first, n);
    CK(cudaGetLastError());
    return AVBD_OK;
}

int avbd_world_sync(AvbdWorld* W) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(W->st));
    return AVBD_OK;
}

static int begin_steps(AvbdWorld* W) {
    cudaSetDevice(W->device);
    if (W->host_valid && W->dev_valid) {
        W->host_valid = false;
        return AVBD_OK;
    }
    int rc = ensure_device(W);
    if (rc) return rc;
    W->host_valid = false;
    return AVBD_OK;
}

// Does substep i of an n-substep call report events?  The reference emits on
// the last substep of each step (mod.rs:1226-1231); a fixed-step call is one
// step unless an event period splits it.
static bool emit_at(const AvbdWorld* W, int i, int n, bool last_only) {
    if (W->ev_period < 0) return false;
    if (W->ev_period > 0 && !last_only) return (i + 1) % W->ev_period == 0;
    return i == n - 1;
}
static int step_plain_n(AvbdWorld* W, int32_t substeps, bool last_only) {
    for (int i = 0; i < substeps; i++) {
        int rc = substep_plain(W, emit_at(W, i, substeps, last_only));
        if (rc) return rc;
    }
    return AVBD_OK;
}
int avbd_world_step_fixed(AvbdWorld* W, int32_t substeps) {
    if (!W || substeps < 0) return AVBD_ERR_INVALID_ARG;
    if (W->bodies.empty() && W->host_valid) return AVBD_OK;
    int rc = begin_steps(W);
    if (rc) return rc;
    return step_plain_n(W, substeps, false);
}

static int step_graph_n(AvbdWorld* W, int32_t substeps, bool last_only);
int avbd_world_step(AvbdWorld* W, float dt) {  // mod.rs:1212-1235
    if (!W) return AVBD_ERR_INVALID_ARG;
    if (!std::isfinite(dt) || dt <= 0.0f) return AVBD_OK;
    float sd = W->prm.step_dt;
    W->time_debt = std::fmin(W->time_debt + dt, sd * (float)W->prm.max_substeps);
    int n = 0;
    while (W->time_debt >= sd && n < W->prm.max_substeps) {
        W->time_debt -= sd;
        n++;
    }
    if (!n || (W->bodies.empty() && W->host_valid)) return AVBD_OK;
    int rc = begin_steps(W);
    if (rc) return rc;
    // CUDA-graph replay of each substep (identical results to plain launches,
    // one launch per substep instead of a few hundred); events on the last
    // substep of the call, as the reference reports them
    return step_graph_n(W, n, true);
}

// Graph replay: one captured substep per pair-buffer parity.  The primal is
// captured for `graph_cols` colours; a substep that needs more colours stops
// before its iterations (the colouring flags it) and is finished with plain
// launches, then the graphs are re-captured wider.
static int capture(AvbdWorld* W) {
    free_graphs(W, false);
    int base = W->cur;
    for (int emit = 0; emit < 2; emit++)
        for (int k = 0; k < 2; k++) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(W->st, cudaStreamCaptureModeThreadLocal));
            // the per-scene solve walks as many colours as each scene has
            W->w.max_cols = use_scene_solve(W->w, W->tune) ? MAX_COLOURS : W->graph_cols;
            enqueue_front(W, emit != 0);
            enqueue_back(W, W->graph_cols, emit != 0);
            W->w.max_cols = MAX_COLOURS;
            CK(cudaStreamEndCapture(W->st, &g));
            size_t nn = 0;
            cudaGraphGetNodes(g, nullptr, &nn);
            (emit ? W->graph_nodes_emit : W->graph_nodes) = nn;
            cudaError_t e = cudaGraphInstantiate(&W->gexec[W->cur][emit], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                free_graphs(W, false);
                W->cur = base;
                set_pair_ptrs(W);
                return AVBD_ERR_DEVICE;
            }
        }
    // each capture flipped the parity: back where we started
    W->cur = base;
    set_pair_ptrs(W);
    return AVBD_OK;
}

static int step_graph_n(AvbdWorld* W, int32_t substeps, bool last_only) {
    int rc = AVBD_OK;
    for (int i = 0; i < substeps; i++) {
        const bool emit = emit_at(W, i, substeps, last_only);
        if (!W->gexec[0][0] || W->last_ncol > W->graph_cols) {
            if (W->last_ncol == 0) {
                rc = substep_plain(W, emit);  // learn the colour count first
                if (rc) return rc;
                continue;
            }
            W->graph_cols = W->last_ncol + 2;
            rc = capture(W);
            if (rc) return rc;
        }
        int next = 1 - W->cur;  // the parity this substep writes
        CK(cudaGraphLaunch(W->gexec[next][emit ? 1 : 0], W->st));
        W->cur = next;
        set_pair_ptrs(W);
        rc = read_ctr(W);
        if (rc) return rc;
        if (W->h_ctr[C_ERR] & E_CAND_OVERFLOW) {
            W->cur = 1 - W->cur;
            set_pair_ptrs(W);
            CK(cudaMemsetAsync(W->w.ctr + C_ERR, 0, 4, W->st));
            rc = grow_candidates(W);
            if (rc) return rc;
            W->host_valid = false;
            rc = substep_plain(W, emit);
            if (rc) return rc;
            continue;
        }
        int ncol = (int)W->h_ctr[C_NCOL];
        W->last_ncol = ncol;
        if (W->h_ctr[C_ERR] & E_COLOUR_RANGE) {
            // the graph's iterations were skipped: finish this substep plainly
            CK(cudaMemsetAsync(W->w.ctr + C_ERR, 0, 4, W->st));
            enqueue_back(W, ncol, emit);
            rc = read_ctr(W);
            if (rc) return rc;
        }
        accumulate(W);
    }
    return AVBD_OK;
}
int avbd_world_step_graph(AvbdWorld* W, int32_t substeps) {
    if (!W || substeps < 0) return AVBD_ERR_INVALID_ARG;
    if (W->bodies.empty() && W->host_valid) return AVBD_OK;
    int rc = begin_steps(W);
    if (rc) return rc;
    return step_graph_n(W, substeps, false);
}

int avbd_world_get_counters(AvbdWorld* W, AvbdCounters* out) {
    if (!W || !out) return AVBD_ERR_INVALID_ARG;
    *out = W->cum;
    return AVBD_OK;
}

int avbd_world_state_sizes(AvbdWorld* W, uint32_t* nb, uint32_t* np, uint32_t* nj) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = download_all(W);
    if (rc) return rc;
    if (nb) *nb = (uint32_t)W->bodies.size();
    if (np) *np = (uint32_t)W->pairs.size();
    if (nj) *nj = (uint32_t)W->joints.size();
    return AVBD_OK;
}

int avbd_world_export_state(AvbdWorld* W, AvbdBody* bodies, AvbdBodyAux* aux, AvbdPairState* pairs,
                            AvbdPointState* points, AvbdJointState* joints, uint32_t pair_capacity) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = download_all(W);
    if (rc) return rc;
    if ((pairs || points) && pair_capacity < W->pairs.size()) return AVBD_ERR_CAPACITY;
    if (bodies) std::memcpy(bodies, W->bodies.data(), W->bodies.size() * sizeof(AvbdBody));
    if (aux) std::memcpy(aux, W->aux.data(), W->aux.size() * sizeof(AvbdBodyAux));
    if (pairs) std::memcpy(pairs, W->pairs.data(), W->pairs.size() * sizeof(AvbdPairState));
    if (points) std::memcpy(points, W->points.data(), W->points.size() * sizeof(AvbdPointState));
    if (joints)
        for (size_t i = 0; i < W->joints.size(); i++) joints[i] = W->joints[i].st;
    return AVBD_OK;
}

int avbd_world_import_state(AvbdWorld* W, const AvbdBody* bodies, const AvbdBodyAux* aux, const AvbdPairState* pairs,
                            const AvbdPointState* points, uint32_t npairs, const AvbdJointState* joints) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = host_edit(W);
    if (rc) return rc;
    size_t n = W->bodies.size();
    if (bodies) {
        for (size_t i = 0; i < n; i++)
            if (!body_finite(bodies[i])) return AVBD_ERR_NONFINITE;
        std::memcpy(W->bodies.data(), bodies, n * sizeof(AvbdBody));
    }
    if (aux) std::memcpy(W->aux.data(), aux, n * sizeof(AvbdBodyAux));
    if (pairs) {
        if (npairs && !points) return AVBD_ERR_INVALID_ARG;
        for (uint32_t i = 0; i < npairs; i++)
            if (pairs[i].a >= n || pairs[i].b >= n || pairs[i].a >= pairs[i].b || pairs[i].npoints > MAX_PTS)
                return AVBD_ERR_INVALID_ARG;
        W->pairs.assign(pairs, pairs + npairs);
        W->points.assign(points, points + (size_t)npairs * MAX_PTS);
    }
    if (joints)
        for (size_t i = 0; i < W->joints.size(); i++) W->joints[i].st = joints[i];
    W->time_debt = 0.0f;
    return AVBD_OK;
}

int avbd_world_get_colours(AvbdWorld* W, int32_t* colours, uint32_t n) {
    if (!W || !colours) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    if (!W->dev_valid || !W->w.colour) {
        for (uint32_t i = 0; i < n; i++) colours[i] = -1;
        return AVBD_OK;
    }
    if (n > (uint32_t)W->w.N) return AVBD_ERR_INVALID_ARG;
    CK(cudaMemcpyAsync(colours, W->w.colour, n * 4, cudaMemcpyDeviceToHost, W->st));
    CK(cudaStreamSynchronize(W->st));
    return AVBD_OK;
}

// RigidBody::new_sphere / new_box / new_capsule / try_new_halfspace
// (body.rs:346-376, :470-576, :873-889): default materials and mass triple.
int avbd_body_init(AvbdBody* out, uint32_t shape, const float* params, const float* position, float mass) {
    if (!out || !params || !position) return AVBD_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    float rest = 0.3f, fric = 0.5f;
    float sp[3] = {params[0], params[1], params[2]};
    if (shape == AVBD_SHAPE_SPHERE) { rest = 0.5f; fric = 0.3f; }
    else if (shape == AVBD_SHAPE_CAPSULE || shape == AVBD_SHAPE_CYLINDER) { rest = 0.4f; fric = 0.4f; }
    else if (shape == AVBD_SHAPE_CONE) { rest = 0.3f; fric = 0.5f; }
    else if (shape == AVBD_SHAPE_HALFSPACE) {
        if (mass > 0.0f && std::isfinite(mass)) return AVBD_ERR_INVALID_ARG;
        float l = std::sqrt((sp[0] * sp[0] + sp[1] * sp[1]) + sp[2] * sp[2]);
        float r = 1.0f / l;
        if (!std::isfinite(r) || !(r > 0.0f)) return AVBD_ERR_INVALID_ARG;
        for (float& v : sp) v *= r;
        rest = 0.3f; fric = 0.6f;
    } else if (shape != AVBD_SHAPE_BOX && shape != AVBD_SHAPE_CYLINDER && shape != AVBD_SHAPE_CONE) {
        return AVBD_ERR_UNSUPPORTED;  // hulls: fill the record with the hull's mass properties
    }
    bool free_mass = mass > 0.0f && std::isfinite(mass);
    std::memcpy(out->position, position, 12);
    out->orientation[3] = 1.0f;
    out->mass = free_mass ? mass : 0.0f;
    out->inv_mass = free_mass ? 1.0f / mass : 0.0f;
    shape_inertia(shape, sp, free_mass ? mass : 0.0f, out->inertia);
    out->restitution = rest;
    out->friction = fric;
    out->friction_transverse = fric;
    out->shape = shape;
    std::memcpy(out->shape_params, sp, 12);
    out->collision_layer = 1;
    out->collision_mask = 0xffffffffu;
    out->body_type = mass > 0.0f ? AVBD_BODY_DYNAMIC : AVBD_BODY_STATIC;
    return AVBD_OK;
}

int avbd_set_precision(AvbdWorld* W, int fast) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    W->tune.fast = fast ? 1 : 0;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_set_work_order(AvbdWorld* W, int by_work) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    W->tune.sort_work = by_work ? 1 : 0;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_set_occupancy(AvbdWorld* W, int min_blocks) {
    if (!W || (min_blocks != 4 && min_blocks != 6 && min_blocks != 8)) return AVBD_ERR_INVALID_ARG;
    W->tune.primal_minb = min_blocks;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_set_tuning(AvbdWorld* W, int primal_lanes, int primal_block) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    if (primal_lanes != AVBD_PRIMAL_SCENES && primal_lanes != 0 && primal_lanes != 1 && primal_lanes != 4 &&
        primal_lanes != 8 && primal_lanes != 16 && primal_lanes != 32)
        return AVBD_ERR_INVALID_ARG;
    if (primal_block < 32 || primal_block > 1024 || primal_block % 32) return AVBD_ERR_INVALID_ARG;
    // the thread-per-body primal is register-bounded for 128-thread blocks
    if (primal_lanes == 1 && primal_block > 128) return AVBD_ERR_INVALID_ARG;
    if (primal_lanes == AVBD_PRIMAL_SCENES && primal_block != 128 && primal_block != 256 && primal_block != 512)
        return AVBD_ERR_INVALID_ARG;
    const bool need_contrib = primal_lanes == 0 ||
                              (primal_lanes < 0 && W->w.max_scene > (uint32_t)SCENE_MAX_BODIES);
    if (need_contrib && W->w.ctr && !W->w.contrib) {
        // the split primal's per-incidence partial systems
        cudaSetDevice(W->device);
        W->w.contrib = W->mem.get<float4>((size_t)W->cand_cap * 2 * 7);
        if (!W->w.contrib) return AVBD_ERR_DEVICE;
        W->w.contrib_slots = (uint32_t)(W->cand_cap * 2);
        W->mem_gen++;
    }
    W->tune.primal_lanes = primal_lanes;
    W->tune.primal_block = primal_block;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_set_joint_stiffness(AvbdWorld* W, float k) {
    if (!W || !std::isfinite(k) || k < 0.0f) return AVBD_ERR_INVALID_ARG;
    W->w.joint_k = k;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_set_broadphase(AvbdWorld* W, int small_scene_max) {
    if (!W || small_scene_max < 0 || small_scene_max > 2048) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = host_edit(W);  // the sweep plan is built with the device buffers
    if (rc) return rc;
    W->tune.small_scene_max = small_scene_max;
    W->n_alloc = 0;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_set_sweep(AvbdWorld* W, int rows) {
    if (!W || rows < 0 || rows > 1) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = host_edit(W);  // the sweep plan is built with the device buffers
    if (rc) return rc;
    W->tune.sweep_rows = rows;
    W->n_alloc = 0;
    free_graphs(W);
    return AVBD_OK;
}

int avbd_abi_version(void) { return AVBD_ABI_VERSION; }

// Bracket a region for profilers started with collection off
// (`ncu --profile-from-start off`).
int avbd_profiler(int on) {
    cudaError_t e = on ? cudaProfilerStart() : cudaProfilerStop();
    return e == cudaSuccess ? AVBD_OK : AVBD_ERR_DEVICE;
}

// Device time of `substeps` substeps, bracketed by CUDA events on the world's
// stream (graph replay when use_graph != 0).
int avbd_world_step_timed(AvbdWorld* W, int32_t substeps, int32_t use_graph, float* ms) {
    if (!W || !ms || substeps < 0) return AVBD_ERR_INVALID_ARG;
    int rc = begin_steps(W);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaStreamSynchronize(W->st));
    CK(cudaEventRecord(e0, W->st));
    rc = use_graph ? avbd_world_step_graph(W, substeps) : avbd_world_step_fixed(W, substeps);
    CK(cudaEventRecord(e1, W->st));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int avbd_world_flush_cache(AvbdWorld* W) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    const size_t bytes = size_t(256) << 20;
    if (!W->flush_buf) CK(cudaMalloc(&W->flush_buf, bytes));
    CK(cudaMemsetAsync(W->flush_buf, W->cum.steps & 0xff, bytes, W->st));
    CK(cudaStreamSynchronize(W->st));
    return AVBD_OK;
}

// One substep through plain launches with an event between phases:
// ms[0] wake+torque, [1] broadphase, [2] CCD, [3] discovery, [4] wake+CSR+
// targets+decay, [5] colouring, [6] primal (all colours, all iterations),
// [7] dual (all iterations), [8] BDF1+sleep.  info[0] = colours,
// info[1] = primal launches, info[2] = awake dynamic bodies swept,
// info[3] = pairs, info[4] = points.
int avbd_world_profile_substep(AvbdWorld* W, float* ms, uint32_t* info) {
    if (!W || !ms || !info) return AVBD_ERR_INVALID_ARG;
    int rc = begin_steps(W);
    if (rc) return rc;
    cudaEvent_t ev[10];
    for (auto& e : ev) CK(cudaEventCreate(&e));
    cudaStream_t st = W->st;
    CK(cudaStreamSynchronize(st));
    W->cur = 1 - W->cur;
    set_pair_ptrs(W);
    const DW& w = W->w;
    CK(cudaEventRecord(ev[0], st));
    launch_begin_substep(w, st);
    launch_wake_joint_motion(w, st);
    launch_gear_mem(w, st);
    launch_torque(w, st);
    CK(cudaEventRecord(ev[1], st));
    launch_broadphase(w, W->plan, st);
    CK(cudaEventRecord(ev[2], st));
    launch_ccd(w, st);
    CK(cudaEventRecord(ev[3], st));
    launch_discovery(w, W->scan_tmp, st, W->ev_period >= 0 && W->has_trig);
    CK(cudaEventRecord(ev[4], st));
    launch_post_discovery(w, W->scan_tmp, st);
    CK(cudaEventRecord(ev[5], st));
    launch_colouring(w, W->tune, W->scan_tmp, st);
    const bool scene_solve = use_scene_solve(w, W->tune);
    if (!scene_solve) launch_solve_prep(w, W->tune, st);
    CK(cudaEventRecord(ev[6], st));
    rc = read_ctr(W);
    if (rc) return rc;
    for (int i = 0; i < 6; i++) CK(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
    if (W->h_ctr[C_ERR]) return AVBD_ERR_CAPACITY;
    int ncol = (int)W->h_ctr[C_NCOL];
    uint32_t col_total = 0;
    CK(cudaMemcpy(&col_total, w.col_cnt + MAX_COLOURS, 4, cudaMemcpyDeviceToHost));
    float prim = 0.0f, dual = 0.0f;
    if (scene_solve) {
        // primal and dual of every iteration in one launch: reported as primal
        CK(cudaEventRecord(ev[6], st));
        launch_scene_solve(w, W->tune, st);
        CK(cudaEventRecord(ev[7], st));
        CK(cudaEventSynchronize(ev[7]));
        CK(cudaEventElapsedTime(&prim, ev[6], ev[7]));
    }
    for (int it = 0; it < (scene_solve ? 0 : w.iterations); it++) {
        float t;
        CK(cudaEventRecord(ev[6], st));
        for (int c = 0; c < ncol; c++) launch_primal_colour(w, W->tune, c, (uint32_t)w.N, st);
        CK(cudaEventRecord(ev[7], st));
        launch_dual(w, W->tune, st);
        CK(cudaEventRecord(ev[8], st));
        CK(cudaEventSynchronize(ev[8]));
        CK(cudaEventElapsedTime(&t, ev[6], ev[7]));
        prim += t;
        CK(cudaEventElapsedTime(&t, ev[7], ev[8]));
        dual += t;
    }
    CK(cudaEventRecord(ev[8], st));
    launch_finish_substep(w, W->tune, st);
    if (W->ev_period >= 0) launch_events(w, 1, W->has_trig, W->scan_tmp, st);
    CK(cudaEventRecord(ev[9], st));
    CK(cudaEventSynchronize(ev[9]));
    ms[6] = prim;
    ms[7] = dual;
    CK(cudaEventElapsedTime(&ms[8], ev[8], ev[9]));
    rc = read_ctr(W);
    if (rc) return rc;
    accumulate(W);
    info[0] = (uint32_t)ncol;
    info[1] = scene_solve ? 1u : (uint32_t)(ncol * w.iterations);
    info[2] = col_total;
    info[3] = W->h_ctr[C_PAIRS];
    info[4] = W->h_ctr[C_POINTS];
    for (auto& e : ev) cudaEventDestroy(e);
    return AVBD_OK;
}

int avbd_world_graph_nodes(AvbdWorld* W, uint32_t* n) {
    if (!W || !n) return AVBD_ERR_INVALID_ARG;
    *n = (uint32_t)W->graph_nodes;
    return AVBD_OK;
}
int avbd_world_graph_nodes_emit(AvbdWorld* W, uint32_t* n) {
    if (!W || !n) return AVBD_ERR_INVALID_ARG;
    *n = (uint32_t)W->graph_nodes_emit;
    return AVBD_OK;
}

// ---- events ---------------------------------------------------------------------
int avbd_set_events(AvbdWorld* W, int32_t period) {
    if (!W) return AVBD_ERR_INVALID_ARG;
    W->ev_period = period < 0 ? -1 : period;
    free_graphs(W);
    return AVBD_OK;
}
// counts[4]: contact events queued, trigger events queued, contact events
// dropped (queue full, cumulative), trigger events dropped
int avbd_world_event_counts(AvbdWorld* W, uint32_t* counts) {
    if (!W || !counts) return AVBD_ERR_INVALID_ARG;
    std::memset(counts, 0, 16);
    if (!W->w.evs) return AVBD_OK;
    cudaSetDevice(W->device);
    uint32_t e[EV_NUM];
    CK(cudaStreamSynchronize(W->st));
    CK(cudaMemcpy(e, W->w.evs, sizeof(e), cudaMemcpyDeviceToHost));
    counts[0] = e[EV_N];
    counts[1] = e[EV_TN];
    counts[2] = e[EV_DROP];
    counts[3] = e[EV_TDROP];
    return AVBD_OK;
}
int avbd_world_drain_contact_events(AvbdWorld* W, AvbdContactEvent* out, uint32_t cap, uint32_t* n) {
    return drain(W, 0, out, cap, n);
}
int avbd_world_drain_trigger_events(AvbdWorld* W, AvbdTriggerEvent* out, uint32_t cap, uint32_t* n) {
    return drain(W, 1, out, cap, n);
}

int avbd_adjoint_forward(AvbdWorld* W, int32_t steps, int32_t substeps, int32_t every) {
    if (!W || steps <= 0 || substeps <= 0 || every <= 0) return AVBD_ERR_INVALID_ARG;
    for (const AvbdBody& b : W->bodies)
        if (b.rolling_friction > 0.0f || b.torsion_friction > 0.0f || b.shape >= AVBD_SHAPE_ROUND)
            return AVBD_ERR_UNSUPPORTED;
    // the reverse sweep differentiates ball and revolute rows without motors
    for (const JointRec& j : W->joints)
        if (j.kind > AVBD_JOINT_REVOLUTE || j.mot_max > 0.0f) return AVBD_ERR_UNSUPPORTED;
    int rc = begin_steps(W);
    if (rc) return rc;
    if (W->tune.primal_lanes != 0) {
        // the reverse sweep reuses the split primal's per-incidence row sums
        rc = avbd_set_tuning(W, 0, W->tune.primal_block);
        if (rc) return rc;
    }
    if (!W->w.sort_static) {
        // one pair order for every run: point state crosses checkpoints by index
        W->w.sort_static = 1;
        free_graphs(W);
    }
    AdjTape* t = W->adj;
    if (t && t->N == (uint32_t)W->w.N && t->J == (uint32_t)W->w.J && t->S == (uint32_t)W->w.S) {
        // the same world again: keep the frames, the adjoint state and the
        // recording graphs (still valid while the world's generation holds)
        for (Snap* s : t->ckpt) snap_free(s);
        t->ckpt.clear();
        snap_free(t->fin);
        t->fin = nullptr;
        t->max_pairs = 0;
        t->gk_scene.clear();
    } else {
        adj_free(t);
        t = W->adj = new AdjTape();
    }
    t->steps = steps;
    t->substeps = substeps;
    t->every = every;
    t->N = (uint32_t)W->w.N;
    t->J = (uint32_t)W->w.J;
    t->S = (uint32_t)W->w.S;
    for (int s = 0; s < steps; s++) {
        if (s % every == 0) {
            Snap* sn = nullptr;
            rc = snap_take(W, &sn);
            if (rc) return rc;
            t->ckpt.push_back(sn);
        }
        for (int k = 0; k < substeps; k++) {
            rc = avbd_world_step_graph(W, 1);
            if (rc) return rc;
            t->max_pairs = std::max(t->max_pairs, W->h_ctr[C_PAIRS]);
        }
    }
    return snap_take(W, &t->fin);
}

int avbd_adjoint_grad_joint_stiffness(AvbdWorld* W, float* per_scene) {
    if (!W || !per_scene || !W->adj || W->adj->gk_scene.empty()) return AVBD_ERR_INVALID_ARG;
    std::copy(W->adj->gk_scene.begin(), W->adj->gk_scene.end(), per_scene);
    return AVBD_OK;
}

int avbd_adjoint_trace(AvbdWorld* W, float* max_abs, uint32_t* body, int32_t cap, int32_t* n) {
    if (!W || !n || !W->adj || (cap > 0 && (!max_abs || !body))) return AVBD_ERR_INVALID_ARG;
    const std::vector<uint2>& tr = W->adj->trace;
    *n = (int32_t)tr.size();
    for (int32_t i = 0; i < cap && i < (int32_t)tr.size(); i++) {
        uint32_t bits = tr[i].x;
        std::memcpy(&max_abs[i], &bits, 4);
        body[i] = tr[i].y;
    }
    return AVBD_OK;
}

int avbd_adjoint_timing(AvbdWorld* W, float* ms) {
    if (!W || !ms || !W->adj) return AVBD_ERR_INVALID_ARG;
    ms[0] = W->adj->ms_recompute;
    ms[1] = W->adj->ms_reverse;
    return AVBD_OK;
}

int avbd_adjoint_backward(AvbdWorld* W, const float* grad_final, float* grad_initial, float* grad_friction) {
    if (!W || !W->adj || !grad_final || !grad_initial) return AVBD_ERR_INVALID_ARG;
    AdjTape* t = W->adj;
    if ((uint32_t)W->w.N != t->N || (uint32_t)W->w.J != t->J || (uint32_t)W->w.S != t->S) return AVBD_ERR_INVALID_ARG;
    if (W->tune.primal_lanes != 0) return AVBD_ERR_INVALID_ARG;  // retuned since the forward
    cudaSetDevice(W->device);
    cudaStream_t st = W->st;
    const int per_seg = t->every * t->substeps;
    uint32_t pmax = t->max_pairs;  // point inheritance also indexes the checkpoints' generations
    for (const Snap* s : t->ckpt) pmax = std::max(pmax, s->P);
    int rc = adj_storage(W, t, per_seg, pmax + 64);
    if (rc) return rc;
    if (t->rg.empty() || t->rg_key != adj_graph_key(W)) {
        rc = adj_capture(W, t);
        if (rc) return rc;
    }
    const size_t N = t->N;
    AdjState& A = t->A;
    {
        std::vector<float4> x(N), q(N), v(N), w(N);
        for (size_t h = 0; h < N; h++) {
            const float* g = grad_final + 13 * h;
            x[h] = make_float4(g[0], g[1], g[2], 0.0f);
            q[h] = make_float4(g[3], g[4], g[5], g[6]);
            v[h] = make_float4(g[7], g[8], g[9], 0.0f);
            w[h] = make_float4(g[10], g[11], g[12], 0.0f);
        }
        CK(cudaMemcpyAsync(A.ax, x.data(), N * 16, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(A.aq, q.data(), N * 16, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(A.av, v.data(), N * 16, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(A.aw, w.data(), N * 16, cudaMemcpyHostToDevice, st));
        const size_t Qc = (size_t)t->pcap * MAX_PTS;
        CK(cudaMemsetAsync(A.alam, 0, Qc * 16, st));
        CK(cudaMemsetAsync(A.apen, 0, Qc * 16, st));
        CK(cudaMemsetAsync(A.ascene_mu, 0, t->S * 4, st));
        if (t->J) {
            CK(cudaMemsetAsync(A.ajs, 0, (size_t)t->J * 5 * 16, st));
            CK(cudaMemsetAsync(A.ajk, 0, (size_t)t->J * 4, st));
        }
        CK(cudaStreamSynchronize(st));  // the staging vectors go out of scope
    }
    const int nseg = (int)t->ckpt.size();
    const int total = t->steps * t->substeps;
    if (t->trace_cap < total) {
        if (t->d_trace) cudaFree(t->d_trace);
        t->d_trace = nullptr;
        t->trace_cap = 0;
        CK(cudaMalloc(&t->d_trace, (size_t)total * sizeof(uint2)));
        t->trace_cap = total;
    }
    cudaEvent_t ev[3];
    for (auto& e : ev) CK(cudaEventCreate(&e));
    t->ms_recompute = t->ms_reverse = 0.0f;
    for (int seg = nseg - 1; seg >= 0 && !rc; seg--) {
        CK(cudaEventRecord(ev[0], st));
        rc = snap_restore(W, t->ckpt[seg]);
        const int nsteps = std::min(t->every, t->steps - seg * t->every);
        const int nsub = nsteps * t->substeps;
        for (int k = 0; k < nsub && !rc; k++) rc = adj_substep(W, t, k);
        CK(cudaEventRecord(ev[1], st));
        for (int k = nsub - 1; k >= 0 && !rc; k--) {
            rc = adj_reverse(W, t, t->frames[k]);
            if (!rc) launch_adjoint_trace(W->w, t->A, t->d_trace + seg * t->every * t->substeps + k, st);
        }
        CK(cudaEventRecord(ev[2], st));
        CK(cudaEventSynchronize(ev[2]));
        float a = 0.0f, b = 0.0f;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        t->ms_recompute += a;
        t->ms_reverse += b;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    t->trace.resize((size_t)total);
    CK(cudaMemcpyAsync(t->trace.data(), t->d_trace, (size_t)total * sizeof(uint2), cudaMemcpyDeviceToHost, st));
    {
        std::vector<float4> x(N), q(N), v(N), w(N);
        CK(cudaMemcpyAsync(x.data(), A.ax, N * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(q.data(), A.aq, N * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(v.data(), A.av, N * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(w.data(), A.aw, N * 16, cudaMemcpyDeviceToHost, st));
        if (grad_friction) CK(cudaMemcpyAsync(grad_friction, A.ascene_mu, t->S * 4, cudaMemcpyDeviceToHost, st));
        std::vector<float> gk(t->J);
        if (t->J) CK(cudaMemcpyAsync(gk.data(), A.ajk, (size_t)t->J * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        // the stiffness adjoint per scene: a joint belongs to its first body's scene
        t->gk_scene.assign(t->S, 0.0f);
        for (size_t j = 0; j < gk.size() && j < W->joints.size(); j++) {
            uint32_t a = W->joints[j].a;
            size_t sc = std::upper_bound(W->scene_off.begin(), W->scene_off.end(), a) - W->scene_off.begin() - 1;
            if (sc < t->gk_scene.size()) t->gk_scene[sc] += gk[j];
        }
        for (size_t h = 0; h < N; h++) {
            float* g = grad_initial + 13 * h;
            g[0] = x[h].x; g[1] = x[h].y; g[2] = x[h].z;
            g[3] = q[h].x; g[4] = q[h].y; g[5] = q[h].z; g[6] = q[h].w;
            g[7] = v[h].x; g[8] = v[h].y; g[9] = v[h].z;
            g[10] = w[h].x; g[11] = w[h].y; g[12] = w[h].z;
        }
    }
    return snap_restore(W, t->fin);
}

}  // extern "C"

// ---- on-disk snapshot ---------------------------------------------------------------
// A whole world as bytes: a fixed 128-byte header, then the payload sections
// in the order snap_payload writes them.  The header's record sizes tie the
// payload to this format version (JointRec is stored as the world holds it,
// its assembly references already resolved: re-admitting the joints at the
// saved poses would resolve them again from other poses).
namespace {

constexpr char SNAP_MAGIC[8] = {'O', 'R', 'N', 'A', 'V', 'B', 'D', '\0'};
constexpr uint32_t SNAP_ENDIAN = 0x01020304u;

struct SnapHeader {
    char magic[8];
    uint32_t format, abi, header_bytes, endian;
    uint32_t rec[10];  // record sizes: params, settings, body, aux, pair, point, joint, contact event,
                       // trigger event; points per pair
    uint32_t cnt[10];  // bodies, scenes, pairs, joints, hulls, touching pairs, trigger overlaps,
                       // queued contact events, queued trigger events, event words
    uint64_t bytes, checksum, substeps;
};
static_assert(sizeof(SnapHeader) == 128, "the snapshot header is 128 bytes");

// The world's settings that change what a step computes or reports.
struct SnapSettings {
    int32_t primal_lanes, primal_block, primal_minb, small_scene_max, sweep_rows, fast, sort_work;
    int32_t ev_period, sort_static;
    float joint_k, time_debt;
    uint32_t reserved;
};
static_assert(sizeof(SnapSettings) == 48, "settings record");
// The format stores the joint record as the world holds it: a change of
// its layout is a new format version.
static_assert(sizeof(JointRec) == 364, "format 2 joint record");
static_assert(sizeof(AvbdShapePart) == 48, "format 2 shape part record");

// The event state a snapshot carries.
struct SnapEvents {
    uint32_t evs[EV_NUM] = {};
    std::vector<uint32_t> tof, tkeys;         // previous touch set (CSR by the higher handle)
    std::vector<unsigned long long> trig;     // previous trigger overlaps, (b << 32 | a)
    std::vector<AvbdContactEvent> ce;         // undrained queues
    std::vector<AvbdTriggerEvent> te;
};

// FNV-1a, 64-bit (Fowler, Noll, Vo): offset basis 14695981039346656037,
// prime 1099511628211, one byte at a time.
uint64_t fnv1a64(const uint8_t* p, uint64_t n) {
    uint64_t h = 14695981039346656037ull;
    for (uint64_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

struct SnapOut {  // counts when p is null
    uint8_t* p = nullptr;
    uint64_t n = 0;
    void put(const void* src, uint64_t bytes) {
        if (p && bytes) std::memcpy(p + n, src, bytes);
        n += bytes;
    }
    template <class T> void vec(const std::vector<T>& v) { put(v.data(), v.size() * sizeof(T)); }
};

struct SnapIn {
    const uint8_t* p;
    uint64_t n, at = 0;
    bool ok = true;
    bool get(void* dst, uint64_t bytes) {
        if (!ok || bytes > n - at) return ok = false;
        if (bytes) std::memcpy(dst, p + at, bytes);
        at += bytes;
        return true;
    }
    template <class T> bool vec(std::vector<T>& v, uint64_t count) {
        if (!ok || count > (n - at) / sizeof(T)) return ok = false;
        v.resize(count);
        return get(v.data(), count * sizeof(T));
    }
};

void snap_records(SnapHeader& h) {
    const uint32_t rec[10] = {sizeof(AvbdParams), sizeof(SnapSettings), sizeof(AvbdBody), sizeof(AvbdBodyAux),
                              sizeof(AvbdPairState), sizeof(AvbdPointState), sizeof(JointRec),
                              sizeof(AvbdContactEvent), sizeof(AvbdTriggerEvent), (uint32_t)MAX_PTS};
    std::memcpy(h.rec, rec, sizeof(rec));
}

// Header checks shared by every reader: magic, format, layout, size, checksum.
int snap_check(const void* buf, uint64_t size, SnapHeader& h) {
    if (!buf) return AVBD_ERR_INVALID_ARG;
    if (size < sizeof(SnapHeader)) return AVBD_ERR_FORMAT;
    std::memcpy(&h, buf, sizeof(h));
    SnapHeader want{};
    snap_records(want);
    if (std::memcmp(h.magic, SNAP_MAGIC, 8) || h.endian != SNAP_ENDIAN || h.format != AVBD_SNAPSHOT_FORMAT ||
        h.header_bytes != sizeof(SnapHeader) || std::memcmp(h.rec, want.rec, sizeof(want.rec)) ||
        h.cnt[9] != EV_NUM || h.bytes != size)
        return AVBD_ERR_FORMAT;
    const uint8_t* p = (const uint8_t*)buf;
    if (fnv1a64(p + sizeof(h), size - sizeof(h)) != h.checksum) return AVBD_ERR_FORMAT;
    return AVBD_OK;
}

// The event state of a world: empty while it has no device arrays.
int snap_capture_events(AvbdWorld* W, SnapEvents& e) {
    const uint32_t N = (uint32_t)W->bodies.size();
    e.tof.assign(N + 1, 0);
    if (!W->w.evs) return AVBD_OK;
    CK(cudaStreamSynchronize(W->st));
    read_touch_set(W, N, e.tof, e.tkeys);
    if (e.tof.size() != N + 1) e.tof.assign(N + 1, 0);
    CK(cudaMemcpy(e.evs, W->w.evs, sizeof(e.evs), cudaMemcpyDeviceToHost));
    const uint32_t nt = std::min<uint32_t>(e.evs[EV_TRIG_PREV], TRIG_CAP);
    const uint32_t nce = std::min<uint32_t>(e.evs[EV_N], W->w.ev_cap);
    const uint32_t nte = std::min<uint32_t>(e.evs[EV_TN], W->w.tev_cap);
    e.trig.resize(nt);
    e.ce.resize(nce);
    e.te.resize(nte);
    if (nt) CK(cudaMemcpy(e.trig.data(), W->w.trig_prev, nt * 8ull, cudaMemcpyDeviceToHost));
    if (nce) CK(cudaMemcpy(e.ce.data(), W->w.ev, nce * sizeof(AvbdContactEvent), cudaMemcpyDeviceToHost));
    if (nte) CK(cudaMemcpy(e.te.data(), W->w.tev, nte * sizeof(AvbdTriggerEvent), cudaMemcpyDeviceToHost));
    // the keys are written back into the first key buffer; scratch words cleared
    e.evs[EV_PAR] = 0;
    e.evs[EV_TRIG_NOW] = 0;
    e.evs[EV_TRIG_PREV] = nt;
    e.evs[EV_N] = nce;
    e.evs[EV_TN] = nte;
    for (int k = EV_TRIG_OVF + 1; k < EV_NUM; k++) e.evs[k] = 0;
    return AVBD_OK;
}

void snap_payload(const AvbdWorld* W, const SnapEvents& e, SnapOut& o) {
    SnapSettings s{};
    s.primal_lanes = W->tune.primal_lanes;
    s.primal_block = W->tune.primal_block;
    s.primal_minb = W->tune.primal_minb;
    s.small_scene_max = W->tune.small_scene_max;
    s.sweep_rows = W->tune.sweep_rows;
    s.fast = W->tune.fast;
    s.sort_work = W->tune.sort_work;
    s.ev_period = W->ev_period;
    s.sort_static = W->w.sort_static;
    s.joint_k = W->w.joint_k;
    s.time_debt = W->time_debt;
    o.put(&W->prm, sizeof(AvbdParams));
    o.put(&s, sizeof(s));
    o.vec(W->scene_off);
    o.vec(W->bodies);
    o.vec(W->aux);
    o.vec(W->pairs);
    o.vec(W->points);
    o.vec(W->joints);
    for (const HostHull& hh : W->hulls) {
        const uint32_t nv = (uint32_t)hh.v.size(), nf = (uint32_t)hh.f.size();
        o.put(&nv, 4);
        o.put(&nf, 4);
        o.put(hh.unit_inertia, 12);
        o.put(&hh.bound, 4);
        o.put(&hh.min_ext, 4);
        o.vec(hh.v);
        o.vec(hh.f);
    }
    const uint32_t nx = (uint32_t)W->exts.size();
    o.put(&nx, 4);
    for (const HostExt& x : W->exts) {
        const uint32_t flag = x.compound ? 1u : 0u, np = (uint32_t)x.parts.size();
        o.put(&flag, 4);
        o.put(&np, 4);
        o.put(x.unit_inertia, 12);
        o.vec(x.parts);
    }
    const uint32_t nf = (uint32_t)W->hfs.size(), nm = (uint32_t)W->meshes.size();
    o.put(&nf, 4);
    for (const HostHf& f : W->hfs) {
        o.put(&f.rows, 4);
        o.put(&f.cols, 4);
        o.put(&f.cell, 4);
        o.vec(f.h);
    }
    o.put(&nm, 4);
    for (const HostMesh& m : W->meshes) {
        const uint32_t nvf = (uint32_t)m.verts.size(), nti = (uint32_t)m.tris_in.size();
        o.put(&nvf, 4);
        o.put(&nti, 4);
        o.vec(m.verts);
        o.vec(m.tris_in);
    }
    o.put(e.evs, sizeof(e.evs));
    o.vec(e.tof);
    o.vec(e.tkeys);
    o.vec(e.trig);
    o.vec(e.ce);
    o.vec(e.te);
}

// Everything a loaded world's host model needs, checked before any device
// work: every index the device will follow stays inside its array.
int snap_parse(const void* buf, uint64_t size, AvbdWorld* W, SnapEvents& e) {
    SnapHeader h;
    int rc = snap_check(buf, size, h);
    if (rc) return rc;
    const uint32_t N = h.cnt[0], S = h.cnt[1], P = h.cnt[2], J = h.cnt[3], H = h.cnt[4];
    SnapIn in{(const uint8_t*)buf, size, sizeof(SnapHeader)};
    SnapSettings s{};
    in.get(&W->prm, sizeof(AvbdParams));
    in.get(&s, sizeof(s));
    in.vec(W->scene_off, (uint64_t)S + 1);
    in.vec(W->bodies, N);
    in.vec(W->aux, N);
    in.vec(W->pairs, P);
    in.vec(W->points, (uint64_t)P * MAX_PTS);
    in.vec(W->joints, J);
    for (uint32_t k = 0; k < H && in.ok; k++) {
        HostHull hh;
        uint32_t nv = 0, nf = 0;
        in.get(&nv, 4);
        in.get(&nf, 4);
        in.get(hh.unit_inertia, 12);
        in.get(&hh.bound, 4);
        in.get(&hh.min_ext, 4);
        in.vec(hh.v, nv);
        in.vec(hh.f, nf);
        if (!in.ok || nv == 0 || nf % 3) return AVBD_ERR_FORMAT;
        for (uint32_t x : hh.f)
            if (x >= nv) return AVBD_ERR_FORMAT;
        W->hulls.push_back(std::move(hh));
    }
    uint32_t nx = 0;
    in.get(&nx, 4);
    for (uint32_t k = 0; k < nx && in.ok; k++) {
        uint32_t flag = 0, np = 0;
        float ui[3];
        std::vector<AvbdShapePart> parts;
        in.get(&flag, 4);
        in.get(&np, 4);
        in.get(ui, 12);
        in.vec(parts, np);
        if (!in.ok || flag > 1u) return AVBD_ERR_FORMAT;
        HostExt x;
        if (make_ext(W, flag != 0, parts.data(), np, ui, x)) return AVBD_ERR_FORMAT;
        W->exts.push_back(std::move(x));
    }
    uint32_t nf = 0, nm = 0;
    in.get(&nf, 4);
    for (uint32_t k = 0; k < nf && in.ok; k++) {
        uint32_t rows = 0, cols = 0;
        float cell = 0.0f;
        std::vector<float> h;
        in.get(&rows, 4);
        in.get(&cols, 4);
        in.get(&cell, 4);
        in.vec(h, (uint64_t)rows * cols);
        HostHf f;
        if (!in.ok || make_hf(rows, cols, cell, h.data(), f)) return AVBD_ERR_FORMAT;
        W->hfs.push_back(std::move(f));
    }
    in.get(&nm, 4);
    for (uint32_t k = 0; k < nm && in.ok; k++) {
        uint32_t nvf = 0, nti = 0;
        std::vector<float> v;
        std::vector<uint32_t> t;
        in.get(&nvf, 4);
        in.get(&nti, 4);
        in.vec(v, nvf);
        in.vec(t, nti);
        HostMesh m;
        if (!in.ok || nvf % 3 || nti % 3 || make_mesh(v.data(), nvf / 3, t.data(), nti / 3, m)) return AVBD_ERR_FORMAT;
        W->meshes.push_back(std::move(m));
    }
    in.get(e.evs, sizeof(e.evs));
    in.vec(e.tof, (uint64_t)N + 1);
    in.vec(e.tkeys, h.cnt[5]);
    in.vec(e.trig, h.cnt[6]);
    in.vec(e.ce, h.cnt[7]);
    in.vec(e.te, h.cnt[8]);
    if (!in.ok || in.at != size) return AVBD_ERR_FORMAT;
    // parameters and settings as the setters would accept them
    const AvbdParams& p = W->prm;
    if (!(p.step_dt > 0.0f) || !std::isfinite(p.step_dt) || p.iterations < 0 || p.max_substeps < 1)
        return AVBD_ERR_FORMAT;
    const int lanes_ok[] = {AVBD_PRIMAL_SCENES, 0, 1, 4, 8, 16, 32};
    if (std::find(std::begin(lanes_ok), std::end(lanes_ok), s.primal_lanes) == std::end(lanes_ok) ||
        s.primal_block < 32 || s.primal_block > 1024 || s.primal_block % 32 ||
        (s.primal_lanes == 1 && s.primal_block > 128) ||
        (s.primal_lanes == AVBD_PRIMAL_SCENES && s.primal_block != 128 && s.primal_block != 256 &&
         s.primal_block != 512) ||
        (s.primal_minb != 4 && s.primal_minb != 6 && s.primal_minb != 8) || s.small_scene_max < 0 ||
        s.small_scene_max > 2048 || (s.sweep_rows != 0 && s.sweep_rows != 1) || !std::isfinite(s.joint_k) ||
        s.joint_k < 0.0f || !std::isfinite(s.time_debt))
        return AVBD_ERR_FORMAT;
    W->tune.primal_lanes = s.primal_lanes;
    W->tune.primal_block = s.primal_block;
    W->tune.primal_minb = s.primal_minb;
    W->tune.small_scene_max = s.small_scene_max;
    W->tune.sweep_rows = s.sweep_rows;
    W->tune.fast = s.fast ? 1 : 0;
    W->tune.sort_work = s.sort_work ? 1 : 0;
    W->ev_period = s.ev_period < 0 ? -1 : s.ev_period;
    W->w.sort_static = s.sort_static ? 1 : 0;
    W->w.joint_k = s.joint_k;
    W->time_debt = s.time_debt;
    W->cum.steps = h.substeps;
    // scenes, bodies, pairs, joints
    if (S == 0 || W->scene_off[0] != 0 || W->scene_off[S] != N) return AVBD_ERR_FORMAT;
    for (uint32_t k = 0; k < S; k++)
        if (W->scene_off[k + 1] < W->scene_off[k]) return AVBD_ERR_FORMAT;
    auto scene_of = [&](uint32_t x) {
        return (uint32_t)(std::upper_bound(W->scene_off.begin(), W->scene_off.end(), x) - W->scene_off.begin()) - 1;
    };
    for (const AvbdBody& b : W->bodies) {
        if (!body_finite(b) || b.shape > AVBD_SHAPE_TRIMESH) return AVBD_ERR_FORMAT;
        if (b.shape == AVBD_SHAPE_HEIGHTFIELD &&
            (!(b.shape_params[0] >= 0.0f && (size_t)b.shape_params[0] < W->hfs.size()) ||
             b.body_type == AVBD_BODY_DYNAMIC))
            return AVBD_ERR_FORMAT;
        if (b.shape == AVBD_SHAPE_TRIMESH &&
            (!(b.shape_params[0] >= 0.0f && (size_t)b.shape_params[0] < W->meshes.size()) ||
             b.body_type == AVBD_BODY_DYNAMIC))
            return AVBD_ERR_FORMAT;
        if (b.shape == AVBD_SHAPE_HULL && !((size_t)b.shape_params[0] < W->hulls.size())) return AVBD_ERR_FORMAT;
        if ((b.shape == AVBD_SHAPE_ROUND || b.shape == AVBD_SHAPE_COMPOUND) &&
            (!(b.shape_params[0] >= 0.0f && (size_t)b.shape_params[0] < W->exts.size()) ||
             W->exts[(size_t)b.shape_params[0]].compound != (b.shape == AVBD_SHAPE_COMPOUND)))
            return AVBD_ERR_FORMAT;
    }
    for (const AvbdPairState& q : W->pairs)
        if (q.a >= q.b || q.b >= N || q.npoints > (uint32_t)MAX_PTS || scene_of(q.a) != scene_of(q.b))
            return AVBD_ERR_FORMAT;
    for (const JointRec& j : W->joints) {
        if (j.kind > AVBD_JOINT_GEAR || j.a >= N || j.b >= N || j.a == j.b || scene_of(j.a) != scene_of(j.b))
            return AVBD_ERR_FORMAT;
        if (j.kind != AVBD_JOINT_GEAR) continue;
        for (uint32_t r : j.gb)
            if (r >= J || (W->joints[r].kind != AVBD_JOINT_REVOLUTE && W->joints[r].kind != AVBD_JOINT_PRISMATIC) ||
                scene_of(W->joints[r].a) != scene_of(j.a))
                return AVBD_ERR_FORMAT;
    }
    // event state: a CSR over the bodies, each row's lower handles ascending
    if (e.tof[0] != 0 || e.tof[N] != e.tkeys.size()) return AVBD_ERR_FORMAT;
    for (uint32_t b = 0; b < N; b++) {
        if (e.tof[b + 1] < e.tof[b]) return AVBD_ERR_FORMAT;
        for (uint32_t k = e.tof[b]; k < e.tof[b + 1]; k++)
            if (e.tkeys[k] >= b || (k > e.tof[b] && e.tkeys[k] <= e.tkeys[k - 1])) return AVBD_ERR_FORMAT;
    }
    if (e.trig.size() > (size_t)TRIG_CAP) return AVBD_ERR_FORMAT;
    for (size_t k = 0; k < e.trig.size(); k++) {
        const unsigned long long t = e.trig[k];
        if ((uint32_t)(t >> 32) >= N || (uint32_t)t >= (uint32_t)(t >> 32) || (k && t <= e.trig[k - 1]))
            return AVBD_ERR_FORMAT;
    }
    if (e.evs[EV_N] != e.ce.size() || e.evs[EV_TN] != e.te.size() || e.evs[EV_TRIG_PREV] != e.trig.size() ||
        e.evs[EV_PAR] != 0)
        return AVBD_ERR_FORMAT;
    return AVBD_OK;
}

// Put a parsed event state into a world whose device arrays were just made.
int snap_restore_events(AvbdWorld* W, const SnapEvents& e) {
    DW& w = W->w;
    const uint32_t N = (uint32_t)W->bodies.size();
    if (!w.evs) return (e.tkeys.empty() && e.trig.empty() && e.ce.empty() && e.te.empty()) ? AVBD_OK : AVBD_ERR_FORMAT;
    if (e.ce.size() > w.ev_cap || e.te.size() > w.tev_cap || e.tkeys.size() > W->cand_cap || (uint32_t)w.N != N)
        return AVBD_ERR_FORMAT;
    CK(cudaStreamSynchronize(W->st));
    CK(cudaMemcpy(w.evs, e.evs, sizeof(e.evs), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.toff, e.tof.data(), ((size_t)N + 1) * 4, cudaMemcpyHostToDevice));
    if (!e.tkeys.empty()) CK(cudaMemcpy(w.tk0, e.tkeys.data(), e.tkeys.size() * 4, cudaMemcpyHostToDevice));
    if (!e.trig.empty()) CK(cudaMemcpy(w.trig_prev, e.trig.data(), e.trig.size() * 8, cudaMemcpyHostToDevice));
    if (!e.ce.empty())
        CK(cudaMemcpy(w.ev, e.ce.data(), e.ce.size() * sizeof(AvbdContactEvent), cudaMemcpyHostToDevice));
    if (!e.te.empty())
        CK(cudaMemcpy(w.tev, e.te.data(), e.te.size() * sizeof(AvbdTriggerEvent), cudaMemcpyHostToDevice));
    return AVBD_OK;
}

}  // namespace

extern "C" {

int avbd_snapshot_info(const void* buf, uint64_t size, AvbdSnapshotInfo* info) {
    if (!info) return AVBD_ERR_INVALID_ARG;
    SnapHeader h;
    int rc = snap_check(buf, size, h);
    if (rc) return rc;
    {
        // every check a load makes on the host, the contents included
        AvbdWorld probe;
        SnapEvents e;
        rc = snap_parse(buf, size, &probe, e);
        if (rc) return rc;
    }
    std::memset(info, 0, sizeof(*info));
    info->format = h.format;
    info->abi = h.abi;
    info->nbodies = h.cnt[0];
    info->nscenes = h.cnt[1];
    info->npairs = h.cnt[2];
    info->njoints = h.cnt[3];
    info->nhulls = h.cnt[4];
    info->ntouch = h.cnt[5];
    info->ntrigger = h.cnt[6];
    info->ncontact_events = h.cnt[7];
    info->ntrigger_events = h.cnt[8];
    info->bytes = h.bytes;
    info->substeps = h.substeps;
    return AVBD_OK;
}

int avbd_world_snapshot(AvbdWorld* W, void* buf, uint64_t cap, uint64_t* size) {
    if (!W || !size) return AVBD_ERR_INVALID_ARG;
    cudaSetDevice(W->device);
    int rc = download_all(W);
    if (rc) return rc;
    SnapEvents e;
    rc = snap_capture_events(W, e);
    if (rc) return rc;
    SnapOut count;
    snap_payload(W, e, count);
    *size = sizeof(SnapHeader) + count.n;
    if (!buf) return AVBD_OK;
    if (cap < *size) return AVBD_ERR_CAPACITY;
    SnapHeader h{};
    std::memcpy(h.magic, SNAP_MAGIC, 8);
    h.format = AVBD_SNAPSHOT_FORMAT;
    h.abi = AVBD_ABI_VERSION;
    h.header_bytes = sizeof(SnapHeader);
    h.endian = SNAP_ENDIAN;
    snap_records(h);
    const uint32_t cnt[10] = {(uint32_t)W->bodies.size(), (uint32_t)W->scene_off.size() - 1,
                              (uint32_t)W->pairs.size(), (uint32_t)W->joints.size(), (uint32_t)W->hulls.size(),
                              (uint32_t)e.tkeys.size(), (uint32_t)e.trig.size(), (uint32_t)e.ce.size(),
                              (uint32_t)e.te.size(), (uint32_t)EV_NUM};
    std::memcpy(h.cnt, cnt, sizeof(cnt));
    h.bytes = *size;
    h.substeps = W->cum.steps;
    uint8_t* p = (uint8_t*)buf;
    SnapOut out{p + sizeof(SnapHeader), 0};
    snap_payload(W, e, out);
    h.checksum = fnv1a64(p + sizeof(SnapHeader), out.n);
    std::memcpy(p, &h, sizeof(h));
    return AVBD_OK;
}

int avbd_world_from_snapshot(const void* buf, uint64_t size, int device, AvbdWorld** out) {
    if (!buf || !out) return AVBD_ERR_INVALID_ARG;
    // the whole snapshot is checked on the host before any device work
    AvbdWorld* W = new AvbdWorld();
    SnapEvents e;
    int rc = snap_parse(buf, size, W, e);
    if (rc) {
        delete W;
        return rc;
    }
    rc = open_device(W, device);
    if (rc) return rc;
    if (!W->bodies.empty()) {
        // room for the saved touch set in the key buffers
        W->cand_cap = std::max<uint32_t>(W->cand_cap, (uint32_t)e.tkeys.size() + 1024u);
        rc = upload_all(W);
        if (!rc) rc = snap_restore_events(W, e);
    } else {
        rc = snap_restore_events(W, e);
    }
    if (rc) {
        avbd_world_destroy(W);
        return rc;
    }
    *out = W;
    return AVBD_OK;
}

int avbd_world_save(AvbdWorld* W, const char* path) {
    if (!W || !path) return AVBD_ERR_INVALID_ARG;
    uint64_t n = 0;
    int rc = avbd_world_snapshot(W, nullptr, 0, &n);
    if (rc) return rc;
    std::vector<uint8_t> buf(n);
    rc = avbd_world_snapshot(W, buf.data(), n, &n);
    if (rc) return rc;
    std::string tmp = std::string(path) + ".partial";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return AVBD_ERR_IO;
    const bool ok = std::fwrite(buf.data(), 1, n, f) == n;
    if (std::fclose(f) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return AVBD_ERR_IO;
    }
    return AVBD_OK;
}

int avbd_world_load(const char* path, int device, AvbdWorld** out) {
    if (!path || !out) return AVBD_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return AVBD_ERR_IO;
    std::vector<uint8_t> buf;
    uint8_t chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return AVBD_ERR_IO;
    return avbd_world_from_snapshot(buf.data(), buf.size(), device, out);
}

}  // extern "C"
