// avbd_world.cuh — device-side layout of an AVBD world (flat multi-scene SoA)
// and the solver constants of the reference (crates/physics/src/avbd/mod.rs:154-247,
// crates/physics/src/constants.rs:26-79).
#pragma once
#include "../../include/ornis_avbd.h"
#include "avbd_vec.cuh"

namespace avbd {

constexpr float ALPHA = 0.99f;
constexpr float GAMMA = 0.999f;
constexpr float BETA = 10000.0f;
constexpr float BETA_ANG = 100.0f;
constexpr float MARGIN = 0.01f;
constexpr float PENALTY_MIN = 1.0f;
constexpr float PENALTY_MAX = 1.0e10f;
constexpr float PENALTY_INIT = 1.0f;
constexpr float JOINT_PENALTY_INIT = 1.0f;
constexpr float GEN_MARGIN = 0.05f;
constexpr float EXPAND_SLOP = 0.005f;
constexpr float POINT_MATCH_DIST = 0.03f;
constexpr float LAMBDA_MATCH_DIST = 0.05f;
constexpr float C_EPS = 1e-7f;
constexpr float STICK_THRESH = 0.00001f;
constexpr float SLEEP_LIN = 0.15f;
constexpr float SLEEP_ANG = 0.15f;
constexpr float HALF = 0.5f;
constexpr float SLEEP_TIME = 0.5f;
constexpr float WAKE_IMPACT_SPEED = 0.5f;
constexpr float WAKE_PENETRATION = 0.01f;
constexpr float LIMIT_SLOP_ANG = 0.005f;
constexpr float LIMIT_SLOP_LIN = 0.002f;      // mod.rs:222
constexpr float MIN_EFFECTIVE_MASS = 1e-10f;  // constants.rs:16
constexpr float LIM_PEN_MAX = 1e4f;
constexpr float ROLL_PEN = 100.0f;
constexpr float MIN_TOI_DISP_LENGTH = 1e-9f;
constexpr float SPIN_REST_EPS = 1e-9f;
constexpr float CCD_BOUNCE_SPEED = 1.0f;
constexpr float DEGENERATE_LEN2 = 1e-12f;
constexpr float NEAR_ZERO = 1e-9f;
constexpr float SHAPE_TOUCH = 1e-3f;
constexpr float AXIS_REST_LEN2 = 1e-16f;
constexpr float CCD_TRAVEL_GATE_FRACTION = 0.5f;
constexpr float DEGENERATE_EPS = 1e-12f;
constexpr float FACE_AXIS_EPS = 1e-6f;
constexpr float SPINE_ALIGNMENT_EPS = 1e-6f;
constexpr float TANGENT_REF_AXIS_DOT = 0.9f;
constexpr float JOINT_REST_ERROR = 0.005f;
constexpr float PI_F = 3.14159265358979323846f;
constexpr float TAU_F = 6.28318530717958647692f;
constexpr float POS_CORRECTION_EPS = 1e-6f;  // constants.rs:71
constexpr int MAX_PTS = AVBD_MAX_POINTS;
constexpr int MAX_COLOURS = 64;
constexpr int CCD_ROUNDS = 8;
constexpr int COLOUR_ROUNDS = 24;  // device-wide colouring rounds for scenes above the one-CTA limit
constexpr int SCENE_MAX_BODIES = 2048;  // scenes up to this size are solved by one block each (k_scene_solve)

// body info word: shape kind in bits 0-3, body type in bits 4-5, trigger bit 6
__host__ __device__ __forceinline__ uint32_t info_shape(uint32_t i) { return i & 15u; }
__host__ __device__ __forceinline__ uint32_t info_type(uint32_t i) { return (i >> 4) & 3u; }
__host__ __device__ __forceinline__ bool info_trigger(uint32_t i) { return (i >> 6) & 1u; }

// device counters (indices into DW::ctr)
enum Ctr {
    C_CAND = 0,       // broadphase candidates written this substep
    C_PAIRS = 1,      // live pairs after discovery
    C_ERR = 2,        // error bits (E_*)
    C_BREAKDOWN = 3,  // cumulative LDL breakdowns
    C_CCD = 4,        // cumulative TOI clamps
    C_NCOL = 5,       // colours used this substep (max over scenes)
    C_TIMEOUT = 6,    // cumulative bounded-wait give-ups
    C_FAST = 7,       // fast (CCD) bodies this substep
    C_POINTS = 8,     // live points
    C_SLEEP = 9,      // bodies asleep
    C_CCD_LEFT = 10,  // fast bodies left after the bounded CCD rounds
    C_CCD_PENDING = 11,  // fast bodies not yet clamped this substep
    C_BOXPAIRS = 12,     // box-box pairs handed to the witness kernel
    C_FCAND = 13,        // candidates with a fast (swept) body, this substep
    C_BOXONE = 14,       // pairs with exactly one box (listed from the back of boxlist)
    C_NOBOX = 15,        // pairs without a box (clist)
    C_LONGSEG = 16,      // long static pair segments put in order by the chunk sort
    C_SCENE_Q = 17,      // next entry of scene_order a block of the per-scene solve takes
    C_CCD_HITS = 18,     // swept-cast hits recorded this substep (ccd_hit)
    C_NUM = 19
};
enum ErrBits { E_CAND_OVERFLOW = 1, E_COLOUR_OVERFLOW = 2, E_TIMEOUT = 4, E_COLOUR_RANGE = 8 };

// event state words (indices into DW::evs)
enum EvState {
    EV_N = 0,          // contact events queued
    EV_DROP = 1,       // contact events dropped (queue full), cumulative
    EV_PAR = 2,        // which key buffer holds the previous touch set
    EV_TN = 3,         // trigger events queued
    EV_TDROP = 4,      // trigger events dropped, cumulative
    EV_TRIG_NOW = 5,   // trigger overlaps found by this substep's discovery
    EV_TRIG_PREV = 6,  // size of the previous trigger overlap set
    EV_TRIG_OVF = 7,   // overlaps beyond TRIG_CAP were seen (set is then truncated)
    EV_NUM = 16
};
constexpr int TRIG_CAP = 4096;  // trigger overlaps tracked per world

// A convex hull on the device (ConvexHull, collision/shape.rs:317-365):
// centroid-relative vertices and the reference's triangle faces.
struct HullDesc {
    const float4* v;     // nv vertices
    const uint32_t* f;   // 3 * nf vertex indices
    uint32_t nv, nf;
    float bound, min_ext;  // longest vertex (rows.rs:268-272), smallest extent (shape.rs:1468-1479)
};
// A part of a rounded or compound shape (Shape::Round's inner, a compound
// child and its Pose, collision/shape.rs:95-135): a primitive, its params
// (w = border radius, 0: not rounded) and its pose in the parent frame.
struct PartDesc {
    float4 p;
    float4 pos;
    float4 rot;
    const HullDesc* hull;  // a hull part
    uint32_t kind;
    uint32_t pad;
};
// A heightfield (shape.rs:352-361): row-major heights, rows along +Z, cols
// along +X, spacing `cell`, and its lowest sample.
struct HfDesc {
    const float* h;
    uint32_t rows, cols;
    float cell, y_min;
};
// One node of a mesh's median-split tree: a leaf owns order[a .. a+b), an
// inner node branches to nodes a and b.
struct MeshNodeD {
    float lo[3], hi[3];
    uint32_t leaf, a, b;
};
// A triangle mesh (shape.rs:377-396): centroid-relative triangle hulls, their
// centroids, the tree and its permutation.
struct MeshDesc {
    const HullDesc* tris;
    const float4* cent;
    const MeshNodeD* nodes;
    const uint32_t* order;
    uint32_t ntris, nnodes, norder;
    float min_feature;
};
// A rounded shape (one part, pose unused) or a compound (parts in order).
struct ExtDesc {
    uint32_t first, count;
    uint32_t compound;
    float min_dim;  // shape_min_dimension (rows.rs:393-400)
};

// Everything a kernel needs, passed by value (pointers into one world's
// device allocations).  Scene s owns bodies [scene_off[s], scene_off[s+1]).
struct DW {
    int N;  // bodies
    int S;  // scenes
    int J;  // joints
    int j_all;  // 1: a joint is neither a ball nor a revolute joint (the all-kinds solve kernels)
    float dt;
    V3 gravity;
    int iterations;
    int enable_sleep, enable_ccd;
    uint32_t cand_cap, pair_cap;
    int max_cols;  // colours the launched iteration covers (a CUDA graph fixes it at capture)
    int n_large_scenes;  // host: scenes above the one-CTA sweep and colouring limit
    int sort_static;     // also order static bodies' pair segments (differentiable rollouts)
    float joint_k;       // finite joint stiffness (0: hard joints, the reference's)

    const uint32_t* scene_off;  // S+1
    const uint32_t* scene_of;   // N
    const uint32_t* scene_order;  // S: scenes by descending body count (the per-scene solve's queue)
    uint32_t max_scene;           // bodies of the largest scene
    const uint32_t* plane_off;  // S+1: half-space bodies of each scene
    const uint32_t* plane_list;
    const HullDesc* hulls;  // convex hulls named by AVBD_SHAPE_HULL bodies (shape_params[0])
    uint32_t nhulls;
    const ExtDesc* exts;    // rounded and compound shapes named by their bodies (shape_params[0])
    const PartDesc* parts;
    uint32_t nexts;
    const HfDesc* hfs;      // heightfields named by their bodies
    const MeshDesc* meshes; // triangle meshes named by their bodies
    uint32_t nhfs, nmeshes;

    // bodies
    float4 *pos, *rot, *vel, *angvel, *torque;
    float4 *pos0, *rot0, *inertial, *inertial_rot, *prev_pos, *prev_rot;
    float4 *inertia, *inertia_rest;
    // what a contact row reads of a body, packed in one 64-byte record (4 float4
    // per body), refreshed whenever a pose changes during the iterations of a
    // substep: (x, first shape parameter), q, (x - x0, info word bits),
    // (quat_diff_vec(q, q0), 0)
    float4* kin;
    float4* mat;  // restitution, friction, rolling, torsion
    float4* shp;  // shape params xyz, bound radius w
    float *inv_mass, *inv_mass_rest, *mass, *friction_t, *sleep_timer;
    uint32_t *info, *asleep;
    uint2* filter;  // collision layer, mask
    int32_t* colour;
    int32_t* comp;  // joint component id (-1: no joint)

    // joints (AvbdJoint, avbd/mod.rs:327-402)
    uint32_t* j_kind;
    uint2* j_ab;
    float4 *j_la, *j_lb, *j_axa, *j_axb;  // w of j_axa = reference twist (revolute)
    float4* j_lim;                         // lo, hi, has_limit, acc_lim
    float4 *j_lam_l, *j_lam_a, *j_pen_l, *j_pen_a;
    // reference length (prismatic) / rest length (distance) / maximum (rope),
    // prismatic limit force, motor target speed, motor budget (0: no motor)
    float4* j_ref;
    float4 *j_dref, *j_qref;  // fixed / sixdof assembly anchor separation (A's frame) and qa^-1 qb
    uint32_t* j_cfg;          // sixdof axis configuration: 2 bits per axis, linear x y z then angular
    float4* j_six;            // 3 per joint: (min, max) of the six axes in pairs
    float4* j_sacc;           // 2 per joint: sixdof limited-axis forces (6 used)
    // gears (j_dref.x = ratio, j_ref.x = the constant): the coupled joints,
    // their coordinates at the last step start (raw a, raw b, unwrapped a,
    // unwrapped b) and whether those are set yet
    uint2* j_gb;
    float4* j_gmem;
    uint32_t* j_gset;
    int n_gear;
    // per-body joint adjacency (N+1; 4J): a joint on its two bodies, a gear
    // once on each body of its coupled joints, ascending joint index
    const uint32_t *jofs, *jlist;
    // joints with a motor or a rope, per scene in joint order (their velocity
    // impulses run before the warm start); n_imp of them in all
    const uint32_t *jimp_off, *jimp_list;
    int n_imp;

    // contact pairs: current generation (read by the solver) ...
    uint2* p_ab;
    float4* p_n;  // normal xyz, gap w
    float2* p_mu;
    uint32_t* p_np;
    float4 *q_ra, *q_rb, *q_lam, *q_pen, *q_roll;  // q_rb.w = stuck
    int32_t* q_matched;
    int32_t* p_old;  // previous-generation index of each pair, -1 when new (read by the adjoint)
    uint32_t* offA;  // N+1: pairs whose A side is body h are [offA[h], offA[h+1])
    uint32_t* offB;  // N+1: B-side incidence list
    uint32_t* listB;
    uint32_t* posB;  // pair -> its index in listB
    // split primal: per-colour (pair, side) work lists and per-incidence partial systems
    uint32_t* side_list;  // 2*pair_cap entries: pair * 2 + (1 for the A side, 0 for the B side)
    uint32_t* side_cnt;   // [0, MAX_COLOURS]: list starts; [MAX_COLOURS+1, 2*MAX_COLOURS+1]: cursors
    float4* contrib;      // 7 float4 per incidence slot (21 Hessian + 6 rhs + pad)
    uint32_t contrib_slots;  // incidence slots contrib holds
    // ... and the previous generation (read by discovery for the warm merge)
    uint2* o_ab;
    float4* o_n;
    uint32_t* o_np;
    float4 *oq_ra, *oq_rb, *oq_lam, *oq_pen, *oq_roll;
    uint32_t* o_offA;

    // broadphase / discovery scratch
    uint2* cand;       // candidate (a, b), a < b
    uint8_t* keep;     // per candidate
    uint32_t* cnt;     // per body counters (N+1)
    uint32_t* cur;     // per body cursors
    uint32_t* slot_c;  // final pair slot -> candidate index
    uint32_t* long_seg;            // N: static bodies with a long pair segment (C_LONGSEG of them)
    unsigned long long* seg_key;  // cand_cap: (b, candidate) keys of those segments, sorted per chunk
    uint32_t* boxlist; // box-box pair slots from the front, one-box pair slots from the back
    uint32_t* clist;   // pair slots without a box
    float4 *bd_pa, *bd_pb;  // box-box witnesses per pair slot: (pa, dist), (pb, SAT gap)
    float4 *aabb_lo, *aabb_hi;
    uint32_t* sort_key;
    uint32_t* sort_idx;

    // CCD scratch
    uint32_t* fbody;  // N: the fast bodies of this substep (C_FAST of them)
    uint32_t* fcand;  // cand_cap: candidates with a fast body (C_FCAND of them)
    uint8_t* fast;
    unsigned long long* ccd_best;
    uint32_t* ccd_deps;
    uint8_t* ccd_state;  // 0 pending, 1 final, 2 final+moved
    uint8_t* ccd_recompute;
    // the hits of this substep's casts, 3 float4 each: (t, other, body, cast
    // round as float bits), normal, target witness; ccd_win[h] = the record
    // of h's winning cast, or ~0 (then the apply recomputes it).  Null: the
    // apply always recomputes.
    float4* ccd_hit;
    uint32_t ccd_hit_cap;
    uint32_t* ccd_win;

    // wake / sleep scratch
    uint8_t* flag;  // per body
    uint32_t* comp_flag;

    // events (all null when the world keeps none)
    float4* pre_vel;      // N: linear velocity at the substep start, after torque (mod.rs:874-876)
    // differentiable rollouts: per body, the swept impact applied this
    // substep as [2h] = (normal, velocity factor: 0 kept, else the bounce)
    // and [2h + 1] = (fraction of the sweep x dt, 1 when applied, 0, 0)
    float4* ccd_rec;
    int32_t* ccd_ev_o;    // N: partner of this substep's swept-hit event, -1 none
    float4* ccd_ev_p;     // N: hit point xyz, approach speed w
    float4* ccd_ev_n;     // N: event normal (A toward B)
    uint8_t* t_flag;      // pair_cap: touching (deepest point beyond the begin slop)
    float4* t_wit;        // pair_cap: deepest point xyz, approach speed w
    uint32_t* toff;       // N+1: previous touch set, CSR by the higher handle
    uint32_t *tk0, *tk1;  // pair_cap each: its lower handles (ascending), alternating buffers
    uint32_t *ev_cbe, *ev_ch, *ev_cc, *ev_ct;  // N+1 each: begin/end, hit, swept-hit, touch counts -> slots
    uint32_t* evs;        // EV_* words
    AvbdContactEvent* ev;
    uint32_t ev_cap;
    unsigned long long *trig_now, *trig_prev;  // TRIG_CAP each: (b << 32 | a) overlap keys
    AvbdTriggerEvent* tev;
    uint32_t tev_cap;

    // colouring
    uint32_t* col_cnt;   // MAX_COLOURS+1
    uint32_t* col_list;  // N: swept bodies grouped by colour, ascending index within a colour
    uint32_t *col_key, *col_key2, *col_val, *col_hist;
    uint32_t* ctr;       // counters
};

// One recomputed substep as the adjoint kernels read it: the frozen contact
// set and colouring, the step-start and target poses, and the iterates.
// Pose slice 0 is the pose the iterations start from, slice i+1 the pose
// after the primal sweep of iteration i; point slice 0 is the warm state
// after the decay (lambda.w = the step-start gap C0), slice i+1 the state
// after the dual update of iteration i.
struct AdjFrame {
    uint32_t npairs, ncol;
    size_t qstride;  // point entries per point slice
    // bodies
    float4 *pos0, *rot0, *inertial, *inertial_rot, *vel, *angvel, *inertia;
    float* inv_mass;
    uint32_t* asleep_end;  // asleep after the substep's sleep pass
    float4 *it_pos, *it_rot;  // (iterations + 1) slices of N
    int32_t* colour;
    uint32_t *col_cnt, *col_list;
    uint32_t *offA, *offB, *listB, *posB;
    // pairs and points
    uint2* p_ab;
    float4* p_n;
    float2* p_mu;
    uint32_t* p_np;
    int32_t* p_old;
    float4 *q_ra, *q_rb;
    int32_t* q_matched;
    float4 *it_lam, *it_pen;  // (iterations + 1) slices of qstride
    // split primal: per-colour side lists and, per iteration, the 7 float4
    // row sums of every incidence slot
    uint32_t *side_list, *side_cnt;
    float4* it_contrib;  // iterations slices of cstride
    size_t cstride;
    // joints: per slice (iterations + 1), 5 arrays of J float4: lambda and
    // penalty of the anchor rows, of the hinge rows, and the limit record
    float4* it_joint;
    float4* ccd;  // 2N: the swept impacts of the substep (null without CCD)
};
// Adjoint state.  Body adjoints are of the state between substeps (pose,
// velocities) plus per-substep accumulators; every (pair, side) incidence
// slot holds 4 float4 (pose adjoint pending for the body, step-start pose
// adjoint) so that contributions to a body from its partners are summed in
// a fixed order.
struct AdjState {
    float4 *ax, *aq, *av, *aw;
    float4 *ax0, *aq0, *ay, *aqt;
    float4* slot;
    float4 *alam, *apen;          // points of the current generation (alam.w: adjoint of C0)
    float4 *alam_old, *apen_old;  // points of the previous generation
    float2* amu;                  // per pair
    float* ascene_mu;             // per scene: friction coefficient adjoint
    float4* wd;                   // 3 per body: w = H^-1 d_bar and the step d of its last reversed solve
    float4* jslot;                // 4 per (joint, side): as slot, for joint partners
    float4* ajs;                  // 5 per joint: adjoint of its warm state (lambda, penalty, limit force in .w)
    float* ajk;                   // per joint: adjoint of the joint stiffness, summed over the rollout
    uint32_t* nlong;              // bodies whose incidence slots a block gathers (a floor under many bodies)
    uint32_t* long_list;          // N: those bodies
};

}  // namespace avbd
