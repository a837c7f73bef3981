/*
 * ornis_avbd.h — C ABI of the GB300-native AVBD rigid-body step.
 *
 * This is the drop-in boundary for the AVBD step of Ornis's physics crate.
 * Every entry point replaces one method of the reference's engine seam:
 *
 *   trait PhysicsEngine            crates/physics/src/engine.rs:24-133
 *   impl PhysicsEngine for AvbdEngine   crates/physics/src/avbd/mod.rs:1211-1602
 *   trait GpuAvbdDispatch          crates/physics/src/gpu/avbd.rs:146-151
 *
 * Conventions (kept from the reference):
 *   - Body handles are dense uint32 indices in insertion order
 *     (engine.rs:40-43, avbd/mod.rs:1236-1239).
 *   - A step with a non-finite or non-positive dt is a no-op
 *     (avbd/mod.rs:1213-1215).
 *   - Buffers passed in are caller-owned host memory and are copied; the
 *     library owns all device memory.  One CUDA stream per world; a world is
 *     not thread-safe, distinct worlds are independent.
 *   - Every function returns an int status: AVBD_OK (0) or a negative code.
 *
 * A world holds one or more independent scenes packed into one flat
 * structure-of-arrays on the device (scene s owns the body handles
 * [scene_offsets[s], scene_offsets[s+1])).  Bodies of different scenes never
 * interact.  A world with one scene is the reference's AvbdEngine.
 */
#ifndef ORNIS_AVBD_H
#define ORNIS_AVBD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AVBD_ABI_VERSION 4

/* ---- status codes ------------------------------------------------------ */
#define AVBD_OK 0
#define AVBD_ERR_INVALID_ARG (-1)    /* null pointer, bad size, bad enum       */
#define AVBD_ERR_CAPACITY (-2)       /* a device buffer would overflow         */
#define AVBD_ERR_DEVICE (-3)         /* a CUDA call failed                     */
#define AVBD_ERR_TIMEOUT (-4)        /* a bounded device wait gave up          */
#define AVBD_ERR_NONFINITE (-5)      /* NaN/Inf in an input body               */
#define AVBD_ERR_UNSUPPORTED (-6)    /* shape / joint kind not implemented     */
#define AVBD_ERR_FORMAT (-7)         /* not a snapshot of this format version,
                                        or a damaged one                       */
#define AVBD_ERR_IO (-8)             /* a snapshot file could not be read or
                                        written                                */
/* joint admission errors, mirroring JointError (avbd/mod.rs:1323-1328) */
#define AVBD_ERR_JOINT_SELF (-10)    /* JointError::SelfJoint                  */
#define AVBD_ERR_JOINT_HANDLES (-11) /* JointError::InvalidHandles             */
#define AVBD_ERR_JOINT_BAD_AXIS (-12)/* JointError::BadAxis                    */
#define AVBD_ERR_JOINT_NONFINITE (-13) /* JointError::NonFinite (motor fields)   */
#define AVBD_ERR_JOINT_BAD_BOUNDS (-14)/* JointError::BadBounds (limits, rope)     */
#define AVBD_ERR_JOINT_UNKNOWN_REF (-15)/* JointError::UnknownRef (a gear's joints) */

/* ---- enums --------------------------------------------------------------- */
/* Shape variants on the path (collision/shape.rs); shape_params meaning:     */
#define AVBD_SHAPE_SPHERE 0    /* [radius, -, -]                                */
#define AVBD_SHAPE_BOX 1       /* [hx, hy, hz] half extents                     */
#define AVBD_SHAPE_CAPSULE 2   /* [radius, half_height, -], axis = local +Y     */
#define AVBD_SHAPE_HALFSPACE 3 /* [nx, ny, nz] outward unit normal, body-local */
#define AVBD_SHAPE_CYLINDER 4  /* [radius, half_height, -], axis = local +Y     */
#define AVBD_SHAPE_CONE 5      /* [radius, half_height, -], apex at +half_height */
#define AVBD_SHAPE_HULL 6      /* [hull index, -, -]: a hull of avbd_world_add_hull */
#define AVBD_SHAPE_ROUND 7     /* [shape id, -, -]: a rounded shape of avbd_world_add_round */
#define AVBD_SHAPE_COMPOUND 8  /* [shape id, -, -]: a compound of avbd_world_add_compound */
#define AVBD_SHAPE_HEIGHTFIELD 9 /* [terrain id, -, -]: a grid of avbd_world_add_heightfield */
#define AVBD_SHAPE_TRIMESH 10  /* [mesh id, -, -]: a triangle mesh of avbd_world_add_trimesh */

#define AVBD_BODY_DYNAMIC 0   /* BodyType::Dynamic   */
#define AVBD_BODY_STATIC 1    /* BodyType::Static    */
#define AVBD_BODY_KINEMATIC 2 /* BodyType::Kinematic */

#define AVBD_FLAG_TRIGGER 1u /* RigidBody::is_trigger */

#define AVBD_JOINT_BALL 0      /* JointKind::Ball      (joint.rs:209+)               */
#define AVBD_JOINT_REVOLUTE 1  /* JointKind::Revolute  (optional limit and motor)    */
#define AVBD_JOINT_PRISMATIC 2 /* JointKind::Prismatic (optional limit and motor)    */
#define AVBD_JOINT_FIXED 3     /* JointKind::Fixed     (weld)                        */
#define AVBD_JOINT_DISTANCE 4  /* JointKind::Distance  (rod of the assembly length)  */
#define AVBD_JOINT_ROPE 5      /* JointKind::Rope      (max_distance)                */
#define AVBD_JOINT_SIXDOF 6    /* JointKind::SixDof    (axis_config per axis)        */
#define AVBD_JOINT_MOTOR 7     /* JointKind::Motor     (free velocity drive, no rows) */
#define AVBD_JOINT_SPRING 8    /* JointKind::Spring    (spring-damper along the anchors) */
#define AVBD_JOINT_WHEEL 9     /* JointKind::Wheel     (suspension slide + axle spin)    */
#define AVBD_JOINT_GEAR 10     /* JointKind::Gear      (couples two revolute / prismatic joints) */

/* JointMotor of a spring (joint.rs:951-996) */
#define AVBD_MOTOR_VELOCITY 0  /* MotorKind::Velocity */
#define AVBD_MOTOR_POSITION 1  /* MotorKind::Position */
#define AVBD_MOTOR_SERVO 2     /* MotorKind::Servo */
#define AVBD_MODEL_ACCELERATION 0 /* MotorModel::AccelerationBased (the default) */
#define AVBD_MODEL_FORCE 1        /* MotorModel::ForceBased */

/* SixDof per-axis configuration (AxisConfig, joint.rs) */
#define AVBD_AXIS_FREE 0
#define AVBD_AXIS_LOCKED 1
#define AVBD_AXIS_LIMITED 2

/* ---- plain-old-data records --------------------------------------------- */

/* One rigid body: the fields of RigidBody (body.rs:248-342) that the AVBD
 * step reads or writes.  Orientation is a unit quaternion (x, y, z, w). */
typedef struct AvbdBody {
    float position[3];
    float orientation[4];
    float velocity[3];
    float angular_velocity[3];
    float torque[3];
    float mass;     /* 0 = static                                            */
    float inv_mass; /* 1/mass, or 0                                           */
    float inertia[3]; /* body-frame diagonal inertia                          */
    float restitution;
    float friction;
    float friction_transverse;
    float rolling_friction;
    float torsion_friction;
    uint32_t shape;
    float shape_params[3];
    uint32_t collision_layer;
    uint32_t collision_mask;
    uint32_t body_type;
    uint32_t flags;
} AvbdBody;

/* Joint specification (JointKind, joint.rs:209-330).  Fields a kind does not
 * use are ignored. */
typedef struct AvbdJointDesc {
    uint32_t kind;
    uint32_t body_a;
    uint32_t body_b;
    float local_anchor_a[3];
    float local_anchor_b[3];
    float local_axis_a[3]; /* revolute hinge / prismatic slide axis */
    float local_axis_b[3];
    int32_t has_limit;     /* revolute (rad) / prismatic (m): RevoluteLimit / PrismaticLimit */
    float limit_min;
    float limit_max;
    int32_t has_motor;     /* revolute / prismatic velocity motor (RevoluteMotor / PrismaticMotor) */
    float motor_speed;     /* target_speed (rad/s or m/s) */
    float motor_max;       /* max_torque / max_force */
    float max_distance;    /* rope */
    uint32_t axis_config[6]; /* sixdof: linear x y z, angular x y z in body A's assembly frame */
    float axis_min[6];       /* sixdof limited axes: travel window */
    float axis_max[6];
    /* free motor (JointKind::Motor): B-minus-A velocity targets in the world
     * frame, the force and torque budgets, and the assembly pull (0..1,
     * validated; the AVBD step runs the velocity drive only, as the
     * reference's does) */
    float motor_linear[3];
    float motor_angular[3];
    float motor_max_force;
    float motor_max_torque;
    float motor_correction;
    /* spring (JointKind::Spring): its JointMotor — rest length
     * (target_position), target_velocity, stiffness, damping, max_force,
     * kind (AVBD_MOTOR_*) and model (AVBD_MODEL_*) */
    float spring_rest;
    float spring_velocity;
    float spring_stiffness;
    float spring_damping;
    float spring_max_force;
    uint32_t spring_kind;
    uint32_t spring_model;
    /* wheel (JointKind::Wheel): local_axis_a/b are the suspension axes;
     * the spin axles, and the suspension's frequency (Hz; 0 = rigid) and
     * damping ratio (WheelSuspension); the axle motor is has_motor /
     * motor_speed / motor_max */
    float local_axle_a[3];
    float local_axle_b[3];
    float suspension_hz;
    float suspension_damping;
    /* gear (JointKind::Gear): the handles of the two revolute or prismatic
     * joints it couples and the ratio (coordinate_a + ratio * coordinate_b
     * stays at its value at creation); body_a and body_b are the gear's own
     * bodies (admission, support for sleep) and its anchors are not used */
    uint32_t gear_joint_a;
    uint32_t gear_joint_b;
    float gear_ratio;
    uint32_t reserved;
} AvbdJointDesc;

/* A part of a rounded or compound shape (Shape::Round's inner, a compound
 * child with its Pose; collision/shape.rs:95-135, :144-230). */
typedef struct AvbdShapePart {
    uint32_t shape;       /* AVBD_SHAPE_SPHERE .. AVBD_SHAPE_HULL (no half-space)  */
    float params[3];      /* as a body's shape_params (a hull: its id)            */
    float border_radius;  /* a Shape::Round around the part: > 0; 0 = none        */
    float position[3];    /* pose in the compound's frame (a rounded shape: unused) */
    float orientation[4]; /* x y z w                                              */
} AvbdShapePart;

/* Solver parameters.  avbd_default_params() fills the reference's constants
 * (avbd/mod.rs:154-247, :1205-1210); dt, iterations and the substep count
 * are runtime parameters here because the workloads need 1/120 s, 8 or 12
 * iterations and 2 substeps, which the reference hard-codes. */
typedef struct AvbdParams {
    float gravity[3];
    float step_dt;        /* fixed substep length  (reference DT_STEP 1/60)   */
    int32_t iterations;   /* primal+dual sweeps    (reference ITERS 10)       */
    int32_t max_substeps; /* accumulator cap       (reference MAX_SUBSTEPS 4) */
    int32_t enable_sleep; /* 1 = reference sleep bookkeeping                  */
    int32_t enable_ccd;   /* 1 = reference linear TOI clamp                   */
} AvbdParams;

/* Per-body solver state outside RigidBody (avbd/mod.rs:425-464). */
typedef struct AvbdBodyAux {
    float prev_position[3];
    float prev_orientation[4];
    float sleep_timer;
    uint32_t asleep;
} AvbdBodyAux;

/* One contact pair (AvbdPair, avbd/mod.rs:269-281).  Pairs are exported in
 * ascending (a, b) order; a < b are body handles. */
typedef struct AvbdPairState {
    uint32_t a;
    uint32_t b;
    float normal[3];
    float mu[2];
    float gap;
    uint32_t npoints;
} AvbdPairState;

/* One contact point (AvbdPoint, avbd/mod.rs:253-265).  Points are exported
 * in fixed slots of AVBD_MAX_POINTS per pair.  `matched` is the contact ID
 * link: the slot of the previous step's point whose warm state this point
 * inherited, or -1 for a fresh point. */
#define AVBD_MAX_POINTS 8
typedef struct AvbdPointState {
    float ra[3];
    float rb[3];
    float lam[3];
    float pen[3];
    float roll_lam[3];
    uint32_t stuck;
    int32_t matched;
} AvbdPointState;

/* Joint dual state (AvbdJoint, avbd/mod.rs:327-402). */
typedef struct AvbdJointState {
    float lam_l[3];
    float lam_a[3];
    float pen_l[3];
    float pen_a[3];
    float acc_lim;   /* revolute limit accumulator */
    float lim_dual;  /* prismatic limit force */
    float sacc[6];   /* sixdof limited-axis forces: linear x y z, angular x y z */
    /* gear: the coupled joints' coordinates at the last step start (raw and
     * unwrapped across turns, gear_mem in avbd/mod.rs:377-383); gear_mem_set
     * 0 until the gear's first step */
    float gear_raw[2];
    float gear_cont[2];
    uint32_t gear_mem_set;
} AvbdJointState;

/* Per-step observability counters (the reference exposes sleeping_count(),
 * avbd/mod.rs:788-790; the rest are new). */
typedef struct AvbdCounters {
    uint64_t steps;        /* fixed substeps taken                            */
    uint64_t pairs;        /* live contact pairs after the last substep       */
    uint64_t points;       /* live contact points                             */
    uint64_t candidates;   /* broadphase candidate pairs (last substep)       */
    uint64_t colours;      /* colours used by the last substep (max over scenes) */
    uint64_t breakdowns;   /* LDL^T breakdowns (body skipped its update), cumulative */
    uint64_t ccd_hits;     /* TOI clamps, cumulative                          */
    uint64_t sleeping;     /* bodies asleep after the last substep            */
    uint64_t timeouts;     /* bounded device waits that gave up, cumulative   */
} AvbdCounters;

/* Contact transition of a body pair (ContactEvent / ContactEventKind,
 * crates/physics/src/trigger.rs; emitted by avbd/mod.rs:1606-1669 and the
 * CCD hit pass mod.rs:935-960, :1126-1136).  body_a < body_b.  Begin / End:
 * the pair's deepest point crossed CONTACT_BEGIN_SLOP (5 mm) between two
 * emitting substeps.  Hit: a pair that began touching, or a swept body's
 * time-of-impact clamp, with a closing speed above CONTACT_HIT_THRESHOLD
 * (1 m/s); point, normal (A toward B) and approach_speed are set for hits. */
#define AVBD_CONTACT_BEGIN 0
#define AVBD_CONTACT_END 1
#define AVBD_CONTACT_HIT 2
typedef struct AvbdContactEvent {
    uint32_t body_a;
    uint32_t body_b;
    uint32_t kind;
    float point[3];
    float normal[3];
    float approach_speed;
} AvbdContactEvent;

/* Trigger overlap transition (TriggerEvent, trigger.rs:20-36). */
typedef struct AvbdTriggerEvent {
    uint32_t body_a;
    uint32_t body_b;
    uint32_t entered; /* 1 = Entered, 0 = Exited */
} AvbdTriggerEvent;

typedef struct AvbdWorld AvbdWorld;

/* ---- world lifecycle ----------------------------------------------------- */

/* Fill `p` with the reference's defaults: gravity (0,-9.81,0), 1/60 s,
 * 10 iterations, 4 max substeps, sleep and CCD on. */
int avbd_default_params(AvbdParams* p);

/* AvbdEngine::new (avbd/mod.rs:1147).  `device` is the CUDA ordinal. */
int avbd_world_create(const AvbdParams* params, int device, AvbdWorld** out);

/* Build a multi-scene world in one call: bodies[0..n) with scene s owning
 * [scene_offsets[s], scene_offsets[s+1]), scene_offsets has nscenes+1
 * entries, scene_offsets[0] == 0, scene_offsets[nscenes] == n. */
int avbd_world_create_batch(const AvbdParams* params, int device,
                            const AvbdBody* bodies, uint32_t n,
                            const uint32_t* scene_offsets, uint32_t nscenes,
                            AvbdWorld** out);

int avbd_world_destroy(AvbdWorld* world);

/* PhysicsEngine::add_body (avbd/mod.rs:1236-1239): appends to the last
 * scene; the first new handle is written to *first_handle. */
int avbd_world_add_bodies(AvbdWorld* world, const AvbdBody* bodies, uint32_t n,
                          uint32_t* first_handle);

/* Register a convex hull (ConvexHull, collision/shape.rs:317-365) that
 * bodies of shape AVBD_SHAPE_HULL name by index in shape_params[0]: the
 * reference hull's centroid-relative vertices (3 floats each, support scans
 * them in this order), its triangle faces (3 vertex indices each, used to
 * re-seat contact witnesses; may be empty) and its body-frame inertia per
 * unit mass (ConvexHull::try_inertia(1)), used when a sleeping body wakes.
 * The hull's bodies carry their own mass and inertia in their records. */
int avbd_world_add_hull(AvbdWorld* world, const float* verts, uint32_t nverts, const uint32_t* faces,
                        uint32_t nfaces, const float* unit_inertia, uint32_t* hull_id);

/* Shape::try_round (collision/shape.rs:563-575): `inner` is a primitive part
 * (sphere, box, capsule, cylinder, cone or a hull already added) and its
 * border_radius the skin, finite and > 0 (AVBD_ERR_INVALID_ARG otherwise; a
 * half-space or a nested rounded or compound inner -> AVBD_ERR_UNSUPPORTED).
 * Bodies of shape AVBD_SHAPE_ROUND name the returned id in shape_params[0].
 * unit_inertia is the body-frame inertia per unit mass (Shape::try_inertia
 * (1)), used when a sleeping body wakes; bodies carry their own in their
 * records.  Distances peel the skin (distance.rs:519-545, :654-685). */
int avbd_world_add_round(AvbdWorld* world, const AvbdShapePart* inner, const float* unit_inertia, uint32_t* id);

/* Shape::try_compound (shape.rs:556-561): n >= 1 primitive parts, each
 * optionally rounded (border_radius > 0) and placed by its pose; an empty
 * list or a non-finite or negative radius -> AVBD_ERR_INVALID_ARG, a
 * half-space or nested compound part -> AVBD_ERR_UNSUPPORTED.  Distances
 * take the deepest part in order (distance.rs:550-599); compound against
 * compound is separation, as in the reference.  Bodies of shape
 * AVBD_SHAPE_COMPOUND name the id in shape_params[0]. */
int avbd_world_add_compound(AvbdWorld* world, const AvbdShapePart* parts, uint32_t n, const float* unit_inertia,
                            uint32_t* id);

/* Heightfield::new (collision/shape.rs:1485-1505, invariants.rs:403-425):
 * rows x cols row-major heights (rows along +Z, cols along +X) on a grid of
 * spacing `cell`, centred on the body; an empty grid, a non-positive or
 * non-finite cell -> AVBD_ERR_INVALID_ARG, a non-finite height ->
 * AVBD_ERR_NONFINITE.  Distances take the nearest overlapped column, each a
 * solid box from the lowest sample up (distance.rs:246-350); terrain
 * against terrain, and terrain against a triangle mesh, are separation.
 * Bodies of shape AVBD_SHAPE_HEIGHTFIELD name the id in shape_params[0]. */
int avbd_world_add_heightfield(AvbdWorld* world, uint32_t rows, uint32_t cols, float cell, const float* heights,
                               uint32_t* id);

/* TriMesh::from_indexed (shape.rs:1646-1772): vertices (3 floats each) and
 * triangles (3 indices each); degenerate triangles are dropped, an index out
 * of range -> AVBD_ERR_INVALID_ARG, a non-finite vertex ->
 * AVBD_ERR_NONFINITE.  Each kept triangle becomes a centroid-relative hull
 * under a median-split AABB tree built as the reference builds it
 * (shape.rs:1793-1890); distances take the nearest triangle the tree
 * overlaps (distance.rs:416-517).  Mesh against mesh is separation.  Bodies
 * of shape AVBD_SHAPE_TRIMESH name the id in shape_params[0]. */
int avbd_world_add_trimesh(AvbdWorld* world, const float* verts, uint32_t nverts, const uint32_t* tris,
                           uint32_t ntris, uint32_t* id);

/* PhysicsEngine::remove_body (engine.rs:40-43, avbd/mod.rs:1241-1300): the
 * last body moves into the freed handle; pairs and joints of the removed
 * body are dropped (with the gears that couple those joints), the others
 * renumbered; trigger pairs of the removed body
 * report Exited, touches and queued contact events are cleared, every
 * sleeping body wakes.  A pair whose two handles change order under the
 * renumbering is dropped at once: the reference keeps it until its next
 * discovery drops it (it never matches again), so stepping is the same, but
 * an export taken right after the removal lacks it.  An invalid handle is a
 * no-op.  One-scene worlds only (AVBD_ERR_UNSUPPORTED for a batch). */
int avbd_world_remove_body(AvbdWorld* world, uint32_t handle);

/* PhysicsEngine::add_joint (avbd/mod.rs:1310-1529) with the admission
 * checks of validate_joint (migration.rs:160-330): non-finite anchors or
 * axes -> AVBD_ERR_JOINT_BAD_AXIS, inverted or non-finite limits and a rope
 * length <= 0 -> AVBD_ERR_JOINT_BAD_BOUNDS, non-finite motor fields ->
 * AVBD_ERR_JOINT_NONFINITE, then both bodies wake, then self / invalid
 * handles; a degenerate hinge or slide axis -> AVBD_ERR_JOINT_BAD_AXIS.
 * A free motor: non-finite targets or budgets, or a negative budget ->
 * AVBD_ERR_JOINT_NONFINITE, a correction outside [0, 1] ->
 * AVBD_ERR_JOINT_BAD_BOUNDS (its anchors are not used).  A spring's motor
 * (validate_motor, migration.rs:366-394): non-finite targets, a negative or
 * non-finite stiffness, damping or budget -> AVBD_ERR_JOINT_NONFINITE.
 * A wheel: non-finite suspension or axle axes -> AVBD_ERR_JOINT_BAD_AXIS, a
 * negative or non-finite frequency or damping ratio ->
 * AVBD_ERR_JOINT_NONFINITE, a degenerate suspension axis ->
 * AVBD_ERR_JOINT_BAD_AXIS.  A gear (mod.rs:1329-1404): a non-finite ratio ->
 * AVBD_ERR_JOINT_NONFINITE, then both bodies wake, then self / invalid
 * handles, then a coupled joint that does not exist ->
 * AVBD_ERR_JOINT_UNKNOWN_REF, one that is neither revolute nor prismatic ->
 * AVBD_ERR_UNSUPPORTED.
 * Kinds: Ball, Revolute (limit, velocity motor), Prismatic (limit, velocity
 * motor), Fixed, Distance, Rope, SixDof, Motor (free velocity drive),
 * Spring, Wheel (velocity motor about the axle), Gear. */
int avbd_world_add_joint(AvbdWorld* world, const AvbdJointDesc* desc, uint32_t* handle);

/* PhysicsEngine::remove_joint (engine.rs, avbd/mod.rs:1531-1540): both
 * bodies of the joint wake, the joint and its warm state go, gears that
 * couple it go too, and the handles of later joints move down (the
 * reference's retain_joints, mod.rs:766-784, joint_remap migration.rs:74-115).
 * An invalid handle is a no-op. */
int avbd_world_remove_joint(AvbdWorld* world, uint32_t handle);

/* PhysicsEngine::wake_body (engine.rs:109, avbd/mod.rs:1599-1601): a sleeping
 * body wakes with its mass and inertia restored and its sleep timer reset
 * (mod.rs:833-842, body.rs:412-418); awake bodies and invalid handles are
 * untouched. */
int avbd_world_wake_body(AvbdWorld* world, uint32_t handle);

int avbd_world_body_count(const AvbdWorld* world, uint32_t* n);
int avbd_world_scene_count(const AvbdWorld* world, uint32_t* n);

/* PhysicsEngine::get_body / get_body_mut (engine.rs:45-48) for a range of
 * handles: host copies of the device body records.  Edits written back by
 * avbd_world_set_bodies apply at the next step. */
int avbd_world_get_bodies(AvbdWorld* world, uint32_t first, uint32_t n, AvbdBody* out);
int avbd_world_set_bodies(AvbdWorld* world, uint32_t first, uint32_t n, const AvbdBody* in);

/* PhysicsEngine::step (avbd/mod.rs:1212-1235): fixed-step accumulator,
 * at most max_substeps substeps of step_dt per call. */
int avbd_world_step(AvbdWorld* world, float dt);

/* Advance exactly `substeps` fixed substeps of step_dt (no accumulator). */
int avbd_world_step_fixed(AvbdWorld* world, int32_t substeps);

/* Same as avbd_world_step_fixed, replayed through a captured CUDA graph of
 * one substep (captured on first use, re-captured when capacities change). */
int avbd_world_step_graph(AvbdWorld* world, int32_t substeps);

/* Block until the world's stream is idle. */
int avbd_world_sync(AvbdWorld* world);

int avbd_world_get_counters(AvbdWorld* world, AvbdCounters* out);

/* ---- state exchange: checkpoint / restore and parity ---------------------- */

/* Sizes of the exported state: bodies, pairs, joints. */
int avbd_world_state_sizes(AvbdWorld* world, uint32_t* nbodies, uint32_t* npairs,
                           uint32_t* njoints);

/* Copy the whole solver state to host arrays (points: AVBD_MAX_POINTS slots
 * per pair).  Any pointer may be NULL to skip that part. */
int avbd_world_export_state(AvbdWorld* world, AvbdBody* bodies, AvbdBodyAux* aux,
                            AvbdPairState* pairs, AvbdPointState* points,
                            AvbdJointState* joints, uint32_t pair_capacity);

/* Replace the whole solver state (body count and joints must match). */
int avbd_world_import_state(AvbdWorld* world, const AvbdBody* bodies,
                            const AvbdBodyAux* aux, const AvbdPairState* pairs,
                            const AvbdPointState* points, uint32_t npairs,
                            const AvbdJointState* joints);

/* ---- on-disk snapshot ------------------------------------------------------
 * A versioned, bit-faithful capture of a whole world: parameters, scene
 * offsets, bodies with their solver state (previous poses, sleep timers),
 * contact pairs and points with their warm state, joints with their
 * assembly references and warm state, convex hulls, the world's settings
 * (launch tuning, precision, event period, joint stiffness, the fixed-step
 * accumulator's remainder), rounded and compound shapes, and the event
 * state: the previous touch set, the
 * previous trigger overlap set, the drop counters and the undrained event
 * queues.  A world made from a snapshot continues bit for bit as the saved
 * world would have (the reference's WorldSnapshot makes the same promise
 * for the sequential-impulse engine and refuses AVBD, snapshot.rs:1-60,
 * :815-830; this closes that gap).
 *
 * Layout: a 128-byte header (magic "ORNAVBD\0", format version, the
 * writer's ABI version, an endianness mark, the size of every record the
 * payload holds, the counts, the total size and a 64-bit FNV-1a checksum of
 * the payload) followed by the payload sections in a fixed order.  A reader
 * refuses, with AVBD_ERR_FORMAT, any other format version, record size or
 * endianness, a truncated or oversized buffer and a checksum mismatch —
 * never a silent reinterpretation (the reference's VersionMismatch,
 * snapshot.rs:815-830).  Queued events beyond the loaded world's queue
 * capacity are refused the same way. */
#define AVBD_SNAPSHOT_FORMAT 2

typedef struct AvbdSnapshotInfo {
    uint32_t format;          /* format version of the snapshot              */
    uint32_t abi;             /* avbd_abi_version() of the writer            */
    uint32_t nbodies, nscenes, npairs, njoints, nhulls;
    uint32_t ntouch;          /* previous touch set: touching pairs          */
    uint32_t ntrigger;        /* previous trigger overlap set                */
    uint32_t ncontact_events; /* undrained contact events                    */
    uint32_t ntrigger_events; /* undrained trigger events                    */
    uint32_t reserved;
    uint64_t bytes;           /* the whole snapshot, header included         */
    uint64_t substeps;        /* substeps the saved world had taken          */
} AvbdSnapshotInfo;

/* Write the world's snapshot into buf.  *size receives the snapshot's size;
 * buf may be NULL to ask for it (then nothing is written).  A non-NULL buf
 * with cap < *size -> AVBD_ERR_CAPACITY, nothing written. */
int avbd_world_snapshot(AvbdWorld* world, void* buf, uint64_t cap, uint64_t* size);

/* A new world on `device` from a snapshot (the caller destroys it). */
int avbd_world_from_snapshot(const void* buf, uint64_t size, int device, AvbdWorld** out);

/* Validate a snapshot as a load would on the host (header, checksum and
 * contents) and describe it; needs no GPU. */
int avbd_snapshot_info(const void* buf, uint64_t size, AvbdSnapshotInfo* info);

/* The same to and from a file (written whole, then renamed into place). */
int avbd_world_save(AvbdWorld* world, const char* path);
int avbd_world_load(const char* path, int device, AvbdWorld** out);

/* Colour of every body in the last substep's primal sweep (-1 = not swept:
 * static, kinematic, asleep). */
int avbd_world_get_colours(AvbdWorld* world, int32_t* colours, uint32_t n);

/* ---- helpers -------------------------------------------------------------- */

/* RigidBody::new_sphere / new_box / new_capsule / try_new_halfspace
 * (body.rs:346-376, :470-576, :873-889): fills one body record with the
 * reference's default material for the shape and the mass triple of
 * Mass::from_kind (invariants.rs:175-199).  mass <= 0 makes a static body;
 * a half-space must be static. */
int avbd_body_init(AvbdBody* out, uint32_t shape, const float* params, const float* position, float mass);

/* Launch shape of the primal kernel: lanes cooperating on one body (1, 4, 8,
 * 16 or 32) and threads per block; 0 = the split launch (per colour, one
 * thread per (pair, side) for the rows, then one per body for the sums and
 * the solve); AVBD_PRIMAL_SCENES = the per-scene solve (one block takes a
 * scene through every iteration of a substep — all colours' primal and the
 * dual — in one launch per substep; block 128, 256 or 512; the split
 * arithmetic; a world with a scene above 2048 bodies runs the split launches
 * instead).  No reference counterpart (the reference sweeps on one CPU
 * thread); picked by the autotuner in ornis_gb300/tune.py. */
#define AVBD_PRIMAL_SCENES (-1)
int avbd_set_tuning(AvbdWorld* world, int primal_lanes, int primal_block);

/* Arithmetic of the iteration kernels: 0 (default) = exact build, the same
 * f32 operation order as the reference (no contraction, IEEE divide and
 * square root, correctly rounded sin / cos / asin / atan2): from identical
 * state it reproduces the CPU restatement bit for bit; 1 = fast build
 * (contracted multiply-adds, approximate divide and square root), a few
 * percent faster but not bit-faithful: the stiff contact and joint rows
 * amplify its last-bit differences to 1e-5 .. 3e-4 per step in settled piles
 * and ragdolls.  Discovery (pair sets, contact IDs, colours) is exact in
 * both. */
int avbd_set_precision(AvbdWorld* world, int fast);

/* Register budget of the one-thread-per-body primal: built for 4, 6 or 8
 * resident 128-thread blocks per SM.  Picked by the autotuner. */
int avbd_set_occupancy(AvbdWorld* world, int min_blocks);

/* Start (on != 0) or stop profiler collection (cudaProfilerStart/Stop). */
int avbd_profiler(int on);

/* Order of the bodies inside each colour's launch: 0 = ascending handle,
 * 1 = by incident-pair count (less warp divergence).  Results do not depend
 * on it: bodies of one colour are independent. */
int avbd_set_work_order(AvbdWorld* world, int by_work);

/* Scenes of at most `small_scene_max` bodies (0..2048, default 2048) are
 * swept by one CTA each; larger ones by the device-wide radix sort and
 * sweep.  Both give the same candidate set.  No reference counterpart. */
int avbd_set_broadphase(AvbdWorld* world, int small_scene_max);

/* How the device-wide path sweeps a large scene: rows = 1 (default) cuts
 * space into cells at least as wide as the scene's widest box, sorts the
 * bodies by the Morton code of their (y, z) cell row and then by min x, and
 * sweeps each body's row and the four forward neighbouring rows; rows = 0
 * sorts by min x alone and sweeps once.  Both give the same candidate set.
 * No reference counterpart. */
int avbd_set_sweep(AvbdWorld* world, int rows);

int avbd_abi_version(void);

/* ---- measurement (no reference counterpart: the reference publishes no
 * timing for this path) ---------------------------------------------------- */

/* Advance `substeps` fixed substeps (CUDA-graph replay when use_graph != 0)
 * and return their device time in *ms, from CUDA events recorded on the
 * world's stream before the first and after the last substep. */
int avbd_world_step_timed(AvbdWorld* world, int32_t substeps, int32_t use_graph, float* ms);

/* Evict the world's state from the L2 cache: write a 256 MB scratch array
 * (twice the GB300's L2, allocated on the first call, freed with the world)
 * on the world's stream and wait for it.  For timing a state smaller than
 * L2 without carrying it over in cache between timed steps. */
int avbd_world_flush_cache(AvbdWorld* world);

/* Advance one substep through plain launches with a CUDA event between the
 * phases.  ms[9]: wake+torque, broadphase, CCD, discovery, post-discovery,
 * colouring, primal (all colours and iterations), dual (all iterations),
 * BDF1+sleep.  info[5]: colours, primal launches, bodies swept per
 * iteration, pairs, points. */
int avbd_world_profile_substep(AvbdWorld* world, float* ms, uint32_t* info);

/* Kernel nodes in one captured substep graph (0 before the first capture). */
int avbd_world_graph_nodes(AvbdWorld* world, uint32_t* n);
/* ... and in the captured substep that also reports events. */
int avbd_world_graph_nodes_emit(AvbdWorld* world, uint32_t* n);

/* ---- events (PhysicsEngine::drain_contact_events / drain_trigger_events,
 * engine.rs; emitted by avbd/mod.rs:1606-1669 and :1126-1136) ------------- */

/* Which substeps report events.  As in the reference, avbd_world_step
 * reports on the last substep of each call.  For fixed-step calls
 * (avbd_world_step_fixed / _graph / _timed): period 0 (default) = the last
 * substep of each call, k > 0 = every k-th substep of a call, -1 = no
 * events at all (not even swept hits). */
int avbd_set_events(AvbdWorld* world, int32_t period);

/* Move every queued contact / trigger event into `out` (room for `cap`) and
 * set *n to how many.  If more than `cap` are queued nothing is moved,
 * *n = the number queued and AVBD_ERR_CAPACITY is returned.  Within one
 * substep Begin / End come first, then hits of new touches, then swept
 * hits; Begin / End and hits are ordered by (body_b, body_a) — the
 * reference's set of events, in the reference's kinds-then-keys grouping
 * but keyed on the higher handle first. */
int avbd_world_drain_contact_events(AvbdWorld* world, AvbdContactEvent* out, uint32_t cap, uint32_t* n);
int avbd_world_drain_trigger_events(AvbdWorld* world, AvbdTriggerEvent* out, uint32_t cap, uint32_t* n);

/* counts[4]: contact events queued, trigger events queued, contact events
 * dropped because the queue was full, trigger events dropped (cumulative). */
int avbd_world_event_counts(AvbdWorld* world, uint32_t* counts);

/* Finite joint stiffness k (N/m for the anchor rows, N m/rad for the hinge
 * alignment rows; 0, the default, keeps the reference's hard joints,
 * mod.rs:176-181).  With k > 0 those rows are springs of stiffness k
 * (penalty k, lambda zero: the AVBD treatment of a finite-stiffness
 * constraint); the hinge limit row stays hard.  No counterpart in the reference: the
 * articulated workload's gradient is taken with respect to k. */
int avbd_set_joint_stiffness(AvbdWorld* world, float k);

/* ---- allocation-free stepping (no counterpart in the reference) ----------- */

#define AVBD_STATIC_MAX_BODIES 128u      /* bodies per call */
#define AVBD_STATIC_PAIR_CAP 2048u       /* broadphase candidates per substep */
#define AVBD_STATIC_SCRATCH_BYTES 3481600u /* device array every GPU that loads the library holds */

/* Step one scene of at most AVBD_STATIC_MAX_BODIES bodies (no joints) for
 * `substeps` fixed substeps of params->step_dt, from host records `bodies`
 * to host records `out` (out may equal bodies), without allocating: for
 * callers that cannot call cudaMalloc (an engine that owns every device
 * allocation through its own pools, a process whose device memory is capped
 * or fully reserved).  All device scratch is one file-scope device array of
 * AVBD_STATIC_SCRATCH_BYTES on the caller's current device; its address is
 * looked up on every call.  The first call on a device loads the library's
 * device code and with it the array (CUDA's lazy module loading): make that
 * first call before any stream capture and before the caller reserves or
 * caps device memory, or run with CUDA_MODULE_LOADING=EAGER.  Later calls
 * allocate nothing.  The results equal an AvbdWorld created from the same
 * bodies and advanced by avbd_world_step_fixed(substeps).  Each call starts
 * fresh: no contact warm start carries over from an earlier call.  Calls
 * share the array, so calls that overlap on the GPU (two host threads, two
 * streams) race.  Returns AVBD_ERR_CAPACITY for more than
 * AVBD_STATIC_MAX_BODIES bodies, when a substep finds more than
 * AVBD_STATIC_PAIR_CAP candidates, or when a substep needs more than 64
 * colours; out is then not written.  AVBD_ERR_NONFINITE for a non-finite
 * body. */
int avbd_scene_step_static(const AvbdParams* params, const AvbdBody* bodies, uint32_t n, int32_t substeps,
                           AvbdBody* out);

/* ---- differentiable rollouts (no counterpart in the reference: its AVBD
 * engine has no adjoint; the interface shape follows the forward/backward
 * pair the Rust side wraps as one Function-style type) ------------------- */

/* Advance the world `steps` steps of `substeps` fixed substeps (as
 * avbd_world_step_graph) and keep a device checkpoint of the full step
 * state every `checkpoint_every` steps, for avbd_adjoint_backward.  Worlds
 * with rolling / torsion friction, motors, or joints other than Ball and
 * Revolute return AVBD_ERR_UNSUPPORTED.  The rollout runs the split primal launch
 * (avbd_set_tuning lanes 0) and orders every body's contact pairs (the
 * static bodies' too), which the world keeps afterwards; retuning the
 * world before the backward invalidates the recording.  A new forward
 * replaces the previous recording and, on the same world, keeps its frame
 * storage and recording graphs. */
int avbd_adjoint_forward(AvbdWorld* world, int32_t steps, int32_t substeps, int32_t checkpoint_every);

/* Reverse-mode gradient of a scalar loss of the recorded rollout's final
 * state.  grad_final: dLoss/d(final state), 13 floats per body (position 3,
 * orientation x y z w, velocity 3, angular velocity 3).  Writes
 * grad_initial (the same layout, dLoss/d(initial state)) and, when not
 * null, grad_friction: one float per scene, dLoss/d(mu) for a friction
 * coefficient mu that every body of the scene shares (pair friction is the
 * larger of the two bodies', so it moves with mu).  The contact set, the
 * contact frames (normal, friction basis, local anchors; a capsule's
 * witness anchor rolls with the body) and the colouring are held at the
 * values of the recorded rollout, and so are a swept impact's time of
 * impact, normal and bounce, and a hinge's twist angle once its axes part
 * by more than 120 degrees; the step-start gap stays a function of the
 * step-start poses.  Joint rows are differentiated (see
 * avbd_adjoint_grad_joint_stiffness).  Each segment between checkpoints is
 * recomputed from its checkpoint.  The world is left at the end of the
 * recorded rollout. */
int avbd_adjoint_backward(AvbdWorld* world, const float* grad_final, float* grad_initial, float* grad_friction);

/* dLoss/d(joint stiffness) of the last avbd_adjoint_backward, one float per
 * scene (the contributions of the scene's joints; their sum is the gradient
 * for the world's one stiffness, avbd_set_joint_stiffness).  Zero for hard
 * joints (stiffness 0). */
int avbd_adjoint_grad_joint_stiffness(AvbdWorld* world, float* per_scene);

/* Device time of the last avbd_adjoint_backward: ms[0] the segment
 * recomputes (restores included), ms[1] the reverse sweeps. */
int avbd_adjoint_timing(AvbdWorld* world, float* ms);

/* Magnitude of the adjoint along the last avbd_adjoint_backward: for each
 * substep s of the rollout (in forward order, steps x substeps of them), the
 * largest |component| of the body adjoints (position, orientation, velocity,
 * angular velocity) of the state at the start of substep s, and the first
 * body holding it; a non-finite adjoint reads as infinity.  Fills up to cap
 * entries and sets *n to the substep count.  A diagnostic for gradients that
 * grow without bound along a trajectory. */
int avbd_adjoint_trace(AvbdWorld* world, float* max_abs, uint32_t* body, int32_t cap, int32_t* n);

#ifdef __cplusplus
}
#endif
#endif /* ORNIS_AVBD_H */
