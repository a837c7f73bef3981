//! Raw declarations of `include/ornis_avbd.h`: `#[repr(C)]` mirrors of its
//! records (same field order and sizes; `AvbdBody` is 136 bytes,
//! `AvbdJointDesc` 272, `AvbdJointState` 100) and its
//! `extern "C"` entry points.  Every function returns an `i32` status: 0 or a
//! negative `AVBD_ERR_*` code.

#![allow(non_camel_case_types)]

pub const AVBD_OK: i32 = 0;
pub const AVBD_ERR_INVALID_ARG: i32 = -1;
pub const AVBD_ERR_CAPACITY: i32 = -2;
pub const AVBD_ERR_DEVICE: i32 = -3;
pub const AVBD_ERR_TIMEOUT: i32 = -4;
pub const AVBD_ERR_NONFINITE: i32 = -5;
pub const AVBD_ERR_UNSUPPORTED: i32 = -6;
pub const AVBD_ERR_FORMAT: i32 = -7;
pub const AVBD_ERR_IO: i32 = -8;
pub const AVBD_SNAPSHOT_FORMAT: u32 = 2;
pub const AVBD_STATIC_MAX_BODIES: u32 = 128;
pub const AVBD_STATIC_PAIR_CAP: u32 = 2048;
pub const AVBD_STATIC_SCRATCH_BYTES: u32 = 3481600;
pub const AVBD_ERR_JOINT_SELF: i32 = -10;
pub const AVBD_ERR_JOINT_HANDLES: i32 = -11;
pub const AVBD_ERR_JOINT_BAD_AXIS: i32 = -12;
pub const AVBD_ERR_JOINT_NONFINITE: i32 = -13;
pub const AVBD_ERR_JOINT_BAD_BOUNDS: i32 = -14;
pub const AVBD_ERR_JOINT_UNKNOWN_REF: i32 = -15;

pub const AVBD_SHAPE_SPHERE: u32 = 0;
pub const AVBD_SHAPE_BOX: u32 = 1;
pub const AVBD_SHAPE_CAPSULE: u32 = 2;
pub const AVBD_SHAPE_HALFSPACE: u32 = 3;
pub const AVBD_SHAPE_CYLINDER: u32 = 4;
pub const AVBD_SHAPE_CONE: u32 = 5;
pub const AVBD_SHAPE_HULL: u32 = 6;
pub const AVBD_SHAPE_ROUND: u32 = 7;
pub const AVBD_SHAPE_COMPOUND: u32 = 8;
pub const AVBD_SHAPE_HEIGHTFIELD: u32 = 9;
pub const AVBD_SHAPE_TRIMESH: u32 = 10;

pub const AVBD_BODY_DYNAMIC: u32 = 0;
pub const AVBD_BODY_STATIC: u32 = 1;
pub const AVBD_BODY_KINEMATIC: u32 = 2;
pub const AVBD_FLAG_TRIGGER: u32 = 1;

pub const AVBD_JOINT_BALL: u32 = 0;
pub const AVBD_JOINT_REVOLUTE: u32 = 1;
pub const AVBD_JOINT_PRISMATIC: u32 = 2;
pub const AVBD_JOINT_FIXED: u32 = 3;
pub const AVBD_JOINT_DISTANCE: u32 = 4;
pub const AVBD_JOINT_ROPE: u32 = 5;
pub const AVBD_JOINT_SIXDOF: u32 = 6;
pub const AVBD_JOINT_MOTOR: u32 = 7;
pub const AVBD_JOINT_SPRING: u32 = 8;
pub const AVBD_JOINT_WHEEL: u32 = 9;
pub const AVBD_JOINT_GEAR: u32 = 10;
pub const AVBD_MOTOR_VELOCITY: u32 = 0;
pub const AVBD_MOTOR_POSITION: u32 = 1;
pub const AVBD_MOTOR_SERVO: u32 = 2;
pub const AVBD_MODEL_ACCELERATION: u32 = 0;
pub const AVBD_MODEL_FORCE: u32 = 1;

pub const AVBD_AXIS_FREE: u32 = 0;
pub const AVBD_AXIS_LOCKED: u32 = 1;
pub const AVBD_AXIS_LIMITED: u32 = 2;
pub const AVBD_ABI_VERSION: i32 = 4;

pub const AVBD_MAX_POINTS: usize = 8;
pub const AVBD_PRIMAL_SCENES: i32 = -1;

pub const AVBD_CONTACT_BEGIN: u32 = 0;
pub const AVBD_CONTACT_END: u32 = 1;
pub const AVBD_CONTACT_HIT: u32 = 2;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct AvbdBody {
    pub position: [f32; 3],
    pub orientation: [f32; 4], // x y z w
    pub velocity: [f32; 3],
    pub angular_velocity: [f32; 3],
    pub torque: [f32; 3],
    pub mass: f32,
    pub inv_mass: f32,
    pub inertia: [f32; 3],
    pub restitution: f32,
    pub friction: f32,
    pub friction_transverse: f32,
    pub rolling_friction: f32,
    pub torsion_friction: f32,
    pub shape: u32,
    pub shape_params: [f32; 3],
    pub collision_layer: u32,
    pub collision_mask: u32,
    pub body_type: u32,
    pub flags: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdJointDesc {
    pub kind: u32,
    pub body_a: u32,
    pub body_b: u32,
    pub local_anchor_a: [f32; 3],
    pub local_anchor_b: [f32; 3],
    pub local_axis_a: [f32; 3],
    pub local_axis_b: [f32; 3],
    pub has_limit: i32,
    pub limit_min: f32,
    pub limit_max: f32,
    pub has_motor: i32,
    pub motor_speed: f32,
    pub motor_max: f32,
    pub max_distance: f32,
    pub axis_config: [u32; 6],
    pub axis_min: [f32; 6],
    pub axis_max: [f32; 6],
    /// free motor (`JointKind::Motor`): B-minus-A velocity targets, budgets, assembly pull
    pub motor_linear: [f32; 3],
    pub motor_angular: [f32; 3],
    pub motor_max_force: f32,
    pub motor_max_torque: f32,
    pub motor_correction: f32,
    /// spring (`JointKind::Spring`): its `JointMotor`
    pub spring_rest: f32,
    pub spring_velocity: f32,
    pub spring_stiffness: f32,
    pub spring_damping: f32,
    pub spring_max_force: f32,
    pub spring_kind: u32,
    pub spring_model: u32,
    /// wheel (`JointKind::Wheel`): spin axles and the suspension
    pub local_axle_a: [f32; 3],
    pub local_axle_b: [f32; 3],
    pub suspension_hz: f32,
    pub suspension_damping: f32,
    /// gear (`JointKind::Gear`): the coupled joints and the ratio
    pub gear_joint_a: u32,
    pub gear_joint_b: u32,
    pub gear_ratio: f32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdParams {
    pub gravity: [f32; 3],
    pub step_dt: f32,
    pub iterations: i32,
    pub max_substeps: i32,
    pub enable_sleep: i32,
    pub enable_ccd: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdBodyAux {
    pub prev_position: [f32; 3],
    pub prev_orientation: [f32; 4],
    pub sleep_timer: f32,
    pub asleep: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdPairState {
    pub a: u32,
    pub b: u32,
    pub normal: [f32; 3],
    pub mu: [f32; 2],
    pub gap: f32,
    pub npoints: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdPointState {
    pub ra: [f32; 3],
    pub rb: [f32; 3],
    pub lam: [f32; 3],
    pub pen: [f32; 3],
    pub roll_lam: [f32; 3],
    pub stuck: u32,
    pub matched: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdJointState {
    pub lam_l: [f32; 3],
    pub lam_a: [f32; 3],
    pub pen_l: [f32; 3],
    pub pen_a: [f32; 3],
    pub acc_lim: f32,
    pub lim_dual: f32,
    pub sacc: [f32; 6],
    /// gear: the coupled joints' coordinates at the last step start
    pub gear_raw: [f32; 2],
    pub gear_cont: [f32; 2],
    pub gear_mem_set: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdCounters {
    pub steps: u64,
    pub pairs: u64,
    pub points: u64,
    pub candidates: u64,
    pub colours: u64,
    pub breakdowns: u64,
    pub ccd_hits: u64,
    pub sleeping: u64,
    pub timeouts: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdContactEvent {
    pub body_a: u32,
    pub body_b: u32,
    pub kind: u32,
    pub point: [f32; 3],
    pub normal: [f32; 3],
    pub approach_speed: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdTriggerEvent {
    pub body_a: u32,
    pub body_b: u32,
    pub entered: u32,
}

/// A part of a rounded or compound shape (`Shape::Round`'s inner, a
/// compound child and its `Pose`).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdShapePart {
    pub shape: u32,
    pub params: [f32; 3],
    pub border_radius: f32,
    pub position: [f32; 3],
    pub orientation: [f32; 4],
}

/// What `avbd_snapshot_info` reports about a snapshot.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct AvbdSnapshotInfo {
    pub format: u32,
    pub abi: u32,
    pub nbodies: u32,
    pub nscenes: u32,
    pub npairs: u32,
    pub njoints: u32,
    pub nhulls: u32,
    pub ntouch: u32,
    pub ntrigger: u32,
    pub ncontact_events: u32,
    pub ntrigger_events: u32,
    pub reserved: u32,
    pub bytes: u64,
    pub substeps: u64,
}

/// Opaque world handle.
#[repr(C)]
pub struct AvbdWorld {
    _private: [u8; 0],
}

extern "C" {
    pub fn avbd_abi_version() -> i32;
    pub fn avbd_default_params(p: *mut AvbdParams) -> i32;
    pub fn avbd_world_create(params: *const AvbdParams, device: i32, out: *mut *mut AvbdWorld) -> i32;
    pub fn avbd_world_create_batch(
        params: *const AvbdParams,
        device: i32,
        bodies: *const AvbdBody,
        n: u32,
        scene_offsets: *const u32,
        nscenes: u32,
        out: *mut *mut AvbdWorld,
    ) -> i32;
    pub fn avbd_world_destroy(world: *mut AvbdWorld) -> i32;
    pub fn avbd_world_add_bodies(world: *mut AvbdWorld, bodies: *const AvbdBody, n: u32, first: *mut u32) -> i32;
    pub fn avbd_world_add_hull(
        world: *mut AvbdWorld,
        verts: *const f32,
        nverts: u32,
        faces: *const u32,
        nfaces: u32,
        unit_inertia: *const f32,
        hull_id: *mut u32,
    ) -> i32;
    pub fn avbd_world_add_round(
        world: *mut AvbdWorld,
        inner: *const AvbdShapePart,
        unit_inertia: *const f32,
        id: *mut u32,
    ) -> i32;
    pub fn avbd_world_add_compound(
        world: *mut AvbdWorld,
        parts: *const AvbdShapePart,
        n: u32,
        unit_inertia: *const f32,
        id: *mut u32,
    ) -> i32;
    pub fn avbd_world_add_heightfield(
        world: *mut AvbdWorld,
        rows: u32,
        cols: u32,
        cell: f32,
        heights: *const f32,
        id: *mut u32,
    ) -> i32;
    pub fn avbd_world_add_trimesh(
        world: *mut AvbdWorld,
        verts: *const f32,
        nverts: u32,
        tris: *const u32,
        ntris: u32,
        id: *mut u32,
    ) -> i32;
    pub fn avbd_world_remove_body(world: *mut AvbdWorld, handle: u32) -> i32;
    pub fn avbd_world_add_joint(world: *mut AvbdWorld, desc: *const AvbdJointDesc, handle: *mut u32) -> i32;
    pub fn avbd_world_remove_joint(world: *mut AvbdWorld, handle: u32) -> i32;
    pub fn avbd_world_wake_body(world: *mut AvbdWorld, handle: u32) -> i32;
    pub fn avbd_world_body_count(world: *const AvbdWorld, n: *mut u32) -> i32;
    pub fn avbd_world_scene_count(world: *const AvbdWorld, n: *mut u32) -> i32;
    pub fn avbd_world_get_bodies(world: *mut AvbdWorld, first: u32, n: u32, out: *mut AvbdBody) -> i32;
    pub fn avbd_world_set_bodies(world: *mut AvbdWorld, first: u32, n: u32, bodies: *const AvbdBody) -> i32;
    pub fn avbd_world_step(world: *mut AvbdWorld, dt: f32) -> i32;
    pub fn avbd_world_step_fixed(world: *mut AvbdWorld, substeps: i32) -> i32;
    pub fn avbd_world_step_graph(world: *mut AvbdWorld, substeps: i32) -> i32;
    pub fn avbd_world_sync(world: *mut AvbdWorld) -> i32;
    pub fn avbd_world_get_counters(world: *mut AvbdWorld, out: *mut AvbdCounters) -> i32;
    pub fn avbd_world_state_sizes(world: *mut AvbdWorld, nbodies: *mut u32, npairs: *mut u32, njoints: *mut u32) -> i32;
    pub fn avbd_world_export_state(
        world: *mut AvbdWorld,
        bodies: *mut AvbdBody,
        aux: *mut AvbdBodyAux,
        pairs: *mut AvbdPairState,
        points: *mut AvbdPointState,
        joints: *mut AvbdJointState,
        pair_capacity: u32,
    ) -> i32;
    pub fn avbd_world_import_state(
        world: *mut AvbdWorld,
        bodies: *const AvbdBody,
        aux: *const AvbdBodyAux,
        pairs: *const AvbdPairState,
        points: *const AvbdPointState,
        npairs: u32,
        joints: *const AvbdJointState,
    ) -> i32;
    pub fn avbd_world_snapshot(world: *mut AvbdWorld, buf: *mut u8, cap: u64, size: *mut u64) -> i32;
    pub fn avbd_world_from_snapshot(buf: *const u8, size: u64, device: i32, out: *mut *mut AvbdWorld) -> i32;
    pub fn avbd_snapshot_info(buf: *const u8, size: u64, info: *mut AvbdSnapshotInfo) -> i32;
    pub fn avbd_world_save(world: *mut AvbdWorld, path: *const std::os::raw::c_char) -> i32;
    pub fn avbd_world_load(path: *const std::os::raw::c_char, device: i32, out: *mut *mut AvbdWorld) -> i32;
    pub fn avbd_world_get_colours(world: *mut AvbdWorld, colours: *mut i32, n: u32) -> i32;
    pub fn avbd_body_init(out: *mut AvbdBody, shape: u32, params: *const f32, position: *const f32, mass: f32) -> i32;
    pub fn avbd_set_tuning(world: *mut AvbdWorld, primal_lanes: i32, primal_block: i32) -> i32;
    pub fn avbd_set_precision(world: *mut AvbdWorld, fast: i32) -> i32;
    pub fn avbd_set_events(world: *mut AvbdWorld, period: i32) -> i32;
    pub fn avbd_world_drain_contact_events(
        world: *mut AvbdWorld,
        out: *mut AvbdContactEvent,
        cap: u32,
        n: *mut u32,
    ) -> i32;
    pub fn avbd_world_drain_trigger_events(
        world: *mut AvbdWorld,
        out: *mut AvbdTriggerEvent,
        cap: u32,
        n: *mut u32,
    ) -> i32;
    pub fn avbd_world_event_counts(world: *mut AvbdWorld, counts: *mut u32) -> i32;
    pub fn avbd_set_joint_stiffness(world: *mut AvbdWorld, k: f32) -> i32;
    pub fn avbd_adjoint_forward(world: *mut AvbdWorld, steps: i32, substeps: i32, checkpoint_every: i32) -> i32;
    pub fn avbd_adjoint_backward(
        world: *mut AvbdWorld,
        grad_final: *const f32,
        grad_initial: *mut f32,
        grad_friction: *mut f32,
    ) -> i32;
    pub fn avbd_adjoint_grad_joint_stiffness(world: *mut AvbdWorld, per_scene: *mut f32) -> i32;
    pub fn avbd_scene_step_static(
        params: *const AvbdParams,
        bodies: *const AvbdBody,
        n: u32,
        substeps: i32,
        out: *mut AvbdBody,
    ) -> i32;
}
