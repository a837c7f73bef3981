//! `GpuAvbdDispatch` (crates/physics/src/gpu/avbd.rs:146-151) for Ornis's
//! `AvbdEngine`: every step of an engine the dispatch is attached to
//! (`AvbdEngine::set_gpu_avbd`, avbd/mod.rs:800-803; consulted at the top of
//! `step`, mod.rs:1220-1223) runs on the GPU world this type owns.
//!
//! Per step: bodies added since the last step are mirrored (handles are
//! dense and in insertion order on both sides), host edits made through
//! `get_body_mut` are written back, the accumulator and every substep run on
//! the device, and the stepped state is read back into the engine's bodies.
//! Removals and joints go through [`CudaAvbd::remove_body`],
//! [`CudaAvbd::add_joint`], [`CudaAvbd::remove_joint`] next to the engine's
//! own calls, so both sides renumber identically.

use std::cell::RefCell;

use glam::{Quat, Vec3};
use ornis_physics::avbd::AvbdEngine;
use ornis_physics::body::{BodyHandle, BodyType, RigidBody};
use ornis_physics::collision::shape::Shape;
use ornis_physics::engine::PhysicsEngine;
use ornis_physics::gpu::GpuAvbdDispatch;

use crate::ffi::*;
use crate::{Error, World};

pub struct CudaAvbd {
    world: RefCell<World>,
    synced: RefCell<u32>,
}

// The engine is stepped by one thread at a time (PhysicsEngine: Send + Sync
// with &mut self steps); the dispatch is only touched from inside that step.
unsafe impl Sync for CudaAvbd {}

impl CudaAvbd {
    pub fn new(device: i32) -> Result<Self, Error> {
        Ok(CudaAvbd { world: RefCell::new(World::new(&crate::default_params(), device)?), synced: RefCell::new(0) })
    }

    pub fn remove_body(&self, handle: u32) -> Result<(), Error> {
        let r = self.world.borrow_mut().remove_body(handle);
        let mut s = self.synced.borrow_mut();
        *s = s.saturating_sub(1);
        r
    }

    pub fn add_joint(&self, desc: &AvbdJointDesc) -> Result<u32, Error> {
        self.world.borrow_mut().add_joint(desc)
    }

    pub fn remove_joint(&self, handle: u32) -> Result<(), Error> {
        self.world.borrow_mut().remove_joint(handle)
    }
}

fn count(engine: &AvbdEngine) -> u32 {
    let mut n = 0u32;
    while engine.get_body(BodyHandle::from(n as usize)).is_some() {
        n += 1;
    }
    n
}

/// RigidBody (body.rs:248-342) to the C record.
pub fn to_ffi(b: &RigidBody) -> AvbdBody {
    let (shape, params) = match b.shape {
        Shape::Sphere { radius } => (AVBD_SHAPE_SPHERE, [radius, 0.0, 0.0]),
        Shape::Box { half_extents } => (AVBD_SHAPE_BOX, half_extents.to_array()),
        Shape::Capsule { radius, half_height } => (AVBD_SHAPE_CAPSULE, [radius, half_height, 0.0]),
        Shape::HalfSpace { normal } => (AVBD_SHAPE_HALFSPACE, normal.to_array()),
        Shape::Cylinder { radius, half_height } => (AVBD_SHAPE_CYLINDER, [radius, half_height, 0.0]),
        Shape::Cone { radius, half_height } => (AVBD_SHAPE_CONE, [radius, half_height, 0.0]),
        // hulls are registered with avbd_world_add_hull and named by index
        _ => (AVBD_SHAPE_HULL, [0.0, 0.0, 0.0]),
    };
    AvbdBody {
        position: b.position.to_array(),
        orientation: b.orientation.to_array(),
        velocity: b.velocity.to_array(),
        angular_velocity: b.angular_velocity.to_array(),
        torque: b.torque.to_array(),
        mass: b.mass,
        inv_mass: b.inv_mass,
        inertia: b.inertia.to_array(),
        restitution: b.restitution,
        friction: b.friction,
        friction_transverse: b.friction_transverse,
        rolling_friction: b.rolling_friction,
        torsion_friction: b.torsion_friction,
        shape,
        shape_params: params,
        collision_layer: b.collision_layer,
        collision_mask: b.collision_mask,
        body_type: match b.body_type {
            BodyType::Dynamic => AVBD_BODY_DYNAMIC,
            BodyType::Static => AVBD_BODY_STATIC,
            BodyType::Kinematic => AVBD_BODY_KINEMATIC,
        },
        flags: if b.is_trigger { AVBD_FLAG_TRIGGER } else { 0 },
    }
}

/// The state the step writes back (pose, velocities, the sleep-frozen mass
/// triple, torque cleared by the step).
pub fn from_ffi(b: &mut RigidBody, r: &AvbdBody) {
    b.position = Vec3::from_array(r.position);
    b.orientation = Quat::from_array(r.orientation);
    b.velocity = Vec3::from_array(r.velocity);
    b.angular_velocity = Vec3::from_array(r.angular_velocity);
    b.torque = Vec3::from_array(r.torque);
    b.inv_mass = r.inv_mass;
    b.inertia = Vec3::from_array(r.inertia);
}

impl GpuAvbdDispatch for CudaAvbd {
    fn runs_on_device(&self) -> bool {
        true
    }

    fn step_avbd(&self, engine: &mut AvbdEngine, dt: f32) {
        let mut w = self.world.borrow_mut();
        let n = count(engine);
        let synced = *self.synced.borrow();
        if n > synced {
            let recs: Vec<AvbdBody> =
                (synced..n).map(|h| to_ffi(engine.get_body(BodyHandle::from(h as usize)).unwrap())).collect();
            w.add_bodies(&recs).expect("avbd_world_add_bodies");
            *self.synced.borrow_mut() = n;
        }
        let recs: Vec<AvbdBody> = (0..n).map(|h| to_ffi(engine.get_body(BodyHandle::from(h as usize)).unwrap())).collect();
        w.set_bodies(0, &recs).expect("avbd_world_set_bodies");
        w.step(dt).expect("avbd_world_step");
        let mut out = vec![AvbdBody::default(); n as usize];
        w.bodies(0, &mut out).expect("avbd_world_get_bodies");
        for (h, r) in out.iter().enumerate() {
            if let Some(b) = engine.get_body_mut(BodyHandle::from(h)) {
                from_ffi(b, r);
            }
        }
    }
}
