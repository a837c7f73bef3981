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
use ornis_physics::collision::shape::{ConvexHull, Pose, Shape};
use ornis_physics::engine::PhysicsEngine;
use ornis_physics::joint::{AxisConfig, JointKind, MotorKind, MotorModel};
use ornis_physics::gpu::GpuAvbdDispatch;

use crate::ffi::*;
use crate::{Error, World};

pub struct CudaAvbd {
    world: RefCell<World>,
    synced: RefCell<u32>,
    /// Per mirrored body: its shape as the library names it (table-backed
    /// shapes are registered once, when the body is first mirrored).
    shapes: RefCell<Vec<(u32, [f32; 3])>>,
}

// The engine is stepped by one thread at a time (PhysicsEngine: Send + Sync
// with &mut self steps); the dispatch is only touched from inside that step.
unsafe impl Sync for CudaAvbd {}

impl CudaAvbd {
    pub fn new(device: i32) -> Result<Self, Error> {
        Ok(CudaAvbd {
            world: RefCell::new(World::new(&crate::default_params(), device)?),
            synced: RefCell::new(0),
            shapes: RefCell::new(Vec::new()),
        })
    }

    pub fn remove_body(&self, handle: u32) -> Result<(), Error> {
        let r = self.world.borrow_mut().remove_body(handle);
        let mut s = self.synced.borrow_mut();
        *s = s.saturating_sub(1);
        // the last body moves into the freed handle (engine.rs:40-43)
        let mut shapes = self.shapes.borrow_mut();
        if (handle as usize) < shapes.len() {
            shapes.swap_remove(handle as usize);
        }
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

/// A primitive shape's kind and parameters; `None` for the table-backed ones.
fn primitive(shape: &Shape) -> Option<(u32, [f32; 3])> {
    Some(match *shape {
        Shape::Sphere { radius } => (AVBD_SHAPE_SPHERE, [radius, 0.0, 0.0]),
        Shape::Box { half_extents } => (AVBD_SHAPE_BOX, half_extents.to_array()),
        Shape::Capsule { radius, half_height } => (AVBD_SHAPE_CAPSULE, [radius, half_height, 0.0]),
        Shape::HalfSpace { normal } => (AVBD_SHAPE_HALFSPACE, normal.get().to_array()),
        Shape::Cylinder { radius, half_height } => (AVBD_SHAPE_CYLINDER, [radius, half_height, 0.0]),
        Shape::Cone { radius, half_height } => (AVBD_SHAPE_CONE, [radius, half_height, 0.0]),
        _ => return None,
    })
}

fn unit_inertia(shape: &Shape) -> [f32; 3] {
    shape.try_inertia(1.0).unwrap_or(Vec3::ZERO).to_array()
}

/// A part of a rounded or compound shape: a primitive or a hull (registered
/// here), placed by `pose` (identity for a rounded shape's inner).
fn part_of(w: &mut World, shape: &Shape, pose: Option<&Pose>) -> Result<AvbdShapePart, Error> {
    // a rounded part carries its skin around a primitive inner
    let (base, skin) = match shape {
        Shape::Round { inner, border_radius } => (inner.as_ref(), *border_radius),
        other => (other, 0.0),
    };
    let (kind, params) = match primitive(base) {
        Some(p) => p,
        None => match base {
            Shape::ConvexHull(hull) => (AVBD_SHAPE_HULL, [register_hull(w, base, hull)? as f32, 0.0, 0.0]),
            _ => return Err(Error::Unsupported), // nested wrappers, terrain, meshes
        },
    };
    Ok(AvbdShapePart {
        shape: kind,
        params,
        border_radius: skin,
        position: pose.map(|p| p.position.to_array()).unwrap_or([0.0; 3]),
        orientation: pose.map(|p| p.rotation.to_array()).unwrap_or([0.0, 0.0, 0.0, 1.0]),
    })
}

fn register_hull(w: &mut World, shape: &Shape, hull: &ConvexHull) -> Result<u32, Error> {
    let verts: Vec<f32> = hull.vertices.iter().flat_map(|v| v.to_array()).collect();
    let faces: Vec<u32> = hull.faces.iter().flat_map(|t| t.as_u32()).collect();
    w.add_hull(&verts, &faces, unit_inertia(shape))
}

/// A body's shape as the library names it: a primitive's fields, or the id
/// of a table-backed shape registered now (hull, rounded, compound,
/// heightfield, triangle mesh).
pub fn register_shape(w: &mut World, shape: &Shape) -> Result<(u32, [f32; 3]), Error> {
    if let Some(p) = primitive(shape) {
        return Ok(p);
    }
    let id = |v: u32| [v as f32, 0.0, 0.0];
    Ok(match shape {
        Shape::ConvexHull(hull) => (AVBD_SHAPE_HULL, id(register_hull(w, shape, hull)?)),
        Shape::Round { .. } => {
            let part = part_of(w, shape, None)?;
            (AVBD_SHAPE_ROUND, id(w.add_round(&part, unit_inertia(shape))?))
        }
        Shape::Compound { shapes } => {
            let parts = shapes.iter().map(|(s, pose)| part_of(w, s, Some(pose))).collect::<Result<Vec<_>, _>>()?;
            (AVBD_SHAPE_COMPOUND, id(w.add_compound(&parts, unit_inertia(shape))?))
        }
        Shape::Heightfield(hf) => {
            (AVBD_SHAPE_HEIGHTFIELD, id(w.add_heightfield(hf.rows as u32, hf.cols as u32, hf.cell, &hf.heights)?))
        }
        Shape::TriMesh(mesh) => {
            // the engine keeps centroid-relative triangle hulls: the vertices
            // come back as hull vertex + centroid (the library recomputes the
            // centroid from them, which can differ from the original in the
            // last bit)
            let mut verts = Vec::new();
            let mut tris = Vec::new();
            for (t, tri) in mesh.tris.iter().enumerate() {
                if let Shape::ConvexHull(h) = tri {
                    let base = (verts.len() / 3) as u32;
                    for v in &h.vertices {
                        verts.extend_from_slice(&(*v + mesh.centroids[t]).to_array());
                    }
                    tris.extend_from_slice(&[base, base + 1, base + 2]);
                }
            }
            (AVBD_SHAPE_TRIMESH, id(w.add_trimesh(&verts, &tris)?))
        }
        _ => return Err(Error::Unsupported),
    })
}

/// `JointKind` (joint.rs:209-410) to the C descriptor the library admits
/// (`avbd_world_add_joint`), for bodies `a` and `b`.  The spring's
/// integration choice has no device counterpart (the AVBD step integrates
/// every spring the same way) and is not carried.
pub fn joint_desc(kind: &JointKind, a: u32, b: u32) -> AvbdJointDesc {
    let mut d = AvbdJointDesc { body_a: a, body_b: b, ..Default::default() };
    let v = |x: Vec3| x.to_array();
    match *kind {
        JointKind::Ball { local_anchor_a, local_anchor_b } => {
            d.kind = AVBD_JOINT_BALL;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
        }
        JointKind::Revolute { local_anchor_a, local_anchor_b, local_axis_a, local_axis_b, limit, motor } => {
            d.kind = AVBD_JOINT_REVOLUTE;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
            d.local_axis_a = v(local_axis_a);
            d.local_axis_b = v(local_axis_b);
            if let Some(l) = limit {
                d.has_limit = 1;
                d.limit_min = l.min;
                d.limit_max = l.max;
            }
            if let Some(m) = motor {
                d.has_motor = 1;
                d.motor_speed = m.target_speed;
                d.motor_max = m.max_torque;
            }
        }
        JointKind::Prismatic { local_anchor_a, local_anchor_b, local_axis_a, local_axis_b, limit, motor } => {
            d.kind = AVBD_JOINT_PRISMATIC;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
            d.local_axis_a = v(local_axis_a);
            d.local_axis_b = v(local_axis_b);
            if let Some(l) = limit {
                d.has_limit = 1;
                d.limit_min = l.min;
                d.limit_max = l.max;
            }
            if let Some(m) = motor {
                d.has_motor = 1;
                d.motor_speed = m.target_speed;
                d.motor_max = m.max_force;
            }
        }
        JointKind::Fixed { local_anchor_a, local_anchor_b } => {
            d.kind = AVBD_JOINT_FIXED;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
        }
        JointKind::Distance { local_anchor_a, local_anchor_b } => {
            d.kind = AVBD_JOINT_DISTANCE;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
        }
        JointKind::Rope { local_anchor_a, local_anchor_b, max_distance } => {
            d.kind = AVBD_JOINT_ROPE;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
            d.max_distance = max_distance;
        }
        JointKind::Spring { local_anchor_a, local_anchor_b, motor, .. } => {
            d.kind = AVBD_JOINT_SPRING;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
            d.spring_rest = motor.target_position;
            d.spring_velocity = motor.target_velocity;
            d.spring_stiffness = motor.stiffness;
            d.spring_damping = motor.damping;
            d.spring_max_force = motor.max_force;
            d.spring_kind = match motor.kind {
                MotorKind::Velocity => AVBD_MOTOR_VELOCITY,
                MotorKind::Position => AVBD_MOTOR_POSITION,
                MotorKind::Servo => AVBD_MOTOR_SERVO,
            };
            d.spring_model = match motor.model {
                MotorModel::AccelerationBased => AVBD_MODEL_ACCELERATION,
                MotorModel::ForceBased => AVBD_MODEL_FORCE,
            };
        }
        JointKind::Wheel {
            local_anchor_a,
            local_anchor_b,
            local_suspension_a,
            local_suspension_b,
            local_axle_a,
            local_axle_b,
            suspension,
            motor,
        } => {
            d.kind = AVBD_JOINT_WHEEL;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
            d.local_axis_a = v(local_suspension_a);
            d.local_axis_b = v(local_suspension_b);
            d.local_axle_a = v(local_axle_a);
            d.local_axle_b = v(local_axle_b);
            d.suspension_hz = suspension.frequency_hz;
            d.suspension_damping = suspension.damping_ratio;
            if let Some(m) = motor {
                d.has_motor = 1;
                d.motor_speed = m.target_speed;
                d.motor_max = m.max_torque;
            }
        }
        JointKind::Gear { joint_a, joint_b, ratio } => {
            d.kind = AVBD_JOINT_GEAR;
            d.gear_joint_a = joint_a.index() as u32;
            d.gear_joint_b = joint_b.index() as u32;
            d.gear_ratio = ratio;
        }
        JointKind::SixDof { local_anchor_a, local_anchor_b, linear, angular } => {
            d.kind = AVBD_JOINT_SIXDOF;
            d.local_anchor_a = v(local_anchor_a);
            d.local_anchor_b = v(local_anchor_b);
            for (k, c) in linear.iter().chain(angular.iter()).enumerate() {
                match *c {
                    AxisConfig::Free => d.axis_config[k] = AVBD_AXIS_FREE,
                    AxisConfig::Locked => d.axis_config[k] = AVBD_AXIS_LOCKED,
                    AxisConfig::Limited { min, max } => {
                        d.axis_config[k] = AVBD_AXIS_LIMITED;
                        d.axis_min[k] = min;
                        d.axis_max[k] = max;
                    }
                }
            }
        }
        JointKind::Motor { linear_target, angular_target, max_force, max_torque, correction } => {
            d.kind = AVBD_JOINT_MOTOR;
            d.motor_linear = v(linear_target);
            d.motor_angular = v(angular_target);
            d.motor_max_force = max_force;
            d.motor_max_torque = max_torque;
            d.motor_correction = correction;
        }
    }
    d
}

/// RigidBody (body.rs:248-342) to the C record, its shape named as
/// `register_shape` named it.
pub fn to_ffi(b: &RigidBody, named: (u32, [f32; 3])) -> AvbdBody {
    let (shape, params) = named;
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
        let mut shapes = self.shapes.borrow_mut();
        if n > synced {
            let mut recs = Vec::new();
            for h in synced..n {
                let b = engine.get_body(BodyHandle::from(h as usize)).unwrap();
                let named = register_shape(&mut w, &b.shape).expect("a shape the library accepts");
                shapes.push(named);
                recs.push(to_ffi(b, named));
            }
            w.add_bodies(&recs).expect("avbd_world_add_bodies");
            *self.synced.borrow_mut() = n;
        }
        let recs: Vec<AvbdBody> = (0..n)
            .map(|h| to_ffi(engine.get_body(BodyHandle::from(h as usize)).unwrap(), shapes[h as usize]))
            .collect();
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
