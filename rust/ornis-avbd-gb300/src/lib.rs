//! Safe Rust types over the GB300 AVBD step (`libornis_avbd.so`, declared in
//! `include/ornis_avbd.h`): the drop-in for Ornis's `AvbdEngine` step.
//!
//! * [`World`]: one engine-equivalent world (the reference's `AvbdEngine`):
//!   bodies, joints, the fixed-step accumulator, host edits, events.
//! * [`Batch`]: many independent scenes packed in one world, stepped by
//!   CUDA-graph replay.
//! * [`Rollout`]: the differentiable rollout as one forward/backward
//!   Function-style type.
//! * `dispatch::CudaAvbd` (feature `ornis`): `GpuAvbdDispatch` for
//!   `AvbdEngine`, the seam `crates/physics/src/gpu/avbd.rs:146-151` defines.
//!
//! Status codes become [`Error`]; a world is `Send` but not `Sync` (one
//! `&mut` step at a time, the reference's threading contract).

pub mod ffi;
#[cfg(feature = "ornis")]
pub mod dispatch;

use ffi::*;

/// A failed call: the header's status code.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Error {
    InvalidArg,
    Capacity,
    Device,
    Timeout,
    NonFinite,
    Unsupported,
    /// Not an intact snapshot of this format version (the reference's
    /// `SnapshotError::VersionMismatch`, snapshot.rs:815-830, and damage).
    Format,
    /// A snapshot file could not be read or written.
    Io,
    /// `JointError::SelfJoint` (avbd/mod.rs:1323-1328)
    JointSelf,
    /// `JointError::InvalidHandles`
    JointHandles,
    /// `JointError::BadAxis`
    JointBadAxis,
    /// `JointError::NonFinite`
    JointNonFinite,
    /// `JointError::BadBounds`
    JointBadBounds,
    /// `JointError::UnknownRef` (a gear's coupled joint does not exist)
    JointUnknownRef,
    Other(i32),
}

impl Error {
    fn check(rc: i32) -> Result<(), Error> {
        Err(match rc {
            AVBD_OK => return Ok(()),
            AVBD_ERR_INVALID_ARG => Error::InvalidArg,
            AVBD_ERR_CAPACITY => Error::Capacity,
            AVBD_ERR_DEVICE => Error::Device,
            AVBD_ERR_TIMEOUT => Error::Timeout,
            AVBD_ERR_NONFINITE => Error::NonFinite,
            AVBD_ERR_UNSUPPORTED => Error::Unsupported,
            AVBD_ERR_FORMAT => Error::Format,
            AVBD_ERR_IO => Error::Io,
            AVBD_ERR_JOINT_SELF => Error::JointSelf,
            AVBD_ERR_JOINT_HANDLES => Error::JointHandles,
            AVBD_ERR_JOINT_BAD_AXIS => Error::JointBadAxis,
            AVBD_ERR_JOINT_NONFINITE => Error::JointNonFinite,
            AVBD_ERR_JOINT_BAD_BOUNDS => Error::JointBadBounds,
            AVBD_ERR_JOINT_UNKNOWN_REF => Error::JointUnknownRef,
            other => Error::Other(other),
        })
    }
}

/// The reference's solver constants (avbd/mod.rs:154-247, DT_STEP 1/60,
/// ITERS 10, MAX_SUBSTEPS 4, sleep and CCD on).
pub fn default_params() -> AvbdParams {
    let mut p = AvbdParams::default();
    unsafe { avbd_default_params(&mut p) };
    p
}

/// `RigidBody::new_*` (body.rs:346-376, :470-576): one body record with the
/// reference's material for the shape; `mass <= 0` makes a static body.
pub fn body(shape: u32, params: [f32; 3], position: [f32; 3], mass: f32) -> Result<AvbdBody, Error> {
    let mut b = AvbdBody::default();
    Error::check(unsafe { avbd_body_init(&mut b, shape, params.as_ptr(), position.as_ptr(), mass) })?;
    Ok(b)
}

/// One world on one GPU (the reference's `AvbdEngine`).
pub struct World {
    raw: *mut AvbdWorld,
}

// One thread at a time steps a world; the library keeps no thread-local state.
unsafe impl Send for World {}

impl World {
    pub fn new(params: &AvbdParams, device: i32) -> Result<Self, Error> {
        let mut raw = std::ptr::null_mut();
        Error::check(unsafe { avbd_world_create(params, device, &mut raw) })?;
        Ok(World { raw })
    }

    pub fn raw(&self) -> *mut AvbdWorld {
        self.raw
    }

    /// `ConvexHull`: centroid-relative vertices, triangle faces and the
    /// per-unit-mass inertia; bodies of shape `AVBD_SHAPE_HULL` name the id.
    pub fn add_hull(&mut self, verts: &[f32], faces: &[u32], unit_inertia: [f32; 3]) -> Result<u32, Error> {
        let mut id = 0u32;
        Error::check(unsafe {
            avbd_world_add_hull(
                self.raw,
                verts.as_ptr(),
                (verts.len() / 3) as u32,
                if faces.is_empty() { std::ptr::null() } else { faces.as_ptr() },
                (faces.len() / 3) as u32,
                unit_inertia.as_ptr(),
                &mut id,
            )
        })?;
        Ok(id)
    }

    /// `Heightfield`: rows x cols row-major heights on a grid of `cell`.
    pub fn add_heightfield(&mut self, rows: u32, cols: u32, cell: f32, heights: &[f32]) -> Result<u32, Error> {
        if heights.len() != (rows as usize) * (cols as usize) {
            return Err(Error::InvalidArg);
        }
        let mut id = 0u32;
        Error::check(unsafe { avbd_world_add_heightfield(self.raw, rows, cols, cell, heights.as_ptr(), &mut id) })?;
        Ok(id)
    }

    /// `TriMesh::from_indexed`: vertices (3 floats each) and triangles (3
    /// indices each).
    pub fn add_trimesh(&mut self, verts: &[f32], tris: &[u32]) -> Result<u32, Error> {
        let mut id = 0u32;
        Error::check(unsafe {
            avbd_world_add_trimesh(
                self.raw,
                verts.as_ptr(),
                (verts.len() / 3) as u32,
                tris.as_ptr(),
                (tris.len() / 3) as u32,
                &mut id,
            )
        })?;
        Ok(id)
    }

    /// `Shape::Round` around one primitive part: bodies of shape
    /// `AVBD_SHAPE_ROUND` name the returned id in `shape_params[0]`.
    pub fn add_round(&mut self, inner: &AvbdShapePart, unit_inertia: [f32; 3]) -> Result<u32, Error> {
        let mut id = 0u32;
        Error::check(unsafe { avbd_world_add_round(self.raw, inner, unit_inertia.as_ptr(), &mut id) })?;
        Ok(id)
    }

    /// `Shape::Compound` of primitive parts placed by their poses.
    pub fn add_compound(&mut self, parts: &[AvbdShapePart], unit_inertia: [f32; 3]) -> Result<u32, Error> {
        let mut id = 0u32;
        Error::check(unsafe {
            avbd_world_add_compound(self.raw, parts.as_ptr(), parts.len() as u32, unit_inertia.as_ptr(), &mut id)
        })?;
        Ok(id)
    }

    /// The whole world as a versioned snapshot: a world made from it
    /// continues bit for bit, events included.
    pub fn snapshot(&mut self) -> Result<Vec<u8>, Error> {
        let mut n = 0u64;
        Error::check(unsafe { avbd_world_snapshot(self.raw, std::ptr::null_mut(), 0, &mut n) })?;
        let mut buf = vec![0u8; n as usize];
        Error::check(unsafe { avbd_world_snapshot(self.raw, buf.as_mut_ptr(), n, &mut n) })?;
        buf.truncate(n as usize);
        Ok(buf)
    }

    /// A new world on `device` from `snapshot`'s bytes.
    pub fn from_snapshot(bytes: &[u8], device: i32) -> Result<Self, Error> {
        let mut raw = std::ptr::null_mut();
        Error::check(unsafe { avbd_world_from_snapshot(bytes.as_ptr(), bytes.len() as u64, device, &mut raw) })?;
        Ok(World { raw })
    }

    /// Write the snapshot to `path` (whole, then renamed into place).
    pub fn save(&mut self, path: &std::path::Path) -> Result<(), Error> {
        let c = path_cstring(path)?;
        Error::check(unsafe { avbd_world_save(self.raw, c.as_ptr()) })
    }

    /// A new world on `device` from a snapshot file.
    pub fn load(path: &std::path::Path, device: i32) -> Result<Self, Error> {
        let c = path_cstring(path)?;
        let mut raw = std::ptr::null_mut();
        Error::check(unsafe { avbd_world_load(c.as_ptr(), device, &mut raw) })?;
        Ok(World { raw })
    }

    /// `PhysicsEngine::add_body`: returns the first new handle.
    pub fn add_bodies(&mut self, bodies: &[AvbdBody]) -> Result<u32, Error> {
        let mut first = 0u32;
        Error::check(unsafe { avbd_world_add_bodies(self.raw, bodies.as_ptr(), bodies.len() as u32, &mut first) })?;
        Ok(first)
    }

    /// `PhysicsEngine::remove_body`: the last body moves into the handle.
    pub fn remove_body(&mut self, handle: u32) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_remove_body(self.raw, handle) })
    }

    /// `PhysicsEngine::add_joint`, with `JointError` as [`Error::Joint*`].
    pub fn add_joint(&mut self, desc: &AvbdJointDesc) -> Result<u32, Error> {
        let mut h = 0u32;
        Error::check(unsafe { avbd_world_add_joint(self.raw, desc, &mut h) })?;
        Ok(h)
    }

    /// `PhysicsEngine::remove_joint`: both members wake; later handles move down one.
    pub fn remove_joint(&mut self, handle: u32) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_remove_joint(self.raw, handle) })
    }

    /// `PhysicsEngine::wake_body`.
    pub fn wake_body(&mut self, handle: u32) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_wake_body(self.raw, handle) })
    }

    pub fn body_count(&self) -> u32 {
        let mut n = 0u32;
        unsafe { avbd_world_body_count(self.raw, &mut n) };
        n
    }

    /// `PhysicsEngine::step`: the fixed-step accumulator (a bad `dt` is a no-op).
    pub fn step(&mut self, dt: f32) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_step(self.raw, dt) })
    }

    /// Exactly `substeps` fixed substeps by CUDA-graph replay.
    pub fn step_substeps(&mut self, substeps: i32) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_step_graph(self.raw, substeps) })
    }

    /// `get_body` for a range of handles (host copies).
    pub fn bodies(&mut self, first: u32, out: &mut [AvbdBody]) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_get_bodies(self.raw, first, out.len() as u32, out.as_mut_ptr()) })
    }

    /// `get_body_mut` edits written back: they apply at the next step.
    pub fn set_bodies(&mut self, first: u32, bodies: &[AvbdBody]) -> Result<(), Error> {
        Error::check(unsafe { avbd_world_set_bodies(self.raw, first, bodies.len() as u32, bodies.as_ptr()) })
    }

    /// `drain_contact_events`.
    pub fn drain_contact_events(&mut self) -> Result<Vec<AvbdContactEvent>, Error> {
        let mut counts = [0u32; 4];
        Error::check(unsafe { avbd_world_event_counts(self.raw, counts.as_mut_ptr()) })?;
        let mut out = vec![AvbdContactEvent::default(); counts[0] as usize];
        let mut n = 0u32;
        Error::check(unsafe {
            avbd_world_drain_contact_events(self.raw, out.as_mut_ptr(), out.len() as u32, &mut n)
        })?;
        out.truncate(n as usize);
        Ok(out)
    }

    /// `drain_trigger_events`.
    pub fn drain_trigger_events(&mut self) -> Result<Vec<AvbdTriggerEvent>, Error> {
        let mut counts = [0u32; 4];
        Error::check(unsafe { avbd_world_event_counts(self.raw, counts.as_mut_ptr()) })?;
        let mut out = vec![AvbdTriggerEvent::default(); counts[1] as usize];
        let mut n = 0u32;
        Error::check(unsafe {
            avbd_world_drain_trigger_events(self.raw, out.as_mut_ptr(), out.len() as u32, &mut n)
        })?;
        out.truncate(n as usize);
        Ok(out)
    }

    /// `sleeping_count` and the rest of the counters (avbd/mod.rs:788-790).
    pub fn counters(&mut self) -> AvbdCounters {
        let mut c = AvbdCounters::default();
        unsafe { avbd_world_get_counters(self.raw, &mut c) };
        c
    }
}

fn path_cstring(path: &std::path::Path) -> Result<std::ffi::CString, Error> {
    let s = path.to_str().ok_or(Error::InvalidArg)?;
    std::ffi::CString::new(s).map_err(|_| Error::InvalidArg)
}

/// Validate a snapshot on the host (header, checksum, contents) without a GPU.
pub fn snapshot_info(bytes: &[u8]) -> Result<AvbdSnapshotInfo, Error> {
    let mut info = AvbdSnapshotInfo::default();
    Error::check(unsafe { avbd_snapshot_info(bytes.as_ptr(), bytes.len() as u64, &mut info) })?;
    Ok(info)
}

impl Drop for World {
    fn drop(&mut self) {
        unsafe { avbd_world_destroy(self.raw) };
    }
}

/// Independent scenes in one flat world: scene `s` owns the handles
/// `[offsets[s], offsets[s + 1])`.  Scenes never interact.
pub struct Batch {
    pub world: World,
    pub offsets: Vec<u32>,
}

impl Batch {
    pub fn new(params: &AvbdParams, device: i32, bodies: &[AvbdBody], offsets: &[u32]) -> Result<Self, Error> {
        let mut raw = std::ptr::null_mut();
        Error::check(unsafe {
            avbd_world_create_batch(
                params,
                device,
                bodies.as_ptr(),
                bodies.len() as u32,
                offsets.as_ptr(),
                (offsets.len() - 1) as u32,
                &mut raw,
            )
        })?;
        Ok(Batch { world: World { raw }, offsets: offsets.to_vec() })
    }

    /// `substeps` fixed substeps of every scene by CUDA-graph replay.
    pub fn step(&mut self, substeps: i32) -> Result<(), Error> {
        self.world.step_substeps(substeps)
    }
}

/// A differentiable rollout as one forward/backward Function-style type:
/// `forward` steps the world and keeps checkpoints, `backward` maps
/// dLoss/d(final state) to dLoss/d(initial state) and dLoss/d(friction) per
/// scene (13 floats per body: position, orientation xyzw, velocity, angular
/// velocity).  Contact frames, colouring and swept impacts are held at the
/// forward's values (the header states the convention).
pub struct Rollout<'w> {
    world: &'w mut World,
    steps: i32,
    substeps: i32,
    checkpoint_every: i32,
}

impl<'w> Rollout<'w> {
    pub fn new(world: &'w mut World, steps: i32, substeps: i32, checkpoint_every: i32) -> Self {
        Rollout { world, steps, substeps, checkpoint_every }
    }

    pub fn forward(&mut self) -> Result<(), Error> {
        Error::check(unsafe {
            avbd_adjoint_forward(self.world.raw, self.steps, self.substeps, self.checkpoint_every)
        })
    }

    /// Returns (dLoss/d(initial state), dLoss/d(friction) per scene).
    pub fn backward(&mut self, grad_final: &[f32], nscenes: usize) -> Result<(Vec<f32>, Vec<f32>), Error> {
        let mut g0 = vec![0.0f32; grad_final.len()];
        let mut gmu = vec![0.0f32; nscenes];
        Error::check(unsafe {
            avbd_adjoint_backward(self.world.raw, grad_final.as_ptr(), g0.as_mut_ptr(), gmu.as_mut_ptr())
        })?;
        Ok((g0, gmu))
    }

    /// dLoss/d(joint stiffness) per scene of the last backward.
    pub fn grad_joint_stiffness(&mut self, nscenes: usize) -> Result<Vec<f32>, Error> {
        let mut g = vec![0.0f32; nscenes];
        Error::check(unsafe { avbd_adjoint_grad_joint_stiffness(self.world.raw, g.as_mut_ptr()) })?;
        Ok(g)
    }
}
