"""Host-side mirror of the reference's AVBD engine API over the C ABI.

`AvbdWorld` follows `AvbdEngine` / `PhysicsEngine` (crates/physics/src/
avbd/mod.rs:1147-1602, engine.rs:24-133): bodies are added in handle order,
`step(dt)` runs the fixed-step accumulator, `get_body`/`set_body` read and
write the body records, `add_joint` returns a handle or raises the
JointError-style status.  Every call goes to libornis_avbd.so, whose step runs
only on the GPU: there is no CPU path behind this class.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libornis_avbd.so")

_lib = None


class AvbdError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what} failed with status {code}")
        self.code = code


def lib():
    """Load libornis_avbd.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build
            build.build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        u32 = C.c_uint32
        sigs = {
            "avbd_default_params": [C.POINTER(abi.AvbdParams)],
            "avbd_world_create": [C.POINTER(abi.AvbdParams), C.c_int, C.POINTER(vp)],
            "avbd_world_create_batch": [C.POINTER(abi.AvbdParams), C.c_int, vp, u32, vp, u32, C.POINTER(vp)],
            "avbd_world_destroy": [vp],
            "avbd_world_add_bodies": [vp, vp, u32, C.POINTER(u32)],
            "avbd_world_add_joint": [vp, C.POINTER(abi.AvbdJointDesc), C.POINTER(u32)],
            "avbd_world_remove_body": [vp, u32],
            "avbd_world_remove_joint": [vp, u32],
            "avbd_world_wake_body": [vp, u32],
            "avbd_world_add_hull": [vp, vp, u32, vp, u32, vp, C.POINTER(u32)],
            "avbd_world_add_round": [vp, C.POINTER(abi.AvbdShapePart), vp, C.POINTER(u32)],
            "avbd_world_add_compound": [vp, vp, u32, vp, C.POINTER(u32)],
            "avbd_world_add_heightfield": [vp, u32, u32, C.c_float, vp, C.POINTER(u32)],
            "avbd_world_add_trimesh": [vp, vp, u32, vp, u32, C.POINTER(u32)],
            "avbd_world_body_count": [vp, C.POINTER(u32)],
            "avbd_world_scene_count": [vp, C.POINTER(u32)],
            "avbd_world_get_bodies": [vp, u32, u32, vp],
            "avbd_world_set_bodies": [vp, u32, u32, vp],
            "avbd_world_step": [vp, C.c_float],
            "avbd_world_step_fixed": [vp, C.c_int32],
            "avbd_world_step_graph": [vp, C.c_int32],
            "avbd_world_sync": [vp],
            "avbd_world_get_counters": [vp, C.POINTER(abi.AvbdCounters)],
            "avbd_world_state_sizes": [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)],
            "avbd_world_export_state": [vp, vp, vp, vp, vp, vp, u32],
            "avbd_world_import_state": [vp, vp, vp, vp, vp, u32, vp],
            "avbd_world_get_colours": [vp, vp, u32],
            "avbd_body_init": [C.POINTER(abi.AvbdBody), u32, vp, vp, C.c_float],
            "avbd_set_tuning": [vp, C.c_int, C.c_int],
            "avbd_set_precision": [vp, C.c_int],
            "avbd_set_occupancy": [vp, C.c_int],
            "avbd_profiler": [C.c_int],
            "avbd_set_work_order": [vp, C.c_int],
            "avbd_abi_version": [],
            "avbd_world_step_timed": [vp, C.c_int32, C.c_int32, C.POINTER(C.c_float)],
            "avbd_world_flush_cache": [vp],
            "avbd_world_profile_substep": [vp, vp, vp],
            "avbd_world_graph_nodes": [vp, C.POINTER(u32)],
            "avbd_scene_step_static": [C.POINTER(abi.AvbdParams), vp, u32, C.c_int32, vp],
            "avbd_world_graph_nodes_emit": [vp, C.POINTER(u32)],
            "avbd_set_events": [vp, C.c_int32],
            "avbd_set_broadphase": [vp, C.c_int],
            "avbd_set_sweep": [vp, C.c_int],
            "avbd_world_drain_contact_events": [vp, vp, u32, C.POINTER(u32)],
            "avbd_world_drain_trigger_events": [vp, vp, u32, C.POINTER(u32)],
            "avbd_world_event_counts": [vp, vp],
            "avbd_adjoint_forward": [vp, C.c_int32, C.c_int32, C.c_int32],
            "avbd_adjoint_backward": [vp, vp, vp, vp],
            "avbd_adjoint_timing": [vp, vp],
            "avbd_adjoint_trace": [vp, vp, vp, C.c_int32, C.POINTER(C.c_int32)],
            "avbd_set_joint_stiffness": [vp, C.c_float],
            "avbd_adjoint_grad_joint_stiffness": [vp, vp],
            "avbd_world_snapshot": [vp, vp, C.c_uint64, C.POINTER(C.c_uint64)],
            "avbd_world_from_snapshot": [vp, C.c_uint64, C.c_int, C.POINTER(vp)],
            "avbd_snapshot_info": [vp, C.c_uint64, C.POINTER(abi.AvbdSnapshotInfo)],
            "avbd_world_save": [vp, C.c_char_p],
            "avbd_world_load": [C.c_char_p, C.c_int, C.POINTER(vp)],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def _check(rc, what):
    if rc != abi.AVBD_OK:
        raise AvbdError(rc, what)


def body(shape, params, position, mass):
    """RigidBody::new_* (body.rs:470-576): one body record with default material."""
    b = abi.AvbdBody()
    p = np.zeros(3, dtype=np.float32)
    p[: len(params)] = params
    pos = np.asarray(position, dtype=np.float32)
    _check(lib().avbd_body_init(C.byref(b), shape, abi.ptr(p), abi.ptr(pos), float(mass)), "avbd_body_init")
    return b


def bodies_array(records):
    arr = np.zeros(len(records), dtype=abi.BODY_DTYPE)
    if records:
        C.memmove(arr.ctypes.data, (abi.AvbdBody * len(records))(*records), arr.nbytes)
    return arr


def scene_step_static(params, bodies, substeps):
    """Step one small scene without any device allocation (avbd_scene_step_static).

    For callers that cannot call cudaMalloc: the library keeps one fixed
    device array for this entry point (abi.STATIC_SCRATCH_BYTES per GPU) and
    accepts at most abi.STATIC_MAX_BODIES bodies.  Returns the stepped body
    records; the input array is not modified.
    """
    src = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
    out = np.empty_like(src)
    rc = lib().avbd_scene_step_static(C.byref(params), src.ctypes.data, len(src), int(substeps), out.ctypes.data)
    _check(rc, "avbd_scene_step_static")
    return out


def snapshot_info(data):
    """Header of a world snapshot (avbd_snapshot_info): validated, checksum
    included, without a GPU.  Raises AvbdError(AVBD_ERR_FORMAT) for anything
    that is not an intact snapshot of this format version."""
    buf = bytes(data)
    info = abi.AvbdSnapshotInfo()
    _check(lib().avbd_snapshot_info(buf, len(buf), C.byref(info)), "avbd_snapshot_info")
    return info


class AvbdWorld:
    """One AVBD world on one GPU: one scene (AvbdEngine) or many (a batch)."""

    def __init__(self, params=None, device=0, bodies=None, scene_offsets=None):
        self.params = params if params is not None else abi.default_params()
        h = C.c_void_p()
        if bodies is not None:
            bodies = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
            if scene_offsets is None:
                scene_offsets = [0, len(bodies)]
            so = np.ascontiguousarray(scene_offsets, dtype=np.uint32)
            _check(lib().avbd_world_create_batch(C.byref(self.params), device, abi.ptr(bodies), len(bodies),
                                                 abi.ptr(so), len(so) - 1, C.byref(h)), "avbd_world_create_batch")
        else:
            _check(lib().avbd_world_create(C.byref(self.params), device, C.byref(h)), "avbd_world_create")
        self.h = h

    @classmethod
    def _adopt(cls, h, params):
        self = cls.__new__(cls)
        self.h = h
        self.params = params
        return self

    @classmethod
    def from_snapshot(cls, data, device=0):
        """A new world from the bytes of AvbdWorld.snapshot() (avbd_world_from_snapshot)."""
        buf = bytes(data)
        h = C.c_void_p()
        _check(lib().avbd_world_from_snapshot(buf, len(buf), device, C.byref(h)), "avbd_world_from_snapshot")
        off = abi.SNAPSHOT_HEADER_BYTES
        return cls._adopt(h, abi.AvbdParams.from_buffer_copy(buf[off:off + C.sizeof(abi.AvbdParams)]))

    @classmethod
    def load(cls, path, device=0):
        """A new world from a snapshot file (avbd_world_load)."""
        h = C.c_void_p()
        _check(lib().avbd_world_load(os.fsencode(path), device, C.byref(h)), "avbd_world_load")
        with open(path, "rb") as f:
            head = f.read(abi.SNAPSHOT_HEADER_BYTES + C.sizeof(abi.AvbdParams))
        return cls._adopt(h, abi.AvbdParams.from_buffer_copy(head[abi.SNAPSHOT_HEADER_BYTES:]))

    def snapshot(self):
        """The whole world as snapshot bytes (avbd_world_snapshot)."""
        n = C.c_uint64()
        _check(lib().avbd_world_snapshot(self.h, None, 0, C.byref(n)), "avbd_world_snapshot")
        buf = C.create_string_buffer(n.value)
        _check(lib().avbd_world_snapshot(self.h, buf, n.value, C.byref(n)), "avbd_world_snapshot")
        return buf.raw[: n.value]

    def save(self, path):
        """Write the world's snapshot to a file (avbd_world_save)."""
        _check(lib().avbd_world_save(self.h, os.fsencode(path)), "avbd_world_save")

    def close(self):
        if getattr(self, "h", None):
            lib().avbd_world_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # PhysicsEngine::add_body
    def add_bodies(self, arr):
        arr = np.ascontiguousarray(arr, dtype=abi.BODY_DTYPE)
        first = C.c_uint32()
        _check(lib().avbd_world_add_bodies(self.h, abi.ptr(arr), len(arr), C.byref(first)), "add_bodies")
        return first.value

    def add_body(self, rec):
        return self.add_bodies(bodies_array([rec]))

    # PhysicsEngine::add_joint
    def add_hull(self, verts, faces=(), unit_inertia=(1.0, 1.0, 1.0)):
        """Register a convex hull; bodies of shape SHAPE_HULL name it by index."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float32).reshape(-1))
        f = np.ascontiguousarray(np.asarray(faces, dtype=np.uint32).reshape(-1))
        ui = np.ascontiguousarray(np.asarray(unit_inertia, dtype=np.float32))
        out = C.c_uint32()
        _check(lib().avbd_world_add_hull(self.h, abi.ptr(v), len(v) // 3, abi.ptr(f) if len(f) else None,
                                         len(f) // 3, abi.ptr(ui), C.byref(out)), "add_hull")
        return out.value

    def add_round(self, inner, unit_inertia=(1.0, 1.0, 1.0)):
        """A rounded shape (Shape::Round) around one primitive part; bodies of
        shape SHAPE_ROUND name the returned id."""
        ui = np.ascontiguousarray(np.asarray(unit_inertia, dtype=np.float32))
        out = C.c_uint32()
        _check(lib().avbd_world_add_round(self.h, C.byref(inner), abi.ptr(ui), C.byref(out)), "add_round")
        return out.value

    def add_compound(self, parts, unit_inertia=(1.0, 1.0, 1.0)):
        """A compound (Shape::Compound) of primitive parts; bodies of shape
        SHAPE_COMPOUND name the returned id."""
        ui = np.ascontiguousarray(np.asarray(unit_inertia, dtype=np.float32))
        out = C.c_uint32()
        arr = abi.parts_array(parts) if parts else None
        _check(lib().avbd_world_add_compound(self.h, arr, len(parts), abi.ptr(ui), C.byref(out)), "add_compound")
        return out.value

    def add_heightfield(self, heights, cell):
        """A heightfield (Heightfield::new) of rows x cols samples, rows along
        +Z; static bodies of shape SHAPE_HEIGHTFIELD name the returned id."""
        h = np.ascontiguousarray(np.asarray(heights, dtype=np.float32))
        rows, cols = h.shape
        out = C.c_uint32()
        _check(lib().avbd_world_add_heightfield(self.h, rows, cols, float(cell), abi.ptr(h), C.byref(out)),
               "add_heightfield")
        return out.value

    def add_trimesh(self, verts, tris):
        """A triangle mesh (TriMesh::from_indexed); static bodies of shape
        SHAPE_TRIMESH name the returned id."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float32).reshape(-1))
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.uint32).reshape(-1))
        out = C.c_uint32()
        _check(lib().avbd_world_add_trimesh(self.h, abi.ptr(v), len(v) // 3, abi.ptr(t), len(t) // 3, C.byref(out)),
               "add_trimesh")
        return out.value

    def remove_body(self, handle):
        """PhysicsEngine::remove_body: the last body takes over the handle."""
        _check(lib().avbd_world_remove_body(self.h, int(handle)), "remove_body")

    def remove_joint(self, handle):
        """PhysicsEngine::remove_joint: both bodies wake; later joint handles move down one."""
        _check(lib().avbd_world_remove_joint(self.h, int(handle)), "remove_joint")

    def wake_body(self, handle):
        """PhysicsEngine::wake_body: a sleeping body wakes (mass and inertia restored)."""
        _check(lib().avbd_world_wake_body(self.h, int(handle)), "wake_body")

    def add_joint(self, desc):
        hj = C.c_uint32()
        _check(lib().avbd_world_add_joint(self.h, C.byref(desc), C.byref(hj)), "add_joint")
        return hj.value

    @property
    def body_count(self):
        n = C.c_uint32()
        _check(lib().avbd_world_body_count(self.h, C.byref(n)), "body_count")
        return n.value

    # PhysicsEngine::step
    def step(self, dt):
        _check(lib().avbd_world_step(self.h, float(dt)), "step")

    def step_fixed(self, substeps=1):
        _check(lib().avbd_world_step_fixed(self.h, int(substeps)), "step_fixed")

    def step_graph(self, substeps=1):
        _check(lib().avbd_world_step_graph(self.h, int(substeps)), "step_graph")

    def sync(self):
        _check(lib().avbd_world_sync(self.h), "sync")

    # PhysicsEngine::get_body / get_body_mut, for all handles at once
    def bodies(self, first=0, n=None):
        if n is None:
            n = self.body_count - first
        out = np.zeros(n, dtype=abi.BODY_DTYPE)
        _check(lib().avbd_world_get_bodies(self.h, first, n, abi.ptr(out)), "get_bodies")
        return out

    def set_bodies(self, arr, first=0):
        arr = np.ascontiguousarray(arr, dtype=abi.BODY_DTYPE)
        _check(lib().avbd_world_set_bodies(self.h, first, len(arr), abi.ptr(arr)), "set_bodies")

    def step_timed(self, substeps, use_graph=True):
        """Device milliseconds of `substeps` substeps (CUDA events on the world's stream)."""
        ms = C.c_float()
        _check(lib().avbd_world_step_timed(self.h, int(substeps), int(use_graph), C.byref(ms)), "step_timed")
        return ms.value

    def flush_cache(self):
        """Evict the world's state from L2 (a 256 MB write on its stream)."""
        _check(lib().avbd_world_flush_cache(self.h), "flush_cache")

    def profile_substep(self):
        ms = np.zeros(9, np.float32)
        info = np.zeros(5, np.uint32)
        _check(lib().avbd_world_profile_substep(self.h, abi.ptr(ms), abi.ptr(info)), "profile_substep")
        names = ["wake_torque", "broadphase", "ccd", "discovery", "post_discovery", "colouring", "primal", "dual",
                 "finish"]
        return dict(zip(names, map(float, ms))), dict(zip(["colours", "primal_launches", "swept", "pairs",
                                                           "points"], map(int, info)))

    def graph_nodes(self):
        n = C.c_uint32()
        _check(lib().avbd_world_graph_nodes(self.h, C.byref(n)), "graph_nodes")
        return n.value

    def counters(self):
        c = abi.AvbdCounters()
        _check(lib().avbd_world_get_counters(self.h, C.byref(c)), "get_counters")
        return c

    def set_precision(self, fast):
        _check(lib().avbd_set_precision(self.h, int(bool(fast))), "set_precision")

    def set_work_order(self, by_work):
        _check(lib().avbd_set_work_order(self.h, int(bool(by_work))), "set_work_order")

    def set_occupancy(self, min_blocks):
        _check(lib().avbd_set_occupancy(self.h, int(min_blocks)), "set_occupancy")

    def set_joint_stiffness(self, k):
        """Finite joint stiffness (0: hard joints, the reference's)."""
        _check(lib().avbd_set_joint_stiffness(self.h, float(k)), "set_joint_stiffness")

    def set_broadphase(self, small_scene_max):
        _check(lib().avbd_set_broadphase(self.h, int(small_scene_max)), "set_broadphase")

    def set_sweep(self, rows):
        """Large scenes: 1 sweeps Morton-ordered cell rows, 0 one x-sweep (same candidates)."""
        _check(lib().avbd_set_sweep(self.h, int(rows)), "set_sweep")

    def set_tuning(self, lanes, block):
        _check(lib().avbd_set_tuning(self.h, int(lanes), int(block)), "set_tuning")

    def graph_nodes_emit(self):
        n = C.c_uint32()
        _check(lib().avbd_world_graph_nodes_emit(self.h, C.byref(n)), "graph_nodes_emit")
        return n.value

    # ---- events (PhysicsEngine::drain_contact_events / drain_trigger_events) ----
    def set_events(self, period):
        """0: events on the last substep of each call; k: every k substeps; -1: none."""
        _check(lib().avbd_set_events(self.h, int(period)), "set_events")

    def event_counts(self):
        out = np.zeros(4, dtype=np.uint32)
        _check(lib().avbd_world_event_counts(self.h, abi.ptr(out)), "event_counts")
        return dict(contact=int(out[0]), trigger=int(out[1]), contact_dropped=int(out[2]),
                    trigger_dropped=int(out[3]))

    def _drain(self, fn, dtype):
        n = C.c_uint32()
        cap = 1024
        while True:
            out = np.zeros(cap, dtype=dtype)
            rc = fn(self.h, abi.ptr(out), cap, C.byref(n))
            if rc == abi.AVBD_ERR_CAPACITY:
                cap = int(n.value)
                continue
            _check(rc, "drain events")
            return out[: n.value]

    def contact_events(self):
        return self._drain(lib().avbd_world_drain_contact_events, abi.CONTACT_EVENT_DTYPE)

    def trigger_events(self):
        return self._drain(lib().avbd_world_drain_trigger_events, abi.TRIGGER_EVENT_DTYPE)

    def colours(self):
        n = self.body_count
        out = np.zeros(n, dtype=np.int32)
        _check(lib().avbd_world_get_colours(self.h, abi.ptr(out), n), "get_colours")
        return out

    # checkpoint / restore of the whole solver state
    def export_state(self):
        nb, npr, nj = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(lib().avbd_world_state_sizes(self.h, C.byref(nb), C.byref(npr), C.byref(nj)), "state_sizes")
        st = dict(
            bodies=np.zeros(nb.value, dtype=abi.BODY_DTYPE),
            aux=np.zeros(nb.value, dtype=abi.AUX_DTYPE),
            pairs=np.zeros(npr.value, dtype=abi.PAIR_DTYPE),
            points=np.zeros(npr.value * abi.MAX_POINTS, dtype=abi.POINT_DTYPE),
            joints=np.zeros(nj.value, dtype=abi.JOINT_STATE_DTYPE),
        )
        _check(lib().avbd_world_export_state(self.h, abi.ptr(st["bodies"]), abi.ptr(st["aux"]),
                                             abi.ptr(st["pairs"]), abi.ptr(st["points"]),
                                             abi.ptr(st["joints"]), npr.value), "export_state")
        return st

    def import_state(self, st):
        _check(lib().avbd_world_import_state(self.h, abi.ptr(st["bodies"]), abi.ptr(st["aux"]),
                                             abi.ptr(st["pairs"]), abi.ptr(st["points"]), len(st["pairs"]),
                                             abi.ptr(st.get("joints"))), "import_state")

    # ---- differentiable rollouts ----
    def adjoint_forward(self, steps, substeps=1, checkpoint_every=10):
        """Advance `steps` steps, recording checkpoints for adjoint_backward."""
        _check(lib().avbd_adjoint_forward(self.h, int(steps), int(substeps), int(checkpoint_every)),
               "adjoint_forward")

    def adjoint_backward(self, grad_final):
        """dLoss/d(initial state) (bodies x 13) and dLoss/d(scene friction)
        (scenes) from dLoss/d(final state) (bodies x 13: position, quaternion
        x y z w, velocity, angular velocity)."""
        g = np.ascontiguousarray(grad_final, dtype=np.float32).reshape(-1, 13)
        n = self.body_count
        if g.shape[0] != n:
            raise ValueError("grad_final must have one row of 13 per body")
        out = np.zeros((n, 13), dtype=np.float32)
        ns = C.c_uint32()
        _check(lib().avbd_world_scene_count(self.h, C.byref(ns)), "scene_count")
        mu = np.zeros(ns.value, dtype=np.float32)
        _check(lib().avbd_adjoint_backward(self.h, abi.ptr(g), abi.ptr(out), abi.ptr(mu)), "adjoint_backward")
        return out, mu


    def adjoint_grad_joint_stiffness(self):
        """dLoss/d(joint stiffness) per scene from the last adjoint_backward."""
        ns = C.c_uint32()
        _check(lib().avbd_world_scene_count(self.h, C.byref(ns)), "scene_count")
        out = np.zeros(ns.value, dtype=np.float32)
        _check(lib().avbd_adjoint_grad_joint_stiffness(self.h, abi.ptr(out)), "adjoint_grad_joint_stiffness")
        return out

    def adjoint_trace(self):
        """Per substep of the last rollout (forward order): the largest body
        adjoint magnitude of the substep's start state and the body holding it."""
        n = C.c_int32()
        _check(lib().avbd_adjoint_trace(self.h, None, None, 0, C.byref(n)), "adjoint_trace")
        mx = np.zeros(n.value, dtype=np.float32)
        body = np.zeros(n.value, dtype=np.uint32)
        _check(lib().avbd_adjoint_trace(self.h, abi.ptr(mx), abi.ptr(body), n.value, C.byref(n)), "adjoint_trace")
        return mx, body

    def adjoint_timing(self):
        """(recompute ms, reverse ms) of the last adjoint_backward, device time."""
        ms = np.zeros(2, dtype=np.float32)
        _check(lib().avbd_adjoint_timing(self.h, abi.ptr(ms)), "adjoint_timing")
        return float(ms[0]), float(ms[1])


class Rollout:
    """A differentiable rollout as a forward/backward pair over one world:
    forward() advances and records, backward(dloss_dfinal) returns the
    gradients of the initial state and of each scene's friction; the joint
    stiffness gradient per scene follows from
    world.adjoint_grad_joint_stiffness()."""

    def __init__(self, world, steps, substeps=1, checkpoint_every=10):
        self.world = world
        self.steps, self.substeps, self.every = steps, substeps, checkpoint_every

    def forward(self):
        self.world.adjoint_forward(self.steps, self.substeps, self.every)
        return self.world.bodies()

    def backward(self, grad_final):
        return self.world.adjoint_backward(grad_final)
