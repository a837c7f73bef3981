"""ctypes access to the CPU oracle (oracle/_build/libavbd_oracle.so).

Test infrastructure: the oracle is the checker for the CUDA path, never the
thing measured or shipped.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from ornis_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "libavbd_oracle.so")

REFERENCE = 0
COLOURED = 1
DUAL = 2  # use_double value of an f64 dual-number (forward-mode) world
DUAL_F32 = 3  # dual numbers whose values follow the f32 world bit for bit

# fields of OracleWorld.seed
F_POS, F_ROT, F_VEL, F_ANGVEL, F_FRICTION = 0, 1, 2, 3, 4

_lib = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = C.CDLL(ORACLE_SO)
        vp = C.c_void_p
        L.oracle_world_create.restype = vp
        L.oracle_world_create.argtypes = [C.POINTER(abi.AvbdParams), C.c_int, C.c_int, C.c_int]
        L.oracle_world_destroy.argtypes = [vp]
        L.oracle_set_faithful_scan.argtypes = [vp, C.c_int]
        L.oracle_set_split_sums.argtypes = [vp, C.c_int]
        L.oracle_add_bodies.argtypes = [vp, vp, C.c_uint32]
        L.oracle_add_joint.argtypes = [vp, C.POINTER(abi.AvbdJointDesc), C.POINTER(C.c_uint32)]
        L.oracle_step.argtypes = [vp, C.c_float]
        L.oracle_step_fixed.argtypes = [vp, C.c_int32]
        L.oracle_body_count.restype = C.c_uint32
        L.oracle_body_count.argtypes = [vp]
        L.oracle_get_bodies.argtypes = [vp, vp]
        L.oracle_get_state13.argtypes = [vp, vp]
        L.oracle_set_bodies.argtypes = [vp, vp, C.c_uint32]
        L.oracle_joint_count.restype = C.c_uint32
        L.oracle_joint_count.argtypes = [vp]
        L.oracle_pair_count.restype = C.c_uint32
        L.oracle_pair_count.argtypes = [vp]
        L.oracle_export_state.argtypes = [vp, vp, vp, vp, vp, vp]
        L.oracle_import_state.argtypes = [vp, vp, vp, vp, vp, C.c_uint32, vp]
        L.oracle_get_colours.argtypes = [vp, vp]
        L.oracle_get_counters.argtypes = [vp, C.POINTER(abi.AvbdCounters)]
        L.oracle_stamp_row.argtypes = [vp, vp, vp, C.c_float, C.c_float, vp, C.c_float]
        L.oracle_solve_6x6.restype = C.c_int
        L.oracle_solve_6x6.argtypes = [vp, vp, vp]
        L.oracle_tangent_basis.argtypes = [vp, vp, vp]
        L.oracle_shape_inertia.argtypes = [C.c_uint32, vp, C.c_float, vp]
        L.oracle_colour_hash.restype = C.c_uint32
        L.oracle_colour_hash.argtypes = [C.c_uint32]
        L.oracle_generate_pairs.argtypes = [vp]
        L.oracle_gap_c0.restype = C.c_double
        L.oracle_gap_c0.argtypes = [vp, C.c_uint32, C.c_uint32]
        L.oracle_body_new.argtypes = [C.c_uint32, vp, vp, C.c_float, C.POINTER(abi.AvbdBody)]
        L.oracle_set_emit_period.argtypes = [vp, C.c_int32]
        L.oracle_remove_body.argtypes = [vp, C.c_uint32]
        L.oracle_remove_joint.argtypes = [vp, C.c_uint32]
        L.oracle_wake_body.argtypes = [vp, C.c_uint32]
        L.oracle_add_heightfield.restype = C.c_int
        L.oracle_add_heightfield.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_float, vp, C.POINTER(C.c_uint32)]
        L.oracle_add_trimesh.restype = C.c_int
        L.oracle_add_trimesh.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32, C.POINTER(C.c_uint32)]
        L.oracle_add_ext.restype = C.c_int
        L.oracle_add_ext.argtypes = [vp, C.c_int, vp, C.c_uint32, vp, C.POINTER(C.c_uint32)]
        L.oracle_add_hull.restype = C.c_uint32
        L.oracle_add_hull.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32, vp]
        L.oracle_convex_distance.argtypes = [vp, C.c_uint32, C.c_uint32, vp]
        L.oracle_shape_distance.argtypes = [vp, C.c_uint32, C.c_uint32, vp]
        L.oracle_drain_contact_events.restype = C.c_uint32
        L.oracle_drain_contact_events.argtypes = [vp, vp, C.c_uint32]
        L.oracle_drain_trigger_events.restype = C.c_uint32
        L.oracle_drain_trigger_events.argtypes = [vp, vp, C.c_uint32]
        L.oracle_dual_seed.argtypes = [vp, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_double]
        L.oracle_dual_freeze_frames.argtypes = [vp, C.c_int]
        L.oracle_dual_tangents.argtypes = [vp, vp]
        L.oracle_set_joint_stiffness.argtypes = [vp, C.c_float]
        L.oracle_dual_seed_joint_stiffness.argtypes = [vp, C.c_int, C.c_double]
        _lib = L
    return _lib


def f32(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float32))


def body_new(shape, params, position, mass):
    """RigidBody::new_* through the oracle's restatement of the constructors."""
    b = abi.AvbdBody()
    p = f32(list(params) + [0.0] * (3 - len(params)))
    pos = f32(position)
    rc = lib().oracle_body_new(shape, abi.ptr(p), abi.ptr(pos), float(mass), C.byref(b))
    assert rc == 0, rc
    return b


def bodies_to_array(bodies):
    arr = np.zeros(len(bodies), dtype=abi.BODY_DTYPE)
    C.memmove(arr.ctypes.data, (abi.AvbdBody * len(bodies))(*bodies), arr.nbytes)
    return arr


class OracleWorld:
    """One single-scene oracle engine (Reference or Coloured sweep)."""

    def __init__(self, params=None, mode=REFERENCE, use_double=False, threads=1):
        self.params = params if params is not None else abi.default_params()
        self.h = lib().oracle_world_create(C.byref(self.params), mode, int(use_double), int(threads))

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_world_destroy(self.h)
            self.h = None

    def faithful_scan(self, on=True):
        lib().oracle_set_faithful_scan(self.h, int(on))

    def split_sums(self, on=True):
        """Sum each pair's rows before they join the body's system (the
        device's split primal launch)."""
        lib().oracle_set_split_sums(self.h, int(on))

    def add_bodies(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.dtype == abi.BODY_DTYPE
        assert lib().oracle_add_bodies(self.h, abi.ptr(arr), len(arr)) == 0

    def add_joint(self, desc):
        h = C.c_uint32(0)
        rc = lib().oracle_add_joint(self.h, C.byref(desc), C.byref(h))
        return rc, h.value

    def step(self, dt):
        lib().oracle_step(self.h, float(dt))

    def step_fixed(self, n=1):
        lib().oracle_step_fixed(self.h, int(n))

    @property
    def nbodies(self):
        return lib().oracle_body_count(self.h)

    def bodies(self):
        out = np.zeros(self.nbodies, dtype=abi.BODY_DTYPE)
        lib().oracle_get_bodies(self.h, abi.ptr(out))
        return out

    def state13(self):
        out = np.zeros((self.nbodies, 13), dtype=np.float64)
        lib().oracle_get_state13(self.h, abi.ptr(out))
        return out

    def set_bodies(self, arr):
        arr = np.ascontiguousarray(arr)
        assert lib().oracle_set_bodies(self.h, abi.ptr(arr), len(arr)) == 0

    def export_state(self):
        n = self.nbodies
        npairs = lib().oracle_pair_count(self.h)
        bodies = np.zeros(n, dtype=abi.BODY_DTYPE)
        aux = np.zeros(n, dtype=abi.AUX_DTYPE)
        pairs = np.zeros(npairs, dtype=abi.PAIR_DTYPE)
        points = np.zeros(npairs * abi.MAX_POINTS, dtype=abi.POINT_DTYPE)
        joints = np.zeros(lib().oracle_joint_count(self.h), dtype=abi.JOINT_STATE_DTYPE)
        lib().oracle_export_state(self.h, abi.ptr(bodies), abi.ptr(aux), abi.ptr(pairs), abi.ptr(points),
                                  abi.ptr(joints))
        return dict(bodies=bodies, aux=aux, pairs=pairs, points=points, joints=joints)

    def import_state(self, st):
        lib().oracle_import_state(self.h, abi.ptr(st["bodies"]), abi.ptr(st["aux"]), abi.ptr(st["pairs"]),
                                  abi.ptr(st["points"]), len(st["pairs"]), abi.ptr(st.get("joints")))

    def generate_pairs(self):
        lib().oracle_generate_pairs(self.h)

    def gap_c0(self, pi, qi):
        return lib().oracle_gap_c0(self.h, pi, qi)

    def colours(self):
        out = np.zeros(self.nbodies, dtype=np.int32)
        lib().oracle_get_colours(self.h, abi.ptr(out))
        return out

    def counters(self):
        c = abi.AvbdCounters()
        lib().oracle_get_counters(self.h, C.byref(c))
        return c

    def add_hull(self, verts, faces=(), unit_inertia=(1.0, 1.0, 1.0)):
        v = f32(np.asarray(verts).reshape(-1))
        fc = np.ascontiguousarray(np.asarray(faces, dtype=np.uint32).reshape(-1))
        ui = f32(unit_inertia)
        return lib().oracle_add_hull(self.h, abi.ptr(v), len(v) // 3, abi.ptr(fc) if len(fc) else None,
                                     len(fc) // 3, abi.ptr(ui))

    def add_round(self, inner, unit_inertia=(1.0, 1.0, 1.0)):
        """A rounded shape around one primitive part; returns (status, id)."""
        out = C.c_uint32()
        rc = lib().oracle_add_ext(self.h, 0, C.byref(inner), 1, abi.ptr(f32(unit_inertia)), C.byref(out))
        return rc, out.value

    def add_heightfield(self, heights, cell):
        """A heightfield of rows x cols samples (rows along +Z); returns (status, id)."""
        h = f32(np.asarray(heights))
        rows, cols = h.shape
        out = C.c_uint32()
        rc = lib().oracle_add_heightfield(self.h, rows, cols, float(cell), abi.ptr(np.ascontiguousarray(h.reshape(-1))),
                                          C.byref(out))
        return rc, out.value

    def add_trimesh(self, verts, tris):
        """A triangle mesh; returns (status, id)."""
        v = f32(np.asarray(verts).reshape(-1))
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.uint32).reshape(-1))
        out = C.c_uint32()
        rc = lib().oracle_add_trimesh(self.h, abi.ptr(v), len(v) // 3, abi.ptr(t), len(t) // 3, C.byref(out))
        return rc, out.value

    def add_compound(self, parts, unit_inertia=(1.0, 1.0, 1.0)):
        """A compound of primitive parts; returns (status, id)."""
        out = C.c_uint32()
        arr = abi.parts_array(parts) if parts else None
        rc = lib().oracle_add_ext(self.h, 1, arr, len(parts), abi.ptr(f32(unit_inertia)), C.byref(out))
        return rc, out.value

    def convex_distance(self, ia, ib):
        out = np.zeros(10, dtype=np.float32)
        lib().oracle_convex_distance(self.h, ia, ib, abi.ptr(out))
        return float(out[0]), out[1:4].copy(), out[4:7].copy(), out[7:10].copy()

    def shape_distance(self, ia, ib):
        out = np.zeros(10, dtype=np.float32)
        lib().oracle_shape_distance(self.h, ia, ib, abi.ptr(out))
        return float(out[0]), out[4:7].copy(), out[7:10].copy()

    def remove_body(self, handle):
        lib().oracle_remove_body(self.h, int(handle))

    def remove_joint(self, handle):
        lib().oracle_remove_joint(self.h, int(handle))

    def wake_body(self, handle):
        lib().oracle_wake_body(self.h, int(handle))

    def set_emit_period(self, period):
        lib().oracle_set_emit_period(self.h, int(period))

    def contact_events(self, cap=1 << 20):
        out = np.zeros(cap, dtype=abi.CONTACT_EVENT_DTYPE)
        n = lib().oracle_drain_contact_events(self.h, abi.ptr(out), cap)
        return out[:n]

    def trigger_events(self, cap=1 << 16):
        out = np.zeros(cap, dtype=abi.TRIGGER_EVENT_DTYPE)
        n = lib().oracle_drain_trigger_events(self.h, abi.ptr(out), cap)
        return out[:n]

    # ---- dual-number worlds (use_double=DUAL) ----
    def seed(self, body, field, comp, direction, value=1.0):
        """d(field[comp] of body)/d(direction) = value in the initial state."""
        assert lib().oracle_dual_seed(self.h, int(body), int(field), int(comp), int(direction), float(value)) == 0

    def set_joint_stiffness(self, k):
        assert lib().oracle_set_joint_stiffness(self.h, float(k)) == 0

    def seed_joint_stiffness(self, direction, value=1.0):
        assert lib().oracle_dual_seed_joint_stiffness(self.h, int(direction), float(value)) == 0

    def freeze_frames(self, on=True):
        assert lib().oracle_dual_freeze_frames(self.h, int(on)) == 0

    def tangents(self):
        """(bodies, 13, directions): derivatives of pos, quat, vel, angvel."""
        nd = lib().oracle_dual_dirs()
        out = np.zeros((self.nbodies, 13, nd), dtype=np.float64)
        assert lib().oracle_dual_tangents(self.h, abi.ptr(out)) == 0
        return out
