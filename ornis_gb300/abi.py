"""ctypes mirror of include/ornis_avbd.h (the C ABI of the AVBD step).

Record layouts match the C structs field for field; numpy structured dtypes
with the same layout let whole arrays cross the boundary without copies.
"""
import ctypes as C

import numpy as np

AVBD_OK = 0
AVBD_ERR_INVALID_ARG = -1
AVBD_ERR_CAPACITY = -2
AVBD_ERR_DEVICE = -3
AVBD_ERR_TIMEOUT = -4
AVBD_ERR_NONFINITE = -5
AVBD_ERR_UNSUPPORTED = -6
AVBD_ERR_FORMAT = -7
AVBD_ERR_IO = -8
AVBD_ERR_JOINT_SELF = -10
AVBD_ERR_JOINT_HANDLES = -11
AVBD_ERR_JOINT_BAD_AXIS = -12
AVBD_ERR_JOINT_NONFINITE = -13
AVBD_ERR_JOINT_BAD_BOUNDS = -14
AVBD_ERR_JOINT_UNKNOWN_REF = -15

# limits of the allocation-free entry point (avbd_scene_step_static)
STATIC_MAX_BODIES = 128
STATIC_PAIR_CAP = 2048
STATIC_SCRATCH_BYTES = 3481600

SHAPE_SPHERE = 0
SHAPE_BOX = 1
SHAPE_CAPSULE = 2
SHAPE_HALFSPACE = 3
SHAPE_CYLINDER = 4
SHAPE_CONE = 5
SHAPE_HULL = 6
SHAPE_ROUND = 7
SHAPE_COMPOUND = 8
SHAPE_HEIGHTFIELD = 9
SHAPE_TRIMESH = 10

BODY_DYNAMIC = 0
BODY_STATIC = 1
BODY_KINEMATIC = 2

FLAG_TRIGGER = 1

JOINT_BALL = 0
JOINT_REVOLUTE = 1
JOINT_PRISMATIC = 2
JOINT_FIXED = 3
JOINT_DISTANCE = 4
JOINT_ROPE = 5
JOINT_SIXDOF = 6
JOINT_MOTOR = 7
JOINT_SPRING = 8
JOINT_WHEEL = 9
JOINT_GEAR = 10
MOTOR_VELOCITY, MOTOR_POSITION, MOTOR_SERVO = 0, 1, 2
MODEL_ACCELERATION, MODEL_FORCE = 0, 1

AXIS_FREE = 0
AXIS_LOCKED = 1
AXIS_LIMITED = 2

MAX_POINTS = 8

# avbd_set_tuning lanes value of the per-scene solve (one block per scene)
PRIMAL_SCENES = -1

F3 = C.c_float * 3
F4 = C.c_float * 4


class AvbdBody(C.Structure):
    _fields_ = [
        ("position", F3),
        ("orientation", F4),
        ("velocity", F3),
        ("angular_velocity", F3),
        ("torque", F3),
        ("mass", C.c_float),
        ("inv_mass", C.c_float),
        ("inertia", F3),
        ("restitution", C.c_float),
        ("friction", C.c_float),
        ("friction_transverse", C.c_float),
        ("rolling_friction", C.c_float),
        ("torsion_friction", C.c_float),
        ("shape", C.c_uint32),
        ("shape_params", F3),
        ("collision_layer", C.c_uint32),
        ("collision_mask", C.c_uint32),
        ("body_type", C.c_uint32),
        ("flags", C.c_uint32),
    ]


class AvbdJointDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32),
        ("body_a", C.c_uint32),
        ("body_b", C.c_uint32),
        ("local_anchor_a", F3),
        ("local_anchor_b", F3),
        ("local_axis_a", F3),
        ("local_axis_b", F3),
        ("has_limit", C.c_int32),
        ("limit_min", C.c_float),
        ("limit_max", C.c_float),
        ("has_motor", C.c_int32),
        ("motor_speed", C.c_float),
        ("motor_max", C.c_float),
        ("max_distance", C.c_float),
        ("axis_config", C.c_uint32 * 6),
        ("axis_min", C.c_float * 6),
        ("axis_max", C.c_float * 6),
        ("motor_linear", F3),
        ("motor_angular", F3),
        ("motor_max_force", C.c_float),
        ("motor_max_torque", C.c_float),
        ("motor_correction", C.c_float),
        ("spring_rest", C.c_float),
        ("spring_velocity", C.c_float),
        ("spring_stiffness", C.c_float),
        ("spring_damping", C.c_float),
        ("spring_max_force", C.c_float),
        ("spring_kind", C.c_uint32),
        ("spring_model", C.c_uint32),
        ("local_axle_a", F3),
        ("local_axle_b", F3),
        ("suspension_hz", C.c_float),
        ("suspension_damping", C.c_float),
        ("gear_joint_a", C.c_uint32),
        ("gear_joint_b", C.c_uint32),
        ("gear_ratio", C.c_float),
        ("reserved", C.c_uint32),
    ]


class AvbdShapePart(C.Structure):
    _fields_ = [
        ("shape", C.c_uint32),
        ("params", F3),
        ("border_radius", C.c_float),
        ("position", F3),
        ("orientation", F4),
    ]


def shape_part(shape, params, border_radius=0.0, position=(0.0, 0.0, 0.0), orientation=(0.0, 0.0, 0.0, 1.0)):
    """One part of a rounded or compound shape."""
    p = AvbdShapePart()
    p.shape = shape
    pp = list(map(float, params)) + [0.0] * (3 - len(params))
    p.params[:] = pp
    p.border_radius = float(border_radius)
    p.position[:] = list(map(float, position))
    p.orientation[:] = list(map(float, orientation))
    return p


def parts_array(parts):
    return (AvbdShapePart * len(parts))(*parts)


class AvbdParams(C.Structure):
    _fields_ = [
        ("gravity", F3),
        ("step_dt", C.c_float),
        ("iterations", C.c_int32),
        ("max_substeps", C.c_int32),
        ("enable_sleep", C.c_int32),
        ("enable_ccd", C.c_int32),
    ]


class AvbdBodyAux(C.Structure):
    _fields_ = [
        ("prev_position", F3),
        ("prev_orientation", F4),
        ("sleep_timer", C.c_float),
        ("asleep", C.c_uint32),
    ]


class AvbdPairState(C.Structure):
    _fields_ = [
        ("a", C.c_uint32),
        ("b", C.c_uint32),
        ("normal", F3),
        ("mu", C.c_float * 2),
        ("gap", C.c_float),
        ("npoints", C.c_uint32),
    ]


class AvbdPointState(C.Structure):
    _fields_ = [
        ("ra", F3),
        ("rb", F3),
        ("lam", F3),
        ("pen", F3),
        ("roll_lam", F3),
        ("stuck", C.c_uint32),
        ("matched", C.c_int32),
    ]


class AvbdJointState(C.Structure):
    _fields_ = [
        ("lam_l", F3),
        ("lam_a", F3),
        ("pen_l", F3),
        ("pen_a", F3),
        ("acc_lim", C.c_float),
        ("lim_dual", C.c_float),
        ("sacc", C.c_float * 6),
        ("gear_raw", C.c_float * 2),
        ("gear_cont", C.c_float * 2),
        ("gear_mem_set", C.c_uint32),
    ]


SNAPSHOT_FORMAT = 2
SNAPSHOT_HEADER_BYTES = 128
SNAPSHOT_MAGIC = b"ORNAVBD\0"
SNAPSHOT_SETTINGS_BYTES = 48       # launch tuning, precision, event period, joint stiffness, accumulator
SNAPSHOT_JOINT_RECORD_BYTES = 364  # a joint as the world holds it (assembly references resolved)
SNAPSHOT_EVENT_WORDS = 16


class AvbdSnapshotInfo(C.Structure):
    _fields_ = [("format", C.c_uint32), ("abi", C.c_uint32),
                ("nbodies", C.c_uint32), ("nscenes", C.c_uint32), ("npairs", C.c_uint32),
                ("njoints", C.c_uint32), ("nhulls", C.c_uint32),
                ("ntouch", C.c_uint32), ("ntrigger", C.c_uint32),
                ("ncontact_events", C.c_uint32), ("ntrigger_events", C.c_uint32), ("reserved", C.c_uint32),
                ("bytes", C.c_uint64), ("substeps", C.c_uint64)]


class AvbdCounters(C.Structure):
    _fields_ = [
        ("steps", C.c_uint64),
        ("pairs", C.c_uint64),
        ("points", C.c_uint64),
        ("candidates", C.c_uint64),
        ("colours", C.c_uint64),
        ("breakdowns", C.c_uint64),
        ("ccd_hits", C.c_uint64),
        ("sleeping", C.c_uint64),
        ("timeouts", C.c_uint64),
    ]


def _dtype_of(struct):
    """numpy structured dtype with the exact layout of a ctypes Structure."""
    fields = []
    for name, ctype in struct._fields_:
        if issubclass(ctype, C.Array):
            base = ctype._type_
            fields.append((name, np.dtype(base), (ctype._length_,)))
        else:
            fields.append((name, np.dtype(ctype)))
    dt = np.dtype(fields, align=True)
    assert dt.itemsize == C.sizeof(struct), (struct.__name__, dt.itemsize, C.sizeof(struct))
    return dt


class AvbdContactEvent(C.Structure):
    _fields_ = [
        ("body_a", C.c_uint32),
        ("body_b", C.c_uint32),
        ("kind", C.c_uint32),
        ("point", C.c_float * 3),
        ("normal", C.c_float * 3),
        ("approach_speed", C.c_float),
    ]


class AvbdTriggerEvent(C.Structure):
    _fields_ = [
        ("body_a", C.c_uint32),
        ("body_b", C.c_uint32),
        ("entered", C.c_uint32),
    ]


CONTACT_BEGIN, CONTACT_END, CONTACT_HIT = 0, 1, 2

BODY_DTYPE = _dtype_of(AvbdBody)
AUX_DTYPE = _dtype_of(AvbdBodyAux)
PAIR_DTYPE = _dtype_of(AvbdPairState)
POINT_DTYPE = _dtype_of(AvbdPointState)
JOINT_STATE_DTYPE = _dtype_of(AvbdJointState)
CONTACT_EVENT_DTYPE = _dtype_of(AvbdContactEvent)
TRIGGER_EVENT_DTYPE = _dtype_of(AvbdTriggerEvent)


def ptr(arr, ctype=C.c_void_p):
    """Raw pointer to a contiguous numpy array (None for None)."""
    if arr is None:
        return None
    assert arr.flags["C_CONTIGUOUS"]
    return C.cast(arr.ctypes.data, ctype)


def default_params(gravity=(0.0, -9.81, 0.0), step_dt=1.0 / 60.0, iterations=10,
                   max_substeps=4, enable_sleep=1, enable_ccd=1):
    p = AvbdParams()
    p.gravity[:] = [float(g) for g in gravity]
    p.step_dt = float(np.float32(step_dt))
    p.iterations = int(iterations)
    p.max_substeps = int(max_substeps)
    p.enable_sleep = int(enable_sleep)
    p.enable_ccd = int(enable_ccd)
    return p


def joint_desc(kind, a, b, anchor_a, anchor_b, axis_a=(1, 0, 0), axis_b=(1, 0, 0),
               limit=None, motor=None, max_distance=0.0, axes=None, drive=None, spring=None, wheel=None,
               gear=None):
    """A joint record.  limit = (min, max); motor = (target speed, max
    torque or force); axes (sixdof) = 6 entries, each "free", "locked" or
    (min, max), linear x y z then angular x y z; drive (free motor) =
    (linear target, angular target, max force, max torque, correction);
    spring = (rest, target velocity, stiffness, damping, max force, kind,
    model); wheel = (axle a, axle b, suspension Hz, damping ratio), axis_a/b
    being the suspension axes; gear = (joint a, joint b, ratio)."""
    d = AvbdJointDesc()
    d.kind = kind
    d.body_a = a
    d.body_b = b
    d.local_anchor_a[:] = list(map(float, anchor_a))
    d.local_anchor_b[:] = list(map(float, anchor_b))
    d.local_axis_a[:] = list(map(float, axis_a))
    d.local_axis_b[:] = list(map(float, axis_b))
    if limit is not None:
        d.has_limit = 1
        d.limit_min, d.limit_max = float(limit[0]), float(limit[1])
    if motor is not None:
        d.has_motor = 1
        d.motor_speed, d.motor_max = float(motor[0]), float(motor[1])
    d.max_distance = float(max_distance)
    for i, ax in enumerate(axes or ()):
        if ax == "free":
            d.axis_config[i] = AXIS_FREE
        elif ax == "locked":
            d.axis_config[i] = AXIS_LOCKED
        else:
            d.axis_config[i] = AXIS_LIMITED
            d.axis_min[i], d.axis_max[i] = float(ax[0]), float(ax[1])
    if drive is not None:
        lin, ang, fmax, tmax, corr = drive
        d.motor_linear[:] = list(map(float, lin))
        d.motor_angular[:] = list(map(float, ang))
        d.motor_max_force, d.motor_max_torque, d.motor_correction = float(fmax), float(tmax), float(corr)
    if spring is not None:
        rest, vel, k, c, fmax, kind_, model = spring
        d.spring_rest, d.spring_velocity, d.spring_stiffness = float(rest), float(vel), float(k)
        d.spring_damping, d.spring_max_force = float(c), float(fmax)
        d.spring_kind, d.spring_model = int(kind_), int(model)
    if wheel is not None:
        xa, xb, hz, zeta = wheel
        d.local_axle_a[:] = list(map(float, xa))
        d.local_axle_b[:] = list(map(float, xb))
        d.suspension_hz, d.suspension_damping = float(hz), float(zeta)
    if gear is not None:
        d.gear_joint_a, d.gear_joint_b, d.gear_ratio = int(gear[0]), int(gear[1]), float(gear[2])
    return d
