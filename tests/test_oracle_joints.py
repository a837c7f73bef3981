"""The joint kinds beyond Ball and Revolute on the oracle: the reference's
behavioural gates (crates/physics/tests/avbd_engine.rs) restated — hinge
motor (:552-596), prismatic slider on its line and at its limit (:598-646),
prismatic motor (:782-822), fixed weld (:891-938), distance rod (:940-968),
six-DOF all locked / free axis / angular limit (:1452-1556), the free motor
(crates/physics/tests/motor_joint.rs:90-110), the spring oscillator
(p6_rope_spring_motor.rs:193-216), the wheel's axle motor and suspension
(avbd_engine.rs:969-1061), the gears (a 2:1 hinge pair, :1359-1450; two
sliders through a teleport, :822-889) — plus a rope that never
exceeds its length, the free motor's angular drive and budget, and the
admission errors of validate_joint (migration.rs:160-356).  Reference order, dt 1/60, 10 iterations."""
import math

import numpy as np
import pytest

from ornis_gb300 import abi

import oracle_api as O

DT = 1.0 / 60.0


def world(recs, gravity=(0.0, -9.81, 0.0)):
    w = O.OracleWorld(abi.default_params(gravity=gravity))
    w.add_bodies(O.bodies_to_array(recs))
    return w


def add(w, d):
    rc, h = w.add_joint(d)
    assert rc == 0, rc
    return h


def z_twist(q):  # avbd_engine.rs:502-504
    return 2.0 * math.asin(float(q[2]))


def test_hinge_motor_spins_up():
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.05], [0, 0, 0], 0.0)
    anchor.flags = abi.FLAG_TRIGGER
    w = world([anchor, O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_REVOLUTE, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 1], [0, 0, 1], motor=(3.0, 20.0)))
    for _ in range(300):
        w.step(DT)
    mean = 0.0
    for _ in range(60):
        w.step(DT)
        mean += w.bodies()["angular_velocity"][1][2]
    assert abs(mean / 60.0 - 3.0) < 0.6


def test_prismatic_slider_holds_line_and_limit():
    w = world([O.body_new(abi.SHAPE_BOX, [0.25, 0.25, 0.25], [0, 0, 0], 0.0),
               O.body_new(abi.SHAPE_SPHERE, [0.25], [0, -2.9, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [0, 1, 0], [0, 1, 0], [0, 1, 0], limit=(-2.0, 0.0)))
    for _ in range(300):
        w.step(DT)
        p = w.bodies()["position"][1]
        assert abs(p[0]) < 0.08 and abs(p[2]) < 0.08, p
    assert -5.4 < w.bodies()["position"][1][1] < -4.4


def test_prismatic_motor_drives():
    w = world([O.body_new(abi.SHAPE_BOX, [0.25, 0.25, 0.25], [0, 0, 0], 0.0),
               O.body_new(abi.SHAPE_SPHERE, [0.25], [1, 0, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [-1, 0, 0], [1, 0, 0], [1, 0, 0], motor=(2.0, 50.0)))
    for _ in range(300):
        w.step(DT)
    b = w.bodies()
    assert abs(b["velocity"][1][0] - 2.0) < 0.4
    assert abs(b["position"][1][1]) < 0.15 and abs(b["position"][1][2]) < 0.1


def test_fixed_weld_holds():
    w = world([O.body_new(abi.SHAPE_BOX, [5, 1, 5], [0, -1, 0], 0.0),
               O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [-0.5, 3, 0], 1.0),
               O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0.5, 3, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_FIXED, 1, 2, [0.5, 0, 0], [-0.5, 0, 0]))
    for _ in range(300):
        w.step(DT)
    b = w.bodies()
    assert abs(np.linalg.norm(b["position"][2] - b["position"][1]) - 1.0) < 0.15
    assert b["position"][1][1] > 0.2 and b["position"][2][1] > 0.2


def test_distance_rod_holds_length():
    w = world([O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 0.0),
               O.body_new(abi.SHAPE_SPHERE, [0.25], [2, 0, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_DISTANCE, 0, 1, [0, 0, 0], [0, 0, 0]))
    swung = False
    for _ in range(300):
        w.step(DT)
        p = w.bodies()["position"][1]
        assert abs(np.linalg.norm(p) - 2.0) < 0.25
        swung |= p[1] < -0.5
    assert swung


def test_rope_never_stretches_past_its_length():
    # a bob 1 m from the anchor on a 2 m rope: it falls slack, then the rope
    # catches it and it swings on a 2 m radius
    w = world([O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 0.0),
               O.body_new(abi.SHAPE_SPHERE, [0.25], [1, 0, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_ROPE, 0, 1, [0, 0, 0], [0, 0, 0], max_distance=2.0))
    longest = 0.0
    for _ in range(300):
        w.step(DT)
        longest = max(longest, float(np.linalg.norm(w.bodies()["position"][1])))
    assert 1.9 < longest < 2.25


def test_sixdof_all_locked_behaves_like_fixed():
    w = world([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 1.0),
               O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 1.4, 0], 1.0)])
    add(w, abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0], axes=["locked"] * 6))
    for _ in range(180):
        w.step(DT)
    b = w.bodies()
    assert abs((b["position"][1] - b["position"][0])[1] - 1.4) < 0.05


def test_sixdof_free_axis_slides_but_locked_holds():
    w = world([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 1.0),
               O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [1, 0, 0], 1.0)], gravity=(0, 0, 0))
    add(w, abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0],
                          axes=["free", "locked", "locked", "locked", "locked", "locked"]))
    b = w.bodies()
    b["velocity"][1] = [3.0, 1.0, 0.0]
    w.set_bodies(b)
    for _ in range(60):
        w.step(DT)
    b = w.bodies()
    d = b["position"][1] - b["position"][0]
    assert d[0] > 1.5 and abs(d[1]) < 0.08


def test_sixdof_angular_limit_blocks_spin():
    w = world([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 0.0),
               O.body_new(abi.SHAPE_BOX, [0.4, 0.4, 0.4], [0, 0, 0], 1.0)], gravity=(0, 0, 0))
    add(w, abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0],
                          axes=["locked"] * 5 + [(-0.2, 0.2)]))
    b = w.bodies()
    b["angular_velocity"][1] = [0.0, 0.0, 8.0]
    w.set_bodies(b)
    for _ in range(120):
        w.step(DT)
    assert abs(z_twist(w.bodies()["orientation"][1])) < 0.4


def _motor_scene():
    """A box resting on a static floor box, driven along +x by a free motor
    from a static anchor above (motor_joint.rs:38-57, :90-110)."""
    floor = O.body_new(abi.SHAPE_BOX, [10.0, 0.5, 10.0], [0, -0.5, 0], 0.0)
    block = O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0.5, 0], 1.0)
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 5, 0], 0.0)
    drive = abi.joint_desc(abi.JOINT_MOTOR, 2, 1, [0, 0, 0], [0, 0, 0],
                           drive=((2.0, 0.0, 0.0), (0.0, 0.0, 0.0), 8.0, 10.0, 0.0))
    return [floor, block, anchor], drive


def test_free_motor_drives_box_against_friction():
    # avbd_motor_drives_box_to_target_against_friction (motor_joint.rs:90-110)
    recs, drive = _motor_scene()
    w = world(recs)
    add(w, drive)
    for _ in range(300):
        w.step(DT)
    v = w.bodies()["velocity"][1]
    assert abs(v[0] - 2.0) < 0.4, v


def test_free_motor_spins_to_angular_target_within_budget():
    """No gravity: the angular drive reaches its target, and a starved
    budget changes the rate by at most max_torque dt through the body's
    inverse inertia per step."""
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 5, 0], 0.0)
    ball = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0, 0], 1.0)
    w = world([anchor, ball], gravity=(0.0, 0.0, 0.0))
    add(w, abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0],
                          drive=((0.0, 0.0, 0.0), (0.0, 3.0, 0.0), 0.0, 50.0, 0.0)))
    for _ in range(30):
        w.step(DT)
    assert abs(w.bodies()["angular_velocity"][1][1] - 3.0) < 1e-3
    w2 = world([anchor, ball], gravity=(0.0, 0.0, 0.0))
    add(w2, abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0],
                           drive=((0.0, 0.0, 0.0), (0.0, 3.0, 0.0), 0.0, 0.01, 0.0)))
    w2.step(DT)
    inertia = 0.4 * 1.0 * 0.5 ** 2  # solid sphere
    assert 0.0 < w2.bodies()["angular_velocity"][1][1] <= 0.01 * DT / inertia * 1.001


def test_free_motor_bodies_do_not_collide():
    # rows.rs:434-474: the free motor is on the no-collide list
    a = O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0.5, 0], 1.0)
    b = O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0.3, 0.5, 0], 1.0)
    w = world([a, b], gravity=(0.0, 0.0, 0.0))
    add(w, abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0],
                          drive=((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 1.0, 0.3)))
    w.step(DT)
    assert w.counters().pairs == 0


def _spring_scene(model=abi.MODEL_ACCELERATION, stiffness=30.0, damping=6.0):
    """A ball on a spring stretched to 2.5 times its rest length from a static
    anchor, zero gravity (p6_rope_spring_motor.rs:120-160, :193-216)."""
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 0.0)
    bob = O.body_new(abi.SHAPE_SPHERE, [0.2], [0, -2.5, 0], 1.0)
    d = abi.joint_desc(abi.JOINT_SPRING, 0, 1, [0, 0, 0], [0, 0.5, 0],
                       spring=(1.0, 0.0, stiffness, damping, 1e6, abi.MOTOR_POSITION, model))
    return [anchor, bob], d


def spring_length(w):
    b = w.bodies()
    q = b["orientation"][1]
    qv, qw = q[:3].astype(np.float64), float(q[3])
    lb = np.array([0.0, 0.5, 0.0])
    rot = lb + 2.0 * qw * np.cross(qv, lb) + 2.0 * np.cross(qv, np.cross(qv, lb))
    return float(np.linalg.norm(b["position"][1] + rot - b["position"][0]))


@pytest.mark.parametrize("model", [abi.MODEL_ACCELERATION, abi.MODEL_FORCE])
def test_spring_oscillator_settles_at_rest_length(model):
    # avbd_spring_oscillator_settles_at_rest_length (p6_rope_spring_motor.rs:193-216)
    recs, d = _spring_scene(model)
    w = world(recs, gravity=(0.0, 0.0, 0.0))
    add(w, d)
    lengths = []
    for _ in range(600):
        w.step(DT)
        lengths.append(spring_length(w))
    assert abs(lengths[-1] - 1.0) < 0.1, lengths[-1]
    assert np.linalg.norm(w.bodies()["velocity"][1]) < 0.4
    assert min(lengths) < 1.2  # it oscillated through its rest length


def test_spring_damper_only_slows_without_centering():
    recs, d = _spring_scene(stiffness=0.0, damping=4.0)
    w = world(recs, gravity=(0.0, 0.0, 0.0))
    b = w.bodies()
    b["velocity"][1] = [0.0, -3.0, 0.0]
    w.set_bodies(b)
    add(w, d)
    for _ in range(120):
        w.step(DT)
    v = np.linalg.norm(w.bodies()["velocity"][1])
    assert 0.0 < v < 1.5
    assert spring_length(w) > 2.0  # no rest-length pull


def _wheel_motor_scene():
    """A wheel spun about its z axle by a motor, zero gravity
    (avbd_engine.rs:1020-1061)."""
    anchor = O.body_new(abi.SHAPE_BOX, [0.2, 0.2, 0.2], [0, 0, 0], 0.0)
    wheel = O.body_new(abi.SHAPE_BOX, [0.2, 0.2, 0.1], [0, -0.5, 0], 1.0)
    d = abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 0], motor=(6.0, 50.0),
                       wheel=((0, 0, 1), (0, 0, 1), 2.0, 0.5))
    return [anchor, wheel], d


def _wheel_suspension_scene(hz=3.0):
    """A 2 kg chassis sprung over a 1 kg wheel, both falling
    (avbd_engine.rs:969-1017)."""
    chassis = O.body_new(abi.SHAPE_BOX, [0.5, 0.2, 0.3], [0, 1, 0], 2.0)
    wheel = O.body_new(abi.SHAPE_BOX, [0.25, 0.25, 0.15], [0, 0, 0], 1.0)
    d = abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 0],
                       wheel=((0, 0, 1), (0, 0, 1), hz, 0.7))
    return [chassis, wheel], d


def test_wheel_motor_spins_axle():
    recs, d = _wheel_motor_scene()
    w = world(recs, gravity=(0.0, 0.0, 0.0))
    add(w, d)
    for _ in range(240):
        w.step(DT)
    assert abs(w.bodies()["angular_velocity"][1][2] - 6.0) < 1.5


@pytest.mark.parametrize("hz", [3.0, 0.0])
def test_wheel_suspension_holds_chassis(hz):
    # avbd_wheel_suspension_holds_chassis; a zero frequency is the rigid row
    recs, d = _wheel_suspension_scene(hz)
    w = world(recs)
    add(w, d)
    for _ in range(300):
        w.step(DT)
    p = w.bodies()["position"]
    sep = p[0][1] - p[1][1]
    assert 0.5 <= sep <= 1.1, sep
    if hz == 0.0:
        assert abs(sep - 1.0) < 0.05, sep


def _gear_hinge_scene():
    """Motor-driven hinge A coupled 2:1 to a free hinge B on a static mount,
    no gravity (avbd_engine.rs:1359-1410)."""
    recs = [O.body_new(abi.SHAPE_BOX, [0.2, 0.2, 0.2], [0, 0, 0], 0.0),
            O.body_new(abi.SHAPE_BOX, [0.1, 0.6, 0.1], [0, 0.6, 0], 1.0),
            O.body_new(abi.SHAPE_BOX, [0.1, 0.6, 0.1], [1, 0.6, 0], 1.0)]
    joints = [abi.joint_desc(abi.JOINT_REVOLUTE, 0, 1, [0, 0, 0], [0, -0.6, 0], [0, 0, 1], [0, 0, 1],
                             motor=(1.5, 20.0)),
              abi.joint_desc(abi.JOINT_REVOLUTE, 0, 2, [1, 0, 0], [0, -0.6, 0], [0, 0, 1], [0, 0, 1]),
              abi.joint_desc(abi.JOINT_GEAR, 1, 2, [0, 0, 0], [0, 0, 0], gear=(0, 1, 2.0))]
    return recs, joints


def _gear_slider_scene():
    """Two sliders on a static anchor, the first motor-driven, coupled with
    ratio -1 (co-directional travel; avbd_engine.rs:822-855)."""
    recs = [O.body_new(abi.SHAPE_BOX, [0.25, 0.25, 0.25], [0, 0, 0], 0.0),
            O.body_new(abi.SHAPE_SPHERE, [0.25], [1, 0, 0], 1.0),
            O.body_new(abi.SHAPE_SPHERE, [0.25], [3, 0, 0], 1.0)]
    joints = [abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [1, 0, 0], [0, 0, 0], [1, 0, 0], [1, 0, 0],
                             motor=(2.0, 50.0)),
              abi.joint_desc(abi.JOINT_PRISMATIC, 0, 2, [3, 0, 0], [0, 0, 0], [1, 0, 0], [1, 0, 0]),
              abi.joint_desc(abi.JOINT_GEAR, 1, 2, [0, 0, 0], [0, 0, 0], gear=(0, 1, -1.0))]
    return recs, joints


def atan_twist(q):  # the folding-free twist of avbd_engine.rs:1431-1433
    return 2.0 * math.atan2(float(q[2]), float(q[3]))


def wrap(x):
    return (x + math.pi) % (2.0 * math.pi) - math.pi


def test_gear_couples_hinges_two_to_one():
    recs, joints = _gear_hinge_scene()
    w = world(recs, gravity=(0.0, 0.0, 0.0))
    for d in joints:
        add(w, d)
    ua = ub = pa = pb = 0.0
    for i in range(180):
        w.step(DT)
        q = w.bodies()["orientation"]
        xa, xb = atan_twist(q[1]), atan_twist(q[2])
        if i == 0:
            pa, pb = xa, xb
        ua += wrap(xa - pa)
        ub += wrap(xb - pb)
        pa, pb = xa, xb
    assert abs(z_twist(w.bodies()["orientation"][1])) > 0.5
    assert abs(ua + 2.0 * ub) < 0.35 * max(abs(ua), 1.0), (ua, ub)
    assert abs(ua) > math.pi  # the motor turned hinge A past a half turn: the unwrap held


def test_gear_sliders_travel_together_through_a_teleport():
    recs, joints = _gear_slider_scene()
    w = world(recs)
    for d in joints:
        add(w, d)
    for _ in range(120):
        w.step(DT)
    b = w.bodies()
    b["position"][1][0] += 4.0  # a host teleport: meters never wrap like angles
    w.set_bodies(b)
    for _ in range(120):
        w.step(DT)
    p = w.bodies()["position"]
    sa, sb = p[1][0] - 1.0, p[2][0] - 3.0
    assert sa > 2.0 and sb > 2.0, (sa, sb)
    assert abs(sa - sb) < 0.6, (sa, sb)


def test_gear_goes_with_its_joint():
    """Removing a coupled joint removes the gear (joint_remap,
    migration.rs:74-115); the survivors move down."""
    recs, joints = _gear_hinge_scene()
    w = world(recs, gravity=(0.0, 0.0, 0.0))
    for d in joints:
        add(w, d)
    add(w, abi.joint_desc(abi.JOINT_GEAR, 1, 2, [0, 0, 0], [0, 0, 0], gear=(1, 0, 0.5)))
    w.remove_joint(1)
    assert len(w.export_state()["joints"]) == 1
    recs, joints = _gear_hinge_scene()
    w = world(recs, gravity=(0.0, 0.0, 0.0))
    for d in joints:
        add(w, d)
    w.remove_body(2)  # hinge B's body: the hinge and the gear go
    assert len(w.export_state()["joints"]) == 1


def test_joint_admission_errors():
    w = world([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 1.0),
               O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [2, 0, 0], 1.0)])
    nan = float("nan")
    cases = [
        (abi.joint_desc(abi.JOINT_BALL, 0, 1, [nan, 0, 0], [0, 0, 0]), abi.AVBD_ERR_JOINT_BAD_AXIS),
        (abi.joint_desc(abi.JOINT_REVOLUTE, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 1], [0, 0, 1], limit=(1.0, -1.0)),
         abi.AVBD_ERR_JOINT_BAD_BOUNDS),
        (abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [0, 0, 0], [1, 0, 0], [1, 0, 0], motor=(nan, 1.0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 0], [1, 0, 0]),
         abi.AVBD_ERR_JOINT_BAD_AXIS),
        (abi.joint_desc(abi.JOINT_ROPE, 0, 1, [0, 0, 0], [0, 0, 0], max_distance=0.0), abi.AVBD_ERR_JOINT_BAD_BOUNDS),
        (abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0], axes=["locked"] * 5 + [(0.3, -0.3)]),
         abi.AVBD_ERR_JOINT_BAD_BOUNDS),
    ]
    inf = float("inf")
    cases += [
        (abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((nan, 0, 0), (0, 0, 0), 1.0, 1.0, 0.0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((0, 0, 0), (0, 0, 0), -1.0, 1.0, 0.0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((0, 0, 0), (0, 0, 0), 1.0, inf, 0.0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((0, 0, 0), (0, 0, 0), 1.0, 1.0, 1.5)),
         abi.AVBD_ERR_JOINT_BAD_BOUNDS),
    ]
    P = abi.MOTOR_POSITION
    cases += [
        (abi.joint_desc(abi.JOINT_SPRING, 0, 1, [0, 0, 0], [0, 0, 0], spring=(nan, 0, 1, 1, 1, P, 0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_SPRING, 0, 1, [0, 0, 0], [0, 0, 0], spring=(1, 0, -1, 1, 1, P, 0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_SPRING, 0, 1, [0, 0, 0], [0, 0, 0], spring=(1, 0, 1, inf, 1, P, 0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_SPRING, 0, 1, [0, 0, 0], [0, 0, 0], spring=(1, 0, 1, 1, -2, P, 0)),
         abi.AVBD_ERR_JOINT_NONFINITE),
    ]
    # gears (mod.rs:1329-1404; avbd_engine.rs:183-255): a non-finite ratio,
    # a joint that does not exist, a joint that is neither hinge nor slide
    cases += [
        (abi.joint_desc(abi.JOINT_GEAR, 0, 1, [0, 0, 0], [0, 0, 0], gear=(0, 0, nan)), abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_GEAR, 1, 1, [0, 0, 0], [0, 0, 0], gear=(7, 8, 2.0)), abi.AVBD_ERR_JOINT_SELF),
        (abi.joint_desc(abi.JOINT_GEAR, 0, 1, [0, 0, 0], [0, 0, 0], gear=(7, 8, 2.0)),
         abi.AVBD_ERR_JOINT_UNKNOWN_REF),
    ]
    Wz = ((0, 0, 1), (0, 0, 1), 2.0, 0.5)
    cases += [
        (abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, nan, 0], [0, 1, 0], wheel=Wz),
         abi.AVBD_ERR_JOINT_BAD_AXIS),
        (abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 0],
                        wheel=((0, 0, inf), (0, 0, 1), 2.0, 0.5)), abi.AVBD_ERR_JOINT_BAD_AXIS),
        (abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 0],
                        wheel=((0, 0, 1), (0, 0, 1), -1.0, 0.5)), abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 0],
                        wheel=((0, 0, 1), (0, 0, 1), 2.0, nan)), abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 0], motor=(1.0, -1.0),
                        wheel=Wz), abi.AVBD_ERR_JOINT_NONFINITE),
        (abi.joint_desc(abi.JOINT_WHEEL, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 0], [0, 1, 0], wheel=Wz),
         abi.AVBD_ERR_JOINT_BAD_AXIS),
    ]
    for d, code in cases:
        assert w.add_joint(d)[0] == code
    # a free motor has no anchors: they are not checked
    assert w.add_joint(abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [nan, 0, 0], [0, 0, 0],
                                      drive=((0, 0, 0), (0, 0, 0), 1.0, 1.0, 0.3)))[0] == 0
    assert w.add_joint(abi.joint_desc(abi.JOINT_FIXED, 0, 1, [0, 0, 0], [0, 0, 0]))[0] == 0
    # a gear over joints that neither turn nor slide (the motor and the weld)
    assert w.add_joint(abi.joint_desc(abi.JOINT_GEAR, 0, 1, [0, 0, 0], [0, 0, 0],
                                      gear=(0, 1, 1.0)))[0] == abi.AVBD_ERR_UNSUPPORTED
