"""The joint kinds beyond Ball and Revolute on the CUDA path, per step from
identical state against the oracle (Coloured order): the reference's
behavioural joint scenes (hinge motor, prismatic slider at its limit,
prismatic motor, fixed weld, distance rod, six-DOF locked / free / limited,
free motor, spring oscillator and damper, wheel axle motor and suspension,
gears over hinges and sliders) plus a rope, a mixed scene where every kind
meets contacts, and a batch of two such scenes equal to each scene alone.  The exact build computes the
oracle's arithmetic, so poses are identical; the parity bars (integers
identical, poses within 1e-5) are asserted too.  Admission errors equal the
oracle's."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld

import oracle_api as O
import parity as P
import test_oracle_joints as T

pytestmark = pytest.mark.gpu


def run_pair(recs, joints, steps, gravity=(0.0, -9.81, 0.0), setup=None, exact=True):
    bodies = O.bodies_to_array(recs) if not isinstance(recs, np.ndarray) else recs
    if setup is not None:
        setup(bodies)
    params = abi.default_params(gravity=gravity)
    o, g = P.make_pair(bodies, params, joints)
    worst = 0.0
    for _ in range(steps):
        so, sg = P.step_from_oracle_state(o, g)
        worst = max(worst, *P.compare_states(so, sg, params.step_dt, o, g))
    if exact:
        assert worst == 0.0, worst
    return g.bodies()


def anchored(shape, params, pos, radius=0.25):
    return [O.body_new(abi.SHAPE_BOX, [0.25, 0.25, 0.25], [0, 0, 0], 0.0), O.body_new(shape, params, pos, 1.0)]


def test_hinge_motor():
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.05], [0, 0, 0], 0.0)
    anchor.flags = abi.FLAG_TRIGGER
    b = run_pair([anchor, O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 1.0)],
                 [abi.joint_desc(abi.JOINT_REVOLUTE, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 1], [0, 0, 1],
                                 motor=(3.0, 20.0))], 120)
    assert b["angular_velocity"][1][2] > 1.0


def test_prismatic_slider_limit_and_motor():
    run_pair(anchored(abi.SHAPE_SPHERE, [0.25], [0, -2.9, 0]),
             [abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [0, 1, 0], [0, 1, 0], [0, 1, 0],
                             limit=(-2.0, 0.0))], 120)
    b = run_pair(anchored(abi.SHAPE_SPHERE, [0.25], [1, 0, 0]),
                 [abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [-1, 0, 0], [1, 0, 0], [1, 0, 0],
                                 motor=(2.0, 50.0))], 120)
    assert b["velocity"][1][0] > 1.0


def test_free_motor():
    """A box driven along +x across a floor by a free motor from a static
    anchor (motor_joint.rs:90-110), per step; then a spin drive without
    gravity."""
    recs, drive = T._motor_scene()
    b = run_pair(recs, [drive], 120)
    assert b["velocity"][1][0] > 1.0
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 5, 0], 0.0)
    ball = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0, 0], 1.0)
    b = run_pair([anchor, ball], [abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0],
                                                 drive=((0.5, 0.0, 0.0), (0.0, 3.0, 0.0), 2.0, 0.05, 0.0))],
                 60, gravity=(0.0, 0.0, 0.0))
    assert b["angular_velocity"][1][1] > 0.5


@pytest.mark.parametrize("model", [abi.MODEL_ACCELERATION, abi.MODEL_FORCE])
def test_spring(model):
    """The spring oscillator (p6_rope_spring_motor.rs:193-216) per step."""
    recs, d = T._spring_scene(model)
    run_pair(recs, [d], 150, gravity=(0.0, 0.0, 0.0))
    recs, d = T._spring_scene(model, stiffness=0.0, damping=4.0)

    def push(arr):
        arr["velocity"][1] = [0.0, -3.0, 0.0]
    run_pair(recs, [d], 60, gravity=(0.0, 0.0, 0.0), setup=push)


def test_wheel():
    """The wheel's axle motor (zero gravity) and its suspension, sprung and
    rigid (avbd_engine.rs:969-1061), per step."""
    recs, d = T._wheel_motor_scene()
    b = run_pair(recs, [d], 120, gravity=(0.0, 0.0, 0.0))
    assert b["angular_velocity"][1][2] > 2.0
    for hz in (3.0, 0.0):
        recs, d = T._wheel_suspension_scene(hz)
        run_pair(recs, [d], 120)


def test_gears():
    """The 2:1 hinge gear past a half turn of its driven hinge, and the
    slider pair through a host teleport, per step."""
    recs, joints = T._gear_hinge_scene()
    b = run_pair(recs, joints, 180, gravity=(0.0, 0.0, 0.0))
    assert abs(T.z_twist(b["orientation"][1])) > 0.5
    recs, joints = T._gear_slider_scene()
    params = abi.default_params()
    o, g = P.make_pair(O.bodies_to_array(recs), params, joints)
    for step in range(160):
        if step == 80:
            for w in (o, g):
                arr = w.bodies()
                arr["position"][1][0] += 4.0
                w.set_bodies(arr)
        so, sg = P.step_from_oracle_state(o, g)
        assert max(P.compare_states(so, sg, params.step_dt, o, g)) == 0.0
    p = g.bodies()["position"]
    assert p[1][0] - 1.0 > 2.0 and p[2][0] - 3.0 > 2.0


def test_gear_goes_with_its_joint():
    """Removing a coupled joint or one of its bodies removes the gear
    (joint_remap, migration.rs:74-115), on the device as in the oracle."""
    recs, joints = T._gear_hinge_scene()
    for edit in ("joint", "body"):
        o, g = P.make_pair(O.bodies_to_array(recs), abi.default_params(gravity=(0.0, 0.0, 0.0)), joints)
        for w in (o, g):
            w.add_joint(abi.joint_desc(abi.JOINT_GEAR, 1, 2, [0, 0, 0], [0, 0, 0], gear=(1, 0, 0.5)))
        for _ in range(20):
            P.step_from_oracle_state(o, g)
        for w in (o, g):
            if edit == "joint":
                w.remove_joint(1)
            else:
                w.remove_body(2)
        assert len(g.export_state()["joints"]) == len(o.export_state()["joints"]) == 1
        for _ in range(20):
            so, sg = P.step_from_oracle_state(o, g)
            assert max(P.compare_states(so, sg, 1.0 / 60.0, o, g)) == 0.0


def test_fixed_distance_and_rope():
    floor = O.body_new(abi.SHAPE_BOX, [5, 1, 5], [0, -1, 0], 0.0)
    run_pair([floor, O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [-0.5, 3, 0], 1.0),
              O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0.5, 3, 0], 1.0)],
             [abi.joint_desc(abi.JOINT_FIXED, 1, 2, [0.5, 0, 0], [-0.5, 0, 0])], 150)
    run_pair([O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 0.0), O.body_new(abi.SHAPE_SPHERE, [0.25], [2, 0, 0], 1.0)],
             [abi.joint_desc(abi.JOINT_DISTANCE, 0, 1, [0, 0, 0], [0, 0, 0])], 120)
    b = run_pair([O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 0, 0], 0.0),
                  O.body_new(abi.SHAPE_SPHERE, [0.25], [1, 0, 0], 1.0)],
                 [abi.joint_desc(abi.JOINT_ROPE, 0, 1, [0, 0, 0], [0, 0, 0], max_distance=2.0)], 150)
    assert np.linalg.norm(b["position"][1]) < 2.25


def test_sixdof_locked_free_and_limited():
    run_pair([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 1.0),
              O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 1.4, 0], 1.0)],
             [abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0], axes=["locked"] * 6)], 90)

    def push(v):
        def f(b):
            b["velocity"][1] = v
        return f

    def spin(b):
        b["angular_velocity"][1] = [0.0, 0.0, 8.0]
    run_pair([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 1.0),
              O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [1, 0, 0], 1.0)],
             [abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0],
                             axes=["free", "locked", "locked", "locked", "locked", "locked"])], 60,
             gravity=(0, 0, 0), setup=push([3.0, 1.0, 0.0]))
    b = run_pair([O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 0.0),
                  O.body_new(abi.SHAPE_BOX, [0.4, 0.4, 0.4], [0, 0, 0], 1.0)],
                 [abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0],
                                 axes=["locked"] * 5 + [(-0.2, 0.2)])], 90, gravity=(0, 0, 0), setup=spin)
    assert abs(T.z_twist(b["orientation"][1])) < 0.4


def zoo(x0):
    """Every joint kind in one scene with contacts: a slider-mounted arm,
    a welded pair, a rod, a rope, a six-DOF pair, a free motor pushing
    the rod's end, a spring, a driven sprung wheel and a gear between the
    slider and the hinge, falling onto a floor."""
    rec = [O.body_new(abi.SHAPE_BOX, [6, 0.5, 6], [x0, -0.5, 0], 0.0),
           O.body_new(abi.SHAPE_BOX, [0.2, 0.2, 0.2], [x0, 4, 0], 0.0)]
    for k, (shape, p) in enumerate([(abi.SHAPE_BOX, [0.3, 0.3, 0.3]), (abi.SHAPE_SPHERE, [0.3]),
                                    (abi.SHAPE_BOX, [0.3, 0.2, 0.3]), (abi.SHAPE_BOX, [0.3, 0.3, 0.3]),
                                    (abi.SHAPE_SPHERE, [0.25]), (abi.SHAPE_CAPSULE, [0.15, 0.3]),
                                    (abi.SHAPE_BOX, [0.25, 0.25, 0.25]), (abi.SHAPE_BOX, [0.25, 0.25, 0.25])]):
        rec.append(O.body_new(shape, p, [x0 - 2.0 + 0.8 * k, 2.0 + 0.3 * (k % 3), 0.3 * (k % 2)], 1.0))
    js = [abi.joint_desc(abi.JOINT_PRISMATIC, 1, 2, [0, 0, 0], [0, 0.5, 0], [1, 0, 0], [1, 0, 0], limit=(-1.5, 1.5),
                         motor=(1.0, 5.0)),
          abi.joint_desc(abi.JOINT_REVOLUTE, 2, 3, [0.4, 0, 0], [-0.4, 0, 0], [0, 0, 1], [0, 0, 1], limit=(-0.5, 0.5),
                         motor=(-2.0, 3.0)),
          abi.joint_desc(abi.JOINT_FIXED, 4, 5, [0.4, 0, 0], [-0.4, 0, 0]),
          abi.joint_desc(abi.JOINT_DISTANCE, 5, 6, [0, 0, 0], [0, 0, 0]),
          abi.joint_desc(abi.JOINT_ROPE, 1, 7, [0, 0, 0], [0, 0, 0], max_distance=3.0),
          abi.joint_desc(abi.JOINT_SIXDOF, 8, 9, [0, 0, 0], [0, 0, 0],
                         axes=["locked", (-0.2, 0.3), "free", "locked", (-0.4, 0.4), "locked"]),
          abi.joint_desc(abi.JOINT_MOTOR, 1, 6, [0, 0, 0], [0, 0, 0],
                         drive=((0.5, 0.0, 0.0), (0.0, 1.0, 0.0), 3.0, 0.5, 0.2)),
          abi.joint_desc(abi.JOINT_SPRING, 3, 9, [0.2, 0, 0], [0, 0.2, 0],
                         spring=(1.2, 0.0, 40.0, 3.0, 1e4, abi.MOTOR_POSITION, abi.MODEL_ACCELERATION)),
          abi.joint_desc(abi.JOINT_WHEEL, 4, 7, [0, -0.3, 0], [0, 0.3, 0], [0, 1, 0], [0, 1, 0], motor=(4.0, 2.0),
                         wheel=((0, 0, 1), (0, 0, 1), 2.5, 0.6)),
          # the slider and the hinge geared together (a slide side and a turn side sharing body 2)
          abi.joint_desc(abi.JOINT_GEAR, 2, 3, [0, 0, 0], [0, 0, 0], gear=(0, 1, 0.3))]
    return rec, js


def test_every_kind_with_contacts_per_step():
    rec, js = zoo(0.0)
    run_pair(rec, js, 150)


def test_joint_batch_equals_scenes_alone():
    r0, j0 = zoo(0.0)
    r1, j1 = zoo(30.0)
    n0 = len(r0)
    bodies = O.bodies_to_array(r0 + r1)
    offs = np.array([0, n0, len(bodies)], dtype=np.uint32)
    params, nsub = scenes.params_for("ragdoll_8192")
    batch = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    alone = [AvbdWorld(params, bodies=bodies[:n0]), AvbdWorld(params, bodies=bodies[n0:])]
    for d in j0:
        batch.add_joint(d)
        alone[0].add_joint(d)
    for d in j1:
        alone[1].add_joint(d)
        d.body_a += n0
        d.body_b += n0
        if d.kind == abi.JOINT_GEAR:  # joint handles of the batch world
            d.gear_joint_a += len(j0)
            d.gear_joint_b += len(j0)
        batch.add_joint(d)
    for _ in range(60):
        batch.step_graph(nsub)
        for w in alone:
            w.step_graph(nsub)
    got = batch.bodies()
    assert got[:n0].tobytes() == alone[0].bodies().tobytes()
    assert got[n0:].tobytes() == alone[1].bodies().tobytes()


def test_admission_errors_equal_the_oracle():
    recs = [O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0, 0], 1.0),
            O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [2, 0, 0], 1.0)]
    nan = float("nan")
    descs = [abi.joint_desc(abi.JOINT_BALL, 0, 1, [nan, 0, 0], [0, 0, 0]),
             abi.joint_desc(abi.JOINT_REVOLUTE, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 1], [0, 0, 1], limit=(1.0, -1.0)),
             abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [0, 0, 0], [1, 0, 0], [1, 0, 0], motor=(nan, 1.0)),
             abi.joint_desc(abi.JOINT_PRISMATIC, 0, 1, [0, 0, 0], [0, 0, 0], [0, 0, 0], [1, 0, 0]),
             abi.joint_desc(abi.JOINT_ROPE, 0, 1, [0, 0, 0], [0, 0, 0], max_distance=0.0),
             abi.joint_desc(abi.JOINT_SIXDOF, 0, 1, [0, 0, 0], [0, 0, 0], axes=["locked"] * 5 + [(0.3, -0.3)]),
             abi.joint_desc(abi.JOINT_FIXED, 0, 0, [0, 0, 0], [0, 0, 0]),
             abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((nan, 0, 0), (0, 0, 0), 1, 1, 0)),
             abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((0, 0, 0), (0, 0, 0), -1, 1, 0)),
             abi.joint_desc(abi.JOINT_MOTOR, 0, 1, [0, 0, 0], [0, 0, 0], drive=((0, 0, 0), (0, 0, 0), 1, 1, 2)),
             abi.joint_desc(abi.JOINT_GEAR, 0, 1, [0, 0, 0], [0, 0, 0], gear=(0, 0, nan)),
             abi.joint_desc(abi.JOINT_GEAR, 0, 1, [0, 0, 0], [0, 0, 0], gear=(5, 6, 1.0)),
             abi.joint_desc(abi.JOINT_BALL, 0, 1, [0, 0, 0], [0, 0, 0]),  # admitted: a gear over it is not
             abi.joint_desc(abi.JOINT_GEAR, 0, 1, [0, 0, 0], [0, 0, 0], gear=(0, 0, 1.0))]
    o = O.OracleWorld()
    o.add_bodies(O.bodies_to_array(recs))
    g = AvbdWorld(abi.default_params(), bodies=O.bodies_to_array(recs))
    for d in descs:
        want = o.add_joint(d)[0]
        try:
            g.add_joint(d)
            got = 0
        except AvbdError as e:
            got = e.code
        assert got == want
        assert got != 0 or d.kind == abi.JOINT_BALL
