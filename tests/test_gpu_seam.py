"""The engine-seam calls beyond stepping, on the CUDA path against the
oracle, per step from identical state:

* remove_joint (avbd/mod.rs:1531-1540): both members wake, the joint and its
  warm state go, later joint handles move down by one;
* wake_body (mod.rs:1599-1601, :833-842): a sleeper wakes with its mass and
  inertia back;
* torque (mod.rs:855-871: omega += I_w^-1 tau h, then tau cleared) and a
  kinematic body driven by the host (its pose set between steps);
* the LDL^T breakdown contract (assembly.rs:38-40, :891): a body whose
  system has a zero pivot skips its update, and the breakdown counter counts
  it like the oracle's.

The device state right after remove_joint / wake_body is compared with the
oracle's (bodies, sleep state, joint warm state) before stepping on.
"""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu


def hanging_chain(n=6):
    """A static anchor and n boxes hanging straight down in a ball-jointed chain, at rest."""
    recs = [scenes.make_bodies([abi.SHAPE_BOX], [[0.2, 0.1, 0.2]], [[0, 5.0, 0]], [0.0])]
    for i in range(n):
        recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.1, 0.2, 0.1]], [[0, 5.0 - 0.35 - 0.5 * i, 0]], [1.0]))
    joints = [abi.joint_desc(abi.JOINT_BALL, 0, 1, [0, -0.1, 0], [0, 0.25, 0])]
    joints += [abi.joint_desc(abi.JOINT_BALL, i, i + 1, [0, -0.25, 0], [0, 0.25, 0]) for i in range(1, n)]
    return np.concatenate(recs), joints


def resting_stack():
    recs = [scenes.make_bodies([abi.SHAPE_BOX], [[5, 1, 5]], [[0, -1, 0]], [0.0])]
    for i in range(3):
        recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.5, 0.5, 0.5]], [[0, 0.5 + i * 1.0, 0]], [1.0]))
    return np.concatenate(recs)


def assert_same_state(o, g, dt):
    so, sg = o.export_state(), g.export_state()
    pe, ve = P.pose_errors(sg["bodies"], so["bodies"], dt)
    assert pe == 0.0 and ve == 0.0
    for f in ("inv_mass", "inertia", "mass"):
        assert np.array_equal(sg["bodies"][f], so["bodies"][f]), f
    assert np.array_equal(sg["aux"]["asleep"], so["aux"]["asleep"])
    assert np.array_equal(sg["aux"]["sleep_timer"], so["aux"]["sleep_timer"])
    assert len(sg["joints"]) == len(so["joints"])
    for f in sg["joints"].dtype.names:
        assert np.array_equal(sg["joints"][f], so["joints"][f]), f


def test_remove_joint_wakes_both_and_renumbers():
    bodies, joints = hanging_chain()
    params = abi.default_params()
    o, g = P.make_pair(bodies, params, joints)
    for _ in range(130):  # the chain settles and falls asleep (about step 120)
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
    assert so["aux"]["asleep"][1:].all() and sg["aux"]["asleep"][1:].all()
    g.import_state(o.export_state())
    o.remove_joint(2)
    g.remove_joint(2)
    o.remove_joint(99)  # invalid handles are a no-op
    g.remove_joint(99)
    assert_same_state(o, g, params.step_dt)
    st = g.export_state()
    assert len(st["joints"]) == len(joints) - 1
    assert list(st["aux"]["asleep"][1:]) == [1, 0, 0, 1, 1, 1]  # the removed joint's two bodies woke
    o.step_fixed(1)
    g.step_fixed(1)
    P.compare_states(o.export_state(), g.export_state(), params.step_dt, o, g)
    for _ in range(60):  # the lower half drops away
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
    assert g.bodies()["position"][-1, 1] < 1.5


def test_wake_body_restores_a_sleeper():
    bodies = resting_stack()
    params = abi.default_params()
    o, g = P.make_pair(bodies, params)
    for _ in range(60):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
    st = o.export_state()
    assert st["aux"]["asleep"][1:].all() and (st["bodies"]["inv_mass"][1:] == 0).all()
    g.import_state(st)
    o.wake_body(2)
    g.wake_body(2)
    g.wake_body(0)  # static, awake: untouched
    o.wake_body(0)
    assert_same_state(o, g, params.step_dt)
    b = g.bodies()
    assert b["inv_mass"][2] == np.float32(1.0) and b["inertia"][2].min() > 0
    o.step_fixed(1)
    g.step_fixed(1)
    P.compare_states(o.export_state(), g.export_state(), params.step_dt, o, g)
    for _ in range(20):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)


def test_torque_and_kinematic_body_per_step():
    recs = [scenes.make_bodies([abi.SHAPE_BOX], [[8, 1, 8]], [[0, -1, 0]], [0.0])]
    plat = scenes.make_bodies([abi.SHAPE_BOX], [[2, 0.2, 2]], [[0, 0.4, 0]], [0.0])
    plat["body_type"] = abi.BODY_KINEMATIC
    recs.append(plat)
    recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.4, 0.4, 0.4]], [[0.5, 1.0, 0]], [2.0]))
    recs.append(scenes.make_bodies([abi.SHAPE_SPHERE], [[0.3, 0, 0]], [[-0.8, 0.9, 0.3]], [1.0]))
    recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.3, 0.3, 0.3]], [[4.0, 0.3, 0]], [1.0]))
    bodies = np.concatenate(recs)
    params = abi.default_params()
    o, g = P.make_pair(bodies, params)
    spun = 0.0
    for k in range(90):
        b = o.bodies()
        b["position"][1] += np.array([0.01, 0.004 * np.sin(0.1 * k), 0.0], np.float32)  # the host drives it
        b["torque"][4] = [0.0, 3.0, 0.0] if k < 60 else [0.0, 0.0, 0.0]  # a twist on the lone box
        o.set_bodies(b)
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
        spun = max(spun, abs(float(sg["bodies"]["angular_velocity"][4][1])))
    assert spun > 0.5  # the torque turned the box
    assert g.bodies()["position"][1][0] > 0.8  # the platform moved


def test_ldl_breakdown_skips_the_body_and_counts():
    bodies = resting_stack()
    bodies["inertia"][2] = 0.0  # zero rotational block: the pivot of the first angular row is 0
    params = abi.default_params()
    o, g = P.make_pair(bodies, params)
    for _ in range(30):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
    assert g.counters().breakdowns > 0
    assert o.counters().breakdowns > 0
