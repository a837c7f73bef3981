"""CUDA path vs the CPU oracle (Coloured schedule) on identical input state.

Every test here runs the step through libornis_avbd.so on the GPU and checks
it against the oracle each step: pair sets, point counts, contact IDs and
colours bit-exact; poses within POSE_RTOL (see parity.py).
"""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdWorld

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu


def run_parity(bodies, params, steps, joints=(), nsub=1):
    o, g = P.make_pair(bodies, params, joints)
    worst = (0.0, 0.0)
    for _ in range(steps):
        so, sg = P.step_from_oracle_state(o, g, nsub)
        pe, ve = P.compare_states(so, sg, params.step_dt, o, g)
        worst = (max(worst[0], pe), max(worst[1], ve))
    return worst


def snapshot_scene():
    """The reference's canonical determinism scene (tests/avbd_engine.rs:1560-1606)."""
    recs = [scenes.make_bodies([abi.SHAPE_BOX], [[10, 1, 10]], [[0, -1, 0]], [0.0])]
    for i in range(4):
        y = np.float32(0.5) + np.float32(i) * np.float32(1.02)
        recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.5, 0.5, 0.5]], [[0, y, 0]], [1.0]))
    recs.append(scenes.make_bodies([abi.SHAPE_SPHERE], [[0.5, 0, 0]], [[3, 6, 0]], [1.0]))
    fast = scenes.make_bodies([abi.SHAPE_BOX], [[0.4, 0.4, 0.4]], [[-3, 8, 0]], [1.0])
    fast["velocity"][0, 1] = -30.0
    recs.append(fast)
    recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.5, 0.5, 0.5]], [[6, 3, 0]], [0.0]))
    recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[0.5, 0.5, 0.5]], [[6, 1, 0]], [1.0]))
    joint = abi.joint_desc(abi.JOINT_BALL, 7, 8, [0, -1, 0], [0, 1, 0])
    return np.concatenate(recs), [joint]


def test_snapshot_scene_per_step():
    bodies, joints = snapshot_scene()
    run_parity(bodies, abi.default_params(), 120, joints)


def test_pyramid_per_step():
    bodies = scenes.pyramid_210(rows=8)
    run_parity(bodies, abi.default_params(), 90)


def test_mixed_shapes_per_step():
    rng = np.random.default_rng(7)
    kind, params, mass, fric = scenes._mixed(rng, 60, with_capsules=True)
    pos = np.stack([rng.uniform(-3, 3, 60), rng.uniform(0.8, 8, 60), rng.uniform(-3, 3, 60)], axis=1)
    q = scenes.random_quats(rng, 60)
    bodies = np.concatenate([scenes.halfspace([0, 0, 0], [0, 1, 0]),
                             scenes.make_bodies(kind, params, pos.astype(np.float32), mass, q, fric)])
    run_parity(bodies, abi.default_params(), 80)


def test_bin_scene_small_dt_per_step():
    rng = np.random.default_rng([2, 3])
    bodies = scenes.bin_scene(rng, 120)
    params, nsub = scenes.params_for("batched_4096")
    run_parity(bodies, params, 60, nsub=1)


def test_hinge_chain_with_limits_per_step():
    # a capsule chain hanging from a static anchor by revolute joints with limits
    recs = [scenes.make_bodies([abi.SHAPE_BOX], [[0.2, 0.2, 0.2]], [[0, 5, 0]], [0.0])]
    n = 6
    for i in range(n):
        recs.append(scenes.make_bodies([abi.SHAPE_CAPSULE], [[0.1, 0.25, 0]], [[0.7 * (i + 1), 5, 0]], [1.0],
                                       orientation=[[0, 0, np.sin(np.pi / 4), np.cos(np.pi / 4)]]))
    bodies = np.concatenate(recs)
    joints = [abi.joint_desc(abi.JOINT_REVOLUTE, 0, 1, [0.35, 0, 0], [0, 0.35, 0], [0, 0, 1], [0, 0, 1],
                             limit=(-0.8, 0.8))]
    for i in range(1, n):
        joints.append(abi.joint_desc(abi.JOINT_REVOLUTE, i, i + 1, [0, -0.35, 0], [0, 0.35, 0], [0, 0, 1],
                                     [0, 0, 1], limit=(-0.5, 0.5)))
    run_parity(bodies, abi.default_params(), 90, joints)


def test_free_run_matches_oracle_snapshot_scene():
    """Both sides run 120 steps on their own; the stack sleeps identically."""
    bodies, joints = snapshot_scene()
    o, g = P.make_pair(bodies, abi.default_params(), joints)
    for _ in range(120):
        o.step(np.float32(1 / 60))
        g.step(np.float32(1 / 60))
    so, sg = o.export_state(), g.export_state()
    pe, _ = P.pose_errors(sg["bodies"], so["bodies"], 1 / 60)
    assert pe < 1e-4
    assert o.counters().sleeping == g.counters().sleeping


def test_pyramid_210_600_steps_within_1e3():
    """The 20-row, 210-cube pyramid (dt 1/60, 10 iterations) run freely for
    600 steps: final poses within 1e-3 of the oracle's (the long-run bar for
    stable stacks), and both against the f64 oracle."""
    bodies = scenes.pyramid_210()
    params = abi.default_params()
    o = O.OracleWorld(params, mode=O.COLOURED)
    o.add_bodies(bodies)
    o64 = O.OracleWorld(params, mode=O.COLOURED, use_double=True)
    o64.add_bodies(bodies)
    g = AvbdWorld(params, bodies=bodies)
    o.step_fixed(600)
    o64.step_fixed(600)
    g.step_graph(600)
    ref, ref64, got = o.bodies(), o64.bodies(), g.bodies()
    err, _ = P.pose_errors(got, ref, params.step_dt)
    err64, _ = P.pose_errors(got, ref64, params.step_dt)
    err_o64, _ = P.pose_errors(ref, ref64, params.step_dt)
    print(f"pyramid 600 steps: gpu vs f32 oracle {err:.2e}, gpu vs f64 {err64:.2e}, f32 oracle vs f64 {err_o64:.2e}")
    assert err <= 1e-3
