"""The CPU oracle pinned against the reference's own fixtures and tests.

  * avbd_snapshot.hex — the reference's bit-exact determinism fixture
    (crates/physics/tests/avbd_engine.rs:1550-1645): the oracle in Reference
    mode must reproduce it bit for bit.
  * known answers of the row stamp and the LDL^T solve
    (crates/physics/tests/gpu_batches.rs:781-898);
  * the in-module contact tests (crates/physics/src/avbd/contact_tests.rs);
  * behavioural gates and run-to-run determinism (tests/avbd_engine.rs:31-62,
    :256-272).
"""
import ctypes as C
import os
import struct

import numpy as np
import pytest

from ornis_gb300 import abi

import oracle_api as O

HERE = os.path.dirname(os.path.abspath(__file__))


def f32(x):
    return np.float32(x)


def snapshot_bodies():
    """tests/avbd_engine.rs:1560-1606, built with the oracle's constructors."""
    bl = [O.body_new(abi.SHAPE_BOX, [10, 1, 10], [0, -1, 0], 0)]
    for i in range(4):
        bl.append(O.body_new(abi.SHAPE_BOX, [0.5] * 3, [0, f32(0.5) + f32(i) * f32(1.02), 0], 1))
    bl.append(O.body_new(abi.SHAPE_SPHERE, [0.5], [3, 6, 0], 1))
    fast = O.body_new(abi.SHAPE_BOX, [0.4] * 3, [-3, 8, 0], 1)
    fast.velocity[1] = -30.0
    bl.append(fast)
    bl.append(O.body_new(abi.SHAPE_BOX, [0.5] * 3, [6, 3, 0], 0))
    bl.append(O.body_new(abi.SHAPE_BOX, [0.5] * 3, [6, 1, 0], 1))
    return O.bodies_to_array(bl)


def render(bodies):
    out = []
    for r in bodies:
        vals = list(r["position"]) + list(r["orientation"]) + list(r["velocity"]) + list(r["angular_velocity"])
        out.append(" ".join("%08x" % struct.unpack("<I", struct.pack("<f", v))[0] for v in vals))
    return out


def test_snapshot_hex_bit_exact():
    w = O.OracleWorld(mode=O.REFERENCE)
    w.add_bodies(snapshot_bodies())
    rc, _ = w.add_joint(abi.joint_desc(abi.JOINT_BALL, 7, 8, [0, -1, 0], [0, 1, 0]))
    assert rc == 0
    for _ in range(120):
        w.step(f32(1 / 60))
    lines = open(os.path.join(HERE, "golden", "avbd_snapshot.hex")).read().splitlines()
    assert lines[0].startswith("ornis-avbd-snapshot v1 bodies=9 steps=120")
    assert render(w.bodies()) == lines[1:]
    c = w.counters()
    assert c.ccd_hits == 1  # the -30 m/s box is caught by the TOI clamp
    assert c.sleeping == 5  # the stack and the sphere are asleep


def test_snapshot_f64_close_to_f32():
    ws = []
    for dbl in (False, True):
        w = O.OracleWorld(mode=O.REFERENCE, use_double=dbl)
        w.add_bodies(snapshot_bodies())
        w.add_joint(abi.joint_desc(abi.JOINT_BALL, 7, 8, [0, -1, 0], [0, 1, 0]))
        for _ in range(120):
            w.step(f32(1 / 60))
        ws.append(w.state13())
    err = np.abs(ws[0][:, :3] - ws[1][:, :3]).max()
    assert err < 1e-2


def test_stamp_row_known_answer():
    """gpu_batches.rs:781-856: axis +Y, lever +X, pen 2, force 3."""
    lhs = np.zeros(36, np.float32)
    rhs = np.zeros(6, np.float32)
    ax = np.array([0, 1, 0], np.float32)
    lev = np.array([1, 0, 0], np.float32)
    O.lib().oracle_stamp_row(abi.ptr(lhs), abi.ptr(rhs), abi.ptr(ax), 2.0, 3.0, abi.ptr(lev), 1.0)
    exp = np.zeros((6, 6), np.float32)
    exp[1, 1] = exp[5, 5] = exp[1, 5] = exp[5, 1] = 2.0
    assert np.array_equal(lhs.reshape(6, 6), exp)
    assert np.array_equal(rhs, np.array([0, 3, 0, 0, 0, 3], np.float32))
    lhs_b = np.zeros(36, np.float32)
    rhs_b = np.zeros(6, np.float32)
    O.lib().oracle_stamp_row(abi.ptr(lhs_b), abi.ptr(rhs_b), abi.ptr(ax), 2.0, 3.0, abi.ptr(lev), -1.0)
    assert np.array_equal(lhs_b.reshape(6, 6), exp)  # Hessian is quadratic in the side
    assert np.array_equal(rhs_b, -rhs)  # rhs flips


def test_ldl_known_answer_and_breakdown():
    """gpu_batches.rs:863-898: SPD solve equals dense; singular / indefinite break down."""
    lhs = np.zeros((6, 6), np.float32)
    for i in range(6):
        for j in range(6):
            lhs[i, j] = 4.0 + i if i == j else 0.1 * ((i + j) + 1.0)
    lhs = np.triu(lhs) + np.triu(lhs, 1).T
    rhs = np.array([1, -2, 3, -4, 5, -6], np.float32)
    x = np.zeros(6, np.float32)
    ok = O.lib().oracle_solve_6x6(abi.ptr(np.ascontiguousarray(lhs)), abi.ptr(rhs), abi.ptr(x))
    assert ok == 1
    assert np.allclose(x, np.linalg.solve(lhs.astype(np.float64), rhs.astype(np.float64)), atol=1e-6)
    z = np.zeros(36, np.float32)
    assert O.lib().oracle_solve_6x6(abi.ptr(z), abi.ptr(rhs), abi.ptr(x)) == 0
    assert np.all(x == 0)
    neg = np.ascontiguousarray(lhs.copy())
    neg[0, 0] = -1.0
    assert O.lib().oracle_solve_6x6(abi.ptr(neg), abi.ptr(rhs), abi.ptr(x)) == 0


def test_tangent_basis_orthonormal():
    """avbd/contact_tests.rs:168-186."""
    for n in ([1, 0, 0], [0, 1, 0], [0, 0, 1], list(np.array([1, 2, 3]) / np.linalg.norm([1, 2, 3]))):
        nn = np.asarray(n, np.float32)
        t1 = np.zeros(3, np.float32)
        t2 = np.zeros(3, np.float32)
        O.lib().oracle_tangent_basis(abi.ptr(nn), abi.ptr(t1), abi.ptr(t2))
        assert abs(t1 @ nn) < 1e-6 and abs(t2 @ nn) < 1e-6 and abs(t1 @ t2) < 1e-6
        assert abs(np.linalg.norm(t1) - 1) < 1e-6


def _buried_box_world(gravity=(0, 0, 0)):
    w = O.OracleWorld(abi.default_params(gravity=gravity))
    w.add_bodies(O.bodies_to_array([O.body_new(abi.SHAPE_BOX, [10, 1, 10], [0, -1, 0], 0),
                                    O.body_new(abi.SHAPE_BOX, [0.4] * 3, [-3, 0.3, 0], 1)]))
    return w


def test_refreshed_face_contacts_preserve_penetration():
    """avbd/contact_tests.rs:38-63."""
    w = _buried_box_world()
    w.generate_pairs()
    st = w.export_state()
    assert st["pairs"][0]["npoints"] >= 3
    for qi in range(st["pairs"][0]["npoints"]):
        assert w.gap_c0(0, qi) < -0.08


def test_face_anchors_lie_on_their_own_surface():
    """avbd/contact_tests.rs:65-90."""
    w = _buried_box_world()
    w.generate_pairs()
    st = w.export_state()
    p = st["pairs"][0]
    for pt in st["points"][: p["npoints"]]:
        assert abs(pt["ra"][1] - 1.0) < 1e-6
        assert abs(pt["rb"][1] + 0.4) < 1e-6
        assert abs(pt["rb"][0]) <= 0.401 and abs(pt["rb"][2]) <= 0.401


def floor_stack():
    """tests/avbd_engine.rs:14-28."""
    bl = [O.body_new(abi.SHAPE_BOX, [5, 1, 5], [0, -1, 0], 0)]
    for level in range(4):
        bl.append(O.body_new(abi.SHAPE_BOX, [0.5] * 3, [0, f32(0.5) + f32(level) * f32(1.02), 0], 1))
    return O.bodies_to_array(bl)


@pytest.mark.parametrize("mode", [O.REFERENCE, O.COLOURED])
def test_stack_stands(mode):
    """avbd_stack_stands_like_si (tests/avbd_engine.rs:31-62), both sweep schedules."""
    w = O.OracleWorld(mode=mode)
    w.add_bodies(floor_stack())
    for _ in range(300):
        w.step(f32(1 / 60))
    b = w.bodies()
    for level in range(4):
        r = b[1 + level]
        assert abs(r["position"][1] - (0.5 + level)) < 0.1
        assert abs(r["position"][0]) < 0.15 and abs(r["position"][2]) < 0.15
        assert np.linalg.norm(r["velocity"]) < 0.08
        assert np.linalg.norm(r["angular_velocity"]) < 0.08


def test_determinism_run_to_run():
    """avbd_determinism_run_to_run (tests/avbd_engine.rs:256-272)."""
    runs = []
    for _ in range(2):
        w = O.OracleWorld()
        w.add_bodies(floor_stack())
        for _ in range(60):
            w.step(f32(1 / 60))
        runs.append(w.bodies()["position"].copy())
    assert np.array_equal(runs[0], runs[1])


def test_threaded_discovery_is_confluent():
    """1 vs 4 discovery threads give identical bits (tests/avbd_engine.rs:1661-1768)."""
    from ornis_gb300 import scenes

    bodies = scenes.pyramid_210(rows=24)  # 300 cubes: above the 256-body threading threshold
    res = []
    for t in (1, 4):
        w = O.OracleWorld(threads=t)
        w.add_bodies(bodies)
        for _ in range(5):
            w.step(f32(1 / 60))
        res.append(w.bodies().tobytes())
    assert res[0] == res[1]


def test_faithful_scan_equals_adjacency():
    """The O(P) pair scan of assembly.rs:99-106 and the adjacency lists give identical bits."""
    out = []
    for faithful in (True, False):
        w = O.OracleWorld()
        w.faithful_scan(faithful)
        w.add_bodies(floor_stack())
        for _ in range(40):
            w.step(f32(1 / 60))
        out.append(w.bodies().tobytes())
    assert out[0] == out[1]


def test_joint_errors():
    """JointError admission (avbd/mod.rs:1323-1328)."""
    w = O.OracleWorld()
    w.add_bodies(floor_stack())
    assert w.add_joint(abi.joint_desc(abi.JOINT_BALL, 1, 1, [0, 0, 0], [0, 0, 0]))[0] == abi.AVBD_ERR_JOINT_SELF
    assert w.add_joint(abi.joint_desc(abi.JOINT_BALL, 1, 99, [0, 0, 0], [0, 0, 0]))[0] == abi.AVBD_ERR_JOINT_HANDLES
    d = abi.joint_desc(abi.JOINT_REVOLUTE, 1, 2, [0, 0, 0], [0, 0, 0], [0, 0, 0], [0, 1, 0])
    assert w.add_joint(d)[0] == abi.AVBD_ERR_JOINT_BAD_AXIS
    assert w.add_joint(abi.joint_desc(abi.JOINT_BALL, 1, 2, [0, 0, 0], [0, 0, 0]))[0] == 0


def test_bad_dt_is_noop():
    """mod.rs:1213-1215."""
    w = O.OracleWorld()
    w.add_bodies(floor_stack())
    before = w.bodies().tobytes()
    for dt in (0.0, -1.0, float("nan"), float("inf")):
        w.step(dt)
    assert w.bodies().tobytes() == before
