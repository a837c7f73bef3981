"""Contact and trigger events of the CUDA path against the CPU oracle and
the reference's own event tests (crates/physics/tests/avbd_engine.rs:274-320).

The device reports the reference's events; within one substep it orders
Begin / End and hits by (body_b, body_a) instead of (body_a, body_b), so
comparisons sort both sides."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdWorld

import oracle_api as O

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def zero_g():
    p = abi.default_params()
    p.gravity[0] = p.gravity[1] = p.gravity[2] = 0.0
    return p


def move(w, h, pos):
    b = w.bodies()
    b["position"][h] = pos
    w.set_bodies(b)


def keyset(ev):
    return sorted((int(e["kind"]), int(e["body_b"]), int(e["body_a"])) for e in ev)


def test_trigger_enter_exit_roundtrip():
    sensor = O.body_new(abi.SHAPE_SPHERE, [1.0], [0, 0, 0], 0.0)
    sensor.flags = abi.FLAG_TRIGGER
    mover = O.body_new(abi.SHAPE_SPHERE, [0.5], [5, 0, 0], 1.0)
    w = AvbdWorld(zero_g(), bodies=O.bodies_to_array([sensor, mover]))
    w.step(DT)
    assert len(w.trigger_events()) == 0
    move(w, 1, [0, 0, 0])
    w.step(DT)
    ev = w.trigger_events()
    assert len(ev) == 1 and ev[0]["entered"] == 1 and (ev[0]["body_a"], ev[0]["body_b"]) == (0, 1)
    move(w, 1, [5, 0, 0])
    w.step(DT)
    ev = w.trigger_events()
    assert len(ev) == 1 and ev[0]["entered"] == 0
    assert len(w.contact_events()) == 0


def test_contact_begin_end_roundtrip():
    a = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0, 0], 0.0)
    b = O.body_new(abi.SHAPE_SPHERE, [0.5], [5, 0, 0], 1.0)
    w = AvbdWorld(zero_g(), bodies=O.bodies_to_array([a, b]))
    w.step(DT)
    assert len(w.contact_events()) == 0
    move(w, 1, [0.9, 0, 0])
    w.step(DT)
    assert any(e["kind"] == abi.CONTACT_BEGIN for e in w.contact_events())
    move(w, 1, [5, 0, 0])
    w.step(DT)
    assert any(e["kind"] == abi.CONTACT_END for e in w.contact_events())


@pytest.mark.parametrize("speed", [10.0, 30.0])
def test_hits_match_oracle(speed):
    """A landing (discrete contact hit) and a swept impact (time-of-impact hit)."""
    ground = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    balls = []
    for i in range(3):
        b = O.body_new(abi.SHAPE_SPHERE, [0.5], [2.0 * i, 0.52, 0], 1.0)
        b.velocity[1] = -speed
        balls.append(b)
    arr = O.bodies_to_array([ground] + balls)
    params = abi.default_params()
    o = O.OracleWorld(params, mode=O.COLOURED)
    o.add_bodies(arr)
    g = AvbdWorld(params, bodies=arr)
    for _ in range(4):
        o.step(DT)
        g.step(DT)
        eo, eg = o.contact_events(), g.contact_events()
        assert keyset(eo) == keyset(eg)
        ho = sorted((int(e["body_b"]), tuple(e["point"]), tuple(e["normal"]), float(e["approach_speed"]))
                    for e in eo if e["kind"] == abi.CONTACT_HIT)
        hg = sorted((int(e["body_b"]), tuple(e["point"]), tuple(e["normal"]), float(e["approach_speed"]))
                    for e in eg if e["kind"] == abi.CONTACT_HIT)
        for x, y in zip(ho, hg):
            assert x[0] == y[0]
            np.testing.assert_allclose(x[1], y[1], rtol=1e-5, atol=1e-5)
            np.testing.assert_allclose(x[2], y[2], rtol=1e-5, atol=1e-5)
            np.testing.assert_allclose(x[3], y[3], rtol=1e-5)


def test_pile_events_match_oracle_per_step():
    """A bin filling up: from the oracle's state each step, the step's event
    set equals the oracle's (the touch sets carry over on both sides)."""
    rng = np.random.default_rng([3, 5])
    bodies = scenes.bin_scene(rng, 100)
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    o = O.OracleWorld(params, mode=O.COLOURED)
    o.add_bodies(bodies)
    o.set_emit_period(2)
    g = AvbdWorld(params, bodies=bodies)
    g.set_events(2)
    total = 0
    for step in range(80):
        g.import_state(o.export_state())
        o.step_fixed(2)
        g.step_fixed(2)
        eo, eg = o.contact_events(), g.contact_events()
        assert keyset(eo) == keyset(eg), f"step {step}"
        total += len(eo)
    assert total > 50
    assert g.event_counts()["contact_dropped"] == 0


def test_graph_replay_reports_the_same_events():
    bodies, offs, _ = scenes.batched(8, seed=4, lo=20, hi=120)
    params, nsub = scenes.params_for("batched_4096")
    a = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    b = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    a.set_events(nsub)
    b.set_events(nsub)
    for _ in range(40):
        a.step_fixed(nsub)
        b.step_graph(nsub)
        assert keyset(a.contact_events()) == keyset(b.contact_events())


def test_events_off():
    ground = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    ball = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0.52, 0], 1.0)
    ball.velocity[1] = -10.0
    w = AvbdWorld(abi.default_params(), bodies=O.bodies_to_array([ground, ball]))
    w.set_events(-1)
    for _ in range(3):
        w.step(DT)
    assert len(w.contact_events()) == 0
