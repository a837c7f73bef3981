"""Contact and trigger events of the CPU oracle, mirroring the reference's
event tests (crates/physics/tests/avbd_engine.rs:274-320) and the emission
rules of avbd/mod.rs:1606-1669 and :935-960 / :1126-1136."""
import numpy as np

from ornis_gb300 import abi

import oracle_api as O

DT = 1.0 / 60.0


def zero_g():
    p = abi.default_params()
    p.gravity[0] = p.gravity[1] = p.gravity[2] = 0.0
    return p


def world(bodies, params=None, mode=O.REFERENCE):
    w = O.OracleWorld(params or zero_g(), mode=mode)
    w.add_bodies(O.bodies_to_array(bodies))
    return w


def move(w, h, pos):
    b = w.bodies()
    b["position"][h] = pos
    w.set_bodies(b)


def test_trigger_enter_exit_roundtrip():
    sensor = O.body_new(abi.SHAPE_SPHERE, [1.0], [0, 0, 0], 0.0)
    sensor.flags = abi.FLAG_TRIGGER
    mover = O.body_new(abi.SHAPE_SPHERE, [0.5], [5, 0, 0], 1.0)
    w = world([sensor, mover])
    w.step(DT)
    assert len(w.trigger_events()) == 0
    move(w, 1, [0, 0, 0])
    w.step(DT)
    ev = w.trigger_events()
    assert len(ev) == 1 and ev[0]["entered"] == 1
    assert (ev[0]["body_a"], ev[0]["body_b"]) == (0, 1)
    move(w, 1, [5, 0, 0])
    w.step(DT)
    ev = w.trigger_events()
    assert len(ev) == 1 and ev[0]["entered"] == 0
    assert len(w.contact_events()) == 0  # a trigger forms no contact


def test_contact_begin_end_roundtrip():
    a = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0, 0], 0.0)
    b = O.body_new(abi.SHAPE_SPHERE, [0.5], [5, 0, 0], 1.0)
    w = world([a, b])
    w.step(DT)
    assert len(w.contact_events()) == 0
    move(w, 1, [0.9, 0, 0])
    w.step(DT)
    ev = w.contact_events()
    assert any(e["kind"] == abi.CONTACT_BEGIN for e in ev), ev
    move(w, 1, [5, 0, 0])
    w.step(DT)
    ev = w.contact_events()
    assert any(e["kind"] == abi.CONTACT_END for e in ev), ev


def test_landing_is_a_hit_with_its_approach_speed():
    ground = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    ball = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0.52, 0], 1.0)
    ball.velocity[1] = -10.0  # lands within the first step, 3.7 cm deep: Begin + Hit
    w = world([ground, ball], params=abi.default_params())
    hits = []
    for _ in range(5):
        w.step(DT)
        hits += [e for e in w.contact_events() if e["kind"] == abi.CONTACT_HIT]
    assert len(hits) == 1
    h = hits[0]
    assert (h["body_a"], h["body_b"]) == (0, 1)
    assert 9.9 < h["approach_speed"] < 10.3
    # normal from A (the ground) toward B (the ball): up
    assert h["normal"][1] > 0.99


def test_fast_body_hit_comes_from_the_swept_pass():
    ground = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    ball = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0.52, 0], 1.0)
    ball.velocity[1] = -30.0  # 0.5 m per step: clamped by the time-of-impact pass
    w = world([ground, ball], params=abi.default_params())
    w.step(DT)
    ev = w.contact_events()
    assert [int(e["kind"]) for e in ev] == [abi.CONTACT_HIT]
    assert abs(ev[0]["approach_speed"] - 30.0) < 1e-4
    assert ev[0]["normal"][1] > 0.99


def test_events_only_on_the_emitting_substep():
    a = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0, 0], 0.0)
    b = O.body_new(abi.SHAPE_SPHERE, [0.5], [0.9, 0, 0], 1.0)
    w = world([a, b])
    w.step_fixed(3)  # one emitting substep: one Begin
    ev = w.contact_events()
    assert [e["kind"] for e in ev] == [abi.CONTACT_BEGIN]
    w2 = world([a, b])
    w2.set_emit_period(1)
    w2.step_fixed(3)  # every substep emits; the touch persists: still one Begin
    assert [e["kind"] for e in w2.contact_events()] == [abi.CONTACT_BEGIN]


def test_event_order_is_key_order():
    """Begin/End of one step come out in ascending (a, b) order, hits after."""
    ground = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    balls = []
    for i in range(4):
        b = O.body_new(abi.SHAPE_SPHERE, [0.5], [2.0 * i, 0.52, 0], 1.0)
        b.velocity[1] = -10.0
        balls.append(b)
    w = world([ground] + balls, params=abi.default_params())
    w.step(DT)
    ev = w.contact_events()
    kinds = [int(e["kind"]) for e in ev]
    assert kinds == [abi.CONTACT_BEGIN] * 4 + [abi.CONTACT_HIT] * 4
    keys = [(int(e["body_a"]), int(e["body_b"])) for e in ev[:4]]
    assert keys == sorted(keys) == [(0, 1), (0, 2), (0, 3), (0, 4)]


def test_remove_body_swaps_last_and_reports_trigger_exit():
    """PhysicsEngine::remove_body (avbd/mod.rs:1241-1300)."""
    sensor = O.body_new(abi.SHAPE_SPHERE, [1.0], [0, 0, 0], 0.0)
    sensor.flags = abi.FLAG_TRIGGER
    inside = O.body_new(abi.SHAPE_SPHERE, [0.3], [0.2, 0, 0], 1.0)
    other = O.body_new(abi.SHAPE_SPHERE, [0.3], [9, 0, 0], 2.0)
    w = world([sensor, inside, other])
    w.step(DT)
    assert [int(e["entered"]) for e in w.trigger_events()] == [1]
    w.remove_body(1)
    ev = w.trigger_events()
    assert len(ev) == 1 and ev[0]["entered"] == 0 and (ev[0]["body_a"], ev[0]["body_b"]) == (0, 1)
    b = w.bodies()
    assert len(b) == 2 and b["mass"][1] == 2.0  # the last body took handle 1
    w.remove_body(7)  # invalid handle: no-op
    assert w.nbodies == 2
