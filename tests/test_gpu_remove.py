"""PhysicsEngine::remove_body on the CUDA path against the oracle
(avbd/mod.rs:1241-1300): after a removal both keep stepping in step."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu


def test_remove_body_then_step_matches_oracle():
    bodies = scenes.pyramid_210(rows=6)
    params = abi.default_params()
    o, g = P.make_pair(bodies, params)
    for _ in range(20):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
    for h in (3, 7):
        o.remove_body(h)
        g.remove_body(h)
        assert g.body_count == o.nbodies
        np.testing.assert_array_equal(g.bodies()["mass"], o.bodies()["mass"])
        # the state right after the removal: the reference keeps a renumbered
        # pair whose (a, b) order flipped until its next discovery drops it;
        # the device drops it at once (its pair list is kept in (a, b) order).
        # Everything else is the same state.
        so, sg = o.export_state(), g.export_state()
        keep = so["pairs"]["a"] < so["pairs"]["b"]
        so = dict(so, pairs=so["pairs"][keep],
                  points=so["points"].reshape(-1, abi.MAX_POINTS)[keep].reshape(-1))
        ro, io = P.pair_table(so)
        rg, ig = P.pair_table(sg)
        assert np.array_equal(ro, rg) and np.array_equal(io, ig)
        assert P.pose_errors(sg["bodies"], so["bodies"], params.step_dt) == (0.0, 0.0)
        # the first step after a removal runs from each side's own state: the
        # reference keeps renumbered pairs whose (a, b) order flipped until its
        # next discovery drops them, the device drops them at once
        o.step_fixed(1)
        g.step_fixed(1)
        P.compare_states(o.export_state(), g.export_state(), params.step_dt, o, g)
        for _ in range(15):
            so, sg = P.step_from_oracle_state(o, g)
            P.compare_states(so, sg, params.step_dt, o, g)


def test_remove_body_trigger_exit_and_batch_rejected():
    sensor = O.body_new(abi.SHAPE_SPHERE, [1.0], [0, 0, 0], 0.0)
    sensor.flags = abi.FLAG_TRIGGER
    inside = O.body_new(abi.SHAPE_SPHERE, [0.3], [0.2, 0, 0], 1.0)
    other = O.body_new(abi.SHAPE_SPHERE, [0.3], [9, 0, 0], 2.0)
    p = abi.default_params()
    p.gravity[1] = 0.0
    w = AvbdWorld(p, bodies=O.bodies_to_array([sensor, inside, other]))
    w.step(1.0 / 60.0)
    assert [int(e["entered"]) for e in w.trigger_events()] == [1]
    w.remove_body(1)
    ev = w.trigger_events()
    assert len(ev) == 1 and ev[0]["entered"] == 0 and (ev[0]["body_a"], ev[0]["body_b"]) == (0, 1)
    assert w.body_count == 2 and w.bodies()["mass"][1] == 2.0
    w.step(1.0 / 60.0)
    bodies, offs, _ = scenes.batched(2, seed=1, lo=8, hi=16)
    b = AvbdWorld(p, bodies=bodies, scene_offsets=offs)
    with pytest.raises(AvbdError) as e:
        b.remove_body(0)
    assert e.value.code == abi.AVBD_ERR_UNSUPPORTED
