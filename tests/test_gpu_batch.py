"""Batching, graph replay, launch shapes, checkpoint/restore and input
validation of the CUDA path."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld

import parity as P

pytestmark = pytest.mark.gpu


def small_batch(n=6, seed=5):
    bodies, offs, counts = scenes.batched(n, seed=seed, lo=8, hi=120)
    params, nsub = scenes.params_for("batched_4096")
    return bodies, offs, params, nsub


def test_batch_equals_one_world_per_scene():
    """Scenes packed into one flat SoA step exactly like scenes stepped alone."""
    bodies, offs, params, nsub = small_batch()
    batch = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    singles = [AvbdWorld(params, bodies=bodies[offs[s]:offs[s + 1]]) for s in range(len(offs) - 1)]
    for _ in range(30):
        batch.step_fixed(nsub)
        for w in singles:
            w.step_fixed(nsub)
    got = batch.bodies()
    for s, w in enumerate(singles):
        assert got[offs[s]:offs[s + 1]].tobytes() == w.bodies().tobytes(), f"scene {s}"


def test_graph_replay_equals_plain_launches():
    bodies, offs, params, nsub = small_batch(seed=9)
    a = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    b = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    for _ in range(40):
        a.step_fixed(nsub)
        b.step_graph(nsub)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    assert b.graph_nodes() > 0


@pytest.mark.parametrize("lanes,fast", [(4, 0), (8, 0), (32, 0), (1, 1), (4, 1), (0, 0), (0, 1)])
def test_lane_and_precision_variants_within_tolerance(lanes, fast):
    """Lane-parallel and split primal, and the fast build: different rounding, same integer outputs."""
    rng = np.random.default_rng([2, 11])
    bodies = scenes.bin_scene(rng, 150)
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    o, g = P.make_pair(bodies, params)
    g.set_tuning(lanes, 128)
    g.set_precision(fast)
    for _ in range(40):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)


def test_checkpoint_restore_is_exact():
    bodies, offs, params, nsub = small_batch(seed=13)
    a = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    for _ in range(25):
        a.step_fixed(nsub)
    snap = a.export_state()
    for _ in range(20):
        a.step_fixed(nsub)
    b = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    b.import_state(snap)
    for _ in range(20):
        b.step_fixed(nsub)
    assert a.bodies().tobytes() == b.bodies().tobytes()


def test_nonfinite_input_is_rejected():
    bodies, offs, params, nsub = small_batch(n=2)
    w = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    bad = w.bodies()
    bad["position"][7, 1] = np.nan
    with pytest.raises(AvbdError) as e:
        w.set_bodies(bad)
    assert e.value.code == abi.AVBD_ERR_NONFINITE
    w.step_fixed(nsub)  # the world is still usable
    assert np.all(np.isfinite(w.bodies()["position"]))


def test_add_bodies_after_stepping_keeps_state():
    params = abi.default_params()
    recs = np.concatenate([scenes.halfspace([0, 0, 0], [0, 1, 0]),
                           scenes.make_bodies([abi.SHAPE_BOX], [[0.5, 0.5, 0.5]], [[0, 0.5, 0]], [1.0])])
    w = AvbdWorld(params)
    w.add_bodies(recs)
    w.step_fixed(10)
    st = w.export_state()
    h = w.add_bodies(scenes.make_bodies([abi.SHAPE_SPHERE], [[0.3, 0, 0]], [[2, 3, 0]], [1.0]))
    assert h == 2
    st2 = w.export_state()
    assert st2["pairs"].tobytes() == st["pairs"].tobytes()
    w.step_fixed(5)
    assert w.body_count == 3


def test_step_with_bad_dt_is_noop():
    bodies, offs, params, nsub = small_batch(n=2)
    w = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    before = w.bodies().tobytes()
    for dt in (0.0, -1.0, float("nan"), float("inf")):
        w.step(dt)
    assert w.bodies().tobytes() == before


def test_work_order_does_not_change_results():
    """Bodies of one colour are independent: their launch order cannot matter."""
    bodies, offs, params, nsub = small_batch(seed=21)
    a = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    b = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    b.set_work_order(1)
    for _ in range(30):
        a.step_fixed(nsub)
        b.step_graph(nsub)
    assert a.bodies().tobytes() == b.bodies().tobytes()
