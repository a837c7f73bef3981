"""Scenes above the one-CTA sweep limit (2048 bodies): the device-wide radix
sort + sweep path of the broadphase, against the one-CTA sweep and the
oracle, and the 100k-body scene of the large single-scene workload."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdWorld

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu


def test_device_wide_sweep_equals_one_cta_sweep():
    rng = np.random.default_rng([9, 1])
    bodies = scenes.bin_scene(rng, 600)
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    a = AvbdWorld(params, bodies=bodies)
    b = AvbdWorld(params, bodies=bodies)
    b.set_broadphase(0)  # every scene through the radix sort
    for _ in range(30):
        a.step_fixed(2)
        b.step_fixed(2)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    ca, cb = a.counters(), b.counters()
    assert (ca.candidates, ca.pairs, ca.points) == (cb.candidates, cb.pairs, cb.points)


@pytest.mark.parametrize("scene", ["bin600", "large_100k", "far"])
def test_row_sweep_equals_x_sweep(scene):
    """The Morton-ordered cell-row sweep of large scenes gives the one-axis
    sweep's candidate set: same counters and the same bodies bit for bit,
    step after step (a bin forced through the device-wide path, the 100k
    drop, and a scene far from the origin with one wide body)."""
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    steps, nsub = 30, 2
    if scene == "bin600":
        bodies = scenes.bin_scene(np.random.default_rng([9, 1]), 600)
    elif scene == "large_100k":
        bodies = scenes.large_100k()
        params, nsub, steps = abi.default_params(), 1, 12
    else:
        rng = np.random.default_rng(5)
        n = 3000
        kind, prm, mass, fric = scenes._mixed(rng, n, with_capsules=True)
        pos = np.stack([rng.uniform(-20, 20, n) + 4.0e4, rng.uniform(0.8, 6.0, n), rng.uniform(-20, 20, n) - 3.0e4],
                       axis=1)
        slab = scenes.make_bodies([abi.SHAPE_BOX], [[6.0, 0.5, 6.0]], [[4.0e4, 8.0, -3.0e4]], [50.0])
        bodies = np.concatenate([scenes.halfspace([0, 0, 0], [0, 1, 0]), slab,  # the slab sets the cell size
                                 scenes.make_bodies(kind, prm, pos.astype(np.float32), mass,
                                                    scenes.random_quats(rng, n), fric)])
    a = AvbdWorld(params, bodies=bodies)
    b = AvbdWorld(params, bodies=bodies)
    for w in (a, b):
        w.set_broadphase(0)  # every scene through the device-wide sort
    b.set_sweep(0)
    for _ in range(steps):
        a.step_fixed(nsub)
        b.step_fixed(nsub)
        ca, cb = a.counters(), b.counters()
        assert (ca.candidates, ca.pairs, ca.points) == (cb.candidates, cb.pairs, cb.points)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    assert ca.candidates > 0


def test_large_scene_per_step_parity():
    """2,501 bodies in one scene: the radix path, per step against the oracle."""
    n = 2500
    rng = np.random.default_rng(17)
    kind, prm, mass, fric = scenes._mixed(rng, n, with_capsules=True)
    pos = np.stack([rng.uniform(-12, 12, n), rng.uniform(0.8, 9.0, n), rng.uniform(-12, 12, n)], axis=1)
    bodies = np.concatenate([scenes.halfspace([0, 0, 0], [0, 1, 0]),
                             scenes.make_bodies(kind, prm, pos.astype(np.float32), mass,
                                                scenes.random_quats(rng, n), fric)])
    params = abi.default_params()
    o = O.OracleWorld(params, mode=O.COLOURED, threads=8)
    o.add_bodies(bodies)
    g = AvbdWorld(params)
    g.add_bodies(bodies)
    for _ in range(6):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
    assert len(so["pairs"]) > 100


def test_large_100k_scene_runs():
    bodies = scenes.large_100k()
    params = abi.default_params()
    w = AvbdWorld(params, bodies=bodies)
    for _ in range(20):
        w.step_graph(1)
    b = w.bodies()
    assert np.all(np.isfinite(b["position"])) and np.all(np.isfinite(b["orientation"]))
    c = w.counters()
    assert c.pairs > 0 and c.breakdowns == 0
