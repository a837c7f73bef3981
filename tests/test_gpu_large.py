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
