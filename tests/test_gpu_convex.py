"""Cylinders, cones and convex hulls (GJK / EPA narrowphase) on the CUDA
path, per step against the oracle: pair sets, contact IDs and colours
identical, poses within 1e-5."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdWorld

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu


def hull_faces(verts):
    spatial = pytest.importorskip("scipy.spatial")
    return spatial.ConvexHull(np.asarray(verts, dtype=np.float64)).simplices.astype(np.uint32)


def hulls():
    r = 1.0 / np.sqrt(2.0)
    tet = np.array([[1, 0, -r], [-1, 0, -r], [0, 1, r], [0, -1, r]], dtype=np.float32) * 0.5
    cube = np.array([[x, y, z] for x in (-0.4, 0.4) for y in (-0.3, 0.3) for z in (-0.5, 0.5)], dtype=np.float32)
    rng = np.random.default_rng(4)
    pts = rng.normal(size=(14, 3)).astype(np.float32)
    pts = pts / np.linalg.norm(pts, axis=1, keepdims=True) * np.float32(0.45)
    pts -= pts.mean(axis=0)
    return [(tet, hull_faces(tet)), (cube, hull_faces(cube)), (pts, hull_faces(pts))]


def convex_scene(n=36, seed=3):
    rng = np.random.default_rng(seed)
    kinds = [abi.SHAPE_CYLINDER, abi.SHAPE_CONE, abi.SHAPE_HULL, abi.SHAPE_BOX, abi.SHAPE_SPHERE]
    recs = [scenes.halfspace([0, 0, 0], [0, 1, 0])]
    for i in range(n):
        k = kinds[i % len(kinds)]
        pos = [rng.uniform(-2, 2), 0.6 + 0.9 * i / 3.0, rng.uniform(-2, 2)]
        if k == abi.SHAPE_CYLINDER:
            b = scenes.make_bodies([k], [[0.3, 0.35, 0]], [pos], [1.0])
        elif k == abi.SHAPE_CONE:
            b = scenes.make_bodies([k], [[0.35, 0.3, 0]], [pos], [1.0])
        elif k == abi.SHAPE_HULL:
            hid = i % 3
            b = scenes.make_bodies([k], [[float(hid), 0, 0]], [pos], [1.0])
            b["inertia"] = np.float32(0.1)
            b["rolling_friction"] = 0.2  # body.rs:650-653 (hull debris recipe)
            b["torsion_friction"] = 0.05
        elif k == abi.SHAPE_BOX:
            b = scenes.make_bodies([k], [[0.3, 0.25, 0.35]], [pos], [1.0])
        else:
            b = scenes.make_bodies([k], [[0.3, 0, 0]], [pos], [1.0])
        b["orientation"] = scenes.random_quats(rng, 1)
        recs.append(b)
    return np.concatenate(recs)


def make_pair(bodies, params):
    o = O.OracleWorld(params, mode=O.COLOURED)
    g = AvbdWorld(params)
    for verts, faces in hulls():
        o.add_hull(verts, faces, (0.1, 0.1, 0.1))
        g.add_hull(verts, faces, (0.1, 0.1, 0.1))
    o.add_bodies(bodies)
    g.add_bodies(bodies)
    return o, g


def test_convex_shapes_per_step():
    bodies = convex_scene()
    params = abi.default_params()
    o, g = make_pair(bodies, params)
    seen = 0
    for _ in range(150):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)
        seen = max(seen, len(so["pairs"]))
    assert seen > 20


def test_resting_convex_shapes_free_run_graph():
    """Upright cylinders, cones and box hulls on the ground (no tumbling, so
    rounding differences do not grow) run freely for 120 steps with graph
    replay: within 1e-3 of the oracle.  (A hull resting on a half-space
    touches it at one support vertex, as in the reference, and sinks slowly:
    the comparison is of the trajectory, whatever it does.)"""
    recs = [scenes.halfspace([0, 0, 0], [0, 1, 0])]
    for i in range(6):
        x = -3.0 + 1.2 * i
        recs.append(scenes.make_bodies([abi.SHAPE_CYLINDER], [[0.3, 0.35, 0]], [[x, 0.37, -1.0]], [1.0]))
        recs.append(scenes.make_bodies([abi.SHAPE_CONE], [[0.35, 0.3, 0]], [[x, 0.32, 0.0]], [1.0]))
        hb = scenes.make_bodies([abi.SHAPE_HULL], [[1.0, 0, 0]], [[x, 0.32, 1.0]], [1.0])
        hb["inertia"] = np.float32(0.1)
        recs.append(hb)
    bodies = np.concatenate(recs)
    params = abi.default_params()
    o, g = make_pair(bodies, params)
    o.step_fixed(120)
    g.step_graph(120)
    pe, _ = P.pose_errors(g.bodies(), o.bodies(), params.step_dt)
    assert pe <= 1e-3


def test_hull_index_out_of_range_is_rejected():
    from ornis_gb300.avbd import AvbdError

    b = scenes.make_bodies([abi.SHAPE_HULL], [[5.0, 0, 0]], [[0, 1, 0]], [1.0])
    g = AvbdWorld(abi.default_params(), bodies=b)
    with pytest.raises(AvbdError) as e:
        g.step_fixed(1)
    assert e.value.code == abi.AVBD_ERR_INVALID_ARG
