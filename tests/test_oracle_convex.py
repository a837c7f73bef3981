"""The oracle's convex narrowphase (GJK / EPA, cylinders, cones, hulls)
against the reference's own tests (crates/physics/src/collision/gjk.rs test
module) and basic geometric facts."""
import math

import numpy as np
import pytest

from ornis_gb300 import abi, scenes

import oracle_api as O


def world_with(recs, hulls=()):
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED)
    for verts in hulls:
        w.add_hull(verts)
    w.add_bodies(np.concatenate(recs))
    return w


def body(shape, params, pos, mass=1.0):
    return scenes.make_bodies([shape], [list(params) + [0.0] * (3 - len(params))], [pos], [mass])


CUBE = [[x, y, z] for x in (-1.0, 1.0) for y in (-1.0, 1.0) for z in (-1.0, 1.0)]


def test_sphere_vs_cylinder_separation():  # gjk.rs gjk_sphere_vs_cylinder_separation
    w = world_with([body(abi.SHAPE_SPHERE, [1.0], [4, 0, 0]), body(abi.SHAPE_CYLINDER, [1.0, 1.0], [0, 0, 0])])
    d, n, pa, pb = w.convex_distance(0, 1)
    assert abs(d - 2.0) < 1e-4
    assert np.linalg.norm(pa - [3, 0, 0]) < 1e-3 and np.linalg.norm(pb - [1, 0, 0]) < 1e-3


def test_tetra_vertex_buried_reports_penetration():  # gjk.rs gjk_tetra_vertex_buried_reports_penetration
    r = 1.0 / math.sqrt(2.0)
    tet = [[1, 0, -r], [-1, 0, -r], [0, 1, r], [0, -1, r]]
    w = world_with([body(abi.SHAPE_BOX, [5, 0.5, 5], [0, -0.5, 0], 0.0), body(abi.SHAPE_HULL, [0], [0, 0.6, 0])],
                   hulls=[tet])
    d, n, pa, pb = w.convex_distance(0, 1)
    assert abs(d + 0.4) < 1e-3
    assert n[1] > 0.999


def test_cube_hull_matches_box_oracle():  # gjk.rs gjk_cube_hull_matches_box_oracle
    w = world_with([body(abi.SHAPE_HULL, [0], [0, 0, 0]), body(abi.SHAPE_SPHERE, [0.5], [3, 0, 0])], hulls=[CUBE])
    d, *_ = w.convex_distance(0, 1)
    assert abs(d - 1.5) < 1e-3


def test_epa_box_box_penetration():  # gjk.rs epa_reports_box_box_penetration
    w = world_with([body(abi.SHAPE_BOX, [1, 1, 1], [0, 0, 0]), body(abi.SHAPE_BOX, [1, 1, 1], [1.5, 0, 0])])
    d, *_ = w.convex_distance(0, 1)
    assert d < 0.0 and abs(d + 0.5) < 1e-3


def test_epa_cylinder_box_overlap_returns():  # gjk.rs epa_cylinder_box_overlap_returns
    w = world_with([body(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [-4.7e-5, 0.453, 2.6e-6]),
                    body(abi.SHAPE_CYLINDER, [0.5, 0.5], [6.3e-7, 1.414, -1.2e-8])])
    d, n, *_ = w.convex_distance(0, 1)
    assert math.isfinite(d) and np.all(np.isfinite(n))
    assert d < 0.0 and n[1] > 0.99


def test_refined_witnesses_on_surfaces():
    """shape_distance re-seats GJK witnesses onto both surfaces (distance.rs:364-421)."""
    w = world_with([body(abi.SHAPE_CYLINDER, [0.5, 1.0], [0, 0, 0]), body(abi.SHAPE_CONE, [0.5, 0.5], [2.0, 0.2, 0])])
    d, pa, pb = w.shape_distance(0, 1)
    assert 0.0 < d < 1.2
    # pa on the cylinder wall, pb on the cone
    assert abs(math.hypot(pa[0], pa[2]) - 0.5) < 1e-4


@pytest.mark.parametrize("shape,params", [(abi.SHAPE_CYLINDER, [0.4, 0.5]), (abi.SHAPE_CONE, [0.5, 0.5])])
def test_new_shapes_rest_on_ground(shape, params):
    ground = scenes.halfspace([0, 0, 0], [0, 1, 0])
    b = body(shape, params, [0, 0.6, 0])
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED)
    w.add_bodies(np.concatenate([ground, b]))
    for _ in range(120):
        w.step(1.0 / 60.0)
    y = w.bodies()["position"][1, 1]
    assert abs(y - params[1]) < 0.02, y
