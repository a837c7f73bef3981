"""Rounded and compound shapes on the oracle: the reference's distance tests
(collision/distance.rs test module: round_distance_offsets_inner_by_radius,
round_penetration_matches_inner_minus_radius, compound_picks_deepest_child,
compound_vs_compound_reports_separation) restated through the oracle's
shape_distance, the registration rules of Shape::try_round / try_compound
(shape.rs:556-575), and a drop onto a floor: a rounded sphere and a rounded
cylinder rest at their rounded heights; a dumbbell compound stays finite
(one witness point per pair, as in the reference, cannot hold two ends)."""
import numpy as np
import pytest

from ornis_gb300 import abi

import oracle_api as O

EPS = 1e-5


def ext_body(shape, sid, pos, mass, unit_inertia=(0.2, 0.2, 0.2)):
    """A body of a rounded or compound shape: the default material of a box,
    the shape's id, its per-unit-mass inertia times the mass."""
    b = O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], pos, mass)
    b.shape = shape
    b.shape_params[:] = [float(sid), 0.0, 0.0]
    b.inertia[:] = [u * mass for u in unit_inertia] if mass > 0 else [0.0, 0.0, 0.0]
    return b


def rounded_box(w, half, r):
    rc, sid = w.add_round(abi.shape_part(abi.SHAPE_BOX, half, r))
    assert rc == 0, rc
    return sid


def two_boxes(w, half=0.5, x=2.0):
    rc, sid = w.add_compound([abi.shape_part(abi.SHAPE_BOX, [half] * 3, position=(-x, 0, 0)),
                              abi.shape_part(abi.SHAPE_BOX, [half] * 3, position=(x, 0, 0))])
    assert rc == 0, rc
    return sid


def test_round_distance_offsets_inner_by_radius():
    w = O.OracleWorld()
    sid = rounded_box(w, [1, 1, 1], 0.5)
    w.add_bodies(O.bodies_to_array([O.body_new(abi.SHAPE_BOX, [1, 1, 1], [0, 0, 0], 0.0),
                                    ext_body(abi.SHAPE_ROUND, sid, [0, 0, 0], 0.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [2, 0, 0], 1.0)]))
    d, _, _ = w.shape_distance(0, 2)
    assert abs(d - 0.75) < EPS
    d, pa, pb = w.shape_distance(1, 2)
    assert abs(d - 0.25) < EPS
    assert np.allclose(pa, [1.5, 0, 0], atol=EPS) and np.allclose(pb, [1.75, 0, 0], atol=EPS)
    n = (pb - pa) / np.linalg.norm(pb - pa)
    assert np.allclose(n, [1, 0, 0], atol=EPS)
    # the other order: the rounded shape second
    d2, pa2, pb2 = w.shape_distance(2, 1)
    assert abs(d2 - 0.25) < EPS and np.allclose(pa2, [1.75, 0, 0], atol=EPS) and np.allclose(pb2, [1.5, 0, 0], atol=EPS)


def test_round_penetration_matches_inner_minus_radius():
    w = O.OracleWorld()
    sid = rounded_box(w, [1, 1, 1], 0.5)
    w.add_bodies(O.bodies_to_array([O.body_new(abi.SHAPE_BOX, [1, 1, 1], [0, 0, 0], 0.0),
                                    ext_body(abi.SHAPE_ROUND, sid, [0, 0, 0], 0.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [1, 0, 0], 1.0)]))
    d_inner, _, _ = w.shape_distance(0, 2)
    d, _, _ = w.shape_distance(1, 2)
    assert abs(d - (d_inner - 0.5)) < EPS and d < 0.0


def test_compound_picks_deepest_child():
    w = O.OracleWorld()
    sid = two_boxes(w)
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_COMPOUND, sid, [0, 0, 0], 0.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [0.75, 0, 0], 1.0)]))
    d, pa, _ = w.shape_distance(0, 1)
    assert abs(d - 0.5) < EPS and np.allclose(pa, [1.5, 0, 0], atol=EPS)
    d2, _, pb2 = w.shape_distance(1, 0)
    assert abs(d2 - 0.5) < EPS and np.allclose(pb2, [1.5, 0, 0], atol=EPS)


def test_compound_vs_compound_reports_separation():
    w = O.OracleWorld()
    one = w.add_compound([abi.shape_part(abi.SHAPE_BOX, [1, 1, 1])])[1]
    two = w.add_compound([abi.shape_part(abi.SHAPE_BOX, [1, 1, 1])])[1]
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_COMPOUND, one, [0, 0, 0], 1.0),
                                    ext_body(abi.SHAPE_COMPOUND, two, [0, 0, 0], 1.0)]))
    assert w.shape_distance(0, 1)[0] == float("inf")


def test_rounded_part_of_a_compound_and_a_rounded_cylinder():
    """A rounded sphere part of a compound peels inside its own query; a
    rounded cylinder goes through GJK for its inner and peels after."""
    w = O.OracleWorld()
    rc, cid = w.add_compound([abi.shape_part(abi.SHAPE_SPHERE, [0.5], 0.25, position=(0, 1, 0))])
    assert rc == 0
    rc, rid = w.add_round(abi.shape_part(abi.SHAPE_CYLINDER, [0.5, 0.5], 0.1))
    assert rc == 0
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_COMPOUND, cid, [0, 0, 0], 1.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [0, 3, 0], 1.0),
                                    ext_body(abi.SHAPE_ROUND, rid, [3, 0, 0], 1.0),
                                    O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [3, 1.7, 0], 1.0)]))
    d, pa, pb = w.shape_distance(0, 1)  # sphere r 0.75 at y 1 vs sphere r 0.25 at y 3
    assert abs(d - 1.0) < EPS and np.allclose(pa, [0, 1.75, 0], atol=EPS) and np.allclose(pb, [0, 2.75, 0], atol=EPS)
    d, _, _ = w.shape_distance(2, 3)  # cylinder top at 0.5 + 0.1 skin vs box bottom at 1.2
    assert abs(d - 0.6) < 1e-4


def test_registration_rules():
    w = O.OracleWorld()
    nan = float("nan")
    assert w.add_round(abi.shape_part(abi.SHAPE_BOX, [1, 1, 1], 0.0))[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_round(abi.shape_part(abi.SHAPE_BOX, [1, 1, 1], nan))[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_round(abi.shape_part(abi.SHAPE_HALFSPACE, [0, 1, 0], 0.1))[0] == abi.AVBD_ERR_UNSUPPORTED
    assert w.add_round(abi.shape_part(abi.SHAPE_COMPOUND, [0], 0.1))[0] == abi.AVBD_ERR_UNSUPPORTED
    assert w.add_compound([])[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_compound([abi.shape_part(abi.SHAPE_ROUND, [0])])[0] == abi.AVBD_ERR_UNSUPPORTED
    assert w.add_compound([abi.shape_part(abi.SHAPE_HULL, [5])])[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_compound([abi.shape_part(abi.SHAPE_BOX, [1, 1, 1], -0.1)])[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_compound([abi.shape_part(abi.SHAPE_BOX, [1, 1, 1], 0.1)]) == (0, 0)


def rest_scene():
    """A rounded sphere, a dumbbell compound of two spheres and a rounded
    cylinder dropped on a floor (their single witness point per pair holds
    them: corner expansion is for box bodies only, rows.rs:346-363, so a
    rounded box or a compound of boxes tips over its support corner as in
    the reference)."""
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED)
    rs = w.add_round(abi.shape_part(abi.SHAPE_SPHERE, [0.3], 0.1))[1]
    db = w.add_compound([abi.shape_part(abi.SHAPE_SPHERE, [0.25], position=(-0.5, 0.0, 0.0)),
                         abi.shape_part(abi.SHAPE_SPHERE, [0.25], position=(0.5, 0.0, 0.0)),
                         abi.shape_part(abi.SHAPE_CAPSULE, [0.08, 0.4], orientation=(0.0, 0.0, 0.7071068, 0.7071068))])[1]
    cy = w.add_round(abi.shape_part(abi.SHAPE_CYLINDER, [0.3, 0.2], 0.05))[1]
    recs = [O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0),
            ext_body(abi.SHAPE_ROUND, rs, [0, 2.0, 0], 1.0, (0.064, 0.064, 0.064)),
            ext_body(abi.SHAPE_COMPOUND, db, [3, 1.5, 0], 1.0, (0.03, 0.3, 0.3)),
            ext_body(abi.SHAPE_ROUND, cy, [-3, 1.0, 0], 1.0, (0.04, 0.05, 0.04))]
    return w, recs


def test_shapes_come_to_rest():
    w, recs = rest_scene()
    w.add_bodies(O.bodies_to_array(recs))
    for _ in range(300):
        w.step(1.0 / 60.0)
    b = w.bodies()
    assert abs(b["position"][1][1] - 0.4) < 0.02, b["position"][1]  # radius 0.3 + skin 0.1
    assert abs(b["position"][3][1] - 0.25) < 0.03, b["position"][3]  # half height 0.2 + skin 0.05
    assert np.linalg.norm(b["velocity"][1]) < 0.05 and np.linalg.norm(b["velocity"][3]) < 0.05
    # the compound meets the floor through its deepest part's single witness
    # point (rows.rs:571-715): it rocks between its ends but stays bounded
    assert np.all(np.isfinite(b["position"][2])) and -0.3 < b["position"][2][1] < 0.3


# ---- heightfields and triangle meshes -----------------------------------------

def slope(n=9, cell=1.0, rise=0.1):
    xs = (np.arange(n) - (n - 1) / 2.0) * cell
    return np.array([[rise * x for x in xs] for _ in xs], dtype=np.float32)


def floor_grid(m=5, half=5.0):
    """m x m quads of a flat floor at y = 0 spanning [-half, half]^2."""
    g = np.linspace(-half, half, m + 1)
    verts = [[x, 0.0, z] for z in g for x in g]
    tris = []
    for i in range(m):
        for j in range(m):
            a = i * (m + 1) + j
            tris += [[a, a + m + 1, a + 1], [a + 1, a + m + 1, a + m + 2]]
    return verts, tris


def test_heightfield_distance_and_rules():
    """Columns are solid boxes from the lowest sample up (distance.rs:246-350);
    a flat plain is a one-cell skirt; terrain against terrain is separation."""
    w = O.OracleWorld()
    assert w.add_heightfield(slope(), 1.0) == (0, 0)
    assert w.add_heightfield(np.zeros((4, 4), np.float32), 1.0) == (0, 1)
    assert w.add_heightfield(np.zeros((0, 4), np.float32), 1.0)[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_heightfield(np.zeros((2, 2), np.float32), 0.0)[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_heightfield(np.full((2, 2), np.nan, np.float32), 1.0)[0] == abi.AVBD_ERR_NONFINITE
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_HEIGHTFIELD, 0, [0, 0, 0], 0.0),
                                    ext_body(abi.SHAPE_HEIGHTFIELD, 1, [20, 0, 0], 0.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.3], [1.2, 2, 0.4], 1.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [20, 1, 0], 1.0)]))
    d, pa, pb = w.shape_distance(0, 2)  # the column under x = 1.2 tops out at 0.1 (sample x = 1)
    assert abs(d - 1.6) < EPS and abs(pa[1] - 0.1) < EPS and abs(pb[1] - 1.7) < EPS
    d2, pa2, pb2 = w.shape_distance(2, 0)
    assert abs(d2 - 1.6) < EPS and np.allclose(pa2, pb, atol=EPS) and np.allclose(pb2, pa, atol=EPS)
    assert abs(w.shape_distance(1, 3)[0] - 0.75) < EPS  # flat: the skirt's top at 0
    assert w.shape_distance(0, 1)[0] == float("inf")


def test_trimesh_distance_and_rules():
    """The nearest triangle under the convex side's window (distance.rs:416-517);
    the witnesses come back in the reference's order (the convex side's first
    when the mesh is first, the mesh's first when it is second)."""
    w = O.OracleWorld()
    verts, tris = floor_grid()
    assert w.add_trimesh(verts, tris) == (0, 0)
    assert w.add_trimesh([[0, 0, 0], [1, 0, 0], [0, 0, 1]], [[0, 1, 3]])[0] == abi.AVBD_ERR_INVALID_ARG
    assert w.add_trimesh([[0, 0, 0], [1, np.nan, 0], [0, 0, 1]], [[0, 1, 2]])[0] == abi.AVBD_ERR_NONFINITE
    # a sliver is dropped, the mesh stays valid
    assert w.add_trimesh([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 0, 1]], [[0, 1, 2], [0, 1, 3]]) == (0, 1)
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_TRIMESH, 0, [0, 0, 0], 0.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [0.3, 0.2, -0.7], 1.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.25], [0.3, 0.5, -0.7], 1.0)]))
    d, pa, pb = w.shape_distance(0, 1)  # 5 cm deep
    assert abs(d + 0.05) < 1e-4
    assert abs(pb[1]) < 1e-5 and abs(pa[1]) > 1e-3  # the sphere's witness first, the mesh's on its plane
    d2, pa2, pb2 = w.shape_distance(1, 0)
    assert d2 == d and np.array_equal(pa2, pb) and np.array_equal(pb2, pa)  # the mesh's first
    # a sphere whose box misses the triangles' boxes sees no mesh at all
    assert w.shape_distance(0, 2)[0] == float("inf")


def test_bodies_rest_on_terrain_and_mesh():
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED)
    w.add_heightfield(slope(), 1.0)
    verts, tris = floor_grid()
    w.add_trimesh(verts, tris)
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_HEIGHTFIELD, 0, [0, 0, 0], 0.0),
                                    ext_body(abi.SHAPE_TRIMESH, 0, [20, 0, 0], 0.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.3], [1, 2, 0], 1.0),
                                    O.body_new(abi.SHAPE_BOX, [0.3, 0.3, 0.3], [-1, 2, 1], 1.0),
                                    O.body_new(abi.SHAPE_SPHERE, [0.3], [20, 1, 0], 1.0),
                                    O.body_new(abi.SHAPE_BOX, [0.3, 0.3, 0.3], [21, 1, 1], 1.0)]))
    for _ in range(240):
        w.step_fixed(1)
    b = w.bodies()
    assert abs(b["position"][2][1] - 0.4) < 0.02  # on the column of height 0.1
    assert abs(b["position"][3][1] - 0.2) < 0.02  # on the column of height -0.1
    assert abs(b["position"][4][1] - 0.3) < 0.03 and abs(b["position"][5][1] - 0.3) < 0.03  # on the mesh floor
    assert np.all(np.linalg.norm(b["velocity"][2:], axis=1) < 0.05)
