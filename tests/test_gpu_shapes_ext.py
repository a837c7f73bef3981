"""Rounded and compound shapes on the CUDA path, per step from identical
state against the oracle (Coloured order): pair sets, contact IDs and
colours identical and poses bit-identical (the exact build computes the
oracle's arithmetic; the 1e-5 bars are asserted too); swept casts of a fast
compound; the registration codes equal the oracle's; a snapshot carries the
shape tables."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld

import oracle_api as O
import parity as P
from test_gpu_convex import hulls
from test_oracle_shapes_ext import ext_body

pytestmark = pytest.mark.gpu

Q45Z = (0.0, 0.0, 0.38268343, 0.9238795)


def shape_tables():
    """(kind, parts) in registration order; ids follow it."""
    S = abi.shape_part
    return [
        ("round", [S(abi.SHAPE_BOX, [0.3, 0.25, 0.35], 0.08)]),
        ("round", [S(abi.SHAPE_CYLINDER, [0.3, 0.25], 0.05)]),
        ("round", [S(abi.SHAPE_CONE, [0.3, 0.3], 0.04)]),
        ("round", [S(abi.SHAPE_HULL, [1], 0.06)]),
        ("round", [S(abi.SHAPE_SPHERE, [0.25], 0.1)]),
        ("compound", [S(abi.SHAPE_BOX, [0.5, 0.12, 0.12]), S(abi.SHAPE_BOX, [0.12, 0.35, 0.12], position=(0.4, 0.45, 0))]),
        ("compound", [S(abi.SHAPE_SPHERE, [0.22], position=(-0.45, 0, 0)), S(abi.SHAPE_SPHERE, [0.22], position=(0.45, 0, 0)),
                      S(abi.SHAPE_CAPSULE, [0.07, 0.35], orientation=(0.0, 0.0, 0.70710677, 0.70710677))]),
        ("compound", [S(abi.SHAPE_BOX, [0.2, 0.2, 0.2], 0.05, position=(0.0, 0.3, 0.0), orientation=Q45Z),
                      S(abi.SHAPE_CYLINDER, [0.2, 0.15], position=(0.0, -0.2, 0.0)),
                      S(abi.SHAPE_HULL, [2], 0.03, position=(0.35, 0.0, 0.1))]),
    ]


def register(w, tables):
    ids = []
    for kind, parts in tables:
        if kind == "round":
            got = w.add_round(parts[0])
        else:
            got = w.add_compound(parts)
        ids.append(got[1] if isinstance(got, tuple) else got)
    return ids


def ext_scene(seed=11, n=30):
    rng = np.random.default_rng(seed)
    tables = shape_tables()
    recs = [O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0),
            O.body_new(abi.SHAPE_BOX, [0.6, 0.6, 0.6], [1.5, 0.6, 0.0], 0.0)]
    for i in range(n):
        k = i % (len(tables) + 2)
        pos = [rng.uniform(-2.5, 2.5), 0.8 + 0.7 * i / 2.0, rng.uniform(-2.5, 2.5)]
        if k < len(tables):
            shape = abi.SHAPE_ROUND if tables[k][0] == "round" else abi.SHAPE_COMPOUND
            b = ext_body(shape, k, pos, 1.0, (0.12, 0.12, 0.12))
        elif k == len(tables):
            b = O.body_new(abi.SHAPE_BOX, [0.3, 0.3, 0.3], pos, 1.0)
        else:
            b = O.body_new(abi.SHAPE_SPHERE, [0.3], pos, 1.0)
        q = scenes.random_quats(rng, 1)[0]
        b.orientation[:] = [float(x) for x in q]
        recs.append(b)
    return tables, O.bodies_to_array(recs)


def make_pair(tables, bodies, params):
    o = O.OracleWorld(params, mode=O.COLOURED)
    g = AvbdWorld(params)
    for verts, faces in hulls():
        o.add_hull(verts, faces, (0.1, 0.1, 0.1))
        g.add_hull(verts, faces, (0.1, 0.1, 0.1))
    assert register(o, tables) == register(g, tables)
    o.add_bodies(bodies)
    g.add_bodies(bodies)
    return o, g


def test_rounded_and_compound_shapes_per_step():
    tables, bodies = ext_scene()
    params = abi.default_params()
    o, g = make_pair(tables, bodies, params)
    seen = 0
    for _ in range(150):
        so, sg = P.step_from_oracle_state(o, g)
        assert max(P.compare_states(so, sg, params.step_dt, o, g)) == 0.0
        seen = max(seen, len(so["pairs"]))
    assert seen > 15


def test_fast_compound_is_swept():
    """A compound thrown at 40 m/s at a thin wall: the swept cast (through
    the compound's parts) clamps it, on the device as in the oracle."""
    tables = shape_tables()
    wall = O.body_new(abi.SHAPE_BOX, [0.05, 2.0, 2.0], [3.0, 1.0, 0.0], 0.0)
    mover = ext_body(abi.SHAPE_COMPOUND, 5, [0.0, 1.0, 0.0], 1.0, (0.12, 0.12, 0.12))
    mover.velocity[:] = [40.0, 0.0, 0.0]
    bodies = O.bodies_to_array([wall, mover])
    params = abi.default_params(gravity=(0.0, 0.0, 0.0))
    o, g = make_pair(tables, bodies, params)
    for _ in range(12):
        so, sg = P.step_from_oracle_state(o, g)
        assert max(P.compare_states(so, sg, params.step_dt, o, g)) == 0.0
    assert g.bodies()["position"][1][0] < 3.0
    assert g.counters().ccd_hits > 0


def test_registration_codes_equal_the_oracle():
    S = abi.shape_part
    nan = float("nan")
    o = O.OracleWorld()
    g = AvbdWorld(abi.default_params())
    rounds = [S(abi.SHAPE_BOX, [1, 1, 1], 0.0), S(abi.SHAPE_BOX, [1, 1, 1], nan),
              S(abi.SHAPE_HALFSPACE, [0, 1, 0], 0.1), S(abi.SHAPE_COMPOUND, [0], 0.1), S(abi.SHAPE_HULL, [3], 0.1),
              S(abi.SHAPE_SPHERE, [0.5], 0.1)]
    for part in rounds:
        want = o.add_round(part)[0]
        try:
            g.add_round(part)
            got = 0
        except AvbdError as e:
            got = e.code
        assert got == want
    compounds = [[], [S(abi.SHAPE_ROUND, [0])], [S(abi.SHAPE_BOX, [1, 1, 1], -0.1)], [S(abi.SHAPE_BOX, [1, 1, 1])]]
    for parts in compounds:
        want = o.add_compound(parts)[0]
        try:
            g.add_compound(parts)
            got = 0
        except AvbdError as e:
            got = e.code
        assert got == want
    # a body naming a shape of the other kind, or none, is refused at the upload
    w = AvbdWorld(abi.default_params())
    w.add_round(S(abi.SHAPE_SPHERE, [0.5], 0.1))
    w.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_COMPOUND, 0, [0, 0, 0], 1.0)]))
    with pytest.raises(AvbdError) as e:
        w.step(1.0 / 60.0)
    assert e.value.code == abi.AVBD_ERR_INVALID_ARG


def test_snapshot_carries_the_shape_tables():
    tables, bodies = ext_scene(seed=3, n=16)
    params = abi.default_params()
    a = AvbdWorld(params)
    for verts, faces in hulls():
        a.add_hull(verts, faces, (0.1, 0.1, 0.1))
    register(a, tables)
    a.add_bodies(bodies)
    for _ in range(30):
        a.step(params.step_dt)
    b = AvbdWorld.from_snapshot(a.snapshot())
    for _ in range(40):
        a.step(params.step_dt)
        b.step(params.step_dt)
    assert a.bodies().tobytes() == b.bodies().tobytes()


def terrain_scene(seed=21, n=24):
    """A sloped heightfield and a mesh floor (static), with spheres, boxes,
    capsules, cylinders, hulls and rounded and compound bodies falling onto
    both."""
    from test_oracle_shapes_ext import floor_grid, slope
    rng = np.random.default_rng(seed)
    tables = shape_tables()
    recs = [ext_body(abi.SHAPE_HEIGHTFIELD, 0, [0.0, 0.0, 0.0], 0.0),
            ext_body(abi.SHAPE_TRIMESH, 0, [12.0, 0.0, 0.0], 0.0)]
    kinds = ["sphere", "box", "capsule", "cylinder", "hull", "ext"]
    for i in range(n):
        x0 = 0.0 if i % 2 == 0 else 12.0
        pos = [x0 + rng.uniform(-3, 3), 1.0 + 0.5 * i, rng.uniform(-3, 3)]
        k = kinds[i % len(kinds)]
        if k == "sphere":
            b = O.body_new(abi.SHAPE_SPHERE, [0.3], pos, 1.0)
        elif k == "box":
            b = O.body_new(abi.SHAPE_BOX, [0.3, 0.25, 0.35], pos, 1.0)
        elif k == "capsule":
            b = O.body_new(abi.SHAPE_CAPSULE, [0.2, 0.3], pos, 1.0)
        elif k == "cylinder":
            b = O.body_new(abi.SHAPE_CYLINDER, [0.3, 0.25], pos, 1.0)
        elif k == "hull":
            b = O.body_new(abi.SHAPE_BOX, [0.3, 0.3, 0.3], pos, 1.0)
            b.shape = abi.SHAPE_HULL
            b.shape_params[:] = [float(i % 3), 0.0, 0.0]
            b.inertia[:] = [0.1, 0.1, 0.1]
        else:
            sid = i % len(tables)
            shape = abi.SHAPE_ROUND if tables[sid][0] == "round" else abi.SHAPE_COMPOUND
            b = ext_body(shape, sid, pos, 1.0, (0.12, 0.12, 0.12))
        b.orientation[:] = [float(x) for x in scenes.random_quats(rng, 1)[0]]
        recs.append(b)
    verts, tris = floor_grid(6, 6.0)
    return tables, O.bodies_to_array(recs), slope(13, 1.0, 0.15), (verts, tris)


def test_heightfield_and_mesh_per_step():
    tables, bodies, heights, (verts, tris) = terrain_scene()
    params = abi.default_params()
    o = O.OracleWorld(params, mode=O.COLOURED)
    g = AvbdWorld(params)
    for verts_h, faces in hulls():
        o.add_hull(verts_h, faces, (0.1, 0.1, 0.1))
        g.add_hull(verts_h, faces, (0.1, 0.1, 0.1))
    register(o, tables)
    register(g, tables)
    assert o.add_heightfield(heights, 1.0) == (0, g.add_heightfield(heights, 1.0))
    assert o.add_trimesh(verts, tris) == (0, g.add_trimesh(verts, tris))
    o.add_bodies(bodies)
    g.add_bodies(bodies)
    seen = 0
    for _ in range(150):
        so, sg = P.step_from_oracle_state(o, g)
        assert max(P.compare_states(so, sg, params.step_dt, o, g)) == 0.0
        seen = max(seen, len(so["pairs"]))
    assert seen > 10
    # a snapshot carries the terrain and the mesh
    b = AvbdWorld.from_snapshot(g.snapshot())
    for _ in range(20):
        g.step(params.step_dt)
        b.step(params.step_dt)
    assert g.bodies().tobytes() == b.bodies().tobytes()


def test_terrain_and_mesh_rules():
    g = AvbdWorld(abi.default_params())
    for bad, code in [((np.zeros((0, 3), np.float32), 1.0), abi.AVBD_ERR_INVALID_ARG),
                      ((np.zeros((2, 2), np.float32), -1.0), abi.AVBD_ERR_INVALID_ARG),
                      ((np.full((2, 2), np.inf, np.float32), 1.0), abi.AVBD_ERR_NONFINITE)]:
        with pytest.raises(AvbdError) as e:
            g.add_heightfield(*bad)
        assert e.value.code == code
    with pytest.raises(AvbdError) as e:
        g.add_trimesh([[0, 0, 0], [1, 0, 0], [0, 0, 1]], [[0, 1, 5]])
    assert e.value.code == abi.AVBD_ERR_INVALID_ARG
    # terrain is static: a dynamic one is refused at the upload
    g.add_heightfield(np.zeros((3, 3), np.float32), 1.0)
    g.add_bodies(O.bodies_to_array([ext_body(abi.SHAPE_HEIGHTFIELD, 0, [0, 0, 0], 1.0)]))
    with pytest.raises(AvbdError) as e:
        g.step(1.0 / 60.0)
    assert e.value.code == abi.AVBD_ERR_UNSUPPORTED
