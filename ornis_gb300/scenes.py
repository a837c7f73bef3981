"""Seeded synthetic scenes for the AVBD workloads.

No public dataset or benchmark suite is involved: every scene is generated
from a seed.  Body records are built exactly like the reference's
constructors (RigidBody::new_box / new_sphere / new_capsule, body.rs:470-576;
Shape::inertia, collision/shape.rs:713-790), in f32 with the same operation
order, so a record made here equals one made by avbd_body_init.

Workloads (sizes as named by the benchmark configuration):
  pyramid_210      20-row pyramid of 210 unit cubes on a ground plane, 1e-3
                   jitter from seed 0; dt 1/60, 10 iterations.
  large_100k       100,000 bodies (60% boxes half-extents U[0.2,0.8], 30%
                   spheres r U[0.2,0.6], 10% capsules r 0.3 length U[0.5,1.5]),
                   density 1, friction U[0.3,0.8], dropped from a 200x200x50
                   volume above a ground plane, random orientations; seed 1.
  batched_4096     4096 scenes, body count per scene floor(exp(U[ln 8, ln 1025)))
                   (seeded), boxes and spheres with the large_100k size laws,
                   dropped into a 20x20 bin (ground + 4 wall half-spaces) from
                   a jittered column grid; dt 1/120, 2 substeps, 8 iterations;
                   seed 2.
  diff_1024        1024 scenes of a 32-box tower (unit cubes, friction 0.6) on
                   a ground plane hit by a ball (r 0.5, mass 5) whose initial
                   velocity is N((10,0,0), I) per scene (seed 3); every body of
                   a scene shares the friction coefficient 0.6; dt 1/60, 10
                   iterations, 120 steps, a checkpoint every 10 steps; the loss
                   is the sum of squared final tower-body positions.
  ragdoll_8192     2 scenes of 3000 and 5192 ragdolls of 15 capsules with
                   ball and limited hinge joints (seed 4); dt 1/120, 2
                   substeps, 12 iterations.
"""
import math

import numpy as np

from . import abi

F = np.float32

RESTITUTION = {abi.SHAPE_BOX: 0.3, abi.SHAPE_SPHERE: 0.5, abi.SHAPE_CAPSULE: 0.4, abi.SHAPE_HALFSPACE: 0.3,
               abi.SHAPE_CYLINDER: 0.4, abi.SHAPE_CONE: 0.3, abi.SHAPE_HULL: 0.3}
FRICTION = {abi.SHAPE_BOX: 0.5, abi.SHAPE_SPHERE: 0.3, abi.SHAPE_CAPSULE: 0.4, abi.SHAPE_HALFSPACE: 0.6,
            abi.SHAPE_CYLINDER: 0.4, abi.SHAPE_CONE: 0.5, abi.SHAPE_HULL: 0.5}


def _inertia(shape, p, m):
    """Shape::inertia in f32, reference operation order; zeros for m <= 0."""
    p = p.astype(F)
    m = m.astype(F)
    out = np.zeros((len(m), 3), dtype=F)
    pos = m > 0
    sph = (shape == abi.SHAPE_SPHERE) & pos
    v = F(0.4) * m[sph] * p[sph, 0] * p[sph, 0]
    out[sph] = v[:, None]
    box = (shape == abi.SHAPE_BOX) & pos
    s = p[box] * F(2.0)
    x, y, z = s[:, 0] * s[:, 0], s[:, 1] * s[:, 1], s[:, 2] * s[:, 2]
    k = m[box] / F(12.0)
    out[box, 0] = k * (y + z)
    out[box, 1] = k * (z + x)
    out[box, 2] = k * (x + y)
    cap = (shape == abi.SHAPE_CAPSULE) & pos
    r, h, mc = p[cap, 0], p[cap, 1], m[cap]
    iy = F(0.5) * mc * r * r
    ixz = F(0.25) * mc * (r * r) + (mc / F(3.0)) * h * r + F(0.25) * mc * h * h
    out[cap, 0] = ixz
    out[cap, 1] = iy
    out[cap, 2] = ixz
    for kind, axial, tr2, th2, div in ((abi.SHAPE_CYLINDER, 0.5, 3.0, 4.0, 12.0), (abi.SHAPE_CONE, 0.3, 3.0, 8.0, 20.0)):
        sel = (shape == kind) & pos
        r, h, mc = p[sel, 0], p[sel, 1], m[sel]
        ixz = mc * (F(tr2) * r * r + F(th2) * h * h) / F(div)
        out[sel, 0] = ixz
        out[sel, 1] = F(axial) * mc * r * r
        out[sel, 2] = ixz
    return out


def make_bodies(shape, params, position, mass, orientation=None, friction=None):
    """Vectorised RigidBody constructors -> structured array of AvbdBody."""
    n = len(shape)
    shape = np.asarray(shape, dtype=np.uint32)
    params = np.asarray(params, dtype=F).reshape(n, 3)
    mass = np.asarray(mass, dtype=F)
    b = np.zeros(n, dtype=abi.BODY_DTYPE)
    b["position"] = np.asarray(position, dtype=F)
    if orientation is None:
        b["orientation"][:, 3] = 1.0
    else:
        b["orientation"] = np.asarray(orientation, dtype=F)
    free = (mass > 0) & np.isfinite(mass)
    b["mass"] = np.where(free, mass, F(0))
    with np.errstate(divide="ignore"):
        b["inv_mass"] = np.where(free, F(1.0) / np.where(free, mass, F(1)), F(0))
    b["inertia"] = _inertia(shape, params, np.where(free, mass, F(0)))
    b["restitution"] = np.array([RESTITUTION[int(s)] for s in shape], dtype=F)
    fr = np.array([FRICTION[int(s)] for s in shape], dtype=F)
    if friction is not None:
        fr = np.asarray(friction, dtype=F)
    b["friction"] = fr
    b["friction_transverse"] = fr
    b["shape"] = shape
    b["shape_params"] = params
    b["collision_layer"] = 1
    b["collision_mask"] = 0xFFFFFFFF
    b["body_type"] = np.where(mass > 0, abi.BODY_DYNAMIC, abi.BODY_STATIC)
    return b


def halfspace(position, normal):
    nrm = np.asarray(normal, dtype=F)
    r = F(1.0) / np.sqrt((nrm[0] * nrm[0] + nrm[1] * nrm[1]) + nrm[2] * nrm[2])
    return make_bodies([abi.SHAPE_HALFSPACE], [nrm * r], [position], [0.0])


def random_quats(rng, n):
    """Uniform unit quaternions (Shoemake's method), x y z w."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1).astype(F)
    q /= np.linalg.norm(q, axis=1, keepdims=True).astype(F)
    return q


def pyramid_210(seed=0, rows=20):
    rng = np.random.default_rng(seed)
    pos = []
    for r in range(rows):
        for i in range(rows - r):
            pos.append([(i - (rows - 1 - r) / 2.0) * 1.0, 0.5 + r * 1.0, 0.0])
    pos = np.asarray(pos, dtype=np.float64)
    pos += rng.uniform(-1e-3, 1e-3, size=pos.shape)
    n = len(pos)
    ground = halfspace([0, 0, 0], [0, 1, 0])
    cubes = make_bodies([abi.SHAPE_BOX] * n, np.full((n, 3), 0.5), pos.astype(F), np.ones(n))
    return np.concatenate([ground, cubes])


def _mixed(rng, n, with_capsules):
    u = rng.random(n)
    if with_capsules:
        kind = np.where(u < 0.6, abi.SHAPE_BOX, np.where(u < 0.9, abi.SHAPE_SPHERE, abi.SHAPE_CAPSULE))
    else:
        kind = np.where(u < 2.0 / 3.0, abi.SHAPE_BOX, abi.SHAPE_SPHERE)
    params = np.zeros((n, 3))
    box = kind == abi.SHAPE_BOX
    params[box] = rng.uniform(0.2, 0.8, size=(box.sum(), 3))
    sph = kind == abi.SHAPE_SPHERE
    params[sph, 0] = rng.uniform(0.2, 0.6, size=sph.sum())
    cap = kind == abi.SHAPE_CAPSULE
    params[cap, 0] = 0.3
    params[cap, 1] = rng.uniform(0.5, 1.5, size=cap.sum()) / 2.0
    params = params.astype(F)
    vol = np.zeros(n)
    vol[box] = 8 * params[box].prod(axis=1)
    vol[sph] = 4.0 / 3.0 * math.pi * params[sph, 0] ** 3
    r, h = params[cap, 0].astype(np.float64), params[cap, 1].astype(np.float64)
    vol[cap] = math.pi * r * r * 2 * h + 4.0 / 3.0 * math.pi * r ** 3
    mass = vol.astype(F)  # density 1
    friction = rng.uniform(0.3, 0.8, size=n).astype(F)
    return kind, params, mass, friction


def large_100k(seed=1, n=100_000):
    rng = np.random.default_rng(seed)
    kind, params, mass, friction = _mixed(rng, n, with_capsules=True)
    pos = np.stack([rng.uniform(-100, 100, n), rng.uniform(1.0, 51.0, n), rng.uniform(-100, 100, n)], axis=1)
    q = random_quats(rng, n)
    ground = halfspace([0, 0, 0], [0, 1, 0])
    bodies = make_bodies(kind, params, pos.astype(F), mass, q, friction)
    return np.concatenate([ground, bodies])


BIN_HALF = 10.0
BIN_PITCH = 2.8


def bin_scene(rng, n):
    """One batched scene: 5 half-spaces (floor + walls of a 20x20 bin) then n bodies."""
    planes = np.concatenate([
        halfspace([0, 0, 0], [0, 1, 0]),
        halfspace([-BIN_HALF, 0, 0], [1, 0, 0]),
        halfspace([BIN_HALF, 0, 0], [-1, 0, 0]),
        halfspace([0, 0, -BIN_HALF], [0, 0, 1]),
        halfspace([0, 0, BIN_HALF], [0, 0, -1]),
    ])
    kind, params, mass, friction = _mixed(rng, n, with_capsules=False)
    cols = int(round(2 * (BIN_HALF - 1.4) / BIN_PITCH)) + 1  # 7 columns per side
    idx = np.arange(n)
    layer, cell = idx // (cols * cols), idx % (cols * cols)
    cx, cz = cell % cols, cell // cols
    off = -(cols - 1) * BIN_PITCH / 2.0
    pos = np.stack([off + cx * BIN_PITCH, 1.5 + layer * BIN_PITCH, off + cz * BIN_PITCH], axis=1)
    pos += rng.uniform(-0.2, 0.2, size=pos.shape)
    q = random_quats(rng, n)
    return np.concatenate([planes, make_bodies(kind, params, pos.astype(F), mass, q, friction)])


def batched(nscenes=4096, seed=2, lo=8, hi=1024):
    """nscenes bin scenes of log-uniform body counts in [lo, hi]; returns (bodies, scene_offsets, counts)."""
    rng = np.random.default_rng(seed)
    counts = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi + 1), size=nscenes))).astype(np.int64)
    counts = np.clip(counts, lo, hi)
    parts = []
    offs = [0]
    for s in range(nscenes):
        srng = np.random.default_rng([seed, s])
        sc = bin_scene(srng, int(counts[s]))
        parts.append(sc)
        offs.append(offs[-1] + len(sc))
    return np.concatenate(parts), np.asarray(offs, dtype=np.uint32), counts


def diff_towers(nscenes=1024, seed=3, height=32, mu=0.6):
    """The differentiable batch: per scene a ground plane, `height` stacked
    unit cubes and a ball 2 m in front of the tower's base.  Returns
    (bodies, scene_offsets, ball_index, tower_mask)."""
    rng = np.random.default_rng(seed)
    per = height + 2
    kinds = [abi.SHAPE_BOX] * height + [abi.SHAPE_SPHERE]
    params = [[0.5, 0.5, 0.5]] * height + [[0.5, 0.0, 0.0]]
    mass = [1.0] * height + [5.0]
    pos = [[0.0, 0.5 + i, 0.0] for i in range(height)] + [[-2.5, 1.0, 0.0]]
    scene = np.concatenate([halfspace([0, 0, 0], [0, 1, 0]), make_bodies(kinds, params, pos, mass)])
    scene["friction"] = mu
    scene["friction_transverse"] = mu
    bodies = np.tile(scene, nscenes)
    ball = np.arange(nscenes) * per + per - 1
    bodies["velocity"][ball] = (rng.normal(size=(nscenes, 3)) + np.array([10.0, 0.0, 0.0])).astype(F)
    offs = (np.arange(nscenes + 1) * per).astype(np.uint32)
    tower = np.zeros(len(bodies), dtype=bool)
    for k in range(height):
        tower[np.arange(nscenes) * per + 1 + k] = True
    return bodies, offs, ball, tower


def params_for(workload):
    """Solver parameters of a workload (gravity -9.81 y, reference constants)."""
    if workload == "batched_4096":
        return abi.default_params(step_dt=1.0 / 120.0, iterations=8), 2
    if workload == "ragdoll_8192":
        return abi.default_params(step_dt=1.0 / 120.0, iterations=12), 2
    return abi.default_params(step_dt=1.0 / 60.0, iterations=10), 1


def dynamic_count(bodies):
    return int(np.count_nonzero(bodies["body_type"] == abi.BODY_DYNAMIC))


# ---- articulated ragdolls ---------------------------------------------------------
# 15 capsule links; (parent, hinge?) per link; hinges bend about local x with
# limits, the rest are ball joints.  Links hang along -y from their parent's
# bottom end, arms and legs offset sideways from the trunk.
_RAGDOLL = [
    # name, parent, joint kind, x offset from parent bottom, limit
    ("pelvis", -1, None, 0.0, None),
    ("spine", 0, "ball", 0.0, None),
    ("chest", 1, "ball", 0.0, None),
    ("head", 2, "ball", 0.0, None),
    ("l_upper_arm", 2, "ball", -0.35, None),
    ("l_forearm", 4, "hinge", 0.0, (0.0, 2.5)),
    ("l_hand", 5, "ball", 0.0, None),
    ("r_upper_arm", 2, "ball", 0.35, None),
    ("r_forearm", 7, "hinge", 0.0, (0.0, 2.5)),
    ("r_hand", 8, "ball", 0.0, None),
    ("l_thigh", 0, "ball", -0.15, None),
    ("l_shin", 10, "hinge", 0.0, (-2.5, 0.0)),
    ("l_foot", 11, "ball", 0.0, None),
    ("r_thigh", 0, "ball", 0.15, None),
    ("r_shin", 13, "hinge", 0.0, (-2.5, 0.0)),
]


def _rotate(q, v):
    """q (xyzw) applied to v, numpy float64."""
    x, y, z, w = q
    t = 2.0 * np.cross([x, y, z], v)
    return v + w * t + np.cross([x, y, z], t)


def ragdolls(counts=(3000, 5192), seed=4, density=1000.0):
    """Scenes of 15-capsule ragdolls dropped onto a ground plane.

    Capsule radii U[0.05, 0.12], lengths U[0.15, 0.45] (half_height =
    length / 2), mass = density x volume; drop height U[1, 3], random root
    orientation; ragdolls on a 2.5 m grid.  Returns (bodies, scene_offsets,
    joints) with joints as AvbdJointDesc records in global handles.
    """
    rng = np.random.default_rng(seed)
    parts, offs, joints = [], [0], []
    base = 0
    for count in counts:
        side = int(math.ceil(math.sqrt(count)))
        recs = [halfspace([0, 0, 0], [0, 1, 0])]
        nb = 1
        for k in range(count):
            r = rng.uniform(0.05, 0.12, len(_RAGDOLL))
            hh = rng.uniform(0.15, 0.45, len(_RAGDOLL)) / 2.0
            q = random_quats(rng, 1)[0].astype(np.float64)
            drop = rng.uniform(1.0, 3.0)
            root = np.array([(k % side - side / 2) * 2.5, 0.0, (k // side - side / 2) * 2.5])
            # upright layout in the ragdoll frame: link i's top end meets its
            # parent's bottom end (plus the sideways offset)
            top = np.zeros((len(_RAGDOLL), 3))
            centre = np.zeros((len(_RAGDOLL), 3))
            for i, (_, parent, _, dx, _) in enumerate(_RAGDOLL):
                if parent < 0:
                    top[i] = [0.0, 0.0, 0.0]
                else:
                    pb = centre[parent] - [0.0, hh[parent] + r[parent], 0.0]
                    top[i] = pb + [dx, 0.0, 0.0]
                centre[i] = top[i] - [0.0, hh[i] + r[i], 0.0]
            lowest = (centre[:, 1] - hh - r).min()
            first = base + nb
            for i in range(len(_RAGDOLL)):
                p = root + _rotate(q, centre[i]) + [0.0, drop - lowest, 0.0]
                vol = math.pi * r[i] ** 2 * (2 * hh[i]) + 4.0 / 3.0 * math.pi * r[i] ** 3
                b = make_bodies([abi.SHAPE_CAPSULE], [[r[i], hh[i], 0.0]], [p.astype(F)], [density * vol],
                                q[None, :].astype(F))
                recs.append(b)
            for i, (_, parent, kind, dx, lim) in enumerate(_RAGDOLL):
                if parent < 0:
                    continue
                # anchors in each link's frame: the child's top, the parent's bottom (+ offset)
                la = [dx, -(hh[parent] + r[parent]), 0.0]
                lb = [0.0, hh[i] + r[i], 0.0]
                jk = abi.JOINT_REVOLUTE if kind == "hinge" else abi.JOINT_BALL
                joints.append(abi.joint_desc(jk, first + parent, first + i, la, lb, (1, 0, 0), (1, 0, 0), lim))
            nb += len(_RAGDOLL)
        sc = np.concatenate(recs)
        parts.append(sc)
        base += len(sc)
        offs.append(base)
    return np.concatenate(parts), np.asarray(offs, dtype=np.uint32), joints
