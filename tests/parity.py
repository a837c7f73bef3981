"""Parity helpers: step the CUDA path and the CPU oracle from identical state.

Bars (stated once, used by every parity test):
  * integer outputs — contact pair set (a, b), points per pair, contact IDs
    (the previous-step slot each point inherited its warm state from) and
    body colours — must be identical;
  * positions and orientations within POSE_RTOL relative, the scale being
    max(1, |reference value|);
  * velocities are BDF1 differences (x - x0)/dt, so their tolerance is the pose
    tolerance divided by dt.
"""
import numpy as np

from ornis_gb300 import abi
from ornis_gb300.avbd import AvbdWorld

import oracle_api as O

POSE_RTOL = 1e-5


def state13(bodies):
    return np.concatenate([bodies["position"], bodies["orientation"], bodies["velocity"],
                           bodies["angular_velocity"]], axis=1).astype(np.float64)


def pose_errors(got, ref, dt):
    """Max relative pose error and max velocity error normalised by the pose tolerance scale."""
    g, r = state13(got), state13(ref) if ref.dtype == abi.BODY_DTYPE else ref
    scale = np.maximum(1.0, np.abs(r))
    e = np.abs(g - r) / scale
    pose = float(e[:, :7].max()) if len(e) else 0.0
    vel = float(e[:, 7:].max() * dt) if len(e) else 0.0
    return pose, vel


def pair_table(st):
    """(a, b, npoints) rows and matched IDs, canonical (a, b) order."""
    pairs = st["pairs"]
    order = np.lexsort((pairs["b"], pairs["a"]))
    rows = np.stack([pairs["a"][order], pairs["b"][order], pairs["npoints"][order]], axis=1)
    pts = st["points"].reshape(-1, abi.MAX_POINTS)[order]
    ids = np.where(np.arange(abi.MAX_POINTS)[None, :] < rows[:, 2:3], pts["matched"], -2)
    return rows.astype(np.int64), ids.astype(np.int64)


def make_pair(bodies, params, joints=(), use_double=False):
    o = O.OracleWorld(params, mode=O.COLOURED, use_double=use_double)
    o.add_bodies(bodies)
    g = AvbdWorld(params)
    g.add_bodies(bodies)
    for j in joints:
        rc, _ = o.add_joint(j)
        assert rc == 0
        g.add_joint(j)
    return o, g


def step_from_oracle_state(o, g, nsub=1):
    """Load the oracle's full state into the GPU world, step both, return both states."""
    st = o.export_state()
    g.import_state(st)
    o.step_fixed(nsub)
    g.step_fixed(nsub)
    return o.export_state(), g.export_state()


def compare_states(so, sg, dt, o=None, g=None, rtol=POSE_RTOL):
    """Assert the parity bars; returns (pose_err, vel_err)."""
    ro, io = pair_table(so)
    rg, ig = pair_table(sg)
    assert ro.shape == rg.shape, f"pair count {len(ro)} (oracle) vs {len(rg)} (gpu)"
    assert np.array_equal(ro, rg), "pair set / point counts differ"
    assert np.array_equal(io, ig), "contact IDs differ"
    if o is not None and g is not None:
        co, cg = o.colours(), g.colours()
        assert np.array_equal(co, cg), f"colours differ at {np.nonzero(co != cg)[0][:10]}"
    pe, ve = pose_errors(sg["bodies"], so["bodies"], dt)
    assert pe <= rtol, f"pose error {pe:.3e} > {rtol}"
    assert ve <= rtol, f"velocity error (x dt) {ve:.3e} > {rtol}"
    return pe, ve


def scene_state(st, offs, s):
    """Scene s of a multi-scene state with scene-local handles (what a
    one-scene world of that scene would export).  Contact IDs are point slots
    within a pair, so they need no renumbering."""
    a0, a1 = int(offs[s]), int(offs[s + 1])
    pairs = st["pairs"]
    m = (pairs["a"] >= a0) & (pairs["a"] < a1)
    sp = pairs[m].copy()
    sp["a"] -= a0
    sp["b"] -= a0
    pts = st["points"].reshape(-1, abi.MAX_POINTS)[m].reshape(-1).copy()
    return dict(bodies=st["bodies"][a0:a1].copy(), aux=st["aux"][a0:a1].copy(), pairs=sp, points=pts,
                joints=np.zeros(0, dtype=abi.JOINT_STATE_DTYPE))


def scene_step_errors(so, sg, co, cg, dt):
    """Per-step comparison of one scene without asserting: (integers identical,
    pose error, velocity error x dt)."""
    ro, io = pair_table(so)
    rg, ig = pair_table(sg)
    same = ro.shape == rg.shape and np.array_equal(ro, rg) and np.array_equal(io, ig) and np.array_equal(co, cg)
    pe, ve = pose_errors(sg["bodies"], so["bodies"], dt)
    return bool(same), pe, ve
