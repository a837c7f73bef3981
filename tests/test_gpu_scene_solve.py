"""The per-scene solve (one block takes a scene through every iteration of
a substep: all colours' primal and the dual in one launch) against the split
launches and the oracle.

It computes the split launches' arithmetic (rows summed per pair, then per
body the inertial block, the pairs in incidence order and the joints), so in
the exact build it must equal them bit for bit, through plain launches and
graph replay, for every block size, and equal the oracle (Coloured order,
per-pair row sums) bit for bit from identical state.  The fast build lets
the compiler contract multiply-adds where it likes, which can differ between
the two kernels, so there both are held to the parity bars instead.
"""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdWorld

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu

SCENES = abi.PRIMAL_SCENES


def run(bodies, offs, params, nsub, lanes, block, fast, graph, steps, joints=()):
    w = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    for j in joints:
        w.add_joint(j)
    w.set_tuning(lanes, block)
    w.set_precision(fast)
    for _ in range(steps):
        (w.step_graph if graph else w.step_fixed)(nsub)
    out = w.bodies()
    c = w.counters()
    w.close()
    return out, c


@pytest.mark.parametrize("block,fast,graph", [(128, 0, 0), (256, 0, 1), (512, 0, 1), (256, 0, 0)])
def test_scene_solve_equals_split_launches(block, fast, graph):
    # scenes up to 600 bodies: colours with more items than a block's round
    bodies, offs, _ = scenes.batched(12, seed=21, lo=8, hi=600)
    params, nsub = scenes.params_for("batched_4096")
    ref, cr = run(bodies, offs, params, nsub, 0, 128, fast, graph, 60)
    got, cg = run(bodies, offs, params, nsub, SCENES, block, fast, graph, 60)
    assert cr.pairs > 500 and cr.colours >= 3  # piles, several colours
    assert got.tobytes() == ref.tobytes()
    assert (cg.pairs, cg.points, cg.colours) == (cr.pairs, cr.points, cr.colours)


def test_scene_solve_with_joints_equals_split_launches():
    bodies, offs, joints = scenes.ragdolls((3, 5), seed=6)
    params, nsub = scenes.params_for("ragdoll_8192")
    ref, _ = run(bodies, offs, params, nsub, 0, 128, 0, 1, 50, joints)
    got, _ = run(bodies, offs, params, nsub, SCENES, 256, 0, 1, 50, joints)
    assert got.tobytes() == ref.tobytes()


def test_body_with_more_pairs_than_a_block_round():
    """A plank resting on 15 x 15 spheres has 226 pairs: more items than a
    128-thread block computes in one round, so its sum spans several rounds."""
    recs = [scenes.halfspace([0, 0, 0], [0, 1, 0])]
    g = (np.arange(15) - 7) * 0.42
    xs, zs = np.meshgrid(g, g)
    n = xs.size
    recs.append(scenes.make_bodies([abi.SHAPE_SPHERE] * n, [[0.2, 0, 0]] * n,
                                   np.stack([xs.ravel(), np.full(n, 0.2), zs.ravel()], 1), [0.1] * n))
    recs.append(scenes.make_bodies([abi.SHAPE_BOX], [[3.4, 0.1, 3.4]], [[0.0, 0.5, 0.0]], [20.0]))
    bodies = np.concatenate(recs)
    offs = np.array([0, len(bodies)], dtype=np.uint32)
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    ref, cr = run(bodies, offs, params, 2, 0, 128, 0, 0, 40)
    got, _ = run(bodies, offs, params, 2, SCENES, 128, 0, 0, 40)
    assert cr.pairs >= 2 * n
    assert got.tobytes() == ref.tobytes()


def test_scene_above_block_limit_falls_back_to_split_launches():
    rng = np.random.default_rng([5, 5])
    bodies = scenes.bin_scene(rng, 2100)  # 2105 bodies: above the per-block limit
    offs = np.array([0, len(bodies)], dtype=np.uint32)
    params, nsub = scenes.params_for("batched_4096")
    ref, _ = run(bodies, offs, params, nsub, 0, 128, 1, 1, 30)
    got, _ = run(bodies, offs, params, nsub, SCENES, 256, 1, 1, 30)
    assert got.tobytes() == ref.tobytes()


@pytest.mark.parametrize("fast", [0, 1])
def test_scene_solve_per_step_against_oracle(fast):
    rng = np.random.default_rng([2, 11])
    bodies = scenes.bin_scene(rng, 150)
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    o, g = P.make_pair(bodies, params)
    o.split_sums(True)
    g.set_tuning(SCENES, 256)
    g.set_precision(fast)
    worst = 0.0
    for _ in range(60):
        so, sg = P.step_from_oracle_state(o, g)
        worst = max(worst, P.compare_states(so, sg, params.step_dt, o, g)[0])
    print(f"per-scene solve, fast={fast}: worst per-step pose error {worst:.2e}")
    if not fast:
        assert worst == 0.0  # correctly rounded sin / asin on both sides: the same arithmetic
