"""The benchmarked configuration at the state it is timed in.

The batched workload (4096 scenes, dt 1/120, 2 substeps, 8 iterations) run
as the benchmark runs it — exact build, launch shape picked by the autotuner
at step 150, CUDA-graph replay, events every step — to step 200, where the
piles have formed (millions of contact pairs, several colours).  From there,
for 10 steps (20 substeps, the reference's step_inner each), sampled scenes
of the batch are exported from the device before every substep and stepped
by the oracle (Coloured order; rows summed per pair when the split or
per-scene launch runs, as they sum them) while the device steps the whole
batch.  Per substep: pair sets, points per pair, contact IDs and colours
identical; poses within 1e-5 relative (scale max(1, |x|)), velocities the
same times dt.

The exact build computes the oracle's arithmetic (sin / asin correctly
rounded on both sides), so the poses are expected to be identical, and the
test asserts that too.  The comparison restarts from the device's state
every substep so that a failure names the substep where it starts.  (The
fast build is not held to this: at these piles its contracted multiply-adds
move poses by up to 4e-5 within a substep, because the stiff contact rows
amplify last-bit differences, and a pose 1 ulp away can move a box corner
across the manifold's slop in the next discovery.)
"""
import numpy as np
import pytest

from ornis_gb300 import scenes
from ornis_gb300.avbd import AvbdWorld
from ornis_gb300.tune import autotune

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu


def test_batched_piles_bench_configuration_per_step():
    bodies, offs, _ = scenes.batched(4096)
    params, nsub = scenes.params_for("batched_4096")
    w = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    w.set_precision(False)
    w.set_events(nsub)
    w.step_graph(nsub * 150)
    (lanes, _, _, _), _ = autotune(w, substeps_per_trial=2 * nsub)
    w.step_graph(nsub * 50)
    sizes = np.diff(offs)
    rng = np.random.default_rng(97531)
    big = [int(x) for x in np.argsort(-sizes, kind="stable")[:4]]
    chosen = big + [int(x) for x in rng.permutation(len(sizes)) if int(x) not in big][:4]
    st = w.export_state()
    assert len(st["pairs"]) > 1_000_000  # the piles the benchmark times
    worst = 0.0
    for _ in range(10 * nsub):
        ors = []
        for sc in chosen:
            sub = P.scene_state(st, offs, sc)
            o = O.OracleWorld(params, mode=O.COLOURED)
            o.split_sums(lanes <= 0)
            o.add_bodies(sub["bodies"])
            o.import_state(sub)
            o.step_fixed(1)
            ors.append(o)
        w.step_graph(1)
        st = w.export_state()
        cols = w.colours()
        for sc, o in zip(chosen, ors):
            a0, a1 = int(offs[sc]), int(offs[sc + 1])
            so, sg = o.export_state(), P.scene_state(st, offs, sc)
            ro, io = P.pair_table(so)
            rg, ig = P.pair_table(sg)
            assert np.array_equal(ro, rg), f"scene {sc}: pair set / point counts differ"
            assert np.array_equal(io, ig), f"scene {sc}: contact IDs differ"
            assert np.array_equal(o.colours(), cols[a0:a1]), f"scene {sc}: colours differ"
            pe, ve = P.pose_errors(sg["bodies"], so["bodies"], params.step_dt)
            assert pe <= P.POSE_RTOL and ve <= P.POSE_RTOL, f"scene {sc}: pose {pe:.2e}, velocity {ve:.2e}"
            worst = max(worst, pe)
    print(f"bench configuration (lanes {lanes}) at the piles: worst per-step pose error {worst:.2e}")
    assert worst == 0.0
