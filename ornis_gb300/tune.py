"""Autotuner of the primal launch.

Candidates: one thread per body built for 4, 6 or 8 resident blocks per SM
(128, 80 or 64 registers) with the bodies of a colour in handle order or
ordered by work, 4 / 8 lanes per body, the split primal (one thread per
(pair, side) for the rows, then one per body for the sums and the solve),
or the per-scene solve (one block of 128, 256 or 512 threads takes a scene
through every iteration of the substep).  Every candidate is timed (CUDA
events, graph replay) from the same saved solver state, which is restored
afterwards, so tuning leaves the simulation where it found it.
"""
from . import abi

# (lanes, block, min blocks per SM, order colour lists by work)
CANDIDATES = [(1, 128, 4, 0), (1, 128, 4, 1), (1, 128, 6, 1), (4, 128, 4, 1), (8, 128, 4, 1), (0, 128, 4, 0),
              (0, 128, 4, 1), (abi.PRIMAL_SCENES, 128, 4, 0), (abi.PRIMAL_SCENES, 256, 4, 0),
              (abi.PRIMAL_SCENES, 512, 4, 0)]


def apply(world, cand):
    lanes, block, minb, by_work = cand
    world.set_tuning(lanes, block)
    world.set_occupancy(minb)
    world.set_work_order(by_work)


def autotune(world, substeps_per_trial=2, candidates=CANDIDATES):
    state = world.export_state()
    results = []
    for cand in candidates:
        world.import_state(state)
        apply(world, cand)
        world.step_graph(substeps_per_trial)  # capture and warm the graphs
        world.import_state(state)
        ms = world.step_timed(substeps_per_trial, use_graph=True)
        results.append((cand, ms))
    best = min(results, key=lambda r: r[1])[0]
    world.import_state(state)
    apply(world, best)
    return best, results
