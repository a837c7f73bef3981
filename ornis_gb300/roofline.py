"""Algorithmic byte model of the AVBD iterations (v1) and the primal roofline.

None of the AVBD kernels is a dense contraction, so the bound is HBM
bandwidth.  Algorithmic bytes are what the math must move at least once per
iteration, independent of how the kernels stage it:

  primal, per iteration
    swept body   128 B  (x,q 28 + x0,q0 28 + y,q~ 28 + inv_mass + inertia 16
                         read; x,q 28 written)
    contact point 48 B  (ra, rb, lambda, penalty read)
    pair header   32 B  (normal, gap, mu, a, b)
  dual, per iteration
    contact point 76 B  (48 B read + lambda, penalty, stuck 28 B written)
    body          56 B  per body referenced (x,q,x0,q0 of both sides, counted
                        once per swept body)
    pair header   32 B

A launch of the per-colour primal kernels covers one colour; their roofline
uses the sum over all colours of one iteration (the same ratio as per
launch).  The per-scene solve is one launch per substep covering every
iteration's primal and dual: its algorithmic bytes are iterations x (primal
+ dual bytes per iteration).  It keeps a scene's data on chip and in L2
across the iterations, so its DRAM traffic is below these bytes.
"""

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture)
# per algorithmic byte of the split primal (k_side_rows + k_side_solve, all
# launches of one step): 512 scenes of the batched workload at step 200,
# exact build, 96 non-empty colour launches of each kernel moved 4,836 MB
# against 764 MB of model bytes.  The bench scales it to its own launches by
# the model bytes (the same mix of bodies, points and pairs per byte).
SPLIT_TRAFFIC_PER_MODEL_BYTE = 6.33
TRAFFIC_SOURCE = ("ncu capture (512 scenes, step 200, exact build): 6.33 DRAM bytes per model byte, "
                  "scaled to this launch by its model bytes")

PRIMAL_BODY_B = 128
PRIMAL_POINT_B = 48
PAIR_HEADER_B = 32
DUAL_POINT_B = 76
DUAL_BODY_B = 56


def primal_bytes_per_iteration(swept, points, pairs):
    return PRIMAL_BODY_B * swept + PRIMAL_POINT_B * points + PAIR_HEADER_B * pairs


def dual_bytes_per_iteration(swept, points, pairs):
    return DUAL_POINT_B * points + DUAL_BODY_B * swept + PAIR_HEADER_B * pairs


KERNELS = {
    "thread": "k_primal_thread (one launch per colour)",
    "lanes": "k_primal_lanes (one launch per colour)",
    "split": "k_side_rows + k_side_solve (one pair of launches per colour)",
    "scene": "k_scene_solve (one launch per substep: every iteration's primal and dual, a block per scene)",
}


def primal_roofline(phases_ms, info, peak, kind="thread", iterations=1):
    """Roofline entry for the primal kernel from one profiled substep.

    kind: the launch that ran ("thread", "lanes", "split" — the pair of
    kernels per colour, its time is the pair's — or "scene", the per-scene
    solve, one launch covering every iteration's primal and dual).
    """
    peak_gbs, source = peak
    if kind == "scene":
        b = iterations * (primal_bytes_per_iteration(info["swept"], info["points"], info["pairs"]) +
                          dual_bytes_per_iteration(info["swept"], info["points"], info["pairs"]))
        ms = phases_ms["primal"]
        achieved = b / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        return {
            "bound": "hbm", "kernel": KERNELS[kind], "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
            "frac": achieved / peak_gbs,
            "peak_source": f"{source} (MEASURED_PEAKS.json hbm_gbs)" if source == "measured" else "fallback 6.8 TB/s",
            "traffic": None, "bytes_per_launch": b, "launch_ms": ms,
            "model": "v1: per iteration 128 B/swept body + 48 B/point + 32 B/pair (primal) + 56 B/swept body + "
                     "76 B/point + 32 B/pair (dual), times the iterations of the launch",
        }
    iters = max(1, info["primal_launches"] // max(1, info["colours"]))
    per_iter_ms = phases_ms["primal"] / iters
    per_launch_ms = phases_ms["primal"] / max(1, info["primal_launches"])
    b = primal_bytes_per_iteration(info["swept"], info["points"], info["pairs"])
    achieved = b / (per_iter_ms / 1e3) / 1e9 if per_iter_ms > 0 else 0.0
    dual_b = dual_bytes_per_iteration(info["swept"], info["points"], info["pairs"])
    dual_ms = phases_ms["dual"] / iters
    return {
        "bound": "hbm",
        "kernel": KERNELS[kind],
        "achieved": achieved,
        "peak": peak_gbs,
        "unit": "GB/s",
        "frac": achieved / peak_gbs,
        "peak_source": f"{source} (MEASURED_PEAKS.json hbm_gbs)" if source == "measured" else "fallback 6.8 TB/s",
        "traffic": SPLIT_TRAFFIC_PER_MODEL_BYTE * b / max(1, info["colours"]) if kind == "split" else None,
        "traffic_source": TRAFFIC_SOURCE if kind == "split" else None,
        "bytes_per_launch": b / max(1, info["colours"]),
        "launch_ms": per_launch_ms,
        "model": "v1: 128 B/swept body + 48 B/point + 32 B/pair per iteration",
        "dual": {"achieved": dual_b / (dual_ms / 1e3) / 1e9 if dual_ms > 0 else 0.0,
                 "frac": (dual_b / (dual_ms / 1e3) / 1e9) / peak_gbs if dual_ms > 0 else 0.0,
                 "launch_ms": dual_ms},
    }
