"""The C caller (tests/c_abi/seam.c) on the GPU: the dispatch's call
sequence — records written back, the accumulator step, records read back,
events drained each step; remove_joint and wake_body midway — through the
C ABI from C, against the same sequence through the Python binding: the
final bodies and the event count are identical bit for bit."""
import subprocess

import numpy as np
import pytest

from ornis_gb300 import abi
from ornis_gb300.avbd import AvbdWorld, body, bodies_array

from test_c_abi_cpu import build_seam, parse_bodies

pytestmark = pytest.mark.gpu


def python_sequence():
    recs = [body(abi.SHAPE_BOX, [10, 1, 10], [0, -1, 0], 0.0)]
    for i in range(4):
        recs.append(body(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, np.float32(0.5) + np.float32(1.02) * np.float32(i), 0], 1.0))
    recs += [body(abi.SHAPE_SPHERE, [0.5, 0, 0], [2.5, 3, 0], 1.0), body(abi.SHAPE_BOX, [0.3, 0.3, 0.3], [-3, 4, 0], 0.0),
             body(abi.SHAPE_BOX, [0.3, 0.3, 0.3], [-2, 4, 0], 1.0)]
    host = bodies_array(recs)
    w = AvbdWorld(abi.default_params())
    w.add_bodies(host)
    jh = w.add_joint(abi.joint_desc(abi.JOINT_BALL, 6, 7, [0.5, 0, 0], [-0.5, 0, 0]))
    nev = 0
    for s in range(90):
        w.set_bodies(host)
        w.step(1.0 / 60.0)
        host = w.bodies()
        nev += len(w.contact_events())
        if s == 45:
            w.remove_joint(jh)
            w.wake_body(2)
            host = w.bodies()
    return host, nev, w.counters().steps


def test_c_caller_on_the_gpu_matches_the_binding(tmp_path):
    exe = build_seam(tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    head = r.stdout.splitlines()[0].split()
    got = parse_bodies(r.stdout)
    host, nev, steps = python_sequence()
    assert int(head[1]) == nev and int(head[3]) == steps
    assert len(got) == len(host)
    for (shape, btype, vals), b in zip(got, host):
        ref = list(b["position"]) + list(b["orientation"]) + [b["mass"], b["inv_mass"]] + list(b["inertia"]) + \
            [b["friction"], b["restitution"]]
        assert np.array_equal(np.float32(vals), np.float32(ref))
