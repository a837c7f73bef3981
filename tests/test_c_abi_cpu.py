"""A C program (tests/c_abi/seam.c) built against include/ornis_avbd.h and
linked to libornis_avbd.so: the ABI has a non-Python caller.  On the host
(no GPU): the ABI version, the default parameters (the reference's
constants) and avbd_body_init's records equal what the Python binding
reads through the same library."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from ornis_gb300 import abi
from ornis_gb300.avbd import body, lib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(ROOT, "ornis_gb300", "_lib")


def build_seam(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib()  # the library is built
    exe = str(tmp_path / "seam")
    r = subprocess.run([cc, "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "c_abi", "seam.c"), "-L", LIBDIR, "-lornis_avbd",
                        f"-Wl,-rpath,{LIBDIR}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def parse_bodies(text):
    out = []
    for line in text.splitlines():
        if line.startswith("body "):
            f = line.split()[1:]
            out.append((int(f[0]), int(f[1]), [float.fromhex(x) for x in f[2:]]))
    return out


def test_c_caller_on_the_host(tmp_path):
    exe = build_seam(tmp_path)
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == f"abi {lib().avbd_abi_version()}"
    p = abi.default_params()
    f = lines[1].split()[1:]
    assert [float.fromhex(x) for x in f[:4]] == [p.gravity[0], p.gravity[1], p.gravity[2], np.float32(p.step_dt)]
    assert [int(x) for x in f[4:]] == [p.iterations, p.max_substeps, p.enable_sleep, p.enable_ccd]
    got = parse_bodies(r.stdout)
    want = [body(abi.SHAPE_SPHERE, [0.4, 0, 0], [1, 2, 3], 2.0), body(abi.SHAPE_BOX, [0.5, 0.25, 1.0], [1, 2, 3], 3.0),
            body(abi.SHAPE_CAPSULE, [0.3, 0.6, 0], [1, 2, 3], 1.5), body(abi.SHAPE_HALFSPACE, [0, 1, 0], [1, 2, 3], 0.0)]
    assert len(got) == 4
    for (shape, btype, vals), w in zip(got, want):
        assert shape == w.shape and btype == w.body_type
        ref = list(w.position) + list(w.orientation) + [w.mass, w.inv_mass] + list(w.inertia) + [w.friction,
                                                                                                    w.restitution]
        assert np.array_equal(np.float32(vals), np.float32(ref))
