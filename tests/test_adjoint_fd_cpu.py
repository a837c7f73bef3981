"""The adjoint's hand-written vector-Jacobian products against central
differences, on the host (no GPU): the harnesses in tests/adjoint_fd/ include
ornis_gb300/csrc/avbd_adjoint.cuh, build with nvcc as host code and compare
every VJP with the difference quotient of the forward function it reverses.

Float differences carry noise, so a handful of the several thousand checks
may miss the 3% bar; the tests allow at most 0.5% of them (the counts seen
are 1 in 4560 and 6 in 7179)."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        pytest.skip("nvcc not found")
    return exe


def _run(name, tmp_path):
    exe = str(tmp_path / name)
    src = os.path.join(HERE, "adjoint_fd", name + ".cu")
    r = subprocess.run([_nvcc(), "-std=c++17", "-O2", "-x", "cu", src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    m = re.search(r"(\d+) checks, (\d+) failures", out.stdout)
    assert m, out.stdout
    return int(m.group(1)), int(m.group(2)), out.stdout


def test_rotation_contact_and_twist_vjps(tmp_path):
    checks, fails, log = _run("primitives", tmp_path)
    assert checks > 4000
    assert fails <= 0.005 * checks, log


def test_joint_row_vjps(tmp_path):
    checks, fails, log = _run("joints", tmp_path)
    assert checks > 5000
    assert fails <= 0.005 * checks, log
