"""The device's row stamp and 6x6 LDL^T on the reference's known-answer
systems (crates/physics/tests/gpu_batches.rs:781-856, :863-898), run on the
GPU (tests/device_kat/rows_kat.cu, built here with -fmad=false as the
library's exact build is):

* one row along +Y with lever +X, penalty 2, force 3: Hessian entries
  (1,1), (5,5), (5,1) equal 2, rhs entries 1 and 5 equal 3; the B side
  (sign -1) leaves the Hessian and flips the rhs;
* an SPD system solves to the dense solution, and bit for bit to the
  oracle's LDL^T; a zero system and one with a -1 pivot break down (the
  body would skip its update).
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from ornis_gb300 import abi

import oracle_api as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def tri(i, j):
    return i * (i + 1) // 2 + j


def test_stamp_and_ldl_known_answers_on_the_device(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "rows_kat")
    r = subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false",
                        "-Xcompiler", "-ffp-contract=off", os.path.join(HERE, "device_kat", "rows_kat.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = {m.group(1): m.group(2).split() for m in re.finditer(r"^(\w+) (.*)$", out.stdout, re.M)}
    # stamp
    exp_h = np.zeros(21, np.float32)
    for i, j in ((1, 1), (5, 5), (5, 1)):
        exp_h[tri(i, j)] = 2.0
    for side, sgn in ((0, 1.0), (1, -1.0)):
        v = np.array([float.fromhex(x) for x in rows[f"stamp{side}"]], np.float32)
        assert np.array_equal(v[:21], exp_h)
        assert np.array_equal(v[21:], sgn * np.array([0, 3, 0, 0, 0, 3], np.float32))
    # solve
    lhs = np.zeros((6, 6), np.float32)
    for i in range(6):
        for j in range(6):
            lhs[i, j] = 4.0 + i if i == j else np.float32(0.1) * np.float32((i + j) + 1.0)
    rhs = np.array([1, -2, 3, -4, 5, -6], np.float32)
    ok0 = int(rows["solve0"][0])
    x0 = np.array([float.fromhex(x) for x in rows["solve0"][1:]], np.float32)
    assert ok0 == 1
    assert np.allclose(x0, np.linalg.solve(lhs.astype(np.float64), rhs.astype(np.float64)), atol=1e-6)
    xo = np.zeros(6, np.float32)
    assert O.lib().oracle_solve_6x6(abi.ptr(np.ascontiguousarray(lhs)), abi.ptr(rhs), abi.ptr(xo)) == 1
    assert np.array_equal(x0, xo)  # the same LDL^T arithmetic
    assert int(rows["solve1"][0]) == 0 and int(rows["solve2"][0]) == 0
