"""The device's correctly rounded sin / cos / asin / atan2
(ornis_gb300/csrc/avbd_crmath.cuh, built with nvcc as host code) against
long-double references rounded once to float, on the host (no GPU).

Three builds: the normal one (the float stage for small arguments, the
double evaluation, double-double only when Ziv's rounding test fails), one
without the float stage (the double evaluation checked over the whole
sweep), and one that takes the double-double path for every argument, so
that the rarely taken path is checked over the same sweep.  The sweep: every
40961st bit pattern of all 2^32 floats (signs, subnormals, huge arguments,
NaN, infinities), every 7th float in [2^-14, 4), every 3rd float in [1/2, 1]
for asin, random pairs plus special values for atan2, and a million atan2
arguments of the float stage (x near 1, |y| up to x/16).  Every result must be bit-identical to the
reference (NaN to NaN)."""
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


def _sweep(tmp_path, extra, args):
    exe = str(tmp_path / "sweep")
    src = os.path.join(HERE, "crmath", "sweep.cu")
    r = subprocess.run([_nvcc(), "-std=c++17", "-O2", "-x", "cu", "-Xcompiler", "-ffp-contract=off"] + extra +
                       [src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    res = {m.group(1): (int(m.group(2)), int(m.group(3)))
           for m in re.finditer(r"^(\w+) (\d+) (\d+)$", out.stdout, re.M)}
    assert set(res) == {"sin", "cos", "sincos", "asin", "atan2"}, out.stdout
    return res, out.stdout


BUILDS = {"float": [], "double": ["-DAVBD_CRMATH_TEST_DOUBLE"],
          "double-double": ["-DAVBD_CRMATH_TEST_DOUBLE", "-DAVBD_CRMATH_TEST_SLOW"]}


@pytest.mark.parametrize("build", list(BUILDS))
def test_correctly_rounded_against_long_double(tmp_path, build):
    res, log = _sweep(tmp_path, BUILDS[build], [40961, 100000])
    for name, (n, bad) in res.items():
        assert n > 100000, (name, n)
        assert bad == 0, log
