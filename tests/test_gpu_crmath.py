"""The correctly rounded sin / cos / asin / atan2 on the GPU
(tests/crmath/device_sweep.cu, built here for sm_103a): every device result
equals the same function built for the host and the long-double reference
rounded to float, over a sweep of ~100k arguments (every 65537th float bit
pattern, dense ranges near the physics' arguments, special values).  Built
with contracted multiply-adds on: the functions round every double
operation explicitly, so the build flags cannot change a result."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_device_functions_match_host_and_reference(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "device_sweep")
    r = subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=true",
                        "-Xcompiler", "-ffp-contract=off", os.path.join(HERE, "crmath", "device_sweep.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = re.findall(r"^(\w+) (\d+) (\d+) (\d+)$", out.stdout, re.M)
    assert {r[0] for r in rows} == {"sin", "cos", "sincos", "asin", "atan2"}, out.stdout
    for name, n, bad_host, bad_ref in rows:
        assert int(n) > 50000
        assert int(bad_host) == 0 and int(bad_ref) == 0, out.stdout
