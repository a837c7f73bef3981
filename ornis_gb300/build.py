"""Build the GB300 AVBD library (ornis_gb300/_lib/libornis_avbd.so) with nvcc.

One -gencode for sm_103a, translation units compiled in parallel, no cmake.
-fmad=false keeps every multiply and add separately rounded, so the pair
sets, contact IDs and colours the kernels decide match the reference's f32
arithmetic on identical input.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libornis_avbd.so")

# (source, object, extra flags).  The iteration kernels are built twice:
# exact (the default flags) and fast (contracted FMAs, approximate div/sqrt).
SOURCES = [
    ("avbd_util.cu", "avbd_util.o", []),
    ("avbd_phase_pre.cu", "avbd_phase_pre.o", []),
    ("avbd_phase_disc.cu", "avbd_phase_disc.o", []),
    ("avbd_phase_solve.cu", "avbd_phase_solve.o", []),
    ("avbd_phase_solve.cu", "avbd_phase_solve_fast.o",
     ["-DAVBD_SOLVE_FAST", "-fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
    ("avbd_events.cu", "avbd_events.o", []),
    ("avbd_world.cu", "avbd_world.o", []),
    ("avbd_static.cu", "avbd_static.o", []),
    # the reverse sweep: contracted FMAs, approximate div/sqrt (its gradients
    # are checked to 5e-3; it repeats bit for bit run to run on one build)
    ("avbd_adjoint.cu", "avbd_adjoint.o", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--extended-lambda", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "ornis_avbd.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src, obj, extra in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        objs.append(o)
        if not force and _newer(o, [s] + headers):
            continue
        flags = [f for f in FLAGS if not (extra and f == "-fmad=false")]
        jobs.append([cc] + ARCH + flags + extra + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = False
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                failed = True
    if failed:
        raise RuntimeError("nvcc failed")
    if force or jobs or not os.path.exists(LIB):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
