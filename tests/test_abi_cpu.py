"""Host-only checks of the C ABI (no GPU needed): the library loads, every
function include/ornis_avbd.h declares is exported, record layouts match,
and the host-side constructors agree with the oracle's restatement of the
reference constructors."""
import ctypes as C
import os
import re

import numpy as np

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import LIB_PATH, bodies_array, body, lib

import oracle_api as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*int\s+(avbd_\w+)\s*\(", txt, flags=re.M)
    return names


def test_library_exports_every_declared_symbol():
    lib()
    L = C.CDLL(LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version_and_defaults():
    assert lib().avbd_abi_version() == 4
    p = abi.AvbdParams()
    assert lib().avbd_default_params(C.byref(p)) == 0
    assert abs(p.step_dt - 1 / 60) < 1e-9 and p.iterations == 10 and p.max_substeps == 4
    assert tuple(p.gravity) == (0.0, np.float32(-9.81), 0.0)


def test_record_sizes():
    assert C.sizeof(abi.AvbdBody) == 136
    assert C.sizeof(abi.AvbdPointState) == 68
    assert abi.BODY_DTYPE.itemsize == 136
    assert C.sizeof(abi.AvbdJointDesc) == 272
    assert C.sizeof(abi.AvbdJointState) == 100


def test_body_init_matches_oracle_constructors():
    cases = [
        (abi.SHAPE_BOX, [0.5, 0.25, 0.75], [1, 2, 3], 2.5),
        (abi.SHAPE_SPHERE, [0.3], [0, 1, 0], 1.7),
        (abi.SHAPE_CAPSULE, [0.3, 0.6], [0, 2, 0], 3.1),
        (abi.SHAPE_BOX, [10, 1, 10], [0, -1, 0], 0.0),
        (abi.SHAPE_HALFSPACE, [0, 2, 0], [0, 0, 0], 0.0),
        (abi.SHAPE_CYLINDER, [0.4, 0.7], [1, 1, 1], 2.0),
        (abi.SHAPE_CONE, [0.5, 0.3], [2, 1, 0], 1.3),
    ]
    for shape, params, pos, mass in cases:
        a = bodies_array([body(shape, params, pos, mass)])
        b = O.bodies_to_array([O.body_new(shape, params, pos, mass)])
        assert a.tobytes() == b.tobytes(), shape
        p3 = list(params) + [0.0] * (3 - len(params))
        if shape == abi.SHAPE_HALFSPACE:
            m = scenes.halfspace(pos, params)
        else:
            m = scenes.make_bodies([shape], [p3], [pos], [mass])
        assert m.tobytes() == a.tobytes(), shape


def test_body_init_rejects_dynamic_halfspace():
    b = abi.AvbdBody()
    p = np.array([0, 1, 0], np.float32)
    pos = np.zeros(3, np.float32)
    assert lib().avbd_body_init(C.byref(b), abi.SHAPE_HALFSPACE, abi.ptr(p), abi.ptr(pos), 1.0) == \
        abi.AVBD_ERR_INVALID_ARG


def test_world_create_rejects_bad_params():
    p = abi.default_params()
    p.step_dt = 0.0
    h = C.c_void_p()
    assert lib().avbd_world_create(C.byref(p), 0, C.byref(h)) == abi.AVBD_ERR_INVALID_ARG


def test_batched_scene_layout():
    bodies, offs, counts = scenes.batched(64)
    assert offs[0] == 0 and offs[-1] == len(bodies)
    assert np.all(np.diff(offs) == counts + 5)
    assert counts.min() >= 8 and counts.max() <= 1024
    # every scene starts with its five static half-spaces
    for s in range(64):
        sc = bodies[offs[s]:offs[s + 1]]
        assert np.all(sc["shape"][:5] == abi.SHAPE_HALFSPACE)
        assert np.all(sc["body_type"][5:] == abi.BODY_DYNAMIC)


# Launch-shape, profiling and timing hooks of the bench: not part of the seam
# the Rust crate binds.
BENCH_HOOKS = {"avbd_adjoint_timing", "avbd_adjoint_trace", "avbd_profiler", "avbd_set_broadphase",
               "avbd_set_occupancy", "avbd_set_sweep", "avbd_set_work_order", "avbd_world_flush_cache",
               "avbd_world_graph_nodes", "avbd_world_graph_nodes_emit", "avbd_world_profile_substep",
               "avbd_world_step_timed"}


def test_rust_crate_binds_the_header():
    """The Rust crate cannot be built in this image: its FFI module is checked
    against the header as text — every entry point but the bench hooks is
    declared, and every constant it repeats has the header's value."""
    ffi = open(os.path.join(ROOT, "rust", "ornis-avbd-gb300", "src", "ffi.rs")).read()
    declared = set(re.findall(r"pub fn (avbd_\w+)\s*\(", ffi))
    assert set(declared_functions()) - BENCH_HOOKS <= declared
    assert declared <= set(declared_functions())
    hdr = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "ornis_avbd.h")).read(), flags=re.S)
    defines = {k: int(v) for k, v in re.findall(r"#define\s+(AVBD_\w+)\s+\(?(-?\d+)u?\)?", hdr)}
    consts = {k: int(v) for k, v in re.findall(r"pub const (AVBD_\w+): \w+ = (-?\d+);", ffi)}
    assert consts, "no constants found"
    for k, v in consts.items():
        assert defines.get(k) == v, k
    assert set(defines) <= set(consts)


def _c_struct_fields(hdr, name):
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), hdr, flags=re.S)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "type a, b[3], c" -> a, b, c
        parts = decl.split(",")
        names.append(re.findall(r"(\w+)\s*(?:\[[^\]]*\])?$", parts[0].strip())[0])
        names += [re.match(r"\s*(\w+)", q).group(1) for q in parts[1:]]
    return names


def _rust_struct_fields(ffi, name):
    m = re.search(r"pub struct %s \{(.*?)\n\}" % name, ffi, flags=re.S)
    assert m, name
    return re.findall(r"pub (\w+):", m.group(1))


def test_rust_records_follow_the_header():
    """Every record the Rust crate mirrors has the header's fields in the
    header's order (the #[repr(C)] layout then follows)."""
    hdr = open(os.path.join(ROOT, "include", "ornis_avbd.h")).read()
    ffi = open(os.path.join(ROOT, "rust", "ornis-avbd-gb300", "src", "ffi.rs")).read()
    names = [n for n in re.findall(r"pub struct (Avbd\w+) \{", ffi) if _rust_struct_fields(ffi, n)]  # not opaque
    assert len(names) >= 10
    for name in names:
        assert _rust_struct_fields(ffi, name) == _c_struct_fields(hdr, name), name
