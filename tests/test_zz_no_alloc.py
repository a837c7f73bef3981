"""The allocation-free entry point (avbd_scene_step_static) against a world
and against the CPU oracle.

Callers that cannot allocate device memory (an engine that hands out device
memory only from its own pools, a process whose device memory is capped or
already reserved) step a small scene through one fixed device array; the
results must match an AvbdWorld stepped from the same bodies and the oracle
(Coloured order, the order the device sweeps in).  Two calls in a row: the
second, on a different and smaller scene, also shows that nothing left in the
shared array by the first leaks into it, and that it allocates no device
memory (the device's free memory is the same before and after it).  This
file is collected last, so it runs both alone and after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld, lib, scene_step_static

import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu

SUBSTEPS = 24


def world_result(params, bodies, substeps):
    w = AvbdWorld(params, bodies=bodies)
    w.step_fixed(substeps)
    out = w.bodies()
    w.close()
    return out


def oracle_result(params, bodies, substeps):
    o = O.OracleWorld(params, mode=O.COLOURED)
    o.add_bodies(bodies)
    o.step_fixed(substeps)
    return o.bodies()


def device_free_bytes():
    """cudaMemGetInfo's free bytes, from the CUDA runtime the library uses."""
    lib()  # the library (and with it libcudart) is loaded
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def assert_close(got, ref, dt):
    pe, ve = P.pose_errors(got, ref, dt)
    assert pe <= P.POSE_RTOL, f"pose error {pe:.3e} > {P.POSE_RTOL}"
    assert ve <= P.POSE_RTOL, f"velocity error (x dt) {ve:.3e} > {P.POSE_RTOL}"


def test_static_step_matches_world_on_two_calls():
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    first = scenes.bin_scene(np.random.default_rng([7, 1]), 120)    # 125 bodies: 5 walls + 120 shapes
    second = scenes.bin_scene(np.random.default_rng([7, 2]), 40)    # 45 bodies
    assert len(first) <= abi.STATIC_MAX_BODIES

    got1 = scene_step_static(params, first, SUBSTEPS)
    free_before = device_free_bytes()
    got2 = scene_step_static(params, second, SUBSTEPS)
    free_after = device_free_bytes()
    assert free_after == free_before, f"the second call changed free device memory by {free_before - free_after} B"
    ref1 = world_result(params, first, SUBSTEPS)
    ref2 = world_result(params, second, SUBSTEPS)

    assert_close(got1, ref1, params.step_dt)
    assert_close(got2, ref2, params.step_dt)
    assert_close(got1, oracle_result(params, first, SUBSTEPS), params.step_dt)
    assert_close(got2, oracle_result(params, second, SUBSTEPS), params.step_dt)
    # the scenes moved (a no-op would not be a test)
    assert np.abs(got1["position"] - first["position"]).max() > 1e-3
    # records other than the state pass through unchanged
    for f in ("shape", "shape_params", "mass", "friction", "collision_mask", "body_type"):
        assert np.array_equal(got2[f], second[f]), f


def test_static_step_rejects_too_many_bodies():
    params = abi.default_params()
    big = scenes.bin_scene(np.random.default_rng([7, 3]), abi.STATIC_MAX_BODIES)  # + 5 walls
    with pytest.raises(AvbdError) as e:
        scene_step_static(params, big, 1)
    assert e.value.code == abi.AVBD_ERR_CAPACITY
