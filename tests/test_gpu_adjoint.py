"""The device adjoint of the AVBD rollout against the f64 dual-number
oracle with the same frozen contact frames, and against central
differences on contact-stable scenes.  The loss is a random linear form of
the final positions and velocities; directions are the last body's
velocity, a position, an angular velocity and the scene friction."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld, Rollout

import adjoint_scenes as S
import oracle_api as O
from test_oracle_adjoint import CONTACT_STABLE, _tower32, central, loss_weights, tower32_central

pytestmark = pytest.mark.gpu

STEPS = 40


def device_grad(arr, wts, steps=STEPS, every=10, offsets=None):
    w = AvbdWorld(abi.default_params(), bodies=arr, scene_offsets=offsets)
    r = Rollout(w, steps, 1, every)
    r.forward()
    return r.backward(wts.astype(np.float32))


def oracle_dirs(arr, wts, steps=STEPS, values=O.DUAL_F32):
    """Directional derivatives from the dual-number oracle (frozen frames).
    By default its values are the f32 step's in the device's split-primal
    summation order, i.e. the device rollout bit for bit, so both sides take
    every branch alike; values=O.DUAL differentiates the f64 step."""
    b = len(arr) - 1
    seeds = [(b, O.F_VEL, 0, 0), (b, O.F_VEL, 2, 1), (1, O.F_POS, 0, 3), (b, O.F_ANGVEL, 1, 4)]
    seeds += [(i, O.F_FRICTION, 0, 2) for i in range(len(arr))]
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED, use_double=values)
    w.split_sums(True)
    w.add_bodies(arr)
    for s in seeds:
        w.seed(*s)
    w.freeze_frames(7)
    for _ in range(steps):
        w.step_fixed(1)
    tg = w.tangents()
    return np.array([np.sum(wts * tg[:, :, d]) for d in range(5)])


def device_dirs(arr, g0, gmu):
    b = len(arr) - 1
    return np.array([g0[b, 7], g0[b, 9], gmu[0], g0[1, 0], g0[b, 11]], dtype=np.float64)


@pytest.mark.parametrize("name,steps", [("slide", 40), ("roll", 40), ("pile", 60), ("stack", 40), ("tower", 40),
                                        ("capsule_rest", 120)])
def test_adjoint_matches_dual_oracle(name, steps):
    arr = getattr(S, name)()
    wts = loss_weights(arr, seed=5)
    g0, gmu = device_grad(arr, wts, steps=steps)
    got = device_dirs(arr, g0, gmu)
    want = oracle_dirs(arr, wts, steps=steps)
    scale = np.max(np.abs(want))
    assert np.all(np.isfinite(got)) and scale > 0
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-3 * scale)


@pytest.mark.parametrize("name,steps", CONTACT_STABLE)
def test_adjoint_matches_central_differences(name, steps):
    """Contact-stable scenes: the frozen-frame adjoint is the derivative of
    the step, so f64 central differences of the oracle agree with it to
    1e-3."""
    arr = getattr(S, name)()
    wts = loss_weights(arr)
    g0, gmu = device_grad(arr, wts, steps=steps)
    b = len(arr) - 1
    got = np.array([g0[b, 7], g0[b, 9], gmu[0]], dtype=np.float64)
    fd = central(arr, wts, steps=steps)
    scale = np.max(np.abs(fd))
    np.testing.assert_allclose(got, fd, rtol=1e-3, atol=1e-3 * scale)


def _tower32_device(H, wts=None):
    """The differentiable workload's scene (one 32-box tower and its ball):
    device gradients along the ball's velocity and the friction after H
    steps, for a linear loss (wts) or the workload's own loss (the sum of
    squared final tower-body positions)."""
    bodies, offs, ball, tower = scenes.diff_towers(nscenes=1)
    params, nsub = scenes.params_for("diff_1024")
    w = AvbdWorld(params, bodies=bodies)
    r = Rollout(w, H, nsub, 10)
    r.forward()
    end = w.bodies()
    if wts is None:
        g = np.zeros((len(bodies), 13), dtype=np.float32)
        g[tower, 0:3] = 2.0 * end["position"][tower]
    else:
        g = wts.astype(np.float32)
    g0, gmu = r.backward(g)
    b = int(ball[0])
    return np.array([g0[b, 7], g0[b, 8], g0[b, 9], gmu[0]], dtype=np.float64), end


def test_tower32_before_impact_matches_central_differences():
    """The 32-box tower of the differentiable workload, 6 steps (the ball
    reaches the tower at step 8): device gradients within 1e-3 of f64
    central differences."""
    _, _, _, _, wts = _tower32()
    got, _ = _tower32_device(6, wts)
    fd = tower32_central(6)
    np.testing.assert_allclose(got, fd, rtol=1e-3, atol=1e-3 * np.max(np.abs(fd)))


def test_tower32_rollout_matches_dual_oracle():
    """The whole 120-step rollout of the differentiable workload's scene with
    its own loss: the device adjoint against the dual-number oracle that
    follows the same f32 trajectory with the same frozen frames, within
    1e-3."""
    got, end = _tower32_device(120)
    bodies, offs, ball, tower = scenes.diff_towers(nscenes=1)
    params, nsub = scenes.params_for("diff_1024")
    o = O.OracleWorld(params, mode=O.COLOURED, use_double=O.DUAL_F32)
    o.split_sums(True)
    o.add_bodies(bodies)
    b = int(ball[0])
    for c in range(3):
        o.seed(b, O.F_VEL, c, c)
    for i in range(len(bodies)):
        o.seed(i, O.F_FRICTION, 0, 3)
    o.freeze_frames(7)
    for _ in range(120):
        o.step_fixed(nsub)
    st = o.state13()
    np.testing.assert_array_equal(st[:, 0:3].astype(np.float32), end["position"])
    wts = np.zeros((len(bodies), 13))
    wts[tower, 0:3] = 2.0 * st[tower, 0:3]
    tg = o.tangents()
    want = np.array([np.sum(wts * tg[:, :, d]) for d in range(4)])
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-3 * np.max(np.abs(want)))


def test_checkpoint_spacing_does_not_change_gradients():
    arr = S.tower()
    wts = loss_weights(arr, seed=7)
    a = device_grad(arr, wts, steps=30, every=1)
    b = device_grad(arr, wts, steps=30, every=7)
    c = device_grad(arr, wts, steps=30, every=100)
    for x, y in ((a, b), (a, c)):
        np.testing.assert_array_equal(x[0], y[0])
        np.testing.assert_array_equal(x[1], y[1])


def test_long_floor_segment_keeps_one_order():
    """1296 spheres on one floor: the floor's pair segment is longer than a
    thread sorts and goes through the chunk sort.  Gradients are the same bit
    for bit for any checkpoint spacing, and the recorded forward ends where
    the plain forward (segment left as placed) ends."""
    arr = S.carpet()
    wts = loss_weights(arr, seed=5)
    a = device_grad(arr, wts, steps=12, every=1)
    b = device_grad(arr, wts, steps=12, every=5)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert np.all(np.isfinite(a[0]))
    w = AvbdWorld(abi.default_params(), bodies=arr)
    r = Rollout(w, 12, 1, 5)
    r.forward()
    rec = w.bodies()["position"]
    p = AvbdWorld(abi.default_params(), bodies=arr)
    p.step_fixed(12)
    np.testing.assert_allclose(rec, p.bodies()["position"], atol=1e-5)


def test_adjoint_trace_covers_every_substep():
    """The adjoint-magnitude trace has one entry per substep of the rollout,
    finite on a bounded scene, the bodies named being in range."""
    arr = S.tower()
    wts = loss_weights(arr, seed=3)
    w = AvbdWorld(abi.default_params(), bodies=arr)
    r = Rollout(w, 20, 1, 7)
    r.forward()
    r.backward(wts.astype(np.float32))
    mx, body = w.adjoint_trace()
    assert len(mx) == 20 and len(body) == 20
    assert np.all(np.isfinite(mx)) and np.all(mx > 0)
    assert np.all(body < len(arr))


def test_tower_batch_gradients_are_reproducible():
    """Colliding towers (the differentiable workload, 16 scenes): repeated
    backward passes and any checkpoint spacing give the same gradients bit
    for bit (point state crosses checkpoints by pair index, so the pair order
    must not depend on the run)."""
    bodies, offs, ball, tower = scenes.diff_towers(nscenes=16)
    params, nsub = scenes.params_for("diff_1024")
    res = []
    for every in (1, 9, 40):
        w = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
        w.set_precision(True)
        w.adjoint_forward(40, nsub, every)
        end = w.bodies()
        g = np.zeros((len(bodies), 13), dtype=np.float32)
        g[tower, 0:3] = 2.0 * end["position"][tower]
        a, b = w.adjoint_backward(g), w.adjoint_backward(g)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        res.append(a)
    for r in res[1:]:
        np.testing.assert_array_equal(res[0][0], r[0])
        np.testing.assert_array_equal(res[0][1], r[1])


def test_batch_gradients_equal_scenes_alone():
    parts = [S.tower(seed=1), S.slide(), S.pile(n=10, seed=3), S.roll()]
    arr = np.concatenate(parts)
    offs = np.cumsum([0] + [len(p) for p in parts])
    wts = np.concatenate([loss_weights(p, seed=i) for i, p in enumerate(parts)])
    g0, gmu = device_grad(arr, wts, steps=25, every=5, offsets=offs)
    for i, p in enumerate(parts):
        h0, hmu = device_grad(p, loss_weights(p, seed=i), steps=25, every=5)
        np.testing.assert_array_equal(g0[offs[i]:offs[i + 1]], h0)
        assert gmu[i] == hmu[0]


def test_world_left_at_the_end_of_the_rollout():
    arr = S.pile(n=10, seed=2)
    w = AvbdWorld(abi.default_params(), bodies=arr)
    w.adjoint_forward(20, 1, 6)
    end = w.bodies()
    w.adjoint_backward(np.ones((len(arr), 13), dtype=np.float32))
    np.testing.assert_array_equal(w.bodies(), end)
    ref = AvbdWorld(abi.default_params(), bodies=arr)
    for _ in range(20):
        ref.step_graph(1)
    np.testing.assert_array_equal(ref.bodies(), end)


def test_adjoint_rejects_rolling_friction():
    arr = S.roll()
    arr["rolling_friction"] = 0.1
    w = AvbdWorld(abi.default_params(), bodies=arr)
    with pytest.raises(AvbdError):
        w.adjoint_forward(2, 1, 1)
