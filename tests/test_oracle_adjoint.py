"""The f64 forward-mode (dual-number) oracle against central differences.

The dual-number world differentiates the CPU step exactly for the branch
pattern its values take; on contact-stable scenes (oracle scenes in
adjoint_scenes.py) it must agree with central differences of the f64 step,
with and without the contact frames frozen (the device adjoint's
convention).  These checks need no GPU."""
import numpy as np
import pytest

from ornis_gb300 import abi

import adjoint_scenes as S
import oracle_api as O

STEPS = 40


def run(arr, use_double, steps=STEPS, seeds=(), freeze=0, tweak=None):
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED, use_double=use_double)
    a = arr.copy()
    if tweak:
        tweak(a)
    w.add_bodies(a)
    for s in seeds:
        w.seed(*s)
    if freeze:
        w.freeze_frames(freeze)
    for _ in range(steps):
        w.step_fixed(1)
    return w


def loss_weights(arr, seed=0):
    """A random linear loss of the final positions and velocities."""
    rng = np.random.default_rng(seed)
    wts = np.zeros((len(arr), 13))
    dyn = S.dynamic_mask(arr)
    wts[dyn, 0:3] = rng.normal(size=(dyn.sum(), 3))
    wts[dyn, 7:10] = 0.3 * rng.normal(size=(dyn.sum(), 3))
    return wts


def directional(arr, wts, freeze, steps=STEPS):
    """dLoss along: velocity x / z of the last body, and the friction coefficient."""
    b = len(arr) - 1
    seeds = [(b, O.F_VEL, 0, 0), (b, O.F_VEL, 2, 1)] + [(i, O.F_FRICTION, 0, 2) for i in range(len(arr))]
    w = run(arr, O.DUAL, steps=steps, seeds=seeds, freeze=freeze)
    tg = w.tangents()
    return np.array([np.sum(wts * tg[:, :, d]) for d in range(3)])


def central(arr, wts, eps=1e-5, steps=STEPS):
    """f64 central differences of the loss along the last body's velocity x, z
    and the friction coefficient.  The inputs are f32 records, so the step
    is the difference of the two perturbed values as stored (x + eps and
    x - eps rounded to f32), not 2 eps: at eps = 1e-4 on a value near 2 the
    rounding alone would move the quotient by 0.2%."""
    b = len(arr) - 1
    f32 = np.float32

    def loss(fn):
        return float(np.sum(wts * run(arr, True, steps=steps, tweak=fn).state13()))

    def quotient(get, put):
        v = get(arr)
        hi, lo = f32(v + f32(eps)), f32(v - f32(eps))
        return (loss(lambda a: put(a, hi)) - loss(lambda a: put(a, lo))) / (float(hi) - float(lo))

    out = []
    for k in (0, 2):
        def put(a, x, k=k):
            a["velocity"][b][k] = x
        out.append(quotient(lambda a, k=k: a["velocity"][b][k], put))

    def put_mu(a, x):
        a["friction"][:] = x
        a["friction_transverse"][:] = x
    out.append(quotient(lambda a: a["friction"][0], put_mu))
    return np.array(out)


# contact-stable scenes and horizons: a box sliding the whole horizon, a ball
# rolling, a capsule resting on its cap with a rolling witness anchor
CONTACT_STABLE = [("slide", 20), ("roll", 40), ("capsule_rest", 120)]


@pytest.mark.parametrize("name,steps", CONTACT_STABLE)
def test_dual_matches_central_differences(name, steps):
    """The dual world differentiates the f64 step exactly (1e-6 of central
    differences), and on contact-stable scenes the frozen-frame convention
    of the device adjoint is that derivative too (1e-4)."""
    arr = getattr(S, name)()
    wts = loss_weights(arr)
    full = directional(arr, wts, freeze=0, steps=steps)
    frozen = directional(arr, wts, freeze=7, steps=steps)
    fd = central(arr, wts, steps=steps)
    scale = np.max(np.abs(fd))
    assert scale > 1e-2
    np.testing.assert_allclose(full, fd, rtol=1e-6, atol=1e-6 * scale)
    np.testing.assert_allclose(frozen, full, rtol=1e-4, atol=1e-4 * scale)


def _tower32():
    from ornis_gb300 import scenes
    bodies, _, ball, _ = scenes.diff_towers(nscenes=1)
    params, nsub = scenes.params_for("diff_1024")
    rng = np.random.default_rng(11)
    wts = np.zeros((len(bodies), 13))
    wts[1:, 0:3] = rng.normal(size=(len(bodies) - 1, 3))
    wts[1:, 7:10] = 0.3 * rng.normal(size=(len(bodies) - 1, 3))
    return bodies, int(ball[0]), params, nsub, wts


def tower32_dirs(H, freeze, values=O.DUAL):
    """dLoss/d(ball velocity x, y, z) and d/d(friction) on the differentiable
    workload's scene (a 32-box tower hit by the ball) after H steps."""
    bodies, b, params, nsub, wts = _tower32()
    w = O.OracleWorld(params, mode=O.COLOURED, use_double=values)
    w.add_bodies(bodies)
    for c in range(3):
        w.seed(b, O.F_VEL, c, c)
    for i in range(len(bodies)):
        w.seed(i, O.F_FRICTION, 0, 3)
    if freeze:
        w.freeze_frames(freeze)
    for _ in range(H):
        w.step_fixed(nsub)
    tg = w.tangents()
    return np.array([np.sum(wts * tg[:, :, d]) for d in range(4)])


def tower32_central(H, eps=1e-5):
    bodies, b, params, nsub, wts = _tower32()
    f32 = np.float32

    def loss(a):
        w = O.OracleWorld(params, mode=O.COLOURED, use_double=True)
        w.add_bodies(a)
        for _ in range(H):
            w.step_fixed(nsub)
        return float(np.sum(wts * w.state13()))

    out = []
    for c in range(4):
        v = bodies["velocity"][b][c] if c < 3 else bodies["friction"][0]
        hi, lo = f32(v + f32(eps)), f32(v - f32(eps))
        pair = []
        for x in (hi, lo):
            a = bodies.copy()
            if c < 3:
                a["velocity"][b][c] = x
            else:
                a["friction"][:] = x
                a["friction_transverse"][:] = x
            pair.append(loss(a))
        out.append((pair[0] - pair[1]) / (float(hi) - float(lo)))
    return np.array(out)


def test_tower32_dual_matches_central_differences():
    """The differentiable workload's scene: the f64 dual world is the exact
    derivative of the f64 step before and after the ball hits the tower
    (step 8 of the drop); the frozen-frame convention of the device adjoint
    is exact before the impact (6 steps) and not after it (the new contact's
    frame and the refreshed anchors of the tower's contacts depend on the
    ball's velocity; 8 steps)."""
    for H in (6, 10):
        fd = tower32_central(H)
        scale = np.max(np.abs(fd))
        np.testing.assert_allclose(tower32_dirs(H, freeze=0), fd, rtol=1e-5, atol=1e-5 * scale)
    fd6 = tower32_central(6)
    np.testing.assert_allclose(tower32_dirs(6, freeze=7), fd6, rtol=1e-6, atol=1e-6 * np.max(np.abs(fd6)))
    fd8 = tower32_central(8)
    assert np.max(np.abs(tower32_dirs(8, freeze=7) - fd8)) > 0.01 * np.max(np.abs(fd8))


def test_dual_values_equal_f64_run():
    """The dual world's values are the f64 world's, bit for bit."""
    arr = S.tower()
    a = run(arr, True, steps=20).state13()
    d = run(arr, O.DUAL, steps=20, seeds=[(1, O.F_POS, 0, 0)]).state13()
    np.testing.assert_array_equal(a, d)


def _world(arr, use_double, joints=(), k=0.0, seeds=(), freeze=0, params=None):
    w = O.OracleWorld(params or abi.default_params(), mode=O.COLOURED, use_double=use_double)
    w.add_bodies(arr)
    for j in joints:
        assert w.add_joint(j)[0] == 0
    w.set_joint_stiffness(k)
    for s in seeds:
        w.seed(*s)
    if freeze:
        w.freeze_frames(freeze)
    return w


def _swept_sphere():
    """A small fast sphere crossing a thin wall within one step: a swept
    impact (time of impact clamp and bounce) every time it reaches it."""
    g = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    wall = O.body_new(abi.SHAPE_BOX, [0.05, 1.0, 1.0], [2.0, 1.0, 0.0], 0.0)
    ball = O.body_new(abi.SHAPE_SPHERE, [0.05], [0.0, 0.5, 0.1], 1.0)
    ball.velocity[0] = 45.0
    ball.restitution = 0.5
    return S._finish([g, wall, ball], 0.4)


@pytest.mark.parametrize("case", ["capsule_rest", "ragdoll", "swept"])
def test_frozen_conventions_change_no_value(case):
    """The frozen-frame conventions of the dual world (rolling capsule
    anchors, the hinge twist held past a 120-degree swing, the swept
    impact's time of impact, normal and bounce) drop tangents only: its
    trajectory is the f64 world's bit for bit."""
    joints, k, steps = (), 0.0, 60
    if case == "capsule_rest":
        arr = S.capsule_rest()
    elif case == "ragdoll":
        from ornis_gb300 import scenes
        arr, _, joints = scenes.ragdolls(counts=(1,), seed=4)
        k, steps = 2e4, 90
    else:
        arr = _swept_sphere()
    b = len(arr) - 1
    seeds = [(b, O.F_VEL, 0, 0), (b, O.F_ANGVEL, 1, 1), (1, O.F_POS, 1, 2)]
    plain = _world(arr, True, joints, k)
    dual = _world(arr, O.DUAL, joints, k, seeds=seeds, freeze=7)
    for _ in range(steps):
        plain.step_fixed(1)
        dual.step_fixed(1)
    np.testing.assert_array_equal(plain.state13(), dual.state13())
    assert np.all(np.isfinite(dual.tangents()))
    if case == "swept":
        assert dual.counters().ccd_hits > 0
