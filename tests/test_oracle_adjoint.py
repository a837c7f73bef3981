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


def directional(arr, wts, freeze):
    """dLoss along: velocity x / z of the last body, and the friction coefficient."""
    b = len(arr) - 1
    seeds = [(b, O.F_VEL, 0, 0), (b, O.F_VEL, 2, 1)] + [(i, O.F_FRICTION, 0, 2) for i in range(len(arr))]
    w = run(arr, O.DUAL, seeds=seeds, freeze=freeze)
    tg = w.tangents()
    return np.array([np.sum(wts * tg[:, :, d]) for d in range(3)])


def central(arr, wts, eps=1e-4):
    b = len(arr) - 1

    def loss(fn):
        return float(np.sum(wts * run(arr, True, tweak=fn).state13()))

    out = []
    for k in (0, 2):
        def up(a, k=k):
            a["velocity"][b][k] += eps
        def dn(a, k=k):
            a["velocity"][b][k] -= eps
        out.append((loss(up) - loss(dn)) / (2 * eps))

    def mu_up(a):
        a["friction"] += eps
        a["friction_transverse"] += eps

    def mu_dn(a):
        a["friction"] -= eps
        a["friction_transverse"] -= eps
    out.append((loss(mu_up) - loss(mu_dn)) / (2 * eps))
    return np.array(out)


@pytest.mark.parametrize("name", ["slide", "roll"])
def test_dual_matches_central_differences(name):
    arr = getattr(S, name)()
    wts = loss_weights(arr)
    full = directional(arr, wts, freeze=0)
    frozen = directional(arr, wts, freeze=7)
    fd = central(arr, wts)
    scale = np.max(np.abs(fd))
    assert scale > 1e-2
    np.testing.assert_allclose(full, fd, rtol=2e-3, atol=2e-3 * scale)
    # contact-stable: the frozen-frame convention is the exact derivative
    np.testing.assert_allclose(frozen, full, rtol=1e-3, atol=1e-3 * scale)


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
