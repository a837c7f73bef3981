"""Finite joint stiffness on the CPU oracle: the dual-number derivative with
respect to the stiffness and the initial velocity against f64 central
differences, on a swinging pendulum chain (no contacts: smooth)."""
import numpy as np
import pytest

from ornis_gb300 import abi

import adjoint_scenes as S
import oracle_api as O

STEPS = 30


def run(arr, joints, k, use_double, steps=STEPS, seeds=(), seed_k=None, tweak=None):
    w = O.OracleWorld(abi.default_params(), mode=O.COLOURED, use_double=use_double)
    a = arr.copy()
    if tweak:
        tweak(a)
    w.add_bodies(a)
    for j in joints:
        assert w.add_joint(j)[0] == 0
    w.set_joint_stiffness(k)
    for s in seeds:
        w.seed(*s)
    if seed_k is not None:
        w.seed_joint_stiffness(seed_k)
    for _ in range(steps):
        w.step_fixed(1)
    return w


@pytest.mark.parametrize("k", [300.0, 3000.0])
def test_stiffness_derivative_matches_central_differences(k):
    arr, joints = S.pendulum()
    rng = np.random.default_rng(1)
    wts = np.zeros((len(arr), 13))
    wts[1:, 0:3] = rng.normal(size=(len(arr) - 1, 3))
    wts[1:, 7:10] = 0.3 * rng.normal(size=(len(arr) - 1, 3))
    b = len(arr) - 1
    w = run(arr, joints, k, O.DUAL, seeds=[(b, O.F_VEL, 0, 0)], seed_k=1)
    tg = w.tangents()
    dual = np.array([np.sum(wts * tg[:, :, d]) for d in (0, 1)])

    def loss(kk, dv=0.0):
        def tw(a):
            a["velocity"][b][0] += dv
        return float(np.sum(wts * run(arr, joints, kk, True, tweak=tw).state13()))

    hk = 1e-3 * k
    fd_k = (loss(k + hk) - loss(k - hk)) / (2 * hk)
    fd_v = (loss(k, 1e-4) - loss(k, -1e-4)) / 2e-4
    np.testing.assert_allclose(dual, [fd_v, fd_k], rtol=2e-3, atol=1e-6 * max(abs(fd_v), abs(fd_k) * k))


def test_soft_joints_stretch_and_hard_joints_do_not():
    arr, joints = S.pendulum(offset=0.0)
    gap = {}
    for k in (0.0, 200.0):
        w = run(arr, joints, k, True, steps=40)
        st = w.state13()
        # anchor separation of the ball joint between links 1 and 2
        def rot(q, v):
            x, y, z, ww = q
            t = 2.0 * np.cross([x, y, z], v)
            return v + ww * t + np.cross([x, y, z], t)
        pa = st[1, 0:3] + rot(st[1, 3:7], np.array([0, -0.25, 0]))
        pb = st[2, 0:3] + rot(st[2, 3:7], np.array([0, 0.25, 0]))
        gap[k] = float(np.linalg.norm(pa - pb))
    # the hard joint's residual is the solver's (about 6 mm on this swing);
    # a 200 N/m joint holding a 1 kg link stretches by centimetres
    assert gap[200.0] > 3.0 * gap[0.0] and gap[200.0] > 0.02
