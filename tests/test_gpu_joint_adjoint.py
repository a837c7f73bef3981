"""Finite joint stiffness and the adjoint through joint rows: the device
forward against the oracle per step, and the device gradient (initial state
and stiffness) against the f64 dual-number oracle and central differences."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdWorld, Rollout

import adjoint_scenes as S
import oracle_api as O
import parity as P

pytestmark = pytest.mark.gpu

STEPS = 30
FIELD = {0: (O.F_POS, 0), 1: (O.F_POS, 1), 2: (O.F_POS, 2), 7: (O.F_VEL, 0), 8: (O.F_VEL, 1), 9: (O.F_VEL, 2),
         10: (O.F_ANGVEL, 0), 11: (O.F_ANGVEL, 1), 12: (O.F_ANGVEL, 2)}


def weights(n, seed=0):
    rng = np.random.default_rng(seed)
    wts = np.zeros((n, 13))
    wts[1:, 0:3] = rng.normal(size=(n - 1, 3))
    wts[1:, 7:10] = 0.3 * rng.normal(size=(n - 1, 3))
    return wts


def device(arr, joints, k, wts, steps=STEPS, offsets=None, every=10):
    w = AvbdWorld(abi.default_params(), bodies=arr, scene_offsets=offsets)
    for j in joints:
        w.add_joint(j)
    w.set_joint_stiffness(k)
    r = Rollout(w, steps, 1, every)
    r.forward()
    g0, gmu = r.backward(wts.astype(np.float32))
    return g0, gmu, w.adjoint_grad_joint_stiffness()


def dual(arr, joints, k, wts, dirs, steps=STEPS, freeze=7, values=O.DUAL_F32):
    """Dual-number oracle; by default with the device rollout's f32 values
    (split-primal sums), so that both take the same branches."""
    o = O.OracleWorld(abi.default_params(), mode=O.COLOURED, use_double=values)
    o.split_sums(True)
    o.add_bodies(arr)
    for j in joints:
        assert o.add_joint(j)[0] == 0
    o.set_joint_stiffness(k)
    for d, (b, c) in enumerate(dirs):
        f, comp = FIELD[c]
        o.seed(b, f, comp, d)
    o.seed_joint_stiffness(len(dirs))
    o.freeze_frames(freeze)
    for _ in range(steps):
        o.step_fixed(1)
    tg = o.tangents()
    return np.array([np.sum(wts * tg[:, :, d]) for d in range(len(dirs) + 1)])


def test_soft_joint_forward_parity():
    arr, joints = S.pendulum()
    params = abi.default_params()
    o, g = P.make_pair(arr, params, joints)
    o.set_joint_stiffness(2000.0)
    g.set_joint_stiffness(2000.0)
    for _ in range(30):
        so, sg = P.step_from_oracle_state(o, g)
        P.compare_states(so, sg, params.step_dt, o, g)


@pytest.mark.parametrize("k", [300.0, 0.0])
def test_joint_adjoint_matches_dual_oracle(k):
    arr, joints = S.pendulum()
    wts = weights(len(arr))
    b = len(arr) - 1
    dirs = [(b, 7), (2, 1), (3, 12), (1, 9)]
    g0, _, gk = device(arr, joints, k, wts)
    got = np.array([g0[bb, c] for bb, c in dirs] + [gk[0]], dtype=np.float64)
    want = dual(arr, joints, k, wts, dirs)
    scale = np.max(np.abs(want))
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-3 * scale)


def test_joint_adjoint_matches_central_differences():
    """No contacts: the adjoint is the derivative of the step; f64 central
    differences of the oracle in the stiffness and a velocity agree with it."""
    arr, joints = S.pendulum()
    k = 400.0
    wts = weights(len(arr), seed=3)
    b = len(arr) - 1
    g0, _, gk = device(arr, joints, k, wts)

    def loss(kk, v=None):
        o = O.OracleWorld(abi.default_params(), mode=O.COLOURED, use_double=True)
        a = arr.copy()
        if v is not None:
            a["velocity"][b][0] = v
        o.add_bodies(a)
        for j in joints:
            o.add_joint(j)
        o.set_joint_stiffness(kk)
        for _ in range(STEPS):
            o.step_fixed(1)
        return float(np.sum(wts * o.state13()))

    # the stiffness is passed as an f32: the step is that of the rounded values
    khi, klo = np.float32(k * 1.0001), np.float32(k * 0.9999)
    fd_k = (loss(float(khi)) - loss(float(klo))) / (float(khi) - float(klo))
    # the velocity is an f32 record: likewise
    v0 = arr["velocity"][b][0]
    vhi, vlo = np.float32(v0 + np.float32(1e-5)), np.float32(v0 - np.float32(1e-5))
    fd_v = (loss(k, vhi) - loss(k, vlo)) / (float(vhi) - float(vlo))
    np.testing.assert_allclose([g0[b, 7], gk[0]], [fd_v, fd_k], rtol=1e-3)


def test_ragdoll_adjoint_matches_dual_oracle():
    """One ragdoll with soft joints dropped just above the ground: joint rows
    and contacts (self-contacts included) together.  Its derivatives move by
    about 1% under 1e-6 changes of the initial state (limits and grip flags
    switch), hence the tolerance."""
    bodies, offs, joints = scenes.ragdolls(counts=(1,), seed=4)
    dyn = bodies["inv_mass"] > 0
    low = bodies["position"][dyn, 1].min() - bodies["shape_params"][dyn, 0].max() - 0.25
    bodies["position"][dyn, 1] -= low
    wts = weights(len(bodies), seed=2)
    dirs = [(3, 7), (8, 1), (12, 8), (15, 12)]
    g0, _, gk = device(bodies, joints, 2000.0, wts, steps=20, offsets=offs)
    got = np.array([g0[bb, c] for bb, c in dirs], dtype=np.float64)
    want = dual(bodies, joints, 2000.0, wts, dirs, steps=20)
    scale = np.max(np.abs(want[:-1]))
    np.testing.assert_allclose(got, want[:-1], rtol=3e-2, atol=3e-2 * scale)
    np.testing.assert_allclose(gk[0], want[-1], rtol=3e-2, atol=1e-3 * scale)
