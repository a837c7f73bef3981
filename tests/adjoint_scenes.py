"""Small scenes for the gradient checks of the differentiable rollout.

Contact-stable scenes are ones whose contacts keep their normal and their
body-fixed anchors for the whole horizon (a box sliding on the ground plane,
a ball rolling on it): there the frozen-frame adjoint is the exact derivative
of the step and central differences must agree with it."""
import numpy as np

from ornis_gb300 import abi

import oracle_api as O


def _finish(bodies, mu):
    for b in bodies:
        b.friction = mu
        b.friction_transverse = mu
    return O.bodies_to_array(bodies)


def slide(mu=0.6, v=2.0):
    g = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    b = O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0.5, 0], 1.0)
    b.velocity[0] = v
    b.velocity[2] = 0.3
    return _finish([g, b], mu)


def roll(mu=0.6, v=2.0):
    g = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    b = O.body_new(abi.SHAPE_SPHERE, [0.5], [0, 0.5, 0], 1.0)
    b.velocity[0] = v
    b.velocity[2] = -0.5
    return _finish([g, b], mu)


def stack(mu=0.6, n=3, v=1.0):
    """A box stack sheared at its base.  The boxes start 1 mm into their
    supports, offset 5 cm and turned 0.02 rad per level, so that no contact
    sits on a selection threshold (touching at exactly zero gap, or a corner
    at the edge of the manifold patch): there the f32 and f64 rollouts would
    pick different contact points and differentiate different functions."""
    bs = [O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)]
    for i in range(n):
        b = O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0.05 * i, 0.499 + 0.999 * i, -0.03 * i], 1.0)
        yaw = 0.02 * (i + 1)
        b.orientation[:] = [0.0, np.sin(yaw / 2), 0.0, np.cos(yaw / 2)]
        bs.append(b)
    bs[1].velocity[0] = v
    return _finish(bs, mu)


def tower(mu=0.6, n=4, speed=6.0, seed=0):
    """A short box tower hit by a heavy ball (the differentiable-batch
    workload's scene, smaller)."""
    rng = np.random.default_rng(seed)
    bs = [O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)]
    for i in range(n):
        bs.append(O.body_new(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 0.5 + i, 0], 1.0))
    ball = O.body_new(abi.SHAPE_SPHERE, [0.5], [-1.6, 1.0 + 0.2 * rng.random(), 0], 5.0)
    ball.velocity[0] = speed
    bs.append(ball)
    return _finish(bs, mu)


def pile(n=12, seed=1, mu=0.5):
    """Boxes and spheres dropped into a bin (ground plane + four walls)."""
    from ornis_gb300 import scenes
    rng = np.random.default_rng(seed)
    arr = scenes.bin_scene(rng, n)
    arr["friction"] = mu
    arr["friction_transverse"] = mu
    return arr


def capsule_rest(mu=0.5, tilt=0.05, v=0.4):
    """A capsule lying on the ground plane, tilted slightly about its
    horizontal axis so one end cap touches first, sliding and turning: its
    one witness point moves over the rounded caps (rolling anchors)."""
    g = O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)
    c = O.body_new(abi.SHAPE_CAPSULE, [0.1, 0.2, 0.0], [0, 0.1 + 0.2 * np.sin(tilt) - 0.002, 0], 13.0)
    # capsule axis (local y) turned to lie along x, then tilted by `tilt` about z
    ang = np.pi / 2 - tilt
    c.orientation[:] = [0.0, 0.0, np.sin(ang / 2), np.cos(ang / 2)]
    c.velocity[0] = v
    c.velocity[2] = 0.1
    c.angular_velocity[1] = 0.5
    return _finish([g, c], mu)


def carpet(n=36, r=0.2, spacing=0.5, seed=2, mu=0.5):
    """n x n spheres resting 1 mm into one ground plane with small random
    velocities: the plane's pair segment holds n^2 slots (over 1024 for the
    default, i.e. several chunks of the long-segment sort)."""
    rng = np.random.default_rng(seed)
    bs = [O.body_new(abi.SHAPE_HALFSPACE, [0, 1, 0], [0, 0, 0], 0.0)]
    for i in range(n):
        for k in range(n):
            b = O.body_new(abi.SHAPE_SPHERE, [r], [spacing * i, r - 0.001, spacing * k], 1.0)
            b.velocity[0], b.velocity[2] = 0.4 * rng.standard_normal(2)
            bs.append(b)
    return _finish(bs, mu)


def dynamic_mask(arr):
    return arr["inv_mass"] > 0


def pendulum(links=4, kind_hinge=(2,), limit=(-0.6, 0.6), v=1.5, mu=0.5, offset=0.05):
    """A chain of capsules hanging from a static anchor, swinging without
    contacts: ball joints, with the links in kind_hinge joined by a limited
    hinge.  Returns (bodies, joint descriptors)."""
    anchor = O.body_new(abi.SHAPE_SPHERE, [0.1], [0, 5, 0], 0.0)
    bs = [anchor]
    for i in range(links):
        b = O.body_new(abi.SHAPE_CAPSULE, [0.08, 0.2], [offset * i, 5 - 0.5 * (i + 1), 0.4 * offset * i], 1.0)
        bs.append(b)
    bs[-1].velocity[0] = v
    bs[-1].velocity[2] = 0.4
    arr = _finish(bs, mu)
    joints = []
    for i in range(links):
        a, b = i, i + 1
        la = [0, -0.1, 0] if i == 0 else [0, -0.25, 0]
        lb = [0, 0.25, 0]
        if i in kind_hinge:
            joints.append(abi.joint_desc(abi.JOINT_REVOLUTE, a, b, la, lb, (0, 0, 1), (0, 0, 1), limit=limit))
        else:
            joints.append(abi.joint_desc(abi.JOINT_BALL, a, b, la, lb))
    return arr, joints
