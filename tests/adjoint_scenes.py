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


def dynamic_mask(arr):
    return arr["inv_mass"] > 0
