"""The on-disk world snapshot (avbd_world_snapshot / avbd_world_from_snapshot /
avbd_world_save / avbd_world_load): a world made from a snapshot continues
bit for bit as the saved world does — bodies, solver state, joints and the
events it reports, queued ones included — and a snapshot of the loaded world
is the same bytes."""
import numpy as np
import pytest

from ornis_gb300 import abi, scenes
from ornis_gb300.avbd import AvbdError, AvbdWorld

from test_gpu_convex import convex_scene, hulls

pytestmark = pytest.mark.gpu


def state_bytes(w):
    st = w.export_state()
    return b"".join(st[k].tobytes() for k in ("bodies", "aux", "pairs", "points", "joints"))


def mixed_world(params):
    """Hulls, cylinders, cones, boxes and spheres on a floor, a trigger
    sphere they fall through, a jointed chain (ball, revolute with a limit
    and a motor, wheel with a sprung suspension) and a driven slider geared
    to the chain's hinge."""
    bodies = convex_scene(n=30, seed=5)
    sensor = scenes.make_bodies([abi.SHAPE_SPHERE], [[1.2, 0, 0]], [[0.0, 3.0, 0.0]], [0.0])
    sensor["flags"] = abi.FLAG_TRIGGER
    chain = scenes.make_bodies([abi.SHAPE_BOX] * 6, [[0.2, 0.2, 0.2]] * 6,
                               [[5.0, 4.0, 0.0], [5.6, 4.0, 0.0], [6.2, 4.0, 0.0], [6.8, 4.0, 0.0],
                                [-5.0, 4.0, 0.0], [-4.0, 4.0, 0.0]],
                               [0.0, 1.0, 1.0, 1.0, 0.0, 1.0])
    w = AvbdWorld(params)
    for verts, faces in hulls():
        w.add_hull(verts, faces, (0.1, 0.1, 0.1))
    w.add_bodies(np.concatenate([bodies, sensor, chain]))
    c = len(bodies) + 1
    w.add_joint(abi.joint_desc(abi.JOINT_BALL, c, c + 1, [0.3, 0, 0], [-0.3, 0, 0]))
    w.add_joint(abi.joint_desc(abi.JOINT_REVOLUTE, c + 1, c + 2, [0.3, 0, 0], [-0.3, 0, 0], (0, 0, 1), (0, 0, 1),
                               limit=(-0.6, 0.6), motor=(1.5, 20.0)))
    w.add_joint(abi.joint_desc(abi.JOINT_WHEEL, c + 2, c + 3, [0.3, 0, 0], [-0.3, 0, 0], (0, 1, 0), (0, 1, 0),
                               wheel=((0, 0, 1), (0, 0, 1), 4.0, 0.7)))
    w.add_joint(abi.joint_desc(abi.JOINT_PRISMATIC, c + 4, c + 5, [1, 0, 0], [0, 0, 0], (1, 0, 0), (1, 0, 0),
                               motor=(1.0, 30.0)))
    w.add_joint(abi.joint_desc(abi.JOINT_GEAR, c + 1, c + 5, [0, 0, 0], [0, 0, 0], gear=(1, 3, 0.5)))
    w.set_events(0)
    return w


def run(w, steps, dt, log):
    for _ in range(steps):
        w.step(dt)
        log.append((w.contact_events().tobytes(), w.trigger_events().tobytes()))


@pytest.mark.parametrize("kind", ["bytes", "file"])
def test_snapshot_continues_bit_for_bit(kind, tmp_path):
    params = abi.default_params()
    dt = 0.021  # one or two substeps per call: the accumulator keeps a remainder
    a = mixed_world(params)
    before = []
    run(a, 45, dt, before)
    a.step(dt)  # its events stay queued across the snapshot
    if kind == "bytes":
        snap = a.snapshot()
        b = AvbdWorld.from_snapshot(snap)
    else:
        path = tmp_path / "world.avbd"
        a.save(path)
        b = AvbdWorld.load(path)
        snap = path.read_bytes()
    assert b.snapshot() == snap
    la, lb = [], []
    for w, log in ((a, la), (b, lb)):
        log.append((w.contact_events().tobytes(), w.trigger_events().tobytes()))
        run(w, 60, dt, log)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    assert state_bytes(a) == state_bytes(b)
    assert la == lb
    assert a.event_counts() == b.event_counts()
    assert sum(len(c) + len(t) for c, t in la) > 0
    assert any(len(t) for _, t in before + la), "the trigger saw no body"


def test_snapshot_of_batch_with_launch_settings():
    """A batch with the fast build, the split primal, events every second
    substep and graph replay: the settings travel with the world."""
    bodies, offs, _ = scenes.batched(nscenes=12, seed=7, lo=8, hi=160)
    params = abi.default_params(step_dt=1.0 / 120.0, iterations=8)
    a = AvbdWorld(params, bodies=bodies, scene_offsets=offs)
    a.set_precision(1)
    a.set_tuning(0, 128)
    a.set_events(2)
    for _ in range(30):
        a.step_graph(2)
    snap = a.snapshot()
    b = AvbdWorld.from_snapshot(snap)
    assert b.snapshot() == snap
    for _ in range(25):
        a.step_graph(2)
        b.step_graph(2)
        assert a.contact_events().tobytes() == b.contact_events().tobytes()
    assert a.bodies().tobytes() == b.bodies().tobytes()
    assert state_bytes(a) == state_bytes(b)


def test_snapshot_of_unstepped_and_edited_worlds():
    params = abi.default_params()
    bodies = convex_scene(n=12, seed=9)
    # never stepped: no device state yet
    a = AvbdWorld(params)
    for verts, faces in hulls():
        a.add_hull(verts, faces, (0.1, 0.1, 0.1))
    a.add_bodies(bodies)
    b = AvbdWorld.from_snapshot(a.snapshot())
    for _ in range(20):
        a.step(params.step_dt)
        b.step(params.step_dt)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    # stepped, then edited on the host (a body added): the touch set is kept
    extra = scenes.make_bodies([abi.SHAPE_SPHERE], [[0.3, 0, 0]], [[0.0, 6.0, 0.0]], [1.0])
    a.add_bodies(extra)
    b.add_bodies(extra)
    c = AvbdWorld.from_snapshot(a.snapshot())
    for _ in range(30):
        for w in (a, b, c):
            w.step(params.step_dt)
        ea = a.contact_events().tobytes()
        assert ea == b.contact_events().tobytes() == c.contact_events().tobytes()
    assert a.bodies().tobytes() == b.bodies().tobytes() == c.bodies().tobytes()


def test_damaged_snapshot_is_refused_before_any_device_work():
    a = AvbdWorld(abi.default_params(), bodies=np.concatenate([
        scenes.halfspace([0, 0, 0], [0, 1, 0]),
        scenes.make_bodies([abi.SHAPE_BOX] * 2, [[0.5, 0.5, 0.5]] * 2, [[0, 0.6, 0], [0, 1.8, 0]], [1.0, 1.0])]))
    a.step(1.0 / 60.0)
    snap = bytearray(a.snapshot())
    snap[200] ^= 1
    with pytest.raises(AvbdError) as e:
        AvbdWorld.from_snapshot(bytes(snap))
    assert e.value.code == abi.AVBD_ERR_FORMAT
