"""The world snapshot's format on the CPU (no GPU): a snapshot written here
from the documented layout is accepted, and every kind of damage — magic,
format version, endianness, record sizes, length, checksum, and contents
whose indices would leave their arrays — is refused with AVBD_ERR_FORMAT
before any device work."""
import ctypes as C
import struct

import pytest

from ornis_gb300 import abi
from ornis_gb300.avbd import AvbdError, AvbdWorld, body, snapshot_info


def fnv1a64(data):
    h = 14695981039346656037
    for x in data:
        h = ((h ^ x) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def records():
    return [C.sizeof(abi.AvbdParams), abi.SNAPSHOT_SETTINGS_BYTES, C.sizeof(abi.AvbdBody),
            C.sizeof(abi.AvbdBodyAux), C.sizeof(abi.AvbdPairState), C.sizeof(abi.AvbdPointState),
            abi.SNAPSHOT_JOINT_RECORD_BYTES, C.sizeof(abi.AvbdContactEvent), C.sizeof(abi.AvbdTriggerEvent),
            abi.MAX_POINTS]


def snapshot(scene_offsets=(0, 0), bodies=b"", nbodies=0, tof=None, substeps=7, fmt=abi.SNAPSHOT_FORMAT,
             endian=0x01020304, magic=abi.SNAPSHOT_MAGIC, rec=None, trailing=b"", shapes=b"\0" * 12):
    """A snapshot of a world without pairs, joints, hulls or events, laid out
    section by section: params, settings, scene offsets, bodies, aux, (pairs,
    points, joints, hulls: none), event words, touch CSR, (touch keys,
    trigger keys, queued events: none)."""
    payload = bytes(abi.default_params())
    payload += struct.pack("<9i2fI", 1, 128, 4, 2048, 1, 0, 0, 0, 0, 0.0, 0.0, 0)
    payload += struct.pack(f"<{len(scene_offsets)}I", *scene_offsets)
    payload += bodies
    payload += bytes(C.sizeof(abi.AvbdBodyAux) * nbodies)
    payload += shapes  # rounded and compound shapes, heightfields, meshes (shape_sections)
    payload += bytes(4 * abi.SNAPSHOT_EVENT_WORDS)
    tof = [0] * (nbodies + 1) if tof is None else tof
    payload += struct.pack(f"<{len(tof)}I", *tof)
    payload += trailing
    cnt = [nbodies, len(scene_offsets) - 1, 0, 0, 0, 0, 0, 0, 0, abi.SNAPSHOT_EVENT_WORDS]
    head = (magic + struct.pack("<4I", fmt, 4, abi.SNAPSHOT_HEADER_BYTES, endian) +
            struct.pack("<10I", *(rec or records())) + struct.pack("<10I", *cnt) +
            struct.pack("<3Q", abi.SNAPSHOT_HEADER_BYTES + len(payload), fnv1a64(payload), substeps))
    assert len(head) == abi.SNAPSHOT_HEADER_BYTES
    return head + payload


def refused(data):
    with pytest.raises(AvbdError) as e:
        snapshot_info(data)
    assert e.value.code == abi.AVBD_ERR_FORMAT
    with pytest.raises(AvbdError) as e:
        AvbdWorld.from_snapshot(data)
    assert e.value.code == abi.AVBD_ERR_FORMAT


def test_documented_layout_is_accepted():
    data = snapshot()
    info = snapshot_info(data)
    assert (info.format, info.abi, info.nbodies, info.nscenes, info.substeps, info.bytes) == \
        (abi.SNAPSHOT_FORMAT, 4, 0, 1, 7, len(data))
    assert (info.npairs, info.njoints, info.nhulls, info.ntouch, info.ntrigger) == (0, 0, 0, 0, 0)


def test_header_damage_is_refused():
    refused(snapshot(magic=b"ORNAVBX\0"))
    refused(snapshot(fmt=abi.SNAPSHOT_FORMAT + 1))
    refused(snapshot(endian=0x04030201))
    rec = records()
    rec[6] += 4  # another joint record layout
    refused(snapshot(rec=rec))
    good = snapshot()
    refused(good[:-1])
    refused(good + b"\0")
    refused(good[:100])
    bad = bytearray(good)
    bad[abi.SNAPSHOT_HEADER_BYTES + 3] ^= 0x10  # checksum no longer matches
    refused(bytes(bad))


def test_contents_are_checked_on_the_host():
    box = bytes(body(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 1, 0], 1.0))
    # scene offsets that do not end at the body count
    refused(snapshot(scene_offsets=(0, 2), bodies=box, nbodies=1))
    # a touch set whose CSR does not end at its key count
    refused(snapshot(scene_offsets=(0, 1), bodies=box, nbodies=1, tof=[0, 1]))
    # a hull body without hulls
    hull = bytearray(box)
    struct.pack_into("<I", hull, abi.AvbdBody.shape.offset, abi.SHAPE_HULL)
    refused(snapshot(scene_offsets=(0, 1), bodies=bytes(hull), nbodies=1))
    # a non-finite pose
    nan = bytearray(box)
    struct.pack_into("<f", nan, abi.AvbdBody.position.offset, float("nan"))
    refused(snapshot(scene_offsets=(0, 1), bodies=bytes(nan), nbodies=1))
    # bytes after the last section
    refused(snapshot(trailing=b"\0\0\0\0"))
    # the same world without the damage is well formed
    assert snapshot_info(snapshot(scene_offsets=(0, 1), bodies=box, nbodies=1)).nbodies == 1


def shape_sections(exts=(), hfs=(), meshes=()):
    """The three table sections: each a count, then per rounded or compound
    shape (flag, part count, unit inertia, parts), per heightfield (rows,
    cols, cell, heights row by row), per mesh (vertex floats, triangle
    indices, the floats, the indices)."""
    out = struct.pack("<I", len(exts))
    for flag, parts, ui in exts:
        out += struct.pack("<2I3f", flag, len(parts), *ui) + b"".join(bytes(q) for q in parts)
    out += struct.pack("<I", len(hfs))
    for rows, cols, cell, h in hfs:
        out += struct.pack(f"<2If{len(h)}f", rows, cols, cell, *h)
    out += struct.pack("<I", len(meshes))
    for v, t in meshes:
        out += struct.pack(f"<2I{len(v)}f{len(t)}I", len(v), len(t), *v, *t)
    return out


def retyped(shape, index, mass):
    """A body record of a table-backed shape: its kind and table index
    patched into a box's record."""
    b = bytearray(bytes(body(abi.SHAPE_BOX, [0.5, 0.5, 0.5], [0, 1, 0], mass)))
    struct.pack_into("<I", b, abi.AvbdBody.shape.offset, shape)
    struct.pack_into("<f", b, abi.AvbdBody.shape_params.offset, float(index))
    return bytes(b)


def test_table_shapes_are_checked_on_the_host():
    rounded = (0, [abi.shape_part(abi.SHAPE_SPHERE, [0.3], 0.1)], (0.1, 0.1, 0.1))
    dumbbell = (1, [abi.shape_part(abi.SHAPE_SPHERE, [0.2], position=(-0.5, 0, 0)),
                    abi.shape_part(abi.SHAPE_SPHERE, [0.2], position=(0.5, 0, 0))], (0.1, 0.1, 0.1))
    terrain = (2, 3, 1.0, [0.0, 0.1, 0.0, 0.2, 0.0, 0.1])
    tri = ([0, 0, 0, 1, 0, 0, 0, 0, 1], [0, 1, 2])
    world = [retyped(abi.SHAPE_ROUND, 0, 1.0), retyped(abi.SHAPE_COMPOUND, 1, 1.0),
             retyped(abi.SHAPE_HEIGHTFIELD, 0, 0.0), retyped(abi.SHAPE_TRIMESH, 0, 0.0)]

    def snap(bodies=world, exts=(rounded, dumbbell), hfs=(terrain,), meshes=(tri,)):
        return snapshot(scene_offsets=(0, len(bodies)), bodies=b"".join(bodies), nbodies=len(bodies),
                        shapes=shape_sections(exts, hfs, meshes))

    assert snapshot_info(snap()).nbodies == 4
    # a body naming a table entry that is not there, or one of the other kind
    refused(snap(bodies=world[:2] + [retyped(abi.SHAPE_HEIGHTFIELD, 1, 0.0)] + world[3:]))
    refused(snap(bodies=world[:3] + [retyped(abi.SHAPE_TRIMESH, 1, 0.0)]))
    refused(snap(bodies=[retyped(abi.SHAPE_ROUND, 1, 1.0)] + world[1:]))
    refused(snap(bodies=[world[0], retyped(abi.SHAPE_COMPOUND, 0, 1.0)] + world[2:]))
    refused(snap(bodies=[retyped(abi.SHAPE_ROUND, -1, 1.0)] + world[1:]))
    # terrain and meshes are never dynamic
    refused(snap(bodies=world[:2] + [retyped(abi.SHAPE_HEIGHTFIELD, 0, 1.0)] + world[3:]))
    refused(snap(bodies=world[:3] + [retyped(abi.SHAPE_TRIMESH, 0, 1.0)]))
    # table entries the registration calls would refuse
    refused(snap(exts=((2,) + rounded[1:], dumbbell)))                         # unknown flag
    refused(snap(exts=((0, dumbbell[1], rounded[2]), dumbbell)))               # rounded with two parts
    refused(snap(exts=((0, [abi.shape_part(abi.SHAPE_SPHERE, [0.3])], rounded[2]), dumbbell)))  # no border
    refused(snap(exts=(rounded, (1, [abi.shape_part(abi.SHAPE_HALFSPACE, [0, 1, 0])], (0.1, 0.1, 0.1)))))
    refused(snap(exts=(rounded, (1, [abi.shape_part(abi.SHAPE_HULL, [0])], (0.1, 0.1, 0.1)))))  # no hulls
    refused(snap(exts=(rounded, (1, dumbbell[1], (0.1, float("nan"), 0.1)))))
    refused(snap(hfs=((2, 3, 0.0, terrain[3]),)))                              # no cell size
    refused(snap(hfs=((2, 3, 1.0, terrain[3][:5] + [float("inf")]),)))
    refused(snap(meshes=((tri[0], [0, 1, 3]),)))                               # a vertex that is not there
    refused(snap(meshes=((tri[0][:8], tri[1]),)))                              # not whole vertices
    refused(snap(meshes=((tri[0], [0, 1]),)))                                  # not whole triangles
    # a section shorter than its counts say: the rest of the payload is misread
    refused(snap(hfs=((2, 3, 1.0, terrain[3][:4]),)))
