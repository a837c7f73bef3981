"""Regenerate the golden fixtures under tests/golden/ from the reference tree.

Run in a container where the reference checkout is mounted (read-only):
    python tests/golden/make_golden.py /root/reference

avbd_snapshot.hex is the reference's own bit-exact determinism fixture
(crates/physics/tests/data/avbd_snapshot.hex, pinned by
avbd_snapshot_matches_canonical in crates/physics/tests/avbd_engine.rs:1632-1645):
9 bodies x 13 f32 (position, quaternion xyzw, velocity, angular velocity)
after 120 steps of 1/60 s.  It is data, copied byte for byte.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    src = os.path.join(ref_root, "crates", "physics", "tests", "data", "avbd_snapshot.hex")
    shutil.copyfile(src, os.path.join(HERE, "avbd_snapshot.hex"))
    print("copied", src)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
