"""GB300-native AVBD rigid-body step (the AVBD path of Ornis's physics crate).

The product is libornis_avbd.so (C ABI in include/ornis_avbd.h), built from
ornis_gb300/csrc by ornis_gb300/build.py.  This package is its Python host
binding: `AvbdWorld` mirrors the reference's AvbdEngine API, `scenes` builds
the seeded workloads.
"""
from . import abi  # noqa: F401
from .avbd import AvbdError, AvbdWorld, bodies_array, body, lib  # noqa: F401
