"""tahoe_gb300: the Tahoe implicit hex8 solid path, GB300-native.

C ABI: include/tahoe_gb300.h (library built in-tree by tahoe_gb300/build.py).
Python layers: ``lib`` (ctypes binding), ``model`` (deck-level host driver),
``meshgen`` (seeded synthetic meshes), ``workloads`` (benchmark configs).
"""
from . import build, lib, meshgen, model  # noqa: F401

__all__ = ["build", "lib", "meshgen", "model"]
