"""physkit_gb300 — GB300-native (sm_103a) world step of the PhysKit rigid-body engine.

The step (broadphase, narrowphase, contact solver, integrator) runs as hand-written CUDA kernels in
libphyskit_gb300.so behind the C ABI of include/physkit_gb300.h; `World` is the Python mirror of the
reference's world API over that ABI. There is no CPU fallback.
"""
from .world import (BODY_DTYPE, World, lib, library_path, object_desc, world_desc)  # noqa: F401
from . import scenes  # noqa: F401

__all__ = ["World", "world_desc", "object_desc", "BODY_DTYPE", "lib", "library_path", "scenes"]
