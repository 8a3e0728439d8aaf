"""pk_collide_noalloc: the narrowphase batch without any device allocation.

Some callers cannot allocate device memory when they call in (a strict memory budget, or an
allocator that must not see per-call cudaMalloc/cudaFree). pk_collide_noalloc stages its descriptors
and results in a fixed array inside the library instead. This file is collected last so that a
run stopping at the first failure has already run every other test; it also passes on its own in a
fresh process.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _pairs():
    ka = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))
    cases = ka["gjk"] + ka["epa"] + ka["epa_positive"]
    return [(c["a"], c["b"]) for c in cases] + [(c["b"], c["a"]) for c in cases]


def _shape(world, spec, cache):
    import math

    def quat(rot):
        if rot is None:
            return [1.0, 0.0, 0.0, 0.0]
        h = 0.5 * rot[0]
        s = math.sin(h)
        return [math.cos(h), s * rot[1][0], s * rot[1][1], s * rot[1][2]]

    if spec[0] == "aabb":
        return (0, list(spec[1]) + list(spec[2]), -1)
    if spec[0] == "obb":
        return (1, list(spec[1]) + quat(spec[2]) + list(spec[3]), -1)
    ms = tuple(spec[1])
    if ms not in cache:
        if ms[0] == "box":
            cache[ms] = world.mesh_box(*ms[1:4])
        elif ms[0] == "sphere":
            cache[ms] = world.mesh_sphere(ms[1])
        else:
            cache[ms] = world.mesh_pyramid(ms[1], ms[2])
    return (2, list(spec[2]) + quat(spec[3]), cache[ms])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_noalloc_matches_pk_collide_twice(precision):
    from physkit_gb300 import World, world_desc

    w = World(world_desc.make().with_precision(precision).with_capacity(64))
    cache = {}
    pairs = _pairs()
    A = [_shape(w, a, cache) for a, _ in pairs]
    B = [_shape(w, b, cache) for _, b in pairs]
    hit_ref, out_ref = w.collide(A, B)  # existing entry point (also uploads the shapes)
    tol = 0.0 if precision == "f64" else 1e-6
    for call in range(2):
        # reversed order on the second call so stale results of the first call would show up
        order = list(range(len(A))) if call == 0 else list(range(len(A)))[::-1]
        hit, out = w.collide([A[i] for i in order], [B[i] for i in order], noalloc=True)
        assert np.array_equal(hit, hit_ref[order]), f"call {call}: hit flags differ"
        assert np.allclose(out, out_ref[order], rtol=0.0, atol=tol), f"call {call}: max diff {np.abs(out - out_ref[order]).max()}"
    w.close()


def test_noalloc_rejects_oversized_batch():
    from physkit_gb300 import World, world_desc

    w = World(world_desc.make().with_capacity(16))
    shape = (0, [-1, -1, -1, 1, 1, 1], -1)
    with pytest.raises(MemoryError):
        w.collide([shape] * 4097, [shape] * 4097, noalloc=True)
    w.close()


def test_noalloc_leaves_free_device_memory_unchanged():
    # The property the entry point exists for, seen from outside: free device memory is the same
    # before and after a few hundred calls (a leaked allocation on this path would show up here;
    # test_noalloc_path_names_no_allocation in test_capi_cpu.py reads the code path itself).
    import torch

    from physkit_gb300 import World, world_desc

    w = World(world_desc.make().with_capacity(64))
    cache = {}
    pairs = _pairs()
    A = [_shape(w, a, cache) for a, _ in pairs]
    B = [_shape(w, b, cache) for _, b in pairs]
    w.collide(A, B)  # uploads the shapes
    w.collide(A, B, noalloc=True)  # first call on the device: looks up the array's address
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(300):
        w.collide(A, B, noalloc=True)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    w.close()
