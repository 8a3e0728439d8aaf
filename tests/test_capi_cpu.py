"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, exports every symbol that
include/*.h declares, and refuses to run without a device (no CPU fallback)."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(pk_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from physkit_gb300 import build

    path = build.build()
    L = C.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_descriptor_layouts_match_header():
    from physkit_gb300 import world

    assert world.BODY_DTYPE.itemsize == 216
    assert C.sizeof(world.WorldDescC) == 64  # 3 doubles, 9 int32, padded to 8 bytes
    assert C.sizeof(world.CollideShapeC) == 88
    assert C.sizeof(world.RayC) == 64


def test_no_device_is_an_error_not_a_fallback():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from physkit_gb300 import World, lib

    L = lib()
    with pytest.raises(RuntimeError, match="no CUDA device"):
        World()
    assert L.pk_version().decode().startswith("physkit_gb300")


def test_host_register_rejects_invalid_arguments():
    # argument checks come before any CUDA call, so they hold without a device too
    from physkit_gb300 import lib
    from physkit_gb300.world import PK_ERR_INVALID

    L = lib()
    assert L.pk_host_register(None, 0) == PK_ERR_INVALID
    assert L.pk_host_unregister(None) == PK_ERR_INVALID


def test_tune_result_layout():
    from physkit_gb300 import world

    # solve_threads, small_world, narrow_grid, traverse_threads, 2 doubles, steps_used, big_threads,
    # group_bodies, group_threads, group_warp (the doubles start at offset 16)
    assert C.sizeof(world.TuneResultC) == 56
    assert world.TuneResultC.step_ms_before.offset == 16


def _function_body(src, signature_start):
    i = src.index(signature_start)
    j = src.index("{", i)
    depth, k = 0, j
    while True:
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[j:k + 1]
        k += 1


def test_noalloc_path_names_no_allocation():
    # pk_collide_noalloc and everything it calls on the device path: no device or host allocation
    csrc = os.path.join(ROOT, "physkit_gb300", "csrc")
    capi = open(os.path.join(csrc, "pk_capi.cu")).read()
    host = open(os.path.join(csrc, "pk_engine_host.cuh")).read()
    bodies = [_function_body(capi, "int pk_collide_noalloc("),
              _function_body(capi, "int scratch_for_world_device("),
              _function_body(host, "int collide_device(")]
    banned = re.compile(r"cudaMalloc|cudaFree|cuMem|malloc\(|\bnew\b|std::vector|torch")
    for b in bodies:
        assert not banned.search(b), banned.search(b).group(0)
    assert "cudaGetSymbolAddress" in bodies[1]
