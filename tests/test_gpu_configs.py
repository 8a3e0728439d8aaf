"""Configs 2 and 5 at reduced size on the GPU.

- config 2 (mixed convex bodies in a cube, one world): a 20,000-body world at config 2's density,
  bit-identical to the FP64 oracle for 20 steps (pair set every step, full state at the end). Above
  16,384 bodies the world runs the grid-wide solver and the LBVH broadphase.
- config 5 (dense sphere pile): its 10,000-sphere sub-region replica bit-identical to the FP64
  oracle over the first steps of the pour (parallel first-fit colouring), and the FP32 form's
  kinetic energy and penetration depth against the FP64 form over 120 steps, measured against what
  rounding the start to float32 does to the FP64 form (the pile is chaotic), bounds written below.
"""
import numpy as np
import pytest

import bench
import pyoracle
from physkit_gb300 import scenes
from test_gpu_world_parity import compare_step

pytestmark = pytest.mark.gpu


def _pair(scene, precision="f64", pair_factor=8, contact_factor=0):
    world, _ = scenes.make_world(scene, precision=precision, pair_factor=pair_factor, contact_factor=contact_factor)
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    pyoracle.load_scene(ow, scene)
    return world, ow


def test_fp64_config2_20k_world_bit_identical():
    scene = scenes.config2(n=20_000, extent=200.0 * (20_000 / 100_000) ** (1 / 3))
    world, ow = _pair(scene, pair_factor=4)
    for step in range(20):
        world.step(scene.dt)
        ow.step(scene.dt)
        assert np.array_equal(world.pairs(), ow.pairs()), f"pair set differs at step {step}"
    compare_step(world, ow, 20)
    world.close()


def test_fp64_config5_replica_bit_identical():
    scene = scenes.config5(n=10_000, half=1.0)
    world, ow = _pair(scene, pair_factor=128, contact_factor=8)
    for step in range(6):
        world.step(scene.dt)
        ow.step(scene.dt)
        compare_step(world, ow, step)
    assert len(world.pairs()) > 500_000  # the lattice's fat boxes overlap: a dense broadphase
    k, col, nc = world.colours()
    assert len(k) > 1000 and nc > 4  # contacts were coloured and solved
    world.close()


def test_config5_replica_fp32_energy_and_depth_at_the_rounding_control():
    sc = scenes.config5(n=10_000, half=1.0)
    ws = {"f32": scenes.make_world(sc, precision="f32", pair_factor=128, contact_factor=8)[0],
          "f64": scenes.make_world(sc, precision="f64", pair_factor=128, contact_factor=8)[0],
          "control": scenes.make_world(bench._rounded_to_f32(sc), precision="f64", pair_factor=128,
                                       contact_factor=8)[0]}
    for s in range(1, 121):
        for w in ws.values():
            w.step(sc.dt)  # raises on a device status bit (caps, overflow, non-finite state)
        if s in (60, 120):
            st = {k: bench.pile_stats(w, sc) for k, w in ws.items()}
            ref = st["f64"]
            ke = {k: abs(st[k]["ke_j"] - ref["ke_j"]) / ref["ke_j"] for k in ("f32", "control")}
            dp = {k: abs(st[k]["depth_p99_m"] - ref["depth_p99_m"]) for k in ("f32", "control")}
            pe = abs(st["f32"]["pe_j"] - ref["pe_j"]) / abs(ref["pe_j"])
            # kinetic energy within 3x the control's error or 2 %; p99 penetration depth within 3x
            # the control's or 1 mm; potential energy (where the pile's mass sits) within 0.1 %
            assert ke["f32"] <= max(3.0 * ke["control"], 0.02), (s, ke)
            assert dp["f32"] <= max(3.0 * dp["control"], 1e-3), (s, dp)
            assert pe <= 1e-3, (s, pe)
    for w in ws.values():
        w.close()
