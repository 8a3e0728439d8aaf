"""The FP32 precision form against the FP64 oracle over the full 240-step horizon.

Three scenes, with the tolerance written in each test:
- resting boxes (not chaotic): positions within 1e-4 relative after 240 steps and the pair set
  equal to the oracle's in every step;
- resting stacks of three boxes: the pair set equal in every step, positions within 10x of what
  rounding the FP64 oracle's state to float32 after every step does;
- config 1 (1,000 boxes falling into a pile, chaotic): a rounding-sized difference grows into
  different contact outcomes, so the FP32 error is measured against a control, the FP64 oracle
  started from the float32-rounded initial state. FP32 must stay within a small factor of it.
"""
import numpy as np
import pytest

import pyoracle
from physkit_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a[:, 0:3] - b[:, 0:3], axis=1) / np.maximum(np.linalg.norm(b[:, 0:3], axis=1), 1.0)


def _oracle(scene):
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    pyoracle.load_scene(ow, scene)
    return ow


def _oracle_rounded_each_step(scene, steps):
    """The FP64 oracle with every dynamic body's state rounded to float32 after each step: what
    storing the state in FP32 alone does to this scene."""
    ow = _oracle(scene)
    dyn = np.nonzero(scene.bodies["type"] == 0)[0]
    for _ in range(steps):
        ow.step(scene.dt)
        b = ow.bodies()
        for i in dyn:
            ow.write_state(int(i), b[i, :13].astype(np.float32).astype(np.float64))
    return ow


def test_fp32_resting_boxes_240_steps_within_1e4_relative_and_same_pairs():
    # single boxes dropped flat onto the ground: the 1e-4 bound after 240 steps holds outright
    scene = scenes.resting_stacks(height=1)
    world, _ = scenes.make_world(scene, precision="f32")
    ow = _oracle(scene)
    dyn = scene.bodies["type"] == 0
    for step in range(240):
        world.step(scene.dt)
        ow.step(scene.dt)
        assert np.array_equal(world.pairs(), ow.pairs()), f"pair set differs at step {step}"
    rel = _rel(world.bodies()[dyn], ow.bodies()[dyn])
    assert rel.max() <= 1e-4, rel.max()
    world.close()


def test_fp32_resting_stacks_240_steps_at_the_fp32_storage_floor_and_same_pairs():
    # stacks of three boxes: box-on-box contacts amplify rounding (the FP64 oracle with its state
    # rounded to float32 after every step already moves up to ~3e-5 relative), so the FP32 form is
    # held to a factor of that floor; the pair set must still equal the oracle's in every step
    scene = scenes.resting_stacks(height=3)
    world, _ = scenes.make_world(scene, precision="f32")
    ow = _oracle(scene)
    dyn = scene.bodies["type"] == 0
    for step in range(240):
        world.step(scene.dt)
        ow.step(scene.dt)
        assert np.array_equal(world.pairs(), ow.pairs()), f"pair set differs at step {step}"
    ref = ow.bodies()[dyn]
    floor = _rel(_oracle_rounded_each_step(scene, 240).bodies()[dyn], ref).max()
    rel = _rel(world.bodies()[dyn], ref).max()
    assert rel <= 10.0 * floor, (rel, floor)
    world.close()


def test_fp32_config1_error_at_the_rounding_control():
    import bench

    scene = scenes.config1()
    world, _ = scenes.make_world(scene, precision="f32")
    ow, oc = _oracle(scene), _oracle(bench._rounded_to_f32(scene))
    dyn = scene.bodies["type"] == 0
    for _ in range(60):
        world.step(scene.dt, check=False)
        ow.step(scene.dt)
        oc.step(scene.dt)
    ref = ow.bodies()[dyn]
    err32 = _rel(world.bodies()[dyn], ref).max()
    errc = _rel(oc.bodies()[dyn], ref).max()
    # FP32 per-step rounding against one FP32-sized perturbation of the start: same order
    assert err32 <= 10.0 * errc + 1e-6, (err32, errc)
    world.close()
