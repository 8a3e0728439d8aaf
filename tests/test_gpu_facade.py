"""A pile of boxes stepped through the C++20 facade (tests/cpp/facade_pile.cpp) ends bit-identical
to the FP64 oracle stepped with the same removal, and the pair sets agree."""
import subprocess

import numpy as np
import pytest

import pyoracle
from facade_build import build_facade_pile, read_result, write_scene
from physkit_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_facade_pile_bit_identical_to_oracle(tmp_path):
    exe = build_facade_pile()
    scene = scenes.small_pile(n=40, seed=21)
    steps = 80
    write_scene(scene, tmp_path / "scene.bin")
    r = subprocess.run([exe, str(tmp_path / "scene.bin"), str(steps), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    rows, pairs = read_result(tmp_path / "out.bin")
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    handles = pyoracle.load_scene(ow, scene)
    for s in range(steps):
        if s == steps // 2:
            assert ow.remove(handles[-1])
        ow.step(scene.dt)
    ob = ow.bodies()
    assert rows.shape == ob.shape
    assert np.array_equal(rows[:, :13], ob[:, :13]), np.abs(rows[:, :13] - ob[:, :13]).max()
    assert np.array_equal(pairs, ow.pairs())
