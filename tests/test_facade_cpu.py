"""The C++20 facade (include/physkit_gb300.hpp) compiles with -Wall -Wextra -Werror against the
C ABI, links the in-tree library, keeps the reference's error conventions and, without a device,
reports the C ABI's PK_ERR_NO_DEVICE as physkit_gb300::error instead of falling back to the CPU."""
import os
import subprocess

import pytest

from facade_build import build_facade_pile, write_scene


def test_facade_compiles_links_and_reports_no_device(tmp_path):
    import torch

    from physkit_gb300 import scenes

    exe = build_facade_pile()
    scene = scenes.small_pile(n=8, seed=3)
    write_scene(scene, tmp_path / "scene.bin")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: tests/test_gpu_facade.py runs the program")
    r = subprocess.run([exe, str(tmp_path / "scene.bin"), "4", str(tmp_path / "out.bin")], capture_output=True,
                       text=True, timeout=120)
    assert "missing mesh: std::invalid_argument" in r.stdout
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert not os.path.exists(tmp_path / "out.bin")
