"""Scenes in the reference's demo JSON format (tests/helper/src/graphics.cpp:20-140) through
scenes.load_json: defaults, single-precision mesh fields, the reference's pyramid argument order,
mesh sharing, and a short oracle run of the fixture scene."""
import os

import numpy as np

import pyoracle
from physkit_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scene_mixed_stack.json")


def test_fields_defaults_and_rounding():
    sc = scenes.load_json(FIXTURE)
    assert sc.gravity == (0.0, -9.81, 0.0) and sc.iterations == 10
    b = sc.bodies
    assert len(b) == 8
    assert b["type"].tolist() == [1, 0, 0, 0, 0, 0, 0, 0]
    # defaults: restitution 0.5, friction 0.5, orientation identity, zero velocities
    assert b["restitution"][4] == 0.5 and b["friction"][4] == 0.5
    assert b["quat"][1].tolist() == [1.0, 0.0, 0.0, 0.0]
    assert b["vel"][1].tolist() == [0.0, 0.0, 0.0] and b["vel"][4].tolist() == [-0.5, 0.0, 0.0]
    assert b["inertia"][5].tolist() == [0.05, 0, 0, 0, 0.08, 0, 0, 0, 0.05]
    # mesh fields are single precision in the reference
    box = sc.shapes[b["shape"][1]]
    assert box == ("box", float(np.float32(0.3)), float(np.float32(0.3)), float(np.float32(0.3)))
    assert box[1] != 0.3
    # the three 0.3 boxes share one mesh; sphere defaults to 16 x 32; the nameless box is a box
    assert b["shape"][1] == b["shape"][2] == b["shape"][3]
    assert sc.shapes[b["shape"][4]] == ("sphere", float(np.float32(0.25)), 16, 32)
    assert sc.shapes[b["shape"][7]] == ("sphere", float(np.float32(0.25)), 8, 16)
    assert sc.shapes[b["shape"][6]][0] == "box"
    # pyramid: `height` goes in as the base half size, `base_size` as the height
    assert sc.shapes[b["shape"][5]] == ("pyramid", float(np.float32(0.3)), float(np.float32(0.6)))


def test_oracle_runs_the_json_scene():
    sc = scenes.load_json(FIXTURE)
    ow = pyoracle.OracleWorld(gravity=sc.gravity, iterations=sc.iterations)
    pyoracle.load_scene(ow, sc)
    # the pyramid mesh (mesh.cpp:117-137): base half 0.3 on y = 0, apex at 0.6
    pyr = np.asarray(ow.vertices(int(sc.bodies["shape"][5]))).reshape(-1, 3)
    assert pyr.shape == (5, 3)
    assert np.allclose(pyr[0], [-0.3, 0.0, -0.3]) and np.allclose(pyr[4], [0.0, 0.6, 0.0])
    for _ in range(120):
        ow.step(sc.dt)
    st = ow.bodies()
    dyn = sc.bodies["type"] == 0
    assert np.isfinite(st[:, :13]).all()
    assert (st[dyn, 1] > -0.2).all()  # nothing falls through the ground
    assert len(ow.pairs()) > 0


def test_json_text_and_unknown_mesh():
    sc = scenes.load_json('{"objects": [{"pos": [0, 1, 0], "mass": 2.0}]}')
    assert sc.shapes == [("box", 0.5, 0.5, 0.5)] and sc.bodies["mass"][0] == 2.0
    try:
        scenes.load_json('{"objects": [{"pos": [0, 1, 0], "mass": 1.0, "mesh": {"name": "torus"}}]}')
    except ValueError:
        pass
    else:
        raise AssertionError("unknown mesh kind accepted")
