"""Joints (constraint.h:139-865) on the GPU against the FP64 oracle: every joint type, alone and in
a chain that also touches the ground, bit-identical body states and joint impulses every step
(FP64 form); a joint removed mid-run; the FP32 form close to FP64 over a short horizon."""
import numpy as np
import pytest

import pyoracle
from physkit_gb300 import scenes
from physkit_gb300.world import BODY_DTYPE

pytestmark = pytest.mark.gpu


def _scene(n_dyn, spacing=1.0, y=4.4):
    shapes = [("box", 0.2, 0.2, 0.2), ("box", 8.0, 0.5, 8.0)]
    b = np.zeros(2 + n_dyn, dtype=BODY_DTYPE)
    b["quat"][:, 0] = 1.0
    b["mass"] = 1.0
    b["inertia"][:, [0, 4, 8]] = 0.03
    b["restitution"] = 0.2
    b["friction"] = 0.5
    b["type"][:2] = 1
    b["shape"][1] = 1
    b["pos"][0] = (0.0, 5.0, 0.0)     # static anchor box
    b["pos"][1] = (0.0, -0.5, 0.0)    # ground
    for i in range(n_dyn):
        b["pos"][2 + i] = (-3.0 + spacing * i, y, 0.3 * (i % 2))
    rng = np.random.default_rng(5)
    b["quat"][2:] = scenes.random_quats(rng, n_dyn) if n_dyn else b["quat"][2:]
    return scenes.Scene("joints", shapes, b, 1, (0.0, -9.81, 0.0))


JOINTS = [
    ("distance", dict(local_a=(0, 0, 0), local_b=(0.1, 0.2, 0), distance=1.2)),
    ("ball_socket", dict(anchor=(-2.0, 4.8, 0.0))),
    ("hinge", dict(local_a=(0, 0, 0), local_b=(0, 0.6, 0), axis_a=(0, 0, 1), axis_b=(0.1, 0.0, 1.0))),
    ("slider", dict(anchor=(0.0, 4.6, 0.0), axis_a=(0.2, 1.0, 0.0))),
    ("weld", dict(anchor=(1.0, 4.7, 0.1))),
    ("spring", dict(local_b=(0, 0.2, 0), distance=1.0, stiffness=60.0, damping=0.8)),
]


def _pair(scene, joints, precision="f64"):
    world, gh = scenes.make_world(scene, precision=precision)
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    oh = pyoracle.load_scene(ow, scene)
    gj, oj = [], []
    for kind, kw, ia, ib in joints:
        gj.append(world.add_joint(kind, gh[ia], gh[ib], **kw))
        oj.append(ow.add_joint(kind, oh[ia], oh[ib], **kw))
    return world, ow, gj, oj


@pytest.mark.parametrize("idx", range(len(JOINTS)))
def test_fp64_each_joint_type_bit_identical(idx):
    kind, kw = JOINTS[idx]
    scene = _scene(1, y=4.4)
    world, ow, gj, oj = _pair(scene, [(kind, kw, 0, 2)])
    for step in range(200):
        world.step(scene.dt)
        ow.step(scene.dt)
        g, o = world.bodies(), ow.bodies()
        assert np.array_equal(g[:, :13], o[:, :13]), f"{kind} step {step}: {np.abs(g[:, :13] - o[:, :13]).max()}"
        assert np.array_equal(world.joint_impulses(gj[0]), ow.joint_impulses(oj[0])), f"{kind} impulses step {step}"
    assert np.any(world.joint_impulses(gj[0]) != 0)
    world.close()
    ow.close()


def test_fp64_chain_with_contacts_and_removal_bit_identical():
    # a chain of all joint types hanging from the static box, swinging into the ground
    scene = _scene(6, spacing=0.7, y=3.0)
    joints = [(k, kw, 0 if i == 0 else 1 + i, 2 + i) for i, (k, kw) in enumerate(JOINTS)]
    world, ow, gj, oj = _pair(scene, joints)
    for step in range(240):
        if step == 120:
            world.remove_joint(gj[2])
            assert ow.remove_joint(oj[2])
        world.step(scene.dt)
        ow.step(scene.dt)
        g, o = world.bodies(), ow.bodies()
        assert np.array_equal(g[:, :13], o[:, :13]), f"step {step}: {np.abs(g[:, :13] - o[:, :13]).max()}"
        assert np.array_equal(world.pairs(), ow.pairs())
    for k, (h, hh) in enumerate(zip(gj, oj)):
        if k != 2:
            assert np.array_equal(world.joint_impulses(h), ow.joint_impulses(hh))
    world.close()
    ow.close()


def test_fp32_joints_close_to_fp64():
    scene = _scene(6, spacing=0.7, y=3.0)
    joints = [(k, kw, 0 if i == 0 else 1 + i, 2 + i) for i, (k, kw) in enumerate(JOINTS)]
    world, ow, gj, oj = _pair(scene, joints, precision="f32")
    for _ in range(60):
        world.step(scene.dt)
        ow.step(scene.dt)
    g, o = world.bodies(), ow.bodies()
    assert np.isfinite(g[:, :13]).all()
    assert np.abs(g[:, 0:3] - o[:, 0:3]).max() < 1e-3
    world.close()
    ow.close()
