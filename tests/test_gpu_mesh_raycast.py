"""Mesh ray queries on the GPU (pk_mesh_raycast) against the oracle's restatement of
mesh::instance::ray_intersect (mesh.cpp:169-197, 400-415): boxes, UV spheres, 16-point hulls and a
pyramid at random poses, rays aimed at the shapes (some from inside, some missing, some beyond the
limit). FP64: hit, triangle, distance, point and normal bit-identical; FP32: the same triangle where
the hit is not within rounding of a triangle edge, distance within 1e-5 relative. Then rays against
bodies of a stepped pile, whose poses the device reads itself."""
import numpy as np
import pytest

import pyoracle
from physkit_gb300 import World, scenes, world_desc

pytestmark = pytest.mark.gpu


def _shapes(world, ow, rng):
    ids = []
    for k in range(9):
        if k % 4 == 0:
            he = rng.uniform(0.1, 0.6, 3)
            ids.append((world.mesh_box(*he), ow.box(*he)))
        elif k % 4 == 1:
            r = float(rng.uniform(0.2, 0.8))
            ids.append((world.mesh_sphere(r, 16, 32), ow.sphere(r, 16, 32)))
        elif k % 4 == 2:
            sh, _, _ = scenes.hull_shape(rng, 0.5)
            ids.append((world.mesh_make(sh[1], sh[2]), ow.mesh(sh[1], sh[2])))
        else:
            ids.append((world.mesh_pyramid(0.4, 0.7), ow.pyramid(0.4, 0.7)))
    return ids


def _rays(rng, n):
    out = []
    for i in range(n):
        pose = list(rng.uniform(-2, 2, 3)) + list(scenes.random_quats(rng, 1)[0])
        o = np.asarray(pose[:3]) + rng.normal(size=3) * (0.1 if i % 7 == 0 else 2.0)  # some start inside
        d = np.asarray(pose[:3]) - o + rng.normal(size=3) * 0.4
        maxd = 1.0 if i % 11 == 0 else 50.0
        out.append((pose, o, d, maxd))
    return out


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_mesh_raycast_matches_oracle(precision):
    rng = np.random.default_rng(17)
    w = World(world_desc.make().with_precision(precision).with_capacity(64, max_shape_vertices=8192))
    ow = pyoracle.OracleWorld()
    ids = _shapes(w, ow, rng)
    rays, expect = [], []
    for k, (pose, o, d, maxd) in enumerate(_rays(rng, 900)):
        gid, oid = ids[k % len(ids)]
        rays.append({"shape": gid, "pos": pose[:3], "quat": pose[3:], "origin": o, "direction": d, "max_distance": maxd})
        expect.append(ow.mesh_raycast(oid, pose, o, d, maxd))
    got = w.mesh_raycast(rays)
    nhit, agree = 0, 0
    for g, e in zip(got, expect):
        if precision == "f64":
            assert (g is None) == (e is None)
            if e is None:
                continue
            nhit += 1
            assert g[3] == e[3] and g[2] == e[2]
            assert np.array_equal(g[0], e[0]) and np.array_equal(g[1], e[1])
        else:
            if g is None or e is None:
                continue  # grazing rays may flip in FP32
            nhit += 1
            assert abs(g[2] - e[2]) <= 1e-5 * max(1.0, e[2])
            agree += g[3] == e[3]
    assert nhit > 300
    if precision == "f32":
        assert agree >= 0.97 * nhit
    w.close()


def test_mesh_raycast_on_stepped_bodies():
    scene = scenes.small_pile(n=30, seed=4, kinds=(0, 1, 2))
    world, handles = scenes.make_world(scene, precision="f64")
    ow = pyoracle.OracleWorld()
    oids = []
    for s in scene.shapes:
        if s[0] == "box":
            oids.append(ow.box(*s[1:4]))
        elif s[0] == "sphere":
            oids.append(ow.sphere(s[1], s[2], s[3]))
        else:
            oids.append(ow.mesh(s[1], s[2]))
    for _ in range(30):
        world.step(scene.dt)
    b = world.bodies()
    rng = np.random.default_rng(5)
    rays, expect = [], []
    for i, h in enumerate(handles):
        slot = int(h) & 0xFFFFFFFF
        pose = b[slot, 0:7]
        for _ in range(6):
            o = pose[:3] + rng.normal(size=3) * 3.0
            d = pose[:3] - o + rng.normal(size=3) * 0.2
            rays.append({"body": int(h), "origin": o, "direction": d, "max_distance": 30.0})
            expect.append(ow.mesh_raycast(oids[int(scene.bodies["shape"][i])], pose, o, d, 30.0))
    got = world.mesh_raycast(rays)
    nhit = 0
    for g, e in zip(got, expect):
        assert (g is None) == (e is None)
        if e is not None:
            nhit += 1
            assert g[3] == e[3] and g[2] == e[2] and np.array_equal(g[0], e[0]) and np.array_equal(g[1], e[1])
    assert nhit > 60
    world.close()
