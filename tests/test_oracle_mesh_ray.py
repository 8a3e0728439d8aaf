"""The oracle's mesh ray query (mesh::instance::ray_intersect, mesh.cpp:169-197, 400-415; ray::intersect,
bvh.h:97-135) against analytic hits and an independent numpy Moeller-Trumbore over every triangle."""
import math

import numpy as np

import pyoracle
from physkit_gb300 import scenes


def _rot(q, v):
    w, x, y, z = q
    u = np.array([x, y, z])
    return v + 2 * w * np.cross(u, v) + 2 * np.cross(u, np.cross(u, v))


def _brute(verts, tris, pose, o, d, maxd):
    q = np.asarray(pose[3:7])
    qi = q * np.array([1, -1, -1, -1])
    d = np.asarray(d) / np.linalg.norm(d)
    lo = _rot(qi, np.asarray(o) - np.asarray(pose[:3]))
    ld = _rot(qi, d)
    ld = ld / np.linalg.norm(ld)
    best, bt = None, maxd
    for k, t in enumerate(tris):
        v0, v1, v2 = verts[t[0]], verts[t[1]], verts[t[2]]
        e1, e2 = v1 - v0, v2 - v0
        h = np.cross(ld, e2)
        a = e1 @ h
        if -1e-12 < a < 1e-12:
            continue
        f = 1 / a
        s = lo - v0
        u = f * (s @ h)
        if u < 0 or u > 1:
            continue
        qq = np.cross(s, e1)
        v = f * (ld @ qq)
        if v < 0 or u + v > 1:
            continue
        tt = f * (e2 @ qq)
        if tt < 0 or tt > bt:
            continue
        bt, best = tt, k
    return best, bt


def test_box_hits_are_analytic():
    ow = pyoracle.OracleWorld()
    b = ow.box(0.5, 0.3, 0.2)
    hit = ow.mesh_raycast(b, [0, 0, 0, 1, 0, 0, 0], [5, 0, 0], [-1, 0, 0], 100)
    assert np.allclose(hit[0], [0.5, 0, 0]) and np.allclose(hit[1], [1, 0, 0]) and hit[2] == 4.5
    hit = ow.mesh_raycast(b, [1, 2, 3, 1, 0, 0, 0], [1, 2, 10], [0, 0, -2], 100)
    assert np.allclose(hit[0], [1, 2, 3.2]) and np.allclose(hit[1], [0, 0, 1]) and abs(hit[2] - 6.8) < 1e-12
    assert ow.mesh_raycast(b, [0, 0, 0, 1, 0, 0, 0], [5, 0, 0], [1, 0, 0], 100) is None  # pointing away
    assert ow.mesh_raycast(b, [0, 0, 0, 1, 0, 0, 0], [5, 0, 0], [-1, 0, 0], 4.0) is None  # beyond max distance


def test_random_rays_match_brute_force_numpy():
    rng = np.random.default_rng(3)
    ow = pyoracle.OracleWorld()
    shapes = []
    for k in range(6):
        if k % 3 == 0:
            sid = ow.box(*rng.uniform(0.1, 0.6, 3))
        elif k % 3 == 1:
            sid = ow.sphere(float(rng.uniform(0.2, 0.8)), 8, 16)
        else:
            sh, _, _ = scenes.hull_shape(rng, 0.5)
            sid = ow.mesh(sh[1], sh[2])
        shapes.append(sid)
    nhit = 0
    for sid in shapes:
        verts = ow.vertices(sid)
        tris = ow.triangles(sid)
        for _ in range(80):
            pose = list(rng.uniform(-1, 1, 3)) + list(scenes.random_quats(rng, 1)[0])
            o = np.asarray(pose[:3]) + rng.normal(size=3) * 2.0
            d = np.asarray(pose[:3]) - o + rng.normal(size=3) * 0.3
            got = ow.mesh_raycast(sid, pose, o, d, 50.0)
            tri, t = _brute(verts, tris, pose, o, d, 50.0)
            assert (got is None) == (tri is None)
            if got is not None:
                nhit += 1
                assert got[3] == tri and math.isclose(got[2], t, rel_tol=1e-12, abs_tol=1e-12)
    assert nhit > 100
