"""Device world raycast (pk_world_raycast) against the FP64 oracle's world_base::raycast
(world.h:260-319): after some steps, every ray's hit set (body, entry distance) must equal the
oracle's. FP64 form: bit-identical distances. FP32 form: distances within 1e-5 relative, with hits
that graze a box boundary allowed to differ (at most 1% of hits).
"""
import numpy as np
import pytest

import pyoracle
from physkit_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rays(rng, n, centre, spread):
    o = centre + rng.uniform(-spread, spread, (n, 3))
    d = rng.normal(size=(n, 3))
    d[::7, 1] = 0.0  # rays parallel to the y slabs
    d[::9, 0] = 0.0
    o[::13] = centre  # some from inside the pile
    maxd = rng.uniform(0.5, 3 * spread, n)
    return o, d, maxd


def _oracle_hits(ow, o, d, maxd):
    return [sorted(ow.raycast(o[i], d[i], maxd[i]), key=lambda x: (x[1], x[0])) for i in range(len(o))]


def test_fp64_raycast_equals_oracle_after_steps():
    scene = scenes.small_pile(n=45, seed=5, kinds=(0, 1, 2))
    world, handles = scenes.make_world(scene, precision="f64")
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    ohandles = pyoracle.load_scene(ow, scene)
    for _ in range(40):
        world.step(scene.dt)
        ow.step(scene.dt)
    to_idx = {int(h): i for i, h in enumerate(handles)}
    o_to_idx = {int(h): i for i, h in enumerate(ohandles)}
    rng = np.random.default_rng(1)
    o, d, maxd = _rays(rng, 400, np.array([0.0, 1.0, 0.0]), 4.0)
    got, cnt = world.raycast(o, d, maxd, cap=128)
    want = _oracle_hits(ow, o, d, maxd)
    nhits = 0
    for i in range(len(o)):
        g = sorted((to_idx[h], t) for h, t in got[i])
        w = sorted((o_to_idx[h], t) for h, t in want[i])
        assert int(cnt[i]) == len(w)
        assert g == w, f"ray {i}: {g[:4]} vs {w[:4]}"
        nhits += len(w)
    assert nhits > 200  # the rays do hit the pile
    world.close()
    ow.close()


def test_raycast_cap_keeps_nearest_and_counts_all():
    scene = scenes.small_pile(n=60, seed=11)
    world, handles = scenes.make_world(scene, precision="f64")
    for _ in range(20):
        world.step(scene.dt)
    rng = np.random.default_rng(2)
    o, d, maxd = _rays(rng, 200, np.array([0.0, 1.0, 0.0]), 3.0)
    full, cnt_full = world.raycast(o, d, maxd, cap=256)
    few, cnt_few = world.raycast(o, d, maxd, cap=3)
    assert np.array_equal(cnt_full, cnt_few)
    for i in range(len(o)):
        assert len(full[i]) == int(cnt_full[i])
        assert few[i] == full[i][:3]
        assert all(full[i][k][1] <= full[i][k + 1][1] for k in range(len(full[i]) - 1))
    world.close()


def test_raycast_stays_in_its_world_in_a_batch():
    scene = scenes.config3(nworlds=4, nmin=20, nmax=60, seed=21)
    batch, handles = scenes.make_world(scene, precision="f64")
    for _ in range(30):
        batch.step(scene.dt)
    rng = np.random.default_rng(3)
    for w in range(scene.nworlds):
        sub = scenes.Scene("world %d" % w, scene.shapes, scene.world_slice(w).copy(), 1)
        sub.bodies["world"] = 0
        ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
        oh = pyoracle.load_scene(ow, sub)
        for _ in range(30):
            ow.step(scene.dt)
        mine = np.asarray(handles)[scene.bodies["world"] == w]
        to_idx = {int(h): i for i, h in enumerate(mine)}
        o_to_idx = {int(h): i for i, h in enumerate(oh)}
        o, d, maxd = _rays(rng, 150, np.array([0.0, 1.5, 0.0]), 3.0)
        got, cnt = batch.raycast(o, d, maxd, worlds=w, cap=128)
        want = _oracle_hits(ow, o, d, maxd)
        for i in range(len(o)):
            assert all(int(h) in to_idx for h, _ in got[i])  # only this world's bodies
            assert sorted((to_idx[h], t) for h, t in got[i]) == sorted((o_to_idx[h], t) for h, t in want[i])
        ow.close()
    batch.close()


def test_fp32_raycast_close_to_oracle():
    scene = scenes.small_pile(n=45, seed=5, kinds=(0, 1, 2))
    world, handles = scenes.make_world(scene, precision="f32")
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    ohandles = pyoracle.load_scene(ow, scene)  # no steps: both hold the creation state
    to_idx = {int(h): i for i, h in enumerate(handles)}
    o_to_idx = {int(h): i for i, h in enumerate(ohandles)}
    rng = np.random.default_rng(4)
    o, d, maxd = _rays(rng, 400, np.array([0.0, 1.0, 0.0]), 4.0)
    got, _ = world.raycast(o, d, maxd, cap=128)
    want = _oracle_hits(ow, o, d, maxd)
    total = differ = 0
    for i in range(len(o)):
        g = dict((to_idx[h], t) for h, t in got[i])
        w = dict((o_to_idx[h], t) for h, t in want[i])
        total += len(w)
        differ += len(set(g) ^ set(w))
        for k in set(g) & set(w):
            assert abs(g[k] - w[k]) <= 1e-5 * max(1.0, abs(w[k])), (g[k], w[k])
    assert total > 200
    assert differ <= 0.01 * total
    world.close()
    ow.close()
