"""World-step parity on the GPU (through the C ABI) against the FP64 oracle.

FP64 form: the oracle runs the reference's step with the solver in the GPU's colour order; every
step the pair set, manifolds, colours, events and body states must be bit-identical.
FP32 form: per-quantity error against the FP64 oracle over a short horizon, with the tolerances
written in each test.
"""
import numpy as np
import pytest

import pyoracle
from physkit_gb300 import scenes

pytestmark = pytest.mark.gpu


def run_pair(scene, steps, precision="f64", check_every=1, graph=False):
    world, handles = scenes.make_world(scene, precision=precision)
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    pyoracle.load_scene(ow, scene)
    return world, ow, handles


def compare_step(world, ow, step):
    gp, op = world.pairs(), ow.pairs()
    assert np.array_equal(gp, op), f"pair sets differ at step {step}: {len(gp)} vs {len(op)}"
    gk, gc, gct = world.manifolds()
    ok, oc, oct_ = ow.manifolds()
    assert np.array_equal(gk, ok)
    assert np.array_equal(gc, oc), f"contact counts differ at step {step}"
    assert np.array_equal(gct, oct_), f"contacts differ at step {step}: {np.abs(gct - oct_).max()}"
    gck, gcol, gnc = world.colours()
    ock, ocol, onc = ow.colours()
    assert np.array_equal(gck, ock) and np.array_equal(gcol, ocol) and gnc == onc, f"colours differ at step {step}"
    ge, gkind = world.events()
    oe, okind = ow.events()
    assert np.array_equal(np.sort(ge), np.sort(oe))
    gb, ob = world.bodies(), ow.bodies()
    assert np.array_equal(gb[:, :13], ob[:, :13]), f"body state differs at step {step}: {np.abs(gb[:, :13] - ob[:, :13]).max()}"


def test_fp64_small_box_pile_bit_identical():
    scene = scenes.small_pile(n=60, seed=11)
    world, ow, _ = run_pair(scene, 0)
    for step in range(150):
        world.step(scene.dt)
        ow.step(scene.dt)
        compare_step(world, ow, step)
    world.close()


def test_fp64_mixed_shapes_bit_identical():
    # boxes, UV spheres (482 vertices) and 16-point hulls
    scene = scenes.small_pile(n=45, seed=5, kinds=(0, 1, 2))
    world, ow, _ = run_pair(scene, 0)
    for step in range(120):
        world.step(scene.dt)
        ow.step(scene.dt)
        compare_step(world, ow, step)
    world.close()


def test_fp64_config1_1000_boxes_240_steps():
    scene = scenes.config1()
    world, ow, _ = run_pair(scene, 0)
    for step in range(scene.steps):
        world.step(scene.dt)
        ow.step(scene.dt)
        assert np.array_equal(world.pairs(), ow.pairs()), f"pair set differs at step {step}"
        if step % 20 == 19:
            compare_step(world, ow, step)
    compare_step(world, ow, scene.steps)
    world.close()


def test_fp64_remove_and_add_bodies():
    # world_base::remove_rigid / create_rigid between steps (world.h:202-218)
    scene = scenes.small_pile(n=40, seed=2)
    world, ow, handles = run_pair(scene, 0)
    oh = list(range(len(handles)))
    for step in range(100):
        if step == 40:
            for i in (5, 17, 30):
                assert world.remove_rigid(int(handles[i]))
                assert ow.remove(int(handles[i]))
            assert not world.remove_rigid(int(handles[5]))  # stale handle
        if step == 60:
            rec = scene.bodies[[6, 7]].copy()
            rec["pos"][:, 1] += 3.0
            gh = world.create_rigids(rec.copy())  # shape ids equal scene indices (loaded in order)
            for r in rec:
                ow.add(int(r["shape"]), r["pos"], r["quat"], r["vel"], r["ang_vel"], float(r["mass"]),
                       np.asarray(r["inertia"]).reshape(3, 3), float(r["restitution"]), float(r["friction"]))
            assert [int(h) & 0xFFFFFFFF for h in gh] == [30, 17]  # the arena's free stack is LIFO
        world.step(scene.dt)
        ow.step(scene.dt)
        compare_step(world, ow, step)
    world.close()


# launch shapes of pk_world_set_tuning: one world per solver CTA, and solve groups (several small
# worlds per solver CTA, their colours swept together) at two packings
PER_WORLD = {"solve_threads": 256, "small_world": 512, "narrow_grid": 2, "traverse_threads": 128,
             "big_threads": 256, "group_bodies": 0, "group_threads": 128, "group_warp": 0}
GROUPS = [dict(PER_WORLD, group_bodies=512, group_threads=128),
          dict(PER_WORLD, group_bodies=256, group_threads=64),
          dict(PER_WORLD, group_bodies=1024, group_threads=256, group_warp=1)]  # a warp per member


@pytest.mark.parametrize("tuning", [PER_WORLD, GROUPS[0], GROUPS[2]],
                         ids=["one_world_per_cta", "solve_groups", "solve_groups_warp"])
def test_fp64_dense_cluster_queue_overflow_and_colour_fallback(tuning):
    # 150 boxes crammed into 0.4 m: about 11,000 overlapping pairs, more than the sweep-and-prune
    # queue holds (10,240), so the world's pairs come from its second sweep; and bodies carry ~150
    # manifolds, so first-fit colouring (128 colours at most) gives way to claiming rounds (in a
    # solve group: the group falls back to one world at a time). All paths give the oracle's bits.
    scene = scenes.small_pile(n=150, seed=13, kinds=(1,))
    rng = np.random.default_rng(0)
    dyn = scene.bodies["type"] == 0
    m = int(dyn.sum())
    scene.bodies["pos"][dyn] = np.stack([rng.uniform(-0.2, 0.2, m), 1.5 + rng.uniform(-0.2, 0.2, m),
                                         rng.uniform(-0.2, 0.2, m)], 1)
    world, _ = scenes.make_world(scene, precision="f64", pair_factor=200)
    world.set_tuning(tuning)
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    pyoracle.load_scene(ow, scene)
    for step in range(4):
        world.step(scene.dt)
        ow.step(scene.dt)
        compare_step(world, ow, step)
    assert len(world.pairs()) > 10240
    assert world.colours()[2] > 128
    world.close()
    ow.close()


def test_async_read_back_per_step_equals_synchronous_reads():
    # pk_world_read_bodies_async after each enqueued step (two staging buffers in turn, copies on
    # their own stream) delivers every step's rows, equal to a synchronous read after that step
    scene = scenes.small_pile(n=60, seed=8)
    a, _ = scenes.make_world(scene, precision="f64")
    b, _ = scenes.make_world(scene, precision="f64")
    want = []
    for _ in range(6):
        a.step(scene.dt)
        want.append(a.bodies().copy())
    outs = [np.full((len(scene.bodies), 14), -1.0) for _ in range(6)]
    for o in outs:
        b.pin(o)
    for o in outs:
        b.step_async(scene.dt)
        b.bodies_async(o)
    b.synchronize()
    for k, (w, o) in enumerate(zip(want, outs)):
        assert np.array_equal(w, o), f"step {k + 1}"
    for o in outs:
        b.unpin(o)
    a.close()
    b.close()


def test_read_back_into_pinned_array_equals_fresh_read():
    # pk_world_read_bodies into a caller's page-locked buffer gives the same rows as a fresh read,
    # FP32 and FP64, with an empty slot reading as zeros
    for precision in ("f32", "f64"):
        scene = scenes.small_pile(n=40, seed=9, kinds=(0, 1, 2))
        world, handles = scenes.make_world(scene, precision=precision)
        for _ in range(30):
            world.step(scene.dt)
        assert world.remove_rigid(int(handles[5]))
        world.step(scene.dt)
        host = np.full((len(scene.bodies) + 3, 14), 7.0)
        world.pin(host)
        got = world.bodies(out=host)
        fresh = world.bodies()
        world.unpin(host)
        assert got.base is host
        assert np.array_equal(got, fresh)
        slot = int(handles[5]) & 0xFFFFFFFF
        assert np.all(fresh[slot] == 0.0)
        assert np.all(host[len(fresh):] == 7.0)  # rows past the slots are not touched
        with pytest.raises(ValueError):
            world.bodies(out=np.zeros((2, 14)))
        world.close()


def test_fp64_graph_replay_matches_plain_steps():
    scene = scenes.small_pile(n=50, seed=4)
    a, _ = scenes.make_world(scene, precision="f64")
    b, _ = scenes.make_world(scene, precision="f64")
    b.capture(scene.dt)
    for _ in range(80):
        a.step(scene.dt)
        b.step_graph()
    b.synchronize()
    assert np.array_equal(a.bodies(), b.bodies())
    assert np.array_equal(a.pairs(), b.pairs())
    a.close()
    b.close()


def test_batched_worlds_equal_alone_and_oracle():
    # each world of a batch gives the same bits as the world run alone and as the FP64 oracle
    scene = scenes.config3(nworlds=6, nmin=8, nmax=80, seed=21)
    batch, _ = scenes.make_world(scene, precision="f64")
    for _ in range(60):
        batch.step(scene.dt)
    bb = batch.bodies()
    for w in range(scene.nworlds):
        sub = scenes.Scene("world %d" % w, scene.shapes, scene.world_slice(w).copy(), 1)
        sub.bodies["world"] = 0
        alone, _ = scenes.make_world(sub, precision="f64")
        ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
        pyoracle.load_scene(ow, sub)
        for _ in range(60):
            alone.step(scene.dt)
            ow.step(scene.dt)
        mine = bb[scene.bodies["world"] == w]
        assert np.array_equal(mine, alone.bodies())
        assert np.array_equal(mine[:, :13], ow.bodies()[:, :13])
        alone.close()
        ow.close()
    batch.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_solve_groups_same_bits_as_one_world_per_cta(precision):
    # worlds of 8-300 bodies packed up to 8 per solver CTA (colours swept together, or one member
    # per warp): every body, pair and colour equals the one-world-per-CTA launch bit for bit (members share no bodies, and each keeps its own colours
    # and per-body sweep order); in FP64 three of the worlds are also checked against the oracle
    scene = scenes.config3(nworlds=40, nmin=8, nmax=300, seed=5)
    steps = 60
    ref, _ = scenes.make_world(scene, precision=precision)
    ref.set_tuning(PER_WORLD)
    runs = []
    for t in GROUPS:
        w, _ = scenes.make_world(scene, precision=precision)
        w.set_tuning(t)
        runs.append(w)
    for step in range(steps):
        ref.step(scene.dt)
        for w in runs:
            w.step(scene.dt)
    rk, rc, rn = ref.colours()
    assert rn > 1 and len(rk) > 100  # contacts were solved
    for w in runs:
        assert np.array_equal(w.bodies(), ref.bodies())
        assert np.array_equal(w.pairs(), ref.pairs())
        k, c, n = w.colours()
        assert np.array_equal(k, rk) and np.array_equal(c, rc) and n == rn
    if precision == "f64":
        bb = runs[0].bodies()
        for wi in (0, 17, 39):
            sub = scenes.Scene("world %d" % wi, scene.shapes, scene.world_slice(wi).copy(), 1)
            sub.bodies["world"] = 0
            ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
            pyoracle.load_scene(ow, sub)
            for _ in range(steps):
                ow.step(scene.dt)
            assert np.array_equal(bb[scene.bodies["world"] == wi][:, :13], ow.bodies()[:, :13]), f"world {wi}"
            ow.close()
    for w in [ref] + runs:
        w.close()


def test_fp64_all_pairs_and_tree_worlds_in_one_batch():
    # worlds of at most 2,304 leaves find their pairs by the all-pairs pass in shared memory, larger
    # ones by their LBVH; in one batch both give every world the oracle's bits
    scene = scenes.config3(nworlds=3, nmin=1200, nmax=3600, seed=1, kinds=(1,))
    counts = np.bincount(scene.bodies["world"])
    assert counts.max() > 2304 and counts.min() < 2304
    batch, _ = scenes.make_world(scene, precision="f64", max_bodies_per_world=4096)
    steps = 30
    for _ in range(steps):
        batch.step(scene.dt)
    bb = batch.bodies()
    for w in range(scene.nworlds):
        sub = scenes.Scene("world %d" % w, scene.shapes, scene.world_slice(w).copy(), 1)
        sub.bodies["world"] = 0
        ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
        pyoracle.load_scene(ow, sub)
        for _ in range(steps):
            ow.step(scene.dt)
        assert len(ow.pairs()) > counts[w]  # the piles are in contact
        assert np.array_equal(bb[scene.bodies["world"] == w][:, :13], ow.bodies()[:, :13]), f"world {w}"
        ow.close()
    batch.close()


def test_fp32_error_against_fp64_oracle():
    # precision form: FP32 bulk arithmetic, FP64 accumulated impulses. Free flight + first contacts
    # over 60 steps of config1: positions within 1e-4 relative of the FP64 oracle.
    scene = scenes.config1(n=300)
    world, _ = scenes.make_world(scene, precision="f32")
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    pyoracle.load_scene(ow, scene)
    for _ in range(60):
        world.step(scene.dt)
        ow.step(scene.dt)
    g, o = world.bodies(), ow.bodies()
    dyn = scene.bodies["type"] == 0
    rel = np.linalg.norm(g[dyn, 0:3] - o[dyn, 0:3], axis=1) / np.maximum(np.linalg.norm(o[dyn, 0:3], axis=1), 1.0)
    assert rel.max() < 1e-4, rel.max()
    world.close()


def test_fp64_grid_solver_large_world_bit_identical():
    # 17,000 boxes: above the CTA solver's 16,384-index limit, so the cooperative grid solver runs
    scene = scenes.config1(n=17000, seed=77)
    scene.bodies["pos"][1:, 1] = 0.6 + (scene.bodies["pos"][1:, 1] % 6.0)  # start near the ground
    scene.bodies["pos"][1:, 0] *= 3.0
    scene.bodies["pos"][1:, 2] *= 3.0
    world, ow, _ = run_pair(scene, 0)
    for step in range(40):
        world.step(scene.dt, check=False)
        assert not world.synchronize()["flags"], world.last_info
        ow.step(scene.dt)
        assert np.array_equal(world.pairs(), ow.pairs()), f"pair set differs at step {step}"
    compare_step(world, ow, 40)
    k, col, nc = world.colours()
    assert len(k) > 100 and nc > 1  # contacts were solved
    world.close()


def test_autotune_keeps_results():
    scene = scenes.small_pile(n=60, seed=13)
    a, _ = scenes.make_world(scene, precision="f64")
    b, _ = scenes.make_world(scene, precision="f64")
    r = b.autotune(scene.dt, 1)
    for _ in range(r["steps_used"]):
        a.step(scene.dt)
    for _ in range(20):
        a.step(scene.dt)
        b.step(scene.dt)
    assert np.array_equal(a.bodies(), b.bodies())
    a.close()
    b.close()


def test_fp64_json_scene_bit_identical():
    # a scene in the reference's demo JSON format (boxes, UV spheres of two layouts, a pyramid)
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scene_mixed_stack.json")
    scene = scenes.load_json(path)
    world, ow, _ = run_pair(scene, 0)
    for step in range(180):
        world.step(scene.dt)
        ow.step(scene.dt)
        compare_step(world, ow, step)
    world.close()
