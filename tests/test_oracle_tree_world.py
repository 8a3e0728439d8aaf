"""Oracle pins beyond GJK/EPA: the dynamic AABB tree known answers (tests/dynamic_bvh/main.cpp),
mesh factories and support (tests/mesh/main.cpp), the deterministic sine/cosine, and the world-level
collision event semantics (tests/co/co_tests.cpp:383-430)."""
import math

import numpy as np
import pytest

import pyoracle


def box(cx, cy, cz, half=0.5):
    return [cx - half, cy - half, cz - half, cx + half, cy + half, cz + half]


def inter(a, b):
    return all(a[i] <= b[i + 3] and a[i + 3] >= b[i] for i in range(3))


def test_tree_update_hysteresis():
    # dynamic_bvh/main.cpp:149-163: first update always reinserts, a tiny move then does not.
    t = pyoracle.OracleTree()
    h = t.add(0, box(0, 0, 0))
    assert np.allclose(t.bounds(h), box(0, 0, 0))
    assert t.update(h, box(0.01, 0, 0), [0.01, 0, 0])
    assert not t.update(h, box(0.02, 0, 0), [0, 0, 0])
    fat = t.bounds(h)
    # margin 0.1 m plus the displacement on its sign side (bvh.cpp:487-506)
    assert np.allclose(fat, [-0.49 - 0.1, -0.6, -0.6, 0.51 + 0.1 + 0.01, 0.6, 0.6])


def test_tree_update_escape_and_predictive():
    # dynamic_bvh/main.cpp:165-208
    t = pyoracle.OracleTree()
    h = t.add(0, box(0, 0, 0))
    assert t.update(h, box(10, 10, 10), [10, 10, 10])
    assert 0 in set(t.query(box(10, 10, 10, 2)).tolist())
    t2 = pyoracle.OracleTree()
    h2 = t2.add(0, box(0, 0, 0))
    t2.update(h2, box(5, 0, 0), [2, 0, 0])
    assert t2.bounds(h2)[3] > box(5, 0, 0)[3]


@pytest.mark.parametrize("seed", [12345, 2025, 1337])
def test_tree_query_bruteforce(seed):
    # dynamic_bvh/main.cpp:279-311, 600-635: query results cover every brute-force overlap.
    rng = np.random.default_rng(seed)
    t = pyoracle.OracleTree()
    boxes, leaves = [], []
    for i in range(200):
        b = box(*rng.uniform(-50, 50, 3), 0.5)
        leaves.append(t.add(i, b))
        boxes.append(b)
    assert t.validate()
    q = box(0, 0, 0, 10)
    found = set(t.query(q).tolist())
    brute = {i for i, b in enumerate(boxes) if inter(b, q)}
    assert brute <= found
    # interleaved churn (main.cpp:787-856): moves, removals, queries stay consistent
    alive = set(range(200))
    for step in range(500):
        i = int(rng.integers(0, 200))
        if i in alive and rng.random() < 0.1:
            t.remove(leaves[i])
            alive.discard(i)
            continue
        if i in alive:
            c = rng.uniform(-50, 50, 3)
            boxes[i] = box(*c, 0.5)
            t.update(leaves[i], boxes[i], rng.uniform(-1, 1, 3))
    assert t.validate()
    for _ in range(20):
        q = box(*rng.uniform(-50, 50, 3), 8)
        found = set(t.query(q).tolist())
        fat_hits = {i for i in alive if inter(t.bounds(leaves[i]), q)}
        assert found == fat_hits


def test_mesh_factories_and_support():
    w = pyoracle.OracleWorld()
    b = w.box(1, 2, 3)
    v = w.vertices(b)
    assert v.shape == (8, 3)  # mesh/main.cpp:325-326
    assert np.allclose(v[0], [-1, -2, -3]) and np.allclose(v[6], [1, 2, 3])
    s = w.sphere(1.0)
    assert w.vertices(s).shape == (2 + 15 * 32, 3)  # 482 vertices (mesh.cpp:60-115)
    assert abs(w.volume(b) - 48.0) < 1e-12
    # unit sphere volume converges to 4/3 pi from below for a UV mesh
    assert 3.9 < w.volume(s) < 4.0 * math.pi / 3.0


def test_sincos_accuracy():
    xs = np.concatenate([np.linspace(-50, 50, 20001), np.geomspace(1e-12, 3.0, 2000)])
    worst = 0.0
    for x in xs:
        s, c = pyoracle.sincos(x)
        es, ec = math.sin(x), math.cos(x)
        us = abs(s - es) / max(abs(math.ulp(es)), 5e-324)
        uc = abs(c - ec) / max(abs(math.ulp(ec)), 5e-324)
        worst = max(worst, min(us, abs(s - es) / 1e-300), min(uc, abs(c - ec) / 1e-300))
    assert worst <= 4.0, worst


def test_world_collision_events():
    # co_tests.cpp:383-430 restated: zero gravity, unit boxes at x=-1 and x=1 approach at 1 m/s
    # under a 5 ms fixed step; a-b begin then end, nothing with the far box c.
    w = pyoracle.OracleWorld(gravity=(0, 0, 0))
    m = w.box(1, 1, 1)
    a = w.add(m, [-1, 0, 0], vel=[1, 0, 0])
    b = w.add(m, [1, 0, 0], vel=[-1, 0, 0])
    c = w.add(m, [0, 10, 0])
    key_ab = (0 << 32) | 1
    seen = []
    for _ in range(1000):
        w.step(0.005)
        ks, kinds = w.events()
        seen += list(zip(ks.tolist(), kinds.tolist()))
    kinds_ab = [k for key, k in seen if key == key_ab]
    assert kinds_ab and kinds_ab[0] == 1 and 2 in kinds_ab
    assert all(key == key_ab for key, _ in seen)
    w.close()


def test_box_comes_to_rest_on_ground():
    w = pyoracle.OracleWorld()
    g = w.box(10, 0.5, 10)
    m = w.box(0.5, 0.5, 0.5)
    w.add(g, [0, -0.5, 0], static=True)
    w.add(m, [0, 2, 0], mass=1.0, inertia=np.eye(3) / 6.0, restitution=0.0)
    for _ in range(600):
        w.step(1 / 120)
    st = w.bodies()[1]
    assert abs(st[1] - 0.5) < 0.02
    assert np.linalg.norm(st[7:10]) < 0.05
    w.close()


def _slab_hit(box, o, d, maxd):
    """ray::intersect_distance (bvh.h:62-93) restated in numpy float64 for the brute-force check."""
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.float64(1.0) / d
        lo = (box[:3] - o) * inv
        hi = (box[3:] - o) * inv
    lo = np.where(np.isnan(lo), -np.inf, lo)
    hi = np.where(np.isnan(hi), np.inf, hi)
    tmin = np.max(np.minimum(lo, hi))
    tmax = np.min(np.maximum(lo, hi))
    if tmax >= 0.0 and tmin <= tmax and tmin <= maxd:
        return max(0.0, tmin)
    return None


@pytest.mark.parametrize("seed", [3, 4])
def test_world_raycast_bruteforce_and_merge_order(seed):
    """world_base::raycast (world.h:260-319): the hit set equals a brute-force slab test over every
    body's broadphase box (exact boxes before the first step), distances bit-identical, each body
    once."""
    rng = np.random.default_rng(seed)
    ow = pyoracle.OracleWorld(gravity=(0, 0, 0))
    boxes, handles = [], []
    for k in range(60):
        he = rng.uniform(0.1, 0.6, 3)
        sh = ow.box(*he)
        pos = rng.uniform(-6, 6, 3)
        static = k % 7 == 0
        handles.append(ow.add(sh, tuple(pos), static=static))
        boxes.append(np.concatenate([pos - he, pos + he]))
    boxes = np.array(boxes)
    for r in range(200):
        o = rng.uniform(-8, 8, 3)
        dv = rng.normal(size=3)
        if r % 5 == 0:
            dv[r % 3] = 0.0  # parallel to a slab pair: the NaN limits
        if r % 11 == 0:
            o = boxes[r % len(boxes)][:3] + 0.01  # origin inside a box: distance 0
        maxd = float(rng.uniform(1, 20))
        got = ow.raycast(o, dv, maxd)
        n2 = float(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2])
        dn = dv / math.sqrt(n2)
        want = {}
        for i, b in enumerate(boxes):
            t = _slab_hit(b, o, dn, maxd)
            if t is not None:
                want[int(handles[i])] = t
        assert {h for h, _ in got} == set(want)
        for h, t in got:
            assert t == want[h]
        assert len(got) == len(want)  # no body twice


def _joint_world():
    ow = pyoracle.OracleWorld(gravity=(0, -9.81, 0))
    box = ow.box(0.2, 0.2, 0.2)
    anchor = ow.add(box, (0, 5, 0), static=True)
    return ow, box, anchor


def test_oracle_ball_socket_pendulum_keeps_the_anchor():
    # ball_socket_constraint (constraint.h:368-453): the shared anchor point stays together
    ow, box, anchor = _joint_world()
    bob = ow.add(box, (1.0, 5.0, 0.0), mass=1.0, inertia=(0.03, 0.03, 0.03))
    h = ow.add_joint("ball_socket", anchor, bob, anchor=(0.0, 5.0, 0.0))
    for _ in range(240):
        ow.step(1 / 120)
    st = ow.bodies()[int(bob) & 0xFFFFFFFF]
    assert st[1] < 5.0  # it swung down
    assert abs(np.linalg.norm(st[0:3] - np.array([0.0, 5.0, 0.0])) - 1.0) < 0.05  # ~1 m from the anchor
    assert len(ow.joint_impulses(h)) == 3 and np.any(ow.joint_impulses(h) != 0)


def test_oracle_joint_types_stay_finite_and_hold():
    ow, box, anchor = _joint_world()
    bodies = [ow.add(box, (x, 5.0 - 0.6, 0.0), mass=1.0, inertia=(0.03, 0.03, 0.03)) for x in (-3, -1.5, 0, 1.5, 3, 4.5)]
    hs = [ow.add_joint("distance", anchor, bodies[0], local_a=(0, 0, 0), local_b=(0, 0.2, 0), distance=1.0),
          ow.add_joint("hinge", anchor, bodies[1], local_a=(0, 0, 0), local_b=(0, 0.6, 0), axis_a=(0, 0, 1), axis_b=(0, 0, 1)),
          ow.add_joint("slider", anchor, bodies[2], anchor=(0, 4.4, 0), axis_a=(0, 1, 0)),
          ow.add_joint("weld", anchor, bodies[3], anchor=(1.5, 5.0, 0)),
          ow.add_joint("spring", anchor, bodies[4], local_b=(0, 0.2, 0), distance=1.0, stiffness=50.0, damping=1.0),
          ow.add_joint("ball_socket", bodies[4], bodies[5], anchor=(3.75, 4.4, 0))]
    for _ in range(120):
        ow.step(1 / 120)
    st = ow.bodies()
    assert np.isfinite(st[:, :13]).all()
    w = st[int(bodies[3]) & 0xFFFFFFFF]
    assert np.linalg.norm(w[0:3] - np.array([1.5, 4.4, 0.0])) < 0.05  # the weld holds the box in place
    assert [len(ow.joint_impulses(h)) for h in hs] == [1, 5, 5, 6, 1, 3]
    assert ow.remove_joint(hs[0]) and not ow.remove_joint(hs[0])
    ow.step(1 / 120)


def test_colour_order_first_fit_in_key_order():
    # the colour order the device solver sweeps in, as the oracle restates it: in a world of at
    # most 4,096 slots every manifold takes the lowest colour no earlier manifold (key order) on one
    # of its dynamic bodies has; colours are then a proper colouring of the shared dynamic bodies
    from physkit_gb300 import scenes

    scene = scenes.small_pile(n=80, seed=3, kinds=(0, 1, 2))
    ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="colour")
    pyoracle.load_scene(ow, scene)
    static = scene.bodies["type"] != 0
    checked = 0
    for step in range(90):
        ow.step(scene.dt)
        if step % 10:
            continue
        keys, cols, nc = ow.colours()
        used = {}
        for k, c in zip(keys.tolist(), cols.tolist()):
            lo, hi = k >> 32, k & 0xFFFFFFFF
            dyn = [b for b in (lo, hi) if not static[b]]
            taken = set().union(*(used.get(b, set()) for b in dyn)) if dyn else set()
            want = next(x for x in range(len(keys) + 1) if x not in taken)
            assert c == want, (step, k, c, want)
            for b in dyn:
                used.setdefault(b, set()).add(c)
            checked += 1
        assert nc == (max(cols) + 1 if len(cols) else 0)
    assert checked > 50
    ow.close()
