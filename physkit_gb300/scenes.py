"""Seeded synthetic scenes for the world-step workloads (no dataset is involved).

Every scene is a list of shapes plus a structured array of body descriptors (world.BODY_DTYPE)
that both the device library and the FP64 oracle consume unchanged, so their inputs are identical.

  config1  1,000 dynamic boxes (half-extents U[0.1,0.5] m, density 1000 kg/m^3) above a static
           ground box (100 x 1 x 100 m, top at y = 0), uniform random orientation, at rest.
  config2  N convex bodies in a 200 m cube: 1/3 UV spheres (r ~ lognormal(ln 0.3, 0.4)),
           1/3 boxes (half-extents U[0.1,0.6]), 1/3 hulls of 16 points on a sphere of radius
           U[0.2,0.6]; velocities N(0, 1 m/s) per axis.
  config3  W independent worlds with log-uniform body counts in [nmin, nmax]; each a pile of
           boxes/spheres/hulls dropped into a 5 m walled bin (static floor + 4 walls).
  config5  spheres (r ~ lognormal(ln 0.05, 0.3)) poured into a 20 x 20 m open box.

Mass properties (the reference's mesh::mass_center / inertia_tensor throw, mesh.cpp:154-166):
box m = rho*8*hx*hy*hz, I = m/3 diag(hy^2+hz^2, hx^2+hz^2, hx^2+hy^2); sphere m = rho*4/3*pi*r^3,
I = 2/5 m r^2; hull m = rho*volume(hull), I = the box inertia of its local AABB.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .world import BODY_DTYPE

RHO = 1000.0
SEED_BASE = 0x50484B0000000000


@dataclasses.dataclass
class Scene:
    name: str
    shapes: list            # ("box", hx, hy, hz) | ("sphere", r, stacks, sectors) | ("pyramid", base_half, height)
                            # | ("mesh", verts, tris)
    bodies: np.ndarray      # BODY_DTYPE records; "shape" indexes `shapes`
    nworlds: int = 1
    gravity: tuple = (0.0, -9.81, 0.0)
    dt: float = 1.0 / 120.0
    steps: int = 240
    iterations: int = 10

    @property
    def n_dynamic(self):
        return int(np.count_nonzero(self.bodies["type"] == 0))

    def vertex_count(self):
        n = 0
        for s in self.shapes:
            if s[0] == "box":
                n += 8
            elif s[0] == "sphere":
                n += 2 + (s[2] - 1) * s[3]
            elif s[0] == "pyramid":
                n += 5
            else:
                n += len(s[1])
        return n

    def world_slice(self, w):
        """The bodies of world w, in creation order (their local arena indices)."""
        return self.bodies[self.bodies["world"] == w]


def rng_for(config: int, seed: int | None = None):
    s = SEED_BASE + config if seed is None else seed
    return np.random.Generator(np.random.PCG64(s))


def random_quats(rng, n):
    """Shoemake's uniform random unit quaternions, returned (w, x, y, z)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    x, y = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    z, w = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    return np.stack([w, x, y, z], axis=1)


def box_mass(hx, hy, hz):
    m = RHO * 8.0 * hx * hy * hz
    return m, np.array([m / 3.0 * (hy * hy + hz * hz), m / 3.0 * (hx * hx + hz * hz), m / 3.0 * (hx * hx + hy * hy)])


def sphere_mass(r):
    m = RHO * 4.0 / 3.0 * math.pi * r ** 3
    i = 0.4 * m * r * r
    return m, np.array([i, i, i])


def hull_shape(rng, scale):
    """16 points uniform on a sphere of radius `scale`, triangulated by their convex hull."""
    from scipy.spatial import ConvexHull

    p = rng.normal(size=(16, 3))
    p = p / np.linalg.norm(p, axis=1, keepdims=True) * scale
    hull = ConvexHull(p)
    tris = hull.simplices.copy()
    # orient every triangle outward (signed-tetrahedron volume of mesh::volume, mesh.cpp:139-151)
    c = p.mean(axis=0)
    a, b, d = p[tris[:, 0]], p[tris[:, 1]], p[tris[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(b - a, d - a), a - c) < 0
    tris[flip, 1], tris[flip, 2] = tris[flip, 2], tris[flip, 1].copy()
    vol = float(abs(hull.volume))
    lo, hi = p.min(axis=0), p.max(axis=0)
    he = 0.5 * (hi - lo)
    m = RHO * vol
    I = np.array([m / 3.0 * (he[1] ** 2 + he[2] ** 2), m / 3.0 * (he[0] ** 2 + he[2] ** 2),
                  m / 3.0 * (he[0] ** 2 + he[1] ** 2)])
    # centre the vertices on their AABB so the body position is the shape's middle
    p = p - 0.5 * (hi + lo)
    return ("mesh", p, tris), m, I


def _records(n):
    r = np.zeros(n, dtype=BODY_DTYPE)
    r["quat"][:, 0] = 1.0
    r["restitution"] = 0.5
    r["friction"] = 0.5
    r["mass"] = 1.0
    r["inertia"][:, [0, 4, 8]] = 1.0
    return r


def _static(shape, pos, world=0):
    r = _records(1)
    r["type"] = 1
    r["shape"] = shape
    r["pos"] = pos
    r["world"] = world
    return r


def config1(n=1000, seed=None, ground=True, restitution=0.0, friction=0.5):
    rng = rng_for(1, seed)
    shapes, recs = [], []
    if ground:
        shapes.append(("box", 100.0, 0.5, 100.0))
        recs.append(_static(0, (0.0, -0.5, 0.0)))
    he = rng.uniform(0.1, 0.5, size=(n, 3))
    q = random_quats(rng, n)
    r = _records(n)
    for i in range(n):
        hx, hy, hz = he[i]
        shapes.append(("box", float(hx), float(hy), float(hz)))
        m, I = box_mass(hx, hy, hz)
        h = math.sqrt(hx * hx + hy * hy + hz * hz)
        r[i]["shape"] = len(shapes) - 1
        r[i]["mass"] = m
        r[i]["inertia"] = np.diag(I).reshape(-1)
        r[i]["pos"] = (rng.uniform(-10, 10), rng.uniform(h, 20 + h), rng.uniform(-10, 10))
        r[i]["quat"] = q[i]
    r["restitution"] = restitution
    r["friction"] = friction
    recs.append(r)
    return Scene("config1: %d boxes on a static ground, FP64, dt=1/120, 240 steps, 10 iterations" % n,
                 shapes, np.concatenate(recs), 1, dt=1 / 120, steps=240, iterations=10)


def _mixed_body(rng, kind, shapes, size_scale=1.0):
    if kind == 0:
        r = float(np.exp(rng.normal(math.log(0.3), 0.4))) * size_scale
        shapes.append(("sphere", r, 16, 32))
        m, I = sphere_mass(r)
        return m, I, r
    if kind == 1:
        he = rng.uniform(0.1, 0.6, 3) * size_scale
        shapes.append(("box", float(he[0]), float(he[1]), float(he[2])))
        m, I = box_mass(*he)
        return m, I, float(np.linalg.norm(he))
    sh, m, I = hull_shape(rng, float(rng.uniform(0.2, 0.6)) * size_scale)
    shapes.append(sh)
    return m, I, float(np.max(np.linalg.norm(sh[1], axis=1)))


def config2(n=100_000, seed=None, extent=200.0):
    rng = rng_for(2, seed)
    shapes = []
    r = _records(n)
    q = random_quats(rng, n)
    for i in range(n):
        m, I, _ = _mixed_body(rng, i % 3, shapes)
        r[i]["shape"] = len(shapes) - 1
        r[i]["mass"] = m
        r[i]["inertia"] = np.diag(I).reshape(-1)
    r["pos"] = rng.uniform(-extent / 2, extent / 2, size=(n, 3))
    r["vel"] = rng.normal(0.0, 1.0, size=(n, 3))
    r["quat"] = q
    return Scene("config2: %d mixed convex bodies in a %g m cube, dt=1/120, 120 steps" % (n, extent),
                 shapes, r, 1, gravity=(0.0, -9.81, 0.0), dt=1 / 120, steps=120, iterations=10)


def bin_statics(shapes, world, half=2.5, wall_h=6.0, thick=0.25):
    """Static floor + 4 walls of a (2*half) m square bin; shapes shared across worlds."""
    recs = []
    floor, wall_x, wall_z = 0, 1, 2
    recs.append(_static(floor, (0.0, -thick, 0.0), world))
    recs.append(_static(wall_x, (half + thick, wall_h, 0.0), world))
    recs.append(_static(wall_x, (-half - thick, wall_h, 0.0), world))
    recs.append(_static(wall_z, (0.0, wall_h, half + thick), world))
    recs.append(_static(wall_z, (0.0, wall_h, -half - thick), world))
    return recs


def config3(nworlds=4096, nmin=8, nmax=2048, seed=None, kinds=(0, 1, 2), half=2.5, pool_per_kind=64):
    """Batched piles. Bodies draw their meshes from a pool generated once (`pool_per_kind` shapes per
    kind), shared between bodies and worlds like the reference's shared_ptr meshes (object.h:61-65).
    Vectorised so that millions of bodies are generated in seconds."""
    rng = rng_for(3, seed)
    thick, wall_h = 0.25, 6.0
    shapes = [("box", half + thick, thick, half + thick), ("box", thick, wall_h, half + 2 * thick),
              ("box", half + 2 * thick, wall_h, thick)]
    pool_shape, pool_m, pool_I, pool_rad = [], [], [], []
    for k in kinds:
        for _ in range(pool_per_kind):
            m, I, rad = _mixed_body(rng, k, shapes, size_scale=0.5)
            pool_shape.append(len(shapes) - 1)
            pool_m.append(m)
            pool_I.append(I)
            pool_rad.append(rad)
    pool_shape, pool_m = np.array(pool_shape), np.array(pool_m)
    pool_I, pool_rad = np.array(pool_I), np.array(pool_rad)
    counts = np.round(np.exp(rng.uniform(math.log(nmin), math.log(nmax), nworlds))).astype(np.int64)
    total = int(counts.sum())
    world = np.repeat(np.arange(nworlds), counts)
    pick = rng.integers(0, len(pool_shape), total)
    rad = pool_rad[pick]
    lim = np.maximum(half - rad, 0.0)
    height = 0.5 + counts[world] * 0.02
    dyn = _records(total)
    dyn["world"] = world
    dyn["shape"] = pool_shape[pick]
    dyn["mass"] = pool_m[pick]
    dyn["inertia"][:, 0] = pool_I[pick, 0]
    dyn["inertia"][:, 4] = pool_I[pick, 1]
    dyn["inertia"][:, 8] = pool_I[pick, 2]
    dyn["pos"][:, 0] = rng.uniform(-1.0, 1.0, total) * lim
    dyn["pos"][:, 1] = rad + rng.uniform(0.0, 1.0, total) * height
    dyn["pos"][:, 2] = rng.uniform(-1.0, 1.0, total) * lim
    dyn["quat"] = random_quats(rng, total)
    dyn["restitution"] = 0.0
    # per world: its 5 statics first, then its dynamic bodies (creation order = local index)
    stat = np.concatenate([np.concatenate(bin_statics(shapes, 0, half, wall_h, thick))] * nworlds)
    stat["world"] = np.repeat(np.arange(nworlds), 5)
    recs = np.empty(total + 5 * nworlds, dtype=BODY_DTYPE)
    starts = np.concatenate([[0], np.cumsum(counts + 5)[:-1]])
    sidx = (starts[:, None] + np.arange(5)[None, :]).reshape(-1)
    didx = np.repeat(starts + 5, counts) + (np.arange(total) - np.repeat(np.cumsum(counts) - counts, counts))
    recs[sidx] = stat
    recs[didx] = dyn
    return Scene("config3: %d worlds, %d-%d bodies each (log-uniform), boxes/spheres/hulls in %g m bins, "
                 "dt=1/120, 240 steps" % (nworlds, nmin, nmax, 2 * half),
                 shapes, recs, nworlds, dt=1 / 120, steps=240, iterations=10)


def config5(n=1_000_000, seed=None, half=10.0, nradii=32, spacing=0.125):
    """Spheres (r ~ lognormal(ln 0.05, 0.3)) poured into a (2*half) m square open box: they start
    on a jittered cubic lattice of `spacing` just above the floor, filling the box's footprint layer
    by layer, and fall into a dense pile in the first ~100 steps (about 6 contacts per body once
    settled). Radii come from a pool of `nradii` lognormal radii so the UV meshes are shared.
    config5(n=10_000, half=1.0) is a sub-region replica of the full pile: the same lattice, depth
    and radii on a 2 x 2 m footprint."""
    rng = rng_for(5, seed)
    thick, wall_h = 0.25, 4.0
    shapes = [("box", half + thick, thick, half + thick), ("box", thick, wall_h, half + 2 * thick),
              ("box", half + 2 * thick, wall_h, thick)]
    radii = np.exp(rng.normal(math.log(0.05), 0.3, nradii))
    for rr in radii:
        shapes.append(("sphere", float(rr), 16, 32))
    recs = bin_statics(shapes, 0, half, wall_h, thick)
    r = _records(n)
    pick = rng.integers(0, nradii, n)
    rad = radii[pick]
    m = RHO * 4.0 / 3.0 * math.pi * rad ** 3
    r["shape"] = 3 + pick
    r["mass"] = m
    r["inertia"][:, 0] = r["inertia"][:, 4] = r["inertia"][:, 8] = 0.4 * m * rad * rad
    side = int((2.0 * half - 2.0 * 0.1) // spacing)  # lattice sites per row, 0.1 m clear of the walls
    k = np.arange(n)
    layer, cell = k // (side * side), k % (side * side)
    jit = rng.uniform(-0.01, 0.01, size=(n, 2))
    r["pos"][:, 0] = -half + 0.1 + (cell % side + 0.5) * spacing + jit[:, 0]
    r["pos"][:, 2] = -half + 0.1 + (cell // side + 0.5) * spacing + jit[:, 1]
    r["pos"][:, 1] = 0.5 * spacing + layer * spacing
    r["quat"] = random_quats(rng, n)
    r["restitution"] = 0.0
    recs.append(r)
    return Scene("config5: %d spheres poured into a %g x %g m box, dt=1/240, 480 steps, 20 iterations"
                 % (n, 2 * half, 2 * half), shapes, np.concatenate(recs), 1, dt=1 / 240, steps=480, iterations=20)


def resting_stacks(rows=10, cols=10, height=3, spacing=3.0, gap=0.01, seed=None):
    """Separated stacks of boxes on a ground box: each stack is `height` boxes with vertical axes,
    each turned about the vertical by a random angle and placed `gap` m above the one below, so
    the boxes drop flat and come to rest. The stacks are far apart (no pair between stacks), and
    nothing tips over, so the trajectory is not chaotic: a perturbation stays of its own size."""
    rng = rng_for(11, seed)
    shapes = [("box", 0.6 * spacing * max(rows, cols), 0.5, 0.6 * spacing * max(rows, cols))]
    recs = [_static(0, (0.0, -0.5, 0.0))]
    n = rows * cols * height
    r = _records(n)
    k = 0
    for i in range(rows):
        for j in range(cols):
            x, z = (i - (rows - 1) / 2) * spacing, (j - (cols - 1) / 2) * spacing
            y = 0.0
            for lvl in range(height):
                hx, hz = (0.5 - 0.08 * lvl) * rng.uniform(0.8, 1.0, 2)
                hy = rng.uniform(0.15, 0.3)
                shapes.append(("box", float(hx), float(hy), float(hz)))
                m, I = box_mass(hx, hy, hz)
                ang = rng.uniform(-0.3, 0.3)
                r[k]["shape"] = len(shapes) - 1
                r[k]["mass"] = m
                r[k]["inertia"] = np.diag(I).reshape(-1)
                r[k]["pos"] = (x, y + gap + hy, z)
                r[k]["quat"] = (math.cos(ang / 2), 0.0, math.sin(ang / 2), 0.0)
                y += gap + 2 * hy
                k += 1
    r["restitution"] = 0.0
    r["friction"] = 0.5
    recs.append(r)
    return Scene("resting stacks: %dx%d stacks of %d boxes on a ground box, dt=1/120" % (rows, cols, height),
                 shapes, np.concatenate(recs), 1, dt=1 / 120, steps=240, iterations=10)


def small_pile(n=60, seed=7, extent=3.0, kinds=(1,), ground=True, restitution=0.0):
    """A small pile for parity tests: bodies close together above a ground box."""
    rng = rng_for(9, seed)
    shapes, recs = [], []
    if ground:
        shapes.append(("box", 20.0, 0.5, 20.0))
        recs.append(_static(0, (0.0, -0.5, 0.0)))
    r = _records(n)
    q = random_quats(rng, n)
    for i in range(n):
        m, I, rad = _mixed_body(rng, kinds[i % len(kinds)], shapes, size_scale=0.8)
        r[i]["shape"] = len(shapes) - 1
        r[i]["mass"] = m
        r[i]["inertia"] = np.diag(I).reshape(-1)
        r[i]["pos"] = (rng.uniform(-extent, extent), rng.uniform(rad, rad + 4.0), rng.uniform(-extent, extent))
        r[i]["quat"] = q[i]
    r["restitution"] = restitution
    recs.append(r)
    return Scene("small pile", shapes, np.concatenate(recs), 1)


def load(world, scene: Scene, shape_offset_map=None):
    """Create the scene's shapes and bodies in a physkit_gb300.World; returns body handles."""
    ids = []
    for s in scene.shapes:
        if s[0] == "box":
            ids.append(world.mesh_box(*s[1:4]))
        elif s[0] == "sphere":
            ids.append(world.mesh_sphere(s[1], s[2], s[3]))
        elif s[0] == "pyramid":
            ids.append(world.mesh_pyramid(s[1], s[2]))
        else:
            ids.append(world.mesh_make(s[1], s[2]))
    rec = scene.bodies.copy()
    rec["shape"] = np.asarray(ids, dtype=np.int32)[rec["shape"]]
    return world.create_rigids(rec)


def make_world(scene: Scene, precision="f64", pair_factor=8, iterations=None, max_bodies_per_world=0,
               contact_factor=0):
    from .world import World, world_desc

    nb = len(scene.bodies)
    per_world = max_bodies_per_world or (nb if scene.nworlds == 1 else
                                         int(np.bincount(scene.bodies["world"]).max()))
    d = (world_desc.make().with_gravity(scene.gravity)
         .with_solver_iterations(iterations if iterations is not None else scene.iterations)
         .with_precision(precision)
         .with_capacity(max_bodies=nb, max_pairs=max(pair_factor * nb, 1024), max_worlds=scene.nworlds,
                        max_bodies_per_world=per_world, max_shape_vertices=scene.vertex_count() + 16,
                        max_shapes=len(scene.shapes) + 4,
                        max_contact_pairs=int(contact_factor * nb) if contact_factor else 0))
    w = World(d)
    handles = load(w, scene)
    return w, handles


def load_json(path_or_text, name=None) -> Scene:
    """A scene in the reference's demo JSON format (tests/helper/src/graphics.cpp:20-140):
    {"gravity": [3], "solver_iterations": n, "objects": [{"pos": [3], "vel": [3],
    "orientation": [w, x, y, z], "angular_velocity": [3], "inertia_tensor": [Ixx, Iyy, Izz],
    "type": "dynam" | "stat", "mesh": {...}, "mass": m, "restitution": e, "friction": mu}]}, with
    the reference's defaults (vel, angular velocity 0, orientation identity, inertia (1, 1, 1),
    dynamic, box half extents 0.5, restitution 0.5, friction 0.5, sphere 16 stacks x 32 sectors).
    Mesh fields are single precision in the reference (graphics.cpp:24-41), so they are rounded to
    float32 here too. A pyramid gets `height` as its base half size and `base_size` as its height,
    the order in which the reference's loader passes them to mesh::pyramid(base_half, height)
    (graphics.cpp:101-102, mesh.h:236). Camera and window fields are ignored (no rendering).
    Identical meshes are shared, as the reference keys them by their JSON text."""
    import json
    import os

    if isinstance(path_or_text, str) and os.path.exists(path_or_text):
        with open(path_or_text) as f:
            cfg = json.load(f)
        name = name or os.path.basename(path_or_text)
    else:
        cfg = json.loads(path_or_text)
    f32 = lambda x: float(np.float32(x))
    gravity = tuple(float(v) for v in cfg.get("gravity", (0.0, -9.81, 0.0)))
    iterations = int(cfg.get("solver_iterations", 10))
    shapes, keys, recs = [], {}, []
    for o in cfg.get("objects", []):
        mesh = o.get("mesh", {"name": "box", "half_extents": [0.5, 0.5, 0.5]})
        kind = mesh.get("name")
        if kind is None:  # a variant is also recognised by its fields
            kind = "box" if "half_extents" in mesh else ("pyramid" if "height" in mesh else "sphere")
        if kind == "box":
            shape = ("box",) + tuple(f32(v) for v in mesh["half_extents"])
        elif kind == "pyramid":
            shape = ("pyramid", f32(mesh["height"]), f32(mesh["base_size"]))
        elif kind == "sphere":
            shape = ("sphere", f32(mesh["radius"]), int(mesh.get("stacks", 16)), int(mesh.get("sectors", 32)))
        else:
            raise ValueError(f"unknown mesh kind {kind!r}")
        if shape not in keys:
            keys[shape] = len(shapes)
            shapes.append(shape)
        r = np.zeros((), dtype=BODY_DTYPE)
        r["type"] = 1 if o.get("type", "dynam") == "stat" else 0
        r["shape"] = keys[shape]
        r["pos"] = o["pos"]
        r["vel"] = o.get("vel", (0.0, 0.0, 0.0))
        r["quat"] = o.get("orientation", (1.0, 0.0, 0.0, 0.0))
        r["ang_vel"] = o.get("angular_velocity", (0.0, 0.0, 0.0))
        it = o.get("inertia_tensor", (1.0, 1.0, 1.0))
        r["inertia"] = (it[0], 0, 0, 0, it[1], 0, 0, 0, it[2])
        r["mass"] = float(o["mass"])
        r["restitution"] = float(o.get("restitution", 0.5))
        r["friction"] = float(o.get("friction", 0.5))
        recs.append(r)
    bodies = np.array(recs, dtype=BODY_DTYPE) if recs else np.zeros(0, dtype=BODY_DTYPE)
    return Scene(name or "json scene", shapes, bodies, 1, gravity, iterations=iterations)
