"""Serving form: continuous batching of world-step requests on one device-resident pool.

A pool is one device world object with `max_worlds` world slots and a fixed body capacity that
was reserved in device memory at creation (admission is by that memory: a world is admitted when a
world slot and room for its bodies are free). Requests are either "open a world of n bodies that
lives for L steps" or "advance world w by one step". Each iteration of the loop

  1. admits waiting opens while a slot and body capacity are free (FIFO),
  2. marks every world with at least one pending step request active, the rest inactive,
  3. runs one batched step on the device for all active worlds at once,
  4. completes the oldest pending request of each stepped world, and retires worlds whose
     lifetime is used up (their slot and bodies become free for the next admission).

Requests that arrive while a step is on the device join the next iteration. A world's results do
not depend on the mix: inactive worlds keep their pairs and manifolds untouched, pair keys and the
per-world solver use world-local indices only, so a world stepped k times in any mix ends in the
same state as the same world stepped k times alone.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from . import scenes
from .world import BODY_DTYPE, World, world_desc


@dataclasses.dataclass
class LiveWorld:
    wid: int
    nbodies: int
    steps_left: int
    pending: collections.deque
    slots: np.ndarray = None  # device slots of the world's bodies, creation order
    steps_done: int = 0


class BoxPileTemplates:
    """Box piles like config 1 (half-extents U[0.1,0.5] scaled to fit a 5 m bin), drawn from a
    shared pool of box meshes so admission uploads only body records."""

    def __init__(self, world: World, seed=4, nshapes=128, half=2.5):
        rng = scenes.rng_for(4, seed)
        self.half = half
        thick, wall_h = 0.25, 6.0
        self.static_shapes = [world.mesh_box(half + thick, thick, half + thick),
                              world.mesh_box(thick, wall_h, half + 2 * thick),
                              world.mesh_box(half + 2 * thick, wall_h, thick)]
        self.he = rng.uniform(0.1, 0.5, size=(nshapes, 3)) * 0.5
        self.shapes = [world.mesh_box(*h) for h in self.he]
        self.mass = np.array([scenes.box_mass(*h)[0] for h in self.he])
        self.inertia = np.array([scenes.box_mass(*h)[1] for h in self.he])
        self.rad = np.linalg.norm(self.he, axis=1)
        self.thick, self.wall_h = thick, wall_h

    def records(self, rng, n, wid):
        stat = np.zeros(5, dtype=BODY_DTYPE)
        stat["type"] = 1
        stat["quat"][:, 0] = 1.0
        stat["shape"] = [self.static_shapes[0], self.static_shapes[1], self.static_shapes[1],
                         self.static_shapes[2], self.static_shapes[2]]
        h, t, wh = self.half, self.thick, self.wall_h
        stat["pos"] = [(0, -t, 0), (h + t, wh, 0), (-h - t, wh, 0), (0, wh, h + t), (0, wh, -h - t)]
        stat["inertia"][:, [0, 4, 8]] = 1.0
        dyn = np.zeros(n, dtype=BODY_DTYPE)
        k = rng.integers(0, len(self.shapes), n)
        dyn["shape"] = np.asarray(self.shapes)[k]
        dyn["mass"] = self.mass[k]
        dyn["inertia"][:, 0] = self.inertia[k, 0]
        dyn["inertia"][:, 4] = self.inertia[k, 1]
        dyn["inertia"][:, 8] = self.inertia[k, 2]
        lim = np.maximum(self.half - self.rad[k], 0.0)
        dyn["pos"][:, 0] = rng.uniform(-1, 1, n) * lim
        dyn["pos"][:, 1] = self.rad[k] + rng.uniform(0, 1, n) * (0.5 + n * 0.02)
        dyn["pos"][:, 2] = rng.uniform(-1, 1, n) * lim
        dyn["quat"] = scenes.random_quats(rng, n)
        dyn["restitution"] = 0.0
        dyn["friction"] = 0.5
        rec = np.concatenate([stat, dyn])
        rec["world"] = wid
        return rec


class StepServer:
    def __init__(self, max_worlds=1024, max_bodies=2_000_000, max_bodies_per_world=4101, precision="f32",
                 pair_factor=6, iterations=10, dt=1.0 / 120.0, seed=4):
        d = (world_desc.make().with_precision(precision).with_solver_iterations(iterations)
             .with_capacity(max_bodies=max_bodies, max_pairs=pair_factor * max_bodies, max_worlds=max_worlds,
                            max_bodies_per_world=max_bodies_per_world, max_shape_vertices=4096, max_shapes=256))
        self.world = World(d)
        # latency first: the largest worlds set a step's length, so they get the widest solver CTA
        self.world.set_tuning({"solve_threads": 128, "small_world": 1024, "narrow_grid": 2, "traverse_threads": 128,
                               "big_threads": 512})
        self.dt = dt
        self.templates = BoxPileTemplates(self.world, seed)
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self.max_worlds, self.max_bodies = max_worlds, max_bodies
        self.free_ids = collections.deque(range(max_worlds))
        self.bodies_in_use = 0
        self.live: dict[int, LiveWorld] = {}
        self.waiting = collections.deque()      # (req_id, nbodies, lifetime, t_arrival, records or None)
        self.mask = np.zeros(max_worlds, dtype=np.uint8)
        self.latency = []                       # seconds, completed step requests
        self.body_steps = 0
        self.steps = 0
        self.admit_wait = []
        self.world.set_active_mask(self.mask)

    # requests -----------------------------------------------------------------------------------
    def open(self, req_id, nbodies, lifetime, t_arrival, records=None):
        self.waiting.append((req_id, int(nbodies), int(lifetime), t_arrival, records))

    def advance(self, wid, t_arrival):
        lw = self.live.get(wid)
        if lw is None:
            return False
        lw.pending.append(t_arrival)
        return True

    # loop ---------------------------------------------------------------------------------------
    def admit(self, now):
        admitted = []
        while self.waiting and self.free_ids:
            req_id, n, life, t_arr, rec = self.waiting[0]
            if self.bodies_in_use + n + 5 > self.max_bodies:
                break  # device memory reserved for bodies is full: wait for a retirement
            self.waiting.popleft()
            wid = self.free_ids.popleft()
            if rec is None:
                rec = self.templates.records(self.rng, n, wid)
            else:
                rec = rec.copy()
                rec["world"] = wid
            handles = self.world.create_rigids(rec)
            self.bodies_in_use += len(rec)
            self.live[wid] = LiveWorld(wid, n, life, collections.deque(), (handles & 0xFFFFFFFF).astype(np.int64))
            self.admit_wait.append(now - t_arr)
            admitted.append((req_id, wid))
        return admitted

    def step_once(self):
        """One batched device step over every world with a pending step request."""
        batch = [lw for lw in self.live.values() if lw.pending]
        if not batch:
            return 0
        self.mask[:] = 0
        for lw in batch:
            self.mask[lw.wid] = 1
        self.world.set_active_mask(self.mask)
        self.world.step_async(self.dt)
        self.world.synchronize()
        t_done = time.perf_counter()
        for lw in batch:
            t_arr = lw.pending.popleft()
            self.latency.append(t_done - t_arr)
            lw.steps_left -= 1
            lw.steps_done += 1
            self.body_steps += lw.nbodies
            if lw.steps_left <= 0:
                self.retire(lw.wid)
        self.steps += 1
        return len(batch)

    def retire(self, wid):
        lw = self.live.pop(wid)
        self.world.clear_world(wid)
        self.bodies_in_use -= lw.nbodies + 5
        self.free_ids.append(wid)

    def world_state(self, wid):
        """Body states (14 doubles each) of a live world in creation order."""
        return self.world.bodies()[self.live[wid].slots]

    def close(self):
        self.world.close()


def poisson_load(rate, duration, target_live=256, nmin=16, nmax=4096, life=(60, 600), seed=5):
    """Arrival schedule: Poisson requests at `rate`/s for `duration` s. A request opens a world
    (n ~ log-uniform[nmin, nmax], lifetime ~ U[life]) with the probability that keeps about
    `target_live` worlds alive, otherwise it advances a uniformly chosen live world."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = rng.poisson(rate * duration)
    t = np.sort(rng.uniform(0.0, duration, n))
    mean_life = 0.5 * (life[0] + life[1])
    p_open = 1.0 / (mean_life + 1.0)
    kind = rng.random(n) < p_open
    sizes = np.round(np.exp(rng.uniform(math.log(nmin), math.log(nmax), n))).astype(int)
    lifes = rng.integers(life[0], life[1] + 1, n)
    pick = rng.random(n)
    return t, kind, sizes, lifes, pick, target_live


def run_served(rate, duration=4.0, warm_live=128, precision="f32", max_worlds=1024, max_bodies=1_500_000,
               nmax=4096, seed=5):
    """Drive a StepServer with a Poisson request stream in real time; returns the latency report."""
    srv = StepServer(max_worlds=max_worlds, max_bodies=max_bodies, precision=precision)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    # start from a populated pool so the measured window is in steady state
    for i in range(warm_live):
        n = int(round(math.exp(rng.uniform(math.log(16), math.log(nmax)))))
        srv.open(-1 - i, n, int(rng.integers(60, 601)), time.perf_counter())
    srv.admit(time.perf_counter())
    t, kind, sizes, lifes, pick, _ = poisson_load(rate, duration, nmax=nmax, seed=seed)
    t0 = time.perf_counter()
    i, nreq = 0, len(t)
    dropped = 0
    while True:
        now = time.perf_counter() - t0
        while i < nreq and t[i] <= now:
            arrival = t0 + t[i]
            if kind[i] or not srv.live:
                srv.open(i, int(sizes[i]), int(lifes[i]), arrival)
            else:
                ids = list(srv.live.keys())
                wid = ids[int(pick[i] * len(ids)) % len(ids)]
                if not srv.advance(wid, arrival):
                    dropped += 1
            i += 1
        srv.admit(time.perf_counter())
        served = srv.step_once()
        if i >= nreq and not any(lw.pending for lw in srv.live.values()):
            break
        if served == 0 and i < nreq:
            time.sleep(max(0.0, min(1e-4, t[i] - (time.perf_counter() - t0))))
    wall = time.perf_counter() - t0
    lat = np.array(srv.latency) * 1e3
    rep = {"rate_req_s": rate, "duration_s": duration, "requests": int(nreq), "completed_steps": int(len(lat)),
           "dropped": dropped, "batched_steps": srv.steps,
           "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
           "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
           "p999_ms": float(np.percentile(lat, 99.9)) if len(lat) else None,
           "body_steps_per_s": srv.body_steps / wall, "live_worlds_end": len(srv.live),
           "admission_wait_p99_ms": float(np.percentile(np.array(srv.admit_wait) * 1e3, 99)) if srv.admit_wait else None}
    srv.close()
    return rep
