"""Serving form: continuous batching of world-step requests over the C ABI server (pk_batch_*).

The server (include/physkit_gb300.h, pk_batch_*) keeps a device-resident pool of world slots whose
size is set by device memory at creation, and its loop runs in C++: admission into a free slot
(refused while the pool is full), one request per step of one world, batched steps enqueued behind
the ones in flight without waiting for the GPU, and completions polled from CUDA events. This
module adds the request bookkeeping of a caller (arrival times, world lifetimes) and a Poisson
load driver. Requests are either "open a world of n bodies that lives for L steps" or "advance
world w by one step"; a request that arrives while steps are on the device joins the next batched
step that is enqueued.

A world's results do not depend on the mix: a world sits out every batched step that serves none
of its requests, with its pairs and manifolds untouched, and pair keys and the per-world solver use
world-local indices only, so a world stepped k times in any mix ends in the same state as the same
world stepped k times alone.
"""
from __future__ import annotations

import collections
import ctypes as C
import dataclasses
import math
import time

import numpy as np

from . import scenes
from .world import (BATCH_STEPPED, BODY_DTYPE, PK_ERR_CAPACITY, PRECISION, BatchDescC, BatchEventC, BatchInfoC,
                    World, _check, _ptr, lib)


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
    """A caller of the C ABI server: request tags index the arrival times kept here."""

    def __init__(self, max_worlds=1024, max_bodies=2_000_000, max_bodies_per_world=4101, precision="f32",
                 pair_factor=6, contact_factor=2, iterations=10, dt=1.0 / 120.0, seed=4, pipeline_depth=1,
                 memory_fraction=0.5, tuning=None):
        self.L = lib()
        d = BatchDescC()
        self.L.pk_batch_desc_init(C.byref(d))
        d.dt = dt
        d.solver_iterations = iterations
        d.precision = PRECISION[precision]
        d.max_worlds = max_worlds
        d.max_bodies_per_world = max_bodies_per_world
        d.max_bodies = max_bodies  # 0: sized from free device memory (memory_fraction)
        d.memory_fraction = memory_fraction
        d.pair_factor = pair_factor
        d.contact_factor = contact_factor
        d.max_shapes = 256
        d.max_shape_vertices = 4096
        d.pipeline_depth = pipeline_depth
        h = C.c_void_p()
        _check(self.L.pk_batch_create(C.byref(d), C.byref(h)), "pk_batch_create")
        self.b = h
        self.world = World(_borrow=self.L.pk_batch_world(self.b))
        # latency first: the largest worlds set a step's length, so they get the widest solver CTA
        self.world.set_tuning(tuning or {"solve_threads": 128, "small_world": 1024, "narrow_grid": 2,
                                         "traverse_threads": 128, "big_threads": 512})
        self.dt = dt
        self.templates = BoxPileTemplates(self.world, seed)
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self.live: dict[int, LiveWorld] = {}
        self.waiting = collections.deque()      # (req_id, nbodies, lifetime, t_arrival, records or None)
        self.arrival = []                       # request tag -> arrival time
        self.latency = []                       # seconds, completed step requests
        self.body_steps = 0
        self.admit_wait = []
        self.events = (BatchEventC * 4096)()
        self.max_worlds = max_worlds

    def stats(self):
        st = BatchInfoC()
        _check(self.L.pk_batch_stats(self.b, C.byref(st)), "pk_batch_stats")
        return {f: getattr(st, f) for f, _ in BatchInfoC._fields_}

    @property
    def steps(self):
        return self.stats()["steps"]

    # requests -----------------------------------------------------------------------------------
    def open(self, req_id, nbodies, lifetime, t_arrival, records=None):
        self.waiting.append((req_id, int(nbodies), int(lifetime), t_arrival, records))

    def advance(self, wid, t_arrival):
        lw = self.live.get(wid)
        if lw is None or lw.steps_left <= len(lw.pending):
            return False
        tag = len(self.arrival)
        self.arrival.append(t_arrival)
        _check(self.L.pk_batch_request(self.b, int(wid), tag), "pk_batch_request")
        lw.pending.append(tag)
        return True

    # loop ---------------------------------------------------------------------------------------
    def admit(self, now):
        admitted = []
        wid = C.c_int32()
        while self.waiting:
            req_id, n, life, t_arr, rec = self.waiting[0]
            if rec is None:  # drawn once: a request that waits for room keeps its bodies
                rec = self.templates.records(self.rng, n, 0)
                self.waiting[0] = (req_id, n, life, t_arr, rec)
            rec = np.ascontiguousarray(rec, dtype=BODY_DTYPE)
            hs = np.zeros(len(rec), dtype=np.uint64)
            rc = self.L.pk_batch_admit(self.b, rec.ctypes.data, len(rec), _ptr(hs, C.c_uint64), C.byref(wid))
            if rc == PK_ERR_CAPACITY:
                break  # no free slot or no room in the pool: wait for a retirement
            _check(rc, "pk_batch_admit")
            self.waiting.popleft()
            self.live[wid.value] = LiveWorld(wid.value, n, life, collections.deque(), (hs & 0xFFFFFFFF).astype(np.int64))
            self.admit_wait.append(now - t_arr)
            admitted.append((req_id, wid.value))
        return admitted

    def launch(self):
        """Enqueue one batched step of every world with a request not yet in flight."""
        n = C.c_int32()
        _check(self.L.pk_batch_step_async(self.b, C.byref(n)), "pk_batch_step_async")
        return n.value

    def poll(self, wait=False):
        """Account the completed requests; returns how many completed."""
        done = 0
        while True:
            n = C.c_int32()
            _check(self.L.pk_batch_poll(self.b, self.events, len(self.events), C.byref(n), int(wait)), "pk_batch_poll")
            wait = False
            t_done = time.perf_counter()
            for i in range(n.value):
                e = self.events[i]
                if e.kind != BATCH_STEPPED:
                    continue
                self.latency.append(t_done - self.arrival[e.tag])
                lw = self.live[e.world]
                lw.pending.popleft()
                lw.steps_left -= 1
                lw.steps_done += 1
                self.body_steps += lw.nbodies
                done += 1
                if lw.steps_left <= 0:
                    self.live.pop(e.world)
                    _check(self.L.pk_batch_retire(self.b, e.world), "pk_batch_retire")
            if n.value < len(self.events):
                return done

    def step_once(self):
        """One batched step over every world with a pending request, waited for."""
        served = self.launch()
        if served:
            self.poll(wait=True)
        return served

    def world_state(self, wid):
        """Body states (14 doubles each) of a live world in creation order."""
        n = C.c_int32()
        cap = self.live[wid].slots.size
        out = np.zeros((max(cap, 1), 14))
        _check(self.L.pk_batch_read_world(self.b, int(wid), _ptr(out, C.c_double), cap, C.byref(n)),
               "pk_batch_read_world")
        return out[: n.value]

    def close(self):
        if self.b:
            self.world.close()
            self.L.pk_batch_destroy(self.b)
            self.b = None


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


class LaneServer:
    """Worlds split by size over independent servers (lanes), each with its own pool, stream and
    step cadence: a request for a small world then waits only for the small worlds' steps, which
    the GPU runs beside the large ones. A lane may have several servers (replicas), its worlds
    dealt to them in turn, so that a request for one large world does not wait for the step of
    another. World ids are (server << 20) | slot."""

    def __init__(self, lanes, precision="f32", pipeline_depth=1, **kw):
        # lanes: (largest world in bodies, world slots, body pool[, servers]) per lane, ascending
        self.bounds = [ln[0] for ln in lanes]
        self.lanes, self.servers_of = [], []
        for ln in lanes:
            b, mw, mb = ln[:3]
            reps = ln[3] if len(ln) > 3 else 1
            self.servers_of.append(list(range(len(self.lanes), len(self.lanes) + reps)))
            self.lanes += [StepServer(max_worlds=max(8, mw // reps), max_bodies=max(2 * b, mb // reps),
                                      max_bodies_per_world=b + 5, precision=precision,
                                      pipeline_depth=pipeline_depth, **kw) for _ in range(reps)]
        self.next = [0] * len(lanes)

    def lane_of(self, n):
        for k, b in enumerate(self.bounds):
            if n <= b:
                return k
        return len(self.bounds) - 1

    def lane_latency(self, k):
        return [x for s in self.servers_of[k] for x in self.lanes[s].latency]

    @property
    def live(self):
        return {(k << 20) | w: lw for k, srv in enumerate(self.lanes) for w, lw in srv.live.items()}

    @property
    def latency(self):
        return [x for srv in self.lanes for x in srv.latency]

    @property
    def admit_wait(self):
        return [x for srv in self.lanes for x in srv.admit_wait]

    @property
    def body_steps(self):
        return sum(srv.body_steps for srv in self.lanes)

    def open(self, req_id, nbodies, lifetime, t_arrival, records=None):
        k = self.lane_of(nbodies)
        srv = self.servers_of[k][self.next[k] % len(self.servers_of[k])]
        self.next[k] += 1
        self.lanes[srv].open(req_id, nbodies, lifetime, t_arrival, records)

    def advance(self, gid, t_arrival):
        return self.lanes[gid >> 20].advance(gid & 0xFFFFF, t_arrival)

    def admit(self, now):
        return [(r, (k << 20) | w) for k, srv in enumerate(self.lanes) for r, w in srv.admit(now)]

    def launch(self):
        return sum(srv.launch() for srv in self.lanes)

    def poll(self, wait=False):
        done = sum(srv.poll() for srv in self.lanes)
        while wait and done == 0 and any(srv.stats()["steps_in_flight"] for srv in self.lanes):
            done = sum(srv.poll() for srv in self.lanes)  # spin: each lane completes on its own
        return done

    def stats(self):
        st = [srv.stats() for srv in self.lanes]
        return {k: sum(x[k] for x in st) for k in st[0]}

    def close(self):
        for srv in self.lanes:
            srv.close()


def lane_layout(lanes, max_worlds, max_bodies, nmax=4096, lane_servers=1, nmin=16):
    """(largest world in bodies, world slots, body pool, servers) per size lane, ascending. Lanes
    are finer at the top (the largest worlds set a step's length); world slots follow each lane's
    share of worlds under the log-uniform size law, bodies its share of bodies; lanes of worlds
    above 1,024 bodies, whose steps take about a millisecond, get `lane_servers` servers so that a
    request rarely waits for another large world's step."""
    bounds = {2: [1024, nmax], 3: [512, 2048, nmax], 4: [256, 1024, 2048, nmax]}[lanes]
    edges = [nmin] + bounds
    wshare = [math.log(edges[k + 1] / edges[k]) / math.log(nmax / nmin) for k in range(lanes)]
    bshare = [(edges[k + 1] - edges[k]) / (nmax - nmin) for k in range(lanes)]
    reps = [1 if b <= 1024 else lane_servers for b in bounds]
    return [(b, max(16, int(max_worlds * ws)), max(4 * b, int(max_bodies * bs)), r)
            for b, ws, bs, r in zip(bounds, wshare, bshare, reps)]


def run_served(rate, duration=4.0, warm_live=128, precision="f32", max_worlds=1024, max_bodies=1_500_000,
               nmax=4096, seed=5, pipeline_depth=1, lanes=2, lane_servers=1):
    """Drive the server with a Poisson request stream in real time; returns the latency report.
    The host loop takes arrivals, admits opens, enqueues a batched step whenever a lane's pipeline
    has room and polls completions; it waits on the GPU only when it has nothing else to do. With
    lanes > 1, worlds are served by separate pools by size (2 lanes: up to 1,024 bodies and above;
    3: 512 / 2,048 / 4,096; 4: 256 / 1,024 / 2,048 / 4,096), each with its own stream, and the
    lanes of worlds above 1,024 bodies by `lane_servers` servers each."""
    if lanes > 1:
        srv = LaneServer(lane_layout(lanes, max_worlds, max_bodies, nmax, lane_servers), precision=precision,
                         pipeline_depth=pipeline_depth)
    else:
        srv = StepServer(max_worlds=max_worlds, max_bodies=max_bodies, precision=precision,
                         pipeline_depth=pipeline_depth)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    # start from a populated pool so the measured window is in steady state
    for i in range(warm_live):
        n = int(round(math.exp(rng.uniform(math.log(16), math.log(nmax)))))
        srv.open(-1 - i, n, int(rng.integers(60, 601)), time.perf_counter())
    srv.admit(time.perf_counter())
    srv.poll()
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
        srv.launch()
        srv.poll()
        st = srv.stats()
        if i >= nreq and st["pending_requests"] == 0 and st["steps_in_flight"] == 0:
            break
        # one server: with its pipeline full there is nothing to launch until a step ends, so wait
        # for it; with several lanes the others may still launch, so keep polling
        if lanes <= 1 and st["steps_in_flight"] > 0 and (st["steps_in_flight"] >= pipeline_depth or i >= nreq):
            srv.poll(wait=True)
        elif st["steps_in_flight"] == 0 and i < nreq:
            time.sleep(max(0.0, min(1e-4, t[i] - (time.perf_counter() - t0))))
    wall = time.perf_counter() - t0
    lat = np.array(srv.latency) * 1e3
    st = srv.stats()
    aw = srv.admit_wait
    rep = {"rate_req_s": rate, "duration_s": duration, "requests": int(nreq), "completed_steps": int(len(lat)),
           "dropped": dropped, "batched_steps": st["steps"],
           "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
           "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
           "p999_ms": float(np.percentile(lat, 99.9)) if len(lat) else None,
           "body_steps_per_s": srv.body_steps / wall, "live_worlds_end": len(srv.live),
           "admission_wait_p99_ms": float(np.percentile(np.array(aw) * 1e3, 99)) if aw else None,
           "pool_bodies": st["pool_bodies"], "pipeline_depth": pipeline_depth, "lanes": lanes,
           "graph_captures": st["graph_captures"],
           "lane_p99_ms": ([float(np.percentile(np.array(srv.lane_latency(k)) * 1e3, 99))
                            if srv.lane_latency(k) else None for k in range(lanes)] if lanes > 1 else None),
           "lane_servers": lane_servers,
           "lane_bounds": srv.bounds if lanes > 1 else None,
           "loop": "C ABI server (pk_batch_*): admission, batching and completion in C++, one server per size "
                   "lane; Poisson arrivals and latency accounting in Python"}
    srv.close()
    return rep
