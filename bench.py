"""World-step throughput benchmark (body-steps/s) on the batched-worlds workload.

Workload (headline): 4,096 independent worlds with log-uniform body counts in [8, 2048] (~1.5 M
dynamic bodies: UV spheres, boxes and 16-point hulls dropped into 5 m walled bins), dt = 1/120,
10 solver iterations, in the FP64 parity form: the reference's own precision (it computes in
double throughout), bit-identical to the FP64 oracle. One step = one world-step of every world.
Inputs are synthetic (seeded generator in physkit_gb300/scenes.py).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision f64|f32]

Every timed window is the same: W warm-up steps from the initial state, then K timed steps.
value: dynamic bodies x K / device time of the K steps (CUDA events on the world's stream, no
stage instrumentation, max over ranks). e2e: the same window on a fresh copy of the batch through
the C ABI, pk_world_step + pk_world_read_bodies of every body into pinned host memory each step
(wall clock). stage_ms_per_step and the roofline come from a third copy stepped with per-stage
CUDA events over the same window. precision_form: the FP32 form on the same window. The
reference arm times the FP64 CPU restatement of the reference step (oracle/) on the whole batch
and the same window, with one process per host core. Under torchrun each rank steps its own
independent batch (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "world-step throughput, batched worlds (body-steps/s)"
UNIT = "body-steps/s"

# Algorithmic bytes per unit (FP32 SoA compulsory traffic; each datum once per kernel pass).
BYTES = {
    "integrate_vel": ("body", 152.0),
    "morton_sort": ("body", 64.0),
    "lbvh_build_refit": ("body", 90.0),
    "traverse": ("body", 56.0),
    "pair_sort": ("pair", 16.0 * 6),
    "narrow": ("pair", 504.0),
    "contact_setup": ("contact", 150.0),
    "solve": ("contact_iter", 250.0),
    "integrate_pos": ("body", 116.0),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--worlds", type=int, default=4096)
    ap.add_argument("--nmin", type=int, default=8)
    ap.add_argument("--nmax", type=int, default=2048)
    ap.add_argument("--precision", default="f64", choices=["f32", "f64"])
    ap.add_argument("--cpu-sample-worlds", type=int, default=24)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-precision-form", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-raycast", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip configs 2 and 5")
    ap.add_argument("--config5-bodies", type=int, default=1_000_000)
    ap.add_argument("--no-stages", action="store_true")
    ap.add_argument("--served-rates", default="1000,2000,5000,10000,20000,50000",
                    help="Poisson request rates (req/s) for the served form; empty to skip")
    ap.add_argument("--served-seconds", type=float, default=1.5)
    return ap.parse_args()


def window(a):
    return f"steps {a.warmup + 1}-{a.warmup + a.steps} after {a.warmup} warm-up steps from the initial state"


def config_dict(a, n_dynamic, world_size):
    return {"workload": f"batched worlds: {a.worlds} worlds x log-uniform[{a.nmin},{a.nmax}] bodies "
                        f"(spheres/boxes/hulls in 5 m bins), {a.precision.upper()}"
                        f"{' parity form (bit-identical to the FP64 oracle)' if a.precision == 'f64' else ' bulk + FP64 impulses'}, "
                        f"dt=1/120, 10 iterations",
            "worlds_per_gpu": a.worlds, "dynamic_bodies_per_gpu": n_dynamic,
            "window": window(a),
            "parallelism": f"replicas x{world_size} (independent worlds per GPU, no collective)",
            "l2": "inputs larger than L2 (device-resident body state > 129 MB)",
            "seed": "scenes.config3 seed 0x50484B0000000003 + rank"}


# ------------------------------------------------------------------------------------------------
# clocks
# ------------------------------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.index = index

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
# CPU legs: the FP64 oracle on worlds of the same batch, same window
# ------------------------------------------------------------------------------------------------
def world_ranges(scene):
    """[start, end) of each world's records (config3 keeps every world's records contiguous)."""
    import numpy as np

    w = scene.bodies["world"]
    starts = np.searchsorted(w, np.arange(scene.nworlds), side="left")
    ends = np.searchsorted(w, np.arange(scene.nworlds), side="right")
    return starts, ends


def _cpu_worker(args):
    scene_kw, worlds, steps, warmup, barrier, out_q = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from physkit_gb300 import scenes

    scene = scenes.config3(**scene_kw)
    starts, ends = world_ranges(scene)
    ows, nb = [], 0
    for w in worlds:
        sub = scenes.Scene("w", scene.shapes, scene.bodies[starts[w]:ends[w]].copy(), 1)
        ow = pyoracle.OracleWorld(gravity=scene.gravity, iterations=scene.iterations, order="key")
        pyoracle.load_scene(ow, sub)
        ows.append(ow)
        nb += sub.n_dynamic
    for _ in range(warmup):
        for ow in ows:
            ow.step(scene.dt)
    if barrier is not None:
        barrier.wait()
    t0 = time.perf_counter()
    for _ in range(steps):
        for ow in ows:
            ow.step(scene.dt)
    t1 = time.perf_counter()
    if barrier is not None:
        barrier.wait()
    out_q.put((nb, t1 - t0))


def cpu_baseline(scene_kw, worlds, steps, warmup, procs, sizes=None):
    """FP64 oracle over `worlds` with `procs` processes (spawned, one world list each, largest
    worlds dealt first to the least loaded process); returns (body-steps/s, bodies, wall s)."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    shards = [[] for _ in range(procs)]
    if sizes is None:
        for i, w in enumerate(worlds):
            shards[i % procs].append(w)
    else:
        load = [0] * procs
        for w in sorted(worlds, key=lambda w: -sizes[w]):
            k = min(range(procs), key=load.__getitem__)
            shards[k].append(w)
            load[k] += sizes[w]
    shards = [s for s in shards if s]
    q = ctx.Queue()
    barrier = ctx.Barrier(len(shards) + 1) if len(shards) > 1 else None
    ps = [ctx.Process(target=_cpu_worker, args=((scene_kw, s, steps, warmup, barrier, q),)) for s in shards]
    for p in ps:
        p.start()
    if barrier is not None:
        barrier.wait()
        t0 = time.perf_counter()
        barrier.wait()
        wall = time.perf_counter() - t0
    res = [q.get() for _ in ps]
    for p in ps:
        p.join()
    nb = sum(r[0] for r in res)
    if barrier is None:
        wall = res[0][1]
    return nb * steps / wall, nb, wall


# ------------------------------------------------------------------------------------------------
def run_reference(a, rank, world_size):
    """The reference's CPU path (the FP64 oracle restating it; the reference itself does not
    build here) on the whole batch of this configuration and the same window as our arm."""
    if rank != 0:
        return
    import numpy as np
    from physkit_gb300 import scenes

    ncpu = os.cpu_count() or 1
    kw = {"nworlds": a.worlds, "nmin": a.nmin, "nmax": a.nmax}
    scene = scenes.config3(**kw)
    starts, ends = world_ranges(scene)
    sizes = (ends - starts).tolist()
    value, nb, wall = cpu_baseline(kw, list(range(a.worlds)), a.steps, a.warmup, ncpu, sizes)
    assert nb == scene.n_dynamic
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": wall * 1e3 / a.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(argparse.Namespace(**{**vars(a), "precision": "f64"}),
                                                       nb, world_size),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncpu, "kind": "port",
                             "sample": f"FP64 oracle restating the reference step on all {a.worlds} worlds "
                                       f"({nb} dynamic bodies), {window(a)}, {ncpu} processes "
                                       f"(worlds dealt largest first), {wall:.1f} s timed"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _make(scene, precision, tuned, pair_factor=12, contact_factor=0):
    from physkit_gb300 import scenes

    # pair capacity 12 per body: settled piles keep ~6 fat-box pairs per body
    world, _ = scenes.make_world(scene, precision=precision, pair_factor=pair_factor, contact_factor=contact_factor)
    if tuned:
        world.set_tuning(tuned)
    return world


def _tune(scene, precision, warmup):
    """The project's autotuner on a scratch copy of the batch, from the step the timed window starts."""
    scratch = _make(scene, precision, None)
    for _ in range(warmup):
        scratch.step_async(scene.dt)
    scratch.synchronize()
    tuned = scratch.autotune(scene.dt, 2)
    scratch.close()
    return tuned


def _device_window(world, dt, warmup, steps, dist, local_rank, clocks=False):
    """W untimed steps, then K steps timed by CUDA events on the world's stream between a barrier
    and synchronisations; returns (max-over-ranks ms, step info, clocks)."""
    import torch
    from physkit_gb300 import replicas

    for _ in range(warmup):
        world.step_async(dt)
    world.synchronize()
    stream = torch.cuda.ExternalStream(world.stream())
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = None
    if clocks:
        clk = Clocks(local_rank)
        clk.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        world.step_async(dt)
    ev1.record(stream)
    info = world.synchronize()
    torch.cuda.synchronize()
    clk = clk.stop() if clk else None
    ms = replicas.max_over_ranks(ev0.elapsed_time(ev1), dist, device="cuda")
    return ms, info, clk


def run_ours(a, rank, world_size, local_rank):
    import numpy as np
    import torch

    torch.cuda.set_device(local_rank)
    from physkit_gb300 import replicas, scenes

    dist = None
    if world_size > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl")
        dist = dist_mod

    scene = scenes.config3(nworlds=a.worlds, nmin=a.nmin, nmax=a.nmax,
                           seed=replicas.rank_seed(scenes.SEED_BASE + 3, rank))
    dt = scene.dt
    nb = scene.n_dynamic
    nb_all = replicas.sum_over_ranks(nb, dist, device="cuda")
    tuned = None if a.no_tune else _tune(scene, a.precision, a.warmup)

    # headline: no stage events inside the timed region
    world = _make(scene, a.precision, tuned)
    ms, info, clk = _device_window(world, dt, a.warmup, a.steps, dist, local_rank, clocks=True)
    value = replicas.job_throughput(nb_all, a.steps, ms)
    keys, counts, _ = world.manifolds()
    P, Cn = len(keys), int(counts.sum())
    world.close()

    # end to end through the C ABI, same window on a fresh copy: step + host read-back of every
    # body's state into a pinned host array (registered once, before the window)
    e2e = None
    if not a.no_e2e:
        world = _make(scene, a.precision, tuned)
        hosts = [np.empty((len(scene.bodies), 14)) for _ in range(2)]
        for h in hosts:
            world.pin(h)
        for _ in range(a.warmup):
            world.step(dt, check=False)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(a.steps):
            world.step_async(dt)
            world.bodies_async(hosts[k % 2])
        info_e2e = world.synchronize()
        e2e_s = time.perf_counter() - t0
        for h in hosts:
            world.unpin(h)
        world.close()
        e2e_s = replicas.max_over_ranks(e2e_s, dist, device="cuda")
        e2e = {"value": nb_all * a.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": int(hosts[0].nbytes), "ms_per_step": e2e_s * 1e3 / a.steps,
               "note": "fresh copy of the batch, same window, host clock: every step pk_world_step_async then "
                       "pk_world_read_bodies_async of every slot (14 doubles, packed on the device) into one of "
                       "two pinned host arrays in turn, the copy of step k overlapping step k+1; "
                       "pk_world_synchronize at the end; dt is the only per-step input (a kernel argument)",
               "device_status_flags": info_e2e["flags"]}

    # stage split and roofline: a third copy, same window, CUDA events between the stages
    per_stage, roof = {}, None
    if not a.no_stages:
        world = _make(scene, a.precision, tuned)
        for _ in range(a.warmup):
            world.step_async(dt)
        world.synchronize()
        world.set_timing(True)
        world.stage_times()  # clear
        for _ in range(a.steps):
            world.step_async(dt)
        world.synchronize()
        stages = world.stage_times()
        world.close()
        per_stage = {k: v[0] / max(v[1], 1) for k, v in stages.items()}
        units = {"body": nb, "pair": P, "contact": Cn, "contact_iter": Cn * (scene.iterations + 1)}
        dom = max((k for k in per_stage if ":" not in k), key=per_stage.get)  # "narrow:*" split narrow
        unit, bpu = BYTES[dom]
        achieved = bpu * units[unit] / (per_stage[dom] / 1e3) / 1e9
        peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(peaks_path):
            peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured"
        else:
            peak, peak_src = 6800.0, "fallback"
        traffic = None
        prof = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(prof):
            traffic = json.load(open(prof)).get(f"{a.precision}:{dom}")
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "peak_source": peak_src,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "model": f"{bpu:g} B per {unit} x {units[unit]} {unit}s per launch"}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": a.precision, "data": "synthetic",
           "config": config_dict(a, nb, world_size), "e2e": e2e,
           "gpu_launches": info["launches"] * a.steps, "clocks": clk, "roofline": roof,
           "stage_ms_per_step": {k: round(v, 4) for k, v in per_stage.items()},
           "roofline_support": _support_roofline(info, per_stage.get("narrow"), a.precision),
           "autotune": tuned,
           "counts": {"pairs": P, "contacts": Cn, "gjk": info["gjk"], "epa": info["epa"],
                      "gjk_large_mesh": info["gjk_large_mesh"], "epa_large_mesh": info["epa_large_mesh"],
                      "gjk_iterations": info["gjk_iterations"], "epa_iterations": info["epa_iterations"],
                      "epa_iterations_large_mesh": info["epa_iterations_large_mesh"],
                      "status": info["flags"]}}

    if not a.no_precision_form:
        # the other precision form on the same window
        other = "f32" if a.precision == "f64" else "f64"
        t2 = None if a.no_tune else _tune(scene, other, a.warmup)
        world = _make(scene, other, t2)
        ms2, _, _ = _device_window(world, dt, a.warmup, a.steps, dist, local_rank)
        world.close()
        v2 = replicas.job_throughput(nb_all, a.steps, ms2)
        out["precision_form"] = {"dtype": other, "value": v2, "unit": UNIT, "ms_per_step": ms2 / a.steps,
                                 f"ratio_to_{a.precision}": v2 / value, "autotune": t2,
                                 "accuracy": "per-quantity error against the FP64 form: precision_f32_vs_f64"}

    if rank == 0 and not a.no_configs:
        out["config2"] = config2_report(a)
        out["config5"] = config5_report(a)
        out["config5_replica_f32_vs_f64"] = config5_replica_report()
    if rank == 0 and not a.no_raycast:
        out["raycast"] = raycast_bench(scene, a, rank)
    if rank == 0 and not a.no_plain:
        out["plain_single_world"] = plain_world(a)
        out["batched_vs_plain"] = value / world_size / out["plain_single_world"]["value"]
    if rank == 0 and not a.no_precision:
        out["precision_f32_vs_f64"] = precision_report()
    if rank == 0 and a.served_rates:
        from physkit_gb300.serve import run_served

        out["served"] = [run_served(rate=float(r), duration=a.served_seconds, warm_live=256, max_worlds=1024,
                                    max_bodies=1_500_000, lanes=4, lane_servers=6)
                         for r in a.served_rates.split(",")]
    if rank == 0 and not a.no_cpu_baseline:
        kw = {"nworlds": a.worlds, "nmin": a.nmin, "nmax": a.nmax}
        sample = list(range(min(a.cpu_sample_worlds, a.worlds)))
        csteps = max(1, min(a.steps, 10))
        v, cnb, wall = cpu_baseline(kw, sample, csteps, a.warmup, 1)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"FP64 oracle, worlds 0-{len(sample) - 1} of the batch ({cnb} dynamic "
                                         f"bodies), steps {a.warmup + 1}-{a.warmup + csteps} after {a.warmup} "
                                         f"warm-up steps, 1 thread, {wall:.1f} s"}
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def _stage_split(world, dt, steps):
    world.set_timing(True)
    world.stage_times()  # clear
    for _ in range(steps):
        world.step_async(dt)
    world.synchronize()
    st = world.stage_times()
    world.set_timing(False)
    return {k: round(v[0] / max(v[1], 1), 4) for k, v in st.items()}


def _support_roofline(info, narrow_ms, precision):
    """Secondary bound of the narrowphase: the FLOPs of the reference's support scans (5 per
    vertex a linear first-strict-max scan visits, over the separating-axis, GJK and EPA supports of
    the last step) over the narrow stage's time, against the CUDA-core peak of the form's
    precision (nominal: 152 SMs x FMA lanes x 2 FLOP x the maximum SM clock; 128 FP32 lanes, 2
    FP64 lanes per SM per clock). The device search visits vertex clusters and UV-sphere
    neighbourhoods instead of every vertex, so the fraction can exceed 1."""
    sv = info.get("support_vertices")
    if not narrow_ms or not sv:
        return None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    mhz = json.load(open(peaks_path)).get("sm_max_mhz", 2070.0) if os.path.exists(peaks_path) else 2070.0
    lanes = 128 if precision == "f32" else 2
    peak = 152 * lanes * 2 * mhz * 1e6 / 1e12
    flops = 5.0 * sv
    achieved = flops / (narrow_ms / 1e3) / 1e12
    return {"bound": "fma", "pipe": "fp32" if precision == "f32" else "fp64", "kernel": "narrow",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "nominal", "flops_per_step": flops,
            "model": "5 FLOP x vertices of linear support scans per step / narrow stage time"}


def _roofline(stages, units):
    dom = max((k for k in stages if ":" not in k), key=stages.get)
    unit, bpu = BYTES[dom]
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak = json.load(open(peaks_path))["hbm_gbs"] if os.path.exists(peaks_path) else 6800.0
    achieved = bpu * units[unit] / (stages[dom] / 1e3) / 1e9
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "model": f"{bpu:g} B per {unit} x {units[unit]} {unit}s per launch"}


def config2_report(a):
    """Config 2: one world of 100,000 mixed convex bodies (1/3 UV spheres of 482 vertices, 1/3
    boxes, 1/3 hulls of 16 points) in a 200 m cube with v ~ N(0, 1 m/s): the LBVH broadphase, the
    grid-wide solver and GJK/EPA on large meshes in a single world; FP64 and FP32 forms."""
    from physkit_gb300 import scenes

    sc = scenes.config2()
    w_, k_ = a.warmup, a.steps
    out = {"workload": "config2: 100,000 mixed convex bodies in a 200 m cube, one world, dt=1/120, 10 iterations",
           "window": f"steps {w_ + 1}-{w_ + k_} after {w_} warm-up steps", "dynamic_bodies": sc.n_dynamic}
    for prec in ("f64", "f32"):
        world = _make(sc, prec, None, pair_factor=4)
        ms, info, _ = _device_window(world, sc.dt, w_, k_, None, 0)
        keys, counts, _ = world.manifolds()
        stages = _stage_split(world, sc.dt, 5)
        world.close()
        units = {"body": sc.n_dynamic, "pair": len(keys), "contact": int(counts.sum()),
                 "contact_iter": int(counts.sum()) * (sc.iterations + 1)}
        out[prec] = {"value": sc.n_dynamic * k_ / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / k_,
                     "pairs": len(keys), "contacts": int(counts.sum()), "status": info["flags"],
                     "stage_ms_per_step": stages, "roofline": _roofline(stages, units),
                     "stage_window": f"steps {w_ + k_ + 1}-{w_ + k_ + 5}"}
    return out


def config5_report(a):
    """Config 5: dense-contact stress, N spheres (r ~ lognormal(ln 0.05, 0.3)) poured into a
    20 x 20 m box, 20 iterations, dt = 1/240, FP32 form (FP64 is compared on the 10k replica)."""
    from physkit_gb300 import scenes

    n = a.config5_bodies
    sc = scenes.config5(n=n)
    w_, k_ = min(a.warmup, 3), max(1, min(a.steps, 5))
    world = _make(sc, "f32", None, pair_factor=128, contact_factor=8)
    ms, info, clk = _device_window(world, sc.dt, w_, k_, None, 0, clocks=True)
    keys, counts, _ = world.manifolds()
    stages = _stage_split(world, sc.dt, 2)
    world.close()
    units = {"body": sc.n_dynamic, "pair": len(keys), "contact": int(counts.sum()),
             "contact_iter": int(counts.sum()) * (sc.iterations + 1)}
    return {"workload": f"config5: {n:,} spheres poured into a 20 x 20 m box (jittered lattice, falls into a dense "
                        f"pile), FP32 form, dt=1/240, 20 iterations",
            "window": f"steps {w_ + 1}-{w_ + k_} after {w_} warm-up steps (the pour's first steps: every sphere "
                      f"falls onto the ones below)",
            "dynamic_bodies": sc.n_dynamic, "value": sc.n_dynamic * k_ / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms / k_, "pairs": len(keys), "pairs_per_body": len(keys) / sc.n_dynamic,
            "contacts": int(counts.sum()), "contacts_per_body": int(counts.sum()) / sc.n_dynamic,
            "status": info["flags"], "clocks": clk, "stage_ms_per_step": stages,
            "roofline": _roofline(stages, units), "stage_window": f"steps {w_ + k_ + 1}-{w_ + k_ + 2}"}


def pile_stats(world, scene):
    """Kinetic and potential energy, penetration depth percentiles over the contacts with positive
    depth, pairs and contacts of a world after its last step."""
    import numpy as np

    b = world.bodies()
    dyn = scene.bodies["type"] == 0
    m, I = scene.bodies["mass"][dyn], scene.bodies["inertia"][dyn]
    v, w = b[dyn, 7:10], b[dyn, 10:13]
    ke = 0.5 * (m * (v * v).sum(1)).sum() + 0.5 * (I[:, 0] * w[:, 0] ** 2 + I[:, 4] * w[:, 1] ** 2
                                                  + I[:, 8] * w[:, 2] ** 2).sum()
    pe = float((m * 9.81 * b[dyn, 1]).sum())
    k, c, ct = world.manifolds()
    depth = np.concatenate([ct[i, :c[i], 9] for i in np.nonzero(c)[0]]) if c.sum() else np.zeros(0)
    pos = depth[depth > 0]
    q = (lambda p: float(np.percentile(pos, p)) if len(pos) else 0.0)
    return {"ke_j": float(ke), "pe_j": pe, "depth_mean_m": float(pos.mean()) if len(pos) else 0.0,
            "depth_p50_m": q(50), "depth_p99_m": q(99), "depth_max_m": float(pos.max()) if len(pos) else 0.0,
            "pairs": int(len(k)), "contacts": int(c.sum())}


def config5_replica_report(steps=(20, 60, 120, 240, 480)):
    """Config 5's 10,000-sphere sub-region replica (same lattice, radii and depth on a 2 x 2 m
    footprint), 480 steps: FP32 form against the FP64 form (bit-identical to the FP64 oracle) for
    kinetic energy and penetration depth; control: the FP64 form from the float32-rounded start,
    which bounds what rounding alone does to this chaotic pile."""
    from physkit_gb300 import scenes

    sc = scenes.config5(n=10_000, half=1.0)
    ws = {"f32": _make(sc, "f32", None, 128, 8), "f64": _make(sc, "f64", None, 128, 8),
          "control": _make(_rounded_to_f32(sc), "f64", None, 128, 8)}
    rows, flags = [], set()
    for s in range(1, max(steps) + 1):
        for name, w in ws.items():
            if w.step(sc.dt, check=False):
                flags.add(f"{name}: device status raised")
        if s in steps:
            r = {"step": s}
            for name, w in ws.items():
                r[name] = pile_stats(w, sc)
            ref = r["f64"]
            for name in ("f32", "control"):
                r[name]["ke_rel_err"] = abs(r[name]["ke_j"] - ref["ke_j"]) / max(ref["ke_j"], 1e-12)
                r[name]["pe_rel_err"] = abs(r[name]["pe_j"] - ref["pe_j"]) / max(abs(ref["pe_j"]), 1e-12)
                r[name]["depth_p99_abs_err_m"] = abs(r[name]["depth_p99_m"] - ref["depth_p99_m"])
            rows.append(r)
    for w in ws.values():
        w.close()
    return {"workload": "config5 replica: 10,000 spheres on a 2 x 2 m footprint, dt=1/240, 20 iterations", "rows": rows,
            "status": sorted(flags)}


def raycast_bench(scene, a, rank):
    """World raycasts through the C ABI on the batch after the window's steps: 1 M rays spread over
    the worlds' bins; the call rebuilds the LBVH over every body and returns each ray's 16 nearest."""
    import numpy as np

    world = _make(scene, a.precision, None)
    for _ in range(a.warmup):
        world.step_async(scene.dt)
    world.synchronize()
    rr = np.random.default_rng(7 + rank)
    nr = 1_000_000
    org = np.column_stack([rr.uniform(-2.5, 2.5, nr), rr.uniform(0.0, 6.0, nr), rr.uniform(-2.5, 2.5, nr)])
    drc = rr.normal(size=(nr, 3))
    wid = rr.integers(0, a.worlds, nr).astype(np.int32)
    world.raycast_arrays(org[:1000], drc[:1000], 10.0, wid[:1000], cap=16)  # warm
    t0 = time.perf_counter()
    _, _, cnt = world.raycast_arrays(org, drc, 10.0, wid, cap=16)
    rs = time.perf_counter() - t0
    world.close()
    return {"rays": nr, "ms": rs * 1e3, "rays_per_s": nr / rs, "hits_per_ray": float(cnt.mean()),
            "note": "pk_world_raycast with host arrays: LBVH rebuild over all bodies + one thread per ray, "
                    "16 nearest hits kept per ray"}


def _rounded_to_f32(scene):
    """The scene with every value the FP32 form rounds at upload rounded to float32 (pose,
    velocities, mass, inertia, box half extents), still stepped in FP64."""
    import copy

    import numpy as np

    s = copy.deepcopy(scene)
    for f in ("pos", "quat", "vel", "ang_vel", "mass", "inertia", "restitution", "friction"):
        s.bodies[f] = s.bodies[f].astype(np.float32).astype(np.float64)
    s.shapes = [(sh[0],) + tuple(float(np.float32(x)) for x in sh[1:]) if sh[0] == "box" else sh
                for sh in s.shapes]
    return s


def precision_report(steps=240):
    """FP32 precision form against FP64 per quantity, 240 steps, on two scenes. The FP64 run is
    the device FP64 form, bit-identical to the FP64 oracle (tests/test_gpu_world_parity.py).

    config1 (1,000 boxes falling into a pile): control = the FP64 form started from the initial
    state rounded to float32 (an FP32-sized perturbation, once) against the FP64 form; it shows how
    far the pile's own dynamics amplify FP32 rounding, which bounds what any FP32 form can reach.
    resting stacks (scenes.resting_stacks): separated stacks of aligned boxes, not chaotic."""
    import numpy as np
    from physkit_gb300 import scenes

    def body_err(a, b):
        dpos = np.linalg.norm(a[:, 0:3] - b[:, 0:3], axis=1)
        scale = np.maximum(np.linalg.norm(b[:, 0:3], axis=1), 1.0)
        return {"pos_rel_max": float((dpos / scale).max()), "pos_rel_p50": float(np.median(dpos / scale)),
                "pos_abs_max_m": float(dpos.max()),
                "quat_1mdot_max": float((1.0 - np.abs(np.sum(a[:, 3:7] * b[:, 3:7], axis=1))).max()),
                "vel_abs_max_mps": float(np.linalg.norm(a[:, 7:10] - b[:, 7:10], axis=1).max())}

    def contact_err(wa, wb):
        ka, ca, ta = wa.manifolds()
        kb, cb, tb = wb.manifolds()
        ib = {int(k): i for i, k in enumerate(kb)}
        dd, dn, same = [], [], 0
        for i, k in enumerate(ka):
            j = ib.get(int(k))
            if j is None or ca[i] != cb[j] or ca[i] == 0:
                continue
            same += 1
            for c in range(ca[i]):
                dd.append(abs(ta[i, c, 9] - tb[j, c, 9]))
                dn.append(np.linalg.norm(ta[i, c, 0:3] - tb[j, c, 0:3]))
        return {"manifolds_compared": same, "depth_abs_max_m": float(max(dd)) if dd else 0.0,
                "normal_abs_max": float(max(dn)) if dn else 0.0}

    def same_pairs(wa, wb):
        p, q = wa.pairs(), wb.pairs()
        return int(len(p) == len(q) and bool(np.array_equal(np.sort(p), np.sort(q))))

    def run(scene, control, marks):
        dyn = scene.bodies["type"] == 0
        w32, _ = scenes.make_world(scene, precision="f32")
        w64, _ = scenes.make_world(scene, precision="f64")
        wct = scenes.make_world(control, precision="f64")[0] if control is not None else None
        rep, eq32, eqct = {}, 0, 0
        for s in range(1, steps + 1):
            for w in (w32, w64, wct):
                if w is not None:
                    w.step(scene.dt, check=False)
            eq32 += same_pairs(w32, w64)
            if wct is not None:
                eqct += same_pairs(wct, w64)
            if s in marks:
                a, b = w32.bodies()[dyn], w64.bodies()[dyn]
                r = body_err(a, b)
                r.update(contact_err(w32, w64))
                r["steps_with_equal_pair_set"] = eq32
                if wct is not None:
                    r["control_fp64_from_f32_rounded_start"] = dict(body_err(wct.bodies()[dyn], b),
                                                                    steps_with_equal_pair_set=eqct)
                rep[f"step{s}"] = r
        for w in (w32, w64, wct):
            if w is not None:
                w.close()
        return rep

    c1 = scenes.config1(n=1000)
    rep = {"config1": run(c1, _rounded_to_f32(c1), (60, 120, 240)),
           "resting_boxes": run(scenes.resting_stacks(height=1), None, (240,)),
           "resting_stacks": run(scenes.resting_stacks(height=3), None, (240,))}
    rep["workload"] = ("config1: 1,000 boxes + ground, dt=1/120, FP32 form vs FP64 form; control: FP64 form from "
                       "the float32-rounded initial state vs FP64 form. resting_boxes / resting_stacks: "
                       "10 x 10 separated stacks of 1 / 3 aligned boxes dropped 1 cm onto a ground box, FP32 vs FP64 "
                       "(the FP64 oracle with its state rounded to float32 after every step reaches 1.1e-6 / 3.4e-5)")
    return rep


def plain_world(a):
    """The plain single-world GPU step on one world of the same size class (config 1: 1,000 boxes on
    a ground box), replayed from a captured CUDA graph."""
    import torch
    from physkit_gb300 import scenes

    scene = scenes.config1()
    world, _ = scenes.make_world(scene, precision=a.precision)
    world.capture(scene.dt)
    for _ in range(a.warmup):
        world.step_graph()
    world.synchronize()
    stream = torch.cuda.ExternalStream(world.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 100
    ev0.record(stream)
    for _ in range(n):
        world.step_graph()
    ev1.record(stream)
    world.synchronize()
    ms = ev0.elapsed_time(ev1)
    world.close()
    return {"workload": f"config1: 1,000 boxes + ground, one world, {a.precision.upper()}, CUDA-graph replay, "
                        f"steps {a.warmup + 1}-{a.warmup + n}",
            "value": scene.n_dynamic * n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / n}


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world_size = int(os.environ.get("WORLD_SIZE", str(a.gpus)))
    if "RANK" not in os.environ:
        world_size = 1  # without torchrun this process is the only rank
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank, world_size)
    else:
        run_ours(a, rank, world_size, local_rank)


if __name__ == "__main__":
    main()
