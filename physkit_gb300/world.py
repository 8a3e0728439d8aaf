"""Python mirror of the reference's world API over the C ABI (include/physkit_gb300.h).

Names follow the reference: world_desc (core/world.h:23-49), object_desc (core/object.h:15-109),
world::create_rigid / remove_rigid / get_rigid / step (core/world.h:202-242), mesh::box / sphere /
pyramid / make (collision/mesh.h:219-236). Invalid input raises ValueError like the reference's
std::invalid_argument (object.h:121); stale handles give None like get_rigid's std::nullopt.

The device library is required: there is no CPU fallback. Without a CUDA device, World() raises
RuntimeError.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

_lib = None
_lock = threading.Lock()

PK_OK = 0
PK_ERR_INVALID = -1
PK_ERR_STALE_HANDLE = -2
PK_ERR_CAPACITY = -3
PK_ERR_CUDA = -4
PK_ERR_DEVICE_STATUS = -5
PK_ERR_NO_DEVICE = -6
PRECISION = {"f64": 0, "f32": 1}

STATUS_BITS = {1: "pair_overflow", 2: "epa_cap", 4: "colour_cap", 8: "traversal_stack", 16: "nan",
               32: "contact_overflow"}


class WorldDescC(C.Structure):
    _fields_ = [("gravity", C.c_double * 3), ("solver_iterations", C.c_int32), ("precision", C.c_int32),
                ("max_bodies", C.c_int32), ("max_pairs", C.c_int32), ("max_worlds", C.c_int32),
                ("max_bodies_per_world", C.c_int32), ("max_shape_vertices", C.c_int32),
                ("max_shapes", C.c_int32), ("max_contact_pairs", C.c_int32)]


BODY_DTYPE = np.dtype([("type", np.int32), ("shape", np.int32), ("world", np.int32), ("reserved", np.int32),
                       ("pos", np.float64, 3), ("quat", np.float64, 4), ("vel", np.float64, 3),
                       ("ang_vel", np.float64, 3), ("mass", np.float64), ("inertia", np.float64, 9),
                       ("restitution", np.float64), ("friction", np.float64)], align=True)
assert BODY_DTYPE.itemsize == 216


class StepInfoC(C.Structure):
    _fields_ = [("pairs", C.c_int32), ("leaves", C.c_int32), ("status", C.c_int32), ("launches", C.c_int32),
                ("gjk", C.c_int32), ("epa", C.c_int32), ("gjk_large_mesh", C.c_int32), ("epa_large_mesh", C.c_int32),
                ("gjk_iterations", C.c_int64), ("epa_iterations", C.c_int64), ("epa_iterations_large_mesh", C.c_int64),
                ("support_vertices", C.c_int64)]


class TuneResultC(C.Structure):
    _fields_ = [("solve_threads", C.c_int32), ("small_world", C.c_int32), ("narrow_grid", C.c_int32),
                ("traverse_threads", C.c_int32), ("step_ms_before", C.c_double), ("step_ms_after", C.c_double),
                ("steps_used", C.c_int32), ("big_threads", C.c_int32), ("group_bodies", C.c_int32),
                ("group_threads", C.c_int32), ("group_warp", C.c_int32)]


class RayC(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("direction", C.c_double * 3), ("max_distance", C.c_double),
                ("world", C.c_int32), ("reserved", C.c_int32)]


class JointDescC(C.Structure):
    _fields_ = [("type", C.c_int32), ("reserved", C.c_int32), ("a", C.c_uint64), ("b", C.c_uint64),
                ("anchor", C.c_double * 3), ("local_a", C.c_double * 3), ("local_b", C.c_double * 3),
                ("axis_a", C.c_double * 3), ("axis_b", C.c_double * 3), ("distance", C.c_double),
                ("stiffness", C.c_double), ("damping", C.c_double)]


JOINT_TYPES = {"distance": 0, "ball_socket": 1, "hinge": 2, "slider": 3, "weld": 4, "spring": 5}


class WakeC(C.Structure):
    _fields_ = [("waiter", C.c_uint64), ("object", C.c_uint64), ("other", C.c_uint64), ("kind", C.c_int32),
                ("failed", C.c_int32)]


HANDLE_ANY = 0xFFFFFFFFFFFFFFFF
WAIT_COLLISION, WAIT_SEPARATION, WAIT_DESTROYED = 1, 2, 3


class BatchDescC(C.Structure):
    _fields_ = [("gravity", C.c_double * 3), ("dt", C.c_double), ("solver_iterations", C.c_int32),
                ("precision", C.c_int32), ("max_worlds", C.c_int32), ("max_bodies_per_world", C.c_int32),
                ("max_bodies", C.c_int64), ("memory_fraction", C.c_double), ("pair_factor", C.c_int32),
                ("contact_factor", C.c_int32), ("max_shapes", C.c_int32), ("max_shape_vertices", C.c_int32),
                ("pipeline_depth", C.c_int32), ("reserved", C.c_int32)]


class BatchEventC(C.Structure):
    _fields_ = [("tag", C.c_int64), ("world", C.c_int32), ("kind", C.c_int32)]


class BatchInfoC(C.Structure):
    _fields_ = [("pool_bodies", C.c_int64), ("bodies_in_use", C.c_int64), ("steps", C.c_int64),
                ("pending_requests", C.c_int64), ("worlds_live", C.c_int32), ("worlds_free", C.c_int32),
                ("steps_in_flight", C.c_int32), ("reserved", C.c_int32), ("graph_captures", C.c_int64)]


BATCH_STEPPED, BATCH_RETIRED = 1, 2


class MeshRayC(C.Structure):
    _fields_ = [("body", C.c_uint64), ("shape", C.c_int32), ("reserved", C.c_int32), ("pos", C.c_double * 3),
                ("quat", C.c_double * 4), ("origin", C.c_double * 3), ("direction", C.c_double * 3),
                ("max_distance", C.c_double)]


class MeshHitC(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("normal", C.c_double * 3), ("distance", C.c_double), ("hit", C.c_int32),
                ("triangle", C.c_int32)]


class CollideShapeC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("shape", C.c_int32), ("p", C.c_double * 10)]


def library_path() -> str:
    return _build.LIB


def lib():
    """Load libphyskit_gb300.so (building it in-tree first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build()
        L = C.CDLL(path)
        P = C.POINTER
        vp, dp, i32p, u64p = C.c_void_p, P(C.c_double), P(C.c_int32), P(C.c_uint64)
        sig = {
            "pk_world_desc_init": (None, [P(WorldDescC)]),
            "pk_world_create": (C.c_int, [P(WorldDescC), P(C.c_void_p)]),
            "pk_world_destroy": (None, [vp]),
            "pk_shape_mesh": (C.c_int, [vp, dp, C.c_int32, i32p, C.c_int32, i32p]),
            "pk_shape_box": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, i32p]),
            "pk_shape_sphere": (C.c_int, [vp, C.c_double, C.c_int32, C.c_int32, i32p]),
            "pk_shape_pyramid": (C.c_int, [vp, C.c_double, C.c_double, i32p]),
            "pk_body_add": (C.c_int, [vp, C.c_void_p, C.c_int32, u64p]),
            "pk_body_remove": (C.c_int, [vp, C.c_uint64]),
            "pk_world_clear": (C.c_int, [vp, C.c_int32]),
            "pk_world_set_active": (C.c_int, [vp, C.c_int32, C.c_int32]),
            "pk_world_set_active_mask": (C.c_int, [vp, P(C.c_uint8), C.c_int32]),
            "pk_world_set_gravity": (C.c_int, [vp, C.c_int32, dp]),
            "pk_world_step": (C.c_int, [vp, C.c_double]),
            "pk_world_step_async": (C.c_int, [vp, C.c_double]),
            "pk_world_synchronize": (C.c_int, [vp, P(StepInfoC)]),
            "pk_world_capture": (C.c_int, [vp, C.c_double]),
            "pk_world_step_graph": (C.c_int, [vp]),
            "pk_world_stream": (C.c_void_p, [vp]),
            "pk_world_read_bodies": (C.c_int, [vp, dp, C.c_int32, i32p]),
            "pk_world_read_bodies_async": (C.c_int, [vp, dp, C.c_int32, i32p]),
            "pk_host_register": (C.c_int, [vp, C.c_size_t]),
            "pk_host_unregister": (C.c_int, [vp]),
            "pk_world_write_body": (C.c_int, [vp, C.c_uint64, dp]),
            "pk_body_alive": (C.c_int, [vp, C.c_uint64]),
            "pk_world_read_pairs": (C.c_int, [vp, u64p, i32p, C.c_int32, i32p]),
            "pk_world_read_manifolds": (C.c_int, [vp, u64p, i32p, i32p, dp, C.c_int32, i32p]),
            "pk_world_read_events": (C.c_int, [vp, u64p, i32p, i32p, C.c_int32, i32p]),
            "pk_world_read_colours": (C.c_int, [vp, u64p, i32p, C.c_int32, i32p, i32p]),
            "pk_world_raycast": (C.c_int, [vp, P(RayC), C.c_int32, C.c_int32, u64p, dp, i32p]),
            "pk_world_wait": (C.c_int, [vp, C.c_int32, C.c_uint64, C.c_uint64, u64p]),
            "pk_joint_add": (C.c_int, [vp, P(JointDescC), u64p]),
            "pk_joint_remove": (C.c_int, [vp, C.c_uint64]),
            "pk_joint_read_impulses": (C.c_int, [vp, C.c_uint64, dp, i32p]),
            "pk_world_cancel_wait": (C.c_int, [vp, C.c_uint64]),
            "pk_world_dispatch": (C.c_int, [vp, P(WakeC), C.c_int32, i32p]),
            "pk_collide": (C.c_int, [vp, P(CollideShapeC), P(CollideShapeC), C.c_int32, dp, i32p]),
            "pk_collide_noalloc": (C.c_int, [vp, P(CollideShapeC), P(CollideShapeC), C.c_int32, dp, i32p]),
            "pk_world_set_timing": (C.c_int, [vp, C.c_int32]),
            "pk_world_autotune": (C.c_int, [vp, C.c_double, C.c_int32, P(TuneResultC)]),
            "pk_world_set_tuning": (C.c_int, [vp, P(TuneResultC)]),
            "pk_world_read_stage_times": (C.c_int, [vp, dp, i32p, C.c_int32, i32p]),
            "pk_stage_name": (C.c_char_p, [C.c_int32]),
            "pk_batch_desc_init": (None, [P(BatchDescC)]),
            "pk_batch_create": (C.c_int, [P(BatchDescC), P(C.c_void_p)]),
            "pk_batch_destroy": (None, [vp]),
            "pk_batch_world": (C.c_void_p, [vp]),
            "pk_batch_admit": (C.c_int, [vp, C.c_void_p, C.c_int32, u64p, i32p]),
            "pk_batch_request": (C.c_int, [vp, C.c_int32, C.c_int64]),
            "pk_batch_retire": (C.c_int, [vp, C.c_int32]),
            "pk_batch_step_async": (C.c_int, [vp, i32p]),
            "pk_batch_poll": (C.c_int, [vp, P(BatchEventC), C.c_int32, i32p, C.c_int32]),
            "pk_batch_stats": (C.c_int, [vp, P(BatchInfoC)]),
            "pk_batch_read_world": (C.c_int, [vp, C.c_int32, dp, C.c_int32, i32p]),
            "pk_mesh_raycast": (C.c_int, [vp, P(MeshRayC), C.c_int32, P(MeshHitC)]),
            "pk_last_cuda_error": (C.c_int, []),
            "pk_version": (C.c_char_p, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _check(rc, what):
    if rc == PK_OK:
        return
    if rc == PK_ERR_INVALID:
        raise ValueError(f"{what}: invalid argument")
    if rc == PK_ERR_CAPACITY:
        raise MemoryError(f"{what}: capacity exhausted")
    if rc == PK_ERR_NO_DEVICE:
        raise RuntimeError(f"{what}: no CUDA device (physkit_gb300 has no CPU fallback)")
    if rc == PK_ERR_CUDA:
        raise RuntimeError(f"{what}: CUDA error {lib().pk_last_cuda_error()}")
    if rc == PK_ERR_DEVICE_STATUS:
        raise RuntimeError(f"{what}: a device status bit was raised (a capacity of the device path was hit)")
    raise RuntimeError(f"{what}: error {rc}")


class world_desc:
    """world_desc (core/world.h:23-49) plus the device capacities of this implementation."""

    def __init__(self):
        self.gravity = (0.0, -9.81, 0.0)
        self.solver_iterations = 10
        self.precision = "f64"
        self.max_bodies = 4096
        self.max_pairs = 0
        self.max_worlds = 1
        self.max_bodies_per_world = 0
        self.max_shape_vertices = 0
        self.max_shapes = 0
        self.max_contact_pairs = 0

    @staticmethod
    def make():
        return world_desc()

    def with_gravity(self, g):
        self.gravity = tuple(float(x) for x in g)
        return self

    def with_solver_iterations(self, n):
        self.solver_iterations = int(n)
        return self

    def with_precision(self, p):
        if p not in PRECISION:
            raise ValueError(f"precision must be one of {list(PRECISION)}")
        self.precision = p
        return self

    def with_capacity(self, max_bodies, max_pairs=0, max_worlds=1, max_bodies_per_world=0,
                      max_shape_vertices=0, max_shapes=0, max_contact_pairs=0):
        self.max_bodies, self.max_pairs, self.max_worlds = int(max_bodies), int(max_pairs), int(max_worlds)
        self.max_bodies_per_world = int(max_bodies_per_world)
        self.max_shape_vertices, self.max_shapes = int(max_shape_vertices), int(max_shapes)
        self.max_contact_pairs = int(max_contact_pairs)
        return self

    def to_c(self):
        d = WorldDescC()
        lib().pk_world_desc_init(C.byref(d))
        for k in range(3):
            d.gravity[k] = self.gravity[k]
        d.solver_iterations = self.solver_iterations
        d.precision = PRECISION[self.precision]
        d.max_bodies = self.max_bodies
        d.max_pairs = self.max_pairs
        d.max_worlds = self.max_worlds
        d.max_bodies_per_world = self.max_bodies_per_world
        d.max_shape_vertices = self.max_shape_vertices
        d.max_shapes = self.max_shapes
        d.max_contact_pairs = self.max_contact_pairs
        return d


class object_desc:
    """object_desc (core/object.h:15-109): builder for one rigid body."""

    def __init__(self, static=False):
        self.static = static
        self.pos = (0.0, 0.0, 0.0)
        self.vel = (0.0, 0.0, 0.0)
        self.mass = 1.0
        self.orientation = (1.0, 0.0, 0.0, 0.0)
        self.ang_vel = (0.0, 0.0, 0.0)
        self.inertia = np.eye(3)
        self.mesh = None
        self.restitution = 0.5
        self.friction = 0.5
        self.world = 0

    @staticmethod
    def dynam():
        return object_desc(False)

    @staticmethod
    def stat():
        return object_desc(True)

    def with_pos(self, p):
        self.pos = tuple(map(float, p))
        return self

    def with_vel(self, v):
        self.vel = tuple(map(float, v))
        return self

    def with_mass(self, m):
        self.mass = float(m)
        return self

    def with_orientation(self, q):
        self.orientation = tuple(map(float, q))
        return self

    def with_ang_vel(self, w):
        self.ang_vel = tuple(map(float, w))
        return self

    def with_inertia_tensor(self, inertia):
        a = np.asarray(inertia, dtype=np.float64)
        self.inertia = np.diag(a) if a.shape == (3,) else a.reshape(3, 3)
        return self

    def with_mesh(self, shape_id):
        self.mesh = shape_id
        return self

    def with_restitution(self, r):
        self.restitution = float(r)
        return self

    def with_friction(self, f):
        self.friction = float(f)
        return self

    def in_world(self, w):
        self.world = int(w)
        return self

    def record(self):
        if self.mesh is None:
            raise ValueError("Object must have a mesh")  # object.h:121
        r = np.zeros(1, dtype=BODY_DTYPE)
        r["type"] = 1 if self.static else 0
        r["shape"] = self.mesh
        r["world"] = self.world
        r["pos"] = self.pos
        r["quat"] = self.orientation
        r["vel"] = self.vel
        r["ang_vel"] = self.ang_vel
        r["mass"] = self.mass
        r["inertia"] = self.inertia.reshape(-1)
        r["restitution"] = self.restitution
        r["friction"] = self.friction
        return r


class World:
    """A device-resident world (or batch of independent worlds) behind the C ABI."""

    def __init__(self, desc: world_desc | None = None, _borrow=None):
        self.L = lib()
        self.last_info = None
        self.owned = _borrow is None
        if _borrow is not None:  # the world object of a pk_batch (the batch owns it)
            self.desc = None
            self.h = C.c_void_p(_borrow)
            return
        self.desc = desc or world_desc()
        h = C.c_void_p()
        _check(self.L.pk_world_create(C.byref(self.desc.to_c()), C.byref(h)), "pk_world_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            if self.owned:
                self.L.pk_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # meshes (mesh.h:219-236) ------------------------------------------------------------------
    def mesh_box(self, hx, hy, hz):
        out = C.c_int32()
        _check(self.L.pk_shape_box(self.h, hx, hy, hz, C.byref(out)), "pk_shape_box")
        return out.value

    def mesh_sphere(self, r, stacks=16, sectors=32):
        out = C.c_int32()
        _check(self.L.pk_shape_sphere(self.h, r, stacks, sectors, C.byref(out)), "pk_shape_sphere")
        return out.value

    def mesh_pyramid(self, b, h):
        out = C.c_int32()
        _check(self.L.pk_shape_pyramid(self.h, b, h, C.byref(out)), "pk_shape_pyramid")
        return out.value

    def mesh_make(self, verts, tris):
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1))
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.int32).reshape(-1))
        out = C.c_int32()
        _check(self.L.pk_shape_mesh(self.h, _ptr(v, C.c_double), len(v) // 3, _ptr(t, C.c_int32), len(t) // 3,
                                    C.byref(out)), "pk_shape_mesh")
        return out.value

    # bodies ------------------------------------------------------------------------------------
    def create_rigid(self, desc: object_desc):
        return int(self.create_rigids(desc.record())[0])

    def create_rigids(self, records: np.ndarray):
        rec = np.ascontiguousarray(records, dtype=BODY_DTYPE)
        n = len(rec)
        out = np.zeros(max(n, 1), dtype=np.uint64)
        _check(self.L.pk_body_add(self.h, rec.ctypes.data, n, _ptr(out, C.c_uint64)), "pk_body_add")
        return out[:n]

    def remove_rigid(self, handle):
        rc = self.L.pk_body_remove(self.h, C.c_uint64(int(handle)))
        if rc == PK_ERR_STALE_HANDLE:
            return False
        _check(rc, "pk_body_remove")
        return True

    def clear_world(self, w):
        """Retire world w: its bodies, pairs and manifolds go; its slots become free."""
        _check(self.L.pk_world_clear(self.h, int(w)), "pk_world_clear")

    def set_active(self, w, active):
        _check(self.L.pk_world_set_active(self.h, int(w), int(bool(active))), "pk_world_set_active")

    def set_active_mask(self, mask):
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        _check(self.L.pk_world_set_active_mask(self.h, _ptr(m, C.c_uint8), len(m)), "pk_world_set_active_mask")

    # stepping ----------------------------------------------------------------------------------
    def step(self, dt, check=True):
        """One synchronous step. With check=False a raised device status bit (pair overflow, caps,
        non-finite state) is returned as True instead of raising."""
        rc = self.L.pk_world_step(self.h, float(dt))
        if rc == PK_ERR_DEVICE_STATUS and not check:
            return True
        _check(rc, "pk_world_step")
        return False

    def step_async(self, dt):
        _check(self.L.pk_world_step_async(self.h, float(dt)), "pk_world_step_async")

    def capture(self, dt):
        _check(self.L.pk_world_capture(self.h, float(dt)), "pk_world_capture")

    def step_graph(self):
        _check(self.L.pk_world_step_graph(self.h), "pk_world_step_graph")

    def synchronize(self):
        info = StepInfoC()
        rc = self.L.pk_world_synchronize(self.h, C.byref(info))
        if rc not in (PK_OK, PK_ERR_DEVICE_STATUS):
            _check(rc, "pk_world_synchronize")
        self.last_info = {"pairs": info.pairs, "leaves": info.leaves, "status": info.status,
                          "launches": info.launches, "gjk": info.gjk, "epa": info.epa,
                          "gjk_large_mesh": info.gjk_large_mesh, "epa_large_mesh": info.epa_large_mesh,
                          "gjk_iterations": info.gjk_iterations, "epa_iterations": info.epa_iterations,
                          "epa_iterations_large_mesh": info.epa_iterations_large_mesh,
                          "support_vertices": info.support_vertices,
                          "flags": [v for k, v in STATUS_BITS.items() if info.status & k]}
        return self.last_info

    def stream(self):
        return self.L.pk_world_stream(self.h)

    def autotune(self, dt, steps_per_candidate=2):
        """Pick launch shapes by timing real steps (which advance the world); returns the choice."""
        r = TuneResultC()
        _check(self.L.pk_world_autotune(self.h, float(dt), int(steps_per_candidate), C.byref(r)), "pk_world_autotune")
        return {f: getattr(r, f) for f, _ in TuneResultC._fields_}

    def set_tuning(self, tuned):
        r = TuneResultC()
        for f, _ in TuneResultC._fields_:
            if f in tuned:
                setattr(r, f, tuned[f])
        _check(self.L.pk_world_set_tuning(self.h, C.byref(r)), "pk_world_set_tuning")

    def set_timing(self, enable=True):
        _check(self.L.pk_world_set_timing(self.h, int(bool(enable))), "pk_world_set_timing")

    def stage_times(self):
        """{stage: (total ms, steps)} accumulated since the last call (CUDA events per stage)."""
        ms = np.zeros(16)
        cnt = np.zeros(16, dtype=np.int32)
        n = C.c_int32()
        _check(self.L.pk_world_read_stage_times(self.h, _ptr(ms, C.c_double), _ptr(cnt, C.c_int32), 16,
                                                C.byref(n)), "pk_world_read_stage_times")
        return {self.L.pk_stage_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(n.value)}

    # reads -------------------------------------------------------------------------------------
    def bodies(self, out=None):
        """State rows of every slot (pos3 quat4 vel3 ang_vel3 alive). With `out` (a C-contiguous
        float64 array of shape (>= slots, 14), ideally pinned with pin()), the rows are read into it
        and a view of the filled part is returned."""
        n = C.c_int32()
        self.L.pk_world_read_bodies(self.h, None, 0, C.byref(n))
        if out is None:
            out = np.empty((max(n.value, 1), 14))
        elif out.dtype != np.float64 or out.ndim != 2 or out.shape[1] != 14 or not out.flags.c_contiguous \
                or out.shape[0] < n.value:
            raise ValueError("out must be a C-contiguous float64 array of shape (>= %d, 14)" % n.value)
        _check(self.L.pk_world_read_bodies(self.h, _ptr(out, C.c_double), n.value, C.byref(n)),
               "pk_world_read_bodies")
        return out[: n.value]

    def bodies_async(self, out):
        """Enqueue a read of the state rows into `out` (C-contiguous float64, shape (>= slots, 14),
        pinned with pin() for the copy to overlap later steps); the rows land by the next
        synchronize() or step(). Returns the number of rows."""
        n = C.c_int32()
        self.L.pk_world_read_bodies(self.h, None, 0, C.byref(n))
        if out.dtype != np.float64 or out.ndim != 2 or out.shape[1] != 14 or not out.flags.c_contiguous \
                or out.shape[0] < n.value:
            raise ValueError("out must be a C-contiguous float64 array of shape (>= %d, 14)" % n.value)
        _check(self.L.pk_world_read_bodies_async(self.h, _ptr(out, C.c_double), n.value, C.byref(n)),
               "pk_world_read_bodies_async")
        return n.value

    def pin(self, arr):
        """Page-lock a host array that is read into (or written from) every step."""
        _check(self.L.pk_host_register(C.c_void_p(arr.ctypes.data), arr.nbytes), "pk_host_register")

    def unpin(self, arr):
        _check(self.L.pk_host_unregister(C.c_void_p(arr.ctypes.data)), "pk_host_unregister")

    def get_rigid(self, handle):
        """world_base::get_rigid (world.h:220-224): state row, or None for a stale handle."""
        slot = int(handle) & 0xFFFFFFFF
        b = self.bodies()
        if slot >= len(b) or b[slot, 13] == 0.0:
            return None
        return b[slot]

    def write_body(self, handle, state13):
        s = np.ascontiguousarray(state13, dtype=np.float64)
        _check(self.L.pk_world_write_body(self.h, C.c_uint64(int(handle)), _ptr(s, C.c_double)),
               "pk_world_write_body")

    # joints ------------------------------------------------------------------------------------
    def add_joint(self, kind, a, b, anchor=(0, 0, 0), local_a=(0, 0, 0), local_b=(0, 0, 0), axis_a=(0, 0, 0),
                  axis_b=(0, 0, 0), distance=0.0, stiffness=0.0, damping=0.0):
        """A joint between bodies a and b (constraint.h:139-865); returns its handle."""
        d = JointDescC()
        d.type = JOINT_TYPES[kind]
        d.a, d.b = int(a), int(b)
        d.anchor[:] = list(map(float, anchor))
        d.local_a[:] = list(map(float, local_a))
        d.local_b[:] = list(map(float, local_b))
        d.axis_a[:] = list(map(float, axis_a))
        d.axis_b[:] = list(map(float, axis_b))
        d.distance, d.stiffness, d.damping = float(distance), float(stiffness), float(damping)
        out = C.c_uint64()
        _check(self.L.pk_joint_add(self.h, C.byref(d), C.byref(out)), "pk_joint_add")
        return out.value

    def remove_joint(self, handle):
        _check(self.L.pk_joint_remove(self.h, int(handle)), "pk_joint_remove")

    def joint_impulses(self, handle):
        out = np.zeros(6)
        n = C.c_int32()
        _check(self.L.pk_joint_read_impulses(self.h, int(handle), _ptr(out, C.c_double), C.byref(n)),
               "pk_joint_read_impulses")
        return out[:n.value]

    # waiting on collision events ---------------------------------------------------------------
    def wait(self, kind, obj, with_=None):
        """Register a waiter (WAIT_COLLISION / WAIT_SEPARATION with an object or any, or
        WAIT_DESTROYED); returns its id, or None when `obj` is not alive (nothing to wait for)."""
        out = C.c_uint64()
        rc = self.L.pk_world_wait(self.h, int(kind), int(obj), HANDLE_ANY if with_ is None else int(with_),
                                  C.byref(out))
        if rc == PK_ERR_STALE_HANDLE:
            return None
        _check(rc, "pk_world_wait")
        return out.value

    def cancel_wait(self, waiter):
        _check(self.L.pk_world_cancel_wait(self.h, int(waiter)), "pk_world_cancel_wait")

    def dispatch(self, cap=1024):
        """Offer the last step's events to the waiters; returns the fired ones as
        (waiter, object, other or None, kind, failed)."""
        out, res = (WakeC * cap)(), []
        while True:
            n = C.c_int32()
            _check(self.L.pk_world_dispatch(self.h, out, cap, C.byref(n)), "pk_world_dispatch")
            for i in range(n.value):
                k = out[i]
                res.append((k.waiter, k.object, None if k.other == HANDLE_ANY else k.other, k.kind, bool(k.failed)))
            if n.value < cap:
                return res

    RAY_DTYPE = np.dtype([("origin", np.float64, 3), ("direction", np.float64, 3), ("max_distance", np.float64),
                          ("world", np.int32), ("reserved", np.int32)])

    def raycast_arrays(self, origins, directions, max_distance, worlds=0, cap=64):
        """World raycast (world.h:260-319) for n rays: handles (n, cap), distances (n, cap) nearest
        first (the first min(count, cap) of each row are valid) and total hit counts (n,)."""
        o = np.atleast_2d(np.asarray(origins, dtype=np.float64))
        n = len(o)
        rays = np.zeros(n, dtype=self.RAY_DTYPE)
        rays["origin"] = o
        rays["direction"] = np.atleast_2d(np.asarray(directions, dtype=np.float64))
        rays["max_distance"] = np.broadcast_to(np.asarray(max_distance, dtype=np.float64), (n,))
        rays["world"] = np.broadcast_to(np.asarray(worlds, dtype=np.int32), (n,))
        hs = np.zeros((max(n, 1), cap), dtype=np.uint64)
        ds = np.zeros((max(n, 1), cap))
        cnt = np.zeros(max(n, 1), dtype=np.int32)
        _check(self.L.pk_world_raycast(self.h, rays.ctypes.data_as(C.POINTER(RayC)), n, cap, _ptr(hs, C.c_uint64),
                                       _ptr(ds, C.c_double), _ptr(cnt, C.c_int32)), "pk_world_raycast")
        return hs[:n], ds[:n], cnt[:n]

    def raycast(self, origins, directions, max_distance, worlds=0, cap=64):
        """As raycast_arrays, as a list of [(handle, distance)] per ray, and the counts."""
        hs, ds, cnt = self.raycast_arrays(origins, directions, max_distance, worlds, cap)
        out = []
        for i in range(len(cnt)):
            k = min(int(cnt[i]), cap)
            out.append(list(zip(hs[i, :k].tolist(), ds[i, :k].tolist())))
        return out, cnt.copy()

    def mesh_raycast(self, rays):
        """Rays against mesh instances (mesh::instance::ray_intersect). rays: a list of dicts with
        origin, direction, max_distance and either body (a handle) or shape + pos + quat (w,x,y,z).
        Returns per ray None or (pos3, normal3, distance, triangle)."""
        n = len(rays)
        R = (MeshRayC * max(n, 1))()
        for i, r in enumerate(rays):
            R[i].body = int(r["body"]) if "body" in r else HANDLE_ANY
            R[i].shape = int(r.get("shape", -1))
            R[i].pos[:] = list(map(float, r.get("pos", (0, 0, 0))))
            R[i].quat[:] = list(map(float, r.get("quat", (1, 0, 0, 0))))
            R[i].origin[:] = list(map(float, r["origin"]))
            R[i].direction[:] = list(map(float, r["direction"]))
            R[i].max_distance = float(r.get("max_distance", 1e300))
        H = (MeshHitC * max(n, 1))()
        _check(self.L.pk_mesh_raycast(self.h, R, n, H), "pk_mesh_raycast")
        out = []
        for i in range(n):
            h = H[i]
            out.append((np.array(h.pos[:]), np.array(h.normal[:]), h.distance, h.triangle) if h.hit else None)
        return out

    def pairs(self, with_worlds=False):
        n = C.c_int32()
        self.L.pk_world_read_pairs(self.h, None, None, 0, C.byref(n))
        k = np.zeros(max(n.value, 1), dtype=np.uint64)
        w = np.zeros(max(n.value, 1), dtype=np.int32)
        _check(self.L.pk_world_read_pairs(self.h, _ptr(k, C.c_uint64), _ptr(w, C.c_int32), n.value, C.byref(n)),
               "pk_world_read_pairs")
        return (k[: n.value], w[: n.value]) if with_worlds else k[: n.value]

    def manifolds(self, with_worlds=False):
        n = C.c_int32()
        self.L.pk_world_read_manifolds(self.h, None, None, None, None, 0, C.byref(n))
        m = max(n.value, 1)
        k = np.zeros(m, dtype=np.uint64)
        w = np.zeros(m, dtype=np.int32)
        c = np.zeros(m, dtype=np.int32)
        ct = np.zeros((m, 4, 13))
        _check(self.L.pk_world_read_manifolds(self.h, _ptr(k, C.c_uint64), _ptr(w, C.c_int32), _ptr(c, C.c_int32),
                                              _ptr(ct, C.c_double), n.value, C.byref(n)), "pk_world_read_manifolds")
        r = (k[: n.value], c[: n.value], ct[: n.value])
        return r + (w[: n.value],) if with_worlds else r

    def events(self, with_worlds=False):
        n = C.c_int32()
        self.L.pk_world_read_events(self.h, None, None, None, 0, C.byref(n))
        m = max(n.value, 1)
        k = np.zeros(m, dtype=np.uint64)
        w = np.zeros(m, dtype=np.int32)
        kd = np.zeros(m, dtype=np.int32)
        _check(self.L.pk_world_read_events(self.h, _ptr(k, C.c_uint64), _ptr(w, C.c_int32), _ptr(kd, C.c_int32),
                                           n.value, C.byref(n)), "pk_world_read_events")
        r = (k[: n.value], kd[: n.value])
        return r + (w[: n.value],) if with_worlds else r

    def colours(self):
        n = C.c_int32()
        nc = C.c_int32()
        self.L.pk_world_read_colours(self.h, None, None, 0, C.byref(n), C.byref(nc))
        m = max(n.value, 1)
        k = np.zeros(m, dtype=np.uint64)
        col = np.zeros(m, dtype=np.int32)
        _check(self.L.pk_world_read_colours(self.h, _ptr(k, C.c_uint64), _ptr(col, C.c_int32), n.value, C.byref(n),
                                            C.byref(nc)), "pk_world_read_colours")
        return k[: n.value], col[: n.value], nc.value

    def collide(self, shapes_a, shapes_b, noalloc=False):
        """gjk_epa on primitive shape pairs; each shape is (kind, params list, mesh id).
        noalloc=True goes through pk_collide_noalloc (no device allocation; at most 4096 pairs)."""
        n = len(shapes_a)
        A = (CollideShapeC * max(n, 1))()
        B = (CollideShapeC * max(n, 1))()
        for i, (sa, sb) in enumerate(zip(shapes_a, shapes_b)):
            for dst, (kind, params, sid) in ((A[i], sa), (B[i], sb)):
                dst.kind = kind
                dst.shape = sid
                for k, v in enumerate(params):
                    dst.p[k] = v
        out = np.zeros((max(n, 1), 10))
        hit = np.zeros(max(n, 1), dtype=np.int32)
        fn = self.L.pk_collide_noalloc if noalloc else self.L.pk_collide
        _check(fn(self.h, A, B, n, _ptr(out, C.c_double), _ptr(hit, C.c_int32)),
               "pk_collide_noalloc" if noalloc else "pk_collide")
        return hit[:n].astype(bool), out[:n]
