"""ctypes binding of the FP64 CPU oracle (test infrastructure only).

Loaded by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py. It builds
oracle/_build/libpk_oracle.so on first use (g++ only, no GPU needed).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build as _build  # noqa: E402

_lib = None
D3 = C.c_double * 3
P = C.POINTER


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp, ip, up = P(C.c_double), P(C.c_int), P(C.c_uint64)
        u32p = P(C.c_uint32)
        sig = {
            "pko_world_create": (C.c_void_p, [C.c_double] * 3 + [C.c_int, C.c_int]),
            "pko_world_destroy": (None, [C.c_void_p]),
            "pko_shape_box": (C.c_int, [C.c_void_p] + [C.c_double] * 3),
            "pko_shape_sphere": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int]),
            "pko_shape_pyramid": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
            "pko_shape_mesh": (C.c_int, [C.c_void_p, dp, C.c_int, ip, C.c_int]),
            "pko_shape_vertex_count": (C.c_int, [C.c_void_p, C.c_int]),
            "pko_shape_triangles": (C.c_int, [C.c_void_p, C.c_int, ip, C.c_int]),
            "pko_shape_vertices": (C.c_int, [C.c_void_p, C.c_int, dp, C.c_int]),
            "pko_shape_volume": (C.c_double, [C.c_void_p, C.c_int]),
            "pko_body_add": (C.c_uint64, [C.c_void_p, C.c_int, dp, dp, dp, dp, C.c_double, dp,
                                          C.c_double, C.c_double, C.c_int]),
            "pko_body_remove": (C.c_int, [C.c_void_p, C.c_uint64]),
            "pko_body_count": (C.c_int, [C.c_void_p]),
            "pko_world_step": (None, [C.c_void_p, C.c_double]),
            "pko_read_bodies": (C.c_int, [C.c_void_p, dp, C.c_int]),
            "pko_write_body_state": (C.c_int, [C.c_void_p, C.c_int, dp]),
            "pko_read_pairs": (C.c_int, [C.c_void_p, up, C.c_int]),
            "pko_read_manifolds": (C.c_int, [C.c_void_p, up, ip, dp, C.c_int]),
            "pko_read_events": (C.c_int, [C.c_void_p, up, ip, C.c_int]),
            "pko_world_raycast": (C.c_int, [C.c_void_p, dp, dp, C.c_double, up, dp, C.c_int]),
            "pko_mesh_raycast": (C.c_int, [C.c_void_p, C.c_int, dp, dp, dp, C.c_double, dp, ip]),
            "pko_joint_add": (C.c_uint64, [C.c_void_p, C.c_int, C.c_uint64, C.c_uint64, dp]),
            "pko_joint_remove": (C.c_int, [C.c_void_p, C.c_uint64]),
            "pko_joint_impulses": (C.c_int, [C.c_void_p, C.c_uint64, dp]),
            "pko_read_colours": (C.c_int, [C.c_void_p, up, ip, C.c_int, ip]),
            "pko_last_moved": (C.c_int, [C.c_void_p]),
            "pko_gjk_epa": (C.c_int, [C.c_void_p, C.c_int, dp, C.c_int, C.c_int, dp, C.c_int, dp]),
            "pko_tree_create": (C.c_void_p, []),
            "pko_tree_destroy": (None, [C.c_void_p]),
            "pko_tree_add": (C.c_uint32, [C.c_void_p, C.c_uint32, dp]),
            "pko_tree_update": (C.c_int, [C.c_void_p, C.c_uint32, dp, dp]),
            "pko_tree_remove": (None, [C.c_void_p, C.c_uint32]),
            "pko_tree_bounds": (None, [C.c_void_p, C.c_uint32, dp]),
            "pko_tree_query": (C.c_int, [C.c_void_p, dp, u32p, C.c_int]),
            "pko_tree_height": (C.c_int, [C.c_void_p]),
            "pko_tree_validate": (C.c_int, [C.c_void_p]),
            "pko_sincos": (None, [C.c_double, dp, dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(P(C.c_double))


def quat_angle_axis(angle, axis):
    """Eigen AngleAxis -> quaternion (w, x, y, z): (cos(a/2), sin(a/2) * axis)."""
    h = 0.5 * angle
    s = math.sin(h)
    return [math.cos(h), s * axis[0], s * axis[1], s * axis[2]]


class OracleWorld:
    """One reference-semantics world (world_desc + world, world.h:23-49, 379-425)."""

    def __init__(self, gravity=(0.0, -9.81, 0.0), iterations=10, order="key"):
        self.L = lib()
        self.h = self.L.pko_world_create(*map(float, gravity), int(iterations),
                                         0 if order == "key" else 1)

    def close(self):
        if self.h:
            self.L.pko_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # shapes ---------------------------------------------------------------------------------
    def box(self, hx, hy, hz):
        return self.L.pko_shape_box(self.h, hx, hy, hz)

    def sphere(self, r, stacks=16, sectors=32):
        return self.L.pko_shape_sphere(self.h, r, stacks, sectors)

    def pyramid(self, b, h):
        return self.L.pko_shape_pyramid(self.h, b, h)

    def mesh(self, verts, tris):
        v, vp = _dp(np.asarray(verts).reshape(-1))
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.int32).reshape(-1))
        return self.L.pko_shape_mesh(self.h, vp, len(v) // 3,
                                     t.ctypes.data_as(P(C.c_int)), len(t) // 3)

    def vertices(self, shape):
        n = self.L.pko_shape_vertex_count(self.h, shape)
        out = np.zeros(3 * n)
        self.L.pko_shape_vertices(self.h, shape, out.ctypes.data_as(P(C.c_double)), n)
        return out.reshape(n, 3)

    def triangles(self, shape):
        n = self.L.pko_shape_triangles(self.h, shape, None, 0)
        out = np.zeros(3 * max(n, 1), dtype=np.int32)
        self.L.pko_shape_triangles(self.h, shape, out.ctypes.data_as(P(C.c_int)), n)
        return out[: 3 * n].reshape(n, 3)

    def volume(self, shape):
        return self.L.pko_shape_volume(self.h, shape)

    # bodies ---------------------------------------------------------------------------------
    def add(self, shape, pos, quat=(1, 0, 0, 0), vel=(0, 0, 0), ang_vel=(0, 0, 0), mass=1.0,
            inertia=None, restitution=0.5, friction=0.5, static=False):
        if inertia is None:
            inertia = np.eye(3)
        inertia = np.asarray(inertia, dtype=np.float64)
        if inertia.shape == (3,):
            inertia = np.diag(inertia)
        arrs = [_dp(x) for x in (pos, quat, vel, ang_vel, inertia.reshape(-1))]
        return self.L.pko_body_add(self.h, int(bool(static)), arrs[0][1], arrs[1][1], arrs[2][1],
                                   arrs[3][1], float(mass), arrs[4][1], float(restitution),
                                   float(friction), int(shape))

    def remove(self, handle):
        return bool(self.L.pko_body_remove(self.h, C.c_uint64(handle)))

    def step(self, dt):
        self.L.pko_world_step(self.h, float(dt))

    def bodies(self):
        n = self.L.pko_body_count(self.h)
        out = np.zeros(14 * max(n, 1))
        self.L.pko_read_bodies(self.h, out.ctypes.data_as(P(C.c_double)), n)
        return out[: 14 * n].reshape(n, 14)

    def write_state(self, slot, state13):
        a, p = _dp(state13)
        return self.L.pko_write_body_state(self.h, int(slot), p)

    def pairs(self):
        n = self.L.pko_read_pairs(self.h, None, 0)
        out = np.zeros(max(n, 1), dtype=np.uint64)
        self.L.pko_read_pairs(self.h, out.ctypes.data_as(P(C.c_uint64)), n)
        return out[:n]

    def manifolds(self):
        n = self.L.pko_read_manifolds(self.h, None, None, None, 0)
        keys = np.zeros(max(n, 1), dtype=np.uint64)
        counts = np.zeros(max(n, 1), dtype=np.int32)
        contacts = np.zeros((max(n, 1), 4, 13))
        self.L.pko_read_manifolds(self.h, keys.ctypes.data_as(P(C.c_uint64)),
                                  counts.ctypes.data_as(P(C.c_int)),
                                  contacts.ctypes.data_as(P(C.c_double)), n)
        return keys[:n], counts[:n], contacts[:n]

    def events(self):
        n = self.L.pko_read_events(self.h, None, None, 0)
        keys = np.zeros(max(n, 1), dtype=np.uint64)
        kinds = np.zeros(max(n, 1), dtype=np.int32)
        self.L.pko_read_events(self.h, keys.ctypes.data_as(P(C.c_uint64)),
                               kinds.ctypes.data_as(P(C.c_int)), n)
        return keys[:n], kinds[:n]

    def colours(self):
        nc = C.c_int(0)
        n = self.L.pko_read_colours(self.h, None, None, 0, C.byref(nc))
        keys = np.zeros(max(n, 1), dtype=np.uint64)
        cols = np.zeros(max(n, 1), dtype=np.int32)
        self.L.pko_read_colours(self.h, keys.ctypes.data_as(P(C.c_uint64)),
                                cols.ctypes.data_as(P(C.c_int)), n, C.byref(nc))
        return keys[:n], cols[:n], nc.value

    def last_moved(self):
        return self.L.pko_last_moved(self.h)

    JOINT_TYPES = {"distance": 0, "ball_socket": 1, "hinge": 2, "slider": 3, "weld": 4, "spring": 5}

    def add_joint(self, kind, a, b, anchor=(0, 0, 0), local_a=(0, 0, 0), local_b=(0, 0, 0), axis_a=(0, 0, 0),
                  axis_b=(0, 0, 0), distance=0.0, stiffness=0.0, damping=0.0):
        """constraint_solver::add_constraint (constraint.h:1036-1041); returns the joint handle."""
        p, pp = _dp(list(anchor) + list(local_a) + list(local_b) + list(axis_a) + list(axis_b) +
                    [distance, stiffness, damping])
        return self.L.pko_joint_add(self.h, self.JOINT_TYPES[kind], int(a), int(b), pp)

    def remove_joint(self, handle):
        return bool(self.L.pko_joint_remove(self.h, int(handle)))

    def joint_impulses(self, handle):
        out, op = _dp(np.zeros(6))
        n = self.L.pko_joint_impulses(self.h, int(handle), op)
        return out[:max(n, 0)]

    def mesh_raycast(self, shape, pose7, origin, direction, max_dist):
        """mesh::instance::ray_intersect of `shape` at pose7 (pos, quat wxyz): None or
        (pos3, normal3, distance, triangle)."""
        p, pp = _dp(pose7)
        o, op = _dp(origin)
        d, dp_ = _dp(direction)
        out = np.zeros(7)
        tri = C.c_int()
        if not self.L.pko_mesh_raycast(self.h, int(shape), pp, op, dp_, float(max_dist),
                                       out.ctypes.data_as(P(C.c_double)), C.byref(tri)):
            return None
        return out[0:3].copy(), out[3:6].copy(), float(out[6]), tri.value

    def raycast(self, origin, direction, max_dist):
        """world_base::raycast (world.h:260-319): [(handle, distance)] in the reference's order."""
        o, op = _dp(origin)
        dv, dp_ = _dp(direction)
        n = self.L.pko_world_raycast(self.h, op, dp_, float(max_dist), None, None, 0)
        hs = np.zeros(max(n, 1), dtype=np.uint64)
        ds = np.zeros(max(n, 1))
        self.L.pko_world_raycast(self.h, op, dp_, float(max_dist), hs.ctypes.data_as(P(C.c_uint64)),
                                 ds.ctypes.data_as(P(C.c_double)), n)
        return list(zip(hs[:n].tolist(), ds[:n].tolist()))

    # narrowphase on primitive shapes ---------------------------------------------------------
    def shape_params(self, spec):
        """Known-answer shape spec -> (kind, params, shape id)."""
        kind = spec[0]
        if kind == "aabb":
            return 0, list(spec[1]) + list(spec[2]), -1
        q = [1.0, 0.0, 0.0, 0.0] if spec[-1] is None and kind == "mesh" else None
        if kind == "obb":
            rot = spec[2]
            q = [1.0, 0.0, 0.0, 0.0] if rot is None else quat_angle_axis(rot[0], rot[1])
            return 1, list(spec[1]) + q + list(spec[3]), -1
        ms = spec[1]
        if ms[0] == "box":
            sid = self.box(*ms[1:4])
        elif ms[0] == "sphere":
            sid = self.sphere(ms[1])
        else:
            sid = self.pyramid(ms[1], ms[2])
        rot = spec[3]
        q = [1.0, 0.0, 0.0, 0.0] if rot is None else quat_angle_axis(rot[0], rot[1])
        return 2, list(spec[2]) + q, sid

    def gjk_epa(self, spec_a, spec_b):
        ka, pa, sa = self.shape_params(spec_a)
        kb, pb, sb = self.shape_params(spec_b)
        a, ap = _dp(pa)
        b, bp = _dp(pb)
        out = np.zeros(10)
        hit = self.L.pko_gjk_epa(self.h, ka, ap, sa, kb, bp, sb, out.ctypes.data_as(P(C.c_double)))
        if not hit:
            return None
        return {"normal": out[0:3], "world_a": out[3:6], "world_b": out[6:9], "depth": out[9]}


class OracleTree:
    """The reference's dynamic AABB tree (bvh.h:270-535) for its own known answers."""

    def __init__(self):
        self.L = lib()
        self.h = self.L.pko_tree_create()

    def __del__(self):
        try:
            self.L.pko_tree_destroy(self.h)
        except Exception:
            pass

    def add(self, oid, box6):
        b, bp = _dp(box6)
        return self.L.pko_tree_add(self.h, oid, bp)

    def update(self, leaf, box6, disp):
        b, bp = _dp(box6)
        d, dp_ = _dp(disp)
        return bool(self.L.pko_tree_update(self.h, leaf, bp, dp_))

    def remove(self, leaf):
        self.L.pko_tree_remove(self.h, leaf)

    def bounds(self, leaf):
        out = np.zeros(6)
        self.L.pko_tree_bounds(self.h, leaf, out.ctypes.data_as(P(C.c_double)))
        return out

    def query(self, box6):
        b, bp = _dp(box6)
        n = self.L.pko_tree_query(self.h, bp, None, 0)
        out = np.zeros(max(n, 1), dtype=np.uint32)
        self.L.pko_tree_query(self.h, bp, out.ctypes.data_as(P(C.c_uint32)), n)
        return out[:n]

    def height(self):
        return self.L.pko_tree_height(self.h)

    def validate(self):
        return bool(self.L.pko_tree_validate(self.h))


def sincos(x):
    s, c = C.c_double(), C.c_double()
    lib().pko_sincos(float(x), C.byref(s), C.byref(c))
    return s.value, c.value


def load_scene(ow: "OracleWorld", scene):
    """Create a physkit_gb300.scenes.Scene (one world) in an oracle world, in record order."""
    ids = []
    for s in scene.shapes:
        if s[0] == "box":
            ids.append(ow.box(*s[1:4]))
        elif s[0] == "sphere":
            ids.append(ow.sphere(s[1], s[2], s[3]))
        elif s[0] == "pyramid":
            ids.append(ow.pyramid(s[1], s[2]))
        else:
            ids.append(ow.mesh(s[1], s[2]))
    handles = []
    for r in scene.bodies:
        handles.append(ow.add(ids[int(r["shape"])], r["pos"], r["quat"], r["vel"], r["ang_vel"],
                              float(r["mass"]), np.asarray(r["inertia"]).reshape(3, 3),
                              float(r["restitution"]), float(r["friction"]), static=bool(r["type"] == 1)))
    return handles
