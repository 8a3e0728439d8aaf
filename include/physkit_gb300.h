/*
 * physkit_gb300.h — C ABI of the GB300-native PhysKit world step.
 *
 * The reference has no plugin or operator interface; its drop-in seam is the virtual
 * world_base::step_impl(dt) (include/physkit/core/world.h:340, overridden by world at world.h:423
 * and implemented in src/world.cpp:20-56). This ABI is what a C++ `gpu_world : world_base`
 * override (or any FFI) binds: body creation/removal replaces world_base::create_rigid /
 * remove_rigid (world.h:202-218), pk_world_step replaces world_base::step's call of step_impl
 * (world.h:234-242), and the read-back calls replace get_rigid (world.h:220-224) and the
 * on_collision / on_collision_exit callbacks (world.h:327-338).
 *
 * Conventions: plain C types, caller-owned descriptors (copied), library-owned device memory,
 * int status returns (0 = PK_OK, negative = error), no exceptions across the ABI. One world
 * object is single-threaded like the reference (swappable_queue.h:13); distinct world objects
 * may be used from distinct threads. All device work of a world runs on its own CUDA stream.
 *
 * A world object may hold several independent sub-worlds ("worlds" below) that are stepped
 * together by the same launches (the batched form); max_worlds = 1 is the plain single world.
 */
#ifndef PHYSKIT_GB300_H
#define PHYSKIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PK_OK 0
#define PK_ERR_INVALID (-1)       /* bad argument (e.g. missing shape: object.h:121 throws) */
#define PK_ERR_STALE_HANDLE (-2)  /* handle generation mismatch (arena.h:234-244) */
#define PK_ERR_CAPACITY (-3)      /* a fixed capacity given at creation is exhausted */
#define PK_ERR_CUDA (-4)          /* a CUDA runtime call failed; pk_last_cuda_error() tells which */
#define PK_ERR_DEVICE_STATUS (-5) /* the step finished but flagged a status bit (pk_step_info.status) */
#define PK_ERR_NO_DEVICE (-6)     /* no CUDA device: this library has no CPU fallback */

/* pk_step_info.status bits */
#define PK_STATUS_PAIR_OVERFLOW 1   /* more overlap pairs than max_pairs: extra pairs dropped */
#define PK_STATUS_EPA_CAP 2         /* an EPA polytope hit the fixed face/horizon capacity */
#define PK_STATUS_COLOUR_CAP 4      /* more than 512 colouring rounds in one world */
#define PK_STATUS_TRAVERSAL_STACK 8 /* LBVH traversal stack overflow */
#define PK_STATUS_NAN 16            /* a non-finite position appeared */
#define PK_STATUS_CONTACT_OVERFLOW 32 /* more pairs with contacts (or in EPA) than max_contact_pairs */

enum
{
    PK_PRECISION_F64 = 0, /* FP64 throughout; arithmetic order identical to the FP64 oracle */
    PK_PRECISION_F32 = 1  /* FP32 state and geometry; FP64 accumulated impulses */
};
enum
{
    PK_BODY_DYNAMIC = 0, /* body_type::dynam (object.h:9-13) */
    PK_BODY_STATIC = 1   /* body_type::stat: infinite mass, never integrated (object.h:81-85) */
};

typedef struct pk_world pk_world;

typedef struct pk_world_desc
{
    double gravity[3];            /* world_desc gravity, default (0,-9.81,0): world.h:43-47 */
    int32_t solver_iterations;    /* world_desc solver_iterations, default 10: world.h:48 */
    int32_t precision;            /* PK_PRECISION_* */
    int32_t max_bodies;           /* body slots over all worlds */
    int32_t max_pairs;            /* broadphase pairs (0: 8 per body) */
    int32_t max_worlds;           /* independent worlds stepped together (1: plain world) */
    int32_t max_bodies_per_world; /* 0: max_bodies */
    int32_t max_shape_vertices;   /* 0: 65536 */
    int32_t max_shapes;           /* 0: 1024 */
    int32_t max_contact_pairs;    /* pairs with contact rows (and pairs in EPA) per step; 0: max_pairs.
                                     Contact rows take ~1 KB per pair, so a world with many more
                                     broadphase pairs than touching pairs sets this lower */
} pk_world_desc;

typedef struct pk_body_desc /* object_desc (object.h:15-109) */
{
    int32_t type;   /* PK_BODY_* */
    int32_t shape;  /* from pk_shape_*; object.h:61-65 (shared mesh) */
    int32_t world;  /* sub-world index, 0 for the plain world */
    int32_t reserved;
    double pos[3];
    double quat[4]; /* w, x, y, z (lin_alg.h:428-432) */
    double vel[3];
    double ang_vel[3];
    double mass;        /* ignored for static bodies (infinite) */
    double inertia[9];  /* local inertia tensor, row-major; inverted here like particle.h:126-131 */
    double restitution; /* default 0.5 (object.h:107) */
    double friction;    /* default 0.5 (object.h:108) */
} pk_body_desc;

typedef struct pk_step_info
{
    int32_t pairs;  /* broadphase pairs of the last step (all worlds) */
    int32_t leaves; /* bodies in the LBVH of the last step */
    int32_t status;   /* PK_STATUS_* bits seen since the previous synchronize */
    int32_t launches; /* kernels launched by one step */
    int32_t gjk;      /* pairs that reached GJK in the last step (after the bounding-sphere cull) */
    int32_t epa;      /* pairs that reached EPA (GJK found them intersecting) */
    int32_t gjk_large_mesh; /* of those, pairs involving a mesh above 32 vertices */
    int32_t epa_large_mesh;
    int64_t gjk_iterations; /* GJK iterations summed over the last step's pairs */
    int64_t epa_iterations; /* EPA expansions summed over the last step's pairs */
    int64_t epa_iterations_large_mesh;
    /* Vertices that linear support scans (mesh::support, mesh.cpp:341-358) visit for the last
     * step's supports (separating-axis pass, GJK, EPA expansions): x5 gives the reference's
     * support FLOPs. The device search visits fewer (vertex clusters, UV neighbourhoods). */
    int64_t support_vertices;
} pk_step_info;

/* Primitive shape for pk_collide: kind 0 aabb (p = min3 max3), 1 obb (p = center3 quat4 half3),
 * 2 mesh instance (p = pos3 quat4, shape = mesh id). */
typedef struct pk_collide_shape
{
    int32_t kind;
    int32_t shape;
    double p[10];
} pk_collide_shape;

void pk_world_desc_init(pk_world_desc *desc);
void pk_body_desc_init(pk_body_desc *desc);

/* world_base(world_desc) / world(world_desc) (world.h:188-190, 382-385). */
int pk_world_create(const pk_world_desc *desc, pk_world **out);
void pk_world_destroy(pk_world *w);

/* mesh::make / box / sphere / pyramid (mesh.h:219-236, mesh.cpp:16-137). Shapes are shared. */
int pk_shape_mesh(pk_world *w, const double *verts, int32_t nverts, const int32_t *tris, int32_t ntris,
                  int32_t *out_shape);
int pk_shape_box(pk_world *w, double hx, double hy, double hz, int32_t *out_shape);
int pk_shape_sphere(pk_world *w, double radius, int32_t stacks, int32_t sectors, int32_t *out_shape);
int pk_shape_pyramid(pk_world *w, double base_half, double height, int32_t *out_shape);

/* world_base::create_rigid (world.h:202-208) for n bodies; handles are arena ids
 * (slot | generation << 32, arena.h:179-206). Bodies join the broadphase with exact bounds. */
int pk_body_add(pk_world *w, const pk_body_desc *descs, int32_t n, uint64_t *out_handles);
/* world_base::remove_rigid (world.h:209-218): drops the body, its pairs and manifolds. */
int pk_body_remove(pk_world *w, uint64_t handle);
/* Retire a whole sub-world (all its bodies, pairs and manifolds) and free its slots for reuse. */
int pk_world_clear(pk_world *w, int32_t world);
/* Worlds that are not active sit out the following steps unchanged: no integration, and their
 * pairs and manifolds are carried over, so a world's trajectory depends only on how many steps it
 * took, not on which batched steps those were. */
int pk_world_set_active(pk_world *w, int32_t world, int32_t active);
/* One flag per world (n = max_worlds), enqueued on the world's stream (no synchronisation). */
int pk_world_set_active_mask(pk_world *w, const uint8_t *mask, int32_t n);
int pk_world_set_gravity(pk_world *w, int32_t world, const double gravity[3]);

/* One world step: world::step_impl (src/world.cpp:20-56) on the device. pk_world_step waits for
 * completion and returns PK_ERR_DEVICE_STATUS if a status bit was raised. */
int pk_world_step(pk_world *w, double dt);
int pk_world_step_async(pk_world *w, double dt);
int pk_world_synchronize(pk_world *w, pk_step_info *info);
/* Record the step for a fixed dt as CUDA graphs; pk_world_step_graph replays one step async. */
int pk_world_capture(pk_world *w, double dt);
int pk_world_step_graph(pk_world *w);
/* The CUDA stream (cudaStream_t) the world's work runs on. */
void *pk_world_stream(pk_world *w);

/* Stage timing: with timing on, plain (non-graph) steps record CUDA events around each stage;
 * pk_world_read_stage_times returns the summed milliseconds and step counts per stage since the
 * last read. The reference has no timers; this is the per-stage trace of the step. The first 9
 * rows are the step's stages in order; rows named "narrow:..." then split the narrowphase. */
int pk_world_set_timing(pk_world *w, int32_t enable);
int pk_world_read_stage_times(pk_world *w, double *total_ms, int32_t *counts, int32_t cap, int32_t *nstages);
const char *pk_stage_name(int32_t stage);

/* Autotuner: picks the launch shapes of the step (solver CTA size and the split between the
 * solver's large- and small-world launches, narrowphase grid, traversal block size) by timing
 * each stage over `steps_per_candidate` real steps per candidate; large worlds get their own
 * solver CTA size. These steps advance the world
 * like pk_world_step; launch shapes do not change results. Call before pk_world_capture. */
typedef struct pk_tune_result
{
    int32_t solve_threads;
    int32_t small_world;
    int32_t narrow_grid;
    int32_t traverse_threads;
    double step_ms_before; /* summed stage times per step before and after tuning */
    double step_ms_after;
    int32_t steps_used;
    int32_t big_threads; /* solver CTA size of the worlds above small_world (0: solve_threads) */
    int32_t group_bodies;  /* solve groups: worlds below small_world packed up to 8 per CTA while
                              their local indices sum to at most this (0: one world per CTA) */
    int32_t group_threads; /* CTA size of the solve groups (0: 128) */
    int32_t group_warp;    /* 1: at most one world per warp of a group, each swept by its warp */
} pk_tune_result;
int pk_world_autotune(pk_world *w, double dt, int32_t steps_per_candidate, pk_tune_result *out);
/* Apply launch shapes found by pk_world_autotune (e.g. on a scratch copy of the same scene). */
int pk_world_set_tuning(pk_world *w, const pk_tune_result *t);

/* Per slot: pos3 quat4 vel3 ang_vel3 alive = 14 doubles (particle.h:135-149). */
int pk_world_read_bodies(pk_world *w, double *out, int32_t cap_slots, int32_t *n_slots);
/* The same rows as of the steps enqueued so far, without waiting: they are packed on the world's
 * stream and copied out on a copy stream while later steps run, and land in `out` by the next
 * pk_world_synchronize (or pk_world_step). `out` must stay valid until then, and should be pinned
 * (pk_host_register) for the copy to overlap; two calls in flight use two staging buffers in turn. */
int pk_world_read_bodies_async(pk_world *w, double *out, int32_t cap_slots, int32_t *n_slots);
/* Page-lock (pin) a host buffer the caller reads into or writes from every step, so that
 * pk_world_read_bodies copies straight into it; unregister before freeing it. */
int pk_host_register(void *ptr, size_t bytes);
int pk_host_unregister(void *ptr);
/* PK_OK while the handle names a live body, PK_ERR_STALE_HANDLE after its removal: the arena's
 * generation check of get_rigid (arena.h:234-253), without touching the device. */
int pk_body_alive(pk_world *w, uint64_t handle);
/* Overwrite pos/quat/vel/ang_vel of one body and refresh its cached world inertia. */
int pk_world_write_body(pk_world *w, uint64_t handle, const double *state13);
/* Sorted broadphase pairs of the last step. keys use the reference layout
 * (min_local << 32 | max_local, collision_phases.h:63-69); worlds gives each pair's world. */
int pk_world_read_pairs(pk_world *w, uint64_t *keys, int32_t *worlds, int32_t cap, int32_t *n);
/* Manifolds of the last step in key order: 4 contacts x 13 doubles each
 * (normal3 local_a3 local_b3 depth normal_impulse tangent_impulse2), collision_phases.h:75-99. */
int pk_world_read_manifolds(pk_world *w, uint64_t *keys, int32_t *worlds, int32_t *counts, double *contacts,
                            int32_t cap, int32_t *n);
/* Begin (1) / end (2) collision events of the last step (collision_phases.h:309-318). */
int pk_world_read_events(pk_world *w, uint64_t *keys, int32_t *worlds, int32_t *kinds, int32_t cap, int32_t *n);
/* World raycast, replaces world_base::raycast (world.h:260-319), which walks the static and the
 * dynamic tree (bvh.h:402-450) and yields every body whose broadphase box the ray enters within
 * max_distance, with the entry distance (0 when the origin is inside; ray::intersect_distance,
 * bvh.h:62-93; the direction is normalised, bvh.h:47-50). The hit set is the reference's; the order
 * here is ascending (distance, handle) instead of its trees' depth-first order. For ray i,
 * handles/distances[i * cap + k] hold the min(counts[i], cap) nearest hits. Uses the body state after
 * the last step (or after any later add/remove): the tree is rebuilt over all worlds per call. */
typedef struct pk_ray
{
    double origin[3];
    double direction[3];
    double max_distance;
    int32_t world;
    int32_t reserved;
} pk_ray;
int pk_world_raycast(pk_world *w, const pk_ray *rays, int32_t n, int32_t cap, uint64_t *handles, double *distances,
                     int32_t *counts);
/* Ray against one mesh instance: mesh::instance::ray_intersect (mesh.cpp:400-415) over
 * mesh::ray_intersect (mesh.cpp:169-197) and ray::intersect (bvh.h:97-135, Moeller-Trumbore,
 * |a| < 1e-12 parallel). The ray goes into the body frame (its direction normalised, bvh.h:47-50),
 * the nearest triangle hit within max_distance is kept, and its point and normal come back in world
 * space. `body` names a live body (its shape and its pose after the last step); with
 * body = PK_HANDLE_ANY, `shape` and the pose given here are used (identity pose: the mesh's own
 * frame, mesh::ray_intersect). Triangles hit at exactly the same distance resolve to the later
 * triangle index; the reference takes the later one in its static BVH's visiting order. */
typedef struct pk_mesh_ray
{
    uint64_t body;
    int32_t shape;
    int32_t reserved;
    double pos[3];
    double quat[4]; /* w, x, y, z */
    double origin[3];
    double direction[3];
    double max_distance;
} pk_mesh_ray;
typedef struct pk_mesh_hit
{
    double pos[3];
    double normal[3];
    double distance;
    int32_t hit;      /* 1 on a hit */
    int32_t triangle; /* index of the triangle in the shape's triangle list */
} pk_mesh_hit;
int pk_mesh_raycast(pk_world *w, const pk_mesh_ray *rays, int32_t n, pk_mesh_hit *hits);

/* Joints, replacing constraint_solver::add_constraint / remove_constraint (constraint.h:1036-1049)
 * and the joint types of constraint.h:139-865, added through the world's command queue
 * (world.h:155-175). type: 0 distance (local_a, local_b, distance), 1 ball_socket (anchor, world
 * space), 2 hinge (local_a, local_b, axis_a, axis_b: local anchors and axes), 3 slider (anchor and
 * axis_a in world space), 4 weld (anchor, world space), 5 spring (local_a, local_b, distance,
 * stiffness, damping). Anchors given in world space are projected into both bodies at the call,
 * from their current poses, as the reference's constructors do. Joint rows are solved before the
 * contacts in every iteration, in the reference's order (per world: types in order, then arena
 * slots). Removing a body removes its joints (the reference leaves that to the caller). A step
 * graph captured before joints are added must be captured again. */
enum
{
    PK_JOINT_DISTANCE = 0,
    PK_JOINT_BALL_SOCKET = 1,
    PK_JOINT_HINGE = 2,
    PK_JOINT_SLIDER = 3,
    PK_JOINT_WELD = 4,
    PK_JOINT_SPRING = 5
};
typedef struct pk_joint_desc
{
    int32_t type;
    int32_t reserved;
    uint64_t a, b; /* body handles, same world */
    double anchor[3];
    double local_a[3], local_b[3];
    double axis_a[3], axis_b[3];
    double distance, stiffness, damping;
} pk_joint_desc;
void pk_joint_desc_init(pk_joint_desc *d);
int pk_joint_add(pk_world *w, const pk_joint_desc *d, uint64_t *out_handle);
int pk_joint_remove(pk_world *w, uint64_t handle);
/* Accumulated impulses of the joint's rows (up to 6) after the last step; nrows = its row count. */
int pk_joint_read_impulses(pk_world *w, uint64_t handle, double *out6, int32_t *nrows);

/* Waiting on collision events: the part of the reference's task handler that consumes them
 * (wait_for_collision / wait_for_separation / wait_until_destroyed, core/awaitables.h:136-300;
 * task_handler::on_collision, on_collision_exit, on_destruction, core/co.h:495-595). A waiter watches
 * one object for a begin (PK_WAIT_COLLISION) or end (PK_WAIT_SEPARATION) event with `with` or with
 * any object (PK_HANDLE_ANY), or for its removal (PK_WAIT_DESTROYED). pk_world_dispatch offers the
 * last step's events in pair-key order (each event to the first object's waiters, then the
 * second's; every matching waiter fires once and is removed) and returns the fired waiters; call it
 * after each step, before bodies are added or removed. Removing an object fails its collision and
 * separation waiters and those that name it as `with` (failed = 1) and fires its destruction
 * waiters. pk_world_wait returns PK_ERR_STALE_HANDLE for an object that is not alive (the
 * reference's await_ready resumes at once). */
#define PK_HANDLE_ANY UINT64_MAX
enum
{
    PK_WAIT_COLLISION = 1,
    PK_WAIT_SEPARATION = 2,
    PK_WAIT_DESTROYED = 3
};
typedef struct pk_wake
{
    uint64_t waiter;
    uint64_t object;
    uint64_t other; /* PK_HANDLE_ANY for destruction and failures */
    int32_t kind;
    int32_t failed;
} pk_wake;
int pk_world_wait(pk_world *w, int32_t kind, uint64_t object, uint64_t with, uint64_t *waiter);
int pk_world_cancel_wait(pk_world *w, uint64_t waiter);
int pk_world_dispatch(pk_world *w, pk_wake *out, int32_t cap, int32_t *n);
/* Solver colour of each manifold with contact rows in the last step (key order). */
int pk_world_read_colours(pk_world *w, uint64_t *keys, int32_t *colours, int32_t cap, int32_t *n,
                          int32_t *ncolours_world0);

/* Narrowphase (gjk_epa, collision.cpp:512-518) on n primitive shape pairs; out has 10 doubles per
 * pair: normal3 world_a3 world_b3 depth. hit[i] = 1 on collision. Returns PK_ERR_DEVICE_STATUS
 * (with every result written) when a pair's EPA hit a fixed capacity of this implementation (face,
 * horizon or flood-fill stack): that pair's result is the best face found so far, which can differ
 * from the reference's. The reference's own 64-expansion limit is not an error. */
int pk_collide(pk_world *w, const pk_collide_shape *a, const pk_collide_shape *b, int32_t n, double *out,
               int32_t *hit);

/* Allocation-free variant of pk_collide (this entry point has no counterpart in the reference).
 * For callers that cannot allocate device memory at call time: code running inside a strict
 * memory budget, or under an allocator that must not see per-call cudaMalloc/cudaFree. Nothing
 * is allocated: the device staging for the descriptors and results is a fixed array inside the
 * library, holding at most PK_COLLIDE_NOALLOC_MAX pairs (about 1 MiB, kept by every GPU that
 * loads the library until the process exits). Larger n returns PK_ERR_CAPACITY. Inputs and
 * outputs are the caller's host arrays, as for pk_collide, and the results are the same.
 * The first call on a device looks up the array's device address; make that first call before
 * any stream capture. All calls share the one array: calls whose GPU work overlaps (several
 * threads, or several world objects on one device) race and must be serialised by the caller.
 * The world's shapes must already be on the device (after a pk_body_add, a step or a pk_collide).
 * Call it with the device current on which the world was created (PK_ERR_INVALID otherwise); a
 * device reset ends the world and this cache with it. Capacity status as for pk_collide
 * (PK_ERR_DEVICE_STATUS with every result written). */
#define PK_COLLIDE_NOALLOC_MAX 4096
int pk_collide_noalloc(pk_world *w, const pk_collide_shape *a, const pk_collide_shape *b, int32_t n, double *out,
                       int32_t *hit);

/* Serving: continuous batching of step requests over one device-resident pool of worlds.
 * The reference steps one world per call (world_base::step, world.h:234-242); a server holding
 * many such worlds calls this instead. Worlds are admitted into slots of the pool (their state
 * stays on the device), each request asks for one step of one world, and pk_batch_step_async
 * enqueues one batched step of every world with a request not yet in flight, behind the steps
 * already enqueued (up to pipeline_depth), without waiting for the GPU. Admission, request and
 * retirement never wait for the GPU either: uploads are staged through pinned memory and ordered
 * behind the steps in flight. pk_batch_poll returns the requests whose steps have completed (and
 * the worlds retired) in completion order. A world sits out every batched step that does not
 * serve one of its requests, unchanged (pk_world_set_active), so its trajectory is the same alone
 * and in any mix. Admission is by device memory: with max_bodies 0 the pool takes
 * memory_fraction of the HBM free at creation, and a world that does not fit in what is left gets
 * PK_ERR_CAPACITY until a retirement frees room. One pk_batch is single-threaded. */
typedef struct pk_batch pk_batch;
typedef struct pk_batch_desc
{
    double gravity[3];
    double dt;                    /* the step every request asks for */
    int32_t solver_iterations;
    int32_t precision;            /* PK_PRECISION_* (default F32) */
    int32_t max_worlds;           /* world slots (default 1024) */
    int32_t max_bodies_per_world; /* default 4101 */
    int64_t max_bodies;           /* body pool; 0: from free device memory (memory_fraction) */
    double memory_fraction;       /* default 0.5 */
    int32_t pair_factor;          /* broadphase pairs per body of the pool (default 6) */
    int32_t contact_factor;       /* pairs with contact rows per body (default 2) */
    int32_t max_shapes, max_shape_vertices;
    int32_t pipeline_depth;       /* batched steps enqueued ahead of completion (default 1) */
    int32_t reserved;
} pk_batch_desc;
enum
{
    PK_BATCH_STEPPED = 1, /* the request `tag` of `world` got its step */
    PK_BATCH_RETIRED = 2  /* `world` was retired; its slot and bodies are free */
};
typedef struct pk_batch_event
{
    int64_t tag;
    int32_t world;
    int32_t kind;
} pk_batch_event;
typedef struct pk_batch_info
{
    int64_t pool_bodies, bodies_in_use, steps, pending_requests;
    int32_t worlds_live, worlds_free, steps_in_flight, reserved;
    int64_t graph_captures; /* the batched step is replayed from a CUDA graph, captured again after
                               admissions or retirements change the solver schedule */
} pk_batch_info;
void pk_batch_desc_init(pk_batch_desc *desc);
int pk_batch_create(const pk_batch_desc *desc, pk_batch **out);
void pk_batch_destroy(pk_batch *b);
/* The pool's world object: shapes (pk_shape_*) are made on it before admissions, and tuning
 * (pk_world_set_tuning) and read-backs go through it. */
pk_world *pk_batch_world(pk_batch *b);
/* Open a world of n bodies (their `world` field is ignored); returns its slot. */
int pk_batch_admit(pk_batch *b, const pk_body_desc *bodies, int32_t n, uint64_t *out_handles, int32_t *out_world);
int pk_batch_request(pk_batch *b, int32_t world, int64_t tag);
/* Retire a world once its pending requests are served (reported as PK_BATCH_RETIRED). */
int pk_batch_retire(pk_batch *b, int32_t world);
int pk_batch_step_async(pk_batch *b, int32_t *nworlds);
/* Completed requests and retirements, up to cap; wait = 1 first waits for the oldest step in flight. */
int pk_batch_poll(pk_batch *b, pk_batch_event *out, int32_t cap, int32_t *n, int32_t wait);
int pk_batch_stats(pk_batch *b, pk_batch_info *st);
/* State rows (14 doubles, as pk_world_read_bodies) of one world's live bodies in creation order;
 * waits for the steps in flight. */
int pk_batch_read_world(pk_batch *b, int32_t world, double *out14, int32_t cap, int32_t *n);

int pk_last_cuda_error(void);
const char *pk_version(void);

#ifdef __cplusplus
}
#endif
#endif
