// pk_engine_api.h — precision-independent interface between the C ABI layer and the device engine.
#pragma once

#include <cstdint>
#include <vector>

namespace pk
{

struct EngineConfig
{
    int body_cap = 0;
    int pair_cap = 0;
    int contact_cap = 0; // pairs with contact rows per step (0: pair_cap)
    int max_worlds = 1;
    int vert_cap = 0;
    int shape_cap = 0;
    int iterations = 10;
    int lbits = 1;   // bits of a world-local body index in pair keys
    int wbits = 1;   // bits of a world index in Morton keys (max_worlds itself must fit)
    int sort_blocks_bodies = 1;
    int sort_blocks_pairs = 1;
};

// One body as the host staged it (double precision; converted to the engine's scalar on upload).
struct HostBody
{
    int world, local, shape, flags, created;
    double pos[3], quat[4], vel[3], ang_vel[3];
    double mass, inv_mass, restitution, friction;
    double il[9], il_inv[9];
};

// Launch shapes chosen at run time (by pk_world_autotune or left at these defaults). They do not
// change results: colour-parallel solver updates are independent and the other kernels are
// per-element.
struct Tunables
{
    int solve_threads = 256;   // threads per solver CTA (one CTA per world)
    int small_world = 512;     // worlds up to this many local indices share the small solver launch
    int narrow_grid = 2;       // GJK/EPA grid = narrow_grid x the default grid
    int traverse_threads = 128;
    int big_threads = 256;     // threads per solver CTA of the worlds above small_world
    int group_bodies = 0;      // solve groups: worlds packed up to 8 per CTA while their local
    int group_threads = 128;   // indices sum to at most group_bodies (0: one world per CTA)
    int group_warp = 0;        // 1: one member per warp, each swept by its own warp
};

struct StepCounters
{
    int npairs = 0;
    int nleaf = 0;
    int status = 0;
    int launches = 0; // kernels one step launches
    int gjk = 0, gjk_heavy = 0, epa = 0, epa_heavy = 0; // narrowphase work items of the last step
    long long gjk_iters = 0, epa_iters = 0, epa_iters_heavy = 0;
    long long support_verts = 0; // vertices linear support scans would visit (separating axis, GJK, EPA)
};

// A ray against one mesh instance (pk_mesh_raycast): the body's slot (its shape and current pose
// on the device), or slot -1 with the shape and pose given here.
struct MeshRayIn
{
    int slot, shape;
    double pos[3], q[4], o[3], d[3], maxd;
};
struct MeshHitOut
{
    double pos[3], normal[3], distance;
    int32_t hit, triangle;
};

constexpr int kStages = 9;     // the step's stages, in order (they sum to the step)
constexpr int kStageRows = 13; // then the narrowphase's parts: pre-pass, separating axis, GJK, EPA
extern const char *const kStageNames[kStageRows];

class EngineBase
{
public:
    virtual ~EngineBase() = default;
    virtual int precision_bits() const = 0;
    virtual int init(const EngineConfig &cfg) = 0;
    // ranges: 8 ints per shape (vertex start/count, cluster start/count, group start/count, 2 pad);
    // clusters: 4 doubles per record (centre, radius), vertex blocks and groups of blocks;
    // rmax: bounding radius per shape.
    virtual int set_shapes(const std::vector<double> &verts, const std::vector<int> &ranges,
                           const std::vector<double> &boxes, const std::vector<double> &clusters,
                           const std::vector<double> &rmax) = 0;
    virtual int set_world(int w, const double g[3], double gnorm, int active) = 0;
    virtual int upload_bodies(const int *slots, const HostBody *b, int n, int nslots) = 0;
    virtual int kill_body(int slot, int world, int local) = 0;
    virtual int kill_world(const int *slots, int n, int world) = 0; // all bodies of a world at once
    virtual int set_active_mask(const uint8_t *mask, int n) = 0;    // stream-ordered, no sync
    // solver schedule (largest worlds first) and local indices in use per world
    virtual int set_world_order(const int *order, const int *nlocal, int n) = 0;
    // The same four updates without waiting for the GPU (pinned staging, stream-ordered behind the
    // work already enqueued): the serving loop changes worlds while earlier steps run.
    virtual int upload_bodies_async(const int *slots, const HostBody *b, int n, int nslots) = 0;
    virtual int kill_world_async(const int *slots, int n, int world) = 0;
    virtual int set_active_mask_async(const uint8_t *mask, int n) = 0;
    virtual int set_world_order_async(const int *order, const int *nlocal, int n) = 0;
    virtual int step(double dt) = 0;                 // enqueue only
    virtual int synchronize(StepCounters *c) = 0;   // wait + read counters, clears status
    virtual int read_bodies(double *out14, int nslots) = 0;
    // the same rows packed after the work enqueued so far and copied on a copy stream: the call
    // returns at once and the rows land by the next synchronize (out stays valid until then)
    virtual int read_bodies_async(double *out14, int nslots) = 0;
    virtual int write_state(int slot, const double *state13) = 0;
    virtual int read_pairs(uint64_t *keys, uint64_t *slots, int cap) = 0;
    virtual int read_manifolds(uint64_t *keys, int *counts, double *contacts13, int cap) = 0;
    virtual int read_events(uint64_t *keys, int *kinds, int cap) = 0;
    virtual int read_colours(uint64_t *keys, int *colours, int cap, int *ncolours_world0) = 0;
    virtual int collide(const void *specs_a, const void *specs_b, int n, double *out, int *hit, int *status) = 0;
    virtual int set_joints(const int *ints, const double *params, const double *acc, int n, const int *jstart,
                           const int *jend) = 0;
    virtual int read_joint_acc(double *acc, int n) = 0;
    virtual int read_pose(int slot, double *out7) = 0;
    // rays: 8 doubles each (origin, direction, distance limit, world); per ray up to `cap` nearest
    // hits (device slot, distance) ordered by (distance, slot), and the total hit count
    virtual int raycast(const double *rays, int n, int cap, int *counts, int *slots, double *dists) = 0;
    // triangles of every shape (3 vertex indices within the shape each) and each shape's range
    virtual int set_triangles(const std::vector<int> &tris, const std::vector<int> &range) = 0;
    virtual int mesh_raycast(const MeshRayIn *rays, int n, MeshHitOut *out) = 0;
    // The narrowphase launch of collide on device buffers the caller provides; allocates nothing.
    // status_any_dev (may be null): OR of every pair's status bits
    virtual int collide_device(const void *specs_a_dev, const void *specs_b_dev, int n, double *out_dev,
                               int *hit_dev, int *status_dev, int *status_any_dev) = 0;
    virtual int capture_graph(double dt) = 0;        // record the step as CUDA graphs
    virtual int launch_graph() = 0;                  // replay one captured step
    virtual void *stream() = 0;
    virtual int set_timing(int enable) = 0;                 // CUDA events around each stage
    virtual int read_stage_times(double *ms, int *count) = 0; // totals since the last read
    virtual int set_tunables(const Tunables &t) = 0;
    virtual Tunables tunables() const = 0;
    virtual int last_error() const = 0;
};

EngineBase *make_engine_f64();
EngineBase *make_engine_f32();

} // namespace pk
