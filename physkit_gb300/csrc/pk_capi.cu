// pk_capi.cu — the C ABI (include/physkit_gb300.h) over the device engine.
//
// Host-side bookkeeping mirrors the reference's world_base: each sub-world owns a generational
// arena of local indices (detail/arena.h:169-267: a free stack of indices, generations bumped on
// removal), and the local index is what pair keys are built from (world.h:206). Each local index
// of a world is bound to one device slot for its lifetime, so results do not depend on where in
// device memory a world lives.
#include "../../include/physkit_gb300.h"
#include "pk_engine_api.h"
#include "pk_events.h"
#include "pk_narrow.cuh"
#include "pk_math.cuh"

#include <algorithm>
#include <deque>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

#include <cuda_runtime.h>

namespace pk
{
const char *const kStageNames[kStageRows] = {"integrate_vel", "morton_sort",   "lbvh_build_refit", "traverse",
                                             "pair_sort",     "narrow",        "contact_setup",    "solve",
                                             "integrate_pos", "narrow:pre",    "narrow:axis",      "narrow:gjk",
                                             "narrow:epa"};
}

namespace
{
int g_last_cuda = 0;

struct SlotInfo
{
    int world = -1;
    int local = -1;
    uint32_t gen = 0;
    bool alive = false;
    bool is_static = false;
};

struct SubWorld
{
    std::vector<int> local_slot;   // local index -> device slot (-1 when never bound)
    std::vector<uint32_t> local_gen;
    std::vector<int> free_locals;  // arena free stack (arena.h:208-232)
    std::vector<char> local_alive;
    double gravity[3] = {0.0, -9.81, 0.0};
    int active = 1;
    // joint arenas, one per constraint type (constraint.h:969-1020): slot -> joint index or -1
    std::vector<int> jslot[6];
    std::vector<uint32_t> jgen[6];
    std::vector<int> jfree[6];
};

struct JointHost
{
    int type = 0, world = 0, arena = 0;
    int slot_a = 0, slot_b = 0, local_a = 0, local_b = 0;
    double p[25] = {}; // la3 lb3 axa3 axb3 va3 wa3 qrel4 distance stiffness damping
    double acc[6] = {};
    bool alive = false;
};

int bits_for(long long v)
{
    int b = 1;
    while ((1LL << b) < v) ++b;
    return b;
}
} // namespace

struct pk_world
{
    pk::EngineBase *eng = nullptr;
    pk::EngineConfig cfg;
    pk_world_desc desc;
    std::vector<double> verts;   // all shape vertices
    std::vector<int> ranges;     // 8 ints per shape: vertices, clusters, groups (start, count), 2 pad
    std::vector<double> clusters; // (centre xyz, radius) per cluster of 8 consecutive vertices
    std::vector<double> rmax;     // bounding radius of each shape about its origin
    std::vector<double> boxes;   // local aabb per shape
    std::vector<int> tris;       // triangles of all shapes (vertex indices within the shape)
    std::vector<int> tri_range;  // per shape: first triangle, triangle count
    std::vector<SubWorld> worlds;
    std::vector<SlotInfo> slots;
    std::vector<int> free_slots;
    int nslots = 0;
    int steps = 0;
    bool shapes_dirty = false;
    bool order_dirty = false; // solver schedule needs recomputing (bodies added or removed)
    std::vector<JointHost> joints; // every joint ever added (dead ones keep their index)
    std::vector<int> joint_order;  // joints as last uploaded, in (world, type, arena slot) order
    bool joints_dirty = false;
    pk::EventDispatcher waiters; // collision / separation / destruction waiters (pk_world_wait)
    std::vector<pk::Wake> wakes; // fired, not yet returned by pk_world_dispatch
    size_t wake_head = 0;
    int dispatched_step = 0;     // host step whose events were last offered to the waiters
    int device = 0;              // CUDA device current at pk_world_create: its stream and buffers live there
    int launch_version = 0;      // bumped when launch shapes change (a captured step graph is stale)
};

// Allocation-free narrowphase (pk_collide_noalloc). Its device staging lives in this file-scope
// array instead of memory from cudaMalloc: pair descriptors in, results out, for at most
// PK_COLLIDE_NOALLOC_MAX pairs per call. Every GPU that loads this library holds the array
// (about 1 MiB) until the process exits.
namespace
{
constexpr int kNoAllocMax = PK_COLLIDE_NOALLOC_MAX;
constexpr size_t kNoAllocSpecs = sizeof(pk_collide_shape) * kNoAllocMax; // one side's descriptors
constexpr size_t kNoAllocOut = sizeof(double) * 10 * kNoAllocMax;
constexpr size_t kNoAllocInts = sizeof(int32_t) * kNoAllocMax;
// + 256 bytes at the end: the OR of every pair's status bits
constexpr size_t kNoAllocBytes = 2 * kNoAllocSpecs + kNoAllocOut + 2 * kNoAllocInts + 256;
} // namespace

static __device__ __align__(256) unsigned char g_collide_scratch[kNoAllocBytes];

namespace
{
// Device address of g_collide_scratch, looked up once per device (with that device current):
// in host code the array's name is only a host-side stand-in, not a device address.
constexpr int kMaxDevices = 64;
unsigned char *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// The world's stream and shape tables live on the device that was current at pk_world_create, so
// the call must run with that device current; any other current device is PK_ERR_INVALID.
int scratch_for_world_device(int world_device, unsigned char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    if (dev != world_device || dev < 0 || dev >= kMaxDevices) return PK_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev])
    {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_collide_scratch);
        if (e != cudaSuccess)
        {
            g_last_cuda = int(e);
            return PK_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return PK_OK;
}
} // namespace

extern "C" {

void pk_world_desc_init(pk_world_desc *d)
{
    std::memset(d, 0, sizeof(*d));
    d->gravity[0] = 0.0;
    d->gravity[1] = -9.81;
    d->gravity[2] = 0.0;
    d->solver_iterations = 10;
    d->precision = PK_PRECISION_F64;
    d->max_bodies = 4096;
    d->max_pairs = 0;
    d->max_worlds = 1;
    d->max_bodies_per_world = 0;
    d->max_shape_vertices = 0;
    d->max_shapes = 0;
}

void pk_body_desc_init(pk_body_desc *d)
{
    std::memset(d, 0, sizeof(*d));
    d->type = PK_BODY_DYNAMIC;
    d->quat[0] = 1.0;
    d->mass = 1.0;
    d->inertia[0] = d->inertia[4] = d->inertia[8] = 1.0;
    d->restitution = 0.5;
    d->friction = 0.5;
}

int pk_collide_noalloc(pk_world *w, const pk_collide_shape *a, const pk_collide_shape *b, int32_t n, double *out,
                       int32_t *hit)
{
    if (!w || n < 0 || (n > 0 && (!a || !b || !out || !hit))) return PK_ERR_INVALID;
    if (n > kNoAllocMax) return PK_ERR_CAPACITY; // larger batches: split them, or use pk_collide
    int nshapes = int(w->ranges.size() / 8);
    for (int i = 0; i < n; ++i)
        for (const pk_collide_shape *s : {a + i, b + i})
        {
            if (s->kind < 0 || s->kind > 2) return PK_ERR_INVALID;
            if (s->kind == 2 && (s->shape < 0 || s->shape >= nshapes)) return PK_ERR_INVALID;
        }
    if (n == 0) return PK_OK;
    if (w->shapes_dirty) return PK_ERR_INVALID; // shapes are uploaded by a step, a body add or pk_collide first
    unsigned char *base = nullptr;
    if (int rc = scratch_for_world_device(w->device, &base)) return rc;
    unsigned char *da = base, *db = base + kNoAllocSpecs;
    double *dout = reinterpret_cast<double *>(base + 2 * kNoAllocSpecs);
    int32_t *dhit = reinterpret_cast<int32_t *>(base + 2 * kNoAllocSpecs + kNoAllocOut);
    int32_t *dst = dhit + kNoAllocMax;
    int32_t *dany = dst + kNoAllocMax;
    cudaStream_t st = static_cast<cudaStream_t>(w->eng->stream());
    size_t spec_bytes = sizeof(pk_collide_shape) * size_t(n);
    int32_t any = 0; // copied back into this stack variable: nothing is allocated, on the host either
    cudaError_t e;
    if ((e = cudaMemcpyAsync(da, a, spec_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(db, b, spec_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        // the array keeps the previous call's results: misses leave `out` untouched, so clear it,
        // and the status word must start at zero
        (e = cudaMemsetAsync(dout, 0, sizeof(double) * 10 * size_t(n), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(dany, 0, sizeof(int32_t), st)) != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    if (w->eng->collide_device(da, db, n, dout, dhit, dst, dany))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    if ((e = cudaMemcpyAsync(out, dout, sizeof(double) * 10 * size_t(n), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(hit, dhit, sizeof(int32_t) * size_t(n), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&any, dany, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    return any ? PK_ERR_DEVICE_STATUS : PK_OK;
}

int pk_last_cuda_error(void) { return g_last_cuda; }
const char *pk_version(void) { return "physkit_gb300 0.1.0 (sm_103a)"; }

int pk_world_create(const pk_world_desc *desc, pk_world **out)
{
    if (!desc || !out) return PK_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
    {
        g_last_cuda = int(e);
        return PK_ERR_NO_DEVICE;
    }
    if (desc->max_bodies <= 0 || desc->max_worlds <= 0 || desc->solver_iterations < 0 || desc->max_contact_pairs < 0)
        return PK_ERR_INVALID;
    if (desc->precision != PK_PRECISION_F64 && desc->precision != PK_PRECISION_F32) return PK_ERR_INVALID;
    auto *w = new (std::nothrow) pk_world;
    if (!w) return PK_ERR_CAPACITY;
    w->desc = *desc;
    pk::EngineConfig &c = w->cfg;
    c.body_cap = desc->max_bodies;
    c.pair_cap = desc->max_pairs > 0 ? desc->max_pairs : 8 * desc->max_bodies;
    c.contact_cap = desc->max_contact_pairs > 0 && desc->max_contact_pairs < c.pair_cap ? desc->max_contact_pairs
                                                                                        : c.pair_cap;
    c.max_worlds = desc->max_worlds;
    c.vert_cap = desc->max_shape_vertices > 0 ? desc->max_shape_vertices : 65536;
    c.shape_cap = desc->max_shapes > 0 ? desc->max_shapes : 1024;
    c.iterations = desc->solver_iterations;
    int per_world = desc->max_bodies_per_world > 0 ? desc->max_bodies_per_world : desc->max_bodies;
    c.lbits = bits_for(per_world);
    c.wbits = bits_for((long long)desc->max_worlds + 1);
    if (c.wbits + 2 * c.lbits > 64 || c.wbits + 31 > 64)
    {
        delete w;
        return PK_ERR_INVALID;
    }
    int sms = 148;
    int dev = 0;
    cudaGetDevice(&dev);
    w->device = dev;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto blocks_for = [&](long long n)
    {
        long long b = (n + 4095) / 4096;
        if (b > 2LL * sms) b = 2LL * sms;
        return int(b < 1 ? 1 : b);
    };
    c.sort_blocks_bodies = blocks_for(c.body_cap);
    c.sort_blocks_pairs = blocks_for(c.pair_cap);
    w->eng = desc->precision == PK_PRECISION_F64 ? pk::make_engine_f64() : pk::make_engine_f32();
    int rc = w->eng->init(c);
    if (rc)
    {
        g_last_cuda = w->eng->last_error();
        delete w->eng;
        delete w;
        return PK_ERR_CUDA;
    }
    w->worlds.resize(size_t(desc->max_worlds));
    w->slots.resize(size_t(desc->max_bodies));
    for (int i = 0; i < desc->max_worlds; ++i)
    {
        SubWorld &sw = w->worlds[size_t(i)];
        for (int k = 0; k < 3; ++k) sw.gravity[k] = desc->gravity[k];
        double gn = std::sqrt(sw.gravity[0] * sw.gravity[0] + sw.gravity[1] * sw.gravity[1] +
                              sw.gravity[2] * sw.gravity[2]);
        if (w->eng->set_world(i, sw.gravity, gn, 1))
        {
            g_last_cuda = w->eng->last_error();
            delete w->eng;
            delete w;
            return PK_ERR_CUDA;
        }
    }
    *out = w;
    return PK_OK;
}

void pk_world_destroy(pk_world *w)
{
    if (!w) return;
    delete w->eng;
    delete w;
}

// True for mesh::box's layout (mesh.cpp:31-40): 8 vertices (+-hx, +-hy, +-hz) with its sign pattern,
// exactly (vertex 6 holds +h).
static bool box_layout(const std::vector<double> &v)
{
    if (v.size() != 24) return false;
    static const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                 {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int i = 0; i < 8; ++i)
        for (int k = 0; k < 3; ++k)
            if (!(v[size_t(3 * i + k)] == double(sg[i][k]) * v[size_t(18 + k)])) return false;
    return true;
}

// uv_stacks/uv_sectors: the layout of a UV sphere from pk_shape_sphere (0: any other vertex list);
// the device's support search then looks only near the query direction. A vertex list in
// mesh::box's layout is marked (kBoxLayout) for the box support search.
static int add_shape(pk_world *w, const std::vector<double> &v, const std::vector<int> &tris, int32_t *out,
                     int uv_stacks = 0, int uv_sectors = 0)
{
    size_t nv = v.size() / 3;
    if (nv == 0) return PK_ERR_INVALID;
    if (uv_stacks == 0 && box_layout(v)) uv_stacks = pk::kBoxLayout;
    if (w->verts.size() / 3 + nv > size_t(w->cfg.vert_cap) || w->ranges.size() / 8 + 1 > size_t(w->cfg.shape_cap))
        return PK_ERR_CAPACITY;
    // aabb::from_points (bounds.h:33-49)
    double mn[3] = {v[0], v[1], v[2]}, mx[3] = {v[0], v[1], v[2]};
    for (size_t i = 1; i < nv; ++i)
        for (int k = 0; k < 3; ++k)
        {
            double x = v[3 * i + k];
            mn[k] = (x < mn[k]) ? x : mn[k];
            mx[k] = (mx[k] < x) ? x : mx[k];
        }
    int id = int(w->ranges.size() / 8);
    // Bounding spheres of blocks of 8 consecutive vertices (large meshes only): they let the
    // device support search skip blocks that cannot hold the maximum.
    double rm = 0.0;
    for (size_t i = 0; i < nv; ++i)
        rm = std::fmax(rm, std::sqrt(v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]));
    int cstart = int(w->clusters.size() / 4), ncl = 0;
    if (nv > 32)
    {
        for (size_t b = 0; b < nv; b += 8)
        {
            size_t e = b + 8 < nv ? b + 8 : nv;
            double c[3] = {0, 0, 0};
            for (size_t i = b; i < e; ++i)
                for (int k = 0; k < 3; ++k) c[k] += v[3 * i + k] / double(e - b);
            double r = 0.0;
            for (size_t i = b; i < e; ++i)
            {
                double dx = v[3 * i] - c[0], dy = v[3 * i + 1] - c[1], dz = v[3 * i + 2] - c[2];
                r = std::fmax(r, std::sqrt(dx * dx + dy * dy + dz * dz));
            }
            // widen so the bound still holds after rounding the centre and radius to FP32
            r = r * (1.0 + 1e-9) + 1e-6 * rm;
            w->clusters.insert(w->clusters.end(), {c[0], c[1], c[2], r});
            ++ncl;
        }
    }
    // groups of 8 consecutive blocks (64 vertices), bounded the same way
    int gstart = int(w->clusters.size() / 4), ngr = 0;
    if (ncl > 0)
    {
        for (size_t b = 0; b < nv; b += 64)
        {
            size_t e = b + 64 < nv ? b + 64 : nv;
            double c[3] = {0, 0, 0};
            for (size_t i = b; i < e; ++i)
                for (int k = 0; k < 3; ++k) c[k] += v[3 * i + k] / double(e - b);
            double r = 0.0;
            for (size_t i = b; i < e; ++i)
            {
                double dx = v[3 * i] - c[0], dy = v[3 * i + 1] - c[1], dz = v[3 * i + 2] - c[2];
                r = std::fmax(r, std::sqrt(dx * dx + dy * dy + dz * dz));
            }
            r = r * (1.0 + 1e-9) + 1e-6 * rm;
            w->clusters.insert(w->clusters.end(), {c[0], c[1], c[2], r});
            ++ngr;
        }
    }
    w->ranges.push_back(int(w->verts.size() / 3));
    w->ranges.push_back(int(nv));
    w->ranges.push_back(cstart);
    w->ranges.push_back(ncl);
    w->ranges.push_back(gstart);
    w->ranges.push_back(ngr);
    w->ranges.push_back(uv_stacks);
    w->ranges.push_back(uv_sectors);
    w->rmax.push_back(rm);
    w->verts.insert(w->verts.end(), v.begin(), v.end());
    for (int k = 0; k < 3; ++k) w->boxes.push_back(mn[k]);
    for (int k = 0; k < 3; ++k) w->boxes.push_back(mx[k]);
    w->tri_range.push_back(int(w->tris.size() / 3));
    w->tri_range.push_back(int(tris.size() / 3));
    w->tris.insert(w->tris.end(), tris.begin(), tris.end());
    w->shapes_dirty = true; // uploaded in one copy before the next use (flush_shapes)
    if (out) *out = id;
    return PK_OK;
}

// Solver CTAs take worlds largest first so the longest solves start earliest.
static int flush_order(pk_world *w, bool async = false)
{
    if (!w->order_dirty) return PK_OK;
    int nw = w->cfg.max_worlds;
    std::vector<int> cnt(static_cast<size_t>(nw), 0), order(static_cast<size_t>(nw));
    for (int s = 0; s < w->nslots; ++s)
        if (w->slots[size_t(s)].alive && !w->slots[size_t(s)].is_static) cnt[size_t(w->slots[size_t(s)].world)]++;
    std::vector<int> nlocal(static_cast<size_t>(nw));
    for (int i = 0; i < nw; ++i)
    {
        order[size_t(i)] = i;
        nlocal[size_t(i)] = int(w->worlds[size_t(i)].local_slot.size());
    }
    // largest first by local indices in use (this also keeps the worlds that need the large
    // solver cache contiguous at the front), then by dynamic bodies
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (nlocal[size_t(a)] != nlocal[size_t(b)]) return nlocal[size_t(a)] > nlocal[size_t(b)];
        return cnt[size_t(a)] > cnt[size_t(b)];
    });
    if (async ? w->eng->set_world_order_async(order.data(), nlocal.data(), nw)
              : w->eng->set_world_order(order.data(), nlocal.data(), nw))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    w->order_dirty = false;
    return PK_OK;
}

// Joints go to the device in the reference's solve order: per world, constraint types in order,
// arena slots in order (constraint.h:1109-1119). Accumulated impulses carry over.
static int flush_joints(pk_world *w)
{
    if (!w->joints_dirty) return PK_OK;
    const size_t nup = w->joint_order.size();
    if (nup > 0)
    {
        std::vector<double> acc(nup * 6);
        if (w->eng->read_joint_acc(acc.data(), int(nup))) return PK_ERR_CUDA;
        for (size_t i = 0; i < nup; ++i)
            for (int k = 0; k < 6; ++k) w->joints[size_t(w->joint_order[i])].acc[k] = acc[i * 6 + size_t(k)];
    }
    const int nw = w->cfg.max_worlds;
    std::vector<int> order, js(size_t(nw), 0), je(size_t(nw), 0);
    for (int wi = 0; wi < nw; ++wi)
    {
        const SubWorld &sw = w->worlds[size_t(wi)];
        js[size_t(wi)] = int(order.size());
        for (int t = 0; t < 6; ++t)
            for (int j : sw.jslot[t])
                if (j >= 0 && w->joints[size_t(j)].alive) order.push_back(j);
        je[size_t(wi)] = int(order.size());
    }
    const size_t n = order.size();
    std::vector<int> ints(n * 5);
    std::vector<double> params(n * 25), acc(n * 6);
    for (size_t i = 0; i < n; ++i)
    {
        const JointHost &j = w->joints[size_t(order[i])];
        const int v[5] = {j.type, j.slot_a, j.slot_b, j.local_a, j.local_b};
        for (int k = 0; k < 5; ++k) ints[i * 5 + size_t(k)] = v[k];
        for (int k = 0; k < 25; ++k) params[i * 25 + size_t(k)] = j.p[k];
        for (int k = 0; k < 6; ++k) acc[i * 6 + size_t(k)] = j.acc[k];
    }
    if (w->eng->set_joints(ints.data(), params.data(), acc.data(), int(n), js.data(), je.data()))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    w->joint_order = order;
    w->joints_dirty = false;
    return PK_OK;
}

static void drop_joint(pk_world *w, int j)
{
    JointHost &jh = w->joints[size_t(j)];
    if (!jh.alive) return;
    SubWorld &sw = w->worlds[size_t(jh.world)];
    jh.alive = false;
    sw.jslot[jh.type][size_t(jh.arena)] = -1;
    sw.jgen[jh.type][size_t(jh.arena)]++;
    sw.jfree[jh.type].push_back(jh.arena);
    w->joints_dirty = true;
}

static int flush_shapes(pk_world *w)
{
    if (!w->shapes_dirty) return PK_OK;
    if (w->eng->set_shapes(w->verts, w->ranges, w->boxes, w->clusters, w->rmax) ||
        w->eng->set_triangles(w->tris, w->tri_range))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    w->shapes_dirty = false;
    return PK_OK;
}

int pk_shape_mesh(pk_world *w, const double *verts, int32_t nverts, const int32_t *tris, int32_t ntris, int32_t *out)
{
    if (!w || !verts || nverts <= 0 || ntris <= 0 || !tris) return PK_ERR_INVALID;
    for (int i = 0; i < 3 * ntris; ++i)
        if (tris[i] < 0 || tris[i] >= nverts) return PK_ERR_INVALID;
    return add_shape(w, std::vector<double>(verts, verts + 3 * size_t(nverts)),
                     std::vector<int>(tris, tris + 3 * size_t(ntris)), out);
}

int pk_shape_box(pk_world *w, double hx, double hy, double hz, int32_t *out)
{
    if (!w) return PK_ERR_INVALID;
    // mesh::box vertex order (mesh.cpp:31-40)
    std::vector<double> v = {-hx, -hy, -hz, +hx, -hy, -hz, +hx, +hy, -hz, -hx, +hy, -hz,
                             -hx, -hy, +hz, +hx, -hy, +hz, +hx, +hy, +hz, -hx, +hy, +hz};
    // its 12 triangles, two per face (mesh.cpp:41-52)
    std::vector<int> t = {4, 5, 6, 4, 6, 7, 0, 3, 2, 0, 2, 1, 1, 2, 6, 1, 6, 5,
                          0, 4, 7, 0, 7, 3, 3, 7, 6, 3, 6, 2, 0, 1, 5, 0, 5, 4};
    return add_shape(w, v, t, out);
}

int pk_shape_sphere(pk_world *w, double r, int32_t stacks, int32_t sectors, int32_t *out)
{
    if (!w || stacks < 2 || sectors < 3) return PK_ERR_INVALID;
    // mesh::sphere UV layout (mesh.cpp:60-115)
    std::vector<double> v = {0.0, r, 0.0};
    for (int i = 1; i < stacks; ++i)
    {
        double phi = M_PI * double(i) / double(stacks);
        for (int j = 0; j < sectors; ++j)
        {
            double theta = 2.0 * M_PI * double(j) / double(sectors);
            v.push_back(r * std::sin(phi) * std::cos(theta));
            v.push_back(r * std::cos(phi));
            v.push_back(r * std::sin(phi) * std::sin(theta));
        }
    }
    v.push_back(0.0);
    v.push_back(-r);
    v.push_back(0.0);
    // triangles: the north cap, two per quad of each band, the south cap (mesh.cpp:83-113)
    std::vector<int> t;
    const int S = stacks, K = sectors, south = 1 + (S - 1) * K;
    for (int j = 0; j < K; ++j) t.insert(t.end(), {0, 1 + (j + 1) % K, 1 + j});
    for (int i = 1; i + 1 < S; ++i)
        for (int j = 0; j < K; ++j)
        {
            const int top = 1 + (i - 1) * K + j, top_next = 1 + (i - 1) * K + (j + 1) % K;
            const int bot = 1 + i * K + j, bot_next = 1 + i * K + (j + 1) % K;
            t.insert(t.end(), {top, top_next, bot_next, top, bot_next, bot});
        }
    const int last = 1 + (S - 2) * K;
    for (int j = 0; j < K; ++j) t.insert(t.end(), {south, last + j, last + (j + 1) % K});
    // the neighbourhood search is proven for these layouts (pk_narrow.cuh, argmax_uv)
    const bool uv = pk::uv_layout_ok(stacks, sectors);
    return add_shape(w, v, t, out, uv ? stacks : 0, uv ? sectors : 0);
}

int pk_shape_pyramid(pk_world *w, double b, double h, int32_t *out)
{
    if (!w) return PK_ERR_INVALID;
    // mesh::pyramid (mesh.cpp:117-137)
    std::vector<double> v = {-b, 0.0, -b, +b, 0.0, -b, +b, 0.0, +b, -b, 0.0, +b, 0.0, h, 0.0};
    std::vector<int> t = {0, 1, 2, 0, 2, 3, 1, 0, 4, 2, 1, 4, 3, 2, 4, 0, 3, 4};
    return add_shape(w, v, t, out);
}

static int add_bodies(pk_world *w, const pk_body_desc *descs, int32_t n, uint64_t *out, bool async);

int pk_body_add(pk_world *w, const pk_body_desc *descs, int32_t n, uint64_t *out)
{ return add_bodies(w, descs, n, out, false); }

static int add_bodies(pk_world *w, const pk_body_desc *descs, int32_t n, uint64_t *out, bool async)
{
    if (!w || (n > 0 && !descs)) return PK_ERR_INVALID;
    int nshapes = int(w->ranges.size() / 8);
    for (int i = 0; i < n; ++i)
    {
        const pk_body_desc &d = descs[i];
        if (d.shape < 0 || d.shape >= nshapes) return PK_ERR_INVALID; // object.h:121
        if (d.world < 0 || d.world >= w->cfg.max_worlds) return PK_ERR_INVALID;
        if (d.type != PK_BODY_DYNAMIC && d.type != PK_BODY_STATIC) return PK_ERR_INVALID;
    }
    if (int rc = flush_shapes(w)) return rc;
    std::vector<int> slots;
    std::vector<pk::HostBody> hb;
    slots.reserve(size_t(n));
    hb.reserve(size_t(n));
    const long long per_world_cap = 1LL << w->cfg.lbits;
    for (int i = 0; i < n; ++i)
    {
        const pk_body_desc &d = descs[i];
        SubWorld &sw = w->worlds[size_t(d.world)];
        int local;
        if (!sw.free_locals.empty())
        {
            local = sw.free_locals.back();
            sw.free_locals.pop_back();
        }
        else
        {
            if ((long long)sw.local_slot.size() >= per_world_cap) return PK_ERR_CAPACITY;
            local = int(sw.local_slot.size());
            sw.local_slot.push_back(-1);
            sw.local_gen.push_back(0);
            sw.local_alive.push_back(0);
        }
        int slot = sw.local_slot[size_t(local)];
        if (slot < 0)
        {
            if (!w->free_slots.empty())
            {
                slot = w->free_slots.back();
                w->free_slots.pop_back();
            }
            else
            {
                if (w->nslots >= w->cfg.body_cap)
                {
                    sw.free_locals.push_back(local);
                    return PK_ERR_CAPACITY;
                }
                slot = w->nslots++;
            }
            sw.local_slot[size_t(local)] = slot;
        }
        sw.local_alive[size_t(local)] = 1;
        SlotInfo &si = w->slots[size_t(slot)];
        si.world = d.world;
        si.local = local;
        si.gen = sw.local_gen[size_t(local)];
        si.alive = true;
        si.is_static = d.type == PK_BODY_STATIC;

        pk::HostBody h;
        std::memset(&h, 0, sizeof(h));
        h.world = d.world;
        h.local = local;
        h.shape = d.shape;
        h.flags = 1 | (si.is_static ? 2 : 0);
        h.created = w->steps;
        for (int k = 0; k < 3; ++k)
        {
            h.pos[k] = d.pos[k];
            h.vel[k] = d.vel[k];
            h.ang_vel[k] = d.ang_vel[k];
        }
        for (int k = 0; k < 4; ++k) h.quat[k] = d.quat[k];
        // particle(...) constructor (particle.h:121-133): inv_mass = 1/m, I^-1 of the local tensor,
        // zeroed for static bodies (infinite mass, object.h:81-85)
        h.mass = si.is_static ? std::numeric_limits<double>::infinity() : d.mass;
        h.inv_mass = 1.0 / h.mass;
        pk::M3<double> I;
        for (int k = 0; k < 9; ++k) I.m[k] = d.inertia[k];
        pk::M3<double> Ii = pk::inverse(I);
        for (int k = 0; k < 9; ++k)
        {
            h.il[k] = d.inertia[k];
            h.il_inv[k] = (h.inv_mass == 0.0) ? 0.0 : Ii.m[k];
        }
        h.restitution = d.restitution;
        h.friction = d.friction;
        slots.push_back(slot);
        hb.push_back(h);
        if (out) out[i] = uint64_t(uint32_t(slot)) | (uint64_t(si.gen) << 32);
    }
    if (async ? w->eng->upload_bodies_async(slots.data(), hb.data(), n, w->nslots)
              : w->eng->upload_bodies(slots.data(), hb.data(), n, w->nslots))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    w->order_dirty = true;
    return PK_OK;
}

static SlotInfo *resolve(pk_world *w, uint64_t handle, int *slot_out)
{
    uint32_t slot = uint32_t(handle & 0xFFFFFFFFu), gen = uint32_t(handle >> 32);
    if (slot >= uint32_t(w->nslots)) return nullptr;
    SlotInfo &si = w->slots[slot];
    if (!si.alive || si.gen != gen) return nullptr;
    *slot_out = int(slot);
    return &si;
}

static int kill_slot(pk_world *w, int slot)
{
    SlotInfo &si = w->slots[size_t(slot)];
    SubWorld &sw = w->worlds[size_t(si.world)];
    w->waiters.destroyed(uint64_t(uint32_t(slot)) | (uint64_t(si.gen) << 32), w->wakes);
    for (size_t j = 0; j < w->joints.size(); ++j) // joints cannot outlive their bodies
        if (w->joints[j].alive && (w->joints[j].slot_a == slot || w->joints[j].slot_b == slot)) drop_joint(w, int(j));
    si.alive = false;
    sw.local_alive[size_t(si.local)] = 0;
    sw.local_gen[size_t(si.local)]++;
    sw.free_locals.push_back(si.local);
    si.gen = sw.local_gen[size_t(si.local)];
    w->order_dirty = true;
    if (w->eng->kill_body(slot, si.world, si.local))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_body_remove(pk_world *w, uint64_t handle)
{
    if (!w) return PK_ERR_INVALID;
    int slot;
    if (!resolve(w, handle, &slot)) return PK_ERR_STALE_HANDLE;
    return kill_slot(w, slot);
}

static int clear_world(pk_world *w, int32_t world, bool async);

int pk_world_clear(pk_world *w, int32_t world) { return clear_world(w, world, false); }

static int clear_world(pk_world *w, int32_t world, bool async)
{
    if (!w || world < 0 || world >= w->cfg.max_worlds) return PK_ERR_INVALID;
    SubWorld &sw = w->worlds[size_t(world)];
    std::vector<int> dead;
    for (size_t l = 0; l < sw.local_slot.size(); ++l)
    {
        int slot = sw.local_slot[l];
        if (slot < 0) continue;
        if (w->slots[size_t(slot)].alive)
        {
            dead.push_back(slot);
            w->waiters.destroyed(uint64_t(uint32_t(slot)) | (uint64_t(w->slots[size_t(slot)].gen) << 32), w->wakes);
        }
        w->slots[size_t(slot)] = SlotInfo{};
        w->free_slots.push_back(slot);
    }
    for (size_t j = 0; j < w->joints.size(); ++j)
        if (w->joints[j].alive && w->joints[j].world == world) drop_joint(w, int(j));
    for (int t = 0; t < 6; ++t)
    {
        sw.jslot[t].clear();
        sw.jgen[t].clear();
        sw.jfree[t].clear();
    }
    // one kernel kills the bodies, one empties every cached manifold of the world
    if (async ? w->eng->kill_world_async(dead.data(), int(dead.size()), world)
              : w->eng->kill_world(dead.data(), int(dead.size()), world))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    sw.local_slot.clear();
    sw.local_gen.clear();
    sw.local_alive.clear();
    sw.free_locals.clear();
    w->order_dirty = true;
    return PK_OK;
}

int pk_world_set_active_mask(pk_world *w, const uint8_t *mask, int32_t n)
{
    if (!w || !mask || n != w->cfg.max_worlds) return PK_ERR_INVALID;
    for (int i = 0; i < n; ++i) w->worlds[size_t(i)].active = mask[i] ? 1 : 0;
    if (w->eng->set_active_mask(mask, n))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_world_set_active(pk_world *w, int32_t world, int32_t active)
{
    if (!w || world < 0 || world >= w->cfg.max_worlds) return PK_ERR_INVALID;
    SubWorld &sw = w->worlds[size_t(world)];
    sw.active = active ? 1 : 0;
    double gn = std::sqrt(sw.gravity[0] * sw.gravity[0] + sw.gravity[1] * sw.gravity[1] + sw.gravity[2] * sw.gravity[2]);
    if (w->eng->set_world(world, sw.gravity, gn, sw.active)) return PK_ERR_CUDA;
    return PK_OK;
}

int pk_world_set_gravity(pk_world *w, int32_t world, const double g[3])
{
    if (!w || !g || world < 0 || world >= w->cfg.max_worlds) return PK_ERR_INVALID;
    SubWorld &sw = w->worlds[size_t(world)];
    for (int k = 0; k < 3; ++k) sw.gravity[k] = g[k];
    // constraint_solver keeps |g| for the restitution threshold (world.h:383)
    double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    if (w->eng->set_world(world, sw.gravity, gn, sw.active)) return PK_ERR_CUDA;
    return PK_OK;
}

static int step_async(pk_world *w, double dt, bool async_order)
{
    if (!w || !(dt > 0.0)) return PK_ERR_INVALID;
    if (int frc = flush_shapes(w)) return frc;
    if (int orc = flush_order(w, async_order)) return orc;
    if (int jrc = flush_joints(w)) return jrc;
    int rc = w->eng->step(dt);
    if (rc)
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    w->steps++;
    return PK_OK;
}

int pk_world_step_async(pk_world *w, double dt) { return step_async(w, dt, false); }

int pk_world_synchronize(pk_world *w, pk_step_info *info)
{
    if (!w) return PK_ERR_INVALID;
    pk::StepCounters c;
    if (w->eng->synchronize(&c))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    if (info)
    {
        info->pairs = c.npairs;
        info->leaves = c.nleaf;
        info->status = c.status;
        info->launches = c.launches;
        info->gjk = c.gjk;
        info->epa = c.epa;
        info->gjk_large_mesh = c.gjk_heavy;
        info->epa_large_mesh = c.epa_heavy;
        info->gjk_iterations = c.gjk_iters;
        info->epa_iterations = c.epa_iters;
        info->epa_iterations_large_mesh = c.epa_iters_heavy;
        info->support_vertices = c.support_verts;
    }
    return c.status ? PK_ERR_DEVICE_STATUS : PK_OK;
}

int pk_world_step(pk_world *w, double dt)
{
    int rc = pk_world_step_async(w, dt);
    if (rc) return rc;
    return pk_world_synchronize(w, nullptr);
}

int pk_world_capture(pk_world *w, double dt)
{
    if (!w || !(dt > 0.0)) return PK_ERR_INVALID;
    if (int rc = flush_shapes(w)) return rc;
    if (int orc = flush_order(w)) return orc;
    if (int jrc = flush_joints(w)) return jrc;
    if (w->eng->capture_graph(dt))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_world_step_graph(pk_world *w)
{
    if (!w) return PK_ERR_INVALID;
    int rc = w->eng->launch_graph();
    if (rc == -2) return PK_ERR_INVALID;
    if (rc)
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    w->steps++;
    return PK_OK;
}

void *pk_world_stream(pk_world *w) { return w ? w->eng->stream() : nullptr; }

int pk_world_set_timing(pk_world *w, int32_t enable)
{
    if (!w) return PK_ERR_INVALID;
    w->eng->set_timing(enable);
    return PK_OK;
}

int pk_world_read_stage_times(pk_world *w, double *total_ms, int32_t *counts, int32_t cap, int32_t *nstages)
{
    if (!w) return PK_ERR_INVALID;
    double ms[pk::kStageRows];
    int cnt[pk::kStageRows];
    if (w->eng->read_stage_times(ms, cnt) < 0)
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    if (nstages) *nstages = pk::kStageRows;
    for (int k = 0; k < pk::kStageRows && k < cap; ++k)
    {
        if (total_ms) total_ms[k] = ms[k];
        if (counts) counts[k] = cnt[k];
    }
    return PK_OK;
}

const char *pk_stage_name(int32_t stage)
{
    if (stage < 0 || stage >= pk::kStageRows) return nullptr;
    return pk::kStageNames[stage];
}

// Time `k` plain steps with per-stage CUDA events; returns mean ms per step of every stage.
static int timed_steps(pk_world *w, double dt, int k, double *stage_ms)
{
    double ms[pk::kStageRows];
    int cnt[pk::kStageRows];
    if (w->eng->read_stage_times(ms, cnt) < 0) return PK_ERR_CUDA; // clear
    for (int i = 0; i < k; ++i)
        if (int rc = pk_world_step_async(w, dt)) return rc;
    if (w->eng->synchronize(nullptr)) return PK_ERR_CUDA;
    if (w->eng->read_stage_times(ms, cnt) < 0) return PK_ERR_CUDA;
    for (int s = 0; s < pk::kStages; ++s) stage_ms[s] = cnt[s] ? ms[s] / cnt[s] : 0.0;
    return PK_OK;
}

int pk_world_autotune(pk_world *w, double dt, int32_t steps_per_candidate, pk_tune_result *out)
{
    if (!w || !(dt > 0.0) || steps_per_candidate < 1) return PK_ERR_INVALID;
    if (int rc = flush_shapes(w)) return rc;
    if (int rc = flush_order(w)) return rc;
    if (int jrc = flush_joints(w)) return jrc;
    const int k = steps_per_candidate;
    int used = 0;
    double st[pk::kStages];
    auto total = [&](const double *x) {
        double t = 0.0;
        for (int i = 0; i < pk::kStages; ++i) t += x[i];
        return t;
    };
    w->eng->set_timing(1);
    pk::Tunables best = w->eng->tunables();
    int rc = timed_steps(w, dt, k, st);
    used += k;
    if (rc) return rc;
    const double before = total(st);
    enum { S_TRAVERSE = 3, S_NARROW = 5, S_SOLVE = 7 };
    // solver: CTA size x small-world split
    {
        double bt = 1e300;
        pk::Tunables bc = best;
        for (int th : {64, 128, 256})
            for (int sw : {256, 512, 1024})
            {
                pk::Tunables t = best;
                t.solve_threads = th;
                t.small_world = sw;
                w->eng->set_tunables(t);
                if ((rc = timed_steps(w, dt, k, st))) return rc;
                used += k;
                if (st[S_SOLVE] < bt)
                {
                    bt = st[S_SOLVE];
                    bc = t;
                }
            }
        best = bc;
    }
    // CTA size of the large-world launch (its worlds are the solver's critical path)
    {
        double bt = 1e300;
        pk::Tunables bc = best;
        for (int th : {128, 256, 512})
        {
            pk::Tunables t = best;
            t.big_threads = th;
            w->eng->set_tunables(t);
            if ((rc = timed_steps(w, dt, k, st))) return rc;
            used += k;
            if (st[S_SOLVE] < bt)
            {
                bt = st[S_SOLVE];
                bc = t;
            }
        }
        best = bc;
    }
    // solve groups: small worlds packed several per CTA, their colours swept together
    {
        double bt = 1e300;
        pk::Tunables bc = best;
        // (local indices per group, CTA size, one member per warp)
        const int tw[][3] = {{0, 128, 0},    {128, 32, 0},    {256, 64, 0},    {512, 128, 0},
                             {1024, 128, 0}, {1024, 256, 0},  {2048, 256, 0},  {512, 128, 1},
                             {1024, 256, 1}, {2048, 256, 1}};
        for (const auto &c : tw)
        {
            pk::Tunables t = best;
            t.group_bodies = c[0];
            t.group_threads = c[1];
            t.group_warp = c[2];
            w->eng->set_tunables(t);
            if ((rc = timed_steps(w, dt, k, st))) return rc;
            used += k;
            if (st[S_SOLVE] < bt)
            {
                bt = st[S_SOLVE];
                bc = t;
            }
        }
        best = bc;
    }
    // narrowphase grid
    {
        double bt = 1e300;
        pk::Tunables bc = best;
        for (int g : {1, 2, 4})
        {
            pk::Tunables t = best;
            t.narrow_grid = g;
            w->eng->set_tunables(t);
            if ((rc = timed_steps(w, dt, k, st))) return rc;
            used += k;
            if (st[S_NARROW] < bt)
            {
                bt = st[S_NARROW];
                bc = t;
            }
        }
        best = bc;
    }
    // traversal block size
    {
        double bt = 1e300;
        pk::Tunables bc = best;
        for (int th : {64, 128, 256})
        {
            pk::Tunables t = best;
            t.traverse_threads = th;
            w->eng->set_tunables(t);
            if ((rc = timed_steps(w, dt, k, st))) return rc;
            used += k;
            if (st[S_TRAVERSE] < bt)
            {
                bt = st[S_TRAVERSE];
                bc = t;
            }
        }
        best = bc;
    }
    w->eng->set_tunables(best);
    if ((rc = timed_steps(w, dt, k, st))) return rc;
    used += k;
    w->eng->set_timing(0);
    if (out)
    {
        out->solve_threads = best.solve_threads;
        out->small_world = best.small_world;
        out->narrow_grid = best.narrow_grid;
        out->traverse_threads = best.traverse_threads;
        out->step_ms_before = before;
        out->step_ms_after = total(st);
        out->steps_used = used;
        out->big_threads = best.big_threads;
        out->group_bodies = best.group_bodies;
        out->group_threads = best.group_threads;
        out->group_warp = best.group_warp;
    }
    return PK_OK;
}

int pk_world_set_tuning(pk_world *w, const pk_tune_result *t)
{
    if (!w || !t) return PK_ERR_INVALID;
    if (t->solve_threads < 32 || t->solve_threads > 512 || (t->solve_threads & 31) || t->small_world < 1 ||
        t->narrow_grid < 1 || t->narrow_grid > 16 || t->traverse_threads < 32 || t->traverse_threads > 1024 ||
        (t->traverse_threads & 31) || t->big_threads < 0 || t->big_threads > 512 || (t->big_threads & 31) ||
        t->group_bodies < 0 || t->group_threads < 0 || t->group_threads > 256 || (t->group_threads & 31) ||
        t->group_warp < 0 || t->group_warp > 1)
        return PK_ERR_INVALID;
    pk::Tunables tu;
    tu.solve_threads = t->solve_threads;
    tu.small_world = t->small_world;
    tu.narrow_grid = t->narrow_grid;
    tu.traverse_threads = t->traverse_threads;
    tu.big_threads = t->big_threads > 0 ? t->big_threads : t->solve_threads;
    tu.group_bodies = t->group_bodies;
    tu.group_threads = t->group_threads > 0 ? t->group_threads : 128;
    tu.group_warp = t->group_warp;
    w->eng->set_tunables(tu);
    w->launch_version++;
    return PK_OK;
}

int pk_world_read_bodies(pk_world *w, double *out, int32_t cap, int32_t *n)
{
    if (!w) return PK_ERR_INVALID;
    if (n) *n = w->nslots;
    if (!out || cap <= 0) return PK_OK;
    int m = cap < w->nslots ? cap : w->nslots;
    if (w->eng->read_bodies(out, m) < 0) return PK_ERR_CUDA;
    return PK_OK;
}

int pk_world_read_bodies_async(pk_world *w, double *out, int32_t cap, int32_t *n)
{
    if (!w) return PK_ERR_INVALID;
    if (n) *n = w->nslots;
    if (!out || cap <= 0) return PK_OK;
    int m = cap < w->nslots ? cap : w->nslots;
    if (w->eng->read_bodies_async(out, m) < 0)
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_host_register(void *ptr, size_t bytes)
{
    if (!ptr || bytes == 0) return PK_ERR_INVALID;
    cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_host_unregister(void *ptr)
{
    if (!ptr) return PK_ERR_INVALID;
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_body_alive(pk_world *w, uint64_t handle)
{
    if (!w) return PK_ERR_INVALID;
    int slot;
    return resolve(w, handle, &slot) ? PK_OK : PK_ERR_STALE_HANDLE;
}

int pk_world_write_body(pk_world *w, uint64_t handle, const double *s)
{
    if (!w || !s) return PK_ERR_INVALID;
    int slot;
    if (!resolve(w, handle, &slot)) return PK_ERR_STALE_HANDLE;
    if (w->eng->write_state(slot, s)) return PK_ERR_CUDA;
    return PK_OK;
}

static void split_key(const pk_world *w, uint64_t k, uint64_t *ref, int32_t *world)
{
    int lb = w->cfg.lbits;
    uint64_t mask = (uint64_t(1) << lb) - 1;
    uint64_t lo = (k >> lb) & mask, hi = k & mask;
    if (ref) *ref = (lo << 32) | hi;
    if (world) *world = int32_t(k >> (2 * lb));
}

int pk_world_read_pairs(pk_world *w, uint64_t *keys, int32_t *worlds, int32_t cap, int32_t *n)
{
    if (!w) return PK_ERR_INVALID;
    int np = w->eng->read_pairs(nullptr, nullptr, 0);
    if (np < 0) return PK_ERR_CUDA;
    if (n) *n = np;
    int m = cap < np ? cap : np;
    if (m <= 0) return PK_OK;
    std::vector<uint64_t> raw(static_cast<size_t>(m));
    if (w->eng->read_pairs(raw.data(), nullptr, m) < 0) return PK_ERR_CUDA;
    for (int i = 0; i < m; ++i) split_key(w, raw[size_t(i)], keys ? keys + i : nullptr, worlds ? worlds + i : nullptr);
    return PK_OK;
}

int pk_world_read_manifolds(pk_world *w, uint64_t *keys, int32_t *worlds, int32_t *counts, double *contacts,
                            int32_t cap, int32_t *n)
{
    if (!w) return PK_ERR_INVALID;
    int np = w->eng->read_manifolds(nullptr, nullptr, nullptr, 0);
    if (np < 0) return PK_ERR_CUDA;
    if (n) *n = np;
    int m = cap < np ? cap : np;
    if (m <= 0) return PK_OK;
    std::vector<uint64_t> raw(static_cast<size_t>(m));
    if (w->eng->read_manifolds(raw.data(), counts, contacts, m) < 0) return PK_ERR_CUDA;
    for (int i = 0; i < m; ++i) split_key(w, raw[size_t(i)], keys ? keys + i : nullptr, worlds ? worlds + i : nullptr);
    return PK_OK;
}

int pk_world_read_events(pk_world *w, uint64_t *keys, int32_t *worlds, int32_t *kinds, int32_t cap, int32_t *n)
{
    if (!w) return PK_ERR_INVALID;
    int ne = w->eng->read_events(nullptr, nullptr, 0);
    if (ne < 0) return PK_ERR_CUDA;
    if (n) *n = ne;
    int m = cap < ne ? cap : ne;
    if (m <= 0) return PK_OK;
    std::vector<uint64_t> raw(static_cast<size_t>(m));
    std::vector<int> kd(static_cast<size_t>(m));
    if (w->eng->read_events(raw.data(), kd.data(), m) < 0) return PK_ERR_CUDA;
    for (int i = 0; i < m; ++i)
    {
        split_key(w, raw[size_t(i)], keys ? keys + i : nullptr, worlds ? worlds + i : nullptr);
        if (kinds) kinds[i] = kd[size_t(i)];
    }
    return PK_OK;
}

void pk_joint_desc_init(pk_joint_desc *d)
{
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
}

// The constructors of the joint types (constraint.h:183-187, 298-305, 386-392, 494-500, 635-652,
// 779-785), from the bodies' current poses.
int pk_joint_add(pk_world *w, const pk_joint_desc *d, uint64_t *out)
{
    using V = pk::V3<double>;
    using Q = pk::Qt<double>;
    if (!w || !d || d->type < PK_JOINT_DISTANCE || d->type > PK_JOINT_SPRING) return PK_ERR_INVALID;
    int sa, sb;
    SlotInfo *ia = resolve(w, d->a, &sa), *ib = resolve(w, d->b, &sb);
    if (!ia || !ib) return PK_ERR_STALE_HANDLE;
    if (ia->world != ib->world || sa == sb) return PK_ERR_INVALID;
    double pa[7], pb[7];
    if (w->eng->read_pose(sa, pa) || w->eng->read_pose(sb, pb)) return PK_ERR_CUDA;
    const V xa{pa[0], pa[1], pa[2]}, xb{pb[0], pb[1], pb[2]};
    const Q qa{pa[3], pa[4], pa[5], pa[6]}, qb{pb[3], pb[4], pb[5], pb[6]};
    auto vec = [](const double *v) { return V{v[0], v[1], v[2]}; };
    auto basis = [](V n, V &t1, V &t2) { // build_orthonormal_basis (constraint.h:104-113)
        double sign = std::copysign(1.0, n.z);
        double a = -1.0 / (sign + n.z);
        double b = n.x * n.y * a;
        t1 = V{1.0 + sign * n.x * n.x * a, sign * b, -sign * n.x};
        t2 = V{b, sign + n.y * n.y * a, -n.y};
    };
    JointHost j;
    j.type = d->type;
    j.world = ia->world;
    j.slot_a = sa;
    j.slot_b = sb;
    j.local_a = ia->local;
    j.local_b = ib->local;
    j.alive = true;
    V la{0, 0, 0}, lb{0, 0, 0}, axa{0, 0, 0}, axb{0, 0, 0}, va{0, 0, 0}, wa{0, 0, 0};
    Q qrel{1, 0, 0, 0};
    const V anchor = vec(d->anchor);
    switch (d->type)
    {
    case PK_JOINT_DISTANCE:
    case PK_JOINT_SPRING:
        la = vec(d->local_a);
        lb = vec(d->local_b);
        break;
    case PK_JOINT_BALL_SOCKET:
    case PK_JOINT_WELD:
        la = pk::rotate(pk::conj(qa), anchor - xa); // project_to_local (particle.h:107-108)
        lb = pk::rotate(pk::conj(qb), anchor - xb);
        qrel = pk::qmul(pk::conj(qa), qb);
        break;
    case PK_JOINT_HINGE:
        la = vec(d->local_a);
        lb = vec(d->local_b);
        axa = pk::normalized(vec(d->axis_a));
        axb = pk::normalized(vec(d->axis_b));
        basis(axa, va, wa);
        break;
    case PK_JOINT_SLIDER: {
        la = pk::rotate(pk::conj(qa), anchor - xa);
        lb = pk::rotate(pk::conj(qb), anchor - xb);
        V n = pk::normalized(vec(d->axis_a));
        axa = pk::rotate(pk::conj(qa), n);
        V t1, t2;
        basis(n, t1, t2);
        va = pk::rotate(pk::conj(qa), t1);
        wa = pk::rotate(pk::conj(qa), t2);
        qrel = pk::qmul(pk::conj(qa), qb);
        break;
    }
    default:
        return PK_ERR_INVALID;
    }
    const V vs[6] = {la, lb, axa, axb, va, wa};
    for (int k = 0; k < 6; ++k)
    {
        j.p[3 * k + 0] = vs[k].x;
        j.p[3 * k + 1] = vs[k].y;
        j.p[3 * k + 2] = vs[k].z;
    }
    j.p[18] = qrel.w;
    j.p[19] = qrel.x;
    j.p[20] = qrel.y;
    j.p[21] = qrel.z;
    j.p[22] = d->distance;
    j.p[23] = d->stiffness;
    j.p[24] = d->damping;
    SubWorld &sw = w->worlds[size_t(j.world)];
    const int t = d->type;
    int idx;
    if (sw.jfree[t].empty())
    {
        idx = int(sw.jslot[t].size());
        sw.jslot[t].push_back(-1);
        sw.jgen[t].push_back(0);
    }
    else
    {
        idx = sw.jfree[t].back();
        sw.jfree[t].pop_back();
    }
    j.arena = idx;
    sw.jslot[t][size_t(idx)] = int(w->joints.size());
    w->joints.push_back(j);
    w->joints_dirty = true;
    if (out)
        *out = uint64_t(uint32_t(idx) & 0xFFFFFFu) | (uint64_t(sw.jgen[t][size_t(idx)] & 0xFFFFu) << 24) |
               (uint64_t(uint32_t(j.world) & 0xFFFFFu) << 40) | (uint64_t(t) << 60);
    return PK_OK;
}

static int resolve_joint(pk_world *w, uint64_t h)
{
    const int t = int(h >> 60), world = int((h >> 40) & 0xFFFFFu), idx = int(h & 0xFFFFFFu);
    const uint32_t gen = uint32_t((h >> 24) & 0xFFFFu);
    if (t > PK_JOINT_SPRING || world >= w->cfg.max_worlds) return -1;
    const SubWorld &sw = w->worlds[size_t(world)];
    if (size_t(idx) >= sw.jslot[t].size() || (sw.jgen[t][size_t(idx)] & 0xFFFFu) != gen) return -1;
    return sw.jslot[t][size_t(idx)];
}

int pk_joint_remove(pk_world *w, uint64_t h)
{
    if (!w) return PK_ERR_INVALID;
    const int j = resolve_joint(w, h);
    if (j < 0) return PK_ERR_STALE_HANDLE;
    if (int rc = flush_joints(w)) return rc; // keep the other joints' impulses
    drop_joint(w, j);
    return PK_OK;
}

int pk_joint_read_impulses(pk_world *w, uint64_t h, double *out6, int32_t *nrows)
{
    if (!w || !out6) return PK_ERR_INVALID;
    const int j = resolve_joint(w, h);
    if (j < 0) return PK_ERR_STALE_HANDLE;
    static const int rows[6] = {1, 3, 5, 5, 6, 1};
    const JointHost &jh = w->joints[size_t(j)];
    for (int k = 0; k < 6; ++k) out6[k] = jh.acc[k];
    for (size_t i = 0; i < w->joint_order.size(); ++i)
        if (w->joint_order[i] == j && !w->joints_dirty)
        {
            std::vector<double> acc(w->joint_order.size() * 6);
            if (w->eng->read_joint_acc(acc.data(), int(w->joint_order.size()))) return PK_ERR_CUDA;
            for (int k = 0; k < 6; ++k) out6[k] = acc[i * 6 + size_t(k)];
        }
    if (nrows) *nrows = rows[jh.type];
    return PK_OK;
}

int pk_world_wait(pk_world *w, int32_t kind, uint64_t object, uint64_t with, uint64_t *waiter)
{
    if (!w || kind < PK_WAIT_COLLISION || kind > PK_WAIT_DESTROYED || !waiter) return PK_ERR_INVALID;
    int slot;
    if (!resolve(w, object, &slot)) return PK_ERR_STALE_HANDLE; // await_ready: nothing to wait for
    *waiter = w->waiters.add(kind, object, with);
    return PK_OK;
}

int pk_world_cancel_wait(pk_world *w, uint64_t waiter)
{
    if (!w) return PK_ERR_INVALID;
    return w->waiters.cancel(waiter) ? PK_OK : PK_ERR_INVALID;
}

int pk_world_dispatch(pk_world *w, pk_wake *out, int32_t cap, int32_t *n)
{
    if (!w || cap < 0 || (cap > 0 && !out)) return PK_ERR_INVALID;
    if (w->dispatched_step != w->steps)
    {
        // the last step's begin/end events, in pair-key order, as (handle, handle) pairs
        int ne = w->eng->read_events(nullptr, nullptr, 0);
        if (ne < 0) return PK_ERR_CUDA;
        std::vector<uint64_t> raw(static_cast<size_t>(ne));
        std::vector<int> kd(static_cast<size_t>(ne));
        if (ne > 0 && w->eng->read_events(raw.data(), kd.data(), ne) < 0) return PK_ERR_CUDA;
        for (int i = 0; i < ne; ++i)
        {
            uint64_t ref;
            int32_t wid;
            split_key(w, raw[size_t(i)], &ref, &wid);
            const SubWorld &sw = w->worlds[size_t(wid)];
            uint64_t h[2];
            const uint32_t loc[2] = {uint32_t(ref >> 32), uint32_t(ref & 0xFFFFFFFFu)};
            for (int k = 0; k < 2; ++k)
            {
                const int slot = loc[k] < sw.local_slot.size() ? sw.local_slot[loc[k]] : -1;
                h[k] = slot < 0 ? pk::EventDispatcher::kAny
                                : uint64_t(uint32_t(slot)) | (uint64_t(sw.local_gen[loc[k]]) << 32);
            }
            w->waiters.event(kd[size_t(i)], h[0], h[1], w->wakes);
        }
        w->dispatched_step = w->steps;
    }
    int m = 0;
    while (m < cap && w->wake_head < w->wakes.size())
    {
        const pk::Wake &k = w->wakes[w->wake_head++];
        out[m++] = pk_wake{k.waiter, k.object, k.other, k.kind, k.failed};
    }
    if (w->wake_head == w->wakes.size())
    {
        w->wakes.clear();
        w->wake_head = 0;
    }
    if (n) *n = m;
    return PK_OK;
}

int pk_world_read_colours(pk_world *w, uint64_t *keys, int32_t *colours, int32_t cap, int32_t *n, int32_t *nc0)
{
    if (!w) return PK_ERR_INVALID;
    int nc = 0;
    int na = w->eng->read_colours(nullptr, nullptr, 0, &nc);
    if (na < 0) return PK_ERR_CUDA;
    if (n) *n = na;
    if (nc0) *nc0 = nc;
    int m = cap < na ? cap : na;
    if (m <= 0) return PK_OK;
    std::vector<uint64_t> raw(static_cast<size_t>(m));
    std::vector<int> col(static_cast<size_t>(m));
    if (w->eng->read_colours(raw.data(), col.data(), m, &nc) < 0) return PK_ERR_CUDA;
    for (int i = 0; i < m; ++i)
    {
        split_key(w, raw[size_t(i)], keys ? keys + i : nullptr, nullptr);
        if (colours) colours[i] = col[size_t(i)];
    }
    return PK_OK;
}

int pk_world_raycast(pk_world *w, const pk_ray *rays, int32_t n, int32_t cap, uint64_t *handles, double *distances,
                     int32_t *counts)
{
    if (!w || n < 0 || (n > 0 && (!rays || !counts || cap < 1 || !handles || !distances))) return PK_ERR_INVALID;
    if (n == 0) return PK_OK;
    for (int i = 0; i < n; ++i)
        if (rays[i].world < 0 || rays[i].world >= w->cfg.max_worlds || !(rays[i].max_distance >= 0.0))
            return PK_ERR_INVALID;
    if (int rc = flush_shapes(w)) return rc;
    std::vector<double> r(size_t(n) * 8);
    for (int i = 0; i < n; ++i)
    {
        double *o = r.data() + size_t(i) * 8;
        for (int k = 0; k < 3; ++k)
        {
            o[k] = rays[i].origin[k];
            o[3 + k] = rays[i].direction[k];
        }
        o[6] = rays[i].max_distance;
        o[7] = double(rays[i].world);
    }
    const size_t m = size_t(n) * size_t(cap);
    std::vector<int> slots(m);
    std::vector<double> dist(m);
    if (w->eng->raycast(r.data(), n, cap, counts, slots.data(), dist.data()))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    // device slots -> handles, then (distance, handle) order within each ray
    std::vector<std::pair<double, uint64_t>> hit;
    for (int i = 0; i < n; ++i)
    {
        const int k = counts[i] < cap ? counts[i] : cap;
        hit.clear();
        for (int j = 0; j < k; ++j)
        {
            const size_t q = size_t(i) * size_t(cap) + size_t(j);
            const int s = slots[q];
            hit.push_back({dist[q], uint64_t(uint32_t(s)) | (uint64_t(w->slots[size_t(s)].gen) << 32)});
        }
        std::sort(hit.begin(), hit.end());
        for (int j = 0; j < k; ++j)
        {
            handles[size_t(i) * size_t(cap) + size_t(j)] = hit[size_t(j)].second;
            distances[size_t(i) * size_t(cap) + size_t(j)] = hit[size_t(j)].first;
        }
    }
    return PK_OK;
}

int pk_mesh_raycast(pk_world *w, const pk_mesh_ray *rays, int32_t n, pk_mesh_hit *hits)
{
    if (!w || n < 0 || (n > 0 && (!rays || !hits))) return PK_ERR_INVALID;
    const int nshapes = int(w->ranges.size() / 8);
    std::vector<pk::MeshRayIn> in(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i)
    {
        const pk_mesh_ray &r = rays[i];
        pk::MeshRayIn &q = in[size_t(i)];
        q.slot = -1;
        q.shape = r.shape;
        if (r.body != PK_HANDLE_ANY)
        {
            int slot;
            if (!resolve(w, r.body, &slot)) return PK_ERR_STALE_HANDLE;
            q.slot = slot;
        }
        else if (r.shape < 0 || r.shape >= nshapes)
            return PK_ERR_INVALID;
        if (!(r.max_distance >= 0.0)) return PK_ERR_INVALID;
        for (int k = 0; k < 3; ++k)
        {
            q.pos[k] = r.pos[k];
            q.o[k] = r.origin[k];
            q.d[k] = r.direction[k];
        }
        for (int k = 0; k < 4; ++k) q.q[k] = r.quat[k];
        q.maxd = r.max_distance;
    }
    if (int rc = flush_shapes(w)) return rc;
    if (n == 0) return PK_OK;
    static_assert(sizeof(pk_mesh_hit) == sizeof(pk::MeshHitOut), "layout shared with the device result");
    if (w->eng->mesh_raycast(in.data(), n, reinterpret_cast<pk::MeshHitOut *>(hits)))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    return PK_OK;
}

int pk_collide(pk_world *w, const pk_collide_shape *a, const pk_collide_shape *b, int32_t n, double *out, int32_t *hit)
{
    if (!w || n < 0 || (n > 0 && (!a || !b || !out || !hit))) return PK_ERR_INVALID;
    int nshapes = int(w->ranges.size() / 8);
    for (int i = 0; i < n; ++i)
    {
        for (const pk_collide_shape *s : {a + i, b + i})
        {
            if (s->kind < 0 || s->kind > 2) return PK_ERR_INVALID;
            if (s->kind == 2 && (s->shape < 0 || s->shape >= nshapes)) return PK_ERR_INVALID;
        }
    }
    if (int rc = flush_shapes(w)) return rc;
    std::vector<int> status(size_t(n > 0 ? n : 1));
    static_assert(sizeof(pk_collide_shape) == 4 + 4 + 80, "layout shared with the device ShapeSpec");
    if (w->eng->collide(a, b, n, out, hit, status.data()))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    for (int i = 0; i < n; ++i)
        if (status[size_t(i)]) return PK_ERR_DEVICE_STATUS; // results written; a pair hit a capacity cap
    return PK_OK;
}

// ------------------------------------------------------------------------------------------------
// Serving: continuous batching of step requests over one device-resident pool of worlds
// ------------------------------------------------------------------------------------------------
} // extern "C"

struct pk_batch
{
    pk_world *w = nullptr;
    pk_batch_desc desc{};
    int64_t pool_bodies = 0, bodies_in_use = 0;
    struct Slot
    {
        bool live = false, retiring = false;
        int32_t nbodies = 0;
        int in_flight = 0;           // pending requests already in enqueued steps
        std::deque<int64_t> pending; // request tags, oldest first
    };
    std::vector<Slot> slots;
    std::deque<int32_t> free_ids;
    struct Flight
    {
        cudaEvent_t ev;
        std::vector<std::pair<int32_t, int64_t>> served;
    };
    std::deque<Flight> flight;
    std::vector<cudaEvent_t> spare;
    std::vector<uint8_t> mask;
    std::deque<pk_batch_event> ready; // completions not yet returned by pk_batch_poll
    int64_t steps = 0;
    int graph_version = -1; // launch_version of the world when the step graph was captured
    int64_t captures = 0;
};

namespace
{
int batch_retire_now(pk_batch *b, int32_t wid)
{
    pk_batch::Slot &s = b->slots[size_t(wid)];
    if (int rc = clear_world(b->w, wid, true)) return rc;
    b->bodies_in_use -= s.nbodies;
    s = pk_batch::Slot{};
    b->free_ids.push_back(wid);
    pk_batch_event e{};
    e.tag = -1;
    e.world = wid;
    e.kind = PK_BATCH_RETIRED;
    b->ready.push_back(e);
    return PK_OK;
}
} // namespace

extern "C" {

void pk_batch_desc_init(pk_batch_desc *d)
{
    std::memset(d, 0, sizeof(*d));
    d->gravity[1] = -9.81;
    d->dt = 1.0 / 120.0;
    d->solver_iterations = 10;
    d->precision = PK_PRECISION_F32;
    d->max_worlds = 1024;
    d->max_bodies_per_world = 4096 + 5;
    d->max_bodies = 0;
    d->memory_fraction = 0.5;
    d->pair_factor = 6;
    d->contact_factor = 2;
    d->max_shapes = 1024;
    d->max_shape_vertices = 65536;
    d->pipeline_depth = 1;
}

int pk_batch_create(const pk_batch_desc *desc, pk_batch **out)
{
    if (!desc || !out) return PK_ERR_INVALID;
    *out = nullptr;
    if (desc->max_worlds <= 0 || desc->max_bodies < 0 || !(desc->dt > 0.0) || desc->pair_factor <= 0 ||
        desc->contact_factor < 0 || desc->pipeline_depth < 0 || desc->pipeline_depth > 8 ||
        !(desc->memory_fraction >= 0.0 && desc->memory_fraction <= 0.9))
        return PK_ERR_INVALID;
    int64_t pool = desc->max_bodies;
    if (pool == 0)
    {
        // admission is by device memory: the pool takes a share of the HBM free now, at the
        // engine's cost per body slot (body state and its share of the pair and contact capacity)
        size_t free_b = 0, total_b = 0;
        cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
        if (e != cudaSuccess)
        {
            g_last_cuda = int(e);
            return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? PK_ERR_NO_DEVICE : PK_ERR_CUDA;
        }
        const double scale = desc->precision == PK_PRECISION_F64 ? 1.5 : 1.0;
        const double per_body = scale * (600.0 + 720.0 * desc->pair_factor + 1250.0 * desc->contact_factor);
        const double frac = desc->memory_fraction > 0.0 ? desc->memory_fraction : 0.5;
        pool = int64_t(double(free_b) * frac / per_body);
        const int64_t lim = (int64_t(1) << 30) / std::max(1, desc->pair_factor);
        if (pool > lim) pool = lim;
    }
    if (pool <= 0 || pool > INT32_MAX / 16) return PK_ERR_CAPACITY;
    pk_world_desc wd;
    pk_world_desc_init(&wd);
    for (int k = 0; k < 3; ++k) wd.gravity[k] = desc->gravity[k];
    wd.solver_iterations = desc->solver_iterations;
    wd.precision = desc->precision;
    wd.max_bodies = int32_t(pool);
    wd.max_pairs = int32_t(std::min<int64_t>(int64_t(desc->pair_factor) * pool, INT32_MAX));
    wd.max_contact_pairs =
        desc->contact_factor > 0 ? int32_t(std::min<int64_t>(int64_t(desc->contact_factor) * pool, INT32_MAX)) : 0;
    wd.max_worlds = desc->max_worlds;
    wd.max_bodies_per_world = desc->max_bodies_per_world;
    wd.max_shapes = desc->max_shapes;
    wd.max_shape_vertices = desc->max_shape_vertices;
    pk_world *w = nullptr;
    if (int rc = pk_world_create(&wd, &w)) return rc;
    auto *b = new (std::nothrow) pk_batch;
    if (!b)
    {
        pk_world_destroy(w);
        return PK_ERR_CAPACITY;
    }
    b->w = w;
    b->desc = *desc;
    if (b->desc.pipeline_depth == 0) b->desc.pipeline_depth = 1;
    b->pool_bodies = pool;
    b->slots.resize(size_t(desc->max_worlds));
    for (int32_t i = 0; i < desc->max_worlds; ++i) b->free_ids.push_back(i);
    b->mask.assign(size_t(desc->max_worlds), 0);
    // every world sits out until a request names it
    if (w->eng->set_active_mask_async(b->mask.data(), desc->max_worlds))
    {
        g_last_cuda = w->eng->last_error();
        pk_world_destroy(w);
        delete b;
        return PK_ERR_CUDA;
    }
    for (int32_t i = 0; i < desc->max_worlds; ++i) w->worlds[size_t(i)].active = 0;
    *out = b;
    return PK_OK;
}

void pk_batch_destroy(pk_batch *b)
{
    if (!b) return;
    cudaStreamSynchronize(static_cast<cudaStream_t>(b->w->eng->stream()));
    for (auto &f : b->flight) cudaEventDestroy(f.ev);
    for (cudaEvent_t e : b->spare) cudaEventDestroy(e);
    pk_world_destroy(b->w);
    delete b;
}

pk_world *pk_batch_world(pk_batch *b) { return b ? b->w : nullptr; }

int pk_batch_admit(pk_batch *b, const pk_body_desc *bodies, int32_t n, uint64_t *out_handles, int32_t *out_world)
{
    if (!b || n <= 0 || !bodies || !out_world) return PK_ERR_INVALID;
    if (n > b->desc.max_bodies_per_world) return PK_ERR_INVALID;
    if (b->free_ids.empty() || b->bodies_in_use + n > b->pool_bodies) return PK_ERR_CAPACITY; // wait for a retirement
    const int32_t wid = b->free_ids.front();
    std::vector<pk_body_desc> d(bodies, bodies + n);
    for (pk_body_desc &x : d) x.world = wid;
    std::vector<uint64_t> h(static_cast<size_t>(n));
    if (int rc = add_bodies(b->w, d.data(), n, out_handles ? out_handles : h.data(), true)) return rc;
    b->free_ids.pop_front();
    pk_batch::Slot &s = b->slots[size_t(wid)];
    s.live = true;
    s.retiring = false;
    s.nbodies = n;
    s.in_flight = 0;
    s.pending.clear();
    b->bodies_in_use += n;
    *out_world = wid;
    return PK_OK;
}

int pk_batch_request(pk_batch *b, int32_t world, int64_t tag)
{
    if (!b || world < 0 || world >= b->desc.max_worlds) return PK_ERR_INVALID;
    pk_batch::Slot &s = b->slots[size_t(world)];
    if (!s.live || s.retiring) return PK_ERR_STALE_HANDLE;
    s.pending.push_back(tag);
    return PK_OK;
}

int pk_batch_retire(pk_batch *b, int32_t world)
{
    if (!b || world < 0 || world >= b->desc.max_worlds) return PK_ERR_INVALID;
    pk_batch::Slot &s = b->slots[size_t(world)];
    if (!s.live || s.retiring) return PK_ERR_STALE_HANDLE;
    s.retiring = true;
    if (s.pending.empty() && s.in_flight == 0) return batch_retire_now(b, world);
    return PK_OK; // after its pending steps (pk_batch_poll reports PK_BATCH_RETIRED)
}

int pk_batch_step_async(pk_batch *b, int32_t *nworlds)
{
    if (!b) return PK_ERR_INVALID;
    if (nworlds) *nworlds = 0;
    if (int(b->flight.size()) >= b->desc.pipeline_depth) return PK_OK;
    pk_batch::Flight f;
    int32_t cnt = 0;
    for (size_t i = 0; i < b->slots.size(); ++i)
    {
        pk_batch::Slot &s = b->slots[i];
        const bool go = s.live && int(s.pending.size()) > s.in_flight;
        b->mask[i] = go ? 1 : 0;
        if (!go) continue;
        f.served.push_back({int32_t(i), s.pending[size_t(s.in_flight)]});
        s.in_flight++;
        ++cnt;
    }
    if (cnt == 0) return PK_OK;
    pk_world *w = b->w;
    for (size_t i = 0; i < b->slots.size(); ++i) w->worlds[i].active = b->mask[i];
    if (w->eng->set_active_mask_async(b->mask.data(), b->desc.max_worlds))
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    // The step is replayed from a CUDA graph: one launch instead of ~60. Its launch shapes depend
    // on the solver schedule (which changes with admissions and retirements) and the tuning, so it
    // is captured again after either changed; the active mask lives in device memory.
    if (w->order_dirty || b->graph_version != w->launch_version)
    {
        if (int rc = flush_shapes(w)) return rc;
        if (int rc = flush_order(w, true)) return rc;
        if (w->eng->capture_graph(b->desc.dt))
        {
            g_last_cuda = w->eng->last_error();
            return PK_ERR_CUDA;
        }
        b->graph_version = w->launch_version;
        b->captures++;
    }
    if (int rc = pk_world_step_graph(w)) return rc;
    if (!b->spare.empty())
    {
        f.ev = b->spare.back();
        b->spare.pop_back();
    }
    else if (cudaError_t e = cudaEventCreateWithFlags(&f.ev, cudaEventDisableTiming); e != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    if (cudaError_t e = cudaEventRecord(f.ev, static_cast<cudaStream_t>(w->eng->stream())); e != cudaSuccess)
    {
        g_last_cuda = int(e);
        return PK_ERR_CUDA;
    }
    b->flight.push_back(std::move(f));
    b->steps++;
    if (nworlds) *nworlds = cnt;
    return PK_OK;
}

int pk_batch_poll(pk_batch *b, pk_batch_event *out, int32_t cap, int32_t *n, int32_t wait)
{
    if (!b || !n || cap < 0 || (cap > 0 && !out)) return PK_ERR_INVALID;
    bool first = true;
    while (!b->flight.empty())
    {
        pk_batch::Flight &f = b->flight.front();
        cudaError_t e = (wait && first) ? cudaEventSynchronize(f.ev) : cudaEventQuery(f.ev);
        if (e == cudaErrorNotReady) break;
        if (e != cudaSuccess)
        {
            g_last_cuda = int(e);
            return PK_ERR_CUDA;
        }
        first = false;
        for (auto &[wid, tag] : f.served)
        {
            pk_batch::Slot &s = b->slots[size_t(wid)];
            s.pending.pop_front();
            s.in_flight--;
            pk_batch_event ev{};
            ev.tag = tag;
            ev.world = wid;
            ev.kind = PK_BATCH_STEPPED;
            b->ready.push_back(ev);
            if (s.retiring && s.pending.empty() && s.in_flight == 0)
                if (int rc = batch_retire_now(b, wid)) return rc;
        }
        b->spare.push_back(f.ev);
        b->flight.pop_front();
    }
    int32_t k = 0;
    while (k < cap && !b->ready.empty())
    {
        out[k++] = b->ready.front();
        b->ready.pop_front();
    }
    *n = k;
    return PK_OK;
}

int pk_batch_stats(pk_batch *b, pk_batch_info *st)
{
    if (!b || !st) return PK_ERR_INVALID;
    std::memset(st, 0, sizeof(*st));
    st->pool_bodies = b->pool_bodies;
    st->bodies_in_use = b->bodies_in_use;
    st->worlds_free = int32_t(b->free_ids.size());
    st->worlds_live = b->desc.max_worlds - st->worlds_free;
    st->steps_in_flight = int32_t(b->flight.size());
    st->steps = b->steps;
    st->graph_captures = b->captures;
    int64_t pend = 0;
    for (const auto &s : b->slots) pend += int64_t(s.pending.size());
    st->pending_requests = pend;
    return PK_OK;
}

int pk_batch_read_world(pk_batch *b, int32_t world, double *out14, int32_t cap, int32_t *n)
{
    if (!b || !n || world < 0 || world >= b->desc.max_worlds) return PK_ERR_INVALID;
    pk_world *w = b->w;
    const pk_batch::Slot &s = b->slots[size_t(world)];
    if (!s.live) return PK_ERR_STALE_HANDLE;
    const SubWorld &sw = w->worlds[size_t(world)];
    std::vector<double> rows(size_t(w->nslots) * 14);
    if (w->eng->read_bodies(rows.data(), w->nslots) < 0)
    {
        g_last_cuda = w->eng->last_error();
        return PK_ERR_CUDA;
    }
    int32_t k = 0;
    for (size_t l = 0; l < sw.local_slot.size(); ++l)
    {
        if (!sw.local_alive[l]) continue;
        if (k < cap && out14)
            std::memcpy(out14 + size_t(k) * 14, rows.data() + size_t(sw.local_slot[l]) * 14, 14 * sizeof(double));
        ++k;
    }
    *n = k;
    return PK_OK;
}

} // extern "C"
