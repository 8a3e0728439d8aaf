// pk_engine.cuh — the GPU world step: body state in HBM, one kernel per stage.
//
// Stage order is that of world::step_impl (src/world.cpp:20-56):
//   k_integrate_vel   gravity + semi-implicit velocity update (integrate.h:36-40, particle.h:72-79),
//                     world AABB of the rotated mesh bounds (mesh.cpp:398, bounds.h:144-158) and the
//                     fat-box hysteresis of dynamic_bvh::update_leaf (bvh.cpp:475-514)
//   k_morton + radix sort       the step's leaves grouped by world (static ones last), Morton order
//   k_broad_small               overlap pairs of worlds up to kBroadMax leaves: sweep and prune in
//                               shared memory (collision_phases.h:377-436)
//   k_lbvh_build + k_lbvh_refit + k_traverse    the same for larger worlds, on a per-step LBVH
//   pair radix sort + assembly  the step's sorted pair list, world by world
//   k_old_index, k_narrow_pre, k_narrow_axis, k_narrow_gjk, k_narrow_epa
//                     GJK/EPA + manifold update + begin/end events (collision_phases.h:244-320)
//   k_contact_setup   contact Jacobians (constraint.h:874-953, 1052-1104)
//   k_solve_world     colouring + warm start + sequential impulses, one CTA per world
//                     (constraint.h:1107-1201)
//   k_integrate_pos   position/orientation update and cached inertia (integrate.h:42-46,
//                     particle.h:140-146)
// The pair set equals the reference's incremental one: a pair of bodies of one world exists when
// their fat boxes overlap (inclusive compares), not both are static, and one of them was
// reinserted in the tree at or after the step in which the younger of the two was created.
#pragma once

#include "pk_engine_api.h"
#include "pk_math.cuh"
#include "pk_narrow.cuh"
#include "pk_sort.cuh"

#include <climits>
#include <cooperative_groups.h>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>
#include <cstdio>
#include <cuda_runtime.h>
#include <vector>

namespace pk
{

enum : uint32_t
{
    BODY_ALIVE = 1u,
    BODY_STATIC = 2u,
};

// Device status bits (OR-ed into a word the host reads after a step).
enum : int
{
    ST_PAIR_OVERFLOW = 1 << 0,
    ST_EPA_CAP = 1 << 1,
    ST_COLOUR_CAP = 1 << 2,
    ST_TRAVERSAL_STACK = 1 << 3,
    ST_NAN = 1 << 4,
    ST_CONTACT_OVERFLOW = 1 << 5,
};

constexpr int kMaxColours = 512;
constexpr int kPairClasses = 16; // GJK work classes: the support kinds of a pair's two shapes (4 x 4)
// Worlds with at most this many local indices are coloured first-fit in pair order (one thread,
// a 128-bit mask of used colours per body in shared memory); larger worlds by claiming rounds.
constexpr int kFirstFitMax = 4096;
constexpr int kSolveMaxThreads = 512; // largest solver CTA (FP32 form; the FP64 form's register need caps it at 256)
template <class T> constexpr int solve_max_threads() { return sizeof(T) == 4 ? kSolveMaxThreads : 256; }
constexpr uint32_t kLeafBit = 0x80000000u;
// Worlds with at most this many leaves find their pairs by testing all pairs in shared memory
// (k_broad_small); larger worlds traverse their LBVH.
constexpr int kBroadMax = 2304;

template <class T> struct Pose
{
    T p[3];
    T q[4];
};
template <class T> struct Vel
{
    T v[3];
    T w[3];
};
template <class T> struct Params
{
    T mass, inv_mass, restitution, friction;
    T il[9];
    T il_inv[9];
};
struct Meta
{
    uint32_t world, local, shape, flags;
    int32_t created, reinserted;
};
template <class T> struct Contact
{
    T n[3], la[3], lb[3], depth;
    double imp[3];
};
template <class T> struct alignas(32) Manifold // header in one 32-byte sector
{
    int n;
    int pad;
    T sep[3]; // a direction that separated the pair when it was last found apart (zero: none)
    Contact<T> c[4];
};
template <class T> struct Row
{
    T n[3], wa_n[3], wb_n[3];
    T meff_n, bias;
    T t1[3], wa_t1[3], wb_t1[3];
    T meff_t1;
    T t2[3], wa_t2[3], wb_t2[3];
    T meff_t2;
    T inv11, inv12, inv22, mu;
    T pad; // 36 values: whole 16-byte vectors
};
static_assert(sizeof(Row<float>) == 144 && sizeof(Row<double>) == 288, "Row is loaded as 16-byte vectors");
// FP32 form's row: besides the Jacobian (direction, angular parts wa/wb) it stores the velocity
// change per unit impulse of each body's rotation, ka = I_a^-1 wa and kb = I_b^-1 wb (computed
// anyway for the effective masses), so applying an impulse is three multiply-adds per body and
// the sweep reads no inertia tensors.
struct RowF
{
    float n[3], wa_n[3], wb_n[3], ka_n[3], kb_n[3];
    float t1[3], wa_t1[3], wb_t1[3], ka_t1[3], kb_t1[3];
    float t2[3], wa_t2[3], wb_t2[3], ka_t2[3], kb_t2[3];
    float meff_n, bias, inv11, inv12, inv22, mu;
    float pad;
};
static_assert(sizeof(RowF) == 208, "RowF is loaded as 16-byte vectors");
template <class T> struct RowSel
{
    using type = Row<T>;
};
template <> struct RowSel<float>
{
    using type = RowF;
};
template <class T> using RowT = typename RowSel<T>::type;

// Joints (constraint.h:139-865): type as constraint_type (0 distance, 1 ball_socket, 2 hinge,
// 3 slider, 4 weld, 5 spring); bodies as device slots and world-local indices; the parameters
// fixed at creation.
template <class T> struct JointDev
{
    int type, a, b, local_a, local_b, pad[3];
    T la[3], lb[3]; // local anchors
    T axa[3], axb[3]; // hinge: local axes; slider: local axis of a
    T va[3], wa[3];   // hinge: basis of axa; slider: local tangents of a
    T qrel[4];        // slider, weld: conj(q_a) q_b at creation
    T distance, stiffness, damping;
};
// One joint row (jacobian_row, constraint.h:29-88); the clamp bounds are -+DBL_MAX for all joints.
template <class T> struct JRow
{
    T Jv[3], Jwa[3], Jwb[3];
    T meff, bias, gamma;
};
constexpr int kJointMaxRows = 6;
template <class T> struct WorldParams
{
    T g[3];
    T gnorm;
    int active;
    int pad;
};

// Where a shape's data lives: vertices, vertex-block bounds (clusters of 8) and bounds of groups of
// 8 clusters, the latter two in one array of (centre xyz, radius) records.
struct ShapeRange
{
    int vstart, nverts, cstart, ncl, gstart, ngr, uv_stacks, uv_sectors; // uv: 0 unless a UV sphere
};

template <class T> struct Dev
{
    // bodies
    Pose<T> *pose;
    Vel<T> *vel;
    T *iw;
    T *iwinv;
    Params<T> *prm;
    Aabb<T> *tbox;
    Meta *meta;
    const int *nslots;
    // shapes
    const T *verts;
    const float *verts32;    // FP64 form: the vertices rounded to FP32 (separation screens); else null
    const float *shape32;    // FP64 form: per shape its local box and bounding radius in FP32 (8 floats)
    float4 *pose32;          // FP64 form: per body its position and orientation (w, x, y, z) in FP32
    const ShapeRange *shape_range;
    const Aabb<T> *shape_box;
    const T *clusters;       // 4 per cluster: centre xyz, radius
    const T *shape_rmax;     // bounding radius about the shape origin
    // worlds
    WorldParams<T> *wp;
    unsigned *wbounds;
    int *wroot;
    int *wleaf_lo;         // each world's range of leaf positions in the sorted leaf list
    int *wleaf_hi;
    int *wlive;            // bodies of each world that take part in this step's broadphase
    int *all_small;        // 1 while no world of the step has more than kBroadMax such bodies
    int *mstart;
    int *mend;
    int max_worlds;
    // broadphase
    uint64_t *mkey;
    uint64_t *mval;
    int *nleaf;
    float4 *nodes;
    int *parent;     // parent of internal node i
    int *leaf_parent;
    int *refit_flag;
    // pairs
    uint64_t *pkey;
    uint64_t *pval;
    int *npairs;
    int pair_cap;
    // manifolds
    Manifold<T> *man_old;
    uint64_t *key_old;
    uint64_t *val_old;     // slot pairs of last step's sorted pairs
    int *mstart_old;       // last step's pair range of each world
    int *mend_old;
    int *nstart;           // active world: its range in the sorted list of new pairs;
    int *nend;             // idle world: 0 and the number of its kept pairs
    int *nnew;             // pairs found by this step's traversal
    int *npairs_old;
    Manifold<T> *man_new;
    uint8_t *event;
    int *old_idx;          // per pair: index of last step's manifold or -1
    // GJK / EPA work lists. Pairs involving a large (clustered) mesh fill a list from its end,
    // the others from its start, so each warp works on one cost class; heavy items run first.
    int *gjk_list;
    int *gjk_count;        // light items
    int *gjk_count_heavy;
    int *gjk_list2;        // the items the separating-direction check left for GJK, same two classes
    int *gcls;             // per shape-kind class of those items: count[16], start[16], cursor[16]
    int *gjk2_count;
    int *gjk2_count_heavy;
    int *epa_list;         // contact_cap entries: light items from the start, heavy ones from the end
    Simplex<T> *epa_simplex;
    int *epa_count;
    int *epa_count_heavy;
    int *epa_total;        // items admitted to the EPA list (at most contact_cap)
    unsigned long long *np_iters; // [0] GJK iterations, [1] EPA expansions, [2] of which in heavy pairs
    unsigned long long *np_verts; // vertices a linear support scan visits, summed over the supports
    int *clist;            // pairs of active worlds whose new manifold holds contacts (any order)
    int *ccount;
    // Contact rows live at the pair's position in clist (rowidx), so they take memory only for the
    // pairs that have contacts: at most contact_cap of them per step.
    int contact_cap;
    int *rowidx;           // per pair: its row block (valid while rowmask != 0)
    RowT<T> *rows;         // 4 per row block, read-only while the solver sweeps
    double *racc;          // 12 per row block: accumulated impulses (normal, t1, t2) of the 4 rows
    float *raccf;          // FP32 form: running totals in FP32 (clamp decisions, warm start)
    float *rdel;           // FP32 form: this step's change, added to racc once after the sweeps
    const JointDev<T> *joints; // ordered by (world, type, arena slot)
    JRow<T> *jrows;        // kJointMaxRows per joint, built every step
    int *jnrows;           // rows built for each joint this step
    double *jacc;          // kJointMaxRows accumulated impulses per joint (kept across steps)
    int *jstart;           // each world's joint range
    int *jend;
    const int *njoints;
    uint8_t *rowmask;
    int *colour;      // solver scratch: compacted active manifolds of each world
    int *colour_tmp;  // solver scratch: colour of each compacted manifold
    int *pair_colour; // colour of each pair of the last step (-2: no contact rows)
    uint64_t *owner;       // colouring rounds: the lowest key on each body
    ulonglong2 *used;      // parallel first fit: colours (0..127) taken on each body
    uint32_t *order;
    int *ncolours;
    const int *world_order; // solver CTA -> world, largest worlds first
    uint4 *srec;            // solve records of the active manifolds, colour-ordered per world
    uint4 *crec;            // the same records in pair order (colouring input)
    const int *world_nlocal; // local indices in use per world (bounds the shared-memory cache)
    // control
    int *status;
    int *epoch;
    int lbits, wbits, iterations;
};

// ------------------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned f2ord(float f)
{
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u)
{ return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u); }

__device__ __forceinline__ float down_f(double x) { return __double2float_rd(x); }
__device__ __forceinline__ float up_f(double x) { return __double2float_ru(x); }
__device__ __forceinline__ float down_f(float x) { return x; }
__device__ __forceinline__ float up_f(float x) { return x; }

template <class T> __device__ __forceinline__ V3<T> ld3(const T *a) { return {a[0], a[1], a[2]}; }
template <class T> __device__ __forceinline__ void st3(T *a, V3<T> v)
{
    a[0] = v.x;
    a[1] = v.y;
    a[2] = v.z;
}
template <class T> __device__ __forceinline__ Qt<T> ldq(const T *a) { return {a[0], a[1], a[2], a[3]}; }

__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Slot in a compacted list for every active lane of the warp: one atomic per warp.
__device__ __forceinline__ int warp_push(int *counter)
{
    unsigned m = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// Adds every active lane's value to a 64-bit counter: one atomic per warp.
__device__ __forceinline__ void warp_add(unsigned long long *counter, unsigned v)
{
    const unsigned m = __activemask();
    const unsigned s = __reduce_add_sync(m, v);
    if (int(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(counter, (unsigned long long)s);
}

// Slot in a per-key list for every active lane: one atomic per key present in the warp.
__device__ __forceinline__ int warp_push_key(int *counters, int key)
{
    const unsigned m = __match_any_sync(__activemask(), key);
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counters + key, __popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// Vertices the reference's support (mesh::support, mesh.cpp:341-358, a linear first-strict-max
// scan) visits for one Minkowski support of the pair; a support costs the reference 5 FLOP per
// vertex (a 3-term dot product and a compare).
template <class T> __device__ __forceinline__ unsigned scan_verts(const ShapeRef<T> &A, const ShapeRef<T> &B)
{
    return unsigned((A.kind == SHAPE_MESH ? A.nverts : 8) + (B.kind == SHAPE_MESH ? B.nverts : 8));
}

// Key of a manifold in a round of parallel first fit (colour_rounds_pick / _claim / _commit): its
// tentative colour on top, then a scramble of its pair's world-local indices (MurmurHash3's 64-bit
// finaliser), then its position in the world's key order. Of the uncoloured manifolds on one body,
// the lowest key keeps its colour in a round; the scramble keeps neighbouring manifolds from
// forming long chains of falling priority in a dense pile. Local indices and key order do not
// depend on the batch, so a world gets the same colours alone and in any mix.
__host__ __device__ __forceinline__ uint64_t ff_key(int colour, uint32_t la, uint32_t lb, uint32_t pos)
{
    const uint32_t lo = la < lb ? la : lb, hi = la < lb ? lb : la;
    uint64_t x = (uint64_t(lo) << 32) | hi;
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return (uint64_t(uint32_t(colour)) << 56) | ((x >> 40) << 32) | pos;
}

#define PK_GRID_STRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += blockDim.x * gridDim.x)

// ------------------------------------------------------------------------------------------------
// step begin: per-world resets
// ------------------------------------------------------------------------------------------------
template <class T> __global__ void k_begin_step(Dev<T> d)
{
    PK_GRID_STRIDE(w, d.max_worlds)
    {
        d.wbounds[6 * w + 0] = d.wbounds[6 * w + 1] = d.wbounds[6 * w + 2] = 0xFFFFFFFFu;
        d.wbounds[6 * w + 3] = d.wbounds[6 * w + 4] = d.wbounds[6 * w + 5] = 0u;
        d.wroot[w] = -1;
        d.wleaf_lo[w] = 0;
        d.wleaf_hi[w] = 0;
        d.wlive[w] = 0;
        d.mstart[w] = 0;
        d.mend[w] = 0;
        d.nstart[w] = 0;
        d.nend[w] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        *d.npairs = 0;
        *d.nleaf = 0;
        *d.gjk_count = 0;
        *d.epa_count = 0;
        *d.gjk_count_heavy = 0;
        *d.epa_count_heavy = 0;
        *d.gjk2_count = 0;
        *d.gjk2_count_heavy = 0;
        for (int c = 0; c < kPairClasses; ++c) d.gcls[c] = 0;
        *d.ccount = 0;
        *d.epa_total = 0;
        *d.all_small = 1;
        d.np_iters[0] = d.np_iters[1] = d.np_iters[2] = 0ull;
        *d.np_verts = 0ull;
        *d.epoch += 1;
    }
}

// ------------------------------------------------------------------------------------------------
// velocity integration, world AABB, fat-box hysteresis, world bounds for Morton codes
// ------------------------------------------------------------------------------------------------
template <class T> __device__ __forceinline__ Aabb<T> world_bounds(const Aabb<T> &lb, Qt<T> q, V3<T> p)
{
    // aabb * quat: corner 0 is the min corner, corners 1..7 follow bit order (bounds.h:65-71, 144-158)
    V3<T> p0 = rotate(q, lb.mn);
    Aabb<T> r{p0, p0};
#pragma unroll
    for (unsigned i = 1; i < 8; ++i)
    {
        V3<T> c{(i & 1) ? lb.mx.x : lb.mn.x, (i & 2) ? lb.mx.y : lb.mn.y, (i & 4) ? lb.mx.z : lb.mn.z};
        V3<T> pt = rotate(q, c);
        r.mn.x = tmin(r.mn.x, pt.x);
        r.mn.y = tmin(r.mn.y, pt.y);
        r.mn.z = tmin(r.mn.z, pt.z);
        r.mx.x = tmax(r.mx.x, pt.x);
        r.mx.y = tmax(r.mx.y, pt.y);
        r.mx.z = tmax(r.mx.z, pt.z);
    }
    return {r.mn + p, r.mx + p};
}

template <class T> __global__ void k_integrate_vel(Dev<T> d, T dt)
{
    const int n = *d.nslots;
    const int epoch = *d.epoch;
    PK_GRID_STRIDE(i, n)
    {
        Meta m = d.meta[i];
        const bool live = (m.flags & BODY_ALIVE) && d.wp[m.world].active;
        Aabb<T> tb{};
        if (live) tb = d.tbox[i];
        if (live && d.pose32)
        {
            // the FP32 copy the narrowphase's separation screens read this step
            const Pose<T> &ps = d.pose[i];
            d.pose32[2 * i] = make_float4(float(ps.p[0]), float(ps.p[1]), float(ps.p[2]), 0.0f);
            d.pose32[2 * i + 1] = make_float4(float(ps.q[0]), float(ps.q[1]), float(ps.q[2]), float(ps.q[3]));
        }
        if (live && !(m.flags & BODY_STATIC))
        {
            const Params<T> &pr = d.prm[i];
            const WorldParams<T> &wp = d.wp[m.world];
            Vel<T> ve = d.vel[i];
            V3<T> v = ld3(ve.v), w = ld3(ve.w);
            // apply_force(g*m): acc = 0 + (g*m)*inv_mass; v += acc*dt
            V3<T> acc = (ld3(wp.g) * pr.mass) * pr.inv_mass;
            v = v + acc * dt;
            // angular_accel = I_w^-1 (tau - w x (I_w w)), tau = 0
            V3<T> c = cross(w, matvec(d.iw + 9 * i, w));
            V3<T> zero{T(0), T(0), T(0)};
            V3<T> aa = matvec(d.iwinv + 9 * i, zero - c);
            w = w + aa * dt;
            st3(ve.v, v);
            st3(ve.w, w);
            d.vel[i] = ve;
            const Pose<T> &ps = d.pose[i];
            Aabb<T> tru = world_bounds(d.shape_box[m.shape], ldq(ps.q), ld3(ps.p));
            if (!aabb_contains(tb, tru))
            {
                const T margin = T(0.1);
                V3<T> mv{margin, margin, margin};
                Aabb<T> nb{tru.mn - mv, tru.mx + mv};
                V3<T> disp = v * dt;
                if (disp.x < T(0)) nb.mn.x = nb.mn.x + disp.x; else nb.mx.x = nb.mx.x + disp.x;
                if (disp.y < T(0)) nb.mn.y = nb.mn.y + disp.y; else nb.mx.y = nb.mx.y + disp.y;
                if (disp.z < T(0)) nb.mn.z = nb.mn.z + disp.z; else nb.mx.z = nb.mx.z + disp.z;
                tb = nb;
                d.tbox[i] = nb;
                d.meta[i].reinserted = epoch;
            }
        }
        // world bounds of the fat-box centres (Morton quantisation, sweep axis): reduced over the
        // lanes of the same world first, so a warp of one world does 6 atomics, not 6 per body
        const unsigned peers = __match_any_sync(__activemask(), live ? int(m.world) : -1);
        if (live)
        {
            const unsigned ox = f2ord(float(T(0.5) * (tb.mn.x + tb.mx.x)));
            const unsigned oy = f2ord(float(T(0.5) * (tb.mn.y + tb.mx.y)));
            const unsigned oz = f2ord(float(T(0.5) * (tb.mn.z + tb.mx.z)));
            const unsigned lx = __reduce_min_sync(peers, ox), ly = __reduce_min_sync(peers, oy),
                           lz = __reduce_min_sync(peers, oz);
            const unsigned hx = __reduce_max_sync(peers, ox), hy = __reduce_max_sync(peers, oy),
                           hz = __reduce_max_sync(peers, oz);
            if (int(threadIdx.x & 31) == __ffs(peers) - 1)
            {
                atomicAdd(d.wlive + m.world, __popc(peers));
                unsigned *wb = d.wbounds + 6 * m.world;
                atomicMin(wb + 0, lx);
                atomicMin(wb + 1, ly);
                atomicMin(wb + 2, lz);
                atomicMax(wb + 3, hx);
                atomicMax(wb + 4, hy);
                atomicMax(wb + 5, hz);
            }
        }
    }
}

// ------------------------------------------------------------------------------------------------
// LBVH: Morton keys (world id above 30 Morton bits), Karras build, bottom-up refit
// ------------------------------------------------------------------------------------------------
// Keys of the bodies of active worlds only, compacted (one atomic per warp); the sort and the
// LBVH then cover just those bodies.
template <class T> __global__ void k_morton(Dev<T> d, bool all_worlds = false)
{
    const int n = *d.nslots;
    PK_GRID_STRIDE(i, n)
    {
        Meta m = d.meta[i];
        if ((m.flags & BODY_ALIVE) && (all_worlds || d.wp[m.world].active))
        {
            if (!all_worlds && d.wlive[m.world] > kBroadMax) *d.all_small = 0; // some world traverses
            Aabb<T> tb = d.tbox[i];
            const unsigned *wb = d.wbounds + 6 * m.world;
            float c[3] = {float(T(0.5) * (tb.mn.x + tb.mx.x)), float(T(0.5) * (tb.mn.y + tb.mx.y)),
                          float(T(0.5) * (tb.mn.z + tb.mx.z))};
            uint32_t code = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                float lo = ord2f(wb[a]), hi = ord2f(wb[3 + a]);
                float ext = hi - lo;
                float u = ext > 0.f ? (c[a] - lo) / ext : 0.f;
                u = fminf(fmaxf(u, 0.f), 1.f);
                uint32_t q = min(1023u, uint32_t(u * 1024.f));
                code |= spread10(q) << (2 - a);
            }
            int slot = warp_push(d.nleaf);
            // world | static | Morton: a world's static bodies form their own subtree (the reference
            // keeps them in a separate tree too), so queries prune dynamic subtrees by position alone
            d.mkey[slot] = (uint64_t(m.world) << 31) | (uint64_t((m.flags & BODY_STATIC) ? 1 : 0) << 30) | code;
            d.mval[slot] = uint64_t(i);
        }
    }
}

__device__ __forceinline__ int lbvh_delta(const uint64_t *k, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz(uint32_t(i) ^ uint32_t(j));
    return __clzll(a ^ b);
}

// With `tree_if_needed`, the internal nodes are built only when some world of the step traverses
// (all_small == 0): the all-pairs worlds need just their leaf ranges, and their leaves may then be
// ordered by the world and static bits alone.
template <class T> __global__ void k_lbvh_build(Dev<T> d, const uint64_t *__restrict__ skey, bool tree_if_needed = false)
{
    const int n = *d.nleaf;
    const int ninner = (tree_if_needed && *d.all_small) ? 0 : n - 1;
    PK_GRID_STRIDE(i, ninner)
    {
        int dir = (lbvh_delta(skey, n, i, i + 1) - lbvh_delta(skey, n, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = lbvh_delta(skey, n, i, i - dir);
        int lmax = 2;
        while (lbvh_delta(skey, n, i, i + lmax * dir) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (lbvh_delta(skey, n, i, i + (l + t) * dir) > dmin) l += t;
        int j = i + l * dir;
        int dnode = lbvh_delta(skey, n, i, j);
        int s = 0;
        int div = 2;
        int t = (l + div - 1) / div;
        while (true)
        {
            if (lbvh_delta(skey, n, i, i + (s + t) * dir) > dnode) s += t;
            if (t <= 1) break;
            div <<= 1;
            t = (l + div - 1) / div;
        }
        int gamma = i + s * dir + min(dir, 0);
        int first = min(i, j), last = max(i, j);
        uint32_t left = (first == gamma) ? (uint32_t(gamma) | kLeafBit) : uint32_t(gamma);
        uint32_t right = (last == gamma + 1) ? (uint32_t(gamma + 1) | kLeafBit) : uint32_t(gamma + 1);
        d.nodes[4 * i + 0].w = __uint_as_float(left);
        d.nodes[4 * i + 2].w = __uint_as_float(right);
        if (left & kLeafBit)
            d.leaf_parent[gamma] = i;
        else
            d.parent[gamma] = i;
        if (right & kLeafBit)
            d.leaf_parent[gamma + 1] = i;
        else
            d.parent[gamma + 1] = i;
        if (i == 0) d.parent[0] = -1;
        // the node spanning exactly one world's leaves is that world's root
        uint64_t wf = skey[first] >> 31, wl = skey[last] >> 31;
        if (wf == wl && (first == 0 || (skey[first - 1] >> 31) != wf) && (last == n - 1 || (skey[last + 1] >> 31) != wl))
            d.wroot[wf] = i;
    }
    // each world's leaf range; single-leaf worlds
    PK_GRID_STRIDE(j, n)
    {
        uint64_t w = skey[j] >> 31;
        const bool first = j == 0 || (skey[j - 1] >> 31) != w, last = j == n - 1 || (skey[j + 1] >> 31) != w;
        if (first) d.wleaf_lo[w] = j;
        if (last) d.wleaf_hi[w] = j + 1;
        if (first && last) d.wroot[w] = int(uint32_t(j) | kLeafBit);
    }
}

// With `skip_small`, the leaves of worlds the all-pairs pass covers are left out: only the larger
// worlds' subtrees (below their roots) get boxes.
template <class T> __global__ void k_lbvh_refit(Dev<T> d, const uint64_t *__restrict__ sval, bool skip_small = false)
{
    const int n = *d.nleaf;
    if (n < 2 || (skip_small && *d.all_small)) return;
    PK_GRID_STRIDE(j, n)
    {
        int slot = int(sval[j]);
        if (skip_small)
        {
            const int w = int(d.meta[slot].world);
            if (d.wleaf_hi[w] - d.wleaf_lo[w] <= kBroadMax) continue;
        }
        Aabb<T> b = d.tbox[slot];
        float mn[3] = {down_f(b.mn.x), down_f(b.mn.y), down_f(b.mn.z)};
        float mx[3] = {up_f(b.mx.x), up_f(b.mx.y), up_f(b.mx.z)};
        int p = d.leaf_parent[j];
        uint32_t me = uint32_t(j) | kLeafBit;
        // .w of a child's max box: (last leaf position in the child << 1) | (child holds a static body)
        uint32_t span = (uint32_t(j) << 1) | ((d.meta[slot].flags & BODY_STATIC) ? 1u : 0u);
        while (true)
        {
            int c = (__float_as_uint(d.nodes[4 * p].w) == me) ? 0 : 1;
            float4 *slotp = d.nodes + 4 * p + 2 * c;
            float wv = slotp[0].w;
            __stcg(slotp + 0, make_float4(mn[0], mn[1], mn[2], wv));
            __stcg(slotp + 1, make_float4(mx[0], mx[1], mx[2], __uint_as_float(span)));
            __threadfence();
            if (atomicAdd(d.refit_flag + p, 1) == 0) break;
            __threadfence();
            float4 a0 = __ldcg(d.nodes + 4 * p + 0), a1 = __ldcg(d.nodes + 4 * p + 1);
            float4 b0 = __ldcg(d.nodes + 4 * p + 2), b1 = __ldcg(d.nodes + 4 * p + 3);
            mn[0] = fminf(a0.x, b0.x);
            mn[1] = fminf(a0.y, b0.y);
            mn[2] = fminf(a0.z, b0.z);
            mx[0] = fmaxf(a1.x, b1.x);
            mx[1] = fmaxf(a1.y, b1.y);
            mx[2] = fmaxf(a1.z, b1.z);
            // the right child ends the node's leaf range; statics in either child
            span = (__float_as_uint(b1.w) & ~1u) | ((__float_as_uint(a1.w) | __float_as_uint(b1.w)) & 1u);
            int pp = d.parent[p];
            if (pp < 0) break;
            me = uint32_t(p);
            p = pp;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// pair search: each dynamic body walks its world's subtree
// ------------------------------------------------------------------------------------------------
template <class T> __device__ __forceinline__ bool pair_allowed(const Meta &a, const Meta &b)
{
    int re = a.reinserted > b.reinserted ? a.reinserted : b.reinserted;
    int cr = a.created > b.created ? a.created : b.created;
    return re >= cr;
}

// Threads take bodies in Morton (leaf) order, so a warp's queries are spatially close and walk
// similar paths through the tree. A pair of dynamic bodies is emitted by the one earlier in that
// order, so a query skips every subtree that ends at or before its own leaf and holds no static
// body (static bodies do not query; their pairs come from the dynamic side).
template <class T> __global__ void k_traverse(Dev<T> d, const uint64_t *__restrict__ sval)
{
    const int n = *d.all_small ? 0 : *d.nleaf; // no world traverses in this step
    PK_GRID_STRIDE(leaf, n)
    {
        const int i = int(sval[leaf]);
        Meta mi = d.meta[i];
        if (!(mi.flags & BODY_ALIVE) || (mi.flags & BODY_STATIC) || !d.wp[mi.world].active) continue;
        if (d.wleaf_hi[mi.world] - d.wleaf_lo[mi.world] <= kBroadMax) continue; // all-pairs pass
        int root = d.wroot[mi.world];
        if (root < 0 || (uint32_t(root) & kLeafBit)) continue;
        Aabb<T> qb = d.tbox[i];
        float qmn[3] = {down_f(qb.mn.x), down_f(qb.mn.y), down_f(qb.mn.z)};
        float qmx[3] = {up_f(qb.mx.x), up_f(qb.mx.y), up_f(qb.mx.z)};
        // the node being visited stays in a register: a visit descends into one child it overlaps
        // and pushes the other, and pops only when neither child is an internal node to visit
        int stack[96];
        int sp = 0;
        int node = root;
        while (node >= 0)
        {
            const float4 *nd = d.nodes + 4 * node;
            int next = -1;
#pragma unroll
            for (int c = 0; c < 2; ++c)
            {
                float4 bmn = nd[2 * c], bmx = nd[2 * c + 1];
                const uint32_t span = __float_as_uint(bmx.w);
                if (int(span >> 1) <= leaf && !(span & 1u)) continue; // only earlier dynamic leaves
                if (!(bmn.x <= qmx[0] && bmx.x >= qmn[0] && bmn.y <= qmx[1] && bmx.y >= qmn[1] &&
                      bmn.z <= qmx[2] && bmx.z >= qmn[2]))
                    continue;
                uint32_t ch = __float_as_uint(bmn.w);
                if (ch & kLeafBit)
                {
                    const int pos = int(ch & ~kLeafBit);
                    int sj = int(sval[pos]);
                    if (sj == i) continue;
                    Meta mj = d.meta[sj];
                    bool sj_static = (mj.flags & BODY_STATIC) != 0;
                    if (!sj_static && pos < leaf) continue; // dynamic pairs once, from the earlier leaf
                    // FP32 form: the node boxes are the exact fat boxes, so the node test was the exact test
                    if constexpr (!std::is_same<T, float>::value)
                        if (!aabb_intersects(qb, d.tbox[sj])) continue;
                    if (!pair_allowed<T>(mi, mj)) continue;
                    uint32_t lo = min(mi.local, mj.local), hi = max(mi.local, mj.local);
                    uint32_t slo = (mi.local < mj.local) ? uint32_t(i) : uint32_t(sj);
                    uint32_t shi = (mi.local < mj.local) ? uint32_t(sj) : uint32_t(i);
                    uint64_t key = (uint64_t(mi.world) << (2 * d.lbits)) | (uint64_t(lo) << d.lbits) | uint64_t(hi);
                    int slot = warp_push(d.npairs); // one atomic per group of lanes emitting together
                    if (slot < d.pair_cap)
                    {
                        d.pkey[slot] = key;
                        d.pval[slot] = (uint64_t(slo) << 32) | shi;
                    }
                    else
                        atomicOr(d.status, ST_PAIR_OVERFLOW);
                }
                else if (next < 0)
                    next = int(ch);
                else if (sp < 96)
                    stack[sp++] = int(ch);
                else
                    atomicOr(d.status, ST_TRAVERSAL_STACK);
            }
            node = next >= 0 ? next : (sp > 0 ? stack[--sp] : -1);
        }
    }
}

// Writes the pair of leaves ja, jb (positions lo + ja, lo + jb of the sorted leaf list) of world w
// at `slot`, or at a fresh slot of the pair list (slot < 0; pairs the reference does not pair yet
// are dropped there).
template <class T>
__device__ __forceinline__ void broad_emit(const Dev<T> &d, int w, int lo, const uint64_t *__restrict__ sval, int ja,
                                           int jb, int slot)
{
    const int i = int(sval[lo + ja]), sj = int(sval[lo + jb]);
    const Meta mi = d.meta[i], mj = d.meta[sj];
    if (slot < 0)
    {
        if (!pair_allowed<T>(mi, mj)) return;
        slot = atomicAdd(d.npairs, 1);
    }
    const uint32_t l0 = min(mi.local, mj.local), l1 = max(mi.local, mj.local);
    const uint32_t slo = (mi.local < mj.local) ? uint32_t(i) : uint32_t(sj);
    const uint32_t shi = (mi.local < mj.local) ? uint32_t(sj) : uint32_t(i);
    if (slot < d.pair_cap)
    {
        d.pkey[slot] = (uint64_t(w) << (2 * d.lbits)) | (uint64_t(l0) << d.lbits) | uint64_t(l1);
        d.pval[slot] = (uint64_t(slo) << 32) | shi;
    }
    else
        atomicOr(d.status, ST_PAIR_OVERFLOW);
}

// Broadphase of a world with at most kBroadMax leaves, one CTA per world, by sweep and prune in
// shared memory:
//  1. sort the leaves by the lower bound of their box along the axis on which the world's box
//     centres spread most (bitonic sort of (bound, leaf) keys, the stages of strides below a
//     warp's chunk on registers);
//  2. copy the leaves' boxes into shared memory in that order;
//  3. each sorted leaf a tests the leaves after it up to the first whose lower bound passes a's
//     upper bound (found by binary search), so every pair overlapping on the axis is met once,
//     from its earlier leaf: a lane per leaf, four candidates a turn, and the whole warp for the
//     rest of long windows; each thread queues the overlapping pairs it finds in its own slice of
//     a queue in shared memory;
//  4. the CTA drops queued pairs the reference does not pair yet (pair_allowed; only checked in a
//     world where some dynamic body was not reinserted since the newest creation), reserves its
//     range of the pair list with one atomic and writes the pairs there.
// A world's static leaves sort after its dynamic ones in the leaf list, so "leaf >= first static"
// marks them and static-static pairs are skipped. The pair test is the traversal's (closed
// intervals on the exact fat boxes), so the pair set is the same; sweep bounds are rounded outward
// to FP32, which only widens the window. A world whose pairs overflow the queue (the slices and the
// shared region after them) sweeps again and emits straight to the pair list.
constexpr int kBroadPow2 = 4096;  // sort capacity, a power of two >= kBroadMax, indices in 12 bits
constexpr int kBroadQueue = 10240; // queued pairs per world (two 12-bit sorted positions each)
static_assert(kBroadPow2 >= kBroadMax && kBroadPow2 <= 4096, "sort capacity");
constexpr int kBroadLaneSpan = 64; // window positions a lane tests before its warp helps
constexpr int kBroadLong = 32;     // long windows shared out to every warp of the CTA
static_assert(kBroadQueue * 4 >= kBroadPow2 * 8, "the sort keys live in the queue's space");

// Shared memory of a sweep-and-prune CTA: the queue, then per leaf its box in FP32 (rounded outward
// in the FP64 form), its lower bound on the sweep axis and its leaf index.
// Worlds are swept by size class, each class with CTAs and shared memory for its largest world,
// so the many small worlds of a batch do not each hold the shared memory of a 2,304-leaf world:
// (MINN, MAXN] leaves, QCAP queued pairs (a fuller queue moves the world to the second sweep).
template <int MAXN, int QCAP> constexpr size_t broad_smem_bytes()
{ return size_t(QCAP) * 4 + (6 * sizeof(float) + 4 + 2) * size_t(MAXN); }
// Bitonic stages of one sequence size on a warp's chunk of 32 * E keys held in registers (key
// cb + 32 k + lane in v[k]): strides below 32 exchange through shuffles, larger ones swap within
// the thread. Strides from min(size, 32 E) / 2 down to 1; the stride loop is unrolled, so every
// register index is a constant.
template <int E> __device__ __forceinline__ void bitonic_warp_stages(uint64_t (&v)[E], int cb, int lane, int size)
{
#pragma unroll
    for (int s = 16 * E; s > 0; s >>= 1)
    {
        if (s >= size) continue;
        if (s >= 32)
        {
            const int sk = s >> 5;
#pragma unroll
            for (int k = 0; k < E; ++k)
            {
                if (k & sk) continue;
                const bool asc = ((cb + 32 * k + lane) & size) == 0;
                const uint64_t a = v[k], b = v[k + sk];
                const bool sw = (a > b) == asc;
                v[k] = sw ? b : a;
                v[k + sk] = sw ? a : b;
            }
        }
        else
        {
            const bool lower = (lane & s) == 0;
#pragma unroll
            for (int k = 0; k < E; ++k)
            {
                const uint64_t o = __shfl_xor_sync(0xFFFFFFFFu, v[k], s);
                const bool take_min = lower == (((cb + 32 * k + lane) & size) == 0);
                v[k] = take_min ? (o < v[k] ? o : v[k]) : (o > v[k] ? o : v[k]);
            }
        }
    }
}

struct BroadClass
{
    int minn, maxn, qcap, threads;
};
constexpr BroadClass kBroadClasses[3] = {{1, 256, 4096, 128}, {256, 1024, 8192, 256}, {1024, kBroadMax, kBroadQueue, 512}};

template <class T, int MINN, int MAXN, int QCAP, int THREADS>
__global__ void __launch_bounds__(THREADS) k_broad_small(Dev<T> d, const uint64_t *__restrict__ skey,
                                                         const uint64_t *__restrict__ sval)
{
    static_assert(QCAP * 4 >= 8 * MAXN * 2 && MAXN <= 4096, "the sort keys live in the queue's space");
    // sort: E keys per thread, so that the CTA's warps hold the largest sequence in registers
    constexpr int MAXP = MAXN <= 256 ? 256 : (MAXN <= 512 ? 512 : (MAXN <= 1024 ? 1024 : (MAXN <= 2048 ? 2048 : 4096)));
    constexpr int E = MAXP / THREADS, SE = 32 * E;
    static_assert(E >= 1 && E * THREADS == MAXP && QCAP * 4 >= 8 * MAXP, "sort layout");
    // Queue: SLICE entries per thread (entry c of thread t at c * THREADS + t, so a warp's stores
    // touch distinct banks), then OCAP entries that threads with full slices take by an atomic.
    constexpr int SLICE = QCAP * 3 / 4 / THREADS, OCAP = QCAP - SLICE * THREADS;
    static_assert(SLICE >= 8 && OCAP > 0, "queue layout");
    extern __shared__ __align__(16) unsigned char broad_smem[];
    __shared__ int ndyn, ofill, cta_base, newest_created, oldest_reinserted, nlong;
    __shared__ unsigned coord_max; // largest |coordinate| of the world's FP32 boxes (as bits)
    __shared__ int long_at[kBroadLong], long_from[kBroadLong], long_to[kBroadLong];
    __shared__ int warp_count[16];
    const int w = blockIdx.x;
    const int lo = d.wleaf_lo[w];
    const int n = d.wleaf_hi[w] - lo;
    if (n < 2 || n <= MINN || n > MAXN) return;
    int P = SE; // sorted length: a power of two, at least one warp's chunk (keys past n are ~0)
    while (P < n) P <<= 1;
    uint32_t *queue = reinterpret_cast<uint32_t *>(broad_smem); // QCAP entries
    uint64_t *srt = reinterpret_cast<uint64_t *>(broad_smem);   // sort keys, before the sweep
    float *box = reinterpret_cast<float *>(queue + QCAP);        // 6 per sorted position: mn, mx
    float *lowax = reinterpret_cast<float *>(box + 6 * n);       // lower bound on the sweep axis
    uint16_t *leaf = reinterpret_cast<uint16_t *>(lowax + n);     // leaf index | 0x8000 if static
    const int tid = threadIdx.x, bs = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
    // sweep axis: the widest spread of box centres (world bounds kept for the Morton codes)
    const unsigned *wb = d.wbounds + 6 * w;
    int ax = 0;
    float ext = ord2f(wb[3]) - ord2f(wb[0]);
    for (int k = 1; k < 3; ++k)
    {
        const float e = ord2f(wb[3 + k]) - ord2f(wb[k]);
        if (e > ext)
        {
            ext = e;
            ax = k;
        }
    }
    if (tid == 0)
    {
        ndyn = n;
        ofill = 0;
        coord_max = 0u;
        newest_created = INT_MIN;
        oldest_reinserted = INT_MAX;
    }
    __syncthreads();
    int my_created = INT_MIN, my_reinserted = INT_MAX;
    for (int j = tid; j < P; j += bs)
    {
        if (j >= n)
        {
            srt[j] = ~0ull;
            continue;
        }
        const int i = int(sval[lo + j]);
        const Aabb<T> b = d.tbox[i];
        const T lower = ax == 0 ? b.mn.x : (ax == 1 ? b.mn.y : b.mn.z);
        srt[j] = (uint64_t(f2ord(down_f(lower))) << 32) | uint32_t(j);
        my_created = max(my_created, int(d.meta[i].created));
        if ((skey[lo + j] >> 30) & 1u)
            atomicMin(&ndyn, j);
        else
            my_reinserted = min(my_reinserted, int(d.meta[i].reinserted));
    }
    my_created = __reduce_max_sync(0xFFFFFFFFu, my_created);
    my_reinserted = __reduce_min_sync(0xFFFFFFFFu, my_reinserted);
    if (lane == 0)
    {
        atomicMax(&newest_created, my_created);
        atomicMin(&oldest_reinserted, my_reinserted);
    }
    __syncthreads();
    {
        // bitonic sort: stages with strides below SE on the registers of the warp holding the
        // chunk, larger strides through shared memory
        const int cb = warp * SE;
        const bool holds = cb < P;
        uint64_t v[E];
        if (holds)
        {
#pragma unroll
            for (int k = 0; k < E; ++k) v[k] = srt[cb + 32 * k + lane];
            for (int size = 2; size <= SE; size <<= 1) bitonic_warp_stages<E>(v, cb, lane, size);
#pragma unroll
            for (int k = 0; k < E; ++k) srt[cb + 32 * k + lane] = v[k];
        }
        __syncthreads();
        for (int size = 2 * SE; size <= P; size <<= 1)
        {
            for (int stride = size >> 1; stride >= SE; stride >>= 1)
            {
                for (int t = tid; t < (P >> 1); t += bs)
                {
                    const int i = 2 * t - (t & (stride - 1));
                    const int j = i + stride;
                    const uint64_t x = srt[i], y = srt[j];
                    if ((x > y) == ((i & size) == 0))
                    {
                        srt[i] = y;
                        srt[j] = x;
                    }
                }
                __syncthreads();
            }
            if (holds)
            {
#pragma unroll
                for (int k = 0; k < E; ++k) v[k] = srt[cb + 32 * k + lane];
                bitonic_warp_stages<E>(v, cb, lane, size);
#pragma unroll
                for (int k = 0; k < E; ++k) srt[cb + 32 * k + lane] = v[k];
            }
            __syncthreads();
        }
    }
    const int nd = ndyn;
    float my_max = 0.f;
    for (int r = tid; r < n; r += bs)
    {
        const uint64_t e = srt[r];
        const int j = int(uint32_t(e));
        const Aabb<T> b = d.tbox[int(sval[lo + j])];
        float *o = box + 6 * r;
        // FP64 form: rounded outward, so the FP32 test below never misses an overlap; the pairs
        // it finds are confirmed on the exact boxes
        o[0] = down_f(b.mn.x);
        o[1] = down_f(b.mn.y);
        o[2] = down_f(b.mn.z);
        o[3] = up_f(b.mx.x);
        o[4] = up_f(b.mx.y);
        o[5] = up_f(b.mx.z);
        lowax[r] = ord2f(uint32_t(e >> 32));
        leaf[r] = uint16_t(j | (j >= nd ? 0x8000 : 0));
        if constexpr (sizeof(T) == 8)
            my_max = fmaxf(my_max, fmaxf(fmaxf(fmaxf(fabsf(o[0]), fabsf(o[1])), fmaxf(fabsf(o[2]), fabsf(o[3]))),
                                         fmaxf(fabsf(o[4]), fabsf(o[5]))));
    }
    if constexpr (sizeof(T) == 8)
    {
        const unsigned mb = __reduce_max_sync(0xFFFFFFFFu, __float_as_uint(my_max)); // >= 0: orders as bits
        if (lane == 0) atomicMax(&coord_max, mb);
    }
    __syncthreads(); // the sort keys are dead from here on; their space holds the queue
    // The box test of sorted positions a < b: closed intervals on the exact fat boxes, static-static
    // pairs skipped. Written without short-circuits, so that the loads of a test issue together.
    // The FP32 boxes are rounded outward in the FP64 form. Two FP32 roundings move an overlap by
    // less than 2 eps M, M the largest coordinate magnitude of the world, so where the FP32 boxes
    // overlap by more than slack = 4 eps M on every axis (tested on a's box shrunk by the slack,
    // rounded inward: qs) the exact boxes overlap as well; only the other hits are confirmed by the
    // inclusive compares of the exact fat boxes.
    const float slack = 4.0f * EpsOf<float>::v * __uint_as_float(coord_max) + 1e-30f;
    auto shrink = [&](const float *qa, float *qs) {
        for (int k = 0; k < 3; ++k)
        {
            qs[k] = __fadd_ru(qa[k], slack);
            qs[k + 3] = __fsub_rd(qa[k + 3], slack);
        }
    };
    auto overlaps = [&](int ra, const float *qa, const float *qs, bool a_static, int rb) {
        const float *qb = box + 6 * rb;
        const float b0 = qb[0], b1 = qb[1], b2 = qb[2], b3 = qb[3], b4 = qb[4], b5 = qb[5];
        bool hit = !(a_static & ((leaf[rb] & 0x8000) != 0)) & (b0 <= qa[3]) & (b3 >= qa[0]) & (b1 <= qa[4]) &
                   (b4 >= qa[1]) & (b2 <= qa[5]) & (b5 >= qa[2]);
        if constexpr (sizeof(T) == 8)
        {
            const bool sure = (b0 < qs[3]) & (b3 > qs[0]) & (b1 < qs[4]) & (b4 > qs[1]) & (b2 < qs[5]) & (b5 > qs[2]);
            if (hit & !sure)
            {
                const Aabb<T> ba = d.tbox[int(sval[lo + (leaf[ra] & 0xFFF)])];
                const Aabb<T> bb = d.tbox[int(sval[lo + (leaf[rb] & 0xFFF)])];
                hit = bb.mn.x <= ba.mx.x && bb.mx.x >= ba.mn.x && bb.mn.y <= ba.mx.y && bb.mx.y >= ba.mn.y &&
                      bb.mn.z <= ba.mx.z && bb.mx.z >= ba.mn.z;
            }
        }
        return hit;
    };
    // the end of a window: the first sorted position after ra whose lower bound passes upa
    auto window_end = [&](int ra, float upa) {
        int a = ra + 1, b = n;
        while (a < b)
        {
            const int m = (a + b) >> 1;
            if (lowax[m] > upa)
                b = m;
            else
                a = m + 1;
        }
        return a;
    };
    int own = 0; // pairs this thread queued (those past SLICE went to the overflow region)
    for (int pass = 0; pass < 2; ++pass)
    {
        // pass 0 queues; pass 1 only runs after a queue overflow and emits straight to the list
        if (pass == 1 && ofill <= OCAP) break;
        if (tid == 0) nlong = 0;
        __syncthreads();
        auto push = [&](bool hit, int ra, int rb) {
            if (!hit) return;
            if (pass == 1)
            {
                broad_emit(d, w, lo, sval, int(leaf[ra] & 0xFFF), int(leaf[rb] & 0xFFF), -1);
                return;
            }
            const uint32_t e = uint32_t(ra) | (uint32_t(rb) << 12);
            if (own < SLICE)
                queue[own * THREADS + tid] = e;
            else
            {
                const int o = atomicAdd(&ofill, 1);
                if (o < OCAP) queue[SLICE * THREADS + o] = e;
            }
            ++own;
        };
        // a warp tests sorted position ra against positions [from, to), 64 a turn, taking every
        // `step`-th block of 64
        auto sweep_warp = [&](int ra, int from, int to, int step) {
            float qa[6], qs[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) qa[k] = box[6 * ra + k];
            if constexpr (sizeof(T) == 8) shrink(qa, qs);
            const bool a_static = (leaf[ra] & 0x8000) != 0;
            for (int base = from; base < to; base += 64 * step)
            {
                const int s0 = base + lane, s1 = base + 32 + lane;
                const bool h0 = (s0 < to) & overlaps(ra, qa, qs, a_static, min(s0, n - 1));
                const bool h1 = (s1 < to) & overlaps(ra, qa, qs, a_static, min(s1, n - 1));
                push(h0, ra, s0);
                push(h1, ra, s1);
            }
        };
        // A warp takes 32 consecutive sorted positions, one per lane; each lane finds the end of
        // its window and tests up to kBroadLaneSpan candidates of it, four a turn (neighbouring
        // positions have windows of similar length). The rest of longer windows, such as those of
        // static walls that span the world, is listed and shared out to all warps afterwards.
        for (int g = warp * 32; g < n - 1; g += nw * 32)
        {
            const int r = g + lane;
            const bool has = r < n - 1;
            float qa[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, qs[6];
            bool a_static = false;
            int end = r + 1;
            if (has)
            {
#pragma unroll
                for (int k = 0; k < 6; ++k) qa[k] = box[6 * r + k];
                a_static = (leaf[r] & 0x8000) != 0;
                end = window_end(r, ax == 0 ? qa[3] : (ax == 1 ? qa[4] : qa[5]));
            }
            if constexpr (sizeof(T) == 8) shrink(qa, qs);
            const int lane_end = min(end, r + 1 + kBroadLaneSpan);
            for (int k = r + 1; __any_sync(0xFFFFFFFFu, k < lane_end); k += 4)
            {
                bool h[4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    h[u] = (k + u < lane_end) & overlaps(r, qa, qs, a_static, min(k + u, n - 1));
#pragma unroll
                for (int u = 0; u < 4; ++u) push(h[u], r, k + u);
            }
            const bool longer = end > lane_end;
            const unsigned rest = __ballot_sync(0xFFFFFFFFu, longer);
            if (rest)
            {
                int at = 0;
                if (lane == 0) at = atomicAdd(&nlong, __popc(rest));
                at = __shfl_sync(0xFFFFFFFFu, at, 0) + __popc(rest & ((1u << lane) - 1u));
                if (longer && at < kBroadLong)
                {
                    long_at[at] = r;
                    long_from[at] = lane_end;
                    long_to[at] = end;
                }
                // a full list: this warp tests its own
                unsigned own = __ballot_sync(0xFFFFFFFFu, longer && at >= kBroadLong);
                while (own)
                {
                    const int l = __ffs(own) - 1;
                    own &= own - 1;
                    sweep_warp(g + l, __shfl_sync(0xFFFFFFFFu, lane_end, l), __shfl_sync(0xFFFFFFFFu, end, l), 1);
                }
            }
        }
        __syncthreads();
        for (int k = 0, nl = min(nlong, kBroadLong); k < nl; ++k)
            sweep_warp(long_at[k], long_from[k] + 64 * warp, long_to[k], nw);
        __syncthreads();
    }
    if (ofill > OCAP) return; // emitted by the second sweep
    const int mine_own = min(own, SLICE), novf = ofill;
    // Per sorted position its device slot and world-local index, in the space of the boxes (no
    // longer read): the pair checks and writes below then read shared memory only.
    uint32_t *pslot = reinterpret_cast<uint32_t *>(box), *ploc = pslot + n;
    for (int r = tid; r < n; r += bs)
    {
        const int i = int(sval[lo + (leaf[r] & 0xFFF)]);
        pslot[r] = uint32_t(i);
        ploc[r] = d.meta[i].local;
    }
    __syncthreads();
    // drop the pairs the reference does not pair yet, then one reservation for the rest. Every
    // pair has a dynamic end, so where each dynamic body was reinserted at or after the newest
    // creation in the world, every pair is allowed and the check is skipped.
    const bool young = oldest_reinserted < newest_created;
    // a thread's entries: its slice, then every bs-th entry of the overflow region
    auto entry_at = [&](int k) {
        return k < mine_own ? k * THREADS + tid : SLICE * THREADS + tid + (k - mine_own) * THREADS;
    };
    const int nmine = mine_own + (novf > tid ? (novf - tid + THREADS - 1) / THREADS : 0);
    int mine = 0;
    for (int k = 0; k < nmine; ++k)
    {
        const int q = entry_at(k);
        const uint32_t e = queue[q];
        if (!young || pair_allowed<T>(d.meta[pslot[e & 0xFFFu]], d.meta[pslot[(e >> 12) & 0xFFFu]]))
            ++mine;
        else
            queue[q] = e | 0x80000000u;
    }
    int before = mine;
    for (int o = 1; o < 32; o <<= 1)
    {
        const int y = __shfl_up_sync(0xFFFFFFFFu, before, o);
        if (lane >= o) before += y;
    }
    if (lane == 31) warp_count[warp] = before;
    __syncthreads();
    if (tid == 0)
    {
        int t = 0;
        for (int k = 0; k < nw; ++k)
        {
            const int c = warp_count[k];
            warp_count[k] = t;
            t += c;
        }
        cta_base = t ? atomicAdd(d.npairs, t) : 0;
    }
    __syncthreads();
    int slot = cta_base + warp_count[warp] + before - mine;
    const uint64_t wkey = uint64_t(w) << (2 * d.lbits);
    for (int k = 0; k < nmine; ++k)
    {
        const uint32_t e = queue[entry_at(k)];
        if (e & 0x80000000u) continue;
        const int ra = int(e & 0xFFFu), rb = int((e >> 12) & 0xFFFu);
        const uint32_t la = ploc[ra], lb = ploc[rb];
        const bool a_first = la < lb;
        if (slot < d.pair_cap)
        {
            d.pkey[slot] = wkey | (uint64_t(a_first ? la : lb) << d.lbits) | uint64_t(a_first ? lb : la);
            d.pval[slot] = (uint64_t(a_first ? pslot[ra] : pslot[rb]) << 32) | (a_first ? pslot[rb] : pslot[ra]);
        }
        else
            atomicOr(d.status, ST_PAIR_OVERFLOW);
        ++slot;
    }
}

// ------------------------------------------------------------------------------------------------
// world raycast (world.h:260-319): every body whose broadphase box the ray enters within the
// distance limit, with the entry distance, on the LBVH of the ray's world
// ------------------------------------------------------------------------------------------------
template <class T> __global__ void k_tree_reset(Dev<T> d)
{
    PK_GRID_STRIDE(w, d.max_worlds)
    {
        d.wroot[w] = -1;
        d.wleaf_lo[w] = 0;
        d.wleaf_hi[w] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d.nleaf = 0;
}

// ray::intersect_distance (bvh.h:62-93): slab test with 1/x (+-inf at zero) and the reference's
// NaN limits, in the engine's precision.
template <class T>
__device__ __forceinline__ bool ray_box(V3<T> o, V3<T> inv, T maxd, V3<T> mn, V3<T> mx, T &out)
{
    const T inf = std::numeric_limits<T>::infinity();
    auto slab = [&](T lo, T hi, T &a, T &c) {
        if (lo != lo) lo = -inf;
        if (hi != hi) hi = inf;
        a = fmin(lo, hi);
        c = fmax(lo, hi);
    };
    T tminx, tmaxx, tminy, tmaxy, tminz, tmaxz;
    slab((mn.x - o.x) * inv.x, (mx.x - o.x) * inv.x, tminx, tmaxx);
    slab((mn.y - o.y) * inv.y, (mx.y - o.y) * inv.y, tminy, tmaxy);
    slab((mn.z - o.z) * inv.z, (mx.z - o.z) * inv.z, tminz, tmaxz);
    const T t0 = tmax(tmax(tminx, tminy), tminz); // std::max / std::min over the three axes
    const T t1 = tmin(tmin(tmaxx, tmaxy), tmaxz);
    if (t1 >= T(0) && t0 <= t1 && t0 <= maxd)
    {
        out = tmax(T(0), t0);
        return true;
    }
    return false;
}

// One thread per ray (8 doubles: origin, direction, distance limit, world). Keeps the `cap`
// nearest hits ordered by (distance, slot) and counts all of them.
template <class T>
__global__ void k_raycast(Dev<T> d, const uint64_t *__restrict__ sval, const double *__restrict__ rays, int n, int cap,
                          int *__restrict__ counts, int *__restrict__ hit_slot, T *__restrict__ hit_t)
{
    PK_GRID_STRIDE(r, n)
    {
        const double *ry = rays + 8 * size_t(r);
        const V3<T> o{T(ry[0]), T(ry[1]), T(ry[2])};
        const V3<T> dir = normalized(V3<T>{T(ry[3]), T(ry[4]), T(ry[5])});
        const V3<T> inv{T(1) / dir.x, T(1) / dir.y, T(1) / dir.z};
        const T maxd = T(ry[6]);
        const int world = int(ry[7]);
        int *os = hit_slot + size_t(r) * cap;
        T *ot = hit_t + size_t(r) * cap;
        int cnt = 0;
        auto emit = [&](int slot, T t) {
            int k = cnt < cap ? cnt : cap;
            ++cnt;
            if (k == cap && !(t < ot[cap - 1] || (t == ot[cap - 1] && slot < os[cap - 1]))) return;
            int pos = k == cap ? cap - 1 : k;
            while (pos > 0 && (t < ot[pos - 1] || (t == ot[pos - 1] && slot < os[pos - 1])))
            {
                os[pos] = os[pos - 1];
                ot[pos] = ot[pos - 1];
                --pos;
            }
            os[pos] = slot;
            ot[pos] = t;
        };
        auto leaf_test = [&](int pos) {
            const int slot = int(sval[pos]);
            const Aabb<T> b = d.tbox[slot];
            T t;
            if (ray_box(o, inv, maxd, b.mn, b.mx, t)) emit(slot, t);
        };
        const int root = (world >= 0 && world < d.max_worlds) ? d.wroot[world] : -1;
        if (root >= 0 && (uint32_t(root) & kLeafBit))
            leaf_test(int(uint32_t(root) & ~kLeafBit));
        else if (root >= 0)
        {
            int stack[96];
            int sp = 0;
            stack[sp++] = root;
            while (sp > 0)
            {
                const float4 *nd = d.nodes + 4 * stack[--sp];
#pragma unroll
                for (int c = 0; c < 2; ++c)
                {
                    const float4 bmn = nd[2 * c], bmx = nd[2 * c + 1];
                    T t;
                    // node boxes enclose their leaves' boxes, and the slab test only widens with the box
                    if (!ray_box(o, inv, maxd, V3<T>{T(bmn.x), T(bmn.y), T(bmn.z)}, V3<T>{T(bmx.x), T(bmx.y), T(bmx.z)}, t))
                        continue;
                    const uint32_t ch = __float_as_uint(bmn.w);
                    if (ch & kLeafBit)
                        leaf_test(int(ch & ~kLeafBit));
                    else if (sp < 96)
                        stack[sp++] = int(ch);
                    else
                        atomicOr(d.status, ST_TRAVERSAL_STACK);
                }
            }
        }
        counts[r] = cnt;
    }
}

template <class T> __global__ void k_clamp_pairs(Dev<T> d)
{
    if (*d.npairs > d.pair_cap) *d.npairs = d.pair_cap;
    *d.nnew = *d.npairs;
}

// ------------------------------------------------------------------------------------------------
// narrowphase + manifold update (collision_phases.h:244-320)
// ------------------------------------------------------------------------------------------------
template <class T> __device__ __forceinline__ ShapeRef<T> body_shape(const Dev<T> &d, int slot)
{
    ShapeRef<T> s;
    const Meta m = d.meta[slot];
    const ShapeRange r = d.shape_range[m.shape];
    s.kind = SHAPE_MESH;
    s.nverts = r.nverts;
    s.verts = d.verts + 3 * r.vstart;
    s.ncl = r.ncl;
    s.cl = d.clusters + 4 * r.cstart;
    s.ngr = r.ngr;
    s.gr = d.clusters + 4 * r.gstart;
    s.rmax = d.shape_rmax[m.shape];
    s.uv_stacks = r.uv_stacks;
    s.uv_sectors = r.uv_sectors;
    const Pose<T> &p = d.pose[slot];
    s.pos = ld3(p.p);
    s.q = ldq(p.q);
    return s;
}

template <class T> __device__ __forceinline__ void add_contact(Manifold<T> &m, const Contact<T> &c)
{
    if (m.n < 4)
    {
        m.c[m.n++] = c;
        return;
    }
    // manifold::add_reduce (collision_phases.h:139-198)
    Contact<T> pool[5] = {m.c[0], m.c[1], m.c[2], m.c[3], c};
    int best[4] = {0, 1, 2, 3};
    for (int i = 1; i < 5; ++i)
        if (pool[i].depth > pool[best[0]].depth) best[0] = i;
    T md = T(-1);
    for (int i = 0; i < 5; ++i)
    {
        if (i == best[0]) continue;
        T d2 = sqnorm(ld3(pool[i].la) - ld3(pool[best[0]].la));
        if (d2 > md)
        {
            md = d2;
            best[1] = i;
        }
    }
    T ma = T(-1);
    V3<T> e0 = ld3(pool[best[1]].la) - ld3(pool[best[0]].la);
    for (int i = 0; i < 5; ++i)
    {
        if (i == best[0] || i == best[1]) continue;
        V3<T> e1 = ld3(pool[i].la) - ld3(pool[best[0]].la);
        T a2 = sqnorm(cross(e0, e1));
        if (a2 > ma)
        {
            ma = a2;
            best[2] = i;
        }
    }
    md = T(-1);
    for (int i = 0; i < 5; ++i)
    {
        if (i == best[0] || i == best[1] || i == best[2]) continue;
        T d2 = sqnorm(ld3(pool[i].la) - ld3(pool[best[2]].la));
        if (d2 > md)
        {
            md = d2;
            best[3] = i;
        }
    }
    for (int k = 0; k < 4; ++k) m.c[k] = pool[best[k]];
    m.n = 4;
}


// The manifold update of narrow_phase::calculate for one pair given its new contact (if any):
// warm-start transfer, re-projection of old contacts, reduction to four and begin/end events
// (collision_phases.h:261-318).
template <class T>
__device__ void manifold_update(const Dev<T> &d, int p, int old_idx, const ShapeRef<T> &A, const ShapeRef<T> &B,
                                bool hit, const Collision<T> &col, V3<T> sep = V3<T>{T(0), T(0), T(0)})
{
    const T d2eps = T(0.005 * 0.005), breaking = T(0.05), drift2_eps = T(0.06);
    // only the contacts in use are read and written: most pairs have an empty manifold
    Manifold<T> old;
    old.n = 0;
    if (old_idx >= 0)
    {
        const Manifold<T> *src = d.man_old + old_idx;
        old.n = src->n;
        for (int k = 0; k < old.n; ++k) old.c[k] = src->c[k];
    }
    Contact<T> nc;
    if (hit)
    {
        st3(nc.n, col.normal);
        st3(nc.la, rotate(conj(A.q), col.world_a - A.pos));
        st3(nc.lb, rotate(conj(B.q), col.world_b - B.pos));
        nc.depth = col.depth;
        nc.imp[0] = nc.imp[1] = nc.imp[2] = 0.0;
    }
    Manifold<T> nm;
    nm.n = 0;
    nm.pad = 0;
    for (int k = 0; k < old.n; ++k)
    {
        Contact<T> oc = old.c[k];
        if (hit)
        {
            if (sqnorm(ld3(nc.la) - ld3(oc.la)) < d2eps || sqnorm(ld3(nc.lb) - ld3(oc.lb)) < d2eps)
            {
                nc.imp[0] = oc.imp[0];
                nc.imp[1] = oc.imp[1];
                nc.imp[2] = oc.imp[2];
                continue;
            }
        }
        V3<T> wa = rotate(A.q, ld3(oc.la)) + A.pos;
        V3<T> wb = rotate(B.q, ld3(oc.lb)) + B.pos;
        V3<T> normal = hit ? ld3(nc.n) : ld3(oc.n);
        V3<T> rel = wb - wa;
        T depth = dot(rel, normal);
        V3<T> pa = wa + normal * depth;
        T drift2 = sqnorm(pa - wb);
        if (depth > -breaking && drift2 < drift2_eps)
        {
            oc.depth = depth;
            st3(oc.n, normal);
            add_contact(nm, oc);
        }
    }
    if constexpr (sizeof(T) == 4)
    {
        // FP32 form: a contact that did not come out finite is not kept (the FP64 form follows the
        // reference exactly, whatever it computes)
        if (hit && !(isfinite(nc.depth) && isfinite(nc.n[0] + nc.n[1] + nc.n[2]) && isfinite(nc.la[0] + nc.la[1] + nc.la[2]) &&
                     isfinite(nc.lb[0] + nc.lb[1] + nc.lb[2])))
            hit = false;
    }
    if (hit) add_contact(nm, nc);
    bool was = old.n != 0, is = nm.n != 0;
    d.event[p] = (!was && is) ? 1 : ((was && !is) ? 2 : 0);
    Manifold<T> *dst = d.man_new + p;
    dst->n = nm.n;
    dst->pad = 0;
    st3(dst->sep, sep);
    for (int k = 0; k < nm.n; ++k) dst->c[k] = nm.c[k];
    if (nm.n > 0) d.clist[warp_push(d.ccount)] = p; // contact rows are built for these pairs only
}

// Separating-axis test of the two bodies' oriented local AABBs (15 axes). True only when some axis
// separates them by more than `margin`: then the shapes inside are disjoint too.
template <class T>
__device__ __forceinline__ bool obb_separated(const Aabb<T> &la, Qt<T> qa, V3<T> pa, const Aabb<T> &lb, Qt<T> qb,
                                              V3<T> pb, T margin)
{
    M3<T> Ra = to_matrix(qa), Rb = to_matrix(qb);
    V3<T> ha = (la.mx - la.mn) * T(0.5), hb = (lb.mx - lb.mn) * T(0.5);
    V3<T> ca = pa + matvec(Ra.m, (la.mx + la.mn) * T(0.5));
    V3<T> cb = pb + matvec(Rb.m, (lb.mx + lb.mn) * T(0.5));
    V3<T> t = cb - ca;
    // axes of A and B are the columns of Ra, Rb
    T a[3] = {ha.x, ha.y, ha.z}, b[3] = {hb.x, hb.y, hb.z};
    T C[3][3], AC[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
        {
            C[i][j] = Ra.m[i] * Rb.m[j] + Ra.m[3 + i] * Rb.m[3 + j] + Ra.m[6 + i] * Rb.m[6 + j];
            AC[i][j] = tabs(C[i][j]) + T(1e-6);
        }
    T ta[3];
    for (int i = 0; i < 3; ++i) ta[i] = Ra.m[i] * t.x + Ra.m[3 + i] * t.y + Ra.m[6 + i] * t.z;
    for (int i = 0; i < 3; ++i)
        if (tabs(ta[i]) > a[i] + b[0] * AC[i][0] + b[1] * AC[i][1] + b[2] * AC[i][2] + margin) return true;
    for (int j = 0; j < 3; ++j)
    {
        T tb = ta[0] * C[0][j] + ta[1] * C[1][j] + ta[2] * C[2][j];
        if (tabs(tb) > b[j] + a[0] * AC[0][j] + a[1] * AC[1][j] + a[2] * AC[2][j] + margin) return true;
    }
    for (int i = 0; i < 3; ++i)
    {
        int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        for (int j = 0; j < 3; ++j)
        {
            int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            T tt = tabs(ta[i2] * C[i1][j] - ta[i1] * C[i2][j]);
            T ra = a[i1] * AC[i2][j] + a[i2] * AC[i1][j];
            T rb = b[j1] * AC[i][j2] + b[j2] * AC[i][j1];
            if (tt > ra + rb + margin) return true;
        }
    }
    return false;
}

// FP64 form: a body's shape in FP32 (pose rounded, the FP32 copies of its vertices) for tests that
// only decide that two shapes are certainly apart. Shapes with clustered vertex blocks (large
// non-UV meshes) have no FP32 form here: ok is false.
__device__ __forceinline__ ShapeRef<float> body_shape32(const Dev<double> &d, int slot, bool &ok)
{
    ShapeRef<float> s;
    const Meta m = d.meta[slot];
    const ShapeRange r = d.shape_range[m.shape];
    ok = r.ncl == 0 && d.verts32 != nullptr;
    s.kind = SHAPE_MESH;
    s.nverts = r.nverts;
    s.verts = ok ? d.verts32 + 3 * r.vstart : nullptr;
    s.ncl = 0;
    s.cl = nullptr;
    s.ngr = 0;
    s.gr = nullptr;
    s.rmax = d.shape32[8 * m.shape + 6];
    s.uv_stacks = r.uv_stacks;
    s.uv_sectors = r.uv_sectors;
    const float4 p = d.pose32[2 * slot], q = d.pose32[2 * slot + 1];
    s.pos = V3<float>{p.x, p.y, p.z};
    s.q = Qt<float>{q.x, q.y, q.z, q.w};
    return s;
}

// FP64 form: the pre-pass tests (bounding spheres, then the 15-axis test of the oriented local
// boxes) in FP32. They only decide that a pair is certainly apart (GJK then returns no collision,
// collision.cpp:181-182), so no FP64 result is needed: the margin, 1024 FP32 epsilons of the
// pair's scale plus the FP64 test's own terms, covers the rounding of the FP32 poses, boxes and
// products many times over. A pair it cannot settle goes on to the separating-axis pass and GJK.
// Support kind of a shape, as ShapeRef::support dispatches: 0 the box search (FP64 form), 1 a
// linear scan, 2 the UV-sphere neighbourhood, 3 vertex clusters.
template <class T> __device__ __forceinline__ int support_kind(const Dev<T> &d, int slot)
{
    const ShapeRange r = d.shape_range[d.meta[slot].shape];
    if (sizeof(T) == 8 && r.uv_stacks == kBoxLayout) return 0;
    if (r.uv_stacks > 0) return 2;
    return r.ncl > 0 ? 3 : 1;
}
// A pair's GJK work class: warps given one class run one support path per shape. Classes with a
// UV sphere or a clustered mesh (the costly supports) come first in the class order.
template <class T> __device__ __forceinline__ int pair_class(const Dev<T> &d, int sa, int sb)
{ return 4 * support_kind(d, sa) + support_kind(d, sb); }
__device__ __forceinline__ int class_rank(int c) { return ((c >> 2) >= 2 || (c & 3) >= 2) ? c : kPairClasses + c; }

// The FP32 copies of poses (written each step by k_integrate_vel) and of shape boxes and radii
// (written with the shapes) spare the per-pair conversions, which GB300 issues on the FP64 pipe.
__device__ __forceinline__ bool apart_f32(const Dev<double> &d, int sa, int sb)
{
    const float *fa = d.shape32 + 8 * d.meta[sa].shape, *fb = d.shape32 + 8 * d.meta[sb].shape;
    const float4 pa = d.pose32[2 * sa], pb = d.pose32[2 * sb];
    const V3<float> xa{pa.x, pa.y, pa.z}, xb{pb.x, pb.y, pb.z};
    const float rs = fa[6] + fb[6];
    const float margin = (rs + norm(xa) + norm(xb)) * (1024.0f * EpsOf<float>::v) + 1e-6f + 1e-5f * rs;
    const float cull = rs + margin;
    if (sqnorm(xb - xa) > cull * cull) return true;
    const float4 ra = d.pose32[2 * sa + 1], rb = d.pose32[2 * sb + 1];
    const Qt<float> qa{ra.x, ra.y, ra.z, ra.w}, qb{rb.x, rb.y, rb.z, rb.w};
    const Aabb<float> ba{{fa[0], fa[1], fa[2]}, {fa[3], fa[4], fa[5]}};
    const Aabb<float> bb{{fb[0], fb[1], fb[2]}, {fb[3], fb[4], fb[5]}};
    return obb_separated(ba, qa, xa, bb, qb, xb, margin);
}

// Last step's manifold of each pair of an active world. Last step's pairs of a world are the
// segment [mstart_old, mend_old) of last step's sorted keys, and this step's pairs are sorted the
// same way, so each thread takes a run of consecutive pairs: one binary search for the first,
// then a forward walk (with a binary search again past a long gap) for the rest. Pairs of idle
// worlds keep the index their assembly gave them.
constexpr int kOldRun = 8;
template <class T> __global__ void k_old_index(Dev<T> d, const uint64_t *__restrict__ skey)
{
    const int np = *d.npairs;
    PK_GRID_STRIDE(t, (np + kOldRun - 1) / kOldRun)
    {
        const int p0 = t * kOldRun, p1 = min(np, p0 + kOldRun);
        int cw = -1, lo = 0, end = -1;
        for (int p = p0; p < p1; ++p)
        {
            const uint64_t key = skey[p];
            const int w = int(key >> (2 * d.lbits));
            if (w != cw)
            {
                cw = w;
                end = d.wp[w].active ? d.mend_old[w] : -1;
                lo = d.mstart_old[w];
            }
            if (end < 0) continue;
            int step = 0;
            while (lo < end && d.key_old[lo] < key && step < 4)
            {
                ++lo;
                ++step;
            }
            if (lo < end && d.key_old[lo] < key)
            {
                int hi = end;
                while (lo < hi)
                {
                    const int mid = (lo + hi) >> 1;
                    if (d.key_old[mid] < key) lo = mid + 1; else hi = mid;
                }
            }
            d.old_idx[p] = (lo < end && d.key_old[lo] == key) ? lo : -1;
        }
    }
}

// Narrowphase pass 1: per pair, take last step's manifold, then either settle the pair at once or
// queue it for GJK. A pair is settled without a new contact when the bodies' bounding spheres or
// their oriented local boxes are apart by more than a rounding margin: the shapes are then
// disjoint, and the reference's GJK returns no collision for them (collision.cpp:181-182).
template <class T>
__global__ void __launch_bounds__(256, 3) k_narrow_pre(Dev<T> d, const uint64_t *__restrict__ skey, const uint64_t *__restrict__ sval)
{
    const int np = *d.npairs;
    PK_GRID_STRIDE(p, np)
    {
        uint64_t key = skey[p];
        uint64_t val = sval[p];
        int sa = int(val >> 32), sb = int(val & 0xFFFFFFFFu);
        int world = int(key >> (2 * d.lbits));
        d.rowmask[p] = 0; // no contact rows unless the contact setup builds some
        if (!d.wp[world].active)
        {
            // kept pair of a world that sits out this step: unchanged, no event
            const Manifold<T> &src = d.man_old[d.old_idx[p]];
            Manifold<T> &dst = d.man_new[p];
            dst.n = src.n;
            dst.pad = 0;
            for (int k = 0; k < 3; ++k) dst.sep[k] = src.sep[k];
            for (int k = 0; k < src.n; ++k) dst.c[k] = src.c[k];
            d.event[p] = 0;
            continue;
        }
        const int old_idx = d.old_idx[p]; // k_old_index
        bool apart = false;
        if constexpr (sizeof(T) == 8)
        {
            apart = apart_f32(d, sa, sb);
            if (apart)
            {
                // the FP64 shapes are needed only to carry last step's contacts forward
                const bool had = old_idx >= 0 && d.man_old[old_idx].n > 0;
                const ShapeRef<T> A = had ? body_shape(d, sa) : ShapeRef<T>{};
                const ShapeRef<T> B = had ? body_shape(d, sb) : ShapeRef<T>{};
                Collision<T> none;
                manifold_update(d, p, old_idx, A, B, false, none);
            }
        }
        else
        {
            ShapeRef<T> A = body_shape(d, sa), B = body_shape(d, sb);
            V3<T> dc = B.pos - A.pos;
            T rs = A.rmax + B.rmax;
            T cull = rs + (rs + norm(A.pos) + norm(B.pos)) * T(1024) * EpsOf<T>::v + T(1e-6);
            const T margin = (rs + norm(A.pos) + norm(B.pos)) * T(1024) * EpsOf<T>::v + T(1e-6);
            apart = sqnorm(dc) > cull * cull ||
                    obb_separated(d.shape_box[d.meta[sa].shape], A.q, A.pos, d.shape_box[d.meta[sb].shape], B.q,
                                  B.pos, margin + T(1e-5) * rs);
            if (apart)
            {
                Collision<T> none;
                manifold_update(d, p, old_idx, A, B, false, none);
            }
        }
        if (!apart)
        {
            // pairs with a large mesh (vertex clusters) fill the list from its far end
            if (d.shape_range[d.meta[sa].shape].ncl > 0 || d.shape_range[d.meta[sb].shape].ncl > 0)
                d.gjk_list[d.pair_cap - 1 - warp_push(d.gjk_count_heavy)] = p;
            else
                d.gjk_list[warp_push(d.gjk_count)] = p;
        }
    }
}

// Work item i of a two-class list: heavy items (stored from the end) first, then light ones.
__device__ __forceinline__ int list_slot(int i, int nheavy, int cap)
{ return i < nheavy ? cap - 1 - i : i - nheavy; }

// Narrowphase pass 2: GJK (collision.cpp:165-189) over the queued pairs; enclosing simplices are
// queued for EPA, the rest are settled without a new contact.
#ifndef PK_GJK_MIN_BLOCKS
#define PK_GJK_MIN_BLOCKS 5
#endif
// EPA waits on its per-thread polytope: the FP32 form runs faster with more resident warps (64
// registers: EPA 2.03 -> 1.92 ms on the bench batch), the FP64 form with fewer spills (128)
#ifndef PK_EPA_MIN_BLOCKS
#define PK_EPA_MIN_BLOCKS 4
#endif
#ifndef PK_EPA_MIN_BLOCKS_F32
#define PK_EPA_MIN_BLOCKS_F32 8
#endif

// Narrowphase pass 2a: last step's separating direction. If A - B still lies short of the origin
// along it by more than a rounding margin, the shapes are disjoint and GJK returns no collision
// (collision.cpp:181-182), so the pair is settled with one support query per shape; the others go
// on to GJK. A separate pass keeps the GJK warps on pairs that all run the full iteration.
template <class T>
__global__ void __launch_bounds__(128) k_narrow_axis(Dev<T> d, const uint64_t *__restrict__ sval)
{
    const int nh = *d.gjk_count_heavy;
    const int n = nh + *d.gjk_count;
    PK_GRID_STRIDE(i, n)
    {
        const int p = d.gjk_list[list_slot(i, nh, d.pair_cap)];
        const int oi = d.old_idx[p];
        bool settled = false;
        if (oi >= 0)
        {
            const V3<T> ax = ld3(d.man_old[oi].sep);
            if (sqnorm(ax) > T(0))
            {
                const uint64_t val = sval[p];
                const int sa = int(val >> 32), sb = int(val & 0xFFFFFFFFu);
                const ShapeRef<T> A = body_shape(d, sa), B = body_shape(d, sb);
                warp_add(d.np_verts, scan_verts(A, B));
                bool overlaps = false; // A - B certainly reaches past the origin along ax
                if constexpr (sizeof(T) == 8)
                {
                    // FP32 first: support values within a few tens of FP32 ulps of the pair's
                    // scale, far inside a margin of 1024 FP32 epsilons of it. Above +256 ulps the
                    // FP64 value is positive too, so the FP64 test below cannot settle the pair.
                    bool oka, okb;
                    const ShapeRef<float> A32 = body_shape32(d, sa, oka), B32 = body_shape32(d, sb, okb);
                    if (oka && okb)
                    {
                        const float rs = A32.rmax + B32.rmax;
                        const float scale = rs + norm(A32.pos) + norm(B32.pos);
                        const float m32 = scale * (1024.0f * EpsOf<float>::v) + 1e-6f + 1e-5f * rs;
                        const V3<float> ax32{float(ax.x), float(ax.y), float(ax.z)};
                        const SupPt<float> sp = minkowski(A32, B32, ax32);
                        const float v32 = dot(sp.p, ax32);
                        if (v32 < -m32)
                        {
                            Collision<T> none;
                            manifold_update(d, p, oi, A, B, false, none, ax);
                            settled = true;
                        }
                        else
                            overlaps = v32 > scale * (256.0f * EpsOf<float>::v);
                    }
                }
                const T rs = A.rmax + B.rmax;
                const T margin = (rs + norm(A.pos) + norm(B.pos)) * T(1024) * EpsOf<T>::v + T(1e-6) + T(1e-5) * rs;
                const SupPt<T> sp = (settled || overlaps) ? SupPt<T>{} : minkowski(A, B, ax);
                if (!settled && !overlaps && dot(sp.p, ax) < -margin)
                {
                    Collision<T> none;
                    manifold_update(d, p, oi, A, B, false, none, ax);
                    settled = true;
                }
            }
        }
        if (!settled)
        {
            if (i < nh)
                d.gjk_list2[d.pair_cap - 1 - warp_push(d.gjk2_count_heavy)] = p;
            else
                d.gjk_list2[warp_push(d.gjk2_count)] = p;
            const uint64_t val = sval[p];
            warp_push_key(d.gcls, pair_class(d, int(val >> 32), int(val & 0xFFFFFFFFu)));
        }
    }
}

// GJK's list laid out by work class: class starts (one warp), then every item moved to its class's
// range of the separating-direction pass's first list (free by then). Order within a class does
// not matter: each pair's GJK is computed on its own.
template <class T> __global__ void k_gjk_class_start(Dev<T> d)
{
    if (threadIdx.x != 0) return;
    int *gcls = d.gcls;
    int order[kPairClasses];
    for (int c = 0; c < kPairClasses; ++c) order[c] = c;
    for (int a = 1; a < kPairClasses; ++a) // by rank: the few classes, an insertion sort
        for (int b = a; b > 0 && class_rank(order[b]) < class_rank(order[b - 1]); --b)
        {
            const int t = order[b];
            order[b] = order[b - 1];
            order[b - 1] = t;
        }
    int run = 0;
    for (int k = 0; k < kPairClasses; ++k)
    {
        const int c = order[k];
        gcls[kPairClasses + c] = run;
        gcls[2 * kPairClasses + c] = 0;
        run += gcls[c];
    }
}

template <class T> __global__ void k_gjk_class_scatter(Dev<T> d, const uint64_t *__restrict__ sval)
{
    const int nh = *d.gjk2_count_heavy;
    const int n = nh + *d.gjk2_count;
    PK_GRID_STRIDE(i, n)
    {
        const int p = d.gjk_list2[list_slot(i, nh, d.pair_cap)];
        const uint64_t val = sval[p];
        const int c = pair_class(d, int(val >> 32), int(val & 0xFFFFFFFFu));
        d.gjk_list[d.gcls[kPairClasses + c] + warp_push_key(d.gcls + 2 * kPairClasses, c)] = p;
    }
}

// Narrowphase pass 2b: GJK (collision.cpp:165-189) over the remaining pairs; enclosing simplices are
// queued for EPA, the rest are settled without a new contact and keep GJK's separating direction.
template <class T>
__global__ void __launch_bounds__(128, PK_GJK_MIN_BLOCKS) k_narrow_gjk(Dev<T> d, const uint64_t *__restrict__ sval)
{
    const int n = *d.gjk2_count_heavy + *d.gjk2_count;
    PK_GRID_STRIDE(i, n)
    {
        int p = d.gjk_list[i]; // in class order (k_gjk_class_scatter)
        uint64_t val = sval[p];
        int sa = int(val >> 32), sb = int(val & 0xFFFFFFFFu);
        ShapeRef<T> A = body_shape(d, sa), B = body_shape(d, sb);
        Simplex<T> s;
        V3<T> sep{T(0), T(0), T(0)};
        bool enclosed = gjk(A, B, s, &sep);
        warp_add(d.np_iters, unsigned(s.iters));
        warp_add(d.np_verts, unsigned(s.iters + 1) * scan_verts(A, B));
        // admitted first against the list's capacity, so the two ends never meet
        const bool admit = enclosed && warp_push(d.epa_total) < d.contact_cap;
        if (enclosed && !admit)
        {
            // no room for this pair's EPA: flagged, and the pair keeps last step's contacts
            atomicOr(d.status, ST_CONTACT_OVERFLOW);
            Collision<T> none;
            manifold_update(d, p, d.old_idx[p], A, B, false, none);
        }
        else if (admit)
        {
            int j;
            if (A.ncl > 0 || B.ncl > 0)
                j = d.contact_cap - 1 - warp_push(d.epa_count_heavy);
            else
                j = warp_push(d.epa_count);
            d.epa_list[j] = p;
            d.epa_simplex[j] = s;
        }
        else
        {
            Collision<T> none;
            manifold_update(d, p, d.old_idx[p], A, B, false, none, sep);
        }
    }
}

// Narrowphase pass 3: EPA (collision.cpp:411-504) over intersecting pairs, then the manifold update.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? PK_EPA_MIN_BLOCKS_F32 : PK_EPA_MIN_BLOCKS)
    k_narrow_epa(Dev<T> d, const uint64_t *__restrict__ sval)
{
    const int nh = *d.epa_count_heavy;
    const int n = nh + *d.epa_count;
    PK_GRID_STRIDE(i, n)
    {
        int j = list_slot(i, nh, d.contact_cap);
        int p = d.epa_list[j];
        uint64_t val = sval[p];
        int sa = int(val >> 32), sb = int(val & 0xFFFFFFFFu);
        ShapeRef<T> A = body_shape(d, sa), B = body_shape(d, sb);
        Simplex<T> s = d.epa_simplex[j];
        EpaState<T> es;
        Collision<T> col;
        bool hit = epa(A, B, s, es, col);
        if (es.status) atomicOr(d.status, ST_EPA_CAP);
        warp_add(d.np_iters + 1, unsigned(es.iters));
        if (A.ncl > 0 || B.ncl > 0) warp_add(d.np_iters + 2, unsigned(es.iters));
        warp_add(d.np_verts, unsigned(es.iters) * scan_verts(A, B));
        manifold_update(d, p, d.old_idx[p], A, B, hit, col);
    }
}

// ------------------------------------------------------------------------------------------------
// contact rows (build_contact_jacobian, constraint.h:874-953; setup_contacts :1052-1104)
// ------------------------------------------------------------------------------------------------
template <class T> __global__ void k_contact_setup(Dev<T> d, const uint64_t *__restrict__ skey,
                                                   const uint64_t *__restrict__ sval, T dt)
{
    // the pairs of active worlds with contacts, queued by the manifold update; every other pair
    // was given no rows (rowmask 0, colour -2) by the narrowphase pre-pass
    const int nc = *d.ccount;
    if (nc > d.contact_cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(d.status, ST_CONTACT_OVERFLOW);
    PK_GRID_STRIDE(ci, nc)
    {
        const int p = d.clist[ci];
        if (ci >= d.contact_cap) continue; // no room for rows: the pair is not solved (flagged)
        d.rowidx[p] = ci;
        const Manifold<T> &m = d.man_new[p];
        const int mn = m.n;
        uint64_t val = sval[p];
        int sa = int(val >> 32), sb = int(val & 0xFFFFFFFFu);
        int world = int(skey[p] >> (2 * d.lbits));
        const Pose<T> &PA = d.pose[sa];
        const Pose<T> &PB = d.pose[sb];
        const Params<T> &ra = d.prm[sa];
        const Params<T> &rb = d.prm[sb];
        const Vel<T> &VA = d.vel[sa];
        const Vel<T> &VB = d.vel[sb];
        const T *Ia = d.iwinv + 9 * sa;
        const T *Ib = d.iwinv + 9 * sb;
        Qt<T> qa = ldq(PA.q), qb = ldq(PB.q);
        V3<T> xa = ld3(PA.p), xb = ld3(PB.p);
        const T rthr = T(2) * d.wp[world].gnorm * dt;
        uint8_t mask = 0;
        for (int k = 0; k < mn; ++k)
        {
            const Contact<T> &c = m.c[k];
            V3<T> nn = normalized(ld3(c.n));
            V3<T> lnb = rotate(conj(qb), nn);
            V3<T> r_a = rotate(qa, ld3(c.la));
            V3<T> r_b = rotate(qb, ld3(c.lb));
            V3<T> n = rotate(qb, lnb);
            T pen = dot((xb + r_b) - (xa + r_a), n);
            if (pen <= T(0)) continue;
            Row<T> row;
            // normal row
            V3<T> wa = cross(r_a, n), wb = -cross(r_b, n);
            V3<T> ka = matvec(Ia, wa), kb = matvec(Ib, wb);
            row.meff_n = T(1) / (ra.inv_mass + rb.inv_mass + dot(wa, ka) + dot(wb, kb));
            V3<T> vca = ld3(VA.v) + cross(ld3(VA.w), r_a);
            V3<T> vcb = ld3(VB.v) + cross(ld3(VB.w), r_b);
            T vreln = dot(vca - vcb, n);
            T e = tmax(ra.restitution, rb.restitution);
            T rbias = T(0);
            if (vreln < -rthr) rbias = e * vreln;
            T bbias = (T(-0.1) / dt) * tmax(T(0), pen - T(0.005));
            row.bias = tmin(bbias, rbias);
            st3(row.n, n);
            st3(row.wa_n, wa);
            st3(row.wb_n, wb);
            // friction rows on the orthonormal basis of n (constraint.h:104-113)
            T sign = copysign_one(n.z);
            T a_ = T(-1) / (sign + n.z);
            T b_ = n.x * n.y * a_;
            V3<T> t1{T(1) + sign * n.x * n.x * a_, sign * b_, -sign * n.x};
            V3<T> t2{b_, sign + n.y * n.y * a_, -n.y};
            V3<T> wa1 = cross(r_a, t1), wb1 = -cross(r_b, t1);
            V3<T> ka1 = matvec(Ia, wa1), kb1 = matvec(Ib, wb1);
            row.meff_t1 = T(1) / (ra.inv_mass + rb.inv_mass + dot(wa1, ka1) + dot(wb1, kb1));
            V3<T> wa2 = cross(r_a, t2), wb2 = -cross(r_b, t2);
            V3<T> ka2 = matvec(Ia, wa2), kb2 = matvec(Ib, wb2);
            row.meff_t2 = T(1) / (ra.inv_mass + rb.inv_mass + dot(wa2, ka2) + dot(wb2, kb2));
            st3(row.t1, t1);
            st3(row.wa_t1, wa1);
            st3(row.wb_t1, wb1);
            st3(row.t2, t2);
            st3(row.wa_t2, wa2);
            st3(row.wb_t2, wb2);
            row.mu = pk_sqrt(ra.friction * rb.friction);
            T m11 = T(1) / row.meff_t1, m22 = T(1) / row.meff_t2;
            T m12 = dot(wa1, matvec(Ia, wa2)) + dot(wb1, matvec(Ib, wb2));
            T det = m11 * m22 - m12 * m12;
            if (det > T(0))
            {
                row.inv11 = m22 / det;
                row.inv22 = m11 / det;
                row.inv12 = -m12 / det;
            }
            else
            {
                row.inv11 = row.meff_t1;
                row.inv22 = row.meff_t2;
                row.inv12 = T(0);
            }
            row.pad = T(0);
            if constexpr (std::is_same<T, float>::value)
            {
                RowF rf;
                st3(rf.n, n);
                st3(rf.wa_n, wa);
                st3(rf.wb_n, wb);
                st3(rf.ka_n, ka);
                st3(rf.kb_n, kb);
                st3(rf.t1, t1);
                st3(rf.wa_t1, wa1);
                st3(rf.wb_t1, wb1);
                st3(rf.ka_t1, ka1);
                st3(rf.kb_t1, kb1);
                st3(rf.t2, t2);
                st3(rf.wa_t2, wa2);
                st3(rf.wb_t2, wb2);
                st3(rf.ka_t2, ka2);
                st3(rf.kb_t2, kb2);
                rf.meff_n = row.meff_n;
                rf.bias = row.bias;
                rf.inv11 = row.inv11;
                rf.inv12 = row.inv12;
                rf.inv22 = row.inv22;
                rf.mu = row.mu;
                rf.pad = 0.0f;
                d.rows[4 * size_t(ci) + k] = rf;
                for (int j = 0; j < 3; ++j)
                {
                    d.raccf[12 * size_t(ci) + 3 * k + j] = float(c.imp[j]);
                    d.rdel[12 * size_t(ci) + 3 * k + j] = 0.0f;
                }
            }
            else
                d.rows[4 * size_t(ci) + k] = row;
            d.racc[12 * size_t(ci) + 3 * k + 0] = c.imp[0];
            d.racc[12 * size_t(ci) + 3 * k + 1] = c.imp[1];
            d.racc[12 * size_t(ci) + 3 * k + 2] = c.imp[2];
            mask |= uint8_t(1u << k);
        }
        d.rowmask[p] = mask;
    }
}

// ------------------------------------------------------------------------------------------------
// solver: one CTA per world; colouring, warm start, iterations (constraint.h:1107-1201)
// ------------------------------------------------------------------------------------------------
// A body as the solver sees it while one thread processes one manifold: velocities and the world
// inverse inertia in registers, loaded once and stored once per manifold. Within a colour no
// other thread touches the same dynamic body, so the result equals updating memory in place.
template <class T> struct SBody
{
    V3<T> v, w;
    T I[9];
    T inv_mass;
    bool is_static;
};

template <class T> __device__ __forceinline__ T jv_reg(const T *J, const T *Wa, const T *Wb, const SBody<T> &a, const SBody<T> &b)
{
    // J_v.v_a + J_w_a.w_a - J_v.v_b + J_w_b.w_b (constraint.h:52-53), left to right
    return dot(ld3(J), a.v) + dot(ld3(Wa), a.w) - dot(ld3(J), b.v) + dot(ld3(Wb), b.w);
}

template <class T> __device__ __forceinline__ void apply_reg(SBody<T> &a, SBody<T> &b, V3<T> J, V3<T> Wa, V3<T> Wb, T lam)
{
    // apply_impulse / apply_angular_impulse (particle.h:88-93); static bodies are not written
    if (!a.is_static)
    {
        a.v = a.v + (J * lam) * a.inv_mass;
        a.w = a.w + matvec(a.I, Wa * lam);
    }
    if (!b.is_static)
    {
        b.v = b.v + ((-J) * lam) * b.inv_mass;
        b.w = b.w + matvec(b.I, Wb * lam);
    }
}

template <class T> __device__ __forceinline__ void warm_contact(SBody<T> &A, SBody<T> &B, const Row<T> &r, const double *acc)
{
    // jacobian_row::warm_start for the three rows (constraint.h:73-87, 1125-1130)
    if (acc[0] != 0.0) apply_reg(A, B, ld3(r.n), ld3(r.wa_n), ld3(r.wb_n), T(acc[0]));
    if (acc[1] != 0.0) apply_reg(A, B, ld3(r.t1), ld3(r.wa_t1), ld3(r.wb_t1), T(acc[1]));
    if (acc[2] != 0.0) apply_reg(A, B, ld3(r.t2), ld3(r.wa_t2), ld3(r.wb_t2), T(acc[2]));
}

// Rows of every joint from the bodies' current poses (build_jacobian_impl of each type,
// constraint.h:187-231, 309-352, 407-446, 512-580, 654-738, 789-855), in the oracle's order of
// operations.
template <class T> __global__ void k_joint_setup(Dev<T> d, T dt)
{
    const int nj = *d.njoints;
    PK_GRID_STRIDE(j, nj)
    {
        const JointDev<T> jd = d.joints[j];
        const int sa = jd.a, sb = jd.b;
        const Pose<T> &PA = d.pose[sa];
        const Pose<T> &PB = d.pose[sb];
        const Qt<T> qa = ldq(PA.q), qb = ldq(PB.q);
        const V3<T> xa = ld3(PA.p), xb = ld3(PB.p);
        const T *Ia = d.iwinv + 9 * sa;
        const T *Ib = d.iwinv + 9 * sb;
        const T ima = d.prm[sa].inv_mass, imb = d.prm[sb].inv_mass;
        const V3<T> r_a = rotate(qa, ld3(jd.la)), r_b = rotate(qb, ld3(jd.lb));
        const V3<T> delta = (xa + r_a) - (xb + r_b);
        JRow<T> *out = d.jrows + size_t(j) * kJointMaxRows;
        int nr = 0;
        auto linear = [&](V3<T> n, V3<T> arm_a, T bias_factor, bool slider) {
            JRow<T> r;
            V3<T> Jwa = cross(arm_a, n), Jwb = -cross(r_b, n);
            V3<T> ka = matvec(Ia, Jwa), kb = matvec(Ib, Jwb);
            r.gamma = T(0);
            if (slider)
            {
                T lin = ima + imb;
                T ang = dot(Jwa, ka) + dot(Jwb, kb);
                T reg = T(0.01) * ang;
                r.gamma = reg;
                r.meff = T(1) / (lin + ang + reg);
                T e = dot(delta, n);
                e = (e < T(-0.2)) ? T(-0.2) : ((T(0.2) < e) ? T(0.2) : e);
                r.bias = (bias_factor / dt) * e;
            }
            else
            {
                r.meff = T(1) / (ima + imb + dot(Jwa, ka) + dot(Jwb, kb));
                r.bias = (bias_factor / dt) * dot(delta, n);
            }
            st3(r.Jv, n);
            st3(r.Jwa, Jwa);
            st3(r.Jwb, Jwb);
            out[nr++] = r;
        };
        auto angular = [&](V3<T> n, T bias_factor, V3<T> err) {
            JRow<T> r;
            V3<T> Jwa = n, Jwb = -n;
            V3<T> ka = matvec(Ia, Jwa), kb = matvec(Ib, Jwb);
            r.meff = T(1) / (dot(Jwa, ka) + dot(Jwb, kb));
            r.bias = (bias_factor / dt) * dot(err, n);
            r.gamma = T(0);
            st3(r.Jv, V3<T>{T(0), T(0), T(0)});
            st3(r.Jwa, Jwa);
            st3(r.Jwb, Jwb);
            out[nr++] = r;
        };
        auto rel_error = [&]() {
            Qt<T> cur = qmul(conj(qa), qb);
            Qt<T> e = qmul(ldq(jd.qrel), conj(cur));
            if (e.w < T(0)) e = Qt<T>{-e.w, -e.x, -e.y, -e.z};
            return rotate(qa, V3<T>{e.x, e.y, e.z} * T(2));
        };
        const V3<T> ex{T(1), T(0), T(0)}, ey{T(0), T(1), T(0)}, ez{T(0), T(0), T(1)};
        switch (jd.type)
        {
        case 0:
        case 5: {
            T cur = norm(delta);
            if (cur < T(1e-6)) break;
            V3<T> u = delta / cur;
            JRow<T> r;
            V3<T> Jwa = cross(r_a, u), Jwb = -cross(r_b, u);
            V3<T> ka = matvec(Ia, Jwa), kb = matvec(Ib, Jwb);
            if (jd.type == 0)
            {
                r.meff = T(1) / (ima + imb + dot(Jwa, ka) + dot(Jwb, kb));
                r.bias = (T(0.1) / dt) * (cur - jd.distance);
                r.gamma = T(0);
            }
            else
            {
                T mc = ima + imb + dot(Jwa, ka) + dot(Jwb, kb);
                T gamma = T(1) / (dt * (jd.damping + dt * jd.stiffness));
                T beta = dt * jd.stiffness / (jd.damping + dt * jd.stiffness);
                r.meff = T(1) / (mc + gamma);
                r.bias = (beta / dt) * (cur - jd.distance);
                r.gamma = gamma;
            }
            st3(r.Jv, u);
            st3(r.Jwa, Jwa);
            st3(r.Jwb, Jwb);
            out[nr++] = r;
            break;
        }
        case 1:
            linear(ex, r_a, T(0.1), false);
            linear(ey, r_a, T(0.1), false);
            linear(ez, r_a, T(0.1), false);
            break;
        case 2: {
            linear(ex, r_a, T(0.2), false);
            linear(ey, r_a, T(0.2), false);
            linear(ez, r_a, T(0.2), false);
            V3<T> u_a = rotate(qa, ld3(jd.axa)), u_b = rotate(qb, ld3(jd.axb));
            V3<T> err = -cross(u_a, u_b);
            angular(rotate(qa, ld3(jd.va)), T(0.2), err);
            angular(rotate(qa, ld3(jd.wa)), T(0.2), err);
            break;
        }
        case 3: {
            V3<T> axis_a = rotate(qa, ld3(jd.axa));
            V3<T> t1 = rotate(qa, ld3(jd.va)), t2 = rotate(qa, ld3(jd.wa));
            V3<T> lever = r_a - delta;
            linear(t1, lever, T(0.1), true);
            linear(t2, lever, T(0.1), true);
            V3<T> err = rel_error();
            angular(axis_a, T(0.1), err);
            angular(t1, T(0.1), err);
            angular(t2, T(0.1), err);
            break;
        }
        case 4: {
            linear(ex, r_a, T(0.1), false);
            linear(ey, r_a, T(0.1), false);
            linear(ez, r_a, T(0.1), false);
            V3<T> err = rel_error();
            angular(ex, T(0.1), err);
            angular(ey, T(0.1), err);
            angular(ez, T(0.1), err);
            break;
        }
        default:
            break;
        }
        d.jnrows[j] = nr;
    }
}

// The joints [js, je) of one world, in order, by one thread: warm start, or one pass of
// jacobian_row::apply (constraint.h:49-71) over their rows. Solved before the contacts of the same
// pass, as the reference does (constraint.h:1121-1137).
template <class T>
__device__ __noinline__ void solve_joints(const Dev<T> &d, int js, int je, Vel<T> *cache, bool warm, bool coherent)
{
    for (int j = js; j < je; ++j)
    {
        const JointDev<T> &jd = d.joints[j];
        const int nr = d.jnrows[j];
        if (nr == 0) continue;
        SBody<T> A, B;
        const int sl[2] = {jd.a, jd.b}, lc[2] = {jd.local_a, jd.local_b};
        SBody<T> *bs[2] = {&A, &B};
        for (int k = 0; k < 2; ++k)
        {
            SBody<T> &bb = *bs[k];
            const int s = sl[k];
            bb.is_static = (d.meta[s].flags & BODY_STATIC) != 0;
            Vel<T> ve;
            if (cache && !bb.is_static)
                ve = cache[lc[k]];
            else if (coherent)
            {
                const T *src = reinterpret_cast<const T *>(d.vel + s);
                for (int q = 0; q < 3; ++q)
                {
                    ve.v[q] = __ldcg(src + q);
                    ve.w[q] = __ldcg(src + 3 + q);
                }
            }
            else
                ve = d.vel[s];
            bb.v = ld3(ve.v);
            bb.w = ld3(ve.w);
            for (int q = 0; q < 9; ++q) bb.I[q] = d.iwinv[9 * s + q];
            bb.inv_mass = d.prm[s].inv_mass;
        }
        for (int r = 0; r < nr; ++r)
        {
            const JRow<T> row = d.jrows[size_t(j) * kJointMaxRows + r];
            double &acc = d.jacc[size_t(j) * kJointMaxRows + r];
            if (warm)
            {
                if (acc != 0.0) apply_reg(A, B, ld3(row.Jv), ld3(row.Jwa), ld3(row.Jwb), T(acc));
                continue;
            }
            T Jv = jv_reg(row.Jv, row.Jwa, row.Jwb, A, B);
            T cfp = row.gamma * T(acc);
            T lambda = -(Jv + row.bias + cfp) * row.meff;
            double old = acc;
            double v = old + double(lambda);
            const double lo = -1.7976931348623157e308, hi = 1.7976931348623157e308;
            acc = (v < lo) ? lo : ((hi < v) ? hi : v);
            apply_reg(A, B, ld3(row.Jv), ld3(row.Jwa), ld3(row.Jwb), T(acc - old));
        }
        for (int k = 0; k < 2; ++k)
        {
            const SBody<T> &bb = *bs[k];
            if (bb.is_static) continue;
            Vel<T> ve;
            st3(ve.v, bb.v);
            st3(ve.w, bb.w);
            if (cache)
                cache[lc[k]] = ve;
            else
                d.vel[sl[k]] = ve;
        }
    }
}

// FP32 form: apply an impulse along one direction (J, with the rotation responses ka and kb).
__device__ __forceinline__ void apply_f32(SBody<float> &A, SBody<float> &B, const float *J, const float *ka, const float *kb,
                                          float lam)
{
    if (!A.is_static)
    {
        A.v = A.v + ld3(J) * (lam * A.inv_mass);
        A.w = A.w + ld3(ka) * lam;
    }
    if (!B.is_static)
    {
        B.v = B.v - ld3(J) * (lam * B.inv_mass);
        B.w = B.w + ld3(kb) * lam;
    }
}

// FP32 form of one contact (constraint.h:49-71 and 1138-1187 in FP32). The accumulated impulses
// are FP64 across steps; within a step, the running total is carried in FP32 (tot: clamp
// decisions) and the change in FP32 (del), which is added to the FP64 accumulator (base) once
// after the sweeps. Clamping the normal impulse at zero sets the FP64 accumulator to exactly zero.
// FP64 issues at a small fraction of the FP32 rate here, so the sweeps hold no FP64 arithmetic.
__device__ __forceinline__ void solve_contact_f32(SBody<float> &A, SBody<float> &B, const RowF &r, float *tot, float *del,
                                                  double *base)
{
    {
        float Jv = jv_reg(r.n, r.wa_n, r.wb_n, A, B);
        float lambda = -(Jv + r.bias) * r.meff_n;
        float nf = tot[0] + lambda;
        float dl;
        if (nf < 0.0f)
        {
            dl = -tot[0];
            tot[0] = 0.0f;
            del[0] = 0.0f;
            *base = 0.0;
        }
        else
        {
            dl = lambda;
            tot[0] = nf;
            del[0] = del[0] + lambda;
        }
        apply_f32(A, B, r.n, r.ka_n, r.kb_n, dl);
    }
    float maxf = r.mu * tot[0];
    float b1 = jv_reg(r.t1, r.wa_t1, r.wb_t1, A, B);
    float b2 = jv_reg(r.t2, r.wa_t2, r.wb_t2, A, B);
    float l1 = -(r.inv11 * b1 + r.inv12 * b2);
    float l2 = -(r.inv12 * b1 + r.inv22 * b2);
    float o1 = tot[1], o2 = tot[2];
    float n1 = o1 + l1, n2 = o2 + l2;
    float mag2 = n1 * n1 + n2 * n2;
    if (mag2 > maxf * maxf)
    {
        // IEEE square root and divide: with a tiny normal impulse maxf^2 underflows and mag2 can be
        // subnormal, where an approximate reciprocal square root would return infinity
        float sc = maxf / sqrtf(mag2);
        n1 = n1 * sc;
        n2 = n2 * sc;
    }
    float a1 = n1 - o1, a2 = n2 - o2;
    tot[1] = n1;
    tot[2] = n2;
    del[1] = del[1] + a1;
    del[2] = del[2] + a2;
    if (!A.is_static)
    {
        A.v = A.v + (ld3(r.t1) * a1 + ld3(r.t2) * a2) * A.inv_mass;
        A.w = A.w + ld3(r.ka_t1) * a1 + ld3(r.ka_t2) * a2;
    }
    if (!B.is_static)
    {
        B.v = B.v - (ld3(r.t1) * a1 + ld3(r.t2) * a2) * B.inv_mass;
        B.w = B.w + ld3(r.kb_t1) * a1 + ld3(r.kb_t2) * a2;
    }
}

__device__ __forceinline__ void warm_contact_f32(SBody<float> &A, SBody<float> &B, const RowF &r, const float *tot)
{
    if (tot[0] != 0.0f) apply_f32(A, B, r.n, r.ka_n, r.kb_n, tot[0]);
    if (tot[1] != 0.0f) apply_f32(A, B, r.t1, r.ka_t1, r.kb_t1, tot[1]);
    if (tot[2] != 0.0f) apply_f32(A, B, r.t2, r.ka_t2, r.kb_t2, tot[2]);
}

template <class T> __device__ __forceinline__ void solve_contact(SBody<T> &A, SBody<T> &B, const Row<T> &r, double *acc_)
{
    // normal row: jacobian_row::apply (constraint.h:49-71), gamma = 0
    {
        T Jv = jv_reg(r.n, r.wa_n, r.wb_n, A, B);
        T cfp = T(0) * T(acc_[0]);
        T lambda = -(Jv + r.bias + cfp) * r.meff_n;
        double old = acc_[0];
        double v = old + double(lambda);
        double lo = 0.0, hi = 1.7976931348623157e308;
        double acc = (v < lo) ? lo : ((hi < v) ? hi : v);
        acc_[0] = acc;
        apply_reg(A, B, ld3(r.n), ld3(r.wa_n), ld3(r.wb_n), T(acc - old));
    }
    // coupled 2D friction with circular cone clamp (constraint.h:1138-1187)
    T maxf = r.mu * T(acc_[0]);
    T Jv1 = jv_reg(r.t1, r.wa_t1, r.wb_t1, A, B);
    T Jv2 = jv_reg(r.t2, r.wa_t2, r.wb_t2, A, B);
    T b1 = Jv1 + T(0), b2 = Jv2 + T(0);
    T l1 = -(r.inv11 * b1 + r.inv12 * b2);
    T l2 = -(r.inv12 * b1 + r.inv22 * b2);
    double o1 = acc_[1], o2 = acc_[2];
    double n1 = o1 + double(l1), n2 = o2 + double(l2);
    double mag = pk_sqrt(n1 * n1 + n2 * n2);
    if (mag > double(maxf))
    {
        n1 = n1 * (double(maxf) / mag);
        n2 = n2 * (double(maxf) / mag);
    }
    acc_[1] = n1;
    acc_[2] = n2;
    T a1 = T(n1 - o1), a2 = T(n2 - o2);
    if (!A.is_static)
    {
        V3<T> imp = ld3(r.t1) * a1 + ld3(r.t2) * a2;
        A.v = A.v + imp * A.inv_mass;
        A.w = A.w + matvec(A.I, ld3(r.wa_t1) * a1 + ld3(r.wa_t2) * a2);
    }
    if (!B.is_static)
    {
        V3<T> imp = (-ld3(r.t1)) * a1 - ld3(r.t2) * a2;
        B.v = B.v + imp * B.inv_mass;
        B.w = B.w + matvec(B.I, ld3(r.wb_t1) * a1 + ld3(r.wb_t2) * a2);
    }
}

template <class T>
__device__ __forceinline__ void load_sbody(const Dev<T> &d, int s, const Vel<T> *cache, SBody<T> &b, bool coherent)
{
    const Meta m = d.meta[s];
    b.is_static = (m.flags & BODY_STATIC) != 0;
    if (coherent)
    {
        // other SMs wrote this body in earlier colours: read through L2, not a stale L1 line
        const T *src = reinterpret_cast<const T *>(d.vel + s);
        b.v = V3<T>{__ldcg(src + 0), __ldcg(src + 1), __ldcg(src + 2)};
        b.w = V3<T>{__ldcg(src + 3), __ldcg(src + 4), __ldcg(src + 5)};
    }
    else
    {
        const Vel<T> ve = (cache && !b.is_static) ? cache[m.local] : d.vel[s];
        b.v = ld3(ve.v);
        b.w = ld3(ve.w);
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) b.I[k] = d.iwinv[9 * s + k];
    b.inv_mass = d.prm[s].inv_mass;
}

template <class T> __device__ __forceinline__ void store_sbody(const Dev<T> &d, int s, Vel<T> *cache, const SBody<T> &b)
{
    if (b.is_static) return;
    Vel<T> ve;
    st3(ve.v, b.v);
    st3(ve.w, b.w);
    if (cache)
        cache[d.meta[s].local] = ve;
    else
        d.vel[s] = ve;
}

// Rows do not change while the solver sweeps: read-only vector loads, which the compiler may issue
// for all of a manifold's rows before the first contact is solved.
template <class R> __device__ __forceinline__ R ldg_row(const R *src)
{
    constexpr int nv = int(sizeof(R) / 16);
    float4 v[nv];
    const float4 *s = reinterpret_cast<const float4 *>(src);
#pragma unroll
    for (int i = 0; i < nv; ++i) v[i] = __ldg(s + i);
    R r;
    memcpy(&r, v, sizeof(r));
    return r;
}

// The contact rows of one manifold: warm start (warm = true) or one Gauss-Seidel pass in order.
__device__ __forceinline__ void solve_rows(const Dev<float> &d, int p, SBody<float> &A, SBody<float> &B, bool warm)
{
    const uint8_t mask = d.rowmask[p];
    const size_t ri = size_t(d.rowidx[p]);
    float tot[12];
    float4 *tp = reinterpret_cast<float4 *>(d.raccf + 12 * ri);
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float4 v = tp[i];
        tot[4 * i] = v.x;
        tot[4 * i + 1] = v.y;
        tot[4 * i + 2] = v.z;
        tot[4 * i + 3] = v.w;
    }
    const RowF *rp = d.rows + 4 * ri;
    if (warm)
    {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (mask & (1u << q)) warm_contact_f32(A, B, ldg_row(rp + q), tot + 3 * q);
        return;
    }
    float del[12];
    float4 *dp = reinterpret_cast<float4 *>(d.rdel + 12 * ri);
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float4 v = dp[i];
        del[4 * i] = v.x;
        del[4 * i + 1] = v.y;
        del[4 * i + 2] = v.z;
        del[4 * i + 3] = v.w;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (mask & (1u << q)) solve_contact_f32(A, B, ldg_row(rp + q), tot + 3 * q, del + 3 * q, d.racc + 12 * ri + 3 * q);
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        tp[i] = make_float4(tot[4 * i], tot[4 * i + 1], tot[4 * i + 2], tot[4 * i + 3]);
        dp[i] = make_float4(del[4 * i], del[4 * i + 1], del[4 * i + 2], del[4 * i + 3]);
    }
}

__device__ __forceinline__ void solve_rows(const Dev<double> &d, int p, SBody<double> &A, SBody<double> &B, bool warm)
{
    const uint8_t mask = d.rowmask[p];
    const size_t ri = size_t(d.rowidx[p]);
    double acc[12];
    double2 *ap = reinterpret_cast<double2 *>(d.racc + 12 * ri);
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        double2 v = ap[i];
        acc[2 * i] = v.x;
        acc[2 * i + 1] = v.y;
    }
    const Row<double> *rp = d.rows + 4 * ri;
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        if (!(mask & (1u << q))) continue;
        const Row<double> r = ldg_row(rp + q);
        if (warm)
            warm_contact(A, B, r, acc + 3 * q);
        else
            solve_contact(A, B, r, acc + 3 * q);
    }
    if (!warm)
    {
#pragma unroll
        for (int i = 0; i < 6; ++i) ap[i] = make_double2(acc[2 * i], acc[2 * i + 1]);
    }
}

// Accumulated impulses of row q of pair p into the manifold cache (the FP32 form adds this
// step's change to the FP64 accumulator here, once).
template <class T> __device__ __forceinline__ void store_impulses(const Dev<T> &d, int p, int q)
{
    const size_t o = 12 * size_t(d.rowidx[p]) + 3 * q;
    Contact<T> &c = d.man_new[p].c[q];
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
        if constexpr (std::is_same<T, float>::value)
            c.imp[j] = d.racc[o + j] + double(d.rdel[o + j]);
        else
            c.imp[j] = d.racc[o + j];
    }
}

// One manifold by pair index (the grid-wide solver).
template <class T>
__device__ __forceinline__ void solve_manifold(const Dev<T> &d, int p, uint64_t sv, Vel<T> *cache, bool warm,
                                               bool coherent = false)
{
    int sa = int(sv >> 32), sb = int(sv & 0xFFFFFFFFu);
    SBody<T> A, B;
    load_sbody(d, sa, cache, A, coherent);
    load_sbody(d, sb, cache, B, coherent);
    solve_rows(d, p, A, B, warm);
    store_sbody(d, sa, cache, A);
    store_sbody(d, sb, cache, B);
}

// Solve record of an active manifold, written once per step by the colouring: the pair index, both
// slots with the static flag in bit 31, and both world-local indices (16 bits each; read only when
// the world's velocities are cached in shared memory, whose size keeps them below 2^16). One load
// replaces the chain pair index -> slot pair -> body meta on every sweep.
template <class T> __device__ __forceinline__ uint4 make_solve_rec(const Dev<T> &d, int p, uint64_t sv)
{
    int a = int(sv >> 32), b = int(sv & 0xFFFFFFFFu);
    const Meta ma = d.meta[a], mb = d.meta[b];
    uint4 r;
    r.x = uint32_t(p);
    r.y = uint32_t(a) | ((ma.flags & BODY_STATIC) ? 0x80000000u : 0u);
    r.z = uint32_t(b) | ((mb.flags & BODY_STATIC) ? 0x80000000u : 0u);
    r.w = (uint32_t(ma.local) & 0xFFFFu) | (uint32_t(mb.local) << 16);
    return r;
}

template <class T>
__device__ __forceinline__ void store_rec_body(const Dev<T> &d, uint32_t sw, int local, Vel<T> *cache, const SBody<T> &b)
{
    if (b.is_static) return;
    Vel<T> ve;
    st3(ve.v, b.v);
    st3(ve.w, b.w);
    if (cache)
        cache[local] = ve;
    else
        d.vel[int(sw & 0x7FFFFFFFu)] = ve;
}

template <class T>
__device__ __forceinline__ void load_rec_body(const Dev<T> &d, uint32_t sw, int local, const Vel<T> *cache, SBody<T> &b)
{
    const int s = int(sw & 0x7FFFFFFFu);
    b.is_static = (sw >> 31) != 0;
    const Vel<T> ve = (cache && !b.is_static) ? cache[local] : d.vel[s];
    b.v = ld3(ve.v);
    b.w = ld3(ve.w);
    if constexpr (!std::is_same<T, float>::value) // the FP32 rows carry I^-1 J
    {
#pragma unroll
        for (int k = 0; k < 9; ++k) b.I[k] = d.iwinv[9 * s + k];
    }
    b.inv_mass = d.prm[s].inv_mass;
}

template <class T> __device__ __forceinline__ void solve_manifold_rec(const Dev<T> &d, uint4 rec, Vel<T> *cache, bool warm)
{
    const int la = int(rec.w & 0xFFFFu), lb = int(rec.w >> 16);
    SBody<T> A, B;
    load_rec_body(d, rec.y, la, cache, A);
    load_rec_body(d, rec.z, lb, cache, B);
    solve_rows(d, int(rec.x), A, B, warm);
    store_rec_body(d, rec.y, la, cache, A);
    store_rec_body(d, rec.z, lb, cache, B);
}

// One round of parallel first fit, in three phases separated by block- or grid-wide barriers.
// pick: the lowest colour taken on neither dynamic body (and both bodies' keys reset); all 128
// taken sets *over. claim: the lowest key wins each body. commit: a manifold that won both bodies
// takes its colour, marked on its bodies for the next rounds.
template <class T> __device__ __forceinline__ int colour_rounds_pick(const Dev<T> &d, uint4 r, int *over)
{
    unsigned long long u0 = 0ull, u1 = 0ull;
    if (!(r.y >> 31))
    {
        const ulonglong2 u = __ldcg(d.used + r.y);
        u0 |= u.x;
        u1 |= u.y;
        d.owner[r.y] = ~0ull;
    }
    if (!(r.z >> 31))
    {
        const ulonglong2 u = __ldcg(d.used + (r.z & 0x7FFFFFFFu));
        u0 |= u.x;
        u1 |= u.y;
        d.owner[r.z & 0x7FFFFFFFu] = ~0ull;
    }
    if (~u0) return __ffsll(~u0) - 1;
    if (~u1) return 64 + __ffsll(~u1) - 1;
    *over = 1;
    return 0;
}
template <class T> __device__ __forceinline__ void colour_rounds_claim(const Dev<T> &d, uint4 r, uint64_t key)
{
    if (!(r.y >> 31)) atomicMin(reinterpret_cast<unsigned long long *>(d.owner + r.y), (unsigned long long)key);
    if (!(r.z >> 31)) atomicMin(reinterpret_cast<unsigned long long *>(d.owner + (r.z & 0x7FFFFFFFu)), (unsigned long long)key);
}
template <class T> __device__ __forceinline__ bool colour_rounds_commit(const Dev<T> &d, uint4 r, uint64_t key, int c)
{
    const bool da = !(r.y >> 31), db = !(r.z >> 31);
    const int sa = int(r.y & 0x7FFFFFFFu), sb = int(r.z & 0x7FFFFFFFu);
    const bool won = (!da || __ldcg(reinterpret_cast<const unsigned long long *>(d.owner + sa)) == key) &&
                     (!db || __ldcg(reinterpret_cast<const unsigned long long *>(d.owner + sb)) == key);
    if (!won) return false;
    unsigned long long *ua = reinterpret_cast<unsigned long long *>(d.used + sa);
    unsigned long long *ub = reinterpret_cast<unsigned long long *>(d.used + sb);
    const int w = c >> 6;
    const unsigned long long bit = 1ull << (c & 63);
    if (da) atomicOr(ua + w, bit);
    if (db) atomicOr(ub + w, bit);
    return true;
}

// MAXT: the largest CTA the instance is compiled for (256, or 512 for the FP32 form's large worlds;
// the 512 instance gives up registers for threads).
#ifndef PK_SOLVE_MIN_BLOCKS
#define PK_SOLVE_MIN_BLOCKS 2
#endif
// Solve records are laid out in two passes within each colour: first the manifolds with rows in
// contact slots 2-3, then the others, so that the lanes of a warp mostly run the same contact
// slots. Order within a colour does not change results: its manifolds share no dynamic body.
template <class T> __device__ __forceinline__ bool wide_manifold(const Dev<T> &d, const uint4 &r)
{ return (d.rowmask[r.x] >> 2) != 0; }

// First fit in pair order for one world (one thread): each manifold takes the lowest colour that
// none of the earlier manifolds on its dynamic bodies has, from a 128-bit used-colour mask per
// local index (`used`, 2 words per local index, zeroed by the caller). Returns the number of
// colours, or -1 when a body would need a colour above 127.
__device__ __forceinline__ int first_fit_colours(const uint4 *__restrict__ rec, int na, uint64_t *used, int *colour)
{
    int top = 0;
    constexpr int kAhead = 8; // records loaded ahead of the mask chain
    for (int k0 = 0; k0 < na; k0 += kAhead)
    {
        uint4 rr[kAhead];
#pragma unroll
        for (int j = 0; j < kAhead; ++j) rr[j] = k0 + j < na ? rec[k0 + j] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
        for (int j = 0; j < kAhead; ++j)
        {
            if (k0 + j >= na) break;
            const uint4 r = rr[j];
            const bool da = !(r.y >> 31), db = !(r.z >> 31);
            const int la = int(r.w & 0xFFFFu), lb = int(r.w >> 16);
            uint64_t u0 = 0ull, u1 = 0ull;
            if (da)
            {
                u0 |= used[2 * la];
                u1 |= used[2 * la + 1];
            }
            if (db)
            {
                u0 |= used[2 * lb];
                u1 |= used[2 * lb + 1];
            }
            int c;
            if (~u0)
                c = __ffsll(~u0) - 1;
            else if (~u1)
                c = 64 + __ffsll(~u1) - 1;
            else
                return -1; // a body with 128 manifolds in one step
            colour[k0 + j] = c;
            const uint64_t b0 = c < 64 ? (1ull << c) : 0ull, b1 = c < 64 ? 0ull : (1ull << (c - 64));
            if (da)
            {
                used[2 * la] |= b0;
                used[2 * la + 1] |= b1;
            }
            if (db)
            {
                used[2 * lb] |= b0;
                used[2 * lb + 1] |= b1;
            }
            top = c + 1 > top ? c + 1 : top;
        }
    }
    return top;
}

// One active world's compaction, colouring, sweeps and write-back on the whole CTA (every thread
// calls it). solve_smem caches the world's body velocities when it has at most cache_bodies local
// indices.
template <class T, int MAXT, bool JOINTS>
__device__ __forceinline__ void solve_world_cta(const Dev<T> &d, const uint64_t *__restrict__ sval, int w,
                                                int cache_bodies, unsigned char *solve_smem)
{
    __shared__ int ccount[kMaxColours];
    __shared__ int cstart[kMaxColours];
    __shared__ int cursor[kMaxColours];
    __shared__ int wsum[MAXT / 32];
    __shared__ int remaining;
    __shared__ int nactive;
    const int ms = d.mstart[w], me = d.mend[w];
    const int js = JOINTS ? d.jstart[w] : 0, je = JOINTS ? d.jend[w] : 0; // instance without joints
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    if (me <= ms && je <= js)
    {
        if (tid == 0) d.ncolours[w] = 0;
        return;
    }
    const bool fits = d.world_nlocal[w] <= cache_bodies;
    Vel<T> *cache = fits ? reinterpret_cast<Vel<T> *>(solve_smem) : nullptr;
    uint64_t *sowner = fits ? reinterpret_cast<uint64_t *>(solve_smem) : nullptr; // during colouring only
    uint4 *rec = d.crec + ms; // solve records of the active manifolds, ascending pair index

    // 1. compact the manifolds that have contact rows (stable: ascending pair index). Each thread
    //    takes a contiguous run of pairs, counts, and after one block scan writes its records.
    {
        const int per = (me - ms + nt - 1) / nt;
        const int lo = min(me, ms + tid * per), hi = min(me, lo + per);
        int cnt = 0;
        for (int p = lo; p < hi; ++p) cnt += d.rowmask[p] != 0;
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1)
        {
            int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (tid == 0)
        {
            int run = 0;
            for (int k = 0; k < nt / 32; ++k)
            {
                int v = wsum[k];
                wsum[k] = run;
                run += v;
            }
            nactive = run;
        }
        __syncthreads();
        int off = wsum[warp] + incl - cnt;
        for (int p = lo; p < hi; ++p)
            if (d.rowmask[p] != 0) rec[off++] = make_solve_rec(d, p, sval[p]);
    }
    __syncthreads();
    const int na = nactive;
    int *colour = d.colour_tmp + ms; // colour of rec[k]
    for (int k = tid; k < na; k += nt) colour[k] = -1;
    for (int c = tid; c < kMaxColours; c += nt)
    {
        ccount[c] = 0;
        cursor[c] = 0;
    }
    if (tid == 0) remaining = na;
    __syncthreads();

    // 2. colouring. Worlds up to kFirstFitMax local indices: first fit in pair order, each manifold
    //    taking the lowest colour that none of the earlier manifolds on its dynamic bodies has
    //    (one thread; a 128-bit used-colour mask per body). Larger worlds, and worlds where a body
    //    would need a first-fit colour above 127: rounds of parallel first fit (ff_key); where a
    //    body would need a colour above 127 there too: each uncoloured manifold claims its dynamic
    //    bodies with its index; the winners of all their bodies take the round number. Bodies are
    //    keyed by world-local index when the table fits in shared memory, else by slot.
    __shared__ int ff_ncol;
    int round = 0;
    bool coloured = false;
    if (d.world_nlocal[w] <= kFirstFitMax)
    {
        uint64_t *used = reinterpret_cast<uint64_t *>(solve_smem); // 2 words per local index
        for (int l = tid; l < 2 * d.world_nlocal[w]; l += nt) used[l] = 0ull;
        __syncthreads();
        if (tid == 0) ff_ncol = first_fit_colours(rec, na, used, colour);
        __syncthreads();
        if (ff_ncol >= 0)
        {
            round = ff_ncol;
            coloured = true;
        }
        else
        {
            for (int k = tid; k < na; k += nt) colour[k] = -1; // claiming rounds from scratch
            __syncthreads();
        }
    }
    if (!coloured)
    {
        // rounds of parallel first fit, global tables by slot (16 B of taken colours, 8 B of key)
        __shared__ int rb_left, rb_over, rb_top;
        int *tcol = reinterpret_cast<int *>(d.order) + ms; // free until the grid solver's ordering
        for (int k = tid; k < na; k += nt)
        {
            colour[k] = -1;
            const uint4 r = rec[k];
            if (!(r.y >> 31)) d.used[r.y] = make_ulonglong2(0ull, 0ull);
            if (!(r.z >> 31)) d.used[r.z & 0x7FFFFFFFu] = make_ulonglong2(0ull, 0ull);
        }
        if (tid == 0)
        {
            rb_left = 0;
            rb_over = 0;
            rb_top = 0;
        }
        __syncthreads();
        for (int rr = 0;; ++rr)
        {
            for (int k = tid; k < na; k += nt)
                if (colour[k] < 0) tcol[k] = colour_rounds_pick(d, rec[k], &rb_over);
            __syncthreads();
            if (rb_over) break; // a body would need a colour above 127
            for (int k = tid; k < na; k += nt)
                if (colour[k] < 0) colour_rounds_claim(d, rec[k], ff_key(tcol[k], rec[k].w & 0xFFFFu, rec[k].w >> 16, uint32_t(k)));
            __syncthreads();
            int left = 0;
            for (int k = tid; k < na; k += nt)
            {
                if (colour[k] >= 0) continue;
                const int c = tcol[k];
                if (colour_rounds_commit(d, rec[k], ff_key(c, rec[k].w & 0xFFFFu, rec[k].w >> 16, uint32_t(k)), c))
                {
                    colour[k] = c;
                    atomicMax(&rb_top, c + 1);
                }
                else
                    ++left;
            }
            if (left) atomicAdd(&rb_left, left);
            __syncthreads();
            const int lft = rb_left;
            __syncthreads(); // every thread has read rb_left before it is reset
            if (lft == 0)
            {
                coloured = true;
                round = rb_top;
                break;
            }
            if (rr + 1 >= kMaxColours) break;
            if (tid == 0) rb_left = 0;
        }
        __syncthreads();
        if (!coloured)
        {
            for (int k = tid; k < na; k += nt) colour[k] = -1; // claiming rounds from scratch
            __syncthreads();
        }
    }
    while (!coloured && remaining > 0)
    {
        __syncthreads();
        for (int k = tid; k < na; k += nt)
        {
            if (colour[k] != -1) continue;
            const uint4 r = rec[k];
            if (!(r.y >> 31)) { if (sowner) sowner[r.w & 0xFFFFu] = ~0ull; else d.owner[r.y & 0x7FFFFFFFu] = ~0ull; }
            if (!(r.z >> 31)) { if (sowner) sowner[r.w >> 16] = ~0ull; else d.owner[r.z & 0x7FFFFFFFu] = ~0ull; }
        }
        if (tid == 0) remaining = 0;
        __syncthreads();
        for (int k = tid; k < na; k += nt)
        {
            if (colour[k] != -1) continue;
            const uint4 r = rec[k];
            const unsigned long long key = uint32_t(k);
            if (!(r.y >> 31)) { if (sowner) atomicMin(reinterpret_cast<unsigned long long *>(sowner + (r.w & 0xFFFFu)), key); else atomicMin(reinterpret_cast<unsigned long long *>(d.owner + (r.y & 0x7FFFFFFFu)), key); }
            if (!(r.z >> 31)) { if (sowner) atomicMin(reinterpret_cast<unsigned long long *>(sowner + (r.w >> 16)), key); else atomicMin(reinterpret_cast<unsigned long long *>(d.owner + (r.z & 0x7FFFFFFFu)), key); }
        }
        __syncthreads();
        int left = 0;
        for (int k = tid; k < na; k += nt)
        {
            if (colour[k] != -1) continue;
            const uint4 r = rec[k];
            const uint64_t key = uint32_t(k);
            bool oka = (r.y >> 31) || (sowner ? sowner[r.w & 0xFFFFu] : d.owner[r.y & 0x7FFFFFFFu]) == key;
            bool okb = (r.z >> 31) || (sowner ? sowner[r.w >> 16] : d.owner[r.z & 0x7FFFFFFFu]) == key;
            if (oka && okb)
                colour[k] = round;
            else
                ++left;
        }
        if (left) atomicAdd(&remaining, left);
        __syncthreads();
        ++round;
        if (round >= kMaxColours && remaining > 0)
        {
            if (tid == 0) atomicOr(d.status, ST_COLOUR_CAP);
            break;
        }
    }
    const int ncol = round;
    for (int k = tid; k < na; k += nt)
    {
        int c = colour[k];
        if (c >= 0 && c < kMaxColours) atomicAdd(&ccount[c], 1);
    }
    __syncthreads();
    if (tid == 0)
    {
        int s = 0;
        for (int c = 0; c < ncol; ++c)
        {
            cstart[c] = s;
            s += ccount[c];
        }
        d.ncolours[w] = ncol;
    }
    __syncthreads();
    for (int pass = 0; pass < 2; ++pass)
    {
        for (int k = tid; k < na; k += nt)
        {
            const uint4 r = rec[k];
            if (wide_manifold(d, r) != (pass == 0)) continue;
            int c = colour[k];
            if (c >= 0 && c < kMaxColours) d.srec[ms + cstart[c] + atomicAdd(&cursor[c], 1)] = r;
            d.pair_colour[r.x] = c; // per-pair colour for read-back (-2: no contact rows)
        }
        __syncthreads();
    }
    if (cache)
    {
        // the owner table is done; the shared memory now caches body velocities
        for (int k = tid; k < na; k += nt)
        {
            const uint4 r = rec[k];
            if (!(r.y >> 31)) cache[r.w & 0xFFFFu] = d.vel[r.y];
            if (!(r.z >> 31)) cache[r.w >> 16] = d.vel[r.z];
        }
        for (int j = js + tid; JOINTS && j < je; j += nt) // bodies of the world's joints
        {
            const JointDev<T> &jd = d.joints[j];
            if (!(d.meta[jd.a].flags & BODY_STATIC)) cache[jd.local_a] = d.vel[jd.a];
            if (!(d.meta[jd.b].flags & BODY_STATIC)) cache[jd.local_b] = d.vel[jd.b];
        }
    }
    __syncthreads();

    // 3. warm start, then the iterations, colour by colour. Each thread reads its first record of
    //    the next colour before it solves the current one, taking that load off the sweep's path.
    uint4 cur = make_uint4(0u, 0u, 0u, 0u);
    if (ncol > 0 && tid < ccount[0]) cur = d.srec[ms + cstart[0] + tid];
    for (int it = -1; it < d.iterations; ++it)
    {
        if (JOINTS && je > js)
        {
            if (tid == 0) solve_joints(d, js, je, cache, it < 0, false);
            __syncthreads();
        }
        for (int c = 0; c < ncol; ++c)
        {
            const int cs = ms + cstart[c], cn = ccount[c];
            const int nc = c + 1 < ncol ? c + 1 : 0;
            uint4 nxt = make_uint4(0u, 0u, 0u, 0u);
            if ((c + 1 < ncol || it + 1 < d.iterations) && tid < ccount[nc]) nxt = d.srec[ms + cstart[nc] + tid];
            for (int k = tid; k < cn; k += nt) solve_manifold_rec(d, k == tid ? cur : d.srec[cs + k], cache, it < 0);
            __syncthreads();
            cur = nxt;
        }
    }
    if (cache)
    {
        for (int k = tid; k < na; k += nt)
        {
            const uint4 r = rec[k];
            if (!(r.y >> 31)) d.vel[r.y] = cache[r.w & 0xFFFFu];
            if (!(r.z >> 31)) d.vel[r.z] = cache[r.w >> 16];
        }
        for (int j = js + tid; JOINTS && j < je; j += nt)
        {
            const JointDev<T> &jd = d.joints[j];
            if (!(d.meta[jd.a].flags & BODY_STATIC)) d.vel[jd.a] = cache[jd.local_a];
            if (!(d.meta[jd.b].flags & BODY_STATIC)) d.vel[jd.b] = cache[jd.local_b];
        }
    }
    // 4. write the accumulated impulses back into the manifold cache
    for (int k = tid; k < na; k += nt)
    {
        const int p = int(rec[k].x);
        const uint8_t mask = d.rowmask[p];
        for (int q = 0; q < 4; ++q)
        {
            if (!(mask & (1u << q))) continue;
            store_impulses(d, p, q);
        }
    }
}

template <class T, int MAXT, bool JOINTS>
__global__ void __launch_bounds__(MAXT, MAXT == 256 ? PK_SOLVE_MIN_BLOCKS : 1)
    k_solve_world(Dev<T> d, const uint64_t *__restrict__ sval, int first_block, int cache_bodies, int grid_world)
{
    extern __shared__ __align__(16) unsigned char solve_smem[];
    const int blk = first_block + int(blockIdx.x);
    if (blk >= d.max_worlds) return;
    const int w = d.world_order[blk];
    if (!d.wp[w].active || d.world_nlocal[w] > grid_world) return; // large worlds: k_solve_grid
    solve_world_cta<T, MAXT, JOINTS>(d, sval, w, cache_bodies, solve_smem);
}

// Solve groups: several small worlds per CTA (worlds world_order[goff[g]] .. [goff[g + 1] - 1] for
// group g, at most kGroupMax, their local indices together at most cache_bodies). Each member is
// compacted and coloured on its own, one warp per member, by the same first fit in pair order as a
// world alone; the sweeps then run colour c of every member together, or, in warp mode (at most
// one member per warp), each member's sweeps run on its own warp with warp barriers only. Members share no bodies, so
// each world gets its colours, its sweep order per body and its results exactly as alone, while the
// CTA's lanes hold the manifolds of several worlds. If a member needs more than 128 colours the
// group is solved member by member on the one-world path.
constexpr int kGroupMax = 8;
constexpr int kGroupColours = 128; // first fit's colours

#ifndef PK_GROUP_MIN_BLOCKS
#define PK_GROUP_MIN_BLOCKS 2
#endif
template <class T, bool WARP>
__global__ void __launch_bounds__(256, PK_GROUP_MIN_BLOCKS)
    k_solve_group(Dev<T> d, const uint64_t *__restrict__ sval, const int *__restrict__ goff, int cache_bodies)
{
    extern __shared__ __align__(16) unsigned char solve_smem[];
    __shared__ int gw[kGroupMax], gms[kGroupMax], gna[kGroupMax], gbase[kGroupMax], gncol[kGroupMax];
    __shared__ int ccount[kGroupMax][kGroupColours];
    __shared__ int cstart[kGroupMax][kGroupColours];
    __shared__ int cursor[kGroupMax][kGroupColours];
    __shared__ int cpre[kGroupColours][kGroupMax + 1];
    __shared__ int ng, ntotal, ncol, capped;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    if (tid == 0)
    {
        int n = 0, base = 0;
        for (int k = goff[blockIdx.x]; k < goff[blockIdx.x + 1] && n < kGroupMax; ++k)
        {
            const int w = d.world_order[k];
            if (!d.wp[w].active) continue;
            gw[n] = w;
            gms[n] = d.mstart[w];
            gbase[n] = base;
            base += d.world_nlocal[w];
            ++n;
        }
        ng = n;
        ntotal = base;
        capped = 0;
    }
    __syncthreads();
    const int G = ng;
    if (G == 0) return;
    if (ntotal > cache_bodies)
    {
        // the host packs groups within cache_bodies from the same local-index counts; a group
        // beyond it has no room for its colour masks and is flagged, not solved
        if (tid == 0) atomicOr(d.status, ST_COLOUR_CAP);
        return;
    }

    // 1. per member, one warp: the manifolds with contact rows, ascending pair index; then first fit
    for (int g = warp; g < G; g += nw)
    {
        const int w = gw[g], ms = gms[g], me = d.mend[w];
        uint4 *rec = d.crec + ms;
        int off = 0;
        for (int p0 = ms; p0 < me; p0 += 32)
        {
            const int p = p0 + lane;
            const bool on = p < me && d.rowmask[p] != 0;
            const unsigned m = __ballot_sync(0xFFFFFFFFu, on);
            if (on) rec[off + __popc(m & ((1u << lane) - 1u))] = make_solve_rec(d, p, sval[p]);
            off += __popc(m);
        }
        uint64_t *used = reinterpret_cast<uint64_t *>(solve_smem) + 2 * gbase[g];
        for (int l = lane; l < 2 * d.world_nlocal[w]; l += 32) used[l] = 0ull;
        __syncwarp();
        if (lane == 0)
        {
            gna[g] = off;
            const int c = first_fit_colours(rec, off, used, d.colour_tmp + ms);
            gncol[g] = c;
            if (c < 0) capped = 1;
        }
        __syncwarp();
    }
    __syncthreads();
    if (capped)
    {
        for (int g = 0; g < G; ++g) solve_world_cta<T, 256, false>(d, sval, gw[g], cache_bodies, solve_smem);
        return;
    }

    if constexpr (WARP)
    {
        // warp mode (the host packs at most one member per warp): from here on each member is
        // solved by its own warp, with __syncwarp between its colours and no CTA-wide barrier
        Vel<T> *cache = reinterpret_cast<Vel<T> *>(solve_smem);
        for (int g = warp; g < G; g += nw)
        {
            const int ms = gms[g], na = gna[g], ncg = gncol[g];
            const int *colour = d.colour_tmp + ms;
            const uint4 *rec = d.crec + ms;
            for (int c = lane; c < ncg; c += 32)
            {
                ccount[g][c] = 0;
                cursor[g][c] = 0;
            }
            __syncwarp();
            for (int k = lane; k < na; k += 32) atomicAdd(&ccount[g][colour[k]], 1);
            __syncwarp();
            if (lane == 0)
            {
                int s = 0;
                for (int c = 0; c < ncg; ++c)
                {
                    cstart[g][c] = s;
                    s += ccount[g][c];
                }
                d.ncolours[gw[g]] = ncg;
            }
            __syncwarp();
            Vel<T> *cg = cache + gbase[g];
            for (int pass = 0; pass < 2; ++pass)
            {
                for (int k = lane; k < na; k += 32)
                {
                    const uint4 r = rec[k];
                    if (wide_manifold(d, r) != (pass == 0)) continue;
                    const int c = colour[k];
                    d.srec[ms + cstart[g][c] + atomicAdd(&cursor[g][c], 1)] = r;
                    d.pair_colour[r.x] = c; // per-pair colour for read-back
                    if (!(r.y >> 31)) cg[r.w & 0xFFFFu] = d.vel[r.y];
                    if (!(r.z >> 31)) cg[r.w >> 16] = d.vel[r.z];
                }
                __syncwarp();
            }
            for (int it = -1; it < d.iterations; ++it)
                for (int c = 0; c < ncg; ++c)
                {
                    const int cs = ms + cstart[g][c], cn = ccount[g][c];
                    for (int i = lane; i < cn; i += 32) solve_manifold_rec(d, d.srec[cs + i], cg, it < 0);
                    __syncwarp();
                }
            for (int k = lane; k < na; k += 32)
            {
                const uint4 r = rec[k];
                if (!(r.y >> 31)) d.vel[r.y] = cg[r.w & 0xFFFFu];
                if (!(r.z >> 31)) d.vel[r.z] = cg[r.w >> 16];
                const int p = int(r.x);
                const uint8_t mask = d.rowmask[p];
                for (int q = 0; q < 4; ++q)
                    if (mask & (1u << q)) store_impulses(d, p, q);
            }
        }
        return;
    }

    // 2. each member's colours laid out in order (srec), and per colour the members' prefix counts
    for (int i = tid; i < kGroupMax * kGroupColours; i += nt)
    {
        (&ccount[0][0])[i] = 0;
        (&cursor[0][0])[i] = 0;
    }
    __syncthreads();
    for (int g = 0; g < G; ++g)
    {
        const int *colour = d.colour_tmp + gms[g];
        for (int k = tid; k < gna[g]; k += nt) atomicAdd(&ccount[g][colour[k]], 1);
    }
    __syncthreads();
    if (tid < G)
    {
        int s = 0;
        for (int c = 0; c < gncol[tid]; ++c)
        {
            cstart[tid][c] = s;
            s += ccount[tid][c];
        }
        d.ncolours[gw[tid]] = gncol[tid];
    }
    if (tid == 0)
    {
        int m = 0;
        for (int g = 0; g < G; ++g) m = gncol[g] > m ? gncol[g] : m;
        ncol = m;
    }
    __syncthreads();
    const int nc = ncol;
    for (int c = tid; c < nc; c += nt)
    {
        int s = 0;
        for (int g = 0; g < G; ++g)
        {
            cpre[c][g] = s;
            s += ccount[g][c];
        }
        cpre[c][G] = s;
    }
    for (int pass = 0; pass < 2; ++pass)
    {
        for (int g = 0; g < G; ++g)
        {
            const int ms = gms[g];
            const int *colour = d.colour_tmp + ms;
            const uint4 *rec = d.crec + ms;
            for (int k = tid; k < gna[g]; k += nt)
            {
                const uint4 r = rec[k];
                if (wide_manifold(d, r) != (pass == 0)) continue;
                const int c = colour[k];
                d.srec[ms + cstart[g][c] + atomicAdd(&cursor[g][c], 1)] = r;
                d.pair_colour[r.x] = c; // per-pair colour for read-back
            }
        }
        __syncthreads();
    }
    // the colour masks are done; the shared memory now caches the members' body velocities
    Vel<T> *cache = reinterpret_cast<Vel<T> *>(solve_smem);
    __syncthreads();
    for (int g = 0; g < G; ++g)
    {
        const uint4 *rec = d.crec + gms[g];
        Vel<T> *cg = cache + gbase[g];
        for (int k = tid; k < gna[g]; k += nt)
        {
            const uint4 r = rec[k];
            if (!(r.y >> 31)) cg[r.w & 0xFFFFu] = d.vel[r.y];
            if (!(r.z >> 31)) cg[r.w >> 16] = d.vel[r.z];
        }
    }
    __syncthreads();

    // 3. warm start, then the iterations: colour c of every member in one sweep
    for (int it = -1; it < d.iterations; ++it)
        for (int c = 0; c < nc; ++c)
        {
            const int n = cpre[c][G];
            for (int i = tid; i < n; i += nt)
            {
                int g = 0;
                while (g + 1 < G && i >= cpre[c][g + 1]) ++g;
                const uint4 r = d.srec[gms[g] + cstart[g][c] + (i - cpre[c][g])];
                solve_manifold_rec(d, r, cache + gbase[g], it < 0);
            }
            __syncthreads();
        }

    // 4. velocities back to the bodies, accumulated impulses back into the manifold cache
    for (int g = 0; g < G; ++g)
    {
        const uint4 *rec = d.crec + gms[g];
        const Vel<T> *cg = cache + gbase[g];
        for (int k = tid; k < gna[g]; k += nt)
        {
            const uint4 r = rec[k];
            if (!(r.y >> 31)) d.vel[r.y] = cg[r.w & 0xFFFFu];
            if (!(r.z >> 31)) d.vel[r.z] = cg[r.w >> 16];
            const int p = int(r.x);
            const uint8_t mask = d.rowmask[p];
            for (int q = 0; q < 4; ++q)
                if (mask & (1u << q)) store_impulses(d, p, q);
        }
    }
}

// The same colouring and colour-ordered sweeps for one world too large for a CTA: every block of a
// cooperative launch takes part, and grid-wide barriers separate the phases. The keys of the
// parallel first fit and the claim priority of the fallback use the pair index (monotone in the
// compacted index the CTA solver uses), so the colours are the same as the CTA solver's and the
// oracle's.
struct GridScratch
{
    int ccount[kMaxColours];
    int cstart[kMaxColours];
    int cursor[kMaxColours];
    int left[2];
    int ncol;
    int ff_left, ff_over, ff_top; // rounds of parallel first fit
    int nact;                     // the world's pairs with contact rows
};

template <class T>
__global__ void __launch_bounds__(256) k_solve_grid(Dev<T> d, const uint64_t *__restrict__ sval, int w, GridScratch *g)
{
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    if (!d.wp[w].active) return;
    const int ms = d.mstart[w], me = d.mend[w];
    const int js = d.jstart[w], je = d.jend[w];
    const int gtid = int(grid.thread_rank()), gn = int(grid.size());
    if (me <= ms && je <= js)
    {
        if (gtid == 0) d.ncolours[w] = 0;
        return;
    }
    // the world's pairs with contact rows, compacted once (in any order: colours depend on the
    // keys only, and manifolds of one colour are solved in any order); the colouring rounds and
    // the orderings below run over this list instead of all of the world's pairs
    int *colour = d.colour_tmp;
    int *alist = d.colour + ms;
    for (int c = gtid; c < kMaxColours; c += gn) g->ccount[c] = g->cursor[c] = 0;
    if (gtid == 0)
    {
        g->left[0] = 1; // any value > 0: first round runs
        g->left[1] = 0;
        g->nact = 0;
    }
    grid.sync();
    for (int p = ms + gtid; p < me; p += gn)
    {
        const bool act = d.rowmask[p] != 0;
        colour[p] = act ? -1 : -2;
        d.pair_colour[p] = -2;
        if (act) alist[warp_push(&g->nact)] = p;
    }
    grid.sync();
    const int na = *((volatile int *)&g->nact);
    int round = 0;
    int active_left = 1;
    // rounds of parallel first fit (as the CTA solver for worlds above kFirstFitMax local indices),
    // keyed by the bodies' full local indices; claiming rounds if a body would need a colour above 127
    {
        int *tcol = reinterpret_cast<int *>(d.order); // free until the colour-ordered list is built
        auto rec_of = [&](int p) {
            const uint64_t v = sval[p];
            const uint32_t a = uint32_t(v >> 32), b = uint32_t(v & 0xFFFFFFFFu);
            return make_uint4(uint32_t(p), a | ((d.meta[a].flags & BODY_STATIC) ? 0x80000000u : 0u),
                              b | ((d.meta[b].flags & BODY_STATIC) ? 0x80000000u : 0u), 0u);
        };
        auto key_of = [&](int p, int c) {
            const uint64_t v = sval[p];
            return ff_key(c, d.meta[uint32_t(v >> 32)].local, d.meta[uint32_t(v & 0xFFFFFFFFu)].local, uint32_t(p));
        };
        for (int k = gtid; k < na; k += gn)
        {
            const uint4 r = rec_of(alist[k]);
            if (!(r.y >> 31)) d.used[r.y] = make_ulonglong2(0ull, 0ull);
            if (!(r.z >> 31)) d.used[r.z & 0x7FFFFFFFu] = make_ulonglong2(0ull, 0ull);
        }
        if (gtid == 0)
        {
            g->ff_left = 0;
            g->ff_over = 0;
            g->ff_top = 0;
        }
        grid.sync();
        bool coloured = false;
        for (int rr = 0;; ++rr)
        {
            for (int k = gtid; k < na; k += gn)
            {
                const int p = alist[k];
                if (colour[p] == -1) tcol[p] = colour_rounds_pick(d, rec_of(p), &g->ff_over);
            }
            grid.sync();
            if (*((volatile int *)&g->ff_over)) break;
            for (int k = gtid; k < na; k += gn)
            {
                const int p = alist[k];
                if (colour[p] == -1) colour_rounds_claim(d, rec_of(p), key_of(p, tcol[p]));
            }
            grid.sync();
            int left = 0;
            for (int k = gtid; k < na; k += gn)
            {
                const int p = alist[k];
                if (colour[p] != -1) continue;
                const int c = tcol[p];
                if (colour_rounds_commit(d, rec_of(p), key_of(p, c), c))
                {
                    colour[p] = c;
                    atomicMax(&g->ff_top, c + 1);
                }
                else
                    ++left;
            }
            if (left) atomicAdd(&g->ff_left, left);
            grid.sync();
            const int lft = *((volatile int *)&g->ff_left);
            grid.sync(); // every thread has read ff_left before it is reset
            if (lft == 0)
            {
                coloured = true;
                break;
            }
            if (rr + 1 >= kMaxColours) break;
            if (gtid == 0) g->ff_left = 0;
        }
        if (coloured)
        {
            round = *((volatile int *)&g->ff_top);
            active_left = 0; // the claiming rounds below do not run
        }
        else
        {
            for (int k = gtid; k < na; k += gn) colour[alist[k]] = -1; // claiming rounds from scratch
            grid.sync();
        }
    }
    while (active_left > 0)
    {
        int *cnt = &g->left[round & 1];
        for (int k = gtid; k < na; k += gn)
        {
            const int p = alist[k];
            if (colour[p] != -1) continue;
            uint64_t v = sval[p];
            int a = int(v >> 32), b = int(v & 0xFFFFFFFFu);
            if (!(d.meta[a].flags & BODY_STATIC)) d.owner[a] = ~0ull;
            if (!(d.meta[b].flags & BODY_STATIC)) d.owner[b] = ~0ull;
        }
        if (gtid == 0) *cnt = 0;
        grid.sync();
        for (int k = gtid; k < na; k += gn)
        {
            const int p = alist[k];
            if (colour[p] != -1) continue;
            uint64_t v = sval[p];
            int a = int(v >> 32), b = int(v & 0xFFFFFFFFu);
            if (!(d.meta[a].flags & BODY_STATIC)) atomicMin(reinterpret_cast<unsigned long long *>(d.owner + a), (unsigned long long)uint32_t(p));
            if (!(d.meta[b].flags & BODY_STATIC)) atomicMin(reinterpret_cast<unsigned long long *>(d.owner + b), (unsigned long long)uint32_t(p));
        }
        grid.sync();
        int left = 0;
        for (int k = gtid; k < na; k += gn)
        {
            const int p = alist[k];
            if (colour[p] != -1) continue;
            uint64_t v = sval[p];
            int a = int(v >> 32), b = int(v & 0xFFFFFFFFu);
            bool oka = (d.meta[a].flags & BODY_STATIC) || __ldcg(reinterpret_cast<const unsigned long long *>(d.owner + a)) == uint64_t(uint32_t(p));
            bool okb = (d.meta[b].flags & BODY_STATIC) || __ldcg(reinterpret_cast<const unsigned long long *>(d.owner + b)) == uint64_t(uint32_t(p));
            if (oka && okb)
                colour[p] = round;
            else
                ++left;
        }
        if (left) atomicAdd(cnt, left);
        grid.sync();
        active_left = *((volatile int *)cnt);
        ++round;
        if (round >= kMaxColours && active_left > 0)
        {
            if (gtid == 0) atomicOr(d.status, ST_COLOUR_CAP);
            break;
        }
    }
    const int ncol_guess = round;
    for (int k = gtid; k < na; k += gn)
    {
        int c = colour[alist[k]];
        if (c >= 0 && c < kMaxColours) atomicAdd(&g->ccount[c], 1);
    }
    grid.sync();
    if (gtid == 0)
    {
        int s = 0, nc = 0;
        for (int c = 0; c < ncol_guess; ++c)
        {
            g->cstart[c] = s;
            s += g->ccount[c];
            if (g->ccount[c] > 0) nc = c + 1;
        }
        g->ncol = nc;
        d.ncolours[w] = nc;
    }
    grid.sync();
    const int ncol = *((volatile int *)&g->ncol);
    for (int k = gtid; k < na; k += gn)
    {
        const int p = alist[k];
        int c = colour[p];
        if (c >= 0 && c < kMaxColours) d.order[ms + __ldcg(&g->cstart[c]) + atomicAdd(&g->cursor[c], 1)] = uint32_t(p);
        d.pair_colour[p] = c >= 0 ? c : -2;
    }
    grid.sync();
    for (int it = -1; it < d.iterations; ++it)
    {
        if (je > js)
        {
            if (gtid == 0) solve_joints(d, js, je, (Vel<T> *)nullptr, it < 0, true);
            grid.sync();
        }
        for (int c = 0; c < ncol; ++c)
        {
            const int cs = ms + __ldcg(&g->cstart[c]), cn = __ldcg(&g->ccount[c]);
            for (int k = gtid; k < cn; k += gn)
            {
                int p = int(__ldcg(d.order + cs + k));
                solve_manifold(d, p, sval[p], (Vel<T> *)nullptr, it < 0, true);
            }
            grid.sync();
        }
    }
    for (int k = gtid; k < na; k += gn)
    {
        const int p = alist[k];
        uint8_t mask = d.rowmask[p];
        for (int q = 0; q < 4; ++q)
        {
            if (!(mask & (1u << q))) continue;
            store_impulses(d, p, q);
        }
    }
}

// ------------------------------------------------------------------------------------------------
// position integration + cached inertia (integrate.h:20-46, particle.h:140-146)
// ------------------------------------------------------------------------------------------------
template <class T> __global__ void k_integrate_pos(Dev<T> d, T dt)
{
    const int n = *d.nslots;
    PK_GRID_STRIDE(i, n)
    {
        Meta m = d.meta[i];
        if (!(m.flags & BODY_ALIVE) || (m.flags & BODY_STATIC) || !d.wp[m.world].active) continue;
        Pose<T> ps = d.pose[i];
        Vel<T> ve = d.vel[i];
        V3<T> v = ld3(ve.v), w = ld3(ve.w);
        V3<T> x = ld3(ps.p) + v * dt;
        V3<T> ang = w * dt;
        T mag = norm(ang);
        Qt<T> dq;
        if (mag < T(1e-12))
        {
            V3<T> h = ang * T(0.5);
            dq = qnormalized(Qt<T>{T(1), h.x, h.y, h.z});
        }
        else
        {
            V3<T> ax = ang / mag;
            T s, c;
            sincos_det(T(0.5) * mag, &s, &c);
            dq = Qt<T>{c, s * ax.x, s * ax.y, s * ax.z};
        }
        Qt<T> q = qmul(dq, ldq(ps.q));
        st3(ps.p, x);
        ps.q[0] = q.w;
        ps.q[1] = q.x;
        ps.q[2] = q.y;
        ps.q[3] = q.z;
        d.pose[i] = ps;
        M3<T> R = to_matrix(q), Rt = transpose(R);
        M3<T> il, ili;
        for (int k = 0; k < 9; ++k)
        {
            il.m[k] = d.prm[i].il[k];
            ili.m[k] = d.prm[i].il_inv[k];
        }
        M3<T> iw = matmul(matmul(R, il), Rt);
        M3<T> iwi = matmul(matmul(R, ili), Rt);
        bool bad = false;
        for (int k = 0; k < 9; ++k)
        {
            d.iw[9 * i + k] = iw.m[k];
            d.iwinv[9 * i + k] = iwi.m[k];
        }
        if (!(x.x == x.x) || !(x.y == x.y) || !(x.z == x.z)) bad = true;
        if (bad) atomicOr(d.status, ST_NAN);
    }
}

// Pair assembly. The sorted new pairs cover the active worlds only; each world that sits out the
// step keeps last step's pair segment (and, through it, its manifolds and warm-start impulses), so
// its trajectory does not depend on which steps it skipped. Pair keys are world-major, so the step's
// full sorted list is the concatenation, world by world, of one of the two segments.
template <class T> __global__ void k_pair_bounds(Dev<T> d, const uint64_t *__restrict__ skey)
{
    const int n = *d.nnew;
    PK_GRID_STRIDE(p, n)
    {
        int w = int(skey[p] >> (2 * d.lbits));
        if (p == 0 || int(skey[p - 1] >> (2 * d.lbits)) != w) d.nstart[w] = p;
        if (p == n - 1 || int(skey[p + 1] >> (2 * d.lbits)) != w) d.nend[w] = p + 1;
    }
}

// Kept pairs of an idle world: last step's segment minus pairs of bodies removed since (their
// manifolds were already emptied by the removal). One CTA per world.
template <class T> __device__ __forceinline__ bool kept_pair(const Dev<T> &d, int p)
{
    uint64_t v = d.val_old[p];
    return (d.meta[int(v >> 32)].flags & BODY_ALIVE) && (d.meta[int(v & 0xFFFFFFFFu)].flags & BODY_ALIVE);
}

template <class T> __global__ void __launch_bounds__(256) k_kept_count(Dev<T> d)
{
    __shared__ int warp_sum[8];
    const int w = blockIdx.x;
    if (d.wp[w].active) return;
    const int a = d.mstart_old[w], b = d.mend_old[w];
    if (a >= b) return;
    int c = 0;
    for (int p = a + threadIdx.x; p < b; p += blockDim.x) c += kept_pair(d, p);
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int t = 0;
        for (int k = 0; k < int(blockDim.x >> 5); ++k) t += warp_sum[k];
        d.nend[w] = t;
    }
}

// One CTA: segment length of every world, exclusive scan -> the world's range in the assembled list.
template <class T> __global__ void __launch_bounds__(1024) k_pair_segments(Dev<T> d)
{
    __shared__ int part[1024];
    const int W = d.max_worlds;
    const int per = (W + 1023) / 1024;
    const int lo = min(W, int(threadIdx.x) * per), hi = min(W, lo + per);
    int s = 0;
    for (int w = lo; w < hi; ++w) s += d.nend[w] - d.nstart[w];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1)
    {
        int v = int(threadIdx.x) >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (int w = lo; w < hi; ++w)
    {
        int len = d.nend[w] - d.nstart[w];
        d.mstart[w] = min(run, d.pair_cap);
        d.mend[w] = min(run + len, d.pair_cap);
        run += len;
    }
    if (threadIdx.x == 1023)
    {
        if (run > d.pair_cap) atomicOr(d.status, ST_PAIR_OVERFLOW);
        *d.npairs = min(run, d.pair_cap);
    }
}

template <class T>
__global__ void k_assemble_new(Dev<T> d, const uint64_t *__restrict__ skey, const uint64_t *__restrict__ sval,
                               uint64_t *__restrict__ akey, uint64_t *__restrict__ aval)
{
    const int n = *d.nnew;
    PK_GRID_STRIDE(p, n)
    {
        uint64_t key = skey[p];
        int w = int(key >> (2 * d.lbits));
        int q = d.mstart[w] + (p - d.nstart[w]);
        if (q < d.mend[w])
        {
            akey[q] = key;
            aval[q] = sval[p];
        }
    }
}

// Order-preserving compaction of each idle world's kept pairs into its assembled range.
template <class T> __global__ void __launch_bounds__(256) k_assemble_kept(Dev<T> d, uint64_t *__restrict__ akey,
                                                                        uint64_t *__restrict__ aval)
{
    __shared__ int warp_cnt[8];
    const int w = blockIdx.x;
    if (d.wp[w].active) return;
    const int a = d.mstart_old[w], b = d.mend_old[w];
    const int out0 = d.mstart[w], out1 = d.mend[w];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int base = out0;
    for (int c = a; c < b; c += blockDim.x)
    {
        int p = c + threadIdx.x;
        bool keep = p < b && kept_pair(d, p);
        unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
        if (lane == 0) warp_cnt[wid] = __popc(m);
        __syncthreads();
        int off = 0, tot = 0;
        for (int k = 0; k < nw; ++k)
        {
            off += k < wid ? warp_cnt[k] : 0;
            tot += warp_cnt[k];
        }
        int q = base + off + __popc(m & ((1u << lane) - 1u));
        if (keep && q < out1)
        {
            akey[q] = d.key_old[p];
            aval[q] = d.val_old[p];
            d.old_idx[q] = p;
        }
        base += tot;
        __syncthreads();
    }
}

// Retiring a world: every cached manifold of its pairs becomes empty.
template <class T> __global__ void k_purge_world(Dev<T> d, uint32_t world)
{
    const int n = *d.npairs_old;
    PK_GRID_STRIDE(p, n)
    {
        if (uint32_t(d.key_old[p] >> (2 * d.lbits)) == world) d.man_old[p].n = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) d.mend_old[world] = d.mstart_old[world]; // nothing to keep
}

template <class T> __global__ void k_kill_bodies(Dev<T> d, const int *slots, int n)
{
    PK_GRID_STRIDE(i, n) d.meta[slots[i]].flags = 0;
}

template <class T> __global__ void k_set_active(Dev<T> d, const uint8_t *mask, int n)
{
    PK_GRID_STRIDE(w, n) d.wp[w].active = mask[w] ? 1 : 0;
}

template <class T> __global__ void k_finish(Dev<T> d, const uint64_t *__restrict__ skey, const uint64_t *__restrict__ sval)
{
    const int np = *d.npairs;
    PK_GRID_STRIDE(p, np)
    {
        d.key_old[p] = skey[p];
        d.val_old[p] = sval[p];
    }
    PK_GRID_STRIDE(w, d.max_worlds)
    {
        d.mstart_old[w] = d.mstart[w];
        d.mend_old[w] = d.mend[w];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d.npairs_old = np;
}

// Removal of a body invalidates the cached manifolds of its pairs (collision_phases.h:38-52).
template <class T> __global__ void k_purge_pairs(Dev<T> d, uint32_t world, uint32_t local)
{
    const int n = *d.npairs_old;
    const uint64_t mask = (uint64_t(1) << d.lbits) - 1;
    PK_GRID_STRIDE(p, n)
    {
        uint64_t k = d.key_old[p];
        uint32_t w = uint32_t(k >> (2 * d.lbits));
        uint32_t lo = uint32_t((k >> d.lbits) & mask), hi = uint32_t(k & mask);
        if (w == world && (lo == local || hi == local)) d.man_old[p].n = 0;
    }
}

// Rays against mesh instances (mesh::instance::ray_intersect, mesh.cpp:400-415): one thread per
// ray. The ray is moved into the body frame and its direction normalised again (the ray
// constructor, bvh.h:47-50); every triangle is tested in index order by Moeller-Trumbore
// (ray::intersect, bvh.h:97-135) with the running best distance as its limit, so a later triangle
// at the same distance replaces an earlier one; the hit goes back to world space.
template <class T>
__global__ void k_mesh_raycast(Dev<T> d, const int *__restrict__ tris, const int2 *__restrict__ trange,
                               const MeshRayIn *__restrict__ rays, int n, MeshHitOut *__restrict__ out)
{
    PK_GRID_STRIDE(i, n)
    {
        const MeshRayIn r = rays[i];
        int shape = r.shape;
        V3<T> P{T(r.pos[0]), T(r.pos[1]), T(r.pos[2])};
        Qt<T> q{T(r.q[0]), T(r.q[1]), T(r.q[2]), T(r.q[3])};
        if (r.slot >= 0)
        {
            shape = int(d.meta[r.slot].shape);
            P = ld3(d.pose[r.slot].p);
            q = ldq(d.pose[r.slot].q);
        }
        const V3<T> dw = normalized(V3<T>{T(r.d[0]), T(r.d[1]), T(r.d[2])});
        const V3<T> ow{T(r.o[0]), T(r.o[1]), T(r.o[2])};
        const Qt<T> iq = conj(q);
        const V3<T> o = rotate(iq, ow - P);
        const V3<T> dl = normalized(rotate(iq, dw));
        const T *vb = d.verts + 3 * d.shape_range[shape].vstart;
        const int2 tr = trange[shape];
        T best = T(r.maxd);
        int best_tri = -1;
        V3<T> e1b{}, e2b{};
        for (int k = 0; k < tr.y; ++k)
        {
            const int *t = tris + 3 * (tr.x + k);
            const V3<T> v0 = ld3(vb + 3 * t[0]), v1 = ld3(vb + 3 * t[1]), v2 = ld3(vb + 3 * t[2]);
            const V3<T> e1 = v1 - v0, e2 = v2 - v0;
            const V3<T> h = cross(dl, e2);
            const T a = dot(e1, h);
            if (a > T(-1e-12) && a < T(1e-12)) continue;
            const T f = T(1) / a;
            const V3<T> sv = o - v0;
            const T u = f * dot(sv, h);
            if (u < T(0) || u > T(1)) continue;
            const V3<T> qv = cross(sv, e1);
            const T v = f * dot(dl, qv);
            if (v < T(0) || u + v > T(1)) continue;
            const T tt = f * dot(e2, qv);
            if (tt < T(0) || tt > best) continue;
            best = tt;
            best_tri = k;
            e1b = e1;
            e2b = e2;
        }
        MeshHitOut h{};
        h.hit = best_tri >= 0;
        h.triangle = best_tri;
        if (best_tri >= 0)
        {
            const V3<T> pl = o + dl * best;
            const V3<T> pw = rotate(q, pl) + P;
            const V3<T> nw = rotate(q, normalized(cross(e1b, e2b)));
            h.pos[0] = double(pw.x);
            h.pos[1] = double(pw.y);
            h.pos[2] = double(pw.z);
            h.normal[0] = double(nw.x);
            h.normal[1] = double(nw.y);
            h.normal[2] = double(nw.z);
            h.distance = double(best);
        }
        out[i] = h;
    }
}

// Standalone narrowphase over primitive shape pairs (known-answer checks of collision.cpp).
struct ShapeSpec
{
    int kind;  // SHAPE_AABB / SHAPE_OBB / SHAPE_MESH
    int shape; // mesh shape id
    double p[10];
};
template <class T> __global__ void k_collide_batch(const ShapeSpec *sa, const ShapeSpec *sb, int n, const T *verts,
                                                   const ShapeRange *ranges, const T *clusters, const T *rmax,
                                                   double *out, int *hit, int *status, int *status_any)
{
    PK_GRID_STRIDE(i, n)
    {
        ShapeRef<T> s[2];
        const ShapeSpec *sp[2] = {sa + i, sb + i};
        for (int k = 0; k < 2; ++k)
        {
            const ShapeSpec &q = *sp[k];
            ShapeRef<T> &r = s[k];
            r.kind = q.kind;
            r.nverts = 0;
            r.verts = nullptr;
            r.ncl = 0;
            r.cl = nullptr;
            r.ngr = 0;
            r.gr = nullptr;
            r.rmax = T(0);
            r.uv_stacks = r.uv_sectors = 0;
            r.q = Qt<T>{T(1), T(0), T(0), T(0)};
            r.pos = r.a = r.b = V3<T>{T(0), T(0), T(0)};
            if (q.kind == SHAPE_AABB)
            {
                r.a = V3<T>{T(q.p[0]), T(q.p[1]), T(q.p[2])};
                r.b = V3<T>{T(q.p[3]), T(q.p[4]), T(q.p[5])};
            }
            else if (q.kind == SHAPE_OBB)
            {
                r.pos = V3<T>{T(q.p[0]), T(q.p[1]), T(q.p[2])};
                r.q = Qt<T>{T(q.p[3]), T(q.p[4]), T(q.p[5]), T(q.p[6])};
                r.b = V3<T>{T(q.p[7]), T(q.p[8]), T(q.p[9])};
            }
            else
            {
                r.pos = V3<T>{T(q.p[0]), T(q.p[1]), T(q.p[2])};
                r.q = Qt<T>{T(q.p[3]), T(q.p[4]), T(q.p[5]), T(q.p[6])};
                const ShapeRange rg = ranges[q.shape];
                r.verts = verts + 3 * rg.vstart;
                r.nverts = rg.nverts;
                r.ncl = rg.ncl;
                r.cl = clusters + 4 * rg.cstart;
                r.ngr = rg.ngr;
                r.gr = clusters + 4 * rg.gstart;
                r.rmax = rmax[q.shape];
                r.uv_stacks = rg.uv_stacks;
                r.uv_sectors = rg.uv_sectors;
            }
        }
        EpaState<T> es;
        Collision<T> c;
        int st = 0;
        bool h = gjk_epa(s[0], s[1], es, c, &st);
        hit[i] = h ? 1 : 0;
        status[i] = st;
        if (st && status_any) atomicOr(status_any, st); // a capacity of this implementation was hit
        double *o = out + 10 * i;
        if (h)
        {
            o[0] = double(c.normal.x);
            o[1] = double(c.normal.y);
            o[2] = double(c.normal.z);
            o[3] = double(c.world_a.x);
            o[4] = double(c.world_a.y);
            o[5] = double(c.world_a.z);
            o[6] = double(c.world_b.x);
            o[7] = double(c.world_b.y);
            o[8] = double(c.world_b.z);
            o[9] = double(c.depth);
        }
    }
}

} // namespace pk
