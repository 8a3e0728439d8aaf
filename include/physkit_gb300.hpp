/*
 * physkit_gb300.hpp — C++20 facade over the C ABI (physkit_gb300.h), shaped like the reference's
 * own world API so that code written against it reads the same:
 *
 *   world_desc   (include/physkit/core/world.h:23-49)    make(), with_gravity, with_solver_iterations
 *   object_desc  (include/physkit/core/object.h:15-109)  dynam(), stat(), with_pos / vel / mass /
 *                orientation / ang_vel / inertia_tensor / mesh / restitution / friction
 *   world        (world.h:188-242, 379-425)              create_rigid, remove_rigid, get_rigid, step
 *   mesh         (include/physkit/collision/mesh.h:219-236)  box, sphere, pyramid, make; shared by
 *                the bodies that use it (object.h:61-65)
 *
 * Differences, by design: quantities are plain doubles in SI units (no mp-units); meshes belong to
 * the world they were made in; get_rigid returns a copy of the body's state (the state lives on the
 * GPU) instead of a pointer into the world; remove_rigid returns whether the handle was live.
 * Errors follow the reference's conventions: invalid input throws std::invalid_argument
 * (object.h:121), a stale handle gives std::nullopt (arena.h:89-108), and a failure of the device
 * path throws physkit_gb300::error with the C ABI's status code. Header only; link
 * libphyskit_gb300.so.
 */
#ifndef PHYSKIT_GB300_HPP
#define PHYSKIT_GB300_HPP

#include "physkit_gb300.h"

#include <array>
#include <cstdint>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace physkit_gb300
{

struct vec3
{
    double x = 0.0, y = 0.0, z = 0.0;
};
struct quat /* w first, like the reference's quat constructor (lin_alg.h:428-432) */
{
    double w = 1.0, x = 0.0, y = 0.0, z = 0.0;
    static constexpr quat identity() { return {}; }
};
using mat3 = std::array<double, 9>; /* row-major */
constexpr mat3 identity3() { return {1, 0, 0, 0, 1, 0, 0, 0, 1}; }

enum class precision : int32_t
{
    f64 = PK_PRECISION_F64, /* the reference's arithmetic, bit-identical to the FP64 oracle */
    f32 = PK_PRECISION_F32
};
enum class body_type : int32_t
{
    dynam = PK_BODY_DYNAMIC,
    stat = PK_BODY_STATIC
};

/* A failed call of the device path: code is the C ABI status (PK_ERR_*). */
class error : public std::runtime_error
{
public:
    error(const std::string &what, int code) : std::runtime_error(what + " (status " + std::to_string(code) + ")"), M_code(code) {}
    [[nodiscard]] int code() const { return M_code; }

private:
    int M_code;
};

namespace detail
{
inline void check(int rc, const char *what)
{
    if (rc == PK_OK) return;
    if (rc == PK_ERR_INVALID) throw std::invalid_argument(std::string(what) + ": invalid argument");
    throw error(what, rc);
}
} // namespace detail

class world_desc
{
public:
    static world_desc make() { return {}; }

    [[nodiscard]] vec3 gravity() const { return M_gravity; }
    world_desc &with_gravity(const vec3 &g) &
    {
        M_gravity = g;
        return *this;
    }
    world_desc &&with_gravity(const vec3 &g) && { return std::move(with_gravity(g)); }

    [[nodiscard]] std::size_t solver_iterations() const { return M_iterations; }
    world_desc &with_solver_iterations(std::size_t n) &
    {
        M_iterations = n;
        return *this;
    }
    world_desc &&with_solver_iterations(std::size_t n) && { return std::move(with_solver_iterations(n)); }

    /* device-side choices of this implementation (no counterpart in the reference) */
    world_desc &with_precision(precision p) &
    {
        M_precision = p;
        return *this;
    }
    world_desc &&with_precision(precision p) && { return std::move(with_precision(p)); }
    world_desc &with_capacity(int32_t max_bodies, int32_t max_pairs = 0, int32_t max_worlds = 1) &
    {
        M_max_bodies = max_bodies;
        M_max_pairs = max_pairs;
        M_max_worlds = max_worlds;
        return *this;
    }
    world_desc &&with_capacity(int32_t max_bodies, int32_t max_pairs = 0, int32_t max_worlds = 1) &&
    { return std::move(with_capacity(max_bodies, max_pairs, max_worlds)); }

    [[nodiscard]] pk_world_desc to_c() const
    {
        pk_world_desc d;
        pk_world_desc_init(&d);
        d.gravity[0] = M_gravity.x;
        d.gravity[1] = M_gravity.y;
        d.gravity[2] = M_gravity.z;
        d.solver_iterations = int32_t(M_iterations);
        d.precision = int32_t(M_precision);
        d.max_bodies = M_max_bodies;
        d.max_pairs = M_max_pairs;
        d.max_worlds = M_max_worlds;
        return d;
    }

private:
    vec3 M_gravity{0.0, -9.81, 0.0}; /* world.h:43-47 */
    std::size_t M_iterations = 10;   /* world.h:48 */
    precision M_precision = precision::f64;
    int32_t M_max_bodies = 4096, M_max_pairs = 0, M_max_worlds = 1;
};

/* A mesh made in (and shared within) one world. */
class mesh
{
public:
    mesh() = default;
    explicit mesh(int32_t id) : M_id(id) {}
    [[nodiscard]] int32_t id() const { return M_id; }
    [[nodiscard]] bool valid() const { return M_id >= 0; }

private:
    int32_t M_id = -1;
};

class object_desc
{
public:
    [[nodiscard]] static object_desc dynam() { return object_desc(body_type::dynam); }
    [[nodiscard]] static object_desc stat() { return object_desc(body_type::stat); }
    explicit object_desc(body_type t) : M_type(t) {}

#define PK_GB300_WITH(name, type, field)                                                                    \
    object_desc &name(const type &v) &                                                                       \
    {                                                                                                        \
        field = v;                                                                                           \
        return *this;                                                                                        \
    }                                                                                                        \
    object_desc &&name(const type &v) && { return std::move(name(v)); }
    PK_GB300_WITH(with_pos, vec3, M_pos)
    PK_GB300_WITH(with_vel, vec3, M_vel)
    PK_GB300_WITH(with_mass, double, M_mass)
    PK_GB300_WITH(with_orientation, quat, M_orientation)
    PK_GB300_WITH(with_ang_vel, vec3, M_ang_vel)
    PK_GB300_WITH(with_inertia_tensor, mat3, M_inertia)
    PK_GB300_WITH(with_mesh, mesh, M_mesh)
    PK_GB300_WITH(with_restitution, double, M_restitution)
    PK_GB300_WITH(with_friction, double, M_friction)
    PK_GB300_WITH(in_world, int32_t, M_world) /* sub-world of a batched world object */
#undef PK_GB300_WITH

    [[nodiscard]] body_type type() const { return M_type; }
    [[nodiscard]] const mesh &mesh_ref() const { return M_mesh; }

    /* object(object_desc) throws without a mesh (object.h:119-122) */
    [[nodiscard]] pk_body_desc to_c() const
    {
        if (!M_mesh.valid()) throw std::invalid_argument("Object must have a mesh");
        pk_body_desc d;
        pk_body_desc_init(&d);
        d.type = int32_t(M_type);
        d.shape = M_mesh.id();
        d.world = M_world;
        const double p[3] = {M_pos.x, M_pos.y, M_pos.z}, v[3] = {M_vel.x, M_vel.y, M_vel.z},
                     w[3] = {M_ang_vel.x, M_ang_vel.y, M_ang_vel.z};
        for (int k = 0; k < 3; ++k)
        {
            d.pos[k] = p[k];
            d.vel[k] = v[k];
            d.ang_vel[k] = w[k];
        }
        d.quat[0] = M_orientation.w;
        d.quat[1] = M_orientation.x;
        d.quat[2] = M_orientation.y;
        d.quat[3] = M_orientation.z;
        d.mass = M_mass;
        for (int k = 0; k < 9; ++k) d.inertia[k] = M_inertia[size_t(k)];
        d.restitution = M_restitution;
        d.friction = M_friction;
        return d;
    }

private:
    body_type M_type;
    vec3 M_pos{}, M_vel{}, M_ang_vel{};
    double M_mass = 1.0;
    quat M_orientation{};
    mat3 M_inertia = identity3();
    mesh M_mesh{};
    double M_restitution = 0.5; /* object.h:107 */
    double M_friction = 0.5;    /* object.h:108 */
    int32_t M_world = 0;
};

/* A body's state as get_rigid sees it (particle.h:135-149). */
struct body_state
{
    vec3 pos;
    quat orientation;
    vec3 vel;
    vec3 ang_vel;
};

/* Arena handle (slot | generation << 32, arena.h:179-206). */
struct handle
{
    uint64_t id = 0;
    friend bool operator==(const handle &, const handle &) = default;
};

class world
{
public:
    explicit world(const world_desc &desc)
    {
        const pk_world_desc d = desc.to_c();
        detail::check(pk_world_create(&d, &M_w), "pk_world_create");
    }
    ~world()
    {
        if (M_w) pk_world_destroy(M_w);
    }
    world(const world &) = delete;
    world &operator=(const world &) = delete;
    world(world &&o) noexcept : M_w(std::exchange(o.M_w, nullptr)), M_rows(std::move(o.M_rows)) {}
    world &operator=(world &&o) noexcept
    {
        if (this != &o)
        {
            if (M_w) pk_world_destroy(M_w);
            M_w = std::exchange(o.M_w, nullptr);
            M_rows = std::move(o.M_rows);
        }
        return *this;
    }

    /* mesh::box / sphere / pyramid / make (mesh.h:219-236) */
    mesh make_box(const vec3 &half_extents)
    {
        int32_t id = -1;
        detail::check(pk_shape_box(M_w, half_extents.x, half_extents.y, half_extents.z, &id), "pk_shape_box");
        return mesh(id);
    }
    mesh make_sphere(double radius, int32_t stacks = 16, int32_t sectors = 32)
    {
        int32_t id = -1;
        detail::check(pk_shape_sphere(M_w, radius, stacks, sectors, &id), "pk_shape_sphere");
        return mesh(id);
    }
    mesh make_pyramid(double base_half, double height)
    {
        int32_t id = -1;
        detail::check(pk_shape_pyramid(M_w, base_half, height, &id), "pk_shape_pyramid");
        return mesh(id);
    }
    mesh make_mesh(std::span<const vec3> verts, std::span<const std::array<int32_t, 3>> tris)
    {
        std::vector<double> v;
        v.reserve(verts.size() * 3);
        for (const vec3 &p : verts) v.insert(v.end(), {p.x, p.y, p.z});
        std::vector<int32_t> t;
        t.reserve(tris.size() * 3);
        for (const auto &tr : tris) t.insert(t.end(), tr.begin(), tr.end());
        int32_t id = -1;
        detail::check(pk_shape_mesh(M_w, v.data(), int32_t(verts.size()), t.data(), int32_t(tris.size()), &id),
                      "pk_shape_mesh");
        return mesh(id);
    }

    /* world_base::create_rigid (world.h:202-208) */
    handle create_rigid(const object_desc &desc)
    {
        const pk_body_desc d = desc.to_c();
        handle h;
        detail::check(pk_body_add(M_w, &d, 1, &h.id), "pk_body_add");
        return h;
    }
    std::vector<handle> create_rigids(std::span<const object_desc> descs)
    {
        std::vector<pk_body_desc> d;
        d.reserve(descs.size());
        for (const object_desc &o : descs) d.push_back(o.to_c());
        std::vector<uint64_t> ids(descs.size());
        detail::check(pk_body_add(M_w, d.data(), int32_t(d.size()), ids.data()), "pk_body_add");
        std::vector<handle> out;
        out.reserve(ids.size());
        for (uint64_t id : ids) out.push_back(handle{id});
        return out;
    }
    /* world_base::remove_rigid (world.h:209-218): false for a stale handle */
    bool remove_rigid(handle h)
    {
        const int rc = pk_body_remove(M_w, h.id);
        if (rc == PK_ERR_STALE_HANDLE) return false;
        detail::check(rc, "pk_body_remove");
        return true;
    }
    /* world_base::get_rigid (world.h:220-224): the state, or nullopt for a stale handle */
    std::optional<body_state> get_rigid(handle h)
    {
        const int rc = pk_body_alive(M_w, h.id);
        if (rc == PK_ERR_STALE_HANDLE) return std::nullopt;
        detail::check(rc, "pk_body_alive");
        read_rows();
        const size_t slot = size_t(h.id & 0xFFFFFFFFu);
        if (slot * 14 >= M_rows.size()) return std::nullopt;
        const double *r = M_rows.data() + slot * 14;
        return body_state{{r[0], r[1], r[2]}, {r[3], r[4], r[5], r[6]}, {r[7], r[8], r[9]}, {r[10], r[11], r[12]}};
    }
    /* every slot's state row: pos3 quat4 vel3 ang_vel3 alive (14 doubles) */
    const std::vector<double> &read_all()
    {
        read_rows();
        return M_rows;
    }

    /* world_base::step (world.h:234-242) around the device step_impl */
    void step(double dt) { detail::check(pk_world_step(M_w, dt), "pk_world_step"); }

    /* Broadphase pairs of the last step (min_local << 32 | max_local, collision_phases.h:63-69). */
    std::vector<uint64_t> pairs()
    {
        int32_t n = 0;
        detail::check(pk_world_read_pairs(M_w, nullptr, nullptr, 0, &n), "pk_world_read_pairs");
        std::vector<uint64_t> k(static_cast<size_t>(n));
        detail::check(pk_world_read_pairs(M_w, k.data(), nullptr, n, &n), "pk_world_read_pairs");
        return k;
    }

    [[nodiscard]] pk_world *raw() const { return M_w; }

private:
    pk_world *M_w = nullptr;
    std::vector<double> M_rows;

    void read_rows()
    {
        int32_t n = 0;
        detail::check(pk_world_read_bodies(M_w, nullptr, 0, &n), "pk_world_read_bodies");
        M_rows.resize(size_t(n) * 14);
        detail::check(pk_world_read_bodies(M_w, M_rows.data(), n, &n), "pk_world_read_bodies");
    }
};

} // namespace physkit_gb300
#endif
