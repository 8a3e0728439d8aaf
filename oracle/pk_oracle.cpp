// pk_oracle.cpp — FP64 CPU oracle for the PhysKit world step.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA step in physkit_gb300/ and the CPU baseline
// timed by bench.py. No product code links or calls it.
//
// A faithful, dependency-free restatement of the reference's step path. Each part names the
// reference file:line it follows. Where the reference is unpinned or non-deterministic, this
// file fixes a choice and says so:
//  * Summation order of dot products and 3x3 products is left to right (the reference's order
//    is whatever Eigen's vectorisation picks, which its tests do not pin).
//  * The half-angle sine/cosine of the orientation update (integrate.h:20-31 via Eigen
//    AngleAxis) uses an own Cody-Waite + Taylor evaluation, accurate to ~1 ulp, so CPU and GPU
//    can be compared bit for bit; hypot (constraint.h:1162) is sqrt(x*x+y*y).
//  * The pair set and manifold store iterate in ascending pair-key order (the reference iterates
//    an absl hash set whose order is unspecified, collision_phases.h:383-403).
//  * The EPA face heap uses libstdc++'s std::push_heap/std::pop_heap, as the reference does when
//    built with GCC (collision.cpp:390-408).
// Compile with -ffp-contract=off: no fused multiply-adds anywhere.

#include "pk_oracle.h"

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <numbers>
#include <optional>
#include <unordered_set>
#include <vector>

namespace ora
{

// ---------------------------------------------------------------------------------------------
// Linear algebra (restates algebra/lin_alg.h semantics over Eigen: Hamilton quaternions stored
// w-first in the constructor, lin_alg.h:428-432; quat*vec = Eigen _transformVector,
// lin_alg.h:493-499; normalized() leaves a zero vector unchanged).
// ---------------------------------------------------------------------------------------------
struct V3
{
    double x = 0, y = 0, z = 0;
};
struct Qt
{
    double w = 1, x = 0, y = 0, z = 0;
};
struct M3
{
    double m[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
};

inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b)
{ return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double sqnorm(V3 a) { return dot(a, a); }
inline double norm(V3 a) { return std::sqrt(sqnorm(a)); }
inline V3 normalized(V3 a)
{
    double n2 = sqnorm(a);
    if (n2 > 0.0) return a / std::sqrt(n2);
    return a;
}

inline Qt qmul(Qt a, Qt b)
{
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
            a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z,
            a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
}
inline Qt conj(Qt q) { return {q.w, -q.x, -q.y, -q.z}; }
inline V3 rotate(Qt q, V3 v)
{
    V3 u{q.x, q.y, q.z};
    V3 uv = cross(u, v);
    uv = uv + uv;
    return v + q.w * uv + cross(u, uv);
}
inline Qt qnormalized(Qt q)
{
    // Eigen stores (x,y,z,w); squaredNorm runs in storage order.
    double n2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (n2 > 0.0)
    {
        double n = std::sqrt(n2);
        return {q.w / n, q.x / n, q.y / n, q.z / n};
    }
    return q;
}

inline M3 to_matrix(Qt q)
{
    // Standard unit-quaternion rotation matrix (Eigen toRotationMatrix form).
    double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
    double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    M3 r;
    r.m[0][0] = 1.0 - (tyy + tzz);
    r.m[0][1] = txy - twz;
    r.m[0][2] = txz + twy;
    r.m[1][0] = txy + twz;
    r.m[1][1] = 1.0 - (txx + tzz);
    r.m[1][2] = tyz - twx;
    r.m[2][0] = txz - twy;
    r.m[2][1] = tyz + twx;
    r.m[2][2] = 1.0 - (txx + tyy);
    return r;
}
inline M3 transpose(const M3 &a)
{
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
inline M3 matmul(const M3 &a, const M3 &b)
{
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}
inline V3 matvec(const M3 &a, V3 v)
{
    return {a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z,
            a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
            a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z};
}
// 3x3 inverse by the adjugate: inv(i,j) = cof(j,i) / det, det expanded along row 0.
inline M3 inverse(const M3 &a)
{
    const auto &m = a.m;
    double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    double c10 = m[0][2] * m[2][1] - m[0][1] * m[2][2];
    double c11 = m[0][0] * m[2][2] - m[0][2] * m[2][0];
    double c12 = m[0][1] * m[2][0] - m[0][0] * m[2][1];
    double c20 = m[0][1] * m[1][2] - m[0][2] * m[1][1];
    double c21 = m[0][2] * m[1][0] - m[0][0] * m[1][2];
    double c22 = m[0][0] * m[1][1] - m[0][1] * m[1][0];
    double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    M3 r;
    r.m[0][0] = c00 / det;
    r.m[0][1] = c10 / det;
    r.m[0][2] = c20 / det;
    r.m[1][0] = c01 / det;
    r.m[1][1] = c11 / det;
    r.m[1][2] = c21 / det;
    r.m[2][0] = c02 / det;
    r.m[2][1] = c12 / det;
    r.m[2][2] = c22 / det;
    return r;
}

// Deterministic sine/cosine: Cody-Waite reduction by pi/2 (pi/2 split into three doubles with
// 30-bit leading parts so k*P1 and k*P2 are exact for |k| < 2^23) and Taylor series on
// [-pi/4, pi/4] in Horner form (terms to r^19 / r^18, truncation below 2^-60 relative).
void sincos_det(double x, double *s, double *c)
{
    constexpr double two_over_pi = 0.6366197723675814;
    constexpr double p1 = 1.570796325802803;      // 0x1.921fb54p+0
    constexpr double p2 = 9.920935791635221e-10;  // 0x1.10b46118p-30
    constexpr double p3 = 5.170182981794105e-19;  // 0x1.313198a2e037p-61
    double k = std::nearbyint(x * two_over_pi);
    double r = x - k * p1;
    r = r - k * p2;
    r = r - k * p3;
    double r2 = r * r;
    double ps = -1.0 / 121645100408832000.0; // -1/19!
    ps = ps * r2 + 1.0 / 355687428096000.0;  // 1/17!
    ps = ps * r2 - 1.0 / 1307674368000.0;    // 1/15!
    ps = ps * r2 + 1.0 / 6227020800.0;       // 1/13!
    ps = ps * r2 - 1.0 / 39916800.0;         // 1/11!
    ps = ps * r2 + 1.0 / 362880.0;           // 1/9!
    ps = ps * r2 - 1.0 / 5040.0;             // 1/7!
    ps = ps * r2 + 1.0 / 120.0;              // 1/5!
    ps = ps * r2 - 1.0 / 6.0;                // 1/3!
    double sr = r + r * (r2 * ps);
    double pc = 1.0 / 6402373705728000.0;    // 1/18!
    pc = pc * r2 - 1.0 / 20922789888000.0;   // 1/16!
    pc = pc * r2 + 1.0 / 87178291200.0;      // 1/14!
    pc = pc * r2 - 1.0 / 479001600.0;        // 1/12!
    pc = pc * r2 + 1.0 / 3628800.0;          // 1/10!
    pc = pc * r2 - 1.0 / 40320.0;            // 1/8!
    pc = pc * r2 + 1.0 / 720.0;              // 1/6!
    pc = pc * r2 - 1.0 / 24.0;               // 1/4!
    pc = pc * r2 + 0.5;                      // 1/2!
    double cr = 1.0 - r2 * pc;
    long long q = static_cast<long long>(k);
    switch (static_cast<int>(q & 3))
    {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}

inline double hypot_det(double a, double b) { return std::sqrt(a * a + b * b); }

inline double dmin(double a, double b) { return (b < a) ? b : a; } // std::min
inline double dmax(double a, double b) { return (a < b) ? b : a; } // std::max

// ---------------------------------------------------------------------------------------------
// Bounds (collision/bounds.h:27-205, 539-548)
// ---------------------------------------------------------------------------------------------
struct Aabb
{
    V3 min, max;
    V3 point(unsigned i) const
    {
        return {(i & 1) ? max.x : min.x, (i & 2) ? max.y : min.y, (i & 4) ? max.z : min.z};
    }
    bool contains(const Aabb &o) const
    {
        return (o.min.x >= min.x && o.max.x <= max.x) && (o.min.y >= min.y && o.max.y <= max.y) &&
               (o.min.z >= min.z && o.max.z <= max.z);
    }
    bool intersects(const Aabb &o) const
    {
        return (min.x <= o.max.x && max.x >= o.min.x) && (min.y <= o.max.y && max.y >= o.min.y) &&
               (min.z <= o.max.z && max.z >= o.min.z);
    }
    double surface_area() const
    {
        V3 s = max - min;
        return 2.0 * (s.x * s.y + s.y * s.z + s.z * s.x);
    }
    V3 support(V3 d) const
    {
        double sx = d.x >= 0 ? 1 : -1, sy = d.y >= 0 ? 1 : -1, sz = d.z >= 0 ? 1 : -1;
        return {sx > 0 ? max.x : min.x, sy > 0 ? max.y : min.y, sz > 0 ? max.z : min.z};
    }
};

// ray (bvh.h:38-93): the direction is normalised at construction; slab test with safe_inv
// (1/x, +-inf at zero, bvh.h:24-35) and NaN limits (an axis the ray is parallel to is unconstrained
// when the origin lies between its slabs, empty otherwise).
struct Ray
{
    V3 o, d;
    Ray(V3 origin, V3 dir) : o(origin), d(normalized(dir)) {}
    static double safe_inv(double x) { return 1.0 / x; }
    bool intersect_distance(const Aabb &b, double max_d, double &out) const
    {
        auto slab = [](double lo, double hi, double &a, double &c) {
            if (std::isnan(lo)) lo = -std::numeric_limits<double>::infinity();
            if (std::isnan(hi)) hi = std::numeric_limits<double>::infinity();
            a = std::fmin(lo, hi);
            c = std::fmax(lo, hi);
        };
        double tminx, tmaxx, tminy, tmaxy, tminz, tmaxz;
        slab((b.min.x - o.x) * safe_inv(d.x), (b.max.x - o.x) * safe_inv(d.x), tminx, tmaxx);
        slab((b.min.y - o.y) * safe_inv(d.y), (b.max.y - o.y) * safe_inv(d.y), tminy, tmaxy);
        slab((b.min.z - o.z) * safe_inv(d.z), (b.max.z - o.z) * safe_inv(d.z), tminz, tmaxz);
        double tmin = std::max({tminx, tminy, tminz});
        double tmax = std::min({tmaxx, tmaxy, tmaxz});
        if (tmax >= 0.0 && tmin <= tmax && tmin <= max_d)
        {
            out = std::max(0.0, tmin);
            return true;
        }
        return false;
    }
};
inline Aabb aabb_union(const Aabb &a, const Aabb &b)
{
    return {{dmin(a.min.x, b.min.x), dmin(a.min.y, b.min.y), dmin(a.min.z, b.min.z)},
            {dmax(a.max.x, b.max.x), dmax(a.max.y, b.max.y), dmax(a.max.z, b.max.z)}};
}
inline Aabb aabb_from_points(const std::vector<V3> &p)
{
    Aabb b{p[0], p[0]};
    for (size_t i = 1; i < p.size(); ++i)
    {
        b.min.x = dmin(b.min.x, p[i].x);
        b.min.y = dmin(b.min.y, p[i].y);
        b.min.z = dmin(b.min.z, p[i].z);
        b.max.x = dmax(b.max.x, p[i].x);
        b.max.y = dmax(b.max.y, p[i].y);
        b.max.z = dmax(b.max.z, p[i].z);
    }
    return b;
}
// aabb * quat (bounds.h:144-158): bounds of the 8 rotated corners, corner 0 first.
inline Aabb aabb_rotate(const Aabb &b, Qt q)
{
    V3 p0 = rotate(q, b.min);
    Aabb r{p0, p0};
    for (unsigned i = 1; i < 8; ++i)
    {
        V3 pt = rotate(q, b.point(i));
        r.min.x = dmin(r.min.x, pt.x);
        r.min.y = dmin(r.min.y, pt.y);
        r.min.z = dmin(r.min.z, pt.z);
        r.max.x = dmax(r.max.x, pt.x);
        r.max.y = dmax(r.max.y, pt.y);
        r.max.z = dmax(r.max.z, pt.z);
    }
    return r;
}

struct Obb
{
    V3 center;
    Qt orientation;
    V3 half;
    V3 support(V3 d) const
    {
        V3 ld = rotate(conj(orientation), d);
        V3 s{ld.x >= 0 ? 1.0 : -1.0, ld.y >= 0 ? 1.0 : -1.0, ld.z >= 0 ? 1.0 : -1.0};
        return center + rotate(orientation, V3{s.x * half.x, s.y * half.y, s.z * half.z});
    }
};

// ---------------------------------------------------------------------------------------------
// Meshes (collision/mesh.h:117-285, src/mesh.cpp:25-151, 341-358, 398, 442-448)
// ---------------------------------------------------------------------------------------------
struct Mesh
{
    std::vector<V3> verts;
    std::vector<std::array<unsigned, 3>> tris;
    Aabb bounds;

    // mesh::support: first strictly maximal vertex in vertex order (mesh.cpp:341-358).
    V3 support(V3 d) const
    {
        size_t best = 0;
        double best_dot = dot(verts[0], d);
        for (size_t i = 1; i < verts.size(); ++i)
        {
            double v = dot(verts[i], d);
            if (v > best_dot)
            {
                best_dot = v;
                best = i;
            }
        }
        return verts[best];
    }
    double volume() const
    {
        double vol = 0.0;
        for (auto &t : tris) vol += dot(verts[t[0]], cross(verts[t[1]], verts[t[2]]));
        return vol / 6.0;
    }
};

std::shared_ptr<Mesh> make_mesh(std::vector<V3> v, std::vector<std::array<unsigned, 3>> t)
{
    auto m = std::make_shared<Mesh>();
    m->verts = std::move(v);
    m->tris = std::move(t);
    m->bounds = aabb_from_points(m->verts);
    return m;
}

std::shared_ptr<Mesh> mesh_box(double hx, double hy, double hz)
{
    std::vector<V3> v = {{-hx, -hy, -hz}, {+hx, -hy, -hz}, {+hx, +hy, -hz}, {-hx, +hy, -hz},
                         {-hx, -hy, +hz}, {+hx, -hy, +hz}, {+hx, +hy, +hz}, {-hx, +hy, +hz}};
    std::vector<std::array<unsigned, 3>> t = {{4, 5, 6}, {4, 6, 7}, {0, 3, 2}, {0, 2, 1},
                                              {1, 2, 6}, {1, 6, 5}, {0, 4, 7}, {0, 7, 3},
                                              {3, 7, 6}, {3, 6, 2}, {0, 1, 5}, {0, 5, 4}};
    return make_mesh(std::move(v), std::move(t));
}

std::shared_ptr<Mesh> mesh_sphere(double r, unsigned stacks, unsigned sectors)
{
    std::vector<V3> v;
    std::vector<std::array<unsigned, 3>> t;
    v.push_back({0.0, r, 0.0});
    for (unsigned i = 1; i < stacks; ++i)
    {
        double phi = std::numbers::pi * static_cast<double>(i) / static_cast<double>(stacks);
        for (unsigned j = 0; j < sectors; ++j)
        {
            double theta =
                2.0 * std::numbers::pi * static_cast<double>(j) / static_cast<double>(sectors);
            v.push_back({r * std::sin(phi) * std::cos(theta), r * std::cos(phi),
                         r * std::sin(phi) * std::sin(theta)});
        }
    }
    v.push_back({0.0, -r, 0.0});
    unsigned south = static_cast<unsigned>(v.size() - 1);
    for (unsigned j = 0; j < sectors; ++j) t.push_back({0, 1 + ((j + 1) % sectors), 1 + j});
    for (unsigned i = 1; i + 1 < stacks; ++i)
        for (unsigned j = 0; j < sectors; ++j)
        {
            unsigned top = 1 + (i - 1) * sectors + j, top_next = 1 + (i - 1) * sectors + (j + 1) % sectors;
            unsigned bot = 1 + i * sectors + j, bot_next = 1 + i * sectors + (j + 1) % sectors;
            t.push_back({top, top_next, bot_next});
            t.push_back({top, bot_next, bot});
        }
    unsigned last = 1 + (stacks - 2) * sectors;
    for (unsigned j = 0; j < sectors; ++j) t.push_back({south, last + j, last + (j + 1) % sectors});
    return make_mesh(std::move(v), std::move(t));
}

std::shared_ptr<Mesh> mesh_pyramid(double b, double h)
{
    std::vector<V3> v = {{-b, 0.0, -b}, {+b, 0.0, -b}, {+b, 0.0, +b}, {-b, 0.0, +b}, {0.0, h, 0.0}};
    std::vector<std::array<unsigned, 3>> t = {{0, 1, 2}, {0, 2, 3}, {1, 0, 4},
                                              {2, 1, 4}, {3, 2, 4}, {0, 3, 4}};
    return make_mesh(std::move(v), std::move(t));
}

// ray::intersect, Moeller-Trumbore (bvh.h:97-135): the hit of one triangle within max_d.
struct TriHit
{
    V3 pos, normal;
    double t;
};
inline bool ray_triangle(const V3 &o, const V3 &d, const V3 &v0, const V3 &v1, const V3 &v2, double max_d, TriHit &out)
{
    const double eps = 1e-12;
    V3 e1 = v1 - v0, e2 = v2 - v0;
    V3 h = cross(d, e2);
    double a = dot(e1, h);
    if (a > -eps && a < eps) return false;
    double f = 1.0 / a;
    V3 sv = o - v0;
    double u = f * dot(sv, h);
    if (u < 0.0 || u > 1.0) return false;
    V3 q = cross(sv, e1);
    double v = f * dot(d, q);
    if (v < 0.0 || u + v > 1.0) return false;
    double t = f * dot(e2, q);
    if (t < 0.0 || t > max_d) return false;
    out = {o + d * t, normalized(cross(e1, e2)), t};
    return true;
}

// mesh::instance::ray_intersect (mesh.cpp:400-415) over mesh::ray_intersect (mesh.cpp:169-197):
// the ray goes into the body frame (and its direction is normalised again by the ray
// constructor), every triangle is tested with the running best distance as the limit, so a later
// triangle at the same distance replaces an earlier one, and the hit comes back to world space.
// Triangles are visited in index order: the reference visits them in its static BVH's order, which
// can only differ where two triangles are hit at exactly the same distance.
inline bool mesh_ray_intersect(const Mesh &m, V3 pos, Qt q, V3 origin, V3 dir, double max_d, TriHit &out, int &tri)
{
    Ray world(origin, dir);
    Qt inv = conj(q);
    Ray local(rotate(inv, world.o - pos), rotate(inv, world.d));
    double best_t = max_d;
    bool found = false;
    for (size_t i = 0; i < m.tris.size(); ++i)
    {
        TriHit h;
        const auto &t = m.tris[i];
        if (ray_triangle(local.o, local.d, m.verts[t[0]], m.verts[t[1]], m.verts[t[2]], best_t, h))
        {
            best_t = h.t;
            out = h;
            tri = int(i);
            found = true;
        }
    }
    if (found)
    {
        out.pos = rotate(q, out.pos) + pos;
        out.normal = rotate(q, out.normal);
    }
    return found;
}

struct MeshInst
{
    const Mesh *mesh;
    V3 pos;
    Qt q;
    // instance::support (mesh.cpp:442-448)
    V3 support(V3 d) const
    {
        V3 ld = rotate(conj(q), d);
        return rotate(q, mesh->support(ld)) + pos;
    }
    // instance::bounds (mesh.cpp:398)
    Aabb bounds() const
    {
        Aabb r = aabb_rotate(mesh->bounds, q);
        return {r.min + pos, r.max + pos};
    }
};

// ---------------------------------------------------------------------------------------------
// GJK / EPA (collision/collision.h:27-59, src/collision.cpp:10-518)
// ---------------------------------------------------------------------------------------------
struct SupportPt
{
    V3 p, pa, pb;
};
struct CollisionInfo
{
    V3 normal, world_a, world_b;
    double depth = 0;
};

template <class A, class B> inline SupportPt minkowski(const A &a, const B &b, V3 d)
{
    V3 pa = a.support(d);
    V3 pb = b.support(-d);
    return {pa - pb, pa, pb};
}

struct Simplex
{
    std::array<SupportPt, 4> v{};
    int n = 0;
    void push(const SupportPt &p) { v[n++] = p; }
    void erase(int i)
    {
        for (int k = i; k + 1 < n; ++k) v[k] = v[k + 1];
        --n;
    }
};

bool handle_line(Simplex &s, V3 &dir)
{
    constexpr double eps = 1e-12;
    const SupportPt a = s.v[1], b = s.v[0];
    V3 ab = b.p - a.p, ao = -a.p;
    if (dot(ab, ao) > 0.0)
    {
        V3 triple = cross(cross(ab, ao), ab);
        if (sqnorm(triple) < eps)
        {
            V3 ab_hat = normalized(ab);
            V3 perp = cross(ab_hat, V3{0.0, 1.0, 0.0});
            if (sqnorm(perp) < eps) perp = cross(ab_hat, V3{0.0, 0.0, 1.0});
            dir = normalized(perp);
        }
        else
            dir = normalized(triple);
    }
    else
    {
        s.erase(0);
        dir = normalized(ao);
    }
    return false;
}

bool handle_triangle(Simplex &s, V3 &dir)
{
    const SupportPt a = s.v[2], b = s.v[1], c = s.v[0];
    V3 ab = b.p - a.p, ac = c.p - a.p, ao = -a.p;
    V3 abc = cross(ab, ac);
    V3 ab_perp = cross(ab, abc);
    if (dot(ab_perp, ao) > 0.0)
    {
        s.erase(0);
        V3 triple = cross(cross(ab, ao), ab);
        dir = (sqnorm(triple) < 1e-12) ? normalized(ao) : normalized(triple);
        return false;
    }
    V3 ac_perp = cross(abc, ac);
    if (dot(ac_perp, ao) > 0.0)
    {
        s.erase(1);
        V3 triple = cross(cross(ac, ao), ac);
        dir = (sqnorm(triple) < 1e-12) ? normalized(ao) : normalized(triple);
        return false;
    }
    if (dot(abc, ao) <= 0.0)
    {
        std::swap(s.v[0], s.v[1]);
        dir = normalized(-abc);
    }
    else
        dir = normalized(abc);
    return false;
}

bool handle_tetrahedron(Simplex &s, V3 &dir)
{
    const SupportPt a = s.v[3], b = s.v[2], c = s.v[1], d = s.v[0];
    V3 ao = -a.p;
    V3 abc = cross(b.p - a.p, c.p - a.p);
    V3 acd = cross(c.p - a.p, d.p - a.p);
    V3 adb = cross(d.p - a.p, b.p - a.p);
    auto orient = [](V3 &n, const SupportPt &fa, const SupportPt &opp)
    {
        if (dot(n, opp.p - fa.p) > 0.0) n = -n;
    };
    orient(abc, a, d);
    orient(acd, a, b);
    orient(adb, a, c);
    if (dot(abc, ao) > 0.0)
    {
        s.n = 0;
        s.push(c);
        s.push(b);
        s.push(a);
        dir = normalized(abc);
        return handle_triangle(s, dir);
    }
    if (dot(acd, ao) > 0.0)
    {
        s.n = 0;
        s.push(d);
        s.push(c);
        s.push(a);
        dir = normalized(acd);
        return handle_triangle(s, dir);
    }
    if (dot(adb, ao) > 0.0)
    {
        s.n = 0;
        s.push(b);
        s.push(d);
        s.push(a);
        dir = normalized(adb);
        return handle_triangle(s, dir);
    }
    return true;
}

bool handle_simplex(Simplex &s, V3 &dir)
{
    switch (s.n)
    {
    case 2: return handle_line(s, dir);
    case 3: return handle_triangle(s, dir);
    case 4: return handle_tetrahedron(s, dir);
    default: return false;
    }
}

template <class A, class B> std::optional<Simplex> gjk_collision(const A &a, const B &b)
{
    Simplex s;
    V3 dir{1.0, 0.0, 0.0};
    SupportPt pt = minkowski(a, b, dir);
    s.push(pt);
    if (sqnorm(pt.p) < 1e-12) return s;
    dir = -normalized(pt.p);
    for (int iter = 0; iter < 100; ++iter)
    {
        SupportPt np = minkowski(a, b, dir);
        if (dot(np.p, dir) <= 0.0) return std::nullopt;
        s.push(np);
        if (handle_simplex(s, dir)) return s;
    }
    return std::nullopt;
}

template <class A, class B> bool pad_simplex(const A &a, const B &b, Simplex &s)
{
    int n0 = s.n;
    if (n0 <= 1)
    {
        V3 dir{1.0, 0.0, 0.0};
        SupportPt p2 = minkowski(a, b, dir);
        if (sqnorm(p2.p - s.v[0].p) < 1e-6) p2 = minkowski(a, b, -dir);
        s.push(p2);
    }
    if (n0 <= 2)
    {
        V3 line = s.v[1].p - s.v[0].p;
        V3 dir = cross(normalized(line), V3{0.0, 1.0, 0.0});
        if (sqnorm(dir) < 1e-6) dir = cross(normalized(line), V3{0.0, 0.0, 1.0});
        dir = normalized(dir);
        SupportPt p3 = minkowski(a, b, dir);
        if (sqnorm(cross(line, p3.p - s.v[0].p)) < 1e-6) p3 = minkowski(a, b, -dir);
        s.push(p3);
    }
    if (n0 <= 3)
    {
        V3 ab = s.v[1].p - s.v[0].p, ac = s.v[2].p - s.v[0].p;
        V3 dir = normalized(cross(ab, ac));
        SupportPt p4 = minkowski(a, b, dir);
        if (std::abs(dot(p4.p - s.v[0].p, dir)) < 1e-6) p4 = minkowski(a, b, -dir);
        s.push(p4);
    }
    V3 ad = s.v[0].p - s.v[3].p, bd = s.v[1].p - s.v[3].p, cd = s.v[2].p - s.v[3].p;
    double triple = dot(ad, cross(bd, cd));
    return std::abs(triple) > 1e-12;
}

struct Epa
{
    using idx_t = std::uint16_t;
    static constexpr idx_t null_index = static_cast<idx_t>(-1);
    struct Face
    {
        std::array<idx_t, 3> v{};
        std::array<idx_t, 3> adj{null_index, null_index, null_index};
        V3 normal;
        double distance = 0;
        bool obsolete = false;
    };
    struct Edge
    {
        idx_t start, end, adj;
    };
    std::vector<Face> faces;
    std::vector<SupportPt> poly;
    std::vector<size_t> heap;

    void init_face(size_t f, size_t i, size_t j, size_t k, idx_t opp = null_index)
    {
        Face &fc = faces[f];
        fc.v = {static_cast<idx_t>(i), static_cast<idx_t>(j), static_cast<idx_t>(k)};
        V3 ab = poly[j].p - poly[i].p, ac = poly[k].p - poly[i].p;
        fc.normal = cross(ab, ac);
        if (sqnorm(fc.normal) < 1e-12)
            fc.normal = V3{0, 0, 0};
        else
            fc.normal = normalized(fc.normal);
        if (opp != null_index && dot(fc.normal, poly[opp].p - poly[i].p) > 0.0)
        {
            std::swap(fc.v[1], fc.v[2]);
            fc.normal = -fc.normal;
        }
        fc.distance = dot(fc.normal, poly[i].p);
    }
    size_t alloc_face()
    {
        faces.emplace_back();
        return faces.size() - 1;
    }
    void link(size_t f1, size_t f2, size_t va, size_t vb)
    {
        Face &a = faces[f1];
        Face &b = faces[f2];
        int e1 = (a.v[0] == va) ? 0 : (a.v[1] == va ? 1 : 2);
        int e2 = (b.v[0] == vb) ? 0 : (b.v[1] == vb ? 1 : 2);
        a.adj[e1] = static_cast<idx_t>(f2);
        b.adj[e2] = static_cast<idx_t>(f1);
    }
    auto cmp()
    {
        return [this](size_t f1, size_t f2) { return faces[f1].distance > faces[f2].distance; };
    }
    void push_face(size_t f)
    {
        heap.push_back(f);
        std::push_heap(heap.begin(), heap.end(), cmp());
    }
    size_t pop_face()
    {
        while (!heap.empty())
        {
            std::pop_heap(heap.begin(), heap.end(), cmp());
            size_t f = heap.back();
            heap.pop_back();
            if (!faces[f].obsolete) return f;
        }
        return static_cast<size_t>(null_index);
    }
    std::vector<Edge> silhouette(idx_t face, V3 p)
    {
        constexpr double tol = 1e-6;
        std::vector<size_t> stack{face};
        faces[face].obsolete = true;
        std::vector<Edge> horizon;
        while (!stack.empty())
        {
            size_t cur = stack.back();
            stack.pop_back();
            for (int i = 0; i < 3; ++i)
            {
                size_t n = faces[cur].adj[i];
                if (n == null_index) continue;
                Face &nb = faces[n];
                if (nb.obsolete) continue;
                if (dot(nb.normal, p) > nb.distance + tol)
                {
                    nb.obsolete = true;
                    stack.push_back(n);
                }
                else
                    horizon.push_back({faces[cur].v[i], faces[cur].v[(i + 1) % 3], static_cast<idx_t>(n)});
            }
        }
        return horizon;
    }
    void initial_tetrahedron()
    {
        auto aip = [&](size_t i, size_t j, size_t k, idx_t opp)
        {
            size_t f = alloc_face();
            init_face(f, i, j, k, opp);
            push_face(f);
        };
        aip(0, 1, 2, 3);
        aip(0, 2, 3, 1);
        aip(0, 3, 1, 2);
        aip(1, 3, 2, 0);
        for (size_t i = 0; i < 4; ++i)
            for (size_t j = i + 1; j < 4; ++j)
                for (int e1 = 0; e1 < 3; ++e1)
                {
                    idx_t u1 = faces[i].v[e1], v1 = faces[i].v[(e1 + 1) % 3];
                    for (int e2 = 0; e2 < 3; ++e2)
                    {
                        idx_t u2 = faces[j].v[e2], v2 = faces[j].v[(e2 + 1) % 3];
                        if (u1 == v2 && v1 == u2)
                        {
                            faces[i].adj[e1] = static_cast<idx_t>(j);
                            faces[j].adj[e2] = static_cast<idx_t>(i);
                        }
                    }
                }
    }
    CollisionInfo barycentric(const Face &f) const
    {
        const SupportPt &p0 = poly[f.v[0]], &p1 = poly[f.v[1]], &p2 = poly[f.v[2]];
        V3 pm = f.normal * f.distance;
        V3 v0 = p1.p - p0.p, v1 = p2.p - p0.p, v2 = pm - p0.p;
        double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
        double d20 = dot(v2, v0), d21 = dot(v2, v1);
        double denom = d00 * d11 - d01 * d01;
        double v = (d11 * d20 - d01 * d21) / denom;
        double w = (d00 * d21 - d01 * d20) / denom;
        double u = 1.0 - v - w;
        CollisionInfo ci;
        ci.normal = -f.normal;
        ci.world_a = u * p0.pa + v * p1.pa + w * p2.pa;
        ci.world_b = u * p0.pb + v * p1.pb + w * p2.pb;
        ci.depth = f.distance;
        return ci;
    }

    template <class A, class B>
    static std::optional<CollisionInfo> solve(const A &a, const B &b, Simplex &s)
    {
        if (s.n < 4 && !pad_simplex(a, b, s)) return std::nullopt;
        Epa e;
        e.poly.assign(s.v.begin(), s.v.begin() + s.n);
        e.initial_tetrahedron();
        constexpr double tol = 1e-6;
        for (int iter = 0; iter < 64; ++iter)
        {
            size_t mf = e.pop_face();
            if (mf == null_index) break;
            Face minf = e.faces[mf];
            SupportPt p = minkowski(a, b, minf.normal);
            double pd = dot(minf.normal, p.p);
            if (pd - minf.distance < tol) return e.barycentric(minf);
            auto horizon = e.silhouette(static_cast<idx_t>(mf), p.p);
            if (horizon.empty()) break;
            e.poly.push_back(p);
            idx_t pi = static_cast<idx_t>(e.poly.size() - 1);
            std::vector<size_t> nf;
            for (const auto &h : horizon)
            {
                size_t f = e.alloc_face();
                e.init_face(f, h.start, h.end, pi);
                e.link(f, h.adj, h.start, h.end);
                e.push_face(f);
                nf.push_back(f);
            }
            size_t n = nf.size();
            for (size_t i = 0; i < n; ++i)
                for (size_t j = i + 1; j < n; ++j)
                {
                    if (horizon[i].end == horizon[j].start)
                        e.link(nf[i], nf[j], horizon[i].end, pi);
                    else if (horizon[i].start == horizon[j].end)
                        e.link(nf[j], nf[i], horizon[j].end, pi);
                }
        }
        size_t mf = e.pop_face();
        if (mf == null_index) return std::nullopt;
        return e.barycentric(e.faces[mf]);
    }
};

template <class A, class B> std::optional<CollisionInfo> gjk_epa(const A &a, const B &b)
{
    auto s = gjk_collision(a, b);
    if (s) return Epa::solve(a, b, *s);
    return std::nullopt;
}

// ---------------------------------------------------------------------------------------------
// Dynamic AABB tree (collision/bvh.h:270-535, src/bvh.cpp:235-515)
// ---------------------------------------------------------------------------------------------
struct DynTree
{
    static constexpr uint32_t null = 0xFFFFFFFFu;
    static constexpr uint32_t free_h = 0xFFFFFFFFu;
    struct Node
    {
        Aabb bounds;
        uint32_t parent = null;
        uint32_t left = null, right = null; // children (internal)
        uint32_t data = null;               // object id (leaf) / next free
        uint32_t height = free_h;
        bool is_leaf() const { return height == 0; }
    };
    std::vector<Node> nodes;
    uint32_t root = null, free_head = null;

    uint32_t alloc()
    {
        if (free_head != null)
        {
            uint32_t n = free_head;
            free_head = nodes[n].data;
            nodes[n].parent = null;
            nodes[n].height = 0;
            return n;
        }
        nodes.emplace_back();
        nodes.back().height = 0;
        return static_cast<uint32_t>(nodes.size() - 1);
    }
    void free_node(uint32_t n)
    {
        nodes[n].height = free_h;
        nodes[n].data = free_head;
        free_head = n;
    }
    uint32_t add(uint32_t id, const Aabb &b)
    {
        uint32_t leaf = alloc();
        nodes[leaf].data = id;
        nodes[leaf].bounds = b;
        insert_leaf(leaf);
        refit_and_rotate(nodes[leaf].parent);
        return leaf;
    }
    void remove_leaf(uint32_t leaf)
    {
        extract_leaf(leaf);
        free_node(leaf);
    }
    void insert_leaf(uint32_t leaf)
    {
        constexpr double ct = 2.0, cm = 2.0;
        if (root == null)
        {
            root = leaf;
            nodes[leaf].parent = null;
            return;
        }
        Aabb lb = nodes[leaf].bounds;
        uint32_t cur = root;
        while (!nodes[cur].is_leaf())
        {
            uint32_t l = nodes[cur].left, r = nodes[cur].right;
            double area_cur = nodes[cur].bounds.surface_area();
            double area_new = aabb_union(nodes[cur].bounds, lb).surface_area();
            double cost_new = cm * area_new;
            double inherited = ct * (area_new - area_cur);
            double cost_l = nodes[l].is_leaf()
                                ? ct * aabb_union(lb, nodes[l].bounds).surface_area() + inherited
                                : ct * (aabb_union(lb, nodes[l].bounds).surface_area() -
                                        nodes[l].bounds.surface_area()) +
                                      inherited;
            double cost_r = nodes[r].is_leaf()
                                ? ct * aabb_union(lb, nodes[r].bounds).surface_area() + inherited
                                : ct * (aabb_union(lb, nodes[r].bounds).surface_area() -
                                        nodes[r].bounds.surface_area()) +
                                      inherited;
            if (cost_new < cost_l && cost_new < cost_r) break;
            cur = (cost_l < cost_r) ? l : r;
        }
        uint32_t sib = cur;
        uint32_t old_parent = nodes[sib].parent;
        uint32_t np = alloc();
        nodes[np].bounds = aabb_union(lb, nodes[sib].bounds);
        nodes[np].parent = old_parent;
        nodes[np].left = sib;
        nodes[np].right = leaf;
        nodes[np].height = nodes[sib].height + 1;
        nodes[sib].parent = np;
        nodes[leaf].parent = np;
        if (old_parent != null)
        {
            if (nodes[old_parent].left == sib)
                nodes[old_parent].left = np;
            else
                nodes[old_parent].right = np;
        }
        else
            root = np;
    }
    void extract_leaf(uint32_t leaf)
    {
        if (leaf == root)
        {
            root = null;
            return;
        }
        uint32_t parent = nodes[leaf].parent;
        uint32_t grand = nodes[parent].parent;
        uint32_t sib = (nodes[parent].left == leaf) ? nodes[parent].right : nodes[parent].left;
        if (grand != null)
        {
            if (nodes[grand].left == parent)
                nodes[grand].left = sib;
            else
                nodes[grand].right = sib;
            nodes[sib].parent = grand;
            free_node(parent);
            refit_and_rotate(grand);
        }
        else
        {
            root = sib;
            nodes[sib].parent = null;
            free_node(parent);
        }
        nodes[leaf].parent = null;
    }
    void refit_and_rotate(uint32_t n)
    {
        while (n != null)
        {
            n = balance(n);
            Node &nd = nodes[n];
            nd.height = 1 + std::max(nodes[nd.left].height, nodes[nd.right].height);
            nd.bounds = aabb_union(nodes[nd.left].bounds, nodes[nd.right].bounds);
            n = nd.parent;
        }
    }
    uint32_t balance(uint32_t ia)
    {
        Node &a = nodes[ia];
        if (a.is_leaf() || a.height < 2) return ia;
        uint32_t ib = a.left, ic = a.right;
        Node &b = nodes[ib];
        Node &c = nodes[ic];
        int bal = static_cast<int>(c.height) - static_cast<int>(b.height);
        if (bal > 1)
        {
            uint32_t iff = c.left, ig = c.right;
            Node &f = nodes[iff];
            Node &g = nodes[ig];
            c.left = ia;
            c.parent = a.parent;
            a.parent = ic;
            if (c.parent != null)
            {
                if (nodes[c.parent].left == ia)
                    nodes[c.parent].left = ic;
                else
                    nodes[c.parent].right = ic;
            }
            else
                root = ic;
            if (f.height > g.height)
            {
                c.right = iff;
                a.right = ig;
                g.parent = ia;
            }
            else
            {
                c.right = ig;
                a.right = iff;
                f.parent = ia;
            }
            a.bounds = aabb_union(b.bounds, nodes[a.right].bounds);
            a.height = 1 + std::max(nodes[a.left].height, nodes[a.right].height);
            return ic;
        }
        if (bal < -1)
        {
            uint32_t id = b.left, ie = b.right;
            Node &d = nodes[id];
            Node &e = nodes[ie];
            b.left = ia;
            b.parent = a.parent;
            a.parent = ib;
            if (b.parent != null)
            {
                if (nodes[b.parent].left == ia)
                    nodes[b.parent].left = ib;
                else
                    nodes[b.parent].right = ib;
            }
            else
                root = ib;
            if (d.height > e.height)
            {
                b.right = id;
                a.left = ie;
                e.parent = ia;
            }
            else
            {
                b.right = ie;
                a.left = id;
                d.parent = ia;
            }
            a.bounds = aabb_union(c.bounds, nodes[a.left].bounds);
            a.height = 1 + std::max(nodes[a.left].height, nodes[a.right].height);
            return ib;
        }
        return ia;
    }
    // update_leaf (bvh.cpp:475-514): margin 0.1 m plus the displacement on its sign side.
    bool update_leaf(uint32_t leaf, const Aabb &true_b, V3 disp)
    {
        Aabb &fat = nodes[leaf].bounds;
        if (fat.contains(true_b)) return false;
        extract_leaf(leaf);
        constexpr double margin = 0.1;
        V3 mv{margin, margin, margin};
        Aabb nb{true_b.min - mv, true_b.max + mv};
        if (disp.x < 0.0) nb.min.x = nb.min.x + disp.x; else nb.max.x = nb.max.x + disp.x;
        if (disp.y < 0.0) nb.min.y = nb.min.y + disp.y; else nb.max.y = nb.max.y + disp.y;
        if (disp.z < 0.0) nb.min.z = nb.min.z + disp.z; else nb.max.z = nb.max.z + disp.z;
        nodes[leaf].bounds = nb;
        insert_leaf(leaf);
        refit_and_rotate(nodes[leaf].parent);
        return true;
    }
    // dynamic_bvh::raycast (bvh.h:402-450): depth first, the nearer child first
    template <class F> void raycast(const Ray &r, double max_d, F &&cb) const
    {
        if (root == null) return;
        std::array<uint32_t, 64> stack{};
        int sp = 0;
        stack[sp++] = root;
        while (sp > 0)
        {
            uint32_t ni = stack[--sp];
            const Node &nd = nodes[ni];
            double dn;
            if (!r.intersect_distance(nd.bounds, max_d, dn)) continue;
            if (nd.is_leaf())
            {
                cb(nd.data, dn);
                continue;
            }
            assert(sp + 1 < 64);
            double dl, dr;
            bool hl = r.intersect_distance(nodes[nd.left].bounds, max_d, dl);
            bool hr = r.intersect_distance(nodes[nd.right].bounds, max_d, dr);
            if (hl && hr)
            {
                if (dl > dr)
                {
                    stack[sp++] = nd.left;
                    stack[sp++] = nd.right;
                }
                else
                {
                    stack[sp++] = nd.right;
                    stack[sp++] = nd.left;
                }
            }
            else if (hl)
                stack[sp++] = nd.left;
            else if (hr)
                stack[sp++] = nd.right;
        }
    }
    template <class F> void query(const Aabb &box, F &&cb) const
    {
        if (root == null) return;
        std::array<uint32_t, 64> stack{};
        int sp = 0;
        stack[sp++] = root;
        while (sp > 0)
        {
            uint32_t ni = stack[--sp];
            const Node &nd = nodes[ni];
            if (!nd.bounds.intersects(box)) continue;
            if (nd.is_leaf())
            {
                if (!cb(nd.data)) return;
                continue;
            }
            assert(sp + 1 < 64);
            if (nodes[nd.left].bounds.surface_area() > nodes[nd.right].bounds.surface_area())
            {
                stack[sp++] = nd.left;
                stack[sp++] = nd.right;
            }
            else
            {
                stack[sp++] = nd.right;
                stack[sp++] = nd.left;
            }
        }
    }
    int height() const { return root == null ? -1 : static_cast<int>(nodes[root].height); }
    bool validate() const
    {
        if (root == null) return true;
        if (nodes[root].parent != null) return false;
        std::vector<uint32_t> st{root};
        while (!st.empty())
        {
            uint32_t n = st.back();
            st.pop_back();
            const Node &nd = nodes[n];
            if (nd.is_leaf()) continue;
            const Node &l = nodes[nd.left], &r = nodes[nd.right];
            if (l.parent != n || r.parent != n) return false;
            if (nd.height != 1 + std::max(l.height, r.height)) return false;
            Aabb u = aabb_union(l.bounds, r.bounds);
            if (!(u.min.x == nd.bounds.min.x && u.max.x == nd.bounds.max.x &&
                  u.min.y == nd.bounds.min.y && u.max.y == nd.bounds.max.y &&
                  u.min.z == nd.bounds.min.z && u.max.z == nd.bounds.max.z))
                return false;
            int bal = static_cast<int>(l.height) - static_cast<int>(r.height);
            if (bal > 1 || bal < -1) return false;
            st.push_back(nd.left);
            st.push_back(nd.right);
        }
        return true;
    }
};

// ---------------------------------------------------------------------------------------------
// Bodies (core/particle.h:16-146, core/object.h:111-144)
// ---------------------------------------------------------------------------------------------
struct Body
{
    V3 pos, vel, acc;
    double mass = 1, inv_mass = 1;
    V3 ang_vel, torque;
    Qt q;
    M3 I_l, I_l_inv, R, I_w, I_w_inv;
    std::shared_ptr<Mesh> mesh;
    bool is_static = false;
    double restitution = 0.5, friction = 0.5;
    uint32_t broad_handle = 0;

    void update_derived()
    {
        R = to_matrix(q);
        M3 rt = transpose(R);
        I_w = matmul(matmul(R, I_l), rt);
        I_w_inv = matmul(matmul(R, I_l_inv), rt);
    }
    V3 angular_accel() const
    {
        V3 c = cross(ang_vel, matvec(I_w, ang_vel));
        return matvec(I_w_inv, torque - c);
    }
    MeshInst instance() const { return {mesh.get(), pos, q}; }
    V3 to_local(V3 p) const { return rotate(conj(q), p - pos); }
    V3 to_world(V3 p) const { return rotate(q, p) + pos; }
};

// ---------------------------------------------------------------------------------------------
// Broadphase + narrowphase (collision/collision_phases.h:29-445)
// ---------------------------------------------------------------------------------------------
inline uint64_t pair_key(uint32_t a, uint32_t b)
{
    uint32_t lo = std::min(a, b), hi = std::max(a, b);
    return (static_cast<uint64_t>(lo) << 32) | hi;
}

struct ContactPoint
{
    V3 normal, local_a, local_b;
    double depth = 0;
};
struct ContactInfo
{
    ContactPoint point;
    double normal_impulse = 0;
    double tangent_impulse[2] = {0, 0};
};
struct Manifold
{
    std::array<ContactInfo, 4> c{};
    int n = 0;
    void add_contact(const ContactInfo &ci)
    {
        if (n < 4)
            c[n++] = ci;
        else
            add_reduce(ci);
    }
    // manifold::add_reduce (collision_phases.h:139-198)
    void add_reduce(const ContactInfo &np)
    {
        std::array<ContactInfo, 5> pool;
        for (int i = 0; i < 4; ++i) pool[i] = c[i];
        pool[4] = np;
        std::array<size_t, 4> best = {0, 1, 2, 3};
        for (size_t i = 1; i < 5; ++i)
            if (pool[i].point.depth > pool[best[0]].point.depth) best[0] = i;
        double md = -1.0;
        for (size_t i = 0; i < 5; ++i)
        {
            if (i == best[0]) continue;
            double d2 = sqnorm(pool[i].point.local_a - pool[best[0]].point.local_a);
            if (d2 > md)
            {
                md = d2;
                best[1] = i;
            }
        }
        double ma = -1.0;
        V3 e0 = pool[best[1]].point.local_a - pool[best[0]].point.local_a;
        for (size_t i = 0; i < 5; ++i)
        {
            if (i == best[0] || i == best[1]) continue;
            V3 e1 = pool[i].point.local_a - pool[best[0]].point.local_a;
            double a2 = sqnorm(cross(e0, e1));
            if (a2 > ma)
            {
                ma = a2;
                best[2] = i;
            }
        }
        md = -1.0;
        for (size_t i = 0; i < 5; ++i)
        {
            if (i == best[0] || i == best[1] || i == best[2]) continue;
            double d2 = sqnorm(pool[i].point.local_a - pool[best[2]].point.local_a);
            if (d2 > md)
            {
                md = d2;
                best[3] = i;
            }
        }
        n = 0;
        for (auto i : best) c[n++] = pool[i];
    }
};

struct Event
{
    uint64_t key;
    int kind;
};

// ---------------------------------------------------------------------------------------------
// Solver (collision/constraint.h:29-113, 867-953, 1024-1201)
// ---------------------------------------------------------------------------------------------
struct Row
{
    V3 J_v, J_w_a, J_w_b;
    double M_eff = 0, bias = 0, gamma = 0, acc = 0;
    double lo = -std::numeric_limits<double>::max(), hi = std::numeric_limits<double>::max();
    Body *a = nullptr, *b = nullptr;

    void apply()
    {
        double Jv = dot(J_v, a->vel) + dot(J_w_a, a->ang_vel) - dot(J_v, b->vel) + dot(J_w_b, b->ang_vel);
        double cfp = gamma * acc;
        double lambda = -(Jv + bias + cfp) * M_eff;
        double old = acc;
        double v = old + lambda;
        acc = (v < lo) ? lo : ((hi < v) ? hi : v); // std::clamp
        double applied = acc - old;
        if (!a->is_static)
        {
            a->vel = a->vel + (J_v * applied) * a->inv_mass;
            a->ang_vel = a->ang_vel + matvec(a->I_w_inv, J_w_a * applied);
        }
        if (!b->is_static)
        {
            b->vel = b->vel + ((-J_v) * applied) * b->inv_mass;
            b->ang_vel = b->ang_vel + matvec(b->I_w_inv, J_w_b * applied);
        }
    }
    void warm_start() const
    {
        if (acc == 0.0) return;
        if (!a->is_static)
        {
            a->vel = a->vel + (J_v * acc) * a->inv_mass;
            a->ang_vel = a->ang_vel + matvec(a->I_w_inv, J_w_a * acc);
        }
        if (!b->is_static)
        {
            b->vel = b->vel + ((-J_v) * acc) * b->inv_mass;
            b->ang_vel = b->ang_vel + matvec(b->I_w_inv, J_w_b * acc);
        }
    }
};

inline std::pair<V3, V3> orthonormal_basis(V3 n)
{
    double sign = std::copysign(1.0, n.z);
    double a = -1.0 / (sign + n.z);
    double b = n.x * n.y * a;
    return {V3{1.0 + sign * n.x * n.x * a, sign * b, -sign * n.x}, V3{b, sign + n.y * n.y * a, -n.y}};
}

struct ContactRows
{
    Row normal, t1, t2;
    double mu = 0, inv11 = 0, inv12 = 0, inv22 = 0;
    ContactInfo *cache = nullptr;
    int manifold = 0; // index of the owning manifold in the step's active list
};

// ---------------------------------------------------------------------------------------------
// joints (collision/constraint.h:139-865): per-world arenas per type, built into rows every step
// ---------------------------------------------------------------------------------------------
enum JointType
{
    J_DISTANCE = 0, // constraint_type order (constraint.h:15-24), which is also the arenas' order
    J_BALL_SOCKET,
    J_HINGE,
    J_SLIDER,
    J_WELD,
    J_SPRING,
    J_COUNT
};
constexpr int kJointRows[J_COUNT] = {1, 3, 5, 5, 6, 1}; // jacobian_dimension of each type

struct Joint
{
    int type = J_DISTANCE;
    uint32_t a = 0, b = 0; // body arena indices
    V3 la, lb;             // local anchors
    V3 axa, axb;           // hinge: local axes (normalised); slider: local axis of a
    V3 va, wa;             // hinge: orthonormal basis of axa; slider: local tangents of a
    Qt qrel;               // slider, weld: conj(q_a) q_b at creation
    double distance = 0, stiffness = 0, damping = 0;
    double acc[6] = {0, 0, 0, 0, 0, 0}; // accumulated impulses, kept for warm starting
};
struct JointSlot
{
    std::optional<Joint> value;
    uint32_t gen = 0;
};
struct JointRow
{
    Row row;
    double *dst; // the joint's accumulated impulse this row writes back
};

// The rows of one joint in the reference's build order (build_jacobian_impl of each type).
inline void build_joint_rows(Joint &j, Body &a, Body &b, double dt, std::vector<JointRow> &out)
{
    const V3 r_a = rotate(a.q, j.la), r_b = rotate(b.q, j.lb);
    auto linear = [&](V3 n, V3 arm_a, double bias_factor, V3 delta, double *acc, bool slider) {
        Row r;
        r.J_v = n;
        r.J_w_a = cross(arm_a, n);
        r.J_w_b = -cross(r_b, n);
        r.acc = *acc;
        r.a = &a;
        r.b = &b;
        V3 k_a = matvec(a.I_w_inv, r.J_w_a), k_b = matvec(b.I_w_inv, r.J_w_b);
        if (slider)
        {
            double lin = a.inv_mass + b.inv_mass;
            double ang = dot(r.J_w_a, k_a) + dot(r.J_w_b, k_b);
            double reg = 0.01 * ang;
            r.gamma = reg;
            r.M_eff = 1.0 / (lin + ang + reg);
            double e = dot(delta, n);
            e = (e < -0.2) ? -0.2 : ((0.2 < e) ? 0.2 : e); // std::clamp to +-0.2 m
            r.bias = (bias_factor / dt) * e;
        }
        else
        {
            r.M_eff = 1.0 / (a.inv_mass + b.inv_mass + dot(r.J_w_a, k_a) + dot(r.J_w_b, k_b));
            r.bias = (bias_factor / dt) * dot(delta, n);
        }
        out.push_back({r, acc});
    };
    auto angular = [&](V3 n, double bias_factor, V3 err, double *acc) {
        Row r;
        r.J_v = V3{0.0, 0.0, 0.0};
        r.J_w_a = n;
        r.J_w_b = -n;
        r.acc = *acc;
        r.a = &a;
        r.b = &b;
        V3 k_a = matvec(a.I_w_inv, r.J_w_a), k_b = matvec(b.I_w_inv, r.J_w_b);
        r.M_eff = 1.0 / (dot(r.J_w_a, k_a) + dot(r.J_w_b, k_b));
        r.bias = (bias_factor / dt) * dot(err, n);
        out.push_back({r, acc});
    };
    const V3 axes[3] = {V3{1.0, 0.0, 0.0}, V3{0.0, 1.0, 0.0}, V3{0.0, 0.0, 1.0}};
    switch (j.type)
    {
    case J_DISTANCE:
    case J_SPRING: {
        // distance_constraint / spring_constraint::build_jacobian_impl (constraint.h:187-231, 309-352)
        V3 delta = (a.pos + r_a) - (b.pos + r_b);
        double cur = norm(delta);
        if (cur < 1e-6) return;
        V3 u = delta / cur;
        Row r;
        r.J_v = u;
        r.J_w_a = cross(r_a, u);
        r.J_w_b = -cross(r_b, u);
        r.acc = j.acc[0];
        r.a = &a;
        r.b = &b;
        V3 k_a = matvec(a.I_w_inv, r.J_w_a), k_b = matvec(b.I_w_inv, r.J_w_b);
        if (j.type == J_DISTANCE)
        {
            r.M_eff = 1.0 / (a.inv_mass + b.inv_mass + dot(r.J_w_a, k_a) + dot(r.J_w_b, k_b));
            r.bias = (0.1 / dt) * (cur - j.distance);
        }
        else
        {
            double mc = a.inv_mass + b.inv_mass + dot(r.J_w_a, k_a) + dot(r.J_w_b, k_b);
            double gamma = 1.0 / (dt * (j.damping + dt * j.stiffness));
            double beta = dt * j.stiffness / (j.damping + dt * j.stiffness);
            r.M_eff = 1.0 / (mc + gamma);
            r.bias = (beta / dt) * (cur - j.distance);
            r.gamma = gamma;
        }
        out.push_back({r, &j.acc[0]});
        return;
    }
    case J_BALL_SOCKET: {
        // ball_socket_constraint::build_jacobian_impl (constraint.h:407-446)
        V3 delta = (a.pos + r_a) - (b.pos + r_b);
        for (int k = 0; k < 3; ++k) linear(axes[k], r_a, 0.1, delta, &j.acc[k], false);
        return;
    }
    case J_HINGE: {
        // hinge_constraint::build_jacobian_impl (constraint.h:512-580)
        V3 delta = (a.pos + r_a) - (b.pos + r_b);
        for (int k = 0; k < 3; ++k) linear(axes[k], r_a, 0.2, delta, &j.acc[k], false);
        V3 u_a = rotate(a.q, j.axa), u_b = rotate(b.q, j.axb);
        V3 err = -cross(u_a, u_b);
        angular(rotate(a.q, j.va), 0.2, err, &j.acc[3]);
        angular(rotate(a.q, j.wa), 0.2, err, &j.acc[4]);
        return;
    }
    case J_SLIDER: {
        // slider_constraint::build_jacobian_impl (constraint.h:654-738)
        V3 delta = (a.pos + r_a) - (b.pos + r_b);
        V3 axis_a = rotate(a.q, j.axa);
        V3 t1 = rotate(a.q, j.va), t2 = rotate(a.q, j.wa);
        V3 lever = r_a - delta;
        linear(t1, lever, 0.1, delta, &j.acc[0], true);
        linear(t2, lever, 0.1, delta, &j.acc[1], true);
        Qt cur = qmul(conj(a.q), b.q);
        Qt e = qmul(j.qrel, conj(cur));
        if (e.w < 0) e = Qt{-e.w, -e.x, -e.y, -e.z};
        V3 err = rotate(a.q, V3{e.x, e.y, e.z} * 2.0);
        angular(axis_a, 0.1, err, &j.acc[2]);
        angular(t1, 0.1, err, &j.acc[3]);
        angular(t2, 0.1, err, &j.acc[4]);
        return;
    }
    case J_WELD: {
        // weld_constraint::build_jacobian_impl (constraint.h:789-855)
        V3 delta = (a.pos + r_a) - (b.pos + r_b);
        for (int k = 0; k < 3; ++k) linear(axes[k], r_a, 0.1, delta, &j.acc[k], false);
        Qt cur = qmul(conj(a.q), b.q);
        Qt e = qmul(j.qrel, conj(cur));
        if (e.w < 0) e = Qt{-e.w, -e.x, -e.y, -e.z};
        V3 err = rotate(a.q, V3{e.x, e.y, e.z} * 2.0);
        for (int k = 0; k < 3; ++k) angular(axes[k], 0.1, err, &j.acc[3 + k]);
        return;
    }
    default:
        return;
    }
}

// build_contact_jacobian (constraint.h:874-953)
std::optional<ContactRows> build_contact(Body &a, Body &b, V3 la, V3 lb, V3 wn, double dt, double rthr)
{
    constexpr double beta = 0.1, slop = 0.005;
    V3 nn = normalized(wn);
    V3 ln_b = rotate(conj(b.q), nn);
    V3 r_a = rotate(a.q, la);
    V3 r_b = rotate(b.q, lb);
    V3 n = rotate(b.q, ln_b);
    double pen = dot((b.pos + r_b) - (a.pos + r_a), n);
    if (pen <= 0.0) return std::nullopt;
    ContactRows res;
    {
        Row row;
        row.J_v = n;
        row.J_w_a = cross(r_a, n);
        row.J_w_b = -cross(r_b, n);
        row.lo = 0.0;
        row.a = &a;
        row.b = &b;
        V3 ka = matvec(a.I_w_inv, row.J_w_a);
        V3 kb = matvec(b.I_w_inv, row.J_w_b);
        row.M_eff = 1.0 / (a.inv_mass + b.inv_mass + dot(row.J_w_a, ka) + dot(row.J_w_b, kb));
        V3 vca = a.vel + cross(a.ang_vel, r_a);
        V3 vcb = b.vel + cross(b.ang_vel, r_b);
        double vreln = dot(vca - vcb, n);
        double e = dmax(a.restitution, b.restitution);
        double rbias = 0.0;
        if (vreln < -rthr) rbias = e * vreln;
        double bbias = (-beta / dt) * dmax(0.0, pen - slop);
        row.bias = dmin(bbias, rbias);
        res.normal = row;
    }
    auto tangent = [&](V3 t)
    {
        Row row;
        row.J_v = t;
        row.J_w_a = cross(r_a, t);
        row.J_w_b = -cross(r_b, t);
        row.bias = 0.0;
        row.a = &a;
        row.b = &b;
        V3 ka = matvec(a.I_w_inv, row.J_w_a);
        V3 kb = matvec(b.I_w_inv, row.J_w_b);
        row.M_eff = 1.0 / (a.inv_mass + b.inv_mass + dot(row.J_w_a, ka) + dot(row.J_w_b, kb));
        return row;
    };
    auto [t1, t2] = orthonormal_basis(n);
    res.t1 = tangent(t1);
    res.t2 = tangent(t2);
    return res;
}

// Deterministic colouring of the step's active manifolds (in key order), as the device solver
// colours them. A world of at most 4,096 arena slots is coloured first-fit: each manifold takes
// the lowest colour that no earlier manifold on one of its dynamic bodies has, unless that needs a
// colour above 127. Other worlds are coloured by rounds of parallel first fit: in each round every
// uncoloured manifold picks the lowest colour (below 128) taken on neither of its dynamic bodies,
// and claims both bodies with the key (colour, scramble of the pair's arena indices, index in key
// order) (ff_key); the manifolds that hold the lowest key on all their dynamic bodies keep their
// colour. Where a body would need a colour above 127 there too, the world is coloured by min-index
// claiming rounds: in each round every uncoloured manifold claims its dynamic bodies with its
// index, and the manifolds that won all their dynamic bodies take the round number as colour.
static uint64_t ff_key(int colour, uint32_t la, uint32_t lb, uint32_t pos)
{
    const uint32_t lo = std::min(la, lb), hi = std::max(la, lb);
    uint64_t x = (uint64_t(lo) << 32) | hi;
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return (uint64_t(uint32_t(colour)) << 56) | ((x >> 40) << 32) | pos;
}

static bool colour_first_fit_rounds(const std::vector<std::pair<uint32_t, uint32_t>> &bodies,
                                    const std::vector<std::pair<bool, bool>> &stat, size_t nslots,
                                    std::vector<int> &col, int *ncolours)
{
    const size_t m = bodies.size();
    std::vector<std::array<uint64_t, 2>> used(nslots, {0ull, 0ull});
    std::vector<uint64_t> owner(nslots, ~0ull);
    std::vector<int> tcol(m, 0);
    std::fill(col.begin(), col.end(), -1);
    size_t left = m;
    int top = 0;
    for (int round = 0; left > 0; ++round)
    {
        if (round >= 512) return false;
        for (size_t i = 0; i < m; ++i)
        {
            if (col[i] >= 0) continue;
            uint64_t u0 = 0ull, u1 = 0ull;
            for (auto [b, st] : {std::pair<uint32_t, bool>{bodies[i].first, stat[i].first},
                                 std::pair<uint32_t, bool>{bodies[i].second, stat[i].second}})
            {
                if (st) continue;
                u0 |= used[b][0];
                u1 |= used[b][1];
                owner[b] = ~0ull;
            }
            int c = -1;
            for (int k = 0; k < 128 && c < 0; ++k)
                if (!((((k < 64) ? u0 : u1) >> (k & 63)) & 1ull)) c = k;
            if (c < 0) return false; // a body with all 128 colours taken
            tcol[i] = c;
        }
        for (size_t i = 0; i < m; ++i)
        {
            if (col[i] >= 0) continue;
            const uint64_t key = ff_key(tcol[i], bodies[i].first, bodies[i].second, uint32_t(i));
            if (!stat[i].first) owner[bodies[i].first] = std::min(owner[bodies[i].first], key);
            if (!stat[i].second) owner[bodies[i].second] = std::min(owner[bodies[i].second], key);
        }
        for (size_t i = 0; i < m; ++i)
        {
            if (col[i] >= 0) continue;
            const uint64_t key = ff_key(tcol[i], bodies[i].first, bodies[i].second, uint32_t(i));
            if ((stat[i].first || owner[bodies[i].first] == key) && (stat[i].second || owner[bodies[i].second] == key))
            {
                const int c = tcol[i];
                col[i] = c;
                for (auto [b, st] : {std::pair<uint32_t, bool>{bodies[i].first, stat[i].first},
                                     std::pair<uint32_t, bool>{bodies[i].second, stat[i].second}})
                    if (!st) used[b][size_t(c >> 6)] |= 1ull << (c & 63);
                top = std::max(top, c + 1);
                --left;
            }
        }
    }
    *ncolours = top;
    return true;
}

std::vector<int> colour_manifolds(const std::vector<std::pair<uint32_t, uint32_t>> &bodies,
                                  const std::vector<std::pair<bool, bool>> &stat, size_t nslots,
                                  int *ncolours)
{
    size_t m = bodies.size();
    std::vector<int> col(m, -1);
    if (nslots <= 4096)
    {
        std::vector<std::vector<bool>> used(nslots);
        int top = 0;
        for (size_t i = 0; i < m; ++i)
        {
            auto taken = [&](uint32_t b, bool st, int c)
            { return !st && size_t(c) < used[b].size() && used[b][size_t(c)]; };
            int c = 0;
            while (taken(bodies[i].first, stat[i].first, c) || taken(bodies[i].second, stat[i].second, c)) ++c;
            col[i] = c;
            for (auto [b, st] : {std::pair<uint32_t, bool>{bodies[i].first, stat[i].first},
                                 std::pair<uint32_t, bool>{bodies[i].second, stat[i].second}})
            {
                if (st) continue;
                if (used[b].size() <= size_t(c)) used[b].resize(size_t(c) + 1, false);
                used[b][size_t(c)] = true;
            }
            top = std::max(top, c + 1);
        }
        if (top <= 128)
        {
            *ncolours = top;
            return col;
        }
        std::fill(col.begin(), col.end(), -1);
    }
    if (colour_first_fit_rounds(bodies, stat, nslots, col, ncolours)) return col;
    std::fill(col.begin(), col.end(), -1);
    std::vector<uint32_t> owner(nslots, 0xFFFFFFFFu);
    size_t left = m;
    int round = 0;
    while (left > 0)
    {
        std::fill(owner.begin(), owner.end(), 0xFFFFFFFFu);
        for (size_t i = 0; i < m; ++i)
        {
            if (col[i] >= 0) continue;
            if (!stat[i].first) owner[bodies[i].first] = std::min<uint32_t>(owner[bodies[i].first], i);
            if (!stat[i].second) owner[bodies[i].second] = std::min<uint32_t>(owner[bodies[i].second], i);
        }
        for (size_t i = 0; i < m; ++i)
        {
            if (col[i] >= 0) continue;
            bool ok = (stat[i].first || owner[bodies[i].first] == i) &&
                      (stat[i].second || owner[bodies[i].second] == i);
            if (ok)
            {
                col[i] = round;
                --left;
            }
        }
        ++round;
    }
    *ncolours = round;
    return col;
}

// ---------------------------------------------------------------------------------------------
// World (core/world.h:184-425, src/world.cpp:20-56)
// ---------------------------------------------------------------------------------------------
struct Slot
{
    std::optional<Body> value;
    uint32_t gen = 0;
};

struct World
{
    V3 gravity{0.0, -9.81, 0.0};
    double gravity_norm = 9.81;
    int iterations = 10;
    int order = PKO_ORDER_KEY;
    std::vector<std::shared_ptr<Mesh>> shapes;

    std::vector<Slot> slots;
    std::vector<uint32_t> free_stack;

    DynTree static_tree, dynamic_tree;
    std::array<std::vector<JointSlot>, J_COUNT> joints;
    std::array<std::vector<uint32_t>, J_COUNT> joint_free;
    std::vector<uint32_t> moved;
    std::unordered_set<uint64_t> pairs;
    std::map<uint64_t, Manifold> manifolds; // narrow_phase store, iterated in key order
    std::vector<Event> events;

    // last-step diagnostics
    std::vector<uint64_t> colour_keys;
    std::vector<int> colours;
    int ncolours = 0;
    int last_moved = 0;

    uint32_t next_index() const
    {
        return free_stack.empty() ? static_cast<uint32_t>(slots.size()) : free_stack.back();
    }
    Body *get(uint32_t idx) { return slots[idx].value ? &*slots[idx].value : nullptr; }

    // world_base::create_rigid (world.h:202-208)
    uint64_t create(Body b)
    {
        uint32_t idx = next_index();
        MeshInst inst = b.instance();
        if (b.is_static)
            b.broad_handle = static_tree.add(idx, inst.bounds());
        else
            b.broad_handle = dynamic_tree.add(idx, inst.bounds());
        uint32_t gen;
        if (free_stack.empty())
        {
            slots.push_back({});
            slots.back().value.emplace(std::move(b));
            gen = 0;
        }
        else
        {
            free_stack.pop_back();
            slots[idx].value.emplace(std::move(b));
            gen = slots[idx].gen;
        }
        return static_cast<uint64_t>(idx) | (static_cast<uint64_t>(gen) << 32);
    }
    // constraint_solver::add_constraint via the world's command (world.h:155-166): the joint is
    // built from the bodies' current poses (constructors, constraint.h:183-187, 386-392, 494-500,
    // 635-652, 779-785)
    uint64_t add_joint(int type, uint64_t ha, uint64_t hb, V3 anchor, V3 la, V3 lb, V3 axis_a, V3 axis_b,
                       double distance, double stiffness, double damping)
    {
        uint32_t ia = static_cast<uint32_t>(ha & 0xFFFFFFFFu), ib = static_cast<uint32_t>(hb & 0xFFFFFFFFu);
        Body &a = *get(ia);
        Body &b = *get(ib);
        Joint j;
        j.type = type;
        j.a = ia;
        j.b = ib;
        j.distance = distance;
        j.stiffness = stiffness;
        j.damping = damping;
        switch (type)
        {
        case J_DISTANCE:
        case J_SPRING:
            j.la = la;
            j.lb = lb;
            break;
        case J_BALL_SOCKET:
        case J_WELD:
            j.la = a.to_local(anchor);
            j.lb = b.to_local(anchor);
            j.qrel = qmul(conj(a.q), b.q);
            break;
        case J_HINGE: {
            j.la = la;
            j.lb = lb;
            j.axa = normalized(axis_a);
            j.axb = normalized(axis_b);
            auto t = orthonormal_basis(j.axa);
            j.va = t.first;
            j.wa = t.second;
            break;
        }
        case J_SLIDER: {
            j.la = a.to_local(anchor);
            j.lb = b.to_local(anchor);
            V3 n = normalized(axis_a);
            j.axa = rotate(conj(a.q), n);
            auto t = orthonormal_basis(n);
            j.va = rotate(conj(a.q), t.first);
            j.wa = rotate(conj(a.q), t.second);
            j.qrel = qmul(conj(a.q), b.q);
            break;
        }
        default:
            return ~uint64_t(0);
        }
        auto &ar = joints[static_cast<size_t>(type)];
        auto &fr = joint_free[static_cast<size_t>(type)];
        uint32_t idx, gen;
        if (fr.empty())
        {
            idx = static_cast<uint32_t>(ar.size());
            ar.push_back({});
            ar.back().value.emplace(j);
            gen = 0;
        }
        else
        {
            idx = fr.back();
            fr.pop_back();
            ar[idx].value.emplace(j);
            gen = ar[idx].gen;
        }
        return static_cast<uint64_t>(idx) | (static_cast<uint64_t>(gen & 0xFFFFFFu) << 32) |
               (static_cast<uint64_t>(type) << 56);
    }
    bool remove_joint(uint64_t h)
    {
        int type = static_cast<int>(h >> 56);
        uint32_t idx = static_cast<uint32_t>(h & 0xFFFFFFFFu), gen = static_cast<uint32_t>((h >> 32) & 0xFFFFFFu);
        if (type < 0 || type >= J_COUNT) return false;
        auto &ar = joints[static_cast<size_t>(type)];
        if (idx >= ar.size() || !ar[idx].value || (ar[idx].gen & 0xFFFFFFu) != gen) return false;
        ar[idx].value.reset();
        ar[idx].gen++;
        joint_free[static_cast<size_t>(type)].push_back(idx);
        return true;
    }
    const Joint *joint(uint64_t h) const
    {
        int type = static_cast<int>(h >> 56);
        uint32_t idx = static_cast<uint32_t>(h & 0xFFFFFFFFu);
        if (type < 0 || type >= J_COUNT || idx >= joints[static_cast<size_t>(type)].size()) return nullptr;
        const auto &s = joints[static_cast<size_t>(type)][idx];
        return s.value ? &*s.value : nullptr;
    }

    // world_base::raycast (world.h:260-319): both trees' hits, merged by their current distance
    // (static first on a tie), as (handle, distance)
    std::vector<std::pair<uint64_t, double>> raycast(V3 origin, V3 dir, double max_d) const
    {
        Ray r(origin, dir);
        std::vector<std::pair<uint32_t, double>> sh, dh;
        static_tree.raycast(r, max_d, [&](uint32_t id, double t) { sh.push_back({id, t}); });
        dynamic_tree.raycast(r, max_d, [&](uint32_t id, double t) { dh.push_back({id, t}); });
        auto handle = [&](uint32_t idx) { return static_cast<uint64_t>(idx) | (static_cast<uint64_t>(slots[idx].gen) << 32); };
        std::vector<std::pair<uint64_t, double>> out;
        size_t i = 0, j = 0;
        while (i < sh.size() && j < dh.size())
        {
            if (sh[i].second <= dh[j].second)
            {
                out.push_back({handle(sh[i].first), sh[i].second});
                ++i;
            }
            else
            {
                out.push_back({handle(dh[j].first), dh[j].second});
                ++j;
            }
        }
        for (; i < sh.size(); ++i) out.push_back({handle(sh[i].first), sh[i].second});
        for (; j < dh.size(); ++j) out.push_back({handle(dh[j].first), dh[j].second});
        return out;
    }
    // world_base::remove_rigid (world.h:209-218) -> broad_phase::remove (collision_phases.h:350-369)
    bool remove(uint64_t h)
    {
        uint32_t idx = static_cast<uint32_t>(h & 0xFFFFFFFFu), gen = static_cast<uint32_t>(h >> 32);
        if (idx >= slots.size()) return false;
        Slot &s = slots[idx];
        if (s.gen != gen || !s.value) return false;
        s.gen++;
        free_stack.push_back(idx);
        Body b = std::move(*s.value);
        s.value.reset();
        if (b.is_static)
            static_tree.remove_leaf(b.broad_handle);
        else
        {
            dynamic_tree.remove_leaf(b.broad_handle);
            moved.erase(std::remove(moved.begin(), moved.end(), b.broad_handle), moved.end());
        }
        for (auto it = pairs.begin(); it != pairs.end();)
        {
            uint32_t a = static_cast<uint32_t>(*it >> 32), c = static_cast<uint32_t>(*it & 0xFFFFFFFFu);
            if (a == idx || c == idx)
            {
                manifolds.erase(*it);
                it = pairs.erase(it);
            }
            else
                ++it;
        }
        return true;
    }

    const Aabb &tree_bounds(uint32_t idx)
    {
        Body &b = *get(idx);
        return b.is_static ? static_tree.nodes[b.broad_handle].bounds
                           : dynamic_tree.nodes[b.broad_handle].bounds;
    }

    // broad_phase::calculate_pairs (collision_phases.h:377-436)
    void calculate_pairs()
    {
        // Removal pass (hash-set order in the reference; set semantics are order-independent).
        for (auto it = pairs.begin(); it != pairs.end();)
        {
            uint32_t a = static_cast<uint32_t>(*it >> 32), b = static_cast<uint32_t>(*it & 0xFFFFFFFFu);
            if (!tree_bounds(a).intersects(tree_bounds(b)))
            {
                manifolds.erase(*it);
                it = pairs.erase(it);
            }
            else
                ++it;
        }
        for (uint32_t leaf : moved)
        {
            const Aabb mb = dynamic_tree.nodes[leaf].bounds;
            uint32_t ea = dynamic_tree.nodes[leaf].data;
            auto cb = [&](uint32_t eb)
            {
                if (ea != eb)
                {
                    uint64_t k = pair_key(ea, eb);
                    if (pairs.insert(k).second) manifolds.emplace(k, Manifold{});
                }
                return true;
            };
            dynamic_tree.query(mb, cb);
            static_tree.query(mb, cb);
        }
        moved.clear();
    }

    // narrow_phase::calculate (collision_phases.h:244-320)
    void narrow()
    {
        constexpr double d2eps = 0.005 * 0.005;
        constexpr double breaking = 0.05;
        constexpr double drift2_eps = 0.06;
        events.clear();
        for (auto &[key, man] : manifolds)
        {
            uint32_t ia = static_cast<uint32_t>(key >> 32), ib = static_cast<uint32_t>(key & 0xFFFFFFFFu);
            Body &a = *get(ia);
            Body &b = *get(ib);
            auto col = gjk_epa(a.instance(), b.instance());
            std::optional<ContactInfo> nc;
            if (col)
            {
                ContactInfo ci;
                ci.point.normal = col->normal;
                ci.point.local_a = a.to_local(col->world_a);
                ci.point.local_b = b.to_local(col->world_b);
                ci.point.depth = col->depth;
                nc = ci;
            }
            Manifold nm;
            for (int k = 0; k < man.n; ++k)
            {
                ContactInfo old = man.c[k];
                if (nc)
                {
                    if (sqnorm(nc->point.local_a - old.point.local_a) < d2eps ||
                        sqnorm(nc->point.local_b - old.point.local_b) < d2eps)
                    {
                        nc->normal_impulse = old.normal_impulse;
                        nc->tangent_impulse[0] = old.tangent_impulse[0];
                        nc->tangent_impulse[1] = old.tangent_impulse[1];
                        continue;
                    }
                }
                V3 wa = a.to_world(old.point.local_a);
                V3 wb = b.to_world(old.point.local_b);
                V3 normal = nc ? nc->point.normal : old.point.normal;
                V3 rel = wb - wa;
                double depth = dot(rel, normal);
                V3 pa = wa + normal * depth;
                double drift2 = sqnorm(pa - wb);
                if (depth > -breaking && drift2 < drift2_eps)
                {
                    old.point.depth = depth;
                    old.point.normal = normal;
                    nm.add_contact(old);
                }
            }
            if (nc) nm.add_contact(*nc);
            bool was = man.n != 0, is = nm.n != 0;
            man = nm;
            if (!was && is)
                events.push_back({key, 1});
            else if (was && !is)
                events.push_back({key, 2});
        }
    }

    // constraint_solver::setup_contacts + solve_constraints (constraint.h:1052-1201)
    void solve(double dt)
    {
        double rthr = 2.0 * gravity_norm * dt;
        std::vector<ContactRows> rows;
        std::vector<uint64_t> active_keys;
        std::vector<std::pair<uint32_t, uint32_t>> mbodies;
        std::vector<std::pair<bool, bool>> mstatic;
        for (auto &[key, man] : manifolds)
        {
            if (man.n == 0) continue;
            uint32_t ia = static_cast<uint32_t>(key >> 32), ib = static_cast<uint32_t>(key & 0xFFFFFFFFu);
            Body &a = *get(ia);
            Body &b = *get(ib);
            size_t before = rows.size();
            for (int k = 0; k < man.n; ++k)
            {
                ContactInfo &ct = man.c[k];
                auto j = build_contact(a, b, ct.point.local_a, ct.point.local_b, ct.point.normal, dt, rthr);
                if (!j) continue;
                ContactRows p = *j;
                p.mu = std::sqrt(a.friction * b.friction);
                p.cache = &ct;
                double m11 = 1.0 / p.t1.M_eff;
                double m22 = 1.0 / p.t2.M_eff;
                double m12 = dot(p.t1.J_w_a, matvec(a.I_w_inv, p.t2.J_w_a)) +
                             dot(p.t1.J_w_b, matvec(b.I_w_inv, p.t2.J_w_b));
                double det = m11 * m22 - m12 * m12;
                if (det > 0.0)
                {
                    p.inv11 = m22 / det;
                    p.inv22 = m11 / det;
                    p.inv12 = -m12 / det;
                }
                else
                {
                    p.inv11 = p.t1.M_eff;
                    p.inv22 = p.t2.M_eff;
                    p.inv12 = 0.0;
                }
                p.normal.acc = ct.normal_impulse;
                p.t1.acc = ct.tangent_impulse[0];
                p.t2.acc = ct.tangent_impulse[1];
                p.manifold = static_cast<int>(active_keys.size());
                rows.push_back(p);
            }
            if (rows.size() > before)
            {
                active_keys.push_back(key);
                mbodies.push_back({ia, ib});
                mstatic.push_back({a.is_static, b.is_static});
            }
        }

        // Row order: key order, or colour-major with manifolds ascending inside a colour.
        std::vector<size_t> order(rows.size());
        for (size_t i = 0; i < rows.size(); ++i) order[i] = i;
        colour_keys = active_keys;
        if (this->order == PKO_ORDER_COLOUR)
        {
            colours = colour_manifolds(mbodies, mstatic, slots.size(), &ncolours);
            std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y)
                             { return colours[rows[x].manifold] < colours[rows[y].manifold]; });
        }
        else
        {
            colours.assign(active_keys.size(), 0);
            ncolours = active_keys.empty() ? 0 : 1;
        }

        // joint rows: every arena in type order, slots in index order (constraint.h:1109-1119)
        std::vector<JointRow> jrows;
        for (int t = 0; t < J_COUNT; ++t)
            for (auto &js : joints[static_cast<size_t>(t)])
                if (js.value) build_joint_rows(*js.value, *get(js.value->a), *get(js.value->b), dt, jrows);

        for (auto &jr : jrows) jr.row.warm_start();
        for (size_t oi : order)
        {
            rows[oi].normal.warm_start();
            rows[oi].t1.warm_start();
            rows[oi].t2.warm_start();
        }
        for (int it = 0; it < iterations; ++it)
        {
            for (auto &jr : jrows) jr.row.apply();
            for (size_t oi : order)
            {
                ContactRows &pt = rows[oi];
                pt.normal.apply();
                double maxf = pt.mu * pt.normal.acc;
                Row &t1 = pt.t1;
                Row &t2 = pt.t2;
                double Jv1 = dot(t1.J_v, t1.a->vel) + dot(t1.J_w_a, t1.a->ang_vel) - dot(t1.J_v, t1.b->vel) +
                             dot(t1.J_w_b, t1.b->ang_vel);
                double Jv2 = dot(t2.J_v, t2.a->vel) + dot(t2.J_w_a, t2.a->ang_vel) - dot(t2.J_v, t2.b->vel) +
                             dot(t2.J_w_b, t2.b->ang_vel);
                double b1 = Jv1 + t1.bias, b2 = Jv2 + t2.bias;
                double l1 = -(pt.inv11 * b1 + pt.inv12 * b2);
                double l2 = -(pt.inv12 * b1 + pt.inv22 * b2);
                double o1 = t1.acc, o2 = t2.acc;
                double n1 = o1 + l1, n2 = o2 + l2;
                double mag = hypot_det(n1, n2);
                if (mag > maxf)
                {
                    n1 = n1 * (maxf / mag);
                    n2 = n2 * (maxf / mag);
                }
                t1.acc = n1;
                t2.acc = n2;
                double a1 = n1 - o1, a2 = n2 - o2;
                if (!t1.a->is_static)
                {
                    t1.a->vel = t1.a->vel + (t1.J_v * a1 + t2.J_v * a2) * t1.a->inv_mass;
                    t1.a->ang_vel = t1.a->ang_vel + matvec(t1.a->I_w_inv, t1.J_w_a * a1 + t2.J_w_a * a2);
                }
                if (!t1.b->is_static)
                {
                    t1.b->vel = t1.b->vel + ((-t1.J_v) * a1 - t2.J_v * a2) * t1.b->inv_mass;
                    t1.b->ang_vel = t1.b->ang_vel + matvec(t1.b->I_w_inv, t1.J_w_b * a1 + t2.J_w_b * a2);
                }
            }
        }
        for (auto &pt : rows)
        {
            pt.cache->normal_impulse = pt.normal.acc;
            pt.cache->tangent_impulse[0] = pt.t1.acc;
            pt.cache->tangent_impulse[1] = pt.t2.acc;
        }
        for (auto &jr : jrows) *jr.dst = jr.row.acc;
    }

    // world::step_impl (src/world.cpp:20-56)
    void step(double dt)
    {
        int nm = 0;
        for (uint32_t i = 0; i < slots.size(); ++i)
        {
            if (!slots[i].value || slots[i].value->is_static) continue;
            Body &o = *slots[i].value;
            // apply_force(g*m) then integrate_vel (particle.h:78-79, integrate.h:36-40)
            V3 f = gravity * o.mass;
            o.acc = o.acc + f * o.inv_mass;
            o.vel = o.vel + o.acc * dt;
            o.ang_vel = o.ang_vel + o.angular_accel() * dt;
            if (dynamic_tree.update_leaf(o.broad_handle, o.instance().bounds(), o.vel * dt))
            {
                moved.push_back(o.broad_handle);
                ++nm;
            }
            o.acc = V3{};
            o.torque = V3{};
        }
        last_moved = nm;
        calculate_pairs();
        narrow();
        solve(dt);
        for (uint32_t i = 0; i < slots.size(); ++i)
        {
            if (!slots[i].value || slots[i].value->is_static) continue;
            Body &o = *slots[i].value;
            // integrate_pos (integrate.h:42-46) with detail::exp (integrate.h:20-31)
            o.pos = o.pos + o.vel * dt;
            V3 angle = o.ang_vel * dt;
            double mag = norm(angle);
            Qt dq;
            if (mag < 1e-12)
            {
                V3 half = angle * 0.5;
                dq = qnormalized(Qt{1.0, half.x, half.y, half.z});
            }
            else
            {
                V3 axis = angle / mag;
                double s, c;
                sincos_det(0.5 * mag, &s, &c);
                dq = Qt{c, s * axis.x, s * axis.y, s * axis.z};
            }
            o.q = qmul(dq, o.q);
            o.update_derived();
        }
    }
};

} // namespace ora

using namespace ora;

struct pko_world
{
    World w;
};
struct pko_tree
{
    DynTree t;
};

static Aabb aabb_from(const double *p) { return {{p[0], p[1], p[2]}, {p[3], p[4], p[5]}}; }
static Obb obb_from(const double *p)
{ return {{p[0], p[1], p[2]}, {p[3], p[4], p[5], p[6]}, {p[7], p[8], p[9]}}; }

template <class A>
static std::optional<CollisionInfo> dispatch_b(pko_world *w, const A &a, int kb, const double *pb, int sb)
{
    switch (kb)
    {
    case 0: return gjk_epa(a, aabb_from(pb));
    case 1: return gjk_epa(a, obb_from(pb));
    default:
        return gjk_epa(a, MeshInst{w->w.shapes[sb].get(), {pb[0], pb[1], pb[2]}, {pb[3], pb[4], pb[5], pb[6]}});
    }
}


extern "C" {

pko_world *pko_world_create(double gx, double gy, double gz, int iters, int order)
{
    auto *pw = new pko_world;
    pw->w.gravity = {gx, gy, gz};
    pw->w.gravity_norm = norm(pw->w.gravity);
    pw->w.iterations = iters;
    pw->w.order = order;
    return pw;
}
void pko_world_destroy(pko_world *w) { delete w; }

static int add_shape(pko_world *w, std::shared_ptr<Mesh> m)
{
    w->w.shapes.push_back(std::move(m));
    return static_cast<int>(w->w.shapes.size() - 1);
}
int pko_shape_box(pko_world *w, double hx, double hy, double hz) { return add_shape(w, mesh_box(hx, hy, hz)); }
int pko_shape_sphere(pko_world *w, double r, int stacks, int sectors)
{
    if (stacks < 2 || sectors < 3) return -1;
    return add_shape(w, mesh_sphere(r, static_cast<unsigned>(stacks), static_cast<unsigned>(sectors)));
}
int pko_shape_pyramid(pko_world *w, double b, double h) { return add_shape(w, mesh_pyramid(b, h)); }
int pko_shape_mesh(pko_world *w, const double *v, int nv, const int *t, int nt)
{
    if (nv <= 0 || nt <= 0) return -1;
    std::vector<V3> vv(static_cast<size_t>(nv));
    for (int i = 0; i < nv; ++i) vv[i] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
    std::vector<std::array<unsigned, 3>> tt(static_cast<size_t>(nt));
    for (int i = 0; i < nt; ++i)
        tt[i] = {static_cast<unsigned>(t[3 * i]), static_cast<unsigned>(t[3 * i + 1]), static_cast<unsigned>(t[3 * i + 2])};
    return add_shape(w, make_mesh(std::move(vv), std::move(tt)));
}
int pko_shape_vertex_count(pko_world *w, int s) { return static_cast<int>(w->w.shapes[s]->verts.size()); }
int pko_shape_triangles(pko_world *w, int s, int *out, int cap)
{
    const auto &t = w->w.shapes[size_t(s)]->tris;
    for (size_t i = 0; i < t.size() && int(i) < cap; ++i)
        for (int k = 0; k < 3; ++k) out[3 * i + size_t(k)] = int(t[i][size_t(k)]);
    return int(t.size());
}
int pko_shape_vertices(pko_world *w, int s, double *out, int cap)
{
    auto &v = w->w.shapes[s]->verts;
    int n = static_cast<int>(v.size());
    for (int i = 0; i < n && i < cap; ++i)
    {
        out[3 * i] = v[i].x;
        out[3 * i + 1] = v[i].y;
        out[3 * i + 2] = v[i].z;
    }
    return n;
}
double pko_shape_volume(pko_world *w, int s) { return w->w.shapes[s]->volume(); }

uint64_t pko_body_add(pko_world *w, int is_static, const double *pos, const double *quat, const double *vel,
                      const double *ang_vel, double mass, const double *inertia, double restitution,
                      double friction, int shape)
{
    if (shape < 0 || shape >= static_cast<int>(w->w.shapes.size())) return UINT64_MAX;
    Body b;
    b.pos = {pos[0], pos[1], pos[2]};
    b.q = {quat[0], quat[1], quat[2], quat[3]};
    b.vel = {vel[0], vel[1], vel[2]};
    b.ang_vel = {ang_vel[0], ang_vel[1], ang_vel[2]};
    b.is_static = is_static != 0;
    // object_desc::mass (object.h:81-85): static bodies have infinite mass.
    b.mass = b.is_static ? std::numeric_limits<double>::infinity() : mass;
    b.inv_mass = 1.0 / b.mass;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) b.I_l.m[i][j] = inertia[3 * i + j];
    b.I_l_inv = inverse(b.I_l);
    if (b.inv_mass == 0.0) b.I_l_inv = M3{};
    b.update_derived();
    b.mesh = w->w.shapes[shape];
    b.restitution = restitution;
    b.friction = friction;
    return w->w.create(std::move(b));
}
int pko_body_remove(pko_world *w, uint64_t h) { return w->w.remove(h) ? 1 : 0; }
int pko_body_count(pko_world *w) { return static_cast<int>(w->w.slots.size()); }

void pko_world_step(pko_world *w, double dt) { w->w.step(dt); }

int pko_read_bodies(pko_world *w, double *out, int cap)
{
    int n = static_cast<int>(w->w.slots.size());
    for (int i = 0; i < n && i < cap; ++i)
    {
        double *o = out + 14 * i;
        Body *b = w->w.get(static_cast<uint32_t>(i));
        if (!b)
        {
            std::fill(o, o + 14, 0.0);
            continue;
        }
        double v[14] = {b->pos.x, b->pos.y, b->pos.z, b->q.w, b->q.x, b->q.y, b->q.z,
                        b->vel.x, b->vel.y, b->vel.z, b->ang_vel.x, b->ang_vel.y, b->ang_vel.z, 1.0};
        std::copy(v, v + 14, o);
    }
    return n;
}
int pko_write_body_state(pko_world *w, int slot, const double *s)
{
    Body *b = w->w.get(static_cast<uint32_t>(slot));
    if (!b) return 0;
    b->pos = {s[0], s[1], s[2]};
    b->q = {s[3], s[4], s[5], s[6]};
    b->vel = {s[7], s[8], s[9]};
    b->ang_vel = {s[10], s[11], s[12]};
    b->update_derived();
    return 1;
}
int pko_read_pairs(pko_world *w, uint64_t *keys, int cap)
{
    std::vector<uint64_t> k(w->w.pairs.begin(), w->w.pairs.end());
    std::sort(k.begin(), k.end());
    for (int i = 0; i < static_cast<int>(k.size()) && i < cap; ++i) keys[i] = k[i];
    return static_cast<int>(k.size());
}
int pko_read_manifolds(pko_world *w, uint64_t *keys, int *counts, double *contacts, int cap)
{
    int i = 0;
    for (auto &[key, m] : w->w.manifolds)
    {
        if (i < cap)
        {
            keys[i] = key;
            counts[i] = m.n;
            for (int k = 0; k < 4; ++k)
            {
                double *o = contacts + (static_cast<size_t>(i) * 4 + k) * 13;
                const ContactInfo &c = m.c[k];
                double v[13] = {c.point.normal.x, c.point.normal.y, c.point.normal.z,
                                c.point.local_a.x, c.point.local_a.y, c.point.local_a.z,
                                c.point.local_b.x, c.point.local_b.y, c.point.local_b.z,
                                c.point.depth, c.normal_impulse, c.tangent_impulse[0], c.tangent_impulse[1]};
                if (k >= m.n) std::fill(v, v + 13, 0.0);
                std::copy(v, v + 13, o);
            }
        }
        ++i;
    }
    return i;
}
int pko_read_events(pko_world *w, uint64_t *keys, int *kinds, int cap)
{
    int n = static_cast<int>(w->w.events.size());
    for (int i = 0; i < n && i < cap; ++i)
    {
        keys[i] = w->w.events[i].key;
        kinds[i] = w->w.events[i].kind;
    }
    return n;
}
int pko_read_colours(pko_world *w, uint64_t *keys, int *colours, int cap, int *nc)
{
    int n = static_cast<int>(w->w.colour_keys.size());
    for (int i = 0; i < n && i < cap; ++i)
    {
        keys[i] = w->w.colour_keys[i];
        colours[i] = w->w.colours[i];
    }
    *nc = w->w.ncolours;
    return n;
}
int pko_last_moved(pko_world *w) { return w->w.last_moved; }

int pko_gjk_epa(pko_world *w, int ka, const double *pa, int sa, int kb, const double *pb, int sb, double *out)
{
    std::optional<CollisionInfo> r;
    switch (ka)
    {
    case 0: r = dispatch_b(w, aabb_from(pa), kb, pb, sb); break;
    case 1: r = dispatch_b(w, obb_from(pa), kb, pb, sb); break;
    default:
        r = dispatch_b(w, MeshInst{w->w.shapes[sa].get(), {pa[0], pa[1], pa[2]}, {pa[3], pa[4], pa[5], pa[6]}}, kb,
                       pb, sb);
    }
    if (!r) return 0;
    double v[10] = {r->normal.x, r->normal.y, r->normal.z, r->world_a.x, r->world_a.y,
                    r->world_a.z, r->world_b.x, r->world_b.y, r->world_b.z, r->depth};
    std::copy(v, v + 10, out);
    return 1;
}

int pko_mesh_raycast(pko_world *w, int shape, const double *pose7, const double *origin, const double *dir,
                     double max_dist, double *out7, int *tri)
{
    TriHit h;
    int t = -1;
    bool hit = mesh_ray_intersect(*w->w.shapes[size_t(shape)], {pose7[0], pose7[1], pose7[2]},
                                  {pose7[3], pose7[4], pose7[5], pose7[6]}, {origin[0], origin[1], origin[2]},
                                  {dir[0], dir[1], dir[2]}, max_dist, h, t);
    if (!hit) return 0;
    const double v[7] = {h.pos.x, h.pos.y, h.pos.z, h.normal.x, h.normal.y, h.normal.z, h.t};
    std::copy(v, v + 7, out7);
    *tri = t;
    return 1;
}

int pko_world_raycast(pko_world *w, const double *origin, const double *dir, double max_dist, uint64_t *handles,
                      double *dist, int cap)
{
    auto hits = w->w.raycast({origin[0], origin[1], origin[2]}, {dir[0], dir[1], dir[2]}, max_dist);
    int n = static_cast<int>(hits.size());
    for (int i = 0; i < n && i < cap; ++i)
    {
        if (handles) handles[i] = hits[static_cast<size_t>(i)].first;
        if (dist) dist[i] = hits[static_cast<size_t>(i)].second;
    }
    return n;
}

uint64_t pko_joint_add(pko_world *w, int type, uint64_t a, uint64_t b, const double *p16)
{
    // p16: anchor3, local_a3, local_b3, axis_a3, axis_b3, distance (stiffness, damping: p16[16..17])
    const double *p = p16;
    return w->w.add_joint(type, a, b, {p[0], p[1], p[2]}, {p[3], p[4], p[5]}, {p[6], p[7], p[8]}, {p[9], p[10], p[11]},
                          {p[12], p[13], p[14]}, p[15], p[16], p[17]);
}
int pko_joint_remove(pko_world *w, uint64_t h) { return w->w.remove_joint(h) ? 1 : 0; }
int pko_joint_impulses(pko_world *w, uint64_t h, double *out6)
{
    const Joint *j = w->w.joint(h);
    if (!j) return -1;
    for (int k = 0; k < 6; ++k) out6[k] = j->acc[k];
    return kJointRows[j->type];
}

pko_tree *pko_tree_create(void) { return new pko_tree; }
void pko_tree_destroy(pko_tree *t) { delete t; }
uint32_t pko_tree_add(pko_tree *t, uint32_t id, const double *b) { return t->t.add(id, aabb_from(b)); }
int pko_tree_update(pko_tree *t, uint32_t leaf, const double *b, const double *d)
{ return t->t.update_leaf(leaf, aabb_from(b), {d[0], d[1], d[2]}) ? 1 : 0; }
void pko_tree_remove(pko_tree *t, uint32_t leaf) { t->t.remove_leaf(leaf); }
void pko_tree_bounds(pko_tree *t, uint32_t leaf, double *b)
{
    const Aabb &a = t->t.nodes[leaf].bounds;
    double v[6] = {a.min.x, a.min.y, a.min.z, a.max.x, a.max.y, a.max.z};
    std::copy(v, v + 6, b);
}
int pko_tree_query(pko_tree *t, const double *b, uint32_t *out, int cap)
{
    int n = 0;
    t->t.query(aabb_from(b), [&](uint32_t id)
               {
                   if (n < cap) out[n] = id;
                   ++n;
                   return true;
               });
    return n;
}
int pko_tree_height(pko_tree *t) { return t->t.height(); }
int pko_tree_validate(pko_tree *t) { return t->t.validate() ? 1 : 0; }

void pko_sincos(double x, double *s, double *c) { sincos_det(x, s, c); }

} // extern "C"
