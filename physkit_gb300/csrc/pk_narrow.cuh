// pk_narrow.cuh — GJK boolean test + EPA penetration for one shape pair (device and host).
//
// Follows src/collision.cpp:10-518 branch for branch: GJK from direction (1,0,0) with the
// line/triangle/tetrahedron Voronoi cases (collision.cpp:12-162, <=100 iterations), simplex
// padding (collision.cpp:191-248), EPA with a min-distance face heap, silhouette flood fill and
// <=64 expansions (collision.cpp:251-509). The face heap uses the sift rules of the libstdc++
// std::push_heap / std::pop_heap that the reference calls (collision.cpp:390-408), so ties
// between equally distant faces resolve the same way.
//
// Storage is fixed-size per call (no heap allocation on the device). Exceeding a cap sets a
// status bit and returns the best face so far; callers report it.
#pragma once

#include "pk_math.cuh"

#include <cmath>

namespace pk
{

enum : int
{
    PK_NP_FACE_CAP = 1 << 0,
    PK_NP_HORIZON_CAP = 1 << 1,
    PK_NP_STACK_CAP = 1 << 2,
};

constexpr int kMaxPoly = 4 + 64;
constexpr int kMaxFaces = 512;
constexpr int kMaxHorizon = 96;
constexpr uint16_t kNull16 = 0xFFFF;
constexpr int kBoxLayout = -1; // ShapeRef::uv_stacks of a mesh in mesh::box's layout

enum : int
{
    SHAPE_AABB = 0,
    SHAPE_OBB = 1,
    SHAPE_MESH = 2,
};

template <class T> struct EpsOf;
template <> struct EpsOf<double>
{
    static constexpr double v = 2.220446049250313e-16;
};
template <> struct EpsOf<float>
{
    static constexpr float v = 1.1920929e-07f;
};

constexpr int kClusterSize = 8;

// UV-sphere layouts whose support search by neighbourhood (ShapeRef::argmax_uv) is proven exact:
// 8..64 stacks and sectors, and a ring-to-ring value gap of at least 1e-3 (relative).
PK_HD bool uv_layout_ok(int S, int K)
{
    if (S < 8 || S > 64 || K < 8 || K > 64) return false;
    const double pi = 3.14159265358979323846;
    return cos(0.5 * pi / S) - (1.0 - cos(pi / K)) - cos(2.0 * pi / S) >= 1e-3;
}

// A posed convex shape: aabb (a=min, b=max), obb (pos=center, q, b=half) or mesh instance
// (pos, q, vertex list). Large meshes carry clusters of kClusterSize consecutive vertices with a
// bounding sphere each (cx, cy, cz, radius) and the shape's bounding radius `rmax`.
template <class T> struct ShapeRef
{
    int kind;
    int nverts;
    const T *verts; // xyz interleaved, local frame
    V3<T> a, b, pos;
    Qt<T> q;
    int ncl;
    const T *cl;
    int ngr;       // groups of kClusterSize consecutive clusters (64 vertices), same layout
    const T *gr;
    T rmax;
    int uv_stacks;  // > 0: the vertex list is a UV sphere of this layout (pk_shape_sphere);
                    // kBoxLayout: mesh::box's 8 vertices (+-hx, +-hy, +-hz) in its order
    int uv_sectors;

    // First strictly maximal vertex of v.ld over the vertex list, in index order.
    PK_HD int argmax_linear(V3<T> ld, int lo, int hi, int best, T &bd) const
    {
        for (int i = lo; i < hi; ++i)
        {
            T v = verts[3 * i] * ld.x + verts[3 * i + 1] * ld.y + verts[3 * i + 2] * ld.z;
            if (best < 0 || v > bd)
            {
                bd = v;
                best = i;
            }
        }
        return best;
    }
    // Same result as argmax_linear over all vertices: clusters whose bound (with a margin that
    // covers the rounding of both the bound and every vertex dot product) is below the value of a
    // vertex already seen cannot hold the maximum or a tie with it, so they are skipped; the rest
    // are scanned in index order.
    PK_HD int argmax_clustered(V3<T> ld) const
    {
        T dn = norm(ld);
        T margin = T(64) * EpsOf<T>::v * rmax * dn;
        // seed: the best cluster of the best group gives the value B of an actual vertex
        int g0 = 0;
        T ubg = T(0);
        for (int g = 0; g < ngr; ++g)
        {
            const T *c = gr + 4 * g;
            T ub = c[0] * ld.x + c[1] * ld.y + c[2] * ld.z + c[3] * dn;
            if (g == 0 || ub > ubg)
            {
                ubg = ub;
                g0 = g;
            }
        }
        int klo = g0 * kClusterSize, khi = klo + kClusterSize < ncl ? klo + kClusterSize : ncl;
        int kb = klo;
        T ub_best = T(0);
        for (int k = klo; k < khi; ++k)
        {
            const T *c = cl + 4 * k;
            T ub = c[0] * ld.x + c[1] * ld.y + c[2] * ld.z + c[3] * dn;
            if (k == klo || ub > ub_best)
            {
                ub_best = ub;
                kb = k;
            }
        }
        T B;
        int lo = kb * kClusterSize, hi = lo + kClusterSize < nverts ? lo + kClusterSize : nverts;
        argmax_linear(ld, lo, hi, -1, B);
        // every vertex whose value can reach B lies in a cluster and a group whose bound reaches B
        int best = -1;
        T bd = T(0);
        for (int g = 0; g < ngr; ++g)
        {
            const T *c = gr + 4 * g;
            if (c[0] * ld.x + c[1] * ld.y + c[2] * ld.z + c[3] * dn + margin < B) continue;
            int k1 = g * kClusterSize, k2 = k1 + kClusterSize < ncl ? k1 + kClusterSize : ncl;
            for (int k = k1; k < k2; ++k)
            {
                const T *cc = cl + 4 * k;
                if (cc[0] * ld.x + cc[1] * ld.y + cc[2] * ld.z + cc[3] * dn + margin < B) continue;
                int l = k * kClusterSize, h = l + kClusterSize < nverts ? l + kClusterSize : nverts;
                best = argmax_linear(ld, l, h, best, bd);
            }
        }
        return best;
    }

    // Same result as argmax_linear over a UV sphere (north pole, stacks-1 rings of `sectors`
    // vertices at polar angles pi*i/S and azimuths 2*pi*j/K, south pole), for the layouts that
    // uv_layout_ok accepts. With phi, theta the angles of ld, the rings i0-1..i0+2 around
    // phi (i0 = floor(phi S / pi)) and the sectors j0-1..j0+2 around theta hold the maximum of v.ld
    // and every vertex within rounding of it:
    //  - a vertex of any other ring is at least 2 pi/S from ld in polar angle and trails the
    //    nearest in-ring candidate by cos(pi/2S) - (1 - cos(pi/K)) - cos(2 pi/S), which the layout
    //    check keeps >= 1e-3 (times |ld| r);
    //  - another sector of an included ring i trails that ring's nearest sector by
    //    sin(phi) sin(phi_i) (cos(pi/K) - cos(4 pi/K)) >= 1e-4 once sin(phi) is above the
    //    threshold computed below (phi_i >= pi/S); nearer a pole the candidate rings are scanned
    //    whole.
    // Rounding of any vertex value is below 1e-6 |ld| r in FP32 (below 1e-15 in FP64). Candidates
    // are compared by value, then by lower index, so ties resolve as in the linear scan.
    // mesh::box (mesh.cpp:31-40): with px = hx lx, py = hy ly, pz = hz lz, vertex i's value
    // (x lx + y ly) + z lz is +-((px +- py) +- pz), since rounding to nearest commutes with
    // negation; 3 products and 6 sums give the linear scan's 8 values bit for bit (an exact zero may
    // differ in sign, which compares equal), and the same first strict maximum.
    PK_HD int argmax_box(V3<T> ld) const
    {
        const T px = verts[18] * ld.x, py = verts[19] * ld.y, pz = verts[20] * ld.z; // vertex 6: +h
        const T sa = px + py, sd = px - py;
        const T a = sa + pz, b = sa - pz, c = sd + pz, e = sd - pz;
        const T val[8] = {-a, e, b, -c, -b, c, a, -e};
        int best = 0;
        T bd = val[0];
#pragma unroll
        for (int i = 1; i < 8; ++i)
            if (val[i] > bd)
            {
                bd = val[i];
                best = i;
            }
        return best;
    }

    PK_HD int argmax_uv(V3<T> ld) const
    {
        int best = -1;
        T bd = T(0);
        const T n2 = sqnorm(ld);
        if (!(n2 > T(0))) return 0; // every value is zero: the first vertex
        // |ld| only for the FP32 form's polar angle (the FP64 form takes the angles in FP32)
        const T dn = sizeof(T) == 8 ? T(0) : pk_sqrt(n2);
        uv_window(ld, dn, [&](int i) {
            T v = verts[3 * i] * ld.x + verts[3 * i + 1] * ld.y + verts[3 * i + 2] * ld.z;
            if (best < 0 || v > bd || (v == bd && i < best))
            {
                bd = v;
                best = i;
            }
        });
        return best;
    }

    // The UV-sphere vertices argmax_uv compares (see there), visited in the window's order; U is
    // the precision of the vertex values (dn = |ld| > 0). The angles are found in FP32 in both
    // forms. In the FP64 form the window is then widened by a ring (a sector) on the side of a
    // boundary within 1/16 of the FP32 fractional index, and the pole band is entered 6 % early, so
    // it holds every vertex of the window the angles in FP64 would give: the FP32 angle error is
    // below 1e-2 ring or sector (1e-4 away from the poles). Extra candidates are compared exactly
    // like the others, so the result is the same vertex. (Query directions are unit vectors, or
    // zero, which argmax_uv settles first, so the FP32 copy neither underflows nor overflows.)
    template <class U, class F> PK_HD void uv_window(V3<U> ld, U dn, F take) const
    {
        const int S = uv_stacks, K = uv_sectors, last = nverts - 1;
        constexpr bool wide = sizeof(U) == 8;
        const float lx = float(ld.x), ly = float(ld.y), lz = float(ld.z);
        float cy = wide ? ly / pk_sqrt(lx * lx + ly * ly + lz * lz) : float(ld.y / dn);
        cy = cy > 1.0f ? 1.0f : (cy < -1.0f ? -1.0f : cy);
        const float pi = 3.14159265358979323846f;
        const float f = pk_acos(cy) * float(S) / pi; // fractional ring index, 0 at the north pole
        int i0 = int(f);
        i0 = i0 < 0 ? 0 : (i0 > S ? S : i0);
        int ilo = i0 - 1, ihi = i0 + 2;
        if (wide)
        {
            ilo -= f - float(i0) < 0.0625f;
            ihi += f - float(i0) > 0.9375f;
        }
        const float sphi2 = 1.0f - cy * cy;
        // sin(phi) below which the sector gap could fall under 1e-4: 1e-4 / (sin(pi/S) *
        // (cos(pi/K) - cos(4 pi/K))), with x - x^3/6 <= sin x making it an over-estimate
        const float dp = pi / float(S), a1 = 2.5f * pi / float(K), a2 = 1.5f * pi / float(K);
        const float lb = (dp - dp * dp * dp / 6.0f) * 2.0f * (a1 - a1 * a1 * a1 / 6.0f) * (a2 - a2 * a2 * a2 / 6.0f);
        const float thr = 1e-4f / lb;
        if (sphi2 < thr * thr * (wide ? 1.0625f : 1.0f))
        {
            // within asin(0.2) of a pole: the pole and whole rings
            if (ilo <= 0) take(0);
            if (ihi >= S) take(last);
            int a = ilo < 1 ? 1 : ilo, b = ihi > S - 1 ? S - 1 : ihi;
            for (int i = a; i <= b; ++i)
                for (int j = 0; j < K; ++j) take(1 + (i - 1) * K + j);
            return;
        }
        float th = wide ? pk_atan2(lz, lx) : float(pk_atan2(ld.z, ld.x));
        if (th < 0.0f) th = th + 2.0f * pi;
        const float g = th * float(K) / (2.0f * pi);
        int j0 = int(g);
        j0 = j0 > K - 1 ? K - 1 : j0;
        int jlo = j0 - 1, jhi = j0 + 2;
        if (wide)
        {
            jlo -= g - float(j0) < 0.0625f;
            jhi += g - float(j0) > 0.9375f;
        }
        for (int i = ilo; i <= ihi; ++i)
        {
            if (i <= 0)
            {
                take(0);
                continue;
            }
            if (i >= S)
            {
                take(last);
                continue;
            }
            for (int jj = jlo; jj <= jhi; ++jj)
            {
                int j = jj < 0 ? jj + K : (jj >= K ? jj - K : jj); // jj in [-2, K + 2]
                take(1 + (i - 1) * K + j);
            }
        }
    }

    PK_HD V3<T> support(V3<T> d) const
    {
        if (kind == SHAPE_AABB)
        {
            T sx = d.x >= T(0) ? T(1) : T(-1), sy = d.y >= T(0) ? T(1) : T(-1), sz = d.z >= T(0) ? T(1) : T(-1);
            return {sx > T(0) ? b.x : a.x, sy > T(0) ? b.y : a.y, sz > T(0) ? b.z : a.z};
        }
        if (kind == SHAPE_OBB)
        {
            // obb::support (bounds.h:539-548)
            V3<T> ld = rotate(conj(q), d);
            V3<T> s{ld.x >= T(0) ? T(1) : T(-1), ld.y >= T(0) ? T(1) : T(-1), ld.z >= T(0) ? T(1) : T(-1)};
            return pos + rotate(q, V3<T>{s.x * b.x, s.y * b.y, s.z * b.z});
        }
        // mesh::instance::support -> mesh::support: first strictly maximal vertex
        // (mesh.cpp:341-358, 442-448)
        V3<T> ld = rotate(conj(q), d);
        int best;
        if (sizeof(T) == 8 && uv_stacks == kBoxLayout)
            best = argmax_box(ld); // FP64 form (the FP32 form's scan may contract products into FMAs)
        else if (uv_stacks > 0)
            best = argmax_uv(ld);
        else if (ncl > 0)
            best = argmax_clustered(ld);
        else
        {
            T bd;
            best = argmax_linear(ld, 0, nverts, -1, bd);
        }
        V3<T> lv{verts[3 * best], verts[3 * best + 1], verts[3 * best + 2]};
        return rotate(q, lv) + pos;
    }
};

template <class T> struct SupPt
{
    V3<T> p, pa, pb;
};

template <class T> struct Collision
{
    V3<T> normal, world_a, world_b;
    T depth;
};

template <class T> PK_HD SupPt<T> minkowski(const ShapeRef<T> &A, const ShapeRef<T> &B, V3<T> d)
{
    V3<T> pa = A.support(d);
    V3<T> pb = B.support(-d);
    return {pa - pb, pa, pb};
}

template <class T> struct Simplex
{
    SupPt<T> v[4];
    int n;
    int iters; // GJK iterations used
    PK_HD void push(const SupPt<T> &p) { v[n++] = p; }
    PK_HD void erase(int i)
    {
        for (int k = i; k + 1 < n; ++k) v[k] = v[k + 1];
        --n;
    }
};

template <class T> PK_HD void gjk_triangle(Simplex<T> &s, V3<T> &dir)
{
    const SupPt<T> a = s.v[2], b = s.v[1], c = s.v[0];
    V3<T> ab = b.p - a.p, ac = c.p - a.p, ao = -a.p;
    V3<T> abc = cross(ab, ac);
    V3<T> ab_perp = cross(ab, abc);
    if (dot(ab_perp, ao) > T(0))
    {
        s.erase(0);
        V3<T> tr = cross(cross(ab, ao), ab);
        dir = (sqnorm(tr) < T(1e-12)) ? normalized(ao) : normalized(tr);
        return;
    }
    V3<T> ac_perp = cross(abc, ac);
    if (dot(ac_perp, ao) > T(0))
    {
        s.erase(1);
        V3<T> tr = cross(cross(ac, ao), ac);
        dir = (sqnorm(tr) < T(1e-12)) ? normalized(ao) : normalized(tr);
        return;
    }
    if (dot(abc, ao) <= T(0))
    {
        SupPt<T> t = s.v[0];
        s.v[0] = s.v[1];
        s.v[1] = t;
        dir = normalized(-abc);
    }
    else
        dir = normalized(abc);
}

// Returns true when the simplex encloses the origin (collision.cpp:149-162).
template <class T> PK_HD bool gjk_simplex(Simplex<T> &s, V3<T> &dir)
{
    if (s.n == 2)
    {
        const SupPt<T> a = s.v[1], b = s.v[0];
        V3<T> ab = b.p - a.p, ao = -a.p;
        if (dot(ab, ao) > T(0))
        {
            V3<T> tr = cross(cross(ab, ao), ab);
            if (sqnorm(tr) < T(1e-12))
            {
                V3<T> ab_hat = normalized(ab);
                V3<T> perp = cross(ab_hat, V3<T>{T(0), T(1), T(0)});
                if (sqnorm(perp) < T(1e-12)) perp = cross(ab_hat, V3<T>{T(0), T(0), T(1)});
                dir = normalized(perp);
            }
            else
                dir = normalized(tr);
        }
        else
        {
            s.erase(0);
            dir = normalized(ao);
        }
        return false;
    }
    if (s.n == 3)
    {
        gjk_triangle(s, dir);
        return false;
    }
    if (s.n == 4)
    {
        const SupPt<T> a = s.v[3], b = s.v[2], c = s.v[1], d = s.v[0];
        V3<T> ao = -a.p;
        V3<T> abc = cross(b.p - a.p, c.p - a.p);
        V3<T> acd = cross(c.p - a.p, d.p - a.p);
        V3<T> adb = cross(d.p - a.p, b.p - a.p);
        if (dot(abc, d.p - a.p) > T(0)) abc = -abc;
        if (dot(acd, b.p - a.p) > T(0)) acd = -acd;
        if (dot(adb, c.p - a.p) > T(0)) adb = -adb;
        if (dot(abc, ao) > T(0))
        {
            s.n = 0;
            s.push(c);
            s.push(b);
            s.push(a);
            dir = normalized(abc);
            gjk_triangle(s, dir);
            return false;
        }
        if (dot(acd, ao) > T(0))
        {
            s.n = 0;
            s.push(d);
            s.push(c);
            s.push(a);
            dir = normalized(acd);
            gjk_triangle(s, dir);
            return false;
        }
        if (dot(adb, ao) > T(0))
        {
            s.n = 0;
            s.push(b);
            s.push(d);
            s.push(a);
            dir = normalized(adb);
            gjk_triangle(s, dir);
            return false;
        }
        return true;
    }
    return false;
}

// gjk_collision (collision.cpp:165-189). Returns true with the enclosing simplex. On the exit
// where the support in the search direction does not pass the origin, that direction (unit
// length) goes to *sep: no point of A - B lies beyond the origin along it.
template <class T> PK_HD bool gjk(const ShapeRef<T> &A, const ShapeRef<T> &B, Simplex<T> &s, V3<T> *sep = nullptr)
{
    s.n = 0;
    s.iters = 0;
    V3<T> dir{T(1), T(0), T(0)};
    SupPt<T> pt = minkowski(A, B, dir);
    s.push(pt);
    if (sqnorm(pt.p) < T(1e-12)) return true;
    dir = -normalized(pt.p);
    for (int iter = 0; iter < 100; ++iter)
    {
        s.iters = iter + 1;
        SupPt<T> np = minkowski(A, B, dir);
        if (dot(np.p, dir) <= T(0))
        {
            if (sep) *sep = dir;
            return false;
        }
        s.push(np);
        if (gjk_simplex(s, dir)) return true;
    }
    return false;
}

template <class T> PK_HD bool pad_simplex(const ShapeRef<T> &A, const ShapeRef<T> &B, Simplex<T> &s)
{
    int n0 = s.n;
    if (n0 <= 1)
    {
        V3<T> dir{T(1), T(0), T(0)};
        SupPt<T> p2 = minkowski(A, B, dir);
        if (sqnorm(p2.p - s.v[0].p) < T(1e-6)) p2 = minkowski(A, B, -dir);
        s.push(p2);
    }
    if (n0 <= 2)
    {
        V3<T> line = s.v[1].p - s.v[0].p;
        V3<T> dir = cross(normalized(line), V3<T>{T(0), T(1), T(0)});
        if (sqnorm(dir) < T(1e-6)) dir = cross(normalized(line), V3<T>{T(0), T(0), T(1)});
        dir = normalized(dir);
        SupPt<T> p3 = minkowski(A, B, dir);
        if (sqnorm(cross(line, p3.p - s.v[0].p)) < T(1e-6)) p3 = minkowski(A, B, -dir);
        s.push(p3);
    }
    if (n0 <= 3)
    {
        V3<T> ab = s.v[1].p - s.v[0].p, ac = s.v[2].p - s.v[0].p;
        V3<T> dir = normalized(cross(ab, ac));
        SupPt<T> p4 = minkowski(A, B, dir);
        if (tabs(dot(p4.p - s.v[0].p, dir)) < T(1e-6)) p4 = minkowski(A, B, -dir);
        s.push(p4);
    }
    V3<T> ad = s.v[0].p - s.v[3].p, bd = s.v[1].p - s.v[3].p, cd = s.v[2].p - s.v[3].p;
    return tabs(dot(ad, cross(bd, cd))) > T(1e-12);
}

template <class T> struct EpaFace
{
    uint16_t v[3];
    uint16_t adj[3];
    V3<T> n;
    T d;
    uint8_t obsolete;
};

template <class T> struct EpaState
{
    SupPt<T> poly[kMaxPoly];
    EpaFace<T> faces[kMaxFaces];
    uint16_t heap[kMaxFaces];
    int npoly, nfaces, nheap;
    int status;
    int iters; // EPA expansions used

    // heap comparison used by the reference: comp(f1, f2) = dist(f1) > dist(f2)
    PK_HD bool comp(uint16_t f1, uint16_t f2) const { return faces[f1].d > faces[f2].d; }

    // libstdc++ __push_heap
    PK_HD void sift_up(int hole, int top, uint16_t value)
    {
        int parent = (hole - 1) / 2;
        while (hole > top && comp(heap[parent], value))
        {
            heap[hole] = heap[parent];
            hole = parent;
            parent = (hole - 1) / 2;
        }
        heap[hole] = value;
    }
    PK_HD void push_face(uint16_t f)
    {
        heap[nheap++] = f;
        sift_up(nheap - 1, 0, heap[nheap - 1]);
    }
    // libstdc++ pop_heap = move the top to the back, then __adjust_heap on [0, len-1)
    PK_HD uint16_t pop_top()
    {
        int len = nheap;
        if (len > 1)
        {
            uint16_t value = heap[len - 1];
            heap[len - 1] = heap[0];
            int n = len - 1;
            int hole = 0, top = 0, second = 0;
            while (second < (n - 1) / 2)
            {
                second = 2 * (second + 1);
                if (comp(heap[second], heap[second - 1])) second--;
                heap[hole] = heap[second];
                hole = second;
            }
            if ((n & 1) == 0 && second == (n - 2) / 2)
            {
                second = 2 * (second + 1);
                heap[hole] = heap[second - 1];
                hole = second - 1;
            }
            sift_up(hole, top, value);
        }
        return heap[--nheap];
    }
    PK_HD int pop_face()
    {
        while (nheap > 0)
        {
            uint16_t f = pop_top();
            if (!faces[f].obsolete) return f;
        }
        return -1;
    }
    PK_HD void init_face(int f, int i, int j, int k, int opp)
    {
        EpaFace<T> &fc = faces[f];
        fc.v[0] = uint16_t(i);
        fc.v[1] = uint16_t(j);
        fc.v[2] = uint16_t(k);
        fc.adj[0] = fc.adj[1] = fc.adj[2] = kNull16;
        fc.obsolete = 0;
        V3<T> ab = poly[j].p - poly[i].p, ac = poly[k].p - poly[i].p;
        V3<T> n = cross(ab, ac);
        if (sqnorm(n) < T(1e-12))
            n = V3<T>{T(0), T(0), T(0)};
        else
            n = normalized(n);
        if (opp >= 0 && dot(n, poly[opp].p - poly[i].p) > T(0))
        {
            uint16_t t = fc.v[1];
            fc.v[1] = fc.v[2];
            fc.v[2] = t;
            n = -n;
        }
        fc.n = n;
        fc.d = dot(n, poly[i].p);
    }
    PK_HD void link(int f1, int f2, int va, int vb)
    {
        EpaFace<T> &a = faces[f1];
        EpaFace<T> &b = faces[f2];
        int e1 = (a.v[0] == va) ? 0 : (a.v[1] == va ? 1 : 2);
        int e2 = (b.v[0] == vb) ? 0 : (b.v[1] == vb ? 1 : 2);
        a.adj[e1] = uint16_t(f2);
        b.adj[e2] = uint16_t(f1);
    }
    // FP32 form: the termination face's plane and the contact in FP64, from its three support
    // points (normal oriented like the FP32 one; centroid weights if the face is degenerate even
    // in FP64, where the FP32 projection would divide 0 by 0).
    struct PlaneHP
    {
        double n[3], d;
    };
    PK_HD PlaneHP plane_hp(const EpaFace<T> &f) const
    {
        const V3<T> &a = poly[f.v[0]].p, &b = poly[f.v[1]].p, &c = poly[f.v[2]].p;
        double ax = a.x, ay = a.y, az = a.z;
        double ux = double(b.x) - ax, uy = double(b.y) - ay, uz = double(b.z) - az;
        double vx = double(c.x) - ax, vy = double(c.y) - ay, vz = double(c.z) - az;
        double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
        double nn = nx * nx + ny * ny + nz * nz;
        PlaneHP h;
        if (nn > 0.0)
        {
            double inv = 1.0 / pk_sqrt(nn);
            nx *= inv;
            ny *= inv;
            nz *= inv;
            if (nx * double(f.n.x) + ny * double(f.n.y) + nz * double(f.n.z) < 0.0)
            {
                nx = -nx;
                ny = -ny;
                nz = -nz;
            }
        }
        else
        {
            nx = f.n.x;
            ny = f.n.y;
            nz = f.n.z;
        }
        h.n[0] = nx;
        h.n[1] = ny;
        h.n[2] = nz;
        h.d = nx * ax + ny * ay + nz * az;
        return h;
    }
    PK_HD Collision<T> barycentric_hp(const EpaFace<T> &f) const
    {
        const SupPt<T> &q0 = poly[f.v[0]], &q1 = poly[f.v[1]], &q2 = poly[f.v[2]];
        PlaneHP h = plane_hp(f);
        double a[3] = {q0.p.x, q0.p.y, q0.p.z}, b[3] = {q1.p.x, q1.p.y, q1.p.z}, c[3] = {q2.p.x, q2.p.y, q2.p.z};
        double v0[3], v1[3], v2[3];
        for (int k = 0; k < 3; ++k)
        {
            v0[k] = b[k] - a[k];
            v1[k] = c[k] - a[k];
            v2[k] = h.n[k] * h.d - a[k];
        }
        double d00 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
        double d01 = v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2];
        double d11 = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
        double d20 = v2[0] * v0[0] + v2[1] * v0[1] + v2[2] * v0[2];
        double d21 = v2[0] * v1[0] + v2[1] * v1[1] + v2[2] * v1[2];
        double den = d00 * d11 - d01 * d01;
        double v = 1.0 / 3.0, w = 1.0 / 3.0;
        if (den > 0.0)
        {
            v = (d11 * d20 - d01 * d21) / den;
            w = (d00 * d21 - d01 * d20) / den;
        }
        double u = 1.0 - v - w;
        Collision<T> col;
        col.normal = V3<T>{T(-h.n[0]), T(-h.n[1]), T(-h.n[2])};
        col.world_a = V3<T>{T(u * q0.pa.x + v * q1.pa.x + w * q2.pa.x), T(u * q0.pa.y + v * q1.pa.y + w * q2.pa.y),
                            T(u * q0.pa.z + v * q1.pa.z + w * q2.pa.z)};
        col.world_b = V3<T>{T(u * q0.pb.x + v * q1.pb.x + w * q2.pb.x), T(u * q0.pb.y + v * q1.pb.y + w * q2.pb.y),
                            T(u * q0.pb.z + v * q1.pb.z + w * q2.pb.z)};
        col.depth = T(h.d);
        return col;
    }
    PK_HD Collision<T> barycentric(const EpaFace<T> &f) const
    {
        if constexpr (sizeof(T) == 4) return barycentric_hp(f);
        const SupPt<T> &p0 = poly[f.v[0]], &p1 = poly[f.v[1]], &p2 = poly[f.v[2]];
        V3<T> pm = f.n * f.d;
        V3<T> v0 = p1.p - p0.p, v1 = p2.p - p0.p, v2 = pm - p0.p;
        T d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
        T d20 = dot(v2, v0), d21 = dot(v2, v1);
        T denom = d00 * d11 - d01 * d01;
        T v = (d11 * d20 - d01 * d21) / denom;
        T w = (d00 * d21 - d01 * d20) / denom;
        T u = T(1) - v - w;
        Collision<T> c;
        c.normal = -f.n;
        c.world_a = u * p0.pa + v * p1.pa + w * p2.pa;
        c.world_b = u * p0.pb + v * p1.pb + w * p2.pb;
        c.depth = f.d;
        return c;
    }
};

struct HorizonEdge
{
    uint16_t start, end, adj;
};

// epa_solver::solve (collision.cpp:411-504). Returns true with a collision.
template <class T>
PK_HD bool epa(const ShapeRef<T> &A, const ShapeRef<T> &B, Simplex<T> &s, EpaState<T> &e, Collision<T> &out)
{
    e.status = 0;
    e.iters = 0;
    if (s.n < 4 && !pad_simplex(A, B, s)) return false;
    e.npoly = 4;
    for (int i = 0; i < 4; ++i) e.poly[i] = s.v[i];
    e.nfaces = 0;
    e.nheap = 0;
    const int init[4][4] = {{0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {1, 3, 2, 0}};
    for (int f = 0; f < 4; ++f)
    {
        e.init_face(f, init[f][0], init[f][1], init[f][2], init[f][3]);
        e.nfaces = f + 1;
        e.push_face(uint16_t(f));
    }
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j)
            for (int e1 = 0; e1 < 3; ++e1)
            {
                uint16_t u1 = e.faces[i].v[e1], v1 = e.faces[i].v[(e1 + 1) % 3];
                for (int e2 = 0; e2 < 3; ++e2)
                {
                    uint16_t u2 = e.faces[j].v[e2], v2 = e.faces[j].v[(e2 + 1) % 3];
                    if (u1 == v2 && v1 == u2)
                    {
                        e.faces[i].adj[e1] = uint16_t(j);
                        e.faces[j].adj[e2] = uint16_t(i);
                    }
                }
            }

    HorizonEdge horizon[kMaxHorizon];
    uint16_t stack[kMaxFaces];
    uint16_t nf[kMaxHorizon];
    const T tol = T(1e-6);
    for (int iter = 0; iter < 64; ++iter)
    {
        e.iters = iter + 1;
        int mf = e.pop_face();
        if (mf < 0) break;
        const EpaFace<T> minf = e.faces[mf];
        SupPt<T> p = minkowski(A, B, minf.n);
        T pd = dot(minf.n, p.p);
        bool done = pd - minf.d < tol;
        if constexpr (sizeof(T) == 4)
        {
            // FP32 form: near termination the face's plane distance is re-evaluated in FP64
            if (pd - minf.d < T(8) * tol)
            {
                auto h = e.plane_hp(minf);
                done = h.n[0] * double(p.p.x) + h.n[1] * double(p.p.y) + h.n[2] * double(p.p.z) - h.d < double(tol);
            }
        }
        if (done)
        {
            out = e.barycentric(minf);
            return true;
        }
        // find_silhouette (collision.cpp:315-353): depth-first flood over visible faces
        int nh = 0, sp = 0;
        stack[sp++] = uint16_t(mf);
        e.faces[mf].obsolete = 1;
        while (sp > 0)
        {
            int cur = stack[--sp];
            for (int i = 0; i < 3; ++i)
            {
                uint16_t n = e.faces[cur].adj[i];
                if (n == kNull16) continue;
                EpaFace<T> &nb = e.faces[n];
                if (nb.obsolete) continue;
                if (dot(nb.n, p.p) > nb.d + tol)
                {
                    nb.obsolete = 1;
                    if (sp < kMaxFaces)
                        stack[sp++] = n;
                    else
                        e.status |= PK_NP_STACK_CAP;
                }
                else if (nh < kMaxHorizon)
                    horizon[nh++] = {e.faces[cur].v[i], e.faces[cur].v[(i + 1) % 3], n};
                else
                    e.status |= PK_NP_HORIZON_CAP;
            }
        }
        if (nh == 0) break;
        if (e.nfaces + nh > kMaxFaces)
        {
            e.status |= PK_NP_FACE_CAP;
            break;
        }
        e.poly[e.npoly] = p;
        int pi = e.npoly++;
        for (int h = 0; h < nh; ++h)
        {
            int f = e.nfaces++;
            e.init_face(f, horizon[h].start, horizon[h].end, pi, -1);
            e.link(f, horizon[h].adj, horizon[h].start, horizon[h].end);
            e.push_face(uint16_t(f));
            nf[h] = uint16_t(f);
        }
        for (int i = 0; i < nh; ++i)
            for (int j = i + 1; j < nh; ++j)
            {
                if (horizon[i].end == horizon[j].start)
                    e.link(nf[i], nf[j], horizon[i].end, pi);
                else if (horizon[i].start == horizon[j].end)
                    e.link(nf[j], nf[i], horizon[j].end, pi);
            }
    }
    int mf = e.pop_face();
    if (mf < 0) return false;
    out = e.barycentric(e.faces[mf]);
    return true;
}

// gjk_epa (collision.cpp:512-518)
template <class T>
PK_HD bool gjk_epa(const ShapeRef<T> &A, const ShapeRef<T> &B, EpaState<T> &e, Collision<T> &out, int *status)
{
    Simplex<T> s;
    *status = 0;
    if (!gjk(A, B, s)) return false;
    bool hit = epa(A, B, s, e, out);
    *status = e.status;
    return hit;
}

} // namespace pk
