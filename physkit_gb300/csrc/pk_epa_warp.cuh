// pk_epa_warp.cuh — EPA for one shape pair per warp, polytope in shared memory.
//
// Same algorithm and the same arithmetic as pk::epa (collision.cpp:191-509): the 32 lanes share
// the support searches (mesh::support's first strictly maximal vertex, mesh.cpp:341-358, as a
// warp reduction on (value, index)) and the set-up of the new faces; lane 0 runs the steps whose
// order decides the result (face heap in the libstdc++ sift order, silhouette flood fill, face
// linking). Every other lane sees the shared state only after __syncwarp.
#pragma once

#include "pk_narrow.cuh"

namespace pk
{

// Polytope of one warp's pair, in shared memory.
template <class T> struct WarpEpa
{
    EpaState<T> e; // poly, faces, heap, counters (same layout as the per-thread version)
    uint16_t stack[kMaxFaces];
    HorizonEdge horizon[kMaxHorizon];
    uint16_t nf[kMaxHorizon];
    int nh;
    int mf;
};

// (value, index) warp maximum; equal values resolve to the smaller index, so the winner is the
// first strictly maximal element in index order. Lanes without a candidate pass idx = -1.
template <class T> __device__ __forceinline__ int warp_argmax(T v, int idx)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
    {
        T ov = __shfl_xor_sync(0xFFFFFFFFu, v, off);
        int oi = __shfl_xor_sync(0xFFFFFFFFu, idx, off);
        bool take = (oi >= 0) && (idx < 0 || ov > v || (ov == v && oi < idx));
        if (take)
        {
            v = ov;
            idx = oi;
        }
    }
    return idx;
}

template <class T> __device__ __forceinline__ T vdot(const T *verts, int i, V3<T> ld)
{ return verts[3 * i] * ld.x + verts[3 * i + 1] * ld.y + verts[3 * i + 2] * ld.z; }

template <class T> __device__ __forceinline__ T bound_at(const T *c, V3<T> ld, T dn)
{ return c[0] * ld.x + c[1] * ld.y + c[2] * ld.z + c[3] * dn; }

// ShapeRef::support computed by the whole warp; every lane returns the same point.
template <class T> __device__ V3<T> warp_support(const ShapeRef<T> &s, V3<T> d, int lane)
{
    if (s.kind != SHAPE_MESH || s.ngr > 32) return s.support(d); // closed forms / very large meshes: every lane alike
    V3<T> ld = rotate(conj(s.q), d);
    int best;
    if (s.ncl == 0)
    {
        T bv = T(0);
        int bi = -1;
        for (int i = lane; i < s.nverts; i += 32)
        {
            T v = vdot(s.verts, i, ld);
            if (bi < 0 || v > bv)
            {
                bv = v;
                bi = i;
            }
        }
        best = warp_argmax(bv, bi);
    }
    else
    {
        // ShapeRef::argmax_clustered, lane-parallel
        T dn = norm(ld);
        T margin = T(64) * EpsOf<T>::v * s.rmax * dn;
        T ub = T(0);
        int g = lane < s.ngr ? lane : -1;
        if (g >= 0) ub = bound_at(s.gr + 4 * g, ld, dn);
        int g0 = warp_argmax(ub, g);
        int klo = g0 * kClusterSize, khi = min(klo + kClusterSize, s.ncl);
        int k = klo + lane < khi && lane < kClusterSize ? klo + lane : -1;
        ub = k >= 0 ? bound_at(s.cl + 4 * k, ld, dn) : T(0);
        int kb = warp_argmax(ub, k);
        int lo = kb * kClusterSize, hi = min(lo + kClusterSize, s.nverts);
        T bv = T(0);
        int vi = lo + lane < hi && lane < kClusterSize ? lo + lane : -1;
        if (vi >= 0) bv = vdot(s.verts, vi, ld);
        int bidx = warp_argmax(bv, vi);
        T B = __shfl_sync(0xFFFFFFFFu, bv, bidx - lo);
        // candidate groups and clusters in index order; lane l keeps the best of the vertices it
        // sees (positions l mod 8 of each candidate block, in increasing order)
        unsigned gmask = __ballot_sync(0xFFFFFFFFu, lane < s.ngr && bound_at(s.gr + 4 * lane, ld, dn) + margin >= B);
        T lv = T(0);
        int li = -1;
        while (gmask)
        {
            int gg = __ffs(gmask) - 1;
            gmask &= gmask - 1;
            int k1 = gg * kClusterSize, k2 = min(k1 + kClusterSize, s.ncl);
            int kk = k1 + (lane & 7);
            bool cand = lane < kClusterSize && kk < k2 && bound_at(s.cl + 4 * kk, ld, dn) + margin >= B;
            unsigned cmask = __ballot_sync(0xFFFFFFFFu, cand);
            while (cmask)
            {
                int c = k1 + __ffs(cmask) - 1;
                cmask &= cmask - 1;
                int l = c * kClusterSize + lane;
                if (lane < kClusterSize && l < min(c * kClusterSize + kClusterSize, s.nverts))
                {
                    T v = vdot(s.verts, l, ld);
                    if (li < 0 || v > lv)
                    {
                        lv = v;
                        li = l;
                    }
                }
            }
        }
        best = warp_argmax(lv, li);
    }
    V3<T> lvx{s.verts[3 * best], s.verts[3 * best + 1], s.verts[3 * best + 2]};
    return rotate(s.q, lvx) + s.pos;
}

template <class T>
__device__ __forceinline__ SupPt<T> warp_minkowski(const ShapeRef<T> &A, const ShapeRef<T> &B, V3<T> d, int lane)
{
    V3<T> pa = warp_support(A, d, lane);
    V3<T> pb = warp_support(B, -d, lane);
    return {pa - pb, pa, pb};
}

// pad_simplex (collision.cpp:191-248); uniform across the warp.
template <class T> __device__ bool warp_pad_simplex(const ShapeRef<T> &A, const ShapeRef<T> &B, Simplex<T> &s, int lane)
{
    int n0 = s.n;
    if (n0 <= 1)
    {
        V3<T> dir{T(1), T(0), T(0)};
        SupPt<T> p2 = warp_minkowski(A, B, dir, lane);
        if (sqnorm(p2.p - s.v[0].p) < T(1e-6)) p2 = warp_minkowski(A, B, -dir, lane);
        s.push(p2);
    }
    if (n0 <= 2)
    {
        V3<T> line = s.v[1].p - s.v[0].p;
        V3<T> dir = cross(normalized(line), V3<T>{T(0), T(1), T(0)});
        if (sqnorm(dir) < T(1e-6)) dir = cross(normalized(line), V3<T>{T(0), T(0), T(1)});
        dir = normalized(dir);
        SupPt<T> p3 = warp_minkowski(A, B, dir, lane);
        if (sqnorm(cross(line, p3.p - s.v[0].p)) < T(1e-6)) p3 = warp_minkowski(A, B, -dir, lane);
        s.push(p3);
    }
    if (n0 <= 3)
    {
        V3<T> ab = s.v[1].p - s.v[0].p, ac = s.v[2].p - s.v[0].p;
        V3<T> dir = normalized(cross(ab, ac));
        SupPt<T> p4 = warp_minkowski(A, B, dir, lane);
        if (tabs(dot(p4.p - s.v[0].p, dir)) < T(1e-6)) p4 = warp_minkowski(A, B, -dir, lane);
        s.push(p4);
    }
    V3<T> ad = s.v[0].p - s.v[3].p, bd = s.v[1].p - s.v[3].p, cd = s.v[2].p - s.v[3].p;
    return tabs(dot(ad, cross(bd, cd))) > T(1e-12);
}

// epa (pk_narrow.cuh, collision.cpp:411-504) with the warp sharing the work. Returns the same
// result on every lane.
template <class T>
__device__ bool warp_epa(const ShapeRef<T> &A, const ShapeRef<T> &B, Simplex<T> s, WarpEpa<T> &W, Collision<T> &out,
                         int lane)
{
    EpaState<T> &e = W.e;
    if (lane == 0)
    {
        e.status = 0;
        e.iters = 0;
    }
    if (s.n < 4 && !warp_pad_simplex(A, B, s, lane)) return false;
    if (lane == 0)
    {
        e.npoly = 4;
        e.nfaces = 4;
        e.nheap = 0;
    }
    if (lane < 4) e.poly[lane] = s.v[lane];
    __syncwarp();
    const int init[4][4] = {{0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {1, 3, 2, 0}};
    if (lane < 4) e.init_face(lane, init[lane][0], init[lane][1], init[lane][2], init[lane][3]);
    __syncwarp();
    if (lane == 0)
    {
        for (int f = 0; f < 4; ++f) e.push_face(uint16_t(f));
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
    }
    __syncwarp();
    const T tol = T(1e-6);
    for (int iter = 0; iter < 64; ++iter)
    {
        if (lane == 0)
        {
            e.iters = iter + 1;
            W.mf = e.pop_face();
        }
        __syncwarp();
        const int mf = W.mf;
        if (mf < 0) break;
        const EpaFace<T> minf = e.faces[mf];
        SupPt<T> p = warp_minkowski(A, B, minf.n, lane);
        T pd = dot(minf.n, p.p);
        if (pd - minf.d < tol)
        {
            out = e.barycentric(minf);
            return true;
        }
        if (lane == 0)
        {
            // find_silhouette (collision.cpp:315-353)
            int nh = 0, sp = 0;
            W.stack[sp++] = uint16_t(mf);
            e.faces[mf].obsolete = 1;
            while (sp > 0)
            {
                int cur = W.stack[--sp];
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
                            W.stack[sp++] = n;
                        else
                            e.status |= PK_NP_STACK_CAP;
                    }
                    else if (nh < kMaxHorizon)
                        W.horizon[nh++] = {e.faces[cur].v[i], e.faces[cur].v[(i + 1) % 3], n};
                    else
                        e.status |= PK_NP_HORIZON_CAP;
                }
            }
            if (nh > 0 && e.nfaces + nh > kMaxFaces)
            {
                e.status |= PK_NP_FACE_CAP;
                nh = 0;
            }
            if (nh > 0) e.poly[e.npoly] = p;
            W.nh = nh;
        }
        __syncwarp();
        const int nh = W.nh;
        if (nh == 0) break;
        const int pi = e.npoly, f0 = e.nfaces;
        for (int h = lane; h < nh; h += 32) e.init_face(f0 + h, W.horizon[h].start, W.horizon[h].end, pi, -1);
        __syncwarp();
        if (lane == 0)
        {
            e.npoly = pi + 1;
            e.nfaces = f0 + nh;
            for (int h = 0; h < nh; ++h)
            {
                int f = f0 + h;
                e.link(f, W.horizon[h].adj, W.horizon[h].start, W.horizon[h].end);
                e.push_face(uint16_t(f));
                W.nf[h] = uint16_t(f);
            }
            for (int i = 0; i < nh; ++i)
                for (int j = i + 1; j < nh; ++j)
                {
                    if (W.horizon[i].end == W.horizon[j].start)
                        e.link(W.nf[i], W.nf[j], W.horizon[i].end, pi);
                    else if (W.horizon[i].start == W.horizon[j].end)
                        e.link(W.nf[j], W.nf[i], W.horizon[j].end, pi);
                }
        }
        __syncwarp();
    }
    if (lane == 0) W.mf = e.pop_face();
    __syncwarp();
    const int mf = W.mf;
    if (mf < 0) return false;
    out = e.barycentric(e.faces[mf]);
    return true;
}

} // namespace pk
