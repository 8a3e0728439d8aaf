// Host-side checks of device code in physkit_gb300/csrc/pk_narrow.cuh (compiled with g++):
//  1. the EPA face heap pops faces in exactly the order std::push_heap/std::pop_heap would
//     (the reference's heap, collision.cpp:390-408), including ties;
//  2. the clustered support search returns the same vertex as the linear first-strict-max scan
//     (mesh.cpp:341-358) for UV spheres and random hulls, in FP64 and FP32;
//  3. so does the UV-sphere neighbourhood search, for every layout it accepts (uv_layout_ok),
//     including directions at and near the poles, on ring planes and between sectors;
//  4. so does the box search of the FP64 form (mesh::box layout), including axis directions,
//     exact ties, zero and negative-zero components.
#include "../../physkit_gb300/csrc/pk_narrow.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

using namespace pk;

static int check_heap(std::mt19937_64 &rng)
{
    int bad = 0;
    for (int trial = 0; trial < 2000; ++trial)
    {
        static EpaState<double> e;
        e.nfaces = 0;
        e.nheap = 0;
        std::vector<size_t> ref;
        std::vector<double> dist;
        auto cmp = [&](size_t a, size_t b) { return dist[a] > dist[b]; };
        int ops = 1 + int(rng() % 300);
        std::uniform_int_distribution<int> few(0, 6); // many exact ties
        for (int k = 0; k < ops; ++k)
        {
            if (e.nfaces < kMaxFaces && (rng() % 3 != 0 || ref.empty()))
            {
                int f = e.nfaces++;
                double d = double(few(rng)) * 0.25;
                e.faces[f].d = d;
                dist.push_back(d);
                e.push_face(uint16_t(f));
                ref.push_back(size_t(f));
                std::push_heap(ref.begin(), ref.end(), cmp);
            }
            else if (!ref.empty())
            {
                std::pop_heap(ref.begin(), ref.end(), cmp);
                size_t want = ref.back();
                ref.pop_back();
                uint16_t got = e.pop_top();
                if (got != want) ++bad;
            }
        }
    }
    return bad;
}

template <class T> static std::vector<T> make_clusters(const std::vector<double> &v, double &rm, size_t block = 8)
{
    size_t nv = v.size() / 3;
    rm = 0;
    for (size_t i = 0; i < nv; ++i)
        rm = std::fmax(rm, std::sqrt(v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]));
    std::vector<T> c;
    for (size_t b = 0; b < nv; b += block)
    {
        size_t e = std::min(b + block, nv);
        double cc[3] = {0, 0, 0};
        for (size_t i = b; i < e; ++i)
            for (int k = 0; k < 3; ++k) cc[k] += v[3 * i + k] / double(e - b);
        double r = 0;
        for (size_t i = b; i < e; ++i)
        {
            double dx = v[3 * i] - cc[0], dy = v[3 * i + 1] - cc[1], dz = v[3 * i + 2] - cc[2];
            r = std::fmax(r, std::sqrt(dx * dx + dy * dy + dz * dz));
        }
        r = r * (1.0 + 1e-9) + 1e-6 * rm;
        c.push_back(T(cc[0]));
        c.push_back(T(cc[1]));
        c.push_back(T(cc[2]));
        c.push_back(T(r));
    }
    return c;
}

template <class T> static int check_support(const std::vector<double> &vd, std::mt19937_64 &rng, int ndirs)
{
    std::vector<T> v(vd.begin(), vd.end());
    double rm;
    std::vector<T> cl = make_clusters<T>(vd, rm);
    std::vector<T> gr = make_clusters<T>(vd, rm, 64);
    ShapeRef<T> s{};
    s.kind = SHAPE_MESH;
    s.nverts = int(v.size() / 3);
    s.verts = v.data();
    s.ncl = int(cl.size() / 4);
    s.cl = cl.data();
    s.ngr = int(gr.size() / 4);
    s.gr = gr.data();
    s.rmax = T(rm);
    std::normal_distribution<double> nd(0.0, 1.0);
    int bad = 0;
    for (int k = 0; k < ndirs; ++k)
    {
        V3<T> d;
        if (k < 26)
        { // axis and diagonal directions: exact ties on symmetric meshes
            int a = k % 3, sgn = (k / 3) % 2 ? -1 : 1;
            d = V3<T>{T(0), T(0), T(0)};
            if (k < 6) (a == 0 ? d.x : a == 1 ? d.y : d.z) = T(sgn);
            else d = V3<T>{T((k & 1) ? 1 : -1), T((k & 2) ? 1 : -1), T((k & 4) ? 1 : -1)};
        }
        else
            d = V3<T>{T(nd(rng)), T(nd(rng)), T(nd(rng))};
        T bd;
        int lin = s.argmax_linear(d, 0, s.nverts, -1, bd);
        int clu = s.argmax_clustered(d);
        if (lin != clu) ++bad;
    }
    return bad;
}

template <class T> static int check_uv(const std::vector<double> &vd, int stacks, int sectors, std::mt19937_64 &rng, int ndirs)
{
    std::vector<T> v(vd.begin(), vd.end());
    ShapeRef<T> s{};
    s.kind = SHAPE_MESH;
    s.nverts = int(v.size() / 3);
    s.verts = v.data();
    s.uv_stacks = stacks;
    s.uv_sectors = sectors;
    std::normal_distribution<double> nd(0.0, 1.0);
    std::uniform_real_distribution<double> ud(-1.0, 1.0);
    int bad = 0;
    for (int k = 0; k < ndirs; ++k)
    {
        V3<double> d;
        int mode = k % 6;
        if (mode == 0)
            d = V3<double>{nd(rng), nd(rng), nd(rng)};
        else if (mode == 1)
        { // near a pole
            double e = std::pow(10.0, -6.0 * std::fabs(ud(rng)));
            d = V3<double>{e * ud(rng), (ud(rng) < 0 ? -1.0 : 1.0), e * ud(rng)};
        }
        else if (mode == 2)
        { // exactly on a vertex direction (ties between neighbours are common)
            int i = int(rng() % uint64_t(s.nverts));
            d = V3<double>{vd[3 * i], vd[3 * i + 1], vd[3 * i + 2]};
        }
        else if (mode == 3)
        { // half way between two sectors of a ring
            int i = 1 + int(rng() % uint64_t(stacks - 1));
            double phi = M_PI * i / stacks, th = 2.0 * M_PI * (double(rng() % uint64_t(sectors)) + 0.5) / sectors;
            d = V3<double>{std::sin(phi) * std::cos(th), std::cos(phi), std::sin(phi) * std::sin(th)};
        }
        else if (mode == 4)
        { // half way between two rings
            int i = int(rng() % uint64_t(stacks));
            double phi = M_PI * (i + 0.5) / stacks, th = 2.0 * M_PI * double(rng() % uint64_t(sectors)) / sectors;
            d = V3<double>{std::sin(phi) * std::cos(th), std::cos(phi), std::sin(phi) * std::sin(th)};
        }
        else
        { // axes and diagonals
            int a = int(rng() % 26);
            int x = a % 3 - 1, y = (a / 3) % 3 - 1, z = a / 9 - 1;
            if (x == 0 && y == 0 && z == 0) x = 1;
            d = V3<double>{double(x), double(y), double(z)};
        }
        double sc = std::pow(10.0, 3.0 * ud(rng));
        V3<T> dt{T(d.x * sc), T(d.y * sc), T(d.z * sc)};
        T bd;
        int lin = s.argmax_linear(dt, 0, s.nverts, -1, bd);
        int uv = s.argmax_uv(dt);
        if (lin != uv) ++bad;
    }
    return bad;
}

static std::vector<double> uv_sphere(double r, int stacks, int sectors)
{
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
    v.insert(v.end(), {0.0, -r, 0.0});
    return v;
}

static int check_box(std::mt19937_64 &rng)
{
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::normal_distribution<double> nd(0.0, 1.0);
    int bad = 0;
    for (int b = 0; b < 300; ++b)
    {
        const double sc = std::pow(10.0, 4.0 * u(rng) - 2.0);
        double h[3] = {sc * (0.1 + u(rng)), sc * (0.1 + u(rng)), sc * (0.1 + u(rng))};
        if (b % 10 == 0) h[1] = h[0];            // square faces: exact ties
        if (b % 25 == 0) h[2] = 0.0;             // a flat box
        std::vector<double> v;
        const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}};
        for (int i = 0; i < 8; ++i)
            for (int k = 0; k < 3; ++k) v.push_back(double(sg[i][k]) * h[k]);
        ShapeRef<double> s{};
        s.kind = SHAPE_MESH;
        s.nverts = 8;
        s.verts = v.data();
        s.uv_stacks = kBoxLayout;
        for (int k = 0; k < 2000; ++k)
        {
            V3<double> d{nd(rng), nd(rng), nd(rng)};
            const int mode = k % 5;
            if (mode == 1)
            { // axis and diagonal directions, some components exactly zero or negative zero
                const double c[5] = {0.0, -0.0, 1.0, -1.0, 0.5};
                d = V3<double>{c[rng() % 5], c[rng() % 5], c[rng() % 5]};
            }
            else if (mode == 2)
                d.x = 0.0;
            else if (mode == 3)
                d = V3<double>{d.x * 1e-300, d.y, -0.0};
            double bd;
            if (s.argmax_linear(d, 0, 8, -1, bd) != s.argmax_box(d)) ++bad;
        }
    }
    return bad;
}

int main()
{
    std::mt19937_64 rng(12345);
    int bad_heap = check_heap(rng);
    int bad64 = 0, bad32 = 0;
    for (double r : {0.05, 0.3, 1.0, 7.5})
    {
        auto v = uv_sphere(r, 16, 32);
        bad64 += check_support<double>(v, rng, 20000);
        bad32 += check_support<float>(v, rng, 20000);
    }
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int h = 0; h < 50; ++h)
    {
        std::vector<double> v;
        for (int i = 0; i < 64; ++i)
        {
            double x = nd(rng), y = nd(rng), z = nd(rng), n = std::sqrt(x * x + y * y + z * z);
            v.insert(v.end(), {x / n * 0.4, y / n * 0.4, z / n * 0.4});
        }
        bad64 += check_support<double>(v, rng, 500);
        bad32 += check_support<float>(v, rng, 500);
    }
    int baduv64 = 0, baduv32 = 0;
    int layouts = 0;
    for (int S : {8, 9, 12, 16, 24, 31, 48, 64})
        for (int K : {8, 11, 16, 32, 33, 64})
            for (double r : {0.05, 1.0, 7.5})
            {
                if (!uv_layout_ok(S, K)) continue;
                ++layouts;
                auto v = uv_sphere(r, S, K);
                baduv64 += check_uv<double>(v, S, K, rng, 3000);
                baduv32 += check_uv<float>(v, S, K, rng, 3000);
            }
    const int badbox = check_box(rng);
    std::printf("heap_mismatch=%d support_mismatch_f64=%d support_mismatch_f32=%d uv_mismatch_f64=%d uv_mismatch_f32=%d "
                "uv_layouts=%d box_mismatch=%d\n", bad_heap, bad64, bad32, baduv64, baduv32, layouts, badbox);
    return (bad_heap || bad64 || bad32 || baduv64 || baduv32 || !uv_layout_ok(16, 32) || layouts < 60 || badbox) ? 1 : 0;
}
