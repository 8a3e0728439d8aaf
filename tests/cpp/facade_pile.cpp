// Steps a pile of boxes through the C++20 facade (include/physkit_gb300.hpp), the way code written
// against the reference's world API would: world_desc / object_desc builders, create_rigid,
// step, remove_rigid, get_rigid.
//
//   facade_pile <scene.bin> <steps> <out.bin>
//
// scene.bin: int32 n, then per body 33 doubles: type, hx, hy, hz, pos3, quat4 (w first), vel3,
// ang_vel3, mass, inertia9, restitution, friction (float64, little endian). Halfway through, the
// last body is removed; its handle must then read back as stale. out.bin: int32 nslots, the state
// rows (14 doubles per slot), int32 npairs, the pair keys.
// Exit codes: 0 ok, 2 usage or file error, 3 no CUDA device (the facade threw physkit_gb300::error
// with PK_ERR_NO_DEVICE), 4 a check failed.
#include "physkit_gb300.hpp"

#include <cstdio>
#include <vector>

namespace pk = physkit_gb300;

int main(int argc, char **argv)
{
    if (argc != 4) return 2;
    // object(object_desc) without a mesh throws, as in the reference (object.h:119-122)
    bool threw = false;
    try
    {
        (void)pk::object_desc::dynam().with_mass(2.0).to_c();
    }
    catch (const std::invalid_argument &)
    {
        threw = true;
    }
    if (!threw) return 4;
    std::printf("missing mesh: std::invalid_argument\n");

    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t n = 0;
    if (std::fread(&n, 4, 1, f) != 1) return 2;
    std::vector<double> rec(size_t(n) * 33);
    if (std::fread(rec.data(), 8, rec.size(), f) != rec.size()) return 2;
    std::fclose(f);
    const int steps = std::atoi(argv[2]);

    try
    {
        pk::world w(pk::world_desc::make()
                        .with_gravity({0.0, -9.81, 0.0})
                        .with_solver_iterations(10)
                        .with_precision(pk::precision::f64)
                        .with_capacity(n + 16));
        std::vector<pk::object_desc> descs;
        for (int i = 0; i < n; ++i)
        {
            const double *r = rec.data() + size_t(i) * 33;
            pk::mesh m = w.make_box({r[1], r[2], r[3]});
            pk::mat3 I;
            for (int k = 0; k < 9; ++k) I[size_t(k)] = r[21 + k];
            auto d = (r[0] != 0.0 ? pk::object_desc::stat() : pk::object_desc::dynam())
                         .with_pos({r[4], r[5], r[6]})
                         .with_orientation({r[7], r[8], r[9], r[10]})
                         .with_vel({r[11], r[12], r[13]})
                         .with_ang_vel({r[14], r[15], r[16]})
                         .with_mass(r[17])
                         .with_inertia_tensor(I)
                         .with_restitution(r[30])
                         .with_friction(r[31])
                         .with_mesh(m);
            descs.push_back(d);
        }
        // the first body one by one, the rest in one call
        std::vector<pk::handle> h{w.create_rigid(descs[0])};
        auto rest = w.create_rigids(std::span<const pk::object_desc>(descs).subspan(1));
        h.insert(h.end(), rest.begin(), rest.end());
        for (int s = 0; s < steps; ++s)
        {
            if (s == steps / 2)
            {
                if (!w.remove_rigid(h.back())) return 4;
                if (w.remove_rigid(h.back())) return 4;      // second removal: stale
                if (w.get_rigid(h.back()).has_value()) return 4; // get_rigid: nullopt
            }
            w.step(1.0 / 120.0);
        }
        if (!w.get_rigid(h.front()).has_value()) return 4;
        const std::vector<double> &rows = w.read_all();
        const std::vector<uint64_t> pairs = w.pairs();
        FILE *o = std::fopen(argv[3], "wb");
        if (!o) return 2;
        const int32_t ns = int32_t(rows.size() / 14), np = int32_t(pairs.size());
        std::fwrite(&ns, 4, 1, o);
        std::fwrite(rows.data(), 8, rows.size(), o);
        std::fwrite(&np, 4, 1, o);
        std::fwrite(pairs.data(), 8, pairs.size(), o);
        std::fclose(o);
        std::printf("stepped %d bodies x %d steps through the facade; %d pairs\n", n, steps, np);
    }
    catch (const pk::error &e)
    {
        std::printf("%s\n", e.what());
        return e.code() == PK_ERR_NO_DEVICE ? 3 : 4;
    }
    return 0;
}
