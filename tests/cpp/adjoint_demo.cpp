// adjoint_demo.cpp -- the C++ facade's bf::Adjoint: reads a channel's solid
// fraction, inlet profile and target velocity (float32, x fastest) from a
// file, runs forward() and backward(), writes J and both gradients (float64).
// usage: adjoint_demo nx ny nz steps K in.bin out.bin
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bf/LBM.hpp"

int main(int argc, char** argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s nx ny nz steps K in.bin out.bin\n", argv[0]);
        return 1;
    }
    bf::Adjoint::Desc d;
    d.resolution = bf::ivec3(std::atoi(argv[1]), std::atoi(argv[2]), std::atoi(argv[3]));
    d.velocity_set = d.resolution.z == 1 ? bf::D2Q9 : bf::D3Q19;
    d.steps = std::atoi(argv[4]);
    d.checkpoint_interval = std::atoi(argv[5]);
    const size_t n = (size_t)d.resolution.x * d.resolution.y * d.resolution.z;
    const size_t rows = (size_t)d.resolution.y * d.resolution.z;
    std::vector<float> s(n), u_in(rows), target(3 * n);
    FILE* in = std::fopen(argv[6], "rb");
    if (!in || std::fread(s.data(), 4, n, in) != n || std::fread(u_in.data(), 4, rows, in) != rows ||
        std::fread(target.data(), 4, 3 * n, in) != 3 * n) {
        std::fprintf(stderr, "cannot read %s\n", argv[6]);
        return 1;
    }
    std::fclose(in);
    try {
        bf::Adjoint adj(d);
        adj.set_parameters(s, u_in);
        adj.set_target(target);
        const double j = adj.forward();
        std::vector<double> gs, gu;
        adj.backward(gs, gu);
        FILE* out = std::fopen(argv[7], "wb");
        if (!out) return 1;
        std::fwrite(&j, 8, 1, out);
        std::fwrite(gs.data(), 8, gs.size(), out);
        std::fwrite(gu.data(), 8, gu.size(), out);
        std::fclose(out);
    } catch (const bf::LBMError& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 2;
    }
    return 0;
}
