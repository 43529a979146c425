// A reference-style caller of the C++ facade: the D2Q9 lid-driven cavity set
// up through LBM::initialize_fields with a per-cell lambda (as the
// reference's demos do, BoltzmannFluids/Source/Demos/LBMDemo2D.cpp), run
// for N ticks, and the velocity/density field written to a binary file.
//   lid_cavity_demo <n> <steps> <out.bin>
#include <cstdio>
#include <cstdlib>

#include "bf/LBM.hpp"

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 64;
    const int steps = argc > 2 ? std::atoi(argv[2]) : 100;
    const char* out = argc > 3 ? argv[3] : "cavity.bin";
    try {
        bf::LBM solver;
        solver.clear_boundry_properties();
        solver.set_boundry_properties(1, bf::vec3(0, 0, 0));
        solver.set_boundry_properties(2, bf::vec3(0.1f, 0, 0));
        solver.is_collide_esoteric = true;
        solver.boundary_mode = BF_BOUNDARY_BOUNCE_BACK;
        solver.initialize_fields(
            [&](bf::ivec3 c, bf::LBM::FluidProperties& p) {
                if (c.x == 0 || c.x == n - 1 || c.y == 0) p.boundry_id = 1;
                if (c.y == n - 1) p.boundry_id = 2;
            },
            bf::ivec3(n, n, 1), 0.6f, false, false, true, bf::D2Q9, bf::fp32, false);
        solver.iterate_time_steps(steps, true);
        solver.synchronize();
        std::vector<float> f = solver.get_velocity_density_texture().copy_to_host<float>();
        FILE* fp = std::fopen(out, "wb");
        if (!fp) return 3;
        std::fwrite(f.data(), sizeof(float), f.size(), fp);
        std::fclose(fp);
        std::printf("ticks %d cells %zu\n", solver.get_total_ticks_elapsed(), f.size() / 4);
    } catch (const bf::LBMError& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return e.code == BF_ERR_NO_DEVICE ? 2 : 1;
    }
    return 0;
}
