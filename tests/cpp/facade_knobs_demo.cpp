// facade_knobs_demo.cpp -- a reference-style caller that changes the solver's
// public knobs between steps and restarts from a macroscopic file:
//   D2Q9 thermal channel (hot wall y = 0 at T 1.5, cold wall y = ny-1 at T
//   0.5, periodic x, downward force 1e-4) set up through initialize_fields;
//   thermal_relaxation_time set after initialisation (initialize_fields
//   resets it to 2, LBM.cpp:461); 20 ticks; velocity_limit lowered; 20 ticks;
//   an invalid thermal_relaxation_time refused and replaced; five ticks at
//   the reference's cadence (iterate_time); one saving tick; the macroscopic
//   fields saved and loaded back; 3 more ticks.  Writes the tick count, the
//   u/rho and F/T fields to a binary file.
//   facade_knobs_demo <nx> <ny> <out.bin> <macro.bin>
#include <cstdio>
#include <cstdlib>

#include "bf/LBM.hpp"

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: %s nx ny out.bin macro.bin\n", argv[0]);
        return 1;
    }
    const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]);
    try {
        bf::LBM solver;
        solver.clear_boundry_properties();
        solver.set_boundry_properties(1, bf::vec3(0, 0, 0), 1.5f);
        solver.set_boundry_properties(2, bf::vec3(0, 0, 0), 0.5f);
        solver.is_collide_esoteric = true;
        solver.boundary_mode = BF_BOUNDARY_BOUNCE_BACK;
        solver.thermal_init_equilibrium = true;
        solver.initialize_fields(
            [&](bf::ivec3 c, bf::LBM::FluidProperties& p) {
                p.force = bf::vec3(0, -1e-4f, 0);
                p.temperature = 1.0f + 0.01f * (float)((c.x * 7 + c.y * 3) % 5 - 2);
                if (c.y == 0) p.boundry_id = 1;
                if (c.y == ny - 1) p.boundry_id = 2;
            },
            bf::ivec3(nx, ny, 1), 0.6f, true, false, true, bf::D2Q9, bf::fp32, false);
        solver.thermal_relaxation_time = 0.8f;
        solver.iterate_time_steps(20, false);
        solver.velocity_limit = 0.001f;
        solver.iterate_time_steps(20, false);
        solver.thermal_relaxation_time = 0.4f;  // invalid: refused at the next step
        bool refused = false;
        try {
            solver.iterate_time_steps(1, false);
        } catch (const bf::LBMError&) {
            refused = true;
        }
        if (!refused) {
            std::fprintf(stderr, "an invalid thermal relaxation time was accepted\n");
            return 4;
        }
        solver.thermal_relaxation_time = 0.8f;
        for (int k = 0; k < 5; k++) solver.iterate_time();
        solver.iterate_time_steps(1, true);
        solver.save_current_tick_macroscopic(argv[4]);
        solver.iterate_time_steps(7, false);
        solver.load_tick_macroscopic(argv[4]);
        solver.iterate_time_steps(3, true);
        solver.synchronize();
        const int32_t ticks = solver.get_total_ticks_elapsed();
        const double elapsed = solver.get_total_time_elapsed().count();
        if (!(elapsed >= 0.0)) return 5;
        std::vector<float> vd = solver.get_velocity_density_texture().copy_to_host<float>();
        std::vector<float> ft = solver.get_force_temperature_texture().copy_to_host<float>();
        FILE* fp = std::fopen(argv[3], "wb");
        if (!fp) return 3;
        std::fwrite(&ticks, 4, 1, fp);
        std::fwrite(vd.data(), sizeof(float), vd.size(), fp);
        std::fwrite(ft.data(), sizeof(float), ft.size(), fp);
        std::fclose(fp);
    } catch (const bf::LBMError& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return e.code == BF_ERR_NO_DEVICE ? 2 : 1;
    }
    return 0;
}
