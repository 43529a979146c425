// LBM.hpp -- C++ facade with the member names, argument meaning and
// defaults of BoltzmannFluids' solver class (BoltzmannFluids/Source/LBM/LBM.h:26-145),
// implemented over the C ABI of bf_lbm.h.  Header only: link libbfgb300.so.
//
// Differences a caller of the reference sees:
//  * errors throw bf::LBMError (the reference printed "[LBM Error]" and
//    asserted, LBM.cpp:429-437);
//  * the Texture3D getters return bf::Field, a headless device buffer
//    (pointer + shape) instead of a GL texture; copy_to_host() reads it back;
//  * render3d_* write into a headless RGBA float device image (no graphics
//    stack); render2d_* are not provided.
//
// Beyond the reference: bf::Adjoint, the differentiable channel flow as a
// forward/backward pair (gradients of a drag / velocity-mismatch objective
// with respect to a per-cell solid fraction and the inlet profile).
#pragma once

#include <chrono>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../bf_lbm.h"

namespace bf {

struct ivec3 {
    int32_t x = 0, y = 0, z = 0;
    ivec3() = default;
    ivec3(int32_t x_, int32_t y_, int32_t z_) : x(x_), y(y_), z(z_) {}
    template <class V> ivec3(const V& v) : x((int32_t)v.x), y((int32_t)v.y), z((int32_t)v.z) {}
};
struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    template <class V> vec3(const V& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
};

enum VelocitySet { D2Q9 = BF_D2Q9, D3Q15 = BF_D3Q15, D3Q19 = BF_D3Q19, D3Q27 = BF_D3Q27 };
enum FloatingPointAccuracy {
    fp16 = BF_STORE_FP16,
    fp32 = BF_STORE_FP32,
    fp16s = BF_STORE_FP16S,
    fp16c = BF_STORE_FP16C,
    fp64 = BF_STORE_FP64
};

class LBMError : public std::runtime_error {
public:
    LBMError(int code, const std::string& what) : std::runtime_error("[LBM Error] " + what), code(code) {}
    int code;
};

inline void check(int code) {
    if (code != BF_OK) throw LBMError(code, bf_last_error());
}

// headless stand-in for the reference's shared_ptr<Texture3D>
struct Field {
    bf_field desc{};
    bf_solver* owner = nullptr;
    void* device_ptr() const { return desc.device_ptr; }
    size_t bytes() const { return desc.bytes; }
    template <class T> std::vector<T> copy_to_host() const {
        std::vector<T> out(desc.bytes / sizeof(T));
        check(bf_copy_field_to_host(owner, desc.kind, out.data(), out.size() * sizeof(T)));
        return out;
    }
};

class LBM {
public:
    static constexpr uint32_t not_a_boundry = 0;
    static constexpr uint32_t max_boundry_count = 255;
    static constexpr float referance_temperature = 1.0f;
    static constexpr float referance_boundry_density = 1.0f;

    // LBM::FluidProperties (LBM.h:41-47)
    struct FluidProperties {
        vec3 velocity = vec3(0, 0, 0);
        vec3 force = vec3(0, 0, 0);
        float density = 1;
        float temperature = referance_temperature;
        uint32_t boundry_id = not_a_boundry;
    };

    LBM() { check(bf_create(&s_)); }
    ~LBM() { bf_destroy(s_); }
    LBM(const LBM&) = delete;
    LBM& operator=(const LBM&) = delete;

    // ---- simulation controls (LBM.h:34-38) ----
    // LBM::iterate_time (LBM.cpp:220-240): advances one tick unless a
    // positive target_tick_per_second is already met by the ticks run since
    // the first call; saves the macroscopic fields on the first tick and then
    // only when more than 1000/60 ms (whole milliseconds) have passed since
    // the last save, as the reference's visual update does
    void iterate_time(float target_tick_per_second = 0) {
        const auto now = std::chrono::system_clock::now();
        if (first_iteration_) {
            simulation_begin_ = now;
            last_visual_update_ = now;
        }
        const size_t targeted_tick_count = (size_t)(target_tick_per_second * get_total_time_elapsed().count() / 1000.0f);
        if (target_tick_per_second <= 0 || (size_t)get_total_ticks_elapsed() < targeted_tick_count || first_iteration_) {
            const auto since = std::chrono::system_clock::now() - last_visual_update_;
            const bool save = first_iteration_ ||
                              std::chrono::duration_cast<std::chrono::milliseconds>(since).count() > 1000.0 / 60;
            if (save) last_visual_update_ = std::chrono::system_clock::now();
            sync_knobs();
            check(bf_iterate_time(s_, 1, save ? 1 : 0));
        }
        first_iteration_ = false;
    }
    void iterate_time_steps(int32_t steps, bool save_fields = true) {
        sync_knobs();
        check(bf_iterate_time(s_, steps, save_fields));
    }
    int32_t get_total_ticks_elapsed() {
        int64_t t = 0;
        check(bf_get_total_ticks_elapsed(s_, &t));
        return (int32_t)t;
    }
    // wall-clock time since the first iterate_time call (LBM.cpp:247-250;
    // measured from the clock's epoch before that call, as the reference's
    // default-constructed time point does)
    std::chrono::duration<double, std::milli> get_total_time_elapsed() {
        return std::chrono::system_clock::now() - simulation_begin_;
    }
    ivec3 get_resolution() {
        int32_t r[3];
        check(bf_get_resolution(s_, r));
        return ivec3(r[0], r[1], r[2]);
    }
    int32_t get_velocity_set_vector_count() {
        int32_t q = 0;
        check(bf_get_velocity_set_vector_count(s_, &q));
        return q;
    }

    // ---- initialisation (LBM.h:48-58) ----
    void initialize_fields(std::function<void(ivec3, FluidProperties&)> initialization_lambda, ivec3 resolution,
                           float relaxation_time, bool periodic_x = true, bool periodic_y = true,
                           bool periodic_z = true, VelocitySet velocity_set = D2Q9,
                           FloatingPointAccuracy fp_accuracy = fp32, bool is_flow_multiphase = false) {
        const size_t n = (size_t)resolution.x * resolution.y * resolution.z;
        std::vector<float> rho(n), u(3 * n), f(3 * n), T(n);
        std::vector<uint32_t> ids(n);
        size_t k = 0;
        for (int32_t z = 0; z < resolution.z; z++)
            for (int32_t y = 0; y < resolution.y; y++)
                for (int32_t x = 0; x < resolution.x; x++, k++) {
                    FluidProperties p;
                    initialization_lambda(ivec3(x, y, z), p);
                    rho[k] = p.density;
                    u[3 * k] = p.velocity.x; u[3 * k + 1] = p.velocity.y; u[3 * k + 2] = p.velocity.z;
                    f[3 * k] = p.force.x; f[3 * k + 1] = p.force.y; f[3 * k + 2] = p.force.z;
                    T[k] = p.temperature;
                    ids[k] = p.boundry_id;
                }
        thermal_relaxation_time = 2.0f;  // initialize_fields resets it (LBM.cpp:461)
        bf_init_desc d;
        bf_init_desc_default(&d);
        d.resolution[0] = resolution.x; d.resolution[1] = resolution.y; d.resolution[2] = resolution.z;
        d.relaxation_time = relaxation_time;
        d.periodic[0] = periodic_x; d.periodic[1] = periodic_y; d.periodic[2] = periodic_z;
        d.velocity_set = velocity_set;
        d.storage = fp_accuracy;
        d.multiphase = is_flow_multiphase;
        d.esoteric = is_collide_esoteric;
        d.boundary_mode = boundary_mode;
        d.collision = collision;
        d.trt_magic = trt_magic;
        d.velocity_limit = velocity_limit;
        d.velocity_limit_extreme = velocity_limit_extreme;
        d.intermolecular_interaction_strength = intermolecular_interaction_strength;
        d.thermal_relaxation_time = thermal_relaxation_time;
        d.thermal_expansion_coefficient = thermal_expension_coeficient;
        d.thermal_init_equilibrium = thermal_init_equilibrium;
        d.two_buffer_fixed = two_buffer_fixed;
        check(bf_initialize_fields(s_, &d, rho.data(), u.data(), f.data(), T.data(), ids.data()));
        sent_ = {velocity_limit, velocity_limit_extreme, thermal_relaxation_time, thermal_expension_coeficient};
        velocity_set_ = velocity_set;
        fp_ = fp_accuracy;
        periodic_[0] = periodic_x; periodic_[1] = periodic_y; periodic_[2] = periodic_z;
    }

    // ---- boundary objects (LBM.h:60-82) ----
    void set_boundry_properties(uint32_t boundry_id, vec3 velocity_translational, vec3 velocity_angular,
                                vec3 center_of_mass, float temperature = referance_temperature,
                                float effective_density = referance_boundry_density,
                                bf_object_kind kind = BF_OBJECT_SOLID) {
        bf_object o{};
        o.velocity_translational[0] = velocity_translational.x;
        o.velocity_translational[1] = velocity_translational.y;
        o.velocity_translational[2] = velocity_translational.z;
        o.velocity_angular[0] = velocity_angular.x; o.velocity_angular[1] = velocity_angular.y;
        o.velocity_angular[2] = velocity_angular.z;
        o.center_of_mass[0] = center_of_mass.x; o.center_of_mass[1] = center_of_mass.y;
        o.center_of_mass[2] = center_of_mass.z;
        o.temperature = temperature;
        o.effective_density = effective_density;
        o.kind = kind;
        check(bf_set_boundry_properties(s_, boundry_id, &o));
    }
    void set_boundry_properties(uint32_t boundry_id, vec3 velocity_translational,
                                float temperature = referance_temperature,
                                float effective_density = referance_boundry_density) {
        set_boundry_properties(boundry_id, velocity_translational, vec3(), vec3(), temperature, effective_density);
    }
    void set_boundry_properties(uint32_t boundry_id, float temperature,
                                float effective_density = referance_boundry_density) {
        set_boundry_properties(boundry_id, vec3(), vec3(), vec3(), temperature, effective_density);
    }
    void clear_boundry_properties() { check(bf_clear_boundry_properties(s_)); }

    // ---- readback (LBM.h:97-99) ----
    Field get_velocity_density_texture() { return field(BF_FIELD_VELOCITY_DENSITY); }
    Field get_boundry_texture() { return field(BF_FIELD_BOUNDARY); }
    Field get_force_temperature_texture() { return field(BF_FIELD_FORCE_TEMPERATURE); }

    // ---- low-level getters / setters (LBM.h:105-120) ----
    float get_relaxation_time() {
        float t = 0;
        check(bf_get_relaxation_time(s_, &t));
        return t;
    }
    VelocitySet get_velocity_set() { return velocity_set_; }
    int32_t get_dimentionality() { return velocity_set_ == D2Q9 ? 2 : 3; }
    FloatingPointAccuracy get_floating_point_accuracy() { return fp_; }
    bool get_periodic_boundry_x() { return periodic_[0]; }
    bool get_periodic_boundry_y() { return periodic_[1]; }
    bool get_periodic_boundry_z() { return periodic_[2]; }
    bool get_is_forcing_scheme() { return flags() & 1; }
    bool get_is_force_field_constant() { return flags() & 2; }
    bool get_is_flow_multiphase() { return flags() & 8; }
    vec3 get_constant_force() {
        float f[3];
        check(bf_get_constant_force(s_, f));
        return vec3(f[0], f[1], f[2]);
    }
    float get_intermolecular_interaction_strength() {
        float g = 0;
        check(bf_get_intermolecular_interaction_strength(s_, &g));
        return g;
    }
    void set_relaxation_time(float relaxation_time) { check(bf_set_relaxation_time(s_, relaxation_time)); }
    void set_constant_force(vec3 constant_force) {
        const float f[3] = {constant_force.x, constant_force.y, constant_force.z};
        check(bf_set_constant_force(s_, f));
    }
    void set_intermolecular_interaction_strength(float value) {
        intermolecular_interaction_strength = value;
        check(bf_set_intermolecular_interaction_strength(s_, value));
    }

    // ---- snapshots (LBM.h:123-126, declared but not defined upstream) ----
    void save_current_tick_mesoscropic(const std::string& path) { check(bf_save_snapshot(s_, path.c_str())); }
    void load_tick_mesoscropic(const std::string& path, int32_t target_tick = -1) {
        (void)target_tick;
        check(bf_load_snapshot(s_, path.c_str()));
    }
    // the macroscopic fields (u/rho, F/T, boundary ids) of the last saved tick
    void save_current_tick_macroscopic(const std::string& path) { check(bf_save_macroscopic(s_, path.c_str())); }
    // restart from a macroscopic file: equilibrium populations of its fields,
    // the tick counter set to its tick (target_tick >= 0 must match it)
    void load_tick_macroscopic(const std::string& path, int32_t target_tick = -1) {
        sync_knobs();
        check(bf_load_macroscopic(s_, path.c_str(), target_tick));
    }

    // FP64 {mass, momentum x, y, z, kinetic energy} of the current state (extension)
    std::vector<double> reduce() {
        std::vector<double> out(5);
        check(bf_reduce(s_, out.data()));
        return out;
    }
    void synchronize(int32_t timeout_ms = 0) { check(bf_synchronize(s_, timeout_ms)); }

    // ---- volume rendering (LBM.h render3d_*, LBM.cpp:1207-1376), headless ----
    // view / projection: column-major 4x4 (glm::value_ptr of the camera's
    // matrices); rgba_device: width*height*4 floats on the device
    void render3d_density(const float* view, const float* projection, int32_t width, int32_t height,
                          int32_t sample_count, float* rgba_device, void* stream = nullptr) {
        check(bf_render3d(s_, BF_RENDER_DENSITY, view, projection, width, height, sample_count, rgba_device, stream));
    }
    void render3d_velocity(const float* view, const float* projection, int32_t width, int32_t height,
                           int32_t sample_count, float* rgba_device, void* stream = nullptr) {
        check(bf_render3d(s_, BF_RENDER_VELOCITY, view, projection, width, height, sample_count, rgba_device, stream));
    }
    void render3d_boundries(const float* view, const float* projection, int32_t width, int32_t height,
                            int32_t sample_count, float* rgba_device, void* stream = nullptr) {
        check(bf_render3d(s_, BF_RENDER_BOUNDRIES, view, projection, width, height, sample_count, rgba_device, stream));
    }
    void render3d_forces(const float* view, const float* projection, int32_t width, int32_t height,
                         int32_t sample_count, float* rgba_device, void* stream = nullptr) {
        check(bf_render3d(s_, BF_RENDER_FORCES, view, projection, width, height, sample_count, rgba_device, stream));
    }
    void render3d_temperature(const float* view, const float* projection, int32_t width, int32_t height,
                              int32_t sample_count, float* rgba_device, void* stream = nullptr) {
        check(bf_render3d(s_, BF_RENDER_TEMPERATURE, view, projection, width, height, sample_count, rgba_device,
                          stream));
    }

    // ---- public knobs (LBM.h:139-145, :242-243, :257) + extensions ----
    bool is_lattice_texture3d = false;  // storage layout of the GL path: no effect here
    bool is_collide_esoteric = false;
    float velocity_limit = 0.25f;
    float velocity_limit_extreme = 0.30f;
    float thermal_relaxation_time = 2.0f;       // what initialize_fields sets (LBM.cpp:461)
    float thermal_expension_coeficient = 0.5f;  // LBM.h:243
    float intermolecular_interaction_strength = -6.0f;
    bf_boundary_mode boundary_mode = BF_BOUNDARY_SKIP;
    bf_collision collision = BF_COLLISION_BGK;
    float trt_magic = 0.25f;
    bool thermal_init_equilibrium = false;
    bool two_buffer_fixed = false;

    bf_solver* handle() { return s_; }

private:
    // the public knobs are uniforms the reference sets at every dispatch
    // (LBM.cpp:1590-1591, :1612-1613): changed values reach the solver
    // before the next step
    struct Knobs { float vlim, vext, tau_t, beta; };
    Knobs sent_{0.25f, 0.30f, 2.0f, 0.5f};
    void sync_knobs() {
        if (velocity_limit != sent_.vlim || velocity_limit_extreme != sent_.vext) {
            check(bf_set_velocity_limits(s_, velocity_limit, velocity_limit_extreme));
            sent_.vlim = velocity_limit;
            sent_.vext = velocity_limit_extreme;
        }
        // an invalid value (tau_T <= 0.5) throws here, and again at every
        // later step until the knob holds a valid value
        if (thermal_relaxation_time != sent_.tau_t || thermal_expension_coeficient != sent_.beta) {
            check(bf_set_thermal_parameters(s_, thermal_relaxation_time, thermal_expension_coeficient));
            sent_.tau_t = thermal_relaxation_time;
            sent_.beta = thermal_expension_coeficient;
        }
    }
    Field field(int kind) {
        Field f;
        f.owner = s_;
        check(bf_get_field(s_, kind, &f.desc));
        return f;
    }
    int32_t flags() {
        int32_t fl = 0, bits = 0;
        check(bf_get_scheme_flags(s_, &fl, &bits));
        return fl;
    }
    bf_solver* s_ = nullptr;
    bool first_iteration_ = true;
    std::chrono::system_clock::time_point simulation_begin_{};
    std::chrono::system_clock::time_point last_visual_update_{};
    VelocitySet velocity_set_ = D2Q9;
    FloatingPointAccuracy fp_ = fp32;
    bool periodic_[3] = {true, true, true};
};

// MarchingCubes (BoltzmannFluids/Source/MarchingCubes/MarchingCubes.h): the
// triangle list of a device scalar field, on the GPU.
class MarchingCubes {
public:
    MarchingCubes() { check(bf_mc_create(&m_)); }
    ~MarchingCubes() { bf_mc_destroy(m_); }
    MarchingCubes(const MarchingCubes&) = delete;
    MarchingCubes& operator=(const MarchingCubes&) = delete;

    // the density of an LBM's velocity/density field; returns the triangle count
    uint64_t compute(const Field& velocity_density, float threshold = 1.0f, vec3 mesh_scale = vec3(1, 1, 1),
                     void* stream = nullptr) {
        const float sc[3] = {mesh_scale.x, mesh_scale.y, mesh_scale.z};
        uint64_t n = 0;
        check(bf_mc_compute(m_, static_cast<const float*>(velocity_density.desc.device_ptr), 4, 3,
                            velocity_density.desc.resolution, threshold, sc, stream, &n));
        return n;
    }
    // device vertices: triangle_count * 9 floats, valid until the next compute
    const float* vertices(uint64_t* triangle_count) {
        const float* v = nullptr;
        check(bf_mc_get_vertices(m_, &v, triangle_count));
        return v;
    }
    std::vector<float> vertices_host() {
        uint64_t n = 0;
        vertices(&n);
        std::vector<float> out(n * 9);
        uint64_t w = 0;
        check(bf_mc_copy_vertices_to_host(m_, out.data(), n, &w));
        return out;
    }

private:
    static void check(int code) {
        if (code != BF_OK) throw LBMError(code, bf_last_error());
    }
    bf_marching_cubes* m_ = nullptr;
};

// MeshRasterizer3D::rasterize (MeshRasterizer3D.h:16-19) as a GPU ray-parity
// voxeliser: mask[nx*ny*nz] = 1 for voxels inside the closed mesh
inline std::vector<uint8_t> rasterize_mesh(const std::vector<float>& triangle_vertices, ivec3 resolution,
                                           const float* model_matrix = nullptr, int32_t samples_per_voxel = 64) {
    const int32_t res[3] = {resolution.x, resolution.y, resolution.z};
    std::vector<uint8_t> mask((size_t)resolution.x * resolution.y * resolution.z);
    const int code = bf_voxelize_mesh(triangle_vertices.data(), triangle_vertices.size() / 9, model_matrix, res,
                                      samples_per_voxel, mask.data());
    if (code != BF_OK) throw LBMError(code, bf_last_error());
    return mask;
}

// The discrete adjoint of a channel flow (bf_adjoint_*): forward() runs the
// T-step solve with checkpoints and returns the objective J; backward()
// returns dJ/ds per cell and dJ/du_in per (y, z) row of the last forward, in
// FP64.  Parameters and the target are host arrays, x fastest.
struct AdjointDesc {
    ivec3 resolution = ivec3(512, 256, 1);
    float relaxation_time = 0.6f;
    VelocitySet velocity_set = D2Q9;   // D2Q9 (resolution.z = 1) or D3Q19 (periodic z)
    int32_t steps = 2000;              // T
    int32_t checkpoint_interval = 100; // K
    float drag_weight = 1.0f;
    float mismatch_weight = 1.0f;
    int32_t resident_states = 0;       // 0, R >= K - 1, or BF_ADJOINT_RESIDENT_AUTO (bf_lbm.h)
};

class Adjoint {
public:
    using Desc = AdjointDesc;
    explicit Adjoint(const Desc& d = Desc()) : n_((size_t)d.resolution.x * d.resolution.y * d.resolution.z),
                                               rows_((size_t)d.resolution.y * d.resolution.z) {
        bf_adjoint_desc c;
        bf_adjoint_desc_default(&c);
        c.resolution[0] = d.resolution.x; c.resolution[1] = d.resolution.y; c.resolution[2] = d.resolution.z;
        c.relaxation_time = d.relaxation_time;
        c.velocity_set = (int32_t)d.velocity_set;
        c.steps = d.steps;
        c.checkpoint_interval = d.checkpoint_interval;
        c.drag_weight = d.drag_weight;
        c.mismatch_weight = d.mismatch_weight;
        c.resident_states = d.resident_states;
        check(bf_adjoint_create(&a_, &c));
    }
    ~Adjoint() { bf_adjoint_destroy(a_); }
    Adjoint(const Adjoint&) = delete;
    Adjoint& operator=(const Adjoint&) = delete;

    // solid fraction s[N] in [0, 1] and inlet profile u_in[ny*nz]; an empty vector keeps the current one
    void set_parameters(const std::vector<float>& solid_fraction, const std::vector<float>& inlet_velocity) {
        if (!solid_fraction.empty() && solid_fraction.size() != n_) throw LBMError(BF_ERR_INVALID_ARGUMENT, "solid_fraction size");
        if (!inlet_velocity.empty() && inlet_velocity.size() != rows_) throw LBMError(BF_ERR_INVALID_ARGUMENT, "inlet_velocity size");
        check(bf_adjoint_set_parameters(a_, solid_fraction.empty() ? nullptr : solid_fraction.data(),
                                        inlet_velocity.empty() ? nullptr : inlet_velocity.data()));
    }
    // target velocity u*[3N]
    void set_target(const std::vector<float>& u_target) {
        if (u_target.size() != 3 * n_) throw LBMError(BF_ERR_INVALID_ARGUMENT, "u_target size");
        check(bf_adjoint_set_target(a_, u_target.data()));
    }
    double forward() {
        double j = 0.0;
        check(bf_adjoint_forward(a_, &j));
        return j;
    }
    void backward(std::vector<double>& grad_solid_fraction, std::vector<double>& grad_inlet_velocity) {
        grad_solid_fraction.resize(n_);
        grad_inlet_velocity.resize(rows_);
        check(bf_adjoint_backward(a_, grad_solid_fraction.data(), grad_inlet_velocity.data()));
    }
    // the schedule in use: 0 (segment buffers) or the pool's state count
    int32_t resident_states() const {
        int32_t r = 0;
        check(bf_adjoint_get_resident_states(a_, &r));
        return r;
    }

private:
    bf_adjoint* a_ = nullptr;
    size_t n_, rows_;
};

}  // namespace bf
