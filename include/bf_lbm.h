/*
 * bf_lbm.h -- C ABI of the GB300 lattice Boltzmann solver.
 *
 * Drop-in replacement for the GL compute path behind BoltzmannFluids' solver
 * class `LBM` (BoltzmannFluids/Source/LBM/LBM.h:26-332).  Every entry point
 * below names the reference member it replaces.  Plain C types only: device
 * memory is owned by the solver handle; host arrays are caller-owned and are
 * only read or written during the call.
 *
 * Threading: one solver handle belongs to one host thread at a time (the
 * reference's LBM object is likewise bound to the thread owning its GL
 * context, BoltzmannFluids_UI/Source/GUIApplication/SimulationController.cpp:17).
 * Each handle owns one CUDA stream; all calls are ordered on it.
 *
 * Errors: every call returns a bf_status (0 = BF_OK, negative = error) and
 * records a message retrievable with bf_last_error(); the reference printed
 * "[LBM Error] ..." and asserted (LBM.cpp:429-437, :570-573, :1024-1032).
 */
#ifndef BF_LBM_H
#define BF_LBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BF_ABI_VERSION 1

typedef enum {
    BF_OK = 0,
    BF_ERR_INVALID_ARGUMENT = -1, /* bad size, enum, pointer or order of calls */
    BF_ERR_CUDA = -2,             /* a CUDA runtime call failed */
    BF_ERR_OUT_OF_MEMORY = -3,    /* device allocation failed */
    BF_ERR_NOT_INITIALIZED = -4,  /* bf_initialize_fields has not run */
    BF_ERR_UNSTABLE = -5,         /* the step kernels saw a NaN density */
    BF_ERR_TIMEOUT = -6,          /* a bounded host wait gave up */
    BF_ERR_IO = -7,               /* snapshot file could not be read/written */
    BF_ERR_NO_DEVICE = -8         /* no CUDA device is visible */
} bf_status;

/* VelocitySet (BoltzmannFluids/Source/LBMConstants/VelocitySet.h:18-23): same numeric values. */
typedef enum { BF_D2Q9 = 2, BF_D3Q15 = 3, BF_D3Q19 = 4, BF_D3Q27 = 5 } bf_velocity_set;

/* DDF storage.  BF_STORE_FP16 is the reference's FloatingPointAccuracy::fp16
 * (an R16F lattice: IEEE half of f itself, LBM.cpp:446-449);
 * BF_STORE_FP16S stores IEEE half of the shifted population f_i - w_i;
 * BF_STORE_FP16C ("custom-scaled") stores the IEEE half of (f_i - w_i) * 2^12:
 * the shifted populations keep the half's 11-bit relative precision down to
 * |f_i - w_i| = 2^-26 (fp16s turns subnormal below 2^-14); |f_i - w_i| must
 * stay below 16 (beyond it the half overflows and the step reports
 * BF_ERR_UNSTABLE).
 * Arithmetic is FP32 in these four modes.
 * BF_STORE_FP64 (no counterpart in the reference) is the accuracy reference
 * stepper: FP64 populations, thermal lattice and pseudopotential, and FP64
 * arithmetic in the same operation order as the FP32 path, for every
 * esoteric-pull configuration (boundary objects, open faces, force fields,
 * thermal and multiphase flow; the two-buffer mode fails with
 * BF_ERR_INVALID_ARGUMENT); fields read back as FP32. */
typedef enum {
    BF_STORE_FP32 = 0,
    BF_STORE_FP16 = 1,
    BF_STORE_FP16S = 2,
    BF_STORE_FP16C = 3,
    BF_STORE_FP64 = 4
} bf_storage;

/* How a fluid cell next to a solid cell receives populations in the
 * esoteric (AA, in-place) mode.
 * BF_BOUNDARY_SKIP: as the reference's collide.comp reads it (:696-700):
 *   solid cells are skipped and neighbours read whatever their slots hold.
 * BF_BOUNDARY_BOUNCE_BACK: halfway bounce-back with the moving-wall term of
 *   stream.comp:487-496/576-580 (rho_wall = 1), folded into the AA step. */
typedef enum { BF_BOUNDARY_SKIP = 0, BF_BOUNDARY_BOUNCE_BACK = 1 } bf_boundary_mode;

typedef enum { BF_COLLISION_BGK = 0, BF_COLLISION_TRT = 1 } bf_collision;

/* Boundary object kinds.  The reference only has solid objects; the two
 * equilibrium kinds are extensions: a cell of such an object is updated to
 * f_eq(rho_local, u_b) (velocity) or f_eq(rho_b, u_local) (density), where
 * (rho_b, u_b) are the cell's initial density and velocity and populations
 * that would stream in from outside the domain are taken as f_eq(rho_b, u_b). */
typedef enum { BF_OBJECT_SOLID = 0, BF_OBJECT_EQ_VELOCITY = 1, BF_OBJECT_EQ_DENSITY = 2 } bf_object_kind;

typedef enum {
    BF_FIELD_VELOCITY_DENSITY = 0, /* float4 (u.xyz, rho) per cell: get_velocity_density_texture, LBM.h:97 */
    BF_FIELD_BOUNDARY = 1,         /* uint8 boundary id per cell: get_boundry_texture, LBM.h:98 */
    BF_FIELD_FORCE_TEMPERATURE = 2,/* float4 (F.xyz, T) per cell: get_force_temperature_texture, LBM.h:99 */
    BF_FIELD_POPULATIONS = 3,      /* float per (population, cell), SoA i*N+cell, decoded to FP32 */
    BF_FIELD_THERMAL_POPULATIONS = 4, /* float per (population, cell), SoA */
    BF_FIELD_PSEUDOPOTENTIAL = 5   /* float psi = 1 - exp(-rho_eff) per cell, the Shan-Chen field the
                                      next step reads (the reference's multiphase density texture,
                                      LBM.cpp:848-866, holds rho_eff) */
} bf_field_kind;

typedef struct bf_solver bf_solver;

/* Arguments of LBM::initialize_fields (LBM.h:48-58) plus the public knobs of
 * LBM.h:139-145, :242-243, :257 and the extensions. Fill with
 * bf_init_desc_default() first. */
typedef struct {
    int32_t resolution[3];          /* cells; resolution[2] must be 1 for D2Q9 (LBM.cpp:434-437) */
    float relaxation_time;          /* tau */
    int32_t periodic[3];            /* periodic_x/y/z */
    int32_t velocity_set;           /* bf_velocity_set */
    int32_t storage;                /* bf_storage (fp_accuracy) */
    int32_t multiphase;             /* is_flow_multiphase: Shan-Chen pseudopotential */
    int32_t esoteric;               /* is_collide_esoteric: 1 = AA in place, 0 = two buffers */
    int32_t boundary_mode;          /* bf_boundary_mode (esoteric mode only) */
    int32_t collision;              /* bf_collision */
    float trt_magic;                /* TRT magic parameter Lambda (1/4 by default) */
    float velocity_limit;           /* LBM.h:144 (0.25) */
    float velocity_limit_extreme;   /* LBM.h:145 (0.30) */
    float intermolecular_interaction_strength; /* G, LBM.h:257 (-6) */
    float thermal_relaxation_time;  /* tau_T; initialize_fields sets 2 (LBM.cpp:461) */
    float thermal_expansion_coefficient; /* beta, LBM.h:243 (0.5) */
    int32_t thermal_init_equilibrium;/* 0: as the reference reads (thermal lattice left zero), 1: equilibrium */
    int32_t two_buffer_fixed;       /* esoteric=0 only. 0: reference's swap order (stream reads the
                                       un-collided buffer, LBM.cpp:1646-1647/1509-1513); 1: collide then stream */
    int32_t reserved[8];
} bf_init_desc;

/* Fills the defaults of LBM.h (tau 0.53, periodic, D2Q9, fp32, limits 0.25/0.30,
 * G -6, tau_T 2, beta 0.5, two-buffer, skip boundaries, BGK, Lambda 1/4). */
void bf_init_desc_default(bf_init_desc* desc);

/* Object record, the 3 x vec4 layout of LBM.cpp:613-626 plus a kind. */
typedef struct {
    float velocity_translational[3];
    float temperature;
    float velocity_angular[3];
    float center_of_mass[3];
    float effective_density;
    int32_t kind;                   /* bf_object_kind */
} bf_object;

/* device view of a field (headless stand-in for the reference's Texture3D) */
typedef struct {
    void* device_ptr;
    int32_t kind;                   /* bf_field_kind */
    int32_t resolution[3];
    int32_t components;             /* 4, 1 */
    int32_t bytes_per_component;    /* 4 or 1 */
    size_t bytes;
} bf_field;

/* ---- host-only lattice helpers (no device needed) ----------------------- */
/* get_velosity_vectors (VelocitySet.cpp:53-142, :180-204): writes count*4
 * floats (c.x, c.y, c.z, w) of the flow set (BF_D2Q9..BF_D3Q27) or, with
 * thermal != 0, of its thermal set (D2Q5 for D2Q9, D3Q7 otherwise).
 * out may be NULL to query *count. */
int bf_get_velosity_vectors(int32_t velocity_set, int32_t thermal, float* out, int32_t* count);
/* bits per boundary id for a given object count (LBM.cpp:569): 0, 1, 2, 4 or 8 */
int bf_bits_per_boundry(int32_t object_count, int32_t* bits);
/* packs one id per cell into uint32 words, `bits` per id, low bits first,
 * exactly as LBM.cpp:634-659.  out may be NULL to query *words. */
int bf_pack_boundries(const uint32_t* ids, size_t cells, int32_t bits, uint32_t* out, size_t capacity_words,
                      size_t* words);

/* ---- lifetime ---------------------------------------------------------- */
/* LBM::LBM (implicit constructor).  Selects the current CUDA device. */
int bf_create(bf_solver** out);
/* LBM::~LBM: frees every device buffer of the handle. */
int bf_destroy(bf_solver* s);
/* message of the last failed call on this thread */
const char* bf_last_error(void);
int bf_abi_version(void);
/* Host-side fault injection for tests: after `n` further successful device
 * allocations of the solver's buffers the next one fails as out of memory
 * (BF_ERR_OUT_OF_MEMORY from the call that made it); n < 0 turns it off. */
int bf_debug_fail_allocation_after(int32_t n);

/* ---- boundary objects (LBM.h:60-82) ------------------------------------ */
/* LBM::set_boundry_properties (all three overloads, LBM.cpp:1015-1065). id in 1..255. */
int bf_set_boundry_properties(bf_solver* s, uint32_t boundry_id, const bf_object* object);
/* LBM::clear_boundry_properties (LBM.cpp:1067-1070) */
int bf_clear_boundry_properties(bf_solver* s);

/* ---- initialisation ---------------------------------------------------- */
/* LBM::initialize_fields (LBM.cpp:415-506) given the per-cell results of the
 * initialisation lambda as host arrays of N = rx*ry*rz cells, x fastest:
 *   density[N]   (NULL: 1)         velocity[3N] (NULL: 0)
 *   force[3N]    (NULL: 0)         temperature[N] (NULL: 1)
 *   boundry_id[N] (NULL: all 0)
 * Derives the forcing/constant-force/thermal switches and the packed boundary
 * bits exactly as LBM.cpp:523-569, uploads, writes equilibrium populations
 * and runs the reference's save-only first pass (LBM.cpp:502).  A density or
 * velocity array in page-locked memory (cudaHostAlloc / cudaHostRegister) is
 * read in place by the initialisation kernel; others are copied first.  The
 * arrays are not used after the call returns. */
int bf_initialize_fields(bf_solver* s, const bf_init_desc* desc,
                         const float* density, const float* velocity, const float* force,
                         const float* temperature, const uint32_t* boundry_id);

/* ---- time stepping ----------------------------------------------------- */
/* LBM::iterate_time (LBM.cpp:220-240) run n_steps times with
 * target_tick_per_second = 0.  save_fields != 0 writes the macroscopic fields
 * on the last step (the reference's 60 Hz "collide_save" variant).  Steps are
 * launched from a captured CUDA graph per batch; the call returns once the
 * work is queued (use bf_synchronize to wait). */
int bf_iterate_time(bf_solver* s, int32_t n_steps, int32_t save_fields);
/* the handle's CUDA stream (a cudaStream_t, created non-blocking): work a
 * caller enqueues on it runs after the solver's queued steps */
int bf_get_stream(bf_solver* s, void** stream);
/* waits for the handle's stream; gives up with BF_ERR_TIMEOUT after timeout_ms
 * (<= 0: wait without limit), and returns BF_ERR_UNSTABLE if a step saw NaN. */
int bf_synchronize(bf_solver* s, int32_t timeout_ms);

/* ---- getters / setters (LBM.h:35-38, :105-120) -------------------------- */
int bf_get_total_ticks_elapsed(bf_solver* s, int64_t* ticks);
int bf_get_resolution(bf_solver* s, int32_t resolution[3]);
int bf_get_velocity_set_vector_count(bf_solver* s, int32_t* q);
int bf_get_relaxation_time(bf_solver* s, float* tau);
int bf_set_relaxation_time(bf_solver* s, float tau);
int bf_get_constant_force(bf_solver* s, float force[3]);
int bf_set_constant_force(bf_solver* s, const float force[3]);
int bf_get_intermolecular_interaction_strength(bf_solver* s, float* g);
int bf_set_intermolecular_interaction_strength(bf_solver* s, float g);
int bf_set_velocity_limits(bf_solver* s, float limit, float limit_extreme);
int bf_set_thermal_parameters(bf_solver* s, float thermal_relaxation_time, float thermal_expansion_coefficient);
/* flags: bit0 forcing scheme, bit1 constant force field, bit2 thermal, bit3
 * multiphase, bit4 boundaries present; bits_per_boundry as LBM.cpp:569 */
int bf_get_scheme_flags(bf_solver* s, int32_t* flags, int32_t* bits_per_boundry);

/* ---- field readback (LBM.h:97-99, LBM.cpp:1444-1457) -------------------- */
/* device pointer + shape of a field; valid until the next bf_initialize_fields/bf_destroy */
int bf_get_field(bf_solver* s, int32_t kind, bf_field* out);
/* copies a field to host memory (bytes must be at least the field's size);
 * a 16-byte aligned page-locked destination is written by a copy kernel over
 * the CPU-GPU link, any other by cudaMemcpy; returns when the copy is done */
int bf_copy_field_to_host(bf_solver* s, int32_t kind, void* dst, size_t bytes);
/* packed boundary words as built by LBM.cpp:634-659 (count in *words) */
int bf_copy_boundry_bits_to_host(bf_solver* s, uint32_t* dst, size_t capacity_words, size_t* words);

/* ---- conservation reductions (FP64) ------------------------------------ */
/* Sums over non-solid cells of the last saved step: out = {mass, momentum x,
 * y, z, kinetic energy 0.5*rho*|u|^2}.  Runs one step with field saving and
 * a fused FP64 block reduction if the last step did not save. No counterpart
 * in the reference. */
int bf_reduce(bf_solver* s, double out[5]);

/* ---- timing ------------------------------------------------------------ */
/* Runs n_steps steps (no field saving) between two CUDA events recorded on
 * the handle's stream and returns the elapsed device time in milliseconds.
 * No counterpart in the reference, which only counts ticks (LBM.cpp:242-250). */
int bf_benchmark_steps(bf_solver* s, int32_t n_steps, float* ms);

/* ---- snapshots (LBM.h:123-126, declared but never defined upstream) ------ */
/* mesoscopic (LBM::save_current_tick_mesoscropic / load_tick_mesoscropic,
 * LBM.h:124, :126): the whole state -- populations, thermal and
 * pseudopotential buffers, the tick -- restored exactly */
int bf_save_snapshot(bf_solver* s, const char* path);
int bf_load_snapshot(bf_solver* s, const char* path);
/* macroscopic (LBM::save_current_tick_macroscopic, LBM.h:123): the fields of
 * the last saved step -- u/rho, F/T and the boundary ids per cell -- and
 * that step's tick, written through a temporary file renamed when complete */
int bf_save_macroscopic(bf_solver* s, const char* path);
/* LBM::load_tick_macroscopic (LBM.h:125): the solver (initialised with the
 * file's resolution; geometry, objects and knobs are kept) restarts from the
 * file's fields: every cell's populations become the equilibrium of its
 * saved (rho, u), a thermal lattice the equilibrium of its saved T, the tick
 * counter the file's tick, and the fields are saved as at initialisation.
 * target_tick >= 0 must equal the file's tick (else BF_ERR_INVALID_ARGUMENT);
 * -1 takes the file's.  A file of another size leaves the state as it was. */
int bf_load_macroscopic(bf_solver* s, const char* path, int32_t target_tick);

/* ---- differentiable channel flow and its discrete adjoint ---------------- */
/* No counterpart in the reference (it has no adjoint).  A forward/backward
 * pair over the model
 *   pull   g_i(x) = f_i(x - c_i); halfway bounce-back walls where the source
 *          is outside in y; g_i = feq_i(1, (u_in(y,z),0,0)) where it is outside
 *          in x (equilibrium inlet and outlet); periodic in z
 *   BGK    g^c = g + (feq(rho,u) - g)/tau,   PSM  f_i = (1-s) g^c_i + s g_opp(i)
 *   f^0 = feq(1, (u_in,0,0)),  J = wd sum 2 s j_x + wm sum |u - u*|^2 at step T,
 * D2Q9 (resolution[2] = 1) or D3Q19.  bf_adjoint_forward runs T steps and
 * stores a checkpoint every checkpoint_interval steps; bf_adjoint_backward
 * recomputes the states it needs from the checkpoints and runs the
 * hand-written adjoint (transposed pull and transposed BGK/PSM Jacobian),
 * accumulating dJ/ds (per cell) and dJ/du_in (per (y,z) row) in FP64.
 *
 * resident_states picks how much of the trajectory stays in device memory:
 *   0   two segment buffers of K states: the forward leaves the last segment
 *       in one, and the backward recomputes every earlier segment from its
 *       checkpoint into the other while it sweeps (D2Q9 runs both in one
 *       launch per step);
 *   R>0 the forward leaves its last min(R, T-1) states in a pool of R state
 *       slots; the backward sweeps them, then recomputes the earlier states
 *       from the checkpoints in chunks of up to R states into the same pool
 *       (R >= K - 1; with R >= T - 1 nothing is recomputed);
 *   BF_ADJOINT_RESIDENT_AUTO  R as large as the device memory free at
 *       bf_adjoint_create allows, less a reserve of max(8 GiB, 5% of the
 *       device), between K - 1 and T - 1.
 * Every schedule gives bit-identical gradients: the same adjoint steps on the
 * same states in the same order. */
#define BF_ADJOINT_RESIDENT_AUTO (-1)
typedef struct bf_adjoint bf_adjoint;
typedef struct {
    int32_t resolution[3];
    float relaxation_time;
    int32_t velocity_set;          /* BF_D2Q9 or BF_D3Q19 */
    int32_t steps;                 /* T */
    int32_t checkpoint_interval;   /* K */
    float drag_weight;             /* wd */
    float mismatch_weight;         /* wm */
    int32_t resident_states;       /* 0, R > 0 or BF_ADJOINT_RESIDENT_AUTO (above) */
    int32_t reserved[7];
} bf_adjoint_desc;
/* 512 x 256 x 1 D2Q9, tau 0.6, T 2000, K 100, wd = wm = 1, resident_states 0 */
void bf_adjoint_desc_default(bf_adjoint_desc* desc);
int bf_adjoint_create(bf_adjoint** out, const bf_adjoint_desc* desc);
int bf_adjoint_destroy(bf_adjoint* a);
/* host arrays: solid fraction s[N] (x fastest), inlet profile u_in[ny*nz]; either may be NULL to keep it */
int bf_adjoint_set_parameters(bf_adjoint* a, const float* solid_fraction, const float* inlet_velocity);
/* host array u*[3N] */
int bf_adjoint_set_target(bf_adjoint* a, const float* u_target);
/* forward solve; *objective = J (FP64 sum) */
int bf_adjoint_forward(bf_adjoint* a, double* objective);
/* gradients of the last forward's J: grad_solid_fraction[N], grad_inlet_velocity[ny*nz] (host, FP64) */
int bf_adjoint_backward(bf_adjoint* a, double* grad_solid_fraction, double* grad_inlet_velocity);
/* mean device milliseconds of `repeats` forward and backward passes (CUDA events) */
int bf_adjoint_time(bf_adjoint* a, int32_t repeats, float* forward_ms, float* backward_ms);
/* the schedule's resident state count: 0 (two segment buffers) or the pool's R */
int bf_adjoint_get_resident_states(const bf_adjoint* a, int32_t* resident_states);

/* ---- marching cubes ------------------------------------------------------ */
/* Replaces MarchingCubes::compute (BoltzmannFluids/Source/MarchingCubes/
 * MarchingCubes.cpp:3-47, GLSL/MarchingCubes/marching_cubes.comp:41-97), which
 * binds its buffers but never dispatches.  The mesh it sets out to build is
 * computed on the GPU: voxels between lattice nodes are classified by which
 * corner values are >= threshold, triangle counts are prefix-summed, and each
 * voxel writes its triangles (3 vertices x 3 floats, interpolated on the cut
 * edges) at its offset, in voxel order (x fastest).  Vertex coordinates map
 * node i to -0.5 + i / resolution per axis (marching_cubes.comp:52), times
 * mesh_scale (NULL: 1).  Triangles are oriented with normals pointing from
 * the >= threshold side outward.  The case table is derived, not copied;
 * bf_mc_case_table returns it (host only, no GPU needed). */
typedef struct bf_marching_cubes bf_marching_cubes;
int bf_mc_create(bf_marching_cubes** out);
int bf_mc_destroy(bf_marching_cubes* m);
/* field: device array of resolution[0]*resolution[1]*resolution[2] cells with
 * `components` floats each; the value used is float `component` of each cell
 * (the density of BF_FIELD_VELOCITY_DENSITY is components 4, component 3).
 * Runs on `stream` (NULL: the legacy default stream) and returns once the
 * mesh is complete; at most 2^32/5 voxels. */
int bf_mc_compute(bf_marching_cubes* m, const float* field, int32_t components, int32_t component,
                  const int32_t resolution[3], float threshold, const float mesh_scale[3], void* stream,
                  uint64_t* triangle_count);
/* device pointer to the last mesh: triangle_count * 9 floats, owned by m */
int bf_mc_get_vertices(bf_marching_cubes* m, const float** vertices_device, uint64_t* triangle_count);
int bf_mc_copy_vertices_to_host(bf_marching_cubes* m, float* out, uint64_t max_triangles, uint64_t* written);
/* triangles[256*15]: edge numbers (-1 padded), counts[256]; corner k sits at
 * (k&1, k>>1&1, k>>2&1), edge 4d+j joins the j-th corner with bit d clear to
 * its neighbour along axis d */
int bf_mc_case_table(int8_t* triangles, uint8_t* counts);

/* ---- mesh voxeliser ----------------------------------------------------- */
/* Replaces MeshRasterizer3D::rasterize(mesh, target_texture, model_matrix)
 * (BoltzmannFluids/Source/MeshRasterizer3D/MeshRasterizer3D.cpp:7-113), which
 * renders the mesh in 64 depth slabs per voxel layer and toggles a per-pixel
 * inside/outside parity (raster_unifier.comp:18-35).  Here one ray per voxel
 * column (i, j) through its centre finds the mesh crossings on the GPU; the
 * sorted crossing depths bound the inside intervals (an odd count leaves the
 * rest of the column inside), and voxel (i, j, k) is solid (mask 1) when one
 * of its `samples_per_voxel` depth samples lies inside.  vertices: host array
 * of triangle_count * 9 floats; model: column-major 4x4 (NULL: identity)
 * mapping the mesh into the cube [-1, 1]^3 that spans the volume; column i
 * is centred at x = -1 + (2i+1)/nx (likewise y), depth samples at
 * z = -1 + 2(k + (s+1/2)/samples)/nz.  mask: host array of nx*ny*nz bytes
 * (x fastest).  Layer k grows with z (the reference's camera looks down -z,
 * so its layer 0 is the top). */
int bf_voxelize_mesh(const float* vertices, uint64_t triangle_count, const float model[16],
                     const int32_t resolution[3], int32_t samples_per_voxel, uint8_t* mask);

/* ---- headless volume rendering ------------------------------------------ */
/* Replaces LBM::render3d_density / _velocity / _boundries / _forces /
 * _temperature (BoltzmannFluids/Source/LBM/LBM.cpp:1207-1376 with the
 * fragment shaders GLSL/Renderer3D/*_volumetric.frag), which draw into the
 * current GL framebuffer.  A CUDA kernel marches one ray per pixel through
 * the unit cube [-0.5, 0.5]^3 holding the fields of the last saved step and
 * writes straight (not premultiplied) RGBA floats, row 0 at the bottom, into
 * rgba_device (width*height*4 floats; compose over a background with
 * src_alpha / one_minus_src_alpha as the reference's blending does).  view
 * and projection are column-major 4x4 camera matrices (glm layout).  Pixels
 * whose ray misses the cube are (0, 0, 0, 0).  Runs on `stream` after the
 * solver's queued work and returns when the image is complete. */
typedef enum {
    BF_RENDER_DENSITY = 0,
    BF_RENDER_VELOCITY = 1,
    BF_RENDER_BOUNDRIES = 2,
    BF_RENDER_FORCES = 3,
    BF_RENDER_TEMPERATURE = 4
} bf_render_mode;
int bf_render3d(bf_solver* s, int32_t mode, const float view[16], const float projection[16], int32_t width,
                int32_t height, int32_t sample_count, float* rgba_device, void* stream);

/* ---- allocation-free reduction ------------------------------------------ */
/* No counterpart in the reference.  FP64 {mass, momentum x, y, z, kinetic
 * energy 0.5*rho*|u|^2} of n_cells float4 (u.xyz, rho) cells in device
 * memory (the layout of BF_FIELD_VELOCITY_DENSITY), written to the host
 * array out[5].  Meant for callers that must not allocate device memory --
 * a renderer or UI frame callback working under a fixed memory budget, or
 * code that must not stall other streams (cudaFree synchronizes the whole
 * device): it calls no cudaMalloc, cudaFree or allocating library routine.
 * Its scratch is one fixed 327,744-byte device array that every GPU loading
 * the library keeps until the process exits; that limits a call to
 * 134,217,728 cells (512^3), and larger counts return
 * BF_ERR_INVALID_ARGUMENT, as does a field pointer off a 16-byte boundary.
 * The work runs on `stream` and the call returns once it is done.  NULL
 * selects the legacy default stream, which is NOT ordered after a solver's
 * own stream (created non-blocking): to reduce a solver's field, pass the
 * solver's stream (bf_get_stream) or call bf_synchronize first.  The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  All calls share the
 * array and every call overwrites what it reads, so calls that overlap on
 * the GPU (different streams or host threads) race: serialise them. */
int bf_reduce_field_noalloc(const void* vel_den_device, size_t n_cells, void* stream, double out[5]);

#ifdef __cplusplus
}
#endif
#endif
