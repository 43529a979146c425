// lbm_common.cuh -- lattice constants, storage codecs and kernel parameters
// shared by the sm_103a lattice Boltzmann kernels.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace bf {

struct Dir { int x, y, z; };

// Velocity sets in the reference's order (VelocitySet.cpp:53-142, :180-204):
// opposite directions sit in adjacent (odd, odd+1) pairs, which is what the
// AA index arithmetic (collide.comp:219-222) relies on.  Weights are the
// FP32 roundings of the exact fractions, as the reference uploads them.
template <int Q> struct Lattice;

template <> struct Lattice<9> {
    static constexpr int D = 2;
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[9] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0},
                              {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) {
        return i == 0 ? float(4.0 / 9) : (i < 5 ? float(1.0 / 9) : float(1.0 / 36));
    }
    __host__ __device__ static constexpr double wd(int i) {
        return i == 0 ? 4.0 / 9 : (i < 5 ? 1.0 / 9 : 1.0 / 36);
    }
};
template <> struct Lattice<15> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[15] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0},
                               {0, 0, 1}, {0, 0, -1}, {1, 1, 1}, {-1, -1, -1}, {1, 1, -1},
                               {-1, -1, 1}, {1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) {
        return i == 0 ? float(2.0 / 9) : (i < 7 ? float(1.0 / 9) : float(1.0 / 72));
    }
    __host__ __device__ static constexpr double wd(int i) {
        return i == 0 ? 2.0 / 9 : (i < 7 ? 1.0 / 9 : 1.0 / 72);
    }
};
template <> struct Lattice<19> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[19] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0},
                               {0, 0, 1}, {0, 0, -1}, {1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
                               {-1, 1, 0}, {1, 0, 1}, {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                               {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) {
        return i == 0 ? float(1.0 / 3) : (i < 7 ? float(1.0 / 18) : float(1.0 / 36));
    }
    __host__ __device__ static constexpr double wd(int i) {
        return i == 0 ? 1.0 / 3 : (i < 7 ? 1.0 / 18 : 1.0 / 36);
    }
};
template <> struct Lattice<27> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[27] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},  {0, 0, 1},
                               {0, 0, -1},  {1, 1, 0},   {-1, -1, 0}, {1, 0, 1},  {-1, 0, -1}, {0, 1, 1},
                               {0, -1, -1}, {1, -1, 0},  {-1, 1, 0}, {1, 0, -1},  {-1, 0, 1},  {0, 1, -1},
                               {0, -1, 1},  {1, 1, 1},   {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                               {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) {
        return i == 0 ? float(8.0 / 27) : (i < 7 ? float(2.0 / 27) : (i < 19 ? float(1.0 / 54) : float(1.0 / 216)));
    }
    __host__ __device__ static constexpr double wd(int i) {
        return i == 0 ? 8.0 / 27 : (i < 7 ? 2.0 / 27 : (i < 19 ? 1.0 / 54 : 1.0 / 216));
    }
};
// thermal sets D2Q5 / D3Q7
template <int QT> struct ThermalLattice;
template <> struct ThermalLattice<5> {
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[5] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) { return i == 0 ? float(1.0 / 3) : float(1.0 / 6); }
    __host__ __device__ static constexpr double wd(int i) { return i == 0 ? 1.0 / 3 : 1.0 / 6; }
};
template <> struct ThermalLattice<7> {
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[7] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) { return i == 0 ? float(1.0 / 4) : float(1.0 / 8); }
    __host__ __device__ static constexpr double wd(int i) { return i == 0 ? 1.0 / 4 : 1.0 / 8; }
};
// thermal weight in the arithmetic type R
template <int QT, class R> struct ThermalW;
template <int QT> struct ThermalW<QT, float> {
    __host__ __device__ static constexpr float w(int i) { return ThermalLattice<QT>::w(i); }
};
template <int QT> struct ThermalW<QT, double> {
    __host__ __device__ static constexpr double w(int i) { return ThermalLattice<QT>::wd(i); }
};

// the thermal set's directions are the velocity set's first QT directions,
// in the same order, so a flow-lattice source mask also marks the thermal
// lattice's special sources (bits 1 .. QT-1)
template <int Q, int QT>
constexpr bool thermal_dirs_lead() {
    for (int i = 0; i < QT; i++) {
        const Dir a = Lattice<Q>::c(i), b = ThermalLattice<QT>::c(i);
        if (a.x != b.x || a.y != b.y || a.z != b.z) return false;
    }
    return true;
}
static_assert(thermal_dirs_lead<9, 5>() && thermal_dirs_lead<15, 7>() && thermal_dirs_lead<19, 7>() &&
                  thermal_dirs_lead<27, 7>(),
              "thermal directions must lead the velocity set");

// weight of direction i in the arithmetic type R (float: the reference's
// FP32 constants; double: the FP64 reference stepper)
template <int Q, class R> struct LatticeW;
template <int Q> struct LatticeW<Q, float> {
    __host__ __device__ static constexpr float w(int i) { return Lattice<Q>::w(i); }
};
template <int Q> struct LatticeW<Q, double> {
    __host__ __device__ static constexpr double w(int i) { return Lattice<Q>::wd(i); }
};

// collide.comp:219-222: opp(i) = i odd ? i+1 : i-1, opp(0) = 0
__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }

// ---------------------------------------------------------------------------
// storage codecs: encode an FP32 population of direction i for the DDF
// ---------------------------------------------------------------------------
enum Storage { ST_FP32 = 0, ST_FP16 = 1, ST_FP16S = 2, ST_FP16C = 3, ST_FP64 = 4 };

template <int ST> struct Codec;
// T: the stored element type; R: the arithmetic type of the update.
// SHIFTED codecs store the shifted population g = f - w_i and the update
// works on g directly (dec/enc), which drops the two +-w per population and
// keeps the arithmetic on the small deviations; dec_f/enc_f convert from and
// to f itself (initialisation, read-back, snapshots).
// SCALE: the stored value is g * SCALE (a power of two).  raw_dec/raw_enc
// convert without the scale: kernels that run the update on G = g * SCALE
// (every equilibrium and source weight taken times SCALE, the density as
// fma(sum G, 1/SCALE, 1), the momentum times 1/SCALE) get the same bits as
// the update on g, because scaling by a power of two is exact in every
// rounded operation.
template <> struct Codec<ST_FP32> {
    using T = float;
    using R = float;
    static constexpr bool SHIFTED = false;
    static constexpr float SCALE = 1.0f;
    static constexpr int SCALE_EXP = 0;
    __device__ __forceinline__ static R raw_dec(T v) { return dec(v, R(0)); }
    __device__ __forceinline__ static T raw_enc(R v) { return enc(v, R(0)); }
    __device__ __forceinline__ static float dec(T v, float) { return v; }
    __device__ __forceinline__ static T enc(float v, float) { return v; }
    __device__ __forceinline__ static float dec_f(T v, float) { return v; }
    __device__ __forceinline__ static T enc_f(float v, float) { return v; }
};
template <> struct Codec<ST_FP16> {  // R16F: IEEE half of f
    using T = __half;
    using R = float;
    static constexpr bool SHIFTED = false;
    static constexpr float SCALE = 1.0f;
    static constexpr int SCALE_EXP = 0;
    __device__ __forceinline__ static R raw_dec(T v) { return dec(v, R(0)); }
    __device__ __forceinline__ static T raw_enc(R v) { return enc(v, R(0)); }
    __device__ __forceinline__ static float dec(T v, float) { return __half2float(v); }
    __device__ __forceinline__ static T enc(float v, float) { return __float2half_rn(v); }
    __device__ __forceinline__ static float dec_f(T v, float) { return __half2float(v); }
    __device__ __forceinline__ static T enc_f(float v, float) { return __float2half_rn(v); }
};
template <> struct Codec<ST_FP16S> {  // IEEE half of g = f - w
    using T = __half;
    using R = float;
    static constexpr bool SHIFTED = true;
    static constexpr float SCALE = 1.0f;
    static constexpr int SCALE_EXP = 0;
    __device__ __forceinline__ static R raw_dec(T v) { return dec(v, R(0)); }
    __device__ __forceinline__ static T raw_enc(R v) { return enc(v, R(0)); }
    __device__ __forceinline__ static float dec(T v, float) { return __half2float(v); }
    __device__ __forceinline__ static T enc(float g, float) { return __float2half_rn(g); }
    __device__ __forceinline__ static float dec_f(T v, float w) { return __fadd_rn(__half2float(v), w); }
    __device__ __forceinline__ static T enc_f(float v, float w) { return __float2half_rn(__fsub_rn(v, w)); }
};
template <> struct Codec<ST_FP16C> {  // custom-scaled: IEEE half of g * 2^12
    // g = f - w times 2^12 before the conversion: the scaled populations stay
    // in the half's normal range down to |g| = 2^-26 (IEEE half of g itself,
    // fp16s, loses precision below 2^-14), and |g| < 16 fits; one hardware
    // conversion each way, as fp16s
    using T = __half;
    using R = float;
    static constexpr bool SHIFTED = true;
    static constexpr int SCALE_EXP = 12;
    static constexpr float SCALE = float(1 << SCALE_EXP);
    __device__ __forceinline__ static float raw_dec(T v) { return __half2float(v); }
    __device__ __forceinline__ static T raw_enc(float v) { return __float2half_rn(v); }
    __device__ __forceinline__ static float dec(T v, float) { return __fmul_rn(__half2float(v), 1.0f / SCALE); }
    __device__ __forceinline__ static T enc(float g, float) { return __float2half_rn(__fmul_rn(g, SCALE)); }
    __device__ __forceinline__ static float dec_f(T v, float w) { return __fmaf_rn(__half2float(v), 1.0f / SCALE, w); }
    __device__ __forceinline__ static T enc_f(float v, float w) { return __float2half_rn(__fmul_rn(__fsub_rn(v, w), SCALE)); }
};
template <> struct Codec<ST_FP64> {  // FP64 reference stepper: populations and arithmetic in double
    using T = double;
    using R = double;
    static constexpr bool SHIFTED = false;
    static constexpr float SCALE = 1.0f;
    static constexpr int SCALE_EXP = 0;
    __device__ __forceinline__ static R raw_dec(T v) { return dec(v, R(0)); }
    __device__ __forceinline__ static T raw_enc(R v) { return enc(v, R(0)); }
    __device__ __forceinline__ static double dec(T v, double) { return v; }
    __device__ __forceinline__ static T enc(double v, double) { return v; }
    __device__ __forceinline__ static double dec_f(T v, double) { return v; }
    __device__ __forceinline__ static T enc_f(double v, double) { return v; }
};

// ---------------------------------------------------------------------------
// feature switches of the generic step kernel (runtime, uniform per launch)
// ---------------------------------------------------------------------------
enum : uint32_t {
    F_PERIODIC_X = 1u << 0,
    F_PERIODIC_Y = 1u << 1,
    F_PERIODIC_Z = 1u << 2,
    F_BOUNDARIES = 1u << 3,    // packed boundary ids present
    F_BOUNCE_BACK = 1u << 4,   // halfway BB folded into AA
    F_FORCE_CONST = 1u << 5,
    F_FORCE_FIELD = 1u << 6,
    F_THERMAL = 1u << 7,
    F_MULTIPHASE = 1u << 8,
    F_SAVE = 1u << 9,
    F_UPDATE = 1u << 10,       // write populations (0: the reference's save-only first pass)
    F_TRT = 1u << 11,
    F_EQ_BOUNDARIES = 1u << 12,
    F_REDUCE = 1u << 13,
    F_SOURCE = 1u << 14,       // Guo source term active (forcing, thermal or multiphase)
    F_MEASURE = 1u << 15,      // moments only: no thermal / pseudopotential writes
};

// AA access mode of one launch
enum AAMode { AA_EVEN = 0, AA_ODD = 1, AA_LOCAL = 2 };

struct alignas(16) StepParams {
    void* plane[27];          // DDF planes: population slot i of cell n at plane[i][n]
    uint64_t stride;          // elements per population plane (thermal lattice uses the same)
    int nx, ny, nz;
    uint32_t flags;
    uint32_t n_cells;
    int bits;                 // bits per boundary id (0, 1, 2, 4, 8)
    // fast kernel: blocks ahead (in launch order) whose population rows a
    // block prefetches into L2 with bulk copies; 0 = off.  Only set when every
    // population plane starts and ends on a 16-byte boundary.
    uint32_t pf_blocks;
    // 1: the 16-bit fast step may stage its loads through shared memory with
    // bulk copies (lbm_tma.cuh); set by the host when the planes allow it
    uint32_t tma;
    // 1: 16-bit update steps may run two cells per thread (fast2_step_kernel)
    uint32_t two_cell;
    // 1: the two-cell Shan-Chen step stages the psi rows of its block in
    // shared memory (otherwise each neighbour is a cached global load)
    uint32_t psi_tile;
    // 1: the thermal collision pushes each post-collision thermal population
    // to the slot the thermal pull stream would fill with it (th_tgt becomes
    // the next step's pre-collision state; no stream pass).  Set by the host
    // for the split boundary-aware step when the masks mark every special
    // thermal source.
    uint32_t thermal_push;
    // per-cell masks of the boundary-aware fast step (build_mask_kernel):
    // bit i (1..Q-1) = the AA source x - c_i needs special handling (outside
    // the domain, or a solid cell under bounce-back); bit 31 = the cell is
    // solid; bit 30 = the cell is an equilibrium-boundary cell
    const uint32_t* nmask;
    // the cells whose mask is nonzero, in increasing index order
    // (n_special), and a launch schedule (n_sched entries, one per block of
    // masked_mixed_kernel): entry e < 2^31 is a block (x-block bx, row y, z)
    // of the cell grid, packed as below, which updates its cells with an
    // empty mask in the periodic kernel's cell update; entry 2^31 + k updates the listed cells
    // special[k * special_chunk ..] (special_chunk of them, one per thread).
    // When set, the boundary-aware step runs this way.
    const uint32_t* special;
    const uint32_t* special_mask;  // the mask of each listed cell
    const uint32_t* sched;
    uint32_t n_special, n_sched, special_chunk;
    // a plain entry of the schedule packs its block as bx | y << sched_shy |
    // z << sched_shz (bit fields of the grid's x-block count, ny and nz), so
    // that the kernel decodes it with shifts and masks
    uint32_t sched_shy, sched_shz;
    // fast kernel, even step, rows off the y/z faces: element offset of the
    // slot read for direction i relative to the cell, without its x part:
    // i * stride - (c_y nx + c_z nx ny), modulo 2^32
    uint32_t uoff[27];
    // the same in bytes, signed (uoff_b), and the byte offset of plane i
    // (poff_b): the fast kernel adds them to per-thread byte pointers
    int64_t uoff_b[27];
    int64_t poff_b[27];
    // FP64 reference stepper: the launch constants in double, computed as the
    // FP64 oracle does (cs = 1/sqrt(3), tau and the limits from the FP32 inputs)
    struct {
        double R2, R4, R2h, R4h, Rtau, P, Wm, Pp, Pm, vlim, vlim_ext, fconst[3];
        double cs2, cs4, tau, tau_t, beta, G;
    } k64;
    // the FP64 stepper's thermal lattice and pseudopotential (double; the
    // FP32 pointers below serve every other storage)
    const double* th_src64;
    double* th_tgt64;
    const double* psi_src64;
    double* psi_tgt64;
    // the literal evaluation's divisors: cs^2 = cs*cs, cs^4 = cs^2*cs^2 (the
    // shim of pow(cs, 2) / pow(cs, 4)), tau, tau_T
    float cs2, cs4, tau, tau_t;
    // divisors among cs^2 (bit 0), cs^4 (bit 1), tau (bit 2), tau_T (bit 3)
    // for which the host has checked the two-operation division by the split
    // reciprocal (R2 + L2, R4 + L4, Rtau + Ltau, Rtau_t + Ltau_t) against IEEE
    // division for every significand; the fast kernels run only when all four passed
    uint32_t div_ok;
    float L2, L4, Ltau, Ltau_t;  // low parts of 1/cs2, 1/cs4, 1/tau, 1/tau_T (div_m)
    // launch constants, FP32, computed on the host exactly as the oracle
    // does: cs = float(1/sqrt(3)), cs2 = cs*cs, cs4 = cs2*cs2
    float R2;                 // 1/cs2
    float R4;                 // 1/cs4
    float R2h, R4h;           // R2/2, R4/2 (exact halvings)
    float Rtau;               // 1/tau (= TRT omega+)
    float P;                  // 1 - 1/(2 tau), Guo prefactor
    float Wm;                 // TRT omega- = 1/(Lambda/(tau-1/2) + 1/2)
    float Pp, Pm;             // TRT Guo prefactors 1 - omega+/2, 1 - omega-/2
    float vlim, vlim_ext;
    float t_lim, t_ext;       // largest |u|^2 whose IEEE sqrt does not exceed vlim / vlim_ext
    float fconst[3];
    const float4* force;      // per-cell force field (reference vec4 layout)
    const uint32_t* bnd;      // packed boundary ids
    const float4* objects;    // 3 float4 per id: (u,T) (omega,0) (com,rho_eff)
    const uint8_t* obj_kind;  // bf_object_kind per id
    const float4* bvals;      // (rho_b, u_b) per cell for equilibrium boundary cells
    // thermal lattice (SoA, FP32)
    const float* th_src;
    float* th_tgt;
    float Rtau_t, beta;       // 1/tau_T, thermal expansion coefficient
    // Shan-Chen: psi of the effective density, ping-pong
    const float* psi_src;
    float* psi_tgt;
    float G;
    // macroscopic outputs
    float4* vel_den;
    float4* force_temp;
    uint8_t* bnd_tex;
    // FP64 block partials (5 per block) when F_REDUCE
    double* red_partials;
    unsigned int* err;        // bit0: NaN density seen
};

struct StreamParams {
    const void* src;
    void* dst;
    uint64_t stride;
    int nx, ny, nz;
    uint32_t flags;
    int bits;
    const uint32_t* bnd;
    const float4* objects;
    const uint8_t* obj_kind;
};

struct ThermalStreamParams {
    const float* src;
    float* dst;
    // FP64 stepper: the thermal lattice in double (src/dst unused)
    const double* src64;
    double* dst64;
    uint64_t stride;
    int nx, ny, nz;
    uint32_t flags;
    int bits;
    const uint32_t* bnd;
    const float4* objects;
    const uint8_t* obj_kind;
    // the flow lattice's per-cell source masks (build_mask_kernel), set when
    // they mark every special thermal source too (bounce-back mode, or no
    // boundary ids); null: every cell looks its neighbours up
    const uint32_t* nmask;
};

struct InitParams {
    void* f;
    uint64_t stride;
    uint32_t n_cells;
    const float* rho;      // N
    const float* u;        // 3N
    const uint32_t* ids;   // N (may be null)
    const uint8_t* obj_kind;
    // thermal (th64: the FP64 stepper's thermal lattice)
    float* th;
    double* th64;
    const float* T;
    // odd != 0: write the equilibrium state in the slots an odd esoteric-pull
    // step reads (a state loaded at an odd tick): population i of cell n goes
    // to slot opp(i) of n + c_i (dropped outside the domain), and a cell whose
    // source n - c_i lies outside takes its own opp(i) population in slot
    // opp(i), the value the reference's odd step finds there.  nx, ny, nz and
    // flags (F_PERIODIC_*) give the geometry.
    int odd;
    int nx, ny, nz;
    uint32_t flags;
};

__device__ __forceinline__ uint32_t boundary_id(const uint32_t* __restrict__ bnd, int bits, uint64_t cell) {
    if (bits == 0) return 0u;
    uint64_t b = cell * (uint64_t)bits;
    uint32_t word = __ldg(bnd + (b >> 5));
    return (word >> (uint32_t)(b & 31u)) & ((1u << bits) - 1u);
}

// launchers (one translation unit per Q instantiates them)
// kernel choice of one step: the periodic fast kernel, the boundary-aware
// (masked) fast kernel, or the generic kernel
enum StepPath { PATH_FAST = 0, PATH_MASKED = 1, PATH_GENERIC = 2 };
template <int Q> cudaError_t launch_step(const StepParams& p, int storage, int mode, int path, cudaStream_t st);
template <int Q> cudaError_t launch_build_mask(const StepParams& p, uint32_t* mask, cudaStream_t st);
template <int Q> cudaError_t launch_stream(const StreamParams& p, int storage, cudaStream_t st);
template <int Q> cudaError_t launch_init(const InitParams& p, int storage, cudaStream_t st);
template <int Q> cudaError_t launch_decode(const void* f, uint64_t stride, uint32_t n, int storage, float* out, cudaStream_t st);
template <int Q> cudaError_t launch_encode(void* f, uint64_t stride, uint32_t n, int storage, const float* in, cudaStream_t st);
template <int QT> cudaError_t launch_stream_thermal(const ThermalStreamParams& p, cudaStream_t st);
template <int QT> cudaError_t launch_init_thermal(const InitParams& p, cudaStream_t st);

cudaError_t launch_reduce_finish(const double* partials, uint32_t n_blocks, double* out, cudaStream_t st);

// sets the thread's message returned by bf_last_error()
void record_error(const std::string& msg);

#ifndef BF_STEP_BLOCK
#define BF_STEP_BLOCK 256
#endif
constexpr int kStepBlock = BF_STEP_BLOCK;  // threads per block of the step kernels (along x)

}  // namespace bf
