// lbm_common.cuh -- lattice constants, storage codecs and kernel parameters
// shared by the sm_103a lattice Boltzmann kernels.
#pragma once
#include <cstdint>
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
};
// thermal sets D2Q5 / D3Q7
template <int QT> struct ThermalLattice;
template <> struct ThermalLattice<5> {
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[5] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) { return i == 0 ? float(1.0 / 3) : float(1.0 / 6); }
};
template <> struct ThermalLattice<7> {
    __host__ __device__ static constexpr Dir c(int i) {
        constexpr Dir t[7] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        return t[i];
    }
    __host__ __device__ static constexpr float w(int i) { return i == 0 ? float(1.0 / 4) : float(1.0 / 8); }
};

// collide.comp:219-222: opp(i) = i odd ? i+1 : i-1, opp(0) = 0
__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }

// ---------------------------------------------------------------------------
// storage codecs: encode an FP32 population of direction i for the DDF
// ---------------------------------------------------------------------------
enum Storage { ST_FP32 = 0, ST_FP16 = 1, ST_FP16S = 2, ST_FP16C = 3 };

// custom 1-4-11 float: normal 2^(e-13)*(1+m/2048), e=1..15; subnormal
// 2^-12*m/2048; saturating; round to nearest even.  Integer-only code.
__device__ __forceinline__ uint16_t encode_c16(float f) {
    uint32_t x = __float_as_uint(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t mag = x & 0x7fffffffu;
    if (mag > 0x7f800000u) return (uint16_t)sign;
    if (mag >= 0x40fff800u) return (uint16_t)(sign | 0x7fffu);
    if (mag < 0x39800000u) {
        if (mag < 0x33800000u) return (uint16_t)sign;
        uint32_t m = (mag & 0x7fffffu) | 0x800000u;
        uint32_t shift = 127u - (mag >> 23);
        uint32_t q = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        q += (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;
        return (uint16_t)(sign | q);
    }
    uint32_t q = (((mag >> 23) - 114u) << 11) | ((mag & 0x7fffffu) >> 12);
    uint32_t rem = mag & 0xfffu;
    q += (rem > 0x800u || (rem == 0x800u && (q & 1u))) ? 1u : 0u;
    return (uint16_t)(sign | q);
}
__device__ __forceinline__ float decode_c16(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 11) & 0xfu, m = h & 0x7ffu;
    if (e == 0) {
        float v = (float)m * 1.1920928955078125e-07f;
        return __uint_as_float(__float_as_uint(v) | sign);
    }
    return __uint_as_float(sign | ((e + 114u) << 23) | (m << 12));
}

template <int ST> struct Codec;
template <> struct Codec<ST_FP32> {
    using T = float;
    __device__ __forceinline__ static float dec(T v, float) { return v; }
    __device__ __forceinline__ static T enc(float v, float) { return v; }
};
template <> struct Codec<ST_FP16> {  // R16F: IEEE half of f
    using T = __half;
    __device__ __forceinline__ static float dec(T v, float) { return __half2float(v); }
    __device__ __forceinline__ static T enc(float v, float) { return __float2half_rn(v); }
};
template <> struct Codec<ST_FP16S> {  // IEEE half of f - w
    using T = __half;
    __device__ __forceinline__ static float dec(T v, float w) { return __half2float(v) + w; }
    __device__ __forceinline__ static T enc(float v, float w) { return __float2half_rn(v - w); }
};
template <> struct Codec<ST_FP16C> {  // custom 16-bit of (f - w)/w
    using T = uint16_t;
    __device__ __forceinline__ static float dec(T v, float w) { return fmaf(decode_c16(v), w, w); }
    __device__ __forceinline__ static T enc(float v, float w) { return encode_c16((v - w) * (1.0f / w)); }
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
    void* f;                  // DDF, SoA: population i of cell n at f[i*stride + n]
    uint64_t stride;          // elements per population plane
    int nx, ny, nz;
    uint32_t flags;
    uint32_t n_cells;
    int bits;                 // bits per boundary id (0, 1, 2, 4, 8)
    // collision constants (host-computed from the reference's FP32 values)
    float inv_tau;            // 1/tau
    float src_pref;           // 1 - 1/(2 tau)
    float inv_cs2;            // 1/cs^2 with cs = float(1/sqrt(3))
    float half_inv_cs4;       // 1/(2 cs^4)
    float half_inv_cs2;       // 1/(2 cs^2)
    float inv_cs4;            // 1/cs^4
    float trt_inv_tau_minus;  // TRT omega-
    float vlim, vlim_ext;
    float fconst[3];
    const float4* force;      // per-cell force field (reference vec4 layout)
    const uint32_t* bnd;      // packed boundary ids
    const float4* objects;    // 3 float4 per id: (u,T) (omega,0) (com,rho_eff)
    const uint8_t* obj_kind;  // bf_object_kind per id
    const float4* bvals;      // (rho_b, u_b) per cell for equilibrium boundary cells
    // thermal lattice (SoA, FP32)
    const float* th_src;
    float* th_tgt;
    float inv_tau_t, beta;
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
    uint64_t stride;
    int nx, ny, nz;
    uint32_t flags;
    int bits;
    const uint32_t* bnd;
    const float4* objects;
    const uint8_t* obj_kind;
};

struct InitParams {
    void* f;
    uint64_t stride;
    uint32_t n_cells;
    const float* rho;      // N
    const float* u;        // 3N
    const uint32_t* ids;   // N (may be null)
    const uint8_t* obj_kind;
    // thermal
    float* th;
    const float* T;
};

__device__ __forceinline__ uint32_t boundary_id(const uint32_t* __restrict__ bnd, int bits, uint64_t cell) {
    if (bits == 0) return 0u;
    uint64_t b = cell * (uint64_t)bits;
    uint32_t word = __ldg(bnd + (b >> 5));
    return (word >> (uint32_t)(b & 31u)) & ((1u << bits) - 1u);
}

// launchers (one translation unit per Q instantiates them)
template <int Q> cudaError_t launch_step(const StepParams& p, int storage, int mode, bool generic, cudaStream_t st);
template <int Q> cudaError_t launch_stream(const StreamParams& p, int storage, cudaStream_t st);
template <int Q> cudaError_t launch_init(const InitParams& p, int storage, cudaStream_t st);
template <int Q> cudaError_t launch_decode(const void* f, uint64_t stride, uint32_t n, int storage, float* out, cudaStream_t st);
template <int Q> cudaError_t launch_encode(void* f, uint64_t stride, uint32_t n, int storage, const float* in, cudaStream_t st);
template <int QT> cudaError_t launch_stream_thermal(const ThermalStreamParams& p, cudaStream_t st);
template <int QT> cudaError_t launch_init_thermal(const InitParams& p, cudaStream_t st);

cudaError_t launch_reduce_finish(const double* partials, uint32_t n_blocks, double* out, cudaStream_t st);

constexpr int kStepBlock = 256;

}  // namespace bf
