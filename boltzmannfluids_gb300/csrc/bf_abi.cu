// bf_abi.cu -- the C ABI of include/bf_lbm.h: solver state, initialisation,
// the per-step driver (LBM::_iterate_time / _collide / _stream /
// _stream_thermal, BoltzmannFluids/Source/LBM/LBM.cpp:1484-1773) and readback.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bf_lbm.h"
#include "lbm_common.cuh"
#include "scan.cuh"

using namespace bf;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define BF_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA,  \
                        std::string(#call " failed: ") + cudaGetErrorString(e_));              \
    } while (0)

constexpr int kMaxObjects = 256;  // ids 0..255 (LBM.h:29)
constexpr int kGraphSteps = 16;   // steps per captured graph (even: the AA state has period 2)

// host-side fault injection (bf_debug_fail_allocation_after): the number of
// further device allocations that succeed before one fails as out of
// memory; negative = off
int g_alloc_failure_countdown = -1;

struct DeviceBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DeviceBuf() = default;
    DeviceBuf(const DeviceBuf&) = delete;
    DeviceBuf& operator=(const DeviceBuf&) = delete;
    // a buffer is freed when it goes out of scope (staging buffers of an
    // initialisation; the solver releases its own explicitly as well)
    ~DeviceBuf() { release(); }
    cudaError_t alloc(size_t n) {
        release();
        if (n == 0) return cudaSuccess;
        if (g_alloc_failure_countdown == 0) {
            g_alloc_failure_countdown = -1;
            return cudaErrorMemoryAllocation;
        }
        if (g_alloc_failure_countdown > 0) g_alloc_failure_countdown--;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n; else p = nullptr;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

int q_of(int vs) {
    switch (vs) {
    case BF_D2Q9: return 9;
    case BF_D3Q15: return 15;
    case BF_D3Q19: return 19;
    case BF_D3Q27: return 27;
    }
    return 0;
}
size_t storage_bytes(int st) { return st == BF_STORE_FP64 ? 8 : (st == BF_STORE_FP32 ? 4 : 2); }
// element size of the thermal lattice and the pseudopotential field (double
// for the FP64 stepper, float otherwise)
size_t aux_bytes(int st) { return st == BF_STORE_FP64 ? 8 : 4; }

// LBM.cpp:569 / :606: bits per id = exp2(ceil(log2(ceil(log2(count))))), 0 for one object
int bits_per_boundry(int count) {
    if (count <= 1) return 0;
    return (int)std::exp2(std::ceil(std::log2f(std::ceil(std::log2f((float)count)))));
}

}  // namespace

void bf::record_error(const std::string& msg) { g_last_error = msg; }

struct bf_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool initialized = false;
    bf_init_desc desc{};
    int Q = 0, QT = 0, dims = 0;
    uint32_t N = 0;
    // host copies of the object table (slot 0 = fluid)
    std::vector<bf_object> objects;
    // derived switches (LBM.cpp:523-556)
    bool forcing = false, constant_force = true, thermal = false, boundaries = false;
    float fconst[3] = {0, 0, 0};
    int bits = 0;
    size_t bnd_words = 0;
    bool has_eq_objects = false;
    // device memory
    DeviceBuf lat[2], bnd, objs, kinds, force, bvals, th[2], psi[2];
    DeviceBuf vel_den, force_temp, bnd_tex, partials, red_out, err, decode_tmp;
    DeviceBuf nmask;  // per-cell masks of the boundary-aware fast step
    DeviceBuf special;        // the cells with a nonzero mask, in index order
    DeviceBuf special_mask;   // their masks, in the same order
    DeviceBuf sched;          // launch schedule of the boundary-aware step (StepParams::sched)
    uint32_t n_special = 0, n_sched = 0, special_chunk = 0;
    uint32_t sched_shy = 0, sched_shz = 0;  // bit positions of y and z in a plain schedule entry
    uint32_t n_blocks = 0;
    // buffer roles (LBM.h:280-291)
    int lat0_src = 1, th0_src = 1, psi0_src = 1;
    int64_t ticks = 0;
    int64_t fields_tick = 0;  // tick of the step whose fields vel_den / force_temp hold
    bool last_saved = false;
    // graphs keyed by the state that repeats every two steps
    std::map<int, cudaGraphExec_t> graphs;
    bool graphs_enabled = true;
    uint32_t pf_blocks = 0;  // L2 prefetch distance of the fast kernel, in blocks (0 = off)
    uint32_t pf_blocks32 = 0;  // the same for FP32 storage
    uint32_t pf_blocks_masked = 0;  // the same for the boundary-aware step, in schedule entries
    bool tma_step = false;   // 16-bit fast step with loads staged by bulk copies
    // two-cell Shan-Chen step with the psi rows staged in shared memory by bulk
    // copies: 0 off (the default: 256^3 D3Q19 with cached stencil loads 61.6k
    // MLUPs for fp16s and 61.4k for fp16c, staged 60.4k and 61.0k), 1 on
    // (BF_PSI_TILE)
    int psi_tile = 0;
    bool masked_step = true; // boundary-aware fast step for objects and open faces
    bool two_cell = true;    // 16-bit fast step with two cells per thread
    bool masked_split = true; // boundary-aware step with the special cells in blocks of their own
    bool zero_copy = true;    // kernels read/write pinned host buffers directly (initial velocity, field read-back)
    bool thermal_push = true; // split boundary-aware step: thermal stream folded into the collision
    bool pushed_thermal = false;  // the last collide pushed (no thermal stream pass to follow)
};

namespace {

// device address of a page-locked, mapped host buffer (cudaHostAlloc or
// cudaHostRegister, as torch's pin_memory does), or null for any other
// pointer: kernels read and write such buffers directly over the CPU-GPU link
const void* mapped_host_ptr(const void* p) {
    cudaPointerAttributes at{};
    if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// 16-byte copy between device memory and a mapped host buffer
__global__ void copy16_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, uint64_t n16) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__global__ void ids_to_bytes_kernel(const uint32_t* __restrict__ ids, uint32_t n, uint8_t* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint8_t)ids[i];
}

__global__ void d2f_kernel(const double* __restrict__ a, uint64_t n, float* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)a[i];
}

__global__ void fill_f32_kernel(float* __restrict__ p, uint32_t n, float v) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void special_flags_kernel(const uint32_t* __restrict__ mask, uint64_t n, uint32_t* __restrict__ flag) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = mask[i] != 0u ? 1u : 0u;
}

__global__ void special_scatter_kernel(const uint32_t* __restrict__ mask, const uint32_t* __restrict__ offset,
                                       uint64_t n, uint32_t* __restrict__ list, uint32_t* __restrict__ list_mask) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && mask[i] != 0u) {
        list[offset[i]] = (uint32_t)i;
        list_mask[offset[i]] = mask[i];
    }
}

// first list position of each block of the cell grid (lower bound of the
// block's first cell index in the sorted list); entry n_blocks = count
__global__ void special_ptr_kernel(const uint32_t* __restrict__ list, uint32_t count, uint32_t n_blocks,
                                   uint32_t grid_x, uint32_t block, uint32_t nx, uint32_t* __restrict__ ptr) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > n_blocks) return;
    if (b == n_blocks) { ptr[b] = count; return; }
    const uint64_t first = (uint64_t)(b % grid_x) * block + (uint64_t)(b / grid_x) * nx;
    uint32_t lo = 0, hi = count;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if ((uint64_t)list[mid] < first) lo = mid + 1; else hi = mid;
    }
    ptr[b] = lo;
}

// the list of cells with a nonzero mask, in increasing index order (an
// exclusive scan of the 0/1 flags gives each listed cell its position),
// and each cell-grid block's range of it
cudaError_t build_special_list(bf_solver* s, uint64_t n) {
    s->special.release();
    s->special_mask.release();
    s->sched.release();
    s->n_special = 0;
    s->n_sched = 0;
    if (n == 0) return cudaSuccess;
    ScanLevels scan;
    cudaError_t e = scan.reserve(n);
    if (e != cudaSuccess) return e;
    const uint32_t* mask = s->nmask.as<uint32_t>();
    const unsigned blocks = (unsigned)((n + 255) / 256);
    special_flags_kernel<<<blocks, 256, 0, s->stream>>>(mask, n, scan.levels[0]);
    e = scan.scan(0, n, s->stream);
    uint32_t last[2] = {0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last[0], scan.levels[0] + (n - 1), 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last[1], mask + (n - 1), 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    const uint32_t count = last[0] + (last[1] != 0u ? 1u : 0u);
    if (e == cudaSuccess && count > 0) {
        e = s->special.alloc((size_t)count * sizeof(uint32_t));
        if (e == cudaSuccess) e = s->special_mask.alloc((size_t)count * sizeof(uint32_t));
        if (e == cudaSuccess) {
            special_scatter_kernel<<<blocks, 256, 0, s->stream>>>(mask, scan.levels[0], n, s->special.as<uint32_t>(),
                                                                  s->special_mask.as<uint32_t>());
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
    scan.release();
    if (e == cudaSuccess && count > 0) {
        // the step kernels' cell grid (cell_grid() in lbm_kernels.cuh)
        const uint32_t nx = (uint32_t)s->desc.resolution[0];
        const uint32_t block = nx >= (uint32_t)kStepBlock ? (uint32_t)kStepBlock : (nx + 31) / 32 * 32;
        const uint32_t grid_x = (nx + block - 1) / block;
        const uint32_t n_blocks = grid_x * (uint32_t)s->desc.resolution[1] * (uint32_t)s->desc.resolution[2];
        DeviceBuf ptr_dev;
        std::vector<uint32_t> ptr((size_t)n_blocks + 1);
        e = ptr_dev.alloc(ptr.size() * sizeof(uint32_t));
        if (e == cudaSuccess) {
            special_ptr_kernel<<<(unsigned)((n_blocks + 1 + 255) / 256), 256, 0, s->stream>>>(
                s->special.as<uint32_t>(), count, n_blocks, grid_x, block, nx, ptr_dev.as<uint32_t>());
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ptr.data(), ptr_dev.p, ptr.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        ptr_dev.release();
        if (e == cudaSuccess) {
            // each grid block, then every chunk of listed cells whose last
            // cell lies in the blocks launched so far; a block whose cells
            // are all listed is left out.  Chunks of 32 / 64 / 128 / 256
            // cells measured 30.9k / 31.4k / 32.0k / 31.8k MLUPs on flow past
            // a sphere (256x128x128 D3Q19 TRT)
#ifndef BF_SPECIAL_CHUNK
#define BF_SPECIAL_CHUNK 128
#endif
            const uint32_t chunk = std::min<uint32_t>(BF_SPECIAL_CHUNK, block);
            const uint32_t chunks = (count + chunk - 1) / chunk;
            // plain entries hold bx | y << shy | z << shz: the bit widths of
            // grid_x, ny and nz must fit in 31 bits, else no schedule is built
            // (the one-pass boundary-aware step runs instead)
            auto bits = [](uint32_t v) { uint32_t b = 0; while ((1ull << b) < v) b++; return b; };
            const uint32_t ny = (uint32_t)s->desc.resolution[1], nz = (uint32_t)s->desc.resolution[2];
            const uint32_t shy = bits(grid_x), shz = shy + bits(ny);
            const bool packable = shz + bits(nz) <= 31;
            std::vector<uint32_t> sched;
            if (packable) {
                sched.reserve((size_t)n_blocks + chunks);
                uint32_t c = 0;
                for (uint32_t b = 0; b < n_blocks; b++) {
                    const uint32_t bx = b % grid_x, yz = b / grid_x;
                    const uint32_t width = std::min<uint32_t>(block, nx - bx * block);
                    if (ptr[b + 1] - ptr[b] < width) sched.push_back(bx | (yz % ny) << shy | (yz / ny) << shz);
                    while (c < chunks && std::min<uint64_t>((uint64_t)(c + 1) * chunk, count) <= ptr[b + 1])
                        sched.push_back(0x80000000u | c++);
                }
                while (c < chunks) sched.push_back(0x80000000u | c++);
            }
            if (!sched.empty()) e = s->sched.alloc(sched.size() * sizeof(uint32_t));
            if (e == cudaSuccess && !sched.empty())
                e = cudaMemcpy(s->sched.p, sched.data(), sched.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
            if (e == cudaSuccess && !sched.empty()) {
                s->n_sched = (uint32_t)sched.size();
                s->special_chunk = chunk;
                s->sched_shy = shy;
                s->sched_shz = shz;
            }
        }
    }
    if (e == cudaSuccess) s->n_special = count;
    return e;
}

void clear_graphs(bf_solver* s) {
    for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
}

void release_all(bf_solver* s) {
    clear_graphs(s);
    DeviceBuf* bufs[] = {&s->lat[0], &s->lat[1], &s->bnd, &s->objs, &s->kinds, &s->force, &s->bvals,
                         &s->th[0], &s->th[1], &s->psi[0], &s->psi[1], &s->vel_den, &s->force_temp,
                         &s->bnd_tex, &s->partials, &s->red_out, &s->err, &s->decode_tmp, &s->nmask,
                         &s->special, &s->special_mask, &s->sched};
    for (auto* b : bufs) b->release();
    s->n_special = 0;
    s->n_sched = 0;
    s->initialized = false;
}

void* lat_src(bf_solver* s) { return s->lat[s->lat0_src ? 0 : 1].p; }
void* lat_tgt(bf_solver* s) { return s->lat[s->lat0_src ? 1 : 0].p; }
float* th_src(bf_solver* s) { return s->th[s->th0_src ? 0 : 1].as<float>(); }
float* th_tgt(bf_solver* s) { return s->th[s->th0_src ? 1 : 0].as<float>(); }
float* psi_src(bf_solver* s) { return s->psi[s->psi0_src ? 0 : 1].as<float>(); }
float* psi_tgt(bf_solver* s) { return s->psi[s->psi0_src ? 1 : 0].as<float>(); }
void* th_src_v(bf_solver* s) { return s->th[s->th0_src ? 0 : 1].p; }
void* th_tgt_v(bf_solver* s) { return s->th[s->th0_src ? 1 : 0].p; }
void* psi_src_v(bf_solver* s) { return s->psi[s->psi0_src ? 0 : 1].p; }
void* psi_tgt_v(bf_solver* s) { return s->psi[s->psi0_src ? 1 : 0].p; }

cudaError_t dispatch_step(bf_solver* s, const StepParams& p, int mode, int path) {
    switch (s->Q) {
    case 9: return launch_step<9>(p, s->desc.storage, mode, path, s->stream);
    case 15: return launch_step<15>(p, s->desc.storage, mode, path, s->stream);
    case 19: return launch_step<19>(p, s->desc.storage, mode, path, s->stream);
    case 27: return launch_step<27>(p, s->desc.storage, mode, path, s->stream);
    }
    return cudaErrorInvalidValue;
}

uint32_t base_flags(bf_solver* s) {
    uint32_t fl = 0;
    if (s->desc.periodic[0]) fl |= F_PERIODIC_X;
    if (s->desc.periodic[1]) fl |= F_PERIODIC_Y;
    if (s->desc.periodic[2]) fl |= F_PERIODIC_Z;
    if (s->boundaries) fl |= F_BOUNDARIES;
    if (s->boundaries && s->desc.esoteric && s->desc.boundary_mode == BF_BOUNDARY_BOUNCE_BACK) fl |= F_BOUNCE_BACK;
    if (s->forcing && s->constant_force) fl |= F_FORCE_CONST;
    if (s->forcing && !s->constant_force) fl |= F_FORCE_FIELD;
    if (s->thermal) fl |= F_THERMAL;
    if (s->desc.multiphase) fl |= F_MULTIPHASE;
    if (s->desc.collision == BF_COLLISION_TRT) fl |= F_TRT;
    if (s->has_eq_objects) fl |= F_EQ_BOUNDARIES;
    // collide.comp:609: the source term is compiled in with forcing, multiphase or thermal flow
    if (s->forcing || s->desc.multiphase || s->thermal) fl |= F_SOURCE;
    return fl;
}

// Largest float y with sqrtf(y) <= lim (IEEE sqrt is monotone), so that
// "uu > y" decides exactly as "sqrtf(uu) > lim" (collide.comp:723-724).
float sqrt_threshold(float lim) {
    if (!(lim >= 0.0f)) return -1.0f;  // negative or NaN limit: every cell is limited
    if (std::isinf(lim)) return INFINITY;
    float y = lim * lim;
    while (std::sqrt(y) <= lim && std::isfinite(y)) y = std::nextafter(y, INFINITY);
    while (std::sqrt(y) > lim) y = std::nextafter(y, -INFINITY);
    return y;
}

// Whether x / y == fma(x, r, RN(x l)) with r = RN(1/y), for every
// significand of x (so for every x whose quotient and x l stay normal), l the
// low part of the split reciprocal: RN(1/y - r) from the double reciprocal,
// else the first of its float neighbours up to four steps away (nearer
// first) for which the sequence passes.  Split reciprocals give the correctly
// rounded quotient for most divisors (Brisebarre, Muller and Raina, IEEE
// Trans. Computers 53(8), 2004); the exhaustive check decides for each one.
// The fast kernels then divide by the launch-uniform y in two operations.
// Results are kept per divisor (the knobs change rarely).
bool division_checked(float y, float* lo) {
    static std::mutex mu;
    static std::map<uint32_t, std::pair<bool, float>> seen;
    uint32_t key;
    std::memcpy(&key, &y, 4);
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = seen.find(key);
        if (it != seen.end()) {
            *lo = it->second.second;
            return it->second.first;
        }
    }
    bool ok = false;
    float l_ok = 0.0f;
    if (std::isfinite(y) && y != 0.0f) {
        const float r = 1.0f / y;
        const float l0 = (float)(1.0 / (double)y - (double)r);
        auto passes = [&](float l) {
            for (uint32_t m = 0; m < (1u << 23); m++) {
                const uint32_t xb = 0x3f800000u | m;
                float x;
                std::memcpy(&x, &xb, 4);
                const float t = x * l;
                if (std::fma(x, r, t) != x / y) return false;
            }
            return true;
        };
        // l0, then one float up, one down, two up, two down, ...
        for (int k = 0; k <= 8 && !ok; k++) {
            float l = l0;
            for (int j = 0; j < (k + 1) / 2; j++) l = std::nextafter(l, (k & 1) ? INFINITY : -INFINITY);
            if (passes(l)) {
                ok = true;
                l_ok = l;
            }
        }
    }
    std::lock_guard<std::mutex> lock(mu);
    seen[key] = {ok, l_ok};
    *lo = l_ok;
    return ok;
}

void fill_constants(bf_solver* s, StepParams& p) {
    // the reference's FP32 constants: cs = float(1/sqrt(3)) (LBM.cpp:1587)
    const float cs = (float)(1.0 / std::sqrt(3.0));
    const float cs2 = cs * cs, cs4 = cs2 * cs2;
    const float tau = s->desc.relaxation_time;
    p.R2 = 1.0f / cs2;
    p.R4 = 1.0f / cs4;
    p.cs2 = cs2;
    p.cs4 = cs4;
    p.tau = tau;
    p.tau_t = s->desc.thermal_relaxation_time;
    p.div_ok = (division_checked(cs2, &p.L2) ? 1u : 0u) | (division_checked(cs4, &p.L4) ? 2u : 0u) |
               (division_checked(tau, &p.Ltau) ? 4u : 0u) | (division_checked(p.tau_t, &p.Ltau_t) ? 8u : 0u);
    p.R2h = p.R2 * 0.5f;
    p.R4h = p.R4 * 0.5f;
    p.Rtau = 1.0f / tau;
    p.P = 1.0f - 1.0f / (2.0f * tau);
    const float tau_minus = s->desc.trt_magic / (tau - 0.5f) + 0.5f;
    p.Wm = 1.0f / tau_minus;
    p.Pp = 1.0f - p.Rtau * 0.5f;
    p.Pm = 1.0f - p.Wm * 0.5f;
    p.vlim = s->desc.velocity_limit;
    p.vlim_ext = s->desc.velocity_limit_extreme;
    p.t_lim = sqrt_threshold(p.vlim);
    p.t_ext = sqrt_threshold(p.vlim_ext);
    p.fconst[0] = s->fconst[0]; p.fconst[1] = s->fconst[1]; p.fconst[2] = s->fconst[2];
    p.Rtau_t = 1.0f / s->desc.thermal_relaxation_time;
    p.beta = s->desc.thermal_expansion_coefficient;
    p.G = s->desc.intermolecular_interaction_strength;
    // FP64 reference stepper: the same constants in double from the same inputs
    const double cs_d = 1.0 / std::sqrt(3.0);
    const double cs2_d = cs_d * cs_d, cs4_d = cs2_d * cs2_d;
    const double tau_d = (double)tau;
    p.k64.R2 = 1.0 / cs2_d;
    p.k64.R4 = 1.0 / cs4_d;
    p.k64.cs2 = cs2_d;
    p.k64.cs4 = cs4_d;
    p.k64.tau = tau_d;
    p.k64.tau_t = (double)s->desc.thermal_relaxation_time;
    p.k64.beta = (double)s->desc.thermal_expansion_coefficient;
    p.k64.G = (double)s->desc.intermolecular_interaction_strength;
    p.k64.R2h = p.k64.R2 * 0.5;
    p.k64.R4h = p.k64.R4 * 0.5;
    p.k64.Rtau = 1.0 / tau_d;
    p.k64.P = 1.0 - 1.0 / (2.0 * tau_d);
    p.k64.Wm = 1.0 / ((double)s->desc.trt_magic / (tau_d - 0.5) + 0.5);
    p.k64.Pp = 1.0 - p.k64.Rtau * 0.5;
    p.k64.Pm = 1.0 - p.k64.Wm * 0.5;
    p.k64.vlim = (double)s->desc.velocity_limit;
    p.k64.vlim_ext = (double)s->desc.velocity_limit_extreme;
    for (int k = 0; k < 3; k++) p.k64.fconst[k] = (double)s->fconst[k];
}

template <int Q>
void fill_uoff(StepParams& p, size_t elem) {
    const uint32_t nx = (uint32_t)p.nx, nxy = (uint32_t)p.nx * (uint32_t)p.ny;
    for (int i = 0; i < Q; i++) {
        const Dir c = Lattice<Q>::c(i);
        p.uoff[i] = (uint32_t)i * (uint32_t)p.stride - ((uint32_t)c.y * nx + (uint32_t)c.z * nxy);
        const int64_t e = (int64_t)i * (int64_t)p.stride - ((int64_t)c.y * nx + (int64_t)c.z * nxy);
        p.uoff_b[i] = e * (int64_t)elem;
        p.poff_b[i] = (int64_t)i * (int64_t)p.stride * (int64_t)elem;
    }
}

// LBM::_collide (LBM.cpp:1557-1653): one launch of the fused AA step, then the swaps
cudaError_t collide(bf_solver* s, bool save, bool update, bool reduce, bool measure) {
    StepParams p{};
    {
        char* base = static_cast<char*>(lat_src(s));
        const size_t plane_bytes = (size_t)s->N * storage_bytes(s->desc.storage);
        for (int i = 0; i < s->Q; i++) p.plane[i] = base + (size_t)i * plane_bytes;
    }
    p.stride = s->N;
    p.nx = s->desc.resolution[0]; p.ny = s->desc.resolution[1]; p.nz = s->desc.resolution[2];
    p.n_cells = s->N;
    p.flags = base_flags(s);
    if (save) p.flags |= F_SAVE;
    if (update) p.flags |= F_UPDATE;
    if (reduce) p.flags |= F_REDUCE;
    if (measure) p.flags |= F_MEASURE;
    p.bits = s->bits;
    fill_constants(s, p);
    p.force = s->force.as<float4>();
    p.bnd = s->bnd.as<uint32_t>();
    p.objects = s->objs.as<float4>();
    p.obj_kind = s->kinds.as<uint8_t>();
    p.bvals = s->bvals.as<float4>();
    const bool f64 = s->desc.storage == BF_STORE_FP64;
    if (s->thermal) {
        if (f64) { p.th_src64 = static_cast<const double*>(th_src_v(s)); p.th_tgt64 = static_cast<double*>(th_tgt_v(s)); }
        else { p.th_src = th_src(s); p.th_tgt = th_tgt(s); }
    }
    if (s->desc.multiphase) {
        if (f64) { p.psi_src64 = static_cast<const double*>(psi_src_v(s)); p.psi_tgt64 = static_cast<double*>(psi_tgt_v(s)); }
        else { p.psi_src = psi_src(s); p.psi_tgt = psi_tgt(s); }
    }
    p.vel_den = s->vel_den.as<float4>();
    p.force_temp = s->force_temp.as<float4>();
    p.bnd_tex = nullptr;  // the boundary-id field is written once at initialisation
    p.red_partials = s->partials.as<double>();
    p.err = s->err.as<unsigned int>();

    int mode = s->desc.esoteric ? ((s->ticks % 2 == 1) ? AA_ODD : AA_EVEN) : AA_LOCAL;
    // the fast kernel covers periodic boxes without objects, force fields or a
    // thermal lattice; a constant force and the Shan-Chen force are in it
    const uint32_t heavy = F_BOUNDARIES | F_FORCE_FIELD | F_THERMAL | F_EQ_BOUNDARIES;
    const bool all_periodic = (p.flags & (F_PERIODIC_X | F_PERIODIC_Y | F_PERIODIC_Z)) ==
                              (F_PERIODIC_X | F_PERIODIC_Y | F_PERIODIC_Z);
    // the fast kernel indexes every slot with 32 bits off the first plane
    const bool idx32 = (uint64_t)s->N * (uint64_t)s->Q < (1ull << 32);
    // the FP64 stepper's multiphase flow runs the generic kernel
    const bool generic = mode == AA_LOCAL || (p.flags & heavy) || !all_periodic || !idx32 ||
                         (f64 && (p.flags & F_MULTIPHASE));
    // objects and open faces (thermal flow included) without force-field or
    // multiphase flow: the boundary-aware fast kernel, with its masks
    const uint32_t masked_excl = F_FORCE_FIELD | F_MULTIPHASE;
    // the fast and boundary-aware kernels divide by the launch's divisors in
    // two operations, which the host has checked for every divisor
    // (fill_constants); a divisor that failed the check sends the step to the
    // generic kernel, which divides by it in full
    const bool div_checked = f64 || p.div_ok == 0xFu;
    int path = (generic || !div_checked) ? PATH_GENERIC : PATH_FAST;
    if (generic && div_checked && mode != AA_LOCAL && idx32 && !(p.flags & masked_excl) && s->nmask.p &&
        s->desc.storage != BF_STORE_FP64 && s->masked_step)
        path = PATH_MASKED;
    p.nmask = s->nmask.as<uint32_t>();
    if (s->masked_split && s->n_special > 0 && s->n_sched > 0) {
        p.special = s->special.as<uint32_t>();
        p.special_mask = s->special_mask.as<uint32_t>();
        p.sched = s->sched.as<uint32_t>();
        p.n_special = s->n_special;
        p.n_sched = s->n_sched;
        p.special_chunk = s->special_chunk;
        p.sched_shy = s->sched_shy;
        p.sched_shz = s->sched_shz;
    }
    // the split kernel (masked_mixed_kernel) runs the thermal collision as a
    // push when the masks mark every special thermal source: solid sources
    // are marked under bounce-back, and without boundary ids only open ones exist
    s->pushed_thermal = false;
    if (s->thermal && s->thermal_push && path == PATH_MASKED && mode != AA_LOCAL && p.special && !reduce &&
        !measure && ((p.flags & F_BOUNCE_BACK) || !(p.flags & F_BOUNDARIES))) {
        p.thermal_push = 1u;
        s->pushed_thermal = true;
    }
    // the prefetch rounds each row range out to 16 bytes, which stays inside
    // the plane only when every plane starts and ends on a 16-byte boundary
    const size_t plane_bytes = (size_t)s->N * storage_bytes(s->desc.storage);
    if ((!generic || p.sched) && plane_bytes % 16 == 0 && reinterpret_cast<uintptr_t>(lat_src(s)) % 16 == 0)
        p.pf_blocks = generic ? s->pf_blocks_masked
                              : (s->desc.storage == BF_STORE_FP32 ? s->pf_blocks32 : s->pf_blocks);
    p.tma = s->tma_step ? 1u : 0u;
    p.two_cell = s->two_cell ? 1u : 0u;
    p.psi_tile = s->psi_tile != 0 ? 1u : 0u;
    switch (s->Q) {
    case 9: fill_uoff<9>(p, storage_bytes(s->desc.storage)); break;
    case 15: fill_uoff<15>(p, storage_bytes(s->desc.storage)); break;
    case 19: fill_uoff<19>(p, storage_bytes(s->desc.storage)); break;
    default: fill_uoff<27>(p, storage_bytes(s->desc.storage)); break;
    }
    cudaError_t e = dispatch_step(s, p, mode, path);
    if (e != cudaSuccess) return e;
    if (measure) return cudaSuccess;
    if (!s->desc.esoteric && update && !s->desc.two_buffer_fixed) s->lat0_src = !s->lat0_src;
    if (s->desc.multiphase) s->psi0_src = !s->psi0_src;
    s->th0_src = !s->th0_src;
    return cudaSuccess;
}

// LBM::_stream (LBM.cpp:1495-1555)
cudaError_t stream(bf_solver* s) {
    StreamParams p{};
    p.src = lat_src(s);
    p.dst = lat_tgt(s);
    p.stride = s->N;
    p.nx = s->desc.resolution[0]; p.ny = s->desc.resolution[1]; p.nz = s->desc.resolution[2];
    p.flags = base_flags(s);
    p.bits = s->bits;
    p.bnd = s->bnd.as<uint32_t>();
    p.objects = s->objs.as<float4>();
    p.obj_kind = s->kinds.as<uint8_t>();
    cudaError_t e;
    switch (s->Q) {
    case 9: e = launch_stream<9>(p, s->desc.storage, s->stream); break;
    case 15: e = launch_stream<15>(p, s->desc.storage, s->stream); break;
    case 19: e = launch_stream<19>(p, s->desc.storage, s->stream); break;
    default: e = launch_stream<27>(p, s->desc.storage, s->stream); break;
    }
    s->lat0_src = !s->lat0_src;
    return e;
}

// LBM::_stream_thermal (LBM.cpp:1728-1773)
cudaError_t stream_thermal(bf_solver* s) {
    ThermalStreamParams p{};
    if (s->desc.storage == BF_STORE_FP64) {
        p.src64 = static_cast<const double*>(th_src_v(s));
        p.dst64 = static_cast<double*>(th_tgt_v(s));
    } else {
        p.src = th_src(s);
        p.dst = th_tgt(s);
    }
    p.stride = s->N;
    p.nx = s->desc.resolution[0]; p.ny = s->desc.resolution[1]; p.nz = s->desc.resolution[2];
    p.flags = base_flags(s);
    p.bits = s->bits;
    p.bnd = s->bnd.as<uint32_t>();
    p.objects = s->objs.as<float4>();
    p.obj_kind = s->kinds.as<uint8_t>();
    // the flow masks mark solid sources under bounce-back only; the thermal
    // stream treats every solid source (anti-bounce-back)
    if (s->nmask.p && ((p.flags & F_BOUNCE_BACK) || !(p.flags & F_BOUNDARIES))) p.nmask = s->nmask.as<uint32_t>();
    cudaError_t e = s->QT == 5 ? launch_stream_thermal<5>(p, s->stream) : launch_stream_thermal<7>(p, s->stream);
    s->th0_src = !s->th0_src;
    return e;
}

// LBM::_iterate_time (LBM.cpp:1484-1493)
cudaError_t iterate_once(bf_solver* s, bool save, bool update, bool reduce) {
    cudaError_t e = collide(s, save, update, reduce, false);
    if (e != cudaSuccess) return e;
    if (!s->desc.esoteric) { e = stream(s); if (e != cudaSuccess) return e; }
    if (s->thermal && !s->pushed_thermal) { e = stream_thermal(s); if (e != cudaSuccess) return e; }
    return cudaSuccess;
}

int state_key(bf_solver* s) {
    return (int)(s->ticks & 1) | (s->lat0_src << 1) | (s->th0_src << 2) | (s->psi0_src << 3);
}

int run_steps(bf_solver* s, int n, bool save_last) {
    int remaining = n;
    while (remaining > 0) {
        const bool need_save_here = save_last && remaining == 1;
        if (s->graphs_enabled && remaining - (save_last ? 1 : 0) >= kGraphSteps) {
            const int key = state_key(s);
            auto it = s->graphs.find(key);
            if (it == s->graphs.end()) {
                const int saved_key = key;
                const int64_t t0 = s->ticks;
                const int l0 = s->lat0_src, h0 = s->th0_src, p0 = s->psi0_src;
                BF_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = cudaSuccess;
                for (int k = 0; k < kGraphSteps && e == cudaSuccess; k++) {
                    e = iterate_once(s, false, true, false);
                    s->ticks++;
                }
                cudaGraph_t g = nullptr;
                cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
                // restore the state: the captured work has not run yet
                s->ticks = t0; s->lat0_src = l0; s->th0_src = h0; s->psi0_src = p0;
                if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return fail(BF_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(e)); }
                if (e2 != cudaSuccess) return fail(BF_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e2));
                cudaGraphExec_t ex = nullptr;
                cudaError_t e3 = cudaGraphInstantiate(&ex, g, 0);
                cudaGraphDestroy(g);
                if (e3 != cudaSuccess) return fail(BF_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e3));
                it = s->graphs.emplace(saved_key, ex).first;
            }
            BF_CUDA(cudaGraphLaunch(it->second, s->stream));
            // every buffer role has period two in steps and kGraphSteps is
            // even, so only the tick counter moves
            s->ticks += kGraphSteps;
            remaining -= kGraphSteps;
            s->last_saved = false;
            continue;
        }
        cudaError_t e = iterate_once(s, need_save_here, true, false);
        if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
        s->ticks++;
        s->last_saved = need_save_here;
        if (need_save_here) s->fields_tick = s->ticks;
        remaining--;
    }
    return BF_OK;
}

}  // namespace

template <int Q>
static void table_of(float* out) {
    for (int i = 0; i < Q; i++) {
        const Dir c = Lattice<Q>::c(i);
        out[4 * i + 0] = (float)c.x; out[4 * i + 1] = (float)c.y; out[4 * i + 2] = (float)c.z;
        out[4 * i + 3] = Lattice<Q>::w(i);
    }
}
template <int QT>
static void thermal_table_of(float* out) {
    for (int i = 0; i < QT; i++) {
        const Dir c = ThermalLattice<QT>::c(i);
        out[4 * i + 0] = (float)c.x; out[4 * i + 1] = (float)c.y; out[4 * i + 2] = (float)c.z;
        out[4 * i + 3] = ThermalLattice<QT>::w(i);
    }
}

// ===========================================================================
extern "C" {

void bf_init_desc_default(bf_init_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->resolution[0] = d->resolution[1] = d->resolution[2] = 1;
    d->relaxation_time = 0.53f;
    d->periodic[0] = d->periodic[1] = d->periodic[2] = 1;
    d->velocity_set = BF_D2Q9;
    d->storage = BF_STORE_FP32;
    d->multiphase = 0;
    d->esoteric = 0;
    d->boundary_mode = BF_BOUNDARY_SKIP;
    d->collision = BF_COLLISION_BGK;
    d->trt_magic = 0.25f;
    d->velocity_limit = 0.25f;
    d->velocity_limit_extreme = 0.30f;
    d->intermolecular_interaction_strength = -6.0f;
    d->thermal_relaxation_time = 2.0f;
    d->thermal_expansion_coefficient = 0.5f;
    d->thermal_init_equilibrium = 0;
    d->two_buffer_fixed = 0;
}

const char* bf_last_error(void) { return g_last_error.c_str(); }

int bf_get_velosity_vectors(int32_t vs, int32_t thermal, float* out, int32_t* count) {
    const int Q = q_of(vs);
    if (!Q || !count) return fail(BF_ERR_INVALID_ARGUMENT, "get_velosity_vectors(): velocity_set is not supported");
    const int n = thermal ? (vs == BF_D2Q9 ? 5 : 7) : Q;
    *count = n;
    if (!out) return BF_OK;
    if (thermal) { if (n == 5) thermal_table_of<5>(out); else thermal_table_of<7>(out); return BF_OK; }
    switch (Q) {
    case 9: table_of<9>(out); break;
    case 15: table_of<15>(out); break;
    case 19: table_of<19>(out); break;
    default: table_of<27>(out); break;
    }
    return BF_OK;
}

int bf_bits_per_boundry(int32_t object_count, int32_t* bits) {
    if (!bits || object_count < 0) return fail(BF_ERR_INVALID_ARGUMENT, "bits_per_boundry(): bad argument");
    *bits = bits_per_boundry(object_count);
    return BF_OK;
}

int bf_pack_boundries(const uint32_t* ids, size_t cells, int32_t bits, uint32_t* out, size_t cap, size_t* words) {
    if (!words || (bits != 1 && bits != 2 && bits != 4 && bits != 8))
        return fail(BF_ERR_INVALID_ARGUMENT, "pack_boundries(): bits must be 1, 2, 4 or 8");
    *words = (cells * (size_t)bits + 31) / 32;
    if (!out) return BF_OK;
    if (!ids || cap < *words) return fail(BF_ERR_INVALID_ARGUMENT, "pack_boundries(): destination too small");
    std::memset(out, 0, *words * 4);
    for (size_t c = 0; c < cells; c++) {
        const uint64_t b = (uint64_t)c * (uint64_t)bits;
        out[b / 32] |= (ids[c] << (b % 32));
    }
    return BF_OK;
}
int bf_abi_version(void) { return BF_ABI_VERSION; }

int bf_debug_fail_allocation_after(int32_t n) {
    g_alloc_failure_countdown = n < 0 ? -1 : n;
    return BF_OK;
}

int bf_create(bf_solver** out) {
    if (!out) return fail(BF_ERR_INVALID_ARGUMENT, "bf_create: out is NULL");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(BF_ERR_NO_DEVICE, "bf_create: no CUDA device visible");
    }
    bf_solver* s = new bf_solver();
    cudaGetDevice(&s->device);
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete s; return fail(BF_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)); }
    bf_object fluid{};
    fluid.temperature = 1.0f;
    fluid.effective_density = 1.0f;
    s->objects.push_back(fluid);
    bf_init_desc_default(&s->desc);
    // fast-kernel L2 prefetch distance, in blocks: 4 per SM for the 16-bit
    // two-cell step (half a wave of its 128-thread blocks), 2 per SM for FP32
    // (half a wave of 256-thread blocks; 512^3 D3Q19 TRT with the prefetch
    // issued after the warp's own loads: 1/2 / 1 / 1.5 / 2 waves 46.0k / 45.7k
    // / 44.6k / 42.8k MLUPs; fp16s 83.1k / 86.5k / 84.1k / 80.3k at 1/4 / 1/2 /
    // 3/4 / 1 wave); BF_PREFETCH_BLOCKS overrides (0 = off)
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    s->pf_blocks = (uint32_t)std::max(sms, 1) * 4u;
    s->pf_blocks32 = (uint32_t)std::max(sms, 1) * 2u;
    // the boundary-aware step: one wave of schedule entries, issued once the
    // first warp's own loads are in flight (flow past a sphere 256x128x128:
    // 0.5 / 0.75 / 1 / 1.5 waves measured 34.9k / 37.9k / 38.7k / 38.3k MLUPs,
    // Rayleigh-Benard 256x256x130 26.3k / 27.2k / 27.3k / 26.9k)
    s->pf_blocks_masked = (uint32_t)std::max(sms, 1) * 4u;
    if (const char* env = std::getenv("BF_PREFETCH_BLOCKS"))
        s->pf_blocks = s->pf_blocks32 = s->pf_blocks_masked = (uint32_t)std::strtoul(env, nullptr, 10);
    // BF_TWO_CELL=0 keeps the 16-bit fast step at one cell per thread (A/B comparisons)
    if (const char* env = std::getenv("BF_TWO_CELL")) s->two_cell = std::strtoul(env, nullptr, 10) != 0;
    // BF_MASKED_STEP=0 sends objects and open faces to the generic kernel (A/B comparisons)
    if (const char* env = std::getenv("BF_MASKED_STEP")) s->masked_step = std::strtoul(env, nullptr, 10) != 0;
    if (const char* env = std::getenv("BF_MASKED_SPLIT")) s->masked_split = std::strtoul(env, nullptr, 10) != 0;
    // BF_ZERO_COPY=0: stage pinned host buffers through cudaMemcpy like any other (A/B comparisons)
    if (const char* env = std::getenv("BF_ZERO_COPY")) s->zero_copy = std::strtoul(env, nullptr, 10) != 0;
    // BF_THERMAL_PUSH=0: a separate thermal stream pass after every collision (A/B comparisons)
    if (const char* env = std::getenv("BF_THERMAL_PUSH")) s->thermal_push = std::strtoul(env, nullptr, 10) != 0;
    // BF_TMA_STEP=1 selects the staged 16-bit fast step, 0 the plain one
    if (const char* env = std::getenv("BF_TMA_STEP")) s->tma_step = std::strtoul(env, nullptr, 10) != 0;
    if (const char* env = std::getenv("BF_PSI_TILE")) s->psi_tile = std::strtoul(env, nullptr, 10) != 0 ? 1 : 0;
    *out = s;
    return BF_OK;
}

int bf_destroy(bf_solver* s) {
    if (!s) return BF_OK;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    release_all(s);
    cudaStreamDestroy(s->stream);
    delete s;
    return BF_OK;
}

int bf_set_boundry_properties(bf_solver* s, uint32_t id, const bf_object* o) {
    if (!s || !o) return fail(BF_ERR_INVALID_ARGUMENT, "bf_set_boundry_properties: NULL argument");
    if (id > 255) return fail(BF_ERR_INVALID_ARGUMENT, "set_boundry_properties: boundry_id(" + std::to_string(id) + ") is greater than maximum(255)");
    if (id == 0) return fail(BF_ERR_INVALID_ARGUMENT, "set_boundry_properties: boundry_id(0) is defined to be fluid, it cannot be treated as an object");
    if (o->kind < BF_OBJECT_SOLID || o->kind > BF_OBJECT_EQ_DENSITY) return fail(BF_ERR_INVALID_ARGUMENT, "set_boundry_properties: unknown object kind");
    if (id >= s->objects.size()) {
        bf_object def{};
        def.temperature = 1.0f; def.effective_density = 1.0f;
        s->objects.resize(id + 1, def);
    }
    s->objects[id] = *o;
    return BF_OK;
}

int bf_clear_boundry_properties(bf_solver* s) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    s->objects.clear();  // LBM.cpp:1067-1070
    return BF_OK;
}

int bf_initialize_fields(bf_solver* s, const bf_init_desc* d, const float* density, const float* velocity,
                         const float* force, const float* temperature, const uint32_t* ids) {
    if (!s || !d) return fail(BF_ERR_INVALID_ARGUMENT, "bf_initialize_fields: NULL argument");
    cudaSetDevice(s->device);
    const int rx = d->resolution[0], ry = d->resolution[1], rz = d->resolution[2];
    if (rx <= 0 || ry <= 0 || rz <= 0)
        return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields() is called but given resolution is not valid, all components must be greater than zero");
    const int Q = q_of(d->velocity_set);
    if (!Q) return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): velocity set is not supported");
    const int dims = d->velocity_set == BF_D2Q9 ? 2 : 3;
    if (dims == 2 && rz != 1)
        return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields() is called but given velocity set dimention doesn't match the resolution dimention");
    const uint64_t N64 = (uint64_t)rx * ry * rz;
    if (N64 >= (1ull << 32) || ry > 65535 || rz > 65535)
        return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): at most 2^32-1 cells and 65535 cells along y and z");
    if (d->storage < BF_STORE_FP32 || d->storage > BF_STORE_FP64) return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): unknown storage");
    if (d->storage == BF_STORE_FP64 && !d->esoteric)
        return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): FP64 storage (the accuracy reference stepper) runs the esoteric-pull step only");
    if (!(d->relaxation_time > 0.5f)) return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): relaxation_time must exceed 0.5");
    if (d->collision == BF_COLLISION_TRT && !(d->trt_magic > 0.f)) return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): TRT magic parameter must be positive");

    cudaStreamSynchronize(s->stream);
    release_all(s);
    s->desc = *d;
    s->Q = Q; s->dims = dims; s->QT = dims == 2 ? 5 : 7;
    s->N = (uint32_t)N64;
    const uint32_t N = s->N;

    // object table: slot 0 reset to fluid (LBM.cpp:439-441)
    bf_object fluid{};
    fluid.temperature = 1.0f; fluid.effective_density = 1.0f;
    if (s->objects.empty()) s->objects.resize(1);
    s->objects[0] = fluid;
    // LBM.cpp:523-556 -- host passes over the given arrays only (an absent
    // array is the reference's default value everywhere)
    uint32_t maxid = 0;
    std::vector<uint8_t> id_present(256, 0);
    if (ids) {
        for (uint32_t c = 0; c < N; c++) {
            const uint32_t v = ids[c];
            maxid = std::max(maxid, v);
            if (v < 256u) id_present[v] = 1;
        }
    }
    if (maxid > 255) return fail(BF_ERR_INVALID_ARGUMENT, "initialize_fields(): boundry ids above 255");
    if (maxid + 1 > s->objects.size()) {
        bf_object def{};
        def.temperature = 1.0f; def.effective_density = 1.0f;
        s->objects.resize(maxid + 1, def);
    }
    const int nobj = (int)s->objects.size();
    s->constant_force = true;
    s->fconst[0] = force ? force[0] : 0.f; s->fconst[1] = force ? force[1] : 0.f; s->fconst[2] = force ? force[2] : 0.f;
    s->thermal = false;
    const float T0 = temperature ? temperature[0] : 1.0f;
    if (force) {
        for (uint32_t c = 0; c < N; c++) {
            if (force[3 * (uint64_t)c] != s->fconst[0] || force[3 * (uint64_t)c + 1] != s->fconst[1] ||
                force[3 * (uint64_t)c + 2] != s->fconst[2]) {
                s->constant_force = false;
                break;
            }
        }
    }
    if (temperature) {
        for (uint32_t c = 0; c < N; c++) {
            if (temperature[c] != T0) { s->thermal = true; break; }
        }
    }
    // a cell whose object's temperature differs from the first cell's
    for (uint32_t id = 1; id < 256u && id < s->objects.size(); id++)
        if (id_present[id] && s->objects[id].temperature != T0) s->thermal = true;
    s->forcing = !(s->constant_force && s->fconst[0] == 0.f && s->fconst[1] == 0.f && s->fconst[2] == 0.f);
    s->boundaries = nobj > 1;
    s->bits = bits_per_boundry(nobj);
    if (s->bits > 8) return fail(BF_ERR_INVALID_ARGUMENT, "too many objects are defined, maximum of 255 bits are possible but number of objets were: " + std::to_string(nobj));
    s->has_eq_objects = false;
    for (int k = 1; k < nobj; k++) if (s->objects[k].kind != BF_OBJECT_SOLID) s->has_eq_objects = true;

    const size_t sb = storage_bytes(d->storage);
    const size_t lat_bytes = (size_t)N * Q * sb;
    BF_CUDA(s->lat[0].alloc(lat_bytes));
    if (!d->esoteric) BF_CUDA(s->lat[1].alloc(lat_bytes));
    s->lat0_src = 1; s->th0_src = 1; s->psi0_src = 1;
    s->ticks = 0;

    // boundary bits (LBM.cpp:634-659) and the object table (LBM.cpp:613-626)
    std::vector<uint8_t> kinds_h(kMaxObjects, 0);
    std::vector<float4> objs_h((size_t)kMaxObjects * 3, make_float4(0, 0, 0, 0));
    for (int k = 0; k < nobj; k++) {
        const bf_object& o = s->objects[k];
        objs_h[3 * k + 0] = make_float4(o.velocity_translational[0], o.velocity_translational[1], o.velocity_translational[2], o.temperature);
        objs_h[3 * k + 1] = make_float4(o.velocity_angular[0], o.velocity_angular[1], o.velocity_angular[2], 0.f);
        objs_h[3 * k + 2] = make_float4(o.center_of_mass[0], o.center_of_mass[1], o.center_of_mass[2], o.effective_density);
        kinds_h[k] = (uint8_t)(k == 0 ? 0 : o.kind);
    }
    BF_CUDA(s->objs.alloc(objs_h.size() * sizeof(float4)));
    BF_CUDA(s->kinds.alloc(kinds_h.size()));
    BF_CUDA(cudaMemcpy(s->objs.p, objs_h.data(), objs_h.size() * sizeof(float4), cudaMemcpyHostToDevice));
    BF_CUDA(cudaMemcpy(s->kinds.p, kinds_h.data(), kinds_h.size(), cudaMemcpyHostToDevice));
    if (s->boundaries) {
        s->bnd_words = ((uint64_t)N * s->bits + 31) / 32;
        std::vector<uint32_t> words(s->bnd_words + 1, 0u);
        if (ids) {
            size_t nw = 0;
            bf_pack_boundries(ids, N, s->bits, words.data(), words.size(), &nw);
        }
        BF_CUDA(s->bnd.alloc(words.size() * 4));
        BF_CUDA(cudaMemcpy(s->bnd.p, words.data(), words.size() * 4, cudaMemcpyHostToDevice));
    } else {
        s->bnd_words = 0;
    }

    // the given arrays on the device; an absent density or velocity is the
    // init kernel's default (1, 0), so nothing is staged for it
    DeviceBuf d_rho, d_u, d_ids;
    // a pinned density / velocity array is read by the init kernel in place
    const float* rho_in = nullptr;
    const float* u_in = nullptr;
    if (density) {
        rho_in = s->zero_copy ? static_cast<const float*>(mapped_host_ptr(density)) : nullptr;
        if (!rho_in) {
            BF_CUDA(d_rho.alloc((size_t)N * 4));
            BF_CUDA(cudaMemcpy(d_rho.p, density, (size_t)N * 4, cudaMemcpyHostToDevice));
            rho_in = d_rho.as<float>();
        }
    }
    if (velocity) {
        u_in = s->zero_copy ? static_cast<const float*>(mapped_host_ptr(velocity)) : nullptr;
        if (!u_in) {
            BF_CUDA(d_u.alloc((size_t)N * 12));
            BF_CUDA(cudaMemcpy(d_u.p, velocity, (size_t)N * 12, cudaMemcpyHostToDevice));
            u_in = d_u.as<float>();
        }
    }
    // the boundary-id field (LBM.cpp:957-1003): the ids as bytes
    BF_CUDA(s->bnd_tex.alloc(N));
    if (ids) {
        BF_CUDA(d_ids.alloc((size_t)N * 4));
        BF_CUDA(cudaMemcpy(d_ids.p, ids, (size_t)N * 4, cudaMemcpyHostToDevice));
        ids_to_bytes_kernel<<<(unsigned)((N + 255u) / 256u), 256, 0, s->stream>>>(d_ids.as<uint32_t>(), N,
                                                                                 s->bnd_tex.as<uint8_t>());
        BF_CUDA(cudaGetLastError());
    } else {
        BF_CUDA(cudaMemsetAsync(s->bnd_tex.p, 0, N, s->stream));
    }
    // force field (LBM.cpp:693-717), vec4 per cell
    if (s->forcing && !s->constant_force) {
        std::vector<float4> fh(N);
        for (uint64_t c = 0; c < N; c++) fh[c] = make_float4(force[3 * c], force[3 * c + 1], force[3 * c + 2], 0.f);
        BF_CUDA(s->force.alloc((size_t)N * 16));
        BF_CUDA(cudaMemcpy(s->force.p, fh.data(), (size_t)N * 16, cudaMemcpyHostToDevice));
    }
    // equilibrium-boundary values (extension): initial (rho, u) of each cell
    if (s->has_eq_objects) {
        std::vector<float4> bh(N);
        for (uint64_t c = 0; c < N; c++)
            bh[c] = make_float4(density ? density[c] : 1.0f, velocity ? velocity[3 * c] : 0.f,
                                velocity ? velocity[3 * c + 1] : 0.f, velocity ? velocity[3 * c + 2] : 0.f);
        BF_CUDA(s->bvals.alloc((size_t)N * 16));
        BF_CUDA(cudaMemcpy(s->bvals.p, bh.data(), (size_t)N * 16, cudaMemcpyHostToDevice));
    }
    // Shan-Chen pseudopotential textures (LBM.cpp:848-866), zero initial contents
    if (d->multiphase) {
        const size_t pb = (size_t)N * aux_bytes(d->storage);
        BF_CUDA(s->psi[0].alloc(pb));
        BF_CUDA(s->psi[1].alloc(pb));
        BF_CUDA(cudaMemset(s->psi[0].p, 0, pb));
        BF_CUDA(cudaMemset(s->psi[1].p, 0, pb));
    }
    BF_CUDA(s->vel_den.alloc((size_t)N * 16));
    BF_CUDA(s->force_temp.alloc((size_t)N * 16));
    BF_CUDA(cudaMemset(s->vel_den.p, 0, (size_t)N * 16));
    BF_CUDA(cudaMemset(s->force_temp.p, 0, (size_t)N * 16));
    {
        // same block shape as cell_grid() in lbm_kernels.cuh
        const int block = rx >= kStepBlock ? kStepBlock : ((rx + 31) / 32) * 32;
        s->n_blocks = (uint32_t)((rx + block - 1) / block) * (uint32_t)ry * (uint32_t)rz;
    }
    BF_CUDA(s->partials.alloc((size_t)s->n_blocks * 5 * sizeof(double)));
    BF_CUDA(s->red_out.alloc(5 * sizeof(double)));
    BF_CUDA(s->err.alloc(sizeof(unsigned int)));
    BF_CUDA(cudaMemset(s->err.p, 0, sizeof(unsigned int)));

    // set_equilibrium_populations (LBM.cpp:1702-1726)
    InitParams ip{};
    ip.f = s->lat[0].p;
    ip.stride = N;
    ip.n_cells = N;
    ip.rho = rho_in;
    ip.u = u_in;
    ip.ids = d_ids.as<uint32_t>();
    ip.obj_kind = s->kinds.as<uint8_t>();
    cudaError_t e;
    switch (Q) {
    case 9: e = launch_init<9>(ip, d->storage, s->stream); break;
    case 15: e = launch_init<15>(ip, d->storage, s->stream); break;
    case 19: e = launch_init<19>(ip, d->storage, s->stream); break;
    default: e = launch_init<27>(ip, d->storage, s->stream); break;
    }
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA, std::string("init kernel: ") + cudaGetErrorString(e));
    if (s->thermal) {
        const size_t tb = (size_t)N * s->QT * aux_bytes(d->storage);
        BF_CUDA(s->th[0].alloc(tb));
        BF_CUDA(s->th[1].alloc(tb));
        BF_CUDA(cudaMemsetAsync(s->th[0].p, 0, tb, s->stream));
        BF_CUDA(cudaMemsetAsync(s->th[1].p, 0, tb, s->stream));
        if (d->thermal_init_equilibrium) {
            DeviceBuf d_Tb;
            BF_CUDA(d_Tb.alloc((size_t)N * 4));
            if (temperature) {
                BF_CUDA(cudaMemcpy(d_Tb.p, temperature, (size_t)N * 4, cudaMemcpyHostToDevice));
            } else {
                fill_f32_kernel<<<(unsigned)((N + 255u) / 256u), 256, 0, s->stream>>>(d_Tb.as<float>(), N, 1.0f);
                BF_CUDA(cudaGetLastError());
            }
            InitParams tp = ip;
            if (d->storage == BF_STORE_FP64) tp.th64 = s->th[s->th0_src ? 0 : 1].as<double>();
            else tp.th = th_src(s);
            tp.T = d_Tb.as<float>();
            tp.stride = N;
            e = s->QT == 5 ? launch_init_thermal<5>(tp, s->stream) : launch_init_thermal<7>(tp, s->stream);
            if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA, std::string("thermal init kernel: ") + cudaGetErrorString(e));
            // both buffers start alike: slots nothing writes (solid cells) then
            // read the same whichever buffer holds the current state
            BF_CUDA(cudaMemcpyAsync(th_tgt(s), th_src(s), tb, cudaMemcpyDeviceToDevice, s->stream));
            BF_CUDA(cudaStreamSynchronize(s->stream));
        }
        // As the reference reads it, set_equilibrium_populations_thermal.comp:101-107
        // writes past the end of the thermal buffer, which keeps its zero contents.
    }
    // masks of the boundary-aware fast step: built once, the geometry is fixed
    if (d->esoteric && (s->boundaries || !(d->periodic[0] && d->periodic[1] && d->periodic[2])) &&
        d->storage != BF_STORE_FP64) {
        BF_CUDA(s->nmask.alloc((size_t)N * sizeof(uint32_t)));
        StepParams mp{};
        mp.nx = rx; mp.ny = ry; mp.nz = rz;
        mp.flags = base_flags(s);
        mp.bnd = s->bnd.as<uint32_t>();
        mp.bits = s->bits;
        mp.obj_kind = s->kinds.as<uint8_t>();
        mp.objects = s->objs.as<float4>();
        switch (Q) {
        case 9: e = launch_build_mask<9>(mp, s->nmask.as<uint32_t>(), s->stream); break;
        case 15: e = launch_build_mask<15>(mp, s->nmask.as<uint32_t>(), s->stream); break;
        case 19: e = launch_build_mask<19>(mp, s->nmask.as<uint32_t>(), s->stream); break;
        default: e = launch_build_mask<27>(mp, s->nmask.as<uint32_t>(), s->stream); break;
        }
        if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA, std::string("mask kernel: ") + cudaGetErrorString(e));
        e = build_special_list(s, (uint64_t)N);
        if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA,
                                          std::string("special-cell list: ") + cudaGetErrorString(e));
    }
    // LBM.cpp:502: _iterate_time(true, false)
    e = iterate_once(s, true, false, false);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA, std::string("first pass: ") + cudaGetErrorString(e));
    BF_CUDA(cudaStreamSynchronize(s->stream));
    s->last_saved = true;
    s->fields_tick = 0;
    s->initialized = true;
    return BF_OK;
}

int bf_iterate_time(bf_solver* s, int32_t n_steps, int32_t save_fields) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "iterate_time(): initialize_fields has not run");
    if (n_steps < 0) return fail(BF_ERR_INVALID_ARGUMENT, "iterate_time(): negative step count");
    cudaSetDevice(s->device);
    return run_steps(s, n_steps, save_fields != 0);
}

int bf_get_stream(bf_solver* s, void** stream) {
    if (!s || !stream) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *stream = s->stream;
    return BF_OK;
}

int bf_synchronize(bf_solver* s, int32_t timeout_ms) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    cudaSetDevice(s->device);
    if (timeout_ms > 0) {
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            cudaError_t q = cudaStreamQuery(s->stream);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return fail(BF_ERR_CUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(q));
            if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
                return fail(BF_ERR_TIMEOUT, "bf_synchronize: stream still busy after the time limit");
            std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
    } else {
        BF_CUDA(cudaStreamSynchronize(s->stream));
    }
    if (s->initialized) {
        unsigned int h = 0;
        BF_CUDA(cudaMemcpy(&h, s->err.p, sizeof(h), cudaMemcpyDeviceToHost));
        if (h & 1u) return fail(BF_ERR_UNSTABLE, "a step computed a NaN density (simulation unstable)");
        if (h & 2u) return fail(BF_ERR_TIMEOUT, "a step's copy pipeline gave up waiting for its loads");
    }
    return BF_OK;
}

int bf_get_total_ticks_elapsed(bf_solver* s, int64_t* t) {
    if (!s || !t) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *t = s->ticks;
    return BF_OK;
}
int bf_get_resolution(bf_solver* s, int32_t r[3]) {
    if (!s || !r) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    r[0] = s->desc.resolution[0]; r[1] = s->desc.resolution[1]; r[2] = s->desc.resolution[2];
    return BF_OK;
}
int bf_get_velocity_set_vector_count(bf_solver* s, int32_t* q) {
    if (!s || !q) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *q = q_of(s->desc.velocity_set);
    return BF_OK;
}
int bf_get_relaxation_time(bf_solver* s, float* tau) {
    if (!s || !tau) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *tau = s->desc.relaxation_time;
    return BF_OK;
}
int bf_set_relaxation_time(bf_solver* s, float tau) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    if (!(tau > 0.5f)) return fail(BF_ERR_INVALID_ARGUMENT, "set_relaxation_time(): tau must exceed 0.5");
    s->desc.relaxation_time = tau;
    clear_graphs(s);
    return BF_OK;
}
int bf_get_constant_force(bf_solver* s, float f[3]) {
    if (!s || !f) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    f[0] = s->fconst[0]; f[1] = s->fconst[1]; f[2] = s->fconst[2];
    return BF_OK;
}
int bf_set_constant_force(bf_solver* s, const float f[3]) {
    if (!s || !f) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    // LBM::set_constant_force (LBM.cpp:366-369) only changes the uniform; the
    // forcing switches were fixed by initialize_fields
    s->fconst[0] = f[0]; s->fconst[1] = f[1]; s->fconst[2] = f[2];
    clear_graphs(s);
    return BF_OK;
}
int bf_get_intermolecular_interaction_strength(bf_solver* s, float* g) {
    if (!s || !g) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *g = s->desc.intermolecular_interaction_strength;
    return BF_OK;
}
int bf_set_intermolecular_interaction_strength(bf_solver* s, float g) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    s->desc.intermolecular_interaction_strength = g;
    clear_graphs(s);
    return BF_OK;
}
int bf_set_velocity_limits(bf_solver* s, float limit, float limit_extreme) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    s->desc.velocity_limit = limit;
    s->desc.velocity_limit_extreme = limit_extreme;
    clear_graphs(s);
    return BF_OK;
}
int bf_set_thermal_parameters(bf_solver* s, float tau_t, float beta) {
    if (!s) return fail(BF_ERR_INVALID_ARGUMENT, "NULL solver");
    if (!(tau_t > 0.5f)) return fail(BF_ERR_INVALID_ARGUMENT, "thermal relaxation time must exceed 0.5");
    s->desc.thermal_relaxation_time = tau_t;
    s->desc.thermal_expansion_coefficient = beta;
    clear_graphs(s);
    return BF_OK;
}
int bf_get_scheme_flags(bf_solver* s, int32_t* flags, int32_t* bits) {
    if (!s || !flags) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *flags = (s->forcing ? 1 : 0) | (s->constant_force ? 2 : 0) | (s->thermal ? 4 : 0) |
             (s->desc.multiphase ? 8 : 0) | (s->boundaries ? 16 : 0);
    if (bits) *bits = s->bits;
    return BF_OK;
}

int bf_get_field(bf_solver* s, int32_t kind, bf_field* out) {
    if (!s || !out) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "get_field(): initialize_fields has not run");
    std::memset(out, 0, sizeof(*out));
    out->kind = kind;
    out->resolution[0] = s->desc.resolution[0]; out->resolution[1] = s->desc.resolution[1]; out->resolution[2] = s->desc.resolution[2];
    switch (kind) {
    case BF_FIELD_VELOCITY_DENSITY:
        out->device_ptr = s->vel_den.p; out->components = 4; out->bytes_per_component = 4; out->bytes = (size_t)s->N * 16; break;
    case BF_FIELD_BOUNDARY:
        out->device_ptr = s->bnd_tex.p; out->components = 1; out->bytes_per_component = 1; out->bytes = s->N; break;
    case BF_FIELD_FORCE_TEMPERATURE:
        out->device_ptr = s->force_temp.p; out->components = 4; out->bytes_per_component = 4; out->bytes = (size_t)s->N * 16; break;
    case BF_FIELD_POPULATIONS: {
        const size_t bytes = (size_t)s->N * s->Q * 4;
        if (s->decode_tmp.bytes < bytes) BF_CUDA(s->decode_tmp.alloc(bytes));
        cudaError_t e;
        switch (s->Q) {
        case 9: e = launch_decode<9>(lat_src(s), s->N, s->N, s->desc.storage, s->decode_tmp.as<float>(), s->stream); break;
        case 15: e = launch_decode<15>(lat_src(s), s->N, s->N, s->desc.storage, s->decode_tmp.as<float>(), s->stream); break;
        case 19: e = launch_decode<19>(lat_src(s), s->N, s->N, s->desc.storage, s->decode_tmp.as<float>(), s->stream); break;
        default: e = launch_decode<27>(lat_src(s), s->N, s->N, s->desc.storage, s->decode_tmp.as<float>(), s->stream); break;
        }
        if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("decode: ") + cudaGetErrorString(e));
        out->device_ptr = s->decode_tmp.p; out->components = s->Q; out->bytes_per_component = 4; out->bytes = bytes;
        break;
    }
    case BF_FIELD_THERMAL_POPULATIONS:
    case BF_FIELD_PSEUDOPOTENTIAL: {
        const bool th = kind == BF_FIELD_THERMAL_POPULATIONS;
        if (th && !s->thermal) return fail(BF_ERR_INVALID_ARGUMENT, "get_field(): the flow is not thermal");
        if (!th && !s->desc.multiphase) return fail(BF_ERR_INVALID_ARGUMENT, "get_field(): the flow is not multiphase");
        const int comps = th ? s->QT : 1;
        const size_t count = (size_t)s->N * comps;
        out->components = comps; out->bytes_per_component = 4; out->bytes = count * 4;
        void* src = th ? th_src_v(s) : psi_src_v(s);
        if (s->desc.storage != BF_STORE_FP64) { out->device_ptr = src; break; }
        // the FP64 stepper's double values, rounded to float
        if (s->decode_tmp.bytes < count * 4) BF_CUDA(s->decode_tmp.alloc(count * 4));
        d2f_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s->stream>>>(static_cast<const double*>(src), count,
                                                                          s->decode_tmp.as<float>());
        BF_CUDA(cudaGetLastError());
        out->device_ptr = s->decode_tmp.p;
        break;
    }
    default:
        return fail(BF_ERR_INVALID_ARGUMENT, "get_field(): unknown field kind");
    }
    return BF_OK;
}

int bf_copy_field_to_host(bf_solver* s, int32_t kind, void* dst, size_t bytes) {
    if (!dst) return fail(BF_ERR_INVALID_ARGUMENT, "copy_field_to_host(): NULL destination");
    bf_field f;
    int r = bf_get_field(s, kind, &f);
    if (r != BF_OK) return r;
    if (bytes < f.bytes) return fail(BF_ERR_INVALID_ARGUMENT, "copy_field_to_host(): destination too small");
    // a pinned destination is written by a copy kernel (several times the
    // copy engine's rate over the CPU-GPU link); any other by cudaMemcpy
    void* mapped = s->zero_copy ? const_cast<void*>(mapped_host_ptr(dst)) : nullptr;
    const size_t n16 = f.bytes / 16;
    if (mapped && reinterpret_cast<uintptr_t>(mapped) % 16 == 0 && reinterpret_cast<uintptr_t>(f.device_ptr) % 16 == 0 &&
        n16 > 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
        const uint64_t blocks = std::min<uint64_t>((n16 + 255) / 256, (uint64_t)std::max(sms, 1) * 8);
        copy16_kernel<<<(unsigned)blocks, 256, 0, s->stream>>>(static_cast<const uint4*>(f.device_ptr),
                                                              static_cast<uint4*>(mapped), n16);
        BF_CUDA(cudaGetLastError());
        if (f.bytes % 16)
            BF_CUDA(cudaMemcpyAsync(static_cast<char*>(dst) + n16 * 16, static_cast<const char*>(f.device_ptr) + n16 * 16,
                                    f.bytes % 16, cudaMemcpyDeviceToHost, s->stream));
    } else {
        BF_CUDA(cudaMemcpyAsync(dst, f.device_ptr, f.bytes, cudaMemcpyDeviceToHost, s->stream));
    }
    BF_CUDA(cudaStreamSynchronize(s->stream));
    return BF_OK;
}

int bf_copy_boundry_bits_to_host(bf_solver* s, uint32_t* dst, size_t cap, size_t* words) {
    if (!s || !words) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *words = s->bnd_words;
    if (s->bnd_words == 0) return BF_OK;
    if (!dst || cap < s->bnd_words) return fail(BF_ERR_INVALID_ARGUMENT, "copy_boundry_bits_to_host(): destination too small");
    BF_CUDA(cudaStreamSynchronize(s->stream));
    BF_CUDA(cudaMemcpy(dst, s->bnd.p, s->bnd_words * 4, cudaMemcpyDeviceToHost));
    return BF_OK;
}

int bf_reduce(bf_solver* s, double out[5]) {
    if (!s || !out) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "reduce(): initialize_fields has not run");
    cudaSetDevice(s->device);
    // moments of the current state, as the next step would read them
    cudaError_t e = collide(s, true, false, true, true);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("reduce pass: ") + cudaGetErrorString(e));
    s->fields_tick = s->ticks;  // the pass saves the current state's fields
    e = launch_reduce_finish(s->partials.as<double>(), s->n_blocks, s->red_out.as<double>(), s->stream);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("reduce finish: ") + cudaGetErrorString(e));
    BF_CUDA(cudaMemcpyAsync(out, s->red_out.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    BF_CUDA(cudaStreamSynchronize(s->stream));
    return BF_OK;
}

int bf_benchmark_steps(bf_solver* s, int32_t n_steps, float* ms) {
    if (!s || !ms) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "benchmark_steps(): initialize_fields has not run");
    if (n_steps <= 0) return fail(BF_ERR_INVALID_ARGUMENT, "benchmark_steps(): n_steps must be positive");
    cudaSetDevice(s->device);
    cudaEvent_t a, b;
    BF_CUDA(cudaEventCreate(&a));
    BF_CUDA(cudaEventCreate(&b));
    cudaError_t e = cudaEventRecord(a, s->stream);
    int r = e == cudaSuccess ? run_steps(s, n_steps, false) : BF_ERR_CUDA;
    if (r == BF_OK) e = cudaEventRecord(b, s->stream);
    if (r == BF_OK && e == cudaSuccess) e = cudaEventSynchronize(b);
    if (r == BF_OK && e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (r != BF_OK) return r;
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("benchmark_steps: ") + cudaGetErrorString(e));
    return BF_OK;
}

// ---- snapshots ------------------------------------------------------------
static const char kMagic[8] = {'B', 'F', 'G', 'B', '3', 'S', 'N', '1'};

int bf_save_snapshot(bf_solver* s, const char* path) {
    if (!s || !path) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "save_snapshot(): initialize_fields has not run");
    BF_CUDA(cudaStreamSynchronize(s->stream));
    // written to a temporary file beside the target and renamed over it only
    // once complete: an interrupted or failed save leaves no partial snapshot
    const std::string tmp = std::string(path) + ".partial";
    FILE* fp = std::fopen(tmp.c_str(), "wb");
    if (!fp) return fail(BF_ERR_IO, std::string("save_snapshot(): cannot open ") + tmp);
    bool ok = true;
    auto put = [&](const void* p, size_t n) { if (ok && std::fwrite(p, 1, n, fp) != n) ok = false; };
    put(kMagic, 8);
    put(&s->desc, sizeof(s->desc));
    put(&s->ticks, sizeof(s->ticks));
    int32_t st[3] = {s->lat0_src, s->th0_src, s->psi0_src};
    put(st, sizeof(st));
    std::vector<char> h;
    auto dump = [&](const DeviceBuf& b) {
        uint64_t n = b.bytes;
        put(&n, 8);
        if (!n) return;
        h.resize(n);
        if (cudaMemcpy(h.data(), b.p, n, cudaMemcpyDeviceToHost) != cudaSuccess) { ok = false; return; }
        put(h.data(), n);
    };
    dump(s->lat[0]); dump(s->lat[1]); dump(s->th[0]); dump(s->th[1]); dump(s->psi[0]); dump(s->psi[1]);
    dump(s->vel_den); dump(s->force_temp);
    if (std::fclose(fp) != 0) ok = false;
    if (ok && std::rename(tmp.c_str(), path) != 0) ok = false;
    if (!ok) {
        std::remove(tmp.c_str());
        return fail(BF_ERR_IO, std::string("save_snapshot(): write failed for ") + path);
    }
    return BF_OK;
}

int bf_load_snapshot(bf_solver* s, const char* path) {
    if (!s || !path) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "load_snapshot(): initialize_fields with the same configuration must run first");
    BF_CUDA(cudaStreamSynchronize(s->stream));
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(BF_ERR_IO, std::string("load_snapshot(): cannot open ") + path);
    bool ok = true;
    auto get = [&](void* p, size_t n) { if (ok && std::fread(p, 1, n, fp) != n) ok = false; };
    char magic[8];
    get(magic, 8);
    bf_init_desc d;
    get(&d, sizeof(d));
    int64_t ticks = 0;
    get(&ticks, sizeof(ticks));
    int32_t st[3];
    get(st, sizeof(st));
    if (!ok || std::memcmp(magic, kMagic, 8) != 0) { std::fclose(fp); return fail(BF_ERR_IO, "load_snapshot(): not a snapshot file"); }
    if (std::memcmp(d.resolution, s->desc.resolution, sizeof(d.resolution)) != 0 || d.velocity_set != s->desc.velocity_set ||
        d.storage != s->desc.storage || d.esoteric != s->desc.esoteric || d.multiphase != s->desc.multiphase) {
        std::fclose(fp);
        return fail(BF_ERR_INVALID_ARGUMENT, "load_snapshot(): snapshot configuration differs from the solver's");
    }
    std::vector<char> h;
    DeviceBuf* bufs[] = {&s->lat[0], &s->lat[1], &s->th[0], &s->th[1], &s->psi[0], &s->psi[1], &s->vel_den, &s->force_temp};
    // the file must be exactly this solver's snapshot size before any device
    // buffer is touched: a truncated or foreign file leaves the state as it was
    {
        uint64_t expect = 8 + sizeof(d) + sizeof(ticks) + sizeof(st);
        for (DeviceBuf* b : bufs) expect += 8 + b->bytes;
        const long here = std::ftell(fp);
        const bool sized = here >= 0 && std::fseek(fp, 0, SEEK_END) == 0;
        const long end = sized ? std::ftell(fp) : -1;
        if (!sized || end < 0 || (uint64_t)end != expect || std::fseek(fp, here, SEEK_SET) != 0) {
            std::fclose(fp);
            return fail(BF_ERR_IO, "load_snapshot(): truncated or mismatched snapshot");
        }
    }
    for (DeviceBuf* b : bufs) {
        uint64_t n = 0;
        get(&n, 8);
        if (!ok) break;
        if (n != b->bytes) { ok = false; break; }
        if (!n) continue;
        h.resize(n);
        get(h.data(), n);
        if (!ok) break;
        if (cudaMemcpy(b->p, h.data(), n, cudaMemcpyHostToDevice) != cudaSuccess) ok = false;
    }
    std::fclose(fp);
    if (!ok) return fail(BF_ERR_IO, "load_snapshot(): truncated or mismatched snapshot");
    s->ticks = ticks;
    s->fields_tick = ticks;
    s->lat0_src = st[0]; s->th0_src = st[1]; s->psi0_src = st[2];
    s->desc.relaxation_time = d.relaxation_time;
    clear_graphs(s);
    return BF_OK;
}

// ---- macroscopic fields ---------------------------------------------------
static const char kMacroMagic[8] = {'B', 'F', 'G', 'B', '3', 'M', 'C', '1'};
struct MacroHeader {
    char magic[8];
    int32_t resolution[3];
    int32_t thermal;
    int64_t tick;
};

__global__ void bytes_to_ids_kernel(const uint8_t* __restrict__ b, uint32_t n, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ids[i] = b[i];
}

int bf_save_macroscopic(bf_solver* s, const char* path) {
    if (!s || !path) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "save_current_tick_macroscopic(): initialize_fields has not run");
    BF_CUDA(cudaStreamSynchronize(s->stream));
    MacroHeader h{};
    std::memcpy(h.magic, kMacroMagic, 8);
    std::memcpy(h.resolution, s->desc.resolution, sizeof(h.resolution));
    h.thermal = s->thermal ? 1 : 0;
    h.tick = s->fields_tick;
    const std::string tmp = std::string(path) + ".partial";
    FILE* fp = std::fopen(tmp.c_str(), "wb");
    if (!fp) return fail(BF_ERR_IO, std::string("save_current_tick_macroscopic(): cannot open ") + tmp);
    bool ok = std::fwrite(&h, sizeof(h), 1, fp) == 1;
    std::vector<char> buf;
    for (const DeviceBuf* b : {&s->vel_den, &s->force_temp, &s->bnd_tex}) {
        if (!ok) break;
        buf.resize(b->bytes);
        ok = cudaMemcpy(buf.data(), b->p, b->bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
             std::fwrite(buf.data(), 1, b->bytes, fp) == b->bytes;
    }
    if (std::fclose(fp) != 0) ok = false;
    if (ok && std::rename(tmp.c_str(), path) != 0) ok = false;
    if (!ok) {
        std::remove(tmp.c_str());
        return fail(BF_ERR_IO, std::string("save_current_tick_macroscopic(): write failed for ") + path);
    }
    return BF_OK;
}

int bf_load_macroscopic(bf_solver* s, const char* path, int32_t target_tick) {
    if (!s || !path) return fail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->initialized) return fail(BF_ERR_NOT_INITIALIZED, "load_tick_macroscopic(): initialize_fields must run first");
    cudaSetDevice(s->device);
    BF_CUDA(cudaStreamSynchronize(s->stream));
    const uint32_t N = s->N;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(BF_ERR_IO, std::string("load_tick_macroscopic(): cannot open ") + path);
    MacroHeader h{};
    const uint64_t expect = sizeof(h) + (uint64_t)N * (16 + 16 + 1);
    bool ok = std::fread(&h, sizeof(h), 1, fp) == 1 && std::memcmp(h.magic, kMacroMagic, 8) == 0;
    if (ok) {
        const bool sized = std::fseek(fp, 0, SEEK_END) == 0;
        const long end = sized ? std::ftell(fp) : -1;
        ok = sized && end >= 0 && (uint64_t)end == expect && std::fseek(fp, (long)sizeof(h), SEEK_SET) == 0;
    }
    if (!ok || std::memcmp(h.resolution, s->desc.resolution, sizeof(h.resolution)) != 0) {
        std::fclose(fp);
        return fail(BF_ERR_IO, "load_tick_macroscopic(): not a macroscopic file of this solver's resolution");
    }
    if (target_tick >= 0 && (int64_t)target_tick != h.tick) {
        std::fclose(fp);
        return fail(BF_ERR_INVALID_ARGUMENT, "load_tick_macroscopic(): the file holds tick " + std::to_string(h.tick) +
                                                 ", not " + std::to_string(target_tick));
    }
    std::vector<float4> vd(N), ft(N);
    ok = std::fread(vd.data(), 16, N, fp) == N && std::fread(ft.data(), 16, N, fp) == N;
    std::fclose(fp);
    if (!ok) return fail(BF_ERR_IO, "load_tick_macroscopic(): read failed");
    std::vector<float> rho(N), u(3 * (size_t)N), T(N);
    for (uint32_t c = 0; c < N; c++) {
        rho[c] = vd[c].w;
        u[3 * (size_t)c] = vd[c].x; u[3 * (size_t)c + 1] = vd[c].y; u[3 * (size_t)c + 2] = vd[c].z;
        T[c] = ft[c].w;
    }
    DeviceBuf d_rho, d_u, d_ids, d_T;
    BF_CUDA(d_rho.alloc((size_t)N * 4));
    BF_CUDA(d_u.alloc((size_t)N * 12));
    BF_CUDA(d_ids.alloc((size_t)N * 4));
    BF_CUDA(cudaMemcpy(d_rho.p, rho.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
    BF_CUDA(cudaMemcpy(d_u.p, u.data(), (size_t)N * 12, cudaMemcpyHostToDevice));
    // the solver's own boundary ids (its geometry is kept)
    bytes_to_ids_kernel<<<(unsigned)((N + 255u) / 256u), 256, 0, s->stream>>>(s->bnd_tex.as<uint8_t>(), N,
                                                                             d_ids.as<uint32_t>());
    BF_CUDA(cudaGetLastError());
    clear_graphs(s);
    s->ticks = h.tick;
    InitParams ip{};
    ip.f = lat_src(s);
    ip.stride = N;
    ip.n_cells = N;
    ip.rho = d_rho.as<float>();
    ip.u = d_u.as<float>();
    ip.ids = d_ids.as<uint32_t>();
    ip.obj_kind = s->kinds.as<uint8_t>();
    // an odd tick of the esoteric-pull step: the equilibrium goes where the odd step reads it
    ip.odd = (s->desc.esoteric && (s->ticks & 1)) ? 1 : 0;
    ip.nx = s->desc.resolution[0]; ip.ny = s->desc.resolution[1]; ip.nz = s->desc.resolution[2];
    ip.flags = base_flags(s);
    cudaError_t e;
    switch (s->Q) {
    case 9: e = launch_init<9>(ip, s->desc.storage, s->stream); break;
    case 15: e = launch_init<15>(ip, s->desc.storage, s->stream); break;
    case 19: e = launch_init<19>(ip, s->desc.storage, s->stream); break;
    default: e = launch_init<27>(ip, s->desc.storage, s->stream); break;
    }
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("load_tick_macroscopic(): init kernel: ") + cudaGetErrorString(e));
    if (s->thermal) {
        BF_CUDA(d_T.alloc((size_t)N * 4));
        BF_CUDA(cudaMemcpy(d_T.p, T.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
        InitParams tp = ip;
        const size_t tb = (size_t)N * s->QT * aux_bytes(s->desc.storage);
        if (s->desc.storage == BF_STORE_FP64) tp.th64 = static_cast<double*>(th_src_v(s));
        else tp.th = th_src(s);
        tp.T = d_T.as<float>();
        BF_CUDA(cudaMemsetAsync(th_src_v(s), 0, tb, s->stream));
        e = s->QT == 5 ? launch_init_thermal<5>(tp, s->stream) : launch_init_thermal<7>(tp, s->stream);
        if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("load_tick_macroscopic(): thermal init: ") + cudaGetErrorString(e));
        BF_CUDA(cudaMemcpyAsync(th_tgt_v(s), th_src_v(s), tb, cudaMemcpyDeviceToDevice, s->stream));
    }
    // the fields of the loaded state, as initialize_fields saves them (LBM.cpp:502)
    e = iterate_once(s, true, false, false);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("load_tick_macroscopic(): first pass: ") + cudaGetErrorString(e));
    BF_CUDA(cudaStreamSynchronize(s->stream));
    s->last_saved = true;
    s->fields_tick = s->ticks;
    return BF_OK;
}

}  // extern "C"
