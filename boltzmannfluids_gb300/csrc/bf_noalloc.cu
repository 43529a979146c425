// bf_noalloc.cu -- FP64 conservation sums of a velocity/density field with
// no device allocation: a variant of the two-pass block reduction used by
// bf_reduce, whose scratch (per-block partials and the 5-double result)
// lives in a fixed file-scope device array instead of solver-owned buffers.
//
// Who needs it: code that reads the solver's fields from places where it
// may not allocate device memory -- a renderer or UI frame callback working
// under a fixed device-memory budget, or a caller that must not stall other
// streams (cudaFree synchronizes the whole device).  It receives the field
// pointer (BF_FIELD_VELOCITY_DENSITY layout) and a host array for the sums.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/bf_lbm.h"
#include "lbm_common.cuh"

namespace {

constexpr unsigned kThreads = 256;
constexpr unsigned kCellsPerThread = 64;
constexpr unsigned kCellsPerBlock = kThreads * kCellsPerThread;  // 16,384
constexpr unsigned kMaxBlocks = 8192;
constexpr size_t kMaxCells = (size_t)kCellsPerBlock * kMaxBlocks;  // 134,217,728 = 512^3

// kMaxBlocks x 5 partial sums + 5 result sums + padding: 327,744 bytes.
// Every GPU that loads the library holds this array until the process exits.
__device__ __align__(256) double g_noalloc_scratch[kMaxBlocks * 5 + 8];

// One block per 16,384-cell chunk; each thread accumulates its cells in a
// fixed order in FP64, then a fixed shared-memory tree.  Writes partials[b*5+k].
// A cell contributes exactly what the step kernels' fused reduction adds for
// it: rho, rho*u and 0.5*rho*|u|^2 formed in FP32 (|u|^2 as
// fma(uz, uz, fma(uy, uy, ux*ux))), then widened to FP64.
__global__ void __launch_bounds__(kThreads) noalloc_partials_kernel(const float4* __restrict__ field, uint64_t n,
                                                                    double* __restrict__ partials) {
    __shared__ double sm[kThreads][5];
    const uint64_t begin = (uint64_t)blockIdx.x * kCellsPerBlock;
    uint64_t end = begin + kCellsPerBlock;
    if (end > n) end = n;
    double acc[5] = {0, 0, 0, 0, 0};
    for (uint64_t c = begin + threadIdx.x; c < end; c += kThreads) {
        const float4 v = __ldg(field + c);  // (u.x, u.y, u.z, rho)
        const float uu = __fmaf_rn(v.z, v.z, __fmaf_rn(v.y, v.y, __fmul_rn(v.x, v.x)));
        acc[0] += (double)v.w;
        acc[1] += (double)__fmul_rn(v.w, v.x);
        acc[2] += (double)__fmul_rn(v.w, v.y);
        acc[3] += (double)__fmul_rn(v.w, v.z);
        acc[4] += (double)__fmul_rn(__fmul_rn(0.5f, v.w), uu);
    }
#pragma unroll
    for (int k = 0; k < 5; k++) sm[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (unsigned s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
#pragma unroll
            for (int k = 0; k < 5; k++) sm[threadIdx.x][k] += sm[threadIdx.x + s][k];
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 5; k++) partials[(uint64_t)blockIdx.x * 5 + k] = sm[0][k];
}

// The host-side name g_noalloc_scratch is only a stand-in for the symbol;
// the device address comes from cudaGetSymbolAddress, once per device.
std::mutex g_mutex;
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};

int fail(int code, const std::string& msg) {
    bf::record_error(msg);  // readable through bf_last_error()
    return code;
}

}  // namespace

extern "C" int bf_reduce_field_noalloc(const void* vel_den_device, size_t n_cells, void* stream, double out[5]) {
    if (!out) return fail(BF_ERR_INVALID_ARGUMENT, "bf_reduce_field_noalloc: out is NULL");
    if (n_cells == 0) {
        for (int k = 0; k < 5; k++) out[k] = 0.0;
        return BF_OK;
    }
    if (!vel_den_device) return fail(BF_ERR_INVALID_ARGUMENT, "bf_reduce_field_noalloc: field pointer is NULL");
    if (n_cells > kMaxCells)
        return fail(BF_ERR_INVALID_ARGUMENT, "bf_reduce_field_noalloc: " + std::to_string(n_cells) +
                                                 " cells exceed the fixed scratch capacity of " +
                                                 std::to_string(kMaxCells) + " cells");
    // the kernel reads whole float4 cells: a pointer off a 16-byte boundary
    // (an offset into some other buffer) would fault the context
    if (reinterpret_cast<uintptr_t>(vel_den_device) % 16u != 0u)
        return fail(BF_ERR_INVALID_ARGUMENT, "bf_reduce_field_noalloc: field pointer is not 16-byte aligned");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(BF_ERR_INVALID_ARGUMENT, "bf_reduce_field_noalloc: device index out of range");
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return fail(BF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((n_cells + kCellsPerBlock - 1) / kCellsPerBlock);
    double* partials = scratch;
    double* result = scratch + (size_t)kMaxBlocks * 5;
    noalloc_partials_kernel<<<blocks, kThreads, 0, st>>>(static_cast<const float4*>(vel_den_device), n_cells, partials);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("partials kernel: ") + cudaGetErrorString(e));
    e = bf::launch_reduce_finish(partials, blocks, result, st);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("finish kernel: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(out, result, 5 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    return BF_OK;
}
