// scan.cuh -- exclusive prefix sums of uint32 counts on the device (block
// scans of 1024 values, block totals scanned recursively and added back),
// shared by the mesh extraction and the voxeliser.  Everything has internal
// linkage so that several translation units can include it.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;  // values per thread in a scan block
constexpr int kScanBlock = kScanThreads * kScanItems;

// exclusive scan of kScanItems values per thread over one block; returns the block total
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t (&v)[kScanItems]) {
    constexpr int NW = kScanThreads / 32;
    __shared__ uint32_t warp_sum[NW];
    __shared__ uint32_t block_total;
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) { const uint32_t c = v[k]; v[k] = run; run += c; }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = run;  // inclusive scan of the thread totals within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < NW ? warp_sum[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < NW) warp_sum[lane] = wi - w;  // exclusive offset of each warp
        if (lane == NW - 1) block_total = wi;
    }
    __syncthreads();
    const uint32_t base = warp_sum[warp] + (inc - run);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) v[k] += base;
    return block_total;
}

__global__ void __launch_bounds__(kScanThreads) scan_values_kernel(uint32_t* __restrict__ data, uint64_t n,
                                                                   uint32_t* __restrict__ block_sums) {
    uint32_t c[kScanItems];
    const uint64_t first = (uint64_t)blockIdx.x * kScanBlock + (uint64_t)threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) c[k] = first + k < n ? data[first + k] : 0u;
    const uint32_t tot = block_exclusive_scan(c);
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (first + k < n) data[first + k] = c[k];
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void add_block_offsets_kernel(uint32_t* __restrict__ data, uint64_t n, const uint32_t* __restrict__ block_offsets) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += block_offsets[i / kScanBlock];
}

// Level 0 holds the values to scan (n of them); level k+1 holds the block
// totals of level k.  Level 1 must already hold the totals of level 0's
// blocks (a fused producer writes them) when finish_level0 runs.
struct ScanLevels {
    std::vector<uint32_t*> levels;
    uint64_t capacity = 0;

    cudaError_t reserve(uint64_t n) {
        if (n <= capacity && !levels.empty()) return cudaSuccess;
        release();
        // at least two levels: a fused producer always writes its block totals to level 1
        uint64_t m = n;
        while (true) {
            uint32_t* p = nullptr;
            cudaError_t e = cudaMalloc(&p, std::max<uint64_t>(m, 1) * sizeof(uint32_t));
            if (e != cudaSuccess) { release(); return e; }
            levels.push_back(p);
            if (m <= 1 && levels.size() >= 2) break;
            m = (m + kScanBlock - 1) / kScanBlock;
        }
        capacity = n;
        return cudaSuccess;
    }
    void release() {
        for (uint32_t* p : levels) cudaFree(p);
        levels.clear();
        capacity = 0;
    }
    // exclusive scan of levels[k][0..n) in place
    cudaError_t scan(size_t k, uint64_t n, cudaStream_t st) {
        const uint64_t blocks = (n + kScanBlock - 1) / kScanBlock;
        scan_values_kernel<<<(unsigned)blocks, kScanThreads, 0, st>>>(levels[k], n, levels[k + 1]);
        if (blocks > 1) {
            cudaError_t e = scan(k + 1, blocks, st);
            if (e != cudaSuccess) return e;
            add_block_offsets_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(levels[k], n, levels[k + 1]);
        }
        return cudaGetLastError();
    }
    // level 0 was block-scanned by its producer (totals in level 1): finish it
    cudaError_t finish_level0(uint64_t n, cudaStream_t st) {
        const uint64_t blocks = (n + kScanBlock - 1) / kScanBlock;
        if (blocks > 1) {
            cudaError_t e = scan(1, blocks, st);
            if (e != cudaSuccess) return e;
            add_block_offsets_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(levels[0], n, levels[1]);
        }
        return cudaGetLastError();
    }
};

}  // namespace
