// voxelize.cu -- solid voxels of a closed triangle mesh by ray parity, on
// the GPU: the boundary geometry that BoltzmannFluids' MeshRasterizer3D
// (MeshRasterizer3D.cpp:7-113, GLSL/MeshRasterizer3D/raster_unifier.comp,
// copy_to_3d.comp) rasterises slab by slab through OpenGL.
//
// The reference renders the mesh orthographically in 64 depth slabs per
// voxel layer; every slab whose triangles cover a pixel centre toggles that
// pixel's inside/outside parity, and a voxel is solid when the parity was
// "inside" in any of its 64 slabs.  Restated as rays: every voxel column
// (i, j) casts one ray through its centre along z; the depths where the ray
// crosses the mesh, sorted, bound the inside intervals (odd crossings leave
// the rest of the column inside, as an unmatched toggle does); voxel k is
// solid when one of its `samples` equally spaced depth samples lies inside.
//
// Normalised volume coordinates: the model matrix (column-major, as glm)
// maps mesh vertices into the cube [-1, 1]^3, column i has its centre at
// x = -1 + (2i + 1)/nx (likewise y), sample s of voxel k sits at depth
// z = -1 + 2(k + (s + 1/2)/samples)/nz.  (The reference's camera looks down
// -z from z = +1, so its layer 0 is at the top; here layer k grows with z.)
//
// Passes: transform the triangles; each triangle (one warp) visits the column centres
// inside its projection (edge functions with a top-left rule, so a centre on
// an edge shared by two triangles is counted once and a silhouette edge
// twice or never, which keeps the parity) and counts a crossing per column;
// the counts are prefix-summed; a second visit writes the crossing depths;
// one thread per column sorts its depths and marks the voxels.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/bf_lbm.h"
#include "lbm_common.cuh"
#include "scan.cuh"

namespace {

struct VoxParams {
    const float* tri;   // transformed triangles, 9 floats each
    uint64_t tris;
    int nx, ny, nz, samples;
};

// 2D edge function (b - a) x (p - a), rounded operations, evaluated from the
// lexicographically smaller endpoint so that the two triangles sharing an
// edge get exactly opposite values
__device__ __forceinline__ float edge_raw(float ax, float ay, float bx, float by, float px, float py) {
    return __fsub_rn(__fmul_rn(__fsub_rn(bx, ax), __fsub_rn(py, ay)), __fmul_rn(__fsub_rn(by, ay), __fsub_rn(px, ax)));
}
__device__ __forceinline__ float edge_fn(float ax, float ay, float bx, float by, float px, float py) {
    const bool a_first = ax < bx || (ax == bx && ay < by);
    return a_first ? edge_raw(ax, ay, bx, by, px, py) : -edge_raw(bx, by, ax, ay, px, py);
}

// top-left rule for a counter-clockwise triangle: an edge owns its boundary
// points when it is a left edge (going down, dy < 0) or a top edge (dy == 0,
// going left, dx < 0)
__device__ __forceinline__ bool owns(float ax, float ay, float bx, float by) {
    const float dx = __fsub_rn(bx, ax), dy = __fsub_rn(by, ay);
    return dy < 0.0f || (dy == 0.0f && dx < 0.0f);
}

// Visits the column centres covered by triangle t; f(column, depth).  The
// lanes of a warp share the triangle's bounding box (lane, lane + 32, ...).
template <class F>
__device__ __forceinline__ void visit_triangle(const VoxParams& p, uint64_t t, int lane, F f) {
    const float* v = p.tri + t * 9;
    float ax = v[0], ay = v[1], az = v[2];
    float bx = v[3], by = v[4], bz = v[5];
    float cx = v[6], cy = v[7], cz = v[8];
    float area = edge_fn(ax, ay, bx, by, cx, cy);
    if (!(area > 0.0f || area < 0.0f)) return;  // edge-on (or NaN): no column crosses it
    if (area < 0.0f) {  // make it counter-clockwise
        float tx = bx, ty = by, tz = bz;
        bx = cx; by = cy; bz = cz;
        cx = tx; cy = ty; cz = tz;
        area = -area;
    }
    const float minx = fminf(ax, fminf(bx, cx)), maxx = fmaxf(ax, fmaxf(bx, cx));
    const float miny = fminf(ay, fminf(by, cy)), maxy = fmaxf(ay, fmaxf(by, cy));
    // columns with centre -1 + (2i+1)/nx inside [minx, maxx]
    const float hx = 0.5f * p.nx, hy = 0.5f * p.ny;
    int i0 = (int)ceilf(__fsub_rn(__fmul_rn(__fadd_rn(minx, 1.0f), hx), 0.5f));
    int i1 = (int)floorf(__fsub_rn(__fmul_rn(__fadd_rn(maxx, 1.0f), hx), 0.5f));
    int j0 = (int)ceilf(__fsub_rn(__fmul_rn(__fadd_rn(miny, 1.0f), hy), 0.5f));
    int j1 = (int)floorf(__fsub_rn(__fmul_rn(__fadd_rn(maxy, 1.0f), hy), 0.5f));
    i0 = max(i0, 0); j0 = max(j0, 0);
    i1 = min(i1, p.nx - 1); j1 = min(j1, p.ny - 1);
    const bool oa = owns(bx, by, cx, cy), ob = owns(cx, cy, ax, ay), oc = owns(ax, ay, bx, by);
    if (i1 < i0 || j1 < j0) return;
    const int bw = i1 - i0 + 1;
    const int64_t cells = (int64_t)bw * (int64_t)(j1 - j0 + 1);
    for (int64_t k = lane; k < cells; k += 32) {
        const int i = i0 + (int)(k % bw), j = j0 + (int)(k / bw);
        const float py = __fsub_rn(__fdiv_rn((float)(2 * j + 1), (float)p.ny), 1.0f);
        {
            const float px = __fsub_rn(__fdiv_rn((float)(2 * i + 1), (float)p.nx), 1.0f);
            const float wa = edge_fn(bx, by, cx, cy, px, py);  // weight of a
            const float wb = edge_fn(cx, cy, ax, ay, px, py);
            const float wc = edge_fn(ax, ay, bx, by, px, py);
            const bool in = (wa > 0.0f || (wa == 0.0f && oa)) && (wb > 0.0f || (wb == 0.0f && ob)) &&
                            (wc > 0.0f || (wc == 0.0f && oc));
            if (!in) continue;
            // depth by barycentric weights
            const float z = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(wa, az), __fmul_rn(wb, bz)), __fmul_rn(wc, cz)), area);
            f((uint64_t)i + (uint64_t)p.nx * (uint64_t)j, z);
        }
    }
}

__global__ void vox_transform_kernel(const float* __restrict__ in, uint64_t tris, const float* __restrict__ m16,
                                     float* __restrict__ out) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tris) return;
    for (int k = 0; k < 3; k++) {
        const float x = in[t * 9 + 3 * k], y = in[t * 9 + 3 * k + 1], z = in[t * 9 + 3 * k + 2];
        float r[4];
        for (int row = 0; row < 4; row++)  // column-major: M[col * 4 + row]
            r[row] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m16[row], x), __fmul_rn(m16[4 + row], y)),
                                         __fmul_rn(m16[8 + row], z)), m16[12 + row]);
        const float w = r[3];
        out[t * 9 + 3 * k] = __fdiv_rn(r[0], w);
        out[t * 9 + 3 * k + 1] = __fdiv_rn(r[1], w);
        out[t * 9 + 3 * k + 2] = __fdiv_rn(r[2], w);
    }
}

// one warp per triangle
__global__ void vox_count_kernel(const VoxParams p, uint32_t* __restrict__ counts) {
    const uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (t >= p.tris) return;
    visit_triangle(p, t, threadIdx.x & 31, [&](uint64_t col, float) { atomicAdd(counts + col, 1u); });
}

__global__ void vox_fill_kernel(const VoxParams p, const uint32_t* __restrict__ offsets, uint32_t* __restrict__ cursor,
                                float* __restrict__ depths) {
    const uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (t >= p.tris) return;
    visit_triangle(p, t, threadIdx.x & 31, [&](uint64_t col, float z) {
        const uint32_t slot = offsets[col] + atomicAdd(cursor + col, 1u);
        depths[slot] = z;
    });
}

__global__ void vox_resolve_kernel(const VoxParams p, const uint32_t* __restrict__ offsets,
                                   const uint32_t* __restrict__ counts, float* __restrict__ depths,
                                   uint8_t* __restrict__ mask) {
    const uint64_t col = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t ncol = (uint64_t)p.nx * (uint64_t)p.ny;
    if (col >= ncol) return;
    const uint32_t n = counts[col];
    float* d = depths + offsets[col];
    // insertion sort of the column's crossings (few per column)
    for (uint32_t a = 1; a < n; a++) {
        const float key = d[a];
        uint32_t b = a;
        while (b > 0 && d[b - 1] > key) { d[b] = d[b - 1]; b--; }
        d[b] = key;
    }
    // voxels are cleared by the caller; mark those with a sample inside
    const int S = p.samples;
    const long long total = (long long)p.nz * S;
    const float hz = 0.5f * (float)total;
    for (uint32_t a = 0; a < n; a += 2) {
        const float lo = d[a];
        const float hi = a + 1 < n ? d[a + 1] : 3.0f;  // odd count: inside to the end
        // samples t with -1 + (2t + 1)/total strictly inside (lo, hi)
        long long t0 = (long long)floorf(__fsub_rn(__fmul_rn(__fadd_rn(lo, 1.0f), hz), 0.5f)) + 1;
        long long t1 = (long long)ceilf(__fsub_rn(__fmul_rn(__fadd_rn(hi, 1.0f), hz), 0.5f)) - 1;
        t0 = t0 < 0 ? 0 : t0;
        t1 = t1 >= total ? total - 1 : t1;
        if (t0 > t1) continue;
        for (long long k = t0 / S; k <= t1 / S; k++) mask[col + (uint64_t)k * ncol] = 1;
    }
}

int vox_fail(int code, const std::string& msg) {
    bf::record_error(msg);
    return code;
}

struct DevMem {
    std::vector<void*> ptrs;
    ~DevMem() { for (void* p : ptrs) cudaFree(p); }
    cudaError_t alloc(void** p, size_t bytes) {
        cudaError_t e = cudaMalloc(p, bytes == 0 ? 1 : bytes);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
};

#define VCUDA(call)                                                                                      \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return vox_fail(e_ == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA,        \
                            std::string(#call " failed: ") + cudaGetErrorString(e_));                    \
    } while (0)

}  // namespace

extern "C" int bf_voxelize_mesh(const float* vertices, uint64_t triangle_count, const float model[16],
                                const int32_t resolution[3], int32_t samples_per_voxel, uint8_t* mask) {
    if (!resolution || !mask || (!vertices && triangle_count))
        return vox_fail(BF_ERR_INVALID_ARGUMENT, "bf_voxelize_mesh: NULL argument");
    const int nx = resolution[0], ny = resolution[1], nz = resolution[2];
    if (nx < 1 || ny < 1 || nz < 1 || samples_per_voxel < 1 || samples_per_voxel > 4096)
        return vox_fail(BF_ERR_INVALID_ARGUMENT, "bf_voxelize_mesh: bad resolution or sample count");
    const uint64_t ncol = (uint64_t)nx * ny, nvox = ncol * (uint64_t)nz;
    if (triangle_count >= (1ull << 31)) return vox_fail(BF_ERR_INVALID_ARGUMENT, "bf_voxelize_mesh: too many triangles");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return vox_fail(BF_ERR_NO_DEVICE, "bf_voxelize_mesh: no CUDA device visible");
    }
    float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const float* m = model ? model : ident;
    DevMem mem;
    float *d_in = nullptr, *d_tri = nullptr, *d_m = nullptr, *d_depth = nullptr;
    uint32_t *d_count = nullptr, *d_cursor = nullptr;
    uint8_t* d_mask = nullptr;
    ScanLevels scan;
    struct Release { ScanLevels& s; ~Release() { s.release(); } } release_scan{scan};
    const size_t tri_bytes = (size_t)triangle_count * 9 * sizeof(float);
    VCUDA(mem.alloc((void**)&d_in, tri_bytes));
    VCUDA(mem.alloc((void**)&d_tri, tri_bytes));
    VCUDA(mem.alloc((void**)&d_m, 16 * sizeof(float)));
    VCUDA(mem.alloc((void**)&d_cursor, ncol * sizeof(uint32_t)));
    VCUDA(mem.alloc((void**)&d_mask, nvox));
    VCUDA(scan.reserve(ncol));
    VCUDA(mem.alloc((void**)&d_count, ncol * sizeof(uint32_t)));
    if (tri_bytes) VCUDA(cudaMemcpy(d_in, vertices, tri_bytes, cudaMemcpyHostToDevice));
    VCUDA(cudaMemcpy(d_m, m, 16 * sizeof(float), cudaMemcpyHostToDevice));
    VCUDA(cudaMemset(d_count, 0, ncol * sizeof(uint32_t)));
    VCUDA(cudaMemset(d_cursor, 0, ncol * sizeof(uint32_t)));
    VCUDA(cudaMemset(d_mask, 0, nvox));
    VoxParams p{};
    p.tri = d_tri;
    p.tris = triangle_count;
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.samples = samples_per_voxel;
    const unsigned tb = (unsigned)((triangle_count + 127) / 128);
    const unsigned wb = (unsigned)((triangle_count + 3) / 4);  // 4 warps (triangles) per 128-thread block
    if (triangle_count) {
        vox_transform_kernel<<<tb, 128>>>(d_in, triangle_count, d_m, d_tri);
        vox_count_kernel<<<wb, 128>>>(p, d_count);
    }
    // offsets = exclusive scan of the counts (scan level 0 is the offsets array)
    VCUDA(cudaMemcpy(scan.levels[0], d_count, ncol * sizeof(uint32_t), cudaMemcpyDeviceToDevice));
    VCUDA(scan.scan(0, ncol, 0));
    uint32_t last_off = 0, last_cnt = 0;
    VCUDA(cudaMemcpy(&last_off, scan.levels[0] + (ncol - 1), 4, cudaMemcpyDeviceToHost));
    VCUDA(cudaMemcpy(&last_cnt, d_count + (ncol - 1), 4, cudaMemcpyDeviceToHost));
    const uint64_t crossings = (uint64_t)last_off + last_cnt;
    VCUDA(mem.alloc((void**)&d_depth, crossings * sizeof(float)));
    if (triangle_count) vox_fill_kernel<<<wb, 128>>>(p, scan.levels[0], d_cursor, d_depth);
    vox_resolve_kernel<<<(unsigned)((ncol + 127) / 128), 128>>>(p, scan.levels[0], d_count, d_depth, d_mask);
    VCUDA(cudaGetLastError());
    VCUDA(cudaMemcpy(mask, d_mask, nvox, cudaMemcpyDeviceToHost));
    return BF_OK;
}
