// marching_cubes.cu -- iso-surface extraction from a device scalar field
// (the mesh BoltzmannFluids' MarchingCubes sets out to build from the density
// texture, MarchingCubes.cpp:3-64 and GLSL/MarchingCubes/marching_cubes.comp).
//
// Three passes over the voxels between lattice nodes (x fastest):
//   1. classify + block scan: each thread classifies 4 voxels (which of the 8
//      corner values are >= threshold -> case -> triangle count) and the
//      block writes exclusive offsets of its 1024 voxels plus its total;
//   2. the block totals are scanned (recursively) and added back, giving
//      every voxel the index of its first triangle;
//   3. generate: voxels with triangles recompute their case and write
//      3 vertices per triangle, interpolated on the cut edges, at their offset.
// The output is a triangle list in voxel order, deterministic.
//
// The case table is derived at first use (host code below), not transcribed:
// corners k = (k&1, k>>1&1, k>>2&1); edge 4d+j joins the j-th corner with bit
// d clear to its neighbour along d; on each face the cut edges pair into
// segments (a face with two diagonal inside corners cuts each inside corner
// off, a rule of the face alone, so neighbouring voxels agree and the surface
// is closed); segments chain into loops, each loop is oriented so that its
// normal points from the inside corners to the outside ones and is fanned
// into triangles from its first edge.  At most 5 triangles per voxel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bf_lbm.h"
#include "lbm_common.cuh"
#include "scan.cuh"

namespace {

constexpr int kMaxTri = 5;

struct McTable {
    int8_t tri[256][kMaxTri * 3];
    uint8_t count[256];
};

__constant__ McTable c_table;
__constant__ int8_t c_edge_a[12];
__constant__ int8_t c_edge_axis[12];

// ---- host derivation of the case table ----
struct Geometry {
    int corner[8][3];
    int edge[12][2];
    int face[6][4];
};

Geometry geometry() {
    Geometry g{};
    for (int k = 0; k < 8; k++) { g.corner[k][0] = k & 1; g.corner[k][1] = (k >> 1) & 1; g.corner[k][2] = (k >> 2) & 1; }
    int e = 0;
    for (int d = 0; d < 3; d++)
        for (int c = 0; c < 8; c++)
            if (!((c >> d) & 1)) { g.edge[e][0] = c; g.edge[e][1] = c | (1 << d); e++; }
    int f = 0;
    for (int d = 0; d < 3; d++) {
        int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
        for (int side = 0; side < 2; side++) {
            const int base = side << d;
            g.face[f][0] = base;
            g.face[f][1] = base | (1 << a);
            g.face[f][2] = base | (1 << a) | (1 << b);
            g.face[f][3] = base | (1 << b);
            f++;
        }
    }
    return g;
}

int edge_of(const Geometry& g, int a, int b) {
    const int lo = std::min(a, b), hi = std::max(a, b);
    for (int e = 0; e < 12; e++) if (g.edge[e][0] == lo && g.edge[e][1] == hi) return e;
    return -1;
}

McTable derive_table() {
    const Geometry g = geometry();
    McTable t{};
    for (int cs = 0; cs < 256; cs++) {
        int inside[8];
        for (int k = 0; k < 8; k++) inside[k] = (cs >> k) & 1;
        std::vector<int> adj[12];
        for (int f = 0; f < 6; f++) {
            const int* cyc = g.face[f];
            int es[4], cut[4], nc = 0;
            for (int i = 0; i < 4; i++) {
                es[i] = edge_of(g, cyc[i], cyc[(i + 1) & 3]);
                if (inside[cyc[i]] != inside[cyc[(i + 1) & 3]]) cut[nc++] = i;
            }
            auto link = [&](int a, int b) { adj[a].push_back(b); adj[b].push_back(a); };
            if (nc == 2) link(es[cut[0]], es[cut[1]]);
            else if (nc == 4)
                for (int i = 0; i < 4; i++)
                    if (inside[cyc[i]]) link(es[(i + 3) & 3], es[i]);
        }
        bool seen[12] = {false};
        int nt = 0;
        for (int start = 0; start < 12; start++) {
            if (adj[start].empty() || seen[start]) continue;
            std::vector<int> loop{start};
            seen[start] = true;
            int prev = -1, cur = start;
            while (true) {
                const int nxt = adj[cur][0] != prev ? adj[cur][0] : adj[cur][1];
                if (nxt == start) break;
                loop.push_back(nxt);
                seen[nxt] = true;
                prev = cur;
                cur = nxt;
            }
            // Newell normal of the edge midpoints against the inside -> outside direction
            double nrm[3] = {0, 0, 0}, out[3] = {0, 0, 0};
            const size_t L = loop.size();
            for (size_t i = 0; i < L; i++) {
                double p[3], q[3];
                for (int d = 0; d < 3; d++) {
                    p[d] = 0.5 * (g.corner[g.edge[loop[i]][0]][d] + g.corner[g.edge[loop[i]][1]][d]);
                    q[d] = 0.5 * (g.corner[g.edge[loop[(i + 1) % L]][0]][d] + g.corner[g.edge[loop[(i + 1) % L]][1]][d]);
                }
                nrm[0] += p[1] * q[2] - p[2] * q[1];
                nrm[1] += p[2] * q[0] - p[0] * q[2];
                nrm[2] += p[0] * q[1] - p[1] * q[0];
                const int a = g.edge[loop[i]][0], b = g.edge[loop[i]][1];
                const int in = inside[a] ? a : b, ou = inside[a] ? b : a;
                for (int d = 0; d < 3; d++) out[d] += g.corner[ou][d] - g.corner[in][d];
            }
            if (nrm[0] * out[0] + nrm[1] * out[1] + nrm[2] * out[2] < 0) std::reverse(loop.begin(), loop.end());
            for (size_t i = 1; i + 1 < L; i++) {
                if (nt >= kMaxTri) break;  // never reached: the derivation yields at most 5
                t.tri[cs][3 * nt + 0] = (int8_t)loop[0];
                t.tri[cs][3 * nt + 1] = (int8_t)loop[i];
                t.tri[cs][3 * nt + 2] = (int8_t)loop[i + 1];
                nt++;
            }
        }
        for (int k = 3 * nt; k < kMaxTri * 3; k++) t.tri[cs][k] = -1;
        t.count[cs] = (uint8_t)nt;
    }
    return t;
}

const McTable& host_table() {
    static McTable t = derive_table();
    return t;
}

// ---- device ----
struct McParams {
    const float* field;
    int components, component;
    int nx, ny, nz;
    uint32_t vx, vy, vz;  // voxels per axis (nodes - 1)
    uint64_t voxels;
    float threshold;
    float scale[3];
};

__device__ __forceinline__ float node_value(const McParams& p, int x, int y, int z) {
    const size_t node = (size_t)x + (size_t)p.nx * ((size_t)y + (size_t)p.ny * (size_t)z);
    return __ldg(p.field + node * (size_t)p.components + p.component);
}

__device__ __forceinline__ void voxel_xyz(const McParams& p, uint64_t v, int& x, int& y, int& z) {
    x = (int)(v % p.vx);
    const uint64_t r = v / p.vx;
    y = (int)(r % p.vy);
    z = (int)(r / p.vy);
}

__device__ __forceinline__ int voxel_case(const McParams& p, int x, int y, int z, float (&val)[8]) {
    int cs = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        val[k] = node_value(p, x + (k & 1), y + ((k >> 1) & 1), z + ((k >> 2) & 1));
        cs |= (val[k] >= p.threshold ? 1 : 0) << k;
    }
    return cs;
}

__global__ void __launch_bounds__(kScanThreads) mc_classify_scan_kernel(const McParams p, uint32_t* __restrict__ offsets,
                                                                        uint32_t* __restrict__ block_sums) {
    uint32_t c[kScanItems];
    const uint64_t first = (uint64_t)blockIdx.x * kScanBlock + (uint64_t)threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const uint64_t v = first + k;
        c[k] = 0u;
        if (v < p.voxels) {
            int x, y, z;
            voxel_xyz(p, v, x, y, z);
            float val[8];
            c[k] = c_table.count[voxel_case(p, x, y, z, val)];
        }
    }
    const uint32_t tot = block_exclusive_scan(c);
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (first + k < p.voxels) offsets[first + k] = c[k];
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void mc_total_kernel(const McParams p, const uint32_t* __restrict__ offsets, uint64_t* __restrict__ total) {
    int x, y, z;
    voxel_xyz(p, p.voxels - 1, x, y, z);
    float val[8];
    *total = (uint64_t)offsets[p.voxels - 1] + c_table.count[voxel_case(p, x, y, z, val)];
}

__global__ void __launch_bounds__(256) mc_generate_kernel(const McParams p, const uint32_t* __restrict__ offsets,
                                                          const uint64_t* __restrict__ total, float* __restrict__ out) {
    const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= p.voxels) return;
    // empty voxels (equal consecutive offsets) leave before reading their corners
    const uint64_t next = v + 1 < p.voxels ? (uint64_t)offsets[v + 1] : *total;
    if (next == (uint64_t)offsets[v]) return;
    int x, y, z;
    voxel_xyz(p, v, x, y, z);
    float val[8];
    const int cs = voxel_case(p, x, y, z, val);
    const int nt = c_table.count[cs];
    if (nt == 0) return;
    const float res[3] = {(float)p.nx, (float)p.ny, (float)p.nz};
    float* o = out + (size_t)offsets[v] * 9;
    for (int t = 0; t < nt; t++) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const int e = c_table.tri[cs][3 * t + j];
            const int a = c_edge_a[e], d = c_edge_axis[e], b = a | (1 << d);
            // t = (threshold - v_a) / (v_b - v_a), one IEEE division
            const float s = __fdiv_rn(__fsub_rn(p.threshold, val[a]), __fsub_rn(val[b], val[a]));
            float q[3] = {(float)(x + (a & 1)), (float)(y + ((a >> 1) & 1)), (float)(z + ((a >> 2) & 1))};
            q[d] = __fadd_rn(q[d], s);
#pragma unroll
            for (int k = 0; k < 3; k++)
                o[(size_t)(3 * t + j) * 3 + k] = __fmul_rn(__fadd_rn(-0.5f, __fdiv_rn(q[k], res[k])), p.scale[k]);
        }
    }
}

std::map<int, bool> g_table_uploaded;  // per device
std::mutex g_table_mutex;

cudaError_t upload_table() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_table_mutex);
    if (g_table_uploaded[dev]) return cudaSuccess;
    const Geometry g = geometry();
    int8_t ea[12], ed[12];
    for (int k = 0; k < 12; k++) {
        ea[k] = (int8_t)g.edge[k][0];
        ed[k] = (int8_t)(31 - __builtin_clz((unsigned)(g.edge[k][0] ^ g.edge[k][1])));
    }
    e = cudaMemcpyToSymbol(c_table, &host_table(), sizeof(McTable));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_edge_a, ea, sizeof(ea));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_edge_axis, ed, sizeof(ed));
    if (e == cudaSuccess) g_table_uploaded[dev] = true;
    return e;
}

}  // namespace

struct bf_marching_cubes {
    int device = 0;
    ScanLevels scan;  // level 0: per-voxel triangle offsets
    float* vertices = nullptr;
    uint64_t vertex_capacity = 0;  // triangles
    uint64_t* total = nullptr;
    uint64_t triangles = 0;
};

namespace {

int mc_fail(int code, const std::string& msg) {
    bf::record_error(msg);
    return code;
}
#define MCUDA(call)                                                                                      \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return mc_fail(e_ == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA,         \
                           std::string(#call " failed: ") + cudaGetErrorString(e_));                     \
    } while (0)

}  // namespace

extern "C" {

int bf_mc_case_table(int8_t* triangles, uint8_t* counts) {
    if (!triangles || !counts) return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_case_table: NULL argument");
    const McTable& t = host_table();
    std::memcpy(triangles, t.tri, sizeof(t.tri));
    std::memcpy(counts, t.count, sizeof(t.count));
    return BF_OK;
}

int bf_mc_create(bf_marching_cubes** out) {
    if (!out) return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_create: NULL argument");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return mc_fail(BF_ERR_NO_DEVICE, "bf_mc_create: no CUDA device visible");
    }
    bf_marching_cubes* m = new bf_marching_cubes();
    cudaGetDevice(&m->device);
    cudaError_t e = cudaMalloc(&m->total, sizeof(uint64_t));
    if (e != cudaSuccess) {
        delete m;
        return mc_fail(BF_ERR_OUT_OF_MEMORY, std::string("bf_mc_create: ") + cudaGetErrorString(e));
    }
    *out = m;
    return BF_OK;
}

int bf_mc_destroy(bf_marching_cubes* m) {
    if (!m) return BF_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    m->scan.release();
    if (m->vertices) cudaFree(m->vertices);
    if (m->total) cudaFree(m->total);
    delete m;
    return BF_OK;
}

int bf_mc_compute(bf_marching_cubes* m, const float* field, int32_t components, int32_t component,
                  const int32_t resolution[3], float threshold, const float mesh_scale[3], void* stream,
                  uint64_t* triangle_count) {
    if (!m || !field || !resolution) return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_compute: NULL argument");
    if (components < 1 || component < 0 || component >= components)
        return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_compute: component out of range");
    const int nx = resolution[0], ny = resolution[1], nz = resolution[2];
    if (nx < 2 || ny < 2 || nz < 2) return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_compute: at least 2 nodes per axis");
    const uint64_t voxels = (uint64_t)(nx - 1) * (ny - 1) * (nz - 1);
    if (voxels * kMaxTri >= (1ull << 32))
        return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_compute: at most 2^32/5 voxels");
    cudaSetDevice(m->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MCUDA(upload_table());
    MCUDA(m->scan.reserve(voxels));
    McParams p{};
    p.field = field;
    p.components = components;
    p.component = component;
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.vx = (uint32_t)(nx - 1); p.vy = (uint32_t)(ny - 1); p.vz = (uint32_t)(nz - 1);
    p.voxels = voxels;
    p.threshold = threshold;
    for (int k = 0; k < 3; k++) p.scale[k] = mesh_scale ? mesh_scale[k] : 1.0f;
    const uint64_t blocks = (voxels + kScanBlock - 1) / kScanBlock;
    mc_classify_scan_kernel<<<(unsigned)blocks, kScanThreads, 0, st>>>(p, m->scan.levels[0], m->scan.levels[1]);
    MCUDA(m->scan.finish_level0(voxels, st));
    mc_total_kernel<<<1, 1, 0, st>>>(p, m->scan.levels[0], m->total);
    MCUDA(cudaGetLastError());
    uint64_t tris = 0;
    MCUDA(cudaMemcpyAsync(&tris, m->total, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MCUDA(cudaStreamSynchronize(st));
    if (tris > m->vertex_capacity) {
        if (m->vertices) cudaFree(m->vertices);
        m->vertices = nullptr;
        m->vertex_capacity = 0;
        MCUDA(cudaMalloc(&m->vertices, tris * 9 * sizeof(float)));
        m->vertex_capacity = tris;
    }
    if (tris > 0)
        mc_generate_kernel<<<(unsigned)((voxels + 255) / 256), 256, 0, st>>>(p, m->scan.levels[0], m->total, m->vertices);
    MCUDA(cudaGetLastError());
    MCUDA(cudaStreamSynchronize(st));
    m->triangles = tris;
    if (triangle_count) *triangle_count = tris;
    return BF_OK;
}

int bf_mc_get_vertices(bf_marching_cubes* m, const float** vertices_device, uint64_t* triangle_count) {
    if (!m || !vertices_device || !triangle_count) return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_get_vertices: NULL argument");
    *vertices_device = m->vertices;
    *triangle_count = m->triangles;
    return BF_OK;
}

int bf_mc_copy_vertices_to_host(bf_marching_cubes* m, float* out, uint64_t max_triangles, uint64_t* written) {
    if (!m || (!out && max_triangles)) return mc_fail(BF_ERR_INVALID_ARGUMENT, "bf_mc_copy_vertices_to_host: NULL argument");
    const uint64_t n = std::min(max_triangles, m->triangles);
    cudaSetDevice(m->device);
    if (n) MCUDA(cudaMemcpy(out, m->vertices, n * 9 * sizeof(float), cudaMemcpyDeviceToHost));
    if (written) *written = n;
    return BF_OK;
}

}  // extern "C"
