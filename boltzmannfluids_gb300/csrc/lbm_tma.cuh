// lbm_tma.cuh -- the fast AA step with its population loads staged through
// shared memory by the bulk-copy (TMA) engine, for fp16s storage.
//
// The 16-bit steps are issue-bound: half of a plain step's instructions are
// load/store addressing and memory operations.  Here a persistent block walks
// over row tiles of 256 cells (x0 .. x0+255 of one (y, z) row); for each tile
// one warp issues, per direction i, a bulk copy of the row segment the tile
// reads -- on an even step row (y - c_y, z - c_z) of plane i widened by 8
// cells each side (the c_x shift), on an odd step row (y, z) of plane opp(i)
// -- into one of kTmaStages shared-memory stages, completing on the stage's
// mbarrier.  Threads read their 19 populations from the stage with constant
// offsets (no address arithmetic), run the same update as the plain kernel
// (fast_cell) and store to global memory.  The copies of the next tiles are
// in flight while a tile is computed.
//
// Alignment: a bulk copy needs 16-byte aligned addresses and sizes.  Row
// starts are multiples of nx elements with nx % 256 == 0, planes start at
// multiples of N = nx*ny*nz, so every row segment [x0 - 8, x0 + 264) of
// 16-bit data starts on a 16-byte boundary; at the two ends of a row the
// 8-cell halos wrap to the other end of the same row (periodic in x) and are
// copied separately (16 bytes each).  Every wait on an mbarrier is bounded:
// past the limit a warp sets bit 1 of the error word (reported as
// BF_ERR_TIMEOUT), waits, again bounded, on the stages' copies, and returns;
// no block-wide barrier follows the start, so no warp waits on one that left.
#pragma once

namespace bf {

constexpr int kTmaTile = 256;                        // cells per tile = threads per block
constexpr int kTmaHalo = 8;                          // halo cells each side: 16 bytes of 16-bit data
constexpr int kTmaRow = kTmaTile + 2 * kTmaHalo;     // staged elements per row
#ifndef BF_TMA_STAGES
#define BF_TMA_STAGES 3
#endif
constexpr int kTmaStages = BF_TMA_STAGES;
// 16-bit load from a shared-memory address (explicit shared state space: a
// generic pointer into the stage would go through the generic load path)
template <class T>
__device__ __forceinline__ T lds16(uint32_t addr) {
    static_assert(sizeof(T) == 2, "16-bit storage only");
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(addr));
    T out;
    memcpy(&out, &v, 2);
    return out;
}

// direction components packed 2 bits per direction (component + 1), so a
// lane can look up its direction without a table in memory
template <int Q>
struct DirBits {
    static constexpr uint64_t pack(int axis) {
        uint64_t v = 0;
        for (int i = 0; i < Q; i++) {
            const Dir c = Lattice<Q>::c(i);
            const int comp = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
            v |= (uint64_t)(comp + 1) << (2 * i);
        }
        return v;
    }
    static constexpr uint64_t X = pack(0), Y = pack(1), Z = pack(2);
    __device__ __forceinline__ static int cx(int i) { return (int)((X >> (2 * i)) & 3u) - 1; }
    __device__ __forceinline__ static int cy(int i) { return (int)((Y >> (2 * i)) & 3u) - 1; }
    __device__ __forceinline__ static int cz(int i) { return (int)((Z >> (2 * i)) & 3u) - 1; }
};

struct TmaTile {
    int x0, y, z;
};
__device__ __forceinline__ TmaTile tma_tile(const StepParams& p, uint32_t t) {
    const uint32_t tx = (uint32_t)p.nx / kTmaTile;
    TmaTile r;
    r.x0 = (int)(t % tx) * kTmaTile;
    const uint32_t yz = t / tx;
    r.y = (int)(yz % (uint32_t)p.ny);
    r.z = (int)(yz / (uint32_t)p.ny);
    return r;
}

// Warp 0 issues the copies of tile t into the stage at `stage` (shared
// address), completing on `bar`: lane i < Q copies direction i's row.
template <int Q, int ST, int MODE>
__device__ __forceinline__ void tma_issue(const StepParams& p, uint32_t t, uint32_t stage, uint32_t bar, int lane) {
    using T = typename Codec<ST>::T;
    constexpr uint32_t sz = sizeof(T);
    constexpr uint32_t row_bytes = (MODE == AA_EVEN ? kTmaRow : kTmaTile) * sz;
    if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)Q * row_bytes);
    __syncwarp();
    if (lane >= Q) return;
    const TmaTile tl = tma_tile(p, t);
    const int i = lane;
    int ys = tl.y, zs = tl.z, plane = i;
    if (MODE == AA_EVEN) {
        ys -= DirBits<Q>::cy(i);
        zs -= DirBits<Q>::cz(i);
        ys = ys < 0 ? ys + p.ny : (ys >= p.ny ? ys - p.ny : ys);
        zs = zs < 0 ? zs + p.nz : (zs >= p.nz ? zs - p.nz : zs);
    } else {
        plane = opp(i);
    }
    const T* row = static_cast<const T*>(p.plane[0]) + (size_t)plane * p.stride +
                   (size_t)p.nx * ((size_t)ys + (size_t)p.ny * (size_t)zs);
    const uint32_t dst = stage + (uint32_t)i * kTmaRow * sz;
    if (MODE == AA_EVEN) {
        const int x0 = tl.x0;
        if (x0 > 0 && x0 + kTmaTile < p.nx) {
            bulk_g2s(dst, row + (x0 - kTmaHalo), kTmaRow * sz, bar);
        } else {  // the halo of a row end wraps to the other end of the same row
            const int left = x0 == 0 ? p.nx - kTmaHalo : x0 - kTmaHalo;
            const int right = x0 + kTmaTile == p.nx ? 0 : x0 + kTmaTile;
            bulk_g2s(dst, row + left, kTmaHalo * sz, bar);
            bulk_g2s(dst + kTmaHalo * sz, row + x0, kTmaTile * sz, bar);
            bulk_g2s(dst + (kTmaHalo + kTmaTile) * sz, row + right, kTmaHalo * sz, bar);
        }
    } else {
        bulk_g2s(dst + kTmaHalo * sz, row + tl.x0, kTmaTile * sz, bar);
    }
}

#ifndef BF_TMA_MIN_BLOCKS
#define BF_TMA_MIN_BLOCKS 4
#endif
// Pipeline per stage s: full[s] completes when the stage's copies have
// landed (one arrival with the byte count, then the copies' bytes); empty[s]
// completes when all eight warps are done with the tile in it.  Warp 0 also
// produces: after its own part of tile k it waits for empty[s] and issues
// tile k + kTmaStages into stage s, while the other warps go on to the next
// tile without a block-wide barrier.  64 registers (the even step spills at 48).
template <int Q, int ST, int MODE, bool TRT, bool FORCED>
__global__ void __launch_bounds__(kTmaTile, BF_TMA_MIN_BLOCKS) tma_step_kernel(const __grid_constant__ StepParams p) {
    using C = Codec<ST>;
    using T = typename C::T;
    using L = Lattice<Q>;
    constexpr int kWarps = kTmaTile / 32;
    extern __shared__ __align__(128) unsigned char tma_smem[];
    uint64_t* const bars = reinterpret_cast<uint64_t*>(tma_smem + (size_t)kTmaStages * Q * kTmaRow * sizeof(T));
    const uint32_t stage0 = smem_addr(tma_smem), full0 = smem_addr(bars), empty0 = full0 + 8u * kTmaStages;
    constexpr uint32_t stage_bytes = (uint32_t)Q * kTmaRow * sizeof(T);
    const uint32_t tiles_x = (uint32_t)p.nx / kTmaTile;
    const uint32_t n_tiles = tiles_x * (uint32_t)p.ny * (uint32_t)p.nz;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    if (tid == 0) {
        for (int s = 0; s < kTmaStages; s++) {
            mbar_init(full0 + 8u * s, 1);
            mbar_init(empty0 + 8u * s, kWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == 0) {
        for (int s = 0; s < kTmaStages; s++) {
            const uint32_t t = blockIdx.x + (uint32_t)s * gridDim.x;
            if (t < n_tiles) tma_issue<Q, ST, MODE>(p, t, stage0 + s * stage_bytes, full0 + 8u * s, lane);
        }
    }
    // tile coordinates, advanced by the grid stride without divisions
    TmaTile tl = tma_tile(p, blockIdx.x);
    const TmaTile step = tma_tile(p, gridDim.x);
    bool failed = false;
    for (uint32_t k = 0, t = blockIdx.x; t < n_tiles; k++, t += gridDim.x) {
        const int s = (int)(k % kTmaStages);
        const uint32_t parity = (k / kTmaStages) & 1u;
        if (!mbar_wait_bounded(full0 + 8u * s, parity)) { failed = true; break; }
        const uint32_t sbase = stage0 + (uint32_t)s * stage_bytes + (uint32_t)(kTmaHalo + tid) * (uint32_t)sizeof(T);
        auto load = [&](int i, auto&&) -> T {
            const Dir c = L::c(i);
            return lds16<T>(sbase + (uint32_t)((i * kTmaRow - (MODE == AA_EVEN ? c.x : 0)) * (int)sizeof(T)));
        };
        const bool edge = MODE == AA_EVEN && (tl.y == 0 || tl.y == p.ny - 1 || (L::D == 3 && (tl.z == 0 || tl.z == p.nz - 1)));
        if (edge) fast_cell<Q, ST, MODE, TRT, FORCED, false, true>(p, tl.x0 + tid, tl.y, tl.z, load);
        else fast_cell<Q, ST, MODE, TRT, FORCED, false, false>(p, tl.x0 + tid, tl.y, tl.z, load);
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8u * s);  // this warp is done with stage s
        if (warp == 0) {
            const uint32_t tn = t + (uint32_t)kTmaStages * gridDim.x;
            if (tn < n_tiles) {
                if (!mbar_wait_bounded(empty0 + 8u * s, parity)) { failed = true; break; }
                // order the block's reads of the stage before the copy engine overwrites it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                tma_issue<Q, ST, MODE>(p, tn, stage0 + s * stage_bytes, full0 + 8u * s, lane);
            }
        }
        // next tile: x0 += step.x0 (carry into y), y += step.y (carry into z), z += step.z
        tl.x0 += step.x0;
        int cy = 0;
        if (tl.x0 >= p.nx) { tl.x0 -= p.nx; cy = 1; }
        tl.y += step.y + cy;
        if (tl.y >= p.ny) { tl.y -= p.ny; tl.z += 1; }
        tl.z += step.z;
    }
    if (failed) {
        // give up: report, let this warp's view of the copies in flight land, return
        if (lane == 0) atomicOr(p.err, 2u);
        for (int s = 0; s < kTmaStages; s++) mbar_wait_bounded(full0 + 8u * s, 0u), mbar_wait_bounded(full0 + 8u * s, 1u);
    }
}

template <int Q, int ST>
constexpr size_t tma_smem_bytes() {
    return (size_t)kTmaStages * Q * kTmaRow * sizeof(typename Codec<ST>::T) + 2 * kTmaStages * sizeof(uint64_t);
}

}  // namespace bf
