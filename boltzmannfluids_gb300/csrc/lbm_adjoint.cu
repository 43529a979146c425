// lbm_adjoint.cu -- differentiable channel-flow model and its hand-written
// discrete adjoint (no counterpart in the reference, which has no adjoint).
//
// Model (D2Q9 with nz = 1, or D3Q19; periodic in z).  One step maps the
// post-collision state f^(t-1) to f^t:
//   pull   g_i(x) = f_i(x - c_i)                 source inside the domain
//          g_i(x) = f_opp(i)(x)                  source outside in y: halfway bounce-back wall
//          g_i(x) = feq_i(1, (u_in(y,z),0,0))    source at x < 0 or x >= nx: equilibrium inlet/outlet
//   BGK    g^c_i = g_i + (feq_i(rho,u) - g_i)/tau,  feq = w rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u.u)
//   PSM    f_i = (1 - s) g^c_i + s g_opp(i)      partial bounce-back, solid fraction s in [0,1]
// f^0 = feq(1, (u_in,0,0)).  The objective reads the pulled populations of step T:
//   J = wd sum 2 s j_x + wm sum |u - u*|^2.
//
// The adjoint step is the transposed pull (a push) of the transposed
// per-cell Jacobian.  With the equilibrium inlet/outlet every population of
// f^(t-1) feeds at most one g of step t, so every adjoint slot is written by
// exactly one thread (plain stores; slots that feed nothing get 0).  The
// transposed BGK Jacobian costs O(Q) per cell:
//   mu_i = (1-w)(1-s) L_i + w (A0 + (c_i - u).V) + s L_opp(i),
//   A0 = sum_k (1-s) L_k w_k B_k,  V = sum_k (1-s) L_k w_k (3 c_k + 9 (c_k.u) c_k - 3 u),
// with w = 1/tau and B_k = feq_k/(w_k rho).  Parameter gradients accumulate in
// FP64: dJ/ds per cell in FP32 over at most kGradFold steps, then folded into
// FP64 (the fold steps are fixed by t, so every schedule sums alike).  The forward trajectory is
// checkpointed every K steps, under one of two schedules:
//  - segment buffers: the forward leaves the last segment's states in a
//    segment buffer and every earlier segment is recomputed from its
//    checkpoint.  Two segment buffers alternate: while the adjoint sweeps
//    segment k, segment k-1 is recomputed into the other buffer (for D2Q9
//    each adjoint step shares one launch with one recomputation step, so the
//    recomputation runs beside the latency-bound sweep);
//  - a resident pool of R state slots: the forward leaves its last R states
//    there, so the sweep over them recomputes nothing, and the earlier states
//    are recomputed from the checkpoints in chunks of up to R states into the
//    slots the sweep has finished with.  A 128^3 D3Q19 state is 159 MB, so
//    device memory holds most of a 2000-step trajectory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bf_lbm.h"
#include "lbm_common.cuh"

namespace bf {
namespace {

constexpr int kAdjBlock = 256;
// dJ/ds: the adjoint step t adds its term to an FP32 partial and folds the
// partial into the FP64 gradient when (t - 1) % kGradFold == 0 (t = 1, the
// sweep's last step, always folds)
constexpr int kGradFold = 64;

struct AdjParams {
    int nx, ny, nz;
    uint32_t n;
    float omega, wd, wm;
    const float* f_prev;    // f^(t-1), SoA planes of n
    float* f_next;          // forward output f^t
    const float* s;         // solid fraction, n
    const float* uin;       // inlet/outlet profile, ny*nz
    const float* ustar;     // target velocity, 3n
    const float* lam_in;    // adjoint of f^t
    float* lam_out;         // adjoint of f^(t-1)
    double* grad_s;         // n
    float* grad_acc;        // n: dJ/ds of the steps since the last fold into grad_s
    double* grad_in;        // ny*nz, from the x = 0 cells
    double* grad_out;       // ny*nz, from the x = nx-1 cells
    double* partials;       // one per block (objective)
};

// c . u for a lattice vector (components -1, 0, 1): only the nonzero terms
__device__ __forceinline__ float lattice_dot(const Dir c, float ux, float uy, float uz) {
    float r = 0.f;
    bool any = false;
    if (c.x) { r = c.x > 0 ? ux : -ux; any = true; }
    if (c.y) { r = any ? (c.y > 0 ? r + uy : r - uy) : (c.y > 0 ? uy : -uy); any = true; }
    if (c.z) { r = any ? (c.z > 0 ? r + uz : r - uz) : (c.z > 0 ? uz : -uz); }
    return r;
}
// acc += c v for a lattice component c in {-1, 0, 1}
__device__ __forceinline__ void lattice_axpy(int c, float v, float& acc) {
    if (c > 0) acc += v;
    else if (c < 0) acc -= v;
}

template <int Q>
__device__ __forceinline__ float feq_plain(int i, float rho, float ux, float uy, float uz) {
    const Dir c = Lattice<Q>::c(i);
    const float cu = c.x * ux + c.y * uy + c.z * uz;
    const float uu = ux * ux + uy * uy + uz * uz;
    return Lattice<Q>::w(i) * rho * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
}
// d feq_i(1, (u,0,0)) / d u
template <int Q>
__device__ __forceinline__ float dfeq_du(int i, float u) {
    const Dir c = Lattice<Q>::c(i);
    return Lattice<Q>::w(i) * (3.0f * c.x + 9.0f * (float)(c.x * c.x) * u - 3.0f * u);
}

__device__ __forceinline__ uint32_t adj_cell(const AdjParams& p, int x, int y, int z) {
    return (uint32_t)x + (uint32_t)p.nx * ((uint32_t)y + (uint32_t)p.ny * (uint32_t)z);
}
// 0 interior (X, Y, Z set), 1 wall, 2 equilibrium inlet/outlet
template <int Q>
__device__ __forceinline__ int adj_source(const AdjParams& p, int x, int y, int z, int i, int& X, int& Y, int& Z) {
    const Dir c = Lattice<Q>::c(i);
    X = x - c.x; Y = y - c.y; Z = z - c.z;
    if (Y < 0 || Y >= p.ny) return 1;
    if (X < 0 || X >= p.nx) return 2;
    Z = Z < 0 ? Z + p.nz : (Z >= p.nz ? Z - p.nz : Z);
    return 0;
}

template <int Q>
__device__ __forceinline__ void adj_pull(const AdjParams& p, int x, int y, int z, uint32_t n, float (&g)[Q]) {
    const float ui = p.uin[(uint32_t)z * p.ny + y];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        int X, Y, Z;
        const int kind = adj_source<Q>(p, x, y, z, i, X, Y, Z);
        if (kind == 0) g[i] = p.f_prev[(uint64_t)i * p.n + adj_cell(p, X, Y, Z)];
        else if (kind == 1) g[i] = p.f_prev[(uint64_t)opp(i) * p.n + n];
        else g[i] = feq_plain<Q>(i, 1.0f, ui, 0.f, 0.f);
    }
}

// A row (y, z) off the walls (0 < y < ny - 1): population i of cell x comes
// from cell x - c_i of plane i, z periodic, except where x - c_i leaves the
// domain in x (the equilibrium inlet and outlet).  A block covers part of one
// row, so the source's offset from the cell is the same for all its threads
// and a source index costs one integer add.
struct RowGeom {
    uint32_t n;          // the thread's cell
    uint32_t nx;
    uint32_t zup, zdn;   // index shift to the source plane z - c_z for c_z = +1 / -1 (periodic)
    bool xlo, xhi;       // x = 0, x = nx - 1
};
__device__ __forceinline__ RowGeom row_geom(const AdjParams& p, int x, int y, int z) {
    RowGeom r;
    const uint32_t nx = (uint32_t)p.nx, nxny = nx * (uint32_t)p.ny, last = (uint32_t)(p.nz - 1) * nxny;
    r.n = (uint32_t)x + nx * ((uint32_t)y + (uint32_t)p.ny * (uint32_t)z);
    r.nx = nx;
    r.zup = z == 0 ? last : 0u - nxny;
    r.zdn = z == p.nz - 1 ? 0u - last : nxny;
    r.xlo = x == 0;
    r.xhi = x == p.nx - 1;
    return r;
}
// index of cell x - c_i (in [0, n) for a row off the walls and a source inside in x)
template <int Q>
__device__ __forceinline__ uint32_t row_src(const RowGeom& r, int i) {
    const Dir c = Lattice<Q>::c(i);
    uint32_t d = 0u - (uint32_t)c.x;
    if (c.y > 0) d -= r.nx;
    else if (c.y < 0) d += r.nx;
    if (c.z > 0) d += r.zup;
    else if (c.z < 0) d += r.zdn;
    return r.n + d;
}
// the source of population i lies outside in x (equilibrium inlet/outlet)
template <int Q>
__device__ __forceinline__ bool row_outside(const RowGeom& r, int i) {
    const Dir c = Lattice<Q>::c(i);
    return (c.x > 0 && r.xlo) || (c.x < 0 && r.xhi);
}
template <int Q>
__device__ __forceinline__ void adj_pull_row(const AdjParams& p, const RowGeom& r, float ui, float (&g)[Q]) {
#pragma unroll
    for (int i = 0; i < Q; i++) {
        if (row_outside<Q>(r, i)) g[i] = feq_plain<Q>(i, 1.0f, ui, 0.f, 0.f);
        else g[i] = p.f_prev[(uint64_t)i * p.n + row_src<Q>(r, i)];
    }
}
// density and momentum of the pulled populations (zero lattice components left out)
template <int Q>
__device__ __forceinline__ void adj_moments(const float (&g)[Q], float& rho, float& jx, float& jy, float& jz) {
    rho = 0.f; jx = 0.f; jy = 0.f; jz = 0.f;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const Dir c = Lattice<Q>::c(i);
        rho += g[i];
        lattice_axpy(c.x, g[i], jx); lattice_axpy(c.y, g[i], jy); lattice_axpy(c.z, g[i], jz);
    }
}

__device__ __forceinline__ void block_sum_store(double v, double* out) {
    __shared__ double sm[kAdjBlock / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double t = lane < nw ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) out[blockIdx.x + (uint64_t)gridDim.x * (blockIdx.y + (uint64_t)gridDim.y * blockIdx.z)] = t;
    }
}

template <int Q>
__global__ void __launch_bounds__(kAdjBlock) adj_init_kernel(AdjParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= p.nx) return;
    const uint32_t n = adj_cell(p, x, y, z);
    const float ui = p.uin[(uint32_t)z * p.ny + y];
#pragma unroll
    for (int i = 0; i < Q; i++) p.f_next[(uint64_t)i * p.n + n] = feq_plain<Q>(i, 1.0f, ui, 0.f, 0.f);
}

template <int Q, bool FINAL>
__device__ __forceinline__ double adj_forward_cell(const AdjParams& p, int x, int y, int z) {
    using L = Lattice<Q>;
    double contrib = 0.0;
    {
        const uint32_t n = adj_cell(p, x, y, z);
        float g[Q];
        if (y > 0 && y < p.ny - 1) adj_pull_row<Q>(p, row_geom(p, x, y, z), p.uin[(uint32_t)z * p.ny + y], g);
        else adj_pull<Q>(p, x, y, z, n, g);
        float rho, jx, jy, jz;
        adj_moments<Q>(g, rho, jx, jy, jz);
        const float rr = 1.0f / rho;
        const float ux = jx * rr, uy = jy * rr, uz = jz * rr;
        const float s = p.s[n];
        if (FINAL) {
            const float dx = ux - p.ustar[3 * (uint64_t)n], dy = uy - p.ustar[3 * (uint64_t)n + 1],
                        dz = uz - p.ustar[3 * (uint64_t)n + 2];
            contrib = (double)p.wd * 2.0 * (double)s * (double)jx +
                      (double)p.wm * ((double)dx * dx + (double)dy * dy + (double)dz * dz);
        } else {
#pragma unroll
            for (int i = 0; i < Q; i++) {
                const float gc = g[i] + (feq_plain<Q>(i, rho, ux, uy, uz) - g[i]) * p.omega;
                const float gco = g[opp(i)];
                p.f_next[(uint64_t)i * p.n + n] = (1.0f - s) * gc + s * gco;
            }
        }
    }
    return contrib;
}

template <int Q, bool FINAL>
__global__ void __launch_bounds__(kAdjBlock) adj_forward_kernel(AdjParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    const double contrib = x < p.nx ? adj_forward_cell<Q, FINAL>(p, x, y, z) : 0.0;
    if (FINAL) block_sum_store(contrib, p.partials);
}

// ROW: a row off the walls (the sources at block-uniform offsets); else the
// general pull and push of the wall rows
template <int Q, bool FINAL, bool FOLD, bool ROW>
__device__ __forceinline__ void adj_backward_cell(const AdjParams& p, int x, int y, int z) {
    using L = Lattice<Q>;
    const uint32_t n = adj_cell(p, x, y, z);
    constexpr bool off_walls = ROW;
    const RowGeom r = row_geom(p, x, y, z);
    const uint32_t row = (uint32_t)z * p.ny + y;
    const float ui = p.uin[row];
    // every load of the step is issued before any arithmetic, so the step
    // waits on memory once: the pulled state, the incoming adjoint, the
    // solid fraction and the running parameter gradient
    float g[Q], lam[Q];
    if constexpr (off_walls) adj_pull_row<Q>(p, r, ui, g);
    else adj_pull<Q>(p, x, y, z, n, g);
    if (!FINAL) {
#pragma unroll
        for (int k = 0; k < Q; k++) lam[k] = p.lam_in[(uint64_t)k * p.n + n];
    }
    const float s = p.s[n];
    const float gs_acc = p.grad_acc[n];
    float rho, jx, jy, jz;
    adj_moments<Q>(g, rho, jx, jy, jz);
    const float rr = 1.0f / rho;
    const float ux = jx * rr, uy = jy * rr, uz = jz * rr;
    // the cell's transposed Jacobian as a few scalars; mu_i is formed where
    // it is stored (no array of Q adjoint populations held in registers)
    float gs;
    float fdx = 0.f, fdy = 0.f, fdz = 0.f;        // final step
    float a0 = 0.f, a1 = 0.f;                     // other steps
    const float om = p.omega;
    float Vx = 0.f, Vy = 0.f, Vz = 0.f;
    if constexpr (FINAL) {
        // dJ/dg_i = wd 2 s c_ix + wm sum_a 2 (u_a - u*_a)(c_ia - u_a)/rho,  dJ/ds = wd 2 j_x
        fdx = 2.0f * p.wm * (ux - p.ustar[3 * (uint64_t)n]) * rr;
        fdy = 2.0f * p.wm * (uy - p.ustar[3 * (uint64_t)n + 1]) * rr;
        fdz = 2.0f * p.wm * (uz - p.ustar[3 * (uint64_t)n + 2]) * rr;
        gs = 2.0f * p.wd * jx;
    } else {
        // The lattice components are -1, 0 or 1 and known per unrolled
        // direction: terms with a zero component are left out and the others
        // added or subtracted (IEEE arithmetic does not let the compiler drop
        // x * 0 or x + 0 itself).  With B_k = 1 + 3 cu_k + 4.5 cu_k^2 - 1.5 uu
        // (shared by A0 and the equilibrium) and L_k = (1 - s) lam_k w_k:
        //   A0 = sum_k L_k B_k,  V = sum_k L_k (3 + 9 cu_k) c_k - 3 u sum_k L_k.
        const float oms = 1.0f - s;
        const float base = 1.0f - 1.5f * (ux * ux + uy * uy + uz * uz);
        float A0 = 0.f, Lsum = 0.f, gsf = 0.f;
#pragma unroll
        for (int k = 0; k < Q; k++) {
            const Dir c = L::c(k);
            const float cu = lattice_dot(c, ux, uy, uz);
            const float Bk = fmaf(fmaf(4.5f, cu, 3.0f), cu, base);
            const float Lk = oms * lam[k] * L::w(k);
            A0 = fmaf(Lk, Bk, A0);
            Lsum += Lk;
            const float q = Lk * fmaf(9.0f, cu, 3.0f);
            lattice_axpy(c.x, q, Vx); lattice_axpy(c.y, q, Vy); lattice_axpy(c.z, q, Vz);
            const float feq = L::w(k) * rho * Bk;
            const float gck = g[k] + (feq - g[k]) * om;
            gsf += lam[k] * (g[opp(k)] - gck);
        }
        Vx = fmaf(-3.0f * ux, Lsum, Vx); Vy = fmaf(-3.0f * uy, Lsum, Vy); Vz = fmaf(-3.0f * uz, Lsum, Vz);
        gs = gsf;
        // mu_i = (1 - om)(1 - s) lam_i + om (A0 + (c_i - u).V) + s lam_opp(i)
        a1 = (1.0f - om) * oms;
        a0 = om * (A0 - (ux * Vx + uy * Vy + uz * Vz));
    }
    auto mu_of = [&](int i) -> float {
        const Dir c = L::c(i);
        if constexpr (FINAL) {
            return 2.0f * p.wd * s * c.x + fdx * (c.x - ux) + fdy * (c.y - uy) + fdz * (c.z - uz);
        } else {
            float cv = 0.f;
            lattice_axpy(c.x, Vx, cv); lattice_axpy(c.y, Vy, cv); lattice_axpy(c.z, Vz, cv);
            return fmaf(a1, lam[i], fmaf(om, cv, a0)) + s * lam[opp(i)];
        }
    };
    if (FOLD) {
        p.grad_s[n] += (double)(gs_acc + gs);
        p.grad_acc[n] = 0.0f;
    } else {
        p.grad_acc[n] = gs_acc + gs;
    }
    // transpose of the pull: mu_i goes where g_i came from; the part sent to
    // an equilibrium source becomes dJ/du of the inlet/outlet row
    if constexpr (off_walls) {
        // the push indices are the pull's; recomputing them (one add each)
        // from a copy of the cell index the compiler cannot match keeps 19
        // indices from staying live across the step
        RowGeom rs = r;
        asm volatile("mov.b32 %0, %1;" : "=r"(rs.n) : "r"(r.n));
        float guf = 0.f;
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const float mi = mu_of(i);
            if (!row_outside<Q>(rs, i)) p.lam_out[(uint64_t)i * p.n + row_src<Q>(rs, i)] = mi;
            else guf += mi * dfeq_du<Q>(i, ui);
        }
        if (r.xlo || r.xhi) {
            // populations of f^(t-1) that leave through the inlet or outlet feed nothing
#pragma unroll
            for (int j = 0; j < Q; j++) {
                const Dir c = L::c(j);
                if ((c.x < 0 && r.xlo) || (c.x > 0 && r.xhi)) p.lam_out[(uint64_t)j * p.n + n] = 0.0f;
            }
            if (r.xlo) p.grad_in[row] += (double)guf;
            else p.grad_out[row] += (double)guf;
        }
    } else {
        float guf = 0.f;
        bool eq_source = false;
#pragma unroll
        for (int i = 0; i < Q; i++) {
            int X, Y, Z;
            const int kind = adj_source<Q>(p, x, y, z, i, X, Y, Z);
            const float mi = mu_of(i);
            if (kind == 0) p.lam_out[(uint64_t)i * p.n + adj_cell(p, X, Y, Z)] = mi;
            else if (kind == 1) p.lam_out[(uint64_t)opp(i) * p.n + n] = mi;
            else { guf += mi * dfeq_du<Q>(i, ui); eq_source = true; }
        }
        // populations of f^(t-1) that leave through the inlet or outlet feed nothing
#pragma unroll
        for (int j = 0; j < Q; j++) {
            const Dir c = L::c(j);
            const int X = x + c.x, Y = y + c.y;
            if (Y >= 0 && Y < p.ny && (X < 0 || X >= p.nx)) p.lam_out[(uint64_t)j * p.n + n] = 0.0f;
        }
        if (eq_source) {
            if (x == 0) p.grad_in[row] += (double)guf;
            else p.grad_out[row] += (double)guf;
        }
    }
}

// the wall rows' step as a call of its own, so that its registers do not
// weigh on the rows off the walls (the kernel's common case)
template <int Q, bool FINAL, bool FOLD>
__device__ __noinline__ void adj_backward_wall_row(const AdjParams p, int x, int y, int z) {
    adj_backward_cell<Q, FINAL, FOLD, false>(p, x, y, z);
}
template <int Q, bool FINAL, bool FOLD>
__device__ __forceinline__ void adj_backward_any(const AdjParams& p, int x, int y, int z) {
    if (y > 0 && y < p.ny - 1) adj_backward_cell<Q, FINAL, FOLD, true>(p, x, y, z);
    else adj_backward_wall_row<Q, FINAL, FOLD>(p, x, y, z);
}

// blocks per SM of the adjoint step: D2Q9 5 (48 registers; the 512x256
// channel's backward measured 13.3 ms, 14.0 ms at 4 blocks); D3Q19 4 (64
// registers; the 128^3 channel's backward measured 474 / 394 / 351 / 362 ms
// at 2 / 3 / 4 / 5 blocks, 640 ms at 1)
#ifndef BF_ADJ_MIN_BLOCKS_Q19
#define BF_ADJ_MIN_BLOCKS_Q19 4
#endif
#ifndef BF_ADJ_MIN_BLOCKS_Q9
#define BF_ADJ_MIN_BLOCKS_Q9 5
#endif
template <int Q>
constexpr int adj_min_blocks() { return Q == 9 ? BF_ADJ_MIN_BLOCKS_Q9 : BF_ADJ_MIN_BLOCKS_Q19; }

template <int Q, bool FINAL, bool FOLD>
__global__ void __launch_bounds__(kAdjBlock, adj_min_blocks<Q>()) adj_backward_kernel(AdjParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x < p.nx) adj_backward_any<Q, FINAL, FOLD>(p, x, y, z);
}

// One adjoint step (blocks z < nz, first in launch order: the longer of the
// two) and one step of the recomputation of the previous segment (blocks
// z >= nz) in one launch.  The two read and write disjoint buffers, so their
// blocks run side by side; stream order keeps each chain in sequence.
template <int Q, bool FOLD>
__global__ void __launch_bounds__(kAdjBlock, adj_min_blocks<Q>()) adj_sweep_recompute_kernel(AdjParams pb, AdjParams pf) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= pb.nx) return;
    if (z < pb.nz) adj_backward_any<Q, false, FOLD>(pb, x, y, z);
    else adj_forward_cell<Q, false>(pf, x, y, z - pb.nz);
}

// d f^0 / d u_in: grad[row] += sum_x sum_i lam^0_i(x) dfeq_i/du, one block per (y, z) row
template <int Q>
__global__ void __launch_bounds__(kAdjBlock) adj_init_grad_kernel(AdjParams p) {
    const int y = blockIdx.x, z = blockIdx.y;
    const uint32_t row = (uint32_t)z * p.ny + y;
    const float ui = p.uin[row];
    double acc = 0.0;
    for (int x = threadIdx.x; x < p.nx; x += blockDim.x) {
        const uint32_t n = adj_cell(p, x, y, z);
#pragma unroll
        for (int i = 0; i < Q; i++) acc += (double)(p.lam_in[(uint64_t)i * p.n + n] * dfeq_du<Q>(i, ui));
    }
    __shared__ double sm[kAdjBlock];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kAdjBlock / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) p.grad_in[row] += sm[0];
}

__global__ void sum_partials_kernel(const double* partials, uint32_t nb, double* out) {
    __shared__ double sm[256];
    double acc = 0.0;
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) acc += partials[b];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

}  // namespace
}  // namespace bf

using namespace bf;

struct bf_adjoint {
    bf_adjoint_desc d{};
    int Q = 0;
    uint32_t n = 0, rows = 0, nblocks = 0;
    int nseg = 0;
    int resident = 0;             // R: 0 for the segment buffers, else the pool's slot count
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    float *s = nullptr, *uin = nullptr, *ustar = nullptr;
    std::vector<float*> ckpt, seg[2];
    float* pool = nullptr;        // R states, slot j at pool + j Q n
    float* slot(int j) const { return pool + (size_t)j * Q * n; }
    float *pp[2] = {nullptr, nullptr}, *lam[2] = {nullptr, nullptr};
    double *grad_s = nullptr, *grad_in = nullptr, *grad_out = nullptr, *partials = nullptr, *J = nullptr;
    float* grad_acc = nullptr;
    cudaGraphExec_t fwd_graph = nullptr, bwd_graph = nullptr;
    bool forward_done = false;
};

namespace {

int afail(int code, const std::string& msg) {
    bf::record_error(msg);
    return code;
}
#define ACUDA(call)                                                                                       \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return afail(e_ == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA,            \
                         std::string(#call " failed: ") + cudaGetErrorString(e_));                        \
    } while (0)

AdjParams base_params(bf_adjoint* a) {
    AdjParams p{};
    p.nx = a->d.resolution[0]; p.ny = a->d.resolution[1]; p.nz = a->d.resolution[2];
    p.n = a->n;
    p.omega = 1.0f / a->d.relaxation_time;
    p.wd = a->d.drag_weight;
    p.wm = a->d.mismatch_weight;
    p.s = a->s; p.uin = a->uin; p.ustar = a->ustar;
    p.grad_s = a->grad_s; p.grad_in = a->grad_in; p.grad_out = a->grad_out; p.partials = a->partials;
    p.grad_acc = a->grad_acc;
    return p;
}

dim3 adj_grid(const bf_adjoint* a, int& block) {
    const int nx = a->d.resolution[0];
    block = nx >= kAdjBlock ? kAdjBlock : ((nx + 31) / 32) * 32;
    return dim3((unsigned)((nx + block - 1) / block), (unsigned)a->d.resolution[1], (unsigned)a->d.resolution[2]);
}

bool grad_fold(int t) { return (t - 1) % kGradFold == 0; }

// the adjoint step t (the last step T seeds the adjoint from dJ/dg)
template <int Q>
void launch_adjoint_step(bf_adjoint* a, const AdjParams& p, int t, dim3 grid, int block) {
    const bool fin = t == a->d.steps, fold = grad_fold(t);
    if (fin && fold) adj_backward_kernel<Q, true, true><<<grid, block, 0, a->stream>>>(p);
    else if (fin) adj_backward_kernel<Q, true, false><<<grid, block, 0, a->stream>>>(p);
    else if (fold) adj_backward_kernel<Q, false, true><<<grid, block, 0, a->stream>>>(p);
    else adj_backward_kernel<Q, false, false><<<grid, block, 0, a->stream>>>(p);
}

// first state of the resident tail under the pool schedule: f^P .. f^(T-1)
// stay in slots 0 .. R-1 (P = T when nothing is resident, T = 1)
int pool_tail_start(const bf_adjoint* a) { return a->d.steps - std::min(a->resident, a->d.steps - 1); }

template <int Q>
cudaError_t enqueue_forward(bf_adjoint* a) {
    int block;
    const dim3 grid = adj_grid(a, block);
    const int T = a->d.steps, K = a->d.checkpoint_interval;
    AdjParams p = base_params(a);
    p.f_next = a->ckpt[0];
    adj_init_kernel<Q><<<grid, block, 0, a->stream>>>(p);
    const float* cur = a->ckpt[0];
    // states of the last segment (or the resident tail) go straight to the
    // buffer where the backward sweep starts, so they need no recomputation
    const int t_last = (a->nseg - 1) * K;
    const int P = a->resident ? pool_tail_start(a) : T;
    for (int t = 1; t < T; t++) {
        float* dst;
        if (a->resident) dst = t >= P ? a->slot(t - P) : (t % K == 0 ? a->ckpt[t / K] : a->pp[t & 1]);
        else dst = (t % K == 0) ? a->ckpt[t / K] : (t > t_last ? a->seg[(a->nseg - 1) & 1][t - t_last] : a->pp[t & 1]);
        p.f_prev = cur;
        p.f_next = dst;
        adj_forward_kernel<Q, false><<<grid, block, 0, a->stream>>>(p);
        cur = dst;
    }
    p.f_prev = cur;
    p.f_next = nullptr;
    adj_forward_kernel<Q, true><<<grid, block, 0, a->stream>>>(p);
    sum_partials_kernel<<<1, 256, 0, a->stream>>>(a->partials, a->nblocks, a->J);
    return cudaGetLastError();
}

// D2Q9 merges each adjoint step with a recomputation step; D3Q19's adjoint
// kernel holds many more registers than its forward, so there the
// recomputation runs as its own launches at the forward's occupancy (the
// 128^3 channel's backward: 351 ms against 527 ms merged)
#ifndef BF_ADJ_MERGE_Q19
#define BF_ADJ_MERGE_Q19 0
#endif
template <int Q>
constexpr bool kMergeRecompute = Q == 9 || BF_ADJ_MERGE_Q19;

// The pool schedule's backward: adjoint steps t = T .. P+1 over the resident
// tail, then the states below P in chunks from the top.  A chunk starts at
// the checkpoint `start` that leaves at most R states start+1 .. top above it
// (start <= top because R >= K - 1); they are recomputed into slots 0 ..
// top-start-1, which the sweep has finished with, and swept.
template <int Q>
cudaError_t enqueue_backward_pool(bf_adjoint* a) {
    int block;
    const dim3 grid = adj_grid(a, block);
    const int T = a->d.steps, K = a->d.checkpoint_interval, R = a->resident;
    const int P = pool_tail_start(a);
    AdjParams p = base_params(a);
    int cur = -1;
    auto sweep = [&](int t, const float* f_prev) {
        const int out = cur == 0 ? 1 : 0;
        p.f_prev = f_prev;
        p.lam_out = a->lam[out];
        p.lam_in = t == T ? nullptr : a->lam[cur];
        launch_adjoint_step<Q>(a, p, t, grid, block);
        cur = out;
    };
    for (int t = T; t > P; t--) sweep(t, a->slot(t - 1 - P));
    AdjParams q = p;
    for (int top = P - 1; top >= 0;) {
        const int start = top > R ? K * ((top - R + K - 1) / K) : 0;
        const float* prev = a->ckpt[start / K];
        for (int j = start + 1; j <= top; j++) {
            q.f_prev = prev;
            q.f_next = a->slot(j - start - 1);
            adj_forward_kernel<Q, false><<<grid, block, 0, a->stream>>>(q);
            prev = q.f_next;
        }
        for (int t = top + 1; t > start; t--) sweep(t, t - 1 == start ? a->ckpt[start / K] : a->slot(t - 2 - start));
        top = start - 1;
    }
    p.lam_in = a->lam[cur];
    adj_init_grad_kernel<Q><<<dim3((unsigned)a->d.resolution[1], (unsigned)a->d.resolution[2]), kAdjBlock, 0, a->stream>>>(p);
    return cudaGetLastError();
}

template <int Q>
cudaError_t enqueue_backward(bf_adjoint* a) {
    int block;
    const dim3 grid = adj_grid(a, block);
    const int T = a->d.steps, K = a->d.checkpoint_interval, nseg = a->nseg;
    AdjParams p = base_params(a);
    cudaMemsetAsync(a->grad_s, 0, (size_t)a->n * sizeof(double), a->stream);
    cudaMemsetAsync(a->grad_acc, 0, (size_t)a->n * sizeof(float), a->stream);
    cudaMemsetAsync(a->grad_in, 0, (size_t)a->rows * sizeof(double), a->stream);
    cudaMemsetAsync(a->grad_out, 0, (size_t)a->rows * sizeof(double), a->stream);
    if (a->resident) return enqueue_backward_pool<Q>(a);
    // one stream: adjoint step i of segment k together with step i + 1
    // of the recomputation of segment k - 1 (into the other segment
    // buffer, which the sweep of segment k + 1 has finished with)
    const dim3 grid2(grid.x, grid.y, grid.z * 2);
    int cur = -1;
    for (int k = nseg - 1; k >= 0; k--) {
        const int t0 = k * K, t1 = std::min(t0 + K, T);
        const int r = k - 1;  // segment being recomputed, if any
        const int r_steps = r >= 0 ? K - 1 : 0;
        AdjParams q = p;
        const float* rprev = r >= 0 ? a->ckpt[r] : nullptr;
        int j = 1;  // next recomputation step, f^(r K + j)
        for (int t = t1; t >= t0 + 1; t--) {
            p.f_prev = (t - 1 == t0) ? a->ckpt[k] : a->seg[k & 1][t - 1 - t0];
            const int out = cur == 0 ? 1 : 0;
            p.lam_out = a->lam[out];
            p.lam_in = t == T ? nullptr : a->lam[cur];
            if (kMergeRecompute<Q> && t != T && j <= r_steps) {
                q.f_prev = rprev;
                q.f_next = a->seg[r & 1][j];
                if (grad_fold(t)) adj_sweep_recompute_kernel<Q, true><<<grid2, block, 0, a->stream>>>(p, q);
                else adj_sweep_recompute_kernel<Q, false><<<grid2, block, 0, a->stream>>>(p, q);
                rprev = q.f_next;
                j++;
            } else {
                launch_adjoint_step<Q>(a, p, t, grid, block);
            }
            cur = out;
        }
        for (; j <= r_steps; j++) {  // a short last segment leaves recomputation steps over
            q.f_prev = rprev;
            q.f_next = a->seg[r & 1][j];
            adj_forward_kernel<Q, false><<<grid, block, 0, a->stream>>>(q);
            rprev = q.f_next;
        }
    }
    p.lam_in = a->lam[cur];
    adj_init_grad_kernel<Q><<<dim3((unsigned)a->d.resolution[1], (unsigned)a->d.resolution[2]), kAdjBlock, 0, a->stream>>>(p);
    return cudaGetLastError();
}

int run_graph(bf_adjoint* a, cudaGraphExec_t* exec, bool forward) {
    if (!*exec) {
        ACUDA(cudaStreamBeginCapture(a->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e;
        if (a->Q == 9) e = forward ? enqueue_forward<9>(a) : enqueue_backward<9>(a);
        else e = forward ? enqueue_forward<19>(a) : enqueue_backward<19>(a);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(a->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return afail(BF_ERR_CUDA, std::string("adjoint capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        cudaError_t e3 = cudaGraphInstantiate(exec, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) return afail(BF_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e3));
    }
    ACUDA(cudaGraphLaunch(*exec, a->stream));
    return BF_OK;
}

}  // namespace

extern "C" {

void bf_adjoint_desc_default(bf_adjoint_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->resolution[0] = 512; d->resolution[1] = 256; d->resolution[2] = 1;
    d->relaxation_time = 0.6f;
    d->velocity_set = BF_D2Q9;
    d->steps = 2000;
    d->checkpoint_interval = 100;
    d->drag_weight = 1.0f;
    d->mismatch_weight = 1.0f;
}

int bf_adjoint_destroy(bf_adjoint* a) {
    if (!a) return BF_OK;
    if (a->stream) cudaStreamSynchronize(a->stream);
    if (a->fwd_graph) cudaGraphExecDestroy(a->fwd_graph);
    if (a->bwd_graph) cudaGraphExecDestroy(a->bwd_graph);
    for (void* p : a->allocs) cudaFree(p);
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
    return BF_OK;
}

int bf_adjoint_create(bf_adjoint** out, const bf_adjoint_desc* d) {
    if (!out || !d) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: NULL argument");
    *out = nullptr;
    const int Q = d->velocity_set == BF_D2Q9 ? 9 : (d->velocity_set == BF_D3Q19 ? 19 : 0);
    if (!Q) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: velocity set must be D2Q9 or D3Q19");
    const int nx = d->resolution[0], ny = d->resolution[1], nz = d->resolution[2];
    if (nx <= 0 || ny <= 0 || nz <= 0 || (Q == 9 && nz != 1) || ny > 65535 || nz > 65535)
        return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: bad resolution");
    if (d->steps < 1 || d->checkpoint_interval < 1) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: steps and checkpoint_interval must be positive");
    if (d->resident_states < BF_ADJOINT_RESIDENT_AUTO)
        return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: resident_states must be 0, positive or BF_ADJOINT_RESIDENT_AUTO");
    // a pool below K - 1 slots could not hold the states between two checkpoints
    const int min_resident = std::min(d->checkpoint_interval - 1, d->steps - 1);
    if (d->resident_states > 0 && d->resident_states < min_resident)
        return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: resident_states must be at least checkpoint_interval - 1");
    if (!(d->relaxation_time > 0.5f)) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: relaxation_time must exceed 0.5");
    const uint64_t n64 = (uint64_t)nx * ny * nz;
    if (n64 * Q >= (1ull << 40)) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_create: domain too large");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return afail(BF_ERR_NO_DEVICE, "bf_adjoint_create: no CUDA device visible");
    }
    bf_adjoint* a = new bf_adjoint();
    a->d = *d;
    a->Q = Q;
    a->n = (uint32_t)n64;
    a->rows = (uint32_t)ny * nz;
    a->nseg = (d->steps + d->checkpoint_interval - 1) / d->checkpoint_interval;
    {
        const int block = nx >= kAdjBlock ? kAdjBlock : ((nx + 31) / 32) * 32;
        a->nblocks = (uint32_t)((nx + block - 1) / block) * (uint32_t)ny * (uint32_t)nz;
    }
    auto alloc = [&](size_t bytes, void** p) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) a->allocs.push_back(*p);
        return e;
    };
    const size_t state = (size_t)Q * a->n * sizeof(float);
    // the adjoint's one stream (forward, and the backward's merged sweep and
    // recomputation launches) runs at the highest stream priority
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    cudaError_t e = cudaStreamCreateWithPriority(&a->stream, cudaStreamNonBlocking, prio_high);
    if (e == cudaSuccess) e = alloc((size_t)a->n * 4, (void**)&a->s);
    if (e == cudaSuccess) e = alloc((size_t)a->rows * 4, (void**)&a->uin);
    if (e == cudaSuccess) e = alloc((size_t)a->n * 12, (void**)&a->ustar);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = alloc(state, (void**)&a->pp[k]);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = alloc(state, (void**)&a->lam[k]);
    if (e == cudaSuccess) e = alloc((size_t)a->n * 8, (void**)&a->grad_s);
    if (e == cudaSuccess) e = alloc((size_t)a->n * 4, (void**)&a->grad_acc);
    if (e == cudaSuccess) e = alloc((size_t)a->rows * 8, (void**)&a->grad_in);
    if (e == cudaSuccess) e = alloc((size_t)a->rows * 8, (void**)&a->grad_out);
    if (e == cudaSuccess) e = alloc((size_t)a->nblocks * 8, (void**)&a->partials);
    if (e == cudaSuccess) e = alloc(8, (void**)&a->J);
    int64_t R = d->resident_states;
    if (e == cudaSuccess && R == BF_ADJOINT_RESIDENT_AUTO) {
        // what is free now, less the reserve and the checkpoints' upper bound
        size_t free_b = 0, total_b = 0;
        e = cudaMemGetInfo(&free_b, &total_b);
        const uint64_t reserve = std::max<uint64_t>(8ull << 30, total_b / 20);
        const uint64_t ckpts = (uint64_t)a->nseg * state;
        R = free_b > reserve + ckpts ? (int64_t)((free_b - reserve - ckpts) / state) : 0;
        R = std::max<int64_t>(R, min_resident);
    }
    R = std::min<int64_t>(R, d->steps - 1);
    a->resident = (int)R;
    if (a->resident) {
        // the pool, and checkpoints at the multiples of K below the resident tail
        if (e == cudaSuccess) e = alloc((size_t)a->resident * state, (void**)&a->pool);
        a->ckpt.assign((d->steps - a->resident - 1) / d->checkpoint_interval + 1, nullptr);
    } else {
        a->ckpt.assign(a->nseg, nullptr);
        for (int b = 0; b < (a->nseg >= 2 ? 2 : 1); b++) {
            a->seg[b].assign(d->checkpoint_interval, nullptr);
            for (int j = 1; j < d->checkpoint_interval && e == cudaSuccess; j++) e = alloc(state, (void**)&a->seg[b][j]);
        }
    }
    for (size_t k = 0; k < a->ckpt.size() && e == cudaSuccess; k++) e = alloc(state, (void**)&a->ckpt[k]);
    if (e == cudaSuccess) e = cudaMemset(a->s, 0, (size_t)a->n * 4);
    if (e == cudaSuccess) e = cudaMemset(a->uin, 0, (size_t)a->rows * 4);
    if (e == cudaSuccess) e = cudaMemset(a->ustar, 0, (size_t)a->n * 12);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? BF_ERR_OUT_OF_MEMORY : BF_ERR_CUDA;
        std::string msg = std::string("bf_adjoint_create: ") + cudaGetErrorString(e);
        cudaGetLastError();
        bf_adjoint_destroy(a);
        return afail(code, msg);
    }
    *out = a;
    return BF_OK;
}

int bf_adjoint_set_parameters(bf_adjoint* a, const float* solid_fraction, const float* inlet_velocity) {
    if (!a) return afail(BF_ERR_INVALID_ARGUMENT, "NULL adjoint");
    ACUDA(cudaStreamSynchronize(a->stream));
    if (solid_fraction) ACUDA(cudaMemcpy(a->s, solid_fraction, (size_t)a->n * 4, cudaMemcpyHostToDevice));
    if (inlet_velocity) ACUDA(cudaMemcpy(a->uin, inlet_velocity, (size_t)a->rows * 4, cudaMemcpyHostToDevice));
    a->forward_done = false;
    return BF_OK;
}

int bf_adjoint_set_target(bf_adjoint* a, const float* u_target) {
    if (!a || !u_target) return afail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    ACUDA(cudaStreamSynchronize(a->stream));
    ACUDA(cudaMemcpy(a->ustar, u_target, (size_t)a->n * 12, cudaMemcpyHostToDevice));
    a->forward_done = false;
    return BF_OK;
}

int bf_adjoint_forward(bf_adjoint* a, double* objective) {
    if (!a) return afail(BF_ERR_INVALID_ARGUMENT, "NULL adjoint");
    int r = run_graph(a, &a->fwd_graph, true);
    if (r != BF_OK) return r;
    a->forward_done = true;
    if (objective) {
        ACUDA(cudaMemcpyAsync(objective, a->J, sizeof(double), cudaMemcpyDeviceToHost, a->stream));
        ACUDA(cudaStreamSynchronize(a->stream));
    }
    return BF_OK;
}

int bf_adjoint_backward(bf_adjoint* a, double* grad_solid_fraction, double* grad_inlet_velocity) {
    if (!a) return afail(BF_ERR_INVALID_ARGUMENT, "NULL adjoint");
    if (!a->forward_done) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_backward: run bf_adjoint_forward with the current parameters first");
    int r = run_graph(a, &a->bwd_graph, false);
    if (r != BF_OK) return r;
    if (grad_solid_fraction)
        ACUDA(cudaMemcpyAsync(grad_solid_fraction, a->grad_s, (size_t)a->n * 8, cudaMemcpyDeviceToHost, a->stream));
    if (grad_inlet_velocity) {
        std::vector<double> gin(a->rows), gout(a->rows);
        ACUDA(cudaMemcpyAsync(gin.data(), a->grad_in, (size_t)a->rows * 8, cudaMemcpyDeviceToHost, a->stream));
        ACUDA(cudaMemcpyAsync(gout.data(), a->grad_out, (size_t)a->rows * 8, cudaMemcpyDeviceToHost, a->stream));
        ACUDA(cudaStreamSynchronize(a->stream));
        for (uint32_t k = 0; k < a->rows; k++) grad_inlet_velocity[k] = gin[k] + gout[k];
    }
    ACUDA(cudaStreamSynchronize(a->stream));
    return BF_OK;
}

int bf_adjoint_time(bf_adjoint* a, int32_t repeats, float* forward_ms, float* backward_ms) {
    if (!a || repeats <= 0) return afail(BF_ERR_INVALID_ARGUMENT, "bf_adjoint_time: bad argument");
    cudaEvent_t e0, e1, e2;
    ACUDA(cudaEventCreate(&e0));
    ACUDA(cudaEventCreate(&e1));
    ACUDA(cudaEventCreate(&e2));
    float fsum = 0.f, bsum = 0.f;
    int r = BF_OK;
    for (int k = 0; k < repeats && r == BF_OK; k++) {
        cudaEventRecord(e0, a->stream);
        r = run_graph(a, &a->fwd_graph, true);
        if (r != BF_OK) break;
        a->forward_done = true;
        cudaEventRecord(e1, a->stream);
        r = run_graph(a, &a->bwd_graph, false);
        if (r != BF_OK) break;
        cudaEventRecord(e2, a->stream);
        cudaEventSynchronize(e2);
        float f = 0.f, b = 0.f;
        cudaEventElapsedTime(&f, e0, e1);
        cudaEventElapsedTime(&b, e1, e2);
        fsum += f;
        bsum += b;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (r != BF_OK) return r;
    if (forward_ms) *forward_ms = fsum / repeats;
    if (backward_ms) *backward_ms = bsum / repeats;
    return BF_OK;
}

int bf_adjoint_get_resident_states(const bf_adjoint* a, int32_t* resident_states) {
    if (!a || !resident_states) return afail(BF_ERR_INVALID_ARGUMENT, "NULL argument");
    *resident_states = a->resident;
    return BF_OK;
}

}  // extern "C"
