// lbm_kernels.cuh -- sm_103a kernels of the lattice Boltzmann update.
//
// Threads of a block run along x and the DDF is one structure-of-arrays
// buffer (population plane i at f + i*stride), so every population
// load/store of a warp touches consecutive elements.  The kernels:
//   step_kernel          generic fused stream+collide, one thread per cell
//   fast_step_kernel     periodic boxes, one thread per cell
//   fast2_step_kernel    periodic boxes, 16-bit storage, two cells per thread
//   masked_mixed_kernel  objects, open faces, thermal lattice: plain cells in
//                        the fast cell update, listed special cells in
//                        blocks of their own (masked_step_kernel: one pass)
//   stream_kernel, stream_thermal_kernel, init_kernel, ... the reference's
//                        other passes
// All evaluate the same expression trees (below), so they agree with one
// another and with the oracle bit for bit.
//
// The update is the fused stream+collide of the reference's esoteric-pull
// mode (collide.comp main, :676-794).  The AA pattern follows
// collide.comp:244-369: on an even step a cell reads population i from
// (x - c_i, slot i) and writes its post-collision population i to
// (x + c_i, slot opp(i)); on an odd step it reads (x, slot opp(i)) and
// writes (x, slot i).  A cell reads and writes the same private set of slots,
// so the update is race free in place.
#pragma once
#include "lbm_common.cuh"
#include "lbm_async.cuh"

#include <algorithm>
#include <type_traits>

namespace bf {

template <class R> struct CellSumT { R m, px, py, pz, ke; };
using CellSum = CellSumT<float>;

// Rounded, never-contracted operations: the kernels evaluate the same
// expression trees as the oracle, so results agree bit for bit.  Two trees:
//  * literal (FP32 and FP16 storage of f, and the FP64 reference stepper):
//    the reference's expressions (collide.comp:383-395, :512-629, :702-782)
//    in their written order, one IEEE operation per operator, divisions as
//    correctly rounded divisions (FDIV), no fused multiply-adds; products
//    with a lattice component (0, +-1) are exact and their zero terms are
//    left out, which changes nothing but the sign of a zero;
//  * shifted (fp16s / fp16c, extensions): the update on g = f - w with
//    divisions by launch uniforms as multiplications by once-rounded
//    reciprocals, u = j * (1/rho) with one IEEE division, opposite
//    populations summed pairwise (s = f_i + f_opp, d = f_i - f_opp), and the
//    multiply-adds marked FFMA single-rounding fused operations.  TRT (an
//    extension) uses this fixed order with every storage.
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float r_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float r_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double r_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }
#define FMUL r_mul
#define FADD r_add
#define FSUB r_sub
#define FDIV r_div

// exp for the pseudopotential psi = 1 - exp(-rho), the same operations as the
// oracle's exp_f32: Cody-Waite reduction x = k ln2 + r (ln2 split in a 15-bit
// head and a tail), degree-7 Taylor polynomial of exp(r) in Horner form
// (|r| <= ln2/2, truncation < 6e-9 relative), exact scaling by 2^k.
// Valid for x in [-87, 88].
__device__ __forceinline__ float exp_f32(float x) {
    const float L2E = 0x1.715476p+0f, LN2_HI = 0x1.62e4p-1f, LN2_LO = 0x1.7f7d1cp-20f;
    const float kf = rintf(FMUL(x, L2E));
    const float r = FSUB(FSUB(x, FMUL(kf, LN2_HI)), FMUL(kf, LN2_LO));
    float q = 0x1.a01a02p-13f;
    q = FADD(FMUL(q, r), 0x1.6c16c2p-10f);
    q = FADD(FMUL(q, r), 0x1.111112p-7f);
    q = FADD(FMUL(q, r), 0x1.555556p-5f);
    q = FADD(FMUL(q, r), 0x1.555556p-3f);
    q = FADD(FMUL(q, r), 0x1p-1f);
    q = FADD(FMUL(q, r), 1.0f);
    q = FADD(FMUL(q, r), 1.0f);
    return FMUL(q, __uint_as_float((uint32_t)((int)kf + 127) << 23));
}

// exp for the FP64 pseudopotential, the same operations as the oracle's
// exp_f64: Cody-Waite reduction (ln2 split in a head with 21 zero low bits
// and a tail), degree-13 Taylor polynomial in Horner form (|r| <= ln2/2,
// truncation < 5e-18 relative), exact scaling by 2^k.  Valid for x in
// [-708, 709]; within 1.1 ulp of the exact exponential.
__device__ __forceinline__ double exp_f64(double x) {
    const double L2E = 0x1.71547652b82fep+0, LN2_HI = 0x1.62e42fee00000p-1, LN2_LO = 0x1.a39ef35793c76p-33;
    const double kf = rint(FMUL(x, L2E));
    const double r = FSUB(FSUB(x, FMUL(kf, LN2_HI)), FMUL(kf, LN2_LO));
    double q = 0x1.6124613a86d09p-33;  // 1/13!
    q = FADD(FMUL(q, r), 0x1.1eed8eff8d898p-29);
    q = FADD(FMUL(q, r), 0x1.ae64567f544e4p-26);
    q = FADD(FMUL(q, r), 0x1.27e4fb7789f5cp-22);
    q = FADD(FMUL(q, r), 0x1.71de3a556c734p-19);
    q = FADD(FMUL(q, r), 0x1.a01a01a01a01ap-16);
    q = FADD(FMUL(q, r), 0x1.a01a01a01a01ap-13);
    q = FADD(FMUL(q, r), 0x1.6c16c16c16c17p-10);
    q = FADD(FMUL(q, r), 0x1.1111111111111p-7);
    q = FADD(FMUL(q, r), 0x1.5555555555555p-5);
    q = FADD(FMUL(q, r), 0x1.5555555555555p-3);
    q = FADD(FMUL(q, r), 0x1p-1);
    q = FADD(FMUL(q, r), 1.0);
    q = FADD(FMUL(q, r), 1.0);
    return FMUL(q, __longlong_as_double((long long)((int64_t)kf + 1023) << 52));
}
// psi = 1 - exp(-rho) (collide.comp:512-516, rho0 = 1) in the arithmetic type
__device__ __forceinline__ float psi_of(float rho) { return FSUB(1.0f, exp_f32(-rho)); }
__device__ __forceinline__ double psi_of(double rho) { return FSUB(1.0, exp_f64(-rho)); }

// c . v for a lattice direction with components in {-1, 0, 1}: the dot
// product's x, y, z sum with the zero terms dropped (they add +-0 only)
template <int CX, int CY, int CZ>
__device__ __forceinline__ float cdot(float vx, float vy, float vz) {
    float acc = 0.0f;
    bool first = true;
    if (CX != 0) { acc = CX > 0 ? vx : -vx; first = false; }
    if (CY != 0) { const float t = CY > 0 ? vy : -vy; acc = first ? t : FADD(acc, t); first = false; }
    if (CZ != 0) { const float t = CZ > 0 ? vz : -vz; acc = first ? t : FADD(acc, t); first = false; }
    return acc;
}
template <class R>
__device__ __forceinline__ R cdot_rt(const Dir c, R vx, R vy, R vz) {
    R acc = R(0);
    bool first = true;
    if (c.x != 0) { acc = c.x > 0 ? vx : -vx; first = false; }
    if (c.y != 0) { const R t = c.y > 0 ? vy : -vy; acc = first ? t : FADD(acc, t); first = false; }
    if (c.z != 0) { const R t = c.z > 0 ? vz : -vz; acc = first ? t : FADD(acc, t); first = false; }
    return acc;
}
#define FFMA r_fma
// u.u = fma(uz, uz, fma(uy, uy, ux*ux))
template <class R>
__device__ __forceinline__ R uu_of(R ux, R uy, R uz) {
    return FFMA(uz, uz, FFMA(uy, uy, FMUL(ux, ux)));
}
// (1 + cu/cs2 + cu^2/2/cs4 - uu/2/cs2) = fma(cu^2, R4/2, fma(cu, R2, 1 - uu R2/2))
template <class R>
__device__ __forceinline__ R bracket(R cu, R one_m, R R2, R R4h) {
    return FFMA(FMUL(cu, cu), R4h, FFMA(cu, R2, one_m));
}

// x / y for a launch-uniform divisor y, from the reciprocal split as
// r = RN(1/y) and a low part l close to 1/y - r: q = fma(x, r, RN(x l)), two
// operations (Brisebarre, Muller and Raina, "Accelerating correctly rounded
// floating-point division when the divisor is known in advance", IEEE Trans.
// Computers 53(8), 2004).  The host takes l = RN(1/y - r), or the nearest
// float to it for which the sequence passes, and checks the sequence against
// IEEE division for every significand of x with each launch divisor
// (StepParams::div_ok); the fast and boundary-aware kernels use it only when
// every check passed (div_m), the generic kernel per divisor (div_u).
// Double: the full division.
__device__ __forceinline__ float div_m(float x, float, float r, float l) {
    return __fmaf_rn(x, r, __fmul_rn(x, l));
}
__device__ __forceinline__ double div_m(double x, double y, double, double) { return __ddiv_rn(x, y); }
__device__ __forceinline__ float div_u(float x, float y, float r, float l, bool ok) {
    return ok ? div_m(x, y, r, l) : __fdiv_rn(x, y);
}
__device__ __forceinline__ double div_u(double x, double y, double, double, bool) { return __ddiv_rn(x, y); }
template <bool MK, class R>
__device__ __forceinline__ R div_k(R x, R y, R r, R l, bool ok) {
    if constexpr (MK) return div_m(x, y, r, l);
    else return div_u(x, y, r, l, ok);
}
// the divisors cs^2 and cs^4 of the literal evaluation, their reciprocals
// and checks
template <class R> struct Div { R cs2, rcs2, lcs2, cs4, rcs4, lcs4; bool ok2, ok4; };

// GLSL's dot(a, b) as written: a.x*b.x + a.y*b.y + a.z*b.z
template <class R>
__device__ __forceinline__ R dot_lit(R ax, R ay, R az, R bx, R by, R bz) {
    return FADD(FADD(FMUL(ax, bx), FMUL(ay, by)), FMUL(az, bz));
}
// collide.comp:589-604 (and the thermal :634-651) as written:
// (w p) (((1 + cu/cs2) + cu^2/2/cs4) - uuh), uuh = (u.u/2)/cs2 of the cell
template <bool MK, class R>
__device__ __forceinline__ R feq_lit(R wp, R cu, const Div<R>& d, R uuh) {
    return FMUL(wp, FSUB(FADD(FADD(R(1), div_k<MK>(cu, d.cs2, d.rcs2, d.lcs2, d.ok2)),
                              div_k<MK>(FMUL(FMUL(cu, cu), R(0.5)), d.cs4, d.rcs4, d.lcs4, d.ok4)),
                         uuh));
}
template <bool MK, class R>
__device__ __forceinline__ R uuh_of(R ux, R uy, R uz, const Div<R>& d) {
    return div_k<MK>(FMUL(dot_lit(ux, uy, uz, ux, uy, uz), R(0.5)), d.cs2, d.rcs2, d.lcs2, d.ok2);
}

template <int Q>
__device__ __forceinline__ void coords_wrap(int& cx, int& cy, int& cz, int nx, int ny, int nz, bool& open, uint32_t flags) {
    open = false;
    if (flags & F_PERIODIC_X) { cx = cx < 0 ? cx + nx : (cx >= nx ? cx - nx : cx); }
    else open |= (cx < 0 || cx >= nx);
    if (flags & F_PERIODIC_Y) { cy = cy < 0 ? cy + ny : (cy >= ny ? cy - ny : cy); }
    else open |= (cy < 0 || cy >= ny);
    if (flags & F_PERIODIC_Z) { cz = cz < 0 ? cz + nz : (cz >= nz ? cz - nz : cz); }
    else open |= (cz < 0 || cz >= nz);
}

__device__ __forceinline__ bool solid_id(const uint8_t* __restrict__ kind, uint32_t id) {
    return id != 0u && __ldg(kind + id) == 0;
}

// FP64 block reduction of the five conserved sums; one partial per block.
template <class R>
__device__ __forceinline__ void block_reduce_store(CellSumT<R> cs, double* __restrict__ out) {
    double v[5] = {(double)cs.m, (double)cs.px, (double)cs.py, (double)cs.pz, (double)cs.ke};
#pragma unroll
    for (int k = 0; k < 5; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    __shared__ double sm[kStepBlock / 32][5];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 5; k++) sm[warp][k] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int k = 0; k < 5; k++) {
            double t = lane < nw ? sm[lane][k] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            v[k] = t;
        }
        if (lane == 0) {
            const uint64_t b = blockIdx.x + (uint64_t)gridDim.x * (blockIdx.y + (uint64_t)gridDim.y * blockIdx.z);
#pragma unroll
            for (int k = 0; k < 5; k++) out[b * 5 + k] = v[k];
        }
    }
}

// ---------------------------------------------------------------------------
// moments, limiter and collision shared by the fast and the generic kernels
// ---------------------------------------------------------------------------
template <class R> struct MomentsT {
    R rho, ux, uy, uz, Fx, Fy, Fz;
    R drho;  // shifted storage: rho - 1 as summed from the populations (before the +1), 0.01 - 1 when clamped
    bool out_ext;
};
using Moments = MomentsT<float>;

// s_k = f_i + f_opp, d_k = f_i - f_opp for the pair (i, i+1), i = 2k+1
template <int Q, class R>
__device__ __forceinline__ R pair_sum(const R (&f)[Q], int i) { return FADD(f[i], f[i + 1]); }
template <int Q, class R>
__device__ __forceinline__ R pair_diff(const R (&f)[Q], int i) { return FSUB(f[i], f[i + 1]); }

// compute_density (collide.comp:383-388): the populations in order
template <int Q, class R>
__device__ __forceinline__ R density_lit(const R (&f)[Q]) {
    R rho = f[0];
#pragma unroll
    for (int i = 1; i < Q; i++) rho = FADD(rho, f[i]);
    return rho;
}
// m.rho: unshifted storage compute_density as written; shifted storage
// rho = 1 + (g_0 + s_1 + s_2 + ...) in pairwise order (s_k the opposite
// pairs' sums), the populations held times 2^SCE: rho = fma(sum, 2^-SCE, 1);
// m.drho = the population sum itself, times 2^-SCE.  rho is clamped to
// max(rho, 0.01) with NaN kept; a clamped shifted cell takes drho = 0.01 - 1.
// Flags NaN densities in *err.
template <int Q, bool SH, int SCE, class R>
__device__ __forceinline__ void density_into(const R (&f)[Q], MomentsT<R>& m, uint32_t* err) {
    if constexpr (SH) {
        R sum = f[0];
#pragma unroll
        for (int i = 1; i < Q; i += 2) sum = FADD(sum, pair_sum<Q>(f, i));
        m.rho = SCE ? FFMA(sum, R(1.0 / (double)(1 << SCE)), R(1)) : FADD(R(1), sum);
        m.drho = SCE ? FMUL(sum, R(1.0 / (double)(1 << SCE))) : sum;
    } else {
        m.rho = density_lit<Q>(f);
        m.drho = R(0);
    }
    if (!(m.rho == m.rho)) atomicOr(err, 1u);
    if (m.rho < R(0.01)) {
        m.rho = R(0.01);
        m.drho = FSUB(R(0.01), R(1));
    }
}

// 16-bit multiphase storage, mass-conserving rounding: the mass a cell's
// populations carry after the collision, as stored (times 2^SCE).  The
// relaxation and the source term conserve the population sum in exact
// arithmetic, so T = drho 2^SCE, the cell's own sum (a clamped cell keeps the
// clamped density's, (0.01 - 1) 2^SCE).  Populations 0..Q-2 are stored
// rounded, population Q-1 as the rounding of T less their stored values, so
// the stored populations sum to T up to that one rounding.
template <int SCE, class R>
__device__ __forceinline__ R collided_sum(const MomentsT<R>& m) {
    return SCE ? FMUL(m.drho, R(1 << SCE)) : m.drho;
}

// shifted storage: u = j/rho (+ F/(2 rho)) and the velocity limiter
// (collide.comp:722-725): j from the pair differences, r = 1/rho once,
// u = j r, u = fma(F, r/2, u).
// |u| > limit is tested on |u|^2 against thresholds t = the largest float
// whose IEEE square root does not exceed the limit, which decides exactly as
// sqrt(|u|^2) > limit does; the square root is taken only for limited cells.
// SCE: the populations are held times 2^SCE (scaled shifted storage): the
// momentum takes r * 2^-SCE (exact), the force term r itself.
template <int Q, int SCE = 0>
__device__ __forceinline__ void velocity_and_limit(const float (&f)[Q], Moments& m, bool forced, float vlim,
                                                   float t_lim, float t_ext) {
    using L = Lattice<Q>;
    float jx = 0.f, jy = 0.f, jz = 0.f;
    bool fx = true, fy = true, fz = true;
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        const Dir c = L::c(i);
        const float d = pair_diff<Q>(f, i);
        if (c.x) { const float t = c.x > 0 ? d : -d; jx = fx ? t : FADD(jx, t); fx = false; }
        if (c.y) { const float t = c.y > 0 ? d : -d; jy = fy ? t : FADD(jy, t); fy = false; }
        if (c.z) { const float t = c.z > 0 ? d : -d; jz = fz ? t : FADD(jz, t); fz = false; }
    }
    const float r = __fdiv_rn(1.0f, m.rho);
    const float rj = SCE ? FMUL(r, 1.0f / float(1 << SCE)) : r;
    m.ux = FMUL(jx, rj);
    m.uy = FMUL(jy, rj);
    m.uz = FMUL(jz, rj);
    if (forced) {
        const float h = FMUL(r, 0.5f);
        m.ux = FFMA(m.Fx, h, m.ux);
        m.uy = FFMA(m.Fy, h, m.uy);
        m.uz = FFMA(m.Fz, h, m.uz);
    }
    const float uu = uu_of(m.ux, m.uy, m.uz);
    m.out_ext = uu > t_ext;
    if (uu > t_lim) {  // normalize(u) * limit
        const float q = __fdiv_rn(vlim, sqrtf(uu));
        m.ux = FMUL(m.ux, q);
        m.uy = FMUL(m.uy, q);
        m.uz = FMUL(m.uz, q);
    }
}

// compute_velocity (collide.comp:390-395) and the limiter (:722-725) as
// written: j = the populations times their lattice vectors summed in order,
// u = j/rho, + F/(2 rho) (each a correctly rounded division); |u| > limit
// decided on the literal u.u (float: against the square-root thresholds,
// which decides exactly as sqrt(u.u) > limit; double: on the square root);
// a limited u becomes (u/|u|) * limit.  Forced: the force term is compiled in
// (adding F/(2 rho) = +0 would change nothing but the sign of a zero).  ZF:
// zero force components skip their division (bit for bit the same; kernels
// whose forces are rarely exactly zero, Shan-Chen's, leave the test out).
template <int Q, bool ZF = true, class R>
__device__ __forceinline__ void velocity_literal(const R (&f)[Q], MomentsT<R>& m, bool forced, R vlim, R t_lim,
                                                 R t_ext) {
    using L = Lattice<Q>;
    R jx = R(0), jy = R(0), jz = R(0);
    bool fx = true, fy = true, fz = true;
#pragma unroll
    for (int i = 1; i < Q; i++) {
        const Dir c = L::c(i);
        const R d = f[i];
        if (c.x) { const R t = c.x > 0 ? d : -d; jx = fx ? t : FADD(jx, t); fx = false; }
        if (c.y) { const R t = c.y > 0 ? d : -d; jy = fy ? t : FADD(jy, t); fy = false; }
        if (c.z) { const R t = c.z > 0 ? d : -d; jz = fz ? t : FADD(jz, t); fz = false; }
    }
    m.ux = FDIV(jx, m.rho);
    m.uy = FDIV(jy, m.rho);
    m.uz = FDIV(jz, m.rho);
    if (forced) {
        // d2 >= 0.02 (the clamped density) or NaN: a zero force component's
        // quotient is that signed zero, so it is added without the division,
        // whose slow path takes zero dividends (a force along one axis leaves
        // two components zero in every cell); with d2 NaN, u is NaN already
        const R d2 = FMUL(R(2), m.rho);
        auto half_f = [&](R F) -> R { return (ZF && F == R(0)) ? F : FDIV(F, d2); };
        m.ux = FADD(m.ux, half_f(m.Fx));
        m.uy = FADD(m.uy, half_f(m.Fy));
        m.uz = FADD(m.uz, half_f(m.Fz));
    }
    const R uu = dot_lit(m.ux, m.uy, m.uz, m.ux, m.uy, m.uz);
    bool lim;
    R len = R(0);
    if constexpr (sizeof(R) == 4) {
        m.out_ext = uu > t_ext;
        lim = uu > t_lim;
        if (lim) len = sqrtf(uu);
    } else {
        len = __dsqrt_rn(uu);
        m.out_ext = len > t_ext;
        lim = len > vlim;
    }
    if (lim) {
        m.ux = FMUL(FDIV(m.ux, len), vlim);
        m.uy = FMUL(FDIV(m.uy, len), vlim);
        m.uz = FMUL(FDIV(m.uz, len), vlim);
    }
}

// Post-collision populations, handed to emit(i, value) as soon as each is
// known.  BGK with unshifted storage is collide.comp:589-629/727-745 as
// written (feq_lit, f + (-(f - feq)/tau) + (P w)(F.c/cs2 + ((F.c)(u.c)/cs4 -
// F.u/cs2))); with shifted storage (SH) the fixed order
//   feq = (w rho) bracket(cu),  f <- fma(feq - f, 1/tau, f)
//   + fma(P w, fma(F.c, R2, fma((F.c) cu, R4, -(F.u) R2)), .)   [Guo]
// TRT is an extension, evaluated over the pair (i, opp i):
//   e+ = (w rho) fma(cu^2, R4/2, 1 - uu R2/2),  e- = (w rho R2) cu
//   P = fma(f_i + f_opp, 1/2, -e+),  M = fma(f_i - f_opp, 1/2, -e-)
//   f_i <- fma(-M, omega-, fma(-P, omega+, f_i)),  f_opp <- fma(M, omega-, fma(-P, omega+, f_opp))
// with the Guo term split into its even part (1-omega+/2) w ((F.c)(u.c)/cs4 - F.u/cs2)
// and odd part (1-omega-/2) w F.c/cs2.  Above the extreme velocity limit the
// populations become the equilibrium (BGK: feq, TRT: e+ +- e-).
// SH (shifted storage): f holds g = f - w and every equilibrium is formed
// as g_eq = fma(w rho, bracket, -w); the rest of the update is unchanged.
// launch constants of the collision in the arithmetic type
template <class R> struct Coef {
    R R2, R4, R2h, R4h, Rtau, P, Wm, Pp, Pm;
    Div<R> d;
    R tau;
    bool ok_tau;
    R ltau;  // low part of 1/tau (div_m)
};
__device__ __forceinline__ Coef<float> coef_of(const StepParams& p, float) {
    return Coef<float>{p.R2, p.R4, p.R2h, p.R4h, p.Rtau, p.P, p.Wm, p.Pp, p.Pm,
                       Div<float>{p.cs2, p.R2, p.L2, p.cs4, p.R4, p.L4, (p.div_ok & 1u) != 0, (p.div_ok & 2u) != 0},
                       p.tau, (p.div_ok & 4u) != 0, p.Ltau};
}
__device__ __forceinline__ Coef<double> coef_of(const StepParams& p, double) {
    return Coef<double>{p.k64.R2, p.k64.R4, p.k64.R2h, p.k64.R4h, p.k64.Rtau, p.k64.P, p.k64.Wm, p.k64.Pp,
                        p.k64.Pm, Div<double>{p.k64.cs2, p.k64.R2, 0.0, p.k64.cs4, p.k64.R4, 0.0, false, false},
                        p.k64.tau, false, 0.0};
}

// Shifted storage with a source term (Guo forcing, Shan-Chen, buoyancy): the
// relaxation and the source folded into one polynomial per opposite pair.
// With delta = rho - 1 (the population sum), omega+ = 1/tau and omega- (TRT;
// BGK: both 1/tau), P+- = 1 - omega+-/2:
//   A = fma(omega+, delta, -fma(omega+ rho, u.u R2/2, P+ (F.u) R2))
//   V = R4 fma(omega+ rho / 2, u, P+ F)       (even part, times c.u)
//   U = R2 fma(omega- rho, u, P- F)           (odd part)
//   g_0 <- fma(w_0, A, (1 - omega+) g_0)
//   E = fma(c.u, c.V, A)
//   BGK: g_i   <- fma(w, E + c.U, (1 - omega) g_i),  g_opp <- fma(w, E - c.U, (1 - omega) g_opp)
//   TRT: g_i   <- fma(w, E + c.U, fma(a, g_i, b g_opp)),  g_opp <- fma(w, E - c.U, fma(a, g_opp, b g_i))
//        a = 1 - (omega+ + omega-)/2,  b = (omega- - omega+)/2
// which is, term by term, g + omega+-(g_eq - g) + P+- w S+- of the update on
// g = f - w (g_eq = w rho bracket - w) with the omega+ rho - omega+ of the
// equilibrium taken as omega+ delta.  SCE: weights times 2^SCE (the
// populations are held times 2^SCE; delta is unscaled).  Above the extreme
// velocity limit the populations become the equilibrium: the same tree with
// omega+- = 1 and P+- = 0.
template <int Q, bool TRT, int SCE, class R, class Emit>
__device__ __forceinline__ void shifted_source_collide(const R (&f)[Q], const MomentsT<R>& m, const Coef<R>& k,
                                                       Emit emit) {
    using L = Lattice<Q>;
    struct W {
        __device__ __forceinline__ static constexpr R w(int i) { return LatticeW<Q, R>::w(i) * R(1 << SCE); }
    };
    const bool ext = m.out_ext;
    const R op = ext ? R(1) : k.Rtau;
    const R om = ext ? R(1) : (TRT ? k.Wm : k.Rtau);
    const R pp = ext ? R(0) : (TRT ? k.Pp : k.P);
    const R pm = ext ? R(0) : (TRT ? k.Pm : k.P);
    const R fuR2 = FMUL(FFMA(m.Fz, m.uz, FFMA(m.Fy, m.uy, FMUL(m.Fx, m.ux))), k.R2);
    const R wp = FMUL(op, m.rho), wm = FMUL(om, m.rho);
    const R A = FFMA(op, m.drho, -FFMA(wp, FMUL(uu_of(m.ux, m.uy, m.uz), k.R2h), FMUL(pp, fuR2)));
    const R wph = FMUL(wp, R(0.5));
    const R Vx = FMUL(FFMA(wph, m.ux, FMUL(pp, m.Fx)), k.R4);
    const R Vy = FMUL(FFMA(wph, m.uy, FMUL(pp, m.Fy)), k.R4);
    const R Vz = FMUL(FFMA(wph, m.uz, FMUL(pp, m.Fz)), k.R4);
    const R Ux = FMUL(FFMA(wm, m.ux, FMUL(pm, m.Fx)), k.R2);
    const R Uy = FMUL(FFMA(wm, m.uy, FMUL(pm, m.Fy)), k.R2);
    const R Uz = FMUL(FFMA(wm, m.uz, FMUL(pm, m.Fz)), k.R2);
    const R keep = FSUB(R(1), op);
    emit(0, FFMA(W::w(0), A, FMUL(keep, f[0])));
    const R a = TRT ? FSUB(R(1), FMUL(FADD(op, om), R(0.5))) : keep;
    const R b = TRT ? FMUL(FSUB(om, op), R(0.5)) : R(0);
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        const int j = i + 1;
        const Dir c = L::c(i);
        const R w = W::w(i);
        const R E = FFMA(cdot_rt(c, m.ux, m.uy, m.uz), cdot_rt(c, Vx, Vy, Vz), A);
        const R cU = cdot_rt(c, Ux, Uy, Uz);
        const R bi = TRT ? FFMA(a, f[i], FMUL(b, f[j])) : FMUL(a, f[i]);
        const R bj = TRT ? FFMA(a, f[j], FMUL(b, f[i])) : FMUL(a, f[j]);
        emit(i, FFMA(w, FADD(E, cU), bi));
        emit(j, FFMA(w, FSUB(E, cU), bj));
    }
}

template <int Q, bool SH, class R, class Emit>
__device__ __forceinline__ void collide_emit(const R (&f)[Q], const MomentsT<R>& m, const Coef<R>& k, bool trt,
                                             bool src, bool to_equilibrium, Emit emit) {
    using L = Lattice<Q>;
    using W = LatticeW<Q, R>;
    if constexpr (SH) {
        if (src && !to_equilibrium) {
            if (trt) shifted_source_collide<Q, true, 0>(f, m, k, emit);
            else shifted_source_collide<Q, false, 0>(f, m, k, emit);
            return;
        }
    }
    if (!SH && (to_equilibrium || !trt)) {
        // collide.comp:727-745 with :589-629 as written: f + (-(f - feq)/tau) + source
        const Div<R>& d = k.d;
        const R uuh = uuh_of<false>(m.ux, m.uy, m.uz, d);
        const R fuc = src ? div_u(dot_lit(m.Fx, m.Fy, m.Fz, m.ux, m.uy, m.uz), d.cs2, d.rcs2, d.lcs2, d.ok2) : R(0);
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const Dir c = L::c(i);
            const R w = W::w(i);
            const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
            const R fe = feq_lit<false>(FMUL(w, m.rho), cu, d, uuh);
            R v = FSUB(f[i], div_u(FSUB(f[i], fe), k.tau, k.Rtau, k.ltau, k.ok_tau));
            if (src) {
                const R fc = cdot_rt(c, m.Fx, m.Fy, m.Fz);
                v = FADD(v, FMUL(FMUL(k.P, w), FADD(div_u(fc, d.cs2, d.rcs2, d.lcs2, d.ok2),
                                                    FSUB(div_u(FMUL(fc, cu), d.cs4, d.rcs4, d.lcs4, d.ok4), fuc))));
            }
            emit(i, (to_equilibrium || m.out_ext) ? fe : v);
        }
        return;
    }
    const R one_m = FSUB(R(1), FMUL(uu_of(m.ux, m.uy, m.uz), k.R2h));
    const R fuR2 = FMUL(FFMA(m.Fz, m.uz, FFMA(m.Fy, m.uy, FMUL(m.Fx, m.ux))), k.R2);
    if (to_equilibrium || !trt) {
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const Dir c = L::c(i);
            const R w = W::w(i);
            const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
            const R br = bracket(cu, one_m, k.R2, k.R4h);
            const R fe = SH ? FFMA(FMUL(w, m.rho), br, -w) : FMUL(FMUL(w, m.rho), br);
            R v = FFMA(FSUB(fe, f[i]), k.Rtau, f[i]);  // old + (-(old - feq)/tau)
            if (src) {
                const R fc = cdot_rt(c, m.Fx, m.Fy, m.Fz);
                v = FFMA(FMUL(k.P, w), FFMA(fc, k.R2, FFMA(FMUL(fc, cu), k.R4, -fuR2)), v);
            }
            emit(i, (to_equilibrium || m.out_ext) ? fe : v);
        }
        return;
    }
    {
        const R w0 = W::w(0);
        const R fe0 = SH ? FFMA(FMUL(w0, m.rho), one_m, -w0) : FMUL(FMUL(w0, m.rho), one_m);
        R v = FFMA(FSUB(fe0, f[0]), k.Rtau, f[0]);
        if (src) v = FFMA(FMUL(k.Pp, w0), -fuR2, v);
        emit(0, m.out_ext ? fe0 : v);
    }
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        const int j = i + 1;
        const Dir c = L::c(i);
        const R w = W::w(i);
        const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
        const R wr = FMUL(w, m.rho);
        const R be = FFMA(FMUL(cu, cu), k.R4h, one_m);
        const R ep = SH ? FFMA(wr, be, -w) : FMUL(wr, be);
        const R em = FMUL(FMUL(wr, k.R2), cu);
        const R Pd = FFMA(pair_sum<Q>(f, i), R(0.5), -ep);
        const R Md = FFMA(pair_diff<Q>(f, i), R(0.5), -em);
        R vi = FFMA(-Md, k.Wm, FFMA(-Pd, k.Rtau, f[i]));
        R vj = FFMA(Md, k.Wm, FFMA(-Pd, k.Rtau, f[j]));
        if (src) {
            const R fc = cdot_rt(c, m.Fx, m.Fy, m.Fz);
            const R Sp = FMUL(FMUL(k.Pp, w), FFMA(FMUL(fc, cu), k.R4, -fuR2));
            const R Sm = FMUL(FMUL(k.Pm, w), FMUL(fc, k.R2));
            vi = FADD(vi, FADD(Sp, Sm));
            vj = FADD(vj, FSUB(Sp, Sm));
        }
        emit(i, m.out_ext ? FADD(ep, em) : vi);
        emit(j, m.out_ext ? FSUB(ep, em) : vj);
    }
}

// The same arithmetic as collide_emit with the collision model, the source
// term and the extreme-velocity case fixed at compile time (the fast kernel
// branches once per cell on the rare extreme case instead of selecting per
// population); R = float is the FP32 evaluation, R = double the FP64
// reference stepper (the literal tree in double).
// SCE (shifted storage only): f holds G = g * 2^SCE and every weight of the
// shifted arithmetic is taken times 2^SCE, so that the emitted values are the
// g update's times 2^SCE exactly.
template <int Q, bool TRT, bool SRC, bool EXT, bool SH, int SCE = 0, class R, class Emit>
__device__ __forceinline__ void collide_fixed(const R (&f)[Q], const MomentsT<R>& m, const Coef<R>& k, Emit emit) {
    using L = Lattice<Q>;
    struct W {
        __device__ __forceinline__ static constexpr R w(int i) { return LatticeW<Q, R>::w(i) * R(1 << SCE); }
    };
    static_assert(SH || SCE == 0, "scaled populations are shifted");
    if constexpr (SH && SRC) {  // the extreme case is taken inside, from m.out_ext
        shifted_source_collide<Q, TRT, SCE>(f, m, k, emit);
        return;
    }
    if (!SH && !TRT) {
        // collide.comp:727-745 with :589-629 as written: f + (-(f - feq)/tau) + source
        const Div<R>& d = k.d;
        const R uuh = uuh_of<true>(m.ux, m.uy, m.uz, d);
        const R fuc = SRC ? div_m(dot_lit(m.Fx, m.Fy, m.Fz, m.ux, m.uy, m.uz), d.cs2, d.rcs2, d.lcs2) : R(0);
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const Dir c = L::c(i);
            const R w = W::w(i);
            const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
            const R fe = feq_lit<true>(FMUL(w, m.rho), cu, d, uuh);
            if (EXT) { emit(i, fe); continue; }
            R v = FSUB(f[i], div_m(FSUB(f[i], fe), k.tau, k.Rtau, k.ltau));
            if (SRC) {
                const R fc = cdot_rt(c, m.Fx, m.Fy, m.Fz);
                v = FADD(v, FMUL(FMUL(k.P, w), FADD(div_m(fc, d.cs2, d.rcs2, d.lcs2),
                                                    FSUB(div_m(FMUL(fc, cu), d.cs4, d.rcs4, d.lcs4), fuc))));
            }
            emit(i, v);
        }
        return;
    }
    const R one_m = FSUB(R(1), FMUL(uu_of(m.ux, m.uy, m.uz), k.R2h));
    const R fuR2 = SRC ? FMUL(FFMA(m.Fz, m.uz, FFMA(m.Fy, m.uy, FMUL(m.Fx, m.ux))), k.R2) : R(0);
    if (!TRT) {
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const Dir c = L::c(i);
            const R w = W::w(i);
            const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
            const R br = bracket(cu, one_m, k.R2, k.R4h);
            const R fe = SH ? FFMA(FMUL(w, m.rho), br, -w) : FMUL(FMUL(w, m.rho), br);
            if (EXT) { emit(i, fe); continue; }
            R v = FFMA(FSUB(fe, f[i]), k.Rtau, f[i]);
            if (SRC) {
                const R fc = cdot_rt(c, m.Fx, m.Fy, m.Fz);
                v = FFMA(FMUL(k.P, w), FFMA(fc, k.R2, FFMA(FMUL(fc, cu), k.R4, -fuR2)), v);
            }
            emit(i, v);
        }
        return;
    }
    {
        const R w0 = W::w(0);
        const R fe0 = SH ? FFMA(FMUL(w0, m.rho), one_m, -w0) : FMUL(FMUL(w0, m.rho), one_m);
        if (EXT) {
            emit(0, fe0);
        } else {
            R v = FFMA(FSUB(fe0, f[0]), k.Rtau, f[0]);
            if (SRC) v = FFMA(FMUL(k.Pp, w0), -fuR2, v);
            emit(0, v);
        }
    }
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        const int j = i + 1;
        const Dir c = L::c(i);
        const R w = W::w(i);
        const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
        const R wr = FMUL(w, m.rho);
        const R be = FFMA(FMUL(cu, cu), k.R4h, one_m);
        const R ep = SH ? FFMA(wr, be, -w) : FMUL(wr, be);
        const R em = FMUL(FMUL(wr, k.R2), cu);
        if (EXT) {
            emit(i, FADD(ep, em));
            emit(j, FSUB(ep, em));
            continue;
        }
        const R Pd = FFMA(pair_sum<Q>(f, i), R(0.5), -ep);
        const R Md = FFMA(pair_diff<Q>(f, i), R(0.5), -em);
        R vi = FFMA(-Md, k.Wm, FFMA(-Pd, k.Rtau, f[i]));
        R vj = FFMA(Md, k.Wm, FFMA(-Pd, k.Rtau, f[j]));
        if (SRC) {
            const R fc = cdot_rt(c, m.Fx, m.Fy, m.Fz);
            const R Sp = FMUL(FMUL(k.Pp, w), FFMA(FMUL(fc, cu), k.R4, -fuR2));
            const R Sm = FMUL(FMUL(k.Pm, w), FMUL(fc, k.R2));
            vi = FADD(vi, FADD(Sp, Sm));
            vj = FADD(vj, FSUB(Sp, Sm));
        }
        emit(i, vi);
        emit(j, vj);
    }
}

struct NoHook {
    __device__ __forceinline__ void operator()() const {}
};

// L2 prefetch of a byte range with the bulk-copy engine (no registers held,
// no completion to wait for).  The range must be 16-byte aligned and sized.
__device__ __forceinline__ void l2_prefetch_bulk(const void* ptr, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(ptr), "r"(bytes) : "memory");
}

// c_y + 1 (axis 1) or c_z + 1 (axis 2) of every direction, two bits each
template <int Q>
__host__ __device__ constexpr uint64_t packed_axis(int axis) {
    uint64_t k = 0;
    for (int i = 0; i < Q; i++) {
        const Dir c = Lattice<Q>::c(i);
        k |= (uint64_t)((axis == 1 ? c.y : c.z) + 1) << (2 * i);
    }
    return k;
}

// Prefetch into L2 the population rows that block `b` (linear launch order,
// x fastest) reads, one plane per lane of the calling warp (lanes >= Q do
// nothing): on an even step lane i takes row (y - c_y, z - c_z) of plane i
// over the block's x range widened by 8 cells each side (the c_x shift), on
// an odd step row (y, z) of plane i.  `tile` is the block's width in cells.
// Ranges are clipped to the row and rounded out to 16 bytes; that stays
// inside the plane because planes start and end on 16-byte boundaries
// whenever pf_blocks is set.  Planes lie `stride` elements apart.
template <int Q, int ST, int MODE>
__device__ __forceinline__ void prefetch_rows_at(const StepParams& p, uint32_t bx, int ys, int zs, int lane, int tile) {
    using T = typename Codec<ST>::T;
    if (lane >= Q) return;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int x0 = (int)bx * tile;
    const int xlo = MODE == AA_EVEN ? max(x0 - 8, 0) : x0;
    const int xhi = min(x0 + tile + (MODE == AA_EVEN ? 8 : 0), nx);
    if (MODE == AA_EVEN) {
        constexpr uint64_t ky = packed_axis<Q>(1), kz = packed_axis<Q>(2);
        ys -= (int)((ky >> (2 * lane)) & 3u) - 1;
        zs -= (int)((kz >> (2 * lane)) & 3u) - 1;
        ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
        zs = zs < 0 ? zs + nz : (zs >= nz ? zs - nz : zs);
    }
    const uintptr_t plane_bytes = (uintptr_t)p.n_cells * sizeof(T);
    const uintptr_t base = reinterpret_cast<uintptr_t>(p.plane[0]) + (uintptr_t)lane * (uintptr_t)p.stride * sizeof(T);
    const uintptr_t row = (uintptr_t)nx * ((uintptr_t)ys + (uintptr_t)ny * (uintptr_t)zs);
    const uintptr_t lo = (base + (row + (uintptr_t)xlo) * sizeof(T)) & ~(uintptr_t)15;
    uintptr_t hi = (base + (row + (uintptr_t)xhi) * sizeof(T) + 15) & ~(uintptr_t)15;
    hi = min(hi, base + plane_bytes);
    if (hi > lo) l2_prefetch_bulk(reinterpret_cast<const void*>(lo), (uint32_t)(hi - lo));
}
// the same for block b of a launch in linear order over a gx x gy x . grid
template <int Q, int ST, int MODE>
__device__ __forceinline__ void prefetch_block_rows(const StepParams& p, uint32_t b, int lane, int tile,
                                                    uint32_t gx = gridDim.x, uint32_t gy = gridDim.y) {
    if (lane >= Q) return;
    const uint32_t bx = b % gx, yz = b / gx;
    prefetch_rows_at<Q, ST, MODE>(p, bx, (int)(yz % gy), (int)(yz / gy), lane, tile);
}

// Thermal flow: lanes Q .. Q + QT - 1 of the calling warp prefetch into L2
// thermal plane (lane - Q) over row yz of x-block bx (the cell's own row: the
// thermal populations are read at the cell and pushed at the write), with
// the flow planes' alignment rule (thermal planes are FP32 and share their
// plane stride, so they start and end on 16-byte boundaries too).
template <int Q>
__device__ __forceinline__ void prefetch_thermal_rows_at(const StepParams& p, uint32_t bx, uint32_t yz, int lane,
                                                         int tile) {
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    const int k = lane - Q;
    if (k < 0 || k >= QT) return;
    const int x0 = (int)bx * tile;
    const int xhi = min(x0 + tile, p.nx);
    const uintptr_t plane_bytes = (uintptr_t)p.n_cells * sizeof(float);
    const uintptr_t base = reinterpret_cast<uintptr_t>(p.th_src) + (uintptr_t)k * (uintptr_t)p.stride * sizeof(float);
    const uintptr_t row = (uintptr_t)p.nx * (uintptr_t)yz;
    const uintptr_t lo = (base + (row + (uintptr_t)x0) * sizeof(float)) & ~(uintptr_t)15;
    uintptr_t hi = (base + (row + (uintptr_t)xhi) * sizeof(float) + 15) & ~(uintptr_t)15;
    hi = min(hi, base + plane_bytes);
    if (hi > lo) l2_prefetch_bulk(reinterpret_cast<const void*>(lo), (uint32_t)(hi - lo));
}

// ---------------------------------------------------------------------------
// fast AA step: fully periodic box, no objects, no thermal / Shan-Chen /
// force field (constant force allowed; TRT and forcing fixed per launch).
// Slots are addressed by byte offsets off the first plane.  The first warp of
// each block prefetches into L2 the rows of the block pf_blocks ahead in
// launch order (one plane per lane), so that the block's own loads mostly
// hit L2 and 16-bit storage needs fewer loads in flight to saturate HBM.
// ---------------------------------------------------------------------------
#ifndef BF_FAST_MIN_BLOCKS
#define BF_FAST_MIN_BLOCKS 4
#endif
#ifndef BF_FAST_MIN_BLOCKS_16
#define BF_FAST_MIN_BLOCKS_16 5
#endif
// resident blocks per SM the fast kernel is compiled for: 256 threads x 4
// blocks allow at most 64 registers (FP32 storage); the 16-bit storages,
// which are issue-bound rather than bandwidth-bound, fit 48 registers and 5
// blocks up to D3Q19 (measured faster at 512^3; D3Q27 would spill); FP64:
// 2 blocks, 128 registers
constexpr int kFastMinBlocks = BF_FAST_MIN_BLOCKS;
constexpr int kFastMinBlocks16 = BF_FAST_MIN_BLOCKS_16;

// One cell of the fast step.  EDGE: the block's row lies on a y or z face of
// the box, so the y/z neighbour offsets wrap and are computed in the block;
// otherwise they are the launch constants p.uoff (plane offset minus
// c_y nx + c_z nx ny), one constant-bank operand per index.
// load(i, ptr_of) returns the stored element of direction i; ptr_of(k) is
// the address of the slot read for direction k (the plain kernel loads
// *ptr_of(i), the staged kernel reads shared memory and never calls it)
// Shan-Chen pseudopotential force (collide.comp:534-584): psi of the
// previous step at the periodic neighbours x + c_i (offsets ox*/oy*/oz* from
// cell n to x -+ 1, y -+ 1, z -+ 1), summed, times -G psi(rho) of the cell;
// returns psi(rho), which is also this step's psi field value of the cell.
// nb(c) returns psi at x + c.
// Sums (sc_sums_t): unshifted storage as written, w_i psi_i c_i in
// direction order; shifted storage (GROUPED, an extension) over opposite
// pairs, d_k = psi(c_i) - psi(-c_i) for i = 2k + 1, then per component the
// signed d_k of each weight class summed in pair order and the classes
// combined as fma(w, class sum, .) in class order -- the same sum in about
// half the operations.
template <int Q, bool GROUPED, class R, class NB>
__device__ __forceinline__ void sc_sums_t(NB nb, R& sx, R& sy, R& sz) {
    using L = Lattice<Q>;
    using W = LatticeW<Q, R>;
    if constexpr (!GROUPED) {
        sx = R(0); sy = R(0); sz = R(0);
#pragma unroll
        for (int i = 1; i < Q; i++) {
            const Dir c = L::c(i);
            const R wp = FMUL(W::w(i), nb(c));
            if (c.x) sx = FADD(sx, c.x > 0 ? wp : -wp);
            if (c.y) sy = FADD(sy, c.y > 0 ? wp : -wp);
            if (c.z) sz = FADD(sz, c.z > 0 ? wp : -wp);
        }
    } else {
        R d[Q / 2];
#pragma unroll
        for (int k = 0; k < Q / 2; k++) d[k] = FSUB(nb(L::c(2 * k + 1)), nb(L::c(2 * k + 2)));
        R out[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            R acc = R(0), cls = R(0), wc = R(0);
            bool have = false, open = false;
#pragma unroll
            for (int k = 0; k < Q / 2; k++) {
                const int i = 2 * k + 1;
                if (open && W::w(i) != wc) {  // the class ends: fold its sum in
                    acc = have ? FFMA(wc, cls, acc) : FMUL(wc, cls);
                    have = true;
                    open = false;
                }
                const Dir c = L::c(i);
                const int comp = a == 0 ? c.x : (a == 1 ? c.y : c.z);
                if (comp == 0) continue;
                const R t = comp > 0 ? d[k] : -d[k];
                cls = open ? FADD(cls, t) : t;
                wc = W::w(i);
                open = true;
            }
            if (open) {
                acc = have ? FFMA(wc, cls, acc) : FMUL(wc, cls);
                have = true;
            }
            out[a] = have ? acc : R(0);
        }
        sx = out[0]; sy = out[1]; sz = out[2];
    }
}
struct ScSum { float x, y, z; };
template <int Q, bool GROUPED, class NB>
__device__ __forceinline__ ScSum sc_sums(NB nb) {
    ScSum s;
    sc_sums_t<Q, GROUPED, float>(nb, s.x, s.y, s.z);
    return s;
}
// interaction_force *= -self_psi * G; force += interaction_force (:580-583, :718-720)
__device__ __forceinline__ float sc_apply(float G, Moments& m, const ScSum& s) {
    const float self_psi = FSUB(1.0f, exp_f32(-m.rho));
    const float k = FMUL(-self_psi, G);
    m.Fx = FADD(m.Fx, FMUL(s.x, k)); m.Fy = FADD(m.Fy, FMUL(s.y, k)); m.Fz = FADD(m.Fz, FMUL(s.z, k));
    return self_psi;
}
template <int Q, bool GROUPED, class NB>
__device__ __forceinline__ float sc_force_nb(float G, Moments& m, NB nb) {
    return sc_apply(G, m, sc_sums<Q, GROUPED>(nb));
}
template <int Q, bool GROUPED>
__device__ __forceinline__ float sc_force(const StepParams& p, uint32_t n, int oxm, int oxp, int oym, int oyp, int ozm,
                                          int ozp, Moments& m) {
    return sc_force_nb<Q, GROUPED>(p.G, m, [&](const Dir c) {
        const uint32_t a = n + (uint32_t)((c.x > 0 ? oxp : (c.x < 0 ? oxm : 0)) + (c.y > 0 ? oyp : (c.y < 0 ? oym : 0)) +
                                          (c.z > 0 ? ozp : (c.z < 0 ? ozm : 0)));
        return __ldg(p.psi_src + a);
    });
}
// psi of a cell pair's stencil (cells x and x + 1, x even, nx even): the
// row (y + dy, z + dz) of a direction with c = (., dy, dz) at x - 1, x, x + 1
// and x + 2 (slots 0..3), x and x + 1 as one aligned float2, x - 1 and x + 2
// (periodic) only where some direction of the row has c_x = -1 / +1.  Both
// cells' forces then read registers: D3Q19 takes 19 loads per pair instead
// of 36, the sums unchanged.
template <int Q>
__host__ __device__ constexpr int psi_row(Dir c) {
    return Lattice<Q>::D == 2 ? c.y + 1 : (c.y + 1) * 3 + (c.z + 1);
}
template <int Q>
__host__ __device__ constexpr uint32_t psi_row_xs(int r) {  // bit c_x + 1 for each direction i >= 1 of row r
    uint32_t m = 0;
    for (int i = 1; i < Q; i++)
        if (psi_row<Q>(Lattice<Q>::c(i)) == r) m |= 1u << (Lattice<Q>::c(i).x + 1);
    return m;
}
template <int Q> constexpr int kPsiRows = Lattice<Q>::D == 2 ? 3 : 9;
template <int Q>
__device__ __forceinline__ void psi_pair_load(const float* __restrict__ ps, uint32_t n, int x, int nx, int oym,
                                              int oyp, int ozm, int ozp, float (&pv)[kPsiRows<Q>][4]) {
    const int oxm = x == 0 ? nx - 1 : -1;          // x - 1 from x
    const int oxq = x + 2 == nx ? 2 - nx : 2;      // x + 2 from x
#pragma unroll
    for (int r = 0; r < kPsiRows<Q>; r++) {
        constexpr int D = Lattice<Q>::D;
        const uint32_t xs = psi_row_xs<Q>(r);
        if (xs == 0u) continue;
        const int dy = D == 2 ? r - 1 : r / 3 - 1, dz = D == 2 ? 0 : r % 3 - 1;
        const uint32_t rb = n + (uint32_t)((dy > 0 ? oyp : (dy < 0 ? oym : 0)) + (dz > 0 ? ozp : (dz < 0 ? ozm : 0)));
        const float2 mid = __ldg(reinterpret_cast<const float2*>(ps + rb));
        pv[r][1] = mid.x;
        pv[r][2] = mid.y;
        // element indices wrap in 32 bits before they meet the pointer
        if (xs & 1u) pv[r][0] = __ldg(ps + (rb + (uint32_t)oxm));
        if (xs & 4u) pv[r][3] = __ldg(ps + (rb + (uint32_t)oxq));
    }
}

// The same stencil from a shared-memory tile of whole rows: row r (as
// psi_row) of nx floats at tile + r * nx, the x wrap inside the row.
template <int Q>
__device__ __forceinline__ void psi_pair_load_tile(const float* tile, int x, int nx, float (&pv)[kPsiRows<Q>][4]) {
    const int xm = x == 0 ? nx - 1 : x - 1, xq = x + 2 == nx ? 0 : x + 2;
#pragma unroll
    for (int r = 0; r < kPsiRows<Q>; r++) {
        const uint32_t xs = psi_row_xs<Q>(r);
        if (xs == 0u) continue;
        const float* row = tile + r * nx;
        const float2 mid = *reinterpret_cast<const float2*>(row + x);
        pv[r][1] = mid.x;
        pv[r][2] = mid.y;
        if (xs & 1u) pv[r][0] = row[xm];
        if (xs & 4u) pv[r][3] = row[xq];
    }
}

// Boussinesq buoyancy of the thermal lattice (collide.comp:709-716): the
// temperature T = sum of the cell's thermal populations scales the force by
// 1 - beta (T - 1); returns T
template <int Q>
__device__ __forceinline__ float thermal_buoyancy_of(const float (&th)[Lattice<Q>::D == 2 ? 5 : 7], float beta, Moments& m) {
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    float temperature = 0.f;
#pragma unroll
    for (int i = 0; i < QT; i++) temperature = FADD(temperature, th[i]);
    // buoyancy = -beta (T - 1) force; force += buoyancy
    const float k = FMUL(-beta, FSUB(temperature, 1.0f));
    m.Fx = FADD(m.Fx, FMUL(k, m.Fx)); m.Fy = FADD(m.Fy, FMUL(k, m.Fy)); m.Fz = FADD(m.Fz, FMUL(k, m.Fz));
    return temperature;
}

// the same with the cell's thermal populations loaded here (special cells)
template <int Q>
__device__ __forceinline__ float thermal_buoyancy(const StepParams& p, uint32_t n, Moments& m) {
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    float th[QT];
#pragma unroll
    for (int i = 0; i < QT; i++) th[i] = __ldg(p.th_src + (uint64_t)i * p.stride + n);
    return thermal_buoyancy_of<Q>(th, p.beta, m);
}

// thermal BGK towards g_eq(T, u) as written (collide.comp:771-782, :634-651,
// :668-670): g + (-(g - g_eq)/tau_T)
__device__ __forceinline__ float thermal_relax(const StepParams& p, float g, float geq) {
    return FSUB(g, div_m(FSUB(g, geq), p.tau_t, p.Rtau_t, p.Ltau_t));
}
__device__ __forceinline__ Div<float> div_of(const StepParams& p) {
    return Div<float>{p.cs2, p.R2, p.L2, p.cs4, p.R4, p.L4, (p.div_ok & 1u) != 0, (p.div_ok & 2u) != 0};
}
template <int Q>
__device__ __forceinline__ void thermal_collide(const StepParams& p, uint32_t n, const Moments& m, float temperature) {
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    const Div<float> d = div_of(p);
    const float uuh = uuh_of<true>(m.ux, m.uy, m.uz, d);
#pragma unroll
    for (int i = 0; i < QT; i++) {
        const Dir c = ThermalLattice<QT>::c(i);
        const float w = ThermalLattice<QT>::w(i);
        const float cu = cdot_rt(c, m.ux, m.uy, m.uz);
        const float geq = feq_lit<true>(FMUL(w, temperature), cu, d, uuh);
        const float g = __ldg(p.th_src + (uint64_t)i * p.stride + n);
        p.th_tgt[(uint64_t)i * p.stride + n] = thermal_relax(p, g, geq);
    }
}

// the generic step's thermal lattice, pseudopotential and launch constants
// in the arithmetic type R (float: the FP32 buffers; double: the FP64
// stepper's)
__device__ __forceinline__ const float* th_src_of(const StepParams& p, float) { return p.th_src; }
__device__ __forceinline__ float* th_tgt_of(const StepParams& p, float) { return p.th_tgt; }
__device__ __forceinline__ const float* psi_src_of(const StepParams& p, float) { return p.psi_src; }
__device__ __forceinline__ float* psi_tgt_of(const StepParams& p, float) { return p.psi_tgt; }
__device__ __forceinline__ const double* th_src_of(const StepParams& p, double) { return p.th_src64; }
__device__ __forceinline__ double* th_tgt_of(const StepParams& p, double) { return p.th_tgt64; }
__device__ __forceinline__ const double* psi_src_of(const StepParams& p, double) { return p.psi_src64; }
__device__ __forceinline__ double* psi_tgt_of(const StepParams& p, double) { return p.psi_tgt64; }
template <class R> struct Knobs { R tau_t, beta, G, vlim, t_lim, t_ext, fx, fy, fz; };
__device__ __forceinline__ Knobs<float> knobs_of(const StepParams& p, float) {
    return Knobs<float>{p.tau_t, p.beta, p.G, p.vlim, p.t_lim, p.t_ext, p.fconst[0], p.fconst[1], p.fconst[2]};
}
// double: the limiter compares the square root itself (t_lim = vlim, t_ext = the extreme limit)
__device__ __forceinline__ Knobs<double> knobs_of(const StepParams& p, double) {
    return Knobs<double>{p.k64.tau_t, p.k64.beta, p.k64.G, p.k64.vlim, p.k64.vlim, p.k64.vlim_ext,
                         p.k64.fconst[0], p.k64.fconst[1], p.k64.fconst[2]};
}
// the thermal collision of the generic step in the arithmetic type R
template <int Q, class R>
__device__ __forceinline__ void thermal_collide_r(const StepParams& p, uint32_t n, const MomentsT<R>& m, R temperature,
                                                  const Coef<R>& k, R tau_t) {
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    const R uuh = uuh_of<false>(m.ux, m.uy, m.uz, k.d);
    const R* src = th_src_of(p, R(0));
    R* tgt = th_tgt_of(p, R(0));
    const R rtau_t = sizeof(R) == 4 ? R(p.Rtau_t) : R(0);
    const R ltau_t = sizeof(R) == 4 ? R(p.Ltau_t) : R(0);
    const bool ok_t = sizeof(R) == 4 && (p.div_ok & 8u) != 0;
#pragma unroll
    for (int i = 0; i < QT; i++) {
        const Dir c = ThermalLattice<QT>::c(i);
        const R w = ThermalW<QT, R>::w(i);
        const R cu = cdot_rt(c, m.ux, m.uy, m.uz);
        const R geq = feq_lit<false>(FMUL(w, temperature), cu, k.d, uuh);
        const R g = __ldg(src + (uint64_t)i * p.stride + n);
        tgt[(uint64_t)i * p.stride + n] = FSUB(g, div_u(FSUB(g, geq), tau_t, rtau_t, ltau_t, ok_t));
    }
}

// The thermal BGK with the thermal pull stream (stream_thermal.comp:457-526)
// folded in as a push.  The stream fills slot i of fluid cell m with
// B_i(m - c_i) when that source is a fluid cell in the domain, with
// -B_opp(i)(m) + 2 w_opp T_wall when it is solid (anti-bounce-back), and
// leaves it as it was (the pre-collision value) when it lies outside.  Here
// cell n writes its post-collision b_i to slot i of n + c_i unless that
// destination is outside or solid (mask bit opp(i): the source n - c_opp(i)
// is special), and fills its own slot i itself when its source n - c_i is
// special (mask bit i).  Every slot of the target keeps exactly one writer;
// solid cells write nothing, as in the stream.  The values are the stream's.
template <int Q>
__device__ __forceinline__ void thermal_collide_push(const StepParams& p, uint32_t n, int x, int y, int z, uint32_t mask,
                                                     const Moments& m, float temperature) {
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    using TL = ThermalLattice<QT>;
    const uint64_t S = p.stride;
    const Div<float> d = div_of(p);
    const float uuh = uuh_of<true>(m.ux, m.uy, m.uz, d);
    float a[QT], b[QT];
#pragma unroll
    for (int i = 0; i < QT; i++) {
        const Dir c = TL::c(i);
        const float w = TL::w(i);
        const float cu = cdot_rt(c, m.ux, m.uy, m.uz);
        const float geq = feq_lit<true>(FMUL(w, temperature), cu, d, uuh);
        a[i] = __ldg(p.th_src + (uint64_t)i * S + n);
        b[i] = thermal_relax(p, a[i], geq);
    }
    p.th_tgt[n] = b[0];
#pragma unroll
    for (int i = 1; i < QT; i++) {
        const Dir c = TL::c(i);
        if (!((mask >> opp(i)) & 1u)) {
            int dx = x + c.x, dy = y + c.y, dz = z + c.z;
            bool open;
            coords_wrap<Q>(dx, dy, dz, p.nx, p.ny, p.nz, open, p.flags);
            p.th_tgt[(uint64_t)i * S + (uint32_t)dx + (uint32_t)p.nx * ((uint32_t)dy + (uint32_t)p.ny * (uint32_t)dz)] = b[i];
        }
        if ((mask >> i) & 1u) {
            int sx = x - c.x, sy = y - c.y, sz = z - c.z;
            bool open;
            coords_wrap<Q>(sx, sy, sz, p.nx, p.ny, p.nz, open, p.flags);
            float v = a[i];
            if (!open) {
                const uint32_t sn = (uint32_t)sx + (uint32_t)p.nx * ((uint32_t)sy + (uint32_t)p.ny * (uint32_t)sz);
                const uint32_t sid = boundary_id(p.bnd, p.bits, sn);
                const int inv = opp(i);
                const float Tw = __ldg(p.objects + 3u * sid).w;
                v = __fadd_rn(-b[inv], __fmul_rn(2.f * TL::w(inv), Tw));
            }
            p.th_tgt[(uint64_t)i * S + n] = v;
        }
    }
}

// THERMAL (FP32 and 16-bit storage; FORCED set with it): the buoyancy and
// the thermal collision of the boundary-aware kernel, for cells whose
// sources are all plain.  GUARD: the cell's mask is loaded beside its
// populations and a cell with a nonzero mask stops after the loads (the
// periodic addresses stay inside the lattice), so that the mask costs no
// round trip of its own; returns whether the cell was updated.
template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool MP, bool EDGE, bool THERMAL = false,
          bool GUARD = false, class Load, class AfterLoads = NoHook>
__device__ __forceinline__ CellSumT<typename Codec<ST>::R> fast_cell(const StepParams& p, int x, int y, int z,
                                                                     Load&& load, AfterLoads after_loads = {}) {
    using L = Lattice<Q>;
    using C = Codec<ST>;
    using T = typename C::T;
    using R = typename C::R;
    using W = LatticeW<Q, R>;
    CellSumT<R> cs = {R(0), R(0), R(0), R(0), R(0)};
    const int nx = p.nx, ny = p.ny, nz = p.nz, nxy = nx * ny;
    const uint32_t n = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
    // The planes are contiguous (plane k at element k * stride of plane 0)
    // and Q * stride < 2^32, so every slot has a 32-bit element index off
    // one base: n + (plane offset + y/z neighbour offset, uniform over the
    // block) + x neighbour offset (per thread, periodic).
    T* const base = static_cast<T*>(p.plane[0]);
    const uint32_t S = (uint32_t)p.stride;
    const int oxm = x == 0 ? nx - 1 : -1, oxp = x == nx - 1 ? 1 - nx : 1;
    const int oym = y == 0 ? (ny - 1) * nx : -nx, oyp = y == ny - 1 ? (1 - ny) * nx : nx;
    const int ozm = z == 0 ? (nz - 1) * nxy : -nxy, ozp = z == nz - 1 ? (1 - nz) * nxy : nxy;
    // slot read for direction i; population i is written to the slot read
    // for opp(i): even (x + c_i, plane opp i), odd (x, plane i)
    auto slot = [&](int i, uint32_t nn, int xm, int xp) -> uint32_t {
        if (MODE == AA_EVEN) {
            const Dir c = L::c(i);
            const uint32_t u = EDGE ? (uint32_t)i * S + (uint32_t)((c.y > 0 ? oym : (c.y < 0 ? oyp : 0)) +
                                                                   (c.z > 0 ? ozm : (c.z < 0 ? ozp : 0)))
                                    : p.uoff[i];
            return nn + u + (uint32_t)(c.x > 0 ? xm : (c.x < 0 ? xp : 0));
        }
        return nn + (uint32_t)opp(i) * S;
    };
#ifndef BF_PTR_ADDR
#define BF_PTR_ADDR 1
#endif
#if BF_PTR_ADDR
    // byte pointers to this cell in plane 0 and to its x neighbours
    // (periodic); a slot is one of them plus a launch constant, a 64-bit
    // add of a uniform value (interior rows of even steps, all odd steps)
    const char* const cb = reinterpret_cast<const char*>(base) + (size_t)n * sizeof(T);
    const char* const cbm = cb + (ptrdiff_t)oxm * (ptrdiff_t)sizeof(T);
    const char* const cbp = cb + (ptrdiff_t)oxp * (ptrdiff_t)sizeof(T);
    auto make_ptr = [&](int i, const char* c0, const char* cm, const char* cp, uint32_t nn, int xm, int xp) -> T* {
        if (MODE == AA_EVEN && EDGE) return base + slot(i, nn, xm, xp);
        if (MODE == AA_EVEN) {
            const Dir c = L::c(i);
            const char* b = c.x > 0 ? cm : (c.x < 0 ? cp : c0);
            return reinterpret_cast<T*>(const_cast<char*>(b) + p.uoff_b[i]);
        }
        return reinterpret_cast<T*>(const_cast<char*>(c0) + p.poff_b[opp(i)]);
    };
    auto ptr_of = [&](int i) -> T* { return make_ptr(i, cb, cbm, cbp, n, oxm, oxp); };
    // the store phase recomputes its addresses from opaque copies of the
    // per-thread pointers instead of keeping Q addresses live
    const char *cb_st = cb, *cbm_st = cbm, *cbp_st = cbp;
    uint32_t n_st = n;
    int oxm_st = oxm, oxp_st = oxp;
    asm volatile("" : "+l"(cb_st), "+l"(cbm_st), "+l"(cbp_st), "+r"(n_st), "+r"(oxm_st), "+r"(oxp_st));
    auto ptr_st = [&](int i) -> T* { return make_ptr(i, cb_st, cbm_st, cbp_st, n_st, oxm_st, oxp_st); };
#else
    auto ptr_of = [&](int k) -> T* { return base + slot(k, n, oxm, oxp); };
    // the store phase recomputes its indices (one add each) from opaque
    // copies of the per-thread terms instead of keeping Q indices live
    uint32_t n_st = n;
    int oxm_st = oxm, oxp_st = oxp;
    asm volatile("" : "+r"(n_st), "+r"(oxm_st), "+r"(oxp_st));
    auto ptr_st = [&](int k) -> T* { return base + slot(k, n_st, oxm_st, oxp_st); };
#endif
    const uint32_t guard_mask = GUARD ? __ldg(p.nmask + n) : 0u;
    R f[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) f[i] = C::raw_dec(load(i, ptr_of));
    // thermal flow: the cell's thermal populations (the buoyancy's
    // temperature) are loaded with its flow populations, one round trip
    constexpr int QT = Lattice<Q>::D == 2 ? 5 : 7;
    float th[QT];
    if constexpr (THERMAL && sizeof(R) == 4) {
#pragma unroll
        for (int i = 0; i < QT; i++) th[i] = __ldg(p.th_src + (uint64_t)i * p.stride + n);
    }
    // work the caller issues while the loads are in flight
    after_loads();
    if (GUARD && guard_mask != 0u) return cs;
    // the update runs on the stored values times 1/SCALE implied: G = g * SCALE
    constexpr int SCE = C::SCALE_EXP;
    MomentsT<R> m;
    density_into<Q, C::SHIFTED, SCE>(f, m, p.err);
    constexpr bool F64 = sizeof(R) == 8;
    m.Fx = FORCED ? (F64 ? R(p.k64.fconst[0]) : R(p.fconst[0])) : R(0);
    m.Fy = FORCED ? (F64 ? R(p.k64.fconst[1]) : R(p.fconst[1])) : R(0);
    m.Fz = FORCED ? (F64 ? R(p.k64.fconst[2]) : R(p.fconst[2])) : R(0);
    // psi(rho) of the cell: the force's factor and, unchanged (rho is not
    // modified after it), this step's psi field value
    float psi_self = 0.f;
    if constexpr (MP && !F64) psi_self = sc_force<Q, C::SHIFTED>(p, n, oxm, oxp, oym, oyp, ozm, ozp, m);
    float temperature = 0.f;
    if constexpr (THERMAL && !F64) {
        static_assert(FORCED, "thermal flow runs with the source term on");
        temperature = thermal_buoyancy_of<Q>(th, p.beta, m);
    }
    if constexpr (F64) velocity_literal<Q, !MP>(f, m, FORCED, p.k64.vlim, p.k64.vlim, p.k64.vlim_ext);
    else if constexpr (C::SHIFTED) velocity_and_limit<Q, SCE>(f, m, FORCED, p.vlim, p.t_lim, p.t_ext);
    else velocity_literal<Q, !MP>(f, m, FORCED, p.vlim, p.t_lim, p.t_ext);
    if (p.flags & F_UPDATE) {
        const Coef<R> k = coef_of(p, R(0));
        // 16-bit multiphase flow: mass-conserving rounding (collided_sum);
        // rest is T less the stored values of the populations emitted so far
        R rest = R(0);
        if constexpr (MP && C::SHIFTED) rest = collided_sum<SCE>(m);
        auto emit = [&](int i, R v) {
            if constexpr (MP && C::SHIFTED) {
                if (i == Q - 1) return;  // stored below, from rest
                const T h = C::raw_enc(v);
                rest = FSUB(rest, C::raw_dec(h));
                *ptr_st(opp(i)) = h;
            } else {
                *ptr_st(opp(i)) = C::raw_enc(v);
            }
        };
        if constexpr (C::SHIFTED && FORCED) shifted_source_collide<Q, TRT, SCE>(f, m, k, emit);
        else if (m.out_ext) collide_fixed<Q, TRT, FORCED, true, C::SHIFTED, SCE>(f, m, k, emit);
        else collide_fixed<Q, TRT, FORCED, false, C::SHIFTED, SCE>(f, m, k, emit);
        if constexpr (MP && C::SHIFTED) *ptr_st(opp(Q - 1)) = C::raw_enc(rest);
    }
    if constexpr (MP && !F64) {
        // psi of this step's density for the next step (collide.comp:763-769)
        if (!(p.flags & F_MEASURE)) p.psi_tgt[n] = psi_self;
    }
    if constexpr (THERMAL && !F64) {
        // plain cells: every thermal source and destination is a fluid cell in the domain
        if (!(p.flags & F_MEASURE)) {
            if (p.thermal_push) thermal_collide_push<Q>(p, n, x, y, z, 0u, m, temperature);
            else thermal_collide<Q>(p, n, m, temperature);
        }
    }
    if (p.flags & F_SAVE) {
        p.vel_den[n] = make_float4((float)m.ux, (float)m.uy, (float)m.uz, (float)m.rho);
        if (p.force_temp) p.force_temp[n] = make_float4((float)m.Fx, (float)m.Fy, (float)m.Fz, temperature);
    }
    if (p.flags & F_REDUCE) {
        const R uu = uu_of(m.ux, m.uy, m.uz);
        cs.m = m.rho; cs.px = m.rho * m.ux; cs.py = m.rho * m.uy; cs.pz = m.rho * m.uz;
        cs.ke = R(0.5f) * m.rho * uu;
    }
    return cs;
}

template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool MP>
__global__ void __launch_bounds__(kStepBlock,
                                  ST == ST_FP64 ? 2 : ((ST == ST_FP32 || Q == 27) ? kFastMinBlocks : kFastMinBlocks16))
    fast_step_kernel(const __grid_constant__ StepParams p) {
    // the first warp prefetches the rows of the block pf_blocks ahead: once
    // its own cell's loads are in flight, or (Shan-Chen flow, whose psi
    // stencil loads come after) before them -- each measured the faster
    auto prefetch = [&]() {
        if (p.pf_blocks != 0u && threadIdx.x < 32) {
            const uint32_t b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z) + p.pf_blocks;
            if (b < gridDim.x * gridDim.y * gridDim.z) prefetch_block_rows<Q, ST, MODE>(p, b, (int)threadIdx.x, (int)blockDim.x);
        }
    };
    if constexpr (MP) prefetch();
    auto prefetch_ahead = [&]() {
        if constexpr (!MP) prefetch();
    };
    using R = typename Codec<ST>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    CellSumT<R> cs = {R(0), R(0), R(0), R(0), R(0)};
    if (x < p.nx) {
        // block-uniform choice: rows on a y or z face wrap their neighbour offsets
        const bool edge = MODE == AA_EVEN &&
                          (y == 0 || y == p.ny - 1 || (Lattice<Q>::D == 3 && (z == 0 || z == p.nz - 1)));
        using T = typename Codec<ST>::T;
        auto load = [&](int i, auto&& ptr_of) -> T { return *ptr_of(i); };
        if (edge) cs = fast_cell<Q, ST, MODE, TRT, FORCED, MP, true, false, false>(p, x, y, z, load, prefetch_ahead);
        else cs = fast_cell<Q, ST, MODE, TRT, FORCED, MP, false, false, false>(p, x, y, z, load, prefetch_ahead);
    }
    if (p.flags & F_REDUCE) block_reduce_store(cs, p.red_partials);
}

// ---------------------------------------------------------------------------
// fast step, two cells per thread (16-bit storage): a thread updates the
// cells x and x+1 (x even) of one row.  Directions with c_x = 0 move both
// cells' populations as one aligned 32-bit word (one address, one load, one
// store, one packed conversion); directions with c_x != 0 load and store the
// two 16-bit values through one address.  The arithmetic of each cell is the
// one-cell kernel's (fast_cell), so results agree bit for bit.
// ---------------------------------------------------------------------------
template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool MP, bool EDGE, bool TILE, class AfterLoads = NoHook>
__device__ __forceinline__ void fast2_cells(const StepParams& p, int x, int y, int z, const float* tile = nullptr,
                                            uint32_t tile_bar = 0u, AfterLoads after_loads = {}) {
    using L = Lattice<Q>;
    using C = Codec<ST>;
    using T = typename C::T;
    static_assert(sizeof(T) == 2, "16-bit storage only");
    const int nx = p.nx, ny = p.ny, nz = p.nz, nxy = nx * ny;
    const uint32_t n = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
    const uint64_t S = p.stride;
    char* const base = static_cast<char*>(p.plane[0]);
    // byte pointers (plane 0, this row): cell x, x + 1, and the wrapped x - 1, x + 2
    char* const c0 = base + (size_t)n * 2;
    char* const cm = base + (size_t)(n + (uint32_t)(x == 0 ? nx - 1 : -1)) * 2;
    char* const cq = base + (size_t)(n + (uint32_t)(x + 2 == nx ? 2 - nx : 2)) * 2;
    const int oym = y == 0 ? (ny - 1) * nx : -nx, oyp = y == ny - 1 ? (1 - ny) * nx : nx;
    const int ozm = z == 0 ? (nz - 1) * nxy : -nxy, ozp = z == nz - 1 ? (1 - nz) * nxy : nxy;
    // byte offset of the slot read for direction i from a plane-0 pointer at the source's x
    auto uoff = [&](int i) -> int64_t {
        if (MODE == AA_ODD) return p.poff_b[opp(i)];
        if (!EDGE) return p.uoff_b[i];
        const Dir c = L::c(i);
        return ((int64_t)i * (int64_t)S + (int64_t)((c.y > 0 ? oym : (c.y < 0 ? oyp : 0)) +
                                                    (c.z > 0 ? ozm : (c.z < 0 ? ozp : 0)))) * 2;
    };
    // sources of direction i for cells x (a) and x + 1 (b): even step x - c_i, odd step x
    auto src_a = [&](int i) -> char* {
        const Dir c = L::c(i);
        if (MODE == AA_ODD || c.x == 0) return c0 + uoff(i);
        return (c.x > 0 ? cm : c0 + 2) + uoff(i);
    };
    auto src_b = [&](int i) -> char* {
        const Dir c = L::c(i);
        if (MODE == AA_ODD || c.x == 0) return c0 + 2 + uoff(i);
        return (c.x > 0 ? c0 : cq) + uoff(i);
    };
    auto paired = [&](int i) -> bool { return MODE == AA_ODD || L::c(i).x == 0; };
    // ---- loads: every population of both cells before any arithmetic ----
    uint32_t ld[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        if (paired(i)) {
            ld[i] = __ldg(reinterpret_cast<const unsigned int*>(src_a(i)));
        } else {
            const uint32_t a = __ldg(reinterpret_cast<const unsigned short*>(src_a(i)));
            const uint32_t b = __ldg(reinterpret_cast<const unsigned short*>(src_b(i)));
            ld[i] = a | (b << 16);
        }
    }
    // Shan-Chen (cached-load variant): the pair's psi stencil, loaded while
    // the populations are in flight, and both cells' stencil sums, so that
    // six sums stay live through the first cell's update instead of the stencil
    ScSum sc_pair[2];
    float pv[kPsiRows<Q>][4];
    if constexpr (MP && !TILE) psi_pair_load<Q>(p.psi_src, n, x, nx, oym, oyp, ozm, ozp, pv);
    // work the caller issues while the loads are in flight
    after_loads();
    if constexpr (MP && TILE) {
        // the block's psi rows arrive by bulk copy on tile_bar (bounded
        // wait; past the limit bit 1 of the error word is set and the step's
        // results are not to be used)
        if (!mbar_wait_bounded(tile_bar, 0u)) atomicOr(p.err, 2u);
        psi_pair_load_tile<Q>(tile, x, nx, pv);
    }
    if constexpr (MP) {
        sc_pair[0] = sc_sums<Q, C::SHIFTED>([&](const Dir c) { return pv[psi_row<Q>(c)][c.x + 1]; });
        sc_pair[1] = sc_sums<Q, C::SHIFTED>([&](const Dir c) { return pv[psi_row<Q>(c)][c.x + 2]; });
    }
    // the stores recompute their addresses from opaque copies of the pointers
    char *c0s = c0, *cms = cm, *cqs = cq;
    asm volatile("" : "+l"(c0s), "+l"(cms), "+l"(cqs));
    // store of population i goes to the slot read for opp(i)
    auto dst_a = [&](int i) -> char* {
        const int o = opp(i);
        const Dir c = L::c(o);
        if (MODE == AA_ODD || c.x == 0) return c0s + uoff(o);
        return (c.x > 0 ? cms : c0s + 2) + uoff(o);
    };
    auto dst_b = [&](int i) -> char* {
        const int o = opp(i);
        const Dir c = L::c(o);
        if (MODE == AA_ODD || c.x == 0) return c0s + 2 + uoff(o);
        return (c.x > 0 ? c0s : cqs) + uoff(o);
    };
    auto to16 = [](uint32_t v) -> T { const unsigned short u = (unsigned short)v; T t; memcpy(&t, &u, 2); return t; };
    auto bits16 = [](T t) -> uint32_t { unsigned short u; memcpy(&u, &t, 2); return u; };
    // cell a's populations of the paired directions until cell b's are known,
    // as floats that one cvt.rn.f16x2.f32 converts together with cell b's
    // (IEEE half storages; the same rounding as two conversions)
    uint32_t keep[Q];
    const Coef<float> k = coef_of(p, 0.0f);
    // the update runs on the stored values: G = g * SCALE for scaled storage
    constexpr int SCE = C::SCALE_EXP;
    float psi_first = 0.f;  // the first cell's psi, stored with the second's
#pragma unroll
    for (int half = 0; half < 2; half++) {
        float f[Q];
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = C::raw_dec(to16(half ? (ld[i] >> 16) : ld[i]));
        Moments m;
        density_into<Q, C::SHIFTED, SCE>(f, m, p.err);
        m.Fx = FORCED ? p.fconst[0] : 0.f;
        m.Fy = FORCED ? p.fconst[1] : 0.f;
        m.Fz = FORCED ? p.fconst[2] : 0.f;
        float psi_self = 0.f;
        if constexpr (MP) {
            psi_self = sc_apply(p.G, m, sc_pair[half]);
        }
        if constexpr (C::SHIFTED) velocity_and_limit<Q, SCE>(f, m, FORCED, p.vlim, p.t_lim, p.t_ext);
        else velocity_literal<Q, !MP>(f, m, FORCED, p.vlim, p.t_lim, p.t_ext);
        // multiphase: the mass-conserving rounding of the one-cell kernel
        // (collided_sum; rest is T less the stored values emitted so far)
        float rest = 0.f;
        if constexpr (MP && C::SHIFTED) rest = collided_sum<SCE>(m);
        // store of this cell's encoded population i (a paired slot keeps the
        // first cell's half until the second cell's is known)
        auto put = [&](int i, uint32_t e) {
            if (paired(opp(i))) {
                if (half == 0) keep[i] = e;
                else *reinterpret_cast<unsigned int*>(dst_a(i)) = keep[i] | (e << 16);
            } else {
                *reinterpret_cast<unsigned short*>(half ? dst_b(i) : dst_a(i)) = (unsigned short)e;
            }
        };
        // both populations of the opposite pair (i, i + 1) of this cell, packed
        // lo | hi << 16 (a paired slot keeps the first cell's word in keep[i])
        auto put2 = [&](int i, uint32_t w2) {
            if (paired(opp(i))) {
                if (half == 0) {
                    keep[i] = w2;
                } else {
                    *reinterpret_cast<unsigned int*>(dst_a(i)) = __byte_perm(keep[i], w2, 0x5410u);
                    *reinterpret_cast<unsigned int*>(dst_a(i + 1)) = __byte_perm(keep[i], w2, 0x7632u);
                }
            } else {
                *reinterpret_cast<unsigned short*>(half ? dst_b(i) : dst_a(i)) = (unsigned short)w2;
                *reinterpret_cast<unsigned short*>(half ? dst_b(i + 1) : dst_a(i + 1)) = (unsigned short)(w2 >> 16);
            }
        };
        float pend = 0.f;  // the first population of an opposite pair until the second is emitted
        auto emit = [&](int i, float v) {
            if constexpr (MP && C::SHIFTED) {
                // populations 1..Q-1 come as opposite pairs (i, i + 1), i odd:
                // one cvt.rn.f16x2.f32 rounds both (each as its own conversion
                // would); population Q-1 is stored after the collision, from rest
                if (i == 0) {
                    const T h = C::raw_enc(v);
                    rest = FSUB(rest, C::raw_dec(h));
                    put(0, bits16(h));
                } else if (i & 1) {
                    pend = v;
                } else if (i == Q - 1) {
                    const T h = C::raw_enc(pend);
                    rest = FSUB(rest, C::raw_dec(h));
                    put(i - 1, bits16(h));
                } else {
                    const __half2 h2 = __floats2half2_rn(pend, v);
                    rest = FSUB(rest, __low2float(h2));
                    rest = FSUB(rest, __high2float(h2));
                    uint32_t w2;
                    memcpy(&w2, &h2, 4);
                    put2(i - 1, w2);
                }
                return;
            }
            if constexpr (std::is_same<T, __half>::value) {
                if (paired(opp(i))) {
                    if (half == 0) {
                        keep[i] = __float_as_uint(v);
                    } else {
                        const __half2 h = __floats2half2_rn(__uint_as_float(keep[i]), v);
                        uint32_t w2;
                        memcpy(&w2, &h, 4);
                        *reinterpret_cast<unsigned int*>(dst_a(i)) = w2;
                    }
                    return;
                }
            }
            put(i, bits16(C::raw_enc(v)));
        };
        if constexpr (C::SHIFTED && FORCED) shifted_source_collide<Q, TRT, SCE>(f, m, k, emit);
        else if (m.out_ext) collide_fixed<Q, TRT, FORCED, true, C::SHIFTED, SCE>(f, m, k, emit);
        else collide_fixed<Q, TRT, FORCED, false, C::SHIFTED, SCE>(f, m, k, emit);
        if constexpr (MP && C::SHIFTED) put(Q - 1, bits16(C::raw_enc(rest)));
        if constexpr (MP) {
            // psi of this step's density for the next step (collide.comp:763-769):
            // both cells' values as one aligned float2 (n even)
            if (half == 0) psi_first = psi_self;
            else if (!(p.flags & F_MEASURE))
                *reinterpret_cast<float2*>(p.psi_tgt + n) = make_float2(psi_first, psi_self);
        }
        if (p.flags & F_SAVE) {
            p.vel_den[n + half] = make_float4(m.ux, m.uy, m.uz, m.rho);
            if (p.force_temp) p.force_temp[n + half] = make_float4(m.Fx, m.Fy, m.Fz, 0.f);
        }
    }
}

#ifndef BF_FAST2_MIN_BLOCKS
#define BF_FAST2_MIN_BLOCKS 4
#endif
// 64 registers (4 blocks of 256 per SM): a thread holds both cells' loads; a few
// TRT and forced variants spill a handful of words, which measured cheaper than
// the latency of running at 3 blocks (Shan-Chen 256^3 at 3 blocks, 80 registers
// and no spills: fp16s 60.2k / fp16c 59.2k MLUPs against 61.8k / 61.6k)
#ifndef BF_FAST2_MP_MIN_BLOCKS
#define BF_FAST2_MP_MIN_BLOCKS BF_FAST2_MIN_BLOCKS
#endif
// TILE (Shan-Chen only): the psi stencil staged in shared memory (p.psi_tile)
template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool MP, bool TILE>
__global__ void __launch_bounds__(kStepBlock, MP ? BF_FAST2_MP_MIN_BLOCKS : BF_FAST2_MIN_BLOCKS)
    fast2_step_kernel(const __grid_constant__ StepParams p) {
    // the first warp prefetches the rows of the block pf_blocks ahead: once
    // its own cells' loads are in flight, or (Shan-Chen flow) before them --
    // each measured the faster
    auto prefetch = [&]() {
        if (p.pf_blocks != 0u && threadIdx.x < 32) {
            const uint32_t b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z) + p.pf_blocks;
            if (b < gridDim.x * gridDim.y * gridDim.z)
                prefetch_block_rows<Q, ST, MODE>(p, b, (int)threadIdx.x, 2 * (int)blockDim.x);
        }
    };
    if constexpr (MP && !TILE) prefetch();
    auto prefetch_ahead = [&]() {
        if constexpr (!MP) prefetch();
    };
    const int x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y, z = blockIdx.z;
    const float* tile = nullptr;
    uint32_t tile_bar = 0u;
    if constexpr (MP && TILE) {
        // the block's row is the whole row (nx <= 2 x block, nx % 4 == 0): the
        // psi rows (y + dy, z + dz), dy, dz in {-1, 0, 1} (dz = 0 in 2D), come
        // into shared memory as one bulk copy each, completing on an mbarrier
        // that the cells wait on after issuing their population loads
        constexpr int ROWS = kPsiRows<Q>;
        extern __shared__ __align__(16) float s_psi[];
        __shared__ __align__(8) uint64_t s_bar;
        tile_bar = smem_addr(&s_bar);
        if (threadIdx.x == 0) {
            mbar_init(tile_bar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int nx = p.nx, ny = p.ny, nz = p.nz;
            const uint32_t row_bytes = (uint32_t)nx * (uint32_t)sizeof(float);
            mbar_arrive_expect_tx(tile_bar, (uint32_t)ROWS * row_bytes);
            for (int r = 0; r < ROWS; r++) {
                const int dy = Lattice<Q>::D == 2 ? r - 1 : r / 3 - 1, dz = Lattice<Q>::D == 2 ? 0 : r % 3 - 1;
                const int yy = y + dy < 0 ? y + dy + ny : (y + dy >= ny ? y + dy - ny : y + dy);
                const int zz = z + dz < 0 ? z + dz + nz : (z + dz >= nz ? z + dz - nz : z + dz);
                bulk_g2s(smem_addr(s_psi + r * nx), p.psi_src + (size_t)nx * ((size_t)yy + (size_t)ny * (size_t)zz),
                         row_bytes, tile_bar);
            }
        }
        // the look-ahead prefetch after the block barrier, which it would delay
        prefetch();
        tile = s_psi;
    }
    if (x >= p.nx) return;
    const bool edge = MODE == AA_EVEN && (y == 0 || y == p.ny - 1 || (Lattice<Q>::D == 3 && (z == 0 || z == p.nz - 1)));
    if (edge) fast2_cells<Q, ST, MODE, TRT, FORCED, MP, true, TILE>(p, x, y, z, tile, tile_bar, prefetch_ahead);
    else fast2_cells<Q, ST, MODE, TRT, FORCED, MP, false, TILE>(p, x, y, z, tile, tile_bar, prefetch_ahead);
}

// ---------------------------------------------------------------------------
// boundary-aware fast step: objects (solid cells, halfway bounce-back with
// moving walls, equilibrium velocity/density cells), open (non-periodic)
// domain faces and a constant force, in the esoteric-pull modes.  A per-cell
// mask built once at initialisation marks the directions whose AA source
// needs the generic treatment; every other direction uses the fast kernel's
// addressing, and the arithmetic is the generic kernel's, so results agree
// bit for bit.
// ---------------------------------------------------------------------------
// per-cell mask of the boundary-aware step: bit i (1 <= i < Q) marks a
// direction whose AA source is outside the domain or solid under bounce-back;
// bit 31 a solid cell, bit 30 an equilibrium-boundary cell with its object
// kind in bits 27-28 (1 velocity, 2 density); bit 29, on a cell with a
// solid source: every solid source's object moves with velocity (+0, +0, +0)
// (the bounce-back wall term needs no object lookup).  Q - 1 <= 26 direction bits stay below bit 27.
constexpr int kMaskKindShift = 27;
constexpr int kMaskRestingBit = 29;
template <int Q>
__global__ void build_mask_kernel(const __grid_constant__ StepParams p, uint32_t* __restrict__ mask) {
    using L = Lattice<Q>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= p.nx) return;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint32_t flags = p.flags;
    const uint32_t n = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
    const uint32_t bid = (flags & F_BOUNDARIES) ? boundary_id(p.bnd, p.bits, n) : 0u;
    uint32_t m = 0u;
    if (solid_id(p.obj_kind, bid)) m |= 1u << 31;
    else if (bid != 0u) m |= (1u << 30) | ((uint32_t)__ldg(p.obj_kind + bid) & 3u) << kMaskKindShift;
    bool resting = true, solid_source = false;  // every solid source's wall velocity is (+0, +0, +0)
#pragma unroll
    for (int i = 1; i < Q; i++) {
        const Dir c = L::c(i);
        int sx = x - c.x, sy = y - c.y, sz = z - c.z;
        bool sopen;
        coords_wrap<Q>(sx, sy, sz, nx, ny, nz, sopen, flags);
        bool special = sopen;
        if (!sopen && (flags & F_BOUNCE_BACK) && (flags & F_BOUNDARIES)) {
            const uint32_t sn = (uint32_t)sx + (uint32_t)nx * ((uint32_t)sy + (uint32_t)ny * (uint32_t)sz);
            const uint32_t sid = boundary_id(p.bnd, p.bits, sn);
            special = solid_id(p.obj_kind, sid);
            if (special) {
                solid_source = true;
                const float4 uw = __ldg(p.objects + 3u * sid);
                if ((__float_as_uint(uw.x) | __float_as_uint(uw.y) | __float_as_uint(uw.z)) != 0u) resting = false;
            }
        }
        if (special) m |= 1u << i;
    }
    // only on a cell the direction bits already make special (a zero mask
    // means a plain cell)
    if (solid_source && resting) m |= 1u << kMaskRestingBit;
    mask[n] = m;
}

template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool THERMAL, bool EDGE>
__device__ __forceinline__ CellSum masked_cell(const StepParams& p, int x, int y, int z, uint32_t mask) {
    using L = Lattice<Q>;
    using C = Codec<ST>;
    using T = typename C::T;
    CellSum cs = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int nx = p.nx, ny = p.ny, nz = p.nz, nxy = nx * ny;
    const uint32_t flags = p.flags;
    const uint32_t n = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
    if (mask >> 31) {  // solid cell (collide.comp:696-700)
        if (flags & F_SAVE) {
            p.vel_den[n] = make_float4(0.f, 0.f, 0.f, 0.f);
            p.force_temp[n] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p.bnd_tex) p.bnd_tex[n] = (uint8_t)boundary_id(p.bnd, p.bits, n);
        }
        return cs;
    }
    const bool eqb = (mask >> 30) & 1u;
    const bool resting = (mask >> kMaskRestingBit) & 1u;
    float4 bv = make_float4(1.f, 0.f, 0.f, 0.f);
    if (eqb && p.bvals) bv = __ldg(p.bvals + n);
    T* const base = static_cast<T*>(p.plane[0]);
    const uint32_t S = (uint32_t)p.stride;
    const int oxm = x == 0 ? nx - 1 : -1, oxp = x == nx - 1 ? 1 - nx : 1;
    const int oym = y == 0 ? (ny - 1) * nx : -nx, oyp = y == ny - 1 ? (1 - ny) * nx : nx;
    const int ozm = z == 0 ? (nz - 1) * nxy : -nxy, ozp = z == nz - 1 ? (1 - nz) * nxy : nxy;
    auto slot = [&](int i, uint32_t nn, int xm, int xp) -> uint32_t {
        if (MODE == AA_EVEN) {
            const Dir c = L::c(i);
            const uint32_t u = EDGE ? (uint32_t)i * S + (uint32_t)((c.y > 0 ? oym : (c.y < 0 ? oyp : 0)) +
                                                                   (c.z > 0 ? ozm : (c.z < 0 ? ozp : 0)))
                                    : p.uoff[i];
            return nn + u + (uint32_t)(c.x > 0 ? xm : (c.x < 0 ? xp : 0));
        }
        return nn + (uint32_t)opp(i) * S;
    };
    float f[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const float w = L::w(i);
        if (i == 0 || !((mask >> i) & 1u)) {  // direction bits only (i < 27)
            f[i] = C::dec(base[slot(i, n, oxm, oxp)], w);
            continue;
        }
        // the generic kernel's treatment of a source outside the domain or solid
        const Dir c = L::c(i);
        int sx = x - c.x, sy = y - c.y, sz = z - c.z;
        bool sopen;
        coords_wrap<Q>(sx, sy, sz, nx, ny, nz, sopen, flags);
        const uint32_t sn = sopen ? 0u : (uint32_t)sx + (uint32_t)nx * ((uint32_t)sy + (uint32_t)ny * (uint32_t)sz);
        if (eqb && sopen) {  // population entering from outside: f_eq(rho_b, u_b)
            const float cu = cdot_rt(c, bv.y, bv.z, bv.w);
            const float one_mb = FSUB(1.0f, FMUL(uu_of(bv.y, bv.z, bv.w), p.R2h));
            const float br = bracket(cu, one_mb, p.R2, p.R4h);
            f[i] = C::SHIFTED ? FFMA(FMUL(w, bv.x), br, -w) : FMUL(FMUL(w, bv.x), br);
        } else if (!sopen) {  // solid source under bounce-back (stream.comp:487-496, rho_wall = 1)
            // resting walls: the same expression on the (+0, +0, +0) velocity the object holds
            const float4 uw = resting ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(p.objects + 3u * boundary_id(p.bnd, p.bits, sn));
            const Dir co = L::c(opp(i));
            const float wall = FMUL(FMUL(-2.f * w, co.x * uw.x + co.y * uw.y + co.z * uw.z), 3.f);
            const float v = (MODE == AA_EVEN) ? C::dec(base[(uint32_t)opp(i) * S + n], w)
                                              : C::dec(base[(uint32_t)i * S + sn], w);
            f[i] = FADD(v, wall);
        } else if (MODE == AA_EVEN) {  // out-of-domain read (collide.comp:278-298)
            f[i] = C::SHIFTED ? FSUB(0.01f, w) : 0.01f;
        } else {  // odd steps read the cell's own slot whatever lies outside
            f[i] = C::dec(base[slot(i, n, oxm, oxp)], w);
        }
    }
    uint32_t n_st = n;
    int oxm_st = oxm, oxp_st = oxp;
    asm volatile("" : "+r"(n_st), "+r"(oxm_st), "+r"(oxp_st));

    Moments m;
    density_into<Q, C::SHIFTED, 0>(f, m, p.err);
    m.Fx = FORCED ? p.fconst[0] : 0.f;
    m.Fy = FORCED ? p.fconst[1] : 0.f;
    m.Fz = FORCED ? p.fconst[2] : 0.f;
    float temperature = 0.f;
    if (THERMAL) temperature = thermal_buoyancy<Q>(p, n, m);  // the generic kernel's buoyancy
    // thermal flow is forced with the source term on, as in the generic kernel
    constexpr bool FRC = FORCED || THERMAL;
    if constexpr (C::SHIFTED) velocity_and_limit<Q>(f, m, FRC, p.vlim, p.t_lim, p.t_ext);
    else velocity_literal<Q>(f, m, FRC, p.vlim, p.t_lim, p.t_ext);
    if (eqb) {
        const uint32_t kind = (mask >> kMaskKindShift) & 3u;
        if (kind == 1u) { m.ux = bv.y; m.uy = bv.z; m.uz = bv.w; } else { m.rho = bv.x; }
        m.Fx = m.Fy = m.Fz = 0.f;
    }
    if (flags & F_UPDATE) {
        const Coef<float> k = coef_of(p, 0.0f);
        auto emit = [&](int i, float v) {
            if (MODE == AA_EVEN && ((mask >> opp(i)) & 1u)) {
                // the destination x + c_i is the source of opp(i): dropped when outside
                const Dir c = L::c(i);
                int dx = x + c.x, dy = y + c.y, dz = z + c.z;
                bool dopen;
                coords_wrap<Q>(dx, dy, dz, nx, ny, nz, dopen, flags);
                if (dopen) return;
            }
            base[slot(opp(i), n_st, oxm_st, oxp_st)] = C::enc(v, L::w(i));
        };
        if (eqb) collide_fixed<Q, false, false, true, C::SHIFTED>(f, m, k, emit);  // f_eq of the cell
        else if constexpr (C::SHIFTED && FRC) shifted_source_collide<Q, TRT, 0>(f, m, k, emit);
        else if (m.out_ext) collide_fixed<Q, TRT, FRC, true, C::SHIFTED>(f, m, k, emit);
        else collide_fixed<Q, TRT, FRC, false, C::SHIFTED>(f, m, k, emit);
    }
    if (THERMAL && !(flags & F_MEASURE)) {
        if (p.thermal_push) thermal_collide_push<Q>(p, n, x, y, z, mask, m, temperature);
        else thermal_collide<Q>(p, n, m, temperature);
    }
    if (flags & F_SAVE) {
        p.vel_den[n] = make_float4(m.ux, m.uy, m.uz, m.rho);
        p.force_temp[n] = make_float4(m.Fx, m.Fy, m.Fz, temperature);
        if (p.bnd_tex) p.bnd_tex[n] = eqb ? (uint8_t)boundary_id(p.bnd, p.bits, n) : (uint8_t)0;
    }
    if (flags & F_REDUCE) {
        const float uu = uu_of(m.ux, m.uy, m.uz);
        cs.m = m.rho; cs.px = m.rho * m.ux; cs.py = m.rho * m.uy; cs.pz = m.rho * m.uz;
        cs.ke = 0.5f * m.rho * uu;
    }
    return cs;
}

// 64 registers (4 blocks of 256 per SM); D3Q27 gets 80 (3 blocks), below which it spills
template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool THERMAL>
__global__ void __launch_bounds__(kStepBlock, Q == 27 ? 3 : kFastMinBlocks)
    masked_step_kernel(const __grid_constant__ StepParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    CellSum cs = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (x < p.nx) {
        const uint32_t n = (uint32_t)x + (uint32_t)p.nx * ((uint32_t)y + (uint32_t)p.ny * (uint32_t)z);
        const uint32_t mask = __ldg(p.nmask + n);
        const bool edge = MODE == AA_EVEN &&
                          (y == 0 || y == p.ny - 1 || (Lattice<Q>::D == 3 && (z == 0 || z == p.nz - 1)));
        if (!THERMAL && !edge && mask == 0u) {
            // no special source, no boundary id: every source and destination
            // is an ordinary in-domain slot (x +- 1 never wraps here), so the
            // periodic kernel's cell update applies as it is
            using T = typename Codec<ST>::T;
            auto load = [&](int i, auto&& ptr_of) -> T { return *ptr_of(i); };
            cs = fast_cell<Q, ST, MODE, TRT, FORCED, false, false>(p, x, y, z, load);
            if ((p.flags & F_SAVE) && p.bnd_tex) p.bnd_tex[n] = 0;
        } else if (edge) {
            cs = masked_cell<Q, ST, MODE, TRT, FORCED, THERMAL, true>(p, x, y, z, mask);
        } else {
            cs = masked_cell<Q, ST, MODE, TRT, FORCED, THERMAL, false>(p, x, y, z, mask);
        }
    }
    if (p.flags & F_REDUCE) block_reduce_store(cs, p.red_partials);
}

// The boundary-aware step with the special cells taken out of the lanes (no
// reduction).  In an AA step every slot is read and written by exactly one
// cell, so the cells of a step are independent and any partition of them
// over blocks gives the same result.  Plain blocks update the cells whose
// mask is empty, in the periodic kernel's cell update, and leave the others:
// their warps never wait for one lane's special treatment (every row of a
// channel with inlet and outlet faces starts and ends with a special cell).
// Blocks of special_chunk listed cells follow in launch order as soon as the
// plain blocks of their rows have been launched (the host's schedule).
// Blocks are dispatched about in launch order, so the special cells are
// updated right after their neighbours streamed the same 32-byte sectors
// through L2, in short blocks of their own, however dense they lie (a wall
// plane is a run of special blocks).
// 4 blocks per SM (64 registers; some even-step variants spill 12-64 bytes):
// 3 blocks without spills measured 31.4k against 35.1k MLUPs on flow past a
// sphere, 18.6k against 20.8k on Rayleigh-Benard.  Thermal flow: 5 blocks
// (48 registers; the spills cost less than the latency they hide: 27.2k ->
// 28.9k on Rayleigh-Benard; flow past a sphere at 5: 38.6k -> 37.8k)
#ifndef BF_MIXED_MIN_BLOCKS
#define BF_MIXED_MIN_BLOCKS kFastMinBlocks
#endif
#ifndef BF_MIXED_MIN_BLOCKS_THERMAL
#define BF_MIXED_MIN_BLOCKS_THERMAL 5
#endif
template <int Q, int ST, int MODE, bool TRT, bool FORCED, bool THERMAL>
__global__ void __launch_bounds__(kStepBlock, THERMAL ? BF_MIXED_MIN_BLOCKS_THERMAL : BF_MIXED_MIN_BLOCKS)
    masked_mixed_kernel(const __grid_constant__ StepParams p) {
    const uint32_t nx = (uint32_t)p.nx, ny = (uint32_t)p.ny;
    const uint32_t e = __ldg(p.sched + blockIdx.x);
    // a plain entry: bx | y << sched_shy | z << sched_shz
    const uint32_t shy = p.sched_shy, shz = p.sched_shz;
    const uint32_t mx = (1u << shy) - 1u, my = (1u << (shz - shy)) - 1u;
    // the entry pf_blocks ahead, loaded beside this block's own entry
    const bool has_ahead = p.pf_blocks != 0u && threadIdx.x < 32 && blockIdx.x + p.pf_blocks < p.n_sched;
    const uint32_t ahead = has_ahead ? __ldg(p.sched + blockIdx.x + p.pf_blocks) : 0x80000000u;
    if (!(e >> 31)) {
        // the first warp prefetches the rows of that plain block (one plane
        // per lane) once its own cell's loads are in flight
        auto prefetch_ahead = [&]() {
            if (!(ahead >> 31)) {
                const uint32_t abx = ahead & mx, ay = (ahead >> shy) & my, az = ahead >> shz;
                prefetch_rows_at<Q, ST, MODE>(p, abx, (int)ay, (int)az, (int)threadIdx.x, (int)blockDim.x);
                if (THERMAL && ST != ST_FP64 && p.th_src)
                    prefetch_thermal_rows_at<Q>(p, abx, ay + ny * az, (int)threadIdx.x, (int)blockDim.x);
            }
        };
        const int x = (int)((e & mx) * blockDim.x + threadIdx.x);
        const int y = (int)((e >> shy) & my), z = (int)(e >> shz);
        const uint32_t yz = (uint32_t)y + ny * (uint32_t)z;
        if (x >= p.nx) return;
        using T = typename Codec<ST>::T;
        auto load = [&](int i, auto&& ptr_of) -> T { return *ptr_of(i); };
        const bool edge = MODE == AA_EVEN && (y == 0 || y == p.ny - 1 || (Lattice<Q>::D == 3 && (z == 0 || z == p.nz - 1)));
        if (edge) fast_cell<Q, ST, MODE, TRT, FORCED, false, true, THERMAL, true>(p, x, y, z, load, prefetch_ahead);
        else fast_cell<Q, ST, MODE, TRT, FORCED, false, false, THERMAL, true>(p, x, y, z, load, prefetch_ahead);
        if ((p.flags & F_SAVE) && p.bnd_tex) {
            const uint32_t n = (uint32_t)x + nx * yz;
            if (__ldg(p.nmask + n) == 0u) p.bnd_tex[n] = 0;
        }
        return;
    }
    if (threadIdx.x < p.special_chunk) {
        const uint32_t k = (e & 0x7fffffffu) * p.special_chunk + threadIdx.x;
        if (k >= p.n_special) return;
        // the cell and its mask, listed side by side (one round trip)
        const uint32_t n = __ldg(p.special + k), cell_mask = __ldg(p.special_mask + k);
        const uint32_t yz = n / nx;
        const int x = (int)(n - yz * nx), y = (int)(yz % ny), z = (int)(yz / ny);
        // the face-row variant computes every neighbour offset with its wrap,
        // which is right for any row
        masked_cell<Q, ST, MODE, TRT, FORCED, THERMAL, true>(p, x, y, z, cell_mask);
    }
}


// ---------------------------------------------------------------------------
// generic AA / two-buffer step: open boundaries, packed boundary ids, solid
// skipping or bounce-back, equilibrium boundary cells, force fields, thermal
// lattice, Shan-Chen pseudopotential, field saving and reductions
// ---------------------------------------------------------------------------
template <int Q, int ST, int MODE>
__device__ __forceinline__ CellSumT<typename Codec<ST>::R> cell_update(const StepParams& p, int x, int y, int z) {
    using L = Lattice<Q>;
    using C = Codec<ST>;
    using T = typename C::T;
    using R = typename C::R;
    using W = LatticeW<Q, R>;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint32_t flags = p.flags;
    const uint32_t n = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
    auto plane = [&](int i) -> T* { return static_cast<T*>(p.plane[i]); };
    CellSumT<R> out = {R(0), R(0), R(0), R(0), R(0)};
    const Coef<R> k = coef_of(p, R(0));
    const Knobs<R> kn = knobs_of(p, R(0));

    uint32_t bid = 0;
    if (flags & F_BOUNDARIES) {
        bid = boundary_id(p.bnd, p.bits, n);
        if (solid_id(p.obj_kind, bid)) {  // collide.comp:696-700
            if (flags & F_SAVE) {
                p.vel_den[n] = make_float4(0.f, 0.f, 0.f, 0.f);
                p.force_temp[n] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (p.bnd_tex) p.bnd_tex[n] = (uint8_t)bid;
            }
            return out;
        }
    }
    const bool eqb = bid != 0u;  // equilibrium boundary cell (non-solid object)
    float4 bv = make_float4(1.f, 0.f, 0.f, 0.f);
    if (eqb && p.bvals) bv = __ldg(p.bvals + n);

    // ---- load (AA read, collide.comp:244-305) ----
    R f[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const Dir c = L::c(i);
        const R w = W::w(i);
        int sx = x - c.x, sy = y - c.y, sz = z - c.z;
        bool sopen;
        coords_wrap<Q>(sx, sy, sz, nx, ny, nz, sopen, flags);
        const uint32_t sn = sopen ? 0u : (uint32_t)sx + (uint32_t)nx * ((uint32_t)sy + (uint32_t)ny * (uint32_t)sz);
        bool done = false;
        if (MODE != AA_LOCAL && (eqb || (flags & F_BOUNCE_BACK)) && i != 0) {
            if (eqb && sopen) {
                // population entering from outside the domain: f_eq(rho_b, u_b)
                const R bx = R(bv.y), by = R(bv.z), bz = R(bv.w);
                const R cu = cdot_rt(c, bx, by, bz);
                const R one_mb = FSUB(R(1), FMUL(uu_of(bx, by, bz), k.R2h));
                const R br = bracket(cu, one_mb, k.R2, k.R4h);
                f[i] = C::SHIFTED ? FFMA(FMUL(w, R(bv.x)), br, -w) : FMUL(FMUL(w, R(bv.x)), br);
                done = true;
            } else if ((flags & F_BOUNCE_BACK) && !sopen && (flags & F_BOUNDARIES)) {
                const uint32_t sid = boundary_id(p.bnd, p.bits, sn);
                if (solid_id(p.obj_kind, sid)) {
                    // halfway bounce-back: the cell's own outgoing opposite
                    // population sits in the other AA slot; moving-wall term of
                    // stream.comp:487-496 with rho_wall = 1
                    const float4 uw = __ldg(p.objects + 3u * sid);
                    const Dir co = L::c(opp(i));
                    const R dw = FADD(FADD(FMUL(R(co.x), R(uw.x)), FMUL(R(co.y), R(uw.y))), FMUL(R(co.z), R(uw.z)));
                    const R wall = FMUL(FMUL(R(-2) * w, dw), R(3));
                    const R v = (MODE == AA_EVEN) ? C::dec(plane(opp(i))[n], w) : C::dec(plane(i)[sn], w);
                    f[i] = FADD(v, wall);
                    done = true;
                }
            }
        }
        if (!done) {
            // out-of-domain reads give 0.01 (collide.comp:278-298), g = 0.01 - w when shifted
            if (MODE == AA_EVEN) f[i] = sopen ? (C::SHIFTED ? FSUB(R(0.01), w) : R(0.01)) : C::dec(plane(i)[sn], w);
            else if (MODE == AA_ODD) f[i] = C::dec(plane(opp(i))[n], w);
            else f[i] = C::dec(plane(i)[n], w);
        }
    }

    // ---- moments and forces (collide.comp:702-725) ----
    MomentsT<R> m;
    density_into<Q, C::SHIFTED, 0>(f, m, p.err);  // max(density, 0.01), NaN kept
    m.Fx = m.Fy = m.Fz = R(0);
    if (flags & F_FORCE_CONST) { m.Fx = kn.fx; m.Fy = kn.fy; m.Fz = kn.fz; }
    if (flags & F_FORCE_FIELD) { const float4 fv = __ldg(p.force + n); m.Fx = R(fv.x); m.Fy = R(fv.y); m.Fz = R(fv.z); }
    R temperature = R(0);
    constexpr int QT = L::D == 2 ? 5 : 7;
    if (flags & F_THERMAL) {
        const R* th = th_src_of(p, R(0));
#pragma unroll
        for (int i = 0; i < QT; i++) temperature = FADD(temperature, __ldg(th + (uint64_t)i * p.stride + n));
        const R kb = FMUL(-kn.beta, FSUB(temperature, R(1)));  // buoyancy (collide.comp:709-716)
        m.Fx = FADD(m.Fx, FMUL(kb, m.Fx)); m.Fy = FADD(m.Fy, FMUL(kb, m.Fy)); m.Fz = FADD(m.Fz, FMUL(kb, m.Fz));
    }
    if (flags & F_MULTIPHASE) {  // collide.comp:534-584
        const R self_psi = psi_of(m.rho);
        const R* ps_src = psi_src_of(p, R(0));
        R sx, sy, sz;
        sc_sums_t<Q, C::SHIFTED, R>([&](const Dir c) -> R {
            int ax = x + c.x, ay = y + c.y, az = z + c.z;
            bool aopen;
            coords_wrap<Q>(ax, ay, az, nx, ny, nz, aopen, flags);
            return aopen ? self_psi
                         : __ldg(ps_src + (uint32_t)ax + (uint32_t)nx * ((uint32_t)ay + (uint32_t)ny * (uint32_t)az));
        }, sx, sy, sz);
        const R ks = FMUL(-self_psi, kn.G);
        m.Fx = FADD(m.Fx, FMUL(sx, ks)); m.Fy = FADD(m.Fy, FMUL(sy, ks)); m.Fz = FADD(m.Fz, FMUL(sz, ks));
    }
    const bool forced = (flags & (F_FORCE_CONST | F_FORCE_FIELD | F_THERMAL | F_MULTIPHASE)) != 0;
    if constexpr (C::SHIFTED) velocity_and_limit<Q>(f, m, forced, p.vlim, p.t_lim, p.t_ext);
    else velocity_literal<Q>(f, m, forced, kn.vlim, kn.t_lim, kn.t_ext);
    if (eqb) {
        const int kind = __ldg(p.obj_kind + bid);
        if (kind == 1) { m.ux = R(bv.y); m.uy = R(bv.z); m.uz = R(bv.w); } else { m.rho = R(bv.x); }
        m.Fx = m.Fy = m.Fz = R(0);
    }

    // ---- collision + AA store (collide.comp:727-760) ----
    if (flags & F_UPDATE) {
        // 16-bit multiphase flow: the mass-conserving rounding (collided_sum;
        // an equilibrium boundary cell's populations sum to rho - 1); rest is
        // T less the stored values of the populations emitted so far, written or not
        const bool carry_on = C::SHIFTED && (flags & F_MULTIPHASE);
        R rest = R(0);
        if (carry_on) rest = eqb ? FSUB(m.rho, R(1)) : collided_sum<0>(m);
        auto store = [&](int i, T h) {
            const Dir c = L::c(i);
            if (MODE == AA_EVEN) {
                int dx = x + c.x, dy = y + c.y, dz = z + c.z;
                bool dopen;
                coords_wrap<Q>(dx, dy, dz, nx, ny, nz, dopen, flags);
                if (!dopen)
                    plane(opp(i))[(uint32_t)dx + (uint32_t)nx * ((uint32_t)dy + (uint32_t)ny * (uint32_t)dz)] = h;
            } else {
                plane(i)[n] = h;
            }
        };
        collide_emit<Q, C::SHIFTED>(f, m, k, (flags & F_TRT) != 0, (flags & F_SOURCE) != 0, eqb, [&](int i, R v) {
            const R w = W::w(i);
            if (carry_on) {
                if (i == Q - 1) return;  // stored after the collision, from rest
                const T h = C::enc(v, w);
                rest = FSUB(rest, C::dec(h, w));
                store(i, h);
            } else {
                store(i, C::enc(v, w));
            }
        });
        if (carry_on) store(Q - 1, C::enc(rest, W::w(Q - 1)));
    }

    if ((flags & F_MULTIPHASE) && !(flags & F_MEASURE)) {  // collide.comp:763-769, psi of the effective density
        R eff = m.rho;
        if (bid != 0u) eff = R(__ldg(p.objects + 3u * bid + 2u).w);
        psi_tgt_of(p, R(0))[n] = psi_of(eff);
    }
    if ((flags & F_THERMAL) && !(flags & F_MEASURE)) thermal_collide_r<Q>(p, n, m, temperature, k, kn.tau_t);  // :771-782
    if (flags & F_SAVE) {  // collide.comp:784-792
        p.vel_den[n] = make_float4((float)m.ux, (float)m.uy, (float)m.uz, (float)m.rho);
        p.force_temp[n] = make_float4((float)m.Fx, (float)m.Fy, (float)m.Fz, (float)temperature);
        if (p.bnd_tex) p.bnd_tex[n] = (uint8_t)bid;
    }
    if (flags & F_REDUCE) {
        const R uu = uu_of(m.ux, m.uy, m.uz);
        out.m = m.rho; out.px = m.rho * m.ux; out.py = m.rho * m.uy; out.pz = m.rho * m.uz;
        out.ke = R(0.5f) * m.rho * uu;
    }
    return out;
}

template <int Q, int ST, int MODE>
__global__ void __launch_bounds__(kStepBlock) step_kernel(const __grid_constant__ StepParams p) {
    using R = typename Codec<ST>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    CellSumT<R> cs = {R(0), R(0), R(0), R(0), R(0)};
    if (x < p.nx) cs = cell_update<Q, ST, MODE>(p, x, blockIdx.y, blockIdx.z);
    if (p.flags & F_REDUCE) block_reduce_store(cs, p.red_partials);
}

// ---------------------------------------------------------------------------
// two-buffer pull streaming (stream.comp main, :498-584)
// ---------------------------------------------------------------------------
template <int Q, int ST>
__global__ void __launch_bounds__(kStepBlock) stream_kernel(const __grid_constant__ StreamParams p) {
    using L = Lattice<Q>;
    using C = Codec<ST>;
    using T = typename C::T;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= p.nx) return;
    const T* __restrict__ src = static_cast<const T*>(p.src);
    T* __restrict__ dst = static_cast<T*>(p.dst);
    const uint64_t S = p.stride;
    const uint32_t n = (uint32_t)x + (uint32_t)p.nx * ((uint32_t)y + (uint32_t)p.ny * (uint32_t)z);
    if (p.flags & F_BOUNDARIES) {
        if (solid_id(p.obj_kind, boundary_id(p.bnd, p.bits, n))) return;
    }
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const Dir c = L::c(i);
        const float w = L::w(i);
        int sx = x - c.x, sy = y - c.y, sz = z - c.z;
        bool open;
        coords_wrap<Q>(sx, sy, sz, p.nx, p.ny, p.nz, open, p.flags);
        if (open) { dst[(uint64_t)i * S + n] = C::enc(C::SHIFTED ? __fsub_rn(0.01f, w) : 0.01f, w); continue; }
        const uint32_t sn = (uint32_t)sx + (uint32_t)p.nx * ((uint32_t)sy + (uint32_t)p.ny * (uint32_t)sz);
        uint32_t sid = (p.flags & F_BOUNDARIES) ? boundary_id(p.bnd, p.bits, sn) : 0u;
        if (sid != 0u && solid_id(p.obj_kind, sid)) {
            const int inv = opp(i);
            const Dir ci = L::c(inv);
            const float4 uw = __ldg(p.objects + 3u * sid);
            const float corr = __fmul_rn(__fmul_rn(-2.f * L::w(inv), ci.x * uw.x + ci.y * uw.y + ci.z * uw.z), 3.f);
            dst[(uint64_t)i * S + n] = C::enc(__fadd_rn(C::dec(src[(uint64_t)inv * S + n], L::w(inv)), corr), w);
        } else {
            dst[(uint64_t)i * S + n] = src[(uint64_t)i * S + sn];
        }
    }
}

// ---------------------------------------------------------------------------
// thermal pull streaming (stream_thermal.comp main, :457-526), SoA layout
// ---------------------------------------------------------------------------
template <int QT, class R>
__global__ void __launch_bounds__(kStepBlock) stream_thermal_kernel(const __grid_constant__ ThermalStreamParams p) {
    using TL = ThermalLattice<QT>;
    // the thermal lattice in the arithmetic type (double: the FP64 stepper)
    const R* __restrict__ src = sizeof(R) == 8 ? reinterpret_cast<const R*>(p.src64) : reinterpret_cast<const R*>(p.src);
    R* __restrict__ dst = sizeof(R) == 8 ? reinterpret_cast<R*>(p.dst64) : reinterpret_cast<R*>(p.dst);
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= p.nx) return;
    const uint64_t S = p.stride;
    const uint32_t n = (uint32_t)x + (uint32_t)p.nx * ((uint32_t)y + (uint32_t)p.ny * (uint32_t)z);
    if (p.nmask) {
        const uint32_t m = __ldg(p.nmask + n);
        if (m >> 31) return;  // solid cell
        if ((m & ((1u << QT) - 2u)) == 0u) {
            // every source in the domain and fluid: the plain pull, no
            // boundary lookups (periodic wrap only where the domain wraps)
#pragma unroll
            for (int i = 0; i < QT; i++) {
                const Dir c = TL::c(i);
                int sx = x - c.x, sy = y - c.y, sz = z - c.z;
                bool open;
                coords_wrap<QT>(sx, sy, sz, p.nx, p.ny, p.nz, open, p.flags);
                const uint32_t sn = (uint32_t)sx + (uint32_t)p.nx * ((uint32_t)sy + (uint32_t)p.ny * (uint32_t)sz);
                dst[(uint64_t)i * S + n] = __ldg(src + (uint64_t)i * S + sn);
            }
            return;
        }
    } else if (p.flags & F_BOUNDARIES) {
        if (solid_id(p.obj_kind, boundary_id(p.bnd, p.bits, n))) return;
    }
#pragma unroll
    for (int i = 0; i < QT; i++) {
        const Dir c = TL::c(i);
        int sx = x - c.x, sy = y - c.y, sz = z - c.z;
        bool open;
        coords_wrap<QT>(sx, sy, sz, p.nx, p.ny, p.nz, open, p.flags);
        if (open) continue;  // no write (stream_thermal.comp:481-503)
        const uint32_t sn = (uint32_t)sx + (uint32_t)p.nx * ((uint32_t)sy + (uint32_t)p.ny * (uint32_t)sz);
        uint32_t sid = (p.flags & F_BOUNDARIES) ? boundary_id(p.bnd, p.bits, sn) : 0u;
        if (sid != 0u && solid_id(p.obj_kind, sid)) {
            const int inv = (i == 0) ? 0 : ((i & 1) ? i + 1 : i - 1);
            const R Tw = R(__ldg(p.objects + 3u * sid).w);
            // -g_opp + 2 w_opp T_wall (stream_thermal.comp:440-447, :520-522)
            dst[(uint64_t)i * S + n] = FADD(-__ldg(src + (uint64_t)inv * S + n), FMUL(R(2) * ThermalW<QT, R>::w(inv), Tw));
        } else {
            dst[(uint64_t)i * S + n] = __ldg(src + (uint64_t)i * S + sn);
        }
    }
}

// ---------------------------------------------------------------------------
// equilibrium initialisation (set_equilibrium_populations.comp:179-221)
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R feq_init_dot(R ax, R ay, R az, R bx, R by, R bz) {
    return r_add(r_add(r_mul(ax, bx), r_mul(ay, by)), r_mul(az, bz));
}
template <class R>
__device__ __forceinline__ R feq_init_literal(R w, R r, R cu, R uu) {
    R a = r_add(R(1), r_mul(R(3), cu));
    a = r_add(a, r_div(r_mul(R(9), r_mul(cu, cu)), R(2)));
    a = r_sub(a, r_div(r_mul(R(3), uu), R(2)));
    return r_mul(r_mul(w, r), a);
}

template <int Q, int ST>
__global__ void init_kernel(const __grid_constant__ InitParams p) {
    using L = Lattice<Q>;
    using C = Codec<ST>;
    using T = typename C::T;
    using R = typename C::R;
    const uint64_t n = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (n >= p.n_cells) return;
    T* F = static_cast<T*>(p.f);
    const R r = p.rho ? R(p.rho[n]) : R(1);
    R ux = R(0), uy = R(0), uz = R(0);
    const uint32_t id = p.ids ? p.ids[n] : 0u;
    const bool solid = id != 0u && p.obj_kind[id] == 0;
    if (p.u && !solid) { ux = p.u[3 * n]; uy = p.u[3 * n + 1]; uz = p.u[3 * n + 2]; }
    // w*rho*(1 + 3*cu + 9*cu^2/2 - 3*uu/2) with the shader's literal constants
    // and operation order, rounded operations only (init runs once)
    const R uu = feq_init_dot(ux, uy, uz, ux, uy, uz);
    if (!p.odd) {
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const Dir c = L::c(i);
            const R w = LatticeW<Q, R>::w(i);
            const R cu = feq_init_dot(R(c.x), R(c.y), R(c.z), ux, uy, uz);
            F[i * p.stride + n] = C::enc_f(feq_init_literal(w, r, cu, uu), w);
        }
        return;
    }
    const int x = (int)(n % (uint64_t)p.nx), y = (int)((n / (uint64_t)p.nx) % (uint64_t)p.ny),
              z = (int)(n / ((uint64_t)p.nx * (uint64_t)p.ny));
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const Dir c = L::c(i);
        const R w = LatticeW<Q, R>::w(i);
        const R cu = feq_init_dot(R(c.x), R(c.y), R(c.z), ux, uy, uz);
        const T v = C::enc_f(feq_init_literal(w, r, cu, uu), w);
        // destination n + c_i: read there as population i at the odd step
        int dx = x + c.x, dy = y + c.y, dz = z + c.z;
        bool dopen;
        coords_wrap<Q>(dx, dy, dz, p.nx, p.ny, p.nz, dopen, p.flags);
        if (!dopen)
            F[(uint64_t)opp(i) * p.stride + (uint64_t)dx + (uint64_t)p.nx * ((uint64_t)dy + (uint64_t)p.ny * (uint64_t)dz)] = v;
        int sx = x - c.x, sy = y - c.y, sz = z - c.z;
        bool sopen;
        coords_wrap<Q>(sx, sy, sz, p.nx, p.ny, p.nz, sopen, p.flags);
        if (sopen) {
            // slot opp(i) of n is read as population i, whose source n - c_i is
            // outside: it holds the cell's own population opp(i)
            const int o = opp(i);
            const Dir co = L::c(o);
            const R wo = LatticeW<Q, R>::w(o);
            const R cuo = feq_init_dot(R(co.x), R(co.y), R(co.z), ux, uy, uz);
            F[(uint64_t)o * p.stride + n] = C::enc_f(feq_init_literal(wo, r, cuo, uu), wo);
        }
    }
}

template <int QT, class R>
__global__ void init_thermal_kernel(const __grid_constant__ InitParams p) {
    using TL = ThermalLattice<QT>;
    const uint64_t n = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (n >= p.n_cells) return;
    const R t = p.T ? R(p.T[n]) : R(1);
    if (t == R(0)) return;  // set_equilibrium_populations_thermal.comp:171-172
    R ux = R(0), uy = R(0), uz = R(0);
    const uint32_t id = p.ids ? p.ids[n] : 0u;
    const bool solid = id != 0u && p.obj_kind[id] == 0;
    if (p.u && !solid) { ux = R(p.u[3 * n]); uy = R(p.u[3 * n + 1]); uz = R(p.u[3 * n + 2]); }
    const R uu = feq_init_dot(ux, uy, uz, ux, uy, uz);
    R* th = sizeof(R) == 8 ? reinterpret_cast<R*>(p.th64) : reinterpret_cast<R*>(p.th);
#pragma unroll
    for (int i = 0; i < QT; i++) {
        const Dir c = TL::c(i);
        const R cu = feq_init_dot(R(c.x), R(c.y), R(c.z), ux, uy, uz);
        th[i * p.stride + n] = feq_init_literal(ThermalW<QT, R>::w(i), t, cu, uu);
    }
}

// decode / encode the whole DDF (readback, snapshots)
template <int Q, int ST>
__global__ void decode_kernel(const void* f, uint64_t stride, uint32_t n_cells, float* out) {
    using C = Codec<ST>;
    using T = typename C::T;
    const uint64_t n = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (n >= n_cells) return;
    const T* F = static_cast<const T*>(f);
#pragma unroll
    for (int i = 0; i < Q; i++)
        out[(uint64_t)i * n_cells + n] = (float)C::dec_f(F[(uint64_t)i * stride + n], LatticeW<Q, typename C::R>::w(i));
}
template <int Q, int ST>
__global__ void encode_kernel(void* f, uint64_t stride, uint32_t n_cells, const float* in) {
    using C = Codec<ST>;
    using T = typename C::T;
    const uint64_t n = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (n >= n_cells) return;
    T* F = static_cast<T*>(f);
#pragma unroll
    for (int i = 0; i < Q; i++)
        F[(uint64_t)i * stride + n] = C::enc_f(in[(uint64_t)i * n_cells + n], LatticeW<Q, typename C::R>::w(i));
}

}  // namespace bf
#include "lbm_tma.cuh"
namespace bf {

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
inline dim3 cell_grid(int nx, int ny, int nz, int& block) {
    block = nx >= kStepBlock ? kStepBlock : ((nx + 31) / 32) * 32;
    return dim3((unsigned)((nx + block - 1) / block), (unsigned)ny, (unsigned)nz);
}

// persistent grid of the staged kernel: every SM filled with resident blocks
template <int Q, int ST, int MODE, bool TRT, bool FORCED>
cudaError_t launch_tma(const StepParams& p, cudaStream_t st) {
    auto kernel = tma_step_kernel<Q, ST, MODE, TRT, FORCED>;
    constexpr size_t smem = tma_smem_bytes<Q, ST>();
    static int per_sm = -1, sms = 0;  // per instantiation, first device
    if (per_sm < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTmaTile, smem);
        if (per_sm < 1) per_sm = 1;
    }
    const uint32_t tiles = ((uint32_t)p.nx / kTmaTile) * (uint32_t)p.ny * (uint32_t)p.nz;
    const uint32_t blocks = std::min<uint32_t>(tiles, (uint32_t)(sms * per_sm));
    kernel<<<blocks, kTmaTile, smem, st>>>(p);
    return cudaGetLastError();
}

template <int Q, int ST>
cudaError_t launch_step_st(const StepParams& p, int mode, int path, cudaStream_t st) {
    int block;
    dim3 grid = cell_grid(p.nx, p.ny, p.nz, block);
    const bool generic = path != PATH_FAST;
    if constexpr (ST != ST_FP64) {
        if (path == PATH_MASKED && mode != AA_LOCAL) {
            const bool trt = (p.flags & F_TRT) != 0, forced = (p.flags & F_FORCE_CONST) != 0;
            const bool thermal = (p.flags & F_THERMAL) != 0;
            if (p.special && p.sched && !(p.flags & F_REDUCE)) {
                const unsigned total = p.n_sched;
#define BF_MIXED(MODE_, TRT_, F_, TH_) masked_mixed_kernel<Q, ST, MODE_, TRT_, F_, TH_><<<total, block, 0, st>>>(p)
#define BF_MIXED_MODE(MODE_)                                                                                          \
    if (thermal) { if (trt) BF_MIXED(MODE_, true, true, true); else BF_MIXED(MODE_, false, true, true); }              \
    else if (trt) { if (forced) BF_MIXED(MODE_, true, true, false); else BF_MIXED(MODE_, true, false, false); }       \
    else { if (forced) BF_MIXED(MODE_, false, true, false); else BF_MIXED(MODE_, false, false, false); }
                if (mode == AA_EVEN) { BF_MIXED_MODE(AA_EVEN) }
                else { BF_MIXED_MODE(AA_ODD) }
#undef BF_MIXED_MODE
#undef BF_MIXED
                return cudaGetLastError();
            }
#define BF_MASKED(MODE_, TRT_, F_, TH_) masked_step_kernel<Q, ST, MODE_, TRT_, F_, TH_><<<grid, block, 0, st>>>(p)
#define BF_MASKED_MODE(MODE_)                                                                       \
    if (thermal) { if (trt) BF_MASKED(MODE_, true, true, true); else BF_MASKED(MODE_, false, true, true); } \
    else if (trt) { if (forced) BF_MASKED(MODE_, true, true, false); else BF_MASKED(MODE_, true, false, false); } \
    else { if (forced) BF_MASKED(MODE_, false, true, false); else BF_MASKED(MODE_, false, false, false); }
            if (mode == AA_EVEN) { BF_MASKED_MODE(AA_EVEN) }
            else { BF_MASKED_MODE(AA_ODD) }
#undef BF_MASKED_MODE
#undef BF_MASKED
            return cudaGetLastError();
        }
    }
    // staged loads: 16-bit storage, an update step without reduction or
    // multiphase, whole 256-cell tiles per row, 16-byte aligned planes
    if constexpr (ST == ST_FP16S) {  // the staged variant exists for fp16s only
        if (!generic && p.tma && (p.flags & F_UPDATE) && !(p.flags & (F_REDUCE | F_MULTIPHASE)) &&
            p.nx % kTmaTile == 0 && reinterpret_cast<uintptr_t>(p.plane[0]) % 16 == 0) {
            const bool trt = (p.flags & F_TRT) != 0, forced = (p.flags & F_FORCE_CONST) != 0;
            if (mode == AA_EVEN) {
                if (trt) return forced ? launch_tma<Q, ST, AA_EVEN, true, true>(p, st) : launch_tma<Q, ST, AA_EVEN, true, false>(p, st);
                return forced ? launch_tma<Q, ST, AA_EVEN, false, true>(p, st) : launch_tma<Q, ST, AA_EVEN, false, false>(p, st);
            }
            if (trt) return forced ? launch_tma<Q, ST, AA_ODD, true, true>(p, st) : launch_tma<Q, ST, AA_ODD, true, false>(p, st);
            return forced ? launch_tma<Q, ST, AA_ODD, false, true>(p, st) : launch_tma<Q, ST, AA_ODD, false, false>(p, st);
        }
    }
    // two cells per thread: 16-bit update steps without reduction or multiphase, even nx
    if constexpr ((ST == ST_FP16S || ST == ST_FP16C) && Q != 27) {
        if (!generic && p.two_cell && (p.flags & F_UPDATE) && !(p.flags & F_REDUCE) && p.nx % 2 == 0) {
            // one block spans a row where the row is shorter than 2 x kStepBlock cells
            const int threads = min(kStepBlock, (p.nx / 2 + 31) / 32 * 32);
            const dim3 g2((unsigned)((p.nx / 2 + threads - 1) / threads), (unsigned)p.ny, (unsigned)p.nz);
            // multiphase flow is forced (the pseudopotential) with the source term on
            const bool trt = (p.flags & F_TRT) != 0, mp = (p.flags & F_MULTIPHASE) != 0;
            const bool forced = (p.flags & F_FORCE_CONST) != 0 || mp;
            // the Shan-Chen variant with the psi rows staged by bulk copies
            // (p.psi_tile): one block per row (nx <= 2 x kStepBlock) and rows
            // of whole 16-byte units (nx % 4 == 0); ROWS x nx floats
            const bool tile = mp && p.psi_tile && g2.x == 1u && p.nx % 4 == 0;
            const size_t tile_bytes = tile ? (size_t)kPsiRows<Q> * (size_t)p.nx * sizeof(float) : 0;
#define BF_FAST2(MODE_, TRT_, F_, MP_) fast2_step_kernel<Q, ST, MODE_, TRT_, F_, MP_, false><<<g2, threads, tile_bytes, st>>>(p)
#define BF_FAST2T(MODE_, TRT_) fast2_step_kernel<Q, ST, MODE_, TRT_, true, true, true><<<g2, threads, tile_bytes, st>>>(p)
#define BF_FAST2_MODE(MODE_)                                                                                  \
    if (tile) { if (trt) BF_FAST2T(MODE_, true); else BF_FAST2T(MODE_, false); }                              \
    else if (mp) { if (trt) BF_FAST2(MODE_, true, true, true); else BF_FAST2(MODE_, false, true, true); }     \
    else if (trt) { if (forced) BF_FAST2(MODE_, true, true, false); else BF_FAST2(MODE_, true, false, false); } \
    else { if (forced) BF_FAST2(MODE_, false, true, false); else BF_FAST2(MODE_, false, false, false); }
            if (mode == AA_EVEN) { BF_FAST2_MODE(AA_EVEN) }
            else { BF_FAST2_MODE(AA_ODD) }
#undef BF_FAST2_MODE
#undef BF_FAST2T
#undef BF_FAST2
            return cudaGetLastError();
        }
    }
    if (!generic) {
        // multiphase flow is forced (the pseudopotential) with the source term on
        const bool trt = (p.flags & F_TRT) != 0, mp = (p.flags & F_MULTIPHASE) != 0;
        const bool forced = (p.flags & F_FORCE_CONST) != 0 || mp;
        auto go = [&](auto kernel) { kernel<<<grid, block, 0, st>>>(p); };
#define BF_FAST(MODE_, TRT_, F_, MP_) go(fast_step_kernel<Q, ST, MODE_, TRT_, F_, MP_>)
        // the FP64 stepper's multiphase flow runs the generic kernel (path set by the host)
        if (ST == ST_FP64 && mp) return cudaErrorInvalidValue;
        constexpr bool MPX = ST != ST_FP64;  // no multiphase variants of the FP64 fast kernel
        if (mode == AA_EVEN) {
            if (mp) { if (trt) BF_FAST(AA_EVEN, true, true, MPX); else BF_FAST(AA_EVEN, false, true, MPX); }
            else if (trt) { if (forced) BF_FAST(AA_EVEN, true, true, false); else BF_FAST(AA_EVEN, true, false, false); }
            else { if (forced) BF_FAST(AA_EVEN, false, true, false); else BF_FAST(AA_EVEN, false, false, false); }
        } else {
            if (mp) { if (trt) BF_FAST(AA_ODD, true, true, MPX); else BF_FAST(AA_ODD, false, true, MPX); }
            else if (trt) { if (forced) BF_FAST(AA_ODD, true, true, false); else BF_FAST(AA_ODD, true, false, false); }
            else { if (forced) BF_FAST(AA_ODD, false, true, false); else BF_FAST(AA_ODD, false, false, false); }
        }
#undef BF_FAST
    } else {
        // the FP64 reference stepper runs the esoteric-pull modes only
        if (ST == ST_FP64 && mode == AA_LOCAL) return cudaErrorInvalidValue;  // rejected at initialisation
        if (mode == AA_EVEN) step_kernel<Q, ST, AA_EVEN><<<grid, block, 0, st>>>(p);
        else if (mode == AA_ODD) step_kernel<Q, ST, AA_ODD><<<grid, block, 0, st>>>(p);
        else if constexpr (ST != ST_FP64) step_kernel<Q, ST, AA_LOCAL><<<grid, block, 0, st>>>(p);
    }
    return cudaGetLastError();
}

template <int Q>
cudaError_t launch_step(const StepParams& p, int storage, int mode, int path, cudaStream_t st) {
    switch (storage) {
    case ST_FP32: return launch_step_st<Q, ST_FP32>(p, mode, path, st);
    case ST_FP16: return launch_step_st<Q, ST_FP16>(p, mode, path, st);
    case ST_FP16S: return launch_step_st<Q, ST_FP16S>(p, mode, path, st);
    case ST_FP16C: return launch_step_st<Q, ST_FP16C>(p, mode, path, st);
    case ST_FP64: return launch_step_st<Q, ST_FP64>(p, mode, path, st);
    }
    return cudaErrorInvalidValue;
}

template <int Q>
cudaError_t launch_build_mask(const StepParams& p, uint32_t* mask, cudaStream_t st) {
    int block;
    dim3 grid = cell_grid(p.nx, p.ny, p.nz, block);
    build_mask_kernel<Q><<<grid, block, 0, st>>>(p, mask);
    return cudaGetLastError();
}

template <int Q>
cudaError_t launch_stream(const StreamParams& p, int storage, cudaStream_t st) {
    int block;
    dim3 grid = cell_grid(p.nx, p.ny, p.nz, block);
    switch (storage) {
    case ST_FP32: stream_kernel<Q, ST_FP32><<<grid, block, 0, st>>>(p); break;
    case ST_FP16: stream_kernel<Q, ST_FP16><<<grid, block, 0, st>>>(p); break;
    case ST_FP16S: stream_kernel<Q, ST_FP16S><<<grid, block, 0, st>>>(p); break;
    case ST_FP16C: stream_kernel<Q, ST_FP16C><<<grid, block, 0, st>>>(p); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int Q>
cudaError_t launch_init(const InitParams& p, int storage, cudaStream_t st) {
    const unsigned blocks = (unsigned)((p.n_cells + 255u) / 256u);
    switch (storage) {
    case ST_FP32: init_kernel<Q, ST_FP32><<<blocks, 256, 0, st>>>(p); break;
    case ST_FP16: init_kernel<Q, ST_FP16><<<blocks, 256, 0, st>>>(p); break;
    case ST_FP16S: init_kernel<Q, ST_FP16S><<<blocks, 256, 0, st>>>(p); break;
    case ST_FP16C: init_kernel<Q, ST_FP16C><<<blocks, 256, 0, st>>>(p); break;
    case ST_FP64: init_kernel<Q, ST_FP64><<<blocks, 256, 0, st>>>(p); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int Q>
cudaError_t launch_decode(const void* f, uint64_t stride, uint32_t n, int storage, float* out, cudaStream_t st) {
    const unsigned blocks = (n + 255u) / 256u;
    switch (storage) {
    case ST_FP32: decode_kernel<Q, ST_FP32><<<blocks, 256, 0, st>>>(f, stride, n, out); break;
    case ST_FP16: decode_kernel<Q, ST_FP16><<<blocks, 256, 0, st>>>(f, stride, n, out); break;
    case ST_FP16S: decode_kernel<Q, ST_FP16S><<<blocks, 256, 0, st>>>(f, stride, n, out); break;
    case ST_FP16C: decode_kernel<Q, ST_FP16C><<<blocks, 256, 0, st>>>(f, stride, n, out); break;
    case ST_FP64: decode_kernel<Q, ST_FP64><<<blocks, 256, 0, st>>>(f, stride, n, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
template <int Q>
cudaError_t launch_encode(void* f, uint64_t stride, uint32_t n, int storage, const float* in, cudaStream_t st) {
    const unsigned blocks = (n + 255u) / 256u;
    switch (storage) {
    case ST_FP32: encode_kernel<Q, ST_FP32><<<blocks, 256, 0, st>>>(f, stride, n, in); break;
    case ST_FP16: encode_kernel<Q, ST_FP16><<<blocks, 256, 0, st>>>(f, stride, n, in); break;
    case ST_FP16S: encode_kernel<Q, ST_FP16S><<<blocks, 256, 0, st>>>(f, stride, n, in); break;
    case ST_FP16C: encode_kernel<Q, ST_FP16C><<<blocks, 256, 0, st>>>(f, stride, n, in); break;
    case ST_FP64: encode_kernel<Q, ST_FP64><<<blocks, 256, 0, st>>>(f, stride, n, in); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// The step kernels of one (velocity set, storage) pair are instantiated in
// their own translation unit (generated by build.py, compiled in parallel);
// the velocity set's main unit declares them extern.
#define BF_INSTANTIATE_STEP(Q, ST) template cudaError_t launch_step_st<Q, ST>(const StepParams&, int, int, cudaStream_t);
#define BF_EXTERN_STEP(Q)                                                                                     \
    extern template cudaError_t launch_step_st<Q, ST_FP32>(const StepParams&, int, int, cudaStream_t);       \
    extern template cudaError_t launch_step_st<Q, ST_FP16>(const StepParams&, int, int, cudaStream_t);       \
    extern template cudaError_t launch_step_st<Q, ST_FP16S>(const StepParams&, int, int, cudaStream_t);      \
    extern template cudaError_t launch_step_st<Q, ST_FP16C>(const StepParams&, int, int, cudaStream_t);      \
    extern template cudaError_t launch_step_st<Q, ST_FP64>(const StepParams&, int, int, cudaStream_t);

#define BF_INSTANTIATE_Q(Q)                                                                                   \
    BF_EXTERN_STEP(Q)                                                                                         \
    template cudaError_t launch_step<Q>(const StepParams&, int, int, int, cudaStream_t);                     \
    template cudaError_t launch_build_mask<Q>(const StepParams&, uint32_t*, cudaStream_t);                   \
    template cudaError_t launch_stream<Q>(const StreamParams&, int, cudaStream_t);                           \
    template cudaError_t launch_init<Q>(const InitParams&, int, cudaStream_t);                               \
    template cudaError_t launch_decode<Q>(const void*, uint64_t, uint32_t, int, float*, cudaStream_t);        \
    template cudaError_t launch_encode<Q>(void*, uint64_t, uint32_t, int, const float*, cudaStream_t);

}  // namespace bf
