/*
 * lbm_oracle.c -- CPU restatement of BoltzmannFluids' per-timestep lattice
 * Boltzmann update.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py load this library as the
 * checker; the product (boltzmannfluids_gb300) never links or calls it.
 *
 * Parity status: the reference's shaders cannot run here (no graphics stack,
 * GraphicsCortex not vendored).  This restatement is pinned by
 *   - golden tables parsed from the reference's own source text
 *     (tests/golden/, generated by tests/golden/make_golden.py), and
 *   - oracle/build_ref.py, which compiles the reference's collide/stream
 *     shader sources as C++ on the host (oracle/_ref/) where that recipe
 *     succeeds; tests/test_oracle_vs_ref.py compares the two.
 * Without the second item the restatement is "parity unpinned".
 *
 * The file is compiled twice: REAL=float gives the FP32 stepper (the
 * shaders' expressions in their written order, no FMA contraction: bit for
 * bit the reference's shader code as the reference-built checker runs it),
 * REAL=double the FP64 accuracy oracle (orc64_* symbols, the same order in
 * double).
 *
 * Memory-level restatement: the DDF lives in one buffer with the reference's
 * SoA address  i*N + cell  (collide.comp:196-200), and every read/write goes
 * through the same AA index functions as collide.comp:244-369, so the
 * in-place esoteric-pull semantics (0.01 open-boundary reads, dropped
 * out-of-range writes, skipped solid cells) fall out exactly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif
#ifndef ORC
#define ORC(n) orc32_##n
#endif
#define IS_F32 (sizeof(REAL) == 4)

/* ------------------------------------------------------------------------ */
/* velocity sets: VelocitySet.cpp:53-142 (flow), :180-204 (thermal).         */
/* enum values follow VelocitySet.h:9-19.                                     */
/* ------------------------------------------------------------------------ */
enum { ORC_D2Q9 = 2, ORC_D3Q15 = 3, ORC_D3Q19 = 4, ORC_D3Q27 = 5 };
enum { ORC_STORE_FP32 = 0, ORC_STORE_FP16 = 1, ORC_STORE_FP16S = 2, ORC_STORE_FP16C = 3 };
enum { ORC_BOUNDARY_SKIP = 0, ORC_BOUNDARY_BOUNCE_BACK = 1 };
enum { ORC_BGK = 0, ORC_TRT = 1 };
enum { ORC_OBJ_SOLID = 0, ORC_OBJ_EQ_VELOCITY = 1, ORC_OBJ_EQ_DENSITY = 2 };

typedef struct { int cx, cy, cz; double w; } orc_dir;

static const orc_dir D2Q9_T[9] = {
    {0, 0, 0, 4.0 / 9}, {1, 0, 0, 1.0 / 9}, {-1, 0, 0, 1.0 / 9}, {0, 1, 0, 1.0 / 9}, {0, -1, 0, 1.0 / 9},
    {1, 1, 0, 1.0 / 36}, {-1, -1, 0, 1.0 / 36}, {1, -1, 0, 1.0 / 36}, {-1, 1, 0, 1.0 / 36}};
static const orc_dir D3Q15_T[15] = {
    {0, 0, 0, 2.0 / 9}, {1, 0, 0, 1.0 / 9}, {-1, 0, 0, 1.0 / 9}, {0, 1, 0, 1.0 / 9}, {0, -1, 0, 1.0 / 9},
    {0, 0, 1, 1.0 / 9}, {0, 0, -1, 1.0 / 9}, {1, 1, 1, 1.0 / 72}, {-1, -1, -1, 1.0 / 72}, {1, 1, -1, 1.0 / 72},
    {-1, -1, 1, 1.0 / 72}, {1, -1, 1, 1.0 / 72}, {-1, 1, -1, 1.0 / 72}, {-1, 1, 1, 1.0 / 72}, {1, -1, -1, 1.0 / 72}};
static const orc_dir D3Q19_T[19] = {
    {0, 0, 0, 1.0 / 3}, {1, 0, 0, 1.0 / 18}, {-1, 0, 0, 1.0 / 18}, {0, 1, 0, 1.0 / 18}, {0, -1, 0, 1.0 / 18},
    {0, 0, 1, 1.0 / 18}, {0, 0, -1, 1.0 / 18}, {1, 1, 0, 1.0 / 36}, {-1, -1, 0, 1.0 / 36}, {1, -1, 0, 1.0 / 36},
    {-1, 1, 0, 1.0 / 36}, {1, 0, 1, 1.0 / 36}, {-1, 0, -1, 1.0 / 36}, {1, 0, -1, 1.0 / 36}, {-1, 0, 1, 1.0 / 36},
    {0, 1, 1, 1.0 / 36}, {0, -1, -1, 1.0 / 36}, {0, 1, -1, 1.0 / 36}, {0, -1, 1, 1.0 / 36}};
static const orc_dir D3Q27_T[27] = {
    {0, 0, 0, 8.0 / 27}, {1, 0, 0, 2.0 / 27}, {-1, 0, 0, 2.0 / 27}, {0, 1, 0, 2.0 / 27}, {0, -1, 0, 2.0 / 27},
    {0, 0, 1, 2.0 / 27}, {0, 0, -1, 2.0 / 27}, {1, 1, 0, 1.0 / 54}, {-1, -1, 0, 1.0 / 54}, {1, 0, 1, 1.0 / 54},
    {-1, 0, -1, 1.0 / 54}, {0, 1, 1, 1.0 / 54}, {0, -1, -1, 1.0 / 54}, {1, -1, 0, 1.0 / 54}, {-1, 1, 0, 1.0 / 54},
    {1, 0, -1, 1.0 / 54}, {-1, 0, 1, 1.0 / 54}, {0, 1, -1, 1.0 / 54}, {0, -1, 1, 1.0 / 54}, {1, 1, 1, 1.0 / 216},
    {-1, -1, -1, 1.0 / 216}, {1, 1, -1, 1.0 / 216}, {-1, -1, 1, 1.0 / 216}, {1, -1, 1, 1.0 / 216},
    {-1, 1, -1, 1.0 / 216}, {-1, 1, 1, 1.0 / 216}, {1, -1, -1, 1.0 / 216}};
static const orc_dir D2Q5_T[5] = {
    {0, 0, 0, 1.0 / 3}, {1, 0, 0, 1.0 / 6}, {-1, 0, 0, 1.0 / 6}, {0, 1, 0, 1.0 / 6}, {0, -1, 0, 1.0 / 6}};
static const orc_dir D3Q7_T[7] = {
    {0, 0, 0, 1.0 / 4}, {1, 0, 0, 1.0 / 8}, {-1, 0, 0, 1.0 / 8}, {0, 1, 0, 1.0 / 8},
    {0, -1, 0, 1.0 / 8}, {0, 0, 1, 1.0 / 8}, {0, 0, -1, 1.0 / 8}};

/* ------------------------------------------------------------------------ */
/* 16-bit storage emulation                                                  */
/* ------------------------------------------------------------------------ */
/* IEEE binary32 -> binary16 with round-to-nearest-even (the conversion an
 * R16F imageStore is assumed to perform), then back to binary32. */
static uint16_t f32_to_f16_rne(float f) {
    uint32_t x; memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t mag = x & 0x7fffffffu;
    if (mag >= 0x7f800000u) return (uint16_t)(sign | (mag > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (mag >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to >= 65520 -> inf */
    if (mag < 0x38800000u) { /* result is subnormal or zero */
        if (mag < 0x33000000u) return (uint16_t)sign; /* < 2^-25 rounds to 0 (2^-25 ties to even 0) */
        uint32_t m = (mag & 0x7fffffu) | 0x800000u;
        int e = (int)(mag >> 23); /* 102..112 */
        int shift = 126 - e;      /* value = m * 2^(e-150); half sub unit 2^-24 */
        uint32_t q = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (q & 1u))) q++;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (mag >> 23) - 112u;
    uint32_t m = mag & 0x7fffffu;
    uint32_t q = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q++;
    return (uint16_t)(sign | q);
}
static float f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu, x;
    if (e == 0) {
        float v = (float)m * 5.9604644775390625e-08f; /* m * 2^-24, exact */
        return sign ? -v : v;
    }
    if (e == 31) x = sign | 0x7f800000u | (m << 13);
    else x = sign | ((e + 112u) << 23) | (m << 13);
    float f; memcpy(&f, &x, 4); return f;
}
/* custom-scaled 16-bit (fp16c): the IEEE half of g * 2^12, g = f - w.  The
 * scale keeps shifted populations in the half's normal range down to
 * |g| = 2^-26; decoding multiplies by 2^-12 (exact). */
#define C16_SCALE 4096.0f
static float c16_round(float g) { return f16_to_f32(f32_to_f16_rne(g * C16_SCALE)) * (1.0f / C16_SCALE); }

/* ------------------------------------------------------------------------ */
/* solver state                                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    int nx, ny, nz, velocity_set, storage, multiphase, esoteric;
    int periodic[3];
    float tau;
    int boundary_mode, collision;
    float trt_magic, velocity_limit, velocity_limit_extreme;
    float G, tau_t, beta;
    int thermal_init_equilibrium;  /* 0: as read (lattice left at zero), 1: equilibrium */
    int two_buffer_fixed;          /* 0: as read (double swap), 1: collide -> stream */
} orc_desc;

typedef struct {
    orc_desc d;
    int Q, Qt, dims;
    size_t N;
    const orc_dir* V;
    const orc_dir* Vt;
    REAL cs;
    /* launch constants, computed once per launch as the host does: the
     * shifted tree multiplies by the correctly rounded reciprocals, the
     * literal tree divides by cs2, cs4, tau, tau_t (see the note below). */
    REAL R2, R4, R2h, R4h, Rtau, P, Rtau_t, Wm, Pp, Pm;
    REAL cs2, cs4, tau, tau_t;  /* the literal evaluation divides by these */
    int forced; /* force term in u: forcing, thermal or multiphase */
    REAL* lat[2];
    int lat0_src;
    uint32_t* boundries;
    int bits, nobj;
    float* objects;   /* 12 floats per id: (u,T) (omega,0) (com,rho_eff) as LBM.cpp:613-626 */
    int* obj_kind;
    int forcing, constant_force, thermal, src_on;
    REAL fconst[3];
    float* forces;    /* N*4 */
    REAL* th[2];
    int th0_src;
    REAL* mp[2];
    int mp0_src;
    float* bvals;     /* N*4 (rho_b, u_b) for equilibrium boundary cells */
    REAL* vel_den;    /* N*4 */
    REAL* force_temp; /* N*4 */
    float* bnd_tex;   /* N */
    long ticks;
} orc_t;

typedef struct { REAL x, y, z; } v3;
static v3 mk3(REAL x, REAL y, REAL z) { v3 r = {x, y, z}; return r; }
static REAL dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* DDF storage emulation.  The lattice array holds what the device stores,
 * decoded to a float: f itself for fp32 and fp16 (rounded to half);
 * the shifted population g = f - w (rounded to half) for fp16s; g rounded
 * through the scaled half for fp16c.  The shifted storages run the update
 * on g (see collide), as the kernels do. */
static int shifted(const orc_t* s) {
    return IS_F32 && (s->d.storage == ORC_STORE_FP16S || s->d.storage == ORC_STORE_FP16C);
}
/* stored value of slot i -> the value the update works on (g when shifted) */
static REAL lat_load(const orc_t* s, REAL raw, int i) {
    (void)s; (void)i;
    return raw;
}
/* value the update produced -> stored value */
static REAL lat_store(const orc_t* s, REAL v, int i) {
    if (!IS_F32) return v;
    switch (s->d.storage) {
    case ORC_STORE_FP16:
    case ORC_STORE_FP16S: return (REAL)f16_to_f32(f32_to_f16_rne((float)v));
    case ORC_STORE_FP16C: return (REAL)c16_round((float)v);
    default: return v;
    }
}
/* population f -> stored value (initialisation, set_lattice) */
static REAL lat_from_f(const orc_t* s, REAL f, int i) {
    if (shifted(s)) {
        float w = (float)s->V[i].w;
        if (s->d.storage == ORC_STORE_FP16S) return (REAL)f16_to_f32(f32_to_f16_rne((float)f - w));
        return (REAL)c16_round((float)f - w);
    }
    return lat_store(s, f, i);
}
/* stored value -> population f (get_lattice) */
static REAL lat_to_f(const orc_t* s, REAL raw, int i) {
    if (!shifted(s)) return raw;
    float w = (float)s->V[i].w;
    return (REAL)((float)raw + w);
}

static int opp(int i) { /* collide.comp:219-222 */
    int r = (i % 2 == 1) ? i + 1 : i - 1;
    return r < 0 ? 0 : r;
}
static int opp_t(int i, int Qt) { /* stream_thermal.comp:249-255 */
    if (i == 0 || i >= Qt) return 0;
    return (i % 2 == 1) ? i + 1 : i - 1;
}
static int pmod(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }

static size_t cid(const orc_t* s, int x, int y, int z) { return ((size_t)z * s->d.ny + y) * s->d.nx + x; }

static uint32_t get_boundry(const orc_t* s, size_t cell) { /* collide.comp:401-418 */
    if (s->nobj <= 1) return 0;
    uint64_t bits_begin = (uint64_t)cell * (uint64_t)s->bits;
    uint64_t dw = bits_begin / 32;
    uint32_t sub = (uint32_t)(bits_begin % 32);
    uint32_t mask = (1u << s->bits) - 1u;
    return (s->boundries[dw] & (mask << sub)) >> sub;
}
static int is_solid(const orc_t* s, uint32_t id) {
    return id != 0 && s->obj_kind[id] == ORC_OBJ_SOLID;
}

/* wrap / open-boundary test shared by all neighbour lookups (collide.comp:278-295) */
static int wrap(const orc_t* s, int* x, int* y, int* z) {
    int open = 0;
    if (s->d.periodic[0]) *x = pmod(*x, s->d.nx); else open |= (*x < 0 || *x >= s->d.nx);
    if (s->d.periodic[1]) *y = pmod(*y, s->d.ny); else open |= (*y < 0 || *y >= s->d.ny);
    if (s->d.periodic[2]) *z = pmod(*z, s->d.nz); else open |= (*z < 0 || *z >= s->d.nz);
    return open;
}

static REAL* LSRC(orc_t* s) { return s->lat[s->lat0_src ? 0 : 1]; }
static REAL* LTGT(orc_t* s) { return s->lat[s->lat0_src ? 1 : 0]; }
static REAL* TSRC(orc_t* s) { return s->th[s->th0_src ? 0 : 1]; }
static REAL* TTGT(orc_t* s) { return s->th[s->th0_src ? 1 : 0]; }
static REAL* MSRC(orc_t* s) { return s->mp[s->mp0_src ? 0 : 1]; }
static REAL* MTGT(orc_t* s) { return s->mp[s->mp0_src ? 1 : 0]; }

/* AA read address (collide.comp:244-305): returns 0 and fills (cell,slot),
 * or returns 1 for an open-boundary read. */
static int aa_read_addr(orc_t* s, int x, int y, int z, int i, int odd, size_t* cell, int* slot) {
    int rx = x, ry = y, rz = z, ri = i;
    if (s->d.esoteric) {
        if (!odd) { rx = x - s->V[i].cx; ry = y - s->V[i].cy; rz = z - s->V[i].cz; ri = i; }
        else { ri = opp(i); }
    }
    if (wrap(s, &rx, &ry, &rz)) return 1;
    *cell = cid(s, rx, ry, rz); *slot = ri;
    return 0;
}
/* AA write address (collide.comp:307-369) */
static int aa_write_addr(orc_t* s, int x, int y, int z, int i, int odd, size_t* cell, int* slot) {
    int wx = x, wy = y, wz = z, wi = i;
    if (s->d.esoteric) {
        if (!odd) { wi = opp(i); wx = x - s->V[wi].cx; wy = y - s->V[wi].cy; wz = z - s->V[wi].cz; }
        else { wi = i; }
    }
    if (wrap(s, &wx, &wy, &wz)) return 1;
    *cell = cid(s, wx, wy, wz); *slot = wi;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* physics (collide.comp:512-629, :634-673)                                  */
/* ------------------------------------------------------------------------ */
/*
 * Two evaluations, each shared bit for bit with the CUDA kernels.
 *
 * Literal (FP32 and FP16 storage of f itself, and the FP64 oracle): the
 * reference's expressions (collide.comp:383-395, :512-629, :634-673,
 * :702-782) in the order they are written, one IEEE operation per operator,
 * divisions as correctly rounded divisions, no contraction (the file is
 * compiled with -ffp-contract=off).  Products with a lattice component
 * (0 or +-1) are exact and the zero terms of such dot products are left
 * out (cdot below), which changes nothing but the sign of a zero.
 *
 * Shifted (fp16s / fp16c, extensions with no counterpart in the reference):
 * the update on g = f - w in a fixed order where divisions by launch
 * uniforms (cs^2, cs^4, tau) are multiplications by their once-rounded
 * reciprocals, u = j * (1/rho) with one IEEE division, and the sums marked
 * FMA are single-rounding fused multiply-adds.  The TRT collision (an
 * extension) uses the same fixed order with either storage.
 */
#define FMA(a, b, c) (IS_F32 ? (REAL)fmaf((float)(a), (float)(b), (float)(c)) : (REAL)fma((double)(a), (double)(b), (double)(c)))
/* u.u = fma(uz, uz, fma(uy, uy, ux*ux)) */
static REAL uu_of(v3 u) { return FMA(u.z, u.z, FMA(u.y, u.y, u.x * u.x)); }
/* c . v for c in {-1,0,1}^3: the nonzero terms summed in x, y, z order */
static REAL cdot(int cx, int cy, int cz, v3 v) {
    REAL acc = 0; int first = 1;
    if (cx) { acc = cx > 0 ? v.x : -v.x; first = 0; }
    if (cy) { REAL t = cy > 0 ? v.y : -v.y; acc = first ? t : acc + t; first = 0; }
    if (cz) { REAL t = cz > 0 ? v.z : -v.z; acc = first ? t : acc + t; first = 0; }
    return acc;
}
/* (1 + cu/cs2 + cu^2/2/cs4 - uu/2/cs2) = fma(cu^2, R4/2, fma(cu, R2, 1 - uu R2/2)) */
static REAL bracket(const orc_t* s, REAL cu, REAL one_m) { return FMA(cu * cu, s->R4h, FMA(cu, s->R2, one_m)); }
/* collide.comp:589-604 as written: (w p)(((1 + cu/cs2) + cu^2/2/cs4) - uu/2/cs2),
 * uuh = (u.u/2)/cs2 of the cell; the thermal form (:634-651) is the same with T */
static REAL feq_lit(const orc_t* s, REAL wp, REAL cu, REAL uuh) {
    return wp * ((((REAL)1 + cu / s->cs2) + (cu * cu / (REAL)2) / s->cs4) - uuh);
}
static REAL feq_init(const orc_t* s, REAL rho, v3 u, int i) { /* set_equilibrium_populations.comp:179-196 */
    REAL w = (REAL)s->V[i].w;
    v3 c = mk3((REAL)s->V[i].cx, (REAL)s->V[i].cy, (REAL)s->V[i].cz);
    REAL cu = dot3(c, u);
    REAL cu2 = cu * cu;
    REAL uu = dot3(u, u);
    return w * rho * ((REAL)1 + (REAL)3 * cu + (REAL)9 * cu2 / (REAL)2 - (REAL)3 * uu / (REAL)2);
}
static REAL feq_t_init(const orc_t* s, REAL T, v3 u, int i) { /* set_equilibrium_populations_thermal.comp:139-156 */
    REAL w = (REAL)s->Vt[i].w;
    v3 c = mk3((REAL)s->Vt[i].cx, (REAL)s->Vt[i].cy, (REAL)s->Vt[i].cz);
    REAL cu = dot3(c, u);
    REAL cu2 = cu * cu;
    REAL uu = dot3(u, u);
    return w * T * ((REAL)1 + (REAL)3 * cu + (REAL)9 * cu2 / (REAL)2 - (REAL)3 * uu / (REAL)2);
}
/* exp for the FP32 pseudopotential, identical to the CUDA kernels' copy:
 * Cody-Waite reduction x = k ln2 + r with ln2 split in a 15-bit head (exact
 * products for |k| < 2^9) and a tail, exp(r) by the degree-7 Taylor
 * polynomial in Horner form (|r| <= ln2/2, truncation < 6e-9 relative),
 * then an exact scaling by 2^k.  Valid for x in [-87, 88]. */
static float exp_f32(float x) {
    const float L2E = 0x1.715476p+0f, LN2_HI = 0x1.62e4p-1f, LN2_LO = 0x1.7f7d1cp-20f;
    float kf = rintf(x * L2E);
    float r = (x - kf * LN2_HI) - kf * LN2_LO;
    float q = 0x1.a01a02p-13f;                 /* 1/5040 */
    q = q * r + 0x1.6c16c2p-10f;               /* 1/720 */
    q = q * r + 0x1.111112p-7f;                /* 1/120 */
    q = q * r + 0x1.555556p-5f;                /* 1/24 */
    q = q * r + 0x1.555556p-3f;                /* 1/6 */
    q = q * r + 0x1p-1f;
    q = q * r + 1.0f;
    q = q * r + 1.0f;
    uint32_t sb = (uint32_t)((int)kf + 127) << 23;
    float sc; memcpy(&sc, &sb, 4);
    return q * sc;
}
/* exp for the FP64 pseudopotential, identical to the CUDA kernels' copy:
 * Cody-Waite reduction with ln2 split in a head whose low 21 bits are zero
 * (exact products for |k| < 2^21) and a tail, exp(r) by the degree-13
 * Taylor polynomial in Horner form (|r| <= ln2/2, truncation < 5e-18
 * relative), exact scaling by 2^k.  Valid for x in [-708, 709]. */
static double exp_f64(double x) {
    const double L2E = 0x1.71547652b82fep+0, LN2_HI = 0x1.62e42fee00000p-1, LN2_LO = 0x1.a39ef35793c76p-33;
    static const double C[12] = {0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26,
                                 0x1.27e4fb7789f5cp-22, 0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16,
                                 0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7,
                                 0x1.5555555555555p-5, 0x1.5555555555555p-3, 0x1p-1}; /* 1/13! .. 1/2! */
    double kf = rint(x * L2E);
    double r = (x - kf * LN2_HI) - kf * LN2_LO;
    double q = C[0];
    for (int i = 1; i < 12; i++) q = q * r + C[i];
    q = q * r + 1.0;
    q = q * r + 1.0;
    uint64_t sb = (uint64_t)((int64_t)kf + 1023) << 52;
    double sc; memcpy(&sc, &sb, 8);
    return q * sc;
}
static REAL psi(REAL rho) { /* collide.comp:512-516, rho0 = 1 */
    REAL rho0 = 1;
    return rho0 * ((REAL)1 - (IS_F32 ? (REAL)exp_f32((float)(-rho / rho0)) : (REAL)exp_f64((double)(-rho / rho0))));
}

/* Shan-Chen interaction force sum (collide.comp:534-584): acc = sum over
 * i >= 1 of w_i psi(rho(x + c_i)) c_i, the nonzero terms added in order; the
 * caller multiplies by -psi(rho_self) G.  Out-of-domain neighbours use rho_self. */
#define QMAX 27
static v3 sc_force_acc(orc_t* s, int x, int y, int z, REAL self_density) {
    v3 f = mk3(0, 0, 0);
    int fx = 1, fy = 1, fz = 1;
    REAL* src = MSRC(s);
    REAL ps[QMAX];
    for (int i = 1; i < s->Q; i++) {
        int nx = x + s->V[i].cx, ny = y + s->V[i].cy, nz = z + s->V[i].cz;
        int open = wrap(s, &nx, &ny, &nz);
        ps[i] = open ? psi(self_density) : src[cid(s, nx, ny, nz)];
    }
    if (shifted(s)) {
        /* shifted storages (extension): over opposite pairs, d_k = psi(c_i) -
         * psi(-c_i) for i = 2k + 1; per component the signed d_k of each
         * weight class summed in pair order, the classes combined as
         * fma(w, class sum, .) in class order */
        REAL d[QMAX / 2], out[3];
        for (int k = 0; k < s->Q / 2; k++) d[k] = ps[2 * k + 1] - ps[2 * k + 2];
        for (int a = 0; a < 3; a++) {
            REAL acc = 0, cls = 0, wc = 0;
            int have = 0, open = 0;
            for (int k = 0; k < s->Q / 2; k++) {
                const int i = 2 * k + 1;
                if (open && (REAL)s->V[i].w != wc) { /* the class ends: fold its sum in */
                    acc = have ? FMA(wc, cls, acc) : wc * cls;
                    have = 1;
                    open = 0;
                }
                const int comp = a == 0 ? s->V[i].cx : (a == 1 ? s->V[i].cy : s->V[i].cz);
                if (!comp) continue;
                const REAL t = comp > 0 ? d[k] : -d[k];
                cls = open ? cls + t : t;
                wc = (REAL)s->V[i].w;
                open = 1;
            }
            if (open) {
                acc = have ? FMA(wc, cls, acc) : wc * cls;
                have = 1;
            }
            out[a] = have ? acc : 0;
        }
        return mk3(out[0], out[1], out[2]);
    }
    for (int i = 1; i < s->Q; i++) {
        REAL wp = (REAL)s->V[i].w * ps[i];
        if (s->V[i].cx) { REAL t = s->V[i].cx > 0 ? wp : -wp; f.x = fx ? t : f.x + t; fx = 0; }
        if (s->V[i].cy) { REAL t = s->V[i].cy > 0 ? wp : -wp; f.y = fy ? t : f.y + t; fy = 0; }
        if (s->V[i].cz) { REAL t = s->V[i].cz > 0 ? wp : -wp; f.z = fz ? t : f.z + t; fz = 0; }
    }
    return f;
}

static v3 get_force(orc_t* s, size_t cell) { /* collide.comp:451-463 */
    if (!s->forcing) return mk3(0, 0, 0);
    if (s->constant_force) return mk3(s->fconst[0], s->fconst[1], s->fconst[2]);
    return mk3((REAL)s->forces[cell * 4 + 0], (REAL)s->forces[cell * 4 + 1], (REAL)s->forces[cell * 4 + 2]);
}

/* ------------------------------------------------------------------------ */
/* collide.comp main (:676-794) over every cell                               */
/* ------------------------------------------------------------------------ */
static void collide(orc_t* s, int save, int update) {
    const int Q = s->Q;
    const int odd = (int)(s->ticks % 2 == 1);
    REAL* L = LSRC(s);
    const size_t N = s->N;
    const int bb = s->d.esoteric && s->d.boundary_mode == ORC_BOUNDARY_BOUNCE_BACK;
    const int sh = shifted(s);
    /* cells are independent within one dispatch: the AA step reads and
     * writes the same private set of slots per cell, so the loop is safe to
     * run in parallel exactly as the GPU dispatch is. */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < s->d.nz; z++)
    for (int y = 0; y < s->d.ny; y++)
    for (int x = 0; x < s->d.nx; x++) {
        size_t cell = cid(s, x, y, z);
        uint32_t bid = get_boundry(s, cell);
        if (is_solid(s, bid)) continue; /* collide.comp:696-700 */
        int eqb = bid != 0; /* equilibrium boundary cell (extension) */
        REAL f[QMAX];
        for (int i = 0; i < Q; i++) {
            size_t rc; int rs;
            int open = aa_read_addr(s, x, y, z, i, odd, &rc, &rs);
            if ((bb || eqb) && s->d.esoteric) {
                /* halfway bounce-back folded into AA (extension): when the
                 * streaming source x-c_i is solid, take the cell's own
                 * outgoing opposite population instead (stored in the other
                 * AA slot) plus the moving-wall term of stream.comp:487-496. */
                int sx = x - s->V[i].cx, sy = y - s->V[i].cy, sz = z - s->V[i].cz;
                int sopen = wrap(s, &sx, &sy, &sz);
                uint32_t sid = sopen ? 0 : get_boundry(s, cid(s, sx, sy, sz));
                if (eqb && sopen) {
                    REAL rb = (REAL)s->bvals[cell * 4 + 0];
                    v3 ub = mk3((REAL)s->bvals[cell * 4 + 1], (REAL)s->bvals[cell * 4 + 2], (REAL)s->bvals[cell * 4 + 3]);
                    REAL br = bracket(s, cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, ub), (REAL)1 - uu_of(ub) * s->R2h);
                    f[i] = sh ? FMA((REAL)s->V[i].w * rb, br, -(REAL)s->V[i].w) : ((REAL)s->V[i].w * rb) * br;
                    continue;
                }
                if (bb && !sopen && is_solid(s, sid)) {
                    int oi = opp(i);
                    size_t oc; int os;
                    if (!odd) { oc = cell; os = oi; }
                    else { oc = cid(s, sx, sy, sz); os = i; }
                    const float* ob = &s->objects[sid * 12];
                    v3 uw = mk3((REAL)ob[0], (REAL)ob[1], (REAL)ob[2]);
                    v3 co = mk3((REAL)s->V[oi].cx, (REAL)s->V[oi].cy, (REAL)s->V[oi].cz);
                    f[i] = lat_load(s, L[(size_t)os * N + oc], os) + (REAL)(-2) * (REAL)s->V[oi].w * (REAL)1.0 * dot3(co, uw) * (REAL)3;
                    continue;
                }
            }
            /* out-of-domain reads give 0.01 (collide.comp:278-298); g = 0.01 - w when shifted */
            f[i] = open ? (sh ? (REAL)0.01 - (REAL)s->V[i].w : (REAL)0.01) : lat_load(s, L[(size_t)rs * N + rc], rs);
        }
        /* opposite populations pair as (i, i+1), i odd:  s = f_i + f_i+1,
         * d = f_i - f_i+1 (the shifted density and momentum, and TRT) */
        REAL sp[QMAX / 2 + 1], dp_[QMAX / 2 + 1];
        for (int i = 1; i < Q; i += 2) { sp[i / 2] = f[i] + f[i + 1]; dp_[i / 2] = f[i] - f[i + 1]; }
        REAL density, delta = 0; /* delta: shifted storage's rho - 1, the population sum itself */
        if (sh) { /* pairwise, plus the sum of w */
            density = f[0];
            for (int i = 1; i < Q; i += 2) density = density + sp[i / 2];
            delta = density;
            density = (REAL)1 + density;
        } else { /* compute_density (collide.comp:383-388): in population order */
            density = f[0];
            for (int i = 1; i < Q; i++) density = density + f[i];
        }
        if (density < (REAL)0.01) { /* max(density, 0.01) */
            density = (REAL)0.01;
            delta = (REAL)0.01 - (REAL)1;
        }
        v3 force = get_force(s, cell);
        REAL temperature = 0;
        if (s->thermal) { /* collide.comp:709-716 */
            REAL* TS = TSRC(s);
            for (int i = 0; i < s->Qt; i++) temperature += TS[cell * s->Qt + i];
            REAL k = -(REAL)s->d.beta * (temperature - (REAL)1);
            force.x = force.x + k * force.x;
            force.y = force.y + k * force.y;
            force.z = force.z + k * force.z;
        }
        if (s->d.multiphase) { /* collide.comp:580-583, :718-720 */
            v3 sc = sc_force_acc(s, x, y, z, density);
            REAL k = -psi(density) * (REAL)s->d.G;
            force.x = force.x + sc.x * k;
            force.y = force.y + sc.y * k;
            force.z = force.z + sc.z * k;
        }
        REAL jx = 0, jy = 0, jz = 0;
        int fx = 1, fy = 1, fz = 1;
        v3 vel;
        if (sh) {
            for (int i = 1; i < Q; i += 2) {
                REAL d = dp_[i / 2];
                if (s->V[i].cx) { REAL t = s->V[i].cx > 0 ? d : -d; jx = fx ? t : jx + t; fx = 0; }
                if (s->V[i].cy) { REAL t = s->V[i].cy > 0 ? d : -d; jy = fy ? t : jy + t; fy = 0; }
                if (s->V[i].cz) { REAL t = s->V[i].cz > 0 ? d : -d; jz = fz ? t : jz + t; fz = 0; }
            }
            REAL r = (REAL)1 / density;
            vel = mk3(jx * r, jy * r, jz * r);
            if (s->forced) {
                REAL h = r * (REAL)0.5;
                vel.x = FMA(force.x, h, vel.x);
                vel.y = FMA(force.y, h, vel.y);
                vel.z = FMA(force.z, h, vel.z);
            }
        } else {
            /* compute_velocity (collide.comp:390-395): the populations times
             * their lattice vectors summed in order, divided by the density;
             * plus force/(2 density) (:722) */
            for (int i = 0; i < Q; i++) {
                REAL d = f[i];
                if (s->V[i].cx) { REAL t = s->V[i].cx > 0 ? d : -d; jx = fx ? t : jx + t; fx = 0; }
                if (s->V[i].cy) { REAL t = s->V[i].cy > 0 ? d : -d; jy = fy ? t : jy + t; fy = 0; }
                if (s->V[i].cz) { REAL t = s->V[i].cz > 0 ? d : -d; jz = fz ? t : jz + t; fz = 0; }
            }
            vel = mk3(jx / density, jy / density, jz / density);
            if (s->forced) {
                REAL d2 = (REAL)2 * density;
                vel.x = vel.x + force.x / d2;
                vel.y = vel.y + force.y / d2;
                vel.z = vel.z + force.z / d2;
            }
        }
        REAL uu = sh ? uu_of(vel) : dot3(vel, vel);
        REAL len = IS_F32 ? (REAL)sqrtf((float)uu) : (REAL)sqrt((double)uu);
        int out_lim = len > (REAL)s->d.velocity_limit;
        int out_ext = len > (REAL)s->d.velocity_limit_extreme;
        if (out_lim) { /* normalize(u) * limit */
            if (sh) {
                REAL q = (REAL)s->d.velocity_limit / len;
                vel.x = vel.x * q; vel.y = vel.y * q; vel.z = vel.z * q;
            } else {
                vel.x = (vel.x / len) * (REAL)s->d.velocity_limit;
                vel.y = (vel.y / len) * (REAL)s->d.velocity_limit;
                vel.z = (vel.z / len) * (REAL)s->d.velocity_limit;
            }
        }
        if (eqb) {
            /* equilibrium boundary cell (extension): velocity kind keeps the
             * prescribed u with the received density, density kind keeps the
             * prescribed rho with the received velocity. */
            int kind = s->obj_kind[bid];
            REAL rb = (REAL)s->bvals[cell * 4 + 0];
            v3 ub = mk3((REAL)s->bvals[cell * 4 + 1], (REAL)s->bvals[cell * 4 + 2], (REAL)s->bvals[cell * 4 + 3]);
            if (kind == ORC_OBJ_EQ_VELOCITY) vel = ub; else density = rb;
            force = mk3(0, 0, 0);
        }
        const REAL one_m = (REAL)1 - uu_of(vel) * s->R2h;
        /* (u.u/2)/cs2 of the (limited) velocity: the literal equilibria's last term */
        const REAL uuh = (dot3(vel, vel) / (REAL)2) / s->cs2;
        if (update) {
            REAL fn[QMAX];
            const REAL fuR2 = FMA(force.z, vel.z, FMA(force.y, vel.y, force.x * vel.x)) * s->R2;
            if (sh && s->src_on && !eqb) {
                /* shifted storage with a source term: relaxation and source
                 * folded into one polynomial per opposite pair (extension):
                 *   A = fma(w+, delta, -fma(w+ rho, u.u R2/2, P+ (F.u) R2))
                 *   V = R4 fma(w+ rho/2, u, P+ F),  U = R2 fma(w- rho, u, P- F)
                 *   g_0 <- fma(w_0, A, (1 - w+) g_0),  E = fma(c.u, c.V, A)
                 *   BGK: g_i <- fma(w, E +- c.U, (1 - w) g_i)
                 *   TRT: g_i <- fma(w, E +- c.U, fma(a, g_i, b g_opp)),
                 *        a = 1 - (w+ + w-)/2, b = (w- - w+)/2
                 * (w+- the relaxation rates, P+- = 1 - w+-/2; BGK: w- = w+).
                 * Above the extreme velocity limit: the equilibrium, the same
                 * tree with w+- = 1 and P+- = 0. */
                const int trt = s->d.collision == ORC_TRT;
                const REAL op = out_ext ? (REAL)1 : s->Rtau, om = out_ext ? (REAL)1 : (trt ? s->Wm : s->Rtau);
                const REAL pp = out_ext ? (REAL)0 : (trt ? s->Pp : s->P), pm = out_ext ? (REAL)0 : (trt ? s->Pm : s->P);
                const REAL wp = op * density, wm = om * density;
                const REAL A = FMA(op, delta, -FMA(wp, uu_of(vel) * s->R2h, pp * fuR2));
                const REAL wph = wp * (REAL)0.5;
                const v3 V = mk3(FMA(wph, vel.x, pp * force.x) * s->R4, FMA(wph, vel.y, pp * force.y) * s->R4,
                                 FMA(wph, vel.z, pp * force.z) * s->R4);
                const v3 U = mk3(FMA(wm, vel.x, pm * force.x) * s->R2, FMA(wm, vel.y, pm * force.y) * s->R2,
                                 FMA(wm, vel.z, pm * force.z) * s->R2);
                const REAL keep = (REAL)1 - op;
                fn[0] = FMA((REAL)s->V[0].w, A, keep * f[0]);
                const REAL a = trt ? (REAL)1 - (op + om) * (REAL)0.5 : keep;
                const REAL b = trt ? (om - op) * (REAL)0.5 : (REAL)0;
                for (int i = 1; i < Q; i += 2) {
                    const int j = i + 1;
                    const int cx = s->V[i].cx, cy = s->V[i].cy, cz = s->V[i].cz;
                    const REAL w = (REAL)s->V[i].w;
                    const REAL E = FMA(cdot(cx, cy, cz, vel), cdot(cx, cy, cz, V), A);
                    const REAL cU = cdot(cx, cy, cz, U);
                    const REAL bi = trt ? FMA(a, f[i], b * f[j]) : a * f[i];
                    const REAL bj = trt ? FMA(a, f[j], b * f[i]) : a * f[j];
                    fn[i] = FMA(w, E + cU, bi);
                    fn[j] = FMA(w, E - cU, bj);
                }
            } else if (!sh && (eqb || s->d.collision != ORC_TRT)) {
                /* collide.comp:727-745 with :589-629: f + (-(f - feq)/tau) + source */
                const REAL fuc = dot3(force, vel) / s->cs2;
                for (int i = 0; i < Q; i++) {
                    REAL w = (REAL)s->V[i].w;
                    REAL cu = cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, vel);
                    REAL fe = feq_lit(s, w * density, cu, uuh);
                    REAL v = f[i] + -((f[i] - fe) / s->tau);
                    if (s->src_on) {
                        REAL fc = cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, force);
                        v = v + (s->P * w) * (fc / s->cs2 + ((fc * cu) / s->cs4 - fuc));
                    }
                    fn[i] = (eqb || out_ext) ? fe : v;
                }
            } else if (eqb || s->d.collision != ORC_TRT) {
                for (int i = 0; i < Q; i++) {
                    REAL w = (REAL)s->V[i].w;
                    REAL cu = cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, vel);
                    /* shifted storages form g_eq = fma(w rho, bracket, -w) */
                    REAL br = bracket(s, cu, one_m);
                    REAL fe = sh ? FMA(w * density, br, -w) : (w * density) * br;
                    REAL v = FMA(fe - f[i], s->Rtau, f[i]); /* old + (-(old - feq)/tau) */
                    if (s->src_on) {
                        REAL fc = cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, force);
                        REAL inner = FMA(fc, s->R2, FMA(fc * cu, s->R4, -fuR2));
                        v = FMA(s->P * w, inner, v);
                    }
                    fn[i] = (eqb || out_ext) ? fe : v;
                }
            } else {
                /* TRT (extension), pairwise over (i, opp i):
                 *   e+ = w rho ((1 - uu/2/cs2) + cu^2/2/cs4),  e- = w rho cu/cs2
                 *   f_i <- f_i - omega+ (f+ - e+) -+ omega- (f- - e-)
                 * omega+ = 1/tau, omega- = 1/(Lambda/(tau-1/2) + 1/2); the Guo
                 * term's even part (F.c)(u.c)/cs4 - F.u/cs2 gets (1-omega+/2),
                 * its odd part F.c/cs2 gets (1-omega-/2).  Above the extreme
                 * velocity limit the populations become e+ +- e-. */
                {
                    REAL w0 = (REAL)s->V[0].w;
                    REAL fe0 = sh ? FMA(w0 * density, one_m, -w0) : (w0 * density) * one_m;
                    REAL v = FMA(fe0 - f[0], s->Rtau, f[0]);
                    if (s->src_on) v = FMA(s->Pp * w0, -fuR2, v);
                    fn[0] = out_ext ? fe0 : v;
                }
                for (int i = 1; i < Q; i += 2) {
                    const int j = i + 1;
                    REAL w = (REAL)s->V[i].w;
                    REAL cu = cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, vel);
                    REAL wr = w * density;
                    REAL be = FMA(cu * cu, s->R4h, one_m);
                    REAL ep = sh ? FMA(wr, be, -w) : wr * be;
                    REAL em = (wr * s->R2) * cu;
                    REAL Pd = FMA(sp[i / 2], (REAL)0.5, -ep);
                    REAL Md = FMA(dp_[i / 2], (REAL)0.5, -em);
                    REAL vi = FMA(-Md, s->Wm, FMA(-Pd, s->Rtau, f[i]));
                    REAL vj = FMA(Md, s->Wm, FMA(-Pd, s->Rtau, f[j]));
                    if (s->src_on) {
                        REAL fc = cdot(s->V[i].cx, s->V[i].cy, s->V[i].cz, force);
                        REAL Sp = (s->Pp * w) * FMA(fc * cu, s->R4, -fuR2);
                        REAL Sm = (s->Pm * w) * (fc * s->R2);
                        vi = vi + (Sp + Sm);
                        vj = vj + (Sp - Sm);
                    }
                    fn[i] = out_ext ? ep + em : vi;
                    fn[j] = out_ext ? ep - em : vj;
                }
            }
            if (sh && s->d.multiphase) {
                /* 16-bit storage of multiphase flow: mass-conserving rounding
                 * (extension; Shan-Chen interfaces otherwise gain mass at
                 * ~1e-5 per step from rounding).  The relaxation and the
                 * source term conserve the population sum in exact
                 * arithmetic, so the cell's populations carry T = delta, its
                 * own sum (a clamped cell the clamped density's); an
                 * equilibrium boundary cell's rho - 1.  Populations
                 * 0..Q-2 are stored rounded, population Q-1 as the rounding of
                 * T less their stored values, so the stored populations sum to
                 * T up to that one rounding. */
                REAL rest = eqb ? density - (REAL)1 : delta;
                for (int i = 0; i < Q - 1; i++) {
                    const REAL h = lat_store(s, fn[i], i);
                    rest = rest - h;
                    fn[i] = h;
                }
                fn[Q - 1] = lat_store(s, rest, Q - 1);
            }
            for (int i = 0; i < Q; i++) {
                size_t wc; int ws;
                if (aa_write_addr(s, x, y, z, i, odd, &wc, &ws)) continue;
                L[(size_t)ws * N + wc] = lat_store(s, fn[i], ws);
            }
        }
        if (s->d.multiphase) {
            /* the ping-pong texture holds psi of the effective density
             * (the reference stores the density and applies psi on reading;
             * psi is a pure function of it, so the two are equivalent) */
            REAL eff = density;
            if (s->nobj > 1 && bid != 0) eff = (REAL)s->objects[bid * 12 + 11];
            MTGT(s)[cell] = psi(eff);
        }
        if (s->thermal) {
            REAL* TS = TSRC(s); REAL* TT = TTGT(s);
            for (int i = 0; i < s->Qt; i++) { /* collide.comp:771-782, :634-651, :668-670 */
                REAL cu = cdot(s->Vt[i].cx, s->Vt[i].cy, s->Vt[i].cz, vel);
                REAL ge = feq_lit(s, (REAL)s->Vt[i].w * temperature, cu, uuh);
                REAL g = TS[cell * s->Qt + i];
                TT[cell * s->Qt + i] = g + -((g - ge) / s->tau_t);
            }
        }
        if (save) {
            s->vel_den[cell * 4 + 0] = vel.x; s->vel_den[cell * 4 + 1] = vel.y;
            s->vel_den[cell * 4 + 2] = vel.z; s->vel_den[cell * 4 + 3] = density;
            s->bnd_tex[cell] = (float)bid;
            s->force_temp[cell * 4 + 0] = force.x; s->force_temp[cell * 4 + 1] = force.y;
            s->force_temp[cell * 4 + 2] = force.z; s->force_temp[cell * 4 + 3] = temperature;
        }
    }
    /* LBM.cpp:1646-1652 */
    if (!s->d.esoteric && update && !s->d.two_buffer_fixed) s->lat0_src = !s->lat0_src;
    if (s->d.multiphase) s->mp0_src = !s->mp0_src;
    s->th0_src = !s->th0_src;
}

/* stream.comp main (:498-584), two-buffer mode */
static void stream(orc_t* s) {
    const int Q = s->Q;
    const size_t N = s->N;
    REAL* S = LSRC(s); REAL* T = LTGT(s);
    #pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < Q; i++)
    for (int z = 0; z < s->d.nz; z++)
    for (int y = 0; y < s->d.ny; y++)
    for (int x = 0; x < s->d.nx; x++) {
        size_t cell = cid(s, x, y, z);
        int inv = (i == 0 || i >= Q) ? 0 : ((i % 2 == 1) ? i + 1 : i - 1);
        if (is_solid(s, get_boundry(s, cell))) continue;
        int sx = x - s->V[i].cx, sy = y - s->V[i].cy, sz = z - s->V[i].cz;
        if (wrap(s, &sx, &sy, &sz)) {
            T[(size_t)i * N + cell] = lat_store(s, shifted(s) ? (REAL)0.01 - (REAL)s->V[i].w : (REAL)0.01, i);
            continue;
        }
        size_t sc = cid(s, sx, sy, sz);
        uint32_t sid = get_boundry(s, sc);
        if (is_solid(s, sid)) {
            const float* ob = &s->objects[sid * 12];
            v3 uw = mk3((REAL)ob[0], (REAL)ob[1], (REAL)ob[2]);
            v3 c = mk3((REAL)s->V[inv].cx, (REAL)s->V[inv].cy, (REAL)s->V[inv].cz);
            REAL corr = (REAL)(-2) * (REAL)s->V[inv].w * (REAL)1.0 * dot3(c, uw) * (REAL)3;
            T[(size_t)i * N + cell] = lat_store(s, lat_load(s, S[(size_t)inv * N + cell], inv) + corr, i);
        } else {
            T[(size_t)i * N + cell] = S[(size_t)i * N + sc];
        }
    }
    s->lat0_src = !s->lat0_src; /* LBM.cpp:1553-1554 */
}

/* stream_thermal.comp main (:457-526) */
static void stream_thermal(orc_t* s) {
    const int Qt = s->Qt;
    REAL* S = TSRC(s); REAL* T = TTGT(s);
    #pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < s->d.nz; z++)
    for (int y = 0; y < s->d.ny; y++)
    for (int x = 0; x < s->d.nx; x++)
    for (int i = 0; i < Qt; i++) {
        size_t cell = cid(s, x, y, z);
        int inv = opp_t(i, Qt);
        if (is_solid(s, get_boundry(s, cell))) continue;
        int sx = x - s->Vt[i].cx, sy = y - s->Vt[i].cy, sz = z - s->Vt[i].cz;
        if (wrap(s, &sx, &sy, &sz)) continue;
        size_t sc = cid(s, sx, sy, sz);
        uint32_t sid = get_boundry(s, sc);
        if (is_solid(s, sid)) {
            REAL Tw = (REAL)s->objects[sid * 12 + 3];
            T[cell * Qt + i] = -S[cell * Qt + inv] + (REAL)2 * (REAL)s->Vt[inv].w * Tw;
        } else {
            T[cell * Qt + i] = S[sc * Qt + i];
        }
    }
    s->th0_src = !s->th0_src;
}

/* LBM.cpp:1484-1493 */
static void iterate(orc_t* s, int save, int update) {
    collide(s, save, update);
    if (!s->d.esoteric) stream(s);
    if (s->thermal) stream_thermal(s);
}

/* ------------------------------------------------------------------------ */
/* public API                                                                 */
/* ------------------------------------------------------------------------ */
/* bits per boundary id, LBM.cpp:569 / :606 (float log2 as the reference) */
int ORC(bits_per_boundry)(int object_count) {
    if (object_count <= 1) return 0;
    return (int)exp2(ceil(log2f(ceilf(log2f((float)object_count)))));
}

/* boundary bit packing, LBM.cpp:634-659; returns number of uint32 words */
size_t ORC(pack_boundries)(const uint32_t* ids, size_t n, int bits, uint32_t* out, size_t out_words) {
    size_t words = (n * (size_t)bits + 31) / 32;
    if (!out) return words;
    memset(out, 0, out_words * 4);
    for (size_t v = 0; v < n; v++) {
        size_t b = v * (size_t)bits;
        out[b / 32] |= (ids[v] << (b % 32));
    }
    return words;
}

void ORC(destroy)(orc_t* s) {
    if (!s) return;
    free(s->lat[0]); free(s->lat[1]); free(s->boundries); free(s->objects); free(s->obj_kind);
    free(s->forces); free(s->th[0]); free(s->th[1]); free(s->mp[0]); free(s->mp[1]); free(s->bvals);
    free(s->vel_den); free(s->force_temp); free(s->bnd_tex);
    free(s);
}

/*
 * Mirrors LBM::initialize_fields (LBM.cpp:415-506) given the per-cell
 * results of the initialisation lambda as arrays:
 *   rho[N], u[N*3], force[N*3], T[N], ids[N]; objects: nobj*12 floats laid
 *   out as (u,T)(omega,0)(com,rho_eff); obj_kind: nobj ints (0 = solid).
 * Flag derivation follows LBM.cpp:523-556.
 */
orc_t* ORC(create)(const orc_desc* d, const float* rho, const float* u, const float* force,
                   const float* T, const uint32_t* ids, int nobj_in, const float* objects, const int* obj_kind) {
    orc_t* s = (orc_t*)calloc(1, sizeof(orc_t));
    s->d = *d;
    switch (d->velocity_set) {
    case ORC_D2Q9: s->Q = 9; s->V = D2Q9_T; s->dims = 2; s->Qt = 5; s->Vt = D2Q5_T; break;
    case ORC_D3Q15: s->Q = 15; s->V = D3Q15_T; s->dims = 3; s->Qt = 7; s->Vt = D3Q7_T; break;
    case ORC_D3Q19: s->Q = 19; s->V = D3Q19_T; s->dims = 3; s->Qt = 7; s->Vt = D3Q7_T; break;
    case ORC_D3Q27: s->Q = 27; s->V = D3Q27_T; s->dims = 3; s->Qt = 7; s->Vt = D3Q7_T; break;
    default: free(s); return NULL;
    }
    s->cs = (REAL)(1.0 / sqrt(3.0));
    {
        REAL cs2 = s->cs * s->cs, cs4 = cs2 * cs2;
        REAL tau = (REAL)d->tau;
        s->R2 = (REAL)1 / cs2;
        s->R4 = (REAL)1 / cs4;
        s->R2h = s->R2 * (REAL)0.5;
        s->R4h = s->R4 * (REAL)0.5;
        s->Rtau = (REAL)1 / tau;
        s->P = (REAL)1 - (REAL)1 / ((REAL)2 * tau);
        s->Rtau_t = (REAL)1 / (REAL)d->tau_t;
        s->cs2 = cs2;
        s->cs4 = cs4;
        s->tau = tau;
        s->tau_t = (REAL)d->tau_t;
        REAL taum = (REAL)d->trt_magic / (tau - (REAL)0.5) + (REAL)0.5;
        s->Wm = (REAL)1 / taum;
        s->Pp = (REAL)1 - s->Rtau * (REAL)0.5;
        s->Pm = (REAL)1 - s->Wm * (REAL)0.5;
    }
    s->N = (size_t)d->nx * d->ny * d->nz;
    const size_t N = s->N;
    s->lat0_src = 1; s->th0_src = 1; s->mp0_src = 1;
    s->lat[0] = (REAL*)calloc(N * s->Q, sizeof(REAL));
    if (!d->esoteric) s->lat[1] = (REAL*)calloc(N * s->Q, sizeof(REAL));

    /* objects: slot 0 is fluid with default temperature/density (LBM.cpp:439-441) */
    uint32_t maxid = 0;
    for (size_t c = 0; c < N; c++) if (ids && ids[c] > maxid) maxid = ids[c];
    int nobj = nobj_in > 1 ? nobj_in : 1;
    if ((int)maxid + 1 > nobj) nobj = (int)maxid + 1;
    s->nobj = nobj;
    s->objects = (float*)calloc((size_t)nobj * 12, sizeof(float));
    s->obj_kind = (int*)calloc((size_t)nobj, sizeof(int));
    for (int k = 0; k < nobj; k++) { s->objects[k * 12 + 3] = 1.0f; s->objects[k * 12 + 11] = 1.0f; }
    if (objects) for (int k = 1; k < nobj_in; k++) memcpy(&s->objects[k * 12], &objects[k * 12], 12 * sizeof(float));
    if (obj_kind) for (int k = 1; k < nobj_in; k++) s->obj_kind[k] = obj_kind[k];

    /* LBM.cpp:523-556: constant-force and thermal detection relative to cell (0,0,0) */
    s->constant_force = 1;
    float f0[3] = {0, 0, 0};
    if (force) { f0[0] = force[0]; f0[1] = force[1]; f0[2] = force[2]; }
    s->fconst[0] = f0[0]; s->fconst[1] = f0[1]; s->fconst[2] = f0[2];
    s->thermal = 0;
    float T0 = T ? T[0] : 1.0f;
    for (size_t c = 0; c < N; c++) {
        if (force && (force[c * 3] != f0[0] || force[c * 3 + 1] != f0[1] || force[c * 3 + 2] != f0[2])) s->constant_force = 0;
        if (T && T[c] != T0) s->thermal = 1;
        uint32_t id = ids ? ids[c] : 0;
        if (id != 0 && s->objects[id * 12 + 3] != T0) s->thermal = 1;
    }
    s->forcing = !(s->constant_force && f0[0] == 0 && f0[1] == 0 && f0[2] == 0);
    /* collide.comp:609: the source term exists with forcing, multiphase or thermal flow */
    s->src_on = s->forcing || d->multiphase || s->thermal;
    s->forced = s->src_on;
    if (s->forcing && !s->constant_force) {
        s->forces = (float*)calloc(N * 4, sizeof(float));
        for (size_t c = 0; c < N; c++) for (int k = 0; k < 3; k++) s->forces[c * 4 + k] = force[c * 3 + k];
    }

    s->bits = ORC(bits_per_boundry)(nobj);
    if (nobj > 1) {
        size_t words = ORC(pack_boundries)(NULL, N, s->bits, NULL, 0);
        s->boundries = (uint32_t*)calloc(words + 1, 4);
        uint32_t* tmp = (uint32_t*)calloc(N, 4);
        if (ids) memcpy(tmp, ids, N * 4);
        ORC(pack_boundries)(tmp, N, s->bits, s->boundries, words + 1);
        free(tmp);
    }
    /* equilibrium boundary values: the cell's initial (rho, u) */
    s->bvals = (float*)calloc(N * 4, sizeof(float));
    for (size_t c = 0; c < N; c++) {
        s->bvals[c * 4 + 0] = rho ? rho[c] : 1.0f;
        for (int k = 0; k < 3; k++) s->bvals[c * 4 + 1 + k] = u ? u[c * 3 + k] : 0.0f;
    }

    if (d->multiphase) {
        s->mp[0] = (REAL*)calloc(N, sizeof(REAL));
        s->mp[1] = (REAL*)calloc(N, sizeof(REAL));
    }
    s->vel_den = (REAL*)calloc(N * 4, sizeof(REAL));
    s->force_temp = (REAL*)calloc(N * 4, sizeof(REAL));
    s->bnd_tex = (float*)calloc(N, sizeof(float));

    /* host side of LBM.cpp:537-538: solid cells get zero velocity */
    /* set_equilibrium_populations.comp main (:198-221) */
    REAL* L = s->lat[0];
    for (size_t c = 0; c < N; c++) {
        uint32_t id = ids ? ids[c] : 0;
        v3 uc = mk3(0, 0, 0);
        if (u && !is_solid(s, id)) uc = mk3((REAL)u[c * 3], (REAL)u[c * 3 + 1], (REAL)u[c * 3 + 2]);
        REAL r = rho ? (REAL)rho[c] : (REAL)1;
        for (int i = 0; i < s->Q; i++) L[(size_t)i * N + c] = lat_from_f(s, feq_init(s, r, uc, i), i);
    }
    if (s->thermal) {
        s->th[0] = (REAL*)calloc(N * s->Qt, sizeof(REAL));
        s->th[1] = (REAL*)calloc(N * s->Qt, sizeof(REAL));
        if (d->thermal_init_equilibrium) {
            for (size_t c = 0; c < N; c++) {
                REAL t = T ? (REAL)T[c] : (REAL)1;
                if (t == 0) continue; /* set_equilibrium_populations_thermal.comp:171-172 */
                uint32_t id = ids ? ids[c] : 0;
                v3 uc = mk3(0, 0, 0);
                if (u && !is_solid(s, id)) uc = mk3((REAL)u[c * 3], (REAL)u[c * 3 + 1], (REAL)u[c * 3 + 2]);
                for (int i = 0; i < s->Qt; i++) s->th[0][c * s->Qt + i] = feq_t_init(s, t, uc, i);
            }
        }
        /* as read, set_equilibrium_populations_thermal.comp:101-107 writes
         * index Qt*N+cell for every population, past the end of the buffer:
         * the thermal lattice keeps its initial (zero) contents. */
    }
    s->ticks = 0;
    iterate(s, 1, 0); /* LBM.cpp:502: _iterate_time(true, false) */
    return s;
}

/* LBM::iterate_time with target_tick_per_second = 0 (LBM.cpp:220-240) */
void ORC(iterate)(orc_t* s, int n, int save_last) {
    for (int k = 0; k < n; k++) {
        iterate(s, save_last && k == n - 1, 1);
        s->ticks++;
    }
}

/* the thermal knobs between steps (the reference sets them as uniforms at
 * every dispatch, LBM.cpp:1612-1613) */
void ORC(set_thermal)(orc_t* s, float tau_t, float beta) {
    s->d.tau_t = tau_t;
    s->d.beta = beta;
    s->Rtau_t = (REAL)1 / (REAL)tau_t;
    s->tau_t = (REAL)tau_t;
}
long ORC(ticks)(orc_t* s) { return s->ticks; }
int ORC(thermal)(orc_t* s) { return s->thermal; }
int ORC(forcing)(orc_t* s) { return s->forcing; }
int ORC(constant_force)(orc_t* s) { return s->constant_force; }
int ORC(bits)(orc_t* s) { return s->bits; }
size_t ORC(cells)(orc_t* s) { return s->N; }
int ORC(q)(orc_t* s) { return s->Q; }

/* copies out the macroscopic textures: vel_den N*4, force_temp N*4, bnd N */
void ORC(get_fields)(orc_t* s, double* vel_den, double* force_temp, float* bnd) {
    for (size_t k = 0; k < s->N * 4; k++) {
        if (vel_den) vel_den[k] = (double)s->vel_den[k];
        if (force_temp) force_temp[k] = (double)s->force_temp[k];
    }
    if (bnd) memcpy(bnd, s->bnd_tex, s->N * sizeof(float));
}
/* copies the raw DDF buffer (source lattice, SoA i*N+cell) */
void ORC(get_lattice)(orc_t* s, double* out) {
    REAL* L = LSRC(s);
    for (size_t k = 0; k < s->N * (size_t)s->Q; k++) out[k] = (double)lat_to_f(s, L[k], (int)(k / s->N));
}
void ORC(set_lattice)(orc_t* s, const double* in) {
    REAL* L = LSRC(s);
    for (size_t k = 0; k < s->N * (size_t)s->Q; k++) L[k] = lat_from_f(s, (REAL)in[k], (int)(k / s->N));
}
void ORC(get_thermal)(orc_t* s, double* out) {
    if (!s->thermal) return;
    REAL* L = TSRC(s);
    for (size_t k = 0; k < s->N * (size_t)s->Qt; k++) out[k] = (double)L[k];
}
void ORC(get_boundries)(orc_t* s, uint32_t* out, size_t words) {
    if (s->boundries) memcpy(out, s->boundries, words * 4);
}
/* FP64 sums over non-solid cells of the last saved fields: mass, momentum xyz, kinetic energy */
void ORC(reduce)(orc_t* s, double out[5]) {
    double m = 0, px = 0, py = 0, pz = 0, ke = 0;
    for (size_t c = 0; c < s->N; c++) {
        uint32_t id = get_boundry(s, c);
        if (is_solid(s, id)) continue;
        double r = (double)s->vel_den[c * 4 + 3];
        double ux = (double)s->vel_den[c * 4 + 0], uy = (double)s->vel_den[c * 4 + 1], uz = (double)s->vel_den[c * 4 + 2];
        m += r; px += r * ux; py += r * uy; pz += r * uz; ke += 0.5 * r * (ux * ux + uy * uy + uz * uz);
    }
    out[0] = m; out[1] = px; out[2] = py; out[3] = pz; out[4] = ke;
}
uint16_t ORC(f32_to_f16)(float f) { return f32_to_f16_rne(f); }
float ORC(f16_to_f32)(uint16_t h) { return f16_to_f32(h); }
/* the hand-written exps of the pseudopotential */
float ORC(exp_f32)(float x) { return exp_f32(x); }
double ORC(exp_f64)(double x) { return exp_f64(x); }
/* the fp16c round trip of a shifted population g (encode, then decode) */
float ORC(fp16c_round)(float g) { return c16_round(g); }
