/*
 * adjoint_oracle.c -- FP64 reference of the differentiable channel-flow
 * model and its discrete adjoint (reverse mode).  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/ and bench.py as the checker of the CUDA adjoint; the
 * product never calls it.  It has no counterpart in the reference, which
 * has no adjoint; the model is defined here and in the CUDA kernels alike:
 *
 * Lattice D2Q9 (nz = 1) or D3Q19, velocity sets and pairing as
 * VelocitySet.cpp:53-107.  Domain nx x ny x nz, periodic in z.  One step
 * maps the post-collision state f^{t-1} to f^t:
 *   pull   g_i(x) = f_i(x - c_i)                       source inside
 *          g_i(x) = f_opp(i)(x)                        source outside in y (halfway bounce-back wall)
 *          g_i(x) = feq_i(1, (u_in(y,z), 0, 0))        source at x < 0 or x >= nx (equilibrium inlet
 *                                                      and outlet, both with the inlet profile)
 * Every population of f^(t-1) then feeds at most one g of step t, so the
 * adjoint's transposed pull (a push) writes every slot at most once.
 *   BGK    g^c_i = g_i + (feq_i(rho, u) - g_i) / tau,  feq = w rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u.u)
 *   PSM    f_i = (1 - s) g^c_i + s g_opp(i)            (partial bounce-back, solid fraction s in [0,1])
 * f^0 = feq(1, (u_in(y,z), 0, 0)) everywhere.  After T steps the objective
 * uses the pulled populations g^T of the last step:
 *   J = wd * sum_x 2 s(x) j_x(x)  +  wm * sum_x |u(x) - u*(x)|^2,   j = sum_i g_i c_i, u = j / rho
 * (2 s j_x is the x momentum the partial bounce-back removes: the drag.)
 * Gradients: dJ/ds per cell and dJ/du_in per inlet row (y, z).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int cx, cy, cz; double w; } adj_dir;

static const adj_dir A_D2Q9[9] = {
    {0, 0, 0, 4.0 / 9}, {1, 0, 0, 1.0 / 9}, {-1, 0, 0, 1.0 / 9}, {0, 1, 0, 1.0 / 9}, {0, -1, 0, 1.0 / 9},
    {1, 1, 0, 1.0 / 36}, {-1, -1, 0, 1.0 / 36}, {1, -1, 0, 1.0 / 36}, {-1, 1, 0, 1.0 / 36}};
static const adj_dir A_D3Q19[19] = {
    {0, 0, 0, 1.0 / 3}, {1, 0, 0, 1.0 / 18}, {-1, 0, 0, 1.0 / 18}, {0, 1, 0, 1.0 / 18}, {0, -1, 0, 1.0 / 18},
    {0, 0, 1, 1.0 / 18}, {0, 0, -1, 1.0 / 18}, {1, 1, 0, 1.0 / 36}, {-1, -1, 0, 1.0 / 36}, {1, -1, 0, 1.0 / 36},
    {-1, 1, 0, 1.0 / 36}, {1, 0, 1, 1.0 / 36}, {-1, 0, -1, 1.0 / 36}, {1, 0, -1, 1.0 / 36}, {-1, 0, 1, 1.0 / 36},
    {0, 1, 1, 1.0 / 36}, {0, -1, -1, 1.0 / 36}, {0, 1, -1, 1.0 / 36}, {0, -1, 1, 1.0 / 36}};

#define QM 19

typedef struct {
    int nx, ny, nz, Q, T;
    double tau, wd, wm;
    const adj_dir* V;
    size_t N;
    double* s;      /* N */
    double* uin;    /* ny*nz */
    double* ustar;  /* 3N */
    double* traj;   /* (T+1) * Q * N: every post-collision state */
} adj_t;

static int opp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }
static size_t cell(const adj_t* a, int x, int y, int z) { return ((size_t)z * a->ny + y) * a->nx + x; }
static double* state(adj_t* a, int t) { return a->traj + (size_t)t * a->Q * a->N; }

static double feq(const adj_t* a, int i, double rho, double ux, double uy, double uz) {
    const adj_dir* d = &a->V[i];
    double cu = d->cx * ux + d->cy * uy + d->cz * uz;
    double uu = ux * ux + uy * uy + uz * uz;
    return d->w * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * uu);
}

/* source kind of population i at (x, y, z): 0 interior (fills *sx..), 1 wall, 2 inlet/outlet equilibrium */
static int source(const adj_t* a, int x, int y, int z, int i, int* sx, int* sy, int* sz) {
    const adj_dir* d = &a->V[i];
    int X = x - d->cx, Y = y - d->cy, Z = z - d->cz;
    if (Y < 0 || Y >= a->ny) return 1;
    if (X < 0 || X >= a->nx) return 2;
    Z = ((Z % a->nz) + a->nz) % a->nz;
    *sx = X; *sy = Y; *sz = Z;
    return 0;
}

static void pull(adj_t* a, const double* f, int x, int y, int z, double* g) {
    const size_t N = a->N, c = cell(a, x, y, z);
    for (int i = 0; i < a->Q; i++) {
        int sx, sy, sz;
        switch (source(a, x, y, z, i, &sx, &sy, &sz)) {
        case 0: g[i] = f[(size_t)i * N + cell(a, sx, sy, sz)]; break;
        case 1: g[i] = f[(size_t)opp(i) * N + c]; break;
        default: g[i] = feq(a, i, 1.0, a->uin[(size_t)z * a->ny + y], 0, 0); break;
        }
    }
}

static void moments(const adj_t* a, const double* g, double* rho, double* j) {
    double r = 0, jx = 0, jy = 0, jz = 0;
    for (int i = 0; i < a->Q; i++) {
        r += g[i];
        jx += g[i] * a->V[i].cx; jy += g[i] * a->V[i].cy; jz += g[i] * a->V[i].cz;
    }
    *rho = r; j[0] = jx; j[1] = jy; j[2] = jz;
}

adj_t* adj_create(int nx, int ny, int nz, int q, double tau, int T, const double* s, const double* uin,
                  const double* ustar, double wd, double wm) {
    adj_t* a = (adj_t*)calloc(1, sizeof(adj_t));
    a->nx = nx; a->ny = ny; a->nz = nz; a->Q = q; a->T = T; a->tau = tau; a->wd = wd; a->wm = wm;
    a->V = q == 9 ? A_D2Q9 : A_D3Q19;
    a->N = (size_t)nx * ny * nz;
    a->s = (double*)malloc(a->N * sizeof(double));
    a->uin = (double*)malloc((size_t)ny * nz * sizeof(double));
    a->ustar = (double*)malloc(3 * a->N * sizeof(double));
    memcpy(a->s, s, a->N * sizeof(double));
    memcpy(a->uin, uin, (size_t)ny * nz * sizeof(double));
    memcpy(a->ustar, ustar, 3 * a->N * sizeof(double));
    a->traj = (double*)malloc((size_t)(T + 1) * q * a->N * sizeof(double));
    return a;
}

void adj_destroy(adj_t* a) {
    if (!a) return;
    free(a->s); free(a->uin); free(a->ustar); free(a->traj); free(a);
}

void adj_set_params(adj_t* a, const double* s, const double* uin) {
    memcpy(a->s, s, a->N * sizeof(double));
    memcpy(a->uin, uin, (size_t)a->ny * a->nz * sizeof(double));
}

/* runs f^0 .. f^(T-1) (storing every state) and returns J from step T */
double adj_forward(adj_t* a) {
    const size_t N = a->N;
    const int Q = a->Q;
    double* f0 = state(a, 0);
    for (int z = 0; z < a->nz; z++)
    for (int y = 0; y < a->ny; y++)
    for (int x = 0; x < a->nx; x++)
        for (int i = 0; i < Q; i++) f0[(size_t)i * N + cell(a, x, y, z)] = feq(a, i, 1.0, a->uin[(size_t)z * a->ny + y], 0, 0);
    double J = 0;
    for (int t = 1; t <= a->T; t++) {
        double* f = state(a, t - 1);
        double* fn = state(a, t);
        for (int z = 0; z < a->nz; z++)
        for (int y = 0; y < a->ny; y++)
        for (int x = 0; x < a->nx; x++) {
            const size_t c = cell(a, x, y, z);
            double g[QM], rho, j[3];
            pull(a, f, x, y, z, g);
            moments(a, g, &rho, j);
            double ux = j[0] / rho, uy = j[1] / rho, uz = j[2] / rho;
            if (t == a->T) {
                double dx = ux - a->ustar[3 * c], dy = uy - a->ustar[3 * c + 1], dz = uz - a->ustar[3 * c + 2];
                J += a->wd * 2.0 * a->s[c] * j[0] + a->wm * (dx * dx + dy * dy + dz * dz);
                continue;
            }
            const double s = a->s[c];
            double gc[QM];
            for (int i = 0; i < Q; i++) gc[i] = g[i] + (feq(a, i, rho, ux, uy, uz) - g[i]) / a->tau;
            for (int i = 0; i < Q; i++) fn[(size_t)i * N + c] = (1.0 - s) * gc[i] + s * g[opp(i)];
        }
    }
    return J;
}

/* reverse sweep; grad_s[N], grad_uin[ny*nz] are overwritten */
void adj_backward(adj_t* a, double* grad_s, double* grad_uin) {
    const size_t N = a->N;
    const int Q = a->Q;
    const double om = 1.0 / a->tau;
    memset(grad_s, 0, N * sizeof(double));
    memset(grad_uin, 0, (size_t)a->ny * a->nz * sizeof(double));
    double* lam = (double*)calloc((size_t)Q * N, sizeof(double));  /* adjoint of f^t */
    double* lamp = (double*)calloc((size_t)Q * N, sizeof(double)); /* adjoint of f^(t-1) */
    for (int t = a->T; t >= 1; t--) {
        const double* f = state(a, t - 1);
        memset(lamp, 0, (size_t)Q * N * sizeof(double));
        for (int z = 0; z < a->nz; z++)
        for (int y = 0; y < a->ny; y++)
        for (int x = 0; x < a->nx; x++) {
            const size_t c = cell(a, x, y, z);
            double g[QM], rho, j[3], mu[QM];
            pull(a, (double*)f, x, y, z, g);
            moments(a, g, &rho, j);
            double u[3] = {j[0] / rho, j[1] / rho, j[2] / rho};
            const double s = a->s[c];
            if (t == a->T) {
                /* dJ/dg_i = wd 2 s c_ix + wm sum_a 2 (u_a - u*_a)(c_ia - u_a)/rho ; dJ/ds = wd 2 j_x */
                double du[3] = {u[0] - a->ustar[3 * c], u[1] - a->ustar[3 * c + 1], u[2] - a->ustar[3 * c + 2]};
                for (int i = 0; i < Q; i++) {
                    const adj_dir* d = &a->V[i];
                    double ci[3] = {d->cx, d->cy, d->cz};
                    double m = a->wd * 2.0 * s * d->cx;
                    for (int k = 0; k < 3; k++) m += a->wm * 2.0 * du[k] * (ci[k] - u[k]) / rho;
                    mu[i] = m;
                }
                grad_s[c] += a->wd * 2.0 * j[0];
            } else {
                /* mu_i = sum_k lam_k d f_k / d g_i with f_k = (1-s) g^c_k + s g_opp(k):
                 * d g^c_k / d g_i = (1-om) delta_ki + om d feq_k / d g_i,
                 * d feq_k / d g_i = w_k B_k + sum_a w_k (3 c_ka + 9 cu_k c_ka - 3 u_a)(c_ia - u_a) */
                double L[QM], A0 = 0, Vv[3] = {0, 0, 0};
                for (int k = 0; k < Q; k++) L[k] = lam[(size_t)k * N + c];
                double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
                double gs = 0;
                for (int k = 0; k < Q; k++) {
                    const adj_dir* d = &a->V[k];
                    double ck[3] = {d->cx, d->cy, d->cz};
                    double cu = ck[0] * u[0] + ck[1] * u[1] + ck[2] * u[2];
                    double Lk = (1.0 - s) * L[k];
                    A0 += Lk * d->w * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * uu);
                    for (int q = 0; q < 3; q++) Vv[q] += Lk * d->w * (3.0 * ck[q] + 9.0 * cu * ck[q] - 3.0 * u[q]);
                    double gck = g[k] + (feq(a, k, rho, u[0], u[1], u[2]) - g[k]) * om;
                    gs += L[k] * (g[opp(k)] - gck);
                }
                grad_s[c] += gs;
                for (int i = 0; i < Q; i++) {
                    const adj_dir* d = &a->V[i];
                    double ci[3] = {d->cx, d->cy, d->cz};
                    double dot = (ci[0] - u[0]) * Vv[0] + (ci[1] - u[1]) * Vv[1] + (ci[2] - u[2]) * Vv[2];
                    mu[i] = (1.0 - om) * (1.0 - s) * L[i] + om * (A0 + dot) + s * L[opp(i)];
                }
            }
            /* transpose of the pull */
            for (int i = 0; i < Q; i++) {
                int sx, sy, sz;
                switch (source(a, x, y, z, i, &sx, &sy, &sz)) {
                case 0: lamp[(size_t)i * N + cell(a, sx, sy, sz)] += mu[i]; break;
                case 1: lamp[(size_t)opp(i) * N + c] += mu[i]; break;
                default: {
                    const adj_dir* d = &a->V[i];
                    double ui = a->uin[(size_t)z * a->ny + y];
                    grad_uin[(size_t)z * a->ny + y] += mu[i] * d->w * (3.0 * d->cx + 9.0 * d->cx * d->cx * ui - 3.0 * ui);
                    break;
                }
                }
            }
        }
        double* tmp = lam; lam = lamp; lamp = tmp;
    }
    /* f^0 = feq(1, u_in): d f^0_i / d u_in = w_i (3 c_ix + 9 c_ix^2 u_in - 3 u_in) */
    for (int z = 0; z < a->nz; z++)
    for (int y = 0; y < a->ny; y++)
    for (int x = 0; x < a->nx; x++) {
        const size_t c = cell(a, x, y, z);
        double ui = a->uin[(size_t)z * a->ny + y];
        for (int i = 0; i < Q; i++) {
            const adj_dir* d = &a->V[i];
            grad_uin[(size_t)z * a->ny + y] += lam[(size_t)i * N + c] * d->w * (3.0 * d->cx + 9.0 * d->cx * d->cx * ui - 3.0 * ui);
        }
    }
    free(lam);
    free(lamp);
}
