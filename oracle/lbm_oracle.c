/*
 * lbm_oracle.c -- CPU restatement of the reference D3Q19 A-A kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links, loads or
 * calls this file: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline arm use it, as the checker.  The GPU path never falls back to it.
 *
 * What it restates (reference paths are relative to the reference project):
 *   init   -> src/cl_programs/lbm_init.cl:32-237
 *   alpha  -> src/cl_programs/lbm_alpha.cl:12-498
 *   beta   -> src/cl_programs/lbm_beta.cl:13-802 (the USE_SHARED_MEMORY=1
 *             path that the reference hard-codes at lbm_beta.cl:6)
 *   eq     -> src/cl_programs/lbm_header.h:55-94
 *   wrap   -> src/cl_programs/wrap.h:112-127 (linear wrap modulo the cell
 *             count) and the work-group realignment of lbm_beta.cl:218-234
 *
 * Every floating-point operation is performed in the same order as in the
 * reference kernels, so that with contraction disabled (-ffp-contract=off)
 * results are bit-identical to the reference kernel source compiled as C++
 * (oracle/ref_shim) and to the CUDA kernels built with -fmad=false.
 *
 * The Smagorinsky term has no counterpart in the reference.  It follows
 * Hou, Sterling, Chen & Doolen (1996), "A lattice Boltzmann subgrid model for
 * high Reynolds number flows": the total relaxation time per cell is
 *     tau_eff = (tau0 + sqrt(tau0^2 + C * sqrt(Q))) / 2,
 *     Q = Pi_ab Pi_ab,  Pi_ab = sum_i e_ia e_ib (f_i - f_i^eq)
 *                             = sum_i e_ia e_ib f_i - rho/3 delta_ab - u_a u_b,
 *     C = 18 * sqrt(2) * Cs^2  (lattice units, Delta = 1, rho0 = 1 of the
 *                               incompressible equilibrium),
 * inserted into the reference BGK update in place of the constant inv_tau.
 *
 * The file is compiled once per storage variant (VARIANT = 0 f32, 1 f64,
 * 2 shifted f16, 3 shifted bf16, 4 shifted c16).  Shifted variants store g_i = f_i - w_i
 * and do all arithmetic in float, in deviation form: the same model with
 * the operations the GB300 kernels perform for these types (pair sums,
 * explicit fused multiply-adds via fmaf, see dev_* below).  The reference
 * has no 16-bit storage, so for these variants this file is the definition
 * the kernels are held to; the f32 and f64 variants are pinned to the
 * reference itself.
 */
#include <stdint.h>
#include <string.h>
#include <math.h>

#ifndef VARIANT
#define VARIANT 0
#endif
#if VARIANT != 1
#define RSQRT sqrtf
#endif

#if VARIANT == 0
typedef float REAL;
typedef float STOR;
#define SFX(n) n##_f32
#define SHIFTED 0
#elif VARIANT == 1
typedef double REAL;
typedef double STOR;
#define SFX(n) n##_f64
#define SHIFTED 0
#define RSQRT sqrt
#elif VARIANT == 2
typedef float REAL;
typedef _Float16 STOR;
#define SFX(n) n##_f16
#define SHIFTED 1
#elif VARIANT == 3
typedef float REAL;
typedef uint16_t STOR;
#define SFX(n) n##_bf16
#define SHIFTED 1
#else
typedef float REAL;
typedef uint16_t STOR;
#define SFX(n) n##_c16
#define SHIFTED 1
#endif

/* flags: src/CLbmSolver.hpp:30-33 */
#define FL_OBSTACLE 1
#define FL_FLUID 2
#define FL_LID 4
#define FL_GHOST 8

/* D3Q19 directions in reference order: src/main.cpp:38-66 and
 * src/cl_programs/lbm_header.h:15-19.  opp(2k) = 2k+1, 18 is the rest. */
static const int EX[19] = {1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0};
static const int EY[19] = {0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0};
static const int EZ[19] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0};

static inline int opp(int i) { return i == 18 ? 18 : (i ^ 1); }

/* constants exactly as the reference writes them: (T)(float literal) */
#define C18 ((REAL)(1.0f / 18.0f))
#define C36 ((REAL)(1.0f / 36.0f))
#define C3 ((REAL)(1.0f / 3.0f))
#define K3 ((REAL)(3.0f))
#define KM3 ((REAL)(-3.0f))
#define K45 ((REAL)(9.0f / 2.0f))
#define K15 ((REAL)(3.0f / 2.0f))

static REAL weight(int i) { return i == 18 ? C3 : (i < 4 || i >= 16) ? C18 : C36; }

/* ---------------------------------------------------------------- storage */
#if VARIANT == 3
static inline REAL bf16_to_f(uint16_t b) {
    uint32_t u = ((uint32_t)b) << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static inline uint16_t f_to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u); /* quiet NaN */
    u += 0x7fffu + ((u >> 16) & 1u); /* round to nearest even */
    return (uint16_t)(u >> 16);
}
#define LD(p, i) (bf16_to_f(p) + weight(i))
#define STV(v, i) (f_to_bf16((v) - weight(i)))
#define LDD(p) (bf16_to_f(p))
#define STD(v) (f_to_bf16(v))
#elif VARIANT == 4
/* c16, this project's 16-bit float for the deviations (no reference
 * counterpart): sign, 3 exponent bits e, 12 fraction bits m; e = 1..7 gives
 * (1 + m/2^12) 2^(e-12), e = 0 gives m 2^-23; |g| < 2^-4, larger magnitudes
 * saturate.  It is float's bit layout with the exponents moved down by 115
 * binades.  Encoding scales |g| by 2^-115 (one float rounding, which only
 * values in the subnormal range undergo), then rounds the float's fraction
 * to 12 bits, halves away from zero; decoding places the bits into a float
 * and scales back by 2^115 (exact).  Needs subnormal floats (no flush to
 * zero). */
static inline REAL c16_dec(uint16_t c) {
    int32_t w = (int32_t)((uint32_t)c << 16);
    uint32_t u = (uint32_t)(w >> 5) & 0x83fff800u; /* arithmetic shift: the sign stays in bit 31 */
    float x;
    memcpy(&x, &u, 4);
    return x * 0x1p115f;
}
static inline uint16_t c16_enc(REAL v) {
    float x = fabsf(v) * 0x1p-115f;
    uint32_t a, u;
    memcpy(&a, &x, 4);
    memcpy(&u, &v, 4);
    uint32_t r = (a + 0x400u) >> 11;
    return (uint16_t)(((u >> 16) & 0x8000u) | (r < 0x7fffu ? r : 0x7fffu));
}
#define LD(p, i) (c16_dec(p) + weight(i))
#define STV(v, i) (c16_enc((v) - weight(i)))
#define LDD(p) (c16_dec(p))
#define STD(v) (c16_enc(v))
#elif VARIANT == 2
#define LD(p, i) ((REAL)(p) + weight(i))
#define STV(v, i) ((STOR)((v) - weight(i)))
#define LDD(p) ((REAL)(p))
#define STD(v) ((STOR)(v))
#else
#define LD(p, i) (p)
#define STV(v, i) (v)
#endif

/* --------------------------------------------------------------- indexing */
typedef struct {
    int64_t nx, ny, nz, n, slice;
    int64_t wg;      /* work-group size of the reference beta kernel, 0 = none */
    int group_wrap;  /* 1 when nx divides wg: lbm_beta.cl:221-227 */
} grid_t;

static grid_t mkgrid(int64_t nx, int64_t ny, int64_t nz, int64_t wg) {
    grid_t g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.slice = nx * ny;
    g.n = nx * ny * nz;
    g.wg = wg;
    g.group_wrap = (wg > 0) && ((wg / nx) * nx == wg);
    return g;
}

static inline int64_t modn(int64_t a, int64_t n) {
    int64_t r = a % n;
    return r < 0 ? r + n : r;
}

/* Cell reached from c by moving along (dx,dy,dz), wrapped linearly over the
 * whole buffer (wrap.h:112-127).  When the reference's beta work-group
 * realignment applies (group_wrap), the x part of the move wraps inside the
 * work-group instead (lbm_beta.cl:218-234,258-262,716-743). */
static inline int64_t nbr(const grid_t *g, int64_t c, int dx, int dy, int dz) {
    int64_t yz = (int64_t)dy * g->nx + (int64_t)dz * g->slice;
    if (dx != 0 && g->group_wrap) {
        int64_t lid = c % g->wg;
        int64_t start = c - lid;
        return modn(start + modn(lid + dx, g->wg) + yz, g->n);
    }
    return modn(c + dx + yz, g->n);
}

/* ------------------------------------------------------------- equilibria */
/* lbm_header.h:68-94 */
static inline REAL eq_a0(REAL v, REAL v2, REAL r) { return C18 * ((r + K3 * v) + K45 * v2); }
static inline REAL eq_a1(REAL v, REAL v2, REAL r) { return C18 * ((r + KM3 * v) + K45 * v2); }
static inline REAL eq_d4(REAL s, REAL s2, REAL r) { return C36 * ((r + K3 * s) + K45 * s2); }
static inline REAL eq_d5(REAL s, REAL s2, REAL r) { return C36 * ((r + KM3 * s) + K45 * s2); }

/* All 19 equilibria for velocity (vx,vy,vz) and dd_param dp, each value
 * computed with the reference's expression (lbm_alpha.cl:180-300). */
static void equilibria(REAL vx, REAL vy, REAL vz, REAL dp, REAL eq[19]) {
    REAL v2, s;
    v2 = vx * vx;
    eq[0] = eq_a0(vx, v2, dp);
    eq[1] = eq_a1(vx, v2, dp);
    v2 = vy * vy;
    eq[2] = eq_a0(vy, v2, dp);
    eq[3] = eq_a1(vy, v2, dp);
    s = vx + vy; v2 = s * s;
    eq[4] = eq_d4(s, v2, dp);
    eq[5] = eq_d5(s, v2, dp);
    s = vx - vy; v2 = s * s;
    eq[6] = eq_d4(s, v2, dp);
    eq[7] = eq_d5(s, v2, dp);
    s = vx + vz; v2 = s * s;
    eq[8] = eq_d4(s, v2, dp);
    eq[9] = eq_d5(s, v2, dp);
    s = vx - vz; v2 = s * s;
    eq[10] = eq_d4(s, v2, dp);
    eq[11] = eq_d5(s, v2, dp);
    s = vy + vz; v2 = s * s;
    eq[12] = eq_d4(s, v2, dp);
    eq[13] = eq_d5(s, v2, dp);
    s = vy - vz; v2 = s * s;
    eq[14] = eq_d4(s, v2, dp);
    eq[15] = eq_d5(s, v2, dp);
    v2 = vz * vz;
    eq[16] = eq_a0(vz, v2, dp);
    eq[17] = eq_a1(vz, v2, dp);
    eq[18] = C3 * dp;
}

/* Relaxation rate for one cell: the constant inv_tau when the subgrid model
 * is off (les_c == 0, identical to the reference), else the Smagorinsky rate.
 * The non-equilibrium stress is taken from moments of the pre-collision
 * populations, Pi_ab = sum_i e_ia e_ib f_i - rho/3 delta_ab - u_a u_b (the
 * second moment of the incompressible equilibrium is rho/3 delta + u u),
 * built from the nine opposite-pair sums p_k = f_2k + f_2k+1. */
static inline REAL relax_rate(const REAL f[19], REAL rho, REAL vx, REAL vy, REAL vz, REAL inv_tau, REAL tau0,
                              REAL les_c) {
    if (les_c == (REAL)0) return inv_tau;
    REAL p[9];
    for (int k = 0; k < 9; k++) p[k] = f[2 * k] + f[2 * k + 1];
    REAL sxx = (((p[0] + p[2]) + p[3]) + p[4]) + p[5];
    REAL syy = (((p[1] + p[2]) + p[3]) + p[6]) + p[7];
    REAL szz = (((p[4] + p[5]) + p[6]) + p[7]) + p[8];
    REAL r3 = rho * C3;
    REAL pxx = (sxx - r3) - vx * vx;
    REAL pyy = (syy - r3) - vy * vy;
    REAL pzz = (szz - r3) - vz * vz;
    REAL pxy = (p[2] - p[3]) - vx * vy;
    REAL pxz = (p[4] - p[5]) - vx * vz;
    REAL pyz = (p[6] - p[7]) - vy * vz;
    REAL q = ((pxx * pxx + pyy * pyy) + pzz * pzz) + (REAL)2 * ((pxy * pxy + pxz * pxz) + pyz * pyz);
    REAL te = (REAL)0.5 * (tau0 + RSQRT(tau0 * tau0 + les_c * RSQRT(q)));
    return (REAL)1 / te;
}

/* BGK collision of a FLUID cell, f updated in place: lbm_beta.cl:497-559 /
 * lbm_alpha.cl:179-303 without the gravity terms.  rho is the population
 * sum (before the reference aliases it), dp the equilibrium's dd_param. */
static void collide(REAL f[19], REAL rho, REAL vx, REAL vy, REAL vz, REAL dp, REAL inv_tau, REAL tau0,
                    REAL les_c) {
    REAL eq[19];
    REAL w = relax_rate(f, rho, vx, vy, vz, inv_tau, tau0, les_c);
    equilibria(vx, vy, vz, dp, eq);
    for (int i = 0; i < 19; i++) f[i] += w * (eq[i] - f[i]);
}

/* The alpha kernel's gravity terms.  The reference aliases its temporary to
 * rho (lbm_alpha.cl:173), so each pair's force term is the previous term
 * times the next coefficient and the stored density is the last term.
 * t[k] is added to f[2k] and subtracted from f[2k+1].  gmode 1 is the
 * optional per-term forcing: term k = coefficient k times the density. */
static REAL gravity_chain(REAL rho, REAL gx, REAL gy, REAL gz, REAL t[9], int gmode) {
    if (gmode) { /* per-term forcing (not the reference's): coefficient k times the density */
        t[0] = gx * C18 * rho;
        t[1] = gy * ((REAL)(-1.0f / 18.0f)) * rho;
        t[2] = (gx - gy) * C36 * rho;
        t[3] = (gx + gy) * C36 * rho;
        t[4] = (gx + gz) * C36 * rho;
        t[5] = (gx - gz) * C36 * rho;
        t[6] = (gz - gy) * C36 * rho;
        t[7] = (gz + gy) * ((REAL)(-1.0f / 36.0f)) * rho;
        t[8] = gz * C18 * rho;
        return rho;
    }
    REAL r = rho;
    r = gx * C18 * r; t[0] = r;
    r = gy * ((REAL)(-1.0f / 18.0f)) * r; t[1] = r;
    r = (gx - gy) * C36 * r; t[2] = r;
    r = (gx + gy) * C36 * r; t[3] = r;
    r = (gx + gz) * C36 * r; t[4] = r;
    r = (gx - gz) * C36 * r; t[5] = r;
    r = (gz - gy) * C36 * r; t[6] = r;
    r = (gz + gy) * ((REAL)(-1.0f / 36.0f)) * r; t[7] = r;
    r = gz * C18 * r; t[8] = r;
    return r;
}

#if SHIFTED
/* ----------------------------------------------------------- deviation form
 * Collision of the shifted types on the stored deviations g_i = f_i - w_i:
 *   rho - 1 = sum g_i + CW,  j = sum e_i g_i,  u = j (incompressible form),
 *   A = dd_param - 1 = (rho - 1) - 3/2 |u|^2,
 *   f_i^eq - w_i = w_i (A + 3 e_i.u + 9/2 (e_i.u)^2),
 *   g_i' = (1 - omega) g_i + omega (f_i^eq - w_i),
 * per opposite pair (2k, 2k+1) as P +- Q, P = omega w A + (9/2 omega w s) s,
 * Q = 3 omega w s, s = e_2k.u, Q folded into each population's last fused
 * multiply-add.  CW = sum of the float weights - 1 = 2^-26 and
 * CP = 2 w18 + 8 w36 - (float)(1/3) = -2^-27 keep the float weights' exact
 * offsets, so the model is the reference's one.  Subgrid rate:
 *   Pi_ab = sum e_a e_b g + CP delta - (rho - 1)/3 delta - u_a u_b,
 *   omega = 2 / (tau0 + sqrt(tau0^2 + C sqrt(Pi:Pi))).
 * Every fmaf is a single-rounding fused multiply-add, as on the GPU. */
#define CW 0x1p-26f
#define CP (-0x1p-27f)

static void dev_moments(const REAL g[19], REAL *dl, REAL *jx, REAL *jy, REAL *jz, REAL m2[6]) {
    REAL s[9], t[9];
    for (int k = 0; k < 9; k++) {
        s[k] = g[2 * k] + g[2 * k + 1];
        t[k] = g[2 * k] - g[2 * k + 1];
    }
    REAL a23 = s[2] + s[3], a45 = s[4] + s[5], a67 = s[6] + s[7];
    *dl = ((((s[0] + s[1]) + a23) + (a45 + a67)) + (s[8] + g[18])) + CW;
    *jx = ((t[0] + t[2]) + (t[3] + t[4])) + t[5];
    *jy = ((t[1] + t[2]) - t[3]) + (t[6] + t[7]);
    *jz = ((t[4] - t[5]) + (t[6] - t[7])) + t[8];
    m2[0] = (s[0] + a23) + a45;
    m2[1] = (s[1] + a23) + a67;
    m2[2] = (s[8] + a45) + a67;
    m2[3] = s[2] - s[3];
    m2[4] = s[4] - s[5];
    m2[5] = s[6] - s[7];
}

static void dev_pair(REAL g[19], int k, REAL v, REAL aA, REAL a45, REAL b, REAL om1) {
    REAL P = fmaf(a45 * v, v, aA);
    g[2 * k] = fmaf(b, v, fmaf(om1, g[2 * k], P));
    g[2 * k + 1] = fmaf(-b, v, fmaf(om1, g[2 * k + 1], P));
}

static void dev_relax(REAL g[19], REAL om, REAL A, REAL vx, REAL vy, REAL vz) {
    REAL om1 = (REAL)1.0f - om;
    REAL a18 = om * C18, a36 = om * C36, a3 = om * C3;
    REAL b18 = K3 * a18, b36 = K3 * a36;
    REAL aA18 = a18 * A, aA36 = a36 * A;
    REAL h18 = K45 * a18, h36 = K45 * a36;
    dev_pair(g, 0, vx, aA18, h18, b18, om1);
    dev_pair(g, 1, vy, aA18, h18, b18, om1);
    dev_pair(g, 2, vx + vy, aA36, h36, b36, om1);
    dev_pair(g, 3, vx - vy, aA36, h36, b36, om1);
    dev_pair(g, 4, vx + vz, aA36, h36, b36, om1);
    dev_pair(g, 5, vx - vz, aA36, h36, b36, om1);
    dev_pair(g, 6, vy + vz, aA36, h36, b36, om1);
    dev_pair(g, 7, vy - vz, aA36, h36, b36, om1);
    dev_pair(g, 8, vz, aA18, h18, b18, om1);
    g[18] = fmaf(om1, g[18], a3 * A);
}

static void dev_equilibria(REAL vx, REAL vy, REAL vz, REAL A, REAL g[19]) {
    REAL b18 = K3 * C18, b36 = K3 * C36;
    REAL v[9] = {vx, vy, vx + vy, vx - vy, vx + vz, vx - vz, vy + vz, vy - vz, vz};
    for (int k = 0; k < 9; k++) {
        int axis = k < 2 || k == 8;
        REAL h = fmaf(K45 * v[k], v[k], A);
        REAL P = (axis ? C18 : C36) * h, Q = (axis ? b18 : b36) * v[k];
        g[2 * k] = P + Q;
        g[2 * k + 1] = P - Q;
    }
    g[18] = C3 * A;
}

static void dev_collide(REAL g[19], REAL dl, REAL vx, REAL vy, REAL vz, const REAL m2[6], REAL A, REAL inv_tau,
                        REAL tau0, REAL les_c) {
    REAL om = inv_tau;
    if (les_c != (REAL)0) {
        REAL pxx = fmaf(-vx, vx, fmaf(-C3, dl, m2[0] + CP));
        REAL pyy = fmaf(-vy, vy, fmaf(-C3, dl, m2[1] + CP));
        REAL pzz = fmaf(-vz, vz, fmaf(-C3, dl, m2[2] + CP));
        REAL pxy = fmaf(-vx, vy, m2[3]);
        REAL pxz = fmaf(-vx, vz, m2[4]);
        REAL pyz = fmaf(-vy, vz, m2[5]);
        REAL off = fmaf(pyz, pyz, fmaf(pxz, pxz, pxy * pxy));
        REAL dia = fmaf(pzz, pzz, fmaf(pyy, pyy, pxx * pxx));
        REAL q = fmaf((REAL)2.0f, off, dia);
        om = (REAL)2.0f / (tau0 + sqrtf(fmaf(les_c, sqrtf(q), tau0 * tau0)));
    }
    dev_relax(g, om, A, vx, vy, vz);
}

static REAL dev_dp1(REAL vx, REAL vy, REAL vz, REAL dl) {
    REAL u2 = fmaf(vz, vz, fmaf(vy, vy, vx * vx));
    return fmaf(-K15, u2, dl);
}
#endif

/* ------------------------------------------------------------------- init */
/* lbm_init.cl:32-237: flags from the six face conditions (x faces win over
 * y faces, y over z), populations at rest equilibrium rho = 1, u = 0 in
 * standard slots, u = 0, rho = 1. */
void SFX(orc_init)(STOR *dd, int32_t *flags, REAL *vel, REAL *rho, const int32_t *bc,
                   int64_t nx, int64_t ny, int64_t nz) {
    grid_t g = mkgrid(nx, ny, nz, 0);
    REAL eq[19];
    REAL dp = (REAL)1.0f - K15 * ((REAL)0 * (REAL)0);
    equilibria((REAL)0, (REAL)0, (REAL)0, dp, eq);
    for (int64_t c = 0; c < g.n; c++) {
        int64_t x = c % nx, y = (c / nx) % ny, z = c / g.slice;
        int32_t fl = FL_FLUID;
        if (x == 0) fl = bc[0];
        else if (x == nx - 1) fl = bc[1];
        else if (y == 0) fl = bc[2];
        else if (y == ny - 1) fl = bc[3];
        else if (z == 0) fl = bc[4];
        else if (z == nz - 1) fl = bc[5];
        for (int i = 0; i < 19; i++) dd[i * g.n + c] = STV(eq[i], i);
        flags[c] = fl;
        if (vel) { vel[c] = 0; vel[g.n + c] = 0; vel[2 * g.n + c] = 0; }
        if (rho) rho[c] = (REAL)1.0f;
    }
}

/* ------------------------------------------------------------------ alpha */
void SFX(orc_alpha)(STOR *dd, const int32_t *flags, REAL *vel, REAL *rho, int64_t nx, int64_t ny,
                    int64_t nz, REAL inv_tau, REAL gx, REAL gy, REAL gz, REAL lid, int store_vel,
                    int store_rho, REAL tau0, REAL les_c, int gmode) {
    grid_t g = mkgrid(nx, ny, nz, 0);
    const int64_t n = g.n;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; c++) {
        int32_t fl = flags[c];
        if (fl == FL_GHOST) continue; /* lbm_alpha.cl:31-32 */
#if SHIFTED
        {
            REAL g[19], m2[6], dl, vx, vy, vz, r, t[9];
            int write = 0;
            for (int i = 0; i < 19; i++) g[i] = LDD(dd[i * n + c]);
            dev_moments(g, &dl, &vx, &vy, &vz, m2);
            r = (REAL)1.0f + dl;
            if (fl == FL_FLUID) {
                REAL A = dev_dp1(vx, vy, vz, dl);
                dev_collide(g, dl, vx, vy, vz, m2, A, inv_tau, tau0, les_c);
                r = gravity_chain(r, gx, gy, gz, t, gmode);
                write = 1;
            } else if (fl == FL_OBSTACLE) {
                vx = 0; vy = 0; vz = 0;
            } else if (fl == FL_LID) {
                vx = lid; vy = 0; vz = 0;
                REAL A = -K15 * (vx * vx);
                dev_equilibria(vx, vy, vz, A, g);
                r = gravity_chain((REAL)1.0f, gx, gy, gz, t, gmode);
                write = 1;
            }
            if (write) {
                if (gx != 0 || gy != 0 || gz != 0)
                    for (int k = 0; k < 9; k++) {
                        g[2 * k + 1] -= t[k];
                        g[2 * k] += t[k];
                    }
                for (int i = 0; i < 19; i++) dd[opp(i) * n + c] = STD(g[i]);
            }
            if (store_vel) { vel[c] = vx; vel[n + c] = vy; vel[2 * n + c] = vz; }
            if (store_rho) rho[c] = r;
            continue;
        }
#endif
        REAL f[19];
        for (int i = 0; i < 19; i++) f[i] = LD(dd[i * n + c], i);
        /* moments in the order of lbm_alpha.cl:61-156 */
        REAL r, vx, vy, vz;
        r = f[0]; vx = f[0];
        r += f[1]; vx -= f[1];
        r += f[2]; vy = f[2];
        r += f[3]; vy -= f[3];
        r += f[4]; vx += f[4]; vy += f[4];
        r += f[5]; vx -= f[5]; vy -= f[5];
        r += f[6]; vx += f[6]; vy -= f[6];
        r += f[7]; vx -= f[7]; vy += f[7];
        r += f[8]; vx += f[8]; vz = f[8];
        r += f[9]; vx -= f[9]; vz -= f[9];
        r += f[10]; vx += f[10]; vz -= f[10];
        r += f[11]; vx -= f[11]; vz += f[11];
        r += f[12]; vy += f[12]; vz += f[12];
        r += f[13]; vy -= f[13]; vz -= f[13];
        r += f[14]; vy += f[14]; vz -= f[14];
        r += f[15]; vy -= f[15]; vz += f[15];
        r += f[16]; vz += f[16];
        r += f[17]; vz -= f[17];
        r += f[18];
        int write = 0;
        REAL t[9];
        if (fl == FL_FLUID) {
            REAL v2 = (vx * vx + vy * vy) + vz * vz;
            REAL dp = r - K15 * v2;
            collide(f, r, vx, vy, vz, dp, inv_tau, tau0, les_c);
            r = gravity_chain(r, gx, gy, gz, t, gmode);
            write = 1;
        } else if (fl == FL_OBSTACLE) {
            vx = 0; vy = 0; vz = 0; /* lbm_alpha.cl:338-342, no population write */
        } else if (fl == FL_LID) {
            vx = lid; vy = 0; vz = 0;
            r = (REAL)1.0f;
            REAL v2 = (vx * vx + vy * vy) + vz * vz;
            REAL dp = r - K15 * v2;
            equilibria(vx, vy, vz, dp, f);
            r = gravity_chain(r, gx, gy, gz, t, gmode);
            write = 1;
        }
        if (write) {
            for (int k = 0; k < 9; k++) {
                f[2 * k + 1] -= t[k];
                f[2 * k] += t[k];
            }
            /* store into the opposite slot (lbm_alpha.cl:185-301) */
            for (int i = 0; i < 19; i++) dd[opp(i) * n + c] = STV(f[i], opp(i));
        }
        if (store_vel) { vel[c] = vx; vel[n + c] = vy; vel[2 * n + c] = vz; }
        if (store_rho) rho[c] = r;
    }
}

/* ------------------------------------------------------------------- beta */
void SFX(orc_beta)(STOR *dd, const int32_t *flags, REAL *vel, REAL *rho, int64_t nx, int64_t ny,
                   int64_t nz, REAL inv_tau, REAL gx, REAL gy, REAL gz, REAL lid, int store_vel,
                   int store_rho, REAL tau0, REAL les_c, int64_t wg) {
    (void)gx; (void)gy; (void)gz; /* gravity is compiled out of beta: lbm_beta.cl:2,658 */
    grid_t g = mkgrid(nx, ny, nz, wg);
    const int64_t n = g.n;
    /* In-place A-A update: the only cell that reads a location another cell
     * writes in this step is that same cell, so cells are independent. */
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; c++) {
        int32_t fl = flags[c];
        REAL f[19];
        int64_t src[19], dst[19];
        for (int i = 0; i < 19; i++) {
            src[i] = nbr(&g, c, -EX[i], -EY[i], -EZ[i]);
            dst[i] = nbr(&g, c, EX[i], EY[i], EZ[i]);
        }
#if SHIFTED
        {
            REAL g[19], m2[6], dl, vx, vy, vz, r;
            for (int i = 0; i < 19; i++) g[i] = LDD(dd[opp(i) * n + src[i]]);
            dev_moments(g, &dl, &vx, &vy, &vz, m2);
            r = (REAL)1.0f + dl;
            if (fl == FL_FLUID) {
                REAL A = dev_dp1(vx, vy, vz, dl);
                dev_collide(g, dl, vx, vy, vz, m2, A, inv_tau, tau0, les_c);
                r = (REAL)1.0f + A;
            } else if (fl == FL_OBSTACLE) {
                vx = 0; vy = 0; vz = 0;
                for (int k = 0; k < 9; k++) {
                    REAL tmp = g[2 * k + 1];
                    g[2 * k + 1] = g[2 * k];
                    g[2 * k] = tmp;
                }
            } else if (fl == FL_LID) {
                vx = lid; vy = 0; vz = 0;
                REAL A = -K15 * (vx * vx);
                dev_equilibria(vx, vy, vz, A, g);
                r = (REAL)1.0f + A;
            }
            for (int i = 0; i < 19; i++) dd[i * n + dst[i]] = STD(g[i]);
            if (fl == FL_GHOST) continue;
            if (store_vel) { vel[c] = vx; vel[n + c] = vy; vel[2 * n + c] = vz; }
            if (store_rho) rho[c] = r;
            continue;
        }
#endif
        for (int i = 0; i < 19; i++) f[i] = LD(dd[opp(i) * n + src[i]], i);
        /* moments in the order of lbm_beta.cl:261-483 */
        REAL r, vx, vy, vz;
        r = f[3]; vy = -f[3];
        r += f[2]; vy += f[2];
        r += f[0]; vx = f[0];
        r += f[1]; vx -= f[1];
        r += f[4]; vx += f[4]; vy += f[4];
        r += f[5]; vx -= f[5]; vy -= f[5];
        r += f[6]; vx += f[6]; vy -= f[6];
        r += f[7]; vx -= f[7]; vy += f[7];
        r += f[8]; vx += f[8]; vz = f[8];
        r += f[9]; vx -= f[9]; vz -= f[9];
        r += f[10]; vx += f[10]; vz -= f[10];
        r += f[11]; vx -= f[11]; vz += f[11];
        r += f[13]; vy -= f[13]; vz -= f[13];
        r += f[12]; vy += f[12]; vz += f[12];
        r += f[15]; vy -= f[15]; vz += f[15];
        r += f[14]; vy += f[14]; vz -= f[14];
        r += f[17]; vz -= f[17];
        r += f[16]; vz += f[16];
        r += f[18];
        if (fl == FL_FLUID) {
            REAL v2 = (vx * vx + vy * vy) + vz * vz;
            REAL dp = r - K15 * v2;
            collide(f, r, vx, vy, vz, dp, inv_tau, tau0, les_c);
            r = dp; /* dd_param aliases rho: lbm_beta.cl:493 */
        } else if (fl == FL_OBSTACLE) {
            vx = 0; vy = 0; vz = 0;
            for (int k = 0; k < 9; k++) { /* bounce back: lbm_beta.cl:570-578 */
                REAL tmp = f[2 * k + 1];
                f[2 * k + 1] = f[2 * k];
                f[2 * k] = tmp;
            }
        } else if (fl == FL_LID) {
            vx = lid; vy = 0; vz = 0;
            r = (REAL)1.0f;
            REAL v2 = (vx * vx + vy * vy) + vz * vz;
            r = r - K15 * v2;
            equilibria(vx, vy, vz, r, f);
        }
        /* scatter to the neighbours (lbm_beta.cl:708-784) */
        for (int i = 0; i < 19; i++) dd[i * n + dst[i]] = STV(f[i], i);
        if (fl == FL_GHOST) continue;
        if (store_vel) { vel[c] = vx; vel[n + c] = vy; vel[2 * n + c] = vz; }
        if (store_rho) rho[c] = r;
    }
}

/* ---------------------------------------------- seeded perturbed start-up */
/* Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11, "Parallel random
 * numbers: as easy as 1, 2, 3").  Keyed by the seed, counter = physical cell
 * index, so that the field is independent of the decomposition. */
static void philox4x32_10(uint32_t ctr[4], uint32_t key0, uint32_t key1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int round = 0; round < 10; round++) {
        uint64_t p0 = (uint64_t)M0 * ctr[0];
        uint64_t p1 = (uint64_t)M1 * ctr[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ ctr[1] ^ key0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ ctr[3] ^ key1;
        uint32_t n3 = lo0;
        ctr[0] = n0; ctr[1] = n1; ctr[2] = n2; ctr[3] = n3;
        key0 += W0;
        key1 += W1;
    }
}

#if VARIANT == 0
void orc_philox(uint64_t idx, uint64_t seed, uint32_t out[4]);
void orc_philox(uint64_t idx, uint64_t seed, uint32_t out[4]) {
    uint32_t c[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    memcpy(out, c, sizeof(c));
}
#endif

static void philox_cell(uint64_t idx, uint64_t seed, uint32_t out[4]) {
    uint32_t c[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    memcpy(out, c, sizeof(c));
}

/* Velocity perturbation of one physical cell, uniform on [-amp, amp). */
static void perturb_velocity(uint64_t idx, uint64_t seed, double amp, REAL u[3]) {
    uint32_t r[4];
    philox_cell(idx, seed, r);
    for (int a = 0; a < 3; a++) {
        double unit = (double)(r[a] >> 8) * (1.0 / 16777216.0);
        u[a] = (REAL)((unit * 2.0 - 1.0) * amp);
    }
}

/* Overwrite every cell that lies strictly inside the physical domain with
 * eq(rho = 1, u) for a seeded random u, in opposite-slot order (the layout
 * the first beta step reads).  (ox,oy,oz) is the subdomain's physical
 * origin and (gx,gy,gz) the physical domain size; cells on the physical
 * boundary keep the rest state written by init. */
void SFX(orc_perturb)(STOR *dd, REAL *vel, REAL *rho, int64_t nx, int64_t ny, int64_t nz,
                      int64_t ox, int64_t oy, int64_t oz, int64_t gx, int64_t gy, int64_t gz,
                      uint64_t seed, double amp) {
    grid_t g = mkgrid(nx, ny, nz, 0);
    const int64_t n = g.n;
    for (int64_t c = 0; c < n; c++) {
        int64_t px = ox + c % nx, py = oy + (c / nx) % ny, pz = oz + c / g.slice;
        if (px <= 0 || py <= 0 || pz <= 0 || px >= gx - 1 || py >= gy - 1 || pz >= gz - 1) continue;
        REAL u[3], eq[19];
        perturb_velocity((uint64_t)((pz * gy + py) * gx + px), seed, amp, u);
        REAL v2 = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2];
        REAL dp = (REAL)1.0f - K15 * v2;
        equilibria(u[0], u[1], u[2], dp, eq);
        for (int i = 0; i < 19; i++) dd[opp(i) * n + c] = STV(eq[i], opp(i));
        if (vel) { vel[c] = u[0]; vel[n + c] = u[1]; vel[2 * n + c] = u[2]; }
        if (rho) rho[c] = (REAL)1.0f;
    }
}

/* -------------------------------------------------------- storage helpers */
/* Decode stored populations to REAL (adds the shift back for f16/bf16). */
void SFX(orc_decode)(const STOR *dd, REAL *out, int64_t n) {
    for (int i = 0; i < 19; i++)
        for (int64_t c = 0; c < n; c++) out[i * n + c] = LD(dd[i * n + c], i);
}

/* Encode REAL populations into storage (subtracts the shift for f16/bf16). */
void SFX(orc_encode)(const REAL *in, STOR *dd, int64_t n) {
    for (int i = 0; i < 19; i++)
        for (int64_t c = 0; c < n; c++) dd[i * n + c] = STV(in[i * n + c], i);
}

#if VARIANT == 4
/* The c16 format alone (no weight shift): for the format's own tests. */
void orc_c16_encode_raw(const float *in, uint16_t *out, int64_t n);
void orc_c16_decode_raw(const uint16_t *in, float *out, int64_t n);
void orc_c16_encode_raw(const float *in, uint16_t *out, int64_t n) {
    for (int64_t k = 0; k < n; k++) out[k] = c16_enc(in[k]);
}
void orc_c16_decode_raw(const uint16_t *in, float *out, int64_t n) {
    for (int64_t k = 0; k < n; k++) out[k] = c16_dec(in[k]);
}
#endif
