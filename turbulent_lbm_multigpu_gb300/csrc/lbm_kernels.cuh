// lbm_kernels.cuh -- D3Q19 A-A lattice Boltzmann kernels for sm_103a.
//
// One in-place population buffer per lattice, structure of arrays: 19 planes
// of `pstride` elements, cells x-fastest (the reference layout,
// src/cl_programs/lbm_header.h:22-27, with each plane padded to a 256-byte
// boundary).  Steps alternate between
//   beta  (even step counter): gather f_i from (c - e_i, slot opp(i)),
//         collide, scatter f_i to (c + e_i, slot i)
//         -- src/cl_programs/lbm_beta.cl:13-802;
//   alpha (odd step counter):  read the 19 slots of c, collide, write each
//         f_i back into slot opp(i) of c -- src/cl_programs/lbm_alpha.cl:12-498.
// The only thread that reads a location another thread writes in a step is
// the writing thread itself, so both kernels update the buffer in place with
// no synchronisation.
//
// Arithmetic follows the reference kernels operation by operation.  This file
// is compiled with -fmad=false and IEEE division/square root, which makes the
// results bit-identical to the reference kernel source run on a CPU.
//
// Population storage: float, double, or the shifted half / bfloat16 forms
// that store f_i - w_i and compute in float.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lbm {

enum : uint8_t { kObstacle = 1, kFluid = 2, kLid = 4, kGhost = 8 };
enum Storage : int { kF32 = 0, kF64 = 1, kF16 = 2, kBF16 = 3 };

// D3Q19 directions in reference order (src/main.cpp:38-66).
__host__ __device__ constexpr int dir_x(int i) {
    return (i == 0 || i == 4 || i == 6 || i == 8 || i == 10) ? 1
           : (i == 1 || i == 5 || i == 7 || i == 9 || i == 11) ? -1 : 0;
}
__host__ __device__ constexpr int dir_y(int i) {
    return (i == 2 || i == 4 || i == 7 || i == 12 || i == 14) ? 1
           : (i == 3 || i == 5 || i == 6 || i == 13 || i == 15) ? -1 : 0;
}
__host__ __device__ constexpr int dir_z(int i) {
    return (i == 8 || i == 11 || i == 12 || i == 15 || i == 16) ? 1
           : (i == 9 || i == 10 || i == 13 || i == 14 || i == 17) ? -1 : 0;
}
__host__ __device__ constexpr int opp(int i) { return i == 18 ? 18 : (i ^ 1); }

// ---------------------------------------------------------------- storage
template <typename S> struct Store;
template <> struct Store<float> {
    using R = float;
    static constexpr bool kShifted = false;
    __device__ static __forceinline__ R ld(const float *p, R) { return *p; }
    __device__ static __forceinline__ void st(float *p, R v, R) { *p = v; }
};
template <> struct Store<double> {
    using R = double;
    static constexpr bool kShifted = false;
    __device__ static __forceinline__ R ld(const double *p, R) { return *p; }
    __device__ static __forceinline__ void st(double *p, R v, R) { *p = v; }
};
template <> struct Store<__half> {
    using R = float;
    static constexpr bool kShifted = true;
    __device__ static __forceinline__ R ld(const __half *p, R w) { return __half2float(*p) + w; }
    __device__ static __forceinline__ void st(__half *p, R v, R w) { *p = __float2half_rn(v - w); }
};
template <> struct Store<__nv_bfloat16> {
    using R = float;
    static constexpr bool kShifted = true;
    __device__ static __forceinline__ R ld(const __nv_bfloat16 *p, R w) { return __bfloat162float(*p) + w; }
    __device__ static __forceinline__ void st(__nv_bfloat16 *p, R v, R w) { *p = __float2bfloat16_rn(v - w); }
};

// Constants exactly as the reference writes them: (T)(float literal).
template <typename R> struct K {
    static constexpr R c18 = (R)(1.0f / 18.0f);
    static constexpr R c36 = (R)(1.0f / 36.0f);
    static constexpr R c3 = (R)(1.0f / 3.0f);
    static constexpr R k3 = (R)(3.0f);
    static constexpr R km3 = (R)(-3.0f);
    static constexpr R k45 = (R)(9.0f / 2.0f);
    static constexpr R k15 = (R)(3.0f / 2.0f);
};
template <typename R> __host__ __device__ constexpr R weight(int i) {
    return i == 18 ? K<R>::c3 : (i < 4 || i >= 16) ? K<R>::c18 : K<R>::c36;
}

// ---------------------------------------------------------- lattice table
// One entry per lattice (a subdomain or a cavity of a batch).  Kernel
// parameters are held in both precisions, already rounded to the
// arithmetic type on the host, so the device picks the one it computes in.
struct LatDesc {
    void *dd;          // population planes
    uint8_t *flags;    // one flag byte per cell
    void *vel;         // 3 planes of the arithmetic type, or null
    void *rho;         // 1 plane, or null
    int64_t pstride;   // plane stride in elements
    int64_t n;         // cells
    int32_t nx, ny, nz;
    int32_t first_block;  // first block of this lattice in a batched launch
    int32_t nblocks;
    int32_t grav;      // gravity chain non-zero (alpha kernel)
    double pd[16];     // inv_tau, tau0, les_c, lid, k0..k8 (gravity chain)
    float pf[16];
};
enum { P_INV_TAU = 0, P_TAU0 = 1, P_LES = 2, P_LID = 3, P_K0 = 4 };

template <typename R> __device__ __forceinline__ R par(const LatDesc &d, int i);
template <> __device__ __forceinline__ float par<float>(const LatDesc &d, int i) { return d.pf[i]; }
template <> __device__ __forceinline__ double par<double>(const LatDesc &d, int i) { return d.pd[i]; }

// Lattice of a block in a batched launch: binary search on first_block.
__device__ __forceinline__ int find_lattice(const LatDesc *tab, int ntab, int block) {
    int lo = 0, hi = ntab - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tab[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Arguments of a step launch.  Up to kParamLattices descriptors travel in
// the kernel parameter space (constant bank: block-uniform values stay in
// uniform registers); larger batches use a device table.
constexpr int kParamLattices = 8;
struct StepArgs {
    LatDesc tab[kParamLattices];
    const LatDesc *dtab;
    int ntab;
    int store_v, store_rho;
};

template <bool PT>
__device__ __forceinline__ const LatDesc &lattice_of(const StepArgs &a) {
    if (PT) {
        int li = 0;
        if (a.ntab > 1) {
            int hi = a.ntab - 1;
            while (li < hi) {
                const int mid = (li + hi + 1) >> 1;
                if (a.tab[mid].first_block <= (int)blockIdx.x) li = mid; else hi = mid - 1;
            }
        }
        return a.tab[li];
    }
    return a.dtab[find_lattice(a.dtab, a.ntab, blockIdx.x)];
}

// ------------------------------------------------------------- equilibria
// src/cl_programs/lbm_header.h:68-94
template <typename R> __device__ __forceinline__ R eq_a0(R v, R v2, R r) {
    return K<R>::c18 * ((r + K<R>::k3 * v) + K<R>::k45 * v2);
}
template <typename R> __device__ __forceinline__ R eq_a1(R v, R v2, R r) {
    return K<R>::c18 * ((r + K<R>::km3 * v) + K<R>::k45 * v2);
}
template <typename R> __device__ __forceinline__ R eq_d4(R s, R s2, R r) {
    return K<R>::c36 * ((r + K<R>::k3 * s) + K<R>::k45 * s2);
}
template <typename R> __device__ __forceinline__ R eq_d5(R s, R s2, R r) {
    return K<R>::c36 * ((r + K<R>::km3 * s) + K<R>::k45 * s2);
}

template <typename R>
__device__ __forceinline__ void equilibria(R vx, R vy, R vz, R dp, R eq[19]) {
    R v2, s;
    v2 = vx * vx; eq[0] = eq_a0(vx, v2, dp); eq[1] = eq_a1(vx, v2, dp);
    v2 = vy * vy; eq[2] = eq_a0(vy, v2, dp); eq[3] = eq_a1(vy, v2, dp);
    s = vx + vy; v2 = s * s; eq[4] = eq_d4(s, v2, dp); eq[5] = eq_d5(s, v2, dp);
    s = vx - vy; v2 = s * s; eq[6] = eq_d4(s, v2, dp); eq[7] = eq_d5(s, v2, dp);
    s = vx + vz; v2 = s * s; eq[8] = eq_d4(s, v2, dp); eq[9] = eq_d5(s, v2, dp);
    s = vx - vz; v2 = s * s; eq[10] = eq_d4(s, v2, dp); eq[11] = eq_d5(s, v2, dp);
    s = vy + vz; v2 = s * s; eq[12] = eq_d4(s, v2, dp); eq[13] = eq_d5(s, v2, dp);
    s = vy - vz; v2 = s * s; eq[14] = eq_d4(s, v2, dp); eq[15] = eq_d5(s, v2, dp);
    v2 = vz * vz; eq[16] = eq_a0(vz, v2, dp); eq[17] = eq_a1(vz, v2, dp);
    eq[18] = K<R>::c3 * dp;
}

__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }

// BGK collision of a fluid cell; with LES the relaxation rate comes from the
// Smagorinsky model of Hou, Sterling, Chen & Doolen (1996):
//   tau_eff = (tau0 + sqrt(tau0^2 + C sqrt(Q))) / 2,  Q = Pi:Pi,  C = 18 sqrt(2) Cs^2,
//   Pi_ab = sum_i e_ia e_ib f_i - rho/3 delta_ab - u_a u_b
// (the second moment of the incompressible equilibrium is rho/3 delta + u u),
// from the nine opposite-pair sums of the pre-collision populations.  rho is
// the population sum, dp the equilibrium's dd_param.
template <typename R, bool LES>
__device__ __forceinline__ void collide(R f[19], R rho, R vx, R vy, R vz, R dp, const LatDesc &d) {
    R w = par<R>(d, P_INV_TAU);
    if (LES && par<R>(d, P_LES) != (R)0) {
        R p[9];
#pragma unroll
        for (int k = 0; k < 9; k++) p[k] = f[2 * k] + f[2 * k + 1];
        const R sxx = (((p[0] + p[2]) + p[3]) + p[4]) + p[5];
        const R syy = (((p[1] + p[2]) + p[3]) + p[6]) + p[7];
        const R szz = (((p[4] + p[5]) + p[6]) + p[7]) + p[8];
        const R r3 = rho * K<R>::c3;
        const R pxx = (sxx - r3) - vx * vx;
        const R pyy = (syy - r3) - vy * vy;
        const R pzz = (szz - r3) - vz * vz;
        const R pxy = (p[2] - p[3]) - vx * vy;
        const R pxz = (p[4] - p[5]) - vx * vz;
        const R pyz = (p[6] - p[7]) - vy * vz;
        const R q = ((pxx * pxx + pyy * pyy) + pzz * pzz) + (R)2 * ((pxy * pxy + pxz * pxz) + pyz * pyz);
        const R tau0 = par<R>(d, P_TAU0);
        const R te = (R)0.5 * (tau0 + dsqrt(tau0 * tau0 + par<R>(d, P_LES) * dsqrt(q)));
        w = (R)1 / te;
    }
    R eq[19];
    equilibria<R>(vx, vy, vz, dp, eq);
#pragma unroll
    for (int i = 0; i < 19; i++) f[i] += w * (eq[i] - f[i]);
}

// Gravity terms of the alpha kernel.  The reference aliases its temporary to
// rho (lbm_alpha.cl:173): term k is coefficient k times term k-1, and the
// stored density is the last term.  Coefficients k0..k8 come pre-multiplied
// from the host.
template <typename R>
__device__ __forceinline__ R gravity_chain(R rho, const LatDesc &d, R t[9]) {
    R r = rho;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        r = par<R>(d, P_K0 + k) * r;
        t[k] = r;
    }
    return r;
}

__device__ __forceinline__ int64_t dir_off(int i, int64_t nx, int64_t slice) {
    return (int64_t)dir_x(i) + (int64_t)dir_y(i) * nx + (int64_t)dir_z(i) * slice;
}

// Cell reached from c by the signed offset `off`, wrapped over the whole
// buffer like the reference's DOMAIN_WRAP (src/cl_programs/wrap.h:112-127).
__device__ __forceinline__ int64_t wrap_cell(int64_t c, int64_t off, int64_t n) {
    int64_t i = c + off;
    if (i < 0) i += n;
    else if (i >= n) i -= n;
    return i;
}

// Resident blocks of 256 threads per SM the launch bounds ask for: 4 (64
// registers) where the float kernels fit without spilling, fewer for double.
template <typename S, bool LES, bool BETA>
__host__ __device__ constexpr int min_blocks() {
    return sizeof(typename Store<S>::R) == 8 ? 1 : (BETA || LES) ? 4 : 3;
}

// ------------------------------------------------------------------ beta
// WRAP: the block holds cells within reach of either end of the buffer;
// otherwise every neighbour address is the cell's address plus a
// block-uniform offset.
template <typename S, bool LES, bool WRAP>
__device__ __forceinline__ void beta_cell(const LatDesc &d, int64_t c, int store_v, int store_rho) {
    using R = typename Store<S>::R;
    S *const dd = (S *)d.dd;
    S *const pc = dd + c;
    const int64_t ps = d.pstride, nx = d.nx, sl = (int64_t)d.nx * d.ny, n = d.n;
    const int fl = d.flags[c];

    R f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const int64_t off = dir_off(i, nx, sl);
        const S *p = WRAP ? dd + opp(i) * ps + wrap_cell(c, -off, n) : pc + (opp(i) * ps - off);
        f[i] = Store<S>::ld(p, weight<R>(i));
    }
    // moments in the order of lbm_beta.cl:261-483
    R r, vx, vy, vz;
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

    if (fl == kFluid) {
        const R v2 = (vx * vx + vy * vy) + vz * vz;
        const R dp = r - K<R>::k15 * v2;
        collide<R, LES>(f, r, vx, vy, vz, dp, d);
        r = dp;  // dd_param aliases rho (lbm_beta.cl:493)
    } else if (fl == kObstacle) {
        vx = 0; vy = 0; vz = 0;
#pragma unroll
        for (int k = 0; k < 9; k++) {  // bounce back, lbm_beta.cl:570-578
            const R t = f[2 * k + 1];
            f[2 * k + 1] = f[2 * k];
            f[2 * k] = t;
        }
    } else if (fl == kLid) {
        vx = par<R>(d, P_LID); vy = 0; vz = 0;
        r = (R)1.0f;
        const R v2 = (vx * vx + vy * vy) + vz * vz;
        r = r - K<R>::k15 * v2;
        equilibria<R>(vx, vy, vz, r, f);
    }
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const int64_t off = dir_off(i, nx, sl);
        S *p = WRAP ? dd + i * ps + wrap_cell(c, off, n) : pc + (i * ps + off);
        Store<S>::st(p, f[i], weight<R>(i));
    }
    if (fl == kGhost) return;
    if (store_v) {
        R *u = (R *)d.vel + c;
        u[0] = vx; u[n] = vy; u[2 * n] = vz;
    }
    if (store_rho) ((R *)d.rho)[c] = r;
}

template <typename S, bool LES, bool PT>
__global__ void __launch_bounds__(256, (min_blocks<S, LES, true>())) k_beta(const __grid_constant__ StepArgs a) {
    const LatDesc &d = lattice_of<PT>(a);
    const int64_t c0 = (int64_t)(blockIdx.x - d.first_block) * blockDim.x;
    const int64_t c = c0 + threadIdx.x;
    if (c >= d.n) return;
    const int64_t reach = (int64_t)d.nx + (int64_t)d.nx * d.ny;
    if (c0 < reach || c0 + (int64_t)blockDim.x - 1 + reach >= d.n)
        beta_cell<S, LES, true>(d, c, a.store_v, a.store_rho);
    else
        beta_cell<S, LES, false>(d, c, a.store_v, a.store_rho);
}

// ----------------------------------------------------------------- alpha
template <typename S, bool LES, bool PT>
__global__ void __launch_bounds__(256, (min_blocks<S, LES, false>())) k_alpha(const __grid_constant__ StepArgs a) {
    using R = typename Store<S>::R;
    const LatDesc &d = lattice_of<PT>(a);
    const int64_t c = (int64_t)(blockIdx.x - d.first_block) * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const int fl = d.flags[c];
    if (fl == kGhost) return;  // lbm_alpha.cl:31-32
    S *const pc = (S *)d.dd + c;
    const int64_t ps = d.pstride;

    R f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) f[i] = Store<S>::ld(pc + i * ps, weight<R>(i));
    // moments in the order of lbm_alpha.cl:61-156
    R r, vx, vy, vz;
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

    bool write = false;
    R t[9];
    if (fl == kFluid) {
        const R v2 = (vx * vx + vy * vy) + vz * vz;
        const R dp = r - K<R>::k15 * v2;
        collide<R, LES>(f, r, vx, vy, vz, dp, d);
        r = gravity_chain<R>(r, d, t);
        write = true;
    } else if (fl == kObstacle) {
        vx = 0; vy = 0; vz = 0;  // lbm_alpha.cl:305-343, populations untouched
    } else if (fl == kLid) {
        vx = par<R>(d, P_LID); vy = 0; vz = 0;
        r = (R)1.0f;
        const R v2 = (vx * vx + vy * vy) + vz * vz;
        const R dp = r - K<R>::k15 * v2;
        equilibria<R>(vx, vy, vz, dp, f);
        r = gravity_chain<R>(r, d, t);
        write = true;
    }
    if (write) {
        if (d.grav) {
#pragma unroll
            for (int k = 0; k < 9; k++) {
                f[2 * k + 1] -= t[k];
                f[2 * k] += t[k];
            }
        }
        // each population goes to the opposite slot (lbm_alpha.cl:185-301)
#pragma unroll
        for (int i = 0; i < 19; i++) Store<S>::st(pc + opp(i) * ps, f[i], weight<R>(i));
    }
    if (a.store_v) {
        R *u = (R *)d.vel + c;
        u[0] = vx; u[d.n] = vy; u[2 * d.n] = vz;
    }
    if (a.store_rho) ((R *)d.rho)[c] = r;
}

}  // namespace lbm
