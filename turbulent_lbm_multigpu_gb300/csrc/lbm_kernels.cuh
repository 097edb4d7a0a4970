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
// For float and double storage the arithmetic follows the reference kernels
// operation by operation.  This file is compiled with -fmad=false and IEEE
// division/square root, which makes those results bit-identical to the
// reference kernel source run on a CPU.  The shifted 16-bit storage types
// (which the reference does not have) compute the same model in deviation
// form with explicit fused multiply-adds (see "deviation form" below); the
// CPU oracle states that arithmetic with fmaf, so it is bit-exact as well.
//
// Two kernel shapes:
//   k_beta / k_alpha    one cell per thread, any storage and size;
//   k_beta2 / k_alpha2  two neighbouring x cells per thread for the float
//                       arithmetic types and even nx: 64-bit loads/stores
//                       (32-bit for the 16-bit storage types), pairwise
//                       IEEE arithmetic, warp shuffles for the populations
//                       that move along x.
// Population storage: float, double, or the shifted half / bfloat16 forms
// that store f_i - w_i and compute in float.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>

namespace lbm {

enum : uint8_t { kObstacle = 1, kFluid = 2, kLid = 4, kGhost = 8 };
enum Storage : int { kF32 = 0, kF64 = 1, kF16 = 2, kBF16 = 3, kC16 = 4 };

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

// ------------------------------------------------------ float pairs
// Two float lanes (two cells).  Every lane is one IEEE round-to-nearest
// operation (__fadd_rn/__fsub_rn/__fmul_rn are never contracted into a
// multiply-add), so a pair computes exactly what two scalar cells compute.
// Blackwell's packed FP32x2 instructions (add/sub/mul/fma.rn.f32x2) are
// exact per lane when used alone (measured on GB300 against the scalar
// intrinsics over 2^20 random operands, subnormals included), but the
// assembler may fuse a packed multiply into a following packed add: the
// collision with packed arithmetic differed from the scalar one by up to
// 4 ulp in 1.4 % of the values.  So the lanes stay scalar.
struct P2 {
    float x, y;
};
__device__ __forceinline__ P2 operator+(P2 a, P2 b) { return P2{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)}; }
__device__ __forceinline__ P2 operator-(P2 a, P2 b) { return P2{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)}; }
__device__ __forceinline__ P2 operator*(P2 a, P2 b) { return P2{__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)}; }
__device__ __forceinline__ P2 operator-(P2 a) { return P2{-a.x, -a.y}; }
__device__ __forceinline__ P2 &operator+=(P2 &a, P2 b) { return a = a + b; }
__device__ __forceinline__ P2 &operator-=(P2 &a, P2 b) { return a = a - b; }

// broadcast of a scalar to the math type
template <typename M> struct Bc;
template <> struct Bc<float> { __device__ static __forceinline__ float of(float v) { return v; } };
template <> struct Bc<double> { __device__ static __forceinline__ double of(double v) { return v; } };
template <> struct Bc<P2> { __device__ static __forceinline__ P2 of(float v) { return P2{v, v}; } };
template <typename M> struct Scalar { using T = M; };
template <> struct Scalar<P2> { using T = float; };

__device__ __forceinline__ float msqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double msqrt(double x) { return sqrt(x); }
__device__ __forceinline__ P2 msqrt(P2 x) { return P2{sqrtf(x.x), sqrtf(x.y)}; }
__device__ __forceinline__ float mrcp(float x) { return 1.0f / x; }
__device__ __forceinline__ double mrcp(double x) { return 1.0 / x; }
__device__ __forceinline__ P2 mrcp(P2 x) { return P2{1.0f / x.x, 1.0f / x.y}; }
// a * b + c rounded once (IEEE fused multiply-add)
__device__ __forceinline__ float mfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ P2 mfma(P2 a, P2 b, P2 c) {
    return P2{__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y)};
}
__device__ __forceinline__ float mdiv(float a, float b) { return a / b; }
__device__ __forceinline__ P2 mdiv(P2 a, P2 b) { return P2{a.x / b.x, a.y / b.y}; }

// ---------------------------------------------------------------- storage
template <typename S> struct Store;
// ld/st convert between stored values and full populations f_i (used by
// init, start-up, box IO and reductions).  The step kernels of the shifted
// types move the stored deviations g_i = f_i - w_i without shifting (dld /
// dst), because their collision works on deviations (kDev).
template <> struct Store<float> {
    using R = float;
    static constexpr bool kDev = false;
    __device__ static __forceinline__ R ld(const float *p, R) { return *p; }
    __device__ static __forceinline__ void st(float *p, R v, R) { *p = v; }
    __device__ static __forceinline__ P2 ld2(const float *p, R) {
        const float2 v = *(const float2 *)p;
        return P2{v.x, v.y};
    }
    __device__ static __forceinline__ void st2(float *p, P2 v, R) { *(float2 *)p = make_float2(v.x, v.y); }
};
template <> struct Store<double> {
    using R = double;
    static constexpr bool kDev = false;
    __device__ static __forceinline__ R ld(const double *p, R) { return *p; }
    __device__ static __forceinline__ void st(double *p, R v, R) { *p = v; }
};
template <> struct Store<__half> {
    using R = float;
    static constexpr bool kDev = true;
    __device__ static __forceinline__ R dld(const __half *p) { return __half2float(*p); }
    __device__ static __forceinline__ void dst(__half *p, R v) { *p = __float2half_rn(v); }
    __device__ static __forceinline__ P2 dld2(const __half *p) {
        const float2 v = __half22float2(*(const __half2 *)p);
        return P2{v.x, v.y};
    }
    __device__ static __forceinline__ void dst2(__half *p, P2 v) { *(__half2 *)p = __floats2half2_rn(v.x, v.y); }
    __device__ static __forceinline__ uint32_t dbits(R v) { return __half_as_ushort(__float2half_rn(v)); }
    __device__ static __forceinline__ R ld(const __half *p, R w) { return __half2float(*p) + w; }
    __device__ static __forceinline__ void st(__half *p, R v, R w) { *p = __float2half_rn(v - w); }
    __device__ static __forceinline__ P2 ld2(const __half *p, R w) {
        const float2 v = __half22float2(*(const __half2 *)p);
        return P2{v.x, v.y} + P2{w, w};
    }
    __device__ static __forceinline__ void st2(__half *p, P2 v, R w) {
        const P2 t = v - P2{w, w};
        *(__half2 *)p = __floats2half2_rn(t.x, t.y);
    }
};
template <> struct Store<__nv_bfloat16> {
    using R = float;
    static constexpr bool kDev = true;
    __device__ static __forceinline__ R dld(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
    __device__ static __forceinline__ void dst(__nv_bfloat16 *p, R v) { *p = __float2bfloat16_rn(v); }
    __device__ static __forceinline__ P2 dld2(const __nv_bfloat16 *p) {
        const float2 v = __bfloat1622float2(*(const __nv_bfloat162 *)p);
        return P2{v.x, v.y};
    }
    __device__ static __forceinline__ void dst2(__nv_bfloat16 *p, P2 v) {
        *(__nv_bfloat162 *)p = __floats2bfloat162_rn(v.x, v.y);
    }
    __device__ static __forceinline__ uint32_t dbits(R v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
    __device__ static __forceinline__ R ld(const __nv_bfloat16 *p, R w) { return __bfloat162float(*p) + w; }
    __device__ static __forceinline__ void st(__nv_bfloat16 *p, R v, R w) { *p = __float2bfloat16_rn(v - w); }
    __device__ static __forceinline__ P2 ld2(const __nv_bfloat16 *p, R w) {
        const float2 v = __bfloat1622float2(*(const __nv_bfloat162 *)p);
        return P2{v.x, v.y} + P2{w, w};
    }
    __device__ static __forceinline__ void st2(__nv_bfloat16 *p, P2 v, R w) {
        const P2 t = v - P2{w, w};
        *(__nv_bfloat162 *)p = __floats2bfloat162_rn(t.x, t.y);
    }
};

// c16: a 16-bit float of this project for the shifted deviations g = f - w,
// with more significand and less range than binary16 (whose five exponent
// bits span magnitudes the deviations never reach): 1 sign bit, 3 exponent
// bits e, 12 fraction bits m;
//   e = 1..7: |g| = (1 + m / 2^12) 2^(e - 12)   (binades 2^-11 .. 2^-4),
//   e = 0:    |g| = m 2^-23                      (subnormal),
// so |g| < 2^-4 (|f_i - w_i| < 1/16, flows up to |u| ~ 0.28) with a 13-bit
// significand: 4x finer than binary16's 11 bits.  The format is float's
// bit layout with the exponent range moved down by 115 binades: scaling by
// 2^-115 maps the format's subnormal range onto float's subnormals, so
// float's own subnormal rounding and bit layout do most of the work.
// Encoding: |g| 2^-115 (one float rounding, which only values in the
// subnormal range undergo), then the fraction rounded to 12 bits, halves
// away from zero; magnitudes beyond the largest value (2 - 2^-12) 2^-5
// saturate to it.  Decoding is exact.  The CPU oracle states the same steps.
struct c16_t {
    uint16_t bits;
};
__host__ __device__ __forceinline__ uint32_t c16_encode(float v) {
    const float x = fabsf(v) * 0x1p-115f;
    uint32_t a, u;
    memcpy(&a, &x, 4);
    memcpy(&u, &v, 4);
    const uint32_t r = (a + 0x400u) >> 11;
    return ((u >> 16) & 0x8000u) | (r < 0x7fffu ? r : 0x7fffu);
}
// The code in the upper half of a 32-bit word (the lower half is ignored).
__host__ __device__ __forceinline__ float c16_decode_hi(uint32_t w) {
    const uint32_t u = (uint32_t)((int32_t)w >> 5) & 0x83fff800u;
    float x;
    memcpy(&x, &u, 4);
    return x * 0x1p115f;  // exact, subnormal x included
}
__host__ __device__ __forceinline__ float c16_decode(uint32_t c) { return c16_decode_hi(c << 16); }
template <> struct Store<c16_t> {
    using R = float;
    static constexpr bool kDev = true;
    __device__ static __forceinline__ R dld(const c16_t *p) { return c16_decode(p->bits); }
    __device__ static __forceinline__ void dst(c16_t *p, R v) { p->bits = (uint16_t)c16_encode(v); }
    __device__ static __forceinline__ P2 dld2(const c16_t *p) {
        const uint32_t w = *(const uint32_t *)p;
        return P2{c16_decode(w), c16_decode_hi(w)};
    }
    __device__ static __forceinline__ void dst2(c16_t *p, P2 v) {
        *(uint32_t *)p = c16_encode(v.x) | (c16_encode(v.y) << 16);
    }
    __device__ static __forceinline__ uint32_t dbits(R v) { return c16_encode(v); }
    __device__ static __forceinline__ R ld(const c16_t *p, R w) { return c16_decode(p->bits) + w; }
    __device__ static __forceinline__ void st(c16_t *p, R v, R w) { p->bits = (uint16_t)c16_encode(v - w); }
    __device__ static __forceinline__ P2 ld2(const c16_t *p, R w) { return dld2(p) + P2{w, w}; }
    __device__ static __forceinline__ void st2(c16_t *p, P2 v, R w) { dst2(p, v - P2{w, w}); }
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

// What the step kernels hold per population: f_i (float/double storage) or
// g_i = f_i - w_i (shifted 16-bit storage).
template <typename S> __device__ __forceinline__ typename Store<S>::R pop_ld(const S *p, int i) {
    using R = typename Store<S>::R;
    if constexpr (Store<S>::kDev) return Store<S>::dld(p);
    else return Store<S>::ld(p, weight<R>(i));
}
template <typename S> __device__ __forceinline__ void pop_st(S *p, typename Store<S>::R v, int i) {
    using R = typename Store<S>::R;
    if constexpr (Store<S>::kDev) Store<S>::dst(p, v);
    else Store<S>::st(p, v, weight<R>(i));
}
template <typename S> __device__ __forceinline__ P2 pop_ld2(const S *p, int i) {
    if constexpr (Store<S>::kDev) return Store<S>::dld2(p);
    else return Store<S>::ld2(p, weight<float>(i));
}
template <typename S> __device__ __forceinline__ void pop_st2(S *p, P2 v, int i) {
    if constexpr (Store<S>::kDev) Store<S>::dst2(p, v);
    else Store<S>::st2(p, v, weight<float>(i));
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
    int32_t nblocks;      // blocks of the launched kernel shape
    int32_t grav;         // gravity terms non-zero (alpha kernel)
    int32_t gmode;        // 0: the reference's chained terms, 1: per-term forcing
    int32_t parity;       // step counter parity at the start of a batch tick
    // Subdomains of a domain whose one-cell alpha steps also do the x part of
    // the exchange that follows them (CController::syncAlpha,
    // src/CController.hpp:265-320): after its own update, the thread of a
    // cell at x = nx-2 copies the planes in xmask_hi of that cell into the
    // ghost cell x = 0 of the +x neighbour (population planes xhi), a cell at
    // x = 1 the planes in xmask_lo into x = nx-1 of the -x neighbour (xlo).
    // Null: no such neighbour (or the exchange runs as its own launch).
    void *xhi, *xlo;
    uint32_t xmask_hi, xmask_lo;
    uint32_t xdiv_m, xdiv_s1, xdiv_s2;  // c / nx by multiply and shifts
    double pd[13];        // inv_tau, tau0, les_c, lid, k0..k8 (gravity chain)
    float pf[13];
};
enum { P_INV_TAU = 0, P_TAU0 = 1, P_LES = 2, P_LID = 3, P_K0 = 4, P_COUNT = 13 };

template <typename R> __device__ __forceinline__ R par(const LatDesc &d, int i);
template <> __device__ __forceinline__ float par<float>(const LatDesc &d, int i) { return d.pf[i]; }
template <> __device__ __forceinline__ double par<double>(const LatDesc &d, int i) { return d.pd[i]; }
template <typename M> __device__ __forceinline__ M parm(const LatDesc &d, int i) {
    return Bc<M>::of(par<typename Scalar<M>::T>(d, i));
}

// Arguments of a step launch: the descriptors of all lattices it covers
// travel in the kernel parameter space (the constant bank, so block-uniform
// fields are read in place or re-read instead of held in registers).
// Domains and single lattices launch up to kParamLattices per launch; the
// batched tick kernels take up to kBatchLattices (the 32 KB parameter
// space), larger ensembles launch once per chunk.  first_block and nblocks
// count blocks of the launched kernel shape from the start of the launch.
constexpr int kParamLattices = 8;
constexpr int kBatchLattices = 112;
template <int N> struct StepArgs {
    LatDesc tab[N];
    const int32_t *block_lattice;  // lattice of every block of the launch, or null
    int ntab;
    // Nonzero: the lattices have equal block counts and their blocks are
    // interleaved, block b running block b / ntab of lattice b % ntab, so
    // that the same rows of all subdomains are in flight together.
    int interleave;
    int store_v, store_rho;
    // Element offsets i pstride + e_i . (1, nx, nx ny) (mod 2^32) of the beta
    // scatter targets, when every lattice of the launch shares nx, ny and the
    // plane stride (the subdomains of a domain, a single lattice): set for
    // the staged beta's table addressing (kAddrTab), else unused.
    uint32_t koff[19];
};
using DomainArgs = StepArgs<kParamLattices>;
using BatchArgs = StepArgs<kBatchLattices>;
static_assert(sizeof(BatchArgs) + sizeof(int) <= 32764, "kernel parameters exceed 32 KB");

// Lattice of this block: one load from the block map, else a binary search
// on first_block.
template <int N>
__device__ __forceinline__ const LatDesc &lattice_of(const StepArgs<N> &a) {
    int li = 0;
    if (a.interleave) {
        li = (int)(blockIdx.x % (unsigned)a.ntab);
    } else if (a.block_lattice) {
        li = a.block_lattice[blockIdx.x];
    } else if (a.ntab > 1) {
        int hi = a.ntab - 1;
        while (li < hi) {
            const int mid = (li + hi + 1) >> 1;
            if (a.tab[mid].first_block <= (int)blockIdx.x) li = mid; else hi = mid - 1;
        }
    }
    return a.tab[li];
}

// Index of this block within its lattice (see StepArgs::interleave).
template <int N>
__device__ __forceinline__ int64_t block_in_lattice(const StepArgs<N> &a, const LatDesc &d) {
    return a.interleave ? (int64_t)(blockIdx.x / (unsigned)a.ntab) : (int64_t)blockIdx.x - d.first_block;
}

// ------------------------------------------------------------- equilibria
// src/cl_programs/lbm_header.h:68-94, for a scalar or a packed pair M.
template <typename M> __device__ __forceinline__ M eq_a0(M v, M v2, M r) {
    using R = typename Scalar<M>::T;
    return Bc<M>::of(K<R>::c18) * ((r + Bc<M>::of(K<R>::k3) * v) + Bc<M>::of(K<R>::k45) * v2);
}
template <typename M> __device__ __forceinline__ M eq_a1(M v, M v2, M r) {
    using R = typename Scalar<M>::T;
    return Bc<M>::of(K<R>::c18) * ((r + Bc<M>::of(K<R>::km3) * v) + Bc<M>::of(K<R>::k45) * v2);
}
template <typename M> __device__ __forceinline__ M eq_d4(M s, M s2, M r) {
    using R = typename Scalar<M>::T;
    return Bc<M>::of(K<R>::c36) * ((r + Bc<M>::of(K<R>::k3) * s) + Bc<M>::of(K<R>::k45) * s2);
}
template <typename M> __device__ __forceinline__ M eq_d5(M s, M s2, M r) {
    using R = typename Scalar<M>::T;
    return Bc<M>::of(K<R>::c36) * ((r + Bc<M>::of(K<R>::km3) * s) + Bc<M>::of(K<R>::k45) * s2);
}

template <typename M>
__device__ __forceinline__ void equilibria(M vx, M vy, M vz, M dp, M eq[19]) {
    using R = typename Scalar<M>::T;
    M v2, s;
    v2 = vx * vx; eq[0] = eq_a0(vx, v2, dp); eq[1] = eq_a1(vx, v2, dp);
    v2 = vy * vy; eq[2] = eq_a0(vy, v2, dp); eq[3] = eq_a1(vy, v2, dp);
    s = vx + vy; v2 = s * s; eq[4] = eq_d4(s, v2, dp); eq[5] = eq_d5(s, v2, dp);
    s = vx - vy; v2 = s * s; eq[6] = eq_d4(s, v2, dp); eq[7] = eq_d5(s, v2, dp);
    s = vx + vz; v2 = s * s; eq[8] = eq_d4(s, v2, dp); eq[9] = eq_d5(s, v2, dp);
    s = vx - vz; v2 = s * s; eq[10] = eq_d4(s, v2, dp); eq[11] = eq_d5(s, v2, dp);
    s = vy + vz; v2 = s * s; eq[12] = eq_d4(s, v2, dp); eq[13] = eq_d5(s, v2, dp);
    s = vy - vz; v2 = s * s; eq[14] = eq_d4(s, v2, dp); eq[15] = eq_d5(s, v2, dp);
    v2 = vz * vz; eq[16] = eq_a0(vz, v2, dp); eq[17] = eq_a1(vz, v2, dp);
    eq[18] = Bc<M>::of(K<R>::c3) * dp;
}

// BGK collision of a fluid cell; with LES the relaxation rate comes from the
// Smagorinsky model of Hou, Sterling, Chen & Doolen (1996):
//   tau_eff = (tau0 + sqrt(tau0^2 + C sqrt(Q))) / 2,  Q = Pi:Pi,  C = 18 sqrt(2) Cs^2,
//   Pi_ab = sum_i e_ia e_ib f_i - rho/3 delta_ab - u_a u_b
// (the second moment of the incompressible equilibrium is rho/3 delta + u u),
// from the nine opposite-pair sums of the pre-collision populations.  rho is
// the population sum, dp the equilibrium's dd_param.
template <typename M, bool LES>
__device__ __forceinline__ void collide(M f[19], M rho, M vx, M vy, M vz, M dp, const LatDesc &d) {
    using R = typename Scalar<M>::T;
    M w = parm<M>(d, P_INV_TAU);
    if (LES && par<R>(d, P_LES) != (R)0) {
        M p[9];
#pragma unroll
        for (int k = 0; k < 9; k++) p[k] = f[2 * k] + f[2 * k + 1];
        const M sxx = (((p[0] + p[2]) + p[3]) + p[4]) + p[5];
        const M syy = (((p[1] + p[2]) + p[3]) + p[6]) + p[7];
        const M szz = (((p[4] + p[5]) + p[6]) + p[7]) + p[8];
        const M r3 = rho * Bc<M>::of(K<R>::c3);
        const M pxx = (sxx - r3) - vx * vx;
        const M pyy = (syy - r3) - vy * vy;
        const M pzz = (szz - r3) - vz * vz;
        const M pxy = (p[2] - p[3]) - vx * vy;
        const M pxz = (p[4] - p[5]) - vx * vz;
        const M pyz = (p[6] - p[7]) - vy * vz;
        const M q = ((pxx * pxx + pyy * pyy) + pzz * pzz) + Bc<M>::of((R)2) * ((pxy * pxy + pxz * pxz) + pyz * pyz);
        const M tau0 = parm<M>(d, P_TAU0);
        const M te = Bc<M>::of((R)0.5) * (tau0 + msqrt(tau0 * tau0 + parm<M>(d, P_LES) * msqrt(q)));
        w = mrcp(te);
    }
    M eq[19];
    equilibria<M>(vx, vy, vz, dp, eq);
#pragma unroll
    for (int i = 0; i < 19; i++) f[i] += w * (eq[i] - f[i]);
}

// Gravity terms of the alpha kernel.  The reference aliases its temporary to
// rho (lbm_alpha.cl:173): term k is coefficient k times term k-1, and the
// stored density is the last term.  Coefficients k0..k8 come pre-multiplied
// from the host.  gmode 1 (off by default) computes what the reference
// intends instead: term k = coefficient k times the density.
template <typename M>
__device__ __forceinline__ M gravity_chain(M rho, const LatDesc &d, M t[9]) {
    if (d.gmode) {  // per-term forcing: coefficient k times the density, density stored as is
#pragma unroll
        for (int k = 0; k < 9; k++) t[k] = parm<M>(d, P_K0 + k) * rho;
        return rho;
    }
    M r = rho;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        r = parm<M>(d, P_K0 + k) * r;
        t[k] = r;
    }
    return r;
}

// Moments in the order of lbm_beta.cl:261-483 (the shared-memory path the
// reference hard-codes): rho and the momentum j = sum e_i f_i.
template <typename M>
__device__ __forceinline__ void moments_beta(const M f[19], M &r, M &vx, M &vy, M &vz) {
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
}

// Moments in the order of lbm_alpha.cl:61-156.
template <typename M>
__device__ __forceinline__ void moments_alpha(const M f[19], M &r, M &vx, M &vy, M &vz) {
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
}

// The beta kernel's flag switch (lbm_beta.cl:495-656) on moments already
// taken: fluid collision (rho becomes dd_param, lbm_beta.cl:493), obstacle
// bounce-back of the nine opposite pairs, lid equilibrium.  Other flags,
// the ghost layer included, stream unchanged.
template <typename M, bool LES>
__device__ __forceinline__ void beta_case(int fl, M f[19], M &r, M &vx, M &vy, M &vz, const LatDesc &d) {
    using R = typename Scalar<M>::T;
    if (fl == kFluid) {
        const M v2 = (vx * vx + vy * vy) + vz * vz;
        const M dp = r - Bc<M>::of(K<R>::k15) * v2;
        collide<M, LES>(f, r, vx, vy, vz, dp, d);
        r = dp;
    } else if (fl == kObstacle) {
        vx = Bc<M>::of(0); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const M t = f[2 * k + 1];
            f[2 * k + 1] = f[2 * k];
            f[2 * k] = t;
        }
    } else if (fl == kLid) {
        vx = parm<M>(d, P_LID); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
        r = Bc<M>::of((R)1.0f);
        const M v2 = (vx * vx + vy * vy) + vz * vz;
        r = r - Bc<M>::of(K<R>::k15) * v2;
        equilibria<M>(vx, vy, vz, r, f);
    }
}

// The alpha kernel's flag switch (lbm_alpha.cl:177-484): returns whether the
// cell writes its populations (fluid and lid, gravity terms applied).  The
// gravity terms (and the density they leave, lbm_alpha.cl:173) are computed
// only when there is gravity or the density is stored (need_rho).
template <typename M, bool LES>
__device__ __forceinline__ bool alpha_case(int fl, M f[19], M &r, M &vx, M &vy, M &vz, const LatDesc &d,
                                           bool need_rho) {
    using R = typename Scalar<M>::T;
    M t[9];
    if (fl == kFluid) {
        const M v2 = (vx * vx + vy * vy) + vz * vz;
        const M dp = r - Bc<M>::of(K<R>::k15) * v2;
        collide<M, LES>(f, r, vx, vy, vz, dp, d);
        if (d.grav || need_rho) r = gravity_chain<M>(r, d, t);
    } else if (fl == kLid) {
        vx = parm<M>(d, P_LID); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
        r = Bc<M>::of((R)1.0f);
        const M v2 = (vx * vx + vy * vy) + vz * vz;
        const M dp = r - Bc<M>::of(K<R>::k15) * v2;
        equilibria<M>(vx, vy, vz, dp, f);
        if (d.grav || need_rho) r = gravity_chain<M>(r, d, t);
    } else {
        if (fl == kObstacle) {  // lbm_alpha.cl:305-343, populations untouched
            vx = Bc<M>::of(0); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
        }
        return false;
    }
    if (d.grav) {
#pragma unroll
        for (int k = 0; k < 9; k++) {
            f[2 * k + 1] -= t[k];
            f[2 * k] += t[k];
        }
    }
    return true;
}

// ---------------------------------------------------------- deviation form
// The shifted 16-bit types hold g_i = f_i - w_i.  Their collision is the
// same incompressible BGK / Smagorinsky model as above, written on the
// deviations so that no population is shifted back and forth and the
// multiply-adds fuse (every fmaf below is one IEEE fused multiply-add; the
// oracle states the same operations in the same order):
//   rho - 1 = sum_i g_i + kCW,  j = sum_i e_i g_i  (sum_i e_i w_i = 0),
//   A = dd_param - 1 = (rho - 1) - 3/2 |u|^2  (u = j, as in the reference),
//   f_i^eq - w_i = w_i (A + 3 e_i.u + 9/2 (e_i.u)^2),
//   g_i' = (1 - omega) g_i + omega (f_i^eq - w_i),
// taken per opposite pair (2k, 2k+1) as P +- Q with P = omega w A +
// (9/2 omega w s) s, Q = 3 omega w s, s = e_2k . u, and Q folded into the
// last multiply-add of each population.  kCW and kCP are the float weights'
// exact offsets: sum_i w_i - 1 = 2^-26 and sum_i e_ix^2 w_i - (float)(1/3) = -2^-27.
constexpr float kCW = 0x1p-26f;
constexpr float kCP = -0x1p-27f;

// rho - 1, j and the second moments sum_i e_ia e_ib g_i (xx, yy, zz, xy, xz,
// yz) from the nine opposite-pair sums and differences.
template <typename M>
__device__ __forceinline__ void dev_moments(const M g[19], M &dl, M &jx, M &jy, M &jz, M m2[6]) {
    M s[9], t[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        s[k] = g[2 * k] + g[2 * k + 1];
        t[k] = g[2 * k] - g[2 * k + 1];
    }
    const M a23 = s[2] + s[3], a45 = s[4] + s[5], a67 = s[6] + s[7];
    dl = ((((s[0] + s[1]) + a23) + (a45 + a67)) + (s[8] + g[18])) + Bc<M>::of(kCW);
    jx = ((t[0] + t[2]) + (t[3] + t[4])) + t[5];
    jy = ((t[1] + t[2]) - t[3]) + (t[6] + t[7]);
    jz = ((t[4] - t[5]) + (t[6] - t[7])) + t[8];
    m2[0] = (s[0] + a23) + a45;
    m2[1] = (s[1] + a23) + a67;
    m2[2] = (s[8] + a45) + a67;
    m2[3] = s[2] - s[3];
    m2[4] = s[4] - s[5];
    m2[5] = s[6] - s[7];
}

// One opposite pair: g_2k' = (1-omega) g_2k + P + Q, g_2k+1' = ... + P - Q,
// P = aA + (a45 v) v, Q = b v (six operations).
template <typename M>
__device__ __forceinline__ void dev_pair(M g[19], int k, M v, M aA, M a45, M b, M om1) {
    const M P = mfma(a45 * v, v, aA);
    g[2 * k] = mfma(b, v, mfma(om1, g[2 * k], P));
    g[2 * k + 1] = mfma(-b, v, mfma(om1, g[2 * k + 1], P));
}

// Relaxation of all 19 deviations with rate om towards the equilibrium of
// (A, u).
template <typename M>
__device__ __forceinline__ void dev_relax(M g[19], M om, M A, M vx, M vy, M vz) {
    const M om1 = Bc<M>::of(1.0f) - om;
    const M a18 = om * Bc<M>::of(K<float>::c18), a36 = om * Bc<M>::of(K<float>::c36);
    const M a3 = om * Bc<M>::of(K<float>::c3);
    const M b18 = Bc<M>::of(K<float>::k3) * a18, b36 = Bc<M>::of(K<float>::k3) * a36;
    const M aA18 = a18 * A, aA36 = a36 * A;
    const M h18 = Bc<M>::of(K<float>::k45) * a18, h36 = Bc<M>::of(K<float>::k45) * a36;
    dev_pair(g, 0, vx, aA18, h18, b18, om1);
    dev_pair(g, 1, vy, aA18, h18, b18, om1);
    dev_pair(g, 2, vx + vy, aA36, h36, b36, om1);
    dev_pair(g, 3, vx - vy, aA36, h36, b36, om1);
    dev_pair(g, 4, vx + vz, aA36, h36, b36, om1);
    dev_pair(g, 5, vx - vz, aA36, h36, b36, om1);
    dev_pair(g, 6, vy + vz, aA36, h36, b36, om1);
    dev_pair(g, 7, vy - vz, aA36, h36, b36, om1);
    dev_pair(g, 8, vz, aA18, h18, b18, om1);
    g[18] = mfma(om1, g[18], a3 * A);
}

// Equilibrium deviations w_i (A + 3 e_i.u + 9/2 (e_i.u)^2) (lid cells).
template <typename M>
__device__ __forceinline__ void dev_equilibria(M vx, M vy, M vz, M A, M g[19]) {
    const M w18 = Bc<M>::of(K<float>::c18), w36 = Bc<M>::of(K<float>::c36);
    const M b18 = Bc<M>::of(K<float>::k3) * w18, b36 = Bc<M>::of(K<float>::k3) * w36;
    const M v[9] = {vx, vy, vx + vy, vx - vy, vx + vz, vx - vz, vy + vz, vy - vz, vz};
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const bool axis = k < 2 || k == 8;
        const M h = mfma(Bc<M>::of(K<float>::k45) * v[k], v[k], A);
        const M P = (axis ? w18 : w36) * h, Q = (axis ? b18 : b36) * v[k];
        g[2 * k] = P + Q;
        g[2 * k + 1] = P - Q;
    }
    g[18] = Bc<M>::of(K<float>::c3) * A;
}

// Fluid collision in deviation form; with LES the Hou et al. rate from
// Pi_ab = sum e_a e_b g + kCP delta_ab - (rho - 1)/3 delta_ab - u_a u_b,
// omega = 2 / (tau0 + sqrt(tau0^2 + C sqrt(Pi:Pi))).
template <typename M, bool LES>
__device__ __forceinline__ void dev_collide(M g[19], M dl, M vx, M vy, M vz, const M m2[6], M A,
                                            const LatDesc &d) {
    M om = parm<M>(d, P_INV_TAU);
    if (LES && par<float>(d, P_LES) != 0.0f) {
        const M mc3 = Bc<M>::of(-K<float>::c3), cp = Bc<M>::of(kCP);
        const M pxx = mfma(-vx, vx, mfma(mc3, dl, m2[0] + cp));
        const M pyy = mfma(-vy, vy, mfma(mc3, dl, m2[1] + cp));
        const M pzz = mfma(-vz, vz, mfma(mc3, dl, m2[2] + cp));
        const M pxy = mfma(-vx, vy, m2[3]);
        const M pxz = mfma(-vx, vz, m2[4]);
        const M pyz = mfma(-vy, vz, m2[5]);
        const M off = mfma(pyz, pyz, mfma(pxz, pxz, pxy * pxy));
        const M dia = mfma(pzz, pzz, mfma(pyy, pyy, pxx * pxx));
        const M q = mfma(Bc<M>::of(2.0f), off, dia);
        const M tau0 = parm<M>(d, P_TAU0);
        om = mdiv(Bc<M>::of(2.0f), tau0 + msqrt(mfma(parm<M>(d, P_LES), msqrt(q), tau0 * tau0)));
    }
    dev_relax(g, om, A, vx, vy, vz);
}

template <typename M>
__device__ __forceinline__ M dev_dp1(M vx, M vy, M vz, M dl) {
    const M u2 = mfma(vz, vz, mfma(vy, vy, vx * vx));
    return mfma(Bc<M>::of(-K<float>::k15), u2, dl);
}

// The beta kernel's flag switch (as beta_case) in deviation form.  r is the
// stored density: dd_param for fluid cells (lbm_beta.cl:493), the population
// sum otherwise.
template <typename M, bool LES>
__device__ __forceinline__ void dev_beta(int fl, M g[19], M &r, M &vx, M &vy, M &vz, const LatDesc &d) {
    M dl, m2[6];
    dev_moments<M>(g, dl, vx, vy, vz, m2);
    r = Bc<M>::of(1.0f) + dl;
    if (fl == kFluid) {
        const M A = dev_dp1(vx, vy, vz, dl);
        dev_collide<M, LES>(g, dl, vx, vy, vz, m2, A, d);
        r = Bc<M>::of(1.0f) + A;
    } else if (fl == kObstacle) {
        vx = Bc<M>::of(0); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const M t = g[2 * k + 1];
            g[2 * k + 1] = g[2 * k];
            g[2 * k] = t;
        }
    } else if (fl == kLid) {
        vx = parm<M>(d, P_LID); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
        const M A = Bc<M>::of(-K<float>::k15) * (vx * vx);
        dev_equilibria<M>(vx, vy, vz, A, g);
        r = Bc<M>::of(1.0f) + A;
    }
}

// The alpha kernel's flag switch (as alpha_case) in deviation form.
template <typename M, bool LES>
__device__ __forceinline__ bool dev_alpha(int fl, M g[19], M &r, M &vx, M &vy, M &vz, const LatDesc &d,
                                          bool need_rho) {
    M dl, m2[6], t[9];
    dev_moments<M>(g, dl, vx, vy, vz, m2);
    r = Bc<M>::of(1.0f) + dl;
    if (fl == kFluid) {
        const M A = dev_dp1(vx, vy, vz, dl);
        dev_collide<M, LES>(g, dl, vx, vy, vz, m2, A, d);
        if (d.grav || need_rho) r = gravity_chain<M>(r, d, t);
    } else if (fl == kLid) {
        vx = parm<M>(d, P_LID); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
        const M A = Bc<M>::of(-K<float>::k15) * (vx * vx);
        dev_equilibria<M>(vx, vy, vz, A, g);
        if (d.grav || need_rho) r = gravity_chain<M>(Bc<M>::of(1.0f), d, t);
    } else {
        if (fl == kObstacle) {
            vx = Bc<M>::of(0); vy = Bc<M>::of(0); vz = Bc<M>::of(0);
        }
        return false;
    }
    if (d.grav) {
#pragma unroll
        for (int k = 0; k < 9; k++) {
            g[2 * k + 1] -= t[k];
            g[2 * k] += t[k];
        }
    }
    return true;
}

// Moments plus flag switch for either form.
template <typename M, bool LES, bool DEV>
__device__ __forceinline__ void beta_phys(int fl, M f[19], M &r, M &vx, M &vy, M &vz, const LatDesc &d) {
    if constexpr (DEV) {
        dev_beta<M, LES>(fl, f, r, vx, vy, vz, d);
    } else {
        moments_beta<M>(f, r, vx, vy, vz);
        beta_case<M, LES>(fl, f, r, vx, vy, vz, d);
    }
}
template <typename M, bool LES, bool DEV>
__device__ __forceinline__ bool alpha_phys(int fl, M f[19], M &r, M &vx, M &vy, M &vz, const LatDesc &d,
                                           bool need_rho) {
    if constexpr (DEV) {
        return dev_alpha<M, LES>(fl, f, r, vx, vy, vz, d, need_rho);
    } else {
        moments_alpha<M>(f, r, vx, vy, vz);
        return alpha_case<M, LES>(fl, f, r, vx, vy, vz, d, need_rho);
    }
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

// Resident blocks of 256 threads per SM the launch bounds ask for.  The
// step kernels wait on the loads each warp keeps in flight (a warp loads,
// then computes for about twice the load latency with nothing in flight),
// so they take the most blocks that compile without spilling:
//   float populations: alpha 5 (48 registers, with or without the subgrid
//     model; 256^3 in 2x2x1 subdomains 447 -> 424 us, 512^3 3.32 -> 3.15 ms,
//     95 % of the measured copy bandwidth; without the subgrid model
//     478 -> 406 us), beta 4 (64; without the subgrid model it spilled at
//     80; with it, it spills at 48 and ran slower there, 415 -> 452 us, and
//     at 56 in blocks of 128, 9 per SM, 413 -> 425 us);
//   double arithmetic: alpha 3 (85 registers), the others 2 (128); at the
//     compiler's own choice, 122-140 registers, one block fit per SM;
//   otherwise 4 (64) with the subgrid model, 3 (80) without it.
// KIND: 0 any step, 1 alpha, 2 beta.
template <typename S, bool LES, int KIND = 0>
__host__ __device__ constexpr int min_blocks() {
    if (sizeof(typename Store<S>::R) == 8) return KIND == 1 ? 3 : 2;
    if (KIND == 1 && sizeof(S) == 4) return 5;
    if (KIND == 2 && sizeof(S) == 4) return 4;
    return LES ? 4 : 3;
}

// ---------------------------------------------------- one cell per thread
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
        f[i] = pop_ld<S>(p, i);
    }
    R r, vx, vy, vz;
    beta_phys<R, LES, Store<S>::kDev>(fl, f, r, vx, vy, vz, d);
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const int64_t off = dir_off(i, nx, sl);
        S *p = WRAP ? dd + i * ps + wrap_cell(c, off, n) : pc + (i * ps + off);
        pop_st<S>(p, f[i], i);
    }
    if (fl == kGhost) return;  // lbm_beta.cl:787-788
    if (store_v) {
        R *u = (R *)d.vel + c;
        u[0] = vx; u[n] = vy; u[2 * n] = vz;
    }
    if (store_rho) ((R *)d.rho)[c] = r;
}

template <typename S, bool LES>
__global__ void __launch_bounds__(256, (min_blocks<S, LES, 2>())) k_beta(const __grid_constant__ DomainArgs a) {
    const LatDesc &d = lattice_of(a);
    const int64_t c0 = block_in_lattice(a, d) * blockDim.x;
    const int64_t c = c0 + threadIdx.x;
    if (c >= d.n) return;
    const int64_t reach = (int64_t)d.nx + (int64_t)d.nx * d.ny;
    if (c0 < reach || c0 + (int64_t)blockDim.x - 1 + reach >= d.n)
        beta_cell<S, LES, true>(d, c, a.store_v, a.store_rho);
    else
        beta_cell<S, LES, false>(d, c, a.store_v, a.store_rho);
}

// Exact quotient of a 32-bit n by an invariant divisor from its multiplier
// and shifts (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, figure 4.1).
__device__ __forceinline__ uint32_t div_invariant(uint32_t n, uint32_t m, uint32_t s1, uint32_t s2) {
    const uint32_t t = __umulhi(m, n);
    return (t + ((n - t) >> s1)) >> s2;
}

// The x part of the exchange after an alpha step, done by the cells that
// send it (see LatDesc::xhi): which way(s) cell c sends, bit 0 towards +x
// (c at x = nx - 2), bit 1 towards -x (x = 1).  The receiving ghost cells
// are not touched by their own lattice's alpha step (lbm_alpha.cl:31-32),
// and the y and z parts run after the launch, so the corners still travel
// in two hops.
__device__ __forceinline__ int alpha_push_dirs(const LatDesc &d, int64_t c) {
    if (!d.xhi && !d.xlo) return 0;
    const uint32_t cc = (uint32_t)c, nx = (uint32_t)d.nx;
    const uint32_t x = cc - div_invariant(cc, d.xdiv_m, d.xdiv_s1, d.xdiv_s2) * nx;
    return (d.xhi && x == nx - 2 ? 1 : 0) | (d.xlo && x == 1 ? 2 : 0);
}

// Slot f of cell c after its alpha step is v(f); copy the selected slots to
// the neighbours' ghost cells (the same conversion as the cell's own stores,
// so the bits are those a copy of the slots would move).
template <typename S, typename V>
__device__ __forceinline__ void alpha_push(const LatDesc &d, int64_t c, int dirs, V v) {
    const int64_t ps = d.pstride, sh = (int64_t)d.nx - 2;
    if (dirs & 1) {
        S *dst = (S *)d.xhi + (c - sh);
#pragma unroll
        for (int f = 0; f < 19; f++)
            if (d.xmask_hi & (1u << f)) pop_st<S>(dst + f * ps, v(f), f);
    }
    if (dirs & 2) {
        S *dst = (S *)d.xlo + (c + sh);
#pragma unroll
        for (int f = 0; f < 19; f++)
            if (d.xmask_lo & (1u << f)) pop_st<S>(dst + f * ps, v(f), f);
    }
}

template <typename S, bool LES>
__device__ __forceinline__ void alpha_cell(const LatDesc &d, int64_t c, int store_v, int store_rho) {
    using R = typename Store<S>::R;
    const int fl = d.flags[c];
    const int dirs = alpha_push_dirs(d, c);
    S *const pc = (S *)d.dd + c;
    const int64_t ps = d.pstride;
    if (fl == kGhost) {  // lbm_alpha.cl:31-32; a sending ghost cell forwards its slots as they are
        if (dirs) alpha_push<S>(d, c, dirs, [&](int f) { return pop_ld<S>(pc + f * ps, f); });
        return;
    }
    R f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) f[i] = pop_ld<S>(pc + i * ps, i);
    R r, vx, vy, vz;
    if (alpha_phys<R, LES, Store<S>::kDev>(fl, f, r, vx, vy, vz, d, store_rho != 0)) {
        // each population goes to the opposite slot (lbm_alpha.cl:185-301)
#pragma unroll
        for (int i = 0; i < 19; i++) pop_st<S>(pc + opp(i) * ps, f[i], opp(i));
        if (dirs) alpha_push<S>(d, c, dirs, [&](int s) { return f[opp(s)]; });
    } else if (dirs) {  // populations untouched
        alpha_push<S>(d, c, dirs, [&](int s) { return f[s]; });
    }
    if (store_v) {
        R *u = (R *)d.vel + c;
        u[0] = vx; u[d.n] = vy; u[2 * d.n] = vz;
    }
    if (store_rho) ((R *)d.rho)[c] = r;
}

template <typename S, bool LES>
__global__ void __launch_bounds__(256, (min_blocks<S, LES, 1>())) k_alpha(const __grid_constant__ DomainArgs a) {
    const LatDesc &d = lattice_of(a);
    const int64_t c = block_in_lattice(a, d) * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    alpha_cell<S, LES>(d, c, a.store_v, a.store_rho);
}

// ---------------------------------------------------- two cells per thread
// Thread t of a block owns cells c, c+1 (c even, same x row because nx is
// even).  Populations along y/z are one aligned 64-bit access per pair.
// Populations that move along x are one cell off the pair alignment: the
// missing element comes from the neighbouring lane by a shuffle, and lanes
// 0 / 31 complete the warp's edge with one scalar access.
constexpr int kPairCells = 512;  // cells per block of 256 threads
constexpr unsigned kFull = 0xffffffffu;

// u and rho of a pair; ghost cells store nothing (lbm_beta.cl:787-788).
__device__ __forceinline__ void store_pair_moments(const LatDesc &d, int64_t c, int fl0, int fl1, P2 r, P2 vx,
                                                   P2 vy, P2 vz, int store_v, int store_rho) {
    if (!(store_v | store_rho)) return;
    const int64_t n = d.n;
    float *u = (float *)d.vel + c, *rh = (float *)d.rho + c;
    if (fl0 != kGhost && fl1 != kGhost) {
        if (store_v) {
            *(float2 *)u = make_float2(vx.x, vx.y);
            *(float2 *)(u + n) = make_float2(vy.x, vy.y);
            *(float2 *)(u + 2 * n) = make_float2(vz.x, vz.y);
        }
        if (store_rho) *(float2 *)rh = make_float2(r.x, r.y);
        return;
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if ((h ? fl1 : fl0) == kGhost) continue;
        if (store_v) {
            u[h] = h ? vx.y : vx.x;
            u[n + h] = h ? vy.y : vy.x;
            u[2 * n + h] = h ? vz.y : vz.x;
        }
        if (store_rho) rh[h] = h ? r.y : r.x;
    }
}

template <typename S, bool LES>
__device__ __forceinline__ void beta_pair(const LatDesc &d, int64_t c, int lane, int store_v, int store_rho) {
    using R = float;
    S *const dd = (S *)d.dd;
    const int64_t ps = d.pstride, nx = d.nx, sl = (int64_t)d.nx * d.ny;
    const uint16_t fl2 = *(const uint16_t *)(d.flags + c);
    const int fl0 = fl2 & 0xff, fl1 = fl2 >> 8;

    P2 f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const int ex = dir_x(i);
        // aligned pair (c, c+1) of the source row: c - e_i without its x part
        const S *p = dd + opp(i) * ps + c - ((int64_t)dir_y(i) * nx + (int64_t)dir_z(i) * sl);
        const P2 q = pop_ld2<S>(p, i);
        if (ex == 0) {
            f[i] = q;
        } else if (ex > 0) {  // sources (c-1, c)
            float lo = __shfl_up_sync(kFull, q.y, 1);
            if (lane == 0) lo = pop_ld<S>(p - 1, i);
            f[i] = P2{lo, q.x};
        } else {  // sources (c+1, c+2)
            float hi = __shfl_down_sync(kFull, q.x, 1);
            if (lane == 31) hi = pop_ld<S>(p + 2, i);
            f[i] = P2{q.y, hi};
        }
    }
    constexpr bool DEV = Store<S>::kDev;
    P2 r, vx, vy, vz;
    if (fl0 == kFluid && fl1 == kFluid) {
        beta_phys<P2, LES, DEV>(kFluid, f, r, vx, vy, vz, d);
    } else {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            R g[19], rr, ux, uy, uz;
#pragma unroll
            for (int i = 0; i < 19; i++) g[i] = h ? f[i].y : f[i].x;
            beta_phys<R, LES, DEV>(h ? fl1 : fl0, g, rr, ux, uy, uz, d);
#pragma unroll
            for (int i = 0; i < 19; i++) (h ? f[i].y : f[i].x) = g[i];
            (h ? r.y : r.x) = rr; (h ? vx.y : vx.x) = ux; (h ? vy.y : vy.x) = uy; (h ? vz.y : vz.x) = uz;
        }
    }
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const int ex = dir_x(i);
        S *p = dd + i * ps + c + ((int64_t)dir_y(i) * nx + (int64_t)dir_z(i) * sl);
        if (ex == 0) {
            pop_st2<S>(p, f[i], i);
        } else if (ex > 0) {  // destinations (c+1, c+2)
            const float lo = __shfl_up_sync(kFull, f[i].y, 1);
            if (lane != 0) pop_st2<S>(p, P2{lo, f[i].x}, i);
            else pop_st<S>(p + 1, f[i].x, i);
            if (lane == 31) pop_st<S>(p + 2, f[i].y, i);
        } else {  // destinations (c-1, c)
            const float hi = __shfl_down_sync(kFull, f[i].x, 1);
            if (lane != 31) pop_st2<S>(p, P2{f[i].y, hi}, i);
            else pop_st<S>(p, f[i].y, i);
            if (lane == 0) pop_st<S>(p - 1, f[i].x, i);
        }
    }
    store_pair_moments(d, c, fl0, fl1, r, vx, vy, vz, store_v, store_rho);
}

template <typename S, bool LES>
__global__ void __launch_bounds__(256, 2) k_beta2(const __grid_constant__ DomainArgs a) {
    const LatDesc &d = lattice_of(a);
    const int64_t c0 = (int64_t)(blockIdx.x - d.first_block) * kPairCells;
    const int64_t reach = (int64_t)d.nx + (int64_t)d.nx * d.ny + 2;
    if (c0 < reach || c0 + kPairCells + reach >= d.n) {
        // near either end of the buffer: one cell at a time with the wrap
        for (int h = 0; h < 2; h++) {
            const int64_t c = c0 + 2 * threadIdx.x + h;
            if (c < d.n) beta_cell<S, LES, true>(d, c, a.store_v, a.store_rho);
        }
        return;
    }
    beta_pair<S, LES>(d, c0 + 2 * threadIdx.x, threadIdx.x & 31, a.store_v, a.store_rho);
}

template <typename S, bool LES>
__device__ __forceinline__ void alpha_pair(const LatDesc &d, int64_t c, int store_v, int store_rho) {
    using R = float;
    S *const pc = (S *)d.dd + c;
    const int64_t ps = d.pstride;
    const uint16_t fl2 = *(const uint16_t *)(d.flags + c);
    const int fl0 = fl2 & 0xff, fl1 = fl2 >> 8;
    if (fl0 == kGhost && fl1 == kGhost) return;  // lbm_alpha.cl:31-32
    P2 f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) f[i] = pop_ld2<S>(pc + i * ps, i);
    constexpr bool DEV = Store<S>::kDev;
    P2 r, vx, vy, vz;
    if (fl0 == kFluid && fl1 == kFluid) {
        alpha_phys<P2, LES, DEV>(kFluid, f, r, vx, vy, vz, d, store_rho != 0);
#pragma unroll
        for (int i = 0; i < 19; i++) pop_st2<S>(pc + opp(i) * ps, f[i], opp(i));
    } else {
        r = vx = vy = vz = P2{0.0f, 0.0f};
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int fl = h ? fl1 : fl0;
            if (fl == kGhost) continue;
            R g[19], rr, ux, uy, uz;
#pragma unroll
            for (int i = 0; i < 19; i++) g[i] = h ? f[i].y : f[i].x;
            if (alpha_phys<R, LES, DEV>(fl, g, rr, ux, uy, uz, d, store_rho != 0)) {
#pragma unroll
                for (int i = 0; i < 19; i++) pop_st<S>(pc + opp(i) * ps + h, g[i], opp(i));
            }
            (h ? r.y : r.x) = rr; (h ? vx.y : vx.x) = ux; (h ? vy.y : vy.x) = uy; (h ? vz.y : vz.x) = uz;
        }
    }
    store_pair_moments(d, c, fl0, fl1, r, vx, vy, vz, store_v, store_rho);
}

template <typename S, bool LES>
__global__ void __launch_bounds__(256, 2) k_alpha2(const __grid_constant__ DomainArgs a) {
    const LatDesc &d = lattice_of(a);
    const int64_t c = (int64_t)(blockIdx.x - d.first_block) * kPairCells + 2 * threadIdx.x;
    if (c + 1 < d.n) alpha_pair<S, LES>(d, c, a.store_v, a.store_rho);
    else if (c < d.n) alpha_cell<S, LES>(d, c, a.store_v, a.store_rho);
}

// ------------------------------------------------ tiles staged by TMA
// The staged kernels move tiles of T consecutive cells between HBM and
// shared memory with the Tensor Memory Accelerator's bulk copies
// (cp.async.bulk).  A persistent block has one producer warp and eight
// compute warps around a ring of kStages tile buffers: the producer keeps
// the next tiles' 19 plane segments (+ flag bytes) in flight while the
// compute warps work on the current one from shared memory ("full" /
// "empty" mbarriers per buffer, no block-wide barrier in the loop).  This
// decouples the bytes in flight from the registers of the collision (the
// one-cell kernels are latency-bound at 64 registers a thread) and removes
// the per-population 64-bit address arithmetic of the loads.
//   alpha: segment i is plane i of the tile itself; the updated populations
//          go back into the segments (slot opp(i)) and the producer writes
//          the tile back with bulk stores.
//   beta:  segment i holds the tile's sources of f_i, plane opp(i) at
//          c - e_i, from the 16-byte boundary below (T + A elements; nx is
//          a multiple of A, so the offset into the segment is fixed per
//          direction); the results scatter to c + e_i with ordinary
//          stores.  Tiles within reach of either end of the buffer (their
//          sources wrap) and a partial last tile take the one-cell path
//          with the wrap instead.
// Every wait on a barrier is bounded; a wait that runs out records
// kStageTimeout in g_stage_error and the warp stops: a compute warp leaves
// its loop (it issues no asynchronous copies of its own), the producer stops
// issuing tiles, then waits -- bounded again -- until the loads it issued
// have landed and its bulk stores are done, and only then returns, so no
// copy into the block's shared memory outlives the block.
constexpr int kStages = 3;
constexpr int kStageBlocksPerSM = 3;
constexpr int kConsumerWarps = 8;
constexpr int kStageThreads = 32 * (kConsumerWarps + 1);
constexpr unsigned kStageTimeout = 1u;
constexpr uint32_t kStageWaitLimit = 1u << 22;
// Header of the dynamic shared memory: full/empty barriers from byte 0, the
// tiles' descriptor indices from byte 64, the ring from byte 128.
static_assert(2 * kStages * 8 <= 64 && 64 + 4 * kStages <= 128, "the ring header holds the barriers and indices");

__device__ unsigned int g_stage_error;

template <typename S> struct Tile {
    static_assert(sizeof(S) <= 4, "staged tiles hold float or 16-bit populations");
    static constexpr int T = 1024 / (int)sizeof(S);  // cells per tile: 1 KB per plane
    static constexpr int A = 16 / (int)sizeof(S);    // elements per 16-byte boundary
    static constexpr int PER = (T + 32 * kConsumerWarps - 1) / (32 * kConsumerWarps);  // cells per compute thread
    static constexpr int SEG = (T + A) * (int)sizeof(S);   // bytes per plane segment
    static constexpr int STAGE = 19 * SEG + T;       // 19 segments + flag bytes
    static constexpr int SMEM = 128 + kStages * STAGE;  // barriers + the ring
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = kStageWaitLimit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Descriptor index of the lattice of tile t (first_block / nblocks count
// tiles here).  ONE: the launch covers a single lattice, whose descriptor
// fields are then read at fixed parameter offsets (measured 4 % faster than
// the indexed reads).  The producer searches once per tile and leaves the
// index beside the ring buffer for the compute warps.
template <bool ONE, int N>
__device__ __forceinline__ int lattice_index(const StepArgs<N> &a, int t) {
    if (ONE) return 0;
    int li = 0, hi = a.ntab - 1;
    while (li < hi) {
        const int mid = (li + hi + 1) >> 1;
        if (a.tab[mid].first_block <= t) li = mid; else hi = mid - 1;
    }
    return li;
}

// A beta tile whose shifted segments lie inside the lattice: every source
// range [c0 - off_i - (A - 1), c0 - off_i + T + A) within [0, n).
template <typename S>
__device__ __forceinline__ bool beta_tile_inside(const LatDesc &d, int64_t c0) {
    using TL = Tile<S>;
    const int64_t reach = (int64_t)d.nx + (int64_t)d.nx * d.ny + 1;
    return c0 >= reach + TL::A && c0 + TL::T + TL::A + reach <= d.n;
}

// Issue the bulk loads of tile t into a ring buffer: lane i < 19 copies
// plane segment i, lane 19 the flag bytes (the producer warp spreads the
// address arithmetic over its lanes).  A beta tile that is not inside gets
// no copies: its phase completes at once and the compute warps read it from
// global memory.
template <typename S, bool BETA, bool ONE, int N>
__device__ __forceinline__ void stage_tile(const StepArgs<N> &a, int t, unsigned char *stage, uint64_t *bar,
                                           int *lat_slot, int lane) {
    using TL = Tile<S>;
    const int li = lattice_index<ONE>(a, t);
    const LatDesc &d = a.tab[li];
    const int64_t c0 = (int64_t)(t - d.first_block) * TL::T;
    const bool inside = !BETA || beta_tile_inside<S>(d, c0);
    const int cells = (int)min((int64_t)TL::T, d.n - c0);
    const uint32_t pb = BETA ? (uint32_t)TL::SEG : (uint32_t)((cells * (int)sizeof(S) + 15) & ~15);
    const uint32_t fb = BETA ? (uint32_t)TL::T : (uint32_t)((cells + 15) & ~15);
    if (lane == 0) {
        *lat_slot = li;  // ordered before the arrival (release) that completes with the copies
        mbar_expect_tx(bar, inside ? 19 * pb + fb : 0);
    }
    __syncwarp();
    if (!inside) return;
    if (lane < 19) {
        int64_t start = c0;
        if (BETA) {
            const int64_t off = (int64_t)dir_x(lane) + (int64_t)dir_y(lane) * d.nx + (int64_t)dir_z(lane) * d.nx * d.ny;
            start = (c0 - off) & ~(int64_t)(TL::A - 1);
        }
        const int plane = BETA ? opp(lane) : lane;
        bulk_load(stage + lane * TL::SEG, (const S *)d.dd + plane * d.pstride + start, pb, bar);
    } else if (lane == 19) {
        bulk_load(stage + 19 * TL::SEG, d.flags + c0, fb, bar);
    }
}

// Write an alpha tile back from its ring buffer, lane i < 19 plane i, and
// wait until the buffer has been read out.
template <typename S, bool ONE, int N>
__device__ __forceinline__ void unstage_tile(const StepArgs<N> &a, int t, int li, const unsigned char *stage,
                                             int lane) {
    using TL = Tile<S>;
    if (lane < 19) {
        const LatDesc &d = a.tab[ONE ? 0 : li];
        const int64_t c0 = (int64_t)(t - d.first_block) * TL::T;
        const int cells = (int)min((int64_t)TL::T, d.n - c0);
        const uint32_t pb = (uint32_t)((cells * (int)sizeof(S) + 15) & ~15);
        bulk_store((S *)d.dd + lane * d.pstride + c0, stage + lane * TL::SEG, pb);
        bulk_commit();
        bulk_wait_read_all();
    }
    __syncwarp();
}

// Scatter target of population i of cell c: c + e_i in plane i.  When the
// lattice's 19 planes span fewer than 2^32 elements (19 pstride < 2^32) the
// element offset from the buffer start is formed in 32-bit unsigned
// arithmetic and widened once by the address computation: from the
// launch's offset table (kAddrTab, lattices of equal shape) or computed
// (kAddr32); otherwise in 64 bits (kAddr64).
enum : int { kAddr64 = 0, kAddr32 = 1, kAddrTab = 2 };
template <typename S, int ADDR>
__device__ __forceinline__ S *scatter_ptr(const LatDesc &d, int64_t c, int i, const uint32_t *koff) {
    if constexpr (ADDR == kAddrTab) {
        return (S *)d.dd + ((uint32_t)c + koff[i]);
    } else if constexpr (ADDR == kAddr32) {
        const uint32_t nx = (uint32_t)d.nx, sl = (uint32_t)d.nx * (uint32_t)d.ny;
        const uint32_t o = (uint32_t)c + (uint32_t)i * (uint32_t)d.pstride + (uint32_t)dir_x(i) +
                           (uint32_t)dir_y(i) * nx + (uint32_t)dir_z(i) * sl;
        return (S *)d.dd + o;
    } else {
        return (S *)d.dd + (c + (i * d.pstride + dir_off(i, (int64_t)d.nx, (int64_t)d.nx * d.ny)));
    }
}

// One beta cell of an inside tile: sources from the ring buffer (the
// offset (-e_i . (1, nx, nx ny)) mod A is -e_ix mod A because A divides
// nx), results scattered to the neighbours.
template <typename S, bool LES, int ADDR>
__device__ __forceinline__ void beta_staged_cell(const LatDesc &d, const unsigned char *stage, int l, int64_t c,
                                                 int store_v, int store_rho, const uint32_t *koff) {
    using TL = Tile<S>;
    using R = typename Store<S>::R;
    const int fl = stage[19 * TL::SEG + l];
    R f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const int rem = (-dir_x(i)) & (TL::A - 1);
        f[i] = pop_ld<S>((const S *)(stage + i * TL::SEG) + (l + rem), i);
    }
    R r, vx, vy, vz;
    beta_phys<R, LES, Store<S>::kDev>(fl, f, r, vx, vy, vz, d);
#pragma unroll
    for (int i = 0; i < 19; i++) pop_st<S>(scatter_ptr<S, ADDR>(d, c, i, koff), f[i], i);
    if (fl == kGhost) return;  // lbm_beta.cl:787-788
    if (store_v) {
        R *u = (R *)d.vel + c;
        u[0] = vx; u[d.n] = vy; u[2 * d.n] = vz;
    }
    if (store_rho) ((R *)d.rho)[c] = r;
}

// Two neighbouring cells l, l + 1 (l and c even) of an inside beta tile in
// 16-bit storage.  The ten populations with an x component scatter one by
// one; the nine without one land at the same in-row offset for both cells,
// a 4-byte aligned pair (c, nx and the plane stride are even), and go out
// as one 32-bit store after the second cell, the first cell's halves held
// two to a register meanwhile.  Used with the subgrid model (measured at
// 512^3: f16 70.1k -> 73.6k MLUPS); without it the held halves push the
// register-capped kernel into spills and the one-cell loop stays faster.
template <typename S, bool LES, int ADDR>
__device__ __forceinline__ void beta_staged_pair(const LatDesc &d, const unsigned char *stage, int l, int64_t c,
                                                 int store_v, int store_rho, const uint32_t *koff) {
    using TL = Tile<S>;
    using R = typename Store<S>::R;
    static_assert(Store<S>::kDev, "pairs of 16-bit populations");
    uint32_t keep[5];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int fl = stage[19 * TL::SEG + l + h];
        R f[19];
#pragma unroll
        for (int i = 0; i < 19; i++) {
            const int rem = (-dir_x(i)) & (TL::A - 1);
            f[i] = pop_ld<S>((const S *)(stage + i * TL::SEG) + (l + h + rem), i);
        }
        R r, vx, vy, vz;
        beta_phys<R, LES, true>(fl, f, r, vx, vy, vz, d);
        int k = 0;
#pragma unroll
        for (int i = 0; i < 19; i++) {
            if (dir_x(i) != 0) {
                pop_st<S>(scatter_ptr<S, ADDR>(d, c + h, i, koff), f[i], i);
                continue;
            }
            const uint32_t bits = Store<S>::dbits(f[i]);
            if (h == 0) {
                keep[k >> 1] = (k & 1) ? (keep[k >> 1] | (bits << 16)) : bits;
            } else {
                const uint32_t first = (k & 1) ? (keep[k >> 1] >> 16) : (keep[k >> 1] & 0xffffu);
                *(uint32_t *)scatter_ptr<S, ADDR>(d, c, i, koff) = first | (bits << 16);
            }
            k++;
        }
        if (fl == kGhost) continue;  // lbm_beta.cl:787-788
        if (store_v) {
            R *u = (R *)d.vel + c + h;
            u[0] = vx; u[d.n] = vy; u[2 * d.n] = vz;
        }
        if (store_rho) ((R *)d.rho)[c + h] = r;
    }
}

template <typename S, bool LES>
__device__ __forceinline__ void alpha_staged_cell(const LatDesc &d, unsigned char *stage, int l, int64_t c,
                                                  int store_v, int store_rho) {
    using TL = Tile<S>;
    using R = typename Store<S>::R;
    const int fl = stage[19 * TL::SEG + l];
    if (fl == kGhost) return;  // lbm_alpha.cl:31-32
    R f[19];
#pragma unroll
    for (int i = 0; i < 19; i++) f[i] = pop_ld<S>((const S *)(stage + i * TL::SEG) + l, i);
    R r, vx, vy, vz;
    if (alpha_phys<R, LES, Store<S>::kDev>(fl, f, r, vx, vy, vz, d, store_rho != 0)) {
#pragma unroll
        for (int i = 0; i < 19; i++) pop_st<S>((S *)(stage + opp(i) * TL::SEG) + l, f[i], opp(i));
    }
    if (store_v) {
        R *u = (R *)d.vel + c;
        u[0] = vx; u[d.n] = vy; u[2 * d.n] = vz;
    }
    if (store_rho) ((R *)d.rho)[c] = r;
}

// N: descriptors in the parameter space (kParamLattices for domains and
// single lattices; kBatchLattices for the alpha steps of an ensemble chunk
// whose members are all at an alpha step).
// ADDR: how the beta step forms its scatter addresses (scatter_ptr).
template <typename S, bool LES, bool BETA, bool ONE, int N = kParamLattices, int ADDR = kAddr64>
__global__ void __launch_bounds__(kStageThreads, kStageBlocksPerSM) k_step_staged(const __grid_constant__ StepArgs<N> a,
                                                                                  int tiles) {
    using TL = Tile<S>;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *full = (uint64_t *)smem, *empty = full + kStages;
    int *tile_lat = (int *)(smem + 64);  // descriptor index of the tile in each buffer
    unsigned char *buf = smem + 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        fence_barrier_init();
    }
    __syncthreads();
    const int stride = gridDim.x;
    const int mine = (int)blockIdx.x < tiles ? (tiles - 1 - (int)blockIdx.x) / stride + 1 : 0;

    if (warp == kConsumerWarps) {  // producer warp
        bool ok = true;
        int staged = 0;  // tiles whose loads this warp has issued (ring slot k % kStages for tile k)
        const int rounds = mine + (BETA ? 0 : kStages);
        for (int k = 0; k < rounds; ++k) {
            const int s = k % kStages;
            unsigned char *stage = buf + s * TL::STAGE;
            if (k >= kStages) {
                // the compute warps are done with the tile k - kStages in this buffer
                ok = __all_sync(0xffffffffu, mbar_wait(&empty[s], (uint32_t)((k / kStages - 1) & 1)));
                if (!ok) break;
                if (!BETA) unstage_tile<S, ONE, N>(a, blockIdx.x + (k - kStages) * stride, tile_lat[s], stage, lane);
            }
            if (k < mine) {
                stage_tile<S, BETA, ONE, N>(a, blockIdx.x + k * stride, stage, &full[s], &tile_lat[s], lane);
                staged = k + 1;
            }
        }
        // Leave only after every load this warp issued has landed: the block's
        // shared memory must outlive the copies into it, and the compute warps
        // may already have left (normally they consume the last tiles, but one
        // that ran out of time on a "full" barrier does not).  Each buffer has at
        // most one armed phase that nobody may have waited for: the one of the
        // last tile staged into it.  These waits are bounded as well.
        bool drained = true;
        for (int s = 0; s < kStages && s < staged; s++) {
            const int k_last = s + kStages * ((staged - 1 - s) / kStages);
            drained &= mbar_wait(&full[s], (uint32_t)((k_last / kStages) & 1));
        }
        if ((!ok || !drained) && lane == 0) atomicOr(&g_stage_error, kStageTimeout);
        bulk_wait_all();
        return;
    }

    for (int k = 0; k < mine; ++k) {  // compute warps
        const int s = k % kStages;
        unsigned char *stage = buf + s * TL::STAGE;
        if (!mbar_wait(&full[s], (uint32_t)((k / kStages) & 1))) {
            if (lane == 0) atomicOr(&g_stage_error, kStageTimeout);
            break;
        }
        const int t = blockIdx.x + k * stride;
        const LatDesc &d = a.tab[ONE ? 0 : tile_lat[s]];
        const int64_t c0 = (int64_t)(t - d.first_block) * TL::T;
        if (BETA && !beta_tile_inside<S>(d, c0)) {
#pragma unroll 1
            for (int m = 0; m < TL::PER; m++) {
                const int l = threadIdx.x + 32 * kConsumerWarps * m;
                const int64_t c = c0 + l;
                if (l < TL::T && c < d.n) beta_cell<S, LES, true>(d, c, a.store_v, a.store_rho);
            }
        } else if constexpr (BETA && LES && Store<S>::kDev) {
#pragma unroll 1
            for (int l = 2 * threadIdx.x; l < TL::T; l += 64 * kConsumerWarps)
                beta_staged_pair<S, LES, ADDR>(d, stage, l, c0 + l, a.store_v, a.store_rho, a.koff);
        } else {
#pragma unroll 1
            for (int m = 0; m < TL::PER; m++) {
                const int l = threadIdx.x + 32 * kConsumerWarps * m;
                const int64_t c = c0 + l;
                if (l >= TL::T || c >= d.n) break;
                if (BETA) beta_staged_cell<S, LES, ADDR>(d, stage, l, c, a.store_v, a.store_rho, a.koff);
                else alpha_staged_cell<S, LES>(d, stage, l, c, a.store_v, a.store_rho);
            }
        }
        if (!BETA) fence_async_smem();  // the bulk stores read what this warp wrote
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

// ------------------------------------------------ batches of lattices
// Every lattice of a batch keeps its own step counter: step j of a tick is
// a beta step for a lattice whose counter was even at the tick start and j
// even (and so on), chosen per block.  Used for ensembles of cavities and
// for the serving loop, where solves start at different times.
// UNI: 0 each lattice at its own kind of step; 1 every lattice at an alpha
// step, 2 at a beta step (the other kind's code compiled out, and the launch
// bounds of that kind: min_blocks).
template <typename S, bool LES, int UNI = 0>
__global__ void __launch_bounds__(256, (min_blocks<S, LES, UNI>())) k_step(const __grid_constant__ BatchArgs a, int j) {
    const LatDesc &d = lattice_of(a);
    const int64_t c0 = (int64_t)(blockIdx.x - d.first_block) * blockDim.x;
    const int64_t c = c0 + threadIdx.x;
    if (c >= d.n) return;
    if (UNI == 1 || (UNI == 0 && ((d.parity + j) & 1))) {
        alpha_cell<S, LES>(d, c, a.store_v, a.store_rho);
        return;
    }
    const int64_t reach = (int64_t)d.nx + (int64_t)d.nx * d.ny;
    if (c0 < reach || c0 + (int64_t)blockDim.x - 1 + reach >= d.n)
        beta_cell<S, LES, true>(d, c, a.store_v, a.store_rho);
    else
        beta_cell<S, LES, false>(d, c, a.store_v, a.store_rho);
}

template <typename S, bool LES>
__global__ void __launch_bounds__(256, 2) k_step2(const __grid_constant__ BatchArgs a, int j) {
    const LatDesc &d = lattice_of(a);
    const int64_t c0 = (int64_t)(blockIdx.x - d.first_block) * kPairCells;
    if ((d.parity + j) & 1) {
        const int64_t c = c0 + 2 * threadIdx.x;
        if (c + 1 < d.n) alpha_pair<S, LES>(d, c, a.store_v, a.store_rho);
        else if (c < d.n) alpha_cell<S, LES>(d, c, a.store_v, a.store_rho);
        return;
    }
    const int64_t reach = (int64_t)d.nx + (int64_t)d.nx * d.ny + 2;
    if (c0 < reach || c0 + kPairCells + reach >= d.n) {
        for (int h = 0; h < 2; h++) {
            const int64_t c = c0 + 2 * threadIdx.x + h;
            if (c < d.n) beta_cell<S, LES, true>(d, c, a.store_v, a.store_rho);
        }
        return;
    }
    beta_pair<S, LES>(d, c0 + 2 * threadIdx.x, threadIdx.x & 31, a.store_v, a.store_rho);
}

}  // namespace lbm
