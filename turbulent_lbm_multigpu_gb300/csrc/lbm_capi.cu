// lbm_capi.cu -- the C ABI of include/lbm_gb300.h over the sm_103a kernels.
//
// Host-side runtime: lattice handles own their device fields (like the
// reference's CLbmSolver owns its CL buffers), parameters are rounded to the
// arithmetic type once, and domains hold all subdomains of a decomposition on
// one GPU with device-local halo copies and a captured CUDA graph per pair
// of steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lbm_internal.h"

using namespace lbm;
using namespace lbm_rt;

namespace lbm_rt {
thread_local std::string g_err;

int fail(const std::string &m) {
    g_err = m;
    return -1;
}
}  // namespace lbm_rt

namespace lbm_rt {
bool valid_box(const lbm_lattice *l, const int o[3], const int s[3]) {
    const int d[3] = {l->nx, l->ny, l->nz};
    for (int a = 0; a < 3; a++)
        if (o[a] < 0 || s[a] < 0 || (int64_t)o[a] + s[a] > d[a]) return false;
    return true;
}

int ensure_stage(lbm_lattice *l, size_t bytes) {
    if (bytes <= l->stage_bytes) return 0;
    if (l->stage) CU(cudaFree(l->stage));
    l->stage = nullptr;
    l->stage_bytes = 0;
    CU(cudaMalloc(&l->stage, bytes));
    l->stage_bytes = bytes;
    return 0;
}

// Parameters rounded to the arithmetic type R, plus the gravity chain
// coefficients of lbm_alpha.cl:183-291 computed in R.
template <typename R> void fill_params(const lbm_params &p, R out[P_COUNT], int *grav) {
    const R gx = (R)p.gravity[0], gy = (R)p.gravity[1], gz = (R)p.gravity[2];
    const R c18 = (R)(1.0f / 18.0f), c36 = (R)(1.0f / 36.0f);
    out[P_INV_TAU] = (R)p.inv_tau;
    out[P_TAU0] = (R)p.tau0;
    out[P_LES] = (R)p.les_c;
    out[P_LID] = (R)p.lid;
    R k[9];
    k[0] = gx * c18;
    k[1] = gy * (R)(-1.0f / 18.0f);
    k[2] = (gx - gy) * c36;
    k[3] = (gx + gy) * c36;
    k[4] = (gx + gz) * c36;
    k[5] = (gx - gz) * c36;
    k[6] = (gz - gy) * c36;
    k[7] = (gz + gy) * (R)(-1.0f / 36.0f);
    k[8] = gz * c18;
    int any = 0;
    for (int i = 0; i < 9; i++) {
        out[P_K0 + i] = k[i];
        if (k[i] != (R)0) any = 1;
    }
    *grav = any;
}

void set_params_desc(LatDesc &h, int storage, const lbm_params &p) {
    int grav = 0;
    if (storage == kF64) {
        fill_params<double>(p, h.pd, &grav);
        for (int i = 0; i < P_COUNT; i++) h.pf[i] = (float)h.pd[i];
    } else {
        fill_params<float>(p, h.pf, &grav);
        for (int i = 0; i < P_COUNT; i++) h.pd[i] = (double)h.pf[i];
    }
    h.grav = grav;
    h.gmode = p.gravity_mode ? 1 : 0;
}

// ---------------------------------------------------------------- kernels
template <typename S>
__global__ void k_init(LatDesc d, int b0, int b1, int b2, int b3, int b4, int b5, int store_v, int store_rho) {
    using R = typename Store<S>::R;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const int64_t x = c % d.nx, y = (c / d.nx) % d.ny, z = c / ((int64_t)d.nx * d.ny);
    int fl = kFluid;  // x faces win over y faces, y over z (lbm_init.cl:53-68)
    if (x == 0) fl = b0;
    else if (x == d.nx - 1) fl = b1;
    else if (y == 0) fl = b2;
    else if (y == d.ny - 1) fl = b3;
    else if (z == 0) fl = b4;
    else if (z == d.nz - 1) fl = b5;
    R eq[19];
    const R dp = (R)1.0f - K<R>::k15 * ((R)0 * (R)0);
    equilibria<R>((R)0, (R)0, (R)0, dp, eq);
    S *dd = (S *)d.dd;
#pragma unroll
    for (int i = 0; i < 19; i++) Store<S>::st(dd + i * d.pstride + c, eq[i], weight<R>(i));
    d.flags[c] = (uint8_t)fl;
    if (store_v) {
        R *u = (R *)d.vel;
        u[c] = 0; u[d.n + c] = 0; u[2 * d.n + c] = 0;
    }
    if (store_rho) ((R *)d.rho)[c] = (R)1.0f;
}

// Philox4x32-10 (Salmon et al., SC'11), same as the oracle's.
__device__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

template <typename S>
__global__ void k_perturb(LatDesc d, int ox, int oy, int oz, int gx, int gy, int gz, uint64_t seed, double amp,
                          int store_v, int store_rho) {
    using R = typename Store<S>::R;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const int64_t px = ox + c % d.nx, py = oy + (c / d.nx) % d.ny, pz = oz + c / ((int64_t)d.nx * d.ny);
    if (px <= 0 || py <= 0 || pz <= 0 || px >= gx - 1 || py >= gy - 1 || pz >= gz - 1) return;
    const uint64_t idx = (uint64_t)((pz * gy + py) * gx + px);
    uint32_t r[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0u};
    philox(r, (uint32_t)seed, (uint32_t)(seed >> 32));
    R u[3];
    for (int a = 0; a < 3; a++) {
        const double unit = (double)(r[a] >> 8) * (1.0 / 16777216.0);
        u[a] = (R)((unit * 2.0 - 1.0) * amp);
    }
    const R v2 = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2];
    const R dp = (R)1.0f - K<R>::k15 * v2;
    R eq[19];
    equilibria<R>(u[0], u[1], u[2], dp, eq);
    S *dd = (S *)d.dd;
#pragma unroll
    for (int i = 0; i < 19; i++) Store<S>::st(dd + opp(i) * d.pstride + c, eq[i], weight<R>(opp(i)));
    if (store_v) {
        R *v = (R *)d.vel;
        v[c] = u[0]; v[d.n + c] = u[1]; v[2 * d.n + c] = u[2];
    }
    if (store_rho) ((R *)d.rho)[c] = (R)1.0f;
}

// Exact quotient of a 32-bit unsigned n by an invariant d >= 1 with one
// multiply-high and two shifts (Granlund & Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994, figure 4.1).
struct FastDiv {
    uint32_t d, m, s1, s2;
    static FastDiv make(uint32_t d) {
        FastDiv f;
        uint32_t l = 0;
        while ((1ull << l) < d) l++;
        f.d = d;
        f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
        f.s1 = l < 1 ? l : 1;
        f.s2 = l > 1 ? l - 1 : 0;
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        const uint32_t t = __umulhi(m, n);
        return (t + ((n - t) >> s1)) >> s2;
    }
};

// A rectangle of a lattice: origin, size, and the lattice's row/slice pitch.
struct Box {
    int64_t lat_nx, lat_slice;
    int ox, oy, oz, sx, sy, sz;
    int64_t cells;
    FastDiv dx, dy;
};

__device__ __forceinline__ int64_t box_cell(const Box &b, uint32_t k) {
    const uint32_t r = b.dx.div(k);
    const uint32_t x = k - r * b.sx;
    const uint32_t z = b.dy.div(r);
    const uint32_t y = r - z * b.sy;
    return (int64_t)(b.oz + z) * b.lat_slice + (int64_t)(b.oy + y) * b.lat_nx + (b.ox + x);
}

// Up to 19 population planes to copy.
struct Planes {
    uint8_t f[20];
    int n;
};

// Populations between the lattice and a packed [plane][z][y][x] buffer of
// the arithmetic type: decoded when packing, encoded when unpacking.
// grid.y = index into the plane list.
template <typename S, bool PACK>
__global__ void k_box_dd(S *dd, int64_t pstride, typename Store<S>::R *buf, Box b, Planes pl) {
    using R = typename Store<S>::R;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= b.cells) return;
    const int f = pl.f[blockIdx.y];
    S *p = dd + f * pstride + box_cell(b, k);
    const int64_t t = (int64_t)f * b.cells + k;
    if (PACK) buf[t] = Store<S>::ld(p, weight<R>(f));
    else Store<S>::st(p, buf[t], weight<R>(f));
}

// Velocity / density planes: plain copies.
template <typename R, bool PACK>
__global__ void k_box_real(R *field, int64_t pstride, R *buf, Box b) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= b.cells) return;
    const int f = blockIdx.y;
    R *p = field + f * pstride + box_cell(b, k);
    const int64_t t = (int64_t)f * b.cells + k;
    if (PACK) buf[t] = *p;
    else *p = buf[t];
}

template <bool PACK>
__global__ void k_box_flags(uint8_t *flags, int32_t *buf, Box b) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= b.cells) return;
    uint8_t *p = flags + box_cell(b, k);
    if (PACK) buf[k] = *p;
    else *p = (uint8_t)buf[k];
}

__global__ void k_check_flags(const int32_t *buf, int64_t cells, int *bad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cells && (buf[t] < 0 || buf[t] > 255)) *bad = 1;
}

// Halo copy between two lattices of the same storage: raw elements of the
// selected planes.  grid = (cells, plane list index, copy index).
struct HaloDesc {
    void *src, *dst;
    int64_t sps, dps;
    Box sb, db;
    Planes pl;
};

template <typename E>
__device__ __forceinline__ void halo_elem(const HaloDesc &h) {
    if ((int)blockIdx.y >= h.pl.n) return;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= h.sb.cells) return;
    const int f = h.pl.f[blockIdx.y];
    ((E *)h.dst)[f * h.dps + box_cell(h.db, k)] = ((const E *)h.src)[f * h.sps + box_cell(h.sb, k)];
}

template <typename E>
__global__ void k_halo_one(HaloDesc h) {
    halo_elem<E>(h);
}

// All copies of one exchange phase (up to N) in the kernel parameters:
// their descriptor reads come from the constant bank (measured against a
// descriptor array in global memory at 256^3 in 2x2x1 subdomains, float:
// 16 instead of 30 registers, x faces 28.9 -> 27.2 us, y faces 10.8 ->
// 8.1 us per phase).
template <int N> struct HaloArgs {
    HaloDesc h[N];
};
constexpr int kHaloParam = 64;
static_assert(sizeof(HaloArgs<kHaloParam>) <= 32764, "halo descriptors exceed the kernel parameter space");

template <typename E, int N>
__global__ void k_halo_batch(const __grid_constant__ HaloArgs<N> a) {
    halo_elem<E>(a.h[blockIdx.z]);
}

// Neumaier-compensated FP64 accumulation.
struct Acc {
    double s, c;
    __device__ __forceinline__ void add(double v) {
        const double t = s + v;
        if (fabs(s) >= fabs(v)) c += (s - t) + v;
        else c += (v - t) + s;
        s = t;
    }
    __device__ __forceinline__ void merge(const Acc &o) {
        add(o.s);
        c += o.c;
    }
};

constexpr int kRedBlocks = 1024;

template <typename S>
__global__ void __launch_bounds__(kBlock) k_reduce(LatDesc d, int layout, double *partial) {
    using R = typename Store<S>::R;
    __shared__ Acc sh[5][kBlock];
    Acc a[5];
    for (int q = 0; q < 5; q++) a[q] = Acc{0.0, 0.0};
    const S *dd = (const S *)d.dd;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < d.n; c += (int64_t)gridDim.x * blockDim.x) {
        if (d.flags[c] != kFluid) continue;
        double r = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll
        for (int i = 0; i < 19; i++) {
            const int slot = layout ? opp(i) : i;
            const double f = (double)Store<S>::ld(dd + slot * d.pstride + c, weight<R>(slot));
            r += f;
            jx += dir_x(i) * f;
            jy += dir_y(i) * f;
            jz += dir_z(i) * f;
        }
        a[0].add(r);
        a[1].add(jx);
        a[2].add(jy);
        a[3].add(jz);
        a[4].add(0.5 * (jx * jx + jy * jy + jz * jz));
    }
    for (int q = 0; q < 5; q++) sh[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < 5; q++) sh[q][threadIdx.x].merge(sh[q][threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; q++) {
            partial[(blockIdx.x * 5 + q) * 2] = sh[q][0].s;
            partial[(blockIdx.x * 5 + q) * 2 + 1] = sh[q][0].c;
        }
}

// Velocity difference of two lattices of the same size over the fluid cells
// of `a`: max |ua - ub|, sum |ua - ub|^2, sum |ub|^2, max |ub|, cell count,
// with u the momentum of the stored populations in the given slot layouts.
template <typename SA, typename SB>
__global__ void __launch_bounds__(kBlock) k_compare(LatDesc a, int la, LatDesc b, int lb, double *partial) {
    using RA = typename Store<SA>::R;
    using RB = typename Store<SB>::R;
    __shared__ double sh[5][kBlock];
    double mx = 0, se = 0, sr = 0, mr = 0, cnt = 0;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.n; c += (int64_t)gridDim.x * blockDim.x) {
        if (a.flags[c] != kFluid) continue;
        double ua[3] = {0, 0, 0}, ub[3] = {0, 0, 0};
#pragma unroll
        for (int i = 0; i < 19; i++) {
            const int sa = la ? opp(i) : i, sb = lb ? opp(i) : i;
            const double fa = (double)Store<SA>::ld((const SA *)a.dd + sa * a.pstride + c, weight<RA>(sa));
            const double fb = (double)Store<SB>::ld((const SB *)b.dd + sb * b.pstride + c, weight<RB>(sb));
            ua[0] += dir_x(i) * fa; ua[1] += dir_y(i) * fa; ua[2] += dir_z(i) * fa;
            ub[0] += dir_x(i) * fb; ub[1] += dir_y(i) * fb; ub[2] += dir_z(i) * fb;
        }
        const double d0 = ua[0] - ub[0], d1 = ua[1] - ub[1], d2 = ua[2] - ub[2];
        const double e2 = d0 * d0 + d1 * d1 + d2 * d2, r2 = ub[0] * ub[0] + ub[1] * ub[1] + ub[2] * ub[2];
        mx = fmax(mx, sqrt(e2));
        mr = fmax(mr, sqrt(r2));
        se += e2;
        sr += r2;
        cnt += 1;
    }
    sh[0][threadIdx.x] = mx; sh[1][threadIdx.x] = se; sh[2][threadIdx.x] = sr; sh[3][threadIdx.x] = mr;
    sh[4][threadIdx.x] = cnt;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[0][threadIdx.x] = fmax(sh[0][threadIdx.x], sh[0][threadIdx.x + w]);
            sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
            sh[2][threadIdx.x] += sh[2][threadIdx.x + w];
            sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + w]);
            sh[4][threadIdx.x] += sh[4][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < 5) partial[blockIdx.x * 5 + threadIdx.x] = sh[threadIdx.x][0];
}

// Classes of the stored 16-bit deviations (fluid cells, all 19 slots):
// counts of all, zero, subnormal (nonzero below the format's smallest
// normal magnitude) and saturated (the format's largest finite magnitude or
// beyond) values, and the largest magnitude.  raw: the stored bits.
template <typename S> struct DevClass;
template <> struct DevClass<__half> {
    __device__ static int of(uint16_t b) {
        const uint32_t e = (b >> 10) & 31u, m = b & 1023u;
        return e == 0 ? (m ? 2 : 1) : (e == 31 || (b & 0x7fffu) == 0x7bffu) ? 3 : 0;
    }
};
template <> struct DevClass<__nv_bfloat16> {
    __device__ static int of(uint16_t b) {
        const uint32_t e = (b >> 7) & 255u, m = b & 127u;
        return e == 0 ? (m ? 2 : 1) : (e == 255 || (b & 0x7fffu) == 0x7f7fu) ? 3 : 0;
    }
};
template <> struct DevClass<c16_t> {
    __device__ static int of(uint16_t b) {
        const uint32_t e = (b >> 12) & 7u, m = b & 4095u;
        return e == 0 ? (m ? 2 : 1) : (b & 0x7fffu) == 0x7fffu ? 3 : 0;
    }
};

template <typename S>
__global__ void __launch_bounds__(kBlock) k_dev_stats(LatDesc d, unsigned long long *count, unsigned int *maxbits) {
    unsigned long long n[4] = {0, 0, 0, 0};
    float mx = 0.0f;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < d.n; c += (int64_t)gridDim.x * blockDim.x) {
        if (d.flags[c] != kFluid) continue;
#pragma unroll
        for (int i = 0; i < 19; i++) {
            const S *p = (const S *)d.dd + i * d.pstride + c;
            n[0]++;
            const int k = DevClass<S>::of(*(const uint16_t *)p);
            if (k) n[k]++;
            mx = fmaxf(mx, fabsf(Store<S>::dld(p)));
        }
    }
    for (int q = 0; q < 4; q++) {
        unsigned long long v = n[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&count[q], v);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, __float_as_uint(mx));  // non-negative floats order as integers
}

__global__ void k_compare_final(const double *partial, int nblocks, double *out) {
    if (threadIdx.x != 0) return;
    double r[5] = {0, 0, 0, 0, 0};
    for (int b = 0; b < nblocks; b++) {
        r[0] = fmax(r[0], partial[b * 5 + 0]);
        r[1] += partial[b * 5 + 1];
        r[2] += partial[b * 5 + 2];
        r[3] = fmax(r[3], partial[b * 5 + 3]);
        r[4] += partial[b * 5 + 4];
    }
    for (int q = 0; q < 5; q++) out[q] = r[q];
}

__global__ void k_reduce_final(const double *partial, int nblocks, double *out) {
    if (threadIdx.x >= 5) return;
    const int q = threadIdx.x;
    Acc a{0.0, 0.0};
    for (int b = 0; b < nblocks; b++) {
        a.add(partial[(b * 5 + q) * 2]);
        a.c += partial[(b * 5 + q) * 2 + 1];
    }
    out[q] = a.s + a.c;
}

// ------------------------------------------------------------- dispatchers
template <typename S, bool PAIR>
int launch_step_t(int parity, bool les, const DomainArgs &a, int blocks, cudaStream_t st) {
    if (blocks <= 0) return 0;
#define STEP(K_, L_) K_<S, L_><<<blocks, kBlock, 0, st>>>(a)
    if constexpr (PAIR) {
        if (parity) { if (les) STEP(k_alpha2, true); else STEP(k_alpha2, false); }
        else { if (les) STEP(k_beta2, true); else STEP(k_beta2, false); }
    } else {
        if (parity) { if (les) STEP(k_alpha, true); else STEP(k_alpha, false); }
        else { if (les) STEP(k_beta, true); else STEP(k_beta, false); }
    }
#undef STEP
    CU(cudaGetLastError());
    return 0;
}

// The two-cell kernels apply to the float arithmetic types when every
// lattice of the launch has an even x extent.
bool pair_shape(int storage, const LatDesc *tab, int ntab) {
    if (storage == kF64) return false;
    for (int i = 0; i < ntab; i++)
        if (tab[i].nx & 1) return false;
    return true;
}

int effective_shape(int storage, int shape, const LatDesc *tab, int ntab) {
    if (shape == 0) shape = (storage == kF16 || storage == kBF16 || storage == kC16) ? 3 : 1;  // the measured best per storage
    if (shape == 2 && pair_shape(storage, tab, ntab)) return 2;
    if (shape == 3 && storage != kF64) return 3;
    return 1;
}

static int launch_chunk(int storage, bool pair, int parity, bool les, const DomainArgs &a, int blocks,
                        cudaStream_t st) {
    if (pair) {
        switch (storage) {
            case kF32: return launch_step_t<float, true>(parity, les, a, blocks, st);
            case kF16: return launch_step_t<__half, true>(parity, les, a, blocks, st);
            case kBF16: return launch_step_t<__nv_bfloat16, true>(parity, les, a, blocks, st);
            case kC16: return launch_step_t<c16_t, true>(parity, les, a, blocks, st);
        }
        return fail("the two-cell kernels need a float arithmetic type");
    }
    switch (storage) {
        case kF32: return launch_step_t<float, false>(parity, les, a, blocks, st);
        case kF64: return launch_step_t<double, false>(parity, les, a, blocks, st);
        case kF16: return launch_step_t<__half, false>(parity, les, a, blocks, st);
        case kBF16: return launch_step_t<__nv_bfloat16, false>(parity, les, a, blocks, st);
        case kC16: return launch_step_t<c16_t, false>(parity, les, a, blocks, st);
    }
    return fail("unknown storage type");
}

// Streaming multiprocessors of the current device (cached per device).
static int sm_count() {
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

template <typename S, bool LES, bool BETA, bool ONE, int N, int ADDR>
static int launch_staged_w(const StepArgs<N> &a, int tiles, cudaStream_t st) {
    // the ring exceeds the default 48 KB of dynamic shared memory; the limit
    // is raised once per device
    static bool attr[64] = {};
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail("device index out of range");
    if (!attr[dev]) {
        CU(cudaFuncSetAttribute(k_step_staged<S, LES, BETA, ONE, N, ADDR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                Tile<S>::SMEM));
        attr[dev] = true;
    }
    const int grid = std::min(tiles, sm_count() * kStageBlocksPerSM);
    k_step_staged<S, LES, BETA, ONE, N, ADDR><<<grid, kStageThreads, Tile<S>::SMEM, st>>>(a, tiles);
    CU(cudaGetLastError());
    return 0;
}

// Beta steps whose lattices all span fewer than 2^32 population elements
// form their scatter addresses in 32-bit arithmetic (scatter_ptr): from a
// table of the 19 offsets when the lattices share their shape (domains and
// single lattices), else computed per lattice (ensembles).
template <typename S, bool LES, bool BETA, bool ONE, int N = kParamLattices>
static int launch_staged_one(const StepArgs<N> &a, int tiles, cudaStream_t st) {
    if constexpr (BETA) {
        bool w32 = true, same = true;
        for (int i = 0; i < a.ntab; i++) {
            if (19 * a.tab[i].pstride >= ((int64_t)1 << 32)) w32 = false;
            if (a.tab[i].nx != a.tab[0].nx || a.tab[i].ny != a.tab[0].ny || a.tab[i].pstride != a.tab[0].pstride)
                same = false;
        }
        if constexpr (N == kParamLattices) {
            if (w32 && same) {
                StepArgs<N> b = a;
                const uint32_t nx = (uint32_t)a.tab[0].nx, sl = nx * (uint32_t)a.tab[0].ny;
                for (int i = 0; i < 19; i++)
                    b.koff[i] = (uint32_t)i * (uint32_t)a.tab[0].pstride + (uint32_t)dir_x(i) +
                                (uint32_t)dir_y(i) * nx + (uint32_t)dir_z(i) * sl;
                return launch_staged_w<S, LES, BETA, ONE, N, kAddrTab>(b, tiles, st);
            }
        } else {
            (void)same;
            if (w32) return launch_staged_w<S, LES, BETA, ONE, N, kAddr32>(a, tiles, st);
        }
    }
    return launch_staged_w<S, LES, BETA, ONE, N, kAddr64>(a, tiles, st);
}

template <typename S, bool LES, bool BETA>
static int launch_staged_k(const DomainArgs &a, int tiles, cudaStream_t st) {
    return a.ntab == 1 ? launch_staged_one<S, LES, BETA, true>(a, tiles, st)
                       : launch_staged_one<S, LES, BETA, false>(a, tiles, st);
}

template <typename S>
static int launch_staged_t(int parity, bool les, const DomainArgs &a, int tiles, cudaStream_t st) {
    if (tiles <= 0) return 0;
    if (parity) return les ? launch_staged_k<S, true, false>(a, tiles, st) : launch_staged_k<S, false, false>(a, tiles, st);
    return les ? launch_staged_k<S, true, true>(a, tiles, st) : launch_staged_k<S, false, true>(a, tiles, st);
}

int staged_cells(int storage) {
    switch (storage) {
        case kF32: return Tile<float>::T;
        case kF16: return Tile<__half>::T;
        case kBF16: return Tile<__nv_bfloat16>::T;
        case kC16: return Tile<c16_t>::T;
    }
    return 0;
}

template <typename S>
static int launch_staged_batch_t(bool beta, bool les, const BatchArgs &a, int tiles, cudaStream_t st) {
    if (tiles <= 0) return 0;
    if (beta)
        return les ? launch_staged_one<S, true, true, false, kBatchLattices>(a, tiles, st)
                   : launch_staged_one<S, false, true, false, kBatchLattices>(a, tiles, st);
    return les ? launch_staged_one<S, true, false, false, kBatchLattices>(a, tiles, st)
               : launch_staged_one<S, false, false, false, kBatchLattices>(a, tiles, st);
}

int launch_staged_batch(int storage, bool beta, bool les, const BatchArgs &a, int tiles, cudaStream_t st) {
    switch (storage) {
        case kF32: return launch_staged_batch_t<float>(beta, les, a, tiles, st);
        case kF16: return launch_staged_batch_t<__half>(beta, les, a, tiles, st);
        case kBF16: return launch_staged_batch_t<__nv_bfloat16>(beta, les, a, tiles, st);
        case kC16: return launch_staged_batch_t<c16_t>(beta, les, a, tiles, st);
    }
    return fail("the staged kernels take float, half or bfloat16 storage");
}

int launch_step(int storage, int shape, int parity, bool les, const LatDesc *htab, int ntab, int sv, int sr,
                cudaStream_t st) {
    // the staged beta needs rows of whole 16-byte units (nx a multiple of 4
    // float or 8 half populations)
    bool staged = shape == 3 && storage != kF64;
    if (staged && parity == 0)
        for (int i = 0; i < ntab; i++)
            if ((htab[i].nx * storage_bytes(storage)) % 16) staged = false;
    const bool pair = shape == 2;
    const int per = staged ? staged_cells(storage) : cells_per_block(pair);
    for (int c0 = 0; c0 < ntab; c0 += kParamLattices) {
        DomainArgs a;
        memset(&a, 0, sizeof(a));
        a.ntab = std::min(kParamLattices, ntab - c0);
        a.store_v = sv;
        a.store_rho = sr;
        int units = 0;
        for (int i = 0; i < a.ntab; i++) {
            a.tab[i] = htab[c0 + i];
            a.tab[i].first_block = units;
            a.tab[i].nblocks = (int)((a.tab[i].n + per - 1) / per);
            units += a.tab[i].nblocks;
        }
        // One-cell alpha steps that push x faces into their neighbours' ghost
        // columns, over subdomains of equal block counts: interleave the
        // blocks, so that a pushed element and the receiver's own stores to
        // the same 32-byte sector meet in L2 and leave it as one full sector
        // (measured at 256^3 in 2x2x1 subdomains, f32: alpha 460 -> 448 us
        // with 5 pushed populations, 519 -> 475 us with 19; beta steps, which
        // push nothing, ran 1 % slower interleaved and keep the plain order).
        bool inter = !staged && !pair && parity == 1 && a.ntab > 1;
        bool push = false;
        for (int i = 0; i < a.ntab; i++) {
            inter = inter && a.tab[i].nblocks == a.tab[0].nblocks;
            push = push || a.tab[i].xhi || a.tab[i].xlo;
        }
        a.interleave = inter && push ? 1 : 0;
        int rc;
        if (shape == kShapeF64Fma && storage == kF64) {
            rc = launch_step_f64_fma(parity, les, a, units, st);
        } else if (staged) {
            switch (storage) {
                case kF32: rc = launch_staged_t<float>(parity, les, a, units, st); break;
                case kF16: rc = launch_staged_t<__half>(parity, les, a, units, st); break;
                case kBF16: rc = launch_staged_t<__nv_bfloat16>(parity, les, a, units, st); break;
                default: rc = launch_staged_t<c16_t>(parity, les, a, units, st); break;
            }
        } else {
            rc = launch_chunk(storage, pair, parity, les, a, units, st);
        }
        if (rc) return -1;
    }
    return 0;
}

Box make_box(const lbm_lattice *l, const int o[3], const int s[3]) {
    Box b;
    b.lat_nx = l->nx;
    b.lat_slice = (int64_t)l->nx * l->ny;
    b.ox = o[0]; b.oy = o[1]; b.oz = o[2];
    b.sx = s[0]; b.sy = s[1]; b.sz = s[2];
    b.cells = (int64_t)s[0] * s[1] * s[2];
    b.dx = FastDiv::make(s[0] > 0 ? s[0] : 1);
    b.dy = FastDiv::make(s[1] > 0 ? s[1] : 1);
    return b;
}

// Planes f with sign * (norm . e_f) > 0, or all 19 when norm is null.
Planes plane_list(const int norm[3], int sign = 1) {
    Planes p;
    p.n = 0;
    for (int f = 0; f < 19; f++)
        if (!norm || sign * (norm[0] * dir_x(f) + norm[1] * dir_y(f) + norm[2] * dir_z(f)) > 0) p.f[p.n++] = (uint8_t)f;
    return p;
}

dim3 halo_grid(int64_t cells, int planes, int copies) {
    return dim3((unsigned)((cells + kBlock - 1) / kBlock), (unsigned)planes, (unsigned)copies);
}

template <typename E>
int launch_halo_one(const HaloDesc &h, cudaStream_t st) {
    k_halo_one<E><<<halo_grid(h.sb.cells, h.pl.n, 1), kBlock, 0, st>>>(h);
    CU(cudaGetLastError());
    return 0;
}

template <typename E, int N>
static int launch_halo_param(const HaloDesc *hd, int n, int64_t max_cells, int max_planes, cudaStream_t st) {
    HaloArgs<N> a;
    memset(&a, 0, sizeof(a));
    memcpy(a.h, hd, (size_t)n * sizeof(HaloDesc));
    k_halo_batch<E, N><<<halo_grid(max_cells, max_planes, n), kBlock, 0, st>>>(a);
    CU(cudaGetLastError());
    return 0;
}

template <typename E>
static int launch_halo_chunks(const HaloDesc *hd, int nd, int64_t max_cells, int max_planes, cudaStream_t st) {
    for (int c0 = 0; c0 < nd; c0 += kHaloParam) {
        const int n = std::min(kHaloParam, nd - c0);
        const int rc = n <= 8 ? launch_halo_param<E, 8>(hd + c0, n, max_cells, max_planes, st)
                              : launch_halo_param<E, kHaloParam>(hd + c0, n, max_cells, max_planes, st);
        if (rc) return rc;
    }
    return 0;
}

// All copies of one exchange phase (independent of one another): one launch
// per kHaloParam copies, descriptors from host memory.
int launch_halo_batch(int storage, const HaloDesc *hd, int nd, int64_t max_cells, int max_planes, cudaStream_t st) {
    if (nd <= 0 || max_cells <= 0) return 0;
    switch (storage_bytes(storage)) {
        case 2: return launch_halo_chunks<uint16_t>(hd, nd, max_cells, max_planes, st);
        case 4: return launch_halo_chunks<uint32_t>(hd, nd, max_cells, max_planes, st);
        default: return launch_halo_chunks<uint64_t>(hd, nd, max_cells, max_planes, st);
    }
}
}  // namespace lbm_rt

// Check of the bounded waits: one block waits, `polls` polls at most, on a
// barrier phase that nothing completes (no copy is issued), records
// kStageTimeout in g_stage_error as the staged kernels do, and returns.
static __global__ void k_wait_probe(uint32_t polls) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    const bool ok = mbar_wait(&bar, 0, polls);
    if (!__any_sync(0xffffffffu, ok) && threadIdx.x == 0) atomicOr(&g_stage_error, kStageTimeout);
}

// =================================================================== C ABI
extern "C" {

const char *lbm_cu_last_error(void) { return g_err.c_str(); }

const char *lbm_cu_version(void) {
    return "lbm_gb300 D3Q19 A-A (alpha/beta), sm_103a, -fmad=false, IEEE div/sqrt";
}

int lbm_cu_synchronize(void *stream) {
    if (stream) CU(cudaStreamSynchronize(S(stream)));
    else CU(cudaDeviceSynchronize());
    unsigned int err = 0;
    CU(cudaMemcpyFromSymbol(&err, g_stage_error, sizeof(err)));
    if (err) {
        const unsigned int zero = 0;
        CU(cudaMemcpyToSymbol(g_stage_error, &zero, sizeof(zero)));
        return fail("a staged step kernel gave up waiting for its bulk copies");
    }
    return 0;
}

int lbm_cu_check_wait_timeout(unsigned int polls, void *stream) {
    if (polls == 0 || polls > kStageWaitLimit) return fail("polls must be in 1..2^22");
    k_wait_probe<<<1, 32, 0, S(stream)>>>(polls);
    CU(cudaGetLastError());
    return 0;
}

int lbm_cu_create(int nx, int ny, int nz, int storage, int store_velocity, int store_density, lbm_lattice **out) {
    if (!out) return fail("out is NULL");
    *out = nullptr;
    if (nx < 3 || ny < 3 || nz < 3) return fail("each lattice dimension must be at least 3");
    if (storage < kF32 || storage > kC16) return fail("unknown storage type");
    const int64_t n = (int64_t)nx * ny * nz;
    if (n > ((int64_t)1 << 31) - 1) return fail("lattice has more than 2^31-1 cells");
    lbm_lattice *l = new lbm_lattice();
    l->nx = nx; l->ny = ny; l->nz = nz;
    l->n = n;
    l->pstride = round_up(n, 256 / (int64_t)storage_bytes(storage));
    l->storage = storage;
    l->store_v = store_velocity ? 1 : 0;
    l->store_rho = store_density ? 1 : 0;
    auto cleanup = [&](const std::string &m) {
        lbm_cu_destroy(l);
        return fail(m);
    };
    if (cudaMalloc(&l->dd, (size_t)l->pstride * 19 * storage_bytes(storage)) != cudaSuccess)
        return cleanup("cudaMalloc of the population planes failed");
    if (cudaMalloc((void **)&l->flags, (size_t)round_up(n, 256)) != cudaSuccess) return cleanup("cudaMalloc of flags failed");
    if (l->store_v && cudaMalloc(&l->vel, (size_t)n * 3 * real_bytes(storage)) != cudaSuccess)
        return cleanup("cudaMalloc of velocity failed");
    if (l->store_rho && cudaMalloc(&l->rho, (size_t)n * real_bytes(storage)) != cudaSuccess)
        return cleanup("cudaMalloc of density failed");
    if (cudaMalloc((void **)&l->d_desc, sizeof(LatDesc)) != cudaSuccess) return cleanup("cudaMalloc of descriptor failed");
    LatDesc &h = l->h;
    h.dd = l->dd; h.flags = l->flags; h.vel = l->vel; h.rho = l->rho;
    h.pstride = l->pstride; h.n = n;
    h.nx = nx; h.ny = ny; h.nz = nz;
    h.first_block = 0;
    h.nblocks = grid_for(n);
    lbm_params p{};
    p.inv_tau = 1.0 / 0.953575;  // reference default tau (src/CLbmSkeleton.hpp:142)
    p.tau0 = 0.953575;
    set_params_desc(h, storage, p);
    l->dirty = true;
    cudaGetLastError();
    *out = l;
    return 0;
}

int lbm_cu_destroy(lbm_lattice *l) {
    if (!l) return 0;
    if (l->dd) cudaFree(l->dd);
    if (l->flags) cudaFree(l->flags);
    if (l->vel) cudaFree(l->vel);
    if (l->rho) cudaFree(l->rho);
    if (l->d_desc) cudaFree(l->d_desc);
    if (l->stage) cudaFree(l->stage);
    delete l;
    return 0;
}

int lbm_cu_dims(const lbm_lattice *l, int dims[3]) {
    if (!l || !dims) return fail("NULL argument");
    dims[0] = l->nx; dims[1] = l->ny; dims[2] = l->nz;
    return 0;
}

int lbm_cu_set_params(lbm_lattice *l, const lbm_params *p) {
    if (!l || !p) return fail("NULL argument");
    if (p->les_c != 0.0 && !(p->tau0 > 0.5)) return fail("the subgrid model needs tau0 > 0.5");
    set_params_desc(l->h, l->storage, *p);
    l->dirty = true;
    return 0;
}

int lbm_cu_init(lbm_lattice *l, const int bc[6], void *stream) {
    if (!l || !bc) return fail("NULL argument");
    for (int i = 0; i < 6; i++)
        if (bc[i] < 0 || bc[i] > 255) return fail("boundary flags must fit in one byte");
    const int g = grid_for(l->n);
    switch (l->storage) {
        case kF32: k_init<float><<<g, kBlock, 0, S(stream)>>>(l->h, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], l->store_v, l->store_rho); break;
        case kF64: k_init<double><<<g, kBlock, 0, S(stream)>>>(l->h, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], l->store_v, l->store_rho); break;
        case kF16: k_init<__half><<<g, kBlock, 0, S(stream)>>>(l->h, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], l->store_v, l->store_rho); break;
        case kBF16: k_init<__nv_bfloat16><<<g, kBlock, 0, S(stream)>>>(l->h, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], l->store_v, l->store_rho); break;
        case kC16: k_init<c16_t><<<g, kBlock, 0, S(stream)>>>(l->h, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], l->store_v, l->store_rho); break;
    }
    CU(cudaGetLastError());
    return 0;
}

int lbm_cu_perturb(lbm_lattice *l, const int o[3], const int ph[3], uint64_t seed, double amp, void *stream) {
    if (!l || !o || !ph) return fail("NULL argument");
    const int g = grid_for(l->n);
#define PERT(S_) k_perturb<S_><<<g, kBlock, 0, S(stream)>>>(l->h, o[0], o[1], o[2], ph[0], ph[1], ph[2], seed, amp, l->store_v, l->store_rho)
    switch (l->storage) {
        case kF32: PERT(float); break;
        case kF64: PERT(double); break;
        case kF16: PERT(__half); break;
        case kBF16: PERT(__nv_bfloat16); break;
        case kC16: PERT(c16_t); break;
    }
#undef PERT
    CU(cudaGetLastError());
    return 0;
}

int lbm_cu_step(lbm_lattice *l, int parity, void *stream) {
    if (!l) return fail("NULL lattice");
    const LatDesc &h = l->h;
    const int shape = l->fma64 && l->storage == kF64 ? kShapeF64Fma : effective_shape(l->storage, l->shape, &h, 1);
    return launch_step(l->storage, shape, parity & 1, uses_les(h), &h, 1,
                       l->store_v, l->store_rho, S(stream));
}

static int box_io(lbm_lattice *l, int field, const int o[3], const int s[3], void *host, const int norm[3],
                  bool read, cudaStream_t st) {
    static const int zero[3] = {0, 0, 0};
    int full[3] = {l->nx, l->ny, l->nz};
    if (!o) o = zero;
    if (!s) s = full;
    if (!valid_box(l, o, s)) return fail("rectangle outside the lattice");
    if (!host) return fail("NULL host buffer");
    const int64_t cells = (int64_t)s[0] * s[1] * s[2];
    if (cells == 0) return 0;
    const size_t rb = real_bytes(l->storage);
    int nplanes;
    size_t ebytes;
    switch (field) {
        case LBM_FIELD_DD: nplanes = 19; ebytes = rb; break;
        case LBM_FIELD_VELOCITY:
            if (!l->vel) return fail("velocity is not stored by this lattice");
            nplanes = 3; ebytes = rb; break;
        case LBM_FIELD_DENSITY:
            if (!l->rho) return fail("density is not stored by this lattice");
            nplanes = 1; ebytes = rb; break;
        case LBM_FIELD_FLAGS: nplanes = 1; ebytes = 4; break;
        default: return fail("unknown field");
    }
    const size_t bytes = (size_t)cells * nplanes * ebytes;
    if (cells > INT32_MAX) return fail("rectangle has more than 2^31-1 cells");
    // The whole lattice of a field whose host layout is its device layout
    // (float / double populations: stored values are the populations; velocity
    // and density planes of n cells): copy engine transfers straight between
    // the host buffer and the planes, no staging buffer and no kernel.
    const bool whole = o[0] == 0 && o[1] == 0 && o[2] == 0 && s[0] == l->nx && s[1] == l->ny && s[2] == l->nz;
    if (whole && field != LBM_FIELD_FLAGS && (field != LBM_FIELD_DD || storage_bytes(l->storage) == rb)) {
        const auto kind = read ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
        char *h = (char *)host;
        if (field == LBM_FIELD_DD) {
            const Planes pl = plane_list(read ? nullptr : norm);
            const size_t pb = (size_t)l->n * rb;
            for (int k = 0; k < pl.n; k++) {
                const int f = pl.f[k];
                char *dev = (char *)l->dd + (size_t)f * l->pstride * rb;
                CU(cudaMemcpyAsync(read ? (void *)(h + f * pb) : (void *)dev, read ? (const void *)dev : h + f * pb, pb,
                                   kind, st));
            }
        } else {
            char *dev = (char *)(field == LBM_FIELD_VELOCITY ? l->vel : l->rho);
            CU(cudaMemcpyAsync(read ? (void *)h : (void *)dev, read ? (const void *)dev : (const void *)h, bytes, kind,
                               st));
        }
        CU(cudaStreamSynchronize(st));
        return 0;
    }
    if (ensure_stage(l, bytes + 256)) return -1;
    Box b = make_box(l, o, s);
    if (!read) CU(cudaMemcpyAsync(l->stage, host, bytes, cudaMemcpyHostToDevice, st));
    const unsigned gx = (unsigned)((cells + kBlock - 1) / kBlock);
    if (field == LBM_FIELD_DD) {
        const Planes pl = plane_list(read ? nullptr : norm);
        const dim3 g(gx, (unsigned)pl.n);
#define BOX(S_, R_)                                                                                          \
    (read ? k_box_dd<S_, true><<<g, kBlock, 0, st>>>((S_ *)l->dd, l->pstride, (R_ *)l->stage, b, pl)         \
          : k_box_dd<S_, false><<<g, kBlock, 0, st>>>((S_ *)l->dd, l->pstride, (R_ *)l->stage, b, pl))
        switch (l->storage) {
            case kF32: BOX(float, float); break;
            case kF64: BOX(double, double); break;
            case kF16: BOX(__half, float); break;
            case kBF16: BOX(__nv_bfloat16, float); break;
            case kC16: BOX(c16_t, float); break;
        }
#undef BOX
    } else if (field == LBM_FIELD_FLAGS) {
        if (!read) {
            int *bad = (int *)((char *)l->stage + bytes);
            CU(cudaMemsetAsync(bad, 0, sizeof(int), st));
            k_check_flags<<<grid_for(cells), kBlock, 0, st>>>((const int32_t *)l->stage, cells, bad);
            int hbad = 0;
            CU(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
            if (hbad) return fail("flag values must lie in [0, 255]");
            k_box_flags<false><<<gx, kBlock, 0, st>>>(l->flags, (int32_t *)l->stage, b);
        } else {
            k_box_flags<true><<<gx, kBlock, 0, st>>>(l->flags, (int32_t *)l->stage, b);
        }
    } else {
        void *fieldp = field == LBM_FIELD_VELOCITY ? l->vel : l->rho;
        const dim3 g(gx, (unsigned)nplanes);
        if (rb == 8) {
            if (read) k_box_real<double, true><<<g, kBlock, 0, st>>>((double *)fieldp, l->n, (double *)l->stage, b);
            else k_box_real<double, false><<<g, kBlock, 0, st>>>((double *)fieldp, l->n, (double *)l->stage, b);
        } else {
            if (read) k_box_real<float, true><<<g, kBlock, 0, st>>>((float *)fieldp, l->n, (float *)l->stage, b);
            else k_box_real<float, false><<<g, kBlock, 0, st>>>((float *)fieldp, l->n, (float *)l->stage, b);
        }
    }
    CU(cudaGetLastError());
    if (read) CU(cudaMemcpyAsync(host, l->stage, bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return 0;
}

int lbm_cu_read(lbm_lattice *l, int field, const int origin[3], const int size[3], void *host_dst, void *stream) {
    if (!l) return fail("NULL lattice");
    return box_io(l, field, origin, size, host_dst, nullptr, true, S(stream));
}

int lbm_cu_write(lbm_lattice *l, int field, const int origin[3], const int size[3], const void *host_src,
                 const int norm[3], void *stream) {
    if (!l) return fail("NULL lattice");
    if (norm && field != LBM_FIELD_DD) return fail("a normal mask applies to populations only");
    return box_io(l, field, origin, size, const_cast<void *>(host_src), norm, false, S(stream));
}

int lbm_cu_halo(lbm_lattice *src, const int so[3], lbm_lattice *dst, const int dof[3], const int size[3],
                const int norm[3], void *stream) {
    if (!src || !dst || !so || !dof || !size) return fail("NULL argument");
    if (src->storage != dst->storage) return fail("halo copy between lattices of different storage");
    if (!valid_box(src, so, size) || !valid_box(dst, dof, size)) return fail("halo rectangle outside a lattice");
    HaloDesc h;
    h.src = src->dd; h.dst = dst->dd;
    h.sps = src->pstride; h.dps = dst->pstride;
    h.sb = make_box(src, so, size);
    h.db = make_box(dst, dof, size);
    h.pl = plane_list(norm);
    if (h.sb.cells == 0) return 0;
    if (h.sb.cells > INT32_MAX) return fail("halo rectangle has more than 2^31-1 cells");
    switch (storage_bytes(src->storage)) {
        case 2: return launch_halo_one<uint16_t>(h, S(stream));
        case 4: return launch_halo_one<uint32_t>(h, S(stream));
        default: return launch_halo_one<uint64_t>(h, S(stream));
    }
}

int lbm_cu_reduce_conserved(lbm_lattice *l, int layout, double out[5], void *stream) {
    if (!l || !out) return fail("NULL argument");
    const size_t need = (size_t)kRedBlocks * 10 * sizeof(double) + 8 * sizeof(double);
    if (ensure_stage(l, need)) return -1;
    double *partial = (double *)l->stage;
    double *res = partial + (size_t)kRedBlocks * 10;
    const int blocks = std::min<int64_t>(kRedBlocks, std::max<int64_t>(1, grid_for(l->n)));
    cudaStream_t st = S(stream);
    switch (l->storage) {
        case kF32: k_reduce<float><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kF64: k_reduce<double><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kF16: k_reduce<__half><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kBF16: k_reduce<__nv_bfloat16><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kC16: k_reduce<c16_t><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
    }
    CU(cudaGetLastError());
    k_reduce_final<<<1, 32, 0, st>>>(partial, blocks, res);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(out, res, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return 0;
}

int lbm_cu_compare_velocity(lbm_lattice *a, int layout_a, lbm_lattice *b, int layout_b, double out[5],
                            void *stream) {
    if (!a || !b || !out) return fail("NULL argument");
    if (a->nx != b->nx || a->ny != b->ny || a->nz != b->nz) return fail("lattices differ in size");
    const size_t need = (size_t)kRedBlocks * 5 * sizeof(double) + 8 * sizeof(double);
    if (ensure_stage(a, need)) return -1;
    double *partial = (double *)a->stage;
    double *res = partial + (size_t)kRedBlocks * 5;
    const int blocks = std::min<int64_t>(kRedBlocks, std::max<int64_t>(1, grid_for(a->n)));
    cudaStream_t st = S(stream);
#define CMP(SA_, SB_) k_compare<SA_, SB_><<<blocks, kBlock, 0, st>>>(a->h, layout_a & 1, b->h, layout_b & 1, partial)
#define CMPB(SA_)                                   \
    switch (b->storage) {                           \
        case kF32: CMP(SA_, float); break;          \
        case kF64: CMP(SA_, double); break;         \
        case kF16: CMP(SA_, __half); break;         \
        case kBF16: CMP(SA_, __nv_bfloat16); break; \
        case kC16: CMP(SA_, c16_t); break;          \
    }
    switch (a->storage) {
        case kF32: CMPB(float); break;
        case kF64: CMPB(double); break;
        case kF16: CMPB(__half); break;
        case kBF16: CMPB(__nv_bfloat16); break;
        case kC16: CMPB(c16_t); break;
    }
#undef CMPB
#undef CMP
    CU(cudaGetLastError());
    k_compare_final<<<1, 32, 0, st>>>(partial, blocks, res);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(out, res, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return 0;
}

int lbm_cu_deviation_stats(lbm_lattice *l, double out[5], void *stream) {
    if (!l || !out) return fail("NULL argument");
    if (l->storage != kF16 && l->storage != kBF16 && l->storage != kC16)
        return fail("deviation statistics exist for the 16-bit storage types");
    if (ensure_stage(l, 64)) return -1;
    unsigned long long *cnt = (unsigned long long *)l->stage;
    unsigned int *mx = (unsigned int *)(cnt + 4);
    cudaStream_t st = S(stream);
    CU(cudaMemsetAsync(l->stage, 0, 64, st));
    const int blocks = std::min<int64_t>(kRedBlocks, std::max<int64_t>(1, grid_for(l->n)));
    switch (l->storage) {
        case kF16: k_dev_stats<__half><<<blocks, kBlock, 0, st>>>(l->h, cnt, mx); break;
        case kBF16: k_dev_stats<__nv_bfloat16><<<blocks, kBlock, 0, st>>>(l->h, cnt, mx); break;
        default: k_dev_stats<c16_t><<<blocks, kBlock, 0, st>>>(l->h, cnt, mx); break;
    }
    CU(cudaGetLastError());
    unsigned long long h[4];
    unsigned int hm = 0;
    CU(cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&hm, mx, sizeof(hm), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    float m;
    memcpy(&m, &hm, 4);
    for (int q = 0; q < 4; q++) out[q] = (double)h[q];
    out[4] = m;
    return 0;
}

}  // extern "C"

// ------------------------------------------ reduction without allocation
// Some callers must not allocate device memory: a serving loop that has
// handed every free byte of HBM to resident fields under a budget, a monitor
// thread that checks conservation while other streams run and cannot take
// the device-wide synchronisation cudaMalloc/cudaFree may imply, or a host
// framework whose own allocator owns the device.  For them the partial sums
// of the conservation reduction live in this fixed array instead of the
// lattice's staging buffer: one partial (sum and compensation of 5
// quantities) per block of 256 threads x 32 cells, at most kStaticPartials
// blocks, so lattices of up to kStaticPartials * kStaticCellsPerBlock cells.
// The array exists once per GPU that loads this library and stays allocated
// until the process exits.  Every call reuses it: each call writes every
// partial it later reads, so nothing has to be cleared, but two calls whose
// work overlaps on the GPU (different streams, no ordering) race on it.
constexpr int kStaticPartials = 16384;
constexpr int64_t kStaticCellsPerBlock = (int64_t)kBlock * 32;
static __device__ __align__(256) double g_reduce_scratch[kStaticPartials * 10 + 8];

// Final stage over up to kStaticPartials partials: warp q sums quantity q,
// each lane a strided share with its own compensated sum, then the lanes'
// sums are merged by shuffles (one block of 5 warps; a single thread per
// quantity would walk all 16384 partials one after another).
__global__ void __launch_bounds__(160) k_reduce_final_warps(const double *partial, int nblocks, double *out) {
    const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Acc a{0.0, 0.0};
    for (int b = lane; b < nblocks; b += 32) {
        a.add(partial[(b * 5 + q) * 2]);
        a.c += partial[(b * 5 + q) * 2 + 1];
    }
    for (int o = 16; o > 0; o >>= 1) {
        const Acc other{__shfl_down_sync(0xffffffffu, a.s, o), __shfl_down_sync(0xffffffffu, a.c, o)};
        if (lane + o < 32) a.merge(other);
    }
    if (lane == 0) out[q] = a.s + a.c;
}

namespace {
// Device address of g_reduce_scratch, looked up once per device with that
// device current (the host-side symbol is not a device address).
int static_scratch(double **out) {
    static std::mutex mu;
    static double *addr[128] = {};
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return fail("device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        CU(cudaGetSymbolAddress(&p, g_reduce_scratch));
        addr[dev] = (double *)p;
    }
    *out = addr[dev];
    return 0;
}
}  // namespace

extern "C" int lbm_cu_reduce_conserved_noalloc(lbm_lattice *l, int layout, double out[5], void *stream) {
    if (!l || !out) return fail("NULL argument");
    const int64_t max_cells = (int64_t)kStaticPartials * kStaticCellsPerBlock;
    if (l->n > max_cells)
        return fail("lattice has " + std::to_string(l->n) + " cells; the no-allocation reduction handles at most " +
                    std::to_string(max_cells));
    double *partial = nullptr;
    if (static_scratch(&partial)) return -1;
    double *res = partial + (size_t)kStaticPartials * 10;
    const int blocks = (int)std::max<int64_t>(1, (l->n + kStaticCellsPerBlock - 1) / kStaticCellsPerBlock);
    cudaStream_t st = S(stream);
    switch (l->storage) {
        case kF32: k_reduce<float><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kF64: k_reduce<double><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kF16: k_reduce<__half><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kBF16: k_reduce<__nv_bfloat16><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
        case kC16: k_reduce<c16_t><<<blocks, kBlock, 0, st>>>(l->h, layout & 1, partial); break;
    }
    CU(cudaGetLastError());
    k_reduce_final_warps<<<1, 160, 0, st>>>(partial, blocks, res);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(out, res, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return 0;
}

// ================================================================== domain
struct CommGeom {
    int dst;
    int axis;
    int send_origin[3], recv_origin[3], size[3], dir[3];
};

struct lbm_domain {
    int size[3], nums[3], sub[3];
    int storage, store_v, store_rho, lid_geometry;
    bool owns = true;  // false: a view over lattices the caller owns (lbm_cu_domain_wrap)
    std::vector<lbm_lattice *> subs;
    std::vector<std::vector<CommGeom>> comms;
    std::vector<std::vector<int>> bc;
    std::vector<int> coords;  // 3 per subdomain
    std::vector<LatDesc> h_tab;  // descriptors of the subdomains
    int shape = 0;               // requested kernel shape (0: per storage type)
    int eff_shape = 1;           // the shape the subdomains run
    int fma64 = 0;               // double storage: contracted FP64 kernels
    bool tab_dirty = true;
    // halo plans [0 = after beta, 1 = after alpha][axis]
    std::vector<HaloDesc> plan[2][3];
    int64_t plan_cells[2][3] = {};
    int plan_planes[2][3] = {};
    int halo_mode = 0;  // 0: all 19 populations after alpha (reference), 1: the 5 read inward
    bool fuse_x = true;    // let one-cell alpha steps do the x part of the exchange after them
    bool x_fused = false;  // ... and they do, for the current kernel shape (domain_upload_tab)
    int64_t counter = 0;
    int store_interval = 1;  // write u/rho every k-th step; 0 = last step of a run
    cudaGraphExec_t graph = nullptr;
    cudaStream_t cap_stream = nullptr;
    // one captured graph of a whole timed run (lbm_cu_domain_prepare_timed_run):
    // its steps, the counter parity it starts at, and an event pair around
    // every step kernel, read by lbm_cu_domain_kernel_time after it ran
    cudaGraphExec_t tgraph = nullptr;
    int tgraph_steps = 0, tgraph_parity = 0, tgraph_every = 1;
    bool tgraph_ran = false;
    std::vector<cudaEvent_t> tev;
    // step-kernel timing with CUDA events (eager steps only)
    bool profile = false;
    std::vector<cudaEvent_t> ev;  // pairs: start, stop
    size_t ev_used = 0;
    std::vector<int> ev_parity;  // step parity of every recorded pair
    double kernel_ms = 0.0;
    int64_t kernel_launches = 0;
    double kernel_ms_par[2] = {0.0, 0.0};  // the same split into beta (0) and alpha (1) steps
    int64_t kernel_launches_par[2] = {0, 0};
};

namespace {
int domain_build_plans(lbm_domain *D) {
    for (int ph = 0; ph < 2; ph++)
        for (int a = 0; a < 3; a++) {
            auto &v = D->plan[ph][a];
            v.clear();
            int64_t cells = 0;
            int planes = 0;
            for (size_t b = 0; b < D->subs.size(); b++) {
                for (const CommGeom &cm : D->comms[b]) {
                    if (cm.axis != a) continue;
                    // neighbour's comm pointing back at b
                    const CommGeom *back = nullptr;
                    for (const CommGeom &o : D->comms[cm.dst])
                        if (o.dst == (int)b && o.axis == a) back = &o;
                    if (!back) return fail("inconsistent CComm geometry");
                    lbm_lattice *A = D->subs[cm.dst], *B = D->subs[b];
                    HaloDesc h;
                    h.src = A->dd; h.dst = B->dd;
                    h.sps = A->pstride; h.dps = B->pstride;
                    if (ph == 1) {
                        // syncAlpha: neighbour's inner layer -> own ghost layer.  All 19
                        // populations as the reference, or only those the inner
                        // neighbours of the ghost layer gather (direction . e < 0).
                        h.sb = make_box(A, back->send_origin, back->size);
                        h.db = make_box(B, cm.recv_origin, cm.size);
                        h.pl = D->halo_mode ? plane_list(cm.dir, -1) : plane_list(nullptr);
                    } else {
                        // syncBeta: neighbour's ghost layer -> own inner layer, direction . e > 0
                        h.sb = make_box(A, back->recv_origin, back->size);
                        h.db = make_box(B, cm.send_origin, cm.size);
                        h.pl = plane_list(cm.dir);
                    }
                    cells = std::max<int64_t>(cells, h.sb.cells);
                    planes = std::max(planes, h.pl.n);
                    v.push_back(h);
                }
            }
            D->plan_cells[ph][a] = cells;
            D->plan_planes[ph][a] = planes;
        }
    return 0;
}

int domain_geometry(lbm_domain *D);

void drop_graph(lbm_domain *D);

// The x part of the exchange after alpha steps, moved into the one-cell
// alpha kernel: each sender's descriptor gets its x neighbours' population
// planes and the planes to copy (those of the x plan after alpha).
void domain_fuse_x(lbm_domain *D, std::vector<LatDesc> &t, int eff_shape) {
    const bool fuse = D->fuse_x && eff_shape == 1 && !D->plan[1][0].empty();
    for (auto &d : t) {
        d.xhi = d.xlo = nullptr;
        d.xmask_hi = d.xmask_lo = 0;
        d.xdiv_m = d.xdiv_s1 = d.xdiv_s2 = 0;
    }
    if (!fuse) return;
    for (const HaloDesc &h : D->plan[1][0]) {
        size_t a = 0;
        while (a < D->subs.size() && D->subs[a]->dd != h.src) a++;
        if (a == D->subs.size()) continue;
        LatDesc &d = t[a];
        uint32_t mask = 0;
        for (int k = 0; k < h.pl.n; k++) mask |= 1u << h.pl.f[k];
        if (h.db.ox == 0) {  // the receiver's ghost layer x = 0: the +x neighbour, sent from x = nx - 2
            d.xhi = h.dst;
            d.xmask_hi = mask;
        } else {  // x = nx - 1 of the -x neighbour, sent from x = 1
            d.xlo = h.dst;
            d.xmask_lo = mask;
        }
        const FastDiv fd = FastDiv::make((uint32_t)d.nx);
        d.xdiv_m = fd.m;
        d.xdiv_s1 = fd.s1;
        d.xdiv_s2 = fd.s2;
    }
}

int domain_upload_tab(lbm_domain *D, cudaStream_t st) {
    (void)st;
    if (!D->tab_dirty && D->owns) return 0;
    // a view's lattices may have changed parameters through their own handles:
    // compare, and drop a graph captured with the old descriptors
    std::vector<LatDesc> t;
    for (auto *l : D->subs) t.push_back(l->h);
    const int eff = D->fma64 && D->storage == kF64 ? kShapeF64Fma
                                                   : effective_shape(D->storage, D->shape, t.data(), (int)t.size());
    domain_fuse_x(D, t, eff);
    if (!D->tab_dirty && t.size() == D->h_tab.size() &&
        memcmp(t.data(), D->h_tab.data(), t.size() * sizeof(LatDesc)) == 0)
        return 0;
    drop_graph(D);
    D->h_tab.swap(t);
    D->eff_shape = eff;
    D->x_fused = D->fuse_x && eff == 1 && !D->plan[1][0].empty();
    D->tab_dirty = false;
    return 0;
}

int domain_record(lbm_domain *D, cudaStream_t st, cudaEvent_t *out) {
    if (D->ev_used == D->ev.size()) {
        cudaEvent_t e;
        CU(cudaEventCreate(&e));
        D->ev.push_back(e);
    }
    *out = D->ev[D->ev_used++];
    CU(cudaEventRecord(*out, st));
    return 0;
}

int domain_one_step(lbm_domain *D, int parity, cudaStream_t st, bool store, bool timed) {
    const bool les = uses_les(D->subs[0]->h);
    const int sv = store ? D->store_v : 0, sr = store ? D->store_rho : 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timed && domain_record(D, st, &e0)) return -1;
    if (launch_step(D->storage, D->eff_shape, parity, les, D->h_tab.data(), (int)D->subs.size(), sv, sr, st))
        return -1;
    if (timed && domain_record(D, st, &e1)) return -1;
    if (timed) {
        D->ev_parity.resize(D->ev_used / 2);
        D->ev_parity.back() = parity;
    }
    for (int a = 0; a < 3; a++)
        if (!D->plan[parity][a].empty() && !(parity == 1 && a == 0 && D->x_fused) &&
            launch_halo_batch(D->storage, D->plan[parity][a].data(), (int)D->plan[parity][a].size(), D->plan_cells[parity][a],
                              D->plan_planes[parity][a], st))
            return -1;
    return 0;
}

void drop_graph(lbm_domain *D) {
    if (D->graph) cudaGraphExecDestroy(D->graph);
    D->graph = nullptr;
    if (D->tgraph) cudaGraphExecDestroy(D->tgraph);
    D->tgraph = nullptr;
    D->tgraph_ran = false;
}
}  // namespace

extern "C" {

int lbm_cu_domain_create(const int size[3], const int nums[3], int storage, int store_velocity, int store_density,
                         int lid_geometry, lbm_domain **out) {
    if (!size || !nums || !out) return fail("NULL argument");
    *out = nullptr;
    for (int a = 0; a < 3; a++) {
        if (nums[a] < 1 || size[a] < 1) return fail("sizes and subdomain counts must be positive");
        if (size[a] % nums[a] != 0) return fail("Number of subdomains does not match with the grid size!");
    }
    lbm_domain *D = new lbm_domain();
    for (int a = 0; a < 3; a++) {
        D->size[a] = size[a];
        D->nums[a] = nums[a];
        D->sub[a] = size[a] / nums[a];
    }
    D->storage = storage;
    D->store_v = store_velocity ? 1 : 0;
    D->store_rho = store_density ? 1 : 0;
    D->lid_geometry = lid_geometry;
    const int nsub = nums[0] * nums[1] * nums[2];
    for (int id = 0; id < nsub; id++) {
        lbm_lattice *l = nullptr;
        if (lbm_cu_create(D->sub[0], D->sub[1], D->sub[2], storage, store_velocity, store_density, &l)) {
            std::string m = g_err;
            lbm_cu_domain_destroy(D);
            return fail(m);
        }
        D->subs.push_back(l);
    }
    if (domain_geometry(D)) {
        std::string m = g_err;
        lbm_cu_domain_destroy(D);
        return fail(m);
    }
    *out = D;
    return 0;
}

int lbm_cu_domain_wrap(lbm_lattice *const *subdomains, const int size[3], const int nums[3], int lid_geometry,
                       lbm_domain **out) {
    if (!subdomains || !size || !nums || !out) return fail("NULL argument");
    *out = nullptr;
    for (int a = 0; a < 3; a++) {
        if (nums[a] < 1 || size[a] < 1) return fail("sizes and subdomain counts must be positive");
        if (size[a] % nums[a] != 0) return fail("Number of subdomains does not match with the grid size!");
    }
    const int nsub = nums[0] * nums[1] * nums[2];
    const lbm_lattice *l0 = subdomains[0];
    for (int id = 0; id < nsub; id++) {
        const lbm_lattice *l = subdomains[id];
        if (!l) return fail("NULL subdomain lattice");
        if (l->nx != size[0] / nums[0] || l->ny != size[1] / nums[1] || l->nz != size[2] / nums[2])
            return fail("a subdomain lattice does not have the subdomain size");
        if (l->storage != l0->storage || l->store_v != l0->store_v || l->store_rho != l0->store_rho)
            return fail("subdomain lattices differ in storage type or stored fields");
    }
    lbm_domain *D = new lbm_domain();
    D->owns = false;
    for (int a = 0; a < 3; a++) {
        D->size[a] = size[a];
        D->nums[a] = nums[a];
        D->sub[a] = size[a] / nums[a];
    }
    D->storage = l0->storage;
    D->store_v = l0->store_v;
    D->store_rho = l0->store_rho;
    D->lid_geometry = lid_geometry;
    D->subs.assign(subdomains, subdomains + nsub);
    if (domain_geometry(D)) {
        std::string m = g_err;
        lbm_cu_domain_destroy(D);
        return fail(m);
    }
    *out = D;
    return 0;
}

int lbm_cu_domain_set_counter(lbm_domain *D, int64_t counter) {
    if (!D) return fail("NULL domain");
    if (counter < 0) return fail("negative step counter");
    D->counter = counter;
    return 0;
}

}  // extern "C"

namespace {
// Faces of every subdomain (walls outside, ghost layers inside), its CComm
// list in the reference's order and the halo plans (src/CManager.hpp:78-204).
int domain_geometry(lbm_domain *D) {
    const int *nums = D->nums;
    const int nsub = nums[0] * nums[1] * nums[2];
    const int stride[3] = {1, nums[0], nums[0] * nums[1]};
    for (int id = 0; id < nsub; id++) {
        const int c[3] = {id % nums[0], (id / nums[0]) % nums[1], id / (nums[0] * nums[1])};
        D->coords.insert(D->coords.end(), c, c + 3);
        std::vector<int> bc(6, LBM_FLAG_GHOST_LAYER);
        for (int a = 0; a < 3; a++) {
            if (c[a] == 0) bc[2 * a] = LBM_FLAG_OBSTACLE;
            if (c[a] == nums[a] - 1) bc[2 * a + 1] = LBM_FLAG_OBSTACLE;
        }
        std::vector<CommGeom> cms;
        for (int a = 0; a < 3; a++)
            for (int up = 0; up < 2; up++) {
                if (bc[2 * a + up] != LBM_FLAG_GHOST_LAYER) continue;
                CommGeom g{};
                g.dst = id + (up ? stride[a] : -stride[a]);
                g.axis = a;
                for (int q = 0; q < 3; q++) {
                    g.size[q] = q == a ? 1 : D->sub[q];
                    g.send_origin[q] = g.recv_origin[q] = g.dir[q] = 0;
                }
                g.send_origin[a] = up ? D->sub[a] - 2 : 1;
                g.recv_origin[a] = up ? D->sub[a] - 1 : 0;
                g.dir[a] = up ? -1 : 1;
                cms.push_back(g);
            }
        D->bc.push_back(bc);
        D->comms.push_back(cms);
    }
    return domain_build_plans(D);
}
}  // namespace

extern "C" {

int lbm_cu_domain_destroy(lbm_domain *D) {
    if (!D) return 0;
    drop_graph(D);
    if (D->cap_stream) cudaStreamDestroy(D->cap_stream);
    for (cudaEvent_t e : D->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : D->tev) cudaEventDestroy(e);
    if (D->owns)
        for (auto *l : D->subs) lbm_cu_destroy(l);
    delete D;
    return 0;
}

int lbm_cu_domain_set_params(lbm_domain *D, const lbm_params *p) {
    if (!D || !p) return fail("NULL argument");
    for (auto *l : D->subs)
        if (lbm_cu_set_params(l, p)) return -1;
    D->tab_dirty = true;
    drop_graph(D);
    return 0;
}

int lbm_cu_domain_reset(lbm_domain *D, void *stream) {
    if (!D) return fail("NULL domain");
    for (size_t i = 0; i < D->subs.size(); i++) {
        lbm_lattice *l = D->subs[i];
        if (lbm_cu_init(l, D->bc[i].data(), stream)) return -1;
        if (D->lid_geometry && D->coords[3 * i + 1] == D->nums[1] - 1) {
            // CController::setGeometry: lid plane y = Y-2, x in [1,X-2], z in [1,Z-2]
            const int o[3] = {1, l->ny - 2, 1};
            const int s[3] = {l->nx - 2, 1, l->nz - 2};
            std::vector<int32_t> v((size_t)s[0] * s[1] * s[2], LBM_FLAG_VELOCITY_INJECTION);
            if (lbm_cu_write(l, LBM_FIELD_FLAGS, o, s, v.data(), nullptr, stream)) return -1;
        }
    }
    D->counter = 0;
    return 0;
}

int lbm_cu_domain_perturb(lbm_domain *D, uint64_t seed, double amp, void *stream) {
    if (!D) return fail("NULL domain");
    int ph[3];
    for (int a = 0; a < 3; a++) ph[a] = D->nums[a] * (D->sub[a] - 2) + 2;
    for (size_t i = 0; i < D->subs.size(); i++) {
        int o[3];
        for (int a = 0; a < 3; a++) o[a] = D->coords[3 * i + a] * (D->sub[a] - 2);
        if (lbm_cu_perturb(D->subs[i], o, ph, seed, amp, stream)) return -1;
    }
    return 0;
}

// Steps of a timed run whose step kernel an event pair brackets: the pair of
// steps (a beta and an alpha step) at the start of every `every` steps.
static bool timed_step(int k, int every) { return k % every < 2; }

int lbm_cu_domain_prepare_timed_run(lbm_domain *D, int steps, int every, void *stream) {
    if (!D) return fail("NULL domain");
    if (steps < 1) return fail("a timed run has at least one step");
    if (every < 1) return fail("the sampling interval of a timed run is at least 1");
    if (D->store_interval != 0 && (D->store_v || D->store_rho))
        return fail("a timed run writes velocity and density on its last step only (store interval 0)");
    if (domain_upload_tab(D, S(stream))) return -1;
    if (D->tgraph) cudaGraphExecDestroy(D->tgraph);
    D->tgraph = nullptr;
    D->tgraph_ran = false;
    while (D->tev.size() < 2 * (size_t)steps) {
        cudaEvent_t e;
        CU(cudaEventCreate(&e));
        D->tev.push_back(e);
    }
    if (!D->cap_stream) CU(cudaStreamCreateWithFlags(&D->cap_stream, cudaStreamNonBlocking));
    const bool les = uses_les(D->subs[0]->h);
    cudaGraph_t g = nullptr;
    CU(cudaStreamBeginCapture(D->cap_stream, cudaStreamCaptureModeThreadLocal));
    bool ok = true;
    for (int k = 0; k < steps && ok; k++) {
        const int parity = (int)((D->counter + k) & 1);
        const bool store = k + 1 == steps;
        const int sv = store ? D->store_v : 0, sr = store ? D->store_rho : 0;
        const bool timed = timed_step(k, every);
        if (timed) ok = cudaEventRecordWithFlags(D->tev[2 * k], D->cap_stream, cudaEventRecordExternal) == cudaSuccess;
        ok = ok && !launch_step(D->storage, D->eff_shape, parity, les, D->h_tab.data(), (int)D->subs.size(), sv, sr,
                                D->cap_stream);
        if (timed)
            ok = ok && cudaEventRecordWithFlags(D->tev[2 * k + 1], D->cap_stream, cudaEventRecordExternal) == cudaSuccess;
        for (int a = 0; a < 3 && ok; a++)
            if (!D->plan[parity][a].empty() && !(parity == 1 && a == 0 && D->x_fused))
                ok = !launch_halo_batch(D->storage, D->plan[parity][a].data(), (int)D->plan[parity][a].size(),
                                        D->plan_cells[parity][a], D->plan_planes[parity][a], D->cap_stream);
    }
    const cudaError_t e = cudaStreamEndCapture(D->cap_stream, &g);
    if (!ok || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(std::string("capturing the timed run: ") + (e != cudaSuccess ? cudaGetErrorString(e) : g_err));
    }
    const cudaError_t ei = cudaGraphInstantiate(&D->tgraph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        D->tgraph = nullptr;
        return fail(std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    D->tgraph_steps = steps;
    D->tgraph_every = every;
    D->tgraph_parity = (int)(D->counter & 1);
    return 0;
}

int lbm_cu_domain_run(lbm_domain *D, int steps, int use_graph, void *stream) {
    if (!D) return fail("NULL domain");
    if (steps < 0) return fail("negative step count");
    cudaStream_t st = S(stream);
    if (domain_upload_tab(D, st)) return -1;  // may drop a timed graph captured with other descriptors
    if (D->tgraph && use_graph && D->profile && steps == D->tgraph_steps && (int)(D->counter & 1) == D->tgraph_parity) {
        CU(cudaGraphLaunch(D->tgraph, st));
        D->counter += steps;
        D->tgraph_ran = true;
        return 0;
    }
    int done = 0;
    // u/rho are written on steps whose new counter is a multiple of the
    // interval, or (interval 0) on the last step of this call
    auto stores_on = [&](int64_t next_counter, bool last) {
        return D->store_interval == 0 ? last : (next_counter % D->store_interval) == 0;
    };
    auto single = [&]() -> int {
        const bool last = done + 1 == steps;
        if (domain_one_step(D, (int)(D->counter & 1), st, stores_on(D->counter + 1, last), D->profile)) return -1;
        D->counter++;
        done++;
        return 0;
    };
    if ((D->counter & 1) && done < steps)
        if (single()) return -1;
    // graph replay only where no pair needs a store or a timing record
    const bool plain_pairs = (D->store_interval == 0) || (!D->store_v && !D->store_rho);
    int pairs = (steps - done) / 2;
    if (D->store_interval == 0 && (steps - done) % 2 == 0 && pairs > 0) pairs--;  // last pair stores
    if (pairs > 0 && use_graph && plain_pairs && !D->profile) {
        if (!D->graph) {
            if (!D->cap_stream) CU(cudaStreamCreateWithFlags(&D->cap_stream, cudaStreamNonBlocking));
            cudaGraph_t g = nullptr;
            CU(cudaStreamBeginCapture(D->cap_stream, cudaStreamCaptureModeThreadLocal));
            int rc = domain_one_step(D, 0, D->cap_stream, false, false);
            if (!rc) rc = domain_one_step(D, 1, D->cap_stream, false, false);
            cudaError_t e = cudaStreamEndCapture(D->cap_stream, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return -1;
            }
            if (e != cudaSuccess) return fail(std::string("graph capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&D->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                D->graph = nullptr;
                return fail(std::string("graph instantiate: ") + cudaGetErrorString(e));
            }
        }
        for (int p = 0; p < pairs; p++) CU(cudaGraphLaunch(D->graph, st));
        D->counter += 2 * pairs;
        done += 2 * pairs;
    }
    while (done < steps)
        if (single()) return -1;
    return 0;
}

int lbm_cu_domain_set_store_interval(lbm_domain *D, int interval) {
    if (!D) return fail("NULL domain");
    if (interval < 0) return fail("negative store interval");
    D->store_interval = interval;
    return 0;
}

int lbm_cu_set_kernel_shape(lbm_lattice *l, int cells_per_thread) {
    if (!l) return fail("NULL lattice");
    if (cells_per_thread < 0 || cells_per_thread > 3) return fail("kernel shape is 0 (automatic), 1, 2 or 3");
    l->shape = cells_per_thread;
    return 0;
}

int lbm_cu_domain_set_kernel_shape(lbm_domain *D, int cells_per_thread) {
    if (!D) return fail("NULL domain");
    if (cells_per_thread < 0 || cells_per_thread > 3) return fail("kernel shape is 0 (automatic), 1, 2 or 3");
    D->shape = cells_per_thread;
    D->tab_dirty = true;
    drop_graph(D);
    return 0;
}

int lbm_cu_set_fp64_contraction(lbm_lattice *l, int enable) {
    if (!l) return fail("NULL lattice");
    if (l->storage != kF64) return fail("contracted kernels exist for double storage only");
    l->fma64 = enable ? 1 : 0;
    return 0;
}

int lbm_cu_domain_set_fp64_contraction(lbm_domain *D, int enable) {
    if (!D) return fail("NULL domain");
    if (D->storage != kF64) return fail("contracted kernels exist for double storage only");
    D->fma64 = enable ? 1 : 0;
    D->tab_dirty = true;
    drop_graph(D);
    return 0;
}

int lbm_cu_domain_set_halo_mode(lbm_domain *D, int mode) {
    if (!D) return fail("NULL domain");
    if (mode != 0 && mode != 1) return fail("halo mode is 0 (all populations) or 1 (inward populations)");
    if (mode == D->halo_mode) return 0;
    D->halo_mode = mode;
    drop_graph(D);
    D->tab_dirty = true;  // the fused x copies take their planes from the plans
    return domain_build_plans(D);
}

int lbm_cu_domain_set_fused_exchange(lbm_domain *D, int enable) {
    if (!D) return fail("NULL domain");
    D->fuse_x = enable != 0;
    D->tab_dirty = true;
    drop_graph(D);
    return 0;
}

int lbm_cu_domain_profile(lbm_domain *D, int enable) {
    if (!D) return fail("NULL domain");
    D->profile = enable != 0;
    return 0;
}

// Fold the recorded event pairs into the accumulated step-kernel times.
static int domain_collect_times(lbm_domain *D) {
    auto add = [&](float ms, int parity) {
        D->kernel_ms += ms;
        D->kernel_launches++;
        D->kernel_ms_par[parity & 1] += ms;
        D->kernel_launches_par[parity & 1]++;
    };
    if (D->tgraph_ran) {
        for (int k = 0; k < D->tgraph_steps; k++) {
            if (!timed_step(k, D->tgraph_every)) continue;
            CU(cudaEventSynchronize(D->tev[2 * k + 1]));
            float ms = 0.f;
            CU(cudaEventElapsedTime(&ms, D->tev[2 * k], D->tev[2 * k + 1]));
            add(ms, D->tgraph_parity + k);
        }
        D->tgraph_ran = false;
    }
    for (size_t i = 0; i + 1 < D->ev_used; i += 2) {
        CU(cudaEventSynchronize(D->ev[i + 1]));
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, D->ev[i], D->ev[i + 1]));
        add(ms, D->ev_parity[i / 2]);
    }
    D->ev_used = 0;
    D->ev_parity.clear();
    return 0;
}

static void domain_reset_times(lbm_domain *D) {
    D->kernel_ms = 0.0;
    D->kernel_launches = 0;
    D->kernel_ms_par[0] = D->kernel_ms_par[1] = 0.0;
    D->kernel_launches_par[0] = D->kernel_launches_par[1] = 0;
}

int lbm_cu_domain_kernel_time(lbm_domain *D, double *ms_total, int64_t *launches, int reset) {
    if (!D) return fail("NULL domain");
    if (domain_collect_times(D)) return -1;
    if (ms_total) *ms_total = D->kernel_ms;
    if (launches) *launches = D->kernel_launches;
    if (reset) domain_reset_times(D);
    return 0;
}

int lbm_cu_domain_kernel_time_by_step(lbm_domain *D, double ms[2], int64_t launches[2], int reset) {
    if (!D || !ms || !launches) return fail("NULL argument");
    if (domain_collect_times(D)) return -1;
    for (int p = 0; p < 2; p++) {
        ms[p] = D->kernel_ms_par[p];
        launches[p] = D->kernel_launches_par[p];
    }
    if (reset) domain_reset_times(D);
    return 0;
}

int lbm_cu_domain_counter(const lbm_domain *D, int64_t *counter) {
    if (!D || !counter) return fail("NULL argument");
    *counter = D->counter;
    return 0;
}

int lbm_cu_domain_subdomains(const lbm_domain *D, int *count, int sub_size[3]) {
    if (!D) return fail("NULL domain");
    if (count) *count = (int)D->subs.size();
    if (sub_size)
        for (int a = 0; a < 3; a++) sub_size[a] = D->sub[a];
    return 0;
}

// Domain checkpoint: a header with the decomposition and the step counter,
// then every subdomain's lattice block (lbm_io.cu).
namespace {
struct DomHeader {
    char magic[8];
    int32_t storage;
    int32_t size[3], nums[3];
    int32_t reserved;
    int64_t counter;
};
static_assert(sizeof(DomHeader) == 48, "domain checkpoint header layout");
constexpr char kDomMagic[8] = {'L', 'B', 'M', 'D', 'C', 'K', 'P', '1'};
struct FileCloser {
    FILE *f;
    ~FileCloser() {
        if (f) fclose(f);
    }
};
}  // namespace

int lbm_cu_domain_checkpoint_save(lbm_domain *D, const char *path, void *stream) {
    if (!D || !path) return fail("NULL argument");
    CU(cudaStreamSynchronize(S(stream)));
    FileCloser fc{fopen(path, "wb")};
    if (!fc.f) return fail(std::string("cannot open ") + path + " for writing");
    DomHeader hd{};
    memcpy(hd.magic, kDomMagic, 8);
    hd.storage = D->storage;
    for (int a = 0; a < 3; a++) {
        hd.size[a] = D->size[a];
        hd.nums[a] = D->nums[a];
    }
    hd.counter = D->counter;
    if (fwrite(&hd, sizeof(hd), 1, fc.f) != 1) return fail("checkpoint write failed");
    for (auto *l : D->subs)
        if (ckpt_write_lattice(fc.f, l, D->counter)) return -1;
    if (fflush(fc.f)) return fail("checkpoint write failed");
    return 0;
}

int lbm_cu_domain_checkpoint_load(lbm_domain *D, const char *path, void *stream) {
    if (!D || !path) return fail("NULL argument");
    CU(cudaStreamSynchronize(S(stream)));
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) return fail(std::string("cannot open ") + path);
    DomHeader hd{};
    if (fread(&hd, sizeof(hd), 1, fc.f) != 1) return fail("checkpoint file is truncated");
    if (memcmp(hd.magic, kDomMagic, 8)) return fail("not a domain checkpoint (bad magic)");
    if (hd.storage != D->storage) return fail("checkpoint storage type does not match");
    for (int a = 0; a < 3; a++)
        if (hd.size[a] != D->size[a] || hd.nums[a] != D->nums[a])
            return fail("checkpoint decomposition does not match");
    for (auto *l : D->subs) {
        int64_t c = 0;
        if (ckpt_read_lattice(fc.f, l, &c)) return -1;
        if (c != hd.counter) return fail("checkpoint subdomain counters disagree");
    }
    D->counter = hd.counter;
    return 0;
}

lbm_lattice *lbm_cu_domain_lattice(lbm_domain *D, int index) {
    if (!D || index < 0 || index >= (int)D->subs.size()) {
        fail("subdomain index out of range");
        return nullptr;
    }
    return D->subs[index];
}

}  // extern "C"
