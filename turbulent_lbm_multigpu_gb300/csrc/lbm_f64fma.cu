// lbm_f64fma.cu -- the one-cell step kernels for double populations with
// fused multiply-adds.
//
// This translation unit is compiled with -fmad=true (every other one with
// -fmad=false), so the compiler may contract each product that feeds a sum
// into one FP64 fused multiply-add.  The arithmetic is otherwise the same
// expressions in the same order as the bit-exact kernels; every contraction
// rounds once instead of twice, so a step differs from the reference
// arithmetic by a few units in the last place (a relative 1e-15, well inside
// the 1e-12 per-step bound for double), while the FP64 pipe -- which bounds
// the double kernels on GB300, not HBM -- issues fewer operations.
//
// The kernels are instantiated for a storage tag type of their own (F64Fma:
// one double), so that their template instances can never be confused with
// the bit-exact k_beta<double> / k_alpha<double> of the other units.
#include "lbm_internal.h"

namespace lbm {
struct F64Fma {
    double v;
};
static_assert(sizeof(F64Fma) == sizeof(double), "same layout as double populations");

template <> struct Store<F64Fma> {
    using R = double;
    static constexpr bool kDev = false;
    __device__ static __forceinline__ R ld(const F64Fma *p, R) { return p->v; }
    __device__ static __forceinline__ void st(F64Fma *p, R v, R) { p->v = v; }
};
}  // namespace lbm

namespace lbm_rt {
int launch_step_f64_fma(int parity, bool les, const DomainArgs &a, int blocks, cudaStream_t st) {
    if (blocks <= 0) return 0;
    if (parity) {
        if (les) k_alpha<F64Fma, true><<<blocks, kBlock, 0, st>>>(a);
        else k_alpha<F64Fma, false><<<blocks, kBlock, 0, st>>>(a);
    } else {
        if (les) k_beta<F64Fma, true><<<blocks, kBlock, 0, st>>>(a);
        else k_beta<F64Fma, false><<<blocks, kBlock, 0, st>>>(a);
    }
    CU(cudaGetLastError());
    return 0;
}
}  // namespace lbm_rt
