// lbm_internal.h -- host runtime shared by the translation units of
// liblbm_gb300.so (not part of the public C ABI).
#pragma once
#include <cstdio>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "lbm_gb300.h"
#include "lbm_kernels.cuh"

namespace lbm_rt {
using namespace lbm;

// Records the message returned by lbm_cu_last_error() on this thread; -1.
int fail(const std::string &m);

#define CU(call)                                                                                \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) return ::lbm_rt::fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

constexpr int kBlock = 256;

inline size_t storage_bytes(int st) { return st == kF64 ? 8 : st == kF32 ? 4 : 2; }
inline size_t real_bytes(int st) { return st == kF64 ? 8 : 4; }
inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }
inline int grid_for(int64_t work) { return (int)((work + kBlock - 1) / kBlock); }

// Kernel arguments of a lattice, rounded to its arithmetic type.
void set_params_desc(LatDesc &h, int storage, const lbm_params &p);
inline bool uses_les(const LatDesc &h) { return h.pd[P_LES] != 0.0; }

// The two-cell kernels apply when every lattice has an even x extent and a
// float arithmetic type.
bool pair_shape(int storage, const LatDesc *tab, int ntab);
inline int cells_per_block(bool pair) { return pair ? kPairCells : kBlock; }

// Kernel shapes of a step: 1 one cell per thread, 2 two cells per thread,
// 3 tiles staged through shared memory by bulk copies, 0 automatic (3 for
// the 16-bit storage types, 1 otherwise: the fastest measured on GB300).
// The shape a set of lattices runs: 2 needs float arithmetic and even nx,
// 3 float/half/bfloat16 storage; otherwise 1.
int effective_shape(int storage, int shape, const LatDesc *tab, int ntab);

// Internal kernel shape of double lattices that run the contracted FP64
// kernels (lbm_cu_set_fp64_contraction): one cell per thread, fused
// multiply-adds (lbm_f64fma.cu).
constexpr int kShapeF64Fma = 4;
// One step of up to kParamLattices double lattices with the contracted
// kernels (lbm_f64fma.cu); blocks of kBlock cells.
int launch_step_f64_fma(int parity, bool les, const DomainArgs &a, int blocks, cudaStream_t st);

// One step over `ntab` lattices of one storage type, kParamLattices
// descriptors per launch.
int launch_step(int storage, int shape, int parity, bool les, const LatDesc *htab, int ntab, int sv, int sr,
                cudaStream_t st);
// Cells per staged tile of a storage type (0: not staged).
int staged_cells(int storage);
// One step of up to kBatchLattices lattices, all at an alpha step or all at
// a beta step, through the staged tiles (first_block / nblocks of the
// descriptors count tiles of staged_cells; a beta step needs every nx a
// multiple of 16 bytes of populations).
int launch_staged_batch(int storage, bool beta, bool les, const BatchArgs &a, int tiles, cudaStream_t st);
// One lattice block of a checkpoint file (lbm_io.cu).
int ckpt_write_lattice(FILE *f, lbm_lattice *l, int64_t counter);
int ckpt_read_lattice(FILE *f, lbm_lattice *l, int64_t *counter);
}  // namespace lbm_rt

struct lbm_lattice {
    int nx, ny, nz;
    int64_t n, pstride;
    int storage;
    int store_v, store_rho;
    void *dd = nullptr;
    uint8_t *flags = nullptr;
    void *vel = nullptr;
    void *rho = nullptr;
    lbm::LatDesc h{};
    lbm::LatDesc *d_desc = nullptr;
    bool dirty = true;
    void *stage = nullptr;  // staging for host copies and reduction partials
    size_t stage_bytes = 0;
    int shape = 0;  // requested kernel shape (0: per storage type, see effective_shape)
    int fma64 = 0;  // double storage: contracted FP64 kernels (lbm_cu_set_fp64_contraction)
};
