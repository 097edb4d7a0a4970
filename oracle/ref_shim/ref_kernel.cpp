// ref_kernel.cpp -- one translation unit per reference kernel file.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle).  Compiled by
// oracle/build_ref.py with
//   -DREF_PREFIX="<generated prefix>"   sizes, T, flags, work-group size
//   -DREF_SOURCE="<reference .cl path>"  the kernel source, in place
//   -DREF_KIND=1..4                      init, alpha, beta, copy_buffer_rect
// Each .cl file gets its own translation unit because the kernels leave
// function-scope macros defined (e.g. `#define dd_param rho`,
// src/cl_programs/lbm_beta.cl:493) that would break the next file.
//
// The extern "C" launchers below play the role of the host's
// enqueueNDRangeKernel calls (src/CLbmSolver.hpp:619-659,172-209): a 1-D
// range of DOMAIN_CELLS work-items in groups of LOCAL_WORK_GROUP_SIZE, or
// the 2-D (block_y, block_z) range of copy_buffer_rect.
#include "ocl_shim.hpp"
#include REF_PREFIX

#include <vector>

#define KIND_INIT 1
#define KIND_ALPHA 2
#define KIND_BETA 3
#define KIND_COPY 4

namespace refk {
#if REF_KIND == KIND_BETA
// The beta kernel's __local work-group buffer (lbm_beta.cl:167) must be one
// array shared by the work-items of a group.  The name is redirected to a
// per-OS-thread buffer; each OS thread runs one work-group at a time.
static thread_local T oclshim_buf[12][LOCAL_WORK_GROUP_SIZE];
T (*oclshim_wg_buf())[12][LOCAL_WORK_GROUP_SIZE] { return &oclshim_buf; }
#define dd_buf (*oclshim_wg_buf())
#endif
#include REF_SOURCE
}  // namespace refk

static const long kCells = (long)DOMAIN_CELLS_X * DOMAIN_CELLS_Y * DOMAIN_CELLS_Z;

#if REF_KIND == KIND_INIT
extern "C" void ref_init(T *dd, int *flags, T *vel, T *dens, int *bc, T lid) {
#pragma omp parallel for schedule(static)
    for (long g = 0; g < kCells; g++) {
        oclshim::g_item = {{(size_t)g, 0}, (size_t)(g % LOCAL_WORK_GROUP_SIZE)};
        refk::init_kernel(dd, flags, vel, dens, bc, lid);
    }
}
#endif

#if REF_KIND == KIND_ALPHA
extern "C" void ref_alpha(T *dd, const int *flags, T *vel, T *dens, T inv_tau, T gx, T gy, T gz,
                          T lid) {
#pragma omp parallel for schedule(static)
    for (long g = 0; g < kCells; g++) {
        oclshim::g_item = {{(size_t)g, 0}, (size_t)(g % LOCAL_WORK_GROUP_SIZE)};
        refk::lbm_kernel_alpha(dd, flags, vel, dens, inv_tau, gx, gy, gz, lid);
    }
}
#endif

#if REF_KIND == KIND_BETA
namespace {
struct Launch {
    T *dd;
    const int *flags;
    T *vel, *dens;
    T inv_tau, gx, gy, gz, lid;
};
struct Fiber {
    ucontext_t ctx;
    size_t gid, lid;
    bool done;
};
thread_local const Launch *t_launch = nullptr;
thread_local Fiber *t_fiber = nullptr;

void fiber_main() {
    const Launch *a = t_launch;
    refk::lbm_kernel_beta(a->dd, a->flags, a->vel, a->dens, a->inv_tau, a->gx, a->gy, a->gz,
                          a->lid);
    t_fiber->done = true;  // returning resumes uc_link, the scheduler
}
}  // namespace

extern "C" int ref_beta(T *dd, const int *flags, T *vel, T *dens, T inv_tau, T gx, T gy, T gz,
                        T lid) {
    const long wg = LOCAL_WORK_GROUP_SIZE;
    if (kCells % wg != 0) return -1;  // partial groups are undefined in the reference
    const long groups = kCells / wg;
    const Launch launch{dd, flags, vel, dens, inv_tau, gx, gy, gz, lid};
    const size_t stack_bytes = 1 << 16;
#pragma omp parallel
    {
        std::vector<Fiber> fibers(wg);
        std::vector<char> stacks((size_t)wg * stack_bytes);
        t_launch = &launch;
#pragma omp for schedule(static)
        for (long grp = 0; grp < groups; grp++) {
            for (long l = 0; l < wg; l++) {
                Fiber &f = fibers[l];
                f.gid = (size_t)(grp * wg + l);
                f.lid = (size_t)l;
                f.done = false;
                getcontext(&f.ctx);
                f.ctx.uc_stack.ss_sp = &stacks[(size_t)l * stack_bytes];
                f.ctx.uc_stack.ss_size = stack_bytes;
                f.ctx.uc_link = &oclshim::g_sched;
                makecontext(&f.ctx, fiber_main, 0);
            }
            long alive = wg;
            while (alive > 0) {
                for (long l = 0; l < wg; l++) {
                    Fiber &f = fibers[l];
                    if (f.done) continue;
                    t_fiber = &f;
                    oclshim::g_cur = &f.ctx;
                    oclshim::g_item = {{f.gid, 0}, f.lid};
                    swapcontext(&oclshim::g_sched, &f.ctx);
                    if (f.done) alive--;
                }
            }
        }
    }
    return 0;
}
#endif

#if REF_KIND == KIND_COPY
extern "C" void ref_copy_rect(T *src, int src_offset, int sox, int soy, int soz, int ssx, int ssy,
                              int ssz, T *dst, int dst_offset, int dox, int doy, int doz, int dsx,
                              int dsy, int dsz, int bx, int by, int bz) {
    for (int k = 0; k < bz; k++)
        for (int j = 0; j < by; j++) {
            oclshim::g_item = {{(size_t)j, (size_t)k}, 0};
            refk::copy_buffer_rect(src, src_offset, sox, soy, soz, ssx, ssy, ssz, dst, dst_offset,
                                   dox, doy, doz, dsx, dsy, dsz, bx);
        }
}
#endif
