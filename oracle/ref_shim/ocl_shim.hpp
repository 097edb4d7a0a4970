// ocl_shim.hpp -- lets the reference OpenCL C 1.0 kernels compile as C++.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle).  The reference kernel
// sources are never copied: oracle/build_ref.py compiles them where they lie
// in the reference tree, with this header and a generated definition prefix
// (the one the reference host writes at src/CLbmSolver.hpp:319-373).
//
// What the shim supplies:
//  * the address-space keywords (__kernel, __global, __local) as nothing;
//    `__const` is GCC's own spelling of const;
//  * get_global_id / get_local_id from the current work-item;
//  * barrier(): every work-item of a work-group runs as a ucontext fiber, and
//    barrier() switches back to the work-group scheduler, which resumes the
//    fibers round-robin.  One scheduler pass advances every live work-item
//    to its next barrier, which is exactly the OpenCL barrier guarantee;
//  * the OpenCL vector types the kernels name (float2..16, double2..16).
#pragma once
#include <cstddef>
#include <cstdint>
#include <ucontext.h>

namespace oclshim {
struct WorkItem {
    size_t gid[2];
    size_t lid;
};
inline thread_local WorkItem g_item{{0, 0}, 0};
inline thread_local ucontext_t g_sched;
inline thread_local ucontext_t *g_cur = nullptr;
inline void barrier_yield() { swapcontext(g_cur, &g_sched); }
}  // namespace oclshim

inline size_t get_global_id(int d) { return oclshim::g_item.gid[d]; }
inline size_t get_local_id(int) { return oclshim::g_item.lid; }
#define CLK_LOCAL_MEM_FENCE 1
inline void barrier(int) { oclshim::barrier_yield(); }

#define __kernel
#define __global
#define __local

struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
struct float8 { float s[8]; };
struct float16 { float s[16]; };
struct double2 { double x, y; };
struct double4 { double x, y, z, w; };
struct double8 { double s[8]; };
struct double16 { double s[16]; };
