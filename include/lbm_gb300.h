/*
 * lbm_gb300.h -- C ABI of the GB300 D3Q19 lattice Boltzmann hot path.
 *
 * Plain C: opaque handles, plain pointers and sizes, status codes.  Every
 * function returns 0 on success and a negative value on failure, with the
 * message available from lbm_cu_last_error() on the calling thread.
 * `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * Host buffers are caller-owned and caller-sized, as in the reference.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the reference project).  The reference compiles OpenCL programs per
 * domain size at run time and launches them through CCL; here the kernels
 * are compiled once for sm_103a and take sizes at run time.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Cell flags: src/CLbmSolver.hpp:30-33 (src/common.h:19-22). */
#define LBM_FLAG_OBSTACLE 1
#define LBM_FLAG_FLUID 2
#define LBM_FLAG_VELOCITY_INJECTION 4
#define LBM_FLAG_GHOST_LAYER 8

/* Population storage.  F32/F64 correspond to the reference's T = float /
 * double.  F16/BF16/C16 store the shifted deviations f_i - w_i in 16 bits and
 * compute in float (no reference counterpart).  C16 is a 16-bit float of this
 * project with a 13-bit significand (1 sign, 3 exponent, 12 fraction bits;
 * |f_i - w_i| < 1/16, larger values saturate): finer than binary16 within
 * the range the deviations of a flow with |u| < ~0.28 occupy. */
enum lbm_storage { LBM_F32 = 0, LBM_F64 = 1, LBM_F16 = 2, LBM_BF16 = 3, LBM_C16 = 4 };

/* Fields for rectangular reads and writes. */
enum lbm_field {
    LBM_FIELD_DD = 0,       /* 19 population planes */
    LBM_FIELD_VELOCITY = 1, /* 3 planes: the momentum sum_i e_i f_i */
    LBM_FIELD_DENSITY = 2,  /* 1 plane */
    LBM_FIELD_FLAGS = 3     /* 1 plane of int32 on the host */
};

/* Kernel arguments, given in double and rounded to the arithmetic type.
 * inv_tau, gravity and lid are the reference kernel arguments
 * (src/CLbmSolver.hpp:593-612).  les_c = 18*sqrt(2)*Cs^2 switches on the
 * Smagorinsky subgrid model (0 = off, the reference's plain BGK) and tau0 is
 * the molecular relaxation time it builds on. */
typedef struct lbm_params {
    double inv_tau;
    double tau0;
    double les_c;
    double gravity[3];
    double lid;
    /* 0: the reference's alpha forcing, whose temporary aliases rho
     * (lbm_alpha.cl:173): the term of pair k is coefficient k times the term of
     * pair k-1, and the stored density is the last term.  1: each pair's term
     * is its coefficient times the density, and the stored density is the
     * density (not the reference's results; off by default). */
    int32_t gravity_mode;
} lbm_params;

typedef struct lbm_lattice lbm_lattice; /* one subdomain's device fields */
typedef struct lbm_domain lbm_domain;   /* a decomposed domain on one GPU */

/* Message of the last failed call on this thread ("" if none). */
const char *lbm_cu_last_error(void);

/* Library build string (kernels, architecture, compile options). */
const char *lbm_cu_version(void);

/* Wait for all work on `stream` (NULL: the whole device).  Replaces
 * CLbmSolver::wait / clFinish (src/CLbmSolver.hpp:681-683). */
int lbm_cu_synchronize(void *stream);

/* Check of the staged kernels' failure path (no reference counterpart):
 * launches one block whose bounded barrier wait (`polls` polls, at most the
 * staged kernels' 2^22) runs out because nothing completes the barrier; the
 * block records the timeout like a staged kernel that gave up waiting for
 * its bulk copies and returns, so the next lbm_cu_synchronize fails with
 * that message, clears it, and the device stays usable.  No fault, no trap. */
int lbm_cu_check_wait_timeout(unsigned int polls, void *stream);

/* ---------------------------------------------------------------- lattice */

/* Allocate the fields of one nx*ny*nz lattice on the current device.
 * Replaces the buffer creation of CLbmSolver::reload
 * (src/CLbmSolver.hpp:381-403).  Velocity and density planes exist only when
 * requested, like STORE_VELOCITY / STORE_DENSITY (src/CLbmSolver.hpp:369-373). */
int lbm_cu_create(int nx, int ny, int nz, int storage, int store_velocity, int store_density,
                  lbm_lattice **out);
int lbm_cu_destroy(lbm_lattice *lat);
int lbm_cu_dims(const lbm_lattice *lat, int dims[3]);

/* Set the kernel arguments.  Replaces the setArg calls of
 * CLbmSolver::reload / addDrivenCavityValue (src/CLbmSolver.hpp:592-612,262-270). */
int lbm_cu_set_params(lbm_lattice *lat, const lbm_params *p);

/* init_kernel (src/cl_programs/lbm_init.cl:32-237), enqueued by
 * CLbmSolver::reset (src/CLbmSolver.hpp:619-635): flags from the six face
 * conditions bc = {x-, x+, y-, y+, z-, z+}, rest equilibrium, u = 0, rho = 1. */
int lbm_cu_init(lbm_lattice *lat, const int bc[6], void *stream);

/* Seeded start-up field (no reference counterpart): every cell strictly
 * inside the physical domain gets eq(rho = 1, u) with u uniform on
 * [-amp, amp) per component from Philox4x32-10 keyed by (seed, physical cell
 * index), stored in the slot order the first (beta) step reads.
 * origin = physical position of cell (0,0,0), phys = physical domain size. */
int lbm_cu_perturb(lbm_lattice *lat, const int origin[3], const int phys[3], uint64_t seed,
                   double amp, void *stream);

/* One step: parity 0 = lbm_kernel_beta (src/cl_programs/lbm_beta.cl),
 * parity 1 = lbm_kernel_alpha (src/cl_programs/lbm_alpha.cl).  Replaces
 * CLbmSolver::simulationStepBeta / simulationStepAlpha
 * (src/CLbmSolver.hpp:637-659); the caller keeps the step counter like
 * CLbmSolver::simulationStep (src/CLbmSolver.hpp:664-676). */
int lbm_cu_step(lbm_lattice *lat, int parity, void *stream);

/* Kernel shape of the step.  1: one cell per thread.  2: two neighbouring x
 * cells per thread with 64-bit accesses (32-bit for 16-bit storage) where the
 * arithmetic type is float and nx is even, else 1.  3: persistent blocks
 * that stream tiles of cells through shared memory with TMA bulk copies (a
 * producer warp keeps the next tiles in flight while eight warps compute);
 * float and the 16-bit storage types, else 1; the beta step of a lattice whose
 * nx is not a multiple of 16 bytes of populations runs shape 1.  0
 * (default): 3 for the 16-bit storage types, 1 for float and double, the
 * fastest measured on GB300.  All shapes give bit-identical results.  No
 * reference counterpart (the reference's work-group size list,
 * src/CLbmSolver.hpp:279-312, tunes its OpenCL launch instead). */
int lbm_cu_set_kernel_shape(lbm_lattice *lat, int cells_per_thread);

/* Double lattices only: enable != 0 runs the step with kernels whose FP64
 * products may fuse into the following sum (one rounding instead of two);
 * 0 (default) keeps the bit-exact reference arithmetic.  A contracted step
 * differs from the reference's by a relative 1e-15 (bound: 1e-12 per step),
 * and runs faster because the double kernels are bound by the FP64 pipe.
 * One cell per thread; overrides the kernel shape.  No reference counterpart
 * (the reference builds its double kernels with the OpenCL compiler's
 * defaults, src/CLbmSolver.hpp:319-373). */
int lbm_cu_set_fp64_contraction(lbm_lattice *lat, int enable);

/* Rectangular copy of one field between the lattice and a HOST buffer laid
 * out [plane][z][y][x] of size[0]*size[1]*size[2] cells per plane, elements
 * of the arithmetic type (float for F32/F16/BF16/C16, double for F64) or int32
 * for flags.  Blocking, like the reference's CL_TRUE reads.  Replaces
 * storeDensityDistribution / storeVelocity / storeDensity / storeFlags and
 * their set* counterparts, with or without a rectangle
 * (src/CLbmSolver.hpp:688-978).  For writes of LBM_FIELD_DD, `norm` (may be
 * NULL) restricts the copy to populations f with norm . e_f > 0, as the
 * masked setDensityDistribution (src/CLbmSolver.hpp:738-757). */
int lbm_cu_read(lbm_lattice *lat, int field, const int origin[3], const int size[3], void *host_dst,
                void *stream);
int lbm_cu_write(lbm_lattice *lat, int field, const int origin[3], const int size[3],
                 const void *host_src, const int norm[3], void *stream);

/* Device-to-device CComm exchange between two lattices of the same storage
 * (no host staging): dst[dst_origin + box] = src[src_origin + box] for every
 * population plane, or only for those with norm . e_f > 0 when norm is not
 * NULL.  Replaces one storeDensityDistribution -> MPI -> setDensityDistribution
 * round trip of CController::syncAlpha / syncBeta (src/CController.hpp:265-383). */
int lbm_cu_halo(lbm_lattice *src, const int src_origin[3], lbm_lattice *dst, const int dst_origin[3],
                const int size[3], const int norm[3], void *stream);

/* FP64 compensated (Neumaier) sums over fluid cells of mass, momentum and
 * kinetic energy of the populations currently stored: out = {sum rho,
 * sum jx, sum jy, sum jz, sum |j|^2/2}.  `layout` 0: standard slots (after a
 * beta step), 1: opposite slots (after an alpha step or the seeded start-up).
 * No reference counterpart. */
int lbm_cu_reduce_conserved(lbm_lattice *lat, int layout, double out[5], void *stream);

/* Velocity error of lattice a against lattice b (same size) over the fluid
 * cells of a, in FP64: out = {max |ua - ub|, sum |ua - ub|^2, sum |ub|^2,
 * max |ub|, number of cells}, u = sum_i e_i f_i of the stored populations
 * in each lattice's slot layout.  For precision studies against an FP64
 * run; no reference counterpart. */
int lbm_cu_compare_velocity(lbm_lattice *a, int layout_a, lbm_lattice *b, int layout_b, double out[5],
                            void *stream);

/* How the stored deviations of a 16-bit lattice (F16, BF16, C16) use their
 * format, over the 19 slots of the fluid cells: out = {values, zeros,
 * subnormals (nonzero below the smallest normal magnitude), values at the
 * largest finite magnitude or beyond, largest |f_i - w_i|}.  For precision
 * studies; no reference counterpart. */
int lbm_cu_deviation_stats(lbm_lattice *lat, double out[5], void *stream);

/* The same sums, for callers that must not allocate device memory (no
 * counterpart in the reference).  lbm_cu_reduce_conserved may grow the
 * lattice's staging buffer with cudaMalloc; a serving loop whose HBM is all
 * handed out under a budget, or a monitor that must not trigger the implicit
 * synchronisation of cudaMalloc/cudaFree, cannot afford that.  This variant
 * keeps its partial sums in a fixed device array inside the library
 * (1.3 MB, present on every GPU that loads the library until the process
 * exits) and calls no allocator.  Limit: lattices of at most 134,217,728
 * cells (512^3); larger ones are rejected with an error.  The first call on
 * a device looks up the array's device address, so make that first call
 * before any stream capture.  With CUDA's lazy module loading that first
 * call may also be what loads this part of the library onto the device (an
 * implicit allocation of the array itself), so make one warm-up call on each
 * device before handing out the rest of its memory.  All calls share the
 * array: calls whose work overlaps on the GPU race and must be ordered by
 * the caller. */
int lbm_cu_reduce_conserved_noalloc(lbm_lattice *lat, int layout, double out[5], void *stream);

/* Checkpoint / restart (no reference counterpart: the reference writes VTK
 * snapshots only).  The file holds the lattice's raw stored populations
 * (bit for bit, any storage type), its flags and `counter`, the step counter
 * of the caller; the counter's parity is the A-A slot layout of the stored
 * populations (odd after an alpha step), so restarting with the returned
 * counter continues the exact kernel sequence: the results are identical to
 * an uninterrupted run.  Load checks the size and storage type and an FNV-1a
 * hash of the data.  Both synchronise `stream` first and block. */
int lbm_cu_checkpoint_save(lbm_lattice *lat, const char *path, int64_t counter, void *stream);
int lbm_cu_checkpoint_load(lbm_lattice *lat, const char *path, int64_t *counter, void *stream);

/* ----------------------------------------------------------------- domain */

/* A decomposed domain held on one GPU: the even split and CComm geometry of
 * CManager::initSimulation (src/CManager.hpp:49-204) for every subdomain at
 * once, the lid plane of CController::setGeometry (src/CController.hpp:531-546)
 * in the top row of subdomains when lid_geometry != 0, and halo exchanges as
 * device-local copies.  Subdomain i has coordinates (i % nx, i / nx % ny,
 * i / (nx*ny)) like the reference's rank mapping. */
int lbm_cu_domain_create(const int size[3], const int nums[3], int storage, int store_velocity,
                         int store_density, int lid_geometry, lbm_domain **out);
/* The same domain over lattices the caller already owns and initialised
 * (one per subdomain, in subdomain order, each of the subdomain size, one
 * storage type and the same stored fields): CManager's controllers run their
 * lock-step time loop through it (one step launch over all subdomains and
 * one halo launch per axis instead of one launch per subdomain and per
 * CComm).  Destroying the view leaves the lattices alone; parameters set on
 * a lattice directly take effect at the next lbm_cu_domain_run. */
int lbm_cu_domain_wrap(lbm_lattice *const *subdomains, const int size[3], const int nums[3], int lid_geometry,
                       lbm_domain **out);
int lbm_cu_domain_destroy(lbm_domain *dom);
int lbm_cu_domain_set_params(lbm_domain *dom, const lbm_params *p);
/* init + geometry for all subdomains, step counter 0 (CLbmSolver::reset). */
int lbm_cu_domain_reset(lbm_domain *dom, void *stream);
/* Seeded start-up keyed by physical cell (neighbours overlap by two cells). */
int lbm_cu_domain_perturb(lbm_domain *dom, uint64_t seed, double amp, void *stream);
/* `steps` calls of CController::computeNextStep for every subdomain
 * (src/CController.hpp:385-391): one batched step launch over all
 * subdomains, then the halo exchange in x, y, z order.  Whole pairs of steps
 * replay a captured CUDA graph when use_graph != 0. */
int lbm_cu_domain_run(lbm_domain *dom, int steps, int use_graph, void *stream);
/* Velocity and density (when the domain stores them) are written on every
 * `interval`-th step, like STORE_VELOCITY / STORE_DENSITY at interval 1
 * (the default); interval 0 writes them only on the last step of each
 * lbm_cu_domain_run call. */
int lbm_cu_domain_set_store_interval(lbm_domain *dom, int interval);
/* Populations exchanged after an alpha step: mode 0 copies all 19 of the
 * neighbour's inner layer into the ghost layer, as syncAlpha does
 * (src/CController.hpp:265-320); mode 1 copies only the 5 that the ghost
 * layer's inner neighbours gather in the next beta step (direction . e < 0).
 * Both give identical fluid, lid and wall cells; ghost-layer populations
 * differ in the 14 slots no other cell reads. */
int lbm_cu_domain_set_halo_mode(lbm_domain *dom, int mode);
/* enable != 0 (default): where the subdomains run the one-cell kernels
 * (kernel shape 1, the default for float and double), each alpha step also
 * does the x part of the exchange after it -- the thread of a cell at
 * x = nx-2 (x = 1) copies that cell's exchanged planes straight into the
 * ghost cell x = 0 (x = nx-1) of its x neighbour -- instead of a separate
 * copy launch that reads the face back.  The results are identical; the y
 * and z parts still follow in their own launches, so the corners travel in
 * two hops as in CController::syncAlpha (src/CController.hpp:265-320).
 * 0: the x part runs as its own launch. */
int lbm_cu_domain_set_fused_exchange(lbm_domain *dom, int enable);
/* Kernel shape of every subdomain's step (see lbm_cu_set_kernel_shape). */
int lbm_cu_domain_set_kernel_shape(lbm_domain *dom, int cells_per_thread);
/* Contracted FP64 kernels for every subdomain (see lbm_cu_set_fp64_contraction). */
int lbm_cu_domain_set_fp64_contraction(lbm_domain *dom, int enable);
/* Time every step-kernel launch with a pair of CUDA events on the launching
 * stream (steps then run without graph replay), and read the accumulated
 * milliseconds and launch count (reset != 0 clears them).  Stands in for the
 * reference's -DPROFILE event timestamps (src/libcl/CCL.hpp:1752-1776). */
int lbm_cu_domain_profile(lbm_domain *dom, int enable);
int lbm_cu_domain_kernel_time(lbm_domain *dom, double *ms_total, int64_t *launches, int reset);
/* The same times split by step kind: index 0 beta steps (even counter),
 * 1 alpha steps (odd counter). */
int lbm_cu_domain_kernel_time_by_step(lbm_domain *dom, double ms[2], int64_t launches[2], int reset);
/* Capture the next `steps` steps (from the current step counter's parity)
 * into one CUDA graph without running them, with an event pair around the
 * step kernels of steps k with k % every < 2 (every = 1: all of them; every
 * event record in the graph costs about 1 % at 256^3 in 2x2x1 subdomains, so
 * a sample of beta/alpha pairs times the kernels at a smaller cost).  While
 * profiling is on (lbm_cu_domain_profile), the next lbm_cu_domain_run of
 * exactly that many steps with use_graph != 0 from a counter of the same
 * parity launches this graph, and lbm_cu_domain_kernel_time then reads its
 * events: kernel times of a run replayed as a graph.  Velocity and density,
 * if stored, are written on the last step only (store interval 0).  Any
 * change of the domain's parameters or kernel options drops the graph.  No
 * reference counterpart (the reference times its steps with host clocks,
 * src/CController.hpp:396-522). */
int lbm_cu_domain_prepare_timed_run(lbm_domain *dom, int steps, int every, void *stream);
int lbm_cu_domain_counter(const lbm_domain *dom, int64_t *counter);
/* Step counter of the next lbm_cu_domain_run (its parity picks beta or alpha;
 * CLbmSolver::simulation_step_counter). */
int lbm_cu_domain_set_counter(lbm_domain *dom, int64_t counter);
int lbm_cu_domain_subdomains(const lbm_domain *dom, int *count, int sub_size[3]);
lbm_lattice *lbm_cu_domain_lattice(lbm_domain *dom, int index);

/* Checkpoint / restart of a whole decomposed domain: every subdomain's raw
 * populations and flags and the domain's step counter, which load restores
 * (see lbm_cu_checkpoint_save).  The domain must have the same size,
 * decomposition and storage type. */
int lbm_cu_domain_checkpoint_save(lbm_domain *dom, const char *path, void *stream);
int lbm_cu_domain_checkpoint_load(lbm_domain *dom, const char *path, void *stream);

/* ------------------------------------------------------ batches, serving */

/* One lid-driven cavity of an ensemble, in lattice units: walls on all six
 * faces and the lid plane of CController::setGeometry
 * (src/CController.hpp:531-546) moving at `lid`; relaxation time tau0,
 * Smagorinsky constant cs (0 = plain BGK); `steps` time steps; optional
 * seeded start-up velocity amplitude `amp` (0 = rest).  No reference
 * counterpart (the reference runs one domain per process). */
typedef struct lbm_cavity {
    int nx, ny, nz;
    int storage;
    double tau0;
    double cs;
    double lid;
    int64_t steps;
    uint64_t seed;
    double amp;
} lbm_cavity;

typedef struct lbm_batch lbm_batch;
typedef struct lbm_server lbm_server;

/* `steps` time steps of one lattice whose step counter is `first_step`, one
 * launch per step (CLbmSolver::simulationStep in a loop). */
int lbm_cu_run(lbm_lattice *lat, int64_t first_step, int64_t steps, void *stream);

/* An ensemble of cavities of different sizes, parameters, storage types and
 * step counts, all resident, advanced together: one launch per storage type
 * and step covers every unfinished cavity, pairs of steps replay a captured
 * CUDA graph, every cavity stops at its own step count.  Each cavity's
 * fields are the same as when it runs alone (lbm_cu_batch_lattice gives
 * its lattice for readback; velocity is written on its last step when
 * store_velocity is set). */
int lbm_cu_batch_create(const lbm_cavity *cavities, int count, int store_velocity, lbm_batch **out);
int lbm_cu_batch_destroy(lbm_batch *b);
int lbm_cu_batch_reset(lbm_batch *b, void *stream);
/* Ensemble kernel shape: 1 one cell per thread (default), 2 two cells per
 * thread (cavities with even nx), 3 as 1 but the alpha steps of half and
 * bfloat16 cavities run the staged tiles when every member of a launch is
 * at an alpha step.  Results are the same for every shape. */
int lbm_cu_batch_set_kernel_shape(lbm_batch *b, int cells_per_thread);
/* Autotuner: times `trial_steps` steps of the whole ensemble for each kernel
 * shape (1, 2, 3), keeps the fastest, and resets. */
int lbm_cu_batch_tune(lbm_batch *b, int trial_steps, int *cells_per_thread, double *ms_per_step, void *stream);
/* Run until every cavity has taken its steps, or at most max_steps steps
 * (max_steps < 0: no limit). */
int lbm_cu_batch_run(lbm_batch *b, int64_t max_steps, int use_graph, void *stream);
int lbm_cu_batch_status(const lbm_batch *b, int64_t *min_done, int *active);
lbm_lattice *lbm_cu_batch_lattice(lbm_batch *b, int index);

/* Continuous-batching solve server.  Submitted solves queue; each tick
 * admits queued solves in arrival order while their device memory fits the
 * HBM budget (and fewer than max_active run), advances every running solve
 * by up to max_steps steps in shared launches (stopping when the first one
 * completes), and retires completed solves, whose fields stay resident
 * until released.  A solve's result does not depend on what else runs. */
int lbm_cu_server_create(double hbm_budget_bytes, int max_active, int store_velocity, lbm_server **out);
int lbm_cu_server_destroy(lbm_server *s);
/* As lbm_cu_batch_set_kernel_shape; a server starts with shape 3. */
int lbm_cu_server_set_kernel_shape(lbm_server *s, int cells_per_thread);
int lbm_cu_server_submit(lbm_server *s, const lbm_cavity *c, int64_t *id);
int lbm_cu_server_tick(lbm_server *s, int64_t max_steps, int use_graph, int *admitted, void *stream);
int lbm_cu_server_poll(lbm_server *s, int64_t *ids, int capacity, int *count);
lbm_lattice *lbm_cu_server_lattice(lbm_server *s, int64_t id);
int lbm_cu_server_release(lbm_server *s, int64_t id);
int lbm_cu_server_status(const lbm_server *s, int *queued, int *active, double *hbm_used, int64_t *cell_updates);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
