// CLbmSolver.hpp -- the reference's solver interface (src/CLbmSolver.hpp:67-1124)
// over the C ABI of lbm_gb300.h.  Same public members and methods; the three
// OpenCL handles of the reference constructor become one CDeviceContext, and
// an optional CLbmOptions (storage type, Smagorinsky constant, lattice
// units) may follow the reference's arguments.  The kernels are compiled
// once for sm_103a, so reload() allocates and binds instead of building
// OpenCL programs; the work-group and register lists are kept for interface
// compatibility and do not change the CUDA launch shape.
#ifndef LBM_GB300_CLBMSOLVER_HPP
#define LBM_GB300_CLBMSOLVER_HPP

#include <cmath>
#include <iomanip>
#include <iostream>
#include <list>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../lbm_gb300.h"
#include "CLbmSkeleton.hpp"

#define LBM_FLAG_GHOST_LAYER_BETA (LBM_FLAG_GHOST_LAYER | (1 << 4))

/** Device and stream the solver runs on (stands in for the reference's
 *  CCL::CCommandQueue / CContext / CDevice). */
struct CDeviceContext {
    int device = 0;
    void *stream = nullptr;  // cudaStream_t; nullptr = legacy default stream
};

/** Options with no counterpart in the reference. */
template <typename T>
struct CLbmOptions {
    int storage = -1;           // LBM_F32/F64 from T when -1; LBM_F16/BF16/C16 need T = float
    T smagorinsky = T(0);       // Cs; 0 keeps the reference's plain BGK
    bool lattice_units = false; // take tau and the lid speed below as given
    T lattice_tau = T(0);
    T lattice_lid = T(0);
    int gravity_mode = 0;       // 1: per-term gravity forcing instead of the reference's (lbm_params)
};

/** D3Q19 direction vectors in reference order (src/main.cpp:38-66). */
inline const CVector<3, int> &lbm_unit(int f) {
    static const CVector<3, int> e[19] = {
        {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},
        {-1, 1, 0}, {1, 0, 1},  {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1}, {0, 1, 1},   {0, -1, -1},
        {0, 1, -1}, {0, -1, 1}, {0, 0, 1},  {0, 0, -1}, {0, 0, 0}};
    return e[f];
}

template <typename T>
class CLbmSolver : public CLbmSkeleton<T> {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "T is float or double");

public:
    CVector<4, T> drivenCavityVelocity;
    static const size_t SIZE_DD_HOST = 19;

private:
    int _UID;
    int _BC[3][2];
    CDeviceContext &ctx;
    CLbmOptions<T> opt;
    lbm_lattice *lat = nullptr;
    size_t computation_kernel_count;
    size_t domain_cells_count = 0;
    bool store_velocity, store_density;

    void fail(const char *what) {
        error << what << ": " << lbm_cu_last_error() << CError::endl;
    }
    int storage() const {
        if (opt.storage >= 0) return opt.storage;
        return std::is_same<T, double>::value ? LBM_F64 : LBM_F32;
    }
    lbm_params params(T lid) const {
        lbm_params p{};
        p.inv_tau = this->inv_tau;
        p.tau0 = this->tau;
        p.les_c = (double)(T)(18.0 * std::sqrt(2.0) * (double)opt.smagorinsky * (double)opt.smagorinsky);
        for (int a = 0; a < 3; a++) p.gravity[a] = this->gravitation[a];
        p.lid = lid;
        p.gravity_mode = opt.gravity_mode;
        return p;
    }
    int o3(const CVector<3, int> &v, int out[3]) const {
        out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
        return 0;
    }

public:
    size_t simulation_step_counter = 0;
    CError error;
    std::list<int> lbm_opencl_number_of_work_items_list;
    std::list<int> lbm_opencl_number_of_registers_list;

    CLbmSolver(int UID, CDeviceContext &p_ctx, int BC[3][2], CDomain<T> &domain, CVector<3, T> &p_d_gravitation,
               T p_d_viscosity, size_t p_computation_kernel_count, bool p_store_velocity, bool p_store_density,
               T p_d_timestep, CVector<4, T> &_drivenCavityVelocity, std::list<int> &p_work_items_list,
               std::list<int> &p_registers_list, const CLbmOptions<T> &p_opt = CLbmOptions<T>())
        : CLbmSkeleton<T>(CDomain<T>(domain), _drivenCavityVelocity),
          drivenCavityVelocity(_drivenCavityVelocity),
          _UID(UID),
          ctx(p_ctx),
          opt(p_opt),
          computation_kernel_count(p_computation_kernel_count),
          store_velocity(p_store_velocity),
          store_density(p_store_density),
          lbm_opencl_number_of_work_items_list(p_work_items_list),
          lbm_opencl_number_of_registers_list(p_registers_list) {
        (void)p_d_timestep;  // read but unused by the reference as well
        if (opt.lattice_units)
            CLbmSkeleton<T>::initLattice(opt.lattice_tau, opt.lattice_lid, p_d_gravitation);
        else
            CLbmSkeleton<T>::init(p_d_gravitation, p_d_viscosity, 1.0);
        if (CLbmSkeleton<T>::error()) error << CLbmSkeleton<T>::error.getString();
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 2; j++) _BC[i][j] = BC[i][j];
        reload();
    }

    ~CLbmSolver() {
        if (lat) lbm_cu_destroy(lat);
    }
    CLbmSolver(const CLbmSolver &) = delete;
    CLbmSolver &operator=(const CLbmSolver &) = delete;

    /** the device lattice (for halo exchanges) */
    lbm_lattice *lattice() { return lat; }
    /** the stream every operation of this solver is issued on */
    void *stream() const { return ctx.stream; }
    int getUid() const { return _UID; }

    void addDrivenCavityValue(T value) {
        drivenCavityVelocity[0] += value;
        CVector<4, T> p = drivenCavityVelocity;
        p *= CLbmSkeleton<T>::d_timestep;
        if (lbm_cu_set_params(lat, ptr(params(p[0])))) fail("addDrivenCavityValue");
    }

    void reload() {
        if (lat) {
            lbm_cu_destroy(lat);
            lat = nullptr;
        }
        domain_cells_count = (size_t)this->domain_cells.elements();
        if (lbm_cu_create(this->domain_cells[0], this->domain_cells[1], this->domain_cells[2], storage(),
                          store_velocity, store_density, &lat)) {
            fail("creating the lattice");
            return;
        }
        if (lbm_cu_set_params(lat, ptr(params(CLbmSkeleton<T>::drivenCavityVelocity[0])))) fail("kernel arguments");
        reset();
    }

    void reset() {
        simulation_step_counter = 0;
        int bc[6];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 2; j++) bc[i * 2 + j] = _BC[i][j];
        if (lbm_cu_init(lat, bc, ctx.stream)) fail("init");
    }

    void simulationStepAlpha() {
        if (lbm_cu_step(lat, 1, ctx.stream)) fail("alpha step");
    }
    void simulationStepBeta() {
        if (lbm_cu_step(lat, 0, ctx.stream)) fail("beta step");
    }
    void simulationStep() {
        if (simulation_step_counter & 1) simulationStepAlpha();
        else simulationStepBeta();
        simulation_step_counter++;
    }
    void wait() {
        if (lbm_cu_synchronize(ctx.stream)) fail("wait");
    }

    /** Restart file of this subdomain: raw populations, flags and
     *  simulation_step_counter (lbm_cu_checkpoint_save; no reference
     *  counterpart).  false (and the error sink) on failure. */
    bool saveCheckpoint(const std::string &path) {
        if (lbm_cu_checkpoint_save(lat, path.c_str(), (int64_t)simulation_step_counter, ctx.stream)) {
            fail("checkpoint save");
            return false;
        }
        return true;
    }
    /** Restores a checkpoint of a subdomain of the same size and storage,
     *  including simulation_step_counter, so the next simulationStep() runs
     *  the kernel the interrupted run would have run. */
    bool loadCheckpoint(const std::string &path) {
        int64_t c = 0;
        if (lbm_cu_checkpoint_load(lat, path.c_str(), &c, ctx.stream)) {
            fail("checkpoint load");
            return false;
        }
        simulation_step_counter = (size_t)c;
        return true;
    }

    // ---------------------------------------------------------- transfers
    void storeDensityDistribution(T *dst) { io(LBM_FIELD_DD, nullptr, nullptr, dst, nullptr, true); }
    void storeDensityDistribution(T *dst, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_DD, &origin, &size, dst, nullptr, true);
    }
    void setDensityDistribution(T *src, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_DD, &origin, &size, src, nullptr, false);
    }
    void setDensityDistribution(T *src, CVector<3, int> &origin, CVector<3, int> &size, CVector<3, int> norm) {
        io(LBM_FIELD_DD, &origin, &size, src, &norm, false);
    }
    void storeVelocity(T *dst) { io(LBM_FIELD_VELOCITY, nullptr, nullptr, dst, nullptr, true); }
    void storeVelocity(T *dst, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_VELOCITY, &origin, &size, dst, nullptr, true);
    }
    void setVelocity(T *src, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_VELOCITY, &origin, &size, src, nullptr, false);
    }
    void storeDensity(T *dst) { io(LBM_FIELD_DENSITY, nullptr, nullptr, dst, nullptr, true); }
    void storeDensity(T *dst, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_DENSITY, &origin, &size, dst, nullptr, true);
    }
    void setDensity(T *src, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_DENSITY, &origin, &size, src, nullptr, false);
    }
    /** reads domain_cells ints (the reference sizes this read by the density
     *  buffer, src/CLbmSolver.hpp:907-912) */
    void storeFlags(int *dst) { io(LBM_FIELD_FLAGS, nullptr, nullptr, dst, nullptr, true); }
    void storeFlags(int *dst, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_FLAGS, &origin, &size, dst, nullptr, true);
    }
    void setFlags(int *src, CVector<3, int> &origin, CVector<3, int> &size) {
        io(LBM_FIELD_FLAGS, &origin, &size, src, nullptr, false);
    }

    // ------------------------------------------------------------- debug
    void debug_print() {
        std::vector<T> dd(domain_cells_count * SIZE_DD_HOST);
        storeDensityDistribution(dd.data());
        std::cout << "DENSITY DISTRIBUTIONS:";
        dump(dd.data(), dd.size(), 16);
        if (store_velocity) {
            std::vector<T> v(domain_cells_count * 3);
            storeVelocity(v.data());
            std::cout << std::endl << "VELOCITY:";
            dump(v.data(), v.size(), 12);
        }
        if (store_density) {
            std::vector<T> r(domain_cells_count);
            storeDensity(r.data());
            std::cout << std::endl << "DENSITY:";
            dump(r.data(), r.size(), 4);
        }
        std::vector<int> fl(domain_cells_count);
        storeFlags(fl.data());
        std::cout << std::endl << "FLAGS:";
        for (size_t i = 0; i < fl.size(); i++) {
            if (i % 16 == 0) std::cout << std::endl << (i / 16) << ": ";
            std::cout << fl[i] << " ";
        }
        std::cout << std::endl;
    }

    void debugDD(size_t dd_id = 0, size_t wrap_size = 16, size_t empty_line = 16) {
        std::vector<T> dd(domain_cells_count * SIZE_DD_HOST);
        storeDensityDistribution(dd.data());
        std::streamsize ss = std::cout.precision();
        std::cout.precision(4);
        std::cout.setf(std::ios::fixed, std::ios::floatfield);
        const size_t start = domain_cells_count * dd_id, end = domain_cells_count * (dd_id + 1);
        for (size_t i = start; i < end; i++) {
            if (empty_line != wrap_size && i % empty_line == 0 && i != start) std::cout << std::endl;
            if (i % wrap_size == 0) {
                if (i != start) std::cout << std::endl;
                std::cout << (i / wrap_size) << ": ";
            }
            std::cout << dd[i] << " ";
        }
        std::cout.precision(ss);
        std::cout << std::resetiosflags(std::ios::fixed) << std::endl;
    }

    /** sum of vx+vy+vz over fluid cells, in float (src/CLbmSolver.hpp:1103-1123) */
    float getVelocityChecksum() {
        std::vector<T> v(domain_cells_count * 3);
        std::vector<int> fl(domain_cells_count);
        storeVelocity(v.data());
        storeFlags(fl.data());
        float checksum = 0;
        const size_t n = domain_cells_count;
        for (size_t a = 0; a < n; a++)
            if (fl[a] == LBM_FLAG_FLUID) checksum += v[a] + v[n + a] + v[2 * n + a];
        return checksum;
    }

private:
    static const lbm_params *ptr(const lbm_params &p) {
        static thread_local lbm_params keep;
        keep = p;
        return &keep;
    }
    void io(int field, CVector<3, int> *origin, CVector<3, int> *size, void *host, CVector<3, int> *norm, bool read) {
        int o[3], s[3], nm[3];
        if (origin) o3(*origin, o);
        if (size) o3(*size, s);
        if (norm) o3(*norm, nm);
        const int rc = read ? lbm_cu_read(lat, field, origin ? o : nullptr, size ? s : nullptr, host, ctx.stream)
                            : lbm_cu_write(lat, field, origin ? o : nullptr, size ? s : nullptr, host,
                                           norm ? nm : nullptr, ctx.stream);
        if (rc) fail(read ? "read" : "write");
    }
    static void dump(const T *b, size_t n, size_t wrap) {
        std::streamsize ss = std::cout.precision();
        std::cout.precision(4);
        std::cout.setf(std::ios::fixed, std::ios::floatfield);
        for (size_t i = 0; i < n; i++) {
            if (i % wrap == 0) std::cout << std::endl << (i / wrap) << ": ";
            std::cout << b[i] << " ";
        }
        std::cout.precision(ss);
        std::cout << std::resetiosflags(std::ios::fixed);
    }
};

#endif
