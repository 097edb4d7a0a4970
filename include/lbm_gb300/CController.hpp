// CController.hpp -- one subdomain's controller (src/CController.hpp:54-563):
// owns a CLbmSolver and its CComm list, exchanges halos, runs the time loop.
//
// All subdomains of a run live in one process on one GPU, so syncAlpha /
// syncBeta pull the neighbour's face straight out of its device lattice
// (lbm_cu_halo) instead of staging through the host and MPI.  The exchange
// semantics are the reference's: after an alpha step the neighbour's inner
// layer (all 19 populations) lands in this subdomain's ghost layer; after a
// beta step the neighbour's ghost layer returns to this subdomain's inner
// layer, populations with direction . e > 0 only.  The neighbours must have
// finished the same step first, which CManager::startSimulation guarantees
// by stepping every subdomain and then exchanging axis by axis (x, y, z),
// the order in which each reference rank walks its CComm list.
#ifndef LBM_GB300_CCONTROLLER_HPP
#define LBM_GB300_CCONTROLLER_HPP

#include <fstream>
#include <iostream>
#include <list>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "CComm.hpp"
#include "CConfiguration.hpp"
#include "CDomain.hpp"
#include "CLbmSolver.hpp"
#include "CLbmVisualizationVTK.hpp"
#include "CStopwatch.hpp"

// output folders of the reference (src/common.h:26-28)
#ifndef BENCHMARK_OUTPUT_DIR
#define BENCHMARK_OUTPUT_DIR "output/benchmark"
#endif
#ifndef VTK_OUTPUT_DIR
#define VTK_OUTPUT_DIR "output/vtk"
#endif

// mkdir -p
inline void lbm_make_dirs(const std::string &path) {
    for (size_t i = 1; i <= path.size(); i++)
        if (i == path.size() || path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

template <typename T>
using ConfigSingletonT = Singleton<CConfiguration<T>>;

template <typename T>
class CController {
    int _UID;
    CDomain<T> _domain;
    CLbmSolver<T> *cLbmPtr = nullptr;
    int _BC[3][2];
    std::vector<CComm<T> *> _comm_container;
    std::vector<CController<T> *> *_peers = nullptr;
    CDeviceContext _ctx;

    int initLBMSolver() {
        CConfiguration<T> *cfg = ConfigSingletonT<T>::Instance();
        _ctx.device = cfg->device_nr < 0 ? 0 : cfg->device_nr;
        CLbmOptions<T> opt;
        if (cfg->lattice_units) {
            opt.lattice_units = true;
            opt.lattice_lid = cfg->lattice_lid;
            // tau = 3 nu + 1/2 with nu = U L / Re on the global x length in cells
            opt.lattice_tau = cfg->lattice_tau > T(0)
                                  ? cfg->lattice_tau
                                  : (T)(3.0 * (double)cfg->lattice_lid * (double)cfg->domain_size[0] /
                                            (double)cfg->lattice_reynolds + 0.5);
            opt.smagorinsky = cfg->smagorinsky;
            if (cfg->storage == "f16") opt.storage = LBM_F16;
            else if (cfg->storage == "bf16") opt.storage = LBM_BF16;
            else if (cfg->storage == "c16") opt.storage = LBM_C16;
        }
        const bool store = cfg->do_visualization || cfg->debug_mode;
        cLbmPtr = new CLbmSolver<T>(_UID, _ctx, _BC, _domain, cfg->gravitation, cfg->viscosity,
                                    cfg->computation_kernel_count, store, store, cfg->timestep,
                                    cfg->drivenCavityVelocity, cfg->lbm_opencl_number_of_threads_list,
                                    cfg->lbm_opencl_number_of_registers_list, opt);
        if (cLbmPtr->error()) {
            std::cout << cLbmPtr->error.getString();
            return -1;
        }
        cLbmPtr->wait();
        return 0;
    }

    const CComm<T> *peerComm(const CController<T> *peer, int axis) const {
        for (const CComm<T> *c : peer->_comm_container)
            if (c->getDstId() == _UID && c->axis() == axis) return c;
        return nullptr;
    }

    void exchange(bool beta, int axis) {
        if (!_peers) throw "CController: neighbours unknown (use CManager)";
        for (CComm<T> *c : _comm_container) {
            if (axis >= 0 && c->axis() != axis) continue;
            CController<T> *peer = (*_peers)[c->getDstId()];
            const CComm<T> *back = peerComm(peer, c->axis());
            if (!back) throw "CController: no matching CComm on the neighbour";
            int so[3], dof[3], sz[3], nm[3];
            for (int a = 0; a < 3; a++) {
                if (beta) {  // src/CController.hpp:333-377
                    so[a] = back->getRecvOrigin()[a];
                    dof[a] = c->getSendOrigin()[a];
                    sz[a] = c->getSendSize()[a];
                } else {     // src/CController.hpp:272-314
                    so[a] = back->getSendOrigin()[a];
                    dof[a] = c->getRecvOrigin()[a];
                    sz[a] = c->getRecvSize()[a];
                }
                nm[a] = c->getCommDirection()[a];
            }
            if (lbm_cu_halo(peer->cLbmPtr->lattice(), so, cLbmPtr->lattice(), dof, sz, beta ? nm : nullptr,
                            _ctx.stream))
                throw "CController: halo exchange failed";
        }
    }

public:
    CController(int UID, CDomain<T> domain, int BC[3][2]) : _UID(UID), _domain(domain) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 2; j++) _BC[i][j] = BC[i][j];
        if (-1 == initLBMSolver()) throw "Initialization of LBM Solver failed!";
    }
    ~CController() {
        delete cLbmPtr;
        for (CComm<T> *c : _comm_container) delete c;
    }
    CController(const CController &) = delete;
    CController &operator=(const CController &) = delete;

    /** the controllers of all subdomains, indexed by id (set by CManager) */
    void setPeers(std::vector<CController<T> *> *peers) { _peers = peers; }

    void syncAlpha() { exchange(false, -1); }
    void syncBeta() { exchange(true, -1); }
    void syncAlpha(int axis) { exchange(false, axis); }
    void syncBeta(int axis) { exchange(true, axis); }

    /** src/CController.hpp:385-391, for a subdomain whose neighbours have
     *  already stepped (a single subdomain, or driven by CManager). */
    void computeNextStep() {
        cLbmPtr->simulationStep();
        if (_comm_container.empty()) return;
        if (cLbmPtr->simulation_step_counter & 1) syncBeta();
        else syncAlpha();
    }

    /** The time loop of one subdomain and its report (src/CController.hpp:396-522):
     *  with visualization on, a VTK snapshot ./output/vtk/OUTPUT.<UID>.<step>.vtk
     *  after every step. */
    int run() {
        CConfiguration<T> *cfg = ConfigSingletonT<T>::Instance();
        int loops = cfg->loops < 0 ? 100 : cfg->loops;
        CLbmVisualizationVTK<T> *vis = nullptr;
        if (cfg->do_visualization) vis = newVisualization();
        CStopwatch sw;
        sw.start();
        for (int i = 0; i < loops; i++) {
            computeNextStep();
            if (vis) vis->render(i);
        }
        cLbmPtr->wait();
        sw.stop();
        delete vis;  // waits for the last snapshots
        benchmarkRecord(loops, sw.time, cfg->do_visualization || cfg->debug_mode);
        report(_domain.getSize(), loops, sw.time, cfg->do_visualization || cfg->debug_mode);
        return 0;
    }

    /** A VTK writer of this subdomain into ./output/vtk (created if missing). */
    CLbmVisualizationVTK<T> *newVisualization() {
        lbm_make_dirs(VTK_OUTPUT_DIR);
        auto *vis = new CLbmVisualizationVTK<T>(_UID, std::string("./") + VTK_OUTPUT_DIR + "/OUTPUT");
        vis->setup(cLbmPtr);
        return vis;
    }

    /** The console report of a run (src/CController.hpp:478-510). */
    static void report(CVector<3, int> cube, int loops, double seconds, bool vis) {
        double floats_per_cell = 19.0 * 2.0 + 1.0 + (vis ? 3.0 : 0.0);
        double fps = ((double)loops) / seconds;
        double mlups = ((double)fps * (double)cube.elements()) * (double)0.000001;
        std::cout << std::endl << "Cube: " << cube << std::endl;
        std::cout << "Seconds: " << seconds << std::endl;
        std::cout << "FPS: " << fps << std::endl;
        std::cout << "MLUPS: " << mlups << std::endl;
        std::cout << "Bandwidth: " << (mlups * floats_per_cell * (double)sizeof(T)) << " MB/s (RW, bidirectional)"
                  << std::endl;
        std::cout << "done." << std::endl;
    }

    /** With cfg->benchmark, the record of the reference's BENCHMARK build
     *  (src/CController.hpp:445-477): the whole configured domain's timing
     *  appended to output/benchmark/benchmark_<number of subdomains>.ini. */
    static void benchmarkRecord(int loops, double seconds, bool vis) {
        CConfiguration<T> *cfg = ConfigSingletonT<T>::Instance();
        if (!cfg->benchmark) return;
        const double floats_per_cell = 19.0 * 2.0 + 1.0 + (vis ? 3.0 : 0.0);
        const double fps = ((double)loops) / seconds;
        const double mlups = fps * (double)cfg->domain_size.elements() * 0.000001;
        lbm_make_dirs(BENCHMARK_OUTPUT_DIR);
        std::stringstream name;
        name << "./" << BENCHMARK_OUTPUT_DIR << "/benchmark_" << cfg->subdomain_num.elements() << ".ini";
        std::ofstream f(name.str().c_str(), std::ios::out | std::ios::app);
        if (!f.is_open()) {
            std::cout << "Unable to open file";
            return;
        }
        f << "CUBE_X : " << cfg->domain_size[0] << std::endl;
        f << "CUBE_Y : " << cfg->domain_size[1] << std::endl;
        f << "CUBE_Z : " << cfg->domain_size[2] << std::endl;
        f << "SECONDS : " << seconds << std::endl;
        f << "FPS : " << fps << std::endl;
        f << "MLUPS : " << mlups << std::endl;
        f << "BANDWIDTH : " << (mlups * floats_per_cell * (double)sizeof(T)) << std::endl;
        f << std::endl;
    }

    void addCommunication(CComm<T> *comm) { _comm_container.push_back(comm); }
    const std::vector<CComm<T> *> &getCommunications() const { return _comm_container; }

    /** Lid plane y = Y-2, x in [1, X-2], z in [1, Z-2] (src/CController.hpp:531-546). */
    void setGeometry() {
        CVector<3, int> origin(1, _domain.getSize()[1] - 2, 1);
        CVector<3, int> size(_domain.getSize()[0] - 2, 1, _domain.getSize()[2] - 2);
        std::vector<int> src((size_t)size.elements(), LBM_FLAG_VELOCITY_INJECTION);
        cLbmPtr->setFlags(src.data(), origin, size);
    }

    CLbmSolver<T> *getSolver() const { return cLbmPtr; }
    void setSolver(CLbmSolver<T> *p) { cLbmPtr = p; }
    CDomain<T> getDomain() const { return _domain; }
    int getUid() const { return _UID; }
};

#endif
