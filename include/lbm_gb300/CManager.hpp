// CManager.hpp -- domain decomposition (src/CManager.hpp:15-224): even split
// into subdomains, outer faces as walls and inner faces as ghost layers, one
// CComm per ghost face in the reference's order (x-, x+, y-, y+, z-, z+),
// lid geometry on the top row of subdomains.
//
// The reference runs one subdomain per MPI rank; here initSimulation builds
// every subdomain's controller in this process (on one GPU) and
// startSimulation steps them in lock-step: all subdomains take the step,
// then the halo exchange runs axis by axis.  The lock-step loop runs through
// a domain view over the controllers' lattices (lbm_cu_domain_wrap: one step
// launch over all subdomains, one halo launch per axis, CUDA-graph replay of
// whole runs without per-step output) -- the same steps and copies as the
// controllers' simulationStep / syncAlpha / syncBeta, which the environment
// variable LBM_GB300_CONTROLLER_LOOP=1 selects instead.  `my_rank` selects
// the controller getController() returns, so the reference's validate-mode
// flow (src/main.cpp:309-408) keeps working.
#ifndef LBM_GB300_CMANAGER_HPP
#define LBM_GB300_CMANAGER_HPP

#include <cstdlib>
#include <iostream>
#include <vector>

#include "CController.hpp"

template <typename T>
class CManager {
    CDomain<T> _domain;
    CVector<3, int> _subdomain_size;
    CVector<3, T> _subdomain_length;
    CVector<3, int> _subdomain_nums;
    std::vector<CController<T> *> _controllers;
    int _rank = 0;
    lbm_domain *_view = nullptr;  // all subdomains as one domain (nullptr: controller loop)

    // The view when every solver issues on the same stream (else nullptr).
    void buildView() {
        const char *e = std::getenv("LBM_GB300_CONTROLLER_LOOP");
        if (e && e[0] == '1') return;
        std::vector<lbm_lattice *> subs;
        for (auto *c : _controllers) {
            if (c->getSolver()->stream() != _controllers[0]->getSolver()->stream()) return;
            subs.push_back(c->getSolver()->lattice());
        }
        const CVector<3, int> s = _domain.getSize();
        const int size[3] = {s[0], s[1], s[2]};
        const int nums[3] = {_subdomain_nums[0], _subdomain_nums[1], _subdomain_nums[2]};
        if (lbm_cu_domain_wrap(subs.data(), size, nums, 1, &_view)) _view = nullptr;
    }

    // `n` lock-step steps of every subdomain through the view.
    void runView(int n, bool graph) {
        CLbmSolver<T> *s0 = _controllers[0]->getSolver();
        if (lbm_cu_domain_set_counter(_view, (int64_t)s0->simulation_step_counter) ||
            lbm_cu_domain_run(_view, n, graph ? 1 : 0, s0->stream()))
            throw lbm_cu_last_error();
        for (auto *c : _controllers) c->getSolver()->simulation_step_counter += n;
    }

public:
    CManager(CDomain<T> domain, CVector<3, int> subdomainNums) : _domain(domain) { setSubdomainNums(subdomainNums); }
    ~CManager() {
        if (_view) lbm_cu_domain_destroy(_view);  // a view: the lattices stay with the solvers
        for (auto *c : _controllers) delete c;
    }
    CManager(const CManager &) = delete;
    CManager &operator=(const CManager &) = delete;

    CDomain<T> getDomain() const { return _domain; }
    void setDomain(CDomain<T> grid) { _domain = grid; }
    CVector<3, int> getSubdomainNums() const { return _subdomain_nums; }
    CVector<3, int> getSubdomainSize() const { return _subdomain_size; }

    void setSubdomainNums(CVector<3, int> n) {
        CVector<3, int> s = _domain.getSize();
        if (s[0] % n[0] != 0 || s[1] % n[1] != 0 || s[2] % n[2] != 0)
            throw "Number of subdomains does not match with the grid size!";
        for (int a = 0; a < 3; a++) {
            _subdomain_size[a] = s[a] / n[a];
            _subdomain_length[a] = _domain.getLength()[a] / n[a];
        }
        _subdomain_nums = n;
    }

    void initSimulation(int my_rank) {
        _rank = my_rank < 0 ? 0 : my_rank;
        const int count = _subdomain_nums[0] * _subdomain_nums[1] * _subdomain_nums[2];
        const int stride[3] = {1, _subdomain_nums[0], _subdomain_nums[0] * _subdomain_nums[1]};
        for (int id = 0; id < count; id++) {
            int nx = id % _subdomain_nums[0], ny = (id / _subdomain_nums[0]) % _subdomain_nums[1],
                nz = id / (_subdomain_nums[0] * _subdomain_nums[1]);
            const int c[3] = {nx, ny, nz};
            int BC[3][2];
            for (int a = 0; a < 3; a++) {
                BC[a][0] = c[a] == 0 ? LBM_FLAG_OBSTACLE : LBM_FLAG_GHOST_LAYER;
                BC[a][1] = c[a] == _subdomain_nums[a] - 1 ? LBM_FLAG_OBSTACLE : LBM_FLAG_GHOST_LAYER;
            }
            CVector<3, int> origin(nx * _subdomain_size[0], ny * _subdomain_size[1], nz * _subdomain_size[2]);
            CDomain<T> sub(id, _subdomain_size, origin, _subdomain_length);
            auto *ctl = new CController<T>(id, sub, BC);
            for (int a = 0; a < 3; a++)
                for (int up = 0; up < 2; up++) {
                    if (BC[a][up] != LBM_FLAG_GHOST_LAYER) continue;
                    CVector<3, int> size = _subdomain_size, so(0, 0, 0), ro(0, 0, 0), dir(0, 0, 0);
                    size[a] = 1;
                    so[a] = up ? _subdomain_size[a] - 2 : 1;
                    ro[a] = up ? _subdomain_size[a] - 1 : 0;
                    dir[a] = up ? -1 : 1;
                    ctl->addCommunication(new CComm<T>(id + (up ? stride[a] : -stride[a]), size, size, so, ro, dir));
                }
            if (ny == _subdomain_nums[1] - 1) ctl->setGeometry();
            _controllers.push_back(ctl);
        }
        for (auto *c : _controllers) c->setPeers(&_controllers);
        buildView();
    }

    /** One time step of every subdomain followed by the halo exchange. */
    void step() {
        if (_view) {
            runView(1, false);
            return;
        }
        for (auto *c : _controllers) c->getSolver()->simulationStep();
        const bool beta = _controllers[0]->getSolver()->simulation_step_counter & 1;
        for (int axis = 0; axis < 3; axis++)
            for (auto *c : _controllers) {
                if (beta) c->syncBeta(axis);
                else c->syncAlpha(axis);
            }
    }

    /** All subdomains' time loops in lock-step and the report of the whole
     *  domain; with visualization on, every subdomain writes its VTK snapshot
     *  after every step, as each reference rank does. */
    void startSimulation() {
        if (_controllers.empty()) throw "CManager: Initialize the simulation before starting it!";
        CConfiguration<T> *cfg = ConfigSingletonT<T>::Instance();
        int loops = cfg->loops < 0 ? 100 : cfg->loops;
        std::vector<CLbmVisualizationVTK<T> *> vis;
        if (cfg->do_visualization)
            for (auto *c : _controllers) vis.push_back(c->newVisualization());
        CStopwatch sw;
        sw.start();
        if (_view && vis.empty()) {
            // nothing reads the fields between steps: velocity and density
            // are written on the last step only, and pairs of steps replay
            lbm_cu_domain_set_store_interval(_view, 0);
            runView(loops, true);
            lbm_cu_domain_set_store_interval(_view, 1);
        } else {
            for (int i = 0; i < loops; i++) {
                step();
                for (auto *v : vis) v->render(i);
            }
        }
        for (auto *c : _controllers) c->getSolver()->wait();
        sw.stop();
        for (auto *v : vis) delete v;  // waits for the last snapshots
        CController<T>::benchmarkRecord(loops, sw.time, cfg->do_visualization || cfg->debug_mode);
        CController<T>::report(_domain.getSize(), loops, sw.time, cfg->do_visualization || cfg->debug_mode);
    }

    CController<T> *getController() const { return _controllers.empty() ? nullptr : _controllers[_rank]; }
    CController<T> *getController(int id) const { return _controllers[id]; }
    int controllerCount() const { return (int)_controllers.size(); }
    void setController(CController<T> *c) {
        if (!_controllers.empty()) _controllers[_rank] = c;
    }
};

#endif
