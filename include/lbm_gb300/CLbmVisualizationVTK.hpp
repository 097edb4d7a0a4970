// CLbmVisualizationVTK.hpp -- VTK snapshots of one subdomain
// (src/libvis/ILbmVisualization.hpp:1-54, src/libvis/CLbmVisualizationVTK.hpp:8-99):
// the same class names, constructor (UID, file name), setup(solver) and
// render(increment), the same files "<file>.<UID>.<increment>.vtk" and the
// same ASCII content (VTK_Common.hpp).
//
// render() reads velocity, density and flags from the device (the solver
// must store velocity and density, as the reference requires) and hands the
// host copies to a writer thread, so the time loop steps on while the text
// is formatted (by all host cores) and written; at most one snapshot waits
// behind the one being written, which bounds the host memory to three
// copies of the fields.  finish() (and the destructor) wait for the writes.
#ifndef LBM_GB300_CLBMVISUALIZATIONVTK_HPP
#define LBM_GB300_CLBMVISUALIZATIONVTK_HPP

#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "CLbmSolver.hpp"
#include "VTK_Common.hpp"

template <typename T>
class ILbmVisualization {
protected:
    T *velocity = nullptr;
    T *density = nullptr;
    int *flags = nullptr;
    CLbmSolver<T> *cLbmOpencl = nullptr;

public:
    virtual ~ILbmVisualization() {
        delete[] velocity;
        delete[] density;
        delete[] flags;
    }
    virtual void setup(CLbmSolver<T> *p_cLbmOpencl) {
        cLbmOpencl = p_cLbmOpencl;
        const size_t n = (size_t)cLbmOpencl->domain_cells.elements();
        delete[] velocity;
        velocity = new T[n * 3];
        delete[] density;
        density = new T[n];
        delete[] flags;
        flags = new int[n];
    }
    virtual void render(int increment = -1) = 0;
};

template <typename T>
class CLbmVisualizationVTK : virtual public ILbmVisualization<T> {
    struct Snapshot {
        std::string path;
        CVector<3, int> cells, origin;
        T dx;
        std::vector<T> vel, rho;
        std::vector<int> fl;
    };
    int _UID;
    std::string _file_name;
    int _timeStepNumber = -1;
    bool _async = true;
    unsigned _threads;
    std::mutex _m;
    std::condition_variable _cv;
    std::deque<Snapshot> _queue;
    bool _busy = false, _stop = false, _failed = false;
    std::thread _writer;

    void write(const Snapshot &s) {
        const bool ok = lbm_vtk::write_vtk_cells<T>(s.path.c_str(), s.cells[0], s.cells[1], s.cells[2], s.dx,
                                                    s.origin, s.rho.data(), s.fl.data(), s.vel.data(), _threads);
        if (!ok) {
            fprintf(stderr, "Failed to write %s\n", s.path.c_str());
            std::lock_guard<std::mutex> g(_m);
            _failed = true;
        }
    }
    void loop() {
        for (;;) {
            Snapshot s;
            {
                std::unique_lock<std::mutex> g(_m);
                _cv.wait(g, [&] { return _stop || !_queue.empty(); });
                if (_queue.empty()) return;
                s = std::move(_queue.front());
                _queue.pop_front();
                _busy = true;
            }
            _cv.notify_all();
            write(s);
            {
                std::lock_guard<std::mutex> g(_m);
                _busy = false;
            }
            _cv.notify_all();
        }
    }

public:
    CLbmVisualizationVTK(int UID, std::string file_name) : _UID(UID), _file_name(file_name) {
        _threads = std::max(1u, std::thread::hardware_concurrency());
    }
    ~CLbmVisualizationVTK() {
        finish();
        {
            std::lock_guard<std::mutex> g(_m);
            _stop = true;
        }
        _cv.notify_all();
        if (_writer.joinable()) _writer.join();
    }

    /** Write in the calling thread (false) or behind the time loop (true, default). */
    void setAsync(bool async) { _async = async; }
    /** Host threads that format the text (default: all). */
    void setThreads(unsigned n) { _threads = std::max(1u, n); }
    /** true once a file could not be written */
    bool failed() {
        std::lock_guard<std::mutex> g(_m);
        return _failed;
    }

    void setup(CLbmSolver<T> *p_cLbmOpencl) { ILbmVisualization<T>::setup(p_cLbmOpencl); }

    void render(int increment = -1) {
        _timeStepNumber = increment;
        CLbmSolver<T> *s = this->cLbmOpencl;
        const size_t n = (size_t)s->domain_cells.elements();
        s->storeVelocity(this->velocity);
        s->storeDensity(this->density);
        s->storeFlags(this->flags);
        Snapshot snap;
        char name[4096];
        snprintf(name, sizeof(name), "%s.%i.%i.vtk", _file_name.c_str(), _UID, _timeStepNumber);
        snap.path = name;
        snap.cells = s->domain_cells;
        snap.origin = s->domain.getOrigin();
        snap.dx = s->d_cell_length;
        snap.vel.assign(this->velocity, this->velocity + 3 * n);
        snap.rho.assign(this->density, this->density + n);
        snap.fl.assign(this->flags, this->flags + n);
        if (!_async) {
            write(snap);
            return;
        }
        std::unique_lock<std::mutex> g(_m);
        if (!_writer.joinable()) _writer = std::thread([this] { loop(); });
        _cv.wait(g, [&] { return _queue.empty(); });  // at most one snapshot waits
        _queue.push_back(std::move(snap));
        g.unlock();
        _cv.notify_all();
    }

    /** Wait until every rendered snapshot is on disk. */
    void finish() {
        std::unique_lock<std::mutex> g(_m);
        _cv.wait(g, [&] { return _queue.empty() && !_busy; });
    }
};

#endif
