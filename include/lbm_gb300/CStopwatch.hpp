// CStopwatch.hpp -- wall-clock stopwatch with the reference's interface
// (src/libtools/CStopwatch.hpp): start(), stop() accumulates into `time`.
#ifndef LBM_GB300_CSTOPWATCH_HPP
#define LBM_GB300_CSTOPWATCH_HPP

#include <chrono>

class CStopwatch {
    std::chrono::steady_clock::time_point t0_;

public:
    double time = 0.0;
    CStopwatch() { reset(); }
    void reset() { time = 0.0; }
    void start() { t0_ = std::chrono::steady_clock::now(); }
    void stop() { time += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count(); }
    double getTime() const { return time + std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count(); }
};

#endif
