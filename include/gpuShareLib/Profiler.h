// TimeGauge: adds the microseconds between its construction and complete()
// (or destruction) to a counter, when enabled (the reference's
// gpuShareLib/Profiler.h:28-46, used by its callers).
#ifndef GPUSHARESAT_GB300_PROFILER_H
#define GPUSHARESAT_GB300_PROFILER_H

#include "Utils.h"

namespace GpuShare {

class TimeGauge {
public:
    TimeGauge(unsigned long &counter, bool enabled) : counter_(counter), start_(enabled ? realTimeMicros() : -1) {}
    void complete() {
        if (start_ >= 0) counter_ += (unsigned long) (realTimeMicros() - start_);
        start_ = -1;
    }
    ~TimeGauge() { complete(); }

private:
    unsigned long &counter_;
    long start_;
};

}  // namespace GpuShare

#endif
