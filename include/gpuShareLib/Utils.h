// Logging helpers the sharer's callers use (the reference's
// gpuShareLib/Utils.h:128-154): a Logger with a verbosity and an output
// function, the LOG macro, directPrint and a wall clock in microseconds.
// The solvers also rely on what this header brings in (the reference's
// gpuShareLib/Utils.h:22-30): the assertion macros and <mutex>, <atomic>,
// <memory> and <time.h>.
#ifndef GPUSHARESAT_GB300_UTILS_H
#define GPUSHARESAT_GB300_UTILS_H

#include <sys/time.h>
#include <time.h>

#include <atomic>
#include <functional>
#include <iostream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>

#include "Assert.h"

namespace GpuShare {

inline long realTimeMicros() {
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (long) tv.tv_sec * 1000000L + tv.tv_usec;
}

inline void directPrint(const std::string &str) { std::cout << str; }

struct Logger {
    int verb;
    std::function<void(const std::string &str)> logFunc;
};

}  // namespace GpuShare

// Formats `expr` (an ostream expression) and passes it to the logger when its
// verbosity is at least `level`.
#define LOG(logger_, level_, expr_)                  \
    {                                                \
        if ((logger_).verb >= (level_)) {            \
            std::ostringstream gss_log_stream_;      \
            gss_log_stream_ << expr_;                \
            (logger_).logFunc(gss_log_stream_.str()); \
        }                                            \
    }

#endif
