// make_unique for C++11 callers (the solvers that use the sharer include it,
// gpuShareLib/my_make_unique.h in the reference).
#ifndef GPUSHARESAT_GB300_MY_MAKE_UNIQUE_H
#define GPUSHARESAT_GB300_MY_MAKE_UNIQUE_H

#include <memory>
#include <utility>

template <typename T, typename... Args>
std::unique_ptr<T> my_make_unique(Args &&...args) {
    return std::unique_ptr<T>(new T(std::forward<Args>(args)...));
}

#endif
