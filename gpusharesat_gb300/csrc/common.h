// Internal helpers shared by the engine, the kernels and the clause sharer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "gpusharesat.h"

namespace gss {

// Longest clause the engine accepts. The reference stops at 100
// (MAX_CL_SIZE, gpuShareLib/BaseTypes.cuh:28); the sharer keeps that limit
// by default, the engine itself takes clauses up to this length.
constexpr int kMaxClauseLen = 4096;

// Sets the calling thread's error message and returns `code`.
int set_error(int code, const char *fmt, ...);

// Checks a CUDA call; on failure records the message and returns GSS_ERR_CUDA.
#define GSS_CUDA_TRY(call)                                                        \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) {                                                  \
            return ::gss::set_error(GSS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, \
                                    cudaGetErrorString(_e), __FILE__, __LINE__);  \
        }                                                                         \
    } while (0)

#define GSS_TRY(expr)          \
    do {                       \
        int _rc = (expr);      \
        if (_rc != GSS_OK) {   \
            return _rc;        \
        }                      \
    } while (0)

// A device buffer that grows by doubling and never shrinks.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need);  // keeps nothing of the old contents
    int grow_keep(size_t need, cudaStream_t stream, size_t keep_bytes);
    void release();
    ~DevBuf() { release(); }
};

struct PinnedBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need);
    void release();
    ~PinnedBuf() { release(); }
};

// Arguments of one check pass over a CSR clause database.
struct CheckArgs {
    const int32_t *lits;        // device, CSR literals
    const int64_t *offsets;     // device, n_clauses + 1
    uint32_t n_clauses;
    const uint2 *state;         // device, [n_vars][n_words] {isDef, isTrue}
    uint32_t n_words;
    const uint32_t *start;      // device, [n_words]
    const int32_t *solver_of_word;  // device, [n_words]
    gss_report *out;            // device, n_parts * cap_per_part records
    uint32_t *counts;           // device, n_parts counters (zeroed by the caller)
    uint32_t n_parts;
    uint32_t cap_per_part;
};

// Launches the check kernel on `stream` (the counters must already be zero).
// Returns a GSS status.
int launch_check(const CheckArgs &a, cudaStream_t stream, int sm_count);

}  // namespace gss
