// Random-row gather probe: the access pattern the check kernels are bound by,
// without the rule. Groups of 8 lanes each load one random 256-byte row (32
// bytes a lane, one 256-bit load), `depth` rows in flight per group, over a
// buffer of a given size; the rate at which rows arrive, for working sets
// that fit in L2 and for those that do not, is the ceiling a check pass can
// reach when each literal visit gathers one state row.
#include <stdint.h>

#include "common.h"

namespace gss {
namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

template <int K>
__global__ void __launch_bounds__(256) gather_probe_kernel(const uint32_t *__restrict__ buf, uint32_t n_rows,
                                                           uint32_t iters, uint32_t seed, uint32_t *__restrict__ sink) {
    const int sub = threadIdx.x & 7;
    const uint32_t grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    uint32_t acc = 0;
    for (uint32_t it = 0; it < iters; it++) {
        uint32_t v[K][8];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t row = mix32(grp * 0x9E3779B9U ^ (it * K + k) * 0x85ebca6bU ^ seed) % n_rows;
            const uint32_t *p = buf + (size_t) row * 64 + sub * 8;
            asm("ld.global.nc.L1::no_allocate.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=r"(v[k][0]), "=r"(v[k][1]), "=r"(v[k][2]), "=r"(v[k][3]), "=r"(v[k][4]), "=r"(v[k][5]),
                  "=r"(v[k][6]), "=r"(v[k][7])
                : "l"(p));
        }
#pragma unroll
        for (int k = 0; k < K; k++)
#pragma unroll
            for (int q = 0; q < 8; q++) acc ^= v[k][q];
    }
    if (acc == 0x9E3779B9U) sink[0] = acc;  // keeps the loads; practically never taken
}

template <int K>
int run_probe(const uint32_t *buf, uint32_t n_rows, uint32_t *sink, int grid, int iters, int reps, cudaStream_t st,
              float *ms) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GSS_CUDA_TRY(cudaEventCreate(&e0));
    GSS_CUDA_TRY(cudaEventCreate(&e1));
    for (int w = 0; w < 2; w++) gather_probe_kernel<K><<<grid, 256, 0, st>>>(buf, n_rows, iters, w, sink);
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; r++) gather_probe_kernel<K><<<grid, 256, 0, st>>>(buf, n_rows, iters, 100 + r, sink);
    cudaEventRecord(e1, st);
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    GSS_CUDA_TRY(e);
    GSS_CUDA_TRY(cudaGetLastError());
    *ms /= reps;
    return GSS_OK;
}

}  // namespace
}  // namespace gss

using namespace gss;

extern "C" int gss_probe_gather(int device, uint64_t buffer_bytes, int depth, int blocks_per_sm, double *rows_per_s,
                                double *ms_per_launch) {
    if (!rows_per_s || !ms_per_launch || buffer_bytes < 256 || buffer_bytes / 256 > 0xFFFFFFFFull ||
        (depth != 1 && depth != 2 && depth != 4) || blocks_per_sm < 1 || blocks_per_sm > 32)
        return set_error(GSS_ERR_INVALID, "gss_probe_gather: bad arguments");
    GSS_CUDA_TRY(cudaSetDevice(device));
    int sms = 0;
    GSS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const uint32_t n_rows = (uint32_t) (buffer_bytes / 256);
    uint32_t *buf = nullptr, *sink = nullptr;
    GSS_CUDA_TRY(cudaMalloc(&buf, (size_t) n_rows * 256));
    if (cudaMalloc(&sink, sizeof(uint32_t)) != cudaSuccess) {
        cudaFree(buf);
        return set_error(GSS_ERR_NOMEM, "gss_probe_gather: no room for the sink word");
    }
    int rc = GSS_OK;
    if (cudaMemset(buf, 1, (size_t) n_rows * 256) != cudaSuccess) rc = set_error(GSS_ERR_CUDA, "memset failed");
    const int grid = sms * blocks_per_sm, iters = 64, reps = 10;
    float ms = 0.f;
    if (rc == GSS_OK) {
        if (depth == 1) rc = run_probe<1>(buf, n_rows, sink, grid, iters, reps, 0, &ms);
        if (depth == 2) rc = run_probe<2>(buf, n_rows, sink, grid, iters, reps, 0, &ms);
        if (depth == 4) rc = run_probe<4>(buf, n_rows, sink, grid, iters, reps, 0, &ms);
    }
    cudaFree(buf);
    cudaFree(sink);
    if (rc != GSS_OK) return rc;
    const double rows = (double) grid * 256 / 8 * iters * depth;
    *ms_per_launch = ms;
    *rows_per_s = rows / (ms * 1e-3);
    return GSS_OK;
}
