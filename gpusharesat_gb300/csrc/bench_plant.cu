// Workload helper of the learned-order measurement: plants reports into a
// device-resident assignment state at per-clause rates, and puts the state
// back afterwards. Not used by the check path itself.
#include <stdint.h>

#include "common.h"

namespace gss {
namespace {

__device__ __forceinline__ uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void plant_kernel(const int32_t *__restrict__ lits, const int64_t *__restrict__ offsets, uint64_t n,
                             const float *__restrict__ rate, uint32_t *__restrict__ state,
                             const uint32_t *__restrict__ base, uint64_t n_vars, uint32_t n_words, uint64_t seed,
                             uint64_t pass, int restore) {
    for (uint64_t c = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (uint64_t) gridDim.x * blockDim.x) {
        const uint64_t h = mix(seed ^ mix(pass * 0x9E3779B97F4A7C15ull + c));
        const float u = (float) (h >> 40) * (1.0f / 16777216.0f);
        if (!(u < rate[c])) continue;
        const uint64_t h2 = mix(h + 0x632BE59BD9B4E019ull);
        const uint32_t w = (uint32_t) (h2 % n_words);
        const uint32_t bit = 1u << ((h2 >> 32) & 31u);
        const int64_t b0 = offsets[c], b1 = offsets[c + 1];
        for (int64_t k = b0; k < b1; k++) {
            const uint32_t lit = (uint32_t) lits[k];
            const uint64_t v = lit >> 1;
            if (v >= n_vars) continue;
            uint32_t *word = state + (v * n_words + w) * 2;
            if (restore) {
                const uint32_t *bw = base + (v * n_words + w) * 2;
                word[0] = bw[0];
                word[1] = bw[1];
            } else if (k + 1 < b1) {
                // false in the slot: assigned, true exactly for a negative literal
                atomicOr(word, bit);
                if (lit & 1u)
                    atomicOr(word + 1, bit);
                else
                    atomicAnd(word + 1, ~bit);
            } else {
                atomicAnd(word, ~bit);  // the last literal: unassigned
            }
        }
    }
}

}  // namespace
}  // namespace gss

using namespace gss;

extern "C" int gss_bench_plant(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, const float *rate,
                               uint32_t *state, const uint32_t *base, int64_t n_vars, int n_words, uint64_t seed,
                               int64_t pass, int restore, void *stream) {
    if (n_clauses < 0 || n_vars < 0 || n_words < 1 || pass < 0 ||
        (n_clauses > 0 && (!lits || !offsets || !rate || !state || (restore && !base))))
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_bench_plant");
    if (n_clauses == 0) return GSS_OK;
    int dev = 0, sm = 0;
    GSS_CUDA_TRY(cudaGetDevice(&dev));
    GSS_CUDA_TRY(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    uint64_t blocks = ((uint64_t) n_clauses + 255) / 256;
    if (blocks > (uint64_t) sm * 8) blocks = (uint64_t) sm * 8;
    plant_kernel<<<(unsigned) blocks, 256, 0, (cudaStream_t) stream>>>(
        lits, offsets, (uint64_t) n_clauses, rate, state, base, (uint64_t) n_vars, (uint32_t) n_words, seed,
        (uint64_t) pass, restore);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}
