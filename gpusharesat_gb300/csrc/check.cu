// The clause-check kernel: every clause of the database against every started
// assignment slot, reporting the slots where all literals are false or where
// exactly one is undefined and the rest are false.
//
// Rule (restated from gpuShareLib/GpuRunner.cu:34-57, ReportComputer): per
// 32-slot word, starting from the started slots,
//     oneUndef' = (allFalse & isUndef) | (oneUndef & isFalse)
//     allFalse' = allFalse & isFalse
//     report    = allFalse | oneUndef
// with the literal's value from the variable's {isDef, isTrue} word as in
// GpuRunner.cu:74-81. The scan of a clause stops once no slot can report
// (GpuRunner.cu:82-84). The reference walks one clause per thread and first
// tests a 32-bit cross-solver aggregate (GpuRunner.cu:152-170); here one warp
// walks one clause and each lane owns one 32-slot word, so the 32 lanes read a
// variable's state as one contiguous 256-byte row, and no prefilter is needed.
//
// Reports: each warp stages its records in shared memory and reserves room in
// global memory with one atomicAdd per flush on its block's partition
// counter (the reference does one atomicAdd per report, Reporter.cuh:41-49,
// and drops reports when a category is full; here nothing is dropped: a full
// partition keeps counting so the host sees the overflow and runs again).
#include "common.h"

namespace gss {

namespace {

constexpr int kWarps = 8;          // warps per block
constexpr int kStage = 128;        // staged records per warp
constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ void flush_stage(gss_report *stage, uint32_t n, gss_report *out,
                                            uint32_t *counter, uint32_t cap, int lane) {
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, n);
    base = __shfl_sync(kFull, base, 0);
    for (uint32_t i = lane; i < n; i += 32) {
        uint32_t idx = base + i;
        if (idx < cap) out[idx] = stage[i];
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kWarps * 32)
check_csr_kernel(CheckArgs a, uint32_t n_wblocks) {
    __shared__ gss_report stage_all[kWarps][kStage];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    gss_report *stage = stage_all[wib];
    const uint32_t part = blockIdx.x % a.n_parts;
    gss_report *out = a.out + (size_t) part * a.cap_per_part;
    uint32_t *counter = a.counts + part;
    uint32_t nstaged = 0;

    const uint64_t n_tasks = (uint64_t) a.n_clauses * n_wblocks;
    const uint64_t stride = (uint64_t) gridDim.x * kWarps;
    for (uint64_t task = (uint64_t) blockIdx.x * kWarps + wib; task < n_tasks; task += stride) {
        const uint32_t c = (uint32_t) (task / n_wblocks);
        const uint32_t wb = (uint32_t) (task - (uint64_t) c * n_wblocks);
        const uint32_t w = wb * 32 + lane;
        const bool active = w < a.n_words;
        uint32_t all_false = active ? __ldg(a.start + w) : 0u;
        uint32_t one_undef = 0;
        const int64_t b = __ldg(a.offsets + c);
        const int64_t e = __ldg(a.offsets + c + 1);
        for (int64_t base = b; base < e; base += 32) {
            const int32_t mine = (base + lane < e) ? __ldg(a.lits + base + lane) : 0;
            const int n = (int) min((int64_t) 32, e - base);
            bool alive = true;
            for (int k = 0; k < n; k++) {
                const uint32_t lit = (uint32_t) __shfl_sync(kFull, mine, k);
                if (all_false | one_undef) {
                    const uint2 st = __ldg(a.state + (size_t) (lit >> 1) * a.n_words + w);
                    const uint32_t f = ((lit & 1u) ? st.y : ~st.y) & st.x;
                    const uint32_t u = ~st.x;
                    one_undef = (all_false & u) | (one_undef & f);
                    all_false &= f;
                }
                if (!__any_sync(kFull, all_false | one_undef)) {
                    alive = false;
                    break;
                }
            }
            if (!alive) break;
        }
        const uint32_t rep = all_false | one_undef;
        const unsigned bal = __ballot_sync(kFull, rep != 0u);
        if (bal) {
            if (nstaged + 32 > (uint32_t) kStage) {
                flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane);
                nstaged = 0;
            }
            if (rep) {
                gss_report r;
                r.clause = c;
                r.word = w;
                r.mask = rep;
                r.solver = (uint32_t) __ldg(a.solver_of_word + w);
                stage[nstaged + __popc(bal & lanemask_lt())] = r;
            }
            nstaged += __popc(bal);
        }
    }
    if (nstaged) flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane);
}

}  // namespace

int launch_check(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    if (a.n_clauses == 0 || a.n_words == 0) return GSS_OK;
    const uint32_t n_wblocks = (a.n_words + 31) / 32;
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_csr_kernel, kWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    const uint64_t n_tasks = (uint64_t) a.n_clauses * n_wblocks;
    uint64_t blocks = (uint64_t) sm_count * per_sm;
    const uint64_t need = (n_tasks + kWarps - 1) / kWarps;
    if (blocks > need) blocks = need;
    check_csr_kernel<<<(unsigned) blocks, kWarps * 32, 0, stream>>>(a, n_wblocks);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

}  // namespace gss
