// Bucketed persistent check kernel: one launch over the whole scan, where
// each range of scan positions (a length class of the length-sorted
// database) is checked with its own lane layout: words per lane x lanes per
// clause = 32 (one 32-word state row per slot block, the layout of the wide
// kinds), and the loads in flight. The ranges and their layouts come from an
// autotuner; the rule and the report records are those of check_wide_kernel.
//
// Tasks are (slot block, clause group of one range) pairs, slot block
// outermost as in the other kernels, taken in chunks from a device work
// counter. A task finds its range by binary search over the ranges' first
// group indices, then runs the body compiled for that range's layout.
#include <stdint.h>

#include "common.h"

namespace gss {
namespace {

constexpr int kWarps = 8;
constexpr int kStage = 128;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kTaskChunk = 4;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <int WPL>
struct Row {
    uint32_t v[2 * WPL];
};

template <int WPL>
__device__ __forceinline__ void ld_row(const uint2 *p, Row<WPL> &r);
template <>
__device__ __forceinline__ void ld_row<1>(const uint2 *p, Row<1> &r) {
    asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(r.v[0]), "=r"(r.v[1]) : "l"(p));
}
template <>
__device__ __forceinline__ void ld_row<2>(const uint2 *p, Row<2> &r) {
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]) : "l"(p));
}
template <>
__device__ __forceinline__ void ld_row<4>(const uint2 *p, Row<4> &r) {
    asm("ld.global.nc.L1::no_allocate.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]),
          "=r"(r.v[7])
        : "l"(p));
}

__device__ __forceinline__ void flush(gss_report *stage, uint32_t n, gss_report *out, uint32_t *counter, uint32_t cap,
                                      int lane) {
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, n);
    base = __shfl_sync(kFull, base, 0);
    for (uint32_t i = lane; i < n; i += 32) {
        const uint32_t idx = base + i;
        if (idx < cap) out[idx] = stage[i];
    }
    __syncwarp();
}

struct WarpOut {
    gss_report *stage;
    gss_report *out;
    uint32_t *counter;
    uint32_t nstaged;
};

// One task: clause group g of range [rb, re) against slot block blk.
template <int WPL, int LPC, int G>
__device__ __forceinline__ void range_task(const CheckArgs &a, uint32_t blk, uint32_t rb, uint32_t re, uint32_t g,
                                           WarpOut &wo) {
    static_assert(WPL * LPC == 32, "one 32-word row per slot block");
    constexpr int CPW = 32 / LPC;
    constexpr int BW = 32;
    const int lane = threadIdx.x & 31;
    const int sub = lane % LPC;
    const int grp = lane / LPC;
    const int gbase = grp * LPC;
    const uint32_t p = rb + g * CPW + grp;
    const uint32_t c = p < re ? ((a.perm && p < a.perm_end) ? __ldg(a.perm + p) : p) : 0xFFFFFFFFu;
    const bool valid = c < a.n_clauses && clause_live(a, c);
    const uint32_t w0 = blk * BW + sub * WPL;
    uint32_t af[WPL], ou[WPL];
#pragma unroll
    for (int j = 0; j < WPL; j++) {
        af[j] = valid ? __ldg(a.start + w0 + j) : 0u;
        ou[j] = 0u;
    }
    uint32_t pos = 0, end = 0;
    if (valid) {
        pos = (uint32_t) __ldg(a.offsets + c);
        end = (uint32_t) __ldg(a.offsets + c + 1);
    }
    const uint2 *rows = a.state + (size_t) blk * a.n_vars * BW + sub * WPL;
    while (true) {
        bool alive = false;
#pragma unroll
        for (int j = 0; j < WPL; j++) alive |= (af[j] | ou[j]) != 0u;
        if (!__any_sync(kFull, alive && pos < end)) break;
        const int32_t chunk = (pos + sub < end) ? __ldg(a.lits + pos + sub) : 0;
        const int navail = (int) min((uint32_t) LPC, end > pos ? end - pos : 0u);
#pragma unroll 1
        for (int k0 = 0; k0 < LPC; k0 += G) {
            alive = false;
#pragma unroll
            for (int j = 0; j < WPL; j++) alive |= (af[j] | ou[j]) != 0u;
            if (!__any_sync(kFull, alive && k0 < navail)) break;
            uint32_t lit[G];
            Row<WPL> st[G];
#pragma unroll
            for (int i = 0; i < G; i++) lit[i] = (uint32_t) __shfl_sync(kFull, chunk, gbase + k0 + i);
#pragma unroll
            for (int i = 0; i < G; i++) {
#pragma unroll
                for (int q = 0; q < 2 * WPL; q++) st[i].v[q] = 0u;
                if (alive && k0 + i < navail) ld_row<WPL>(rows + (size_t) (lit[i] >> 1) * BW, st[i]);
            }
#pragma unroll
            for (int i = 0; i < G; i++) {
                if (k0 + i < navail) {
                    const bool neg = (lit[i] & 1u) != 0u;
#pragma unroll
                    for (int j = 0; j < WPL; j++) {
                        const uint32_t d = st[i].v[2 * j], t = st[i].v[2 * j + 1];
                        const uint32_t f = (neg ? t : ~t) & d;
                        ou[j] = (af[j] & ~d) | (ou[j] & f);
                        af[j] &= f;
                    }
                }
            }
        }
        pos += LPC;
    }
#pragma unroll
    for (int j = 0; j < WPL; j++) {
        const uint32_t rep = af[j] | ou[j];
        const unsigned bal = __ballot_sync(kFull, rep != 0u);
        if (bal) {
            if (wo.nstaged + 32 > (uint32_t) kStage) {
                flush(wo.stage, wo.nstaged, wo.out, wo.counter, a.cap_per_part, lane);
                wo.nstaged = 0;
            }
            if (rep) {
                gss_report r;
                r.clause = __ldg(a.orig + c);
                r.word = w0 + j;
                r.mask = rep;
                r.solver = (uint32_t) __ldg(a.solver_of_word + w0 + j);
                wo.stage[wo.nstaged + __popc(bal & lanemask_lt())] = r;
            }
            wo.nstaged += __popc(bal);
        }
    }
}

__global__ void __launch_bounds__(kWarps * 32, 6) check_bucketed_kernel(const CheckArgs *__restrict__ pa,
                                                                        const BucketPlan *__restrict__ plan,
                                                                        uint32_t *__restrict__ work) {
    __shared__ CheckArgs sa;
    __shared__ gss_report stage_all[kWarps][kStage];
    if (threadIdx.x == 0) sa = *pa;
    __syncthreads();
    const CheckArgs &a = sa;
    const int lane = threadIdx.x & 31;
    WarpOut wo;
    wo.stage = stage_all[threadIdx.x >> 5];
    const uint32_t part = blockIdx.x % a.n_parts;
    wo.out = a.out + (size_t) part * a.cap_per_part;
    wo.counter = a.counts + part;
    wo.nstaged = 0;
    const uint32_t n_ranges = plan->n_ranges;
    const uint32_t groups = plan->group_base[n_ranges];  // clause groups over all ranges
    const uint64_t n_tasks = (uint64_t) groups * a.n_blocks;
    while (true) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(work, kTaskChunk);
        first = __shfl_sync(kFull, first, 0);
        if ((uint64_t) first >= n_tasks) break;
        const uint64_t last = min((uint64_t) first + kTaskChunk, n_tasks);
        for (uint64_t task = first; task < last; task++) {
            const uint32_t blk = (uint32_t) (task / groups);
            const uint32_t gg = (uint32_t) (task - (uint64_t) blk * groups);
            // the range holding clause group gg: last k with group_base[k] <= gg
            uint32_t lo = 0, hi = n_ranges - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (__ldg(plan->group_base + mid) <= gg)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const uint32_t k = lo;
            const uint32_t g = gg - __ldg(plan->group_base + k);
            const uint32_t rb = __ldg(plan->range_begin + k), re = __ldg(plan->range_end + k);
            switch (__ldg(plan->layout + k)) {
                case GSS_LAYOUT_4x8_G1: range_task<4, 8, 1>(a, blk, rb, re, g, wo); break;
                case GSS_LAYOUT_4x8_G2: range_task<4, 8, 2>(a, blk, rb, re, g, wo); break;
                case GSS_LAYOUT_2x16_G1: range_task<2, 16, 1>(a, blk, rb, re, g, wo); break;
                case GSS_LAYOUT_2x16_G2: range_task<2, 16, 2>(a, blk, rb, re, g, wo); break;
                case GSS_LAYOUT_1x32_G1: range_task<1, 32, 1>(a, blk, rb, re, g, wo); break;
                case GSS_LAYOUT_1x32_G2: range_task<1, 32, 2>(a, blk, rb, re, g, wo); break;
                default: break;
            }
        }
    }
    if (wo.nstaged) flush(wo.stage, wo.nstaged, wo.out, wo.counter, a.cap_per_part, lane);
}

}  // namespace

int layout_lanes(int layout) {
    switch (layout) {
        case GSS_LAYOUT_4x8_G1:
        case GSS_LAYOUT_4x8_G2: return 8;
        case GSS_LAYOUT_2x16_G1:
        case GSS_LAYOUT_2x16_G2: return 16;
        case GSS_LAYOUT_1x32_G1:
        case GSS_LAYOUT_1x32_G2: return 32;
        default: return 0;
    }
}

int launch_check_bucketed(const CheckArgs *d_args, const BucketPlan *d_plan, uint32_t *work, cudaStream_t stream,
                          int sm_count) {
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_bucketed_kernel, kWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    check_bucketed_kernel<<<(unsigned) (sm_count * per_sm), kWarps * 32, 0, stream>>>(d_args, d_plan, work);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

}  // namespace gss
