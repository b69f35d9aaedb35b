// The clause-check kernels: every clause of the database against every started
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
// (GpuRunner.cu:82-84).
//
// Mapping. The reference walks one clause per thread and first tests a 32-bit
// cross-solver aggregate (GpuRunner.cu:152-170), then each solver's words
// one by one. Here a group of LPC lanes walks one clause and each lane owns one
// 32-slot word of a "slot block" of LPC words; a warp holds 32/LPC clauses of
// equal or similar length (the database is sorted by length, like the
// reference's per-size buckets, Clauses.cu:47-126). The state of one slot block
// is stored block-major, [block][var][LPC words]{isDef,isTrue}, so a group reads
// a variable's LPC words as one contiguous run of 8*LPC bytes, and the blocks
// are scanned one after another so that the block being scanned can stay
// resident in L2 while the clause literals stream past it (evict-first hint).
// No prefilter is needed: a lane that has no slot left stops loading, and a
// group stops reading literals once all its lanes are done.
//
// Memory-level parallelism: a group issues the state loads of G literals
// before it consumes any of them (lanes that die inside the G are harmless: the
// loaded words are simply not used), so a warp has up to G independent
// gathers in flight instead of one.
//
// Reports: each warp stages its records in shared memory and reserves room in
// global memory with one atomicAdd per flush on its block's partition counter.
// The reference does one atomicAdd per report and drops reports when a
// category is full (Reporter.cuh:41-49); here nothing is dropped: a full
// partition keeps counting, so the host sees the overflow and runs again.
#include <string.h>


#include "common.h"

namespace gss {

namespace {

constexpr int kWarps = 8;     // warps per block
constexpr int kStage = 128;   // staged records per warp
constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// L2 eviction-priority policies (createpolicy): the slot block's state is
// kept (evict-last), the clause literals stream past it (evict-first).
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// State gather: read-only, no L1 allocation (random rows are not reused
// within an SM), with the L2 policy when hints are on.
__device__ __forceinline__ uint2 ld_state(const uint2 *p, bool hint, uint64_t pol) {
    uint2 v;
    if (hint) {
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
            : "=r"(v.x), "=r"(v.y) : "l"(p), "l"(pol));
    } else {
        asm("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    }
    return v;
}

__device__ __forceinline__ int32_t ld_lit(const int32_t *p, bool hint, uint64_t pol) {
    int32_t v;
    if (hint) {
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    } else {
        asm("ld.global.nc.s32 %0, [%1];" : "=r"(v) : "l"(p));
    }
    return v;
}

// Writes a warp's staged records: one atomic reservation, then the records.
// streaming = cache-streaming stores (the records are read back by the host,
// not by the kernel: they need not displace state rows from L2).
__device__ __forceinline__ void flush_stage(gss_report *stage, uint32_t n, gss_report *out, uint32_t *counter,
                                            uint32_t cap, int lane, bool streaming = false) {
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, n);
    base = __shfl_sync(kFull, base, 0);
    for (uint32_t i = lane; i < n; i += 32) {
        uint32_t idx = base + i;
        if (idx < cap) {
            if (streaming)
                __stcs(reinterpret_cast<int4 *>(out + idx), *reinterpret_cast<const int4 *>(stage + i));
            else
                out[idx] = stage[i];
        }
    }
    __syncwarp();
}

template <int LPC, int G>
__global__ void __launch_bounds__(kWarps * 32) check_kernel(CheckArgs a) {
    static_assert(LPC == 1 || LPC == 2 || LPC == 4 || LPC == 8 || LPC == 16 || LPC == 32, "lanes per clause");
    static_assert(G >= 1 && G <= LPC, "prefetch depth");
    constexpr int CPW = 32 / LPC;  // clauses per warp
    __shared__ gss_report stage_all[kWarps][kStage];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int sub = lane % LPC;     // word within the slot block
    const int grp = lane / LPC;     // clause within the warp
    const int gbase = grp * LPC;    // first lane of this clause group
    gss_report *stage = stage_all[wib];
    const uint32_t part = blockIdx.x % a.n_parts;
    gss_report *out = a.out + (size_t) part * a.cap_per_part;
    uint32_t *counter = a.counts + part;
    uint32_t nstaged = 0;
    const bool hint = a.cache_hints != 0;
    const uint64_t pol_keep = policy_evict_last();
    const uint64_t pol_stream = policy_evict_first();

    const uint32_t n_scan = scan_count(a);
    const uint32_t n_groups = (n_scan + CPW - 1) / CPW;
    const uint64_t n_tasks = (uint64_t) n_groups * a.n_blocks;
    const uint64_t stride = (uint64_t) gridDim.x * kWarps;
    for (uint64_t task = (uint64_t) blockIdx.x * kWarps + wib; task < n_tasks; task += stride) {
        // Slot block outermost: all warps sweep block 0 first, then block 1...
        const uint32_t blk = (uint32_t) (task / n_groups);
        const uint32_t g = (uint32_t) (task - (uint64_t) blk * n_groups);
        const uint32_t i = g * CPW + grp;
        const uint32_t c = i < n_scan ? scan_clause(a, i) : 0xFFFFFFFFu;
        const bool valid = c < a.n_clauses && clause_live(a, c);
        const uint32_t w = blk * LPC + sub;
        uint32_t all_false = valid ? __ldg(a.start + w) : 0u;  // start is padded to n_blocks*LPC
        uint32_t one_undef = 0;
        int64_t pos = 0, end = 0;
        if (valid) {
            pos = __ldg(a.offsets + c);
            end = __ldg(a.offsets + c + 1);
        }
        const uint2 *rows = a.state + (size_t) blk * a.n_vars * LPC + sub;
        while (true) {
            const bool mine = (all_false | one_undef) != 0u && pos < end;
            const unsigned live = __ballot_sync(kFull, mine);
            if (live == 0u) break;
            // LPC literals of this clause, one per lane of the group.
            const int32_t chunk = (pos + sub < end) ? ld_lit(a.lits + pos + sub, hint, pol_stream) : 0;
            const int navail = (int) min((int64_t) LPC, end - pos);
#pragma unroll 1
            for (int k0 = 0; k0 < LPC; k0 += G) {
                // Groups that are done idle (no loads) until the whole warp is done.
                if (!__any_sync(kFull, (all_false | one_undef) != 0u && k0 < navail)) break;
                uint32_t lit[G];
                uint2 st[G];
#pragma unroll
                for (int j = 0; j < G; j++) {
                    lit[j] = (uint32_t) __shfl_sync(kFull, chunk, gbase + k0 + j);
                }
                const bool alive = (all_false | one_undef) != 0u;
#pragma unroll
                for (int j = 0; j < G; j++) {
                    st[j] = make_uint2(0u, 0u);
                    if (alive && k0 + j < navail) st[j] = ld_state(rows + (size_t) (lit[j] >> 1) * LPC, hint, pol_keep);
                }
#pragma unroll
                for (int j = 0; j < G; j++) {
                    if (k0 + j < navail) {
                        const uint32_t f = ((lit[j] & 1u) ? st[j].y : ~st[j].y) & st[j].x;
                        const uint32_t u = ~st[j].x;
                        one_undef = (all_false & u) | (one_undef & f);
                        all_false &= f;
                    }
                }
            }
            pos += LPC;
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
                r.clause = __ldg(a.orig + c);
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


// Wide variant: each lane owns WPL consecutive 32-slot words (WPL = 4: one
// 256-bit load of {isDef, isTrue} x 4 per literal), a group of LPC lanes owns
// a clause, and the slot block is LPC * WPL words. With WPL = 4 and LPC = 8 a
// warp checks 4 clauses against all 1024 slots of a 32-word pass with one
// load instruction per literal step: 4 rows of 256 contiguous bytes.
template <int WPL>
struct Row;
template <>
struct Row<1> {
    uint32_t v[2];
};
template <>
struct Row<2> {
    uint32_t v[4];
};
template <>
struct Row<4> {
    uint32_t v[8];
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

// The same gathers with an L2 eviction policy (cache_hints on).
template <int WPL>
__device__ __forceinline__ void ld_row_hint(const uint2 *p, Row<WPL> &r, uint64_t pol);
template <>
__device__ __forceinline__ void ld_row_hint<1>(const uint2 *p, Row<1> &r, uint64_t pol) {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
        : "=r"(r.v[0]), "=r"(r.v[1]) : "l"(p), "l"(pol));
}
template <>
__device__ __forceinline__ void ld_row_hint<2>(const uint2 *p, Row<2> &r, uint64_t pol) {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]) : "l"(p), "l"(pol));
}
template <>
__device__ __forceinline__ void ld_row_hint<4>(const uint2 *p, Row<4> &r, uint64_t pol) {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8], %9;"
        : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]),
          "=r"(r.v[7])
        : "l"(p), "l"(pol));
}

// Register cap of the wide kernels without the occupancy flag. With four
// words per lane and at most two loads in flight, six blocks of 256 threads
// per SM (40 registers a thread, a few bytes of spills) keep 48 warps of
// gathers in flight instead of 32 at the uncapped 64 registers; measured on
// GB300 on the at-scale workload, the pass takes about 10% less time. Deeper
// variants need their registers for the rows in flight and stay uncapped.
constexpr int default_min_blocks(int wpl, int g) { return (wpl == 4 && g <= 2) ? 6 : 1; }

// MAP_IDS = false: reports carry the clause's CSR index itself (a.orig unused).
// With cache_hints: state rows evict-last in L2, clause literals evict-first,
// report records streamed.
template <int WPL, int LPC, int G, int MINB, bool MAP_IDS = true, bool HINT = false>
__global__ void __launch_bounds__(kWarps * 32, MINB) check_wide_kernel(CheckArgs a) {
    constexpr int CPW = 32 / LPC;
    constexpr int BW = WPL * LPC;
    static_assert(G >= 1 && G <= LPC, "depth");
    __shared__ gss_report stage_all[kWarps][kStage];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int sub = lane % LPC;
    const int grp = lane / LPC;
    const int gbase = grp * LPC;
    gss_report *stage = stage_all[wib];
    const uint32_t part = blockIdx.x % a.n_parts;
    gss_report *out = a.out + (size_t) part * a.cap_per_part;
    uint32_t *counter = a.counts + part;
    uint32_t nstaged = 0;
    constexpr bool hint = HINT;
    const uint64_t pol_keep = hint ? policy_evict_last() : 0ull;
    const uint64_t pol_stream = hint ? policy_evict_first() : 0ull;

    const uint32_t n_scan = scan_count(a);
    const uint32_t n_groups = (n_scan + CPW - 1) / CPW;
    const uint64_t n_tasks = (uint64_t) n_groups * a.n_blocks;
    const uint64_t stride = (uint64_t) gridDim.x * kWarps;
    // the state rows of the literals in flight: zeroed once; a lane that is
    // done loads nothing and its all-zero masks ignore what the rows hold
    Row<WPL> st[G];
#pragma unroll
    for (int i = 0; i < G; i++)
#pragma unroll
        for (int q = 0; q < 2 * WPL; q++) st[i].v[q] = 0u;
    for (uint64_t task = (uint64_t) blockIdx.x * kWarps + wib; task < n_tasks; task += stride) {
        const uint32_t blk = (uint32_t) (task / n_groups);
        const uint32_t g = (uint32_t) (task - (uint64_t) blk * n_groups);
        const uint32_t i = g * CPW + grp;
        const uint32_t c = i < n_scan ? scan_clause(a, i) : 0xFFFFFFFFu;
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
            const int32_t chunk = (pos + sub < end) ? ld_lit(a.lits + pos + sub, hint, pol_stream) : 0;
            const int navail = (int) min((uint32_t) LPC, end > pos ? end - pos : 0u);
#pragma unroll 1
            for (int k0 = 0; k0 < LPC; k0 += G) {
                alive = false;
#pragma unroll
                for (int j = 0; j < WPL; j++) alive |= (af[j] | ou[j]) != 0u;
                if (!__any_sync(kFull, alive && k0 < navail)) break;
                uint32_t lit[G];
#pragma unroll
                for (int i = 0; i < G; i++) lit[i] = (uint32_t) __shfl_sync(kFull, chunk, gbase + k0 + i);
#pragma unroll
                for (int i = 0; i < G; i++) {
                    if (alive && k0 + i < navail) {
                        if (hint)
                            ld_row_hint<WPL>(rows + (size_t) (lit[i] >> 1) * BW, st[i], pol_keep);
                        else
                            ld_row<WPL>(rows + (size_t) (lit[i] >> 1) * BW, st[i]);
                    }
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
                if (nstaged + 32 > (uint32_t) kStage) {
                    flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane, hint);
                    nstaged = 0;
                }
                if (rep) {
                    gss_report r;
                    r.clause = MAP_IDS ? __ldg(a.orig + c) : c;
                    r.word = w0 + j;
                    r.mask = rep;
                    r.solver = (uint32_t) __ldg(a.solver_of_word + w0 + j);
                    stage[nstaged + __popc(bal & lanemask_lt())] = r;
                }
                nstaged += __popc(bal);
            }
        }
    }
    if (nstaged) flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane, hint);
}

// Pipelined wide variant: the same schedule and rule as check_wide_kernel,
// with the loads a clause waits on before its first state gather moved off
// its critical path. The next task's offsets are loaded when a task starts,
// its first literal chunk after the task's first gather round, and a long
// clause's next chunk while its current chunk is being checked. All these
// loads are in bounds (guarded like the ones they replace) and at most one
// chunk ahead.
template <int WPL, int LPC, int G, int MINB>
__global__ void __launch_bounds__(kWarps * 32, MINB) check_wide_pf_kernel(CheckArgs a) {
    constexpr int CPW = 32 / LPC;
    constexpr int BW = WPL * LPC;
    static_assert(G >= 1 && G <= LPC, "depth");
    __shared__ gss_report stage_all[kWarps][kStage];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int sub = lane % LPC;
    const int grp = lane / LPC;
    const int gbase = grp * LPC;
    gss_report *stage = stage_all[wib];
    const uint32_t part = blockIdx.x % a.n_parts;
    gss_report *out = a.out + (size_t) part * a.cap_per_part;
    uint32_t *counter = a.counts + part;
    uint32_t nstaged = 0;

    const uint32_t n_scan = scan_count(a);
    const uint32_t n_groups = (n_scan + CPW - 1) / CPW;
    const uint64_t n_tasks = (uint64_t) n_groups * a.n_blocks;
    const uint64_t stride = (uint64_t) gridDim.x * kWarps;
    uint64_t task = (uint64_t) blockIdx.x * kWarps + wib;

    // clause of this lane's group for a task
    auto clause_of = [&](uint64_t t) -> uint32_t {
        const uint32_t b = (uint32_t) (t / n_groups);
        const uint32_t i = (uint32_t) (t - (uint64_t) b * n_groups) * CPW + grp;
        return i < n_scan ? scan_clause(a, i) : 0xFFFFFFFFu;
    };
    // prefetched: offsets and first literal chunk of the current task
    uint32_t nx_pos = 0, nx_end = 0;
    int32_t nx_chunk = 0;
    if (task < n_tasks) {
        const uint32_t c0 = clause_of(task);
        if (c0 < a.n_clauses) {
            nx_pos = (uint32_t) __ldg(a.offsets + c0);
            nx_end = (uint32_t) __ldg(a.offsets + c0 + 1);
            nx_chunk = (nx_pos + sub < nx_end) ? __ldg(a.lits + nx_pos + sub) : 0;
        }
    }
    for (; task < n_tasks; task += stride) {
        const uint32_t blk = (uint32_t) (task / n_groups);
        const uint32_t c = clause_of(task);
        const bool valid = c < a.n_clauses && clause_live(a, c);
        const uint32_t w0 = blk * BW + sub * WPL;
        uint32_t af[WPL], ou[WPL];
#pragma unroll
        for (int j = 0; j < WPL; j++) {
            af[j] = valid ? __ldg(a.start + w0 + j) : 0u;
            ou[j] = 0u;
        }
        uint32_t pos = valid ? nx_pos : 0u, end = valid ? nx_end : 0u;
        int32_t chunk = valid ? nx_chunk : 0;
        // start the next task's offsets now
        const uint64_t nt = task + stride;
        const uint32_t nc = nt < n_tasks ? clause_of(nt) : 0xFFFFFFFFu;
        const bool nvalid = nt < n_tasks && nc < a.n_clauses && clause_live(a, nc);
        nx_pos = nvalid ? (uint32_t) __ldg(a.offsets + nc) : 0u;
        nx_end = nvalid ? (uint32_t) __ldg(a.offsets + nc + 1) : 0u;
        bool next_chunk_due = true;
        const uint2 *rows = a.state + (size_t) blk * a.n_vars * BW + sub * WPL;
        while (true) {
            bool alive = false;
#pragma unroll
            for (int j = 0; j < WPL; j++) alive |= (af[j] | ou[j]) != 0u;
            if (!__any_sync(kFull, alive && pos < end)) break;
            // this clause's next chunk, while the current one is checked
            const int32_t after = (pos + LPC + sub < end) ? __ldg(a.lits + pos + LPC + sub) : 0;
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
                if (next_chunk_due) {
                    // the next task's offsets have had a gather round to arrive
                    nx_chunk = (nvalid && nx_pos + sub < nx_end) ? __ldg(a.lits + nx_pos + sub) : 0;
                    next_chunk_due = false;
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
            chunk = after;
        }
        if (next_chunk_due) nx_chunk = (nvalid && nx_pos + sub < nx_end) ? __ldg(a.lits + nx_pos + sub) : 0;
#pragma unroll
        for (int j = 0; j < WPL; j++) {
            const uint32_t rep = af[j] | ou[j];
            const unsigned bal = __ballot_sync(kFull, rep != 0u);
            if (bal) {
                if (nstaged + 32 > (uint32_t) kStage) {
                    flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane);
                    nstaged = 0;
                }
                if (rep) {
                    gss_report r;
                    r.clause = __ldg(a.orig + c);
                    r.word = w0 + j;
                    r.mask = rep;
                    r.solver = (uint32_t) __ldg(a.solver_of_word + w0 + j);
                    stage[nstaged + __popc(bal & lanemask_lt())] = r;
                }
                nstaged += __popc(bal);
            }
        }
    }
    if (nstaged) flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane);
}

// Persistent wide variant: as check_wide_kernel, with (1) its arguments read
// from device memory, so a captured CUDA graph can run it pass after pass
// while the database and the assignment state change, and (2) tasks taken in
// chunks from a device work counter (zeroed before the launch) instead of a
// fixed stride, so clauses of very different lengths balance across warps.
constexpr uint32_t kTaskChunk = 4;

template <int WPL, int LPC, int G, int MINB>
__global__ void __launch_bounds__(kWarps * 32, MINB) check_wide_persist_kernel(const CheckArgs *__restrict__ pa,
                                                                                const CheckArgs av,
                                                                                uint32_t *__restrict__ work) {
    constexpr int CPW = 32 / LPC;
    constexpr int BW = WPL * LPC;
    __shared__ CheckArgs sa;
    __shared__ gss_report stage_all[kWarps][kStage];
    if (threadIdx.x == 0) sa = pa ? *pa : av;
    __syncthreads();
    const CheckArgs &a = sa;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int sub = lane % LPC;
    const int grp = lane / LPC;
    const int gbase = grp * LPC;
    gss_report *stage = stage_all[wib];
    const uint32_t part = blockIdx.x % a.n_parts;
    gss_report *out = a.out + (size_t) part * a.cap_per_part;
    uint32_t *counter = a.counts + part;
    uint32_t nstaged = 0;

    const uint32_t n_scan = scan_count(a);
    const uint32_t n_groups = (n_scan + CPW - 1) / CPW;
    const uint64_t n_tasks = (uint64_t) n_groups * a.n_blocks;
    Row<WPL> st[G];  // zeroed once, as in check_wide_kernel
#pragma unroll
    for (int i = 0; i < G; i++)
#pragma unroll
        for (int q = 0; q < 2 * WPL; q++) st[i].v[q] = 0u;
    while (true) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(work, kTaskChunk);
        first = __shfl_sync(kFull, first, 0);
        if ((uint64_t) first >= n_tasks) break;
        const uint64_t last = min((uint64_t) first + kTaskChunk, n_tasks);
        for (uint64_t task = first; task < last; task++) {
            const uint32_t blk = (uint32_t) (task / n_groups);
            const uint32_t g = (uint32_t) (task - (uint64_t) blk * n_groups);
            const uint32_t i = g * CPW + grp;
            const uint32_t c = i < n_scan ? scan_clause(a, i) : 0xFFFFFFFFu;
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
#pragma unroll
                    for (int i = 0; i < G; i++) lit[i] = (uint32_t) __shfl_sync(kFull, chunk, gbase + k0 + i);
#pragma unroll
                    for (int i = 0; i < G; i++) {
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
                    if (nstaged + 32 > (uint32_t) kStage) {
                        flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane);
                        nstaged = 0;
                    }
                    if (rep) {
                        gss_report r;
                        r.clause = __ldg(a.orig + c);
                        r.word = w0 + j;
                        r.mask = rep;
                        r.solver = (uint32_t) __ldg(a.solver_of_word + w0 + j);
                        stage[nstaged + __popc(bal & lanemask_lt())] = r;
                    }
                    nstaged += __popc(bal);
                }
            }
        }
    }
    if (nstaged) flush_stage(stage, nstaged, out, counter, a.cap_per_part, lane);
}

template <int WPL, int LPC, int G>
int launch_wide_persist_variant(const CheckArgs *d_args, const CheckArgs &h_args, uint32_t *work, cudaStream_t stream,
                                int sm_count) {
    constexpr int MINB = default_min_blocks(WPL, G);
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_wide_persist_kernel<WPL, LPC, G, MINB>,
                                                               kWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    check_wide_persist_kernel<WPL, LPC, G, MINB><<<(unsigned) (sm_count * per_sm), kWarps * 32, 0, stream>>>(
        d_args, h_args, work);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

template <int WPL, int LPC, int G, int MINB>
int launch_wide_pf_variant(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_wide_pf_kernel<WPL, LPC, G, MINB>,
                                                               kWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    constexpr int CPW = 32 / LPC;
    const uint64_t n_tasks = (uint64_t) ((scan_count(a) + CPW - 1) / CPW) * a.n_blocks;
    uint64_t blocks = (uint64_t) sm_count * per_sm;
    const uint64_t need = (n_tasks + kWarps - 1) / kWarps;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    check_wide_pf_kernel<WPL, LPC, G, MINB><<<(unsigned) blocks, kWarps * 32, 0, stream>>>(a);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

template <int WPL, int LPC, int G, int MINB, bool MAP_IDS = true, bool HINT = false>
int launch_wide_variant(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, check_wide_kernel<WPL, LPC, G, MINB, MAP_IDS, HINT>, kWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    constexpr int CPW = 32 / LPC;
    const uint64_t n_tasks = (uint64_t) ((scan_count(a) + CPW - 1) / CPW) * a.n_blocks;
    uint64_t blocks = (uint64_t) sm_count * per_sm;
    const uint64_t need = (n_tasks + kWarps - 1) / kWarps;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    check_wide_kernel<WPL, LPC, G, MINB, MAP_IDS, HINT><<<(unsigned) blocks, kWarps * 32, 0, stream>>>(a);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

// Host layout [n_vars][n_words]{isDef,isTrue} -> block-major
// [n_blocks][n_vars][lpc]{isDef,isTrue}, words past n_words zero.
__global__ void relayout_kernel(const uint2 *__restrict__ src, uint2 *__restrict__ dst, uint32_t n_vars,
                                uint32_t n_words, uint32_t lpc, uint32_t n_blocks) {
    const uint64_t total = (uint64_t) n_blocks * n_vars * lpc;
    for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t) gridDim.x * blockDim.x) {
        const uint32_t s = (uint32_t) (i % lpc);
        const uint64_t r = i / lpc;
        const uint32_t v = (uint32_t) (r % n_vars);
        const uint32_t b = (uint32_t) (r / n_vars);
        const uint32_t w = b * lpc + s;
        dst[i] = (w < n_words) ? src[(uint64_t) v * n_words + w] : make_uint2(0u, 0u);
    }
}

template <int LPC, int G>
int launch_variant(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_kernel<LPC, G>, kWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    constexpr int CPW = 32 / LPC;
    const uint64_t n_tasks = (uint64_t) ((scan_count(a) + CPW - 1) / CPW) * a.n_blocks;
    uint64_t blocks = (uint64_t) sm_count * per_sm;
    const uint64_t need = (n_tasks + kWarps - 1) / kWarps;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    check_kernel<LPC, G><<<(unsigned) blocks, kWarps * 32, 0, stream>>>(a);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

}  // namespace

// Wide variants: (words per lane, lanes per clause, depth, occupancy hint).
bool valid_wide_variant(int wpl, int lpc, int g, int occ) {
    if (occ != 0 && occ != 1) return false;
    if (wpl == 4 && lpc == 8) return g == 1 || g == 2 || g == 4;
    if (wpl == 4 && lpc == 4) return g == 1 || g == 2 || g == 4;
    if (wpl == 4 && lpc == 2) return g == 1 || g == 2;
    if (wpl == 2 && lpc == 16) return g == 1 || g == 2 || g == 4;
    if (wpl == 2 && lpc == 8) return g == 1 || g == 2 || g == 4;
    if (wpl == 1 && lpc == 32) return g == 1 || g == 2 || g == 4;
    return false;
}

int launch_check_wide_pf(const CheckArgs &a, int wpl, int occ, cudaStream_t stream, int sm_count) {
    if (a.n_clauses == 0 || a.n_blocks == 0 || scan_count(a) == 0) return GSS_OK;
#define GSS_PV(W, L, GG)                                                                      \
    if (wpl == W && a.lpc == L && a.g == GG)                                                  \
        return occ ? launch_wide_pf_variant<W, L, GG, 4>(a, stream, sm_count)                 \
                   : launch_wide_pf_variant<W, L, GG, 1>(a, stream, sm_count);
    GSS_PV(4, 8, 1) GSS_PV(4, 8, 2) GSS_PV(4, 8, 4)
    GSS_PV(4, 4, 2) GSS_PV(4, 4, 4)
    GSS_PV(2, 16, 2) GSS_PV(2, 16, 4)
#undef GSS_PV
    return set_error(GSS_ERR_INVALID, "no pipelined wide kernel variant for %d words per lane, %d lanes, depth %d",
                     wpl, a.lpc, a.g);
}

int launch_check_wide_persist(const CheckArgs *d_args, const CheckArgs &h_args, int wpl, int lpc, int g, uint32_t *work,
                              cudaStream_t stream, int sm_count) {
#define GSS_QV(W, L, GG)                 \
    if (wpl == W && lpc == L && g == GG) \
        return launch_wide_persist_variant<W, L, GG>(d_args, h_args, work, stream, sm_count);
    GSS_QV(4, 8, 1) GSS_QV(4, 8, 2) GSS_QV(4, 8, 4)
    GSS_QV(4, 4, 2) GSS_QV(4, 2, 2)
    GSS_QV(2, 16, 2) GSS_QV(2, 8, 2)
#undef GSS_QV
    return set_error(GSS_ERR_INVALID, "no persistent wide kernel variant for %d words per lane, %d lanes, depth %d",
                     wpl, lpc, g);
}

bool valid_wide_persist_variant(int wpl, int lpc, int g) {
    if (wpl == 4 && lpc == 8) return g == 1 || g == 2 || g == 4;
    if (wpl == 4 && (lpc == 4 || lpc == 2)) return g == 2;
    if (wpl == 2 && (lpc == 16 || lpc == 8)) return g == 2;
    return false;
}

bool valid_wide_pf_variant(int wpl, int lpc, int g) {
    if (wpl == 4 && lpc == 8) return g == 1 || g == 2 || g == 4;
    if (wpl == 4 && lpc == 4) return g == 2 || g == 4;
    if (wpl == 2 && lpc == 16) return g == 2 || g == 4;
    return false;
}

int launch_check_wide(const CheckArgs &a, int wpl, int occ, cudaStream_t stream, int sm_count) {
    if (a.n_clauses == 0 || a.n_blocks == 0 || scan_count(a) == 0) return GSS_OK;
    // L2 policies (cache_hints) for the 4-words-per-lane, 8-lane kinds
    if (wpl == 4 && a.lpc == 8 && !occ && a.cache_hints) {
        if (a.g == 1) return launch_wide_variant<4, 8, 1, 1, true, true>(a, stream, sm_count);
        if (a.g == 2) return launch_wide_variant<4, 8, 2, 1, true, true>(a, stream, sm_count);
        if (a.g == 4) return launch_wide_variant<4, 8, 4, 1, true, true>(a, stream, sm_count);
    }
#define GSS_WV(W, L, GG)                                                                      \
    if (wpl == W && a.lpc == L && a.g == GG)                                                  \
        return occ ? launch_wide_variant<W, L, GG, 8>(a, stream, sm_count)                    \
                   : launch_wide_variant<W, L, GG, default_min_blocks(W, GG)>(a, stream, sm_count);
    GSS_WV(4, 8, 1) GSS_WV(4, 8, 2) GSS_WV(4, 8, 4)
    GSS_WV(4, 4, 1) GSS_WV(4, 4, 2) GSS_WV(4, 4, 4)
    GSS_WV(4, 2, 1) GSS_WV(4, 2, 2)
    GSS_WV(2, 16, 1) GSS_WV(2, 16, 2) GSS_WV(2, 16, 4)
    GSS_WV(2, 8, 1) GSS_WV(2, 8, 2) GSS_WV(2, 8, 4)
    GSS_WV(1, 32, 1) GSS_WV(1, 32, 2) GSS_WV(1, 32, 4)
#undef GSS_WV
    return set_error(GSS_ERR_INVALID, "no wide kernel variant for %d words per lane, %d lanes, depth %d", wpl,
                     a.lpc, a.g);
}

bool valid_variant(int lpc, int g) {
    switch (lpc) {
        case 1: return g == 1;
        case 2: return g == 1 || g == 2;
        case 4: return g == 1 || g == 2 || g == 4;
        case 8: return g == 1 || g == 2 || g == 4 || g == 8;
        case 16: return g == 1 || g == 2 || g == 4 || g == 8;
        case 32: return g == 1 || g == 2 || g == 4 || g == 8;
        default: return false;
    }
}

int launch_check(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    if (a.n_clauses == 0 || a.n_blocks == 0 || scan_count(a) == 0) return GSS_OK;
#define GSS_VARIANT(L, GG) \
    if (a.lpc == L && a.g == GG) return launch_variant<L, GG>(a, stream, sm_count);
    GSS_VARIANT(1, 1)
    GSS_VARIANT(2, 1) GSS_VARIANT(2, 2)
    GSS_VARIANT(4, 1) GSS_VARIANT(4, 2) GSS_VARIANT(4, 4)
    GSS_VARIANT(8, 1) GSS_VARIANT(8, 2) GSS_VARIANT(8, 4) GSS_VARIANT(8, 8)
    GSS_VARIANT(16, 1) GSS_VARIANT(16, 2) GSS_VARIANT(16, 4) GSS_VARIANT(16, 8)
    GSS_VARIANT(32, 1) GSS_VARIANT(32, 2) GSS_VARIANT(32, 4) GSS_VARIANT(32, 8)
#undef GSS_VARIANT
    return set_error(GSS_ERR_INVALID, "no kernel variant for %d lanes per clause, depth %d", a.lpc, a.g);
}

int launch_relayout(const uint2 *src, uint2 *dst, uint32_t n_vars, uint32_t n_words, uint32_t lpc,
                    uint32_t n_blocks, cudaStream_t stream, int sm_count) {
    const uint64_t total = (uint64_t) n_blocks * n_vars * lpc;
    if (total == 0) return GSS_OK;
    uint64_t blocks = (total + 255) / 256;
    const uint64_t cap = (uint64_t) sm_count * 8;
    if (blocks > cap) blocks = cap;
    relayout_kernel<<<(unsigned) blocks, 256, 0, stream>>>(src, dst, n_vars, n_words, lpc, n_blocks);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

}  // namespace gss

// ------------------------------------------------ allocation-free pass ----
//
// gss_check_noalloc: the wide check kernel for callers that cannot allocate
// device memory. The kernel's only working memory is its report reservation
// counters (one per output partition); here they live in a fixed,
// file-scope device array instead of a cudaMalloc'ed buffer, so the call
// allocates nothing. Every GPU that loads this library holds the array
// (256 bytes) until the process exits.

namespace {

constexpr uint32_t kNoAllocMaxParts = 64;

// Report reservation counters of gss_check_noalloc, shared by all its calls.
static __device__ __align__(256) uint32_t g_noalloc_counters[kNoAllocMaxParts];

// The counters' device address on the current device. In host code the
// array's name is only a host-side stand-in, so every call asks the runtime
// for the real address (a host-side lookup: it allocates nothing, and it
// stays right if the device's context is torn down and created again).
int noalloc_counters(uint32_t **out) {
    void *p = nullptr;
    GSS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_counters));
    *out = (uint32_t *) p;
    return GSS_OK;
}

}  // namespace

extern "C" int gss_check_noalloc(const int32_t *lits, const int64_t *offsets, uint32_t n_clauses,
                                 const uint32_t *state, uint32_t n_vars, uint32_t n_blocks, const uint32_t *start,
                                 const int32_t *solver_of_word, gss_report *out, uint32_t n_parts,
                                 uint32_t cap_per_part, uint32_t *counts_out, void *stream) {
    using namespace gss;
    if (n_parts == 0 || n_parts > kNoAllocMaxParts)
        return set_error(GSS_ERR_INVALID,
                         "gss_check_noalloc: %u report partitions requested; the allocation-free pass has a fixed "
                         "array of %u counters",
                         n_parts, kNoAllocMaxParts);
    if (!counts_out || (n_clauses > 0 && (!lits || !offsets)) || (n_blocks > 0 && (!state || !start ||
                                                                                  !solver_of_word)) ||
        (cap_per_part > 0 && !out))
        return set_error(GSS_ERR_INVALID, "gss_check_noalloc: NULL input or output");
    if (n_clauses > 0 && n_vars == 0)
        return set_error(GSS_ERR_INVALID, "gss_check_noalloc: %u clauses over 0 variables", n_clauses);
    if ((uint64_t) cap_per_part * n_parts > 0xFFFFFFFFull)
        return set_error(GSS_ERR_INVALID, "gss_check_noalloc: output capacity above 2^32 records");
    cudaStream_t st = (cudaStream_t) stream;
    uint32_t *counters = nullptr;
    GSS_TRY(noalloc_counters(&counters));
    // every call starts from zeroed counters: they keep the previous call's values
    GSS_CUDA_TRY(cudaMemsetAsync(counters, 0, n_parts * sizeof(uint32_t), st));
    if (n_clauses > 0 && n_blocks > 0) {
        int dev = 0, sms = 0;
        GSS_CUDA_TRY(cudaGetDevice(&dev));
        GSS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CheckArgs a;
        memset(&a, 0, sizeof a);
        a.lits = lits;
        a.offsets = offsets;
        a.orig = nullptr;
        a.n_clauses = n_clauses;
        a.scan_begin = 0;
        a.scan_end = n_clauses;
        a.state = (const uint2 *) state;
        a.n_vars = n_vars;
        a.n_blocks = n_blocks;
        a.start = start;
        a.solver_of_word = solver_of_word;
        a.out = out;
        a.counts = counters;
        a.n_parts = n_parts;
        a.cap_per_part = cap_per_part;
        a.lpc = 8;
        a.g = 2;
        GSS_TRY((launch_wide_variant<4, 8, 2, default_min_blocks(4, 2), false>(a, st, sms)));
    }
    GSS_CUDA_TRY(cudaMemcpyAsync(counts_out, counters, n_parts * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    return GSS_OK;
}
