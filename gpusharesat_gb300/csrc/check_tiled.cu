// Tiled check kernel: the default path of the check pass.
//
// Same rule as check.cu (gpuShareLib/GpuRunner.cu:34-89 restated there); a
// different schedule, built so that every warp keeps many independent state
// gathers in flight:
//
//  * The length-sorted database is cut on the host into tiles of consecutive
//    clauses holding at most kTileLits literals. Each warp takes tiles in turn
//    and stages the tile's literals into its own shared-memory buffer with one
//    bulk asynchronous copy (cp.async.bulk, completion on an mbarrier), double
//    buffered: the copy of the warp's next tile runs while it checks the
//    current one. A clause longer than kTileLits gets a tile of its own and is
//    read straight from global memory.
//  * A group of LPC lanes owns LPC 32-slot words of one clause (the slot
//    block); a warp has 32/LPC groups, each with K clause slots. Every step,
//    each slot of each group reads its clause's next literal from shared
//    memory and gathers that variable's state row, so a lane has up to K
//    gathers in flight and none of them is speculative. A slot whose clause is
//    done (no live slot left, or no literal left) reports and takes the next
//    clause of the tile.
//  * Reports are staged per warp in shared memory and written with one
//    atomicAdd per flush, as in check.cu.
//
// Waits on the mbarrier are bounded: after kSpinLimit polls the warp records an
// error code in a device flag, stops, and the host turns it into an error.
#include "common.h"

namespace gss {

namespace {

constexpr int kTWarps = 8;         // warps per block
constexpr int kTStage = 64;        // staged report records per warp
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kSpinLimit = 1u << 24;

struct __align__(16) WarpSmem {
    int32_t buf[2][kBufLits];
    unsigned long long bar[2];
    gss_report stage[kTStage];
};

// Lanes that lead a group of LPC lanes (sub == 0).
template <int LPC>
__device__ constexpr unsigned leader_mask() {
    unsigned m = 0;
    for (int i = 0; i < 32; i += LPC) m |= 1u << i;
    return m;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}

// One lane: expect `bytes` and start the bulk copy global -> shared.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait for phase `parity` of the barrier. Returns false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
    const uint32_t addr = smem_addr(bar);
    for (uint32_t i = 0; i < kSpinLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint2 ld_state(const uint2 *p, bool hint, uint64_t pol) {
    uint2 v;
    if (hint) {
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
            : "=r"(v.x), "=r"(v.y) : "l"(p), "l"(pol));
    } else {
        asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    }
    return v;
}

__device__ __forceinline__ void flush_stage(gss_report *stage, uint32_t n, gss_report *out, uint32_t *counter,
                                            uint32_t cap, int lane) {
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

// Clause range [c0, c1) and literal range [l0, l1) of tile t.
__device__ __forceinline__ void tile_range(const CheckArgs &a, uint32_t t, uint32_t &c0, uint32_t &c1,
                                           uint32_t &l0, uint32_t &l1) {
    c0 = __ldg(a.tile_clause + t);
    c1 = __ldg(a.tile_clause + t + 1);
    l0 = __ldg(a.tile_lit + t);
    l1 = __ldg(a.tile_lit + t + 1);
}

template <int LPC, int K>
__global__ void __launch_bounds__(kTWarps * 32) check_tiled_kernel(CheckArgs a) {
    constexpr int CPW = 32 / LPC;
    __shared__ WarpSmem smem_all[kTWarps];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int sub = lane % LPC;
    const int grp = lane / LPC;
    const unsigned gmask = (LPC == 32) ? kFull : (((1u << LPC) - 1u) << (grp * LPC));
    WarpSmem &sm = smem_all[wib];
    const uint32_t part = blockIdx.x % a.n_parts;
    gss_report *out = a.out + (size_t) part * a.cap_per_part;
    uint32_t *counter = a.counts + part;
    uint32_t nstaged = 0;
    const bool hint = a.cache_hints != 0;
    const uint64_t pol_keep = policy_evict_last();

    if (lane == 0) {
        mbar_init(&sm.bar[0]);
        mbar_init(&sm.bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();

    const uint64_t n_tasks = (uint64_t) a.n_tiles * a.n_blocks;
    const uint64_t stride = (uint64_t) gridDim.x * kTWarps;
    uint64_t task = (uint64_t) blockIdx.x * kTWarps + wib;
    uint32_t phase[2] = {0u, 0u};

    bool pending[2] = {false, false};
    // Starts the copy of `tk`'s tile into buffer b (lane 0); no-op for long
    // tiles. The literal range is rounded out to 16-byte boundaries (the
    // literal array is padded so the rounded end stays inside it).
    auto issue = [&](uint64_t tk, int b) {
        if (tk >= n_tasks) return;
        const uint32_t t = (uint32_t) (tk % a.n_tiles);
        uint32_t c0, c1, l0, l1;
        tile_range(a, t, c0, c1, l0, l1);
        if (l1 - l0 > (uint32_t) kTileLits) return;  // long clause: read from global memory
        const uint32_t a0 = l0 & ~3u;
        const uint32_t a1 = (l1 + 3u) & ~3u;
        if (lane == 0) bulk_load(sm.buf[b], a.lits + a0, (a1 - a0) * 4u, &sm.bar[b]);
        pending[b] = true;
    };

    issue(task, 0);
    for (int it = 0; task < n_tasks; task += stride, it++) {
        const int b = it & 1;
        issue(task + stride, b ^ 1);
        const uint32_t blk = (uint32_t) (task / a.n_tiles);
        const uint32_t t = (uint32_t) (task - (uint64_t) blk * a.n_tiles);
        uint32_t c0, c1, l0, l1;
        tile_range(a, t, c0, c1, l0, l1);
        const bool staged = (l1 - l0) <= (uint32_t) kTileLits;
        const uint32_t base = l0 & ~3u;
        if (staged) {
            const bool ok = mbar_wait(&sm.bar[b], phase[b]);
            phase[b] ^= 1u;
            pending[b] = false;
            if (!__all_sync(kFull, ok)) {
                // Give up on this pass: flag it, let the other copy land, stop.
                if (lane == 0) atomicExch(a.err, 1u);
                if (pending[b ^ 1]) mbar_wait(&sm.bar[b ^ 1], phase[b ^ 1]);
                return;
            }
        }
        const int32_t *tl = sm.buf[b];
        const uint2 *rows = a.state + (size_t) blk * a.n_vars * LPC + sub;
        const uint32_t w = blk * LPC + sub;
        const uint32_t start_w = __ldg(a.start + w);

        // slots
        uint32_t cl[K], pos[K], end[K];
        uint32_t af[K], ou[K];
        uint32_t next = c0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t c = next + k * CPW + grp;
            cl[k] = c;
            if (c < c1) {
                pos[k] = (uint32_t) __ldg(a.offsets + c);
                end[k] = (uint32_t) __ldg(a.offsets + c + 1);
                af[k] = start_w;
            } else {
                pos[k] = end[k] = 0;
                af[k] = 0u;
            }
            ou[k] = 0u;
        }
        next += K * CPW;

        while (true) {
            uint2 st[K];
            uint32_t lit[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                const bool has = cl[k] < c1 && pos[k] < end[k];
                lit[k] = 0u;
                st[k] = make_uint2(0u, 0u);
                if (has) {
                    lit[k] = (uint32_t) (staged ? tl[pos[k] - base] : __ldg(a.lits + pos[k]));
                    if ((af[k] | ou[k]) != 0u) st[k] = ld_state(rows + (size_t) (lit[k] >> 1) * LPC, hint, pol_keep);
                }
            }
            bool any_slot = false;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const bool has = cl[k] < c1 && pos[k] < end[k];
                if (has) {
                    const uint32_t f = ((lit[k] & 1u) ? st[k].y : ~st[k].y) & st[k].x;
                    const uint32_t u = ~st[k].x;
                    ou[k] = (af[k] & u) | (ou[k] & f);
                    af[k] &= f;
                    pos[k]++;
                }
                // slot done: its clause has no live word left in the group, or no literal left
                const bool live = cl[k] < c1 && (af[k] | ou[k]) != 0u;
                const unsigned glive = __ballot_sync(kFull, live) & gmask;
                const bool occupied = cl[k] < c1;
                const bool done = occupied && (glive == 0u || pos[k] >= end[k]);
                const unsigned dmask = __ballot_sync(kFull, done);
                if (dmask) {
                    const uint32_t rep = done ? (af[k] | ou[k]) : 0u;
                    const unsigned bal = __ballot_sync(kFull, rep != 0u);
                    if (bal) {
                        if (nstaged + 32 > (uint32_t) kTStage) {
                            flush_stage(sm.stage, nstaged, out, counter, a.cap_per_part, lane);
                            nstaged = 0;
                        }
                        if (rep) {
                            gss_report r;
                            r.clause = __ldg(a.orig + cl[k]);
                            r.word = w;
                            r.mask = rep;
                            r.solver = (uint32_t) __ldg(a.solver_of_word + w);
                            sm.stage[nstaged + __popc(bal & lanemask_lt())] = r;
                        }
                        nstaged += __popc(bal);
                    }
                    // refill the finished slots of this k, in group order
                    const unsigned leaders = dmask & leader_mask<LPC>();
                    const uint32_t rank = __popc(leaders & ((1u << (grp * LPC)) - 1u));
                    if (done) {
                        const uint32_t c = next + rank;
                        cl[k] = c;
                        if (c < c1) {
                            pos[k] = (uint32_t) __ldg(a.offsets + c);
                            end[k] = (uint32_t) __ldg(a.offsets + c + 1);
                            af[k] = start_w;
                        } else {
                            af[k] = 0u;
                        }
                        ou[k] = 0u;
                    }
                    next += __popc(leaders);
                }
                any_slot |= cl[k] < c1;
            }
            if (!__any_sync(kFull, any_slot)) break;
        }
        __syncwarp();
    }
    if (nstaged) flush_stage(sm.stage, nstaged, out, counter, a.cap_per_part, lane);
}

template <int LPC, int K>
int launch_tiled_variant(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    int per_sm = 0;
    GSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_tiled_kernel<LPC, K>, kTWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
    const uint64_t n_tasks = (uint64_t) a.n_tiles * a.n_blocks;
    uint64_t blocks = (uint64_t) sm_count * per_sm;
    const uint64_t need = (n_tasks + kTWarps - 1) / kTWarps;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    check_tiled_kernel<LPC, K><<<(unsigned) blocks, kTWarps * 32, 0, stream>>>(a);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

}  // namespace

bool valid_tiled_variant(int lpc, int k) {
    return (lpc == 32 || lpc == 16 || lpc == 8 || lpc == 4 || lpc == 2 || lpc == 1) && (k == 2 || k == 4 || k == 8);
}

int launch_check_tiled(const CheckArgs &a, cudaStream_t stream, int sm_count) {
    if (a.n_clauses == 0 || a.n_blocks == 0 || a.n_tiles == 0) return GSS_OK;
#define GSS_TV(L, KK) \
    if (a.lpc == L && a.g == KK) return launch_tiled_variant<L, KK>(a, stream, sm_count);
    GSS_TV(32, 2) GSS_TV(32, 4) GSS_TV(32, 8)
    GSS_TV(16, 2) GSS_TV(16, 4) GSS_TV(16, 8)
    GSS_TV(8, 2) GSS_TV(8, 4) GSS_TV(8, 8)
    GSS_TV(4, 2) GSS_TV(4, 4) GSS_TV(4, 8)
    GSS_TV(2, 2) GSS_TV(2, 4) GSS_TV(2, 8)
    GSS_TV(1, 2) GSS_TV(1, 4) GSS_TV(1, 8)
#undef GSS_TV
    return set_error(GSS_ERR_INVALID, "no tiled kernel variant for %d lanes per clause, %d slots", a.lpc, a.g);
}

}  // namespace gss
