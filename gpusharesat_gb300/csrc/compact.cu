// Order-preserving compaction of the device clause database, on the device.
//
// The sharer evicts clauses by clearing their bit in an alive bitmap indexed
// by clause id (the id a report carries, CheckArgs::orig). Tombstoned clauses
// cost the check kernels one bitmap test each; once they are a large share
// of the database this pass drops them without a host round trip: the live
// clauses keep their order, their literals move to a second buffer, and the
// id map follows. HBM-bound: every literal is read once and written once.
//
// gather_clauses rebuilds a database in a new order chosen on the host (a
// reduceDb): the host sends, per kept clause, its old position and its new
// offset (12 bytes); the literals move on the device.
//
// Four launches:
//   1. per tile of kTileClauses clauses: live clause count and literal count
//   2. one block: exclusive scan of the tile totals, the final offset and the
//      zero padding after the last literal
//   3. per tile again: exclusive scan inside the tile, write the new offset,
//      id and source position of each live clause
//   4. a warp per live clause copies its literals (coalesced)
#include <stdint.h>

#include <algorithm>

#include "common.h"

namespace gss {
namespace {

constexpr int kThreads = 1024;
constexpr int kItems = 4;  // clauses per thread
constexpr uint32_t kTileClauses = kThreads * kItems;
constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ bool live_by_id(const uint32_t *alive, const uint32_t *ids, uint32_t c) {
    const uint32_t id = __ldg(ids + c);
    return (__ldg(alive + (id >> 5)) >> (id & 31)) & 1u;
}

// Exclusive scan over the block of a per-thread value; *total gets the sum.
template <typename T>
__device__ T block_exclusive_scan(T v, T *warp_sums, T *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T s = lane < (int) (blockDim.x >> 5) ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(kFull, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    const T base = warp ? warp_sums[warp - 1] : T(0);
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();  // warp_sums may be reused by the caller
    return base + x - v;
}

__global__ void __launch_bounds__(kThreads) tile_totals_kernel(const int64_t *offsets, const uint32_t *ids,
                                                               const uint32_t *alive, uint32_t n,
                                                               uint32_t *tile_cnt, int64_t *tile_lits) {
    __shared__ uint32_t ws_c[32];
    __shared__ int64_t ws_l[32];
    const uint32_t c0 = blockIdx.x * kTileClauses + threadIdx.x * kItems;
    uint32_t cnt = 0;
    int64_t lits = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        const uint32_t c = c0 + k;
        if (c < n && live_by_id(alive, ids, c)) {
            cnt++;
            lits += __ldg(offsets + c + 1) - __ldg(offsets + c);
        }
    }
    uint32_t tc;
    int64_t tl;
    block_exclusive_scan<uint32_t>(cnt, ws_c, &tc);
    block_exclusive_scan<int64_t>(lits, ws_l, &tl);
    if (threadIdx.x == 0) {
        tile_cnt[blockIdx.x] = tc;
        tile_lits[blockIdx.x] = tl;
    }
}

// One block: tile totals -> exclusive bases, in place. Writes the new final
// offset, the zero padding after the last literal and the totals.
__global__ void __launch_bounds__(kThreads) tile_scan_kernel(uint32_t *tile_cnt, int64_t *tile_lits, uint32_t n_tiles,
                                                             int64_t *new_offsets, int32_t *new_lits,
                                                             uint32_t *out_clauses, int64_t *out_lits) {
    __shared__ uint32_t ws_c[32];
    __shared__ int64_t ws_l[32];
    uint32_t carry_c = 0;
    int64_t carry_l = 0;
    for (uint32_t base = 0; base < n_tiles; base += kThreads) {
        const uint32_t t = base + threadIdx.x;
        const uint32_t c = t < n_tiles ? tile_cnt[t] : 0;
        const int64_t l = t < n_tiles ? tile_lits[t] : 0;
        uint32_t sc;
        int64_t sl;
        const uint32_t ec = block_exclusive_scan<uint32_t>(c, ws_c, &sc);
        const int64_t el = block_exclusive_scan<int64_t>(l, ws_l, &sl);
        if (t < n_tiles) {
            tile_cnt[t] = carry_c + ec;
            tile_lits[t] = carry_l + el;
        }
        carry_c += sc;
        carry_l += sl;
    }
    if (threadIdx.x == 0) {
        new_offsets[carry_c] = carry_l;
        *out_clauses = carry_c;
        *out_lits = carry_l;
    }
    if (threadIdx.x < kClausePad) new_lits[carry_l + threadIdx.x] = 0;
}

__global__ void __launch_bounds__(kThreads) scatter_kernel(const int64_t *offsets, const uint32_t *ids,
                                                           const uint32_t *alive, uint32_t n,
                                                           const uint32_t *tile_cnt, const int64_t *tile_lits,
                                                           int64_t *new_offsets, uint32_t *new_ids,
                                                           uint32_t *src) {
    __shared__ uint32_t ws_c[32];
    __shared__ int64_t ws_l[32];
    const uint32_t c0 = blockIdx.x * kTileClauses + threadIdx.x * kItems;
    bool keep[kItems];
    int64_t len[kItems];
    uint32_t cnt = 0;
    int64_t lits = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        const uint32_t c = c0 + k;
        keep[k] = c < n && live_by_id(alive, ids, c);
        len[k] = keep[k] ? __ldg(offsets + c + 1) - __ldg(offsets + c) : 0;
        cnt += keep[k];
        lits += len[k];
    }
    uint32_t tc;
    int64_t tl;
    uint32_t pos = tile_cnt[blockIdx.x] + block_exclusive_scan<uint32_t>(cnt, ws_c, &tc);
    int64_t off = tile_lits[blockIdx.x] + block_exclusive_scan<int64_t>(lits, ws_l, &tl);
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        if (!keep[k]) continue;
        new_offsets[pos] = off;
        new_ids[pos] = __ldg(ids + c0 + k);
        src[pos] = c0 + k;
        pos++;
        off += len[k];
    }
}

__global__ void copy_kernel(const int32_t *lits, const int64_t *offsets, const uint32_t *src,
                            const int64_t *new_offsets, int32_t *new_lits, const uint32_t *n_new) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n = *n_new;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n; c += warps) {
        const int64_t from = __ldg(offsets + __ldg(src + c));
        const int64_t to = new_offsets[c];
        const int64_t len = new_offsets[c + 1] - to;
        for (int64_t i = lane; i < len; i += 32) new_lits[to + i] = __ldg(lits + from + i);
    }
}

// A warp per clause of the new database copies clause src[c]'s literals;
// its lane 0 writes the clause's id (its new position).
__global__ void gather_kernel(const int32_t *__restrict__ lits, const int64_t *__restrict__ offsets,
                              const uint32_t *__restrict__ src, const int64_t *__restrict__ new_offsets, uint32_t n,
                              int32_t *__restrict__ new_lits, uint32_t *__restrict__ new_ids) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n; c += warps) {
        const int64_t from = __ldg(offsets + __ldg(src + c));
        const int64_t to = __ldg(new_offsets + c);
        const int64_t len = __ldg(new_offsets + c + 1) - to;
        for (int64_t i = lane; i < len; i += 32) new_lits[to + i] = __ldg(lits + from + i);
        if (lane == 0) new_ids[c] = c;
    }
}

__global__ void pad_kernel(int32_t *new_lits, int64_t n_lits) {
    if (threadIdx.x < kClausePad) new_lits[n_lits + threadIdx.x] = 0;
}

// Packs the records of n_parts report partitions into one contiguous array:
// partition p's first counts[p] records (at most cap) go after the records of
// partitions 0..p-1. cell_words == 0: 12-byte records {clause, word, mask};
// otherwise 8-byte records {clause * cell_words + word, mask}.
__global__ void pack_reports_kernel(const gss_report *__restrict__ parts, const uint32_t *__restrict__ counts,
                                    uint32_t n_parts, uint32_t cap, uint32_t cell_words,
                                    uint32_t *__restrict__ packed) {
    const uint64_t total = (uint64_t) n_parts * cap;
    for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t) gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t) (i / cap), k = (uint32_t) (i - (uint64_t) p * cap);
        if (k >= min(__ldg(counts + p), cap)) continue;
        uint64_t base = 0;
        for (uint32_t q = 0; q < p; q++) base += min(__ldg(counts + q), cap);
        const gss_report r = parts[i];
        if (cell_words) {
            reinterpret_cast<uint2 *>(packed)[base + k] = make_uint2(r.clause * cell_words + r.word, r.mask);
        } else {
            uint32_t *o = packed + 3 * (base + k);
            o[0] = r.clause;
            o[1] = r.word;
            o[2] = r.mask;
        }
    }
}

}  // namespace

int launch_pack_reports(const gss_report *parts, const uint32_t *counts, uint32_t n_parts, uint32_t cap,
                        uint32_t cell_words, uint32_t *packed, cudaStream_t stream, int sm_count) {
    const uint64_t total = (uint64_t) n_parts * cap;
    if (total == 0) return GSS_OK;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > (uint64_t) sm_count * 16) blocks = (uint64_t) sm_count * 16;
    pack_reports_kernel<<<(unsigned) blocks, 256, 0, stream>>>(parts, counts, n_parts, cap, cell_words, packed);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

int gather_clauses(const GatherArgs &a, cudaStream_t stream, int sm_count) {
    if (a.n_new > 0) {
        gather_kernel<<<(unsigned) std::max(sm_count, 1) * 8, 256, 0, stream>>>(a.lits, a.offsets, a.src, a.new_offsets,
                                                                                a.n_new, a.new_lits, a.new_ids);
        GSS_CUDA_TRY(cudaGetLastError());
    }
    pad_kernel<<<1, 32, 0, stream>>>(a.new_lits, a.n_new_lits);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

size_t compact_scratch_bytes(uint32_t n_clauses) {
    const size_t tiles = ((size_t) n_clauses + kTileClauses - 1) / kTileClauses;
    return 256 + 8 + tiles * (sizeof(uint32_t) + sizeof(int64_t)) + (size_t) n_clauses * sizeof(uint32_t);
}

int compact_by_id(const CompactArgs &a, cudaStream_t stream, int sm_count, uint32_t *n_out, int64_t *lits_out) {
    if (a.n_clauses == 0) {
        *n_out = 0;
        *lits_out = 0;
        const int64_t zero = 0;
        GSS_CUDA_TRY(cudaMemcpyAsync(a.new_offsets, &zero, sizeof zero, cudaMemcpyHostToDevice, stream));
        GSS_CUDA_TRY(cudaMemsetAsync(a.new_lits, 0, kClausePad * sizeof(int32_t), stream));
        GSS_CUDA_TRY(cudaStreamSynchronize(stream));
        return GSS_OK;
    }
    const uint32_t tiles = (uint32_t) (((size_t) a.n_clauses + kTileClauses - 1) / kTileClauses);
    char *s = (char *) a.scratch;
    uint32_t *totals_c = (uint32_t *) s;
    int64_t *totals_l = (int64_t *) (s + 8);
    uint32_t *tile_cnt = (uint32_t *) (s + 256);
    int64_t *tile_lits = (int64_t *) (s + 256 + (((size_t) tiles * sizeof(uint32_t) + 7) & ~(size_t) 7));
    uint32_t *src = (uint32_t *) (tile_lits + tiles);
    tile_totals_kernel<<<tiles, kThreads, 0, stream>>>(a.offsets, a.ids, a.alive, a.n_clauses, tile_cnt, tile_lits);
    GSS_CUDA_TRY(cudaGetLastError());
    tile_scan_kernel<<<1, kThreads, 0, stream>>>(tile_cnt, tile_lits, tiles, a.new_offsets, a.new_lits, totals_c,
                                                 totals_l);
    GSS_CUDA_TRY(cudaGetLastError());
    scatter_kernel<<<tiles, kThreads, 0, stream>>>(a.offsets, a.ids, a.alive, a.n_clauses, tile_cnt, tile_lits,
                                                   a.new_offsets, a.new_ids, src);
    GSS_CUDA_TRY(cudaGetLastError());
    copy_kernel<<<(unsigned) std::max(sm_count, 1) * 8, 256, 0, stream>>>(a.lits, a.offsets, src, a.new_offsets,
                                                                          a.new_lits, totals_c);
    GSS_CUDA_TRY(cudaGetLastError());
    uint64_t host_totals[2];
    GSS_CUDA_TRY(cudaMemcpyAsync(host_totals, s, 16, cudaMemcpyDeviceToHost, stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(stream));
    *n_out = (uint32_t) host_totals[0];
    *lits_out = (int64_t) host_totals[1];
    return GSS_OK;
}

}  // namespace gss
