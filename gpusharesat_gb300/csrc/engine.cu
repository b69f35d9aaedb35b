// The engine: device-resident clause database, assignment bit planes and
// report queues, and the C ABI of include/gpusharesat.h (engine layer).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "common.h"
#include "engine.h"

namespace gss {

static thread_local std::string g_last_error = "no error";

int set_error(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

// Host-side fault injection for tests (gss_debug_fail_device_alloc): the
// next `count` device allocations of at least `min_bytes` made through DevBuf
// fail as if the device were out of memory. Nothing reaches the GPU.
static std::atomic<int64_t> g_fail_min_bytes{0};
static std::atomic<int> g_fail_count{0};

bool injected_alloc_failure(size_t bytes) {
    if (g_fail_count.load() <= 0 || (int64_t) bytes < g_fail_min_bytes.load()) return false;
    return g_fail_count.fetch_sub(1) > 0;
}

int DevBuf::reserve(size_t need) {
    if (need <= bytes && ptr) return GSS_OK;
    release();
    size_t cap = 256;
    while (cap < need) cap *= 2;
    if (injected_alloc_failure(cap))
        return set_error(GSS_ERR_NOMEM, "cudaMalloc(%zu) failed: out of memory (injected)", cap);
    cudaError_t e = cudaMalloc(&ptr, cap);
    if (e != cudaSuccess) {
        ptr = nullptr;
        cudaGetLastError();
        return set_error(GSS_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", cap, cudaGetErrorString(e));
    }
    bytes = cap;
    return GSS_OK;
}

int DevBuf::grow_keep(size_t need, cudaStream_t stream, size_t keep_bytes) {
    if (need <= bytes && ptr) return GSS_OK;
    size_t cap = bytes ? bytes : 256;
    while (cap < need) cap *= 2;
    if (injected_alloc_failure(cap))
        return set_error(GSS_ERR_NOMEM, "cudaMalloc(%zu) failed: out of memory (injected)", cap);
    void *np = nullptr;
    cudaError_t e = cudaMalloc(&np, cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(GSS_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", cap, cudaGetErrorString(e));
    }
    if (ptr && keep_bytes) {
        GSS_CUDA_TRY(cudaMemcpyAsync(np, ptr, keep_bytes, cudaMemcpyDeviceToDevice, stream));
        GSS_CUDA_TRY(cudaStreamSynchronize(stream));
    }
    release();
    ptr = np;
    bytes = cap;
    return GSS_OK;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

int PinnedBuf::reserve(size_t need) {
    if (need <= bytes && ptr) return GSS_OK;
    release();
    size_t cap = 4096;
    while (cap < need) cap *= 2;
    cudaError_t e = cudaMallocHost(&ptr, cap);
    if (e != cudaSuccess) {
        ptr = nullptr;
        cudaGetLastError();
        return set_error(GSS_ERR_NOMEM, "cudaMallocHost(%zu) failed: %s", cap, cudaGetErrorString(e));
    }
    bytes = cap;
    return GSS_OK;
}

void PinnedBuf::release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

// Variable-range order key of one clause (see range_order) and, into
// `reordered` when given, its literals with the most frequent range first.
uint64_t range_order_key(const int32_t *lits, int64_t len, int shift, int32_t *reordered) {
    thread_local std::vector<std::pair<int32_t, int32_t>> cnt;  // (range, count)
    cnt.clear();
    for (int64_t i = 0; i < len; i++) {
        const int32_t r = (int32_t) ((uint32_t) lits[i] >> 1 >> shift);
        bool found = false;
        for (auto &p : cnt)
            if (p.first == r) {
                p.second++;
                found = true;
                break;
            }
        if (!found) cnt.push_back({r, 1});
    }
    std::sort(cnt.begin(), cnt.end(), [](const std::pair<int32_t, int32_t> &x, const std::pair<int32_t, int32_t> &y) {
        return x.second != y.second ? x.second > y.second : x.first < y.first;
    });
    if (reordered) {
        int64_t o = 0;
        for (const auto &p : cnt)
            for (int64_t i = 0; i < len; i++)
                if ((int32_t) ((uint32_t) lits[i] >> 1 >> shift) == p.first) reordered[o++] = lits[i];
    }
    if (cnt.empty()) return (uint64_t) len;
    const uint64_t home = (uint64_t) cnt[0].first;
    const uint64_t second = cnt.size() > 1 ? (uint64_t) cnt[1].first : home;
    // 20 bits per range index (ranges of 2^11 variables or more), 13 for the length
    return (home << 33) | (second << 13) | (uint64_t) len;
}

int range_shift_for(int64_t max_var, int range_log2) {
    const int shift = range_log2 < 0 ? 17 : range_log2;
    if (shift == 0 || max_var < 0 || (max_var >> shift) == 0) return 0;
    return shift;
}


}  // namespace gss

using namespace gss;

namespace {

int words_per_lane(int kind) { return kind == GSS_KERNEL_WIDE4 ? 4 : kind == GSS_KERNEL_WIDE2 ? 2 : 1; }

int ensure_device(gss_engine *eng) {
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    return GSS_OK;
}

int ensure_queues(gss_engine *eng) {
    int64_t want = eng->requested_cap;
    if (want <= 0) {
        // Automatic: room for a report per clause and word-block, at least 1M.
        int64_t wb = (eng->n_words + 31) / 32;
        want = std::max<int64_t>(int64_t(1) << 20, eng->n_clauses * std::max<int64_t>(wb, 1) * 2);
    }
    int64_t per = (want + eng->n_parts - 1) / eng->n_parts;
    if (per > 0x7FFFFFFF) per = 0x7FFFFFFF;
    if ((uint32_t) per > eng->cap_per_part || !eng->reports.ptr) {
        GSS_TRY(eng->reports.reserve((size_t) per * eng->n_parts * sizeof(gss_report)));
        eng->cap_per_part = (uint32_t) per;
    }
    GSS_TRY(eng->counts.reserve(sizeof(uint32_t) * eng->n_parts));
    GSS_TRY(eng->h_counts.reserve(sizeof(uint32_t) * (eng->n_parts + 1)));
    return GSS_OK;
}

}  // namespace

extern "C" {

const char *gss_last_error(void) { return g_last_error.c_str(); }

const char *gss_version(void) { return "gpusharesat-gb300 0.1 sm_103a"; }

int gss_debug_fail_device_alloc(int64_t min_bytes, int count) {
    if (count < 0 || min_bytes < 0) return set_error(GSS_ERR_INVALID, "bad arguments to gss_debug_fail_device_alloc");
    g_fail_min_bytes = min_bytes;
    g_fail_count = count;
    return GSS_OK;
}

int gss_max_clause_len(void) { return kMaxClauseLen; }

int gss_engine_create(int device, gss_engine **out) {
    if (!out) return set_error(GSS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int n = 0;
    GSS_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return set_error(GSS_ERR_INVALID, "device %d out of range (%d devices)", device, n);
    gss_engine *eng = new gss_engine();
    eng->device = device;
    int rc = ensure_device(eng);
    if (rc == GSS_OK) {
        cudaError_t e = cudaDeviceGetAttribute(&eng->sm_count, cudaDevAttrMultiProcessorCount, device);
        // the engine's own stream at the highest priority: its check kernels
        // go before work of lower priority, such as the learned order's
        // scoring of the next pass
        int least = 0, greatest = 0;
        if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (e == cudaSuccess)
            e = cudaStreamCreateWithPriority(&eng->own_stream, cudaStreamNonBlocking, greatest);
        if (e != cudaSuccess) rc = set_error(GSS_ERR_CUDA, "engine setup failed: %s", cudaGetErrorString(e));
    }
    if (rc != GSS_OK) {
        delete eng;
        return rc;
    }
    eng->stream = eng->own_stream;
    *out = eng;
    return GSS_OK;
}

int gss_engine_destroy(gss_engine *eng) {
    if (!eng) return GSS_OK;
    cudaSetDevice(eng->device);
    if (eng->stream) cudaStreamSynchronize(eng->stream);
    if (eng->own_stream) cudaStreamDestroy(eng->own_stream);
    if (eng->graph_exec) cudaGraphExecDestroy(eng->graph_exec);
    if (eng->graph) cudaGraphDestroy(eng->graph);
    if (eng->h2d) cudaStreamDestroy(eng->h2d);
    if (eng->d2h) cudaStreamDestroy(eng->d2h);
    for (int b = 0; b < 3; b++) {
        if (eng->ev_h2d[b]) cudaEventDestroy(eng->ev_h2d[b]);
        if (eng->ev_kernel[b]) cudaEventDestroy(eng->ev_kernel[b]);
        if (eng->ev_d2h[b]) cudaEventDestroy(eng->ev_d2h[b]);
    }
    for (auto &p : eng->ev_pending) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    for (auto e : eng->ev_pool) cudaEventDestroy(e);
    order_destroy(eng);
    delete eng;
    return GSS_OK;
}

int gss_engine_set_stream(gss_engine *eng, void *stream) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    eng->stream = stream ? (cudaStream_t) stream : eng->own_stream;
    return GSS_OK;
}

int64_t gss_engine_launch_count(const gss_engine *eng) { return eng ? eng->launches : -1; }

int gss_engine_set_graph(gss_engine *eng, int on) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    eng->use_graph = on != 0;
    return GSS_OK;
}

int64_t gss_engine_graph_captures(const gss_engine *eng) { return eng ? eng->graph_captures : -1; }

int gss_engine_set_timing(gss_engine *eng, int on) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    eng->timing = on != 0;
    return GSS_OK;
}

int gss_engine_kernel_time(gss_engine *eng, double *total_ms, int64_t *n_launches) {
    if (!eng || !total_ms || !n_launches) return set_error(GSS_ERR_INVALID, "bad arguments to gss_engine_kernel_time");
    GSS_TRY(ensure_device(eng));
    double t = 0;
    int64_t n = 0;
    for (auto &p : eng->ev_pending) {
        GSS_CUDA_TRY(cudaEventSynchronize(p.second));
        float ms = 0;
        GSS_CUDA_TRY(cudaEventElapsedTime(&ms, p.first, p.second));
        t += ms;
        n++;
        eng->ev_pool.push_back(p.first);
        eng->ev_pool.push_back(p.second);
    }
    eng->ev_pending.clear();
    *total_ms = t;
    *n_launches = n;
    return GSS_OK;
}

namespace {

// Checks a CSR batch (lengths 1..kMaxClauseLen, non-negative literals) and
// returns its largest variable.
int validate_batch(const int32_t *lits, const int64_t *offsets, int64_t n, int64_t &max_var) {
    if (!offsets || n < 0) return set_error(GSS_ERR_INVALID, "bad clause batch");
    if (n > 0 && offsets[0] != 0) return set_error(GSS_ERR_INVALID, "offsets[0] must be 0");
    for (int64_t c = 0; c < n; c++) {
        const int64_t len = offsets[c + 1] - offsets[c];
        if (len < 1 || len > kMaxClauseLen)
            return set_error(GSS_ERR_INVALID, "clause %lld has length %lld (allowed 1..%d)", (long long) c,
                             (long long) len, kMaxClauseLen);
    }
    const int64_t n_lits = n > 0 ? offsets[n] : 0;
    if (n_lits > 0 && !lits) return set_error(GSS_ERR_INVALID, "lits is NULL");
    max_var = -1;
    for (int64_t i = 0; i < n_lits; i++) {
        if (lits[i] < 0) return set_error(GSS_ERR_INVALID, "literal %lld is negative", (long long) i);
        max_var = std::max<int64_t>(max_var, lits[i] >> 1);
    }
    return GSS_OK;
}

// Stable counting sort of a batch by clause length, as the reference keeps
// clauses in per-size buckets (Clauses.cu:47-51).
void length_order(const int64_t *offsets, int64_t n, std::vector<uint32_t> &order) {
    std::vector<int64_t> count(kMaxClauseLen + 2, 0);
    for (int64_t c = 0; c < n; c++) count[offsets[c + 1] - offsets[c] + 1]++;
    for (int L = 1; L <= kMaxClauseLen + 1; L++) count[L] += count[L - 1];
    order.assign(n, 0);
    for (int64_t c = 0; c < n; c++) order[count[offsets[c + 1] - offsets[c]]++] = (uint32_t) c;
}

// Tiles of the tiled kernel: greedy runs of clauses (in device order) with at
// most kTileLits literals; a longer clause is a tile on its own.
int upload_tiles(gss_engine *eng) {
    const int64_t n = (int64_t) eng->h_off.size() - 1;
    std::vector<uint32_t> tclause, tlit;
    for (int64_t i = 0; i < n;) {
        tclause.push_back((uint32_t) i);
        tlit.push_back((uint32_t) eng->h_off[i]);
        int64_t j = i + 1;
        while (j < n && eng->h_off[j + 1] - eng->h_off[i] <= kTileLits) j++;
        i = j;
    }
    tclause.push_back((uint32_t) n);
    tlit.push_back((uint32_t) eng->h_off[n]);
    GSS_TRY(eng->tile_clause.reserve(tclause.size() * sizeof(uint32_t)));
    GSS_TRY(eng->tile_lit.reserve(tlit.size() * sizeof(uint32_t)));
    GSS_CUDA_TRY(cudaMemcpy(eng->tile_clause.ptr, tclause.data(), tclause.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice));
    GSS_CUDA_TRY(cudaMemcpy(eng->tile_lit.ptr, tlit.data(), tlit.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    eng->n_tiles = (uint32_t) (tclause.size() - 1);
    eng->tiles_stale = false;
    return GSS_OK;
}

// Copies the whole host mirror to the device (after a set or a compaction).
int upload_all(gss_engine *eng) {
    const int64_t n = (int64_t) eng->h_ids.size();
    const int64_t n_lits = eng->h_off.back();
    GSS_TRY(ensure_device(eng));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    // 8 literals of zero padding: tile copies round their end up to 16 bytes
    GSS_TRY(eng->lits.reserve((n_lits + 8) * sizeof(int32_t)));
    GSS_CUDA_TRY(cudaMemset(eng->lits.ptr, 0, (n_lits + 8) * sizeof(int32_t)));
    GSS_TRY(eng->offsets.reserve((n + 1) * sizeof(int64_t)));
    GSS_TRY(eng->orig.reserve(std::max<int64_t>(n, 1) * sizeof(uint32_t)));
    if (n_lits)
        GSS_CUDA_TRY(cudaMemcpy(eng->lits.ptr, eng->h_lits.data(), n_lits * sizeof(int32_t), cudaMemcpyHostToDevice));
    GSS_CUDA_TRY(cudaMemcpy(eng->offsets.ptr, eng->h_off.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    if (n) GSS_CUDA_TRY(cudaMemcpy(eng->orig.ptr, eng->h_ids.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    eng->n_clauses = n;
    eng->n_lits = n_lits;
    eng->n_dead = 0;
    eng->h_alive.assign((n + 31) / 32, ~0u);
    eng->alive_dirty = false;
    eng->tiles_stale = true;
    return GSS_OK;
}

// Variable-range order of a batch. The variables are cut into ranges of
// 2^shift; each clause's literals are reordered by how many of them fall in
// their range (the most frequent range first, ties by range; stable inside a
// range), and the clauses are ordered by (first range, second range, length,
// batch order). Warps that run side by side then gather the state rows of
// one or two ranges for their first literals, a working set that stays in
// L2, where a length-only order gathers rows from the whole state. The rule
// is a symmetric function of a clause's literal values, so neither order
// changes a report. `relits` receives the batch's literals, each clause's
// reordered in place (same offsets as the batch).
void range_order(const int32_t *lits, const int64_t *offsets, int64_t n, int shift, std::vector<uint32_t> &order,
                 std::vector<int32_t> &relits) {
    std::vector<std::pair<uint64_t, uint32_t>> keys((size_t) n);
    const int64_t base = n > 0 ? offsets[0] : 0;
    relits.resize((size_t) (n > 0 ? offsets[n] - base : 0));
    for (int64_t c = 0; c < n; c++) {
        const int64_t b = offsets[c], e = offsets[c + 1];
        keys[c] = {range_order_key(lits + b, e - b, shift, relits.data() + (b - base)), (uint32_t) c};
    }
    std::sort(keys.begin(), keys.end());
    order.resize((size_t) n);
    for (int64_t k = 0; k < n; k++) order[k] = keys[k].second;
}

// log2 of the variables per range for a database whose largest variable is
// max_var: ranges of 2^17 variables (32 MB of state rows at 32 words per
// block) by default; 0 (no ranges) when there would be a single range.
int effective_range_shift(const gss_engine *eng, int64_t max_var) { return range_shift_for(max_var, eng->range_log2); }

// Adds a batch to the host mirror in length order (or variable-range order,
// see range_order); returns the first index.
void mirror_append(gss_engine *eng, const int32_t *lits, const int64_t *offsets, int64_t n, const uint32_t *ids,
                   int64_t max_var) {
    eng->db_version++;
    std::vector<uint32_t> order;
    std::vector<int32_t> relits;
    const int shift = effective_range_shift(eng, max_var);
    const int32_t *src = lits;
    int64_t src_base = 0;  // offsets[c] - src_base indexes src
    if (shift > 0) {
        range_order(lits, offsets, n, shift, order, relits);
        src = relits.data();
        src_base = n > 0 ? offsets[0] : 0;
    } else {
        length_order(offsets, n, order);
    }
    if (eng->h_off.empty()) eng->h_off.push_back(0);
    // room by doubling: an exact reserve per append would copy the whole
    // host database at every append of a clause stream
    const size_t want = eng->h_lits.size() + (size_t) (n > 0 ? offsets[n] - offsets[0] : 0);
    if (want > eng->h_lits.capacity()) eng->h_lits.reserve(std::max(want, 2 * eng->h_lits.capacity()));
    for (int64_t k = 0; k < n; k++) {
        const int64_t c = order[k];
        const int64_t len = offsets[c + 1] - offsets[c];
        const int32_t *cl = src + (offsets[c] - src_base);
        eng->h_lits.insert(eng->h_lits.end(), cl, cl + len);
        eng->h_off.push_back(eng->h_off.back() + len);
        const uint32_t id = ids ? ids[c] : (uint32_t) (eng->next_id + c);
        if (id >= eng->index_of.size()) eng->index_of.resize((size_t) id + 1 + (id >> 3), 0xFFFFFFFFu);
        eng->index_of[id] = (uint32_t) eng->h_ids.size();
        eng->h_ids.push_back(id);
    }
    if (!ids) {
        eng->next_id += (uint32_t) n;
    } else {
        // automatic ids continue after the largest explicit one
        for (int64_t c = 0; c < n; c++) eng->next_id = std::max<uint32_t>(eng->next_id, ids[c] + 1);
    }
}

}  // namespace

int gss_db_set(gss_engine *eng, const int32_t *lits, const int64_t *offsets, int64_t n_clauses) {
    if (!eng || !offsets || n_clauses < 0) return set_error(GSS_ERR_INVALID, "bad arguments to gss_db_set");
    if (n_clauses > 0xFFFFFFF0LL) return set_error(GSS_ERR_INVALID, "too many clauses (%lld)", (long long) n_clauses);
    int64_t max_var = -1;
    GSS_TRY(validate_batch(lits, offsets, n_clauses, max_var));
    order_quiesce(eng);
    if (n_clauses > 0 && offsets[n_clauses] > 0x7FFFFF00LL)
        return set_error(GSS_ERR_INVALID, "too many literals (%lld)", (long long) offsets[n_clauses]);
    eng->h_lits.clear();
    eng->h_off.assign(1, 0);
    eng->h_ids.clear();
    eng->index_of.clear();
    eng->next_id = 0;
    eng->db_epoch++;
    eng->layout_epoch++;
    mirror_append(eng, lits, offsets, n_clauses, nullptr, max_var);
    GSS_TRY(upload_all(eng));
    eng->max_var = max_var;
    return GSS_OK;
}

int gss_db_append(gss_engine *eng, const int32_t *lits, const int64_t *offsets, int64_t n_clauses,
                  const uint32_t *ids) {
    if (!eng || !offsets || n_clauses < 0) return set_error(GSS_ERR_INVALID, "bad arguments to gss_db_append");
    if (n_clauses == 0) return GSS_OK;
    order_quiesce(eng);
    int64_t max_var = -1;
    GSS_TRY(validate_batch(lits, offsets, n_clauses, max_var));
    const int64_t first = (int64_t) eng->h_ids.size();
    if (first + n_clauses > 0xFFFFFFF0LL) return set_error(GSS_ERR_INVALID, "too many clauses");
    if (ids) {
        for (int64_t c = 0; c < n_clauses; c++)
            if (ids[c] < eng->index_of.size() && eng->index_of[ids[c]] != 0xFFFFFFFFu)
                return set_error(GSS_ERR_INVALID, "clause id %u is already in the database", ids[c]);
    }
    const int64_t base = eng->h_off.empty() ? 0 : eng->h_off.back();
    if (base + offsets[n_clauses] > 0x7FFFFF00LL) return set_error(GSS_ERR_INVALID, "too many literals");
    mirror_append(eng, lits, offsets, n_clauses, ids, std::max(eng->max_var, max_var));
    const int64_t n = (int64_t) eng->h_ids.size();
    const int64_t n_lits = eng->h_off.back();
    GSS_TRY(ensure_device(eng));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    GSS_TRY(eng->lits.grow_keep((n_lits + 8) * sizeof(int32_t), eng->stream, base * sizeof(int32_t)));
    GSS_TRY(eng->offsets.grow_keep((n + 1) * sizeof(int64_t), eng->stream, (first + 1) * sizeof(int64_t)));
    GSS_TRY(eng->orig.grow_keep(n * sizeof(uint32_t), eng->stream, first * sizeof(uint32_t)));
    // new literals, then zero padding past the end
    std::vector<int32_t> tail(eng->h_lits.begin() + base, eng->h_lits.end());
    tail.resize(tail.size() + 8, 0);
    GSS_CUDA_TRY(cudaMemcpy((int32_t *) eng->lits.ptr + base, tail.data(), tail.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
    GSS_CUDA_TRY(cudaMemcpy((int64_t *) eng->offsets.ptr + first, eng->h_off.data() + first,
                            (n - first + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    GSS_CUDA_TRY(cudaMemcpy((uint32_t *) eng->orig.ptr + first, eng->h_ids.data() + first,
                            (n - first) * sizeof(uint32_t), cudaMemcpyHostToDevice));
    // alive bits of the new clauses
    eng->h_alive.resize((n + 31) / 32, 0u);
    for (int64_t i = first; i < n; i++) eng->h_alive[i >> 5] |= 1u << (i & 31);
    eng->alive_dirty = true;
    eng->n_clauses = n;
    eng->n_lits = n_lits;
    eng->max_var = std::max(eng->max_var, max_var);
    eng->tiles_stale = true;
    return GSS_OK;
}

int gss_db_delete(gss_engine *eng, const uint32_t *ids, int64_t n) {
    if (!eng || n < 0 || (n > 0 && !ids)) return set_error(GSS_ERR_INVALID, "bad arguments to gss_db_delete");
    order_quiesce(eng);
    int64_t missing = 0;
    for (int64_t k = 0; k < n; k++) {
        const uint32_t id = ids[k];
        if (id >= eng->index_of.size() || eng->index_of[id] == 0xFFFFFFFFu) {
            missing++;
            continue;
        }
        const uint32_t i = eng->index_of[id];
        if (eng->h_alive[i >> 5] & (1u << (i & 31))) {
            eng->h_alive[i >> 5] &= ~(1u << (i & 31));
            eng->n_dead++;
        }
        eng->index_of[id] = 0xFFFFFFFFu;
    }
    eng->alive_dirty = true;
    if (missing) return set_error(GSS_ERR_NOT_FOUND, "%lld clause id(s) not in the database", (long long) missing);
    return GSS_OK;
}

int gss_db_compact(gss_engine *eng) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    if (eng->n_dead == 0) return GSS_OK;
    order_quiesce(eng);
    eng->layout_epoch++;
    // the live clauses, re-sorted by length (stable)
    std::vector<int32_t> lits;
    std::vector<int64_t> off(1, 0);
    std::vector<uint32_t> ids;
    const int64_t n = (int64_t) eng->h_ids.size();
    for (int64_t i = 0; i < n; i++) {
        if (!(eng->h_alive[i >> 5] & (1u << (i & 31)))) continue;
        lits.insert(lits.end(), eng->h_lits.begin() + eng->h_off[i], eng->h_lits.begin() + eng->h_off[i + 1]);
        off.push_back((int64_t) lits.size());
        ids.push_back(eng->h_ids[i]);
    }
    const uint32_t next = eng->next_id;
    eng->h_lits.clear();
    eng->h_off.assign(1, 0);
    eng->h_ids.clear();
    std::fill(eng->index_of.begin(), eng->index_of.end(), 0xFFFFFFFFu);
    mirror_append(eng, lits.data(), off.data(), (int64_t) ids.size(), ids.data(), eng->max_var);
    eng->next_id = next;
    return upload_all(eng);
}

int gss_db_set_locality(gss_engine *eng, int range_log2) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    if (range_log2 != -1 && range_log2 != 0 && (range_log2 < 11 || range_log2 > 31))
        return set_error(GSS_ERR_INVALID, "range_log2 must be -1 (automatic), 0 (off) or 11..31, not %d", range_log2);
    eng->range_log2 = range_log2;
    return GSS_OK;
}

int gss_db_locality_shift(const gss_engine *eng) { return eng ? effective_range_shift(eng, eng->max_var) : -1; }

int64_t gss_db_live_count(const gss_engine *eng) { return eng ? eng->n_clauses - eng->n_dead : -1; }

int64_t gss_db_clause_count(const gss_engine *eng) { return eng ? eng->n_clauses : -1; }
int64_t gss_db_literal_count(const gss_engine *eng) { return eng ? eng->n_lits : -1; }
int64_t gss_db_max_var(const gss_engine *eng) { return eng ? eng->max_var : -1; }

int gss_engine_set_length_plan(gss_engine *eng, int n_classes, const int32_t *max_len, const int32_t *layout) {
    if (!eng || n_classes < 0 || (n_classes > 0 && (!max_len || !layout)))
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_engine_set_length_plan");
    for (int k = 0; k < n_classes; k++) {
        if (layout[k] != GSS_LAYOUT_SKIP && layout_lanes(layout[k]) == 0)
            return set_error(GSS_ERR_INVALID, "unknown lane layout %d", layout[k]);
        if (k > 0 && max_len[k] <= max_len[k - 1])
            return set_error(GSS_ERR_INVALID, "class bounds must increase");
    }
    eng->plan_max_len.assign(max_len, max_len + n_classes);
    eng->plan_layout.assign(layout, layout + n_classes);
    eng->plan_built = ~0ull;
    return GSS_OK;
}

int gss_db_positions(const gss_engine *eng, const uint32_t *ids, int64_t n, int64_t *positions) {
    if (!eng || n < 0 || (n > 0 && (!ids || !positions))) return set_error(GSS_ERR_INVALID, "bad arguments");
    for (int64_t i = 0; i < n; i++) {
        const uint32_t id = ids[i];
        const uint32_t pos = id < eng->index_of.size() ? eng->index_of[id] : 0xFFFFFFFFu;
        positions[i] = pos == 0xFFFFFFFFu ? -1 : (int64_t) pos;
    }
    return GSS_OK;
}

int gss_state_set(gss_engine *eng, const uint32_t *state, int64_t n_vars, int n_words, const uint32_t *start,
                  const int32_t *solver_of_word, int on_device) {
    if (!eng || n_vars < 0 || n_words < 0 || (n_vars > 0 && n_words > 0 && !state) || (n_words > 0 && !start))
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_state_set");
    if (n_words > 4096) return set_error(GSS_ERR_INVALID, "at most 4096 words (131072 slots) per pass");
    if (n_vars > 0x7FFFFFFF) return set_error(GSS_ERR_INVALID, "too many variables");
    GSS_TRY(ensure_device(eng));
    int kind = eng->kind, lpc = eng->lpc, depth = eng->g;
    if (kind == GSS_KERNEL_AUTO) {
        // Measured on GB300 for the at-scale workload: four words per lane with
        // 256-bit loads, two loads in flight, is fastest once a clause spans
        // eight or more words; below that one word per lane.
        depth = 2;
        if (n_words >= 8) {
            kind = GSS_KERNEL_WIDE4;
            lpc = n_words >= 32 ? 8 : n_words >= 16 ? 4 : 2;
        } else {
            kind = GSS_KERNEL_DIRECT;
            lpc = 1;
            while (lpc < n_words) lpc *= 2;
            if (lpc == 1) depth = 1;
        }
    }
    const int wpl = words_per_lane(kind);
    if (lpc == 0) {
        // one word per lane up to a full warp (wide kinds: 32 words per block)
        lpc = 1;
        if (wpl == 1) {
            while (lpc < n_words && lpc < 32) lpc *= 2;
            if (depth > lpc) depth = lpc;  // a lane group has lpc literals in flight at most
        } else {
            lpc = 32 / wpl;
        }
    }
    const int bw = lpc * wpl;
    const int n_blocks = (n_words + bw - 1) / bw;
    const int padded = n_blocks * bw;
    const size_t sbytes = (size_t) n_vars * n_words * 2 * sizeof(uint32_t);
    const size_t bbytes = (size_t) n_blocks * n_vars * bw * 2 * sizeof(uint32_t);
    if (eng->pass_pending) GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    GSS_TRY(eng->state.reserve(std::max<size_t>(bbytes, 8)));
    GSS_TRY(eng->start.reserve(std::max<size_t>(padded * sizeof(uint32_t), 4)));
    GSS_TRY(eng->solver_of_word.reserve(std::max<size_t>(padded * sizeof(int32_t), 4)));
    // start and solver_of_word, padded with zero words
    std::vector<uint32_t> st(padded, 0u);
    std::vector<int32_t> sw(padded, 0);
    if (n_words) {
        if (on_device) {
            GSS_CUDA_TRY(cudaMemcpy(st.data(), start, n_words * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            if (solver_of_word)
                GSS_CUDA_TRY(cudaMemcpy(sw.data(), solver_of_word, n_words * sizeof(int32_t), cudaMemcpyDeviceToHost));
        } else {
            memcpy(st.data(), start, n_words * sizeof(uint32_t));
            if (solver_of_word) memcpy(sw.data(), solver_of_word, n_words * sizeof(int32_t));
        }
        if (!solver_of_word)
            for (int w = 0; w < n_words; w++) sw[w] = w;
    }
    if (padded) {
        GSS_CUDA_TRY(cudaMemcpyAsync(eng->start.ptr, st.data(), padded * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                     eng->stream));
        GSS_CUDA_TRY(cudaMemcpyAsync(eng->solver_of_word.ptr, sw.data(), padded * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, eng->stream));
    }
    if (sbytes) {
        if (n_blocks == 1 && n_words == bw) {
            // block-major and host layouts coincide
            GSS_CUDA_TRY(cudaMemcpyAsync(eng->state.ptr, state, sbytes,
                                         on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, eng->stream));
        } else {
            const uint2 *src = (const uint2 *) state;
            if (!on_device) {
                GSS_TRY(eng->state_raw.reserve(sbytes));
                GSS_CUDA_TRY(cudaMemcpyAsync(eng->state_raw.ptr, state, sbytes, cudaMemcpyHostToDevice, eng->stream));
                src = (const uint2 *) eng->state_raw.ptr;
            }
            GSS_TRY(launch_relayout(src, (uint2 *) eng->state.ptr, (uint32_t) n_vars, (uint32_t) n_words,
                                    (uint32_t) bw, (uint32_t) n_blocks, eng->stream, eng->sm_count));
        }
    }
    // the host vectors above are pageable: the async copies from them complete before return
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    eng->n_vars = n_vars;
    eng->n_words = n_words;
    eng->n_blocks = n_blocks;
    eng->state_kind = kind;
    eng->state_lpc = lpc;
    eng->state_g = depth;
    eng->state_bw = bw;
    return GSS_OK;
}

int gss_state_set_start(gss_engine *eng, const uint32_t *start, int n_words) {
    if (!eng || n_words != eng->n_words || (n_words > 0 && !start))
        return set_error(GSS_ERR_INVALID, "gss_state_set_start needs the %d words of the current state", eng ? eng->n_words : 0);
    GSS_TRY(ensure_device(eng));
    std::vector<uint32_t> st((size_t) eng->n_blocks * eng->state_bw, 0u);
    memcpy(st.data(), start, n_words * sizeof(uint32_t));
    if (eng->pass_pending) GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    GSS_CUDA_TRY(cudaMemcpyAsync(eng->start.ptr, st.data(), st.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 eng->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    return GSS_OK;
}

int gss_engine_set_variant(gss_engine *eng, int kind, int lanes_per_clause, int depth, int flags) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    if (kind == GSS_KERNEL_AUTO) {
        // nothing to validate: resolved per word count
    } else if (kind == GSS_KERNEL_WIDE4 || kind == GSS_KERNEL_WIDE2) {
        const int wpl = words_per_lane(kind);
        const int l = lanes_per_clause ? lanes_per_clause : 32 / wpl;
        if ((flags & GSS_VARIANT_PERSISTENT) ? !valid_wide_persist_variant(wpl, l, depth)
            : (flags & GSS_VARIANT_PIPELINED) ? !valid_wide_pf_variant(wpl, l, depth)
                                              : !valid_wide_variant(wpl, l, depth, (flags & GSS_VARIANT_OCCUPANCY) ? 1 : 0))
            return set_error(GSS_ERR_INVALID, "no wide kernel variant for %d words per lane, %d lanes, depth %d", wpl,
                             l, depth);
    } else if (kind == GSS_KERNEL_DIRECT) {
        if (lanes_per_clause == 0 ? !(depth == 1 || depth == 2 || depth == 4 || depth == 8)
                                  : !valid_variant(lanes_per_clause, depth))
            return set_error(GSS_ERR_INVALID, "no direct kernel variant for %d lanes per clause, depth %d",
                             lanes_per_clause, depth);
    } else if (kind == GSS_KERNEL_TILED) {
        if (lanes_per_clause != 0 && !valid_tiled_variant(lanes_per_clause, depth))
            return set_error(GSS_ERR_INVALID, "no tiled kernel variant for %d lanes per clause, %d slots",
                             lanes_per_clause, depth);
        if (lanes_per_clause == 0 && !valid_tiled_variant(32, depth))
            return set_error(GSS_ERR_INVALID, "no tiled kernel variant with %d slots", depth);
    } else {
        return set_error(GSS_ERR_INVALID, "unknown kernel kind %d", kind);
    }
    eng->kind = kind;
    eng->lpc = lanes_per_clause;
    eng->g = depth;
    eng->flags = flags;
    return GSS_OK;
}

int gss_check_set_capacity(gss_engine *eng, int64_t records) {
    if (!eng || records < 0) return set_error(GSS_ERR_INVALID, "bad arguments to gss_check_set_capacity");
    eng->requested_cap = records;
    return GSS_OK;
}

namespace {

// Launches one check pass of the engine's database against `state` (laid out
// as the engine's current state), into `reports`/`counts`, then copies the
// counts and the error flag into `h_counts` (pinned), all on the engine's
// stream.
int launch_pass_into(gss_engine *eng, const void *state, DevBuf &reports, DevBuf &counts, PinnedBuf &h_counts);

}  // namespace

int gss_check_launch(gss_engine *eng) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    GSS_TRY(ensure_device(eng));
    GSS_TRY(ensure_queues(eng));
    GSS_TRY(launch_pass_into(eng, eng->state.ptr, eng->reports, eng->counts, eng->h_counts));
    eng->launches++;
    eng->pass_pending = true;
    return GSS_OK;
}

namespace {

// The position ranges of the length plan over the database as it is now:
// runs of positions whose clauses fall in one length class (the database is
// sorted by length, appended batches each sorted), skipped classes left out.
int build_plan(gss_engine *eng) {
    if (eng->plan_built == eng->db_version) return GSS_OK;
    static_assert(sizeof(BucketPlan) < (1u << 20), "plan size");
    std::vector<BucketPlan> hp(1);
    BucketPlan &p = hp[0];
    memset(&p, 0, sizeof p);
    const std::vector<int32_t> &bound = eng->plan_max_len;
    const int n_classes = (int) bound.size();
    int prev_class = -1;
    uint32_t groups = 0;
    auto close_range = [&]() {
        if (p.n_ranges == 0) return;
        const uint32_t k = p.n_ranges - 1;
        const uint32_t cpw = 32u / (uint32_t) layout_lanes(p.layout[k]);
        p.group_base[k] = groups;
        groups += (p.range_end[k] - p.range_begin[k] + cpw - 1) / cpw;
    };
    for (int64_t c = 0; c < eng->n_clauses; c++) {
        const int32_t len = (int32_t) (eng->h_off[c + 1] - eng->h_off[c]);
        int cls = (int) (std::lower_bound(bound.begin(), bound.end(), len) - bound.begin());
        if (cls >= n_classes) cls = n_classes - 1;
        if (cls == prev_class && p.n_ranges > 0 && p.range_end[p.n_ranges - 1] == (uint32_t) c) {
            p.range_end[p.n_ranges - 1] = (uint32_t) (c + 1);
            continue;
        }
        prev_class = cls;
        if (eng->plan_layout[cls] == GSS_LAYOUT_SKIP) continue;
        if (p.n_ranges == kMaxRanges)
            return set_error(GSS_ERR_STATE, "the length plan needs more than %u position ranges (compact the database)",
                             kMaxRanges);
        close_range();
        p.range_begin[p.n_ranges] = (uint32_t) c;
        p.range_end[p.n_ranges] = (uint32_t) (c + 1);
        p.layout[p.n_ranges] = eng->plan_layout[cls];
        p.n_ranges++;
    }
    close_range();
    p.group_base[p.n_ranges] = groups;
    GSS_TRY(eng->d_plan.reserve(sizeof(BucketPlan)));
    GSS_CUDA_TRY(cudaMemcpyAsync(eng->d_plan.ptr, &p, sizeof(BucketPlan), cudaMemcpyHostToDevice, eng->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));  // pageable source
    eng->plan_ranges = p.n_ranges;
    eng->plan_built = eng->db_version;
    return GSS_OK;
}

int launch_pass_into(gss_engine *eng, const void *state, DevBuf &reports, DevBuf &counts, PinnedBuf &h_counts) {
    order_quiesce(eng);  // a scoring in flight reads the buffers this pass may reallocate
    if (eng->n_clauses > 0 && eng->max_var >= eng->n_vars)
        return set_error(GSS_ERR_INVALID, "database uses variable %lld but the state has %lld variables",
                         (long long) eng->max_var, (long long) eng->n_vars);
    if (eng->n_words > 0 && eng->kind != GSS_KERNEL_AUTO &&
        (eng->state_kind != eng->kind || (eng->lpc != 0 && eng->state_lpc != eng->lpc) || eng->state_g != eng->g))
        return set_error(GSS_ERR_STATE, "the state was laid out for another kernel variant; set it again after "
                         "changing the variant");
    if (eng->state_kind == GSS_KERNEL_DIRECT && !valid_variant(eng->state_lpc, eng->state_g) && eng->n_words > 0)
        return set_error(GSS_ERR_STATE, "no direct kernel variant for %d lanes per clause", eng->state_lpc);
    CheckArgs a;
    memset(&a, 0, sizeof a);
    a.lits = (const int32_t *) eng->lits.ptr;
    a.offsets = (const int64_t *) eng->offsets.ptr;
    a.orig = (const uint32_t *) eng->orig.ptr;
    a.n_clauses = (uint32_t) eng->n_clauses;
    a.scan_begin = 0;
    a.scan_end = a.n_clauses;
    a.state = (const uint2 *) state;
    a.n_vars = (uint32_t) eng->n_vars;
    a.n_blocks = (uint32_t) eng->n_blocks;
    a.lpc = eng->state_lpc;
    a.g = eng->state_g;
    a.cache_hints = (eng->flags & GSS_VARIANT_L2_HINT) ? 1 : 0;
    if (eng->state_kind == GSS_KERNEL_TILED) {
        if (eng->n_dead > 0)
            return set_error(GSS_ERR_STATE, "the tiled kernel needs a compacted database (gss_db_compact)");
        if (eng->tiles_stale) GSS_TRY(upload_tiles(eng));
    }
    a.tile_clause = (const uint32_t *) eng->tile_clause.ptr;
    a.tile_lit = (const uint32_t *) eng->tile_lit.ptr;
    a.n_tiles = eng->n_tiles;
    a.alive = nullptr;
    if (eng->n_dead > 0) {
        if (eng->alive_dirty) {
            GSS_TRY(eng->alive.reserve(std::max<size_t>(eng->h_alive.size(), 1) * sizeof(uint32_t)));
            GSS_CUDA_TRY(cudaMemcpyAsync(eng->alive.ptr, eng->h_alive.data(), eng->h_alive.size() * sizeof(uint32_t),
                                         cudaMemcpyHostToDevice, eng->stream));
            GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));  // pageable source
            eng->alive_dirty = false;
        }
        a.alive = (const uint32_t *) eng->alive.ptr;
    }
    GSS_TRY(eng->err.reserve(sizeof(uint32_t)));
    a.err = (uint32_t *) eng->err.ptr;
    a.start = (const uint32_t *) eng->start.ptr;
    a.solver_of_word = (const int32_t *) eng->solver_of_word.ptr;
    a.out = (gss_report *) reports.ptr;
    a.counts = (uint32_t *) counts.ptr;
    a.n_parts = eng->n_parts;
    a.cap_per_part = eng->cap_per_part;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (eng->timing) {
        for (cudaEvent_t *ev : {&ev0, &ev1}) {
            if (!eng->ev_pool.empty()) {
                *ev = eng->ev_pool.back();
                eng->ev_pool.pop_back();
            } else {
                GSS_CUDA_TRY(cudaEventCreate(ev));
            }
        }
    }
    const bool wide = eng->state_kind == GSS_KERNEL_WIDE4 || eng->state_kind == GSS_KERNEL_WIDE2;
    const bool ordered = order_active(eng);
    const bool bucketed = !eng->plan_layout.empty();
    // The automatic variant runs the persistent form of the wide kernel: tasks
    // from a work counter keep the warps on neighbouring clause groups (the
    // database order's L2 locality holds) and balance uneven clause lengths;
    // measured 0.91 ms against 1.13 ms for the grid-stride form on the
    // at-scale workload.
    const bool persistent =
        wide && ((eng->flags & GSS_VARIANT_PERSISTENT) ||
                 (eng->kind == GSS_KERNEL_AUTO &&
                  valid_wide_persist_variant(words_per_lane(eng->state_kind), eng->state_lpc, eng->state_g)));
    if (ordered && (eng->state_kind == GSS_KERNEL_TILED || bucketed))
        return set_error(GSS_ERR_STATE, "the learned scan order runs the direct, wide and persistent kernels (not the "
                         "tiled or bucketed ones)");
    if (bucketed && eng->n_words > 0 && eng->state_bw != 32)
        return set_error(GSS_ERR_STATE, "the length plan needs a state laid out in 32-word blocks (%d here)",
                         eng->state_bw);
    if (ordered && (&reports != &eng->reports || &counts != &eng->counts))
        return set_error(GSS_ERR_STATE, "the learned scan order runs through gss_check_launch");
    if (bucketed || (persistent && eng->use_graph && !ordered)) {
        // arguments through device memory, so the same graph serves every pass
        if (bucketed) GSS_TRY(build_plan(eng));
        GSS_TRY(eng->d_args.reserve(sizeof(CheckArgs)));
        GSS_TRY(eng->work.reserve(sizeof(uint32_t)));
        GSS_CUDA_TRY(cudaMemcpyAsync(eng->d_args.ptr, &a, sizeof a, cudaMemcpyHostToDevice, eng->stream));
        if (ev0) GSS_CUDA_TRY(cudaEventRecord(ev0, eng->stream));
        auto body = [&]() -> int {
            GSS_CUDA_TRY(cudaMemsetAsync(a.counts, 0, sizeof(uint32_t) * a.n_parts, eng->stream));
            GSS_CUDA_TRY(cudaMemsetAsync(a.err, 0, sizeof(uint32_t), eng->stream));
            GSS_CUDA_TRY(cudaMemsetAsync(eng->work.ptr, 0, sizeof(uint32_t), eng->stream));
            if (a.n_clauses > 0 && a.n_blocks > 0) {
                if (bucketed) {
                    if (eng->plan_ranges > 0)
                        GSS_TRY(launch_check_bucketed((const CheckArgs *) eng->d_args.ptr,
                                                      (const BucketPlan *) eng->d_plan.ptr, (uint32_t *) eng->work.ptr,
                                                      eng->stream, eng->sm_count));
                } else {
                    GSS_TRY(launch_check_wide_persist((const CheckArgs *) eng->d_args.ptr, a,
                                                      words_per_lane(eng->state_kind), eng->state_lpc, eng->state_g,
                                                      (uint32_t *) eng->work.ptr, eng->stream, eng->sm_count));
                }
            }
            GSS_CUDA_TRY(cudaMemcpyAsync(h_counts.ptr, counts.ptr, sizeof(uint32_t) * eng->n_parts,
                                         cudaMemcpyDeviceToHost, eng->stream));
            GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) h_counts.ptr + eng->n_parts, a.err, sizeof(uint32_t),
                                         cudaMemcpyDeviceToHost, eng->stream));
            return GSS_OK;
        };
        if (eng->use_graph) {
            const std::vector<uintptr_t> key = {
                (uintptr_t) a.counts, (uintptr_t) h_counts.ptr, (uintptr_t) a.err, (uintptr_t) eng->work.ptr,
                (uintptr_t) eng->d_args.ptr, (uintptr_t) eng->state_kind, (uintptr_t) eng->state_lpc,
                (uintptr_t) eng->state_g, (uintptr_t) eng->n_parts, (uintptr_t) (a.n_clauses > 0 && a.n_blocks > 0),
                (uintptr_t) bucketed, (uintptr_t) eng->d_plan.ptr, (uintptr_t) (eng->plan_ranges > 0)};
            if (key != eng->graph_key || !eng->graph_exec) {
                if (eng->graph_exec) cudaGraphExecDestroy(eng->graph_exec);
                if (eng->graph) cudaGraphDestroy(eng->graph);
                eng->graph_exec = nullptr;
                eng->graph = nullptr;
                GSS_CUDA_TRY(cudaStreamBeginCapture(eng->stream, cudaStreamCaptureModeThreadLocal));
                const int rc = body();
                cudaGraph_t g = nullptr;
                const cudaError_t e = cudaStreamEndCapture(eng->stream, &g);
                GSS_TRY(rc);
                if (e != cudaSuccess) return set_error(GSS_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
                eng->graph = g;
                GSS_CUDA_TRY(cudaGraphInstantiate(&eng->graph_exec, g, 0));
                eng->graph_key = key;
                eng->graph_captures++;
            }
            GSS_CUDA_TRY(cudaGraphLaunch(eng->graph_exec, eng->stream));
        } else {
            GSS_TRY(body());
        }
        if (ev1) {
            GSS_CUDA_TRY(cudaEventRecord(ev1, eng->stream));
            eng->ev_pending.emplace_back(ev0, ev1);
        }
        return GSS_OK;
    }
    GSS_CUDA_TRY(cudaMemsetAsync(a.counts, 0, sizeof(uint32_t) * a.n_parts, eng->stream));
    GSS_CUDA_TRY(cudaMemsetAsync(a.err, 0, sizeof(uint32_t), eng->stream));
    if (ev0) GSS_CUDA_TRY(cudaEventRecord(ev0, eng->stream));
    if (persistent) GSS_TRY(eng->work.reserve(sizeof(uint32_t)));
    auto launch = [&](const CheckArgs &args) -> int {
        if (eng->state_kind == GSS_KERNEL_TILED) return launch_check_tiled(args, eng->stream, eng->sm_count);
        if (persistent) {
            // arguments by value; the work counter restarts for each launch
            GSS_CUDA_TRY(cudaMemsetAsync(eng->work.ptr, 0, sizeof(uint32_t), eng->stream));
            if (args.n_clauses == 0 || args.n_blocks == 0 || scan_count(args) == 0) return GSS_OK;
            return launch_check_wide_persist(nullptr, args, words_per_lane(eng->state_kind), eng->state_lpc,
                                             eng->state_g, (uint32_t *) eng->work.ptr, eng->stream, eng->sm_count);
        }
        const int occ = (eng->flags & GSS_VARIANT_OCCUPANCY) ? 1 : 0;
        if (wide && (eng->flags & GSS_VARIANT_PIPELINED))
            return launch_check_wide_pf(args, words_per_lane(eng->state_kind), occ, eng->stream, eng->sm_count);
        if (wide) return launch_check_wide(args, words_per_lane(eng->state_kind), occ, eng->stream, eng->sm_count);
        return launch_check(args, eng->stream, eng->sm_count);
    };
    if (ordered) {
        // learned order: score and sort, then the head of the scan, its
        // counts for early delivery, the tail, and the history update
        uint32_t head = 0, covered = 0;
        GSS_TRY(order_prepare(eng, &a.perm, &head, &covered));
        // positions appended since the order was computed (from `covered`
        // on) are scanned in place at the end of the tail
        a.perm_end = covered;
        a.scan_begin = 0;
        a.scan_end = head;
        if (head) GSS_TRY(launch(a));
        GSS_TRY(order_after_head(eng, counts));
        a.scan_begin = head;
        a.scan_end = a.n_clauses;
        if (head < a.n_clauses) GSS_TRY(launch(a));
        GSS_TRY(order_after_pass(eng, reports, counts));
    } else {
        GSS_TRY(launch(a));
    }
    if (ev1) {
        GSS_CUDA_TRY(cudaEventRecord(ev1, eng->stream));
        eng->ev_pending.emplace_back(ev0, ev1);
    }
    GSS_CUDA_TRY(cudaMemcpyAsync(h_counts.ptr, counts.ptr, sizeof(uint32_t) * eng->n_parts, cudaMemcpyDeviceToHost,
                                 eng->stream));
    GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) h_counts.ptr + eng->n_parts, a.err, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, eng->stream));
    return GSS_OK;
}

}  // namespace


int gss_check_wait(gss_engine *eng, int64_t *n_reports) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    GSS_TRY(ensure_device(eng));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    eng->pass_pending = false;
    if (!eng->h_counts.ptr) {  // no pass launched yet: nothing to report
        if (n_reports) *n_reports = 0;
        return GSS_OK;
    }
    const uint32_t *hc = (const uint32_t *) eng->h_counts.ptr;
    int64_t total = 0;
    bool overflow = false;
    for (uint32_t p = 0; p < eng->n_parts; p++) {
        total += hc[p];
        if (hc[p] > eng->cap_per_part) overflow = true;
    }
    if (n_reports) *n_reports = total;
    if (hc[eng->n_parts] != 0)
        return set_error(GSS_ERR_CUDA, "a bounded wait in the check kernel gave up (flag %u); the pass is incomplete",
                         hc[eng->n_parts]);
    if (overflow) {
        // Next automatic capacity: twice what this pass needed.
        eng->requested_cap = std::max<int64_t>(eng->requested_cap, total * 2 + eng->n_parts * 1024);
        return set_error(GSS_ERR_OVERFLOW, "report queues overflowed (%lld reports, %u per partition)",
                         (long long) total, eng->cap_per_part);
    }
    return GSS_OK;
}

int gss_check_copy_reports(gss_engine *eng, gss_report *out, int64_t cap, int64_t *n_reports) {
    if (!eng || (cap > 0 && !out)) return set_error(GSS_ERR_INVALID, "bad arguments to gss_check_copy_reports");
    int64_t total = 0;
    GSS_TRY(gss_check_wait(eng, &total));
    if (n_reports) *n_reports = total;
    if (total > cap) return set_error(GSS_ERR_OVERFLOW, "output holds %lld records, pass has %lld", (long long) cap,
                                      (long long) total);
    if (total == 0) return GSS_OK;
    const uint32_t *hc = (const uint32_t *) eng->h_counts.ptr;
    int64_t pos = 0;
    for (uint32_t p = 0; p < eng->n_parts; p++) {
        if (hc[p] == 0) continue;
        GSS_CUDA_TRY(cudaMemcpyAsync(out + pos, (gss_report *) eng->reports.ptr + (size_t) p * eng->cap_per_part,
                                     (size_t) hc[p] * sizeof(gss_report), cudaMemcpyDeviceToHost, eng->stream));
        pos += hc[p];
    }
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    return GSS_OK;
}

int gss_check_pass_host(gss_engine *eng, const uint32_t *state, int64_t n_vars, int n_words, const uint32_t *start,
                        const int32_t *solver_of_word, gss_report *out, int64_t cap, int64_t *n_reports) {
    GSS_TRY(gss_state_set(eng, state, n_vars, n_words, start, solver_of_word, 0));
    for (int attempt = 0; attempt < 4; attempt++) {
        GSS_TRY(gss_check_launch(eng));
        int64_t total = 0;
        int rc = gss_check_wait(eng, &total);
        if (rc == GSS_ERR_OVERFLOW) continue;  // capacity was raised; run the pass again
        GSS_TRY(rc);
        return gss_check_copy_reports(eng, out, cap, n_reports);
    }
    return set_error(GSS_ERR_OVERFLOW, "report queues kept overflowing");
}

}  // extern "C"

namespace {

// Record formats of passes through host buffers.
enum HostRecords { kRecordsFull = 0, kRecordsPacked = 1, kRecordsCells = 2 };

// Passes through host buffers; outs[i] receives gss_report records, or
// records packed on the device: 12-byte {clause, word, mask} (kRecordsPacked)
// or 8-byte {clause * n_words + word, mask} (kRecordsCells).
int passes_host(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars, int n_words,
                const uint32_t *start, const int32_t *solver_of_word, void *const *outs, const int64_t *caps,
                int64_t *n_reports, int format) {
    const bool packed = format != kRecordsFull;
    const uint32_t rec_words = format == kRecordsCells ? 2u : 3u;  // 32-bit words per packed record
    if (format == kRecordsCells && eng && n_words > 0 && (uint64_t) eng->next_id * (uint64_t) n_words > 0xFFFFFFFFull)
        return set_error(GSS_ERR_INVALID, "cell records need (largest clause id + 1) x words <= 2^32 (%u ids x %d words)",
                         eng->next_id, n_words);
    // Passes i = 0..n-1 over three streams: the state of pass i+1 goes
    // host->device (h2d stream) and the reports of pass i-1 come back (d2h
    // stream) while pass i runs (engine stream). Three buffer slots: state b
    // and report set b belong to passes b, b+3, b+6..., so a copy waits for
    // the pass three back, not the one just before.
    if (!eng || n_passes < 0 || (n_passes > 0 && (!states || !outs || !caps || !n_reports)))
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_check_passes_host");
    if (n_passes == 0) return GSS_OK;
    GSS_TRY(ensure_device(eng));
    // layout, start and solver words from the first pass (copies its state too)
    GSS_TRY(gss_state_set(eng, states[0], n_vars, n_words, start, solver_of_word, 0));
    GSS_TRY(ensure_queues(eng));
    const bool direct = eng->n_blocks == 1 && eng->n_words == eng->state_bw;
    const size_t sbytes = (size_t) n_vars * n_words * 2 * sizeof(uint32_t);
    const size_t bbytes = (size_t) eng->n_blocks * n_vars * eng->state_bw * sizeof(uint2);
    if (!eng->h2d) GSS_CUDA_TRY(cudaStreamCreateWithFlags(&eng->h2d, cudaStreamNonBlocking));
    if (!eng->d2h) GSS_CUDA_TRY(cudaStreamCreateWithFlags(&eng->d2h, cudaStreamNonBlocking));
    constexpr int NB = 3;
    for (int b = 0; b < NB; b++) {
        if (!eng->ev_h2d[b]) GSS_CUDA_TRY(cudaEventCreateWithFlags(&eng->ev_h2d[b], cudaEventDisableTiming));
        if (!eng->ev_kernel[b]) GSS_CUDA_TRY(cudaEventCreateWithFlags(&eng->ev_kernel[b], cudaEventDisableTiming));
        if (!eng->ev_d2h[b]) GSS_CUDA_TRY(cudaEventCreateWithFlags(&eng->ev_d2h[b], cudaEventDisableTiming));
    }
    GSS_TRY(eng->state2.reserve(std::max<size_t>(bbytes, 8)));
    GSS_TRY(eng->state3.reserve(std::max<size_t>(bbytes, 8)));
    if (!direct) {
        GSS_TRY(eng->state_raw.reserve(std::max<size_t>(sbytes, 8)));
        GSS_TRY(eng->state_raw2.reserve(std::max<size_t>(sbytes, 8)));
        GSS_TRY(eng->state_raw3.reserve(std::max<size_t>(sbytes, 8)));
    }
    auto reserve_reports = [&]() -> int {
        GSS_TRY(eng->reports2.reserve((size_t) eng->cap_per_part * eng->n_parts * sizeof(gss_report)));
        GSS_TRY(eng->reports3.reserve((size_t) eng->cap_per_part * eng->n_parts * sizeof(gss_report)));
        return GSS_OK;
    };
    GSS_TRY(reserve_reports());
    GSS_TRY(eng->counts2.reserve(sizeof(uint32_t) * eng->n_parts));
    GSS_TRY(eng->counts3.reserve(sizeof(uint32_t) * eng->n_parts));
    auto reserve_packed = [&]() -> int {
        for (int b = 0; b < NB && packed; b++)
            GSS_TRY(eng->packed[b].reserve((size_t) eng->cap_per_part * eng->n_parts * rec_words * sizeof(uint32_t)));
        return GSS_OK;
    };
    GSS_TRY(reserve_packed());
    // packs pass b's reports (after its check, on the engine stream)
    auto pack = [&](int b, const DevBuf &rep, const DevBuf &cnt) -> int {
        if (!packed) return GSS_OK;
        return launch_pack_reports((const gss_report *) rep.ptr, (const uint32_t *) cnt.ptr, eng->n_parts,
                                   eng->cap_per_part, format == kRecordsCells ? (uint32_t) n_words : 0u,
                                   (uint32_t *) eng->packed[b].ptr, eng->stream, eng->sm_count);
    };
    GSS_TRY(eng->h_counts2.reserve(sizeof(uint32_t) * (eng->n_parts + 1)));
    GSS_TRY(eng->h_counts3.reserve(sizeof(uint32_t) * (eng->n_parts + 1)));
    DevBuf *state_buf[NB] = {&eng->state, &eng->state2, &eng->state3};
    DevBuf *raw_buf[NB] = {&eng->state_raw, &eng->state_raw2, &eng->state_raw3};
    DevBuf *rep_buf[NB] = {&eng->reports, &eng->reports2, &eng->reports3};
    DevBuf *cnt_buf[NB] = {&eng->counts, &eng->counts2, &eng->counts3};
    PinnedBuf *hcnt_buf[NB] = {&eng->h_counts, &eng->h_counts2, &eng->h_counts3};
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));  // pass 0's state is in buffer 0

    int launched = 0;
    // copies the reports of pass j back (the host waits for its kernel)
    auto finish = [&](int j) -> int {
        const int b = j % NB;
        GSS_CUDA_TRY(cudaEventSynchronize(eng->ev_kernel[b]));
        const uint32_t *hc = (const uint32_t *) hcnt_buf[b]->ptr;
        if (hc[eng->n_parts] != 0)
            return set_error(GSS_ERR_CUDA, "a bounded wait in the check kernel gave up (pass %d)", j);
        int64_t total = 0;
        bool overflow = false;
        for (uint32_t p = 0; p < eng->n_parts; p++) {
            total += hc[p];
            overflow |= hc[p] > eng->cap_per_part;
        }
        if (overflow) {
            // Rare after the first passes: grow both report sets and check this
            // pass again from its state buffer (not reused before pass j+2).
            // Pass j+1, already launched into the other set, runs again too:
            // growing the sets drops what it wrote.
            GSS_CUDA_TRY(cudaDeviceSynchronize());
            eng->requested_cap = std::max<int64_t>(eng->requested_cap, total * 2 + eng->n_parts * 1024);
            GSS_TRY(ensure_queues(eng));
            GSS_TRY(reserve_reports());
            GSS_TRY(reserve_packed());
            GSS_TRY(launch_pass_into(eng, state_buf[b]->ptr, *rep_buf[b], *cnt_buf[b], *hcnt_buf[b]));
            GSS_TRY(pack(b, *rep_buf[b], *cnt_buf[b]));
            eng->launches++;
            GSS_CUDA_TRY(cudaEventRecord(eng->ev_kernel[b], eng->stream));
            if (j + 1 < launched) {
                const int nb = (j + 1) % NB;
                GSS_TRY(launch_pass_into(eng, state_buf[nb]->ptr, *rep_buf[nb], *cnt_buf[nb], *hcnt_buf[nb]));
                GSS_TRY(pack(nb, *rep_buf[nb], *cnt_buf[nb]));
                eng->launches++;
                GSS_CUDA_TRY(cudaEventRecord(eng->ev_kernel[nb], eng->stream));
            }
            GSS_CUDA_TRY(cudaEventSynchronize(eng->ev_kernel[b]));
            total = 0;
            for (uint32_t p = 0; p < eng->n_parts; p++) total += hc[p];
        }
        n_reports[j] = total;
        if (total > caps[j])
            return set_error(GSS_ERR_OVERFLOW, "output %d holds %lld records, pass has %lld", j, (long long) caps[j],
                             (long long) total);
        if (packed) {
            if (total)
                GSS_CUDA_TRY(cudaMemcpyAsync(outs[j], eng->packed[b].ptr,
                                             (size_t) total * rec_words * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                             eng->d2h));
        } else {
            int64_t pos = 0;
            for (uint32_t p = 0; p < eng->n_parts; p++) {
                if (!hc[p]) continue;
                GSS_CUDA_TRY(cudaMemcpyAsync((gss_report *) outs[j] + pos,
                                             (gss_report *) rep_buf[b]->ptr + (size_t) p * eng->cap_per_part,
                                             (size_t) hc[p] * sizeof(gss_report), cudaMemcpyDeviceToHost, eng->d2h));
                pos += hc[p];
            }
        }
        GSS_CUDA_TRY(cudaEventRecord(eng->ev_d2h[b], eng->d2h));
        return GSS_OK;
    };

    auto pipeline = [&]() -> int {
    for (int i = 0; i < n_passes; i++) {
        const int b = i % NB;
        if (i > 0) {
            // state i -> buffer b, once pass i-3 (the last reader of b) is done
            if (i >= NB) GSS_CUDA_TRY(cudaStreamWaitEvent(eng->h2d, eng->ev_kernel[b], 0));
            void *dst = direct ? state_buf[b]->ptr : raw_buf[b]->ptr;
            if (!states[i]) return set_error(GSS_ERR_INVALID, "state %d is NULL", i);
            GSS_CUDA_TRY(cudaMemcpyAsync(dst, states[i], sbytes, cudaMemcpyHostToDevice, eng->h2d));
            GSS_CUDA_TRY(cudaEventRecord(eng->ev_h2d[b], eng->h2d));
            GSS_CUDA_TRY(cudaStreamWaitEvent(eng->stream, eng->ev_h2d[b], 0));
            if (!direct)
                GSS_TRY(launch_relayout((const uint2 *) raw_buf[b]->ptr, (uint2 *) state_buf[b]->ptr, (uint32_t) n_vars,
                                        (uint32_t) n_words, (uint32_t) eng->state_bw, (uint32_t) eng->n_blocks,
                                        eng->stream, eng->sm_count));
        }
        // report set b is free once pass i-3's reports are back
        if (i >= NB) GSS_CUDA_TRY(cudaStreamWaitEvent(eng->stream, eng->ev_d2h[b], 0));
        GSS_TRY(launch_pass_into(eng, state_buf[b]->ptr, *rep_buf[b], *cnt_buf[b], *hcnt_buf[b]));
        GSS_TRY(pack(b, *rep_buf[b], *cnt_buf[b]));
        eng->launches++;
        launched = i + 1;
        GSS_CUDA_TRY(cudaEventRecord(eng->ev_kernel[b], eng->stream));
        if (i > 0) GSS_TRY(finish(i - 1));
    }
    GSS_TRY(finish(n_passes - 1));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->d2h));
    return GSS_OK;
    };
    const int rc = pipeline();
    // on an early error, let everything already queued finish before the
    // buffers can be reused
    if (rc != GSS_OK) cudaDeviceSynchronize();
    eng->pass_pending = false;
    return rc;
}

}  // namespace

extern "C" {

int gss_check_passes_host(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars,
                          int n_words, const uint32_t *start, const int32_t *solver_of_word, gss_report *const *outs,
                          const int64_t *caps, int64_t *n_reports) {
    return passes_host(eng, n_passes, states, n_vars, n_words, start, solver_of_word, (void *const *) outs, caps,
                       n_reports, kRecordsFull);
}

int gss_check_passes_host_packed(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars,
                                 int n_words, const uint32_t *start, const int32_t *solver_of_word,
                                 gss_report_packed *const *outs, const int64_t *caps, int64_t *n_reports) {
    return passes_host(eng, n_passes, states, n_vars, n_words, start, solver_of_word, (void *const *) outs, caps,
                       n_reports, kRecordsPacked);
}

int gss_check_passes_host_cells(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars,
                                int n_words, const uint32_t *start, const int32_t *solver_of_word,
                                gss_report_cell *const *outs, const int64_t *caps, int64_t *n_reports) {
    return passes_host(eng, n_passes, states, n_vars, n_words, start, solver_of_word, (void *const *) outs, caps,
                       n_reports, kRecordsCells);
}

}  // extern "C"
