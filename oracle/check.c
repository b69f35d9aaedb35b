/*
 * CPU oracle for the clause-check pass of GpuShareSat's gpuShareLib.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark compare the CUDA
 * path against. The shipped library never links, loads or calls it.
 *
 * What it restates (paths relative to the GpuShareSat repository):
 *   - The per-slot report rule, gpuShareLib/GpuRunner.cu:34-57 (ReportComputer):
 *       allFalse'         = allFalse & isFalse
 *       justOneUndefined' = (allFalse & isUndef) | (justOneUndefined & isFalse)
 *       report            = allFalse | justOneUndefined
 *     started from the mask of completed slots (GpuRunner.cu:72,146;
 *     Assigs.cu:291 startVals = ~notCompletedMask).
 *   - The literal convention lit = 2*var + sign, sign 1 = negative literal,
 *     gpuShareLib/SolverTypes.h:56-60, and its value under a slot,
 *     GpuRunner.cu:74-81: a negative literal is false where the variable is
 *     true, a positive literal is false where the variable is defined and
 *     not true; an undefined variable gives an undefined literal.
 *   - Early exit once no slot can report any more, GpuRunner.cu:82-84.
 *
 * The reference's 32-bit aggregate prefilter (GpuRunner.cu:152-170) is a
 * sound over-approximation and never changes the reported set, so the oracle
 * checks every clause exactly, without it.
 *
 * Data layout (the same as the CUDA engine's host-facing layout):
 *   clauses   CSR: lits[offsets[c] .. offsets[c+1]) for clause c
 *   state     uint32 [n_vars][n_words][2] = {isDef, isTrue} per 32-slot word
 *   start     uint32 [n_words]: the slots of each word that are checked
 * A report is (clause index, word, 32-bit slot mask), emitted in increasing
 * (clause, word) order.
 *
 * Bit-parallel: two 32-slot words are evaluated together in one uint64, so
 * one pass over a clause checks 64 assignments. Threads split the clause
 * range; their outputs are concatenated in clause order.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef struct {
    uint32_t clause;
    uint32_t word;
    uint32_t mask;
    uint32_t pad;
} oracle_report;

/* One clause against one 64-slot lane pair (words w0 and w0+1; w0+1 may be
 * absent, in which case its start bits are zero). Returns the 64-bit report. */
static inline uint64_t check_pair(const int32_t *lits, int64_t len,
                                  const uint32_t *state, int n_words, int w0,
                                  uint64_t start) {
    uint64_t all_false = start;
    uint64_t one_undef = 0;
    int has_hi = (w0 + 1) < n_words;
    for (int64_t i = 0; i < len; i++) {
        uint32_t lit = (uint32_t) lits[i];
        uint32_t var = lit >> 1;
        const uint32_t *row = state + ((size_t) var * (size_t) n_words + (size_t) w0) * 2;
        uint64_t is_def = row[0];
        uint64_t is_true = row[1];
        if (has_hi) {
            is_def |= (uint64_t) row[2] << 32;
            is_true |= (uint64_t) row[3] << 32;
        }
        uint64_t is_false = (lit & 1) ? is_true : ~is_true;
        is_false &= is_def;
        uint64_t is_undef = ~is_def;
        one_undef = (all_false & is_undef) | (one_undef & is_false);
        all_false &= is_false;
        if ((all_false | one_undef) == 0) return 0;
    }
    return all_false | one_undef;
}

/* Checks clauses [c_begin, c_end). Writes at most cap reports; returns the
 * number of reports found (which can exceed cap). */
static int64_t check_range(const int32_t *lits, const int64_t *offsets,
                           int64_t c_begin, int64_t c_end,
                           const uint32_t *state, int n_words,
                           const uint32_t *start_mask,
                           oracle_report *out, int64_t cap) {
    int64_t n = 0;
    for (int64_t c = c_begin; c < c_end; c++) {
        const int32_t *cl = lits + offsets[c];
        int64_t len = offsets[c + 1] - offsets[c];
        for (int w0 = 0; w0 < n_words; w0 += 2) {
            uint64_t start = start_mask[w0];
            if (w0 + 1 < n_words) start |= (uint64_t) start_mask[w0 + 1] << 32;
            if (start == 0) continue;
            uint64_t rep = check_pair(cl, len, state, n_words, w0, start);
            if (rep == 0) continue;
            for (int half = 0; half < 2; half++) {
                uint32_t m = (uint32_t) (rep >> (32 * half));
                if (m == 0) continue;
                if (n < cap) {
                    out[n].clause = (uint32_t) c;
                    out[n].word = (uint32_t) (w0 + half);
                    out[n].mask = m;
                    out[n].pad = 0;
                }
                n++;
            }
        }
    }
    return n;
}

typedef struct {
    const int32_t *lits;
    const int64_t *offsets;
    int64_t c_begin, c_end;
    const uint32_t *state;
    int n_words;
    const uint32_t *start_mask;
    oracle_report *buf;
    int64_t cap;
    int64_t found;
} range_job;

static void *range_worker(void *arg) {
    range_job *j = (range_job *) arg;
    j->found = check_range(j->lits, j->offsets, j->c_begin, j->c_end, j->state,
                           j->n_words, j->start_mask, j->buf, j->cap);
    return NULL;
}

/* Checks every clause against every started slot of every word.
 * Returns the total number of reports (may exceed cap: then only the first
 * cap, in (clause, word) order, are written), or -1 on a bad argument or an
 * allocation failure. n_threads <= 1 runs on the calling thread. */
int64_t oracle_check(const int32_t *lits, const int64_t *offsets, int64_t n_clauses,
                     const uint32_t *state, int n_vars, int n_words,
                     const uint32_t *start_mask, int n_threads,
                     oracle_report *out, int64_t cap) {
    (void) n_vars;
    if (n_clauses < 0 || n_words < 0 || cap < 0) return -1;
    if (n_clauses == 0 || n_words == 0) return 0;
    if (n_threads <= 1 || n_clauses < 1024) {
        return check_range(lits, offsets, 0, n_clauses, state, n_words, start_mask, out, cap);
    }
    if (n_threads > 256) n_threads = 256;
    range_job jobs[256];
    pthread_t tids[256];
    /* Each thread gets its own report buffer sized for its share, grown on
     * demand by a second pass when it overflows. */
    int64_t per = (n_clauses + n_threads - 1) / n_threads;
    for (int t = 0; t < n_threads; t++) {
        int64_t b = (int64_t) t * per;
        int64_t e = b + per;
        if (b > n_clauses) b = n_clauses;
        if (e > n_clauses) e = n_clauses;
        jobs[t] = (range_job){lits, offsets, b, e, state, n_words, start_mask, NULL, 0, 0};
        int64_t guess = (e - b) / 64 + 1024;
        jobs[t].buf = (oracle_report *) malloc(sizeof(oracle_report) * (size_t) guess);
        if (!jobs[t].buf) {
            for (int u = 0; u < t; u++) free(jobs[u].buf);
            return -1;
        }
        jobs[t].cap = guess;
    }
    for (int t = 0; t < n_threads; t++) pthread_create(&tids[t], NULL, range_worker, &jobs[t]);
    for (int t = 0; t < n_threads; t++) pthread_join(tids[t], NULL);
    int64_t total = 0;
    int failed = 0;
    for (int t = 0; t < n_threads; t++) {
        if (jobs[t].found > jobs[t].cap) {
            free(jobs[t].buf);
            jobs[t].cap = jobs[t].found;
            jobs[t].buf = (oracle_report *) malloc(sizeof(oracle_report) * (size_t) jobs[t].cap);
            if (!jobs[t].buf) { failed = 1; continue; }
            range_worker(&jobs[t]);
        }
    }
    for (int t = 0; t < n_threads; t++) {
        if (!failed) {
            for (int64_t i = 0; i < jobs[t].found; i++) {
                if (total + i < cap) out[total + i] = jobs[t].buf[i];
            }
            total += jobs[t].found;
        }
        free(jobs[t].buf);
    }
    return failed ? -1 : total;
}

/* The rule for a single clause and a single 32-slot word, exposed so the
 * tests can pin it on hand-written cases. vals[i] is the value of literal i's
 * variable under each slot, given as isDef/isTrue words. */
uint32_t oracle_check_one(const int32_t *lits, int64_t len, const uint32_t *is_def,
                          const uint32_t *is_true, uint32_t start) {
    uint32_t all_false = start, one_undef = 0;
    for (int64_t i = 0; i < len; i++) {
        uint32_t f = ((lits[i] & 1) ? is_true[i] : ~is_true[i]) & is_def[i];
        uint32_t u = ~is_def[i];
        one_undef = (all_false & u) | (one_undef & f);
        all_false &= f;
    }
    return all_false | one_undef;
}

/* ---- order-independent digest of a report set ----
 *
 * For passes too large to compare record by record in a test (hundreds of
 * millions of records), the checker compares the number of (clause, word)
 * records and the wrapping sum over records of
 *     mix(mix((id << 32) | word) ^ mask)
 * where id is the clause's id (ids[c], or c when ids is NULL) and mix is the
 * SplitMix64 finaliser (Steele, Lea and Flood, "Fast splittable pseudorandom
 * number generators", OOPSLA 2014). The sum does not depend on record order,
 * so it can be computed the same way from the GPU's unordered output. */
static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    const int32_t *lits;
    const int64_t *offsets;
    const uint32_t *ids;
    int64_t c_begin, c_end;
    const uint32_t *state;
    int n_words;
    const uint32_t *start_mask;
    uint64_t count, digest;
} digest_job;

static void *digest_worker(void *arg) {
    digest_job *j = (digest_job *) arg;
    uint64_t count = 0, digest = 0;
    for (int64_t c = j->c_begin; c < j->c_end; c++) {
        const int32_t *cl = j->lits + j->offsets[c];
        int64_t len = j->offsets[c + 1] - j->offsets[c];
        uint64_t id = j->ids ? j->ids[c] : (uint64_t) c;
        for (int w0 = 0; w0 < j->n_words; w0 += 2) {
            uint64_t start = j->start_mask[w0];
            if (w0 + 1 < j->n_words) start |= (uint64_t) j->start_mask[w0 + 1] << 32;
            if (start == 0) continue;
            uint64_t rep = check_pair(cl, len, j->state, j->n_words, w0, start);
            for (int half = 0; half < 2 && rep; half++) {
                uint32_t m = (uint32_t) (rep >> (32 * half));
                if (m == 0) continue;
                count++;
                digest += mix64(mix64((id << 32) | (uint64_t) (w0 + half)) ^ (uint64_t) m);
            }
        }
    }
    j->count = count;
    j->digest = digest;
    return NULL;
}

/* Count and digest of the reports of every clause against every started
 * slot (see above). Returns 0, or -1 on a bad argument. */
int oracle_check_digest(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, const uint32_t *ids,
                        const uint32_t *state, int n_words, const uint32_t *start_mask, int n_threads,
                        uint64_t *count, uint64_t *digest) {
    if (n_clauses < 0 || n_words < 0 || !count || !digest) return -1;
    *count = 0;
    *digest = 0;
    if (n_clauses == 0 || n_words == 0) return 0;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    digest_job jobs[256];
    pthread_t tids[256];
    int64_t per = (n_clauses + n_threads - 1) / n_threads;
    for (int t = 0; t < n_threads; t++) {
        int64_t b = (int64_t) t * per, e = b + per;
        if (b > n_clauses) b = n_clauses;
        if (e > n_clauses) e = n_clauses;
        jobs[t] = (digest_job){lits, offsets, ids, b, e, state, n_words, start_mask, 0, 0};
    }
    for (int t = 1; t < n_threads; t++) pthread_create(&tids[t], NULL, digest_worker, &jobs[t]);
    digest_worker(&jobs[0]);
    for (int t = 1; t < n_threads; t++) pthread_join(tids[t], NULL);
    for (int t = 0; t < n_threads; t++) {
        *count += jobs[t].count;
        *digest += jobs[t].digest;
    }
    return 0;
}
