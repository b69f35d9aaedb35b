// Learned scan order: a 12-64-64-1 MLP scores every clause before a pass, and
// the pass scans clauses in decreasing score so that clauses likely to report
// are checked, and their reports delivered, first. Every clause is still
// checked each pass: the report set is the plain scan's.
//
// Per pass (score_pass):
//   1. the history step: birth_kernel (records of the ids first seen),
//      log_kernel (a hashed sample of (features, reported) rows of pass q-2
//      for training), fold_kernel (a sweep over the ids in id order: pass
//      q-2's report counts folded into the 8-pass histories of the clauses it
//      reported; the others are not written, their histories read as shifted
//      by the passes since their last report)
//   Every rescore_interval passes (or when the layout changed), the scan
//   permutation is rebuilt; the passes between reuse it:
//   2. score_kernel, a lane per clause position (a warp per 32): computes
//      the features; the warp runs the MLP on tensor cores (mma.sync
//      m16n8k16, BF16 operands, FP32 accumulation) over its 32 clauses as two
//      m16 tiles, and each lane writes its clause's score bucket
//   3. bucket_hist_kernel, bucket_scan_kernel, head_key_kernel, then a
//      stable one-digit radix sort of positions (bucket_hist, bucket_scan,
//      bucket_base, bucket_scatter) by key: the octave of predicted
//      probability for the clauses of the head (the best buckets up to
//      head_fraction of the clauses), one key for the tail. Inside a key the
//      plain database order holds (variable ranges, then length), so the
//      head keeps much of its state-row locality (its reports are delivered
//      at the end of the head launch, whatever its inner order), and the
//      tail keeps the plain order and its locality
// After the pass (order_after_pass): history_kernel adds each report's slot
// count to its clause's counter for the pass, and the scoring of the next
// pass is enqueued on a stream of its own, behind the head of this pass: it
// runs while the tail of this pass runs, so a pass usually starts with its
// order ready. The scoring of pass q therefore sees reports up to pass q-2
// (each clause keeps two counters, for even and odd passes). Calls that
// change the engine's buffers wait for it first (order_quiesce).
//
// Training (every retrain_interval passes, on a stream of its own, over a
// snapshot of the log; and gss_scorer_train_step): FP32 forward and backward
// kernels over a minibatch, per-32-row partial gradients reduced in a fixed
// order (no atomics), and Adam. The passes take the new weights once the
// training is done.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#include "common.h"
#include "engine.h"

namespace gss {

constexpr int kF = GSS_SCORER_FEATURES;
constexpr int kH = GSS_SCORER_HIDDEN;
constexpr int kP = GSS_SCORER_PARAMS;
// flat parameter layout: W1[kH][kF], b1[kH], W2[kH][kH], b2[kH], w3[kH], b3
constexpr int oW1 = 0, oB1 = kH * kF, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH, oB3 = oW3 + kH;
static_assert(oB3 + 1 == kP, "parameter layout");
static_assert(kF <= 16 && kH == 64, "the tensor-core MLP is written for K1 <= 16 and 64 hidden units");

// Fragments of the two matrix layers for mma.m16n8k16 (B operand): layer 1 as
// 8 n-tiles, layer 2 as 4 k-tiles x 8 n-tiles; per tile and lane two 32-bit
// registers of two BF16 each.
constexpr int kFrag1 = 8 * 32;
constexpr int kFrag2 = 32 * 32;

// Sort key: the score bucket, 16 per octave of the predicted report
// probability (0 = most likely); the last bucket holds deleted clauses.
constexpr int kBucketsPerOctave = 16;
constexpr int kBuckets = 256;
// radix sort tiles: kSortThreads threads x kSortRounds positions
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 16;
constexpr uint32_t kSortTile = kSortThreads * kSortRounds;
static_assert(kSortThreads == kBuckets, "one sort thread per bucket");

constexpr unsigned kFullMask = 0xFFFFFFFFu;

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ float unit_hash(uint64_t seed, uint64_t a, uint64_t b) {
    const uint64_t h = mix64(seed ^ mix64(a * 0x9E3779B97F4A7C15ull + b + 0x632BE59BD9B4E019ull));
    return (float) (h >> 40) * (1.0f / 16777216.0f);
}

// ---------------------------------------------------------------- features

// The 12 features of a clause. since_last < 0: never reported.
__host__ __device__ __forceinline__ void clause_features(uint32_t len, uint32_t lbd, int32_t age, uint64_t hist,
                                                         uint32_t total, int32_t since_last, float (&x)[kF]) {
    if (lbd == 0) lbd = len;  // unknown: the sharer's convention, LBD := length
    uint32_t b[8];
    uint32_t npass = 0;
    for (int k = 0; k < 8; k++) {
        b[k] = (uint32_t) (hist >> (8 * k)) & 0xFFu;
        npass += b[k] != 0;
    }
    const uint32_t s1 = b[0], s2 = s1 + b[1], s4 = s2 + b[2] + b[3], s8 = s4 + b[4] + b[5] + b[6] + b[7];
    const float fage = (float) (age > 0 ? age : 0);
    x[0] = (float) len / 64.0f;
    x[1] = (float) lbd / 64.0f;
    x[2] = (float) lbd / (float) (len ? len : 1);
    x[3] = log2f(1.0f + fage) / 16.0f;
    x[4] = (float) (s1 < 8 ? s1 : 8) / 8.0f;
    x[5] = (float) (s2 < 16 ? s2 : 16) / 16.0f;
    x[6] = (float) (s4 < 32 ? s4 : 32) / 32.0f;
    x[7] = (float) (s8 < 64 ? s8 : 64) / 64.0f;
    x[8] = (float) npass / 8.0f;
    const float rec = since_last < 0 ? 1.0f : log2f(1.0f + (float) since_last) / 16.0f;
    x[9] = rec < 1.0f ? rec : 1.0f;
    x[10] = log2f(1.0f + (float) total) / 16.0f;
    const float rate = (float) total / (fage > 1.0f ? fage : 1.0f);
    x[11] = rate < 1.0f ? rate : 1.0f;
}

// Per-id history (device), one 32-byte record per clause id. The history is
// kept lazily: a pass touches only the records of the clauses it reported
// (history_kernel lists them, fold_kernel folds them in), and `hist` holds the
// counts as of the pass of the last report; readers shift it to the pass they
// need (hist_at), the passes in between having had no report.
struct alignas(32) ClauseRecord {  // field order is read as two uint4 by score_kernel
    uint64_t hist;   // byte k = slot reports in pass (last - k), saturated at 255
    uint32_t total;  // slot reports over the clause's life
    int32_t last;    // pass of the last report, -1 never
    int32_t birth;   // the `now` of the first scoring that saw the clause
    uint32_t cur0;   // slot reports of the last even pass not yet folded in (history_kernel)
    uint16_t lbd;    // 0 = unknown (read as the length)
    uint16_t pad;
    uint32_t cur1;   // the same for odd passes
};
static_assert(sizeof(ClauseRecord) == 32, "one sector per clause");

// The history word with byte 0 = pass t, from a record whose byte 0 is pass
// `last` (no report after it): all zero for a clause that never reported.
__host__ __device__ __forceinline__ uint64_t hist_at(uint64_t hist, int32_t last, int32_t t) {
    if (last < 0) return 0;
    const int32_t d = t - last;
    return d >= 8 ? 0ull : d <= 0 ? hist : hist << (8 * d);
}

// The step before the scoring of pass q folds the counts of pass q-2 (slot
// q & 1) into the history: pass q-1 may still be running when pass q is
// scored. Features are then those of a prediction for the pass after
// `now` = q-1, with the history through pass q-2.
struct HistoryArgs {
    ClauseRecord *rec;
    uint32_t n_ids;
    uint32_t known_ids;  // ids below this were seen by an earlier scoring
    int32_t now;         // q - 1
    int32_t fold;        // the pass whose counts are folded, q - 2 (negative: none)
    uint32_t slot;       // its count slot, q & 1
};

// ------------------------------------------------------------ the scorer

struct Scorer {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    DevBuf w, m, v, grad;  // FP32 parameters, Adam moments, gradient
    DevBuf frag;           // BF16 mma fragments of W1 and W2
    bool frag_stale = true;
    int64_t adam_steps = 0;
    DevBuf act;            // training activations
    DevBuf io_x, io_y, io_out, loss;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&p);
}

__global__ void build_frags_kernel(const float *__restrict__ w, uint32_t *__restrict__ frag) {
    for (int idx = threadIdx.x; idx < kFrag1 + kFrag2; idx += blockDim.x) {
        const int lane = idx & 31, g = lane >> 2, t = lane & 3;
        if (idx < kFrag1) {
            const int n = (idx >> 5) * 8 + g;  // output unit
            auto B = [&](int k) { return k < kF ? w[oW1 + n * kF + k] : 0.0f; };
            frag[2 * idx] = pack_bf16(B(2 * t), B(2 * t + 1));
            frag[2 * idx + 1] = pack_bf16(B(2 * t + 8), B(2 * t + 9));
        } else {
            const int tile = (idx - kFrag1) >> 5, kt = tile >> 3, nt = tile & 7;
            const int n = nt * 8 + g;
            const float *row = w + oW2 + n * kH + kt * 16;
            frag[2 * idx] = pack_bf16(row[2 * t], row[2 * t + 1]);
            frag[2 * idx + 1] = pack_bf16(row[2 * t + 8], row[2 * t + 9]);
        }
    }
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct MlpShared {
    uint2 w1[8][32];   // layer-1 fragments [tile][lane]
    uint2 w2[32][32];  // layer-2 fragments [tile][lane]
    float b1[kH], b2[kH], w3[kH];
    float b3;
};

__device__ void load_mlp_shared(MlpShared &sm, const float *w, const uint32_t *frag) {
    const uint2 *f1 = reinterpret_cast<const uint2 *>(frag);
    for (int i = threadIdx.x; i < kFrag1; i += blockDim.x) sm.w1[i >> 5][i & 31] = f1[i];
    const uint2 *f2 = f1 + kFrag1;
    for (int i = threadIdx.x; i < kFrag2; i += blockDim.x) sm.w2[i >> 5][i & 31] = f2[i];
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
        sm.b1[i] = w[oB1 + i];
        sm.b2[i] = w[oB2 + i];
        sm.w3[i] = w[oW3 + i];
    }
    if (threadIdx.x == 0) sm.b3 = w[oB3];
}

// One warp, 16 rows: lane (g = lane/4, t = lane%4) brings the features of
// rows g and g+8 and gets back both logits (every lane of the group).
// v: columns 2t, 2t+1, 2t+8, 2t+9 of rows g (v[0..3]) and g+8 (v[4..7]).
__device__ __forceinline__ void mlp16v(const float (&v)[8], const MlpShared &sm, float &out0, float &out1) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    const uint32_t a0 = pack_bf16(v[0], v[1]), a1 = pack_bf16(v[4], v[5]);
    const uint32_t a2 = pack_bf16(v[2], v[3]), a3 = pack_bf16(v[6], v[7]);
    // layer 1 one k-tile of layer 2 at a time (n-tiles 2kt and 2kt+1): bias
    // + ReLU, re-packed as the A operand of layer 2 (the accumulator layout
    // of n-tiles 2kt and 2kt+1 is the A layout of k-tile kt)
    uint32_t h[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        float p0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, p1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const uint2 b0 = sm.w1[2 * kt][lane], b1 = sm.w1[2 * kt + 1][lane];
        mma_bf16(p0, a0, a1, a2, a3, b0.x, b0.y);
        mma_bf16(p1, a0, a1, a2, a3, b1.x, b1.y);
        const int c0 = 16 * kt + 2 * t, c1 = c0 + 8;
        h[kt][0] = pack_bf16(fmaxf(p0[0] + sm.b1[c0], 0.0f), fmaxf(p0[1] + sm.b1[c0 + 1], 0.0f));
        h[kt][1] = pack_bf16(fmaxf(p0[2] + sm.b1[c0], 0.0f), fmaxf(p0[3] + sm.b1[c0 + 1], 0.0f));
        h[kt][2] = pack_bf16(fmaxf(p1[0] + sm.b1[c1], 0.0f), fmaxf(p1[1] + sm.b1[c1 + 1], 0.0f));
        h[kt][3] = pack_bf16(fmaxf(p1[2] + sm.b1[c1], 0.0f), fmaxf(p1[3] + sm.b1[c1 + 1], 0.0f));
    }
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float d2[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            const uint2 b = sm.w2[kt * 8 + nt][lane];
            mma_bf16(d2, h[kt][0], h[kt][1], h[kt][2], h[kt][3], b.x, b.y);
        }
        const int c = nt * 8 + 2 * t;
        s0 += fmaxf(d2[0] + sm.b2[c], 0.0f) * sm.w3[c] + fmaxf(d2[1] + sm.b2[c + 1], 0.0f) * sm.w3[c + 1];
        s1 += fmaxf(d2[2] + sm.b2[c], 0.0f) * sm.w3[c] + fmaxf(d2[3] + sm.b2[c + 1], 0.0f) * sm.w3[c + 1];
    }
    s0 += __shfl_xor_sync(kFullMask, s0, 1);
    s0 += __shfl_xor_sync(kFullMask, s0, 2);
    s1 += __shfl_xor_sync(kFullMask, s1, 1);
    s1 += __shfl_xor_sync(kFullMask, s1, 2);
    out0 = s0 + sm.b3;
    out1 = s1 + sm.b3;
}

__device__ __forceinline__ void mlp16(const float (&x0)[kF], const float (&x1)[kF], const MlpShared &sm,
                                      float &out0, float &out1) {
    const int t = threadIdx.x & 3;
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = 0.0f;
#pragma unroll
    for (int c = 0; c < kF; c++) {
        if (c == 2 * t) v[0] = x0[c], v[4] = x1[c];
        if (c == 2 * t + 1) v[1] = x0[c], v[5] = x1[c];
        if (c == 2 * t + 8) v[2] = x0[c], v[6] = x1[c];
        if (c == 2 * t + 9) v[3] = x0[c], v[7] = x1[c];
    }
    mlp16v(v, sm, out0, out1);
}


constexpr int kMlpThreads = 256;

// Logits of rows of features given in memory (x[n][kF]).
__global__ void __launch_bounds__(kMlpThreads) infer_rows_kernel(const float *__restrict__ w,
                                                                  const uint32_t *__restrict__ frag,
                                                                  const float *__restrict__ x, uint32_t n,
                                                                  float *__restrict__ out) {
    __shared__ MlpShared sm;
    load_mlp_shared(sm, w, frag);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        float x0[kF], x1[kF];
#pragma unroll
        for (int c = 0; c < kF; c++) {
            x0[c] = r0 < n ? x[(size_t) r0 * kF + c] : 0.0f;
            x1[c] = r1 < n ? x[(size_t) r1 * kF + c] : 0.0f;
        }
        float o0, o1;
        mlp16(x0, x1, sm, o0, o1);
        if (t == 0) {
            if (r0 < n) out[r0] = o0;
            if (r1 < n) out[r1] = o1;
        }
    }
}

// ------------------------------------------------------------ training

// Activations of a minibatch of B rows, unit-major so that threads (rows)
// access them coalesced: h1, h2, d1, d2 [kH][B], dz[B], loss[B].
__global__ void train_fwd_bwd_kernel(const float *__restrict__ w, const float *__restrict__ x,
                                     const float *__restrict__ y, uint32_t start, uint32_t n_rows, uint32_t B,
                                     float *__restrict__ act) {
    __shared__ float sw[kP];
    for (int i = threadIdx.x; i < kP; i += blockDim.x) sw[i] = w[i];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    const uint32_t r = (uint32_t) (((uint64_t) start + i) % n_rows);
    float xr[kF];
    for (int k = 0; k < kF; k++) xr[k] = x[(size_t) r * kF + k];
    float *h1 = act + i;
    float *h2 = act + (size_t) kH * B + i;
    float *d1 = act + (size_t) 2 * kH * B + i;
    float *d2 = act + (size_t) 3 * kH * B + i;
    float *dz = act + (size_t) 4 * kH * B;
    float *loss = dz + B;
    for (int j = 0; j < kH; j++) {
        float z = sw[oB1 + j];
        for (int k = 0; k < kF; k++) z = fmaf(sw[oW1 + j * kF + k], xr[k], z);
        h1[(size_t) j * B] = fmaxf(z, 0.0f);
    }
    float z3 = sw[oB3];
    for (int j = 0; j < kH; j++) {
        float z = sw[oB2 + j];
        for (int k = 0; k < kH; k++) z = fmaf(sw[oW2 + j * kH + k], h1[(size_t) k * B], z);
        const float hj = fmaxf(z, 0.0f);
        h2[(size_t) j * B] = hj;
        z3 = fmaf(sw[oW3 + j], hj, z3);
    }
    const float yr = y[r];
    // logistic loss with logits: max(z,0) - z*y + log(1 + exp(-|z|))
    loss[i] = fmaxf(z3, 0.0f) - z3 * yr + log1pf(expf(-fabsf(z3)));
    const float p = 1.0f / (1.0f + expf(-z3));
    const float g = (p - yr) / (float) B;
    dz[i] = g;
    for (int j = 0; j < kH; j++) d2[(size_t) j * B] = h2[(size_t) j * B] > 0.0f ? g * sw[oW3 + j] : 0.0f;
    for (int k = 0; k < kH; k++) {
        float s = 0.0f;
        for (int j = 0; j < kH; j++) s = fmaf(sw[oW2 + j * kH + k], d2[(size_t) j * B], s);
        d1[(size_t) k * B] = h1[(size_t) k * B] > 0.0f ? s : 0.0f;
    }
}

// Rows per gradient chunk: each block sums its chunk into one partial
// gradient; grad_reduce_kernel adds the partials in chunk order.
constexpr int kGradRows = 32;

__global__ void __launch_bounds__(256) train_grad_kernel(const float *__restrict__ x, uint32_t start,
                                                         uint32_t n_rows, uint32_t B,
                                                         const float *__restrict__ act,
                                                         float *__restrict__ partial) {
    __shared__ float xs[kGradRows][kF];
    __shared__ float h1s[kGradRows][kH + 1], h2s[kGradRows][kH + 1], d1s[kGradRows][kH + 1],
        d2s[kGradRows][kH + 1];
    __shared__ float dzs[kGradRows];
    const uint32_t r0 = blockIdx.x * kGradRows;
    const uint32_t rows = min((uint32_t) kGradRows, B - r0);
    for (int e = threadIdx.x; e < kH * kGradRows; e += blockDim.x) {
        const int j = e / kGradRows, rr = e % kGradRows;
        const bool in = (uint32_t) rr < rows;
        const size_t g = (size_t) j * B + r0 + rr;
        h1s[rr][j] = in ? act[g] : 0.0f;
        h2s[rr][j] = in ? act[(size_t) kH * B + g] : 0.0f;
        d1s[rr][j] = in ? act[(size_t) 2 * kH * B + g] : 0.0f;
        d2s[rr][j] = in ? act[(size_t) 3 * kH * B + g] : 0.0f;
    }
    for (int e = threadIdx.x; e < kF * kGradRows; e += blockDim.x) {
        const int rr = e / kF, k = e % kF;
        const uint32_t r = (uint32_t) (((uint64_t) start + r0 + rr) % n_rows);
        xs[rr][k] = (uint32_t) rr < rows ? x[(size_t) r * kF + k] : 0.0f;
    }
    if (threadIdx.x < kGradRows)
        dzs[threadIdx.x] = threadIdx.x < rows ? act[(size_t) 4 * kH * B + r0 + threadIdx.x] : 0.0f;
    __syncthreads();
    for (int p = threadIdx.x; p < kP; p += blockDim.x) {
        float s = 0.0f;
        if (p < oB1) {
            const int j = p / kF, k = p % kF;
            for (int rr = 0; rr < kGradRows; rr++) s = fmaf(d1s[rr][j], xs[rr][k], s);
        } else if (p < oW2) {
            for (int rr = 0; rr < kGradRows; rr++) s += d1s[rr][p - oB1];
        } else if (p < oB2) {
            const int j = (p - oW2) / kH, k = (p - oW2) % kH;
            for (int rr = 0; rr < kGradRows; rr++) s = fmaf(d2s[rr][j], h1s[rr][k], s);
        } else if (p < oW3) {
            for (int rr = 0; rr < kGradRows; rr++) s += d2s[rr][p - oB2];
        } else if (p < oB3) {
            for (int rr = 0; rr < kGradRows; rr++) s = fmaf(dzs[rr], h2s[rr][p - oW3], s);
        } else {
            for (int rr = 0; rr < kGradRows; rr++) s += dzs[rr];
        }
        partial[(size_t) blockIdx.x * kP + p] = s;
    }
}

__global__ void grad_reduce_kernel(const float *__restrict__ partial, uint32_t n_chunks, float *__restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kP) return;
    float s = 0.0f;
    for (uint32_t c = 0; c < n_chunks; c++) s += partial[(size_t) c * kP + p];
    grad[p] = s;
}

__global__ void mean_kernel(const float *__restrict__ v, uint32_t n, float *__restrict__ out) {
    __shared__ float part[32];
    float s = 0.0f;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(kFullMask, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0f;
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(kFullMask, s, o);
        if (threadIdx.x == 0) *out = s / (float) (n ? n : 1);
    }
}

__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, float lr, float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kP) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gp = g[p];
    const float mp = b1 * m[p] + (1.0f - b1) * gp;
    const float vp = b2 * v[p] + (1.0f - b2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    w[p] -= lr * (mp / c1) / (sqrtf(vp / c2) + eps);
}

int scorer_init(Scorer *s, int device, uint64_t seed, cudaStream_t stream) {
    s->device = device;
    GSS_TRY(s->w.reserve(kP * sizeof(float)));
    GSS_TRY(s->m.reserve(kP * sizeof(float)));
    GSS_TRY(s->v.reserve(kP * sizeof(float)));
    GSS_TRY(s->grad.reserve(kP * sizeof(float)));
    GSS_TRY(s->frag.reserve((kFrag1 + kFrag2) * 2 * sizeof(uint32_t)));
    GSS_TRY(s->loss.reserve(sizeof(float)));
    // He-uniform weights, zero biases
    std::vector<float> w(kP, 0.0f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int n, int fan_in) {
        const float lim = sqrtf(6.0f / (float) fan_in);
        std::uniform_real_distribution<float> u(-lim, lim);
        for (int i = 0; i < n; i++) w[off + i] = u(rng);
    };
    fill(oW1, kH * kF, kF);
    fill(oW2, kH * kH, kH);
    fill(oW3, kH, kH);
    GSS_CUDA_TRY(cudaMemcpyAsync(s->w.ptr, w.data(), kP * sizeof(float), cudaMemcpyHostToDevice, stream));
    GSS_CUDA_TRY(cudaMemsetAsync(s->m.ptr, 0, kP * sizeof(float), stream));
    GSS_CUDA_TRY(cudaMemsetAsync(s->v.ptr, 0, kP * sizeof(float), stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(stream));
    s->adam_steps = 0;
    s->frag_stale = true;
    return GSS_OK;
}

int scorer_frags(Scorer *s, cudaStream_t stream) {
    if (!s->frag_stale) return GSS_OK;
    build_frags_kernel<<<1, 256, 0, stream>>>((const float *) s->w.ptr, (uint32_t *) s->frag.ptr);
    GSS_CUDA_TRY(cudaGetLastError());
    s->frag_stale = false;
    return GSS_OK;
}

// Gradient (and mean loss, left in s->loss) of B rows starting at `start`
// (wrapping) of x/y with n_rows rows, all on the device.
int scorer_grad_dev(Scorer *s, const float *x, const float *y, uint32_t n_rows, uint32_t start, uint32_t B,
                    cudaStream_t stream) {
    const uint32_t n_chunks = (B + kGradRows - 1) / kGradRows;
    const size_t act_floats = (size_t) 4 * B * kH + 2 * (size_t) B;
    GSS_TRY(s->act.reserve((act_floats + (size_t) n_chunks * kP) * sizeof(float)));
    float *act = (float *) s->act.ptr;
    float *partial = act + act_floats;
    train_fwd_bwd_kernel<<<(B + 63) / 64, 64, 0, stream>>>((const float *) s->w.ptr, x, y, start, n_rows, B, act);
    GSS_CUDA_TRY(cudaGetLastError());
    train_grad_kernel<<<n_chunks, 256, 0, stream>>>(x, start, n_rows, B, act, partial);
    GSS_CUDA_TRY(cudaGetLastError());
    grad_reduce_kernel<<<(kP + 127) / 128, 128, 0, stream>>>(partial, n_chunks, (float *) s->grad.ptr);
    GSS_CUDA_TRY(cudaGetLastError());
    mean_kernel<<<1, 1024, 0, stream>>>(act + (size_t) 4 * B * kH + B, B, (float *) s->loss.ptr);
    GSS_CUDA_TRY(cudaGetLastError());
    return GSS_OK;
}

int scorer_adam_dev(Scorer *s, float lr, cudaStream_t stream) {
    s->adam_steps++;
    const float c1 = 1.0f - powf(0.9f, (float) s->adam_steps), c2 = 1.0f - powf(0.999f, (float) s->adam_steps);
    adam_kernel<<<(kP + 127) / 128, 128, 0, stream>>>((float *) s->w.ptr, (const float *) s->grad.ptr,
                                                       (float *) s->m.ptr, (float *) s->v.ptr, lr, c1, c2);
    GSS_CUDA_TRY(cudaGetLastError());
    s->frag_stale = true;
    return GSS_OK;
}

// ------------------------------------------------------------ the order

struct OrderState {
    gss_order_params prm;
    Scorer scorer;   // the weights the passes score with
    Scorer trainer;  // the training copy (weights, Adam moments), trained on its own stream
    cudaStream_t train_stream = nullptr;
    cudaEvent_t ev_train_start = nullptr, ev_train_done = nullptr;
    bool training = false;
    DevBuf snap_x, snap_y;  // the log as the training in flight saw it
    bool active = true;
    int64_t pass = 0;        // ordered passes prepared so far
    int64_t known_ids = 0;
    uint64_t epoch = 0;
    int64_t cap_ids = 0;
    DevBuf rec;                                 // ClauseRecord per clause id
    DevBuf lbd_pairs;                           // staging of gss_db_set_lbd
    DevBuf bucket, offs, totals, key_of;        // per position; per (bucket, sort tile); per bucket (x2)
    DevBuf perm[2];                             // scan permutations: the current one and the next one
    // the scan permutation in force (rescored every rescore_interval passes):
    // its buffer, the positions it covers and the layout it was built for;
    // inflight_buf is the buffer of the pass in flight, which a rescoring
    // must leave alone
    bool perm_valid = false;
    int perm_buf = 0, inflight_buf = 0;
    uint32_t perm_n = 0;
    uint64_t perm_layout = 0;
    // the order of the next pass, computed on score_stream while the tail of
    // the current pass runs (pre_*: what it was computed for)
    cudaStream_t score_stream = nullptr;
    cudaEvent_t ev_score_done = nullptr;
    bool pre_ready = false, pre_in_flight = false;
    int64_t pre_pass = -1;
    int64_t folded_pass = -1;  // the last pass q whose scoring folded pass q-2's counts
    uint32_t pre_n = 0;
    int pre_buf = 0;
    uint64_t pre_layout = 0;
    DevBuf log_x, log_y, log_count;
    PinnedBuf h_head_counts, h_log_count;
    // score start/end, head end, tail end, head counts copied, head start
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint32_t scored_n = 0;  // positions covered by the permutation of the pass in flight
    bool have_times = false;
    uint32_t head = 0;
    bool pending = false;  // a pass with a head launch is in flight
    int64_t trainings = 0;
    double last_loss = 0.0;
    std::mt19937_64 rng;
};

namespace {

__device__ __forceinline__ uint32_t bucket_of(float logit) {
    // -log2(sigmoid(z)) = log2(1 + exp(-z)), 16 buckets per octave
    const float nl = logit > 0.0f ? log1pf(expf(-logit)) : -logit + log1pf(expf(logit));
    const float b = nl * (1.4426950408889634f * kBucketsPerOctave);
    return b < (float) (kBuckets - 2) ? (uint32_t) b : (uint32_t) (kBuckets - 2);
}

// Training log: a share `rate` of the clauses, as (features, reported) rows.
struct LogArgs {
    float *x, *y;
    unsigned long long *count;
    uint32_t cap;
    float rate;
    uint64_t seed;
};

// One warp per 32 positions, a lane per position: the features of each live
// clause from its history (through pass now - 1), then the lanes pass the
// features to the MLP's fragment layout (two m16 tiles) and each lane writes
// its clause's score bucket.
__global__ void __launch_bounds__(kMlpThreads, 3) score_kernel(HistoryArgs h, const float *__restrict__ w,
                                                               const uint32_t *__restrict__ frag,
                                                               const int64_t *__restrict__ offsets,
                                                               const uint32_t *__restrict__ orig,
                                                               const uint32_t *__restrict__ alive, uint32_t n,
                                                               uint8_t *__restrict__ bucket) {
    __shared__ MlpShared sm;
    __shared__ float xs[kMlpThreads / 32][32][kF + 1];  // each warp's rows of features
    load_mlp_shared(sm, w, frag);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float(*wx)[kF + 1] = xs[threadIdx.x >> 5];
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 32 < n; tile += warps) {
        const uint32_t r = tile * 32 + lane;
        float x[kF];
#pragma unroll
        for (int k = 0; k < kF; k++) x[k] = 0.0f;
        bool live = r < n && (alive == nullptr || ((alive[r >> 5] >> (r & 31)) & 1u));
        const uint32_t id = r < n ? orig[r] : 0u;
        live = live && id < h.n_ids;
        if (live) {
            const uint32_t len = (uint32_t) (offsets[r + 1] - offsets[r]);
            // the record as two 16-byte words: {hist lo, hist hi, total, last}, {birth, cur0, lbd|pad, cur1}
            const ClauseRecord *rec = h.rec + id;
            const uint4 ra = reinterpret_cast<const uint4 *>(rec)[0], rb = reinterpret_cast<const uint4 *>(rec)[1];
            const int32_t last = (int32_t) ra.w;
            const uint64_t hist = hist_at(((uint64_t) ra.y << 32) | ra.x, last, h.now - 1);
            clause_features(len, rb.z & 0xFFFFu, h.now - (int32_t) rb.x, hist, ra.z, last < 0 ? -1 : h.now - last, x);
        }
        // two m16 tiles: rows 0-15 and 16-31 of the warp's positions, their
        // features passed to the fragment layout through shared memory
#pragma unroll
        for (int k = 0; k < kF; k++) wx[lane][k] = x[k];
        __syncwarp();
        float logit = 0.0f;
#pragma unroll 1
        for (int sub = 0; sub < 2; sub++) {
            const float *f0 = wx[sub * 16 + g], *f1 = wx[sub * 16 + g + 8];
            const int c = 2 * t;
            float v[8];
            v[0] = f0[c];
            v[1] = f0[c + 1];
            v[2] = c + 8 < kF ? f0[c + 8] : 0.0f;
            v[3] = c + 9 < kF ? f0[c + 9] : 0.0f;
            v[4] = f1[c];
            v[5] = f1[c + 1];
            v[6] = c + 8 < kF ? f1[c + 8] : 0.0f;
            v[7] = c + 9 < kF ? f1[c + 9] : 0.0f;
            float o0, o1;
            mlp16v(v, sm, o0, o1);
            // back to the lane that owns the row: row i of the tile is in lanes 4(i%8)..
            const int i = lane & 15;
            const float a = __shfl_sync(kFullMask, o0, 4 * (i & 7));
            const float b = __shfl_sync(kFullMask, o1, 4 * (i & 7));
            if ((lane >> 4) == sub) logit = (i < 8) ? a : b;
        }
        if (r < n) bucket[r] = (uint8_t) (live ? bucket_of(logit) : (uint32_t) (kBuckets - 1));
        __syncwarp();  // wx is rewritten by the next tile
    }
}

// Records of the ids first seen by the scoring step at `now` (ids in
// [from, to)): born at `now`, no report yet. Their pass counters are kept
// (a clause appended while a pass ran may already hold counts of it).
__global__ void birth_kernel(ClauseRecord *__restrict__ rec, uint32_t from, uint32_t to, int32_t now) {
    for (uint32_t id = from + blockIdx.x * blockDim.x + threadIdx.x; id < to; id += gridDim.x * blockDim.x) {
        ClauseRecord &r = rec[id];
        r.hist = 0;
        r.total = 0;
        r.last = -1;
        r.birth = now;
    }
}

// Training log of pass `fold` (before its counts are folded in): a share
// `rate` of the live clauses known before this step (a hash of (seed, fold,
// id) picks them), as (features a prediction for pass `fold` would have used,
// whether the clause reported in it) rows.
__global__ void log_kernel(HistoryArgs h, LogArgs lg, const int64_t *__restrict__ offsets,
                           const uint32_t *__restrict__ orig, const uint32_t *__restrict__ alive, uint32_t n) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        if (alive != nullptr && !((alive[r >> 5] >> (r & 31)) & 1u)) continue;
        const uint32_t id = orig[r];
        if (id >= h.known_ids || id >= h.n_ids || !(unit_hash(lg.seed, (uint64_t) h.fold, id) < lg.rate)) continue;
        const ClauseRecord &rec = h.rec[id];
        if (!(rec.birth < h.fold)) continue;
        const uint32_t c = h.slot ? rec.cur1 : rec.cur0;
        float xl[kF];
        clause_features((uint32_t) (offsets[r + 1] - offsets[r]), rec.lbd, h.fold - rec.birth,
                        hist_at(rec.hist, rec.last, h.fold - 1), rec.total, rec.last < 0 ? -1 : h.fold - rec.last, xl);
        const unsigned long long slot = atomicAdd(lg.count, 1ull) % lg.cap;
#pragma unroll
        for (int k = 0; k < kF; k++) lg.x[slot * kF + k] = xl[k];
        lg.y[slot] = c ? 1.0f : 0.0f;
    }
}

// Folds the counts of pass `fold` (slot h.slot) into the histories of the
// clauses that pass reported and clears the counters for the pass two later.
// A thread per id, in id order: the counters are read as one coalesced sweep
// over the records, and only the reported clauses' records are written.
__global__ void fold_kernel(HistoryArgs h, uint32_t n) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
        ClauseRecord &r = h.rec[id];
        const uint32_t c = h.slot ? r.cur1 : r.cur0;
        if (c == 0) continue;
        if (h.slot)
            r.cur1 = 0;
        else
            r.cur0 = 0;
        r.hist = hist_at(r.hist, r.last, h.fold) | (uint64_t) (c < 255u ? c : 255u);
        r.total += c;
        r.last = h.fold;
    }
}

// Exclusive scan of a[0..n) in place by one block; returns the total.
__device__ uint32_t block_scan_inplace(uint32_t *__restrict__ a, uint32_t n) {
    __shared__ uint32_t warp_sums[32];
    uint32_t carry = 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < n ? a[i] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = lane < (int) (blockDim.x >> 5) ? warp_sums[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFullMask, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        const uint32_t excl = (wid ? warp_sums[wid - 1] : 0u) + x - v;
        if (i < n) a[i] = carry + excl;
        carry += warp_sums[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    return carry;
}

// The sort key of each score bucket for the final order: the bucket's octave
// of predicted probability while the clauses of better buckets number fewer
// than `cut` (the head, by octave, in database order inside an octave),
// kBuckets - 2 for the rest (the tail, which then keeps the plain position
// order and its memory locality), kBuckets - 1 for deleted clauses. totals
// holds the clause count of each bucket. One block of kBuckets threads.
__global__ void head_key_kernel(const uint32_t *__restrict__ totals, uint32_t cut, uint8_t *__restrict__ key_of) {
    __shared__ uint32_t before[kBuckets];
    const int b = threadIdx.x;
    before[b] = totals[b];
    __syncthreads();
    if (b == 0) {
        uint32_t acc = 0;
        for (int k = 0; k < kBuckets; k++) {
            const uint32_t c = before[k];
            before[k] = acc;
            acc += c;
        }
    }
    __syncthreads();
    // head buckets by octave of the predicted probability: within an octave
    // the head keeps the database order (its state-row locality); the head's
    // reports are delivered when the whole head launch ends, so the order
    // inside it does not delay them
    key_of[b] = (uint8_t) (b == kBuckets - 1 ? kBuckets - 1 : before[b] < cut ? b / kBucketsPerOctave : kBuckets - 2);
}

// Block b: exclusive scan of bucket b's per-tile counts; totals[b] = its sum.
__global__ void bucket_scan_kernel(uint32_t *__restrict__ offs, uint32_t n_tiles, uint32_t *__restrict__ totals) {
    const uint32_t t = block_scan_inplace(offs + (size_t) blockIdx.x * n_tiles, n_tiles);
    if (threadIdx.x == 0) totals[blockIdx.x] = t;
}

// Exclusive scan of the bucket totals (one block): the first scan position of
// each bucket.
__global__ void bucket_base_kernel(uint32_t *__restrict__ totals, uint32_t n) { block_scan_inplace(totals, n); }

// Per sort tile: how many positions fall in each bucket, stored bucket-major
// (offs[b * n_tiles + tile]) for the scan.
__global__ void __launch_bounds__(kSortThreads) bucket_hist_kernel(const uint8_t *__restrict__ bucket,
                                                                   const uint8_t *__restrict__ key_of, uint32_t n,
                                                                   uint32_t n_tiles, uint32_t *__restrict__ offs) {
    __shared__ uint32_t hist[kBuckets];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; r++) {
        const uint32_t pos = base + r * kSortThreads + threadIdx.x;
        if (pos < n) atomicAdd(&hist[key_of ? key_of[bucket[pos]] : bucket[pos]], 1u);
    }
    __syncthreads();
    offs[(size_t) threadIdx.x * n_tiles + blockIdx.x] = hist[threadIdx.x];
}

// Stable scatter: positions of a bucket keep their order. Each round takes
// kSortThreads consecutive positions; a position's rank is its rank among the
// equal buckets of its warp (match) plus the counts of the earlier warps.
__global__ void __launch_bounds__(kSortThreads) bucket_scatter_kernel(const uint8_t *__restrict__ bucket,
                                                                      const uint8_t *__restrict__ key_of, uint32_t n,
                                                                      uint32_t n_tiles,
                                                                      const uint32_t *__restrict__ offs,
                                                                      const uint32_t *__restrict__ base_of,
                                                                      uint32_t *__restrict__ perm) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ uint32_t run[kBuckets];
    __shared__ uint16_t wcnt[kWarps][kBuckets];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    run[threadIdx.x] = base_of[threadIdx.x] + offs[(size_t) threadIdx.x * n_tiles + blockIdx.x];
    const uint32_t base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; r++) {
#pragma unroll
        for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t pos = base + r * kSortThreads + threadIdx.x;
        const bool valid = pos < n;
        const uint32_t b = valid ? (key_of ? key_of[bucket[pos]] : bucket[pos]) : (uint32_t) kBuckets;  // kBuckets: none
        const unsigned peers = __match_any_sync(kFullMask, b);
        const unsigned lt = (1u << lane) - 1u;
        const uint32_t rank = (uint32_t) __popc(peers & lt);
        if (valid && rank == 0) wcnt[wid][b] = (uint16_t) __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t dst = run[b] + rank;
            for (int w = 0; w < wid; w++) dst += wcnt[w][b];
            perm[dst] = pos;
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) add += wcnt[w][threadIdx.x];
        run[threadIdx.x] += add;
        __syncthreads();
    }
}

// Per report record of the pass: its slot count goes to its clause's counter
// for the pass. The partitions' records are spread over all the blocks (a
// block takes a stripe of one partition).
__global__ void history_kernel(const gss_report *__restrict__ reports, const uint32_t *__restrict__ counts,
                               uint32_t n_parts, uint32_t cap_per_part, ClauseRecord *__restrict__ rec,
                               uint32_t n_ids, uint32_t slot) {
    const uint32_t stripes = max(gridDim.x / n_parts, 1u);
    const uint32_t q = blockIdx.x % n_parts, stripe = blockIdx.x / n_parts;
    if (stripe >= stripes) return;
    const uint32_t m = min(counts[q], cap_per_part);
    const gss_report *r = reports + (size_t) q * cap_per_part;
    for (uint32_t i = stripe * blockDim.x + threadIdx.x; i < m; i += stripes * blockDim.x) {
        const uint32_t id = r[i].clause;
        if (id < n_ids) atomicAdd(slot ? &rec[id].cur1 : &rec[id].cur0, (uint32_t) __popc(r[i].mask));
    }
}

__global__ void set_lbd_kernel(const uint32_t *__restrict__ pairs, uint32_t n, ClauseRecord *__restrict__ rec) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        rec[pairs[2 * i]].lbd = (uint16_t) pairs[2 * i + 1];
}

unsigned grid_for_n(uint64_t n, int sm_count, int threads) {
    uint64_t b = (n + threads - 1) / threads;
    const uint64_t cap = (uint64_t) std::max(sm_count, 1) * 8;
    if (b > cap) b = cap;
    return (unsigned) std::max<uint64_t>(b, 1);
}

template <typename T>
int grow_ids(DevBuf &b, int64_t old_n, int64_t new_n, cudaStream_t stream, bool zero_tail) {
    GSS_TRY(b.grow_keep((size_t) new_n * sizeof(T), stream, (size_t) old_n * sizeof(T)));
    if (zero_tail && new_n > old_n)
        GSS_CUDA_TRY(cudaMemsetAsync((T *) b.ptr + old_n, 0, (size_t) (new_n - old_n) * sizeof(T), stream));
    return GSS_OK;
}

int ensure_ids(gss_engine *eng, int64_t n_ids) {
    OrderState &o = *eng->order;
    if (n_ids <= o.cap_ids) return GSS_OK;
    int64_t cap = std::max<int64_t>(o.cap_ids * 2, 1024);
    while (cap < n_ids) cap *= 2;
    GSS_TRY(grow_ids<ClauseRecord>(o.rec, o.cap_ids, cap, eng->stream, true));
    o.cap_ids = cap;
    return GSS_OK;
}

HistoryArgs history_args(gss_engine *eng, int32_t now) {
    OrderState &o = *eng->order;
    HistoryArgs h;
    h.rec = (ClauseRecord *) o.rec.ptr;
    h.n_ids = eng->next_id;
    h.known_ids = (uint32_t) o.known_ids;
    h.now = now;
    return h;
}

// Most minibatch steps one training issues (the launches are asynchronous,
// but issuing them takes host time in the pass that starts the training).
constexpr uint64_t kMaxTrainSteps = 512;

// Starts a training on the training stream over a snapshot of the log; the
// passes keep scoring with the current weights until it is done.
int train_start(gss_engine *eng) {
    OrderState &o = *eng->order;
    if (o.training) return GSS_OK;
    GSS_CUDA_TRY(cudaMemcpyAsync(o.h_log_count.ptr, o.log_count.ptr, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, eng->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    const uint64_t logged = std::min<uint64_t>(*(unsigned long long *) o.h_log_count.ptr, (uint64_t) o.prm.log_capacity);
    if (logged < 2) return GSS_OK;
    const uint32_t B = (uint32_t) std::min<uint64_t>((uint64_t) std::max(o.prm.batch, 1), logged);
    const uint64_t steps = std::min<uint64_t>(kMaxTrainSteps,
                                              (uint64_t) std::max(o.prm.train_epochs, 1) * ((logged + B - 1) / B));
    GSS_TRY(o.snap_x.reserve((size_t) logged * kF * sizeof(float)));
    GSS_TRY(o.snap_y.reserve((size_t) logged * sizeof(float)));
    GSS_CUDA_TRY(cudaEventRecord(o.ev_train_start, eng->stream));
    GSS_CUDA_TRY(cudaStreamWaitEvent(o.train_stream, o.ev_train_start, 0));
    GSS_CUDA_TRY(cudaMemcpyAsync(o.snap_x.ptr, o.log_x.ptr, (size_t) logged * kF * sizeof(float),
                                 cudaMemcpyDeviceToDevice, o.train_stream));
    GSS_CUDA_TRY(cudaMemcpyAsync(o.snap_y.ptr, o.log_y.ptr, (size_t) logged * sizeof(float), cudaMemcpyDeviceToDevice,
                                 o.train_stream));
    for (uint64_t st = 0; st < steps; st++) {
        const uint32_t start = (uint32_t) (o.rng() % logged);
        GSS_TRY(scorer_grad_dev(&o.trainer, (const float *) o.snap_x.ptr, (const float *) o.snap_y.ptr,
                                (uint32_t) logged, start, B, o.train_stream));
        GSS_TRY(scorer_adam_dev(&o.trainer, o.prm.learning_rate, o.train_stream));
    }
    GSS_CUDA_TRY(cudaEventRecord(o.ev_train_done, o.train_stream));
    o.training = true;
    return GSS_OK;
}

// Takes the trained weights once the training is done (wait: block for it).
int train_finish(gss_engine *eng, bool wait) {
    OrderState &o = *eng->order;
    if (!o.training) return GSS_OK;
    if (wait) {
        GSS_CUDA_TRY(cudaEventSynchronize(o.ev_train_done));
    } else {
        const cudaError_t q = cudaEventQuery(o.ev_train_done);
        if (q == cudaErrorNotReady) return GSS_OK;
        GSS_CUDA_TRY(q);
    }
    GSS_CUDA_TRY(cudaMemcpyAsync(o.scorer.w.ptr, o.trainer.w.ptr, kP * sizeof(float), cudaMemcpyDeviceToDevice,
                                 eng->stream));
    float l = 0.0f;
    GSS_CUDA_TRY(cudaMemcpy(&l, o.trainer.loss.ptr, sizeof l, cudaMemcpyDeviceToHost));
    o.scorer.frag_stale = true;
    o.training = false;
    o.trainings++;
    o.last_loss = l;
    return GSS_OK;
}

}  // namespace

bool order_active(const gss_engine *eng) { return eng->order && eng->order->active; }

void order_destroy(gss_engine *eng) {
    if (!eng->order) return;
    OrderState *o = eng->order;
    if (o->train_stream) {
        cudaStreamSynchronize(o->train_stream);
        cudaStreamDestroy(o->train_stream);
    }
    if (o->score_stream) {
        cudaStreamSynchronize(o->score_stream);
        cudaStreamDestroy(o->score_stream);
    }
    if (o->ev_score_done) cudaEventDestroy(o->ev_score_done);
    for (cudaEvent_t &e : o->ev)
        if (e) cudaEventDestroy(e);
    if (o->ev_train_start) cudaEventDestroy(o->ev_train_start);
    if (o->ev_train_done) cudaEventDestroy(o->ev_train_done);
    delete o;
    eng->order = nullptr;
}

void order_quiesce(gss_engine *eng) {
    if (!eng->order || !eng->order->pre_in_flight) return;
    cudaEventSynchronize(eng->order->ev_score_done);
    eng->order->pre_in_flight = false;
}

namespace {

// Scan positions in the head of a pass over n clauses.
uint32_t head_cut(const OrderState &o, uint32_t n) {
    double hf = o.prm.head_fraction;
    if (!(hf > 0.0)) hf = 0.0;
    if (hf > 1.0) hf = 1.0;
    return (uint32_t) std::min<double>((double) n, ceil(hf * (double) n));
}

// Enqueues on `st` the scoring and ordering of pass q over the database as it
// is now, into perm[q & 1]; returns the positions covered.
int score_pass(gss_engine *eng, cudaStream_t st, int64_t q, uint32_t *covered, int *buf) {
    OrderState &o = *eng->order;
    const uint32_t n = (uint32_t) eng->n_clauses;
    const int64_t n_ids = eng->next_id;
    GSS_TRY(ensure_ids(eng, std::max<int64_t>(n_ids, 1)));
    // Between rescorings the last permutation serves (positions appended
    // since it was built are scanned in place after it); a new layout, or
    // every rescore_interval-th pass, scores and sorts again.
    const int R = o.prm.rescore_interval;
    const bool rescore = R <= 1 || q % R == 0 || !o.perm_valid || o.perm_layout != eng->layout_epoch || o.perm_n > n;
    if (rescore) GSS_TRY(scorer_frags(&o.scorer, st));
    GSS_CUDA_TRY(cudaEventRecord(o.ev[0], st));
    HistoryArgs h = history_args(eng, (int32_t) (q - 1));
    // a pass's counts are folded once, by the first scoring of pass q
    h.fold = o.folded_pass < q ? (int32_t) (q - 2) : -1;
    h.slot = (uint32_t) (q & 1);
    o.folded_pass = std::max(o.folded_pass, q);
    LogArgs lg;
    lg.x = (float *) o.log_x.ptr;
    lg.y = (float *) o.log_y.ptr;
    lg.count = (unsigned long long *) o.log_count.ptr;
    lg.cap = (uint32_t) o.prm.log_capacity;
    lg.rate = (float) std::min(1.0, o.prm.log_rate > 0 ? o.prm.log_rate
                                                        : 2000.0 / (double) std::max<int64_t>(n_ids, 1));
    lg.seed = o.prm.seed;
    // The history step of every pass: births of the ids first seen, the
    // training rows of pass q-2, and the fold of its counts (only the clauses
    // it reported are touched).
    if (n_ids > o.known_ids) {
        const uint32_t from = (uint32_t) o.known_ids, to = (uint32_t) n_ids;
        birth_kernel<<<grid_for_n(to - from, eng->sm_count, 256), 256, 0, st>>>((ClauseRecord *) o.rec.ptr, from, to,
                                                                               h.now);
        GSS_CUDA_TRY(cudaGetLastError());
    }
    const uint32_t *alive = eng->n_dead > 0 ? (const uint32_t *) eng->alive.ptr : nullptr;
    if (h.fold >= 0) {
        if (lg.cap && n) {
            log_kernel<<<grid_for_n(n, eng->sm_count, 256), 256, 0, st>>>(h, lg, (const int64_t *) eng->offsets.ptr,
                                                                         (const uint32_t *) eng->orig.ptr, alive, n);
            GSS_CUDA_TRY(cudaGetLastError());
        }
        // the ids known before this step (a newer id cannot have reported in pass q-2)
        const uint32_t n_fold = (uint32_t) std::min<int64_t>(o.known_ids, o.cap_ids);
        if (n_fold) {
            fold_kernel<<<grid_for_n(n_fold, eng->sm_count, 256), 256, 0, st>>>(h, n_fold);
            GSS_CUDA_TRY(cudaGetLastError());
        }
    }
    o.known_ids = n_ids;
    h.known_ids = (uint32_t) n_ids;
    if (!rescore) {
        // the permutation in force serves this pass
        GSS_CUDA_TRY(cudaEventRecord(o.ev[1], st));
        *covered = o.perm_n;
        *buf = o.perm_buf;
        return GSS_OK;
    }
    // the new permutation goes to the buffer the pass in flight is not reading
    const int b = 1 - o.inflight_buf;
    DevBuf &perm = o.perm[b];
    const uint32_t n_tiles = (uint32_t) (((size_t) n + kSortTile - 1) / kSortTile);
    GSS_TRY(perm.reserve(std::max<size_t>(n, 1) * sizeof(uint32_t)));
    GSS_TRY(o.bucket.reserve(std::max<size_t>(n, 1)));
    GSS_TRY(o.offs.reserve(std::max<size_t>((size_t) kBuckets * n_tiles, 1) * sizeof(uint32_t)));
    GSS_TRY(o.totals.reserve(kBuckets * sizeof(uint32_t)));
    GSS_TRY(o.key_of.reserve(kBuckets));
    if (n) {
        // features, MLP, score bucket
        score_kernel<<<grid_for_n((uint64_t) (n + 31) / 32 * 32, eng->sm_count, kMlpThreads), kMlpThreads, 0, st>>>(
            h, (const float *) o.scorer.w.ptr, (const uint32_t *) o.scorer.frag.ptr,
            (const int64_t *) eng->offsets.ptr, (const uint32_t *) eng->orig.ptr, alive, n, (uint8_t *) o.bucket.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
        // the clauses per score bucket, then the sort key of each bucket:
        // score order in the head, plain order in the tail
        bucket_hist_kernel<<<n_tiles, kSortThreads, 0, st>>>((const uint8_t *) o.bucket.ptr, nullptr, n, n_tiles,
                                                              (uint32_t *) o.offs.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
        bucket_scan_kernel<<<kBuckets, 1024, 0, st>>>((uint32_t *) o.offs.ptr, n_tiles, (uint32_t *) o.totals.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
        head_key_kernel<<<1, kBuckets, 0, st>>>((const uint32_t *) o.totals.ptr, head_cut(o, n),
                                                (uint8_t *) o.key_of.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
        // stable radix sort of positions by key
        bucket_hist_kernel<<<n_tiles, kSortThreads, 0, st>>>((const uint8_t *) o.bucket.ptr,
                                                              (const uint8_t *) o.key_of.ptr, n, n_tiles,
                                                              (uint32_t *) o.offs.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
        bucket_scan_kernel<<<kBuckets, 1024, 0, st>>>((uint32_t *) o.offs.ptr, n_tiles, (uint32_t *) o.totals.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
        bucket_base_kernel<<<1, kBuckets, 0, st>>>((uint32_t *) o.totals.ptr, kBuckets);
        GSS_CUDA_TRY(cudaGetLastError());
        bucket_scatter_kernel<<<n_tiles, kSortThreads, 0, st>>>((const uint8_t *) o.bucket.ptr,
                                                                 (const uint8_t *) o.key_of.ptr, n, n_tiles,
                                                                 (const uint32_t *) o.offs.ptr,
                                                                 (const uint32_t *) o.totals.ptr,
                                                                 (uint32_t *) perm.ptr);
        GSS_CUDA_TRY(cudaGetLastError());
    }
    GSS_CUDA_TRY(cudaEventRecord(o.ev[1], st));
    o.perm_valid = true;
    o.perm_buf = b;
    o.perm_n = n;
    o.perm_layout = eng->layout_epoch;
    *covered = n;
    *buf = b;
    return GSS_OK;
}

}  // namespace

int order_prepare(gss_engine *eng, const uint32_t **perm, uint32_t *head, uint32_t *covered) {
    OrderState &o = *eng->order;
    cudaStream_t st = eng->stream;
    order_quiesce(eng);
    if (o.epoch != eng->db_epoch) {  // a new database: forget the history
        o.epoch = eng->db_epoch;
        o.known_ids = 0;
        o.pre_ready = false;
        o.folded_pass = o.pass - 1;  // nothing of the old database to fold
        if (o.cap_ids) GSS_CUDA_TRY(cudaMemsetAsync(o.rec.ptr, 0, (size_t) o.cap_ids * sizeof(ClauseRecord), st));
    }
    GSS_TRY(ensure_ids(eng, std::max<int64_t>(eng->next_id, 1)));
    const int64_t q = o.pass;
    // new weights from a finished training; a training every retrain_interval passes
    GSS_TRY(train_finish(eng, false));
    if (o.prm.retrain_interval > 0 && q > 0 && q % o.prm.retrain_interval == 0) GSS_TRY(train_start(eng));
    uint32_t n_scored = 0;
    int buf = 0;
    if (o.pre_ready && o.pre_pass == q && o.pre_layout == eng->layout_epoch) {
        n_scored = o.pre_n;  // computed while the previous pass ran
        buf = o.pre_buf;
    } else {
        GSS_TRY(score_pass(eng, st, q, &n_scored, &buf));
    }
    o.pre_ready = false;
    o.pass = q + 1;
    o.head = head_cut(o, n_scored);
    o.scored_n = n_scored;
    o.inflight_buf = buf;
    *perm = (const uint32_t *) o.perm[buf].ptr;
    *head = o.head;
    *covered = n_scored;
    GSS_CUDA_TRY(cudaEventRecord(o.ev[5], st));
    return GSS_OK;
}

int order_after_head(gss_engine *eng, const DevBuf &counts) {
    OrderState &o = *eng->order;
    GSS_CUDA_TRY(cudaEventRecord(o.ev[2], eng->stream));
    GSS_TRY(o.h_head_counts.reserve(sizeof(uint32_t) * (eng->n_parts + 1)));
    GSS_CUDA_TRY(cudaMemcpyAsync(o.h_head_counts.ptr, counts.ptr, sizeof(uint32_t) * eng->n_parts,
                                 cudaMemcpyDeviceToHost, eng->stream));
    GSS_CUDA_TRY(cudaEventRecord(o.ev[4], eng->stream));
    o.pending = true;
    return GSS_OK;
}

int order_after_pass(gss_engine *eng, const DevBuf &reports, const DevBuf &counts) {
    OrderState &o = *eng->order;
    GSS_CUDA_TRY(cudaEventRecord(o.ev[3], eng->stream));
    const int64_t q = o.pass - 1;  // the pass just enqueued
    const unsigned hist_blocks = eng->n_parts * (unsigned) std::max(1, (eng->sm_count * 4) / (int) eng->n_parts);
    history_kernel<<<hist_blocks, 256, 0, eng->stream>>>((const gss_report *) reports.ptr,
                                                          (const uint32_t *) counts.ptr, eng->n_parts,
                                                          eng->cap_per_part, (ClauseRecord *) o.rec.ptr,
                                                          (uint32_t) std::min<int64_t>(eng->next_id, o.cap_ids),
                                                          (uint32_t) (q & 1));
    GSS_CUDA_TRY(cudaGetLastError());
    o.have_times = true;
    // the order of pass q+1, on the scoring stream once the head of pass q is
    // done (overlap) or pass q is: it folds the counts of pass q-1 (complete)
    GSS_CUDA_TRY(cudaStreamWaitEvent(o.score_stream, o.prm.overlap ? o.ev[2] : o.ev[3], 0));
    uint32_t covered = 0;
    int buf = 0;
    GSS_TRY(score_pass(eng, o.score_stream, q + 1, &covered, &buf));
    GSS_CUDA_TRY(cudaEventRecord(o.ev_score_done, o.score_stream));
    o.pre_in_flight = true;
    o.pre_ready = true;
    o.pre_pass = q + 1;
    o.pre_n = covered;
    o.pre_buf = buf;
    o.pre_layout = eng->layout_epoch;
    return GSS_OK;
}

}  // namespace gss

using namespace gss;

struct gss_scorer {
    Scorer s;
    cudaStream_t stream = nullptr;
};

extern "C" {

void gss_order_params_default(gss_order_params *p) {
    if (!p) return;
    p->head_fraction = 0.1;
    p->retrain_interval = 1000;
    p->train_epochs = 2;
    p->batch = 4096;
    p->learning_rate = 1e-3f;
    p->log_capacity = 1 << 20;
    p->log_rate = 0.0;
    p->seed = 1;
    p->overlap = 1;
    p->rescore_interval = 1;
}

int gss_order_enable(gss_engine *eng, const gss_order_params *p) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    gss_order_params prm;
    gss_order_params_default(&prm);
    if (p) prm = *p;
    if (!(prm.head_fraction >= 0.0 && prm.head_fraction <= 1.0) || prm.retrain_interval < 0 || prm.batch < 1 ||
        prm.log_capacity < 0 || prm.log_capacity > (int64_t) 1 << 31 || !(prm.learning_rate > 0.0f) ||
        prm.rescore_interval < 1)
        return set_error(GSS_ERR_INVALID, "bad learned-order parameters");
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    if (eng->order) order_destroy(eng);
    OrderState *o = new OrderState();
    o->prm = prm;
    o->rng.seed(prm.seed * 0x9E3779B97F4A7C15ull + 7);
    o->epoch = eng->db_epoch;
    eng->order = o;
    int rc = scorer_init(&o->scorer, eng->device, prm.seed, eng->stream);
    if (rc == GSS_OK) rc = scorer_init(&o->trainer, eng->device, prm.seed, eng->stream);  // the same weights
    for (int k = 0; rc == GSS_OK && k < 6; k++)
        if (cudaEventCreate(&o->ev[k]) != cudaSuccess) rc = set_error(GSS_ERR_CUDA, "cudaEventCreate failed");
    if (rc == GSS_OK && (cudaEventCreateWithFlags(&o->ev_score_done, cudaEventDisableTiming) != cudaSuccess ||
                         cudaStreamCreateWithFlags(&o->score_stream, cudaStreamNonBlocking) != cudaSuccess))
        rc = set_error(GSS_ERR_CUDA, "creating the scoring stream failed");
    if (rc == GSS_OK && (cudaEventCreateWithFlags(&o->ev_train_start, cudaEventDisableTiming) != cudaSuccess ||
                         cudaEventCreateWithFlags(&o->ev_train_done, cudaEventDisableTiming) != cudaSuccess ||
                         cudaStreamCreateWithFlags(&o->train_stream, cudaStreamNonBlocking) != cudaSuccess))
        rc = set_error(GSS_ERR_CUDA, "creating the training stream failed");
    if (rc == GSS_OK && prm.log_capacity > 0) {
        rc = o->log_x.reserve((size_t) prm.log_capacity * kF * sizeof(float));
        if (rc == GSS_OK) rc = o->log_y.reserve((size_t) prm.log_capacity * sizeof(float));
    }
    if (rc == GSS_OK) rc = o->log_count.reserve(sizeof(unsigned long long));
    if (rc == GSS_OK) rc = o->h_log_count.reserve(sizeof(unsigned long long));
    if (rc == GSS_OK && cudaMemsetAsync(o->log_count.ptr, 0, sizeof(unsigned long long), eng->stream) != cudaSuccess)
        rc = set_error(GSS_ERR_CUDA, "cudaMemsetAsync failed");
    if (rc == GSS_OK) rc = ensure_ids(eng, std::max<int64_t>(eng->next_id, 1));
    if (rc != GSS_OK) {
        order_destroy(eng);
        return rc;
    }
    return GSS_OK;
}

int gss_order_disable(gss_engine *eng) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    order_quiesce(eng);
    if (eng->pass_pending) return set_error(GSS_ERR_STATE, "a pass is in flight");
    order_destroy(eng);
    return GSS_OK;
}

int gss_order_set_active(gss_engine *eng, int on) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    order_quiesce(eng);
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    if (eng->pass_pending) return set_error(GSS_ERR_STATE, "a pass is in flight");
    eng->order->active = on != 0;
    return GSS_OK;
}

int gss_db_set_lbd(gss_engine *eng, const uint32_t *ids, const uint16_t *lbd, int64_t n) {
    if (!eng || n < 0 || (n > 0 && (!ids || !lbd))) return set_error(GSS_ERR_INVALID, "bad arguments to gss_db_set_lbd");
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    if (n == 0) return GSS_OK;
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    uint32_t max_id = 0;
    for (int64_t i = 0; i < n; i++) max_id = std::max(max_id, ids[i]);
    if (max_id >= eng->next_id) return set_error(GSS_ERR_NOT_FOUND, "clause id %u is not in the database", max_id);
    order_quiesce(eng);
    GSS_TRY(ensure_ids(eng, eng->next_id));
    // (id, lbd) pairs up, then a scatter into the records
    OrderState &o = *eng->order;
    std::vector<uint32_t> pairs((size_t) n * 2);
    for (int64_t i = 0; i < n; i++) {
        pairs[2 * i] = ids[i];
        pairs[2 * i + 1] = lbd[i];
    }
    GSS_TRY(o.lbd_pairs.reserve(pairs.size() * sizeof(uint32_t)));
    GSS_CUDA_TRY(cudaMemcpyAsync(o.lbd_pairs.ptr, pairs.data(), pairs.size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, eng->stream));
    set_lbd_kernel<<<grid_for_n((uint64_t) n, eng->sm_count, 256), 256, 0, eng->stream>>>(
        (const uint32_t *) o.lbd_pairs.ptr, (uint32_t) n, (ClauseRecord *) o.rec.ptr);
    GSS_CUDA_TRY(cudaGetLastError());
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));  // the pairs are pageable
    return GSS_OK;
}

int gss_check_wait_head(gss_engine *eng, gss_report *out, int64_t cap, int64_t *n_reports) {
    if (!eng || (cap > 0 && !out)) return set_error(GSS_ERR_INVALID, "bad arguments to gss_check_wait_head");
    if (!eng->order || !eng->order->active || !eng->order->pending || !eng->pass_pending)
        return set_error(GSS_ERR_STATE, "no ordered pass in flight");
    OrderState &o = *eng->order;
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    GSS_CUDA_TRY(cudaEventSynchronize(o.ev[4]));
    const uint32_t *hc = (const uint32_t *) o.h_head_counts.ptr;
    int64_t total = 0;
    for (uint32_t q = 0; q < eng->n_parts; q++) {
        if (hc[q] > eng->cap_per_part) {
            if (n_reports) *n_reports = -1;
            return set_error(GSS_ERR_OVERFLOW, "report queues overflowed in the head of the pass");
        }
        total += hc[q];
    }
    if (n_reports) *n_reports = total;
    if (total > cap) return set_error(GSS_ERR_OVERFLOW, "output holds %lld records, the head has %lld",
                                      (long long) cap, (long long) total);
    if (!eng->d2h) GSS_CUDA_TRY(cudaStreamCreateWithFlags(&eng->d2h, cudaStreamNonBlocking));
    int64_t pos = 0;
    for (uint32_t q = 0; q < eng->n_parts; q++) {
        if (!hc[q]) continue;
        GSS_CUDA_TRY(cudaMemcpyAsync(out + pos, (gss_report *) eng->reports.ptr + (size_t) q * eng->cap_per_part,
                                     (size_t) hc[q] * sizeof(gss_report), cudaMemcpyDeviceToHost, eng->d2h));
        pos += hc[q];
    }
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->d2h));
    return GSS_OK;
}

int gss_check_copy_tail(gss_engine *eng, gss_report *out, int64_t cap, int64_t *n_reports) {
    if (!eng || (cap > 0 && !out)) return set_error(GSS_ERR_INVALID, "bad arguments to gss_check_copy_tail");
    if (!eng->order || !eng->order->active || !eng->order->pending)
        return set_error(GSS_ERR_STATE, "no ordered pass whose head was taken");
    int64_t total = 0;
    GSS_TRY(gss_check_wait(eng, &total));
    OrderState &o = *eng->order;
    const uint32_t *hc = (const uint32_t *) o.h_head_counts.ptr;
    const uint32_t *ac = (const uint32_t *) eng->h_counts.ptr;
    int64_t n = 0;
    for (uint32_t q = 0; q < eng->n_parts; q++) n += (int64_t) ac[q] - hc[q];
    if (n_reports) *n_reports = n;
    if (n > cap) return set_error(GSS_ERR_OVERFLOW, "output holds %lld records, the tail has %lld", (long long) cap,
                                  (long long) n);
    int64_t pos = 0;
    for (uint32_t q = 0; q < eng->n_parts; q++) {
        if (ac[q] == hc[q]) continue;
        GSS_CUDA_TRY(cudaMemcpyAsync(out + pos,
                                     (gss_report *) eng->reports.ptr + (size_t) q * eng->cap_per_part + hc[q],
                                     (size_t) (ac[q] - hc[q]) * sizeof(gss_report), cudaMemcpyDeviceToHost,
                                     eng->stream));
        pos += ac[q] - hc[q];
    }
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    return GSS_OK;
}

int gss_order_scan_ranks(gss_engine *eng, const uint32_t *ids, int64_t n, int64_t *ranks) {
    if (!eng || n < 0 || (n > 0 && (!ids || !ranks))) return set_error(GSS_ERR_INVALID, "bad arguments");
    if (!eng->order || eng->order->pass == 0) return set_error(GSS_ERR_STATE, "no ordered pass yet");
    if (n == 0) return GSS_OK;
    OrderState &o = *eng->order;
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    // the last pass's permutation, inverted on the host (a diagnostic)
    const uint32_t covered = o.scored_n;
    std::vector<uint32_t> perm(covered);
    if (covered)
        GSS_CUDA_TRY(cudaMemcpy(perm.data(), o.perm[o.inflight_buf].ptr, covered * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost));
    std::vector<int64_t> rank_of_pos((size_t) eng->n_clauses, -1);
    for (uint32_t r = 0; r < covered; r++)
        if (perm[r] < rank_of_pos.size()) rank_of_pos[perm[r]] = r;
    for (int64_t p = covered; p < eng->n_clauses; p++) rank_of_pos[p] = p;  // scanned in place
    for (int64_t i = 0; i < n; i++) {
        const uint32_t id = ids[i];
        const uint32_t pos = id < eng->index_of.size() ? eng->index_of[id] : 0xFFFFFFFFu;
        ranks[i] = pos == 0xFFFFFFFFu || pos >= rank_of_pos.size() ? -1 : rank_of_pos[pos];
    }
    return GSS_OK;
}

int gss_order_get_stats(gss_engine *eng, gss_order_stats *out) {
    if (!eng || !out) return set_error(GSS_ERR_INVALID, "bad arguments to gss_order_get_stats");
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    OrderState &o = *eng->order;
    memset(out, 0, sizeof *out);
    out->passes = o.pass;
    out->trainings = o.trainings;
    out->last_loss = o.last_loss;
    out->head_positions = o.head;
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    GSS_CUDA_TRY(cudaMemcpy(o.h_log_count.ptr, o.log_count.ptr, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    out->logged = (int64_t) std::min<unsigned long long>(*(unsigned long long *) o.h_log_count.ptr,
                                                          (unsigned long long) o.prm.log_capacity);
    if (o.have_times && !eng->pass_pending) {
        float a = 0, b = 0, c = 0;
        order_quiesce(eng);
        GSS_CUDA_TRY(cudaEventSynchronize(o.ev[3]));
        GSS_CUDA_TRY(cudaEventElapsedTime(&a, o.ev[0], o.ev[1]));
        GSS_CUDA_TRY(cudaEventElapsedTime(&b, o.ev[5], o.ev[2]));
        GSS_CUDA_TRY(cudaEventElapsedTime(&c, o.ev[2], o.ev[3]));
        out->score_ms = a;
        out->head_ms = b;
        out->tail_ms = c;
    }
    return GSS_OK;
}

int gss_order_train(gss_engine *eng) {
    if (!eng) return set_error(GSS_ERR_INVALID, "engine is NULL");
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    if (eng->pass_pending) return set_error(GSS_ERR_STATE, "a pass is in flight");
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    order_quiesce(eng);
    GSS_TRY(train_finish(eng, true));
    GSS_TRY(train_start(eng));
    return train_finish(eng, true);
}

int gss_order_clause_features(gss_engine *eng, const uint32_t *ids, int64_t n, float *x) {
    if (!eng || n < 0 || (n > 0 && (!ids || !x))) return set_error(GSS_ERR_INVALID, "bad arguments");
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    if (eng->pass_pending) return set_error(GSS_ERR_STATE, "a pass is in flight");
    if (n == 0) return GSS_OK;
    OrderState &o = *eng->order;
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    order_quiesce(eng);
    const int64_t n_rec = std::min<int64_t>(eng->next_id, o.cap_ids);
    // a host copy of the records (a diagnostic, not a hot path)
    std::vector<ClauseRecord> rec((size_t) n_rec);
    if (n_rec) GSS_CUDA_TRY(cudaMemcpy(rec.data(), o.rec.ptr, n_rec * sizeof(ClauseRecord), cudaMemcpyDeviceToHost));
    // features of the next pass q: now = q - 1, and the counts of pass q - 2
    // folded in (already done when the next pass was scored in advance)
    const int64_t q = o.pass;
    const int32_t now = (int32_t) (q - 1);
    const bool fold = o.folded_pass < q && q >= 2;
    for (int64_t i = 0; i < n; i++) {
        const uint32_t id = ids[i];
        if (id >= eng->next_id || eng->index_of.size() <= id || eng->index_of[id] == 0xFFFFFFFFu ||
            (int64_t) id >= n_rec)
            return set_error(GSS_ERR_NOT_FOUND, "clause id %u is not in the database", id);
        const uint32_t pos = eng->index_of[id];
        const uint32_t len = (uint32_t) (eng->h_off[pos + 1] - eng->h_off[pos]);
        const ClauseRecord &r = rec[id];
        float f[kF];
        if (id < o.known_ids) {
            uint64_t hh = r.hist;
            uint32_t tot = r.total;
            int32_t lst = r.last;
            if (fold) {
                const uint32_t c = (q & 1) ? r.cur1 : r.cur0;
                if (c) {
                    hh = hist_at(hh, lst, (int32_t) (q - 2)) | (uint64_t) std::min<uint32_t>(c, 255u);
                    tot += c;
                    lst = (int32_t) (q - 2);
                }
            }
            clause_features(len, r.lbd, now - r.birth, hist_at(hh, lst, now - 1), tot, lst < 0 ? -1 : now - lst, f);
        } else {
            clause_features(len, r.lbd, 0, 0, 0, -1, f);  // first scored in the next pass
        }
        memcpy(x + i * kF, f, sizeof f);
    }
    return GSS_OK;
}

int gss_order_get_weights(gss_engine *eng, float *w) {
    if (!eng || !w) return set_error(GSS_ERR_INVALID, "bad arguments to gss_order_get_weights");
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    GSS_CUDA_TRY(cudaMemcpyAsync(w, eng->order->scorer.w.ptr, kP * sizeof(float), cudaMemcpyDeviceToHost,
                                 eng->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    return GSS_OK;
}

int gss_order_set_weights(gss_engine *eng, const float *w) {
    if (!eng || !w) return set_error(GSS_ERR_INVALID, "bad arguments to gss_order_set_weights");
    if (!eng->order) return set_error(GSS_ERR_STATE, "the learned order is not enabled");
    if (eng->pass_pending) return set_error(GSS_ERR_STATE, "a pass is in flight");
    GSS_CUDA_TRY(cudaSetDevice(eng->device));
    order_quiesce(eng);
    GSS_TRY(train_finish(eng, true));
    GSS_CUDA_TRY(cudaMemcpyAsync(eng->order->scorer.w.ptr, w, kP * sizeof(float), cudaMemcpyHostToDevice,
                                 eng->stream));
    GSS_CUDA_TRY(cudaMemcpyAsync(eng->order->trainer.w.ptr, w, kP * sizeof(float), cudaMemcpyHostToDevice,
                                 eng->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(eng->stream));
    eng->order->scorer.frag_stale = true;
    return GSS_OK;
}

// ---- the scorer on its own ----

int gss_scorer_create(int device, uint64_t seed, gss_scorer **out) {
    if (!out) return set_error(GSS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    GSS_CUDA_TRY(cudaSetDevice(device));
    gss_scorer *s = new gss_scorer();
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return set_error(GSS_ERR_CUDA, "cudaStreamCreate failed");
    }
    const int rc = scorer_init(&s->s, device, seed, s->stream);
    if (rc != GSS_OK) {
        cudaStreamDestroy(s->stream);
        delete s;
        return rc;
    }
    *out = s;
    return GSS_OK;
}

int gss_scorer_destroy(gss_scorer *s) {
    if (!s) return GSS_OK;
    cudaSetDevice(s->s.device);
    if (s->stream) {
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    delete s;
    return GSS_OK;
}

int gss_scorer_get_weights(gss_scorer *s, float *w) {
    if (!s || !w) return set_error(GSS_ERR_INVALID, "bad arguments to gss_scorer_get_weights");
    GSS_CUDA_TRY(cudaSetDevice(s->s.device));
    GSS_CUDA_TRY(cudaMemcpyAsync(w, s->s.w.ptr, kP * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return GSS_OK;
}

int gss_scorer_set_weights(gss_scorer *s, const float *w) {
    if (!s || !w) return set_error(GSS_ERR_INVALID, "bad arguments to gss_scorer_set_weights");
    GSS_CUDA_TRY(cudaSetDevice(s->s.device));
    GSS_CUDA_TRY(cudaMemcpyAsync(s->s.w.ptr, w, kP * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->s.frag_stale = true;
    return GSS_OK;
}

namespace {
int upload_rows(gss_scorer *s, const float *x, const float *y, int64_t n) {
    GSS_TRY(s->s.io_x.reserve((size_t) n * kF * sizeof(float)));
    GSS_CUDA_TRY(cudaMemcpyAsync(s->s.io_x.ptr, x, (size_t) n * kF * sizeof(float), cudaMemcpyHostToDevice,
                                 s->stream));
    if (y) {
        GSS_TRY(s->s.io_y.reserve((size_t) n * sizeof(float)));
        GSS_CUDA_TRY(cudaMemcpyAsync(s->s.io_y.ptr, y, (size_t) n * sizeof(float), cudaMemcpyHostToDevice,
                                     s->stream));
    }
    return GSS_OK;
}
}  // namespace

int gss_scorer_infer(gss_scorer *s, const float *x, int64_t n, float *logits) {
    if (!s || n < 0 || (n > 0 && (!x || !logits)) || n > 0x7FFFFFFF)
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_scorer_infer");
    if (n == 0) return GSS_OK;
    GSS_CUDA_TRY(cudaSetDevice(s->s.device));
    GSS_TRY(upload_rows(s, x, nullptr, n));
    GSS_TRY(s->s.io_out.reserve((size_t) n * sizeof(float)));
    GSS_TRY(scorer_frags(&s->s, s->stream));
    int sm = 0;
    GSS_CUDA_TRY(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, s->s.device));
    infer_rows_kernel<<<grid_for_n((uint64_t) (n + 15) / 16 * 32, sm, kMlpThreads), kMlpThreads, 0, s->stream>>>(
        (const float *) s->s.w.ptr, (const uint32_t *) s->s.frag.ptr, (const float *) s->s.io_x.ptr, (uint32_t) n,
        (float *) s->s.io_out.ptr);
    GSS_CUDA_TRY(cudaGetLastError());
    GSS_CUDA_TRY(cudaMemcpyAsync(logits, s->s.io_out.ptr, (size_t) n * sizeof(float), cudaMemcpyDeviceToHost,
                                 s->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return GSS_OK;
}

int gss_scorer_gradient(gss_scorer *s, const float *x, const float *y, int64_t n, float *grad, float *loss) {
    if (!s || n <= 0 || n > (1 << 24) || !x || !y || !grad)
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_scorer_gradient");
    GSS_CUDA_TRY(cudaSetDevice(s->s.device));
    GSS_TRY(upload_rows(s, x, y, n));
    GSS_TRY(scorer_grad_dev(&s->s, (const float *) s->s.io_x.ptr, (const float *) s->s.io_y.ptr, (uint32_t) n, 0,
                            (uint32_t) n, s->stream));
    GSS_CUDA_TRY(cudaMemcpyAsync(grad, s->s.grad.ptr, kP * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    float l = 0.0f;
    GSS_CUDA_TRY(cudaMemcpyAsync(&l, s->s.loss.ptr, sizeof l, cudaMemcpyDeviceToHost, s->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (loss) *loss = l;
    return GSS_OK;
}

int gss_scorer_train_step(gss_scorer *s, const float *x, const float *y, int64_t n, float lr, float *loss) {
    if (!s || n <= 0 || n > (1 << 24) || !x || !y || !(lr > 0.0f))
        return set_error(GSS_ERR_INVALID, "bad arguments to gss_scorer_train_step");
    GSS_CUDA_TRY(cudaSetDevice(s->s.device));
    GSS_TRY(upload_rows(s, x, y, n));
    GSS_TRY(scorer_grad_dev(&s->s, (const float *) s->s.io_x.ptr, (const float *) s->s.io_y.ptr, (uint32_t) n, 0,
                            (uint32_t) n, s->stream));
    GSS_TRY(scorer_adam_dev(&s->s, lr, s->stream));
    float l = 0.0f;
    GSS_CUDA_TRY(cudaMemcpyAsync(&l, s->s.loss.ptr, sizeof l, cudaMemcpyDeviceToHost, s->stream));
    GSS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (loss) *loss = l;
    return GSS_OK;
}

}  // extern "C"
