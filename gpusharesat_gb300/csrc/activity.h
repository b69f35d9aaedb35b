// Clause activity and the reduceDb policy (host only).
//
// Restates gpuShareLib/Clauses.cu:231-291 (bump, decay, rescale),
// :377-417 (median LBD and the removal thresholds) and :488-525
// (approxNthAct), with the same float arithmetic, so that the set of clauses a
// reduceDb keeps is the reference's.
#pragma once

#include <stdint.h>

#include <vector>

namespace gss {

constexpr float kActivityRescale = 1e19f;  // RESCALE_CONST, gpuShareLib/Clauses.cuh:39
constexpr int kLbdLimit = 100;             // MAX_CL_SIZE, gpuShareLib/BaseTypes.cuh:28

class ClauseActivity {
public:
    explicit ClauseActivity(float decay) : decay_(decay) {}

    // Decays the increment, then gives a new clause that increment as its
    // activity (getUpdatesForDevice + PerSizeKeeper::addClause). Returns its index.
    uint32_t add(int lbd);
    void bump(uint32_t i);
    void decay() { incr_ /= decay_; }
    float activity(uint32_t i) const { return act_[i]; }
    int lbd(uint32_t i) const { return lbd_[i]; }
    uint32_t size() const { return (uint32_t) act_.size(); }
    float increment() const { return incr_; }

    // Keeps the entries whose flag is set, in order.
    void compact(const std::vector<uint8_t> &keep);
    // Reorders: new entry k is old entry order[k].
    void permute(const std::vector<uint32_t> &order);
    // Reorders the entries from `first` on: new entry first + k is old entry
    // first + order[k].
    void permute_tail(size_t first, const std::vector<uint32_t> &order);
    // room for n clauses without reallocating
    void reserve(size_t n) {
        act_.reserve(n);
        lbd_.reserve(n);
    }

    // An approximation, from above, of the n-th lowest activity among entries
    // with min_lbd <= lbd < max_lbd (20000 logarithmic buckets). 0 for n = 0;
    // the largest float when fewer than n entries qualify.
    float approx_nth(int min_lbd, int max_lbd, int64_t n) const;

    // The thresholds of a reduceDb that keeps about half of `total` clauses:
    // keep lbd < min_lim, or lbd < max_lim with activity >= act.
    // act_only: by activity alone (min_lim 0, max_lim 100).
    void removing_thresholds(bool act_only, int64_t total, int &min_lim, int &max_lim, float &act) const;
    static bool keep(int lbd, float activity, int min_lim, int max_lim, float act) {
        return lbd < min_lim || (lbd < max_lim && activity >= act);
    }

private:
    void rescale();
    float incr_ = 1.0f;
    float decay_;
    std::vector<float> act_;
    std::vector<int> lbd_;
};

}  // namespace gss
