// Clause activity and the reduceDb policy; see activity.h.
#include "activity.h"

#include <math.h>

#include <algorithm>
#include <limits>
#include <vector>

#include "gpusharesat.h"

namespace gss {

uint32_t ClauseActivity::add(int lbd) {
    decay();
    act_.push_back(incr_);
    lbd_.push_back(lbd);
    if (incr_ > kActivityRescale) rescale();
    return (uint32_t) act_.size() - 1;
}

void ClauseActivity::bump(uint32_t i) {
    act_[i] += incr_;
    if (act_[i] > kActivityRescale) rescale();
}

void ClauseActivity::rescale() {
    for (float &a : act_) a /= kActivityRescale;
    incr_ /= kActivityRescale;
}

void ClauseActivity::compact(const std::vector<uint8_t> &keep) {
    size_t j = 0;
    for (size_t i = 0; i < act_.size(); i++) {
        if (keep[i]) {
            act_[j] = act_[i];
            lbd_[j] = lbd_[i];
            j++;
        }
    }
    act_.resize(j);
    lbd_.resize(j);
}

void ClauseActivity::permute(const std::vector<uint32_t> &order) {
    std::vector<float> a(order.size());
    std::vector<int> l(order.size());
    for (size_t k = 0; k < order.size(); k++) {
        a[k] = act_[order[k]];
        l[k] = lbd_[order[k]];
    }
    act_.swap(a);
    lbd_.swap(l);
}

void ClauseActivity::permute_tail(size_t first, const std::vector<uint32_t> &order) {
    std::vector<float> a(order.size());
    std::vector<int> l(order.size());
    for (size_t k = 0; k < order.size(); k++) {
        a[k] = act_[first + order[k]];
        l[k] = lbd_[first + order[k]];
    }
    std::copy(a.begin(), a.end(), act_.begin() + first);
    std::copy(l.begin(), l.end(), lbd_.begin() + first);
}

float ClauseActivity::approx_nth(int min_lbd, int max_lbd, int64_t n) const {
    if (n == 0) return 0.0f;
    const int buckets = 20000;
    std::vector<int64_t> counts(buckets, 0);
    const float lo = logf(std::numeric_limits<float>::min());
    const float hi = logf(std::numeric_limits<float>::max());
    const float step = (hi - lo) / buckets;
    for (size_t i = 0; i < act_.size(); i++) {
        if (lbd_[i] < min_lbd || lbd_[i] >= max_lbd) continue;
        int b = (int) floor(((double) logf(act_[i]) - (double) lo) / (double) step);
        if (b < 0) b = 0;
        if (b >= buckets) b = buckets - 1;
        counts[b]++;
    }
    int64_t seen = 0;
    for (int b = 0; b < buckets; b++) {
        seen += counts[b];
        if (seen >= n) return expf(lo + (b + 1) * step);  // upper bound of the bucket
    }
    return std::numeric_limits<float>::max();
}

void ClauseActivity::removing_thresholds(bool act_only, int64_t total, int &min_lim, int &max_lim,
                                         float &act) const {
    if (act_only) {
        min_lim = 0;
        max_lim = kLbdLimit;
        act = approx_nth(min_lim, max_lim, total / 2);
        return;
    }
    // median LBD (HostClauses::getMedianLbd)
    std::vector<int64_t> at_lbd(kLbdLimit + 1, 0);
    for (int l : lbd_)
        if (l >= 0 && l <= kLbdLimit) at_lbd[l]++;
    int64_t seen = 0, under = 0, at_med = 0;
    int med = kLbdLimit;
    for (int l = 0; l <= kLbdLimit; l++) {
        seen += at_lbd[l];
        if (seen >= total / 2) {
            med = l;
            under = seen - at_lbd[l];
            at_med = at_lbd[l];
            break;
        }
    }
    min_lim = med;
    if (min_lim <= 2) {
        // clauses with lbd <= 2 are never removed
        min_lim = 2;
        max_lim = 3;
        act = 0.0f;
        return;
    }
    max_lim = min_lim + 1;
    const int64_t target = total / 2;
    const int64_t keep_at_med = target - under;
    act = approx_nth(min_lim, max_lim, at_med - keep_at_med);
}

}  // namespace gss

// ---- C ABI: the reduceDb policy on its own, for callers and tests ----

struct gss_activity {
    gss::ClauseActivity impl;
    explicit gss_activity(float d) : impl(d) {}
};

extern "C" {

gss_activity *gss_activity_create(float decay) { return new gss_activity(decay); }

void gss_activity_destroy(gss_activity *a) { delete a; }

int64_t gss_activity_add(gss_activity *a, int lbd) { return a ? (int64_t) a->impl.add(lbd) : -1; }

int gss_activity_bump(gss_activity *a, int64_t i) {
    if (!a || i < 0 || i >= a->impl.size()) return GSS_ERR_INVALID;
    a->impl.bump((uint32_t) i);
    return GSS_OK;
}

int gss_activity_decay(gss_activity *a) {
    if (!a) return GSS_ERR_INVALID;
    a->impl.decay();
    return GSS_OK;
}

float gss_activity_get(const gss_activity *a, int64_t i) {
    if (!a || i < 0 || i >= a->impl.size()) return -1.0f;
    return a->impl.activity((uint32_t) i);
}

float gss_activity_approx_nth(const gss_activity *a, int min_lbd, int max_lbd, int64_t n) {
    return a ? a->impl.approx_nth(min_lbd, max_lbd, n) : -1.0f;
}

int gss_activity_removing_thresholds(const gss_activity *a, int act_only, int64_t total, int *min_lim, int *max_lim,
                                     float *act) {
    if (!a || !min_lim || !max_lim || !act) return GSS_ERR_INVALID;
    a->impl.removing_thresholds(act_only != 0, total, *min_lim, *max_lim, *act);
    return GSS_OK;
}

}  // extern "C"
