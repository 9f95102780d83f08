// gbmp_autotune.h -- launch-shape autotuner of the batched planner (host side, plain C++).
//
// A batched planning launch has one free shape parameter, the lanes (4-warp blocks) each
// problem starts with; how many pay off depends on the mix of problems (how many, their
// DOF, sphere and obstacle counts) and on the settings.  The tuner keys a decision by a
// signature of that shape, tries each candidate `trials` times on the caller's own
// solves (each call of an undecided key takes the next candidate still short of its
// trials and reports its time), then keeps the fastest for the key.  A candidate's time
// is the least of its trials, so a first call that also captured a CUDA graph for the
// new launch shape does not count against it.  No CUDA types: the timing comes from the
// caller, so the policy is testable on a machine without a GPU
// (tests/cpp/autotune_check.cpp).
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

namespace gbmp {

struct ShapeKey {
    uint64_t hash = 1469598103934665603ULL;   // FNV-1a over the fields added
    void add(uint64_t v) {
        for (int i = 0; i < 8; ++i) {
            hash ^= (v >> (8 * i)) & 0xffu;
            hash *= 1099511628211ULL;
        }
    }
};

// Bucket of a count for the key: exact below 16, then powers of two (problems that
// differ by a few spheres or obstacles share a decision).
inline uint64_t shape_bucket(int64_t v) {
    if (v < 16) return (uint64_t)(v < 0 ? 0 : v);
    uint64_t b = 16;
    while ((int64_t)(b * 2) <= v) b *= 2;
    return 1000 + b;
}

class LaneTuner {
  public:
    struct Entry {
        std::vector<int> cand;       // candidates in trial order
        std::vector<double> ms;      // least time per candidate (< 0: not yet tried)
        std::vector<int> runs;       // trials reported per candidate
        int best = -1;               // index into cand once decided
    };

    LaneTuner(std::vector<int> candidates, int trials) : candidates_(std::move(candidates)), trials_(trials) {}

    // Lanes per problem for the next solve of `key`, among the candidates allowed by
    // `max_lanes` (at least the smallest candidate).  `trial` is set when the value is an
    // exploration whose time must be reported.
    int choose(uint64_t key, int max_lanes, bool *trial) {
        std::lock_guard<std::mutex> lock(mu_);
        Entry &e = entry(key, max_lanes);
        if (e.best >= 0) {
            *trial = false;
            return e.cand[e.best];
        }
        for (size_t i = 0; i < e.cand.size(); ++i)
            if (e.runs[i] < trials_) {
                *trial = true;
                return e.cand[i];
            }
        *trial = false;
        return e.cand[pick(e)];
    }

    // Time of a solve of `key` run with `lanes` chosen as a trial.
    void report(uint64_t key, int lanes, double ms) {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = table_.find(key);
        if (it == table_.end() || it->second.best >= 0) return;
        Entry &e = it->second;
        for (size_t i = 0; i < e.cand.size(); ++i)
            if (e.cand[i] == lanes && e.runs[i] < trials_) {
                e.ms[i] = e.ms[i] < 0.0 ? ms : (ms < e.ms[i] ? ms : e.ms[i]);
                ++e.runs[i];
            }
        bool all = true;
        for (int r : e.runs) all &= r >= trials_;
        if (all) e.best = pick(e);
    }

    // Decision for `key`: its candidates, their times (-1 untried) and the chosen lanes
    // (-1 while exploring).  Returns false for an unknown key.
    bool lookup(uint64_t key, std::vector<int> *cand, std::vector<double> *ms, int *best) {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = table_.find(key);
        if (it == table_.end()) return false;
        if (cand) *cand = it->second.cand;
        if (ms) *ms = it->second.ms;
        if (best) *best = it->second.best >= 0 ? it->second.cand[it->second.best] : -1;
        return true;
    }

    void reset() {
        std::lock_guard<std::mutex> lock(mu_);
        table_.clear();
    }

  private:
    Entry &entry(uint64_t key, int max_lanes) {
        auto it = table_.find(key);
        if (it != table_.end()) return it->second;
        Entry e;
        for (int c : candidates_)
            if (c <= max_lanes) e.cand.push_back(c);
        if (e.cand.empty()) e.cand.push_back(candidates_.front());
        e.ms.assign(e.cand.size(), -1.0);
        e.runs.assign(e.cand.size(), 0);
        return table_.emplace(key, e).first->second;
    }
    static int pick(const Entry &e) {
        int b = 0;
        for (size_t i = 1; i < e.ms.size(); ++i)
            if (e.ms[i] < e.ms[b]) b = (int)i;   // ties keep the earlier (fewer lanes)
        return b;
    }

    std::vector<int> candidates_;
    int trials_;
    std::mutex mu_;
    std::map<uint64_t, Entry> table_;
};

}  // namespace gbmp
