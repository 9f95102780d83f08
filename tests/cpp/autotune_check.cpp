// Host-side check of the batched planner's launch-shape tuner (gbmp_autotune.h) with a
// fake timer: every candidate allowed for a key is tried `trials` times in order, the
// least time of each counts, the fastest is kept, keys are independent, candidates above
// the key's lane limit are never chosen, and concurrent reports are consistent.
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "gbmp_autotune.h"

#define CHECK(c)                                                    \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAILED %s at line %d\n", #c, __LINE__);    \
            std::exit(1);                                           \
        }                                                           \
    } while (0)

// fake solve time of a lane count for key k: a valley at 16 lanes (key 1) or 4 (key 2);
// the first run of each candidate is slower (a graph capture)
static double fake_ms(int key, int lanes, int run) {
    const double base = key == 1 ? (lanes == 16 ? 10.0 : 20.0 + lanes) : (lanes == 4 ? 5.0 : 9.0 + lanes);
    return run == 0 ? base + 100.0 : base;
}

int main() {
    gbmp::LaneTuner t({4, 8, 16, 32, 64}, 2);
    // key 1: explores 4, 4, 8, 8, 16, 16, 32, 32, 64, 64, then keeps 16
    std::vector<int> seen;
    for (int call = 0; call < 10; ++call) {
        bool trial = false;
        const int l = t.choose(1, 4096, &trial);
        CHECK(trial);
        seen.push_back(l);
        t.report(1, l, fake_ms(1, l, call % 2));
    }
    const int order[10] = {4, 4, 8, 8, 16, 16, 32, 32, 64, 64};
    for (int i = 0; i < 10; ++i) CHECK(seen[i] == order[i]);
    for (int call = 0; call < 5; ++call) {
        bool trial = true;
        CHECK(t.choose(1, 4096, &trial) == 16);
        CHECK(!trial);
    }
    std::vector<int> cand;
    std::vector<double> ms;
    int best = 0;
    CHECK(t.lookup(1, &cand, &ms, &best));
    CHECK(best == 16 && cand.size() == 5 && ms[2] == 10.0 && ms[0] == 24.0);
    // reports after the decision change nothing
    t.report(1, 64, 0.001);
    CHECK(t.lookup(1, nullptr, nullptr, &best) && best == 16);

    // key 2 with a lane limit of 10: only 4 and 8 are candidates; 4 wins
    for (int call = 0; call < 4; ++call) {
        bool trial = false;
        const int l = t.choose(2, 10, &trial);
        CHECK(trial && l <= 10);
        t.report(2, l, fake_ms(2, l, call % 2));
    }
    bool trial = true;
    CHECK(t.choose(2, 10, &trial) == 4 && !trial);
    CHECK(t.lookup(2, &cand, nullptr, &best) && cand.size() == 2 && best == 4);

    // a limit below every candidate still gives the smallest one
    CHECK(t.choose(3, 2, &trial) == 4);
    CHECK(!t.lookup(99, nullptr, nullptr, nullptr));

    // concurrent callers on one key: the decision is made once and is one of the candidates
    gbmp::LaneTuner c({4, 8, 16, 32, 64}, 2);
    std::vector<std::thread> th;
    for (int w = 0; w < 8; ++w)
        th.emplace_back([&c, w] {
            for (int i = 0; i < 50; ++i) {
                bool tr = false;
                const int l = c.choose(7, 4096, &tr);
                if (tr) c.report(7, l, fake_ms(1, l, (i + w) % 2));
            }
        });
    for (auto &x : th) x.join();
    CHECK(c.lookup(7, nullptr, nullptr, &best) && best == 16);
    t.reset();
    CHECK(!t.lookup(1, nullptr, nullptr, nullptr));
    std::printf("autotune ok\n");
    return 0;
}
