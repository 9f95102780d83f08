// Host-side check of the edge state orders (gbmp_order.h): for every edge length up to
// 6,000 states, both chunk sizes and both orders, the chunks cover every state exactly
// once; the state order walks the edge from its start; the coarse-to-fine order takes the
// first 4 states, then the last chunk, then the chunks between pass by pass in
// bit-reversed offset order; the state-by-state coarse-to-fine order is a permutation
// starting with the first and last states; indices past the end give empty answers.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbmp_order.h"

#define CHECK(c)                                                                   \
    do {                                                                           \
        if (!(c)) {                                                                \
            std::printf("FAILED %s at line %d (n=%d)\n", #c, __LINE__, n_now);      \
            std::exit(1);                                                          \
        }                                                                          \
    } while (0)

static int n_now = 0;

int main() {
    using namespace gbmp;
    CHECK(order_pass_offset(0) == 0 && order_pass_offset(1) == 8 && order_pass_offset(2) == 4 &&
          order_pass_offset(3) == 12 && order_pass_offset(15) == 15);
    for (int K : {4, 10}) {
        for (int any = 0; any < 2; ++any) {
            for (int n = 1; n <= 6000; ++n) {
                n_now = n;
                std::vector<int> seen(n, 0);
                const int nch = edge_chunk_count(n, K, any != 0);
                int prev_end = 0;
                for (int c = 0; c < nch; ++c) {
                    const StateRange r = edge_chunk_range(c, n, K, any != 0);
                    CHECK(0 <= r.x && r.x < r.y && r.y <= n);
                    CHECK(r.y - r.x <= (c == 0 ? kFirstChunk : K));
                    for (int s = r.x; s < r.y; ++s) seen[s]++;
                    if (!any) {
                        CHECK(r.x == prev_end);   // state order: consecutive chunks
                        prev_end = r.y;
                    }
                }
                for (int s = 0; s < n; ++s) CHECK(seen[s] == 1);
                const StateRange past = edge_chunk_range(nch, n, K, any != 0);
                CHECK(past.x >= past.y);   // empty
                if (any && n > kFirstChunk) {
                    const StateRange first = edge_chunk_range(0, n, K, true);
                    const StateRange last = edge_chunk_range(1, n, K, true);
                    CHECK(first.x == 0 && first.y == kFirstChunk);
                    CHECK(last.y == n && (last.x == n - K || last.x == kFirstChunk));
                    // the chunks between, pass by pass
                    const int ts = last.x, nm = (ts - kFirstChunk + K - 1) / K;
                    int idx = 2;
                    for (int p = 0; p < kOrderPasses; ++p)
                        for (int j = order_pass_offset(p); j < nm; j += kOrderPasses, ++idx) {
                            const StateRange r = edge_chunk_range(idx, n, K, true);
                            CHECK(r.x == kFirstChunk + j * K);
                        }
                    CHECK(idx == nch);
                }
            }
        }
    }
    for (int n = 1; n <= 6000; ++n) {
        n_now = n;
        std::vector<int> seen(n, 0);
        for (int c = 0; c < n; ++c) {
            const int s = verdict_order_state(c, n);
            CHECK(0 <= s && s < n);
            seen[s]++;
        }
        for (int s = 0; s < n; ++s) CHECK(seen[s] == 1);
        CHECK(verdict_order_state(0, n) == 0);
        if (n >= 2) CHECK(verdict_order_state(1, n) == n - 1);
        if (n >= 3) CHECK(verdict_order_state(2, n) == 1);   // pass 0 starts at offset 0
        CHECK(verdict_order_state(n, n) == 0 || n <= 2);
    }
    std::printf("order ok\n");
    return 0;
}
