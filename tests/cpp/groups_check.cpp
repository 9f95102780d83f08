// Host-side check of the sphere grouping (gbmp_groups.h): one group per sphere-carrying
// link with piece 0; with a piece size, every group holds spheres of one link, at most M
// of them, M the smallest size from the piece up that keeps the robot within the group
// limit; a link's pieces follow its longest extent and differ in size by at most one;
// groups come in link order; with no size that fits, one group per link.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "gbmp_groups.h"

#define CHECK(c)                                                    \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAILED %s at line %d\n", #c, __LINE__);    \
            std::exit(1);                                           \
        }                                                           \
    } while (0)

struct Robot {
    int L;
    std::vector<int> slink;
    std::vector<float> pos;
};

// spheres per link; centres spread along a per-link axis with jitter on the others
static Robot make(const std::vector<int> &per_link, unsigned seed) {
    Robot r{(int)per_link.size(), {}, {}};
    std::mt19937 g(seed);
    std::uniform_real_distribution<float> u(-0.01f, 0.01f);
    for (int l = 0; l < r.L; ++l)
        for (int k = 0; k < per_link[l]; ++k) {
            r.slink.push_back(l);
            const int ax = l % 3;
            for (int a = 0; a < 3; ++a) r.pos.push_back(a == ax ? 0.02f * (float)((k * 7) % per_link[l]) : u(g));
        }
    return r;
}

static void check_groups(const Robot &r, int piece, int max_groups, int expect_groups, int expect_m) {
    const int S = (int)r.slink.size();
    std::vector<int> glink, sgrp;
    gbmp::split_sphere_groups(r.L, S, r.slink.data(), r.pos.data(), piece, max_groups, glink, sgrp);
    const int G = (int)glink.size();
    CHECK(G == expect_groups);
    for (int g = 1; g < G; ++g) CHECK(glink[g] >= glink[g - 1]);   // link order
    std::vector<int> size(G, 0);
    for (int k = 0; k < S; ++k) {
        CHECK(sgrp[k] >= 0 && sgrp[k] < G);
        CHECK(glink[sgrp[k]] == r.slink[k]);   // a group holds spheres of one link
        size[sgrp[k]]++;
    }
    for (int g = 0; g < G; ++g) {
        CHECK(size[g] >= 1 && size[g] <= expect_m);
        // the pieces of one link differ in size by at most one
        if (g > 0 && glink[g] == glink[g - 1]) CHECK(size[g] - size[g - 1] <= 1 && size[g - 1] - size[g] <= 1);
    }
    // a link's pieces are consecutive along the longest extent of its centres
    for (int g = 1; g < G; ++g) {
        if (glink[g] != glink[g - 1]) continue;
        const int ax = glink[g] % 3;
        float hi_prev = -1e30f, lo_this = 1e30f;
        for (int k = 0; k < S; ++k) {
            if (sgrp[k] == g - 1) hi_prev = std::max(hi_prev, r.pos[3 * k + ax]);
            if (sgrp[k] == g) lo_this = std::min(lo_this, r.pos[3 * k + ax]);
        }
        CHECK(hi_prev <= lo_this);
    }
}

int main() {
    // the 8-DOF benchmark arm: 13-14 spheres on links 1..8, 9 links
    const Robot arm = make({0, 14, 14, 14, 14, 14, 14, 13, 13}, 1);
    check_groups(arm, 0, 0, 8, 14);    // one group per link
    check_groups(arm, 8, 27, 16, 7);   // pieces of 8 or fewer: two per link
    check_groups(arm, 4, 27, 24, 5);   // pieces of 4 would give 32 > 27 groups: size 5, three a link
    // 100 spheres on 4 links with room for 12 groups: pieces of 9 (three a link)
    check_groups(make({25, 25, 25, 25}, 2), 4, 12, 12, 9);
    // one heavy link among two: the smallest size within 6 groups is 17 (6 pieces of the 100)
    check_groups(make({0, 100}, 3), 1, 6, 6, 17);
    // 40 one-sphere links and a limit of 32: no piece size fits, one group per link
    check_groups(make(std::vector<int>(40, 1), 4), 8, 32, 40, 1);
    // no spheres
    {
        std::vector<int> glink, sgrp;
        gbmp::split_sphere_groups(3, 0, nullptr, nullptr, 8, 9, glink, sgrp);
        CHECK(glink.empty());
    }
    std::printf("groups ok\n");
    return 0;
}
