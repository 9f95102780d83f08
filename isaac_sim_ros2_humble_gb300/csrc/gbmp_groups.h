// gbmp_groups.h -- the sphere groups of a robot (host side, plain C++; tested on the CPU
// by tests/cpp/groups_check.cpp).
//
// A group is a set of spheres of one link with one bounding sphere; the kernels' broad
// phase and self-pair tests work on groups first.  With piece == 0 a group is all the
// spheres of one link.  Otherwise each link's spheres, ordered along the longest extent of
// their centres, are cut into ceil(n / M) pieces of consecutive spheres (sizes differing by
// at most one), M the smallest piece size from `piece` up that keeps the robot within
// max_groups groups; if none does, one group per link.  Groups come in link order.
#pragma once

#include <algorithm>
#include <vector>

namespace gbmp {

// slink [S]: link of each sphere (0 <= slink < L); pos [3 S]: sphere centres in their link
// frames.  Fills glink (link of each group) and sgrp [S] (group of each sphere).
inline void split_sphere_groups(int L, int S, const int *slink, const float *pos, int piece, int max_groups,
                                std::vector<int> &glink, std::vector<int> &sgrp) {
    glink.clear();
    sgrp.assign(S ? S : 1, 0);
    std::vector<std::vector<int>> by_link(L);
    for (int k = 0; k < S; ++k) by_link[slink[k]].push_back(k);
    int most = 1;
    for (int l = 0; l < L; ++l) most = std::max(most, (int)by_link[l].size());
    auto count = [&](int m) {
        int g = 0;
        for (int l = 0; l < L; ++l) g += ((int)by_link[l].size() + m - 1) / m;
        return g;
    };
    int M = most;
    if (piece > 0) {
        M = std::min(piece, most);
        while (M < most && count(M) > max_groups) ++M;
    }
    for (int l = 0; l < L; ++l) {
        std::vector<int> &ks = by_link[l];
        const int nl = (int)ks.size();
        if (nl == 0) continue;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int k : ks)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], (double)pos[3 * k + a]);
                hi[a] = std::max(hi[a], (double)pos[3 * k + a]);
            }
        int ax = 0;
        for (int a = 1; a < 3; ++a)
            if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
        std::stable_sort(ks.begin(), ks.end(), [&](int x, int y) { return pos[3 * x + ax] < pos[3 * y + ax]; });
        const int pieces = (nl + M - 1) / M;
        for (int q = 0; q < pieces; ++q) {
            const int g = (int)glink.size();
            glink.push_back(l);
            for (int i = (int)((long long)q * nl / pieces); i < (int)((long long)(q + 1) * nl / pieces); ++i)
                sgrp[ks[i]] = g;
        }
    }
}

}  // namespace gbmp
