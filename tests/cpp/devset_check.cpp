// Keying of the library's once-per-device kernel set-up record (gbmp_devset.h): the same
// kernel on two devices is two entries, so a host thread that configures a kernel on
// device 0 and then uses it on device 1 configures it there too.
#include <cstdio>
#include <thread>
#include <vector>

#include "gbmp_devset.h"

static void k_a() {}
static void k_b() {}

int main() {
    gbmp::DeviceKernelSet set;
    const void *a = (const void *)&k_a, *b = (const void *)&k_b;
    int fails = 0;
    auto expect = [&](bool c, const char *what) {
        if (!c) { std::printf("FAIL %s\n", what); ++fails; }
    };
    expect(!set.contains(0, a), "empty set");
    expect(set.insert(0, a), "first insert on device 0");
    expect(set.contains(0, a), "recorded on device 0");
    expect(!set.contains(1, a), "device 1 not configured by device 0");
    expect(!set.insert(0, a), "second insert on device 0 is not new");
    expect(set.insert(1, a), "same kernel on device 1 is new");
    expect(!set.contains(0, b), "other kernel not configured");
    // one thread per device inserting the same kernel: each device recorded once
    gbmp::DeviceKernelSet shared;
    std::vector<std::thread> th;
    std::vector<int> fresh(8, 0);
    for (int t = 0; t < 8; ++t)
        th.emplace_back([&, t] { fresh[t] = shared.insert(t % 4, b) ? 1 : 0; });
    for (auto &x : th) x.join();
    int n_fresh = 0;
    for (int v : fresh) n_fresh += v;
    expect(n_fresh == 4 && shared.size() == 4, "four devices, four entries");
    std::printf(fails ? "devset FAILED\n" : "devset ok\n");
    return fails ? 1 : 0;
}
