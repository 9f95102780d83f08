// gbmp_prof.cu -- instrumentation of libgbmp: per-family CUDA-event timing of kernel
// launches, a global launch counter, and the FP32 FMA throughput probe used as the
// CUDA-core roofline denominator.
#include <atomic>
#include <chrono>

#include "gbmp_internal.h"

namespace gbmp {

namespace {
struct ProfState {
    std::atomic<bool> on{false};
    std::mutex mu;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[kProfFamilies];
    std::vector<cudaEvent_t> pool;
    double ms[kProfFamilies] = {};
    long long launches[kProfFamilies] = {};
};
ProfState &prof() {
    static ProfState *p = new ProfState();   // leaked on purpose: destroyed after the CUDA runtime otherwise
    return *p;
}
std::atomic<long long> g_launches{0};

cudaEvent_t take_event(ProfState &p) {
    if (!p.pool.empty()) {
        cudaEvent_t e = p.pool.back();
        p.pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Wait for and fold in every pending event pair (caller holds the mutex).
void drain(ProfState &p) {
    for (int f = 0; f < kProfFamilies; ++f) {
        for (auto &pr : p.pending[f]) {
            float ms = 0.f;
            cudaEventSynchronize(pr.second);
            if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) p.ms[f] += ms;
            p.launches[f] += 1;
            p.pool.push_back(pr.first);
            p.pool.push_back(pr.second);
        }
        p.pending[f].clear();
    }
}
}  // namespace

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {
std::mutex g_work_mu;
unsigned long long *g_work = nullptr;   // [flops, states] on the device
std::atomic<bool> g_work_on{false};
}  // namespace

unsigned long long *work_counter() { return g_work_on.load() ? g_work : nullptr; }

ProfScope::ProfScope(int family, cudaStream_t stream) : fam(family), s(stream) {
    count_launch(1);
    ProfState &p = prof();
    if (!p.on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lock(p.mu);
    a = take_event(p);
    b = take_event(p);
    if (a && b) cudaEventRecord(a, s);
}

ProfScope::~ProfScope() {
    if (!a || !b) return;
    ProfState &p = prof();
    cudaEventRecord(b, s);
    std::lock_guard<std::mutex> lock(p.mu);
    p.pending[fam].push_back({a, b});
}

// Register-resident FMA chains: 8 independent accumulators per thread.
__global__ void __launch_bounds__(512) k_fma_probe(float *out, int iters, float seed) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + 1e-7f * (threadIdx.x + 37 * k);
    const float m = 0.9999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = __fmaf_rn(a[k], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 1234.5f) out[blockIdx.x] = s;
}

}  // namespace gbmp

using namespace gbmp;

extern "C" {

gbmp_status gbmp_profile_enable(int32_t enable) {
    prof().on.store(enable != 0);
    return GBMP_OK;
}

gbmp_status gbmp_profile_reset(void) {
    ProfState &p = prof();
    std::lock_guard<std::mutex> lock(p.mu);
    drain(p);
    for (int f = 0; f < kProfFamilies; ++f) {
        p.ms[f] = 0.0;
        p.launches[f] = 0;
    }
    return GBMP_OK;
}

gbmp_status gbmp_profile_read(int32_t family, double *ms, int64_t *launches) {
    GBMP_CHECK_ARG(family >= 0 && family < kProfFamilies, "unknown family %d", family);
    ProfState &p = prof();
    std::lock_guard<std::mutex> lock(p.mu);
    drain(p);
    if (ms) *ms = p.ms[family];
    if (launches) *launches = p.launches[family];
    return GBMP_OK;
}

gbmp_status gbmp_work_counting(int32_t enable) {
    std::lock_guard<std::mutex> lock(g_work_mu);
    if (enable) {
        if (!g_work) GBMP_CUDA(cudaMalloc(&g_work, 2 * sizeof(unsigned long long)));
        GBMP_CUDA(cudaMemset(g_work, 0, 2 * sizeof(unsigned long long)));
    }
    g_work_on.store(enable != 0);
    return GBMP_OK;
}

gbmp_status gbmp_work_read(uint64_t *flops, uint64_t *states) {
    std::lock_guard<std::mutex> lock(g_work_mu);
    unsigned long long h[2] = {0ull, 0ull};
    if (g_work) GBMP_CUDA(cudaMemcpy(h, g_work, sizeof h, cudaMemcpyDeviceToHost));
    if (flops) *flops = h[0];
    if (states) *states = h[1];
    return GBMP_OK;
}

gbmp_status gbmp_launch_count(int64_t *count) {
    GBMP_CHECK_ARG(count, "count is NULL");
    *count = g_launches.load();
    return GBMP_OK;
}

gbmp_status gbmp_measure_fp32_peak(double seconds, double *tflops) {
    GBMP_CHECK_ARG(tflops, "tflops is NULL");
    int dev = 0, sms = 0;
    GBMP_CUDA(cudaGetDevice(&dev));
    GBMP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    float *out = nullptr;
    const int threads = 512, blocks = sms * 4;
    GBMP_CUDA(cudaMalloc(&out, sizeof(float) * blocks));
    cudaEvent_t a, b;
    GBMP_CUDA(cudaEventCreate(&a));
    GBMP_CUDA(cudaEventCreate(&b));
    int iters = 1 << 14;
    double best = 0.0;
    auto t0 = std::chrono::steady_clock::now();
    for (int rep = 0; rep < 1000; ++rep) {
        cudaEventRecord(a);
        k_fma_probe<<<blocks, threads>>>(out, iters, 1.0f + rep * 1e-6f);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double fl = 2.0 * 8.0 * (double)iters * threads * blocks;
        if (ms > 0.f) best = std::max(best, fl / (ms * 1e-3) / 1e12);
        if (ms < 20.f && iters < (1 << 24)) iters *= 2;
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > seconds && rep >= 3) break;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) {
        set_error("fp32 probe failed: %s", cudaGetErrorString(e));
        return GBMP_ERR_CUDA;
    }
    *tflops = best;
    return GBMP_OK;
}

}  // extern "C"
