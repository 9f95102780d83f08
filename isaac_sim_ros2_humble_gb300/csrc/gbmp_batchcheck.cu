// gbmp_batchcheck.cu -- state checks of many (robot, scene) requests in one launch.
//
// The reference checks one space's states per call (SingleArmSpace::checkStates,
// SingleArmSpace.cu:1572-1602): requests of different robots or scenes are separate
// launches.  Here a descriptor table lists the requests (robot tables, scene, inputs,
// outputs), and a second table splits their states into block-sized ranges; every block
// stages the tables of its own request into shared memory (bulk asynchronous copies) and
// checks its range, one warp per state, with the per-state routine of k_check_states
// (check_state), so each request's outputs are bit-identical to a gbmp_check_states_fk
// call of its own.  Shared memory is sized for the largest request; the spheres-per-lane
// template covers the robot with the most spheres (smaller robots leave slots empty).
#include "gbmp_internal.h"

namespace gbmp {

struct CheckTask {
    DevRobot R;
    DevEnv E;
    const float *q;
    long long n;
    unsigned char *verdict;
    float *costs, *total, *poses, *centers;
};

struct CheckRange {
    int task, pad;
    long long lo, hi;
};

template <bool COST, int SPL>
__global__ void __launch_bounds__(kWarpsPerBlock *kWarp, 4)
    k_check_batch(const CheckTask *__restrict__ tasks, const CheckRange *__restrict__ ranges) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CheckTask sT;
    __shared__ CheckRange sB;
    if (threadIdx.x == 0) {
        sB = ranges[blockIdx.x];
        sT = tasks[sB.task];
    }
    __syncthreads();
    const DevRobot &R = sT.R;
    const DevEnv &E = sT.E;
    const int nwords = env_words(E.ns, E.nb, E.nc);
    SmemTables t = carve_tables(smem, R, nwords);
    if (!stage_tables(R, E, t, nwords)) return;
    WarpScratch w = carve_warp(smem + smem_tables_bytes(R, nwords), R, threadIdx.x / kWarp);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (long long s = sB.lo + threadIdx.x / kWarp; s < sB.hi; s += kWarpsPerBlock)
        check_state<COST, SPL>(t, R, E, w, sT.q, s, sT.n, sT.verdict, sT.costs, sT.total, sT.poses, sT.centers,
                               lane);
}

#define GBMP_BATCH_SPL_SWITCH(spl, ...)                    \
    switch (spl) {                                         \
    case 1: { constexpr int SPL = 1; __VA_ARGS__; } break; \
    case 2: { constexpr int SPL = 2; __VA_ARGS__; } break; \
    case 3: { constexpr int SPL = 3; __VA_ARGS__; } break; \
    case 4: { constexpr int SPL = 4; __VA_ARGS__; } break; \
    case 5: { constexpr int SPL = 5; __VA_ARGS__; } break; \
    case 6: { constexpr int SPL = 6; __VA_ARGS__; } break; \
    case 7: { constexpr int SPL = 7; __VA_ARGS__; } break; \
    default: { constexpr int SPL = 8; __VA_ARGS__; } break; \
    }

// Blocks per SM a launch may use: eight waves of the most blocks an SM can hold (eight
// of 256 threads), so that ranges of uneven requests even out across the SMs.
constexpr int kBatchBlocksPerSm = 64;

}  // namespace gbmp

using namespace gbmp;

struct gbmp_check_batch_s {
    int device = 0, num_sms = 0, max_requests = 0, max_ranges = 0;
    unsigned char *h_buf = nullptr;   // pinned: tasks, then ranges
    unsigned char *d_buf = nullptr;
    size_t ranges_off = 0, bytes = 0;
    cudaEvent_t uploaded = nullptr;   // the last upload from h_buf has been read
    bool pending = false;
};

extern "C" {

gbmp_status gbmp_check_batch_create(int32_t max_requests, gbmp_check_batch *out) {
    GBMP_CHECK_ARG(out, "out is NULL");
    GBMP_CHECK_ARG(max_requests >= 1 && max_requests <= (1 << 20), "max_requests %d outside [1, 2^20]",
                   max_requests);
    *out = nullptr;
    auto *b = new gbmp_check_batch_s();
    b->max_requests = max_requests;
    gbmp_status st = GBMP_OK;
    do {
        if (cudaGetDevice(&b->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess) {
            set_error("no CUDA device");
            st = GBMP_ERR_CUDA;
            break;
        }
        b->max_ranges = max_requests + kBatchBlocksPerSm * b->num_sms;
        b->ranges_off = align16(sizeof(CheckTask) * (size_t)max_requests);
        b->bytes = b->ranges_off + sizeof(CheckRange) * (size_t)b->max_ranges;
        if (cudaMallocHost(&b->h_buf, b->bytes) != cudaSuccess || cudaMalloc(&b->d_buf, b->bytes) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->uploaded, cudaEventDisableTiming) != cudaSuccess) {
            set_error("check batch: allocation of %zu bytes failed", b->bytes);
            st = GBMP_ERR_OUT_OF_MEMORY;
        }
    } while (false);
    if (st) {
        gbmp_check_batch_destroy(b);
        return st;
    }
    *out = b;
    return GBMP_OK;
}

gbmp_status gbmp_check_batch_destroy(gbmp_check_batch b) {
    if (!b) return GBMP_OK;
    if (b->uploaded) {
        cudaEventSynchronize(b->uploaded);
        cudaEventDestroy(b->uploaded);
    }
    if (b->h_buf) cudaFreeHost(b->h_buf);
    if (b->d_buf) cudaFree(b->d_buf);
    delete b;
    return GBMP_OK;
}

gbmp_status gbmp_check_batch_run(gbmp_check_batch b, const gbmp_check_request *reqs, int32_t n_reqs, int32_t mode,
                                 void *stream) {
    GBMP_CHECK_ARG(b, "batch is NULL");
    GBMP_CHECK_ARG(n_reqs >= 0 && n_reqs <= b->max_requests, "%d requests, the batch holds %d", n_reqs,
                   b->max_requests);
    GBMP_CHECK_ARG(n_reqs == 0 || reqs, "requests is NULL");
    GBMP_CHECK_ARG(mode == GBMP_CHECK_VERDICT || mode == GBMP_CHECK_COST, "unknown mode %d", mode);
    int dev = 0;
    GBMP_CUDA(cudaGetDevice(&dev));
    GBMP_CHECK_ARG(dev == b->device, "the batch was created on device %d, current device is %d", b->device, dev);
    for (int i = 0; i < n_reqs; ++i) {
        const gbmp_check_request &q = reqs[i];
        GBMP_CHECK_ARG(q.robot && q.env, "request %d: robot/env is NULL", i);
        GBMP_CHECK_ARG(q.n >= 0, "request %d: n < 0", i);
        GBMP_CHECK_ARG(q.n == 0 || q.d_q, "request %d: q is NULL", i);
        GBMP_CHECK_ARG(q.robot->device == dev, "request %d: robot on device %d", i, q.robot->device);
    }
    // the previous call's upload must have been read before the pinned tables change
    if (b->pending) {
        GBMP_CUDA(cudaEventSynchronize(b->uploaded));
        b->pending = false;
    }
    auto *tasks = reinterpret_cast<CheckTask *>(b->h_buf);
    auto *ranges = reinterpret_cast<CheckRange *>(b->h_buf + b->ranges_off);
    int nt = 0, spl = 1;
    size_t smem = 0;
    long long total = 0;
    unsigned long long *work = work_counter();
    for (int i = 0; i < n_reqs; ++i) {
        const gbmp_check_request &q = reqs[i];
        if (q.n == 0) continue;
        CheckTask &T = tasks[nt++];
        T.R = q.robot->dev;
        T.R.work = work;
        T.E = q.env->dev();
        T.q = q.d_q;
        T.n = q.n;
        T.verdict = q.d_verdict;
        T.costs = mode == GBMP_CHECK_COST ? q.d_costs : nullptr;
        T.total = mode == GBMP_CHECK_COST ? q.d_total : nullptr;
        T.poses = q.d_poses;
        T.centers = q.d_centers;
        spl = std::max(spl, T.R.spl);
        smem = std::max(smem, smem_tables_bytes(T.R, env_words(T.E.ns, T.E.nb, T.E.nc)) +
                                  smem_warp_bytes(T.R) * kWarpsPerBlock);
        total += q.n;
    }
    if (nt == 0) return GBMP_OK;
    // requests of one robot and scene next to each other, so that the blocks the GPU
    // schedules together share their tables (in L2) and their path through the routine
    // (measured 5.74 against 6.05 ms on the 256-request benchmark mix)
    std::stable_sort(tasks, tasks + nt, [](const CheckTask &x, const CheckTask &y) {
        if (x.R.stage != y.R.stage) return x.R.stage < y.R.stage;
        return x.E.words < y.E.words;
    });
    int optin = 0;
    GBMP_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem + 1024 > (size_t)optin) {
        set_error("check batch: the largest request needs %zu bytes of shared memory", smem);
        return GBMP_ERR_CAPACITY;
    }
    cudaStream_t s = (cudaStream_t)stream;
    gbmp_status st = GBMP_OK;
    const bool cost = mode == GBMP_CHECK_COST;
    GBMP_BATCH_SPL_SWITCH(spl, {
        const void *fn = cost ? (const void *)k_check_batch<true, SPL> : (const void *)k_check_batch<false, SPL>;
        st = ensure_smem_optin(fn);
        if (st) return st;
        int per_sm = 0;
        GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kWarpsPerBlock * kWarp, smem));
        if (per_sm < 1) per_sm = 1;
        // states per block: about eight waves over all requests (measured 6.03 ms against
        // 6.14 for four, 6.5 for two and 7.6 for one on the 256-request benchmark mix), at
        // least four states a warp
        const long long target = 8LL * per_sm * b->num_sms;
        long long spb = (total + target - 1) / target;
        spb = std::max<long long>(spb, 4 * kWarpsPerBlock);
        spb = (spb + kWarpsPerBlock - 1) / kWarpsPerBlock * kWarpsPerBlock;
        int nr = 0;
        for (int ti = 0; ti < nt; ++ti)
            for (long long lo = 0; lo < tasks[ti].n; lo += spb) {
                if (nr == b->max_ranges) {
                    set_error("check batch: more than %d block ranges", b->max_ranges);
                    return GBMP_ERR_CAPACITY;
                }
                ranges[nr++] = CheckRange{ti, 0, lo, std::min(lo + spb, tasks[ti].n)};
            }
        // tasks and ranges in one copy (the ranges follow the tasks at ranges_off)
        const size_t nbytes = b->ranges_off + sizeof(CheckRange) * (size_t)nr;
        if (b->ranges_off > sizeof(CheckTask) * (size_t)nt) {
            GBMP_CUDA(cudaMemcpyAsync(b->d_buf, b->h_buf, sizeof(CheckTask) * (size_t)nt, cudaMemcpyHostToDevice, s));
            GBMP_CUDA(cudaMemcpyAsync(b->d_buf + b->ranges_off, b->h_buf + b->ranges_off,
                                      sizeof(CheckRange) * (size_t)nr, cudaMemcpyHostToDevice, s));
        } else {
            GBMP_CUDA(cudaMemcpyAsync(b->d_buf, b->h_buf, nbytes, cudaMemcpyHostToDevice, s));
        }
        GBMP_CUDA(cudaEventRecord(b->uploaded, s));
        b->pending = true;
        const auto *d_tasks = reinterpret_cast<const CheckTask *>(b->d_buf);
        const auto *d_ranges = reinterpret_cast<const CheckRange *>(b->d_buf + b->ranges_off);
        ProfScope ps(GBMP_PROF_CHECK_STATES, s);
        if (cost)
            k_check_batch<true, SPL><<<nr, kWarpsPerBlock * kWarp, smem, s>>>(d_tasks, d_ranges);
        else
            k_check_batch<false, SPL><<<nr, kWarpsPerBlock * kWarp, smem, s>>>(d_tasks, d_ranges);
    });
    GBMP_CUDA(cudaGetLastError());
    return st;
}

}  // extern "C"
