// gbmp_internal.h -- host-side handle structures and helpers shared by the
// translation units of libgbmp.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbmp.h"
#include "gbmp_device.cuh"
#include "gbmp_devset.h"

namespace gbmp {

void set_error(const char *fmt, ...);

#define GBMP_CUDA(call)                                                                        \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            ::gbmp::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                              __LINE__);                                                       \
            return e_ == cudaErrorMemoryAllocation ? GBMP_ERR_OUT_OF_MEMORY : GBMP_ERR_CUDA;   \
        }                                                                                      \
    } while (0)

#define GBMP_CHECK_ARG(cond, ...)                 \
    do {                                          \
        if (!(cond)) {                            \
            ::gbmp::set_error(__VA_ARGS__);       \
            return GBMP_ERR_INVALID_ARGUMENT;     \
        }                                         \
    } while (0)

// Raises the dynamic shared-memory limit of kernel `fn` to 227 KB (with the largest
// shared-memory carveout) on the current device, once per (device, kernel).
gbmp_status ensure_smem_optin(const void *fn);

constexpr int kMaxSelfPairs = 65535 * 4;
constexpr int kMaxEnvWords = 12 * 1024;     // 192 KB of float4 staged in shared memory
constexpr int kWarpsPerBlock = 8;

// Growable device buffer owned by a handle.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    gbmp_status reserve(size_t n) {
        if (n <= bytes) return GBMP_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t want = n + n / 4 + 256;
        GBMP_CUDA(cudaMalloc(&ptr, want));
        bytes = want;
        return GBMP_OK;
    }
    ~DevBuf() {
        if (ptr) cudaFree(ptr);
    }
};

// Runtime-generated robot kernels (gbmp_codegen.cu).
struct Codegen {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t fk = nullptr, edge_setup = nullptr;
    std::string source, arch;
    unsigned long long hash = 0;
    int cache = 0;              // 0 compiled now, 1 in-process cache, 2 disk cache
    double compile_ms = 0.0;
};

// Instrumentation (gbmp_prof.cu).  A ProfScope around a launch counts it and, when
// profiling is on, records CUDA events on the launching stream around it.
constexpr int kProfFamilies = 4;
void count_launch(int n);
unsigned long long *work_counter();   // device [flops, states] or nullptr when counting is off
struct ProfScope {
    int fam;
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(int family, cudaStream_t stream);
    ~ProfScope();
    ProfScope(const ProfScope &) = delete;
    ProfScope &operator=(const ProfScope &) = delete;
};

// Batched planning in two halves (gbmp_rrtc.cu), used by the request server to hand
// results out as each problem of a launch ends: batch_begin queues the launch on `st`,
// batch_flag reads problem i's host-mapped completion word (0 running, path length + 1
// when solved, -status otherwise), batch_copy_path copies a finished problem's path
// while the launch continues, batch_end waits and fills every result.  The caller
// holds batch_mutex(b) from begin to end.
gbmp_status batch_begin(gbmp_batch_planner b, int n, const gbmp_rrtc_problem *problems, const gbmp_rrtc_settings *s,
                        int lanes_per_problem, int use_graph, cudaStream_t st);
int batch_flag(gbmp_batch_planner b, int i);
gbmp_status batch_copy_path(gbmp_batch_planner b, int i, int L, int len, float *h_path, cudaStream_t st);
gbmp_status batch_end(gbmp_batch_planner b, const gbmp_rrtc_problem *problems, gbmp_rrtc_result *results,
                      float *h_paths, cudaStream_t st);
std::mutex &batch_mutex(gbmp_batch_planner b);

}  // namespace gbmp

struct gbmp_robot_s {
    int L = 0, S = 0, P = 0, dim = 0;
    float resolution = 0.02f;
    int device = 0;
    int num_sms = 0;
    // host copies
    std::vector<int> type, parent, slink;
    std::vector<float> pose16, axis, sph_pos, sph_r, lower, upper, defv;
    std::vector<unsigned char> active, enables;
    std::vector<float> h_jl, h_axn, h_axr;   // host copies of the uploaded joint tables
    std::vector<int> pairs;          // 2*P
    std::vector<float> thr;          // P
    // device tables: sphere groups by link (dev, the per-state kernels) and by pieces of
    // links (dev_chunk, the chunk kernels); one allocation each
    void *d_block = nullptr, *d_block_chunk = nullptr;
    gbmp::DevRobot dev{}, dev_chunk{};
    // edge validation form: 0 automatic, 1 state by state, 4 or 10 states per chunk
    int edge_form = 0;
    // edge-check scratch
    std::mutex scratch_mu;
    gbmp::DevBuf scratch;
    gbmp::Codegen *cg = nullptr;
    bool use_cg = false;
};

namespace gbmp {
gbmp_status codegen_build(gbmp_robot_s *r);
void codegen_free(Codegen *cg);
gbmp_status codegen_fk(const gbmp_robot_s *r, const float *q, long long n, float *poses, float *centers,
                       cudaStream_t s);
gbmp_status codegen_edge_setup(const gbmp_robot_s *r, const float *from, const float *to, long long E, float res,
                               int rule, int *nsteps, float *dir, int *hist, float *length_out, int *nsteps_out,
                               cudaStream_t s);
// Edge validation by chunks of consecutive states (gbmp_chunk.cu).  K = states per
// chunk for this robot (0: use the per-state kernels); `form` is the robot handle's
// edge_form (0 automatic, 1 per state, 4 or 10 states per chunk).
int edge_chunk_states(const DevRobot &R, int form);
// FK alone of n states by chunks of consecutive states (robots of at most 16 links).
gbmp_status fk_chunk_launch(const DevRobot &R, int num_sms, const float *q, long long n, float *poses,
                            float *centers, cudaStream_t s);
gbmp_status edge_chunk_prepare(const DevRobot &R, const DevEnv &E, int num_sms, int K, size_t *smem, int *grid);
gbmp_status edge_chunk_launch(const DevRobot &R, const DevEnv &E, int K, int grid, size_t smem, cudaStream_t s,
                              const float *from, const float *to, const int *nsteps, const float *dir,
                              const int *order, long long n_edges, int *next, unsigned char *ok, int *first_hit);
}  // namespace gbmp

struct gbmp_env_s {
    int ns = 0, nb = 0, nc = 0;
    float4 *d_words = nullptr;
    std::vector<float4> h_words;
    gbmp::DevEnv dev() const {
        gbmp::DevEnv e;
        e.ns = ns; e.nb = nb; e.nc = nc;
        e.words = d_words;
        return e;
    }
};
