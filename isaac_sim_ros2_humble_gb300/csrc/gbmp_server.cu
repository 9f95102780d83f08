// gbmp_server.cu -- continuous-batching request server over resident robots,
// environments and planner trees.  The reference has no serving layer; callers of
// the reference run checkStates / solve one request at a time on the default stream
// (cudampl/CUDAMPLib/src/spaces/SingleArmSpace.cu:1572-1602,
// cudampl/CPRRTC/src/RobotSolver.cu:348-473).
//
// Design
//  * Robots and environments are registered once and stay resident.
//  * FK+collision requests go to the check queue.  A scheduler thread repeatedly
//    takes every pending check request that fits the HBM budget and the batch cap,
//    groups them by (robot, environment), packs their joint states into one pinned
//    staging buffer, and issues per group one H2D copy, one gbmp_check_states launch
//    and one D2H copy on the next of `num_streams` streams.  Batches on different
//    streams overlap on the device; a completion thread waits for each batch's event,
//    scatters verdicts to the requests and returns the budget, so requests that arrive
//    while others run are admitted as soon as memory frees up.
//  * Plan requests go to the plan queue; `plan_workers` threads each own a batch
//    planner (device-resident trees) and solve everything pending in one batched,
//    graph-captured launch, so plan batches overlap with check batches and with each
//    other.
//  * Every request records submit, start and finish times; the server keeps latency
//    percentiles.
#include <algorithm>
#include <climits>
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <thread>

#include "gbmp_internal.h"

using gbmp::align16;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    int kind = 0;                     // 0 check, 1 plan
    int robot = 0, env = 0;
    const float *q = nullptr;         // check: host [n * L]
    int64_t n = 0;
    uint8_t *verdict = nullptr;       // check: host [n]
    const float *start = nullptr, *goal = nullptr;
    uint64_t seed = 0;
    float *path = nullptr;
    int32_t path_cap = 0;
    size_t bytes = 0;                 // device bytes reserved while in flight
    Clock::time_point t_submit, t_start, t_done;
    gbmp_status status = GBMP_OK;
    int32_t solved = 0, path_len = 0;
    float cost = 0.f;
    bool done = false;
};

// A batch slot: stream, completion event and staging buffers allocated once at start,
// so that nothing in the request path allocates or frees device or pinned memory
// (cudaFree and cudaFreeHost synchronise with the whole device and would serialise
// the check batches behind running plan batches).
struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    float *d_q = nullptr, *h_q = nullptr;   // [cap_states * max_L]
    uint8_t *d_v = nullptr, *h_v = nullptr; // [cap_states]
    gbmp_check_batch cb = nullptr;          // one launch for all (robot, scene) groups
};

struct Batch {
    std::vector<std::shared_ptr<Request>> reqs;
    int slot = -1;
    size_t bytes = 0;
};

}  // namespace

struct gbmp_server_s {
    gbmp_server_config cfg{};
    std::vector<gbmp_robot> robots;
    std::vector<gbmp_env> envs;
    std::vector<cudaStream_t> streams;
    std::vector<Slot> slots;
    std::vector<int> free_slots;
    int64_t cap_states = 0;                 // states per slot
    int max_L = 0;
    int device = 0;
    int num_sms = 152;

    std::mutex mu;
    std::condition_variable cv_sched, cv_done, cv_plan, cv_complete;
    std::deque<std::shared_ptr<Request>> check_q, plan_q;
    std::deque<Batch> in_flight;
    std::map<int64_t, std::shared_ptr<Request>> tickets;
    int64_t next_id = 1;
    size_t budget_used = 0;
    bool stop = false;
    gbmp_status fatal = GBMP_OK;

    std::vector<double> lat_check, lat_plan;    // ms
    int64_t completed = 0, batches = 0, plan_batches = 0, states_checked = 0;
    Clock::time_point t0 = Clock::now();

    std::thread sched, completer;
    std::vector<std::thread> planners;
};

namespace {

void finish_request(gbmp_server_s *s, const std::shared_ptr<Request> &r) {
    r->t_done = Clock::now();
    r->done = true;
    const double ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    (r->kind == 0 ? s->lat_check : s->lat_plan).push_back(ms);
    ++s->completed;
}

// Scheduler: forms check batches from everything pending that fits a free slot and
// the budget, then stages, launches and hands the batch to the completion thread.
void scheduler_loop(gbmp_server_s *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_sched.wait(lk, [&] {
            return s->stop || (!s->check_q.empty() && !s->free_slots.empty() && s->fatal == GBMP_OK);
        });
        if (s->stop) return;
        std::vector<std::shared_ptr<Request>> take;
        size_t bytes = 0;
        int64_t states = 0;
        while (!s->check_q.empty()) {
            auto &r = s->check_q.front();
            if (r->n > s->cap_states) {
                // larger than a slot (the budget split over the streams): never admissible
                r->status = GBMP_ERR_CAPACITY;
                finish_request(s, r);
                s->check_q.pop_front();
                s->cv_complete.notify_all();
                continue;
            }
            if (states + r->n > s->cap_states) break;
            if (s->budget_used + bytes + r->bytes > (size_t)s->cfg.hbm_budget_bytes) break;
            bytes += r->bytes;
            states += r->n;
            take.push_back(r);
            s->check_q.pop_front();
        }
        if (take.empty()) continue;
        s->budget_used += bytes;
        const int si = s->free_slots.back();
        s->free_slots.pop_back();
        lk.unlock();

        Slot &sl = s->slots[si];
        Batch b;
        b.reqs = take;
        b.slot = si;
        b.bytes = bytes;
        const auto now = Clock::now();
        for (auto &r : take) r->t_start = now;
        // group by (robot, env): requests of a group become adjacent, one task per group,
        // all groups in one batched launch
        std::stable_sort(b.reqs.begin(), b.reqs.end(), [](const std::shared_ptr<Request> &a,
                                                          const std::shared_ptr<Request> &c) {
            return a->robot != c->robot ? a->robot < c->robot : a->env < c->env;
        });
        size_t qfloats = 0, vbytes = 0;
        for (auto &r : b.reqs) {
            memcpy(sl.h_q + qfloats, r->q, sizeof(float) * (size_t)r->n * s->robots[r->robot]->L);
            qfloats += (size_t)r->n * s->robots[r->robot]->L;
            vbytes += (size_t)r->n;
        }
        gbmp_status st = GBMP_OK;
        if (cudaMemcpyAsync(sl.d_q, sl.h_q, sizeof(float) * qfloats, cudaMemcpyHostToDevice, sl.stream) != cudaSuccess)
            st = GBMP_ERR_CUDA;
        size_t qoff = 0, voff = 0;
        std::vector<gbmp_check_request> tasks;
        for (size_t i = 0; i < b.reqs.size();) {
            const size_t q0 = qoff, v0 = voff;
            int64_t n = 0;
            size_t j = i;
            while (j < b.reqs.size() && b.reqs[j]->robot == b.reqs[i]->robot && b.reqs[j]->env == b.reqs[i]->env) {
                n += b.reqs[j]->n;
                qoff += (size_t)b.reqs[j]->n * s->robots[b.reqs[j]->robot]->L;
                voff += (size_t)b.reqs[j]->n;
                ++j;
            }
            gbmp_check_request t{};
            t.robot = s->robots[b.reqs[i]->robot];
            t.env = s->envs[b.reqs[i]->env];
            t.d_q = sl.d_q + q0;
            t.n = n;
            t.d_verdict = sl.d_v + v0;
            tasks.push_back(t);
            i = j;
        }
        if (st == GBMP_OK)
            st = gbmp_check_batch_run(sl.cb, tasks.data(), (int32_t)tasks.size(), GBMP_CHECK_VERDICT, sl.stream);
        if (st == GBMP_OK &&
            (cudaMemcpyAsync(sl.h_v, sl.d_v, vbytes, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess ||
             cudaEventRecord(sl.done, sl.stream) != cudaSuccess))
            st = GBMP_ERR_CUDA;
        lk.lock();
        if (st != GBMP_OK) {
            for (auto &r : b.reqs) {
                r->status = st;
                finish_request(s, r);
            }
            s->budget_used -= bytes;
            s->free_slots.push_back(si);
            s->cv_complete.notify_all();
            continue;
        }
        s->states_checked += states;
        ++s->batches;
        s->in_flight.push_back(b);
        s->cv_done.notify_one();
    }
}

// Completion: waits for batches in issue order, scatters verdicts, frees the slot
// and the budget.
void completion_loop(gbmp_server_s *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_done.wait(lk, [&] { return s->stop || !s->in_flight.empty(); });
        if (s->in_flight.empty() && s->stop) return;
        Batch b = s->in_flight.front();
        s->in_flight.pop_front();
        lk.unlock();
        Slot &sl = s->slots[b.slot];
        const cudaError_t ce = cudaEventSynchronize(sl.done);
        size_t voff = 0;
        for (auto &r : b.reqs) {
            if (ce == cudaSuccess) memcpy(r->verdict, sl.h_v + voff, (size_t)r->n);
            voff += (size_t)r->n;
        }
        lk.lock();
        for (auto &r : b.reqs) {
            r->status = ce == cudaSuccess ? GBMP_OK : GBMP_ERR_CUDA;
            finish_request(s, r);
        }
        s->budget_used -= b.bytes;
        s->free_slots.push_back(b.slot);
        s->cv_sched.notify_all();
        s->cv_complete.notify_all();
    }
}

// Plan worker: solves everything pending in one batched launch and hands each result
// out as soon as its problem ends (host-mapped completion words), while the launch
// continues for the others.
void plan_loop(gbmp_server_s *s, int worker) {
    cudaSetDevice(s->device);
    gbmp_batch_planner bp = nullptr;
    cudaStream_t st = nullptr, cst = nullptr;
    int max_links = 1;
    for (auto r : s->robots) max_links = std::max(max_links, r->L);
    gbmp_status cs = gbmp_batch_planner_create(s->cfg.plan_batch, s->cfg.planner_max_nodes, max_links,
                                               s->cfg.plan_path_cap, &bp);
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (cs == GBMP_OK && (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lo_prio) != cudaSuccess ||
                          cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking) != cudaSuccess))
        cs = GBMP_ERR_CUDA;
    std::unique_lock<std::mutex> lk(s->mu);
    if (cs != GBMP_OK) s->fatal = cs;
    (void)worker;
    auto path_cost = [&](const std::shared_ptr<Request> &r, int len) {
        const gbmp_robot rb = s->robots[r->robot];
        double c = 0.0;
        for (int k = 1; k < len; ++k) {
            double s2 = 0.0;
            for (int j = 0; j < rb->L; ++j)
                if (rb->active[j]) {
                    const double d = (double)r->path[k * rb->L + j] - r->path[(k - 1) * rb->L + j];
                    s2 += d * d;
                }
            c += std::sqrt(s2);
        }
        return (float)c;
    };
    while (true) {
        s->cv_plan.wait(lk, [&] { return s->stop || !s->plan_q.empty(); });
        if (s->stop) break;
        std::vector<std::shared_ptr<Request>> take;
        while (!s->plan_q.empty() && (int)take.size() < s->cfg.plan_batch) {
            take.push_back(s->plan_q.front());
            s->plan_q.pop_front();
        }
        ++s->plan_batches;
        lk.unlock();
        const int n = (int)take.size();
        const auto now = Clock::now();
        std::vector<gbmp_rrtc_problem> probs(n);
        for (int i = 0; i < n; ++i) {
            take[i]->t_start = now;
            probs[i] = {s->robots[take[i]->robot], s->envs[take[i]->env], take[i]->start, take[i]->goal, take[i]->seed};
        }
        gbmp_rrtc_settings set{};
        set.lanes = s->cfg.plan_lanes;
        set.max_iters = s->cfg.plan_max_iters;
        set.range = s->cfg.plan_range;
        set.resolution = s->cfg.plan_resolution;
        set.step_rule = s->cfg.step_rule;
        set.time_limit_s = s->cfg.plan_time_limit_s;
        std::vector<char> done(n, 0);
        // small batches get more lanes per problem (up to 1024 blocks per launch), large
        // ones at least plan_lanes; with plan_max_blocks the launch's blocks stay within it so
        // that check batches find room on every SM (persistent plan blocks hold their SMs)
        const int cap = s->cfg.plan_max_blocks > 0 ? s->cfg.plan_max_blocks : INT_MAX;
        const int lpp = std::max(1, std::min(std::max(s->cfg.plan_lanes, std::min(1024, 1024 / n)), cap / n));
        gbmp_status ps = cs != GBMP_OK ? cs : gbmp::batch_begin(bp, n, probs.data(), &set, lpp, 0, st);
        // hand out results as problems end
        auto deliver = [&](int i, int flag) {
            auto &r = take[i];
            if (flag > 0) {
                const int len = flag - 1;
                if (len > r->path_cap || !r->path) {
                    r->status = GBMP_ERR_CAPACITY;
                    r->path_len = len;
                } else {
                    r->status = gbmp::batch_copy_path(bp, i, s->robots[r->robot]->L, len, r->path, cst);
                    r->solved = r->status == GBMP_OK;
                    r->path_len = len;
                    r->cost = path_cost(r, len);
                }
            } else {
                r->status = flag == -4 ? GBMP_ERR_TIMEOUT : (flag == -5 ? GBMP_ERR_CAPACITY : GBMP_ERR_NOT_SOLVED);
            }
            std::lock_guard<std::mutex> g(s->mu);
            finish_request(s, r);
            s->cv_complete.notify_all();
        };
        if (ps == GBMP_OK) {
            int left = n;
            while (left > 0) {
                for (int i = 0; i < n; ++i)
                    if (!done[i]) {
                        const int f = gbmp::batch_flag(bp, i);
                        if (f != 0) {
                            done[i] = 1;
                            --left;
                            deliver(i, f);
                        }
                    }
                if (left == 0 || cudaStreamQuery(st) != cudaErrorNotReady) break;
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            }
            std::vector<gbmp_rrtc_result> res(n);
            ps = gbmp::batch_end(bp, probs.data(), res.data(), nullptr, st);
            for (int i = 0; i < n; ++i) {
                if (done[i]) continue;
                done[i] = 1;
                if (ps == GBMP_OK && res[i].solved) deliver(i, res[i].path_len + 1);
                else if (ps == GBMP_OK) deliver(i, -res[i].status);
                else {
                    take[i]->status = ps;
                    std::lock_guard<std::mutex> g(s->mu);
                    finish_request(s, take[i]);
                    s->cv_complete.notify_all();
                }
            }
        } else {
            std::lock_guard<std::mutex> g(s->mu);
            for (auto &r : take) {
                r->status = ps;
                finish_request(s, r);
            }
            s->cv_complete.notify_all();
        }
        lk.lock();
    }
    lk.unlock();
    if (bp) gbmp_batch_planner_destroy(bp);
    if (st) cudaStreamDestroy(st);
    if (cst) cudaStreamDestroy(cst);
}

double pct(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double idx = p / 100.0 * (v.size() - 1);
    const size_t lo = (size_t)idx, hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (idx - lo) * (v[hi] - v[lo]);
}

}  // namespace

using namespace gbmp;

extern "C" {

gbmp_status gbmp_server_create(const gbmp_server_config *cfg, gbmp_server *out) {
    GBMP_CHECK_ARG(cfg && out, "NULL argument");
    *out = nullptr;
    GBMP_CHECK_ARG(cfg->num_streams >= 1 && cfg->num_streams <= 64, "num_streams outside [1, 64]");
    GBMP_CHECK_ARG(cfg->hbm_budget_bytes > 0, "hbm_budget_bytes <= 0");
    GBMP_CHECK_ARG(cfg->max_batch_states >= 1, "max_batch_states < 1");
    GBMP_CHECK_ARG(cfg->plan_workers >= 0 && cfg->plan_workers <= 16, "plan_workers outside [0, 16]");
    GBMP_CHECK_ARG(cfg->plan_workers == 0 || (cfg->plan_batch >= 1 && cfg->planner_max_nodes >= 2 &&
                                              cfg->plan_lanes >= 1 && cfg->plan_path_cap >= 2 &&
                                              cfg->plan_range > 0.f && cfg->plan_max_iters >= 1),
                   "bad planner configuration");
    GBMP_CHECK_ARG(cfg->plan_max_blocks >= 0, "plan_max_blocks < 0");
    auto *s = new gbmp_server_s();
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device);
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    for (int i = 0; i < cfg->num_streams; ++i) {
        cudaStream_t st;
        // check batches are short: give them the highest priority so their blocks are
        // scheduled ahead of the long planning launches
        if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, hi_prio) != cudaSuccess) {
            set_error("stream creation failed");
            gbmp_server_destroy(s);
            return GBMP_ERR_CUDA;
        }
        s->streams.push_back(st);
    }
    *out = s;
    return GBMP_OK;
}

gbmp_status gbmp_server_add_robot(gbmp_server s, gbmp_robot r, int32_t *id) {
    GBMP_CHECK_ARG(s && r && id, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    GBMP_CHECK_ARG(!s->sched.joinable(), "resources must be registered before gbmp_server_start");
    s->robots.push_back(r);
    *id = (int32_t)s->robots.size() - 1;
    return GBMP_OK;
}

gbmp_status gbmp_server_add_env(gbmp_server s, gbmp_env e, int32_t *id) {
    GBMP_CHECK_ARG(s && e && id, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    GBMP_CHECK_ARG(!s->sched.joinable(), "resources must be registered before gbmp_server_start");
    s->envs.push_back(e);
    *id = (int32_t)s->envs.size() - 1;
    return GBMP_OK;
}

gbmp_status gbmp_server_start(gbmp_server s) {
    GBMP_CHECK_ARG(s, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    GBMP_CHECK_ARG(!s->sched.joinable(), "server already started");
    GBMP_CHECK_ARG(!s->robots.empty() && !s->envs.empty(), "register robots and environments first");
    s->max_L = 1;
    for (auto r : s->robots) s->max_L = std::max(s->max_L, r->L);
    const int64_t per_state = 4LL * s->max_L + 1;
    s->cap_states = std::min<int64_t>(s->cfg.max_batch_states,
                                      s->cfg.hbm_budget_bytes / ((int64_t)s->streams.size() * per_state));
    GBMP_CHECK_ARG(s->cap_states >= 1, "hbm_budget_bytes too small for one state per stream");
    // a batch holds at most one task per (robot, scene) group
    const int64_t groups64 = (int64_t)s->robots.size() * (int64_t)s->envs.size();
    GBMP_CHECK_ARG(groups64 <= (1 << 20), "%lld (robot, scene) groups, at most 2^20", (long long)groups64);
    const int32_t groups = (int32_t)groups64;
    for (size_t i = 0; i < s->streams.size(); ++i) {
        Slot sl;
        sl.stream = s->streams[i];
        const size_t qb = align16(sizeof(float) * (size_t)s->cap_states * s->max_L);
        cudaError_t ce = cudaMalloc(&sl.d_q, qb + align16((size_t)s->cap_states));
        if (ce == cudaSuccess) ce = cudaMallocHost(&sl.h_q, qb + align16((size_t)s->cap_states));
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        gbmp_status bs = GBMP_OK;
        if (ce == cudaSuccess) bs = gbmp_check_batch_create(groups, &sl.cb);
        if (ce != cudaSuccess || bs != GBMP_OK) {
            if (sl.d_q) cudaFree(sl.d_q);
            if (sl.h_q) cudaFreeHost(sl.h_q);
            if (sl.done) cudaEventDestroy(sl.done);
            if (ce != cudaSuccess) set_error("server slot allocation failed: %s", cudaGetErrorString(ce));
            return ce == cudaErrorMemoryAllocation ? GBMP_ERR_OUT_OF_MEMORY : (ce != cudaSuccess ? GBMP_ERR_CUDA : bs);
        }
        sl.d_v = reinterpret_cast<uint8_t *>(sl.d_q) + qb;
        sl.h_v = reinterpret_cast<uint8_t *>(sl.h_q) + qb;
        s->slots.push_back(sl);
        s->free_slots.push_back((int)i);
    }
    s->t0 = Clock::now();
    s->sched = std::thread(scheduler_loop, s);
    s->completer = std::thread(completion_loop, s);
    for (int i = 0; i < s->cfg.plan_workers; ++i) s->planners.emplace_back(plan_loop, s, i);
    return GBMP_OK;
}

gbmp_status gbmp_server_submit_check(gbmp_server s, int32_t robot, int32_t env, const float *h_q, int64_t n,
                                     uint8_t *h_verdict, int64_t *ticket) {
    GBMP_CHECK_ARG(s && h_q && h_verdict && ticket, "NULL argument");
    GBMP_CHECK_ARG(n >= 1, "n < 1");
    std::lock_guard<std::mutex> lk(s->mu);
    GBMP_CHECK_ARG(robot >= 0 && robot < (int)s->robots.size(), "unknown robot %d", robot);
    GBMP_CHECK_ARG(env >= 0 && env < (int)s->envs.size(), "unknown environment %d", env);
    GBMP_CHECK_ARG(s->sched.joinable() && !s->stop, "server not running");
    auto r = std::make_shared<Request>();
    r->id = s->next_id++;
    r->kind = 0;
    r->robot = robot;
    r->env = env;
    r->q = h_q;
    r->n = n;
    r->verdict = h_verdict;
    r->bytes = align16(sizeof(float) * n * s->robots[robot]->L) + align16((size_t)n);
    r->t_submit = Clock::now();
    s->tickets[r->id] = r;
    s->check_q.push_back(r);
    *ticket = r->id;
    s->cv_sched.notify_one();
    return GBMP_OK;
}

gbmp_status gbmp_server_submit_plan(gbmp_server s, int32_t robot, int32_t env, const float *h_start,
                                    const float *h_goal, uint64_t seed, float *h_path, int32_t path_cap,
                                    int64_t *ticket) {
    GBMP_CHECK_ARG(s && h_start && h_goal && ticket, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    GBMP_CHECK_ARG(s->cfg.plan_workers > 0, "server has no plan workers");
    GBMP_CHECK_ARG(robot >= 0 && robot < (int)s->robots.size(), "unknown robot %d", robot);
    GBMP_CHECK_ARG(env >= 0 && env < (int)s->envs.size(), "unknown environment %d", env);
    GBMP_CHECK_ARG(s->sched.joinable() && !s->stop, "server not running");
    auto r = std::make_shared<Request>();
    r->id = s->next_id++;
    r->kind = 1;
    r->robot = robot;
    r->env = env;
    r->start = h_start;
    r->goal = h_goal;
    r->seed = seed;
    r->path = h_path;
    r->path_cap = path_cap;
    r->t_submit = Clock::now();
    s->tickets[r->id] = r;
    s->plan_q.push_back(r);
    *ticket = r->id;
    s->cv_plan.notify_one();
    return GBMP_OK;
}

gbmp_status gbmp_server_wait(gbmp_server s, int64_t ticket, double timeout_s, gbmp_request_info *info) {
    GBMP_CHECK_ARG(s, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    GBMP_CHECK_ARG(it != s->tickets.end(), "unknown ticket %lld", (long long)ticket);
    auto r = it->second;
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9);
    if (!s->cv_complete.wait_until(lk, deadline, [&] { return r->done; })) {
        set_error("request %lld not finished within %.3f s", (long long)ticket, timeout_s);
        return GBMP_ERR_TIMEOUT;
    }
    if (info) {
        info->status = r->status;
        info->solved = r->solved;
        info->path_len = r->path_len;
        info->cost = r->cost;
        info->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        info->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    }
    s->tickets.erase(it);
    return GBMP_OK;
}

gbmp_status gbmp_server_stats(gbmp_server s, gbmp_server_metrics *out) {
    GBMP_CHECK_ARG(s && out, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof *out);
    out->completed = s->completed;
    out->batches = s->batches;
    out->plan_batches = s->plan_batches;
    out->states_checked = s->states_checked;
    out->check_p50_ms = pct(s->lat_check, 50);
    out->check_p95_ms = pct(s->lat_check, 95);
    out->check_p99_ms = pct(s->lat_check, 99);
    out->plan_p50_ms = pct(s->lat_plan, 50);
    out->plan_p95_ms = pct(s->lat_plan, 95);
    out->plan_p99_ms = pct(s->lat_plan, 99);
    out->elapsed_s = std::chrono::duration<double>(Clock::now() - s->t0).count();
    out->budget_in_use = (int64_t)s->budget_used;
    return GBMP_OK;
}

gbmp_status gbmp_server_destroy(gbmp_server s) {
    if (!s) return GBMP_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_sched.notify_all();
    s->cv_done.notify_all();
    s->cv_plan.notify_all();
    if (s->sched.joinable()) s->sched.join();
    if (s->completer.joinable()) s->completer.join();
    for (auto &t : s->planners) t.join();
    for (auto &sl : s->slots) {
        cudaEventSynchronize(sl.done);
        cudaEventDestroy(sl.done);
        gbmp_check_batch_destroy(sl.cb);
        cudaFree(sl.d_q);
        cudaFreeHost(sl.h_q);
    }
    for (auto st : s->streams) cudaStreamDestroy(st);
    delete s;
    return GBMP_OK;
}

}  // extern "C"
