// gbmp_cudampl_rrg.hpp -- the reference's RRG planner, motion task and termination
// conditions over the libgbmp C++ facade (gbmp_cudampl.hpp).  Header-only.
//
// Kept surface (reference declarations in parentheses):
//   CUDAMPLib::BaseTermination, StepTermination, TimeoutTermination
//                                      (include/base/Termination.h, include/termination/*.h)
//   CUDAMPLib::BaseTask, SingleArmTask (include/base/Task.h, include/tasks/SingleArmTask.h)
//   CUDAMPLib::RRG                     (include/planners/RRG.h, src/planners/RRG.cpp:9-544)
// Every batch operation of the planner loop (sampling, nearest neighbours, steering,
// state and motion checks) is one libgbmp kernel call; the graph, which the reference
// keeps in a Boost adjacency list, is a plain adjacency list searched with Dijkstra.
#pragma once

#include <chrono>
#include <cstdio>
#include <functional>
#include <limits>
#include <queue>
#include <unordered_map>

#include "gbmp_cudampl.hpp"

namespace CUDAMPLib {

typedef SingleArmSpacePtr BaseSpacePtr;
typedef std::shared_ptr<SingleArmStateManager> BaseStateManagerPtr;

// ---------------------------------------------------------------------------------
// Termination conditions.
// ---------------------------------------------------------------------------------
class BaseTermination {
  public:
    virtual ~BaseTermination() = default;
    virtual void reset() = 0;
    virtual bool checkTerminationCondition() = 0;
    virtual void printTerminationReason() = 0;
};
typedef std::shared_ptr<BaseTermination> BaseTerminationPtr;

// Met after step_limit checks (each check counts one step).
class StepTermination : public BaseTermination {
  public:
    explicit StepTermination(int step_limit) : step_limit_(step_limit), step_count_(0) {}
    void reset() override { step_count_ = 0; }
    bool checkTerminationCondition() override { return ++step_count_ > step_limit_; }
    void printTerminationReason() override { std::printf("Step limit reached\n"); }

  private:
    int step_limit_, step_count_;
};
typedef std::shared_ptr<StepTermination> StepTerminationPtr;

// Met once `timeout` seconds have passed since reset().
class TimeoutTermination : public BaseTermination {
  public:
    explicit TimeoutTermination(float timeout) : timeout_ms_(timeout * 1000.0f) { reset(); }
    void reset() override { start_ = std::chrono::steady_clock::now(); }
    bool checkTerminationCondition() override {
        return std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - start_).count() >
               timeout_ms_;
    }
    void printTerminationReason() override { std::printf("Timeout reached\n"); }

  private:
    float timeout_ms_;
    std::chrono::steady_clock::time_point start_;
};
typedef std::shared_ptr<TimeoutTermination> TimeoutTerminationPtr;

// ---------------------------------------------------------------------------------
// Motion tasks: start and goal configurations in active joints.
// ---------------------------------------------------------------------------------
class BaseTask {
  public:
    virtual ~BaseTask() = default;
    virtual BaseStatesPtr getStartStates(BaseSpacePtr space) = 0;
    virtual BaseStatesPtr getGoalStates(BaseSpacePtr space) = 0;
    virtual std::vector<std::vector<float>> getStartStatesVector() = 0;
    virtual std::vector<std::vector<float>> getGoalStatesVector() = 0;
    virtual void setSolution(const BaseStatesPtr &solution, const BaseSpacePtr space) = 0;
    virtual void setSolution(const std::vector<std::vector<float>> &solution) = 0;
    bool hasSolution() const { return has_solution; }
    void setFailureReason(const std::string &reason) { failure_reason = reason; }
    std::string getFailureReason() const { return failure_reason; }

  protected:
    bool has_solution = false;
    std::string failure_reason;
};
typedef std::shared_ptr<BaseTask> BaseTaskPtr;

// Vectors of `vec` without the ones within `tol` (per element) of an earlier kept one
// (util.cpp:250-266).
inline std::vector<std::vector<float>> removeRedundantVectors(const std::vector<std::vector<float>> &vec, float tol) {
    std::vector<std::vector<float>> unique;
    for (const auto &v : vec) {
        bool dup = false;
        for (const auto &u : unique) {
            bool same = u.size() == v.size();
            for (size_t k = 0; same && k < v.size(); ++k) same = std::fabs(v[k] - u[k]) <= tol;
            if (same) { dup = true; break; }
        }
        if (!dup) unique.push_back(v);
    }
    return unique;
}

class SingleArmTask : public BaseTask {
  public:
    SingleArmTask(const std::vector<std::vector<float>> &start_joint_values,
                  const std::vector<std::vector<float>> &goal_joint_values)
        : start_(start_joint_values), goal_(goal_joint_values) {}
    // Goal region (SingleArmTask.cpp:12-39): `goal_config_sampling_attempts` samples of a
    // space whose projectable constraints describe the region (sampling projects them),
    // kept when feasible, duplicates within 1e-5 removed.
    SingleArmTask(const std::vector<std::vector<float>> &start_joint_values, const BaseSpacePtr &goal_region,
                  int goal_config_sampling_attempts = 50)
        : start_(start_joint_values) {
        auto goals = goal_region->sample(goal_config_sampling_attempts);
        if (!goals) throw std::runtime_error("goal region sampling failed");
        std::vector<bool> feasible;
        goal_region->checkStates(goals, feasible);
        goals->filterStates(feasible);
        goal_ = removeRedundantVectors(goals->getJointStatesHost(), 1e-5f);
    }
    std::vector<std::vector<float>> getStartStatesVector() override { return start_; }
    std::vector<std::vector<float>> getGoalStatesVector() override { return goal_; }
    BaseStatesPtr getStartStates(BaseSpacePtr space) override { return space->createStatesFromVector(start_); }
    BaseStatesPtr getGoalStates(BaseSpacePtr space) override { return space->createStatesFromVector(goal_); }
    void setSolution(const BaseStatesPtr &solution, const BaseSpacePtr space) override {
        setSolution(space->getJointVectorInActiveJointsFromStates(solution));
    }
    void setSolution(const std::vector<std::vector<float>> &solution) override {
        solution_ = solution;
        has_solution = !solution.empty();
    }
    std::vector<std::vector<float>> getSolution() { return solution_; }

  private:
    std::vector<std::vector<float>> start_, goal_, solution_;
};
typedef std::shared_ptr<SingleArmTask> SingleArmTaskPtr;

}  // namespace CUDAMPLib

namespace CUDAMPLib {

// ---------------------------------------------------------------------------------
// Rapidly-exploring random graph (RRG.cpp:9-544).  Vertices are states of the state
// manager, labelled start group (1), goal group (2) or other (0); two super nodes join
// the start and the goal states with zero-cost edges; a vertex that connects both
// groups closes the search and Dijkstra gives the path.
// ---------------------------------------------------------------------------------
class RRG {
  public:
    explicit RRG(BaseSpacePtr space) : space_(std::move(space)), state_manager(space_->createStateManager()) {}

    BaseStateManagerPtr getStateManager() { return state_manager; }
    void setMaxTravelDistance(float max_travel_distance) { max_travel_distance_ = max_travel_distance; }
    void setSampleAttemptsInEachIteration(int n) { sample_attempts_in_each_iteration_ = n; }
    int getNumOfVertices() const { return (int)vertices_.size(); }

    // RRG.cpp:30-90: start / goal states into the manager, each joined to its super node.
    void setMotionTask(BaseTaskPtr task, bool get_full_path = true) {
        get_full_path_ = get_full_path;
        vertices_.clear();
        adj_.clear();
        vertex_of_state_.clear();
        start_nodes_.clear();
        goal_nodes_.clear();
        auto starts = state_manager->add_states(task->getStartStates(space_));
        start_node_ = add_vertex(-1, 1);
        for (int idx : starts) {
            const int v = add_vertex(idx, 1);
            start_nodes_.push_back(v);
            add_edge(v, start_node_, 0.f);
        }
        auto goals = state_manager->add_states(task->getGoalStates(space_));
        goal_node_ = add_vertex(-1, 2);
        for (int idx : goals) {
            const int v = add_vertex(idx, 2);
            goal_nodes_.push_back(v);
            add_edge(v, goal_node_, 0.f);
        }
        task_ = std::move(task);
    }

    void getStartAndGoalGroupStates(BaseStatesPtr &start_group_states, BaseStatesPtr &goal_group_states) {
        std::vector<int> s, g;
        group_indexes(s, g);
        start_group_states = state_manager->get_states(s);
        goal_group_states = state_manager->get_states(g);
    }

    void solve(BaseTerminationPtr termination_condition);

  private:
    struct Vertex {
        int index_in_manager;   // -1 for the two super nodes
        int group;              // 0 other, 1 start, 2 goal
    };

    int add_vertex(int index_in_manager, int group) {
        vertices_.push_back({index_in_manager, group});
        adj_.emplace_back();
        if (index_in_manager >= 0) vertex_of_state_[index_in_manager] = (int)vertices_.size() - 1;
        return (int)vertices_.size() - 1;
    }
    void add_edge(int a, int b, float w) {
        adj_[a].push_back({b, w});
        adj_[b].push_back({a, w});
    }
    // RRG.cpp:122-139
    void group_indexes(std::vector<int> &start, std::vector<int> &goal) const {
        for (const auto &v : vertices_) {
            if (v.index_in_manager < 0) continue;
            if (v.group == 1) start.push_back(v.index_in_manager);
            else if (v.group == 2) goal.push_back(v.index_in_manager);
        }
    }
    // Dijkstra from the start super node; returns manager indexes start -> goal.
    std::vector<int> shortest_path() const {
        const int n = (int)vertices_.size();
        std::vector<float> dist(n, std::numeric_limits<float>::max());
        std::vector<int> pred(n, -1);
        typedef std::pair<float, int> Item;
        std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
        dist[start_node_] = 0.f;
        pq.push({0.f, start_node_});
        while (!pq.empty()) {
            const Item it = pq.top();
            pq.pop();
            if (it.first > dist[it.second]) continue;
            for (const auto &e : adj_[it.second]) {
                const float d = it.first + e.second;
                if (d < dist[e.first]) {
                    dist[e.first] = d;
                    pred[e.first] = it.second;
                    pq.push({d, e.first});
                }
            }
        }
        std::vector<int> path;
        if (pred[goal_node_] < 0) return path;
        for (int v = goal_node_; v != -1; v = pred[v])
            if (vertices_[v].index_in_manager >= 0) path.push_back(vertices_[v].index_in_manager);
        std::reverse(path.begin(), path.end());
        return path;
    }
    void set_solution(const std::vector<int> &path_indexes) {
        auto waypoints = state_manager->get_states(path_indexes);
        if (get_full_path_) task_->setSolution(space_->getPathFromWaypoints(waypoints), space_);
        else task_->setSolution(waypoints, space_);
    }

    BaseSpacePtr space_;
    BaseStateManagerPtr state_manager;
    BaseTaskPtr task_;
    bool get_full_path_ = true;
    int sample_attempts_in_each_iteration_ = 30;   // RRG.cpp:15-16
    float max_travel_distance_ = 0.5f;
    std::vector<Vertex> vertices_;
    std::vector<std::vector<std::pair<int, float>>> adj_;
    std::unordered_map<int, int> vertex_of_state_;
    std::vector<int> start_nodes_, goal_nodes_;
    int start_node_ = -1, goal_node_ = -1;
};
typedef std::shared_ptr<RRG> RRGPtr;

}  // namespace CUDAMPLib

namespace CUDAMPLib {

// RRG.cpp:140-510.  Each iteration: sample, steer towards the nearest vertex of the
// start group (even t) or goal group (odd t) by at most the group's travel distance,
// drop colliding samples, then try motions from every sample to its nearest start and
// nearest goal vertex; samples with a free motion join the graph (labelled with the
// group they connect to).  A group whose samples connect to nothing halves its travel
// distance (not below 0.1) and the next iteration keeps the same group (RRG.cpp:373-395).
inline void RRG::solve(BaseTerminationPtr termination_condition) {
    std::vector<int> start_idx, goal_idx;
    for (int v : start_nodes_) start_idx.push_back(vertices_[v].index_in_manager);
    for (int v : goal_nodes_) goal_idx.push_back(vertices_[v].index_in_manager);

    // feasibility of the start and goal states (RRG.cpp:144-180)
    std::vector<bool> start_ok, goal_ok;
    space_->checkStates(state_manager->get_states(start_idx), start_ok);
    space_->checkStates(state_manager->get_states(goal_idx), goal_ok);
    if (std::find(start_ok.begin(), start_ok.end(), true) == start_ok.end() ||
        std::find(goal_ok.begin(), goal_ok.end(), true) == goal_ok.end()) {
        task_->setFailureReason("InvalidInput");
        return;
    }

    // direct motions between every start and goal state (RRG.cpp:182-236)
    std::vector<int> left, right;
    for (int a : start_idx)
        for (int b : goal_idx) {
            left.push_back(a);
            right.push_back(b);
        }
    std::vector<bool> direct_ok;
    std::vector<float> direct_cost;
    space_->checkMotions(state_manager->get_states(left), state_manager->get_states(right), direct_ok, direct_cost);
    int best = -1;
    for (size_t i = 0; i < direct_ok.size(); ++i)
        if (direct_ok[i] && (best < 0 || direct_cost[i] < direct_cost[best])) best = (int)i;
    if (best >= 0) {
        set_solution({left[best], right[best]});
        return;
    }

    termination_condition->reset();
    float travel[2] = {max_travel_distance_, max_travel_distance_};
    bool has_solution = false;
    for (int t = 0; t < 1000000; ++t) {
        if (termination_condition->checkTerminationCondition()) {
            termination_condition->printTerminationReason();
            task_->setFailureReason("MeetTerminationCondition");
            break;
        }
        const int side = t % 2;   // 0 grows from the start group, 1 from the goal group
        auto states = space_->sample(sample_attempts_in_each_iteration_);
        if (!states) break;
        std::vector<int> sg, gg;
        group_indexes(sg, gg);
        std::vector<std::vector<int>> nn;
        state_manager->find_the_nearest_neighbors(states, {side == 0 ? sg : gg}, nn);
        std::vector<int> nearest;
        for (auto &r : nn) nearest.push_back(r[0]);
        state_manager->interpolateToStates(states, nearest, travel[side]);

        std::vector<bool> feasible;
        space_->checkStates(states, feasible);
        states->filterStates(feasible);
        const int n = states->getNumOfStates();
        if (n == 0) continue;

        // nearest start-group and goal-group vertex of every sample, motions to both
        std::vector<std::vector<int>> both;
        state_manager->find_the_nearest_neighbors(states, {sg, gg}, both);
        auto from = state_manager->concatinate_states({states, states});
        std::vector<int> to_idx(2 * (size_t)n);
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < n; ++i) to_idx[(size_t)j * n + i] = both[i][j];
        std::vector<bool> motion_ok;
        std::vector<float> motion_cost;
        space_->checkMotions(from, state_manager->get_states(to_idx), motion_ok, motion_cost);

        std::vector<bool> can_connect(n, false);
        std::vector<std::vector<std::pair<int, float>>> links;
        int connections[2] = {0, 0};
        for (int i = 0; i < n; ++i) {
            std::vector<std::pair<int, float>> li;
            for (int j = 0; j < 2; ++j)
                if (motion_ok[(size_t)j * n + i]) {
                    can_connect[i] = true;
                    li.push_back({to_idx[(size_t)j * n + i], motion_cost[(size_t)j * n + i]});
                    ++connections[j];
                }
            if (can_connect[i]) links.push_back(li);
        }
        if (connections[side] == 0) {
            travel[side] = std::max(travel[side] * 0.5f, 0.1f);
            ++t;
            continue;
        }
        travel[side] = max_travel_distance_;

        states->filterStates(can_connect);
        auto added = state_manager->add_states(states);
        for (size_t i = 0; i < added.size(); ++i) {
            const int v = add_vertex(added[i], 0);
            bool to_start = false, to_goal = false;
            for (auto &l : links[i]) {
                const int u = vertex_of_state_.at(l.first);
                if (vertices_[u].group == 1) to_start = true;
                else if (vertices_[u].group == 2) to_goal = true;
                add_edge(v, u, l.second);
            }
            if (to_start && !to_goal) vertices_[v].group = 1;
            else if (!to_start && to_goal) vertices_[v].group = 2;
            else if (to_start && to_goal) has_solution = true;
        }
        if (has_solution) break;
    }
    if (has_solution) set_solution(shortest_path());
}

}  // namespace CUDAMPLib
