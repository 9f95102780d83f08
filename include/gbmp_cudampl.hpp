// gbmp_cudampl.hpp -- C++ facade with the state-space / constraint / planner API of the
// reference (CUDAMPLib and CPRRTC) over the libgbmp C-ABI (gbmp.h).  Header-only; link
// libgbmp.so and the CUDA runtime.
//
// Kept surface (reference declarations in parentheses):
//   CUDAMPLib::SelfCollisionConstraint, EnvConstraintSphere, EnvConstraintCuboid,
//     EnvConstraintCylinder            (include/constraints/*.h)
//   CUDAMPLib::SingleArmSpace          (include/spaces/SingleArmSpace.h:21-176)
//   CUDAMPLib::SingleArmStates         (include/states/SingleArmStates.h:227-330)
//   CUDAMPLib::SingleArmStateManager   (include/states/SingleArmStates.h:332-399)
//   CPRRTC::Sphere/Cuboid/Cylinder, CPRRTC::RobotSolver
//                                      (cudampl/CPRRTC/include/Obstacle.h, RobotSolver.h:19-164)
// Errors follow the reference: invalid arguments throw std::runtime_error (e.g.
// SingleArmSpace.cu:65-77); allocation failures give nullptr / isValid() == false
// (base/States.h:39-52).  Joint pose / axis arguments accept Eigen types (anything with
// .matrix()(r, c) / operator()(i)) or plain arrays (operator[]).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "gbmp.h"

namespace CUDAMPLib {

namespace detail {

inline void check(gbmp_status s) {
    if (s == GBMP_OK) return;
    throw std::runtime_error(std::string("gbmp: ") + gbmp_status_string(s) + ": " + gbmp_last_error());
}

template <typename T, typename = void>
struct has_matrix : std::false_type {};
template <typename T>
struct has_matrix<T, std::void_t<decltype(std::declval<const T &>().matrix()(0, 0))>> : std::true_type {};
template <typename T, typename = void>
struct has_call : std::false_type {};
template <typename T>
struct has_call<T, std::void_t<decltype(std::declval<const T &>()(0))>> : std::true_type {};

template <typename P>
float pose_at(const P &p, int r, int c) {
    if constexpr (has_matrix<P>::value) return (float)p.matrix()(r, c);
    else return (float)p[r * 4 + c];
}
template <typename V>
float vec_at(const V &v, int i) {
    if constexpr (has_call<V>::value) return (float)v(i);
    else return (float)v[i];
}

// Device buffer owned by a states object.
struct DevArray {
    void *p = nullptr;
    size_t bytes = 0;
    DevArray() = default;
    explicit DevArray(size_t n) : bytes(n) {
        if (n && cudaMalloc(&p, n) != cudaSuccess) { cudaGetLastError(); p = nullptr; }
    }
    ~DevArray() { if (p) cudaFree(p); }
    DevArray(const DevArray &) = delete;
    DevArray &operator=(const DevArray &) = delete;
    bool ok() const { return p != nullptr || bytes == 0; }
};

inline void rpy_to_rot(float roll, float pitch, float yaw, float *R) {   // R = Rz(yaw) Ry(pitch) Rx(roll)
    const float cr = std::cos(roll), sr = std::sin(roll), cp = std::cos(pitch), sp = std::sin(pitch);
    const float cy = std::cos(yaw), sy = std::sin(yaw);
    R[0] = cy * cp; R[1] = cy * sp * sr - sy * cr; R[2] = cy * sp * cr + sy * sr;
    R[3] = sy * cp; R[4] = sy * sp * sr + cy * cr; R[5] = sy * sp * cr - cy * sr;
    R[6] = -sp;     R[7] = cp * sr;                R[8] = cp * cr;
}

}  // namespace detail

// ---------------------------------------------------------------------------------
// Constraints.  Only their tables are kept; SingleArmSpace turns them into one robot
// (self-collision link matrix) and one environment (all obstacles).
// ---------------------------------------------------------------------------------
enum class ConstraintKind { Self = 0, Sphere = 1, Cuboid = 2, Cylinder = 3, TaskSpace = 4, Boundary = 5 };

class BaseConstraint {
  public:
    BaseConstraint(std::string name, ConstraintKind k) : constraint_name(std::move(name)), kind(k) {}
    virtual ~BaseConstraint() = default;
    std::string getName() const { return constraint_name; }
    bool isProjectable() const { return kind == ConstraintKind::TaskSpace || kind == ConstraintKind::Boundary; }
    std::string constraint_name;
    ConstraintKind kind;
};
typedef std::shared_ptr<BaseConstraint> BaseConstraintPtr;

class SelfCollisionConstraint : public BaseConstraint {
  public:
    SelfCollisionConstraint(const std::string &name, const std::vector<int> &self_collision_spheres_map,
                            const std::vector<float> &self_collision_spheres_radius,
                            const std::vector<std::vector<bool>> &self_collision_enables_map)
        : BaseConstraint(name, ConstraintKind::Self), enables(self_collision_enables_map) {
        (void)self_collision_spheres_map;
        (void)self_collision_spheres_radius;
    }
    std::vector<std::vector<bool>> enables;
};

class EnvConstraintSphere : public BaseConstraint {
  public:
    EnvConstraintSphere(const std::string &name, const std::vector<std::vector<float>> &pos,
                        const std::vector<float> &radius)
        : BaseConstraint(name, ConstraintKind::Sphere), pos(pos), radius(radius) {
        if (pos.size() != radius.size()) throw std::runtime_error("sphere positions and radii differ in length");
    }
    std::vector<std::vector<float>> pos;
    std::vector<float> radius;
};

class EnvConstraintCuboid : public BaseConstraint {
  public:
    // Argument order of EnvConstraintCuboid.h:23-29: position, orientation (row-major 3x3),
    // max, min (extents in the box frame).
    EnvConstraintCuboid(const std::string &name, const std::vector<std::vector<float>> &pos,
                        const std::vector<std::vector<float>> &orientation, const std::vector<std::vector<float>> &max,
                        const std::vector<std::vector<float>> &min)
        : BaseConstraint(name, ConstraintKind::Cuboid), pos(pos), rot(orientation), mx(max), mn(min) {
        if (pos.size() != orientation.size() || pos.size() != max.size() || pos.size() != min.size())
            throw std::runtime_error("cuboid tables differ in length");
    }
    std::vector<std::vector<float>> pos, rot, mx, mn;
};

class EnvConstraintCylinder : public BaseConstraint {
  public:
    EnvConstraintCylinder(const std::string &name, const std::vector<std::vector<float>> &pos,
                          const std::vector<std::vector<float>> &orientation, const std::vector<float> &radius,
                          const std::vector<float> &height)
        : BaseConstraint(name, ConstraintKind::Cylinder), pos(pos), rot(orientation), radius(radius), height(height) {
        if (pos.size() != orientation.size() || pos.size() != radius.size() || pos.size() != height.size())
            throw std::runtime_error("cylinder tables differ in length");
    }
    std::vector<std::vector<float>> pos, rot;
    std::vector<float> radius, height;
};

// Task-space region of a frame fixed in one link (TaskSpaceConstraint.h): pose of
// `offset_pose_in_task_link` (4x4, Eigen or 16 row-major floats) in link
// `task_link_index`, reference x y z roll pitch yaw and per-axis tolerances.  Projectable:
// samples and interpolated states of a space that holds it are projected onto it.
class TaskSpaceConstraint : public BaseConstraint {
  public:
    template <typename M>
    TaskSpaceConstraint(const std::string &name, int task_link_index, const M &offset_pose_in_task_link,
                        const std::vector<float> &reference_frame, const std::vector<float> &tolerance)
        : BaseConstraint(name, ConstraintKind::TaskSpace), task_link(task_link_index), reference(reference_frame),
          tol(tolerance) {
        if (reference_frame.size() != 6 || tolerance.size() != 6)
            throw std::runtime_error("reference frame and tolerance need 6 values each");
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) offset[4 * r + c] = detail::pose_at(offset_pose_in_task_link, r, c);
    }
    int task_link;
    float offset[16];
    std::vector<float> reference, tol;
};

// Joint limits as a projectable constraint (BoundaryConstraint.h).  The bounds are the
// space's joint limits (the reference builds it from the same limits).
class BoundaryConstraint : public BaseConstraint {
  public:
    BoundaryConstraint(const std::string &name, const std::vector<float> &lower_bound,
                       const std::vector<float> &upper_bound, const std::vector<bool> &active_joint_map)
        : BaseConstraint(name, ConstraintKind::Boundary), lower(lower_bound), upper(upper_bound),
          active(active_joint_map) {}
    std::vector<float> lower, upper;
    std::vector<bool> active;
};

class SingleArmSpace;

// ---------------------------------------------------------------------------------
// States: joint vectors [n x L] on the device plus costs.
// ---------------------------------------------------------------------------------
class SingleArmStates {
  public:
    SingleArmStates(int n, const SingleArmSpace *space);
    int getNumOfStates() const { return n_; }
    bool isValid() const { return valid_; }
    int getNumOfJoints() const { return L_; }
    float *getJointStatesCuda() { return static_cast<float *>(q_->p); }
    const float *getJointStatesCuda() const { return static_cast<const float *>(q_->p); }
    float *getCostsCuda() { return static_cast<float *>(costs_->p); }
    float *getTotalCostsCuda() { return static_cast<float *>(total_->p); }

    // FK + sphere centres (SingleArmStates::update, SingleArmStates.cu:696-723).
    void update();
    std::vector<std::vector<float>> getJointStatesFullHost() const;
    std::vector<std::vector<float>> getJointStatesHost() const;
    std::vector<std::vector<std::vector<float>>> getLinkPosesInBaseLinkHost();
    std::vector<std::vector<std::vector<float>>> getSelfCollisionSpheresPosInBaseLinkHost();
    // Space Jacobians of every link (SingleArmStates::calculateSpaceJacobian,
    // SingleArmStates.cu:793-817, kernel :223-338), kept on the device.
    void calculateSpaceJacobian(bool synchronize = true);
    // One link's space Jacobian per state, [n][joints][6] (the reference returns an
    // Eigen matrix joints x 6 per state, SingleArmStates.cu:999-1039); computed first
    // if calculateSpaceJacobian has not been called; std::runtime_error for an unknown
    // link name.
    std::vector<std::vector<std::vector<float>>> getSpaceJacobianInBaseLinkHost(const std::string &link_name);
    std::vector<float> getTotalCostsHost() const;
    std::vector<std::vector<float>> getCostsHost() const;   // [n][constraints]
    // Keep the states whose flag is true (BaseStates::filterStates, base/States.h:83-140).
    void filterStates(const std::vector<bool> &filter_map);

  private:
    friend class SingleArmSpace;
    friend class SingleArmStateManager;
    int n_, L_, S_;
    bool valid_ = true, updated_ = false;
    const SingleArmSpace *space_;
    std::shared_ptr<detail::DevArray> q_, costs_, total_, poses_, centers_, jac_;
};
typedef std::shared_ptr<SingleArmStates> SingleArmStatesPtr;
typedef SingleArmStatesPtr BaseStatesPtr;

// ---------------------------------------------------------------------------------
// The space: robot tables + constraints.
// ---------------------------------------------------------------------------------
class SingleArmStateManager;

class SingleArmSpace {
  public:
    template <typename Pose, typename Vec>
    SingleArmSpace(size_t dim, const std::vector<BaseConstraintPtr> &constraints, const std::vector<int> &joint_types,
                   const std::vector<Pose> &joint_poses, const std::vector<Vec> &joint_axes,
                   const std::vector<int> &link_parent_link_maps,
                   const std::vector<int> &self_collision_spheres_to_link_map,
                   const std::vector<std::vector<float>> &self_collision_spheres_pos_in_link,
                   const std::vector<float> &self_collision_spheres_radius, const std::vector<bool> &active_joint_map,
                   const std::vector<float> &lower, const std::vector<float> &upper,
                   const std::vector<float> &default_joint_values, const std::vector<std::string> &link_names,
                   float resolution = 0.02f)
        : dim_(dim), constraints_(constraints), resolution_(resolution), link_names_(link_names) {
        const int L = (int)joint_types.size();
        if ((int)link_parent_link_maps.size() != L || (int)joint_poses.size() != L || (int)joint_axes.size() != L)
            throw std::runtime_error("joint tables differ in length");
        if (link_names.size() != (size_t)L) throw std::runtime_error("Number of link names is not equal to the number of links");
        L_ = L;
        S_ = (int)self_collision_spheres_radius.size();
        types_ = joint_types;
        parent_ = link_parent_link_maps;
        poses_.resize(16 * L);
        axes_.resize(3 * L);
        for (int i = 0; i < L; ++i) {
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) poses_[16 * i + 4 * r + c] = detail::pose_at(joint_poses[i], r, c);
            for (int k = 0; k < 3; ++k) axes_[3 * i + k] = detail::vec_at(joint_axes[i], k);
        }
        slink_ = self_collision_spheres_to_link_map;
        spos_.clear();
        for (auto &p : self_collision_spheres_pos_in_link) {
            if (p.size() < 3) throw std::runtime_error("sphere position needs 3 values");
            spos_.insert(spos_.end(), p.begin(), p.begin() + 3);
        }
        srad_ = self_collision_spheres_radius;
        active_.assign(active_joint_map.begin(), active_joint_map.end());
        lower_ = lower;
        upper_ = upper;
        default_ = default_joint_values;
        size_t na = 0;
        for (auto a : active_joint_map) na += a ? 1 : 0;
        if (na != dim) throw std::runtime_error("dim differs from the number of active joints");
        // self-collision link matrix from the SelfCollisionConstraint (none: no self pairs)
        enables_.assign((size_t)L * L, 0);
        for (auto &c : constraints)
            if (c->kind == ConstraintKind::Self) {
                auto *sc = static_cast<SelfCollisionConstraint *>(c.get());
                for (int a = 0; a < L && a < (int)sc->enables.size(); ++a)
                    for (int b = 0; b < L && b < (int)sc->enables[a].size(); ++b) enables_[a * L + b] = sc->enables[a][b];
            }
        build();
    }
    ~SingleArmSpace() {
        if (env_) gbmp_env_destroy(env_);
        if (robot_) gbmp_robot_destroy(robot_);
    }
    SingleArmSpace(const SingleArmSpace &) = delete;
    SingleArmSpace &operator=(const SingleArmSpace &) = delete;

    const std::vector<float> &getLower() const { return lower_; }
    const std::vector<float> &getUpper() const { return upper_; }
    size_t getDim() const { return dim_; }
    int getNumOfJoints() const { return L_; }
    gbmp_robot robot() const { return robot_; }
    // Index of a link by name; std::runtime_error("Link <name> not found in the space") if
    // there is none (the reference's lookup, SingleArmStates.cu:1003-1016).
    int getLinkIndex(const std::string &link_name) const {
        for (size_t i = 0; i < link_names_.size(); ++i)
            if (link_names_[i] == link_name) return (int)i;
        throw std::runtime_error("Link " + link_name + " not found in the space");
    }
    gbmp_env env() const { return env_; }
    int numConstraints() const { return (int)constraints_.size(); }

    // Uniform samples in the limits (SingleArmSpace::sample, SingleArmSpace.cu:251-322).
    BaseStatesPtr sample(int num_of_config) {
        auto st = std::make_shared<SingleArmStates>(num_of_config, this);
        if (!st->isValid()) return nullptr;
        detail::check(gbmp_sample(robot_, seed_, offset_, num_of_config, st->getJointStatesCuda(), nullptr));
        offset_ += (uint64_t)num_of_config;
        if (projectable_) projectStates(st);   // SingleArmSpace.cu:316-320
        return st;
    }

    bool hasProjectableConstraints() const { return projectable_; }
    // Projection onto the projectable constraints (SingleArmSpace.cu:1631-1662).
    void projectStates(const BaseStatesPtr &states) {
        if (!projectable_ || states->getNumOfStates() == 0) return;
        detail::check(gbmp_project_states(robot_, &proj_, states->getJointStatesCuda(), states->getNumOfStates(),
                                          nullptr, nullptr, nullptr));
        cudaDeviceSynchronize();
    }
    void setSeed(uint64_t seed) { seed_ = seed; offset_ = 0; }

    // checkStates (SingleArmSpace.cu:1572-1602): per-constraint costs and total.
    void checkStates(const BaseStatesPtr &states) {
        const int n = states->getNumOfStates();
        if (n == 0) return;
        detail::DevArray slots(sizeof(float) * 4 * (size_t)n);
        detail::check(gbmp_check_states(robot_, env_, states->getJointStatesCuda(), n, GBMP_CHECK_COST, nullptr,
                                        static_cast<float *>(slots.p), states->getTotalCostsCuda(), nullptr));
        // scatter the type slots to the constraint order (the first constraint of a type
        // carries the merged cost of that type)
        int seen[4] = {0, 0, 0, 0};
        for (size_t c = 0; c < constraints_.size(); ++c) {
            const int k = (int)constraints_[c]->kind;
            if (k > 3) continue;   // projectable constraints: below
            float *dst = states->getCostsCuda() + c * (size_t)n;
            if (!seen[k]++) detail::check(cudaMemcpy(dst, static_cast<float *>(slots.p) + (size_t)k * n,
                                                     sizeof(float) * n, cudaMemcpyDeviceToDevice) == cudaSuccess
                                              ? GBMP_OK : GBMP_ERR_CUDA);
            else detail::check(cudaMemset(dst, 0, sizeof(float) * n) == cudaSuccess ? GBMP_OK : GBMP_ERR_CUDA);
        }
        if (projectable_) {
            // task-space and joint-limit costs (computeCost of the two constraints): a
            // projection of zero iterations only evaluates them
            detail::DevArray tc(sizeof(float) * n), bc(sizeof(float) * n);
            gbmp_projection p0 = proj_;
            p0.iterations = 0;
            detail::check(gbmp_project_states(robot_, &p0, states->getJointStatesCuda(), n, static_cast<float *>(tc.p),
                                              static_cast<float *>(bc.p), nullptr));
            std::vector<float> h_tc(n), h_bc(n), tot = states->getTotalCostsHost();
            cudaMemcpy(h_tc.data(), tc.p, sizeof(float) * n, cudaMemcpyDeviceToHost);
            cudaMemcpy(h_bc.data(), bc.p, sizeof(float) * n, cudaMemcpyDeviceToHost);
            for (size_t c = 0; c < constraints_.size(); ++c) {
                const ConstraintKind k = constraints_[c]->kind;
                if (k != ConstraintKind::TaskSpace && k != ConstraintKind::Boundary) continue;
                const std::vector<float> &src = k == ConstraintKind::TaskSpace ? h_tc : h_bc;
                cudaMemcpy(states->getCostsCuda() + c * (size_t)n, src.data(), sizeof(float) * n,
                           cudaMemcpyHostToDevice);
                for (int i = 0; i < n; ++i) tot[i] += src[i];
            }
            cudaMemcpy(states->getTotalCostsCuda(), tot.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
        }
        detail::check(cudaDeviceSynchronize() == cudaSuccess ? GBMP_OK : GBMP_ERR_CUDA);
    }
    void checkStates(const BaseStatesPtr &states, std::vector<bool> &state_feasibility) {
        checkStates(states);
        auto total = states->getTotalCostsHost();
        state_feasibility.assign(total.size(), false);
        for (size_t i = 0; i < total.size(); ++i) state_feasibility[i] = total[i] == 0.0f;
    }

    // checkMotions (SingleArmSpace.cu:628-848): feasibility and L2 motion cost per edge.
    bool checkMotions(const BaseStatesPtr &states1, const BaseStatesPtr &states2, std::vector<bool> &motion_feasibility,
                      std::vector<float> &motion_costs) {
        const int n = states1->getNumOfStates();
        if (n != states2->getNumOfStates()) throw std::runtime_error("Number of states in states1 and states2 are not equal");
        if (n == 0) throw std::runtime_error("No states to check");
        // with projectable constraints the motions follow them (checkConstrainedMotions,
        // SingleArmSpace.cu:636-639, :1466-1477)
        if (projectable_) {
            std::vector<uint8_t> h_ok;
            constrainedMotions(states1->getJointStatesCuda(), states2->getJointStatesCuda(), n, h_ok, motion_costs,
                               nullptr);
            motion_feasibility.assign(n, false);
            for (int i = 0; i < n; ++i) motion_feasibility[i] = h_ok[i] != 0;
            return true;
        }
        detail::DevArray ok((size_t)n), len(sizeof(float) * n);
        if (!ok.ok() || !len.ok()) {
            motion_feasibility.assign(n, false);
            motion_costs.assign(n, 0.f);
            return false;
        }
        detail::check(gbmp_check_edges(robot_, env_, states1->getJointStatesCuda(), states2->getJointStatesCuda(), n,
                                       resolution_, GBMP_STEP_L2, static_cast<uint8_t *>(ok.p), nullptr,
                                       static_cast<float *>(len.p), nullptr, nullptr));
        std::vector<uint8_t> h_ok(n);
        motion_costs.resize(n);
        cudaMemcpy(h_ok.data(), ok.p, n, cudaMemcpyDeviceToHost);
        cudaMemcpy(motion_costs.data(), len.p, sizeof(float) * n, cudaMemcpyDeviceToHost);
        motion_feasibility.resize(n);
        for (int i = 0; i < n; ++i) motion_feasibility[i] = h_ok[i] != 0;
        return true;
    }

    // Steer to_states towards from_states to at most max_distance (SingleArmSpace.cu:1368-1409).
    void interpolate(const BaseStatesPtr &from_states, const BaseStatesPtr &to_states, float max_distance) {
        detail::check(gbmp_steer(robot_, from_states->getJointStatesCuda(), nullptr, to_states->getJointStatesCuda(),
                                 to_states->getNumOfStates(), max_distance, nullptr));
        cudaDeviceSynchronize();
        if (projectable_) projectStates(to_states);   // SingleArmSpace.cu:1400-1405
    }

    BaseStatesPtr createStatesFromVectorFull(const std::vector<std::vector<float>> &joint_values) {
        if (joint_values.empty()) throw std::runtime_error("No joint values is empty");
        std::vector<float> flat;
        for (auto &v : joint_values) {
            if ((int)v.size() != L_) throw std::runtime_error("Joint values size is not correct");
            flat.insert(flat.end(), v.begin(), v.end());
        }
        auto st = std::make_shared<SingleArmStates>((int)joint_values.size(), this);
        if (!st->isValid()) return nullptr;
        cudaMemcpy(st->getJointStatesCuda(), flat.data(), sizeof(float) * flat.size(), cudaMemcpyHostToDevice);
        return st;
    }
    // Active-joint vectors, inactive joints at their defaults (SingleArmSpace.cu:436-497).
    BaseStatesPtr createStatesFromVector(const std::vector<std::vector<float>> &joint_values) {
        if (joint_values.empty()) throw std::runtime_error("No joint values is empty");
        std::vector<std::vector<float>> full;
        for (auto &v : joint_values) {
            if (v.size() != dim_)
                throw std::runtime_error("Joint values size is not correct. Expected: " + std::to_string(dim_) +
                                         " Got: " + std::to_string(v.size()));
            std::vector<float> f(L_);
            size_t k = 0;
            for (int j = 0; j < L_; ++j) f[j] = active_[j] ? v[k++] : default_[j];
            full.push_back(f);
        }
        return createStatesFromVectorFull(full);
    }
    std::vector<std::vector<float>> getJointVectorInActiveJointsFromStates(const BaseStatesPtr &states) {
        return states->getJointStatesHost();
    }
    // Waypoints to a dense path at the space resolution (SingleArmSpace.cu:1411-1464,
    // interpolateVectors in util.cpp:205-248).
    BaseStatesPtr getPathFromWaypoints(const BaseStatesPtr &waypoints) {
        // with projectable constraints (getConstrainedPathFromWaypoints, SingleArmSpace.cu:1416-1419,
        // :1479-1564): each segment as a constrained motion forwards and backwards (a
        // constrained motion need not be feasible both ways); the forward motion's states
        // if it is feasible, else the backward motion's in reverse, else none
        if (projectable_) {
            auto w = waypoints->getJointStatesFullHost();
            if (w.size() < 2) return createStatesFromVectorFull(w);
            const int m = 2 * (int)(w.size() - 1);
            std::vector<float> from((size_t)m * L_), to((size_t)m * L_);
            for (size_t i = 0; i + 1 < w.size(); ++i) {
                std::copy(w[i].begin(), w[i].end(), from.begin() + (2 * i) * L_);
                std::copy(w[i + 1].begin(), w[i + 1].end(), to.begin() + (2 * i) * L_);
                std::copy(w[i + 1].begin(), w[i + 1].end(), from.begin() + (2 * i + 1) * L_);
                std::copy(w[i].begin(), w[i].end(), to.begin() + (2 * i + 1) * L_);
            }
            detail::DevArray d_from(sizeof(float) * from.size()), d_to(sizeof(float) * to.size());
            if (!d_from.ok() || !d_to.ok()) return nullptr;
            cudaMemcpy(d_from.p, from.data(), sizeof(float) * from.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(d_to.p, to.data(), sizeof(float) * to.size(), cudaMemcpyHostToDevice);
            std::vector<uint8_t> ok;
            std::vector<float> cost;
            std::vector<std::vector<std::vector<float>>> motions;
            constrainedMotions(static_cast<float *>(d_from.p), static_cast<float *>(d_to.p), m, ok, cost, &motions);
            std::vector<std::vector<float>> path;
            for (int i = 0; i < m; i += 2) {
                if (ok[i]) path.insert(path.end(), motions[i].begin(), motions[i].end());
                else if (ok[i + 1]) path.insert(path.end(), motions[i + 1].rbegin(), motions[i + 1].rend());
            }
            if (path.empty()) return nullptr;
            return createStatesFromVectorFull(path);
        }
        auto w = waypoints->getJointStatesFullHost();
        std::vector<std::vector<float>> out;
        for (size_t i = 0; i + 1 < w.size(); ++i) {
            const auto &a = w[i], &b = w[i + 1];
            if (a == b) { out.push_back(a); continue; }
            float d = 0.f;
            for (int j = 0; j < L_; ++j) d += (b[j] - a[j]) * (b[j] - a[j]);
            d = std::sqrt(d);
            const int steps = (int)std::floor(d / resolution_);
            out.push_back(a);
            for (int k = 1; k <= steps; ++k) {
                std::vector<float> m(L_);
                for (int j = 0; j < L_; ++j) m[j] = a[j] + k * ((b[j] - a[j]) / steps);
                out.push_back(m);
            }
            out.push_back(b);
        }
        return createStatesFromVectorFull(out);
    }
    std::shared_ptr<SingleArmStateManager> createStateManager();

    const std::vector<uint8_t> &activeMap() const { return active_; }
    int numSpheres() const { return S_; }

  private:
    // Constrained motions d_from[k] -> d_to[k] (device, [n * L] each) on the space's
    // projectable constraints (computeConstrainedMotions, SingleArmSpace.cu:1049-1366, at
    // most 10000 iterations): feasibility, length and, when `motions` is given, the
    // recorded states of every feasible motion.
    void constrainedMotions(const float *d_from, const float *d_to, int n, std::vector<uint8_t> &ok,
                            std::vector<float> &cost, std::vector<std::vector<std::vector<float>>> *motions) {
        constexpr int kMaxIterations = 10000;
        const int cap = motions ? kMaxIterations : 0;
        detail::DevArray d_ok((size_t)n), d_cost(sizeof(float) * n), d_cnt(sizeof(int32_t) * n),
            d_states(sizeof(float) * (size_t)n * cap * L_);
        if (!d_ok.ok() || !d_cost.ok() || !d_cnt.ok() || !d_states.ok())
            throw std::runtime_error("constrained motion buffers could not be allocated");
        detail::check(gbmp_constrained_motions(robot_, env_, &proj_, d_from, d_to, n, resolution_, kMaxIterations,
                                               static_cast<uint8_t *>(d_ok.p), static_cast<float *>(d_cost.p),
                                               static_cast<int32_t *>(d_cnt.p),
                                               cap ? static_cast<float *>(d_states.p) : nullptr, cap ? cap : 1,
                                               nullptr));
        ok.resize(n);
        cost.resize(n);
        std::vector<int32_t> cnt(n);
        cudaMemcpy(ok.data(), d_ok.p, n, cudaMemcpyDeviceToHost);
        cudaMemcpy(cost.data(), d_cost.p, sizeof(float) * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(cnt.data(), d_cnt.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
        if (!motions) return;
        motions->assign(n, {});
        for (int k = 0; k < n; ++k) {
            if (!ok[k]) continue;
            const int c = std::min(cnt[k], cap);
            std::vector<float> flat((size_t)c * L_);
            cudaMemcpy(flat.data(), static_cast<float *>(d_states.p) + (size_t)k * cap * L_, sizeof(float) * flat.size(),
                       cudaMemcpyDeviceToHost);
            for (int j = 0; j < c; ++j) (*motions)[k].emplace_back(flat.begin() + (size_t)j * L_, flat.begin() + (size_t)(j + 1) * L_);
        }
    }

    void build() {
        gbmp_robot_desc d{};
        d.num_links = L_;
        d.joint_types = types_.data();
        d.joint_poses = poses_.data();
        d.joint_axes = axes_.data();
        d.parent = parent_.data();
        d.num_spheres = S_;
        d.sphere_link = slink_.data();
        d.sphere_pos = spos_.data();
        d.sphere_radius = srad_.data();
        d.active_joints = active_.data();
        d.lower = lower_.data();
        d.upper = upper_.data();
        d.default_values = default_.data();
        d.self_enables = enables_.data();
        d.resolution = resolution_;
        detail::check(gbmp_robot_create(&d, GBMP_ROBOT_GENERIC, &robot_));
        // projectable constraints (SingleArmSpace.cu:33-60): one task-space region and / or
        // the joint limits
        proj_.task_link = -1;
        proj_.iterations = 10;   // CUDAMPLib_PROJECT_MAX_ITERATION
        for (int k = 0; k < 16; ++k) proj_.offset[k] = (k % 5 == 0) ? 1.f : 0.f;
        for (auto &c : constraints_) {
            if (c->kind == ConstraintKind::TaskSpace) {
                if (proj_.task_link >= 0) throw std::runtime_error("one task-space constraint per space is supported");
                auto *tc = static_cast<TaskSpaceConstraint *>(c.get());
                if (tc->task_link < 0 || tc->task_link >= L_) throw std::runtime_error("task link index out of range");
                proj_.task_link = tc->task_link;
                for (int k = 0; k < 16; ++k) proj_.offset[k] = tc->offset[k];
                for (int k = 0; k < 6; ++k) {
                    proj_.reference[k] = tc->reference[k];
                    proj_.tolerance[k] = tc->tol[k];
                }
                projectable_ = true;
            } else if (c->kind == ConstraintKind::Boundary) {
                auto *bc = static_cast<BoundaryConstraint *>(c.get());
                for (int j = 0; j < L_; ++j)
                    if (active_[j] && (j >= (int)bc->lower.size() || j >= (int)bc->upper.size() ||
                                       bc->lower[j] != lower_[j] || bc->upper[j] != upper_[j]))
                        throw std::runtime_error("BoundaryConstraint bounds must be the space's joint limits");
                proj_.use_boundary = 1;
                projectable_ = true;
            }
        }
        std::vector<float> sp, sr, bp, br, bmn, bmx, cp, cr, crad, chei;
        for (auto &c : constraints_) {
            if (c->kind == ConstraintKind::Sphere) {
                auto *e = static_cast<EnvConstraintSphere *>(c.get());
                for (size_t i = 0; i < e->pos.size(); ++i) {
                    sp.insert(sp.end(), e->pos[i].begin(), e->pos[i].begin() + 3);
                    sr.push_back(e->radius[i]);
                }
            } else if (c->kind == ConstraintKind::Cuboid) {
                auto *e = static_cast<EnvConstraintCuboid *>(c.get());
                for (size_t i = 0; i < e->pos.size(); ++i) {
                    bp.insert(bp.end(), e->pos[i].begin(), e->pos[i].begin() + 3);
                    br.insert(br.end(), e->rot[i].begin(), e->rot[i].begin() + 9);
                    bmn.insert(bmn.end(), e->mn[i].begin(), e->mn[i].begin() + 3);
                    bmx.insert(bmx.end(), e->mx[i].begin(), e->mx[i].begin() + 3);
                }
            } else if (c->kind == ConstraintKind::Cylinder) {
                auto *e = static_cast<EnvConstraintCylinder *>(c.get());
                for (size_t i = 0; i < e->pos.size(); ++i) {
                    cp.insert(cp.end(), e->pos[i].begin(), e->pos[i].begin() + 3);
                    cr.insert(cr.end(), e->rot[i].begin(), e->rot[i].begin() + 9);
                    crad.push_back(e->radius[i]);
                    chei.push_back(e->height[i]);
                }
            }
        }
        detail::check(gbmp_env_create((int)sr.size(), sp.data(), sr.data(), (int)bmn.size() / 3, bp.data(), br.data(),
                                      bmn.data(), bmx.data(), (int)crad.size(), cp.data(), cr.data(), crad.data(),
                                      chei.data(), &env_));
    }

    bool projectable_ = false;
    gbmp_projection proj_{};
    size_t dim_;
    std::vector<BaseConstraintPtr> constraints_;
    float resolution_;
    std::vector<std::string> link_names_;
    int L_ = 0, S_ = 0;
    std::vector<int> types_, parent_, slink_;
    std::vector<float> poses_, axes_, spos_, srad_, lower_, upper_, default_;
    std::vector<uint8_t> active_, enables_;
    gbmp_robot robot_ = nullptr;
    gbmp_env env_ = nullptr;
    uint64_t seed_ = 0x5eedULL, offset_ = 0;
};
typedef std::shared_ptr<SingleArmSpace> SingleArmSpacePtr;

// ---------------------------------------------------------------------------------
// SingleArmStates implementation.
// ---------------------------------------------------------------------------------
inline SingleArmStates::SingleArmStates(int n, const SingleArmSpace *space)
    : n_(n), L_(space->getNumOfJoints()), S_(space->numSpheres()), space_(space) {
    q_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)n * L_);
    costs_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)n * std::max(space->numConstraints(), 1));
    total_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)n);
    valid_ = q_->ok() && costs_->ok() && total_->ok();
}

inline void SingleArmStates::update() {
    if (n_ == 0) return;
    poses_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)n_ * L_ * 16);
    centers_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)n_ * S_ * 3);
    if (!poses_->ok() || !centers_->ok()) { valid_ = false; return; }
    detail::check(gbmp_fk(space_->robot(), getJointStatesCuda(), n_, static_cast<float *>(poses_->p),
                          static_cast<float *>(centers_->p), nullptr));
    cudaDeviceSynchronize();
    updated_ = true;
}

inline std::vector<std::vector<float>> SingleArmStates::getJointStatesFullHost() const {
    std::vector<float> flat((size_t)n_ * L_);
    if (n_) cudaMemcpy(flat.data(), q_->p, sizeof(float) * flat.size(), cudaMemcpyDeviceToHost);
    std::vector<std::vector<float>> out(n_);
    for (int i = 0; i < n_; ++i) out[i].assign(flat.begin() + (size_t)i * L_, flat.begin() + (size_t)(i + 1) * L_);
    return out;
}

inline std::vector<std::vector<float>> SingleArmStates::getJointStatesHost() const {
    auto full = getJointStatesFullHost();
    std::vector<std::vector<float>> out;
    for (auto &v : full) {
        std::vector<float> a;
        for (int j = 0; j < L_; ++j)
            if (space_->activeMap()[j]) a.push_back(v[j]);
        out.push_back(a);
    }
    return out;
}

inline std::vector<std::vector<std::vector<float>>> SingleArmStates::getLinkPosesInBaseLinkHost() {
    if (!updated_) update();
    std::vector<float> flat((size_t)n_ * L_ * 16);
    cudaMemcpy(flat.data(), poses_->p, sizeof(float) * flat.size(), cudaMemcpyDeviceToHost);
    std::vector<std::vector<std::vector<float>>> out(n_, std::vector<std::vector<float>>(L_));
    for (int i = 0; i < n_; ++i)
        for (int l = 0; l < L_; ++l)
            out[i][l].assign(flat.begin() + ((size_t)i * L_ + l) * 16, flat.begin() + ((size_t)i * L_ + l + 1) * 16);
    return out;
}

inline std::vector<std::vector<std::vector<float>>> SingleArmStates::getSelfCollisionSpheresPosInBaseLinkHost() {
    if (!updated_) update();
    std::vector<float> flat((size_t)n_ * S_ * 3);
    cudaMemcpy(flat.data(), centers_->p, sizeof(float) * flat.size(), cudaMemcpyDeviceToHost);
    std::vector<std::vector<std::vector<float>>> out(n_, std::vector<std::vector<float>>(S_));
    for (int i = 0; i < n_; ++i)
        for (int k = 0; k < S_; ++k)
            out[i][k].assign(flat.begin() + ((size_t)i * S_ + k) * 3, flat.begin() + ((size_t)i * S_ + k + 1) * 3);
    return out;
}

inline void SingleArmStates::calculateSpaceJacobian(bool synchronize) {
    if (n_ == 0) return;
    jac_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)n_ * L_ * L_ * 6);
    if (!jac_->ok()) { valid_ = false; return; }
    detail::check(gbmp_space_jacobian(space_->robot(), getJointStatesCuda(), n_, static_cast<float *>(jac_->p),
                                      nullptr));
    if (synchronize) cudaDeviceSynchronize();
}

inline std::vector<std::vector<std::vector<float>>>
SingleArmStates::getSpaceJacobianInBaseLinkHost(const std::string &link_name) {
    const int li = space_->getLinkIndex(link_name);
    if (!jac_ && n_) calculateSpaceJacobian(true);
    std::vector<float> flat((size_t)n_ * L_ * L_ * 6);
    if (n_) cudaMemcpy(flat.data(), jac_->p, sizeof(float) * flat.size(), cudaMemcpyDeviceToHost);
    std::vector<std::vector<std::vector<float>>> out(n_, std::vector<std::vector<float>>(L_, std::vector<float>(6)));
    for (int i = 0; i < n_; ++i)
        for (int j = 0; j < L_; ++j)
            for (int k = 0; k < 6; ++k) out[i][j][k] = flat[(((size_t)i * L_ + li) * L_ + j) * 6 + k];
    return out;
}

inline std::vector<float> SingleArmStates::getTotalCostsHost() const {
    std::vector<float> t(n_);
    if (n_) cudaMemcpy(t.data(), total_->p, sizeof(float) * n_, cudaMemcpyDeviceToHost);
    return t;
}

inline std::vector<std::vector<float>> SingleArmStates::getCostsHost() const {
    const int C = space_->numConstraints();
    std::vector<float> flat((size_t)n_ * C);
    if (n_ && C) cudaMemcpy(flat.data(), costs_->p, sizeof(float) * flat.size(), cudaMemcpyDeviceToHost);
    std::vector<std::vector<float>> out(n_, std::vector<float>(C));
    for (int i = 0; i < n_; ++i)
        for (int c = 0; c < C; ++c) out[i][c] = flat[(size_t)c * n_ + i];
    return out;
}

inline void SingleArmStates::filterStates(const std::vector<bool> &filter_map) {
    if ((int)filter_map.size() != n_) throw std::runtime_error("filter map size differs from the number of states");
    auto q = getJointStatesFullHost();
    auto tot = getTotalCostsHost();
    std::vector<float> keep_q, keep_t;
    int m = 0;
    for (int i = 0; i < n_; ++i)
        if (filter_map[i]) {
            keep_q.insert(keep_q.end(), q[i].begin(), q[i].end());
            keep_t.push_back(tot[i]);
            ++m;
        }
    n_ = m;
    q_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)m * L_);
    total_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)m);
    costs_ = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)m * std::max(space_->numConstraints(), 1));
    if (m) {
        cudaMemcpy(q_->p, keep_q.data(), sizeof(float) * keep_q.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(total_->p, keep_t.data(), sizeof(float) * keep_t.size(), cudaMemcpyHostToDevice);
    }
    updated_ = false;
}

// ---------------------------------------------------------------------------------
// State manager: a growable device array of joint vectors.
// ---------------------------------------------------------------------------------
class SingleArmStateManager {
  public:
    explicit SingleArmStateManager(const SingleArmSpace *space) : space_(space), L_(space->getNumOfJoints()) {}
    int get_num_of_states() const { return n_; }
    void clear() { n_ = 0; }

    // Append (SingleArmStates.cu:1101-1169), amortised growth instead of a copy per call.
    std::vector<int> add_states(const BaseStatesPtr &states) {
        const int m = states->getNumOfStates();
        std::vector<int> idx(m);
        if (m == 0) return idx;
        reserve(n_ + m);
        cudaMemcpy(static_cast<float *>(buf_->p) + (size_t)n_ * L_, states->getJointStatesCuda(),
                   sizeof(float) * (size_t)m * L_, cudaMemcpyDeviceToDevice);
        for (int i = 0; i < m; ++i) idx[i] = n_ + i;
        n_ += m;
        return idx;
    }

    // Nearest neighbour per group (SingleArmStates.cu:1338-1431): one gbmp_nearest per group.
    void find_the_nearest_neighbors(const BaseStatesPtr &query_states, const std::vector<std::vector<int>> &group_indexs,
                                    std::vector<std::vector<int>> &neighbors_index) {
        if (n_ == 0) throw std::runtime_error("Error in SingleArmStateManager::find_the_nearest_neighbors: manager is empty");
        const int Q = query_states->getNumOfStates();
        if (Q == 0) throw std::runtime_error("Error in SingleArmStateManager::find_the_nearest_neighbors: query states are empty");
        for (size_t g = 0; g < group_indexs.size(); ++g)
            if (group_indexs[g].empty())
                throw std::runtime_error("Error in SingleArmStateManager::find_the_nearest_neighbors: group " +
                                         std::to_string(g) + " is empty");
        neighbors_index.assign(Q, std::vector<int>(group_indexs.size()));
        detail::DevArray out(sizeof(int) * (size_t)Q);
        std::vector<int> h(Q);
        for (size_t g = 0; g < group_indexs.size(); ++g) {
            detail::DevArray cand(sizeof(int) * group_indexs[g].size());
            cudaMemcpy(cand.p, group_indexs[g].data(), cand.bytes, cudaMemcpyHostToDevice);
            detail::check(gbmp_nearest(space_->robot(), static_cast<float *>(buf_->p), n_, static_cast<int *>(cand.p),
                                       (int64_t)group_indexs[g].size(), query_states->getJointStatesCuda(), Q,
                                       static_cast<int *>(out.p), nullptr));
            cudaMemcpy(h.data(), out.p, sizeof(int) * Q, cudaMemcpyDeviceToHost);
            for (int q = 0; q < Q; ++q) neighbors_index[q][g] = h[q];
        }
    }

    // Gather by index (SingleArmStates.cu:1433-1453): one index upload and one gather
    // launch instead of a copy per index.
    BaseStatesPtr get_states(const std::vector<int> &states_index) {
        auto st = std::make_shared<SingleArmStates>((int)states_index.size(), space_);
        if (states_index.empty()) return st;
        for (int i : states_index)
            if (i < 0 || i >= n_) throw std::runtime_error("state index out of range");
        detail::DevArray idx(sizeof(int) * states_index.size());
        cudaMemcpy(idx.p, states_index.data(), idx.bytes, cudaMemcpyHostToDevice);
        detail::check(gbmp_gather_states(L_, static_cast<float *>(buf_->p), n_, static_cast<int *>(idx.p),
                                         (int64_t)states_index.size(), st->getJointStatesCuda(), nullptr, nullptr));
        cudaDeviceSynchronize();
        return st;
    }

    BaseStatesPtr concatinate_states(const std::vector<BaseStatesPtr> &states) {
        int total = 0;
        for (auto &s : states) total += s->getNumOfStates();
        auto st = std::make_shared<SingleArmStates>(total, space_);
        size_t off = 0;
        for (auto &s : states) {
            cudaMemcpy(st->getJointStatesCuda() + off, s->getJointStatesCuda(),
                       sizeof(float) * (size_t)s->getNumOfStates() * L_, cudaMemcpyDeviceToDevice);
            off += (size_t)s->getNumOfStates() * L_;
        }
        return st;
    }

    // Steer states towards their nearest manager states (SingleArmStates.cu:1524-1557).
    void interpolateToStates(const BaseStatesPtr &states, std::vector<int> &nearest_neighbors_indexes, float max_distance) {
        if (states->getNumOfStates() != (int)nearest_neighbors_indexes.size())
            throw std::runtime_error("Error in SingleArmStateManager::interpolateToStates: the number of states is not "
                                     "equal to the size of nearest_neighbors_indexes");
        detail::DevArray idx(sizeof(int) * nearest_neighbors_indexes.size());
        cudaMemcpy(idx.p, nearest_neighbors_indexes.data(), idx.bytes, cudaMemcpyHostToDevice);
        detail::check(gbmp_steer(space_->robot(), static_cast<float *>(buf_->p), static_cast<int *>(idx.p),
                                 states->getJointStatesCuda(), states->getNumOfStates(), max_distance, nullptr));
        cudaDeviceSynchronize();
    }

  private:
    void reserve(int need) {
        if (need <= cap_) return;
        int cap = std::max(need, std::max(1024, 2 * cap_));
        auto nb = std::make_shared<detail::DevArray>(sizeof(float) * (size_t)cap * L_);
        if (!nb->ok()) throw std::runtime_error("state manager allocation failed");
        if (n_) cudaMemcpy(nb->p, buf_->p, sizeof(float) * (size_t)n_ * L_, cudaMemcpyDeviceToDevice);
        buf_ = nb;
        cap_ = cap;
    }
    const SingleArmSpace *space_;
    int L_, n_ = 0, cap_ = 0;
    std::shared_ptr<detail::DevArray> buf_;
};

inline std::shared_ptr<SingleArmStateManager> SingleArmSpace::createStateManager() {
    return std::make_shared<SingleArmStateManager>(this);
}

}  // namespace CUDAMPLib

// ---------------------------------------------------------------------------------
// CPRRTC::RobotSolver (cudampl/CPRRTC/include/RobotSolver.h:19-164).
// ---------------------------------------------------------------------------------
namespace CPRRTC {

struct Cuboid {
    float x_min, x_max, y_min, y_max, z_min, z_max;
    float x, y, z, roll, pitch, yaw;
};
struct Sphere {
    float x, y, z, radius;
};
struct Cylinder {
    float x, y, z, roll, pitch, yaw, radius, height;
};

class RobotSolver {
  public:
    template <typename Pose, typename Vec, typename SVec>
    RobotSolver(std::string robot_name, size_t dim, const std::vector<int> &joint_types,
                const std::vector<Pose> &joint_poses, const std::vector<Vec> &joint_axes,
                const std::vector<int> &link_parent_link_maps, const std::vector<int> &self_collision_spheres_to_link_map,
                const std::vector<SVec> &self_collision_spheres_pos_in_link,
                const std::vector<float> &self_collision_spheres_radius, const std::vector<bool> &active_joint_map,
                const std::vector<float> &lower, const std::vector<float> &upper,
                const std::vector<float> &default_joint_values, const std::vector<std::string> &link_names,
                const std::vector<std::vector<bool>> &self_collision_enables_map, float resolution = 0.02f)
        : name_(std::move(robot_name)), dim_(dim) {
        std::vector<std::vector<float>> spos;
        for (auto &p : self_collision_spheres_pos_in_link)
            spos.push_back({CUDAMPLib::detail::vec_at(p, 0), CUDAMPLib::detail::vec_at(p, 1), CUDAMPLib::detail::vec_at(p, 2)});
        std::vector<CUDAMPLib::BaseConstraintPtr> cons{std::make_shared<CUDAMPLib::SelfCollisionConstraint>(
            "self", self_collision_spheres_to_link_map, self_collision_spheres_radius, self_collision_enables_map)};
        space_ = std::make_shared<CUDAMPLib::SingleArmSpace>(dim, cons, joint_types, joint_poses, joint_axes,
                                                             link_parent_link_maps, self_collision_spheres_to_link_map,
                                                             spos, self_collision_spheres_radius, active_joint_map, lower,
                                                             upper, default_joint_values, link_names, resolution);
        active_ = active_joint_map;
        default_ = default_joint_values;
        CUDAMPLib::detail::check(gbmp_planner_create(space_->robot(), max_nodes_, 65536, &planner_));
        settings_.lanes = 512;            // RobotSolver.cu:76-78: 512 blocks
        settings_.max_iters = 10000;
        settings_.range = 32 * resolution; // up to 32 states per extension (max_step_)
        settings_.resolution = resolution;
        settings_.step_rule = GBMP_STEP_L2;
        settings_.seed = 1;
        settings_.time_limit_s = 10.0;
    }
    ~RobotSolver() {
        if (planner_) gbmp_planner_destroy(planner_);
        if (env_) gbmp_env_destroy(env_);
    }
    RobotSolver(const RobotSolver &) = delete;
    RobotSolver &operator=(const RobotSolver &) = delete;

    void setEnvObstacleCache(int num_of_spheres, int num_of_cuboids, int num_of_cylinders) {
        max_s_ = num_of_spheres;
        max_b_ = num_of_cuboids;
        max_c_ = num_of_cylinders;
    }

    // Unlike the reference (RobotSolver.cu:391-400, :538), cuboids and cylinders are
    // checked too.
    void updateEnvObstacle(std::vector<Sphere> &spheres, std::vector<Cuboid> &cuboids, std::vector<Cylinder> &cylinders) {
        if ((int)spheres.size() > max_s_ || (int)cuboids.size() > max_b_ || (int)cylinders.size() > max_c_)
            throw std::runtime_error("The number of obstacles exceeds the maximum number of obstacles.");
        std::vector<float> sp, sr, bp, br, bmn, bmx, cp, cr, crad, chei;
        for (auto &s : spheres) { sp.insert(sp.end(), {s.x, s.y, s.z}); sr.push_back(s.radius); }
        for (auto &b : cuboids) {
            float R[9];
            CUDAMPLib::detail::rpy_to_rot(b.roll, b.pitch, b.yaw, R);
            bp.insert(bp.end(), {b.x, b.y, b.z});
            br.insert(br.end(), R, R + 9);
            bmn.insert(bmn.end(), {b.x_min, b.y_min, b.z_min});
            bmx.insert(bmx.end(), {b.x_max, b.y_max, b.z_max});
        }
        for (auto &c : cylinders) {
            float R[9];
            CUDAMPLib::detail::rpy_to_rot(c.roll, c.pitch, c.yaw, R);
            cp.insert(cp.end(), {c.x, c.y, c.z});
            cr.insert(cr.end(), R, R + 9);
            crad.push_back(c.radius);
            chei.push_back(c.height);
        }
        if (env_) gbmp_env_destroy(env_);
        env_ = nullptr;
        CUDAMPLib::detail::check(gbmp_env_create((int)sr.size(), sp.data(), sr.data(), (int)cuboids.size(), bp.data(),
                                                 br.data(), bmn.data(), bmx.data(), (int)crad.size(), cp.data(),
                                                 cr.data(), crad.data(), chei.data(), &env_));
    }

    // Start / goal in active joints; returns the path in active joints, empty on failure.
    std::vector<std::vector<float>> solve(std::vector<float> &start, std::vector<float> &goal) {
        if (start.size() != dim_ || goal.size() != dim_) return {};
        if (!env_) {
            std::vector<Sphere> s;
            std::vector<Cuboid> b;
            std::vector<Cylinder> c;
            setEnvObstacleCache(0, 0, 0);
            updateEnvObstacle(s, b, c);
        }
        const int L = space_->getNumOfJoints();
        std::vector<float> fs(L), fg(L);
        for (int j = 0, k = 0; j < L; ++j) {
            fs[j] = active_[j] ? start[k] : default_[j];
            fg[j] = active_[j] ? goal[k] : default_[j];
            if (active_[j]) ++k;
        }
        std::vector<float> path((size_t)65536 * L);
        gbmp_rrtc_result res{};
        gbmp_status st = gbmp_rrtc_solve(planner_, env_, fs.data(), fg.data(), &settings_, path.data(), 65536, &res, nullptr);
        ++settings_.seed;
        last_ = res;
        if (st != GBMP_OK || !res.solved) return {};
        std::vector<std::vector<float>> out;
        for (int k = 0; k < res.path_len; ++k) {
            std::vector<float> a;
            for (int j = 0; j < L; ++j)
                if (active_[j]) a.push_back(path[(size_t)k * L + j]);
            out.push_back(a);
        }
        return out;
    }

    gbmp_rrtc_settings &settings() { return settings_; }
    const gbmp_rrtc_result &lastResult() const { return last_; }
    CUDAMPLib::SingleArmSpacePtr space() const { return space_; }

  private:
    std::string name_;
    size_t dim_;
    CUDAMPLib::SingleArmSpacePtr space_;
    std::vector<bool> active_;
    std::vector<float> default_;
    gbmp_planner planner_ = nullptr;
    gbmp_env env_ = nullptr;
    int max_s_ = 0, max_b_ = 0, max_c_ = 0;
    int max_nodes_ = 1 << 20;
    gbmp_rrtc_settings settings_{};
    gbmp_rrtc_result last_{};
};
typedef std::shared_ptr<RobotSolver> RobotSolverPtr;

}  // namespace CPRRTC
