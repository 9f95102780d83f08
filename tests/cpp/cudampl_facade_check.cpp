// Drives the C++ facade (gbmp_cudampl.hpp) the way the reference's own callers drive
// CUDAMPLib::SingleArmSpace and CPRRTC::RobotSolver, and writes every result to a text
// file that tests/test_cudampl_facade.py compares with the oracle.
//
// usage: cudampl_facade_check <problem.txt> <results.txt>
#include <cstdio>
#include <fstream>
#include <iostream>

#include "gbmp_cudampl_rrg.hpp"

namespace {

// Pose type with the Eigen::Isometry3d access pattern (.matrix()(r, c)).
struct MiniIsometry {
    struct M {
        double d[16];
        double operator()(int r, int c) const { return d[r * 4 + c]; }
    } m;
    const M &matrix() const { return m; }
};
// Vector type with the Eigen::Vector3d access pattern (v(i)).
struct MiniVec3 {
    double d[3];
    double operator()(int i) const { return d[i]; }
};

struct Reader {
    std::ifstream in;
    explicit Reader(const char *p) : in(p) {
        if (!in) throw std::runtime_error(std::string("cannot open ") + p);
    }
    int i() { int v; in >> v; return v; }
    float f() { float v; in >> v; return v; }
    std::vector<int> iv(size_t n) { std::vector<int> v(n); for (auto &x : v) x = i(); return v; }
    std::vector<float> fv(size_t n) { std::vector<float> v(n); for (auto &x : v) x = f(); return v; }
    std::vector<std::vector<float>> rows(size_t n, size_t w) {
        std::vector<std::vector<float>> r(n);
        for (auto &x : r) x = fv(w);
        return r;
    }
};

struct Writer {
    FILE *fp;
    explicit Writer(const char *p) : fp(std::fopen(p, "w")) {
        if (!fp) throw std::runtime_error(std::string("cannot write ") + p);
    }
    ~Writer() { std::fclose(fp); }
    void head(const char *name, size_t n) { std::fprintf(fp, "%s %zu\n", name, n); }
    void put(float v) { std::fprintf(fp, "%.9g ", v); }
    void put(int v) { std::fprintf(fp, "%d ", v); }
    void end() { std::fprintf(fp, "\n"); }
    template <typename T>
    void flat(const char *name, const std::vector<T> &v) {
        head(name, v.size());
        for (auto x : v) put(x);
        end();
    }
};

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s problem.txt results.txt\n", argv[0]);
        return 2;
    }
    try {
        Reader in(argv[1]);
        const int L = in.i(), dim = in.i(), S = in.i();
        auto types = in.iv(L);
        auto poses = in.fv((size_t)L * 16);
        auto axes = in.fv((size_t)L * 3);
        auto parent = in.iv(L);
        auto slink = in.iv(S);
        auto spos = in.rows(S, 3);
        auto srad = in.fv(S);
        auto act = in.iv(L);
        auto lower = in.fv(L), upper = in.fv(L), defv = in.fv(L);
        auto en = in.iv((size_t)L * L);
        const float res = in.f();
        const int ns = in.i();
        auto sp = in.rows(ns, 3);
        auto sr = in.fv(ns);
        const int nb = in.i();
        auto bp = in.rows(nb, 3), brot = in.rows(nb, 9), bmn = in.rows(nb, 3), bmx = in.rows(nb, 3);
        const int nc = in.i();
        auto cp = in.rows(nc, 3), crot = in.rows(nc, 9);
        auto crad = in.fv(nc), chei = in.fv(nc);
        const int n = in.i();
        auto states = in.rows(n, dim);
        const int m = in.i();
        auto e_from = in.rows(m, dim), e_to = in.rows(m, dim);
        const int nq = in.i();
        auto queries = in.rows(nq, dim);
        auto start = in.fv(dim), goal = in.fv(dim);
        const int nshelf = in.i();
        auto shelf_p = in.rows(nshelf, 3), shelf_mn = in.rows(nshelf, 3), shelf_mx = in.rows(nshelf, 3);
        const int region_link = in.i();
        auto region_ref = in.fv(6), region_tol = in.fv(6);

        std::vector<bool> active(L);
        for (int j = 0; j < L; ++j) active[j] = act[j] != 0;
        std::vector<std::vector<bool>> enables(L, std::vector<bool>(L));
        for (int a = 0; a < L; ++a)
            for (int b = 0; b < L; ++b) enables[a][b] = en[a * L + b] != 0;
        std::vector<std::array<float, 16>> pose_arr(L);
        std::vector<std::array<float, 3>> axis_arr(L);
        std::vector<MiniIsometry> pose_iso(L);
        std::vector<MiniVec3> axis_v(L);
        for (int j = 0; j < L; ++j) {
            for (int k = 0; k < 16; ++k) pose_arr[j][k] = poses[j * 16 + k], pose_iso[j].m.d[k] = poses[j * 16 + k];
            for (int k = 0; k < 3; ++k) axis_arr[j][k] = axes[j * 3 + k], axis_v[j].d[k] = axes[j * 3 + k];
        }
        std::vector<std::string> names(L);
        for (int j = 0; j < L; ++j) names[j] = "link" + std::to_string(j);

        // ---- SingleArmSpace with the four collision constraints ----
        std::vector<CUDAMPLib::BaseConstraintPtr> cons;
        cons.push_back(std::make_shared<CUDAMPLib::SelfCollisionConstraint>("self_collision_constraint", slink, srad,
                                                                            enables));
        cons.push_back(std::make_shared<CUDAMPLib::EnvConstraintSphere>("obstacle_sphere", sp, sr));
        cons.push_back(std::make_shared<CUDAMPLib::EnvConstraintCuboid>("obstacle_cuboid", bp, brot, bmx, bmn));
        cons.push_back(std::make_shared<CUDAMPLib::EnvConstraintCylinder>("obstacle_cylinder", cp, crot, crad, chei));
        auto space = std::make_shared<CUDAMPLib::SingleArmSpace>(dim, cons, types, pose_arr, axis_arr, parent, slink,
                                                                 spos, srad, active, lower, upper, defv, names, res);
        Writer out(argv[2]);

        auto st = space->createStatesFromVector(states);
        std::vector<bool> feas;
        space->checkStates(st, feas);
        std::vector<int> fi(feas.begin(), feas.end());
        out.flat("feasible", fi);
        out.flat("total", st->getTotalCostsHost());
        std::vector<float> costs;
        for (auto &row : st->getCostsHost()) costs.insert(costs.end(), row.begin(), row.end());
        out.flat("costs", costs);
        std::vector<float> lp;
        for (auto &state : st->getLinkPosesInBaseLinkHost())
            for (auto &pose : state) lp.insert(lp.end(), pose.begin(), pose.end());
        out.flat("poses", lp);
        // space Jacobian of the last link, and an unknown link name rejected
        st->calculateSpaceJacobian();
        std::vector<float> jl;
        for (auto &state : st->getSpaceJacobianInBaseLinkHost("link" + std::to_string(L - 1)))
            for (auto &col : state) jl.insert(jl.end(), col.begin(), col.end());
        out.flat("jacobian_last", jl);
        bool threw = false;
        try {
            st->getSpaceJacobianInBaseLinkHost("no_such_link");
        } catch (const std::runtime_error &) {
            threw = true;
        }
        if (!threw) throw std::runtime_error("unknown link name accepted");

        auto s1 = space->createStatesFromVector(e_from), s2 = space->createStatesFromVector(e_to);
        std::vector<bool> mf;
        std::vector<float> mc;
        if (!space->checkMotions(s1, s2, mf, mc)) throw std::runtime_error("checkMotions failed");
        std::vector<int> mfi(mf.begin(), mf.end());
        out.flat("motion_ok", mfi);
        out.flat("motion_cost", mc);

        auto smp = space->sample(64);
        std::vector<float> sf;
        for (auto &row : smp->getJointStatesFullHost()) sf.insert(sf.end(), row.begin(), row.end());
        out.flat("sample", sf);

        // ---- state manager: add + nearest neighbour over one group of every state ----
        auto mgr = space->createStateManager();
        auto idx = mgr->add_states(st);
        auto qs = space->createStatesFromVector(queries);
        std::vector<std::vector<int>> nbr;
        mgr->find_the_nearest_neighbors(qs, {idx}, nbr);
        std::vector<int> nn;
        for (auto &r : nbr) nn.push_back(r[0]);
        out.flat("nearest", nn);

        // ---- state manager: gather by index (get_states), unordered and repeated ----
        std::vector<int> pos, pick;
        for (int k = (int)idx.size() - 1; k >= 0; k -= 3) pos.push_back(k);
        pos.push_back(0);
        pos.push_back(0);
        for (int k : pos) pick.push_back(idx[k]);
        auto gathered = mgr->get_states(pick)->getJointStatesFullHost();
        auto stored = st->getJointStatesFullHost();
        std::vector<int> gather_ok{(int)(gathered.size() == pos.size())};
        for (size_t k = 0; gather_ok[0] && k < pos.size(); ++k) gather_ok[0] = gathered[k] == stored[pos[k]];
        out.flat("gather_ok", gather_ok);

        // ---- CPRRTC::RobotSolver in the shelf scene ----
        std::vector<MiniVec3> spos_v(S);
        for (int k = 0; k < S; ++k)
            for (int c = 0; c < 3; ++c) spos_v[k].d[c] = spos[k][c];
        CPRRTC::RobotSolver solver("arm", dim, types, pose_iso, axis_v, parent, slink, spos_v, srad, active, lower,
                                   upper, defv, names, enables, res);
        std::vector<CPRRTC::Sphere> spheres;
        std::vector<CPRRTC::Cuboid> cuboids;
        std::vector<CPRRTC::Cylinder> cylinders;
        for (int k = 0; k < nshelf; ++k)
            cuboids.push_back({shelf_mn[k][0], shelf_mx[k][0], shelf_mn[k][1], shelf_mx[k][1], shelf_mn[k][2],
                               shelf_mx[k][2], shelf_p[k][0], shelf_p[k][1], shelf_p[k][2], 0.f, 0.f, 0.f});
        solver.setEnvObstacleCache(0, nshelf, 0);
        solver.updateEnvObstacle(spheres, cuboids, cylinders);
        auto path = solver.solve(start, goal);
        std::vector<float> pf;
        for (auto &row : path) pf.insert(pf.end(), row.begin(), row.end());
        out.flat("path", pf);

        // ---- RRG (RRG.cpp) over a space whose constraints are the shelf boxes ----
        std::vector<CUDAMPLib::BaseConstraintPtr> shelf_cons;
        shelf_cons.push_back(std::make_shared<CUDAMPLib::SelfCollisionConstraint>("self_collision_constraint", slink,
                                                                                  srad, enables));
        std::vector<std::vector<float>> eye(nshelf, std::vector<float>{1, 0, 0, 0, 1, 0, 0, 0, 1});
        shelf_cons.push_back(
            std::make_shared<CUDAMPLib::EnvConstraintCuboid>("shelf", shelf_p, eye, shelf_mx, shelf_mn));
        auto shelf_space = std::make_shared<CUDAMPLib::SingleArmSpace>(dim, shelf_cons, types, pose_arr, axis_arr,
                                                                       parent, slink, spos, srad, active, lower,
                                                                       upper, defv, names, res);
        CUDAMPLib::RRG rrg(shelf_space);
        auto task = std::make_shared<CUDAMPLib::SingleArmTask>(std::vector<std::vector<float>>{start},
                                                               std::vector<std::vector<float>>{goal});
        rrg.setMotionTask(task);
        rrg.solve(std::make_shared<CUDAMPLib::TimeoutTermination>(30.f));
        std::vector<float> rf;
        for (auto &row : task->getSolution()) rf.insert(rf.end(), row.begin(), row.end());
        out.flat("rrg_path", rf);
        out.flat("rrg_vertices", std::vector<int>{rrg.getNumOfVertices()});

        // ---- goal region (SingleArmTask.cpp:12-39): task-space + joint-limit constraints ----
        std::vector<CUDAMPLib::BaseConstraintPtr> gcons;
        gcons.push_back(std::make_shared<CUDAMPLib::SelfCollisionConstraint>("self_collision_constraint", slink, srad,
                                                                             enables));
        gcons.push_back(std::make_shared<CUDAMPLib::EnvConstraintSphere>("obstacle_sphere", sp, sr));
        gcons.push_back(std::make_shared<CUDAMPLib::EnvConstraintCuboid>("obstacle_cuboid", bp, brot, bmx, bmn));
        gcons.push_back(std::make_shared<CUDAMPLib::EnvConstraintCylinder>("obstacle_cylinder", cp, crot, crad, chei));
        const std::array<float, 16> ident{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        gcons.push_back(std::make_shared<CUDAMPLib::TaskSpaceConstraint>("goal_region", region_link, ident, region_ref,
                                                                         region_tol));
        gcons.push_back(std::make_shared<CUDAMPLib::BoundaryConstraint>("boundary", lower, upper, active));
        auto region = std::make_shared<CUDAMPLib::SingleArmSpace>(dim, gcons, types, pose_arr, axis_arr, parent, slink,
                                                                  spos, srad, active, lower, upper, defv, names, res);
        CUDAMPLib::SingleArmTask gtask(std::vector<std::vector<float>>{start}, region, 256);
        std::vector<float> gf;
        for (auto &row : gtask.getGoalStatesVector()) gf.insert(gf.end(), row.begin(), row.end());
        out.flat("region_goals", gf);
        // constrained motions between region goals, and a path through three of them
        // (checkConstrainedMotions / getConstrainedPathFromWaypoints)
        const auto &gv = gtask.getGoalStatesVector();
        const size_t nm = std::min<size_t>(16, gv.size() > 1 ? gv.size() - 1 : 0);
        if (nm > 0) {
            std::vector<std::vector<float>> a(gv.begin(), gv.begin() + nm), b(gv.begin() + 1, gv.begin() + nm + 1);
            std::vector<bool> cm_ok;
            std::vector<float> cm_cost;
            region->checkMotions(region->createStatesFromVector(a), region->createStatesFromVector(b), cm_ok, cm_cost);
            std::vector<int> oki(cm_ok.begin(), cm_ok.end());
            out.flat("region_motion_ok", oki);
            out.flat("region_motion_cost", cm_cost);
            std::vector<std::vector<float>> wp(gv.begin(), gv.begin() + std::min<size_t>(3, gv.size()));
            auto rp = region->getPathFromWaypoints(region->createStatesFromVector(wp));
            std::vector<float> rf2;
            if (rp)
                for (auto &row : rp->getJointStatesHost()) rf2.insert(rf2.end(), row.begin(), row.end());
            out.flat("region_path", rf2);
        }
        std::printf("facade ok: %d states, %d edges, path of %zu waypoints, RRG path of %zu states (%s), %zu region "
                    "goals\n", n, m, path.size(), task->getSolution().size(), task->getFailureReason().c_str(),
                    gtask.getGoalStatesVector().size());
        return 0;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
