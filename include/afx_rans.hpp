// afx_rans.hpp — header-only C++ layer over the C ABI (afx_rans.h) with the
// shape of AeroFLEX's `rans` classes, so callers written against
// src/rans/include/rans/rans.h keep their call order: Settings from an INI
// file, compute_alphas(), input(), solve_airfoil(name, db), get_wall_profile.
// Errors are re-thrown as std::runtime_error (the reference throws from
// tiny::config / Settings / mesh, tinyconfig.hpp:86-92, core.h:239, mesh.h:154).
//
// Differences from the reference, all deliberate:
//  * both solvers run on the GPU; `solver = implicit` (the reference's
//    default, core.h:178) uses the library's block-Jacobian GMRES in place of
//    Eigen's ILUT-preconditioned GMRES, so its iterates differ while its
//    converged solution is the same;
//  * mesh paths come from the caller (rans.h:84-85 hard-code
//    "../../../../examples/rans/<name>_coarse.msh" and "_mid.msh"); pass
//    both to solve_airfoil for the reference's two-level sequence;
//  * the VTU file of every angle (rans.h:103) is written when solve_airfoil
//    is given a file prefix (the reference always writes it).
#pragma once

#include <atomic>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "afx_rans.h"

namespace rans {

inline void afx_check(int rc) {
    if (rc != AFX_OK) throw std::runtime_error(std::string("[RANS] ") + afx_last_error());
}

// database::airfoil (src/common/database/database.hpp:17-60): polar storage.
struct airfoil_db {
    std::vector<double> alpha, cl, cd, cmy;
};

// rans::Settings (core.h:166-232) as an owning handle over afx_config.
class Settings {
  public:
    Settings() { afx_check(afx_config_create(&h_)); }
    explicit Settings(const std::string& ini_path) { afx_check(afx_config_from_ini(ini_path.c_str(), &h_)); }
    ~Settings() { afx_config_free(h_); }
    Settings(const Settings&) = delete;
    Settings& operator=(const Settings&) = delete;

    // Settings::import_config_file (core.h:238-272)
    void import_config_file(const std::string& ini_path) {
        afx_config c;
        afx_check(afx_config_from_ini(ini_path.c_str(), &c));
        afx_config_free(h_);
        h_ = c;
    }
    double get(const std::string& k) const {
        double v = 0;
        afx_check(afx_config_get_double(h_, k.c_str(), &v));
        return v;
    }
    std::string get_string(const std::string& k) const {
        char buf[256];
        afx_check(afx_config_get_string(h_, k.c_str(), buf, sizeof buf));
        return buf;
    }
    void set(const std::string& k, double v) { afx_check(afx_config_set_double(h_, k.c_str(), v)); }
    void set(const std::string& k, const std::string& v) { afx_check(afx_config_set_string(h_, k.c_str(), v.c_str())); }
    void set_bc(const std::string& name, const std::string& type, double T = 1, double mach = 0.2, double angle = 0,
                double p = 1) {
        afx_check(afx_config_set_bc(h_, name.c_str(), type.c_str(), T, mach, angle, p));
    }
    // bcs[name].vars_far (core.h:112-115): {T, mach, angle, p}
    std::vector<double> bc_vars(const std::string& name) const {
        std::vector<double> v(4);
        afx_check(afx_config_get_bc(h_, name.c_str(), nullptr, 0, &v[0], &v[1], &v[2], &v[3]));
        return v;
    }
    afx_config handle() const { return h_; }

  private:
    afx_config h_ = nullptr;
};

// rans::mesh (mesh.h:198-273)
class mesh {
  public:
    explicit mesh(const std::string& filename) { afx_check(afx_mesh_load(filename.c_str(), &h_)); }
    ~mesh() { afx_mesh_free(h_); }
    mesh(const mesh&) = delete;
    mesh& operator=(const mesh&) = delete;
    mesh(mesh&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
    long long nRealCells() const { return counts()[0]; }
    long long nEdges() const { return counts()[2]; }
    afx_mesh handle() const { return h_; }

  private:
    std::vector<long long> counts() const {
        std::vector<long long> c(5);
        afx_check(afx_mesh_counts(h_, c.data()));
        return c;
    }
    afx_mesh h_ = nullptr;
};

// post.h:41-55
struct wallProfile {
    std::vector<double> cp;
    double cd = 0., cl = 0., cm = 0.;
};

// explicitSolver + multigrid::run_solver on the GPU
class solver {
  public:
    solver(const mesh& m, const Settings& s) { afx_check(afx_solver_create(m.handle(), s.handle(), &h_)); }
    ~solver() { afx_solver_free(h_); }
    solver(const solver&) = delete;
    solver& operator=(const solver&) = delete;
    void init() { afx_check(afx_init_freestream(h_)); }                     // solver.h:615
    double solve(int n = 1) {                                               // solver.h:802
        double r = 0;
        afx_check(afx_iterate(h_, n, &r));
        return r;
    }
    int run_solver(double tol = 0, int max_it = 0) {                        // multigrid.h:182
        int it = 0;
        double err = 0;
        afx_check(afx_run_to_convergence(h_, tol, max_it, &it, &err));
        return it;
    }
    std::vector<double> residual_history() const {
        int n = 0;
        afx_check(afx_residual_history(h_, nullptr, 0, &n));
        std::vector<double> out(n);
        afx_check(afx_residual_history(h_, out.data(), n, &n));
        return out;
    }
    void set_farfield(const std::string& patch, double mach, double angle, double T = 1, double p = 1) {
        afx_check(afx_set_farfield(h_, patch.c_str(), mach, angle, T, p));
    }
    void request_stop() { afx_request_stop(h_); }
    // multigrid::run's level transfer (multigrid.h:316-321)
    void prolongate_from(solver& coarse) { afx_check(afx_prolongate(coarse.h_, h_)); }
    afx_solver handle() const { return h_; }

  private:
    afx_solver h_ = nullptr;
};

// get_wall_profile (post.h:301-387)
inline wallProfile get_wall_profile(solver& s, const std::string& patch_name) {
    wallProfile w;
    int n = 0;
    afx_check(afx_forces(s.handle(), patch_name.c_str(), &w.cl, &w.cd, &w.cm, nullptr, 0, &n));
    w.cp.resize(n);
    afx_check(afx_forces(s.handle(), patch_name.c_str(), &w.cl, &w.cd, &w.cm, w.cp.data(), n, &n));
    return w;
}

// save (post.h:58-180): the ASCII VTU file of the solver's state
inline void save(const std::string& filename, solver& s) { afx_check(afx_save_vtu(s.handle(), filename.c_str())); }

// rans::Rans (rans.h:25-123): alpha sweep with warm restarts.
class Rans {
  public:
    Settings settings;
    std::vector<double> residuals;
    std::atomic<int> iters{0};
    std::vector<double> alphas;
    std::vector<std::string> meshes;  // the last one is solved

    // rans.h:53-57
    void compute_alphas() {
        alphas.clear();
        for (double a = settings.get("alpha_start"); a <= settings.get("alpha_end"); a += settings.get("alpha_step"))
            alphas.push_back(a);
    }
    // rans.h:59-66
    void input() {
        if (!loaded_ && !meshes.empty()) {
            mesh_.reset(new mesh(meshes.back()));
            loaded_ = true;
        }
    }
    // rans.h:78-106 / 116-123: the farfield angle is alpha * 0.01745
    // (rans.h:88,94); for every angle the levels run in order, each finer
    // level starting from the coarser one's solution (multigrid::run,
    // multigrid.h:295-363), and every level keeps its own state from one
    // angle to the next (run(false)).  The polar is read on the last level.
    // vtu_prefix non-empty: the VTU file of the last level after every angle,
    // named prefix + "_" + std::to_string(alpha) + ".vtu" (rans.h:103)
    void solve_airfoil(const std::vector<std::string>& level_paths, airfoil_db& db,
                       const std::string& farfield = "farfield", const std::string& wall = "wall",
                       const std::string& vtu_prefix = "") {
        if (level_paths.empty()) throw std::runtime_error("[RANS] no mesh");
        iters = 0;
        if (alphas.empty()) compute_alphas();
        levels_.clear();
        meshes_.clear();
        for (const auto& p : level_paths) {
            meshes_.emplace_back(new mesh(p));
            levels_.emplace_back(new solver(*meshes_.back(), settings));
        }
        const std::vector<double> v = settings.bc_vars(farfield);  // T, mach, angle, p
        levels_[0]->set_farfield(farfield, v[1], alphas.front() * 0.01745, v[0], v[3]);
        levels_[0]->init();
        for (double a : alphas) {
            for (auto& s : levels_) s->set_farfield(farfield, v[1], a * 0.01745, v[0], v[3]);
            for (size_t i = 0; i < levels_.size(); ++i) {
                if (i > 0) levels_[i]->prolongate_from(*levels_[i - 1]);
                iters += levels_[i]->run_solver();
                for (double r : levels_[i]->residual_history()) residuals.push_back(r);
            }
            wallProfile wp = get_wall_profile(*levels_.back(), wall);
            db.alpha.push_back(a);
            db.cl.push_back(wp.cl);
            db.cd.push_back(wp.cd);
            db.cmy.push_back(wp.cm);
            if (!vtu_prefix.empty()) save(vtu_prefix + "_" + std::to_string(a) + ".vtu", *levels_.back());
        }
    }
    void solve_airfoil(const std::string& mesh_path, airfoil_db& db, const std::string& farfield = "farfield",
                       const std::string& wall = "wall", const std::string& vtu_prefix = "") {
        solve_airfoil(std::vector<std::string>{mesh_path}, db, farfield, wall, vtu_prefix);
    }

  private:
    std::unique_ptr<mesh> mesh_;
    std::vector<std::unique_ptr<mesh>> meshes_;
    std::vector<std::unique_ptr<solver>> levels_;
    bool loaded_ = false;
};

}  // namespace rans
