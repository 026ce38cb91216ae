// C API over the reference's OWN rans code (test infrastructure only).
//
// This file is compiled together with the unmodified reference headers
// src/rans/include/rans/{core,mesh,physics,solver,multigrid,post}.h, read
// where they lie (recipe: oracle/build_ref.py), and with the Eigen-API
// stand-in in oracle/eigen_api.  The library it makes, oracle/_ref/libref.so,
// runs the reference's own mesh reader, metrics, fluxes, gradients, limiters,
// explicit and implicit solvers, run_solver loops and get_wall_profile; the
// tests use it to pin the oracle restatement (oracle/rans_oracle.cpp) and the
// committed golden fixtures to the reference itself.
//
// Build choices, each because the reference's sources call for it:
// - <math.h> and <stdlib.h> come first.  The reference calls unqualified
//   abs() on doubles (mesh.h:435,442; solver.h:335-336,344; physics.h:554,
//   566); with these headers seen first that is the double overload, the
//   semantics under which the reference's solver runs at all (an integer abs
//   would truncate every cell area below 1 to 0).
// - RANS_DEBUG_PUBLIC, the reference's own switch (solver.h:44-48), makes the
//   solver's state and steps (q, qW, dt, gx, gy, limiters, calc_dt,
//   calc_gradients, calc_limiters, ...) public.  The few members that stay
//   private (explicitSolver::qk and calc_residual, implicitSolver::RhoVector
//   and fillRhoRHS) are reached through the explicit-instantiation access rule
//   ([temp.spec] allows naming private members in an explicit instantiation).
// - No FMA contraction (-ffp-contract=off): the arithmetic of an x86-64
//   release build of the reference, which has no FMA instructions.
// - std::cout is silenced during solver calls (run_solver prints a line per
//   iteration).
#include <math.h>
#include <stdlib.h>

#include <atomic>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#define RANS_DEBUG_PUBLIC
#include <rans/multigrid.h>
#include <rans/post.h>

namespace {

// Access to the private members named above.
template <typename Tag, typename Tag::type M>
struct Expose {
    friend typename Tag::type member(Tag) { return M; }
};
struct ExQk {
    typedef Eigen::VectorXd rans::explicitSolver::*type;
    friend type member(ExQk);
};
template struct Expose<ExQk, &rans::explicitSolver::qk>;
struct ExCalcResidual {
    typedef void (rans::explicitSolver::*type)(const Eigen::VectorXd&);
    friend type member(ExCalcResidual);
};
template struct Expose<ExCalcResidual, &rans::explicitSolver::calc_residual>;
struct ImRhs {
    typedef Eigen::VectorXd rans::implicitSolver::*type;
    friend type member(ImRhs);
};
template struct Expose<ImRhs, &rans::implicitSolver::RhoVector>;
struct ImFillRhs {
    typedef void (rans::implicitSolver::*type)();
    friend type member(ImFillRhs);
};
template struct Expose<ImFillRhs, &rans::implicitSolver::fillRhoRHS>;
struct ImMatrix {
    typedef Eigen::SparseMatrix<double, Eigen::RowMajor> rans::implicitSolver::*type;
    friend type member(ImMatrix);
};
template struct Expose<ImMatrix, &rans::implicitSolver::RhoMatrix>;
struct ImFillLhs {
    typedef void (rans::implicitSolver::*type)();
    friend type member(ImFillLhs);
};
template struct Expose<ImFillLhs, &rans::implicitSolver::fillRhoLHS>;

thread_local std::string g_err;

struct Quiet {  // silences std::cout for the lifetime of the object
    std::ostringstream sink;
    std::streambuf* old;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};

// One run of the reference's driver objects: Settings from an INI file,
// the meshes of the grid-sequencing levels, and the multigrid object that
// owns one solver per level (multigrid.h:58-97).
struct Case {
    rans::Settings st;
    GUIHandler gui;
    std::vector<double> residuals = {1.0};
    std::atomic<int> iters{0};
    rans::CpProfile profile;
    bool implicit = false;
    std::unique_ptr<rans::multigrid<rans::explicitSolver>> ex;
    std::unique_ptr<rans::multigrid<rans::implicitSolver>> im;

    rans::solver& level(int i) {
        if (implicit) return im->solvers.at((size_t)i);
        return ex->solvers.at((size_t)i);
    }
    int n_levels() const { return implicit ? (int)im->solvers.size() : (int)ex->solvers.size(); }
};

template <typename F>
int guarded(F f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

std::vector<std::string> split_lines(const char* s) {
    std::vector<std::string> out;
    std::string cur;
    for (const char* p = s; *p; ++p) {
        if (*p == '\n') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur += *p;
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

const std::vector<double>* mesh_array(rans::mesh& m, const std::string& w) {
    if (w == "cx") return &m.cellsCentersX;
    if (w == "cy") return &m.cellsCentersY;
    if (w == "area") return &m.cellsAreas;
    if (w == "ex") return &m.edgesCentersX;
    if (w == "ey") return &m.edgesCentersY;
    if (w == "nx") return &m.edgesNormalsX;
    if (w == "ny") return &m.edgesNormalsY;
    if (w == "L") return &m.edgesLengths;
    if (w == "wall_dist") return &m.wall_dist;
    if (w == "node_x") return &m.nodesX;
    if (w == "node_y") return &m.nodesY;
    return nullptr;
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

// ----------------------------------------------------------------- mesh
// rans::mesh(filename) (mesh.h:250): the reference's gmsh 4.1 reader.
void* ref_mesh_load(const char* path) {
    rans::mesh* m = nullptr;
    if (guarded([&] {
            Quiet q;
            m = new rans::mesh(std::string(path));
        }))
        return nullptr;
    return m;
}

void ref_mesh_free(void* m) { delete (rans::mesh*)m; }

void ref_mesh_counts(void* mp, long long* out) {
    auto* m = (rans::mesh*)mp;
    out[0] = m->nRealCells;
    out[1] = (long long)m->cellsAreas.size();
    out[2] = (long long)m->edgesCells.cols();
    out[3] = (long long)m->boundaryEdges.size();
    out[4] = (long long)m->nodesX.size();
}

long long ref_mesh_get(void* mp, const char* what, double* out) {
    const std::vector<double>* v = mesh_array(*(rans::mesh*)mp, what);
    if (!v) return -1;
    if (out) std::memcpy(out, v->data(), v->size() * sizeof(double));
    return (long long)v->size();
}

long long ref_mesh_get_int(void* mp, const char* what, long long* out) {
    auto* m = (rans::mesh*)mp;
    std::string w(what);
    if (w == "edges_cells" || w == "edges_nodes") {
        auto& a = w == "edges_cells" ? m->edgesCells : m->edgesNodes;
        if (out)
            for (uint e = 0; e < a.cols(); ++e) {
                out[2 * e] = a(e, 0);
                out[2 * e + 1] = a(e, 1);
            }
        return 2 * (long long)a.cols();
    }
    if (w == "boundary_edges") {
        if (out)
            for (size_t b = 0; b < m->boundaryEdges.size(); ++b) out[b] = m->boundaryEdges[b];
        return (long long)m->boundaryEdges.size();
    }
    if (w == "cells_nodes") {  // 4 per real cell, -1 in slot 3 of a triangle
        if (out)
            for (uint c = 0; c < m->nRealCells; ++c)
                for (uint k = 0; k < 4; ++k)
                    out[4 * c + k] = (k == 3 && m->cellsIsTriangle[c]) ? -1 : (long long)m->cellsNodes(c, k);
        return 4 * (long long)m->nRealCells;
    }
    if (w == "boundary_nodes") {  // node pairs of the boundary edges, in file order
        if (out)
            for (size_t b = 0; b < m->boundaryEdges0.size(); ++b) {
                out[2 * b] = m->boundaryEdges0[b];
                out[2 * b + 1] = m->boundaryEdges1[b];
            }
        return 2 * (long long)m->boundaryEdges0.size();
    }
    return -1;
}

const char* ref_mesh_boundary_name(void* mp, int b) {
    return ((rans::mesh*)mp)->boundaryEdgesPhysicals.at((size_t)b).c_str();
}

// ----------------------------------------------------------------- case
// Settings::import_config_file (core.h:238-272) of the INI file, the meshes
// ('\n'-separated paths, coarse to fine) and the multigrid object of the
// solver type the INI names.  mu_L > 0 replaces the gas viscosity (the INI
// cannot set it, core.h:27-46).
void* ref_case_create(const char* ini_path, const char* mesh_paths, double mu_L) {
    Case* c = nullptr;
    if (guarded([&] {
            Quiet q;
            auto cs = std::make_unique<Case>();
            tiny::config io;
            io.read(ini_path);
            cs->st.import_config_file(io);
            if (mu_L > 0) cs->st.g.mu_L = mu_L;
            std::vector<rans::mesh> ms;
            for (const auto& p : split_lines(mesh_paths)) ms.push_back(rans::mesh(p));
            if (ms.empty()) throw std::invalid_argument("no mesh");
            cs->implicit = cs->st.solver_type() == "implicit";
            if (cs->implicit)
                cs->im.reset(new rans::multigrid<rans::implicitSolver>(ms, cs->st, cs->gui, cs->residuals, cs->iters,
                                                                       cs->profile));
            else
                cs->ex.reset(new rans::multigrid<rans::explicitSolver>(ms, cs->st, cs->gui, cs->residuals, cs->iters,
                                                                       cs->profile));
            c = cs.release();
        }))
        return nullptr;
    return c;
}

void ref_case_free(void* c) { delete (Case*)c; }

int ref_case_levels(void* cp, int* implicit) {
    auto* c = (Case*)cp;
    if (implicit) *implicit = c->implicit ? 1 : 0;
    return c->n_levels();
}

// solver::init + refill_bcs (solver.h:615-632, 259-274), as run() starts.
int ref_init(void* cp, int lvl) {
    return guarded([&] {
        auto& s = ((Case*)cp)->level(lvl);
        s.init();
        s.refill_bcs();
    });
}

int ref_refill_bcs(void* cp, int lvl) { return guarded([&] { ((Case*)cp)->level(lvl).refill_bcs(); }); }

// The real-cell entries of q (4 per cell, AoS).
int ref_set_q(void* cp, int lvl, const double* q_real) {
    return guarded([&] {
        auto& s = ((Case*)cp)->level(lvl);
        std::memcpy(s.q.data(), q_real, 4 * (size_t)s.m.nRealCells * sizeof(double));
    });
}

// Copies a solver vector: q, qW, dt, gx, gy, lim, and for the implicit
// solver rhs (RhoVector); returns its length or -1.
long long ref_get(void* cp, int lvl, const char* what, double* out) {
    auto* c = (Case*)cp;
    auto& s = c->level(lvl);
    std::string w(what);
    const Eigen::VectorXd* v = nullptr;
    if (w == "q") v = &s.q;
    else if (w == "qW") v = &s.qW;
    else if (w == "dt") v = &s.dt;
    else if (w == "gx") v = &s.gx;
    else if (w == "gy") v = &s.gy;
    else if (w == "lim") v = &s.limiters;
    else if (w == "rhs" && c->implicit) v = &(c->im->solvers.at((size_t)lvl).*member(ImRhs()));
    if (!v) return -1;
    if (out) std::memcpy(out, v->data(), (size_t)v->size() * sizeof(double));
    return (long long)v->size();
}

long long ref_wall_distance(void* cp, int lvl, double* out) {
    auto& m = ((Case*)cp)->level(lvl).m;
    if (out) std::memcpy(out, m.wall_dist.data(), m.wall_dist.size() * sizeof(double));
    return (long long)m.wall_dist.size();
}

// Explicit solver: the residual of the current state as the first stage of
// explicitSolver::solve forms it (solver.h:802-817 with qk = q): time step,
// wall ghosts, gradients, limiters, calc_residual.  R_out gets the real-cell
// entries of qW.  Implicit solver: fillRhoRHS (solver.h:1079-1152), and
// R_out gets the real-cell entries of RhoVector.
int ref_residual(void* cp, int lvl, double* R_out) {
    return guarded([&] {
        auto* c = (Case*)cp;
        if (c->implicit) {
            auto& s = c->im->solvers.at((size_t)lvl);
            (s.*member(ImFillRhs()))();
            const Eigen::VectorXd& r = s.*member(ImRhs());
            if (R_out) std::memcpy(R_out, r.data(), 4 * (size_t)s.m.nRealCells * sizeof(double));
            return;
        }
        auto& s = c->ex->solvers.at((size_t)lvl);
        Eigen::VectorXd& qk = s.*member(ExQk());
        s.calc_dt();
        qk = s.q;
        if ((s.viscosity_model != "inviscid") | (s.second_order)) {
            s.set_walls_from_internal(qk);
            s.calc_gradients(qk);
            if (s.second_order) s.calc_limiters(qk);
        }
        (s.*member(ExCalcResidual()))(qk);
        if (R_out) std::memcpy(R_out, s.qW.data(), 4 * (size_t)s.m.nRealCells * sizeof(double));
    });
}

// n iterations of the loop body of run_solver without its convergence test
// (multigrid.h:196-214 / 253-271): set_cfl, fill, compute, solve.  The CFL
// is start_cfl for the explicit solver and follows the ramp
// min(start + (i+1) slope, max) of the implicit one, counted from i = 0.
int ref_iterate(void* cp, int lvl, int n, double* norms) {
    return guarded([&] {
        Quiet q;
        auto* c = (Case*)cp;
        auto& s = c->level(lvl);
        double cfl = c->st.start_cfl;
        for (int i = 0; i < n; ++i) {
            s.set_cfl(cfl);
            s.fill();
            if (s.compute() != 0) throw std::runtime_error("compute() failed");
            const double r = c->implicit ? s.solve(c->st.relaxation, 0.0, c->st.rhs_iterations)
                                         : s.solve(c->st.relaxation);
            if (norms) norms[i] = r;
            if (c->implicit) cfl = std::min(c->st.start_cfl + (i + 1) * c->st.slope_cfl, c->st.max_cfl);
        }
    });
}

double ref_uniform_residual(void* cp, int lvl) {
    Quiet q;
    return ((Case*)cp)->level(lvl).get_uniform_residual();
}

// multigrid::run_solver on one level (multigrid.h:182-293): returns its
// status; the history it records (every 10th iteration for the explicit
// solver, every iteration for the implicit one) into hist.
int ref_run_solver(void* cp, int lvl, int* status, double* hist, int cap, int* n_hist) {
    return guarded([&] {
        Quiet q;
        auto* c = (Case*)cp;
        c->iters = 0;
        c->residuals.assign((size_t)std::max(1, c->st.max_iterations), 0.0);
        c->profile.calc_chord_coords(c->level(lvl), c->st.airfoil_name);  // as run() does first
        int st = c->implicit ? c->im->run_solver(c->im->solvers.at((size_t)lvl))
                             : c->ex->run_solver(c->ex->solvers.at((size_t)lvl));
        if (status) *status = st;
        const int n = c->iters;
        if (n_hist) *n_hist = n;
        for (int i = 0; i < n && i < cap; ++i) hist[i] = c->residuals[(size_t)i];
    });
}

// multigrid::run (multigrid.h:295-363): init when reinit, then every level
// with the coarse-to-fine transfer.  Returns the history of all levels.
int ref_run(void* cp, int reinit, double* hist, int cap, int* n_hist) {
    return guarded([&] {
        Quiet q;
        auto* c = (Case*)cp;
        c->iters = 0;
        if (c->implicit) c->im->run(reinit != 0);
        else c->ex->run(reinit != 0);
        const int n = c->iters;
        if (n_hist) *n_hist = n;
        for (int i = 0; i < n && i < cap; ++i) hist[i] = c->residuals[(size_t)i];
    });
}

// The angle step of Rans::run_airfoil (rans.h:92-97): the farfield angle of
// the settings is set (radians) and every level's boundary conditions are
// re-read.
int ref_set_angle(void* cp, const char* patch, double angle) {
    return guarded([&] {
        auto* c = (Case*)cp;
        c->st.bcs.at(patch).vars_far.angle = angle;
        for (int i = 0; i < c->n_levels(); ++i) c->level(i).set_bcs(c->st.bcs);
    });
}

// get_wall_profile (post.h:301-387).
int ref_wall_profile(void* cp, int lvl, const char* patch, double* clcdcm, double* cp_out, int cap, int* n_cp) {
    return guarded([&] {
        auto w = rans::get_wall_profile(((Case*)cp)->level(lvl), patch);
        clcdcm[0] = w.cl;
        clcdcm[1] = w.cd;
        clcdcm[2] = w.cm;
        if (n_cp) *n_cp = (int)w.cp.size();
        for (int i = 0; i < (int)w.cp.size() && i < cap; ++i) cp_out[i] = w.cp[(size_t)i];
    });
}

// Implicit solver: fillRhoLHS (solver.h:975-1076) at the current state and
// CFL, then the 4x4 block (rows 4i.., columns 4j..) of RhoMatrix.
int ref_implicit_block(void* cp, int lvl, double cfl, int i, int j, double* blk, int fill) {
    return guarded([&] {
        auto* c = (Case*)cp;
        if (!c->implicit) throw std::invalid_argument("not an implicit case");
        auto& s = c->im->solvers.at((size_t)lvl);
        if (fill) {
            s.set_cfl(cfl);
            (s.*member(ImFillLhs()))();
        }
        auto& M = s.*member(ImMatrix());
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) blk[4 * a + b] = M.coeff(4 * i + a, 4 * j + b);
    });
}

// One face flux of the reference's functors (physics.h:160-530): type 0 is
// internal_flux, 1-3 farfield / slip-wall / wall with qR the stored boundary
// state; not multiplied by the length.
void ref_face_flux(double gamma, int visc, int type, double nx, double ny, const double* qL, const double* qR,
                   const double* gx, const double* gy, double* f) {
    rans::gas g;
    g.gamma = gamma;
    Eigen::VectorXd L(4), R(4), GX(4), GY(4);
    for (int k = 0; k < 4; ++k) {
        L(k) = qL[k];
        R(k) = qR[k];
        GX(k) = gx[k];
        GY(k) = gy[k];
    }
    Eigen::VectorXd F;
    if (type == 0) F = rans::internal_flux(g, nx, ny, visc)(L, R, GX, GY);
    else if (type == 1) F = rans::farfield_flux(g, nx, ny, visc)(L, R);
    else if (type == 2) F = rans::slip_wall_flux(g, nx, ny, visc)(L, R);
    else F = rans::wall_flux(g, nx, ny, visc)(L, R);
    for (int k = 0; k < 4; ++k) f[k] = F(k);
}

}  // extern "C"
