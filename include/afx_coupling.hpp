// afx_coupling.hpp — config 5's beam and aeroelastic coupling for a C++
// caller, over the C ABI (afx_rans.h) and the C++ layer (afx_rans.hpp).
// It is the C++ form of aeroflex_gb300/coupling.py, call for call: the
// reference's coupler and structure module are C++, and the pieces it names
// are the wall forces of a converged solve (src/rans/include/rans/rans.h:99-102)
// and structure::MODEL's load vector and linear solve
// (src/structure/include/structure/model.hpp:94-100, 225-238).
//
//  * Beam: Euler-Bernoulli elements along the chord, (w, dw/dx) per node:
//    the bending block of the structure module's bar element
//    (element.hpp:77-110: 12EI/L^3, 6EI/L^2, 4EI/L, 2EI/L), assembled as
//    set_K_global does, clamped at x0 as set_K_Final_sparse does (rows and
//    columns zeroed, unit diagonal, load zeroed), solved directly (dense LU
//    with partial pivoting: 2(n+1) unknowns).
//  * Coupling: loads from the wall c_p (the face sums of get_wall_profile,
//    post.h:341-375) lumped onto the beam by its cubic shape functions; the
//    wall moved vertically by the deflection (afx_deform_patch_xy); the flow
//    converged by the implicit iteration and the Newton-Krylov finish; both
//    adjoints and the shape derivatives along the beam modes
//    (afx_adjoint_patch_dirs_xy) give dC_y/du, and the beam is updated by a
//    Newton step with that rank-one load Jacobian (Sherman-Morrison).
#pragma once

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "afx_rans.hpp"

namespace coupling {

class Beam {
  public:
    explicit Beam(int n_elem = 50, double EI = 1e4, double length = 1.0, double x0 = 0.0)
        : ne_(n_elem), n_(2 * (n_elem + 1)), EI_(EI), len_(length), x0_(x0) {
        if (n_elem < 1) throw std::invalid_argument("beam: at least one element");
        Forces.assign(n_, 0.0);
        set_K_global();
        set_K_Final();
    }
    int n_dof() const { return n_; }
    int n_elem() const { return ne_; }

    // MODEL::set_Load_Vector_From_Vector (model.hpp:94-100): a vector of
    // another size is ignored; returns whether it was taken
    bool set_Load_Vector_From_Vector(const std::vector<double>& f) {
        if (f.size() != Forces.size()) return false;
        Forces = f;
        return true;
    }
    // MODEL::get_Solve (model.hpp:225-232): K_final^-1 f, constrained entries of f zeroed
    std::vector<double> get_Solve(std::vector<double> f) const {
        if ((int)f.size() != n_) throw std::invalid_argument("beam: load vector of the wrong size");
        f[0] = f[1] = 0.0;
        for (int i = 0; i < n_; ++i) std::swap(f[i], f[piv_[i]]);
        for (int i = 0; i < n_; ++i)
            for (int k = 0; k < i; ++k) f[i] -= lu_[(size_t)i * n_ + k] * f[k];
        for (int i = n_ - 1; i >= 0; --i) {
            for (int k = i + 1; k < n_; ++k) f[i] -= lu_[(size_t)i * n_ + k] * f[k];
            f[i] /= lu_[(size_t)i * n_ + i];
        }
        return f;
    }
    // MODEL::get_Lin_Solve (model.hpp:234-238)
    std::vector<double> get_Lin_Solve() const { return get_Solve(Forces); }

    // row of the cubic Hermite shape functions at x (clipped to the beam):
    // w(x) = sum_j row[j] u_j, 4 nonzeros starting at 2 e
    void shape_row(double x, std::vector<double>& row) const {
        row.assign(n_, 0.0);
        const double Le = len_ / ne_;
        x = std::min(std::max(x, x0_), x0_ + len_);
        const int e = std::min((int)((x - x0_) / Le), ne_ - 1);
        const double xi = (x - x0_ - e * Le) / Le, x2 = xi * xi, x3 = x2 * xi;
        row[2 * e] = 1 - 3 * x2 + 2 * x3;
        row[2 * e + 1] = Le * (xi - 2 * x2 + x3);
        row[2 * e + 2] = 3 * x2 - 2 * x3;
        row[2 * e + 3] = Le * (x3 - x2);
    }

    std::vector<double> Forces;

  private:
    void set_K_global() {
        const double Le = len_ / ne_, c = EI_ / (Le * Le * Le);
        const double k[4][4] = {{12, 6 * Le, -12, 6 * Le},
                                {6 * Le, 4 * Le * Le, -6 * Le, 2 * Le * Le},
                                {-12, -6 * Le, 12, -6 * Le},
                                {6 * Le, 2 * Le * Le, -6 * Le, 4 * Le * Le}};
        K_.assign((size_t)n_ * n_, 0.0);
        for (int e = 0; e < ne_; ++e)
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) K_[(size_t)(2 * e + a) * n_ + 2 * e + b] += c * k[a][b];
    }
    void set_K_Final() {
        lu_ = K_;
        for (int d : {0, 1}) {
            for (int k = 0; k < n_; ++k) lu_[(size_t)d * n_ + k] = lu_[(size_t)k * n_ + d] = 0.0;
            lu_[(size_t)d * n_ + d] = 1.0;
        }
        // LU with partial pivoting, rows swapped in place; piv_[i] = the row swapped into i
        piv_.assign(n_, 0);
        for (int i = 0; i < n_; ++i) {
            int p = i;
            for (int r = i + 1; r < n_; ++r)
                if (std::fabs(lu_[(size_t)r * n_ + i]) > std::fabs(lu_[(size_t)p * n_ + i])) p = r;
            piv_[i] = p;
            if (p != i)
                for (int k = 0; k < n_; ++k) std::swap(lu_[(size_t)i * n_ + k], lu_[(size_t)p * n_ + k]);
            const double d = lu_[(size_t)i * n_ + i];
            if (d == 0) throw std::runtime_error("beam: singular stiffness");
            for (int r = i + 1; r < n_; ++r) {
                const double f = lu_[(size_t)r * n_ + i] / d;
                lu_[(size_t)r * n_ + i] = f;
                for (int k = i + 1; k < n_; ++k) lu_[(size_t)r * n_ + k] -= f * lu_[(size_t)i * n_ + k];
            }
        }
    }

    int ne_, n_;
    double EI_, len_, x0_;
    std::vector<double> K_, lu_;
    std::vector<int> piv_;
};

inline double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

// x solving K x = F + s g.(x - u) (loads linearised about u): Sherman-Morrison,
// x = y1 + y2 (g.y1) / (1 - g.y2), y1 = K^-1 (F - s g.u), y2 = K^-1 s
inline std::vector<double> rank_one_newton(const Beam& beam, const std::vector<double>& F,
                                           const std::vector<double>& s, const std::vector<double>& g,
                                           const std::vector<double>& u) {
    const double gu = dot(g, u);
    std::vector<double> r(F.size());
    for (size_t i = 0; i < F.size(); ++i) r[i] = F[i] - s[i] * gu;
    const std::vector<double> y1 = beam.get_Solve(r), y2 = beam.get_Solve(s);
    const double t = dot(g, y1) / (1.0 - dot(g, y2));
    std::vector<double> x(y1.size());
    for (size_t i = 0; i < x.size(); ++i) x[i] = y1[i] + y2[i] * t;
    return x;
}

// q_inf = rho (M a)^2 / 2 in Pa, sea-level density and speed of sound
inline double sea_level_dynamic_pressure(double mach, double rho = 1.225, double a = 340.294) {
    const double v = mach * a;
    return 0.5 * rho * v * v;
}

class Coupling {
  public:
    struct Entry {
        double cl = 0, cd = 0, cm = 0, cy = 0, cy_solver = 0, dcl_dalpha = 0, dcd_dalpha = 0;
        double tip_deflection_m = 0, load_N_per_m = 0, dcl_pred = 0, dcd_pred = 0, alpha_equivalent_deg = 0;
        double step_norm_m = 0, flow_err = 0, adjoint_res_cl = 0, adjoint_res_cd = 0;
        int flow_implicit = 0, flow_newton = 0, flow_krylov = 0, adjoint_it_cl = 0, adjoint_it_cd = 0;
    };

    double tol = 1e-12, switch_tol = 1e-6, adjoint_tol = 1e-12, h = 1e-7, newton_cfl = 0;
    int max_it = 400, adjoint_max_it = 600;
    std::vector<double> u;  // beam state
    std::vector<Entry> history;

    // adj: an FP64 implicit solver on mesh m (initialised, converged or
    // not); flow: another solver of the same mesh for the primal (an
    // FP32-mixed one), or null to use adj.  The beam spans the chord from the
    // leading edge (chord_m metres); q_inf in Pa.
    Coupling(rans::solver& adj, const rans::mesh& m, Beam& beam, double q_inf, double chord_m = 1.0,
             const std::string& patch = "wall", rans::solver* flow = nullptr)
        : s_(adj), fs_(flow ? *flow : adj), beam_(beam), q_(q_inf), c_(chord_m), patch_(patch) {
        int n = 0;
        rans::afx_check(afx_patch_nodes(s_.handle(), patch.c_str(), nullptr, nullptr, nullptr, 0, &n));
        ids_.resize(n);
        std::vector<double> nx(n), ny(n);
        rans::afx_check(afx_patch_nodes(s_.handle(), patch.c_str(), ids_.data(), nx.data(), ny.data(), n, &n));
        const std::vector<double> X = get(m, "node_x"), Y = get(m, "node_y"), enx = get(m, "nx"),
                                  eny = get(m, "ny");
        const std::vector<long long> be = get_int(m, "boundary_edges"), en = get_int(m, "edges_nodes");
        std::vector<long long> pos(X.size(), -1);
        for (int k = 0; k < n; ++k) pos[ids_[k]] = k;
        char buf[256];
        px_.resize(n);
        py_.resize(n);
        for (int k = 0; k < n; ++k) {
            px_[k] = X[ids_[k]];
            py_[k] = Y[ids_[k]];
        }
        for (size_t b = 0; b < be.size(); ++b) {
            rans::afx_check(afx_mesh_boundary_name(m.handle(), (int)b, buf, sizeof buf));
            if (patch != buf) continue;
            const long long e = be[b], a = pos[en[2 * e]], c = pos[en[2 * e + 1]];
            if (a < 0 || c < 0) throw std::runtime_error("coupling: wall face with a node off the patch");
            f0_.push_back((int)a);
            f1_.push_back((int)c);
            // orientation of (dy, -dx) along the node order against the mesh normal (into the body)
            const double dx = px_[c] - px_[a], dy = py_[c] - py_[a];
            orient_.push_back(dy * enx[e] - dx * eny[e] >= 0 ? 1.0 : -1.0);
        }
        // T (n x n_dof): vertical displacement of patch node k per beam dof, in chords
        std::vector<double> row;
        T_.assign((size_t)n * beam_.n_dof(), 0.0);
        for (int k = 0; k < n; ++k) {
            beam_.shape_row(px_[k] * c_, row);
            for (int j = 0; j < beam_.n_dof(); ++j) T_[(size_t)k * beam_.n_dof() + j] = row[j] / c_;
        }
        u.assign(beam_.n_dof(), 0.0);
        nreal_ = m.nRealCells();
    }

    // vertical displacement of each patch node (chords)
    std::vector<double> surface_displacement(const std::vector<double>& uu) const {
        const int n = (int)ids_.size(), nd = beam_.n_dof();
        std::vector<double> a(n, 0.0);
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < nd; ++j) a[k] += T_[(size_t)k * nd + j] * uu[j];
        return a;
    }

    // load vector on the beam and C_y from the wall c_p with the patch nodes raised by a
    void loads(const std::vector<double>& a, const std::vector<double>& cp, std::vector<double>& F,
               double& cy) const {
        F.assign(beam_.n_dof(), 0.0);
        double fy = 0, xmin = 1e300, xmax = -1e300;
        std::vector<double> row;
        for (size_t f = 0; f < f0_.size(); ++f) {
            const int p0 = f0_[f], p1 = f1_[f];
            const double dx = px_[p1] - px_[p0], dy = (py_[p1] + a[p1]) - (py_[p0] + a[p0]);
            const double L = std::sqrt(dx * dx + dy * dy), ny = -orient_[f] * dx / L;
            const double xc = 0.5 * (px_[p0] + px_[p1]);
            xmin = std::min(xmin, xc);
            xmax = std::max(xmax, xc);
            fy += cp[f] * ny * L;
            beam_.shape_row(xc * c_, row);
            const double load = q_ * c_ * cp[f] * ny * L;
            for (int j = 0; j < beam_.n_dof(); ++j) F[j] += row[j] * load;
        }
        cy = fy / (xmax - xmin);
    }

    // one coupling iteration from the current beam state
    const Entry& step(double alpha) {
        Entry e;
        std::vector<double> a;
        rans::wallProfile w = flow(u, a, e);
        std::vector<double> F;
        loads(a, w.cp, F, e.cy);
        std::vector<double> gL, gD;
        gradient("cl", gL, e.dcl_dalpha, e.adjoint_it_cl, e.adjoint_res_cl);
        gradient("cd", gD, e.dcd_dalpha, e.adjoint_it_cd, e.adjoint_res_cd);
        const double ca = std::cos(alpha), sa = std::sin(alpha);
        std::vector<double> gY(gL.size()), s(F.size());
        for (size_t j = 0; j < gY.size(); ++j) gY[j] = ca * gL[j] + sa * gD[j];
        for (size_t j = 0; j < F.size(); ++j) s[j] = F[j] / e.cy;
        const std::vector<double> un = rank_one_newton(beam_, F, s, gY, u);
        std::vector<double> du(un.size());
        for (size_t j = 0; j < du.size(); ++j) du[j] = un[j] - u[j];
        beam_.set_Load_Vector_From_Vector(F);
        e.cl = w.cl;
        e.cd = w.cd;
        e.cm = w.cm;
        e.cy_solver = ca * w.cl + sa * w.cd;
        e.tip_deflection_m = u[2 * beam_.n_elem()];
        for (size_t j = 0; j < F.size(); j += 2) e.load_N_per_m += F[j];
        e.dcl_pred = dot(gL, du);
        e.dcd_pred = dot(gD, du);
        e.alpha_equivalent_deg = e.dcl_dalpha != 0 ? e.dcl_pred / e.dcl_dalpha * 57.29577951308232 : 0.0;
        for (size_t j = 0; j < du.size(); j += 2) e.step_norm_m = std::max(e.step_norm_m, std::fabs(du[j]));
        history.push_back(e);
        u = un;
        return history.back();
    }

    // the flow on the shape of beam state uu (implicit iteration to
    // switch_tol, Newton-Krylov finish to tol; the state copied to the
    // adjoint solver when the primal runs on another)
    rans::wallProfile flow(const std::vector<double>& uu, std::vector<double>& a, Entry& e) {
        a = surface_displacement(uu);
        const std::vector<double> zero(a.size(), 0.0);
        for (rans::solver* g : {&s_, &fs_}) {
            rans::afx_check(afx_deform_patch_xy(g->handle(), patch_.c_str(), zero.data(), a.data(), (int)a.size(), 2.0));
            if (&fs_ == &s_) break;
        }
        double err = 0;
        rans::afx_check(afx_run_to_convergence(fs_.handle(), switch_tol, max_it, &e.flow_implicit, &err));
        rans::afx_check(afx_newton_solve(fs_.handle(), tol, 30, newton_cfl, 0, 0, &e.flow_newton, &e.flow_krylov,
                                         &e.flow_err, nullptr, 0));
        if (&fs_ != &s_) {
            std::vector<double> q(4 * (size_t)nreal_);
            rans::afx_check(afx_get_state(fs_.handle(), q.data(), (long long)q.size()));
            rans::afx_check(afx_set_state(s_.handle(), q.data(), (long long)q.size()));
        }
        return rans::get_wall_profile(s_, patch_);
    }

  private:
    static std::vector<double> get(const rans::mesh& m, const char* what) {
        long long n = 0;
        rans::afx_check(afx_mesh_get(m.handle(), what, nullptr, 0, &n));
        std::vector<double> v((size_t)n);
        rans::afx_check(afx_mesh_get(m.handle(), what, v.data(), n, &n));
        return v;
    }
    static std::vector<long long> get_int(const rans::mesh& m, const char* what) {
        long long n = 0;
        rans::afx_check(afx_mesh_get_int(m.handle(), what, nullptr, 0, &n));
        std::vector<long long> v((size_t)n);
        rans::afx_check(afx_mesh_get_int(m.handle(), what, v.data(), n, &n));
        return v;
    }
    void gradient(const char* obj, std::vector<double>& g, double& dalpha, int& it, double& res) {
        double dJ[2];
        rans::afx_check(afx_adjoint_solve(s_.handle(), patch_.c_str(), obj, adjoint_tol, adjoint_max_it, dJ, &it,
                                          &res));
        dalpha = dJ[0];
        const int n = (int)ids_.size(), nd = beam_.n_dof(), nf = nd - 2;
        std::vector<double> dirs((size_t)nf * n * 2, 0.0), out(nf);
        for (int j = 0; j < nf; ++j)
            for (int k = 0; k < n; ++k) dirs[((size_t)j * n + k) * 2 + 1] = T_[(size_t)k * nd + j + 2];
        rans::afx_check(afx_adjoint_patch_dirs_xy(s_.handle(), patch_.c_str(), obj, 2.0, h, dirs.data(), nf, n,
                                                  out.data()));
        g.assign(nd, 0.0);
        for (int j = 0; j < nf; ++j) g[j + 2] = out[j];
    }

    rans::solver& s_;
    rans::solver& fs_;
    Beam& beam_;
    double q_, c_;
    std::string patch_;
    std::vector<long long> ids_;
    std::vector<double> px_, py_, orient_, T_;
    std::vector<int> f0_, f1_;
    long long nreal_ = 0;
};

}  // namespace coupling
