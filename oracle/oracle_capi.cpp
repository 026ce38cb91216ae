// CPU ORACLE — test infrastructure only.  A flat C API over rans_oracle.hpp
// so the Python tests and the CPU-baseline leg of bench.py can drive the
// restatement through ctypes.  Errors are reported by a null handle or a
// non-zero return and a message in orc_last_error().
#include <chrono>
#include <omp.h>
#include <cstdio>
#include <cstring>
#include <string>

#include "rans_oracle.hpp"

using namespace oracle;

static thread_local std::string g_err;

extern "C" {

typedef struct {
    double gamma, R, mu_L, Pr_L, Pr_T;
    int viscosity, gradient, second_order, limiter;
    double limiter_k, cfl, relaxation, tolerance;
    int max_iterations;
} orc_settings;

const char* orc_last_error(void) { return g_err.c_str(); }

void* orc_mesh_load(const char* path) {
    try {
        auto* m = new Mesh();
        m->read_gmsh(path);
        return m;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

// Nodes x/y; cells with 4 node slots (-1 pads a triangle); boundary edges as
// node pairs with a patch index into the '\n'-separated names.  Equivalent to
// reading a gmsh file that lists the nodes, the boundary edges and the cells
// in these orders.
void* orc_mesh_from_arrays(int n_nodes, const double* x, const double* y, int n_cells, const int* cell_nodes,
                           int n_bedges, const int* bedge_nodes, const int* bedge_patch, const char* names) {
    try {
        auto* m = new Mesh();
        m->nodesX.assign(x, x + n_nodes);
        m->nodesY.assign(y, y + n_nodes);
        std::string all(names);
        uint tag = 1;
        size_t pos = 0;
        while (pos <= all.size()) {
            size_t nl = all.find('\n', pos);
            if (nl == std::string::npos) nl = all.size();
            if (nl > pos) m->physicalNames[1000 + tag++] = all.substr(pos, nl - pos);
            pos = nl + 1;
        }
        for (int b = 0; b < n_bedges; ++b) {
            m->boundaryEdges0.push_back((uint)bedge_nodes[2 * b]);
            m->boundaryEdges1.push_back((uint)bedge_nodes[2 * b + 1]);
            m->boundaryEdgesIntTag.push_back(1000 + 1 + (uint)bedge_patch[b]);
        }
        for (int c = 0; c < n_cells; ++c) {
            const int* cn = cell_nodes + 4 * (size_t)c;
            const bool tri = cn[3] < 0;
            m->cellsNodes.push_back({(uint)cn[0], (uint)cn[1], (uint)cn[2], tri ? 0u : (uint)cn[3]});
            m->cellsIsTriangle.push_back(tri);
            m->cellsAreas.push_back(0.);
            m->cellsCentersX.push_back(0.);
            m->cellsCentersY.push_back(0.);
        }
        m->finalize();
        return m;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void orc_mesh_free(void* m) { delete (Mesh*)m; }

void orc_mesh_counts(void* mp, long long* out) {
    auto* m = (Mesh*)mp;
    out[0] = m->nRealCells;
    out[1] = (long long)m->cellsAreas.size();
    out[2] = (long long)m->edgesCells.size();
    out[3] = (long long)m->boundaryEdges.size();
    out[4] = (long long)m->nodesX.size();
}

// Copies one named mesh array; returns its length or -1.
long long orc_mesh_get(void* mp, const char* what, double* out) {
    auto* m = (Mesh*)mp;
    std::string w(what);
    const std::vector<double>* v = nullptr;
    if (w == "cx") v = &m->cellsCentersX;
    else if (w == "cy") v = &m->cellsCentersY;
    else if (w == "area") v = &m->cellsAreas;
    else if (w == "ex") v = &m->edgesCentersX;
    else if (w == "ey") v = &m->edgesCentersY;
    else if (w == "nx") v = &m->edgesNormalsX;
    else if (w == "ny") v = &m->edgesNormalsY;
    else if (w == "L") v = &m->edgesLengths;
    else if (w == "wall_dist") v = &m->wall_dist;
    if (v) {
        if (out) std::memcpy(out, v->data(), v->size() * sizeof(double));
        return (long long)v->size();
    }
    return -1;
}

long long orc_mesh_get_int(void* mp, const char* what, long long* out) {
    auto* m = (Mesh*)mp;
    std::string w(what);
    if (w == "edges_cells") {
        if (out)
            for (size_t e = 0; e < m->edgesCells.size(); ++e) {
                out[2 * e] = m->edgesCells[e][0];
                out[2 * e + 1] = m->edgesCells[e][1];
            }
        return 2 * (long long)m->edgesCells.size();
    }
    if (w == "edges_nodes") {
        if (out)
            for (size_t e = 0; e < m->edgesNodes.size(); ++e) {
                out[2 * e] = m->edgesNodes[e][0];
                out[2 * e + 1] = m->edgesNodes[e][1];
            }
        return 2 * (long long)m->edgesNodes.size();
    }
    if (w == "boundary_edges") {
        if (out)
            for (size_t b = 0; b < m->boundaryEdges.size(); ++b) out[b] = m->boundaryEdges[b];
        return (long long)m->boundaryEdges.size();
    }
    return -1;
}

// save (post.h:58-180) of state q on mesh mp to path; wd per real cell or
// null (the mesh's wall_dist); returns 0, or -1 if the file cannot be written.
int orc_save_vtu(void* mp, const double* q, const double* wd, double gamma, double R, const char* path) {
    Gas g;
    g.gamma = gamma;
    g.R = R;
    const std::string t = save_text(*(Mesh*)mp, q, wd, g);
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return -1;
    const size_t w = std::fwrite(t.data(), 1, t.size(), f);
    std::fclose(f);
    return w == t.size() ? 0 : -1;
}

// Boundary patch name of boundary edge b.
const char* orc_mesh_boundary_name(void* mp, int b) { return ((Mesh*)mp)->boundaryEdgesPhysicals.at(b).c_str(); }

void* orc_solver_create(void* mp, const orc_settings* s, int n_bc, const char** names, const int* types,
                        const double* bcvals) {
    try {
        Settings st;
        st.g.gamma = s->gamma;
        st.g.R = s->R;
        st.g.mu_L = s->mu_L;
        st.g.Pr_L = s->Pr_L;
        st.g.Pr_T = s->Pr_T;
        st.viscosity = s->viscosity;
        st.gradient = s->gradient;
        st.second_order = s->second_order != 0;
        st.limiter = s->limiter;
        st.limiter_k = s->limiter_k;
        st.cfl = s->cfl;
        st.relaxation = s->relaxation;
        st.tolerance = s->tolerance;
        st.max_iterations = s->max_iterations;
        for (int i = 0; i < n_bc; ++i) {
            BoundaryCondition bc;
            bc.type = types[i];
            bc.vars.T = bcvals[4 * i];
            bc.vars.mach = bcvals[4 * i + 1];
            bc.vars.angle = bcvals[4 * i + 2];
            bc.vars.p = bcvals[4 * i + 3];
            st.bcs[names[i]] = bc;
        }
        auto* sv = new ExplicitSolver(*(Mesh*)mp, st);
        return sv;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void orc_solver_free(void* s) { delete (ExplicitSolver*)s; }

void orc_init(void* sp) {
    auto* s = (ExplicitSolver*)sp;
    s->init();
    s->refill_bcs();
    if (s->st.viscosity == VISC_SA) s->sa_init();
}

void orc_refill_bcs(void* sp) { ((ExplicitSolver*)sp)->refill_bcs(); }

// settings.bcs[patch].vars_far = {...}; set_bcs; refill_bcs (rans.h:92-97,
// multigrid.h:301).
int orc_set_farfield(void* sp, const char* patch, double mach, double angle, double T, double p) {
    try {
        auto* s = (ExplicitSolver*)sp;
        auto bcs = s->st.bcs;
        auto& bc = bcs.at(patch);
        bc.vars.mach = mach;
        bc.vars.angle = angle;
        bc.vars.T = T;
        bc.vars.p = p;
        s->set_bcs(bcs);
        s->refill_bcs();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// OpenMP threads of the restated per-cell loops (the reference's own loops
// are OpenMP-parallel the same way); 0 or less: all host threads.
void orc_set_threads(int n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }

void orc_prolongate(void* coarse, void* fine) { prolongate(*(ExplicitSolver*)coarse, *(ExplicitSolver*)fine); }

// mesh::compute_wall_dist (mesh.h:794-830) with the solver's boundary
// conditions, as multigrid's constructor calls it (multigrid.h:72); all
// cells, ghosts included.
long long orc_wall_distance(void* sp, double* out) {
    auto* s = (ExplicitSolver*)sp;
    s->m.compute_wall_dist(s->st.bcs);
    if (out) std::memcpy(out, s->m.wall_dist.data(), s->m.wall_dist.size() * sizeof(double));
    return (long long)s->m.wall_dist.size();
}

// nu~ of the real cells (Spalart-Allmaras solvers).
void orc_set_nu(void* sp, const double* nu_real) {
    auto* s = (ExplicitSolver*)sp;
    std::memcpy(s->nu.data(), nu_real, (size_t)s->m.nRealCells * sizeof(double));
}

// The Spalart-Allmaras source of one cell and its derivative.
void orc_sa_source(double nut, double nul, double omega, double d, double* src, double* dsrc) {
    sa_source(nut, nul, omega, d, src, dsrc);
}

void orc_set_q(void* sp, const double* q_real) {
    auto* s = (ExplicitSolver*)sp;
    std::memcpy(s->q.data(), q_real, 4 * (size_t)s->m.nRealCells * sizeof(double));
}

long long orc_get(void* sp, const char* what, double* out) {
    auto* s = (ExplicitSolver*)sp;
    std::string w(what);
    const std::vector<double>* v = nullptr;
    if (w == "q") v = &s->q;
    else if (w == "qW") v = &s->qW;
    else if (w == "dt") v = &s->dt;
    else if (w == "gx") v = &s->gx;
    else if (w == "gy") v = &s->gy;
    else if (w == "lim") v = &s->limiters;
    else if (w == "nu" && s->st.viscosity == VISC_SA) v = &s->nu;
    else if (w == "nuW" && s->st.viscosity == VISC_SA) v = &s->nuW;
    else if (w == "mut" && s->st.viscosity == VISC_SA) v = &s->mut;
    if (!v) return -1;
    if (out) std::memcpy(out, v->data(), v->size() * sizeof(double));
    return (long long)v->size();
}

// Residual of the current state as the first RK stage computes it
// (solver.h:802-817 with qk = q): walls, gradients, limiters, residual.
// R_out gets the 4*nReal real-cell entries of qW.
int orc_residual(void* sp, double* R_out) {
    try {
        auto* s = (ExplicitSolver*)sp;
        s->calc_dt();
        s->qk = s->q;
        if (s->viscous_or_grad() || s->st.second_order) {
            s->set_walls_from_internal(s->qk);
            s->calc_gradients();
            if (s->st.second_order) s->calc_limiters(s->qk);
        }
        const bool sa = s->st.viscosity == VISC_SA;
        if (sa) s->calc_mut(s->qk, s->nu);
        s->calc_residual(s->qk);
        if (sa) s->calc_nu_residual(s->qk, s->nu);
        if (R_out) std::memcpy(R_out, s->qW.data(), 4 * (size_t)s->m.nRealCells * sizeof(double));
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

int orc_iterate(void* sp, int n, double* norms) {
    try {
        auto* s = (ExplicitSolver*)sp;
        for (int i = 0; i < n; ++i) {
            double r = s->solve();
            if (norms) norms[i] = r;
        }
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

double orc_uniform_residual(void* sp) { return ((ExplicitSolver*)sp)->get_uniform_residual(); }

int orc_run_solver(void* sp, int* iters, double* err, double* hist, int hist_cap, int* n_hist) {
    try {
        auto* s = (ExplicitSolver*)sp;
        std::vector<double> h;
        s->run_solver(iters, err, &h);
        int n = (int)h.size();
        if (n_hist) *n_hist = n;
        for (int i = 0; i < n && i < hist_cap; ++i) hist[i] = h[i];
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

int orc_wall_profile(void* sp, const char* patch, double* clcdcm, double* cp_out, int cap, int* n_cp) {
    try {
        auto w = get_wall_profile(*(ExplicitSolver*)sp, patch);
        clcdcm[0] = w.cl;
        clcdcm[1] = w.cd;
        clcdcm[2] = w.cm;
        if (n_cp) *n_cp = (int)w.cp.size();
        for (int i = 0; i < (int)w.cp.size() && i < cap; ++i) cp_out[i] = w.cp[i];
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// One face flux of the restated functors (physics.h:160-530): type 0 is the
// internal flux (with face gradients gx, gy for the laminar term), types
// 1-3 the farfield / slip-wall / wall functors with qR the stored boundary
// state.
void orc_face_flux(double gamma, int visc, int type, double nx, double ny, const double* qL, const double* qR,
                   const double* gx, const double* gy, double* f) {
    Gas g;
    g.gamma = gamma;
    if (type == BC_INTERNAL) {
        internal_flux(g, nx, ny, visc, qL, qR, gx, gy, f);
    } else {
        double qb[4];
        const double zero[4] = {0, 0, 0, 0};
        boundary_state(g, type, nx, ny, qL, qR, qb);
        internal_flux(g, nx, ny, visc, qL, qb, zero, zero, f);
    }
}

// Wall-clock seconds of n explicit iterations (the CPU baseline leg).
double orc_time_iterations(void* sp, int n) {
    auto* s = (ExplicitSolver*)sp;
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < n; ++i) s->solve();
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Wall-clock seconds of n stage-0 residual evaluations (dt, gradient,
// limiter, face loop) on the current state.
double orc_time_residuals(void* sp, int n) {
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < n; ++i) orc_residual(sp, nullptr);
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
