// CPU ORACLE — test infrastructure only, never product code.
//
// A plain C++17 restatement of AeroFLEX's explicit `rans` residual path
// (reference: src/rans/include/rans/{core,mesh,physics,solver,multigrid,post}.h).
// It keeps the reference's data layout (AoS [rho, rhou, rhov, rhoe] per cell,
// ghost cells appended after the real cells), its serial edge loops and its
// OpenMP per-cell loops, and every floating-point expression in the order the
// reference writes it.  Built with -ffp-contract=off so x86 and aarch64 agree
// bit for bit.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it, and only as the checker.
//
// PARITY STATUS: pinned to the reference's own code.  oracle/build_ref.py
// compiles the reference's unmodified rans headers (with the Eigen-API
// stand-in of oracle/eigen_api) into oracle/_ref; tests/test_ref_pin.py
// checks that this restatement reproduces, bit for bit, every result that
// code committed to tests/golden/ref_pins.json, and, where the reference tree
// is present, that both agree directly on more inputs.
//
// Deliberate decisions where the reference is ill-defined:
//  * unqualified abs() on doubles (mesh.h:435,442; solver.h:335-336,344) is
//    taken as fabs — integer truncation would zero every cell area below 1;
//  * Eigen vectors start uninitialised in the reference; here q, qW, gx, gy
//    and the limiter arrays start at 0 (matters only for get_uniform_residual,
//    which reads the previous qW, solver.h:643-649);
//  * qW.norm() is summed sequentially (Eigen's SIMD blocking is not
//    reproducible across machines anyway).
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace oracle {

using uint = unsigned int;
constexpr uint EDGE_NULL = 4294967295u;  // mesh.h:35

// ---------------------------------------------------------------- core.h ---
// gas constants, core.h:27-46
struct Gas {
    double R = 0.71428571428;
    double mu_L = 1e-5;
    double Pr_L = 0.72;
    double Pr_T = 0.9;
    double cp = 1.;
    double gamma = 1.4;
    double k() const { return cp * mu_L / Pr_L; }  // core.h:43-45
};

// boundary_variables::get_conservative, core.h:61-84
struct BoundaryVars {
    double mach = 0.2, angle = 0., T = 1., p = 1.;
    void conservative(const Gas& g, double out[4]) const {
        double c = std::sqrt(g.gamma * g.R * T);
        double u = mach * c * std::cos(angle);
        double v = mach * c * std::sin(angle);
        double rho = p / (g.R * T);
        double rhoE = p / (g.gamma - 1) + 0.5 * rho * (u * u + v * v);
        out[0] = rho; out[1] = rho * u; out[2] = rho * v; out[3] = rhoE;
    }
};

enum BcType { BC_INTERNAL = 0, BC_FARFIELD = 1, BC_SLIP_WALL = 2, BC_WALL = 3 };

struct BoundaryCondition {
    int type = BC_FARFIELD;  // bc_type string of core.h:112-115
    BoundaryVars vars;
};

// Viscosity selector.  0/1 follow core.h:176 + solver.h:203-208.  2 is the
// Spalart-Allmaras model this project adds (the reference has none,
// physics.h:259-261).  3 reproduces what the reference does for its GUI
// spelling "spallart-allmaras": inviscid flux, but gradients still computed
// because viscosity_model != "inviscid" (solver.h:810).
enum Viscosity { VISC_INVISCID = 0, VISC_LAMINAR = 1, VISC_SA = 2, VISC_SA_MISSPELLED = 3 };

struct Settings {
    Gas g;
    int viscosity = VISC_INVISCID;
    int gradient = 1;       // 0 least-squares, 1 green-gauss (core.h:175,179)
    bool second_order = true;
    int limiter = 0;        // 0 Venkatakrishnan (default branch), 1 Michalak (RANS_MICHALAK_LIMITER)
    double limiter_k = 5.;
    double cfl = 1.;        // explicit solver: start_cfl, never ramped (multigrid.h:187,200)
    double relaxation = 0.9;
    double tolerance = 1e-4;
    int max_iterations = 300;
    std::map<std::string, BoundaryCondition> bcs;
};

// ---------------------------------------------------------------- mesh.h ---
struct Mesh {
    std::map<uint, std::string> physicalNames;
    std::map<uint, uint> entityTagToPhysicalTag;
    std::vector<double> nodesX, nodesY;
    std::map<uint, uint> originalNodesRef;

    std::vector<std::array<uint, 2>> edgesNodes, edgesCells;
    std::vector<double> edgesLengths, edgesNormalsX, edgesNormalsY, edgesCentersX, edgesCentersY;

    std::vector<uint> boundaryEdges, boundaryEdges0, boundaryEdges1, boundaryEdgesIntTag;
    std::vector<std::string> boundaryEdgesPhysicals;

    std::map<std::tuple<uint, uint>, uint> edgesRef;

    std::vector<std::array<uint, 4>> cellsNodes, cellsEdges;
    std::vector<char> cellsIsTriangle;
    std::vector<double> cellsAreas, cellsCentersX, cellsCentersY;
    std::vector<double> wall_dist;
    uint nRealCells = 0;

    void read_gmsh(const std::string& filename);
    void finalize();  // mesh.h:843-884 after the four readers
    void compute_wall_dist(const std::map<std::string, BoundaryCondition>& bcs);

  private:
    uint find_edge_with_nodes(uint n0, uint n1) const;
    void add_cell_edges(uint cell_id);
    void convert_node_face_info();
    void compute_mesh();
    void add_boundary_cells();
};

// -------------------------------------------------------------- solver.h ---
class ExplicitSolver {
  public:
    Settings st;
    Mesh m;
    std::vector<double> q, qW, dt, gx, gy, limiters, q_min, q_max, qk;
    std::vector<int> edge_type;                 // solver.h:211-230 (0..3)
    std::vector<BoundaryVars> boundary_vars;    // solver.h:214-230
    std::vector<std::array<double, 4>> lsq;     // (dᵀd)⁻¹ per real cell, row-major 2×2

    ExplicitSolver(const Mesh& mesh, const Settings& s);
    void set_bcs(const std::map<std::string, BoundaryCondition>& bcs);
    void init();                  // solver.h:615-631
    void refill_bcs();            // solver.h:259-274
    void set_walls_from_internal(std::vector<double>& q_);  // solver.h:289-305
    void calc_dt();               // solver.h:308-356
    void calc_gradients();        // solver.h:425-514 (reads member q, not q_)
    void calc_limiters(const std::vector<double>& q_);      // solver.h:517-593
    void calc_residual(const std::vector<double>& q_);      // solver.h:745-799
    double solve();               // solver.h:802-828
    double get_uniform_residual();                           // solver.h:636-690
    BoundaryVars get_boundary_variables() const;            // solver.h:597-611
    bool viscous_or_grad() const { return st.viscosity != VISC_INVISCID; }

    // Spalart-Allmaras (VISC_SA, sa_oracle.cpp): nu~ per cell (ghosts
    // unused), its stage copy and residual, the eddy viscosity mu_t per cell.
    std::vector<double> nu, nuk, nuW, mut;
    std::vector<std::array<uint, 4>> cellFaces;  // a real cell's edges, ascending, EDGE_NULL padded
    double nu_far = 0.;                          // nu~ of the far field: 3 mu_L / rho_inf
    std::vector<double> sa_wd;                   // distance to the nearest no-slip wall face, per real cell
    void sa_setup();
    void sa_wall_distance();
    void sa_init();                                                        // nu~ = nu_far
    void calc_mut(const std::vector<double>& q_, const std::vector<double>& nu_);
    void calc_nu_residual(const std::vector<double>& q_, const std::vector<double>& nu_);
    void sa_wall_shear(uint e, const double q0[4], double f[4]) const;
    int flux_visc() const { return st.viscosity == VISC_LAMINAR ? 1 : 0; }

    // One explicit update as the driver loop does it, returning ‖qW‖₂.
    // run_solver (multigrid.h:182-237): returns status, writes iterations/err.
    int run_solver(int* iters_out, double* err_out, std::vector<double>* history);

    void average_gradients(double gradx[4], double grady[4], uint c0, uint c1) const;
    void flux(int type, uint e, const double qL[4], const double qR[4], const double gradx[4],
              const double grady[4], double f[4]) const;

  private:
    void calc_least_squares_matrices();  // solver.h:402-422
};

struct WallProfile {
    std::vector<double> x, y, cp;
    double cd = 0., cl = 0., cm = 0.;
};
WallProfile get_wall_profile(const ExplicitSolver& s, const std::string& patch);  // post.h:301-387

// Grid sequencing transfer (multigrid.h:99-178 gen_mapper, applied as in
// multigrid::run, multigrid.h:295-363): coarse.bcs_from_internal(), fine.q =
// mapper * coarse.q, fine.refill_bcs().
void prolongate(ExplicitSolver& coarse, ExplicitSolver& fine);

// Spalart-Allmaras source of one cell (sa_oracle.cpp): src = P - D and its
// derivative with respect to nu~.
void sa_source(double nut, double nul, double omega, double d, double* src, double* dsrc);
double sa_cbrt(double x);

// Laminar terms of internal_flux with viscosity mu and heat conductivity kheat.
void laminar_terms(const Gas& g, double mu, double kheat, double nx, double ny, const double qL[4],
                   const double qR[4], const double gx[4], const double gy[4], double f[4]);

// Face-flux functors, physics.h:160-530.
void internal_flux(const Gas& g, double nx, double ny, int viscous_type, const double qL[4],
                   const double qR[4], const double gx[4], const double gy[4], double f[4]);
void boundary_state(const Gas& g, int type, double nx, double ny, const double qL[4],
                    const double qbc[4], double qR[4]);

// save (post.h:58-180): the VTU text of state q (4 per real cell) on m, with
// wall distances wd (per real cell; null: the mesh's own wall_dist) and gas g.
std::string save_text(const Mesh& m, const double* q, const double* wd, const Gas& g);

}  // namespace oracle
