// Host-side data of the GB300 rans library: the mesh in AeroFLEX's own
// numbering (what the C ABI exposes), the settings, and the device layout
// built from them.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace afx {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum BcType { BC_INTERNAL = 0, BC_FARFIELD = 1, BC_SLIP_WALL = 2, BC_WALL = 3, BC_INLET_OUTLET = 4 };
enum Viscosity { VISC_INVISCID = 0, VISC_LAMINAR = 1, VISC_SA = 2, VISC_SA_MISSPELLED = 3 };

// boundary_variables (src/rans/include/rans/core.h:61-84)
struct FarfieldVars {
    double mach = 0.2, angle = 0., T = 1., p = 1.;
};

struct BoundaryCondition {
    std::string type = "farfield";
    FarfieldVars vars;
};

// rans::Settings (core.h:166-232) plus this library's precision switch.
struct Settings {
    double gamma = 1.4, R = 0.71428571428, mu_L = 1e-5, Pr_L = 0.72, Pr_T = 0.9, cp = 1.;
    std::map<std::string, BoundaryCondition> bcs;
    std::vector<std::string> bc_order;  // [rans-bc] order as read
    std::string solver = "implicit";
    std::string gradient = "green-gauss";
    std::string viscosity = "inviscid";
    std::string limiter = "venkatakrishnan";
    std::string precision = "fp64";
    std::string airfoil_name = "wall";
    bool second_order = true;
    double start_cfl = 40., slope_cfl = 50., max_cfl = 100.;
    double relaxation = 0.9, tolerance = 1e-4;
    int rhs_iterations = 5, max_iterations = 300;
    double alpha_start = 1.0, alpha_end = 7.0, alpha_step = 3.0;
    double limiter_k = 5.;
    // device launch configuration (this library only): residual kernel
    // variant "auto" | "gather" | "face" and threads per block (0 = auto)
    std::string kernel_variant = "auto";
    int block_size = 0;
    // FP32-mixed only: refresh the FP64 defect correction every this many
    // iterations (0 = pure FP32 residual)
    int fp64_correction_interval = 0;
    // FP32-mixed only: run_to_convergence switches to FP64 iterations once the
    // FP32 residual stops falling
    bool fp64_finish = false;
    // implicit solver: run each GMRES solve as one CUDA graph with device-side
    // loops (true), or drive the same kernels from a host loop (false: every
    // kernel is a plain launch that a profiler can list)
    bool krylov_graph = true;
    // preconditioner of the Newton finish and of the implicit adjoint's
    // flexible GMRES: 0 one ILU(0) sweep, 1 a GMRES solve with the matrix
    int krylov_preconditioner = 1;
    // input directions per vector-dual pass of the adjoint's face kernel
    int adjoint_directions = 4;

    int viscosity_code() const;
    static int bc_code(const std::string& t);
};

void import_ini(Settings& s, const std::string& text);  // core.h:238-272 over tinyconfig

// Conservative freestream state, core.h:73-83.
void conservative(const Settings& s, const FarfieldVars& v, double out[4]);

// Mesh in the reference's numbering (mesh.h:198-273).  Ghost cells follow
// the real cells, one per boundary edge.
struct HostMesh {
    std::vector<double> nodesX, nodesY;
    std::vector<std::array<uint32_t, 4>> cellsNodes;
    std::vector<uint8_t> cellsIsTriangle;
    std::vector<std::array<uint32_t, 2>> edgesNodes, edgesCells;
    std::vector<std::array<uint32_t, 4>> cellsEdges;  // real cells: edge of local edge j (nodes j, j+1)
    std::vector<double> edgesLengths, edgesNormalsX, edgesNormalsY, edgesCentersX, edgesCentersY;
    std::vector<double> cellsAreas, cellsCentersX, cellsCentersY;
    std::vector<uint32_t> boundaryEdges;
    std::vector<std::string> boundaryEdgesPhysicals;
    std::vector<double> wall_dist;
    uint32_t nRealCells = 0;
    // batch of independent cases: reference-order cell ranges of each case
    // (empty for a single mesh)
    std::vector<int> segments;

    // raw input before finalize()
    std::vector<uint32_t> bnd0, bnd1;
    std::vector<std::string> bndName;

    void finalize();  // edges, metrics, ghosts (mesh.h:843-884)
    void compute_metrics();  // mesh.h:378-453 for the real cells
    void update_nodes(const double* x, const double* y);  // new coordinates, same topology
};

HostMesh load_gmsh(const std::string& path);

// rans::save (post.h:58-180): the ASCII VTU file of state q (4 per real cell,
// reference order) on m; wall_dist per real cell, or null for zeros.
void write_vtu(const HostMesh& m, const double* q, const double* wall_dist, double gamma, double R,
               const std::string& path);

// Device numbering of cells and faces, with per-cell face slots sorted by the
// reference's edge id (so a per-cell sum over its faces adds in the same
// order as the reference's serial edge loop).
struct DeviceLayout {
    int n_cells = 0, n_faces = 0, n_bnd = 0;
    std::vector<int32_t> cell_old;       // device cell -> reference cell
    std::vector<int32_t> cell_new;       // reference cell -> device cell
    std::vector<int32_t> face_edge;      // device face -> reference edge
    std::vector<int32_t> cslot;          // 4 per device cell: +-(device face + 1), 0 pad
    std::vector<int32_t> cnbr;           // 4 per device cell: other cell or -(b+1)
    std::vector<int32_t> fcell;          // 2 per device face: c0, c1 (c1 < 0: boundary -(b+1))
    std::vector<double> area;            // per device cell
    std::vector<double> fn, fLg, fd0, fd1, ft;  // 2,2,2,2,4 per face
    std::vector<int32_t> bface;          // boundary b -> device face
};

DeviceLayout build_layout(const HostMesh& m);
// The geometric face and cell records of L (fn, fLg, fd0, fd1, ft, area) from
// the metrics of m, keeping L's numbering.
void fill_layout_geometry(const HostMesh& m, DeviceLayout& L);

}  // namespace afx
