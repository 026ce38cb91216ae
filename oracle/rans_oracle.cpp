// CPU ORACLE — test infrastructure only (see rans_oracle.hpp for the status
// and the decisions taken where the reference is ill-defined).
//
// Every function cites the reference lines it restates.  Floating-point
// expressions keep the reference's operand order and grouping exactly: the
// GPU path is required to match this file bit for bit in FP64.
#include "rans_oracle.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <sstream>

namespace oracle {

// ------------------------------------------------------------ text helpers
// cut_str / str_to_ints / str_to_floats, mesh.h:39-109: split on single
// spaces; integers go through std::stoi (so "1.5" reads as 1).
static std::vector<std::string> split_spaces(const std::string& s) {
    std::vector<std::string> out;
    size_t start = 0;
    for (size_t i = 0; i <= s.size(); ++i) {
        if (i == s.size() || s[i] == ' ') {
            if (i > start) out.push_back(s.substr(start, i - start));
            start = i + 1;
        }
    }
    return out;
}
static std::vector<long> to_ints(const std::string& s) {
    std::vector<long> v;
    for (auto& t : split_spaces(s)) v.push_back(std::stoi(t));
    return v;
}
static std::vector<double> to_floats(const std::string& s) {
    std::vector<double> v;
    for (auto& t : split_spaces(s)) v.push_back(std::stod(t));
    return v;
}

// ------------------------------------------------------------ gmsh 4.1 ASCII
// One pass that reproduces read_entities / read_nodes / read_boundaries /
// read_elements (mesh.h:457-738), which each re-read the whole file.
void Mesh::read_gmsh(const std::string& filename) {
    std::ifstream in(filename);
    if (!in) throw std::runtime_error("cannot open mesh file " + filename);
    std::string line, section;
    long ns = 0;
    // Entities state (mesh.h:488-508)
    long n_points = 0, n_curves = 0, n_surfaces = 0, nss = 0;
    // Nodes state (mesh.h:547-570)
    long node_start = 0, node_n = 0, node_nss = 0;
    std::vector<uint> block_tags;
    // Elements state (mesh.h:610-642, 679-729)
    long el_start = 0, el_n = 0, block_dim = 0;
    uint block_phys = 0;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (!line.empty() && line[0] == '$') {
            section = line.substr(1);
            ns = 0;
            ns += 1;
            nss += 1;
            node_nss += 1;
            continue;
        }
        if (section == "PhysicalNames") {
            if (ns > 1) {
                auto t = split_spaces(line);
                std::string name = t.at(2);
                name.erase(std::remove(name.begin(), name.end(), '"'), name.end());
                physicalNames[std::stoi(t.at(1)) + 1000 * std::stoi(t.at(0))] = name;
            }
        } else if (section == "Entities") {
            if (ns == 1) {
                auto l = to_ints(line);
                n_points = l.at(0);
                n_curves = l.at(1) + l.at(0);
                n_surfaces = l.at(2) + l.at(1) + l.at(0);
                nss = 0;
            } else if (nss <= n_points) {
            } else if (nss <= n_curves) {
                auto l = to_ints(line);
                entityTagToPhysicalTag[(uint)l.at(0)] = (uint)(l.at(8) + 1000 * 1);
            }
        } else if (section == "Nodes") {
            if (ns == 1) {
                node_start = 1;
                node_nss = 0;
            } else if (ns > node_start + 2 * node_n) {
                auto l = to_ints(line);
                node_n = l.at(3);
                node_start = ns;
                block_tags.assign(node_n, 0);
                node_nss = 0;
            } else if (node_nss <= node_n) {
                block_tags[node_nss - 1] = (uint)(std::stoi(line) - 1);
            } else {
                uint tag = block_tags[node_nss - 1 - node_n];
                auto l = to_floats(line);
                originalNodesRef[tag] = (uint)nodesX.size();
                nodesX.push_back(l.at(0));
                nodesY.push_back(l.at(1));
            }
        } else if (section == "Elements") {
            if (ns == 1) {
                el_start = 1;
                el_n = 0;
            } else if (ns > el_start + el_n) {
                auto l = to_ints(line);
                block_dim = l.at(0);
                if (block_dim == 1) block_phys = entityTagToPhysicalTag.at((uint)l.at(1));
                el_n = l.at(3);
                el_start = ns;
            } else if (block_dim == 1 || block_dim == 2) {
                auto li = to_ints(line);
                std::vector<uint> l(li.size() - 1);
                for (size_t i = 1; i < li.size(); ++i) l[i - 1] = (uint)(li[i] - 1);
                if (block_dim == 1 && l.size() == 2) {
                    boundaryEdges0.push_back(originalNodesRef.at(l[0]));
                    boundaryEdges1.push_back(originalNodesRef.at(l[1]));
                    boundaryEdgesIntTag.push_back(block_phys);
                } else if (block_dim == 2 && l.size() != 2) {
                    if (l.size() != 3 && l.size() != 4)
                        throw std::invalid_argument("size of input array " + std::to_string(l.size()) +
                                                    " not equal to 4");
                    std::array<uint, 4> c{0, 0, 0, 0};
                    for (size_t i = 0; i < l.size(); ++i) c[i] = originalNodesRef.at(l[i]);
                    cellsIsTriangle.push_back(l.size() == 3);
                    cellsNodes.push_back(c);
                    cellsAreas.push_back(0.);
                    cellsCentersX.push_back(0.);
                    cellsCentersY.push_back(0.);
                }
            }
        }
        ns += 1;
        nss += 1;
        node_nss += 1;
    }
    finalize();
}

uint Mesh::find_edge_with_nodes(uint n0, uint n1) const {  // mesh.h:290-301
    auto it = edgesRef.find(std::make_tuple(std::min(n0, n1), std::max(n0, n1)));
    return it == edgesRef.end() ? EDGE_NULL : it->second;
}

void Mesh::add_cell_edges(uint cell_id) {  // mesh.h:317-341
    uint size = cellsIsTriangle[cell_id] ? 3 : 4;
    for (uint i = 0; i < size; ++i) {
        uint j = (i < (size - 1)) ? (i + 1) : 0;
        uint a = cellsNodes[cell_id][i], b = cellsNodes[cell_id][j];
        auto key = std::make_tuple(std::min(a, b), std::max(a, b));
        if (edgesRef.find(key) == edgesRef.end()) {
            edgesNormalsX.push_back(0.);
            edgesNormalsY.push_back(0.);
            edgesCentersX.push_back(0.);
            edgesCentersY.push_back(0.);
            edgesCells.push_back({cell_id, 0});
            edgesNodes.push_back({a, b});
            edgesLengths.push_back(0.);
            edgesRef.insert({key, (uint)edgesLengths.size() - 1});
        }
    }
}

void Mesh::convert_node_face_info() {  // mesh.h:344-375
    for (uint i = 0; i < cellsAreas.size(); ++i) {
        std::array<uint, 4> ce;
        auto& cn = cellsNodes[i];
        ce[0] = find_edge_with_nodes(cn[0], cn[1]);
        ce[1] = find_edge_with_nodes(cn[1], cn[2]);
        if (cellsIsTriangle[i]) {
            ce[2] = find_edge_with_nodes(cn[2], cn[0]);
            ce[3] = EDGE_NULL;
        } else {
            ce[2] = find_edge_with_nodes(cn[2], cn[3]);
            ce[3] = find_edge_with_nodes(cn[3], cn[0]);
        }
        cellsEdges.push_back(ce);
        for (uint ei : ce)
            if (ei != EDGE_NULL && i != edgesCells[ei][0]) edgesCells[ei][1] = i;
    }
}

void Mesh::compute_mesh() {  // mesh.h:378-453
    const int nc = (int)cellsAreas.size();
#pragma omp parallel for
    for (int i = 0; i < nc; ++i) {
        double cx = 0., cy = 0.;
        uint n = cellsIsTriangle[i] ? 3 : 4;
        for (uint j = 0; j < n; ++j) {
            cx += nodesX[cellsNodes[i][j]] / ((double)n);
            cy += nodesY[cellsNodes[i][j]] / ((double)n);
        }
        cellsCentersX[i] = cx;
        cellsCentersY[i] = cy;
    }
    const int ne = (int)edgesLengths.size();
#pragma omp parallel for
    for (int i = 0; i < ne; ++i) {
        const uint a = edgesNodes[i][0], b = edgesNodes[i][1];
        edgesCentersX[i] = (nodesX[b] + nodesX[a]) * 0.5;
        edgesCentersY[i] = (nodesY[b] + nodesY[a]) * 0.5;
        double dex = nodesX[b] - nodesX[a];
        double dey = nodesY[b] - nodesY[a];
        double l = std::sqrt(dex * dex + dey * dey);
        edgesLengths[i] = l;
        edgesNormalsX[i] = -dey / l;
        edgesNormalsY[i] = dex / l;
        double dot = edgesNormalsX[i] * (edgesCentersX[i] - cellsCentersX[edgesCells[i][0]]) +
                     edgesNormalsY[i] * (edgesCentersY[i] - cellsCentersY[edgesCells[i][0]]);
        if (dot < 0) {
            edgesNormalsX[i] *= -1.;
            edgesNormalsY[i] *= -1.;
        }
    }
#pragma omp parallel for
    for (int i = 0; i < nc; ++i) {
        const auto& n = cellsNodes[i];
        double x1 = nodesX[n[0]], x2 = nodesX[n[1]], x3 = nodesX[n[2]];
        double y1 = nodesY[n[0]], y2 = nodesY[n[1]], y3 = nodesY[n[2]];
        if (cellsIsTriangle[i]) {
            cellsAreas[i] = 0.5 * std::fabs(x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2));
        } else {
            double x4 = nodesX[n[3]], y4 = nodesY[n[3]];
            cellsAreas[i] = 0.5 * std::fabs(x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2)) +
                            0.5 * std::fabs(x1 * (y3 - y4) + x3 * (y4 - y1) + x4 * (y1 - y3));
        }
    }
}

void Mesh::add_boundary_cells() {  // mesh.h:744-787
    for (size_t i = 0; i < boundaryEdges0.size(); ++i) {
        const uint nmin = std::min(boundaryEdges0[i], boundaryEdges1[i]);
        const uint nmax = std::max(boundaryEdges0[i], boundaryEdges1[i]);
        auto it = edgesRef.find(std::make_tuple(nmin, nmax));
        if (it == edgesRef.end())
            throw std::invalid_argument("invalid edge ref (" + std::to_string(nmin) + ", " +
                                        std::to_string(nmax) + ")");
        uint e = it->second;
        uint cell = edgesCells[e][0];
        double area = cellsAreas[cell];
        double dx = edgesCentersX[e] - cellsCentersX[cell];
        double dy = edgesCentersY[e] - cellsCentersY[cell];
        double dist = std::sqrt(dx * dx + dy * dy);
        double cx = edgesCentersX[e] + dist * edgesNormalsX[e];
        double cy = edgesCentersY[e] + dist * edgesNormalsY[e];
        cellsAreas.push_back(area);
        cellsCentersX.push_back(cx);
        cellsCentersY.push_back(cy);
        cellsIsTriangle.push_back(true);
        cellsNodes.push_back({nmin, nmax, 0, 0});
        edgesCells[e][1] = (uint)cellsAreas.size() - 1;
        boundaryEdges.push_back(e);
        boundaryEdgesPhysicals.push_back(physicalNames.at(boundaryEdgesIntTag[i]));
    }
}

void Mesh::finalize() {  // mesh.h:843-884
    for (uint i = 0; i < cellsAreas.size(); ++i) add_cell_edges(i);
    nRealCells = (uint)cellsAreas.size();
    convert_node_face_info();
    compute_mesh();
    add_boundary_cells();
    wall_dist.assign(cellsAreas.size(), 0.);
}

void Mesh::compute_wall_dist(const std::map<std::string, BoundaryCondition>& bcs) {  // mesh.h:794-830
    const int nc = (int)cellsAreas.size();
#pragma omp parallel for
    for (int i = 0; i < nc; ++i) {
        double cx = cellsCentersX[i], cy = cellsCentersY[i];
        double mind = 1;
        bool first = true;
        for (size_t j = 0; j < boundaryEdges.size(); ++j) {
            int t = bcs.at(boundaryEdgesPhysicals[j]).type;
            if (t == BC_WALL || t == BC_SLIP_WALL) {
                const uint e = boundaryEdges[j];
                double dx = cx - edgesCentersX[e];
                double dy = cy - edgesCentersY[e];
                double d = std::sqrt(dx * dx + dy * dy);
                if (first) { mind = d; first = false; }
                else mind = std::min(mind, d);
            }
        }
        wall_dist[i] = mind;
    }
}

// ------------------------------------------------------------- physics.h
static inline double sabs(double x) { return std::sqrt(x * x + 1e-4); }  // physics.h:84-86
static inline double entropy_correction(double l, double d) {            // physics.h:133-135
    return l > d ? l : (l * l + d * d) / (2 * d);
}

// internal_flux::operator(), physics.h:160-264 (laminar branch 230-258 with
// calc_grad_p/temp/u/v, physics.h:33-82).
void internal_flux(const Gas& g, double nx, double ny, int viscous_type, const double qL[4],
                   const double qR[4], const double gx[4], const double gy[4], double f[4]) {
    const double rho_L = qL[0], rho_u_L = qL[1], rho_v_L = qL[2], rho_e_L = qL[3];
    const double rho_R = qR[0], rho_u_R = qR[1], rho_v_R = qR[2], rho_e_R = qR[3];

    const double V_L = (rho_u_L * nx + rho_v_L * ny) / rho_L;
    const double V_R = (rho_u_R * nx + rho_v_R * ny) / rho_R;
    const double p_L = (g.gamma - 1) * (rho_e_L - 0.5 / rho_L * (rho_u_L * rho_u_L + rho_v_L * rho_v_L));
    const double p_R = (g.gamma - 1) * (rho_e_R - 0.5 / rho_R * (rho_u_R * rho_u_R + rho_v_R * rho_v_R));

    f[0] = (V_L * rho_L + V_R * rho_R) * 0.5;
    f[1] = (V_L * rho_u_L + p_L * nx + V_R * rho_u_R + p_R * nx) * 0.5;
    f[2] = (V_L * rho_v_L + p_L * ny + V_R * rho_v_R + p_R * ny) * 0.5;
    f[3] = (V_L * (rho_e_L + p_L) + V_R * (rho_e_R + p_R)) * 0.5;

    const double pL = p_L, pR = p_R;
    const double uL = qL[1] / qL[0];
    const double uR = qR[1] / qR[0];
    const double vL = qL[2] / qL[0];
    const double vR = qR[2] / qR[0];
    const double srhoL = std::sqrt(qL[0]);
    const double srhoR = std::sqrt(qR[0]);
    const double rho = srhoR * srhoL;
    const double u = (uL * srhoL + uR * srhoR) / (srhoL + srhoR);
    const double v = (vL * srhoL + vR * srhoR) / (srhoL + srhoR);
    const double h = ((qL[3] + pL) / qL[0] * srhoL + (qR[3] + pR) / qR[0] * srhoR) / (srhoL + srhoR);
    const double q2 = u * u + v * v;
    const double c = std::sqrt((g.gamma - 1.) * (h - 0.5 * q2));
    const double V = u * nx + v * ny;
    const double VR = uR * nx + vR * ny;
    const double VL = uL * nx + vL * ny;

    const double lambda_cm = entropy_correction(sabs(V - c), 0.05 * c);
    const double lambda_c = entropy_correction(sabs(V), 0.05 * c);
    const double lambda_cp = entropy_correction(sabs(V + c), 0.05 * c);

    const double kF1 = lambda_cm * ((pR - pL) - rho * c * (VR - VL)) / (2. * c * c);
    const double kF234_0 = lambda_c * ((qR[0] - qL[0]) - (pR - pL) / (c * c));
    const double kF234_1 = lambda_c * rho;
    const double kF5 = lambda_cp * ((pR - pL) + rho * c * (VR - VL)) / (2 * c * c);

    f[0] -= 0.5 * (kF1 + kF234_0 + kF5);
    f[1] -= 0.5 * (kF1 * (u - c * nx) + kF234_0 * u + kF234_1 * (uR - uL - (VR - VL) * nx) + kF5 * (u + c * nx));
    f[2] -= 0.5 * (kF1 * (v - c * ny) + kF234_0 * v + kF234_1 * (vR - vL - (VR - VL) * ny) + kF5 * (v + c * ny));
    f[3] -= 0.5 * (kF1 * (h - c * V) + kF234_0 * q2 * 0.5 + kF234_1 * (u * (uR - uL) + v * (vR - vL) - V * (VR - VL)) +
                   kF5 * (h + c * V));

    if (viscous_type == 1) laminar_terms(g, g.mu_L, g.k(), nx, ny, qL, qR, gx, gy, f);
}

// Laminar branch of internal_flux (physics.h:230-258 with calc_grad_p /
// temp / u / v, physics.h:33-82) for viscosity mu and heat conductivity
// kheat: the reference passes g.mu_L and g.k(); the Spalart-Allmaras flux
// passes the face's mu + mu_t and cp (mu / Pr_L + mu_t / Pr_T).
void laminar_terms(const Gas& g, double mu, double kheat, double nx, double ny, const double qL[4],
                   const double qR[4], const double gx[4], const double gy[4], double f[4]) {
    double qc[4];
    for (int k = 0; k < 4; ++k) qc[k] = 0.5 * (qL[k] + qR[k]);
    const double p = (g.gamma - 1) * (qc[3] - 0.5 / qc[0] * (qc[1] * qc[1] + qc[2] * qc[2]));
    double gp0 = 2. * gx[3];
    gp0 -= gx[1] * qc[1] / qc[0] + qc[1] * (gx[1] * qc[0] - gx[0] * qc[1]) / (qc[0] * qc[0]);
    gp0 -= gx[2] * qc[2] / qc[0] + qc[2] * (gx[2] * qc[0] - gx[0] * qc[2]) / (qc[0] * qc[0]);
    gp0 *= 0.5 * (g.gamma - 1);
    double gp1 = 2. * gy[3];
    gp1 -= gy[1] * qc[1] / qc[0] + qc[1] * (gy[1] * qc[0] - gy[0] * qc[1]) / (qc[0] * qc[0]);
    gp1 -= gy[2] * qc[2] / qc[0] + qc[2] * (gy[2] * qc[0] - gy[0] * qc[2]) / (qc[0] * qc[0]);
    gp1 *= 0.5 * (g.gamma - 1);
    const double gT0 = (1. / g.R) * ((gp0 * qc[0] - gx[0] * p) / (qc[0] * qc[0]));
    const double gT1 = (1. / g.R) * ((gp1 * qc[0] - gy[0] * p) / (qc[0] * qc[0]));
    const double gu0 = (qc[0] * gx[1] - qc[1] * gx[0]) / (qc[0] * qc[0]);
    const double gu1 = (qc[0] * gy[1] - qc[1] * gy[0]) / (qc[0] * qc[0]);
    const double gv0 = (qc[0] * gx[2] - qc[2] * gx[0]) / (qc[0] * qc[0]);
    const double gv1 = (qc[0] * gy[2] - qc[2] * gy[0]) / (qc[0] * qc[0]);
    const double div_v = gu0 + gv1;
    const double tau_xx = 2. * mu * (gu0 - div_v / 3.);
    const double tau_yy = 2. * mu * (gv1 - div_v / 3.);
    const double tau_xy = mu * (gu1 + gv0);
    const double phi0 = qc[1] / qc[0] * tau_xx + qc[2] / qc[0] * tau_xy + kheat * gT0;
    const double phi1 = qc[1] / qc[0] * tau_xy + qc[2] / qc[0] * tau_yy + kheat * gT1;
    f[1] -= nx * tau_xx + ny * tau_xy;
    f[2] -= nx * tau_xy + ny * tau_yy;
    f[3] -= nx * phi0 + ny * phi1;
}

// Ghost states: slip_wall_flux::vars (physics.h:311-339), wall_flux::vars
// (physics.h:377-405), farfield_flux::vars (physics.h:446-530, including the
// outside `va` in the subsonic-outlet y-momentum, line 524).
void boundary_state(const Gas& g, int type, double nx, double ny, const double qL[4],
                    const double qbc[4], double qR[4]) {
    if (type == BC_SLIP_WALL) {
        const double rhoV = qL[1] * nx + qL[2] * ny;
        qR[0] = qL[0];
        qR[1] = qL[1] - 2. * rhoV * nx;
        qR[2] = qL[2] - 2. * rhoV * ny;
        qR[3] = qL[3];
        return;
    }
    if (type == BC_WALL) {
        qR[0] = qL[0]; qR[1] = -qL[1]; qR[2] = -qL[2]; qR[3] = qL[3];
        return;
    }
    if (type != BC_FARFIELD) {  // internal_flux::vars, physics.h:267-276
        for (int k = 0; k < 4; ++k) qR[k] = (qL[k] + qbc[k]) * 0.5;
        return;
    }
    const double rho = qL[0], rho_u = qL[1], rho_v = qL[2], rho_e = qL[3];
    const double bc_rho = qbc[0], bc_rhou = qbc[1], bc_rhov = qbc[2], bc_rhoe = qbc[3];
    const double bc_u = bc_rhou / bc_rho;
    const double bc_v = bc_rhov / bc_rho;
    const double bc_p = (g.gamma - 1) * (bc_rhoe - 0.5 / bc_rho * (bc_rhou * bc_rhou + bc_rhov * bc_rhov));
    const double p = (g.gamma - 1) * (rho_e - 0.5 / rho * (rho_u * rho_u + rho_v * rho_v));
    const double c = std::sqrt(g.gamma * p / rho);
    const double mach = std::sqrt(rho_u * rho_u + rho_v * rho_v) / (rho * c);
    const double inlet_outlet = rho_u * nx + rho_v * ny;
    if (mach > 1) {
        if (inlet_outlet < 0) {
            qR[0] = bc_rho;
            qR[1] = bc_rho * bc_u;
            qR[2] = bc_rho * bc_v;
            qR[3] = bc_p / (g.gamma - 1) + 0.5 * bc_rho * (bc_u * bc_u + bc_v * bc_v);
        } else {
            qR[0] = rho; qR[1] = rho_u; qR[2] = rho_v; qR[3] = rho_e;
        }
    } else {
        double pa = bc_p, rhoa = bc_rho, ua = bc_u, va = bc_v;
        double pd = p, rhod = rho, ud = rho_u / rho, vd = rho_v / rho;
        double rho0 = rho, c0 = c;
        (void)vd;
        if (inlet_outlet < 0) {
            double pb = 0.5 * (pa + pd - rho0 * c0 * (nx * (ua - ud) + ny * (va - vd)));
            qR[0] = rhoa + (pb - pa) / (c0 * c0);
            qR[1] = qR[0] * (ua - nx * (pa - pb) / (rho0 * c0));
            qR[2] = qR[0] * (va - ny * (pa - pb) / (rho0 * c0));
            qR[3] = pb / (g.gamma - 1) + 0.5 / qR[0] * (qR[1] * qR[1] + qR[2] * qR[2]);
        } else {
            double pb = pa;
            qR[0] = rhod + (pb - pd) / (c0 * c0);
            qR[1] = qR[0] * (ud + nx * (pd - pb) / (rho0 * c0));
            qR[2] = qR[0] * (va + ny * (pd - pb) / (rho0 * c0));
            qR[3] = pb / (g.gamma - 1) + 0.5 / qR[0] * (qR[1] * qR[1] + qR[2] * qR[2]);
        }
    }
}

// Limiter functions, physics.h:581-607.
static inline double michalak_limiter(double y) {
    constexpr double YT = 2.0;
    if (y >= YT) return 1.0;
    constexpr double a = 1.0 / (YT * YT) - 2.0 / (YT * YT * YT);
    constexpr double b = -3.0 / 2.0 * a * YT - 0.5 / YT;
    return a * y * y * y + b * y * y + y;
}

// -------------------------------------------------------------- solver.h
static inline bool two_sided(int t) { return t != BC_FARFIELD && t != BC_SLIP_WALL && t != BC_WALL; }

ExplicitSolver::ExplicitSolver(const Mesh& mesh, const Settings& s) : st(s), m(mesh) {
    const size_t N = m.cellsAreas.size();  // solver.h:177-197
    q.assign(4 * N, 0.);
    qW.assign(4 * N, 0.);
    dt.assign(N, 0.);
    gx.assign(4 * N, 0.);
    gy.assign(4 * N, 0.);
    limiters.assign(4 * N, 0.);
    q_min.assign(4 * N, 0.);
    q_max.assign(4 * N, 0.);
    qk.assign(4 * N, 0.);
    set_bcs(st.bcs);
    if (st.gradient == 0) calc_least_squares_matrices();
    if (st.viscosity == VISC_SA) sa_setup();
}

void ExplicitSolver::set_bcs(const std::map<std::string, BoundaryCondition>& bcs) {  // solver.h:200-247
    st.bcs = bcs;
    edge_type.assign(m.edgesCells.size(), BC_INTERNAL);
    boundary_vars.assign(m.boundaryEdges.size(), BoundaryVars());
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
        const uint e = m.boundaryEdges[b];
        const BoundaryCondition& bc = st.bcs.at(m.boundaryEdgesPhysicals[b]);
        BoundaryVars v;
        if (bc.type == BC_FARFIELD) {
            edge_type[e] = BC_FARFIELD;
            v = bc.vars;
        } else if (bc.type == BC_SLIP_WALL) {
            edge_type[e] = BC_SLIP_WALL;
        } else if (bc.type == BC_WALL) {
            edge_type[e] = BC_WALL;
        }
        boundary_vars[b] = v;
    }
}

BoundaryVars ExplicitSolver::get_boundary_variables() const {  // solver.h:597-611
    BoundaryVars v;
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
        int t = st.bcs.at(m.boundaryEdgesPhysicals[b]).type;
        if (t == BC_FARFIELD || t == 4 /* inlet-outlet */) { v = boundary_vars[b]; break; }
    }
    return v;
}

void ExplicitSolver::init() {  // solver.h:615-631
    double qi[4];
    get_boundary_variables().conservative(st.g, qi);
    const int N = (int)m.nRealCells;
#pragma omp parallel for
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 4; ++k) q[4 * i + k] = qi[k];
}

void ExplicitSolver::refill_bcs() {  // solver.h:259-274
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
        const uint cell1 = m.edgesCells[m.boundaryEdges[b]][1];
        double qb[4];
        boundary_vars[b].conservative(st.g, qb);
        for (int k = 0; k < 4; ++k) q[4 * cell1 + k] = qb[k];
    }
}

void ExplicitSolver::set_walls_from_internal(std::vector<double>& q_) {  // solver.h:289-305
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
        int t = st.bcs.at(m.boundaryEdgesPhysicals[b]).type;
        if (t == BC_WALL || t == BC_SLIP_WALL) {
            const uint e = m.boundaryEdges[b];
            const uint c0 = m.edgesCells[e][0], c1 = m.edgesCells[e][1];
            for (int k = 0; k < 4; ++k) q_[4 * c1 + k] = q_[4 * c0 + k];
        }
    }
}

void ExplicitSolver::calc_dt() {  // solver.h:308-356
    std::fill(dt.begin(), dt.end(), 0.);
    const double gam = st.g.gamma;
    for (size_t e = 0; e < m.edgesCells.size(); ++e) {
        const uint c0 = m.edgesCells[e][0], c1 = m.edgesCells[e][1];
        const size_t k0 = 4 * (size_t)c0, k1 = 4 * (size_t)c1;
        const double n0 = m.edgesNormalsX[e], n1 = m.edgesNormalsY[e];
        double eig;
        const bool ts = two_sided(edge_type[e]);
        if (ts) {
            const double V_L = (q[k0 + 1] * n0 + q[k0 + 2] * n1) / q[k0];
            const double V_R = (q[k1 + 1] * n0 + q[k1 + 2] * n1) / q[k1];
            const double p_L = (gam - 1) * (q[k0 + 3] - 0.5 / q[k0] * (q[k0 + 1] * q[k0 + 1] + q[k0 + 2] * q[k0 + 2]));
            const double p_R = (gam - 1) * (q[k1 + 3] - 0.5 / q[k1] * (q[k1 + 1] * q[k1 + 1] + q[k1 + 2] * q[k1 + 2]));
            const double eig_L = std::sqrt(p_L * gam / q[k0]) + std::fabs(V_L);
            const double eig_R = std::sqrt(p_R * gam / q[k1]) + std::fabs(V_R);
            eig = std::max(eig_L, eig_R);
        } else {
            const double V_L = (q[k0 + 1] * n0 + q[k0 + 2] * n1) / q[k0];
            const double p_L = (gam - 1) * (q[k0 + 3] - 0.5 / q[k0] * (q[k0 + 1] * q[k0 + 1] + q[k0 + 2] * q[k0 + 2]));
            eig = std::sqrt(p_L * gam / q[k0]) + std::fabs(V_L);
        }
        dt[c0] += eig * m.edgesLengths[e];
        if (ts) dt[c1] += eig * m.edgesLengths[e];
    }
    const int N = (int)dt.size();
#pragma omp parallel for
    for (int i = 0; i < N; ++i) dt[i] = st.cfl * m.cellsAreas[i] / dt[i];
}

void ExplicitSolver::average_gradients(double gradx[4], double grady[4], uint c0, uint c1) const {
    // solver.h:359-398 (the "direction" is built from the SUM of centroids)
    if (c0 == c1) {
        for (int i = 0; i < 4; ++i) { gradx[i] = gx[4 * c0 + i]; grady[i] = gy[4 * c0 + i]; }
        return;
    }
    double t0 = m.cellsCentersX[c0] + m.cellsCentersX[c1];
    double t1 = m.cellsCentersY[c0] + m.cellsCentersY[c1];
    const double lij = std::sqrt(t0 * t0 + t1 * t1);
    t0 /= lij;
    t1 /= lij;
    for (int i = 0; i < 4; ++i) {
        const double grad_dir = (q[4 * c0 + i] - q[4 * c1 + i]) / lij;
        const double gxb = (gx[4 * c0 + i] + gx[4 * c1 + i]) * 0.5;
        const double gyb = (gy[4 * c0 + i] + gy[4 * c1 + i]) * 0.5;
        const double grad_dot = gxb * t0 + gyb * t1;
        gradx[i] = gxb - (grad_dot - grad_dir) * t0;
        grady[i] = gyb - (grad_dot - grad_dir) * t1;
    }
}

void ExplicitSolver::calc_least_squares_matrices() {  // solver.h:402-422
    lsq.assign(m.nRealCells, {0, 0, 0, 0});
    for (uint i = 0; i < m.nRealCells; ++i) {
        const uint size_i = m.cellsIsTriangle[i] ? 3 : 4;
        double a00 = 0, a01 = 0, a11 = 0;
        for (uint j = 0; j < size_i; ++j) {
            const uint e = m.cellsEdges[i][j];
            const uint cn = m.edgesCells[e][0] == i ? m.edgesCells[e][1] : m.edgesCells[e][0];
            const double dx = m.cellsCentersX[cn] - m.cellsCentersX[i];
            const double dy = m.cellsCentersY[cn] - m.cellsCentersY[i];
            a00 += dx * dx;
            a01 += dx * dy;
            a11 += dy * dy;
        }
        // closed-form 2×2 inverse (the reference calls Eigen's inverse())
        const double invdet = 1.0 / (a00 * a11 - a01 * a01);
        lsq[i] = {a11 * invdet, -a01 * invdet, -a01 * invdet, a00 * invdet};
    }
}

void ExplicitSolver::calc_gradients() {  // solver.h:425-514
    const size_t NT = m.cellsAreas.size();
    if (st.gradient == 1) {
        std::fill(gx.begin(), gx.end(), 0.);
        std::fill(gy.begin(), gy.end(), 0.);
        for (size_t e = 0; e < m.edgesNodes.size(); ++e) {
            const uint i = m.edgesCells[e][0], j = m.edgesCells[e][1];
            const double dxif = m.edgesCentersX[e] - m.cellsCentersX[i];
            const double dyif = m.edgesCentersY[e] - m.cellsCentersY[i];
            const double dif = std::sqrt(dxif * dxif + dyif * dyif);
            const double dxij = m.cellsCentersX[i] - m.cellsCentersX[j];
            const double dyij = m.cellsCentersY[i] - m.cellsCentersY[j];
            const double dij = std::sqrt(dxij * dxij + dyij * dyij);
            const double geom_factor = dif / dij;
            const double* qL = &q[4 * (size_t)i];
            double qR[4];
            boundary_state(st.g, edge_type[e], m.edgesNormalsX[e], m.edgesNormalsY[e], qL, &q[4 * (size_t)j], qR);
            for (int k = 0; k < 4; ++k) {
                const double fk = (qL[k] * (1.0 - geom_factor) + qR[k] * geom_factor) * m.edgesLengths[e];
                gx[4 * i + k] += fk * m.edgesNormalsX[e];
                gy[4 * i + k] += fk * m.edgesNormalsY[e];
                gx[4 * j + k] -= fk * m.edgesNormalsX[e];
                gy[4 * j + k] -= fk * m.edgesNormalsY[e];
            }
        }
        const int NR = (int)m.nRealCells;
#pragma omp parallel for
        for (int i = 0; i < NR; ++i)
            for (int k = 0; k < 4; ++k) {
                gx[4 * i + k] /= m.cellsAreas[i];
                gy[4 * i + k] /= m.cellsAreas[i];
            }
        for (size_t i = m.nRealCells; i < NT; ++i)
            for (int k = 0; k < 4; ++k) { gx[4 * i + k] *= 0; gy[4 * i + k] *= 0; }
    } else {
        for (uint i = 0; i < m.nRealCells; ++i) {
            const uint size_i = m.cellsIsTriangle[i] ? 3 : 4;
            double dx[4], dy[4], delta[4][4];
            for (uint j = 0; j < size_i; ++j) {
                const uint e = m.cellsEdges[i][j];
                const uint cn = m.edgesCells[e][0] == i ? m.edgesCells[e][1] : m.edgesCells[e][0];
                dx[j] = m.cellsCentersX[cn] - m.cellsCentersX[i];
                dy[j] = m.cellsCentersY[cn] - m.cellsCentersY[i];
                const double* qL = &q[4 * (size_t)i];
                double qR[4];
                boundary_state(st.g, edge_type[e], m.edgesNormalsX[e], m.edgesNormalsY[e], qL, &q[4 * (size_t)cn], qR);
                for (int k = 0; k < 4; ++k) delta[j][k] = qL[k] - qR[k];
            }
            const auto& M = lsq[i];
            for (int k = 0; k < 4; ++k) {
                double g0 = 0, g1 = 0;
                for (uint j = 0; j < size_i; ++j) {
                    const double p0 = M[0] * dx[j] + M[1] * dy[j];
                    const double p1 = M[2] * dx[j] + M[3] * dy[j];
                    g0 += p0 * delta[j][k];
                    g1 += p1 * delta[j][k];
                }
                gx[4 * i + k] = g0;
                gy[4 * i + k] = g1;
            }
        }
        for (size_t i = m.nRealCells; i < NT; ++i)
            for (int k = 0; k < 4; ++k) { gx[4 * i + k] *= 0; gy[4 * i + k] *= 0; }
    }
}

void ExplicitSolver::calc_limiters(const std::vector<double>& q_) {  // solver.h:517-593
    const int n4 = (int)limiters.size();
#pragma omp parallel for
    for (int i = 0; i < n4; ++i) { limiters[i] = 1; q_min[i] = q_[i]; q_max[i] = q_[i]; }
    for (size_t e = 0; e < m.edgesNodes.size(); ++e) {
        const uint i = m.edgesCells[e][0], j = m.edgesCells[e][1];
        for (int k = 0; k < 4; ++k) {
            q_min[4 * i + k] = std::min(q_min[4 * i + k], q_[4 * j + k]);
            q_min[4 * j + k] = std::min(q_min[4 * j + k], q_[4 * i + k]);
            q_max[4 * i + k] = std::max(q_max[4 * i + k], q_[4 * j + k]);
            q_max[4 * j + k] = std::max(q_max[4 * j + k], q_[4 * i + k]);
        }
    }
    for (size_t e = 0; e < m.edgesNodes.size(); ++e) {
        const uint ids[2] = {m.edgesCells[e][0], m.edgesCells[e][1]};
        for (uint id : ids) {
            if (id >= m.nRealCells) continue;
            const double dx = m.edgesCentersX[e] - m.cellsCentersX[id];
            const double dy = m.edgesCentersY[e] - m.cellsCentersY[id];
            const double sqrt_area = std::sqrt(m.cellsAreas[id]);
            for (int k = 0; k < 4; ++k) {
                double dqg = gx[4 * id + k] * dx + gy[4 * id + k] * dy;
                double delta_max = q_max[4 * id + k] - q_[4 * id + k];
                double delta_min = q_min[4 * id + k] - q_[4 * id + k];
                const double Ka = st.limiter_k * sqrt_area;
                const double K3a = Ka * Ka * Ka;
                const double dMaxMin2 = (delta_max - delta_min) * (delta_max - delta_min);
                double lim = 1.0;
                if (st.limiter == 1) {
                    double sig;
                    if (dMaxMin2 <= K3a) sig = 1.;
                    else if (dMaxMin2 <= 2 * K3a) {
                        const double y = (dMaxMin2 / K3a - 1.0);
                        sig = 2.0 * y * y * y - 3.0 * y * y + 1.0;
                    } else sig = 0.;
                    if (sig < 1.0) {
                        if (dqg > 1e-14) lim = michalak_limiter(delta_max / dqg);
                        else if (dqg < -1e-14) lim = michalak_limiter(delta_min / dqg);
                        else lim = 1.0;
                    }
                    lim = sig + (1.0 - sig) * lim;
                } else {
                    if (dqg > 1e-16) {
                        lim = 1 / dqg * ((delta_max * delta_max + K3a) * dqg + 2 * dqg * dqg * delta_max) /
                              (delta_max * delta_max + 2 * dqg * dqg + delta_max * dqg + K3a);
                    } else if (dqg < -1e-16) {
                        lim = 1 / dqg * ((delta_min * delta_min + K3a) * dqg + 2 * dqg * dqg * delta_min) /
                              (delta_min * delta_min + 2 * dqg * dqg + delta_min * dqg + K3a);
                    } else {
                        lim = 1.0;
                    }
                }
                limiters[4 * id + k] = std::min(limiters[4 * id + k], lim);
            }
        }
    }
}

void ExplicitSolver::flux(int type, uint e, const double qL[4], const double qR[4], const double gradx[4],
                          const double grady[4], double f[4]) const {
    const double nx = m.edgesNormalsX[e], ny = m.edgesNormalsY[e];
    if (two_sided(type) && st.viscosity == VISC_SA) {
        internal_flux(st.g, nx, ny, 0, qL, qR, gradx, grady, f);
        const double mut_f = 0.5 * (mut[m.edgesCells[e][0]] + mut[m.edgesCells[e][1]]);
        laminar_terms(st.g, st.g.mu_L + mut_f, st.g.cp * (st.g.mu_L / st.g.Pr_L + mut_f / st.g.Pr_T), nx, ny, qL, qR,
                      gradx, grady, f);
    } else if (two_sided(type)) {
        internal_flux(st.g, nx, ny, flux_visc(), qL, qR, gradx, grady, f);
    } else {  // boundary functors call the internal flux without gradients (physics.h:298,363,431)
        double qb[4];
        const double zero[4] = {0, 0, 0, 0};
        // Spalart-Allmaras: the inviscid part of a no-slip wall takes the
        // slip-wall ghost (pressure only); calc_residual adds the wall shear
        const int gt = (st.viscosity == VISC_SA && type == BC_WALL) ? BC_SLIP_WALL : type;
        boundary_state(st.g, gt, nx, ny, qL, qR, qb);
        internal_flux(st.g, nx, ny, flux_visc(), qL, qb, zero, zero, f);
    }
}

void ExplicitSolver::calc_residual(const std::vector<double>& q_) {  // solver.h:745-799
    std::fill(qW.begin(), qW.end(), 0.);
    for (size_t e = 0; e < m.edgesCells.size(); ++e) {
        const uint c0 = m.edgesCells[e][0], c1 = m.edgesCells[e][1];
        const size_t k0 = 4 * (size_t)c0, k1 = 4 * (size_t)c1;
        double gradx[4], grady[4], f[4];
        average_gradients(gradx, grady, c0, c1);
        if (st.second_order) {
            const double d0x = m.edgesCentersX[e] - m.cellsCentersX[c0];
            const double d0y = m.edgesCentersY[e] - m.cellsCentersY[c0];
            const double d1x = m.edgesCentersX[e] - m.cellsCentersX[c1];
            const double d1y = m.edgesCentersY[e] - m.cellsCentersY[c1];
            double qL[4], qR[4];
            for (int k = 0; k < 4; ++k) {
                qL[k] = q_[k0 + k] + (gx[k0 + k] * d0x + gy[k0 + k] * d0y) * limiters[k0 + k];
                qR[k] = q_[k1 + k] + (gx[k1 + k] * d1x + gy[k1 + k] * d1y) * limiters[k1 + k];
            }
            flux(edge_type[e], (uint)e, qL, qR, gradx, grady, f);
        } else {
            flux(edge_type[e], (uint)e, &q_[k0], &q_[k1], gradx, grady, f);
        }
        if (st.viscosity == VISC_SA && edge_type[e] == BC_WALL) sa_wall_shear((uint)e, &q_[k0], f);
        const double L = m.edgesLengths[e];
        const bool ts = two_sided(edge_type[e]);
        for (int k = 0; k < 4; ++k) {
            const double fl = f[k] * L;
            qW[k0 + k] -= fl;
            if (ts) qW[k1 + k] += fl;
        }
    }
    const int NR = (int)m.nRealCells;
#pragma omp parallel for
    for (int i = 0; i < NR; ++i)
        for (int j = 0; j < 4; ++j) qW[4 * i + j] /= m.cellsAreas[i];
}

static double norm2(const std::vector<double>& v) {
    double s = 0;
    for (double x : v) s += x * x;
    return std::sqrt(s);
}

double ExplicitSolver::solve() {  // solver.h:802-828
    static const double alpha[3] = {0.25, 0.5, 1.};
    const bool sa = st.viscosity == VISC_SA;
    calc_dt();
    qk = q;
    if (sa) nuk = nu;
    for (double ai : alpha) {
        if (viscous_or_grad() || st.second_order) {
            set_walls_from_internal(qk);
            calc_gradients();
            if (st.second_order) calc_limiters(qk);
        }
        // Spalart-Allmaras: eddy viscosity of the stage state, then the
        // mean-flow and turbulence residuals of the same stage state
        if (sa) calc_mut(qk, nuk);
        calc_residual(qk);
        if (sa) calc_nu_residual(qk, nuk);
        for (uint i = 0; i < m.nRealCells; ++i)
            for (int j = 0; j < 4; ++j)
                qk[4 * i + j] = q[4 * i + j] + qW[4 * i + j] * dt[i] * ai * st.relaxation;
        if (sa)
            for (uint i = 0; i < m.nRealCells; ++i) nuk[i] = nu[i] + nuW[i] * dt[i] * ai * st.relaxation;
    }
    q = qk;
    if (sa) nu = nuk;
    return norm2(qW);
}

double ExplicitSolver::get_uniform_residual() {  // solver.h:636-690
    BoundaryVars vf = get_boundary_variables();
    for (size_t i = m.nRealCells; i < m.cellsAreas.size(); ++i)
        for (int j = 0; j < 4; ++j) qW[4 * i + j] = 0;
    double qf[4];
    vf.conservative(st.g, qf);
    for (size_t e = 0; e < m.edgesCells.size(); ++e) {
        const uint c0 = m.edgesCells[e][0], c1 = m.edgesCells[e][1];
        double gradx[4], grady[4], f[4];
        average_gradients(gradx, grady, c0, c1);
        flux(edge_type[e], (uint)e, qf, qf, gradx, grady, f);
        const bool ts = two_sided(edge_type[e]);
        for (int i = 0; i < 4; ++i) {
            const double fl = f[i] * m.edgesLengths[e];
            qW[4 * c0 + i] -= fl;
            if (ts) qW[4 * c1 + i] += fl;
        }
    }
    return norm2(qW);
}

int ExplicitSolver::run_solver(int* iters_out, double* err_out, std::vector<double>* history) {
    // multigrid<explicitSolver>::run_solver, multigrid.h:182-237
    int i = 0;
    double err = 0;
    double err_0 = get_uniform_residual();
    do {
        err = solve();
        if ((i == 0) & (err > 2 * err_0)) err_0 = err;
        if (err > 0) err /= err_0;
        if (history && i % 10 == 0) history->push_back(err);
        i++;
    } while ((err > st.tolerance) && (i < st.max_iterations));
    *iters_out = i;
    *err_out = err;
    return 0;
}

WallProfile get_wall_profile(const ExplicitSolver& s, const std::string& patch) {  // post.h:301-387
    const BoundaryVars vf = s.get_boundary_variables();
    const double p_inf = vf.p, mach_inf = vf.mach, gam = s.st.g.gamma;
    const Mesh& m = s.m;
    WallProfile w;
    double xmin = 0., xmax = 0., y_moment = 0.;
    unsigned n_added = 0;
    bool first = true;
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
        if (m.boundaryEdgesPhysicals[b] != patch) continue;
        const uint e = m.boundaryEdges[b];
        if (first) {
            xmin = xmax = m.edgesCentersX[e];
            y_moment = m.edgesCentersY[e];
            first = false;
        } else {
            xmin = std::min(xmin, m.edgesCentersX[e]);
            xmax = std::max(xmax, m.edgesCentersX[e]);
            y_moment += m.edgesCentersY[e];
        }
        n_added += 1;
    }
    y_moment /= (double)n_added;
    const double x_moment = (xmax - xmin) * 0.25 + xmin;
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
        if (m.boundaryEdgesPhysicals[b] != patch) continue;
        const uint e = m.boundaryEdges[b];
        const uint cell = m.edgesCells[e][0];
        w.x.push_back(m.edgesCentersX[e]);
        w.y.push_back(m.edgesCentersY[e]);
        const double* qc = &s.q[4 * (size_t)cell];
        const double p = (gam - 1) * (qc[3] - 0.5 / qc[0] * (qc[1] * qc[1] + qc[2] * qc[2]));  // core.h:145-147
        const double cp = 2. / (gam * mach_inf * mach_inf) * (p / p_inf - 1.);
        w.cp.push_back(cp);
        const double ecx = m.edgesCentersX[e], ecy = m.edgesCentersY[e];
        const double fxi = cp * m.edgesNormalsX[e] * m.edgesLengths[e] / (xmax - xmin);
        const double fyi = cp * m.edgesNormalsY[e] * m.edgesLengths[e] / (xmax - xmin);
        const double mi = (ecx - x_moment) / (xmax - xmin) * fyi - (ecy - y_moment) / (xmax - xmin) * fxi;
        w.cd += fxi;
        w.cl += fyi;
        w.cm -= mi;
    }
    const double fx = w.cd, fy = w.cl, aoa = vf.angle;
    w.cd = fx * std::cos(aoa) + fy * std::sin(aoa);
    w.cl = -fx * std::sin(aoa) + fy * std::cos(aoa);
    return w;
}

}  // namespace oracle

// ------------------------------------------------------ multigrid.h:99-178
namespace oracle {
void prolongate(ExplicitSolver& coarse, ExplicitSolver& fine) {
    // bcs_from_internal (solver.h:276-287): ghost = its owner's state
    for (size_t b = 0; b < coarse.m.boundaryEdges.size(); ++b) {
        const uint e = coarse.m.boundaryEdges[b];
        const uint c0 = coarse.m.edgesCells[e][0], c1 = coarse.m.edgesCells[e][1];
        for (int k = 0; k < 4; ++k) coarse.q[4 * c1 + k] = coarse.q[4 * c0 + k];
    }
    const Mesh& cm = coarse.m;
    const Mesh& fm = fine.m;
    const size_t m = fm.cellsAreas.size(), n = cm.cellsAreas.size();
    std::vector<double> out(4 * m, 0.);
#pragma omp parallel for
    for (long i = 0; i < (long)m; ++i) {
        const double xi = fm.cellsCentersX[i], yi = fm.cellsCentersY[i];
        double scale = 0;
        for (size_t j = 0; j < n; ++j) {
            const double xj = cm.cellsCentersX[j], yj = cm.cellsCentersY[j];
            const double d2 = (xi - xj) * (xi - xj) + (yi - yj) * (yi - yj);
            const double r2 = cm.cellsAreas[j];
            if (d2 < 2 * r2) scale += 1 / std::max(0.1 * std::sqrt(r2), std::sqrt(d2));
        }
        // the mapper's column-major product adds the columns in order
        for (size_t j = 0; j < n; ++j) {
            const double xj = cm.cellsCentersX[j], yj = cm.cellsCentersY[j];
            const double d2 = (xi - xj) * (xi - xj) + (yi - yj) * (yi - yj);
            const double r2 = cm.cellsAreas[j];
            if (d2 < 2 * r2) {
                const double w = (1 / std::max(0.1 * std::sqrt(r2), std::sqrt(d2))) / scale;
                for (int k = 0; k < 4; ++k) out[4 * i + k] += w * coarse.q[4 * j + k];
            }
        }
    }
    fine.q = out;
    fine.refill_bcs();
}

// ------------------------------------------------------------ post.h:58-180
// save(): the same text the reference assembles.  Node coordinates through
// std::to_string (double2string is not used there), cell data through a
// fixed-notation stream with 16 digits (double2string, post.h:33-37), the
// derived fields of solution (core.h:119-164).
namespace {
std::string fixed16(double x) {
    std::ostringstream o;
    o << std::fixed << std::setprecision(16) << x;
    return o.str();
}
}  // namespace

std::string save_text(const Mesh& m, const double* q, const double* wd, const Gas& g) {
    const uint nc = m.nRealCells;
    auto rho = [&](uint i) { return q[4 * i]; };
    auto ru = [&](uint i) { return q[4 * i + 1]; };
    auto rv = [&](uint i) { return q[4 * i + 2]; };
    auto re = [&](uint i) { return q[4 * i + 3]; };
    auto pres = [&](uint i) { return (g.gamma - 1) * (re(i) - 0.5 / rho(i) * (ru(i) * ru(i) + rv(i) * rv(i))); };
    auto sound = [&](uint i) { return std::sqrt(g.gamma * pres(i) / rho(i)); };
    std::string t;
    t += "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n";
    t += "  <UnstructuredGrid>\n";
    t += "    <Piece NumberOfPoints=\"" + std::to_string(m.nodesX.size()) + "\" NumberOfCells=\"" +
         std::to_string(nc) + "\">\n";
    t += "      <Points>\n";
    t += "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n";
    for (size_t k = 0; k < m.nodesX.size(); ++k)
        t += "          " + std::to_string(m.nodesX[k]) + " " + std::to_string(m.nodesY[k]) + " 0.0\n";
    t += "        </DataArray>\n";
    t += "      </Points>\n";
    t += "      <Cells>\n";
    t += "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n";
    t += "          ";
    for (uint i = 0; i < nc; ++i) {
        const uint k = m.cellsIsTriangle[i] ? 3 : 4;
        for (uint j = 0; j < k; ++j) t += std::to_string(m.cellsNodes[i][j]) + "  ";
        t += "\n          ";
    }
    t += "        </DataArray>\n";
    t += "        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n";
    t += "          ";
    uint off = 0;
    for (uint i = 0; i < nc; ++i) {
        off += m.cellsIsTriangle[i] ? 3 : 4;
        t += std::to_string(off) + "  ";
    }
    t += "\n";
    t += "        </DataArray>\n";
    t += "        <DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n";
    t += "          ";
    for (uint i = 0; i < nc; ++i) t += m.cellsIsTriangle[i] ? "5  " : "9  ";
    t += "\n";
    t += "        </DataArray>\n";
    t += "      </Cells>\n";
    t += "      <CellData Scalars=\"scalars\">\n";
    auto field = [&](const char* name, auto f) {
        t += std::string("        <DataArray type=\"Float32\" Name=\"") + name + "\" Format=\"ascii\">\n";
        for (uint i = 0; i < nc; ++i) t += "          " + fixed16(f(i)) + "\n";
        t += "        </DataArray>\n";
    };
    field("Wall Distance", [&](uint i) { return wd ? wd[i] : m.wall_dist[i]; });
    field("Mach", [&](uint i) { return std::sqrt(ru(i) * ru(i) + rv(i) * rv(i)) / (rho(i) * sound(i)); });
    field("Density", rho);
    field("Pressure", pres);
    field("Temperature", [&](uint i) { return pres(i) / (g.R * rho(i)); });
    t += "        <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" Format=\"ascii\">\n";
    for (uint i = 0; i < nc; ++i) t += "          " + fixed16(ru(i) / rho(i)) + " " + fixed16(rv(i) / rho(i)) + " 0.0\n";
    t += "        </DataArray>\n";
    t += "      </CellData>\n";
    t += "    </Piece>\n";
    t += "  </UnstructuredGrid>\n";
    t += "</VTKFile>";
    return t;
}
}  // namespace oracle
