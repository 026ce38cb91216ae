// CPU ORACLE — test infrastructure only.  Spalart-Allmaras turbulence model
// for the oracle's explicit solver (viscosity VISC_SA).
//
// The reference has no SA model: its SA branch is empty (physics.h:259-261)
// and its nu / nuW arrays are unused (solver.h:55,59,187-188).  This file is
// therefore not a restatement of reference code but the FP64 definition
// that the GPU kernels (afx_sa.cuh) follow operation for operation.  The
// model is the published one-equation model of Spalart & Allmaras (1992,
// AIAA 92-0439, "A one-equation turbulence model for aerodynamic flows")
// without the trip term and without f_t2 ("SA-noft2"), with the negative-
// nu~ branch and the modified vorticity limit of Allmaras, Johnson &
// Spalart (2012, ICCFD7-1902, "Modifications and clarifications for the
// implementation of the Spalart-Allmaras turbulence model", "SA-neg"):
//
//   dnu~/dt + u.grad nu~ = P - D + (1/sigma) [div((nu + f_n nu~) grad nu~)
//                                             + c_b2 |grad nu~|^2]
//   nu~ >= 0:  chi = nu~/nu, f_v1 = chi^3/(chi^3 + c_v1^3),
//              f_v2 = 1 - chi/(1 + chi f_v1), S_bar = nu~ f_v2/(kappa^2 d^2),
//              S~ = Omega + S_bar                       if S_bar >= -c_v2 Omega
//                 = Omega + Omega (c_v2^2 Omega + c_v3 S_bar)
//                           / ((c_v3 - 2 c_v2) Omega - S_bar)    otherwise,
//              r = min(nu~/(S~ kappa^2 d^2), 10), g = r + c_w2 (r^6 - r),
//              f_w = g ((1 + c_w3^6)/(g^6 + c_w3^6))^(1/6),
//              P = c_b1 S~ nu~,  D = c_w1 f_w (nu~/d)^2,  f_n = 1
//   nu~ < 0:   P = c_b1 (1 - c_t3) Omega nu~,  D = -c_w1 (nu~/d)^2,
//              f_n = (c_n1 + chi^3)/(c_n1 - chi^3)
//   mu_t = rho nu~ f_v1 (nu~ >= 0), 0 otherwise.
//
// Discretisation (per real cell i, faces visited in ascending edge id):
// - convection: first-order upwind, -sum L min(V_f, 0)(nu~_j - nu~_i), with
//   V_f the outward normal of the mean of the two cell-centre velocities;
// - diffusion: two-point gradient along the centroid line, face coefficient
//   (nu_f + f_n nu~_f) from the face means, (nu~_j - nu~_i)(d.n)/(d.d);
// - c_b2 term with the Green-Gauss gradient of nu~ (face value = mean);
// - source with Omega = |dv/dx - du/dy| from the mean-flow cell gradients
//   and d the distance from the centroid to the nearest no-slip wall face
//   (point to segment; the reference's compute_wall_dist, mesh.h:794-830,
//   measures to face centres, which overstates d near a wall by half a face
//   length and weakens the destruction term there);
// - ghosts: nu~ = -nu~_i at no-slip walls (zero on the wall), nu~_i at slip
//   walls, 3 mu_L/rho_inf at the far field; ghost velocity and density from
//   the boundary functors' ghost state (physics.h:311-530).
// Mean flow: the reference's laminar terms (physics.h:230-258) with
// mu_L + mu_t,f and cp (mu_L/Pr_L + mu_t,f/Pr_T), mu_t,f the mean of the two
// cells.  At no-slip walls the reference's boundary flux has no viscous
// part, and its reflected ghost (momentum negated) puts a Roe dissipation on
// the tangential velocity that at high Reynolds numbers outweighs the
// physical shear several times.  Here the inviscid part takes the slip-wall
// ghost (tangential momentum kept: only the pressure acts) and the wall shear
// mu_L u_t / delta is added (u_t the cell's tangential velocity, delta the
// distance from its centroid to the wall face).
// Cube roots (f_w) by Newton-Raphson on y^3 = m after splitting off the
// exponent: only +, -, *, / and sqrt, so the GPU reproduces them bit for bit.
#include <algorithm>
#include <cmath>

#include "rans_oracle.hpp"

namespace oracle {

namespace {
constexpr double SA_CB1 = 0.1355, SA_SIGMA = 2.0 / 3.0, SA_CB2 = 0.622, SA_KAPPA = 0.41;
constexpr double SA_CW2 = 0.3, SA_CW3 = 2.0, SA_CV1 = 7.1, SA_CT3 = 1.2, SA_CN1 = 16.0;
constexpr double SA_CV2 = 0.7, SA_CV3 = 0.9;
constexpr double SA_CW1 = SA_CB1 / (SA_KAPPA * SA_KAPPA) + (1.0 + SA_CB2) / SA_SIGMA;
}  // namespace

double sa_cbrt(double x) {
    if (!(x > 0.)) return 0.;
    int e = 0;
    double mm = std::frexp(x, &e);  // x = mm 2^e, mm in [0.5, 1)
    const int r = ((e % 3) + 3) % 3;
    const int e3 = (e - r) / 3;
    mm = std::ldexp(mm, r);  // mm in [0.5, 4)
    double y = 0.7 + 0.3 * mm;
    for (int it = 0; it < 7; ++it) y = y - (y * y * y - mm) / (3. * y * y);
    return std::ldexp(y, e3);
}

void sa_source(double nut, double nul, double omega, double d, double* src, double* dsrc) {
    const double d2 = d * d;
    if (nut < 0.) {
        const double P = SA_CB1 * (1. - SA_CT3) * omega * nut;
        const double D = -SA_CW1 * (nut * nut) / d2;
        *src = P - D;
        *dsrc = SA_CB1 * (1. - SA_CT3) * omega + 2. * SA_CW1 * nut / d2;
        return;
    }
    const double cv13 = SA_CV1 * SA_CV1 * SA_CV1;
    const double chi = nut / nul;
    const double chi3 = chi * chi * chi;
    const double fv1 = chi3 / (chi3 + cv13);
    const double dfv1 = 3. * chi * chi * cv13 / ((chi3 + cv13) * (chi3 + cv13)) / nul;
    const double fv2 = 1. - chi / (1. + chi * fv1);
    const double dfv2 = -(1. / nul - chi * chi * dfv1) / ((1. + chi * fv1) * (1. + chi * fv1));
    const double kd2 = SA_KAPPA * SA_KAPPA * d2;
    const double Sbar = nut * fv2 / kd2;
    const double dSbar = (fv2 + nut * dfv2) / kd2;
    double Stil, dStil;
    if (Sbar >= -SA_CV2 * omega) {
        Stil = omega + Sbar;
        dStil = dSbar;
    } else {
        const double num = SA_CV2 * SA_CV2 * omega + SA_CV3 * Sbar;
        const double den = (SA_CV3 - 2. * SA_CV2) * omega - Sbar;
        Stil = omega + omega * num / den;
        dStil = omega * dSbar * (SA_CV3 * den + num) / (den * den);
    }
    double r = 10., dr = 0.;
    if (Stil > 0.) {
        const double rr = nut / (Stil * kd2);
        if (rr < 10.) {
            r = rr;
            dr = (Stil - nut * dStil) / (Stil * Stil * kd2);
        }
    }
    const double r2 = r * r;
    const double g = r + SA_CW2 * (r2 * r2 * r2 - r);
    const double dg = (1. + SA_CW2 * (6. * r2 * r2 * r - 1.)) * dr;
    const double cw36 = SA_CW3 * SA_CW3 * SA_CW3 * SA_CW3 * SA_CW3 * SA_CW3;
    const double g2 = g * g;
    const double g6 = g2 * g2 * g2;
    const double s6 = std::sqrt(sa_cbrt((1. + cw36) / (g6 + cw36)));
    const double fw = g * s6;
    const double dfw = s6 * cw36 / (g6 + cw36) * dg;
    const double P = SA_CB1 * Stil * nut;
    const double D = SA_CW1 * fw * (nut * nut) / d2;
    *src = P - D;
    *dsrc = SA_CB1 * (dStil * nut + Stil) - SA_CW1 * (dfw * (nut * nut) + fw * 2. * nut) / d2;
}

void ExplicitSolver::sa_setup() {
    const size_t N = m.cellsAreas.size();
    nu.assign(N, 0.);
    nuk.assign(N, 0.);
    nuW.assign(N, 0.);
    mut.assign(N, 0.);
    cellFaces.assign(m.nRealCells, {EDGE_NULL, EDGE_NULL, EDGE_NULL, EDGE_NULL});
    for (uint i = 0; i < m.nRealCells; ++i) {
        std::array<uint, 4> f = m.cellsEdges[i];
        std::sort(f.begin(), f.end());  // EDGE_NULL (the largest value) sorts last
        cellFaces[i] = f;
    }
    sa_wall_distance();
    double qf[4];
    get_boundary_variables().conservative(st.g, qf);
    nu_far = 3. * st.g.mu_L / qf[0];
    sa_init();
}

// Distance from each real cell's centroid to the nearest no-slip wall face
// (a segment), faces scanned in boundary order; 1e15 without a wall.
void ExplicitSolver::sa_wall_distance() {
    std::vector<double> seg;  // ax, ay, bx, by per wall face
    for (size_t b = 0; b < m.boundaryEdges.size(); ++b)
        if (st.bcs.at(m.boundaryEdgesPhysicals[b]).type == BC_WALL) {
            const uint e = m.boundaryEdges[b];
            seg.push_back(m.nodesX[m.edgesNodes[e][0]]);
            seg.push_back(m.nodesY[m.edgesNodes[e][0]]);
            seg.push_back(m.nodesX[m.edgesNodes[e][1]]);
            seg.push_back(m.nodesY[m.edgesNodes[e][1]]);
        }
    const int NR = (int)m.nRealCells;
    sa_wd.assign(NR, 1e15);
#pragma omp parallel for
    for (int i = 0; i < NR; ++i) {
        const double cx = m.cellsCentersX[i], cy = m.cellsCentersY[i];
        double mind = 1e15;
        bool first = true;
        for (size_t k = 0; k < seg.size(); k += 4) {
            const double ex = seg[k + 2] - seg[k], ey = seg[k + 3] - seg[k + 1];
            const double px = cx - seg[k], py = cy - seg[k + 1];
            double t = (px * ex + py * ey) / (ex * ex + ey * ey);
            t = t < 0. ? 0. : (t > 1. ? 1. : t);
            const double dx = px - t * ex, dy = py - t * ey;
            const double d = std::sqrt(dx * dx + dy * dy);
            if (first) {
                mind = d;
                first = false;
            } else {
                mind = std::min(mind, d);
            }
        }
        sa_wd[i] = mind;
    }
}

void ExplicitSolver::sa_init() {
    for (uint i = 0; i < m.nRealCells; ++i) nu[i] = nu_far;
}

void ExplicitSolver::calc_mut(const std::vector<double>& q_, const std::vector<double>& nu_) {
    const double cv13 = SA_CV1 * SA_CV1 * SA_CV1;
    const int NR = (int)m.nRealCells;
#pragma omp parallel for
    for (int i = 0; i < NR; ++i) {
        const double rho = q_[4 * i];
        const double nt = nu_[i];
        if (nt >= 0.) {
            const double chi = nt * rho / st.g.mu_L;
            const double chi3 = chi * chi * chi;
            mut[i] = rho * nt * (chi3 / (chi3 + cv13));
        } else {
            mut[i] = 0.;
        }
    }
}

void ExplicitSolver::sa_wall_shear(uint e, const double q0[4], double f[4]) const {
    const uint c = m.edgesCells[e][0];
    const double nx = m.edgesNormalsX[e], ny = m.edgesNormalsY[e];
    const double d0x = m.edgesCentersX[e] - m.cellsCentersX[c];
    const double d0y = m.edgesCentersY[e] - m.cellsCentersY[c];
    const double delta = std::fabs(d0x * nx + d0y * ny);
    const double u = q0[1] / q0[0], v = q0[2] / q0[0];
    const double un = u * nx + v * ny;
    f[1] += st.g.mu_L * (u - un * nx) / delta;
    f[2] += st.g.mu_L * (v - un * ny) / delta;
}

void ExplicitSolver::calc_nu_residual(const std::vector<double>& q_, const std::vector<double>& nu_) {
    const double mu = st.g.mu_L;
    const int NR = (int)m.nRealCells;
#pragma omp parallel for
    for (int i = 0; i < NR; ++i) {
        const double rho_i = q_[4 * i];
        const double u_i = q_[4 * i + 1] / rho_i, v_i = q_[4 * i + 2] / rho_i;
        const double nul_i = mu / rho_i;
        const double nut_i = nu_[i];
        const double du_dy = (rho_i * gy[4 * i + 1] - q_[4 * i + 1] * gy[4 * i]) / (rho_i * rho_i);
        const double dv_dx = (rho_i * gx[4 * i + 2] - q_[4 * i + 2] * gx[4 * i]) / (rho_i * rho_i);
        const double omega = std::fabs(dv_dx - du_dy);
        double conv = 0., diff = 0., ggx = 0., ggy = 0.;
        for (int s = 0; s < 4; ++s) {
            const uint e = cellFaces[i][s];
            if (e == EDGE_NULL) break;
            const uint c0 = m.edgesCells[e][0], c1 = m.edgesCells[e][1];
            const bool own = c0 == (uint)i;
            const uint j = own ? c1 : c0;
            const double nox = own ? m.edgesNormalsX[e] : -m.edgesNormalsX[e];
            const double noy = own ? m.edgesNormalsY[e] : -m.edgesNormalsY[e];
            const double L = m.edgesLengths[e];
            double rho_j, u_j, v_j, nut_j;
            if (j < m.nRealCells) {
                rho_j = q_[4 * j];
                u_j = q_[4 * j + 1] / rho_j;
                v_j = q_[4 * j + 2] / rho_j;
                nut_j = nu_[j];
            } else {
                const int t = edge_type[e];
                double qg[4];
                boundary_state(st.g, t, m.edgesNormalsX[e], m.edgesNormalsY[e], &q_[4 * i], &q_[4 * j], qg);
                rho_j = qg[0];
                u_j = qg[1] / qg[0];
                v_j = qg[2] / qg[0];
                nut_j = t == BC_WALL ? -nut_i : (t == BC_FARFIELD ? nu_far : nut_i);
            }
            const double nul_j = mu / rho_j;
            const double un = 0.5 * (u_i + u_j) * nox + 0.5 * (v_i + v_j) * noy;
            conv += L * std::min(un, 0.) * (nut_j - nut_i);
            const double dx = m.cellsCentersX[j] - m.cellsCentersX[i];
            const double dy = m.cellsCentersY[j] - m.cellsCentersY[i];
            const double ddn = dx * nox + dy * noy;
            const double dd = dx * dx + dy * dy;
            const double nuf = 0.5 * (nul_i + nul_j);
            const double ntf = 0.5 * (nut_i + nut_j);
            double fn = 1.;
            if (ntf < 0.) {
                const double chi = ntf / nuf;
                const double chi3 = chi * chi * chi;
                fn = (SA_CN1 + chi3) / (SA_CN1 - chi3);
            }
            diff += L * (nuf + fn * ntf) * (nut_j - nut_i) * ddn / dd;
            ggx += ntf * nox * L;
            ggy += ntf * noy * L;
        }
        const double A = m.cellsAreas[i];
        const double gnx = ggx / A, gny = ggy / A;
        double src, dsrc;
        sa_source(nut_i, nul_i, omega, sa_wd[i], &src, &dsrc);
        const double R = -conv + diff / SA_SIGMA + SA_CB2 / SA_SIGMA * (gnx * gnx + gny * gny) * A + src * A;
        nuW[i] = R / A;
    }
}

}  // namespace oracle
