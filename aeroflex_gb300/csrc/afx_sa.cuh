// Spalart-Allmaras turbulence model on the GPU (viscosity "spalart-allmaras").
//
// The reference has no SA model (physics.h:259-261 is an empty branch, the
// nu / nuW arrays of solver.h:55,59 are unused), so this is the project's own
// model, written from the published equations: Spalart & Allmaras (1992,
// AIAA 92-0439) without trip and f_t2 terms, with the negative-nu~ branch and
// the modified-vorticity limit of Allmaras, Johnson & Spalart (2012,
// ICCFD7-1902, "SA-neg").  The FP64 CPU oracle (oracle/sa_oracle.cpp) states
// the same definition; in FP64 (-fmad=false) every operation here follows its
// order, so the GPU result is bit-identical to it.
//
// Per real cell i, faces in ascending reference edge id (the cslot order):
//   R_i = -sum L min(V_f, 0)(nu~_j - nu~_i)                         upwind convection
//         + (1/sigma) sum L (nu_f + f_n nu~_f)(nu~_j - nu~_i)(d.n)/(d.d)   diffusion
//         + (c_b2/sigma) |grad nu~_i|^2 A_i + (P - D) A_i
//   dnu~_i/dt = R_i / A_i.
// V_f: outward normal component of the mean of the two cell-centre
// velocities; d = c_j - c_i (centroids; a ghost's mirrored centroid on
// boundary faces); grad nu~ by Green-Gauss with face means; Omega =
// |dv/dx - du/dy| from the mean flow's cell gradients; ghost nu~ = -nu~_i at
// no-slip walls, nu~_i at slip walls, 3 mu_L / rho_inf at the far field.
// Mean flow (afx_device.cuh, face_flux with VISC 2): the reference's laminar
// terms with mu_L + mu_t; at no-slip walls the inviscid flux of the slip-wall
// ghost (the reflected ghost's Roe dissipation on the tangential velocity
// would outweigh the physical shear at high Reynolds numbers) plus the wall
// shear mu_L u_t / delta.
#pragma once

#include "afx_kernels.cuh"

namespace afx {
namespace dev {

constexpr double SA_CB1 = 0.1355, SA_SIGMA = 2.0 / 3.0, SA_CB2 = 0.622, SA_KAPPA = 0.41;
constexpr double SA_CW2 = 0.3, SA_CW3 = 2.0, SA_CV1 = 7.1, SA_CT3 = 1.2, SA_CN1 = 16.0;
constexpr double SA_CV2 = 0.7, SA_CV3 = 0.9;
constexpr double SA_CW1 = SA_CB1 / (SA_KAPPA * SA_KAPPA) + (1.0 + SA_CB2) / SA_SIGMA;

__device__ __forceinline__ double sa_frexp(double x, int* e) { return frexp(x, e); }
__device__ __forceinline__ float sa_frexp(float x, int* e) { return frexpf(x, e); }
__device__ __forceinline__ double sa_ldexp(double x, int e) { return ldexp(x, e); }
__device__ __forceinline__ float sa_ldexp(float x, int e) { return ldexpf(x, e); }

// Cube root by Newton-Raphson on y^3 = m, m the mantissa scaled into
// [0.5, 4) by splitting off a multiple of 3 from the exponent: only +, -, *,
// / (the oracle's sa_cbrt, step for step).
template <class T>
__device__ __forceinline__ T sa_cbrt(T x) {
    if (!(x > T(0))) return T(0);
    int e = 0;
    T mm = sa_frexp(x, &e);
    const int r = ((e % 3) + 3) % 3;
    const int e3 = (e - r) / 3;
    mm = sa_ldexp(mm, r);
    T y = T(0.7) + T(0.3) * mm;
#pragma unroll 1
    for (int it = 0; it < 7; ++it) y = y - (y * y * y - mm) / (T(3) * y * y);
    return sa_ldexp(y, e3);
}

// P - D of one cell and its derivative in nu~ (the oracle's sa_source).
template <class T>
__device__ __forceinline__ void sa_source(const T nut, const T nul, const T omega, const T d, T* src, T* dsrc) {
    const T d2 = d * d;
    if (nut < T(0)) {
        const T P = T(SA_CB1) * (T(1) - T(SA_CT3)) * omega * nut;
        const T D = -T(SA_CW1) * (nut * nut) / d2;
        *src = P - D;
        *dsrc = T(SA_CB1) * (T(1) - T(SA_CT3)) * omega + T(2) * T(SA_CW1) * nut / d2;
        return;
    }
    const T cv13 = T(SA_CV1) * T(SA_CV1) * T(SA_CV1);
    const T chi = nut / nul;
    const T chi3 = chi * chi * chi;
    const T fv1 = chi3 / (chi3 + cv13);
    const T dfv1 = T(3) * chi * chi * cv13 / ((chi3 + cv13) * (chi3 + cv13)) / nul;
    const T fv2 = T(1) - chi / (T(1) + chi * fv1);
    const T dfv2 = -(T(1) / nul - chi * chi * dfv1) / ((T(1) + chi * fv1) * (T(1) + chi * fv1));
    const T kd2 = T(SA_KAPPA) * T(SA_KAPPA) * d2;
    const T Sbar = nut * fv2 / kd2;
    const T dSbar = (fv2 + nut * dfv2) / kd2;
    T Stil, dStil;
    if (Sbar >= -T(SA_CV2) * omega) {
        Stil = omega + Sbar;
        dStil = dSbar;
    } else {
        const T num = T(SA_CV2) * T(SA_CV2) * omega + T(SA_CV3) * Sbar;
        const T den = (T(SA_CV3) - T(2) * T(SA_CV2)) * omega - Sbar;
        Stil = omega + omega * num / den;
        dStil = omega * dSbar * (T(SA_CV3) * den + num) / (den * den);
    }
    T r = T(10), dr = T(0);
    if (Stil > T(0)) {
        const T rr = nut / (Stil * kd2);
        if (rr < T(10)) {
            r = rr;
            dr = (Stil - nut * dStil) / (Stil * Stil * kd2);
        }
    }
    const T r2 = r * r;
    const T g = r + T(SA_CW2) * (r2 * r2 * r2 - r);
    const T dg = (T(1) + T(SA_CW2) * (T(6) * r2 * r2 * r - T(1))) * dr;
    const T cw36 = T(SA_CW3) * T(SA_CW3) * T(SA_CW3) * T(SA_CW3) * T(SA_CW3) * T(SA_CW3);
    const T g2 = g * g;
    const T g6 = g2 * g2 * g2;
    const T s6 = dsqrt(sa_cbrt((T(1) + cw36) / (g6 + cw36)));
    const T fw = g * s6;
    const T dfw = s6 * cw36 / (g6 + cw36) * dg;
    const T P = T(SA_CB1) * Stil * nut;
    const T D = T(SA_CW1) * fw * (nut * nut) / d2;
    *src = P - D;
    *dsrc = T(SA_CB1) * (dStil * nut + Stil) - T(SA_CW1) * (dfw * (nut * nut) + fw * T(2) * nut) / d2;
}

// The pointers of one SA evaluation (device cell order).
template <class T>
struct SaView {
    const double* __restrict__ nu0;  // nu~ of the iteration's start state
    const double* __restrict__ nuk;  // nu~ of the stage state
    double* __restrict__ nu_next;    // stage output (null: residual only)
    double* __restrict__ nuW;        // R / A
    const T* __restrict__ wd;        // wall distance
    const V2<T>* __restrict__ cxy;   // centroids
    const V2<T>* __restrict__ gxy;   // ghost centroids, per boundary face
    const T* __restrict__ dt;
    T nu_far;
    double alpha, relax;
};

// Eddy viscosity mu_t = rho nu~ f_v1 (0 for nu~ < 0) of a stage state.
template <class T, class S>
__global__ void __launch_bounds__(256) k_sa_mut(const int n, const V4<S>* __restrict__ qk,
                                                const double* __restrict__ nuk, const T mu, T* __restrict__ mut,
                                                const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T q[4];
    ld4s(&qk[i], q);
    const T rho = q[0];
    const T nt = (T)__ldg(&nuk[i]);
    T out = T(0);
    if (nt >= T(0)) {
        const T cv13 = T(SA_CV1) * T(SA_CV1) * T(SA_CV1);
        const T chi = nt * rho / mu;
        const T chi3 = chi * chi * chi;
        out = rho * nt * (chi3 / (chi3 + cv13));
    }
    mut[i] = out;
}

// R_i (not divided by the area) of cell i, and with DIAG the diagonal of the
// point-implicit update: A/dt + sum of the neighbour couplings + destruction.
template <class T, class S, bool DIAG>
__device__ __forceinline__ T sa_cell_residual(const KM<T>& m, const V4<S>* __restrict__ qk,
                                              const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                              const SaView<T>& v, const int i, T* diag) {
    T qi[4], gxi[4], gyi[4];
    ld4s(&qk[i], qi);
    ld4c<T>(&gx[i], gxi);
    ld4c<T>(&gy[i], gyi);
    const T rho_i = qi[0];
    const T u_i = qi[1] / rho_i, v_i = qi[2] / rho_i;
    const T nul_i = m.mu / rho_i;
    const T nut_i = (T)__ldg(&v.nuk[i]);
    const T du_dy = (rho_i * gyi[1] - qi[1] * gyi[0]) / (rho_i * rho_i);
    const T dv_dx = (rho_i * gxi[2] - qi[2] * gxi[0]) / (rho_i * rho_i);
    const T omega = dabs(dv_dx - du_dy);
    const V2<T> ci = __ldg(&v.cxy[i]);
    const int4 sl = __ldg(&m.cslot[i]);
    const int4 nb = __ldg(&m.cnbr[i]);
    T conv = T(0), diff = T(0), ggx = T(0), ggy = T(0), couple = T(0);
#pragma unroll 1
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(sl, s);
        if (fs == 0) continue;
        const bool own0 = fs > 0;
        const int f = (own0 ? fs : -fs) - 1;
        const int oc = pick(nb, s);
        const V2<T> n = __ldg(&m.fn[f]);
        const T nox = own0 ? n.x : -n.x;
        const T noy = own0 ? n.y : -n.y;
        const T L = __ldg(&m.fLg[f]).x;
        T rho_j, u_j, v_j, nut_j;
        V2<T> cj;
        if (oc >= 0) {
            T qj[4];
            ld4s(&qk[oc], qj);
            rho_j = qj[0];
            u_j = qj[1] / rho_j;
            v_j = qj[2] / rho_j;
            nut_j = (T)__ldg(&v.nuk[oc]);
            cj = __ldg(&v.cxy[oc]);
        } else {
            const int b = -oc - 1;
            const int bt = __ldg(&m.btype[b]);
            T qb[4], qg[4];
            ld4c<T>(&m.bq[b], qb);
            ghost_state(bt, m.gamma, n.x, n.y, qi, qb, qg);
            rho_j = qg[0];
            u_j = qg[1] / qg[0];
            v_j = qg[2] / qg[0];
            nut_j = bt == BT_WALL ? -nut_i : (bt == BT_FARFIELD ? v.nu_far : nut_i);
            cj = __ldg(&v.gxy[b]);
        }
        const T nul_j = m.mu / rho_j;
        const T un = T(0.5) * (u_i + u_j) * nox + T(0.5) * (v_i + v_j) * noy;
        conv += L * smin(un, T(0)) * (nut_j - nut_i);
        const T dx = cj.x - ci.x;
        const T dy = cj.y - ci.y;
        const T ddn = dx * nox + dy * noy;
        const T dd = dx * dx + dy * dy;
        const T nuf = T(0.5) * (nul_i + nul_j);
        const T ntf = T(0.5) * (nut_i + nut_j);
        T fn = T(1);
        if (ntf < T(0)) {
            const T chi = ntf / nuf;
            const T chi3 = chi * chi * chi;
            fn = (T(SA_CN1) + chi3) / (T(SA_CN1) - chi3);
        }
        diff += L * (nuf + fn * ntf) * (nut_j - nut_i) * ddn / dd;
        ggx += ntf * nox * L;
        ggy += ntf * noy * L;
        if (DIAG)
            couple += L * (-smin(un, T(0))) + L * smax(nuf + fn * ntf, T(0)) * smax(ddn, T(0)) / dd / T(SA_SIGMA);
    }
    const T A = __ldg(&m.area[i]);
    const T gnx = ggx / A, gny = ggy / A;
    T src, dsrc;
    sa_source(nut_i, nul_i, omega, __ldg(&v.wd[i]), &src, &dsrc);
    if (DIAG) *diag = A / __ldg(&v.dt[i]) + couple + A * smax(-dsrc, T(0));
    return -conv + diff / T(SA_SIGMA) + T(SA_CB2) / T(SA_SIGMA) * (gnx * gnx + gny * gny) * A + src * A;
}

// One RK stage of nu~ (solver.h:802-828 applied to the SA equation): R / A
// of the stage state into nuW, and the stage update nu0 + R/A dt alpha relax
// (nu_next null: the residual only).
template <class T, class S>
__global__ void __launch_bounds__(256) k_sa_stage(const KM<T> m, const V4<S>* __restrict__ qk,
                                                  const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                                  const SaView<T> v, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_cells) return;
    const T R = sa_cell_residual<T, S, false>(m, qk, gx, gy, v, i, nullptr);
    const T nuW = R / __ldg(&m.area[i]);
    v.nuW[i] = (double)nuW;
    if (v.nu_next) {
        const T inc = nuW * __ldg(&v.dt[i]) * (T)v.alpha * (T)v.relax;
        v.nu_next[i] = __ldg(&v.nu0[i]) + (double)inc;
    }
}

// Point-implicit nu~ update of the implicit solver: nu_next = nu~ + relax R /
// (A/dt + couplings + destruction), from the stage state nuk.
template <class T, class S>
__global__ void __launch_bounds__(256) k_sa_implicit(const KM<T> m, const V4<S>* __restrict__ qk,
                                                     const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                                     const SaView<T> v, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_cells) return;
    T diag = T(1);
    const T R = sa_cell_residual<T, S, true>(m, qk, gx, gy, v, i, &diag);
    v.nuW[i] = (double)(R / __ldg(&m.area[i]));
    v.nu_next[i] = __ldg(&v.nuk[i]) + (double)((T)v.relax * R / diag);
}

}  // namespace dev
}  // namespace afx
