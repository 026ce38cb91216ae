// Device side of the GB300 rans residual path: face physics and the kernels
// of one explicit iteration, templated on the arithmetic type T (double for
// the FP64 path, float for the FP32-mixed path).
//
// Bit parity (FP64): this header is compiled with -fmad=false and every
// expression keeps the operand order and grouping of AeroFLEX's source, so
// each face flux, gradient, limiter and time step equals the reference's
// definition bit for bit.  Per-cell sums visit the cell's faces in the
// reference's edge order (the device layout stores them that way), which
// reproduces the serial edge loops' accumulation order without atomics.
//
// Layout in HBM (N cells, F faces, B boundary faces):
//   cell vectors  q, gx, gy, phi : one 4-vector per cell (32 B FP64 / 16 B FP32)
//   cslot  int4 per cell: its faces (device ids), ascending reference edge id
//   faces  int2 (c0, c1; c1 < 0 marks boundary -(b+1)), and T2 pairs
//          n = (nx, ny), Lg = (length, Green-Gauss weight), d0, d1 = face
//          centre minus cell-0 / cell-1 centroid
#pragma once

#include <cuda_runtime.h>

#include "afx_launch.hpp"

namespace afx {
namespace dev {

struct __align__(32) d4 {
    double x, y, z, w;
};

template <class T> struct V2t;
template <> struct V2t<double> { using type = double2; };
template <> struct V2t<float> { using type = float2; };
template <class T> struct V4t;
template <> struct V4t<double> { using type = d4; };
template <> struct V4t<float> { using type = float4; };
template <class T> using V2 = typename V2t<T>::type;
template <class T> using V4 = typename V4t<T>::type;

enum { BT_INTERNAL = 0, BT_FARFIELD = 1, BT_SLIP = 2, BT_WALL = 3, BT_INOUT = 4 };

__device__ __forceinline__ void ld4(const d4* p, double* v) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldg(q), b = __ldg(q + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void ld4(const float4* p, float* v) {
    float4 a = __ldg(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
template <class T>
__device__ __forceinline__ void ld4c(const V4<T>* p, T* v) { ld4(p, v); }
__device__ __forceinline__ d4 ldv4d(const d4* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldg(q), b = __ldg(q + 1);
    d4 r;
    r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y;
    return r;
}
__device__ __forceinline__ float4 ldv4d(const float4* p) { return __ldg(p); }
template <class T>
__device__ __forceinline__ V4<T> ldv4(const V4<T>* p) { return ldv4d(p); }
// load a state stored as S into T registers
__device__ __forceinline__ void ld4s(const d4* p, double* v) { ld4(p, v); }
__device__ __forceinline__ void ld4s(const float4* p, float* v) { ld4(p, v); }
__device__ __forceinline__ void ld4s(const d4* p, float* v) {
    double t[4];
    ld4(p, t);
    for (int k = 0; k < 4; ++k) v[k] = (float)t[k];
}

__device__ __forceinline__ void st4(d4* p, const double* v) {
    double2* q = reinterpret_cast<double2*>(p);
    q[0] = make_double2(v[0], v[1]);
    q[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ void st4(float4* p, const float* v) { *p = make_float4(v[0], v[1], v[2], v[3]); }
__device__ __forceinline__ void st4(float4* p, const double* v) {
    *p = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
}

__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
__device__ __forceinline__ float dabs(float x) { return fabsf(x); }

// std::min / std::max semantics: min(a,b) = (b < a) ? b : a; max(a,b) = (a < b) ? b : a
template <class T> __device__ __forceinline__ T smin(T a, T b) { return (b < a) ? b : a; }
template <class T> __device__ __forceinline__ T smax(T a, T b) { return (a < b) ? b : a; }

// Kernel view of the mesh and physics.
template <class T>
struct KM {
    int n_cells;
    const int4* __restrict__ cslot;  // +(face+1) if the cell is the face's cell 0, -(face+1) if cell 1, 0 empty
    const int4* __restrict__ cnbr;   // the face's other cell, or -(b+1) for boundary face b
    const T* __restrict__ area;
    const int2* __restrict__ fcell;
    const V2<T>* __restrict__ fn;
    const V2<T>* __restrict__ fLg;
    const V2<T>* __restrict__ fd0;
    const V2<T>* __restrict__ fd1;
    const V4<T>* __restrict__ ft;
    const int* __restrict__ btype;
    const V4<T>* __restrict__ bq;
    T gamma, R, mu, kheat, limk, cfl;
    int limiter;
    int lsq;                          // least-squares gradient
    const V2<T>* __restrict__ lsqw;   // 4 per cell: (M d_j) of local edge j
    const int* __restrict__ lsqs;     // per cell: slot of local edge j (2 bits each), edge count << 8
    // Spalart-Allmaras (VISC 2): eddy viscosity of the stage state per cell,
    // and the gas constants of the turbulent heat conductivity
    const T* __restrict__ mut;
    T cp, PrL, PrT;
};

__device__ __forceinline__ bool two_sided(int bt) { return bt == BT_INTERNAL || bt == BT_INOUT; }

// ---------------------------------------------------------------- physics
// sabs and entropy_correction, physics.h:84-86, 133-135
template <class T> __device__ __forceinline__ T sabs(T x) { return dsqrt(x * x + T(1e-4)); }
template <class T> __device__ __forceinline__ T entropy_corr(T l, T d) {
    return l > d ? l : (l * l + d * d) / (T(2) * d);
}

// Central flux + Roe dissipation with Harten's entropy fix, physics.h:168-228.
template <class T>
__device__ __forceinline__ void roe_flux(const T gamma, const T nx, const T ny, const T* qL, const T* qR, T* f) {
    const T rho_L = qL[0], rho_u_L = qL[1], rho_v_L = qL[2], rho_e_L = qL[3];
    const T rho_R = qR[0], rho_u_R = qR[1], rho_v_R = qR[2], rho_e_R = qR[3];
    const T V_L = (rho_u_L * nx + rho_v_L * ny) / rho_L;
    const T V_R = (rho_u_R * nx + rho_v_R * ny) / rho_R;
    const T p_L = (gamma - T(1)) * (rho_e_L - T(0.5) / rho_L * (rho_u_L * rho_u_L + rho_v_L * rho_v_L));
    const T p_R = (gamma - T(1)) * (rho_e_R - T(0.5) / rho_R * (rho_u_R * rho_u_R + rho_v_R * rho_v_R));
    f[0] = (V_L * rho_L + V_R * rho_R) * T(0.5);
    f[1] = (V_L * rho_u_L + p_L * nx + V_R * rho_u_R + p_R * nx) * T(0.5);
    f[2] = (V_L * rho_v_L + p_L * ny + V_R * rho_v_R + p_R * ny) * T(0.5);
    f[3] = (V_L * (rho_e_L + p_L) + V_R * (rho_e_R + p_R)) * T(0.5);
    const T pL = p_L, pR = p_R;
    const T uL = qL[1] / qL[0];
    const T uR = qR[1] / qR[0];
    const T vL = qL[2] / qL[0];
    const T vR = qR[2] / qR[0];
    const T srhoL = dsqrt(qL[0]);
    const T srhoR = dsqrt(qR[0]);
    const T rho = srhoR * srhoL;
    const T u = (uL * srhoL + uR * srhoR) / (srhoL + srhoR);
    const T v = (vL * srhoL + vR * srhoR) / (srhoL + srhoR);
    const T h = ((qL[3] + pL) / qL[0] * srhoL + (qR[3] + pR) / qR[0] * srhoR) / (srhoL + srhoR);
    const T q2 = u * u + v * v;
    const T c = dsqrt((gamma - T(1)) * (h - T(0.5) * q2));
    const T V = u * nx + v * ny;
    const T VR = uR * nx + vR * ny;
    const T VL = uL * nx + vL * ny;
    const T lambda_cm = entropy_corr(sabs(V - c), T(0.05) * c);
    const T lambda_c = entropy_corr(sabs(V), T(0.05) * c);
    const T lambda_cp = entropy_corr(sabs(V + c), T(0.05) * c);
    const T kF1 = lambda_cm * ((pR - pL) - rho * c * (VR - VL)) / (T(2) * c * c);
    const T kF234_0 = lambda_c * ((qR[0] - qL[0]) - (pR - pL) / (c * c));
    const T kF234_1 = lambda_c * rho;
    const T kF5 = lambda_cp * ((pR - pL) + rho * c * (VR - VL)) / (T(2) * c * c);
    f[0] -= T(0.5) * (kF1 + kF234_0 + kF5);
    f[1] -= T(0.5) * (kF1 * (u - c * nx) + kF234_0 * u + kF234_1 * (uR - uL - (VR - VL) * nx) + kF5 * (u + c * nx));
    f[2] -= T(0.5) * (kF1 * (v - c * ny) + kF234_0 * v + kF234_1 * (vR - vL - (VR - VL) * ny) + kF5 * (v + c * ny));
    f[3] -= T(0.5) * (kF1 * (h - c * V) + kF234_0 * q2 * T(0.5) +
                      kF234_1 * (u * (uR - uL) + v * (vR - vL) - V * (VR - VL)) + kF5 * (h + c * V));
}

// Laminar viscous flux at the mean state, physics.h:230-258 with
// calc_grad_p / calc_grad_temp / calc_grad_u / calc_grad_v (physics.h:33-82).
template <class T>
__device__ __forceinline__ void laminar_flux(const T gamma, const T Rgas, const T mu, const T kheat, const T nx,
                                             const T ny, const T* qL, const T* qR, const T* gx, const T* gy, T* f) {
    T qc[4];
    for (int k = 0; k < 4; ++k) qc[k] = T(0.5) * (qL[k] + qR[k]);
    const T p = (gamma - T(1)) * (qc[3] - T(0.5) / qc[0] * (qc[1] * qc[1] + qc[2] * qc[2]));
    T gp0 = T(2) * gx[3];
    gp0 -= gx[1] * qc[1] / qc[0] + qc[1] * (gx[1] * qc[0] - gx[0] * qc[1]) / (qc[0] * qc[0]);
    gp0 -= gx[2] * qc[2] / qc[0] + qc[2] * (gx[2] * qc[0] - gx[0] * qc[2]) / (qc[0] * qc[0]);
    gp0 *= T(0.5) * (gamma - T(1));
    T gp1 = T(2) * gy[3];
    gp1 -= gy[1] * qc[1] / qc[0] + qc[1] * (gy[1] * qc[0] - gy[0] * qc[1]) / (qc[0] * qc[0]);
    gp1 -= gy[2] * qc[2] / qc[0] + qc[2] * (gy[2] * qc[0] - gy[0] * qc[2]) / (qc[0] * qc[0]);
    gp1 *= T(0.5) * (gamma - T(1));
    const T gT0 = (T(1) / Rgas) * ((gp0 * qc[0] - gx[0] * p) / (qc[0] * qc[0]));
    const T gT1 = (T(1) / Rgas) * ((gp1 * qc[0] - gy[0] * p) / (qc[0] * qc[0]));
    const T gu0 = (qc[0] * gx[1] - qc[1] * gx[0]) / (qc[0] * qc[0]);
    const T gu1 = (qc[0] * gy[1] - qc[1] * gy[0]) / (qc[0] * qc[0]);
    const T gv0 = (qc[0] * gx[2] - qc[2] * gx[0]) / (qc[0] * qc[0]);
    const T gv1 = (qc[0] * gy[2] - qc[2] * gy[0]) / (qc[0] * qc[0]);
    const T div_v = gu0 + gv1;
    const T tau_xx = T(2) * mu * (gu0 - div_v / T(3));
    const T tau_yy = T(2) * mu * (gv1 - div_v / T(3));
    const T tau_xy = mu * (gu1 + gv0);
    const T phi0 = qc[1] / qc[0] * tau_xx + qc[2] / qc[0] * tau_xy + kheat * gT0;
    const T phi1 = qc[1] / qc[0] * tau_xy + qc[2] / qc[0] * tau_yy + kheat * gT1;
    f[1] -= nx * tau_xx + ny * tau_xy;
    f[2] -= nx * tau_xy + ny * tau_yy;
    f[3] -= nx * phi0 + ny * phi1;
}

// Boundary ghost state from the interior state qL and the stored boundary
// state qbc: slip wall (physics.h:311-339), wall (physics.h:377-405),
// farfield characteristics (physics.h:446-530, with the outside `va` of the
// subsonic outlet, line 524), internal average otherwise (physics.h:267-276).
template <class T>
__device__ __forceinline__ void ghost_state(const int type, const T gamma, const T nx, const T ny, const T* qL,
                                            const T* qbc, T* qR) {
    if (type == BT_SLIP) {
        const T rhoV = qL[1] * nx + qL[2] * ny;
        qR[0] = qL[0];
        qR[1] = qL[1] - T(2) * rhoV * nx;
        qR[2] = qL[2] - T(2) * rhoV * ny;
        qR[3] = qL[3];
        return;
    }
    if (type == BT_WALL) {
        qR[0] = qL[0]; qR[1] = -qL[1]; qR[2] = -qL[2]; qR[3] = qL[3];
        return;
    }
    if (type != BT_FARFIELD) {
        for (int k = 0; k < 4; ++k) qR[k] = (qL[k] + qbc[k]) * T(0.5);
        return;
    }
    const T rho = qL[0], rho_u = qL[1], rho_v = qL[2], rho_e = qL[3];
    const T bc_rho = qbc[0], bc_rhou = qbc[1], bc_rhov = qbc[2], bc_rhoe = qbc[3];
    const T bc_u = bc_rhou / bc_rho;
    const T bc_v = bc_rhov / bc_rho;
    const T bc_p = (gamma - T(1)) * (bc_rhoe - T(0.5) / bc_rho * (bc_rhou * bc_rhou + bc_rhov * bc_rhov));
    const T p = (gamma - T(1)) * (rho_e - T(0.5) / rho * (rho_u * rho_u + rho_v * rho_v));
    const T c = dsqrt(gamma * p / rho);
    const T mach = dsqrt(rho_u * rho_u + rho_v * rho_v) / (rho * c);
    const T inlet_outlet = rho_u * nx + rho_v * ny;
    if (mach > T(1)) {
        if (inlet_outlet < T(0)) {
            qR[0] = bc_rho;
            qR[1] = bc_rho * bc_u;
            qR[2] = bc_rho * bc_v;
            qR[3] = bc_p / (gamma - T(1)) + T(0.5) * bc_rho * (bc_u * bc_u + bc_v * bc_v);
        } else {
            qR[0] = rho; qR[1] = rho_u; qR[2] = rho_v; qR[3] = rho_e;
        }
    } else {
        const T pa = bc_p, rhoa = bc_rho, ua = bc_u, va = bc_v;
        const T pd = p, rhod = rho, ud = rho_u / rho, vd = rho_v / rho;
        const T rho0 = rho, c0 = c;
        if (inlet_outlet < T(0)) {
            const T pb = T(0.5) * (pa + pd - rho0 * c0 * (nx * (ua - ud) + ny * (va - vd)));
            qR[0] = rhoa + (pb - pa) / (c0 * c0);
            qR[1] = qR[0] * (ua - nx * (pa - pb) / (rho0 * c0));
            qR[2] = qR[0] * (va - ny * (pa - pb) / (rho0 * c0));
            qR[3] = pb / (gamma - T(1)) + T(0.5) / qR[0] * (qR[1] * qR[1] + qR[2] * qR[2]);
        } else {
            const T pb = pa;
            qR[0] = rhod + (pb - pd) / (c0 * c0);
            qR[1] = qR[0] * (ud + nx * (pd - pb) / (rho0 * c0));
            qR[2] = qR[0] * (va + ny * (pd - pb) / (rho0 * c0));
            qR[3] = pb / (gamma - T(1)) + T(0.5) / qR[0] * (qR[1] * qR[1] + qR[2] * qR[2]);
        }
    }
}

// Face flux F (not yet times length) of the reference's per-face functor:
// internal faces (and frozen-ghost boundaries) with the face gradient for the
// laminar term; wall/farfield faces through their ghost state without
// gradients (physics.h:287-299, 352-364, 417-432).  With zero gradients the
// laminar term is exactly zero, so boundary faces skip it.
// VISC 2 (Spalart-Allmaras): the laminar terms with mu_L + mu_t,f and
// cp (mu_L / Pr_L + mu_t,f / Pr_T), mu_t,f the mean of the face's two cells.
template <class T, int VISC>
__device__ __forceinline__ void face_flux(const KM<T>& m, const int bt, const T nx, const T ny, const T* qL,
                                          const T* qR, const T* fgx, const T* fgy, T* f, const T mut_f = T(0)) {
    if (two_sided(bt)) {
        roe_flux(m.gamma, nx, ny, qL, qR, f);
        if (VISC == 1) laminar_flux(m.gamma, m.R, m.mu, m.kheat, nx, ny, qL, qR, fgx, fgy, f);
        if (VISC == 2)
            laminar_flux(m.gamma, m.R, m.mu + mut_f, m.cp * (m.mu / m.PrL + mut_f / m.PrT), nx, ny, qL, qR, fgx, fgy,
                         f);
    } else {
        // VISC 2: the inviscid part of a no-slip wall takes the slip-wall
        // ghost (pressure only); the caller adds the wall shear
        T qb[4];
        ghost_state(VISC == 2 && bt == BT_WALL ? BT_SLIP : bt, m.gamma, nx, ny, qL, qR, qb);
        roe_flux(m.gamma, nx, ny, qL, qb, f);
    }
}

// Spalart-Allmaras no-slip wall: the wall shear mu_L u_t / delta of the cell
// state q0 (u_t its tangential velocity, delta the distance from its centroid
// to the wall face, d0 = face centre - centroid), added to the face flux F.
template <class T>
__device__ __forceinline__ void sa_wall_shear(const KM<T>& m, const T nx, const T ny, const T d0x, const T d0y,
                                              const T* q0, T* f) {
    const T delta = dabs(d0x * nx + d0y * ny);
    const T u = q0[1] / q0[0], v = q0[2] / q0[0];
    const T un = u * nx + v * ny;
    f[1] += m.mu * (u - un * nx) / delta;
    f[2] += m.mu * (v - un * ny) / delta;
}

// Spectral radius (c + |V_n|) of one side, solver.h:329-344.
template <class T>
__device__ __forceinline__ T face_eig(const T gamma, const T nx, const T ny, const T* q) {
    const T V = (q[1] * nx + q[2] * ny) / q[0];
    const T p = (gamma - T(1)) * (q[3] - T(0.5) / q[0] * (q[1] * q[1] + q[2] * q[2]));
    return dsqrt(p * gamma / q[0]) + dabs(V);
}

// Venkatakrishnan limiter of one cell-face-variable (solver.h:578-584) and
// the Michalak variant (solver.h:557-576, physics.h:581-592).
template <class T>
__device__ __forceinline__ T limiter_value(const int kind, const T dqg, const T delta_max, const T delta_min,
                                           const T K3a) {
    if (kind == 0) {
        if (dqg > T(1e-16)) {
            return T(1) / dqg * ((delta_max * delta_max + K3a) * dqg + T(2) * dqg * dqg * delta_max) /
                   (delta_max * delta_max + T(2) * dqg * dqg + delta_max * dqg + K3a);
        } else if (dqg < T(-1e-16)) {
            return T(1) / dqg * ((delta_min * delta_min + K3a) * dqg + T(2) * dqg * dqg * delta_min) /
                   (delta_min * delta_min + T(2) * dqg * dqg + delta_min * dqg + K3a);
        }
        return T(1);
    }
    const T dMaxMin2 = (delta_max - delta_min) * (delta_max - delta_min);
    T sig;
    if (dMaxMin2 <= K3a) sig = T(1);
    else if (dMaxMin2 <= T(2) * K3a) {
        const T y = (dMaxMin2 / K3a - T(1));
        sig = T(2) * y * y * y - T(3) * y * y + T(1);
    } else sig = T(0);
    T lim = T(1);
    if (sig < T(1)) {
        T y = T(2);
        bool set = false;
        if (dqg > T(1e-14)) { y = delta_max / dqg; set = true; }
        else if (dqg < T(-1e-14)) { y = delta_min / dqg; set = true; }
        if (set) {
            const T YT = T(2);
            const T a = T(1) / (YT * YT) - T(2) / (YT * YT * YT);
            const T b = -T(3) / T(2) * a * YT - T(0.5) / YT;
            lim = (y >= YT) ? T(1) : a * y * y * y + b * y * y + y;
        }
    }
    return sig + (T(1) - sig) * lim;
}

}  // namespace dev
}  // namespace afx
