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
    const int4* __restrict__ cslot;
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
template <class T, int VISC>
__device__ __forceinline__ void face_flux(const KM<T>& m, const int bt, const T nx, const T ny, const T* qL,
                                          const T* qR, const T* fgx, const T* fgy, T* f) {
    if (two_sided(bt)) {
        roe_flux(m.gamma, nx, ny, qL, qR, f);
        if (VISC == 1) laminar_flux(m.gamma, m.R, m.mu, m.kheat, nx, ny, qL, qR, fgx, fgy, f);
    } else {
        T qb[4];
        ghost_state(bt, m.gamma, nx, ny, qL, qR, qb);
        roe_flux(m.gamma, nx, ny, qL, qb, f);
    }
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

// ------------------------------------------------------------------ kernels

// Per cell, from the iteration's starting state q (the solver's member q):
// local time step (solver.h:308-356), Green-Gauss gradient (solver.h:428-469)
// and, when second order, the first stage's neighbour min/max and limiter
// (solver.h:517-593).  One gather over the cell's faces in edge order.
template <class T, class S, bool GRAD, bool SECOND>
__global__ void __launch_bounds__(256) k_prep(const KM<T> m, const V4<S>* __restrict__ q, V4<T>* __restrict__ gx,
                                              V4<T>* __restrict__ gy, V4<T>* __restrict__ phi,
                                              T* __restrict__ dt, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_cells) return;
    const int4 sl = __ldg(&m.cslot[i]);
    const int slots[4] = {sl.x, sl.y, sl.z, sl.w};
    T qi[4];
    ld4s(&q[i], qi);
    T sgx[4] = {T(0), T(0), T(0), T(0)}, sgy[4] = {T(0), T(0), T(0), T(0)};
    T qmn[4], qmx[4];
    for (int k = 0; k < 4; ++k) { qmn[k] = qi[k]; qmx[k] = qi[k]; }
    T eigsum = T(0);
    for (int s = 0; s < 4; ++s) {
        const int f = slots[s];
        if (f < 0) break;
        const int2 cc = __ldg(&m.fcell[f]);
        const bool own0 = (cc.x == i);
        const V2<T> n = __ldg(&m.fn[f]);
        const V2<T> Lg = __ldg(&m.fLg[f]);
        T qo[4];
        int bt = BT_INTERNAL;
        if (cc.y >= 0) {
            ld4s(&q[own0 ? cc.y : cc.x], qo);
        } else {
            const int b = -cc.y - 1;
            bt = __ldg(&m.btype[b]);
            ld4c<T>(&m.bq[b], qo);
        }
        const T* q0c = own0 ? qi : qo;  // state of the face's cell 0
        const T* q1c = own0 ? qo : qi;  // state of the face's cell 1 (ghost: boundary state)
        // time step
        T eig;
        if (two_sided(bt)) {
            const T eL = face_eig(m.gamma, n.x, n.y, q0c);
            const T eR = face_eig(m.gamma, n.x, n.y, q1c);
            eig = smax(eL, eR);
        } else {
            eig = face_eig(m.gamma, n.x, n.y, q0c);
        }
        eigsum += eig * Lg.x;
        if (GRAD) {
            T qRv[4];
            ghost_state(bt, m.gamma, n.x, n.y, q0c, q1c, qRv);
            const T g = Lg.y;
            for (int k = 0; k < 4; ++k) {
                const T fk = (q0c[k] * (T(1) - g) + qRv[k] * g) * Lg.x;
                if (own0) {
                    sgx[k] += fk * n.x;
                    sgy[k] += fk * n.y;
                } else {
                    sgx[k] -= fk * n.x;
                    sgy[k] -= fk * n.y;
                }
            }
        }
        if (SECOND && bt != BT_SLIP && bt != BT_WALL) {
            for (int k = 0; k < 4; ++k) {
                qmn[k] = smin(qmn[k], qo[k]);
                qmx[k] = smax(qmx[k], qo[k]);
            }
        }
    }
    const T A = __ldg(&m.area[i]);
    dt[i] = m.cfl * A / eigsum;
    if (!GRAD) return;
    T gxi[4], gyi[4];
    for (int k = 0; k < 4; ++k) {
        gxi[k] = sgx[k] / A;
        gyi[k] = sgy[k] / A;
    }
    V4<T> vx, vy;
    st4(&vx, gxi);
    st4(&vy, gyi);
    gx[i] = vx;
    gy[i] = vy;
    if (!SECOND) return;
    T lim[4] = {T(1), T(1), T(1), T(1)};
    const T sqrt_area = dsqrt(A);
    const T Ka = m.limk * sqrt_area;
    const T K3a = Ka * Ka * Ka;
    for (int s = 0; s < 4; ++s) {
        const int f = slots[s];
        if (f < 0) break;
        const int2 cc = __ldg(&m.fcell[f]);
        const V2<T> d = (cc.x == i) ? __ldg(&m.fd0[f]) : __ldg(&m.fd1[f]);
        for (int k = 0; k < 4; ++k) {
            const T dqg = gxi[k] * d.x + gyi[k] * d.y;
            const T dmax = qmx[k] - qi[k];
            const T dmin = qmn[k] - qi[k];
            lim[k] = smin(lim[k], limiter_value(m.limiter, dqg, dmax, dmin, K3a));
        }
    }
    V4<T> vp;
    st4(&vp, lim);
    phi[i] = vp;
}

// Limiter of a later RK stage state qk with the iteration's gradients
// (solver.h:517-593; stages 2 and 3 of solver.h:808-816).
template <class T, class S>
__global__ void __launch_bounds__(256) k_limiter(const KM<T> m, const V4<S>* __restrict__ qk,
                                                 const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                                 V4<T>* __restrict__ phi, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_cells) return;
    const int4 sl = __ldg(&m.cslot[i]);
    const int slots[4] = {sl.x, sl.y, sl.z, sl.w};
    T qi[4], gxi[4], gyi[4];
    ld4s(&qk[i], qi);
    ld4c<T>(&gx[i], gxi);
    ld4c<T>(&gy[i], gyi);
    T qmn[4], qmx[4];
    for (int k = 0; k < 4; ++k) { qmn[k] = qi[k]; qmx[k] = qi[k]; }
    for (int s = 0; s < 4; ++s) {
        const int f = slots[s];
        if (f < 0) break;
        const int2 cc = __ldg(&m.fcell[f]);
        T qo[4];
        if (cc.y >= 0) {
            ld4s(&qk[cc.x == i ? cc.y : cc.x], qo);
        } else {
            const int b = -cc.y - 1;
            const int bt = __ldg(&m.btype[b]);
            if (bt == BT_SLIP || bt == BT_WALL) continue;
            ld4c<T>(&m.bq[b], qo);
        }
        for (int k = 0; k < 4; ++k) {
            qmn[k] = smin(qmn[k], qo[k]);
            qmx[k] = smax(qmx[k], qo[k]);
        }
    }
    const T A = __ldg(&m.area[i]);
    T lim[4] = {T(1), T(1), T(1), T(1)};
    const T sqrt_area = dsqrt(A);
    const T Ka = m.limk * sqrt_area;
    const T K3a = Ka * Ka * Ka;
    for (int s = 0; s < 4; ++s) {
        const int f = slots[s];
        if (f < 0) break;
        const int2 cc = __ldg(&m.fcell[f]);
        const V2<T> d = (cc.x == i) ? __ldg(&m.fd0[f]) : __ldg(&m.fd1[f]);
        for (int k = 0; k < 4; ++k) {
            const T dqg = gxi[k] * d.x + gyi[k] * d.y;
            lim[k] = smin(lim[k], limiter_value(m.limiter, dqg, qmx[k] - qi[k], qmn[k] - qi[k], K3a));
        }
    }
    V4<T> vp;
    st4(&vp, lim);
    phi[i] = vp;
}

// Second-order reconstruction of one side, solver.h:780-781:
// q + (gx*dx + gy*dy) .* phi
template <class T>
__device__ __forceinline__ void reconstruct(const T* q, const T* gxc, const T* gyc, const T* ph, const V2<T> d,
                                            T* out) {
    for (int k = 0; k < 4; ++k) out[k] = q[k] + (gxc[k] * d.x + gyc[k] * d.y) * ph[k];
}

// average_gradients (solver.h:359-398) for the laminar face flux: member
// state qa/qb and gradients of the face's two cells, direction from the
// precomputed sum-of-centroids vector t = (t0, t1, lij).
template <class T>
__device__ __forceinline__ void face_gradient(const T* qa, const T* qb, const T* gxa, const T* gya, const T* gxb,
                                              const T* gyb, const V4<T> t, T* fgx, T* fgy) {
    const T t0 = t.x, t1 = t.y, lij = t.z;
    for (int k = 0; k < 4; ++k) {
        const T grad_dir = (qa[k] - qb[k]) / lij;
        const T gxb_ = (gxa[k] + gxb[k]) * T(0.5);
        const T gyb_ = (gya[k] + gyb[k]) * T(0.5);
        const T grad_dot = gxb_ * t0 + gyb_ * t1;
        fgx[k] = gxb_ - (grad_dot - grad_dir) * t0;
        fgy[k] = gyb_ - (grad_dot - grad_dir) * t1;
    }
}

// All inputs one face needs, for one side: stage state, gradient, limiter.
template <class T, class S, bool SECOND>
__device__ __forceinline__ void side_state(const V4<S>* __restrict__ qk, const V4<T>* __restrict__ gx,
                                           const V4<T>* __restrict__ gy, const V4<T>* __restrict__ phi,
                                           const int c, const V2<T> d, T* out) {
    T qc[4];
    ld4s(&qk[c], qc);
    if (!SECOND) {
        for (int k = 0; k < 4; ++k) out[k] = qc[k];
        return;
    }
    T gxc[4], gyc[4], pc[4];
    ld4c<T>(&gx[c], gxc);
    ld4c<T>(&gy[c], gyc);
    ld4c<T>(&phi[c], pc);
    reconstruct(qc, gxc, gyc, pc, d, out);
}

// F*L of face f for stage state qk (solver.h:751-786), returned in fl; the
// boundary state of a ghost side is used as is (ghost gradient is zero).
template <class T, class S, int VISC, bool SECOND>
__device__ __forceinline__ void face_flux_L(const KM<T>& m, const int f, const int2 cc,
                                            const V4<S>* __restrict__ qk, const V4<S>* __restrict__ qmem,
                                            const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                            const V4<T>* __restrict__ phi, T* fl, int* btp) {
    const V2<T> n = __ldg(&m.fn[f]);
    const V2<T> Lg = __ldg(&m.fLg[f]);
    T qL[4], qR[4];
    side_state<T, S, SECOND>(qk, gx, gy, phi, cc.x, __ldg(&m.fd0[f]), qL);
    int bt = BT_INTERNAL;
    if (cc.y >= 0) {
        side_state<T, S, SECOND>(qk, gx, gy, phi, cc.y, __ldg(&m.fd1[f]), qR);
    } else {
        const int b = -cc.y - 1;
        bt = __ldg(&m.btype[b]);
        ld4c<T>(&m.bq[b], qR);
    }
    T fgx[4] = {T(0), T(0), T(0), T(0)}, fgy[4] = {T(0), T(0), T(0), T(0)};
    if (VISC == 1 && two_sided(bt)) {
        T qa[4], qb[4], gxa[4], gya[4], gxb[4], gyb[4];
        ld4s(&qmem[cc.x], qa);
        ld4c<T>(&gx[cc.x], gxa);
        ld4c<T>(&gy[cc.x], gya);
        if (cc.y >= 0) {
            ld4s(&qmem[cc.y], qb);
            ld4c<T>(&gx[cc.y], gxb);
            ld4c<T>(&gy[cc.y], gyb);
        } else {
            ld4c<T>(&m.bq[-cc.y - 1], qb);
            for (int k = 0; k < 4; ++k) { gxb[k] = T(0); gyb[k] = T(0); }
        }
        face_gradient(qa, qb, gxa, gya, gxb, gyb, ldv4<T>(&m.ft[f]), fgx, fgy);
    }
    T F[4];
    face_flux<T, VISC>(m, bt, n.x, n.y, qL, qR, fgx, fgy, F);
    for (int k = 0; k < 4; ++k) fl[k] = F[k] * Lg.x;
    *btp = bt;
}

// Per-stage epilogue of one cell: R = sum/area (solver.h:794-798), the RK
// update qk = q + R*dt*alpha*relaxation (solver.h:818-821) in FP64, and the
// squared norm of qW (solver.h:827) for the last stage.
template <class T, class S>
struct StageOut {
    const d4* __restrict__ q0;   // FP64 iteration start state (member q)
    V4<S>* __restrict__ qnext;   // next stage state in S (stages 0, 1)
    d4* __restrict__ qm_next;    // FP64 new state (stage 2)
    V4<S>* __restrict__ qsh_next;  // new state in S (stage 2, FP32-mixed shadow), may be null
    d4* __restrict__ Rq;         // qW mirror (residual-only launches)
    const T* __restrict__ dt;
    double alpha, relax;
    double* __restrict__ partials;
    int mode;                    // 0 stage 0/1, 1 stage 2 (+norm), 2 residual only (write R)
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0) {
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    }
    return t;
}

template <class T, class S>
__device__ __forceinline__ void stage_epilogue(const StageOut<T, S>& o, const int i, const bool active, const T* Rsum,
                                               const T A, const double extra_sq, double* sh) {
    double sq = extra_sq;
    if (active) {
        T R[4];
        for (int k = 0; k < 4; ++k) R[k] = Rsum[k] / A;
        if (o.mode == 2) {
            double Rd[4] = {(double)R[0], (double)R[1], (double)R[2], (double)R[3]};
            st4(&o.Rq[i], Rd);
        } else {
            double q0[4];
            ld4(&o.q0[i], q0);
            const double dti = (double)o.dt[i];
            double qn[4];
            for (int k = 0; k < 4; ++k) qn[k] = q0[k] + (double)R[k] * dti * o.alpha * o.relax;
            if (o.mode == 0) {
                V4<S> v;
                st4(&v, qn);
                o.qnext[i] = v;
            } else {
                st4(&o.qm_next[i], qn);
                if (o.qsh_next) {
                    V4<S> v;
                    st4(&v, qn);
                    o.qsh_next[i] = v;
                }
                for (int k = 0; k < 4; ++k) sq += (double)R[k] * (double)R[k];
            }
        }
    }
    if (o.mode == 1) {
        const double t = block_sum(sq, sh);
        if (threadIdx.x == 0) o.partials[blockIdx.x] = t;
    }
}

// Cell gather: each cell recomputes the fluxes of its faces (interior faces
// are evaluated twice, identically) and sums them in edge order.  No face
// buffer; this is the HBM-lean variant.
template <class T, class S, int VISC, bool SECOND>
__global__ void __launch_bounds__(256) k_resid_gather(const KM<T> m, const V4<S>* __restrict__ qk,
                                                      const V4<S>* __restrict__ qmem,
                                                      const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                                      const V4<T>* __restrict__ phi, const StageOut<T, S> o,
                                                      const Ctrl* __restrict__ ctrl) {
    __shared__ double sh[32];
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < m.n_cells;
    T Rs[4] = {T(0), T(0), T(0), T(0)};
    double extra = 0;
    T A = T(1);
    if (active) {
        const int4 sl = __ldg(&m.cslot[i]);
        const int slots[4] = {sl.x, sl.y, sl.z, sl.w};
        for (int s = 0; s < 4; ++s) {
            const int f = slots[s];
            if (f < 0) break;
            const int2 cc = __ldg(&m.fcell[f]);
            T fl[4];
            int bt;
            face_flux_L<T, S, VISC, SECOND>(m, f, cc, qk, qmem, gx, gy, phi, fl, &bt);
            if (cc.x == i) {
                for (int k = 0; k < 4; ++k) Rs[k] -= fl[k];
                if (cc.y < 0 && two_sided(bt))
                    for (int k = 0; k < 4; ++k) extra += (double)fl[k] * (double)fl[k];
            } else {
                for (int k = 0; k < 4; ++k) Rs[k] += fl[k];
            }
        }
        A = __ldg(&m.area[i]);
    }
    stage_epilogue<T, S>(o, i, active, Rs, A, o.mode == 1 ? extra : 0.0, sh);
}

// Face variant, part 1: F*L of every face once (FP64 path: the flux is the
// expensive part on GB300's FP64 pipe, so it is not evaluated twice).
template <class T, class S, int VISC, bool SECOND>
__global__ void __launch_bounds__(256) k_face_flux(const KM<T> m, const int n_faces, const V4<S>* __restrict__ qk,
                                                   const V4<S>* __restrict__ qmem, const V4<T>* __restrict__ gx,
                                                   const V4<T>* __restrict__ gy, const V4<T>* __restrict__ phi,
                                                   V4<T>* __restrict__ fflux, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_faces) return;
    const int2 cc = __ldg(&m.fcell[f]);
    T fl[4];
    int bt;
    face_flux_L<T, S, VISC, SECOND>(m, f, cc, qk, qmem, gx, gy, phi, fl, &bt);
    V4<T> v;
    st4(&v, fl);
    fflux[f] = v;
}

// Face variant, part 2: ordered per-cell sum of the face fluxes + epilogue.
template <class T, class S>
__global__ void __launch_bounds__(256) k_cell_sum(const KM<T> m, const V4<T>* __restrict__ fflux,
                                                  const StageOut<T, S> o, const Ctrl* __restrict__ ctrl) {
    __shared__ double sh[32];
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < m.n_cells;
    T Rs[4] = {T(0), T(0), T(0), T(0)};
    double extra = 0;
    T A = T(1);
    if (active) {
        const int4 sl = __ldg(&m.cslot[i]);
        const int slots[4] = {sl.x, sl.y, sl.z, sl.w};
        for (int s = 0; s < 4; ++s) {
            const int f = slots[s];
            if (f < 0) break;
            const int2 cc = __ldg(&m.fcell[f]);
            T fl[4];
            ld4c<T>(&fflux[f], fl);
            if (cc.x == i) {
                for (int k = 0; k < 4; ++k) Rs[k] -= fl[k];
                if (cc.y < 0 && two_sided(__ldg(&m.btype[-cc.y - 1])))
                    for (int k = 0; k < 4; ++k) extra += (double)fl[k] * (double)fl[k];
            } else {
                for (int k = 0; k < 4; ++k) Rs[k] += fl[k];
            }
        }
        A = __ldg(&m.area[i]);
    }
    stage_epilogue<T, S>(o, i, active, Rs, A, o.mode == 1 ? extra : 0.0, sh);
}

// get_uniform_residual (solver.h:636-690): qW keeps its previous real-cell
// entries and gains the freestream fluxes (not divided by the area).
template <class T, class S, int VISC>
__global__ void __launch_bounds__(256) k_uniform(const KM<T> m, const V4<S>* __restrict__ qmem,
                                                 const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                                 const double q0, const double q1, const double q2, const double q3,
                                                 d4* __restrict__ Rq, double* __restrict__ partials) {
    __shared__ double sh[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0;
    if (i < m.n_cells) {
        const T qf[4] = {(T)q0, (T)q1, (T)q2, (T)q3};
        double acc[4];
        ld4(&Rq[i], acc);
        T accT[4] = {(T)acc[0], (T)acc[1], (T)acc[2], (T)acc[3]};
        const int4 sl = __ldg(&m.cslot[i]);
        const int slots[4] = {sl.x, sl.y, sl.z, sl.w};
        for (int s = 0; s < 4; ++s) {
            const int f = slots[s];
            if (f < 0) break;
            const int2 cc = __ldg(&m.fcell[f]);
            const V2<T> n = __ldg(&m.fn[f]);
            const V2<T> Lg = __ldg(&m.fLg[f]);
            int bt = BT_INTERNAL;
            if (cc.y < 0) bt = __ldg(&m.btype[-cc.y - 1]);
            T fgx[4] = {T(0), T(0), T(0), T(0)}, fgy[4] = {T(0), T(0), T(0), T(0)};
            if (VISC == 1 && two_sided(bt)) {
                T qa[4], qb[4], gxa[4], gya[4], gxb[4], gyb[4];
                ld4s(&qmem[cc.x], qa);
                ld4c<T>(&gx[cc.x], gxa);
                ld4c<T>(&gy[cc.x], gya);
                if (cc.y >= 0) {
                    ld4s(&qmem[cc.y], qb);
                    ld4c<T>(&gx[cc.y], gxb);
                    ld4c<T>(&gy[cc.y], gyb);
                } else {
                    ld4c<T>(&m.bq[-cc.y - 1], qb);
                    for (int k = 0; k < 4; ++k) { gxb[k] = T(0); gyb[k] = T(0); }
                }
                face_gradient(qa, qb, gxa, gya, gxb, gyb, ldv4<T>(&m.ft[f]), fgx, fgy);
            }
            T F[4];
            face_flux<T, VISC>(m, bt, n.x, n.y, qf, qf, fgx, fgy, F);
            for (int k = 0; k < 4; ++k) {
                const T fl = F[k] * Lg.x;
                if (cc.x == i) {
                    accT[k] -= fl;
                    if (cc.y < 0 && two_sided(bt)) sq += (double)fl * (double)fl;
                } else {
                    accT[k] += fl;
                }
            }
        }
        double out[4];
        for (int k = 0; k < 4; ++k) {
            out[k] = (double)accT[k];
            sq += out[k] * out[k];
        }
        st4(&Rq[i], out);
    }
    const double t = block_sum(sq, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// Residual-norm finalisation and the run_solver control (multigrid.h:195-234)
// in one block: fixed-order sum of the partials -> ‖qW‖₂, err/err_0,
// convergence test, history every 10th iteration.
static __global__ void k_control(const double* __restrict__ partials, int n, Ctrl* ctrl, double* hist, double* norms,
                          int uniform) {
    __shared__ double sh[32];
    if (!uniform && ctrl->done) return;
    double v = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) v += partials[k];
    const double t = block_sum(v, sh);
    if (threadIdx.x != 0) return;
    const double norm = sqrt(t);
    if (uniform) {
        ctrl->err0 = norm;
        return;
    }
    const int i = ctrl->iter;
    ctrl->last_norm = norm;
    if (norms) norms[i] = norm;
    double err = norm;
    if (!(norm == norm) || norm > 1.7976931348623157e308) {
        ctrl->status = 4;
        ctrl->done = 1;
    }
    if (ctrl->run_mode) {
        if (i == 0 && err > 2 * ctrl->err0) ctrl->err0 = err;
        if (err > 0) err /= ctrl->err0;
        ctrl->err = err;
        if (i % 10 == 0 && ctrl->hist_n < HIST_CAP) hist[ctrl->hist_n++] = err;
        ctrl->iter = i + 1;
        if (!((err > ctrl->tol) && (i + 1 < ctrl->max_it))) ctrl->done = 1;
    } else {
        ctrl->iter = i + 1;
    }
}

}  // namespace dev
}  // namespace afx
