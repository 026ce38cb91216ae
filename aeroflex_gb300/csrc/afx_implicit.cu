// Implicit solver of the rans path on the GPU (implicitSolver, solver.h:852-1213,
// driven by multigrid<implicitSolver>::run_solver, multigrid.h:240-293).
//
// Each iteration assembles the reference's linear system
//     (A_i/dt_i I + sum_faces dF/dq L) dQ = -sum_faces F L
// over the real cells (ghost rows are identity with a zero right-hand side in
// the reference, so ghost unknowns stay zero and drop out), solves it with
// restarted GMRES(30) to a relative tolerance of 1e-2 (at most 500 Krylov
// iterations), and updates q += relaxation dQ, followed by up to
// rhs_iterations chord steps with the same matrix.
//
// GB300 form:
//   * face Jacobians J = dF/dq_c0 L, K = dF/dq_c1 L by the reference's
//     one-sided differences (physics.h:533-578: step max(1e-6, 1e-6 |q|)),
//     one thread per face;
//   * block rows, not a general sparse matrix: rows grouped by colour (no
//     two face neighbours share a colour), one 4x4 diagonal block per row and
//     four off-diagonal ELL blocks (K for the face's cell 0, -J for its cell
//     1), interleaved across rows so every warp load is contiguous;
//   * preconditioner: block ILU(0) in that colour ordering (the factor's
//     diagonal blocks formed colour by colour), applied as a forward then a
//     backward sweep over the colours -- a fixed linear operator, so right
//     preconditioned GMRES applies unchanged;
//   * Krylov vectors and matrix blocks in T = double (FP64 path) or float
//     (FP32-mixed path: the right-hand side, the update and the norms stay
//     FP64, so the iteration converges to the FP64 solution);
//   * CGS2 in three fused passes over the basis, 16-byte loads; every
//     reduction is a fixed-order two-level sum (deterministic);
//   * each solve is one CUDA graph whose restart and Arnoldi loops are
//     device-side WHILE nodes (or, with krylov_graph = 0, the same kernels
//     from a host loop);
//   * the adjoint transposes the filled system in place and reuses all of it.
#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "afx_host.hpp"
#include "afx_kernels_impl.cuh"

namespace afx {
namespace dev {

constexpr int GM_M = 30;       // GMRES restart length (Eigen's default)
constexpr int DOT_THREADS = 256;

struct GmresCtl {
    int stop;    // the current cycle has converged / ended
    int k;       // Arnoldi steps taken in the current cycle
    int iters;   // Krylov iterations of this solve
    int halt;    // no further restart cycle
    int max_iters;
    int graph;   // launched inside the solve graph: set the WHILE conditions
    cudaGraphConditionalHandle hin, hout;  // WHILE conditions: Arnoldi steps, restart cycles
    double tol;  // absolute residual target
    double res;  // current residual estimate
    double H[(GM_M + 1) * GM_M];  // column-major: H[i + (GM_M + 1) * j]
    double g[GM_M + 1], cs[GM_M], sn[GM_M], y[GM_M];
    double hnext;  // h_{j+1,j} of the last step (before rotation)
};

template <class T> struct B4;
template <> struct B4<double> { using type = d4; };
template <> struct B4<float> { using type = float4; };

// Krylov-side vectors in their own precision T: FP32 arithmetic stays in the
// FP32 pipes (a float-to-double conversion per operand would run on GB300's
// FP64 pipe, at ~1/64 of the FP32 rate)
__device__ __forceinline__ void ldt(const d4* p, double* v) { ld4(p, v); }
__device__ __forceinline__ void ldt(const float4* p, float* v) {
    const float4 a = *p;
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void stt(d4* p, const double* v) { st4(p, v); }
__device__ __forceinline__ void stt(float4* p, const float* v) { *p = make_float4(v[0], v[1], v[2], v[3]); }

// y += sgn * B x for a 4x4 block (row-major) in T.  Blocks start on a
// 16-byte boundary (16 T per block, buffers from cudaMalloc), so each row is
// read with 16-byte vector loads: a cell's block is then 4 (FP32) or 8 (FP64)
// load instructions, not 16 scattered scalar ones.
template <class T>
__device__ __forceinline__ void bmv_add(const T* __restrict__ B, const T* x, T* y, const T sgn);
template <>
__device__ __forceinline__ void bmv_add<float>(const float* __restrict__ B, const float* x, float* y,
                                               const float sgn) {
    const float4* b = reinterpret_cast<const float4*>(B);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float4 row = __ldg(&b[r]);
        float s = 0;
        s += row.x * x[0];
        s += row.y * x[1];
        s += row.z * x[2];
        s += row.w * x[3];
        y[r] += sgn * s;
    }
}
template <>
__device__ __forceinline__ void bmv_add<double>(const double* __restrict__ B, const double* x, double* y,
                                                const double sgn) {
    const double2* b = reinterpret_cast<const double2*>(B);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const double2 u = __ldg(&b[2 * r]), v = __ldg(&b[2 * r + 1]);
        double s = 0;
        s += u.x * x[0];
        s += u.y * x[1];
        s += v.x * x[2];
        s += v.y * x[3];
        y[r] += sgn * s;
    }
}

// Batch: a cell of a case that has stopped takes no part in the linear
// solve (its rows and unknowns are zero), so a case that went non-finite
// cannot spread into the others
__device__ __forceinline__ bool held(const int* case_of, const int* case_done, const int i) {
    return case_done && ((volatile const int*)case_done)[__ldg(&case_of[i])];
}

// A batch case whose diagonal block cannot be inverted stops (status 4)
// instead of failing the whole batch; the first cell to find it stops it.
__device__ __forceinline__ void stop_case(const int* case_of, int* case_done, CaseCtrl* cctrl, Ctrl* ctrl,
                                          const int i) {
    const int c = __ldg(&case_of[i]);
    if (atomicCAS(&case_done[c], 0, 1) == 0) {
        cctrl[c].status = 4;
        cctrl[c].done = 1;
        atomicAdd(&ctrl->ndone, 1);
    }
}

// ------------------------------------------------------------- assembly
// F of face f for the cell states (no reconstruction; the ghost side is the
// stored boundary state), as the reference's flux functor evaluates it.
// Spalart-Allmaras (VISC 2): the eddy viscosity is frozen at its current
// value (mut_f) and the no-slip wall shear of the cell state is included.
template <int VISC>
__device__ __forceinline__ void flux_cells(const KM<double>& m, const int bt, const double nx, const double ny,
                                           const double* qL, const double* qR, const double* fgx, const double* fgy,
                                           double* F, const double mut_f = 0.0, const double2 d0 = double2()) {
    face_flux<double, VISC>(m, bt, nx, ny, qL, qR, fgx, fgy, F, mut_f);
    if (VISC == 2 && bt == BT_WALL) sa_wall_shear(m, nx, ny, d0.x, d0.y, qL, F);
}

// calc_convective_jacobian (physics.h:533-578) times the face length:
// J = dF/dq_L, K = dF/dq_R by one-sided differences with the reference's
// step and its in-place perturb/restore of each component.
template <class T, int VISC>
__global__ void __launch_bounds__(128) k_imp_jac(const KM<double> m, const int n_faces, const d4* __restrict__ q,
                                                 const d4* __restrict__ gx, const d4* __restrict__ gy,
                                                 T* __restrict__ jf, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_faces) return;
    const int2 cc = __ldg(&m.fcell[f]);
    const double2 n = __ldg(&m.fn[f]);
    const double L = __ldg(&m.fLg[f]).x;
    double qL[4], qR[4];
    ld4(&q[cc.x], qL);
    int bt = BT_INTERNAL;
    if (cc.y >= 0) {
        ld4(&q[cc.y], qR);
    } else {
        bt = __ldg(&m.btype[-cc.y - 1]);
        ld4(&m.bq[-cc.y - 1], qR);
    }
    double fgx[4] = {0, 0, 0, 0}, fgy[4] = {0, 0, 0, 0};
    double mut_f = 0.0;
    double2 d0 = make_double2(0.0, 0.0);
    if (VISC == 2) {
        if (two_sided(bt)) mut_f = 0.5 * (__ldg(&m.mut[cc.x]) + __ldg(&m.mut[cc.y]));
        d0 = __ldg(&m.fd0[f]);
    }
    if (VISC >= 1 && two_sided(bt)) {
        double gx0[4], gy0[4], gx1[4] = {0, 0, 0, 0}, gy1[4] = {0, 0, 0, 0};
        ld4(&gx[cc.x], gx0);
        ld4(&gy[cc.x], gy0);
        if (cc.y >= 0) {
            ld4(&gx[cc.y], gx1);
            ld4(&gy[cc.y], gy1);
        }
        face_gradient(qL, qR, gx0, gy0, gx1, gy1, ldv4<double>(&m.ft[f]), fgx, fgy);
    }
    double f0[4];
    flux_cells<VISC>(m, bt, n.x, n.y, qL, qR, fgx, fgy, f0, mut_f, d0);
    T* out = jf + 32 * (size_t)f;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        const double upd = fmax(1e-6, fabs(qL[c]) * 1e-6);
        qL[c] += upd;
        double fp[4];
        flux_cells<VISC>(m, bt, n.x, n.y, qL, qR, fgx, fgy, fp, mut_f, d0);
        qL[c] -= upd;
#pragma unroll
        for (int r = 0; r < 4; ++r) out[4 * r + c] = (T)((fp[r] - f0[r]) / upd * L);
    }
    if (cc.y >= 0) {
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            const double upd = fmax(1e-6, fabs(qR[c]) * 1e-6);
            qR[c] += upd;
            double fp[4];
            flux_cells<VISC>(m, bt, n.x, n.y, qL, qR, fgx, fgy, fp, mut_f, d0);
            qR[c] -= upd;
#pragma unroll
            for (int r = 0; r < 4; ++r) out[16 + 4 * r + c] = (T)((fp[r] - f0[r]) / upd * L);
        }
    }
}

// Row layout of the linear system.  Rows are grouped by colour (the cells
// of a colour in device order), so a colour of the Gauss-Seidel sweep is a
// contiguous range of rows and every per-row access is coalesced.  A row's
// four off-diagonal blocks (ELL slots: the cell's face slots) carry the sign
// of the cell's side.
struct Ell {
    const int* perm;      // [N] device cell of row p
    const int4* col;      // [N] row of the neighbour in each slot, -1: none
    const int4* face;     // [N] signed face of each slot (cslot convention), 0: none
    const int4* tr;       // [N] ELL index 4 q + s' of the transposed block of each slot
    const int* case_row;  // [N] batch: case of row p, else null
};

// Off-diagonal blocks are interleaved across rows: 16-byte chunk c of slot
// s of row p (c = the block's row for FP32, half-row for FP64) is chunk
// (s * CPB + c) * N + p, so a warp's loads of one chunk are contiguous.
template <class T> struct Ell16 { static constexpr int W = 16 / sizeof(T), CPB = 16 / W; };
template <class T>
__device__ __forceinline__ size_t ell_at(const int N, const int p, const int s, const int k) {
    constexpr int W = Ell16<T>::W, CPB = Ell16<T>::CPB;
    return ((size_t)(s * CPB + k / W) * N + p) * W + (k % W);
}
// y += sgn * O x for the block of slot s of row p
template <class T>
__device__ __forceinline__ void ell_mv_add(const T* __restrict__ off, const int N, const int p, const int s,
                                           const T* x, T* y, const T sgn);
template <>
__device__ __forceinline__ void ell_mv_add<float>(const float* __restrict__ off, const int N, const int p,
                                                  const int s, const float* x, float* y, const float sgn) {
    const float4* b = reinterpret_cast<const float4*>(off);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float4 row = __ldg(&b[(size_t)(s * 4 + r) * N + p]);
        float t = 0;
        t += row.x * x[0];
        t += row.y * x[1];
        t += row.z * x[2];
        t += row.w * x[3];
        y[r] += sgn * t;
    }
}
template <>
__device__ __forceinline__ void ell_mv_add<double>(const double* __restrict__ off, const int N, const int p,
                                                   const int s, const double* x, double* y, const double sgn) {
    const double2* b = reinterpret_cast<const double2*>(off);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const double2 u = __ldg(&b[(size_t)(s * 8 + 2 * r) * N + p]);
        const double2 v = __ldg(&b[(size_t)(s * 8 + 2 * r + 1) * N + p]);
        double t = 0;
        t += u.x * x[0];
        t += u.y * x[1];
        t += v.x * x[2];
        t += v.y * x[3];
        y[r] += sgn * t;
    }
}

// Diagonal block A/dt I + sum (own: J, other: -K) of row p and its inverse
// (Gauss-Jordan with partial pivoting, in double), and the row's
// off-diagonal blocks (own: K, other: -J) from the face Jacobians.
template <class T>
__global__ void __launch_bounds__(128) k_imp_assemble(const KM<double> m, const Ell e, const double* __restrict__ dt,
                                                      const T* __restrict__ jf, T* __restrict__ dblk,
                                                      T* __restrict__ dinv, T* __restrict__ off,
                                                      int* __restrict__ singular, Ctrl* __restrict__ ctrl,
                                                      int* __restrict__ case_done, CaseCtrl* __restrict__ cctrl) {
    if (ctrl->done) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.n_cells) return;
    const int i = __ldg(&e.perm[p]);
    const int4 fsl = __ldg(&e.face[p]);
    const int4 col = __ldg(&e.col[p]);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(fsl, s);
        if (fs == 0 || pick(col, s) < 0) continue;
        const int f = (fs > 0 ? fs : -fs) - 1;
        const T* B = jf + 32 * (size_t)f + (fs > 0 ? 16 : 0);
#pragma unroll
        for (int k = 0; k < 16; ++k) off[ell_at<T>(m.n_cells, p, s, k)] = fs > 0 ? B[k] : -B[k];
    }
    if (held(e.case_row, case_done, p)) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            dblk[16 * (size_t)p + k] = T((k % 5 == 0) ? 1 : 0);
            dinv[16 * (size_t)p + k] = T((k % 5 == 0) ? 1 : 0);
        }
        return;
    }
    double D[16];
    const double ad = __ldg(&m.area[i]) / __ldg(&dt[i]);
#pragma unroll
    for (int k = 0; k < 16; ++k) D[k] = (k % 5 == 0) ? ad : 0.0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(fsl, s);
        if (fs == 0) continue;
        const int f = (fs > 0 ? fs : -fs) - 1;
        const T* B = jf + 32 * (size_t)f + (fs > 0 ? 0 : 16);
        const double sg = fs > 0 ? 1.0 : -1.0;
#pragma unroll
        for (int k = 0; k < 16; ++k) D[k] += sg * (double)B[k];
    }
    T* Do = dblk + 16 * (size_t)p;
#pragma unroll
    for (int k = 0; k < 16; ++k) Do[k] = (T)D[k];
    double I[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) I[k] = (k % 5 == 0) ? 1.0 : 0.0;
    for (int c = 0; c < 4; ++c) {
        int pv = c;
        double best = fabs(D[4 * c + c]);
        for (int r = c + 1; r < 4; ++r)
            if (fabs(D[4 * r + c]) > best) {
                best = fabs(D[4 * r + c]);
                pv = r;
            }
        if (!(best > 0)) {
            if (case_done) {
                stop_case(e.case_row, case_done, cctrl, ctrl, p);
#pragma unroll
                for (int k = 0; k < 16; ++k) dinv[16 * (size_t)p + k] = T((k % 5 == 0) ? 1 : 0);
            } else {
                *singular = 1;
            }
            return;
        }
        if (pv != c)
            for (int k = 0; k < 4; ++k) {
                double t = D[4 * c + k];
                D[4 * c + k] = D[4 * pv + k];
                D[4 * pv + k] = t;
                t = I[4 * c + k];
                I[4 * c + k] = I[4 * pv + k];
                I[4 * pv + k] = t;
            }
        const double inv = 1.0 / D[4 * c + c];
        for (int k = 0; k < 4; ++k) {
            D[4 * c + k] *= inv;
            I[4 * c + k] *= inv;
        }
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double fct = D[4 * r + c];
            for (int k = 0; k < 4; ++k) {
                D[4 * r + k] -= fct * D[4 * c + k];
                I[4 * r + k] -= fct * I[4 * c + k];
            }
        }
    }
    T* Io = dinv + 16 * (size_t)p;
#pragma unroll
    for (int k = 0; k < 16; ++k) Io[k] = (T)I[k];
}

// Block ILU(0) in the colour ordering: for the cells of colour c,
//     D~_i = D_i - sum_{neighbours o of a lower colour} O_io D~_o^-1 O_oi,
// inverted into dinv (colour 0 keeps D^-1).  With these inverses the
// symmetric multicolour Gauss-Seidel sweep below applies the ILU(0) factors
// (D~ + L) D~^-1 (D~ + U) exactly.
__device__ __forceinline__ void inv4(const double* A, double* I, int* singular) {
    double D[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        D[k] = A[k];
        I[k] = (k % 5 == 0) ? 1.0 : 0.0;
    }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        double best = fabs(D[4 * c + c]);
        for (int r = c + 1; r < 4; ++r)
            if (fabs(D[4 * r + c]) > best) {
                best = fabs(D[4 * r + c]);
                p = r;
            }
        if (!(best > 0)) {
            *singular = 1;
            return;
        }
        if (p != c)
            for (int k = 0; k < 4; ++k) {
                double t = D[4 * c + k];
                D[4 * c + k] = D[4 * p + k];
                D[4 * p + k] = t;
                t = I[4 * c + k];
                I[4 * c + k] = I[4 * p + k];
                I[4 * p + k] = t;
            }
        const double inv = 1.0 / D[4 * c + c];
        for (int k = 0; k < 4; ++k) {
            D[4 * c + k] *= inv;
            I[4 * c + k] *= inv;
        }
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double fct = D[4 * r + c];
            for (int k = 0; k < 4; ++k) {
                D[4 * r + k] -= fct * D[4 * c + k];
                I[4 * r + k] -= fct * I[4 * c + k];
            }
        }
    }
}

template <class T>
__global__ void __launch_bounds__(128) k_imp_ilu(const Ell e, const int N, const T* __restrict__ dblk,
                                                 const T* __restrict__ off, const int c0, const int n,
                                                 T* __restrict__ dinv,
                                                 int* __restrict__ singular, int* __restrict__ case_done,
                                                 CaseCtrl* __restrict__ cctrl, Ctrl* __restrict__ ctrl) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int p = c0 + t;
    if (held(e.case_row, case_done, p)) return;
    double D[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) D[k] = (double)dblk[16 * (size_t)p + k];
    const int4 col = __ldg(&e.col[p]);
    const int4 tr = __ldg(&e.tr[p]);
#pragma unroll 1
    for (int s = 0; s < 4; ++s) {
        const int q = pick(col, s);
        if (q < 0 || q >= c0) continue;  // rows of lower colours precede c0
        const int t2 = pick(tr, s);  // 4 q + s': the block of row q, column p
        double Oio[16], Ooi[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            Oio[k] = (double)off[ell_at<T>(N, p, s, k)];
            Ooi[k] = (double)off[ell_at<T>(N, t2 >> 2, t2 & 3, k)];
        }
        const T* Dinv_o = dinv + 16 * (size_t)q;
        double Y[16];  // D~_q^-1 O_qp
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                double acc = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) acc += (double)Dinv_o[4 * r + k] * Ooi[4 * k + c];
                Y[4 * r + c] = acc;
            }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                double acc = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) acc += Oio[4 * r + k] * Y[4 * k + c];
                D[4 * r + c] -= acc;
            }
    }
    double I[16];
    int sing = 0;
    inv4(D, I, &sing);
    if (sing) {
        if (case_done) {
            stop_case(e.case_row, case_done, cctrl, ctrl, p);
        } else {
            *singular = 1;
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) dinv[16 * (size_t)p + k] = (T)I[k];
}

// --------------------------------------------------------- linear algebra
// y = M x over the rows (diagonal block, then the slots in face order)
template <class T>
__global__ void __launch_bounds__(256) k_imp_spmv(const int n_rows, const Ell e, const T* __restrict__ dblk,
                                                  const T* __restrict__ off,
                                                  const typename B4<T>::type* __restrict__ x,
                                                  typename B4<T>::type* __restrict__ y, const int* __restrict__ stop,
                                                  const int* __restrict__ case_done) {
    if (stop && *stop) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_rows) return;
    if (held(e.case_row, case_done, p)) {
        const T z[4] = {0, 0, 0, 0};
        stt(&y[p], z);
        return;
    }
    T xi[4], yi[4] = {0, 0, 0, 0};
    ldt(&x[p], xi);
    bmv_add<T>(dblk + 16 * (size_t)p, xi, yi, T(1));
    const int4 col = __ldg(&e.col[p]);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int q = pick(col, s);
        if (q < 0) continue;
        T xo[4];
        ldt(&x[q], xo);
        ell_mv_add<T>(off, n_rows, p, s, xo, yi, T(1));
    }
    stt(&y[p], yi);
}

// One colour (rows c0 .. c0+n-1) of a block Gauss-Seidel sweep:
// x_p = D_p^-1 (r_p - sum O x_q).  r = rbase + (*rk) * stride when rk is
// given (the current Krylov vector).  In the forward sweep only rows of
// lower colours (q < c0) are read: the higher colours have no value yet
// (zero start).
template <class T>
__global__ void __launch_bounds__(256) k_imp_gs(const Ell e, const int N, const T* __restrict__ dinv,
                                                const T* __restrict__ off, const int c0, const int n, const T* __restrict__ rbase,
                                                const int* __restrict__ rk, const long long stride,
                                                typename B4<T>::type* __restrict__ x, const int* __restrict__ stop,
                                                const int* __restrict__ case_done, const bool fwd) {
    if (stop && *stop) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const typename B4<T>::type* r =
        reinterpret_cast<const typename B4<T>::type*>(rbase + (rk ? (long long)*rk * stride : 0));
    const int p = c0 + t;
    if (held(e.case_row, case_done, p)) {
        const T z[4] = {0, 0, 0, 0};
        stt(&x[p], z);
        return;
    }
    T s[4];
    ldt(&r[p], s);
    const int4 col = __ldg(&e.col[p]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = pick(col, k);
        if (q < 0 || (fwd && q >= c0)) continue;
        T xo[4];
        ldt(&x[q], xo);
        ell_mv_add<T>(off, N, p, k, xo, s, T(-1));
    }
    T xi[4] = {0, 0, 0, 0};
    bmv_add<T>(dinv + 16 * (size_t)p, s, xi, T(1));
    stt(&x[p], xi);
}

// Dot products against the Krylov basis v_0..v_{nv-1} (v_j = V + j*n) in
// one pass, with the Gram-Schmidt update fused in:
//   MODE 0: out_j = v_j . w
//   MODE 1: w -= sum_j hin_j v_j, then out_j = v_j . w   (CGS pass 1 + dots of pass 2)
//   MODE 2: w -= sum_j hin_j v_j, then out_0 = w . w     (CGS pass 2 + the norm)
// Each block writes its partial sums; the last block to finish adds them in
// a fixed pattern (DOT_G threads per output, each over a fixed stride of
// blocks, then a fixed shuffle tree), so the result is deterministic, and
// re-arms the counter.
// 16-byte chunks of a vector in T, their dot product and w -= h v
template <class T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int W = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int W = 2; };
__device__ __forceinline__ float vdot(const float4 a, const float4 b) {
    return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w;
}
__device__ __forceinline__ double vdot(const double2 a, const double2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ void vsub(float4& w, const float h, const float4 v) {
    w.x -= h * v.x; w.y -= h * v.y; w.z -= h * v.z; w.w -= h * v.w;
}
__device__ __forceinline__ void vsub(double2& w, const double h, const double2 v) {
    w.x -= h * v.x; w.y -= h * v.y;
}
__device__ __forceinline__ void vscale(float4& a, const float s) { a.x *= s; a.y *= s; a.z *= s; a.w *= s; }
__device__ __forceinline__ void vscale(double2& a, const double s) { a.x *= s; a.y *= s; }

constexpr int DOT_G = 8;  // threads of the last block per output
static_assert(DOT_THREADS / DOT_G >= GM_M + 1, "one group per output");

template <class T, int MODE>
__global__ void __launch_bounds__(DOT_THREADS, MODE == 1 ? 1 : 2) k_imp_dots(const int n, int nv, const int* __restrict__ nvk,
                                                          const T* __restrict__ V, T* __restrict__ w,
                                                          const double* __restrict__ hin, double* __restrict__ part,
                                                          unsigned* __restrict__ counter, double* __restrict__ out,
                                                          const int* __restrict__ stop) {
    __shared__ double sh[DOT_THREADS / 32][GM_M + 1];
    __shared__ T hs[GM_M + 1];
    __shared__ bool last;
    if (stop && *stop) return;
    if (nvk) nv = *nvk + 1;  // v_0 .. v_k of the current Arnoldi step
    const int nout = MODE == 2 ? 1 : nv;
    if (MODE > 0) {
        if ((int)threadIdx.x < nv) hs[threadIdx.x] = (T)hin[threadIdx.x];
        __syncthreads();
    }
    // per-thread partial sums in T over 16-byte chunks of the vectors (a few
    // chunks each; n is 4 * cells, so whole chunks), then double
    using VT = typename Vec16<T>::type;
    const int nc = n / Vec16<T>::W;
    const VT* __restrict__ Vv = reinterpret_cast<const VT*>(V);
    VT* __restrict__ wv = reinterpret_cast<VT*>(w);
    T acc[GM_M + 1];
#pragma unroll
    for (int j = 0; j <= GM_M; ++j) acc[j] = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
        VT wi = wv[i];
        if (MODE == 0) {
#pragma unroll
            for (int j = 0; j <= GM_M; ++j)
                if (j < nv) acc[j] += vdot(Vv[(size_t)j * nc + i], wi);
        } else {
            // MODE 1 keeps the basis chunks in registers for the second
            // product (one block per SM; the loads of a chunk are all in
            // flight at once)
            VT vv[GM_M + 1];
#pragma unroll
            for (int j = 0; j <= GM_M; ++j)
                if (j < nv) {
                    vv[j] = Vv[(size_t)j * nc + i];
                    vsub(wi, hs[j], vv[j]);
                }
            wv[i] = wi;
            if (MODE == 1) {
#pragma unroll
                for (int j = 0; j <= GM_M; ++j)
                    if (j < nv) acc[j] += vdot(vv[j], wi);
            } else {
                acc[0] += vdot(wi, wi);
            }
        }
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j <= GM_M; ++j) {
        if (j >= nout) break;
        double v = (double)acc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[wp][j] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < nout) {
        double t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k][threadIdx.x];
        part[(size_t)blockIdx.x * nout + threadIdx.x] = t;
        __threadfence();  // the partials are visible before the block is counted
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block: DOT_G threads per output, each over blocks g, g+DOT_G,
    // ... (L2 reads, several in flight), then a fixed shuffle tree
    const int j = threadIdx.x / DOT_G, g = threadIdx.x % DOT_G;
    double t = 0;
    if (j < nout) {
        const int nb = (int)gridDim.x;
        int b = g;
        double t1 = 0, t2 = 0, t3 = 0;
        for (; b + 3 * DOT_G < nb; b += 4 * DOT_G) {
            t += __ldcg(&part[(size_t)b * nout + j]);
            t1 += __ldcg(&part[(size_t)(b + DOT_G) * nout + j]);
            t2 += __ldcg(&part[(size_t)(b + 2 * DOT_G) * nout + j]);
            t3 += __ldcg(&part[(size_t)(b + 3 * DOT_G) * nout + j]);
        }
        for (; b < nb; b += DOT_G) t += __ldcg(&part[(size_t)b * nout + j]);
        t = (t + t1) + (t2 + t3);
    }
#pragma unroll
    for (int o = DOT_G / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o, DOT_G);
    if (j < nout && g == 0) out[j] = t;
    if (threadIdx.x == 0) *counter = 0;
}

// v = w * scale[0]; with vk given, v = vbase + (*vk) * n (the next Krylov vector)
// (16-byte chunks; w and v may be the same vector)
template <class T>
__global__ void __launch_bounds__(256) k_imp_scale(const int n, const T* w, const double* __restrict__ scale, T* v,
                                                   const int* __restrict__ vk, const int* __restrict__ stop) {
    if (stop && *stop) return;
    using VT = typename Vec16<T>::type;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (vk) v += (long long)*vk * n;
    const T sc = (T)scale[0];
    if (i < n / Vec16<T>::W) {
        VT a = reinterpret_cast<const VT*>(w)[i];
        vscale(a, sc);
        reinterpret_cast<VT*>(v)[i] = a;
    }
}

// Arnoldi step j = c->k, classical Gram-Schmidt twice: h1 (first pass) and
// h2 (second pass) are summed into column j; then the Givens rotations and
// the residual estimate.  One warp: the column and the rotations are staged
// in shared memory so the sequential part runs on shared memory, not on
// dependent global loads.
__global__ void __launch_bounds__(32) k_imp_arnoldi(GmresCtl* c, const double* __restrict__ h1,
                                                    const double* __restrict__ h2, const double* __restrict__ ww,
                                                    double* __restrict__ scale) {
    __shared__ double col[GM_M + 1], cs[GM_M], sn[GM_M], gj[1];
    const int lane = threadIdx.x;
    if (c->stop) {
        if (lane == 0 && c->graph) cudaGraphSetConditional(c->hin, 0);
        return;
    }
    const int j = c->k;
    for (int t = lane; t <= j; t += 32) col[t] = h1[t] + h2[t];
    for (int t = lane; t < j; t += 32) {
        cs[t] = c->cs[t];
        sn[t] = c->sn[t];
    }
    if (lane == 0) gj[0] = c->g[j];
    __syncwarp();
    if (lane == 0) {
        const double hn = sqrt(fmax(ww[0], 0.0));
        col[j + 1] = hn;
        c->hnext = hn;
        scale[0] = hn > 0 ? 1.0 / hn : 0.0;
        for (int i = 0; i < j; ++i) {
            const double a = col[i], b = col[i + 1];
            col[i] = cs[i] * a + sn[i] * b;
            col[i + 1] = -sn[i] * a + cs[i] * b;
        }
        const double a = col[j], b = col[j + 1];
        const double r = sqrt(a * a + b * b);
        const double cj = r > 0 ? a / r : 1.0, sj = r > 0 ? b / r : 0.0;
        c->cs[j] = cj;
        c->sn[j] = sj;
        col[j] = r;
        col[j + 1] = 0;
        const double g = gj[0];
        c->g[j + 1] = -sj * g;
        c->g[j] = cj * g;
        c->res = fabs(sj * g);
        c->k = j + 1;
        c->iters += 1;
        const int st = (c->res <= c->tol || j + 1 == GM_M || hn == 0 || c->iters >= c->max_iters) ? 1 : 0;
        c->stop = st;
        if (c->graph) cudaGraphSetConditional(c->hin, st ? 0 : 1);
    }
    __syncwarp();
    for (int t = lane; t <= j + 1; t += 32) c->H[t + (GM_M + 1) * j] = col[t];
}

// Back substitution R y = g over the k steps of the cycle (one warp; the
// triangle is staged in shared memory)
__global__ void __launch_bounds__(32) k_imp_solve_y(GmresCtl* c) {
    __shared__ double R[GM_M * GM_M], g[GM_M], y[GM_M];
    const int k = c->k;
    for (int t = threadIdx.x; t < k * k; t += 32) {
        const int i = t % k, l = t / k;
        R[i + GM_M * l] = c->H[i + (GM_M + 1) * l];
    }
    for (int t = threadIdx.x; t < k; t += 32) g[t] = c->g[t];
    __syncwarp();
    if (threadIdx.x == 0)
        for (int i = k - 1; i >= 0; --i) {
            double s = g[i];
            for (int l = i + 1; l < k; ++l) s -= R[i + GM_M * l] * y[l];
            const double d = R[i + GM_M * i];
            y[i] = d != 0 ? s / d : 0.0;
        }
    __syncwarp();
    for (int t = threadIdx.x; t < k; t += 32) c->y[t] = y[t];
}

// t = sum_j y_j v_j over the k steps
template <class T>
__global__ void __launch_bounds__(256) k_imp_lincomb(const int n, const T* __restrict__ V, const GmresCtl* __restrict__ c,
                                                     T* __restrict__ t) {
    __shared__ T ys[GM_M];
    const int k = c->k;
    if ((int)threadIdx.x < k) ys[threadIdx.x] = (T)c->y[threadIdx.x];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T s = 0;
    for (int j = 0; j < k; ++j) s += ys[j] * V[(size_t)j * n + i];
    t[i] = s;
}

// x (double) += z;  r = b - y  (b double), both 4N long
template <class T>
__global__ void __launch_bounds__(256) k_imp_addx(const int n, const T* __restrict__ z, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)z[i];
}
// r = b - y, b in device cell order, r and y in row order (4N long)
template <class T>
__global__ void __launch_bounds__(256) k_imp_resid(const int n, const double* __restrict__ b,
                                                   const int* __restrict__ perm, const T* __restrict__ y,
                                                   T* __restrict__ r, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = (T)(b[4 * (size_t)__ldg(&perm[i >> 2]) + (i & 3)] - (double)y[i]);
}
// t = b in row order (b in device cell order)
template <class T>
__global__ void __launch_bounds__(256) k_imp_gather_b(const int n, const double* __restrict__ b,
                                                      const int* __restrict__ perm, T* __restrict__ t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) t[i] = (T)b[4 * (size_t)__ldg(&perm[i >> 2]) + (i & 3)];
}
template <class T>
__global__ void __launch_bounds__(256) k_imp_cast(const int n, const double* __restrict__ x, T* __restrict__ t,
                                                  const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) t[i] = (T)x[i];
}

// q += relax * dq over the real cells; dq also becomes qW (the reference's
// qW holds the last linear solution, read by get_uniform_residual)
// (dq in row order, q and qW in device cell order)
__global__ void __launch_bounds__(256) k_imp_update(const int n, const double* __restrict__ dq,
                                                    const int* __restrict__ perm, const double relax,
                                                    double* __restrict__ q, double* __restrict__ qW) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t j = 4 * (size_t)__ldg(&perm[i >> 2]) + (i & 3);
    q[j] += dq[i] * relax;
    qW[j] = dq[i];
}

// case of each row (batch)
__global__ void k_imp_case_rows(const int n, const int* __restrict__ perm, const int* __restrict__ case_of,
                                int* __restrict__ case_row) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) case_row[p] = case_of[perm[p]];
}

// GMRES initialisation of a cycle: g = (beta, 0, ...), stop = beta <= tol
__global__ void k_imp_cycle_init(GmresCtl* c, const double* __restrict__ rr, double* __restrict__ scale, const int first,
                                 const double rel_tol, const int max_iters) {
    if (!first && c->halt) return;
    const double beta = sqrt(fmax(rr[0], 0.0));
    if (first) {
        c->tol = rel_tol * beta;
        c->iters = 0;
        c->max_iters = max_iters;
    }
    for (int i = 0; i <= GM_M; ++i) c->g[i] = 0;
    c->g[0] = beta;
    c->res = beta;
    c->k = 0;
    c->stop = (beta <= c->tol) ? 1 : 0;
    c->halt = c->stop;
    scale[0] = beta > 0 ? 1.0 / beta : 0.0;
    if (first && c->graph) cudaGraphSetConditional(c->hout, c->stop ? 0 : 1);
}

// Start of a restart cycle (inside the restart loop's body): enter the
// Arnoldi loop unless the cycle is already converged
__global__ void k_imp_enter(GmresCtl* c) {
    if (c->graph) cudaGraphSetConditional(c->hin, c->stop ? 0 : 1);
}

// End of a restart cycle: another one if not converged and under the limit
__global__ void k_imp_outer_check(GmresCtl* c) {
    const int cont = (c->res > c->tol) && (c->iters < c->max_iters) && (c->k > 0);
    c->halt = cont ? 0 : 1;
    if (c->graph) cudaGraphSetConditional(c->hout, cont ? 1 : 0);
}

// ------------------------------------------------------------ adjoint
// M -> M^T in place: row p, slot s takes (O_qp)^T from the copy `src` of the
// off-diagonal blocks; the diagonal block and its ILU(0) inverse are
// transposed in their row.  The transposed inverses are exactly the ILU(0)
// factors of M^T in the same colour order (D~' = D~^T by induction over
// the colours), so the Gauss-Seidel sweep then applies P^T.
template <class T>
__global__ void __launch_bounds__(128) k_imp_transpose(const int N, const Ell e, const T* __restrict__ src,
                                                       T* __restrict__ off, T* __restrict__ dblk,
                                                       T* __restrict__ dinv) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const int4 col = __ldg(&e.col[p]);
    const int4 tr = __ldg(&e.tr[p]);
#pragma unroll 1
    for (int s = 0; s < 4; ++s) {
        if (pick(col, s) < 0) continue;
        const int t2 = pick(tr, s);
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) off[ell_at<T>(N, p, s, 4 * r + c)] = src[ell_at<T>(N, t2 >> 2, t2 & 3, 4 * c + r)];
    }
    T* D = dblk + 16 * (size_t)p;
    T* I = dinv + 16 * (size_t)p;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = r + 1; c < 4; ++c) {
            T t = D[4 * r + c];
            D[4 * r + c] = D[4 * c + r];
            D[4 * c + r] = t;
            t = I[4 * r + c];
            I[4 * r + c] = I[4 * c + r];
            I[4 * c + r] = t;
        }
}

}  // namespace dev

// ----------------------------------------------------------------- host
namespace {

inline int nb_(long long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

struct ImplicitEngine {
    bool f32 = false;
    bool graph = true;  // GMRES as one graph with device-side loops, else a host loop
    int N = 0, F = 0, n4 = 0;
    int n_colors = 0;
    std::vector<int> color_ptr;
    void* jf = nullptr;    // face Jacobians J, K (16 T each)
    void* dblk = nullptr;  // diagonal block of each row
    void* dinv = nullptr;  // its ILU(0) inverse
    void* off = nullptr;   // off-diagonal blocks, 4 slots per row
    int* perm = nullptr;   // device cell of each row (rows grouped by colour)
    int4* ell_col = nullptr;
    int4* ell_face = nullptr;
    int4* ell_tr = nullptr;
    int* case_row = nullptr;          // batch: case of each row
    const int* case_row_src = nullptr;  // the case_of it was formed from
    int* singular = nullptr;
    void* V = nullptr;     // (GM_M+1) x 4N
    void* w = nullptr;     // 4N
    void* z = nullptr;     // 4N
    void* t = nullptr;     // 4N
    double* x = nullptr;   // 4N, the solution dQ
    double* part = nullptr;
    unsigned* counter = nullptr;  // last-block counter of the dot kernel
    double* small = nullptr;  // h1[GM_M+1], h2[GM_M+1], ww, scale
    cudaGraphExec_t cyc[2] = {nullptr, nullptr};  // cyc[0]: the GMRES solve graph
    cudaStream_t s2 = nullptr, s3 = nullptr;      // capture streams of the loop bodies
    const void* cyc_b = nullptr;                  // right-hand side the graphs were captured with
    int nbd = 0, nbd1 = 0;  // blocks of the dot passes (two / one per SM)
    dev::GmresCtl* ctl = nullptr;
    dev::GmresCtl* h_ctl = nullptr;
    int last_iters = 0;

    size_t ts() const { return f32 ? 4 : 8; }
    dev::Ell ell() const { return dev::Ell{perm, ell_col, ell_face, ell_tr, case_row}; }
};

void implicit_destroy(ImplicitEngine* e);

// cslot, cnbr: the host copies of the cell slots (4 per cell, device order)
ImplicitEngine* implicit_create(const StepArgs& a, bool f32, bool graph, const std::vector<int>& colors,
                                const int* cslot, const int* cnbr, cudaStream_t s) {
    // freed again if any step below throws
    std::unique_ptr<ImplicitEngine, void (*)(ImplicitEngine*)> guard(new ImplicitEngine(), implicit_destroy);
    ImplicitEngine* e = guard.get();
    e->f32 = f32;
    e->graph = graph;
    e->N = a.n_cells;
    e->F = a.n_faces;
    e->n4 = 4 * a.n_cells;
    const int N = e->N;
    int nc = 0;
    for (int c : colors) nc = std::max(nc, c + 1);
    e->n_colors = nc;
    e->color_ptr.assign(nc + 1, 0);
    for (int c : colors) e->color_ptr[c + 1]++;
    for (int c = 0; c < nc; ++c) e->color_ptr[c + 1] += e->color_ptr[c];
    // rows: the cells of colour 0, then colour 1, ..., each in device order
    std::vector<int> perm(N), rowof(N), fill(e->color_ptr.begin(), e->color_ptr.end() - 1);
    for (int i = 0; i < N; ++i) perm[fill[colors[i]]++] = i;
    for (int p = 0; p < N; ++p) rowof[perm[p]] = p;
    std::vector<int> ecol(4 * (size_t)N, -1), eface(4 * (size_t)N, 0), etr(4 * (size_t)N, -1);
    for (int p = 0; p < N; ++p) {
        const int i = perm[p];
        for (int k = 0; k < 4; ++k) {
            const int fs = cslot[4 * (size_t)i + k], o = cnbr[4 * (size_t)i + k];
            eface[4 * (size_t)p + k] = fs;
            if (fs != 0 && o >= 0) ecol[4 * (size_t)p + k] = rowof[o];
        }
    }
    for (int p = 0; p < N; ++p)
        for (int k = 0; k < 4; ++k) {
            const int q = ecol[4 * (size_t)p + k];
            if (q < 0) continue;
            const int f = std::abs(eface[4 * (size_t)p + k]);
            for (int k2 = 0; k2 < 4; ++k2)
                if (std::abs(eface[4 * (size_t)q + k2]) == f) etr[4 * (size_t)p + k] = 4 * q + k2;
            if (etr[4 * (size_t)p + k] < 0) throw Error(7, "implicit solver: face slots are not symmetric");
        }
    const size_t T = e->ts();
    auto chk = [](cudaError_t r) {
        if (r != cudaSuccess) throw Error(7, std::string("implicit solver: ") + cudaGetErrorString(r));
    };
    const size_t N1 = std::max(N, 1);
    chk(cudaMalloc(&e->jf, (size_t)e->F * 32 * T));
    chk(cudaMalloc(&e->dblk, N1 * 16 * T));
    chk(cudaMalloc(&e->dinv, N1 * 16 * T));
    chk(cudaMalloc(&e->off, N1 * 64 * T));
    chk(cudaMalloc((void**)&e->perm, N1 * sizeof(int)));
    chk(cudaMalloc((void**)&e->ell_col, N1 * sizeof(int4)));
    chk(cudaMalloc((void**)&e->ell_face, N1 * sizeof(int4)));
    chk(cudaMalloc((void**)&e->ell_tr, N1 * sizeof(int4)));
    chk(cudaMalloc((void**)&e->singular, sizeof(int)));
    chk(cudaMalloc(&e->V, (size_t)(dev::GM_M + 1) * e->n4 * T));
    chk(cudaMalloc(&e->w, (size_t)e->n4 * T));
    chk(cudaMalloc(&e->z, (size_t)e->n4 * T));
    chk(cudaMalloc(&e->t, (size_t)e->n4 * T));
    chk(cudaMalloc((void**)&e->x, (size_t)e->n4 * 8));
    int dev_id = 0, sms = 0;
    cudaGetDevice(&dev_id);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id);
    // two resident blocks per SM at most: the last block then sums few partials
    e->nbd = std::max(1, std::min(2 * std::max(sms, 1), nb_(e->n4, dev::DOT_THREADS * 4)));
    e->nbd1 = std::max(1, std::min(std::max(sms, 1), e->nbd));
    chk(cudaMalloc((void**)&e->part, (size_t)e->nbd * (dev::GM_M + 1) * 8));
    chk(cudaMalloc((void**)&e->small, (2 * (dev::GM_M + 1) + 2) * 8));
    chk(cudaMalloc((void**)&e->counter, sizeof(unsigned)));
    chk(cudaMemsetAsync(e->counter, 0, sizeof(unsigned), s));
    chk(cudaMalloc((void**)&e->ctl, sizeof(dev::GmresCtl)));
    chk(cudaHostAlloc((void**)&e->h_ctl, sizeof(dev::GmresCtl), cudaHostAllocDefault));
    chk(cudaMemcpyAsync(e->perm, perm.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice, s));
    chk(cudaMemcpyAsync(e->ell_col, ecol.data(), (size_t)N * sizeof(int4), cudaMemcpyHostToDevice, s));
    chk(cudaMemcpyAsync(e->ell_face, eface.data(), (size_t)N * sizeof(int4), cudaMemcpyHostToDevice, s));
    chk(cudaMemcpyAsync(e->ell_tr, etr.data(), (size_t)N * sizeof(int4), cudaMemcpyHostToDevice, s));
    chk(cudaMemsetAsync(e->jf, 0, (size_t)e->F * 32 * T, s));
    chk(cudaMemsetAsync(e->off, 0, N1 * 64 * T, s));
    e->h_ctl->graph = graph ? 1 : 0;
    chk(cudaMemcpyAsync(&e->ctl->graph, &e->h_ctl->graph, sizeof(int), cudaMemcpyHostToDevice, s));
    chk(cudaStreamSynchronize(s));
    return guard.release();
}

void implicit_destroy(ImplicitEngine* e) {
    if (!e) return;
    for (int k = 0; k < 2; ++k)
        if (e->cyc[k]) cudaGraphExecDestroy(e->cyc[k]);
    if (e->s2) cudaStreamDestroy(e->s2);
    if (e->s3) cudaStreamDestroy(e->s3);
    for (void* p : {e->jf, e->dblk, e->dinv, e->off, (void*)e->perm, (void*)e->ell_col, (void*)e->ell_face,
                    (void*)e->ell_tr, (void*)e->case_row, (void*)e->singular, e->V, e->w, e->z, e->t, (void*)e->x,
                    (void*)e->part, (void*)e->small, (void*)e->ctl, (void*)e->counter})
        if (p) cudaFree(p);
    if (e->h_ctl) cudaFreeHost(e->h_ctl);
    delete e;
}

// fillRhoLHS (solver.h:1016-1090): dt from the state of parity p at the CFL
// in a.cfl, face Jacobians, diagonal blocks and their inverses.
namespace {
template <class T>
void fill_t(ImplicitEngine* e, const StepArgs& a, const dev::KM<double>& m, const dev::d4* q, cudaStream_t s) {
    using namespace dev;
    const int nf = nb_(a.n_faces, 128), nc = nb_(a.n_cells, 128);
    if (a.visc == 1)
        k_imp_jac<T, 1><<<nf, 128, 0, s>>>(m, a.n_faces, q, (const d4*)a.gx, (const d4*)a.gy, (T*)e->jf, a.ctrl);
    else if (a.visc == 2)
        k_imp_jac<T, 2><<<nf, 128, 0, s>>>(m, a.n_faces, q, (const d4*)a.gx, (const d4*)a.gy, (T*)e->jf, a.ctrl);
    else
        k_imp_jac<T, 0><<<nf, 128, 0, s>>>(m, a.n_faces, q, (const d4*)a.gx, (const d4*)a.gy, (T*)e->jf, a.ctrl);
    const Ell el = e->ell();
    k_imp_assemble<T><<<nc, 128, 0, s>>>(m, el, (const double*)a.dt, (const T*)e->jf, (T*)e->dblk, (T*)e->dinv,
                                         (T*)e->off, e->singular, a.ctrl, a.case_done, a.cctrl);
    for (int c = 1; c < e->n_colors; ++c) {
        const int c0 = e->color_ptr[c], cn = e->color_ptr[c + 1] - c0;
        if (cn > 0)
            k_imp_ilu<T><<<nb_(cn, 128), 128, 0, s>>>(el, e->N, (const T*)e->dblk, (const T*)e->off, c0, cn,
                                                      (T*)e->dinv, e->singular, a.case_done, a.cctrl, a.ctrl);
    }
}
}  // namespace

void implicit_fill(ImplicitEngine* e, const StepArgs& a0, int p, cudaStream_t s) {
    using namespace dev;
    StepArgs a = a0;
    a.variant = 0;  // the prep that also forms dt
    a.second = 0;   // gradients only when viscous (solver.h:1023-1026)
    a.need_grad = a.visc >= 1 ? 1 : 0;
    if (a.case_of && e->case_row_src != a.case_of) {
        // a batch: the case of each row, formed once
        if (!e->case_row && cudaMalloc((void**)&e->case_row, (size_t)std::max(e->N, 1) * sizeof(int)) != cudaSuccess)
            throw Error(7, "implicit solver: out of device memory");
        k_imp_case_rows<<<nb_(e->N, 256), 256, 0, s>>>(e->N, e->perm, a.case_of, e->case_row);
        e->case_row_src = a.case_of;
    }
    const KM<double> m = make_km<double>(a);
    launch_prep<double, double>(a, m, (const d4*)a.qm[p], s);
    cudaMemsetAsync(e->singular, 0, sizeof(int), s);
    const d4* q = (const d4*)a.qm[p];
    if (e->f32) fill_t<float>(e, a, m, q, s);
    else fill_t<double>(e, a, m, q, s);
}

namespace {

template <class T>
struct Ops {
    ImplicitEngine* e;
    const StepArgs& a;
    cudaStream_t s;
    dev::KM<double> m;
    using V4 = typename dev::B4<T>::type;
    Ops(ImplicitEngine* e_, const StepArgs& a_, cudaStream_t s_) : e(e_), a(a_), s(s_), m(dev::make_km<double>(a_)) {}
    T* vec(int j) const { return (T*)e->V + (size_t)j * e->n4; }
    int* stop() const { return &e->ctl->stop; }
    void spmv(const T* x, T* y, const int* st) const {
        dev::k_imp_spmv<T><<<nb_(e->N, 256), 256, 0, s>>>(e->N, e->ell(), (const T*)e->dblk, (const T*)e->off,
                                                          (const V4*)x, (V4*)y, st, a.case_done);
    }
    // t = b in row order
    void gather_b(const double* b, T* t) const {
        dev::k_imp_gather_b<T><<<nb_(e->n4, 256), 256, 0, s>>>(e->n4, b, e->perm, t);
    }
    // one symmetric multicolour block Gauss-Seidel sweep from x = 0 (the
    // ILU(0) factors in the colour ordering); the input is r, or the current
    // Krylov vector V + k*n when rk is given.  The forward sweep forms every
    // cell (reading lower colours only); the backward sweep skips the top
    // colour, whose value it would form again unchanged.
    void precond(const T* r, const int* rk, T* x, const int* st) const {
        const int C = e->n_colors;
        for (int k = 0; k < 2 * C - 1; ++k) {
            const int c = k < C ? k : 2 * C - 2 - k;
            const int c0 = e->color_ptr[c], cn = e->color_ptr[c + 1] - c0;
            if (cn == 0) continue;
            dev::k_imp_gs<T><<<nb_(cn, 256), 256, 0, s>>>(e->ell(), e->N, (const T*)e->dinv, (const T*)e->off, c0,
                                                          cn, r, rk, (long long)e->n4, (V4*)x, st, a.case_done,
                                                          k < C);
        }
    }
    // MODE 0: out = V^T w; 1: w -= V hin, out = V^T w; 2: w -= V hin, out = w.w
    template <int MODE>
    void dots(int nv, const int* nvk, const T* V, T* w, const double* hin, double* out, const int* st) const {
        // MODE 1 holds one block per SM
        const int g = MODE == 1 ? e->nbd1 : e->nbd;
        dev::k_imp_dots<T, MODE><<<g, dev::DOT_THREADS, 0, s>>>(e->n4, nv, nvk, V, w, hin, e->part, e->counter, out,
                                                              st);
    }
    // v = w * scale (k given: v = V_{*k})
    void scale(const T* w, const double* sc, T* v, const int* k, const int* st) const {
        dev::k_imp_scale<T><<<nb_(e->n4 / (16 / (int)sizeof(T)), 256), 256, 0, s>>>(e->n4, w, sc, v, k, st);
    }
};

// Adds a WHILE node at the capture position of stream st (the work captured
// next on st follows the loop) and returns its body graph.
cudaGraph_t add_while(cudaStream_t st, cudaGraphConditionalHandle* h) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* ed = nullptr;
    size_t nd = 0;
    auto chk = [](cudaError_t r) {
        if (r != cudaSuccess) throw Error(7, std::string("implicit solver graph: ") + cudaGetErrorString(r));
    };
    chk(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
    chk(cudaGraphConditionalHandleCreate(h, g, 0, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = *h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    chk(cudaGraphAddNode(&node, g, deps, ed, nd, &p));
    chk(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return p.conditional.phGraph_out[0];
}

// The whole GMRES solve of M dQ = b as one graph: restart cycles and Arnoldi
// steps are WHILE loops whose conditions the kernels set on the device, so
// a solve runs without host round trips and without idle launches.
template <class T>
cudaGraphExec_t build_gmres_graph(ImplicitEngine* e, const Ops<T>& o0, const double* b, cudaStream_t s,
                                  cudaStream_t s2, cudaStream_t s3, int max_iters) {
    using namespace dev;
    const int n = e->n4;
    double* h1 = e->small;
    double* h2 = e->small + (GM_M + 1);
    double* ww = e->small + 2 * (GM_M + 1);
    double* scale = ww + 1;
    int* kptr = &e->ctl->k;
    int* stop = &e->ctl->stop;
    int* halt = &e->ctl->halt;
    auto chk = [](cudaError_t r) {
        if (r != cudaSuccess) throw Error(7, std::string("implicit solver graph: ") + cudaGetErrorString(r));
    };
    cudaGraphConditionalHandle hout, hin;
    // main graph: first cycle set-up, the restart loop, the control block back to the host
    chk(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    Ops<T> o(e, o0.a, s);
    T* v0 = o.vec(0);
    cudaMemsetAsync(e->x, 0, (size_t)n * 8, s);
    o.gather_b(b, v0);
    o.template dots<0>(1, nullptr, v0, v0, nullptr, ww, nullptr);
    k_imp_cycle_init<<<1, 1, 0, s>>>(e->ctl, ww, scale, 1, 1e-2, max_iters);
    o.scale(v0, scale, v0, nullptr, stop);
    cudaGraph_t body_out = add_while(s, &hout);
    cudaMemcpyAsync(e->h_ctl, e->ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, s);
    cudaGraph_t G;
    chk(cudaStreamEndCapture(s, &G));
    // restart-cycle body: the Arnoldi loop, the update of x, the next residual
    chk(cudaStreamBeginCaptureToGraph(s2, body_out, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    {
        Ops<T> q(e, o0.a, s2);
        k_imp_enter<<<1, 1, 0, s2>>>(e->ctl);
        cudaGraph_t body_in = add_while(s2, &hin);
        k_imp_solve_y<<<1, 32, 0, s2>>>(e->ctl);
        k_imp_lincomb<T><<<nb_(n, 256), 256, 0, s2>>>(n, q.vec(0), e->ctl, (T*)e->t);
        q.precond((const T*)e->t, nullptr, (T*)e->z, nullptr);
        k_imp_addx<T><<<nb_(n, 256), 256, 0, s2>>>(n, (const T*)e->z, e->x);
        k_imp_outer_check<<<1, 1, 0, s2>>>(e->ctl);
        k_imp_cast<T><<<nb_(n, 256), 256, 0, s2>>>(n, e->x, (T*)e->t, halt);
        q.spmv((const T*)e->t, (T*)e->w, halt);
        k_imp_resid<T><<<nb_(n, 256), 256, 0, s2>>>(n, b, e->perm, (const T*)e->w, q.vec(0), halt);
        q.template dots<0>(1, nullptr, q.vec(0), q.vec(0), nullptr, ww, halt);
        k_imp_cycle_init<<<1, 1, 0, s2>>>(e->ctl, ww, scale, 0, 1e-2, max_iters);
        q.scale(q.vec(0), scale, q.vec(0), nullptr, halt);
        chk(cudaStreamEndCapture(s2, &body_out));
        // Arnoldi step k: z = P^-1 v_k, w = M z, CGS2 against v_0..v_k, rotations, v_{k+1}
        chk(cudaStreamBeginCaptureToGraph(s3, body_in, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        Ops<T> r(e, o0.a, s3);
        r.precond(r.vec(0), kptr, (T*)e->z, stop);
        r.spmv((const T*)e->z, (T*)e->w, stop);
        // CGS2 in three passes over the basis: h1 = V^T w; w -= V h1 and
        // h2 = V^T w; w -= V h2 and ||w||^2
        r.template dots<0>(0, kptr, r.vec(0), (T*)e->w, nullptr, h1, stop);
        r.template dots<1>(0, kptr, r.vec(0), (T*)e->w, h1, h2, stop);
        r.template dots<2>(0, kptr, r.vec(0), (T*)e->w, h2, ww, stop);
        k_imp_arnoldi<<<1, 32, 0, s3>>>(e->ctl, h1, h2, ww, scale);
        r.scale((const T*)e->w, scale, r.vec(0), kptr, stop);
        chk(cudaStreamEndCapture(s3, &body_in));
    }
    cudaGraphExec_t ex;
    const cudaError_t ri = cudaGraphInstantiate(&ex, G, 0);
    cudaGraphDestroy(G);
    chk(ri);
    e->h_ctl->hin = hin;
    e->h_ctl->hout = hout;
    chk(cudaMemcpyAsync(&e->ctl->hin, &e->h_ctl->hin, 2 * sizeof(cudaGraphConditionalHandle), cudaMemcpyHostToDevice,
                        s));
    chk(cudaStreamSynchronize(s));
    return ex;
}

// The same solve as build_gmres_graph with the two loops on the host: the
// control block is read back after every Arnoldi step, so each kernel is a
// plain launch (for profilers; slower by one host round trip per step).
template <class T>
int gmres_host_loop(ImplicitEngine* e, const StepArgs& a, const double* b, cudaStream_t s, int max_iters) {
    using namespace dev;
    const int n = e->n4;
    double* h1 = e->small;
    double* h2 = e->small + (GM_M + 1);
    double* ww = e->small + 2 * (GM_M + 1);
    double* scale = ww + 1;
    int* kptr = &e->ctl->k;
    int* stop = &e->ctl->stop;
    int* halt = &e->ctl->halt;
    Ops<T> o(e, a, s);
    auto read_ctl = [&]() {
        // stop, k, iters, halt: the loop conditions
        if (cudaMemcpyAsync(e->h_ctl, e->ctl, 4 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            throw Error(7, "implicit solver: GMRES failed");
    };
    T* v0 = o.vec(0);
    cudaMemsetAsync(e->x, 0, (size_t)n * 8, s);
    o.gather_b(b, v0);
    o.template dots<0>(1, nullptr, v0, v0, nullptr, ww, nullptr);
    k_imp_cycle_init<<<1, 1, 0, s>>>(e->ctl, ww, scale, 1, 1e-2, max_iters);
    o.scale(v0, scale, v0, nullptr, stop);
    read_ctl();
    if (!e->h_ctl->stop) {
        for (;;) {
            for (;;) {  // Arnoldi steps of the cycle
                read_ctl();
                if (e->h_ctl->stop) break;
                o.precond(o.vec(0), kptr, (T*)e->z, stop);
                o.spmv((const T*)e->z, (T*)e->w, stop);
                o.template dots<0>(0, kptr, o.vec(0), (T*)e->w, nullptr, h1, stop);
                o.template dots<1>(0, kptr, o.vec(0), (T*)e->w, h1, h2, stop);
                o.template dots<2>(0, kptr, o.vec(0), (T*)e->w, h2, ww, stop);
                k_imp_arnoldi<<<1, 32, 0, s>>>(e->ctl, h1, h2, ww, scale);
                o.scale((const T*)e->w, scale, o.vec(0), kptr, stop);
            }
            k_imp_solve_y<<<1, 32, 0, s>>>(e->ctl);
            k_imp_lincomb<T><<<nb_(n, 256), 256, 0, s>>>(n, o.vec(0), e->ctl, (T*)e->t);
            o.precond((const T*)e->t, nullptr, (T*)e->z, nullptr);
            k_imp_addx<T><<<nb_(n, 256), 256, 0, s>>>(n, (const T*)e->z, e->x);
            k_imp_outer_check<<<1, 1, 0, s>>>(e->ctl);
            k_imp_cast<T><<<nb_(n, 256), 256, 0, s>>>(n, e->x, (T*)e->t, halt);
            o.spmv((const T*)e->t, (T*)e->w, halt);
            k_imp_resid<T><<<nb_(n, 256), 256, 0, s>>>(n, b, e->perm, (const T*)e->w, o.vec(0), halt);
            o.template dots<0>(1, nullptr, o.vec(0), o.vec(0), nullptr, ww, halt);
            k_imp_cycle_init<<<1, 1, 0, s>>>(e->ctl, ww, scale, 0, 1e-2, max_iters);
            o.scale(o.vec(0), scale, o.vec(0), nullptr, halt);
            read_ctl();
            if (e->h_ctl->halt) break;
        }
    }
    read_ctl();
    return e->h_ctl->iters;
}

template <class T>
int gmres(ImplicitEngine* e, const StepArgs& a, const double* b, cudaStream_t s, int max_iters) {
    if (!e->graph) return gmres_host_loop<T>(e, a, b, s, max_iters);
    Ops<T> o(e, a, s);
    if (e->cyc_b != b || !e->cyc[0]) {
        if (e->cyc[0]) cudaGraphExecDestroy(e->cyc[0]);
        e->cyc[0] = nullptr;
        if (!e->s2) {
            cudaStreamCreateWithFlags(&e->s2, cudaStreamNonBlocking);
            cudaStreamCreateWithFlags(&e->s3, cudaStreamNonBlocking);
        }
        e->cyc[0] = build_gmres_graph<T>(e, o, b, s, e->s2, e->s3, max_iters);
        e->cyc_b = b;
    }
    if (cudaGraphLaunch(e->cyc[0], s) != cudaSuccess) throw Error(7, "implicit solver: graph launch failed");
    if (cudaStreamSynchronize(s) != cudaSuccess) throw Error(7, "implicit solver: GMRES failed");
    return e->h_ctl->iters;
}

}  // namespace

// Solves M dQ = b (b: FP64 right-hand side over the real cells, AoS) and
// applies q += relax dQ to the FP64 state; dQ is also copied to qW.
// Returns the Krylov iterations, or -1 if a diagonal block was singular.
int implicit_solve_update(ImplicitEngine* e, const StepArgs& a, int p, const double* b, double relax,
                          cudaStream_t s) {
    int sing = 0;
    cudaMemcpyAsync(&sing, e->singular, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (sing) return -1;
    const int it = e->f32 ? gmres<float>(e, a, b, s, 500) : gmres<double>(e, a, b, s, 500);
    dev::k_imp_update<<<nb_(e->n4, 256), 256, 0, s>>>(e->n4, e->x, e->perm, relax, (double*)a.qm[p],
                                                      (double*)a.Rq);
    e->last_iters = it;
    return it;
}

// out = scale * (area .* x) (area null: 1) in device order, x the engine's
// last GMRES solution (row order)
namespace dev {
template <class T>
__global__ void __launch_bounds__(256) k_imp_scatter(const int n, const T* __restrict__ x,
                                                     const int* __restrict__ perm, const double* __restrict__ area,
                                                     const double scale, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = __ldg(&perm[i >> 2]);
    out[4 * (size_t)c + (i & 3)] = scale * (area ? area[c] : 1.0) * (double)x[i];
}
}  // namespace dev

// The engine's linear solve as an operator: M x = b (M^T after
// implicit_transpose) by the same GMRES the implicit iteration uses, then
// out = scale * (area .* x) in device order.  b must stay at one address
// between calls (the solve graph is captured for it).  Returns the Krylov
// iterations, -1 if a diagonal block was singular.
int implicit_apply_inverse(ImplicitEngine* e, const StepArgs& a, const double* b, const double* area, double scale,
                           double* out, cudaStream_t s) {
    int sing = 0;
    cudaMemcpyAsync(&sing, e->singular, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (sing) return -1;
    const int it = e->f32 ? gmres<float>(e, a, b, s, 500) : gmres<double>(e, a, b, s, 500);
    dev::k_imp_scatter<double><<<nb_(e->n4, 256), 256, 0, s>>>(e->n4, e->x, e->perm, area, scale, out);
    e->last_iters = it;
    return it;
}

namespace {
template <class T>
void sweep_t(ImplicitEngine* e, const StepArgs& a, const double* b, const double* area, double scale, double* out,
             cudaStream_t s) {
    Ops<T> o(e, a, s);
    o.gather_b(b, (T*)e->t);
    o.precond((const T*)e->t, nullptr, (T*)e->z, nullptr);
    dev::k_imp_scatter<T><<<nb_(e->n4, 256), 256, 0, s>>>(e->n4, (const T*)e->z, e->perm, area, scale, out);
}
}  // namespace

// The engine's preconditioner alone as an operator: one symmetric
// multicolour block Gauss-Seidel sweep with the ILU(0) factors (of M, or of
// M^T after implicit_transpose), out = scale * (area .* x) in device order.
// Returns -1 if a diagonal block was singular, else 0.
int implicit_apply_sweep(ImplicitEngine* e, const StepArgs& a, const double* b, const double* area, double scale,
                         double* out, cudaStream_t s) {
    int sing = 0;
    cudaMemcpyAsync(&sing, e->singular, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (sing) return -1;
    if (e->f32) sweep_t<float>(e, a, b, area, scale, out, s);
    else sweep_t<double>(e, a, b, area, scale, out, s);
    return 0;
}

// The filled system transposed in place (M -> M^T, the ILU(0) factors ->
// those of M^T) for the adjoint's linear solves.  The next implicit_fill
// forms M again.  FP64 engines.
void implicit_transpose(ImplicitEngine* e, cudaStream_t s) {
    using namespace dev;
    if (e->f32) throw Error(7, "implicit solver: the adjoint needs an FP64 engine");
    // the Krylov basis (124 T per row) holds the copy of the blocks (64 T per row)
    cudaMemcpyAsync(e->V, e->off, (size_t)e->N * 64 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    k_imp_transpose<double><<<nb_(e->N, 128), 128, 0, s>>>(e->N, e->ell(), (const double*)e->V, (double*)e->off,
                                                           (double*)e->dblk, (double*)e->dinv);
}

}  // namespace afx
