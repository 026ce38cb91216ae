// Kernels of one explicit iteration of the rans residual path.
//
// Cell-centric gathers, one thread per cell.  A cell's faces are read from
// two int4 records (cslot: +/-(face+1), the sign saying whether the cell is
// the face's cell 0 or cell 1; cnbr: the other cell, or -(b+1) for boundary
// face b) in the reference's edge order, so every per-cell sum accumulates
// in the order of the reference's serial edge loop and the result is
// deterministic without atomics.  The slot loops are fully unrolled so the
// loads of all faces of a cell are in flight together.
#pragma once

#include "afx_device.cuh"

namespace afx {
namespace dev {

__device__ __forceinline__ int pick(const int4 v, const int s) {
    return s == 0 ? v.x : (s == 1 ? v.y : (s == 2 ? v.z : v.w));
}

// Plain (non-__ldg) vector loads, for shared memory.
__device__ __forceinline__ void ld4p(const d4* p, double* v) {
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = q[0], b = q[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void ld4p(const float4* p, float* v) {
    const float4 a = *p;
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}

// Per cell, from the iteration's starting state q (the solver's member q):
// local time step (solver.h:308-356; skipped when the face kernel forms it),
// Green-Gauss gradient (solver.h:428-469) and, when second order, the first
// stage's neighbour min/max and limiter (solver.h:517-593).
template <class T, class S, bool GRAD, bool SECOND, bool DTP>
__global__ void __launch_bounds__(256) k_prep(const KM<T> m, const V4<S>* __restrict__ q, V4<T>* __restrict__ gx,
                                              V4<T>* __restrict__ gy, V4<T>* __restrict__ phi,
                                              T* __restrict__ dt, const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_cells) return;
    const int4 sl = __ldg(&m.cslot[i]);
    const int4 nb = __ldg(&m.cnbr[i]);
    T qi[4];
    ld4s(&q[i], qi);
    T sgx[4] = {T(0), T(0), T(0), T(0)}, sgy[4] = {T(0), T(0), T(0), T(0)};
    T qmn[4], qmx[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { qmn[k] = qi[k]; qmx[k] = qi[k]; }
    T eigsum = T(0);
    T dxs[4], dys[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(sl, s);
        dxs[s] = T(0);
        dys[s] = T(0);
        if (fs != 0) {
            const bool own0 = fs > 0;
            const int f = (own0 ? fs : -fs) - 1;
            const int o = pick(nb, s);
            const V2<T> n = __ldg(&m.fn[f]);
            const V2<T> Lg = __ldg(&m.fLg[f]);
            T qo[4];
            int bt = BT_INTERNAL;
            if (o >= 0) {
                ld4s(&q[o], qo);
            } else {
                bt = __ldg(&m.btype[-o - 1]);
                ld4c<T>(&m.bq[-o - 1], qo);
            }
            T q0c[4], q1c[4];  // states of the face's cell 0 and cell 1 (ghost: boundary state)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                q0c[k] = own0 ? qi[k] : qo[k];
                q1c[k] = own0 ? qo[k] : qi[k];
            }
            if (DTP) {
                T eig;
                if (two_sided(bt)) {
                    const T eL = face_eig(m.gamma, n.x, n.y, q0c);
                    const T eR = face_eig(m.gamma, n.x, n.y, q1c);
                    eig = smax(eL, eR);
                } else {
                    eig = face_eig(m.gamma, n.x, n.y, q0c);
                }
                eigsum += eig * Lg.x;
            }
            if (GRAD && !m.lsq) {
                T qRv[4];
                ghost_state(bt, m.gamma, n.x, n.y, q0c, q1c, qRv);
                const T g = Lg.y;
#pragma unroll
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
            if (SECOND) {
                if (bt != BT_SLIP && bt != BT_WALL) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        qmn[k] = smin(qmn[k], qo[k]);
                        qmx[k] = smax(qmx[k], qo[k]);
                    }
                }
                const V2<T> d = own0 ? __ldg(&m.fd0[f]) : __ldg(&m.fd1[f]);
                dxs[s] = d.x;
                dys[s] = d.y;
            }
        }
    }
    const T A = __ldg(&m.area[i]);
    if (DTP) dt[i] = m.cfl * A / eigsum;
    if (!GRAD) return;
    T gxi[4], gyi[4];
    if (m.lsq) {
        // least squares (solver.h:470-513): g = sum_j (M d_j) (q_i - vars(q_i, q_n))
        // over the cell's local edges j in their own order
        const int code = __ldg(&m.lsqs[i]);
        const int nj = code >> 8;
#pragma unroll
        for (int k = 0; k < 4; ++k) gxi[k] = gyi[k] = T(0);
#pragma unroll 1
        for (int j = 0; j < nj; ++j) {
            const int s = (code >> (2 * j)) & 3;
            const int fs = pick(sl, s);
            const int f = (fs > 0 ? fs : -fs) - 1;
            const int o = pick(nb, s);
            const V2<T> n = __ldg(&m.fn[f]);
            T qo[4], qR[4];
            int bt = BT_INTERNAL;
            if (o >= 0) {
                ld4s(&q[o], qo);
            } else {
                bt = __ldg(&m.btype[-o - 1]);
                ld4c<T>(&m.bq[-o - 1], qo);
            }
            ghost_state(bt, m.gamma, n.x, n.y, qi, qo, qR);
            const V2<T> w = __ldg(&m.lsqw[4 * i + j]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const T d = qi[k] - qR[k];
                gxi[k] += w.x * d;
                gyi[k] += w.y * d;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            gxi[k] = sgx[k] / A;
            gyi[k] = sgy[k] / A;
        }
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
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        if (pick(sl, s) != 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const T dqg = gxi[k] * dxs[s] + gyi[k] * dys[s];
                lim[k] = smin(lim[k], limiter_value(m.limiter, dqg, qmx[k] - qi[k], qmn[k] - qi[k], K3a));
            }
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
    const int4 nb = __ldg(&m.cnbr[i]);
    T qi[4], gxi[4], gyi[4];
    ld4s(&qk[i], qi);
    ld4c<T>(&gx[i], gxi);
    ld4c<T>(&gy[i], gyi);
    T qmn[4], qmx[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { qmn[k] = qi[k]; qmx[k] = qi[k]; }
    T dxs[4], dys[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(sl, s);
        dxs[s] = T(0);
        dys[s] = T(0);
        if (fs != 0) {
            const bool own0 = fs > 0;
            const int f = (own0 ? fs : -fs) - 1;
            const int o = pick(nb, s);
            const V2<T> d = own0 ? __ldg(&m.fd0[f]) : __ldg(&m.fd1[f]);
            dxs[s] = d.x;
            dys[s] = d.y;
            bool use = true;
            T qo[4];
            if (o >= 0) {
                ld4s(&qk[o], qo);
            } else {
                const int bt = __ldg(&m.btype[-o - 1]);
                use = bt != BT_SLIP && bt != BT_WALL;
                ld4c<T>(&m.bq[-o - 1], qo);
            }
            if (use) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    qmn[k] = smin(qmn[k], qo[k]);
                    qmx[k] = smax(qmx[k], qo[k]);
                }
            }
        }
    }
    const T A = __ldg(&m.area[i]);
    T lim[4] = {T(1), T(1), T(1), T(1)};
    const T sqrt_area = dsqrt(A);
    const T Ka = m.limk * sqrt_area;
    const T K3a = Ka * Ka * Ka;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        if (pick(sl, s) != 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const T dqg = gxi[k] * dxs[s] + gyi[k] * dys[s];
                lim[k] = smin(lim[k], limiter_value(m.limiter, dqg, qmx[k] - qi[k], qmn[k] - qi[k], K3a));
            }
        }
    }
    V4<T> vp;
    st4(&vp, lim);
    phi[i] = vp;
}

// Second-order reconstruction of one side, solver.h:780-781:
// q + (gx*dx + gy*dy) .* phi
template <class T>
__device__ __forceinline__ void reconstruct(const T* q, const T* gxc, const T* gyc, const T* ph, const T dx,
                                            const T dy, T* out) {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = q[k] + (gxc[k] * dx + gyc[k] * dy) * ph[k];
}

// average_gradients (solver.h:359-398) for the laminar face flux: member
// states qa/qb and gradients of the face's two cells, direction from the
// precomputed sum-of-centroids vector t = (t0, t1, lij).
template <class T>
__device__ __forceinline__ void face_gradient(const T* qa, const T* qb, const T* gxa, const T* gya, const T* gxb,
                                              const T* gyb, const V4<T> t, T* fgx, T* fgy) {
    const T t0 = t.x, t1 = t.y, lij = t.z;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const T grad_dir = (qa[k] - qb[k]) / lij;
        const T gxb_ = (gxa[k] + gxb[k]) * T(0.5);
        const T gyb_ = (gya[k] + gyb[k]) * T(0.5);
        const T grad_dot = gxb_ * t0 + gyb_ * t1;
        fgx[k] = gxb_ - (grad_dot - grad_dir) * t0;
        fgy[k] = gyb_ - (grad_dot - grad_dir) * t1;
    }
}

// Per-stage epilogue of one cell: R = sum/area (solver.h:794-798), the RK
// update qk = q + R*dt*alpha*relaxation (solver.h:818-821) in FP64, and the
// squared norm of qW (solver.h:827) for the last stage.
template <class T, class S>
struct StageOut {
    const d4* __restrict__ q0;     // FP64 iteration start state (member q)
    const V4<S>* __restrict__ q0s; // the same state in S (FP32-mixed: its FP32 shadow)
    V4<S>* __restrict__ qnext;     // next stage state in S (stages 0, 1)
    d4* __restrict__ qm_next;      // FP64 new state (stage 2)
    V4<S>* __restrict__ qsh_next;  // new state in S (stage 2, FP32-mixed shadow), may be null
    d4* __restrict__ Rq;           // qW mirror (residual-only launches)
    T* __restrict__ dt;
    double alpha, relax;
    double* __restrict__ partials;
    const float4* __restrict__ corr;  // FP32-mixed defect correction per cell, or null
    // batch of independent cases (null for a single case): the case of each
    // cell, the cases that have stopped (their state is held), and the
    // per-cell squared residual of the last stage for the per-case norms
    const int* __restrict__ case_of;
    const int* __restrict__ case_done;
    double* __restrict__ cell_sq;
    int mode;                      // 0 stage 0/1, 1 stage 2 (+norm), 2 residual only (write R)
};

// Mixed-precision defect correction: corr = R64(q) - R32(q) at a reference
// state q (both residuals formed with the first-stage semantics).  The FP32
// stages then drive R32 + corr to zero, whose fixed point, once q_ref is
// refreshed to the converged state, is R64 = 0: the FP64 solution, reached
// with FP32 face arithmetic between refreshes.
static __global__ void k_correction(const int n, const d4* __restrict__ R64, const d4* __restrict__ R32,
                             float4* __restrict__ corr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a[4], b[4];
    ld4(&R64[i], a);
    ld4(&R32[i], b);
    corr[i] = make_float4((float)(a[0] - b[0]), (float)(a[1] - b[1]), (float)(a[2] - b[2]), (float)(a[3] - b[3]));
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
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

// FP32-mixed epilogue.  GB300's FP64 pipe issues at ~1/64 of the FP32 rate,
// so FP64 is spent only where it accumulates: the RK increment
// R*dt*alpha*relaxation is formed in FP32; the intermediate stage states
// (which only feed FP32 fluxes) are q_shadow + increment in FP32; the new
// state of the last stage is q (FP64) + increment in FP64, and its FP32
// shadow is re-rounded from the FP64 result every iteration, so FP32
// rounding never accumulates in the state.  The norm sums per-cell FP32
// squares in FP64.
template <class S>
__device__ __forceinline__ void stage_epilogue_mixed(const StageOut<float, S>& o, const int i, const float* R0,
                                                     const float dti, double& sq) {
    // defect correction: R = R32(q) + (R64 - R32)(q_ref), see k_correction
    float R[4] = {R0[0], R0[1], R0[2], R0[3]};
    if (o.corr) {
        const float4 c = __ldg(&o.corr[i]);
        R[0] += c.x; R[1] += c.y; R[2] += c.z; R[3] += c.w;
    }
    const float fac = dti * (float)o.alpha * (float)o.relax;
    float inc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) inc[k] = R[k] * fac;
    if (o.mode == 0) {
        float qs[4];
        ld4(&o.q0s[i], qs);
        float qn[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) qn[k] = qs[k] + inc[k];
        V4<S> v;
        st4(&v, qn);
        o.qnext[i] = v;
    } else {
        double q0[4];
        ld4(&o.q0[i], q0);
        double qn[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) qn[k] = q0[k] + (double)inc[k];
        st4(&o.qm_next[i], qn);
        if (o.qsh_next) {
            V4<S> v;
            st4(&v, qn);
            o.qsh_next[i] = v;
        }
        sq += (double)(R[0] * R[0] + R[1] * R[1] + R[2] * R[2] + R[3] * R[3]);
    }
}
template <class S>
__device__ __forceinline__ void stage_epilogue_mixed(const StageOut<double, S>&, const int, const double*,
                                                     const double, double&) {}

template <class T, class S>
__device__ __forceinline__ void stage_epilogue(const StageOut<T, S>& o, const int i, const bool active, const T* Rsum,
                                               const T A, const T dti, const double extra_sq, double* sh) {
    double sq = extra_sq;
    if (active) {
        T R[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) R[k] = Rsum[k] / A;
        if (o.case_done && o.mode < 2 && __ldg(&o.case_done[__ldg(&o.case_of[i])])) {
            // a case that has stopped keeps its state
            if (o.mode == 0) {
                if (sizeof(T) == 4) {
                    T qs[4];
                    ld4s(&o.q0s[i], qs);
                    V4<S> v;
                    st4(&v, qs);
                    o.qnext[i] = v;
                } else {
                    double q0[4];
                    ld4(&o.q0[i], q0);
                    V4<S> v;
                    st4(&v, q0);
                    o.qnext[i] = v;
                }
            } else {
                double q0[4];
                ld4(&o.q0[i], q0);
                st4(&o.qm_next[i], q0);
                if (o.qsh_next) {
                    V4<S> v;
                    st4(&v, q0);
                    o.qsh_next[i] = v;
                }
                o.cell_sq[i] = 0.0;
            }
        } else if (o.mode == 2) {
            double Rd[4] = {(double)R[0], (double)R[1], (double)R[2], (double)R[3]};
            st4(&o.Rq[i], Rd);
        } else if (o.mode == 3) {
            // implicit right-hand side: the face sums, not divided by the area
            // (solver.h:1079-1152), and their squared norm; in a batch, the
            // rows of a case that has stopped are zero (its update is zero)
            double Rd[4] = {(double)Rsum[0], (double)Rsum[1], (double)Rsum[2], (double)Rsum[3]};
            if (o.case_done && __ldg(&o.case_done[__ldg(&o.case_of[i])])) Rd[0] = Rd[1] = Rd[2] = Rd[3] = 0.0;
            st4(&o.Rq[i], Rd);
#pragma unroll
            for (int k = 0; k < 4; ++k) sq += Rd[k] * Rd[k];
            if (o.cell_sq) o.cell_sq[i] = sq;
        } else if (sizeof(T) == 4) {
            stage_epilogue_mixed<S>(o, i, R, dti, sq);
        } else {
            double q0[4];
            ld4(&o.q0[i], q0);
            const double dtd = (double)dti;
            double qn[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) qn[k] = q0[k] + (double)R[k] * dtd * o.alpha * o.relax;
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
#pragma unroll
                for (int k = 0; k < 4; ++k) sq += (double)R[k] * (double)R[k];
            }
        }
        if (o.cell_sq && o.mode == 1 && !(o.case_done && __ldg(&o.case_done[__ldg(&o.case_of[i])]))) {
            // batch: the last stage's qW stays in Rq for a later
            // get_uniform_residual (each case stops at its own iteration)
            o.cell_sq[i] = sq;
            double Rd[4] = {(double)R[0], (double)R[1], (double)R[2], (double)R[3]};
            st4(&o.Rq[i], Rd);
        }
    }
    if (o.mode == 1 || o.mode == 3) {
        const double t = block_sum(sq, sh);
        if (threadIdx.x == 0) o.partials[blockIdx.x] = t;
    }
}

// Cell gather: each cell recomputes the fluxes of its faces (interior faces
// are evaluated twice, identically) and sums them in edge order.  No face
// buffer: the HBM-lean variant used by the FP32-mixed path.
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
    T A = T(1), dti = T(0);
    if (active) {
        const int4 sl = __ldg(&m.cslot[i]);
        const int4 nb = __ldg(&m.cnbr[i]);
        T qi[4], gxi[4] = {T(0), T(0), T(0), T(0)}, gyi[4] = {T(0), T(0), T(0), T(0)}, phii[4], qmi[4];
        ld4s(&qk[i], qi);
        if (SECOND || VISC >= 1) {
            ld4c<T>(&gx[i], gxi);
            ld4c<T>(&gy[i], gyi);
        }
        if (SECOND) ld4c<T>(&phi[i], phii);
        if (VISC >= 1) ld4s(&qmem[i], qmi);
        // rolled: the face flux is large, four inlined copies thrash the instruction cache
#pragma unroll 1
        for (int s = 0; s < 4; ++s) {
            const int fs = pick(sl, s);
            if (fs != 0) {
                const bool own0 = fs > 0;
                const int f = (own0 ? fs : -fs) - 1;
                const int oc = pick(nb, s);
                const V2<T> n = __ldg(&m.fn[f]);
                const T L = __ldg(&m.fLg[f]).x;
                T qA[4], qB[4];  // own side, other side (reconstructed)
                T gxo[4] = {T(0), T(0), T(0), T(0)}, gyo[4] = {T(0), T(0), T(0), T(0)};
                int bt = BT_INTERNAL;
                V2<T> dO, dN;
                if (SECOND) {
                    const V2<T> d0 = __ldg(&m.fd0[f]);
                    const V2<T> d1 = __ldg(&m.fd1[f]);
                    dO = own0 ? d0 : d1;
                    dN = own0 ? d1 : d0;
                    reconstruct(qi, gxi, gyi, phii, dO.x, dO.y, qA);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) qA[k] = qi[k];
                }
                if (oc >= 0) {
                    T qo[4];
                    ld4s(&qk[oc], qo);
                    if (SECOND || VISC >= 1) {
                        ld4c<T>(&gx[oc], gxo);
                        ld4c<T>(&gy[oc], gyo);
                    }
                    if (SECOND) {
                        T pho[4];
                        ld4c<T>(&phi[oc], pho);
                        reconstruct(qo, gxo, gyo, pho, dN.x, dN.y, qB);
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; ++k) qB[k] = qo[k];
                    }
                } else {
                    bt = __ldg(&m.btype[-oc - 1]);
                    ld4c<T>(&m.bq[-oc - 1], qB);
                }
                T qL[4], qR[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    qL[k] = own0 ? qA[k] : qB[k];
                    qR[k] = own0 ? qB[k] : qA[k];
                }
                T fgx[4] = {T(0), T(0), T(0), T(0)}, fgy[4] = {T(0), T(0), T(0), T(0)};
                if (VISC >= 1 && two_sided(bt)) {
                    T qmo[4];
                    if (oc >= 0) ld4s(&qmem[oc], qmo);
                    else ld4c<T>(&m.bq[-oc - 1], qmo);
                    T qa[4], qb[4], gxa[4], gya[4], gxb[4], gyb[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        qa[k] = own0 ? qmi[k] : qmo[k];
                        qb[k] = own0 ? qmo[k] : qmi[k];
                        gxa[k] = own0 ? gxi[k] : gxo[k];
                        gxb[k] = own0 ? gxo[k] : gxi[k];
                        gya[k] = own0 ? gyi[k] : gyo[k];
                        gyb[k] = own0 ? gyo[k] : gyi[k];
                    }
                    face_gradient(qa, qb, gxa, gya, gxb, gyb, ldv4<T>(&m.ft[f]), fgx, fgy);
                }
                T F[4];
                T mut_f = T(0);
                if (VISC == 2 && two_sided(bt)) mut_f = T(0.5) * (__ldg(&m.mut[i]) + __ldg(&m.mut[oc]));
                face_flux<T, VISC>(m, bt, n.x, n.y, qL, qR, fgx, fgy, F, mut_f);
                if (VISC == 2 && bt == BT_WALL) {
                    const V2<T> d0 = __ldg(&m.fd0[f]);
                    sa_wall_shear(m, n.x, n.y, d0.x, d0.y, qi, F);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const T fl = F[k] * L;
                    if (own0) {
                        Rs[k] -= fl;
                        if (oc < 0 && two_sided(bt)) extra += (double)fl * (double)fl;
                    } else {
                        Rs[k] += fl;
                    }
                }
            }
        }
        A = __ldg(&m.area[i]);
        if (o.mode < 2) dti = o.dt[i];
    }
    stage_epilogue<T, S>(o, i, active, Rs, A, dti, o.mode == 1 ? extra : 0.0, sh);
}

// F*L of face f for stage state qk (solver.h:751-786) and, with EIG, the
// face's spectral radius times length for the time step (solver.h:313-350).
// The ghost side of a boundary face is its stored boundary state (ghost
// gradients are zero).  Returns the face's boundary type in *btp.
template <class T, class S, int VISC, bool SECOND, bool EIG>
__device__ __forceinline__ void face_flux_at(const KM<T>& m, const int f, const V4<S>* __restrict__ qk,
                                             const V4<S>* __restrict__ qmem, const V4<T>* __restrict__ gx,
                                             const V4<T>* __restrict__ gy, const V4<T>* __restrict__ phi, T* fl,
                                             T* eLp, int* btp) {
    const int2 cc = __ldg(&m.fcell[f]);
    const V2<T> n = __ldg(&m.fn[f]);
    const T L = __ldg(&m.fLg[f]).x;
    T q0[4], q1[4], qL[4], qR[4];
    T gx0[4] = {T(0), T(0), T(0), T(0)}, gy0[4] = {T(0), T(0), T(0), T(0)};
    T gx1[4] = {T(0), T(0), T(0), T(0)}, gy1[4] = {T(0), T(0), T(0), T(0)};
    ld4s(&qk[cc.x], q0);
    if (SECOND || VISC >= 1) {
        ld4c<T>(&gx[cc.x], gx0);
        ld4c<T>(&gy[cc.x], gy0);
    }
    int bt = BT_INTERNAL;
    if (SECOND) {
        T p0[4];
        ld4c<T>(&phi[cc.x], p0);
        const V2<T> d0 = __ldg(&m.fd0[f]);
        reconstruct(q0, gx0, gy0, p0, d0.x, d0.y, qL);
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) qL[k] = q0[k];
    }
    if (cc.y >= 0) {
        ld4s(&qk[cc.y], q1);
        if (SECOND || VISC >= 1) {
            ld4c<T>(&gx[cc.y], gx1);
            ld4c<T>(&gy[cc.y], gy1);
        }
        if (SECOND) {
            T p1[4];
            ld4c<T>(&phi[cc.y], p1);
            const V2<T> d1 = __ldg(&m.fd1[f]);
            reconstruct(q1, gx1, gy1, p1, d1.x, d1.y, qR);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) qR[k] = q1[k];
        }
    } else {
        bt = __ldg(&m.btype[-cc.y - 1]);
        ld4c<T>(&m.bq[-cc.y - 1], q1);
#pragma unroll
        for (int k = 0; k < 4; ++k) qR[k] = q1[k];
    }
    if (EIG) {
        T eig;
        if (two_sided(bt)) {
            const T eL = face_eig(m.gamma, n.x, n.y, q0);
            const T eR = face_eig(m.gamma, n.x, n.y, q1);
            eig = smax(eL, eR);
        } else {
            eig = face_eig(m.gamma, n.x, n.y, q0);
        }
        *eLp = eig * L;
    }
    T fgx[4] = {T(0), T(0), T(0), T(0)}, fgy[4] = {T(0), T(0), T(0), T(0)};
    if (VISC >= 1 && two_sided(bt)) {
        T qa[4], qb[4];
        ld4s(&qmem[cc.x], qa);
        if (cc.y >= 0) ld4s(&qmem[cc.y], qb);
        else ld4c<T>(&m.bq[-cc.y - 1], qb);
        face_gradient(qa, qb, gx0, gy0, gx1, gy1, ldv4<T>(&m.ft[f]), fgx, fgy);
    }
    T F[4];
    T mut_f = T(0);
    if (VISC == 2 && two_sided(bt)) mut_f = T(0.5) * (__ldg(&m.mut[cc.x]) + __ldg(&m.mut[cc.y]));
    face_flux<T, VISC>(m, bt, n.x, n.y, qL, qR, fgx, fgy, F, mut_f);
    if (VISC == 2 && bt == BT_WALL) {
        const V2<T> d0 = __ldg(&m.fd0[f]);
        sa_wall_shear(m, n.x, n.y, d0.x, d0.y, q0, F);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) fl[k] = F[k] * L;
    *btp = cc.y >= 0 ? -1 : bt;  // -1: interior face
}

// Face variant, part 1: F*L of every face once (the flux is evaluated once
// per face instead of once per cell side).  With EIG (first stage) it also
// stores eig*L per face for the time step.
template <class T, class S, int VISC, bool SECOND, bool EIG>
__global__ void __launch_bounds__(256) k_face_flux(const KM<T> m, const int n_faces, const V4<S>* __restrict__ qk,
                                                   const V4<S>* __restrict__ qmem, const V4<T>* __restrict__ gx,
                                                   const V4<T>* __restrict__ gy, const V4<T>* __restrict__ phi,
                                                   V4<T>* __restrict__ fflux, T* __restrict__ feL,
                                                   const Ctrl* __restrict__ ctrl) {
    if (ctrl->done) return;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_faces) return;
    T fl[4], eL = T(0);
    int bt;
    face_flux_at<T, S, VISC, SECOND, EIG>(m, f, qk, qmem, gx, gy, phi, fl, &eL, &bt);
    V4<T> v;
    st4(&v, fl);
    fflux[f] = v;
    if (EIG) feL[f] = eL;
}

// Tile variant: one CTA per contiguous range of blockDim cells (cells are
// Hilbert ordered, so a tile is a compact patch).  Phase 1 forms F*L once for
// every face touching the tile — its own faces (a contiguous range, faces
// being sorted by their first cell) and the faces it shares with earlier
// tiles — into shared memory; phase 2 sums each cell's faces from shared
// memory in edge order and applies the stage epilogue.  Only faces on tile
// borders are formed twice; no face buffer goes through HBM.
struct TileView {
    const int* __restrict__ hstart;  // [ntiles+1] first own face of each tile
    const int* __restrict__ xptr;    // [ntiles+1] offsets into xlist
    const int* __restrict__ xlist;   // faces shared with an earlier tile
    const short4* __restrict__ ctile;  // per cell: +-(tile-local face + 1) per slot, edge order
};

template <class T, class S, int VISC, bool SECOND, bool EIG>
__global__ void __launch_bounds__(256, 8) k_resid_tile(const KM<T> m, const TileView tv, const V4<S>* __restrict__ qk,
                                                    const V4<S>* __restrict__ qmem, const V4<T>* __restrict__ gx,
                                                    const V4<T>* __restrict__ gy, const V4<T>* __restrict__ phi,
                                                    const StageOut<T, S> o, const Ctrl* __restrict__ ctrl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sh[32];
    if (ctrl->done) return;
    const int tile = blockIdx.x;
    const int h0 = __ldg(&tv.hstart[tile]), nh = __ldg(&tv.hstart[tile + 1]) - h0;
    const int x0 = __ldg(&tv.xptr[tile]), nf = nh + __ldg(&tv.xptr[tile + 1]) - x0;
    V4<T>* sF = reinterpret_cast<V4<T>*>(smem_raw);  // nf face fluxes F*L
    T* sE = reinterpret_cast<T*>(sF + nf);            // nf eig*L (EIG)
    double extra = 0;
    for (int j = threadIdx.x; j < nf; j += blockDim.x) {
        const int f = j < nh ? h0 + j : __ldg(&tv.xlist[x0 + j - nh]);
        T fl[4], eL = T(0);
        int bt;
        face_flux_at<T, S, VISC, SECOND, EIG>(m, f, qk, qmem, gx, gy, phi, fl, &eL, &bt);
        st4(&sF[j], fl);
        if (EIG) sE[j] = eL;
        if (o.mode == 1 && bt >= 0 && two_sided(bt))  // qW of a frozen ghost (solver.h:789-790)
#pragma unroll
            for (int k = 0; k < 4; ++k) extra += (double)fl[k] * (double)fl[k];
    }
    __syncthreads();
    const int i = tile * blockDim.x + threadIdx.x;
    const bool active = i < m.n_cells;
    T Rs[4] = {T(0), T(0), T(0), T(0)};
    T A = T(1), dti = T(0);
    if (active) {
        const short4 ts = __ldg(&tv.ctile[i]);
        T eigsum = T(0);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int v = s == 0 ? ts.x : (s == 1 ? ts.y : (s == 2 ? ts.z : ts.w));
            if (v != 0) {
                const int lf = (v > 0 ? v : -v) - 1;
                if (EIG) eigsum += sE[lf];
                T fl[4];
                ld4p(&sF[lf], fl);
                if (v > 0) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) Rs[k] -= fl[k];
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) Rs[k] += fl[k];
                }
            }
        }
        A = __ldg(&m.area[i]);
        if (EIG) {
            dti = m.cfl * A / eigsum;
            o.dt[i] = dti;
        } else if (o.mode < 2) {
            dti = o.dt[i];
        }
    }
    stage_epilogue<T, S>(o, i, active, Rs, A, dti, o.mode == 1 ? extra : 0.0, sh);
}

// Face variant, part 2: ordered per-cell sum of the face fluxes + epilogue.
// With DT (first stage) the local time step dt = cfl*A/sum(eig*L) is formed
// here from the face kernel's eig*L, in edge order, and stored.
template <class T, class S, bool DT>
__global__ void __launch_bounds__(256) k_cell_sum(const KM<T> m, const V4<T>* __restrict__ fflux,
                                                  const T* __restrict__ feL, const StageOut<T, S> o,
                                                  const Ctrl* __restrict__ ctrl) {
    __shared__ double sh[32];
    if (ctrl->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < m.n_cells;
    T Rs[4] = {T(0), T(0), T(0), T(0)};
    double extra = 0;
    T A = T(1), dti = T(0);
    if (active) {
        const int4 sl = __ldg(&m.cslot[i]);
        const int4 nb = __ldg(&m.cnbr[i]);
        T eigsum = T(0);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int fs = pick(sl, s);
            if (fs != 0) {
                const bool own0 = fs > 0;
                const int f = (own0 ? fs : -fs) - 1;
                T fl[4];
                ld4c<T>(&fflux[f], fl);
                if (DT) eigsum += __ldg(&feL[f]);
                if (own0) {
                    const int oc = pick(nb, s);
                    const bool ghost2 = oc < 0 && two_sided(__ldg(&m.btype[-oc - 1]));
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        Rs[k] -= fl[k];
                        if (ghost2) extra += (double)fl[k] * (double)fl[k];
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) Rs[k] += fl[k];
                }
            }
        }
        A = __ldg(&m.area[i]);
        if (DT) {
            dti = m.cfl * A / eigsum;
            o.dt[i] = dti;
        } else if (o.mode < 2) {
            dti = o.dt[i];
        }
    }
    stage_epilogue<T, S>(o, i, active, Rs, A, dti, o.mode == 1 ? extra : 0.0, sh);
}

// get_uniform_residual (solver.h:636-690): qW keeps its previous real-cell
// entries and gains the freestream fluxes (not divided by the area).
template <class T, class S, int VISC>
__global__ void __launch_bounds__(256) k_uniform(const KM<T> m, const V4<S>* __restrict__ qmem,
                                                 const V4<T>* __restrict__ gx, const V4<T>* __restrict__ gy,
                                                 const double q0, const double q1, const double q2, const double q3,
                                                 d4* __restrict__ Rq, double* __restrict__ partials,
                                                 const double* __restrict__ qfar_case, const int* __restrict__ case_of,
                                                 double* __restrict__ cell_sq) {
    __shared__ double sh[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0;
    if (i < m.n_cells) {
        T qf[4] = {(T)q0, (T)q1, (T)q2, (T)q3};
        if (qfar_case) {  // batch: the freestream of this cell's case
            const int c = __ldg(&case_of[i]);
#pragma unroll
            for (int k = 0; k < 4; ++k) qf[k] = (T)__ldg(&qfar_case[4 * c + k]);
        }
        double acc[4];
        ld4(&Rq[i], acc);
        T accT[4] = {(T)acc[0], (T)acc[1], (T)acc[2], (T)acc[3]};
        const int4 sl = __ldg(&m.cslot[i]);
        const int4 nb = __ldg(&m.cnbr[i]);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int fs = pick(sl, s);
            if (fs != 0) {
                const bool own0 = fs > 0;
                const int f = (own0 ? fs : -fs) - 1;
                const int oc = pick(nb, s);
                const V2<T> n = __ldg(&m.fn[f]);
                const T L = __ldg(&m.fLg[f]).x;
                int bt = BT_INTERNAL;
                if (oc < 0) bt = __ldg(&m.btype[-oc - 1]);
                T fgx[4] = {T(0), T(0), T(0), T(0)}, fgy[4] = {T(0), T(0), T(0), T(0)};
                if (VISC >= 1 && two_sided(bt)) {
                    T qi[4], qo[4], gxi[4], gyi[4], gxo[4] = {T(0), T(0), T(0), T(0)},
                                                      gyo[4] = {T(0), T(0), T(0), T(0)};
                    ld4s(&qmem[i], qi);
                    ld4c<T>(&gx[i], gxi);
                    ld4c<T>(&gy[i], gyi);
                    if (oc >= 0) {
                        ld4s(&qmem[oc], qo);
                        ld4c<T>(&gx[oc], gxo);
                        ld4c<T>(&gy[oc], gyo);
                    } else {
                        ld4c<T>(&m.bq[-oc - 1], qo);
                    }
                    T qa[4], qb[4], gxa[4], gya[4], gxb[4], gyb[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        qa[k] = own0 ? qi[k] : qo[k];
                        qb[k] = own0 ? qo[k] : qi[k];
                        gxa[k] = own0 ? gxi[k] : gxo[k];
                        gxb[k] = own0 ? gxo[k] : gxi[k];
                        gya[k] = own0 ? gyi[k] : gyo[k];
                        gyb[k] = own0 ? gyo[k] : gyi[k];
                    }
                    face_gradient(qa, qb, gxa, gya, gxb, gyb, ldv4<T>(&m.ft[f]), fgx, fgy);
                }
                T F[4];
                T mut_f = T(0);
                if (VISC == 2 && two_sided(bt)) mut_f = T(0.5) * (__ldg(&m.mut[i]) + __ldg(&m.mut[oc]));
                face_flux<T, VISC>(m, bt, n.x, n.y, qf, qf, fgx, fgy, F, mut_f);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const T fl = F[k] * L;
                    if (own0) {
                        accT[k] -= fl;
                        if (oc < 0 && two_sided(bt)) sq += (double)fl * (double)fl;
                    } else {
                        accT[k] += fl;
                    }
                }
            }
        }
        double out[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            out[k] = (double)accT[k];
            sq += out[k] * out[k];
        }
        st4(&Rq[i], out);
        if (cell_sq) cell_sq[i] = sq;
    }
    const double t = block_sum(sq, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// Per-case norm and run_solver control of a batch (multigrid.h:195-234 for
// every case): one block per case sums the per-cell squares of its cells in
// a fixed order.  A case that stops is marked in case_done (its cells then
// hold their state); the whole run stops when every case has.
// Sum of cell_sq over [b0, b1) by one block: four accumulators per thread
// (several loads in flight), then the fixed-order block sum.
__device__ __forceinline__ double case_sum(const double* __restrict__ cell_sq, const int b0, const int b1,
                                           double* sh) {
    const int st = blockDim.x;
    double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    int k = b0 + threadIdx.x;
    for (; k + 3 * st < b1; k += 4 * st) {
        v0 += cell_sq[k];
        v1 += cell_sq[k + st];
        v2 += cell_sq[k + 2 * st];
        v3 += cell_sq[k + 3 * st];
    }
    for (; k < b1; k += st) v0 += cell_sq[k];
    return block_sum((v0 + v1) + (v2 + v3), sh);
}

static __global__ void __launch_bounds__(1024) k_case_control(const double* __restrict__ cell_sq,
                                                             const int* __restrict__ case_off, CaseCtrl* cctrl,
                                                             int* case_done, double* chist, Ctrl* ctrl, int n_cases,
                                                             int uniform) {
    __shared__ double sh[32];
    if (!uniform && ctrl->done) return;
    const int c = blockIdx.x;
    CaseCtrl& cc = cctrl[c];
    if (!uniform && cc.done) return;
    const int b0 = case_off[c], b1 = case_off[c + 1];
    const double t = case_sum(cell_sq, b0, b1, sh);
    if (threadIdx.x != 0) return;
    const double norm = sqrt(t);
    if (uniform) {
        cc.err0 = norm;
        return;
    }
    const int i = cc.iter;
    cc.last_norm = norm;
    double err = norm;
    bool stop = false;
    if (!(norm == norm) || norm > 1.7976931348623157e308) {
        cc.status = 4;
        stop = true;
    }
    if (ctrl->run_mode) {
        if (i == 0 && err > 2 * cc.err0) cc.err0 = err;
        if (err > 0) err /= cc.err0;
        cc.err = err;
        if (i % 10 == 0 && cc.hist_n < CASE_HIST_CAP) chist[(size_t)c * CASE_HIST_CAP + cc.hist_n++] = err;
        if (!((err > ctrl->tol) && (i + 1 < ctrl->max_it))) stop = true;
    }
    cc.iter = i + 1;
    if (ctrl->run_mode == 0) cc.err = err;
    if (stop) {
        cc.done = 1;
        case_done[c] = 1;
        atomicAdd(&ctrl->ndone, 1);
    }
}

// Implicit batches, right after a right-hand side: a case whose face sums
// are not finite stops (status 4) and its right-hand-side rows are zeroed
// before the linear solve, so it cannot spread into the other cases.
static __global__ void __launch_bounds__(1024) k_case_nonfinite(const double* __restrict__ cell_sq,
                                                               const int* __restrict__ case_off, CaseCtrl* cctrl,
                                                               int* case_done, Ctrl* ctrl, d4* __restrict__ b) {
    __shared__ double sh[32];
    __shared__ int bad;
    const int c = blockIdx.x;
    if (cctrl[c].done) return;
    const int b0 = case_off[c], b1 = case_off[c + 1];
    const double t = case_sum(cell_sq, b0, b1, sh);
    if (threadIdx.x == 0) {
        bad = !(t == t) || t > 1.7976931348623157e308;
        if (bad) {
            cctrl[c].status = 4;
            cctrl[c].done = 1;
            case_done[c] = 1;
            atomicAdd(&ctrl->ndone, 1);
        }
    }
    __syncthreads();
    if (bad) {
        const double z[4] = {0, 0, 0, 0};
        for (int k = b0 + threadIdx.x; k < b1; k += blockDim.x) st4(&b[k], z);
    }
}

// After k_case_control: count the iteration and stop the run once every
// case has stopped (a separate launch, so no block of k_case_control sees
// the run's flag change under it).
static __global__ void k_batch_finalize(Ctrl* ctrl, int n_cases) {
    if (ctrl->done) return;
    ctrl->iter += 1;
    if (ctrl->ndone >= n_cases) ctrl->done = 1;
}

// Residual-norm finalisation and the run_solver control (multigrid.h:195-234)
// in one block: fixed-order sum of the partials -> ‖qW‖₂, err/err_0,
// convergence test, history every 10th iteration.
static __global__ void __launch_bounds__(1024) k_control(const double* __restrict__ partials, int n, Ctrl* ctrl,
                                                         double* hist, double* norms, int uniform) {
    __shared__ double sh[32];
    if (!uniform && ctrl->done) return;
    // four independent accumulators per thread keep four loads in flight
    double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    const int st = blockDim.x;
    int k = threadIdx.x;
    for (; k + 3 * st < n; k += 4 * st) {
        v0 += partials[k];
        v1 += partials[k + st];
        v2 += partials[k + 2 * st];
        v3 += partials[k + 3 * st];
    }
    for (; k < n; k += st) v0 += partials[k];
    const double t = block_sum((v0 + v1) + (v2 + v3), sh);
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
