// Launch sequences of one explicit iteration and its helpers, instantiated
// once per precision (afx_kernels_f64.cu, afx_kernels_f32.cu).
#pragma once

#include "afx_kernels.cuh"
#include "afx_sa.cuh"

namespace afx {
namespace dev {

template <class T>
KM<T> make_km(const StepArgs& a) {
    KM<T> m;
    m.n_cells = a.n_cells;
    m.cslot = (const int4*)a.cslot;
    m.cnbr = (const int4*)a.cnbr;
    m.area = (const T*)a.area;
    m.fcell = (const int2*)a.fcell;
    m.fn = (const V2<T>*)a.fn;
    m.fLg = (const V2<T>*)a.fLg;
    m.fd0 = (const V2<T>*)a.fd0;
    m.fd1 = (const V2<T>*)a.fd1;
    m.ft = (const V4<T>*)a.ft;
    m.btype = (const int*)a.btype;
    m.bq = (const V4<T>*)a.bq;
    m.gamma = (T)a.gamma;
    m.R = (T)a.R;
    m.mu = (T)a.mu;
    m.kheat = (T)a.kheat;
    m.limk = (T)a.limiter_k;
    m.cfl = (T)a.cfl;
    m.limiter = a.limiter;
    m.lsq = a.lsq;
    m.lsqw = (const V2<T>*)a.lsqw;
    m.lsqs = a.lsqs;
    m.mut = (const T*)a.sa_mut;
    m.cp = (T)a.cp;
    m.PrL = (T)a.Pr_L;
    m.PrT = (T)a.Pr_T;
    return m;
}

inline int nblocks(int n, int b) { return (n + b - 1) / b; }

inline void mark(const StepArgs& a, int id, cudaStream_t s) {
    if (a.prof) a.prof->mark(id, s);
}

template <class T, class S>
void launch_prep(const StepArgs& a, const KM<T>& m, const V4<S>* q, cudaStream_t s) {
    const int nb = nblocks(a.n_cells, a.block);
    V4<T>* gx = (V4<T>*)a.gx;
    V4<T>* gy = (V4<T>*)a.gy;
    V4<T>* ph = (V4<T>*)a.phi;
    T* dt = (T*)a.dt;
    // the face and tile variants form dt in their first stage (EIG/DT)
    if (a.variant != 0) {
        if (a.second)
            k_prep<T, S, true, true, false><<<nb, a.block, 0, s>>>(m, q, gx, gy, ph, dt, a.ctrl);
        else if (a.need_grad)
            k_prep<T, S, true, false, false><<<nb, a.block, 0, s>>>(m, q, gx, gy, ph, dt, a.ctrl);
        else
            return;
    } else {
        if (a.second)
            k_prep<T, S, true, true, true><<<nb, a.block, 0, s>>>(m, q, gx, gy, ph, dt, a.ctrl);
        else if (a.need_grad)
            k_prep<T, S, true, false, true><<<nb, a.block, 0, s>>>(m, q, gx, gy, ph, dt, a.ctrl);
        else
            k_prep<T, S, false, false, true><<<nb, a.block, 0, s>>>(m, q, gx, gy, ph, dt, a.ctrl);
    }
    mark(a, K_PREP, s);
}

template <class T, class S, int VISC, bool SECOND>
void launch_stage_v(const StepArgs& a, const KM<T>& m, const V4<S>* qk, const V4<S>* qmem,
                    const StageOut<T, S>& o, bool first, cudaStream_t s) {
    const int nb = nblocks(a.n_cells, a.block);
    const V4<T>* gx = (const V4<T>*)a.gx;
    const V4<T>* gy = (const V4<T>*)a.gy;
    const V4<T>* ph = (const V4<T>*)a.phi;
    if (a.variant == 2) {
        TileView tv;
        tv.hstart = a.tile_hstart;
        tv.xptr = a.tile_xptr;
        tv.xlist = a.tile_xlist;
        tv.ctile = (const short4*)a.tile_ctile;
        const size_t smem = (size_t)a.tile_maxnf * 5 * sizeof(T);
        if (first) {
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(k_resid_tile<T, S, VISC, SECOND, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_resid_tile<T, S, VISC, SECOND, true><<<nb, a.block, smem, s>>>(m, tv, qk, qmem, gx, gy, ph, o, a.ctrl);
        } else {
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(k_resid_tile<T, S, VISC, SECOND, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_resid_tile<T, S, VISC, SECOND, false><<<nb, a.block, smem, s>>>(m, tv, qk, qmem, gx, gy, ph, o, a.ctrl);
        }
        mark(a, K_RESID_TILE, s);
    } else if (a.variant == 1) {
        const int nbf = nblocks(a.n_faces, a.block);
        if (first) {
            k_face_flux<T, S, VISC, SECOND, true><<<nbf, a.block, 0, s>>>(
                m, a.n_faces, qk, qmem, gx, gy, ph, (V4<T>*)a.fflux, (T*)a.feL, a.ctrl);
            mark(a, K_FACE_FLUX, s);
            k_cell_sum<T, S, true><<<nb, a.block, 0, s>>>(m, (const V4<T>*)a.fflux, (const T*)a.feL, o, a.ctrl);
        } else {
            k_face_flux<T, S, VISC, SECOND, false><<<nbf, a.block, 0, s>>>(
                m, a.n_faces, qk, qmem, gx, gy, ph, (V4<T>*)a.fflux, (T*)a.feL, a.ctrl);
            mark(a, K_FACE_FLUX, s);
            k_cell_sum<T, S, false><<<nb, a.block, 0, s>>>(m, (const V4<T>*)a.fflux, (const T*)a.feL, o, a.ctrl);
        }
        mark(a, K_CELL_SUM, s);
    } else {
        k_resid_gather<T, S, VISC, SECOND><<<nb, a.block, 0, s>>>(m, qk, qmem, gx, gy, ph, o, a.ctrl);
        mark(a, K_RESID_GATHER, s);
    }
}

template <class T, class S>
void launch_stage(const StepArgs& a, const KM<T>& m, const V4<S>* qk, const V4<S>* qmem, const StageOut<T, S>& o,
                  bool first, cudaStream_t s) {
    if (a.visc == 2) {
        if (a.second) launch_stage_v<T, S, 2, true>(a, m, qk, qmem, o, first, s);
        else launch_stage_v<T, S, 2, false>(a, m, qk, qmem, o, first, s);
    } else if (a.visc == 1) {
        if (a.second) launch_stage_v<T, S, 1, true>(a, m, qk, qmem, o, first, s);
        else launch_stage_v<T, S, 1, false>(a, m, qk, qmem, o, first, s);
    } else {
        if (a.second) launch_stage_v<T, S, 0, true>(a, m, qk, qmem, o, first, s);
        else launch_stage_v<T, S, 0, false>(a, m, qk, qmem, o, first, s);
    }
}

// Spalart-Allmaras: the view of one evaluation, mu_t of a stage state, one
// stage of nu~ (see afx_sa.cuh).
template <class T>
SaView<T> sa_view(const StepArgs& a) {
    SaView<T> v;
    v.nu0 = v.nuk = nullptr;
    v.nu_next = nullptr;
    v.nuW = (double*)a.sa_nuW;
    v.wd = (const T*)a.sa_wd;
    v.cxy = (const V2<T>*)a.sa_cxy;
    v.gxy = (const V2<T>*)a.sa_gxy;
    v.dt = (const T*)a.dt;
    v.nu_far = (T)a.sa_nu_far;
    v.alpha = 1.0;
    v.relax = a.relax;
    return v;
}

template <class T, class S>
void sa_mut(const StepArgs& a, const V4<S>* qk, const void* nuk, cudaStream_t s) {
    k_sa_mut<T, S><<<nblocks(a.n_cells, 256), 256, 0, s>>>(a.n_cells, qk, (const double*)nuk, (T)a.mu,
                                                           (T*)a.sa_mut, a.ctrl);
}

template <class T, class S>
void sa_stage(const StepArgs& a, const KM<T>& m, const V4<S>* qk, const void* nu0, const void* nuk, void* nu_next,
              double alpha, cudaStream_t s) {
    SaView<T> v = sa_view<T>(a);
    v.nu0 = (const double*)nu0;
    v.nuk = (const double*)nuk;
    v.nu_next = (double*)nu_next;
    v.alpha = alpha;
    k_sa_stage<T, S><<<nblocks(a.n_cells, 256), 256, 0, s>>>(m, qk, (const V4<T>*)a.gx, (const V4<T>*)a.gy, v,
                                                             a.ctrl);
}

template <class T, class S>
StageOut<T, S> base_out(const StepArgs& a, int p) {
    StageOut<T, S> o;
    o.q0 = (const d4*)a.qm[p];
    o.q0s = (const V4<S>*)a.qsh[p];
    o.qnext = nullptr;
    o.qm_next = nullptr;
    o.qsh_next = nullptr;
    o.Rq = (d4*)a.Rq;
    o.dt = (T*)a.dt;
    o.alpha = 1.0;
    o.relax = a.relax;
    o.partials = a.partials;
    o.corr = (const float4*)a.corr;
    o.case_of = a.case_of;
    o.case_done = a.case_done;
    o.cell_sq = a.cell_sq;
    o.mode = 0;
    return o;
}

// explicitSolver::solve (solver.h:802-828): dt, gradients and first limiter
// from q; three stages alpha = 1/4, 1/2, 1 with the limiter re-formed from
// each stage state; the new state goes to parity p^1.
template <class T, class S, bool SHADOW>
void iteration(const StepArgs& a, int p, cudaStream_t s) {
    const KM<T> m = make_km<T>(a);
    const V4<S>* q = (const V4<S>*)a.qsh[p];
    launch_prep<T, S>(a, m, q, s);
    static const double alpha[3] = {0.25, 0.5, 1.0};
    StageOut<T, S> o = base_out<T, S>(a, p);
    for (int st = 0; st < 3; ++st) {
        const V4<S>* qk = st == 0 ? q : (const V4<S>*)a.qs[st - 1];
        if (st > 0 && a.second) {
            k_limiter<T, S><<<nblocks(a.n_cells, a.block), a.block, 0, s>>>(
                m, qk, (const V4<T>*)a.gx, (const V4<T>*)a.gy, (V4<T>*)a.phi, a.ctrl);
            mark(a, K_LIMITER, s);
        }
        // Spalart-Allmaras: eddy viscosity of the stage state first
        const void* nuk = st == 0 ? a.sa_nu[p] : a.sa_nus[st - 1];
        if (a.visc == 2) sa_mut<T, S>(a, qk, nuk, s);
        o.alpha = alpha[st];
        if (st < 2) {
            o.mode = 0;
            o.qnext = (V4<S>*)a.qs[st];
        } else {
            o.mode = 1;
            o.qnext = nullptr;
            o.qm_next = (d4*)a.qm[p ^ 1];
            o.qsh_next = SHADOW ? (V4<S>*)a.qsh[p ^ 1] : nullptr;
        }
        launch_stage<T, S>(a, m, qk, q, o, st == 0, s);
        // ... then its nu~ stage from the same stage state (the time step
        // was formed by the first stage's mean-flow launch)
        if (a.visc == 2)
            sa_stage<T, S>(a, m, qk, a.sa_nu[p], nuk, st < 2 ? a.sa_nus[st] : a.sa_nu[p ^ 1], alpha[st], s);
    }
    if (a.n_cases > 0) {
        k_case_control<<<a.n_cases, 1024, 0, s>>>(a.cell_sq, a.case_off, a.cctrl, a.case_done, a.chist, a.ctrl,
                                                 a.n_cases, 0);
        k_batch_finalize<<<1, 1, 0, s>>>(a.ctrl, a.n_cases);
    } else {
        k_control<<<1, 1024, 0, s>>>(a.partials, nblocks(a.n_cells, a.block), a.ctrl, a.hist, a.norms, 0);
    }
    mark(a, K_CONTROL, s);
}

// Residual of state parity p as the first RK stage forms it -> Rq.
template <class T, class S>
void residual(const StepArgs& a, int p, cudaStream_t s) {
    const KM<T> m = make_km<T>(a);
    const V4<S>* q = (const V4<S>*)a.qsh[p];
    launch_prep<T, S>(a, m, q, s);
    if (a.visc == 2) sa_mut<T, S>(a, q, a.sa_nu[p], s);
    StageOut<T, S> o = base_out<T, S>(a, p);
    o.mode = 2;
    launch_stage<T, S>(a, m, q, q, o, false, s);
    if (a.visc == 2) sa_stage<T, S>(a, m, q, a.sa_nu[p], a.sa_nu[p], nullptr, 1.0, s);
}

// Implicit right-hand side of state parity p (first-stage reconstruction,
// face sums not divided by the area) -> Rq, ||.||^2 block partials.
template <class T, class S>
void rhs(const StepArgs& a, int p, cudaStream_t s) {
    const KM<T> m = make_km<T>(a);
    const V4<S>* q = (const V4<S>*)a.qsh[p];
    launch_prep<T, S>(a, m, q, s);
    if (a.visc == 2) sa_mut<T, S>(a, q, a.sa_nu[p], s);
    StageOut<T, S> o = base_out<T, S>(a, p);
    o.mode = 3;
    launch_stage<T, S>(a, m, q, q, o, false, s);
}

// qW of the last stage of the iteration that read parity p (stage state in
// qs[1], gradients and stage-3 limiter still in place).
template <class T, class S>
void last_stage_residual(const StepArgs& a, int p, cudaStream_t s) {
    const KM<T> m = make_km<T>(a);
    StageOut<T, S> o = base_out<T, S>(a, p);
    o.mode = 2;
    if (a.visc == 2) sa_mut<T, S>(a, (const V4<S>*)a.qs[1], a.sa_nus[1], s);
    launch_stage<T, S>(a, m, (const V4<S>*)a.qs[1], (const V4<S>*)a.qsh[p], o, false, s);
}

template <class T, class S>
void uniform(const StepArgs& a, int p, const double* qf, cudaStream_t s) {
    const KM<T> m = make_km<T>(a);
    const int nb = nblocks(a.n_cells, a.block);
    const V4<S>* q = (const V4<S>*)a.qsh[p];
    if (a.visc == 2) {
        sa_mut<T, S>(a, q, a.sa_nu[p], s);
        k_uniform<T, S, 2><<<nb, a.block, 0, s>>>(m, q, (const V4<T>*)a.gx, (const V4<T>*)a.gy, qf[0], qf[1],
                                                   qf[2], qf[3], (d4*)a.Rq, a.partials, a.qfar_case, a.case_of,
                                                   a.cell_sq);
    } else if (a.visc == 1)
        k_uniform<T, S, 1><<<nb, a.block, 0, s>>>(m, q, (const V4<T>*)a.gx, (const V4<T>*)a.gy, qf[0], qf[1],
                                                   qf[2], qf[3], (d4*)a.Rq, a.partials, a.qfar_case, a.case_of,
                                                   a.cell_sq);
    else
        k_uniform<T, S, 0><<<nb, a.block, 0, s>>>(m, q, (const V4<T>*)a.gx, (const V4<T>*)a.gy, qf[0], qf[1],
                                                   qf[2], qf[3], (d4*)a.Rq, a.partials, a.qfar_case, a.case_of,
                                                   a.cell_sq);
    if (a.n_cases > 0)
        k_case_control<<<a.n_cases, 1024, 0, s>>>(a.cell_sq, a.case_off, a.cctrl, a.case_done, a.chist, a.ctrl,
                                                 a.n_cases, 1);
    else
        k_control<<<1, 1024, 0, s>>>(a.partials, nb, a.ctrl, a.hist, nullptr, 1);
}

// Implicit solver, Spalart-Allmaras: `sweeps` point-implicit nu~ updates
// from the state of parity p (gradients formed here), in place in sa_nu[p]
// through the stage buffer; mu_t of the final nu~ last.
template <class T, class S>
void sa_implicit(const StepArgs& a0, int p, int sweeps, cudaStream_t s) {
    StepArgs a = a0;
    a.variant = 0;  // dt with the prep (the CFL in a.cfl)
    a.second = 0;
    a.need_grad = 1;
    const KM<T> m = make_km<T>(a);
    const V4<S>* q = (const V4<S>*)a.qsh[p];
    launch_prep<T, S>(a, m, q, s);
    SaView<T> v = sa_view<T>(a);
    for (int k = 0; k < sweeps; ++k) {
        v.nuk = (const double*)a.sa_nu[p];
        v.nu_next = (double*)a.sa_nus[0];
        k_sa_implicit<T, S><<<nblocks(a.n_cells, 256), 256, 0, s>>>(m, q, (const V4<T>*)a.gx, (const V4<T>*)a.gy,
                                                                    v, a.ctrl);
        cudaMemcpyAsync(a.sa_nu[p], a.sa_nus[0], (size_t)a.n_cells * 8, cudaMemcpyDeviceToDevice, s);
    }
    sa_mut<T, S>(a, q, a.sa_nu[p], s);
}

}  // namespace dev
}  // namespace afx
