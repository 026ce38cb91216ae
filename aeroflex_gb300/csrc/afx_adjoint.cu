// Adjoint of the FP64 residual: u = (dR/dq)^T v and b = (dR/dbq)^T v for the
// residual R(q) of the explicit solver's first stage (solver.h:745-799 with
// the gradient of solver.h:428-469 and the limiter of solver.h:517-593, all
// formed from q), where bq are the stored boundary (farfield) states.
//
// Reverse sweep in three gather kernels, deterministic and atomic-free:
//   k_adj_face   per face: the face flux's local Jacobians are formed on the
//                fly by forward-mode dual numbers (8 directions: left state,
//                right state or boundary state; 1, 2 or 4 of them per pass
//                as vector duals, which share the value's work) and contracted
//                with the face weight L*(v_c1/A_c1 - v_c0/A_c0) -> 8 numbers
//                per face.
//   k_adj_cell   per cell: gathers its faces' numbers into the state,
//                limiter and gradient adjoints of the reconstruction
//                q + phi .* (grad q . d), then reverses its limiter (active
//                face of the min, neighbour of the max/min) -- the
//                neighbour terms are left as (target, weight) pairs.
//   k_adj_final  per cell: adds the limiter pairs that target it and the
//                Green-Gauss gradient's reverse over its faces, and writes
//                the boundary-state adjoint of its boundary faces.
// Face Jacobians are never stored.  Roe flux with the entropy fix and every
// boundary type, and the laminar term (then 16 directions per face: the
// face gradient's inputs too, reversed through average_gradients);
// first or second order; both limiters.
#include "afx_dual.cuh"
#include "afx_kernels_impl.cuh"

namespace afx {
namespace dev {

constexpr int ADJ_NONE = (int)0x80000000;  // limiter target: none / the cell itself

__device__ __forceinline__ int pick4(const int4 v, const int k) { return pick(v, k); }

// out[j] = sum_m dF_m/d(dir0 + j) * w_m of the face flux, j < K, for input
// directions dir0 .. dir0+K-1 (0-3: left state, 4-7: right state, or the
// boundary state when one-sided; with the laminar term, 8-11 / 12-15: the
// face gradient's x / y parts), all K in one pass of vector duals
template <int VISC, int K>
__device__ __forceinline__ void face_flux_dirs(const KM<double>& m, const int bt, const double nx, const double ny,
                                               const double* qL, const double* qR, const double* fgx,
                                               const double* fgy, const int dir0, const double* w, double* out) {
    using D = DualV<K>;
    D dL[4], dR[4], F[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        dL[k] = D(qL[k]);
        dR[k] = D(qR[k]);
#pragma unroll
        for (int j = 0; j < K; ++j) {
            dL[k].d[j] = dir0 + j == k ? 1.0 : 0.0;
            dR[k].d[j] = dir0 + j == k + 4 ? 1.0 : 0.0;
        }
    }
    if (two_sided(bt)) {
        roe_flux<D>(D(m.gamma), D(nx), D(ny), dL, dR, F);
        if (VISC == 1) {
            D gxd[4], gyd[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                gxd[k] = D(fgx[k]);
                gyd[k] = D(fgy[k]);
#pragma unroll
                for (int j = 0; j < K; ++j) {
                    gxd[k].d[j] = dir0 + j == k + 8 ? 1.0 : 0.0;
                    gyd[k].d[j] = dir0 + j == k + 12 ? 1.0 : 0.0;
                }
            }
            laminar_flux<D>(D(m.gamma), D(m.R), D(m.mu), D(m.kheat), D(nx), D(ny), dL, dR, gxd, gyd, F);
        }
    } else {
        D qb[4];
        ghost_state<D>(bt, D(m.gamma), D(nx), D(ny), dL, dR, qb);
        roe_flux<D>(D(m.gamma), D(nx), D(ny), dL, qb, F);
    }
#pragma unroll
    for (int j = 0; j < K; ++j) out[j] = F[0].d[j] * w[0] + F[1].d[j] * w[1] + F[2].d[j] * w[2] + F[3].d[j] * w[3];
}

// sum_m d ghost_m/d(dir) * w_m (dir 0-3: interior state, 4-7: boundary state)
__device__ __forceinline__ double ghost_dir(const int bt, const double gamma, const double nx, const double ny,
                                            const double* qi, const double* qb, const int dir, const double* w) {
    Dual a[4], b[4], g[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[k] = Dual(qi[k], dir == k ? 1.0 : 0.0);
        b[k] = Dual(qb[k], dir == k + 4 ? 1.0 : 0.0);
    }
    ghost_state<Dual>(bt, Dual(gamma), Dual(nx), Dual(ny), a, b, g);
    return g[0].d * w[0] + g[1].d * w[1] + g[2].d * w[2] + g[3].d * w[3];
}

// Per face, FB = 2 (inviscid) or 8 (laminar) 4-vectors of fbar:
// [qL_bar, qR_bar (or the boundary state's), and with the laminar term
//  gxa_bar, gya_bar, qa_bar, gxb_bar, gyb_bar, qb_bar] -- a/b: the face's
// cells as the face gradient sees them (solver.h:359-398)
template <bool SECOND, int VISC, int ADJ_K>
__global__ void __launch_bounds__(128) k_adj_face(const KM<double> m, const int n_faces, const d4* __restrict__ q,
                                                  const d4* __restrict__ gx, const d4* __restrict__ gy,
                                                  const d4* __restrict__ phi, const d4* __restrict__ v,
                                                  d4* __restrict__ fbar) {
    constexpr int FB = VISC == 1 ? 8 : 2;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_faces) return;
    const int2 cc = __ldg(&m.fcell[f]);
    const double2 n = __ldg(&m.fn[f]);
    const double L = __ldg(&m.fLg[f]).x;
    double q0[4], q1[4], qL[4], qR[4], w[4], v0[4];
    double g0x[4] = {0, 0, 0, 0}, g0y[4] = {0, 0, 0, 0}, g1x[4] = {0, 0, 0, 0}, g1y[4] = {0, 0, 0, 0};
    ld4(&q[cc.x], q0);
    if (SECOND || VISC == 1) {
        ld4(&gx[cc.x], g0x);
        ld4(&gy[cc.x], g0y);
    }
    if (SECOND) {
        double p0[4];
        ld4(&phi[cc.x], p0);
        const double2 d0 = __ldg(&m.fd0[f]);
        reconstruct(q0, g0x, g0y, p0, d0.x, d0.y, qL);
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) qL[k] = q0[k];
    }
    ld4(&v[cc.x], v0);
    const double A0 = __ldg(&m.area[cc.x]);
    int bt = BT_INTERNAL;
    if (cc.y >= 0) {
        double v1[4];
        ld4(&q[cc.y], q1);
        if (SECOND || VISC == 1) {
            ld4(&gx[cc.y], g1x);
            ld4(&gy[cc.y], g1y);
        }
        if (SECOND) {
            double p1[4];
            ld4(&phi[cc.y], p1);
            const double2 d1 = __ldg(&m.fd1[f]);
            reconstruct(q1, g1x, g1y, p1, d1.x, d1.y, qR);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) qR[k] = q1[k];
        }
        ld4(&v[cc.y], v1);
        const double A1 = __ldg(&m.area[cc.y]);
        // R_c0 -= F*L/A_c0, R_c1 += F*L/A_c1
#pragma unroll
        for (int k = 0; k < 4; ++k) w[k] = L * (v1[k] / A1 - v0[k] / A0);
    } else {
        bt = __ldg(&m.btype[-cc.y - 1]);
        ld4(&m.bq[-cc.y - 1], q1);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            qR[k] = q1[k];
            w[k] = -L * (v0[k] / A0);
        }
    }
    // the face gradient of the laminar term (member states, cell gradients;
    // a boundary side has zero gradient)
    const bool lam = VISC == 1 && two_sided(bt);
    double fgx[4] = {0, 0, 0, 0}, fgy[4] = {0, 0, 0, 0};
    double4 t = make_double4(0, 0, 1, 0);  // (t0, t1, lij): zero adjoint on a face without the term
    if (lam) {
        const d4 tt = ldv4d(&m.ft[f]);
        t = make_double4(tt.x, tt.y, tt.z, tt.w);
        face_gradient(q0, q1, g0x, g0y, g1x, g1y, tt, fgx, fgy);
    }
    constexpr int ND = VISC == 1 ? 16 : 8;
    double out[ND];
#pragma unroll 1
    for (int dir = 0; dir < ND; dir += ADJ_K) {
        if (dir < 8 || lam) {
            double o[ADJ_K];
            face_flux_dirs<VISC, ADJ_K>(m, bt, n.x, n.y, qL, qR, fgx, fgy, dir, w, o);
#pragma unroll
            for (int j = 0; j < ADJ_K; ++j) out[dir + j] = o[j];
        } else {
#pragma unroll
            for (int j = 0; j < ADJ_K; ++j) out[dir + j] = 0.0;
        }
    }
    d4* fb = fbar + (size_t)FB * f;
    st4(&fb[0], out);
    st4(&fb[1], out + 4);
    if (VISC == 1) {
        // reverse of face_gradient (solver.h:359-398), component by component:
        // fg = gbar - ((gbar . t) - (qa - qb)/lij) t, gbar the mean gradient
        double ga_x[4], ga_y[4], qa_b[4], gb_x[4], gb_y[4], qb_b[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double fx = out[8 + k], fy = out[12 + k];
            const double e = -(t.x * fx + t.y * fy);  // adjoint of grad_dot - grad_dir
            const double mx = fx + e * t.x, my = fy + e * t.y;
            ga_x[k] = gb_x[k] = 0.5 * mx;
            ga_y[k] = gb_y[k] = 0.5 * my;
            qa_b[k] = -e / t.z;
            qb_b[k] = e / t.z;
        }
        st4(&fb[2], ga_x);
        st4(&fb[3], ga_y);
        st4(&fb[4], qa_b);
        st4(&fb[5], gb_x);
        st4(&fb[6], gb_y);
        st4(&fb[7], qb_b);
    }
}

template <bool SECOND, int VISC>
__global__ void __launch_bounds__(128) k_adj_cell(const KM<double> m, const d4* __restrict__ q,
                                                  const d4* __restrict__ gx, const d4* __restrict__ gy,
                                                  const d4* __restrict__ phi, const d4* __restrict__ fbar,
                                                  d4* __restrict__ qbar, d4* __restrict__ gbx, d4* __restrict__ gby,
                                                  d4* __restrict__ lw, int4* __restrict__ lt) {
    constexpr int FB = VISC == 1 ? 8 : 2;
    constexpr bool GRAD = SECOND || VISC == 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_cells) return;
    const int4 sl = __ldg(&m.cslot[i]);
    const int4 nb = __ldg(&m.cnbr[i]);
    double qb[4] = {0, 0, 0, 0}, pb[4] = {0, 0, 0, 0}, bx[4] = {0, 0, 0, 0}, by[4] = {0, 0, 0, 0};
    double qi[4], gxi[4], gyi[4], ph[4];
    if (SECOND) {
        ld4(&q[i], qi);
        ld4(&gx[i], gxi);
        ld4(&gy[i], gyi);
        ld4(&phi[i], ph);
    }
    double dxs[4] = {0, 0, 0, 0}, dys[4] = {0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(sl, s);
        if (fs == 0) continue;
        const bool own0 = fs > 0;
        const int f = (own0 ? fs : -fs) - 1;
        double side[4];
        const d4* fb = fbar + (size_t)FB * f;
        ld4(&fb[own0 ? 0 : 1], side);
#pragma unroll
        for (int k = 0; k < 4; ++k) qb[k] += side[k];
        if (VISC == 1) {
            // the face gradient's use of this cell's member state and gradient
            double sgx[4], sgy[4], sq[4];
            ld4(&fb[own0 ? 2 : 5], sgx);
            ld4(&fb[own0 ? 3 : 6], sgy);
            ld4(&fb[own0 ? 4 : 7], sq);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                qb[k] += sq[k];
                bx[k] += sgx[k];
                by[k] += sgy[k];
            }
        }
        if (SECOND) {
            const double2 d = own0 ? __ldg(&m.fd0[f]) : __ldg(&m.fd1[f]);
            dxs[s] = d.x;
            dys[s] = d.y;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                pb[k] += side[k] * (gxi[k] * d.x + gyi[k] * d.y);
                bx[k] += side[k] * ph[k] * d.x;
                by[k] += side[k] * ph[k] * d.y;
            }
        }
    }
    if (SECOND) {
        // neighbour max/min with the cell that attains them (smax/smin order)
        double qmx[4], qmn[4];
        int tmx[4], tmn[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            qmx[k] = qmn[k] = qi[k];
            tmx[k] = tmn[k] = ADJ_NONE;
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            if (pick(sl, s) == 0) continue;
            const int o = pick(nb, s);
            double qo[4];
            bool use = true;
            if (o >= 0) {
                ld4(&q[o], qo);
            } else {
                const int bt = __ldg(&m.btype[-o - 1]);
                use = bt != BT_SLIP && bt != BT_WALL;
                ld4(&m.bq[-o - 1], qo);
            }
            if (!use) continue;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (qmx[k] < qo[k]) {
                    qmx[k] = qo[k];
                    tmx[k] = o;
                }
                if (qo[k] < qmn[k]) {
                    qmn[k] = qo[k];
                    tmn[k] = o;
                }
            }
        }
        const double A = __ldg(&m.area[i]);
        const double Ka = m.limk * sqrt(A);
        const double K3a = Ka * Ka * Ka;
        double wmx[4] = {0, 0, 0, 0}, wmn[4] = {0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double lim = 1.0;
            int sa = -1;
            for (int s = 0; s < 4; ++s) {
                if (pick(sl, s) == 0) continue;
                const double dqg = gxi[k] * dxs[s] + gyi[k] * dys[s];
                const double lv = limiter_value(m.limiter, dqg, qmx[k] - qi[k], qmn[k] - qi[k], K3a);
                if (lv < lim) {
                    lim = lv;
                    sa = s;
                }
            }
            if (sa < 0 || pb[k] == 0.0) continue;
            const double dx = sa == 0 ? dxs[0] : sa == 1 ? dxs[1] : sa == 2 ? dxs[2] : dxs[3];
            const double dy = sa == 0 ? dys[0] : sa == 1 ? dys[1] : sa == 2 ? dys[2] : dys[3];
            const double dqg = gxi[k] * dx + gyi[k] * dy;
            double dl[3];
#pragma unroll 1
            for (int dir = 0; dir < 3; ++dir) {
                const Dual r = limiter_value<Dual>(m.limiter, Dual(dqg, dir == 0 ? 1.0 : 0.0),
                                                   Dual(qmx[k] - qi[k], dir == 1 ? 1.0 : 0.0),
                                                   Dual(qmn[k] - qi[k], dir == 2 ? 1.0 : 0.0), Dual(K3a));
                dl[dir] = r.d;
            }
            bx[k] += pb[k] * dl[0] * dx;
            by[k] += pb[k] * dl[0] * dy;
            // delta_max = qmax - q_i, delta_min = qmin - q_i
            if (tmx[k] != ADJ_NONE) {
                wmx[k] = pb[k] * dl[1];
                qb[k] -= wmx[k];
            }
            if (tmn[k] != ADJ_NONE) {
                wmn[k] = pb[k] * dl[2];
                qb[k] -= wmn[k];
            }
        }
        st4(&lw[2 * (size_t)i], wmx);
        st4(&lw[2 * (size_t)i + 1], wmn);
        lt[2 * (size_t)i] = make_int4(tmx[0], tmx[1], tmx[2], tmx[3]);
        lt[2 * (size_t)i + 1] = make_int4(tmn[0], tmn[1], tmn[2], tmn[3]);
    }
    if (GRAD) {
        st4(&gbx[i], bx);
        st4(&gby[i], by);
    }
    st4(&qbar[i], qb);
}

template <bool SECOND, int VISC>
__global__ void __launch_bounds__(128) k_adj_final(const KM<double> m, const d4* __restrict__ q,
                                                   const d4* __restrict__ fbar, const d4* __restrict__ qbar,
                                                   const d4* __restrict__ gbx, const d4* __restrict__ gby,
                                                   const d4* __restrict__ lw, const int4* __restrict__ lt,
                                                   d4* __restrict__ u, d4* __restrict__ bqbar) {
    constexpr int FB = VISC == 1 ? 8 : 2;
    constexpr bool GRAD = SECOND || VISC == 1;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m.n_cells) return;
    const int4 sl = __ldg(&m.cslot[j]);
    const int4 nb = __ldg(&m.cnbr[j]);
    double uj[4];
    ld4(&qbar[j], uj);
    double bxj[4], byj[4], qj[4];
    const double Aj = __ldg(&m.area[j]);
    if (GRAD) {
        ld4(&gbx[j], bxj);
        ld4(&gby[j], byj);
        ld4(&q[j], qj);
    }
#pragma unroll 1
    for (int s = 0; s < 4; ++s) {
        const int fs = pick(sl, s);
        if (fs == 0) continue;
        const bool own0 = fs > 0;
        const int f = (own0 ? fs : -fs) - 1;
        const int o = pick(nb, s);
        const double2 n = __ldg(&m.fn[f]);
        const double2 Lg = __ldg(&m.fLg[f]);
        if (o >= 0) {
            if (!GRAD) continue;
            if (SECOND) {
                // limiter terms of the neighbour that point at this cell
                double wx[4], wn[4];
                ld4(&lw[2 * (size_t)o], wx);
                ld4(&lw[2 * (size_t)o + 1], wn);
                const int4 tx = __ldg(&lt[2 * (size_t)o]);
                const int4 tn = __ldg(&lt[2 * (size_t)o + 1]);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (pick4(tx, k) == j) uj[k] += wx[k];
                    if (pick4(tn, k) == j) uj[k] += wn[k];
                }
            }
            // Green-Gauss face value (q_c0 (1-g) + (q_c0 + q_c1)/2 g) L, added
            // to cell 0's sum and subtracted from cell 1's
            double bxo[4], byo[4];
            ld4(&gbx[o], bxo);
            ld4(&gby[o], byo);
            const double Ao = __ldg(&m.area[o]);
            const double g = Lg.y;
            const double wself = own0 ? ((1.0 - g) + 0.5 * g) : 0.5 * g;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double s0x = own0 ? bxj[k] / Aj : bxo[k] / Ao, s1x = own0 ? bxo[k] / Ao : bxj[k] / Aj;
                const double s0y = own0 ? byj[k] / Aj : byo[k] / Ao, s1y = own0 ? byo[k] / Ao : byj[k] / Aj;
                const double fb = n.x * (s0x - s1x) + n.y * (s0y - s1y);
                uj[k] += fb * wself * Lg.x;
            }
        } else {
            // boundary face b of this cell (always its cell 0)
            const int b = -o - 1;
            double bb[4];
            ld4(&fbar[(size_t)FB * f + 1], bb);
            if (VISC == 1) {
                // a two-sided boundary's face gradient reads the boundary state
                double qbb[4];
                ld4(&fbar[(size_t)FB * f + 7], qbb);
#pragma unroll
                for (int k = 0; k < 4; ++k) bb[k] += qbb[k];
            }
            if (SECOND) {
                double wx[4], wn[4];
                ld4(&lw[2 * (size_t)j], wx);
                ld4(&lw[2 * (size_t)j + 1], wn);
                const int4 tx = __ldg(&lt[2 * (size_t)j]);
                const int4 tn = __ldg(&lt[2 * (size_t)j + 1]);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (pick4(tx, k) == o) bb[k] += wx[k];
                    if (pick4(tn, k) == o) bb[k] += wn[k];
                }
            }
            if (GRAD) {
                // face value (q_j (1-g) + ghost(q_j, bq) g) L
                const int bt = __ldg(&m.btype[b]);
                double qbc[4], fb[4];
                ld4(&m.bq[b], qbc);
                const double g = Lg.y;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    fb[k] = (n.x * bxj[k] + n.y * byj[k]) / Aj * Lg.x;
                    uj[k] += fb[k] * (1.0 - g);
                }
#pragma unroll 1
                for (int dir = 0; dir < 8; ++dir) {
                    const double t = g * ghost_dir(bt, m.gamma, n.x, n.y, qj, qbc, dir, fb);
                    if (dir < 4) uj[dir] += t;
                    else bb[dir - 4] += t;
                }
            }
            st4(&bqbar[b], bb);
        }
    }
    st4(&u[j], uj);
}

// One adjoint pseudo-time stage: lam_k = lam_0 + alpha*relax*dt*(u + g), with
// ||u + g||^2 block partials on the last stage.
__global__ void __launch_bounds__(256) k_adj_update(const int n, const d4* __restrict__ lam0,
                                                    const d4* __restrict__ u, const d4* __restrict__ g,
                                                    const double* __restrict__ dt, const double alpha,
                                                    const double relax, d4* __restrict__ lam_out,
                                                    double* __restrict__ partials) {
    __shared__ double sh[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0;
    if (i < n) {
        double l0[4], ui[4], gi[4], out[4];
        ld4(&lam0[i], l0);
        ld4(&u[i], ui);
        ld4(&g[i], gi);
        const double d = __ldg(&dt[i]);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double r = ui[k] + gi[k];
            out[k] = l0[k] + r * d * alpha * relax;
            sq += r * r;
        }
        st4(&lam_out[i], out);
    }
    if (partials) {
        const double t = block_sum(sq, sh);
        if (threadIdx.x == 0) partials[blockIdx.x] = t;
    }
}

// dJ/dq of a force coefficient J = cx*fx + cy*fy over the patch edges
// (post.h:341-384): cp = 2/(gamma M^2) (p/p_inf - 1) of each edge's cell.
// One thread walks the edges in order, so a cell with two patch edges sums
// them in a fixed order.
__global__ void k_objective_grad(const ForceArgs f, const double cx, const double cy, d4* __restrict__ g) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const d4* q = (const d4*)f.q;
    const double dx = f.xmax - f.xmin;
    const double c = 2. / (f.gamma * f.mach_inf * f.mach_inf) / f.p_inf;
    for (int e = 0; e < f.n; ++e) {
        double qc[4];
        ld4(&q[f.cell[e]], qc);
        const double* ge = f.geo + 5 * e;
        const double u = qc[1] / qc[0], v = qc[2] / qc[0];
        const double s = c * (cx * ge[2] + cy * ge[3]) * ge[4] / dx * (f.gamma - 1);
        d4& o = g[f.cell[e]];
        o.x += s * 0.5 * (u * u + v * v);
        o.y -= s * u;
        o.z -= s * v;
        o.w += s;
    }
}

}  // namespace dev

void enqueue_adjoint_prep(const StepArgs& a0, int p, bool with_dt, cudaStream_t s) {
    StepArgs a = a0;
    a.variant = with_dt ? 0 : 1;  // variant 0's prep also forms the local time step
    const dev::KM<double> m = dev::make_km<double>(a);
    dev::launch_prep<double, double>(a, m, (const dev::d4*)a.qm[p], s);
}

namespace {
template <bool SECOND, int VISC>
void vjp_launch(const StepArgs& a, int p, const AdjArgs& j, cudaStream_t s) {
    using namespace dev;
    const KM<double> m = make_km<double>(a);
    const d4* q = (const d4*)a.qm[p];
    const d4* gx = (const d4*)a.gx;
    const d4* gy = (const d4*)a.gy;
    const d4* ph = (const d4*)a.phi;
    const int B = 128;
    const int nf = nblocks(a.n_faces, B), nc = nblocks(a.n_cells, B);
    // input directions per pass of the face kernel (vector duals)
    if (j.dirs_per_pass == 1)
        k_adj_face<SECOND, VISC, 1><<<nf, B, 0, s>>>(m, a.n_faces, q, gx, gy, ph, (const d4*)j.v, (d4*)j.fbar);
    else if (j.dirs_per_pass == 2)
        k_adj_face<SECOND, VISC, 2><<<nf, B, 0, s>>>(m, a.n_faces, q, gx, gy, ph, (const d4*)j.v, (d4*)j.fbar);
    else
        k_adj_face<SECOND, VISC, 4><<<nf, B, 0, s>>>(m, a.n_faces, q, gx, gy, ph, (const d4*)j.v, (d4*)j.fbar);
    k_adj_cell<SECOND, VISC><<<nc, B, 0, s>>>(m, q, gx, gy, ph, (const d4*)j.fbar, (d4*)j.qbar, (d4*)j.gbx,
                                              (d4*)j.gby, (d4*)j.lw, (int4*)j.lt);
    k_adj_final<SECOND, VISC><<<nc, B, 0, s>>>(m, q, (const d4*)j.fbar, (const d4*)j.qbar, (const d4*)j.gbx,
                                               (const d4*)j.gby, (const d4*)j.lw, (const int4*)j.lt, (d4*)j.u,
                                               (d4*)j.bqbar);
}
}  // namespace

void enqueue_vjp(const StepArgs& a, int p, const AdjArgs& j, cudaStream_t s) {
    if (a.visc == 1) {
        if (a.second) vjp_launch<true, 1>(a, p, j, s);
        else vjp_launch<false, 1>(a, p, j, s);
    } else {
        if (a.second) vjp_launch<true, 0>(a, p, j, s);
        else vjp_launch<false, 0>(a, p, j, s);
    }
}

void enqueue_adjoint_update(int n, const void* lam0, const void* u, const void* g, const void* dt, double alpha,
                            double relax, void* lam_out, double* partials, cudaStream_t s) {
    dev::k_adj_update<<<(n + 255) / 256, 256, 0, s>>>(n, (const dev::d4*)lam0, (const dev::d4*)u,
                                                        (const dev::d4*)g, (const double*)dt, alpha, relax,
                                                        (dev::d4*)lam_out, partials);
}

void enqueue_objective_grad(const ForceArgs& f, double cx, double cy, void* g, cudaStream_t s) {
    dev::k_objective_grad<<<1, 1, 0, s>>>(f, cx, cy, (dev::d4*)g);
}

}  // namespace afx
