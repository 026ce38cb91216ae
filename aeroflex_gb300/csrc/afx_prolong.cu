// Coarse-to-fine solution transfer of grid sequencing (multigrid::gen_mapper,
// multigrid.h:99-178, applied in multigrid::run, multigrid.h:295-363).
//
// For every fine cell i, the coarse cells j (real and ghost, reference order)
// with d2 = |x_i - x_j|^2 < 2 A_j contribute with weight
// s_ij = 1 / max(0.1 sqrt(A_j), sqrt(d2)), normalised by their sum:
//     q_i = sum_j (s_ij / sum_j s_ij) q_j,
// summed in increasing j, as the reference's column-major sparse product
// adds them.  The reference builds the O(m n) mapper on the host once; here
// each fine cell scans the coarse cells from shared-memory tiles, twice (the
// normaliser, then the weighted sum), with the reference's operations in the
// same order (compiled without FMA contraction).
#include "afx_kernels_impl.cuh"

namespace afx {
namespace dev {

constexpr int PT = 512;  // coarse cells per shared-memory tile

// cx, cy, ca: coarse centroids and areas, all cells (ghosts included);
// cq: coarse states (ghosts = their owner's state, bcs_from_internal)
// fx, fy: fine centroids of the fine device cells; out: fine state (device order)
__global__ void __launch_bounds__(256) k_prolong(const int nc, const double* __restrict__ cx,
                                                 const double* __restrict__ cy, const double* __restrict__ ca,
                                                 const d4* __restrict__ cq, const int nf,
                                                 const double* __restrict__ fx, const double* __restrict__ fy,
                                                 d4* __restrict__ out) {
    __shared__ double sx[PT], sy[PT], sa[PT];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < nf;
    const double xi = act ? fx[i] : 0.0, yi = act ? fy[i] : 0.0;
    double scale = 0;
    for (int t0 = 0; t0 < nc; t0 += PT) {
        const int tn = min(PT, nc - t0);
        __syncthreads();
        for (int t = threadIdx.x; t < tn; t += blockDim.x) {
            sx[t] = cx[t0 + t];
            sy[t] = cy[t0 + t];
            sa[t] = ca[t0 + t];
        }
        __syncthreads();
        if (act)
            for (int t = 0; t < tn; ++t) {
                const double d2 = (xi - sx[t]) * (xi - sx[t]) + (yi - sy[t]) * (yi - sy[t]);
                const double r2 = sa[t];
                if (d2 < 2 * r2) {
                    const double a = 0.1 * sqrt(r2), b = sqrt(d2);
                    scale += 1 / ((a < b) ? b : a);
                }
            }
    }
    double q[4] = {0, 0, 0, 0};
    for (int t0 = 0; t0 < nc; t0 += PT) {
        const int tn = min(PT, nc - t0);
        __syncthreads();
        for (int t = threadIdx.x; t < tn; t += blockDim.x) {
            sx[t] = cx[t0 + t];
            sy[t] = cy[t0 + t];
            sa[t] = ca[t0 + t];
        }
        __syncthreads();
        if (act)
            for (int t = 0; t < tn; ++t) {
                const double d2 = (xi - sx[t]) * (xi - sx[t]) + (yi - sy[t]) * (yi - sy[t]);
                const double r2 = sa[t];
                if (d2 < 2 * r2) {
                    const double a = 0.1 * sqrt(r2), b = sqrt(d2);
                    const double w = (1 / ((a < b) ? b : a)) / scale;
                    double qj[4];
                    ld4(&cq[t0 + t], qj);
#pragma unroll
                    for (int k = 0; k < 4; ++k) q[k] += w * qj[k];
                }
            }
    }
    if (act) st4(&out[i], q);
}

// coarse state in reference order with ghosts = owners (bcs_from_internal):
// full[cell_old[d]] = q[d] for the real cells, full[N + b] = full[owner(b)]
__global__ void k_full_state(const int n, const int nb, const int* __restrict__ cell_old,
                             const int* __restrict__ owner_ref, const d4* __restrict__ q, d4* __restrict__ full) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        double v[4];
        ld4(&q[t], v);
        st4(&full[cell_old[t]], v);
    }
}
__global__ void k_full_ghosts(const int n, const int nb, const int* __restrict__ owner_dev, const d4* __restrict__ q,
                              d4* __restrict__ full) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nb) {
        double v[4];
        ld4(&q[owner_dev[b]], v);
        st4(&full[n + b], v);
    }
}

// mesh::compute_wall_dist (mesh.h:794-830): for every cell, the least
// distance from its centroid to a wall / slip-wall edge centre, scanning the
// edges in boundary order (std::min), 1 if there is no wall.
__global__ void __launch_bounds__(256) k_wall_dist(const int nc, const double* __restrict__ cx,
                                                   const double* __restrict__ cy, const int nw,
                                                   const double* __restrict__ wx, const double* __restrict__ wy,
                                                   double* __restrict__ out) {
    __shared__ double sx[PT], sy[PT];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < nc;
    const double xi = act ? cx[i] : 0.0, yi = act ? cy[i] : 0.0;
    double mind = 1;
    bool first = true;
    for (int t0 = 0; t0 < nw; t0 += PT) {
        const int tn = min(PT, nw - t0);
        __syncthreads();
        for (int t = threadIdx.x; t < tn; t += blockDim.x) {
            sx[t] = wx[t0 + t];
            sy[t] = wy[t0 + t];
        }
        __syncthreads();
        if (act)
            for (int t = 0; t < tn; ++t) {
                const double dx = xi - sx[t], dy = yi - sy[t];
                const double d = sqrt(dx * dx + dy * dy);
                if (first) {
                    mind = d;
                    first = false;
                } else {
                    mind = (d < mind) ? d : mind;
                }
            }
    }
    if (act) out[i] = mind;
}

// Spalart-Allmaras wall distance: for every cell, the least distance from its
// centroid to a no-slip wall face (segment a-b, seg = ax, ay, bx, by per
// face), faces scanned in boundary order (std::min); 1e15 without a wall.
__global__ void __launch_bounds__(256) k_wall_seg_dist(const int nc, const double* __restrict__ cx,
                                                       const double* __restrict__ cy, const int nw,
                                                       const double* __restrict__ seg, double* __restrict__ out) {
    __shared__ double ss[4 * PT];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < nc;
    const double xi = act ? cx[i] : 0.0, yi = act ? cy[i] : 0.0;
    double mind = 1e15;
    bool first = true;
    for (int t0 = 0; t0 < nw; t0 += PT) {
        const int tn = min(PT, nw - t0);
        __syncthreads();
        for (int t = threadIdx.x; t < 4 * tn; t += blockDim.x) ss[t] = seg[4 * t0 + t];
        __syncthreads();
        if (act)
            for (int t = 0; t < tn; ++t) {
                const double ex = ss[4 * t + 2] - ss[4 * t], ey = ss[4 * t + 3] - ss[4 * t + 1];
                const double px = xi - ss[4 * t], py = yi - ss[4 * t + 1];
                double u = (px * ex + py * ey) / (ex * ex + ey * ey);
                u = u < 0.0 ? 0.0 : (u > 1.0 ? 1.0 : u);
                const double dx = px - u * ex, dy = py - u * ey;
                const double d = sqrt(dx * dx + dy * dy);
                if (first) {
                    mind = d;
                    first = false;
                } else {
                    mind = (d < mind) ? d : mind;
                }
            }
    }
    if (act) out[i] = mind;
}

}  // namespace dev

void enqueue_wall_seg_dist(int nc, const double* cx, const double* cy, int nw, const double* seg, double* out,
                           cudaStream_t s) {
    dev::k_wall_seg_dist<<<(nc + 255) / 256, 256, 0, s>>>(nc, cx, cy, nw, seg, out);
}

void enqueue_wall_dist(int nc, const double* cx, const double* cy, int nw, const double* wx, const double* wy,
                       double* out, cudaStream_t s) {
    dev::k_wall_dist<<<(nc + 255) / 256, 256, 0, s>>>(nc, cx, cy, nw, wx, wy, out);
}

void enqueue_prolong(int nc, const double* cx, const double* cy, const double* ca, const void* coarse_full, int nf,
                     const double* fx, const double* fy, void* fine_q, cudaStream_t s) {
    dev::k_prolong<<<(nf + 255) / 256, 256, 0, s>>>(nc, cx, cy, ca, (const dev::d4*)coarse_full, nf, fx, fy,
                                                     (dev::d4*)fine_q);
}

void enqueue_full_state(int n, int nb, const int* cell_old, const int* owner_dev, const void* q, void* full,
                        cudaStream_t s) {
    dev::k_full_state<<<(n + 255) / 256, 256, 0, s>>>(n, nb, cell_old, nullptr, (const dev::d4*)q, (dev::d4*)full);
    if (nb > 0)
        dev::k_full_ghosts<<<(nb + 255) / 256, 256, 0, s>>>(n, nb, owner_dev, (const dev::d4*)q, (dev::d4*)full);
}

}  // namespace afx
