// FP64 path.  Compiled with -fmad=false: every product and sum is rounded on
// its own as in the reference's C++ (built without FMA contraction), which
// is what makes the FP64 residuals bit-identical to the reference's
// definition.  Also holds the precision-neutral helpers (state permutation,
// forces).
#include "afx_kernels_impl.cuh"

namespace afx {

void enqueue_iteration_f64(const StepArgs& a, int p, cudaStream_t s) { dev::iteration<double, double, false>(a, p, s); }
void enqueue_residual_f64(const StepArgs& a, int p, cudaStream_t s) { dev::residual<double, double>(a, p, s); }
void enqueue_rhs_f64(const StepArgs& a, int p, cudaStream_t s) { dev::rhs<double, double>(a, p, s); }
void enqueue_case_nonfinite(const StepArgs& a, void* b, cudaStream_t s) {
    dev::k_case_nonfinite<<<a.n_cases, 1024, 0, s>>>(a.cell_sq, a.case_off, a.cctrl, a.case_done, a.ctrl,
                                                    (dev::d4*)b);
}
void enqueue_case_control(const StepArgs& a, cudaStream_t s) {
    dev::k_case_control<<<a.n_cases, 1024, 0, s>>>(a.cell_sq, a.case_off, a.cctrl, a.case_done, a.chist, a.ctrl,
                                                  a.n_cases, 0);
    dev::k_batch_finalize<<<1, 1, 0, s>>>(a.ctrl, a.n_cases);
}
void enqueue_last_stage_residual_f64(const StepArgs& a, int p, cudaStream_t s) {
    dev::last_stage_residual<double, double>(a, p, s);
}
void enqueue_uniform_f64(const StepArgs& a, int p, const double* qf, cudaStream_t s) {
    dev::uniform<double, double>(a, p, qf, s);
}

namespace dev {

// Reference-order AoS <-> device-order cell vectors.
__global__ void k_permute_in(int n, const int* __restrict__ cell_old, const d4* __restrict__ src, d4* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ld4(&src[cell_old[i]], v);
    st4(&dst[i], v);
}
__global__ void k_permute_out(int n, const int* __restrict__ cell_old, const d4* __restrict__ src, d4* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ld4(&src[i], v);
    st4(&dst[cell_old[i]], v);
}
__global__ void k_to_f32(int n, const d4* __restrict__ src, float4* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ld4(&src[i], v);
    st4(&dst[i], v);
}

// get_wall_profile force integration (post.h:341-375) with a fixed-order
// block reduction of (fx, fy, moment).
__global__ void k_forces(const ForceArgs f) {
    __shared__ double sh[3][32];
    double fx = 0, fy = 0, mm = 0;
    const double dx = f.xmax - f.xmin;
    const d4* q = (const d4*)f.q;
    for (int e = threadIdx.x; e < f.n; e += blockDim.x) {
        double qc[4];
        ld4(&q[f.cell[e]], qc);
        const double* g = f.geo + 5 * e;
        const double p = (f.gamma - 1) * (qc[3] - 0.5 / qc[0] * (qc[1] * qc[1] + qc[2] * qc[2]));
        const double cp = 2. / (f.gamma * f.mach_inf * f.mach_inf) * (p / f.p_inf - 1.);
        f.cp[e] = cp;
        const double fxi = cp * g[2] * g[4] / dx;
        const double fyi = cp * g[3] * g[4] / dx;
        const double mi = (g[0] - f.x_moment) / dx * fyi - (g[1] - f.y_moment) / dx * fxi;
        fx += fxi;
        fy += fyi;
        mm -= mi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_down_sync(0xffffffffu, fx, o);
        fy += __shfl_down_sync(0xffffffffu, fy, o);
        mm += __shfl_down_sync(0xffffffffu, mm, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][w] = fx;
        sh[1][w] = fy;
        sh[2][w] = mm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a += sh[0][k];
            b += sh[1][k];
            c += sh[2][k];
        }
        f.sums[0] = a;
        f.sums[1] = b;
        f.sums[2] = c;
    }
}

__global__ void k_permute_in1(int n, const int* __restrict__ cell_old, const double* __restrict__ src,
                              double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[cell_old[i]];
}
__global__ void k_permute_out1(int n, const int* __restrict__ cell_old, const double* __restrict__ src,
                               double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[cell_old[i]] = src[i];
}

}  // namespace dev

void enqueue_permute_in1(int n, const int* cell_old, const void* src, void* dst, cudaStream_t s) {
    dev::k_permute_in1<<<(n + 255) / 256, 256, 0, s>>>(n, cell_old, (const double*)src, (double*)dst);
}
void enqueue_permute_out1(int n, const int* cell_old, const void* src, void* dst, cudaStream_t s) {
    dev::k_permute_out1<<<(n + 255) / 256, 256, 0, s>>>(n, cell_old, (const double*)src, (double*)dst);
}

void enqueue_permute_in(int n, const int* cell_old, const void* src, void* dst, cudaStream_t s) {
    dev::k_permute_in<<<(n + 255) / 256, 256, 0, s>>>(n, cell_old, (const dev::d4*)src, (dev::d4*)dst);
}
void enqueue_permute_out(int n, const int* cell_old, const void* src, void* dst, cudaStream_t s) {
    dev::k_permute_out<<<(n + 255) / 256, 256, 0, s>>>(n, cell_old, (const dev::d4*)src, (dev::d4*)dst);
}
void enqueue_to_f32(int n, const void* src, void* dst, cudaStream_t s) {
    dev::k_to_f32<<<(n + 255) / 256, 256, 0, s>>>(n, (const dev::d4*)src, (float4*)dst);
}
void enqueue_forces(const ForceArgs& f, cudaStream_t s) { dev::k_forces<<<1, 256, 0, s>>>(f); }

void enqueue_sa_implicit_f64(const StepArgs& a, int p, int sweeps, cudaStream_t s) {
    dev::sa_implicit<double, double>(a, p, sweeps, s);
}
void enqueue_sa_mut_f64(const StepArgs& a, int p, cudaStream_t s) {
    dev::sa_mut<double, double>(a, (const dev::V4<double>*)a.qsh[p], a.sa_nu[p], s);
}

}  // namespace afx
