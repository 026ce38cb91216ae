// Flexible GMRES (right preconditioned, restarted) over FP64 device vectors,
// driven from the host: the operator and the preconditioner are callbacks,
// so the same driver serves the Newton-Krylov finish of the implicit solver
// (operator: a finite-difference Jacobian-vector product of the implicit
// right-hand side; preconditioner: a GMRES solve with the implicit matrix)
// and the adjoint solve (operator: the exact transposed Jacobian, the vJP
// kernel; preconditioner: a GMRES solve with the transposed matrix).  The
// preconditioner changes from call to call (an inner Krylov solve to a
// loose tolerance), hence the flexible form: the preconditioned vectors Z
// are kept beside the Arnoldi basis V.
//
// Orthogonalisation: classical Gram-Schmidt applied twice (CGS2), each pass
// one kernel reading the basis once.  Every reduction is a fixed-order
// two-level sum (block partials in a fixed grid, summed on the host in
// order), so a solve is deterministic on a given GPU.
#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>

#include "afx_host.hpp"
#include "afx_krylov.hpp"
#include "afx_rans.h"

namespace afx {
namespace dev {

constexpr int KV_T = 256;     // threads per block
constexpr int KV_BLOCKS = 304;  // fixed grid of the reductions (2 per SM)

// part[i * gridDim.x + block] = this block's share of V_i . w, i < k
__global__ void __launch_bounds__(KV_T) k_kv_vtw(const long long n, const int k, const double* __restrict__ V,
                                                 const double* __restrict__ w, double* __restrict__ part) {
    double acc[KV_MAX];
#pragma unroll
    for (int i = 0; i < KV_MAX; ++i) acc[i] = 0.0;
    for (long long j = (long long)blockIdx.x * KV_T + threadIdx.x; j < n; j += (long long)gridDim.x * KV_T) {
        const double wj = w[j];
#pragma unroll
        for (int i = 0; i < KV_MAX; ++i)
            if (i < k) acc[i] += V[(size_t)i * n + j] * wj;
    }
    __shared__ double red[KV_T / 32][KV_MAX];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < KV_MAX; ++i) {
        if (i >= k) break;
        double v = acc[i];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wp][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < k) {
        double t = 0.0;
        for (int q = 0; q < KV_T / 32; ++q) t += red[q][threadIdx.x];
        part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
    }
}

// w -= sum_i h[i] V_i, i < k
__global__ void __launch_bounds__(KV_T) k_kv_sub(const long long n, const int k, const double* __restrict__ V,
                                                 const double* __restrict__ h, double* __restrict__ w) {
    for (long long j = (long long)blockIdx.x * KV_T + threadIdx.x; j < n; j += (long long)gridDim.x * KV_T) {
        double t = w[j];
        for (int i = 0; i < k; ++i) t -= h[i] * V[(size_t)i * n + j];
        w[j] = t;
    }
}

// out = x .* y (out may alias either)
__global__ void __launch_bounds__(KV_T) k_kv_mul(const long long n, const double* x, const double* y, double* out) {
    for (long long j = (long long)blockIdx.x * KV_T + threadIdx.x; j < n; j += (long long)gridDim.x * KV_T)
        out[j] = x[j] * y[j];
}

// out = a x + b y (out may alias y)
__global__ void __launch_bounds__(KV_T) k_kv_axpby(const long long n, const double a, const double* __restrict__ x,
                                                   const double b, const double* y, double* out) {
    for (long long j = (long long)blockIdx.x * KV_T + threadIdx.x; j < n; j += (long long)gridDim.x * KV_T)
        out[j] = y ? a * x[j] + b * y[j] : a * x[j];
}

}  // namespace dev

namespace {

void kchk(cudaError_t r, const char* what) {
    if (r != cudaSuccess) throw Error(AFX_ERR_CUDA, std::string("krylov: ") + what + ": " + cudaGetErrorString(r));
}

}  // namespace

KrylovSpace::KrylovSpace(long long n_, int m_) : n(n_), m(std::max(1, std::min(m_, KRYLOV_MAX_RESTART))) {
    kchk(cudaMalloc(&V, (size_t)(m + 1) * n * 8), "basis");
    kchk(cudaMalloc(&Z, (size_t)m * n * 8), "preconditioned basis");
    kchk(cudaMalloc(&w, (size_t)n * 8), "work vector");
    kchk(cudaMalloc(&r, (size_t)n * 8), "residual");
    kchk(cudaMalloc(&part, (size_t)dev::KV_MAX * dev::KV_BLOCKS * 8), "partials");
    kchk(cudaMalloc(&hdev, (size_t)(m + 1) * 8), "coefficients");
}

KrylovSpace::~KrylovSpace() {
    for (void* p : {(void*)V, (void*)Z, (void*)w, (void*)r, (void*)part, (void*)hdev})
        if (p) cudaFree(p);
}

// h[i] = V_i . w for i < k (V: k contiguous vectors of length n), in
// chunks of KV_MAX vectors per pass
static void vtw(const KrylovSpace& ks, int k, const double* V, const double* w, double* h, cudaStream_t s) {
    for (int i0 = 0; i0 < k; i0 += dev::KV_MAX) {
        const int kc = std::min(dev::KV_MAX, k - i0);
        dev::k_kv_vtw<<<dev::KV_BLOCKS, dev::KV_T, 0, s>>>(ks.n, kc, V + (size_t)i0 * ks.n, w, ks.part);
        std::vector<double> p((size_t)kc * dev::KV_BLOCKS);
        kchk(cudaMemcpyAsync(p.data(), ks.part, p.size() * 8, cudaMemcpyDeviceToHost, s), "partials");
        kchk(cudaStreamSynchronize(s), "dot");
        for (int i = 0; i < kc; ++i) {
            double t = 0.0;
            for (int b = 0; b < dev::KV_BLOCKS; ++b) t += p[(size_t)i * dev::KV_BLOCKS + b];
            h[i0 + i] = t;
        }
    }
}

double kv_dot(const KrylovSpace& ks, const double* x, const double* y, cudaStream_t s) {
    double h = 0;
    vtw(ks, 1, x, y, &h, s);
    return h;
}

void kv_axpby(const KrylovSpace& ks, double a, const double* x, double b, const double* y, double* out,
              cudaStream_t s) {
    dev::k_kv_axpby<<<dev::KV_BLOCKS, dev::KV_T, 0, s>>>(ks.n, a, x, b, y, out);
}

void kv_mul(const KrylovSpace& ks, const double* x, const double* y, double* out, cudaStream_t s) {
    dev::k_kv_mul<<<dev::KV_BLOCKS, dev::KV_T, 0, s>>>(ks.n, x, y, out);
}

// w -= sum_i h[i] V_i
static void vsub(const KrylovSpace& ks, int k, const double* V, const double* h, double* w, cudaStream_t s) {
    kchk(cudaMemcpyAsync(ks.hdev, h, (size_t)k * 8, cudaMemcpyHostToDevice, s), "coefficients");
    dev::k_kv_sub<<<dev::KV_BLOCKS, dev::KV_T, 0, s>>>(ks.n, k, V, ks.hdev, w);
    kchk(cudaStreamSynchronize(s), "update");  // h is a host temporary
}

FgmresResult fgmres(KrylovSpace& ks, const double* b, double* x, bool x_zero, double rtol, int max_it,
                    const KrylovOp& A, const KrylovOp& P, cudaStream_t s) {
    const long long n = ks.n;
    const int m = ks.m;
    FgmresResult out;
    out.b_norm = std::sqrt(kv_dot(ks, b, b, s));
    if (x_zero) {
        kchk(cudaMemsetAsync(x, 0, (size_t)n * 8, s), "solution");
        kchk(cudaMemcpyAsync(ks.r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, s), "residual");
    } else {
        A(x, ks.w);
        kv_axpby(ks, 1.0, b, -1.0, ks.w, ks.r, s);
    }
    double beta = std::sqrt(kv_dot(ks, ks.r, ks.r, s));
    const double target = rtol * out.b_norm;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), h(m + 1), h2(m + 1), y(m);
    while (beta > target && out.iters < max_it) {
        if (!(beta == beta)) throw Error(AFX_ERR_NONFINITE, "krylov: residual is not finite");
        kv_axpby(ks, 1.0 / beta, ks.r, 0.0, nullptr, ks.V, s);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j_end = 0;
        for (int j = 0; j < m; ++j) {
            double* vj = ks.V + (size_t)j * n;
            double* zj = ks.Z + (size_t)j * n;
            P(vj, zj);
            A(zj, ks.w);
            // CGS2 against v_0 .. v_j
            vtw(ks, j + 1, ks.V, ks.w, h.data(), s);
            vsub(ks, j + 1, ks.V, h.data(), ks.w, s);
            vtw(ks, j + 1, ks.V, ks.w, h2.data(), s);
            vsub(ks, j + 1, ks.V, h2.data(), ks.w, s);
            for (int i = 0; i <= j; ++i) h[i] += h2[i];
            const double hn = std::sqrt(kv_dot(ks, ks.w, ks.w, s));
            if (!(hn == hn)) throw Error(AFX_ERR_NONFINITE, "krylov: basis vector is not finite");
            // Givens rotations of column j
            for (int i = 0; i < j; ++i) {
                const double t = cs[i] * h[i] + sn[i] * h[i + 1];
                h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
                h[i] = t;
            }
            const double rr = std::sqrt(h[j] * h[j] + hn * hn);
            cs[j] = rr > 0 ? h[j] / rr : 1.0;
            sn[j] = rr > 0 ? hn / rr : 0.0;
            h[j] = rr;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = h[i];
            ++out.iters;
            j_end = j + 1;
            if (hn > 0) kv_axpby(ks, 1.0 / hn, ks.w, 0.0, nullptr, ks.V + (size_t)(j + 1) * n, s);
            if (std::fabs(g[j + 1]) <= target || out.iters >= max_it || hn == 0) break;
        }
        // H y = g (upper triangular), x += Z y
        for (int i = j_end - 1; i >= 0; --i) {
            double t = g[i];
            for (int k = i + 1; k < j_end; ++k) t -= H[(size_t)i * m + k] * y[k];
            y[i] = H[(size_t)i * m + i] != 0 ? t / H[(size_t)i * m + i] : 0.0;
        }
        for (int i = 0; i < j_end; ++i) y[i] = -y[i];
        vsub(ks, j_end, ks.Z, y.data(), x, s);  // x -= (-y) Z
        // the true residual of the restart
        A(x, ks.w);
        kv_axpby(ks, 1.0, b, -1.0, ks.w, ks.r, s);
        beta = std::sqrt(kv_dot(ks, ks.r, ks.r, s));
        ++out.restarts;
    }
    out.res = beta;
    return out;
}

}  // namespace afx
