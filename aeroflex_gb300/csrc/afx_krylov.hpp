// Flexible GMRES over FP64 device vectors (afx_krylov.cu).
#pragma once

#include <cuda_runtime.h>

#include <functional>

namespace afx {
namespace dev {
constexpr int KV_MAX = 32;  // basis vectors one orthogonalisation pass reads
}
constexpr int KRYLOV_MAX_RESTART = 120;  // Arnoldi steps per restart cycle, at most

// out = op(in), both device vectors of the space's length, on the space's stream
using KrylovOp = std::function<void(const double* in, double* out)>;

// Device work space of one solve: the Arnoldi basis V (m+1 vectors), the
// preconditioned vectors Z (m), a work vector, the residual and the
// reduction partials.
struct KrylovSpace {
    long long n = 0;
    int m = 0;
    double *V = nullptr, *Z = nullptr, *w = nullptr, *r = nullptr, *part = nullptr, *hdev = nullptr;
    KrylovSpace(long long n, int m);
    ~KrylovSpace();
    KrylovSpace(const KrylovSpace&) = delete;
    KrylovSpace& operator=(const KrylovSpace&) = delete;
};

struct FgmresResult {
    int iters = 0;     // operator applications in Arnoldi steps
    int restarts = 0;  // cycles (each ends with one more operator application)
    double b_norm = 0, res = 0;  // ||b||, the final true residual ||b - A x||
};

double kv_dot(const KrylovSpace& ks, const double* x, const double* y, cudaStream_t s);
// out = a x + b y (y may be null: out = a x)
void kv_axpby(const KrylovSpace& ks, double a, const double* x, double b, const double* y, double* out,
              cudaStream_t s);

// out = x .* y
void kv_mul(const KrylovSpace& ks, const double* x, const double* y, double* out, cudaStream_t s);

// Solves A x = b to ||b - A x|| <= rtol ||b|| or max_it Arnoldi steps, x
// starting from its content (x_zero: from 0, x is overwritten).
FgmresResult fgmres(KrylovSpace& ks, const double* b, double* x, bool x_zero, double rtol, int max_it,
                    const KrylovOp& A, const KrylovOp& P, cudaStream_t s);

}  // namespace afx
