// Residual evaluation that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: a structural or coupling
// code that owns all device memory through its own pool, sized at start-up (a
// library-side cudaMalloc/cudaFree would synchronise the whole device and break
// its stream overlap, and could fail once the pool holds the memory).  For
// them the face-flux form of the FP64 residual keeps its scratch — the state
// in device cell order and the face fluxes F*L — in the fixed device array
// below instead of allocating it.  The work runs on the solver's own stream;
// the entry point synchronises that stream before it returns.
//
// Limits: at most AFX_NOALLOC_MAX_CELLS real cells and AFX_NOALLOC_MAX_FACES
// faces (24 MiB of device memory in total).  Every GPU that loads the library
// holds the array until the process exits.  Every call shares it and it keeps
// the last call's contents; each call writes every byte it later reads, so
// nothing needs clearing.  Calls that overlap on the GPU (two streams, two
// threads, two solvers) race on the array and must be serialised by the
// caller.  On each device, the first call looks up the array's device address
// (cudaGetSymbolAddress) with that device current.
#include <mutex>

#include "afx_kernels_impl.cuh"

namespace afx {

constexpr long long NOALLOC_MAX_CELLS = 262144;
constexpr long long NOALLOC_MAX_FACES = 524288;

static __device__ __align__(256) unsigned char g_noalloc_scratch[(NOALLOC_MAX_CELLS + NOALLOC_MAX_FACES) * 32];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[MAX_DEVICES] = {nullptr};
}  // namespace

long long noalloc_max_cells() { return NOALLOC_MAX_CELLS; }
long long noalloc_max_faces() { return NOALLOC_MAX_FACES; }

namespace dev {
__global__ void k_gather_cells(int n, const int* __restrict__ cell_old, const d4* __restrict__ src,
                               d4* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ld4(&src[cell_old[i]], v);
    st4(&dst[i], v);
}
__global__ void k_scatter_cells(int n, const int* __restrict__ cell_old, const d4* __restrict__ src,
                                d4* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ld4(&src[i], v);
    st4(&dst[cell_old[i]], v);
}
}  // namespace dev

// Device address of the scratch array on the current device (looked up once
// per device).  Returns the CUDA error of the lookup.
static cudaError_t scratch_address(void** out) {
    int devn = 0;
    cudaError_t e = cudaGetDevice(&devn);
    if (e != cudaSuccess) return e;
    if (devn < 0 || devn >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[devn]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[devn] = p;
    }
    *out = g_scratch_ptr[devn];
    return cudaSuccess;
}

// R (reference cell order, device) of the state q (reference cell order,
// device) with the stage-0 semantics of afx_residual: gradients and limiter
// into the solver's own gradient/limiter buffers, face fluxes and the
// device-order state in the scratch array.  Sizes are checked by the caller.
cudaError_t noalloc_residual_f64(const StepArgs& a, const int* cell_old, const double* q_ref, double* R_ref,
                                 cudaStream_t s) {
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return e;
    unsigned char* p = static_cast<unsigned char*>(base);
    dev::d4* state = reinterpret_cast<dev::d4*>(p);                          // NOALLOC_MAX_CELLS x 32 B
    void* fflux = p + NOALLOC_MAX_CELLS * 32;                                // NOALLOC_MAX_FACES x 32 B
    const int n = a.n_cells;
    dev::k_gather_cells<<<(n + 255) / 256, 256, 0, s>>>(n, cell_old, (const dev::d4*)q_ref, state);
    StepArgs b = a;
    b.qm[0] = b.qsh[0] = state;
    b.variant = 1;       // face fluxes through the scratch array
    b.fflux = fflux;
    b.feL = nullptr;     // the time step is not formed by a residual-only launch
    b.Rq = state;        // the state is no longer read when the per-cell sums run
    b.prof = nullptr;
    dev::residual<double, double>(b, 0, s);
    dev::k_scatter_cells<<<(n + 255) / 256, 256, 0, s>>>(n, cell_old, state, (dev::d4*)R_ref);
    return cudaGetLastError();
}

}  // namespace afx
