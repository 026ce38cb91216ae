// Interface between the host orchestrator (afx_solver.cu) and the
// precision-specific kernel translation units (afx_kernels_f64.cu compiled
// without FMA contraction for bit parity, afx_kernels_f32.cu for the
// FP32-mixed path).  Plain pointers only.
#pragma once

#include <cuda_runtime.h>

namespace afx {

// Device-resident control block of an iteration run (one per solver).
struct Ctrl {
    int done;       // set when the run stopped (converged / max iterations / non-finite)
    int iter;       // iterations completed in this run
    int status;     // 0 ok, 4 non-finite
    int run_mode;   // 0: plain iterate (no stopping), 1: run_solver logic
    int max_it;
    int hist_n;
    int nparts;     // partial sums written by the last stage kernel
    int ndone;      // batch: cases that have stopped
    double err0;
    double err;     // last normalised residual (run_mode 1)
    double tol;
    double last_norm;  // ‖qW‖₂ of the last stage of the last iteration
};

constexpr int HIST_CAP = 1 << 16;

// Per-case run_solver state of a batch (one per case).
struct CaseCtrl {
    int done, iter, status, hist_n;
    double err0, err, last_norm;
};
constexpr int CASE_HIST_CAP = 4096;  // history entries kept per case (every 10th iteration)

// Eager-launch profiler: an event after every kernel of an iteration, so the
// host can time each kernel on the stream it runs on.
enum KernelId { K_PREP = 0, K_LIMITER, K_FACE_FLUX, K_CELL_SUM, K_RESID_GATHER, K_CONTROL, K_RESID_TILE, K_COUNT };
struct Prof {
    static constexpr int CAP = 64;
    cudaEvent_t ev[CAP + 1];
    int kid[CAP];
    int n = 0;
    void start(cudaStream_t s) {
        n = 0;
        cudaEventRecord(ev[0], s);
    }
    void mark(int id, cudaStream_t s) {
        if (n < CAP) {
            kid[n] = id;
            cudaEventRecord(ev[n + 1], s);
            ++n;
        }
    }
};

// Everything a launch needs.  Pointers to typed arrays are passed as void*
// and cast in the precision's translation unit (T = double or float).
struct StepArgs {
    int n_cells = 0, n_faces = 0, n_bnd = 0;
    // mesh, device layout (afx_host.hpp DeviceLayout), in T
    const void* cslot = nullptr;  // int4 [N] signed face slots
    const void* cnbr = nullptr;   // int4 [N] other cell per slot
    const void* area = nullptr;   // T [N]
    const void* fcell = nullptr;  // int2 [F]
    const void* fn = nullptr;     // T2 [F]
    const void* fLg = nullptr;    // T2 [F]
    const void* fd0 = nullptr;    // T2 [F]
    const void* fd1 = nullptr;    // T2 [F]
    const void* ft = nullptr;     // T4 [F]
    const void* btype = nullptr;  // int [B]
    const void* bq = nullptr;     // T4 [B] ghost (boundary) states
    // physics / scheme
    double gamma = 1.4, R = 0.71428571428, mu = 1e-5, kheat = 1e-5 / 0.72;
    double limiter_k = 5., cfl = 1., relax = 0.9;
    int visc = 0;         // 0 inviscid, 1 laminar (gradients passed to the flux)
    int second = 1;       // second-order reconstruction
    int need_grad = 1;    // gradients computed (second order or viscous model)
    int limiter = 0;      // 0 Venkatakrishnan, 1 Michalak
    // least-squares gradient (solver.h:402-422, 470-513) instead of Green-Gauss
    int lsq = 0;
    const void* lsqw = nullptr;  // T2 [4N]: (M d_j)^T of each local edge j of each cell
    const int* lsqs = nullptr;   // [N]: cslot slot of local edge j in bits 2j..2j+1, edge count in bits 8..
    // residual kernel: 0 gather (cell gather re-forming fluxes), 1 face (face
    // kernel + ordered cell sum through HBM), 2 tile (shared-memory face tile)
    int variant = 1;
    int block = 256;
    // tile variant data for `block` cells per tile (see TileView)
    const int* tile_hstart = nullptr;
    const int* tile_xptr = nullptr;
    const int* tile_xlist = nullptr;
    const void* tile_ctile = nullptr;  // short4 [N]
    int tile_maxnf = 0;
    // state
    void* qm[2] = {nullptr, nullptr};   // FP64 master state, ping-pong (d4 [N])
    void* qsh[2] = {nullptr, nullptr};  // state in T (== qm for FP64)
    void* qs[2] = {nullptr, nullptr};   // RK stage states in T
    void* gx = nullptr;
    void* gy = nullptr;
    void* phi = nullptr;
    void* dt = nullptr;
    void* Rq = nullptr;        // d4 [N]: qW mirror (real cells)
    void* fflux = nullptr;     // d4 or T4 [F]: F*L per face (face mode)
    void* feL = nullptr;       // T [F]: spectral radius * length per face (face mode)
    double* partials = nullptr;
    int n_partials = 0;
    Ctrl* ctrl = nullptr;
    double* hist = nullptr;    // [HIST_CAP] run_solver history (every 10th)
    double* norms = nullptr;   // optional per-iteration norms
    const void* corr = nullptr;  // float4 [N]: FP32-mixed defect correction (null: off)
    // batch of independent cases (n_cases == 0: a single case)
    int n_cases = 0;
    const int* case_of = nullptr;     // [N] case of each device cell
    const int* case_off = nullptr;    // [n_cases+1] device cell range of each case
    int* case_done = nullptr;         // [n_cases] 1 once a case has stopped
    double* cell_sq = nullptr;        // [N] squared last-stage residual of each cell
    CaseCtrl* cctrl = nullptr;        // [n_cases]
    double* chist = nullptr;          // [n_cases * CASE_HIST_CAP]
    const double* qfar_case = nullptr;  // [4 * n_cases] freestream state of each case
    // Spalart-Allmaras (visc == 2), device cell order
    void* sa_nu[2] = {nullptr, nullptr};   // nu~, FP64, ping-pong with the master state
    void* sa_nus[2] = {nullptr, nullptr};  // nu~ of the RK stages, FP64
    void* sa_mut = nullptr;                // T [N] eddy viscosity of the stage state
    void* sa_nuW = nullptr;                // FP64 [N] nu~ residual of the last evaluation
    const void* sa_wd = nullptr;           // T [N] wall distance
    const void* sa_cxy = nullptr;          // T2 [N] centroids
    const void* sa_gxy = nullptr;          // T2 [B] ghost-cell centroids
    double cp = 1., Pr_L = 0.72, Pr_T = 0.9;
    double sa_nu_far = 0.;                 // nu~ of the far field, 3 mu_L / rho_inf
    Prof* prof = nullptr;      // eager profiling only (never inside a graph)
};

// One explicit iteration reading parity p, writing parity p^1.
void enqueue_iteration_f64(const StepArgs& a, int p, cudaStream_t s);
void enqueue_iteration_f32(const StepArgs& a, int p, cudaStream_t s);
// Residual of state parity p with stage-0 semantics -> Rq (qW mirror).
void enqueue_residual_f64(const StepArgs& a, int p, cudaStream_t s);
void enqueue_residual_f32(const StepArgs& a, int p, cudaStream_t s);
// Implicit right-hand side (face sums, not divided by the area) of parity p
// -> Rq, with ||.||^2 block partials (nblocks(n_cells, block) of them).
void enqueue_rhs_f64(const StepArgs& a, int p, cudaStream_t s);
// Batch: per-case norms of cell_sq and run_solver control (k_case_control),
// then the run's iteration count and stop flag.
void enqueue_case_control(const StepArgs& a, cudaStream_t s);
// Implicit batch: cases with a non-finite right-hand side b stop and get zero rows.
void enqueue_case_nonfinite(const StepArgs& a, void* b, cudaStream_t s);
// Re-form qW of the last RK stage of the iteration that read parity p.
void enqueue_last_stage_residual_f64(const StepArgs& a, int p, cudaStream_t s);
void enqueue_last_stage_residual_f32(const StepArgs& a, int p, cudaStream_t s);
// get_uniform_residual: qW += freestream face fluxes, ‖qW‖₂ -> ctrl->err0.
void enqueue_uniform_f64(const StepArgs& a, int p, const double* qfar, cudaStream_t s);
void enqueue_uniform_f32(const StepArgs& a, int p, const double* qfar, cudaStream_t s);

// Spalart-Allmaras: `sweeps` point-implicit nu~ updates of the implicit
// solver at the state of parity p (then mu_t), and mu_t alone.
void enqueue_sa_implicit_f64(const StepArgs& a, int p, int sweeps, cudaStream_t s);
void enqueue_sa_implicit_f32(const StepArgs& a, int p, int sweeps, cudaStream_t s);
void enqueue_sa_mut_f64(const StepArgs& a, int p, cudaStream_t s);
void enqueue_sa_mut_f32(const StepArgs& a, int p, cudaStream_t s);
// Scalar permutes between reference and device cell order (FP64 [N]).
void enqueue_permute_in1(int n, const int* cell_old, const void* src_ref, void* dst_dev, cudaStream_t s);
void enqueue_permute_out1(int n, const int* cell_old, const void* src_dev, void* dst_ref, cudaStream_t s);

// Pressure forces over one boundary patch (post.h:301-387).
struct ForceArgs {
    int n = 0;
    const int* cell = nullptr;     // device cell of each patch edge
    const double* geo = nullptr;   // 5 per edge: ecx, ecy, nx, ny, L
    double xmin = 0, xmax = 0, x_moment = 0, y_moment = 0;
    double p_inf = 1, mach_inf = 0.2, gamma = 1.4;
    const double* q = nullptr;     // FP64 master state (d4)
    double* cp = nullptr;          // per edge
    double* sums = nullptr;        // fx, fy, m
};
void enqueue_forces(const ForceArgs& f, cudaStream_t s);

// Adjoint of the FP64 residual (afx_adjoint.cu): u = (dR/dq)^T v and
// bqbar = (dR/dbq)^T v at the state of parity p.  Device-order arrays.
struct AdjArgs {
    const void* v = nullptr;  // d4 [N] weights on the residual
    void* fbar = nullptr;     // d4 [2F] per face: adjoint of the left input, of the right input / boundary state
    void* gbx = nullptr;      // d4 [N] adjoint of the x gradient
    void* gby = nullptr;      // d4 [N] adjoint of the y gradient
    void* qbar = nullptr;     // d4 [N] state adjoint before the neighbour terms
    void* lw = nullptr;       // d4 [2N] limiter max/min weights
    void* lt = nullptr;       // int4 [2N] limiter max/min target cells
    void* u = nullptr;        // d4 [N] result
    void* bqbar = nullptr;    // d4 [B] result (boundary states)
    int dirs_per_pass = 4;    // face kernel: input directions per vector-dual pass (1, 2 or 4)
};
// gradients and limiter of state p (and the local time step when with_dt)
void enqueue_adjoint_prep(const StepArgs& a, int p, bool with_dt, cudaStream_t s);
void enqueue_vjp(const StepArgs& a, int p, const AdjArgs& j, cudaStream_t s);
// lam_out = lam0 + alpha*relax*dt*(u + g); ||u + g||^2 block partials (256 cells per block) if partials
void enqueue_adjoint_update(int n, const void* lam0, const void* u, const void* g, const void* dt, double alpha,
                            double relax, void* lam_out, double* partials, cudaStream_t s);
// g += dJ/dq for J = cx*fx + cy*fy over the patch of f (g zeroed by the caller)
void enqueue_objective_grad(const ForceArgs& f, double cx, double cy, void* g, cudaStream_t s);

}  // namespace afx
