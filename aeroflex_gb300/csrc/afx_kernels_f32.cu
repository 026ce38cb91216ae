// FP32-mixed path: face fluxes, gradients and limiters in FP32, the RK state
// update, the residual norm and the forces in FP64.  The FP64 master state is
// kept with an FP32 shadow that the flux kernels read.  Compiled with
// -use_fast_math: FP32 division and square root use the SFU approximations
// (<= 2 ulp), FMA contraction is on and FP32 denormals flush to zero; the
// FP64 update and norm in this file are unaffected by those flags.
#include "afx_kernels_impl.cuh"

namespace afx {

void enqueue_iteration_f32(const StepArgs& a, int p, cudaStream_t s) { dev::iteration<float, float, true>(a, p, s); }
void enqueue_residual_f32(const StepArgs& a, int p, cudaStream_t s) { dev::residual<float, float>(a, p, s); }
void enqueue_last_stage_residual_f32(const StepArgs& a, int p, cudaStream_t s) {
    dev::last_stage_residual<float, float>(a, p, s);
}
void enqueue_uniform_f32(const StepArgs& a, int p, const double* qf, cudaStream_t s) {
    dev::uniform<float, float>(a, p, qf, s);
}
void enqueue_correction(int n, const void* R64, const void* R32, void* corr, cudaStream_t s) {
    dev::k_correction<<<(n + 255) / 256, 256, 0, s>>>(n, (const dev::d4*)R64, (const dev::d4*)R32, (float4*)corr);
}

void enqueue_sa_implicit_f32(const StepArgs& a, int p, int sweeps, cudaStream_t s) {
    dev::sa_implicit<float, float>(a, p, sweeps, s);
}
void enqueue_sa_mut_f32(const StepArgs& a, int p, cudaStream_t s) {
    dev::sa_mut<float, float>(a, (const dev::V4<float>*)a.qsh[p], a.sa_nu[p], s);
}

}  // namespace afx
