// Ned_RT persistent solver, mixed precision, one 512-thread CTA per SM with the
// MINRES workspace in a global slot and z~ in shared memory (multilevel face
// preconditioner with the per-cell shared data only).
#include "nedrt_solver.cuh"

namespace msfec {

cudaError_t nedrt_solve_f32_zs(const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (!prm.prep || !prm.coarse) return cudaErrorInvalidValue;
  return nedrt_launch_variant<float, kNRThreads, true, 3>(prm, smem, grid, st, false);
}

}  // namespace msfec
