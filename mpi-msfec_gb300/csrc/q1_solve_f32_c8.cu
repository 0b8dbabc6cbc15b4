// Instantiation of the persistent Q1 solver: float Krylov arithmetic, cluster size 8.
#include "q1_solve_impl.cuh"

namespace msfec {
cudaError_t q1_solve_launch_f32_c8(bool has_r, const Q1Params &prm, size_t smem, int grid, cudaStream_t st) {
  return has_r ? q1impl::launch<float, 8, true>(prm, smem, grid, st) : q1impl::launch<float, 8, false>(prm, smem, grid, st);
}
cudaError_t q1_solve_occupancy_f32_c8(bool has_r, size_t smem, int *out) {
  return has_r ? q1impl::occupancy<float, 8, true>(smem, out) : q1impl::occupancy<float, 8, false>(smem, out);
}
}  // namespace msfec
