// Instantiation of the persistent Q1 solver: double Krylov arithmetic, cluster size 1.
#include "q1_solve_impl.cuh"

namespace msfec {
cudaError_t q1_solve_launch_f64_c1(bool has_r, const Q1Params &prm, size_t smem, int grid, cudaStream_t st) {
  return has_r ? q1impl::launch<double, 1, true>(prm, smem, grid, st) : q1impl::launch<double, 1, false>(prm, smem, grid, st);
}
cudaError_t q1_solve_occupancy_f64_c1(bool has_r, size_t smem, int *out) {
  return has_r ? q1impl::occupancy<double, 1, true>(smem, out) : q1impl::occupancy<double, 1, false>(smem, out);
}
}  // namespace msfec
