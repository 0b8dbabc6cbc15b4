// Instantiation of the persistent Q1 solver: double Krylov arithmetic, cluster size 8.
#include "q1_solve_impl.cuh"

namespace msfec {
cudaError_t q1_solve_launch_f64_c8(bool has_r, bool slab_only, const Q1Params &prm, size_t smem, int grid,
                                    cudaStream_t st) {
  if (slab_only)
    return has_r ? q1impl::launch<double, 8, true, true>(prm, smem, grid, st)
                 : q1impl::launch<double, 8, false, true>(prm, smem, grid, st);
  return has_r ? q1impl::launch<double, 8, true>(prm, smem, grid, st) : q1impl::launch<double, 8, false>(prm, smem, grid, st);
}
cudaError_t q1_solve_occupancy_f64_c8(bool has_r, bool slab_only, size_t smem, int *out) {
  if (slab_only)
    return has_r ? q1impl::occupancy<double, 8, true, true>(smem, out) : q1impl::occupancy<double, 8, false, true>(smem, out);
  return has_r ? q1impl::occupancy<double, 8, true>(smem, out) : q1impl::occupancy<double, 8, false>(smem, out);
}
}  // namespace msfec
