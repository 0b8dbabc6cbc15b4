// Ned_RT persistent solver, mixed precision, two 256-thread CTAs per SM:
// place 1 = split workspace (preconditioner + 6 FP32 vectors in shared memory,
// x + coefficients in the CTA's global slot), place 0 = whole workspace in the
// CTA's global slot (deep cells: two items per SM overlap each other's
// barriers and reductions).
#include "nedrt_solver.cuh"

namespace msfec {

cudaError_t nedrt_solve_f32_256(bool ml, int place, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (place == 1)
    return ml ? nedrt_launch_variant<float, 256, true, 1>(prm, smem, grid, st, true)
              : nedrt_launch_variant<float, 256, false, 1>(prm, smem, grid, st, true);
  return ml ? nedrt_launch_variant<float, 256, true, 0>(prm, smem, grid, st, true)
            : nedrt_launch_variant<float, 256, false, 0>(prm, smem, grid, st, true);
}

cudaError_t nedrt_solve_f32_256_occupancy(bool ml, int place, size_t smem, int *blocks_per_sm) {
  void (*k)(NRParams);
  if (place == 1)
    k = ml ? nrimpl::nedrt_solve_kernel<float, 256, true, 1> : nrimpl::nedrt_solve_kernel<float, 256, false, 1>;
  else
    k = ml ? nrimpl::nedrt_solve_kernel<float, 256, true, 0> : nrimpl::nedrt_solve_kernel<float, 256, false, 0>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, 256, smem);
}

}  // namespace msfec
