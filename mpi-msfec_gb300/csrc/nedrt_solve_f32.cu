// Ned_RT persistent solver, mixed precision (FP32 MINRES inside FP64
// refinement), one 512-thread CTA per SM.
#include "nedrt_solver.cuh"

namespace msfec {

cudaError_t nedrt_solve_f32(bool ml, int place, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (place == 1)
    return ml ? nedrt_launch_variant<float, kNRThreads, true, 1>(prm, smem, grid, st, false)
              : nedrt_launch_variant<float, kNRThreads, false, 1>(prm, smem, grid, st, false);
  if (place == 2)
    return ml ? nedrt_launch_variant<float, kNRThreads, true, 2>(prm, smem, grid, st, false)
              : nedrt_launch_variant<float, kNRThreads, false, 2>(prm, smem, grid, st, false);
  return ml ? nedrt_launch_variant<float, kNRThreads, true, 0>(prm, smem, grid, st, false)
            : nedrt_launch_variant<float, kNRThreads, false, 0>(prm, smem, grid, st, false);
}

}  // namespace msfec
