// Ned_RT persistent solver, plain FP64 path (MINRES in FP64), 512 threads.
#include "nedrt_solver.cuh"

namespace msfec {

cudaError_t nedrt_solve_f64(bool ml, int place, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (place == 1)
    return ml ? nedrt_launch_variant<double, kNRThreads, true, 1>(prm, smem, grid, st, false)
              : nedrt_launch_variant<double, kNRThreads, false, 1>(prm, smem, grid, st, false);
  return ml ? nedrt_launch_variant<double, kNRThreads, true, 0>(prm, smem, grid, st, false)
            : nedrt_launch_variant<double, kNRThreads, false, 0>(prm, smem, grid, st, false);
}

}  // namespace msfec
