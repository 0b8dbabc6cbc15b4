// Shared types of the Raviart-Thomas x DQ0 (RT_DQ) multiscale basis build (sm_103a).
//
// Fine DoF numbering per coarse cell (n = 2^depth fine cells per edge): faces
// in the Ned_RT numbering (x-faces i + (n+1)(j + n k), then y-, z-faces,
// NF = 3 n^2 (n+1)), then the fine cells c = i + n(j + n k) (NC = n^3).
// Coarse basis b = 0..5: the coarse faces in GeometryInfo<3> face order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nedrt_common.cuh"

namespace msfec {

constexpr int kRTBases = 6;
constexpr int kRTCoarse = 7;  // coarse DoFs per cell: 6 faces + 1 DQ0 value
constexpr int kRTThreads = 512;
constexpr int kRTWarps = kRTThreads / 32;

struct RTParams {
  const NRCell *cells;    // same cell record as Ned_RT (dof_off: sum of NF + NC)
  const NRItem *items;    // (cell, basis 0..5)
  int n_items;
  int *queue;
  const double *ainv6;    // [fine][6]: A^-1 (a00 a11 a22 a01 a02 a12)
  double *phi;            // [6][ndof] per cell
  double *y;              // [6][ndof] per cell: A (sigma_b, 0)
  NRStat *stats;          // [cell][6]
  float *scratch;         // global workspace when the item does not fit shared memory
  size_t scratch_floats;  // per CTA
  int use_smem;
  double rtol;
  double inner_rtol;
  int max_iter;
  int max_refine;
};

__host__ __device__ inline void rt_counts(int n, int &NFx, int &NF, int &NC) {
  NFx = (n + 1) * n * n;
  NF = 3 * NFx;
  NC = n * n * n;
}

// Workspace (floats) of one item: preconditioner + 7 Krylov vectors of
// precision T (tsize bytes) over all DoFs, plus 8 float coefficients per cell.
__host__ __device__ inline size_t rt_workspace_floats(int n, int tsize) {
  int NFx, NF, NC;
  rt_counts(n, NFx, NF, NC);
  const size_t Np = ((size_t)NF + NC + 63) / 64 * 64;
  return Np + 7 * Np * (size_t)(tsize / 4) + (8 * (size_t)NC + 63) / 64 * 64;
}

}  // namespace msfec
