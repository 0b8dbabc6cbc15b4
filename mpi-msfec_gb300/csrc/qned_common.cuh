// Shared types of the Q1 x Nedelec (Q_Ned) multiscale basis build (sm_103a).
//
// Fine DoF numbering per coarse cell (n = 2^depth fine cells per edge):
// vertices i + (n+1)(j + (n+1)k) (NV = (n+1)^3), then the edges in the Ned_RT
// numbering (x-, y-, z-edges, NE = 3 n (n+1)^2). Coarse basis b: 0..7 the
// H1 bases (GeometryInfo<3> vertices, v = x + 2y + 4z), 8..19 the curl bases
// (GeometryInfo<3> lines).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nedrt_common.cuh"

namespace msfec {

constexpr int kQNBases = 20;
constexpr int kQNThreads = 512;
constexpr int kQNWarps = kQNThreads / 32;

struct QNParams {
  const NRCell *cells;    // same cell record as Ned_RT (dof_off: sum of NV + NE)
  const NRItem *items;    // (cell, basis 0..19)
  int n_items;
  int *queue;
  const double *a6;       // [fine][6]: a00 a11 a22 a01 a02 a12 of A (curl-curl weight)
  const double *binv;     // [fine]: B^-1 (sigma mass weight)
  double *phi;            // [20][ndof] per cell
  double *y;              // [20][ndof] per cell: A P_b (primary block of basis b)
  NRStat *stats;          // [cell][20]
  float *scratch;         // global workspace when the item does not fit shared memory
  size_t scratch_floats;  // per CTA
  int use_smem;
  double rtol;
  double inner_rtol;
  int max_iter;
  int max_refine;
};

__host__ __device__ inline void qn_counts(int n, int &NV, int &NEx, int &NE) {
  NV = (n + 1) * (n + 1) * (n + 1);
  NEx = n * (n + 1) * (n + 1);
  NE = 3 * NEx;
}

// Workspace (floats) of one item: preconditioner + 7 Krylov vectors of
// precision T (tsize bytes) over all DoFs, plus 8 float coefficients per cell.
__host__ __device__ inline size_t qn_workspace_floats(int n, int tsize) {
  int NV, NEx, NE;
  qn_counts(n, NV, NEx, NE);
  const size_t Np = ((size_t)NV + NE + 63) / 64 * 64;
  return Np + 7 * Np * (size_t)(tsize / 4) + (8 * (size_t)n * n * n + 63) / 64 * 64;
}

}  // namespace msfec
