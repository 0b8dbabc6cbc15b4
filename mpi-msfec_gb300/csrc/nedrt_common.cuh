// Shared types of the Nedelec x Raviart-Thomas multiscale basis build (sm_103a).
//
// Fine DoF numbering per coarse cell (n = 2^depth fine cells per edge):
//   edges [x | y | z], x-edge (i<n, j<=n, k<=n) -> i + n(j + (n+1)k), y-edge
//   (i<=n, j<n, k<=n) -> NEx + i + (n+1)(j + n k), z-edge (i<=n, j<=n, k<n)
//   -> 2NEx + i + (n+1)(j + (n+1)k); faces [x | y | z] after the NE edges,
//   x-face (i<=n, j<n, k<n) -> i + (n+1)(j + n k), y-face (i<n, j<=n, k<n)
//   -> NFx + i + n(j + (n+1)k), z-face (i<n, j<n, k<=n) -> 2NFx + i + n(j + n k).
// Coarse basis b: 0..11 coarse edges in deal.II GeometryInfo<3> line order,
// 12..17 coarse faces in face order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace msfec {

constexpr int kNRThreads = 512;
constexpr int kNRWarps = kNRThreads / 32;

struct NRCell {
  double origin[3];
  double h[3];
  int depth;
  int n;
  long long coef_off;  // first fine cell in ainv6 / bdiv
  long long dof_off;   // sum of previous cells' DoF counts; Phi base = 18 * dof_off
  long long coarse_off;  // first float of the cell's multilevel preconditioner data, -1: none
  long long prep_off;    // first float of the cell's shared preconditioner + coefficients (NRParams::prep)
};

struct NRItem {
  int cell;
  int basis;  // 0..17 (basis mode); right-hand side 0..3 of the cell (source mode)
  int mode;   // 0 basis function, 1 source: zero Dirichlet data, load from src_rhs,
              // 2 source with natural boundary conditions: every DoF free (standard fine solve)
};

constexpr int kNRSrcRhs = 4;  // source-mode right-hand sides per cell (adjoint)

struct NRStat {
  int iters;
  int refinements;
  int converged;
  int flags;
  double rel_residual;
};

struct NRParams {
  const NRCell *cells;
  const NRItem *items;
  int n_items;
  int *queue;
  const double *ainv6;  // [fine][6]: a00 a11 a22 a01 a02 a12 of A^-1
  const double *bdiv;   // [fine]
  double *phi;          // [18][ndof] per cell
  double *y;            // [18][ndof] per cell: A P_b (primary block of basis b)
  NRStat *stats;        // [cell][18]
  const double *src_rhs;  // source mode: [cell][kNRSrcRhs][ndof] at kNRSrcRhs * dof_off
  double *src_out;        // source mode: solutions, same layout
  const double *src_scale2;  // source mode: [dof_off + d] squared scale of the terms the right-hand side
                             // is a difference of; 1e-3 of its P-norm floors ||f||_P in the stopping test (null: none)
  // global workspace: per cell at NRCell::prep_off, the preconditioner diagonal
  // (Np floats) and the float coefficients (8 per fine cell), built once by
  // nr_cell_prep_kernel and read by the cell's 18 items, whose global slots then
  // hold only Krylov vectors; null: every item builds its own in its slot
  float *prep;
  // with prep and the multilevel face preconditioner: the edge block of the
  // preconditioner is the additive Schwarz operator over fine-cell patches,
  // sum_c R_c^T (M restricted to cell c's 12 edges)^-1 R_c, instead of diag(M)^-1
  int edge_patch;
  float *scratch;       // global workspace when the item does not fit shared memory
  size_t scratch_floats;  // per CTA
  const float *coarse;    // multilevel preconditioner data (per cell at coarse_off); null: diagonal only
  size_t ml_offset;       // byte offset of the multilevel region in the dynamic shared memory
  int use_smem;
  // global workspace, mixed precision: the apply's coefficient tiles staged by
  // bulk copies into the dynamic shared memory at this byte offset (32 KB)
  int stage;
  size_t stage_offset;
  // global workspace, mixed precision, multilevel with prep: z~ (the apply's
  // operand, the patch pass's accumulator) in the dynamic shared memory at this
  // byte offset instead of the slot; the slot's other vectors stay in L2
  int zt_smem;
  size_t zt_offset;
  double rtol;
  double inner_rtol;
  int max_iter;
  int max_refine;
};

__host__ __device__ inline void nr_counts(int n, int &NEx, int &NFx, int &NE, int &NF) {
  NEx = n * (n + 1) * (n + 1);
  NFx = (n + 1) * n * n;
  NE = 3 * NEx;
  NF = 3 * NFx;
}

// Workspace (floats) of one item: preconditioner (float) + 7 Krylov vectors
// of precision T (tsize bytes), all over the full DoF set, plus float copies of
// the coefficients (8 per fine cell: A^-1 (6), B/|K|, pad; 16-byte aligned).
__host__ __device__ inline size_t nr_workspace_floats(int n, int tsize) {
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t N = (size_t)NE + NF;
  const size_t al = 64;
  const size_t Np = (N + al - 1) / al * al;
  const size_t nc = (size_t)n * n * n;
  return Np + 7 * Np * (size_t)(tsize / 4) + (8 * nc + al - 1) / al * al;
}

// Per-cell shared data of the global workspace (NRParams::prep), 64-float
// aligned parts: the preconditioner diagonal over the padded DoFs, 8 float
// coefficients per fine cell, and the cell-patch factors of the edge
// preconditioner (kNRPatchFloats 32-bit words per fine cell in 16-byte groups,
// structure of arrays by group: word t of fine cell c at (t / 4 * n^3 + c) * 4
// + t % 4).
constexpr int kNRPatchFloats = 40;  // L^-1 of a 12 x 12 Cholesky factor: 78 FP16 entries, 2 per word, 1 pad word
__host__ __device__ inline size_t nr_prep_floats(int n) {
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
  const size_t nc = (size_t)n * n * n;
  return Np + (8 * nc + 63) / 64 * 64 + (kNRPatchFloats * nc + 63) / 64 * 64;
}
__host__ __device__ inline size_t nr_prep_patch_offset(int n) {
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
  return Np + (8 * (size_t)n * n * n + 63) / 64 * 64;
}
// Global slot of one item when the cell's data is shared (NRParams::prep):
// the Krylov vectors z~, v~ (2), w (2), x, and the apply's accumulation vector
// for the diagonal-preconditioner path only (the multilevel path accumulates
// the apply into the spent Lanczos vector).
__host__ __device__ inline size_t nr_prep_slot_floats(int n, int tsize, bool multilevel) {
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
  return (multilevel ? 6 : 7) * Np * (size_t)(tsize / 4);
}

// Split workspace of the two-CTAs-per-SM mixed variant (256 threads): the
// shared part holds the preconditioner and 6 FP32 Krylov vectors, the
// per-CTA global slot the correction x and the 8 float coefficients per cell.
__host__ __device__ inline size_t nr_split_smem_floats(int n) {
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
  return 7 * Np;
}
__host__ __device__ inline size_t nr_split_global_floats(int n) {
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
  return Np + (8 * (size_t)n * n * n + 63) / 64 * 64;
}

// ---- multilevel (BPX) preconditioner of the face (Schur) block
// Face-space hierarchy of a cell with n = 2^L fine cells per side: levels
// m = n/2, n/4, ..., 2 (k = 1 .. L-1). Level m holds the lowest-order RT
// functions of the m^3 sub-box grid whose flux sits on an interior plane
// P = 1..m-1: 3 (m-1) m^2 functions, index (d (m-1) + P-1) m^2 + b m + a for
// normal d and patch (a, b) on the two other axes in increasing order.
__host__ __device__ inline int nr_ml_count(int m) { return 3 * (m - 1) * m * m; }

// Per-cell data (floats): inverse diagonals of the Galerkin operators of the
// levels n/2 .. 4, then the 12 x 12 inverse of the level-2 operator.
__host__ __device__ inline int nr_ml_data_floats(int n) {
  if (n < 4) return 0;
  int s = 144;
  for (int m = n / 2; m >= 4; m /= 2) s += nr_ml_count(m);
  return s;
}

// After that data, per cell: the inverse of the assembled diagonal of the
// Schur operator on every face (0 on the boundary), the fine level of the
// multilevel operator; the solver reads it into its preconditioner vector.
__host__ __device__ inline int nr_ml_fine_floats(int n) {
  if (n < 4) return 0;
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  return NF;
}
__host__ __device__ inline int nr_ml_cell_floats(int n) { return nr_ml_data_floats(n) + nr_ml_fine_floats(n); }

// Layout of the solver's multilevel region (bytes from its start): restriction
// accumulator and correction of level n/2 (precision T), the restricted /
// corrected vectors of the levels below, the cell's data, one 16-bit code per
// face DoF (and pad) giving its level-n/2 parents, and one per function of the
// levels n/2 .. 4 giving its parents one level down.
struct NRMLLayout {
  int F1;
  size_t off_y, off_wk, off_data, off_codes, off_lcodes, bytes;
};

__host__ __device__ inline NRMLLayout nr_ml_layout(int n, int tsize) {
  NRMLLayout l{};
  if (n < 4) return l;
  int NEx, NFx, NE, NF;
  nr_counts(n, NEx, NFx, NE, NF);
  const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
  l.F1 = nr_ml_count(n / 2);
  size_t fw = 0, nl = 0;
  for (int m = n / 4; m >= 2; m /= 2) fw += nr_ml_count(m);
  for (int m = n / 2; m >= 4; m /= 2) nl += nr_ml_count(m);
  auto al16 = [](size_t b) { return (b + 15) / 16 * 16; };
  l.off_y = (size_t)l.F1 * tsize;
  l.off_wk = 2 * (size_t)l.F1 * tsize;
  l.off_data = al16(l.off_wk + 2 * fw * tsize);
  l.off_codes = al16(l.off_data + (size_t)nr_ml_data_floats(n) * 4);
  l.off_lcodes = al16(l.off_codes + (Np - NE) * 2);
  l.bytes = al16(l.off_lcodes + nl * 2);
  return l;
}

}  // namespace msfec
