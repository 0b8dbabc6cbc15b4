// Shared device-side types of the Q1 multiscale basis build (sm_103a).
//
// Data layout in HBM (one batch of coarse cells):
//   a, reaction   FP64 per fine cell, per coarse cell n^3 values lexicographic
//   phi, y        FP64 planar per coarse cell: 8 planes (coarse vertex v) of
//                 (n+1)^3 nodes; y = K phi (unconstrained operator)
//   stats         per (cell, coarse vertex) convergence record
// The local PCG state never leaves the SM: the search direction lives in a
// shared-memory z-slab, x / dinv in shared memory, r / q in registers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace msfec {

constexpr int kQ1Threads = 512;
constexpr int kQ1MaxCluster = 8;
constexpr int kQ1Warps = kQ1Threads / 32;
constexpr int kRedVals = 3;

struct Q1Cell {
  double origin[3];
  double h[3];         // fine-cell size per direction
  int depth;
  int n;               // 2^depth
  long long coef_off;  // first fine cell of this coarse cell in a[]
  long long node_off;  // sum of (n+1)^3 over previous cells; phi base = 8*node_off
};

// One local solve job: `nrhs` consecutive coarse vertices of one cell.
struct Q1Item {
  int cell;
  int rhs0;
  int nrhs;
  int slab;  // 1: z-slab decomposition over every CTA of the cluster
  int mode;  // 0: basis (Dirichlet data = coarse vertex function, no load);
             // 1: source (zero Dirichlet data, right-hand side from src_rhs)
  int pad;
};

// One dequeue of the persistent kernel, executed by one cluster.
struct Q1Unit {
  int first_item;
  int n_items;  // independent units: item first+r runs on cluster rank r
  int slab;
  int pad;
};

struct Q1Stat {
  int iters;
  int refinements;
  int converged;
  int flags;  // bit 0: Krylov breakdown (p.Ap <= 0 or non-finite)
  double rel_residual;
};

struct Q1Params {
  const Q1Cell *cells;
  const Q1Item *items;
  const Q1Unit *units;
  int n_units;
  int *queue;
  const double *a;
  const double *react;
  double *phi;
  double *y;
  const double *src_rhs;  // mode 1: [cell][8][(n+1)^3] right-hand sides (FP64)
  double *src_out;        // mode 1: solutions, same layout
  Q1Stat *stats;
  double rtol;
  double inner_rtol;
  int max_iter;
  int max_refine;
};

// Planes per CTA of an item (z-slab decomposition of the m = n-1 interior
// node planes k = 1..m).
__host__ __device__ inline int q1_planes_per_cta(int n, int nslab) {
  const int m = n - 1;
  return (m + nslab - 1) / nslab;
}

// Dynamic shared memory of one item (bytes), identical on host and device.
struct Q1Smem {
  size_t slab_off, caf_off, raf_off, x_off, p_off, s_off, dv_off, total;
};

__host__ __device__ inline size_t q1_align(size_t v) { return (v + 255) & ~(size_t)255; }

// slab: (PS+2) planes of (n+1)^2 nodes x R, sized for FP64 staging (the
//       Krylov search direction of precision T aliases it);
// caf/raf: float coefficient layers k0-1 .. k0+PS-1; x, p, s: owned nodes x R
// (T; iterate, search direction and its image s = K p); dv: Jacobi scaling
// per owned node (float).
__host__ __device__ inline Q1Smem q1_smem_layout(int n, int R, int nslab, bool has_r, int tsize) {
  const int PS = q1_planes_per_cta(n, nslab);
  const int m = n - 1;
  const size_t N1sq = (size_t)(n + 1) * (n + 1);
  Q1Smem s;
  size_t off = 0;
  s.slab_off = off;
  off = q1_align(off + (size_t)(PS + 2) * N1sq * R * sizeof(double));
  const size_t ncf = (size_t)(PS + 1) * n * n;
  s.caf_off = off;
  off = q1_align(off + ncf * sizeof(float));
  s.raf_off = off;
  if (has_r) off = q1_align(off + ncf * sizeof(float));
  s.x_off = off;
  off = q1_align(off + (size_t)PS * m * m * R * tsize);
  s.p_off = off;
  off = q1_align(off + (size_t)PS * m * m * R * tsize);
  s.s_off = off;
  off = q1_align(off + (size_t)PS * m * m * R * tsize);
  s.dv_off = off;
  off = q1_align(off + (size_t)PS * m * m * sizeof(float));
  s.total = off;
  return s;
}

// ---- tensor-coefficient Q1 solver (q1g_solve.cu): one (cell, coarse vertex)
// item per CTA, cell-wise quadrature apply.
struct Q1GItem {
  int cell;
  int vertex;  // coarse vertex 0..7 (basis mode) / right-hand side plane (source mode)
  int mode;    // 0 basis function, 1 source: zero Dirichlet data, right-hand side from src_rhs
  int pad;
};

struct Q1GParams {
  const Q1Cell *cells;
  const Q1GItem *items;
  int n_items;
  int *queue;
  const double *a;  // 6 (tensor) or 48 (Gauss points) doubles per fine cell
  int gauss;
  const double *react;  // per fine cell or null
  const float *ed;      // element data per fine cell, q1g_ed_floats(gauss) floats (q1g_prepare_kernel)
  double *phi;          // basis mode: [cell][8][(n+1)^3] at 8 node_off
  double *y;            // K phi, same layout
  const double *src_rhs;  // source mode: [cell][8][(n+1)^3] right-hand sides
  double *src_out;        // source mode: solutions, same layout
  Q1Stat *stats;          // [cell][8]
  float *scratch;         // per-CTA global workspace (vectors that exceed shared memory)
  size_t scratch_floats;
  double rtol;
  double inner_rtol;
  int max_iter;
  int max_refine;
};

constexpr int kQ1GThreads = 256;
constexpr int kQ1GWarps = kQ1GThreads / 32;

// Floats of element data per fine cell: the scaled tensor(s) B (6 per point,
// one point for a tensor per cell, 8 Gauss points), r |e|, pad to 16 bytes.
__host__ __device__ inline int q1g_ed_floats(int gauss) { return gauss ? 52 : 8; }

// Workspace (floats) of one item: Jacobi scaling (float) + x, r, p, q of
// precision T over the padded node set; ed_floats more when the cell's element
// data is staged too.
__host__ __device__ inline size_t q1g_vec_floats(int n, int tsize) {
  const size_t nn = (size_t)(n + 1) * (n + 1) * (n + 1);
  const size_t Np = (nn + 63) / 64 * 64;
  return Np + 4 * Np * (size_t)(tsize / 4);
}

}  // namespace msfec
