// Persistent Ned_RT local solver, shared by the per-precision translation
// units (nedrt_solve_f32.cu, nedrt_solve_f32_256.cu, nedrt_solve_f64.cu) and
// by nedrt_solve.cu (setup, Galerkin and adjoint kernels reuse the element
// helpers).
//
// Persistent batched Nedelec x Raviart-Thomas local solver (sm_103a).
//
// Restates, for every coarse cell x coarse basis function (12 edge + 6 face),
// the reference's mixed local problem (konsim83/MPI-MSFEC):
//   NedRTBasis::assemble_system   source/Ned_RT/ned_rt_basis.cc:361-576
//     local matrix (A^-1 sigma, tau) - (u, curl tau) + (curl sigma, v) + (B div u, div v)
//   setup_basis_dofs_curl / _div  ned_rt_basis.cc:224-359 (boundary data = coarse
//     Nedelec / RT function, zero for the other field)
//   run solve loop                ned_rt_basis.cc:1338-1381
//   solve_iterative (Schur CG + ILU/GMRES there) ned_rt_basis.cc:636-847
// The saddle-point system is solved (in its symmetric form, face rows negated)
// with MINRES preconditioned by diag(M)^-1 on the edges and, on the faces,
// either diag(D + C^T diag(M)^-1 C)^-1 or (default) that diagonal plus the
// multilevel coarse-RT correction built below (ml_coarse_block,
// nr_ml_setup_kernel), FP32 inside FP64 iterative refinement (MINRES in FP64
// for the plain FP64 path); the
// operator is applied matrix-free, cell by cell, from the per-cell A^-1 / B in
// tensor-product form (1D P1 mass factors), accumulating into shared memory
// with atomics; the closed-form element tables feed the preconditioner.
// The last FP64 pass writes y_b = A P_b (P_b the primary block of basis b:
// sigma of an edge basis, u of a face basis) for the Galerkin product of
// NedRTBasis::assemble_global_element_matrix (ned_rt_basis.cc:849-948).
#pragma once
#include <cuda_fp16.h>
#include "../../include/msfec_cuda.h"
#include "nedrt_common.cuh"

namespace msfec {
namespace nrimpl {

// Per-item constants of the tensor-product element operator (cell sides h).
template <typename TA>
struct NRFactors {
  TA hd[3];     // h_o1 h_o2 / (36 h_p): diagonal edge-mass block of direction p, per unit A_pp
  TA hq[3];     // h_r / 24: block coupling the two edge directions other than r, per unit A_pq
  TA cf[3][3];  // eps(p, fd) h_fd / (6 h_p h_t): edges of direction p against faces of normal fd
};

struct NRShared {
  double wred[kNRWarps][3];
  float fred[kNRWarps][3];  // float slots: no FP64 instruction in the FP32 Krylov loop
  // closed-form element tables of the current item's cell (preconditioner setup):
  float Gf[3][3][4][4];  // edge-mass geometry: M_e = sum_pq A^-1_pq Gf[p][q]
  float Cf[12][6];       // (curl tau_l, v_f) on the fine cell
  NRFactors<float> Ff;  // tensor-product factors of the current item's cell
  NRFactors<double> Fd;
  alignas(16) float fslot[3][kNRWarps];  // per-warp partials of the fused MINRES reductions
  double dslot[3][kNRWarps];              // (slot 2: multilevel share of gamma^2)
  // per-warp completion barriers of the two coefficient stages (staged apply)
  alignas(8) unsigned long long mbar[kNRWarps][2];
  unsigned tph[kNRWarps];  // their phase bits, kept across items
  int item;
};

// ---- bulk-copy (TMA) staging of coefficient tiles: mbarrier + cp.async.bulk
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// One global -> shared bulk copy of `bytes` (multiple of 16, both addresses
// 16-byte aligned) completing on `bar`, which this call arms for the bytes.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Wait for the completion of phase `parity` of `bar`, at most ~2^22 polls;
// false when that limit ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
  const unsigned a = smem_u32(bar);
  for (int i = 0; i < (1 << 22); ++i) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

struct NRGeom {
  int n, L, NEx, NFx, NE, NF, N;  // n = 2^L fine cells per edge
};

__device__ __forceinline__ double psi(int a, double t) { return a ? t : 1.0 - t; }
__device__ __forceinline__ double sgn(int a) { return a ? 1.0 : -1.0; }
__device__ __forceinline__ double m1(int a, int b) { return a == b ? 1.0 / 3.0 : 1.0 / 6.0; }

// The two axes other than p, in increasing order.
__device__ __forceinline__ void other_axes(int p, int &o1, int &o2) {
  o1 = p == 0 ? 1 : 0;
  o2 = p == 2 ? 1 : 2;
}

// Position (0/1) along axis `ax` of local edge l4 (0..3) of direction p.
__device__ __forceinline__ int edge_pos(int p, int l4, int ax) {
  int o1, o2;
  other_axes(p, o1, o2);
  return ax == o1 ? (l4 & 1) : (l4 >> 1);
}

// Closed forms of the 2x2x2-Gauss integrals of lowest-order Nedelec / RT
// functions on a box with sides h (exact: polynomial degree <= 3 per axis).
__device__ inline double table_G(const double h[3], int p, int q, int l4, int m4) {
  if (p == q) {
    int o1, o2;
    other_axes(p, o1, o2);
    return h[o1] * h[o2] / h[p] * m1(l4 & 1, m4 & 1) * m1(l4 >> 1, m4 >> 1);
  }
  const int r = 3 - p - q;
  return 0.25 * h[r] * m1(edge_pos(p, l4, r), edge_pos(q, m4, r));
}

__device__ inline double table_C(const double h[3], int l, int f) {
  const int p = l >> 2, l4 = l & 3;
  const int fd = f >> 1, fa = f & 1;
  if (fd == p) return 0.0;
  const double hx = h[0], hy = h[1], hz = h[2];
  const int a0 = l4 & 1, a1 = l4 >> 1;  // positions along the two other axes
  if (p == 0) {  // (b, c) = (y, z)
    if (fd == 1) return sgn(a1) * hy * m1(a0, fa) / (hx * hz);
    return -sgn(a0) * hz * m1(a1, fa) / (hx * hy);
  }
  if (p == 1) {  // (a, c) = (x, z)
    if (fd == 0) return -sgn(a1) * hx * m1(a0, fa) / (hy * hz);
    return sgn(a0) * hz * m1(a1, fa) / (hx * hy);
  }
  // p == 2, (a, b) = (x, y)
  if (fd == 0) return sgn(a1) * hx * m1(a0, fa) / (hy * hz);
  return -sgn(a0) * hy * m1(a1, fa) / (hx * hz);
}

__device__ __forceinline__ void cell_dofs(const NRGeom &g, int c, int (&e)[12], int (&f)[6]) {
  // one base index per DoF family, the neighbours at constant strides
  const int n = g.n, n1 = n + 1;
  const int i = c & (n - 1), j = (c >> g.L) & (n - 1), k = c >> (2 * g.L);
  const int ex = i + n * (j + n1 * k);
  const int ey = g.NEx + i + n1 * (j + n * k);
  const int ez = 2 * g.NEx + i + n1 * (j + n1 * k);
  e[0] = ex;
  e[1] = ex + n;
  e[2] = ex + n * n1;
  e[3] = ex + n * n1 + n;
  e[4] = ey;
  e[5] = ey + 1;
  e[6] = ey + n1 * n;
  e[7] = ey + n1 * n + 1;
  e[8] = ez;
  e[9] = ez + 1;
  e[10] = ez + n1;
  e[11] = ez + n1 + 1;
  const int fx = g.NE + i + n1 * (j + n * k);
  const int fy = g.NE + g.NFx + i + n * (j + n1 * k);
  const int fz = g.NE + 2 * g.NFx + i + n * (j + n * k);
  f[0] = fx;
  f[1] = fx + 1;
  f[2] = fy;
  f[3] = fy + n;
  f[4] = fz;
  f[5] = fz + n * n;
}

// (dir, i, j, k) of DoF d; returns true for a lattice-boundary DoF.
__device__ inline bool dof_geometry(const NRGeom &g, int d, int &dir, int &i, int &j, int &k) {
  const int n = g.n;
  if (d < g.NE) {
    dir = d / g.NEx;
    const int t = d % g.NEx;
    if (dir == 0) {
      i = t % n; j = (t / n) % (n + 1); k = t / (n * (n + 1));
      return j == 0 || j == n || k == 0 || k == n;
    }
    if (dir == 1) {
      i = t % (n + 1); j = (t / (n + 1)) % n; k = t / ((n + 1) * n);
      return i == 0 || i == n || k == 0 || k == n;
    }
    i = t % (n + 1); j = (t / (n + 1)) % (n + 1); k = t / ((n + 1) * (n + 1));
    return i == 0 || i == n || j == 0 || j == n;
  }
  const int fidx = d - g.NE;
  dir = 3 + fidx / g.NFx;
  const int t = fidx % g.NFx;
  if (dir == 3) {
    i = t % (n + 1); j = (t / (n + 1)) % n; k = t / ((n + 1) * n);
    return i == 0 || i == n;
  }
  if (dir == 4) {
    i = t % n; j = (t / n) % (n + 1); k = t / (n * (n + 1));
    return j == 0 || j == n;
  }
  i = t % n; j = (t / n) % n; k = t / (n * n);
  return k == 0 || k == n;
}

// DoF value of coarse basis b (the reference's BasisNedelec / BasisRaviartThomas,
// include/functions/basis_nedelec.tpp:38-85, basis_raviart_thomas.tpp:38-88, on
// an axis-aligned coarse box): line integral along the fine edge / flux
// through the fine face, exact since the coarse spaces nest in the fine ones.
__device__ inline double coarse_dof(int b, int dir, int i, int j, int k, int n) {
  if (b < 12) {
    // GeometryInfo<3> lines: (direction, position along the two other axes)
    const int ld[12] = {1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 2, 2};
    const int lp[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
    const int lq[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1};
    if (dir != ld[b]) return 0.0;
    const int t1 = dir == 0 ? j : i;
    const int t2 = dir == 2 ? j : k;
    return psi(lp[b], (double)t1 / n) * psi(lq[b], (double)t2 / n) / n;
  }
  const int fd = (b - 12) >> 1, fa = (b - 12) & 1;
  if (dir != 3 + fd) return 0.0;
  const int pos = fd == 0 ? i : (fd == 1 ? j : k);
  return psi(fa, (double)pos / n) / ((double)n * n);
}

// (v_f, curl N_b) for the 6 local faces of fine cell (i,j,k): the curl
// right-hand side of an edge basis (full_rhs, ned_rt_basis.cc:502-511),
// curl N_b as in BasisNedelecCurl (basis_nedelec_curl.tpp:106-147).
__device__ inline void curl_rhs_cell(int b, int i, int j, int k, int n, const double h[3], double (&out)[6]) {
  const int ld[12] = {1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 2, 2};
  const int lp[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
  const int lq[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1};
  const int d = ld[b], p = lp[b], q = lq[b];
  const double Hx = h[0] * n, Hy = h[1] * n, Hz = h[2] * n;
  const double gq = 0.5 / sqrt(3.0);
  const double qp[2] = {0.5 - gq, 0.5 + gq};
  const double jxw = 0.125 * h[0] * h[1] * h[2];
  for (int t = 0; t < 6; ++t) out[t] = 0.0;
  for (int qz = 0; qz < 2; ++qz)
    for (int qy = 0; qy < 2; ++qy)
      for (int qx = 0; qx < 2; ++qx) {
        const double X = (i + qp[qx]) / n, Y = (j + qp[qy]) / n, Z = (k + qp[qz]) / n;
        double cx = 0.0, cy = 0.0, cz = 0.0;
        if (d == 0) {
          cy = psi(p, Y) * sgn(q) / (Hx * Hz);
          cz = -sgn(p) * psi(q, Z) / (Hx * Hy);
        } else if (d == 1) {
          cx = -psi(p, X) * sgn(q) / (Hy * Hz);
          cz = sgn(p) * psi(q, Z) / (Hx * Hy);
        } else {
          cx = psi(p, X) * sgn(q) / (Hy * Hz);
          cy = -sgn(p) * psi(q, Y) / (Hx * Hz);
        }
        const double xl = qp[qx], yl = qp[qy], zl = qp[qz];
        out[0] += jxw * (1.0 - xl) / (h[1] * h[2]) * cx;
        out[1] += jxw * xl / (h[1] * h[2]) * cx;
        out[2] += jxw * (1.0 - yl) / (h[0] * h[2]) * cy;
        out[3] += jxw * yl / (h[0] * h[2]) * cy;
        out[4] += jxw * (1.0 - zl) / (h[0] * h[1]) * cz;
        out[5] += jxw * zl / (h[0] * h[1]) * cz;
      }
}

template <typename TA>
__device__ __forceinline__ void make_factors(const double h[3], NRFactors<TA> &F) {
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    int o1, o2;
    other_axes(p, o1, o2);
    F.hd[p] = (TA)(h[o1] * h[o2] / (36.0 * h[p]));
    F.hq[p] = (TA)(h[p] / 24.0);
#pragma unroll
    for (int fd = 0; fd < 3; ++fd) {
      const int t = 3 - p - fd;
      const double eps = fd == (p + 1) % 3 ? 1.0 : -1.0;
      F.cf[p][fd] = fd == p ? TA(0) : (TA)(eps * h[fd] / (6.0 * h[p] * h[t]));
    }
  }
}

// Element operator of one fine cell, out += A_e z_e (18 DoFs, atomically),
// in tensor-product form instead of tables: the edge-mass block (p, q) is
// A^-1_pq times the 1D P1 mass m = [2 1; 1 2] / 6 along every axis the two
// edge directions share (and the cell length along the others: for p == q a
// Kronecker product m (x) m, for p != q one factor m along the third axis r);
// the curl block couples edges of direction p with faces of normal fd != p
// through m along fd and a -+1 difference along the remaining axis t; the
// div-div block is B/|K| times the outer product of the face signs. Equal to
// table_G / table_C contracted with z. MASK: 0 none, 1 keep only
// lattice-boundary values of z (lift of the Dirichlet data), 2 keep only edge
// values, 3 keep only face values. With DOT set returns
// sum_d S_d z_d (A_e z_e)_d, S = +1 on edges and -1 on faces.
// MERGE: the warp holds complete x-rows of consecutive cells c (n >= 4, all
// lanes active): contributions to the DoFs a cell shares with its x-neighbour
// (the 5 on the plane between them) and then with its y-neighbour in the warp
// (4 on the plane between the rows) are summed by shuffles before the shared-
// memory atomics, ~9.6 atomics per cell instead of 18.
template <typename TA, typename TV, typename TO, int MASK, bool DOT, bool MERGE = false>
__device__ __forceinline__ TA cell_apply_s(const TV *__restrict__ z, TO *out, const NRFactors<TA> &F,
                                           const TA (&ai)[6], TA bdv, const int (&e)[12], const int (&f)[6],
                                           const bool (&eb)[12], const bool (&fb)[6], int c = 0, int L = 0) {
  TA ze[12], zf[6];
#pragma unroll
  for (int l = 0; l < 12; ++l) {
    const bool keep = MASK == 0 || (MASK == 1 && eb[l]) || MASK == 2;
    ze[l] = keep ? (TA)z[e[l]] : TA(0);
  }
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const bool keep = MASK == 0 || (MASK == 1 && fb[t]) || MASK == 3;
    zf[t] = keep ? (TA)z[f[t]] : TA(0);
  }
  const TA A[3][3] = {{ai[0], ai[3], ai[4]}, {ai[3], ai[1], ai[5]}, {ai[4], ai[5], ai[2]}};
  TA ye[12], yf[6];
  // diagonal blocks: m along both other axes (bit 0 and bit 1 of l)
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const TA k = A[p][p] * F.hd[p];
    TA t[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) t[l] = TA(2) * ze[4 * p + l] + ze[4 * p + (l ^ 1)];
#pragma unroll
    for (int l = 0; l < 4; ++l) ye[4 * p + l] = k * (TA(2) * t[l] + t[l ^ 2]);
  }
  // off-diagonal blocks: m along the shared axis r, edge-length integrals elsewhere
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (q == p) continue;
      const int r = 3 - p - q;
      TA s0 = TA(0), s1 = TA(0);
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        if (edge_pos(q, m, r))
          s1 += ze[4 * q + m];
        else
          s0 += ze[4 * q + m];
      }
      const TA k = A[p][q] * F.hq[r];
      const TA u0 = TA(2) * s0 + s1, u1 = s0 + TA(2) * s1;
#pragma unroll
      for (int l = 0; l < 4; ++l) ye[4 * p + l] += k * (edge_pos(p, l, r) ? u1 : u0);
    }
  // div-div
  const TA bd = bdv * ((zf[1] - zf[0]) + (zf[3] - zf[2]) + (zf[5] - zf[4]));
#pragma unroll
  for (int t = 0; t < 6; ++t) yf[t] = (t & 1) ? bd : -bd;
  // curl coupling: edge rows get -C z_f, face rows +C^T z_e
  TA wf[3][2];
#pragma unroll
  for (int fd = 0; fd < 3; ++fd) {
    wf[fd][0] = TA(2) * zf[2 * fd] + zf[2 * fd + 1];
    wf[fd][1] = zf[2 * fd] + TA(2) * zf[2 * fd + 1];
  }
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int fd = 0; fd < 3; ++fd) {
      if (fd == p) continue;
      const int t3 = 3 - p - fd;
      const TA fac = F.cf[p][fd];
      TA u0 = TA(0), u1 = TA(0);
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        const bool up = edge_pos(p, l, t3);
        const TA w = wf[fd][edge_pos(p, l, fd)];
        ye[4 * p + l] += up ? -fac * w : fac * w;
        const TA zv = up ? ze[4 * p + l] : -ze[4 * p + l];
        if (edge_pos(p, l, fd))
          u1 += zv;
        else
          u0 += zv;
      }
      yf[2 * fd] += fac * (TA(2) * u0 + u1);
      yf[2 * fd + 1] += fac * (u0 + TA(2) * u1);
    }
  TA dot = TA(0);
  if constexpr (DOT) {
#pragma unroll
    for (int l = 0; l < 12; ++l) dot += ze[l] * ye[l];
#pragma unroll
    for (int t = 0; t < 6; ++t) dot -= zf[t] * yf[t];
  }
  if constexpr (MERGE) {
    const int n = 1 << L, lane = threadIdx.x & 31;
    const int i = c & (n - 1), j = (c >> L) & (n - 1);
    // plane x = i (fx, ey(k), ey(k+1), ez(j), ez(j+1)) and the same DoFs of plane x = i+1
    TA lf[5] = {yf[0], ye[4], ye[6], ye[8], ye[10]};
    const TA rt[5] = {yf[1], ye[5], ye[7], ye[9], ye[11]};
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      const TA v = __shfl_up_sync(0xffffffffu, rt[t], 1);
      if (i > 0) lf[t] += v;
    }
    if (i == n - 1) {
      atomicAdd(out + f[1], (TO)rt[0]);
      atomicAdd(out + e[5], (TO)rt[1]);
      atomicAdd(out + e[7], (TO)rt[2]);
      atomicAdd(out + e[9], (TO)rt[3]);
      atomicAdd(out + e[11], (TO)rt[4]);
    }
    atomicAdd(out + f[0], (TO)lf[0]);
    atomicAdd(out + e[4], (TO)lf[1]);
    atomicAdd(out + e[6], (TO)lf[2]);
    // plane y = j (ex(k), ex(k+1), fy, ez(i)) and the same DoFs of plane y = j+1
    TA bt[4] = {ye[0], ye[2], yf[2], lf[3]};
    const TA tp[4] = {ye[1], ye[3], yf[3], lf[4]};
    const bool below = lane >= n && j > 0;     // cell (i, j-1, k) sits n lanes down in this warp
    const bool above = lane + n < 32 && j < n - 1;  // cell (i, j+1, k) takes this cell's top set
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const TA v = __shfl_up_sync(0xffffffffu, tp[t], n);
      if (below) bt[t] += v;
    }
    if (!above) {
      atomicAdd(out + e[1], (TO)tp[0]);
      atomicAdd(out + e[3], (TO)tp[1]);
      atomicAdd(out + f[3], (TO)tp[2]);
      atomicAdd(out + e[10], (TO)tp[3]);
    }
    atomicAdd(out + e[0], (TO)bt[0]);
    atomicAdd(out + e[2], (TO)bt[1]);
    atomicAdd(out + f[2], (TO)bt[2]);
    atomicAdd(out + e[8], (TO)bt[3]);
    atomicAdd(out + f[4], (TO)yf[4]);
    atomicAdd(out + f[5], (TO)yf[5]);
  } else {
#pragma unroll
    for (int l = 0; l < 12; ++l) atomicAdd(out + e[l], (TO)ye[l]);
#pragma unroll
    for (int t = 0; t < 6; ++t) atomicAdd(out + f[t], (TO)yf[t]);
  }
  return dot;
}

// Warp-reduce v and store the warp's partial in slot set `slot`; the block
// total is read with slot_total after the next __syncthreads.
// Accumulate a cell's 12 edge contributions y into out with the apply's warp
// merge (full warps of complete x-rows, n >= 4): the 4 edges on the plane
// x = i are summed with the left neighbour's right-plane values by a shuffle,
// then the x-edges and the z-edge of the plane y = j with the row below's
// top values; each shared edge is written once per warp. ~6.5 atomics per
// cell instead of 12.
template <typename TA, typename TO>
__device__ __forceinline__ void edge_scatter_merged(TO *out, const TA (&y)[12], const int (&e)[12], int c, int L) {
  const int n = 1 << L, lane = threadIdx.x & 31;
  const int i = c & (n - 1), j = (c >> L) & (n - 1);
  TA lf[4] = {y[4], y[6], y[8], y[10]};  // plane x = i: ey(k), ey(k+1), ez(j), ez(j+1)
  const TA rt[4] = {y[5], y[7], y[9], y[11]};
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const TA v = __shfl_up_sync(0xffffffffu, rt[t], 1);
    if (i > 0) lf[t] += v;
  }
  if (i == n - 1) {
    atomicAdd(out + e[5], (TO)rt[0]);
    atomicAdd(out + e[7], (TO)rt[1]);
    atomicAdd(out + e[9], (TO)rt[2]);
    atomicAdd(out + e[11], (TO)rt[3]);
  }
  atomicAdd(out + e[4], (TO)lf[0]);
  atomicAdd(out + e[6], (TO)lf[1]);
  // plane y = j: ex(k), ex(k+1), ez(i) and the same edges of plane y = j+1
  TA bt[3] = {y[0], y[2], lf[2]};
  const TA tp[3] = {y[1], y[3], lf[3]};
  const bool below = lane >= n && j > 0;
  const bool above = lane + n < 32 && j < n - 1;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const TA v = __shfl_up_sync(0xffffffffu, tp[t], n);
    if (below) bt[t] += v;
  }
  if (!above) {
    atomicAdd(out + e[1], (TO)tp[0]);
    atomicAdd(out + e[3], (TO)tp[1]);
    atomicAdd(out + e[10], (TO)tp[2]);
  }
  atomicAdd(out + e[0], (TO)bt[0]);
  atomicAdd(out + e[2], (TO)bt[1]);
  atomicAdd(out + e[8], (TO)bt[2]);
}

template <typename VT>
__device__ __forceinline__ void warp_publish(NRShared &sh, int slot, VT v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) {
    if constexpr (sizeof(VT) == 4)
      sh.fslot[slot][threadIdx.x >> 5] = v;
    else
      sh.dslot[slot][threadIdx.x >> 5] = v;
  }
}

// Same summation order in every thread: identical decisions block-wide.
template <typename VT, int NW>
__device__ __forceinline__ VT slot_total(const NRShared &sh, int slot) {
  if constexpr (sizeof(VT) == 4) {  // NW partials: 16-byte loads, pairwise sums
    static_assert(NW == 16 || NW == 8, "slot_total reads 8 or 16 float partials");
    const float4 *p = reinterpret_cast<const float4 *>(sh.fslot[slot]);
    const float4 a = p[0], b = p[1];
    const float s8 = ((a.x + a.y) + (a.z + a.w)) + ((b.x + b.y) + (b.z + b.w));
    if constexpr (NW == 8) {
      return s8;
    } else {
      const float4 c = p[2], d = p[3];
      return s8 + (((c.x + c.y) + (c.z + c.w)) + ((d.x + d.y) + (d.z + d.w)));
    }
  } else {
    VT s = VT(0);
#pragma unroll
    for (int w = 0; w < NW; ++w) s += sh.dslot[slot][w];
    return s;
  }
}

template <typename VT, int NV, int NW>
__device__ __forceinline__ void block_sum(NRShared &sh, VT (&v)[NV], VT (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < NV; ++t) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v[t] += __shfl_xor_sync(0xffffffffu, v[t], off);
  }
  __syncthreads();  // previous readers of the slots are done
  if (lane == 0)
#pragma unroll
    for (int t = 0; t < NV; ++t) {
      if constexpr (sizeof(VT) == 4)
        sh.fred[warp][t] = v[t];
      else
        sh.wred[warp][t] = v[t];
    }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < NV; ++t) {
    VT s = VT(0);
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      if constexpr (sizeof(VT) == 4)
        s += sh.fred[w][t];
      else
        s += sh.wred[w][t];
    }
    out[t] = s;
  }
}

// ---------------- multilevel (BPX) preconditioner of the face block ----------------
// z = P v on the faces is diag^-1 v + sum over the levels m = n/2, ..., 2 of
// P_m X_m P_m^T v: X_m the inverse diagonal of the Galerkin operator
// P_m^T S P_m (levels n/2 .. 4) or its exact inverse (level 2, 12 functions),
// S = D + C^T diag(M)^-1 C the Schur complement with M lumped. The level
// functions nest (index map in nedrt_common.cuh): a level-m function is
// the sum of the level-2m functions at planes 2P-1, 2P, 2P+1 of its four
// child patches, weights 1/8, 1/4, 1/8; a fine face (level n, planes 0..n)
// maps to level n/2 by the same rule. The products are evaluated as a
// restriction cascade, an exact 12 x 12 solve and a prolongation cascade.

__device__ __forceinline__ int ml_index(int lm, int d, int P, int a, int b) {
  const int m = 1 << lm;
  return ((d * (m - 1) + P - 1) << (2 * lm)) + (b << lm) + a;
}

// Parents of the level-2m (or fine) function / face (d, p, x, y) at level m = 2^lm.
__device__ __forceinline__ int ml_parents(int lm, int d, int p, int x, int y, int (&j)[2], float (&w)[2]) {
  const int m = 1 << lm;
  const int a = x >> 1, b = y >> 1;
  int cnt = 0;
  if (!(p & 1)) {
    const int P = p >> 1;
    if (P >= 1 && P <= m - 1) {
      j[0] = ml_index(lm, d, P, a, b);
      w[0] = 0.25f;
      cnt = 1;
    }
  } else {
    const int P0 = p >> 1;
    if (P0 >= 1) {
      j[cnt] = ml_index(lm, d, P0, a, b);
      w[cnt++] = 0.125f;
    }
    if (P0 + 1 <= m - 1) {
      j[cnt] = ml_index(lm, d, P0 + 1, a, b);
      w[cnt++] = 0.125f;
    }
  }
  return cnt;
}

// 16-bit code of a fine face's level-n/2 parents: bits 0-11 the first parent,
// bit 12 first valid, bit 13 second valid (first + m^2), bit 14 odd plane
// (weights 1/8, else 1/4).
__device__ __forceinline__ unsigned short ml_code(int lm, int d, int p, int x, int y) {
  int j[2];
  float w[2];
  const int cnt = ml_parents(lm, d, p, x, y, j, w);
  if (cnt == 0) return 0;
  return (unsigned short)(j[0] | 0x1000 | (cnt == 2 ? 0x2000 : 0) | ((p & 1) ? 0x4000 : 0));
}

template <typename T>
__device__ __forceinline__ T ml_code_prolong(unsigned code, const T *y, int m2) {
  if (!(code & 0x1000u)) return T(0);
  const int j = code & 0xFFF;
  T s = y[j];
  if (code & 0x2000u) s += y[j + m2];
  return s * ((code & 0x4000u) ? T(0.125) : T(0.25));
}

// (d, P, a, b) of function J of level 2^lm.
__device__ __forceinline__ void ml_decode(int lm, int J, int &d, int &P, int &a, int &b) {
  const int m = 1 << lm;
  const int per = (m - 1) << (2 * lm);
  d = (J >= per) + (J >= 2 * per);
  const int rem = J - d * per;
  P = (rem >> (2 * lm)) + 1;
  b = (rem >> lm) & (m - 1);
  a = rem & (m - 1);
}

// Restriction of a level-2^lmc vector to function J of level 2^(lmc-1).
template <typename T>
__device__ __forceinline__ T ml_restrict_one(const T *rc, int lmc, int J) {
  int d, P, a, b;
  ml_decode(lmc - 1, J, d, P, a, b);
  T s = T(0);
#pragma unroll
  for (int q = -1; q <= 1; ++q) {
    const T w = q == 0 ? T(0.25) : T(0.125);
#pragma unroll
    for (int yy = 0; yy < 2; ++yy)
#pragma unroll
      for (int xx = 0; xx < 2; ++xx) s += w * rc[ml_index(lmc, d, 2 * P + q, 2 * a + xx, 2 * b + yy)];
  }
  return s;
}

// Fine face DoF of normal d at plane p, transverse position (x, y).
__device__ __forceinline__ int face_dof(const NRGeom &g, int d, int p, int x, int y) {
  const int n = g.n;
  if (d == 0) return g.NE + p + (n + 1) * (x + n * y);
  if (d == 1) return g.NE + g.NFx + x + n * (p + (n + 1) * y);
  return g.NE + 2 * g.NFx + x + n * (y + n * p);
}

template <typename VT>
__device__ __forceinline__ void warp_publish(NRShared &sh, int slot, VT v);
template <typename VT, int NW>
__device__ __forceinline__ VT slot_total(const NRShared &sh, int slot);

// Coarse part of z = P v, all threads of the block, K = L - 1 coarse levels
// (k = 1..K with 2^(L-k) cells per side; level K is level 2): the level-n/2
// restriction of the face part of v (a gather, one thread per function; at
// K == 2 also the level-2 restriction, by 12-target atomics), the restrictions
// of the levels below (K == 3), the exact level-2 solve in every warp (lanes
// 0..11, kept in a register), the prolongations with the diagonal terms (the
// level above level 2 reads its parents by shuffles); writes the level-n/2
// coefficients y1 (the fine prolongation is left to the caller) and returns
// the coarse share of gamma^2 = v^T (P - diag^-1) v, identical in every
// thread. Barriers: 2 at K <= 2, 4 at K == 3. wk: the vectors of the levels
// below n/2; dat: inverse diagonals and the level-2 inverse; lc: parent codes
// of the level n/2 .. 4 functions one level down.
template <typename T, int NW, int K>
__device__ T ml_coarse_block(NRShared &sh, const NRGeom &g, const T *vsrc, T *r1, T *y1, T *wk, const float *dat,
                             const unsigned short *lc) {
  constexpr int NT = NW * 32;
  constexpr int L = K + 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T *rk[K + 1], *yk[K + 1];
  const float *dk[K + 1];
  int oc[K + 1];
  rk[1] = r1;
  yk[1] = y1;
  int ow = 0, od = 0;
  oc[1] = 0;
#pragma unroll
  for (int k = 1; k <= K; ++k) {
    const int F = nr_ml_count(1 << (L - k));
    if (k >= 2) {
      rk[k] = wk + ow;
      yk[k] = wk + ow + F;
      ow += 2 * F;
      oc[k] = oc[k - 1] + nr_ml_count(1 << (L - k + 1));
    }
    if (k < K) {
      dk[k] = dat + od;
      od += F;
    }
  }
  const float *S2 = dat + od;
  T part = T(0);
  {  // fine -> level n/2: planes 2P-1, 2P, 2P+1 (weights 1/8, 1/4, 1/8) of the 2 x 2 child patches
    constexpr int lm = L - 1;
    const int F = nr_ml_count(1 << lm), n = g.n;
    for (int j = tid; j < F; j += NT) {
      int d, P, a, b;
      ml_decode(lm, j, d, P, a, b);
      // DoF strides along the normal and the two transverse axes of a face family
      const int ps = d == 0 ? 1 : (d == 1 ? n : n * n);
      const int xs = d == 0 ? n + 1 : 1;
      const int ys = d == 0 ? (n + 1) * n : (d == 1 ? n * (n + 1) : n);
      const T *v0 = vsrc + face_dof(g, d, 2 * P - 1, 2 * a, 2 * b);
      T s = T(0);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const T *vq = v0 + q * ps;
        s += (q == 1 ? T(0.25) : T(0.125)) * ((vq[0] + vq[xs]) + (vq[ys] + vq[xs + ys]));
      }
      r1[j] = s;
      if constexpr (K > 1) part += s * (T)dk[1][j] * s;
      if constexpr (K == 2) {  // level-2 restriction accumulated here (12 targets)
        int jj[2];
        float ww[2];
        const int cnt = ml_parents(lm - 1, d, P, a, b, jj, ww);
        for (int t = 0; t < cnt; ++t) atomicAdd(rk[2] + jj[t], (T)ww[t] * s);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 2; k < K; ++k) {  // the diagonal levels below n/2 (K == 3: level 4)
    const int F = nr_ml_count(1 << (L - k));
    for (int J = tid; J < F; J += NT) {
      const T r = ml_restrict_one(rk[k - 1], L - k + 1, J);
      rk[k][J] = r;
      part += r * (T)dk[k][J] * r;
      if (k + 1 == K) {
        int d, P, a, b, jj[2];
        float ww[2];
        ml_decode(L - k, J, d, P, a, b);
        const int cnt = ml_parents(L - k - 1, d, P, a, b, jj, ww);
        for (int t = 0; t < cnt; ++t) atomicAdd(rk[K] + jj[t], (T)ww[t] * r);
      }
    }
    __syncthreads();
  }
  // level 2, exact, in every warp: lane q < 12 holds y_K[q]
  T yK = T(0), rme = T(0);
  if (lane < 12) {
#pragma unroll
    for (int q = 0; q < 12; ++q) yK += (T)S2[lane * 12 + q] * rk[K][q];
    rme = rk[K][lane];
  }
  if (tid < 12) part += rme * yK;  // counted once
  if constexpr (K == 1) {
    if (tid < 12) y1[tid] = yK;
    warp_publish<T>(sh, 2, part);
    __syncthreads();
    return slot_total<T, NW>(sh, 2);
  } else {
    {  // level K-1 from the register y_K (warp-uniform trip count: every lane takes part in the shuffles)
      constexpr int k = K - 1;
      const int F = nr_ml_count(1 << (L - k));
      for (int base = warp * 32; base < F; base += NT) {
        const int j = base + lane;
        const bool ok = j < F;
        const unsigned code = ok ? lc[oc[k] + j] : 0u;
        const int j0 = code & 0xFFF, j1 = j0 + 4;  // level 2: 4 functions per plane
        const T a0 = __shfl_sync(0xffffffffu, yK, j0 & 31);
        const T a1 = __shfl_sync(0xffffffffu, yK, j1 & 31);
        if (ok) {
          T pr = T(0);
          if (code & 0x1000u) pr = a0 + ((code & 0x2000u) ? a1 : T(0));
          pr *= (code & 0x4000u) ? T(0.125) : T(0.25);
          yk[k][j] = (T)dk[k][j] * rk[k][j] + pr;
        }
      }
      if (k == 1) warp_publish<T>(sh, 2, part);
      __syncthreads();
    }
#pragma unroll
    for (int k = K - 2; k >= 1; --k) {  // the levels above, from shared memory
      const int F = nr_ml_count(1 << (L - k));
      const int mp2 = 1 << (2 * (L - k - 1));
      for (int j = tid; j < F; j += NT)
        yk[k][j] = (T)dk[k][j] * rk[k][j] + ml_code_prolong(lc[oc[k] + j], yk[k + 1], mp2);
      if (k == 1) warp_publish<T>(sh, 2, part);
      __syncthreads();
    }
    if (tid < 12) rk[K][tid] = T(0);  // every warp has read it; the next accumulation is barriers away
    return slot_total<T, NW>(sh, 2);
  }
}

// Dispatch on the cell's depth (2..4).
template <typename T, int NW>
__device__ __forceinline__ T ml_coarse(NRShared &sh, const NRGeom &g, const T *vsrc, T *r1, T *y1, T *wk,
                                       const float *dat, const unsigned short *lc) {
  if (g.L == 2) return ml_coarse_block<T, NW, 1>(sh, g, vsrc, r1, y1, wk, dat, lc);
  if (g.L == 3) return ml_coarse_block<T, NW, 2>(sh, g, vsrc, r1, y1, wk, dat, lc);
  return ml_coarse_block<T, NW, 3>(sh, g, vsrc, r1, y1, wk, dat, lc);
}

extern __shared__ __align__(256) unsigned char nr_dyn_smem[];

// Edge l (direction p = l / 4, position l4 = l % 4, as in cell_dofs) of fine
// cell (ci, cj, ck) as its grid line: direction p through lattice point
// (x, y, z), i.e. the edge from (x, y, z) to (x, y, z) + unit_p.
__device__ __forceinline__ void nr_edge_line(int l, int ci, int cj, int ck, int &x, int &y, int &z) {
  const int p = l >> 2, a = l & 1, b = (l >> 1) & 1;
  x = ci + (p == 0 ? 0 : a);
  y = cj + (p == 1 ? 0 : (p == 0 ? a : b));
  z = ck + (p == 2 ? 0 : b);
}
// Position (0..3) of the grid line (p, x, y, z) among fine cell (ci, cj, ck)'s
// edges of direction p, or -1 when the cell does not have it.
__device__ __forceinline__ int nr_edge_pos_in(int p, int x, int y, int z, int ci, int cj, int ck) {
  const int dx = x - ci, dy = y - cj, dz = z - ck;
  if (p == 0) return (dx == 0 && (dy | dz) >= 0 && dy <= 1 && dz <= 1) ? dy + 2 * dz : -1;
  if (p == 1) return (dy == 0 && (dx | dz) >= 0 && dx <= 1 && dz <= 1) ? dx + 2 * dz : -1;
  return (dz == 0 && (dx | dy) >= 0 && dx <= 1 && dy <= 1) ? dx + 2 * dy : -1;
}
// A^-1_pq from a cell's float coefficients (a00 a11 a22 a01 a02 a12).
__device__ __forceinline__ float nr_ainv_pq(const float *a, int p, int q) {
  return p == q ? a[p] : a[p + q + 2];  // (0,1) -> 3, (0,2) -> 4, (1,2) -> 5
}

// Block-Jacobi part of the preconditioner of one cell into pd[0, Np): diag(M)^-1
// on the edges and, on the faces, the inverse of the lumped Schur diagonal
// D_ff + sum_l C_lf^2 / M_ll (cell-local approximation) or, where the
// multilevel setup assembled it (ml_fine: one value per face, 0 on the
// boundary), the inverse assembled Schur diagonal; 0 on Dirichlet DoFs
// (natural: every DoF kept) and on the pad [N, Np). cf: the cell's float
// coefficients (8 per fine cell), written by this block before the call.
// Block-wide (NT threads, ends with a barrier); uses the closed-form element
// tables in sh.
template <int NT>
__device__ void nr_precond_diag(const NRGeom &g, const NRCell &Cc, const float *cf, float *pd, int Np,
                                NRShared &sh, bool natural, const float *ml_fine) {
  const int tid = threadIdx.x, nc = g.n * g.n * g.n;
  for (int t = tid; t < 144 + 72; t += NT) {
    if (t < 144) {
      const int p = t / 48, q = (t / 16) % 3, l4 = (t / 4) % 4, m4 = t % 4;
      sh.Gf[p][q][l4][m4] = (float)table_G(Cc.h, p, q, l4, m4);
    } else {
      const int u = t - 144, l = u / 6, f = u % 6;
      sh.Cf[l][f] = (float)table_C(Cc.h, l, f);
    }
  }
  for (int d = tid; d < Np; d += NT) pd[d] = 0.0f;  // pad [N, Np) stays 0
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int e[12], f[6];
    cell_dofs(g, c, e, f);
    const float *a = cf + 8 * c;
    const float Ad[3] = {a[0], a[1], a[2]};
#pragma unroll
    for (int l = 0; l < 12; ++l) atomicAdd(pd + e[l], Ad[l >> 2] * sh.Gf[l >> 2][l >> 2][l & 3][l & 3]);
  }
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int e[12], f[6];
    cell_dofs(g, c, e, f);
    const float bdv = cf[8 * c + 6];
    float me[12];
#pragma unroll
    for (int l = 0; l < 12; ++l) me[l] = pd[e[l]];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      float s = bdv;
#pragma unroll
      for (int l = 0; l < 12; ++l) s += sh.Cf[l][t] * sh.Cf[l][t] / me[l];
      atomicAdd(pd + f[t], s);
    }
  }
  __syncthreads();
  for (int d = tid; d < g.N; d += NT) {
    int dir, i, j, k;
    const bool bnd = dof_geometry(g, d, dir, i, j, k);
    pd[d] = (bnd && !natural) ? 0.0f : 1.0f / pd[d];
  }
  __syncthreads();
  if (ml_fine) {  // the inverse assembled diagonal of S replaces the cell-lumped one on the faces
    for (int u = tid; u < g.NF; u += NT)
      if (pd[g.NE + u] > 0.0f) pd[g.NE + u] = ml_fine[u];
    __syncthreads();
  }
}

// Float coefficients of one cell, 8 per fine cell (A^-1: 6, B / |K|, pad),
// from the FP64 inputs. Block-wide, no barrier.
template <int NT>
__device__ __forceinline__ void nr_float_coefficients(const double *ag, const double *bg, int nc, double invV,
                                                      float *cf) {
  for (int c = threadIdx.x; c < nc; c += NT) {
#pragma unroll
    for (int q = 0; q < 6; ++q) cf[8 * c + q] = (float)ag[6 * (size_t)c + q];
    cf[8 * c + 6] = (float)(bg[c] * invV);
    cf[8 * c + 7] = 0.0f;
  }
}

// One (cell, basis) item. SMEM: the workspace is the dynamic shared memory
// (known at compile time, so every vector access is a shared-memory access),
// otherwise this CTA's slot of the global scratch.
// STAGE (global workspace, mixed precision): the apply reads each warp's 32
// cells of coefficients from shared memory, where a bulk copy issued two rounds
// earlier put them.
// ZSH (global workspace with prep, mixed precision): z~ lives in the dynamic
// shared memory at NRParams::zt_offset, so the apply's 18 gathers per fine
// cell and the patch pass's atomics stay on the SM.
template <typename T, bool SMEM, int NT, bool ML, bool STAGE = false, bool ZSH = false>
__device__ void solve_item(const NRParams &prm, NRShared &sh, int item_id) {
  static_assert(!ZSH || (sizeof(T) == 4 && !SMEM && !STAGE), "z~ in shared memory: mixed, global workspace");
  // NT = 256 with the shared workspace (two CTAs per SM, mixed precision):
  // the correction x and the float coefficients live in this CTA's global
  // slot so that the shared part (preconditioner + 6 vectors) fits twice per
  // SM. NT = 256 with the global workspace keeps the 512-thread layout.
  constexpr bool kSplitWs = NT == 256 && SMEM;
  constexpr int NW = NT / 32;
  float *ws = SMEM ? reinterpret_cast<float *>(nr_dyn_smem) : prm.scratch + (size_t)blockIdx.x * prm.scratch_floats;
  const NRItem it = prm.items[item_id];
  const NRCell Cc = prm.cells[it.cell];
  NRGeom g;
  g.n = Cc.n;
  g.L = Cc.depth;
  nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
  g.N = g.NE + g.NF;
  const int n = g.n, N = g.N;
  const int nc = n * n * n;
  const int bb = it.basis;
  const bool src = it.mode >= 1;
  const bool natural = it.mode == 2;  // every DoF free (no Dirichlet rows)
  const bool merge = n >= 4;  // full warps of complete x-rows in the apply (block-uniform)
  const int tid = threadIdx.x;
  constexpr bool kMixed = sizeof(T) == 4;
  const double invV = 1.0 / (Cc.h[0] * Cc.h[1] * Cc.h[2]);
  const size_t Np = ((size_t)N + 63) / 64 * 64;
  // workspace carve (floats). zt: P v~_j (unnormalised), operand of the apply;
  // az: the apply's accumulation vector (diagonal path); vA, vB: unnormalised
  // Lanczos vectors v~_j, v~_{j-1}, wA, wB: MINRES directions w_{j-1}, w_j
  // (roles swap); xk: the correction; dacc: the FP64 residual accumulator
  // (Np doubles over two vectors that are free while it is live).
  // prep (global workspace with NRParams::prep): the preconditioner diagonal
  // and the float coefficients are the cell's shared copy, and the slot holds
  // zt, vA, vB, wA, wB, xk, then az (present only when the host sized the slot
  // for the diagonal path).
  const bool prep = ZSH || (!SMEM && prm.prep != nullptr);  // ZSH: z~ is a shared-memory pointer only
  float *gws = prm.scratch + (size_t)blockIdx.x * prm.scratch_floats;  // split workspace only
  float *pd, *cf;
  T *zt, *az, *vA, *vB, *wA, *wB, *xk;
  double *dacc;
  if (prep) {
    pd = prm.prep + Cc.prep_off;
    cf = pd + Np;
    // with ZSH the slot's first Np floats are left unused (the host guarantees
    // prep for ZSH launches)
    zt = ZSH ? reinterpret_cast<T *>(nr_dyn_smem + prm.zt_offset) : reinterpret_cast<T *>(ws);
    vA = reinterpret_cast<T *>(ws) + Np;
    vB = vA + Np;
    wA = vB + Np;
    wB = wA + Np;
    xk = wB + Np;
    az = xk + Np;
    dacc = kMixed ? reinterpret_cast<double *>(wA) : reinterpret_cast<double *>(zt);
  } else {
    pd = ws;
    zt = reinterpret_cast<T *>(ws + Np);
    az = zt + Np;
    vA = az + Np;
    vB = vA + Np;
    wA = vB + Np;
    wB = wA + Np;
    xk = kSplitWs ? reinterpret_cast<T *>(gws) : wB + Np;
    cf = kSplitWs ? gws + Np * (sizeof(T) / 4) : ws + Np + 7 * Np * (sizeof(T) / 4);
    dacc = reinterpret_cast<double *>(ws + Np);  // zt and az
  }
  const NRFactors<float> &Ff = sh.Ff;
  const NRFactors<double> &Fd = sh.Fd;
  if (tid == 0) {
    make_factors(Cc.h, sh.Ff);
    make_factors(Cc.h, sh.Fd);
  }
  float *facc = reinterpret_cast<float *>(zt);  // FP32 residual accumulator (first refinement step)
  const double *ag = prm.ainv6 + 6 * Cc.coef_off;
  const double *bg = prm.bdiv + Cc.coef_off;
  double *phi = src ? prm.src_out + kNRSrcRhs * Cc.dof_off + (size_t)bb * N
                    : prm.phi + 18 * Cc.dof_off + (size_t)bb * N;
  const double *fsrc = src ? prm.src_rhs + kNRSrcRhs * Cc.dof_off + (size_t)bb * N : nullptr;
  double *yout = prm.y + 18 * Cc.dof_off + (size_t)bb * N;
  // multilevel face preconditioner for this item (block-uniform switch)
  const bool ml = ML && prm.coarse != nullptr && Cc.coarse_off >= 0 && !natural;

  // ---- block-Jacobi preconditioner and float coefficients (shared copy: built
  // by nr_cell_prep_kernel before the launch)
  if (!prep) {
    nr_float_coefficients<NT>(ag, bg, nc, invV, cf);
    nr_precond_diag<NT>(g, Cc, cf, pd, (int)Np, sh, natural,
                        ml ? prm.coarse + Cc.coarse_off + nr_ml_data_floats(n) : nullptr);
  }
  if constexpr (STAGE) asm volatile("fence.proxy.async.global;" ::: "memory");  // cf is read by bulk copies
  __syncthreads();

  // ---- multilevel part of the preconditioner: the cell's data from HBM, the
  // faces' level-n/2 parent codes
  const NRMLLayout mll = nr_ml_layout(n, (int)sizeof(T));
  unsigned char *mlb = nr_dyn_smem + prm.ml_offset;
  T *ml_rr = reinterpret_cast<T *>(mlb);
  T *ml_y = reinterpret_cast<T *>(mlb + mll.off_y);
  T *ml_wk = reinterpret_cast<T *>(mlb + mll.off_wk);
  float *ml_dat = reinterpret_cast<float *>(mlb + mll.off_data);
  unsigned short *ml_codes = reinterpret_cast<unsigned short *>(mlb + mll.off_codes);
  unsigned short *ml_lcodes = reinterpret_cast<unsigned short *>(mlb + mll.off_lcodes);
  const int m2 = 1 << (2 * (g.L - 1));
  if (ml) {
    const float *src = prm.coarse + Cc.coarse_off;
    const int nd = nr_ml_data_floats(n);
    for (int t = tid; t < nd; t += NT) ml_dat[t] = src[t];
    for (int t = tid; t < mll.F1; t += NT) ml_rr[t] = T(0);
    for (int t = tid; t < (int)((mll.off_data - mll.off_wk) / sizeof(T)); t += NT) ml_wk[t] = T(0);
    for (int u = tid; u < (int)Np - g.NE; u += NT) {
      const int d = g.NE + u;
      unsigned short code = 0;
      if (d < N) {
        int dir, i, j, k;
        dof_geometry(g, d, dir, i, j, k);
        const int fd = dir - 3;
        const int p = fd == 0 ? i : (fd == 1 ? j : k);
        const int x = fd == 0 ? j : i;
        const int y = fd == 2 ? j : k;
        code = ml_code(g.L - 1, fd, p, x, y);
      }
      ml_codes[u] = code;
    }
    for (int k = 1, o = 0; (1 << (g.L - k)) >= 4; o += nr_ml_count(1 << (g.L - k)), ++k) {
      const int lm = g.L - k;
      for (int j = tid; j < nr_ml_count(1 << lm); j += NT) {
        int d, p, x, y;
        ml_decode(lm, j, d, p, x, y);
        ml_lcodes[o + j] = ml_code(lm - 1, d, p, x, y);
      }
    }
    __syncthreads();
  }

  // ---- cell-patch edge preconditioner (shared per-cell data, multilevel items):
  // z_E += sum_c R_c^T X_c R_c v over the fine cells, X_c = L_c^-T L_c^-1 the
  // inverse of the assembled edge mass restricted to cell c's edges (M_c =
  // L_c L_c^T, Dirichlet edges decoupled; v is zero on them), L_c^-1 stored in
  // FP16 pairs, row-packed lower triangle, in 16-byte groups: word t of cell c
  // at pX[(t / 4 * nc + c) * 4 + t % 4].
  // Per cell t = L^-1 v_c, z += L^-T t; returns this thread's share of
  // v_E^T z_E = sum_c |t|^2.
  // Global-workspace items only: compiled out of the shared-memory variants,
  // where the extra pass cost about what the fewer iterations saved (depth 3,
  // 512 cells: 190 ms with it, 189 ms without) and its code slowed the rest.
  const bool epatch = !SMEM && prm.prep != nullptr && prm.edge_patch && ml;
  const __half2 *pX = epatch ? reinterpret_cast<const __half2 *>(prm.prep + Cc.prep_off + nr_prep_patch_offset(n))
                             : nullptr;
  auto patch_pass = [&](const T *vsrc) -> T {
    T qf = T(0);
    for (int c = tid; c < nc; c += NT) {
      int e[12], f[6];
      cell_dofs(g, c, e, f);
      __half2 Lw[40];  // kept packed: half the registers of the unpacked factor
      const uint4 *pX4 = reinterpret_cast<const uint4 *>(pX);
#pragma unroll
      for (int g4 = 0; g4 < 10; ++g4) {  // 16-byte groups of 4 words, coalesced over the warp's cells
        const uint4 q = pX4[(size_t)g4 * nc + c];
        Lw[4 * g4] = *reinterpret_cast<const __half2 *>(&q.x);
        Lw[4 * g4 + 1] = *reinterpret_cast<const __half2 *>(&q.y);
        Lw[4 * g4 + 2] = *reinterpret_cast<const __half2 *>(&q.z);
        Lw[4 * g4 + 3] = *reinterpret_cast<const __half2 *>(&q.w);
      }
      auto Lv = [&](int idx) -> T {
        return (T)((idx & 1) ? __high2float(Lw[idx >> 1]) : __low2float(Lw[idx >> 1]));
      };
      T vl[12], y[12];
#pragma unroll
      for (int l = 0; l < 12; ++l) {
        vl[l] = vsrc[e[l]];
        y[l] = T(0);
      }
      // row l of L^-1 gives t_l, then at once its share t_l L^-1_lm of (L^-T t)_m
#pragma unroll
      for (int l = 0; l < 12; ++l) {
        T a = T(0);
#pragma unroll
        for (int m = 0; m <= l; ++m) a += Lv(l * (l + 1) / 2 + m) * vl[m];
        qf += a * a;
#pragma unroll
        for (int m = 0; m <= l; ++m) y[m] += Lv(l * (l + 1) / 2 + m) * a;
      }
      edge_scatter_merged<T, T>(zt, y, e, c, g.L);  // n >= 4 (multilevel items): full warps of x-rows
    }
    return qf;
  };

  double bnorm2 = 0.0, rnorm2 = 0.0;
  int conv = 0, its = 0, flags = 0, nref = 0;
  static_assert(!STAGE || (sizeof(T) == 4 && !SMEM && NT == 512), "staged apply: mixed, global workspace");

  // Phase-1 apply with the coefficients staged by bulk copies: in round r warp
  // w applies cells r NT + 32 w .. + 31, whose 32 x 8 floats form one
  // contiguous 1 KB tile of cf; the tile of round r + 2 is copied into the
  // stage the warp has just read while it works on round r + 1, so the apply
  // waits on no global coefficient load. Waits are bounded: a copy that never
  // completes flags the item (bit 2) instead of hanging the SM.
  auto staged_apply = [&](float *acc) -> float {
    float dp = 0.0f;
    if constexpr (STAGE) {
      const int warp = tid >> 5, lane = tid & 31;
      const int R = (nc + NT - 1) / NT;
      float4 *stg = reinterpret_cast<float4 *>(nr_dyn_smem + prm.stage_offset) + warp * 128;
      unsigned long long *mb = sh.mbar[warp];
      unsigned tph = sh.tph[warp];
      auto issue = [&](int r, int sidx) {
        const int c0 = r * NT + warp * 32;
        const int cnt = min(32, nc - c0);
        if (cnt > 0) bulk_load(stg + sidx * 64, cf + 8 * (size_t)c0, (unsigned)cnt * 32u, mb + sidx);
      };
      if (lane == 0) {
        issue(0, 0);
        if (R > 1) issue(1, 1);
      }
      for (int r = 0; r < R; ++r) {
        const int sidx = r & 1;
        if (r * NT + warp * 32 < nc) {  // warp-uniform: lane 0 issued this round's tile
          if (!mbar_wait(mb + sidx, (tph >> sidx) & 1u)) {
            flags |= 4;
            mbar_wait(mb + sidx, (tph >> sidx) & 1u);  // once more, still bounded
          }
          tph ^= 1u << sidx;
          const int c = r * NT + tid;
          if (c < nc) {
            const float4 c0 = stg[sidx * 64 + 2 * lane], c1 = stg[sidx * 64 + 2 * lane + 1];
            int e[12], f[6];
            cell_dofs(g, c, e, f);
            const bool eb[12] = {}, fb[6] = {};
            const float ai[6] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
            dp += merge ? cell_apply_s<float, float, float, 0, true, true>(zt, acc, Ff, ai, c1.z, e, f, eb, fb, c, g.L)
                        : cell_apply_s<float, float, float, 0, true>(zt, acc, Ff, ai, c1.z, e, f, eb, fb);
          }
        }
        __syncwarp();
        if (lane == 0 && r + 2 < R) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the warp's reads of this stage are done
          issue(r + 2, sidx);
        }
      }
      if (lane == 0) sh.tph[warp] = tph;
      __syncwarp();
    }
    return dp;
  };

  for (int ir = 0;; ++ir) {
    const bool fp32_res = kMixed && ir == 0;
    // ---------------- residual r = f - A phi on the interior ----------------
    if (ir == 0) {
      // phi0 = coarse function on every DoF (satisfies the boundary data)
      for (int d = tid; d < N; d += NT) {
        int dir, i, j, k;
        dof_geometry(g, d, dir, i, j, k);
        phi[d] = src ? 0.0 : coarse_dof(bb, dir, i, j, k, n);
      }
      __syncthreads();
    }
    double part[3] = {0.0, 0.0, 0.0};
    for (int pass = (ir == 0 ? 0 : 1); pass < 2; ++pass) {
      // pass 0: lift of the boundary data only (scale of the stopping test)
      // accumulator starts at -f for a source item (r = f - A phi)
      if (fp32_res) {
        for (int d = tid; d < N; d += NT) facc[d] = src ? (float)-fsrc[d] : 0.0f;
      } else {
        for (int d = tid; d < N; d += NT) dacc[d] = src ? -fsrc[d] : 0.0;
      }
      __syncthreads();
      for (int c = tid; c < nc; c += NT) {
        int e[12], f[6];
        cell_dofs(g, c, e, f);
        bool eb[12], fb[6];
#pragma unroll
        for (int l = 0; l < 12; ++l) {
          int dir, i, j, k;
          eb[l] = dof_geometry(g, e[l], dir, i, j, k);
        }
#pragma unroll
        for (int t = 0; t < 6; ++t) {
          int dir, i, j, k;
          fb[t] = dof_geometry(g, f[t], dir, i, j, k);
        }
        double rc[6];
        const bool curl_rhs = !src && bb < 12;
        if (curl_rhs) {
          curl_rhs_cell(bb, c % n, (c / n) % n, c / (n * n), n, Cc.h, rc);
        }
        if (fp32_res) {
          const float *a = cf + 8 * c;
          const float ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          if (pass == 0)
            cell_apply_s<float, double, float, 1, false>(phi, facc, Ff, ai, a[6], e, f, eb, fb);
          else
            cell_apply_s<float, double, float, 0, false>(phi, facc, Ff, ai, a[6], e, f, eb, fb);
          if (curl_rhs)
#pragma unroll
            for (int t = 0; t < 6; ++t) atomicAdd(facc + f[t], (float)-rc[t]);
        } else {
          const double *a = ag + 6 * (size_t)c;
          const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          if (pass == 0)
            cell_apply_s<double, double, double, 1, false>(phi, dacc, Fd, ai, bg[c] * invV, e, f, eb, fb);
          else
            cell_apply_s<double, double, double, 0, false>(phi, dacc, Fd, ai, bg[c] * invV, e, f, eb, fb);
          if (curl_rhs)
#pragma unroll
            for (int t = 0; t < 6; ++t) atomicAdd(dacc + f[t], -rc[t]);
        }
      }
      __syncthreads();
      // r = -(A phi - f) on interior DoFs (boundary: 0), kept in vA. Its size is
      // measured in the preconditioner's norm ||r||_P^2 = r^T P r (the norm MINRES
      // minimises): the face rows of the local system outweigh the edge rows by
      // ~(1/h)^2 (div-div ~ h^-3 against edge mass ~ h), so a plain 2-norm would
      // leave the edge block unresolved on small cells; the P-norm is invariant
      // to that block scaling.
      for (int d = tid; d < (int)Np; d += NT) {
        const bool interior = pd[d] > 0.0f;  // false on the pad [N, Np)
        const double r = interior ? -(fp32_res ? (double)facc[d] : dacc[d]) : 0.0;
        part[pass] += (double)pd[d] * r * r;
        if (ir == 0 && pass == 1 && src && prm.src_scale2 && interior)
          part[2] += (double)pd[d] * prm.src_scale2[Cc.dof_off + d];
        // MINRES runs on the symmetric form S A (S = +1 on edges, -1 on faces):
        // [M -C; -C^T -D] x = S r. vA is disjoint from the accumulator.
        if (pass == 1) vA[d] = (T)(d < g.NE ? r : -r);
      }
      __syncthreads();
    }
    {
      double tot[3];
      block_sum<double, 3, NW>(sh, part, tot);
      if (ir == 0) bnorm2 = tot[0];
      // a source right-hand side that cancelled to rounding is solved to rtol of
      // 1e-3 of its cell's adjoint source scale (in the same norm), not of its own
      // noise-level norm
      if (ir == 0 && src) bnorm2 = fmax(bnorm2, 1e-6 * tot[2]);
      rnorm2 = tot[1];
    }
    ++nref;
    conv = !fp32_res && (rnorm2 <= prm.rtol * prm.rtol * bnorm2);
    if (conv || ir >= prm.max_refine) break;

    if (ML && ml) {
      // ---------------- MINRES with the multilevel face preconditioner ----------------
      // The recurrences of the diagonal path below, with z~_j = P v~_j no longer
      // recomputable from v~_j alone: zt holds the full z~_j. The apply
      // accumulates into the slot of v~_{j-1}, which the previous iteration
      // prefilled with -S (gamma_j^2 / g_{j-1}) v~_{j-1}, so that after the apply
      // it holds B = A z~_j + that term and v~_{j+1} = (S B - delta~ v~_j) / g_j
      // is a pointwise update in place (no separate accumulation vector). Each
      // iteration runs three block-wide phases and the coarse step, each ending
      // in barriers:
      //   phase 1: B += A z~_j (into vp), delta~;
      //   phase 2: v~_{j+1} in place of B; gamma^2 partials (fine part);
      //   coarse:  level-n/2 coefficients y of the coarse part of z~_{j+1} and
      //            its share of gamma_{j+1}^2 (ml_coarse_block);
      //   phase 3: w_j from z~_j (still in zt), x += c eta w_j,
      //            zt <- diag^-1 v~_{j+1} + P_{n/2} y (the full z~_{j+1}), and
      //            the prefill of v~_j's slot for the next apply.
      for (int d = tid; d < (int)Np; d += NT) {
        vB[d] = T(0);  // v~_{-1} = 0: the first apply accumulates from zero
        wA[d] = T(0);
        wB[d] = T(0);
        xk[d] = T(0);
      }
      T *vc = vA, *vp = vB;
      T *wo = wA, *wc = wB;
      T gam;
      {
        T p1[1] = {T(0)};
        for (int d = tid; d < (int)Np; d += NT) {
          const T z = (epatch && d < g.NE) ? T(0) : (T)pd[d] * vc[d];  // patch edges: accumulated below
          zt[d] = z;
          p1[0] += z * vc[d];
        }
        if (epatch) {
          __syncthreads();
          p1[0] += patch_pass(vc);
        }
        T t1[1];
        block_sum<T, 1, NW>(sh, p1, t1);  // its barriers also complete vc and the patch atomics
        const T gc = ml_coarse<T, NW>(sh, g, vc, ml_rr, ml_y, ml_wk, ml_dat, ml_lcodes);
        gam = sqrt(fmax(t1[0] + gc, T(0)));
        for (int d = g.NE + tid; d < N; d += NT) zt[d] += ml_code_prolong(ml_codes[d - g.NE], ml_y, m2);
        __syncthreads();
      }
      const T eta0 = gam;
      T eta = gam, c_prev = T(1), cc = T(1), s_prev = T(0), ss = T(0);
      T gi_c = gam > T(0) ? T(1) / gam : T(0), gi_p = T(0);
      const double tol_abs = prm.rtol * sqrt(bnorm2);
      // (FP64: 0.01, so that the solve lands near the FP64 residual floor, not
      // just under tol_abs: the edge block's error tracks the final residual;
      // mixed: 0.03 at depth 4, where the basis error at 0.1 came within 2x of
      // 1e-10, 0.1 below)
      const double outer = (kMixed ? (n >= 16 ? 0.03 : 0.1) : 0.01) * tol_abs / fmax(sqrt(rnorm2), 1e-300);
      const T target = (T)((kMixed ? fmax(prm.inner_rtol, outer) : outer) * (double)eta0);
      bool active = gam > T(0) && isfinite(gam);
      // patch path: the 1 / a1 scale of w_j and the x update of iteration j
      // are applied in the Lanczos pass of iteration j + 1 (pending)
      bool pending = false;
      T p_step = T(0), p_ia1 = T(0);
      for (int iter = 0; active && iter < prm.max_iter; ++iter) {
        // ---- phase 1
        T dpart = T(0);
        if constexpr (STAGE) dpart = staged_apply(vp); else
        for (int c = tid; c < nc; c += NT) {
          int e[12], f[6];
          cell_dofs(g, c, e, f);
          const bool eb[12] = {}, fb[6] = {};
          if constexpr (kMixed) {
            const float4 c0 = reinterpret_cast<const float4 *>(cf)[2 * c];
            const float4 c1 = reinterpret_cast<const float4 *>(cf)[2 * c + 1];
            const float ai[6] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
            dpart += merge ? cell_apply_s<float, float, float, 0, true, true>(zt, vp, Ff, ai, c1.z, e, f, eb, fb, c, g.L)
                       : cell_apply_s<float, float, float, 0, true>(zt, vp, Ff, ai, c1.z, e, f, eb, fb);
          } else {
            const double *a = ag + 6 * (size_t)c;
            const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
            dpart += merge ? cell_apply_s<double, double, double, 0, true, true>(zt, vp, Fd, ai, bg[c] * invV, e, f,
                                                                                eb, fb, c, g.L)
                       : cell_apply_s<double, double, double, 0, true>(zt, vp, Fd, ai, bg[c] * invV, e, f, eb, fb);
          }
        }
        warp_publish<T>(sh, 0, dpart);
        __syncthreads();
        const T delta = slot_total<T, NW>(sh, 0) * gi_c * gi_c;
        // ---- phase 2: v~_{j+1} = (S B - delta~ v~_j) / g_j in place of B
        T gpart = T(0);
        const T a2 = ss * delta + c_prev * cc * gam;
        const T a3 = s_prev * gam;
        if (epatch) {
          // with the patch edge block z~_{j+1} needs a cell pass, so z~_j is
          // consumed here: the direction w_j = (z~_j / g_j - a3 w_{j-2} - a2 w_{j-1}) / a1
          // is formed up to its 1 / a1 (which needs gamma_{j+1}) in w_{j-2}'s slot,
          // and zt takes the face part of z~_{j+1} (edges 0, accumulated by the
          // pass). The pending scale of w_{j-1} (still unscaled in its slot) and
          // x += c eta w_{j-1} of the previous iteration are applied on the way.
          const T sc = pending ? p_ia1 : T(1), st = pending ? p_step : T(0);
          if constexpr (kMixed) {
            const float4 *pd4 = reinterpret_cast<const float4 *>(pd);
            const float4 *vc4 = reinterpret_cast<const float4 *>(vc);
            float4 *vp4 = reinterpret_cast<float4 *>(vp);
            float4 *zt4 = reinterpret_cast<float4 *>(zt);
            float4 *wo4 = reinterpret_cast<float4 *>(wo);
            float4 *wc4 = reinterpret_cast<float4 *>(wc);
            float4 *xk4 = reinterpret_cast<float4 *>(xk);
            for (int q = tid; q < (int)(Np / 4); q += NT) {
              const float4 pv = pd4[q], b = vp4[q], c = vc4[q], z = zt4[q], a = wo4[q];
              float4 bw = wc4[q];
              if (pending) {
                float4 x = xk4[q];
                bw.x *= sc;
                bw.y *= sc;
                bw.z *= sc;
                bw.w *= sc;
                x.x += st * bw.x;
                x.y += st * bw.y;
                x.z += st * bw.z;
                x.w += st * bw.w;
                wc4[q] = bw;
                xk4[q] = x;
              }
              const bool face = 4 * q >= g.NE;
              const float sg = face ? -1.0f : 1.0f;
              auto lane = [&](float pdd, float bd, float cd) {
                return pdd > 0.0f ? (sg * bd - delta * cd) * gi_c : 0.0f;
              };
              float4 vn, wt, nz = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
              vn.x = lane(pv.x, b.x, c.x);
              vn.y = lane(pv.y, b.y, c.y);
              vn.z = lane(pv.z, b.z, c.z);
              vn.w = lane(pv.w, b.w, c.w);
              wt.x = z.x * gi_c - a3 * a.x - a2 * bw.x;
              wt.y = z.y * gi_c - a3 * a.y - a2 * bw.y;
              wt.z = z.z * gi_c - a3 * a.z - a2 * bw.z;
              wt.w = z.w * gi_c - a3 * a.w - a2 * bw.w;
              if (face) {
                nz = make_float4(pv.x * vn.x, pv.y * vn.y, pv.z * vn.z, pv.w * vn.w);
                gpart += nz.x * vn.x + nz.y * vn.y + nz.z * vn.z + nz.w * vn.w;
              }
              vp4[q] = vn;
              wo4[q] = wt;
              zt4[q] = nz;
            }
          } else {
            for (int d = tid; d < (int)Np; d += NT) {
              const float pdd = pd[d];
              T vn = T(0);
              if (pdd > 0.0f) {
                const T b = d < g.NE ? vp[d] : -vp[d];
                vn = (b - delta * vc[d]) * gi_c;
              }
              vp[d] = vn;
              T bw = wc[d];
              if (pending) {
                bw *= sc;
                wc[d] = bw;
                xk[d] += st * bw;
              }
              wo[d] = zt[d] * gi_c - a3 * wo[d] - a2 * bw;
              const T nz = d < g.NE ? T(0) : (T)pdd * vn;
              zt[d] = nz;
              gpart += nz * vn;
            }
          }
          pending = false;
          __syncthreads();
          gpart += patch_pass(vp);
        } else if constexpr (kMixed) {  // 4 DoFs per access; face quads start at NE (NE % 4 == 0 for n >= 4)
          const float4 *pd4 = reinterpret_cast<const float4 *>(pd);
          const float4 *vc4 = reinterpret_cast<const float4 *>(vc);
          float4 *vp4 = reinterpret_cast<float4 *>(vp);
          for (int q = tid; q < (int)(Np / 4); q += NT) {
            const float4 pv = pd4[q], b = vp4[q], c = vc4[q];
            const float sg = 4 * q >= g.NE ? -1.0f : 1.0f;
            auto lane = [&](float pdd, float bd, float cd) {
              return pdd > 0.0f ? (sg * bd - delta * cd) * gi_c : 0.0f;
            };
            float4 vn;
            vn.x = lane(pv.x, b.x, c.x);
            vn.y = lane(pv.y, b.y, c.y);
            vn.z = lane(pv.z, b.z, c.z);
            vn.w = lane(pv.w, b.w, c.w);
            vp4[q] = vn;
            gpart += pv.x * vn.x * vn.x + pv.y * vn.y * vn.y + pv.z * vn.z * vn.z + pv.w * vn.w * vn.w;
          }
        } else {
          for (int d = tid; d < N; d += NT) {
            const float pdd = pd[d];
            T vn = T(0);
            if (pdd > 0.0f) {
              const T b = d < g.NE ? vp[d] : -vp[d];
              vn = (b - delta * vc[d]) * gi_c;
            }
            vp[d] = vn;
            gpart += (T)pdd * vn * vn;
          }
        }
        warp_publish<T>(sh, 1, gpart);
        // the coarse step reads v~_{j+1}: complete after the Lanczos pass's
        // barrier on the patch path (the patch pass only adds to zt's edges and
        // the coarse step's own barriers publish slot 1), else after this one
        if (!epatch) __syncthreads();
        // ---- coarse step (reads v~_{j+1}, now in vp)
        const T gc = ml_coarse<T, NW>(sh, g, vp, ml_rr, ml_y, ml_wk, ml_dat, ml_lcodes);
        const T gnew = sqrt(fmax(slot_total<T, NW>(sh, 1) + gc, T(0)));
        const T a0 = cc * delta - c_prev * ss * gam;
        const T a1 = sqrt(a0 * a0 + gnew * gnew);
        if (!(a1 > T(0)) || !isfinite(a1)) {
          flags |= 1;
          break;
        }
        const T cn = a0 / a1, sn = gnew / a1;
        const T step = cn * eta, ia1 = T(1) / a1;
        // ---- phase 3 (pre: the prefill scale gamma_{j+1}^2 / g_j of v~_j's slot)
        const T pre = gnew * gnew * gi_c;
        if (epatch) {  // faces of z~_{j+1} += P_{n/2} y, prefill; w_j / x are pending
          if constexpr (kMixed) {
            float4 *vc4 = reinterpret_cast<float4 *>(vc);
            float4 *zt4 = reinterpret_cast<float4 *>(zt);
            for (int q = tid; q < (int)(Np / 4); q += NT) {
              const float4 vo = vc4[q];
              const bool face = 4 * q >= g.NE;
              if (face) {
                float4 nz = zt4[q];
                const uint2 cw = reinterpret_cast<const uint2 *>(ml_codes)[q - g.NE / 4];
                nz.x += ml_code_prolong(cw.x & 0xFFFFu, (const float *)ml_y, m2);
                nz.y += ml_code_prolong(cw.x >> 16, (const float *)ml_y, m2);
                nz.z += ml_code_prolong(cw.y & 0xFFFFu, (const float *)ml_y, m2);
                nz.w += ml_code_prolong(cw.y >> 16, (const float *)ml_y, m2);
                zt4[q] = nz;
              }
              const float ps = face ? (float)pre : -(float)pre;  // -S pre
              vc4[q] = make_float4(ps * vo.x, ps * vo.y, ps * vo.z, ps * vo.w);
            }
          } else {
            for (int d = tid; d < (int)Np; d += NT) {
              if (d >= g.NE) zt[d] += ml_code_prolong(ml_codes[d - g.NE], ml_y, m2);
              vc[d] = (d < g.NE ? -pre : pre) * vc[d];
            }
          }
          pending = true;
          p_step = step;
          p_ia1 = ia1;
        } else if constexpr (kMixed) {
          const float4 *pd4 = reinterpret_cast<const float4 *>(pd);
          const float4 *vp4 = reinterpret_cast<const float4 *>(vp);
          float4 *vc4 = reinterpret_cast<float4 *>(vc);
          float4 *zt4 = reinterpret_cast<float4 *>(zt);
          float4 *wo4 = reinterpret_cast<float4 *>(wo);
          const float4 *wc4 = reinterpret_cast<const float4 *>(wc);
          float4 *xk4 = reinterpret_cast<float4 *>(xk);
          for (int q = tid; q < (int)(Np / 4); q += NT) {
            const float4 z = zt4[q], a = wo4[q], b = wc4[q], pv = pd4[q], vn = vp4[q], vo = vc4[q];
            float4 x = xk4[q], wn, nz;
            wn.x = (z.x * gi_c - a3 * a.x - a2 * b.x) * ia1;
            wn.y = (z.y * gi_c - a3 * a.y - a2 * b.y) * ia1;
            wn.z = (z.z * gi_c - a3 * a.z - a2 * b.z) * ia1;
            wn.w = (z.w * gi_c - a3 * a.w - a2 * b.w) * ia1;
            x.x += step * wn.x;
            x.y += step * wn.y;
            x.z += step * wn.z;
            x.w += step * wn.w;
            nz.x = pv.x * vn.x;
            nz.y = pv.y * vn.y;
            nz.z = pv.z * vn.z;
            nz.w = pv.w * vn.w;
            const bool face = 4 * q >= g.NE;
            if (face) {
              const uint2 cw = reinterpret_cast<const uint2 *>(ml_codes)[q - g.NE / 4];
              nz.x += ml_code_prolong(cw.x & 0xFFFFu, (const float *)ml_y, m2);
              nz.y += ml_code_prolong(cw.x >> 16, (const float *)ml_y, m2);
              nz.z += ml_code_prolong(cw.y & 0xFFFFu, (const float *)ml_y, m2);
              nz.w += ml_code_prolong(cw.y >> 16, (const float *)ml_y, m2);
            }
            const float ps = face ? (float)pre : -(float)pre;  // -S pre
            wo4[q] = wn;
            xk4[q] = x;
            zt4[q] = nz;
            vc4[q] = make_float4(ps * vo.x, ps * vo.y, ps * vo.z, ps * vo.w);
          }
        } else {
          for (int d = tid; d < (int)Np; d += NT) {
            const T wn = (zt[d] * gi_c - a3 * wo[d] - a2 * wc[d]) * ia1;
            wo[d] = wn;
            xk[d] += step * wn;
            T nz = (T)pd[d] * vp[d];
            if (d >= g.NE) nz += ml_code_prolong(ml_codes[d - g.NE], ml_y, m2);
            zt[d] = nz;
            vc[d] = (d < g.NE ? -pre : pre) * vc[d];
          }
        }
        {
          T *t = wo;
          wo = wc;
          wc = t;
          t = vc;  // v~_{j+1} becomes current
          vc = vp;
          vp = t;
        }
        __syncthreads();
        gi_p = gi_c;
        gi_c = gnew > T(0) ? T(1) / gnew : T(0);
        ++its;
        eta = -sn * eta;
        gam = gnew;
        c_prev = cc;
        cc = cn;
        s_prev = ss;
        ss = sn;
        if (fabs(eta) <= target || gnew == T(0)) active = false;
      }
      if (pending)  // the last direction (unscaled, in wc after the swap) and its x update
        for (int d = tid; d < (int)Np; d += NT) xk[d] += p_step * (wc[d] * p_ia1);
      __syncthreads();
    } else {
      // ---------------- MINRES on A_II d = r, precision T ----------------
      // Preconditioned Lanczos + MINRES (Paige-Saunders recurrences in the form
      // of Elman, Silvester & Wathen, preconditioner pd, x0 = 0) in two
      // block-wide phases per iteration, each ending in one barrier:
      //   phase 1: az = A z~_j cell by cell, fused with delta~ = z~_j^T S A z~_j,
      //            plus the w / x update of iteration j-1 (it needs a1, which
      //            depends on gamma_j, known only after phase 2 of j-1);
      //   phase 2: v~_{j+1} = (S az - delta v~_j) / g_j - gamma_j v~_{j-1} / g_{j-1},
      //            z~_{j+1} = P v~_{j+1}, gamma_{j+1}^2 = z~_{j+1}^T v~_{j+1}.
      // The Lanczos vectors are kept unnormalised (v_j = v~_j / g_j, g_j =
      // gamma_j), so there is no normalisation pass; each phase's reduction is
      // published per warp and summed by every thread after the barrier.
      for (int d = tid; d < (int)Np; d += NT) {  // pads included: the float4 passes cover [0, Np)
        vB[d] = T(0);
        wA[d] = T(0);
        wB[d] = T(0);
        xk[d] = T(0);
        az[d] = T(0);
      }
      T *vc = vA, *vp = vB;  // v~_j, v~_{j-1}
      T *wo = wA, *wc = wB;  // w_{j-1}, w_j
      T gam;                 // gamma_j
      {
        T p1[1] = {T(0)};
        for (int d = tid; d < (int)Np; d += NT) {
          const T z = (T)pd[d] * vc[d];
          zt[d] = z;
          p1[0] += z * vc[d];
        }
        T t1[1];
        block_sum<T, 1, NW>(sh, p1, t1);
        gam = sqrt(t1[0]);
      }
      const T eta0 = gam;
      T eta = gam, c_prev = T(1), cc = T(1), s_prev = T(0), ss = T(0);
      T gi_c = gam > T(0) ? T(1) / gam : T(0), gi_p = T(0);  // 1/gamma_j, 1/gamma_{j-1}
      const double tol_abs = prm.rtol * sqrt(bnorm2);
      // inner target on |eta| (preconditioned residual): for the mixed path a
      // relative reduction inner_rtol, relaxed on the last refinement step to
      // what the outer tolerance still asks (0.1 or 0.03 tol_abs / ||r||); for FP64 the
      // outer tolerance itself. Both are mapped through eta0 / ||r||.
      // (FP64: 0.01, so that the solve lands near the FP64 residual floor, not
      // just under tol_abs: the edge block's error tracks the final residual;
      // mixed: 0.03 at depth 4, where the basis error at 0.1 came within 2x of
      // 1e-10, 0.1 below)
      const double outer = (kMixed ? (n >= 16 ? 0.03 : 0.1) : 0.01) * tol_abs / fmax(sqrt(rnorm2), 1e-300);
      const T target = (T)((kMixed ? fmax(prm.inner_rtol, outer) : outer) * (double)eta0);
      bool active = gam > T(0) && isfinite(gam);
      bool pending = false;  // w / x update of the last iteration not yet applied
      T p_step = T(0), p_a2 = T(0), p_a3 = T(0), p_ia1 = T(0);
      __syncthreads();
      for (int iter = 0; active && iter < prm.max_iter; ++iter) {
        // ---- phase 1
        T dpart = T(0);
        if constexpr (STAGE) dpart = staged_apply(az); else
        for (int c = tid; c < nc; c += NT) {
          int e[12], f[6];
          cell_dofs(g, c, e, f);
          const bool eb[12] = {}, fb[6] = {};
          if constexpr (kMixed) {
            const float4 c0 = reinterpret_cast<const float4 *>(cf)[2 * c];
            const float4 c1 = reinterpret_cast<const float4 *>(cf)[2 * c + 1];
            const float ai[6] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
            dpart += merge ? cell_apply_s<float, float, float, 0, true, true>(zt, az, Ff, ai, c1.z, e, f, eb, fb, c, g.L)
                       : cell_apply_s<float, float, float, 0, true>(zt, az, Ff, ai, c1.z, e, f, eb, fb);
          } else {
            const double *a = ag + 6 * (size_t)c;
            const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
            dpart += merge ? cell_apply_s<double, double, double, 0, true, true>(zt, az, Fd, ai, bg[c] * invV, e, f,
                                                                                eb, fb, c, g.L)
                       : cell_apply_s<double, double, double, 0, true>(zt, az, Fd, ai, bg[c] * invV, e, f, eb, fb);
          }
        }
        if (pending) {  // w_j = (z_{j-1} - a3 w_{j-2} - a2 w_{j-1}) / a1, x += c eta w_j
          if constexpr (kMixed) {  // 4 DoFs per thread and vector access (pads are 0)
            const float4 *pd4 = reinterpret_cast<const float4 *>(pd);
            const float4 *vp4 = reinterpret_cast<const float4 *>(vp);
            float4 *wo4 = reinterpret_cast<float4 *>(wo);
            const float4 *wc4 = reinterpret_cast<const float4 *>(wc);
            float4 *xk4 = reinterpret_cast<float4 *>(xk);
            for (int q = tid; q < (int)(Np / 4); q += NT) {
              const float4 pv = pd4[q], v = vp4[q], a = wo4[q], b = wc4[q];
              float4 x = xk4[q], wn;
              wn.x = (pv.x * v.x * gi_p - p_a3 * a.x - p_a2 * b.x) * p_ia1;
              wn.y = (pv.y * v.y * gi_p - p_a3 * a.y - p_a2 * b.y) * p_ia1;
              wn.z = (pv.z * v.z * gi_p - p_a3 * a.z - p_a2 * b.z) * p_ia1;
              wn.w = (pv.w * v.w * gi_p - p_a3 * a.w - p_a2 * b.w) * p_ia1;
              x.x += p_step * wn.x;
              x.y += p_step * wn.y;
              x.z += p_step * wn.z;
              x.w += p_step * wn.w;
              wo4[q] = wn;
              xk4[q] = x;
            }
          } else {
            for (int d = tid; d < N; d += NT) {
              const T z = (T)pd[d] * vp[d] * gi_p;
              const T wn = (z - p_a3 * wo[d] - p_a2 * wc[d]) * p_ia1;
              wo[d] = wn;
              xk[d] += p_step * wn;
            }
          }
          T *t = wo;
          wo = wc;
          wc = t;
        }
        warp_publish<T>(sh, 0, dpart);
        __syncthreads();
        const T delta = slot_total<T, NW>(sh, 0) * gi_c * gi_c;
        // ---- phase 2
        T gpart = T(0);
        const T gg = gam * gi_p;
        if constexpr (kMixed) {  // 4 DoFs per thread and vector access (pads are 0)
          const float4 *pd4 = reinterpret_cast<const float4 *>(pd);
          const float4 *vc4 = reinterpret_cast<const float4 *>(vc);
          float4 *vp4 = reinterpret_cast<float4 *>(vp);
          float4 *az4 = reinterpret_cast<float4 *>(az);
          float4 *zt4 = reinterpret_cast<float4 *>(zt);
          for (int q = tid; q < (int)(Np / 4); q += NT) {
            const float4 pv = pd4[q], a = az4[q], c = vc4[q], v = vp4[q];
            const int d0 = 4 * q;
            auto lane = [&](float pdd, float ad, float cd, float vd, int d) {
              const float sa = d < g.NE ? ad : -ad;
              return pdd > 0.0f ? (sa - delta * cd) * gi_c - gg * vd : 0.0f;
            };
            float4 vn, z;
            vn.x = lane(pv.x, a.x, c.x, v.x, d0);
            vn.y = lane(pv.y, a.y, c.y, v.y, d0 + 1);
            vn.z = lane(pv.z, a.z, c.z, v.z, d0 + 2);
            vn.w = lane(pv.w, a.w, c.w, v.w, d0 + 3);
            z.x = pv.x * vn.x;
            z.y = pv.y * vn.y;
            z.z = pv.z * vn.z;
            z.w = pv.w * vn.w;
            vp4[q] = vn;
            az4[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            zt4[q] = z;
            gpart += z.x * vn.x + z.y * vn.y + z.z * vn.z + z.w * vn.w;
          }
        } else {
          for (int d = tid; d < N; d += NT) {
            const float pdd = pd[d];
            T vn = T(0);
            if (pdd > 0.0f) {
              const T a = d < g.NE ? az[d] : -az[d];
              vn = (a - delta * vc[d]) * gi_c - gg * vp[d];
            }
            vp[d] = vn;
            az[d] = T(0);
            const T z = (T)pdd * vn;
            zt[d] = z;
            gpart += z * vn;
          }
        }
        warp_publish<T>(sh, 1, gpart);
        __syncthreads();
        const T gnew = sqrt(fmax(slot_total<T, NW>(sh, 1), T(0)));
        const T a0 = cc * delta - c_prev * ss * gam;
        const T a1 = sqrt(a0 * a0 + gnew * gnew);
        const T a2 = ss * delta + c_prev * cc * gam;
        const T a3 = s_prev * gam;
        if (!(a1 > T(0)) || !isfinite(a1)) {
          flags |= 1;
          break;
        }
        const T cn = a0 / a1, sn = gnew / a1;
        p_step = cn * eta;
        p_a2 = a2;
        p_a3 = a3;
        p_ia1 = T(1) / a1;
        pending = true;
        {
          T *t = vc;  // v~_{j+1} becomes current
          vc = vp;
          vp = t;
        }
        gi_p = gi_c;
        gi_c = gnew > T(0) ? T(1) / gnew : T(0);
        ++its;
        eta = -sn * eta;
        gam = gnew;
        c_prev = cc;
        cc = cn;
        s_prev = ss;
        ss = sn;
        if (fabs(eta) <= target || gnew == T(0)) active = false;
      }
      if (pending)
        for (int d = tid; d < N; d += NT) {
          const T z = (T)pd[d] * vp[d] * gi_p;
          const T wn = (z - p_a3 * wo[d] - p_a2 * wc[d]) * p_ia1;
          xk[d] += p_step * wn;
        }
      __syncthreads();
    }
    // ---------------- phi_I += x (FP64, HBM) ----------------
    for (int d = tid; d < N; d += NT)
      if (pd[d] > 0.0f) phi[d] += (double)xk[d];
    __syncthreads();
  }

  // ---------------- y_b = A P_b (FP64), P_b = primary block of basis b ----------------
  if (!src) {  // block-uniform
    for (int d = tid; d < N; d += NT) dacc[d] = 0.0;
    __syncthreads();
    for (int c = tid; c < nc; c += NT) {
      int e[12], f[6];
      cell_dofs(g, c, e, f);
      const bool eb[12] = {}, fb[6] = {};
      const double *a = ag + 6 * (size_t)c;
      const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
      if (bb < 12)
        cell_apply_s<double, double, double, 2, false>(phi, dacc, Fd, ai, bg[c] * invV, e, f, eb, fb);
      else
        cell_apply_s<double, double, double, 3, false>(phi, dacc, Fd, ai, bg[c] * invV, e, f, eb, fb);
    }
    __syncthreads();
    for (int d = tid; d < N; d += NT) yout[d] = dacc[d];
  }
  if (tid == 0) {
    NRStat st;
    st.iters = its;
    st.refinements = nref;
    st.converged = conv;
    st.flags = flags;
    st.rel_residual = bnorm2 > 0.0 ? sqrt(rnorm2 / bnorm2) : sqrt(rnorm2);
    prm.stats[(size_t)it.cell * 18 + bb] = st;
  }
  __syncthreads();
}

// ML: multilevel face preconditioner (cells with coarse data), else diagonal.
// PLACE: where the MINRES workspace lives, one kernel per placement so that
// each gets its own register allocation (fewer spills than one kernel that
// branches between them): 1 shared memory (NT = 256: the split workspace of
// the two-CTAs-per-SM variant), 0 this CTA's global slot, 2 the global slot
// with the apply's coefficient tiles staged by bulk copies, 3 the global slot
// with z~ in shared memory. Keeping only the
// apply's accumulation vector in shared memory for the global placement was
// measured slower (3917 vs 3659 ms on 512 depth-4 cells): its 108 KB take L1
// from the apply's scattered global gathers.
template <typename T, int NT, bool ML, int PLACE>
__global__ void __launch_bounds__(NT, 512 / NT) nedrt_solve_kernel(NRParams prm) {
  __shared__ NRShared sh;
  if constexpr (PLACE == 2) {
    if ((threadIdx.x & 31) == 0) {
      mbar_init(&sh.mbar[threadIdx.x >> 5][0], 1);
      mbar_init(&sh.mbar[threadIdx.x >> 5][1], 1);
      sh.tph[threadIdx.x >> 5] = 0;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
  }
  for (;;) {
    if (threadIdx.x == 0) sh.item = atomicAdd(prm.queue, 1);
    __syncthreads();
    const int item = sh.item;
    if (item >= prm.n_items) break;
    solve_item<T, PLACE == 1, NT, ML, PLACE == 2, PLACE == 3>(prm, sh, item);
  }
}

}  // namespace nrimpl

// One persistent launch of nedrt_solve_kernel<T, NT, ML, PLACE>.
template <typename T, int NT, bool ML, int PLACE>
inline cudaError_t nedrt_launch_variant(const NRParams &prm, size_t smem, int grid, cudaStream_t st, bool carveout) {
  auto k = nrimpl::nedrt_solve_kernel<T, NT, ML, PLACE>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (carveout) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, NT, smem, st>>>(prm);
  return cudaGetLastError();
}

}  // namespace msfec
