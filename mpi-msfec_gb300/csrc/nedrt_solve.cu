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
__device__ double table_G(const double h[3], int p, int q, int l4, int m4) {
  if (p == q) {
    int o1, o2;
    other_axes(p, o1, o2);
    return h[o1] * h[o2] / h[p] * m1(l4 & 1, m4 & 1) * m1(l4 >> 1, m4 >> 1);
  }
  const int r = 3 - p - q;
  return 0.25 * h[r] * m1(edge_pos(p, l4, r), edge_pos(q, m4, r));
}

__device__ double table_C(const double h[3], int l, int f) {
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
__device__ bool dof_geometry(const NRGeom &g, int d, int &dir, int &i, int &j, int &k) {
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
__device__ double coarse_dof(int b, int dir, int i, int j, int k, int n) {
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
__device__ void curl_rhs_cell(int b, int i, int j, int k, int n, const double h[3], double (&out)[6]) {
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

// One (cell, basis) item. SMEM: the workspace is the dynamic shared memory
// (known at compile time, so every vector access is a shared-memory access),
// otherwise this CTA's slot of the global scratch.
// STAGE (global workspace, mixed precision): the apply reads each warp's 32
// cells of coefficients from shared memory, where a bulk copy issued two rounds
// earlier put them.
template <typename T, bool SMEM, int NT, bool ML, bool STAGE = false>
__device__ void solve_item(const NRParams &prm, NRShared &sh, int item_id) {
  // NT = 256 (two CTAs per SM, mixed precision, shared workspace): the
  // correction x and the float coefficients live in this CTA's global slot so
  // that the shared part (preconditioner + 6 vectors) fits twice per SM.
  constexpr bool kSplitWs = NT == 256;
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
  // workspace carve (floats)
  float *pd = ws;
  T *zt = reinterpret_cast<T *>(ws + Np);  // P v~_j (unnormalised), operand of the apply
  T *az = zt + Np;
  T *vA = az + Np;  // unnormalised Lanczos vectors v~_j, v~_{j-1} (roles swap)
  T *vB = vA + Np;
  T *wA = vB + Np;  // MINRES directions w_{j-1}, w_j (roles swap)
  T *wB = wA + Np;
  float *gws = prm.scratch + (size_t)blockIdx.x * prm.scratch_floats;  // split workspace only
  T *xk = kSplitWs ? reinterpret_cast<T *>(gws) : wB + Np;
  float *cf = kSplitWs ? gws + Np * (sizeof(T) / 4) : ws + Np + 7 * Np * (sizeof(T) / 4);
  double *dacc = reinterpret_cast<double *>(ws + Np);  // FP64 residual accumulator, aliases zt..
  const NRFactors<float> &Ff = sh.Ff;
  const NRFactors<double> &Fd = sh.Fd;
  if (tid == 0) {
    make_factors(Cc.h, sh.Ff);
    make_factors(Cc.h, sh.Fd);
  }
  float *facc = ws + Np;
  const double *ag = prm.ainv6 + 6 * Cc.coef_off;
  const double *bg = prm.bdiv + Cc.coef_off;
  double *phi = src ? prm.src_out + kNRSrcRhs * Cc.dof_off + (size_t)bb * N
                    : prm.phi + 18 * Cc.dof_off + (size_t)bb * N;
  const double *fsrc = src ? prm.src_rhs + kNRSrcRhs * Cc.dof_off + (size_t)bb * N : nullptr;
  double *yout = prm.y + 18 * Cc.dof_off + (size_t)bb * N;

  // tables
  for (int t = tid; t < 144 + 72; t += NT) {
    if (t < 144) {
      const int p = t / 48, q = (t / 16) % 3, l4 = (t / 4) % 4, m4 = t % 4;
      const double v = table_G(Cc.h, p, q, l4, m4);
      sh.Gf[p][q][l4][m4] = (float)v;
    } else {
      const int u = t - 144, l = u / 6, f = u % 6;
      const double v = table_C(Cc.h, l, f);
      sh.Cf[l][f] = (float)v;
    }
  }
  for (int c = tid; c < nc; c += NT) {
#pragma unroll
    for (int q = 0; q < 6; ++q) cf[8 * c + q] = (float)ag[6 * (size_t)c + q];
    cf[8 * c + 6] = (float)(bg[c] * invV);  // B / |K|
    cf[8 * c + 7] = 0.0f;
  }
  for (int d = tid; d < (int)Np; d += NT) pd[d] = 0.0f;  // pad [N, Np) stays 0
  if constexpr (STAGE) asm volatile("fence.proxy.async.global;" ::: "memory");  // cf is read by bulk copies
  __syncthreads();

  // ---- block-Jacobi preconditioner: diag(M) on edges, then the lumped Schur
  // diagonal D_ff + sum_l C_lf^2 / M_ll on faces (cell-local approximation).
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
  for (int d = tid; d < N; d += NT) {
    int dir, i, j, k;
    const bool bnd = dof_geometry(g, d, dir, i, j, k);
    pd[d] = (bnd && !natural) ? 0.0f : 1.0f / pd[d];
  }
  __syncthreads();

  // ---- multilevel part of the preconditioner (block-uniform switch): the
  // cell's data from HBM, the faces' level-n/2 parent codes
  const bool ml = ML && prm.coarse != nullptr && Cc.coarse_off >= 0 && !natural;
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
    // fine level: the inverse assembled diagonal of S replaces the cell-lumped one on the faces
    for (int u = tid; u < g.NF; u += NT)
      if (pd[g.NE + u] > 0.0f) pd[g.NE + u] = src[nd + u];
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

  double bnorm2 = 0.0, rnorm2 = 0.0;
  int conv = 0, its = 0, flags = 0, nref = 0;
  static_assert(!STAGE || (sizeof(T) == 4 && !SMEM && NT == 512), "staged apply: mixed, global workspace");

  // Phase-1 apply with the coefficients staged by bulk copies: in round r warp
  // w applies cells r NT + 32 w .. + 31, whose 32 x 8 floats form one
  // contiguous 1 KB tile of cf; the tile of round r + 2 is copied into the
  // stage the warp has just read while it works on round r + 1, so the apply
  // waits on no global coefficient load. Waits are bounded: a copy that never
  // completes flags the item (bit 2) instead of hanging the SM.
  auto staged_apply = [&]() -> float {
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
            dp += merge ? cell_apply_s<float, float, float, 0, true, true>(zt, az, Ff, ai, c1.z, e, f, eb, fb, c, g.L)
                        : cell_apply_s<float, float, float, 0, true>(zt, az, Ff, ai, c1.z, e, f, eb, fb);
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
      // recomputable from v~_j alone: zt holds the full z~_j, and each iteration
      // runs three block-wide phases and the coarse step, each ending in barriers:
      //   phase 1: az = A z~_j, delta~;
      //   phase 2: v~_{j+1}; az <- diag^-1 v~_{j+1} (the fine part of z~_{j+1});
      //            gamma^2 partials;
      //   coarse:  level-n/2 coefficients y of the coarse part of z~_{j+1} and
      //            its share of gamma_{j+1}^2 (ml_coarse_block);
      //   phase 3: w_j from z~_j (still in zt), x += c eta w_j, then
      //            zt <- az + P_{n/2} y (the full z~_{j+1}), az <- 0.
      for (int d = tid; d < (int)Np; d += NT) {
        vB[d] = T(0);
        wA[d] = T(0);
        wB[d] = T(0);
        xk[d] = T(0);
        az[d] = T(0);
      }
      T *vc = vA, *vp = vB;
      T *wo = wA, *wc = wB;
      T gam;
      {
        T p1[1] = {T(0)};
        for (int d = tid; d < (int)Np; d += NT) {
          const T z = (T)pd[d] * vc[d];
          zt[d] = z;
          p1[0] += z * vc[d];
        }
        T t1[1];
        block_sum<T, 1, NW>(sh, p1, t1);  // its barriers also complete vc
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
      // just under tol_abs: the edge block's error tracks the final residual)
      const double outer = (kMixed ? 0.1 : 0.01) * tol_abs / fmax(sqrt(rnorm2), 1e-300);
      const T target = (T)((kMixed ? fmax(prm.inner_rtol, outer) : outer) * (double)eta0);
      bool active = gam > T(0) && isfinite(gam);
      for (int iter = 0; active && iter < prm.max_iter; ++iter) {
        // ---- phase 1
        T dpart = T(0);
        if constexpr (STAGE) dpart = staged_apply(); else
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
        warp_publish<T>(sh, 0, dpart);
        __syncthreads();
        const T delta = slot_total<T, NW>(sh, 0) * gi_c * gi_c;
        // ---- phase 2
        T gpart = T(0);
        const T gg = gam * gi_p;
        if constexpr (kMixed) {  // 4 DoFs per access; face quads start at NE (NE % 4 == 0 for n >= 4)
          const float4 *pd4 = reinterpret_cast<const float4 *>(pd);
          const float4 *vc4 = reinterpret_cast<const float4 *>(vc);
          float4 *vp4 = reinterpret_cast<float4 *>(vp);
          float4 *az4 = reinterpret_cast<float4 *>(az);
          for (int q = tid; q < (int)(Np / 4); q += NT) {
            const float4 pv = pd4[q], a = az4[q], c = vc4[q], v = vp4[q];
            const bool face = 4 * q >= g.NE;
            const float sg = face ? -1.0f : 1.0f;
            auto lane = [&](float pdd, float ad, float cd, float vd) {
              return pdd > 0.0f ? (sg * ad - delta * cd) * gi_c - gg * vd : 0.0f;
            };
            float4 vn, z;
            vn.x = lane(pv.x, a.x, c.x, v.x);
            vn.y = lane(pv.y, a.y, c.y, v.y);
            vn.z = lane(pv.z, a.z, c.z, v.z);
            vn.w = lane(pv.w, a.w, c.w, v.w);
            z.x = pv.x * vn.x;
            z.y = pv.y * vn.y;
            z.z = pv.z * vn.z;
            z.w = pv.w * vn.w;
            vp4[q] = vn;
            az4[q] = z;
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
            const T z = (T)pdd * vn;
            az[d] = z;
            gpart += z * vn;
          }
        }
        warp_publish<T>(sh, 1, gpart);
        __syncthreads();
        // ---- coarse step (reads v~_{j+1}, now in vp)
        const T gc = ml_coarse<T, NW>(sh, g, vp, ml_rr, ml_y, ml_wk, ml_dat, ml_lcodes);
        const T gnew = sqrt(fmax(slot_total<T, NW>(sh, 1) + gc, T(0)));
        const T a0 = cc * delta - c_prev * ss * gam;
        const T a1 = sqrt(a0 * a0 + gnew * gnew);
        const T a2 = ss * delta + c_prev * cc * gam;
        const T a3 = s_prev * gam;
        if (!(a1 > T(0)) || !isfinite(a1)) {
          flags |= 1;
          break;
        }
        const T cn = a0 / a1, sn = gnew / a1;
        const T step = cn * eta, ia1 = T(1) / a1;
        // ---- phase 3
        if constexpr (kMixed) {
          const float4 *az4 = reinterpret_cast<const float4 *>(az);
          float4 *zt4 = reinterpret_cast<float4 *>(zt);
          float4 *wo4 = reinterpret_cast<float4 *>(wo);
          const float4 *wc4 = reinterpret_cast<const float4 *>(wc);
          float4 *xk4 = reinterpret_cast<float4 *>(xk);
          float4 *azw = reinterpret_cast<float4 *>(az);
          for (int q = tid; q < (int)(Np / 4); q += NT) {
            const float4 z = zt4[q], a = wo4[q], b = wc4[q], fz = az4[q];
            float4 x = xk4[q], wn, nz = fz;
            wn.x = (z.x * gi_c - a3 * a.x - a2 * b.x) * ia1;
            wn.y = (z.y * gi_c - a3 * a.y - a2 * b.y) * ia1;
            wn.z = (z.z * gi_c - a3 * a.z - a2 * b.z) * ia1;
            wn.w = (z.w * gi_c - a3 * a.w - a2 * b.w) * ia1;
            x.x += step * wn.x;
            x.y += step * wn.y;
            x.z += step * wn.z;
            x.w += step * wn.w;
            if (4 * q >= g.NE) {
              const uint2 cw = reinterpret_cast<const uint2 *>(ml_codes)[q - g.NE / 4];
              nz.x += ml_code_prolong(cw.x & 0xFFFFu, (const float *)ml_y, m2);
              nz.y += ml_code_prolong(cw.x >> 16, (const float *)ml_y, m2);
              nz.z += ml_code_prolong(cw.y & 0xFFFFu, (const float *)ml_y, m2);
              nz.w += ml_code_prolong(cw.y >> 16, (const float *)ml_y, m2);
            }
            wo4[q] = wn;
            xk4[q] = x;
            zt4[q] = nz;
            azw[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          }
        } else {
          for (int d = tid; d < (int)Np; d += NT) {
            const T wn = (zt[d] * gi_c - a3 * wo[d] - a2 * wc[d]) * ia1;
            wo[d] = wn;
            xk[d] += step * wn;
            T nz = az[d];
            if (d >= g.NE) nz += ml_code_prolong(ml_codes[d - g.NE], ml_y, m2);
            zt[d] = nz;
            az[d] = T(0);
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
      // what the outer tolerance still asks (0.1 tol_abs / ||r||); for FP64 the
      // outer tolerance itself. Both are mapped through eta0 / ||r||.
      // (FP64: 0.01, so that the solve lands near the FP64 residual floor, not
      // just under tol_abs: the edge block's error tracks the final residual)
      const double outer = (kMixed ? 0.1 : 0.01) * tol_abs / fmax(sqrt(rnorm2), 1e-300);
      const T target = (T)((kMixed ? fmax(prm.inner_rtol, outer) : outer) * (double)eta0);
      bool active = gam > T(0) && isfinite(gam);
      bool pending = false;  // w / x update of the last iteration not yet applied
      T p_step = T(0), p_a2 = T(0), p_a3 = T(0), p_ia1 = T(0);
      __syncthreads();
      for (int iter = 0; active && iter < prm.max_iter; ++iter) {
        // ---- phase 1
        T dpart = T(0);
        if constexpr (STAGE) dpart = staged_apply(); else
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
// branches between them): 1 shared memory, 0 this CTA's global slot (NT = 256
// is the split workspace of the two-CTAs-per-SM variant). Keeping only the
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
    if constexpr (NT == 256)
      solve_item<T, true, 256, ML>(prm, sh, item);  // split workspace: shared vectors + global x / coefficients
    else
      solve_item<T, PLACE == 1, NT, ML, PLACE == 2>(prm, sh, item);
  }
}

constexpr int kGalThreads = 256;
constexpr int kGalWarps = kGalThreads / 32;

__device__ __forceinline__ void dmma(double &c0, double &c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// Average of sin(w x) over fine cell `cell` along one axis (2-point Gauss).
__device__ double gauss_sin_avg(double x0, double h, int cell, double w) {
  const double gq = 0.5 / sqrt(3.0);
  return 0.5 * (sin(w * (x0 + (cell + 0.5 - gq) * h)) + sin(w * (x0 + (cell + 0.5 + gq) * h)));
}

// K_H[i][j] = P_i . y_j over all DoFs (P_i: primary block of basis i), on
// the FP64 tensor pipe (m8n8k4 tiles of the 24x24 padded product);
// F_H[12+f] = u_f . (v, f) (reference ned_rt_basis.cc:937-944).
__global__ void __launch_bounds__(kGalThreads) nedrt_galerkin_kernel(const NRCell *__restrict__ cells,
                                                                     const double *__restrict__ phi,
                                                                     const double *__restrict__ y, msfec_load load,
                                                                     double *__restrict__ KH, double *__restrict__ FH) {
  __shared__ double red[kGalWarps][24 * 24];
  __shared__ double redf[kGalWarps][8];
  __shared__ double stab[3][65];  // 1D Gauss averages of sin per axis
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  NRGeom g;
  g.n = C.n;
  g.L = C.depth;
  nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
  g.N = g.NE + g.NF;
  const int n = g.n, N = g.N;
  const bool has_load = load.kind == MSFEC_LOAD_VEC_TRIG;
  const double w = load.params[1] * M_PI;
  for (int t = threadIdx.x; t < 3 * n; t += kGalThreads) {
    const int d = t / n, i = t % n;
    stab[d][i] = has_load ? gauss_sin_avg(C.origin[d], C.h[d], i, w) : 0.0;
  }
  __syncthreads();
  const double *P = phi + 18 * C.dof_off;
  const double *Y = y + 18 * C.dof_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gr = lane >> 2, t4 = lane & 3;
  double acc[3][3][2];
#pragma unroll
  for (int I = 0; I < 3; ++I)
#pragma unroll
    for (int J = 0; J < 3; ++J) acc[I][J][0] = acc[I][J][1] = 0.0;
  for (int base = warp * 4; base < N; base += kGalWarps * 4) {
    const int d = base + t4;
    const bool ok = d < N;
    const bool is_edge = d < g.NE;
    double a[3], b[3];
#pragma unroll
    for (int I = 0; I < 3; ++I) {
      const int row = 8 * I + gr;
      const bool prim = row < 18 && ((row < 12) == is_edge);
      a[I] = (ok && prim) ? __ldcs(P + (size_t)row * N + d) : 0.0;
      b[I] = (ok && row < 18) ? __ldcs(Y + (size_t)row * N + d) : 0.0;
    }
#pragma unroll
    for (int I = 0; I < 3; ++I)
#pragma unroll
      for (int J = 0; J < 3; ++J) dmma(acc[I][J][0], acc[I][J][1], a[I], b[J]);
  }
  // F_H: face rows only (edge rows of the reference's global_element_rhs stay 0)
  {
    double f6[6] = {0, 0, 0, 0, 0, 0};
    if (has_load)
      for (int d = g.NE + threadIdx.x; d < N; d += kGalThreads) {
        int dir, i, j, k;
        dof_geometry(g, d, dir, i, j, k);
        const int fd = dir - 3;
        const int pos = fd == 0 ? i : (fd == 1 ? j : k);
        const double nadj = (pos == 0 || pos == n) ? 1.0 : 2.0;
        double s1, s2;
        if (fd == 0) {
          s1 = stab[1][j];
          s2 = stab[2][k];
        } else if (fd == 1) {
          s1 = stab[2][k];
          s2 = stab[0][i];
        } else {
          s1 = stab[0][i];
          s2 = stab[1][j];
        }
        const double bl = load.params[0] * 0.5 * C.h[fd] * nadj * s1 * s2;
#pragma unroll
        for (int q = 0; q < 6; ++q) f6[q] += P[(size_t)(12 + q) * N + d] * bl;
      }
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      double v = f6[q];
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) redf[warp][q] = v;
    }
  }
#pragma unroll
  for (int I = 0; I < 3; ++I)
#pragma unroll
    for (int J = 0; J < 3; ++J) {
      const int row = 8 * I + gr;
      red[warp][row * 24 + 8 * J + 2 * t4] = acc[I][J][0];
      red[warp][row * 24 + 8 * J + 2 * t4 + 1] = acc[I][J][1];
    }
  __syncthreads();
  for (int t = threadIdx.x; t < 18 * 18; t += kGalThreads) {
    const int i = t / 18, j = t % 18;
    double s = 0.0;
    for (int wv = 0; wv < kGalWarps; ++wv) s += red[wv][i * 24 + j];
    KH[(size_t)c * 324 + t] = s;
  }
  if (threadIdx.x < 18) {
    double s = 0.0;
    if (threadIdx.x >= 12)
      for (int wv = 0; wv < kGalWarps; ++wv) s += redf[wv][threadIdx.x - 12];
    FH[(size_t)c * 18 + threadIdx.x] = s;
  }
}

__global__ void nedrt_report_kernel(const NRStat *__restrict__ stats, int ncells, msfec_cell_report *rep) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  msfec_cell_report r;
  r.iterations = 0;
  r.refinements = 0;
  r.converged = 1;
  r.iterations_sum = 0;
  r.residual = 0.0;
  for (int v = 0; v < 18; ++v) {
    const NRStat s = stats[(size_t)c * 18 + v];
    r.iterations = max(r.iterations, s.iters);
    r.iterations_sum += s.iters;
    r.refinements = max(r.refinements, s.refinements);
    r.converged = r.converged && s.converged && !(s.flags & 5);  // breakdown or a stage copy timed out
    r.residual = fmax(r.residual, s.rel_residual);
    if (!isfinite(s.rel_residual)) r.residual = s.rel_residual;
  }
  rep[c] = r;
}


// ---------------------------------------------------------------------------
// Adjoint of the Ned_RT build (parameters: log-scales of A and B per fine
// cell). With s = P U, t = P lambda (P: primary blocks of the basis), the four
// combinations Phi_E lambda, Phi_E U, Phi_F lambda, Phi_F U (E: the 12 edge
// bases, F: the 6 face bases), e = dJ/du_h and the face load b:
//   rhs_k = S Pi_k w_k on interior DoFs, solved with A_II (source items),
//   eta_k = S x_k (A_II^T = S A_II S), and per fine cell
//   dJ/dta = t_s^T M s_s + sum_k eta_k,s^T M c_k,s,  dJ/dtb = -(same with D),
// c_k the k-th combination; w_0 = -A s, w_1 = -A^T t (sigma block),
// w_2 = b - A s, w_3 = e - A^T t (u block).
constexpr int kAdjThreads = 256;

// comb[4][N] per cell (at 4 dof_off): Phi_E lambda, Phi_E U, Phi_F lambda, Phi_F U.
__global__ void __launch_bounds__(kAdjThreads) nr_adj_combine_kernel(const NRCell *__restrict__ cells,
                                                                     const double *__restrict__ phi,
                                                                     const double *__restrict__ U,
                                                                     const double *__restrict__ lam,
                                                                     double *__restrict__ comb) {
  __shared__ double w[2][18];
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  int NEx, NFx, NE, NF;
  nr_counts(C.n, NEx, NFx, NE, NF);
  const int N = NE + NF;
  if (threadIdx.x < 18) {
    w[0][threadIdx.x] = lam[18 * (size_t)c + threadIdx.x];
    w[1][threadIdx.x] = U[18 * (size_t)c + threadIdx.x];
  }
  __syncthreads();
  const double *P = phi + 18 * C.dof_off;
  double *out = comb + kNRSrcRhs * C.dof_off;
  for (int d = threadIdx.x; d < N; d += kAdjThreads) {
    double el = 0.0, eu = 0.0, fl = 0.0, fu = 0.0;
#pragma unroll
    for (int b = 0; b < 12; ++b) {
      const double v = P[(size_t)b * N + d];
      el = fma(w[0][b], v, el);
      eu = fma(w[1][b], v, eu);
    }
#pragma unroll
    for (int b = 12; b < 18; ++b) {
      const double v = P[(size_t)b * N + d];
      fl = fma(w[0][b], v, fl);
      fu = fma(w[1][b], v, fu);
    }
    out[d] = el;
    out[(size_t)N + d] = eu;
    out[2 * (size_t)N + d] = fl;
    out[3 * (size_t)N + d] = fu;
  }
}

// e = dJ/du_h: point k in coarse cell cell_of[k] spreads dJ_du[k][d] onto the
// two faces of normal d of its fine cell with the RT0 weights.
__global__ void nr_adj_point_kernel(const NRCell *__restrict__ cells, int npoints, const int *__restrict__ cell_of,
                                    const double *__restrict__ pts, const double *__restrict__ dJdu,
                                    double *__restrict__ e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npoints) return;
  const NRCell C = cells[cell_of[k]];
  NRGeom g;
  g.n = C.n;
  g.L = C.depth;
  nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
  g.N = g.NE + g.NF;
  int fi[3];
  double tau[3];
  for (int d = 0; d < 3; ++d) {
    const double s = (pts[3 * (size_t)k + d] - C.origin[d]) / C.h[d];
    fi[d] = min(max((int)floor(s), 0), C.n - 1);
    tau[d] = s - fi[d];
  }
  const int cell = fi[0] + C.n * (fi[1] + C.n * fi[2]);
  int ed[12], f[6];
  cell_dofs(g, cell, ed, f);
  for (int d = 0; d < 3; ++d) {
    int o1, o2;
    other_axes(d, o1, o2);
    const double area = C.h[o1] * C.h[o2];
    const double gk = dJdu[3 * (size_t)k + d];
    atomicAdd(e + C.dof_off + f[2 * d], gk * (1.0 - tau[d]) / area);
    atomicAdd(e + C.dof_off + f[2 * d + 1], gk * tau[d] / area);
  }
}

// Face load b_f = (v_f, f) of every fine face (2x2x2 Gauss, the vector trig load).
__global__ void __launch_bounds__(kAdjThreads) nr_adj_face_load_kernel(const NRCell *__restrict__ cells,
                                                                       msfec_load load, double *__restrict__ b) {
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  NRGeom g;
  g.n = C.n;
  g.L = C.depth;
  nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
  g.N = g.NE + g.NF;
  if (load.kind != MSFEC_LOAD_VEC_TRIG) return;
  const int n = g.n, nc = n * n * n;
  const double w = load.params[1] * M_PI, p0 = load.params[0];
  const double gq = 0.5 / sqrt(3.0);
  const double qp[2] = {0.5 - gq, 0.5 + gq};
  const double jxw = 0.125 * C.h[0] * C.h[1] * C.h[2];
  for (int cell = threadIdx.x; cell < nc; cell += kAdjThreads) {
    const int i = cell & (n - 1), j = (cell >> g.L) & (n - 1), k = cell >> (2 * g.L);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < 8; ++q) {
      const double xl[3] = {qp[q & 1], qp[(q >> 1) & 1], qp[q >> 2]};
      const double X = C.origin[0] + (i + xl[0]) * C.h[0], Y = C.origin[1] + (j + xl[1]) * C.h[1],
                   Z = C.origin[2] + (k + xl[2]) * C.h[2];
      const double sx = sin(w * X), sy = sin(w * Y), sz = sin(w * Z);
      const double fv[3] = {p0 * sy * sz, p0 * sz * sx, p0 * sx * sy};
      for (int d = 0; d < 3; ++d) {
        int o1, o2;
        other_axes(d, o1, o2);
        const double sc = jxw * fv[d] / (C.h[o1] * C.h[o2]);
        acc[2 * d] += sc * (1.0 - xl[d]);
        acc[2 * d + 1] += sc * xl[d];
      }
    }
    int ed[12], f[6];
    cell_dofs(g, cell, ed, f);
    for (int t = 0; t < 6; ++t) atomicAdd(b + C.dof_off + f[t], acc[t]);
  }
}

// Right-hand sides of the four adjoint solves (see above). work[4][N] per cell
// (at 4 dof_off): s, S t, A s, A S t.
__global__ void __launch_bounds__(kAdjThreads) nr_adj_rhs_kernel(const NRCell *__restrict__ cells,
                                                                 const double *__restrict__ ainv6,
                                                                 const double *__restrict__ bdiv,
                                                                 const double *__restrict__ comb,
                                                                 const double *__restrict__ bload,
                                                                 const double *__restrict__ e,
                                                                 double *__restrict__ work, double *__restrict__ rhs,
                                                                 double *__restrict__ scale2_out) {
  __shared__ NRFactors<double> F;
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  NRGeom g;
  g.n = C.n;
  g.L = C.depth;
  nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
  g.N = g.NE + g.NF;
  const int N = g.N, n = g.n, nc = n * n * n;
  if (threadIdx.x == 0) make_factors(C.h, F);
  const double *cb = comb + kNRSrcRhs * C.dof_off;
  double *s = work + kNRSrcRhs * C.dof_off, *st = s + N, *as = st + N, *ast = as + N;
  for (int d = threadIdx.x; d < N; d += kAdjThreads) {
    const bool edge = d < g.NE;
    s[d] = edge ? cb[(size_t)N + d] : cb[3 * (size_t)N + d];  // sigma of Phi_E U, u of Phi_F U
    st[d] = edge ? cb[d] : -cb[2 * (size_t)N + d];           // S (sigma of Phi_E lambda, u of Phi_F lambda)
    as[d] = 0.0;
    ast[d] = 0.0;
  }
  __syncthreads();
  const double invV = 1.0 / (C.h[0] * C.h[1] * C.h[2]);
  const double *ag = ainv6 + 6 * C.coef_off;
  const double *bg = bdiv + C.coef_off;
  for (int cell = threadIdx.x; cell < nc; cell += kAdjThreads) {
    int ed[12], f[6];
    cell_dofs(g, cell, ed, f);
    const bool eb[12] = {}, fb[6] = {};
    const double ai[6] = {ag[6 * cell], ag[6 * cell + 1], ag[6 * cell + 2], ag[6 * cell + 3], ag[6 * cell + 4],
                          ag[6 * cell + 5]};
    cell_apply_s<double, double, double, 0, false>(s, as, F, ai, bg[cell] * invV, ed, f, eb, fb);
    cell_apply_s<double, double, double, 0, false>(st, ast, F, ai, bg[cell] * invV, ed, f, eb, fb);
  }
  __syncthreads();
  double *r = rhs + kNRSrcRhs * C.dof_off;
  const double *bl = bload + C.dof_off, *ee = e + C.dof_off;
  double scale2 = 0.0;
  for (int d = threadIdx.x; d < N; d += kAdjThreads) {
    int dir, i, j, k;
    const bool bnd = dof_geometry(g, d, dir, i, j, k);
    const bool edge = d < g.NE;
    const double at = edge ? ast[d] : -ast[d];  // (A^T t)_d = S_d (A S t)_d
    double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
    if (!bnd) {
      if (edge) {
        r0 = -as[d];
        r1 = -at;
      } else {
        r2 = -(bl[d] - as[d]);
        r3 = -(ee[d] - at);
      }
    }
    r[d] = r0;
    r[(size_t)N + d] = r1;
    r[2 * (size_t)N + d] = r2;
    r[3 * (size_t)N + d] = r3;
    // squared scale of the terms whose difference the right-hand sides are
    // (the solver weights it with its preconditioner into the stopping floor)
    scale2_out[C.dof_off + d] = bnd ? 0.0 : as[d] * as[d] + at * at + bl[d] * bl[d] + ee[d] * ee[d];
  }
}

// x^T M_e y over the 12 edges of one fine cell (edge-mass part of cell_apply_s).
__device__ __forceinline__ double edge_mass_form(const NRFactors<double> &F, const double (&ai)[6],
                                                 const double (&x)[12], const double (&y)[12]) {
  const double A[3][3] = {{ai[0], ai[3], ai[4]}, {ai[3], ai[1], ai[5]}, {ai[4], ai[5], ai[2]}};
  double my[12];
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const double k = A[p][p] * F.hd[p];
    double t[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) t[l] = 2.0 * y[4 * p + l] + y[4 * p + (l ^ 1)];
#pragma unroll
    for (int l = 0; l < 4; ++l) my[4 * p + l] = k * (2.0 * t[l] + t[l ^ 2]);
  }
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (q == p) continue;
      const int r = 3 - p - q;
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        if (edge_pos(q, m, r))
          s1 += y[4 * q + m];
        else
          s0 += y[4 * q + m];
      }
      const double k = A[p][q] * F.hq[r];
#pragma unroll
      for (int l = 0; l < 4; ++l) my[4 * p + l] += k * (edge_pos(p, l, r) ? s0 + 2.0 * s1 : 2.0 * s0 + s1);
    }
  double out = 0.0;
#pragma unroll
  for (int l = 0; l < 12; ++l) out = fma(x[l], my[l], out);
  return out;
}

// Per fine cell: dJ/dta (edge-mass forms) and dJ/dtb (div-div forms).
__global__ void __launch_bounds__(kAdjThreads) nr_adj_gradient_kernel(const NRCell *__restrict__ cells,
                                                                      const double *__restrict__ ainv6,
                                                                      const double *__restrict__ bdiv,
                                                                      const double *__restrict__ comb,
                                                                      const double *__restrict__ work,
                                                                      const double *__restrict__ xsol,
                                                                      double *__restrict__ ga, double *__restrict__ gb) {
  __shared__ NRFactors<double> F;
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  NRGeom g;
  g.n = C.n;
  g.L = C.depth;
  nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
  g.N = g.NE + g.NF;
  const int N = g.N, n = g.n, nc = n * n * n;
  if (threadIdx.x == 0) make_factors(C.h, F);
  __syncthreads();
  const double *cb = comb + kNRSrcRhs * C.dof_off;
  const double *s = work + kNRSrcRhs * C.dof_off, *st = s + N;
  const double *xs = xsol + kNRSrcRhs * C.dof_off;
  const double invV = 1.0 / (C.h[0] * C.h[1] * C.h[2]);
  for (int cell = threadIdx.x; cell < nc; cell += kAdjThreads) {
    int ed[12], f[6];
    cell_dofs(g, cell, ed, f);
    const double *a = ainv6 + 6 * (C.coef_off + cell);
    const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
    double xe[12], ye[12];
    // t^T M s and t^T D s (t = S (S t): sigma part of st as is, u part negated)
#pragma unroll
    for (int l = 0; l < 12; ++l) {
      xe[l] = st[ed[l]];
      ye[l] = s[ed[l]];
    }
    double qa = edge_mass_form(F, ai, xe, ye);
    double dt = 0.0, ds = 0.0;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const double sg = (t & 1) ? 1.0 : -1.0;
      dt += sg * -st[f[t]];
      ds += sg * s[f[t]];
    }
    double qd = dt * ds;
#pragma unroll
    for (int k = 0; k < kNRSrcRhs; ++k) {
      const double *xk = xs + (size_t)k * N, *ck = cb + (size_t)k * N;
#pragma unroll
      for (int l = 0; l < 12; ++l) {
        xe[l] = xk[ed[l]];  // eta_k = S x_k: sigma part unchanged
        ye[l] = ck[ed[l]];
      }
      qa += edge_mass_form(F, ai, xe, ye);
      double dx = 0.0, dy = 0.0;
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const double sg = (t & 1) ? 1.0 : -1.0;
        dx += sg * -xk[f[t]];  // u part of eta_k = -x_k
        dy += sg * ck[f[t]];
      }
      qd += dx * dy;
    }
    ga[C.coef_off + cell] = qa;
    gb[C.coef_off + cell] = -bdiv[C.coef_off + cell] * invV * qd;
  }
}

// ---------------- multilevel preconditioner setup ----------------
constexpr int kMLSetupThreads = 512;

// Values at fine face (d, q, x, y) of the level-(n >> k) functions: up to two
// (index, weight, plane) triples; the hat along the normal times the flux share.
__device__ __forceinline__ int ml_fine_weights(int L, int k, int d, int q, int x, int y, int (&j)[2], float (&w)[2],
                                               int (&P)[2]) {
  const int lm = L - k, m = 1 << lm, r = 1 << k;
  const int a = x >> k, b = y >> k, P0 = q >> k, rem = q & (r - 1);
  const float inv = 1.0f / (float)(r * r);
  int cnt = 0;
  if (P0 >= 1 && P0 <= m - 1) {
    j[cnt] = ml_index(lm, d, P0, a, b);
    P[cnt] = P0;
    w[cnt++] = (float)(r - rem) / (float)r * inv;
  }
  if (rem != 0 && P0 + 1 >= 1 && P0 + 1 <= m - 1) {
    j[cnt] = ml_index(lm, d, P0 + 1, a, b);
    P[cnt] = P0 + 1;
    w[cnt++] = (float)rem / (float)r * inv;
  }
  return cnt;
}

// One CTA per coarse cell (persistent over the batch): for the cell's levels
// n/2 .. 4 the inverse diagonal of P_m^T S P_m and for level 2 the inverse of
// the 12 x 12 P_2^T S P_2, S = D + C^T diag(M)^-1 C on the interior faces. S is
// applied as two masked passes of the element operator (faces -> edges, edge
// scaling by diag(M)^-1, edges -> faces); it couples faces up to two fine
// planes apart along their normal (face -> edges of both adjacent cells ->
// their faces) and one cell across. A diagonal level is probed colour by
// colour (normal d, P mod 3, a and b mod 2: functions of one colour then have
// disjoint S-neighbourhoods, so one application of S to their sum gives all
// their diagonal entries: 36 probes per level); level 2 function by function.
// scratch per CTA: edge diagonal, probe vector, two accumulators (4 Np floats).
__global__ void __launch_bounds__(kMLSetupThreads) nr_ml_setup_kernel(const NRCell *__restrict__ cells, int ncells,
                                                                     const double *__restrict__ ainv6,
                                                                     const double *__restrict__ bdiv,
                                                                     float *__restrict__ coarse,
                                                                     float *__restrict__ scratch,
                                                                     size_t scratch_floats) {
  __shared__ NRShared sh;
  __shared__ double s2[144];
  float *acc = reinterpret_cast<float *>(nr_dyn_smem);  // the cell's data, accumulated then inverted
  constexpr int NT = kMLSetupThreads;
  const int tid = threadIdx.x;
  for (int cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    const NRCell Cc = cells[cell];
    if (Cc.coarse_off < 0) continue;  // block-uniform
    NRGeom g;
    g.n = Cc.n;
    g.L = Cc.depth;
    nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
    g.N = g.NE + g.NF;
    const int n = g.n, N = g.N, nc = n * n * n, L = g.L;
    const size_t Np = ((size_t)N + 63) / 64 * 64;
    float *md = scratch + (size_t)blockIdx.x * scratch_floats;
    float *x = md + Np, *a1 = x + Np, *a2 = a1 + Np;
    const double invV = 1.0 / (Cc.h[0] * Cc.h[1] * Cc.h[2]);
    const double *ag = ainv6 + 6 * Cc.coef_off;
    const double *bg = bdiv + Cc.coef_off;
    if (tid == 0) make_factors(Cc.h, sh.Ff);
    for (int t = tid; t < 144; t += NT) {
      const int p = t / 48, q = (t / 16) % 3, l4 = (t / 4) % 4, m4 = t % 4;
      sh.Gf[p][q][l4][m4] = (float)table_G(Cc.h, p, q, l4, m4);
    }
    const int nd = nr_ml_data_floats(n);
    for (int t = tid; t < nd; t += NT) acc[t] = 0.0f;
    for (int d = tid; d < N; d += NT) md[d] = 0.0f;
    __syncthreads();
    for (int c = tid; c < nc; c += NT) {
      int e[12], f[6];
      cell_dofs(g, c, e, f);
      const double *a = ag + 6 * (size_t)c;
#pragma unroll
      for (int l = 0; l < 12; ++l) atomicAdd(md + e[l], (float)a[l >> 2] * sh.Gf[l >> 2][l >> 2][l & 3][l & 3]);
    }
    __syncthreads();
    // probe loop: 36 colours of single fine faces (the assembled diagonal of S,
    // written straight to the cell's fine block), 36 (K - 1) diagonal-level
    // colours, then the 12 level-2 functions
    const int K = L - 1;
    const int nprobe = 36 + 36 * (K - 1) + 12;
    float *fine_out = coarse + Cc.coarse_off + nd;
    for (int u = tid; u < g.NF; u += NT) fine_out[u] = 0.0f;  // boundary faces keep 0
    for (int pr = 0; pr < nprobe; ++pr) {
      const bool fine = pr < 36;
      const int pl = pr - 36;
      const bool exact = !fine && pl >= 36 * (K - 1);
      const int k = fine ? 0 : (exact ? K : 1 + pl / 36);  // level 2^(L-k); k = 0: the fine faces
      const int col = fine ? pr : pl % 36;
      const int cd = col / 12, cP = (col >> 2) % 3, ca = (col >> 1) & 1, cb = col & 1;
      const int J = pl - 36 * (K - 1);  // exact: the probed function
      int od = 0;  // data offset of level k
      for (int kk = 1; kk < k; ++kk) od += nr_ml_count(1 << (L - kk));
      // probe vector on the interior faces; accumulators cleared
      for (int d = tid; d < N; d += NT) {
        float v = 0.0f;
        if (d >= g.NE) {
          int dir, i, jj, kk;
          const bool fbnd = dof_geometry(g, d, dir, i, jj, kk);
          const int fd = dir - 3;
          const int q = fd == 0 ? i : (fd == 1 ? jj : kk);
          const int xx = fd == 0 ? jj : i, yy = fd == 2 ? jj : kk;
          if (fine) {
            v = (!fbnd && fd == cd && q % 3 == cP && (xx & 1) == ca && (yy & 1) == cb) ? 1.0f : 0.0f;
            x[d] = v;
            a1[d] = 0.0f;
            a2[d] = 0.0f;
            continue;
          }
          int fj[2], fP[2];
          float fw[2];
          const int cnt = ml_fine_weights(L, k, fd, q, xx, yy, fj, fw, fP);
          for (int t = 0; t < cnt; ++t) {
            if (exact) {
              if (fj[t] == J) v += fw[t];
            } else if (fd == cd && fP[t] % 3 == cP && ((xx >> k) & 1) == ca && ((yy >> k) & 1) == cb) {
              v += fw[t];
            }
          }
        }
        x[d] = v;
        a1[d] = 0.0f;
        a2[d] = 0.0f;
      }
      __syncthreads();
      const bool eb[12] = {}, fb[6] = {};
      for (int c = tid; c < nc; c += NT) {  // a1 = A (0, x)
        int e[12], f[6];
        cell_dofs(g, c, e, f);
        const double *a = ag + 6 * (size_t)c;
        const float ai[6] = {(float)a[0], (float)a[1], (float)a[2], (float)a[3], (float)a[4], (float)a[5]};
        cell_apply_s<float, float, float, 3, false>(x, a1, sh.Ff, ai, (float)(bg[c] * invV), e, f, eb, fb);
      }
      __syncthreads();
      for (int d = tid; d < g.NE; d += NT) {  // t = diag(M)^-1 C x on the interior edges (A (0, x) = (-C x, D x))
        int dir, i, jj, kk;
        const bool bnd = dof_geometry(g, d, dir, i, jj, kk);
        x[d] = (!bnd && md[d] > 0.0f) ? -a1[d] / md[d] : 0.0f;
      }
      __syncthreads();
      for (int c = tid; c < nc; c += NT) {  // a2 = A (t, 0) = (M t, C^T t)
        int e[12], f[6];
        cell_dofs(g, c, e, f);
        const double *a = ag + 6 * (size_t)c;
        const float ai[6] = {(float)a[0], (float)a[1], (float)a[2], (float)a[3], (float)a[4], (float)a[5]};
        cell_apply_s<float, float, float, 2, false>(x, a2, sh.Ff, ai, (float)(bg[c] * invV), e, f, eb, fb);
      }
      __syncthreads();
      for (int d = g.NE + tid; d < N; d += NT) {  // (S x)_f = a1_f + a2_f against the probed functions
        int dir, i, jj, kk;
        const bool bnd = dof_geometry(g, d, dir, i, jj, kk);
        if (bnd) continue;
        const float sf = a1[d] + a2[d];
        const int fd = dir - 3;
        const int q = fd == 0 ? i : (fd == 1 ? jj : kk);
        const int xx = fd == 0 ? jj : i, yy = fd == 2 ? jj : kk;
        if (fine) {  // faces of one colour are S-decoupled: (S x)_f = S_ff
          if (fd == cd && q % 3 == cP && (xx & 1) == ca && (yy & 1) == cb)
            fine_out[d - g.NE] = sf > 0.0f ? 1.0f / sf : 0.0f;
          continue;
        }
        int fj[2], fP[2];
        float fw[2];
        const int cnt = ml_fine_weights(L, k, fd, q, xx, yy, fj, fw, fP);
        for (int t = 0; t < cnt; ++t) {
          if (exact) {
            atomicAdd(acc + od + fj[t] * 12 + J, fw[t] * sf);
          } else if (fd == cd && fP[t] % 3 == cP && ((xx >> k) & 1) == ca && ((yy >> k) & 1) == cb) {
            atomicAdd(acc + od + fj[t], fw[t] * sf);
          }
        }
      }
      __syncthreads();
    }
    // invert: diagonal levels entrywise; level 2 by Gauss-Jordan (FP64, symmetrised)
    int od2 = 0;
    for (int kk = 1; kk < K; ++kk) od2 += nr_ml_count(1 << (L - kk));
    for (int t = tid; t < od2; t += NT) acc[t] = acc[t] > 0.0f ? 1.0f / acc[t] : 0.0f;
    for (int t = tid; t < 144; t += NT) {
      const int r = t / 12, c = t % 12;
      s2[t] = 0.5 * ((double)acc[od2 + r * 12 + c] + (double)acc[od2 + c * 12 + r]);
    }
    __syncthreads();
    if (tid == 0) {
      double inv[144];
      for (int t = 0; t < 144; ++t) inv[t] = (t / 12 == t % 12) ? 1.0 : 0.0;
      bool ok = true;
      for (int c = 0; c < 12 && ok; ++c) {
        int piv = c;
        for (int r = c + 1; r < 12; ++r)
          if (fabs(s2[r * 12 + c]) > fabs(s2[piv * 12 + c])) piv = r;
        if (!(fabs(s2[piv * 12 + c]) > 0.0)) {
          ok = false;
          break;
        }
        if (piv != c)
          for (int t = 0; t < 12; ++t) {
            double u = s2[c * 12 + t];
            s2[c * 12 + t] = s2[piv * 12 + t];
            s2[piv * 12 + t] = u;
            u = inv[c * 12 + t];
            inv[c * 12 + t] = inv[piv * 12 + t];
            inv[piv * 12 + t] = u;
          }
        const double ip = 1.0 / s2[c * 12 + c];
        for (int t = 0; t < 12; ++t) {
          s2[c * 12 + t] *= ip;
          inv[c * 12 + t] *= ip;
        }
        for (int r = 0; r < 12; ++r) {
          if (r == c) continue;
          const double fct = s2[r * 12 + c];
          if (fct == 0.0) continue;
          for (int t = 0; t < 12; ++t) {
            s2[r * 12 + t] -= fct * s2[c * 12 + t];
            inv[r * 12 + t] -= fct * inv[c * 12 + t];
          }
        }
      }
      for (int r = 0; r < 12; ++r)
        for (int c = 0; c < 12; ++c)  // symmetric by construction of the stored value
          acc[od2 + r * 12 + c] = ok ? (float)(0.5 * (inv[r * 12 + c] + inv[c * 12 + r])) : 0.0f;
    }
    __syncthreads();
    float *out = coarse + Cc.coarse_off;
    for (int t = tid; t < nd; t += NT) out[t] = acc[t];
    __syncthreads();
  }
}

}  // namespace nrimpl

template <typename T, int NT, bool ML, int PLACE>
static cudaError_t launch_solve_p(const NRParams &prm, size_t smem, int grid, cudaStream_t st, bool carveout) {
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

template <typename T, int NT, bool ML>
static cudaError_t launch_solve(const NRParams &prm, size_t smem, int grid, cudaStream_t st, bool carveout) {
  if constexpr (NT == 256) {
    return launch_solve_p<T, NT, ML, 1>(prm, smem, grid, st, carveout);
  } else {
    if (prm.use_smem) return launch_solve_p<T, NT, ML, 1>(prm, smem, grid, st, carveout);
    if constexpr (sizeof(T) == 4)
      if (prm.stage) return launch_solve_p<T, NT, ML, 2>(prm, smem, grid, st, carveout);
    return launch_solve_p<T, NT, ML, 0>(prm, smem, grid, st, carveout);
  }
}

// ml: the multilevel variant (prm.coarse set); smem includes its region.
cudaError_t nedrt_solve_launch(bool fp64, bool ml, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (fp64) return ml ? launch_solve<double, kNRThreads, true>(prm, smem, grid, st, false)
                      : launch_solve<double, kNRThreads, false>(prm, smem, grid, st, false);
  return ml ? launch_solve<float, kNRThreads, true>(prm, smem, grid, st, false)
            : launch_solve<float, kNRThreads, false>(prm, smem, grid, st, false);
}

// Mixed precision, two 256-thread CTAs per SM with the split workspace
// (shared: preconditioner + 6 FP32 vectors; global slot: x + coefficients).
cudaError_t nedrt_solve_launch_split(bool ml, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  return ml ? launch_solve<float, 256, true>(prm, smem, grid, st, true)
            : launch_solve<float, 256, false>(prm, smem, grid, st, true);
}

cudaError_t nedrt_split_occupancy(bool ml, size_t smem, int *blocks_per_sm) {
  auto k = ml ? nrimpl::nedrt_solve_kernel<float, 256, true, 1> : nrimpl::nedrt_solve_kernel<float, 256, false, 1>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, 256, smem);
}

// Multilevel preconditioner data of every cell with coarse_off >= 0.
cudaError_t nedrt_ml_setup_launch(const NRCell *cells, int ncells, const double *ainv6, const double *bdiv,
                                  float *coarse, float *scratch, size_t scratch_floats, size_t smem, int grid,
                                  cudaStream_t st) {
  if (ncells <= 0 || grid <= 0) return cudaSuccess;
  auto k = nrimpl::nr_ml_setup_kernel;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, nrimpl::kMLSetupThreads, smem, st>>>(cells, ncells, ainv6, bdiv, coarse, scratch, scratch_floats);
  return cudaGetLastError();
}

cudaError_t nedrt_galerkin_launch(const NRCell *cells, int ncells, const double *phi, const double *y,
                                  const msfec_load &load, double *KH, double *FH, msfec_cell_report *rep,
                                  const NRStat *stats, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  nrimpl::nedrt_galerkin_kernel<<<ncells, nrimpl::kGalThreads, 0, st>>>(cells, phi, y, load, KH, FH);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !rep) return e;
  nrimpl::nedrt_report_kernel<<<(ncells + 127) / 128, 128, 0, st>>>(stats, ncells, rep);
  return cudaGetLastError();
}


cudaError_t nedrt_adjoint_prepare_launch(const NRCell *cells, int ncells, const double *phi, const double *U,
                                         const double *lam, const msfec_load &load, int npoints, const int *cell_of,
                                         const double *pts, const double *dJdu, const double *ainv6,
                                         const double *bdiv, double *comb, double *bload, double *e, double *work,
                                         double *rhs, double *scale2_out, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  nrimpl::nr_adj_combine_kernel<<<ncells, nrimpl::kAdjThreads, 0, st>>>(cells, phi, U, lam, comb);
  nrimpl::nr_adj_face_load_kernel<<<ncells, nrimpl::kAdjThreads, 0, st>>>(cells, load, bload);
  if (npoints > 0)
    nrimpl::nr_adj_point_kernel<<<(npoints + 127) / 128, 128, 0, st>>>(cells, npoints, cell_of, pts, dJdu, e);
  nrimpl::nr_adj_rhs_kernel<<<ncells, nrimpl::kAdjThreads, 0, st>>>(cells, ainv6, bdiv, comb, bload, e, work, rhs,
                                                                     scale2_out);
  return cudaGetLastError();
}

// Face load b_f = (v_f, f) of every fine face of every cell (b zeroed by the caller).
cudaError_t nedrt_face_load_launch(const NRCell *cells, int ncells, const msfec_load &load, double *b,
                                   cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  nrimpl::nr_adj_face_load_kernel<<<ncells, nrimpl::kAdjThreads, 0, st>>>(cells, load, b);
  return cudaGetLastError();
}

cudaError_t nedrt_adjoint_gradient_launch(const NRCell *cells, int ncells, const double *ainv6, const double *bdiv,
                                          const double *comb, const double *work, const double *xsol, double *ga,
                                          double *gb, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  nrimpl::nr_adj_gradient_kernel<<<ncells, nrimpl::kAdjThreads, 0, st>>>(cells, ainv6, bdiv, comb, work, xsol, ga,
                                                                          gb);
  return cudaGetLastError();
}
}  // namespace msfec
