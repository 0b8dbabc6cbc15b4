// Persistent batched Q1 x Nedelec (Q_Ned) local solver and Galerkin product (sm_103a).
//
// Restates, for every coarse cell x coarse basis function (8 H1 + 12 curl),
// the reference's mixed local problem of the Q_Ned pairing (konsim83/MPI-MSFEC,
// source/Q_Ned/q_ned_basis.cc): sigma in Q1 (vertices), u in lowest-order
// Nedelec (edges), local matrix (q_ned_basis.cc:483-491)
//   [ B^-1 M_Q1      -(grad tau, u) ]   =  [ Mv   -Gm^T ]
//   [ (v, grad sigma) (A curl u, curl v) ]   [ Gm    Kc  ]
// boundary data (setup_basis_dofs_h1 / _curl, :223-354): H1 basis v: sigma =
// coarse Q1 function, u x n = its gradient; curl basis l: sigma = 0, u x n =
// coarse Nedelec function; right-hand side (v, grad phi_v^coarse) on the edge
// rows of the H1 bases (full_rhs, :498-505). The element blocks are applied
// in factored form, exact for lowest order on a box: grad of a Q1 function is
// the Nedelec function whose edge DoFs are end-minus-start differences, so
// Gm = M_N Grad (M_N the unweighted Nedelec mass); the curl of a Nedelec
// function is the RT0 function whose fluxes are the face circulations, so
// Kc = C^T M_RT(A) C. Solved like the Ned_RT pairing: MINRES on the symmetric
// form (edge rows negated), preconditioner diag(Mv)^-1 (+) diag(Kc + Gm
// diag(Mv)^-1 Gm^T)^-1, FP32 inside FP64 iterative refinement, two block-wide
// phases per iteration. The last FP64 pass writes y_b = A P_b for the Galerkin
// product of assemble_global_element_matrix (:841-940).
#include "../../include/msfec_cuda.h"
#include "qned_common.cuh"

namespace msfec {
namespace qnimpl {

struct QNGeom {
  int n, L, NV, NEx, NE, N;
};

__device__ __forceinline__ double psi(int a, double t) { return a ? t : 1.0 - t; }

// The two axes other than p, in increasing order.
__device__ __forceinline__ void other_axes(int p, int &o1, int &o2) {
  o1 = p == 0 ? 1 : 0;
  o2 = p == 2 ? 1 : 2;
}

// Local index 0..3 of the edge of direction p at positions (pos[] on the other axes).
__host__ __device__ constexpr int edge_local(int p, int px, int py, int pz) {
  return p == 0 ? 4 * 0 + py + 2 * pz : (p == 1 ? 4 * 1 + px + 2 * pz : 4 * 2 + px + 2 * py);
}

// Local vertex (x + 2y + 4z) at the start (end = 0) or end (end = 1) of local edge l.
__host__ __device__ constexpr int edge_vertex(int l, int end) {
  return (l >> 2) == 0 ? end + 2 * (l & 1) + 4 * ((l >> 1) & 1)
                       : ((l >> 2) == 1 ? (l & 1) + 2 * end + 4 * ((l >> 1) & 1) : (l & 1) + 2 * ((l >> 1) & 1) + 4 * end);
}

// Per-item constants of the factored element operator (cell sides h).
template <typename TA>
struct QNFactors {
  TA hv;        // |K| / 216: vertex mass per unit B^-1 in the (2,1)^3 pattern
  TA hd[3];     // h_o1 h_o2 / (36 h_p): Nedelec mass block of direction p (unit weight)
  TA rd[3];     // h_d^2 / (6 |K|): RT0 mass, same normal, (2,1) pattern per unit A_dd
  TA ro[3][3];  // h_d h_e / (4 |K|): RT0 mass, normals d != e, per unit A_de
};

template <typename TA>
__device__ __forceinline__ void make_factors(const double h[3], QNFactors<TA> &F) {
  const double V = h[0] * h[1] * h[2];
  F.hv = (TA)(V / 216.0);
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    int o1, o2;
    other_axes(p, o1, o2);
    F.hd[p] = (TA)(h[o1] * h[o2] / (36.0 * h[p]));
    F.rd[p] = (TA)(h[p] * h[p] / (6.0 * V));
#pragma unroll
    for (int e = 0; e < 3; ++e) F.ro[p][e] = (TA)(h[p] * h[e] / (4.0 * V));
  }
}

// y = M_N x over the 12 local edges (unweighted Nedelec mass: per direction the
// Kronecker product of the 1D P1 masses along the two other axes).
template <typename TA>
__device__ __forceinline__ void nedelec_mass(const QNFactors<TA> &F, const TA (&x)[12], TA (&y)[12]) {
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    TA t[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) t[l] = TA(2) * x[4 * p + l] + x[4 * p + (l ^ 1)];
#pragma unroll
    for (int l = 0; l < 4; ++l) y[4 * p + l] = F.hd[p] * (TA(2) * t[l] + t[l ^ 2]);
  }
}

// Face circulations c = C z (face f = 2d + s, counterclockwise seen from +e_d).
template <typename TA>
__device__ __forceinline__ void circulations(const TA (&z)[12], TA (&c)[6]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int o1 = (d + 1) % 3, o2 = (d + 2) % 3;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      int pa[3], pb[3], pc[3], pe[3];  // positions of the four edges
      pa[d] = pb[d] = pc[d] = pe[d] = s;
      pa[o2] = 0;  // +o1 edge at o2 = 0
      pb[o1] = 1;  // +o2 edge at o1 = 1
      pc[o2] = 1;  // -o1 edge at o2 = 1
      pe[o1] = 0;  // -o2 edge at o1 = 0
      pa[o1] = pc[o1] = 0;
      pb[o2] = pe[o2] = 0;
      c[2 * d + s] = z[edge_local(o1, pa[0], pa[1], pa[2])] + z[edge_local(o2, pb[0], pb[1], pb[2])] -
                     z[edge_local(o1, pc[0], pc[1], pc[2])] - z[edge_local(o2, pe[0], pe[1], pe[2])];
    }
  }
}

// y += C^T w (transpose of circulations).
template <typename TA>
__device__ __forceinline__ void circulations_t(const TA (&w)[6], TA (&y)[12]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int o1 = (d + 1) % 3, o2 = (d + 2) % 3;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      int pa[3], pb[3], pc[3], pe[3];
      pa[d] = pb[d] = pc[d] = pe[d] = s;
      pa[o2] = 0;
      pb[o1] = 1;
      pc[o2] = 1;
      pe[o1] = 0;
      pa[o1] = pc[o1] = 0;
      pb[o2] = pe[o2] = 0;
      const TA v = w[2 * d + s];
      y[edge_local(o1, pa[0], pa[1], pa[2])] += v;
      y[edge_local(o2, pb[0], pb[1], pb[2])] += v;
      y[edge_local(o1, pc[0], pc[1], pc[2])] -= v;
      y[edge_local(o2, pe[0], pe[1], pe[2])] -= v;
    }
  }
}

// w = M_RT(A) c for the 6 local faces.
template <typename TA>
__device__ __forceinline__ void rt_mass(const QNFactors<TA> &F, const TA (&A)[3][3], const TA (&c)[6], TA (&w)[6]) {
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      TA acc = A[d][d] * F.rd[d] * (TA(2) * c[2 * d + s] + c[2 * d + (s ^ 1)]);
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        if (e == d) continue;
        acc += A[d][e] * F.ro[d][e] * (c[2 * e] + c[2 * e + 1]);
      }
      w[2 * d + s] = acc;
    }
}

// Element operator of one fine cell, out += A_e z_e (8 vertex + 12 edge DoFs,
// atomically). MASK: 0 none, 1 keep only lattice-boundary values of z (lift
// of the Dirichlet data), 2 keep only vertex values, 3 keep only edge values.
// With DOT returns sum_d S_d z_d (A_e z_e)_d, S = +1 on vertices, -1 on edges.
// MERGE: the warp holds complete x-rows of consecutive cells c (n >= 4, all
// lanes active): contributions to the DoFs shared with the x-neighbour (4
// vertices + 4 edges on the plane between them) and then with the
// y-neighbour in the warp (2 vertices + 3 edges) are summed by shuffles before
// the shared-memory atomics.
template <typename TA, typename TV, typename TO, int MASK, bool DOT, bool MERGE = false>
__device__ __forceinline__ TA cell_apply(const TV *__restrict__ z, TO *out, const QNFactors<TA> &F,
                                         const TA (&ai)[6], TA binv, const int (&vi)[8], const int (&ei)[12],
                                         const bool (&vb)[8], const bool (&eb)[12], int c = 0, int L = 0) {
  TA zv[8], ze[12];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const bool keep = MASK == 0 || (MASK == 1 && vb[t]) || MASK == 2;
    zv[t] = keep ? (TA)z[vi[t]] : TA(0);
  }
#pragma unroll
  for (int l = 0; l < 12; ++l) {
    const bool keep = MASK == 0 || (MASK == 1 && eb[l]) || MASK == 3;
    ze[l] = keep ? (TA)z[ei[l]] : TA(0);
  }
  const TA A[3][3] = {{ai[0], ai[3], ai[4]}, {ai[3], ai[1], ai[5]}, {ai[4], ai[5], ai[2]}};
  TA yv[8], ye[12];
  // vertex mass: B^-1 |K| / 216 (2,1)^3
  {
    TA t1[8], t2[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) t1[u] = TA(2) * zv[u] + zv[u ^ 1];
#pragma unroll
    for (int u = 0; u < 8; ++u) t2[u] = TA(2) * t1[u] + t1[u ^ 2];
    const TA k = binv * F.hv;
#pragma unroll
    for (int u = 0; u < 8; ++u) yv[u] = k * (TA(2) * t2[u] + t2[u ^ 4]);
  }
  // edge rows: M_N Grad z_v + C^T M_RT(A) C z_e
  {
    TA g[12];
#pragma unroll
    for (int l = 0; l < 12; ++l) g[l] = zv[edge_vertex(l, 1)] - zv[edge_vertex(l, 0)];
    nedelec_mass(F, g, ye);
    TA c[6], w[6];
    circulations(ze, c);
    rt_mass(F, A, c, w);
    circulations_t(w, ye);
  }
  // vertex rows: - Grad^T M_N z_e
  {
    TA mz[12];
    nedelec_mass(F, ze, mz);
#pragma unroll
    for (int l = 0; l < 12; ++l) {
      yv[edge_vertex(l, 1)] -= mz[l];
      yv[edge_vertex(l, 0)] += mz[l];
    }
  }
  TA dot = TA(0);
  if constexpr (DOT) {
#pragma unroll
    for (int t = 0; t < 8; ++t) dot += zv[t] * yv[t];
#pragma unroll
    for (int l = 0; l < 12; ++l) dot -= ze[l] * ye[l];
  }
  if constexpr (MERGE) {
    const int n = 1 << L, lane = threadIdx.x & 31;
    const int i = c & (n - 1), j = (c >> L) & (n - 1);
    // plane x = i: vertices 0 2 4 6, y-edges 4 6, z-edges 8 10; plane x = i+1: the same with bit 0 set
    TA lf[8] = {yv[0], yv[2], yv[4], yv[6], ye[4], ye[6], ye[8], ye[10]};
    const TA rt[8] = {yv[1], yv[3], yv[5], yv[7], ye[5], ye[7], ye[9], ye[11]};
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const TA v = __shfl_up_sync(0xffffffffu, rt[t], 1);
      if (i > 0) lf[t] += v;
    }
    if (i == n - 1) {
      atomicAdd(out + vi[1], (TO)rt[0]);
      atomicAdd(out + vi[3], (TO)rt[1]);
      atomicAdd(out + vi[5], (TO)rt[2]);
      atomicAdd(out + vi[7], (TO)rt[3]);
      atomicAdd(out + ei[5], (TO)rt[4]);
      atomicAdd(out + ei[7], (TO)rt[5]);
      atomicAdd(out + ei[9], (TO)rt[6]);
      atomicAdd(out + ei[11], (TO)rt[7]);
    }
    atomicAdd(out + ei[4], (TO)lf[4]);
    atomicAdd(out + ei[6], (TO)lf[5]);
    // plane y = j: vertices 0 4, x-edges 0 2, z-edge 8; plane y = j+1: vertices 2 6, x-edges 1 3, z-edge 10
    TA bt[5] = {lf[0], lf[2], ye[0], ye[2], lf[6]};
    const TA tp[5] = {lf[1], lf[3], ye[1], ye[3], lf[7]};
    const bool below = lane >= n && j > 0;
    const bool above = lane + n < 32 && j < n - 1;
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      const TA v = __shfl_up_sync(0xffffffffu, tp[t], n);
      if (below) bt[t] += v;
    }
    if (!above) {
      atomicAdd(out + vi[2], (TO)tp[0]);
      atomicAdd(out + vi[6], (TO)tp[1]);
      atomicAdd(out + ei[1], (TO)tp[2]);
      atomicAdd(out + ei[3], (TO)tp[3]);
      atomicAdd(out + ei[10], (TO)tp[4]);
    }
    atomicAdd(out + vi[0], (TO)bt[0]);
    atomicAdd(out + vi[4], (TO)bt[1]);
    atomicAdd(out + ei[0], (TO)bt[2]);
    atomicAdd(out + ei[2], (TO)bt[3]);
    atomicAdd(out + ei[8], (TO)bt[4]);
  } else {
#pragma unroll
    for (int t = 0; t < 8; ++t) atomicAdd(out + vi[t], (TO)yv[t]);
#pragma unroll
    for (int l = 0; l < 12; ++l) atomicAdd(out + ei[l], (TO)ye[l]);
  }
  return dot;
}

__device__ __forceinline__ void cell_dofs(const QNGeom &g, int c, int (&v)[8], int (&e)[12]) {
  const int n = g.n, N1 = n + 1;
  const int i = c & (n - 1), j = (c >> g.L) & (n - 1), k = c >> (2 * g.L);
#pragma unroll
  for (int t = 0; t < 8; ++t) v[t] = (i + (t & 1)) + N1 * ((j + ((t >> 1) & 1)) + N1 * (k + (t >> 2)));
  auto ex = [&](int a, int b, int cc) { return g.NV + a + n * (b + (n + 1) * cc); };
  auto ey = [&](int a, int b, int cc) { return g.NV + g.NEx + a + (n + 1) * (b + n * cc); };
  auto ez = [&](int a, int b, int cc) { return g.NV + 2 * g.NEx + a + (n + 1) * (b + (n + 1) * cc); };
  e[0] = ex(i, j, k);
  e[1] = ex(i, j + 1, k);
  e[2] = ex(i, j, k + 1);
  e[3] = ex(i, j + 1, k + 1);
  e[4] = ey(i, j, k);
  e[5] = ey(i + 1, j, k);
  e[6] = ey(i, j, k + 1);
  e[7] = ey(i + 1, j, k + 1);
  e[8] = ez(i, j, k);
  e[9] = ez(i + 1, j, k);
  e[10] = ez(i, j + 1, k);
  e[11] = ez(i + 1, j + 1, k);
}

// (dir, i, j, k) of DoF d (dir -1: vertex); returns true on the lattice boundary.
__device__ bool dof_geometry(const QNGeom &g, int d, int &dir, int &i, int &j, int &k) {
  const int n = g.n, N1 = n + 1;
  if (d < g.NV) {
    dir = -1;
    i = d % N1;
    j = (d / N1) % N1;
    k = d / (N1 * N1);
    return i == 0 || j == 0 || k == 0 || i == n || j == n || k == n;
  }
  const int e = d - g.NV;
  dir = e / g.NEx;
  const int t = e % g.NEx;
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

// Boundary value of coarse basis b at DoF (dir, i, j, k): H1 basis b < 8:
// the coarse Q1 function (BasisQ1, basis_q1.tpp) at vertices, its
// end-minus-start differences on edges; curl basis: 0 at vertices, the coarse
// Nedelec line integral (BasisNedelec, basis_nedelec.tpp:38-85) on edges.
__device__ double coarse_dof(int b, int dir, int i, int j, int k, int n) {
  if (b < 8) {
    auto phi = [&](int x, int y, int z) {
      return psi(b & 1, (double)x / n) * psi((b >> 1) & 1, (double)y / n) * psi(b >> 2, (double)z / n);
    };
    if (dir < 0) return phi(i, j, k);
    return phi(i + (dir == 0), j + (dir == 1), k + (dir == 2)) - phi(i, j, k);
  }
  if (dir < 0) return 0.0;
  const int l = b - 8;
  const int ld[12] = {1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 2, 2};
  const int lp[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
  const int lq[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1};
  if (dir != ld[l]) return 0.0;
  const int t1 = dir == 0 ? j : i;
  const int t2 = dir == 2 ? j : k;
  return psi(lp[l], (double)t1 / n) * psi(lq[l], (double)t2 / n) / n;
}

struct QNShared {
  double wred[kQNWarps][3];
  float fred[kQNWarps][3];
  QNFactors<float> Ff;
  QNFactors<double> Fd;
  alignas(16) float fslot[2][kQNWarps];
  double dslot[2][kQNWarps];
  int item;
};

template <typename VT>
__device__ __forceinline__ void warp_publish(QNShared &sh, int slot, VT v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) {
    if constexpr (sizeof(VT) == 4)
      sh.fslot[slot][threadIdx.x >> 5] = v;
    else
      sh.dslot[slot][threadIdx.x >> 5] = v;
  }
}

template <typename VT, int NW>
__device__ __forceinline__ VT slot_total(const QNShared &sh, int slot) {
  VT s = VT(0);
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    if constexpr (sizeof(VT) == 4)
      s += sh.fslot[slot][w];
    else
      s += sh.dslot[slot][w];
  }
  return s;
}

template <typename VT, int NV, int NW>
__device__ __forceinline__ void block_sum(QNShared &sh, VT (&v)[NV], VT (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < NV; ++t)
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v[t] += __shfl_xor_sync(0xffffffffu, v[t], off);
  __syncthreads();
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

extern __shared__ __align__(256) unsigned char qn_dyn_smem[];

// NT = 512 (one CTA per SM) or 256 (two CTAs per SM, whose barriers and
// scalar recurrences then overlap; the depth-3 workspace fits twice).
template <typename T, bool SMEM, int NT>
__device__ void solve_item(const QNParams &prm, QNShared &sh, int item_id) {
  constexpr int NW = NT / 32;
  float *ws = SMEM ? reinterpret_cast<float *>(qn_dyn_smem) : prm.scratch + (size_t)blockIdx.x * prm.scratch_floats;
  const NRItem it = prm.items[item_id];
  const NRCell Cc = prm.cells[it.cell];
  QNGeom g;
  g.n = Cc.n;
  g.L = Cc.depth;
  qn_counts(g.n, g.NV, g.NEx, g.NE);
  g.N = g.NV + g.NE;
  const int n = g.n, N = g.N;
  const int nc = n * n * n;
  const int bb = it.basis;
  const int tid = threadIdx.x;
  constexpr bool kMixed = sizeof(T) == 4;
  const size_t Np = ((size_t)N + 63) / 64 * 64;
  float *pd = ws;
  T *zt = reinterpret_cast<T *>(ws + Np);
  T *az = zt + Np;
  T *vA = az + Np;
  T *vB = vA + Np;
  T *wA = vB + Np;
  T *wB = wA + Np;
  T *xk = wB + Np;
  float *cf = ws + Np + 7 * Np * (sizeof(T) / 4);
  double *dacc = reinterpret_cast<double *>(ws + Np);  // FP64 residual accumulator, aliases zt..
  float *facc = ws + Np;
  if (tid == 0) {
    make_factors(Cc.h, sh.Ff);
    make_factors(Cc.h, sh.Fd);
  }
  const QNFactors<float> &Ff = sh.Ff;
  const QNFactors<double> &Fd = sh.Fd;
  const double *ag = prm.a6 + 6 * Cc.coef_off;
  const double *bg = prm.binv + Cc.coef_off;
  double *phi = prm.phi + (size_t)kQNBases * Cc.dof_off + (size_t)bb * N;
  double *yout = prm.y + (size_t)kQNBases * Cc.dof_off + (size_t)bb * N;
  for (int c = tid; c < nc; c += NT) {
#pragma unroll
    for (int q = 0; q < 6; ++q) cf[8 * c + q] = (float)ag[6 * (size_t)c + q];
    cf[8 * c + 6] = (float)bg[c];
    cf[8 * c + 7] = 0.0f;
  }
  for (int d = tid; d < (int)Np; d += NT) pd[d] = 0.0f;
  __syncthreads();

  // ---- preconditioner: diag(Mv) on vertices, then diag(Kc) + sum_v Gm_ev^2 / Mv_vv on edges
  for (int c = tid; c < nc; c += NT) {
    int v[8], e[12];
    cell_dofs(g, c, v, e);
    const float d8 = cf[8 * c + 6] * Ff.hv * 8.0f;
#pragma unroll
    for (int t = 0; t < 8; ++t) atomicAdd(pd + v[t], d8);
  }
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int v[8], e[12];
    cell_dofs(g, c, v, e);
    const float *a = cf + 8 * c;
    const float A[3][3] = {{a[0], a[3], a[4]}, {a[3], a[1], a[5]}, {a[4], a[5], a[2]}};
    float diag[12];
    // diag of C^T M_RT C: each edge bounds two faces
#pragma unroll
    for (int l = 0; l < 12; ++l) {
      float z[12];
#pragma unroll
      for (int t = 0; t < 12; ++t) z[t] = t == l ? 1.0f : 0.0f;
      float cc[6], w[6], y[12];
      circulations(z, cc);
      rt_mass(Ff, A, cc, w);
#pragma unroll
      for (int t = 0; t < 12; ++t) y[t] = 0.0f;
      circulations_t(w, y);
      diag[l] = y[l];
    }
    // + sum_v Gm[e][v]^2 / Mv_vv, Gm column v = M_N Grad e_v
    float inv_mv[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) inv_mv[t] = 1.0f / pd[v[t]];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      float gcol[12], mg[12];
#pragma unroll
      for (int l = 0; l < 12; ++l) gcol[l] = (edge_vertex(l, 1) == t ? 1.0f : 0.0f) - (edge_vertex(l, 0) == t ? 1.0f : 0.0f);
      nedelec_mass(Ff, gcol, mg);
#pragma unroll
      for (int l = 0; l < 12; ++l) diag[l] += mg[l] * mg[l] * inv_mv[t];
    }
#pragma unroll
    for (int l = 0; l < 12; ++l) atomicAdd(pd + e[l], diag[l]);
  }
  __syncthreads();
  for (int d = tid; d < N; d += NT) {
    int dir, i, j, k;
    const bool bnd = dof_geometry(g, d, dir, i, j, k);
    pd[d] = bnd ? 0.0f : 1.0f / pd[d];
  }
  __syncthreads();

  double bnorm2 = 0.0, rnorm2 = 0.0;
  int conv = 0, its = 0, flags = 0, nref = 0;
  for (int ir = 0;; ++ir) {
    const bool fp32_res = kMixed && ir == 0;
    if (ir == 0) {
      for (int d = tid; d < N; d += NT) {
        int dir, i, j, k;
        dof_geometry(g, d, dir, i, j, k);
        phi[d] = coarse_dof(bb, dir, i, j, k, n);
      }
      __syncthreads();
    }
    double part[2] = {0.0, 0.0};
    for (int pass = (ir == 0 ? 0 : 1); pass < 2; ++pass) {
      if (fp32_res) {
        for (int d = tid; d < N; d += NT) facc[d] = 0.0f;
      } else {
        for (int d = tid; d < N; d += NT) dacc[d] = 0.0;
      }
      __syncthreads();
      for (int c = tid; c < nc; c += NT) {
        int v[8], e[12];
        cell_dofs(g, c, v, e);
        bool vb[8], eb[12];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          int dir, i, j, k;
          vb[t] = dof_geometry(g, v[t], dir, i, j, k);
        }
#pragma unroll
        for (int l = 0; l < 12; ++l) {
          int dir, i, j, k;
          eb[l] = dof_geometry(g, e[l], dir, i, j, k);
        }
        // H1 basis: right-hand side (v, grad phi_b^coarse) = M_N Grad(phi_b at the cell's vertices)
        double rc[12];
        const bool has_rhs = bb < 8;
        if (has_rhs) {
          double pv[8];
          const int ci = c & (n - 1), cj = (c >> g.L) & (n - 1), ck = c >> (2 * g.L);
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int x = ci + (t & 1), y = cj + ((t >> 1) & 1), z = ck + (t >> 2);
            pv[t] = psi(bb & 1, (double)x / n) * psi((bb >> 1) & 1, (double)y / n) * psi(bb >> 2, (double)z / n);
          }
          double gl[12];
#pragma unroll
          for (int l = 0; l < 12; ++l) gl[l] = pv[edge_vertex(l, 1)] - pv[edge_vertex(l, 0)];
          nedelec_mass(Fd, gl, rc);
        }
        if (fp32_res) {
          const float *a = cf + 8 * c;
          const float ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          if (pass == 0)
            cell_apply<float, double, float, 1, false>(phi, facc, Ff, ai, a[6], v, e, vb, eb);
          else
            cell_apply<float, double, float, 0, false>(phi, facc, Ff, ai, a[6], v, e, vb, eb);
          if (has_rhs)
#pragma unroll
            for (int l = 0; l < 12; ++l) atomicAdd(facc + e[l], (float)-rc[l]);
        } else {
          const double *a = ag + 6 * (size_t)c;
          const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          if (pass == 0)
            cell_apply<double, double, double, 1, false>(phi, dacc, Fd, ai, bg[c], v, e, vb, eb);
          else
            cell_apply<double, double, double, 0, false>(phi, dacc, Fd, ai, bg[c], v, e, vb, eb);
          if (has_rhs)
#pragma unroll
            for (int l = 0; l < 12; ++l) atomicAdd(dacc + e[l], -rc[l]);
        }
      }
      __syncthreads();
      for (int d = tid; d < N; d += NT) {
        const bool interior = pd[d] > 0.0f;
        const double r = interior ? -(fp32_res ? (double)facc[d] : dacc[d]) : 0.0;
        // measured in the preconditioner's norm r^T P r: invariant to the h-scaling
        // of the blocks (mass ~ h^3, curl-curl ~ 1/h), which a plain 2-norm is not
        part[pass] += (double)pd[d] * r * r;
        // symmetric form S A (S = +1 on vertices, -1 on edges)
        if (pass == 1) vA[d] = (T)(d < g.NV ? r : -r);
      }
      __syncthreads();
    }
    {
      double tot[2];
      block_sum<double, 2, NW>(sh, part, tot);
      if (ir == 0) bnorm2 = tot[0];
      rnorm2 = tot[1];
    }
    ++nref;
    conv = !fp32_res && (rnorm2 <= prm.rtol * prm.rtol * bnorm2);
    if (conv || ir >= prm.max_refine) break;

    // ---------------- MINRES (two phases per iteration, as for Ned_RT) ----------------
    for (int d = tid; d < N; d += NT) {
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
      for (int d = tid; d < N; d += NT) {
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
    T gi_c = gam > T(0) ? T(1) / gam : T(0), gi_p = T(0);
    const double tol_abs = prm.rtol * sqrt(bnorm2);
    const double outer = 0.1 * tol_abs / fmax(sqrt(rnorm2), 1e-300);
    const T target = (T)((kMixed ? fmax(prm.inner_rtol, outer) : outer) * (double)eta0);
    bool active = gam > T(0) && isfinite(gam);
    bool pending = false;
    T p_step = T(0), p_a2 = T(0), p_a3 = T(0), p_ia1 = T(0);
    __syncthreads();
    for (int iter = 0; active && iter < prm.max_iter; ++iter) {
      T dpart = T(0);
      for (int c = tid; c < nc; c += NT) {
        int v[8], e[12];
        cell_dofs(g, c, v, e);
        const bool vb[8] = {}, eb[12] = {};
        if constexpr (kMixed) {
          const float4 c0 = reinterpret_cast<const float4 *>(cf)[2 * c];
          const float4 c1 = reinterpret_cast<const float4 *>(cf)[2 * c + 1];
          const float ai[6] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
          dpart += n >= 4 ? cell_apply<float, float, float, 0, true, true>(zt, az, Ff, ai, c1.z, v, e, vb, eb, c, g.L)
                          : cell_apply<float, float, float, 0, true>(zt, az, Ff, ai, c1.z, v, e, vb, eb);
        } else {
          const double *a = ag + 6 * (size_t)c;
          const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          dpart += n >= 4 ? cell_apply<double, double, double, 0, true, true>(zt, az, Fd, ai, bg[c], v, e, vb, eb, c,
                                                                               g.L)
                          : cell_apply<double, double, double, 0, true>(zt, az, Fd, ai, bg[c], v, e, vb, eb);
        }
      }
      if (pending) {
        for (int d = tid; d < N; d += NT) {
          const T z = (T)pd[d] * vp[d] * gi_p;
          const T wn = (z - p_a3 * wo[d] - p_a2 * wc[d]) * p_ia1;
          wo[d] = wn;
          xk[d] += p_step * wn;
        }
        T *t = wo;
        wo = wc;
        wc = t;
      }
      warp_publish<T>(sh, 0, dpart);
      __syncthreads();
      const T delta = slot_total<T, NW>(sh, 0) * gi_c * gi_c;
      T gpart = T(0);
      const T gg = gam * gi_p;
      for (int d = tid; d < N; d += NT) {
        const float pdd = pd[d];
        T vn = T(0);
        if (pdd > 0.0f) {
          const T a = d < g.NV ? az[d] : -az[d];
          vn = (a - delta * vc[d]) * gi_c - gg * vp[d];
        }
        vp[d] = vn;
        az[d] = T(0);
        const T z = (T)pdd * vn;
        zt[d] = z;
        gpart += z * vn;
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
        T *t = vc;
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
    for (int d = tid; d < N; d += NT)
      if (pd[d] > 0.0f) phi[d] += (double)xk[d];
    __syncthreads();
  }

  // ---------------- y_b = A P_b (FP64), P_b = primary block of basis b ----------------
  for (int d = tid; d < N; d += NT) dacc[d] = 0.0;
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int v[8], e[12];
    cell_dofs(g, c, v, e);
    const bool vb[8] = {}, eb[12] = {};
    const double *a = ag + 6 * (size_t)c;
    const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
    if (bb < 8)
      cell_apply<double, double, double, 2, false>(phi, dacc, Fd, ai, bg[c], v, e, vb, eb);
    else
      cell_apply<double, double, double, 3, false>(phi, dacc, Fd, ai, bg[c], v, e, vb, eb);
  }
  __syncthreads();
  for (int d = tid; d < N; d += NT) yout[d] = dacc[d];
  if (tid == 0) {
    NRStat st;
    st.iters = its;
    st.refinements = nref;
    st.converged = conv;
    st.flags = flags;
    st.rel_residual = bnorm2 > 0.0 ? sqrt(rnorm2 / bnorm2) : sqrt(rnorm2);
    prm.stats[(size_t)it.cell * kQNBases + bb] = st;
  }
  __syncthreads();
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT, 512 / NT) qned_solve_kernel(QNParams prm) {
  __shared__ QNShared sh;
  for (;;) {
    if (threadIdx.x == 0) sh.item = atomicAdd(prm.queue, 1);
    __syncthreads();
    const int item = sh.item;
    if (item >= prm.n_items) break;
    if constexpr (NT == 256) {
      solve_item<T, true, 256>(prm, sh, item);
    } else {
      if (prm.use_smem)
        solve_item<T, true, NT>(prm, sh, item);
      else
        solve_item<T, false, NT>(prm, sh, item);
    }
  }
}

constexpr int kGalThreads = 256;
constexpr int kGalWarps = kGalThreads / 32;

__device__ __forceinline__ void dmma(double &c0, double &c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// K_H[i][j] = P_i . y_j over all DoFs (P_i: primary block of basis i: vertex
// DoFs for i < 8, edge DoFs for i >= 8) on the FP64 tensor pipe (m8n8k4 tiles
// of the 24x24 padded product); F_H[8 + l] = u_{8+l} . (N_e, f) from the edge
// load vector (q_ned_basis.cc:927-935).
__global__ void __launch_bounds__(kGalThreads) qned_galerkin_kernel(const NRCell *__restrict__ cells,
                                                                    const double *__restrict__ phi,
                                                                    const double *__restrict__ y,
                                                                    const double *__restrict__ eload,
                                                                    double *__restrict__ KH, double *__restrict__ FH) {
  __shared__ double red[kGalWarps][24 * 24];
  __shared__ double redf[kGalWarps][12];
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  int NV, NEx, NE;
  qn_counts(C.n, NV, NEx, NE);
  const int N = NV + NE;
  const double *P = phi + (size_t)kQNBases * C.dof_off;
  const double *Y = y + (size_t)kQNBases * C.dof_off;
  const double *bl = eload + C.dof_off;
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
    const bool is_vertex = d < NV;
    double a[3], b[3];
#pragma unroll
    for (int I = 0; I < 3; ++I) {
      const int row = 8 * I + gr;
      const bool prim = row < kQNBases && ((row < 8) == is_vertex);
      a[I] = (ok && prim) ? __ldcs(P + (size_t)row * N + d) : 0.0;
      b[I] = (ok && row < kQNBases) ? __ldcs(Y + (size_t)row * N + d) : 0.0;
    }
#pragma unroll
    for (int I = 0; I < 3; ++I)
#pragma unroll
      for (int J = 0; J < 3; ++J) dmma(acc[I][J][0], acc[I][J][1], a[I], b[J]);
  }
  {
    double f12[12];
#pragma unroll
    for (int l = 0; l < 12; ++l) f12[l] = 0.0;
    for (int d = NV + threadIdx.x; d < N; d += kGalThreads) {
      const double bv = bl[d];
#pragma unroll
      for (int l = 0; l < 12; ++l) f12[l] += P[(size_t)(8 + l) * N + d] * bv;
    }
#pragma unroll
    for (int l = 0; l < 12; ++l) {
      double v = f12[l];
      for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) redf[warp][l] = v;
    }
  }
  // C fragment of m8n8k4: lane holds rows gr, cols 2*t4, 2*t4+1
#pragma unroll
  for (int I = 0; I < 3; ++I)
#pragma unroll
    for (int J = 0; J < 3; ++J) {
      red[warp][(8 * I + gr) * 24 + 8 * J + 2 * t4] = acc[I][J][0];
      red[warp][(8 * I + gr) * 24 + 8 * J + 2 * t4 + 1] = acc[I][J][1];
    }
  __syncthreads();
  for (int t = threadIdx.x; t < kQNBases * kQNBases; t += kGalThreads) {
    const int i = t / kQNBases, j = t % kQNBases;
    double s = 0.0;
    for (int w = 0; w < kGalWarps; ++w) s += red[w][i * 24 + j];
    KH[(size_t)c * kQNBases * kQNBases + t] = s;
  }
  if (threadIdx.x < kQNBases) {
    double s = 0.0;
    if (threadIdx.x >= 8)
      for (int w = 0; w < kGalWarps; ++w) s += redf[w][threadIdx.x - 8];
    FH[(size_t)c * kQNBases + threadIdx.x] = s;
  }
}

// Edge load vector (N_e, f) of every fine edge (2x2x2 Gauss, vector trig load).
__global__ void __launch_bounds__(kGalThreads) qned_edge_load_kernel(const NRCell *__restrict__ cells,
                                                                     msfec_load load, double *__restrict__ b) {
  const int c = blockIdx.x;
  const NRCell C = cells[c];
  QNGeom g;
  g.n = C.n;
  g.L = C.depth;
  qn_counts(g.n, g.NV, g.NEx, g.NE);
  g.N = g.NV + g.NE;
  if (load.kind != MSFEC_LOAD_VEC_TRIG) return;
  const int n = g.n, nc = n * n * n;
  const double w = load.params[1] * M_PI, p0 = load.params[0];
  const double gq = 0.5 / sqrt(3.0);
  const double qp[2] = {0.5 - gq, 0.5 + gq};
  const double jxw = 0.125 * C.h[0] * C.h[1] * C.h[2];
  for (int cell = threadIdx.x; cell < nc; cell += kGalThreads) {
    const int i = cell & (n - 1), j = (cell >> g.L) & (n - 1), k = cell >> (2 * g.L);
    double acc[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < 8; ++q) {
      const double xl[3] = {qp[q & 1], qp[(q >> 1) & 1], qp[q >> 2]};
      const double X = C.origin[0] + (i + xl[0]) * C.h[0], Y = C.origin[1] + (j + xl[1]) * C.h[1],
                   Z = C.origin[2] + (k + xl[2]) * C.h[2];
      const double sx = sin(w * X), sy = sin(w * Y), sz = sin(w * Z);
      const double fv[3] = {p0 * sy * sz, p0 * sz * sx, p0 * sx * sy};
      for (int p = 0; p < 3; ++p) {
        int o1, o2;
        other_axes(p, o1, o2);
        for (int l = 0; l < 4; ++l) {
          const double wt = psi(l & 1, xl[o1]) * psi(l >> 1, xl[o2]) / C.h[p];
          acc[4 * p + l] += jxw * wt * fv[p];
        }
      }
    }
    int v[8], e[12];
    cell_dofs(g, cell, v, e);
    for (int l = 0; l < 12; ++l) atomicAdd(b + C.dof_off + e[l], acc[l]);
  }
}

__global__ void qned_report_kernel(const NRStat *__restrict__ stats, int ncells, msfec_cell_report *rep) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  msfec_cell_report r;
  r.iterations = 0;
  r.refinements = 0;
  r.converged = 1;
  r.iterations_sum = 0;
  r.residual = 0.0;
  for (int b = 0; b < kQNBases; ++b) {
    const NRStat s = stats[(size_t)c * kQNBases + b];
    r.iterations = max(r.iterations, s.iters);
    r.iterations_sum += s.iters;
    r.refinements = max(r.refinements, s.refinements);
    r.converged = r.converged && s.converged && !(s.flags & 1);
    r.residual = fmax(r.residual, s.rel_residual);
    if (!isfinite(s.rel_residual)) r.residual = s.rel_residual;
  }
  rep[c] = r;
}

}  // namespace qnimpl

cudaError_t qned_solve_launch(bool fp64, bool two_per_sm, const QNParams &prm, size_t smem, int grid,
                              cudaStream_t st) {
  if (two_per_sm) {  // mixed precision, shared workspace that fits twice per SM
    auto k = qnimpl::qned_solve_kernel<float, 256>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    k<<<grid, 256, smem, st>>>(prm);
    return cudaGetLastError();
  }
  if (fp64) {
    auto k = qnimpl::qned_solve_kernel<double, kQNThreads>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kQNThreads, smem, st>>>(prm);
  } else {
    auto k = qnimpl::qned_solve_kernel<float, kQNThreads>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kQNThreads, smem, st>>>(prm);
  }
  return cudaGetLastError();
}

cudaError_t qned_galerkin_launch(const NRCell *cells, int ncells, const double *phi, const double *y,
                                 const msfec_load &load, double *eload, double *KH, double *FH,
                                 msfec_cell_report *rep, const NRStat *stats, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  qnimpl::qned_edge_load_kernel<<<ncells, qnimpl::kGalThreads, 0, st>>>(cells, load, eload);
  qnimpl::qned_galerkin_kernel<<<ncells, qnimpl::kGalThreads, 0, st>>>(cells, phi, y, eload, KH, FH);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !rep) return e;
  qnimpl::qned_report_kernel<<<(ncells + 127) / 128, 128, 0, st>>>(stats, ncells, rep);
  return cudaGetLastError();
}

}  // namespace msfec
