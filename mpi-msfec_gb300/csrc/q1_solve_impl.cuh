// Persistent batched Q1 local solver (sm_103a) - kernel body.
//
// Restates, batched over every coarse cell x coarse vertex, the reference's
//   QBasis::run loop            source/Q/q_basis.cc:545-565
//   QBasis::solve_iterative     source/Q/q_basis.cc:335-357 (CG + SSOR there)
//   AffineConstraints::condense / distribute (q_basis.cc:556, 348)
// as matrix-free PCG on the interior nodes with the Dirichlet data
// g_v = BasisQ1_v (include/functions/basis_q1.tpp:92-152) lifted to the right
// hand side, and writes y = K phi for the Galerkin product of
// QBasis::assemble_global_element_matrix (q_basis.cc:262-300).
//
// Source items (adjoint local problems) solve K_II x = f_I with zero Dirichlet
// data and a given right-hand side through the same loop.
//
// Execution model: one persistent launch; each cluster dequeues units from a
// device counter. A unit is either up to CL independent items (one CTA each)
// or one item split into z-slabs over the CL CTAs of a cluster (deep cells);
// slabs exchange one halo plane of the search direction through distributed
// shared memory and reduce dot products through DSMEM slots + cluster barriers.
// T is the Krylov arithmetic: float for the mixed path (FP64 iterative
// refinement around FP32 PCG) and double for the plain FP64 path. Residuals
// that decide convergence and the y = K phi output are FP64.
#pragma once

#include <cooperative_groups.h>

#include <type_traits>

#include "q1_common.cuh"

namespace cg = cooperative_groups;

namespace msfec {
namespace q1impl {

struct Q1Shared {
  // reduction slots: per warp, then per (parity, source CTA) of the cluster
  double warp[kQ1Warps][kRedVals][8];
  double part[2][kQ1MaxCluster][kRedVals][8];
  float fwarp[kQ1Warps][kRedVals][8];
  float fpart[2][kQ1MaxCluster][kRedVals][8];
  double cst[2][8];  // element pattern constants: stiffness, mass
  int unit;
};

template <typename VT>
__device__ __forceinline__ VT *red_warp(Q1Shared &sh) {
  if constexpr (sizeof(VT) == 4)
    return &sh.fwarp[0][0][0];
  else
    return &sh.warp[0][0][0];
}
template <typename VT>
__device__ __forceinline__ VT *red_part(Q1Shared &sh) {
  if constexpr (sizeof(VT) == 4)
    return &sh.fpart[0][0][0][0];
  else
    return &sh.part[0][0][0][0];
}
__device__ __forceinline__ int warp_slot(int w, int t, int q) { return (w * kRedVals + t) * 8 + q; }
__device__ __forceinline__ int part_slot(int par, int r, int t, int q) {
  return ((par * kQ1MaxCluster + r) * kRedVals + t) * 8 + q;
}

// Stiffness (unit coefficient) and mass entries of the Q1 element on a box,
// indexed by the pattern of differing coordinates pat = dx + 2 dy + 4 dz
// between the two local vertices (K_e[u][v] = c[u ^ v]); closed form of the
// 2x2x2 Gauss quadrature of QBasis::assemble_system (q_basis.cc:222-237).
__device__ __forceinline__ void pattern_constants(const double h[3], double c[8], double mm[8]) {
#pragma unroll
  for (int pat = 0; pat < 8; ++pat) {
    const int dx = pat & 1, dy = (pat >> 1) & 1, dz = pat >> 2;
    const double kx = (dx ? -1.0 : 1.0) / h[0], ky = (dy ? -1.0 : 1.0) / h[1], kz = (dz ? -1.0 : 1.0) / h[2];
    const double mx = h[0] * (dx ? 1.0 / 6.0 : 1.0 / 3.0), my = h[1] * (dy ? 1.0 / 6.0 : 1.0 / 3.0),
                 mz = h[2] * (dz ? 1.0 / 6.0 : 1.0 / 3.0);
    c[pat] = kx * my * mz + mx * ky * mz + mx * my * kz;
    mm[pat] = mx * my * mz;
  }
}

__device__ __forceinline__ double trilinear(int v, int i, int j, int k, int n) {
  const double inv = 1.0 / n;
  const double tx = i * inv, ty = j * inv, tz = k * inv;
  return ((v & 1) ? tx : 1.0 - tx) * ((v & 2) ? ty : 1.0 - ty) * ((v & 4) ? tz : 1.0 - tz);
}

// Sums of the four fine-cell coefficients of one cell layer around column
// (i, j), indexed [dy+1][dx+1]: weight of the edge node -> node+(dx,dy,.)
// restricted to that layer. p00 points at cell (i-1, j-1) of the layer.
template <typename TA, typename LoadFn>
__device__ __forceinline__ void layer_sums(LoadFn ld, int n, TA (&Y)[3][3]) {
  const TA a00 = (TA)ld(0), a10 = (TA)ld(1), a01 = (TA)ld(n), a11 = (TA)ld(n + 1);
  Y[0][0] = a00;
  Y[0][2] = a10;
  Y[0][1] = a00 + a10;
  Y[2][0] = a01;
  Y[2][2] = a11;
  Y[2][1] = a01 + a11;
  Y[1][0] = a00 + a01;
  Y[1][2] = a10 + a11;
  Y[1][1] = Y[0][1] + Y[2][1];
}

// FP32 Krylov apply: q[pk] = (K p)(i, j, k0 + pk), pk < P, one right-hand
// side, sweeping the column with a 3-plane register window (9 shared loads
// per node). ps is node-major [(kk*N1 + j)*N1 + i][R] with plane kk <-> k0-1+kk,
// caf the float coefficient slab [l][cj][ci] with layer l <-> k0-1+l.
template <int R, int PMAX, bool HAS_R>
__device__ __forceinline__ void column_apply_f32(const float *__restrict__ ps, const float *__restrict__ caf,
                                                 const float *__restrict__ raf, int n, int rho, int i, int j,
                                                 int P, const float (&c)[8], const float (&mm)[8],
                                                 float (&q)[PMAX], float (&ctr)[PMAX]) {
  const int N1 = n + 1;
  const size_t plane = (size_t)N1 * N1 * R;
  const float *vb = ps + ((size_t)(j - 1) * N1 + (i - 1)) * R + rho;
  const float *cb = caf + (size_t)(j - 1) * n + (i - 1);
  const float *rb = HAS_R ? raf + (size_t)(j - 1) * n + (i - 1) : nullptr;
  const size_t clayer = (size_t)n * n;
  float w[3][3][3];
  auto load_plane = [&](int kk, float(&ww)[3][3]) {
    const float *b = vb + (size_t)kk * plane;
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) ww[dy][dx] = b[((size_t)dy * N1 + dx) * R];
  };
  float lo[3][3], hi[3][3], rlo[3][3], rhi[3][3];
  load_plane(0, w[0]);
  load_plane(1, w[1]);
  layer_sums<float>([&](int o) { return cb[o]; }, n, lo);
  if constexpr (HAS_R) layer_sums<float>([&](int o) { return rb[o]; }, n, rlo);
#pragma unroll
  for (int pk = 0; pk < PMAX; ++pk) {
    if (pk < P) {
      load_plane(pk + 2, w[(pk + 2) % 3]);
      const float *cl = cb + (size_t)(pk + 1) * clayer;
      layer_sums<float>([&](int o) { return cl[o]; }, n, hi);
      if constexpr (HAS_R) {
        const float *rl = rb + (size_t)(pk + 1) * clayer;
        layer_sums<float>([&](int o) { return rl[o]; }, n, rhi);
      }
      float acc[8], racc[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = racc[t] = 0.0f;
#pragma unroll
      for (int dz = 0; dz < 3; ++dz)
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) {
            const int pat = (dx != 1) + 2 * (dy != 1) + 4 * (dz != 1);
            const float val = w[(pk + dz) % 3][dy][dx];
            const float A = dz == 0 ? lo[dy][dx] : (dz == 2 ? hi[dy][dx] : lo[dy][dx] + hi[dy][dx]);
            acc[pat] = fmaf(A, val, acc[pat]);
            if constexpr (HAS_R) {
              const float Rr = dz == 0 ? rlo[dy][dx] : (dz == 2 ? rhi[dy][dx] : rlo[dy][dx] + rhi[dy][dx]);
              racc[pat] = fmaf(Rr, val, racc[pat]);
            }
          }
      float s = 0.0f;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        s = fmaf(c[t], acc[t], s);
        if constexpr (HAS_R) s = fmaf(mm[t], racc[t], s);
      }
      q[pk] = s;
      ctr[pk] = w[(pk + 1) % 3][1][1];
#pragma unroll
      for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
          lo[dy][dx] = hi[dy][dx];
          if constexpr (HAS_R) rlo[dy][dx] = rhi[dy][dx];
        }
    }
  }
}

// FP64 Krylov apply (plain FP64 path): per node 27 shared loads, coefficient
// layer sums slide along the column. FP64 issue, not shared bandwidth, bounds
// this loop, so no value window is kept.
template <int R, int PMAX, bool HAS_R>
__device__ __forceinline__ void column_apply_f64(const double *__restrict__ ps, const double *__restrict__ cad,
                                                 const double *__restrict__ rad, int n, int rho, int i, int j,
                                                 int P, const double (&c)[8], const double (&mm)[8],
                                                 double (&q)[PMAX], double (&ctr)[PMAX]) {
  const int N1 = n + 1;
  const size_t plane = (size_t)N1 * N1 * R;
  const double *vb = ps + ((size_t)(j - 1) * N1 + (i - 1)) * R + rho;
  const size_t cofs = (size_t)(j - 1) * n + (i - 1);
  const size_t clayer = (size_t)n * n;
  double lo[3][3], hi[3][3], rlo[3][3], rhi[3][3];
  layer_sums<double>([&](int o) { return __ldg(cad + cofs + o); }, n, lo);
  if constexpr (HAS_R) layer_sums<double>([&](int o) { return __ldg(rad + cofs + o); }, n, rlo);
#pragma unroll
  for (int pk = 0; pk < PMAX; ++pk) {
    if (pk < P) {
      const size_t lofs = cofs + (size_t)(pk + 1) * clayer;
      layer_sums<double>([&](int o) { return __ldg(cad + lofs + o); }, n, hi);
      if constexpr (HAS_R) layer_sums<double>([&](int o) { return __ldg(rad + lofs + o); }, n, rhi);
      double acc[8], racc[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = racc[t] = 0.0;
#pragma unroll
      for (int dz = 0; dz < 3; ++dz)
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) {
            const int pat = (dx != 1) + 2 * (dy != 1) + 4 * (dz != 1);
            const double val = vb[(size_t)(pk + dz) * plane + ((size_t)dy * N1 + dx) * R];
            const double A = dz == 0 ? lo[dy][dx] : (dz == 2 ? hi[dy][dx] : lo[dy][dx] + hi[dy][dx]);
            acc[pat] = fma(A, val, acc[pat]);
            if constexpr (HAS_R) {
              const double Rr = dz == 0 ? rlo[dy][dx] : (dz == 2 ? rhi[dy][dx] : rlo[dy][dx] + rhi[dy][dx]);
              racc[pat] = fma(Rr, val, racc[pat]);
            }
          }
      double s = 0.0;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        s = fma(c[t], acc[t], s);
        if constexpr (HAS_R) s = fma(mm[t], racc[t], s);
      }
      q[pk] = s;
      ctr[pk] = vb[(size_t)(pk + 1) * plane + ((size_t)1 * N1 + 1) * R];
#pragma unroll
      for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
          lo[dy][dx] = hi[dy][dx];
          if constexpr (HAS_R) rlo[dy][dx] = rhi[dy][dx];
        }
    }
  }
}

// The FP64 refinement residual as a call: it runs once per refinement step,
// and out of line it gets its own register allocation instead of raising
// the pressure (and the spills) of the FP32 Krylov loop in the same kernel.
template <int R, int PMAX, bool HAS_R>
__device__ __noinline__ void column_residual_f64(const double *__restrict__ vs, const double *__restrict__ ag,
                                                 const double *__restrict__ rg, int n, int rho, int i, int j, int P,
                                                 const double (&c)[8], const double (&mm)[8], double (&q)[PMAX],
                                                 double (&ctr)[PMAX]) {
  column_apply_f64<R, PMAX, HAS_R>(vs, ag, rg, n, rho, i, j, P, c, mm, q, ctr);
}

// Residual-pass apply at one node for all R right-hand sides: y = K v, and
// (BND) yb = the part of K v coming from lattice-boundary neighbours (K_IB g
// when v carries the Dirichlet data). GUARD: lattice-boundary node, the
// loaders return 0 for absent cells and absent neighbours are skipped.
template <typename TA, int R, bool HAS_R, bool BND, bool GUARD = false, typename TV, typename LoadA,
          typename LoadR>
__device__ __forceinline__ void node_apply(const TV *__restrict__ vs, int n, int kk, int i, int j, int k,
                                           LoadA lda, LoadR ldr, const double (&c)[8], const double (&mm)[8],
                                           TA (&y)[R], TA (&yb)[R]) {
  const int N1 = n + 1;
  TA lo[3][3], hi[3][3], rlo[3][3], rhi[3][3];
  layer_sums<TA>([&](int o) { return lda(kk - 1, o); }, n, lo);
  layer_sums<TA>([&](int o) { return lda(kk, o); }, n, hi);
  if constexpr (HAS_R) {
    layer_sums<TA>([&](int o) { return ldr(kk - 1, o); }, n, rlo);
    layer_sums<TA>([&](int o) { return ldr(kk, o); }, n, rhi);
  }
#pragma unroll
  for (int t = 0; t < R; ++t) y[t] = yb[t] = TA(0);
#pragma unroll
  for (int dz = 0; dz < 3; ++dz)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int pat = (dx != 1) + 2 * (dy != 1) + 4 * (dz != 1);
        const TA A = dz == 0 ? lo[dy][dx] : (dz == 2 ? hi[dy][dx] : lo[dy][dx] + hi[dy][dx]);
        TA wgt = (TA)c[pat] * A;
        if constexpr (HAS_R) {
          const TA Rr = dz == 0 ? rlo[dy][dx] : (dz == 2 ? rhi[dy][dx] : rlo[dy][dx] + rhi[dy][dx]);
          wgt += (TA)mm[pat] * Rr;
        }
        const int ni = i + dx - 1, nj = j + dy - 1, nk = k + dz - 1;
        if constexpr (GUARD) {
          if (ni < 0 || nj < 0 || nk < 0 || ni > n || nj > n || nk > n) continue;
        }
        const bool nb_bnd = BND && (ni == 0 || nj == 0 || nk == 0 || ni == n || nj == n || nk == n);
        const TV *src = vs + (((size_t)(kk + dz - 1) * N1 + nj) * N1 + ni) * R;
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const TA val = (TA)src[t];
          y[t] += wgt * val;
          if constexpr (BND) {
            if (nb_bnd) yb[t] += wgt * val;
          }
        }
      }
}

template <bool SLAB>
__device__ __forceinline__ void xsync() {
  if constexpr (SLAB)
    cg::this_cluster().sync();
  else
    __syncthreads();
}

// Publish per-CTA totals (threads < R hold rhs = threadIdx.x) into every
// peer's slot row, synchronise, and return this thread's rhs total (rank
// order summation: bitwise identical in every CTA of the cluster). VT is the
// accumulation type: float inside the FP32 Krylov loop (no FP64 pipe use),
// double for FP64 residuals and the plain FP64 path.
template <typename VT, bool SLAB, int NV, int R>
__device__ __forceinline__ void publish_and_sum(Q1Shared &sh, int &parity, const VT (&s)[NV], int rank,
                                                int nslab, VT (&out)[NV]) {
  VT *part = red_part<VT>(sh);
  if ((int)threadIdx.x < R) {
    if constexpr (SLAB) {
      cg::cluster_group cluster = cg::this_cluster();
      for (int r = 0; r < nslab; ++r) {
        VT *rp = cluster.map_shared_rank(part, r);
#pragma unroll
        for (int t = 0; t < NV; ++t) rp[part_slot(parity, rank, t, threadIdx.x)] = s[t];
      }
    } else {
#pragma unroll
      for (int t = 0; t < NV; ++t) part[part_slot(parity, 0, t, threadIdx.x)] = s[t];
    }
  }
  xsync<SLAB>();
  const int rho = threadIdx.x % R;
  const int nrows = SLAB ? nslab : 1;
#pragma unroll
  for (int t = 0; t < NV; ++t) {
    VT acc = VT(0);
    for (int r = 0; r < nrows; ++r) acc += part[part_slot(parity, r, t, rho)];
    out[t] = acc;
  }
  parity ^= 1;
}

// Reduction when every thread holds partials of ITS rhs (rho = tid % R).
template <typename VT, bool SLAB, int NV, int R>
__device__ __forceinline__ void reduce_own(Q1Shared &sh, int &parity, VT (&v)[NV], int rank, int nslab,
                                           VT (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  VT *ws = red_warp<VT>(sh);
#pragma unroll
  for (int off = 16; off >= R; off >>= 1)
#pragma unroll
    for (int t = 0; t < NV; ++t) v[t] += __shfl_xor_sync(0xffffffffu, v[t], off);
  if (lane < R)
#pragma unroll
    for (int t = 0; t < NV; ++t) ws[warp_slot(warp, t, lane)] = v[t];
  __syncthreads();
  VT s[NV];
#pragma unroll
  for (int t = 0; t < NV; ++t) s[t] = VT(0);
  if ((int)threadIdx.x < R)
#pragma unroll
    for (int w = 0; w < kQ1Warps; ++w)
#pragma unroll
      for (int t = 0; t < NV; ++t) s[t] += ws[warp_slot(w, t, threadIdx.x)];
  publish_and_sum<VT, SLAB, NV, R>(sh, parity, s, rank, nslab, out);
}

// Reduction when every thread holds partials of ALL R rhs (FP64 residuals).
template <bool SLAB, int NV, int R>
__device__ __forceinline__ void reduce_all(Q1Shared &sh, int &parity, double (&v)[NV][R], int rank, int nslab,
                                           double (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *ws = red_warp<double>(sh);
#pragma unroll
  for (int t = 0; t < NV; ++t)
#pragma unroll
    for (int q = 0; q < R; ++q) {
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) v[t][q] += __shfl_xor_sync(0xffffffffu, v[t][q], off);
      if (lane == 0) ws[warp_slot(warp, t, q)] = v[t][q];
    }
  __syncthreads();
  double s[NV];
#pragma unroll
  for (int t = 0; t < NV; ++t) s[t] = 0.0;
  if ((int)threadIdx.x < R)
#pragma unroll
    for (int w = 0; w < kQ1Warps; ++w)
#pragma unroll
      for (int t = 0; t < NV; ++t) s[t] += ws[warp_slot(w, t, threadIdx.x)];
  publish_and_sum<double, SLAB, NV, R>(sh, parity, s, rank, nslab, out);
}

template <typename T, int R, int UMAX, int PMAX, bool HAS_R, bool SLAB>
__device__ void solve_item(const Q1Params &prm, Q1Shared &sh, unsigned char *smem, int item_id, int rank,
                           int nslab) {
  const Q1Item it = prm.items[item_id];
  const Q1Cell C = prm.cells[it.cell];
  const int n = C.n, m = n - 1, N1 = n + 1;
  const size_t N1sq = (size_t)N1 * N1;
  const size_t nn = N1sq * N1;
  const int PS = q1_planes_per_cta(n, nslab);
  const int k0 = 1 + rank * PS;
  const int P = max(0, min(PS, n - k0));
  const int ncol = m * m;
  const Q1Smem L = q1_smem_layout(n, R, nslab, HAS_R, (int)sizeof(T));
  double *slab_d = reinterpret_cast<double *>(smem + L.slab_off);
  float *slab_f = reinterpret_cast<float *>(smem + L.slab_off);
  T *slab_t = reinterpret_cast<T *>(smem + L.slab_off);
  float *caf = reinterpret_cast<float *>(smem + L.caf_off);
  float *raf = reinterpret_cast<float *>(smem + L.raf_off);
  T *xs = reinterpret_cast<T *>(smem + L.x_off);
  T *ps = reinterpret_cast<T *>(smem + L.p_off);
  T *ss = reinterpret_cast<T *>(smem + L.s_off);
  float *dvs = reinterpret_cast<float *>(smem + L.dv_off);
  const int tid = threadIdx.x;
  const int rho = tid % R;
  const bool src = it.mode == 1;
  double *phi_c = (src ? prm.src_out : prm.phi) + 8 * C.node_off;
  double *y_c = prm.y + 8 * C.node_off;
  const double *f_c = src ? prm.src_rhs + 8 * C.node_off : nullptr;
  const double *ag = prm.a + C.coef_off + (size_t)(k0 - 1) * n * n;  // layer 0 of the slab
  const double *rg = HAS_R ? prm.react + C.coef_off + (size_t)(k0 - 1) * n * n : nullptr;
  const int nplanes = P > 0 ? P + 2 : 0;
  const size_t slab_nodes = (size_t)nplanes * N1sq;
  const size_t own_nodes = (size_t)P * ncol;
  const bool first = (k0 == 1);
  const bool last = (P > 0) && (k0 + P == n);
  constexpr bool kMixed = sizeof(T) == 4;
  int parity = 0;

  if (tid < 8) {
    double cc[8], mmm[8];
    pattern_constants(C.h, cc, mmm);
    sh.cst[0][tid] = cc[tid];
    sh.cst[1][tid] = mmm[tid];
  }
  // Stage the float coefficients of layers k0-1 .. k0+P-1 (Krylov operator).
  {
    const size_t ncl = P > 0 ? (size_t)(P + 1) * n * n : 0;
    for (size_t e = tid; e < ncl; e += kQ1Threads) caf[e] = (float)__ldg(ag + e);
    if constexpr (HAS_R)
      for (size_t e = tid; e < ncl; e += kQ1Threads) raf[e] = (float)__ldg(rg + e);
  }
  __syncthreads();
  double cd[8], mmd[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    cd[t] = sh.cst[0][t];
    mmd[t] = sh.cst[1][t];
  }
  // Jacobi scaling 1 / K_ii of every owned interior node.
  for (size_t e = tid; e < own_nodes; e += kQ1Threads) {
    const int pk = (int)(e / ncol), col = (int)(e % ncol);
    const int i = col % m + 1, j = col / m + 1;
    double sa = 0.0, sr = 0.0;
#pragma unroll
    for (int oz = 0; oz < 2; ++oz)
#pragma unroll
      for (int oy = 0; oy < 2; ++oy)
#pragma unroll
        for (int ox = 0; ox < 2; ++ox) {
          const size_t ce = ((size_t)(pk + oz) * n + (j - 1 + oy)) * n + (i - 1 + ox);
          sa += __ldg(ag + ce);
          if constexpr (HAS_R) sr += __ldg(rg + ce);
        }
    dvs[e] = (float)(1.0 / (cd[0] * sa + mmd[0] * sr));
  }

  // Thread -> (column, rhs) Krylov units.
  int ci[UMAX], cj[UMAX];
  bool cval[UMAX];
#pragma unroll
  for (int s = 0; s < UMAX; ++s) {
    const int col = tid / R + s * (kQ1Threads / R);
    cval[s] = (col < ncol) && (P > 0);
    ci[s] = cval[s] ? col % m + 1 : 1;
    cj[s] = cval[s] ? col / m + 1 : 1;
  }
  auto own_idx = [&](int s, int pk) -> size_t { return ((size_t)pk * m + (cj[s] - 1)) * m + (ci[s] - 1); };
  auto slab_idx = [&](int s, int pk) -> size_t {
    return (((size_t)(pk + 1) * N1 + cj[s]) * N1 + ci[s]) * R + rho;
  };

  // Stage a field into the slab: mode 1 = trilinear phi0 (also written to
  // phi in HBM for owned planes, boundary planes by the first/last slab),
  // mode 2 = phi from HBM (L2, written by peer CTAs).
  auto stage = [&](auto *dst, int mode) {
    using TV = typename std::remove_pointer<decltype(dst)>::type;
    const size_t tot = slab_nodes * R;
    for (size_t e = tid; e < tot; e += kQ1Threads) {
      const int r_e = (int)(e / slab_nodes);
      const size_t nl = e % slab_nodes;
      const int i = (int)(nl % N1), j = (int)((nl / N1) % N1), kk = (int)(nl / N1sq);
      const int k = k0 - 1 + kk;
      const int v = it.rhs0 + r_e;
      const size_t g = (size_t)v * nn + ((size_t)k * N1 + j) * N1 + i;
      double val;
      if (mode == 2) {
        val = __ldcg(phi_c + g);
      } else {
        val = src ? 0.0 : trilinear(v, i, j, k, n);
        if ((kk >= 1 && kk <= P) || (kk == 0 && k == 0) || (kk == P + 1 && k == n)) phi_c[g] = val;
      }
      dst[nl * R + r_e] = (TV)val;
    }
  };

  // State of this thread's rhs.
  double bnorm2 = 0.0, rnorm2 = 0.0;
  int conv = 0, its = 0, flags = 0, nref = 0;

  for (int ir = 0;; ++ir) {
    // ---------------- residual phase: r = -(K phi)_I ----------------
    const bool fp32_res = kMixed && ir == 0;  // first residual of the mixed path in FP32
    if (fp32_res)
      stage(slab_f, ir == 0 ? 1 : 2);
    else
      stage(slab_d, ir == 0 ? 1 : 2);
    __syncthreads();
    {
      double part[2][R];
#pragma unroll
      for (int t = 0; t < R; ++t) part[0][t] = part[1][t] = 0.0;
      if (!fp32_res && ir > 0) {
        // Refinement residual in FP64: the Krylov thread -> (column, rhs) map
        // and a z-column sweep whose coefficient layer sums slide from one
        // plane to the next (half the FP64 layer-sum work of a per-node
        // apply, entries grouped by the 8 stiffness patterns). Writes y = K phi.
        double acc = 0.0;
#pragma unroll
        for (int s = 0; s < UMAX; ++s) {
          if (!cval[s]) continue;
          double q[PMAX], ctr[PMAX];
          column_residual_f64<R, PMAX, HAS_R>(slab_d, ag, rg, n, rho, ci[s], cj[s], P, cd, mmd, q, ctr);
#pragma unroll
          for (int pk = 0; pk < PMAX; ++pk)
            if (pk < P) {
              const size_t gnode = ((size_t)(k0 + pk) * N1 + cj[s]) * N1 + ci[s];
              const double f = src ? __ldg(f_c + (size_t)(it.rhs0 + rho) * nn + gnode) : 0.0;
              const double rr = f - q[pk];
              xs[own_idx(s, pk) * R + rho] = (T)rr;
              acc += rr * rr;
              if (!src) y_c[(size_t)(it.rhs0 + rho) * nn + gnode] = q[pk];
            }
        }
#pragma unroll
        for (int t = 0; t < R; ++t) part[1][t] = t == rho ? acc : 0.0;
      } else
      for (size_t e = tid; e < own_nodes; e += kQ1Threads) {
        const int pk = (int)(e / ncol), col = (int)(e % ncol);
        const int i = col % m + 1, j = col / m + 1, k = k0 + pk;
        const size_t gnode = ((size_t)k * N1 + j) * N1 + i;
        // r = f - K phi (f = 0 for basis items); at ir == 0 also the scale of the
        // stopping test: ||K_IB g|| (basis items) or ||f_I|| (source items)
        auto finish = [&](int t, double yv, double yb, bool write_y) {
          const double f = src ? __ldg(f_c + (size_t)(it.rhs0 + t) * nn + gnode) : 0.0;
          const double rr = f - yv;
          xs[e * R + t] = (T)rr;
          if (ir == 0) part[0][t] += src ? f * f : yb * yb;
          part[1][t] += rr * rr;
          if (write_y && !src) y_c[(size_t)(it.rhs0 + t) * nn + gnode] = yv;
        };
        if (fp32_res) {
          float yv[R], yb[R];
          node_apply<float, R, HAS_R, true>(
              slab_f, n, pk + 1, i, j, k, [&](int l, int o) { return caf[((size_t)l * n + (j - 1)) * n + (i - 1) + o]; },
              [&](int l, int o) { return HAS_R ? raf[((size_t)l * n + (j - 1)) * n + (i - 1) + o] : 0.0f; }, cd, mmd,
              yv, yb);
#pragma unroll
          for (int t = 0; t < R; ++t) finish(t, (double)yv[t], (double)yb[t], false);
        } else if (ir == 0) {
          double yv[R], yb[R];
          node_apply<double, R, HAS_R, true>(
              slab_d, n, pk + 1, i, j, k,
              [&](int l, int o) { return __ldg(ag + ((size_t)l * n + (j - 1)) * n + (i - 1) + o); },
              [&](int l, int o) { return HAS_R ? __ldg(rg + ((size_t)l * n + (j - 1)) * n + (i - 1) + o) : 0.0; }, cd,
              mmd, yv, yb);
#pragma unroll
          for (int t = 0; t < R; ++t) finish(t, yv[t], yb[t], true);
        } else {
          double yv[R], yb[R];
          node_apply<double, R, HAS_R, false>(
              slab_d, n, pk + 1, i, j, k,
              [&](int l, int o) { return __ldg(ag + ((size_t)l * n + (j - 1)) * n + (i - 1) + o); },
              [&](int l, int o) { return HAS_R ? __ldg(rg + ((size_t)l * n + (j - 1)) * n + (i - 1) + o) : 0.0; }, cd,
              mmd, yv, yb);
#pragma unroll
          for (int t = 0; t < R; ++t) finish(t, yv[t], 0.0, true);
        }
      }
      double tot[2];
      reduce_all<SLAB, 2, R>(sh, parity, part, rank, nslab, tot);
      if (ir == 0) bnorm2 = tot[0];
      rnorm2 = tot[1];
    }
    ++nref;
    // the FP32 residual of the mixed path never certifies convergence
    conv = !fp32_res && (rnorm2 <= prm.rtol * prm.rtol * bnorm2);
    const bool all_conv = __syncthreads_and(conv) != 0;
    if (all_conv || ir >= prm.max_refine) break;

    // ---------------- Krylov phase (precision T) ----------------
    // Chronopoulos-Gear PCG: one apply w = K u (u = D^-1 r) and ONE fused
    // reduction (gamma = r.u, delta = w.u, r.r) per iteration; p and s = K p
    // follow by recurrence, so an iteration crosses two barriers (reduction,
    // halo of u). Accumulation is in T: no FP64 instruction in the FP32 loop.
    const double tol_abs2 = prm.rtol * prm.rtol * bnorm2;
    const double target2 = kMixed ? fmax(prm.inner_rtol * prm.inner_rtol * rnorm2, 0.01 * tol_abs2) : 0.25 * tol_abs2;
    bool active = !conv && (rnorm2 > target2);
    const T target2t = (T)target2;
    // r into registers (K u of the iteration in q); x = p = s = 0; u-slab = 0
    // (boundary and halo planes stay zero). Scoped to this phase, so that
    // nothing stays live across the FP64 residual phase (fewer spills).
    T r[UMAX][PMAX], q[UMAX][PMAX];
#pragma unroll
    for (int s = 0; s < UMAX; ++s)
#pragma unroll
      for (int pk = 0; pk < PMAX; ++pk) {
        r[s][pk] = (cval[s] && pk < P) ? xs[own_idx(s, pk) * R + rho] : T(0);
        q[s][pk] = T(0);
      }
    __syncthreads();
    for (size_t e = tid; e < own_nodes * R; e += kQ1Threads) xs[e] = ps[e] = ss[e] = T(0);
    for (size_t e = tid; e < slab_nodes * R; e += kQ1Threads) slab_t[e] = T(0);
    // Peers push halo planes into this slab next: every slab must be zeroed
    // (and done serving the residual phase) first.
    const bool any_active0 = __syncthreads_or(active) != 0;
    if constexpr (SLAB) cg::this_cluster().sync();
    if (any_active0) {
      T ct[8], mmt[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        ct[t] = (T)cd[t];
        mmt[t] = (T)mmd[t];
      }
      auto write_u = [&](int s, int pk, T uv) {
        slab_t[slab_idx(s, pk)] = uv;
        if constexpr (SLAB) {
          if (pk == 0 && rank > 0) {
            T *rem = cg::this_cluster().map_shared_rank(slab_t, rank - 1);
            rem[(((size_t)(PS + 1) * N1 + cj[s]) * N1 + ci[s]) * R + rho] = uv;
          }
          if (pk == P - 1 && rank < nslab - 1) {
            T *rem = cg::this_cluster().map_shared_rank(slab_t, rank + 1);
            rem[((size_t)cj[s] * N1 + ci[s]) * R + rho] = uv;
          }
        }
      };
#pragma unroll
      for (int s = 0; s < UMAX; ++s) {
        if (!cval[s]) continue;
#pragma unroll
        for (int pk = 0; pk < PMAX; ++pk)
          if (pk < P) write_u(s, pk, active ? (T)dvs[own_idx(s, pk)] * r[s][pk] : T(0));
      }
      xsync<SLAB>();
      T gamma_old = T(1), alpha_old = T(1);
      for (int iter = 0; iter < prm.max_iter; ++iter) {
        // w = K u (kept in q), partial gamma, delta, r.r
        T part[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int s = 0; s < UMAX; ++s) {
          if (!cval[s]) continue;
          T uc[PMAX];
          if constexpr (kMixed)
            column_apply_f32<R, PMAX, HAS_R>(slab_t, caf, raf, n, rho, ci[s], cj[s], P, ct, mmt, q[s], uc);
          else
            column_apply_f64<R, PMAX, HAS_R>(slab_t, ag, rg, n, rho, ci[s], cj[s], P, ct, mmt, q[s], uc);
#pragma unroll
          for (int pk = 0; pk < PMAX; ++pk)
            if (pk < P) {
              part[0] += r[s][pk] * uc[pk];
              part[1] += q[s][pk] * uc[pk];
              part[2] += r[s][pk] * r[s][pk];
            }
        }
        T tot[3];
        reduce_own<T, SLAB, 3, R>(sh, parity, part, rank, nslab, tot);
        T alpha = T(0), beta = T(0);
        if (active) {
          const T gamma = tot[0], delta = tot[1], rr = tot[2];
          if (rr <= target2t) {
            active = false;
          } else {
            beta = iter == 0 ? T(0) : gamma / gamma_old;
            const T denom = iter == 0 ? delta : delta - beta * gamma / alpha_old;
            if (!(denom > T(0)) || !(gamma > T(0)) || !isfinite(denom) || !isfinite(gamma)) {
              active = false;
              flags |= 1;
            } else {
              alpha = gamma / denom;
              gamma_old = gamma;
              alpha_old = alpha;
              ++its;
            }
          }
        }
        if (__syncthreads_or(active) == 0) break;
        // p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s, u = D^-1 r
        if (active) {
#pragma unroll
          for (int s = 0; s < UMAX; ++s) {
            if (!cval[s]) continue;
#pragma unroll
            for (int pk = 0; pk < PMAX; ++pk)
              if (pk < P) {
                const size_t oi = own_idx(s, pk);
                const size_t vi = oi * R + rho;
                const T pv = slab_t[slab_idx(s, pk)] + beta * ps[vi];
                const T sv = q[s][pk] + beta * ss[vi];
                ps[vi] = pv;
                ss[vi] = sv;
                xs[vi] += alpha * pv;
                r[s][pk] -= alpha * sv;
                write_u(s, pk, (T)dvs[oi] * r[s][pk]);
              }
          }
        }
        xsync<SLAB>();
      }
    }
    // ---------------- update phi_I += x (FP64, HBM) ----------------
    for (size_t e = tid; e < own_nodes * R; e += kQ1Threads) {
      const int r_e = (int)(e / own_nodes);
      const size_t o = e % own_nodes;
      const int pk = (int)(o / ncol), col = (int)(o % ncol);
      const int i = col % m + 1, j = col / m + 1;
      const size_t g = (size_t)(it.rhs0 + r_e) * nn + ((size_t)(k0 + pk) * N1 + j) * N1 + i;
      __stcg(phi_c + g, __ldcg(phi_c + g) + (double)xs[o * R + r_e]);
    }
    xsync<SLAB>();
  }

  // ---------------- boundary rows of y = K phi ----------------
  // FP64 27-point apply at lattice-boundary nodes with absent cells and
  // neighbours padded out; phi is staged in slab_d by the last residual phase.
  {
    const int nside = P * 4 * n;  // perimeter nodes of the owned planes
    const int nfirst = (P > 0 && first) ? (int)N1sq : 0;
    const int nlast = last ? (int)N1sq : 0;
    const int nb = (P > 0 && !src) ? nside + nfirst + nlast : 0;
    for (int e = tid; e < nb; e += kQ1Threads) {
      int b = e;
      int i, j, kk;
      if (b < nside) {
        kk = b / (4 * n) + 1;
        const int s = b % (4 * n);
        if (s < n) {
          i = s;
          j = 0;
        } else if (s < 2 * n) {
          i = n;
          j = s - n;
        } else if (s < 3 * n) {
          i = n - (s - 2 * n);
          j = n;
        } else {
          i = 0;
          j = n - (s - 3 * n);
        }
      } else if (b < nside + nfirst) {
        b -= nside;
        kk = 0;
        i = b % N1;
        j = b / N1;
      } else {
        b -= nside + nfirst;
        kk = P + 1;
        i = b % N1;
        j = b / N1;
      }
      const int k = k0 - 1 + kk;
      auto pad = [&](const double *base, int l, int o) -> double {
        const int ex = i - 1 + ((o == 1 || o == n + 1) ? 1 : 0);
        const int ey = j - 1 + (o >= n ? 1 : 0);
        const int ez = k0 - 1 + l;
        if (ex < 0 || ey < 0 || ez < 0 || ex >= n || ey >= n || ez >= n) return 0.0;
        return __ldg(base + ((ptrdiff_t)l * n + ey) * n + ex);
      };
      double yv[R], yb[R];
      node_apply<double, R, HAS_R, false, true>(
          slab_d, n, kk, i, j, k, [&](int l, int o) { return pad(ag, l, o); },
          [&](int l, int o) { return HAS_R ? pad(rg, l, o) : 0.0; }, cd, mmd, yv, yb);
      const size_t gnode = ((size_t)k * N1 + j) * N1 + i;
#pragma unroll
      for (int t = 0; t < R; ++t) y_c[(size_t)(it.rhs0 + t) * nn + gnode] = yv[t];
    }
  }
  if (rank == 0 && tid < R) {
    Q1Stat st;
    st.iters = its;
    st.refinements = nref;
    st.converged = conv;
    st.flags = flags;
    st.rel_residual = bnorm2 > 0.0 ? sqrt(rnorm2 / bnorm2) : sqrt(rnorm2);
    prm.stats[(size_t)it.cell * 8 + it.rhs0 + tid] = st;
  }
  // The slab, x, reduction slots and coefficients are reused by the next
  // item (peers write into our DSMEM): everyone must be done with them.
  xsync<SLAB>();
}

// Depth dispatch. Mixed (float): depth <= 3 one CTA x 8 rhs; depth 4 one
// CTA x 2 rhs (15-node columns); depth 5 z-slabs of 4 planes x 1 rhs.
// FP64: depth <= 3 one CTA x 8 rhs; depth 4 z-slabs (2 planes) x 2 rhs;
// depth 5 z-slabs of 4 planes x 1 rhs.
// SLAB_ONLY (cluster launches that carry only slab units, e.g. the cluster
// half of a split launch): the independent-item paths are compiled out, so
// the register allocation is the slab path's alone (fewer spills).
template <typename T, int CL, bool HAS_R, bool SLAB_ONLY = false>
__global__ void __launch_bounds__(kQ1Threads, 1) q1_solve_kernel(Q1Params prm) {
  extern __shared__ __align__(256) unsigned char smem[];
  __shared__ Q1Shared sh;
  int rank = 0;
  if constexpr (CL > 1) rank = (int)cg::this_cluster().block_rank();
  for (;;) {
    if constexpr (CL > 1) {
      if (rank == 0 && threadIdx.x == 0) {
        const int u = atomicAdd(prm.queue, 1);
        cg::cluster_group cluster = cg::this_cluster();
        for (int r = 0; r < CL; ++r) cluster.map_shared_rank(&sh, r)->unit = u;
      }
      cg::this_cluster().sync();
    } else {
      if (threadIdx.x == 0) sh.unit = atomicAdd(prm.queue, 1);
      __syncthreads();
    }
    const int u = sh.unit;
    if (u >= prm.n_units) break;
    const Q1Unit U = prm.units[u];
    if (U.slab) {
      if constexpr (CL > 1) {
        const int depth = prm.cells[prm.items[U.first_item].cell].depth;
        if (depth == 5) solve_item<T, 1, 2, 4, HAS_R, true>(prm, sh, smem, U.first_item, rank, CL);
        if constexpr (sizeof(T) == 8) {
          if (depth == 4) solve_item<T, 2, 1, 2, HAS_R, true>(prm, sh, smem, U.first_item, rank, CL);
        }
      }
    } else if (!SLAB_ONLY && rank < U.n_items) {
      const int item = U.first_item + rank;
      const int depth = prm.cells[prm.items[item].cell].depth;
      switch (depth) {
        case 1: solve_item<T, 8, 1, 1, HAS_R, false>(prm, sh, smem, item, 0, 1); break;
        case 2: solve_item<T, 8, 1, 3, HAS_R, false>(prm, sh, smem, item, 0, 1); break;
        case 3: solve_item<T, 8, 1, 7, HAS_R, false>(prm, sh, smem, item, 0, 1); break;
        case 4:
          if constexpr (sizeof(T) == 4) solve_item<T, 2, 1, 15, HAS_R, false>(prm, sh, smem, item, 0, 1);
          break;
        default: break;
      }
    }
    // Every CTA of the cluster has finished the unit before the next dequeue
    // overwrites sh.unit in peers.
    if constexpr (CL > 1)
      cg::this_cluster().sync();
    else
      __syncthreads();
  }
}

template <typename T, int CL, bool HAS_R, bool SLAB_ONLY = false>
cudaError_t launch(const Q1Params &prm, size_t smem_bytes, int grid, cudaStream_t stream) {
  auto kern = q1_solve_kernel<T, CL, HAS_R, SLAB_ONLY>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(kQ1Threads, 1, 1);
  cfg.dynamicSmemBytes = smem_bytes;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = CL > 1 ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, prm);
}

template <typename T, int CL, bool HAS_R, bool SLAB_ONLY = false>
cudaError_t occupancy(size_t smem_bytes, int *out) {
  auto kern = q1_solve_kernel<T, CL, HAS_R, SLAB_ONLY>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
  if (e != cudaSuccess) return e;
  if (CL == 1) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kern, kQ1Threads, smem_bytes);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL * 64, 1, 1);
  cfg.blockDim = dim3(kQ1Threads, 1, 1);
  cfg.dynamicSmemBytes = smem_bytes;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(out, kern, &cfg);
}

}  // namespace q1impl
}  // namespace msfec
