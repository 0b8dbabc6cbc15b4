// Persistent batched Q1 local solver for a tensor diffusion coefficient (sm_103a).
//
// The scalar-coefficient solver (q1_solve_impl.cuh) applies a * K_unit through
// a node-centred 27-point stencil of layer sums. A full tensor A, and a tensor
// that varies over the Gauss points of a fine cell, break that structure, so
// this solver applies the operator cell by cell the way the reference's
// assembly forms it (QBasis::assemble_system, source/Q/q_basis.cc:222-231;
// Diffusion_A::value_list, source/equation_data/eqn_coeff_A.cc:162-191):
//   (K p)_u = sum_e sum_q grad psi_u(x_q) . A(x_q) grad p_h(x_q) JxW_q
// over the 2x2x2 Gauss points x_q of each fine cell e. The gradient of a
// trilinear function along x is bilinear in (y, z): it is evaluated at the 4
// (y, z) Gauss pairs from the 4 x-differences of the nodal values by one 2x2
// interpolation W d W^T (W_gv = psi_v(xi_g)), and the same for y and z; the
// fluxes B_q grad p (B_q = |e|/8 H A(x_q) H, H = diag(1/h)) are summed along
// their own axis and sent back through the same W. Contributions go to the
// 8 nodes with shared-memory atomics (global atomics for cells whose vectors
// exceed shared memory).
//
// Everything else restates the reference's local problem as the scalar
// solver does (q_basis.cc:117-170, 304-357, 545-565): Dirichlet data of
// coarse vertex v = the trilinear function BasisQ1_v
// (include/functions/basis_q1.tpp:92-152), no load in the basis problems,
// FP32 Jacobi-PCG inside FP64 iterative refinement (plain FP64 PCG for the
// FP64 path), stop when ||r||_2 <= rtol ||K_IB g||_2, then y = K phi with the
// unconstrained K for the Galerkin kernel (q_basis.cc:262-300).
#include "../../include/msfec_cuda.h"
#include "q1_common.cuh"

namespace msfec {

namespace q1gimpl {

struct Q1GShared {
  float fslot[2][kQ1GWarps];
  double dslot[2][kQ1GWarps];
  int item;
};

extern __shared__ __align__(256) unsigned char q1g_dyn_smem[];

// W d W^T with W = [[w0, w1], [w1, w0]], W_gv = psi_v(xi_g) at the two Gauss
// points xi_0 < xi_1 of [0, 1] (psi_0 = 1 - t, psi_1 = t). W is symmetric, so
// the same map is the transpose (Gauss points -> vertices).
template <typename TA>
__device__ __forceinline__ void interp2(const TA (&d)[2][2], TA (&G)[2][2]) {
  const TA w0 = TA(0.78867513459481288225), w1 = TA(0.21132486540518711775);
  const TA t00 = w0 * d[0][0] + w1 * d[1][0], t10 = w1 * d[0][0] + w0 * d[1][0];
  const TA t01 = w0 * d[0][1] + w1 * d[1][1], t11 = w1 * d[0][1] + w0 * d[1][1];
  G[0][0] = w0 * t00 + w1 * t01;
  G[0][1] = w1 * t00 + w0 * t01;
  G[1][0] = w0 * t10 + w1 * t11;
  G[1][1] = w1 * t10 + w0 * t11;
}

// y = K_e p for one fine cell, local vertex v = vx + 2 vy + 4 vz.
// bget(g, k): entry k (b00 b11 b22 b01 b02 b12) of the scaled tensor at Gauss
// point g (x fastest); rv = reaction * |e| (0: none). Returns p . y.
template <typename TA, bool HAS_R, typename BGet>
__device__ __forceinline__ TA elem_apply(const TA (&p)[8], BGet bget, TA rv, TA (&y)[8]) {
  TA dx[2][2], dy[2][2], dz[2][2];  // x-differences at (vy, vz), y- at (vx, vz), z- at (vx, vy)
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      dx[a][b] = p[1 + 2 * a + 4 * b] - p[2 * a + 4 * b];
      dy[a][b] = p[a + 2 + 4 * b] - p[a + 4 * b];
      dz[a][b] = p[a + 2 * b + 4] - p[a + 2 * b];
    }
  TA gx[2][2], gy[2][2], gz[2][2];  // reference gradient components at the Gauss pairs
  interp2(dx, gx);
  interp2(dy, gy);
  interp2(dz, gz);
  TA sx[2][2], sy[2][2], sz[2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) sx[a][b] = sy[a][b] = sz[a][b] = TA(0);
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    const int qx = g & 1, qy = (g >> 1) & 1, qz = g >> 2;
    const TA ux = gx[qy][qz], uy = gy[qx][qz], uz = gz[qx][qy];
    const TA b0 = bget(g, 0), b1 = bget(g, 1), b2 = bget(g, 2), b3 = bget(g, 3), b4 = bget(g, 4), b5 = bget(g, 5);
    sx[qy][qz] += b0 * ux + b3 * uy + b4 * uz;
    sy[qx][qz] += b3 * ux + b1 * uy + b5 * uz;
    sz[qx][qy] += b4 * ux + b5 * uy + b2 * uz;
  }
  TA X[2][2], Y[2][2], Z[2][2];
  interp2(sx, X);
  interp2(sy, Y);
  interp2(sz, Z);
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const int vx = v & 1, vy = (v >> 1) & 1, vz = v >> 2;
    y[v] = (vx ? X[vy][vz] : -X[vy][vz]) + (vy ? Y[vx][vz] : -Y[vx][vz]) + (vz ? Z[vx][vy] : -Z[vx][vy]);
  }
  if constexpr (HAS_R) {  // r |e| (M (x) M (x) M) p, M = [1/3 1/6; 1/6 1/3]
    TA t[8], u[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) t[v] = (TA(2) * p[v] + p[v ^ 1]) * TA(1.0 / 6.0);
#pragma unroll
    for (int v = 0; v < 8; ++v) u[v] = (TA(2) * t[v] + t[v ^ 2]) * TA(1.0 / 6.0);
#pragma unroll
    for (int v = 0; v < 8; ++v) y[v] += rv * (TA(2) * u[v] + u[v ^ 4]) * TA(1.0 / 6.0);
  }
  TA d = TA(0);
#pragma unroll
  for (int v = 0; v < 8; ++v) d += p[v] * y[v];
  return d;
}

// Diagonal entry K_e[u][u] (Jacobi scaling): sum_g grad psi_u(g) . B_g grad psi_u(g) + r |e| / 27.
template <typename BGet>
__device__ __forceinline__ float elem_diag(int u, BGet bget, float rv) {
  const float w[2][2] = {{0.78867513459481288225f, 0.21132486540518711775f},
                         {0.21132486540518711775f, 0.78867513459481288225f}};  // w[g][v] = psi_v(xi_g)
  const int ux = u & 1, uy = (u >> 1) & 1, uz = u >> 2;
  const float sxv = ux ? 1.0f : -1.0f, syv = uy ? 1.0f : -1.0f, szv = uz ? 1.0f : -1.0f;
  float s = rv * (1.0f / 27.0f);
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    const int qx = g & 1, qy = (g >> 1) & 1, qz = g >> 2;
    const float gxv = sxv * w[qy][uy] * w[qz][uz];
    const float gyv = w[qx][ux] * syv * w[qz][uz];
    const float gzv = w[qx][ux] * w[qy][uy] * szv;
    s += bget(g, 0) * gxv * gxv + bget(g, 1) * gyv * gyv + bget(g, 2) * gzv * gzv +
         2.0f * (bget(g, 3) * gxv * gyv + bget(g, 4) * gxv * gzv + bget(g, 5) * gyv * gzv);
  }
  return s;
}

__device__ __forceinline__ double trilinear(int v, int i, int j, int k, int n) {
  const double inv = 1.0 / n;
  const double tx = i * inv, ty = j * inv, tz = k * inv;
  return ((v & 1) ? tx : 1.0 - tx) * ((v & 2) ? ty : 1.0 - ty) * ((v & 4) ? tz : 1.0 - tz);
}

// Same summation order in every thread: identical decisions block-wide.
template <typename VT, int NV>
__device__ __forceinline__ void block_sum(Q1GShared &sh, VT (&v)[NV], VT (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < NV; ++t)
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v[t] += __shfl_xor_sync(0xffffffffu, v[t], off);
  __syncthreads();  // the previous readers of the slots are done
  if (lane == 0)
#pragma unroll
    for (int t = 0; t < NV; ++t) {
      if constexpr (sizeof(VT) == 4)
        sh.fslot[t][warp] = v[t];
      else
        sh.dslot[t][warp] = v[t];
    }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < NV; ++t) {
    VT s = VT(0);
#pragma unroll
    for (int w = 0; w < kQ1GWarps; ++w) {
      if constexpr (sizeof(VT) == 4)
        s += sh.fslot[t][w];
      else
        s += sh.dslot[t][w];
    }
    out[t] = s;
  }
}

// Node indices of fine cell (i, j, k): base + the 8 corner offsets.
__device__ __forceinline__ void cell_nodes(int c, int n, int (&nd)[8]) {
  const int N1 = n + 1;
  const int i = c % n, j = (c / n) % n, k = c / (n * n);
  const int b = i + N1 * (j + N1 * k);
#pragma unroll
  for (int v = 0; v < 8; ++v) nd[v] = b + (v & 1) + ((v >> 1) & 1) * N1 + (v >> 2) * N1 * N1;
}

__device__ __forceinline__ bool lattice_boundary(int node, int n) {
  const int N1 = n + 1;
  const int i = node % N1, j = (node / N1) % N1, k = node / (N1 * N1);
  return i == 0 || j == 0 || k == 0 || i == n || j == n || k == n;
}

// One (cell, vertex) item. VSMEM: the vectors live in dynamic shared memory,
// else in this CTA's slot of the global scratch; ESMEM: the cell's element
// data is staged into shared memory after them, else read from global (L2).
template <typename T, bool VSMEM, bool ESMEM, bool HAS_R>
__device__ void solve_item(const Q1GParams &prm, Q1GShared &sh, int item_id) {
  constexpr int NT = kQ1GThreads;
  constexpr bool kMixed = sizeof(T) == 4;
  const int tid = threadIdx.x;
  const Q1GItem it = prm.items[item_id];
  const Q1Cell C = prm.cells[it.cell];
  const int n = C.n, N1 = n + 1;
  const int nn = N1 * N1 * N1, nc = n * n * n;
  const size_t Np = ((size_t)nn + 63) / 64 * 64;
  const int CW = q1g_ed_floats(prm.gauss);
  float *ws = VSMEM ? reinterpret_cast<float *>(q1g_dyn_smem) : prm.scratch + (size_t)blockIdx.x * prm.scratch_floats;
  float *dinv = ws;
  T *xv = reinterpret_cast<T *>(ws + Np);
  T *rv = xv + Np;
  T *pv = rv + Np;
  T *qv = pv + Np;
  double *dacc = reinterpret_cast<double *>(pv);  // FP64 residual / y accumulator, aliases p, q
  const float *ed = prm.ed + (size_t)C.coef_off * CW;
  if constexpr (ESMEM) {
    float *eds = reinterpret_cast<float *>(q1g_dyn_smem) + q1g_vec_floats(n, (int)sizeof(T));
    const float4 *src = reinterpret_cast<const float4 *>(ed);
    float4 *dst = reinterpret_cast<float4 *>(eds);
    for (int t = tid; t < nc * CW / 4; t += NT) dst[t] = src[t];
    ed = eds;
  }
  const bool src_mode = it.mode == 1;
  const int v0 = it.vertex;
  const size_t plane = (size_t)8 * C.node_off + (size_t)v0 * nn;
  double *phi = src_mode ? prm.src_out + plane : prm.phi + plane;
  const double *fsrc = src_mode ? prm.src_rhs + plane : nullptr;
  const bool gauss = prm.gauss != 0;
  const double *ag = prm.a + (size_t)C.coef_off * (gauss ? 48 : 6);
  const double *rg = HAS_R ? prm.react + C.coef_off : nullptr;
  const double vol = C.h[0] * C.h[1] * C.h[2];
  double bsc[6];  // |e|/8 / (h_p h_q) of entry (p, q) in b00 b11 b22 b01 b02 b12 order
  {
    const double w = vol / 8.0;
    const double ih[3] = {1.0 / C.h[0], 1.0 / C.h[1], 1.0 / C.h[2]};
    bsc[0] = w * ih[0] * ih[0];
    bsc[1] = w * ih[1] * ih[1];
    bsc[2] = w * ih[2] * ih[2];
    bsc[3] = w * ih[0] * ih[1];
    bsc[4] = w * ih[0] * ih[2];
    bsc[5] = w * ih[1] * ih[2];
  }
  // element accessors: float element data, or the FP64 input scaled on the fly
  auto bget_f = [&](int c) {
    const float *b = ed + (size_t)c * CW;
    const int gs = prm.gauss ? 6 : 0;
    return [b, gs](int g, int k) { return b[g * gs + k]; };
  };
  auto bget_d = [&](int c) {
    const double *b = ag + (size_t)c * (gauss ? 48 : 6);
    const int gs = gauss ? 6 : 0;
    return [b, gs, &bsc](int g, int k) { return __ldg(b + g * gs + k) * bsc[k]; };
  };

  // ---- Jacobi scaling: the assembled diagonal on interior nodes, 0 on the boundary
  for (int d = tid; d < (int)Np; d += NT) dinv[d] = 0.0f;
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int nd[8];
    cell_nodes(c, n, nd);
    const float r = HAS_R ? ed[(size_t)c * CW + (prm.gauss ? 48 : 6)] : 0.0f;
    const auto bg = bget_f(c);
#pragma unroll
    for (int u = 0; u < 8; ++u) atomicAdd(dinv + nd[u], elem_diag(u, bg, r));
  }
  __syncthreads();
  for (int d = tid; d < nn; d += NT) dinv[d] = lattice_boundary(d, n) ? 0.0f : 1.0f / dinv[d];
  __syncthreads();

  double bnorm2 = 0.0, rnorm2 = 0.0;
  int conv = 0, its = 0, flags = 0, nref = 0;
  for (int ir = 0;; ++ir) {
    if (ir == 0) {  // phi_0: the coarse vertex function on every node (basis), 0 (source)
      for (int d = tid; d < nn; d += NT)
        phi[d] = src_mode ? 0.0 : trilinear(v0, d % N1, (d / N1) % N1, d / (N1 * N1), n);
      __syncthreads();
    }
    // ---- FP64 residual r = f - K phi on the interior; pass 0: lift of the boundary data only
    double part[2] = {0.0, 0.0};
    for (int pass = (ir == 0 ? 0 : 1); pass < 2; ++pass) {
      for (int d = tid; d < nn; d += NT) dacc[d] = (src_mode && dinv[d] > 0.0f) ? -fsrc[d] : 0.0;
      __syncthreads();
      for (int c = tid; c < nc; c += NT) {
        int nd[8];
        cell_nodes(c, n, nd);
        double pe[8], ye[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) pe[v] = (pass == 1 || dinv[nd[v]] == 0.0f) ? phi[nd[v]] : 0.0;
        elem_apply<double, HAS_R>(pe, bget_d(c), HAS_R ? rg[c] * vol : 0.0, ye);
#pragma unroll
        for (int v = 0; v < 8; ++v) atomicAdd(dacc + nd[v], ye[v]);
      }
      __syncthreads();
      for (int d = tid; d < nn; d += NT) {
        const double r = dinv[d] > 0.0f ? -dacc[d] : 0.0;
        part[pass] += r * r;
        if (pass == 1) rv[d] = (T)r;  // rv is disjoint from the accumulator
      }
      __syncthreads();
    }
    {
      double tot[2];
      block_sum<double, 2>(sh, part, tot);
      if (ir == 0) bnorm2 = src_mode ? tot[1] : tot[0];
      rnorm2 = tot[1];
    }
    ++nref;
    conv = rnorm2 <= prm.rtol * prm.rtol * bnorm2;
    if (conv || ir >= prm.max_refine) break;

    // ---- PCG on K_II x = r (precision T), Jacobi preconditioner
    const double tol_abs2 = prm.rtol * prm.rtol * bnorm2;
    const double target2 = kMixed ? fmax(prm.inner_rtol * prm.inner_rtol * rnorm2, 0.01 * tol_abs2) : 0.25 * tol_abs2;
    T rz;
    {
      T pz[1] = {T(0)};
      for (int d = tid; d < (int)Np; d += NT) {
        const T z = (T)dinv[d] * (d < nn ? rv[d] : T(0));
        if (d >= nn) rv[d] = T(0);
        xv[d] = T(0);
        pv[d] = z;
        qv[d] = T(0);
        pz[0] += z * rv[d];
      }
      T t1[1];
      block_sum<T, 1>(sh, pz, t1);
      rz = t1[0];
    }
    bool active = rz > T(0) && rnorm2 > target2;
    for (int iter = 0; active && iter < prm.max_iter; ++iter) {
      // phase 1: q = K p cell by cell, delta = p . K p from the element sums
      T dpart[1] = {T(0)};
      for (int c = tid; c < nc; c += NT) {
        int nd[8];
        cell_nodes(c, n, nd);
        T pe[8], ye[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) pe[v] = pv[nd[v]];
        if constexpr (kMixed)
          dpart[0] += elem_apply<float, HAS_R>(pe, bget_f(c), HAS_R ? ed[(size_t)c * CW + (prm.gauss ? 48 : 6)] : 0.0f, ye);
        else
          dpart[0] += elem_apply<double, HAS_R>(pe, bget_d(c), HAS_R ? rg[c] * vol : 0.0, ye);
#pragma unroll
        for (int v = 0; v < 8; ++v) atomicAdd(qv + nd[v], ye[v]);
      }
      T delta[1];
      block_sum<T, 1>(sh, dpart, delta);
      if (!(delta[0] > T(0)) || !isfinite(delta[0])) {
        flags |= 1;
        break;
      }
      const T alpha = rz / delta[0];
      // phase 2: x, r updates on the interior, z = D^-1 r, r.z and r.r; q cleared
      T pr[2] = {T(0), T(0)};
      for (int d = tid; d < nn; d += NT) {
        const float di = dinv[d];
        if (di > 0.0f) {
          xv[d] += alpha * pv[d];
          const T r = rv[d] - alpha * qv[d];
          rv[d] = r;
          pr[0] += (T)di * r * r;
          pr[1] += r * r;
        }
        qv[d] = T(0);
      }
      T tot[2];
      block_sum<T, 2>(sh, pr, tot);
      const T beta = tot[0] / rz;
      rz = tot[0];
      ++its;
      if ((double)tot[1] <= target2 || !(rz > T(0))) active = false;
      // phase 3: p = z + beta p
      if (active) {
        for (int d = tid; d < nn; d += NT) pv[d] = (T)dinv[d] * rv[d] + beta * pv[d];
        __syncthreads();
      }
    }
    __syncthreads();
    // ---- phi_I += x (FP64)
    for (int d = tid; d < nn; d += NT)
      if (dinv[d] > 0.0f) phi[d] += (double)xv[d];
    __syncthreads();
  }

  // ---- y = K phi with the unconstrained operator (all nodes), FP64
  if (!src_mode) {
    double *yout = prm.y + plane;
    for (int d = tid; d < nn; d += NT) dacc[d] = 0.0;
    __syncthreads();
    for (int c = tid; c < nc; c += NT) {
      int nd[8];
      cell_nodes(c, n, nd);
      double pe[8], ye[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) pe[v] = phi[nd[v]];
      elem_apply<double, HAS_R>(pe, bget_d(c), HAS_R ? rg[c] * vol : 0.0, ye);
#pragma unroll
      for (int v = 0; v < 8; ++v) atomicAdd(dacc + nd[v], ye[v]);
    }
    __syncthreads();
    for (int d = tid; d < nn; d += NT) yout[d] = dacc[d];
  }
  if (tid == 0) {
    Q1Stat st;
    st.iters = its;
    st.refinements = nref;
    st.converged = conv;
    st.flags = flags;
    st.rel_residual = bnorm2 > 0.0 ? sqrt(rnorm2 / bnorm2) : sqrt(rnorm2);
    prm.stats[(size_t)it.cell * 8 + v0] = st;
  }
  __syncthreads();
}

template <typename T, bool VSMEM, bool ESMEM, bool HAS_R>
__global__ void __launch_bounds__(kQ1GThreads) q1g_solve_kernel(Q1GParams prm) {
  __shared__ Q1GShared sh;
  for (;;) {
    if (threadIdx.x == 0) sh.item = atomicAdd(prm.queue, 1);
    __syncthreads();
    const int item = sh.item;
    if (item >= prm.n_items) break;
    solve_item<T, VSMEM, ESMEM, HAS_R>(prm, sh, item);
  }
}

// Element data of every fine cell: B_q = |e|/8 H A(x_q) H (6 entries per point),
// r |e| and padding, in float.
__global__ void q1g_prepare_kernel(const Q1Cell *__restrict__ cells, int ncells, const double *__restrict__ a,
                                   int gauss, const double *__restrict__ react, float *__restrict__ ed) {
  const int CW = q1g_ed_floats(gauss), np = gauss ? 8 : 1;
  for (int cc = blockIdx.x; cc < ncells; cc += gridDim.x) {
    const Q1Cell C = cells[cc];
    const int nc = C.n * C.n * C.n;
    const double vol = C.h[0] * C.h[1] * C.h[2], w = vol / 8.0;
    const double ih[3] = {1.0 / C.h[0], 1.0 / C.h[1], 1.0 / C.h[2]};
    const double sc[6] = {w * ih[0] * ih[0], w * ih[1] * ih[1], w * ih[2] * ih[2],
                          w * ih[0] * ih[1], w * ih[0] * ih[2], w * ih[1] * ih[2]};
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
      const size_t e = (size_t)C.coef_off + c;
      const double *src = a + e * (size_t)(6 * np);
      float *dst = ed + e * (size_t)CW;
      for (int g = 0; g < np; ++g)
#pragma unroll
        for (int k = 0; k < 6; ++k) dst[6 * g + k] = (float)(src[6 * g + k] * sc[k]);
      dst[6 * np] = react ? (float)(react[e] * vol) : 0.0f;
      for (int k = 6 * np + 1; k < CW; ++k) dst[k] = 0.0f;
    }
  }
}

// Adjoint gradient for A_e -> exp(theta_e) A_e per fine cell (the tensor
// analogue of q1_gradient_kernel; d K_e / d theta_e = K_e(A_e), the reaction
// is not scaled): dJ/dtheta_e = -[(mu + psi_U)_e . K_e psi_l,e + eta_e . K_e psi_U,e]
// with psi_U = Phi U, psi_l = Phi lambda and the adjoint local solutions mu
// (plane 0 of sol) and eta (plane 1). One block per coarse cell.
__global__ void __launch_bounds__(256) q1g_gradient_kernel(const Q1Cell *__restrict__ cells,
                                                          const double *__restrict__ a, int gauss,
                                                          const double *__restrict__ phi,
                                                          const double *__restrict__ sol,
                                                          const double *__restrict__ U,
                                                          const double *__restrict__ lam,
                                                          double *__restrict__ grad) {
  const int c = blockIdx.x;
  const Q1Cell C = cells[c];
  const int n = C.n, N1 = n + 1;
  const size_t nn = (size_t)N1 * N1 * N1;
  const double vol = C.h[0] * C.h[1] * C.h[2], w = vol / 8.0;
  const double ih[3] = {1.0 / C.h[0], 1.0 / C.h[1], 1.0 / C.h[2]};
  const double bsc[6] = {w * ih[0] * ih[0], w * ih[1] * ih[1], w * ih[2] * ih[2],
                         w * ih[0] * ih[1], w * ih[0] * ih[2], w * ih[1] * ih[2]};
  double u8[8], l8[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    u8[v] = U[(size_t)c * 8 + v];
    l8[v] = lam[(size_t)c * 8 + v];
  }
  const double *ph = phi + 8 * C.node_off;
  const double *mu = sol + 8 * C.node_off;
  const double *eta = mu + nn;
  const int nc = n * n * n;
  const int stride = gauss ? 48 : 6, gs = gauss ? 6 : 0;
  for (int e = threadIdx.x; e < nc; e += blockDim.x) {
    int nd[8];
    cell_nodes(e, n, nd);
    double pu[8], pl[8], pm[8], pe[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      double su = 0.0, sl = 0.0;
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const double p = ph[(size_t)v * nn + nd[u]];
        su += u8[v] * p;
        sl += l8[v] * p;
      }
      pu[u] = su;
      pl[u] = sl;
      pm[u] = mu[nd[u]] + su;
      pe[u] = eta[nd[u]];
    }
    const double *b = a + ((size_t)C.coef_off + e) * stride;
    auto bget = [b, gs, &bsc](int g, int k) { return __ldg(b + g * gs + k) * bsc[k]; };
    double kl[8], ku[8];
    elem_apply<double, false>(pl, bget, 0.0, kl);
    elem_apply<double, false>(pu, bget, 0.0, ku);
    double acc = 0.0;
#pragma unroll
    for (int u = 0; u < 8; ++u) acc += pm[u] * kl[u] + pe[u] * ku[u];
    grad[C.coef_off + e] = -acc;
  }
}

}  // namespace q1gimpl

cudaError_t q1g_gradient_launch(const Q1Cell *cells, int ncells, const double *a, int gauss, const double *phi,
                                const double *sol, const double *U, const double *lam, double *grad,
                                cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  q1gimpl::q1g_gradient_kernel<<<ncells, 256, 0, st>>>(cells, a, gauss, phi, sol, U, lam, grad);
  return cudaGetLastError();
}

template <typename T, bool VSMEM, bool ESMEM, bool HAS_R>
static cudaError_t q1g_launch_t(const Q1GParams &prm, size_t smem, int grid, cudaStream_t st) {
  auto k = q1gimpl::q1g_solve_kernel<T, VSMEM, ESMEM, HAS_R>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, kQ1GThreads, smem, st>>>(prm);
  return cudaGetLastError();
}

template <typename T, bool HAS_R>
static cudaError_t q1g_launch_p(int placement, const Q1GParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (placement == 2) return q1g_launch_t<T, true, true, HAS_R>(prm, smem, grid, st);
  if (placement == 1) return q1g_launch_t<T, true, false, HAS_R>(prm, smem, grid, st);
  return q1g_launch_t<T, false, false, HAS_R>(prm, smem, grid, st);
}

// placement: 2 vectors and element data in shared memory, 1 vectors only,
// 0 neither (global scratch slots).
cudaError_t q1g_solve_launch(bool fp64, bool has_r, int placement, const Q1GParams &prm, size_t smem, int grid,
                             cudaStream_t st) {
  if (fp64)
    return has_r ? q1g_launch_p<double, true>(placement, prm, smem, grid, st)
                 : q1g_launch_p<double, false>(placement, prm, smem, grid, st);
  return has_r ? q1g_launch_p<float, true>(placement, prm, smem, grid, st)
               : q1g_launch_p<float, false>(placement, prm, smem, grid, st);
}

cudaError_t q1g_solve_occupancy(bool fp64, bool has_r, int placement, size_t smem, int *blocks_per_sm) {
  auto pick = [&](auto k) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, kQ1GThreads, smem);
  };
  using namespace q1gimpl;
  if (fp64) {
    if (has_r)
      return placement == 2 ? pick(q1g_solve_kernel<double, true, true, true>)
                            : (placement == 1 ? pick(q1g_solve_kernel<double, true, false, true>)
                                              : pick(q1g_solve_kernel<double, false, false, true>));
    return placement == 2 ? pick(q1g_solve_kernel<double, true, true, false>)
                          : (placement == 1 ? pick(q1g_solve_kernel<double, true, false, false>)
                                            : pick(q1g_solve_kernel<double, false, false, false>));
  }
  if (has_r)
    return placement == 2 ? pick(q1g_solve_kernel<float, true, true, true>)
                          : (placement == 1 ? pick(q1g_solve_kernel<float, true, false, true>)
                                            : pick(q1g_solve_kernel<float, false, false, true>));
  return placement == 2 ? pick(q1g_solve_kernel<float, true, true, false>)
                        : (placement == 1 ? pick(q1g_solve_kernel<float, true, false, false>)
                                          : pick(q1g_solve_kernel<float, false, false, false>));
}

cudaError_t q1g_prepare_launch(const Q1Cell *cells, int ncells, const double *a, int gauss, const double *react,
                               float *ed, int grid, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  q1gimpl::q1g_prepare_kernel<<<grid, 256, 0, st>>>(cells, ncells, a, gauss, react, ed);
  return cudaGetLastError();
}

}  // namespace msfec
