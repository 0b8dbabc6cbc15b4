// Persistent batched Raviart-Thomas x DQ0 (RT_DQ) local solver and Galerkin product (sm_103a).
//
// Restates, for every coarse cell x coarse face (6 bases), the reference's
// mixed local problem of the RT_DQ pairing (konsim83/MPI-MSFEC,
// source/RT_DQ/rt_dq_basis.cc): sigma in RT0 (faces), u in DQ0 (cells),
// local matrix (assemble_system, :466-497; reaction rate 0, eqn_coeff_R.cc:7-14)
//   [ (A^-1 sigma, tau)   -(div tau, u) ]   =  [ M   -B^T ]
//   [ (v, div sigma)            0       ]      [ B     0  ]
// boundary data (setup_basis_dofs_div, :267-389): basis b has the fine fluxes
// of the coarse RT function b on the boundary; right-hand side -+ 1/|K| (v, 1)
// on the cell rows (is_laplace, :515-540; minus for the low faces b = 0, 2, 4).
// On a fine box cell, (B sigma)_c is the net outflow of the 6 face fluxes and
// M is the RT0 mass in factored form (same normal: A^-1_dd h_d^2/(6|c|) times
// the 1D P1 pattern (2,1); normals d != e: A^-1_de h_d h_e / (4|c|)).
// The local problem is a pure-Neumann one: the constant pressure spans the
// kernel. The reference solves it by Schur complement CG after removing the
// mean of the Schur right-hand side (solve_iterative, :683-698); here MINRES
// on the symmetric form (cell rows negated), preconditioner diag(M)^-1 (+)
// diag(B diag(M)^-1 B^T)^-1, FP32 inside FP64 iterative refinement, with the
// cell part of every FP64 residual projected to mean zero. sigma is unique;
// the pressure is not stored: run() overwrites every basis's u block by 1
// (set_u_to_std, :1039-1044) before the Galerkin product, and so does this
// kernel. The last FP64 pass writes y_b = A (sigma_b, 0) for the 7 x 7
// Galerkin product of assemble_global_element_matrix (:822-914).
#include "../../include/msfec_cuda.h"
#include "rtdq_common.cuh"

namespace msfec {
namespace rtimpl {

struct RTGeom {
  int n, L, NFx, NF, NC, N;
};

__device__ __forceinline__ double psi(int a, double t) { return a ? t : 1.0 - t; }

// Per-item constants of the factored RT0 mass (cell sides h).
template <typename TA>
struct RTFactors {
  TA rd[3];     // h_d^2 / (6 |c|): same normal, (2,1) pattern per unit A^-1_dd
  TA ro[3][3];  // h_d h_e / (4 |c|): normals d != e, per unit A^-1_de
};

template <typename TA>
__device__ __forceinline__ void make_factors(const double h[3], RTFactors<TA> &F) {
  const double V = h[0] * h[1] * h[2];
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    F.rd[p] = (TA)(h[p] * h[p] / (6.0 * V));
#pragma unroll
    for (int e = 0; e < 3; ++e) F.ro[p][e] = (TA)(h[p] * h[e] / (4.0 * V));
  }
}

// w = M(A^-1) c for the 6 local faces (x0 x1 y0 y1 z0 z1).
template <typename TA>
__device__ __forceinline__ void rt_mass(const RTFactors<TA> &F, const TA (&A)[3][3], const TA (&c)[6], TA (&w)[6]) {
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

// Element operator of one fine cell, out += A_e z_e (6 face DoFs atomically,
// the cell DoF by its owning thread). MASK: 0 none, 1 keep only
// lattice-boundary face values and no cell value (lift of the boundary data),
// 2 keep only face values. With DOT returns z_f . (A z)_f - z_c (A z)_c.
template <typename TA, typename TV, typename TO, int MASK, bool DOT>
__device__ __forceinline__ TA cell_apply(const TV *__restrict__ z, TO *out, const RTFactors<TA> &F,
                                         const TA (&ai)[6], const int (&fi)[6], int ci, const bool (&fb)[6]) {
  TA zf[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const bool keep = MASK != 1 || fb[t];
    zf[t] = keep ? (TA)z[fi[t]] : TA(0);
  }
  const TA zc = MASK == 0 ? (TA)z[ci] : TA(0);
  const TA A[3][3] = {{ai[0], ai[3], ai[4]}, {ai[3], ai[1], ai[5]}, {ai[4], ai[5], ai[2]}};
  TA yf[6];
  rt_mass(F, A, zf, yf);
  // -(div tau, u): the low face of the cell has outward flux -1, the high one +1
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    yf[2 * d] += zc;
    yf[2 * d + 1] -= zc;
  }
  const TA yc = (zf[1] - zf[0]) + (zf[3] - zf[2]) + (zf[5] - zf[4]);
  TA dot = TA(0);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    atomicAdd(out + fi[t], (TO)yf[t]);
    if (DOT) dot += zf[t] * yf[t];
  }
  out[ci] += (TO)yc;
  if (DOT) dot -= zc * yc;
  return dot;
}

// Face DoFs (x0 x1 y0 y1 z0 z1), boundary flags and cell DoF of fine cell c.
__device__ __forceinline__ void cell_dofs(const RTGeom &g, int c, int (&f)[6], bool (&fb)[6], int &ci) {
  const int n = g.n;
  const int i = c & (n - 1), j = (c >> g.L) & (n - 1), k = c >> (2 * g.L);
  auto fx = [&](int a, int b, int cc) { return a + (n + 1) * (b + n * cc); };
  auto fy = [&](int a, int b, int cc) { return g.NFx + a + n * (b + (n + 1) * cc); };
  auto fz = [&](int a, int b, int cc) { return 2 * g.NFx + a + n * (b + n * cc); };
  f[0] = fx(i, j, k);
  f[1] = fx(i + 1, j, k);
  f[2] = fy(i, j, k);
  f[3] = fy(i, j + 1, k);
  f[4] = fz(i, j, k);
  f[5] = fz(i, j, k + 1);
  fb[0] = i == 0;
  fb[1] = i + 1 == n;
  fb[2] = j == 0;
  fb[3] = j + 1 == n;
  fb[4] = k == 0;
  fb[5] = k + 1 == n;
  ci = g.NF + c;
}

// Normal direction and position along it (0..n) of face DoF d < NF.
__device__ __forceinline__ void face_geometry(const RTGeom &g, int d, int &dir, int &pos) {
  const int n = g.n;
  dir = d / g.NFx;
  const int t = d - dir * g.NFx;
  pos = dir == 0 ? t % (n + 1) : (dir == 1 ? (t / n) % (n + 1) : t / (n * n));
}

// Fine flux of coarse RT function b (BasisRaviartThomas,
// include/functions/basis_raviart_thomas.tpp:38-88) through a face of
// normal dir at position pos: the coarse normal component is linear along
// its normal and constant across, 1 per unit coarse face at its own face.
__device__ __forceinline__ double coarse_flux(int b, int dir, int pos, int n) {
  if (dir != (b >> 1)) return 0.0;
  return psi(b & 1, (double)pos / n) / ((double)n * n);
}

struct RTShared {
  double wred[kRTWarps][3];
  float fred[kRTWarps][3];
  RTFactors<float> Ff;
  RTFactors<double> Fd;
  alignas(16) float fslot[2][kRTWarps];
  double dslot[2][kRTWarps];
  int item;
};

template <typename VT>
__device__ __forceinline__ void warp_publish(RTShared &sh, int slot, VT v) {
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
__device__ __forceinline__ VT slot_total(const RTShared &sh, int slot) {
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
__device__ __forceinline__ void block_sum(RTShared &sh, VT (&v)[NV], VT (&out)[NV]) {
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

extern __shared__ __align__(256) unsigned char rt_dyn_smem[];

// NT = 512 (one CTA per SM) or 256 (two CTAs per SM when the workspace fits twice).
template <typename T, bool SMEM, int NT>
__device__ void solve_item(const RTParams &prm, RTShared &sh, int item_id) {
  constexpr int NW = NT / 32;
  float *ws = SMEM ? reinterpret_cast<float *>(rt_dyn_smem) : prm.scratch + (size_t)blockIdx.x * prm.scratch_floats;
  const NRItem it = prm.items[item_id];
  const NRCell Cc = prm.cells[it.cell];
  RTGeom g;
  g.n = Cc.n;
  g.L = Cc.depth;
  rt_counts(g.n, g.NFx, g.NF, g.NC);
  g.N = g.NF + g.NC;
  const int n = g.n, N = g.N, NF = g.NF;
  const int nc = g.NC;
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
  const RTFactors<float> &Ff = sh.Ff;
  const RTFactors<double> &Fd = sh.Fd;
  const double *ag = prm.ainv6 + 6 * Cc.coef_off;
  double *phi = prm.phi + (size_t)kRTBases * Cc.dof_off + (size_t)bb * N;
  double *yout = prm.y + (size_t)kRTBases * Cc.dof_off + (size_t)bb * N;
  // cell right-hand side -+ |c| / |K| = -+ 1 / n^3 (minus for the low coarse faces)
  const double gc = ((bb & 1) ? 1.0 : -1.0) / (double)nc;
  for (int c = tid; c < nc; c += NT) {
#pragma unroll
    for (int q = 0; q < 6; ++q) cf[8 * c + q] = (float)ag[6 * (size_t)c + q];
    cf[8 * c + 6] = 0.0f;
    cf[8 * c + 7] = 0.0f;
  }
  for (int d = tid; d < (int)Np; d += NT) pd[d] = 0.0f;
  __syncthreads();

  // ---- preconditioner: diag(M) on faces, then sum over interior faces of 1 / M_ff on cells
  for (int c = tid; c < nc; c += NT) {
    int f[6], ci;
    bool fb[6];
    cell_dofs(g, c, f, fb, ci);
    const float *a = cf + 8 * c;
#pragma unroll
    for (int t = 0; t < 6; ++t) atomicAdd(pd + f[t], 2.0f * a[t >> 1] * Ff.rd[t >> 1]);
  }
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int f[6], ci;
    bool fb[6];
    cell_dofs(g, c, f, fb, ci);
    float s = 0.0f;
#pragma unroll
    for (int t = 0; t < 6; ++t)
      if (!fb[t]) s += 1.0f / pd[f[t]];
    pd[ci] = s;
  }
  __syncthreads();
  for (int d = tid; d < N; d += NT) {
    bool fixed = false;
    if (d < NF) {
      int dir, pos;
      face_geometry(g, d, dir, pos);
      fixed = pos == 0 || pos == n;
    }
    const float v = pd[d];
    pd[d] = (fixed || !(v > 0.0f)) ? 0.0f : 1.0f / v;
  }
  __syncthreads();

  double bnorm2 = 0.0, rnorm2 = 0.0;
  int conv = 0, its = 0, flags = 0, nref = 0;
  for (int ir = 0;; ++ir) {
    const bool fp32_res = kMixed && ir == 0;
    if (ir == 0) {
      for (int d = tid; d < N; d += NT) {
        double v = 0.0;
        if (d < NF) {
          int dir, pos;
          face_geometry(g, d, dir, pos);
          v = coarse_flux(bb, dir, pos, n);
        }
        phi[d] = v;
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
      // acc = A phi - rhs (pass 0: A applied to the boundary data only)
      for (int c = tid; c < nc; c += NT) {
        int f[6], ci;
        bool fb[6];
        cell_dofs(g, c, f, fb, ci);
        if (fp32_res) {
          const float *a = cf + 8 * c;
          const float ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          if (pass == 0)
            cell_apply<float, double, float, 1, false>(phi, facc, Ff, ai, f, ci, fb);
          else
            cell_apply<float, double, float, 0, false>(phi, facc, Ff, ai, f, ci, fb);
          facc[ci] -= (float)gc;
        } else {
          const double *a = ag + 6 * (size_t)c;
          const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          if (pass == 0)
            cell_apply<double, double, double, 1, false>(phi, dacc, Fd, ai, f, ci, fb);
          else
            cell_apply<double, double, double, 0, false>(phi, dacc, Fd, ai, f, ci, fb);
          dacc[ci] -= gc;
        }
      }
      __syncthreads();
      // mean of the cell residual (the constant pressure mode), removed below
      double msum[1] = {0.0}, mtot[1];
      for (int d = NF + tid; d < N; d += NT)
        if (pd[d] > 0.0f) msum[0] -= fp32_res ? (double)facc[d] : dacc[d];
      block_sum<double, 1, NW>(sh, msum, mtot);
      const double mean = mtot[0] / (double)nc;
      for (int d = tid; d < N; d += NT) {
        const bool interior = pd[d] > 0.0f;
        const double r = interior ? -(fp32_res ? (double)facc[d] : dacc[d]) - (d >= NF ? mean : 0.0) : 0.0;
        // measured in the preconditioner's norm r^T P r: invariant to the h-scaling
        // of the blocks (RT mass ~ 1/h against the unit cell rows)
        part[pass] += (double)pd[d] * r * r;
        // symmetric form S A (S = +1 on faces, -1 on cells)
        if (pass == 1) vA[d] = (T)(d < NF ? r : -r);
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
        int f[6], ci;
        bool fb[6];
        cell_dofs(g, c, f, fb, ci);
        if constexpr (kMixed) {
          const float4 c0 = reinterpret_cast<const float4 *>(cf)[2 * c];
          const float4 c1 = reinterpret_cast<const float4 *>(cf)[2 * c + 1];
          const float ai[6] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
          dpart += cell_apply<float, float, float, 0, true>(zt, az, Ff, ai, f, ci, fb);
        } else {
          const double *a = ag + 6 * (size_t)c;
          const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
          dpart += cell_apply<double, double, double, 0, true>(zt, az, Fd, ai, f, ci, fb);
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
          const T a = d < NF ? az[d] : -az[d];
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

  // ---------------- y_b = A (sigma_b, 0) (FP64), then u block = 1 ----------------
  for (int d = tid; d < N; d += NT) dacc[d] = 0.0;
  __syncthreads();
  for (int c = tid; c < nc; c += NT) {
    int f[6], ci;
    bool fb[6];
    cell_dofs(g, c, f, fb, ci);
    const double *a = ag + 6 * (size_t)c;
    const double ai[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
    cell_apply<double, double, double, 2, false>(phi, dacc, Fd, ai, f, ci, fb);
  }
  __syncthreads();
  for (int d = tid; d < N; d += NT) {
    yout[d] = dacc[d];
    if (d >= NF) phi[d] = 1.0;
  }
  if (tid == 0) {
    NRStat st;
    st.iters = its;
    st.refinements = nref;
    st.converged = conv;
    st.flags = flags;
    st.rel_residual = bnorm2 > 0.0 ? sqrt(rnorm2 / bnorm2) : sqrt(rnorm2);
    prm.stats[(size_t)it.cell * kRTBases + bb] = st;
  }
  __syncthreads();
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT, 512 / NT) rtdq_solve_kernel(RTParams prm) {
  __shared__ RTShared sh;
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

// One coarse cell per CTA. K_H[i][j] = t_i . (A t_j) over all DoFs on the FP64
// tensor pipe (one m8n8k4 tile, k over the DoFs), with the reference's test /
// trial vectors (index i -> basis i % 6, u block set to 1): t_i = (sigma_i, 0)
// for i < 6, t_6 = (0, 1). A t_j = y_j for j < 6; A t_6 = (-B^T 1, 0) is +1 on
// the low and -1 on the high boundary faces of each direction, 0 elsewhere.
// F_H[6] = 1 . (v, f) = the integral of f over the coarse cell (2x2x2 Gauss per
// fine cell), F_H[0..5] = 0.
__global__ void __launch_bounds__(kGalThreads) rtdq_galerkin_kernel(const NRCell *__restrict__ cells,
                                                                    const double *__restrict__ phi,
                                                                    const double *__restrict__ y, msfec_load load,
                                                                    double *__restrict__ KH,
                                                                    double *__restrict__ FH) {
  __shared__ double red[kGalWarps][64];
  __shared__ double redf[kGalWarps];
  const int cc = blockIdx.x;
  const NRCell C = cells[cc];
  RTGeom g;
  g.n = C.n;
  g.L = C.depth;
  rt_counts(g.n, g.NFx, g.NF, g.NC);
  g.N = g.NF + g.NC;
  const int n = g.n, N = g.N, NF = g.NF;
  const double *P = phi + (size_t)kRTBases * C.dof_off;
  const double *Y = y + (size_t)kRTBases * C.dof_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gr = lane >> 2, t4 = lane & 3;
  double acc0 = 0.0, acc1 = 0.0;
  for (int base = warp * 4; base < N; base += kGalWarps * 4) {
    const int d = base + t4;
    const bool ok = d < N;
    const bool face = d < NF;
    double a = 0.0, b = 0.0;
    if (ok) {
      if (gr < kRTBases) {
        a = face ? __ldcs(P + (size_t)gr * N + d) : 0.0;
        b = __ldcs(Y + (size_t)gr * N + d);
      } else if (gr == kRTBases) {
        a = face ? 0.0 : 1.0;
        if (face) {
          int dir, pos;
          face_geometry(g, d, dir, pos);
          b = pos == 0 ? 1.0 : (pos == n ? -1.0 : 0.0);
        }
      }
    }
    dmma(acc0, acc1, a, b);
  }
  // F_H[6]
  double fs = 0.0;
  if (load.kind == MSFEC_LOAD_CONSTANT) {
    if (threadIdx.x == 0) fs = load.params[0] * (C.h[0] * n) * (C.h[1] * n) * (C.h[2] * n);
  } else if (load.kind == MSFEC_LOAD_SIN_PRODUCT) {
    const double w = load.params[1] * M_PI, p0 = load.params[0];
    const double gq = 0.5 / sqrt(3.0);
    const double qp[2] = {0.5 - gq, 0.5 + gq};
    const double jxw = 0.125 * C.h[0] * C.h[1] * C.h[2];
    for (int c = threadIdx.x; c < g.NC; c += kGalThreads) {
      const int i = c & (n - 1), j = (c >> g.L) & (n - 1), k = c >> (2 * g.L);
      for (int q = 0; q < 8; ++q) {
        const double X = C.origin[0] + (i + qp[q & 1]) * C.h[0];
        const double Yq = C.origin[1] + (j + qp[(q >> 1) & 1]) * C.h[1];
        const double Z = C.origin[2] + (k + qp[q >> 2]) * C.h[2];
        fs += jxw * p0 * sin(w * X) * sin(w * Yq) * sin(w * Z);
      }
    }
  }
  for (int off = 16; off >= 1; off >>= 1) fs += __shfl_xor_sync(0xffffffffu, fs, off);
  if (lane == 0) redf[warp] = fs;
  // C fragment of m8n8k4: lane holds row gr, cols 2*t4, 2*t4+1
  red[warp][gr * 8 + 2 * t4] = acc0;
  red[warp][gr * 8 + 2 * t4 + 1] = acc1;
  __syncthreads();
  for (int t = threadIdx.x; t < kRTCoarse * kRTCoarse; t += kGalThreads) {
    const int i = t / kRTCoarse, j = t % kRTCoarse;
    double s = 0.0;
    for (int w = 0; w < kGalWarps; ++w) s += red[w][i * 8 + j];
    KH[(size_t)cc * kRTCoarse * kRTCoarse + t] = s;
  }
  if (threadIdx.x < kRTCoarse) {
    double s = 0.0;
    if (threadIdx.x == kRTBases)
      for (int w = 0; w < kGalWarps; ++w) s += redf[w];
    FH[(size_t)cc * kRTCoarse + threadIdx.x] = s;
  }
}

__global__ void rtdq_report_kernel(const NRStat *__restrict__ stats, int ncells, msfec_cell_report *rep) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  msfec_cell_report r;
  r.iterations = 0;
  r.refinements = 0;
  r.converged = 1;
  r.iterations_sum = 0;
  r.residual = 0.0;
  for (int b = 0; b < kRTBases; ++b) {
    const NRStat s = stats[(size_t)c * kRTBases + b];
    r.iterations = max(r.iterations, s.iters);
    r.iterations_sum += s.iters;
    r.refinements = max(r.refinements, s.refinements);
    r.converged = r.converged && s.converged && !(s.flags & 1);
    r.residual = fmax(r.residual, s.rel_residual);
    if (!isfinite(s.rel_residual)) r.residual = s.rel_residual;
  }
  rep[c] = r;
}

}  // namespace rtimpl

cudaError_t rtdq_solve_launch(bool fp64, bool two_per_sm, const RTParams &prm, size_t smem, int grid,
                              cudaStream_t st) {
  if (two_per_sm) {  // mixed precision, shared workspace that fits twice per SM
    auto k = rtimpl::rtdq_solve_kernel<float, 256>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    k<<<grid, 256, smem, st>>>(prm);
    return cudaGetLastError();
  }
  if (fp64) {
    auto k = rtimpl::rtdq_solve_kernel<double, kRTThreads>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kRTThreads, smem, st>>>(prm);
  } else {
    auto k = rtimpl::rtdq_solve_kernel<float, kRTThreads>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kRTThreads, smem, st>>>(prm);
  }
  return cudaGetLastError();
}

cudaError_t rtdq_galerkin_launch(const NRCell *cells, int ncells, const double *phi, const double *y,
                                 const msfec_load &load, double *KH, double *FH, msfec_cell_report *rep,
                                 const NRStat *stats, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  rtimpl::rtdq_galerkin_kernel<<<ncells, rtimpl::kGalThreads, 0, st>>>(cells, phi, y, load, KH, FH);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !rep) return e;
  rtimpl::rtdq_report_kernel<<<(ncells + 127) / 128, 128, 0, st>>>(stats, ncells, rep);
  return cudaGetLastError();
}

}  // namespace msfec
