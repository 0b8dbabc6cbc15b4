// Ned_RT multilevel setup, Galerkin, report and adjoint kernels, and the
// dispatch of the persistent solver over its per-precision translation
// units (the solver itself: nedrt_solver.cuh).
#include <cuda_fp16.h>

#include "nedrt_solver.cuh"

namespace msfec {
namespace nrimpl {

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

// ---------------- shared per-cell data of the global-workspace solver ----------------
// The float coefficients and the preconditioner diagonal (block-Jacobi, with
// the multilevel fine level where the cell has coarse data) of every cell,
// once per cell into NRParams::prep instead of once per (cell, basis) item in
// each item's workspace slot. One CTA per cell (grid-stride); runs after
// nr_ml_setup_kernel.
__global__ void __launch_bounds__(kNRThreads) nr_cell_prep_kernel(const NRCell *__restrict__ cells, int ncells,
                                                                  const double *__restrict__ ainv6,
                                                                  const double *__restrict__ bdiv,
                                                                  const float *__restrict__ coarse, float *prep,
                                                                  int edge_patch) {
  __shared__ NRShared sh;
  for (int cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    const NRCell C = cells[cell];
    NRGeom g;
    g.n = C.n;
    g.L = C.depth;
    nr_counts(g.n, g.NEx, g.NFx, g.NE, g.NF);
    g.N = g.NE + g.NF;
    const int n = g.n, nc = n * n * n;
    const int Np = (g.N + 63) / 64 * 64;
    float *pd = prep + C.prep_off;
    float *cf = pd + Np;
    nr_float_coefficients<kNRThreads>(ainv6 + 6 * C.coef_off, bdiv + C.coef_off, nc,
                                      1.0 / (C.h[0] * C.h[1] * C.h[2]), cf);
    nr_precond_diag<kNRThreads>(g, C, cf, pd, Np, sh, false,
                                (coarse && C.coarse_off >= 0) ? coarse + C.coarse_off + nr_ml_data_floats(C.n) : nullptr);
    if (!edge_patch || !coarse || C.coarse_off < 0) continue;  // block-uniform
    // Cell-patch factors of the edge preconditioner: per fine cell the
    // assembled edge mass on its 12 edges, M_lm = sum over the fine cells that
    // hold both edges of A^-1_pq G_pq(l4', m4') (positions in that cell), with
    // Dirichlet edges (pd = 0) replaced by identity rows, factorised M = L L^T
    // in FP64; L^-1 is stored.
    float *X = prep + C.prep_off + nr_prep_patch_offset(n);
    for (int c = threadIdx.x; c < nc; c += kNRThreads) {
      const int ci = c & (n - 1), cj = (c >> g.L) & (n - 1), ck = c >> (2 * g.L);
      int e[12], f[6];
      cell_dofs(g, c, e, f);
      double Mb[12][12];
      bool in[12];
#pragma unroll
      for (int l = 0; l < 12; ++l) {
        in[l] = pd[e[l]] > 0.0f;
#pragma unroll
        for (int m = 0; m < 12; ++m) Mb[l][m] = 0.0;
      }
      for (int l = 0; l < 12; ++l) {
        if (!in[l]) continue;
        const int p = l >> 2;
        int x, y, z;
        nr_edge_line(l, ci, cj, ck, x, y, z);
        for (int s = 0; s < 4; ++s) {  // the 4 fine cells around edge l
          const int a = s & 1, b = s >> 1;
          const int qi = p == 0 ? x : x - 1 + a;
          const int qj = p == 1 ? y : (p == 0 ? y - 1 + a : y - 1 + b);
          const int qk = p == 2 ? z : z - 1 + b;
          if (qi < 0 || qj < 0 || qk < 0 || qi >= n || qj >= n || qk >= n) continue;
          const float *ca = cf + 8 * (size_t)((qk * n + qj) * n + qi);
          const int l4 = nr_edge_pos_in(p, x, y, z, qi, qj, qk);
          for (int m = l; m < 12; ++m) {
            if (!in[m]) continue;
            const int q = m >> 2;
            int xm, ym, zm;
            nr_edge_line(m, ci, cj, ck, xm, ym, zm);
            const int m4 = nr_edge_pos_in(q, xm, ym, zm, qi, qj, qk);
            if (m4 < 0) continue;
            Mb[l][m] += (double)nr_ainv_pq(ca, p, q) * (double)sh.Gf[p][q][l4][m4];
          }
        }
      }
      for (int l = 0; l < 12; ++l) {
        for (int m = 0; m < l; ++m) Mb[l][m] = Mb[m][l];
        if (!in[l]) Mb[l][l] = 1.0;
      }
      // Cholesky M = L L^T in place (lower), then L^-1 in place, X = L^-T L^-1
      for (int j = 0; j < 12; ++j) {
        double d = Mb[j][j];
        for (int k = 0; k < j; ++k) d -= Mb[j][k] * Mb[j][k];
        d = sqrt(fmax(d, 1e-300));
        Mb[j][j] = d;
        for (int i = j + 1; i < 12; ++i) {
          double v = Mb[i][j];
          for (int k = 0; k < j; ++k) v -= Mb[i][k] * Mb[j][k];
          Mb[i][j] = v / d;
        }
      }
      for (int j = 0; j < 12; ++j) {
        Mb[j][j] = 1.0 / Mb[j][j];
        for (int i = j + 1; i < 12; ++i) {
          double v = 0.0;
          for (int k = j; k < i; ++k) v -= Mb[i][k] * Mb[k][j];
          Mb[i][j] = v / Mb[i][i];
        }
      }
      // store L^-1 (lower triangle, row by row: entries (l, 0..l)) in FP16
      // pairs; X = L^-T L^-1 is then symmetric positive definite whatever the
      // rounding of the stored entries (a Gram matrix). Dirichlet edges have
      // identity rows and columns in M and a zero v, so they add nothing.
      __half2 *X2 = reinterpret_cast<__half2 *>(X);  // word w of cell c at (w / 4 * nc + c) * 4 + w % 4
      float pend = 0.0f;
      int t = 0;
      for (int l = 0; l < 12; ++l)
        for (int m = 0; m <= l; ++m, ++t) {
          const float v = (float)Mb[l][m];
          if (t & 1) {
            const int w = t >> 1;
            X2[((size_t)(w >> 2) * nc + c) * 4 + (w & 3)] = __floats2half2_rn(pend, v);
          } else {
            pend = v;
          }
        }
      X2[((size_t)9 * nc + c) * 4 + 3] = __floats2half2_rn(0.0f, 0.0f);  // pad word 39
    }
    __syncthreads();  // sh tables are rewritten for the next cell
  }
}

}  // namespace nrimpl

// Per-precision translation units of the persistent solver (one kernel per
// variant; compiled in parallel). place: 0 = per-CTA global workspace slot,
// 1 = shared memory (for 256 threads: the split workspace), 2 = global slot
// with the apply's coefficient tiles staged by bulk copies (FP32 only);
// nedrt_solve_f32_zs: the global slot with z~ in shared memory (FP32,
// multilevel, prep).
cudaError_t nedrt_solve_f64(bool ml, int place, const NRParams &prm, size_t smem, int grid, cudaStream_t st);
cudaError_t nedrt_solve_f32(bool ml, int place, const NRParams &prm, size_t smem, int grid, cudaStream_t st);
cudaError_t nedrt_solve_f32_zs(const NRParams &prm, size_t smem, int grid, cudaStream_t st);
cudaError_t nedrt_solve_f32_256(bool ml, int place, const NRParams &prm, size_t smem, int grid, cudaStream_t st);
cudaError_t nedrt_solve_f32_256_occupancy(bool ml, int place, size_t smem, int *blocks_per_sm);

// ml: the multilevel variant (prm.coarse set); smem includes its region.
cudaError_t nedrt_solve_launch(bool fp64, bool ml, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  if (fp64) return nedrt_solve_f64(ml, prm.use_smem ? 1 : 0, prm, smem, grid, st);
  if (prm.zt_smem) return ml ? nedrt_solve_f32_zs(prm, smem, grid, st) : cudaErrorInvalidValue;
  return nedrt_solve_f32(ml, prm.use_smem ? 1 : (prm.stage ? 2 : 0), prm, smem, grid, st);
}

// Mixed precision, two 256-thread CTAs per SM: with prm.use_smem the split
// workspace (shared: preconditioner + 6 FP32 vectors; global slot: x +
// coefficients), else the whole workspace in a per-CTA global slot.
cudaError_t nedrt_solve_launch_split(bool ml, const NRParams &prm, size_t smem, int grid, cudaStream_t st) {
  return nedrt_solve_f32_256(ml, prm.use_smem ? 1 : 0, prm, smem, grid, st);
}

cudaError_t nedrt_split_occupancy(bool ml, bool use_smem, size_t smem, int *blocks_per_sm) {
  return nedrt_solve_f32_256_occupancy(ml, use_smem ? 1 : 0, smem, blocks_per_sm);
}

// Shared per-cell preconditioner + float coefficients (NRParams::prep) of
// every cell, at its prep_off; coarse: the multilevel data (null: none);
// edge_patch: also the cell-patch edge-mass inverses of multilevel cells.
cudaError_t nedrt_cell_prep_launch(const NRCell *cells, int ncells, const double *ainv6, const double *bdiv,
                                   const float *coarse, float *prep, int edge_patch, int grid, cudaStream_t st) {
  if (ncells <= 0 || grid <= 0) return cudaSuccess;
  nrimpl::nr_cell_prep_kernel<<<grid, kNRThreads, 0, st>>>(cells, ncells, ainv6, bdiv, coarse, prep, edge_patch);
  return cudaGetLastError();
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
