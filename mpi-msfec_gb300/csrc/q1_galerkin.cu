// Coarse Galerkin product of the Q1 multiscale basis (sm_103a).
//
// Restates QBasis::assemble_global_element_matrix (source/Q/q_basis.cc:262-300):
//   K_H[v][w] = phi_v^T K phi_w   with the unconstrained fine operator K,
//   F_H[v]    = phi_v^T b,        b the fine load vector of QBasis::assemble_system
//                                  (q_basis.cc:234-235, 2x2x2 Gauss points).
// y = K phi was produced by the local solver, so this is a streaming FP64
// contraction of two N x 8 panels per cell, issued on the FP64 tensor pipe
// (DMMA mma.sync.m8n8k4.f64: A = phi^T chunk, B = y chunk of 4 nodes).
#include "../../include/msfec_cuda.h"
#include "q1_common.cuh"

namespace msfec {
namespace {

constexpr int kGalThreads = 256;
constexpr int kGalWarps = kGalThreads / 32;
constexpr int kMaxN1 = 65;

__device__ __forceinline__ void dmma_m8n8k4(double &c0, double &c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// One-dimensional factor of the fine load vector for a separable load
// f = p0 g(x) g(y) g(z): beta(i) = sum over the (<= 2) fine cells next to node
// i of the 2-point Gauss sum of g * hat_i * h/2. b(node) = p0 bx(i) by(j) bz(k).
__device__ double q1_load_factor_1d(int kind, const double *p, double x0, double h, int n, int i) {
  const double g = 0.5 / sqrt(3.0);
  const double xi[2] = {0.5 - g, 0.5 + g};
  double s = 0.0;
  for (int cc = i - 1; cc <= i; ++cc) {
    if (cc < 0 || cc >= n) continue;
    for (int q = 0; q < 2; ++q) {
      const double x = x0 + (cc + xi[q]) * h;
      const double psi = (cc == i) ? 1.0 - xi[q] : xi[q];
      const double gv = kind == MSFEC_LOAD_SIN_PRODUCT ? sin(p[1] * M_PI * x) : 1.0;
      s += 0.5 * h * gv * psi;
    }
  }
  return s;
}

__global__ void __launch_bounds__(kGalThreads) q1_galerkin_kernel(const Q1Cell *__restrict__ cells,
                                                                  const double *__restrict__ phi,
                                                                  const double *__restrict__ y,
                                                                  msfec_load load, double *__restrict__ KH,
                                                                  double *__restrict__ FH) {
  __shared__ double beta[3][kMaxN1];
  __shared__ double red_k[kGalWarps][64];
  __shared__ double red_f[kGalWarps][8];
  const int c = blockIdx.x;
  const Q1Cell C = cells[c];
  const int n = C.n, N1 = n + 1;
  const int nn = N1 * N1 * N1;
  const bool has_load = load.kind == MSFEC_LOAD_SIN_PRODUCT || load.kind == MSFEC_LOAD_CONSTANT;
  for (int t = threadIdx.x; t < 3 * N1; t += kGalThreads) {
    const int d = t / N1, i = t % N1;
    beta[d][i] = has_load ? q1_load_factor_1d(load.kind, load.params, C.origin[d], C.h[d], n, i) : 0.0;
  }
  __syncthreads();
  const double *ph = phi + 8 * C.node_off;
  const double *yy = y + 8 * C.node_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t4 = lane & 3;
  const double *prow = ph + (size_t)g * nn;
  const double *yrow = yy + (size_t)g * nn;
  double c0 = 0.0, c1 = 0.0, fh = 0.0;
  for (int base = warp * 4; base < nn; base += kGalWarps * 4) {
    const int node = base + t4;
    double a = 0.0, b = 0.0;
    if (node < nn) {
      a = __ldcs(prow + node);
      b = __ldcs(yrow + node);
      const int i = node % N1, j = (node / N1) % N1, k = node / (N1 * N1);
      fh += a * (beta[0][i] * beta[1][j] * beta[2][k]);
    }
    dmma_m8n8k4(c0, c1, a, b);
  }
  fh += __shfl_xor_sync(0xffffffffu, fh, 1);
  fh += __shfl_xor_sync(0xffffffffu, fh, 2);
  red_k[warp][g * 8 + 2 * t4] = c0;
  red_k[warp][g * 8 + 2 * t4 + 1] = c1;
  if (t4 == 0) red_f[warp][g] = fh;
  __syncthreads();
  if (threadIdx.x < 64) {
    double s = 0.0;
    for (int w = 0; w < kGalWarps; ++w) s += red_k[w][threadIdx.x];
    KH[(size_t)c * 64 + threadIdx.x] = s;
  } else if (threadIdx.x < 72) {
    const int v = threadIdx.x - 64;
    double s = 0.0;
    for (int w = 0; w < kGalWarps; ++w) s += red_f[w][v];
    FH[(size_t)c * 8 + v] = has_load ? load.params[0] * s : 0.0;
  }
}

__global__ void q1_report_kernel(const Q1Stat *__restrict__ stats, int ncells, msfec_cell_report *rep) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  msfec_cell_report r;
  r.iterations = 0;
  r.refinements = 0;
  r.converged = 1;
  r.iterations_sum = 0;
  r.residual = 0.0;
  for (int v = 0; v < 8; ++v) {
    const Q1Stat s = stats[(size_t)c * 8 + v];
    r.iterations = max(r.iterations, s.iters);
    r.iterations_sum += s.iters;
    r.refinements = max(r.refinements, s.refinements);
    r.converged = r.converged && s.converged && !(s.flags & 1);
    r.residual = fmax(r.residual, s.rel_residual);
    if (!isfinite(s.rel_residual)) r.residual = s.rel_residual;
  }
  rep[c] = r;
}

// u(x) = sum_v U_v phi_v(x), phi_v trilinear on each fine cell.
__global__ void q1_eval_kernel(const Q1Cell *__restrict__ cells, const double *__restrict__ phi,
                               const double *__restrict__ weights, int npoints, const int *__restrict__ cell_of,
                               const double *__restrict__ pts, double *__restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npoints) return;
  const int c = cell_of[p];
  const Q1Cell C = cells[c];
  const int n = C.n, N1 = n + 1;
  const size_t nn = (size_t)N1 * N1 * N1;
  int f[3];
  double xi[3];
  for (int d = 0; d < 3; ++d) {
    const double t = (pts[3 * (size_t)p + d] - C.origin[d]) / C.h[d];
    int fi = (int)floor(t);
    fi = fi < 0 ? 0 : (fi > n - 1 ? n - 1 : fi);
    f[d] = fi;
    xi[d] = t - fi;
  }
  const double *ph = phi + 8 * C.node_off;
  double u = 0.0;
  for (int corner = 0; corner < 8; ++corner) {
    const int cx = corner & 1, cy = (corner >> 1) & 1, cz = corner >> 2;
    const double wgt = (cx ? xi[0] : 1.0 - xi[0]) * (cy ? xi[1] : 1.0 - xi[1]) * (cz ? xi[2] : 1.0 - xi[2]);
    const size_t node = ((size_t)(f[2] + cz) * N1 + (f[1] + cy)) * N1 + (f[0] + cx);
    double s = 0.0;
    for (int v = 0; v < 8; ++v) s += weights[(size_t)c * 8 + v] * ph[(size_t)v * nn + node];
    u += wgt * s;
  }
  out[p] = u;
}

}  // namespace

cudaError_t q1_galerkin_launch(const Q1Cell *cells, int ncells, const double *phi, const double *y,
                               const msfec_load &load, double *KH, double *FH, cudaStream_t stream) {
  if (ncells <= 0) return cudaSuccess;
  q1_galerkin_kernel<<<ncells, kGalThreads, 0, stream>>>(cells, phi, y, load, KH, FH);
  return cudaGetLastError();
}

cudaError_t q1_report_launch(const Q1Stat *stats, int ncells, msfec_cell_report *rep, cudaStream_t stream) {
  if (ncells <= 0) return cudaSuccess;
  q1_report_kernel<<<(ncells + 127) / 128, 128, 0, stream>>>(stats, ncells, rep);
  return cudaGetLastError();
}

cudaError_t q1_eval_launch(const Q1Cell *cells, const double *phi, const double *weights, int npoints,
                           const int *cell_of, const double *pts, double *out, cudaStream_t stream) {
  if (npoints <= 0) return cudaSuccess;
  q1_eval_kernel<<<(npoints + 127) / 128, 128, 0, stream>>>(cells, phi, weights, npoints, cell_of, pts, out);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Adjoint of the Q1 multiscale build (dJ/d log a per fine cell).
//
// For J(u_H(x_k)) with u_H = sum_i U_i phi_i, K_H U = F_H, coarse adjoint
// lambda = K_H^-1 dJ/dU, and per coarse cell psi_U = Phi U_e, psi_l = Phi lambda_e:
//   dJ/d log a_e = -a_e [ (mu + psi_U)_e^T Khat psi_l,e + eta_e^T Khat psi_U,e ]
// with the adjoint local problems mu = K_II^-1 b_I (load bubble) and
// eta = K_II^-1 (sum_k g_k E_k)_I (observation bubble, g_k = dJ/du_H(x_k)).
// The basis derivative terms vanish because (K phi)_I = 0 for every basis
// function (the energy-minimising property of the multiscale basis), so no
// basis sensitivities are solved for. Khat = unit-coefficient element
// stiffness; the reaction (if any) does not depend on a.
// ---------------------------------------------------------------------------
namespace {

__global__ void __launch_bounds__(kGalThreads) q1_load_rhs_kernel(const Q1Cell *__restrict__ cells, msfec_load load,
                                                                  double *__restrict__ rhs) {
  __shared__ double beta[3][kMaxN1];
  const int c = blockIdx.x;
  const Q1Cell C = cells[c];
  const int n = C.n, N1 = n + 1;
  const size_t nn = (size_t)N1 * N1 * N1;
  const bool has_load = load.kind == MSFEC_LOAD_SIN_PRODUCT || load.kind == MSFEC_LOAD_CONSTANT;
  for (int t = threadIdx.x; t < 3 * N1; t += kGalThreads) {
    const int d = t / N1, i = t % N1;
    beta[d][i] = has_load ? q1_load_factor_1d(load.kind, load.params, C.origin[d], C.h[d], n, i) : 0.0;
  }
  __syncthreads();
  double *out = rhs + 8 * C.node_off;  // plane 0: the load vector b
  for (size_t node = threadIdx.x; node < nn; node += kGalThreads) {
    const int i = (int)(node % N1), j = (int)((node / N1) % N1), k = (int)(node / ((size_t)N1 * N1));
    out[node] = has_load ? load.params[0] * beta[0][i] * beta[1][j] * beta[2][k] : 0.0;
  }
}

// plane 1: sum_k g_k E_k, E_k the trilinear weights of point k on its fine cell
__global__ void q1_point_source_kernel(const Q1Cell *__restrict__ cells, int npoints, const int *__restrict__ cell_of,
                                       const double *__restrict__ pts, const double *__restrict__ gk,
                                       double *__restrict__ rhs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npoints) return;
  const Q1Cell C = cells[cell_of[p]];
  const int n = C.n, N1 = n + 1;
  const size_t nn = (size_t)N1 * N1 * N1;
  int f[3];
  double xi[3];
  for (int d = 0; d < 3; ++d) {
    const double t = (pts[3 * (size_t)p + d] - C.origin[d]) / C.h[d];
    int fi = (int)floor(t);
    fi = fi < 0 ? 0 : (fi > n - 1 ? n - 1 : fi);
    f[d] = fi;
    xi[d] = t - fi;
  }
  double *out = rhs + 8 * C.node_off + nn;
  for (int corner = 0; corner < 8; ++corner) {
    const int cx = corner & 1, cy = (corner >> 1) & 1, cz = corner >> 2;
    const double w = (cx ? xi[0] : 1.0 - xi[0]) * (cy ? xi[1] : 1.0 - xi[1]) * (cz ? xi[2] : 1.0 - xi[2]);
    atomicAdd(out + ((size_t)(f[2] + cz) * N1 + (f[1] + cy)) * N1 + (f[0] + cx), gk[p] * w);
  }
}

__global__ void __launch_bounds__(kGalThreads) q1_gradient_kernel(const Q1Cell *__restrict__ cells,
                                                                  const double *__restrict__ a,
                                                                  const double *__restrict__ phi,
                                                                  const double *__restrict__ sol,
                                                                  const double *__restrict__ U,
                                                                  const double *__restrict__ lam,
                                                                  double *__restrict__ grad) {
  const int c = blockIdx.x;
  const Q1Cell C = cells[c];
  const int n = C.n, N1 = n + 1;
  const size_t nn = (size_t)N1 * N1 * N1;
  double kh[8];  // unit-coefficient stiffness by coordinate-difference pattern
  for (int pat = 0; pat < 8; ++pat) {
    const int dx = pat & 1, dy = (pat >> 1) & 1, dz = pat >> 2;
    const double kx = (dx ? -1.0 : 1.0) / C.h[0], ky = (dy ? -1.0 : 1.0) / C.h[1], kz = (dz ? -1.0 : 1.0) / C.h[2];
    const double mx = C.h[0] * (dx ? 1.0 / 6.0 : 1.0 / 3.0), my = C.h[1] * (dy ? 1.0 / 6.0 : 1.0 / 3.0),
                 mz = C.h[2] * (dz ? 1.0 / 6.0 : 1.0 / 3.0);
    kh[pat] = kx * my * mz + mx * ky * mz + mx * my * kz;
  }
  double u8[8], l8[8];
  for (int v = 0; v < 8; ++v) {
    u8[v] = U[(size_t)c * 8 + v];
    l8[v] = lam[(size_t)c * 8 + v];
  }
  const double *ph = phi + 8 * C.node_off;
  const double *mu = sol + 8 * C.node_off;
  const double *eta = mu + nn;
  const size_t nc = (size_t)n * n * n;
  for (size_t e = threadIdx.x; e < nc; e += kGalThreads) {
    const int i = (int)(e % n), j = (int)((e / n) % n), k = (int)(e / ((size_t)n * n));
    double pu[8], pl[8], pm[8], pe[8];
    for (int u = 0; u < 8; ++u) {
      const size_t node = ((size_t)(k + (u >> 2)) * N1 + (j + ((u >> 1) & 1))) * N1 + (i + (u & 1));
      double su = 0.0, sl = 0.0;
      for (int v = 0; v < 8; ++v) {
        const double p = ph[(size_t)v * nn + node];
        su += u8[v] * p;
        sl += l8[v] * p;
      }
      pu[u] = su;
      pl[u] = sl;
      pm[u] = mu[node] + su;
      pe[u] = eta[node];
    }
    double acc = 0.0;
    for (int u = 0; u < 8; ++u) {
      double kl = 0.0, ku = 0.0;
      for (int v = 0; v < 8; ++v) {
        kl += kh[u ^ v] * pl[v];
        ku += kh[u ^ v] * pu[v];
      }
      acc += pm[u] * kl + pe[u] * ku;
    }
    grad[C.coef_off + e] = -a[C.coef_off + e] * acc;
  }
}

}  // namespace

cudaError_t q1_adjoint_rhs_launch(const Q1Cell *cells, int ncells, const msfec_load &load, int npoints,
                                  const int *cell_of, const double *pts, const double *gk, double *rhs,
                                  cudaStream_t st) {
  if (ncells > 0) q1_load_rhs_kernel<<<ncells, kGalThreads, 0, st>>>(cells, load, rhs);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (npoints > 0) q1_point_source_kernel<<<(npoints + 127) / 128, 128, 0, st>>>(cells, npoints, cell_of, pts, gk, rhs);
  return cudaGetLastError();
}

cudaError_t q1_gradient_launch(const Q1Cell *cells, int ncells, const double *a, const double *phi, const double *sol,
                               const double *U, const double *lam, double *grad, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  q1_gradient_kernel<<<ncells, kGalThreads, 0, st>>>(cells, a, phi, sol, U, lam, grad);
  return cudaGetLastError();
}

}  // namespace msfec
