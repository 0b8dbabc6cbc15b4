// FP64 CPU oracle, Q1 pairing. TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Restates the reference's Q1 local basis problem (konsim83/MPI-MSFEC):
//   make_grid       source/Q/q_basis.cc:95-102   general_cell + refine_global(L)
//   setup_system    source/Q/q_basis.cc:117-170  8 Dirichlet sets = BasisQ1_i on the boundary
//   assemble_system source/Q/q_basis.cc:175-257  K = sum_e int grad psi A grad psi, b = int f psi
//   run loop        source/Q/q_basis.cc:545-565  condense + solve per coarse vertex
//   solve_direct    source/Q/q_basis.cc:304-330  (UMFPACK)  -> banded Cholesky here
//   solve_iterative source/Q/q_basis.cc:335-357  CG + SSOR(1.6), 1e-12, 1000 its
//   assemble_global_element_matrix q_basis.cc:262-300  K_H = Phi^T K Phi, F_H = Phi^T b
//   BasisQ1<3>      include/functions/basis_q1.tpp:42-152 (trilinear coarse vertex function)
//
// The coarse cells handled here are axis-aligned boxes, so the reference's
// monomial-inverse BasisQ1 reduces to the tensor-product trilinear nodal
// function and the fine Q1 mapping is affine. Coefficient modes:
//   scalar  one value a per fine cell (the seeded workloads): the 2x2x2 Gauss
//           rule of the reference integrates a K_unit exactly, closed form used;
//   tensor  a symmetric 3x3 A per fine cell (a00 a11 a22 a01 a02 a12);
//   gauss   A at each of the cell's 2x2x2 Gauss points (8 x 6 values, points
//           x fastest at 0.5 -+ 1/(2 sqrt 3) of the cell), which is what
//           Diffusion_A::value_list hands the reference's assembly
//           (source/equation_data/eqn_coeff_A.cc:162-191);
// for the last two the element matrix is the reference's quadrature loop
// itself, sum_q grad psi_i . A(x_q) grad psi_j JxW (q_basis.cc:222-231).
// The load uses the same 2x2x2 Gauss rule as the reference.
//
// Parity partially pinned: no reference test or fixture covers the basis /
// Galerkin path (the reference cannot be built here). Pinned by known answers:
// constant coefficients give the trilinear basis and the closed-form coarse
// stiffness, partition of unity, an independent scipy assembly and solve, the
// reference's CG+SSOR mode agreeing with the direct mode, and closed-form
// solutions of the fine and multiscale problems converging at O(h^2) / O(H^2).
#include "oracle.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Box {
  double o[3];
  double h[3];  // fine cell size per direction
  int n;        // fine cells per edge
};

double load_value(int kind, const double *p, double x, double y, double z) {
  switch (kind) {
    case ORACLE_LOAD_ZERO: return 0.0;
    case ORACLE_LOAD_CONSTANT: return p[0];
    case ORACLE_LOAD_SIN_PRODUCT: {
      const double w = p[1] * M_PI;
      return p[0] * std::sin(w * x) * std::sin(w * y) * std::sin(w * z);
    }
    default: return 0.0;
  }
}

// Closed-form Q1 element stiffness (unit coefficient) and mass on a box.
// Local vertex u = ux + 2 uy + 4 uz (deal.II GeometryInfo<3> order).
void element_matrices(const double h[3], double K[8][8], double M[8][8]) {
  double k1[3][2][2], m1[3][2][2];
  for (int d = 0; d < 3; ++d) {
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        k1[d][a][b] = (a == b ? 1.0 : -1.0) / h[d];
        m1[d][a][b] = h[d] * (a == b ? 1.0 / 3.0 : 1.0 / 6.0);
      }
  }
  for (int u = 0; u < 8; ++u)
    for (int v = 0; v < 8; ++v) {
      const int ux = u & 1, uy = (u >> 1) & 1, uz = u >> 2;
      const int vx = v & 1, vy = (v >> 1) & 1, vz = v >> 2;
      K[u][v] = k1[0][ux][vx] * m1[1][uy][vy] * m1[2][uz][vz] +
                m1[0][ux][vx] * k1[1][uy][vy] * m1[2][uz][vz] +
                m1[0][ux][vx] * m1[1][uy][vy] * k1[2][uz][vz];
      M[u][v] = m1[0][ux][vx] * m1[1][uy][vy] * m1[2][uz][vz];
    }
}

// Element stiffness sum_q grad psi_u(x_q) . A_q grad psi_v(x_q) JxW over the
// 2x2x2 Gauss points q (x fastest) of a box; A6 holds 6 entries per point
// (a00 a11 a22 a01 a02 a12), stride 0 for one tensor on the whole cell.
void element_matrix_tensor(const double h[3], const double *A6, int stride, double K[8][8]) {
  const double g = 0.5 / std::sqrt(3.0);
  const double qp[2] = {0.5 - g, 0.5 + g};
  const double jxw = h[0] * h[1] * h[2] / 8.0;
  for (int u = 0; u < 8; ++u)
    for (int v = 0; v < 8; ++v) K[u][v] = 0.0;
  for (int q = 0; q < 8; ++q) {
    const int qx = q & 1, qy = (q >> 1) & 1, qz = q >> 2;
    const double *a = A6 + (size_t)q * stride;
    const double A[3][3] = {{a[0], a[3], a[4]}, {a[3], a[1], a[5]}, {a[4], a[5], a[2]}};
    const double t[3] = {qp[qx], qp[qy], qp[qz]};
    double gr[8][3];
    for (int u = 0; u < 8; ++u) {
      const int b[3] = {u & 1, (u >> 1) & 1, u >> 2};
      double val[3], der[3];
      for (int d = 0; d < 3; ++d) {
        val[d] = b[d] ? t[d] : 1.0 - t[d];
        der[d] = (b[d] ? 1.0 : -1.0) / h[d];
      }
      gr[u][0] = der[0] * val[1] * val[2];
      gr[u][1] = val[0] * der[1] * val[2];
      gr[u][2] = val[0] * val[1] * der[2];
    }
    for (int u = 0; u < 8; ++u) {
      double Ag[3];
      for (int d = 0; d < 3; ++d) Ag[d] = A[d][0] * gr[u][0] + A[d][1] * gr[u][1] + A[d][2] * gr[u][2];
      for (int v = 0; v < 8; ++v) K[v][u] += (gr[v][0] * Ag[0] + gr[v][1] * Ag[1] + gr[v][2] * Ag[2]) * jxw;
    }
  }
}

inline int off27(int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); }

// Doubles of the diffusion coefficient per fine cell of each mode.
inline size_t coef_stride(int mode) { return mode == ORACLE_COEF_TENSOR ? 6 : (mode == ORACLE_COEF_GAUSS ? 48 : 1); }

// Structured assembly: W[node*27 + off27] = K(node, node+offset), b[node].
void assemble(const Box &bx, int coef_mode, const double *a, const double *r, int load_kind,
              const double *lp, std::vector<double> &W, std::vector<double> &b) {
  const int n = bx.n, N1 = n + 1;
  const size_t nn = (size_t)N1 * N1 * N1;
  W.assign(nn * 27, 0.0);
  b.assign(nn, 0.0);
  double K[8][8], M[8][8];
  element_matrices(bx.h, K, M);
  const double g = 0.5 / std::sqrt(3.0);
  const double qp[2] = {0.5 - g, 0.5 + g};
  const double jxw = bx.h[0] * bx.h[1] * bx.h[2] / 8.0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t e = (size_t)i + (size_t)n * (j + (size_t)n * k);
        const double re = r ? r[e] : 0.0;
        double Ke[8][8];
        if (coef_mode == ORACLE_COEF_SCALAR) {
          for (int u = 0; u < 8; ++u)
            for (int v = 0; v < 8; ++v) Ke[u][v] = a[e] * K[u][v];
        } else {
          element_matrix_tensor(bx.h, a + e * coef_stride(coef_mode), coef_mode == ORACLE_COEF_GAUSS ? 6 : 0, Ke);
        }
        for (int u = 0; u < 8; ++u) {
          const int ux = u & 1, uy = (u >> 1) & 1, uz = u >> 2;
          const size_t nu = (size_t)(i + ux) + N1 * ((size_t)(j + uy) + N1 * (size_t)(k + uz));
          for (int v = 0; v < 8; ++v) {
            const int vx = v & 1, vy = (v >> 1) & 1, vz = v >> 2;
            W[nu * 27 + off27(vx - ux, vy - uy, vz - uz)] += Ke[u][v] + re * M[u][v];
          }
        }
        if (load_kind != ORACLE_LOAD_ZERO) {
          for (int qz = 0; qz < 2; ++qz)
            for (int qy = 0; qy < 2; ++qy)
              for (int qx = 0; qx < 2; ++qx) {
                const double x = bx.o[0] + (i + qp[qx]) * bx.h[0];
                const double y = bx.o[1] + (j + qp[qy]) * bx.h[1];
                const double z = bx.o[2] + (k + qp[qz]) * bx.h[2];
                const double fv = load_value(load_kind, lp, x, y, z) * jxw;
                for (int u = 0; u < 8; ++u) {
                  const int ux = u & 1, uy = (u >> 1) & 1, uz = u >> 2;
                  const double psi = (ux ? qp[qx] : 1 - qp[qx]) * (uy ? qp[qy] : 1 - qp[qy]) *
                                     (uz ? qp[qz] : 1 - qp[qz]);
                  const size_t nu = (size_t)(i + ux) + N1 * ((size_t)(j + uy) + N1 * (size_t)(k + uz));
                  b[nu] += fv * psi;
                }
              }
        }
      }
}

// y = K x over the full lattice (unconstrained operator).
void apply_full(int n, const std::vector<double> &W, const double *x, double *y) {
  const int N1 = n + 1;
  for (int k = 0; k <= n; ++k)
    for (int j = 0; j <= n; ++j)
      for (int i = 0; i <= n; ++i) {
        const size_t node = (size_t)i + N1 * ((size_t)j + N1 * (size_t)k);
        double s = 0.0;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int ii = i + dx, jj = j + dy, kk = k + dz;
              if (ii < 0 || jj < 0 || kk < 0 || ii > n || jj > n || kk > n) continue;
              s += W[node * 27 + off27(dx, dy, dz)] * x[(size_t)ii + N1 * ((size_t)jj + N1 * (size_t)kk)];
            }
        y[node] = s;
      }
}

// Trilinear coarse vertex function v at a lattice node (BasisQ1<3>, basis_q1.tpp:42-152,
// which for an axis-aligned box is the tensor product of 1D hats).
inline double coarse_q1(int v, int n, int i, int j, int k) {
  const double t[3] = {(double)i / n, (double)j / n, (double)k / n};
  double s = 1.0;
  for (int d = 0; d < 3; ++d) s *= ((v >> d) & 1) ? t[d] : 1.0 - t[d];
  return s;
}

// Interior system K_II (lexicographic interior order) as 27-point rows.
struct Interior {
  int m;      // n - 1
  size_t N;   // m^3
};

inline size_t lat(int N1, int i, int j, int k) { return (size_t)i + N1 * ((size_t)j + N1 * (size_t)k); }

void interior_apply(int n, const std::vector<double> &W, const double *x, double *y) {
  const int m = n - 1, N1 = n + 1;
  for (int k = 1; k < n; ++k)
    for (int j = 1; j < n; ++j)
      for (int i = 1; i < n; ++i) {
        const size_t node = lat(N1, i, j, k);
        double s = 0.0;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int ii = i + dx, jj = j + dy, kk = k + dz;
              if (ii < 1 || jj < 1 || kk < 1 || ii > m || jj > m || kk > m) continue;
              s += W[node * 27 + off27(dx, dy, dz)] *
                   x[(size_t)(ii - 1) + m * ((size_t)(jj - 1) + m * (size_t)(kk - 1))];
            }
        y[(size_t)(i - 1) + m * ((size_t)(j - 1) + m * (size_t)(k - 1))] = s;
      }
}

// SSOR preconditioner in the form of deal.II SparseMatrix::precondition_SSOR:
// forward sweep, scaling by om(2-om) a_ii, backward sweep.
void ssor(int n, const std::vector<double> &W, double om, const double *src, double *dst) {
  const int m = n - 1, N1 = n + 1;
  const size_t N = (size_t)m * m * m;
  auto idx = [m](int i, int j, int k) { return (size_t)(i - 1) + m * ((size_t)(j - 1) + m * (size_t)(k - 1)); };
  for (int k = 1; k < n; ++k)
    for (int j = 1; j < n; ++j)
      for (int i = 1; i < n; ++i) {
        const size_t node = lat(N1, i, j, k), I = idx(i, j, k);
        double s = 0.0;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int ii = i + dx, jj = j + dy, kk = k + dz;
              if (ii < 1 || jj < 1 || kk < 1 || ii > m || jj > m || kk > m) continue;
              const size_t J = idx(ii, jj, kk);
              if (J < I) s += W[node * 27 + off27(dx, dy, dz)] * dst[J];
            }
        dst[I] = (src[I] - om * s) / W[node * 27 + 13];
      }
  for (int k = 1; k < n; ++k)
    for (int j = 1; j < n; ++j)
      for (int i = 1; i < n; ++i) dst[idx(i, j, k)] *= om * (2.0 - om) * W[lat(N1, i, j, k) * 27 + 13];
  for (int k = n - 1; k >= 1; --k)
    for (int j = n - 1; j >= 1; --j)
      for (int i = n - 1; i >= 1; --i) {
        const size_t node = lat(N1, i, j, k), I = idx(i, j, k);
        double s = 0.0;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int ii = i + dx, jj = j + dy, kk = k + dz;
              if (ii < 1 || jj < 1 || kk < 1 || ii > m || jj > m || kk > m) continue;
              const size_t J = idx(ii, jj, kk);
              if (J > I) s += W[node * 27 + off27(dx, dy, dz)] * dst[J];
            }
        dst[I] = (dst[I] - om * s) / W[node * 27 + 13];
      }
  (void)N;
}

double dot(const double *x, const double *y, size_t N) {
  double s = 0.0;
  for (size_t i = 0; i < N; ++i) s += x[i] * y[i];
  return s;
}

// deal.II SolverCG with SolverControl(max_iter, tol): convergence on ||r||_2.
int cg_ssor(int n, const std::vector<double> &W, const double *b, double *x, double tol, int max_iter,
            int *iters) {
  const int m = n - 1;
  const size_t N = (size_t)m * m * m;
  std::vector<double> r(b, b + N), z(N), p(N), v(N);
  std::fill(x, x + N, 0.0);
  double res = std::sqrt(dot(r.data(), r.data(), N));
  int it = 0;
  if (res <= tol) { *iters = 0; return 0; }
  ssor(n, W, 1.6, r.data(), z.data());
  p = z;
  double rz = dot(r.data(), z.data(), N);
  for (it = 1; it <= max_iter; ++it) {
    interior_apply(n, W, p.data(), v.data());
    const double alpha = rz / dot(p.data(), v.data(), N);
    for (size_t i = 0; i < N; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * v[i]; }
    res = std::sqrt(dot(r.data(), r.data(), N));
    if (res <= tol) { *iters = it; return 0; }
    ssor(n, W, 1.6, r.data(), z.data());
    const double rz_new = dot(r.data(), z.data(), N);
    const double beta = rz_new / rz;
    rz = rz_new;
    for (size_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
  }
  *iters = max_iter;
  return 1;
}

// Banded Cholesky of K_II (lexicographic interior order, bandwidth m^2 + m + 1).
struct BandChol {
  size_t N = 0, bw = 0;
  std::vector<double> L;  // L[I*(bw+1) + (I-J)] for J in [I-bw, I]
  int factor(int n, const std::vector<double> &W) {
    const int m = n - 1, N1 = n + 1;
    N = (size_t)m * m * m;
    bw = (size_t)m * m + m + 1;
    L.assign(N * (bw + 1), 0.0);
    auto at = [&](size_t I, size_t J) -> double & { return L[I * (bw + 1) + (I - J)]; };
    for (int k = 1; k < n; ++k)
      for (int j = 1; j < n; ++j)
        for (int i = 1; i < n; ++i) {
          const size_t node = lat(N1, i, j, k);
          const size_t I = (size_t)(i - 1) + m * ((size_t)(j - 1) + m * (size_t)(k - 1));
          for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                const int ii = i + dx, jj = j + dy, kk = k + dz;
                if (ii < 1 || jj < 1 || kk < 1 || ii > m || jj > m || kk > m) continue;
                const size_t J = (size_t)(ii - 1) + m * ((size_t)(jj - 1) + m * (size_t)(kk - 1));
                if (J <= I) at(I, J) = W[node * 27 + off27(dx, dy, dz)];
              }
        }
    for (size_t I = 0; I < N; ++I) {
      const size_t J0 = I > bw ? I - bw : 0;
      for (size_t J = J0; J <= I; ++J) {
        double s = at(I, J);
        const size_t K0 = std::max(J0, J > bw ? J - bw : (size_t)0);
        const double *li = &L[I * (bw + 1)];
        const double *lj = &L[J * (bw + 1)];
        for (size_t K = K0; K < J; ++K) s -= li[I - K] * lj[J - K];
        if (I == J) {
          if (!(s > 0.0)) return 1;
          at(I, I) = std::sqrt(s);
        } else {
          at(I, J) = s / L[J * (bw + 1)];
        }
      }
    }
    return 0;
  }
  void solve(double *x) const {
    for (size_t I = 0; I < N; ++I) {
      const size_t J0 = I > bw ? I - bw : 0;
      double s = x[I];
      for (size_t J = J0; J < I; ++J) s -= L[I * (bw + 1) + (I - J)] * x[J];
      x[I] = s / L[I * (bw + 1)];
    }
    for (size_t I = N; I-- > 0;) {
      double s = x[I];
      const size_t J1 = std::min(N - 1, I + bw);
      for (size_t J = I + 1; J <= J1; ++J) s -= L[J * (bw + 1) + (J - I)] * x[J];
      x[I] = s / L[I * (bw + 1)];
    }
  }
};

int build_cell(const Box &bx, int coef_mode, const double *a, const double *r, int load_kind, const double *lp,
               int solver, double tol, int max_iter, double *Phi, double *KH, double *FH, int *iters) {
  const int n = bx.n, N1 = n + 1, m = n - 1;
  const size_t nn = (size_t)N1 * N1 * N1, Ni = (size_t)m * m * m;
  std::vector<double> W, b;
  assemble(bx, coef_mode, a, r, load_kind, lp, W, b);
  std::vector<double> phi(8 * nn), rhs(Ni), x(Ni);
  BandChol chol;
  if (solver == ORACLE_SOLVER_DIRECT && Ni > 0 && chol.factor(n, W) != 0) return 2;
  int status = 0;
  for (int v = 0; v < 8; ++v) {
    double *ph = &phi[(size_t)v * nn];
    // Dirichlet data g_v on the boundary, zero inside (condense moves -K_IB g to the rhs).
    for (int k = 0; k <= n; ++k)
      for (int j = 0; j <= n; ++j)
        for (int i = 0; i <= n; ++i) {
          const bool bnd = i == 0 || j == 0 || k == 0 || i == n || j == n || k == n;
          ph[lat(N1, i, j, k)] = bnd ? coarse_q1(v, n, i, j, k) : 0.0;
        }
    if (Ni == 0) { if (iters) iters[v] = 0; continue; }
    // rhs_I = -(K g)_I
    std::vector<double> Kg(nn);
    apply_full(n, W, ph, Kg.data());
    for (int k = 1; k < n; ++k)
      for (int j = 1; j < n; ++j)
        for (int i = 1; i < n; ++i)
          rhs[(size_t)(i - 1) + m * ((size_t)(j - 1) + m * (size_t)(k - 1))] = -Kg[lat(N1, i, j, k)];
    int it = 0;
    if (solver == ORACLE_SOLVER_DIRECT) {
      x = rhs;
      chol.solve(x.data());
    } else {
      if (cg_ssor(n, W, rhs.data(), x.data(), tol, max_iter, &it) != 0) status = 3;
    }
    if (iters) iters[v] = it;
    for (int k = 1; k < n; ++k)
      for (int j = 1; j < n; ++j)
        for (int i = 1; i < n; ++i)
          ph[lat(N1, i, j, k)] = x[(size_t)(i - 1) + m * ((size_t)(j - 1) + m * (size_t)(k - 1))];
  }
  // Galerkin with the unconstrained K (q_basis.cc:275-297).
  std::vector<double> tmp(nn);
  for (int w = 0; w < 8; ++w) {
    apply_full(n, W, &phi[(size_t)w * nn], tmp.data());
    for (int v = 0; v < 8; ++v) KH[v * 8 + w] = dot(&phi[(size_t)v * nn], tmp.data(), nn);
  }
  for (int v = 0; v < 8; ++v) FH[v] = dot(&phi[(size_t)v * nn], b.data(), nn);
  if (Phi) std::memcpy(Phi, phi.data(), sizeof(double) * 8 * nn);
  return status;
}

}  // namespace

extern "C" int oracle_q1_build(int ncells, const double *origin, const double *size, const int *depth,
                               const double *a, const double *r, int load_kind, const double *load_params,
                               int solver, double tol, int max_iter, double *Phi, double *KH, double *FH,
                               int *iters, int nthreads) {
  return oracle_q1_build_coef(ncells, origin, size, depth, ORACLE_COEF_SCALAR, a, r, load_kind, load_params,
                              solver, tol, max_iter, Phi, KH, FH, iters, nthreads);
}

extern "C" int oracle_q1_build_coef(int ncells, const double *origin, const double *size, const int *depth,
                                    int coef_mode, const double *a, const double *r, int load_kind,
                                    const double *load_params, int solver, double tol, int max_iter, double *Phi,
                                    double *KH, double *FH, int *iters, int nthreads) {
  if (ncells < 0 || !origin || !size || !depth || !a || !KH || !FH) return 1;
  if (coef_mode < ORACLE_COEF_SCALAR || coef_mode > ORACLE_COEF_GAUSS) return 1;
  std::vector<size_t> coff(ncells + 1, 0), poff(ncells + 1, 0);
  for (int c = 0; c < ncells; ++c) {
    if (depth[c] < 1 || depth[c] > 6) return 1;
    const size_t n = (size_t)1 << depth[c];
    coff[c + 1] = coff[c] + n * n * n;
    poff[c + 1] = poff[c] + 8 * (n + 1) * (n + 1) * (n + 1);
  }
  const double zero_params[4] = {0, 0, 0, 0};
  const double *lp = load_params ? load_params : zero_params;
  int status = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : status)
#endif
  for (int c = 0; c < ncells; ++c) {
    Box bx;
    bx.n = 1 << depth[c];
    for (int d = 0; d < 3; ++d) {
      bx.o[d] = origin[3 * c + d];
      bx.h[d] = size[3 * c + d] / bx.n;
    }
    status |= build_cell(bx, coef_mode, a + coff[c] * coef_stride(coef_mode), r ? r + coff[c] : nullptr,
                         load_kind, lp, solver, tol, max_iter,
                         Phi ? Phi + poff[c] : nullptr, KH + 64 * (size_t)c, FH + 8 * (size_t)c,
                         iters ? iters + 8 * (size_t)c : nullptr);
  }
  (void)nthreads;
  return status;
}

extern "C" int oracle_q1_assemble(const double *origin, const double *size, int depth, const double *a,
                                  const double *r, int load_kind, const double *load_params, int *rows,
                                  int *cols, double *vals, double *b) {
  return oracle_q1_assemble_coef(origin, size, depth, ORACLE_COEF_SCALAR, a, r, load_kind, load_params, rows, cols,
                                 vals, b);
}

extern "C" int oracle_q1_assemble_coef(const double *origin, const double *size, int depth, int coef_mode,
                                       const double *a, const double *r, int load_kind, const double *load_params,
                                       int *rows, int *cols, double *vals, double *b) {
  if (coef_mode < ORACLE_COEF_SCALAR || coef_mode > ORACLE_COEF_GAUSS) return 1;
  if (depth < 1 || depth > 6) return 1;
  Box bx;
  bx.n = 1 << depth;
  for (int d = 0; d < 3; ++d) {
    bx.o[d] = origin[d];
    bx.h[d] = size[d] / bx.n;
  }
  const double zero_params[4] = {0, 0, 0, 0};
  std::vector<double> W, bb;
  assemble(bx, coef_mode, a, r, load_kind, load_params ? load_params : zero_params, W, bb);
  const int n = bx.n, N1 = n + 1;
  for (int k = 0; k <= n; ++k)
    for (int j = 0; j <= n; ++j)
      for (int i = 0; i <= n; ++i) {
        const size_t node = lat(N1, i, j, k);
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const size_t s = node * 27 + off27(dx, dy, dz);
              const int ii = i + dx, jj = j + dy, kk = k + dz;
              const bool in = !(ii < 0 || jj < 0 || kk < 0 || ii > n || jj > n || kk > n);
              rows[s] = in ? (int)node : 0;
              cols[s] = in ? (int)lat(N1, ii, jj, kk) : 0;
              vals[s] = in ? W[s] : 0.0;
            }
        b[node] = bb[node];
      }
  return 0;
}

// Nedelec DoF values of a constant field on the refined unit cube in deal.II
// enumeration: active cells in Morton order (refine_global creates children
// consecutively, child c = x + 2y + 4z), GeometryInfo<3> lines 0..11, a line's
// DoF numbered on first encounter; lowest-order DoF = int_e u.t ds with t the
// positive axis direction (the reference prints these in
// test/test_fe_projection_nedelec_mpi.cc:124-131).
extern "C" int oracle_nedelec_dof_values_unit_cube(int depth, const double *c, double *out, int capacity) {
  if (depth < 0 || depth > 6) return -1;
  const int n = 1 << depth;
  const long long ndof = 3LL * n * (n + 1) * (n + 1);
  if (capacity < ndof) return -1;
  static const int lo[12][3] = {{0, 0, 0}, {1, 0, 0}, {0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1},
                                {0, 0, 1}, {0, 1, 1}, {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}};
  static const int dir[12] = {1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 2, 2};
  const double h = 1.0 / n;
  std::vector<char> seen((size_t)3 * (n + 1) * (n + 1) * (n + 1), 0);
  int count = 0;
  for (long long mcode = 0; mcode < (long long)n * n * n; ++mcode) {
    int i = 0, j = 0, k = 0;
    for (int lev = depth - 1; lev >= 0; --lev) {
      const int ch = (int)((mcode >> (3 * lev)) & 7);
      i = 2 * i + (ch & 1);
      j = 2 * j + ((ch >> 1) & 1);
      k = 2 * k + ((ch >> 2) & 1);
    }
    for (int l = 0; l < 12; ++l) {
      const int x = i + lo[l][0], y = j + lo[l][1], z = k + lo[l][2];
      const size_t key = (((size_t)z * (n + 1) + y) * (n + 1) + x) * 3 + dir[l];
      if (seen[key]) continue;
      seen[key] = 1;
      out[count++] = h * c[dir[l]];
    }
  }
  return count;
}
