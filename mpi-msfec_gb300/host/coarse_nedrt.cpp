// Global coarse Ned_RT assembly and solve on a structured m^3 coarse grid of the
// unit cube: the consumer of the 18x18 K_H / 18 F_H of every cell. Restates
// NedRTMultiscale::assemble_system (source/Ned_RT/ned_rt_global.cc:191-311,
// distribute_local_to_global of the element matrices) and its solve
// (ned_rt_global.cc:313-461, a Schur complement solver there; preconditioned
// MINRES on the symmetric form here, FP64 on the host).
//
// Boundary conditions: NedRTMultiscale::setup_constraints
// (ned_rt_global.cc:165-188) holds hanging-node constraints only, its
// curl- and div-conforming boundary projections being commented out, so every
// coarse DoF is free (natural conditions; the system is nonsingular on the
// cube): msfec_host_nedrt_coarse_solve. The variant with essential conditions
// (coarse edges tangential to the boundary and coarse boundary faces zero) is
// msfec_host_nedrt_coarse_solve_essential.
//
// Coarse DoFs: edges in the fine-lattice numbering with n = m (x-edges
// i + m(j + (m+1)k), then y-, z-edges), then faces (x-faces
// i + (m+1)(j + mk), then y-, z-faces). Local order of a cell: 12 lines in
// GeometryInfo<3> order, then 6 faces. The block system [K_ee K_ef; K_fe K_ff]
// has K_fe = -K_ef^T (curl coupling), so negating the face rows gives a
// symmetric indefinite matrix, solved by MINRES with the positive diagonal
// diag(K_ee) (+) diag(K_ff - K_fe diag(K_ee)^-1 K_ef), i.e. on face f
// diag(K_ff) + sum_e K_fe^2 / K_ee (K_fe = -K_ef^T).
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <vector>

namespace {

struct Csr {
  std::vector<size_t> ptr;
  std::vector<int> col;
  std::vector<double> val;
};

// Global indices of the 18 coarse DoFs of cell (i, j, k).
void cell_map(int m, int i, int j, int k, int (&g)[18]) {
  const int Ex = m * (m + 1) * (m + 1), Fx = (m + 1) * m * m, NE = 3 * Ex;
  auto ex = [&](int a, int b, int c) { return a + m * (b + (m + 1) * c); };
  auto ey = [&](int a, int b, int c) { return Ex + a + (m + 1) * (b + m * c); };
  auto ez = [&](int a, int b, int c) { return 2 * Ex + a + (m + 1) * (b + (m + 1) * c); };
  // GeometryInfo<3> lines: (direction, position along the two other axes)
  static const int ld[12] = {1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 2, 2};
  static const int lp[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
  static const int lq[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1};
  for (int l = 0; l < 12; ++l) {
    const int p = lp[l], q = lq[l];
    g[l] = ld[l] == 0 ? ex(i, j + p, k + q) : (ld[l] == 1 ? ey(i + p, j, k + q) : ez(i + p, j + q, k));
  }
  g[12] = NE + i + (m + 1) * (j + m * k);
  g[13] = NE + (i + 1) + (m + 1) * (j + m * k);
  g[14] = NE + Fx + i + m * (j + (m + 1) * k);
  g[15] = NE + Fx + i + m * ((j + 1) + (m + 1) * k);
  g[16] = NE + 2 * Fx + i + m * (j + m * k);
  g[17] = NE + 2 * Fx + i + m * (j + m * (k + 1));
}

// Boundary flag of every coarse DoF (tangential edges on the boundary, boundary faces).
std::vector<char> boundary(int m) {
  const int Ex = m * (m + 1) * (m + 1), Fx = (m + 1) * m * m;
  std::vector<char> b(3 * Ex + 3 * Fx, 0);
  for (int t = 0; t < Ex; ++t) {
    int i = t % m, j = (t / m) % (m + 1), k = t / (m * (m + 1));  // x-edge
    b[t] = j == 0 || j == m || k == 0 || k == m;
    i = t % (m + 1), j = (t / (m + 1)) % m, k = t / ((m + 1) * m);  // y-edge
    b[Ex + t] = i == 0 || i == m || k == 0 || k == m;
    i = t % (m + 1), j = (t / (m + 1)) % (m + 1), k = t / ((m + 1) * (m + 1));  // z-edge
    b[2 * Ex + t] = i == 0 || i == m || j == 0 || j == m;
  }
  for (int t = 0; t < Fx; ++t) {
    int i = t % (m + 1);  // x-face
    b[3 * Ex + t] = i == 0 || i == m;
    const int j = (t / m) % (m + 1);  // y-face
    b[3 * Ex + Fx + t] = j == 0 || j == m;
    const int k = t / (m * m);  // z-face
    b[3 * Ex + 2 * Fx + t] = k == 0 || k == m;
  }
  return b;
}

}  // namespace

// Global coarse DoF indices of cell (i, j, k) of the m^3 grid, for the
// assembly and for set_global_weights (18 weights per cell).
extern "C" int msfec_host_nedrt_cell_dofs(int m, int cell, int *g18) {
  if (m < 1 || cell < 0 || cell >= m * m * m || !g18) return 1;
  int g[18];
  cell_map(m, cell % m, (cell / m) % m, cell / (m * m), g);
  for (int t = 0; t < 18; ++t) g18[t] = g[t];
  return 0;
}

namespace {

int nedrt_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol, int max_iter, int *iters,
                       bool essential) {
  if (m < 1 || !KH || !FH || !U) return 1;
  const int Ex = m * (m + 1) * (m + 1), Fx = (m + 1) * m * m, NE = 3 * Ex;
  const size_t N = (size_t)3 * Ex + 3 * Fx;
  const std::vector<char> bnd = essential ? boundary(m) : std::vector<char>(N, 0);
  // assemble the symmetric form (face rows negated) on interior DoFs as CSR
  std::vector<std::vector<std::pair<int, double>>> rows(N);
  std::vector<double> b(N, 0.0);
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        const size_t c = (size_t)i + (size_t)m * (j + (size_t)m * k);
        int g[18];
        cell_map(m, i, j, k, g);
        for (int r = 0; r < 18; ++r) {
          const double s = r < 12 ? 1.0 : -1.0;
          if (!bnd[g[r]]) b[g[r]] += s * FH[c * 18 + r];
          for (int q = 0; q < 18; ++q)
            if (!bnd[g[r]] && !bnd[g[q]]) rows[g[r]].push_back({g[q], s * KH[c * 324 + r * 18 + q]});
        }
      }
  Csr A;
  A.ptr.assign(N + 1, 0);
  for (size_t r = 0; r < N; ++r) {
    auto &v = rows[r];
    std::sort(v.begin(), v.end(), [](const std::pair<int, double> &x, const std::pair<int, double> &y) {
      return x.first < y.first;
    });
    for (size_t t = 0; t < v.size(); ++t) {
      if (t > 0 && v[t].first == v[t - 1].first) {
        A.val.back() += v[t].second;
      } else {
        A.col.push_back(v[t].first);
        A.val.push_back(v[t].second);
      }
    }
    A.ptr[r + 1] = A.col.size();
    std::vector<std::pair<int, double>>().swap(v);
  }
  auto apply = [&](const std::vector<double> &x, std::vector<double> &y) {
    for (size_t r = 0; r < N; ++r) {
      double s = 0.0;
      for (size_t t = A.ptr[r]; t < A.ptr[r + 1]; ++t) s += A.val[t] * x[A.col[t]];
      y[r] = s;
    }
  };
  auto diag_of = [&](size_t r) {
    for (size_t t = A.ptr[r]; t < A.ptr[r + 1]; ++t)
      if ((size_t)A.col[t] == r) return A.val[t];
    return 0.0;
  };
  // preconditioner: 1 / diag(K_ee) on edges, 1 / (diag(K_ff) + sum_e K_fe^2 / K_ee) on faces
  std::vector<double> pinv(N, 0.0);
  for (size_t r = 0; r < (size_t)NE; ++r)
    if (!bnd[r]) pinv[r] = 1.0 / std::fabs(diag_of(r));
  for (size_t r = NE; r < N; ++r) {
    if (bnd[r]) continue;
    double d = std::fabs(diag_of(r));
    for (size_t t = A.ptr[r]; t < A.ptr[r + 1]; ++t)
      if (A.col[t] < NE) d += A.val[t] * A.val[t] * pinv[A.col[t]];
    pinv[r] = d > 0.0 ? 1.0 / d : 0.0;
  }
  auto dot = [&](const std::vector<double> &x, const std::vector<double> &y) {
    double s = 0.0;
    for (size_t t = 0; t < N; ++t) s += x[t] * y[t];
    return s;
  };
  // preconditioned MINRES (Paige-Saunders recurrences, Elman-Silvester-Wathen form), x0 = 0
  std::vector<double> x(N, 0.0), v(b), vP(N, 0.0), z(N), wP(N, 0.0), wC(N, 0.0), az(N), vn(N), zn(N);
  for (size_t t = 0; t < N; ++t) z[t] = pinv[t] * v[t];
  double gam = std::sqrt(std::max(dot(z, v), 0.0));
  const double bnorm = std::sqrt(dot(b, b));
  int it = 0;
  if (gam > 0.0) {
    for (size_t t = 0; t < N; ++t) {
      v[t] /= gam;
      z[t] /= gam;
    }
    double eta = gam, cp = 1.0, cc = 1.0, sp = 0.0, ss = 0.0;
    const double eta0 = gam;
    for (; it < max_iter; ++it) {
      apply(z, az);
      const double delta = dot(az, z);
      for (size_t t = 0; t < N; ++t) vn[t] = az[t] - delta * v[t] - gam * vP[t];
      for (size_t t = 0; t < N; ++t) zn[t] = pinv[t] * vn[t];
      const double gnew = std::sqrt(std::max(dot(zn, vn), 0.0));
      const double a0 = cc * delta - cp * ss * gam, a1 = std::sqrt(a0 * a0 + gnew * gnew);
      const double a2 = ss * delta + cp * cc * gam, a3 = sp * gam;
      if (!(a1 > 0.0)) break;
      const double cn = a0 / a1, sn = gnew / a1;
      for (size_t t = 0; t < N; ++t) {
        const double wn = (z[t] - a3 * wP[t] - a2 * wC[t]) / a1;
        wP[t] = wC[t];
        wC[t] = wn;
        x[t] += cn * eta * wn;
        vP[t] = v[t];
        v[t] = gnew > 0.0 ? vn[t] / gnew : 0.0;
        z[t] = gnew > 0.0 ? zn[t] / gnew : 0.0;
      }
      eta = -sn * eta;
      gam = gnew;
      cp = cc;
      cc = cn;
      sp = ss;
      ss = sn;
      // |eta| is the preconditioned residual; confirm with the true residual
      if (std::fabs(eta) <= 0.1 * rtol * eta0 || gnew == 0.0) {
        apply(x, az);
        double rr = 0.0;
        for (size_t t = 0; t < N; ++t) rr += (b[t] - az[t]) * (b[t] - az[t]);
        if (std::sqrt(rr) <= rtol * bnorm) {
          ++it;
          break;
        }
      }
    }
  }
  apply(x, az);
  double rr = 0.0;
  for (size_t t = 0; t < N; ++t) rr += (b[t] - az[t]) * (b[t] - az[t]);
  for (size_t t = 0; t < N; ++t) U[t] = x[t];
  if (iters) *iters = it;
  return std::sqrt(rr) <= rtol * bnorm || bnorm == 0.0 ? 0 : 2;
}

}  // namespace

// The reference's NedRTMultiscale system: natural conditions, every coarse DoF
// free. U [NE + NF]; returns 0, 1 (bad arguments) or 2 (rtol not reached).
extern "C" int msfec_host_nedrt_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol,
                                             int max_iter, int *iters) {
  return nedrt_coarse_solve(m, KH, FH, U, rtol, max_iter, iters, false);
}

// Essential conditions: boundary-tangential coarse edges and boundary coarse faces fixed at 0.
extern "C" int msfec_host_nedrt_coarse_solve_essential(int m, const double *KH, const double *FH, double *U,
                                                       double rtol, int max_iter, int *iters) {
  return nedrt_coarse_solve(m, KH, FH, U, rtol, max_iter, iters, true);
}
