// Global coarse Q_Ned and RT_DQ assembly and solve on a structured m^3 coarse
// grid of the unit cube: the consumers of the 20x20 / 7x7 element matrices of
// every cell. Restates
//   QNedMultiscale::setup_constraints / assemble_system / solve
//     (source/Q_Ned/q_ned_global.cc:167-209, 213-304, 317-448): zero Dirichlet
//     data for sigma on the boundary vertices and for u x n on the boundary
//     edges, distribute_local_to_global of the element matrices;
//   RTDQMultiscale::setup_constraints / assemble_system / solve_iterative
//     (source/RT_DQ/rt_dq_global.cc:159-215, 217-319, 333-): no essential
//     condition on sigma ("pure neumann" false), the natural condition u = 0
//     on the boundary (BoundaryValues_u is zero, so no boundary term).
// Both block systems [K_pp K_ps; K_sp K_ss] have K_sp = -K_ps^T, so negating
// the secondary rows gives a symmetric indefinite matrix, solved by MINRES
// with the positive diagonal diag(K_pp) (+) diag(-K_ss + K_sp diag(K_pp)^-1 K_ps)
// (FP64 on the host; the reference uses Schur-complement solvers).
//
// Coarse DoFs. Q_Ned: vertices i + (m+1)(j + (m+1)k), then edges in the
// fine-lattice numbering with n = m (x-edges i + m(j + (m+1)k), then y-, z-);
// local order 8 vertices (GeometryInfo<3>: v = x + 2y + 4z), 12 lines in
// GeometryInfo<3> order. RT_DQ: faces (x-faces i + (m+1)(j + mk), then y-,
// z-faces; flux in the positive axis direction), then cells i + m(j + mk);
// local order 6 faces (x0 x1 y0 y1 z0 z1), then the DQ0 value.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <functional>
#include <vector>

namespace {

// Assembles the symmetric form on the free DoFs and solves it. map(c, g) gives
// the nb global DoFs of cell c; secondary[d] marks the rows that are negated.
int mixed_coarse_solve(size_t N, int ncells, int nb, const std::function<void(int, int *)> &map,
                       const std::vector<char> &fixed, const std::vector<char> &secondary, const double *KH,
                       const double *FH, double *U, double rtol, int max_iter, int *iters) {
  std::vector<std::vector<std::pair<int, double>>> rows(N);
  std::vector<double> b(N, 0.0);
  std::vector<int> g(nb);
  for (int c = 0; c < ncells; ++c) {
    map(c, g.data());
    for (int r = 0; r < nb; ++r) {
      if (fixed[g[r]]) continue;
      const double s = secondary[g[r]] ? -1.0 : 1.0;
      b[g[r]] += s * FH[(size_t)c * nb + r];
      for (int q = 0; q < nb; ++q)
        if (!fixed[g[q]]) rows[g[r]].push_back({g[q], s * KH[((size_t)c * nb + r) * nb + q]});
    }
  }
  std::vector<size_t> ptr(N + 1, 0);
  std::vector<int> col;
  std::vector<double> val;
  for (size_t r = 0; r < N; ++r) {
    auto &v = rows[r];
    std::sort(v.begin(), v.end(), [](const std::pair<int, double> &x, const std::pair<int, double> &y) {
      return x.first < y.first;
    });
    for (size_t t = 0; t < v.size(); ++t) {
      if (t > 0 && v[t].first == v[t - 1].first) {
        val.back() += v[t].second;
      } else {
        col.push_back(v[t].first);
        val.push_back(v[t].second);
      }
    }
    ptr[r + 1] = col.size();
    std::vector<std::pair<int, double>>().swap(v);
  }
  auto apply = [&](const std::vector<double> &x, std::vector<double> &y) {
    for (size_t r = 0; r < N; ++r) {
      double s = 0.0;
      for (size_t t = ptr[r]; t < ptr[r + 1]; ++t) s += val[t] * x[col[t]];
      y[r] = s;
    }
  };
  auto diag_of = [&](size_t r) {
    for (size_t t = ptr[r]; t < ptr[r + 1]; ++t)
      if ((size_t)col[t] == r) return val[t];
    return 0.0;
  };
  std::vector<double> pinv(N, 0.0);
  for (size_t r = 0; r < N; ++r)
    if (!fixed[r] && !secondary[r]) {
      const double d = std::fabs(diag_of(r));
      pinv[r] = d > 0.0 ? 1.0 / d : 0.0;
    }
  for (size_t r = 0; r < N; ++r) {
    if (fixed[r] || !secondary[r]) continue;
    double d = std::fabs(diag_of(r));
    for (size_t t = ptr[r]; t < ptr[r + 1]; ++t)
      if (!secondary[col[t]]) d += val[t] * val[t] * pinv[col[t]];
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
      if (std::fabs(eta) <= 0.1 * rtol * eta0 || gnew == 0.0) {  // confirm with the true residual
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

// Q_Ned: global DoFs of cell (i, j, k): 8 vertices, then 12 lines (GeometryInfo<3> order).
void qned_map(int m, int i, int j, int k, int *g) {
  const int N1 = m + 1, NV = N1 * N1 * N1, Ex = m * N1 * N1;
  for (int v = 0; v < 8; ++v) g[v] = (i + (v & 1)) + N1 * ((j + ((v >> 1) & 1)) + N1 * (k + (v >> 2)));
  auto ex = [&](int a, int b, int c) { return NV + a + m * (b + N1 * c); };
  auto ey = [&](int a, int b, int c) { return NV + Ex + a + N1 * (b + m * c); };
  auto ez = [&](int a, int b, int c) { return NV + 2 * Ex + a + N1 * (b + N1 * c); };
  static const int ld[12] = {1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 2, 2};
  static const int lp[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
  static const int lq[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1};
  for (int l = 0; l < 12; ++l) {
    const int p = lp[l], q = lq[l];
    g[8 + l] = ld[l] == 0 ? ex(i, j + p, k + q) : (ld[l] == 1 ? ey(i + p, j, k + q) : ez(i + p, j + q, k));
  }
}

// RT_DQ: global DoFs of cell (i, j, k): 6 faces, then the cell.
void rtdq_map(int m, int i, int j, int k, int *g) {
  const int Fx = (m + 1) * m * m, NF = 3 * Fx;
  g[0] = i + (m + 1) * (j + m * k);
  g[1] = (i + 1) + (m + 1) * (j + m * k);
  g[2] = Fx + i + m * (j + (m + 1) * k);
  g[3] = Fx + i + m * ((j + 1) + (m + 1) * k);
  g[4] = 2 * Fx + i + m * (j + m * k);
  g[5] = 2 * Fx + i + m * (j + m * (k + 1));
  g[6] = NF + i + m * (j + m * k);
}

}  // namespace

// Global coarse DoF indices of cell `cell` of the m^3 grid (20 per cell), for the
// assembly and for set_global_weights.
extern "C" int msfec_host_qned_cell_dofs(int m, int cell, int *g20) {
  if (m < 1 || cell < 0 || cell >= m * m * m || !g20) return 1;
  qned_map(m, cell % m, (cell / m) % m, cell / (m * m), g20);
  return 0;
}

// Solves the Q_Ned coarse system; U has (m+1)^3 + 3 m (m+1)^2 entries (0 on the
// fixed boundary DoFs). Returns 0, 1 (bad arguments) or 2 (rtol not reached).
extern "C" int msfec_host_qned_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol,
                                            int max_iter, int *iters) {
  if (m < 1 || !KH || !FH || !U) return 1;
  const int N1 = m + 1, NV = N1 * N1 * N1, Ex = m * N1 * N1;
  const size_t N = (size_t)NV + 3 * Ex;
  std::vector<char> fixed(N, 0), secondary(N, 0);
  for (int t = 0; t < NV; ++t) {
    const int i = t % N1, j = (t / N1) % N1, k = t / (N1 * N1);
    fixed[t] = i == 0 || i == m || j == 0 || j == m || k == 0 || k == m;
  }
  for (int t = 0; t < Ex; ++t) {
    int i = t % m, j = (t / m) % N1, k = t / (m * N1);  // x-edge
    fixed[NV + t] = j == 0 || j == m || k == 0 || k == m;
    i = t % N1, j = (t / N1) % m, k = t / (N1 * m);  // y-edge
    fixed[NV + Ex + t] = i == 0 || i == m || k == 0 || k == m;
    i = t % N1, j = (t / N1) % N1, k = t / (N1 * N1);  // z-edge
    fixed[NV + 2 * Ex + t] = i == 0 || i == m || j == 0 || j == m;
  }
  for (size_t t = NV; t < N; ++t) secondary[t] = 1;
  auto map = [m](int c, int *g) { qned_map(m, c % m, (c / m) % m, c / (m * m), g); };
  return mixed_coarse_solve(N, m * m * m, 20, map, fixed, secondary, KH, FH, U, rtol, max_iter, iters);
}

// Global coarse DoF indices of cell `cell` of the m^3 grid (7 per cell).
extern "C" int msfec_host_rtdq_cell_dofs(int m, int cell, int *g7) {
  if (m < 1 || cell < 0 || cell >= m * m * m || !g7) return 1;
  rtdq_map(m, cell % m, (cell / m) % m, cell / (m * m), g7);
  return 0;
}

// Solves the RT_DQ coarse system; U has 3 m^2 (m+1) + m^3 entries.
extern "C" int msfec_host_rtdq_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol,
                                            int max_iter, int *iters) {
  if (m < 1 || !KH || !FH || !U) return 1;
  const int NF = 3 * (m + 1) * m * m;
  const size_t N = (size_t)NF + (size_t)m * m * m;
  std::vector<char> fixed(N, 0), secondary(N, 0);
  for (size_t t = NF; t < N; ++t) secondary[t] = 1;
  auto map = [m](int c, int *g) { rtdq_map(m, c % m, (c / m) % m, c / (m * m), g); };
  return mixed_coarse_solve(N, m * m * m, 7, map, fixed, secondary, KH, FH, U, rtol, max_iter, iters);
}
