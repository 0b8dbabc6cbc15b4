// Global coarse Q1 assembly and solve on a structured m^3 coarse grid of the
// unit cube with homogeneous Dirichlet data: the consumer of K_H / F_H.
// Restates QMultiscale::assemble_system (source/Q/q_global.cc:198-297,
// distribute_local_to_global of the element matrices) and solve_iterative
// (q_global.cc:327-363; AMG-CG there, Jacobi-CG here, FP64 on the host).
#include <cmath>
#include <vector>

extern "C" int msfec_host_q1_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol,
                                          int max_iter, int *iters) {
  if (m < 1 || !KH || !FH || !U) return 1;
  const int M1 = m + 1;
  const size_t nn = (size_t)M1 * M1 * M1;
  // 27-point structured storage: W[node][27]
  std::vector<double> W(nn * 27, 0.0), b(nn, 0.0);
  auto off27 = [](int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); };
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        const size_t c = (size_t)i + (size_t)m * (j + (size_t)m * k);
        for (int u = 0; u < 8; ++u) {
          const int ux = u & 1, uy = (u >> 1) & 1, uz = u >> 2;
          const size_t nu = (size_t)(i + ux) + M1 * ((size_t)(j + uy) + M1 * (size_t)(k + uz));
          for (int v = 0; v < 8; ++v) {
            const int vx = v & 1, vy = (v >> 1) & 1, vz = v >> 2;
            W[nu * 27 + off27(vx - ux, vy - uy, vz - uz)] += KH[c * 64 + u * 8 + v];
          }
          b[nu] += FH[c * 8 + u];
        }
      }
  auto interior = [&](int i, int j, int k) { return i > 0 && j > 0 && k > 0 && i < m && j < m && k < m; };
  auto apply = [&](const std::vector<double> &x, std::vector<double> &y) {
    for (int k = 0; k <= m; ++k)
      for (int j = 0; j <= m; ++j)
        for (int i = 0; i <= m; ++i) {
          const size_t node = (size_t)i + M1 * ((size_t)j + M1 * (size_t)k);
          double s = 0.0;
          if (interior(i, j, k))
            for (int dz = -1; dz <= 1; ++dz)
              for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx)
                  if (interior(i + dx, j + dy, k + dz))
                    s += W[node * 27 + off27(dx, dy, dz)] * x[node + dx + M1 * (dy + (ptrdiff_t)M1 * dz)];
          y[node] = s;
        }
  };
  std::vector<double> x(nn, 0.0), r(nn), z(nn), p(nn), q(nn), dinv(nn, 0.0);
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= m; ++j)
      for (int i = 0; i <= m; ++i) {
        const size_t node = (size_t)i + M1 * ((size_t)j + M1 * (size_t)k);
        const bool in = interior(i, j, k);
        r[node] = in ? b[node] : 0.0;
        dinv[node] = in ? 1.0 / W[node * 27 + 13] : 0.0;
      }
  auto dot = [&](const std::vector<double> &a, const std::vector<double> &c) {
    double s = 0.0;
    for (size_t t = 0; t < nn; ++t) s += a[t] * c[t];
    return s;
  };
  const double r0 = std::sqrt(dot(r, r));
  for (size_t t = 0; t < nn; ++t) p[t] = z[t] = dinv[t] * r[t];
  double rz = dot(r, z);
  int it = 0;
  for (; it < max_iter && std::sqrt(dot(r, r)) > rtol * r0; ++it) {
    apply(p, q);
    const double alpha = rz / dot(p, q);
    for (size_t t = 0; t < nn; ++t) {
      x[t] += alpha * p[t];
      r[t] -= alpha * q[t];
      z[t] = dinv[t] * r[t];
    }
    const double rzn = dot(r, z);
    for (size_t t = 0; t < nn; ++t) p[t] = z[t] + rzn / rz * p[t];
    rz = rzn;
  }
  for (size_t t = 0; t < nn; ++t) U[t] = x[t];
  if (iters) *iters = it;
  return std::sqrt(dot(r, r)) <= rtol * r0 || r0 == 0.0 ? 0 : 2;
}
