// Q1 multiscale driver through the QBasis-compatible shim: the flow of the
// reference's QMultiscale::run (source/Q/q_global.cc:520-583) -
// basis objects per coarse cell copied into a std::map (q_global.cc:38-87),
// run(), element matrices into the global coarse system, coarse solve,
// weights back to every cell, point evaluation of the multiscale solution.
// Usage: example_q1 <m> <depth> [reference]   (coarse m^3 cells of the unit cube)
// With "reference" the coefficient is the reference's own example
// (example_parameters/prm_q_test-01.prm): Diffusion_A rotated by the fixed
// Euler angles pi/3, pi/6, pi/4, diag(1 - 0.9 sin(2 pi k_d x_d)), k = 17, 16,
// 15 (source/equation_data/eqn_coeff_A.cc:25-42, 142-160), given to the shim
// as a tensor callback that it evaluates at the Gauss points, and the load
// sin(2 pi x) sin(2 pi y) sin(2 pi z).
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#include "msfec_basis.hpp"

extern "C" int msfec_host_q1_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol,
                                          int max_iter, int *iters);

int main(int argc, char **argv) {
  const int m = argc > 1 ? std::atoi(argv[1]) : 4;
  const unsigned depth = argc > 2 ? (unsigned)std::atoi(argv[2]) : 3;
  const bool reference = argc > 3 && std::string(argv[3]) == "reference";
  using namespace msfec_host;
  Q::Q1Coefficients coeff;
  if (reference) {
    const double al = M_PI / 3, be = M_PI / 6, ga = M_PI / 4;
    const double R[3][3] = {
        {std::cos(al) * std::cos(ga) - std::sin(al) * std::cos(be) * std::sin(ga),
         -std::cos(al) * std::sin(ga) - std::sin(al) * std::cos(be) * std::cos(ga), std::sin(al) * std::sin(be)},
        {std::sin(al) * std::cos(ga) + std::cos(al) * std::cos(be) * std::sin(ga),
         -std::sin(al) * std::sin(ga) + std::cos(al) * std::cos(be) * std::cos(ga), -std::cos(al) * std::sin(be)},
        {std::sin(be) * std::sin(ga), std::sin(be) * std::cos(ga), std::cos(be)}};
    std::array<std::array<double, 3>, 3> Rm;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) Rm[a][b] = R[a][b];
    coeff.diffusion_tensor = [Rm](const Point &p) {
      const int k[3] = {17, 16, 15};
      double d[3];
      for (int q = 0; q < 3; ++q) d[q] = 1.0 - 0.9 * std::sin(2.0 * M_PI * k[q] * p[q]);
      std::array<double, 9> A;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double s = 0.0;
          for (int q = 0; q < 3; ++q) s += Rm[a][q] * d[q] * Rm[b][q];
          A[3 * a + b] = s;
        }
      return A;
    };
    coeff.load = msfec_load{MSFEC_LOAD_SIN_PRODUCT, 0, {1.0, 2.0, 0.0, 0.0}};
  } else {
    coeff.diffusion = [](const Point &p) { return 1.0 + 0.5 * std::sin(20.0 * p[0]) * std::sin(17.0 * p[1]); };
    coeff.load = msfec_load{MSFEC_LOAD_SIN_PRODUCT, 0, {1.0, 1.0, 0.0, 0.0}};
  }
  auto batch = std::make_shared<Q::Q1Batch>(coeff);
  ParametersBasis prm;
  prm.n_refine_local = depth;
  std::map<int, Q::QBasis> cell_basis_map;
  for (int c = 0; c < m * m * m; ++c) {
    CoarseCell cell;
    const int i = c % m, j = (c / m) % m, k = c / (m * m);
    cell.origin = {(double)i / m, (double)j / m, (double)k / m};
    cell.size = {1.0 / m, 1.0 / m, 1.0 / m};
    cell.id = std::to_string(c);
    cell_basis_map.emplace(c, Q::QBasis(prm, "", cell, "0", 0, batch));
  }
  for (auto &kv : cell_basis_map) kv.second.run();
  std::vector<double> KH((size_t)m * m * m * 64), FH((size_t)m * m * m * 8);
  try {
    for (auto &kv : cell_basis_map) {
      const FullMatrix &A = kv.second.get_global_element_matrix();
      const Vector &f = kv.second.get_global_element_rhs();
      for (int t = 0; t < 64; ++t) KH[(size_t)kv.first * 64 + t] = A.data[t];
      for (int t = 0; t < 8; ++t) FH[(size_t)kv.first * 8 + t] = f.data[t];
    }
  } catch (const BasisError &e) {
    std::fprintf(stderr, "basis build failed: %s\n", e.what());
    return 1;
  }
  const int M1 = m + 1;
  std::vector<double> U((size_t)M1 * M1 * M1);
  int iters = 0;
  if (msfec_host_q1_coarse_solve(m, KH.data(), FH.data(), U.data(), 1e-13, 10000, &iters) != 0) return 2;
  for (auto &kv : cell_basis_map) {
    const int c = kv.first, i = c % m, j = (c / m) % m, k = c / (m * m);
    std::vector<double> w(8);
    for (int v = 0; v < 8; ++v)
      w[v] = U[(size_t)(i + (v & 1)) + M1 * ((size_t)(j + ((v >> 1) & 1)) + M1 * (size_t)(k + (v >> 2)))];
    kv.second.set_global_weights(w);
  }
  const Point centre{0.5 + 0.25 / m, 0.5 + 0.25 / m, 0.5 + 0.25 / m};
  const int cc = (int)(centre[0] * m) + m * ((int)(centre[1] * m) + m * (int)(centre[2] * m));
  const double uc = cell_basis_map.at(cc).global_solution_value(centre);
  std::printf("{\"cells\": %d, \"depth\": %u, \"coarse_cg_iterations\": %d, \"KH0_00\": %.17g, \"u_centre\": %.17g, "
              "\"KH\": [", m * m * m, depth, iters, KH[0], uc);
  for (size_t t = 0; t < KH.size(); ++t) std::printf("%s%.17g", t ? ", " : "", KH[t]);
  std::printf("]}\n");
  return 0;
}
