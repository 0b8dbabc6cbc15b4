// Ned_RT multiscale driver through the NedRTBasis-compatible shim: the flow of
// the reference's NedRTMultiscale::run (source/Ned_RT/ned_rt_global.cc) -
// basis objects per coarse cell in a std::map (ned_rt_global.cc:49-99), run(),
// 18x18 element matrices into the global coarse system, coarse solve (host
// MINRES, natural boundary conditions as in NedRTMultiscale::setup_constraints,
// ned_rt_global.cc:165-188), weights back to every cell (set_global_weights,
// ned_rt_basis.cc:1155-1181), fine sigma / u of the multiscale solution.
// Usage: example_nedrt <m> <depth>   (coarse m^3 cells of the unit cube)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

#include "msfec_basis.hpp"

extern "C" int msfec_host_nedrt_coarse_solve(int m, const double *KH, const double *FH, double *U, double rtol,
                                             int max_iter, int *iters);
extern "C" int msfec_host_nedrt_cell_dofs(int m, int cell, int *g18);

int main(int argc, char **argv) {
  const int m = argc > 1 ? std::atoi(argv[1]) : 2;
  const unsigned depth = argc > 2 ? (unsigned)std::atoi(argv[2]) : 2;
  using namespace msfec_host;
  NedRT::NedRTCoefficients coeff;
  coeff.diffusion_inverse = [](const Point &p) {
    const double a = 1.0 / (1.0 + 0.5 * std::sin(20.0 * p[0]) * std::sin(17.0 * p[1]));
    return std::array<double, 9>{a, 0.0, 0.0, 0.0, a, 0.0, 0.0, 0.0, a};
  };
  coeff.div_weight = [](const Point &p) { return 1.0 - 0.9 * std::sin(2.0 * M_PI * 14.0 * p[0]); };
  coeff.load = msfec_load{MSFEC_LOAD_VEC_TRIG, 0, {1.0, 1.0, 0.0, 0.0}};
  auto batch = std::make_shared<NedRT::NedRTBatch>(coeff);
  ParametersBasis prm;
  prm.n_refine_local = depth;
  std::map<int, NedRT::NedRTBasis> cell_basis_map;
  for (int c = 0; c < m * m * m; ++c) {
    CoarseCell cell;
    const int i = c % m, j = (c / m) % m, k = c / (m * m);
    cell.origin = {(double)i / m, (double)j / m, (double)k / m};
    cell.size = {1.0 / m, 1.0 / m, 1.0 / m};
    cell.id = std::to_string(c);
    cell_basis_map.emplace(c, NedRT::NedRTBasis(prm, "", cell, "0", 0, batch));
  }
  for (auto &kv : cell_basis_map) kv.second.run();
  const size_t nc = (size_t)m * m * m;
  std::vector<double> KH(nc * 324), FH(nc * 18);
  try {
    for (auto &kv : cell_basis_map) {
      const FullMatrix &A = kv.second.get_global_element_matrix();
      const Vector &f = kv.second.get_global_element_rhs();
      for (int t = 0; t < 324; ++t) KH[(size_t)kv.first * 324 + t] = A.data[t];
      for (int t = 0; t < 18; ++t) FH[(size_t)kv.first * 18 + t] = f.data[t];
    }
  } catch (const BasisError &e) {
    std::fprintf(stderr, "basis build failed: %s\n", e.what());
    return 1;
  }
  const size_t ncoarse = (size_t)3 * m * (m + 1) * (m + 1) + (size_t)3 * (m + 1) * m * m;
  std::vector<double> U(ncoarse);
  int iters = 0;
  if (msfec_host_nedrt_coarse_solve(m, KH.data(), FH.data(), U.data(), 1e-12, 20000, &iters) != 0) return 2;
  double u2 = 0.0, s2 = 0.0;
  for (auto &kv : cell_basis_map) {
    int g[18];
    msfec_host_nedrt_cell_dofs(m, kv.first, g);
    std::vector<double> w(18);
    for (int t = 0; t < 18; ++t) w[t] = U[g[t]];
    kv.second.set_global_weights(w);
    std::vector<double> sigma, u;
    kv.second.global_solution(sigma, u);
    for (double v : u) u2 += v * v;
    for (double v : sigma) s2 += v * v;
  }
  double unorm = 0.0;
  for (double v : U) unorm += v * v;
  std::printf("{\"cells\": %zu, \"depth\": %u, \"coarse_minres_iterations\": %d, \"KH0_1212\": %.17g, "
              "\"U_norm\": %.17g, \"fine_u_norm\": %.17g, \"fine_sigma_norm\": %.17g}\n",
              nc, depth, iters, KH[12 * 18 + 12], std::sqrt(unorm), std::sqrt(u2), std::sqrt(s2));
  return 0;
}
