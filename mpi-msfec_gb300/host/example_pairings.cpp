// Q_Ned and RT_DQ element builds through the QNedBasis / RTDQBasis-compatible
// shim: basis objects per coarse cell in a std::map (the flow of the
// reference's QNedMultiscale / RTDQMultiscale initialize_and_compute_basis),
// run(), element matrices and right-hand sides, then unit weights back to every
// cell and the fine sigma / u of that combination. Prints one JSON line with
// checksums (the GPU test compares them with the C ABI called directly).
// Usage: example_pairings <m> <depth>   (coarse m^3 cells of the unit cube)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

#include "msfec_basis.hpp"

namespace {

double a_of(const msfec_host::Point &p) { return 1.0 + 0.5 * std::sin(20.0 * p[0]) * std::sin(17.0 * p[1]); }

template <typename Basis, typename Batch>
int run_pairing(const char *name, int m, unsigned depth, std::shared_ptr<Batch> batch, int nb, bool last) {
  using namespace msfec_host;
  ParametersBasis prm;
  prm.n_refine_local = depth;
  std::map<int, Basis> cell_basis_map;
  for (int c = 0; c < m * m * m; ++c) {
    CoarseCell cell;
    const int i = c % m, j = (c / m) % m, k = c / (m * m);
    cell.origin = {(double)i / m, (double)j / m, (double)k / m};
    cell.size = {1.0 / m, 1.0 / m, 1.0 / m};
    cell.id = std::to_string(c);
    cell_basis_map.emplace(c, Basis(prm, "", cell, "0", 0, batch));
  }
  for (auto &kv : cell_basis_map) kv.second.run();
  double ksum = 0.0, kabs = 0.0, fsum = 0.0, s2 = 0.0, u2 = 0.0;
  try {
    for (auto &kv : cell_basis_map) {
      const FullMatrix &A = kv.second.get_global_element_matrix();
      const Vector &f = kv.second.get_global_element_rhs();
      for (int t = 0; t < nb * nb; ++t) {
        ksum += A.data[t];
        kabs += std::fabs(A.data[t]);
      }
      for (int t = 0; t < nb; ++t) fsum += f.data[t];
      kv.second.set_global_weights(std::vector<double>(nb, 1.0));
      std::vector<double> sigma, u;
      kv.second.global_solution(sigma, u);
      for (double v : sigma) s2 += v * v;
      for (double v : u) u2 += v * v;
    }
  } catch (const BasisError &e) {
    std::fprintf(stderr, "%s basis build failed: %s\n", name, e.what());
    return 1;
  }
  std::printf("\"%s\": {\"KH_sum\": %.17g, \"KH_abs\": %.17g, \"FH_sum\": %.17g, \"sigma_norm\": %.17g, "
              "\"u_norm\": %.17g}%s",
              name, ksum, kabs, fsum, std::sqrt(s2), std::sqrt(u2), last ? "" : ", ");
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  const int m = argc > 1 ? std::atoi(argv[1]) : 2;
  const unsigned depth = argc > 2 ? (unsigned)std::atoi(argv[2]) : 2;
  using namespace msfec_host;
  QNed::QNedCoefficients qc;
  qc.diffusion = [](const Point &p) {
    const double a = a_of(p);
    return std::array<double, 9>{a, 0.0, 0.0, 0.0, a, 0.0, 0.0, 0.0, a};
  };
  qc.inverse_b = [](const Point &p) { return 1.0 / (1.0 - 0.9 * std::sin(2.0 * M_PI * 14.0 * p[0])); };
  qc.load = msfec_load{MSFEC_LOAD_VEC_TRIG, 0, {1.0, 1.0, 0.0, 0.0}};
  RTDQ::RTDQCoefficients rc;
  rc.diffusion_inverse = [](const Point &p) {
    const double a = 1.0 / a_of(p);
    return std::array<double, 9>{a, 0.0, 0.0, 0.0, a, 0.0, 0.0, 0.0, a};
  };
  rc.load = msfec_load{MSFEC_LOAD_SIN_PRODUCT, 0, {1.0, 1.0, 0.0, 0.0}};
  std::printf("{\"cells\": %d, \"depth\": %u, ", m * m * m, depth);
  if (run_pairing<QNed::QNedBasis>("qned", m, depth, std::make_shared<QNed::QNedBatch>(qc), 20, false)) return 1;
  if (run_pairing<RTDQ::RTDQBasis>("rtdq", m, depth, std::make_shared<RTDQ::RTDQBatch>(rc), 7, true)) return 1;
  std::printf("}\n");
  return 0;
}
