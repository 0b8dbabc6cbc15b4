// Standard fine-scale solves through the QStd / NedRTStd-compatible shim: the
// unit cube refined n_refine times, coefficients from callbacks, run(), then
// the solution vectors and point values. Prints one JSON line with checksums
// (the GPU test compares them with the C ABI called directly).
// Usage: example_std <n_refine Q1> <n_refine Ned_RT>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "msfec_basis.hpp"

namespace {

double a_of(const msfec_host::Point &p) { return 1.0 + 0.5 * std::sin(20.0 * p[0]) * std::sin(17.0 * p[1]); }

double norm(const std::vector<double> &v) {
  double s = 0.0;
  for (double x : v) s += x * x;
  return std::sqrt(s);
}

}  // namespace

int main(int argc, char **argv) {
  using namespace msfec_host;
  const unsigned rq = argc > 1 ? (unsigned)std::atoi(argv[1]) : 4;
  const unsigned rn = argc > 2 ? (unsigned)std::atoi(argv[2]) : 3;
  const Point probe{0.3, 0.55, 0.7};
  try {
    ParametersStd pq;
    pq.n_refine = rq;
    Q::Q1Coefficients qc;
    qc.diffusion = a_of;
    qc.load = msfec_load{MSFEC_LOAD_SIN_PRODUCT, 0, {1.0, 1.0, 0.0, 0.0}};
    Q::QStd q(pq, qc);
    q.run();
    ParametersStd pn;
    pn.n_refine = rn;
    NedRT::NedRTCoefficients nc;
    nc.diffusion_inverse = [](const Point &p) {
      const double a = 1.0 / a_of(p);
      return std::array<double, 9>{a, 0.0, 0.0, 0.0, a, 0.0, 0.0, 0.0, a};
    };
    nc.div_weight = [](const Point &p) { return 1.0 - 0.9 * std::sin(2.0 * M_PI * 14.0 * p[0]); };
    nc.load = msfec_load{MSFEC_LOAD_VEC_TRIG, 0, {1.0, 1.0, 0.0, 0.0}};
    NedRT::NedRTStd s(pn, nc);
    s.run();
    const Point uv = s.u_value(probe);
    std::printf("{\"q_u_norm\": %.17g, \"q_u_probe\": %.17g, \"q_iterations\": %d, \"nedrt_sigma_norm\": %.17g, "
                "\"nedrt_u_norm\": %.17g, \"nedrt_u_probe\": [%.17g, %.17g, %.17g], \"nedrt_iterations\": %d}\n",
                norm(q.solution()), q.solution_value(probe), q.report().iterations, norm(s.sigma()), norm(s.u()),
                uv[0], uv[1], uv[2], s.report().iterations);
  } catch (const BasisError &e) {
    std::fprintf(stderr, "standard solve failed: %s\n", e.what());
    return 1;
  }
  return 0;
}
