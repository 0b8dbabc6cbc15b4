// Implementation of the QBasis / NedRTBasis-compatible host shim (see
// msfec_basis.hpp). Batches cells, builds them with one C-ABI call, and
// answers the reference's getters from the batch results.
#include "msfec_basis.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace msfec_host {

static void check(msfec_handle *h, msfec_status s, const char *where) {
  if (s != MSFEC_SUCCESS)
    throw BasisError(s, std::string(where) + ": " + msfec_status_string(s) + ": " + (h ? msfec_last_error(h) : ""));
}

BasisBatch::BasisBatch(int device, int precision, int q1_coefficient) {
  msfec_config cfg;
  msfec_config_default(&cfg);
  cfg.device = device;
  cfg.precision = precision;
  cfg.q1_coefficient = q1_coefficient;
  check(nullptr, msfec_create(&handle_, &cfg), "msfec_create");
}

BasisBatch::~BasisBatch() { msfec_destroy(handle_); }

static msfec_cell make_cell(const CoarseCell &c, unsigned depth) {
  msfec_cell m;
  std::memset(&m, 0, sizeof(m));
  for (int d = 0; d < 3; ++d) {
    m.origin[d] = c.origin[d];
    m.size[d] = c.size[d];
  }
  m.depth = (int32_t)depth;
  return m;
}

// Fine-cell centres of a coarse cell in the ABI's lexicographic order.
template <typename F>
static void for_each_fine_centre(const msfec_cell &c, F &&f) {
  const int n = 1 << c.depth;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        f(Point{c.origin[0] + (i + 0.5) * c.size[0] / n, c.origin[1] + (j + 0.5) * c.size[1] / n,
                c.origin[2] + (k + 0.5) * c.size[2] / n});
}

// The 2x2x2 Gauss points (x fastest) of every fine cell of a coarse cell,
// fine cells in the ABI's lexicographic order.
template <typename F>
static void for_each_fine_gauss_point(const msfec_cell &c, F &&f) {
  const int n = 1 << c.depth;
  const double g = 0.5 / std::sqrt(3.0);
  const double xi[2] = {0.5 - g, 0.5 + g};
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int q = 0; q < 8; ++q)
          f(Point{c.origin[0] + (i + xi[q & 1]) * c.size[0] / n, c.origin[1] + (j + xi[(q >> 1) & 1]) * c.size[1] / n,
                  c.origin[2] + (k + xi[q >> 2]) * c.size[2] / n});
}

namespace Q {

QBasis::QBasis(const ParametersBasis &parameters, const std::string &parameter_filename, const CoarseCell &global_cell,
               const std::string &first_cell, unsigned local_subdomain, std::shared_ptr<Q1Batch> batch)
    : parameters_(parameters),
      parameter_filename_(parameter_filename),
      cell_(global_cell),
      first_cell_(first_cell),
      local_subdomain_(local_subdomain),
      batch_(std::move(batch)),
      global_weights_(8, 0.0) {}

void QBasis::run() {
  if (slot_ < 0) slot_ = batch_->enqueue(cell_, parameters_.n_refine_local);
}

const FullMatrix &QBasis::get_global_element_matrix() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "QBasis: run() was not called");
  return batch_->matrix(slot_);
}

const Vector &QBasis::get_global_element_rhs() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "QBasis: run() was not called");
  return batch_->rhs(slot_);
}

const std::string &QBasis::get_filename_global() { return parameters_.filename_global; }

void QBasis::set_global_weights(const std::vector<double> &global_weights) {
  if (global_weights.size() != 8) throw BasisError(MSFEC_ERROR_INVALID_ARGUMENT, "QBasis: 8 weights expected");
  global_weights_ = global_weights;
}

void QBasis::set_output_flag() { output_flag_ = cell_.id == first_cell_; }

double QBasis::global_solution_value(const Point &x) const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "QBasis: run() was not called");
  return batch_->evaluate(slot_, global_weights_, x);
}

Q1Batch::Q1Batch(Q1Coefficients coeff, int device, int precision)
    : coeff_(std::move(coeff)),
      gpu_(device, precision, coeff_.diffusion_tensor ? MSFEC_Q1_COEF_GAUSS : MSFEC_Q1_COEF_SCALAR) {}

int Q1Batch::enqueue(const CoarseCell &cell, unsigned depth) {
  if (built_) {  // a new cell after a build starts a new batch
    cells_.clear();
    built_ = false;
  }
  cells_.push_back(make_cell(cell, depth));
  return (int)cells_.size() - 1;
}

void Q1Batch::flush() {
  if (built_) return;
  std::vector<double> a, r;
  for (const msfec_cell &c : cells_) {
    if (coeff_.diffusion_tensor) {
      for_each_fine_gauss_point(c, [&](const Point &p) {  // a00 a11 a22 a01 a02 a12 of the symmetric part
        const std::array<double, 9> m = coeff_.diffusion_tensor(p);
        a.insert(a.end(), {m[0], m[4], m[8], 0.5 * (m[1] + m[3]), 0.5 * (m[2] + m[6]), 0.5 * (m[5] + m[7])});
      });
    }
    for_each_fine_centre(c, [&](const Point &p) {
      if (!coeff_.diffusion_tensor) a.push_back(coeff_.diffusion(p));
      if (coeff_.reaction) r.push_back(coeff_.reaction(p));
    });
  }
  const int nc = (int)cells_.size();
  std::vector<double> KH((size_t)nc * 64), FH((size_t)nc * 8);
  reports_.assign(nc, msfec_cell_report{});
  check(gpu_.handle(),
        msfec_q1_build(gpu_.handle(), nc, cells_.data(), a.data(), coeff_.reaction ? r.data() : nullptr, &coeff_.load,
                       KH.data(), FH.data(), reports_.data()),
        "msfec_q1_build");
  KH_.assign(nc, FullMatrix(8, 8));
  FH_.assign(nc, Vector(8));
  for (int c = 0; c < nc; ++c) {
    std::memcpy(KH_[c].data.data(), &KH[(size_t)c * 64], 64 * sizeof(double));
    std::memcpy(FH_[c].data.data(), &FH[(size_t)c * 8], 8 * sizeof(double));
  }
  built_ = true;
}

const FullMatrix &Q1Batch::matrix(int slot) {
  flush();
  return KH_.at(slot);
}

const Vector &Q1Batch::rhs(int slot) {
  flush();
  return FH_.at(slot);
}

double Q1Batch::evaluate(int slot, const std::vector<double> &w, const Point &x) {
  flush();
  std::vector<double> weights((size_t)cells_.size() * 8, 0.0);
  for (int v = 0; v < 8; ++v) weights[(size_t)slot * 8 + v] = w[v];
  int32_t cell_of = slot;
  double out = 0.0;
  check(gpu_.handle(), msfec_q1_eval_fine(gpu_.handle(), weights.data(), 1, &cell_of, x.data(), &out),
        "msfec_q1_eval_fine");
  return out;
}

static msfec_cell unit_cube(unsigned n_refine) {
  msfec_cell m;
  std::memset(&m, 0, sizeof(m));
  for (int d = 0; d < 3; ++d) m.size[d] = 1.0;
  m.depth = (int32_t)n_refine;
  return m;
}

QStd::QStd(const ParametersStd &parameters, Q1Coefficients coeff)
    : parameters_(parameters), coeff_(std::move(coeff)), gpu_(parameters.device, parameters.precision) {}

void QStd::run() {
  if (!coeff_.diffusion)
    throw BasisError(MSFEC_ERROR_NOT_SUPPORTED, "QStd: the standard fine solve takes a scalar diffusion callback");
  const msfec_cell dom = unit_cube(parameters_.n_refine);
  std::vector<double> a, r;
  for_each_fine_centre(dom, [&](const Point &p) {
    a.push_back(coeff_.diffusion(p));
    if (coeff_.reaction) r.push_back(coeff_.reaction(p));
  });
  const size_t n1 = ((size_t)1 << parameters_.n_refine) + 1;
  u_.assign(n1 * n1 * n1, 0.0);
  check(gpu_.handle(),
        msfec_q1_fine_solve(gpu_.handle(), &dom, a.data(), coeff_.reaction ? r.data() : nullptr, &coeff_.load,
                            u_.data(), &report_),
        "msfec_q1_fine_solve");
}

// Lattice coordinate of x along one axis: cell index in [0, n) and the local coordinate in [0, 1].
static void lattice_coord(double x, int n, int &i, double &t) {
  const double s = std::fmin(std::fmax(x, 0.0), 1.0) * n;
  i = std::min((int)s, n - 1);
  t = s - i;
}

double QStd::solution_value(const Point &x) const {
  if (u_.empty()) throw BasisError(MSFEC_ERROR_INVALID_ARGUMENT, "QStd::solution_value before run()");
  const int n = 1 << parameters_.n_refine, n1 = n + 1;
  int c[3];
  double t[3];
  for (int d = 0; d < 3; ++d) lattice_coord(x[d], n, c[d], t[d]);
  double v = 0.0;
  for (int q = 0; q < 8; ++q) {
    const int a = q & 1, b = (q >> 1) & 1, e = q >> 2;
    const double w = (a ? t[0] : 1.0 - t[0]) * (b ? t[1] : 1.0 - t[1]) * (e ? t[2] : 1.0 - t[2]);
    v += w * u_[(size_t)(c[0] + a) + (size_t)n1 * ((c[1] + b) + (size_t)n1 * (c[2] + e))];
  }
  return v;
}

}  // namespace Q

namespace NedRT {

NedRTBasis::NedRTBasis(const ParametersBasis &parameters, const std::string &parameter_filename,
                       const CoarseCell &global_cell, const std::string &first_cell, unsigned local_subdomain,
                       std::shared_ptr<NedRTBatch> batch)
    : parameters_(parameters),
      parameter_filename_(parameter_filename),
      cell_(global_cell),
      first_cell_(first_cell),
      local_subdomain_(local_subdomain),
      batch_(std::move(batch)),
      global_weights_(18, 0.0) {}

void NedRTBasis::run() {
  if (slot_ < 0) slot_ = batch_->enqueue(cell_, parameters_.n_refine_local);
}

const FullMatrix &NedRTBasis::get_global_element_matrix() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "NedRTBasis: run() was not called");
  return batch_->matrix(slot_);
}

const Vector &NedRTBasis::get_global_element_rhs() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "NedRTBasis: run() was not called");
  return batch_->rhs(slot_);
}

const std::string &NedRTBasis::get_filename_global() const { return parameters_.filename_global; }

void NedRTBasis::set_global_weights(const std::vector<double> &global_weights) {
  if (global_weights.size() != 18) throw BasisError(MSFEC_ERROR_INVALID_ARGUMENT, "NedRTBasis: 18 weights expected");
  global_weights_ = global_weights;
}

void NedRTBasis::set_output_flag() { output_flag_ = cell_.id == first_cell_; }

void NedRTBasis::global_solution(std::vector<double> &sigma, std::vector<double> &u) const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "NedRTBasis: run() was not called");
  batch_->solution(slot_, global_weights_, sigma, u);
}

NedRTBatch::NedRTBatch(NedRTCoefficients coeff, int device, int precision)
    : coeff_(std::move(coeff)), gpu_(device, precision) {}

int NedRTBatch::enqueue(const CoarseCell &cell, unsigned depth) {
  if (built_) {
    cells_.clear();
    built_ = false;
  }
  cells_.push_back(make_cell(cell, depth));
  return (int)cells_.size() - 1;
}

void NedRTBatch::flush() {
  if (built_) return;
  std::vector<double> ainv6, b;
  for (const msfec_cell &c : cells_)
    for_each_fine_centre(c, [&](const Point &p) {
      const std::array<double, 9> m = coeff_.diffusion_inverse(p);
      const double s[6] = {m[0], m[4], m[8], m[1], m[2], m[5]};
      ainv6.insert(ainv6.end(), s, s + 6);
      b.push_back(coeff_.div_weight(p));
    });
  const int nc = (int)cells_.size();
  std::vector<double> KH((size_t)nc * 324), FH((size_t)nc * 18);
  reports_.assign(nc, msfec_cell_report{});
  check(gpu_.handle(),
        msfec_nedrt_build(gpu_.handle(), nc, cells_.data(), ainv6.data(), b.data(), &coeff_.load, KH.data(),
                          FH.data(), reports_.data()),
        "msfec_nedrt_build");
  KH_.assign(nc, FullMatrix(18, 18));
  FH_.assign(nc, Vector(18));
  for (int c = 0; c < nc; ++c) {
    std::memcpy(KH_[c].data.data(), &KH[(size_t)c * 324], 324 * sizeof(double));
    std::memcpy(FH_[c].data.data(), &FH[(size_t)c * 18], 18 * sizeof(double));
  }
  basis_.resize((size_t)msfec_nedrt_basis_size(gpu_.handle()));
  check(gpu_.handle(), msfec_nedrt_get_basis(gpu_.handle(), basis_.data(), (int64_t)basis_.size()),
        "msfec_nedrt_get_basis");
  basis_off_.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) {
    const size_t n = (size_t)1 << cells_[c].depth;
    basis_off_[c + 1] = basis_off_[c] + 18 * (3 * n * (n + 1) * (n + 1) + 3 * n * n * (n + 1));
  }
  built_ = true;
}

const FullMatrix &NedRTBatch::matrix(int slot) {
  flush();
  return KH_.at(slot);
}

const Vector &NedRTBatch::rhs(int slot) {
  flush();
  return FH_.at(slot);
}

void NedRTBatch::solution(int slot, const std::vector<double> &w, std::vector<double> &sigma, std::vector<double> &u) {
  flush();
  const size_t n = (size_t)1 << cells_[slot].depth;
  const size_t NE = 3 * n * (n + 1) * (n + 1), NF = 3 * n * n * (n + 1), N = NE + NF;
  const double *phi = basis_.data() + basis_off_[slot];
  sigma.assign(NE, 0.0);
  u.assign(NF, 0.0);
  // sigma from the 12 edge bases' sigma block, u from the 6 face bases' u block
  for (int b = 0; b < 12; ++b)
    for (size_t d = 0; d < NE; ++d) sigma[d] += w[b] * phi[(size_t)b * N + d];
  for (int b = 12; b < 18; ++b)
    for (size_t d = 0; d < NF; ++d) u[d] += w[b] * phi[(size_t)b * N + NE + d];
}

NedRTStd::NedRTStd(const ParametersStd &parameters, NedRTCoefficients coeff)
    : parameters_(parameters), coeff_(std::move(coeff)), gpu_(parameters.device, parameters.precision) {}

void NedRTStd::run() {
  const msfec_cell dom = Q::unit_cube(parameters_.n_refine);
  std::vector<double> ainv6, b;
  for_each_fine_centre(dom, [&](const Point &p) {
    const std::array<double, 9> m = coeff_.diffusion_inverse(p);
    const double s6[6] = {m[0], m[4], m[8], m[1], m[2], m[5]};
    ainv6.insert(ainv6.end(), s6, s6 + 6);
    b.push_back(coeff_.div_weight(p));
  });
  const size_t n = (size_t)1 << parameters_.n_refine;
  const size_t NE = 3 * n * (n + 1) * (n + 1), NF = 3 * (n + 1) * n * n;
  std::vector<double> x(NE + NF, 0.0);
  check(gpu_.handle(),
        msfec_nedrt_fine_solve(gpu_.handle(), &dom, ainv6.data(), b.data(), &coeff_.load, x.data(), &report_),
        "msfec_nedrt_fine_solve");
  sigma_.assign(x.begin(), x.begin() + NE);
  u_.assign(x.begin() + NE, x.end());
}

Point NedRTStd::u_value(const Point &x) const {
  if (u_.empty()) throw BasisError(MSFEC_ERROR_INVALID_ARGUMENT, "NedRTStd::u_value before run()");
  const int n = 1 << parameters_.n_refine;
  const size_t Fx = (size_t)(n + 1) * n * n;
  int c[3];
  double t[3];
  for (int d = 0; d < 3; ++d) Q::lattice_coord(x[d], n, c[d], t[d]);
  const double h = 1.0 / n, area = h * h;
  // face (normal d, lattice position) -> index in the face block
  auto face = [&](int d, int i, int j, int k) -> size_t {
    if (d == 0) return (size_t)i + (size_t)(n + 1) * (j + (size_t)n * k);
    if (d == 1) return Fx + (size_t)i + (size_t)n * (j + (size_t)(n + 1) * k);
    return 2 * Fx + (size_t)i + (size_t)n * (j + (size_t)n * k);
  };
  Point v{};
  for (int d = 0; d < 3; ++d) {
    int lo[3] = {c[0], c[1], c[2]}, hi[3] = {c[0], c[1], c[2]};
    hi[d] += 1;
    // flux DoF / face area, linear along the normal (lowest-order RT)
    v[d] = ((1.0 - t[d]) * u_[face(d, lo[0], lo[1], lo[2])] + t[d] * u_[face(d, hi[0], hi[1], hi[2])]) / area;
  }
  return v;
}

}  // namespace NedRT

namespace QNed {

QNedBasis::QNedBasis(const ParametersBasis &parameters, const std::string &parameter_filename,
                     const CoarseCell &global_cell, const std::string &first_cell, unsigned local_subdomain,
                     std::shared_ptr<QNedBatch> batch)
    : parameters_(parameters),
      parameter_filename_(parameter_filename),
      cell_(global_cell),
      first_cell_(first_cell),
      local_subdomain_(local_subdomain),
      batch_(std::move(batch)),
      global_weights_(20, 0.0) {}

void QNedBasis::run() {
  if (slot_ < 0) slot_ = batch_->enqueue(cell_, parameters_.n_refine_local);
}

const FullMatrix &QNedBasis::get_global_element_matrix() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "QNedBasis: run() was not called");
  return batch_->matrix(slot_);
}

const Vector &QNedBasis::get_global_element_rhs() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "QNedBasis: run() was not called");
  return batch_->rhs(slot_);
}

const std::string &QNedBasis::get_filename_global() const { return parameters_.filename_global; }

void QNedBasis::set_global_weights(const std::vector<double> &global_weights) {
  if (global_weights.size() != 20) throw BasisError(MSFEC_ERROR_INVALID_ARGUMENT, "QNedBasis: 20 weights expected");
  global_weights_ = global_weights;
}

void QNedBasis::set_output_flag() { output_flag_ = cell_.id == first_cell_; }

void QNedBasis::global_solution(std::vector<double> &sigma, std::vector<double> &u) const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "QNedBasis: run() was not called");
  batch_->solution(slot_, global_weights_, sigma, u);
}

QNedBatch::QNedBatch(QNedCoefficients coeff, int device, int precision)
    : coeff_(std::move(coeff)), gpu_(device, precision) {}

int QNedBatch::enqueue(const CoarseCell &cell, unsigned depth) {
  if (built_) {
    cells_.clear();
    built_ = false;
  }
  cells_.push_back(make_cell(cell, depth));
  return (int)cells_.size() - 1;
}

void QNedBatch::flush() {
  if (built_) return;
  std::vector<double> a6, binv;
  for (const msfec_cell &c : cells_)
    for_each_fine_centre(c, [&](const Point &p) {
      const std::array<double, 9> m = coeff_.diffusion(p);
      const double s[6] = {m[0], m[4], m[8], m[1], m[2], m[5]};
      a6.insert(a6.end(), s, s + 6);
      binv.push_back(coeff_.inverse_b(p));
    });
  const int nc = (int)cells_.size();
  std::vector<double> KH((size_t)nc * 400), FH((size_t)nc * 20);
  reports_.assign(nc, msfec_cell_report{});
  check(gpu_.handle(),
        msfec_qned_build(gpu_.handle(), nc, cells_.data(), a6.data(), binv.data(), &coeff_.load, KH.data(),
                         FH.data(), reports_.data()),
        "msfec_qned_build");
  KH_.assign(nc, FullMatrix(20, 20));
  FH_.assign(nc, Vector(20));
  for (int c = 0; c < nc; ++c) {
    std::memcpy(KH_[c].data.data(), &KH[(size_t)c * 400], 400 * sizeof(double));
    std::memcpy(FH_[c].data.data(), &FH[(size_t)c * 20], 20 * sizeof(double));
  }
  basis_.resize((size_t)msfec_qned_basis_size(gpu_.handle()));
  check(gpu_.handle(), msfec_qned_get_basis(gpu_.handle(), basis_.data(), (int64_t)basis_.size()),
        "msfec_qned_get_basis");
  basis_off_.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) {
    const size_t n = (size_t)1 << cells_[c].depth;
    basis_off_[c + 1] = basis_off_[c] + 20 * ((n + 1) * (n + 1) * (n + 1) + 3 * n * (n + 1) * (n + 1));
  }
  built_ = true;
}

const FullMatrix &QNedBatch::matrix(int slot) {
  flush();
  return KH_.at(slot);
}

const Vector &QNedBatch::rhs(int slot) {
  flush();
  return FH_.at(slot);
}

void QNedBatch::solution(int slot, const std::vector<double> &w, std::vector<double> &sigma, std::vector<double> &u) {
  flush();
  const size_t n = (size_t)1 << cells_[slot].depth;
  const size_t NV = (n + 1) * (n + 1) * (n + 1), NE = 3 * n * (n + 1) * (n + 1), N = NV + NE;
  const double *phi = basis_.data() + basis_off_[slot];
  sigma.assign(NV, 0.0);
  u.assign(NE, 0.0);
  for (int b = 0; b < 8; ++b)
    for (size_t d = 0; d < NV; ++d) sigma[d] += w[b] * phi[(size_t)b * N + d];
  for (int b = 8; b < 20; ++b)
    for (size_t d = 0; d < NE; ++d) u[d] += w[b] * phi[(size_t)b * N + NV + d];
}

}  // namespace QNed

namespace RTDQ {

RTDQBasis::RTDQBasis(const ParametersBasis &parameters, const std::string &parameter_filename,
                     const CoarseCell &global_cell, const std::string &first_cell, unsigned local_subdomain,
                     std::shared_ptr<RTDQBatch> batch)
    : parameters_(parameters),
      parameter_filename_(parameter_filename),
      cell_(global_cell),
      first_cell_(first_cell),
      local_subdomain_(local_subdomain),
      batch_(std::move(batch)),
      global_weights_(7, 0.0) {}

void RTDQBasis::run() {
  if (slot_ < 0) slot_ = batch_->enqueue(cell_, parameters_.n_refine_local);
}

const FullMatrix &RTDQBasis::get_global_element_matrix() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "RTDQBasis: run() was not called");
  return batch_->matrix(slot_);
}

const Vector &RTDQBasis::get_global_element_rhs() const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "RTDQBasis: run() was not called");
  return batch_->rhs(slot_);
}

const std::string &RTDQBasis::get_filename_global() const { return parameters_.filename_global; }

void RTDQBasis::set_global_weights(const std::vector<double> &global_weights) {
  if (global_weights.size() != 7) throw BasisError(MSFEC_ERROR_INVALID_ARGUMENT, "RTDQBasis: 7 weights expected");
  global_weights_ = global_weights;
}

void RTDQBasis::set_output_flag() { output_flag_ = cell_.id == first_cell_; }

void RTDQBasis::global_solution(std::vector<double> &sigma, std::vector<double> &u) const {
  if (slot_ < 0) throw BasisError(MSFEC_ERROR_INVALID_STATE, "RTDQBasis: run() was not called");
  batch_->solution(slot_, global_weights_, sigma, u);
}

RTDQBatch::RTDQBatch(RTDQCoefficients coeff, int device, int precision)
    : coeff_(std::move(coeff)), gpu_(device, precision) {}

int RTDQBatch::enqueue(const CoarseCell &cell, unsigned depth) {
  if (built_) {
    cells_.clear();
    built_ = false;
  }
  cells_.push_back(make_cell(cell, depth));
  return (int)cells_.size() - 1;
}

void RTDQBatch::flush() {
  if (built_) return;
  std::vector<double> ainv6;
  for (const msfec_cell &c : cells_)
    for_each_fine_centre(c, [&](const Point &p) {
      const std::array<double, 9> m = coeff_.diffusion_inverse(p);
      const double s[6] = {m[0], m[4], m[8], m[1], m[2], m[5]};
      ainv6.insert(ainv6.end(), s, s + 6);
    });
  const int nc = (int)cells_.size();
  std::vector<double> KH((size_t)nc * 49), FH((size_t)nc * 7);
  reports_.assign(nc, msfec_cell_report{});
  check(gpu_.handle(),
        msfec_rtdq_build(gpu_.handle(), nc, cells_.data(), ainv6.data(), &coeff_.load, KH.data(), FH.data(),
                         reports_.data()),
        "msfec_rtdq_build");
  KH_.assign(nc, FullMatrix(7, 7));
  FH_.assign(nc, Vector(7));
  for (int c = 0; c < nc; ++c) {
    std::memcpy(KH_[c].data.data(), &KH[(size_t)c * 49], 49 * sizeof(double));
    std::memcpy(FH_[c].data.data(), &FH[(size_t)c * 7], 7 * sizeof(double));
  }
  basis_.resize((size_t)msfec_rtdq_basis_size(gpu_.handle()));
  check(gpu_.handle(), msfec_rtdq_get_basis(gpu_.handle(), basis_.data(), (int64_t)basis_.size()),
        "msfec_rtdq_get_basis");
  basis_off_.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) {
    const size_t n = (size_t)1 << cells_[c].depth;
    basis_off_[c + 1] = basis_off_[c] + 6 * (3 * n * n * (n + 1) + n * n * n);
  }
  built_ = true;
}

const FullMatrix &RTDQBatch::matrix(int slot) {
  flush();
  return KH_.at(slot);
}

const Vector &RTDQBatch::rhs(int slot) {
  flush();
  return FH_.at(slot);
}

void RTDQBatch::solution(int slot, const std::vector<double> &w, std::vector<double> &sigma, std::vector<double> &u) {
  flush();
  const size_t n = (size_t)1 << cells_[slot].depth;
  const size_t NF = 3 * n * n * (n + 1), NC = n * n * n, N = NF + NC;
  const double *phi = basis_.data() + basis_off_[slot];
  sigma.assign(NF, 0.0);
  for (int b = 0; b < 6; ++b)
    for (size_t d = 0; d < NF; ++d) sigma[d] += w[b] * phi[(size_t)b * N + d];
  u.assign(NC, 0.0);
  for (size_t d = 0; d < NC; ++d) u[d] = w[6] * phi[NF + d];  // basis 0's u block (1 after the build)
}

}  // namespace RTDQ
}  // namespace msfec_host
