// QBasis / NedRTBasis-compatible host shim over the GB300 C ABI.
//
// Keeps the public interface of the reference's basis classes so that its
// global coarse solvers consume the result unchanged:
//   Q::QBasis          include/Q/q_basis.h:77-139
//   NedRT::NedRTBasis  include/Ned_RT/ned_rt_basis.h:99-153
// and, as accuracy references, the standard fine-scale solvers Q::QStd and
// NedRT::NedRTStd (constructor + run(), solution returned instead of written).
// ctor -> run() -> get_global_element_matrix() / get_global_element_rhs()
// -> (coarse solve) -> set_global_weights().
//
// The reference computes each cell's basis inside run() (serially per MPI
// rank, source/Q/q_global.cc:83-86). Here run() only enqueues the cell into a
// shared batch; the first getter on any object of the batch launches ONE
// batched build through msfec_q1_build / msfec_nedrt_build and distributes
// K_H, F_H and the basis to every object. deal.II types are replaced by small
// stand-ins (CoarseCell for the active_cell_iterator, FullMatrix, Vector);
// coefficients come from callbacks evaluated at fine-cell centres (the
// reference evaluates its EquationData functions at Gauss points; the GB300
// path takes one value per fine cell). Errors surface as BasisError carrying
// the msfec_status (the reference throws SolverControl::NoConvergence).
#pragma once

#include <array>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/msfec_cuda.h"

namespace msfec_host {

using Point = std::array<double, 3>;

struct BasisError : std::runtime_error {
  msfec_status status;
  BasisError(msfec_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

// Stand-in for Triangulation<3>::active_cell_iterator: an axis-aligned coarse box.
struct CoarseCell {
  Point origin{};
  Point size{};
  std::string id;  // CellId::to_string() of the reference
};

// Stand-in for deal.II FullMatrix<double> / Vector<double>.
struct FullMatrix {
  unsigned rows = 0, cols = 0;
  std::vector<double> data;
  FullMatrix() = default;
  FullMatrix(unsigned r, unsigned c) : rows(r), cols(c), data((size_t)r * c, 0.0) {}
  double operator()(unsigned i, unsigned j) const { return data[(size_t)i * cols + j]; }
  double &operator()(unsigned i, unsigned j) { return data[(size_t)i * cols + j]; }
  unsigned m() const { return rows; }
  unsigned n() const { return cols; }
};

struct Vector {
  std::vector<double> data;
  Vector() = default;
  explicit Vector(unsigned n) : data(n, 0.0) {}
  double operator()(unsigned i) const { return data[i]; }
  double &operator()(unsigned i) { return data[i]; }
  unsigned size() const { return (unsigned)data.size(); }
};

// The knobs of ParametersBasis the hot path reads (q_parameters.cc:252-262,
// ned_rt_parameters.h:78-96).
struct ParametersBasis {
  unsigned n_refine_local = 3;
  bool verbose = false;
  bool use_direct_solver = false;  // accepted for compatibility; the GPU path is iterative
  int precision = MSFEC_PRECISION_MIXED;
  std::string filename_global = "multiscale_solution";
};

// The knobs of ParametersStd the standard fine-scale solvers read
// (include/Q/q_parameters.h:18-42): the unit cube refined n_refine times
// (2^n_refine fine cells per axis). Output file names are not used (the
// solution is returned instead of written as VTU).
struct ParametersStd {
  unsigned n_refine = 5;
  bool verbose = false;
  bool use_direct_solver = false;  // accepted for compatibility; the GPU path is iterative
  int precision = MSFEC_PRECISION_MIXED;
  int device = 0;
};

// One GPU handle and the pending cells of one batch.
class BasisBatch {
 public:
  explicit BasisBatch(int device = 0, int precision = MSFEC_PRECISION_MIXED,
                      int q1_coefficient = MSFEC_Q1_COEF_SCALAR);
  ~BasisBatch();
  BasisBatch(const BasisBatch &) = delete;
  BasisBatch &operator=(const BasisBatch &) = delete;
  msfec_handle *handle() const { return handle_; }

 private:
  msfec_handle *handle_ = nullptr;
};

namespace Q {

// Diffusion: either a scalar a(x) > 0, sampled at fine-cell centres, or the
// reference's tensor coefficient (Diffusion_A::value, row-major 3x3, SPD),
// evaluated like the reference's assembly at the 2x2x2 Gauss points of every
// fine cell (Diffusion_A::value_list, source/Q/q_basis.cc:218-231); the
// tensor, when set, takes precedence. Reaction r(x) >= 0 (may be empty =
// zero, the reference's ReactionRate), load f as an msfec_load.
struct Q1Coefficients {
  std::function<double(const Point &)> diffusion;
  std::function<std::array<double, 9>(const Point &)> diffusion_tensor;
  std::function<double(const Point &)> reaction;
  msfec_load load{MSFEC_LOAD_ZERO, 0, {0, 0, 0, 0}};
};

class Q1Batch;

class QBasis {
 public:
  QBasis() = delete;
  QBasis(const ParametersBasis &parameters, const std::string &parameter_filename, const CoarseCell &global_cell,
         const std::string &first_cell, unsigned local_subdomain, std::shared_ptr<Q1Batch> batch);
  QBasis(const QBasis &other) = default;

  void run();
  const FullMatrix &get_global_element_matrix() const;
  const Vector &get_global_element_rhs() const;
  const std::string &get_filename_global();
  void set_global_weights(const std::vector<double> &global_weights);
  void set_output_flag();
  // u_h(x) = sum_i w_i phi_i(x) inside this cell (replaces the VTU output of
  // output_global_solution_in_cell, q_basis.cc:484-513).
  double global_solution_value(const Point &x) const;

 private:
  friend class Q1Batch;
  ParametersBasis parameters_;
  std::string parameter_filename_;
  CoarseCell cell_;
  std::string first_cell_;
  unsigned local_subdomain_;
  std::shared_ptr<Q1Batch> batch_;
  int slot_ = -1;
  std::vector<double> global_weights_;
  bool output_flag_ = false;
};

class Q1Batch : public std::enable_shared_from_this<Q1Batch> {
 public:
  Q1Batch(Q1Coefficients coeff, int device = 0, int precision = MSFEC_PRECISION_MIXED);
  int enqueue(const CoarseCell &cell, unsigned depth);
  void flush();  // one batched build of every enqueued cell
  const FullMatrix &matrix(int slot);
  const Vector &rhs(int slot);
  double evaluate(int slot, const std::vector<double> &w, const Point &x);
  const std::vector<msfec_cell_report> &reports() const { return reports_; }

 private:
  Q1Coefficients coeff_;
  BasisBatch gpu_;
  std::vector<msfec_cell> cells_;
  std::vector<FullMatrix> KH_;
  std::vector<Vector> FH_;
  std::vector<msfec_cell_report> reports_;
  bool built_ = false;
};

// Standard fine-scale Q1 solve on the unit cube: the reference's QStd
// (include/Q/q_ref.h:84-110, source/Q/q_ref.cc:139-363) through
// msfec_q1_fine_solve, homogeneous Dirichlet data, coefficients from the same
// callbacks as the basis batch (sampled at fine-cell centres).
class QStd {
 public:
  QStd() = delete;
  QStd(const ParametersStd &parameters, Q1Coefficients coeff);
  QStd(const QStd &) = delete;
  QStd &operator=(const QStd &) = delete;

  void run();  // one GPU solve; throws BasisError
  // Nodal values, node = i + (n+1)(j + (n+1)k), n = 2^n_refine (after run()).
  const std::vector<double> &solution() const { return u_; }
  // u_h(x) by trilinear interpolation (x clamped to the unit cube).
  double solution_value(const Point &x) const;
  const msfec_cell_report &report() const { return report_; }

 private:
  ParametersStd parameters_;
  Q1Coefficients coeff_;
  BasisBatch gpu_;
  std::vector<double> u_;
  msfec_cell_report report_{};
};

}  // namespace Q

namespace NedRT {

// A^-1(x) (SPD 3x3) and B(x) > 0 at a point (the reference's
// DiffusionInverse_A and Diffusion_B), vector load as an msfec_load.
struct NedRTCoefficients {
  std::function<std::array<double, 9>(const Point &)> diffusion_inverse;
  std::function<double(const Point &)> div_weight;
  msfec_load load{MSFEC_LOAD_ZERO, 0, {0, 0, 0, 0}};
};

class NedRTBatch;

class NedRTBasis {
 public:
  NedRTBasis() = delete;
  NedRTBasis(const ParametersBasis &parameters, const std::string &parameter_filename,
             const CoarseCell &global_cell, const std::string &first_cell, unsigned local_subdomain,
             std::shared_ptr<NedRTBatch> batch);
  NedRTBasis(const NedRTBasis &other) = default;

  void run();
  const FullMatrix &get_global_element_matrix() const;
  const Vector &get_global_element_rhs() const;
  const std::string &get_filename_global() const;
  void set_global_weights(const std::vector<double> &global_weights);
  void set_output_flag();
  // Fine DoF vectors of the local multiscale solution: sigma (edge DoFs) and u
  // (face DoFs), as NedRTBasis::set_global_weights forms them (:1155-1181).
  void global_solution(std::vector<double> &sigma, std::vector<double> &u) const;

 private:
  friend class NedRTBatch;
  ParametersBasis parameters_;
  std::string parameter_filename_;
  CoarseCell cell_;
  std::string first_cell_;
  unsigned local_subdomain_;
  std::shared_ptr<NedRTBatch> batch_;
  int slot_ = -1;
  std::vector<double> global_weights_;
  bool output_flag_ = false;
};

class NedRTBatch : public std::enable_shared_from_this<NedRTBatch> {
 public:
  NedRTBatch(NedRTCoefficients coeff, int device = 0, int precision = MSFEC_PRECISION_MIXED);
  int enqueue(const CoarseCell &cell, unsigned depth);
  void flush();
  const FullMatrix &matrix(int slot);
  const Vector &rhs(int slot);
  void solution(int slot, const std::vector<double> &w, std::vector<double> &sigma, std::vector<double> &u);

 private:
  NedRTCoefficients coeff_;
  BasisBatch gpu_;
  std::vector<msfec_cell> cells_;
  std::vector<FullMatrix> KH_;
  std::vector<Vector> FH_;
  std::vector<double> basis_;
  std::vector<size_t> basis_off_;
  std::vector<msfec_cell_report> reports_;
  bool built_ = false;
};

// Standard fine-scale Ned_RT solve on the unit cube: the reference's NedRTStd
// (include/Ned_RT/ned_rt_ref.h:99-120, source/Ned_RT/ned_rt_ref.cc:110-330)
// through msfec_nedrt_fine_solve, natural boundary conditions as there.
class NedRTStd {
 public:
  NedRTStd() = delete;
  NedRTStd(const ParametersStd &parameters, NedRTCoefficients coeff);
  NedRTStd(const NedRTStd &) = delete;
  NedRTStd &operator=(const NedRTStd &) = delete;

  void run();  // one GPU solve; throws BasisError
  // sigma on the fine edges (x-, then y-, then z-edges) and u on the fine faces
  // (x-, y-, z-faces), lattice order of msfec_nedrt_fine_solve (after run()).
  const std::vector<double> &sigma() const { return sigma_; }
  const std::vector<double> &u() const { return u_; }
  // The lowest-order RT field u_h(x) (x clamped to the unit cube).
  Point u_value(const Point &x) const;
  const msfec_cell_report &report() const { return report_; }

 private:
  ParametersStd parameters_;
  NedRTCoefficients coeff_;
  BasisBatch gpu_;
  std::vector<double> sigma_, u_;
  msfec_cell_report report_{};
};

}  // namespace NedRT

namespace QNed {

// A(x) (SPD 3x3, the curl-curl weight: the reference's Diffusion_A), B^-1(x) > 0
// (the sigma mass weight: DiffusionInverse_B), vector load as an msfec_load.
struct QNedCoefficients {
  std::function<std::array<double, 9>(const Point &)> diffusion;
  std::function<double(const Point &)> inverse_b;
  msfec_load load{MSFEC_LOAD_ZERO, 0, {0, 0, 0, 0}};
};

class QNedBatch;

// QNedBasis (include/Q_Ned/q_ned_basis.h) with the same methods; the coarse
// element matrix is 20 x 20 (8 vertices, then 12 lines).
class QNedBasis {
 public:
  QNedBasis() = delete;
  QNedBasis(const ParametersBasis &parameters, const std::string &parameter_filename,
            const CoarseCell &global_cell, const std::string &first_cell, unsigned local_subdomain,
            std::shared_ptr<QNedBatch> batch);
  QNedBasis(const QNedBasis &other) = default;

  void run();
  const FullMatrix &get_global_element_matrix() const;
  const Vector &get_global_element_rhs() const;
  const std::string &get_filename_global() const;
  void set_global_weights(const std::vector<double> &global_weights);
  void set_output_flag();
  // Fine DoF vectors of the local multiscale solution: sigma (vertex DoFs) from
  // the 8 H1 bases and u (edge DoFs) from the 12 curl bases
  // (QNedBasis::set_global_weights, q_ned_basis.cc:1158-1183).
  void global_solution(std::vector<double> &sigma, std::vector<double> &u) const;

 private:
  friend class QNedBatch;
  ParametersBasis parameters_;
  std::string parameter_filename_;
  CoarseCell cell_;
  std::string first_cell_;
  unsigned local_subdomain_;
  std::shared_ptr<QNedBatch> batch_;
  int slot_ = -1;
  std::vector<double> global_weights_;
  bool output_flag_ = false;
};

class QNedBatch : public std::enable_shared_from_this<QNedBatch> {
 public:
  QNedBatch(QNedCoefficients coeff, int device = 0, int precision = MSFEC_PRECISION_MIXED);
  int enqueue(const CoarseCell &cell, unsigned depth);
  void flush();
  const FullMatrix &matrix(int slot);
  const Vector &rhs(int slot);
  void solution(int slot, const std::vector<double> &w, std::vector<double> &sigma, std::vector<double> &u);

 private:
  QNedCoefficients coeff_;
  BasisBatch gpu_;
  std::vector<msfec_cell> cells_;
  std::vector<FullMatrix> KH_;
  std::vector<Vector> FH_;
  std::vector<double> basis_;
  std::vector<size_t> basis_off_;
  std::vector<msfec_cell_report> reports_;
  bool built_ = false;
};

}  // namespace QNed

namespace RTDQ {

// A^-1(x) (SPD 3x3, the sigma mass weight: DiffusionInverse_A), scalar load as
// an msfec_load (ZERO, CONSTANT or SIN_PRODUCT); the reaction rate is 0.
struct RTDQCoefficients {
  std::function<std::array<double, 9>(const Point &)> diffusion_inverse;
  msfec_load load{MSFEC_LOAD_ZERO, 0, {0, 0, 0, 0}};
};

class RTDQBatch;

// RTDQBasis (include/RT_DQ/rt_dq_basis.h) with the same methods; the coarse
// element matrix is 7 x 7 (6 faces, then the DQ0 value).
class RTDQBasis {
 public:
  RTDQBasis() = delete;
  RTDQBasis(const ParametersBasis &parameters, const std::string &parameter_filename,
            const CoarseCell &global_cell, const std::string &first_cell, unsigned local_subdomain,
            std::shared_ptr<RTDQBatch> batch);
  RTDQBasis(const RTDQBasis &other) = default;

  void run();
  const FullMatrix &get_global_element_matrix() const;
  const Vector &get_global_element_rhs() const;
  const std::string &get_filename_global() const;
  void set_global_weights(const std::vector<double> &global_weights);
  void set_output_flag();
  // Fine DoF vectors of the local multiscale solution: sigma (face DoFs) from the
  // 6 bases, u (cell DoFs) = weight 6 times basis 0's u block, which is 1
  // (RTDQBasis::set_global_weights, rt_dq_basis.cc:1011-1036).
  void global_solution(std::vector<double> &sigma, std::vector<double> &u) const;

 private:
  friend class RTDQBatch;
  ParametersBasis parameters_;
  std::string parameter_filename_;
  CoarseCell cell_;
  std::string first_cell_;
  unsigned local_subdomain_;
  std::shared_ptr<RTDQBatch> batch_;
  int slot_ = -1;
  std::vector<double> global_weights_;
  bool output_flag_ = false;
};

class RTDQBatch : public std::enable_shared_from_this<RTDQBatch> {
 public:
  RTDQBatch(RTDQCoefficients coeff, int device = 0, int precision = MSFEC_PRECISION_MIXED);
  int enqueue(const CoarseCell &cell, unsigned depth);
  void flush();
  const FullMatrix &matrix(int slot);
  const Vector &rhs(int slot);
  void solution(int slot, const std::vector<double> &w, std::vector<double> &sigma, std::vector<double> &u);

 private:
  RTDQCoefficients coeff_;
  BasisBatch gpu_;
  std::vector<msfec_cell> cells_;
  std::vector<FullMatrix> KH_;
  std::vector<Vector> FH_;
  std::vector<double> basis_;
  std::vector<size_t> basis_off_;
  std::vector<msfec_cell_report> reports_;
  bool built_ = false;
};

}  // namespace RTDQ
}  // namespace msfec_host
