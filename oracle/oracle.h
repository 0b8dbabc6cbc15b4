/*
 * FP64 CPU oracle for the MsFEC multiscale basis construction.
 *
 * TEST INFRASTRUCTURE ONLY. This library is a plain C++ restatement of the
 * reference algorithm (konsim83/MPI-MSFEC) used to check the CUDA path and to
 * time a CPU baseline. Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs may load it. The product library
 * (libmsfec_cuda.so) never links, loads or calls it.
 *
 * Parity status: the reference needs deal.II + Trilinos + p4est + MPI, which
 * are not installed, so it cannot be built or run here. The restatement is
 * pinned by (a) the reference's only golden file
 * (test/test_fe_projection_nedelec_mpi.mpirun=1.output), reproduced exactly by
 * the Nedelec edge-DoF functional and numbering helper below, and (b)
 * known-answer tests that follow from the mathematics (trilinear functions are
 * A-harmonic for constant A, partition of unity, closed-form Q1 element
 * stiffness).
 *
 * Array conventions (identical to the product C ABI):
 *   coarse cell c: axis-aligned box origin[3*c..], size[3*c..], depth[c] = L,
 *     n = 2^L fine cells per edge.
 *   fine-cell arrays (coefficients): per coarse cell n^3 values, lexicographic
 *     (i fastest), concatenated over cells.
 *   Q1 basis Phi: per coarse cell 8 planes of (n+1)^3 nodal values, plane v =
 *     coarse vertex v (deal.II GeometryInfo<3> order v = x + 2y + 4z), node
 *     index i + (n+1)(j + (n+1)k).
 *   K_H: 8x8 row-major per cell, F_H: 8 per cell.
 */
#ifndef MSFEC_ORACLE_H
#define MSFEC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Load functions f(x). Same numbering as the product ABI's msfec_load_kind. */
enum {
  ORACLE_LOAD_ZERO = 0,
  ORACLE_LOAD_CONSTANT = 1,    /* f = p0 */
  ORACLE_LOAD_SIN_PRODUCT = 2, /* f = p0 sin(p1 pi x) sin(p1 pi y) sin(p1 pi z) */
};

/* Diffusion coefficient layout of the Q1 oracle (doubles per fine cell). */
enum {
  ORACLE_COEF_SCALAR = 0, /* 1: a, the stiffness is a K_unit */
  ORACLE_COEF_TENSOR = 1, /* 6: a00 a11 a22 a01 a02 a12 of a symmetric A */
  ORACLE_COEF_GAUSS = 2,  /* 48: those 6 at each 2x2x2 Gauss point, x fastest */
};

/* Local solver of the oracle. */
enum {
  ORACLE_SOLVER_DIRECT = 0,   /* banded Cholesky: `use direct solver basis = true` */
  ORACLE_SOLVER_CG_SSOR = 1,  /* CG + SSOR(1.6), ||r||_2 <= tol, <= max_iter */
};

/*
 * Q1 basis build for a batch of coarse cells (reference QBasis::run,
 * source/Q/q_basis.cc:518-603). a: diffusion per fine cell (> 0); r: reaction
 * per fine cell or NULL (= 0, which is the reference: ReactionRate is zero,
 * source/equation_data/eqn_coeff_R.cc:7-14). Phi / iters may be NULL.
 * iters (8 per cell) receives CG iterations (0 for the direct solver).
 * Returns 0 on success, nonzero on invalid input or non-convergence.
 */
int oracle_q1_build(int ncells, const double *origin, const double *size,
                    const int *depth, const double *a, const double *r,
                    int load_kind, const double *load_params, int solver,
                    double tol, int max_iter, double *Phi, double *KH,
                    double *FH, int *iters, int nthreads);

/* oracle_q1_build with the diffusion coefficient in layout coef_mode. */
int oracle_q1_build_coef(int ncells, const double *origin, const double *size,
                         const int *depth, int coef_mode, const double *a,
                         const double *r, int load_kind,
                         const double *load_params, int solver, double tol,
                         int max_iter, double *Phi, double *KH, double *FH,
                         int *iters, int nthreads);

/*
 * Assemble the unconstrained fine stiffness K (27-point, COO with exactly
 * 27*(n+1)^3 slots, unused slots carry value 0 and row=col=0) and load b for
 * one coarse cell (reference QBasis::assemble_system, q_basis.cc:175-257).
 */
int oracle_q1_assemble(const double *origin, const double *size, int depth,
                       const double *a, const double *r, int load_kind,
                       const double *load_params, int *rows, int *cols,
                       double *vals, double *b);
int oracle_q1_assemble_coef(const double *origin, const double *size, int depth,
                            int coef_mode, const double *a, const double *r,
                            int load_kind, const double *load_params, int *rows,
                            int *cols, double *vals, double *b);

/*
 * Nedelec lowest-order DoF values of a constant field c on the unit cube
 * refined `depth` times, in deal.II's enumeration (active cells in Morton
 * order, GeometryInfo<3> line order, first-encounter numbering). Returns the
 * number of DoFs written (3 n (n+1)^2) or -1 if out is too small.
 * This restates what the reference test
 * test/test_fe_projection_nedelec_mpi.cc:65-145 prints.
 */
int oracle_nedelec_dof_values_unit_cube(int depth, const double *c,
                                        double *out, int capacity);

#ifdef __cplusplus
}
#endif
#endif
