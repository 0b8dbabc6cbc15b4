/*
 * msfec_cuda.h - C ABI of the GB300 (sm_103a) MsFEC multiscale basis builder.
 *
 * One call builds, for a batch of coarse hexahedral cells, the multiscale
 * basis (all coarse-basis right-hand sides of every cell solved at once) and
 * the coarse Galerkin element matrix K_H = Phi^T K Phi and load F_H = Phi^T f.
 * It replaces the per-cell basis objects of konsim83/MPI-MSFEC:
 *
 *   Q::QBasis            include/Q/q_basis.h:62-305, source/Q/q_basis.cc
 *   NedRT::NedRTBasis    include/Ned_RT/ned_rt_basis.h:81-348,
 *                        source/Ned_RT/ned_rt_basis.cc
 *
 * Conventions (identical for every entry point):
 *  - Coarse cells are axis-aligned boxes msfec_cell{origin, size, depth};
 *    the local problem lives on the depth-times uniformly refined box
 *    (reference QBasis::make_grid, q_basis.cc:95-102: general_cell +
 *    refine_global(n_refine_local)), n = 2^depth fine cells per edge.
 *  - Fine-cell arrays: per coarse cell n^3 values, lexicographic (x fastest),
 *    concatenated over the batch in batch order.
 *  - Coarse numbering follows deal.II GeometryInfo<3>: vertex v = x + 2y + 4z;
 *    K_H is row-major [cell][test][trial].
 *  - Q1 basis Phi: per cell 8 planes (one per coarse vertex) of (n+1)^3 nodal
 *    values, node = i + (n+1)(j + (n+1)k).
 *  - Every call returns msfec_status; nothing aborts or traps. Per-cell
 *    convergence is reported in msfec_cell_report.
 *  - A handle owns its device buffers and one CUDA stream; it is not
 *    thread-safe. Host-buffer entry points are synchronous; *_device entry
 *    points are asynchronous on the handle's stream.
 */
#ifndef MSFEC_CUDA_H
#define MSFEC_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum msfec_status {
  MSFEC_SUCCESS = 0,
  MSFEC_ERROR_INVALID_ARGUMENT = 1,
  MSFEC_ERROR_CUDA = 2,
  MSFEC_ERROR_OUT_OF_MEMORY = 3,
  /* A local solve missed its tolerance; outputs are written, see reports.
     Replaces deal.II's SolverControl::NoConvergence (q_basis.cc:337). */
  MSFEC_ERROR_NOT_CONVERGED = 4,
  MSFEC_ERROR_NOT_SUPPORTED = 5,
  /* NaN/Inf or non-positive coefficient in the input. */
  MSFEC_ERROR_NUMERICAL = 6,
  /* Call order violated (e.g. basis requested before any build). */
  MSFEC_ERROR_INVALID_STATE = 7
} msfec_status;

typedef enum msfec_precision {
  /* Plain FP64 PCG for every local solve. */
  MSFEC_PRECISION_FP64 = 0,
  /* FP32 PCG inner solves wrapped in FP64 iterative refinement. */
  MSFEC_PRECISION_MIXED = 1
} msfec_precision;

/* Load f(x) of the local problems; evaluated on the device at the 2x2x2
   Gauss points of every fine cell, like the reference's RightHandSideParsed
   (source/equation_data/eqn_rhs.cc:57-106) at QGauss<3>(2) points. */
typedef enum msfec_load_kind {
  MSFEC_LOAD_ZERO = 0,
  MSFEC_LOAD_CONSTANT = 1,    /* f = p0 */
  MSFEC_LOAD_SIN_PRODUCT = 2, /* f = p0 sin(p1 pi x) sin(p1 pi y) sin(p1 pi z) */
  /* vector load of the mixed (Ned_RT) problem, w = p1 pi:
     f = p0 (sin(w y) sin(w z), sin(w z) sin(w x), sin(w x) sin(w y)) */
  MSFEC_LOAD_VEC_TRIG = 3
} msfec_load_kind;

typedef struct msfec_load {
  int32_t kind; /* msfec_load_kind */
  int32_t reserved;
  double params[4];
} msfec_load;

typedef struct msfec_config {
  int32_t device;     /* CUDA device ordinal */
  int32_t precision;  /* msfec_precision */
  /* Local solve stops when ||r||_2 <= rtol * ||K_IB g||_2 (the residual norm
     the reference's zero initial guess starts from), per right-hand side. */
  double rtol;
  /* MIXED only: relative residual reduction of each FP32 inner solve. */
  double inner_rtol;
  int32_t max_iter;    /* Krylov iterations per inner solve */
  int32_t max_refine;  /* MIXED: FP64 refinement steps; FP64: verification rounds */
  int32_t verbose;
  /* Q1 launch shape when a batch mixes cluster (z-slab) and independent
     items: 0 = autotuned (msfec_autotune) or else one fused launch,
     1 = one fused launch, 2 = split cluster / non-cluster launches. */
  int32_t q1_launch;
  /* The mixed local solves (Ned_RT, Q_Ned, RT_DQ) stop when
     ||r||_P <= nedrt_rtol * ||f_I - A_IB g||_P, ||v||_P^2 = v^T P v with P the
     solver's (block-diagonal) preconditioner: the norm MINRES minimises, and
     one that weighs the edge and face rows alike whatever the fine mesh size
     (the face rows of the unscaled system outweigh the edge rows by ~h^-2).
     The mixed local system has condition number ~1e4 at depth 3, so 1e-14
     is needed for a 1e-10 basis error. */
  double nedrt_rtol;
  /* Preconditioner of the Ned_RT local solver:
     0 = face (Schur) block multilevel (diagonal + coarse RT levels n/2 .. 4 +
         exact level 2); edge block, for cells whose MINRES workspace is in
         global memory (depth 4, or the FP64 path at depth 3), the additive
         Schwarz operator over fine-cell patches (the inverse of the assembled
         edge mass on each fine cell's 12 edges), else diag(M)^-1;
     1 = diagonal only (both blocks);
     2 = multilevel face block, diagonal edge block. */
  int32_t nedrt_precond;
  /* Layout of the Q1 diffusion coefficient `a` (msfec_q1_coefficient):
     SCALAR one value per fine cell (default); TENSOR a symmetric positive
     definite A per fine cell, 6 doubles a00 a11 a22 a01 a02 a12; GAUSS A at
     each of the fine cell's 2x2x2 Gauss points, 8 x 6 doubles (points x
     fastest at 0.5 -+ 1/(2 sqrt 3) of the cell), which is what the
     reference's Diffusion_A::value_list gives its assembly
     (source/equation_data/eqn_coeff_A.cc:162-191, q_basis.cc:218-231). */
  int32_t q1_coefficient;
  /* Ned_RT cells whose MINRES workspace is in global memory (depth 4, mixed
     precision): 1 = the operator apply reads its coefficient tiles from shared
     memory, put there two rounds ahead by bulk (TMA) copies; 0 = plain global
     loads. Same results either way. */
  int32_t nedrt_stage;
  /* CTAs per SM of the mixed local solvers (Ned_RT, Q_Ned, RT_DQ): 0 = the
     autotuned choice (msfec_autotune) or else the default (two 256-thread
     CTAs per SM where the shared workspace fits twice, one 512-thread CTA
     otherwise); 1 = one 512-thread CTA per SM; 2 = two 256-thread CTAs per SM
     where the workspace allows (shared workspace split between shared memory
     and a global slot, or, for Ned_RT cells with a global workspace, two
     global slots per SM). Same results either way. */
  int32_t nedrt_ctas_per_sm;
  /* Ned_RT cells whose MINRES workspace is in global memory (depth 4, mixed
     precision, multilevel face preconditioner, one 512-thread CTA per SM, not
     staged): where the preconditioned Lanczos vector z~ lives. 0 = the default
     (shared memory), 1 = shared memory after the multilevel region (the
     operator apply gathers it and the edge patch pass accumulates into it on
     the SM), 2 = the CTA's global slot with the other Krylov vectors. Same
     results either way (to the order of the floating-point sums). */
  int32_t nedrt_zt_place;
  /* MIXED: relative residual reduction asked of the FP32 Krylov solve in each
     FP64 refinement step of the Ned_RT basis solves (the last step asks only
     what nedrt_rtol still needs); 0 = inner_rtol. Default 3e-6: fewer MINRES
     iterations in total than 1e-6 for the same final residual. */
  double nedrt_inner_rtol;
} msfec_config;

typedef enum msfec_q1_coefficient {
  MSFEC_Q1_COEF_SCALAR = 0,
  MSFEC_Q1_COEF_TENSOR = 1,
  MSFEC_Q1_COEF_GAUSS = 2
} msfec_q1_coefficient;

typedef struct msfec_cell {
  double origin[3];
  double size[3];
  int32_t depth; /* local refinement levels, 1..5 */
  int32_t reserved;
} msfec_cell;

typedef struct msfec_cell_report {
  int32_t iterations;  /* Krylov iterations summed over refinement steps, max over RHS */
  int32_t refinements; /* FP64 residual evaluations */
  int32_t converged;   /* 1 if every RHS of the cell met rtol */
  int32_t iterations_sum; /* Krylov iterations summed over refinement steps and over the cell's RHS */
  double residual;     /* max over RHS of ||r||_2 / ||K_IB g||_2 */
} msfec_cell_report;

typedef struct msfec_handle msfec_handle;

/* Fills cfg with defaults: device 0, MIXED, rtol 1e-12, inner_rtol 1e-6,
   max_iter 2000, max_refine 6, nedrt_rtol 1e-14, nedrt_precond 0. */
void msfec_config_default(msfec_config *cfg);

msfec_status msfec_create(msfec_handle **handle, const msfec_config *cfg);
void msfec_destroy(msfec_handle *handle);
const char *msfec_status_string(msfec_status status);
/* Text of the last error seen by this handle (CUDA error or argument check). */
const char *msfec_last_error(const msfec_handle *handle);

/* Use an external CUDA stream (cudaStream_t passed as void*) for all work of
   this handle; NULL restores the handle's own stream. */
msfec_status msfec_set_stream(msfec_handle *handle, void *stream);
msfec_status msfec_set_precision(msfec_handle *handle, int32_t precision);

/*
 * Q1 basis build from host buffers (synchronous).
 * Replaces QBasis::run (q_basis.cc:518-603) for every cell of the batch,
 * followed by get_global_element_matrix / get_global_element_rhs
 * (q_basis.cc:361-373).
 *   a        diffusion coefficient per fine cell, FP64, in the handle's
 *            q1_coefficient layout: a > 0 (SCALAR), an SPD tensor (TENSOR),
 *            an SPD tensor at each Gauss point (GAUSS). The tensor layouts
 *            run a cell-wise quadrature apply (the reference's assembly
 *            loop) instead of the scalar 27-point stencil.
 *   reaction reaction coefficient per fine cell, or NULL for none (the
 *            reference's ReactionRate is zero, eqn_coeff_R.cc:7-14)
 *   KH       [ncells][8][8], FH [ncells][8], reports [ncells] or NULL
 * The basis stays on the device until the next build (msfec_q1_get_basis).
 */
msfec_status msfec_q1_build(msfec_handle *handle, int32_t ncells,
                            const msfec_cell *cells, const double *a,
                            const double *reaction, const msfec_load *load,
                            double *KH, double *FH, msfec_cell_report *reports);

/*
 * Same as msfec_q1_build with every array in device memory; asynchronous on
 * the handle's stream. cells is a HOST array (it sizes the work queue).
 */
msfec_status msfec_q1_build_device(msfec_handle *handle, int32_t ncells,
                                   const msfec_cell *cells, const double *d_a,
                                   const double *d_reaction,
                                   const msfec_load *load, double *d_KH,
                                   double *d_FH, msfec_cell_report *d_reports);

/*
 * Adjoint of the Q1 build: dJ/d(log a) for every fine cell of the batch, for a
 * misfit J of the coarse multiscale solution u_H = sum_i U_i phi_i evaluated at
 * points. Host buffers, synchronous. The caller owns the coarse problem:
 *   U        [ncells][8] coarse solution restricted to each cell (vertex order)
 *   lambda   [ncells][8] coarse adjoint K_H^-1 dJ/dU restricted to each cell
 *   points   [npoints][3] in cell cell_of[p]; dJ_du[p] = dJ / d u_H(points[p])
 *   grad     [fine cells] output, total derivative dJ / d log a_e; for the
 *            tensor layouts (q1_coefficient TENSOR / GAUSS) the derivative
 *            with respect to theta_e in A_e -> exp(theta_e) A_e (every
 *            Gauss-point tensor of the fine cell scaled together)
 * Two adjoint local problems per cell (load and observation bubbles) run
 * through the batched local solver; no basis sensitivity is solved for
 * because the multiscale basis is K-harmonic. With reuse_basis != 0 the
 * basis of the last msfec_q1_build on this handle is reused when the batch is
 * the same (same cells; the caller guarantees the same a); otherwise it is
 * recomputed first (the reference keeps no basis either: basis objects are
 * rebuilt per run, q_global.cc:38-87). Coefficients are checked as in
 * msfec_q1_build (MSFEC_ERROR_NUMERICAL). No counterpart in the reference,
 * which has no adjoint; it extends QBasis with the gradient of its outputs.
 */
msfec_status msfec_q1_backward(msfec_handle *handle, int32_t ncells,
                               const msfec_cell *cells, const double *a,
                               const double *reaction, const msfec_load *load,
                               int32_t reuse_basis, const double *U,
                               const double *lambda, int32_t npoints,
                               const int32_t *cell_of, const double *points,
                               const double *dJ_du, double *grad);

/* Per-phase device time of the last build, measured with CUDA events on the
   handle's stream when timing is enabled (the reference's TimerOutput scopes,
   source/Q/q_global.cc:21-24). Milliseconds; -1 when not measured. */
typedef struct msfec_timings {
  float solve_ms;    /* persistent local-solver kernel (alone; see setup_ms) */
  float galerkin_ms; /* Phi^T K Phi / Phi^T f contraction */
  float total_ms;    /* whole build on the device, H2D/D2H excluded */
  int32_t solve_launches;
  int32_t kernel_launches; /* kernels this build launched */
  /* 0: launched directly; 1: captured into a new CUDA graph, then launched;
     2: replayed the cached graph (solve_ms then covers the whole graph) */
  int32_t graph;
  /* preconditioner setup kernel before the solver (Ned_RT multilevel
     data); 0 when the build ran none */
  float setup_ms;
} msfec_timings;

msfec_status msfec_set_timing(msfec_handle *handle, int32_t enable);

/*
 * CUDA-graph mode for repeated builds (default off). The refinement loop of
 * every local solve runs inside the persistent kernel, so one build is a
 * fixed sequence of device operations (queue reset, solver, Galerkin,
 * report). With graph mode on, the first build of a batch captures that
 * sequence into a CUDA graph; a later build of the same kind with the same
 * cells, load, configuration, stream and buffer pointers skips the host
 * planner and the plan upload and replays the graph, reading the current
 * contents of the coefficient buffers (the case of an optimisation or
 * adjoint loop that updates coefficients in place). Any other build of that
 * kind re-captures. Results are those of the direct launches. Turning the
 * mode off drops the cached graphs.
 */
msfec_status msfec_set_graph(msfec_handle *handle, int32_t enable);
/* Synchronises the handle's stream. */
msfec_status msfec_get_timings(msfec_handle *handle, msfec_timings *out);

/* Number of doubles of the last Q1 build's basis (sum over cells of
   8 (n+1)^3), or 0 if none. */
int64_t msfec_q1_basis_size(const msfec_handle *handle);

/* Copy the last Q1 build's basis to host memory (capacity in doubles). */
msfec_status msfec_q1_get_basis(msfec_handle *handle, double *Phi,
                                int64_t capacity);

/* Copy the basis of cells [first, first + count) of the last Q1 build (in
   the batch's cell order, 8 (n+1)^3 doubles per cell) to host memory: the
   per-cell basis of the reference's QBasis objects (each holds its own
   basis_solution, source/Q/q_basis.h:77-139) without copying the whole
   batch. capacity in doubles. */
msfec_status msfec_q1_get_basis_cells(msfec_handle *handle, int32_t first,
                                      int32_t count, double *Phi,
                                      int64_t capacity);

/* Device pointer of the last Q1 build's basis (read-only, valid until the
   next build on this handle). */
const double *msfec_q1_basis_device(const msfec_handle *handle);

/*
 * Fine-scale reconstruction u = sum_v U_v phi_v of the last Q1 build,
 * evaluated at points (reference QBasis::set_global_weights,
 * q_basis.cc:394-416, which forms the same combination on the fine mesh).
 *   weights  [ncells][8] coarse weights U of every cell of the last build
 *   cell_of  [npoints] batch index of the cell containing each point
 *   points   [npoints][3], values [npoints]
 * Host buffers, synchronous.
 */
msfec_status msfec_q1_eval_fine(msfec_handle *handle, const double *weights,
                                int32_t npoints, const int32_t *cell_of,
                                const double *points, double *values);

/*
 * Standard fine-scale Q1 solve (the reference's QReferenceSolution path,
 * source/Q/q_ref.cc:139-363, as an independent accuracy reference for the
 * multiscale solution): -div(a grad u) + r u = f on the box `domain`
 * (uniformly refined depth times, depth 1..5, e.g. the unit cube with depth
 * 5 = the 32^3 fine grid of a coarse 4^3 x depth-3 multiscale run) with
 * homogeneous Dirichlet data. The same persistent solver runs one
 * source-mode item (FP32 PCG + FP64 refinement in MIXED). Host buffers,
 * synchronous. a, reaction: n^3 per fine cell; u: (n+1)^3 nodal values
 * (node = i + (n+1)(j + (n+1)k)). report may be NULL.
 */
msfec_status msfec_q1_fine_solve(msfec_handle *handle, const msfec_cell *domain,
                                 const double *a, const double *reaction,
                                 const msfec_load *load, double *u,
                                 msfec_cell_report *report);

/*
 * Standard fine-scale Ned_RT solve (the reference's NedRTStd path,
 * source/Ned_RT/ned_rt_ref.cc:110-330, as an independent accuracy reference
 * for the Ned_RT multiscale solution): the mixed system
 *   (A^-1 sigma, tau) - (u, curl tau) = 0
 *   (curl sigma, v) + (B div u, div v) = (f, v)
 * on the box `domain` (uniformly refined depth times, depth 1..4) with the
 * reference's boundary treatment: its essential projections are disabled
 * (ned_rt_ref.cc:119-133), so every boundary edge and face is free (natural
 * conditions), and the reaction term is zero (eqn_coeff_R.cc:8-14). The
 * persistent Ned_RT solver runs one source item over the whole lattice with
 * the diagonal preconditioner. Host buffers, synchronous.
 *   ainv6, bdiv  per fine cell, as for msfec_nedrt_build
 *   load         MSFEC_LOAD_ZERO or MSFEC_LOAD_VEC_TRIG
 *   x            [NE + NF]: sigma on the fine edges, then u on the fine faces,
 *                in the lattice order of the Ned_RT basis vectors
 * report may be NULL.
 */
msfec_status msfec_nedrt_fine_solve(msfec_handle *handle, const msfec_cell *domain,
                                    const double *ainv6, const double *bdiv,
                                    const msfec_load *load, double *x,
                                    msfec_cell_report *report);

/*
 * Ned_RT (lowest-order Nedelec sigma x Raviart-Thomas u) basis build from
 * host buffers (synchronous). Replaces NedRTBasis::run
 * (source/Ned_RT/ned_rt_basis.cc:1279-1428) for every cell of the batch,
 * followed by get_global_element_matrix / get_global_element_rhs
 * (ned_rt_basis.cc:1262-1273).
 *   ainv6  A^-1 per fine cell, 6 doubles (a00 a11 a22 a01 a02 a12), SPD
 *          (the reference's DiffusionInverse_A, eqn_coeff_A.cc:193-242)
 *   bdiv   B per fine cell (> 0): the div-div weight (Diffusion_B,
 *          eqn_coeff_B.cc:72-114); the reaction term of the reference is zero
 *   load   MSFEC_LOAD_ZERO or MSFEC_LOAD_VEC_TRIG (global load, F_H only)
 *   KH     [ncells][18][18]: rows/cols 0..11 coarse edges (GeometryInfo<3>
 *          line order), 12..17 coarse faces; FH [ncells][18] (edge rows 0)
 * Coarse Nedelec / RT functions are normalised to unit line integral / unit
 * flux along the positive axis (deal.II FE_Nedelec(0) / FE_RaviartThomas(0)).
 * Depth 1..4.
 */
msfec_status msfec_nedrt_build(msfec_handle *handle, int32_t ncells,
                               const msfec_cell *cells, const double *ainv6,
                               const double *bdiv, const msfec_load *load,
                               double *KH, double *FH,
                               msfec_cell_report *reports);

/* Device-pointer variant (asynchronous on the handle's stream); cells on the host. */
msfec_status msfec_nedrt_build_device(msfec_handle *handle, int32_t ncells,
                                      const msfec_cell *cells,
                                      const double *d_ainv6,
                                      const double *d_bdiv,
                                      const msfec_load *load, double *d_KH,
                                      double *d_FH,
                                      msfec_cell_report *d_reports);

/*
 * Allocation-free variant of msfec_nedrt_build_device. No counterpart in the
 * reference (deal.II allocates per cell inside NedRTBasis::run); it serves
 * callers that must not allocate device memory while they build: a solver
 * whose pooling allocator already holds nearly all of HBM, or a rank whose
 * other streams must not be stalled by the device-wide synchronisation of
 * cudaMalloc / cudaFree. Same arguments, asynchrony and launch shape as
 * msfec_nedrt_build_device on the same handle (the autotuned split / CTA
 * choices) and the same face preconditioner (multilevel for depth >= 2 unless
 * nedrt_precond = 1); the edge block is diag(M)^-1 throughout (the handle's
 * build uses the cell-patch edge block on cells with a global workspace), so
 * K_H, F_H agree with that build within the solver tolerance, and with a
 * build at nedrt_precond = 2 up to the last bits of the shared-memory atomic
 * sums; but every internal buffer
 * comes from one static device pool of 32 MiB per device that is part of the
 * library image; nothing is allocated on the device (host memory only to
 * format an error message). A batch whose cell table, multilevel data, basis
 * Phi, Y = A Phi and status (about 1.06 MB per depth-3 cell, 7.82 MB per
 * depth-4 cell) do not fit, or that holds more than 4096 cells, is rejected
 * with MSFEC_ERROR_INVALID_ARGUMENT and a message naming the bytes needed;
 * split it. Depth-4 cells also take 0.99 MB (mixed) / 1.75 MB (FP64) of
 * MINRES workspace per concurrent CTA from the rest of the pool, so fewer
 * CTAs run when space is short. Every call looks up the pool's address on
 * the current device; the first call on a device may load the library's
 * module for it: make that first call before any stream capture. The basis
 * stays in the pool and is overwritten by the next call: msfec_nedrt_get_basis
 * still returns the last handle-owned build, and msfec_nedrt_backward with
 * reuse_basis set rebuilds the basis (it never reuses a pool basis or an older
 * handle-owned one after this call). There is one pool per device and
 * process: calls that overlap in time on the same device (other threads,
 * handles or streams) race and corrupt each other's results; serialise them
 * on one stream.
 */
msfec_status msfec_nedrt_build_noalloc(msfec_handle *handle, int32_t ncells,
                                       const msfec_cell *cells,
                                       const double *d_ainv6,
                                       const double *d_bdiv,
                                       const msfec_load *load, double *d_KH,
                                       double *d_FH,
                                       msfec_cell_report *d_reports);

/* Problem kinds (msfec_autotune). */
typedef enum msfec_kind {
  MSFEC_KIND_Q1 = 1,
  MSFEC_KIND_NEDRT = 2,
  MSFEC_KIND_QNED = 3,
  MSFEC_KIND_RTDQ = 4
} msfec_kind;

/*
 * Autotuner for launch shapes. Builds the given batch (host buffers, as the
 * kind's build entry point: Q1 coef0 = a, coef1 = reaction or NULL; Ned_RT
 * coef0 = ainv6, coef1 = bdiv; Q_Ned coef0 = a6, coef1 = binv; RT_DQ coef0 =
 * ainv6, coef1 unused) twice per candidate in the handle's precision, times
 * the second build on the device, and keeps the fastest candidate for later
 * builds of that kind on this handle. Pass a representative sample (e.g. one
 * or two GPU waves of cells); the call costs 2 builds per candidate.
 * choice[0] = index of the chosen candidate, choice[1] = number of
 * candidates; times_ms (NULL or >= 16 floats) receives each candidate's time.
 * Candidates, in order:
 *   Q1 (per precision and reaction on/off), when the batch mixes cluster
 *     (z-slab) items with independent ones: 0 = one launch of the cluster
 *     kernel over all items, 1 = the cluster kernel over the slab items and
 *     a non-cluster kernel over the rest, concurrently on two streams.
 *   Ned_RT (per precision and deepest depth): with the MINRES workspace in
 *     shared memory (mixed, depth <= 3): 0 = one 512-thread CTA per SM,
 *     1 = two 256-thread CTAs per SM (split workspace). With it in global
 *     memory (depth 4, or FP64): the number of resident CTAs, i.e. of
 *     workspace slots in L2, the SM count times 1, 7/8, 6/8, 5/8, 4/8, first
 *     with plain coefficient loads, then (mixed only) with the apply's
 *     coefficient tiles staged by bulk copies (nedrt_stage), then (mixed
 *     only) two 256-thread CTAs per SM with a global slot each: 11 candidates.
 *   Q_Ned, RT_DQ (per deepest depth, mixed): 0 = one 512-thread CTA per SM,
 *     1 = two 256-thread CTAs per SM (when the workspace fits twice).
 * Batches with a single candidate return at once (choice = {0, 1}).
 */
msfec_status msfec_autotune(msfec_handle *handle, int32_t kind, int32_t ncells,
                            const msfec_cell *cells, const double *coef0,
                            const double *coef1, const msfec_load *load,
                            int32_t *choice, float *times_ms);

/*
 * Adjoint of the Ned_RT build: dJ/d(log A) and dJ/d(log B) per fine cell
 * (A_e scaled by exp(ta_e), B_e by exp(tb_e)) for a misfit J of the coarse
 * multiscale u field (face bases' u-blocks weighted by the coarse solution,
 * NedRTBasis::set_global_weights, ned_rt_basis.cc:1155-1181) at points. Host
 * buffers, synchronous; the caller owns the coarse problem:
 *   U, lambda  [ncells][18] coarse solution and coarse adjoint
 *              (K_H^-T dJ/dU, K_H nonsymmetric) restricted to each cell
 *   points     [npoints][3] in cell cell_of[p]; dJ_du[p][3] = dJ / d u_h(points[p])
 *   grad_a, grad_b  [fine cells] outputs
 * Four adjoint local problems per cell (edge / face bases x lambda / U
 * weights) run as source items of the batched MINRES solver (A^T = S A S, S
 * = -1 on face rows), to max(nedrt_rtol, 1e-11) relative residual (in the
 * preconditioner's norm), taken relative to max(||f||_P, 1e-3 of the P-norm
 * of the cell's adjoint source scale) (the
 * right-hand sides are projections and differences that can cancel to
 * rounding); the basis is rebuilt unless reuse_basis != 0 and the
 * last Ned_RT build on this handle is the same batch. Coefficients are
 * checked as in msfec_nedrt_build (MSFEC_ERROR_NUMERICAL). grad_a vanishes to
 * rounding when the coarse solution has no edge part (e.g. the divergence-free
 * MSFEC_LOAD_VEC_TRIG load on a coarse 2^3 grid with the boundary edges and
 * faces fixed); B then carries the sensitivity.
 */
msfec_status msfec_nedrt_backward(msfec_handle *handle, int32_t ncells,
                                  const msfec_cell *cells, const double *ainv6,
                                  const double *bdiv, const msfec_load *load,
                                  int32_t reuse_basis, const double *U,
                                  const double *lambda, int32_t npoints,
                                  const int32_t *cell_of, const double *points,
                                  const double *dJ_du, double *grad_a,
                                  double *grad_b);

/*
 * Q1 x Nedelec (Q_Ned) basis build from host buffers (synchronous). Replaces
 * QNedBasis::run (source/Q_Ned/q_ned_basis.cc) for every cell of the batch,
 * followed by get_global_element_matrix / get_global_element_rhs.
 *   a6     A per fine cell, 6 doubles (a00 a11 a22 a01 a02 a12), SPD: the
 *          curl-curl weight (the reference's Diffusion_A)
 *   binv   B^-1 per fine cell (> 0): the sigma mass weight (DiffusionInverse_B)
 *   load   MSFEC_LOAD_ZERO or MSFEC_LOAD_VEC_TRIG (global load (v, f), F_H only)
 *   KH     [ncells][20][20]: rows/cols 0..7 coarse vertices (H1 bases,
 *          GeometryInfo<3>), 8..19 coarse lines (curl bases); FH [ncells][20]
 *          (vertex rows 0)
 * Depth 1..4. Tolerance nedrt_rtol (the same mixed-form solver).
 */
msfec_status msfec_qned_build(msfec_handle *handle, int32_t ncells,
                              const msfec_cell *cells, const double *a6,
                              const double *binv, const msfec_load *load,
                              double *KH, double *FH,
                              msfec_cell_report *reports);

/* Device-pointer variant (asynchronous on the handle's stream); cells on the host. */
msfec_status msfec_qned_build_device(msfec_handle *handle, int32_t ncells,
                                     const msfec_cell *cells, const double *d_a6,
                                     const double *d_binv,
                                     const msfec_load *load, double *d_KH,
                                     double *d_FH,
                                     msfec_cell_report *d_reports);

/* Basis of the last Q_Ned build: per cell 20 rows of NV + NE fine DoFs
   (vertices i + (n+1)(j + (n+1)k), then edges x|y|z). */
int64_t msfec_qned_basis_size(const msfec_handle *handle);
msfec_status msfec_qned_get_basis(msfec_handle *handle, double *Phi,
                                  int64_t capacity);

/*
 * Raviart-Thomas x DQ0 (RT_DQ) basis build from host buffers (synchronous).
 * Replaces RTDQBasis::run (source/RT_DQ/rt_dq_basis.cc:1114-1216) for every
 * cell of the batch, followed by get_global_element_matrix /
 * get_global_element_rhs (:1096-1106).
 *   ainv6  A^-1 per fine cell, 6 doubles (a00 a11 a22 a01 a02 a12), SPD: the
 *          sigma mass weight (the reference's DiffusionInverse_A); the
 *          reaction rate is 0 (source/equation_data/eqn_coeff_R.cc:7-14)
 *   load   MSFEC_LOAD_ZERO, _CONSTANT or _SIN_PRODUCT (scalar global load
 *          (v, f), F_H only)
 *   KH     [ncells][7][7]: rows/cols 0..5 coarse faces (GeometryInfo<3>
 *          face order), 6 the coarse DQ0 value; FH [ncells][7] (face rows 0)
 * The local problems are pure-Neumann ones (is_laplace): sigma is unique,
 * the local pressure is fixed up to a constant and, as in the reference
 * (set_u_to_std, :1039-1044), the stored u block of every basis is 1.
 * Depth 1..4. Tolerance nedrt_rtol (the same mixed-form solver).
 */
msfec_status msfec_rtdq_build(msfec_handle *handle, int32_t ncells,
                              const msfec_cell *cells, const double *ainv6,
                              const msfec_load *load, double *KH, double *FH,
                              msfec_cell_report *reports);

/* Device-pointer variant (asynchronous on the handle's stream); cells on the host. */
msfec_status msfec_rtdq_build_device(msfec_handle *handle, int32_t ncells,
                                     const msfec_cell *cells,
                                     const double *d_ainv6,
                                     const msfec_load *load, double *d_KH,
                                     double *d_FH,
                                     msfec_cell_report *d_reports);

/* Basis of the last RT_DQ build: per cell 6 rows of NF + NC fine DoFs (faces
   x|y|z as for Ned_RT, then cells i + n(j + n k)). */
int64_t msfec_rtdq_basis_size(const msfec_handle *handle);
msfec_status msfec_rtdq_get_basis(msfec_handle *handle, double *Phi,
                                  int64_t capacity);

/* Basis of the last Ned_RT build: per cell 18 rows (coarse basis order) of
   NE + NF fine DoFs (edges x|y|z then faces x|y|z, lexicographic), sigma and u
   of every basis function. Size in doubles, and copy to host. */
int64_t msfec_nedrt_basis_size(const msfec_handle *handle);
msfec_status msfec_nedrt_get_basis(msfec_handle *handle, double *Phi,
                                   int64_t capacity);

/* Copy the basis of cells [first, first + count) of the last handle-owned
   Ned_RT build (batch cell order, 18 (NE + NF) doubles per cell, layout of
   msfec_nedrt_get_basis) to host memory: the per-cell basis_solution of the
   reference's NedRTBasis objects (source/Ned_RT/ned_rt_basis.h:99-153)
   without copying the whole batch (16 GB at coarse 16^3 x depth 4).
   capacity in doubles. */
msfec_status msfec_nedrt_get_basis_cells(msfec_handle *handle, int32_t first,
                                         int32_t count, double *Phi,
                                         int64_t capacity);

#ifdef __cplusplus
}
#endif
#endif /* MSFEC_CUDA_H */
