/*
 * gb_gmg.h -- C ABI of the GB300 matrix-free geometric-multigrid Stokes solver
 * (Q2-Q1 Taylor-Hood, global-coarsening level hierarchy).
 *
 * This is the boundary an ASPECT-side StokesMatrixFreeHandler implementation
 * binds to. It replaces, call for call, the work done behind
 *   include/aspect/simulator/solver/stokes_matrix_free.h:47-98
 *     (StokesMatrixFreeHandler: setup_dofs / assemble / build_preconditioner)
 *   include/aspect/simulator/solver/interface.h:36-58,90-94
 *     (StokesSolver::SolverOutputs, StokesSolver::Interface::solve)
 * as implemented in source/simulator/solver/stokes_matrix_free_local_smoothing.cc
 * and source/simulator/solver/stokes_matrix_free_global_coarsening.cc.
 *
 * Conventions
 *  - Every function returns GB_GMG_OK (0) or an error code; nothing throws
 *    across the ABI. gb_gmg_last_error() gives the message of the last error.
 *    A null array, a block other than 0 (velocity) / 1 (pressure) or a level out
 *    of range returns GB_GMG_INVALID_ARGUMENT, a missing set-up step
 *    GB_GMG_NOT_READY, before any device work. Array lengths are the caller's to
 *    get right: the library reads and writes the sizes each entry states.
 *  - The caller owns every host array; the library copies what it needs into
 *    GB300 device memory (HBM). The handle owns all device memory. Set-up calls
 *    allocate; operator, transfer and V-cycle calls do not. A solve allocates
 *    only the first time it meets a Krylov size it has not held since the last
 *    gb_gmg_finalize_setup (restart length for GMRES/FGMRES, s for IDR(s)):
 *    (restart + 1) + restart FP64 vectors of the finest level, about 1.4 GB at
 *    32^3 with restart 100; later solves of the same size reuse them.
 *  - One host thread per handle. Each handle drives one GPU (the current CUDA
 *    device when gb_gmg_create is called).
 *  - Levels are numbered 0 (coarsest) .. n_levels-1 (finest = active mesh).
 *  - Cell-local DoF order: velocity FE_Q(k)^dim with components blocked and
 *    nodes lexicographic (x fastest): local = c*(k+1)^dim + lex(i,j[,k]);
 *    pressure FE_Q(k-1): local = lex(i,j[,k]). k = degree_v of gb_gmg_create:
 *    2 (velocity nodes {0,1/2,1}, pressure {0,1}) or 3 (velocity nodes the
 *    Gauss-Lobatto points {0, (1-1/sqrt5)/2, (1+1/sqrt5)/2, 1} as deal.II's FE_Q(3),
 *    pressure {0,1/2,1}). Quadrature: QGauss(k+1), points lexicographic.
 *    Degree 3 runs on indexed levels; the Newton / dilation and free-surface
 *    terms, the device body force and the adjoint gradient are degree 2 only.
 *  - Pressure is the scaled unknown p/s on input and output, as in the
 *    reference (stokes_matrix_free_local_smoothing.cc:975,1421). Constraint
 *    distribution, p *= s, nullspace removal and pressure normalisation stay on
 *    the caller's side, as in the reference (:1406-1443).
 */
#ifndef GB_GMG_H
#define GB_GMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_gmg gb_gmg;

enum gb_gmg_status {
  GB_GMG_OK = 0,
  GB_GMG_INVALID_ARGUMENT = 1,
  GB_GMG_NOT_READY = 2,          /* a set-up step is missing */
  GB_GMG_CUDA_ERROR = 3,
  GB_GMG_NO_CONVERGENCE = 4,     /* SolverControl::NoConvergence equivalent */
  GB_GMG_BREAKDOWN = 5,
  GB_GMG_NAN_DETECTED = 6,
  GB_GMG_OUT_OF_MEMORY = 7,
  GB_GMG_EXCEEDS_STATIC_SCRATCH = 8  /* level larger than GB_GMG_NOALLOC_MAX_CELLS */
};

enum gb_gmg_geometry {
  GB_GMG_GEOM_BOX = 0,  /* per cell: lower corner x0[dim], edge lengths h[dim]    */
  GB_GMG_GEOM_Q2 = 1,   /* per cell: 3^dim Q2 mapping support points [node][dim]  */
  GB_GMG_GEOM_TABLE = 2 /* per cell and QGauss(k+1) point (lexicographic): the
                           inverse Jacobian [d*dim+e] = d xi_d / d x_e, then
                           |det J|; dim*dim+1 values per point. The caller's own
                           mapping, e.g. ASPECT's MappingQCache of degree 4 on
                           curved geometries (source/simulator/core.cc:106-119),
                           evaluated at the quadrature points                   */
};

enum gb_gmg_operator {
  GB_GMG_OP_STOKES = 0, /* [A  B^T; B 0] on (u, p): src/dst = [u; p]       */
  GB_GMG_OP_A = 1,      /* velocity block                                  */
  GB_GMG_OP_BT = 2,     /* p -> u                                          */
  GB_GMG_OP_MASS = 3    /* pressure mass matrix scaled by s^2/eta          */
};

enum gb_gmg_precision { GB_GMG_FP64 = 0, GB_GMG_FP32 = 1 };

enum gb_gmg_krylov {
  GB_GMG_GMRES = 0,       /* reference: cheap GMRES, FGMRES fallback          */
  GB_GMG_GMRES_IR = 1,    /* FP64 iterative refinement around FP32 GMRES       */
  GB_GMG_IDR = 2          /* cheap IDR(s), FGMRES fallback ("Krylov method for
                             cheap solver steps = IDR(s)",
                             stokes_matrix_free_local_smoothing.cc:1290-1299)  */
};

enum gb_gmg_projection {
  GB_GMG_VISC_DGQ0 = 0, /* one (averaged) value per cell; levels: cell means     */
  GB_GMG_VISC_DGQ1 = 1, /* values per quadrature point, projected to Q1 per cell
                           (project_to_Q1 averaging); levels: Q1 interpolation,
                           clamped to the active-level range                    */
  GB_GMG_VISC_NONE = 2  /* "Material averaging = none": values per quadrature
                           point for the outer operators (FGMRES product, the
                           expensive inner solves, rhs correction, adjoint);
                           every multigrid level, the finest included, takes the
                           cellwise (DGQ0) projection, as the reference fills its
                           level tables (stokes_matrix_free_local_smoothing.cc:
                           211-294, matrix_free_operators.cc:137-330). gb_gmg_vmult
                           applies the multigrid tables.                        */
};

/* Mirrors "Solver parameters/Stokes solver parameters" and "Matrix Free"
 * (source/simulator/parameters.cc:436-600, stokes_matrix_free_local_smoothing.cc:52-85). */
typedef struct gb_gmg_options {
  int verbose;                  /* Output details                                   */
  int smoother_degree;          /* Chebyshev degree on levels > 0 (4)                */
  double smoothing_range;       /* Chebyshev smoothing range on levels > 0 (15)      */
  int eig_cg_iterations;        /* eigenvalue-estimate CG steps on levels > 0 (10)   */
  int coarse_degree;            /* Chebyshev degree on level 0 (8)                   */
  double coarse_range;          /* level-0 range (1e-3: use the CG minimum estimate) */
  int coarse_eig_cg_iterations; /* level-0 eigenvalue CG steps (100)                 */
  int schur_smoothing_steps;    /* SmootherRelaxation steps for the Schur block (4)  */
  int force_indexed_layout;     /* 1: never use the lattice fast path (testing)      */
  int coarse_solver;            /* gb_gmg_coarse_solver (Chebyshev as the reference)  */
  int fused_a_min_cells;        /* > 0: FP32 A-block applications of 3D lattice levels
                                   with at least this many cells (and 16 x 8 | cells in
                                   x, y) run as one fused cell-and-gather pass (0: never,
                                   the default: the two-pass form measured faster)      */
  int dense_mass_cycle_nodes;   /* FP32 Schur (pressure-mass) V-cycle: the sub-cycle of
                                   the coarse lattice levels up to the highest one with
                                   at most this many pressure nodes is computed once per
                                   preconditioner build as an explicit matrix and applied
                                   as one dense product (1000, the levels one block can
                                   run; up to 6000 adds the next lattice level, built by
                                   batched kernels: 160 ms more per build at 32^3, for
                                   0.036 ms less per V-cycle; 0: off)                  */
  int dense_a_cycle_dofs;       /* the same for the FP32 A-block V-cycle: lattice levels
                                   up to the highest one with at most this many velocity
                                   DoFs (<= 2200; 2200; 0: off)                        */
  int fused_small_smoother;     /* 1: the FP32 A-block smoother of small lattice levels
                                   (one-cell-per-block cell pass) runs each Chebyshev
                                   step's gather and the next step's cell pass as one
                                   launch (the same arithmetic; 1); 0: two launches  */
} gb_gmg_options;

enum gb_gmg_coarse_solver {
  GB_GMG_COARSE_CHEBYSHEV = 0,  /* one smoother application (MGCoarseGridApplySmoother) */
  GB_GMG_COARSE_DENSE_FP64 = 1  /* FP64 pseudo-inverse of the level-0 matrices (handles
                                   null spaces such as the rotations of a free-slip shell) */
};

/* Arithmetic of the classical Gram-Schmidt passes (with the conditional second
   pass) of the GMRES / FGMRES Arnoldi steps; the basis, the Hessenberg matrix, the
   operator and the residuals stay FP64 either way. */
enum gb_gmg_orthogonalization {
  GB_GMG_GS_FLOAT_PAIR = 0,  /* the k n multiply-adds of a step as unevaluated pairs of
                                floats (about 46 significant bits; Hessenberg entries
                                within a few 1e-15 |w| of the FP64 passes), on the FP32
                                pipe at the HBM rate of the basis; steps with more than
                                128 basis vectors and the first step after a (re)start
                                run the FP64 passes */
  GB_GMG_GS_FP64 = 1         /* FP64 passes (bound by the FP64 pipe on this GPU)      */
};

typedef struct gb_gmg_solve_params {
  double linear_solver_tolerance;  /* relative (1e-7); tolerance rule of :977-1041   */
  double absolute_tolerance;       /* > 0: use this absolute tolerance instead        */
  int n_cheap_steps;               /* Number of cheap Stokes solver steps (1000)      */
  int n_expensive_steps;           /* Maximum number of expensive ... steps (1000)    */
  int restart;                     /* GMRES solver restart length (100)               */
  double tol_A;                    /* Linear solver A block tolerance (1e-2)          */
  double tol_S;                    /* Linear solver S block tolerance (1e-6)          */
  int mg_precision;                /* gb_gmg_precision of the V-cycle                 */
  int krylov;                      /* gb_gmg_krylov                                   */
  double ir_inner_tolerance;       /* GMRES_IR: relative tolerance of each inner solve */
  int idr_s;                       /* IDR(s) parameter (2), source/simulator/parameters.cc:483 */
  int solve_newton_system;         /* StokesSolver::Interface::solve's solve_newton_system
                                      (interface.h:90-94): the solution is a Newton update,
                                      so the solve starts from zero and the tolerance and
                                      initial_nonlinear_residual use |rhs| alone
                                      (stokes_matrix_free_local_smoothing.cc:952-1041)   */
  int orthogonalization;           /* gb_gmg_orthogonalization of the GMRES / FGMRES
                                      Arnoldi steps (float pairs)                       */
} gb_gmg_solve_params;

/* StokesSolver::SolverOutputs plus the counters the reference prints. */
typedef struct gb_gmg_outputs {
  double initial_nonlinear_residual;
  double final_linear_residual;
  double solver_tolerance;
  int cheap_iterations;
  int expensive_iterations;
  int A_preconditioner_applications;
  int S_preconditioner_applications;
  int fp64_stokes_applications;     /* FP64 Stokes operator applications in the solve */
  int status;                       /* gb_gmg_status of the solve                     */
  double solve_seconds;             /* device time of the solve                       */
} gb_gmg_outputs;

/* Defaults identical to the reference's parameter defaults. */
void gb_gmg_default_options(gb_gmg_options* opt);
void gb_gmg_default_solve_params(gb_gmg_solve_params* prm);

/* Replaces create_matrix_free_solver (source/simulator/solver/stokes_matrix_free.cc:30-62):
 * degree_v 2 (Q2-Q1) or 3 (Q3-Q2), the reference's two instantiations (:39-40,53-54). */
int gb_gmg_create(const gb_gmg_options* opt, int dim, int degree_v, int n_levels, gb_gmg** out);
void gb_gmg_destroy(gb_gmg* h);
const char* gb_gmg_last_error(const gb_gmg* h);

/* setup_dofs (stokes_matrix_free_global_coarsening.cc:1456-1636): one level's
 * cell-to-DoF maps (n_cells x dim*(k+1)^dim and n_cells x k^dim, in the caller's
 * numbering) and geometry (gb_gmg_geometry). */
int gb_gmg_set_level_mesh(gb_gmg* h, int level, int64_t n_cells, const int32_t* cell_dofs_u,
                          const int32_t* cell_dofs_p, int geometry_kind, const double* cell_geometry,
                          int64_t n_u, int64_t n_p);

/* Closed AffineConstraints of one block (0 velocity, 1 pressure) of one level,
 * CSR: row rows[i] = sum_{k in [ptr[i],ptr[i+1])} weights[k] x[cols[k]] + inhom[i].
 * Lines without entries are Dirichlet lines (hanging nodes, no-normal-flux,
 * Dirichlet boundary values). inhomogeneities may be NULL. */
int gb_gmg_set_level_constraints(gb_gmg* h, int level, int block, int64_t n_lines, const int32_t* rows,
                                 const int32_t* ptr, const int32_t* cols, const double* weights,
                                 const double* inhomogeneities);

/* Parent cell (on level-1) and child index (bit d = upper half in direction d)
 * of every cell of `level` >= 1 (MGTwoLevelTransfer, :1701-1731). A cell that
 * is itself a cell of level-1 (not coarsened) has child index GB_GMG_SAME_CELL
 * and its own index on level-1 as parent. */
#define GB_GMG_SAME_CELL 255
int gb_gmg_set_transfer(gb_gmg* h, int level, const int32_t* child_to_parent, const uint8_t* child_index);

/* Ends setup_dofs: builds colourings, internal numbering, transfer operators. */
int gb_gmg_finalize_setup(gb_gmg* h);

/* assemble() -> evaluate_material_model (stokes_matrix_free_local_smoothing.cc:174-294):
 * finest-level viscosity, n_per_cell = 1 (averaged) or (k+1)^dim (per quadrature
 * point, QGauss(k+1) lexicographic), in the caller's cell order; the level tables
 * follow from `projection`. */
int gb_gmg_set_viscosity(gb_gmg* h, const double* eta, int n_per_cell, int projection,
                         double pressure_scaling, int compressible);

/* Same as gb_gmg_set_viscosity with the projection and pressure scaling of the
 * last call, but keeps the preconditioner of the last gb_gmg_build_preconditioner
 * (diagonals, Chebyshev intervals, captured V-cycles): the operators see the new
 * viscosity, the smoothers keep the old diagonals. For nearby coefficient fields,
 * e.g. finite-difference checks or nonlinear iterations that reuse a
 * preconditioner; ASPECT itself rebuilds after every assemble(). */
int gb_gmg_update_viscosity(gb_gmg* h, const double* eta, int n_per_cell);

/* Newton-derivative and prescribed-dilation terms of the outer Stokes operator
 * (OperatorCellData, include/aspect/simulator/solver/matrix_free_operators.h:92-208;
 * applied in StokesOperator::local_apply, matrix_free_operators.cc:400-538; the
 * tables are filled in stokes_matrix_free_local_smoothing.cc:296-612). Per finest
 * cell (caller order) and QGauss(3) point (lexicographic); symmetric tensors in
 * deal.II's unrolled order (00, 11, 22, 01, 02, 12 in 3D; 00, 11, 01 in 2D).
 * Only the outer Stokes operator (the FGMRES product, gb_gmg_vmult of
 * GB_GMG_OP_STOKES on the finest level) takes the Newton terms; with a
 * prescribed dilation the outer viscous terms are deviatoric as with
 * compressibility; the multigrid levels are unchanged, as in the reference
 * (:311-313). Arrays a flag does not use may be NULL. */
typedef struct gb_gmg_newton_terms {
  int enable_newton_derivatives;
  int symmetrize_newton_system;
  int average_newton_factors;
  int enable_prescribed_dilation;
  const double* strain_rate;                          /* strain_rate_table                 */
  const double* newton_factor_wrt_strain_rate;        /* newton_factor_wrt_strain_rate_table */
  const double* newton_factor_wrt_pressure;           /* newton_factor_wrt_pressure_table  */
  const double* dilation_lhs;                         /* dilation_lhs_term_table           */
  const double* dilation_derivative_wrt_strain_rate;  /* dilation_derivative_wrt_strain_rate_table */
  const double* dilation_derivative_wrt_pressure;     /* dilation_derivative_wrt_pressure_table */
} gb_gmg_newton_terms;

/* Sets (or with NULL clears) the Newton / dilation terms; call after
 * gb_gmg_set_viscosity, as assemble() does. */
int gb_gmg_set_newton_terms(gb_gmg* h, const gb_gmg_newton_terms* terms);

/* build_preconditioner (:1856-1867): level diagonals for both blocks and both
 * precisions and eigenvalue estimates (:834-849); the V-cycle graphs are
 * captured on their first use. The FP64 levels are built on their first use (an FP64 V-cycle or solve, an FP64
 * diagonal or eigenvalue query, gb_gmg_update_viscosity), from the tables of this
 * call; with GB_GMG_COARSE_DENSE_FP64 they are built here. */
int gb_gmg_build_preconditioner(gb_gmg* h);

/* One operator application on one level (host arrays, caller numbering).
 * Constrained rows act as the identity (MatrixFreeOperators::Base::vmult). */
int gb_gmg_vmult(gb_gmg* h, int op, int level, int precision, const double* src, double* dst);

/* StokesMatrixFreeHandler::correct_stokes_rhs
   (source/simulator/solver/stokes_matrix_free_local_smoothing.cc:618-754): rhs -= K u0
   on the finest level, where u0 (caller numbering, velocity then pressure) holds the
   inhomogeneous constraint values at constrained DoFs (what AffineConstraints::
   distribute gives on a zero vector) and zeros elsewhere. K is applied with plain
   reads of u0, contributions are distributed through the constraints, and
   constrained rows of rhs are left unchanged. Host arrays of n_u + n_p doubles.
   The solve then runs with homogeneous constraints; the caller adds u0 (distributes
   the constraints) afterwards, as the reference does. */
int gb_gmg_correct_stokes_rhs(gb_gmg* h, const double* u0, double* rhs);

/* Free-surface stabilisation of the outer Stokes operator
 * (StokesOperator::local_apply_boundary_face, source/simulator/solver/
 * matrix_free_operators.cc:563-602; table of stokes_matrix_free_local_smoothing.cc:
 * 520-612): on each listed boundary face F of the finest level
 *     dst_u(phi) += int_F -(T . u) (n . phi) dS,   T = rho dt theta |g| g_hat,
 * at the face's QGauss(3) points. Applied by the finest level's outer Stokes
 * operator (FGMRES products, gb_gmg_vmult of GB_GMG_OP_STOKES on the finest level)
 * and by gb_gmg_correct_stokes_rhs; not by the multigrid levels or the A block,
 * as in the reference.
 *   face_cell[i]: caller cell index; face_no[i] = 2*d + side (side 0: xi_d = 0),
 *   at most once per (cell, face).
 *   Points: 3^(dim-1) per face, lexicographic in the face's two tangential
 *   reference axes taken in increasing axis order, the lower axis fastest.
 *   stabilization: [n_faces][points][dim], T at the points;
 *   normal_jxw: [n_faces][points][dim], outward unit normal times the surface
 *   JxW, or NULL: computed from the level's geometry (GB_GMG_GEOM_BOX and
 *   GB_GMG_GEOM_Q2; a GB_GMG_GEOM_TABLE level needs it).
 * n_faces = 0 removes the term. finalize_setup clears it. */
int gb_gmg_set_free_surface(gb_gmg* h, int64_t n_faces, const int32_t* face_cell, const int32_t* face_no,
                            const double* stabilization, const double* normal_jxw);

/* The body-force right-hand side of the finest level on the device
 * (source/simulator/assemblers/stokes.cc:285-400, the rho g . phi_u term):
 * rhs_u = int f . phi_u over QGauss(3), condensed with the velocity constraints
 * as AffineConstraints::distribute_local_to_global does (contributions of a
 * constrained DoF go to the DoFs of its line, constrained rows are zero);
 * the pressure part is zero. force: host array [n_cells][3^dim][dim] (caller
 * cell order, lexicographic points), e.g. rho g at the points; rhs: host array
 * of n_u + n_p doubles (caller numbering), overwritten. */
int gb_gmg_assemble_rhs(gb_gmg* h, const double* force, double* rhs);

/* Same, on device arrays of the finest level in the caller's numbering. */
int gb_gmg_vmult_device(gb_gmg* h, int op, int precision, const double* d_src, double* d_dst);

/* Inverse diagonal of block 0 (A) or 1 (mass) on a level (caller numbering). */
int gb_gmg_get_diagonal_inverse(gb_gmg* h, int level, int block, int precision, double* out);

/* Eigenvalue estimates (min, max) of D^-1 A / D^-1 M on a level. */
int gb_gmg_get_eigenvalues(gb_gmg* h, int level, int block, int precision, double* minmax);
int gb_gmg_set_eigenvalues(gb_gmg* h, int level, int block, int precision, const double* minmax);

/* Level transfer on host arrays: restrict (fine -> coarse, P^T) or prolongate. */
int gb_gmg_transfer(gb_gmg* h, int fine_level, int block, int precision, int restrict_, const double* src,
                    double* dst);

/* One V-cycle (PreconditionMG::vmult) of block 0 (A) or 1 (Schur mass). */
int gb_gmg_vcycle(gb_gmg* h, int block, int precision, const double* src, double* dst);

/* BlockSchurPreconditioner::vmult (block_stokes_preconditioner.h:220-255), cheap variant. */
int gb_gmg_block_preconditioner(gb_gmg* h, int precision, const double* src, double* dst);

/* StokesMatrixFreeHandler::solve (:760-1446): rhs = [F_u; F_p] (condensed),
 * sol = initial guess in / solution out, both [u; p/s] in caller numbering. */
int gb_gmg_solve(gb_gmg* h, const double* rhs, double* sol, const gb_gmg_solve_params* prm,
                 gb_gmg_outputs* out);

/* Same, with rhs/sol already resident in device memory (caller numbering). */
int gb_gmg_solve_device(gb_gmg* h, const double* d_rhs, double* d_sol, const gb_gmg_solve_params* prm,
                        gb_gmg_outputs* out);

/* Adjoint viscosity gradient (no reference counterpart): per finest cell c,
 * g_c = -int_c 2 eta eps(u) : eps(lambda) dx, the derivative of
 * lambda . (F - K u) with respect to ln(eta_c) for cellwise (DGQ0) viscosity,
 * i.e. dJ/d ln(eta_c) when lambda solves K lambda = dJ/du. */
int gb_gmg_adjoint_gradient(gb_gmg* h, const double* u, const double* lambda, double* grad_lneta);

/* Operations timed by gb_gmg_time_operation; the names follow the
 * "Execute solver timings" diagnostics of the reference
 * (stokes_matrix_free_local_smoothing.cc:1116-1260). */
enum gb_gmg_timed_operation {
  GB_GMG_TIME_STOKES_VMULT = 0,          /* stokes_vmult (finest level)          */
  GB_GMG_TIME_A_VMULT = 1,               /* A-block vmult (finest level)         */
  GB_GMG_TIME_MASS_VMULT = 2,            /* pressure mass vmult (finest level)   */
  GB_GMG_TIME_STOKES_PRECONDITIONER = 3, /* stokes_preconditioner (cheap)        */
  GB_GMG_TIME_A_PRECONDITIONER = 4,      /* A_preconditioner (one V-cycle)       */
  GB_GMG_TIME_S_PRECONDITIONER = 5,      /* S_preconditioner (one V-cycle)       */
  GB_GMG_TIME_A_CELL_PASS = 6,           /* A-block cell pass alone (finest)     */
  GB_GMG_TIME_STOKES_CELL_PASS = 7       /* Stokes cell pass alone (finest)      */
};

/* Mean device time of one call of `what` in `precision`, over `repeats` calls
 * after one warm-up call, measured with CUDA events on the library's stream. */
int gb_gmg_time_operation(gb_gmg* h, int what, int precision, int repeats, double* seconds_per_call);

/* Device memory held by the handle (get_*_memory_consumption of stokes_matrix_free.h:80-97);
 * the FP64 levels' work vectors count from their first use. */
int gb_gmg_memory_consumption(const gb_gmg* h, size_t* bytes);

/* Number of kernel launches issued by this handle since creation. */
int64_t gb_gmg_kernel_launches(const gb_gmg* h);

/* Allocation-free FP32 A-block apply (no counterpart in the reference; ASPECT
 * always owns its operator scratch). For callers that cannot call cudaMalloc
 * when they need the operator: code under a device-memory budget owned by
 * another allocator, or code that must not block on the driver's allocator. dst = A src on a uniform lattice box level in the
 * lattice numbering (velocity components blocked, Q2 nodes lexicographic, x
 * fastest; constrained rows act as the identity), with the per-cell scratch in
 * a static device array of GB_GMG_NOALLOC_MAX_CELLS cells (1.33 MB, held by
 * every GPU that loads the library until exit). n_cells_dir[dim]: cells per
 * direction; cell_size[dim]: edge lengths; zero_faces: bit (2*d+side)*3+comp
 * set when velocity component comp is Dirichlet-zero on that face; d_eta:
 * n_cells x eta_per_cell (1 or 3^dim) viscosities in lexicographic cell order;
 * d_eta, d_src and d_dst in device memory, n_cells_dir and cell_size on the
 * host; stream (a cudaStream_t) may be NULL. Larger levels return
 * GB_GMG_EXCEEDS_STATIC_SCRATCH. Calls share the one array: calls whose kernels
 * overlap on the GPU race and must be serialised by the caller. The first call
 * on a device looks up the array's address and keeps it; make it before any
 * stream capture. After cudaDeviceReset the kept address is stale: reload the
 * library first. The result is written asynchronously on `stream`. */
#define GB_GMG_NOALLOC_MAX_CELLS 4096
int gb_gmg_ablock_apply_lattice_noalloc(int dim, const int32_t* n_cells_dir, const double* cell_size,
                                        uint32_t zero_faces, int eta_per_cell, const float* d_eta,
                                        const float* d_src, float* d_dst, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GB_GMG_H */
