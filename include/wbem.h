/*
 * wbem.h - C ABI of the GB300 (sm_103a) collocation BEM library.
 *
 * This is the drop-in boundary under WaveBEM's BEMProblem<3>
 * (include/bem_problem.h:87-180 of the reference). Every entry point takes
 * plain host pointers and sizes, returns an int status (WBEM_OK = 0) and keeps
 * its device memory inside an opaque handle. One handle serves one thread at a
 * time; handles share no state. Nothing here falls back to the CPU: without a
 * usable CUDA device wbem_create fails with WBEM_ERR_CUDA.
 *
 * Conventions (identical to the reference's):
 *   - X[3*i+d]: support point of dof i (reference position plus Eulerian
 *     displacement, i.e. what DoFTools::map_dofs_to_support_points returns with
 *     the MappingQEulerian).
 *   - cells[4*c+k]: dof of local vertex k of cell c in deal.II lexicographic
 *     order (0:(0,0) 1:(1,0) 2:(0,1) 3:(1,1)); the cell normal is
 *     d x/d xi  x  d x/d eta normalised. A cell whose direction_flag() is false
 *     is passed with vertices (0,2,1,3).
 *   - double nodes: CSR (dn_ptr[N+1], dn_idx) with row i = double_nodes_set[i]
 *     in ascending order (source/computational_domain.cc:258-307).
 *   - dirichlet_mask[i] = comp_dom.surface_nodes(i) (1 on Dirichlet nodes);
 *     other_nodes = 1 - surface_nodes.
 *   - tmp_rhs: phi on Dirichlet nodes, dphi/dn on Neumann nodes.
 *   - Matrices exported row-major N x N in the caller's dof order.
 */
#ifndef WBEM_H
#define WBEM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WBEM_OK 0
#define WBEM_ERR_ARG 1        /* invalid argument (sizes, indices, NULL pointers) */
#define WBEM_ERR_STATE 2      /* call out of order (e.g. solve before assemble) */
#define WBEM_ERR_CUDA 3       /* CUDA runtime error / no device */
#define WBEM_ERR_NOMEM 4      /* device allocation failed */
#define WBEM_ERR_SINGULAR 5   /* zero or non-finite pivot */
#define WBEM_ERR_NOCONV 6     /* iterative solver hit max_steps (SolverControl::NoConvergence) */
#define WBEM_ERR_NONFINITE 7  /* non-finite input or result */
#define WBEM_ERR_TIMEOUT 8    /* a bounded device wait gave up */

/* precision forms */
#define WBEM_PREC_FP64 0  /* plain: FP64 everywhere */
#define WBEM_PREC_MIXED 1 /* FP32 far field (double-float panel base + FP32 quadrature deltas),
                             FP64 singular/near field and alpha; (hi, lo) FP32 storage;
                             FP32 LU (TF32 tensor-core updates) or FP32 inner GMRES,
                             refined to full accuracy in FP64 */

/* linear solvers */
#define WBEM_SOLVER_AUTO 0     /* FP64 -> GMRES; MIXED -> LU */
#define WBEM_SOLVER_GMRES 1    /* FP64 GMRES(restart) on the assembled operator, block-Jacobi
                                  preconditioner (either precision) */
#define WBEM_SOLVER_LU 2       /* MIXED only: FP32 dense LU (TF32 tensor-core updates) as the
                                  preconditioner of FP64 GMRES; the factors are reused by every
                                  solve until the next assembly */
#define WBEM_SOLVER_GMRES_IR 3 /* MIXED only: FP64 iterative refinement; each correction is an
                                  inner block-Jacobi GMRES on the FP32 system matrix, run to a
                                  relative residual of 10^-inner_digits */

/* solution methods ("Solution method" of the reference, source/bem_problem.cc:87) */
#define WBEM_METHOD_DIRECT 0 /* dense N and D (either precision form) */
#define WBEM_METHOD_FMA 1    /* fast multipole operators: octree, exact near field (FP64 within
                                two panel diameters, FP32 beyond), Chebyshev-interpolation
                                expansions of order fma_order for the far field; O(N) memory
                                and mat-vec; FP64 GMRES with block-Jacobi on the near field.
                                No matrices to export and no adjoint in this method. */

typedef struct wbem_context* wbem_handle;

typedef struct {
  int precision;                 /* WBEM_PREC_* */
  int solver;                    /* WBEM_SOLVER_* */
  int quadrature_order;          /* "Quadrature order" (Gauss points per direction), 4 */
  int singular_quadrature_order; /* "Singular quadrature order", 5 */
  int gmres_restart;             /* SolverGMRES AdditionalData(100) */
  int max_steps;                 /* SolverControl "Max steps" */
  double tolerance;              /* SolverControl "Tolerance" (absolute, on the residual) */
  double near_field_ratio;       /* MIXED: a panel is near when |x_i - centre| < ratio * diameter */
  int keep_matrices;             /* keep FP64 N (dG/dn) and D (G) for wbem_get_matrices */
  int inner_digits;              /* GMRES_IR: inner relative tolerance 10^-inner_digits, 0 -> 4 */
  int method;                    /* WBEM_METHOD_* ("Solution method"), DIRECT by default */
  int fma_order;                 /* FMA: Chebyshev points per direction of the expansions, 3..8
                                    (6 by default; the far field's error falls about 7x per step) */
  int reserved[4];
} wbem_options;

typedef struct {
  /* FMA: t_assemble_ms is the octree and list build (host wall time), 0 when
     the last build still holds; t_singular_ms the close-pair corrections */
  double t_geometry_ms, t_assemble_ms, t_singular_ms, t_alpha_ms, t_system_ms;
  double t_factor_ms, t_solve_ms, t_adjoint_ms;
  int iterations;           /* GMRES iterations of the last solve */
  double residual;          /* final residual norm of the last solve */
  int kernel_launches;      /* kernels launched by the last assemble+solve */
  int n_dofs, n_cells;
  int outer_iterations;     /* GMRES_IR: refinement steps of the last solve */
  int reserved[7];
} wbem_stats;

/* Defaults of prm-files/default.prm:217-230 plus library choices. */
int wbem_default_options(wbem_options* opt);

/* Create / destroy a handle on CUDA device `device`. */
int wbem_create(wbem_handle* h, int device);
int wbem_destroy(wbem_handle h);
/* Text of the last error of this handle (never NULL). */
const char* wbem_last_error(wbem_handle h);

/*
 * Mesh and double nodes. Replaces the implicit inputs BEMProblem reads from
 * ComputationalDomain: dh/fe/mapping support points, cell dof indices and
 * double_nodes_set (source/bem_problem.cc:168-169, :223-230). dn_ptr/dn_idx
 * may be NULL, in which case the library finds the double nodes itself with
 * the reference's rule (boundary dofs, coincidence below 1e-8). A handle may
 * be given a new mesh at any time; the previous assembly is discarded, and a
 * mesh of another size re-allocates the handle's device buffers.
 */
int wbem_set_geometry(wbem_handle h, const double* X, int n_dofs, const int* cells, int n_cells,
                      const int* dn_ptr, const int* dn_idx);
/* New support points for the same topology (the Eulerian map_points update). */
int wbem_update_nodes(wbem_handle h, const double* X);
/* surface_nodes (1 = Dirichlet). Mutable between solves, like the reference's. */
int wbem_set_bc(wbem_handle h, const unsigned char* dirichlet_mask);

/* BEMProblem::assemble_system + compute_alpha (source/bem_problem.cc:106-618),
 * plus, for the LU solvers, the factorisation of the system. */
int wbem_assemble(wbem_handle h, const wbem_options* opt);

/* BEMProblem::solve_system (source/bem_problem.cc:821-895): unknown entries of
 * phi (Neumann nodes) and dphi_dn (Dirichlet nodes) are written, the others are
 * left untouched. Reuses the current assembly (and its factors). */
int wbem_solve_system(wbem_handle h, const double* tmp_rhs, double* phi, double* dphi_dn);

/* BEMProblem::solve (source/bem_problem.cc:969-987): assemble + solve_system. */
int wbem_solve(wbem_handle h, const wbem_options* opt, const double* tmp_rhs, double* phi,
               double* dphi_dn);

/* alpha (source/bem_problem.cc:594-618), N values. */
int wbem_get_alpha(wbem_handle h, double* alpha);
/* neumann_matrix / dirichlet_matrix (include/bem_problem.h:153-154), row-major
 * N x N, caller order. Needs keep_matrices = 1 (or the FP64 form). Either
 * pointer may be NULL. */
int wbem_get_matrices(wbem_handle h, double* neumann, double* dirichlet);
/* BEMProblem::vmult (source/bem_problem.cc:620-670) and compute_rhs (:673-811). */
int wbem_vmult(wbem_handle h, const double* src, double* dst);
int wbem_compute_rhs(wbem_handle h, const double* src, double* dst);
/* BEMProblem::residual (source/bem_problem.cc:903-961): res = A_c sol - rhs_c
 * of the constrained system, with the known data of (phi, dphi_dn) (phi on
 * Dirichlet nodes, dphi_dn elsewhere) forming the right-hand side and the
 * other entries the solution vector. Uses the current assembly; rebuilds the
 * constraint inhomogeneities from the known data, as a solve does. */
int wbem_residual(wbem_handle h, const double* phi, const double* dphi_dn, double* res);

/* ComputationalDomain::compute_normals (source/computational_domain.cc:1525-1620):
 * the L2 projection onto Q1 of the panel normals (consistent mass matrix),
 * normalised per node. normals: N x 3, caller order. Needs only the geometry. */
int wbem_node_normals(wbem_handle h, double* normals);
/* BEMProblem::compute_surface_gradients (source/bem_problem.cc:1153-1293): the
 * L2 projection onto Q1 of the surface gradient of tmp_rhs * surface_nodes
 * (the Dirichlet data, zero elsewhere). tmp_rhs: N; gradients: N x 3, caller
 * order. These two projections give the inhomogeneities of the sharp
 * Dirichlet-Dirichlet constraint lines. */
int wbem_surface_gradients(wbem_handle h, const double* tmp_rhs, double* gradients);

/* Hull force F = sum over cells hull_cells[k] of  int p n_dir dS,
 * p = -(U . grad phi + |grad phi|^2 / 2) (steady, rho = 1, g = 0 form of
 * source/free_surface.cc:6936-6942); dir = 0,1,2 selects the force component. */
int wbem_hull_force(wbem_handle h, const int* hull_cells, int n_hull, const double* U, int dir,
                    const double* phi, const double* dphi_dn, double* force);

/* Adjoint of assemble + solve_system + hull force, at the current solution of
 * the last wbem_solve / wbem_solve_system with tmp_rhs: returns dF/dX (N x 3,
 * with tmp_rhs held fixed) and dF/dtmp_rhs (N). Reuses the factors for the
 * transposed solve and recomputes matrix tiles (no dG/dX storage). The
 * constraint rows are differentiated too: a Dirichlet-Neumann line through
 * its datum, a sharp Dirichlet-Dirichlet line through the projected normals
 * and surface gradients (node positions and Dirichlet data). */
int wbem_force_adjoint(wbem_handle h, const int* hull_cells, int n_hull, const double* U, int dir,
                       const double* tmp_rhs, double* dF_dX, double* dF_drhs);

/* Adjoint of assemble + solve_system for any objective J(phi, dphi_dn) of the
 * last solution (J with no direct dependence on the node positions): given
 * dJ/dphi and dJ/d(dphi_dn) per node (N each, caller order, both the known and
 * the solved entries), returns dJ/dX (N x 3, tmp_rhs held fixed) and
 * dJ/dtmp_rhs (N). Same transposed solve and tile recomputation as
 * wbem_force_adjoint. No counterpart in the reference.
 * Array lengths (N = n_dofs of the last wbem_set_geometry): dJ_dphi N,
 * dJ_ddn N, dJ_dX 3 N, dJ_drhs N doubles; the library cannot check them. */
int wbem_adjoint(wbem_handle h, const double* dJ_dphi, const double* dJ_ddn, double* dJ_dX,
                 double* dJ_drhs);

int wbem_get_stats(wbem_handle h, wbem_stats* st);

#ifdef __cplusplus
}
#endif
#endif /* WBEM_H */
