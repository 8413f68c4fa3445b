/*
 * Drop-in replacements for nbots' FEM hot path (vecn/nbots), implemented in
 * libnbots_gpu.so on the sm_103a kernels of include/nbots_gb300.h.
 *
 * Link libnbots_gpu.so ahead of libnbots.so (or LD_PRELOAD it): the symbols
 * below then resolve to the GPU versions for every caller, including calls
 * from inside libnbots, while the rest of nbots keeps working.  The
 * signatures, argument meanings and return codes are nbots' own; each
 * declaration cites the reference it replaces (paths relative to the nbots
 * tree).  Differences are listed where they exist.
 *
 * The FEM entry reads meshes, boundary conditions, materials and element
 * types only through nbots' public accessors (declared at the end).  Those
 * come from libnbots.so in a real deployment; libnbots_host.so provides a
 * standalone implementation of the same accessors (plus array constructors,
 * nbh_*) for programs and tests without nbots.
 */
#ifndef NBOTS_DROPIN_H
#define NBOTS_DROPIN_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------- nbots types */
/* headers/nb/graph_bot/graph.h:25-31 (public struct) */
typedef struct {
	uint32_t N;
	uint32_t *N_adj;
	uint32_t **adj;
	double *wi;
	double **wij;
} nb_graph_t;

/* sources/nb/solver_bot/sparse/sparse_struct.h:6-11; the drop-in keeps this
 * layout (rows of pointers) so code that walks rows directly still works.
 * nb_sparse_create backs all rows with two contiguous slabs, which the GPU
 * path uploads without copying row by row. */
typedef struct nb_sparse_s {
	double **rows_values;
	uint32_t **rows_index;
	uint32_t *rows_size;
	uint32_t N;
} nb_sparse_t;

/* opaque nbots objects (headers/nb/geometric_bot/mesh/mesh2D.h:14,
 * headers/nb/pde_bot/boundary_conditions/bcond.h:17,
 * headers/nb/pde_bot/material.h, headers/nb/pde_bot/finite_element/element.h:6) */
typedef struct nb_mesh2D_s nb_mesh2D_t;
typedef struct nb_bcond_s nb_bcond_t;
typedef struct nb_bcond_iter_s nb_bcond_iter_t;
typedef struct nb_material_s nb_material_t;
typedef struct nb_fem_elem_s nb_fem_elem_t;

typedef enum { NB_DIRICHLET, NB_NEUMANN } nb_bcond_id;           /* bcond.h:7-10 */
typedef enum { NB_BC_ON_POINT, NB_BC_ON_SEGMENT } nb_bcond_where; /* bcond.h:12-15 */
typedef enum { NB_TRG_LINEAR, NB_QUAD_LINEAR } nb_elem_id;        /* element.h:8-11 */
typedef enum {                                                    /* analysis2D.h:4-8 */
	NB_PLANE_STRESS,
	NB_PLANE_STRAIN,
	NB_SOLID_OF_REVOLUTION
} nb_analysis2D_t;
typedef struct {                                                  /* analysis2D.h:10-14 */
	double thickness;
	double revolution_axe;
	char revolution_coordinate;
} nb_analysis2D_params;

/* ------------------------------------------------------- replaced: sparse */
/* sparse.h:28-30, sparse.c:20-60 */
nb_sparse_t *nb_sparse_create(const nb_graph_t *graph, const uint32_t *perm,
			      uint32_t vars_per_node);
/* sparse.h:32, sparse.c:78-95 */
nb_sparse_t *nb_sparse_clone(nb_sparse_t *A);
/* sparse.h:34, sparse.c:114-125: also frees rows other code allocated */
void nb_sparse_destroy(nb_sparse_t *A);
void nb_sparse_reset(nb_sparse_t *A);                                    /* sparse.c:127-132 */
/* sparse.c:134-171, 186-219: per-row binary search (sparse_struct.c:7-20).
 * nbots exits on a missing entry; the drop-in prints the same message,
 * records the error (nbg_dropin_error) and leaves the matrix unchanged. */
void nb_sparse_set(nb_sparse_t *A, uint32_t i, uint32_t j, double value);
double nb_sparse_get(const nb_sparse_t *A, uint32_t i, uint32_t j);
double nb_sparse_get_and_set(nb_sparse_t *A, uint32_t i, uint32_t j, double value);
bool nb_sparse_is_non_zero(const nb_sparse_t *A, uint32_t i, uint32_t j);
void nb_sparse_add(nb_sparse_t *A, uint32_t i, uint32_t j, double value);
uint32_t nb_sparse_get_size(const nb_sparse_t *A);                      /* sparse.c:342-345 */
uint32_t nb_sparse_get_nnz(const nb_sparse_t *A);                       /* sparse.c:348-354 */
/* sparse.h:54-55, sparse.c:405-414: y = A x on the GPU in nbots' per-row
 * order without FMA, so the result is bit-identical.  omp_parallel_threads
 * is accepted and ignored. */
void nb_sparse_multiply_vector(const nb_sparse_t *A, const double *in, double *out,
			       uint32_t omp_parallel_threads);
/* sparse.h:58-59, sparse.c:416-430 (host side, same order) */
void nb_sparse_set_Dirichlet_condition(nb_sparse_t *A, double *RHS, uint32_t idx,
				       double value);
/* The remaining writers of sparse.h (sparse.c:148-162, 221-227, 289-347,
 * 394-403), replaced so that the drop-in sees every write to a matrix it
 * keeps a device copy of.  The first four run here; transpose,
 * get_transpose and fill_permutation forward to the next definition in link
 * order (nbots' own) and record NBG_ERR_ARG when there is none. */
void nb_sparse_set_identity_row(nb_sparse_t *A, uint32_t row);
void nb_sparse_make_diagonal(nb_sparse_t *A, double diag_val);
void nb_sparse_scale(nb_sparse_t *A, double factor);
void nb_sparse_multiply_scalar(nb_sparse_t *A, double scalar, uint32_t omp_parallel_threads);
void nb_sparse_transpose(nb_sparse_t *A);
void nb_sparse_get_transpose(const nb_sparse_t *A, nb_sparse_t *At);
void nb_sparse_fill_permutation(const nb_sparse_t *A, nb_sparse_t *Ar, const uint32_t *perm,
				const uint32_t *iperm);

/* Device copies.  A matrix made by nb_sparse_create / nb_sparse_clone keeps
 * its pattern, values and block layout on the GPU from one
 * nb_sparse_multiply_vector / nb_sparse_solve_* call to the next; the
 * functions above mark it changed, so the next GPU call re-sends the values
 * (the pattern never changes), and nb_sparse_destroy frees the copy.  Code
 * that writes rows_values directly calls nbg_dropin_sparse_touch(A) before
 * the next GPU call, and so does code that points a row at other memory.
 * NBG_DROPIN_CACHE_MB (default 16384) bounds the device
 * memory of all copies (least recently used dropped first; 0: no copies).
 * Matrices nbots allocated itself are sent whole on every call. */
void nbg_dropin_sparse_touch(const nb_sparse_t *A);

/* ------------------------------------------------------- replaced: solvers */
/* headers/nb/solver_bot/sparse/solvers/cg_precond_jacobi.h:8-15,
 * cg_precond_jacobi.c:13-90: nbots' iteration (g = Ax - b, absolute tolerance,
 * lagged stop test) in one persistent GPU kernel, on the 2x2-block layout
 * with FMAs when the pattern is node-blocked (nb_sparse_create(.., 2)), else
 * on the CSR with nbots' arithmetic; NBG_DROPIN_EXACT_CG=1 selects the CSR
 * form always.  Returns 0 or 1 (tolerance not reached) like nbots, or a
 * negative nbg status on a GPU error. */
int nb_sparse_solve_CG_precond_Jacobi(const nb_sparse_t *A, const double *b, double *x,
				      uint32_t max_iter, double tolerance,
				      uint32_t *niter_performed, double *tolerance_reached,
				      uint32_t omp_parallel_threads);
/* solvers/conjugate_gradient.h, conjugate_gradient.c:13-77 */
int nb_sparse_solve_conjugate_gradient(const nb_sparse_t *A, const double *b, double *x,
				       uint32_t max_iter, double tolerance,
				       uint32_t *niter_performed, double *tolerance_reached,
				       uint32_t omp_parallel_threads);

/* ---------------------------------------------------------- replaced: FEM */
/* headers/nb/pde_bot/finite_element/solid_mechanics/static_elasticity2D.h:13-24,
 * static_elasticity2D.c:31-97: pattern, assembly, boundary conditions,
 * Jacobi-PCG (x0 = 0, max_iter = N, tol 1e-8) and strain, all on the GPU.
 * Returns 0, 1 (distorted element) like nbots, or a negative nbg status.
 * Like nbots, every analysis type is computed as plane stress (the switch in
 * formulas.c:32-46 falls through). */
int nb_fem_compute_2D_Solid_Mechanics(const nb_mesh2D_t *part, const nb_fem_elem_t *elemtype,
				      const nb_material_t *material, const nb_bcond_t *bcond,
				      bool enable_self_weight, double gravity[2],
				      nb_analysis2D_t analysis2D, nb_analysis2D_params *params2D,
				      const bool *elements_enabled, double *displacement,
				      double *strain);
/* static_elasticity2D.h:26-32, static_elasticity2D.c:99-127 */
void nb_fem_compute_stress_from_strain(uint32_t N_elements, const nb_fem_elem_t *elemtype,
				       const nb_material_t *material, nb_analysis2D_t analysis2D,
				       double *strain, const bool *elements_enabled,
				       double *stress);

/* The stages of the FEM entry, for nbots programs that drive them
 * themselves (create, assemble, boundary conditions, solve, strain).  K must
 * be a matrix of nb_sparse_create(nodal graph, NULL, 2) on the same mesh
 * (any other goes to the next definition in link order, nbots' own, or
 * fails with NBG_ERR_ARG when there is none).  Each stage runs on the
 * matrix's device copy and writes K and F back to the caller's arrays, bit
 * for bit what nbots' serial stage writes; the device copy stays current, so
 * the solve that follows sends only the vectors.
 * pipeline.h:21-31, pipeline.c:42-73, 83-264: element stiffness and load in
 * nbots' operation order, summed per matrix entry in element order.  With a
 * lumped mass vector M (not NULL) the call goes to nbots' own stage.
 * Returns 0, 1 (distorted element; K and F are left reset, where nbots
 * leaves them partly summed) or a negative nbg status. */
int pipeline_assemble_system(nb_sparse_t *K, double *M, double *F, const nb_mesh2D_t *part,
			     const nb_fem_elem_t *elemtype, const nb_material_t *material,
			     bool enable_self_weight, double gravity[2],
			     nb_analysis2D_t analysis2D, nb_analysis2D_params *params2D,
			     const bool *elements_enabled);
/* set_bconditions.h:8-11, set_bconditions.c:52-260: Neumann on segments and
 * vertices, then Dirichlet on segments and vertices, in push order. */
void nb_fem_set_bconditions(const nb_mesh2D_t *part, nb_sparse_t *K, double *F,
			    const nb_bcond_t *bcond, double factor);
/* pipeline.h:36-39, pipeline.c:266-319: strain at every Gauss point. */
void pipeline_compute_strain(double *strain, const nb_mesh2D_t *part, double *displacement,
			     const nb_fem_elem_t *elemtype);

/* pipeline.h:42-45, pipeline.c:321-340: principal stresses (sx + sy)/2 +-
 * sqrt((sx - sy)^2/4 + txy^2) per Gauss point, bit-exact. */
void pipeline_compute_main_stress(double *stress, double *main_stress, uint32_t N_elements,
				  const nb_fem_elem_t *const elem);

/* static_damage2D.h:13-32 (opaque in nbots; accessors below) */
typedef struct nb_fem_implicit_s nb_fem_implicit_t;

/* static_damage2D.h:34-45, static_damage2D.c:239-470: quasi-static damage
 * solve, conjugate-gradient branch on the GPU (assembly with damage,
 * boundary conditions, residual, Jacobi-PCG with Gauss-Seidel fallback,
 * strain and damage), nbots' log lines appended to `logfile`.  With
 * enable_Cholesky_solver the call goes to the next definition in link order
 * (nbots' own) when there is one, else it runs the conjugate-gradient
 * branch.  Like nbots, every analysis type is computed as plane stress. */
void nb_fem_compute_2D_Non_Linear_Solid_Mechanics(const nb_mesh2D_t *part,
						  const nb_fem_elem_t *elem,
						  const nb_material_t *material,
						  const nb_bcond_t *bcond, bool enable_self_weight,
						  double gravity[2], bool enable_Cholesky_solver,
						  nb_analysis2D_t analysis2D,
						  nb_analysis2D_params *params2D,
						  nb_fem_implicit_t *params, const char *logfile);

/* A/B switch: with NBG_DROPIN_CPU=1 in the environment every replaced
 * compute entry (SpMV, the two CGs, the FEM entries, stress, principal
 * stresses, the damage solve) calls the next definition of its symbol in
 * link order -- nbots' own CPU code when libnbots.so follows this library --
 * on the same objects.  Unset (the default) the GPU path runs.  Set, with no
 * next definition loaded, the call fails with NBG_ERR_ARG. */
int nbg_dropin_cpu(void);

/* Last error of a drop-in call that nbots would have ended with exit(1)
 * (0 if none); cleared by reading. */
int nbg_dropin_error(void);

/* ---------------------------------------- consumed: nbots public accessors */
uint32_t nb_mesh2D_get_N_nodes(const nb_mesh2D_t *mesh);
uint32_t nb_mesh2D_get_N_edges(const nb_mesh2D_t *mesh);
uint32_t nb_mesh2D_get_N_elems(const nb_mesh2D_t *mesh);
uint32_t nb_mesh2D_get_N_invtx(const nb_mesh2D_t *mesh);
uint32_t nb_mesh2D_get_N_insgm(const nb_mesh2D_t *mesh);
double nb_mesh2D_node_get_x(const nb_mesh2D_t *mesh, uint32_t id);
double nb_mesh2D_node_get_y(const nb_mesh2D_t *mesh, uint32_t id);
uint32_t nb_mesh2D_edge_get_1n(const nb_mesh2D_t *mesh, uint32_t id);
uint32_t nb_mesh2D_edge_get_2n(const nb_mesh2D_t *mesh, uint32_t id);
uint32_t nb_mesh2D_elem_get_N_adj(const nb_mesh2D_t *mesh, uint32_t id);
uint32_t nb_mesh2D_elem_get_adj(const nb_mesh2D_t *mesh, uint32_t elem_id, uint8_t adj_id);
uint32_t nb_mesh2D_get_invtx(const nb_mesh2D_t *mesh, uint32_t id);
uint32_t nb_mesh2D_insgm_get_N_nodes(const nb_mesh2D_t *mesh, uint32_t id);
uint32_t nb_mesh2D_insgm_get_node(const nb_mesh2D_t *mesh, uint32_t sgm_id, uint32_t node_id);

uint16_t nb_bcond_iter_get_memsize(void);
void nb_bcond_iter_init(void *iter_ptr);
void nb_bcond_iter_finish(void *iter_ptr);
void nb_bcond_iter_set_conditions(nb_bcond_iter_t *iter, const nb_bcond_t *bcond,
				  nb_bcond_id type_id, nb_bcond_where type_elem);
bool nb_bcond_iter_has_more(const nb_bcond_iter_t *iter);
void nb_bcond_iter_go_next(nb_bcond_iter_t *iter);
uint32_t nb_bcond_iter_get_id(const nb_bcond_iter_t *iter);
bool nb_bcond_iter_get_mask(const nb_bcond_iter_t *iter, uint8_t dof_id);
bool nb_bcond_iter_val_is_function(const nb_bcond_iter_t *iter);
void nb_bcond_iter_get_val(const nb_bcond_iter_t *iter, uint8_t N_dof, double *x, double t,
			   double val[]);
uint8_t nb_bcond_get_N_dof(const nb_bcond_t *bcond);

double nb_material_get_elasticity_module(const nb_material_t *mat);
double nb_material_get_poisson_module(const nb_material_t *mat);
double nb_material_get_density(const nb_material_t *mat);
double nb_material_get_traction_limit_stress(const nb_material_t *mat);
double nb_material_get_fracture_energy(const nb_material_t *mat);

nb_fem_implicit_t *nb_fem_implicit_create(void);
void nb_fem_implicit_destroy(nb_fem_implicit_t *isparams);
void nb_fem_implicit_set_N_steps(nb_fem_implicit_t *isparams, uint32_t N_steps);
void nb_fem_implicit_set_N_max_iter(nb_fem_implicit_t *isparams, uint32_t N_max_iter);
void nb_fem_implicit_set_N_max_iter_without_enhance(nb_fem_implicit_t *isparams,
						    uint32_t N_max_iter);
void nb_fem_implicit_set_residual_tolerance(nb_fem_implicit_t *isparams, double tol);
uint32_t nb_fem_implicit_get_N_steps(nb_fem_implicit_t *isparams);
uint32_t nb_fem_implicit_get_N_max_iter(nb_fem_implicit_t *isparams);
uint32_t nb_fem_implicit_get_N_max_iter_without_enhance(nb_fem_implicit_t *isparams);
double nb_fem_implicit_get_residual_tolerance(nb_fem_implicit_t *isparams);

uint8_t nb_fem_elem_get_N_nodes(const nb_fem_elem_t *elemtype);
uint8_t nb_fem_elem_get_N_gpoints(const nb_fem_elem_t *elemtype);

#ifdef __cplusplus
}
#endif
#endif
