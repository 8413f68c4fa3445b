/*
 * nbots FEM hot-path oracle: a plain-C restatement of the reference
 * algorithm on flat arrays.  TEST INFRASTRUCTURE ONLY: tests, the smoke
 * check and the CPU-baseline leg of bench.py call it as the checker; the
 * product (libnbots_gpu.so) never links or calls it.
 *
 * Every function follows the reference step for step (file:line in each
 * comment, paths relative to the nbots source tree) so that, with one
 * thread, its results equal nbots' bit for bit.  It is pinned against the
 * reference library built from its own sources (oracle/Makefile.ref) through
 * the fixtures in tests/golden/.
 */
#ifndef NBOTS_ORACLE_H
#define NBOTS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
	uint32_t nen;           /* 3 (T3) or 4 (Q4) */
	uint32_t N_nod, N_elem, N_edg;
	const double *nod;      /* 2*N_nod */
	const uint32_t *conn;   /* nen*N_elem */
	const uint32_t *edg;    /* 2*N_edg */
} orc_mesh_t;

/* One bc atom in nbots' form (bc_atom.h:7-12).  kind 0 Dirichlet /
 * 1 Neumann, where 0 vertex / 1 segment.  node_vals (n_nv x 2) holds a
 * function-valued atom already evaluated where nbots evaluates it. */
typedef struct {
	uint32_t kind, where, id;
	uint8_t mask[2];
	double val[2];
	uint32_t n_nv;
	const double *node_vals;
} orc_bc_t;

typedef struct {
	const uint32_t *vtx;          /* input vertex -> node */
	uint32_t N_sgm;
	const uint32_t *sgm_ptr;      /* N_sgm+1 offsets into sgm_nodes */
	const uint32_t *sgm_nodes;
	uint32_t N_bc;
	const orc_bc_t *bc;
} orc_bcs_t;

/* CSR pattern of nb_sparse_create(graph(NODES_LINKED_BY_ELEMS), NULL, 2).
 * With col_idx == NULL only row_ptr (2*N_nod+1) is filled. */
int orc_pattern(const orc_mesh_t *m, uint32_t *row_ptr, uint32_t *col_idx);

/* pipeline_assemble_system with one Young's modulus per element.
 * Returns 0, or 1 when an element is distorted (detJ < 0). */
int orc_assemble(const orc_mesh_t *m, const uint32_t *row_ptr,
		 const uint32_t *col_idx, const double *E, double nu,
		 double thickness, double density, int self_weight,
		 const double gravity[2], const uint8_t *enabled,
		 double *K, double *F);

/* Element stiffness of one element (row-major 2nen x 2nen) and its load
 * vector; returns 1 for a distorted element. */
int orc_element(const orc_mesh_t *m, uint32_t e, double E, double nu,
		double thickness, double density, int self_weight,
		const double gravity[2], int enabled, double *Ke, double *Fe);

/* nb_fem_set_bconditions with factor 1 (set_bconditions.c:52-61). */
void orc_set_bconditions(const orc_mesh_t *m, const orc_bcs_t *b,
			 const uint32_t *row_ptr, const uint32_t *col_idx,
			 double *K, double *F, double factor);

void orc_set_dirichlet(const uint32_t *row_ptr, const uint32_t *col_idx,
		       double *K, double *F, uint32_t idx, double value);

void orc_spmv(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
	      const double *K, const double *x, double *y, int threads);

int orc_cg_jacobi(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
		  const double *K, const double *b, double *x, uint32_t max_iter,
		  double tol, uint32_t *niter, double *tol_reached, int threads);

int orc_cg(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
	   const double *K, const double *b, double *x, uint32_t max_iter,
	   double tol, uint32_t *niter, double *tol_reached, int threads);

void orc_strain(const orc_mesh_t *m, const double *u, double *strain);
void orc_stress(const orc_mesh_t *m, const double *E, double nu,
		const uint8_t *enabled, const double *strain, double *stress);

/* SIMP element sensitivities: out[e] = -dE(rho_e) * a_e^T Ke0_e b_e, where
 * Ke0_e is the element stiffness for E = 1 and
 * dE = p rho^(p-1) (E0 - Emin).  a = b = u gives compliance; a = lambda
 * (adjoint) and b = u gives one nodal output.  No counterpart in nbots. */
void orc_main_stress(uint32_t n_points, const double *stress, double *main_stress);
int orc_gauss_seidel(uint32_t N, const uint32_t *rp, const uint32_t *ci, const double *K,
		     const double *b, double *x, uint32_t max_iter, double tol,
		     uint32_t *niter, double *tol_reached);
double orc_tension_damage(double E, double nu, double ft, double gf, const double *strain,
			  double r_prev, double *r, double clfd);
int orc_damage_solve(const orc_mesh_t *m, const orc_bcs_t *b, double E, double nu,
		     double thickness, double density, int self_weight, const double gravity[2],
		     double ft, double gf, uint32_t n_steps, uint32_t max_iter,
		     uint32_t max_iter_noenh, double rtol, char *log, size_t cap,
		     double *u_out, double *damage_out);
void orc_simp_sensitivity(const orc_mesh_t *m, double nu, double thickness,
			  const double *rho, double penal, double E0, double Emin,
			  const double *a, const double *b, double *out);

/* Seconds of wall time (omp_get_wtime when OpenMP is on). */
double orc_wtime(void);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
