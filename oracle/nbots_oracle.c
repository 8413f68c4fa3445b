/*
 * nbots FEM hot-path oracle (test infrastructure, see nbots_oracle.h).
 *
 * Built with -std=c99 so GCC keeps -ffp-contract=off, the same arithmetic
 * as nbots' own build (CMakeLists.txt:33): no fused multiply-adds anywhere.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "nbots_oracle.h"

/* ------------------------------------------------------------------
 * Element tables.  The Q4 values are nbots' own 12-significant-digit
 * truncations (pde_bot/finite_element/element.c:75-121): bit parity of the
 * stiffness depends on using them, not the exact Gauss values.  Layout is
 * node-major, [node * N_gp + gp]; the Gauss points run (-,-), (+,-),
 * (+,+), (-,+).
 * ------------------------------------------------------------------ */
#define QA 0.622008467928
#define QB 0.166666666667
#define QC 0.044658198739
#define QD 0.394337567297
#define QE 0.105662432703
static const double q4_N[16] = {QA, QB, QC, QB,  QB, QA, QB, QC,
				QC, QB, QA, QB,  QB, QC, QB, QA};
static const double q4_dpsi[16] = {-QD, -QD, -QE, -QE,  QD, QD, QE, QE,
				   QE, QE, QD, QD,  -QE, -QE, -QD, -QD};
static const double q4_deta[16] = {-QD, -QE, -QE, -QD,  -QE, -QD, -QD, -QE,
				   QE, QD, QD, QE,  QD, QE, QE, QD};
static const double q4_w[4] = {1.0, 1.0, 1.0, 1.0};
/* T3: one Gauss point (element.c:54-73) */
static const double t3_N[3] = {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0};
static const double t3_dpsi[3] = {-1.0, 1.0, 0.0};
static const double t3_deta[3] = {-1.0, 0.0, 1.0};
static const double t3_w[1] = {0.5};

typedef struct {
	int nn, ngp;
	const double *N, *dpsi, *deta, *w;
} tab_t;

static tab_t table(uint32_t nen)
{
	tab_t t;
	if (nen == 4) {
		t.nn = 4; t.ngp = 4; t.N = q4_N; t.dpsi = q4_dpsi; t.deta = q4_deta; t.w = q4_w;
	} else {
		t.nn = 3; t.ngp = 1; t.N = t3_N; t.dpsi = t3_dpsi; t.deta = t3_deta; t.w = t3_w;
	}
	return t;
}

double orc_wtime(void)
{
#ifdef _OPENMP
	return omp_get_wtime();
#else
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + 1e-9 * ts.tv_nsec;
#endif
}

int orc_max_threads(void)
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

static int cmp_u32(const void *a, const void *b)
{
	uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
	return x < y ? -1 : (x > y);
}

/* ------------------------------------------------------------------
 * Pattern: nodal graph of load_graph_nodes_by_elems
 * (geometric_bot/mesh/mesh2D/load_graph.c:230-328): both directions of every
 * mesh edge, then for each element with more than 3 nodes the links
 * i -> (i+j+2) % n for j < n-3; then nb_sparse_create (solver_bot/sparse/
 * sparse.c:20-60): per node two rows of (N_adj+1)*2 columns, neighbours
 * then self, expanded by the two dofs and sorted ascending.
 * ------------------------------------------------------------------ */
int orc_pattern(const orc_mesh_t *m, uint32_t *row_ptr, uint32_t *col_idx)
{
	uint32_t Nn = m->N_nod;
	uint32_t *nadj = calloc(Nn ? Nn : 1, sizeof(uint32_t));
	if (!nadj)
		return -1;
	for (uint32_t i = 0; i < m->N_edg; i++) {
		nadj[m->edg[2 * i]]++;
		nadj[m->edg[2 * i + 1]]++;
	}
	if (m->nen > 3)
		for (uint32_t e = 0; e < m->N_elem; e++)
			for (uint32_t i = 0; i < m->nen; i++)
				nadj[m->conn[e * m->nen + i]] += m->nen - 3;
	row_ptr[0] = 0;
	for (uint32_t i = 0; i < Nn; i++) {
		uint32_t rs = (nadj[i] + 1) * 2;
		row_ptr[2 * i + 1] = row_ptr[2 * i] + rs;
		row_ptr[2 * i + 2] = row_ptr[2 * i + 1] + rs;
	}
	if (!col_idx) {
		free(nadj);
		return 0;
	}
	uint32_t *aptr = malloc(((size_t)Nn + 1) * sizeof(uint32_t));
	aptr[0] = 0;
	for (uint32_t i = 0; i < Nn; i++)
		aptr[i + 1] = aptr[i] + nadj[i];
	uint32_t *adj = malloc(((size_t)aptr[Nn] + 1) * sizeof(uint32_t));
	memset(nadj, 0, Nn * sizeof(uint32_t));
	for (uint32_t i = 0; i < m->N_edg; i++) {
		uint32_t a = m->edg[2 * i], b = m->edg[2 * i + 1];
		adj[aptr[a] + nadj[a]++] = b;
		adj[aptr[b] + nadj[b]++] = a;
	}
	if (m->nen > 3)
		for (uint32_t e = 0; e < m->N_elem; e++)
			for (uint32_t i = 0; i < m->nen; i++) {
				uint32_t id1 = m->conn[e * m->nen + i];
				for (uint32_t j = 0; j < m->nen - 3; j++) {
					uint32_t k = (i + j + 2) % m->nen;
					adj[aptr[id1] + nadj[id1]++] = m->conn[e * m->nen + k];
				}
			}
	for (uint32_t i = 0; i < Nn; i++)
		for (uint32_t k1 = 0; k1 < 2; k1++) {
			uint32_t *row = col_idx + row_ptr[2 * i + k1];
			for (uint32_t j = 0; j < nadj[i]; j++)
				for (uint32_t k2 = 0; k2 < 2; k2++)
					row[j * 2 + k2] = adj[aptr[i] + j] * 2 + k2;
			row[nadj[i] * 2] = 2 * i;
			row[nadj[i] * 2 + 1] = 2 * i + 1;
			qsort(row, (nadj[i] + 1) * 2, sizeof(uint32_t), cmp_u32);
		}
	free(adj);
	free(aptr);
	free(nadj);
	return 0;
}

/* nb_sparse_bsearch_row (solver_bot/sparse/sparse_struct.c:7-20) */
static uint32_t bsearch_row(const uint32_t *cols, uint32_t size, uint32_t col)
{
	int imin = 0, imax = (int)size - 1;
	uint32_t index = (uint32_t)((imin + imax) / 2);
	while (cols[index] != col && imin <= imax) {
		index = (uint32_t)((imin + imax) / 2);
		if (cols[index] < col)
			imin = index + 1;
		else
			imax = index - 1;
	}
	return index;
}

static double *slot(const uint32_t *row_ptr, const uint32_t *col_idx, double *K,
		    uint32_t i, uint32_t j)
{
	uint32_t b = row_ptr[i];
	uint32_t k = bsearch_row(col_idx + b, row_ptr[i + 1] - b, j);
	return col_idx[b + k] == j ? &K[b + k] : NULL;
}

/* set_plane_stress (pde_bot/common_solid_mechanics/formulas.c:48-54); the
 * switch in nb_pde_get_constitutive_matrix (:32-46) has no breaks, so every
 * analysis type lands here. */
static void plane_stress(double D[4], double E, double v)
{
	D[0] = E / (1.0 - v * v);
	D[1] = v * D[0];
	D[2] = D[0];
	D[3] = E / (2.0 * (1.0 + v));
}

/* nb_fem_get_jacobian (pde_bot/finite_element/utils.c:9-41) */
static double jacobian(const orc_mesh_t *m, const tab_t *t, uint32_t e, int gp,
		       double Jinv[4])
{
	double dx_dpsi = 0.0, dy_dpsi = 0.0, dx_deta = 0.0, dy_deta = 0.0;
	for (int i = 0; i < t->nn; i++) {
		uint32_t n = m->conn[e * m->nen + i];
		double xi = m->nod[2 * n], yi = m->nod[2 * n + 1];
		double dp = t->dpsi[i * t->ngp + gp], de = t->deta[i * t->ngp + gp];
		dx_dpsi += dp * xi;
		dx_deta += de * xi;
		dy_dpsi += dp * yi;
		dy_deta += de * yi;
	}
	double detJ = dx_dpsi * dy_deta - dy_dpsi * dx_deta;
	Jinv[0] = dy_deta / detJ;
	Jinv[1] = -dy_dpsi / detJ;
	Jinv[2] = -dx_deta / detJ;
	Jinv[3] = dx_dpsi / detJ;
	return detJ;
}

/* nb_fem_get_derivatives (utils.c:49-60) */
static void derivatives(const tab_t *t, int gp, const double Jinv[4],
			double *dx, double *dy)
{
	for (int i = 0; i < t->nn; i++) {
		double dp = t->dpsi[i * t->ngp + gp], de = t->deta[i * t->ngp + gp];
		dx[i] = Jinv[0] * dp + Jinv[1] * de;
		dy[i] = Jinv[2] * dp + Jinv[3] * de;
	}
}

/* assemble_element + integrate_elemental_system + pipeline_sum_gauss_point
 * (pde_bot/finite_element/solid_mechanics/pipeline.c:83-230), without the
 * mass matrix (the FEM entry passes M = NULL). */
static int element_dmg(const orc_mesh_t *m, uint32_t e, double E, double nu,
		       double thickness, double density, int self_weight,
		       const double gravity[2], int enabled, const double *dmg,
		       double *Ke, double *Fe);

int orc_element(const orc_mesh_t *m, uint32_t e, double E, double nu,
		double thickness, double density, int self_weight,
		const double gravity[2], int enabled, double *Ke, double *Fe)
{
	return element_dmg(m, e, E, nu, thickness, density, self_weight, gravity, enabled,
			   NULL, Ke, Fe);
}

/* With dmg != NULL, the constitutive matrix of Gauss point gp is scaled by
 * (1 - dmg[gp]) first (DMG_pipeline_assemble_system,
 * static_damage2D.c:527-534). */
static int element_dmg(const orc_mesh_t *m, uint32_t e, double E, double nu,
		       double thickness, double density, int self_weight,
		       const double gravity[2], int enabled, const double *dmg,
		       double *Ke, double *Fe)
{
	tab_t t = table(m->nen);
	int n2 = 2 * t.nn;
	double D[4] = {1e-6, 1e-6, 1e-6, 1e-6};
	double dens = 1e-6;
	if (enabled) {
		plane_stress(D, E, nu);
		dens = density;
	}
	double fx = 0.0, fy = 0.0;
	if (self_weight) {
		fx = gravity[0] * dens;
		fy = gravity[1] * dens;
	}
	memset(Ke, 0, sizeof(double) * n2 * n2);
	memset(Fe, 0, sizeof(double) * n2);
	double dx[4], dy[4];
	for (int gp = 0; gp < t.ngp; gp++) {
		double Dg[4] = {D[0], D[1], D[2], D[3]};
		if (dmg)
			for (int k = 0; k < 4; k++)
				Dg[k] *= (1.0 - dmg[gp]);
		double Jinv[4];
		double detJ = jacobian(m, &t, e, gp, Jinv);
		if (detJ < 0)
			return 1;
		derivatives(&t, gp, Jinv, dx, dy);
		double wp = t.w[gp];
		for (int i = 0; i < t.nn; i++) {
			double Ni = t.N[i * t.ngp + gp];
			for (int j = 0; j < t.nn; j++) {
				Ke[(2 * i) * n2 + 2 * j] +=
					(dx[i] * dx[j] * Dg[0] + dy[i] * dy[j] * Dg[3]) *
					detJ * thickness * wp;
				Ke[(2 * i) * n2 + 2 * j + 1] +=
					(dx[i] * dy[j] * Dg[1] + dy[i] * dx[j] * Dg[3]) *
					detJ * thickness * wp;
				Ke[(2 * i + 1) * n2 + 2 * j] +=
					(dy[i] * dx[j] * Dg[1] + dx[i] * dy[j] * Dg[3]) *
					detJ * thickness * wp;
				Ke[(2 * i + 1) * n2 + 2 * j + 1] +=
					(dy[i] * dy[j] * Dg[2] + dx[i] * dx[j] * Dg[3]) *
					detJ * thickness * wp;
			}
			double integral = Ni * detJ * thickness * wp;
			Fe[2 * i] += integral * fx;
			Fe[2 * i + 1] += integral * fy;
		}
	}
	return 0;
}

/* pipeline_assemble_system (pipeline.c:42-73): serial element loop in id
 * order, scatter through the per-row binary search of nb_sparse_add
 * (sparse.c:207-219) in the order of pipeline_add_to_global_system
 * (pipeline.c:232-264). */
int orc_assemble(const orc_mesh_t *m, const uint32_t *row_ptr,
		 const uint32_t *col_idx, const double *E, double nu,
		 double thickness, double density, int self_weight,
		 const double gravity[2], const uint8_t *enabled,
		 double *K, double *F)
{
	uint32_t N = 2 * m->N_nod;
	memset(K, 0, sizeof(double) * row_ptr[N]);
	memset(F, 0, sizeof(double) * N);
	int nn = (int)m->nen, n2 = 2 * nn;
	double Ke[64], Fe[8];
	for (uint32_t e = 0; e < m->N_elem; e++) {
		int en = enabled ? enabled[e] != 0 : 1;
		if (orc_element(m, e, E[e], nu, thickness, density, self_weight,
				gravity, en, Ke, Fe))
			return 1;
		for (int i = 0; i < nn; i++) {
			uint32_t v1 = m->conn[e * m->nen + i];
			for (int j = 0; j < nn; j++) {
				uint32_t v2 = m->conn[e * m->nen + j];
				double *s;
				if (!(s = slot(row_ptr, col_idx, K, 2 * v1, 2 * v2))) return 2;
				*s += Ke[(2 * i) * n2 + 2 * j];
				if (!(s = slot(row_ptr, col_idx, K, 2 * v1 + 1, 2 * v2))) return 2;
				*s += Ke[(2 * i + 1) * n2 + 2 * j];
				if (!(s = slot(row_ptr, col_idx, K, 2 * v1, 2 * v2 + 1))) return 2;
				*s += Ke[(2 * i) * n2 + 2 * j + 1];
				if (!(s = slot(row_ptr, col_idx, K, 2 * v1 + 1, 2 * v2 + 1))) return 2;
				*s += Ke[(2 * i + 1) * n2 + 2 * j + 1];
			}
			F[2 * v1] += Fe[2 * i];
			F[2 * v1 + 1] += Fe[2 * i + 1];
		}
	}
	return 0;
}

/* nb_sparse_set_Dirichlet_condition (sparse.c:416-430) */
void orc_set_dirichlet(const uint32_t *row_ptr, const uint32_t *col_idx,
		       double *K, double *F, uint32_t idx, double value)
{
	for (uint32_t k = row_ptr[idx]; k < row_ptr[idx + 1]; k++) {
		uint32_t jdx = col_idx[k];
		if (idx == jdx) {
			K[k] = 1.0;
			F[idx] = value;
		} else {
			K[k] = 0.0;
			double *s = slot(row_ptr, col_idx, K, jdx, idx);
			double var = 0.0;
			if (s) {
				var = *s;
				*s = 0.0;
			}
			F[jdx] -= var * value;
		}
	}
}

static double seg_len(const double *nod, uint32_t a, uint32_t b)
{
	double dx = nod[2 * a] - nod[2 * b], dy = nod[2 * a + 1] - nod[2 * b + 1];
	return sqrt(dx * dx + dy * dy);
}

/* nb_fem_set_bconditions (set_bconditions.c:52-61): Neumann on segments,
 * Neumann on vertices, Dirichlet on segments, Dirichlet on vertices; each
 * group in push order. */
void orc_set_bconditions(const orc_mesh_t *m, const orc_bcs_t *b,
			 const uint32_t *row_ptr, const uint32_t *col_idx,
			 double *K, double *F, double factor)
{
	static const uint32_t order[4][2] = {{1, 1}, {1, 0}, {0, 1}, {0, 0}};
	for (int g = 0; g < 4; g++) {
		for (uint32_t a = 0; a < b->N_bc; a++) {
			const orc_bc_t *bc = &b->bc[a];
			if (bc->kind != order[g][0] || bc->where != order[g][1])
				continue;
			int fn = bc->n_nv > 0;
			if (g == 0) {
				const uint32_t *sn = b->sgm_nodes + b->sgm_ptr[bc->id];
				uint32_t n = b->sgm_ptr[bc->id + 1] - b->sgm_ptr[bc->id];
				if (fn) {
					/* set_neumann_sgm_function (:87-131) */
					for (uint32_t i = 0; i + 1 < n; i++) {
						double l = seg_len(m->nod, sn[i], sn[i + 1]);
						for (int j = 0; j < 2; j++) {
							if (!bc->mask[j])
								continue;
							double val = 0.5 * (bc->node_vals[2 * i + j] +
									    bc->node_vals[2 * (i + 1) + j]) * l;
							F[sn[i] * 2 + j] += factor * val * 0.5;
							F[sn[i + 1] * 2 + j] += factor * val * 0.5;
						}
					}
				} else {
					/* set_neumann_sgm_integrated (:133-154) + set_neumann (:156-171) */
					double L = seg_len(m->nod, sn[0], sn[n - 1]);
					for (uint32_t i = 0; i + 1 < n; i++) {
						double w = seg_len(m->nod, sn[i], sn[i + 1]) / L;
						double f = factor * w * 0.5;
						for (int j = 0; j < 2; j++)
							if (bc->mask[j])
								F[sn[i] * 2 + j] += f * bc->val[j];
						for (int j = 0; j < 2; j++)
							if (bc->mask[j])
								F[sn[i + 1] * 2 + j] += f * bc->val[j];
					}
				}
			} else if (g == 1) {
				/* set_neumann_vtx (:173-190): function atoms are read at (0,0) */
				uint32_t v = b->vtx[bc->id];
				for (int j = 0; j < 2; j++)
					if (bc->mask[j])
						F[v * 2 + j] += factor * (fn ? bc->node_vals[j] : bc->val[j]);
			} else if (g == 2) {
				/* set_dirichlet_sgm (:192-216) + set_dirichlet (:218-238) */
				const uint32_t *sn = b->sgm_nodes + b->sgm_ptr[bc->id];
				uint32_t n = b->sgm_ptr[bc->id + 1] - b->sgm_ptr[bc->id];
				for (uint32_t i = 0; i < n; i++)
					for (int j = 0; j < 2; j++)
						if (bc->mask[j])
							orc_set_dirichlet(row_ptr, col_idx, K, F, sn[i] * 2 + j,
									  factor * (fn ? bc->node_vals[2 * i + j] : bc->val[j]));
			} else {
				/* set_dirichlet_vtx (:240-260) */
				uint32_t v = b->vtx[bc->id];
				for (int j = 0; j < 2; j++)
					if (bc->mask[j])
						orc_set_dirichlet(row_ptr, col_idx, K, F, v * 2 + j,
								  factor * (fn ? bc->node_vals[j] : bc->val[j]));
			}
		}
	}
}

/* nb_sparse_multiply_vector (sparse.c:405-414) */
void orc_spmv(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
	      const double *K, const double *x, double *y, int threads)
{
	(void)threads;
#pragma omp parallel for num_threads(threads) schedule(guided)
	for (uint32_t i = 0; i < N; i++) {
		double s = 0;
		for (uint32_t k = row_ptr[i]; k < row_ptr[i + 1]; k++)
			s += K[k] * x[col_idx[k]];
		y[i] = s;
	}
}

static double diag_of(const uint32_t *row_ptr, const uint32_t *col_idx,
		      const double *K, uint32_t i)
{
	/* nb_sparse_get (sparse.c:164-171) */
	uint32_t b = row_ptr[i];
	uint32_t k = bsearch_row(col_idx + b, row_ptr[i + 1] - b, i);
	return col_idx[b + k] == i ? K[b + k] : 0.0;
}

/* nb_sparse_solve_CG_precond_Jacobi (solver_bot/sparse/solvers/
 * cg_precond_jacobi.c:13-90).  g = Ax - b is the gradient; the loop test
 * uses dot_gg of the previous iterate (it is refreshed inside the first
 * loop), the stop is absolute, and tol_reached is that lagged norm. */
int orc_cg_jacobi(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
		  const double *K, const double *b, double *x, uint32_t max_iter,
		  double tol, uint32_t *niter, double *tol_reached, int threads)
{
	(void)threads;
	double *blk = calloc(5 * (size_t)(N ? N : 1), sizeof(double));
	double *g = blk, *p = blk + N, *q = blk + 2 * (size_t)N,
	       *w = blk + 3 * (size_t)N, *Aii = blk + 4 * (size_t)N;
	double dot_gg = 0;
#pragma omp parallel for reduction(+:dot_gg) num_threads(threads) schedule(guided)
	for (uint32_t i = 0; i < N; i++) {
		double sum = 0;
		for (uint32_t k = row_ptr[i]; k < row_ptr[i + 1]; k++)
			sum += K[k] * x[col_idx[k]];
		g[i] = sum - b[i];
		Aii[i] = diag_of(row_ptr, col_idx, K, i);
		q[i] = g[i] / Aii[i];
		p[i] = -q[i];
		dot_gg += g[i] * g[i];
	}
	uint32_t k = 0;
	while (dot_gg > tol * tol && k < max_iter) {
		double dot_pw = 0, dot_gq = 0;
		dot_gg = 0;
#pragma omp parallel for reduction(+:dot_pw, dot_gg, dot_gq) num_threads(threads)
		for (uint32_t i = 0; i < N; i++) {
			double s = 0;
			for (uint32_t kk = row_ptr[i]; kk < row_ptr[i + 1]; kk++)
				s += K[kk] * p[col_idx[kk]];
			w[i] = s;
			dot_pw += p[i] * w[i];
			dot_gg += g[i] * g[i];
			dot_gq += g[i] * q[i];
		}
		double alpha = dot_gq / dot_pw;
		double dot_gkqk = 0;
#pragma omp parallel for reduction(+:dot_gkqk) num_threads(threads)
		for (uint32_t i = 0; i < N; i++) {
			x[i] += alpha * p[i];
			g[i] += alpha * w[i];
			q[i] = g[i] / Aii[i];
			dot_gkqk += g[i] * q[i];
		}
		double beta = dot_gkqk / dot_gq;
#pragma omp parallel for num_threads(threads)
		for (uint32_t i = 0; i < N; i++)
			p[i] = -q[i] + beta * p[i];
		k++;
	}
	free(blk);
	if (niter)
		*niter = k;
	if (tol_reached)
		*tol_reached = sqrt(dot_gg);
	return dot_gg > tol * tol ? 1 : 0;
}

/* nb_sparse_solve_conjugate_gradient (solvers/conjugate_gradient.c:13-77) */
int orc_cg(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
	   const double *K, const double *b, double *x, uint32_t max_iter,
	   double tol, uint32_t *niter, double *tol_reached, int threads)
{
	(void)threads;
	double *g = calloc(N ? N : 1, sizeof(double));
	double *p = calloc(N ? N : 1, sizeof(double));
	double *w = calloc(N ? N : 1, sizeof(double));
	double dot_gg = 0;
#pragma omp parallel for reduction(+:dot_gg) num_threads(threads) schedule(guided)
	for (uint32_t i = 0; i < N; i++) {
		double sum = 0;
		for (uint32_t k = row_ptr[i]; k < row_ptr[i + 1]; k++)
			sum += K[k] * x[col_idx[k]];
		g[i] = sum - b[i];
		p[i] = -g[i];
		dot_gg += g[i] * g[i];
	}
	uint32_t k = 0;
	while (dot_gg > tol * tol && k < max_iter) {
		double dot_pw = 0;
		dot_gg = 0;
#pragma omp parallel for reduction(+:dot_pw, dot_gg) num_threads(threads) schedule(guided)
		for (uint32_t i = 0; i < N; i++) {
			double s = 0;
			for (uint32_t kk = row_ptr[i]; kk < row_ptr[i + 1]; kk++)
				s += K[kk] * p[col_idx[kk]];
			w[i] = s;
			dot_pw += p[i] * w[i];
			dot_gg += g[i] * g[i];
		}
		double alpha = dot_gg / dot_pw;
		double dot_gkgk = 0;
#pragma omp parallel for reduction(+:dot_gkgk) num_threads(threads) schedule(guided)
		for (uint32_t i = 0; i < N; i++) {
			x[i] += alpha * p[i];
			g[i] += alpha * w[i];
			dot_gkgk += g[i] * g[i];
		}
		double beta = dot_gkgk / dot_gg;
#pragma omp parallel for num_threads(threads)
		for (uint32_t i = 0; i < N; i++)
			p[i] = -g[i] + beta * p[i];
		k++;
	}
	free(g);
	free(p);
	free(w);
	if (niter)
		*niter = k;
	if (tol_reached)
		*tol_reached = sqrt(dot_gg);
	return dot_gg > tol * tol ? 1 : 0;
}

/* pipeline_compute_strain / get_element_strain (pipeline.c:266-319): a
 * distorted element stops at its first bad Gauss point, leaving zeros. */
void orc_strain(const orc_mesh_t *m, const double *u, double *strain)
{
	tab_t t = table(m->nen);
	memset(strain, 0, sizeof(double) * 3 * t.ngp * (size_t)m->N_elem);
	double dx[4], dy[4];
	for (uint32_t e = 0; e < m->N_elem; e++) {
		for (int gp = 0; gp < t.ngp; gp++) {
			double Jinv[4];
			double detJ = jacobian(m, &t, e, gp, Jinv);
			if (detJ < 0)
				break;
			derivatives(&t, gp, Jinv, dx, dy);
			size_t idx = (size_t)e * t.ngp + gp;
			for (int i = 0; i < t.nn; i++) {
				uint32_t n = m->conn[e * m->nen + i];
				strain[idx * 3] += dx[i] * u[n * 2];
				strain[idx * 3 + 1] += dy[i] * u[n * 2 + 1];
				strain[idx * 3 + 2] += (dy[i] * u[n * 2] + dx[i] * u[n * 2 + 1]);
			}
		}
	}
}

/* nb_fem_compute_stress_from_strain (static_elasticity2D.c:99-127) with one
 * modulus per element. */
void orc_stress(const orc_mesh_t *m, const double *E, double nu,
		const uint8_t *enabled, const double *strain, double *stress)
{
	int ngp = m->nen == 4 ? 4 : 1;
	for (uint32_t e = 0; e < m->N_elem; e++) {
		double D[4] = {1e-6, 1e-6, 1e-6, 1e-6};
		if (!enabled || enabled[e])
			plane_stress(D, E[e], nu);
		for (int j = 0; j < ngp; j++) {
			size_t id = (size_t)e * ngp + j;
			stress[id * 3] = strain[id * 3] * D[0] + strain[id * 3 + 1] * D[1];
			stress[id * 3 + 1] = strain[id * 3] * D[1] + strain[id * 3 + 1] * D[2];
			stress[id * 3 + 2] = strain[id * 3 + 2] * D[3];
		}
	}
}

/* Principal stresses at every Gauss point (pipeline.c:321-340):
 * mean of the normal stresses plus and minus the radius of Mohr's circle. */
void orc_main_stress(uint32_t n_points, const double *stress, double *main_stress)
{
	for (uint32_t i = 0; i < n_points; i++) {
		double sx = stress[i * 3], sy = stress[i * 3 + 1], txy = stress[i * 3 + 2];
		double avg = 0.5 * (sx + sy);
		double d = sx - sy;
		double R = sqrt(0.25 * (d * d) + txy * txy);
		main_stress[i * 2] = avg + R;
		main_stress[i * 2 + 1] = avg - R;
	}
}

void orc_simp_sensitivity(const orc_mesh_t *m, double nu, double thickness,
			  const double *rho, double penal, double E0, double Emin,
			  const double *a, const double *b, double *out)
{
	int nn = (int)m->nen, n2 = 2 * nn;
	double g2[2] = {0, 0};
	for (uint32_t e = 0; e < m->N_elem; e++) {
		double Ke[64], Fe[8], ae[8], be[8];
		orc_element(m, e, 1.0, nu, thickness, 0.0, 0, g2, 1, Ke, Fe);
		for (int i = 0; i < nn; i++) {
			uint32_t n = m->conn[e * m->nen + i];
			ae[2 * i] = a[2 * n];
			ae[2 * i + 1] = a[2 * n + 1];
			be[2 * i] = b[2 * n];
			be[2 * i + 1] = b[2 * n + 1];
		}
		double s = 0.0;
		for (int r = 0; r < n2; r++) {
			double t = 0.0;
			for (int c = 0; c < n2; c++)
				t += Ke[r * n2 + c] * be[c];
			s += ae[r] * t;
		}
		double dE = penal * pow(rho[e], penal - 1.0) * (E0 - Emin);
		out[e] = -dE * s;
	}
}

/* ------------------------------------------------------------ damage model */
#define DMG_MAX(a, b) (((a) > (b)) ? (a) : (b))   /* static_damage2D.c:24 */

/* nb_sparse_forward_solve (solver_bot/sparse/solvers/triangular.c:14-32) */
static void forward_solve(uint32_t N, const uint32_t *rp, const uint32_t *ci, const double *K,
			  const double *b, double *x)
{
	for (uint32_t i = 0; i < N; i++) {
		x[i] = b[i];
		uint32_t q = rp[i];
		while (ci[q] < i) {
			x[i] -= K[q] * x[ci[q]];
			q++;
		}
		if (ci[rp[i + 1] - 1] == i)
			x[i] /= K[rp[i + 1] - 1];
		else
			x[i] /= K[bsearch_row(ci + rp[i], rp[i + 1] - rp[i], i) + rp[i]];
	}
}

/* nb_sparse_solve_Gauss_Seidel (solver_bot/sparse/solvers/gauss_seidel.c:14-58),
 * one thread */
int orc_gauss_seidel(uint32_t N, const uint32_t *rp, const uint32_t *ci, const double *K,
		     const double *b, double *x, uint32_t max_iter, double tol,
		     uint32_t *niter, double *tol_reached)
{
	double *c = calloc(N ? N : 1, sizeof(double));
	uint32_t k = 0;
	double error = 1e10;
	while (k < max_iter) {
		error = 0;
		for (uint32_t i = 0; i < N; i++) {
			c[i] = b[i];
			double error_i = b[i];
			for (uint32_t j = rp[i]; j < rp[i + 1]; j++) {
				error_i -= K[j] * x[ci[j]];
				if (ci[j] > i)
					c[i] -= K[j] * x[ci[j]];
			}
			error += error_i * error_i;
		}
		if (error <= tol * tol)
			break;
		forward_solve(N, rp, ci, K, c, x);
		k++;
	}
	free(c);
	if (niter) *niter = k;
	if (tol_reached) *tol_reached = sqrt(error);
	return error > tol * tol ? 1 : 0;
}

/* tension_damage (static_damage2D.c:134-182) at one Gauss point */
double orc_tension_damage(double E, double nu, double ft, double gf, const double *strain,
			  double r_prev, double *r, double clfd)
{
	double D[4];
	plane_stress(D, E, nu);
	double es[3];
	es[0] = D[0] * strain[0] + D[1] * strain[1];
	es[1] = D[1] * strain[0] + D[2] * strain[1];
	es[2] = D[3] * strain[2];
	double avg = 0.5 * (es[0] + es[1]);
	double d = es[0] - es[1];
	double R = sqrt(0.25 * (d * d) + es[2] * es[2]);
	double p1 = DMG_MAX(0, avg + R);
	double p2 = DMG_MAX(0, avg - R);
	double det = D[0] * D[2] - D[1] * D[1];
	double id11 = D[2] / det, id12 = -D[1] / det, id22 = D[0] / det;
	double sTs = id11 * (p1 * p1) + 2 * id12 * p1 * p2 + id22 * (p2 * p2);
	double tau = sqrt(sTs);
	double r0 = ft / sqrt(E);
	*r = DMG_MAX(r_prev, tau);
	double div = (gf / clfd) * (E / (ft * ft));
	double A = 1.0 / (div - 0.5);
	return 1.0 - (r0 / *r) * exp(A * (1.0 - (*r / r0)));
}

/* get_clfd (static_damage2D.c:633-647): sqrt of twice the area of the
 * triangle of the element's first three nodes */
static double clfd_of(const orc_mesh_t *m, uint32_t e)
{
	const uint32_t *c = m->conn + (size_t)e * m->nen;
	double x1 = m->nod[2 * c[0]], y1 = m->nod[2 * c[0] + 1];
	double x2 = m->nod[2 * c[1]], y2 = m->nod[2 * c[1] + 1];
	double x3 = m->nod[2 * c[2]], y3 = m->nod[2 * c[2] + 1];
	return sqrt((x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1));
}

static void logf_(char *log, size_t cap, size_t *len, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	int n = vsnprintf(log + *len, *len < cap ? cap - *len : 0, fmt, ap);
	va_end(ap);
	if (n > 0)
		*len = *len + (size_t)n < cap ? *len + (size_t)n : cap;
}

/* nb_fem_compute_2D_Non_Linear_Solid_Mechanics (static_damage2D.c:239-470)
 * with the conjugate-gradient path (enable_Cholesky_solver false), one
 * material, all elements enabled.  Writes nbots' log text into `log`
 * (cap bytes, NUL-terminated) and the final displacements and damage (N_gp
 * per element).  Returns how many solves fell back to Gauss-Seidel. */
int orc_damage_solve(const orc_mesh_t *m, const orc_bcs_t *b, double E, double nu,
		     double thickness, double density, int self_weight, const double gravity[2],
		     double ft, double gf, uint32_t n_steps, uint32_t max_iter,
		     uint32_t max_iter_noenh, double rtol, char *log, size_t cap,
		     double *u_out, double *damage_out)
{
	tab_t t = table(m->nen);
	const uint32_t N = 2 * m->N_nod, ngp = (uint32_t)t.ngp, nn = m->nen, n2 = 2 * nn;
	const size_t npt = (size_t)ngp * m->N_elem;
	size_t len = 0;
	if (cap) log[0] = 0;
	uint32_t *rp = malloc(((size_t)N + 1) * sizeof(uint32_t));
	orc_pattern(m, rp, NULL);
	uint32_t *ci = malloc(((size_t)rp[N] + 1) * sizeof(uint32_t));
	orc_pattern(m, rp, ci);
	double *K = calloc(rp[N] + 1, sizeof(double));
	double *disp = calloc(N, sizeof(double)), *F = calloc(N, sizeof(double));
	double *P = calloc(N, sizeof(double)), *res = calloc(N, sizeof(double));
	double *du = calloc(N, sizeof(double));
	double *strain = calloc(3 * npt, sizeof(double)), *dmg = calloc(npt, sizeof(double));
	double *r = malloc(npt * sizeof(double)), *r_prev = malloc(npt * sizeof(double));
	const double r0 = ft / sqrt(E);
	for (size_t i = 0; i < npt; i++)
		r[i] = r0;
	int n_gs = 0;
	logf_(log, cap, &len, "FEM: Damage Model\n");
	for (uint32_t n = 0; n < n_steps; n++) {
		logf_(log, cap, &len, "  [ Load step %i]\n", n + 1);
		memcpy(r_prev, r, npt * sizeof(double));
		memset(du, 0, N * sizeof(double));
		double residual_norm = 1, residual_best = 0;
		uint32_t iter = 0, noenh = 0;
		for (;;) {
			/* DMG_pipeline_assemble_system (static_damage2D.c:474-569) */
			memset(K, 0, rp[N] * sizeof(double));
			memset(F, 0, N * sizeof(double));
			double Ke[64], Fe[8];
			for (uint32_t e = 0; e < m->N_elem; e++) {
				if (element_dmg(m, e, E, nu, thickness, density, self_weight, gravity, 1,
						dmg + (size_t)e * ngp, Ke, Fe))
					break;
				for (uint32_t i = 0; i < nn; i++) {
					uint32_t v1 = m->conn[e * nn + i];
					for (uint32_t j = 0; j < nn; j++) {
						uint32_t v2 = m->conn[e * nn + j];
						*slot(rp, ci, K, 2 * v1, 2 * v2) += Ke[(2 * i) * n2 + 2 * j];
						*slot(rp, ci, K, 2 * v1 + 1, 2 * v2) += Ke[(2 * i + 1) * n2 + 2 * j];
						*slot(rp, ci, K, 2 * v1, 2 * v2 + 1) += Ke[(2 * i) * n2 + 2 * j + 1];
						*slot(rp, ci, K, 2 * v1 + 1, 2 * v2 + 1) +=
							Ke[(2 * i + 1) * n2 + 2 * j + 1];
					}
					F[2 * v1] += Fe[2 * i];
					F[2 * v1 + 1] += Fe[2 * i + 1];
				}
			}
			double factor = (n + 1.0) / (double)n_steps;
			orc_set_bconditions(m, b, rp, ci, K, F, factor);
			orc_spmv(N, rp, ci, K, disp, P, 1);
			residual_norm = 0;
			for (uint32_t i = 0; i < N; i++) {
				res[i] = F[i] - P[i];
				residual_norm += res[i] * res[i];
			}
			residual_norm = sqrt(residual_norm);
			if (iter == 0) {
				residual_best = residual_norm;
			} else {
				if (residual_norm < residual_best) {
					residual_best = residual_norm;
					noenh = 0;
				} else {
					noenh += 1;
				}
			}
			if ((residual_norm < rtol && iter > 0) || iter >= max_iter ||
			    noenh >= max_iter_noenh) {
				logf_(log, cap, &len, "    [%i: Residual: %e ]\n", iter, residual_norm);
				break;
			}
			uint32_t its = 0;
			double err = 0.0;
			int st = orc_cg_jacobi(N, rp, ci, K, res, du, N, 1e-8, &its, &err, 1);
			if (st != 0) {
				n_gs++;
				st = orc_gauss_seidel(N, rp, ci, K, res, du, 60 * N, 1e-8, &its, &err);
				if (st != 0) {
					logf_(log, cap, &len,
					      "    [Conjugate Gradient (p. Jacobi) and Gauss-Seidel fails.]\n");
					logf_(log, cap, &len, "      [Gauss-Seidel iterations: %u]\n", its);
					logf_(log, cap, &len, "      [Gauss-Seidel error: %e ]\n", err);
				}
			}
			logf_(log, cap, &len, "    [%i: Residual: %e]\n", iter, residual_norm);
			for (uint32_t i = 0; i < N; i++)
				disp[i] += du[i];
			/* DMG_pipeline_compute_strain (static_damage2D.c:571-631) */
			orc_strain(m, disp, strain);
			for (uint32_t e = 0; e < m->N_elem; e++) {
				double cl = clfd_of(m, e);
				for (uint32_t g = 0; g < ngp; g++) {
					size_t idx = (size_t)e * ngp + g;
					dmg[idx] = orc_tension_damage(E, nu, ft, gf, strain + 3 * idx,
								      r_prev[idx], r + idx, cl);
				}
			}
			iter++;
		}
	}
	if (u_out) memcpy(u_out, disp, N * sizeof(double));
	if (damage_out) memcpy(damage_out, dmg, npt * sizeof(double));
	free(rp); free(ci); free(K); free(disp); free(F); free(P); free(res); free(du);
	free(strain); free(dmg); free(r); free(r_prev);
	return n_gs;
}
