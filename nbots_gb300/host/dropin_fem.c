/*
 * Drop-in nb_fem_compute_2D_Solid_Mechanics / nb_fem_compute_stress_from_strain
 * (nbots_dropin.h) on the device FEM system (fem.c).
 *
 * The mesh, boundary conditions, material and element type are read through
 * nbots' public accessors only, so the function works on nbots' own objects
 * when linked ahead of libnbots.so, and on libnbots_host.so's otherwise.
 * Function-valued conditions are evaluated here, at the points where nbots
 * evaluates them (set_bconditions.c:63-260): segment nodes, vertex nodes for
 * Dirichlet, and (0,0) for Neumann vertex loads.
 */
#include <stdlib.h>
#include <string.h>

#include "nbots_dropin.h"
#include "nbots_gb300.h"

#include "fem_internal.h"

void nbg_dropin_record_error(int e);
int nbg_dropin_cpu(void);
void *nbg_dropin_next(const char *name);

/* The device copy of a drop-in matrix (dropin_sparse.c). */
nbg_solver_t *nbg_dropin_lock_device(const nb_sparse_t *A, int send_values, int *rc);
void nbg_dropin_unlock_device(const nb_sparse_t *A, int synced);
int nbg_dropin_slab(const nb_sparse_t *A, double **vals, const uint32_t **row_ptr);

/* NBG_DROPIN_EXACT_CG=1: nbots' arithmetic on the CSR for every drop-in CG */
static int exact_cg(void)
{
	const char *v = getenv("NBG_DROPIN_EXACT_CG");
	return v && v[0] == '1' && v[1] == 0;
}

typedef struct {
	nbg_mesh_t m;
	double *nod;
	uint32_t *conn, *edg, *vtx, *sgm_ptr, *sgm_nodes;
	uint32_t N_sgm;
	nbg_bc_t *bc;
	double **vals;
	uint32_t N_bc;
} host_problem_t;

static void free_problem(host_problem_t *h)
{
	free(h->nod);
	free(h->conn);
	free(h->edg);
	free(h->vtx);
	free(h->sgm_ptr);
	free(h->sgm_nodes);
	for (uint32_t k = 0; k < h->N_bc; k++)
		free(h->vals ? h->vals[k] : NULL);
	free(h->vals);
	free(h->bc);
}

static int read_mesh(const nb_mesh2D_t *part, uint32_t nen, host_problem_t *h)
{
	const uint32_t Nn = nb_mesh2D_get_N_nodes(part), Ne = nb_mesh2D_get_N_elems(part);
	const uint32_t Nd = nb_mesh2D_get_N_edges(part);
	h->nod = malloc(16 * (size_t)(Nn ? Nn : 1));
	h->conn = malloc(4 * (size_t)nen * (Ne ? Ne : 1));
	h->edg = malloc(8 * (size_t)(Nd ? Nd : 1));
	if (!h->nod || !h->conn || !h->edg)
		return NBG_ERR_NOMEM;
	for (uint32_t i = 0; i < Nn; i++) {
		h->nod[2 * i] = nb_mesh2D_node_get_x(part, i);
		h->nod[2 * i + 1] = nb_mesh2D_node_get_y(part, i);
	}
	for (uint32_t e = 0; e < Ne; e++)
		for (uint32_t k = 0; k < nen; k++)
			h->conn[e * nen + k] = nb_mesh2D_elem_get_adj(part, e, (uint8_t)k);
	for (uint32_t i = 0; i < Nd; i++) {
		h->edg[2 * i] = nb_mesh2D_edge_get_1n(part, i);
		h->edg[2 * i + 1] = nb_mesh2D_edge_get_2n(part, i);
	}
	h->m = (nbg_mesh_t){nen, Nn, Ne, Nd, h->nod, h->conn, h->edg};
	const uint32_t Nv = nb_mesh2D_get_N_invtx(part), Ns = nb_mesh2D_get_N_insgm(part);
	h->vtx = malloc(4 * (size_t)(Nv ? Nv : 1));
	h->sgm_ptr = malloc(4 * ((size_t)Ns + 1));
	if (!h->vtx || !h->sgm_ptr)
		return NBG_ERR_NOMEM;
	for (uint32_t i = 0; i < Nv; i++)
		h->vtx[i] = nb_mesh2D_get_invtx(part, i);
	h->sgm_ptr[0] = 0;
	for (uint32_t s = 0; s < Ns; s++)
		h->sgm_ptr[s + 1] = h->sgm_ptr[s] + nb_mesh2D_insgm_get_N_nodes(part, s);
	h->sgm_nodes = malloc(4 * (size_t)(h->sgm_ptr[Ns] ? h->sgm_ptr[Ns] : 1));
	if (!h->sgm_nodes)
		return NBG_ERR_NOMEM;
	for (uint32_t s = 0; s < Ns; s++)
		for (uint32_t i = 0; i < h->sgm_ptr[s + 1] - h->sgm_ptr[s]; i++)
			h->sgm_nodes[h->sgm_ptr[s] + i] = nb_mesh2D_insgm_get_node(part, s, i);
	h->N_sgm = Ns;
	return NBG_OK;
}

static int read_bcond(const nb_mesh2D_t *part, const nb_bcond_t *bcond, host_problem_t *h)
{
	static const int cat[4][2] = {{NB_DIRICHLET, NB_BC_ON_POINT}, {NB_NEUMANN, NB_BC_ON_POINT},
				      {NB_DIRICHLET, NB_BC_ON_SEGMENT},
				      {NB_NEUMANN, NB_BC_ON_SEGMENT}};
	if (nb_bcond_get_N_dof(bcond) != 2)
		return NBG_ERR_ARG;
	void *it = malloc(nb_bcond_iter_get_memsize());
	if (!it)
		return NBG_ERR_NOMEM;
	uint32_t cap = 0;
	for (int pass = 0; pass < 2; pass++) {
		uint32_t n = 0;
		for (int c = 0; c < 4; c++) {
			nb_bcond_iter_init(it);
			nb_bcond_iter_set_conditions(it, bcond, (nb_bcond_id)cat[c][0],
						     (nb_bcond_where)cat[c][1]);
			while (nb_bcond_iter_has_more(it)) {
				nb_bcond_iter_go_next(it);
				if (pass == 1) {
					nbg_bc_t *b = &h->bc[n];
					memset(b, 0, sizeof(*b));
					b->kind = cat[c][0] == NB_DIRICHLET ? 0u : 1u;
					b->where = cat[c][1] == NB_BC_ON_POINT ? 0u : 1u;
					b->id = nb_bcond_iter_get_id(it);
					b->mask[0] = nb_bcond_iter_get_mask(it, 0);
					b->mask[1] = nb_bcond_iter_get_mask(it, 1);
					double x0[2] = {0.0, 0.0};
					if (!nb_bcond_iter_val_is_function(it)) {
						nb_bcond_iter_get_val(it, 2, x0, 0.0, b->val);
					} else {
						uint32_t nv = 1;
						if (b->where == 1) {
							if (b->id >= h->N_sgm) {
								free(it);
								return NBG_ERR_ARG;
							}
							nv = h->sgm_ptr[b->id + 1] - h->sgm_ptr[b->id];
						}
						double *v = malloc(16 * (size_t)nv);
						if (!v) {
							free(it);
							return NBG_ERR_NOMEM;
						}
						h->vals[n] = v;
						for (uint32_t i = 0; i < nv; i++) {
							double x[2] = {0.0, 0.0};
							if (!(b->kind == 1 && b->where == 0)) {
								uint32_t nid = b->where == 1 ?
									h->sgm_nodes[h->sgm_ptr[b->id] + i] :
									h->vtx[b->id];
								x[0] = h->nod[2 * nid];
								x[1] = h->nod[2 * nid + 1];
							}
							nb_bcond_iter_get_val(it, 2, x, 0.0, v + 2 * i);
						}
						b->n_nv = nv;
						b->node_vals = v;
					}
				}
				n++;
			}
			nb_bcond_iter_finish(it);
		}
		if (pass == 0) {
			cap = n;
			h->bc = calloc(cap ? cap : 1, sizeof(nbg_bc_t));
			h->vals = calloc(cap ? cap : 1, sizeof(double *));
			if (!h->bc || !h->vals) {
				free(it);
				return NBG_ERR_NOMEM;
			}
			h->N_bc = cap;
		}
	}
	free(it);
	return NBG_OK;
}

int nb_fem_compute_2D_Solid_Mechanics(const nb_mesh2D_t *part, const nb_fem_elem_t *elemtype,
				      const nb_material_t *material, const nb_bcond_t *bcond,
				      bool enable_self_weight, double gravity[2],
				      nb_analysis2D_t analysis2D, nb_analysis2D_params *params2D,
				      const bool *elements_enabled, double *displacement,
				      double *strain)
{
	if (nbg_dropin_cpu()) {
		typedef int (*fn_t)(const nb_mesh2D_t *, const nb_fem_elem_t *,
				    const nb_material_t *, const nb_bcond_t *, bool, double[2],
				    nb_analysis2D_t, nb_analysis2D_params *, const bool *, double *,
				    double *);
		fn_t next = (fn_t)nbg_dropin_next("nb_fem_compute_2D_Solid_Mechanics");
		return next ? next(part, elemtype, material, bcond, enable_self_weight, gravity,
				   analysis2D, params2D, elements_enabled, displacement, strain)
			    : NBG_ERR_ARG;
	}
	(void)analysis2D;
	const uint32_t nen = nb_fem_elem_get_N_nodes(elemtype);
	if (nen != 3 && nen != 4)
		return NBG_ERR_ARG;
	host_problem_t h;
	memset(&h, 0, sizeof(h));
	double *E = NULL;
	uint8_t *en = NULL;
	nbg_fem_t *f = NULL;
	int rc = read_mesh(part, nen, &h);
	if (rc == NBG_OK)
		rc = read_bcond(part, bcond, &h);
	const uint32_t Ne = h.m.N_elem;
	if (rc == NBG_OK) {
		E = malloc(8 * (size_t)(Ne ? Ne : 1));
		if (!E)
			rc = NBG_ERR_NOMEM;
		for (uint32_t e = 0; E && e < Ne; e++)
			E[e] = nb_material_get_elasticity_module(material);
	}
	if (rc == NBG_OK && elements_enabled) {
		en = malloc(Ne ? Ne : 1);
		if (!en)
			rc = NBG_ERR_NOMEM;
		for (uint32_t e = 0; en && e < Ne; e++)
			en[e] = elements_enabled[e] ? 1 : 0;
	}
	if (rc == NBG_OK)
		rc = nbg_fem_create(&f, &h.m, NULL);
	if (rc == NBG_OK) {
		double g2[2] = {gravity ? gravity[0] : 0.0, gravity ? gravity[1] : 0.0};
		rc = nbg_fem_assemble(f, E, nb_material_get_poisson_module(material),
				      params2D->thickness, nb_material_get_density(material),
				      enable_self_weight, g2, en);
	}
	if (rc == NBG_OK) {
		nbg_bcs_t b = {h.vtx, h.N_sgm, h.sgm_ptr, h.sgm_nodes, h.N_bc, h.bc};
		rc = nbg_fem_apply_bcs(f, &b, 1.0);
	}
	if (rc == NBG_OK) {
		/* solver() of static_elasticity2D.c:83-97: x0 = 0, max_iter = N,
		 * tol 1e-8 absolute; "not converged" counts as success.  nbots'
		 * iteration and stop test, on the block layout with FMAs unless
		 * NBG_DROPIN_EXACT_CG=1 asks for nbots' arithmetic on the CSR */
		nbg_cg_result_t r;
		int st = exact_cg() ? nbg_fem_solve(f, nbg_fem_n_dof(f), 1e-8, NBG_CG_JACOBI, &r)
				    : nbg_fem_solve_fast(f, nbg_fem_n_dof(f), 1e-8,
							 NBG_CG_JACOBI | NBG_CG_NBOTS_STOP, &r);
		rc = st < 0 ? st : NBG_OK;
	}
	if (rc == NBG_OK)
		rc = nbg_fem_strain(f);
	if (rc == NBG_OK)
		rc = nbg_fem_download(f, NBG_FEM_U, displacement);
	if (rc == NBG_OK)
		rc = nbg_fem_download(f, NBG_FEM_STRAIN, strain);
	nbg_fem_destroy(f);
	free(E);
	free(en);
	free_problem(&h);
	return rc;
}

void nb_fem_compute_stress_from_strain(uint32_t N_elements, const nb_fem_elem_t *elemtype,
				       const nb_material_t *material, nb_analysis2D_t analysis2D,
				       double *strain, const bool *elements_enabled,
				       double *stress)
{
	if (nbg_dropin_cpu()) {
		typedef void (*fn_t)(uint32_t, const nb_fem_elem_t *, const nb_material_t *,
				     nb_analysis2D_t, double *, const bool *, double *);
		fn_t next = (fn_t)nbg_dropin_next("nb_fem_compute_stress_from_strain");
		if (next)
			next(N_elements, elemtype, material, analysis2D, strain, elements_enabled,
			     stress);
		else
			nbg_dropin_record_error(NBG_ERR_ARG);
		return;
	}
	(void)analysis2D;
	const uint32_t nen = nb_fem_elem_get_N_nodes(elemtype);
	const size_t ng = nen == 4 ? 4 : 1;
	const size_t n3 = 3 * ng * N_elements;
	double *E = malloc(8 * (size_t)(N_elements ? N_elements : 1));
	uint8_t *en = elements_enabled ? malloc(N_elements ? N_elements : 1) : NULL;
	void *dE = NULL, *den = NULL, *ds = NULL, *dt = NULL;
	int rc = E && (!elements_enabled || en) ? NBG_OK : NBG_ERR_NOMEM;
	for (uint32_t e = 0; rc == NBG_OK && e < N_elements; e++) {
		E[e] = nb_material_get_elasticity_module(material);
		if (en)
			en[e] = elements_enabled[e] ? 1 : 0;
	}
	if (rc == NBG_OK) rc = nbg_dev_alloc(&dE, 8 * (size_t)(N_elements ? N_elements : 1));
	if (rc == NBG_OK && en) rc = nbg_dev_alloc(&den, N_elements ? N_elements : 1);
	if (rc == NBG_OK) rc = nbg_dev_alloc(&ds, 8 * (n3 ? n3 : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&dt, 8 * (n3 ? n3 : 1));
	if (rc == NBG_OK) rc = nbg_h2d(dE, E, 8 * (size_t)N_elements, NULL);
	if (rc == NBG_OK && en) rc = nbg_h2d(den, en, N_elements, NULL);
	if (rc == NBG_OK) rc = nbg_h2d(ds, strain, 8 * n3, NULL);
	if (rc == NBG_OK)
		rc = nbg_stress_f64(nen, N_elements, dE, nb_material_get_poisson_module(material),
				    den, ds, dt, NULL);
	if (rc == NBG_OK) rc = nbg_d2h(stress, dt, 8 * n3, NULL);
	if (rc == NBG_OK) rc = nbg_stream_sync(NULL);
	nbg_dev_free(dE);
	nbg_dev_free(den);
	nbg_dev_free(ds);
	nbg_dev_free(dt);
	free(E);
	free(en);
}

void pipeline_compute_main_stress(double *stress, double *main_stress, uint32_t N_elements,
				  const nb_fem_elem_t *const elem)
{
	if (nbg_dropin_cpu()) {
		typedef void (*fn_t)(double *, double *, uint32_t, const nb_fem_elem_t *const);
		fn_t next = (fn_t)nbg_dropin_next("pipeline_compute_main_stress");
		if (next)
			next(stress, main_stress, N_elements, elem);
		else
			nbg_dropin_record_error(NBG_ERR_ARG);
		return;
	}
	const uint32_t nen = nb_fem_elem_get_N_nodes(elem);
	const size_t n = (size_t)nb_fem_elem_get_N_gpoints(elem) * N_elements;
	void *ds = NULL, *dm = NULL;
	int rc = nbg_dev_alloc(&ds, 24 * (n ? n : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&dm, 16 * (n ? n : 1));
	if (rc == NBG_OK) rc = nbg_h2d(ds, stress, 24 * n, NULL);
	if (rc == NBG_OK) rc = nbg_main_stress_f64(nen, N_elements, ds, dm, NULL);
	if (rc == NBG_OK) rc = nbg_d2h(main_stress, dm, 16 * n, NULL);
	if (rc == NBG_OK) rc = nbg_stream_sync(NULL);
	nbg_dev_free(ds);
	nbg_dev_free(dm);
}


typedef void (*nonlinear_fn)(const nb_mesh2D_t *, const nb_fem_elem_t *, const nb_material_t *,
			     const nb_bcond_t *, bool, double[2], bool, nb_analysis2D_t,
			     nb_analysis2D_params *, nb_fem_implicit_t *, const char *);

void nb_fem_compute_2D_Non_Linear_Solid_Mechanics(const nb_mesh2D_t *part,
						  const nb_fem_elem_t *elem,
						  const nb_material_t *material,
						  const nb_bcond_t *bcond, bool enable_self_weight,
						  double gravity[2], bool enable_Cholesky_solver,
						  nb_analysis2D_t analysis2D,
						  nb_analysis2D_params *params2D,
						  nb_fem_implicit_t *params, const char *logfile)
{
	if (enable_Cholesky_solver || nbg_dropin_cpu()) {
		/* the direct-solver branch is nbots' own; so is everything under the
		 * A/B switch */
		nonlinear_fn next = (nonlinear_fn)nbg_dropin_next(
			"nb_fem_compute_2D_Non_Linear_Solid_Mechanics");
		if (next) {
			next(part, elem, material, bcond, enable_self_weight, gravity,
			     enable_Cholesky_solver, analysis2D, params2D, params, logfile);
			return;
		}
		if (nbg_dropin_cpu()) {
			nbg_dropin_record_error(NBG_ERR_ARG);
			return;
		}
	}
	const uint32_t nen = nb_fem_elem_get_N_nodes(elem);
	if (nen != 3 && nen != 4) {
		nbg_dropin_record_error(NBG_ERR_ARG);
		return;
	}
	host_problem_t h;
	memset(&h, 0, sizeof(h));
	nbg_fem_t *f = NULL;
	int rc = read_mesh(part, nen, &h);
	if (rc == NBG_OK)
		rc = read_bcond(part, bcond, &h);
	if (rc == NBG_OK)
		rc = nbg_fem_create(&f, &h.m, NULL);
	if (rc == NBG_OK) {
		double g2[2] = {gravity ? gravity[0] : 0.0, gravity ? gravity[1] : 0.0};
		nbg_bcs_t b = {h.vtx, h.N_sgm, h.sgm_ptr, h.sgm_nodes, h.N_bc, h.bc};
		nbg_damage_info_t info;
		rc = nbg_fem_damage(f, &b, nb_material_get_elasticity_module(material),
				    nb_material_get_poisson_module(material), params2D->thickness,
				    nb_material_get_density(material), enable_self_weight, g2,
				    nb_material_get_traction_limit_stress(material),
				    nb_material_get_fracture_energy(material),
				    nb_fem_implicit_get_N_steps(params),
				    nb_fem_implicit_get_N_max_iter(params),
				    nb_fem_implicit_get_N_max_iter_without_enhance(params),
				    nb_fem_implicit_get_residual_tolerance(params),
				    exact_cg() ? NBG_METHOD_NBOTS : NBG_METHOD_NBOTS_FAST, logfile,
				    &info);
	}
	nbg_dropin_record_error(rc);
	nbg_fem_destroy(f);
	free_problem(&h);
}


/* ------------------------------------------- replaced: the pipeline stages */
typedef int (*assemble_fn)(nb_sparse_t *, double *, double *, const nb_mesh2D_t *,
			   const nb_fem_elem_t *, const nb_material_t *, bool, double[2],
			   nb_analysis2D_t, nb_analysis2D_params *, const bool *);
typedef void (*bcond_fn)(const nb_mesh2D_t *, nb_sparse_t *, double *, const nb_bcond_t *,
			 double);
typedef void (*strain_fn)(double *, const nb_mesh2D_t *, double *, const nb_fem_elem_t *);

/* The device copy of K (a matrix of nb_sparse_create(graph, NULL, 2) on
 * this mesh: node-blocked, 2 N_nod rows) and a FEM system on it; NULL when K
 * is not such a matrix (the caller then goes to nbots' own stage). */
static nbg_fem_t *fem_on_matrix(nb_sparse_t *K, const nbg_mesh_t *m, int send_values,
				int need_incidence, nbg_solver_t **dev, int *rc)
{
	*rc = NBG_OK;
	*dev = NULL;
	if (K->N != 2 * m->N_nod)
		return NULL;
	nbg_solver_t *d = nbg_dropin_lock_device(K, send_values, rc);
	if (!d)
		return NULL;
	const uint32_t *rp, *ci;
	double *val;
	nbg_fem_t *f = NULL;
	if (nbg_solver_block_layout(d, NULL) != NBG_OK ||
	    nbg_solver_device_csr(d, &rp, &ci, &val) != NBG_OK) {
		nbg_dropin_unlock_device(K, 0);
		return NULL;
	}
	double *vals;
	const uint32_t *hrp;
	nbg_dropin_slab(K, &vals, &hrp);
	*rc = nbg_fem_create_on_csr(&f, m, hrp[K->N], (uint32_t *)rp, (uint32_t *)ci, val,
				    need_incidence, NULL);
	if (*rc != NBG_OK) {
		nbg_dropin_unlock_device(K, 0);
		return NULL;
	}
	*dev = d;
	return f;
}

/* Device K and F back to the caller's matrix and vector; the device copy's
 * block layout follows the new values. */
static int write_back(nb_sparse_t *K, nbg_solver_t *dev, nbg_fem_t *f, double *F)
{
	double *vals;
	const uint32_t *hrp;
	nbg_dropin_slab(K, &vals, &hrp);
	int rc = nbg_d2h(vals, f->K, 8 * (size_t)hrp[K->N], NULL);
	if (rc == NBG_OK)
		rc = nbg_d2h(F, f->F, 8 * (size_t)f->N, NULL);
	if (rc == NBG_OK)
		rc = nbg_solver_values_changed(dev);
	if (rc == NBG_OK)
		rc = nbg_stream_sync(NULL);
	return rc;
}

int pipeline_assemble_system(nb_sparse_t *K, double *M, double *F, const nb_mesh2D_t *part,
			     const nb_fem_elem_t *elemtype, const nb_material_t *material,
			     bool enable_self_weight, double gravity[2],
			     nb_analysis2D_t analysis2D, nb_analysis2D_params *params2D,
			     const bool *elements_enabled)
{
	const uint32_t nen = nb_fem_elem_get_N_nodes(elemtype);
	host_problem_t h;
	memset(&h, 0, sizeof(h));
	nbg_fem_t *f = NULL;
	nbg_solver_t *dev = NULL;
	int rc = NBG_OK;
	/* the lumped mass (M) is not computed on the device: nbots' own stage
	 * does it, as everything under the A/B switch */
	if (!nbg_dropin_cpu() && M == NULL && (nen == 3 || nen == 4)) {
		rc = read_mesh(part, nen, &h);
		if (rc == NBG_OK)
			f = fem_on_matrix(K, &h.m, 0, 1, &dev, &rc);
	}
	if (!f) {
		free_problem(&h);
		if (rc != NBG_OK)
			return rc;
		assemble_fn next = (assemble_fn)nbg_dropin_next("pipeline_assemble_system");
		return next ? next(K, M, F, part, elemtype, material, enable_self_weight, gravity,
				   analysis2D, params2D, elements_enabled)
			    : NBG_ERR_ARG;
	}
	const uint32_t Ne = h.m.N_elem;
	double *E = malloc(8 * (size_t)(Ne ? Ne : 1));
	uint8_t *en = elements_enabled ? malloc(Ne ? Ne : 1) : NULL;
	if (!E || (elements_enabled && !en))
		rc = NBG_ERR_NOMEM;
	for (uint32_t e = 0; rc == NBG_OK && e < Ne; e++) {
		E[e] = nb_material_get_elasticity_module(material);
		if (en)
			en[e] = elements_enabled[e] ? 1 : 0;
	}
	int synced = 0;
	if (rc == NBG_OK) {
		double g2[2] = {gravity ? gravity[0] : 0.0, gravity ? gravity[1] : 0.0};
		rc = nbg_fem_assemble(f, E, nb_material_get_poisson_module(material),
				      params2D->thickness, nb_material_get_density(material),
				      enable_self_weight, g2, en);
		if (rc == NBG_OK) {
			rc = write_back(K, dev, f, F);
			synced = rc == NBG_OK;
		} else if (rc == NBG_DISTORTED) {
			/* nbots stops at the distorted element with K and F partly
			 * summed; here they are left reset, and the status is its */
			nb_sparse_reset(K);
			memset(F, 0, 8 * (size_t)K->N);
		}
	}
	nbg_fem_destroy(f);
	nbg_dropin_unlock_device(K, synced);
	free(E);
	free(en);
	free_problem(&h);
	return rc;
}

void nb_fem_set_bconditions(const nb_mesh2D_t *part, nb_sparse_t *K, double *F,
			    const nb_bcond_t *bcond, double factor)
{
	host_problem_t h;
	memset(&h, 0, sizeof(h));
	nbg_fem_t *f = NULL;
	nbg_solver_t *dev = NULL;
	int rc = NBG_OK;
	const uint32_t nen = nb_mesh2D_get_N_elems(part) ? nb_mesh2D_elem_get_N_adj(part, 0) : 0;
	if (!nbg_dropin_cpu() && (nen == 3 || nen == 4)) {
		rc = read_mesh(part, nen, &h);
		if (rc == NBG_OK)
			rc = read_bcond(part, bcond, &h);
		if (rc == NBG_OK)
			f = fem_on_matrix(K, &h.m, 1, 0, &dev, &rc);
	}
	if (!f) {
		free_problem(&h);
		if (rc != NBG_OK) {
			nbg_dropin_record_error(rc);
			return;
		}
		bcond_fn next = (bcond_fn)nbg_dropin_next("nb_fem_set_bconditions");
		if (next)
			next(part, K, F, bcond, factor);
		else
			nbg_dropin_record_error(NBG_ERR_ARG);
		return;
	}
	rc = nbg_h2d(f->F, F, 8 * (size_t)f->N, NULL);
	nbg_bcs_t b = {h.vtx, h.N_sgm, h.sgm_ptr, h.sgm_nodes, h.N_bc, h.bc};
	if (rc == NBG_OK)
		rc = nbg_fem_apply_bcs(f, &b, factor);
	if (rc == NBG_OK)
		rc = write_back(K, dev, f, F);
	nbg_fem_destroy(f);
	nbg_dropin_unlock_device(K, rc == NBG_OK);
	nbg_dropin_record_error(rc);
	free_problem(&h);
}

void pipeline_compute_strain(double *strain, const nb_mesh2D_t *part, double *displacement,
			     const nb_fem_elem_t *elemtype)
{
	const uint32_t nen = nb_fem_elem_get_N_nodes(elemtype);
	if (nbg_dropin_cpu() || (nen != 3 && nen != 4)) {
		strain_fn next = (strain_fn)nbg_dropin_next("pipeline_compute_strain");
		if (next)
			next(strain, part, displacement, elemtype);
		else
			nbg_dropin_record_error(NBG_ERR_ARG);
		return;
	}
	host_problem_t h;
	memset(&h, 0, sizeof(h));
	int rc = read_mesh(part, nen, &h);
	const size_t Nn = h.m.N_nod, Ne = h.m.N_elem, n3 = 3 * (size_t)(nen == 4 ? 4 : 1) * Ne;
	void *dn = NULL, *dc = NULL, *du = NULL, *ds = NULL;
	if (rc == NBG_OK) rc = nbg_dev_alloc(&dn, 16 * (Nn ? Nn : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&dc, 4 * nen * (Ne ? Ne : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&du, 16 * (Nn ? Nn : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&ds, 8 * (n3 ? n3 : 1));
	if (rc == NBG_OK) rc = nbg_h2d(dn, h.nod, 16 * Nn, NULL);
	if (rc == NBG_OK) rc = nbg_h2d(dc, h.conn, 4 * nen * Ne, NULL);
	if (rc == NBG_OK) rc = nbg_h2d(du, displacement, 16 * Nn, NULL);
	if (rc == NBG_OK) rc = nbg_strain_f64(nen, (uint32_t)Ne, dn, dc, du, ds, NULL);
	if (rc == NBG_OK) rc = nbg_d2h(strain, ds, 8 * n3, NULL);
	if (rc == NBG_OK) rc = nbg_stream_sync(NULL);
	nbg_dev_free(dn);
	nbg_dev_free(dc);
	nbg_dev_free(du);
	nbg_dev_free(ds);
	free_problem(&h);
	nbg_dropin_record_error(rc);
}
