/*
 * libnbots_host.so: standalone host objects behind nbots' public interfaces
 * for meshes, boundary conditions, materials and element types, for
 * programs (and tests) that use the drop-in FEM entry without nbots itself.
 * In a deployment next to libnbots.so this library is not loaded and the
 * same names resolve to nbots.
 *
 * Semantics follow nbots' public headers: a mesh answers the mesh2D.h
 * accessors; boundary conditions are four FIFO containers (Dirichlet/Neumann
 * x vertex/segment) walked by an iterator in push order (bcond.c:13,
 * bcond_iter.c); a constant atom's value is copied, a function atom's is
 * evaluated at the point given (bcond_iter.c:116-123).  Meshes are built
 * from arrays with nbh_mesh2D_create, which nbots has no counterpart for
 * (nbots builds them from its tessellator).
 */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "nbots_dropin.h"

/* ---------------------------------------------------------------- mesh */
struct nb_mesh2D_s {
	uint32_t nen, N_nod, N_elem, N_edg, N_vtx, N_sgm;
	double *nod;
	uint32_t *conn, *edg, *vtx, *sgm_ptr, *sgm_nodes;
};

static void *dup(const void *p, size_t n)
{
	void *q = malloc(n ? n : 1);
	if (q && n)
		memcpy(q, p, n);
	return q;
}

nb_mesh2D_t *nbh_mesh2D_create(uint32_t nen, uint32_t N_nod, const double *nod, uint32_t N_elem,
			       const uint32_t *conn, uint32_t N_edg, const uint32_t *edg,
			       uint32_t N_vtx, const uint32_t *vtx, uint32_t N_sgm,
			       const uint32_t *sgm_ptr, const uint32_t *sgm_nodes)
{
	nb_mesh2D_t *m = calloc(1, sizeof(*m));
	if (!m)
		return NULL;
	*m = (nb_mesh2D_t){nen, N_nod, N_elem, N_edg, N_vtx, N_sgm, NULL, NULL, NULL, NULL, NULL, NULL};
	m->nod = dup(nod, 16 * (size_t)N_nod);
	m->conn = dup(conn, 4 * (size_t)nen * N_elem);
	m->edg = dup(edg, 8 * (size_t)N_edg);
	m->vtx = dup(vtx, 4 * (size_t)N_vtx);
	m->sgm_ptr = dup(sgm_ptr, 4 * ((size_t)N_sgm + 1));
	m->sgm_nodes = dup(sgm_nodes, 4 * (size_t)sgm_ptr[N_sgm]);
	return m;
}

void nb_mesh2D_destroy(nb_mesh2D_t *m)
{
	if (!m)
		return;
	free(m->nod);
	free(m->conn);
	free(m->edg);
	free(m->vtx);
	free(m->sgm_ptr);
	free(m->sgm_nodes);
	free(m);
}

uint32_t nb_mesh2D_get_N_nodes(const nb_mesh2D_t *m) { return m->N_nod; }
uint32_t nb_mesh2D_get_N_edges(const nb_mesh2D_t *m) { return m->N_edg; }
uint32_t nb_mesh2D_get_N_elems(const nb_mesh2D_t *m) { return m->N_elem; }
uint32_t nb_mesh2D_get_N_invtx(const nb_mesh2D_t *m) { return m->N_vtx; }
uint32_t nb_mesh2D_get_N_insgm(const nb_mesh2D_t *m) { return m->N_sgm; }
double nb_mesh2D_node_get_x(const nb_mesh2D_t *m, uint32_t id) { return m->nod[2 * id]; }
double nb_mesh2D_node_get_y(const nb_mesh2D_t *m, uint32_t id) { return m->nod[2 * id + 1]; }
uint32_t nb_mesh2D_edge_get_1n(const nb_mesh2D_t *m, uint32_t id) { return m->edg[2 * id]; }
uint32_t nb_mesh2D_edge_get_2n(const nb_mesh2D_t *m, uint32_t id) { return m->edg[2 * id + 1]; }
uint32_t nb_mesh2D_elem_get_N_adj(const nb_mesh2D_t *m, uint32_t id) { (void)id; return m->nen; }

uint32_t nb_mesh2D_elem_get_adj(const nb_mesh2D_t *m, uint32_t elem_id, uint8_t adj_id)
{
	return m->conn[(size_t)elem_id * m->nen + adj_id];
}

uint32_t nb_mesh2D_get_invtx(const nb_mesh2D_t *m, uint32_t id) { return m->vtx[id]; }

uint32_t nb_mesh2D_insgm_get_N_nodes(const nb_mesh2D_t *m, uint32_t id)
{
	return m->sgm_ptr[id + 1] - m->sgm_ptr[id];
}

uint32_t nb_mesh2D_insgm_get_node(const nb_mesh2D_t *m, uint32_t sgm_id, uint32_t node_id)
{
	return m->sgm_nodes[m->sgm_ptr[sgm_id] + node_id];
}

/* mesh2D.c:650-674 */
static double dist(const nb_mesh2D_t *m, uint32_t a, uint32_t b)
{
	double dx = m->nod[2 * a] - m->nod[2 * b], dy = m->nod[2 * a + 1] - m->nod[2 * b + 1];
	return sqrt(dx * dx + dy * dy);
}

double nb_mesh2D_insgm_get_length(const nb_mesh2D_t *m, uint32_t sgm_id)
{
	uint32_t n = nb_mesh2D_insgm_get_N_nodes(m, sgm_id);
	return dist(m, nb_mesh2D_insgm_get_node(m, sgm_id, 0),
		    nb_mesh2D_insgm_get_node(m, sgm_id, n - 1));
}

double nb_mesh2D_insgm_subsgm_get_length(const nb_mesh2D_t *m, uint32_t sgm_id,
					 uint32_t subsgm_id)
{
	return dist(m, nb_mesh2D_insgm_get_node(m, sgm_id, subsgm_id),
		    nb_mesh2D_insgm_get_node(m, sgm_id, subsgm_id + 1));
}

/* ---------------------------------------------------------------- bcond */
typedef struct {
	uint32_t id;
	bool mask[2];
	double val[2];
	void (*fval)(const double *x, double t, double *out);
} atom_t;

typedef struct {
	atom_t *a;
	uint32_t n, cap;
} fifo_t;

struct nb_bcond_s {
	uint8_t N_dof;
	fifo_t c[4]; /* index = where * 2 + kind: D-vtx, N-vtx, D-sgm, N-sgm */
};

static int cat(nb_bcond_id type_id, nb_bcond_where type_elem)
{
	return (type_elem == NB_BC_ON_SEGMENT ? 2 : 0) + (type_id == NB_NEUMANN ? 1 : 0);
}

uint16_t nb_bcond_get_memsize(uint8_t N_dof)
{
	(void)N_dof;
	return (uint16_t)sizeof(struct nb_bcond_s);
}

void nb_bcond_init(void *ptr, uint8_t N_dof)
{
	memset(ptr, 0, sizeof(struct nb_bcond_s));
	((struct nb_bcond_s *)ptr)->N_dof = N_dof;
}

void nb_bcond_finish(void *ptr)
{
	struct nb_bcond_s *b = ptr;
	for (int k = 0; k < 4; k++) {
		free(b->c[k].a);
		b->c[k] = (fifo_t){NULL, 0, 0};
	}
}

void *nb_bcond_create(uint8_t N_dof)
{
	void *b = malloc(sizeof(struct nb_bcond_s));
	if (b)
		nb_bcond_init(b, N_dof);
	return b;
}

void nb_bcond_destroy(void *ptr)
{
	if (!ptr)
		return;
	nb_bcond_finish(ptr);
	free(ptr);
}

uint8_t nb_bcond_get_N_dof(const nb_bcond_t *b) { return b->N_dof; }

static atom_t *push(nb_bcond_t *b, nb_bcond_id t, nb_bcond_where w)
{
	fifo_t *f = &b->c[cat(t, w)];
	if (f->n == f->cap) {
		uint32_t c = f->cap ? 2 * f->cap : 8;
		atom_t *a = realloc(f->a, c * sizeof(atom_t));
		if (!a)
			return NULL;
		f->a = a;
		f->cap = c;
	}
	atom_t *a = &f->a[f->n++];
	memset(a, 0, sizeof(*a));
	return a;
}

void nb_bcond_push(nb_bcond_t *b, nb_bcond_id type_id, nb_bcond_where type_elem,
		   uint32_t elem_id, const bool dof_mask[], const double value[])
{
	atom_t *a = push(b, type_id, type_elem);
	if (!a)
		return;
	a->id = elem_id;
	for (int j = 0; j < 2 && j < b->N_dof; j++) {
		a->mask[j] = dof_mask[j];
		a->val[j] = value[j];
	}
}

void nb_bcond_push_function(nb_bcond_t *b, nb_bcond_id type_id, nb_bcond_where type_elem,
			    uint32_t elem_id, const bool dof_mask[],
			    void (*fval)(const double *x, double t, double *out))
{
	atom_t *a = push(b, type_id, type_elem);
	if (!a)
		return;
	a->id = elem_id;
	for (int j = 0; j < 2 && j < b->N_dof; j++)
		a->mask[j] = dof_mask[j];
	a->fval = fval;
}

struct nb_bcond_iter_s {
	const fifo_t *f;
	uint32_t next;
	const atom_t *cur;
};

uint16_t nb_bcond_iter_get_memsize(void) { return (uint16_t)sizeof(struct nb_bcond_iter_s); }
void nb_bcond_iter_init(void *p) { memset(p, 0, sizeof(struct nb_bcond_iter_s)); }
void nb_bcond_iter_finish(void *p) { memset(p, 0, sizeof(struct nb_bcond_iter_s)); }

void *nb_bcond_iter_create(void)
{
	return calloc(1, sizeof(struct nb_bcond_iter_s));
}

void nb_bcond_iter_destroy(void *p) { free(p); }

void nb_bcond_iter_set_conditions(nb_bcond_iter_t *it, const nb_bcond_t *b,
				  nb_bcond_id type_id, nb_bcond_where type_elem)
{
	it->f = &b->c[cat(type_id, type_elem)];
	it->next = 0;
	it->cur = NULL;
}

bool nb_bcond_iter_has_more(const nb_bcond_iter_t *it) { return it->f && it->next < it->f->n; }
void nb_bcond_iter_go_next(nb_bcond_iter_t *it) { it->cur = &it->f->a[it->next++]; }
uint32_t nb_bcond_iter_get_id(const nb_bcond_iter_t *it) { return it->cur->id; }
bool nb_bcond_iter_get_mask(const nb_bcond_iter_t *it, uint8_t j) { return it->cur->mask[j]; }
bool nb_bcond_iter_val_is_function(const nb_bcond_iter_t *it) { return it->cur->fval != NULL; }

void nb_bcond_iter_get_val(const nb_bcond_iter_t *it, uint8_t N_dof, double *x, double t,
			   double val[])
{
	if (it->cur->fval)
		it->cur->fval(x, t, val);
	else
		memcpy(val, it->cur->val, N_dof * sizeof(double));
}

/* ------------------------------------------------------------- material */
struct nb_material_s {
	double E, nu, density, ft, gf;
};

nb_material_t *nb_material_create(void) { return calloc(1, sizeof(nb_material_t)); }
void nb_material_destroy(nb_material_t *m) { free(m); }
void nb_material_set_elasticity_module(nb_material_t *m, double v) { m->E = v; }
void nb_material_set_poisson_module(nb_material_t *m, double v) { m->nu = v; }
void nb_material_set_density(nb_material_t *m, double v) { m->density = v; }
double nb_material_get_elasticity_module(const nb_material_t *m) { return m->E; }
double nb_material_get_poisson_module(const nb_material_t *m) { return m->nu; }
double nb_material_get_density(const nb_material_t *m) { return m->density; }
void nb_material_set_traction_limit_stress(nb_material_t *m, double v) { m->ft = v; }
void nb_material_set_fracture_energy(nb_material_t *m, double v) { m->gf = v; }
double nb_material_get_traction_limit_stress(const nb_material_t *m) { return m->ft; }
double nb_material_get_fracture_energy(const nb_material_t *m) { return m->gf; }

/* ------------------------------------------- implicit-solve parameters */
/* static_damage2D.c:27-125: four plain fields behind accessors */
struct nb_fem_implicit_s {
	uint32_t N_steps, N_max_iter, N_max_iter_without_enhance;
	double residual_tolerance;
};

nb_fem_implicit_t *nb_fem_implicit_create(void) { return calloc(1, sizeof(nb_fem_implicit_t)); }
void nb_fem_implicit_destroy(nb_fem_implicit_t *p) { free(p); }
void nb_fem_implicit_set_N_steps(nb_fem_implicit_t *p, uint32_t v) { p->N_steps = v; }
void nb_fem_implicit_set_N_max_iter(nb_fem_implicit_t *p, uint32_t v) { p->N_max_iter = v; }
void nb_fem_implicit_set_N_max_iter_without_enhance(nb_fem_implicit_t *p, uint32_t v)
{
	p->N_max_iter_without_enhance = v;
}
void nb_fem_implicit_set_residual_tolerance(nb_fem_implicit_t *p, double v)
{
	p->residual_tolerance = v;
}
uint32_t nb_fem_implicit_get_N_steps(nb_fem_implicit_t *p) { return p->N_steps; }
uint32_t nb_fem_implicit_get_N_max_iter(nb_fem_implicit_t *p) { return p->N_max_iter; }
uint32_t nb_fem_implicit_get_N_max_iter_without_enhance(nb_fem_implicit_t *p)
{
	return p->N_max_iter_without_enhance;
}
double nb_fem_implicit_get_residual_tolerance(nb_fem_implicit_t *p)
{
	return p->residual_tolerance;
}

/* -------------------------------------------------------------- element */
struct nb_fem_elem_s {
	nb_elem_id type;
	uint8_t N_nodes, N_gp;
};

/* element.c:16-33: T3 has 3 nodes and 1 Gauss point, Q4 4 and 4; unknown
 * types fall back to T3 */
nb_fem_elem_t *nb_fem_elem_create(nb_elem_id type)
{
	nb_fem_elem_t *e = calloc(1, sizeof(*e));
	if (!e)
		return NULL;
	if (type == NB_QUAD_LINEAR)
		*e = (nb_fem_elem_t){NB_QUAD_LINEAR, 4, 4};
	else
		*e = (nb_fem_elem_t){NB_TRG_LINEAR, 3, 1};
	return e;
}

void nb_fem_elem_destroy(nb_fem_elem_t *e) { free(e); }
uint8_t nb_fem_elem_get_N_nodes(const nb_fem_elem_t *e) { return e->N_nodes; }
uint8_t nb_fem_elem_get_N_gpoints(const nb_fem_elem_t *e) { return e->N_gp; }
