/*
 * Host side of the FEM path, in C: pattern and incidence builders, the
 * boundary-condition plan, and a device-resident FEM system that drives the
 * sm_103a kernels through the C ABI (include/nbots_gb300.h).
 *
 * The boundary conditions are applied in nbots' order
 * (pde_bot/finite_element/solid_mechanics/set_bconditions.c:52-61):
 * Neumann on segments, Neumann on vertices, Dirichlet on segments,
 * Dirichlet on vertices, each group in push order.  The host turns the
 * Neumann loops into an ordered list of load increments (computed with the
 * same expressions, so the same bits) and the Dirichlet loops into an ordered
 * list of (dof, value) events; the device applies both.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "nbots_gb300.h"

#include "fem_internal.h"

static int cmp_u32(const void *a, const void *b)
{
	uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
	return x < y ? -1 : (x > y);
}

int nbg_host_pattern(const nbg_mesh_t *m, uint32_t *row_ptr, uint32_t *col_idx)
{
	const uint32_t Nn = m->N_nod, nen = m->nen;
	uint32_t *deg = calloc(Nn + 1, sizeof(uint32_t));
	if (!deg)
		return NBG_ERR_NOMEM;
	/* graph degree: both ends of each edge, plus (nen - 3) opposite-corner
	 * links per node of an element with more than three nodes
	 * (load_graph.c:263-286) */
	for (uint32_t i = 0; i < m->N_edg; i++) {
		deg[m->edg[2 * i]]++;
		deg[m->edg[2 * i + 1]]++;
	}
	if (nen > 3)
		for (uint64_t t = 0; t < (uint64_t)m->N_elem * nen; t++)
			deg[m->conn[t]] += nen - 3;
	row_ptr[0] = 0;
	for (uint32_t i = 0; i < Nn; i++) {
		uint32_t width = 2 * (deg[i] + 1);
		row_ptr[2 * i + 1] = row_ptr[2 * i] + width;
		row_ptr[2 * i + 2] = row_ptr[2 * i + 1] + width;
	}
	if (!col_idx) {
		free(deg);
		return NBG_OK;
	}
	/* fill: neighbours in graph order, then self, both dofs; sort row 2i
	 * and copy it to row 2i+1 (both rows list the same columns) */
	uint32_t *fill = calloc(Nn + 1, sizeof(uint32_t));
	if (!fill) {
		free(deg);
		return NBG_ERR_NOMEM;
	}
#define PUSH(a, w) do { uint32_t *r_ = col_idx + row_ptr[2 * (a)]; \
		r_[fill[a]++] = 2 * (w); r_[fill[a]++] = 2 * (w) + 1; } while (0)
	for (uint32_t i = 0; i < m->N_edg; i++) {
		uint32_t a = m->edg[2 * i], b = m->edg[2 * i + 1];
		PUSH(a, b);
		PUSH(b, a);
	}
	if (nen > 3)
		for (uint32_t e = 0; e < m->N_elem; e++)
			for (uint32_t i = 0; i < nen; i++)
				for (uint32_t j = 0; j + 3 < nen; j++)
					PUSH(m->conn[e * nen + i], m->conn[e * nen + (i + j + 2) % nen]);
	for (uint32_t i = 0; i < Nn; i++) {
		PUSH(i, i);
		uint32_t *r0 = col_idx + row_ptr[2 * i];
		uint32_t w = row_ptr[2 * i + 1] - row_ptr[2 * i];
		qsort(r0, w, sizeof(uint32_t), cmp_u32);
		memcpy(col_idx + row_ptr[2 * i + 1], r0, w * sizeof(uint32_t));
	}
#undef PUSH
	free(fill);
	free(deg);
	return NBG_OK;
}

int nbg_host_incidence(const nbg_mesh_t *m, uint32_t *inc_ptr, uint32_t *inc_elem,
		       uint8_t *inc_local)
{
	const uint32_t Nn = m->N_nod, nen = m->nen;
	memset(inc_ptr, 0, (Nn + 1) * sizeof(uint32_t));
	for (uint64_t t = 0; t < (uint64_t)m->N_elem * nen; t++) {
		if (m->conn[t] >= Nn)
			return NBG_ERR_ARG;
		inc_ptr[m->conn[t] + 1]++;
	}
	for (uint32_t i = 0; i < Nn; i++)
		inc_ptr[i + 1] += inc_ptr[i];
	uint32_t *pos = malloc((Nn + 1) * sizeof(uint32_t));
	if (!pos)
		return NBG_ERR_NOMEM;
	memcpy(pos, inc_ptr, (Nn + 1) * sizeof(uint32_t));
	for (uint32_t e = 0; e < m->N_elem; e++)
		for (uint32_t i = 0; i < nen; i++) {
			uint32_t n = m->conn[e * nen + i];
			inc_elem[pos[n]] = e;
			inc_local[pos[n]] = (uint8_t)i;
			pos[n]++;
		}
	free(pos);
	return NBG_OK;
}

/* ------------------------------------------------------------- bc plan */
typedef struct {
	uint32_t n_inc, cap_inc;
	uint32_t *inc_idx;
	double *inc_val;
	uint32_t n_ev, cap_ev;
	uint32_t *ev_dof;
	double *ev_val;
} plan_t;

static int plan_inc(plan_t *p, uint32_t idx, double v)
{
	if (p->n_inc == p->cap_inc) {
		uint32_t c = p->cap_inc ? 2 * p->cap_inc : 256;
		uint32_t *a = realloc(p->inc_idx, c * sizeof(uint32_t));
		double *b = realloc(p->inc_val, c * sizeof(double));
		if (!a || !b) { free(a ? a : p->inc_idx); free(b ? b : p->inc_val); p->inc_idx = NULL; p->inc_val = NULL; return NBG_ERR_NOMEM; }
		p->inc_idx = a;
		p->inc_val = b;
		p->cap_inc = c;
	}
	p->inc_idx[p->n_inc] = idx;
	p->inc_val[p->n_inc] = v;
	p->n_inc++;
	return NBG_OK;
}

static int plan_ev(plan_t *p, uint32_t dof, double v)
{
	if (p->n_ev == p->cap_ev) {
		uint32_t c = p->cap_ev ? 2 * p->cap_ev : 256;
		uint32_t *a = realloc(p->ev_dof, c * sizeof(uint32_t));
		double *b = realloc(p->ev_val, c * sizeof(double));
		if (!a || !b) { free(a ? a : p->ev_dof); free(b ? b : p->ev_val); p->ev_dof = NULL; p->ev_val = NULL; return NBG_ERR_NOMEM; }
		p->ev_dof = a;
		p->ev_val = b;
		p->cap_ev = c;
	}
	p->ev_dof[p->n_ev] = dof;
	p->ev_val[p->n_ev] = v;
	p->n_ev++;
	return NBG_OK;
}

static double dist(const double *nod, uint32_t a, uint32_t b)
{
	/* nb_mesh2D_insgm_subsgm_get_length (mesh2D.c:663-674) */
	double dx = nod[2 * a] - nod[2 * b], dy = nod[2 * a + 1] - nod[2 * b + 1];
	return sqrt(dx * dx + dy * dy);
}

static int build_plan(const nbg_mesh_t *m, const nbg_bcs_t *b, double factor, plan_t *p)
{
	int rc = NBG_OK;
	memset(p, 0, sizeof(*p));
	static const uint32_t grp[4][2] = {{1, 1}, {1, 0}, {0, 1}, {0, 0}};
	for (int g = 0; g < 4 && rc == NBG_OK; g++) {
		for (uint32_t a = 0; a < b->N_bc && rc == NBG_OK; a++) {
			const nbg_bc_t *bc = &b->bc[a];
			if (bc->kind != grp[g][0] || bc->where != grp[g][1])
				continue;
			const int fn = bc->n_nv > 0;
			if (bc->where == 1 && bc->id >= b->N_sgm)
				return NBG_ERR_ARG;
			const uint32_t *sn = bc->where == 1 ? b->sgm_nodes + b->sgm_ptr[bc->id] : NULL;
			const uint32_t n = bc->where == 1 ? b->sgm_ptr[bc->id + 1] - b->sgm_ptr[bc->id] : 1;
			if (fn && bc->n_nv < n)
				return NBG_ERR_ARG;
			if (g == 0 && fn) {
				/* set_neumann_sgm_function (set_bconditions.c:87-131) */
				for (uint32_t i = 0; i + 1 < n && rc == NBG_OK; i++) {
					double l = dist(m->nod, sn[i], sn[i + 1]);
					for (int j = 0; j < 2 && rc == NBG_OK; j++) {
						if (!bc->mask[j])
							continue;
						double val = 0.5 * (bc->node_vals[2 * i + j] +
								    bc->node_vals[2 * (i + 1) + j]) * l;
						rc = plan_inc(p, sn[i] * 2 + j, factor * val * 0.5);
						if (rc == NBG_OK)
							rc = plan_inc(p, sn[i + 1] * 2 + j, factor * val * 0.5);
					}
				}
			} else if (g == 0) {
				/* set_neumann_sgm_integrated (:133-154): a total force spread
				 * by sub-segment length */
				double L = dist(m->nod, sn[0], sn[n - 1]);
				for (uint32_t i = 0; i + 1 < n && rc == NBG_OK; i++) {
					double w = dist(m->nod, sn[i], sn[i + 1]) / L;
					double f = factor * w * 0.5;
					for (int j = 0; j < 2 && rc == NBG_OK; j++)
						if (bc->mask[j])
							rc = plan_inc(p, sn[i] * 2 + j, f * bc->val[j]);
					for (int j = 0; j < 2 && rc == NBG_OK; j++)
						if (bc->mask[j])
							rc = plan_inc(p, sn[i + 1] * 2 + j, f * bc->val[j]);
				}
			} else if (g == 1) {
				/* set_neumann_vtx (:173-190) */
				uint32_t v = b->vtx[bc->id];
				for (int j = 0; j < 2 && rc == NBG_OK; j++)
					if (bc->mask[j])
						rc = plan_inc(p, v * 2 + j,
							      factor * (fn ? bc->node_vals[j] : bc->val[j]));
			} else {
				/* set_dirichlet_sgm / set_dirichlet_vtx (:192-260) */
				for (uint32_t i = 0; i < n && rc == NBG_OK; i++) {
					uint32_t v = bc->where == 1 ? sn[i] : b->vtx[bc->id];
					for (int j = 0; j < 2 && rc == NBG_OK; j++)
						if (bc->mask[j])
							rc = plan_ev(p, v * 2 + j,
								     factor * (fn ? bc->node_vals[2 * i + j] : bc->val[j]));
				}
			}
		}
	}
	return rc;
}

static void plan_free(plan_t *p)
{
	free(p->inc_idx);
	free(p->inc_val);
	free(p->ev_dof);
	free(p->ev_val);
}

/* ------------------------------------------------------------ fem system */
#define TRY(x) do { int rc_ = (x); if (rc_ != NBG_OK) { rc = rc_; goto fail; } } while (0)

uint32_t nbg_fem_n_dof(const nbg_fem_t *f) { return f->N; }
uint64_t nbg_fem_nnz(const nbg_fem_t *f) { return f->nnz; }

static uint32_t n_gp(const nbg_fem_t *f) { return f->m.nen == 4 ? 4 : 1; }

void nbg_fem_destroy(nbg_fem_t *f)
{
	if (!f)
		return;
	if (f->borrowed_csr)
		f->row_ptr = NULL, f->col_idx = NULL, f->K = NULL;
	void *p[] = {f->nod, f->K, f->F, f->u, f->strain, f->stress, f->E, f->Ke, f->Fe, f->main_stress,
		     f->damage,
		     f->conn, f->row_ptr, f->col_idx, f->inc_ptr, f->inc_elem, f->distorted,
		     f->inc_local, f->enabled, f->matched, f->status, f->cg_ws,
		     f->slice_off, f->bcol, f->b64, f->dinv64, f->b32, f->dinv32, f->blo, f->bxt,
		     f->perm, f->iperm, f->simp_rho, f->simp_out, f->simp_e, f->simp_lam};
	for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); i++)
		nbg_dev_free(p[i]);
	free(f);
}

int nbg_fem_create_on_csr(nbg_fem_t **out, const nbg_mesh_t *m, uint64_t nnz,
			  uint32_t *row_ptr, uint32_t *col_idx, double *K, int need_incidence,
			  void *stream)
{
	int rc = NBG_OK;
	*out = NULL;
	if (!m || (m->nen != 3 && m->nen != 4) || m->N_nod == 0)
		return NBG_ERR_ARG;
	nbg_fem_t *f = calloc(1, sizeof(*f));
	if (!f)
		return NBG_ERR_NOMEM;
	f->m = *m;
	f->m.nod = NULL;
	f->m.conn = NULL;
	f->m.edg = NULL;
	f->stream = stream;
	f->N = 2 * m->N_nod;
	f->nnz = nnz;
	f->row_ptr = row_ptr;
	f->col_idx = col_idx;
	f->K = K;
	f->borrowed_csr = 1;
	const size_t ne = m->N_elem, nen = m->nen, Nn = m->N_nod;
	uint32_t *ip = NULL, *ie = NULL;
	uint8_t *il = NULL;
	TRY(nbg_dev_alloc((void **)&f->nod, 16 * Nn));
	TRY(nbg_dev_alloc((void **)&f->conn, 4 * (ne ? ne : 1) * nen));
	TRY(nbg_dev_alloc((void **)&f->F, 8 * (size_t)f->N));
	TRY(nbg_dev_alloc((void **)&f->u, 8 * (size_t)f->N));
	TRY(nbg_dev_alloc((void **)&f->E, 8 * (ne ? ne : 1)));
	TRY(nbg_dev_alloc((void **)&f->enabled, ne ? ne : 1));
	TRY(nbg_dev_alloc((void **)&f->strain, 8 * 3 * (ne ? ne : 1) * (nen == 4 ? 4 : 1)));
	TRY(nbg_dev_alloc((void **)&f->stress, 8 * 3 * (ne ? ne : 1) * (nen == 4 ? 4 : 1)));
	TRY(nbg_dev_alloc((void **)&f->distorted, 256));
	TRY(nbg_dev_alloc((void **)&f->matched, 256));
	TRY(nbg_dev_alloc((void **)&f->status, 256));
	TRY(nbg_h2d(f->nod, m->nod, 16 * Nn, stream));
	TRY(nbg_h2d(f->conn, m->conn, 4 * ne * nen, stream));
	if (need_incidence) {
		ip = malloc(4 * (Nn + 1));
		ie = malloc(4 * (ne ? ne : 1) * nen);
		il = malloc((ne ? ne : 1) * nen);
		if (!ip || !ie || !il)
			TRY(NBG_ERR_NOMEM);
		TRY(nbg_host_incidence(m, ip, ie, il));
		TRY(nbg_dev_alloc((void **)&f->inc_ptr, 4 * (Nn + 1)));
		TRY(nbg_dev_alloc((void **)&f->inc_elem, 4 * (ne ? ne : 1) * nen));
		TRY(nbg_dev_alloc((void **)&f->inc_local, (ne ? ne : 1) * nen));
		TRY(nbg_h2d(f->inc_ptr, ip, 4 * (Nn + 1), stream));
		TRY(nbg_h2d(f->inc_elem, ie, 4 * ne * nen, stream));
		TRY(nbg_h2d(f->inc_local, il, ne * nen, stream));
	}
	TRY(nbg_stream_sync(stream));
	free(ip);
	free(ie);
	free(il);
	*out = f;
	return NBG_OK;
fail:
	free(ip);
	free(ie);
	free(il);
	nbg_fem_destroy(f);
	return rc;
}

int nbg_fem_create(nbg_fem_t **out, const nbg_mesh_t *m, void *stream)
{
	int rc = NBG_OK;
	*out = NULL;
	if (!m || (m->nen != 3 && m->nen != 4) || m->N_nod == 0)
		return NBG_ERR_ARG;
	nbg_fem_t *f = calloc(1, sizeof(*f));
	if (!f)
		return NBG_ERR_NOMEM;
	f->m = *m;
	f->m.nod = NULL;
	f->m.conn = NULL;
	f->m.edg = NULL;
	f->stream = stream;
	f->N = 2 * m->N_nod;
	const size_t ne = m->N_elem, nen = m->nen, Nn = m->N_nod;
	const uint32_t S = (m->N_nod + 31) / 32;
	void *edg_d = NULL;
	TRY(nbg_dev_alloc((void **)&f->nod, 16 * Nn));
	TRY(nbg_dev_alloc((void **)&f->conn, 4 * ne * nen));
	TRY(nbg_dev_alloc((void **)&f->row_ptr, 4 * ((size_t)f->N + 1)));
	TRY(nbg_dev_alloc((void **)&f->inc_ptr, 4 * (Nn + 1)));
	TRY(nbg_dev_alloc((void **)&f->inc_elem, 4 * ne * nen));
	TRY(nbg_dev_alloc((void **)&f->inc_local, ne * nen));
	TRY(nbg_dev_alloc((void **)&f->F, 8 * (size_t)f->N));
	TRY(nbg_dev_alloc((void **)&f->u, 8 * (size_t)f->N));
	TRY(nbg_dev_alloc((void **)&f->E, 8 * ne));
	TRY(nbg_dev_alloc((void **)&f->enabled, ne));
	TRY(nbg_dev_alloc((void **)&f->strain, 8 * 3 * ne * (nen == 4 ? 4 : 1)));
	TRY(nbg_dev_alloc((void **)&f->stress, 8 * 3 * ne * (nen == 4 ? 4 : 1)));
	TRY(nbg_dev_alloc((void **)&f->distorted, 256));
	TRY(nbg_dev_alloc((void **)&f->matched, 256));
	TRY(nbg_dev_alloc((void **)&f->status, 256));
	TRY(nbg_dev_alloc((void **)&f->slice_off, 4 * ((size_t)S + 1)));
	TRY(nbg_dev_alloc(&edg_d, 8 * (size_t)(m->N_edg ? m->N_edg : 1)));
	TRY(nbg_h2d(f->nod, m->nod, 16 * Nn, stream));
	TRY(nbg_h2d(f->conn, m->conn, 4 * ne * nen, stream));
	TRY(nbg_h2d(edg_d, m->edg, 8 * (size_t)m->N_edg, stream));
	/* pattern, incidence and block plan, built on the device (pattern.cu) */
	TRY(nbg_pattern_dev(m->nen, m->N_nod, m->N_elem, m->N_edg, f->conn, edg_d, f->row_ptr,
			    &f->col_idx, &f->nnz, f->inc_ptr, f->inc_elem, f->inc_local,
			    f->slice_off, stream));
	nbg_dev_free(edg_d);
	edg_d = NULL;
	TRY(nbg_dev_alloc((void **)&f->K, 8 * f->nnz));
	{
		/* block layout of the fixed pattern: every node row pairs its two
		 * dof rows by construction, so the plan always applies */
		uint32_t wS = 0;
		TRY(nbg_d2h(&wS, f->slice_off + S, 4, stream));
		TRY(nbg_stream_sync(stream));
		const uint64_t ent = 32ull * wS;
		TRY(nbg_dev_alloc((void **)&f->bcol, 4 * ent));
		f->bsr.N = f->N;
		f->bsr.Nn = m->N_nod;
		f->bsr.n_slices = S;
		f->bsr.n_entries = ent;
		f->bsr.slice_off = f->slice_off;
		f->bsr.bcol = f->bcol;
		f->bsr_ok = 1;
	}
	TRY(nbg_stream_sync(stream));
	*out = f;
	return NBG_OK;
fail:
	nbg_dev_free(edg_d);
	nbg_fem_destroy(f);
	return rc;
}

int nbg_fem_assemble(nbg_fem_t *f, const double *E, double nu, double thickness,
		     double density, int self_weight, const double gravity[2],
		     const uint8_t *enabled)
{
	if (!E)
		return NBG_ERR_ARG;
	return nbg_fem_assemble_dev_damage(f, E, nu, thickness, density, self_weight, gravity,
					   enabled, NULL);
}

int nbg_fem_assemble_dev_damage(nbg_fem_t *f, const double *E, double nu, double thickness,
				double density, int self_weight, const double gravity[2],
				const uint8_t *enabled, const double *damage)
{
	int rc = NBG_OK;
	const size_t ne = f->m.N_elem, nen = f->m.nen, nd = 2 * nen;
	if (!f->Ke) {
		TRY(nbg_dev_alloc((void **)&f->Ke, 8 * nd * nd * (ne ? ne : 1)));
		TRY(nbg_dev_alloc((void **)&f->Fe, 8 * nd * (ne ? ne : 1)));
	}
	f->nu = nu;
	f->has_enabled = enabled != NULL;
	if (E)  /* else the moduli are already in f->E */
		TRY(nbg_h2d(f->E, E, 8 * ne, f->stream));
	if (enabled)
		TRY(nbg_h2d(f->enabled, enabled, ne, f->stream));
	uint32_t init = 0xffffffffu;
	unsigned long long zero = 0;
	TRY(nbg_h2d(f->distorted, &init, 4, f->stream));
	TRY(nbg_h2d(f->matched, &zero, 8, f->stream));
	double gx = gravity ? gravity[0] : 0.0, gy = gravity ? gravity[1] : 0.0;
	TRY(nbg_element_stiffness_damage_f64((uint32_t)nen, (uint32_t)ne, f->nod, f->conn, f->E,
					     nu, thickness, density, self_weight, gx, gy,
					     enabled ? f->enabled : NULL, damage, f->Ke, f->Fe,
					     f->distorted, f->stream));
	uint32_t dist_h = 0;
	TRY(nbg_d2h(&dist_h, f->distorted, 4, f->stream));
	TRY(nbg_stream_sync(f->stream));
	if (dist_h != 0xffffffffu)
		return NBG_DISTORTED;
	TRY(nbg_gather_assemble_f64((uint32_t)nen, f->m.N_nod, (uint32_t)ne, f->inc_ptr,
				    f->inc_elem, f->inc_local, f->row_ptr, f->col_idx, f->Ke,
				    f->Fe, f->K, f->F, f->matched, f->stream));
	unsigned long long matched = 0;
	TRY(nbg_d2h(&matched, f->matched, 8, f->stream));
	TRY(nbg_stream_sync(f->stream));
	if (matched != (unsigned long long)ne * nen * nen)
		return NBG_ERR_PATTERN;
	return NBG_OK;
fail:
	return rc;
}

int nbg_fem_apply_bcs(nbg_fem_t *f, const nbg_bcs_t *b, double factor)
{
	int rc = NBG_OK;
	plan_t p;
	memset(&p, 0, sizeof(p));  /* the fail path frees its arrays */
	uint32_t *gidx = NULL, *gptr = NULL, *order = NULL, *cnt = NULL;
	uint32_t *ev_ptr = NULL, *ev_of = NULL;
	double *ginc = NULL;
	void *d_gidx = NULL, *d_gptr = NULL, *d_ginc = NULL, *d_evptr = NULL, *d_evof = NULL,
	     *d_evval = NULL;
	nbg_mesh_t mh = f->m;
	/* segment lengths need the coordinates on the host */
	double *nod = malloc(16 * (size_t)f->m.N_nod);
	if (!nod)
		return NBG_ERR_NOMEM;
	TRY(nbg_d2h(nod, f->nod, 16 * (size_t)f->m.N_nod, f->stream));
	TRY(nbg_stream_sync(f->stream));
	mh.nod = nod;
	TRY(build_plan(&mh, b, factor, &p));

	const uint32_t N = f->N;
	if (p.n_inc) {
		/* group increments by index, keeping their order within a group */
		cnt = calloc((size_t)N + 1, sizeof(uint32_t));
		order = malloc(p.n_inc * sizeof(uint32_t));
		ginc = malloc(p.n_inc * sizeof(double));
		if (!cnt || !order || !ginc)
			TRY(NBG_ERR_NOMEM);
		for (uint32_t k = 0; k < p.n_inc; k++) {
			if (p.inc_idx[k] >= N)
				TRY(NBG_ERR_ARG);
			cnt[p.inc_idx[k] + 1]++;
		}
		uint32_t ng = 0;
		for (uint32_t i = 0; i < N; i++)
			ng += cnt[i + 1] != 0;
		gidx = malloc(ng * sizeof(uint32_t));
		gptr = malloc((ng + 1) * sizeof(uint32_t));
		if (!gidx || !gptr)
			TRY(NBG_ERR_NOMEM);
		for (uint32_t i = 0; i < N; i++)
			cnt[i + 1] += cnt[i];
		for (uint32_t k = 0; k < p.n_inc; k++)
			ginc[cnt[p.inc_idx[k]]++] = p.inc_val[k];
		/* cnt[i] is now the end of index i's run */
		uint32_t g = 0, start = 0;
		gptr[0] = 0;
		for (uint32_t i = 0; i < N; i++) {
			if (cnt[i] != start) {
				gidx[g] = i;
				gptr[g + 1] = cnt[i];
				g++;
				start = cnt[i];
			}
		}
		TRY(nbg_dev_alloc(&d_gidx, 4 * (size_t)ng));
		TRY(nbg_dev_alloc(&d_gptr, 4 * ((size_t)ng + 1)));
		TRY(nbg_dev_alloc(&d_ginc, 8 * (size_t)p.n_inc));
		TRY(nbg_h2d(d_gidx, gidx, 4 * (size_t)ng, f->stream));
		TRY(nbg_h2d(d_gptr, gptr, 4 * ((size_t)ng + 1), f->stream));
		TRY(nbg_h2d(d_ginc, ginc, 8 * (size_t)p.n_inc, f->stream));
		TRY(nbg_apply_increments_f64(ng, d_gidx, d_gptr, d_ginc, f->F, f->stream));
	}
	if (p.n_ev) {
		ev_ptr = calloc((size_t)N + 1, sizeof(uint32_t));
		ev_of = malloc(p.n_ev * sizeof(uint32_t));
		if (!ev_ptr || !ev_of)
			TRY(NBG_ERR_NOMEM);
		for (uint32_t k = 0; k < p.n_ev; k++) {
			if (p.ev_dof[k] >= N)
				TRY(NBG_ERR_ARG);
			ev_ptr[p.ev_dof[k] + 1]++;
		}
		for (uint32_t i = 0; i < N; i++)
			ev_ptr[i + 1] += ev_ptr[i];
		uint32_t *pos = malloc(((size_t)N + 1) * sizeof(uint32_t));
		if (!pos)
			TRY(NBG_ERR_NOMEM);
		memcpy(pos, ev_ptr, ((size_t)N + 1) * sizeof(uint32_t));
		for (uint32_t k = 0; k < p.n_ev; k++)
			ev_of[pos[p.ev_dof[k]]++] = k;
		free(pos);
		int zero = 0;
		TRY(nbg_h2d(f->status, &zero, sizeof(int), f->stream));
		TRY(nbg_dev_alloc(&d_evptr, 4 * ((size_t)N + 1)));
		TRY(nbg_dev_alloc(&d_evof, 4 * (size_t)p.n_ev));
		TRY(nbg_dev_alloc(&d_evval, 8 * (size_t)p.n_ev));
		TRY(nbg_h2d(d_evptr, ev_ptr, 4 * ((size_t)N + 1), f->stream));
		TRY(nbg_h2d(d_evof, ev_of, 4 * (size_t)p.n_ev, f->stream));
		TRY(nbg_h2d(d_evval, p.ev_val, 8 * (size_t)p.n_ev, f->stream));
		TRY(nbg_dirichlet_f64(N, f->row_ptr, f->col_idx, f->K, f->F, d_evptr, d_evof,
				      d_evval, f->status, f->stream));
		int st = 0;
		TRY(nbg_d2h(&st, f->status, sizeof(int), f->stream));
		TRY(nbg_stream_sync(f->stream));
		if (st)
			TRY(st);
	}
	TRY(nbg_stream_sync(f->stream));
fail:
	plan_free(&p);
	free(nod); free(cnt); free(order); free(ginc); free(gidx); free(gptr);
	free(ev_ptr); free(ev_of);
	nbg_dev_free(d_gidx); nbg_dev_free(d_gptr); nbg_dev_free(d_ginc);
	nbg_dev_free(d_evptr); nbg_dev_free(d_evof); nbg_dev_free(d_evval);
	return rc;
}

int nbg_fem_cg_workspace(nbg_fem_t *f)
{
	int rc = NBG_OK;
	size_t need = nbg_cg_workspace_bytes(f->N);
	if (f->cg_ws_bytes < need) {
		nbg_dev_free(f->cg_ws);
		f->cg_ws = NULL;
		f->cg_ws_bytes = 0;
		TRY(nbg_dev_alloc(&f->cg_ws, need));
		f->cg_ws_bytes = need;
	}
fail:
	return rc;
}

int nbg_fem_solve(nbg_fem_t *f, uint32_t max_iter, double tol, unsigned flags,
		  nbg_cg_result_t *res)
{
	int rc = nbg_fem_cg_workspace(f);
	if (rc != NBG_OK)
		return rc;
	double *zero = calloc(f->N ? f->N : 1, sizeof(double));
	if (!zero)
		return NBG_ERR_NOMEM;
	rc = nbg_h2d(f->u, zero, 8 * (size_t)f->N, f->stream);
	if (rc == NBG_OK)
		rc = nbg_stream_sync(f->stream);
	free(zero);
	if (rc != NBG_OK)
		return rc;
	return nbg_cg_f64(f->N, f->row_ptr, f->col_idx, f->K, f->F, f->u, max_iter, tol, flags,
			  res, f->cg_ws, f->cg_ws_bytes, f->stream);
}

int nbg_fem_set_block_order(nbg_fem_t *f, int order, uint32_t sigma)
{
	if (!f || order < NBG_ORDER_AUTO || order > NBG_ORDER_SIGMA || sigma > 1024)
		return NBG_ERR_ARG;
	if (f->b64)  /* fixed by the first layout */
		return order == f->block_order ? NBG_OK : NBG_ERR_ARG;
	f->block_order = order;
	f->block_sigma = sigma;
	return NBG_OK;
}

/* The SELL-C-sigma order (pattern.cu). */
static int choose_order(nbg_fem_t *f)
{
	int rc = NBG_OK;
	const uint32_t Nn = f->m.N_nod, S = f->bsr.n_slices;
	uint32_t *so = NULL;
	TRY(nbg_dev_alloc((void **)&f->perm, 4 * (size_t)Nn));
	TRY(nbg_dev_alloc((void **)&f->iperm, 4 * (size_t)Nn));
	TRY(nbg_dev_alloc((void **)&so, 4 * ((size_t)S + 1)));
	TRY(nbg_bsr_plan_sigma_dev(Nn, f->row_ptr, f->block_sigma ? f->block_sigma : 512, f->perm,
				   f->iperm, so, f->stream));
	uint32_t w_sigma = 0;
	TRY(nbg_d2h(&w_sigma, so + S, 4, f->stream));
	TRY(nbg_d2d(f->slice_off, so, 4 * ((size_t)S + 1), f->stream));
	TRY(nbg_stream_sync(f->stream));
	f->bsr.n_entries = 32ull * w_sigma;  /* bcol keeps its larger allocation */
	f->bsr.perm = f->perm;
	f->bsr.iperm = f->iperm;
fail:
	nbg_dev_free(so);
	return rc;
}

int nbg_fem_block_layout(nbg_fem_t *f, nbg_bsr_t *out)
{
	int rc = NBG_OK;
	if (!f->bsr_ok)
		return NBG_ERR_PATTERN;
	if (!f->b64 && f->block_order == NBG_ORDER_SIGMA)
		TRY(choose_order(f));
	const uint64_t ent = f->bsr.n_entries;
	if (!f->b64) {
		TRY(nbg_dev_alloc((void **)&f->b64, 32 * ent));
		TRY(nbg_dev_alloc((void **)&f->b32, 16 * ent));
		TRY(nbg_dev_alloc((void **)&f->blo, 8 * ent));
		TRY(nbg_dev_alloc((void **)&f->bxt, 4 * ent));
		TRY(nbg_dev_alloc((void **)&f->dinv64, 8 * (size_t)f->N));
		TRY(nbg_dev_alloc((void **)&f->dinv32, 4 * (size_t)f->N));
		f->bsr.b64 = f->b64;
		f->bsr.b32 = f->b32;
		f->bsr.blo = f->blo;
		f->bsr.bxt = f->bxt;
		f->bsr.dinv64 = f->dinv64;
		f->bsr.dinv32 = f->dinv32;
	}
	TRY(nbg_bsr_fill(&f->bsr, f->row_ptr, f->col_idx, f->K, f->stream));
	TRY(nbg_stream_sync(f->stream));
	if (out)
		*out = f->bsr;
	return NBG_OK;
fail:
	return rc;
}

static int zero_u(nbg_fem_t *f)
{
	double *zero = calloc(f->N ? f->N : 1, sizeof(double));
	if (!zero)
		return NBG_ERR_NOMEM;
	int rc = nbg_h2d(f->u, zero, 8 * (size_t)f->N, f->stream);
	if (rc == NBG_OK)
		rc = nbg_stream_sync(f->stream);
	free(zero);
	return rc;
}

static int ensure_ws(nbg_fem_t *f, size_t need)
{
	if (f->cg_ws_bytes >= need)
		return NBG_OK;
	nbg_dev_free(f->cg_ws);
	f->cg_ws = NULL;
	f->cg_ws_bytes = 0;
	int rc = nbg_dev_alloc(&f->cg_ws, need);
	if (rc == NBG_OK)
		f->cg_ws_bytes = need;
	return rc;
}

int nbg_fem_solve_fast(nbg_fem_t *f, uint32_t max_iter, double tol, unsigned flags,
		       nbg_cg_result_t *res)
{
	int rc = NBG_OK;
	TRY(nbg_fem_block_layout(f, NULL));
	TRY(ensure_ws(f, nbg_cg_bsr_workspace_bytes(f->N)));
	TRY(zero_u(f));
	return nbg_cg_bsr_f64(&f->bsr, f->F, f->u, max_iter, tol, flags, res, f->cg_ws,
			      f->cg_ws_bytes, f->stream);
fail:
	return rc;
}

int nbg_fem_solve_mixed(nbg_fem_t *f, uint32_t max_iter, double tol, double delta,
			unsigned flags, nbg_mixed_result_t *res)
{
	int rc = NBG_OK;
	TRY(nbg_fem_block_layout(f, NULL));
	TRY(ensure_ws(f, nbg_cg_mixed_layout_workspace_bytes(&f->bsr)));
	TRY(zero_u(f));
	return nbg_cg_mixed(&f->bsr, f->F, f->u, max_iter, tol, delta, flags, res, f->cg_ws,
			    f->cg_ws_bytes, f->stream);
fail:
	return rc;
}

int nbg_fem_strain(nbg_fem_t *f)
{
	return nbg_strain_f64(f->m.nen, f->m.N_elem, f->nod, f->conn, f->u, f->strain, f->stream);
}

int nbg_fem_stress(nbg_fem_t *f)
{
	return nbg_stress_f64(f->m.nen, f->m.N_elem, f->E, f->nu,
			      f->has_enabled ? f->enabled : NULL, f->strain, f->stress, f->stream);
}

int nbg_fem_main_stress(nbg_fem_t *f)
{
	if (!f->main_stress) {
		int rc = nbg_dev_alloc((void **)&f->main_stress,
				       16 * (size_t)n_gp(f) * (f->m.N_elem ? f->m.N_elem : 1));
		if (rc != NBG_OK)
			return rc;
	}
	return nbg_main_stress_f64(f->m.nen, f->m.N_elem, f->stress, f->main_stress, f->stream);
}

void *nbg_fem_device_ptr(nbg_fem_t *f, int what)
{
	switch (what) {
	case NBG_FEM_ROW_PTR: return f->row_ptr;
	case NBG_FEM_COL_IDX: return f->col_idx;
	case NBG_FEM_K: return f->K;
	case NBG_FEM_F: return f->F;
	case NBG_FEM_U: return f->u;
	case NBG_FEM_STRAIN: return f->strain;
	case NBG_FEM_STRESS: return f->stress;
	case NBG_FEM_MAIN_STRESS: return f->main_stress;
	case NBG_FEM_DAMAGE: return f->damage;
	case NBG_FEM_E: return f->E;
	case NBG_FEM_NOD: return f->nod;
	case NBG_FEM_CONN: return f->conn;
	default: return NULL;
	}
}

size_t nbg_fem_bytes(const nbg_fem_t *f, int what)
{
	switch (what) {
	case NBG_FEM_ROW_PTR: return 4 * ((size_t)f->N + 1);
	case NBG_FEM_COL_IDX: return 4 * f->nnz;
	case NBG_FEM_K: return 8 * f->nnz;
	case NBG_FEM_F:
	case NBG_FEM_U: return 8 * (size_t)f->N;
	case NBG_FEM_STRAIN:
	case NBG_FEM_STRESS: return 8 * 3 * (size_t)n_gp(f) * f->m.N_elem;
	case NBG_FEM_MAIN_STRESS: return f->main_stress ? 16 * (size_t)n_gp(f) * f->m.N_elem : 0;
	case NBG_FEM_DAMAGE: return f->damage ? 8 * (size_t)n_gp(f) * f->m.N_elem : 0;
	case NBG_FEM_E: return 8 * (size_t)f->m.N_elem;
	case NBG_FEM_NOD: return 16 * (size_t)f->m.N_nod;
	case NBG_FEM_CONN: return 4 * (size_t)f->m.nen * f->m.N_elem;
	default: return 0;
	}
}

int nbg_fem_download(nbg_fem_t *f, int what, void *host)
{
	void *d = nbg_fem_device_ptr(f, what);
	if (!d)
		return NBG_ERR_ARG;
	int rc = nbg_d2h(host, d, nbg_fem_bytes(f, what), f->stream);
	return rc == NBG_OK ? nbg_stream_sync(f->stream) : rc;
}

int nbg_fem_upload(nbg_fem_t *f, int what, const void *host)
{
	void *d = nbg_fem_device_ptr(f, what);
	if (!d)
		return NBG_ERR_ARG;
	int rc = nbg_h2d(d, host, nbg_fem_bytes(f, what), f->stream);
	return rc == NBG_OK ? nbg_stream_sync(f->stream) : rc;
}

/* ------------------------------------------------------------------ SIMP */
static int solve_rhs(nbg_fem_t *f, const double *b, double *x, double tol, int method,
		     uint32_t *iters)
{
	int rc = nbg_fem_block_layout(f, NULL);
	if (rc != NBG_OK)
		return rc;
	const size_t need = method == NBG_METHOD_MIXED ? nbg_cg_mixed_layout_workspace_bytes(&f->bsr)
						      : nbg_cg_bsr_workspace_bytes(f->N);
	if ((rc = ensure_ws(f, need)) != NBG_OK)
		return rc;
	if (method == NBG_METHOD_MIXED) {
		nbg_mixed_result_t r;
		rc = nbg_cg_mixed(&f->bsr, b, x, 8 * f->N, tol, 0.1, NBG_CG_JACOBI | NBG_CG_RELATIVE,
				  &r, f->cg_ws, f->cg_ws_bytes, f->stream);
		*iters = r.niter;
	} else {
		nbg_cg_result_t r;
		rc = nbg_cg_bsr_f64(&f->bsr, b, x, 8 * f->N, tol, NBG_CG_JACOBI | NBG_CG_RELATIVE,
				    &r, f->cg_ws, f->cg_ws_bytes, f->stream);
		*iters = r.niter;
	}
	return rc;
}

int nbg_fem_simp(nbg_fem_t *f, const nbg_bcs_t *bcs, const double *rho, double nu,
		 double thickness, double penal, double E0, double Emin, int objective,
		 uint32_t dof, double tol, int method, double *dJ, nbg_simp_info_t *info)
{
	int rc = NBG_OK;
	const uint32_t Ne = f->m.N_elem, N = f->N;
	double *hu = malloc(8 * (size_t)N), *hF = malloc(8 * (size_t)N);
	memset(info, 0, sizeof(*info));
	if (!hu || !hF)
		TRY(NBG_ERR_NOMEM);
	if (objective == NBG_SIMP_DOF && dof >= N)
		TRY(NBG_ERR_ARG);
	/* device buffers kept across calls: an optimisation loop calls this
	 * once per design update */
	if (!f->simp_rho) {
		TRY(nbg_dev_alloc((void **)&f->simp_rho, 8 * (size_t)(Ne ? Ne : 1)));
		TRY(nbg_dev_alloc((void **)&f->simp_out, 8 * (size_t)(Ne ? Ne : 1)));
	}
	TRY(nbg_h2d(f->simp_rho, rho, 8 * (size_t)Ne, f->stream));
	TRY(nbg_simp_modulus_f64(Ne, f->simp_rho, penal, E0, Emin, f->E, f->stream));
	double g0[2] = {0.0, 0.0};
	TRY(nbg_fem_assemble_dev_damage(f, NULL, nu, thickness, 0.0, 0, g0, NULL, NULL));
	TRY(nbg_fem_apply_bcs(f, bcs, 1.0));
	TRY(zero_u(f));
	/* a solve that stops short of tol (status 1) still gives J and dJ */
	int short_of_tol = 0;
	{
		int st = solve_rhs(f, f->F, f->u, tol, method, &info->fwd_iters);
		if (st == NBG_NOT_CONVERGED)
			short_of_tol = 1;
		else
			TRY(st);
	}
	TRY(nbg_d2h(hu, f->u, 8 * (size_t)N, f->stream));
	TRY(nbg_d2h(hF, f->F, 8 * (size_t)N, f->stream));
	TRY(nbg_stream_sync(f->stream));
	const double *adj = f->u;
	if (objective == NBG_SIMP_COMPLIANCE) {
		double J = 0.0;
		for (uint32_t i = 0; i < N; i++)
			J += hF[i] * hu[i];
		info->J = J;
	} else {
		info->J = hu[dof];
		/* adjoint: K lambda = e_dof (K is symmetric after nbots' elimination) */
		memset(hF, 0, 8 * (size_t)N);
		hF[dof] = 1.0;
		memset(hu, 0, 8 * (size_t)N);
		if (!f->simp_e) {
			TRY(nbg_dev_alloc((void **)&f->simp_e, 8 * (size_t)N));
			TRY(nbg_dev_alloc((void **)&f->simp_lam, 8 * (size_t)N));
		}
		TRY(nbg_h2d(f->simp_e, hF, 8 * (size_t)N, f->stream));
		TRY(nbg_h2d(f->simp_lam, hu, 8 * (size_t)N, f->stream));
		int st = solve_rhs(f, f->simp_e, f->simp_lam, tol, method, &info->adj_iters);
		if (st == NBG_NOT_CONVERGED)
			short_of_tol = 1;
		else
			TRY(st);
		adj = f->simp_lam;
	}
	TRY(nbg_simp_sensitivity_f64(f->m.nen, Ne, f->nod, f->conn, nu, thickness, f->simp_rho,
				     penal, E0, Emin, adj, f->u, f->simp_out, f->stream));
	TRY(nbg_d2h(dJ, f->simp_out, 8 * (size_t)Ne, f->stream));
	TRY(nbg_stream_sync(f->stream));
	rc = short_of_tol ? NBG_NOT_CONVERGED : NBG_OK;
fail:
	info->status = rc;
	free(hu);
	free(hF);
	return rc;
}
