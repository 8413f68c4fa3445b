/* Batched FEM solves: independent problems (meshes of uneven size, each
 * with its own boundary conditions, densities and loads) merged into one
 * block-diagonal system and solved side by side by the batched
 * mixed-precision CG (nbg_mixed_batch_*), followed by the SIMP compliance
 * sensitivities, as one CUDA graph per launch.  No counterpart in nbots.
 *
 * Merged numbering: instance k's nodes start at node_off[k], a multiple of
 * 32 (one slice of the block layout), its elements at elem_off[k], its
 * input vertices and segments after those of instance k-1.  The nodes that
 * pad an instance up to the next multiple of 32 belong to no element, so
 * their rows hold only their zero diagonal block; a Dirichlet condition
 * pushed after all the instances' own atoms turns each into an identity
 * row with zero load.  Because assembly gathers each row in ascending
 * element order and every instance's elements keep their order, and because
 * the boundary conditions of different instances touch disjoint rows and
 * columns, each instance's K and F are bit-identical to the ones the
 * single-system path builds for it. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fem_internal.h"

struct nbg_batch {
	uint32_t n;
	uint32_t *node_off, *elem_off, *slice_ptr;
	nbg_mesh_t m;
	double *nod;
	uint32_t *conn, *edg;
	nbg_bcs_t bcs;
	uint32_t *vtx, *sgm_ptr, *sgm_nodes;
	nbg_bc_t *bc;
	double *nv;
	nbg_fem_t *f;
	nbg_mixed_batch_t *mb;
	double *d_rho, *d_dJ;
	double nu, thickness, penal, E0, Emin;
	int assembled;
	void *stream;
};

#define TRY(x) do { int rc_ = (x); if (rc_ != NBG_OK) { rc = rc_; goto fail; } } while (0)

void nbg_batch_destroy(nbg_batch_t *b)
{
	if (!b)
		return;
	nbg_mixed_batch_destroy(b->mb);
	nbg_fem_destroy(b->f);
	nbg_dev_free(b->d_rho);
	nbg_dev_free(b->d_dJ);
	free(b->node_off);
	free(b->elem_off);
	free(b->slice_ptr);
	free(b->nod);
	free(b->conn);
	free(b->edg);
	free(b->vtx);
	free(b->sgm_ptr);
	free(b->sgm_nodes);
	free(b->bc);
	free(b->nv);
	free(b);
}

int nbg_batch_create(nbg_batch_t **out, uint32_t n, const nbg_mesh_t *meshes,
		     const nbg_bcs_t *bcs, void *stream)
{
	int rc = NBG_OK;
	if (!out)
		return NBG_ERR_ARG;
	*out = NULL;
	if (n == 0 || !meshes || !bcs)
		return NBG_ERR_ARG;
	const uint32_t nen = meshes[0].nen;
	if (nen != 3 && nen != 4)
		return NBG_ERR_ARG;
	nbg_batch_t *b = calloc(1, sizeof(*b));
	if (!b)
		return NBG_ERR_NOMEM;
	b->n = n;
	b->stream = stream;
	b->node_off = calloc((size_t)n + 1, sizeof(uint32_t));
	b->elem_off = calloc((size_t)n + 1, sizeof(uint32_t));
	b->slice_ptr = calloc((size_t)n + 1, sizeof(uint32_t));
	if (!b->node_off || !b->elem_off || !b->slice_ptr)
		TRY(NBG_ERR_NOMEM);

	/* sizes of the merged arrays */
	uint64_t Nn = 0, Ne = 0, Ned = 0, Nv = 0, Ns = 0, Nsn = 0, Nbc = 0, Nnv = 0, Npad = 0;
	for (uint32_t k = 0; k < n; k++) {
		const nbg_mesh_t *m = &meshes[k];
		const nbg_bcs_t *c = &bcs[k];
		if (m->nen != nen || m->N_nod == 0 || !m->nod || (m->N_elem && !m->conn) ||
		    (m->N_edg && !m->edg))
			TRY(NBG_ERR_ARG);
		uint32_t nv = 0;
		for (uint32_t a = 0; a < c->N_bc; a++) {
			const nbg_bc_t *t = &c->bc[a];
			if (t->where == 0 && t->id + 1 > nv)
				nv = t->id + 1;
			if (t->where == 1 && t->id >= c->N_sgm)
				TRY(NBG_ERR_ARG);
			Nnv += 2 * (uint64_t)t->n_nv;
		}
		if (nv && !c->vtx)
			TRY(NBG_ERR_ARG);
		const uint64_t padded = ((uint64_t)m->N_nod + 31) / 32 * 32;
		b->node_off[k] = (uint32_t)Nn;
		b->elem_off[k] = (uint32_t)Ne;
		b->slice_ptr[k] = (uint32_t)(Nn / 32);
		Npad += padded - m->N_nod;
		Nn += padded;
		Ne += m->N_elem;
		Ned += m->N_edg;
		Nv += nv;
		Ns += c->N_sgm;
		Nsn += c->N_sgm ? c->sgm_ptr[c->N_sgm] : 0;
		Nbc += c->N_bc;
		if (2 * Nn > UINT32_MAX || Ne * nen > UINT32_MAX)
			TRY(NBG_ERR_ARG);
	}
	b->node_off[n] = (uint32_t)Nn;
	b->elem_off[n] = (uint32_t)Ne;
	b->slice_ptr[n] = (uint32_t)(Nn / 32);

	b->nod = calloc(2 * Nn, sizeof(double));
	b->conn = malloc((Ne * nen + 1) * sizeof(uint32_t));
	b->edg = malloc((2 * Ned + 1) * sizeof(uint32_t));
	b->vtx = malloc((Nv + Npad + 1) * sizeof(uint32_t));
	b->sgm_ptr = malloc((Ns + 1) * sizeof(uint32_t));
	b->sgm_nodes = malloc((Nsn + 1) * sizeof(uint32_t));
	b->bc = calloc(Nbc + Npad + 1, sizeof(nbg_bc_t));
	b->nv = malloc((Nnv + 1) * sizeof(double));
	if (!b->nod || !b->conn || !b->edg || !b->vtx || !b->sgm_ptr || !b->sgm_nodes || !b->bc ||
	    !b->nv)
		TRY(NBG_ERR_NOMEM);

	uint64_t ie = 0, ied = 0, iv = 0, is = 0, isn = 0, ib = 0, inv = 0;
	b->sgm_ptr[0] = 0;
	for (uint32_t k = 0; k < n; k++) {
		const nbg_mesh_t *m = &meshes[k];
		const nbg_bcs_t *c = &bcs[k];
		const uint32_t no = b->node_off[k];
		memcpy(b->nod + 2 * (uint64_t)no, m->nod, 16 * (size_t)m->N_nod);
		for (uint64_t t = 0; t < (uint64_t)m->N_elem * nen; t++) {
			if (m->conn[t] >= m->N_nod)
				TRY(NBG_ERR_ARG);
			b->conn[ie++] = m->conn[t] + no;
		}
		for (uint64_t t = 0; t < 2 * (uint64_t)m->N_edg; t++) {
			if (m->edg[t] >= m->N_nod)
				TRY(NBG_ERR_ARG);
			b->edg[ied++] = m->edg[t] + no;
		}
		const uint32_t v0 = (uint32_t)iv, s0 = (uint32_t)is;
		uint32_t nv = 0;
		for (uint32_t a = 0; a < c->N_bc; a++)
			if (c->bc[a].where == 0 && c->bc[a].id + 1 > nv)
				nv = c->bc[a].id + 1;
		for (uint32_t t = 0; t < nv; t++) {
			if (c->vtx[t] >= m->N_nod)
				TRY(NBG_ERR_ARG);
			b->vtx[iv++] = c->vtx[t] + no;
		}
		for (uint32_t t = 0; t < c->N_sgm; t++) {
			for (uint32_t q = c->sgm_ptr[t]; q < c->sgm_ptr[t + 1]; q++) {
				if (c->sgm_nodes[q] >= m->N_nod)
					TRY(NBG_ERR_ARG);
				b->sgm_nodes[isn++] = c->sgm_nodes[q] + no;
			}
			b->sgm_ptr[++is] = (uint32_t)isn;
		}
		for (uint32_t a = 0; a < c->N_bc; a++) {
			nbg_bc_t t = c->bc[a];
			t.id += t.where == 0 ? v0 : s0;
			if (t.n_nv) {
				memcpy(b->nv + inv, t.node_vals, 16 * (size_t)t.n_nv);
				t.node_vals = b->nv + inv;
				inv += 2 * (uint64_t)t.n_nv;
			}
			b->bc[ib++] = t;
		}
	}
	/* padding nodes: identity rows with zero load */
	for (uint32_t k = 0; k < n; k++)
		for (uint32_t i = b->node_off[k] + meshes[k].N_nod; i < b->node_off[k + 1]; i++) {
			nbg_bc_t *t = &b->bc[ib++];
			t->kind = 0;
			t->where = 0;
			t->id = (uint32_t)iv;
			t->mask[0] = t->mask[1] = 1;
			b->vtx[iv++] = i;
		}
	b->m.nen = nen;
	b->m.N_nod = (uint32_t)Nn;
	b->m.N_elem = (uint32_t)Ne;
	b->m.N_edg = (uint32_t)Ned;
	b->m.nod = b->nod;
	b->m.conn = b->conn;
	b->m.edg = b->edg;
	b->bcs.vtx = b->vtx;
	b->bcs.N_sgm = (uint32_t)is;
	b->bcs.sgm_ptr = b->sgm_ptr;
	b->bcs.sgm_nodes = b->sgm_nodes;
	b->bcs.N_bc = (uint32_t)ib;
	b->bcs.bc = b->bc;
	TRY(nbg_fem_create(&b->f, &b->m, stream));
	/* each instance owns a contiguous range of slices: mesh order */
	TRY(nbg_fem_set_block_order(b->f, NBG_ORDER_MESH, 0));
	TRY(nbg_dev_alloc((void **)&b->d_rho, 8 * (Ne ? Ne : 1)));
	TRY(nbg_dev_alloc((void **)&b->d_dJ, 8 * (Ne ? Ne : 1)));
	*out = b;
	return NBG_OK;
fail:
	nbg_batch_destroy(b);
	return rc;
}

uint32_t nbg_batch_size(const nbg_batch_t *b) { return b ? b->n : 0; }

int nbg_batch_offsets(const nbg_batch_t *b, uint32_t *node_off, uint32_t *elem_off)
{
	if (!b)
		return NBG_ERR_ARG;
	if (node_off)
		memcpy(node_off, b->node_off, 4 * ((size_t)b->n + 1));
	if (elem_off)
		memcpy(elem_off, b->elem_off, 4 * ((size_t)b->n + 1));
	return NBG_OK;
}

nbg_fem_t *nbg_batch_fem(nbg_batch_t *b) { return b ? b->f : NULL; }

nbg_mixed_batch_t *nbg_batch_solver(nbg_batch_t *b) { return b ? b->mb : NULL; }

int nbg_batch_assemble_simp(nbg_batch_t *b, const double *rho, double nu, double thickness,
			    double penal, double E0, double Emin)
{
	int rc = NBG_OK;
	if (!b || !rho)
		return NBG_ERR_ARG;
	const uint32_t Ne = b->m.N_elem;
	/* the moduli on the device, as nbg_fem_simp computes them */
	TRY(nbg_h2d(b->d_rho, rho, 8 * (size_t)Ne, b->stream));
	TRY(nbg_simp_modulus_f64(Ne, b->d_rho, penal, E0, Emin,
				 nbg_fem_device_ptr(b->f, NBG_FEM_E), b->stream));
	const double g0[2] = {0.0, 0.0};
	rc = nbg_fem_assemble_dev_damage(b->f, NULL, nu, thickness, 0.0, 0, g0, NULL, NULL);
	if (rc != NBG_OK)
		goto fail;
	TRY(nbg_fem_apply_bcs(b->f, &b->bcs, 1.0));
	TRY(nbg_fem_block_layout(b->f, NULL));
	TRY(nbg_stream_sync(b->stream));
	b->nu = nu;
	b->thickness = thickness;
	b->penal = penal;
	b->E0 = E0;
	b->Emin = Emin;
	b->assembled = 1;
	if (b->mb)
		TRY(nbg_mixed_batch_set_sensitivity(b->mb, b->m.nen, Ne,
						     nbg_fem_device_ptr(b->f, NBG_FEM_NOD),
						     nbg_fem_device_ptr(b->f, NBG_FEM_CONN), nu,
						     thickness, b->d_rho, penal, E0, Emin, b->d_dJ));
fail:
	return rc;
}

int nbg_batch_setup(nbg_batch_t *b, uint32_t max_iter, double tol, double delta,
		    unsigned flags)
{
	int rc = NBG_OK;
	if (!b || !b->assembled)
		return NBG_ERR_ARG;
	nbg_bsr_t A;
	TRY(nbg_fem_block_layout(b->f, &A));
	nbg_mixed_batch_destroy(b->mb);
	b->mb = NULL;
	TRY(nbg_mixed_batch_create(&b->mb, &A, nbg_fem_device_ptr(b->f, NBG_FEM_F),
				   nbg_fem_device_ptr(b->f, NBG_FEM_U), b->n, b->slice_ptr,
				   max_iter, tol, delta, flags, b->stream));
	TRY(nbg_mixed_batch_set_sensitivity(b->mb, b->m.nen, b->m.N_elem,
					     nbg_fem_device_ptr(b->f, NBG_FEM_NOD),
					     nbg_fem_device_ptr(b->f, NBG_FEM_CONN), b->nu,
					     b->thickness, b->d_rho, b->penal, b->E0, b->Emin,
					     b->d_dJ));
	return NBG_OK;
fail:
	return rc;
}

int nbg_batch_launch(nbg_batch_t *b)
{
	return b && b->mb ? nbg_mixed_batch_launch(b->mb) : NBG_ERR_ARG;
}

int nbg_batch_results(nbg_batch_t *b, nbg_mixed_result_t *res, double *J)
{
	return b && b->mb ? nbg_mixed_batch_results(b->mb, res, J) : NBG_ERR_ARG;
}

int nbg_batch_sensitivities(nbg_batch_t *b, double *dJ)
{
	int rc = NBG_OK;
	if (!b || !dJ)
		return NBG_ERR_ARG;
	TRY(nbg_d2h(dJ, b->d_dJ, 8 * (size_t)b->m.N_elem, b->stream));
	TRY(nbg_stream_sync(b->stream));
fail:
	return rc;
}
