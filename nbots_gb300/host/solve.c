/*
 * Host-buffer solver context: a CSR system in host memory (the layout of
 * nb_sparse_create(graph, NULL, 2), sparse.c:20-60) is uploaded, converted
 * to the device block layout and solved by one of the CG kernels (nbots'
 * arithmetic on the CSR, nbots' iteration or the fast FP64 CG on the block
 * layout, mixed precision); x comes back to host memory.  The device buffers
 * are kept between calls, and so is the pattern when the caller says it has
 * not changed.  The drop-in nb_sparse_* entries keep one context per matrix.
 */
#include <stdlib.h>
#include <string.h>

#include "nbots_gb300.h"

struct nbg_solver {
	void *stream;
	int host_direct;  /* kernels write the caller's host memory directly */
	uint32_t N;
	uint64_t nnz;
	int have_pattern;
	int bsr_ok;
	/* device */
	uint32_t *rp, *ci, *slice_off, *bcol;
	double *val, *b, *x, *b64, *dinv64;
	float *b32, *dinv32;
	uint16_t *blo;
	uint8_t *bxt;
	void *ws;
	size_t ws_bytes;
	nbg_bsr_t bsr;
};

static void release(nbg_solver_t *s)
{
	void *p[] = {s->rp, s->ci, s->slice_off, s->bcol, s->val, s->b, s->x, s->b64,
		     s->dinv64, s->b32, s->dinv32, s->blo, s->bxt, s->ws};
	for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); i++)
		nbg_dev_free(p[i]);
	void *stream = s->stream;
	const int host_direct = s->host_direct;
	memset(s, 0, sizeof(*s));
	s->stream = stream;
	s->host_direct = host_direct;
}

int nbg_solver_create(nbg_solver_t **out, void *stream)
{
	*out = calloc(1, sizeof(nbg_solver_t));
	if (!*out)
		return NBG_ERR_NOMEM;
	(*out)->stream = stream;
	/* NBG_HOST_DIRECT=0 keeps the copy path (for A/B comparisons) */
	const char *e = getenv("NBG_HOST_DIRECT");
	(*out)->host_direct = (e && e[0] == '0') ? 0 : nbg_host_memory_access();
	return NBG_OK;
}

void nbg_solver_destroy(nbg_solver_t *s)
{
	if (!s)
		return;
	release(s);
	free(s);
}

#define TRY(x) do { int rc_ = (x); if (rc_ != NBG_OK) { rc = rc_; goto fail; } } while (0)

int nbg_solver_set_matrix(nbg_solver_t *s, uint32_t N, const uint32_t *row_ptr,
			  const uint32_t *col_idx, const double *val, unsigned flags)
{
	int rc = NBG_OK;
	const uint64_t nnz = row_ptr[N];
	const int same = (flags & NBG_PATTERN_SAME) && s->have_pattern && s->N == N &&
			 s->nnz == nnz;
	if (!same) {
		release(s);
		s->N = N;
		s->nnz = nnz;
		TRY(nbg_dev_alloc((void **)&s->rp, 4 * ((size_t)N + 1)));
		TRY(nbg_dev_alloc((void **)&s->ci, 4 * (nnz ? nnz : 1)));
		TRY(nbg_dev_alloc((void **)&s->val, 8 * (nnz ? nnz : 1)));
		TRY(nbg_dev_alloc((void **)&s->b, 8 * ((size_t)N ? N : 1)));
		TRY(nbg_dev_alloc((void **)&s->x, 8 * ((size_t)N ? N : 1)));
		TRY(nbg_h2d(s->rp, row_ptr, 4 * ((size_t)N + 1), s->stream));
		TRY(nbg_h2d(s->ci, col_idx, 4 * nnz, s->stream));
		uint32_t S = (N / 2 + 31) / 32;
		uint32_t *so = malloc(((size_t)S + 1) * sizeof(uint32_t));
		if (!so)
			TRY(NBG_ERR_NOMEM);
		s->bsr_ok = N > 0 && !(flags & NBG_CSR_ONLY) &&
			    nbg_bsr_plan(N, row_ptr, col_idx, so) == NBG_OK;
		if (s->bsr_ok) {
			const uint64_t ent = 32ull * so[S];
			int r2 = nbg_dev_alloc((void **)&s->slice_off, 4 * ((size_t)S + 1));
			if (r2 == NBG_OK)
				r2 = nbg_h2d(s->slice_off, so, 4 * ((size_t)S + 1), s->stream);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->bcol, 4 * ent);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->b64, 32 * ent);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->b32, 16 * ent);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->blo, 8 * ent);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->bxt, 4 * ent);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->dinv64, 8 * (size_t)N);
			if (r2 == NBG_OK) r2 = nbg_dev_alloc((void **)&s->dinv32, 4 * (size_t)N);
			if (r2 == NBG_OK) r2 = nbg_stream_sync(s->stream);
			free(so);
			so = NULL;
			TRY(r2);
			s->bsr.N = N;
			s->bsr.Nn = N / 2;
			s->bsr.n_slices = S;
			s->bsr.n_entries = ent;
			s->bsr.slice_off = s->slice_off;
			s->bsr.bcol = s->bcol;
			s->bsr.b64 = s->b64;
			s->bsr.b32 = s->b32;
			s->bsr.blo = s->blo;
			s->bsr.bxt = s->bxt;
			s->bsr.dinv64 = s->dinv64;
			s->bsr.dinv32 = s->dinv32;
		}
		free(so);
		s->have_pattern = 1;
	}
	if (!val)  /* values to come from the device side (nbg_solver_device_csr) */
		return nbg_stream_sync(s->stream);
	TRY(nbg_h2d(s->val, val, 8 * nnz, s->stream));
	if (s->bsr_ok)
		TRY(nbg_bsr_fill(&s->bsr, s->rp, s->ci, s->val, s->stream));
	return NBG_OK;
fail:
	release(s);
	return rc;
}

int nbg_solver_solve(nbg_solver_t *s, const double *b, double *x, uint32_t max_iter,
		     double tol, unsigned flags, int method, nbg_solve_info_t *info)
{
	int rc = NBG_OK;
	memset(info, 0, sizeof(*info));
	if (!s->have_pattern)
		return NBG_ERR_ARG;
	/* nbots' iteration runs on the block layout when the pattern has one,
	 * else on the CSR with nbots' own arithmetic */
	if (method == NBG_METHOD_NBOTS_FAST && !s->bsr_ok)
		method = NBG_METHOD_NBOTS;
	if (method != NBG_METHOD_NBOTS && !s->bsr_ok)
		return NBG_ERR_PATTERN;
	size_t need = method == NBG_METHOD_NBOTS ? nbg_cg_workspace_bytes(s->N)
		    : method == NBG_METHOD_MIXED ? nbg_cg_mixed_layout_workspace_bytes(&s->bsr)
		    : nbg_cg_bsr_workspace_bytes(s->N);
	if (s->ws_bytes < need) {
		nbg_dev_free(s->ws);
		s->ws = NULL;
		s->ws_bytes = 0;
		TRY(nbg_dev_alloc(&s->ws, need));
		s->ws_bytes = need;
	}
	TRY(nbg_h2d(s->b, b, 8 * (size_t)s->N, s->stream));
	TRY(nbg_h2d(s->x, x, 8 * (size_t)s->N, s->stream));
	if (method == NBG_METHOD_MIXED) {
		nbg_mixed_result_t r;
		rc = nbg_cg_mixed(&s->bsr, s->b, s->x, max_iter, tol, 0.1, flags, &r, s->ws,
				  s->ws_bytes, s->stream);
		info->niter = r.niter;
		info->n_updates = r.n_updates;
		info->status = r.status;
		info->relres = r.relres;
		info->tol_reached = r.relres * r.bnorm;
	} else {
		nbg_cg_result_t r;
		if (method == NBG_METHOD_NBOTS)
			rc = nbg_cg_f64(s->N, s->rp, s->ci, s->val, s->b, s->x, max_iter, tol, flags,
					&r, s->ws, s->ws_bytes, s->stream);
		else
			rc = nbg_cg_bsr_f64(&s->bsr, s->b, s->x, max_iter, tol,
					    method == NBG_METHOD_NBOTS_FAST ? flags | NBG_CG_NBOTS_STOP
									   : flags,
					    &r, s->ws, s->ws_bytes, s->stream);
		info->niter = r.niter;
		info->status = r.status;
		info->tol_reached = r.tol_reached;
		info->relres = r.bnorm > 0 ? r.tol_reached / r.bnorm : r.tol_reached;
	}
	if (rc < 0)
		return rc;
	int r2 = nbg_d2h(x, s->x, 8 * (size_t)s->N, s->stream);
	if (r2 == NBG_OK)
		r2 = nbg_stream_sync(s->stream);
	return r2 != NBG_OK ? r2 : rc;
fail:
	return rc;
}

int nbg_solver_multiply(nbg_solver_t *s, const double *in, double *out)
{
	if (!s->have_pattern)
		return NBG_ERR_ARG;
	if (s->N == 0)
		return NBG_OK;
	/* where the GPU reaches the caller's memory coherently (Grace and
	 * NVLink-C2C), the kernel writes the product there itself, overlapping
	 * the transfer with the FP64-bound SpMV (1M dof: 0.18 against 0.22 ms
	 * with a copy back; reading x there too was slower, 0.27 ms, so x is
	 * copied in) */
	const int direct = s->host_direct;
	int rc = nbg_h2d(s->x, in, 8 * (size_t)s->N, s->stream);
	if (rc == NBG_OK)
		rc = nbg_spmv_csr_f64(s->N, s->rp, s->ci, s->val, s->x, direct ? out : s->b,
				      s->stream);
	if (rc == NBG_OK && !direct)
		rc = nbg_d2h(out, s->b, 8 * (size_t)s->N, s->stream);
	if (rc == NBG_OK)
		rc = nbg_stream_sync(s->stream);
	return rc;
}

int nbg_solver_device_csr(nbg_solver_t *s, const uint32_t **row_ptr, const uint32_t **col_idx,
			  double **val)
{
	if (!s->have_pattern)
		return NBG_ERR_ARG;
	if (row_ptr)
		*row_ptr = s->rp;
	if (col_idx)
		*col_idx = s->ci;
	if (val)
		*val = s->val;
	return NBG_OK;
}

int nbg_solver_values_changed(nbg_solver_t *s)
{
	if (!s->have_pattern)
		return NBG_ERR_ARG;
	return s->bsr_ok ? nbg_bsr_fill(&s->bsr, s->rp, s->ci, s->val, s->stream) : NBG_OK;
}

size_t nbg_solver_device_bytes(const nbg_solver_t *s)
{
	if (!s->have_pattern)
		return s->ws_bytes;
	size_t b = 4 * ((size_t)s->N + 1) + 12 * (size_t)s->nnz + 16 * (size_t)s->N + s->ws_bytes;
	if (s->bsr_ok)
		b += 4 * ((size_t)s->bsr.n_slices + 1) + 60 * (size_t)s->bsr.n_entries +
		     12 * (size_t)s->N;
	return b;
}

int nbg_solver_block_layout(nbg_solver_t *s, nbg_bsr_t *out)
{
	if (!s->have_pattern)
		return NBG_ERR_ARG;
	if (!s->bsr_ok)
		return NBG_ERR_PATTERN;
	if (out)
		*out = s->bsr;
	return NBG_OK;
}
