/*
 * Host loop of nbots' quasi-static damage solve
 * (pde_bot/finite_element/solid_mechanics/static_damage2D.c:239-470, the
 * conjugate-gradient branch) on the device FEM system.  Every array stays on
 * the device; per iteration the host reads back one residual norm and the
 * solver's status, and writes nbots' log lines.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fem_internal.h"

#define TRY(x) do { int rc_ = (x); if (rc_ != NBG_OK) { rc = rc_; goto fail; } } while (0)

/* Gauss-Seidel gives up after this long (it has no other bound than
 * 60 N sweeps). */
#define GS_TIME_LIMIT_S 600.0

int nbg_host_lower_levels(uint32_t N, const uint32_t *rp, const uint32_t *ci, uint32_t *lev_ptr,
			  uint32_t *lev_rows, uint32_t *n_levels)
{
	uint32_t *lev = malloc(sizeof(uint32_t) * (N ? N : 1));
	if (!lev)
		return NBG_ERR_NOMEM;
	uint32_t nl = 0;
	for (uint32_t i = 0; i < N; i++) {
		uint32_t L = 0;
		for (uint32_t q = rp[i]; q < rp[i + 1] && ci[q] < i; q++)
			if (lev[ci[q]] + 1 > L)
				L = lev[ci[q]] + 1;
		lev[i] = L;
		if (L + 1 > nl)
			nl = L + 1;
	}
	memset(lev_ptr, 0, sizeof(uint32_t) * ((size_t)N + 1));
	for (uint32_t i = 0; i < N; i++)
		lev_ptr[lev[i] + 1]++;
	for (uint32_t L = 0; L < nl; L++)
		lev_ptr[L + 1] += lev_ptr[L];
	for (uint32_t L = nl + 1; L <= N; L++)
		lev_ptr[L] = lev_ptr[nl];
	/* counting sort keeps ascending row order within a level */
	uint32_t *fill = malloc(sizeof(uint32_t) * ((size_t)nl + 1));
	if (!fill) {
		free(lev);
		return NBG_ERR_NOMEM;
	}
	memcpy(fill, lev_ptr, sizeof(uint32_t) * ((size_t)nl + 1));
	for (uint32_t i = 0; i < N; i++)
		lev_rows[fill[lev[i]]++] = i;
	free(fill);
	free(lev);
	*n_levels = nl;
	return NBG_OK;
}

static void logf_append(FILE *lf, const char *fmt, ...)
{
	if (!lf)
		return;
	va_list ap;
	va_start(ap, fmt);
	vfprintf(lf, fmt, ap);
	va_end(ap);
	fflush(lf);
}

typedef struct {
	double *du, *res, *r, *r_prev, *norm2, *rws, *gws, *bws;
	uint32_t *lev_ptr, *lev_rows, n_levels;
	int have_levels;
} dmg_ws_t;

static void free_ws(dmg_ws_t *w)
{
	void *p[] = {w->du, w->res, w->r, w->r_prev, w->rws, w->gws, w->bws, w->lev_ptr,
		     w->lev_rows};
	for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); i++)
		nbg_dev_free(p[i]);
}

/* Rows' lower-part levels, from the pattern on the device (once). */
static int build_levels(nbg_fem_t *f, dmg_ws_t *w)
{
	int rc = NBG_OK;
	const uint32_t N = f->N;
	uint32_t *rp = malloc(4 * ((size_t)N + 1)), *ci = malloc(4 * (f->nnz ? f->nnz : 1));
	uint32_t *lp = malloc(4 * ((size_t)N + 1)), *lr = malloc(4 * (size_t)(N ? N : 1));
	if (!rp || !ci || !lp || !lr)
		TRY(NBG_ERR_NOMEM);
	TRY(nbg_d2h(rp, f->row_ptr, 4 * ((size_t)N + 1), f->stream));
	TRY(nbg_d2h(ci, f->col_idx, 4 * f->nnz, f->stream));
	TRY(nbg_stream_sync(f->stream));
	TRY(nbg_host_lower_levels(N, rp, ci, lp, lr, &w->n_levels));
	TRY(nbg_dev_alloc((void **)&w->lev_ptr, 4 * ((size_t)N + 1)));
	TRY(nbg_dev_alloc((void **)&w->lev_rows, 4 * (size_t)(N ? N : 1)));
	TRY(nbg_dev_alloc((void **)&w->gws, nbg_gauss_seidel_workspace_bytes(N)));
	TRY(nbg_h2d(w->lev_ptr, lp, 4 * ((size_t)w->n_levels + 1), f->stream));
	TRY(nbg_h2d(w->lev_rows, lr, 4 * (size_t)N, f->stream));
	TRY(nbg_stream_sync(f->stream));
	w->have_levels = 1;
fail:
	free(rp);
	free(ci);
	free(lp);
	free(lr);
	return rc;
}

int nbg_fem_damage(nbg_fem_t *f, const nbg_bcs_t *bcs, double E, double nu, double thickness,
		   double density, int self_weight, const double gravity[2], double ft,
		   double gf, uint32_t n_steps, uint32_t max_iter, uint32_t max_iter_noenh,
		   double rtol, int method, const char *logfile, nbg_damage_info_t *info)
{
	int rc = NBG_OK;
	if (!f || !bcs || (method != NBG_METHOD_NBOTS && method != NBG_METHOD_FP64 &&
			   method != NBG_METHOD_NBOTS_FAST))
		return NBG_ERR_ARG;
	const int blocked = method != NBG_METHOD_NBOTS;
	nbg_damage_info_t inf;
	memset(&inf, 0, sizeof(inf));
	dmg_ws_t w;
	memset(&w, 0, sizeof(w));
	FILE *lf = NULL;
	double *Eh = NULL, *rh = NULL;
	const uint32_t N = f->N, ne = f->m.N_elem;
	const size_t npt = (size_t)(f->m.nen == 4 ? 4 : 1) * ne;
	if (logfile) {
		lf = fopen(logfile, "a");
		if (!lf)
			return NBG_ERR_ARG;
	}
	/* state: displacement in f->u, damage in f->damage, strain in f->strain */
	if (!f->damage)
		TRY(nbg_dev_alloc((void **)&f->damage, 8 * (npt ? npt : 1)));
	TRY(nbg_dev_alloc((void **)&w.du, 8 * (size_t)(N ? N : 1)));
	TRY(nbg_dev_alloc((void **)&w.res, 8 * (size_t)(N ? N : 1)));
	TRY(nbg_dev_alloc((void **)&w.r, 8 * (npt ? npt : 1)));
	TRY(nbg_dev_alloc((void **)&w.r_prev, 8 * (npt ? npt : 1)));
	TRY(nbg_dev_alloc((void **)&w.rws, nbg_residual_workspace_bytes(N) + 8));
	w.norm2 = w.rws + nbg_residual_workspace_bytes(N) / 8;
	TRY(nbg_fem_cg_workspace(f));
	const size_t bws_bytes = nbg_cg_bsr_workspace_bytes(N);
	if (blocked)
		TRY(nbg_dev_alloc((void **)&w.bws, bws_bytes));
	Eh = malloc(8 * (size_t)(ne ? ne : 1));
	rh = malloc(8 * (npt ? npt : 1));
	if (!Eh || !rh)
		TRY(NBG_ERR_NOMEM);
	for (uint32_t e = 0; e < ne; e++)
		Eh[e] = E;
	/* r starts at r0 = ft / sqrt(E) (tension_damage_r0, static_damage2D.c:128-132) */
	const double r0 = ft / sqrt(E);
	for (size_t i = 0; i < npt; i++)
		rh[i] = r0;
	TRY(nbg_h2d(w.r, rh, 8 * npt, f->stream));
	TRY(nbg_memset(f->u, 0, 8 * (size_t)N, f->stream));
	TRY(nbg_memset(f->damage, 0, 8 * npt, f->stream));
	TRY(nbg_memset(f->strain, 0, 24 * npt, f->stream));

	logf_append(lf, "FEM: Damage Model\n");
	for (uint32_t n = 0; n < n_steps; n++) {
		logf_append(lf, "  [ Load step %i]\n", (int)(n + 1));
		TRY(nbg_d2d(w.r_prev, w.r, 8 * npt, f->stream));
		TRY(nbg_memset(w.du, 0, 8 * (size_t)N, f->stream));
		double residual_norm = 1, residual_best = 0;
		uint32_t iter = 0, noenh = 0;
		for (;;) {
			TRY(nbg_fem_assemble_dev_damage(f, Eh, nu, thickness, density, self_weight,
							gravity, NULL, f->damage));
			const double factor = (n + 1.0) / (double)n_steps;
			TRY(nbg_fem_apply_bcs(f, bcs, factor));
			TRY(nbg_residual_f64(N, f->row_ptr, f->col_idx, f->K, f->F, f->u, w.res,
					     w.norm2, w.rws, f->stream));
			double norm2 = 0.0;
			TRY(nbg_d2h(&norm2, w.norm2, 8, f->stream));
			TRY(nbg_stream_sync(f->stream));
			residual_norm = sqrt(norm2);
			inf.iterations++;
			if (iter == 0) {
				residual_best = residual_norm;
			} else if (residual_norm < residual_best) {
				residual_best = residual_norm;
				noenh = 0;
			} else {
				noenh += 1;
			}
			if ((residual_norm < rtol && iter > 0) || iter >= max_iter ||
			    noenh >= max_iter_noenh) {
				logf_append(lf, "    [%i: Residual: %e ]\n", (int)iter, residual_norm);
				break;
			}
			/* returns 1 (and cg.status 1) when the tolerance is not reached */
			nbg_cg_result_t cg;
			int st;
			if (blocked) {
				TRY(nbg_fem_block_layout(f, NULL));  /* from this K */
				st = nbg_cg_bsr_f64(&f->bsr, w.res, w.du, N, 1e-8,
						    method == NBG_METHOD_NBOTS_FAST
							    ? NBG_CG_JACOBI | NBG_CG_NBOTS_STOP
							    : NBG_CG_JACOBI,
						    &cg, w.bws, bws_bytes, f->stream);
			} else {
				st = nbg_cg_f64(N, f->row_ptr, f->col_idx, f->K, w.res, w.du, N, 1e-8,
						NBG_CG_JACOBI, &cg, f->cg_ws, f->cg_ws_bytes, f->stream);
			}
			if (st < 0)
				TRY(st);
			if (cg.status < 0)
				TRY(cg.status);
			inf.cg_solves++;
			inf.cg_iterations += cg.niter;
			if (cg.status != 0) {
				inf.gs_fallbacks++;
				if (!w.have_levels)
					TRY(build_levels(f, &w));
				nbg_gs_result_t gs;
				TRY(nbg_gauss_seidel_f64(N, f->row_ptr, f->col_idx, f->K, w.res, w.du,
							 w.lev_ptr, w.lev_rows, w.n_levels, 60 * N,
							 1e-8, GS_TIME_LIMIT_S, &gs, w.gws,
							 f->stream));
				if (gs.status < 0)
					TRY(gs.status);
				if (gs.status != 0) {
					inf.gs_failures++;
					logf_append(lf, "    [Conjugate Gradient (p. Jacobi) and "
						    "Gauss-Seidel fails.]\n");
					logf_append(lf, "      [Gauss-Seidel iterations: %u]\n",
						    gs.niter);
					logf_append(lf, "      [Gauss-Seidel error: %e ]\n", gs.error);
				}
			}
			logf_append(lf, "    [%i: Residual: %e]\n", (int)iter, residual_norm);
			TRY(nbg_add_to_f64(N, f->u, w.du, f->stream));
			TRY(nbg_strain_damage_f64(f->m.nen, ne, f->nod, f->conn, f->u, E, nu, ft, gf,
						  w.r_prev, w.r, f->damage, f->strain, f->distorted,
						  f->stream));
			iter++;
		}
		inf.residual = residual_norm;
	}
	TRY(nbg_stream_sync(f->stream));
fail:
	if (lf)
		fclose(lf);
	free(Eh);
	free(rh);
	free_ws(&w);
	if (info)
		*info = inf;
	return rc;
}
