/*
 * Drop-in nb_sparse_* and CG entry points (declared in nbots_dropin.h).
 *
 * Matrices made here back all their rows with two slabs (values, column
 * indices) in row order, so the GPU path uploads them without copying row by
 * row; the row-of-pointers struct stays nbots' own (sparse_struct.h:6-11),
 * so code that reads or replaces rows directly keeps working.  A registry
 * remembers which matrices own slabs; destroy frees any row that no longer
 * points into its slab one by one, and matrices nbots allocated row by row
 * entirely that way (nb_free_mem is free(), memory_bot/allocate_mem.c).
 */
#define _POSIX_C_SOURCE 200809L
#define _GNU_SOURCE
#include <dlfcn.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nbots_dropin.h"
#include "nbots_gb300.h"

/* ------------------------------------------------------------ registry */
typedef struct {
	const nb_sparse_t *A;
	double *vals;
	uint32_t *idx;
	uint64_t nnz;
} slab_t;

static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;
static slab_t *g_slabs;
static size_t g_n, g_cap;
static __thread int g_err;

int nbg_dropin_error(void)
{
	int e = g_err;
	g_err = 0;
	return e;
}

/* Records the status of a drop-in entry that returns void in nbots. */
void nbg_dropin_record_error(int e)
{
	if (e)
		g_err = e;
}

/* A/B switch: with NBG_DROPIN_CPU=1 in the environment, the replaced
 * compute entry points call the next definition of the same symbol in link
 * order -- nbots' own CPU code when libnbots.so follows this library -- so
 * both paths run on the same objects.  Off unless set; with it set and no
 * such definition loaded, the call fails with NBG_ERR_ARG instead of running
 * anything. */
int nbg_dropin_cpu(void)
{
	const char *v = getenv("NBG_DROPIN_CPU");
	return v && v[0] == '1' && v[1] == 0;
}

void *nbg_dropin_next(const char *name)
{
	return dlsym(RTLD_NEXT, name);
}

typedef int (*cg_fn)(const nb_sparse_t *, const double *, double *, uint32_t, double,
		     uint32_t *, double *, uint32_t);
typedef void (*spmv_fn)(const nb_sparse_t *, const double *, double *, uint32_t);

static void reg_add(const nb_sparse_t *A, double *v, uint32_t *ix, uint64_t nnz)
{
	pthread_mutex_lock(&g_lock);
	if (g_n == g_cap) {
		size_t c = g_cap ? 2 * g_cap : 64;
		slab_t *s = realloc(g_slabs, c * sizeof(slab_t));
		if (s) {
			g_slabs = s;
			g_cap = c;
		}
	}
	if (g_n < g_cap)
		g_slabs[g_n++] = (slab_t){A, v, ix, nnz};
	pthread_mutex_unlock(&g_lock);
}

static int reg_take(const nb_sparse_t *A, slab_t *out)
{
	int found = 0;
	pthread_mutex_lock(&g_lock);
	for (size_t i = 0; i < g_n; i++)
		if (g_slabs[i].A == A) {
			*out = g_slabs[i];
			g_slabs[i] = g_slabs[--g_n];
			found = 1;
			break;
		}
	pthread_mutex_unlock(&g_lock);
	return found;
}

static int reg_find(const nb_sparse_t *A, slab_t *out)
{
	int found = 0;
	pthread_mutex_lock(&g_lock);
	for (size_t i = 0; i < g_n; i++)
		if (g_slabs[i].A == A) {
			*out = g_slabs[i];
			found = 1;
			break;
		}
	pthread_mutex_unlock(&g_lock);
	return found;
}

static nb_sparse_t *alloc_slab(uint32_t N, const uint32_t *sizes)
{
	nb_sparse_t *A = malloc(sizeof(*A));
	if (!A)
		return NULL;
	A->N = N;
	A->rows_values = malloc((N ? N : 1) * sizeof(double *));
	A->rows_index = malloc((N ? N : 1) * sizeof(uint32_t *));
	A->rows_size = malloc((N ? N : 1) * sizeof(uint32_t));
	uint64_t nnz = 0;
	for (uint32_t i = 0; i < N; i++)
		nnz += sizes[i];
	double *v = calloc(nnz ? nnz : 1, sizeof(double));
	uint32_t *ix = malloc((nnz ? nnz : 1) * sizeof(uint32_t));
	if (!A->rows_values || !A->rows_index || !A->rows_size || !v || !ix) {
		free(A->rows_values); free(A->rows_index); free(A->rows_size);
		free(v); free(ix); free(A);
		return NULL;
	}
	uint64_t o = 0;
	for (uint32_t i = 0; i < N; i++) {
		A->rows_size[i] = sizes[i];
		A->rows_values[i] = v + o;
		A->rows_index[i] = ix + o;
		o += sizes[i];
	}
	reg_add(A, v, ix, nnz);
	return A;
}

static int cmp_u32(const void *a, const void *b)
{
	uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
	return x < y ? -1 : (x > y);
}

nb_sparse_t *nb_sparse_create(const nb_graph_t *graph, const uint32_t *perm,
			      uint32_t vars_per_node)
{
	const uint32_t N = graph->N * vars_per_node;
	uint32_t *sizes = malloc((N ? N : 1) * sizeof(uint32_t));
	if (!sizes)
		return NULL;
	for (uint32_t i = 0; i < graph->N; i++)
		for (uint32_t k1 = 0; k1 < vars_per_node; k1++) {
			uint32_t irow = (perm ? perm[i] : i) * vars_per_node + k1;
			sizes[irow] = (graph->N_adj[i] + 1) * vars_per_node;
		}
	nb_sparse_t *A = alloc_slab(N, sizes);
	free(sizes);
	if (!A)
		return NULL;
	/* rows from the graph: neighbours then self, each expanded to the node's
	 * variables (columns use the graph ids, rows the permuted ones, as in
	 * sparse.c:33-52), sorted ascending */
	for (uint32_t i = 0; i < graph->N; i++)
		for (uint32_t k1 = 0; k1 < vars_per_node; k1++) {
			uint32_t irow = (perm ? perm[i] : i) * vars_per_node + k1;
			uint32_t *row = A->rows_index[irow];
			for (uint32_t j = 0; j < graph->N_adj[i]; j++)
				for (uint32_t k2 = 0; k2 < vars_per_node; k2++)
					row[j * vars_per_node + k2] = graph->adj[i][j] * vars_per_node + k2;
			for (uint32_t k2 = 0; k2 < vars_per_node; k2++)
				row[graph->N_adj[i] * vars_per_node + k2] = i * vars_per_node + k2;
			qsort(row, A->rows_size[irow], sizeof(uint32_t), cmp_u32);
		}
	return A;
}

nb_sparse_t *nb_sparse_clone(nb_sparse_t *A)
{
	nb_sparse_t *C = alloc_slab(A->N, A->rows_size);
	if (!C)
		return NULL;
	for (uint32_t i = 0; i < A->N; i++) {
		memcpy(C->rows_index[i], A->rows_index[i], A->rows_size[i] * sizeof(uint32_t));
		memcpy(C->rows_values[i], A->rows_values[i], A->rows_size[i] * sizeof(double));
	}
	return C;
}

void nb_sparse_destroy(nb_sparse_t *A)
{
	slab_t s;
	const int own = reg_take(A, &s);
	for (uint32_t i = 0; i < A->N; i++) {
		if (!own || A->rows_values[i] < s.vals || A->rows_values[i] >= s.vals + s.nnz)
			free(A->rows_values[i]);
		if (!own || A->rows_index[i] < s.idx || A->rows_index[i] >= s.idx + s.nnz)
			free(A->rows_index[i]);
	}
	if (own) {
		free(s.vals);
		free(s.idx);
	}
	free(A->rows_values);
	free(A->rows_index);
	free(A->rows_size);
	free(A);
}

void nb_sparse_reset(nb_sparse_t *A)
{
	for (uint32_t i = 0; i < A->N; i++)
		memset(A->rows_values[i], 0, A->rows_size[i] * sizeof(double));
}

/* nb_sparse_bsearch_row (sparse_struct.c:7-20) */
static uint32_t bsearch_row(const nb_sparse_t *A, uint32_t i, uint32_t col)
{
	int imin = 0, imax = (int)A->rows_size[i] - 1;
	uint32_t index = (uint32_t)((imin + imax) / 2);
	while (A->rows_index[i][index] != col && imin <= imax) {
		index = (uint32_t)((imin + imax) / 2);
		if (A->rows_index[i][index] < col)
			imin = index + 1;
		else
			imax = index - 1;
	}
	return index;
}

static void missing(const char *fn, const nb_sparse_t *A, uint32_t i, uint32_t j, double v)
{
	printf("ERROR: Entry of sparse matrix is not allocated.\n");
	printf("    -> %s(*A=%p, i=%i, j=%i, value=%lf)\n", fn, (const void *)A, i, j, v);
	g_err = NBG_ERR_PATTERN;
}

void nb_sparse_set(nb_sparse_t *A, uint32_t i, uint32_t j, double value)
{
	uint32_t k = bsearch_row(A, i, j);
	if (A->rows_index[i][k] == j)
		A->rows_values[i][k] = value;
	else
		missing("nb_sparse_set", A, i, j, value);
}

double nb_sparse_get(const nb_sparse_t *A, uint32_t i, uint32_t j)
{
	uint32_t k = bsearch_row(A, i, j);
	return A->rows_index[i][k] == j ? A->rows_values[i][k] : 0.0;
}

double nb_sparse_get_and_set(nb_sparse_t *A, uint32_t i, uint32_t j, double value)
{
	uint32_t k = bsearch_row(A, i, j);
	if (A->rows_index[i][k] == j) {
		double v = A->rows_values[i][k];
		A->rows_values[i][k] = value;
		return v;
	}
	missing("nb_sparse_get_and_set", A, i, j, value);
	return 0.0;
}

bool nb_sparse_is_non_zero(const nb_sparse_t *A, uint32_t i, uint32_t j)
{
	return A->rows_index[i][bsearch_row(A, i, j)] == j;
}

void nb_sparse_add(nb_sparse_t *A, uint32_t i, uint32_t j, double value)
{
	uint32_t k = bsearch_row(A, i, j);
	if (A->rows_index[i][k] == j)
		A->rows_values[i][k] += value;
	else
		missing("nb_sparse_add", A, i, j, value);
}

uint32_t nb_sparse_get_size(const nb_sparse_t *A)
{
	return A->N;
}

uint32_t nb_sparse_get_nnz(const nb_sparse_t *A)
{
	uint32_t nnz = 0;
	for (uint32_t i = 0; i < A->N; i++)
		nnz += A->rows_size[i];
	return nnz;
}

/* sparse.c:416-430, same order of the row walk and of the RHS updates */
void nb_sparse_set_Dirichlet_condition(nb_sparse_t *A, double *RHS, uint32_t idx, double value)
{
	for (uint32_t j = 0; j < A->rows_size[idx]; j++) {
		uint32_t jdx = A->rows_index[idx][j];
		if (idx == jdx) {
			A->rows_values[idx][j] = 1.0;
			RHS[idx] = value;
		} else {
			A->rows_values[idx][j] = 0.0;
			double var = nb_sparse_get_and_set(A, jdx, idx, 0.0);
			RHS[jdx] -= var * value;
		}
	}
}

/* ------------------------------------------------------------ GPU calls */
/* Flat CSR view of a matrix: zero-copy when its rows still sit in their
 * slab in order, else gathered into temporary arrays. */
typedef struct {
	uint32_t *row_ptr;
	const uint32_t *col;
	const double *val;
	void *own_col, *own_val;
} flat_t;

static int flatten(const nb_sparse_t *A, flat_t *f)
{
	memset(f, 0, sizeof(*f));
	f->row_ptr = malloc(((size_t)A->N + 1) * sizeof(uint32_t));
	if (!f->row_ptr)
		return NBG_ERR_NOMEM;
	f->row_ptr[0] = 0;
	for (uint32_t i = 0; i < A->N; i++)
		f->row_ptr[i + 1] = f->row_ptr[i] + A->rows_size[i];
	slab_t s;
	int contiguous = reg_find(A, &s);
	for (uint32_t i = 0; contiguous && i < A->N; i++)
		contiguous = A->rows_values[i] == s.vals + f->row_ptr[i] &&
			     A->rows_index[i] == s.idx + f->row_ptr[i];
	if (contiguous) {
		f->col = s.idx;
		f->val = s.vals;
		return NBG_OK;
	}
	const uint64_t nnz = f->row_ptr[A->N];
	uint32_t *c = malloc((nnz ? nnz : 1) * sizeof(uint32_t));
	double *v = malloc((nnz ? nnz : 1) * sizeof(double));
	if (!c || !v) {
		free(c);
		free(v);
		free(f->row_ptr);
		return NBG_ERR_NOMEM;
	}
	for (uint32_t i = 0; i < A->N; i++) {
		memcpy(c + f->row_ptr[i], A->rows_index[i], A->rows_size[i] * sizeof(uint32_t));
		memcpy(v + f->row_ptr[i], A->rows_values[i], A->rows_size[i] * sizeof(double));
	}
	f->col = f->own_col = c;
	f->val = f->own_val = v;
	return NBG_OK;
}

static void unflatten(flat_t *f)
{
	free(f->row_ptr);
	free(f->own_col);
	free(f->own_val);
}

static pthread_mutex_t g_solver_lock = PTHREAD_MUTEX_INITIALIZER;
static nbg_solver_t *g_solver;

static int solve(const nb_sparse_t *A, const double *b, double *x, uint32_t max_iter,
		 double tol, uint32_t *niter, double *tol_reached, unsigned flags)
{
	flat_t f;
	int rc = flatten(A, &f);
	if (rc != NBG_OK)
		return rc;
	pthread_mutex_lock(&g_solver_lock);
	if (!g_solver)
		rc = nbg_solver_create(&g_solver, NULL);
	if (rc == NBG_OK)
		rc = nbg_solver_set_matrix(g_solver, A->N, f.row_ptr, f.col, f.val, NBG_CSR_ONLY);
	nbg_solve_info_t info;
	memset(&info, 0, sizeof(info));
	if (rc == NBG_OK)
		rc = nbg_solver_solve(g_solver, b, x, max_iter, tol, flags, NBG_METHOD_NBOTS, &info);
	pthread_mutex_unlock(&g_solver_lock);
	unflatten(&f);
	if (rc < 0)
		return rc;
	if (niter)
		*niter = info.niter;
	if (tol_reached)
		*tol_reached = info.tol_reached;
	return info.status;
}

int nb_sparse_solve_CG_precond_Jacobi(const nb_sparse_t *A, const double *b, double *x,
				      uint32_t max_iter, double tolerance,
				      uint32_t *niter_performed, double *tolerance_reached,
				      uint32_t omp_parallel_threads)
{
	if (nbg_dropin_cpu()) {
		cg_fn next = (cg_fn)nbg_dropin_next("nb_sparse_solve_CG_precond_Jacobi");
		return next ? next(A, b, x, max_iter, tolerance, niter_performed,
				   tolerance_reached, omp_parallel_threads) : NBG_ERR_ARG;
	}
	(void)omp_parallel_threads;
	return solve(A, b, x, max_iter, tolerance, niter_performed, tolerance_reached,
		     NBG_CG_JACOBI);
}

int nb_sparse_solve_conjugate_gradient(const nb_sparse_t *A, const double *b, double *x,
				       uint32_t max_iter, double tolerance,
				       uint32_t *niter_performed, double *tolerance_reached,
				       uint32_t omp_parallel_threads)
{
	if (nbg_dropin_cpu()) {
		cg_fn next = (cg_fn)nbg_dropin_next("nb_sparse_solve_conjugate_gradient");
		return next ? next(A, b, x, max_iter, tolerance, niter_performed,
				   tolerance_reached, omp_parallel_threads) : NBG_ERR_ARG;
	}
	(void)omp_parallel_threads;
	return solve(A, b, x, max_iter, tolerance, niter_performed, tolerance_reached, 0);
}

void nb_sparse_multiply_vector(const nb_sparse_t *A, const double *in, double *out,
			       uint32_t omp_parallel_threads)
{
	if (nbg_dropin_cpu()) {
		spmv_fn next = (spmv_fn)nbg_dropin_next("nb_sparse_multiply_vector");
		if (next)
			next(A, in, out, omp_parallel_threads);
		else
			g_err = NBG_ERR_ARG;
		return;
	}
	(void)omp_parallel_threads;
	flat_t f;
	if (flatten(A, &f) != NBG_OK) {
		g_err = NBG_ERR_NOMEM;
		return;
	}
	const size_t N = A->N, nnz = f.row_ptr[N];
	void *d_rp = NULL, *d_ci = NULL, *d_v = NULL, *d_x = NULL, *d_y = NULL;
	int rc = nbg_dev_alloc(&d_rp, 4 * (N + 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&d_ci, 4 * (nnz ? nnz : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&d_v, 8 * (nnz ? nnz : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&d_x, 8 * (N ? N : 1));
	if (rc == NBG_OK) rc = nbg_dev_alloc(&d_y, 8 * (N ? N : 1));
	if (rc == NBG_OK) rc = nbg_h2d(d_rp, f.row_ptr, 4 * (N + 1), NULL);
	if (rc == NBG_OK) rc = nbg_h2d(d_ci, f.col, 4 * nnz, NULL);
	if (rc == NBG_OK) rc = nbg_h2d(d_v, f.val, 8 * nnz, NULL);
	if (rc == NBG_OK) rc = nbg_h2d(d_x, in, 8 * N, NULL);
	if (rc == NBG_OK) rc = nbg_spmv_csr_f64((uint32_t)N, d_rp, d_ci, d_v, d_x, d_y, NULL);
	if (rc == NBG_OK) rc = nbg_d2h(out, d_y, 8 * N, NULL);
	if (rc == NBG_OK) rc = nbg_stream_sync(NULL);
	if (rc != NBG_OK)
		g_err = rc;
	nbg_dev_free(d_rp); nbg_dev_free(d_ci); nbg_dev_free(d_v);
	nbg_dev_free(d_x); nbg_dev_free(d_y);
	unflatten(&f);
}
