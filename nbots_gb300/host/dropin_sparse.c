/*
 * Drop-in nb_sparse_* and CG entry points (declared in nbots_dropin.h).
 *
 * Matrices made here back all their rows with two slabs (values, column
 * indices) in row order, so the GPU path uploads them without copying row by
 * row; the row-of-pointers struct stays nbots' own (sparse_struct.h:6-11),
 * so code that reads or replaces rows directly keeps working.  A registry
 * remembers which matrices own slabs and keeps each one's device copy
 * between GPU calls; destroy frees any row that no longer points into its
 * slab one by one, and matrices nbots allocated row by row entirely that way
 * (nb_free_mem is free(), memory_bot/allocate_mem.c).
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
/* One record per matrix this library created.  Besides the slabs it holds
 * the matrix's device copy (an nbg_solver_t: CSR, block layout, vectors and
 * workspace), kept from one GPU call to the next and dropped by
 * nb_sparse_destroy, and a dirty flag that every host-side write through
 * this library sets (nb_sparse_add / set / get_and_set / reset /
 * set_Dirichlet_condition / set_identity_row / make_diagonal / scale /
 * multiply_scalar / transpose, and the targets of get_transpose and
 * fill_permutation).  nbots itself writes values of a matrix it did not
 * allocate only through those functions, so a clean matrix's device copy
 * is current and a GPU call sends only its vectors. */
typedef struct slab {
	const nb_sparse_t *A;
	double *vals;
	uint32_t *idx;
	uint32_t *row_ptr;       /* N + 1 offsets of the rows in the slabs */
	uint64_t nnz;
	volatile int dirty;      /* host values written since the device copy */
	nbg_solver_t *dev;       /* device copy, or NULL */
	size_t dev_bytes;
	uint64_t last_use;
	pthread_mutex_t lock;    /* one GPU call on this matrix at a time */
} slab_t;

static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;
static slab_t **g_slabs;
static size_t g_n, g_cap;
static uint64_t g_epoch = 1;     /* bumped whenever the registry changes */
static uint64_t g_clock;         /* use counter for the eviction order */
static size_t g_dev_bytes;       /* device bytes held by all copies */
static __thread int g_err;
/* per-thread memo of the last lookup, valid while g_epoch is unchanged */
static __thread const nb_sparse_t *tl_A;
static __thread slab_t *tl_slab;
static __thread uint64_t tl_epoch;

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

/* NBG_DROPIN_EXACT_CG=1: the drop-in CGs run nbots' arithmetic operation for
 * operation on the CSR (no FMA, division by the diagonal) instead of nbots'
 * iteration on the block layout; for bit-level comparisons. */
static int exact_cg(void)
{
	const char *v = getenv("NBG_DROPIN_EXACT_CG");
	return v && v[0] == '1' && v[1] == 0;
}

/* Device bytes the per-matrix copies may hold together before the least
 * recently used ones are dropped: NBG_DROPIN_CACHE_MB (default 16384); 0
 * keeps no copy between calls. */
static size_t cache_limit(void)
{
	const char *v = getenv("NBG_DROPIN_CACHE_MB");
	if (!v || !*v)
		return (size_t)16384 << 20;
	return (size_t)strtoull(v, NULL, 10) << 20;
}

typedef int (*cg_fn)(const nb_sparse_t *, const double *, double *, uint32_t, double,
		     uint32_t *, double *, uint32_t);
typedef void (*spmv_fn)(const nb_sparse_t *, const double *, double *, uint32_t);

static uint64_t epoch_now(void)
{
	return __atomic_load_n(&g_epoch, __ATOMIC_ACQUIRE);
}

static int reg_add(slab_t *s)
{
	int ok = 1;
	pthread_mutex_lock(&g_lock);
	if (g_n == g_cap) {
		size_t c = g_cap ? 2 * g_cap : 64;
		slab_t **a = realloc(g_slabs, c * sizeof(slab_t *));
		if (a) {
			g_slabs = a;
			g_cap = c;
		} else {
			ok = 0;
		}
	}
	if (ok) {
		g_slabs[g_n++] = s;
		/* a matrix may reuse the address of one another thread last saw
		 * as foreign */
		__atomic_add_fetch(&g_epoch, 1, __ATOMIC_RELEASE);
	}
	pthread_mutex_unlock(&g_lock);
	return ok;
}

static slab_t *reg_take(const nb_sparse_t *A)
{
	slab_t *s = NULL;
	pthread_mutex_lock(&g_lock);
	for (size_t i = 0; i < g_n; i++)
		if (g_slabs[i]->A == A) {
			s = g_slabs[i];
			g_slabs[i] = g_slabs[--g_n];
			__atomic_add_fetch(&g_epoch, 1, __ATOMIC_RELEASE);
			break;
		}
	pthread_mutex_unlock(&g_lock);
	return s;
}

/* The record of a matrix this library created, or NULL for one nbots
 * allocated itself (row by row). */
static slab_t *find_slab(const nb_sparse_t *A)
{
	const uint64_t e = epoch_now();
	if (A == tl_A && e == tl_epoch)
		return tl_slab;
	slab_t *s = NULL;
	pthread_mutex_lock(&g_lock);
	for (size_t i = 0; i < g_n; i++)
		if (g_slabs[i]->A == A) {
			s = g_slabs[i];
			break;
		}
	pthread_mutex_unlock(&g_lock);
	tl_A = A;
	tl_slab = s;
	tl_epoch = e;
	return s;
}

/* A host-side write to A's values. */
static void touch(const nb_sparse_t *A)
{
	slab_t *s = find_slab(A);
	if (s)
		s->dirty = 1;
}

void nbg_dropin_sparse_touch(const nb_sparse_t *A)
{
	touch(A);
}

static void drop_device(slab_t *s)
{
	if (!s->dev)
		return;
	nbg_solver_destroy(s->dev);
	s->dev = NULL;
	pthread_mutex_lock(&g_lock);
	g_dev_bytes -= s->dev_bytes;
	pthread_mutex_unlock(&g_lock);
	s->dev_bytes = 0;
}

/* Drop the least recently used device copies (other than `keep`, and none
 * in use by another thread) until `extra` more bytes fit under the limit. */
static void evict_for(const slab_t *keep, size_t extra)
{
	const size_t limit = cache_limit();
	for (;;) {
		slab_t *victim = NULL;
		pthread_mutex_lock(&g_lock);
		if (g_dev_bytes + extra > limit)
			for (size_t i = 0; i < g_n; i++) {
				slab_t *c = g_slabs[i];
				if (c == keep || !c->dev)
					continue;
				if (!victim || c->last_use < victim->last_use)
					victim = c;
			}
		if (victim && pthread_mutex_trylock(&victim->lock) != 0)
			victim = NULL;  /* busy: leave it */
		pthread_mutex_unlock(&g_lock);
		if (!victim)
			return;
		drop_device(victim);
		pthread_mutex_unlock(&victim->lock);
	}
}

static nb_sparse_t *alloc_slab(uint32_t N, const uint32_t *sizes)
{
	nb_sparse_t *A = calloc(1, sizeof(*A));
	slab_t *s = calloc(1, sizeof(*s));
	if (!A || !s) {
		free(A);
		free(s);
		return NULL;
	}
	A->N = N;
	A->rows_values = malloc((N ? N : 1) * sizeof(double *));
	A->rows_index = malloc((N ? N : 1) * sizeof(uint32_t *));
	A->rows_size = malloc((N ? N : 1) * sizeof(uint32_t));
	s->row_ptr = malloc(((size_t)N + 1) * sizeof(uint32_t));
	uint64_t nnz = 0;
	for (uint32_t i = 0; i < N; i++)
		nnz += sizes[i];
	double *v = calloc(nnz ? nnz : 1, sizeof(double));
	uint32_t *ix = malloc((nnz ? nnz : 1) * sizeof(uint32_t));
	if (!A->rows_values || !A->rows_index || !A->rows_size || !s->row_ptr || !v || !ix ||
	    nnz > UINT32_MAX) {
		free(A->rows_values); free(A->rows_index); free(A->rows_size);
		free(s->row_ptr); free(v); free(ix); free(A); free(s);
		return NULL;
	}
	uint64_t o = 0;
	s->row_ptr[0] = 0;
	for (uint32_t i = 0; i < N; i++) {
		A->rows_size[i] = sizes[i];
		A->rows_values[i] = v + o;
		A->rows_index[i] = ix + o;
		o += sizes[i];
		s->row_ptr[i + 1] = (uint32_t)o;
	}
	s->A = A;
	s->vals = v;
	s->idx = ix;
	s->nnz = nnz;
	s->dirty = 1;
	pthread_mutex_init(&s->lock, NULL);
	if (!reg_add(s)) {
		/* out of memory for the registry: give everything back, as
		 * nbots returns NULL when it cannot allocate */
		pthread_mutex_destroy(&s->lock);
		free(A->rows_values); free(A->rows_index); free(A->rows_size);
		free(s->row_ptr); free(v); free(ix); free(A); free(s);
		return NULL;
	}
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
	slab_t *s = reg_take(A);
	for (uint32_t i = 0; i < A->N; i++) {
		if (!s || A->rows_values[i] < s->vals || A->rows_values[i] >= s->vals + s->nnz)
			free(A->rows_values[i]);
		if (!s || A->rows_index[i] < s->idx || A->rows_index[i] >= s->idx + s->nnz)
			free(A->rows_index[i]);
	}
	if (s) {
		pthread_mutex_lock(&s->lock);
		drop_device(s);
		pthread_mutex_unlock(&s->lock);
		pthread_mutex_destroy(&s->lock);
		free(s->vals);
		free(s->idx);
		free(s->row_ptr);
		free(s);
	}
	free(A->rows_values);
	free(A->rows_index);
	free(A->rows_size);
	free(A);
}

void nb_sparse_reset(nb_sparse_t *A)
{
	touch(A);
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
	touch(A);
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
	touch(A);
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
	touch(A);
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
	touch(A);
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

/* The other writers of sparse.h.  The first four are plain loops over the
 * rows; the last three forward to the next definition in link order
 * (nbots' own, sparse.c:289-347) after marking the written matrix. */
void nb_sparse_set_identity_row(nb_sparse_t *A, uint32_t row)          /* sparse.c:148-153 */
{
	touch(A);
	memset(A->rows_values[row], 0, A->rows_size[row] * sizeof(double));
	nb_sparse_set(A, row, row, 1.0);
}

void nb_sparse_make_diagonal(nb_sparse_t *A, double diag_val)          /* sparse.c:155-162 */
{
	touch(A);
	for (uint32_t i = 0; i < A->N; i++) {
		memset(A->rows_values[i], 0, A->rows_size[i] * sizeof(double));
		nb_sparse_set(A, i, i, diag_val);
	}
}

void nb_sparse_scale(nb_sparse_t *A, double factor)                     /* sparse.c:221-227 */
{
	touch(A);
	for (uint32_t i = 0; i < A->N; i++)
		for (uint32_t k = 0; k < A->rows_size[i]; k++)
			A->rows_values[i][k] *= factor;
}

void nb_sparse_multiply_scalar(nb_sparse_t *A, double scalar,           /* sparse.c:394-403 */
			       uint32_t omp_parallel_threads)
{
	(void)omp_parallel_threads;
	nb_sparse_scale(A, scalar);
}

void nb_sparse_transpose(nb_sparse_t *A)                                /* sparse.c:334-346 */
{
	touch(A);
	void (*next)(nb_sparse_t *) = (void (*)(nb_sparse_t *))nbg_dropin_next(
		"nb_sparse_transpose");
	if (next)
		next(A);
	else
		g_err = NBG_ERR_ARG;
}

void nb_sparse_get_transpose(const nb_sparse_t *A, nb_sparse_t *At)     /* sparse.c:316-332 */
{
	touch(At);
	void (*next)(const nb_sparse_t *, nb_sparse_t *) =
		(void (*)(const nb_sparse_t *, nb_sparse_t *))nbg_dropin_next(
			"nb_sparse_get_transpose");
	if (next)
		next(A, At);
	else
		g_err = NBG_ERR_ARG;
}

void nb_sparse_fill_permutation(const nb_sparse_t *A, nb_sparse_t *Ar,  /* sparse.c:289-303 */
				const uint32_t *perm, const uint32_t *iperm)
{
	touch(Ar);
	void (*next)(const nb_sparse_t *, nb_sparse_t *, const uint32_t *, const uint32_t *) =
		(void (*)(const nb_sparse_t *, nb_sparse_t *, const uint32_t *,
			  const uint32_t *))nbg_dropin_next("nb_sparse_fill_permutation");
	if (next)
		next(A, Ar, perm, iperm);
	else
		g_err = NBG_ERR_ARG;
}

/* ------------------------------------------------------------ GPU calls */
/* Flat CSR view of a matrix nbots allocated row by row: gathered into
 * temporary arrays. */
typedef struct {
	uint32_t *row_ptr;
	uint32_t *col;
	double *val;
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
	const uint64_t nnz = f->row_ptr[A->N];
	f->col = malloc((nnz ? nnz : 1) * sizeof(uint32_t));
	f->val = malloc((nnz ? nnz : 1) * sizeof(double));
	if (!f->col || !f->val) {
		free(f->col);
		free(f->val);
		free(f->row_ptr);
		return NBG_ERR_NOMEM;
	}
	for (uint32_t i = 0; i < A->N; i++) {
		memcpy(f->col + f->row_ptr[i], A->rows_index[i], A->rows_size[i] * sizeof(uint32_t));
		memcpy(f->val + f->row_ptr[i], A->rows_values[i], A->rows_size[i] * sizeof(double));
	}
	return NBG_OK;
}

static void unflatten(flat_t *f)
{
	free(f->row_ptr);
	free(f->col);
	free(f->val);
}

/* Every row still sits in its slab, in order (the layout the device copy
 * mirrors). */
static int in_slabs(const slab_t *s)
{
	const nb_sparse_t *A = s->A;
	for (uint32_t i = 0; i < A->N; i++)
		if (A->rows_values[i] != s->vals + s->row_ptr[i] ||
		    A->rows_index[i] != s->idx + s->row_ptr[i] ||
		    A->rows_size[i] != s->row_ptr[i + 1] - s->row_ptr[i])
			return 0;
	return 1;
}

/* Locks a matrix this library created and makes its device copy current:
 * built on first use (pattern, block layout when the pattern is
 * node-blocked, values), values re-sent when the host wrote them since.
 * With send_values 0 a new copy gets the pattern only (the caller writes the
 * values on the device).  Returns NULL, unlocked, when the matrix is not one
 * of this library's, its rows left their slabs, or copies are switched off
 * (NBG_DROPIN_CACHE_MB=0); *rc carries any GPU error. */
static slab_t *lock_device(const nb_sparse_t *A, int send_values, int *rc)
{
	*rc = NBG_OK;
	slab_t *s = find_slab(A);
	if (!s || cache_limit() == 0)
		return NULL;
	pthread_mutex_lock(&s->lock);
	/* the layout is checked whenever the copy is built or re-sent; a clean
	 * copy is used as it is (rows moved by direct writes are announced with
	 * nbg_dropin_sparse_touch, which marks the matrix changed) */
	if ((!s->dev || s->dirty) && !in_slabs(s)) {
		drop_device(s);
		pthread_mutex_unlock(&s->lock);
		return NULL;
	}
	if (!s->dev) {
		int r = nbg_solver_create(&s->dev, NULL);
		if (r == NBG_OK)
			r = nbg_solver_set_matrix(s->dev, A->N, s->row_ptr, s->idx,
						  send_values ? s->vals : NULL, 0);
		if (r != NBG_OK) {
			nbg_solver_destroy(s->dev);
			s->dev = NULL;
			pthread_mutex_unlock(&s->lock);
			*rc = r;
			return NULL;
		}
		s->dev_bytes = nbg_solver_device_bytes(s->dev);
		pthread_mutex_lock(&g_lock);
		g_dev_bytes += s->dev_bytes;
		pthread_mutex_unlock(&g_lock);
		s->dirty = !send_values;
		evict_for(s, 0);
	} else if (s->dirty && send_values) {
		s->dirty = 0;
		int r = nbg_solver_set_matrix(s->dev, A->N, s->row_ptr, s->idx, s->vals,
					      NBG_PATTERN_SAME);
		if (r != NBG_OK) {
			s->dirty = 1;
			drop_device(s);
			pthread_mutex_unlock(&s->lock);
			*rc = r;
			return NULL;
		}
	}
	pthread_mutex_lock(&g_lock);
	s->last_use = ++g_clock;
	pthread_mutex_unlock(&g_lock);
	return s;
}

static void unlock_device(slab_t *s)
{
	if (s->dev) {
		/* workspaces grow on first use: keep the account right */
		size_t b = nbg_solver_device_bytes(s->dev);
		pthread_mutex_lock(&g_lock);
		g_dev_bytes += b - s->dev_bytes;
		pthread_mutex_unlock(&g_lock);
		s->dev_bytes = b;
	}
	pthread_mutex_unlock(&s->lock);
}

/* Device copy access for the other drop-in files (assembly, boundary
 * conditions): lock, the solver context, then unlock with `synced` set when
 * host and device values agree again. */
nbg_solver_t *nbg_dropin_lock_device(const nb_sparse_t *A, int send_values, int *rc)
{
	slab_t *s = lock_device(A, send_values, rc);
	return s ? s->dev : NULL;
}

void nbg_dropin_unlock_device(const nb_sparse_t *A, int synced)
{
	slab_t *s = find_slab(A);
	if (!s)
		return;
	if (synced)
		s->dirty = 0;
	unlock_device(s);
}

/* The slab of a locked matrix (values, host row offsets), for writing back
 * device results. */
int nbg_dropin_slab(const nb_sparse_t *A, double **vals, const uint32_t **row_ptr)
{
	slab_t *s = find_slab(A);
	if (!s)
		return NBG_ERR_ARG;
	*vals = s->vals;
	*row_ptr = s->row_ptr;
	return NBG_OK;
}

/* A matrix nbots allocated (or one whose rows moved): a device copy for
 * this call only. */
static pthread_mutex_t g_transient_lock = PTHREAD_MUTEX_INITIALIZER;
static nbg_solver_t *g_transient;

static int transient_set(const nb_sparse_t *A, flat_t *f, unsigned flags)
{
	int rc = flatten(A, f);
	if (rc != NBG_OK)
		return rc;
	if (!g_transient)
		rc = nbg_solver_create(&g_transient, NULL);
	if (rc == NBG_OK)
		rc = nbg_solver_set_matrix(g_transient, A->N, f->row_ptr, f->col, f->val, flags);
	if (rc != NBG_OK)
		unflatten(f);
	return rc;
}

static int solve(const nb_sparse_t *A, const double *b, double *x, uint32_t max_iter,
		 double tol, uint32_t *niter, double *tol_reached, unsigned flags)
{
	const int method = exact_cg() ? NBG_METHOD_NBOTS : NBG_METHOD_NBOTS_FAST;
	nbg_solve_info_t info;
	memset(&info, 0, sizeof(info));
	int rc = NBG_OK;
	slab_t *s = lock_device(A, 1, &rc);
	if (s) {
		rc = nbg_solver_solve(s->dev, b, x, max_iter, tol, flags, method, &info);
		unlock_device(s);
	} else if (rc == NBG_OK) {
		flat_t f;
		pthread_mutex_lock(&g_transient_lock);
		rc = transient_set(A, &f, method == NBG_METHOD_NBOTS ? NBG_CSR_ONLY : 0);
		if (rc == NBG_OK) {
			rc = nbg_solver_solve(g_transient, b, x, max_iter, tol, flags, method,
					      &info);
			unflatten(&f);
		}
		pthread_mutex_unlock(&g_transient_lock);
	}
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
	int rc = NBG_OK;
	slab_t *s = lock_device(A, 1, &rc);
	if (s) {
		rc = nbg_solver_multiply(s->dev, in, out);
		unlock_device(s);
	} else if (rc == NBG_OK) {
		flat_t f;
		pthread_mutex_lock(&g_transient_lock);
		rc = transient_set(A, &f, NBG_CSR_ONLY);
		if (rc == NBG_OK) {
			rc = nbg_solver_multiply(g_transient, in, out);
			unflatten(&f);
		}
		pthread_mutex_unlock(&g_transient_lock);
	}
	if (rc != NBG_OK)
		g_err = rc;
}
