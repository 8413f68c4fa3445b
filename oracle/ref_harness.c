/*
 * Reference harness: runs the UNMODIFIED nbots library (oracle/_ref/
 * libnbots_ref.so, built from the project's sources by oracle/Makefile.ref)
 * on a problem file and dumps every intermediate of the FEM hot path, so the
 * oracle restatement and the GPU path can be pinned to it.  Test
 * infrastructure only: it is built and run in a container that holds the
 * reference sources, and its outputs are committed as tests/golden/*.npz.
 *
 *   ref_harness problem <problem.bin> <out.bin> [cg_threads]
 *   ref_harness utest   <problem.txt> <N_vtx> <mesh_out.bin> <out.bin> [pwh]
 *
 * "problem" builds nbots mesh objects from the arrays of a problem file
 * (format written by nbots_gb300/problem_io.py) and replays nbots' FEM entry
 * (pde_bot/finite_element/solid_mechanics/static_elasticity2D.c:31-81)
 * step by step so that each stage can be dumped.  Per-element Young's moduli
 * are not expressible through that entry (it takes one material), so the
 * element loop of pipeline_assemble_system (pipeline.c:42-73) is driven here
 * with one material per element, calling nbots' own exported element
 * routines (utils.c:9-60, pipeline.c:174-264); for a uniform modulus the
 * harness also runs pipeline_assemble_system itself and records whether the
 * two agree bit for bit.
 *
 * "utest" reproduces the flow of nbots' FEM unit test
 * (utest/sources/nb/pde_bot/finite_element/solid_mechanics/
 * static_elasticity2D.c:281-338): tessellate the model of a problem text file
 * to N_vtx vertices, call nb_fem_compute_2D_Solid_Mechanics, and dump the
 * generated T3 mesh as a problem file plus the results.  With "pwh" the two
 * function-valued Neumann segments of the plate-with-hole test are added
 * (same file, :208-235), and their values at the segment nodes are stored in
 * the problem file.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <stdbool.h>
#include <math.h>

#include "nb/memory_bot.h"
#include "nb/io_bot.h"
#include "nb/graph_bot.h"
#include "nb/geometric_bot.h"
#include "nb/solver_bot.h"
#include "nb/pde_bot.h"
#include "nb/pde_bot/boundary_conditions/bcond_read.h"

/* private reference headers (struct layouts and non-static internals) */
#include "solver_bot/sparse/sparse_struct.h"
#include "geometric_bot/mesh/mesh2D/elements2D/mshquad_struct.h"
#include "geometric_bot/mesh/mesh2D/elements2D/msh3trg_struct.h"
#include "pde_bot/finite_element/utils.h"
#include "pde_bot/finite_element/solid_mechanics/pipeline.h"
#include "pde_bot/finite_element/solid_mechanics/set_bconditions.h"

/* ------------------------------------------------------------ output */
enum { DT_F64 = 0, DT_U32 = 1, DT_I32 = 2, DT_U8 = 3 };
static FILE *g_out;

static void dump(const char *name, int dt, const void *data, uint64_t n)
{
	static const size_t sz[] = {8, 4, 4, 1};
	uint32_t len = (uint32_t)strlen(name);
	uint32_t d = (uint32_t)dt;
	fwrite(&len, 4, 1, g_out);
	fwrite(name, 1, len, g_out);
	fwrite(&d, 4, 1, g_out);
	fwrite(&n, 8, 1, g_out);
	if (n)
		fwrite(data, sz[dt], n, g_out);
}

static void dump_f64(const char *name, double v) { dump(name, DT_F64, &v, 1); }
static void dump_u32(const char *name, uint32_t v) { dump(name, DT_U32, &v, 1); }
static void dump_i32(const char *name, int32_t v) { dump(name, DT_I32, &v, 1); }

/* ------------------------------------------------------------ problem file */
typedef struct {
	uint32_t kind, where, id;
	uint8_t mask[2];
	double val[2];
	uint32_t n_nv;
	double *nv;          /* n_nv x 2 values at nodes (function-valued) */
	double *nv_xy;       /* coordinates of those nodes */
} pbc_t;

typedef struct {
	uint32_t nen;
	uint32_t N_nod, N_elem, N_edg, N_vtx, N_sgm, N_bc;
	double *nod;
	uint32_t *conn, *edg, *vtx, *N_nod_x_sgm, **nod_x_sgm;
	double *E, nu, thickness, density, gravity[2];
	uint32_t self_weight, has_enabled;
	bool *enabled;
	pbc_t *bc;
} problem_t;

#define RD(ptr, sz, n) do { if (fread((ptr), (sz), (n), f) != (size_t)(n)) { \
	fprintf(stderr, "short read\n"); exit(2); } } while (0)

static void *xalloc(size_t n) { void *p = calloc(1, n ? n : 1); if (!p) exit(3); return p; }

static void read_problem(const char *path, problem_t *p)
{
	FILE *f = fopen(path, "rb");
	if (!f) { perror(path); exit(2); }
	char magic[4];
	RD(magic, 1, 4);
	if (memcmp(magic, "NBGP", 4)) { fprintf(stderr, "bad magic\n"); exit(2); }
	RD(&p->nen, 4, 1);
	RD(&p->N_nod, 4, 1);
	p->nod = xalloc(16 * (size_t)p->N_nod);
	RD(p->nod, 8, 2 * (size_t)p->N_nod);
	RD(&p->N_elem, 4, 1);
	p->conn = xalloc(4 * (size_t)p->nen * p->N_elem);
	RD(p->conn, 4, (size_t)p->nen * p->N_elem);
	RD(&p->N_edg, 4, 1);
	p->edg = xalloc(8 * (size_t)p->N_edg);
	RD(p->edg, 4, 2 * (size_t)p->N_edg);
	RD(&p->N_vtx, 4, 1);
	p->vtx = xalloc(4 * (size_t)p->N_vtx);
	RD(p->vtx, 4, p->N_vtx);
	RD(&p->N_sgm, 4, 1);
	p->N_nod_x_sgm = xalloc(4 * (size_t)p->N_sgm);
	p->nod_x_sgm = xalloc(sizeof(uint32_t *) * p->N_sgm);
	for (uint32_t s = 0; s < p->N_sgm; s++) {
		RD(&p->N_nod_x_sgm[s], 4, 1);
		p->nod_x_sgm[s] = xalloc(4 * (size_t)p->N_nod_x_sgm[s]);
		RD(p->nod_x_sgm[s], 4, p->N_nod_x_sgm[s]);
	}
	p->E = xalloc(8 * (size_t)p->N_elem);
	RD(p->E, 8, p->N_elem);
	RD(&p->nu, 8, 1);
	RD(&p->thickness, 8, 1);
	RD(&p->density, 8, 1);
	RD(&p->self_weight, 4, 1);
	RD(p->gravity, 8, 2);
	RD(&p->has_enabled, 4, 1);
	p->enabled = NULL;
	if (p->has_enabled) {
		uint8_t *en = xalloc(p->N_elem);
		RD(en, 1, p->N_elem);
		p->enabled = xalloc(sizeof(bool) * p->N_elem);
		for (uint32_t e = 0; e < p->N_elem; e++)
			p->enabled[e] = en[e] != 0;
		free(en);
	}
	RD(&p->N_bc, 4, 1);
	p->bc = xalloc(sizeof(pbc_t) * (p->N_bc ? p->N_bc : 1));
	for (uint32_t k = 0; k < p->N_bc; k++) {
		pbc_t *b = &p->bc[k];
		RD(&b->kind, 4, 1);
		RD(&b->where, 4, 1);
		RD(&b->id, 4, 1);
		RD(b->mask, 1, 2);
		RD(b->val, 8, 2);
		RD(&b->n_nv, 4, 1);
		b->nv = NULL;
		if (b->n_nv) {
			b->nv = xalloc(16 * (size_t)b->n_nv);
			RD(b->nv, 8, 2 * (size_t)b->n_nv);
		}
	}
	fclose(f);
}

/* Function-valued atoms: nbots calls fval(x, t, out) at node coordinates.
 * Each atom gets its own callback that looks the coordinates up in the
 * node values stored in the problem file. */
#define MAX_FN 8
static const pbc_t *g_fn[MAX_FN];
static void fn_lookup(int k, const double *x, double *out)
{
	const pbc_t *b = g_fn[k];
	for (uint32_t i = 0; i < b->n_nv; i++) {
		if (b->nv_xy[2 * i] == x[0] && b->nv_xy[2 * i + 1] == x[1]) {
			out[0] = b->nv[2 * i];
			out[1] = b->nv[2 * i + 1];
			return;
		}
	}
	fprintf(stderr, "function BC: no node at (%g,%g)\n", x[0], x[1]);
	exit(4);
}
#define FN(k) static void fn##k(const double *x, double t, double *o) { (void)t; fn_lookup(k, x, o); }
FN(0) FN(1) FN(2) FN(3) FN(4) FN(5) FN(6) FN(7)
static void (*const g_fnp[MAX_FN])(const double *, double, double *) =
	{fn0, fn1, fn2, fn3, fn4, fn5, fn6, fn7};

static void build_mesh(const problem_t *p, nb_mesh2D_t *mesh, void **msh_out)
{
	if (p->nen == 4) {
		struct nb_mshquad_s *q = xalloc(sizeof(*q));
		q->N_nod = p->N_nod;
		q->nod = p->nod;
		q->N_edg = p->N_edg;
		q->edg = p->edg;
		q->N_elems = p->N_elem;
		q->type = xalloc(p->N_elem);   /* 0: quad */
		q->adj = p->conn;
		q->ngb = xalloc(16 * (size_t)p->N_elem);
		for (size_t i = 0; i < 4 * (size_t)p->N_elem; i++)
			q->ngb[i] = p->N_elem;
		q->N_vtx = p->N_vtx;
		q->vtx = p->vtx;
		q->N_sgm = p->N_sgm;
		q->N_nod_x_sgm = p->N_nod_x_sgm;
		q->nod_x_sgm = p->nod_x_sgm;
		nb_mesh2D_init_from_msh(mesh, q, NB_QUAD);
		*msh_out = q;
	} else {
		struct nb_msh3trg_s *t = xalloc(sizeof(*t));
		t->N_nod = p->N_nod;
		t->nod = p->nod;
		t->N_edg = p->N_edg;
		t->edg = p->edg;
		t->N_elems = p->N_elem;
		t->adj = p->conn;
		t->ngb = xalloc(12 * (size_t)p->N_elem);
		for (size_t i = 0; i < 3 * (size_t)p->N_elem; i++)
			t->ngb[i] = p->N_elem;
		t->N_vtx = p->N_vtx;
		t->vtx = p->vtx;
		t->N_sgm = p->N_sgm;
		t->N_nod_x_sgm = p->N_nod_x_sgm;
		t->nod_x_sgm = p->nod_x_sgm;
		nb_mesh2D_init_from_msh(mesh, t, NB_TRIAN);
		*msh_out = t;
	}
}

static void build_bcond(const problem_t *p, nb_bcond_t *bcond)
{
	int nfn = 0;
	for (uint32_t k = 0; k < p->N_bc; k++) {
		pbc_t *b = &p->bc[k];
		bool mask[2] = {b->mask[0] != 0, b->mask[1] != 0};
		nb_bcond_id id = b->kind == 0 ? NB_DIRICHLET : NB_NEUMANN;
		nb_bcond_where wh = b->where == 0 ? NB_BC_ON_POINT : NB_BC_ON_SEGMENT;
		if (b->n_nv) {
			if (nfn >= MAX_FN) { fprintf(stderr, "too many fn BCs\n"); exit(4); }
			b->nv_xy = xalloc(16 * (size_t)b->n_nv);
			for (uint32_t i = 0; i < b->n_nv; i++) {
				uint32_t nid = b->where == 0 ? p->vtx[b->id]
					: p->nod_x_sgm[b->id][i];
				b->nv_xy[2 * i] = p->nod[2 * nid];
				b->nv_xy[2 * i + 1] = p->nod[2 * nid + 1];
				if (b->kind == 1 && b->where == 0) {
					/* set_neumann reads vertex loads at (0,0) */
					b->nv_xy[2 * i] = 0.0;
					b->nv_xy[2 * i + 1] = 0.0;
				}
			}
			g_fn[nfn] = b;
			nb_bcond_push_function(bcond, id, wh, b->id, mask, g_fnp[nfn]);
			nfn++;
		} else {
			nb_bcond_push(bcond, id, wh, b->id, mask, b->val);
		}
	}
}

static void dump_pattern(const nb_sparse_t *K)
{
	uint32_t N = K->N;
	uint32_t *rp = xalloc(4 * ((size_t)N + 1));
	for (uint32_t i = 0; i < N; i++)
		rp[i + 1] = rp[i] + K->rows_size[i];
	uint32_t *ci = xalloc(4 * (size_t)rp[N]);
	for (uint32_t i = 0; i < N; i++)
		memcpy(ci + rp[i], K->rows_index[i], 4 * (size_t)K->rows_size[i]);
	dump("row_ptr", DT_U32, rp, (uint64_t)N + 1);
	dump("col_idx", DT_U32, ci, rp[N]);
	free(rp);
	free(ci);
}

static void dump_values(const char *name, const nb_sparse_t *K)
{
	uint64_t nnz = 0;
	for (uint32_t i = 0; i < K->N; i++)
		nnz += K->rows_size[i];
	double *v = xalloc(8 * nnz);
	uint64_t o = 0;
	for (uint32_t i = 0; i < K->N; i++) {
		memcpy(v + o, K->rows_values[i], 8 * (size_t)K->rows_size[i]);
		o += K->rows_size[i];
	}
	dump(name, DT_F64, v, nnz);
	free(v);
}

/* pipeline_assemble_system (pipeline.c:42-73) with one material per element:
 * assemble_element / integrate_elemental_system (pipeline.c:83-172) are
 * static in nbots, so their control flow is driven here around nbots' own
 * exported element routines. */
static int assemble_per_element(nb_sparse_t *K, double *F, const nb_mesh2D_t *part,
				const nb_fem_elem_t *elem, const problem_t *p,
				nb_analysis2D_params *params2D)
{
	uint32_t N_elem = nb_mesh2D_get_N_elems(part);
	nb_sparse_reset(K);
	memset(F, 0, nb_sparse_get_size(K) * sizeof(*F));
	nb_material_t *mat = nb_material_create();
	nb_material_set_poisson_module(mat, p->nu);
	nb_material_set_density(mat, p->density);
	uint8_t nn = nb_fem_elem_get_N_nodes(elem);
	double Ke[64], Fe[8], dx[4], dy[4];
	for (uint32_t i = 0; i < N_elem; i++) {
		bool en = p->enabled ? p->enabled[i] : true;
		double D[4] = {1e-6, 1e-6, 1e-6, 1e-6};
		double density = 1e-6;
		if (en) {
			nb_material_set_elasticity_module(mat, p->E[i]);
			nb_pde_get_constitutive_matrix(D, mat, NB_PLANE_STRESS);
			density = nb_material_get_density(mat);
		}
		double fx = 0.0, fy = 0.0;
		if (p->self_weight) {
			fx = p->gravity[0] * density;
			fy = p->gravity[1] * density;
		}
		memset(Ke, 0, sizeof(Ke));
		memset(Fe, 0, sizeof(Fe));
		uint8_t ngp = nb_fem_elem_get_N_gpoints(elem);
		for (uint32_t j = 0; j < ngp; j++) {
			double Jinv[4];
			double detJ = nb_fem_get_jacobian(elem, i, part, j, Jinv);
			if (nb_fem_elem_is_distorted(detJ)) {
				nb_material_destroy(mat);
				return 1;
			}
			nb_fem_get_derivatives(elem, j, Jinv, dx, dy);
			pipeline_sum_gauss_point(elem, j, D, density,
						 params2D->thickness, detJ,
						 dx, dy, fx, fy, Ke, NULL, Fe);
		}
		pipeline_add_to_global_system(elem, i, part, Ke, NULL, Fe, K, NULL, F);
		(void)nn;
	}
	nb_material_destroy(mat);
	return 0;
}

static int run_problem(const char *in, const char *out, uint32_t threads)
{
	problem_t p;
	read_problem(in, &p);
	nb_mesh2D_t *part = xalloc(nb_mesh2D_get_memsize(p.nen == 4 ? NB_QUAD : NB_TRIAN));
	void *msh;
	build_mesh(&p, part, &msh);
	nb_fem_elem_t *elem = nb_fem_elem_create(p.nen == 4 ? NB_QUAD_LINEAR : NB_TRG_LINEAR);
	nb_bcond_t *bcond = xalloc(nb_bcond_get_memsize(2));
	nb_bcond_init(bcond, 2);
	build_bcond(&p, bcond);
	nb_analysis2D_params params2D = {p.thickness, 0.0, 0};

	g_out = fopen(out, "wb");
	if (!g_out) { perror(out); return 2; }

	/* static_elasticity2D.c:44-49 */
	nb_graph_t *graph = xalloc(nb_graph_get_memsize());
	nb_graph_init(graph);
	nb_mesh2D_load_graph(part, graph, NB_NODES_LINKED_BY_ELEMS);
	nb_sparse_t *K = nb_sparse_create(graph, NULL, 2);
	nb_graph_finish(graph);
	uint32_t N = nb_sparse_get_size(K);
	dump_pattern(K);

	double *F = xalloc(8 * (size_t)N);
	int st = assemble_per_element(K, F, part, elem, &p, &params2D);
	dump_i32("assemble_status", st);

	bool uniform = true;
	for (uint32_t e = 1; e < p.N_elem; e++)
		uniform = uniform && p.E[e] == p.E[0];
	if (uniform && st == 0) {
		/* cross-check the driven loop against nbots' own assembly */
		nb_sparse_t *K2 = nb_sparse_clone(K);
		double *F2 = xalloc(8 * (size_t)N);
		nb_material_t *mat = nb_material_create();
		nb_material_set_elasticity_module(mat, p.E[0]);
		nb_material_set_poisson_module(mat, p.nu);
		nb_material_set_density(mat, p.density);
		double grav[2] = {p.gravity[0], p.gravity[1]};
		int st2 = pipeline_assemble_system(K2, NULL, F2, part, elem, mat,
						   p.self_weight != 0, grav,
						   NB_PLANE_STRESS, &params2D, p.enabled);
		int same = st2 == 0;
		for (uint32_t i = 0; same && i < N; i++) {
			same = same && !memcmp(K->rows_values[i], K2->rows_values[i],
					       8 * (size_t)K->rows_size[i]);
			same = same && !memcmp(&F[i], &F2[i], 8);
		}
		dump_i32("driven_assembly_matches_pipeline", same);
		nb_material_destroy(mat);
		nb_sparse_destroy(K2);
		free(F2);
	}
	if (st != 0) {
		fclose(g_out);
		return 0;
	}
	dump_values("K_asm", K);
	dump("F_asm", DT_F64, F, N);

	/* static_elasticity2D.c:67 */
	nb_fem_set_bconditions(part, K, F, bcond, 1.0);
	dump_values("K_bc", K);
	dump("F_bc", DT_F64, F, N);

	/* nb_sparse_multiply_vector on a fixed input (sparse.c:405-414) */
	double *xs = xalloc(8 * (size_t)N), *ys = xalloc(8 * (size_t)N);
	for (uint32_t i = 0; i < N; i++)
		xs[i] = (double)((i * 7919u) % 1000u) / 500.0 - 1.0;
	nb_sparse_multiply_vector(K, xs, ys, 1);
	dump("spmv_x", DT_F64, xs, N);
	dump("spmv_y", DT_F64, ys, N);

	/* solver(): static_elasticity2D.c:83-97 */
	double *u = xalloc(8 * (size_t)N);
	uint32_t niter = 0;
	double tol_reached = 0;
	int cg = nb_sparse_solve_CG_precond_Jacobi(K, F, u, N, 1e-8, &niter,
						   &tol_reached, threads);
	dump("u", DT_F64, u, N);
	dump_u32("cg_niter", niter);
	dump_f64("cg_tol_reached", tol_reached);
	dump_i32("cg_status", cg);

	/* the same Jacobi-PCG from a non-zero initial guess (the damage loop
	 * passes the previous increment, static_damage2D.c:410) */
	{
		double *ux = xalloc(8 * (size_t)N);
		memcpy(ux, xs, 8 * (size_t)N);
		uint32_t nx = 0;
		double tx = 0;
		int cgx = nb_sparse_solve_CG_precond_Jacobi(K, F, ux, N, 1e-8, &nx, &tx, 1);
		dump("u_x0", DT_F64, ux, N);
		dump_u32("cgx0_niter", nx);
		dump_f64("cgx0_tol_reached", tx);
		dump_i32("cgx0_status", cgx);
		free(ux);
	}

	/* unpreconditioned CG (conjugate_gradient.c:13-77), same settings */
	{
		double *up = xalloc(8 * (size_t)N);
		uint32_t np_ = 0;
		double tp = 0;
		int cgp = nb_sparse_solve_conjugate_gradient(K, F, up, N, 1e-8, &np_, &tp, 1);
		dump("u_plain", DT_F64, up, N);
		dump_u32("cgp_niter", np_);
		dump_f64("cgp_tol_reached", tp);
		dump_i32("cgp_status", cgp);
		free(up);
	}

	/* a short run (max_iter = 7) pins the not-converged return path */
	double *u7 = xalloc(8 * (size_t)N);
	uint32_t n7 = 0;
	double t7 = 0;
	int cg7 = nb_sparse_solve_CG_precond_Jacobi(K, F, u7, 7, 1e-8, &n7, &t7, 1);
	dump("u_it7", DT_F64, u7, N);
	dump_u32("cg7_niter", n7);
	dump_f64("cg7_tol_reached", t7);
	dump_i32("cg7_status", cg7);

	/* nb_sparse_solve_Gauss_Seidel (gauss_seidel.c:14-58): 40 sweeps from the
	 * SpMV input (tolerance 0 is never met), and up to 2000 sweeps from 0 to
	 * the absolute tolerance 1e-6 */
	{
		double *xg = xalloc(8 * (size_t)N);
		memcpy(xg, xs, 8 * (size_t)N);
		uint32_t gi = 0;
		double ge = 0;
		int gst = nb_sparse_solve_Gauss_Seidel(K, F, xg, 40, 0.0, &gi, &ge, 1);
		dump("gs40_x", DT_F64, xg, N);
		dump_u32("gs40_niter", gi);
		dump_f64("gs40_error", ge);
		dump_i32("gs40_status", gst);
		memset(xg, 0, 8 * (size_t)N);
		gst = nb_sparse_solve_Gauss_Seidel(K, F, xg, 2000, 1e-6, &gi, &ge, 1);
		dump("gs_x", DT_F64, xg, N);
		dump_u32("gs_niter", gi);
		dump_f64("gs_error", ge);
		dump_i32("gs_status", gst);
		free(xg);
	}

	/* pipeline.c:266-278 */
	uint32_t ngp = nb_fem_elem_get_N_gpoints(elem);
	double *strain = xalloc(8 * 3 * (size_t)ngp * p.N_elem);
	pipeline_compute_strain(strain, part, u, elem);
	dump("strain", DT_F64, strain, 3 * (uint64_t)ngp * p.N_elem);

	if (uniform) {
		/* nbots' FEM entry itself (one material) */
		nb_material_t *mat = nb_material_create();
		nb_material_set_elasticity_module(mat, p.E[0]);
		nb_material_set_poisson_module(mat, p.nu);
		nb_material_set_density(mat, p.density);
		double grav[2] = {p.gravity[0], p.gravity[1]};
		double *fu = xalloc(8 * (size_t)N);
		double *fs = xalloc(8 * 3 * (size_t)ngp * p.N_elem);
		int fst = nb_fem_compute_2D_Solid_Mechanics(part, elem, mat, bcond,
				p.self_weight != 0, grav, NB_PLANE_STRESS,
				&params2D, p.enabled, fu, fs);
		dump_i32("fem_status", fst);
		dump("fem_u", DT_F64, fu, N);
		dump("fem_strain", DT_F64, fs, 3 * (uint64_t)ngp * p.N_elem);
		double *stress = xalloc(8 * 3 * (size_t)ngp * p.N_elem);
		nb_fem_compute_stress_from_strain(p.N_elem, elem, mat, NB_PLANE_STRESS,
						  fs, p.enabled, stress);
		dump("fem_stress", DT_F64, stress, 3 * (uint64_t)ngp * p.N_elem);
		/* pipeline.c:321-340 */
		double *mstress = xalloc(8 * 2 * (size_t)ngp * p.N_elem);
		pipeline_compute_main_stress(stress, mstress, p.N_elem, elem);
		dump("fem_main_stress", DT_F64, mstress, 2 * (uint64_t)ngp * p.N_elem);
		nb_material_destroy(mat);
	}
	fclose(g_out);
	return 0;
}

/* ------------------------------------------------------------ utest mode */
static double pwh_stress(double x, double y, int c)
{
	/* Kirsch field of the plate-with-hole test (a = 0.5, tx = 1e4) */
	double a = 0.5, tx = 1e4;
	double r = sqrt(x * x + y * y);
	double th = atan2(y, x);
	double ar2 = (a / r) * (a / r);
	double ar4 = 1.5 * ar2 * ar2;
	double s[3];
	s[0] = tx * (1.0 - ar2 * (1.5 * cos(2 * th) + cos(4 * th)) + ar4 * cos(4 * th));
	s[1] = tx * (-ar2 * (0.5 * cos(2 * th) - cos(4 * th)) - ar4 * cos(4 * th));
	s[2] = tx * (-ar2 * (0.5 * sin(2 * th) + sin(4 * th)) + ar4 * sin(4 * th));
	return s[c];
}
static void pwh_dc(const double *x, double t, double *o) { (void)t; o[0] = pwh_stress(x[0], x[1], 0); o[1] = pwh_stress(x[0], x[1], 2); }
static void pwh_bc(const double *x, double t, double *o) { (void)t; o[0] = pwh_stress(x[0], x[1], 2); o[1] = pwh_stress(x[0], x[1], 1); }

static int run_utest(const char *txt, uint32_t nvtx, const char *mesh_out,
		     const char *out, int pwh)
{
	nb_model_t *model = xalloc(nb_model_get_memsize());
	nb_model_init(model);
	nb_bcond_t *bcond = xalloc(nb_bcond_get_memsize(2));
	nb_bcond_init(bcond, 2);
	nb_material_t *mat = nb_material_create();

	nb_cfreader_t *cfr = nb_cfreader_create();
	nb_cfreader_add_line_comment_token(cfr, "#");
	if (nb_cfreader_open_file(cfr, txt)) { fprintf(stderr, "open %s\n", txt); return 2; }
	uint32_t n;
	nb_cfreader_read_uint(cfr, &n);
	model->N = n;
	model->vertex = malloc(16 * (size_t)n);
	for (uint32_t i = 0; i < 2 * n; i++)
		nb_cfreader_read_double(cfr, &model->vertex[i]);
	nb_cfreader_read_uint(cfr, &n);
	model->M = n;
	model->edge = malloc(8 * (size_t)n);
	for (uint32_t i = 0; i < 2 * n; i++)
		nb_cfreader_read_uint(cfr, &model->edge[i]);
	nb_cfreader_read_uint(cfr, &n);
	model->H = n;
	model->holes = NULL;
	if (n) {
		model->holes = malloc(16 * (size_t)n);
		for (uint32_t i = 0; i < 2 * n; i++)
			nb_cfreader_read_double(cfr, &model->holes[i]);
	}
	if (nb_bcond_read(bcond, cfr)) { fprintf(stderr, "bcond\n"); return 2; }
	double v;
	nb_cfreader_read_double(cfr, &v);
	nb_material_set_poisson_module(mat, v);
	nb_cfreader_read_double(cfr, &v);
	nb_material_set_elasticity_module(mat, v);
	nb_cfreader_read_double(cfr, &v);
	nb_material_set_fracture_energy(mat, v);
	nb_cfreader_read_double(cfr, &v);
	nb_material_set_compression_limit_stress(mat, v);
	nb_cfreader_read_double(cfr, &v);
	nb_material_set_traction_limit_stress(mat, v);
	uint32_t an;
	nb_cfreader_read_uint(cfr, &an);
	nb_analysis2D_params params2D = {0.0, 0.0, 0};
	nb_cfreader_read_double(cfr, &params2D.thickness);
	nb_cfreader_close_file(cfr);
	nb_cfreader_destroy(cfr);

	bool m2[2] = {1, 1};
	if (pwh) {
		nb_bcond_push_function(bcond, NB_NEUMANN, NB_BC_ON_SEGMENT, 11, m2, pwh_dc);
		nb_bcond_push_function(bcond, NB_NEUMANN, NB_BC_ON_SEGMENT, 12, m2, pwh_bc);
	}

	nb_mesh2D_t *part = xalloc(nb_mesh2D_get_memsize(NB_TRIAN));
	nb_mesh2D_init(part, NB_TRIAN);
	nb_tessellator2D_t *t2d = xalloc(nb_tessellator2D_get_memsize());
	nb_tessellator2D_init(t2d);
	nb_tessellator2D_set_size_constraint(t2d, NB_MESH_SIZE_CONSTRAINT_MAX_VTX, nvtx);
	nb_tessellator2D_set_geometric_constraint(t2d, NB_MESH_GEOM_CONSTRAINT_MAX_EDGE_LENGTH,
						  NB_GEOMETRIC_TOL);
	nb_tessellator2D_generate_from_model(t2d, model);
	nb_mesh2D_load_from_tessellator2D(part, t2d);
	nb_tessellator2D_finish(t2d);

	nb_fem_elem_t *elem = nb_fem_elem_create(NB_TRG_LINEAR);
	uint32_t Nn = nb_mesh2D_get_N_nodes(part);
	uint32_t Ne = nb_mesh2D_get_N_elems(part);
	double *disp = xalloc(16 * (size_t)Nn);
	double *strain = xalloc(24 * (size_t)Ne);
	double *stress = xalloc(24 * (size_t)Ne);
	int st = nb_fem_compute_2D_Solid_Mechanics(part, elem, mat, bcond, false, NULL,
						   (nb_analysis2D_t)an, &params2D, NULL,
						   disp, strain);
	nb_fem_compute_stress_from_strain(Ne, elem, mat, (nb_analysis2D_t)an, strain,
					  NULL, stress);

	/* the generated mesh, written as a problem file (same layout as read_problem) */
	FILE *f = fopen(mesh_out, "wb");
	uint32_t u32;
	fwrite("NBGP", 1, 4, f);
	u32 = 3; fwrite(&u32, 4, 1, f);
	fwrite(&Nn, 4, 1, f);
	for (uint32_t i = 0; i < Nn; i++) {
		double xy[2] = {nb_mesh2D_node_get_x(part, i), nb_mesh2D_node_get_y(part, i)};
		fwrite(xy, 8, 2, f);
	}
	fwrite(&Ne, 4, 1, f);
	for (uint32_t e = 0; e < Ne; e++)
		for (int k = 0; k < 3; k++) {
			u32 = nb_mesh2D_elem_get_adj(part, e, k);
			fwrite(&u32, 4, 1, f);
		}
	uint32_t Ned = nb_mesh2D_get_N_edges(part);
	fwrite(&Ned, 4, 1, f);
	for (uint32_t e = 0; e < Ned; e++) {
		uint32_t ab[2] = {nb_mesh2D_edge_get_1n(part, e), nb_mesh2D_edge_get_2n(part, e)};
		fwrite(ab, 4, 2, f);
	}
	uint32_t Nv = nb_mesh2D_get_N_invtx(part);
	fwrite(&Nv, 4, 1, f);
	for (uint32_t i = 0; i < Nv; i++) {
		u32 = nb_mesh2D_get_invtx(part, i);
		fwrite(&u32, 4, 1, f);
	}
	uint32_t Ns = nb_mesh2D_get_N_insgm(part);
	fwrite(&Ns, 4, 1, f);
	for (uint32_t s = 0; s < Ns; s++) {
		uint32_t k = nb_mesh2D_insgm_get_N_nodes(part, s);
		fwrite(&k, 4, 1, f);
		for (uint32_t i = 0; i < k; i++) {
			u32 = nb_mesh2D_insgm_get_node(part, s, i);
			fwrite(&u32, 4, 1, f);
		}
	}
	double E = nb_material_get_elasticity_module(mat);
	for (uint32_t e = 0; e < Ne; e++)
		fwrite(&E, 8, 1, f);
	double nu = nb_material_get_poisson_module(mat);
	double dens = nb_material_get_density(mat);
	double grav[2] = {0, 0};
	fwrite(&nu, 8, 1, f);
	fwrite(&params2D.thickness, 8, 1, f);
	fwrite(&dens, 8, 1, f);
	u32 = 0; fwrite(&u32, 4, 1, f);
	fwrite(grav, 8, 2, f);
	u32 = 0; fwrite(&u32, 4, 1, f);
	/* bc atoms in the order nbots applies them is not needed: write them in
	 * push order per container, containers in file order */
	uint16_t isz = nb_bcond_iter_get_memsize();
	nb_bcond_iter_t *it = xalloc(isz);
	uint32_t nbc = 0;
	for (int pass = 0; pass < 2; pass++) {
		static const int kinds[4][2] = {{NB_DIRICHLET, NB_BC_ON_POINT},
			{NB_NEUMANN, NB_BC_ON_POINT}, {NB_DIRICHLET, NB_BC_ON_SEGMENT},
			{NB_NEUMANN, NB_BC_ON_SEGMENT}};
		if (pass == 1)
			fwrite(&nbc, 4, 1, f);
		for (int c = 0; c < 4; c++) {
			nb_bcond_iter_init(it);
			nb_bcond_iter_set_conditions(it, bcond, kinds[c][0], kinds[c][1]);
			while (nb_bcond_iter_has_more(it)) {
				nb_bcond_iter_go_next(it);
				if (pass == 0) { nbc++; continue; }
				uint32_t hdr[3] = {kinds[c][0] == NB_DIRICHLET ? 0u : 1u,
						   kinds[c][1] == NB_BC_ON_POINT ? 0u : 1u,
						   nb_bcond_iter_get_id(it)};
				fwrite(hdr, 4, 3, f);
				uint8_t m[2] = {nb_bcond_iter_get_mask(it, 0), nb_bcond_iter_get_mask(it, 1)};
				fwrite(m, 1, 2, f);
				double val[2] = {0, 0}, x0[2] = {0, 0};
				uint32_t nnv = 0;
				if (!nb_bcond_iter_val_is_function(it)) {
					nb_bcond_iter_get_val(it, 2, x0, 0, val);
					fwrite(val, 8, 2, f);
					fwrite(&nnv, 4, 1, f);
				} else {
					fwrite(val, 8, 2, f);
					uint32_t id = nb_bcond_iter_get_id(it);
					nnv = kinds[c][1] == NB_BC_ON_POINT ? 1 :
						nb_mesh2D_insgm_get_N_nodes(part, id);
					fwrite(&nnv, 4, 1, f);
					for (uint32_t i = 0; i < nnv; i++) {
						uint32_t nid = kinds[c][1] == NB_BC_ON_POINT ?
							nb_mesh2D_get_invtx(part, id) :
							nb_mesh2D_insgm_get_node(part, id, i);
						double xy[2] = {nb_mesh2D_node_get_x(part, nid),
								nb_mesh2D_node_get_y(part, nid)};
						if (kinds[c][0] == NB_NEUMANN && kinds[c][1] == NB_BC_ON_POINT)
							xy[0] = xy[1] = 0.0;
						double o[2];
						nb_bcond_iter_get_val(it, 2, xy, 0, o);
						fwrite(o, 8, 2, f);
					}
				}
			}
			nb_bcond_iter_finish(it);
		}
	}
	fclose(f);

	g_out = fopen(out, "wb");
	dump_i32("fem_status", st);
	dump("fem_u", DT_F64, disp, 2 * (uint64_t)Nn);
	dump("fem_strain", DT_F64, strain, 3 * (uint64_t)Ne);
	dump("fem_stress", DT_F64, stress, 3 * (uint64_t)Ne);
	{	/* pipeline.c:321-340 (T3: one Gauss point) */
		double *mstress = xalloc(16 * (size_t)Ne);
		pipeline_compute_main_stress(stress, mstress, Ne, elem);
		dump("fem_main_stress", DT_F64, mstress, 2 * (uint64_t)Ne);
	}
	double maxd = 0;
	for (uint32_t i = 0; i < Nn; i++) {
		double d2 = disp[2 * i] * disp[2 * i] + disp[2 * i + 1] * disp[2 * i + 1];
		if (d2 > maxd)
			maxd = d2;
	}
	dump_f64("max_disp", sqrt(maxd));
	fclose(g_out);
	return 0;
}

/* nbots' own nonlinear (damage) solve on a problem file
 * (static_damage2D.c:239-470); its only output is the log, dumped as bytes.
 * Material: E[0], nu of the problem, traction limit ft, fracture energy gf. */
static int run_damage(const char *in, const char *out, double ft, double gf,
		      uint32_t n_steps, uint32_t max_iter, uint32_t max_iter_noenh, double rtol)
{
	problem_t p;
	read_problem(in, &p);
	nb_mesh2D_t *part = xalloc(nb_mesh2D_get_memsize(p.nen == 4 ? NB_QUAD : NB_TRIAN));
	void *msh;
	build_mesh(&p, part, &msh);
	nb_fem_elem_t *elem = nb_fem_elem_create(p.nen == 4 ? NB_QUAD_LINEAR : NB_TRG_LINEAR);
	nb_bcond_t *bcond = xalloc(nb_bcond_get_memsize(2));
	nb_bcond_init(bcond, 2);
	build_bcond(&p, bcond);
	nb_analysis2D_params params2D = {p.thickness, 0.0, 0};
	nb_material_t *mat = nb_material_create();
	nb_material_set_elasticity_module(mat, p.E[0]);
	nb_material_set_poisson_module(mat, p.nu);
	nb_material_set_density(mat, p.density);
	nb_material_set_traction_limit_stress(mat, ft);
	nb_material_set_fracture_energy(mat, gf);
	nb_fem_implicit_t *ip = nb_fem_implicit_create();
	nb_fem_implicit_set_N_steps(ip, n_steps);
	nb_fem_implicit_set_N_max_iter(ip, max_iter);
	nb_fem_implicit_set_N_max_iter_without_enhance(ip, max_iter_noenh);
	nb_fem_implicit_set_residual_tolerance(ip, rtol);
	char logpath[4096];
	snprintf(logpath, sizeof(logpath), "%s.log", out);
	remove(logpath);
	double grav[2] = {p.gravity[0], p.gravity[1]};
	nb_fem_compute_2D_Non_Linear_Solid_Mechanics(part, elem, mat, bcond, p.self_weight != 0,
						     grav, false, NB_PLANE_STRESS, &params2D, ip,
						     logpath);
	FILE *lf = fopen(logpath, "rb");
	if (!lf) { perror(logpath); return 2; }
	fseek(lf, 0, SEEK_END);
	long n = ftell(lf);
	fseek(lf, 0, SEEK_SET);
	char *txt = xalloc((size_t)n + 1);
	if (fread(txt, 1, (size_t)n, lf) != (size_t)n) { fprintf(stderr, "short log\n"); return 2; }
	fclose(lf);
	g_out = fopen(out, "wb");
	if (!g_out) { perror(out); return 2; }
	dump("damage_log", DT_U8, txt, (uint64_t)n);
	fclose(g_out);
	nb_fem_implicit_destroy(ip);
	nb_material_destroy(mat);
	return 0;
}

int main(int argc, char **argv)
{
	if (argc >= 10 && !strcmp(argv[1], "damage"))
		return run_damage(argv[2], argv[3], atof(argv[4]), atof(argv[5]),
				  (uint32_t)atoi(argv[6]), (uint32_t)atoi(argv[7]),
				  (uint32_t)atoi(argv[8]), atof(argv[9]));
	if (argc >= 4 && !strcmp(argv[1], "problem"))
		return run_problem(argv[2], argv[3], argc > 4 ? (uint32_t)atoi(argv[4]) : 1);
	if (argc >= 6 && !strcmp(argv[1], "utest"))
		return run_utest(argv[2], (uint32_t)atoi(argv[3]), argv[4], argv[5],
				 argc > 6 && !strcmp(argv[6], "pwh"));
	fprintf(stderr, "usage: ref_harness problem <in> <out> [threads] | "
		"utest <txt> <nvtx> <mesh_out> <out> [pwh]\n");
	return 1;
}
