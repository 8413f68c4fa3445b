/*
 * The device-resident FEM system shared by fem.c (elastic path) and
 * damage.c (quasi-static damage path).  Private to the host library.
 */
#ifndef NBG_FEM_INTERNAL_H
#define NBG_FEM_INTERNAL_H

#include "nbots_gb300.h"

struct nbg_fem {
	nbg_mesh_t m;
	uint32_t N;        /* dofs */
	uint64_t nnz;
	void *stream;
	/* device arrays */
	double *nod, *K, *F, *u, *strain, *stress, *E, *Ke, *Fe, *main_stress;
	double *damage;    /* per Gauss point, owned by the damage solve */
	uint32_t *conn, *row_ptr, *col_idx, *inc_ptr, *inc_elem, *distorted;
	uint8_t *inc_local, *enabled;
	unsigned long long *matched;
	int *status;
	double nu;
	int has_enabled;
	void *cg_ws;
	size_t cg_ws_bytes;
	/* 2x2-block SELL copy (bsr.cu), filled from K on demand */
	int bsr_ok;
	nbg_bsr_t bsr;
	uint32_t *slice_off, *bcol;
	double *b64, *dinv64;
	float *b32, *dinv32;
	uint16_t *blo;
	uint8_t *bxt;
	int block_order;           /* NBG_ORDER_* */
	uint32_t block_sigma;      /* SELL-C-sigma window, 0: default */
	uint32_t *perm, *iperm;    /* the block layout's node order, or NULL */
	double *simp_rho, *simp_out, *simp_e, *simp_lam;  /* nbg_fem_simp buffers */
	int borrowed_csr;          /* row_ptr, col_idx and K belong to the caller */
};

/* A FEM system on a CSR the caller owns on the device (row_ptr[N + 1],
 * col_idx, values K; not freed by nbg_fem_destroy), N = 2 N_nod: the mesh
 * arrays, F, u, strain and stress, and with need_incidence the node ->
 * element incidence that assembly needs.  No block layout.  The gather
 * assembly writes every pattern entry (those no element reaches get 0) and
 * reports a missing element pair as NBG_ERR_PATTERN. */
int nbg_fem_create_on_csr(nbg_fem_t **out, const nbg_mesh_t *m, uint64_t nnz,
			  uint32_t *row_ptr, uint32_t *col_idx, double *K, int need_incidence,
			  void *stream);

/* Assembly with an optional device array of damage per Gauss point; E NULL
 * means the moduli are already in f->E. */
int nbg_fem_assemble_dev_damage(nbg_fem_t *f, const double *E, double nu, double thickness,
				double density, int self_weight, const double gravity[2],
				const uint8_t *enabled, const double *damage);
/* Grow f's CG workspace to what nbg_cg_f64 needs for f->N dofs. */
int nbg_fem_cg_workspace(nbg_fem_t *f);

#endif
