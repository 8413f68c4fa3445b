/*
 * A C99 program against the two public headers and the two libraries,
 * host calls only (it runs without a GPU): nbots' pattern of a 2x1 Q4 mesh
 * through the C ABI and through the drop-in nb_sparse_create, which must
 * agree, and the forward-substitution levels of that pattern.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nbots_dropin.h"
#include "nbots_gb300.h"

int main(void)
{
	/* 2x1 Q4 grid: nodes 0..5, elements (0 1 4 3), (1 2 5 4) */
	const double nod[12] = {0, 0, 1, 0, 2, 0, 0, 1, 1, 1, 2, 1};
	const uint32_t conn[8] = {0, 1, 4, 3, 1, 2, 5, 4};
	const uint32_t edg[14] = {0, 1, 1, 2, 3, 4, 4, 5, 0, 3, 1, 4, 2, 5};
	const nbg_mesh_t m = {4, 6, 2, 7, nod, conn, edg};
	uint32_t rp[13];
	if (nbg_host_pattern(&m, rp, NULL) != NBG_OK)
		return 1;
	uint32_t *ci = malloc(sizeof(uint32_t) * rp[12]);
	if (!ci || nbg_host_pattern(&m, rp, ci) != NBG_OK)
		return 2;

	/* the same pattern from nbots' graph through the drop-in */
	uint32_t N_adj[6] = {0};
	uint32_t *adj[6];
	for (uint32_t v = 0; v < 6; v++) {
		N_adj[v] = (rp[2 * v + 1] - rp[2 * v]) / 2 - 1;
		adj[v] = malloc(sizeof(uint32_t) * (N_adj[v] ? N_adj[v] : 1));
		uint32_t k = 0;
		for (uint32_t q = rp[2 * v]; q < rp[2 * v + 1]; q += 2)
			if (ci[q] / 2 != v)
				adj[v][k++] = ci[q] / 2;
	}
	nb_graph_t g;
	memset(&g, 0, sizeof(g));
	g.N = 6;
	g.N_adj = N_adj;
	g.adj = adj;
	nb_sparse_t *A = nb_sparse_create(&g, NULL, 2);
	if (!A || nb_sparse_get_size(A) != 12 || nb_sparse_get_nnz(A) != rp[12])
		return 3;
	for (uint32_t i = 0; i < 12; i++)
		for (uint32_t q = rp[i]; q < rp[i + 1]; q++)
			if (!nb_sparse_is_non_zero(A, i, ci[q]))
				return 4;
	nb_sparse_destroy(A);

	uint32_t lp[13], lr[12], nl = 0;
	if (nbg_host_lower_levels(12, rp, ci, lp, lr, &nl) != NBG_OK || lp[nl] != 12)
		return 5;
	printf("ok %s nnz %u levels %u\n", nbg_version(), rp[12], nl);
	for (uint32_t v = 0; v < 6; v++)
		free(adj[v]);
	free(ci);
	return 0;
}
