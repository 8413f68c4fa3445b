"""The unstructured T3 L-shape workload (the 4M-dof benchmark case, here at
small sizes): the generator gives a valid conforming triangulation, and on
the GPU its assembly and boundary conditions equal the oracle's bit for bit
and the fast solvers meet their tolerances."""
import numpy as np
import pytest

from oracle import oracle as O


def lshape(n=6000, seed=3):
    from nbots_gb300 import workloads as W
    return W.t3_lshape(n, seed=seed)


def test_generator_is_a_valid_triangulation():
    p = lshape()
    tri, nod = p.conn.astype(np.int64), p.nod
    # simply connected planar triangulation: V - E + F = 1
    assert p.n_nodes - p.edges.shape[0] + p.n_elems == 1
    a, b, c = nod[tri[:, 0]], nod[tri[:, 1]], nod[tri[:, 2]]
    area2 = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    assert np.all(area2 > 0)                          # counter-clockwise
    assert abs(area2.sum() / 2 - 3.0) < 1e-9          # covers the L exactly
    cen = (a + b + c) / 3
    assert not np.any((cen[:, 0] > 1) & (cen[:, 1] > 1))
    # model vertices at the six corners, segments join them
    assert np.allclose(nod[p.vtx], [[0, 0], [2, 0], [2, 1], [1, 1], [1, 2], [0, 2]])
    for s, seq in enumerate(p.sgm):
        assert seq[0] == p.vtx[s] and seq[-1] == p.vtx[(s + 1) % 6]
    # deterministic for a seed
    q = lshape()
    assert np.array_equal(p.conn, q.conn) and np.array_equal(p.nod, q.nod)


@pytest.mark.gpu
def test_lshape_assembly_and_solvers_on_gpu():
    from nbots_gb300 import _lib as L
    from nbots_gb300.fem import FemSystem
    p = lshape(20000)
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    st, K_ref, F_ref = O.assemble(fl, rp, ci)
    assert st == 0
    r = {"row_ptr": rp, "col_idx": ci, "K_asm": K_ref.copy(), "F_asm": F_ref.copy()}
    O.set_bconditions(fl, rp, ci, K_ref, F_ref)
    r["K_bc"], r["F_bc"] = K_ref, F_ref
    s = FemSystem(p)
    s.set_block_order(L.ORDER_SIGMA)
    assert s.assemble() == 0
    K_asm, F_asm = s.get(L.FEM_K), s.get(L.FEM_F)
    assert np.array_equal(s.get(L.FEM_ROW_PTR), r["row_ptr"])
    assert np.array_equal(s.get(L.FEM_COL_IDX), r["col_idx"])
    assert np.array_equal(K_asm.view(np.uint64), r["K_asm"].view(np.uint64))
    assert np.array_equal(F_asm.view(np.uint64), r["F_asm"].view(np.uint64))
    s.apply_bcs()
    assert np.array_equal(s.get(L.FEM_K).view(np.uint64), r["K_bc"].view(np.uint64))
    assert np.array_equal(s.get(L.FEM_F).view(np.uint64), r["F_bc"].view(np.uint64))
    rp, ci, K, F = r["row_ptr"], r["col_idx"], r["K_bc"], r["F_bc"]
    tight, *_ = O.cg_jacobi(rp, ci, K, F, max_iter=40 * F.shape[0], tol=1e-13 * np.linalg.norm(F))
    # Both fast solvers judge convergence on the true FP64 residual (the FP64
    # CG confirms its recurrence's verdict on b - A u), so both must meet the
    # tolerance on the oracle's SpMV.  They run on a layout in SELL-C-sigma
    # node order and in mesh order (the default); the mesh order stores
    # about 40 % more entries here
    m = FemSystem(p)
    assert m.assemble() == 0
    m.apply_bcs()
    A_sigma, A_mesh = s.block_layout(), m.block_layout()
    assert A_sigma.perm and not A_mesh.perm
    assert A_sigma.n_entries < 0.8 * A_mesh.n_entries
    for sys_ in (s, m):
        # both solvers judge convergence on the true FP64 residual
        for solve, tol, slack, uerr in ((sys_.solve_fast, 1e-10, 1.01, 1e-7),
                                        (sys_.solve_mixed, 1e-11, 1.05, 1e-8)):
            res = solve(tol=tol)
            assert res.status == 0
            u = sys_.get(L.FEM_U)
            rr = np.linalg.norm(F - O.spmv(rp, ci, K, u)) / np.linalg.norm(F)
            assert rr <= slack * tol, (solve.__name__, rr)
            assert np.linalg.norm(u - tight) / np.linalg.norm(tight) < uerr
    m.close()
    s.close()
