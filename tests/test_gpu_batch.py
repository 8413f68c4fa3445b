"""Batched SIMP solves (nbg_batch_*, nbg_mixed_batch_*) on the GPU.

A batch merges independent cantilevers of uneven size (node counts that are
not multiples of 32, so every instance is padded) into one block-diagonal
system.  Checks: each instance's assembled K and F equal the single-system
ones bit for bit and the padding rows are identity rows with zero load; one
graph launch solves every instance to its own relative tolerance with the
displacements within 1e-8 relative L2 of an FP64 solve converged to 1e-13;
compliance and sensitivities agree with the oracle on that FP64 solution;
replays are bit-identical; the block shares and the tuner behave."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
SIZES = ((8, 4), (12, 6), (16, 8), (20, 10))


@pytest.fixture(scope="module")
def L():
    from nbots_gb300 import _lib
    assert _lib.lib().nbg_device_count() > 0
    return _lib


@pytest.fixture(scope="module")
def batch(L):
    from nbots_gb300 import workloads as W
    from nbots_gb300.batch import Batch
    probs = W.config_c5(n_inst=7, seed=21, sizes=SIZES)
    b = Batch(probs)
    rho = [p.meta["rho"] for p in probs]
    b.assemble_simp(rho, nu=probs[0].nu, thickness=probs[0].thickness)
    b.setup(max_iter=20000, tol=1e-10)
    yield b, probs, rho
    b.close()


def converged_fp64(r):
    """An FP64 reference solve: relres 1e-13, or stopped at the system's FP64
    floor (status 1 with a true residual below 1e-10 ||F||, a hundred
    times below the tolerances compared against it)."""
    return r.status == 0 or (r.status == 1 and r.tol_reached <= 1e-10 * r.bnorm)


def single(L, p, E):
    from nbots_gb300.fem import FemSystem
    p.E = E
    s = FemSystem(p)
    assert s.assemble() == 0
    s.apply_bcs()
    return s


def test_merged_assembly_bit_exact(L, batch):
    b, probs, _ = batch
    rp, ci, K, F = (b.merged(w) for w in (L.FEM_ROW_PTR, L.FEM_COL_IDX, L.FEM_K, L.FEM_F))
    E = b.merged(L.FEM_E)
    for k, p in enumerate(probs):
        no, n1 = 2 * int(b.node_off[k]), 2 * int(b.node_off[k + 1])
        e0, e1 = int(b.elem_off[k]), int(b.elem_off[k + 1])
        s = single(L, p, E[e0:e1].copy())
        srp, sci = s.get(L.FEM_ROW_PTR), s.get(L.FEM_COL_IDX)
        r0, r1 = no, no + p.n_dof
        assert np.array_equal(rp[r0:r1 + 1] - rp[r0], srp)
        seg = slice(int(rp[r0]), int(rp[r1]))
        assert np.array_equal(ci[seg] - no, sci)
        assert np.array_equal(K[seg].view(np.uint64), s.get(L.FEM_K).view(np.uint64))
        assert np.array_equal(F[r0:r1].view(np.uint64), s.get(L.FEM_F).view(np.uint64))
        # padding rows: the node's own 2x2 block, identity, zero load
        for r in range(r1, n1):
            cols = ci[rp[r]:rp[r + 1]]
            vals = K[rp[r]:rp[r + 1]]
            assert len(cols) == 2 and list(cols) == [r & ~1, r | 1]
            assert vals[cols == r][0] == 1.0 and vals[cols != r][0] == 0.0
            assert F[r] == 0.0
        s.close()


def test_batched_solve_matches_fp64(L, batch):
    b, probs, rho = batch
    b.launch()
    res, J = b.results()
    us = b.displacements()
    dJs = b.sensitivities()
    E = b.merged(L.FEM_E)
    for k, p in enumerate(probs):
        assert res[k].status == 0 and res[k].relres <= 1e-10, k
        s = single(L, p, E[int(b.elem_off[k]):int(b.elem_off[k + 1])].copy())
        r64 = s.solve_fast(tol=1e-13)
        assert converged_fp64(r64), (r64.status, r64.niter, r64.tol_reached / r64.bnorm)
        u64 = s.get(L.FEM_U)
        F = s.get(L.FEM_F)
        err = np.linalg.norm(us[k] - u64) / np.linalg.norm(u64)
        assert err < 1e-8, (k, err)
        assert abs(J[k] - float(F @ u64)) <= 1e-9 * abs(J[k])
        ref = O.simp_sensitivity(O.Flat(p), rho[k], u64, u64)
        assert np.max(np.abs(dJs[k] - ref)) <= 1e-7 * np.max(np.abs(ref)), k
        s.close()


def test_graph_replay_is_bit_identical(L, batch):
    b, probs, _ = batch
    b.launch()
    _, J1 = b.results()
    u1 = b.merged(L.FEM_U)
    d1 = np.concatenate(b.sensitivities())
    b.launch()
    _, J2 = b.results()
    assert np.array_equal(u1.view(np.uint64), b.merged(L.FEM_U).view(np.uint64))
    assert np.array_equal(d1.view(np.uint64), np.concatenate(b.sensitivities()).view(np.uint64))
    assert np.array_equal(J1, J2)


def test_block_shares_and_tuner(L, batch):
    b, probs, _ = batch
    for gamma in (0.0, 1.0, 2.0):
        b.plan(gamma)
        G, blocks, g = b.blocks()
        assert g == gamma and G == int(blocks.sum()) and blocks.min() >= 1
        slices = np.diff(b.node_off.astype(np.int64)) // 32
        # never more blocks than warps of slices
        assert np.all(blocks <= np.maximum(1, (slices + 15) // 16))
    ms = b.tune((0.5, 1.0, 1.5))
    assert np.all(ms > 0)
    _, _, g = b.blocks()
    assert g in (0.5, 1.0, 1.5)
    b.launch()
    res, _ = b.results()
    assert all(r.status == 0 for r in res)


def test_not_converged_is_reported(L, batch):
    b, probs, _ = batch
    b.setup(max_iter=3, tol=1e-12)
    b.launch()
    res, _ = b.results()
    assert all(r.status == 1 and r.niter == 3 for r in res)
    b.setup(max_iter=20000, tol=1e-10)


def test_t3_batch(L):
    """Unstructured T3 instances (L-shapes of three sizes, uneven row
    lengths, padded slices): merged assembly bit for bit with each single
    system, and the batched solve within 1e-8 of FP64 solves."""
    from nbots_gb300 import workloads as W
    from nbots_gb300.batch import Batch
    probs = [W.t3_lshape(n, seed=30 + n) for n in (1500, 2500, 4000)]
    rng = np.random.default_rng(8)
    rho = [rng.uniform(0.3, 0.9, p.n_elems) for p in probs]
    b = Batch(probs)
    b.assemble_simp(rho, nu=probs[0].nu, thickness=probs[0].thickness)
    b.setup(max_iter=40000, tol=1e-10)
    rp, ci, K = (b.merged(w) for w in (L.FEM_ROW_PTR, L.FEM_COL_IDX, L.FEM_K))
    E = b.merged(L.FEM_E)
    b.launch()
    res, J = b.results()
    us = b.displacements()
    for k, p in enumerate(probs):
        no = 2 * int(b.node_off[k])
        e0, e1 = int(b.elem_off[k]), int(b.elem_off[k + 1])
        s = single(L, p, E[e0:e1].copy())
        r0, r1 = no, no + p.n_dof
        seg = slice(int(rp[r0]), int(rp[r1]))
        assert np.array_equal(ci[seg] - no, s.get(L.FEM_COL_IDX))
        assert np.array_equal(K[seg].view(np.uint64), s.get(L.FEM_K).view(np.uint64))
        assert res[k].status == 0 and res[k].relres <= 1e-10, k
        r64 = s.solve_fast(tol=1e-13)
        assert converged_fp64(r64), (r64.status, r64.niter, r64.tol_reached / r64.bnorm)
        u64 = s.get(L.FEM_U)
        assert np.linalg.norm(us[k] - u64) / np.linalg.norm(u64) < 1e-8, k
        s.close()
    b.close()
