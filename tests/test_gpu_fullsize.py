"""Parity at the benchmark's full size: the 1024x512 Q4 cantilever
(1,051,650 dof, lognormal E).  The device pattern equals the host build
word for word; K and F after assembly and boundary conditions and the
nbots-order SpMV equal the oracle's bit for bit; the mixed solve reaches
relres 1e-8 on the true FP64 residual and lands within 1e-8 (relative L2)
of the fast FP64 solution at the same tolerance."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem
    p = W.config_c2()
    s = FemSystem(p)
    yield p, s
    s.close()


def test_full_size_pattern_assembly_bcs_spmv(c2):
    from nbots_gb300 import _lib as L
    from nbots_gb300.device import DeviceArray
    p, s = c2
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    assert np.array_equal(s.get(L.FEM_ROW_PTR), rp)
    assert np.array_equal(s.get(L.FEM_COL_IDX), ci)
    st, K, F = O.assemble(fl, rp, ci)
    assert st == 0 and s.assemble() == 0
    assert np.array_equal(s.get(L.FEM_K).view(np.uint64), K.view(np.uint64))
    assert np.array_equal(s.get(L.FEM_F).view(np.uint64), F.view(np.uint64))
    O.set_bconditions(fl, rp, ci, K, F)
    s.apply_bcs()
    assert np.array_equal(s.get(L.FEM_K).view(np.uint64), K.view(np.uint64))
    assert np.array_equal(s.get(L.FEM_F).view(np.uint64), F.view(np.uint64))
    x = np.random.default_rng(11).standard_normal(s.N)
    dx, dy = DeviceArray(x), DeviceArray(shape=(s.N,), dtype=np.float64)
    L.check(L.lib().nbg_spmv_csr_f64(s.N, s.dptr(L.FEM_ROW_PTR), s.dptr(L.FEM_COL_IDX),
                                     s.dptr(L.FEM_K), dx.ptr, dy.ptr, None), "spmv")
    assert np.array_equal(dy.numpy().view(np.uint64), O.spmv(rp, ci, K, x).view(np.uint64))


def test_full_size_mixed_solve(c2):
    from nbots_gb300 import _lib as L
    from nbots_gb300.device import DeviceArray
    p, s = c2
    if s.assemble() != 0:
        pytest.fail("assembly")
    s.apply_bcs()
    r64 = s.solve_fast(tol=1e-8)  # the benchmark's pairing: both at relres 1e-8
    assert r64.status == 0
    u64 = s.get(L.FEM_U)
    rm = s.solve_mixed(tol=1e-8)
    assert rm.status == 0 and rm.relres <= 1e-8
    um = s.get(L.FEM_U)
    # the true FP64 residual of the mixed solution, through the exact SpMV
    F = s.get(L.FEM_F)
    du, dy = DeviceArray(um), DeviceArray(shape=(s.N,), dtype=np.float64)
    L.check(L.lib().nbg_spmv_csr_f64(s.N, s.dptr(L.FEM_ROW_PTR), s.dptr(L.FEM_COL_IDX),
                                     s.dptr(L.FEM_K), du.ptr, dy.ptr, None), "spmv")
    assert np.linalg.norm(F - dy.numpy()) <= 1.05e-8 * np.linalg.norm(F)
    assert np.linalg.norm(um - u64) <= 1e-8 * np.linalg.norm(u64)
