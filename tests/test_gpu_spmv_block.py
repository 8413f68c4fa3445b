"""The block-layout SpMVs on the GPU against the oracle's FP64 SpMV of the
same matrix (nbots' K after boundary conditions) and vector.

Bars, relative to max|y|: FP64 block SpMV 1e-14 (FMA order differs from
nbots'); FP32 values and vector 1e-6; the mixed solver's operator (FP32 +
23-bit remainder matrix, about 47 bits, times a float-float vector,
error-free sums) 1e-12.  The cases include systems whose node count is not a
multiple of the 32-row slice."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CASES = ["c1_q4_64x32", "q4_allbc_16x8", "t3_beam_cantilever"]


@pytest.fixture(scope="module")
def L():
    from nbots_gb300 import _lib
    assert _lib.lib().nbg_device_count() > 0
    return _lib


def setup(L, name, seed=0, order=0):
    from nbots_gb300.fem import FemSystem
    p, d = load_golden(name)
    s = FemSystem(p)
    s.set_block_order(order)
    assert s.assemble() == 0
    s.apply_bcs()
    A = s.block_layout()
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(s.N)
    y_ref = O.spmv(d["row_ptr"], d["col_idx"], d["K_bc"], x)
    return s, A, x, y_ref


def err(y, ref):
    return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("order", [1, 2])  # mesh order, SELL-C-sigma order
@pytest.mark.parametrize("name", CASES)
def test_fp64_and_fp32_block_spmv(L, name, order):
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    s, A, x, y_ref = setup(L, name, order=order)
    assert bool(A.perm) == (order == 2)
    dx, dy = DeviceArray(x), DeviceArray(shape=(s.N,), dtype=np.float64)
    assert lib.nbg_spmv_bsr_f64(C.byref(A), dx.ptr, dy.ptr, None) == 0
    assert err(dy.numpy(), y_ref) < 1e-14
    x32 = x.astype(np.float32)
    dx32, dy32 = DeviceArray(x32), DeviceArray(shape=(s.N,), dtype=np.float32)
    assert lib.nbg_spmv_bsr_f32(C.byref(A), dx32.ptr, dy32.ptr, None) == 0
    assert err(dy32.numpy().astype(np.float64), y_ref) < 1e-6
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_mixed_operator(L, name):
    """nbg_spmv_bsr_mixed: the mixed solver's operator with FP32 low parts."""
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    s, A, x, y_ref = setup(L, name, seed=1, order=1)  # the operator alone: mesh order
    xh = x.astype(np.float32)
    xl = (x - xh.astype(np.float64)).astype(np.float32)
    # reference on the exact float-float vector
    d = load_golden(name)[1]
    xff = xh.astype(np.float64) + xl.astype(np.float64)
    y_ff = O.spmv(d["row_ptr"], d["col_idx"], d["K_bc"], xff)
    dxh, dxl = DeviceArray(xh), DeviceArray(xl)
    dwh = DeviceArray(shape=(s.N,), dtype=np.float32)
    dwl = DeviceArray(shape=(s.N,), dtype=np.float32)
    assert lib.nbg_spmv_bsr_mixed(C.byref(A), dxh.ptr, dxl.ptr, dwh.ptr, dwl.ptr, None) == 0
    y = dwh.numpy().astype(np.float64) + dwl.numpy().astype(np.float64)
    assert err(y, y_ff) < 1e-12
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_solvers_in_sigma_order(L, name):
    """The fast FP64 and mixed solvers on a layout in SELL-C-sigma order take
    and return vectors in mesh order: their solutions match the oracle's."""
    from nbots_gb300.fem import FemSystem
    p, d = load_golden(name)
    s = FemSystem(p)
    s.set_block_order(2)
    assert s.assemble() == 0
    s.apply_bcs()
    rp, ci, K, F = d["row_ptr"], d["col_idx"], d["K_bc"], d["F_bc"]
    tight, *_ = O.cg_jacobi(rp, ci, K, F, max_iter=40 * F.shape[0],
                            tol=1e-13 * np.linalg.norm(F))
    for solve, tol in ((s.solve_fast, 1e-9), (s.solve_mixed, 1e-10)):
        assert solve(tol=tol).status == 0
        u = s.get(L.FEM_U)
        rr = np.linalg.norm(F - O.spmv(rp, ci, K, u)) / np.linalg.norm(F)
        assert rr <= 2 * tol
        assert np.linalg.norm(u - tight) / np.linalg.norm(tight) < 1e-6
    # the operator alone serves layouts in mesh order only
    from nbots_gb300.device import DeviceArray
    A = s.block_layout()
    v = [DeviceArray(shape=(s.N,), dtype=np.float32) for _ in range(4)]
    assert L.lib().nbg_spmv_bsr_mixed(C.byref(A), *[a.ptr for a in v], None) == -3
    s.close()
