"""The block-layout SpMVs on the GPU against the oracle's FP64 SpMV of the
same matrix (nbots' K after boundary conditions) and vector.

Bars, relative to max|y|: FP64 block SpMV 1e-14 (FMA order differs from
nbots'); FP32 values and vector 1e-6; the mixed solver's operator (FP32 +
16-bit remainder matrix, about 40 bits, times a float-float vector,
error-free sums) 1e-10.  The cases include systems whose node count is not a
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


def setup(L, name, seed=0):
    from nbots_gb300.fem import FemSystem
    p, d = load_golden(name)
    s = FemSystem(p)
    assert s.assemble() == 0
    s.apply_bcs()
    A = s.block_layout()
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(s.N)
    y_ref = O.spmv(d["row_ptr"], d["col_idx"], d["K_bc"], x)
    return s, A, x, y_ref


def err(y, ref):
    return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("name", CASES)
def test_fp64_and_fp32_block_spmv(L, name):
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    s, A, x, y_ref = setup(L, name)
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
    s, A, x, y_ref = setup(L, name, seed=1)
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
    assert err(y, y_ff) < 1e-10
    s.close()
