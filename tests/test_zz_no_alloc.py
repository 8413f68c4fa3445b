"""The allocation-free CG entry point (nbg_cg_f64_noalloc).

Some callers cannot allocate device memory while they solve, for instance an
application that keeps the GPU's memory in its own pool and forbids
libraries to call cudaMalloc.  This entry point keeps its scratch in a
static device array instead.  Here it is called twice in a row through the
C ABI, on two different systems, and each result is compared with the
allocating entry point's on the same inputs (u within 1e-10 relative L2,
the tolerance of the other CG parity tests; the same iteration count and
status).  The device's free memory (cudaMemGetInfo) is the same before and
after each call once the library's kernels are loaded: the calls allocate
nothing.  A system larger than the array is refused with an error.

The file sorts last so that a run stopping at the first failure has run
every other test before it; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def free_device_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_cg_matches_allocating_entry_on_two_calls():
    from nbots_gb300 import _lib as L
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    assert lib.nbg_device_count() > 0
    free_device_bytes()  # the harness's own CUDA state, before any measurement
    for name in ("c1_q4_64x32", "q4_allbc_16x8"):
        _, d = load_golden(name)
        N = d["F_bc"].shape[0]
        rp, ci = DeviceArray(d["row_ptr"]), DeviceArray(d["col_idx"])
        K, F = DeviceArray(d["K_bc"]), DeviceArray(d["F_bc"])
        x_ref = DeviceArray(np.zeros(N))
        x_na = DeviceArray(np.full(N, 0.0))
        r_ref, r_na = L.CgResult(), L.CgResult()
        rc_ref = lib.nbg_cg_f64(N, rp.ptr, ci.ptr, K.ptr, F.ptr, x_ref.ptr, N, 1e-8,
                                L.CG_JACOBI, C.byref(r_ref), None, 0, None)
        free0 = free_device_bytes()
        rc_na = lib.nbg_cg_f64_noalloc(N, rp.ptr, ci.ptr, K.ptr, F.ptr, x_na.ptr, N, 1e-8,
                                       L.CG_JACOBI, C.byref(r_na), None)
        assert free_device_bytes() == free0
        assert rc_ref == rc_na == 0
        assert (r_na.niter, r_na.status) == (r_ref.niter, r_ref.status)
        u_ref, u_na = x_ref.numpy(), x_na.numpy()
        assert rel(u_na, u_ref) < 1e-10
        assert rel(u_na, d["u"]) < 1e-10


def test_noalloc_cg_rejects_systems_beyond_its_scratch():
    from nbots_gb300 import _lib as L
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    N = 400_000                                   # needs more than the 16 MiB array
    rp = DeviceArray(np.arange(N + 1, dtype=np.uint32))
    ci = DeviceArray(np.arange(N, dtype=np.uint32))
    v, b, x = DeviceArray(np.ones(N)), DeviceArray(np.ones(N)), DeviceArray(np.zeros(N))
    r = L.CgResult()
    rc = lib.nbg_cg_f64_noalloc(N, rp.ptr, ci.ptr, v.ptr, b.ptr, x.ptr, 10, 1e-8,
                                L.CG_JACOBI, C.byref(r), None)
    assert rc == -3
    assert b"345408" in lib.nbg_last_error()
