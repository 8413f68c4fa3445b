"""CUDA path against the reference's own outputs (tests/golden/) and the
oracle.  Integer and FP64 assembly/BC stages are bit-exact; the CG solve
differs from nbots' serial sums only in its reduction order, so the
displacements must agree within 1e-10 relative L2."""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, cg_iters_close, load_golden
from kat import BEAM_MAX_DISP, PWH_MAX_VM_ERR, max_disp, pwh_mean_vm_error

pytestmark = pytest.mark.gpu

U_REL_TOL = 1e-10


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8) if a.dtype == np.float64 else a


def same(a, b):
    return a.shape == b.shape and np.array_equal(bits(a), bits(b))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def lib():
    from nbots_gb300 import _lib as L
    L.lib()
    assert L.lib().nbg_device_count() > 0, "no CUDA device"
    return L


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_fem_stages_vs_reference(lib, name):
    from nbots_gb300.fem import FemSystem
    L = lib
    p, d = load_golden(name)
    s = FemSystem(p)
    assert same(s.get(L.FEM_ROW_PTR), d["row_ptr"])
    assert same(s.get(L.FEM_COL_IDX), d["col_idx"])
    st = s.assemble()
    assert st == int(d["assemble_status"][0])
    if st:
        return
    assert same(s.get(L.FEM_K), d["K_asm"]), "K after assembly"
    assert same(s.get(L.FEM_F), d["F_asm"]), "F after assembly"
    s.apply_bcs()
    assert same(s.get(L.FEM_K), d["K_bc"]), "K after boundary conditions"
    assert same(s.get(L.FEM_F), d["F_bc"]), "F after boundary conditions"
    r = s.solve()
    u = s.get(L.FEM_U)
    assert r.status == int(d["cg_status"][0])
    assert cg_iters_close(r.niter, int(d["cg_niter"][0]), np.linalg.norm(d["F_bc"]))
    assert rel(u, d["u"]) < U_REL_TOL
    # strain of the reference displacements is bit-exact
    s.put(L.FEM_U, d["u"])
    assert same(s.strain(), d["strain"])
    if "fem_stress" in d:
        s.put(L.FEM_U, d["fem_u"])
        s.strain()
        assert same(s.stress(), d["fem_stress"])
        if "fem_main_stress" in d:
            assert same(s.main_stress(), d["fem_main_stress"])
    s.close()


@pytest.mark.parametrize("name", ["c1_q4_64x32", "t3_beam_cantilever", "q4_allbc_16x8"])
def test_spmv_bit_exact(lib, name):
    from nbots_gb300.device import DeviceArray
    p, d = load_golden(name)
    N = d["row_ptr"].shape[0] - 1
    rp, ci, K = DeviceArray(d["row_ptr"]), DeviceArray(d["col_idx"]), DeviceArray(d["K_bc"])
    x = DeviceArray(d["spmv_x"])
    y = DeviceArray(shape=(N,), dtype=np.float64)
    lib.check(lib.lib().nbg_spmv_csr_f64(N, rp.ptr, ci.ptr, K.ptr, x.ptr, y.ptr, None))
    assert same(y.numpy(), d["spmv_y"])


def test_cg_not_converged_path(lib):
    from nbots_gb300.fem import FemSystem
    p, d = load_golden("c1_q4_64x32")
    s = FemSystem(p)
    s.assemble()
    s.apply_bcs()
    r = s.solve(max_iter=7)
    assert (r.status, r.niter) == (1, 7)
    assert rel(s.get(lib.FEM_U), d["u_it7"]) < 1e-12
    assert abs(r.tol_reached - float(d["cg7_tol_reached"][0])) <= 1e-12 * float(d["cg7_tol_reached"][0])


def test_cg_deterministic(lib):
    from nbots_gb300.fem import FemSystem
    p, _ = load_golden("q4_lognormal_32x16")
    s = FemSystem(p)
    s.assemble()
    s.apply_bcs()
    s.solve()
    u1 = s.get(lib.FEM_U)
    s.solve()
    assert same(s.get(lib.FEM_U), u1)


def test_known_answers_on_gpu(lib):
    from nbots_gb300.fem import fem_compute
    p, _ = load_golden("t3_beam_cantilever")
    assert abs(max_disp(fem_compute(p)["u"]) - BEAM_MAX_DISP) < 1e-6
    p, _ = load_golden("t3_plate_with_hole")
    assert pwh_mean_vm_error(p, fem_compute(p)["stress"]) < PWH_MAX_VM_ERR
