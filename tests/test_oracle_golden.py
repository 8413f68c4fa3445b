"""The oracle restatement against the reference's own outputs.

Every fixture in tests/golden/ was produced by the unmodified nbots library
(tests/golden/make_golden.py).  With one thread the oracle follows the same
operation order, so every stage must agree bit for bit.
"""
import numpy as np
import pytest

from conftest import load_golden
from kat import BEAM_MAX_DISP, PWH_MAX_VM_ERR, max_disp, pwh_mean_vm_error
from oracle import oracle as O


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8) if a.dtype == np.float64 else a


def same(a, b):
    return a.shape == b.shape and np.array_equal(bits(a), bits(b))


def test_oracle_stages_bit_exact(golden):
    name, p, d = golden
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    assert same(rp.astype(np.uint32), d["row_ptr"])
    assert same(ci, d["col_idx"])
    st, K, F = O.assemble(fl, rp, ci)
    assert st == int(d["assemble_status"][0])
    if st:
        return
    assert same(K, d["K_asm"]), name
    assert same(F, d["F_asm"]), name
    O.set_bconditions(fl, rp, ci, K, F)
    assert same(K, d["K_bc"]), name
    assert same(F, d["F_bc"]), name
    assert same(O.spmv(rp, ci, K, d["spmv_x"]), d["spmv_y"])
    u, it, tr, cst = O.cg_jacobi(rp, ci, K, F)
    assert it == int(d["cg_niter"][0]) and cst == int(d["cg_status"][0])
    assert same(np.array([tr]), d["cg_tol_reached"])
    assert same(u, d["u"]), name
    # from a non-zero initial guess (the damage loop's case)
    ux, itx, trx, stx = O.cg_jacobi(rp, ci, K, F, x0=d["spmv_x"])
    assert (itx, stx) == (int(d["cgx0_niter"][0]), int(d["cgx0_status"][0]))
    assert same(ux, d["u_x0"]) and same(np.array([trx]), d["cgx0_tol_reached"])
    # unpreconditioned CG (conjugate_gradient.c:13-77)
    up, itp, trp, stp = O.cg_jacobi(rp, ci, K, F, plain=True)
    assert (itp, stp) == (int(d["cgp_niter"][0]), int(d["cgp_status"][0]))
    assert same(up, d["u_plain"]) and same(np.array([trp]), d["cgp_tol_reached"])
    u7, it7, tr7, st7 = O.cg_jacobi(rp, ci, K, F, max_iter=7)
    assert (it7, st7) == (int(d["cg7_niter"][0]), int(d["cg7_status"][0]))
    if int(d["cg_niter"][0]) > 7:  # the not-converged return path
        assert (it7, st7) == (7, 1)
    assert same(u7, d["u_it7"]) and same(np.array([tr7]), d["cg7_tol_reached"])
    assert same(O.strain(fl, u), d["strain"])
    if "fem_u" in d:
        # nbots' FEM entry itself (one material) gives the same displacements
        assert same(u, d["fem_u"])
        assert same(O.stress(fl, d["fem_strain"]), d["fem_stress"])
    if "fem_main_stress" in d:
        # pipeline_compute_main_stress on the reference's own stress
        assert same(O.main_stress(d["fem_stress"]), d["fem_main_stress"])


def test_beam_cantilever_known_answer():
    p, d = load_golden("t3_beam_cantilever")
    r = O.fem(p)
    assert abs(max_disp(r["u"]) - BEAM_MAX_DISP) < 1e-6
    assert abs(float(d["max_disp"][0]) - BEAM_MAX_DISP) < 1e-6


def test_plate_with_hole_known_answer():
    p, d = load_golden("t3_plate_with_hole")
    r = O.fem(p)
    s = O.stress(r["flat"], r["strain"])
    assert pwh_mean_vm_error(p, s) < PWH_MAX_VM_ERR
    assert pwh_mean_vm_error(p, d["fem_stress"]) < PWH_MAX_VM_ERR


def test_oracle_multithreaded_cg_close():
    """OpenMP reductions change the summation order, not the answer."""
    p, d = load_golden("c1_q4_64x32")
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    _, K, F = O.assemble(fl, rp, ci)
    O.set_bconditions(fl, rp, ci, K, F)
    u, it, _, _ = O.cg_jacobi(rp, ci, K, F, threads=4)
    rel = np.linalg.norm(u - d["u"]) / np.linalg.norm(d["u"])
    assert rel < 1e-9 and abs(it - int(d["cg_niter"][0])) <= 3
