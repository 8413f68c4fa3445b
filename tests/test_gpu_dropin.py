"""nbots' own entry points, called as an nbots program calls them, on the
GPU drop-in: SpMV bit-exact, CG within 1e-10 relative L2 of nbots' answer,
the FEM entry on nbots-interface objects, and nbots' known answers."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_CASES, cg_iters_close, load_golden
from kat import BEAM_MAX_DISP, PWH_MAX_VM_ERR, max_disp, pwh_mean_vm_error

pytestmark = pytest.mark.gpu
FEM_CASES = [c for c in GOLDEN_CASES if c != "q4_lognormal_32x16"]  # one material only


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def G():
    from nbots_gb300 import _lib as L
    from nbots_gb300.dropin import libs
    assert L.lib().nbg_device_count() > 0
    return libs()[0]


@pytest.mark.parametrize("name", ["c1_q4_64x32", "t3_beam_cantilever", "q4_allbc_16x8"])
def test_multiply_vector_bit_exact(G, name):
    from nbots_gb300.dropin import sparse_from_csr
    p, d = load_golden(name)
    A, keep = sparse_from_csr(p, d["K_bc"])
    y = np.zeros(p.n_dof)
    x = np.ascontiguousarray(d["spmv_x"])
    G.nb_sparse_multiply_vector(A, x.ctypes.data, y.ctypes.data, 4)
    assert np.array_equal(y.view(np.uint64), d["spmv_y"].view(np.uint64))
    G.nb_sparse_destroy(A)


def test_multiply_vector_both_transfer_paths():
    """Where the GPU reaches host memory coherently (Grace, NVLink-C2C) the
    SpMV writes the caller's y itself; NBG_HOST_DIRECT=0 keeps the copy
    back.  Both give nbots' bits (child processes: each picks its path when
    its first matrix is made)."""
    import os
    import subprocess
    import sys
    from conftest import ROOT
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
        "from conftest import load_golden\n"
        "from nbots_gb300.dropin import libs, sparse_from_csr\n"
        "G = libs()[0]\n"
        "p, d = load_golden('c1_q4_64x32')\n"
        "A, keep = sparse_from_csr(p, d['K_bc'])\n"
        "y = np.zeros(p.n_dof); x = np.ascontiguousarray(d['spmv_x'])\n"
        "for _ in range(3):\n"
        "    G.nb_sparse_multiply_vector(A, x.ctypes.data, y.ctypes.data, 1)\n"
        "    assert np.array_equal(y.view(np.uint64), d['spmv_y'].view(np.uint64))\n"
        "assert G.nbg_dropin_error() == 0\n"
        "print('OK')\n" % (ROOT, os.path.join(ROOT, "tests")))
    for direct in ("0", "1"):
        env = dict(os.environ, NBG_HOST_DIRECT=direct)
        env.pop("NBG_DROPIN_CPU", None)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                           env=env, timeout=300)
        assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c != "q4_distorted_8x4"])
def test_cg_precond_jacobi(G, name):
    from nbots_gb300.dropin import sparse_from_csr
    p, d = load_golden(name)
    A, keep = sparse_from_csr(p, d["K_bc"])
    b = np.ascontiguousarray(d["F_bc"])
    x = np.zeros(p.n_dof)
    it, tr = C.c_uint32(0), C.c_double(0)
    st = G.nb_sparse_solve_CG_precond_Jacobi(A, b.ctypes.data, x.ctypes.data, p.n_dof, 1e-8,
                                              C.byref(it), C.byref(tr), 1)
    assert st == int(d["cg_status"][0])
    assert cg_iters_close(it.value, int(d["cg_niter"][0]), np.linalg.norm(b))
    assert rel(x, d["u"]) < 1e-10
    # from a non-zero initial guess (the damage loop passes the last increment)
    xg = np.ascontiguousarray(d["spmv_x"]).copy()
    stx = G.nb_sparse_solve_CG_precond_Jacobi(A, b.ctypes.data, xg.ctypes.data, p.n_dof, 1e-8,
                                               C.byref(it), C.byref(tr), 1)
    assert stx == int(d["cgx0_status"][0])
    assert cg_iters_close(it.value, int(d["cgx0_niter"][0]), np.linalg.norm(b))
    assert rel(xg, d["u_x0"]) < 1e-10
    # the not-converged return path (max_iter = 7)
    x7 = np.zeros(p.n_dof)
    st7 = G.nb_sparse_solve_CG_precond_Jacobi(A, b.ctypes.data, x7.ctypes.data, 7, 1e-8,
                                               C.byref(it), C.byref(tr), 1)
    assert (st7, it.value) == (int(d["cg7_status"][0]), int(d["cg7_niter"][0]))
    assert rel(x7, d["u_it7"]) < (1e-12 if st7 else 1e-10)
    G.nb_sparse_destroy(A)


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c != "q4_distorted_8x4"])
def test_plain_cg_matches_reference(G, name):
    """nb_sparse_solve_conjugate_gradient against nbots' own run (max_iter
    N, absolute tolerance 1e-8)."""
    from nbots_gb300.dropin import sparse_from_csr
    p, d = load_golden(name)
    A, keep = sparse_from_csr(p, d["K_bc"])
    b = np.ascontiguousarray(d["F_bc"])
    x = np.zeros(p.n_dof)
    it, tr = C.c_uint32(0), C.c_double(0)
    st = G.nb_sparse_solve_conjugate_gradient(A, b.ctypes.data, x.ctypes.data, p.n_dof,
                                               1e-8, C.byref(it), C.byref(tr), 1)
    assert st == int(d["cgp_status"][0])
    assert cg_iters_close(it.value, int(d["cgp_niter"][0]), np.linalg.norm(b))
    assert rel(x, d["u_plain"]) < 1e-10
    G.nb_sparse_destroy(A)


@pytest.mark.parametrize("name", FEM_CASES)
def test_fem_entry(G, name):
    from nbots_gb300.dropin import NbotsObjects
    p, d = load_golden(name)
    ob = NbotsObjects(p)
    st, u, strain = ob.fem()
    if int(d["assemble_status"][0]):
        assert st == 1          # distorted element, like nbots
        return
    assert st == 0
    assert rel(u, d["fem_u"]) < 1e-10
    assert rel(strain, d["fem_strain"]) < 1e-8
    # stress from nbots' own strain is bit-exact
    s = ob.stress(d["fem_strain"])
    assert np.array_equal(s.view(np.uint64), d["fem_stress"].view(np.uint64))
    if "fem_main_stress" in d:
        ms = ob.main_stress(d["fem_stress"])
        assert np.array_equal(ms.view(np.uint64), d["fem_main_stress"].view(np.uint64))
    ob.close()


def test_fem_entry_known_answers(G):
    from nbots_gb300.dropin import NbotsObjects
    p, _ = load_golden("t3_beam_cantilever")
    ob = NbotsObjects(p)
    st, u, _ = ob.fem()
    assert st == 0 and abs(max_disp(u) - BEAM_MAX_DISP) < 1e-6
    p, _ = load_golden("t3_plate_with_hole")
    ob = NbotsObjects(p)
    st, u, strain = ob.fem()
    assert st == 0 and pwh_mean_vm_error(p, ob.stress(strain)) < PWH_MAX_VM_ERR


@pytest.mark.parametrize("name", FEM_CASES)
def test_pipeline_stages(G, name):
    """An nbots program that drives the stages itself (static_elasticity2D.c:
    31-81): nb_sparse_create on the nodal graph, pipeline_assemble_system,
    nb_fem_set_bconditions, nb_sparse_solve_CG_precond_Jacobi (x0 = 0,
    max_iter = N, 1e-8), pipeline_compute_strain, all through the drop-in.
    K and F after each stage equal nbots' bit for bit, u is within 1e-10 of
    nbots', and the strain of nbots' u is bit-exact."""
    from nbots_gb300.dropin import NbotsObjects, csr_of, nodal_graph
    p, d = load_golden(name)
    ob = NbotsObjects(p)
    g, keep = nodal_graph(p)
    K = G.nb_sparse_create(C.byref(g), None, 2)
    F = np.zeros(p.n_dof)
    st = ob.pipeline(K, F)
    assert st == int(d["assemble_status"][0])
    if st:
        G.nb_sparse_destroy(K)
        ob.close()
        return
    rp, ci, vals = csr_of(K)
    assert np.array_equal(rp, d["row_ptr"]) and np.array_equal(ci, d["col_idx"])
    assert np.array_equal(vals.view(np.uint64), d["K_asm"].view(np.uint64))
    assert np.array_equal(F.view(np.uint64), d["F_asm"].view(np.uint64))
    ob.set_bconditions(K, F)
    assert G.nbg_dropin_error() == 0
    _, _, vals = csr_of(K)
    assert np.array_equal(vals.view(np.uint64), d["K_bc"].view(np.uint64))
    assert np.array_equal(F.view(np.uint64), d["F_bc"].view(np.uint64))
    u = np.zeros(p.n_dof)
    it, tr = C.c_uint32(0), C.c_double(0)
    cst = G.nb_sparse_solve_CG_precond_Jacobi(K, F.ctypes.data, u.ctypes.data, p.n_dof, 1e-8,
                                               C.byref(it), C.byref(tr), 1)
    assert cst == int(d["cg_status"][0])
    assert cg_iters_close(it.value, int(d["cg_niter"][0]), np.linalg.norm(F))
    assert rel(u, d["u"]) < 1e-10
    strain = ob.strain_of(d["u"])
    assert G.nbg_dropin_error() == 0
    assert np.array_equal(strain.view(np.uint64), d["strain"].view(np.uint64))
    # the stages again on the same matrix (a second load case): nbots resets K
    F2 = np.zeros(p.n_dof)
    assert ob.pipeline(K, F2) == 0
    _, _, vals = csr_of(K)
    assert np.array_equal(vals.view(np.uint64), d["K_asm"].view(np.uint64))
    G.nb_sparse_destroy(K)
    ob.close()


def test_device_copy_follows_host_writes(G):
    """The matrix's device copy is reused while the matrix is unchanged and
    re-sent after a write through any nb_sparse_* writer: each SpMV equals
    nbots' on the current host values."""
    from nbots_gb300.dropin import sparse_from_csr
    from oracle import oracle as O
    p, d = load_golden("c1_q4_64x32")
    A, keep = sparse_from_csr(p, d["K_bc"])
    x = np.ascontiguousarray(d["spmv_x"])
    y = np.zeros(p.n_dof)
    rp, ci = d["row_ptr"], d["col_idx"]

    def check(K):
        G.nb_sparse_multiply_vector(A, x.ctypes.data, y.ctypes.data, 1)
        assert np.array_equal(y.view(np.uint64), O.spmv(rp, ci, K, x).view(np.uint64))
    K = d["K_bc"].copy()
    check(K)
    check(K)                                    # the device copy, unchanged
    G.nb_sparse_add(A, 0, int(ci[0]), 0.5)       # one write through the API
    K[0] += 0.5
    check(K)
    G.nb_sparse_scale(A, 2.0)
    K *= 2.0
    check(K)
    G.nb_sparse_reset(A)
    check(np.zeros_like(K))
    # a direct write to the rows, announced with nbg_dropin_sparse_touch
    C.memmove(A.contents.rows_values[0], d["K_bc"].ctypes.data, d["K_bc"].nbytes)
    G.nbg_dropin_sparse_touch(A)
    check(d["K_bc"])
    G.nb_sparse_destroy(A)
