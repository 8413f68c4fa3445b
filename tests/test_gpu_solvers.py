"""Fast FP64 and mixed-precision solvers, the host-buffer C ABI, and the
failure paths, on the GPU.

Tolerances: both fast solvers stop on the relative residual they are given;
their true FP64 residual (checked here with the oracle's SpMV) must meet it.
Displacements are compared with nbots' own result (reference fixture) and
with an oracle solution converged to relres 1e-13: the mixed solver at
tol 1e-11 must agree with it to 1e-8 relative L2."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from kat import BEAM_MAX_DISP, max_disp
from oracle import oracle as O

pytestmark = pytest.mark.gpu
Q4_CASES = ["c1_q4_64x32", "q4_lognormal_32x16", "q4_allbc_16x8"]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def L():
    from nbots_gb300 import _lib
    assert _lib.lib().nbg_device_count() > 0
    return _lib


def system(name):
    from nbots_gb300.fem import FemSystem
    p, d = load_golden(name)
    s = FemSystem(p)
    assert s.assemble() == 0
    s.apply_bcs()
    return p, d, s


def true_relres(d, u):
    r = d["F_bc"] - O.spmv(d["row_ptr"], d["col_idx"], d["K_bc"], u)
    return float(np.linalg.norm(r) / np.linalg.norm(d["F_bc"]))


def tight(d):
    u, _, _, _ = O.cg_jacobi(d["row_ptr"], d["col_idx"], d["K_bc"], d["F_bc"],
                             max_iter=20 * d["F_bc"].shape[0],
                             tol=1e-13 * np.linalg.norm(d["F_bc"]))
    return u


@pytest.mark.parametrize("name", Q4_CASES + ["t3_beam_cantilever"])
def test_fast_fp64_solver(L, name):
    p, d, s = system(name)
    r = s.solve_fast(tol=1e-10)
    u = s.get(L.FEM_U)
    assert r.status == 0
    assert true_relres(d, u) <= 1.05e-10
    assert rel(u, tight(d)) < 1e-8


@pytest.mark.parametrize("name", Q4_CASES + ["t3_beam_cantilever"])
def test_mixed_solver(L, name):
    p, d, s = system(name)
    r = s.solve_mixed(tol=1e-8)
    u = s.get(L.FEM_U)
    assert r.status == 0 and r.relres <= 1e-8
    assert true_relres(d, u) <= 1.05e-8
    # both nbots' answer and this one stop near relres 1e-8
    assert rel(u, d["u"]) < 1e-5
    r = s.solve_mixed(tol=1e-11)
    u = s.get(L.FEM_U)
    assert r.status == 0 and true_relres(d, u) <= 1.05e-11
    assert rel(u, tight(d)) < 1e-8


def test_mixed_known_answer_and_determinism(L):
    p, d, s = system("t3_beam_cantilever")
    s.solve_mixed(tol=1e-10)
    u1 = s.get(L.FEM_U)
    assert abs(max_disp(u1) - BEAM_MAX_DISP) < 1e-6
    s.solve_mixed(tol=1e-10)
    assert np.array_equal(s.get(L.FEM_U).view(np.uint64), u1.view(np.uint64))


@pytest.mark.parametrize("method", [0, 1, 2])
def test_host_buffer_solver(L, method):
    lib = L.lib()
    p, d = load_golden("c1_q4_64x32")
    N = d["F_bc"].shape[0]
    h = C.c_void_p()
    assert lib.nbg_solver_create(C.byref(h), None) == 0
    rp, ci, K, F = (np.ascontiguousarray(d[k]) for k in ("row_ptr", "col_idx", "K_bc", "F_bc"))
    for flags in (0, L.PATTERN_SAME):
        assert lib.nbg_solver_set_matrix(h, N, rp.ctypes.data, ci.ctypes.data, K.ctypes.data,
                                         flags) == 0
        x = np.zeros(N)
        info = L.SolveInfo()
        tol = 1e-8 if method == 0 else 1e-10
        fl = L.CG_JACOBI | (0 if method == 0 else L.CG_RELATIVE)
        rc = lib.nbg_solver_solve(h, F.ctypes.data, x.ctypes.data, N * 4, tol, fl, method,
                                  C.byref(info))
        assert rc == 0 and info.status == 0
        if method == 0:
            # nbots' iteration, absolute tolerance: the reference's answer
            assert rel(x, d["u"]) < 1e-10
        else:
            assert true_relres(d, x) <= 1.05e-10
    lib.nbg_solver_destroy(h)


def test_missing_pattern_pair_is_an_error(L):
    """nbots exits when an element pair is not in the pattern
    (sparse.c:213-218); here assembly returns NBG_ERR_PATTERN."""
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem
    p = W.cantilever_q4(8, 4)
    p.edges = p.edges[1:]          # drop one mesh edge
    s = FemSystem(p)
    assert s.assemble() == -5


def test_not_spd_does_not_hang(L):
    """A negative modulus makes K indefinite: the solvers must come back with
    a status, never hang."""
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem
    p = W.cantilever_q4(16, 8)
    p.E[::3] = -1.0
    s = FemSystem(p)
    assert s.assemble() == 0
    s.apply_bcs()
    r = s.solve(max_iter=500)
    assert r.status in (0, 1)
    r2 = s.solve_mixed(max_iter=500)
    assert r2.status in (0, 1)


def test_bounded_device_wait_times_out_and_context_survives(L):
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    flag = DeviceArray(np.zeros(1, np.int32))
    status = DeviceArray(np.zeros(1, np.int32))
    assert lib.nbg_wait_flag(flag.ptr, 1, 50_000_000, status.ptr, None) == 0
    assert lib.nbg_stream_sync(None) == 0
    assert int(status.numpy()[0]) == -2       # NBG_ERR_TIMEOUT
    # the context is still usable
    p, d, s = system("q4_allbc_16x8")
    assert s.solve().status == 0


def mixed_on(L, A, F, N, ws_bytes, tol=1e-10):
    from nbots_gb300.device import DeviceArray
    lib = L.lib()
    u = DeviceArray(np.zeros(N))
    ws = DeviceArray(shape=(max(ws_bytes, 1),), dtype=np.uint8)
    r = L.MixedResult()
    rc = lib.nbg_cg_mixed(C.byref(A), F, u.ptr, 8 * N, tol, 0.1, L.CG_JACOBI | L.CG_RELATIVE,
                          C.byref(r), ws.ptr, ws_bytes, None)
    return rc, r, u.numpy()


@pytest.mark.parametrize("name", ["c1_q4_64x32", "q4_lognormal_32x16"])
def test_mixed_ghost_form_equals_global_gather_form(L, name):
    """With the layout-sized workspace the mixed solver keeps each block's
    ghosts in shared memory (two grid barriers per iteration); with the
    minimal one it gathers p from global memory (three).  The iterates, and
    so the iteration count and the solution, are the same bit for bit."""
    p, d, s = system(name)
    A = s.block_layout()
    lib = L.lib()
    N, F = s.N, s.dptr(L.FEM_F)
    small = lib.nbg_cg_mixed_workspace_bytes(N)
    full = lib.nbg_cg_mixed_layout_workspace_bytes(C.byref(A))
    assert full > small
    rc0, r0, u0 = mixed_on(L, A, F, N, small)
    rc1, r1, u1 = mixed_on(L, A, F, N, full)
    assert rc0 == rc1 == 0
    assert (r1.niter, r1.n_updates) == (r0.niter, r0.n_updates)
    assert np.array_equal(u1.view(np.uint64), u0.view(np.uint64))
    assert true_relres(d, u1) <= 1.05e-10
    s.close()


def test_mixed_ghost_form_full_size_bit_identical(L):
    """The same on the 1M-dof cantilever, where each of the 152 blocks holds
    about 3,500 own node rows and 2,000 ghosts."""
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem
    s = FemSystem(W.config_c2())
    assert s.assemble() == 0
    s.apply_bcs()
    A = s.block_layout()
    lib = L.lib()
    N, F = s.N, s.dptr(L.FEM_F)
    rc0, r0, u0 = mixed_on(L, A, F, N, lib.nbg_cg_mixed_workspace_bytes(N), tol=1e-8)
    rc1, r1, u1 = mixed_on(L, A, F, N, lib.nbg_cg_mixed_layout_workspace_bytes(C.byref(A)),
                           tol=1e-8)
    assert rc0 == rc1 == 0
    assert (r1.niter, r1.n_updates) == (r0.niter, r0.n_updates)
    assert np.array_equal(u1.view(np.uint64), u0.view(np.uint64))
    s.close()
