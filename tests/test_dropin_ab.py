"""The drop-in's A/B switch (NBG_DROPIN_CPU=1): the replaced compute entry
points call the next definition of their symbol, nbots' own, on the same
nb_sparse_t objects; without one they fail instead of running anything.
Runs on the CPU only (no GPU call is made): each case is a child process,
so the reference library loaded there stays out of the test process."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libnbots_ref.so")

CHILD = r"""
import ctypes as C, os, sys
sys.path.insert(0, {root!r}); sys.path.insert(0, os.path.join({root!r}, "tests"))
import numpy as np
from conftest import load_golden
from oracle import oracle as O
from nbots_gb300.dropin import libs, sparse_from_csr
G, H = libs()
os.environ["NBG_DROPIN_CPU"] = "1"
p, d = load_golden("c1_q4_64x32")
A, keep = sparse_from_csr(p, d["K_bc"])
b = np.ascontiguousarray(d["F_bc"])
x = np.zeros(p.n_dof)
it, tr = C.c_uint32(0), C.c_double(0)
st = G.nb_sparse_solve_CG_precond_Jacobi(A, b.ctypes.data, x.ctypes.data, p.n_dof, 1e-8,
                                          C.byref(it), C.byref(tr), 1)
if not {load_ref}:
    assert st == -3, st  # NBG_ERR_ARG: asked for nbots' code, none loaded
    print("OK"); sys.exit(0)
# nbots' own CG, one thread: the reference's numbers exactly
assert st == int(d["cg_status"][0]) and it.value == int(d["cg_niter"][0]), (st, it.value)
assert np.array_equal(x, d["u"])
y = np.zeros(p.n_dof)
G.nb_sparse_multiply_vector(A, x.ctypes.data, y.ctypes.data, 1)
assert np.array_equal(y, O.spmv(d["row_ptr"], d["col_idx"], d["K_bc"], x))
print("OK")
"""


def run_child(load_ref):
    from nbots_gb300 import _lib as L
    env = dict(os.environ)
    env.pop("NBG_DROPIN_CPU", None)
    if load_ref:
        # the deployment's order: the drop-in ahead of nbots (LD_PRELOAD puts
        # them in the global lookup scope in this order)
        env["LD_PRELOAD"] = " ".join([L.HOST_SO, L.GPU_SO, REF_SO])
    code = CHILD.format(root=ROOT, ref=REF_SO, load_ref=load_ref)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.skipif(not os.path.exists(REF_SO),
                    reason="the reference library is built only where its sources are")
def test_switch_runs_nbots_own_code():
    run_child(True)


def test_switch_without_nbots_fails():
    run_child(False)
