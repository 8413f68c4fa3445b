"""The drop-in's replacements of the remaining writers of sparse.h
(nb_sparse_set_identity_row, _make_diagonal, _scale, _multiply_scalar, and
the forwarding transpose, get_transpose and fill_permutation): on a matrix
made by the drop-in they leave the values nbots' own definitions leave,
bit for bit.  They exist so that every write to a matrix reaches the
drop-in, which keeps a device copy of it.  CPU only; each case runs in a
child process so the reference library stays out of the test process."""
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
from nbots_gb300.dropin import Sparse, csr_of, libs, sparse_from_csr
G, H = libs()
sp = C.POINTER(Sparse)
for n, args in (("nb_sparse_set_identity_row", [sp, C.c_uint32]),
                ("nb_sparse_make_diagonal", [sp, C.c_double]),
                ("nb_sparse_multiply_scalar", [sp, C.c_double, C.c_uint32]),
                ("nb_sparse_transpose", [sp]), ("nb_sparse_get_transpose", [sp, sp]),
                ("nb_sparse_fill_permutation", [sp, sp, C.c_void_p, C.c_void_p])):
    getattr(G, n).argtypes = args
    getattr(G, n).restype = None
p, d = load_golden("c1_q4_64x32")
rng = np.random.default_rng(3)
K = rng.standard_normal(d["K_bc"].shape[0])  # not symmetric: transposes show
N = p.n_dof
perm = np.ascontiguousarray(rng.permutation(N), np.uint32)
iperm = np.empty(N, np.uint32); iperm[perm] = np.arange(N, dtype=np.uint32)

def fresh():
    A, keep = sparse_from_csr(p, K)
    return A, keep

def ops(lib):
    out = []
    for name, call in (
            ("set_identity_row", lambda A: lib.nb_sparse_set_identity_row(A, 17)),
            ("make_diagonal", lambda A: lib.nb_sparse_make_diagonal(A, 2.5)),
            ("scale", lambda A: lib.nb_sparse_scale(A, -0.375)),
            ("multiply_scalar", lambda A: lib.nb_sparse_multiply_scalar(A, 3.0, 1)),
            ("transpose", lambda A: lib.nb_sparse_transpose(A))):
        A, keep = fresh()
        call(A)
        out.append((name, csr_of(A)[2]))
        G.nb_sparse_destroy(A)
    # get_transpose writes into a matrix with the transposed pattern, here
    # the same symmetric pattern; fill_permutation into one of PAP'
    A, k1 = fresh(); At, k2 = fresh()
    G.nb_sparse_reset(At)
    lib.nb_sparse_get_transpose(A, At)
    out.append(("get_transpose", np.concatenate([csr_of(At)[1], csr_of(At)[2]])))
    G.nb_sparse_destroy(A); G.nb_sparse_destroy(At)
    return out

mine = ops(G)
if {load_ref}:
    ref = C.CDLL({ref!r})  # its own definitions, looked up in it directly
    for n, args in (("nb_sparse_set_identity_row", [sp, C.c_uint32]),
                    ("nb_sparse_make_diagonal", [sp, C.c_double]),
                    ("nb_sparse_scale", [sp, C.c_double]),
                    ("nb_sparse_multiply_scalar", [sp, C.c_double, C.c_uint32]),
                    ("nb_sparse_transpose", [sp]), ("nb_sparse_get_transpose", [sp, sp])):
        getattr(ref, n).argtypes = args
        getattr(ref, n).restype = None
    theirs = ops(ref)
    for (n1, a), (n2, b) in zip(mine, theirs):
        assert n1 == n2 and np.array_equal(a.view(np.uint64), b.view(np.uint64)), n1
    assert G.nbg_dropin_error() == 0
else:
    # the plain loops against their definition; the forwarding ones report
    # that nbots is not there
    ref_vals = dict(mine)
    rp, ci, _ = csr_of(fresh()[0])
    r17 = slice(int(rp[17]), int(rp[18]))
    want = K.copy(); want[r17] = 0.0; want[int(rp[17]) + list(ci[r17]).index(17)] = 1.0
    assert np.array_equal(ref_vals["set_identity_row"], want)
    diag = np.zeros_like(K)
    for i in range(N):
        diag[int(rp[i]) + list(ci[rp[i]:rp[i + 1]]).index(i)] = 2.5
    assert np.array_equal(ref_vals["make_diagonal"], diag)
    assert np.array_equal(ref_vals["scale"], K * -0.375)
    assert np.array_equal(ref_vals["multiply_scalar"], K * 3.0)
    assert np.array_equal(ref_vals["transpose"], K)  # left unchanged
    assert G.nbg_dropin_error() == -3
print("OK")
"""


def run_child(load_ref):
    from nbots_gb300 import _lib as L
    env = dict(os.environ)
    env.pop("NBG_DROPIN_CPU", None)
    if load_ref:
        env["LD_PRELOAD"] = " ".join([L.HOST_SO, L.GPU_SO, REF_SO])
    code = CHILD.format(root=ROOT, ref=REF_SO, load_ref=load_ref)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.skipif(not os.path.exists(REF_SO),
                    reason="the reference library is built only where its sources are")
def test_writers_equal_nbots_own():
    run_child(True)


def test_writers_without_nbots():
    run_child(False)
