"""Drop-in nb_sparse_* host functions (no GPU): the pattern of
nb_sparse_create, nbots' binary-search semantics, Dirichlet elimination,
missing-entry behaviour, memory ownership, and the exported symbols."""
import ctypes as C
import os
import re

import numpy as np

from conftest import ROOT, load_golden
from oracle import oracle as O


def declared(section_start, section_end):
    txt = open(os.path.join(ROOT, "include", "nbots_dropin.h")).read()
    txt = txt[txt.index(section_start):txt.index(section_end)]
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nbg?_\w+)\s*\(", txt)))


def test_dropin_symbols_exported():
    from nbots_gb300 import _lib as L
    g, h = L.lib(), L.host_lib()
    replaced = declared("replaced: sparse", "consumed: nbots public accessors")
    consumed = declared("consumed: nbots public accessors", "#ifdef __cplusplus\n}")
    assert not [s for s in replaced if not hasattr(g, s)]
    assert not [s for s in consumed if not hasattr(h, s)]


def test_sparse_create_pattern_matches_reference(golden):
    from nbots_gb300.dropin import csr_of, libs, sparse_from_csr
    name, p, d = golden
    if "K_asm" not in d:
        return
    A, keep = sparse_from_csr(p, d["K_asm"])
    rp, ci, v = csr_of(A)
    assert np.array_equal(rp, d["row_ptr"]) and np.array_equal(ci, d["col_idx"])
    assert np.array_equal(v, d["K_asm"])
    G, _ = libs()
    assert G.nb_sparse_get_size(A) == p.n_dof
    assert G.nb_sparse_get_nnz(A) == d["col_idx"].shape[0]
    G.nb_sparse_destroy(A)


def test_sparse_get_set_add_and_missing_entry():
    from nbots_gb300.dropin import libs, sparse_from_csr
    G, _ = libs()
    p, d = load_golden("q4_allbc_16x8")
    A, keep = sparse_from_csr(p, d["K_asm"])
    ref = d["K_asm"]
    rp, ci = d["row_ptr"], d["col_idx"]
    for i in (0, 7, 100, p.n_dof - 1):
        for k in range(rp[i], rp[i + 1]):
            assert G.nb_sparse_get(A, i, int(ci[k])) == ref[k]
            assert G.nb_sparse_is_non_zero(A, i, int(ci[k]))
    i, k = 11, int(rp[11] + 3)
    j = int(ci[k])
    G.nb_sparse_add(A, i, j, 2.5)
    assert G.nb_sparse_get(A, i, j) == ref[k] + 2.5
    assert G.nb_sparse_get_and_set(A, i, j, -1.0) == ref[k] + 2.5
    assert G.nb_sparse_get(A, i, j) == -1.0
    # an entry outside the pattern: nbots exits, the drop-in records an error
    assert G.nbg_dropin_error() == 0
    G.nb_sparse_add(A, 0, p.n_dof - 1, 1.0)
    assert G.nbg_dropin_error() == -5 and G.nbg_dropin_error() == 0
    assert G.nb_sparse_get(A, 0, p.n_dof - 1) == 0.0
    G.nb_sparse_reset(A)
    assert G.nb_sparse_get(A, i, j) == 0.0
    G.nb_sparse_destroy(A)


def test_dirichlet_condition_matches_oracle():
    from nbots_gb300.dropin import csr_of, libs, sparse_from_csr
    G, _ = libs()
    p, d = load_golden("c1_q4_64x32")
    A, keep = sparse_from_csr(p, d["K_asm"])
    F = d["F_asm"].copy() + 0.5
    K2, F2 = d["K_asm"].copy(), F.copy()
    rp, ci = d["row_ptr"], d["col_idx"]
    lib = O.lib()
    for idx, val in ((0, 0.0), (1, 0.25), (130, -0.1), (0, 0.0), (4289, 3.0)):
        G.nb_sparse_set_Dirichlet_condition(A, F.ctypes.data, idx, val)
        lib.orc_set_dirichlet(rp.ctypes.data, ci.ctypes.data, K2.ctypes.data, F2.ctypes.data,
                              idx, val)
    _, _, v = csr_of(A)
    assert np.array_equal(v.view(np.uint64), K2.view(np.uint64))
    assert np.array_equal(F.view(np.uint64), F2.view(np.uint64))
    G.nb_sparse_destroy(A)


def test_clone_and_destroy_with_replaced_rows():
    """destroy frees slab rows and rows that other code allocated."""
    from nbots_gb300.dropin import csr_of, libs, sparse_from_csr
    G, _ = libs()
    libc = C.CDLL(None)
    libc.malloc.restype = C.c_void_p
    libc.malloc.argtypes = [C.c_size_t]
    p, d = load_golden("q4_allbc_16x8")
    A, keep = sparse_from_csr(p, d["K_asm"])
    B = G.nb_sparse_clone(A)
    rp1, ci1, v1 = csr_of(A)
    rp2, ci2, v2 = csr_of(B)
    assert np.array_equal(ci1, ci2) and np.array_equal(v1, v2)
    # replace row 3 of B by a row allocated elsewhere, as nbots' own helpers do
    n = B.contents.rows_size[3]
    newv = libc.malloc(8 * n)
    newi = libc.malloc(4 * n)
    C.memmove(newv, B.contents.rows_values[3], 8 * n)
    C.memmove(newi, B.contents.rows_index[3], 4 * n)
    B.contents.rows_values[3] = C.cast(newv, C.POINTER(C.c_double))
    B.contents.rows_index[3] = C.cast(newi, C.POINTER(C.c_uint32))
    G.nb_sparse_destroy(B)
    G.nb_sparse_destroy(A)


def test_registry_under_threads():
    """Matrices created, written and destroyed from several threads at once
    (the registry of slab-backed matrices, its epoch and the per-thread memo
    of the last lookup that every nb_sparse_add consults): every matrix ends
    with the sums its own thread added, and destroy frees everything without
    error.  ctypes releases the interpreter lock around each C call, so the
    threads do run the C code concurrently."""
    import threading
    from nbots_gb300 import workloads as W
    from nbots_gb300.dropin import csr_of, libs, nodal_graph
    G, _ = libs()
    p = W.cantilever_q4(8, 4)
    g, keep = nodal_graph(p)
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    errors = []

    def work(seed):
        try:
            rng = np.random.default_rng(seed)
            for _ in range(30):
                mats = [G.nb_sparse_create(C.byref(g), None, 2) for _ in range(3)]
                want = [np.zeros(ci.shape[0]) for _ in mats]
                for _ in range(200):
                    m = int(rng.integers(len(mats)))
                    k = int(rng.integers(ci.shape[0]))
                    i = int(np.searchsorted(rp, k, side="right") - 1)
                    G.nb_sparse_add(mats[m], i, int(ci[k]), 1.0)
                    want[m][k] += 1.0
                for A, w in zip(mats, want):
                    if not np.array_equal(csr_of(A)[2], w):
                        errors.append("values")
                    G.nb_sparse_destroy(A)
        except Exception as e:  # reported below
            errors.append(repr(e))
    ts = [threading.Thread(target=work, args=(s,)) for s in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors[:3]
    assert G.nbg_dropin_error() == 0
