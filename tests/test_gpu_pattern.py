"""The device build of nbots' CSR pattern, node incidence and block plan
(nbg_pattern_dev) against the host build (nbg_host_pattern,
nbg_host_incidence, nbg_bsr_plan) and against the pattern nbots itself
built for the committed fixtures: equal word for word.  Cases include
unstructured T3 meshes, a jittered Q4 grid, and the same meshes with their
elements and edges shuffled, so the atomic fills land in another order."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


def host_build(lib, h, p):
    N = 2 * p.n_nodes
    rp = np.zeros(N + 1, np.uint32)
    assert lib.nbg_host_pattern(C.byref(h.mesh), rp.ctypes.data, None) == 0
    ci = np.zeros(int(rp[-1]), np.uint32)
    assert lib.nbg_host_pattern(C.byref(h.mesh), rp.ctypes.data, ci.ctypes.data) == 0
    ip = np.zeros(p.n_nodes + 1, np.uint32)
    nc = p.n_elems * p.conn.shape[1]
    ie = np.zeros(max(nc, 1), np.uint32)
    il = np.zeros(max(nc, 1), np.uint8)
    assert lib.nbg_host_incidence(C.byref(h.mesh), ip.ctypes.data, ie.ctypes.data,
                                  il.ctypes.data) == 0
    S = (p.n_nodes + 31) // 32
    so = np.zeros(S + 1, np.uint32)
    assert lib.nbg_bsr_plan(N, rp.ctypes.data, ci.ctypes.data, so.ctypes.data) == 0
    return rp, ci, ip, ie[:nc], il[:nc], so


def device_build(lib, p):
    from nbots_gb300.device import DeviceArray
    nen = p.conn.shape[1]
    conn = DeviceArray(np.ascontiguousarray(p.conn, np.uint32))
    edg = DeviceArray(np.ascontiguousarray(p.edges, np.uint32).reshape(-1))
    N = 2 * p.n_nodes
    nc = p.n_elems * nen
    S = (p.n_nodes + 31) // 32
    rp = DeviceArray(shape=(N + 1,), dtype=np.uint32)
    ip = DeviceArray(shape=(p.n_nodes + 1,), dtype=np.uint32)
    ie = DeviceArray(shape=(max(nc, 1),), dtype=np.uint32)
    il = DeviceArray(shape=(max(nc, 1),), dtype=np.uint8)
    so = DeviceArray(shape=(S + 1,), dtype=np.uint32)
    ci_ptr, nnz = C.c_void_p(), C.c_uint64()
    rc = lib.nbg_pattern_dev(nen, p.n_nodes, p.n_elems, p.edges.shape[0], conn.ptr, edg.ptr,
                             rp.ptr, C.byref(ci_ptr), C.byref(nnz), ip.ptr, ie.ptr, il.ptr,
                             so.ptr, None)
    if rc != 0:
        return rc, None
    ci = np.empty(nnz.value, np.uint32)
    assert lib.nbg_d2h(ci.ctypes.data, ci_ptr, ci.nbytes, None) == 0
    assert lib.nbg_stream_sync(None) == 0
    lib.nbg_dev_free(ci_ptr)
    return 0, (rp.numpy(), ci, ip.numpy(), ie.numpy()[:nc], il.numpy()[:nc], so.numpy())


def shuffled(p, seed):
    """The same mesh with elements and edges in another order."""
    import copy
    rng = np.random.default_rng(seed)
    q = copy.copy(p)
    q.conn = p.conn[rng.permutation(p.n_elems)]
    q.edges = p.edges[rng.permutation(p.edges.shape[0])]
    return q


def cases():
    from nbots_gb300 import workloads as W
    out = [(n, load_golden(n)[0]) for n in GOLDEN_CASES]
    out.append(("t3_lshape_20k", W.t3_lshape(20000, seed=9)))
    out.append(("q4_jitter_96x40", W.cantilever_q4(96, 40, jitter=0.2, seed=4)))
    return out


@pytest.mark.parametrize("shuffle", [False, True])
def test_device_pattern_equals_host_and_reference(shuffle):
    from nbots_gb300 import _lib as L
    from nbots_gb300.fem import HostArrays
    lib = L.lib()
    for name, p in cases():
        if shuffle:
            p = shuffled(p, 3)
        h = HostArrays(p)
        want = host_build(lib, h, p)
        rc, got = device_build(lib, p)
        assert rc == 0, name
        for k, (a, b) in enumerate(zip(got, want)):
            assert a.dtype == b.dtype and np.array_equal(a, b), (name, k)
        if not shuffle and name in GOLDEN_CASES:
            d = load_golden(name)[1]
            assert np.array_equal(got[0], d["row_ptr"]) and np.array_equal(got[1], d["col_idx"])


def test_device_pattern_rejects_bad_index():
    from nbots_gb300 import _lib as L
    from nbots_gb300 import workloads as W
    p = W.cantilever_q4(8, 4)
    p.conn = p.conn.copy()
    p.conn[5, 2] = p.n_nodes
    assert device_build(L.lib(), p)[0] == -3  # NBG_ERR_ARG
