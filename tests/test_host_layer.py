"""Host-side C (no GPU): the library loads, exports every symbol the C ABI
header declares, and its pattern / incidence builders match the reference."""
import ctypes as C
import os
import re

import numpy as np

from conftest import ROOT, load_golden


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nbg?_\w+)\s*\(", txt)))


def test_library_exports_header_symbols():
    from nbots_gb300 import _lib as L
    lib = L.lib()
    missing = [s for s in declared("nbots_gb300.h") if not hasattr(lib, s)]
    assert not missing, missing


def test_host_pattern_matches_reference(golden):
    from nbots_gb300 import _lib as L
    from nbots_gb300.fem import HostArrays
    name, p, d = golden
    h = HostArrays(p)
    N = p.n_dof
    rp = np.zeros(N + 1, np.uint32)
    assert L.lib().nbg_host_pattern(C.byref(h.mesh), rp.ctypes.data, None) == 0
    ci = np.zeros(int(rp[-1]), np.uint32)
    assert L.lib().nbg_host_pattern(C.byref(h.mesh), rp.ctypes.data, ci.ctypes.data) == 0
    assert np.array_equal(rp, d["row_ptr"]) and np.array_equal(ci, d["col_idx"])


def test_host_incidence_sorted():
    from nbots_gb300 import _lib as L
    from nbots_gb300.fem import HostArrays
    p, _ = load_golden("t3_beam_cantilever")
    h = HostArrays(p)
    nen = p.conn.shape[1]
    ip = np.zeros(p.n_nodes + 1, np.uint32)
    ie = np.zeros(p.n_elems * nen, np.uint32)
    il = np.zeros(p.n_elems * nen, np.uint8)
    assert L.lib().nbg_host_incidence(C.byref(h.mesh), ip.ctypes.data, ie.ctypes.data,
                                      il.ctypes.data) == 0
    for v in range(p.n_nodes):
        es = ie[ip[v]:ip[v + 1]]
        assert np.all(np.diff(es.astype(np.int64)) > 0)
        assert np.all(p.conn[es, il[ip[v]:ip[v + 1]]] == v)
