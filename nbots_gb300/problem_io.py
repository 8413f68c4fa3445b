"""Binary problem files and tagged-array dumps.

A problem file carries one :class:`~nbots_gb300.workloads.Problem` (mesh,
bc atoms, per-element material) in a flat little-endian layout that C code
reads with plain ``fread`` calls:

    "NBGP"  u32 nen
    u32 N_nod  f64 nod[2 N_nod]
    u32 N_elem u32 conn[nen N_elem]
    u32 N_edg  u32 edg[2 N_edg]
    u32 N_vtx  u32 vtx[N_vtx]
    u32 N_sgm  { u32 n  u32 nodes[n] } * N_sgm
    f64 E[N_elem]  f64 nu  f64 thickness  f64 density  u32 self_weight  f64 gravity[2]
    u32 has_enabled  [u8 enabled[N_elem]]
    u32 N_bc   { u32 kind u32 where u32 id u8 mask[2] f64 val[2] u32 n_nv f64 nv[2 n_nv] } * N_bc

A dump is a sequence of ``u32 name_len, name, u32 dtype, u64 count, data``
records (dtype 0 f64, 1 u32, 2 i32, 3 u8).
"""
from __future__ import annotations

import struct

import numpy as np

from .workloads import BC, Problem

_DT = {0: np.float64, 1: np.uint32, 2: np.int32, 3: np.uint8}


def write_problem(p: Problem, path: str) -> None:
    nen = p.conn.shape[1]
    with open(path, "wb") as f:
        f.write(b"NBGP")
        f.write(struct.pack("<I", nen))
        f.write(struct.pack("<I", p.n_nodes))
        f.write(np.ascontiguousarray(p.nod, "<f8").tobytes())
        f.write(struct.pack("<I", p.n_elems))
        f.write(np.ascontiguousarray(p.conn, "<u4").tobytes())
        f.write(struct.pack("<I", p.edges.shape[0]))
        f.write(np.ascontiguousarray(p.edges, "<u4").tobytes())
        f.write(struct.pack("<I", len(p.vtx)))
        f.write(np.ascontiguousarray(p.vtx, "<u4").tobytes())
        f.write(struct.pack("<I", len(p.sgm)))
        for s in p.sgm:
            f.write(struct.pack("<I", len(s)))
            f.write(np.ascontiguousarray(s, "<u4").tobytes())
        f.write(np.ascontiguousarray(p.E, "<f8").tobytes())
        f.write(struct.pack("<dddI", p.nu, p.thickness, p.density, int(p.self_weight)))
        f.write(struct.pack("<dd", *p.gravity))
        if p.enabled is None:
            f.write(struct.pack("<I", 0))
        else:
            f.write(struct.pack("<I", 1))
            f.write(np.ascontiguousarray(p.enabled, np.uint8).tobytes())
        f.write(struct.pack("<I", len(p.bcs)))
        for b in p.bcs:
            f.write(struct.pack("<III", b.kind, b.where, b.id))
            f.write(struct.pack("<BB", int(b.mask[0]), int(b.mask[1])))
            f.write(struct.pack("<dd", float(b.val[0]), float(b.val[1])))
            nv = b.node_vals
            if nv is None:
                f.write(struct.pack("<I", 0))
            else:
                nv = np.ascontiguousarray(nv, "<f8").reshape(-1, 2)
                f.write(struct.pack("<I", nv.shape[0]))
                f.write(nv.tobytes())


def read_problem(path: str, name: str = "") -> Problem:
    with open(path, "rb") as f:
        buf = f.read()
    o = 0

    def take(fmt):
        nonlocal o
        v = struct.unpack_from(fmt, buf, o)
        o += struct.calcsize(fmt)
        return v

    def arr(dt, n):
        nonlocal o
        a = np.frombuffer(buf, dt, n, o).copy()
        o += a.nbytes
        return a

    assert buf[:4] == b"NBGP"
    o = 4
    (nen,) = take("<I")
    (nn,) = take("<I")
    nod = arr("<f8", 2 * nn).reshape(nn, 2)
    (ne,) = take("<I")
    conn = arr("<u4", nen * ne).reshape(ne, nen)
    (ned,) = take("<I")
    edges = arr("<u4", 2 * ned).reshape(ned, 2)
    (nv,) = take("<I")
    vtx = arr("<u4", nv)
    (ns,) = take("<I")
    sgm = []
    for _ in range(ns):
        (k,) = take("<I")
        sgm.append(arr("<u4", k))
    E = arr("<f8", ne)
    nu, th, dens, sw = take("<dddI")
    g = take("<dd")
    (he,) = take("<I")
    enabled = arr("<u1", ne).astype(bool) if he else None
    (nb,) = take("<I")
    bcs = []
    for _ in range(nb):
        kind, where, bid = take("<III")
        m = take("<BB")
        val = take("<dd")
        (nnv,) = take("<I")
        nvv = arr("<f8", 2 * nnv).reshape(nnv, 2) if nnv else None
        bcs.append(BC(kind, where, bid, m, val, nvv))
    elem = "q4" if nen == 4 else "t3"
    return Problem(name or path, elem, nod, conn, edges, vtx, sgm, bcs, E, nu=nu,
                   thickness=th, density=dens, self_weight=bool(sw), gravity=g,
                   enabled=enabled)


def read_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    o = 0
    while o < len(buf):
        (ln,) = struct.unpack_from("<I", buf, o)
        o += 4
        name = buf[o:o + ln].decode()
        o += ln
        dt, n = struct.unpack_from("<IQ", buf, o)
        o += 12
        a = np.frombuffer(buf, _DT[dt], n, o).copy()
        o += a.nbytes
        out[name] = a
    return out
