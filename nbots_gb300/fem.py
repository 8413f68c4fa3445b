"""Python check harness over the C ABI: a Problem driven through the device
FEM system (nbg_fem_*), stage by stage, mirroring nbots' FEM entry
(pde_bot/finite_element/solid_mechanics/static_elasticity2D.c:31-97).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .workloads import Problem


def _p(a):
    return a.ctypes.data if a is not None else None


class HostArrays:
    """A Problem as nbg_mesh_t / nbg_bcs_t structs (keeps buffers alive)."""

    def __init__(self, p: Problem):
        self.p = p
        self.nod = np.ascontiguousarray(p.nod, np.float64)
        self.conn = np.ascontiguousarray(p.conn, np.uint32)
        self.edg = np.ascontiguousarray(p.edges, np.uint32)
        self.mesh = L.Mesh(p.conn.shape[1], p.n_nodes, p.n_elems, p.edges.shape[0],
                           _p(self.nod), _p(self.conn), _p(self.edg))
        self.vtx = np.ascontiguousarray(p.vtx, np.uint32)
        lens = np.array([len(s) for s in p.sgm], np.uint32)
        self.sgm_ptr = np.zeros(len(p.sgm) + 1, np.uint32)
        self.sgm_ptr[1:] = np.cumsum(lens)
        self.sgm_nodes = (np.concatenate(p.sgm).astype(np.uint32) if p.sgm
                          else np.zeros(1, np.uint32))
        self.atoms = (L.BCAtom * max(1, len(p.bcs)))()
        self._nv = []
        for k, b in enumerate(p.bcs):
            a = self.atoms[k]
            a.kind, a.where, a.id = b.kind, b.where, b.id
            a.mask[0], a.mask[1] = int(b.mask[0]), int(b.mask[1])
            a.val[0], a.val[1] = float(b.val[0]), float(b.val[1])
            if b.node_vals is not None:
                nv = np.ascontiguousarray(b.node_vals, np.float64).reshape(-1, 2)
                self._nv.append(nv)
                a.n_nv, a.node_vals = nv.shape[0], _p(nv)
        self.bcs = L.BCs(_p(self.vtx), len(p.sgm), _p(self.sgm_ptr), _p(self.sgm_nodes),
                         len(p.bcs), C.addressof(self.atoms))
        self.E = np.ascontiguousarray(p.E, np.float64)
        self.enabled = (None if p.enabled is None
                        else np.ascontiguousarray(p.enabled, np.uint8))
        self.grav = np.array(p.gravity, np.float64)


class FemSystem:
    """Device-resident FEM system of one problem."""

    def __init__(self, p: Problem, stream=None):
        self.lib = L.lib()
        self.h = HostArrays(p)
        self.p = p
        self.stream = stream
        h = C.c_void_p()
        L.check(self.lib.nbg_fem_create(C.byref(h), C.byref(self.h.mesh), stream), "fem_create")
        self.handle = h
        self.N = self.lib.nbg_fem_n_dof(h)
        self.nnz = int(self.lib.nbg_fem_nnz(h))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nbg_fem_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def assemble(self):
        p = self.p
        return self.lib.nbg_fem_assemble(self.handle, _p(self.h.E), p.nu, p.thickness,
                                         p.density, int(p.self_weight), _p(self.h.grav),
                                         _p(self.h.enabled))

    def apply_bcs(self, factor=1.0):
        return L.check(self.lib.nbg_fem_apply_bcs(self.handle, C.byref(self.h.bcs), factor),
                       "apply_bcs")

    def solve(self, max_iter=None, tol=1e-8, flags=L.CG_JACOBI):
        r = L.CgResult()
        rc = self.lib.nbg_fem_solve(self.handle, self.N if max_iter is None else max_iter, tol,
                                    flags, C.byref(r))
        if rc < 0:
            L.check(rc, "fem_solve")
        return r

    def solve_fast(self, max_iter=None, tol=1e-8, flags=L.CG_JACOBI | L.CG_RELATIVE):
        r = L.CgResult()
        rc = self.lib.nbg_fem_solve_fast(self.handle, self.N if max_iter is None else max_iter,
                                         tol, flags, C.byref(r))
        if rc < 0:
            L.check(rc, "fem_solve_fast")
        return r

    def solve_mixed(self, max_iter=None, tol=1e-8, delta=0.1, flags=L.CG_JACOBI | L.CG_RELATIVE):
        r = L.MixedResult()
        rc = self.lib.nbg_fem_solve_mixed(self.handle,
                                          4 * self.N if max_iter is None else max_iter, tol,
                                          delta, flags, C.byref(r))
        if rc < 0:
            L.check(rc, "fem_solve_mixed")
        return r

    def set_block_order(self, order, sigma=0):
        L.check(self.lib.nbg_fem_set_block_order(self.handle, order, sigma), "set_block_order")

    def block_layout(self):
        b = L.Bsr()
        L.check(self.lib.nbg_fem_block_layout(self.handle, C.byref(b)), "block_layout")
        return b

    def strain(self):
        L.check(self.lib.nbg_fem_strain(self.handle), "strain")
        return self.get(L.FEM_STRAIN)

    def stress(self):
        L.check(self.lib.nbg_fem_stress(self.handle), "stress")
        return self.get(L.FEM_STRESS)

    def main_stress(self):
        L.check(self.lib.nbg_fem_main_stress(self.handle), "main_stress")
        return self.get(L.FEM_MAIN_STRESS)

    def damage(self, ft, gf, n_steps, max_iter, max_iter_noenh, rtol, logfile=None,
               method=L.METHOD_NBOTS):
        """nbots' quasi-static damage solve (static_damage2D.c:239-470) with
        material E = p.E[0]; returns the run's counters.  The log goes to
        `logfile` (appended) when given; `method` picks the inner solver."""
        p = self.p
        info = L.DamageInfo()
        rc = self.lib.nbg_fem_damage(self.handle, C.byref(self.h.bcs), float(p.E[0]), p.nu,
                                     p.thickness, p.density, int(p.self_weight),
                                     _p(self.h.grav), ft, gf, n_steps, max_iter,
                                     max_iter_noenh, rtol, method,
                                     None if logfile is None else str(logfile).encode(),
                                     C.byref(info))
        L.check(rc, "fem_damage")
        return info

    _DT = {L.FEM_ROW_PTR: np.uint32, L.FEM_COL_IDX: np.uint32}

    def get(self, what):
        nb = self.lib.nbg_fem_bytes(self.handle, what)
        dt = self._DT.get(what, np.float64)
        out = np.empty(nb // np.dtype(dt).itemsize, dt)
        L.check(self.lib.nbg_fem_download(self.handle, what, _p(out)), "download")
        return out

    def put(self, what, arr):
        dt = self._DT.get(what, np.float64)
        a = np.ascontiguousarray(arr, dt)
        assert a.nbytes == self.lib.nbg_fem_bytes(self.handle, what)
        L.check(self.lib.nbg_fem_upload(self.handle, what, _p(a)), "upload")

    def dptr(self, what):
        return self.lib.nbg_fem_device_ptr(self.handle, what)


def fem_compute(p: Problem, tol=1e-8, flags=L.CG_JACOBI):
    """nbots' FEM entry on the GPU: returns dict of host arrays."""
    s = FemSystem(p)
    out = dict(assemble_status=s.assemble())
    if out["assemble_status"] != 0:
        s.close()
        return out
    s.apply_bcs()
    r = s.solve(tol=tol, flags=flags)
    out.update(u=s.get(L.FEM_U), cg_niter=r.niter, cg_status=r.status,
               cg_tol_reached=r.tol_reached, strain=s.strain(), stress=s.stress())
    s.close()
    return out
