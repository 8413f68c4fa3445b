"""Batched SIMP solves through the C ABI (nbg_batch_*): many independent
problems of uneven size merged into one block-diagonal system, solved side
by side by one persistent mixed-precision CG launch with the compliance
sensitivities, replayed as a CUDA graph.  No counterpart in nbots.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fem import HostArrays, _p


class Batch:
    def __init__(self, problems, stream=None):
        self.lib = L.lib()
        self.problems = list(problems)
        n = len(self.problems)
        self.h = [HostArrays(p) for p in self.problems]
        meshes = (L.Mesh * n)(*[h.mesh for h in self.h])
        bcs = (L.BCs * n)(*[h.bcs for h in self.h])
        handle = C.c_void_p()
        L.check(self.lib.nbg_batch_create(C.byref(handle), n, meshes, bcs, stream),
                "batch_create")
        self.handle = handle
        self.node_off = np.zeros(n + 1, np.uint32)
        self.elem_off = np.zeros(n + 1, np.uint32)
        L.check(self.lib.nbg_batch_offsets(handle, _p(self.node_off), _p(self.elem_off)),
                "batch_offsets")
        self.fem = self.lib.nbg_batch_fem(handle)
        self.n_dof = int(self.lib.nbg_fem_n_dof(self.fem))
        self.n_elems = int(self.elem_off[-1])

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nbg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def assemble_simp(self, rho, nu, thickness=1.0, penal=3.0, E0=1.0, Emin=1e-9):
        """rho: one array per instance, or the merged array."""
        r = np.ascontiguousarray(np.concatenate(rho) if isinstance(rho, (list, tuple)) else rho,
                                 np.float64)
        assert r.shape == (self.n_elems,)
        L.check(self.lib.nbg_batch_assemble_simp(self.handle, _p(r), nu, thickness, penal, E0,
                                                 Emin), "batch_assemble_simp")

    def setup(self, max_iter=20000, tol=1e-8, delta=0.1, flags=L.CG_JACOBI | L.CG_RELATIVE):
        L.check(self.lib.nbg_batch_setup(self.handle, max_iter, tol, delta, flags),
                "batch_setup")

    @property
    def solver(self):
        return self.lib.nbg_batch_solver(self.handle)

    def plan(self, gamma):
        L.check(self.lib.nbg_mixed_batch_plan(self.solver, gamma), "batch_plan")

    def blocks(self):
        n = len(self.problems)
        b = np.zeros(n, np.uint32)
        g = C.c_double()
        G = self.lib.nbg_mixed_batch_blocks(self.solver, _p(b), C.byref(g))
        return int(G), b, g.value

    def tune(self, gammas=(0.75, 1.0, 1.25, 1.5)):
        gs = np.ascontiguousarray(gammas, np.float64)
        ms = np.zeros(len(gs))
        L.check(self.lib.nbg_mixed_batch_tune(self.solver, len(gs), _p(gs), _p(ms)),
                "batch_tune")
        return ms

    def launch(self):
        L.check(self.lib.nbg_batch_launch(self.handle), "batch_launch")

    def results(self):
        n = len(self.problems)
        res = (L.MixedResult * n)()
        J = np.zeros(n)
        rc = self.lib.nbg_batch_results(self.handle, res, _p(J))
        if rc < 0:
            L.check(rc, "batch_results")
        return list(res), J

    def merged(self, what):
        nb = self.lib.nbg_fem_bytes(self.fem, what)
        dt = np.uint32 if what in (L.FEM_ROW_PTR, L.FEM_COL_IDX, L.FEM_CONN) else np.float64
        out = np.empty(nb // np.dtype(dt).itemsize, dt)
        L.check(self.lib.nbg_fem_download(self.fem, what, _p(out)), "download")
        return out

    def displacements(self):
        u = self.merged(L.FEM_U)
        return [u[2 * int(self.node_off[k]): 2 * (int(self.node_off[k]) + p.n_nodes)].copy()
                for k, p in enumerate(self.problems)]

    def sensitivities(self):
        dJ = np.empty(self.n_elems)
        L.check(self.lib.nbg_batch_sensitivities(self.handle, _p(dJ)), "batch_sensitivities")
        return [dJ[int(self.elem_off[k]): int(self.elem_off[k + 1])].copy()
                for k in range(len(self.problems))]
