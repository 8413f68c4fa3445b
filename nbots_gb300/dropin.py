"""Check harness for the drop-in nbots entry points (include/nbots_dropin.h).

Builds nbots-interface objects (mesh, boundary conditions, material,
element type) for a Problem with libnbots_host.so and calls the drop-in
functions of libnbots_gpu.so exactly as nbots callers would.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .workloads import Problem

vp, u32, f64, b8 = C.c_void_p, C.c_uint32, C.c_double, C.c_bool
FVAL = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double))


class Graph(C.Structure):
    _fields_ = [("N", u32), ("N_adj", C.POINTER(u32)), ("adj", C.POINTER(C.POINTER(u32))),
                ("wi", vp), ("wij", vp)]


class Sparse(C.Structure):
    _fields_ = [("rows_values", C.POINTER(C.POINTER(C.c_double))),
                ("rows_index", C.POINTER(C.POINTER(u32))), ("rows_size", C.POINTER(u32)),
                ("N", u32)]


class Params2D(C.Structure):
    _fields_ = [("thickness", C.c_double), ("revolution_axe", C.c_double),
                ("revolution_coordinate", C.c_char)]


_done = False


def libs():
    global _done
    G = L.lib()
    H = L.host_lib()
    if not _done:
        sp = C.POINTER(Sparse)
        G.nb_sparse_create.argtypes = [C.POINTER(Graph), vp, u32]
        G.nb_sparse_create.restype = sp
        G.nb_sparse_clone.argtypes = [sp]
        G.nb_sparse_clone.restype = sp
        G.nb_sparse_destroy.argtypes = [sp]
        G.nb_sparse_destroy.restype = None
        G.nb_sparse_reset.argtypes = [sp]
        G.nb_sparse_reset.restype = None
        for n in ("nb_sparse_set", "nb_sparse_add"):
            getattr(G, n).argtypes = [sp, u32, u32, f64]
            getattr(G, n).restype = None
        G.nb_sparse_get.argtypes = [sp, u32, u32]
        G.nb_sparse_get.restype = f64
        G.nb_sparse_get_and_set.argtypes = [sp, u32, u32, f64]
        G.nb_sparse_get_and_set.restype = f64
        G.nb_sparse_is_non_zero.argtypes = [sp, u32, u32]
        G.nb_sparse_is_non_zero.restype = b8
        G.nb_sparse_get_size.argtypes = [sp]
        G.nb_sparse_get_size.restype = u32
        G.nb_sparse_get_nnz.argtypes = [sp]
        G.nb_sparse_get_nnz.restype = u32
        G.nb_sparse_multiply_vector.argtypes = [sp, vp, vp, u32]
        G.nb_sparse_multiply_vector.restype = None
        G.nb_sparse_set_Dirichlet_condition.argtypes = [sp, vp, u32, f64]
        G.nb_sparse_set_Dirichlet_condition.restype = None
        for n in ("nb_sparse_solve_CG_precond_Jacobi", "nb_sparse_solve_conjugate_gradient"):
            getattr(G, n).argtypes = [sp, vp, vp, u32, f64, C.POINTER(u32), C.POINTER(f64), u32]
            getattr(G, n).restype = C.c_int
        G.nb_fem_compute_2D_Solid_Mechanics.argtypes = [vp, vp, vp, vp, b8, vp, C.c_int,
                                                        C.POINTER(Params2D), vp, vp, vp]
        G.nb_fem_compute_2D_Solid_Mechanics.restype = C.c_int
        G.nb_fem_compute_stress_from_strain.argtypes = [u32, vp, vp, C.c_int, vp, vp, vp]
        G.nb_fem_compute_stress_from_strain.restype = None
        G.pipeline_compute_main_stress.argtypes = [vp, vp, u32, vp]
        G.pipeline_compute_main_stress.restype = None
        G.nb_fem_compute_2D_Non_Linear_Solid_Mechanics.argtypes = [
            vp, vp, vp, vp, b8, vp, b8, C.c_int, C.POINTER(Params2D), vp, C.c_char_p]
        G.nb_fem_compute_2D_Non_Linear_Solid_Mechanics.restype = None
        G.nbg_dropin_error.restype = C.c_int
        G.pipeline_assemble_system.argtypes = [sp, vp, vp, vp, vp, vp, b8, vp, C.c_int,
                                               C.POINTER(Params2D), vp]
        G.pipeline_assemble_system.restype = C.c_int
        G.nb_fem_set_bconditions.argtypes = [vp, sp, vp, vp, f64]
        G.nb_fem_set_bconditions.restype = None
        G.pipeline_compute_strain.argtypes = [vp, vp, vp, vp]
        G.pipeline_compute_strain.restype = None
        G.nb_sparse_scale.argtypes = [sp, f64]
        G.nb_sparse_scale.restype = None
        G.nbg_dropin_sparse_touch.argtypes = [sp]
        G.nbg_dropin_sparse_touch.restype = None
        H.nbh_mesh2D_create.argtypes = [u32, u32, vp, u32, vp, u32, vp, u32, vp, u32, vp, vp]
        H.nbh_mesh2D_create.restype = vp
        H.nb_mesh2D_destroy.argtypes = [vp]
        H.nb_mesh2D_destroy.restype = None
        H.nb_bcond_create.argtypes = [C.c_uint8]
        H.nb_bcond_create.restype = vp
        H.nb_bcond_destroy.argtypes = [vp]
        H.nb_bcond_destroy.restype = None
        H.nb_bcond_push.argtypes = [vp, C.c_int, C.c_int, u32, C.POINTER(b8), C.POINTER(f64)]
        H.nb_bcond_push.restype = None
        H.nb_bcond_push_function.argtypes = [vp, C.c_int, C.c_int, u32, C.POINTER(b8), FVAL]
        H.nb_bcond_push_function.restype = None
        H.nb_material_create.restype = vp
        H.nb_material_destroy.argtypes = [vp]
        for n in ("elasticity", "poisson"):
            getattr(H, f"nb_material_set_{n}_module").argtypes = [vp, f64]
        H.nb_material_set_density.argtypes = [vp, f64]
        H.nb_material_set_traction_limit_stress.argtypes = [vp, f64]
        H.nb_material_set_fracture_energy.argtypes = [vp, f64]
        H.nb_fem_implicit_create.restype = vp
        H.nb_fem_implicit_destroy.argtypes = [vp]
        for n in ("N_steps", "N_max_iter", "N_max_iter_without_enhance"):
            getattr(H, f"nb_fem_implicit_set_{n}").argtypes = [vp, u32]
        H.nb_fem_implicit_set_residual_tolerance.argtypes = [vp, f64]
        H.nb_fem_elem_create.argtypes = [C.c_int]
        H.nb_fem_elem_create.restype = vp
        H.nb_fem_elem_destroy.argtypes = [vp]
        _done = True
    return G, H


class NbotsObjects:
    """nbots-interface objects of a problem (uniform E: nbots' FEM entry
    takes one material)."""

    def __init__(self, p: Problem):
        G, H = libs()
        self.p = p
        self.H = H
        self.nod = np.ascontiguousarray(p.nod, np.float64)
        self.conn = np.ascontiguousarray(p.conn, np.uint32)
        self.edg = np.ascontiguousarray(p.edges, np.uint32)
        self.vtx = np.ascontiguousarray(p.vtx, np.uint32)
        lens = np.array([len(s) for s in p.sgm], np.uint32)
        self.sgm_ptr = np.zeros(len(p.sgm) + 1, np.uint32)
        self.sgm_ptr[1:] = np.cumsum(lens)
        self.sgm_nodes = (np.concatenate(p.sgm).astype(np.uint32) if p.sgm
                          else np.zeros(1, np.uint32))
        nen = p.conn.shape[1]
        self.mesh = H.nbh_mesh2D_create(nen, p.n_nodes, self.nod.ctypes.data, p.n_elems,
                                        self.conn.ctypes.data, p.edges.shape[0],
                                        self.edg.ctypes.data, len(p.vtx), self.vtx.ctypes.data,
                                        len(p.sgm), self.sgm_ptr.ctypes.data,
                                        self.sgm_nodes.ctypes.data)
        self.bcond = H.nb_bcond_create(2)
        self._cb = []
        for b in p.bcs:
            mask = (b8 * 2)(bool(b.mask[0]), bool(b.mask[1]))
            if b.node_vals is None:
                H.nb_bcond_push(self.bcond, b.kind, b.where, b.id, mask,
                                (f64 * 2)(float(b.val[0]), float(b.val[1])))
            else:
                H.nb_bcond_push_function(self.bcond, b.kind, b.where, b.id, mask,
                                         self._callback(b))
        self.mat = H.nb_material_create()
        H.nb_material_set_elasticity_module(self.mat, float(p.E[0]))
        H.nb_material_set_poisson_module(self.mat, p.nu)
        H.nb_material_set_density(self.mat, p.density)
        self.elem = H.nb_fem_elem_create(1 if nen == 4 else 0)

    def _callback(self, b):
        """Function-valued atom: the stored node values, looked up by the
        coordinates nbots evaluates at."""
        p = self.p
        if b.where == 1:
            nodes = p.sgm[b.id]
            pts = {(float(p.nod[n, 0]), float(p.nod[n, 1])): b.node_vals[k]
                   for k, n in enumerate(nodes)}
        elif b.kind == 1:
            pts = {(0.0, 0.0): b.node_vals[0]}
        else:
            n = p.vtx[b.id]
            pts = {(float(p.nod[n, 0]), float(p.nod[n, 1])): b.node_vals[0]}

        def f(x, t, out):
            v = pts[(x[0], x[1])]
            out[0], out[1] = float(v[0]), float(v[1])
        cb = FVAL(f)
        self._cb.append(cb)
        return cb

    def fem(self):
        G, _ = libs()
        p = self.p
        ngp = 4 if p.conn.shape[1] == 4 else 1
        u = np.zeros(p.n_dof)
        strain = np.zeros(3 * ngp * p.n_elems)
        grav = (f64 * 2)(*p.gravity)
        params = Params2D(p.thickness, 0.0, b"\0")
        en = None if p.enabled is None else np.ascontiguousarray(p.enabled, np.bool_)
        st = G.nb_fem_compute_2D_Solid_Mechanics(self.mesh, self.elem, self.mat, self.bcond,
                                                 bool(p.self_weight), C.addressof(grav), 0,
                                                 C.byref(params),
                                                 None if en is None else en.ctypes.data,
                                                 u.ctypes.data, strain.ctypes.data)
        return st, u, strain

    def pipeline(self, K, F):
        """pipeline_assemble_system on the nbots matrix K and host vector F
        (as nb_fem_compute_2D_Solid_Mechanics calls it): the status."""
        G, _ = libs()
        p = self.p
        grav = (f64 * 2)(*p.gravity)
        params = Params2D(p.thickness, 0.0, b"\0")
        en = None if p.enabled is None else np.ascontiguousarray(p.enabled, np.bool_)
        self._en = en
        return G.pipeline_assemble_system(K, None, F.ctypes.data, self.mesh, self.elem,
                                          self.mat, bool(p.self_weight), C.addressof(grav), 0,
                                          C.byref(params),
                                          None if en is None else en.ctypes.data)

    def set_bconditions(self, K, F, factor=1.0):
        G, _ = libs()
        G.nb_fem_set_bconditions(self.mesh, K, F.ctypes.data, self.bcond, factor)

    def strain_of(self, u):
        G, _ = libs()
        p = self.p
        ngp = 4 if p.conn.shape[1] == 4 else 1
        out = np.zeros(3 * ngp * p.n_elems)
        u = np.ascontiguousarray(u, np.float64)
        G.pipeline_compute_strain(out.ctypes.data, self.mesh, u.ctypes.data, self.elem)
        return out

    def damage(self, ft, gf, n_steps, max_iter, max_iter_noenh, rtol, logfile):
        """nb_fem_compute_2D_Non_Linear_Solid_Mechanics through the drop-in
        symbol (conjugate-gradient branch); the log is appended to
        `logfile`."""
        G, H = libs()
        p = self.p
        H.nb_material_set_traction_limit_stress(self.mat, ft)
        H.nb_material_set_fracture_energy(self.mat, gf)
        ip = H.nb_fem_implicit_create()
        H.nb_fem_implicit_set_N_steps(ip, n_steps)
        H.nb_fem_implicit_set_N_max_iter(ip, max_iter)
        H.nb_fem_implicit_set_N_max_iter_without_enhance(ip, max_iter_noenh)
        H.nb_fem_implicit_set_residual_tolerance(ip, rtol)
        grav = (f64 * 2)(*p.gravity)
        params = Params2D(p.thickness, 0.0, b"\0")
        try:
            G.nb_fem_compute_2D_Non_Linear_Solid_Mechanics(
                self.mesh, self.elem, self.mat, self.bcond, bool(p.self_weight),
                C.addressof(grav), False, 0, C.byref(params), ip, str(logfile).encode())
        finally:
            H.nb_fem_implicit_destroy(ip)
        return G.nbg_dropin_error()

    def stress(self, strain):
        G, _ = libs()
        p = self.p
        s = np.ascontiguousarray(strain, np.float64)
        out = np.zeros_like(s)
        en = None if p.enabled is None else np.ascontiguousarray(p.enabled, np.bool_)
        G.nb_fem_compute_stress_from_strain(p.n_elems, self.elem, self.mat, 0, s.ctypes.data,
                                            None if en is None else en.ctypes.data,
                                            out.ctypes.data)
        return out

    def main_stress(self, stress):
        """pipeline_compute_main_stress through the drop-in symbol."""
        G, _ = libs()
        s = np.ascontiguousarray(stress, np.float64)
        out = np.zeros(2 * (s.size // 3))
        G.pipeline_compute_main_stress(s.ctypes.data, out.ctypes.data, self.p.n_elems, self.elem)
        return out

    def close(self):
        H = self.H
        if self.mesh:
            H.nb_mesh2D_destroy(self.mesh)
            H.nb_bcond_destroy(self.bcond)
            H.nb_material_destroy(self.mat)
            H.nb_fem_elem_destroy(self.elem)
            self.mesh = None


def nodal_graph(p: Problem):
    """nb_mesh2D_load_graph(NB_NODES_LINKED_BY_ELEMS) of a problem's mesh
    (load_graph.c:230-328), as an nb_graph_t with its buffers: both ends of
    every edge, and for elements with more than three nodes the opposite
    corners.  Built with array operations (each node's neighbours in edge
    order, then element order); nb_sparse_create sorts the rows."""
    nen = p.conn.shape[1]
    e = np.asarray(p.edges, np.int64).reshape(-1, 2)
    src = [e[:, 0], e[:, 1]]
    dst = [e[:, 1], e[:, 0]]
    if nen > 3:
        conn = np.asarray(p.conn, np.int64)
        for i in range(nen):
            for j in range(nen - 3):
                src.append(conn[:, i])
                dst.append(conn[:, (i + j + 2) % nen])
    src = np.concatenate(src)
    dst = np.concatenate(dst)
    order = np.argsort(src, kind="stable")
    n_adj = np.bincount(src, minlength=p.n_nodes).astype(np.uint32)
    flat = np.ascontiguousarray(dst[order], np.uint32)
    off = np.zeros(p.n_nodes, np.uint64)
    off[1:] = np.cumsum(n_adj[:-1], dtype=np.uint64)
    addr = np.ascontiguousarray(flat.ctypes.data + 4 * off, np.uint64)
    g = Graph(p.n_nodes, n_adj.ctypes.data_as(C.POINTER(u32)),
              C.cast(addr.ctypes.data, C.POINTER(C.POINTER(u32))), None, None)
    return g, (n_adj, flat, addr)


def sparse_from_csr(p: Problem, values):
    """nb_sparse_create on the problem's nodal graph, filled with CSR values
    in row order (one copy into the slab when the rows sit in it in order,
    as nb_sparse_create lays them out)."""
    G, _ = libs()
    g, keep = nodal_graph(p)
    A = G.nb_sparse_create(C.byref(g), None, 2)
    N = A.contents.N
    values = np.ascontiguousarray(values, np.float64)
    sizes = np.ctypeslib.as_array(A.contents.rows_size, shape=(N,)).astype(np.uint64)
    offs = np.zeros(N, np.uint64)
    offs[1:] = np.cumsum(sizes[:-1])
    rows = np.ctypeslib.as_array(C.cast(A.contents.rows_values, C.POINTER(C.c_uint64)),
                                 shape=(N,))
    base = C.cast(A.contents.rows_values[0], C.c_void_p).value
    if np.array_equal(rows, base + 8 * offs):
        C.memmove(base, values.ctypes.data, values.nbytes)
        return A, keep
    o = 0
    for i in range(N):
        n = A.contents.rows_size[i]
        row = np.ctypeslib.as_array(A.contents.rows_values[i], shape=(n,))
        row[:] = values[o:o + n]
        o += n
    return A, keep


def csr_of(A):
    N = A.contents.N
    rp = np.zeros(N + 1, np.uint32)
    cols, vals = [], []
    for i in range(N):
        n = A.contents.rows_size[i]
        rp[i + 1] = rp[i] + n
        cols.append(np.ctypeslib.as_array(A.contents.rows_index[i], shape=(n,)).copy())
        vals.append(np.ctypeslib.as_array(A.contents.rows_values[i], shape=(n,)).copy())
    return rp, np.concatenate(cols), np.concatenate(vals)
