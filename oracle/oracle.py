"""ctypes binding of the C oracle (nbots_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, ``__graft_entry__.smoke()``
and the CPU-baseline leg of bench.py, always as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "nbots_oracle.c")]
    hdr = os.path.join(HERE, "nbots_oracle.h")
    if not force and os.path.exists(SO) and all(
            os.path.getmtime(SO) >= os.path.getmtime(s) for s in src + [hdr]):
        return SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = SO + ".tmp"
    subprocess.check_call(["gcc", "-std=c99", "-O2", "-fPIC", "-fopenmp", "-shared",
                           "-o", tmp] + src + ["-lm"])
    os.replace(tmp, SO)
    return SO


class Mesh(C.Structure):
    _fields_ = [("nen", C.c_uint32), ("N_nod", C.c_uint32), ("N_elem", C.c_uint32),
                ("N_edg", C.c_uint32), ("nod", C.c_void_p), ("conn", C.c_void_p),
                ("edg", C.c_void_p)]


class BCAtom(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("where", C.c_uint32), ("id", C.c_uint32),
                ("mask", C.c_uint8 * 2), ("val", C.c_double * 2), ("n_nv", C.c_uint32),
                ("node_vals", C.c_void_p)]


class BCs(C.Structure):
    _fields_ = [("vtx", C.c_void_p), ("N_sgm", C.c_uint32), ("sgm_ptr", C.c_void_p),
                ("sgm_nodes", C.c_void_p), ("N_bc", C.c_uint32), ("bc", C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(SO)
        vp, u32, f64, i32 = C.c_void_p, C.c_uint32, C.c_double, C.c_int
        L.orc_pattern.argtypes = [vp, vp, vp]
        L.orc_assemble.argtypes = [vp, vp, vp, vp, f64, f64, f64, i32, vp, vp, vp, vp]
        L.orc_element.argtypes = [vp, u32, f64, f64, f64, f64, i32, vp, i32, vp, vp]
        L.orc_set_bconditions.argtypes = [vp, vp, vp, vp, vp, vp, f64]
        L.orc_set_dirichlet.argtypes = [vp, vp, vp, vp, u32, f64]
        L.orc_set_dirichlet.restype = None
        L.orc_spmv.argtypes = [u32, vp, vp, vp, vp, vp, i32]
        L.orc_spmv.restype = None
        L.orc_cg_jacobi.argtypes = [u32, vp, vp, vp, vp, vp, u32, f64, vp, vp, i32]
        L.orc_cg.argtypes = [u32, vp, vp, vp, vp, vp, u32, f64, vp, vp, i32]
        L.orc_strain.argtypes = [vp, vp, vp]
        L.orc_strain.restype = None
        L.orc_stress.argtypes = [vp, vp, f64, vp, vp, vp]
        L.orc_stress.restype = None
        L.orc_main_stress.argtypes = [u32, vp, vp]
        L.orc_main_stress.restype = None
        L.orc_simp_sensitivity.argtypes = [vp, f64, f64, vp, f64, f64, f64, vp, vp, vp]
        L.orc_simp_sensitivity.restype = None
        L.orc_gauss_seidel.argtypes = [u32, vp, vp, vp, vp, vp, u32, f64, vp, vp]
        L.orc_tension_damage.argtypes = [f64, f64, f64, f64, vp, f64, vp, f64]
        L.orc_tension_damage.restype = f64
        L.orc_damage_solve.argtypes = [vp, vp, f64, f64, f64, f64, i32, vp, f64, f64, u32, u32,
                                       u32, f64, C.c_char_p, C.c_size_t, vp, vp]
        L.orc_wtime.restype = f64
        L.orc_max_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


class Flat:
    """A Problem as C structs; keeps the numpy buffers alive."""

    def __init__(self, p):
        self.p = p
        self.nod = np.ascontiguousarray(p.nod, np.float64)
        self.conn = np.ascontiguousarray(p.conn, np.uint32)
        self.edg = np.ascontiguousarray(p.edges, np.uint32)
        self.mesh = Mesh(p.conn.shape[1], p.n_nodes, p.n_elems, p.edges.shape[0],
                         _p(self.nod), _p(self.conn), _p(self.edg))
        self.vtx = np.ascontiguousarray(p.vtx, np.uint32)
        lens = np.array([len(s) for s in p.sgm], np.uint32)
        self.sgm_ptr = np.zeros(len(p.sgm) + 1, np.uint32)
        self.sgm_ptr[1:] = np.cumsum(lens)
        self.sgm_nodes = (np.concatenate(p.sgm).astype(np.uint32) if p.sgm
                          else np.zeros(1, np.uint32))
        self.atoms = (BCAtom * max(1, len(p.bcs)))()
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
            else:
                a.n_nv, a.node_vals = 0, None
        self.bcs = BCs(_p(self.vtx), len(p.sgm), _p(self.sgm_ptr), _p(self.sgm_nodes),
                       len(p.bcs), C.addressof(self.atoms))
        self.E = np.ascontiguousarray(p.E, np.float64)
        self.enabled = (None if p.enabled is None
                        else np.ascontiguousarray(p.enabled, np.uint8))
        self.grav = np.array(p.gravity, np.float64)


def pattern(fl: Flat):
    L = lib()
    N = fl.p.n_dof
    rp = np.zeros(N + 1, np.uint32)
    L.orc_pattern(C.byref(fl.mesh), _p(rp), None)
    ci = np.zeros(int(rp[-1]), np.uint32)
    L.orc_pattern(C.byref(fl.mesh), _p(rp), _p(ci))
    return rp, ci


def assemble(fl: Flat, rp, ci):
    L = lib()
    p = fl.p
    K = np.zeros(ci.shape[0], np.float64)
    F = np.zeros(p.n_dof, np.float64)
    st = L.orc_assemble(C.byref(fl.mesh), _p(rp), _p(ci), _p(fl.E), p.nu, p.thickness,
                        p.density, int(p.self_weight), _p(fl.grav), _p(fl.enabled),
                        _p(K), _p(F))
    return st, K, F


def set_bconditions(fl: Flat, rp, ci, K, F, factor=1.0):
    lib().orc_set_bconditions(C.byref(fl.mesh), C.byref(fl.bcs), _p(rp), _p(ci),
                              _p(K), _p(F), factor)


def spmv(rp, ci, K, x, threads=1):
    y = np.zeros(rp.shape[0] - 1, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    lib().orc_spmv(rp.shape[0] - 1, _p(rp), _p(ci), _p(K), _p(x), _p(y), threads)
    return y


def cg_jacobi(rp, ci, K, b, x0=None, max_iter=None, tol=1e-8, threads=1, plain=False):
    N = rp.shape[0] - 1
    x = np.zeros(N) if x0 is None else np.array(x0, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    it = C.c_uint32(0)
    tr = C.c_double(0)
    fn = lib().orc_cg if plain else lib().orc_cg_jacobi
    st = fn(N, _p(rp), _p(ci), _p(K), _p(b), _p(x), N if max_iter is None else max_iter,
            tol, C.byref(it), C.byref(tr), threads)
    return x, int(it.value), float(tr.value), int(st)


def strain(fl: Flat, u):
    ngp = 4 if fl.p.conn.shape[1] == 4 else 1
    s = np.zeros(3 * ngp * fl.p.n_elems, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    lib().orc_strain(C.byref(fl.mesh), _p(u), _p(s))
    return s


def stress(fl: Flat, s):
    out = np.zeros_like(s)
    lib().orc_stress(C.byref(fl.mesh), _p(fl.E), fl.p.nu, _p(fl.enabled), _p(s), _p(out))
    return out


def main_stress(stress):
    """Principal stresses per Gauss point from (sx, sy, txy) triples
    (pipeline.c:321-340)."""
    s = np.ascontiguousarray(stress, np.float64)
    out = np.zeros(2 * (s.size // 3))
    lib().orc_main_stress(s.size // 3, _p(s), _p(out))
    return out


def element(fl: Flat, e, E=None):
    p = fl.p
    n2 = 2 * p.conn.shape[1]
    Ke = np.zeros(n2 * n2)
    Fe = np.zeros(n2)
    en = 1 if p.enabled is None else int(p.enabled[e])
    st = lib().orc_element(C.byref(fl.mesh), e, float(p.E[e] if E is None else E), p.nu,
                           p.thickness, p.density, int(p.self_weight), _p(fl.grav), en,
                           _p(Ke), _p(Fe))
    return st, Ke.reshape(n2, n2), Fe


def simp_sensitivity(fl: Flat, rho, a, b, penal=3.0, E0=1.0, Emin=1e-9):
    out = np.zeros(fl.p.n_elems)
    rho = np.ascontiguousarray(rho, np.float64)
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    lib().orc_simp_sensitivity(C.byref(fl.mesh), fl.p.nu, fl.p.thickness, _p(rho), penal,
                               E0, Emin, _p(a), _p(b), _p(out))
    return out


def fem(p, threads=1, tol=1e-8):
    """The whole nbots FEM entry on the oracle: pattern, assembly, boundary
    conditions, Jacobi-PCG (x0 = 0, max_iter = N, absolute tol 1e-8) and
    strain (static_elasticity2D.c:31-97)."""
    fl = Flat(p)
    rp, ci = pattern(fl)
    st, K, F = assemble(fl, rp, ci)
    out = dict(flat=fl, row_ptr=rp, col_idx=ci, assemble_status=st)
    if st:
        return out
    out["K_asm"], out["F_asm"] = K.copy(), F.copy()
    set_bconditions(fl, rp, ci, K, F)
    out["K_bc"], out["F_bc"] = K, F
    u, it, tr, cst = cg_jacobi(rp, ci, K, F, tol=tol, threads=threads)
    out.update(u=u, cg_niter=it, cg_tol_reached=tr, cg_status=cst)
    out["strain"] = strain(fl, u)
    return out


def gauss_seidel(rp, ci, K, b, x0=None, max_iter=None, tol=1e-8):
    """nb_sparse_solve_Gauss_Seidel (gauss_seidel.c:14-58)."""
    N = rp.shape[0] - 1
    x = np.zeros(N) if x0 is None else np.array(x0, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    it, tr = C.c_uint32(0), C.c_double(0)
    st = lib().orc_gauss_seidel(N, _p(rp), _p(ci), _p(K), _p(b), _p(x),
                                60 * N if max_iter is None else max_iter, tol,
                                C.byref(it), C.byref(tr))
    return x, int(it.value), float(tr.value), int(st)


def damage(p, ft, gf, n_steps, max_iter, max_iter_noenh, rtol, log_cap=1 << 20):
    """nbots' quasi-static damage solve (static_damage2D.c:239-470), CG path,
    material E = p.E[0].  Returns (log text, displacements, damage per Gauss
    point, number of Gauss-Seidel fallbacks)."""
    fl = Flat(p)
    ngp = 4 if p.conn.shape[1] == 4 else 1
    u = np.zeros(p.n_dof)
    d = np.zeros(ngp * p.n_elems)
    buf = C.create_string_buffer(log_cap)
    n_gs = lib().orc_damage_solve(C.byref(fl.mesh), C.byref(fl.bcs), float(p.E[0]), p.nu,
                                  p.thickness, p.density, int(p.self_weight), _p(fl.grav), ft,
                                  gf, n_steps, max_iter, max_iter_noenh, rtol, buf, log_cap,
                                  _p(u), _p(d))
    return buf.value.decode(), u, d, n_gs


def wtime():
    return lib().orc_wtime()


def max_threads():
    return lib().orc_max_threads()
