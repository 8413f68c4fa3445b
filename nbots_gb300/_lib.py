"""Loader and ctypes signatures of libnbots_gpu.so.

The library is built in-tree (nbots_gb300/build.py).  Loading fails loudly
when it is missing: there is no CPU fallback anywhere in this package.
libnbots_host.so (standalone nbots mesh / bc / material / element objects)
is loaded first with RTLD_GLOBAL so the drop-in's references to those nbots
interfaces resolve without the nbots library itself.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
GPU_SO = os.path.join(PKG, "libnbots_gpu.so")
HOST_SO = os.path.join(PKG, "libnbots_host.so")

_lib = None
_host = None

vp, u32, u64, f64, i32, sz = (C.c_void_p, C.c_uint32, C.c_uint64, C.c_double, C.c_int,
                              C.c_size_t)


class CgResult(C.Structure):
    _fields_ = [("niter", C.c_uint32), ("status", C.c_int), ("tol_reached", C.c_double),
                ("bnorm", C.c_double)]


class MixedResult(C.Structure):
    _fields_ = [("niter", C.c_uint32), ("n_updates", C.c_uint32), ("status", C.c_int),
                ("relres", C.c_double), ("bnorm", C.c_double)]


class Bsr(C.Structure):
    _fields_ = [("N", u32), ("Nn", u32), ("n_slices", u32), ("n_entries", u64),
                ("slice_off", vp), ("bcol", vp), ("b64", vp), ("b32", vp), ("blo", vp), ("bxt", vp), ("dinv64", vp),
                ("dinv32", vp), ("perm", vp), ("iperm", vp)]


class SolveInfo(C.Structure):
    _fields_ = [("niter", C.c_uint32), ("n_updates", C.c_uint32), ("status", C.c_int),
                ("relres", C.c_double), ("tol_reached", C.c_double)]


class SimpInfo(C.Structure):
    _fields_ = [("J", C.c_double), ("fwd_iters", C.c_uint32), ("adj_iters", C.c_uint32),
                ("status", C.c_int)]


class GsResult(C.Structure):
    _fields_ = [("niter", C.c_uint32), ("status", C.c_int), ("error", C.c_double)]


class DamageInfo(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("cg_solves", C.c_uint32),
                ("cg_iterations", C.c_uint32), ("gs_fallbacks", C.c_uint32),
                ("gs_failures", C.c_uint32), ("residual", C.c_double)]


class Mesh(C.Structure):
    _fields_ = [("nen", u32), ("N_nod", u32), ("N_elem", u32), ("N_edg", u32),
                ("nod", vp), ("conn", vp), ("edg", vp)]


class BCAtom(C.Structure):
    _fields_ = [("kind", u32), ("where", u32), ("id", u32), ("mask", C.c_uint8 * 2),
                ("val", C.c_double * 2), ("n_nv", u32), ("node_vals", vp)]


class BCs(C.Structure):
    _fields_ = [("vtx", vp), ("N_sgm", u32), ("sgm_ptr", vp), ("sgm_nodes", vp),
                ("N_bc", u32), ("bc", vp)]


SIGS = {
    "nbg_version": ([], C.c_char_p),
    "nbg_last_error": ([], C.c_char_p),
    "nbg_device_count": ([], i32),
    "nbg_dev_alloc": ([C.POINTER(vp), sz], i32),
    "nbg_dev_free": ([vp], i32),
    "nbg_h2d": ([vp, vp, sz, vp], i32),
    "nbg_d2h": ([vp, vp, sz, vp], i32),
    "nbg_memset": ([vp, i32, sz, vp], i32),
    "nbg_stream_sync": ([vp], i32),
    "nbg_host_memory_access": ([], i32),
    "nbg_wait_flag": ([vp, i32, u64, vp, vp], i32),
    "nbg_element_stiffness_f64": ([u32, u32, vp, vp, vp, f64, f64, f64, i32, f64, f64, vp, vp,
                                   vp, vp, vp], i32),
    "nbg_element_stiffness_damage_f64": ([u32, u32, vp, vp, vp, f64, f64, f64, i32, f64, f64,
                                          vp, vp, vp, vp, vp, vp], i32),
    "nbg_strain_damage_f64": ([u32, u32, vp, vp, vp, f64, f64, f64, f64, vp, vp, vp, vp, vp, vp],
                              i32),
    "nbg_residual_workspace_bytes": ([u32], sz),
    "nbg_residual_f64": ([u32, vp, vp, vp, vp, vp, vp, vp, vp, vp], i32),
    "nbg_add_to_f64": ([u32, vp, vp, vp], i32),
    "nbg_host_lower_levels": ([u32, vp, vp, vp, vp, C.POINTER(u32)], i32),
    "nbg_gauss_seidel_workspace_bytes": ([u32], sz),
    "nbg_gauss_seidel_f64": ([u32, vp, vp, vp, vp, vp, vp, vp, u32, u32, f64, f64,
                              C.POINTER(GsResult), vp, vp], i32),
    "nbg_fem_damage": ([vp, vp, f64, f64, f64, f64, i32, vp, f64, f64, u32, u32, u32, f64,
                        i32, C.c_char_p, C.POINTER(DamageInfo)], i32),
    "nbg_gather_assemble_f64": ([u32, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp],
                                i32),
    "nbg_apply_increments_f64": ([u32, vp, vp, vp, vp, vp], i32),
    "nbg_dirichlet_f64": ([u32, vp, vp, vp, vp, vp, vp, vp, vp, vp], i32),
    "nbg_strain_f64": ([u32, u32, vp, vp, vp, vp, vp], i32),
    "nbg_stress_f64": ([u32, u32, vp, f64, vp, vp, vp, vp], i32),
    "nbg_main_stress_f64": ([u32, u32, vp, vp, vp], i32),
    "nbg_fem_main_stress": ([vp], i32),
    "nbg_spmv_csr_f64": ([u32, vp, vp, vp, vp, vp, vp], i32),
    "nbg_cg_workspace_bytes": ([u32], sz),
    "nbg_cg_f64": ([u32, vp, vp, vp, vp, vp, u32, f64, C.c_uint, C.POINTER(CgResult), vp, sz,
                    vp], i32),
    "nbg_cg_f64_noalloc": ([u32, vp, vp, vp, vp, vp, u32, f64, C.c_uint, C.POINTER(CgResult),
                            vp], i32),
    "nbg_bsr_plan": ([u32, vp, vp, vp], i32),
    "nbg_bsr_fill": ([C.POINTER(Bsr), vp, vp, vp, vp], i32),
    "nbg_spmv_bsr_f64": ([C.POINTER(Bsr), vp, vp, vp], i32),
    "nbg_spmv_bsr_f32": ([C.POINTER(Bsr), vp, vp, vp], i32),
    "nbg_cg_bsr_workspace_bytes": ([u32], sz),
    "nbg_cg_bsr_f64": ([C.POINTER(Bsr), vp, vp, u32, f64, C.c_uint, C.POINTER(CgResult), vp,
                        sz, vp], i32),
    "nbg_spmv_bsr_mixed": ([C.POINTER(Bsr), vp, vp, vp, vp, vp], i32),
    "nbg_cg_mixed_workspace_bytes": ([u32], sz),
    "nbg_cg_mixed_layout_workspace_bytes": ([C.POINTER(Bsr)], sz),
    "nbg_cg_mixed_last_form": ([], i32),
    "nbg_cg_mixed": ([C.POINTER(Bsr), vp, vp, u32, f64, f64, C.c_uint,
                      C.POINTER(MixedResult), vp, sz, vp], i32),
    "nbg_fem_block_layout": ([vp, C.POINTER(Bsr)], i32),
    "nbg_fem_set_block_order": ([vp, i32, u32], i32),
    "nbg_bsr_plan_sigma_dev": ([u32, vp, u32, vp, vp, vp, vp], i32),
    "nbg_d2d": ([vp, vp, sz, vp], i32),
    "nbg_fem_solve_fast": ([vp, u32, f64, C.c_uint, C.POINTER(CgResult)], i32),
    "nbg_fem_solve_mixed": ([vp, u32, f64, f64, C.c_uint, C.POINTER(MixedResult)], i32),
    "nbg_solver_create": ([C.POINTER(vp), vp], i32),
    "nbg_solver_destroy": ([vp], None),
    "nbg_solver_set_matrix": ([vp, u32, vp, vp, vp, C.c_uint], i32),
    "nbg_solver_solve": ([vp, vp, vp, u32, f64, C.c_uint, i32, C.POINTER(SolveInfo)], i32),
    "nbg_host_alloc": ([C.POINTER(vp), sz], i32),
    "nbg_host_free": ([vp], i32),
    "nbg_simp_modulus_f64": ([u32, vp, f64, f64, f64, vp, vp], i32),
    "nbg_simp_sensitivity_f64": ([u32, u32, vp, vp, f64, f64, vp, f64, f64, f64, vp, vp, vp,
                                  vp], i32),
    "nbg_fem_simp": ([vp, vp, vp, f64, f64, f64, f64, f64, i32, u32, f64, i32, vp,
                      C.POINTER(SimpInfo)], i32),
    "nbg_host_pattern": ([vp, vp, vp], i32),
    "nbg_host_incidence": ([vp, vp, vp, vp], i32),
    "nbg_pattern_dev": ([u32, u32, u32, u32, vp, vp, vp, C.POINTER(vp), C.POINTER(u64), vp, vp,
                         vp, vp, vp], i32),
    "nbg_fem_create": ([C.POINTER(vp), vp, vp], i32),
    "nbg_fem_destroy": ([vp], None),
    "nbg_fem_n_dof": ([vp], u32),
    "nbg_fem_nnz": ([vp], u64),
    "nbg_fem_assemble": ([vp, vp, f64, f64, f64, i32, vp, vp], i32),
    "nbg_fem_apply_bcs": ([vp, vp, f64], i32),
    "nbg_fem_solve": ([vp, u32, f64, C.c_uint, C.POINTER(CgResult)], i32),
    "nbg_fem_strain": ([vp], i32),
    "nbg_fem_stress": ([vp], i32),
    "nbg_fem_device_ptr": ([vp, i32], vp),
    "nbg_fem_bytes": ([vp, i32], sz),
    "nbg_fem_download": ([vp, i32, vp], i32),
    "nbg_fem_upload": ([vp, i32, vp], i32),
    "nbg_mixed_batch_create": ([C.POINTER(vp), C.POINTER(Bsr), vp, vp, u32, vp, u32, f64, f64,
                                C.c_uint, vp], i32),
    "nbg_mixed_batch_destroy": ([vp], None),
    "nbg_mixed_batch_plan": ([vp, f64], i32),
    "nbg_mixed_batch_blocks": ([vp, vp, C.POINTER(f64)], u32),
    "nbg_mixed_batch_set_sensitivity": ([vp, u32, u32, vp, vp, f64, f64, vp, f64, f64, f64, vp],
                                        i32),
    "nbg_mixed_batch_launch": ([vp], i32),
    "nbg_mixed_batch_results": ([vp, vp, vp], i32),
    "nbg_mixed_batch_tune": ([vp, u32, vp, vp], i32),
    "nbg_batch_create": ([C.POINTER(vp), u32, vp, vp, vp], i32),
    "nbg_batch_destroy": ([vp], None),
    "nbg_batch_size": ([vp], u32),
    "nbg_batch_offsets": ([vp, vp, vp], i32),
    "nbg_batch_fem": ([vp], vp),
    "nbg_batch_solver": ([vp], vp),
    "nbg_batch_assemble_simp": ([vp, vp, f64, f64, f64, f64, f64], i32),
    "nbg_batch_setup": ([vp, u32, f64, f64, C.c_uint], i32),
    "nbg_batch_launch": ([vp], i32),
    "nbg_batch_results": ([vp, vp, vp], i32),
    "nbg_batch_sensitivities": ([vp, vp], i32),
}

(FEM_ROW_PTR, FEM_COL_IDX, FEM_K, FEM_F, FEM_U, FEM_STRAIN, FEM_STRESS, FEM_E, FEM_NOD,
 FEM_CONN, FEM_MAIN_STRESS, FEM_DAMAGE) = range(12)
CG_JACOBI, CG_RELATIVE, CG_NBOTS_STOP = 1, 2, 4
ORDER_AUTO, ORDER_MESH, ORDER_SIGMA = 0, 1, 2
METHOD_NBOTS, METHOD_FP64, METHOD_MIXED, METHOD_NBOTS_FAST = 0, 1, 2, 3
PATTERN_SAME = 1


def lib():
    """The loaded libnbots_gpu.so with argtypes set; raises if not built."""
    global _lib, _host
    if _lib is not None:
        return _lib
    if not os.path.exists(GPU_SO):
        raise RuntimeError(f"{GPU_SO} is missing: run nbots_gb300.build.build() first "
                           "(the CUDA path has no fallback)")
    if os.path.exists(HOST_SO):
        _host = C.CDLL(HOST_SO, mode=C.RTLD_GLOBAL)
    L = C.CDLL(GPU_SO, mode=C.RTLD_GLOBAL)
    for name, (args, res) in SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def host_lib():
    lib()
    return _host


def check(rc, what=""):
    if rc != 0:
        err = lib().nbg_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed with status {rc} {err}")
    return rc
