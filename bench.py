#!/usr/bin/env python
"""Benchmark of the nbots FEM hot path on GB300.

Workload (one GPU): 1024x512 Q4 plane-stress cantilever on [0,2]x[0,1],
1,051,650 dof, per-element E = exp(N(0, 0.5^2)) (seed 2), nu = 0.3, left
edge clamped, unit downward point load at the right-edge midpoint plus a
uniform downward traction 0.01 on the top edge.  Synthetic, seeded inputs:
nbots has no public benchmark set.

A step is one solve of K u = F from u = 0 to ||F - K u|| <= 1e-8 ||F|| (true
FP64 residual) with the mixed-precision Jacobi-PCG (FP32 inner iteration,
FP64 reliable updates); the metric is the time per step.  Beside it the line
carries the plain FP64 GPU CG, nbots' own FP64 iteration on the GPU, the SpMV
bandwidths, the end-to-end time through the host-buffer C ABI, the roofline
of the solver kernel and a CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference nbots' own Jacobi-PCG (cg_precond_jacobi.c:13-90)
runs on the host cores (OpenMP, all threads) to convergence in every step:
the library built from the nbots sources (oracle/_ref) where it exists on
the machine, else the oracle's C restatement of the same loop.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 vs mixed-prec time-to-1e-8 relres at 1M DOF (s); SpMV HBM GB/s vs peak"
WORKLOAD = ("C2: 1024x512 Q4 cantilever, 1,051,650 dof, lognormal E (sigma 0.5, seed 2), "
            "clamped left edge, point load + top traction 0.01; Jacobi-PCG to relres 1e-8 from u=0")
TOL = 1e-8


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,"
                 "power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 4 + k and r[4 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU
def mixed_blocks(n_slices, dev):
    """Blocks of the single-system mixed launch: one per SM, at most one per
    32 slices (the solver's own rule)."""
    import torch
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    return max(1, min(nsm, (n_slices + 31) // 32))


def ghost_count(rp, ci, n_slices, G):
    """Ghost node rows over all blocks of a G-block partition of the slices
    (what the solver's plan finds): per block, the distinct column nodes of
    its rows outside its own row slots."""
    rows = np.repeat(np.arange(rp.shape[0] - 1, dtype=np.int64) // 2,
                     np.diff(rp).astype(np.int64))
    cols = ci.astype(np.int64) // 2
    s_of_block = (n_slices * np.arange(G + 1, dtype=np.int64)) // G
    blk = np.searchsorted(s_of_block, rows // 32, side="right") - 1
    lo, hi = 32 * s_of_block[blk], 32 * s_of_block[blk + 1]
    out = (cols < lo) | (cols >= hi)
    key = blk[out] * (int(cols.max()) + 1) + cols[out]
    return int(np.unique(key).size)


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


class CpuSystem:
    """The C2 system (K and F after boundary conditions) on the host, built by
    the oracle (setup, not timed), with nbots' own SpMV and Jacobi-PCG from
    the library built from its sources when it loads here, else the oracle's
    C restatement of the same loops."""

    def __init__(self, p, threads=None):
        from oracle import oracle as O
        from oracle import ref_cpu as R
        self.O, self.R = O, R
        self.threads = threads or os.cpu_count() or 1
        fl = O.Flat(p)
        self.rp, self.ci = O.pattern(fl)
        _, self.K, self.F = O.assemble(fl, self.rp, self.ci)
        O.set_bconditions(fl, self.rp, self.ci, self.K, self.F)
        self.tol = TOL * float(np.linalg.norm(self.F))  # nbots' tolerance is absolute
        self.kind = "reference" if R.available() else "port"
        self.m = R.Matrix(self.rp, self.ci, self.K) if self.kind == "reference" else None

    def what(self):
        return ("nbots' own code (oracle/_ref/libnbots_ref.so, built from the nbots sources)"
                if self.kind == "reference" else
                "the oracle's C restatement of nbots' loops (nbots_oracle.c)")

    def spmv(self, x):
        if self.m is not None:
            return self.R.spmv(self.m, x, self.threads)
        return self.O.spmv(self.rp, self.ci, self.K, x, self.threads)

    def cg(self, max_iter=None):
        """One Jacobi-PCG from x = 0 with nbots' absolute tolerance
        1e-8 ||F||: (seconds, iterations, status)."""
        t0 = time.perf_counter()
        if self.m is not None:
            _, it, _, st = self.R.cg_jacobi(self.m, self.F, self.tol, self.threads,
                                            max_iter=max_iter)
        else:
            _, it, _, st = self.O.cg_jacobi(self.rp, self.ci, self.K, self.F,
                                            max_iter=max_iter, tol=self.tol,
                                            threads=self.threads)
        return time.perf_counter() - t0, it, st

    def spmv_median(self, reps=7):
        x = np.random.default_rng(7).standard_normal(self.F.shape[0])
        self.spmv(x)
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            self.spmv(x)
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts))


def cpu_baseline(p):
    """nbots' Jacobi-PCG run to convergence once on the full workload on the
    host cores, and the median of 7 SpMVs (sparse.c:405-414)."""
    cs = CpuSystem(p)
    cs.cg(max_iter=20)  # threads and pages warm
    t_cg, it, st = cs.cg()
    t_spmv = cs.spmv_median()
    nnz, N = cs.ci.shape[0], cs.F.shape[0]
    b_spmv = 12 * nnz + 4 * (N + 1) + 16 * N
    return {"value": t_cg, "unit": "s", "cores": cs.threads, "kind": cs.kind,
            "cpu": cpu_model(), "iters": it, "status": st,
            "spmv_ms_median_of_7": t_spmv * 1e3, "spmv_gbs": b_spmv / t_spmv / 1e9,
            "sample": f"one full Jacobi-PCG solve to ||g|| <= 1e-8 ||F|| from u = 0 ({it} "
                      f"iterations) with {cs.what()}, OpenMP {cs.threads} threads; SpMV: "
                      f"median of 7"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from nbots_gb300 import workloads as W
    p = W.config_c2()
    cs = CpuSystem(p)
    # warm-up steps: bounded solves (threads, pages and caches warm); each
    # timed step is one full solve to the tolerance
    for _ in range(args.warmup):
        cs.cg(max_iter=50)
    runs = [cs.cg() for _ in range(args.steps)]
    ts = [r[0] for r in runs]
    v = float(np.median(ts))
    cb = {"value": v, "unit": "s", "cores": cs.threads, "kind": cs.kind, "cpu": cpu_model(),
          "iters": runs[0][1], "status": runs[0][2], "s_min_max": [min(ts), max(ts)],
          "sample": f"every step one full Jacobi-PCG solve to ||g|| <= 1e-8 ||F|| from u = 0 "
                    f"({runs[0][1]} iterations) with {cs.what()}, OpenMP {cs.threads} "
                    f"threads; warm-up steps: 50 iterations each"}
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD}, "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU
def bench_c4(lib, L, W):
    """SIMP gradients on the 512x256 grid (rho ~ U(0.3,0.7), p = 3): wall time
    of one objective + gradient through nbg_fem_simp (assembly, boundary
    conditions, forward solve, adjoint solve for the one-dof objective,
    sensitivity kernel, copies), mixed precision and FP64 at relres 1e-8,
    and the mixed gradients' deviation from FP64 ones at relres 1e-12."""
    from nbots_gb300.simp import COMPLIANCE, DOF, SimpProblem
    p = W.config_c4()
    rho = p.meta["rho"]
    nx, ny = p.meta["nx"], p.meta["ny"]
    dof = 2 * ((ny // 2) * (nx + 1) + nx)  # x-displacement of the right-edge midpoint
    out = {"workload": f"C4: {nx}x{ny} Q4 SIMP, {p.n_dof} dof, rho~U(0.3,0.7) seed 4, p=3, "
                       "Emin=1e-9, E0=1; objectives compliance and u_x of the right-edge "
                       "midpoint"}
    ref = SimpProblem(p, tol=1e-12, method=L.METHOD_FP64)
    for name, obj in (("compliance", COMPLIANCE), ("u_x_output", DOF)):
        _, g64, _ = ref.evaluate(rho, obj, dof)
        row = {}
        for mname, m in (("mixed", L.METHOD_MIXED), ("fp64", L.METHOD_FP64)):
            sp_ = SimpProblem(p, tol=1e-8, method=m)
            sp_.evaluate(rho, obj, dof)  # warm
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                J, g, info = sp_.evaluate(rho, obj, dof)
                ts.append(time.perf_counter() - t0)
            row[mname] = {"s_per_gradient": float(np.median(ts)), "fwd_iters": info.fwd_iters,
                          "adj_iters": info.adj_iters,
                          "grad_dev_vs_fp64_1e-12": float(np.max(np.abs(g - g64)) /
                                                          np.max(np.abs(g64)))}
            sp_.close()
        out[name] = row
    ref.close()
    return out


def _damage_step_iters(log):
    """Residual evaluations per load step of an nbots damage log."""
    out = []
    for line in log.splitlines():
        if "Load step" in line:
            out.append(0)
        elif "Residual" in line:
            out[-1] += 1
    return out


def bench_damage(L, W, with_cpu):
    """nbots' quasi-static damage solve (static_damage2D.c:239-470) on a
    cantilever under a uniform top traction: 4 load steps, at most 40
    iterations each, 6 without a new best residual, residual tolerance
    1e-7, ft = 6, Gf = 10, E = 1.  Wall time of nbg_fem_damage (device
    assembly with damage, boundary conditions, residual, Jacobi-PCG with
    nbots' iteration and stop test on the block layout (the drop-in's inner
    solver), strain and damage, host log) against the oracle's one-thread
    restatement of nbots' loop on the same problem; and the same device loop
    with nbots' operation order on the CSR and with the fast FP64 block CG
    as its inner solver."""
    import tempfile
    from nbots_gb300.fem import FemSystem
    out = {}
    args_ = (6.0, 10.0, 4, 40, 6, 1e-7)
    for method in (L.METHOD_NBOTS_FAST, L.METHOD_NBOTS, L.METHOD_FP64):  # warm the modules
        s = FemSystem(W.cantilever_q4(16, 8, point_load=0.0, top_traction=0.35))
        s.damage(*args_, method=method)
        s.close()
    for nx, ny, cpu in ((128, 64, with_cpu), (512, 256, False)):
        p = W.cantilever_q4(nx, ny, point_load=0.0, top_traction=0.35)
        row = {"workload": f"Q4 cantilever {nx}x{ny}, {p.n_dof} dof, top traction 0.35"}
        for method, key in ((L.METHOD_NBOTS_FAST, "nbots_iteration_block_cg"),
                            (L.METHOD_NBOTS, "nbots_order_cg"), (L.METHOD_FP64, "fast_fp64_cg")):
            s = FemSystem(p)
            with tempfile.TemporaryDirectory() as td:
                logf = os.path.join(td, "dmg.log")
                t0 = time.perf_counter()
                info = s.damage(*args_, logfile=logf, method=method)
                t_gpu = time.perf_counter() - t0
                log = open(logf).read()
            s.close()
            res = {"gpu_s": t_gpu, "iterations": info.iterations,
                   "cg_solves": info.cg_solves, "cg_iterations": info.cg_iterations,
                   "gs_fallbacks": info.gs_fallbacks,
                   "step_iterations": _damage_step_iters(log)}
            if method == L.METHOD_NBOTS_FAST:
                row.update(res)  # the drop-in's inner solver: the row's headline
            else:
                row[key] = res
        if cpu:
            from oracle import oracle as O
            t0 = time.perf_counter()
            olog, _, _, _ = O.damage(p, *args_)
            t_cpu = time.perf_counter() - t0
            row.update(cpu_oracle_s=t_cpu, cpu_cores=1,
                       cpu_step_iterations=_damage_step_iters(olog),
                       speedup=t_cpu / row["gpu_s"])
        out[f"{nx}x{ny}"] = row
    return out


def bench_fem_entry(W, with_cpu):
    """nbots' FEM entry through the drop-in symbol (nb_fem_compute_2D_Solid_
    Mechanics with nbots' objects built by the host library): the 1024x512
    cantilever with one material (E = 1, the entry takes one), host arrays in
    and out, pattern, assembly, boundary conditions, nbots' Jacobi-PCG
    iteration (x0 = 0, max_iter = N, absolute 1e-8) and strain, wall time.
    Beside it the same entry on the host as nbots ships it, one thread
    (static_elasticity2D.c:88-90), on the oracle's restatement of each stage."""
    from nbots_gb300.dropin import NbotsObjects
    warm = NbotsObjects(W.cantilever_q4(16, 8))
    warm.fem()
    warm.close()
    p = W.config_c2()
    p.E = np.ones(p.n_elems)
    ob = NbotsObjects(p)
    t0 = time.perf_counter()
    st, u, strain = ob.fem()
    t = time.perf_counter() - t0
    ob.close()
    out = {"workload": "C2 mesh and loads, one material E = 1", "status": int(st),
           "s_per_call": t, "max_abs_u": float(np.max(np.abs(u)))}
    if with_cpu:
        from oracle import oracle as O
        t0 = time.perf_counter()
        ref = O.fem(p, threads=1)
        t_cpu = time.perf_counter() - t0
        out["cpu_one_thread"] = {
            "s_per_call": t_cpu, "kind": "port", "cores": 1, "cg_iters": ref["cg_niter"],
            "u_rel_diff_vs_dropin": float(np.linalg.norm(u - ref["u"]) /
                                          np.linalg.norm(ref["u"])),
            "sample": "one call: pattern, assembly, boundary conditions, Jacobi-PCG to "
                      "absolute 1e-8, strain, on the oracle's C restatement, one thread"}
        out["speedup_vs_cpu_one_thread"] = t_cpu / t
    return out


def bench_dropin_sparse(W, cpu_spmv_s=None):
    """nb_sparse_multiply_vector and nb_sparse_solve_CG_precond_Jacobi called
    as nbots calls them: an nb_sparse_t from nb_sparse_create holding K after
    boundary conditions of the C2 system, host vectors in and out.  The first
    call on the matrix builds its device copy; later calls on the unchanged
    matrix send only the vectors.  After one nb_sparse_add the next call
    re-sends the values."""
    from nbots_gb300.dropin import libs, sparse_from_csr
    from oracle import oracle as O
    G, _ = libs()
    p = W.config_c2()
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    _, K, F = O.assemble(fl, rp, ci)
    O.set_bconditions(fl, rp, ci, K, F)
    A, keep = sparse_from_csr(p, K)
    N = p.n_dof
    x = np.random.default_rng(11).standard_normal(N)
    y = np.zeros(N)

    def spmv():
        t0 = time.perf_counter()
        G.nb_sparse_multiply_vector(A, x.ctypes.data, y.ctypes.data, 1)
        return time.perf_counter() - t0
    t_first = spmv()
    ts = [spmv() for _ in range(7)]
    exact = bool(np.array_equal(y.view(np.uint64), O.spmv(rp, ci, K, x, 8).view(np.uint64)))
    r0 = A.contents.rows_values[0][0]
    G.nb_sparse_add(A, 0, int(ci[0]), 0.0)  # a write: the next call re-sends the values
    t_dirty = spmv()
    G.nb_sparse_set(A, 0, int(ci[0]), r0)
    tol = TOL * float(np.linalg.norm(F))
    it, tr = C.c_uint32(0), C.c_double(0)

    def cg():
        u = np.zeros(N)
        t0 = time.perf_counter()
        st = G.nb_sparse_solve_CG_precond_Jacobi(A, F.ctypes.data, u.ctypes.data, N, tol,
                                                  C.byref(it), C.byref(tr), 1)
        return time.perf_counter() - t0, st, u
    t_cg_first, _, _ = cg()
    t_cg, st, u = cg()
    relres = float(np.linalg.norm(F - O.spmv(rp, ci, K, u, 8)) / np.linalg.norm(F))
    G.nb_sparse_destroy(A)
    t_spmv = float(np.median(ts))
    out = {"workload": "C2 K and F after boundary conditions in an nb_sparse_t, host vectors",
           "spmv": {"s_first_call": t_first, "s_median_of_7": t_spmv,
                    "s_after_one_write": t_dirty, "bit_exact": exact,
                    "h2d_bytes": 8 * N, "d2h_bytes": 8 * N},
           "cg_jacobi": {"s_first_call": t_cg_first, "s_per_call": t_cg, "status": int(st),
                         "iters": it.value, "relres_fp64": relres,
                         "h2d_bytes": 16 * N, "d2h_bytes": 8 * N,
                         "stop": "nbots' (absolute 1e-8 ||F||, lagged test)"}}
    if cpu_spmv_s:
        out["spmv"]["speedup_vs_cpu_spmv"] = cpu_spmv_s / t_spmv
    return out


def bench_c5(args, lib, L, W, sp, dev, stream, flush, share=None):
    """96 batched SIMP cantilevers: one graph launch = zero u, batched mixed
    CG to relres 1e-8 per instance, compliance sensitivities.  Per-instance
    errors against an FP64 solve of the same merged system to relres 1e-13."""
    import torch
    from nbots_gb300.batch import Batch
    t0 = time.perf_counter()
    probs = W.config_c5()
    n_all = len(probs)
    if share is not None:  # this rank's instances
        probs = [probs[k] for k in share]
    b = Batch(probs, stream=sp)
    rho = [p.meta["rho"] for p in probs]
    b.assemble_simp(rho, nu=probs[0].nu, thickness=probs[0].thickness)
    b.setup(max_iter=100000, tol=TOL)
    t_setup = time.perf_counter() - t0
    gammas = (1.0, 1.25, 1.5, 1.75, 2.0)
    ms = b.tune(gammas)
    G, blocks, gamma = b.blocks()
    for _ in range(args.warmup):
        b.launch()
    ts = []
    for _ in range(args.steps):
        flush.fill_(4.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.launch()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    res, J = b.results()
    from nbots_gb300 import replicas as R
    t_all = R.max_over_ranks([float(np.median(ts))], device=dev)[0]  # the slowest share
    us = b.displacements()
    dJ = b.sensitivities()
    t = float(np.median(ts))
    # FP64 reference on the merged system
    A = L.Bsr()
    L.check(lib.nbg_fem_block_layout(b.fem, C.byref(A)), "block_layout")
    N = b.n_dof
    u64 = torch.zeros(N, dtype=torch.float64, device=dev)
    wsb = lib.nbg_cg_bsr_workspace_bytes(N)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    r64 = L.CgResult()
    Fd = lib.nbg_fem_device_ptr(b.fem, L.FEM_F)
    rc = lib.nbg_cg_bsr_f64(C.byref(A), Fd, u64.data_ptr(), 200000, 1e-13,
                            L.CG_JACOBI | L.CG_RELATIVE, C.byref(r64), ws.data_ptr(), wsb, sp)
    # relres 1e-13, or the FP64 floor of the merged system (below 1e-10)
    assert rc == 0 or (rc == 1 and r64.tol_reached <= 1e-10 * r64.bnorm), rc
    rho_d = torch.from_numpy(np.concatenate(rho)).to(dev)
    g64 = torch.empty(b.n_elems, dtype=torch.float64, device=dev)
    L.check(lib.nbg_simp_sensitivity_f64(4, b.n_elems, lib.nbg_fem_device_ptr(b.fem, L.FEM_NOD),
                                         lib.nbg_fem_device_ptr(b.fem, L.FEM_CONN),
                                         probs[0].nu, probs[0].thickness, rho_d.data_ptr(), 3.0,
                                         1.0, 1e-9, u64.data_ptr(), u64.data_ptr(),
                                         g64.data_ptr(), sp), "sensitivity")
    torch.cuda.synchronize()
    u64h, g64h = u64.cpu().numpy(), g64.cpu().numpy()
    Fh = b.merged(L.FEM_F)
    eu, eJ, eg, eu64 = [], [], [], []
    from nbots_gb300.fem import FemSystem
    for k, p in enumerate(probs):
        n0 = 2 * int(b.node_off[k])
        uk = u64h[n0:n0 + p.n_dof]
        eu.append(float(np.linalg.norm(us[k] - uk) / np.linalg.norm(uk)))
        # the FP64 CG stopped at the same relres 1e-8, against the same
        # converged solution: the error the tolerance itself allows
        fs = FemSystem(p)
        assert fs.assemble() == 0
        fs.apply_bcs()
        assert fs.solve_fast(tol=TOL).status == 0
        eu64.append(float(np.linalg.norm(fs.get(L.FEM_U) - uk) / np.linalg.norm(uk)))
        fs.close()
        Jk = float(Fh[n0:n0 + p.n_dof] @ uk)
        eJ.append(abs(J[k] - Jk) / abs(Jk))
        gk = g64h[int(b.elem_off[k]):int(b.elem_off[k + 1])]
        eg.append(float(np.max(np.abs(dJ[k] - gk)) / np.max(np.abs(gk))))
    iters = [r.niter for r in res]
    out = {"workload": "C5: 96 Q4 SIMP cantilevers, sizes U{64x32,128x64,256x128,512x256} "
                       "seed 5, rho~U(0.2,1.0), 1-4 point loads; mixed CG to relres 1e-8 per "
                       "instance + compliance gradients, one CUDA graph launch",
           "instances": n_all, "instances_rank0": len(probs),
           "dof_total_rank0": int(sum(p.n_dof for p in probs)),
           "dof_merged_padded_rank0": N, "s_per_batch": t_all, "solves_per_s": n_all / t_all,
           "ranks_sharing_the_batch": R.world()[1],
           "dof_iters_per_s_rank0": float(sum(p.n_dof * r.niter for p, r in zip(probs, res)))
                                    / t,
           "status_all_zero": all(r.status == 0 for r in res),
           "iters_min_max": [min(iters), max(iters)],
           "max_relres": max(r.relres for r in res),
           "err_u_vs_fp64_rel_l2_max": max(eu), "err_u_vs_fp64_rel_l2_median":
               float(np.median(eu)),
           "err_u_fp64_cg_at_same_tol_max": max(eu64),
           "err_u_fp64_cg_at_same_tol_median": float(np.median(eu64)),
           "err_note": "errors against FP64 solves to relres 1e-13 of the same systems; the "
                       "FP64 CG stopped at the same relres 1e-8 shows the error the tolerance "
                       "allows on these ill-conditioned SIMP systems",
           "err_compliance_vs_fp64_max": max(eJ), "err_grad_vs_fp64_max": max(eg),
           "fp64_reference_iters": r64.niter,
           "autotune": {"gammas": list(gammas), "ms": [float(x) for x in ms], "chosen": gamma,
                        "blocks": G, "blocks_min_max": [int(blocks.min()), int(blocks.max())]},
           "setup_s": t_setup, "gpu_launches_per_batch": 2,
           "l2": "flushed (512 MB write) before every timed launch"}
    b.close()
    return out


def bench_c3(args, with_cpu):
    """The unstructured T3 L-shape (2M seeded points, about 4M dof): mesh
    generation (host, not timed), pattern + upload, assembly + boundary
    conditions, then mixed-precision and fast FP64 Jacobi-PCG to relres 1e-8
    from u = 0 (CUDA events, L2 flushed before each solve), the mixed
    solution's distance from the FP64 one, and nbots' CPU iteration on the
    host cores timed over 200 iterations (per iteration beside the GPU's;
    a full CPU solve takes about two minutes)."""
    import torch
    from nbots_gb300 import _lib as L
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem
    lib = L.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    t0 = time.perf_counter()
    p = W.config_c3()
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    s = FemSystem(p, stream=sp)
    t_create = time.perf_counter() - t0
    t0 = time.perf_counter()
    assert s.assemble() == 0
    s.apply_bcs()
    A = s.block_layout()
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    N, nnz = s.N, s.nnz
    F = s.dptr(L.FEM_F)
    u = torch.zeros(N, dtype=torch.float64, device=dev)
    ws_bytes = max(lib.nbg_cg_mixed_layout_workspace_bytes(C.byref(A)),
                   lib.nbg_cg_bsr_workspace_bytes(N))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def solve(kind):
        u.zero_()
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if kind == "mixed":
            r = L.MixedResult()
            rc = lib.nbg_cg_mixed(C.byref(A), F, u.data_ptr(), 8 * N, TOL, 0.1,
                                  L.CG_JACOBI | L.CG_RELATIVE, C.byref(r), ws.data_ptr(),
                                  ws_bytes, sp)
        else:
            r = L.CgResult()
            rc = lib.nbg_cg_bsr_f64(C.byref(A), F, u.data_ptr(), 8 * N, TOL,
                                    L.CG_JACOBI | L.CG_RELATIVE, C.byref(r), ws.data_ptr(),
                                    ws_bytes, sp)
        e1.record(stream)
        e1.synchronize()
        assert rc == 0 and r.status == 0, (kind, rc, r.status)
        return e0.elapsed_time(e1) / 1e3, r
    solve("mixed")
    tm = [solve("mixed") for _ in range(max(1, args.steps))]
    u_mixed = u.clone()
    tf = [solve("fp64") for _ in range(max(1, min(args.steps, 2)))]
    u_fp64 = u.clone()
    Ft = torch.from_numpy(s.get(L.FEM_F)).to(dev)

    def relres(x):
        y = torch.empty(N, dtype=torch.float64, device=dev)
        lib.nbg_spmv_bsr_f64(C.byref(A), x.data_ptr(), y.data_ptr(), sp)
        torch.cuda.synchronize()
        return float(torch.linalg.norm(Ft - y) / torch.linalg.norm(Ft))
    t_mixed, r_mixed = min(tm, key=lambda x: x[0])
    t_fp64, r_fp64 = min(tf, key=lambda x: x[0])
    nblk = nnz // 4
    # the same solves on a block layout in SELL-C-sigma node order (sigma 512)
    m = FemSystem(p, stream=sp)
    m.set_block_order(L.ORDER_SIGMA)
    assert m.assemble() == 0
    m.apply_bcs()
    A_sig = m.block_layout()
    Fm = m.dptr(L.FEM_F)
    tsig = {}
    for kind in ("mixed", "fp64"):
        u.zero_()
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if kind == "mixed":
            r = L.MixedResult()
            rc = lib.nbg_cg_mixed(C.byref(A_sig), Fm, u.data_ptr(), 8 * N, TOL, 0.1,
                                  L.CG_JACOBI | L.CG_RELATIVE, C.byref(r), ws.data_ptr(),
                                  ws_bytes, sp)
        else:
            r = L.CgResult()
            rc = lib.nbg_cg_bsr_f64(C.byref(A_sig), Fm, u.data_ptr(), 8 * N, TOL,
                                    L.CG_JACOBI | L.CG_RELATIVE, C.byref(r), ws.data_ptr(),
                                    ws_bytes, sp)
        e1.record(stream)
        e1.synchronize()
        assert rc == 0 and r.status == 0
        t_ = e0.elapsed_time(e1) / 1e3
        tsig[kind] = {"s_per_solve": t_, "iters": r.niter, "us_per_iter": t_ / r.niter * 1e6}
    sig_entries = int(A_sig.n_entries)
    m.close()
    # own rows do not fit in shared memory at this size, so besides the p
    # exchange and 1/Aii (24 B/dof) they move through global memory: per node
    # L1 w out, p in (16 + 16 B), L2 p, w, x, r in (16 + 16 + 16 + 16 B) and
    # x, r out (16 + 16 B), L3 r, p in (16 + 16 B): 160 B
    bytes_iter = 32 * nblk + 4 * (A.n_slices + 1) + 24 * N + 160 * (N // 2)
    hbm, peak_kind = peaks()
    cpu = None
    if with_cpu:
        cs = CpuSystem(p)
        cs.cg(max_iter=10)
        t_it, n_it, _ = cs.cg(max_iter=200)
        per_it = t_it / max(n_it, 1)
        cpu = {"ms_per_iteration": per_it * 1e3, "cores": cs.threads, "kind": cs.kind,
               "iterations_timed": n_it,
               "gpu_fp64_ms_per_iteration": t_fp64 / r_fp64.niter * 1e3,
               "per_iteration_speedup_fp64_gpu": per_it / (t_fp64 / r_fp64.niter),
               "sample": f"{n_it} Jacobi-PCG iterations with {cs.what()}, OpenMP "
                         f"{cs.threads} threads, timed (no projection to a full solve)"}
    line = {"workload": "C3: T3 L-shape [0,2]^2 minus (1,2]^2, 2M seeded uniform points + "
                        "boundary points, Delaunay, Z-order numbering; E=1, nu=0.25, bottom "
                        "clamped, unit +x traction on x=1, y in [1,2]; Jacobi-PCG to relres "
                        "1e-8 from u=0",
            "nodes": p.n_nodes, "triangles": p.n_elems, "dof": N, "nnz": nnz,
            "block_entries": int(A.n_entries), "blocks": nblk,
            "block_order": "mesh", "padding": int(A.n_entries) / nblk - 1,
            "sigma_order": dict(tsig, padding=sig_entries / nblk - 1,
                                note="SELL-C-sigma node order, sigma 512: fewer stored "
                                     "entries; not the default (mixed slower)"),
            "setup_s": {"mesh_generation_host": t_gen, "pattern_and_upload": t_create,
                        "assembly_bcs_block_layout": t_asm},
            "mixed": {"s_per_solve": t_mixed, "iters": r_mixed.niter,
                      "updates": r_mixed.n_updates, "relres_fp64": relres(u_mixed),
                      "us_per_iter": t_mixed / r_mixed.niter * 1e6,
                      "err_vs_fp64_rel_l2": float(torch.linalg.norm(u_mixed - u_fp64) /
                                                  torch.linalg.norm(u_fp64)),
                      "bytes_per_iter": bytes_iter,
                      "achieved_gbs": bytes_iter * r_mixed.niter / t_mixed / 1e9},
            "fp64_gpu": {"s_per_solve": t_fp64, "iters": r_fp64.niter,
                         "us_per_iter": t_fp64 / r_fp64.niter * 1e6,
                         "relres_fp64": relres(u_fp64)},
            "speedup_mixed_vs_fp64_gpu": t_fp64 / t_mixed,
            "dof_iters_per_s_mixed": N * r_mixed.niter / t_mixed,
            "peak_gbs": hbm, "peak_kind": peak_kind, "cpu": cpu}
    s.close()
    return line


def run_c3(args):
    print(json.dumps(bench_c3(args, not args.no_cpu_baseline)))
    return 0


def run_gpu(args):
    import torch
    from nbots_gb300 import _lib as L
    from nbots_gb300 import replicas as R
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem

    # replicas only: every rank solves the same system on its own GPU, with
    # no collective on the data path (barrier and max of times only)
    rank, world, local = R.world()
    torch.cuda.set_device(local)
    R.init("nccl")
    lib = L.lib()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize()
        R.barrier()

    # ---- problem: assemble and apply BCs on the device (timed once)
    p = W.config_c2()
    t0 = time.perf_counter()
    s = FemSystem(p, stream=sp)
    t_create_first = time.perf_counter() - t0
    # again, with the kernels loaded: mesh upload + device pattern, incidence
    # and block plan (pattern.cu) + allocations
    s.close()
    t0 = time.perf_counter()
    s = FemSystem(p, stream=sp)
    t_create = time.perf_counter() - t0
    # the host build of the same three structures, for comparison
    from nbots_gb300.fem import HostArrays
    ha = HostArrays(p)
    rp_h = np.zeros(2 * p.n_nodes + 1, np.uint32)
    t0 = time.perf_counter()
    lib.nbg_host_pattern(C.byref(ha.mesh), rp_h.ctypes.data, None)
    ci_h = np.zeros(int(rp_h[-1]), np.uint32)
    lib.nbg_host_pattern(C.byref(ha.mesh), rp_h.ctypes.data, ci_h.ctypes.data)
    ip_h = np.zeros(p.n_nodes + 1, np.uint32)
    ie_h = np.zeros(p.conn.size, np.uint32)
    il_h = np.zeros(p.conn.size, np.uint8)
    lib.nbg_host_incidence(C.byref(ha.mesh), ip_h.ctypes.data, ie_h.ctypes.data,
                           il_h.ctypes.data)
    t_host_pattern = time.perf_counter() - t0
    del rp_h, ci_h, ip_h, ie_h, il_h, ha
    t0 = time.perf_counter()
    assert s.assemble() == 0
    s.apply_bcs()
    A = s.block_layout()
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    N, nnz = s.N, s.nnz
    F = s.dptr(L.FEM_F)
    u = torch.zeros(N, dtype=torch.float64, device=dev)
    ws_bytes = max(lib.nbg_cg_mixed_layout_workspace_bytes(C.byref(A)),
                   lib.nbg_cg_bsr_workspace_bytes(N),
                   lib.nbg_cg_workspace_bytes(N))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def mixed():
        r = L.MixedResult()
        rc = lib.nbg_cg_mixed(C.byref(A), F, u.data_ptr(), 4 * N, TOL, 0.1, L.CG_JACOBI |
                              L.CG_RELATIVE, C.byref(r), ws.data_ptr(), ws_bytes, sp)
        assert rc == 0 and r.status == 0, (rc, r.status, lib.nbg_last_error())
        return r

    def fp64():
        r = L.CgResult()
        rc = lib.nbg_cg_bsr_f64(C.byref(A), F, u.data_ptr(), 4 * N, TOL, L.CG_JACOBI |
                                L.CG_RELATIVE, C.byref(r), ws.data_ptr(), ws_bytes, sp)
        assert rc == 0 and r.status == 0, (rc, r.status)
        return r

    def timed(fn, steps, warmup, clocks=None):
        for _ in range(warmup):
            u.zero_()
            fn()
        times, res = [], None
        barrier()
        ctx = clocks if clocks is not None else _Null()
        with ctx:
            for _ in range(steps):
                u.zero_()
                flush.fill_(1.0)  # evict L2 (512 MB > 129 MB) between steps
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                res = fn()
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1) / 1e3)
        barrier()
        return times, res

    clk = Clocks(local)
    t_mixed, r_mixed = timed(mixed, args.steps, args.warmup, clk)
    mixed_form = lib.nbg_cg_mixed_last_form()
    u_mixed = u.clone()
    t_fp64, r_fp64 = timed(fp64, max(1, min(args.steps, 3)), 1)
    u_fp64 = u.clone()

    # nbots' own iteration on the GPU (same absolute semantics, relative stop)
    rp, ci, K = s.dptr(L.FEM_ROW_PTR), s.dptr(L.FEM_COL_IDX), s.dptr(L.FEM_K)

    def nbots_gpu():
        r = L.CgResult()
        rc = lib.nbg_cg_f64(N, rp, ci, K, F, u.data_ptr(), 4 * N, TOL, L.CG_JACOBI |
                            L.CG_RELATIVE, C.byref(r), ws.data_ptr(), ws_bytes, sp)
        assert rc == 0, rc
        return r
    t_exact, r_exact = timed(nbots_gpu, 1, 0)

    # nbots' iteration and stop test on the block layout with FMAs: the
    # drop-in nb_sparse_solve_CG_precond_Jacobi's solver (absolute tolerance
    # 1e-8 ||F||, as nbots takes it)
    Fnorm = float(np.linalg.norm(s.get(L.FEM_F)))

    def nbots_block():
        r = L.CgResult()
        rc = lib.nbg_cg_bsr_f64(C.byref(A), F, u.data_ptr(), 4 * N, TOL * Fnorm,
                                L.CG_JACOBI | L.CG_NBOTS_STOP, C.byref(r), ws.data_ptr(),
                                ws_bytes, sp)
        assert rc == 0, rc
        return r
    t_nblk, r_nblk = timed(nbots_block, 2, 1)

    # ---- accuracy: true FP64 residuals and displacement differences
    Ft = torch.from_numpy(s.get(L.FEM_F)).to(dev)

    def relres(x):
        y = torch.empty(N, dtype=torch.float64, device=dev)
        lib.nbg_spmv_bsr_f64(C.byref(A), x.data_ptr(), y.data_ptr(), sp)
        torch.cuda.synchronize()
        return float(torch.linalg.norm(Ft - y) / torch.linalg.norm(Ft))
    rr_mixed, rr_fp64 = relres(u_mixed), relres(u_fp64)
    err_vs_fp64 = float(torch.linalg.norm(u_mixed - u_fp64) / torch.linalg.norm(u_fp64))

    # ---- SpMV bandwidth (standalone kernels, L2 flushed before each launch)
    def spmv_time(fn, n=20):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(n):
            flush.fill_(2.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return float(np.median(ts))
    x64 = torch.randn(N, dtype=torch.float64, device=dev)
    y64 = torch.empty_like(x64)
    x32 = x64.float()
    y32 = torch.empty_like(x32)
    ent = A.n_entries
    nblk = nnz // 4
    t_csr = spmv_time(lambda: lib.nbg_spmv_csr_f64(N, rp, ci, K, x64.data_ptr(), y64.data_ptr(), sp))
    t_b64 = spmv_time(lambda: lib.nbg_spmv_bsr_f64(C.byref(A), x64.data_ptr(), y64.data_ptr(), sp))
    t_b32 = spmv_time(lambda: lib.nbg_spmv_bsr_f32(C.byref(A), x32.data_ptr(), y32.data_ptr(), sp))
    # the mixed solver's operator alone: cold (L2 flushed before each launch)
    # and repeated back to back without a flush, as inside a solve, where
    # the evict_last share of the matrix stays in L2 between launches
    ph32 = x64.float()
    pl32 = (x64 - ph32.double()).float()
    wh32 = torch.empty_like(ph32)
    wl32 = torch.empty_like(ph32)

    def mixed_op():
        lib.nbg_spmv_bsr_mixed(C.byref(A), ph32.data_ptr(), pl32.data_ptr(), wh32.data_ptr(),
                               wl32.data_ptr(), sp)
    t_mix_cold = spmv_time(mixed_op)
    for _ in range(5):
        mixed_op()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(50):
        mixed_op()
    e1.record(stream)
    e1.synchronize()
    t_mix_warm = e0.elapsed_time(e1) / 1e3 / 50
    hbm, peak_kind = peaks()
    B_mix = 32 * nblk + 4 * (A.n_slices + 1) + 16 * N
    B_csr = 12 * nnz + 4 * (N + 1) + 8 * N + 8 * N
    B_b64 = 36 * nblk + 4 * (A.n_slices + 1) + 16 * N
    B_b32 = 20 * nblk + 4 * (A.n_slices + 1) + 8 * N
    spmv = {"fp64_csr_nbots_order": {"us": t_csr * 1e6, "gbs": B_csr / t_csr / 1e9,
                                     "frac": B_csr / t_csr / 1e9 / hbm, "bytes": B_csr},
            "fp64_block": {"us": t_b64 * 1e6, "gbs": B_b64 / t_b64 / 1e9,
                           "frac": B_b64 / t_b64 / 1e9 / hbm, "bytes": B_b64},
            "fp32_block": {"us": t_b32 * 1e6, "gbs": B_b32 / t_b32 / 1e9,
                           "frac": B_b32 / t_b32 / 1e9 / hbm, "bytes": B_b32},
            "mixed_operator_cold": {"us": t_mix_cold * 1e6, "gbs": B_mix / t_mix_cold / 1e9,
                                    "frac": B_mix / t_mix_cold / 1e9 / hbm, "bytes": B_mix},
            "mixed_operator_repeated": {"us": t_mix_warm * 1e6, "gbs": B_mix / t_mix_warm / 1e9,
                                        "frac": B_mix / t_mix_warm / 1e9 / hbm,
                                        "bytes": B_mix,
                                        "l2": "50 launches back to back, no flush"},
            "peak_gbs": hbm, "peak_kind": peak_kind, "l2": "flushed before each launch"}

    # ---- roofline of the mixed solver kernel: algorithmic bytes per iteration,
    # counting each array the fused schedule moves through HBM once, in the
    # format it reads.  Matrix stream per 2x2 block: FP32 values (16 B), 23-bit
    # remainders (8 + 4 B), column (4 B), plus the slice offsets.  The block's
    # own rows of x, r, w and p live in shared memory for the whole solve; the
    # search direction p crosses HBM (written as FP32 hi + lo, 8 B/dof, in L3
    # and gathered, 8 B/dof, by the next SpMV) and 1/Aii (4 B/dof) is read in
    # L2 and L3.  A reliable update reads the FP64 matrix (32 B values + 4 B
    # column per block), u and b, writes u.
    it = r_mixed.niter
    t_med = float(np.median(t_mixed))
    form = mixed_form
    if form == 2:
        # ghost-node form: 30 B per block (16-bit local column), and per dof r
        # published (hi and lo, 8 B), x in and out (16 B), 1/Aii in L2 and L3
        # (8 B), plus r and 1/Aii of every block's ghosts (12 B per ghost dof)
        ghost_dofs = 2 * ghost_count(s.get(L.FEM_ROW_PTR), s.get(L.FEM_COL_IDX), A.n_slices,
                                     mixed_blocks(A.n_slices, dev))
        bytes_iter = 30 * nblk + 4 * (A.n_slices + 1) + 32 * N + 12 * ghost_dofs
    else:
        ghost_dofs = 0
        bytes_iter = 32 * nblk + 4 * (A.n_slices + 1) + 24 * N
    upd_bytes = (r_mixed.n_updates + 1) * (36 * nblk + 4 * (A.n_slices + 1) + 24 * N)
    achieved = (bytes_iter * it + upd_bytes) / t_med / 1e9
    # fast FP64 kernel (vectors in global memory): 36 B per block, and per dof
    # L1 p gather + own p + w (24 B), L2 p w 1/Aii x g in, x g q out (64 B),
    # L3 q p in, p out (24 B)
    fp64_bytes_iter = 36 * nblk + 4 * (A.n_slices + 1) + 112 * N
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "mixed_cg_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("dram_bytes_per_iteration")

    # ---- end to end through the host-buffer C ABI (pinned host memory)
    rp_h, ci_h, K_h, F_h = (s.get(L.FEM_ROW_PTR), s.get(L.FEM_COL_IDX), s.get(L.FEM_K),
                            s.get(L.FEM_F))
    pin = []

    def pinned(a):
        ptr = C.c_void_p()
        L.check(lib.nbg_host_alloc(C.byref(ptr), a.nbytes), "host_alloc")
        pin.append(ptr)
        b = np.ctypeslib.as_array((C.c_uint8 * a.nbytes).from_address(ptr.value)).view(a.dtype)
        b[:] = a
        return b
    Kp, Fp, xp = pinned(K_h), pinned(F_h), pinned(np.zeros(N))
    solver = C.c_void_p()
    L.check(lib.nbg_solver_create(C.byref(solver), sp), "solver_create")
    L.check(lib.nbg_solver_set_matrix(solver, N, rp_h.ctypes.data, ci_h.ctypes.data,
                                      Kp.ctypes.data, 0), "set_matrix")
    info = L.SolveInfo()

    def e2e_step():
        xp[:] = 0.0
        L.check(lib.nbg_solver_set_matrix(solver, N, rp_h.ctypes.data, ci_h.ctypes.data,
                                          Kp.ctypes.data, L.PATTERN_SAME), "set_matrix")
        rc = lib.nbg_solver_solve(solver, Fp.ctypes.data, xp.ctypes.data, 4 * N, TOL,
                                  L.CG_JACOBI | L.CG_RELATIVE, L.METHOD_MIXED, C.byref(info))
        assert rc == 0, rc
    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(3.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    lib.nbg_solver_destroy(solver)
    e2e_v = float(np.median(e2e_t))
    for ptr in pin:
        lib.nbg_host_free(ptr)

    # ---- max over ranks
    t_all, e2e_all = R.max_over_ranks([t_med, e2e_v], device=dev)

    # the other workloads and the CPU legs run on one GPU only; with several
    # ranks each solves its own share of the batched instances
    single = world == 1
    with_cpu = rank == 0 and single and not args.no_cpu_baseline
    cpu = cpu_baseline(p) if with_cpu else None
    dropin = None
    if single and not args.no_dropin:
        dropin = bench_dropin_sparse(W, cpu["spmv_ms_median_of_7"] / 1e3 if cpu else None)
    fem_entry = bench_fem_entry(W, with_cpu) if single and not args.no_c4 else None
    c4 = bench_c4(lib, L, W) if single and not args.no_c4 else None
    c5 = None if args.no_c5 else bench_c5(args, lib, L, W, sp, dev, stream, flush,
                                          R.shard(96, rank, world))
    dmg = bench_damage(L, W, with_cpu) if single and not args.no_damage else None
    s.close()
    c3 = bench_c3(args, with_cpu) if single and not args.no_c3 else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": t_all, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_all * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 inner (float-float p, A p, x, r; FP32 + 23-bit remainder matrix) / "
                     "f64 residual", "data": "synthetic",
            "config": {"workload": WORKLOAD, "dof": N, "nnz": nnz, "tol": TOL,
                       "l2": "flushed (512 MB write) before every timed solve",
                       "replicas": world},
            "mixed": {"s_per_solve": t_all, "iters": it, "updates": r_mixed.n_updates,
                      "relres_fp64": rr_mixed, "us_per_iter": t_med / max(it, 1) * 1e6,
                      "err_vs_fp64_rel_l2": err_vs_fp64},
            "fp64_gpu": {"s_per_solve": float(np.median(t_fp64)), "iters": r_fp64.niter,
                         "relres_fp64": rr_fp64,
                         "us_per_iter": float(np.median(t_fp64)) / max(r_fp64.niter, 1) * 1e6,
                         "bytes_per_iter": fp64_bytes_iter,
                         "achieved_gbs": fp64_bytes_iter * r_fp64.niter /
                                         float(np.median(t_fp64)) / 1e9,
                         "bound": "fp64 issue (about 2 FP64 FMA per clock per SM on GB300)"},
            "nbots_order_fp64_gpu": {"s_per_solve": float(t_exact[0]), "iters": r_exact.niter,
                                     "what": "nbots' arithmetic operation for operation on "
                                             "the CSR (k_cg_f64; NBG_DROPIN_EXACT_CG=1)"},
            "nbots_iteration_block_fp64_gpu": {
                "s_per_solve": float(np.median(t_nblk)), "iters": r_nblk.niter,
                "what": "nbots' iteration and lagged stop test on the block layout with FMAs "
                        "(k_cg_bsr_f64, NBG_CG_NBOTS_STOP): the drop-in CG's solver"},
            "speedup_mixed_vs_fp64_gpu": float(np.median(t_fp64)) / t_all,
            "speedup_mixed_vs_nbots_order_fp64_gpu": float(t_exact[0]) / t_all,
            "speedup_note": "fp64 = the tuned FP64 block-layout CG (the headline comparison); "
                            "nbots_order = nbots' arithmetic on the CSR",
            "setup_s": {"pattern_and_upload": t_create, "first_call": t_create_first,
                        "host_pattern_and_incidence": t_host_pattern,
                        "assembly_and_bcs": t_asm},
            "spmv": spmv,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind,
                         "traffic": traffic,
                         "kernel": "k_cg_mixed_ghost" if form == 2 else "k_cg_mixed",
                         "form": ["global rows", "resident rows", "ghost nodes"][form],
                         "ghost_dofs": ghost_dofs, "bytes_per_iter": bytes_iter,
                         "note": "traffic is DRAM bytes per iteration from ncu; below "
                                 "bytes_per_iter because part of the matrix stays in L2 "
                                 "(evict_last) between iterations"},
            "e2e": {"value": e2e_all, "unit": "s",
                    "h2d_bytes_per_step": int(8 * nnz + 16 * N),
                    "d2h_bytes_per_step": int(8 * N),
                    "path": "nbg_solver_set_matrix (values, pattern kept) + nbg_solver_solve "
                            "(mixed) from pinned host buffers"},
            "dropin_sparse": dropin,
            "fem_entry_dropin": fem_entry,
            "c3_lshape": c3,
            "c4_simp": c4,
            "c5_batch": c5,
            "damage": dmg,
            "cpu_baseline": cpu,
            # per timed step: the ghost plan and the solver (ghost form), or
            # the solver alone
            "gpu_launches": args.steps * (2 if form == 2 else 1),
            "dof_iters_per_s": N * it / t_all,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    R.finalize()
    return 0


def run_profile(args):
    """One bounded launch of a solver kernel on the full workload, for ncu:
    `iters` iterations with a tolerance that is never met and reliable
    updates only at the end, so DRAM bytes / iters is the per-iteration
    traffic."""
    import torch
    from nbots_gb300 import _lib as L
    from nbots_gb300 import workloads as W
    from nbots_gb300.fem import FemSystem
    lib = L.lib()
    if args.profile == "damage":
        # the damage solve of the bench's 128x64 case, once
        p = W.cantilever_q4(128, 64, point_load=0.0, top_traction=0.35)
        s = FemSystem(p)
        info = s.damage(6.0, 10.0, 4, 40, 6, 1e-7)
        print(json.dumps({"profile": "damage", "dof": s.N, "iterations": info.iterations,
                          "cg_iterations": info.cg_iterations}))
        s.close()
        return 0
    p = W.config_c2()
    if args.profile == "pattern":
        # pattern, incidence and block plan of the 1M-dof mesh, twice
        for _ in range(2):
            s = FemSystem(p)
            n = s.nnz
            s.close()
        print(json.dumps({"profile": "pattern", "nodes": p.n_nodes, "nnz": n}))
        return 0
    s = FemSystem(p)
    assert s.assemble() == 0
    s.apply_bcs()
    if args.profile == "nbots":
        # the drop-in's solver (nbots' iteration, FP64, CSR), `iters` iterations
        for _ in range(2):
            r = s.solve(max_iter=args.iters)
        print(json.dumps({"profile": "nbots", "iters": r.niter, "dof": s.N}))
        s.close()
        return 0
    A = s.block_layout()
    N = s.N
    F = s.dptr(L.FEM_F)
    u = torch.zeros(N, dtype=torch.float64, device="cuda")
    ws_bytes = max(lib.nbg_cg_mixed_layout_workspace_bytes(C.byref(A)),
                   lib.nbg_cg_bsr_workspace_bytes(N))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    x64 = torch.randn(N, dtype=torch.float64, device="cuda")
    y64 = torch.empty_like(x64)
    x32, y32 = x64.float(), torch.empty(N, dtype=torch.float32, device="cuda")
    for _ in range(2):
        u.zero_()
        if args.profile == "mixed":
            r = L.MixedResult()
            lib.nbg_cg_mixed(C.byref(A), F, u.data_ptr(), args.iters, 1e-30, 1e-12,
                             L.CG_JACOBI | L.CG_RELATIVE, C.byref(r), ws.data_ptr(), ws_bytes,
                             None)
        elif args.profile == "fp64":
            r = L.CgResult()
            lib.nbg_cg_bsr_f64(C.byref(A), F, u.data_ptr(), args.iters, 1e-30,
                               L.CG_JACOBI | L.CG_RELATIVE, C.byref(r), ws.data_ptr(), ws_bytes,
                               None)
        else:
            for _ in range(3):
                lib.nbg_spmv_bsr_f64(C.byref(A), x64.data_ptr(), y64.data_ptr(), None)
                lib.nbg_spmv_bsr_f32(C.byref(A), x32.data_ptr(), y32.data_ptr(), None)
                lib.nbg_spmv_csr_f64(N, s.dptr(L.FEM_ROW_PTR), s.dptr(L.FEM_COL_IDX),
                                     s.dptr(L.FEM_K), x64.data_ptr(), y64.data_ptr(), None)
        torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "iters": args.iters, "dof": N,
                      "block_entries": int(A.n_entries), "blocks": s.nnz // 4}))
    s.close()
    return 0


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c4", action="store_true", help="skip the SIMP gradient timings")
    ap.add_argument("--no-c5", action="store_true", help="skip the batched solves")
    ap.add_argument("--no-damage", action="store_true", help="skip the damage-solve timings")
    ap.add_argument("--no-dropin", action="store_true",
                    help="skip the nb_sparse_* drop-in timings")
    ap.add_argument("--no-c3", action="store_true",
                    help="skip the 4M-dof T3 L-shape (its mesh takes about a minute)")
    ap.add_argument("--c3", action="store_true",
                    help="run only the 4M-dof unstructured T3 L-shape (mesh generation "
                         "takes about a minute on the host)")
    ap.add_argument("--profile", choices=["mixed", "fp64", "spmv", "damage", "pattern", "nbots"],
                    help="one bounded kernel launch for ncu instead of the benchmark")
    ap.add_argument("--iters", type=int, default=100)
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.c3:
        return run_c3(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
