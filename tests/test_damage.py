"""nbots' quasi-static damage solve (static_damage2D.c:239-470).

CPU: the oracle's restatement writes, byte for byte, the log that nbots
itself wrote for the same problem (the committed fixtures come from the
reference library, tests/golden/make_golden.py), and the host level
schedule of the forward substitution is a valid topological order.

GPU: Gauss-Seidel on the device repeats nbots' sweeps bit for bit (the
sweep's per-row arithmetic is nbots'; only the error sum is ordered
differently); the device damage loop, through the C ABI and through the
drop-in symbol, takes the same iterations per load step as nbots and its
residuals agree with nbots' to 1e-6 relative plus the inner solves'
absolute tolerance 1e-8, displacements and damage with the oracle's to
1e-6.  The conjugate-gradient solves inside are the device CG, whose sums
run in another order than nbots', so the run is not bit-exact.
"""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

CASES = ["dmg_q4_16x8", "dmg_t3_beam150", "dmg_q4_16x8_noiter", "dmg_q4_16x8_cap",
         "dmg_q4_16x8_nosteps", "dmg_q4_allbc"]
EDGE = ["dmg_q4_16x8_noiter", "dmg_q4_16x8_cap", "dmg_q4_16x8_nosteps", "dmg_q4_allbc"]


def params(d):
    ft, gf, steps, mi, mne, rtol = d["damage_params"]
    return float(ft), float(gf), int(steps), int(mi), int(mne), float(rtol)


def parse(log):
    """The log as a list of (kind, values) records."""
    out = []
    for line in log.splitlines():
        s = line.strip()
        if s.startswith("FEM:"):
            out.append(("head", ()))
        elif m := re.match(r"\[ Load step (\d+)\]", s):
            out.append(("step", (int(m.group(1)),)))
        elif m := re.match(r"\[(\d+): Residual: (\S+?)( \])?\]?$", s):
            out.append(("res", (int(m.group(1)), float(m.group(2)), m.group(3) is not None)))
        elif s.startswith("[Conjugate Gradient"):
            out.append(("fail", ()))
        elif m := re.match(r"\[Gauss-Seidel iterations: (\d+)\]", s):
            out.append(("gs_iters", (int(m.group(1)),)))
        elif m := re.match(r"\[Gauss-Seidel error: (\S+) \]", s):
            out.append(("gs_err", (float(m.group(1)),)))
        else:
            raise AssertionError(f"unexpected log line {line!r}")
    return out


@pytest.mark.parametrize("name", CASES)
def test_oracle_log_equals_reference(name):
    p, d = load_golden(name)
    ref = bytes(d["damage_log"]).decode()
    log, u, dmg, n_gs = O.damage(p, *params(d))
    assert log == ref
    recs = parse(ref)
    if name == "dmg_t3_beam150":
        assert n_gs > 0 and any(k == "fail" for k, _ in recs)
    elif name == "dmg_q4_16x8_nosteps":
        assert recs == [("head", ())]
    else:
        assert n_gs == 0 and recs[-1][1][2]


def test_oracle_gauss_seidel_equals_reference(golden):
    """The oracle's Gauss-Seidel equals nbots' own run bit for bit: 40 sweeps
    from the SpMV input, and 2000 sweeps from 0 at tolerance 1e-6 (iterate,
    sweep count, error, status)."""
    name, p, d = golden
    if "gs40_x" not in d:
        return
    rp, ci, K, F = d["row_ptr"], d["col_idx"], d["K_bc"], d["F_bc"]
    for x0, mi, tol, key in ((d["spmv_x"], 40, 0.0, "gs40"), (None, 2000, 1e-6, "gs")):
        x, it, err, st = O.gauss_seidel(rp, ci, K, F, x0=x0, max_iter=mi, tol=tol)
        assert np.array_equal(x.view(np.uint64), d[key + "_x"].view(np.uint64)), (name, key)
        assert (it, st) == (int(d[key + "_niter"][0]), int(d[key + "_status"][0]))
        assert err == float(d[key + "_error"][0])


def test_oracle_gauss_seidel_stops_on_tolerance():
    """A diagonally dominant system converges; the returned error is below
    tol and another sweep from the result does not start."""
    p, d = load_golden("q4_allbc_16x8")
    rp, ci, K = d["row_ptr"], d["col_idx"], d["K_bc"]
    b = d["F_bc"]
    x, it, err, st = O.gauss_seidel(rp, ci, K, b, tol=1e-6)
    assert st == 0 and err <= 1e-6 and it > 0
    x2, it2, err2, st2 = O.gauss_seidel(rp, ci, K, b, x0=x, tol=1e-6)
    assert it2 == 0 and np.array_equal(x2, x)


def test_host_lower_levels():
    """nbg_host_lower_levels is host code: every row's lower-part columns sit
    in earlier levels, rows ascend within a level, all rows appear once."""
    from nbots_gb300 import _lib
    lib = _lib.lib()
    for name in ("q4_allbc_16x8", "t3_beam_cantilever"):
        _, d = load_golden(name)
        rp, ci = d["row_ptr"], d["col_idx"]
        N = rp.shape[0] - 1
        lp = np.zeros(N + 1, np.uint32)
        lr = np.zeros(N, np.uint32)
        nl = C.c_uint32(0)
        assert lib.nbg_host_lower_levels(N, rp.ctypes.data, ci.ctypes.data, lp.ctypes.data,
                                         lr.ctypes.data, C.byref(nl)) == 0
        nl = nl.value
        assert lp[0] == 0 and lp[nl] == N
        assert np.array_equal(np.sort(lr), np.arange(N))
        level = np.empty(N, np.int64)
        for L in range(nl):
            rows = lr[lp[L]:lp[L + 1]]
            assert len(rows) > 0 and np.all(np.diff(rows.astype(np.int64)) > 0)
            level[rows] = L
        for i in range(N):
            c = ci[rp[i]:rp[i + 1]]
            c = c[c < i]
            assert np.all(level[c] < level[i])


# ------------------------------------------------------------------- GPU
def gs_gpu(rp, ci, K, b, x0, max_iter, tol):
    from nbots_gb300 import _lib
    from nbots_gb300.device import DeviceArray
    lib = _lib.lib()
    N = rp.shape[0] - 1
    lp = np.zeros(N + 1, np.uint32)
    lr = np.zeros(N, np.uint32)
    nl = C.c_uint32(0)
    assert lib.nbg_host_lower_levels(N, rp.ctypes.data, ci.ctypes.data, lp.ctypes.data,
                                     lr.ctypes.data, C.byref(nl)) == 0
    arrs = [DeviceArray(np.ascontiguousarray(a)) for a in (rp, ci, K, b, x0, lp, lr)]
    ws = DeviceArray(shape=(lib.nbg_gauss_seidel_workspace_bytes(N),), dtype=np.uint8)
    res = _lib.GsResult()
    rc = lib.nbg_gauss_seidel_f64(N, *[a.ptr for a in arrs[:7]], nl.value, max_iter, tol, 60.0,
                                  C.byref(res), ws.ptr, None)
    assert rc == 0
    return arrs[4].numpy(), res


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["q4_allbc_16x8", "t3_beam_cantilever", "c1_q4_64x32"])
def test_gpu_gauss_seidel_equals_reference(name):
    """Device Gauss-Seidel against nbots' own runs: iterates bit for bit."""
    _, d = load_golden(name)
    rp, ci, K, F = d["row_ptr"], d["col_idx"], d["K_bc"], d["F_bc"]
    for x0, mi, tol, key in ((d["spmv_x"], 40, 0.0, "gs40"),
                             (np.zeros(F.shape[0]), 2000, 1e-6, "gs")):
        x, r = gs_gpu(rp, ci, K, F, x0, mi, tol)
        assert np.array_equal(x.view(np.uint64), d[key + "_x"].view(np.uint64)), key
        assert (r.niter, r.status) == (int(d[key + "_niter"][0]), int(d[key + "_status"][0]))
        assert abs(r.error - float(d[key + "_error"][0])) <= 1e-12 * float(d[key + "_error"][0])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["q4_allbc_16x8", "t3_beam_cantilever", "c1_q4_64x32"])
def test_gpu_gauss_seidel_matches_oracle(name):
    _, d = load_golden(name)
    rp, ci, K, b = d["row_ptr"], d["col_idx"], d["K_bc"], d["F_bc"]
    rng = np.random.default_rng(5)
    x0 = rng.standard_normal(b.shape[0]) * np.abs(b).max()
    # a fixed number of sweeps (tolerance out of reach): bit-exact iterates
    xo, it, err, st = O.gauss_seidel(rp, ci, K, b, x0=x0, max_iter=40, tol=0.0)
    xg, r = gs_gpu(rp, ci, K, b, x0, 40, 0.0)
    assert st == 1 and r.status == 1 and r.niter == it == 40
    assert np.array_equal(xg, xo)
    assert abs(r.error - err) <= 1e-12 * err
    if name != "q4_allbc_16x8":
        return  # the others need far more sweeps than a test should run
    # to convergence (3,035 sweeps): same sweep count, same iterate
    tol = 1e-6 * float(np.linalg.norm(b))
    xo, it, err, st = O.gauss_seidel(rp, ci, K, b, x0=x0, max_iter=20000, tol=tol)
    xg, r = gs_gpu(rp, ci, K, b, x0, 20000, tol)
    assert st == 0 and r.status == 0 and r.niter == it
    assert np.array_equal(xg, xo)


def step_iterations(recs):
    """Residual evaluations per load step."""
    out = []
    for k, v in recs:
        if k == "step":
            out.append(0)
        elif k == "res":
            out[-1] += 1
    return out


def check_q4_run(log, u, dmg, p, d):
    ref = parse(bytes(d["damage_log"]).decode())
    got = parse(log)
    assert [k for k, _ in got] == [k for k, _ in ref]
    assert step_iterations(got) == step_iterations(ref)
    for (k, a), (_, b) in zip(got, ref):
        if k == "res":
            assert a[0] == b[0] and a[2] == b[2]
            # the inner solves stop at an absolute residual of 1e-8, and
            # their last digits follow their summation order
            assert abs(a[1] - b[1]) <= 1e-6 * abs(b[1]) + 1e-8, (a, b)
    _, uo, do, _ = O.damage(p, *params(d))
    assert np.linalg.norm(u - uo) <= 1e-6 * np.linalg.norm(uo)
    assert np.max(np.abs(dmg - do)) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("method", [0, 1])  # nbots' CG on the CSR, fast FP64 CG
def test_gpu_damage_q4(tmp_path, method):
    from nbots_gb300 import _lib as L
    from nbots_gb300.fem import FemSystem
    p, d = load_golden("dmg_q4_16x8")
    s = FemSystem(p)
    logf = tmp_path / "dmg.log"
    info = s.damage(*params(d), logfile=logf, method=method)
    log = logf.read_text()
    check_q4_run(log, s.get(L.FEM_U), s.get(L.FEM_DAMAGE), p, d)
    assert info.gs_fallbacks == 0 and info.cg_solves > 0
    assert info.iterations == sum(step_iterations(parse(log)))
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", EDGE)
def test_gpu_damage_edge_settings(tmp_path, name):
    """No iteration, an iteration cap with a break on the first residual that
    is not a new best, no load step, and self weight with every boundary
    condition form: the same records as nbots."""
    from nbots_gb300.fem import FemSystem
    p, d = load_golden(name)
    s = FemSystem(p)
    logf = tmp_path / "edge.log"
    s.damage(*params(d), logfile=logf)
    got = parse(logf.read_text())
    ref = parse(bytes(d["damage_log"]).decode())
    assert [k for k, _ in got] == [k for k, _ in ref]
    for (k, a), (_, b) in zip(got, ref):
        if k == "res":
            assert a[0] == b[0] and a[2] == b[2]
            assert abs(a[1] - b[1]) <= 1e-6 * abs(b[1]) + 1e-8, (a, b)
    s.close()


@pytest.mark.gpu
def test_gpu_damage_dropin(tmp_path):
    """The same run through nbots' own symbol and objects."""
    from nbots_gb300.dropin import NbotsObjects
    p, d = load_golden("dmg_q4_16x8")
    o = NbotsObjects(p)
    logf = tmp_path / "dropin.log"
    assert o.damage(*params(d), logfile=logf) == 0
    ref = parse(bytes(d["damage_log"]).decode())
    got = parse(logf.read_text())
    assert step_iterations(got) == step_iterations(ref)
    o.close()


@pytest.mark.gpu
def test_gpu_damage_gauss_seidel_fallback(tmp_path):
    """From the second iteration on, the solves of this run fall back to
    Gauss-Seidel, which fails: the device run logs the same records in the
    same order, with nbots' sweep count 60 N, and its first residual (the
    load itself) agrees with nbots'."""
    from nbots_gb300.fem import FemSystem
    p, d = load_golden("dmg_t3_beam150")
    s = FemSystem(p)
    logf = tmp_path / "gs.log"
    ft, gf, steps, mi, mne, rtol = params(d)
    info = s.damage(ft, gf, steps, 2, mne, rtol, logfile=logf)
    got = parse(logf.read_text())
    ref = parse(bytes(d["damage_log"]).decode())
    assert info.gs_fallbacks >= 1 and info.gs_failures == info.gs_fallbacks
    assert [k for k, _ in got[:7]] == [k for k, _ in ref[:7]]
    assert got[2][1][1] == pytest.approx(ref[2][1][1], rel=1e-6)
    assert got[4][1][0] == ref[4][1][0] == 60 * p.n_dof
    s.close()
