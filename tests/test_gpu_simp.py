"""SIMP adjoint sensitivities on the GPU.

nbots has no topology-optimisation code, so the checks are: the GPU kernel
against the oracle's CPU restatement of the same formula, and the adjoint
gradients (compliance and one nodal displacement) against central finite
differences of the objective (step 1e-5 on rho; each evaluation a full
assemble + solve to relres 1e-13), within 1e-6 relative to the largest
sensitivity, as the target asks."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def simp_problem(nx=16, ny=8, seed=11):
    from nbots_gb300 import workloads as W
    p = W.cantilever_q4(nx, ny, jitter=0.1, seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    rho = rng.uniform(0.3, 0.7, size=p.n_elems)
    p.E = W.simp_E(rho)
    return p, rho


@pytest.fixture(scope="module")
def L():
    from nbots_gb300 import _lib
    assert _lib.lib().nbg_device_count() > 0
    return _lib


def test_sensitivity_kernel_matches_oracle(L):
    from nbots_gb300.device import DeviceArray
    from nbots_gb300.fem import FemSystem
    p, rho = simp_problem(32, 16)
    s = FemSystem(p)
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal(p.n_dof), rng.standard_normal(p.n_dof)
    da, db, dr = DeviceArray(a), DeviceArray(b), DeviceArray(rho)
    out = DeviceArray(shape=(p.n_elems,), dtype=np.float64)
    lib = L.lib()
    nod = s.h.nod
    dn, dc = DeviceArray(nod), DeviceArray(s.h.conn)
    assert lib.nbg_simp_sensitivity_f64(4, p.n_elems, dn.ptr, dc.ptr, p.nu, p.thickness, dr.ptr,
                                        3.0, 1.0, 1e-9, da.ptr, db.ptr, out.ptr, None) == 0
    ref = O.simp_sensitivity(O.Flat(p), rho, a, b)
    got = out.numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("objective", [0, 1])
def test_adjoint_gradient_vs_finite_differences(L, objective):
    from nbots_gb300.simp import SimpProblem
    p, rho = simp_problem()
    dof = 2 * ((p.meta["ny"] // 2) * (p.meta["nx"] + 1) + p.meta["nx"]) + 1  # u_y of the load node
    sp = SimpProblem(p, tol=1e-13)
    J, dJ, info = sp.evaluate(rho, objective, dof)
    assert info.status in (0, 1)  # 1: at the FP64 floor, just above relres 1e-13
    h = 1e-5
    rng = np.random.default_rng(5)
    scale = np.max(np.abs(dJ))
    for e in rng.choice(p.n_elems, size=16, replace=False):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        fd = (sp.evaluate(rp, objective, dof)[0] - sp.evaluate(rm, objective, dof)[0]) / (2 * h)
        assert abs(fd - dJ[e]) <= 1e-6 * scale, (e, fd, dJ[e])
    sp.close()


def test_adjoint_matches_oracle_cpu_sensitivities(L):
    """The oracle's sensitivities evaluated on the oracle's own FP64 solution."""
    from nbots_gb300.simp import SimpProblem
    p, rho = simp_problem()
    sp = SimpProblem(p, tol=1e-13)
    J, dJ, _ = sp.evaluate(rho, 0)
    r = O.fem(p, tol=1e-13 * 1e-3)
    u_cpu, *_ = O.cg_jacobi(r["row_ptr"], r["col_idx"], r["K_bc"], r["F_bc"],
                           max_iter=40 * p.n_dof, tol=1e-14)
    ref = O.simp_sensitivity(r["flat"], rho, u_cpu, u_cpu)
    assert np.max(np.abs(dJ - ref)) <= 1e-8 * np.max(np.abs(ref))
    assert abs(J - float(r["F_bc"] @ u_cpu)) <= 1e-10 * abs(J)
    sp.close()


def test_mixed_precision_gradient_and_autograd(L):
    import torch
    from nbots_gb300.simp import SimpProblem, autograd_objective
    p, rho = simp_problem()
    ref = SimpProblem(p, tol=1e-13)
    _, dJ64, _ = ref.evaluate(rho, 0)
    mixed = SimpProblem(p, tol=1e-11, method=L.METHOD_MIXED)
    _, dJm, info = mixed.evaluate(rho, 0)
    assert info.status in (0, 1)  # 1: at the FP64 floor, just above relres 1e-13
    assert np.max(np.abs(dJm - dJ64)) <= 1e-6 * np.max(np.abs(dJ64))
    f = autograd_objective(ref, 0)
    t = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    f(t).backward()
    assert np.allclose(t.grad.numpy(), dJ64, rtol=0, atol=1e-12 * np.max(np.abs(dJ64)))


@pytest.mark.parametrize("objective", [0, 1])
def test_c4_full_size_finite_differences(L, objective):
    """The 512x256 SIMP problem (rho ~ U(0.3,0.7), seed 4): adjoint gradients
    against central differences with step 1e-6 on 64 random elements, FP64
    solves to relres 1e-13; objectives compliance and u_x of the right-edge
    midpoint."""
    from nbots_gb300 import workloads as W
    from nbots_gb300.simp import SimpProblem
    p = W.config_c4()
    rho = p.meta["rho"]
    nx, ny = p.meta["nx"], p.meta["ny"]
    dof = 2 * ((ny // 2) * (nx + 1) + nx)
    sp = SimpProblem(p, tol=1e-13)
    J, dJ, info = sp.evaluate(rho, objective, dof)
    assert info.status in (0, 1)  # 1: at the FP64 floor, just above relres 1e-13
    h = 1e-6
    scale = np.max(np.abs(dJ))
    rng = np.random.default_rng(64)
    worst = 0.0
    for e in rng.choice(p.n_elems, size=64, replace=False):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        fd = (sp.evaluate(rp, objective, dof)[0] - sp.evaluate(rm, objective, dof)[0]) / (2 * h)
        worst = max(worst, abs(fd - dJ[e]) / scale)
    sp.close()
    assert worst <= 1e-6, worst
