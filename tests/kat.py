"""Known answers of nbots' own FEM unit test
(utest/sources/nb/pde_bot/finite_element/solid_mechanics/static_elasticity2D.c).
"""
import numpy as np

BEAM_MAX_DISP = 1.00701e-1      # :118, tolerance 1e-6
PWH_MAX_VM_ERR = 9.7e-3         # :136


def max_disp(u):
    u = np.asarray(u).reshape(-1, 2)
    return float(np.sqrt((u * u).sum(1).max()))


def kirsch_stress(x, y, a=0.5, tx=1e4):
    """Plane stress around a circular hole of radius a under uniaxial tension
    tx at infinity (Kirsch solution), the analytic field of the test."""
    r = np.hypot(x, y)
    th = np.arctan2(y, x)
    ar2 = (a / r) ** 2
    ar4 = 1.5 * ar2 * ar2
    c2, c4, s2, s4 = np.cos(2 * th), np.cos(4 * th), np.sin(2 * th), np.sin(4 * th)
    sxx = tx * (1.0 - ar2 * (1.5 * c2 + c4) + ar4 * c4)
    syy = tx * (-ar2 * (0.5 * c2 - c4) - ar4 * c4)
    sxy = tx * (-ar2 * (0.5 * s2 + s4) + ar4 * s4)
    return sxx, syy, sxy


def vm(sxx, syy, sxy):
    return np.sqrt(sxx * sxx + syy * syy - sxx * syy + 3.0 * sxy * sxy)


def pwh_mean_vm_error(problem, stress):
    """Mean |1 - vm_fem / vm_exact| over the T3 Gauss points (centroids)."""
    c = problem.nod[problem.conn].mean(axis=1)
    s = np.asarray(stress).reshape(-1, 3)
    exact = vm(*kirsch_stress(c[:, 0], c[:, 1]))
    return float(np.mean(np.abs(1.0 - vm(s[:, 0], s[:, 1], s[:, 2]) / exact)))
