"""SIMP objectives and their adjoint gradients through the C ABI
(nbg_fem_simp), and a torch.autograd.Function over them for the Python check
harness.  nbots has no topology-optimisation code; the sensitivities follow
the standard SIMP adjoint (see csrc/simp.cu).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fem import FemSystem

COMPLIANCE, DOF = 0, 1


class SimpProblem:
    """A fixed mesh and boundary conditions whose element moduli follow
    E = Emin + rho^p (E0 - Emin)."""

    def __init__(self, p, penal=3.0, E0=1.0, Emin=1e-9, method=L.METHOD_FP64, tol=1e-12):
        self.sys = FemSystem(p)
        self.p = p
        self.penal, self.E0, self.Emin = penal, E0, Emin
        self.method, self.tol = method, tol

    def evaluate(self, rho, objective=COMPLIANCE, dof=0):
        """(J, dJ/drho, info) for densities rho."""
        rho = np.ascontiguousarray(rho, np.float64)
        dJ = np.zeros(self.p.n_elems)
        info = L.SimpInfo()
        rc = self.sys.lib.nbg_fem_simp(self.sys.handle, C.byref(self.sys.h.bcs), rho.ctypes.data,
                                       self.p.nu, self.p.thickness, self.penal, self.E0,
                                       self.Emin, objective, dof, self.tol, self.method,
                                       dJ.ctypes.data, C.byref(info))
        if rc < 0:  # 1: a solve stopped short of tol (info.status), J and dJ still set
            L.check(rc, "fem_simp")
        return info.J, dJ, info

    def close(self):
        self.sys.close()


def autograd_objective(problem: SimpProblem, objective=COMPLIANCE, dof=0):
    """A differentiable torch function rho -> J (check harness only)."""
    import torch

    class _J(torch.autograd.Function):
        @staticmethod
        def forward(ctx, rho):
            J, dJ, _ = problem.evaluate(rho.detach().cpu().double().numpy(), objective, dof)
            ctx.save_for_backward(torch.from_numpy(dJ))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            (dJ,) = ctx.saved_tensors
            return g * dJ

    return _J.apply
