"""Why the mixed solver keeps a float-float residual and 23-bit matrix
remainders: a CPU emulation of its iteration on the 256x128 lognormal
cantilever (66,306 dof), float64 standing in for float-float, with the
residual rounded to FP32 or not and the matrix rounded to FP32 plus a
remainder of a given number of bits (the layout's encoding).  All stop on
the true FP64 residual at relres 1e-8.  FP64 CG lands 3.3e-10 from the
exact solution; the emulated solver with FP32 r and 16-bit remainders
1.0e-8 (the error sits in smooth modes the residual barely sees); with
float-float r and 23-bit remainders 3.2e-10.  CPU only."""
import numpy as np
import pytest

scipy_sparse = pytest.importorskip("scipy.sparse")
spl = pytest.importorskip("scipy.sparse.linalg")

from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def system():
    from nbots_gb300 import workloads as W
    p = W.config_c2(nx=256, ny=128)
    fl = O.Flat(p)
    rp, ci = O.pattern(fl)
    st, K, F = O.assemble(fl, rp, ci)
    assert st == 0
    O.set_bconditions(fl, rp, ci, K, F)
    N = p.n_dof
    shape = (N, N)
    A = scipy_sparse.csr_matrix((K, ci.astype(np.int64), rp.astype(np.int64)), shape=shape)
    u_exact = spl.spsolve(A.tocsc(), F)
    return A, K, rp, ci, F, u_exact


def rounded_matrix(K, rp, ci, bits):
    """FP32 values plus a remainder count of `bits` bits in units of
    2^-(23 + bits) of the FP32 value, as the block layout stores them."""
    hi = K.astype(np.float32).astype(np.float64)
    unit = 2.0 ** -(23 + bits)
    lim = 2.0 ** (bits - 1) - 1
    safe = np.where(hi != 0, hi * unit, 1.0)
    q = np.clip(np.rint(np.where(hi != 0, (K - hi) / safe, 0.0)), -lim, lim)
    n = rp.shape[0] - 1
    return scipy_sparse.csr_matrix((hi + q * unit * hi, ci.astype(np.int64),
                                    rp.astype(np.int64)), shape=(n, n))


def fp64_cg(A, b, dinv, tol):
    u = np.zeros_like(b)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    while np.linalg.norm(r) > tol * np.linalg.norm(b):
        w = A @ p
        al = rz / (p @ w)
        u += al * p
        r -= al * w
        z = dinv * r
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return u


def mixed_cg(A, A_inner, b, dinv, tol, fp32_r, delta=0.1):
    """The mixed solver's iteration: inner operator A_inner, residual
    rounded to FP32 or kept, reliable updates (u += x, r = b - A u) when
    |r| has fallen by delta, p kept across them, stop on the true residual."""
    rnd = (lambda v: v.astype(np.float32).astype(np.float64)) if fp32_r else (lambda v: v)
    u = np.zeros_like(b)
    x = np.zeros_like(b)
    r64 = b.copy()
    rmax2 = r64 @ r64
    target2 = (tol * np.linalg.norm(b)) ** 2
    r = rnd(r64)
    z = dinv * r
    p = z.copy()
    rz = r @ z
    while True:
        w = A_inner @ p
        al = rz / (p @ w)
        x += al * p
        r = rnd(r - al * w)
        z = dinv * r
        rzn = r @ z
        rr = r @ r
        rmax2 = max(rmax2, rr)
        if rr <= delta * delta * rmax2 or rr <= target2:
            u += x
            x[:] = 0.0
            r64 = b - A @ u
            rmax2 = r64 @ r64
            if rmax2 <= target2:
                return u
            r = rnd(r64)
            z = dinv * r
            rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn


def test_residual_and_matrix_precision_set_the_error(system):
    A, K, rp, ci, F, u_exact = system
    dinv = (1.0 / A.diagonal()).astype(np.float32).astype(np.float64)
    n = np.linalg.norm(u_exact)
    e64 = np.linalg.norm(fp64_cg(A, F, dinv, 1e-8) - u_exact) / n
    old = mixed_cg(A, rounded_matrix(K, rp, ci, 16), F, dinv, 1e-8, fp32_r=True)
    new = mixed_cg(A, rounded_matrix(K, rp, ci, 23), F, dinv, 1e-8, fp32_r=False)
    e_old = np.linalg.norm(old - u_exact) / n
    e_new = np.linalg.norm(new - u_exact) / n
    assert e64 < 1e-9
    assert e_old > 5 * e64, (e_old, e64)       # the error the old form kept
    assert e_new < 2 * e64, (e_new, e64)       # the current form: FP64's own
