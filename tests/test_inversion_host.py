"""The InexactGaussNewton minimiser's logic on the CPU (torch CPU tensors stand in for device
vectors): convergence on a convex quadratic with the exact Hessian, the BFGS preconditioner built
from the iterates, the Armijo line search and the stopping rules of the reference's Minimize
(``simpeg/optimization.py:363-852,1265-1415``)."""

import numpy as np
import torch

from simpeg_gb300.inversion import InexactGaussNewton


def _quadratic(n=20, seed=0):
    rng = np.random.default_rng(seed)
    Q = rng.standard_normal((n, n))
    A = Q @ Q.T + n * np.eye(n)
    b = rng.standard_normal(n)
    At, bt = torch.from_numpy(A), torch.from_numpy(b)

    def ev(x, return_g=True, return_H=True):
        xt = torch.from_numpy(np.asarray(x, dtype=np.float64))
        f = float(0.5 * xt @ At @ xt - bt @ xt)
        if not return_g and not return_H:
            return f
        out = (f,)
        if return_g:
            out += (At @ xt - bt,)
        if return_H:
            out += (lambda v: At @ v,)
        return out

    return A, b, ev


def test_converges_to_the_minimiser():
    A, b, ev = _quadratic()
    opt = InexactGaussNewton(maxIter=30, cg_maxiter=40, cg_rtol=1e-12, tolF=1e-16, tolX=1e-16, tolG=1e-10, eps=1e-14)
    opt.remember("f")
    x = opt.minimize(ev, np.zeros(b.size))
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-8, atol=1e-10)
    f = opt.recall("f")
    assert all(f1 <= f0 + 1e-12 for f0, f1 in zip(f, f[1:]))


def test_bfgs_preconditioner_and_inexact_steps():
    """Two CG iterations per step: the BFGS pairs collected from the iterates precondition the later
    steps; the iteration still converges, and the step pairs are stored."""
    A, b, ev = _quadratic(seed=1)
    opt = InexactGaussNewton(maxIter=200, cg_maxiter=2, tolF=1e-16, tolX=1e-16, tolG=1e-9, eps=1e-13)
    x = opt.minimize(ev, np.zeros(b.size))
    assert opt._bfgscnt >= 1 and opt._S[0] is not None
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-6, atol=1e-8)


def test_stopping_rules():
    A, b, ev = _quadratic(seed=2)
    opt = InexactGaussNewton(maxIter=3, cg_maxiter=1)
    opt.minimize(ev, np.zeros(b.size))
    assert opt.iter == 3 and opt.stopped_by == "iteration"
    # a point where the gradient vanishes stops at once (norm_g)
    x_star = np.linalg.solve(A, b)
    opt = InexactGaussNewton(maxIter=10)
    x = opt.minimize(ev, x_star)
    assert opt.iter == 0 and opt.stopped_by in ("norm_g", "optimal")
    np.testing.assert_array_equal(x, x_star)


def test_armijo_backtracking():
    """A search direction 4x too long: the line search halves it until the Armijo condition holds."""
    A, b, ev = _quadratic(seed=3)
    opt = InexactGaussNewton(maxIter=1, cg_maxiter=50, cg_rtol=1e-14, approxHinv=lambda v: v)
    opt.findSearchDirection = lambda: 4.0 * InexactGaussNewton.findSearchDirection(opt)
    opt.minimize(ev, np.zeros(b.size))
    assert opt.iterLS >= 1 and opt._LS_t <= 0.5
