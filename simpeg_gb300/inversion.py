"""The inversion step that consumes the DC path, on the device.

Mirrors the callers of ``dpred / Jvec / Jtvec / getJtJdiag`` in simpeg's
inversion stack:

* :class:`L2DataMisfit` -- ``phi_d = ||W (d(m) - d_obs)||^2``, ``deriv = 2 J^T W^T W r``,
  ``deriv2 v = 2 J^T W W J v`` (``simpeg/data_misfit.py:238-343``);
* :class:`WeightedLeastSquares` -- Smallness + first-order Smoothness on an
  all-active tensor mesh (``simpeg/regularization/base.py:13-466,758-1207,1540-``):
  ``phi_m = alpha_s ||V^1/2 (m - m_ref)||^2 + sum_j alpha_j ||W_j G_j m||^2`` with
  ``W_j^2`` the average volume on the interior faces, ``alpha_j = (length_scale_j *
  base_length)^2`` (base_length: smallest cell width); applied by ``dc_reg_apply``;
* :func:`inexact_gauss_newton_direction` -- ``p = CG(H, -g, M)`` with ``maxiter``
  iterations (``simpeg/optimization.py:1345-1415``) and the Jacobi
  preconditioner of the ``UpdatePreconditioner`` directive
  ``M = diag(1 / (getJtJdiag(m, W) + beta * diag(reg.deriv2)))``
  (``simpeg/directives/_directives.py:2180-2260``).

All model-sized vectors stay on the device; every ``H v`` is one batched Jvec
and one batched Jtvec (two multi-RHS solves over all sources).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, lib


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


class L2DataMisfit:
    """``phi_d = ||W (d(m) - d_obs)||^2`` with diagonal W (``simpeg/data_misfit.py:238-343``).

    Constructed as the reference constructs it, ``L2DataMisfit(data, simulation)``
    (``W = diag(1 / data.standard_deviation)``, which must be positive), or as
    ``L2DataMisfit(simulation, dobs, W=None)`` with the observed data and the weights
    given directly (W: per-datum weights or a diagonal matrix; default ones).
    """

    def __init__(self, *args, data=None, simulation=None, dobs=None, W=None):
        args = list(args)
        if args and hasattr(args[0], "dobs") and hasattr(args[0], "standard_deviation"):
            data = args.pop(0)  # the reference's positional order: (data, simulation)
            if args:
                simulation = args.pop(0)
        else:
            for name in ("simulation", "dobs", "W"):
                if args:
                    val = args.pop(0)
                    if name == "simulation":
                        simulation = val
                    elif name == "dobs":
                        dobs = val
                    else:
                        W = val
        if args:
            raise TypeError("too many positional arguments")
        if simulation is None:
            raise TypeError("L2DataMisfit needs a simulation")
        self.data = data
        if data is not None:
            if dobs is not None:
                raise TypeError("give the observed data either as data or as dobs")
            dobs = data.dobs
            if W is None:
                std = data.standard_deviation
                if std is None or np.any(np.asarray(std, dtype=np.float64) <= 0):
                    raise ValueError("data.standard_deviation must be strictly positive to construct the W matrix: "
                                     "set data.relative_error and/or data.noise_floor, or pass W")
                W = 1.0 / np.asarray(std, dtype=np.float64)
        if dobs is None:
            raise TypeError("L2DataMisfit needs the observed data (data or dobs)")
        self.simulation = simulation
        dev = simulation.device
        self.dobs = torch.as_tensor(np.asarray(dobs, dtype=np.float64), device=dev)
        if W is None:
            w = np.ones(self.dobs.numel())
        elif np.ndim(W) == 1:
            w = np.asarray(W, dtype=np.float64)
        else:  # a (sparse) diagonal weighting matrix, as simpeg's misfit holds it
            w = np.asarray(W.diagonal(), dtype=np.float64)
        self.w = torch.as_tensor(w, device=dev)
        self.W = w

    def residual_dev(self, m):
        sim = self.simulation
        f = sim._fields_for(m, None)
        return sim._gather(f.phi_dev) - self.dobs

    def __call__(self, m):
        r = self.w * self.residual_dev(m)
        return float((r * r).sum().item())

    def deriv_dev(self, m):
        r = self.residual_dev(m)
        return 2.0 * self.simulation.jtvec_dev(self.w * self.w * r)

    def deriv2_dev(self, m, v_dev, f=None):
        sim = self.simulation
        f = sim._fields_for(m, f)  # the products run at m, whatever model was evaluated last
        return 2.0 * sim.jtvec_dev(self.w * self.w * sim.jvec_dev(v_dev, f=f), f=f)

    @property
    def nD(self):
        return int(self.dobs.numel())

    def deriv(self, m, f=None):
        """Gradient ``2 J^T W^T W r`` as a host array (``data_misfit.py:280-304``)."""
        return self.deriv_dev(m).cpu().numpy()

    def deriv2(self, m, v, f=None):
        """Gauss-Newton Hessian product ``2 J^T W^T W J v`` as a host array (``data_misfit.py:306-343``)."""
        v_dev = torch.as_tensor(np.asarray(v, dtype=np.float64), device=self.simulation.device)
        return self.deriv2_dev(m, v_dev, f=f).cpu().numpy()


class _EngineHolder:
    """What the regularization needs of a simulation: an engine on the mesh, its device, nC."""

    def __init__(self, mesh):
        from .engine import DCEngine

        self.engine = DCEngine(mesh.h, None)
        self.device = torch.device("cuda")
        self.nC = self.engine.nC


class WeightedLeastSquares:
    """Smallness + first-order smoothness on an all-active tensor mesh
    (``simpeg/regularization/base.py``), applied on the device by ``dc_reg_apply``.

    ``WeightedLeastSquares(mesh, simulation, ...)`` uses the simulation's engine; as in
    the reference, ``WeightedLeastSquares(mesh, ...)`` (or with an ``active_cells`` mask
    that keeps every cell) gives the regularization an engine of its own."""

    def __init__(self, mesh, simulation=None, alpha_s=1.0, alpha_x=None, alpha_y=None, alpha_z=None,
                 length_scale_x=None, length_scale_y=None, length_scale_z=None, reference_model=None,
                 reference_model_in_smooth=False, active_cells=None):
        if simulation is not None and not hasattr(simulation, "engine"):
            active_cells, simulation = simulation, None  # the reference's second positional argument
        if active_cells is not None and not np.all(np.asarray(active_cells)):
            raise NotImplementedError("inactive cells are not supported: every cell of the mesh is active")
        self.mesh = mesh
        self.simulation = simulation if simulation is not None else _EngineHolder(mesh)
        simulation = self.simulation
        base = min(float(np.min(h)) for h in mesh.h)
        self.base_length = base

        def alpha(a, ls):
            if a is not None:
                if ls is not None:
                    raise ValueError("Attempted to set both alpha and length_scale at the same time")
                return float(a)
            return float((1.0 if ls is None else ls) * base) ** 2

        self.alpha_s = float(alpha_s)
        self.alpha_x = alpha(alpha_x, length_scale_x)
        self.alpha_y = alpha(alpha_y, length_scale_y)
        self.alpha_z = alpha(alpha_z, length_scale_z)
        dev = simulation.device
        nC = simulation.nC
        mref = np.zeros(nC) if reference_model is None else np.asarray(reference_model, dtype=np.float64)
        self.mref = torch.as_tensor(mref, device=dev)
        self.reference_model_in_smooth = bool(reference_model_in_smooth)

    def _apply(self, v, a_s, smooth=True, scale=1.0):
        h = self.simulation.engine._h
        out = torch.empty_like(v)
        ax, ay, az = (self.alpha_x, self.alpha_y, self.alpha_z) if smooth else (0.0, 0.0, 0.0)
        check(lib().dc_reg_apply(h, a_s, ax, ay, az, _p(v.contiguous()), _p(out), C.c_void_p(0), scale, _stream()))
        return out

    def R(self, v):
        """(deriv2 / 2) v."""
        return self._apply(v, self.alpha_s)

    def diag_deriv2(self):
        h = self.simulation.engine._h
        d = torch.empty(self.simulation.nC, dtype=torch.float64, device=self.mref.device)
        check(lib().dc_reg_apply(h, self.alpha_s, self.alpha_x, self.alpha_y, self.alpha_z, C.c_void_p(0),
                                 C.c_void_p(0), _p(d), 2.0, _stream()))
        return d

    def _dev(self, m):
        return m if torch.is_tensor(m) else torch.as_tensor(np.asarray(m, dtype=np.float64), device=self.mref.device)

    def __call__(self, m_dev):
        m_dev = self._dev(m_dev)
        dm = m_dev - self.mref
        ms = dm if self.reference_model_in_smooth else m_dev
        small = self._apply(dm, self.alpha_s, smooth=False)
        smooth = self._apply(ms, 0.0)
        return float((dm * small).sum().item() + (ms * smooth).sum().item())

    def deriv_dev(self, m_dev):
        dm = m_dev - self.mref
        ms = dm if self.reference_model_in_smooth else m_dev
        return 2.0 * (self._apply(dm, self.alpha_s, smooth=False) + self._apply(ms, 0.0))

    def deriv2_dev(self, v_dev):
        return 2.0 * self.R(v_dev)

    def deriv(self, m):
        """Gradient as a host array."""
        return self.deriv_dev(self._dev(m)).cpu().numpy()

    def deriv2(self, m, v):
        """Second derivative times v as a host array (independent of m)."""
        return self.deriv2_dev(self._dev(v)).cpu().numpy()


def inexact_gauss_newton_direction(dmis, reg, beta, m, cg_maxiter=10, cg_rtol=0.0, precondition=True):
    """One Gauss-Newton search direction at model m (host array).

    Returns (p, info) with p a device tensor and info a dict of the pieces
    (gradient, JtJ diagonal, CG residual history)."""
    import time

    sim = dmis.simulation
    secs = {}

    def lap(name, t0):
        torch.cuda.synchronize()
        secs[name] = time.perf_counter() - t0
        return time.perf_counter()

    t = time.perf_counter()
    sim.model = m
    sim._ensure_model()
    dev = sim.device
    mt = torch.as_tensor(np.asarray(m, dtype=np.float64), device=dev)
    sim.fields(m)
    t = lap("fields", t)
    g = dmis.deriv_dev(m) + beta * reg.deriv_dev(mt)
    t = lap("gradient", t)
    info = {"g": g, "seconds": secs}
    if precondition:
        jtj = torch.as_tensor(sim.getJtJdiag(m, W=_Diag(dmis.W)), device=dev)
        dA = jtj + beta * reg.diag_deriv2()
        Minv = torch.where(dA != 0, 1.0 / dA, torch.zeros_like(dA))
        info["jtj_diag"] = jtj
    else:
        Minv = torch.ones_like(g)
    t = lap("jtj_diag", t)

    def H(v):
        return dmis.deriv2_dev(m, v) + beta * reg.deriv2_dev(v)

    # preconditioned CG on H p = -g from p = 0 (scipy.sparse.linalg.cg semantics)
    b = -g
    x = torch.zeros_like(b)
    r = b.clone()
    z = Minv * r
    pvec = z.clone()
    rz = float((r * z).sum())
    bnorm = float(torch.linalg.vector_norm(b))
    hist = [float(torch.linalg.vector_norm(r)) / bnorm]
    for _ in range(cg_maxiter):
        q = H(pvec)
        alpha = rz / float((pvec * q).sum())
        x = x + alpha * pvec
        r = r - alpha * q
        hist.append(float(torch.linalg.vector_norm(r)) / bnorm)
        if hist[-1] <= cg_rtol:
            break
        z = Minv * r
        rz_new = float((r * z).sum())
        pvec = z + (rz_new / rz) * pvec
        rz = rz_new
    lap("cg", t)
    info["cg_rel_res"] = hist
    return x, info


class _Diag:
    def __init__(self, w):
        self._w = np.asarray(w, dtype=np.float64)

    def diagonal(self):
        return self._w


# ---------------------------------------------------------------- the minimiser
class BaseInvProblem:
    """``phi(m) = phi_d(m) + beta phi_m(m)`` and its derivatives on the device
    (``simpeg/inverse_problem.py`` ``BaseInvProblem.evalFunction``): the gradient as a device
    tensor and the Gauss-Newton Hessian as a callable on device vectors (one batched Jvec and one
    batched Jtvec per product)."""

    def __init__(self, dmisfit, reg, beta=1.0):
        self.dmisfit = dmisfit
        self.reg = reg
        self.beta = float(beta)
        self.phi_d = self.phi_m = None

    def evalFunction(self, m, return_g=True, return_H=True):
        m = np.asarray(m, dtype=np.float64)
        self.phi_d = self.dmisfit(m)
        self.phi_m = self.reg(m)
        f = self.phi_d + self.beta * self.phi_m
        if not return_g and not return_H:
            return f
        out = (f,)
        if return_g:
            m_dev = torch.as_tensor(m, device=self.dmisfit.simulation.device)
            out += (self.dmisfit.deriv_dev(m) + self.beta * self.reg.deriv_dev(m_dev),)
        if return_H:
            beta, dmis, reg = self.beta, self.dmisfit, self.reg
            out += (lambda v: dmis.deriv2_dev(m, v) + beta * reg.deriv2_dev(v),)
        return out


def jacobi_preconditioner(dmisfit, reg, beta, m):
    """``diag(1 / (getJtJdiag(m, W) + beta diag(reg.deriv2)))`` as a callable on device vectors: the
    preconditioner the ``UpdatePreconditioner`` directive sets (``directives/_directives.py:2180-2260``)."""
    sim = dmisfit.simulation
    dev = sim.device
    jtj = torch.as_tensor(sim.getJtJdiag(m, W=_Diag(dmisfit.W)), device=dev)
    dA = jtj + beta * reg.diag_deriv2()
    Minv = torch.where(dA != 0, 1.0 / dA, torch.zeros_like(dA))
    return lambda v: Minv * v


class InexactGaussNewton:
    """The reference's ``InexactGaussNewton`` (``simpeg/optimization.py:1345-1415``) with the loop of
    ``Minimize.minimize`` (``:462-530``), its Armijo backtracking line search (``:724-783``), its
    stopping criteria (``tolerance_f``, ``moving_x``, ``tolerance_g`` all met, or ``norm_g`` or
    ``iteration``; in the line search ``armijoGoldstein`` or ``iterationLS``), the ``BFGS``
    preconditioner kept from the iterates (``:1265-1331``, identity ``bfgsH0``) unless ``approxHinv``
    is given, and ``Remember`` (``:853-907``).  Models are host arrays; gradients, search directions
    and the CG vectors of ``H p = -g`` live on the device.

    ``evalFunction(x, return_g, return_H)`` returns ``f`` or ``(f, g, H)`` with g a device tensor and
    H a callable on device vectors (:class:`BaseInvProblem`)."""

    name = "Inexact Gauss Newton"

    def __init__(self, *, maxIter=20, maxIterLS=10, maxStep=np.inf, LSreduction=1e-4, LSshorten=0.5, tolF=1e-1,
                 tolX=1e-1, tolG=1e-1, eps=1e-5, require_decrease=True, cg_rtol=1e-1, cg_atol=0.0, cg_maxiter=5,
                 nbfgs=10, approxHinv=None, callback=None):
        self.maxIter, self.maxIterLS, self.maxStep = maxIter, maxIterLS, maxStep
        self.LSreduction, self.LSshorten = LSreduction, LSshorten
        self.tolF, self.tolX, self.tolG, self.eps = tolF, tolX, tolG, eps
        self.require_decrease = require_decrease
        self.cg_rtol, self.cg_atol, self.cg_maxiter = cg_rtol, cg_atol, cg_maxiter
        self.nbfgs = nbfgs
        self.approxHinv = approxHinv
        self.callback = callback
        self._rememberThese = ()
        self.stopNextIteration = False

    # ---------------------------------------------------------- Remember
    def remember(self, *args):
        self._rememberThese = args

    def recall(self, param):
        if param not in self._rememberList:
            raise KeyError(f"{param!r} was not remembered: name it in remember() first")
        return self._rememberList[param]

    def _remember_now(self):
        for p in self._rememberThese:
            if isinstance(p, str):
                self._rememberList[p].append(getattr(self, p, None))
            else:
                self._rememberList[p[0]].append(p[1](self))

    # ---------------------------------------------------------- stoppers
    @staticmethod
    def _norm(v):
        return float(torch.linalg.vector_norm(v)) if isinstance(v, torch.Tensor) else float(np.linalg.norm(v))

    def _stop(self):
        if self.iter == 0:
            self.f0 = self.f
        gn = self._norm(self.g)
        optimal = [
            self.iter != 0 and abs(self.f - self.f_last) <= self.tolF * (1 + abs(self.f0)),
            self.iter != 0 and np.linalg.norm(self.xc - self.x_last) <= self.tolX * (1 + np.linalg.norm(self.x0)),
            gn <= self.tolG,
        ]
        critical = [gn <= 1e3 * self.eps, self.maxIter <= self.iter]
        self.stopped_by = ("optimal" if all(optimal) else "norm_g" if critical[0] else
                           "iteration" if critical[1] else None)
        return all(optimal) or any(critical)

    def _stop_ls(self):
        return self._LS_ft <= self.f + self.LSreduction * self._LS_descent or self.maxIterLS <= self.iterLS

    # ---------------------------------------------------------- BFGS
    def _bfgs(self, d):
        n = self._bfgscnt
        nn = ktop = min(self.nbfgs, n)
        return self._bfgsrec(ktop, n, nn, d)

    def _bfgsrec(self, k, n, nn, d):
        if k < 0:
            return d  # identity bfgsH0
        khat = 0 if nn == 0 else (n - nn + k) % nn
        S, Y = self._S[khat], self._Y[khat]
        ys = float((Y * S).sum())
        gamma = float((S * d).sum()) / ys
        d = d - gamma * Y
        d = self._bfgsrec(k - 1, n, nn, d)
        return d + (gamma - float((Y * d).sum()) / ys) * S

    def _end_iteration_bfgs(self, xt):
        if not self._was_default_hinv:
            return
        if self.iter == 0:
            self.g_last = self.g
            return
        yy = self.g - self.g_last
        ss = torch.as_tensor(self.xc - xt, device=self.g.device)
        self.g_last = self.g
        if float((yy * ss).sum()) > 0:
            self._bfgscnt += 1
            ktop = self._bfgscnt % self.nbfgs
            self._Y[ktop] = yy
            self._S[ktop] = ss
            self.comment = ""
        else:
            self.comment = "Skip BFGS"

    # ---------------------------------------------------------- search direction
    def findSearchDirection(self):
        """CG on ``H p = -g`` from p = 0 with ``approxHinv`` (BFGS by default) as the preconditioner,
        stopped at ``|r| <= max(cg_rtol |g|, cg_atol)`` or after ``cg_maxiter`` iterations."""
        self._was_default_hinv = self.approxHinv is None
        M = self._bfgs if self.approxHinv is None else self.approxHinv
        b = -self.g
        x = torch.zeros_like(b)
        r = b.clone()
        tol = max(self.cg_rtol * self._norm(b), self.cg_atol)
        z = M(r)
        p = z.clone()
        rz = float((r * z).sum())
        self.cg_iterations = 0
        for _ in range(self.cg_maxiter):
            if self._norm(r) <= tol:
                break
            q = self.H(p)
            alpha = rz / float((p * q).sum())
            x = x + alpha * p
            r = r - alpha * q
            self.cg_iterations += 1
            if self._norm(r) <= tol:
                break
            z = M(r)
            rz_new = float((r * z).sum())
            p = z + (rz_new / rz) * p
            rz = rz_new
        return x

    def scaleSearchDirection(self, p):
        pmax = float(p.max())
        if self.maxStep < abs(pmax):
            p = self.maxStep * p / abs(pmax)
        return p

    def modifySearchDirection(self, p):
        """Armijo backtracking: t = 1, 1/2, ... until f(x + t p) <= f + LSreduction g.(x_t - x)."""
        p_host = p.cpu().numpy()
        g_host = self.g.cpu().numpy()
        self._LS_t = 1.0
        self.iterLS = 0
        while self.iterLS < self.maxIterLS:
            self._LS_xt = self.xc + self._LS_t * p_host
            self._LS_ft = self.evalFunction(self._LS_xt, return_g=False, return_H=False)
            self._LS_descent = float(np.inner(g_host, self._LS_xt - self.xc))
            if self._stop_ls():
                break
            self.iterLS += 1
            self._LS_t = self.LSshorten * self._LS_t
        return self._LS_xt, self.iterLS < self.maxIterLS

    # ---------------------------------------------------------- the loop
    def minimize(self, evalFunction, x0):
        self.evalFunction = evalFunction
        x0 = np.asarray(x0, dtype=np.float64)
        if np.any(np.isnan(x0)):
            raise ValueError("x0 has a nan.")
        self.iter = self.iterLS = 0
        self.stopNextIteration = False
        self.x0 = self.xc = self.x_last = x0
        self.f_last = np.nan
        self._rememberList = {(p if isinstance(p, str) else p[0]): [] for p in self._rememberThese}
        self._bfgscnt = -1
        self._S = [None] * self.nbfgs
        self._Y = [None] * self.nbfgs
        self._was_default_hinv = self.approxHinv is None
        self.comment = ""
        self.f = evalFunction(self.xc, return_g=False, return_H=False)
        while True:
            self.f, self.g, self.H = evalFunction(self.xc, return_g=True, return_H=True)
            if self._stop():
                break
            self.searchDirection = self.findSearchDirection()
            del self.H
            p = self.scaleSearchDirection(self.searchDirection)
            xt, passLS = self.modifySearchDirection(p)
            if not passLS and self.require_decrease:
                self.stopped_by = "line search"
                return self.xc
            # end of the iteration: the hooks first (BFGS pair, remembered values), then the shuffle
            self._end_iteration_bfgs(xt)
            self._remember_now()
            self.f_last = self.f
            self.f = self._LS_ft
            self.x_last, self.xc = self.xc, xt
            self.iter += 1
            if self.callback is not None:
                self.callback(xt)
            if self.stopNextIteration:
                break
        return self.xc
