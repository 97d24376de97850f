"""Differentiable predicted data: ``dpred`` as a ``torch.autograd.Function``.

Forward: fields + receiver gather (one multi-RHS solve over all sources).
Backward: the vector-Jacobian product ``J^T g`` -- a batched adjoint solve of
all sources (``A lambda_s = P_s^T g_s``) followed by the edge-product kernel
for ``(d(A(sigma) u)/d sigma)^T lambda`` contracted through the model map's
diagonal derivative (ExpMap: ``sigma' = sigma``).  This is the reference's
``Jtvec`` (``simpeg/electromagnetics/static/resistivity/simulation.py:189-263``)
driven by autograd, so a misfit written in torch gets its gradient without
forming J.

``recompute=True`` drops the forward fields after the forward pass and solves
them again in backward (for meshes whose fields do not fit next to the
adjoint workspace); ``False`` keeps them on the device between the passes.
"""

from __future__ import annotations

import numpy as np
import torch

from .engine import csr_spmv

__all__ = ["DCPredict", "dpred"]


class DCPredict(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m, sim, recompute):
        m_np = m.detach().cpu().numpy().astype(np.float64)
        f = sim.fields(m_np)
        d = sim._gather(f.phi_dev)
        ctx.sim = sim
        ctx.recompute = bool(recompute)
        ctx.m_np = m_np
        ctx.fields = None if recompute else f
        if recompute:
            sim._f_cache = None
            del f
        ctx.out_device = m.device
        if sim._mini_survey is not None:
            d = torch.from_numpy(sim._mini_survey_data(d.cpu().numpy()))
        return d.to(m.device)

    @staticmethod
    def backward(ctx, grad_d):
        sim = ctx.sim
        m_np = ctx.m_np
        sim.model = m_np
        f = ctx.fields if ctx.fields is not None else sim.fields(m_np)
        t, tq = sim._get_tables()
        g = grad_d.detach().to(sim.device, torch.float64).contiguous()
        if sim._mini_survey is not None:
            g = torch.from_numpy(sim._mini_survey_dataT(g.cpu().numpy())).to(sim.device)
        PTv = torch.zeros(t.nSrc, sim.nN, dtype=torch.float64, device=sim.device)
        csr_spmv(tq["PT_ptr"], tq["PT_idx"], tq["PT_w"], g, PTv.view(-1), out_idx=tq["PT_out"])
        Lam = sim._solve(PTv)
        d = sim._sigma_deriv()
        if isinstance(d, np.ndarray):
            dsig = torch.from_numpy(np.ascontiguousarray(d)).to(sim.device)
            gm = sim.engine.dadm_adj(f.phi_dev, Lam, dsig, scale=-1.0)
        else:
            gs = sim.engine.dadm_adj(f.phi_dev, Lam, None, scale=-1.0).cpu().numpy()
            gm = torch.from_numpy(np.asarray(d.T @ gs).ravel()).to(sim.device)
        if ctx.recompute:
            del f
            sim._f_cache = None
        return gm.to(ctx.out_device), None, None


def dpred(sim, m, recompute=False):
    """Predicted data of ``sim`` at model ``m`` (a float64 torch tensor), differentiable in ``m``."""
    return DCPredict.apply(m, sim, recompute)
