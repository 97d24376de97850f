"""Differentiable predicted data: ``dpred`` as a ``torch.autograd.Function``.

Forward: fields + receiver gather (one multi-RHS solve over all sources).
Backward: the vector-Jacobian product ``J^T g`` -- a batched adjoint solve of
all sources (``A lambda_s = P_s^T g_s``) followed by the edge-product kernel
for ``(d(A(sigma) u)/d sigma)^T lambda`` contracted through the model map's
diagonal derivative (ExpMap: ``sigma' = sigma``).  This is the reference's
``Jtvec`` (``simpeg/electromagnetics/static/resistivity/simulation.py:189-263``)
driven by autograd, so a misfit written in torch gets its gradient without
forming J.

A model on a CUDA device stays there: an elementwise map (ExpMap, Identity,
Reciprocal and chains of them) is applied on the device and its diagonal
derivative too, so the training loop copies no model to the host.

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
        # a CUDA model stays on the device when the map is elementwise (no host round trip)
        on_dev = m.is_cuda and sim._device_model_ok()
        if on_dev:
            m_dev = m.detach().to(sim.device, torch.float64)
            f = sim.fields_dev(m_dev)
            ctx.m_dev, ctx.m_np = m_dev, None
        else:
            m_np = m.detach().cpu().numpy().astype(np.float64)
            f = sim.fields(m_np)
            ctx.m_dev, ctx.m_np = None, m_np
        d = sim._mini_survey_data_dev(sim._gather(f.phi_dev))
        ctx.sim = sim
        ctx.recompute = bool(recompute)
        ctx.fields = None if recompute else f
        if recompute:
            sim._f_cache = None
            del f
        ctx.out_device = m.device
        return d.to(m.device)

    @staticmethod
    def backward(ctx, grad_d):
        sim = ctx.sim
        if ctx.m_dev is not None:
            f = ctx.fields if ctx.fields is not None else sim.fields_dev(ctx.m_dev)
        else:
            sim.model = ctx.m_np
            f = ctx.fields if ctx.fields is not None else sim.fields(ctx.m_np)
        t, tq = sim._get_tables()
        g = sim._mini_survey_dataT_dev(grad_d.detach().to(sim.device, torch.float64).contiguous())
        PTv = torch.zeros(t.nSrc, sim.nN, dtype=torch.float64, device=sim.device)
        csr_spmv(tq["PT_ptr"], tq["PT_idx"], tq["PT_w"], g.contiguous(), PTv.view(-1), out_idx=tq["PT_out"])
        Lam = sim._solve(PTv)
        if ctx.m_dev is not None:
            gm = sim.engine.dadm_adj(f.phi_dev, Lam, sim._dsig_diag_dev(), scale=-1.0)
        else:
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
