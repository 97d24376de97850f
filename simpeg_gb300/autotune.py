"""Autotuner for the solver's RHS-block width and multigrid smoother.

For a given engine (mesh + model) and number of right-hand sides, it times
full solves of a sample RHS set (unit currents at seeded random nodes) for
each candidate ``(kb, nu, ratio)`` -- RHS-block width of the interleaved
layout (how many sources share one node's 16-byte lanes and coefficient
loads), Chebyshev degree and interval of the V-cycle smoother -- and keeps the
fastest.  Results are cached per (mesh shape, RHS count, precision).
"""

from __future__ import annotations

import itertools

import numpy as np
import torch

_CACHE = {}


def _sample_rhs(nN, k, seed, device):
    rng = np.random.default_rng(seed)
    B = torch.zeros(k, nN, dtype=torch.float64, device=device)
    idx = torch.from_numpy(rng.integers(0, nN, k)).to(device)
    B[torch.arange(k, device=device), idx] = 1.0
    return B


def candidates(k):
    kbs = sorted({kb for kb in (8, 16, 32) if (k + kb - 1) // kb <= 32} | {0})
    # intervals lmax/15 and lmax/30: on the 1M- and 2M-cell solves lmax/60 was slower at every degree, and
    # degree 2 wants the wider interval (lmax/15)
    return list(itertools.product(kbs, (2, 3, 4), (15.0, 30.0)))


def tune_engine(engine, k, precision="mixed", rtol=1e-9, sigma=None, cands=None, seed=0):
    """Pick (kb, nu, ratio) for `engine` at k right-hand sides; applies and returns the choice."""
    key = (engine.shape_cells, int(k), precision)
    if key in _CACHE:
        best = _CACHE[key]
    else:
        if sigma is not None:
            engine.set_model(sigma)
        B = _sample_rhs(engine.nN, int(k), seed, torch.device("cuda"))
        times = {}
        for kb, nu, ratio in (cands or candidates(int(k))):
            engine.set_rhs_block(kb)
            engine.set_params(nu_pre=nu, nu_post=nu, cheb_ratio=ratio)
            engine.solve(B, mode=precision, rtol=rtol, raise_on_fail=False)  # warm-up / workspace
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _, info = engine.solve(B, mode=precision, rtol=rtol, raise_on_fail=False)
            e1.record()
            torch.cuda.synchronize()
            if info.status == 0:
                times[(kb, nu, ratio)] = e0.elapsed_time(e1)
        best = min(times, key=times.get) if times else (0, 3, 30.0)
        _CACHE[key] = best
    kb, nu, ratio = best
    engine.set_rhs_block(kb)
    engine.set_params(nu_pre=nu, nu_post=nu, cheb_ratio=ratio)
    return {"kb": kb, "nu": nu, "cheb_ratio": ratio}
