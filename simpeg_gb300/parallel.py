"""Source-sharded DC simulation across ranks (one GPU per rank).

The reference splits a survey's sources over sub-simulations that share the
mesh and model (``simpeg/meta/simulation.py:13-330``, its multiprocessing and
dask variants in ``simpeg/meta/multiprocessing.py`` and ``dask_sim.py``):
``dpred`` and ``Jvec`` concatenate the sub-results, ``Jtvec`` and
``getJtJdiag`` sum them.  :class:`ShardedSimulation` does the same over
``torch.distributed`` ranks: rank r owns the sources ``r::world`` (round-robin,
so uneven source counts balance), ``dpred``/``Jvec`` gather the pieces back
into survey order, and ``Jtvec``/``getJtJdiag`` all-reduce an ``nC`` vector --
the only data-path collective of this path.

``sim_factory(survey_chunk)`` builds the rank's simulation (the GPU
``Simulation3DNodal`` in production; the CPU tests pass stand-ins with the same
methods so the collective logic runs under ``gloo``).

The collectives move tensors: on the rank's CUDA device under NCCL (which only
takes device tensors), on the host under gloo.  The data gather needs no size
exchange: the round-robin split tells every rank how many data every other rank
holds, so the pieces are padded to the largest and gathered with one
``all_gather``.
"""

from __future__ import annotations

import numpy as np
import torch

from .resistivity.survey import Survey

__all__ = ["ShardedSimulation"]


class ShardedSimulation:
    def __init__(self, survey, sim_factory, group=None):
        import torch.distributed as dist

        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group) if dist.is_initialized() else 0
        self.world = dist.get_world_size(group) if dist.is_initialized() else 1
        self.survey = survey
        self.my_sources = list(range(self.rank, survey.nSrc, self.world))
        self.local_survey = Survey([survey.source_list[i] for i in self.my_sources])
        self.local = sim_factory(self.local_survey) if self.my_sources else None
        # datum index ranges of every source in survey order
        nd = [src.nD for src in survey.source_list]
        self._starts = np.r_[0, np.cumsum(nd)].astype(np.int64)
        self._rank_sources = [list(range(r, survey.nSrc, self.world)) for r in range(self.world)]
        self._rank_nd = [int(sum(nd[i] for i in s)) for s in self._rank_sources]
        backend = dist.get_backend(group) if dist.is_initialized() else "gloo"
        self._comm_device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" \
            else torch.device("cpu")

    # --------------------------------------------------------------- helpers
    def _gather_data(self, local):
        """Concatenate per-rank data pieces back into survey order (one padded all_gather)."""
        local = np.asarray(local, dtype=np.float64)
        if self.world > 1:
            width = max(max(self._rank_nd), 1)
            buf = torch.zeros(width, dtype=torch.float64, device=self._comm_device)
            buf[:local.size] = torch.as_tensor(local, device=self._comm_device)
            bufs = [torch.empty_like(buf) for _ in range(self.world)]
            self.dist.all_gather(bufs, buf, group=self.group)
            parts = [(self._rank_sources[r], bufs[r][:self._rank_nd[r]].cpu().numpy()) for r in range(self.world)]
        else:
            parts = [(self.my_sources, local)]
        out = np.zeros(self.survey.nD)
        for srcs, vals in parts:
            if not srcs:
                continue
            pos = 0
            for i in srcs:
                n = self._starts[i + 1] - self._starts[i]
                out[self._starts[i]:self._starts[i + 1]] = vals[pos:pos + n]
                pos += n
        return out

    def _local_slice(self, v):
        v = np.asarray(v, dtype=np.float64)
        return np.concatenate([v[self._starts[i]:self._starts[i + 1]] for i in self.my_sources]) \
            if self.my_sources else np.zeros(0)

    def _sum(self, vec, n):
        t = torch.as_tensor(np.zeros(n) if vec is None else np.asarray(vec, dtype=np.float64),
                            device=self._comm_device)
        if self.world > 1:
            self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return t.cpu().numpy()

    # --------------------------------------------------------------- API
    def dpred(self, m):
        local = self.local.dpred(m) if self.local is not None else np.zeros(0)
        return self._gather_data(local)

    def Jvec(self, m, v):
        local = self.local.Jvec(m, v) if self.local is not None else np.zeros(0)
        return self._gather_data(local)

    def Jtvec(self, m, v):
        n = np.asarray(m).size
        local = self.local.Jtvec(m, self._local_slice(v)) if self.local is not None else None
        return self._sum(local, n)

    def getJtJdiag(self, m, W=None):
        n = np.asarray(m).size
        local = None
        if self.local is not None:
            Wl = None
            if W is not None:
                import scipy.sparse as sp

                Wl = sp.diags(self._local_slice(np.asarray(W.diagonal())))
            local = self.local.getJtJdiag(m, W=Wl)
        return self._sum(local, n)
