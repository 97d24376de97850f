"""Many independent DC forward problems in one CUDA-graph launch.

Each problem is ``(mesh, sigma, survey)`` -- its own mesh size, conductivity
and sources, as the simulations of simpeg's meta-simulation fan-out
(``simpeg/meta/simulation.py:194-330``) or of an inversion over many sites.
:class:`BatchedForward` gives every problem its own engine handle (hierarchy,
coefficients, workspace) and records every problem's adaptive solve on its own
stream into ONE CUDA graph.  The solver's loops (PCG iterations, refinement
sweeps) are conditional WHILE nodes whose conditions are set on the device
from the per-RHS convergence counters, so a single ``cudaGraphLaunch`` runs
every problem exactly as far as the stand-alone solver would, their kernels
overlapping on the GPU, with no host round trip until the launch ends.  After
a launch the device-side convergence state is read back; a problem that hit
the iteration cap is re-solved with the host-driven solver (and reported).

RHS-block width, smoother degree and Chebyshev interval per problem come from
:mod:`simpeg_gb300.autotune` when ``tune=True``.
"""

from __future__ import annotations

import ctypes as C
import numpy as np
import torch

from ._lib import check, lib
from .engine import DCEngine, MODES, csr_spmv, fill_sparse
from .resistivity.boundary import robin_face_weights
from .resistivity.electrodes import SurveyTables

__all__ = ["BatchedForward"]


class _Problem:
    pass


class BatchedForward:
    def __init__(self, problems, precision="mixed", rtol=1e-9, maxit=2000, tune=False, device=None):
        self.precision = precision
        self.rtol = float(rtol)
        self.maxit = int(maxit)
        self.device = torch.device(device if device is not None else "cuda")
        self.problems = []
        for mesh, sigma, survey in problems:
            p = _Problem()
            p.mesh = mesh
            p.engine = DCEngine(mesh.h, robin_face_weights(mesh))
            p.tables = SurveyTables(mesh, survey.source_list, p.engine.nN)
            p.k = len(survey.source_list)
            p.sigma = torch.from_numpy(np.ascontiguousarray(sigma, dtype=np.float64)).to(self.device)
            self.problems.append(p)
        if tune:
            from .autotune import tune_engine

            for p in self.problems:
                p.tuning = tune_engine(p.engine, p.k, self.precision, rtol=self.rtol, sigma=p.sigma)
        self._graph = None
        self._prepare()

    # ------------------------------------------------------------------
    def _prepare(self):
        dev = self.device
        for p in self.problems:
            p.engine.set_model(p.sigma)
            t = p.tables
            p.Q = torch.zeros(p.k, p.engine.nN, dtype=torch.float64, device=dev)
            fill_sparse(torch.from_numpy(t.q_idx).to(dev), torch.from_numpy(t.q_val).to(dev), p.Q.view(-1))
            p.X = torch.empty_like(p.Q)
            p.ws = torch.empty(p.engine.workspace_bytes(p.k, self.precision), dtype=torch.uint8, device=dev)
            p.P = [torch.from_numpy(a).to(dev) for a in (t.P_ptr, t.P_idx, t.P_w)]
        torch.cuda.synchronize()
        n = len(self.problems)
        hs = (C.c_void_p * n)(*[p.engine._h for p in self.problems])
        bs = (C.c_void_p * n)(*[p.Q.data_ptr() for p in self.problems])
        xs = (C.c_void_p * n)(*[p.X.data_ptr() for p in self.problems])
        ks = (C.c_int * n)(*[p.k for p in self.problems])
        ws = (C.c_void_p * n)(*[p.ws.data_ptr() for p in self.problems])
        wb = (C.c_size_t * n)(*[p.ws.numel() for p in self.problems])
        g = C.c_void_p()
        check(lib().dc_batch_graph_create(n, hs, MODES[self.precision], bs, xs, ks, self.rtol, self.maxit, ws, wb,
                                          C.byref(g)))
        self._graph = g

    def launch(self):
        """One graph launch: every problem's solve (no host synchronisation inside)."""
        check(lib().dc_graph_launch(self._graph, C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def convergence(self):
        """Per problem: (max relative residual, RHS above rtol, inner iterations, sweeps) read from the device."""
        out = []
        for p in self.problems:
            mr, na, it, sw = C.c_double(), C.c_int(), C.c_int(), C.c_int()
            check(lib().dc_solve_check(p.engine._h, MODES[self.precision], p.k, C.c_void_p(p.ws.data_ptr()),
                                       C.byref(mr), C.byref(na), C.byref(it), C.byref(sw)))
            out.append((mr.value, na.value, it.value, sw.value))
        return out

    def run(self):
        """Launch, verify convergence (re-solving any problem that missed rtol), return the data per problem."""
        self.launch()
        torch.cuda.synchronize()
        self.resolved = []
        for i, (p, (mr, na, _, _)) in enumerate(zip(self.problems, self.convergence())):
            if na != 0:
                X, _ = p.engine.solve(p.Q, mode=self.precision, rtol=self.rtol, ws=p.ws)
                p.X.copy_(X)  # the graph keeps writing into p.X: refresh it in place
                self.resolved.append(i)
        return self.data()

    def data(self):
        out = []
        for p in self.problems:
            d = torch.empty(p.tables.nD, dtype=torch.float64, device=self.device)
            csr_spmv(p.P[0], p.P[1], p.P[2], p.X.view(-1), d)
            out.append(d.cpu().numpy())
        return out

    def close(self):
        if self._graph is not None and self._graph.value:
            lib().dc_graph_destroy(self._graph)
            self._graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
