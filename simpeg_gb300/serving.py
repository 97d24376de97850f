"""Continuous-batching server for DC forward requests on one GPU.

A request is ``(model, survey)`` on the server's mesh: predict the data of
every source of ``survey`` for conductivity ``sigmaMap * model``.  The server
keeps a fixed pool of *slots*; a slot is one engine handle (per-model stencil
hierarchy), one CUDA stream and one solve workspace sized for ``max_rhs``
right-hand sides, so the pool's device memory is reserved up front and
bounded.  Worker threads (one per slot) take requests as soon as their slot
frees up -- requests that arrive while others are on the GPU are admitted
without waiting for a batch boundary -- and their kernels overlap on the
device through the slots' streams.  A worker merges queued requests that share
the same model into one multi-RHS solve (up to ``max_rhs`` sources), the
batching the reference does with ``Ainv * RHS`` over ``(nN, nSrc)``
(``simpeg/electromagnetics/static/resistivity/simulation.py:111``).

Each right-hand side of a multi-RHS solve has its own CG scalars and
convergence flag, so a request's result does not depend on what it was
batched with beyond rounding of the reductions (the server test checks alone
vs. mixed within the solver tolerance).

Failure handling is host-side: a request whose model is invalid, whose
electrodes fall outside the mesh or that needs more right-hand sides than a
slot holds fails with an exception on its own future; other requests and the
slots are unaffected.  ``engine_factory`` lets tests drive the scheduler with
a fake engine on the CPU.
"""

from __future__ import annotations

import hashlib
import queue
import threading
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

__all__ = ["DCServer", "AdmissionError"]


class AdmissionError(RuntimeError):
    """The request cannot be admitted (too many sources for a slot, or the server is closed)."""


@dataclass
class _Request:
    model: np.ndarray
    survey: object
    future: Future
    key: str
    nsrc: int
    seq: int = 0
    tables: object = None


@dataclass
class _Slot:
    index: int
    engine: object
    stream: object = None
    busy: bool = False
    served: int = 0
    batches: list = field(default_factory=list)


def _model_key(m):
    a = np.ascontiguousarray(m, dtype=np.float64)
    return hashlib.sha1(a.view(np.uint8)).hexdigest()


class DCServer:
    """Serve ``dpred`` requests on one mesh with a bounded pool of GPU slots.

    Parameters
    ----------
    mesh : tensor mesh (``h``, ``origin``)
    sigma_map : model -> conductivity map (default ExpMap: models are ln sigma)
    slots : number of concurrent requests on the device
    max_rhs : right-hand sides per slot (sources of the merged requests)
    precision, rtol : solver arithmetic and tolerance
    engine_factory : callable(slot_index) -> engine (default: CUDA engine)
    """

    def __init__(self, mesh, sigma_map=None, slots=2, max_rhs=256, precision="mixed", rtol=1e-9,
                 surface_faces=None, engine_factory=None, device=None):
        from .maps import ExpMap

        self.mesh = mesh
        self.sigma_map = sigma_map if sigma_map is not None else ExpMap(mesh)
        self.max_rhs = int(max_rhs)
        self.precision = precision
        self.rtol = float(rtol)
        self.nN = int(np.prod([len(h) + 1 for h in mesh.h]))
        self.nC = int(np.prod([len(h) for h in mesh.h]))
        self._q = queue.Queue()
        self._pending = []
        self._lock = threading.Lock()
        self._cv = threading.Condition(self._lock)
        self._closed = False
        self._seq = 0
        self._device = device
        if engine_factory is None:
            engine_factory = self._cuda_engine_factory(surface_faces)
        self.slots = [_Slot(i, engine_factory(i)) for i in range(int(slots))]
        self._reserve()
        self._threads = [threading.Thread(target=self._worker, args=(s,), daemon=True) for s in self.slots]
        for t in self._threads:
            t.start()

    # ------------------------------------------------------------ set-up
    def _cuda_engine_factory(self, surface_faces):
        from .engine import DCEngine
        from .resistivity.boundary import robin_face_weights

        bface = robin_face_weights(self.mesh, surface_faces)

        def make(i):
            return DCEngine(self.mesh.h, bface)

        return make

    def _reserve(self):
        """Reserve each slot's solve workspace and stream up front (bounded device memory)."""
        for s in self.slots:
            reserve = getattr(s.engine, "reserve", None)
            if reserve is not None:
                reserve(self.max_rhs, self.precision)
            mk = getattr(s.engine, "make_stream", None)
            s.stream = mk() if mk is not None else None

    # ------------------------------------------------------------ API
    def submit(self, model, survey):
        """Queue a request; returns a Future of the predicted data (numpy, survey order)."""
        fut = Future()
        nsrc = len(survey.source_list)
        m = np.asarray(model, dtype=np.float64).ravel()
        with self._lock:
            if self._closed:
                raise AdmissionError("server is closed")
            if nsrc > self.max_rhs:
                fut.set_exception(AdmissionError(
                    f"request has {nsrc} sources, a slot holds {self.max_rhs} right-hand sides"))
                return fut
            if m.size != self.nC:
                fut.set_exception(ValueError(f"model has {m.size} entries, the mesh has {self.nC} cells"))
                return fut
            self._seq += 1
            req = _Request(m, survey, fut, _model_key(m), nsrc, self._seq)
            self._pending.append(req)
            self._cv.notify()
        return fut

    def close(self, wait=True):
        with self._lock:
            self._closed = True
            self._cv.notify_all()
        if wait:
            for t in self._threads:
                t.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------ scheduling
    def _take_batch(self):
        """Oldest pending request plus queued requests with the same model, up to max_rhs sources."""
        with self._lock:
            while not self._pending and not self._closed:
                self._cv.wait()
            if not self._pending:
                return None
            head = self._pending.pop(0)
            batch, used = [head], head.nsrc
            rest = []
            for r in self._pending:
                if r.key == head.key and used + r.nsrc <= self.max_rhs:
                    batch.append(r)
                    used += r.nsrc
                else:
                    rest.append(r)
            self._pending = rest
            return batch

    def _worker(self, slot):
        while True:
            batch = self._take_batch()
            if batch is None:
                return
            slot.busy = True
            try:
                self._run(slot, batch)
            except Exception as exc:  # a failure belongs to the requests of this batch only
                for r in batch:
                    if not r.future.done():
                        r.future.set_exception(exc)
            finally:
                slot.busy = False
                slot.served += len(batch)
                slot.batches.append([r.seq for r in batch])

    def _run(self, slot, batch):
        eng = slot.engine
        run = getattr(eng, "run_batch", None)
        if run is not None:  # fake engines used by the CPU tests
            outs = run([r.model for r in batch], [r.survey for r in batch])
            for r, d in zip(batch, outs):
                r.future.set_result(d)
            return
        self._run_cuda(slot, batch)

    def _run_cuda(self, slot, batch):
        import torch

        from .engine import csr_spmv, fill_sparse
        from .resistivity.electrodes import SurveyTables

        m = batch[0].model
        sigma = self.sigma_map * m
        if np.any(~np.isfinite(sigma)) or np.any(sigma <= 0):
            raise ValueError("conductivity must be positive and finite")
        # validate every request's electrodes on its own, so one bad survey
        # fails only its own future, not the requests it was merged with
        ok = []
        for r in batch:
            try:
                SurveyTables(self.mesh, r.survey.source_list, self.nN)
                ok.append(r)
            except Exception as exc:
                r.future.set_exception(exc)
        batch = ok
        if not batch:
            return
        dev = torch.device("cuda", torch.cuda.current_device() if self._device is None else self._device)
        stream = slot.stream if slot.stream is not None else torch.cuda.current_stream(dev)
        src_all = []
        for r in batch:
            src_all.extend(r.survey.source_list)
        tables = SurveyTables(self.mesh, src_all, self.nN)
        with torch.cuda.stream(stream):
            sig = torch.from_numpy(np.ascontiguousarray(sigma)).to(dev, non_blocking=False)
            slot.engine.set_model(sig)
            Q = torch.zeros(len(src_all), self.nN, dtype=torch.float64, device=dev)
            fill_sparse(torch.from_numpy(tables.q_idx).to(dev), torch.from_numpy(tables.q_val).to(dev), Q.view(-1))
            U, info = slot.engine.solve(Q, mode=self.precision, rtol=self.rtol)
            d = torch.empty(tables.nD, dtype=torch.float64, device=dev)
            csr_spmv(torch.from_numpy(tables.P_ptr).to(dev), torch.from_numpy(tables.P_idx).to(dev),
                     torch.from_numpy(tables.P_w).to(dev), U.view(-1), d)
            out = d.cpu().numpy()
        start = 0
        for r in batch:
            nd = sum(rx.nD for s in r.survey.source_list for rx in s.receiver_list)
            r.future.set_result(out[start:start + nd].copy())
            start += nd
