"""Continuous-batching server for DC forward requests on one GPU.

A request is ``(model, survey)`` on the server's mesh: predict the data of
every source of ``survey`` for conductivity ``sigmaMap * model``.  Every
source is one right-hand side of the model's operator, as in the reference's
``Ainv * RHS`` over ``(nN, nSrc)`` (``simpeg/electromagnetics/static/
resistivity/simulation.py:100-113``).

The server keeps a fixed pool of *slots*.  A slot is one engine handle (the
stencil hierarchy of its current model), one CUDA stream and one *lane
session* (``dc_lanes_*`` in ``include/dcgpu.h``): the state of a
mixed-precision solve with ``max_rhs`` right-hand-side lanes that persists
between refinement sweeps.  The slot's worker thread loops:

1. admit: if the slot is idle it takes the oldest queued request and sets its
   model; a running slot admits further queued requests *of its model* into
   its free lanes -- between two sweeps of the solve that is already running;
2. one refinement sweep of every active lane (each lane iterates to its own
   tolerance; a lane's iterates never depend on the others', so a request's
   result is the same alone and in any mix);
3. every request whose lanes have all converged is fetched, gathered at its
   receivers and answered, and its lanes are free for the next admission.

Requests that arrive while others are on the GPU are therefore admitted as
lanes free up, without waiting for the running solve to end, and the slots'
sweeps overlap on the device through their streams.  Admission is FIFO: a
request is not overtaken by later requests of its model, nor by requests of a
model that is running while it has no slot to go to.

Memory: each slot's engine hierarchy, lane workspace and two
``max_rhs x nN`` staging arrays (right-hand sides in, solutions out) are
allocated when the server starts; a request adds only its electrode tables.

Failure handling is host-side: a request whose model is invalid, whose
electrodes fall outside the mesh, that needs more right-hand sides than a
slot holds or that does not converge within ``max_sweeps`` fails with an
exception on its own future; other requests and the slots are unaffected.

``engine_factory(slot_index)`` lets tests drive the scheduler on the CPU: an
engine with ``lanes_backend(capacity)`` gets the lane scheduler with that
backend, one with ``run_batch(models, surveys)`` a batch scheduler that merges
queued requests of one model into one call.
"""

from __future__ import annotations

import hashlib
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

__all__ = ["DCServer", "AdmissionError", "NotConvergedError"]


class AdmissionError(RuntimeError):
    """The request cannot be admitted (too many sources for a slot, or the server is closed)."""


class NotConvergedError(RuntimeError):
    """A request's solve did not reach the tolerance within the sweep limit."""


@dataclass(eq=False)  # requests compare by identity
class _Request:
    model: np.ndarray
    survey: object
    future: Future
    key: str
    nsrc: int
    seq: int = 0
    lanes: list = field(default_factory=list)
    state: object = None
    sweeps: int = 0
    t_submit: float = 0.0


@dataclass
class _Slot:
    index: int
    engine: object
    backend: object = None
    key: object = None
    free: list = field(default_factory=list)
    running: list = field(default_factory=list)
    served: int = 0
    sweeps: int = 0
    batches: list = field(default_factory=list)  # batch mode: request seqs per engine call
    log: list = field(default_factory=list)      # lane mode: (event, seq, sweep, requests running)
    sweep_events: list = field(default_factory=list)


def _model_key(m):
    a = np.ascontiguousarray(m, dtype=np.float64)
    return hashlib.sha1(a.view(np.uint8)).hexdigest()


class _CudaLanes:
    """Lane backend of one slot on the GPU: engine, stream, lane session and staging arrays."""

    def __init__(self, server, engine, capacity):
        import torch

        self.srv = server
        self.engine = engine
        self.stream = torch.cuda.Stream()
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.capacity = capacity
        self.session = None
        nN = engine.nN
        self.Q = torch.zeros(capacity, nN, dtype=torch.float64, device=self.dev)
        self.X = torch.empty(capacity, nN, dtype=torch.float64, device=self.dev)
        # the engine's solve workspace for `capacity` lanes, laid out once
        self.ws = torch.empty(engine.workspace_bytes(capacity, "mixed"), dtype=torch.uint8, device=self.dev)

    def set_model(self, m):
        import torch

        from .engine import LaneSession

        sigma = self.srv.sigma_map * m
        if np.any(~np.isfinite(sigma)) or np.any(sigma <= 0):
            raise ValueError("conductivity must be positive and finite")
        with torch.cuda.stream(self.stream):
            self.engine.set_model(torch.from_numpy(np.ascontiguousarray(sigma)).to(self.dev))
            if self.session is None:
                self.session = LaneSession(self.engine, self.capacity, rtol=self.srv.rtol, ws=self.ws)
                self.capacity = min(self.capacity, self.session.capacity)

    def prepare(self, r):
        import torch

        from .resistivity.electrodes import SurveyTables

        t = SurveyTables(self.srv.mesh, r.survey.source_list, self.engine.nN)
        to = lambda a: torch.from_numpy(a).to(self.dev)
        return dict(t=t, q_idx=to(t.q_idx), q_val=to(t.q_val), P=(to(t.P_ptr), to(t.P_idx), to(t.P_w)))

    def load(self, lanes, r):
        import torch

        from .engine import fill_sparse

        n = len(lanes)
        st = r.state
        with torch.cuda.stream(self.stream):
            Q = self.Q[:n]
            Q.zero_()
            fill_sparse(st["q_idx"], st["q_val"], Q.view(-1))
            self.session.load(lanes, Q)

    def clear(self, lanes):
        import torch

        with torch.cuda.stream(self.stream):
            Q = self.Q[:len(lanes)]
            Q.zero_()
            self.session.load(lanes, Q)

    def sweep(self, extent=0):
        import torch

        with torch.cuda.stream(self.stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.session.set_extent(extent)
            out = self.session.sweep()
            e1.record()
        return out, (e0, e1)

    def active(self):
        import torch

        with torch.cuda.stream(self.stream):
            return self.session.state()[0]

    def finish(self, lanes, r):
        import torch

        from .engine import csr_spmv

        st = r.state
        with torch.cuda.stream(self.stream):
            X = self.session.fetch(lanes, out=self.X[:len(lanes)])
            d = torch.empty(st["t"].nD, dtype=torch.float64, device=self.dev)
            csr_spmv(*st["P"], X.reshape(-1), d)
            return d.cpu().numpy()


class DCServer:
    """Serve ``dpred`` requests on one mesh with a bounded pool of GPU slots.

    Parameters
    ----------
    mesh : tensor mesh (``h``, ``origin``)
    sigma_map : model -> conductivity map (default ExpMap: models are ln sigma)
    slots : number of concurrently running models on the device
    max_rhs : right-hand-side lanes per slot (a request's sources must fit)
    precision, rtol : solver arithmetic and tolerance (the lane sessions are mixed precision)
    max_sweeps : refinement sweeps after which a request fails as not converged
    engine_factory : callable(slot_index) -> engine (default: CUDA engine)
    """

    def __init__(self, mesh, sigma_map=None, slots=2, max_rhs=256, precision="mixed", rtol=1e-9,
                 surface_faces=None, engine_factory=None, device=None, max_sweeps=40):
        from .maps import ExpMap

        self.mesh = mesh
        self.sigma_map = sigma_map if sigma_map is not None else ExpMap(mesh)
        self.max_rhs = int(max_rhs)
        self.precision = precision
        self.rtol = float(rtol)
        self.max_sweeps = int(max_sweeps)
        self.nN = int(np.prod([len(h) + 1 for h in mesh.h]))
        self.nC = int(np.prod([len(h) for h in mesh.h]))
        self._pending = []
        self._lock = threading.Lock()
        self._cv = threading.Condition(self._lock)
        self._closed = False
        self._seq = 0
        self._device = device
        cuda = engine_factory is None
        if cuda:
            import torch

            if precision != "mixed":
                raise ValueError("the server's lane sessions solve in mixed precision")
            engine_factory = self._cuda_engine_factory(surface_faces)
            self._ref_event = torch.cuda.Event(enable_timing=True)
            self._ref_event.record()
            torch.cuda.synchronize()
        self.slots = [_Slot(i, engine_factory(i)) for i in range(int(slots))]
        self.mode = "batch" if hasattr(self.slots[0].engine, "run_batch") else "lanes"
        for s in self.slots:
            if self.mode == "lanes":
                s.backend = _CudaLanes(self, s.engine, self.max_rhs) if cuda else s.engine.lanes_backend(self.max_rhs)
                s.free = list(range(self.max_rhs))
        target = self._lane_worker if self.mode == "lanes" else self._batch_worker
        self._threads = [threading.Thread(target=target, args=(s,), daemon=True) for s in self.slots]
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
            req = _Request(m, survey, fut, _model_key(m), nsrc, self._seq, t_submit=time.perf_counter())
            self._pending.append(req)
            self._cv.notify_all()
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

    def device_intervals(self):
        """Per slot, the (start, end) of every refinement sweep on the device in ms since the server
        started (CUDA events on the slot's stream; lane mode on the GPU)."""
        out = []
        for s in self.slots:
            iv = []
            for e0, e1 in s.sweep_events:
                e1.synchronize()
                iv.append((self._ref_event.elapsed_time(e0), self._ref_event.elapsed_time(e1)))
            out.append(iv)
        return out

    # ------------------------------------------------------------ lane scheduling
    def _lane_admit(self, slot):
        """Requests admitted into the slot's free lanes now, and the model to set (idle slot)."""
        with self._lock:
            while not slot.running and not self._pending and not self._closed:
                self._cv.wait()
            if not slot.running and not self._pending:
                return None, None
            new_model = None
            if not slot.running:
                head = self._pending[0]
                slot.key = head.key
                new_model = head.model
            served = {s.key for s in self.slots if s.key is not None and (s.running or s is slot)}
            admitted, rest, blocked = [], [], False
            for r in self._pending:
                if not blocked and r.key == slot.key and r.nsrc <= len(slot.free):
                    r.lanes, slot.free = slot.free[:r.nsrc], slot.free[r.nsrc:]
                    admitted.append(r)
                    continue
                rest.append(r)
                if r.key == slot.key or r.key not in served:
                    blocked = True  # FIFO: later requests do not overtake this one
            self._pending = rest
            for r in admitted:
                slot.log.append(("admit", r.seq, slot.sweeps, len(slot.running)))
            slot.running.extend(admitted)
            return admitted, new_model

    def _release(self, slot, r):
        with self._lock:
            slot.running.remove(r)
            slot.free = sorted(slot.free + r.lanes)
            if not slot.running:
                slot.key = None
            self._cv.notify_all()

    def _lane_worker(self, slot):
        be = slot.backend
        while True:
            admitted, new_model = self._lane_admit(slot)
            if admitted is None:
                return
            if new_model is not None:
                try:
                    be.set_model(new_model)
                except Exception as exc:
                    for r in admitted:
                        r.future.set_exception(exc)
                        self._release(slot, r)
                    continue
            for r in admitted:
                try:
                    r.state = be.prepare(r)
                    be.load(r.lanes, r)
                except Exception as exc:  # this request only (e.g. electrodes outside the mesh)
                    r.future.set_exception(exc)
                    self._release(slot, r)
            if not slot.running:
                continue
            # lanes are handed out lowest first: the sweep covers the blocks up to the highest lane in use
            extent = 1 + max(l for r in slot.running for l in r.lanes)
            (n_active, _), evs = be.sweep(extent)
            slot.sweeps += 1
            if evs is not None:
                slot.sweep_events.append(evs)
            slot.log.append(("sweep", None, slot.sweeps, len(slot.running)))
            act = be.active()
            for r in list(slot.running):
                r.sweeps += 1
                if not np.any(act[r.lanes]):
                    try:
                        r.future.set_result(be.finish(r.lanes, r))
                    except Exception as exc:
                        r.future.set_exception(exc)
                    slot.log.append(("done", r.seq, slot.sweeps, len(slot.running)))
                    slot.served += 1
                    self._release(slot, r)
                elif r.sweeps >= self.max_sweeps:
                    be.clear(r.lanes)
                    r.future.set_exception(NotConvergedError(
                        f"request {r.seq} did not reach rtol {self.rtol:g} in {r.sweeps} refinement sweeps"))
                    self._release(slot, r)

    # ------------------------------------------------------------ batch scheduling (run_batch engines)
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

    def _batch_worker(self, slot):
        while True:
            batch = self._take_batch()
            if batch is None:
                return
            try:
                outs = slot.engine.run_batch([r.model for r in batch], [r.survey for r in batch])
                for r, d in zip(batch, outs):
                    r.future.set_result(d)
            except Exception as exc:  # a failure belongs to the requests of this batch only
                for r in batch:
                    if not r.future.done():
                        r.future.set_exception(exc)
            finally:
                slot.served += len(batch)
                slot.batches.append([r.seq for r in batch])
