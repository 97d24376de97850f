"""Scheduler logic of the DC server on the CPU with a fake engine (no GPU)."""

import threading
import time

import numpy as np
import pytest

from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.survey import Survey
from simpeg_gb300.serving import AdmissionError, DCServer


class FakeEngine:
    """Returns, per request, sum(model) + source index for each datum; fails on NaN models."""

    def __init__(self, log, delay=0.02):
        self.log = log
        self.delay = delay

    def run_batch(self, models, surveys):
        self.log.append((threading.get_ident(), len(models)))
        time.sleep(self.delay)
        out = []
        for m, sv in zip(models, surveys):
            if np.any(~np.isfinite(m)):
                raise ValueError("conductivity must be positive and finite")
            vals = []
            for i, s in enumerate(sv.source_list):
                for rx in s.receiver_list:
                    vals.extend([m.sum() + i] * rx.nD)
            out.append(np.array(vals))
        return out


def _mesh():
    return TensorMesh([4, 4, 4])


def _survey(n):
    return Survey([sources.Pole([receivers.Pole(np.array([[0.5, 0.5, 1.0], [0.2, 0.2, 1.0]]))],
                                np.r_[0.1 * i, 0.5, 1.0]) for i in range(n)])


def test_results_routed_and_same_model_merged():
    log = []
    mesh = _mesh()
    m1 = np.zeros(mesh.n_cells)
    m2 = np.ones(mesh.n_cells)
    with DCServer(mesh, slots=1, max_rhs=8, engine_factory=lambda i: FakeEngine(log, delay=0.05)) as srv:
        blocker = srv.submit(m2, _survey(1))  # occupies the only slot
        time.sleep(0.01)
        futs = [srv.submit(m1, _survey(2)), srv.submit(m1, _survey(3)), srv.submit(m2, _survey(1))]
        res = [f.result(timeout=10) for f in futs]
        blocker.result(timeout=10)
    np.testing.assert_array_equal(res[0], [0, 0, 1, 1])
    np.testing.assert_array_equal(res[1], [0, 0, 1, 1, 2, 2])
    np.testing.assert_array_equal(res[2], [64, 64])
    # the two m1 requests queued behind the blocker were merged into one batch
    assert (log[1][1] == 2) or (log[2][1] == 2)


def test_admission_limits_and_closed_server():
    mesh = _mesh()
    srv = DCServer(mesh, slots=1, max_rhs=2, engine_factory=lambda i: FakeEngine([]))
    f = srv.submit(np.zeros(mesh.n_cells), _survey(3))
    with pytest.raises(AdmissionError):
        f.result(timeout=5)
    g = srv.submit(np.zeros(5), _survey(1))
    with pytest.raises(ValueError):
        g.result(timeout=5)
    srv.close()
    with pytest.raises(AdmissionError):
        srv.submit(np.zeros(mesh.n_cells), _survey(1))


def test_failure_is_isolated_and_slots_overlap():
    log = []
    mesh = _mesh()
    with DCServer(mesh, slots=3, max_rhs=8, engine_factory=lambda i: FakeEngine(log, delay=0.1)) as srv:
        bad = srv.submit(np.full(mesh.n_cells, np.nan), _survey(1))
        good = [srv.submit(np.full(mesh.n_cells, float(i)), _survey(1)) for i in range(5)]
        with pytest.raises(ValueError):
            bad.result(timeout=10)
        out = [g.result(timeout=10) for g in good]
    for i, o in enumerate(out):
        np.testing.assert_array_equal(o, [64.0 * i] * 2)
    assert len({tid for tid, _ in log}) > 1  # more than one slot worked concurrently


# ---------------------------------------------------------------- lane scheduling (continuous batching)
class FakeLanes:
    """Lane backend: a lane of request r converges after r.nsrc + 1 sweeps; the datum value of source
    i is sum(model) + i.  NaN models fail in set_model; a request with 'diverge' never converges."""

    def __init__(self, capacity, delay=0.005):
        self.capacity = capacity
        self.left = np.zeros(capacity, dtype=int)
        self.val = np.zeros(capacity)
        self.delay = delay
        self.model = None

    def set_model(self, m):
        if np.any(~np.isfinite(m)):
            raise ValueError("conductivity must be positive and finite")
        self.model = m

    def prepare(self, r):
        return None

    def load(self, lanes, r):
        for i, l in enumerate(lanes):
            self.left[l] = 10 ** 6 if getattr(r.survey, "diverge", False) else r.nsrc + 1
            self.val[l] = self.model.sum() + i

    def clear(self, lanes):
        self.left[lanes] = 0

    def sweep(self, extent=0):
        # the scheduler promises that no lane at or beyond the extent is active
        assert extent <= 0 or not np.any(self.left[extent:] > 0), "an active lane lies beyond the sweep extent"
        time.sleep(self.delay)
        self.left[self.left > 0] -= 1
        return (int((self.left > 0).sum()), 1), None

    def active(self):
        return (self.left > 0).astype(np.int32)

    def finish(self, lanes, r):
        vals = []
        for i, s in enumerate(r.survey.source_list):
            for rx in s.receiver_list:
                vals.extend([self.val[lanes[i]]] * rx.nD)
        return np.array(vals)


class FakeLaneEngine:
    def lanes_backend(self, capacity):
        return FakeLanes(capacity)


def _admits(srv):
    return [(seq, sweep, running) for s in srv.slots for ev, seq, sweep, running in s.log if ev == "admit"]


def test_lanes_admit_into_running_solve_and_route_results():
    mesh = _mesh()
    m1 = np.zeros(mesh.n_cells)
    with DCServer(mesh, slots=1, max_rhs=8, engine_factory=lambda i: FakeLaneEngine()) as srv:
        a = srv.submit(m1, _survey(4))          # 5 sweeps
        while srv.slots[0].sweeps < 2:
            time.sleep(0.001)
        b = srv.submit(m1, _survey(2))          # joins the running solve
        ra, rb = a.result(timeout=10), b.result(timeout=10)
    np.testing.assert_array_equal(ra, [0, 0, 1, 1, 2, 2, 3, 3])
    np.testing.assert_array_equal(rb, [0, 0, 1, 1])
    adm = {seq: (sweep, running) for seq, sweep, running in _admits(srv)}
    assert adm[1] == (0, 0)
    assert adm[2][0] >= 2 and adm[2][1] == 1  # admitted between sweeps, next to a running request


def test_lanes_fifo_no_overtaking():
    """With one slot running model 1, a model-2 request that has nowhere to go is not overtaken by a
    later model-1 request; a model-1 request that does not fit the free lanes is not overtaken either."""
    mesh = _mesh()
    m1, m2 = np.zeros(mesh.n_cells), np.ones(mesh.n_cells)
    with DCServer(mesh, slots=1, max_rhs=4, engine_factory=lambda i: FakeLaneEngine()) as srv:
        a = srv.submit(m1, _survey(3))
        while srv.slots[0].sweeps < 1:
            time.sleep(0.001)
        c = srv.submit(m2, _survey(1))
        d = srv.submit(m1, _survey(1))
        for f in (a, c, d):
            f.result(timeout=10)
    order = [seq for seq, _, _ in sorted(_admits(srv), key=lambda x: (x[1], x[0]))]
    assert order.index(2) < order.index(3)


def test_lanes_failures_are_isolated():
    mesh = _mesh()
    sv_bad = _survey(1)
    sv_bad.diverge = True
    with DCServer(mesh, slots=2, max_rhs=8, max_sweeps=6, engine_factory=lambda i: FakeLaneEngine()) as srv:
        nan = srv.submit(np.full(mesh.n_cells, np.nan), _survey(1))
        stuck = srv.submit(np.zeros(mesh.n_cells), sv_bad)
        good = [srv.submit(np.full(mesh.n_cells, float(i)), _survey(2)) for i in range(3)]
        with pytest.raises(ValueError):
            nan.result(timeout=10)
        from simpeg_gb300.serving import NotConvergedError

        with pytest.raises(NotConvergedError):
            stuck.result(timeout=10)
        for i, g in enumerate(good):
            np.testing.assert_array_equal(g.result(timeout=10), [64.0 * i] * 2 + [64.0 * i + 1] * 2)
