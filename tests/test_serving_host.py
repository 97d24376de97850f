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
