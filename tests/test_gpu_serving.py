"""The DC server on the GPU (continuous batching over lane sessions).

Each request's result is the same alone and in the mix (its lanes iterate independently of the
others'), requests join a solve that is already running, the slots' sweeps overlap on the device,
the device memory does not grow with the number of requests served, and a bad request fails alone.

Tolerance: solves run to rtol 1e-10; alone and mixed results agree to 1e-12 relative (the lane
arithmetic does not depend on the other lanes); one request is checked against the CPU oracle
(1e-6)."""

import time

import numpy as np
import pytest

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.survey import Survey
from simpeg_gb300.serving import DCServer

pytestmark = pytest.mark.gpu


def _setup():
    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 14), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 12), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 8)]], origin="CCN")
    rng = np.random.default_rng(5)
    models = [np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells)) for _ in range(3)]
    xs = np.arange(-60.0, 61.0, 10.0)

    def survey(offset, n):
        srcs = []
        for i in range(n):
            a = xs[(offset + i) % 6]
            M = np.c_[xs[7:11], np.zeros(4), np.zeros(4)]
            N = np.c_[xs[8:12], np.zeros(4), np.zeros(4)]
            srcs.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[a, 0, 0], np.r_[a + 10, 10.0, 0]))
        return Survey(srcs)

    reqs = [(models[0], survey(0, 3)), (models[1], survey(1, 5)), (models[0], survey(2, 2)),
            (models[2], survey(3, 4)), (models[1], survey(4, 1)), (models[2], survey(5, 6)),
            (models[0], survey(1, 4)), (models[1], survey(3, 2))]
    return mesh, reqs


def test_continuous_batching(cuda):
    mesh, reqs = _setup()
    alone = []
    with DCServer(mesh, slots=1, max_rhs=16, rtol=1e-10) as srv:
        for m, sv in reqs:
            alone.append(srv.submit(m, sv).result(timeout=120))
    with DCServer(mesh, slots=2, max_rhs=16, rtol=1e-10) as srv:
        futs = [srv.submit(m, sv) for m, sv in reqs[:6]]
        # two more requests arrive while the first ones are on the device
        while min(s.sweeps for s in srv.slots) < 1:
            time.sleep(0.0005)
        futs += [srv.submit(m, sv) for m, sv in reqs[6:]]
        mixed = [f.result(timeout=120) for f in futs]
        intervals = srv.device_intervals()
        logs = [s.log for s in srv.slots]
    for a, b in zip(alone, mixed):
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-12
    m, sv = reqs[3]
    orc = OracleDC3DNodal(mesh, sv, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    d0 = orc.dpred()
    assert np.linalg.norm(mixed[3] - d0) / np.linalg.norm(d0) < 1e-6
    # requests were admitted into solves that were already running (between two sweeps)
    joined = [(seq, sweep) for lg in logs for ev, seq, sweep, running in lg if ev == "admit" and running > 0]
    assert joined, logs
    # a sweep advanced the lanes of more than one request
    assert max(running for lg in logs for ev, _, _, running in lg if ev == "sweep") > 1
    # the two slots' sweeps overlapped on the device
    a_iv, b_iv = intervals
    assert any(a0 < b1 and b0 < a1 for a0, a1 in a_iv for b0, b1 in b_iv)


def test_memory_bounded(cuda):
    """Serving more requests does not grow the device memory beyond what the slots reserved at start
    (lane workspaces, staging arrays) plus the requests' electrode tables."""
    import torch

    mesh, reqs = _setup()
    with DCServer(mesh, slots=2, max_rhs=16, rtol=1e-10) as srv:
        for f in [srv.submit(m, sv) for m, sv in reqs]:
            f.result(timeout=120)
        torch.cuda.synchronize()
        base = torch.cuda.memory_allocated()
        torch.cuda.reset_peak_memory_stats()
        for _ in range(3):
            for f in [srv.submit(m, sv) for m, sv in reqs]:
                f.result(timeout=120)
        torch.cuda.synchronize()
        peak = torch.cuda.max_memory_allocated()
    assert peak - base < 4 << 20, (peak - base)


def test_bad_request_does_not_poison_others(cuda):
    mesh, reqs = _setup()
    with DCServer(mesh, slots=2, max_rhs=16, rtol=1e-10) as srv:
        bad = srv.submit(np.full(mesh.n_cells, np.nan), reqs[0][1])
        outside = Survey([sources.Pole([receivers.Pole(np.array([[0.0, 0.0, 0.0]]))], np.r_[1e5, 0.0, 0.0])])
        bad2 = srv.submit(reqs[0][0], outside)
        good = srv.submit(*reqs[1])
        with pytest.raises(ValueError):
            bad.result(timeout=120)
        with pytest.raises(ValueError):
            bad2.result(timeout=120)
        assert np.all(np.isfinite(good.result(timeout=120)))
