"""The DC server on the GPU: each request's result is the same alone and in
the mix (concurrent slots, same-model requests merged into one solve).

Tolerance: solves run to rtol 1e-10, so alone and mixed results agree to
1e-8 relative; one request is also checked against the CPU oracle (1e-6)."""

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
            (models[2], survey(3, 4)), (models[1], survey(4, 1)), (models[2], survey(5, 6))]
    return mesh, reqs


def test_alone_equals_mixed(cuda):
    mesh, reqs = _setup()
    alone = []
    with DCServer(mesh, slots=1, max_rhs=16, rtol=1e-10) as srv:
        for m, sv in reqs:
            alone.append(srv.submit(m, sv).result(timeout=120))
    with DCServer(mesh, slots=3, max_rhs=16, rtol=1e-10) as srv:
        futs = [srv.submit(m, sv) for m, sv in reqs]
        mixed = [f.result(timeout=120) for f in futs]
        merged = [b for s in srv.slots for b in s.batches if len(b) > 1]
    for a, b in zip(alone, mixed):
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-8
    m, sv = reqs[3]
    orc = OracleDC3DNodal(mesh, sv, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    d0 = orc.dpred()
    assert np.linalg.norm(mixed[3] - d0) / np.linalg.norm(d0) < 1e-6
    assert isinstance(merged, list)


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
