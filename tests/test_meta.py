"""Meta-simulations (simpeg/meta/simulation.py) over child simulations.

The host logic is pinned on the CPU with oracle-backed children (direct
solves), after the reference's own recipe (tests/meta/test_meta_sim.py:12-98:
a survey split into source chunks must reproduce the full simulation); the
GPU tests run the same recipe with GPU children solving concurrently.
"""

import numpy as np
import pytest
import scipy.sparse as sp

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.meta import (MetaSimulation, MultiprocessingMetaSimulation, RepeatedSimulation,
                               SumMetaSimulation)
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.survey import Survey


class _OracleSim:
    """Simulation-like wrapper of the CPU oracle (IdentityMap conductivity model)."""

    def __init__(self, mesh, survey):
        self.survey = survey
        self.sigmaMap = maps.IdentityMap(mesh)
        self._o = OracleDC3DNodal(mesh, survey, sigma_map=self.sigmaMap)
        self._model = None

    @property
    def model(self):
        return self._model

    @model.setter
    def model(self, m):
        self._model = None if m is None else np.asarray(m, dtype=np.float64)
        self._o.set_model(self._model)

    def fields(self, m):
        self.model = m
        return self._o.fields()

    def dpred(self, m=None, f=None):
        if m is not None:
            self.model = m
        return self._o.dpred(f=f)

    def Jvec(self, m, v, f=None):
        self.model = m
        return self._o.Jvec(m, v, f=f)

    def Jtvec(self, m, v, f=None):
        self.model = m
        return self._o.Jtvec(m, v, f=f)

    def getJtJdiag(self, m, W=None, f=None):
        self.model = m
        return self._o.getJtJdiag(m, W=W, f=f)


def _split_case():
    """tests/meta/test_meta_sim.py:13-58: 10 pole sources, 25 pole receivers, chunks of 3."""
    mesh = TensorMesh([16, 16, 16], origin="CCN")
    rx_locs = np.mgrid[-0.25:0.25:5j, -0.25:0.25:5j, 0:1:1j].reshape(3, -1).T
    src_locs = np.mgrid[-0.5:0.5:10j, 0:1:1j, 0:1:1j].reshape(3, -1).T
    src_list = [sources.Pole([receivers.Pole(rx_locs)], location=loc) for loc in src_locs]
    chunks = [src_list[i:i + 3] for i in range(0, len(src_list), 3)]
    m = np.arange(mesh.n_cells) / mesh.n_cells + 0.1
    return mesh, src_list, chunks, m


def _check_split(full, meta, m, nD, rtol, rtol_diag):
    f_full = full.fields(m)
    f_meta = meta.fields(m)
    assert len(f_meta) == len(meta.simulations)
    rng = np.random.default_rng(0)
    u = rng.random(m.size)
    v = rng.random(nD)
    np.testing.assert_allclose(meta.dpred(m, f=f_meta), full.dpred(m, f=f_full), rtol=rtol)
    np.testing.assert_allclose(meta.Jvec(m, u, f=f_meta), full.Jvec(m, u, f=f_full), rtol=rtol)
    np.testing.assert_allclose(meta.Jtvec(m, v, f=f_meta), full.Jtvec(m, v, f=f_full), rtol=rtol)
    np.testing.assert_allclose(meta.getJtJdiag(m, f=f_meta), full.getJtJdiag(m, f=f_full), rtol=rtol_diag)
    # without the optional fields, and with a (sparse) data weighting
    meta.model = m
    np.testing.assert_allclose(meta.dpred(), full.dpred(m, f=f_full), rtol=rtol)
    np.testing.assert_allclose(meta.Jtvec(m, v), full.Jtvec(m, v, f=f_full), rtol=rtol)
    meta._jtjdiag = None
    np.testing.assert_allclose(meta.getJtJdiag(m, W=sp.eye(nD)), full.getJtJdiag(m, f=f_full), rtol=rtol_diag)


def test_meta_source_chunks_equal_full_oracle():
    mesh, src_list, chunks, m = _split_case()
    full = _OracleSim(mesh, Survey(src_list))
    sims = [_OracleSim(mesh, Survey(c)) for c in chunks]
    meta = MetaSimulation(sims, [maps.IdentityMap() for _ in sims], concurrent=False)
    assert meta.survey.nD == full.survey.nD and list(meta.survey.vnD) == [s.survey.nD for s in sims]
    _check_split(full, meta, m, full.survey.nD, 1e-10, 1e-10)


def test_sum_and_repeated_meta_oracle():
    """SumMetaSimulation adds the children's data; RepeatedSimulation evaluates one
    simulation under several mappings (simpeg/meta/simulation.py:332-520)."""
    mesh, src_list, chunks, m = _split_case()
    survey = Survey(src_list[:4])
    a, b = _OracleSim(mesh, survey), _OracleSim(mesh, Survey(src_list[:4]))
    scale2 = sp.diags(np.full(mesh.n_cells, 2.0))

    class Scale2(maps.IdentityMap):
        def _transform(self, x):
            return 2.0 * np.asarray(x, dtype=np.float64).ravel()

        def deriv(self, x, v=None):
            return scale2 @ v if v is not None else scale2

    summ = SumMetaSimulation([a, b], [maps.IdentityMap(), Scale2()], concurrent=False)
    ref_a, ref_b = _OracleSim(mesh, survey), _OracleSim(mesh, survey)
    d = summ.dpred(m)
    np.testing.assert_allclose(d, ref_a.dpred(m) + ref_b.dpred(2.0 * m), rtol=1e-10)
    rng = np.random.default_rng(1)
    u, w = rng.random(m.size), rng.random(survey.nD)
    np.testing.assert_allclose(w @ summ.Jvec(m, u), u @ summ.Jtvec(m, w), rtol=1e-10)
    rep = RepeatedSimulation(_OracleSim(mesh, survey), [maps.IdentityMap(), Scale2()])
    assert rep.survey.nD == 2 * survey.nD
    np.testing.assert_allclose(rep.dpred(m), np.r_[ref_a.dpred(m), ref_b.dpred(2.0 * m)], rtol=1e-10)
    np.testing.assert_allclose(w @ rep.Jvec(m, u)[:survey.nD] + w @ rep.Jvec(m, u)[survey.nD:],
                               u @ rep.Jtvec(m, np.r_[w, w]), rtol=1e-10)


def test_meta_validation():
    mesh, src_list, chunks, m = _split_case()
    sims = [_OracleSim(mesh, Survey(c)) for c in chunks[:2]]
    with pytest.raises(ValueError):
        MetaSimulation(sims, [maps.IdentityMap()], concurrent=False)
    with pytest.raises(ValueError):
        MetaSimulation([sims[0], sims[0]], [maps.IdentityMap()] * 2, concurrent=False)
    with pytest.raises(ValueError):
        MetaSimulation(sims, [maps.IdentityMap(nP=4), maps.IdentityMap(nP=5)], concurrent=False)
    with pytest.raises(ValueError):
        SumMetaSimulation([_OracleSim(mesh, Survey(chunks[0])), _OracleSim(mesh, Survey(chunks[-1]))],
                          [maps.IdentityMap()] * 2, concurrent=False)


@pytest.mark.gpu
@pytest.mark.parametrize("cls", ["meta", "multiprocessing"])
def test_meta_source_chunks_equal_full_gpu(cuda, cls):
    """The reference recipe with GPU children solving at the same time on their own streams."""
    from simpeg_gb300.resistivity import Simulation3DNodal

    mesh, src_list, chunks, m = _split_case()

    def sim(s):
        return Simulation3DNodal(mesh, survey=Survey(s), sigmaMap=maps.IdentityMap(), rtol=1e-11)

    full = sim(src_list)
    sims = [sim(c) for c in chunks]
    mp = [maps.IdentityMap() for _ in sims]
    meta = MetaSimulation(sims, mp) if cls == "meta" else MultiprocessingMetaSimulation(sims, mp, n_processes=2)
    assert meta.concurrent
    _check_split(full, meta, m, full.survey.nD, 1e-8, 1e-6)
