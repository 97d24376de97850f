"""GPU tests of the simulation's API edges: sensitivities through maps with a sparse
derivative (InjectActiveCells), the misfit's Hessian product at a given model, autograd
with a device model, and the Solver plug-in on the reference's Neumann-pinned matrix.

Tolerances: products through the GPU solves (rtol 1e-11) agree with each other to 1e-7
and with the oracle's SuperLU solves to 1e-6 (2-norm relative).
"""

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import Simulation3DNodal, receivers, sources
from simpeg_gb300.resistivity.survey import Survey

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case(seed=3):
    mesh = TensorMesh([[(10.0, 12)], [(10.0, 10)], [(10.0, 8)]], origin="CCN")
    xs = -50.0 + 10.0 * np.arange(11)
    src = []
    for i in range(4):
        rx = receivers.Dipole(np.c_[xs[i + 3:i + 6], np.zeros(3), np.zeros(3)],
                              np.c_[xs[i + 4:i + 7], np.zeros(3), np.zeros(3)])
        src.append(sources.Dipole([rx], np.r_[xs[i], 0.0, 0.0], np.r_[xs[i + 1], 0.0, 0.0]))
    rng = np.random.default_rng(seed)
    act = np.ones(mesh.n_cells, dtype=bool)
    act[rng.choice(mesh.n_cells, 60, replace=False)] = False
    return mesh, Survey(src), act, rng


def test_getj_and_jtj_diag_with_active_cells(cuda):
    """getJ is (nD, nP) under ExpMap * InjectActiveCells; its rows agree with Jvec/Jtvec and
    getJtJdiag equals the column sums of J^2 (the full-J path, the map being non-diagonal)."""
    mesh, survey, act, rng = _case()
    mp = maps.ComboMap([maps.ExpMap(), maps.InjectActiveCells(mesh, act, value_inactive=np.log(0.01))])
    nP = int(act.sum())
    m = np.log(10 ** rng.uniform(-2.5, -1.5, nP))
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=mp, precision="fp64", rtol=1e-11)
    J = sim.getJ(m)
    assert J.shape == (survey.nD, nP)
    v = rng.standard_normal(nP)
    w = rng.standard_normal(survey.nD)
    assert _rel(J @ v, sim.Jvec(m, v)) < 1e-7
    assert _rel(J.T @ w, sim.Jtvec(m, w)) < 1e-7
    W = sp.diags(rng.uniform(0.5, 2.0, survey.nD))
    sim2 = Simulation3DNodal(mesh, survey=survey, sigmaMap=mp, precision="fp64", rtol=1e-11)
    diag = sim2.getJtJdiag(m, W=W)
    assert diag.shape == (nP,)
    assert _rel(diag, ((W @ J) ** 2).sum(axis=0)) < 1e-7
    # the oracle on the same map: Jtvec through the injection's transpose
    orc = OracleDC3DNodal(mesh, survey, sigma_map=mp)
    orc.set_model(m)
    assert _rel(sim.Jtvec(m, w), orc.Jtvec(m, w)) < 1e-6


def test_device_products_with_active_cells(cuda):
    """jvec_dev / jtvec_dev (and so the misfit gradient) under a map with a sparse derivative."""
    import torch

    from simpeg_gb300.inversion import L2DataMisfit

    mesh, survey, act, rng = _case(5)
    mp = maps.ComboMap([maps.ExpMap(), maps.InjectActiveCells(mesh, act, value_inactive=np.log(0.01))])
    nP = int(act.sum())
    m = np.log(10 ** rng.uniform(-2.5, -1.5, nP))
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=mp, precision="fp64", rtol=1e-11)
    v = rng.standard_normal(nP)
    w = rng.standard_normal(survey.nD)
    sim.model = m
    jv = sim.jvec_dev(torch.from_numpy(v).to(cuda)).cpu().numpy()
    jtw = sim.jtvec_dev(torch.from_numpy(w).to(cuda)).cpu().numpy()
    assert _rel(jv, sim.Jvec(m, v)) < 1e-9
    assert _rel(jtw, sim.Jtvec(m, w)) < 1e-9
    dobs = sim.dpred(m) * 1.05
    dmis = L2DataMisfit(sim, dobs)
    g = dmis.deriv(m)
    assert _rel(g, 2.0 * sim.Jtvec(m, sim.dpred(m) - dobs)) < 1e-9


def test_deriv2_uses_the_given_model(cuda):
    """L2DataMisfit.deriv2(m, v) is the Hessian product at m even when another model was
    evaluated last."""
    from simpeg_gb300.inversion import L2DataMisfit

    mesh, survey, _, rng = _case(7)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    m_other = m + 0.3 * rng.standard_normal(mesh.n_cells)
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=1e-11)
    dobs = sim.dpred(m)
    dmis = L2DataMisfit(sim, dobs)
    v = rng.standard_normal(mesh.n_cells)
    h_at_m = dmis.deriv2(m, v)
    sim.dpred(m_other)  # the simulation now holds another model
    h_again = dmis.deriv2(m, v)
    assert _rel(h_again, h_at_m) < 1e-12
    ref = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=1e-11)
    assert _rel(h_at_m, 2.0 * ref.Jtvec(m, ref.Jvec(m, v))) < 1e-9


@pytest.mark.parametrize("miniaturize", [False, True])
def test_autograd_device_model(cuda, miniaturize):
    """A CUDA model goes through dpred's forward and backward on the device and gives what the
    host model gives."""
    import torch

    from simpeg_gb300.autograd import dpred

    mesh, survey, _, rng = _case(9)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=1e-11,
                            miniaturize=miniaturize)
    dobs = torch.from_numpy(sim.dpred(m) * 1.03)
    res = {}
    for where in ("cpu", "cuda"):
        mt = torch.tensor(m, device=where, requires_grad=True)
        r = dpred(sim, mt) - dobs.to(where)
        (0.5 * (r * r).sum()).backward()
        assert mt.grad.device.type == where
        res[where] = (r.detach().cpu().numpy(), mt.grad.cpu().numpy())
    assert _rel(res["cuda"][0], res["cpu"][0]) < 1e-10
    assert _rel(res["cuda"][1], res["cpu"][1]) < 1e-9
    # the device path did not need the model on the host
    sim2 = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=1e-11,
                             miniaturize=miniaturize)
    d2 = dpred(sim2, torch.tensor(m, device="cuda"))
    assert sim2._model is None and sim2._model_dev is not None
    assert _rel(d2.cpu().numpy(), sim.dpred(m)) < 1e-10


def test_gpu_solver_neumann_pinned(cuda):
    """GPUSolver on the reference's Neumann matrix (row 0 replaced by e0) equals SuperLU."""
    from simpeg_gb300.solver import GPUSolver

    mesh, survey, _, rng = _case(11)
    sigma = 10 ** rng.uniform(-2.5, -1.5, mesh.n_cells)
    orc = OracleDC3DNodal(mesh, survey, sigma=sigma, bc_type="Neumann")
    A = orc.getA().tocsr()
    assert abs(A - A.T).max() > 0  # the pinned row makes it non-symmetric
    B = rng.standard_normal((A.shape[0], 3))
    X0 = spla.splu(A.tocsc()).solve(B)
    Ainv = GPUSolver(A, rtol=1e-13)
    X = Ainv * B
    assert _rel(X, X0) < 1e-9
    assert _rel(Ainv * B[:, 0], X0[:, 0]) < 1e-9
    Ainv.clean()


def test_jtj_diag_concurrent_calls_with_different_tiles(cuda):
    """getJtJdiag of four simulations from four threads at once, on surveys with different
    electrode counts (different shared-memory tiles of the reciprocity kernel): every call
    succeeds and equals the simulation's serial result."""
    from concurrent.futures import ThreadPoolExecutor

    import torch

    mesh = TensorMesh([[(10.0, 12)], [(10.0, 10)], [(10.0, 8)]], origin="CCN")
    xs = -50.0 + 10.0 * np.arange(11)

    def survey(n_src):
        src = []
        for i in range(n_src):
            rx = receivers.Dipole(np.c_[xs[i + 3:i + 6], np.zeros(3), np.zeros(3)],
                                  np.c_[xs[i + 4:i + 7], np.zeros(3), np.zeros(3)])
            src.append(sources.Dipole([rx], np.r_[xs[i], 0.0, 0.0], np.r_[xs[i + 1], 0.0, 0.0]))
        return Survey(src)

    rng = np.random.default_rng(21)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    sims = [Simulation3DNodal(mesh, survey=survey(n), sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=1e-11)
            for n in (2, 4, 2, 4)]
    serial = [s.getJtJdiag(m).copy() for s in sims]

    def run(i):
        s = sims[i]
        out = []
        with torch.cuda.stream(torch.cuda.Stream()):
            for _ in range(5):
                s._gtgdiag = None
                out.append(s.getJtJdiag(m).copy())
            torch.cuda.current_stream().synchronize()
        return out

    with ThreadPoolExecutor(len(sims)) as ex:
        results = list(ex.map(run, range(len(sims))))
    for i, outs in enumerate(results):
        for d in outs:
            assert _rel(d, serial[i]) < 1e-12
