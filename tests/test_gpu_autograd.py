"""Autograd backward (adjoint solve + dA/dsigma kernel) vs central finite
differences and vs the oracle's Jtvec, in fp64 and in mixed precision with
forward recomputation (the differentiation workload's checks at test size)."""

import numpy as np
import pytest

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300 import maps
from simpeg_gb300.resistivity import Simulation3DNodal
from simpeg_gb300.workloads import differentiation

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    # same construction as the 96x96x48 differentiation workload, at 24x24x16 cells
    mesh, m, survey = differentiation(seed=3, n_src=16, n_rx=6, ncore_xy=8, ncore_z=8, core_h=10.0)
    return mesh, m, survey


@pytest.mark.parametrize("precision,recompute", [("fp64", False), ("mixed", True)])
def test_misfit_gradient_vs_central_fd(cuda, case, precision, recompute):
    import torch

    from simpeg_gb300.autograd import dpred

    mesh, m, survey = case
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=1e-12)
    rng = np.random.default_rng(0)
    d0 = sim.dpred(m)
    dobs = torch.from_numpy(d0 * (1 + 0.05 * rng.standard_normal(d0.size)))

    def phi(mm):
        r = dpred(sim, mm, recompute=recompute) - dobs
        return 0.5 * (r * r).sum()

    mt = torch.tensor(m, requires_grad=True)
    f = phi(mt)
    f.backward()
    g = mt.grad.numpy()
    h = 1e-4
    errs = []
    for _ in range(8):
        v = rng.standard_normal(m.size)
        v /= np.linalg.norm(v)
        with torch.no_grad():
            fp = phi(torch.from_numpy(m + h * v)).item()
            fm = phi(torch.from_numpy(m - h * v)).item()
        fd = (fp - fm) / (2 * h)
        errs.append(abs(fd - g @ v) / max(abs(fd), 1e-30))
    # central differences with h = 1e-4: O(h^2) truncation, solves at 1e-12
    assert max(errs) < 1e-5, errs


def test_autograd_gradient_matches_oracle_jtvec(cuda, case):
    import torch

    from simpeg_gb300.autograd import dpred

    mesh, m, survey = case
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=1e-10)
    rng = np.random.default_rng(1)
    w = rng.standard_normal(survey.nD)
    mt = torch.tensor(m, requires_grad=True)
    (dpred(sim, mt) * torch.from_numpy(w)).sum().backward()
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    g0 = orc.Jtvec(m, w)
    g = mt.grad.numpy()
    assert np.linalg.norm(g - g0) / np.linalg.norm(g0) < 1e-6
