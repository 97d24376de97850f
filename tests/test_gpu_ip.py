"""GPU induced-polarization Simulation3DNodal vs the CPU IP oracle (SuperLU).

The IP data are the DC sensitivities at a fixed conductivity applied to the
chargeability (``induced_polarization/simulation.py:15-167``).  Solves run to
a relative residual of 1e-11; dpred, Jvec and Jtvec must match the
direct-solve oracle to 1e-7 relative (2-norm), getJtJdiag to 1e-6 (the
reciprocity kernel forms each datum's cell sensitivities in fp32).
"""

import numpy as np
import pytest

from oracle.dc3d import OracleDC3DNodal
from oracle.ip3d import OracleIP3DNodal
from simpeg_gb300 import maps
from simpeg_gb300.induced_polarization import Simulation3DNodal as IPSimulation3DNodal
from simpeg_gb300.induced_polarization import from_dc_to_ip_survey
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import Simulation3DNodal, receivers, sources
from simpeg_gb300.resistivity.survey import Survey

pytestmark = pytest.mark.gpu

TOL = 1e-7
TOL_JTJ = 1e-6


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _case(seed=0):
    """Dipole-dipole and pole sources; volt and apparent-chargeability receivers."""
    mesh = TensorMesh([[(10.0, 4, -1.3), (10.0, 12), (10.0, 4, 1.3)], [(10.0, 4, -1.3), (10.0, 8), (10.0, 4, 1.3)],
                       [(10.0, 4, -1.3), (10.0, 8)]], origin="CCN")
    xs = np.arange(-50.0, 51.0, 10.0)
    srcs = []
    for i in range(4):
        M = np.c_[xs[i + 2:i + 6], np.zeros(4), np.zeros(4)]
        N = np.c_[xs[i + 3:i + 7], np.zeros(4), np.zeros(4)]
        dtype = "apparent_chargeability" if i % 2 else "volt"
        srcs.append(sources.Dipole([receivers.Dipole(M, N, data_type=dtype)], np.r_[xs[i], 0, 0],
                                   np.r_[xs[i + 1], 0, 0]))
    srcs.append(sources.Pole([receivers.Pole(np.c_[xs[5:9], np.full(4, 10.0), np.zeros(4)],
                                             data_type="apparent_chargeability")], np.r_[-20.0, 10.0, 0.0]))
    rng = np.random.default_rng(seed)
    sigma = 10 ** rng.uniform(-2.5, -1.5, mesh.n_cells)
    eta = rng.uniform(0.0, 0.2, mesh.n_cells)
    return mesh, Survey(srcs), sigma, eta


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_ip_dpred_jvec_jtvec_jtjdiag_vs_oracle(cuda, precision):
    mesh, survey, sigma, eta = _case()
    sim = IPSimulation3DNodal(mesh, survey=survey, sigma=sigma, etaMap=maps.IdentityMap(mesh),
                              precision=precision, rtol=1e-11)
    orc = OracleIP3DNodal(mesh, survey, sigma, eta_map=maps.IdentityMap(mesh))
    rng = np.random.default_rng(1)
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.dpred(eta), orc.dpred(eta)) < TOL
    assert _rel(sim.Jvec(eta, v), orc.Jvec(eta, v)) < TOL
    assert _rel(sim.Jtvec(eta, w), orc.Jtvec(eta, w)) < TOL
    assert _rel(sim.getJtJdiag(eta), orc.getJtJdiag(eta)) < TOL_JTJ
    # the reference's adjoint recipe (tests/em/static/test_IP_jvecjtvecadj.py:146-156)
    vu, wu = rng.uniform(size=mesh.n_cells), rng.uniform(size=survey.nD)
    a, b = wu @ sim.Jvec(eta, vu), vu @ sim.Jtvec(eta, wu)
    assert abs(a - b) <= 1e-9 * abs(a)


def test_ip_weighted_jtjdiag_and_device_products(cuda):
    """getJtJdiag with misfit weights is diag(J^T diag(scale W)^2 J); the device-resident
    products used by the inversion equal the host Jvec / Jtvec."""
    import torch

    mesh, survey, sigma, eta = _case(seed=2)
    sim = IPSimulation3DNodal(mesh, survey=survey, sigma=sigma, etaMap=maps.IdentityMap(mesh), rtol=1e-11)
    orc = OracleIP3DNodal(mesh, survey, sigma, eta_map=maps.IdentityMap(mesh))
    wd = np.random.default_rng(3).uniform(0.5, 2.0, survey.nD)

    class W:
        def diagonal(self):
            return wd

    assert _rel(sim.getJtJdiag(eta, W=W()), orc.getJtJdiag(eta, W=wd)) < TOL_JTJ
    rng = np.random.default_rng(4)
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    sim.model = eta
    jv = sim.jvec_dev(torch.from_numpy(v).to(cuda)).cpu().numpy()
    jtw = sim.jtvec_dev(torch.from_numpy(w).to(cuda)).cpu().numpy()
    assert _rel(jv, sim.Jvec(eta, v)) < 1e-12
    assert _rel(jtw, sim.Jtvec(eta, w)) < 1e-12


def test_ip_forward_from_dc_fields(cuda):
    """tests/em/static/test_IP_fwd.py:48-74 on the GPU path: the IP simulation built
    from a DC simulation's fields at sigma_inf predicts DC(sigma0) - DC(sigma_inf),
    sigma0 = sigma_inf (1 - eta), with a mean squared relative error < 0.05; the
    same simulation without ``_f`` gives the same data; the model update does not
    solve again (the forward is linear in eta)."""
    cs = 12.5
    hx = [(cs, 2, -1.3), (cs, 21), (cs, 2, 1.3)]
    hz = [(cs, 2, -1.3), (cs, 20)]
    mesh = TensorMesh([hx, hx, hz], origin="CCN")
    x = mesh.cell_centers_x[(mesh.cell_centers_x > -80.0) & (mesh.cell_centers_x < 80.0)]
    y = mesh.cell_centers_y[(mesh.cell_centers_y > -80.0) & (mesh.cell_centers_y < 80.0)]
    M = TensorMesh._ndgrid(x - 12.5, y, np.r_[0.0])
    N = TensorMesh._ndgrid(x + 12.5, y, np.r_[0.0])
    inside = np.linalg.norm(mesh.cell_centers - np.r_[0.0, 0.0, -100.0], axis=1) < 50.0
    sigma_inf = np.full(mesh.n_cells, 1e-2)
    eta = np.where(inside, 0.1, 0.0)
    src = sources.Dipole([receivers.Dipole(M, N)], np.r_[-100.0, 0.0, 0.0], np.r_[100.0, 0.0, 0.0])
    survey_dc = Survey([src])
    dc = Simulation3DNodal(mesh, survey=survey_dc, sigmaMap=maps.IdentityMap(mesh), rtol=1e-11)
    d0 = dc.dpred(sigma_inf * (1.0 - eta))
    f_inf = dc.fields(sigma_inf)
    dinf = dc.dpred(sigma_inf, f=f_inf)
    ip = IPSimulation3DNodal(mesh, survey=from_dc_to_ip_survey(survey_dc), sigma=sigma_inf,
                             etaMap=maps.IdentityMap(mesh), Ainv=None, _f=f_inf, rtol=1e-11)
    d = ip.dpred(eta)
    full = d0 - dinf
    assert np.linalg.norm((d - full) / full) ** 2 / full.size < 0.05
    ip2 = IPSimulation3DNodal(mesh, survey=survey_dc, sigma=sigma_inf, etaMap=maps.IdentityMap(mesh), rtol=1e-11)
    assert _rel(ip2.dpred(eta), d) < 1e-9
    f_before = ip2._f
    np.testing.assert_allclose(ip2.dpred(2.0 * eta), 2.0 * ip2.dpred(eta), rtol=1e-9)
    assert ip2._f is f_before
    # the DC oracle gives the same DC difference
    orc = OracleDC3DNodal(mesh, survey_dc, sigma=sigma_inf)
    assert _rel(d, OracleIP3DNodal(mesh, survey_dc, sigma_inf, eta_map=maps.IdentityMap(mesh)).dpred(eta)) < TOL
    assert _rel(dinf, orc.dpred()) < TOL


def test_ip_rejects_conductivity_maps(cuda):
    mesh, survey, sigma, _ = _case()
    with pytest.raises(TypeError):
        IPSimulation3DNodal(mesh, survey=survey, sigma=sigma, sigmaMap=maps.ExpMap(mesh))
    with pytest.raises(ValueError):
        IPSimulation3DNodal(mesh, survey=survey, etaMap=maps.IdentityMap(mesh))
