"""GPU Simulation3DCellCentered (and the cell-centred IP simulation) against the CPU oracle
(SuperLU on the assembled ``Div MfRhoI Grad``).

Tolerances: GPU solves to rtol 1e-10 or tighter; dpred, Jvec, Jtvec, getJ and getJtJdiag
within 1e-6 relative of the direct solves (2-norm); operator and derivative products, which
involve no solve, within 1e-12; the reference's analytic recipe within 5 % rms.
"""

import numpy as np
import pytest
import scipy.sparse as sp

from oracle.cc3d import OracleDC3DCellCentered
from oracle.ip3d import OracleIP3DCellCentered
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import Simulation3DCellCentered, receivers, sources
from simpeg_gb300.resistivity.survey import Survey

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _mesh():
    return TensorMesh([[(10.0, 3, -1.3), (10.0, 10), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 8), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 6)]], origin="CCN")


def _survey(appres=False):
    xs = np.arange(-40.0, 41.0, 10.0)
    dt = "apparent_resistivity" if appres else "volt"
    srcs = []
    for i in range(3):
        M = np.c_[xs[4:7], np.zeros(3), np.zeros(3)]
        N = np.c_[xs[5:8], np.zeros(3), np.zeros(3)]
        srcs.append(sources.Dipole([receivers.Dipole(M, N, data_type=dt)], np.r_[xs[i], 0, 0], np.r_[xs[i] + 10, 0, 0]))
    srcs.append(sources.Pole([receivers.Pole(np.c_[xs[:4], np.full(4, 10.0), np.zeros(4)], data_type=dt)],
                             np.r_[20.0, 10.0, 0.0]))
    srcs.append(sources.Dipole([receivers.Dipole(np.c_[xs[:3], np.full(3, -10.0), np.full(3, -15.0)],
                                                 np.c_[xs[1:4], np.full(3, -10.0), np.full(3, -15.0)])],
                               np.r_[3.0, -7.0, -12.0], np.r_[-21.0, 5.0, -31.0]))
    sv = Survey(srcs)
    if appres:
        sv.set_geometric_factor()
    return sv


def _model(mesh, seed=3):
    rng = np.random.default_rng(seed)
    return np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))


@pytest.mark.parametrize("bc", ["Robin", "Neumann", "Dirichlet"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dpred_jvec_jtvec_vs_oracle(cuda, bc, precision):
    mesh, survey = _mesh(), _survey()
    m = _model(mesh)
    orc = OracleDC3DCellCentered(mesh, survey, sigma_map=maps.ExpMap(mesh), bc_type=bc)
    orc.set_model(m)
    f = orc.fields()
    sim = Simulation3DCellCentered(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), bc_type=bc,
                                   precision=precision, rtol=1e-11)
    assert _rel(sim.dpred(m), orc.dpred(f=f)) < TOL
    rng = np.random.default_rng(7)
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.Jvec(m, v), orc.Jvec(m, v, f=f)) < TOL
    assert _rel(sim.Jtvec(m, w), orc.Jtvec(m, w, f=f)) < TOL


def test_rho_map_and_apparent_resistivity(cuda):
    mesh, survey = _mesh(), _survey(appres=True)
    rng = np.random.default_rng(11)
    rho = 10 ** rng.uniform(1.5, 2.5, mesh.n_cells)
    orc = OracleDC3DCellCentered(mesh, survey, rho_map=maps.IdentityMap(mesh))
    orc.set_model(rho)
    f = orc.fields()
    sim = Simulation3DCellCentered(mesh, survey=survey, rhoMap=maps.IdentityMap(mesh), rtol=1e-11)
    assert _rel(sim.dpred(rho), orc.dpred(f=f)) < TOL
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.Jvec(rho, v), orc.Jvec(rho, v, f=f)) < TOL
    assert _rel(sim.Jtvec(rho, w), orc.Jtvec(rho, w, f=f)) < TOL


@pytest.mark.parametrize("bc", ["Robin", "Neumann"])
def test_operator_and_derivatives_vs_oracle(cuda, bc):
    """getA (matrix-free stencil, row 0 pinned for Neumann) and getADeriv against the assembled
    oracle, without a solve."""
    mesh, survey = _mesh(), _survey()
    m = _model(mesh, 5)
    orc = OracleDC3DCellCentered(mesh, survey, sigma_map=maps.ExpMap(mesh), bc_type=bc)
    orc.set_model(m)
    sim = Simulation3DCellCentered(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), bc_type=bc)
    sim.model = m
    rng = np.random.default_rng(2)
    X = rng.standard_normal((mesh.n_cells, 3))
    A0 = orc.getA()
    assert _rel(sim.getA() @ X, A0 @ X) < 1e-12
    assert _rel(sim.getA().T @ X, A0.T @ X) < 1e-12
    u = rng.standard_normal((mesh.n_cells, 2))
    v = rng.standard_normal(mesh.n_cells)
    lam = rng.standard_normal((mesh.n_cells, 2))
    assert _rel(sim.getADeriv(u, v), orc.getADeriv(u, v)) < 1e-12
    assert _rel(sim.getADeriv(u, lam, adjoint=True), orc.getADeriv(u, lam, adjoint=True)) < 1e-12


def test_adjoint_identity_and_jtj(cuda):
    mesh, survey = _mesh(), _survey()
    m = _model(mesh, 9)
    sim = Simulation3DCellCentered(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-12, precision="fp64")
    rng = np.random.default_rng(42)
    v = rng.uniform(size=mesh.n_cells)
    w = rng.uniform(size=survey.nD)
    wJv = w @ sim.Jvec(m, v)
    assert abs(wJv - v @ sim.Jtvec(m, w)) <= 1e-8 * abs(wJv)
    orc = OracleDC3DCellCentered(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    f = orc.fields()
    W = sp.diags(rng.uniform(0.5, 2.0, survey.nD))
    J0 = np.array([orc.Jtvec(m, e, f=f) for e in np.eye(survey.nD)])
    assert _rel(sim.getJ(m), J0) < TOL
    sim2 = Simulation3DCellCentered(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-12, precision="fp64")
    assert _rel(sim2.getJtJdiag(m, W=W), ((W @ J0) ** 2).sum(axis=0)) < TOL


def test_face_fields_vs_oracle(cuda):
    """e, j on the faces and charge, charge density on the cells from the GPU potentials, against
    the oracle's sparse operators applied to the same potentials."""
    from scipy.constants import epsilon_0

    mesh, survey = _mesh(), _survey()
    m = _model(mesh, 13)
    sim = Simulation3DCellCentered(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    f = sim.fields(m)
    srcs = survey.source_list
    phi = f[srcs, "phi"]
    orc = OracleDC3DCellCentered(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    e0, j0 = orc.face_fields(phi)
    assert _rel(f[srcs, "e"], e0) < 1e-12
    assert _rel(f[srcs, "j"], j0) < 1e-12
    q0 = epsilon_0 * (orc.D @ e0)
    assert _rel(f[srcs, "charge"], q0) < 1e-12
    assert _rel(f[srcs, "charge_density"], q0 / mesh.cell_volumes[:, None]) < 1e-12


def test_analytic_halfspace_dipole_dipole(cuda):
    """The reference's analytic recipe (``tests/em/static/test_DC_analytic.py:83-103``): a dipole
    source on a 0.01 S/m half space, rms relative error of the dipole data < 5 %."""
    from oracle import analytic

    cs = 25.0
    hx = [(cs, 7, -1.3), (cs, 21), (cs, 7, 1.3)]
    mesh = TensorMesh([hx, hx, [(cs, 7, -1.3), (cs, 20)]], origin="CCN")
    x = mesh.cell_centers_x[(mesh.cell_centers_x > -100) & (mesh.cell_centers_x < 100)]
    y = mesh.cell_centers_y[(mesh.cell_centers_y > -100) & (mesh.cell_centers_y < 100)]
    X, Y = np.meshgrid(x, y, indexing="ij")
    M = np.c_[X.ravel(order="F") - 25.0, Y.ravel(order="F"), np.zeros(X.size)]
    N = np.c_[X.ravel(order="F") + 25.0, Y.ravel(order="F"), np.zeros(X.size)]
    A, B = np.r_[-200.0, 0, 0], np.r_[200.0, 0, 0]
    ana = analytic.dipole_dipole(A, B, M, N, 1e-2, earth_type="halfspace")
    survey = Survey([sources.Dipole([receivers.Dipole(M, N)], A, B)])
    for bc in ("Mixed", "Neumann"):
        sim = Simulation3DCellCentered(mesh, survey=survey, sigma=np.full(mesh.n_cells, 1e-2), bc_type=bc)
        d = sim.dpred()
        assert np.sqrt((((d - ana) / ana) ** 2).sum() / survey.nD) < 0.05


def test_ip_cell_centered_vs_oracle(cuda):
    from simpeg_gb300 import induced_polarization as ip

    mesh, survey = _mesh(), _survey()
    rng = np.random.default_rng(17)
    sigma = 10 ** rng.uniform(-2.5, -1.5, mesh.n_cells)
    eta = rng.uniform(0.0, 0.1, mesh.n_cells)
    orc = OracleIP3DCellCentered(mesh, survey, sigma=sigma, eta_map=maps.IdentityMap(mesh))
    sim = ip.Simulation3DCellCentered(mesh, survey=survey, sigma=sigma, etaMap=maps.IdentityMap(mesh), rtol=1e-11)
    assert _rel(sim.dpred(eta), orc.dpred(eta)) < TOL
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.Jvec(eta, v), orc.Jvec(eta, v)) < TOL
    assert _rel(sim.Jtvec(eta, w), orc.Jtvec(eta, w)) < TOL
