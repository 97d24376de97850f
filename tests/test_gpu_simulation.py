"""GPU Simulation3DNodal vs the CPU oracle (SuperLU) on the 32x32x16 block model.

Tolerance: the GPU solves run to a relative residual of 1e-10 (fp64 or
fp32-inner + fp64 refinement); dpred, Jvec and Jtvec must match the direct
solve to 1e-6 relative (2-norm over the data / model vector).
"""

import numpy as np
import pytest

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300 import maps
from simpeg_gb300.resistivity import Simulation3DNodal, receivers, sources
from simpeg_gb300.resistivity.survey import Survey
from simpeg_gb300.workloads import block_model_survey

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def block_case():
    mesh, sigma, survey, _ = block_model_survey(seed=0)
    m = np.log(sigma)
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    f = orc.fields()
    return mesh, survey, m, orc, f


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dpred_jvec_jtvec_vs_oracle(cuda, block_case, precision):
    mesh, survey, m, orc, f = block_case
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=1e-10)
    d = sim.dpred(m)
    assert _rel(d, orc.dpred(f=f)) < TOL
    rng = np.random.default_rng(7)
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.Jvec(m, v), orc.Jvec(m, v, f=f)) < TOL
    assert _rel(sim.Jtvec(m, w), orc.Jtvec(m, w, f=f)) < TOL


def test_adjoint_identity_gpu(cuda, block_case):
    mesh, survey, m, _, _ = block_case
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    rng = np.random.default_rng(42)
    v = rng.uniform(size=mesh.n_cells)
    w = rng.uniform(size=survey.nD)
    wJv = w @ sim.Jvec(m, v)
    vJtw = v @ sim.Jtvec(m, w)
    assert abs(wJv - vJtw) <= 1e-8 * abs(wJv)


def test_jtj_diag_vs_oracle(cuda):
    mesh = _small_mesh()
    survey = _small_survey()
    rng = np.random.default_rng(3)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    f = orc.fields()
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    J = sim.getJ(m)
    J0 = orc.getJ(m, f=f)
    assert _rel(J, J0) < TOL
    # reciprocity kernel: fp32 cell arithmetic on fp64 pole solutions staged relative to the tile
    # centre, fp64 accumulation of the per-thread sums (the fp64 reference is 1e-6 away at most)
    diag = sim.getJtJdiag(m)
    diag0 = orc.getJtJdiag(m, f=f)
    assert np.max(np.abs(diag - diag0) / np.abs(diag0).max()) < 1e-6
    assert _rel(diag, diag0) < 1e-6


def test_jtj_diag_weighted_appres(cuda):
    import scipy.sparse as sp

    mesh = _small_mesh()
    survey = _small_survey(appres=True)
    rng = np.random.default_rng(8)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m)
    W = sp.diags(rng.uniform(0.5, 2.0, survey.nD))
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    assert _rel(sim.getJtJdiag(m, W=W), orc.getJtJdiag(m, W=W)) < 1e-6


def _small_mesh():
    from simpeg_gb300.mesh import TensorMesh

    return TensorMesh([[(10.0, 3, -1.3), (10.0, 8), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 6), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 5)]], origin="CCN")


def _small_survey(appres=False):
    xs = np.arange(-30.0, 31.0, 10.0)
    srcs = []
    dt = "apparent_resistivity" if appres else "volt"
    for i in range(3):
        M = np.c_[xs[3:6], np.zeros(3), np.zeros(3)]
        N = np.c_[xs[4:7], np.zeros(3), np.zeros(3)]
        srcs.append(sources.Dipole([receivers.Dipole(M, N, data_type=dt)], np.r_[xs[i], 0, 0], np.r_[xs[i] - 10, 0, 0]))
    srcs.append(sources.Pole([receivers.Pole(np.c_[xs[:4], np.full(4, 10.0), np.zeros(4)], data_type=dt)],
                             np.r_[20.0, 10.0, 0.0]))
    sv = Survey(srcs)
    if appres:
        sv.set_geometric_factor()
    return sv


def test_rho_map_and_apparent_resistivity(cuda):
    mesh = _small_mesh()
    survey = _small_survey(appres=True)
    rng = np.random.default_rng(11)
    rho = 10 ** rng.uniform(1.5, 2.5, mesh.n_cells)
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ComboMap([maps.ReciprocalMap(), maps.IdentityMap(mesh)]))
    orc.set_model(rho)
    f = orc.fields()
    sim = Simulation3DNodal(mesh, survey=survey, rhoMap=maps.IdentityMap(mesh), rtol=1e-11)
    assert _rel(sim.dpred(rho), orc.dpred(f=f)) < TOL
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.Jvec(rho, v), orc.Jvec(rho, v, f=f)) < TOL
    assert _rel(sim.Jtvec(rho, w), orc.Jtvec(rho, w, f=f)) < TOL


def test_miniaturize_matches_full(cuda, block_case):
    """tests/em/static/test_DC_miniaturize.py: dpred/Jvec/Jtvec equal with and without miniaturize."""
    mesh, survey, m, _, _ = block_case
    a = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    b = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11, miniaturize=True)
    assert _rel(b.dpred(m), a.dpred(m)) < TOL
    rng = np.random.default_rng(1)
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(b.Jvec(m, v), a.Jvec(m, v)) < TOL
    assert _rel(b.Jtvec(m, w), a.Jtvec(m, w)) < TOL


def test_fields_indexing(cuda, block_case):
    mesh, survey, m, orc, f0 = block_case
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    f = sim.fields(m)
    src = survey.source_list[3]
    assert _rel(f[src, "phiSolution"], f0[:, 3]) < TOL
    allp = f[:, "phi"]
    assert allp.shape == (mesh.n_nodes, survey.nSrc)


def test_bad_inputs_raise(cuda):
    mesh = _small_mesh()
    survey = _small_survey()
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.IdentityMap(mesh))
    with pytest.raises(ValueError):
        sim.dpred(-np.ones(mesh.n_cells))
    bad = Survey([sources.Pole([receivers.Pole(np.array([[0.0, 0.0, 0.0]]))], np.r_[1e5, 0.0, 0.0])])
    sim2 = Simulation3DNodal(mesh, survey=bad, sigmaMap=maps.IdentityMap(mesh))
    with pytest.raises(ValueError):
        sim2.dpred(np.ones(mesh.n_cells) * 0.01)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_golden_block_model(cuda, precision):
    """GPU path vs the committed oracle fixture (tests/golden/make_golden.py)."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "block_model_oracle.npz"))
    mesh, sigma, survey, _ = block_model_survey(seed=0)
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=1e-10)
    m = g["m"]
    assert _rel(sim.dpred(m), g["dpred"]) < TOL
    assert _rel(sim.Jvec(m, g["v"]), g["jvec"]) < TOL
    assert _rel(sim.Jtvec(m, g["w"]), g["jtvec"]) < TOL


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_neumann_matches_oracle(cuda, precision):
    """bc_type='Neumann': the reference pins row 0 of A (simulation.py:535-540)."""
    mesh = _small_mesh()
    survey = _small_survey()
    rng = np.random.default_rng(21)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh), bc_type="Neumann")
    orc.set_model(m)
    f = orc.fields()
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), bc_type="Neumann",
                            precision=precision, rtol=1e-11)
    assert _rel(sim.fields(m)[:, "phi"], f) < TOL
    assert _rel(sim.dpred(m), orc.dpred(f=f)) < TOL
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    assert _rel(sim.Jvec(m, v), orc.Jvec(m, v, f=f)) < TOL
    assert _rel(sim.Jtvec(m, w), orc.Jtvec(m, w, f=f)) < TOL


@pytest.mark.parametrize("bc", ["Robin", "Neumann"])
def test_analytic_halfspace_gpu(cuda, bc):
    """tests/em/static/test_DC_analytic.py:48-81 on the GPU path: rms relative error < 5 %."""
    from oracle import analytic
    from simpeg_gb300.mesh import TensorMesh

    cs = 25.0
    hx = [(cs, 7, -1.3), (cs, 21), (cs, 7, 1.3)]
    hz = [(cs, 7, -1.3), (cs, 20)]
    mesh = TensorMesh([hx, hx, hz], origin="CCN")
    x = mesh.cell_centers_x[(mesh.cell_centers_x > -100) & (mesh.cell_centers_x < 100)]
    y = mesh.cell_centers_y[(mesh.cell_centers_y > -100) & (mesh.cell_centers_y < 100)]
    A = np.r_[-200.0, 0.0, 0.0]
    B = np.r_[200.0, 0.0, 0.0]
    M = TensorMesh._ndgrid(x - 25.0, y, np.r_[0.0])
    N = TensorMesh._ndgrid(x + 25.0, y, np.r_[0.0])
    ana = analytic.pole_dipole(A, M, N, 1e-2, earth_type="halfspace") - analytic.pole_dipole(
        B, M, N, 1e-2, earth_type="halfspace")
    survey = Survey([sources.Dipole([receivers.Dipole(M, N)], A, B)])
    sim = Simulation3DNodal(mesh, survey=survey, sigma=np.full(mesh.n_cells, 1e-2), bc_type=bc, rtol=1e-10)
    d = sim.dpred()
    err = np.sqrt((((d - ana) / ana) ** 2).sum() / survey.nD)
    assert err < 0.05, err


def test_derived_fields_vs_oracle(cuda, block_case):
    """Fields3DNodal e, j, charge, charge_density (resistivity/fields.py:214-253):
    the device kernels applied to the GPU potentials equal the oracle's sparse
    operators applied to the same potentials (fp64, summation order only)."""
    from scipy.constants import epsilon_0

    mesh, survey, m, orc, _ = block_case
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-10)
    f = sim.fields(m)
    phi = f[:, "phi"]
    e0, j0, q0, rho0 = orc.derived_fields(phi, epsilon_0)
    for name, ref in (("e", e0), ("j", j0), ("charge", q0), ("charge_density", rho0)):
        got = f[:, name]
        assert got.shape == ref.shape, name
        assert _rel(got, ref) < 1e-12, (name, _rel(got, ref))
    src = survey.source_list[3]
    np.testing.assert_allclose(f[src, "e"], e0[:, 3], rtol=1e-12, atol=1e-12 * np.abs(e0).max())
    assert f._GLoc("e") == "E" and f._GLoc("phi") == "N"


def test_multipole_fullspace_fields_gpu(cuda):
    """tests/em/static/test_DC_FieldsMultipoleFullspace.py:284-305 on the GPU path: a
    Multipole source in a whole space; f[src_list, "e"] and "j" within 10 % of the analytic
    field on the region of interest, charge and charge density available."""
    from test_oracle import _multipole_fullspace

    mesh, sigma, survey, e_ana, roi = _multipole_fullspace()
    sim = Simulation3DNodal(mesh, survey=survey, sigma=sigma, rtol=1e-10)
    f = sim.fields()
    e = f[survey.source_list, "e"].ravel()
    j = f[survey.source_list, "j"].ravel()
    assert _rel(e[roi], e_ana[roi]) < 0.1
    assert _rel(j[roi], 1e-2 * e_ana[roi]) < 0.1
    assert np.all(np.isfinite(f[:, "charge"])) and np.all(np.isfinite(f[:, "charge_density"]))


@pytest.mark.parametrize("bc", ["Robin", "Neumann"])
def test_getA_and_getADeriv_vs_oracle(cuda, bc):
    """getA (simulation.py:523-555; row 0 pinned for Neumann) as an operator, A^T, and
    getADeriv forward / adjoint (simulation.py:557-571) through the ExpMap, against the
    oracle's assembled matrices (fp64 stencil: rounding-level agreement)."""
    mesh = _small_mesh()
    survey = _small_survey()
    rng = np.random.default_rng(31)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh), bc_type=bc)
    orc.set_model(m)
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), bc_type=bc)
    sim.model = m
    A0 = orc.getA()
    A = sim.getA()
    X = rng.standard_normal((mesh.n_nodes, 3))
    assert _rel(A @ X, A0 @ X) < 1e-12
    assert _rel(A @ X[:, 0], A0 @ X[:, 0]) < 1e-12
    assert _rel(A.T @ X[:, 1], A0.T @ X[:, 1]) < 1e-12
    u = rng.standard_normal(mesh.n_nodes)
    v = rng.standard_normal(mesh.n_cells)
    lam = rng.standard_normal(mesh.n_nodes)
    assert _rel(sim.getADeriv(u, v), orc.getADeriv(u, v)) < 1e-12
    assert _rel(sim.getADeriv(u, lam, adjoint=True), orc.getADeriv(u, lam, adjoint=True)) < 1e-12
    U = rng.standard_normal((mesh.n_nodes, 2))
    assert _rel(sim.getADeriv(U, v), orc.getADeriv(U, v)) < 1e-12
