"""Pins of the CPU oracle against the reference's own test recipes (no GPU).

The reference has no golden vectors for this path; its DC tests pin the
physics with an analytic half-space (tests/em/static/test_DC_analytic.py),
the adjoint identity and Taylor derivative order
(tests/em/static/test_DC_jvecjtvecadj.py), custom-surface equality
(tests/em/static/test_DC_Boundaries.py) and source-chunk equality
(tests/meta/test_meta_sim.py).  The same recipes are applied here to the
oracle.
"""

import numpy as np
import pytest

from oracle import analytic
from oracle.dc3d import OracleDC3DNodal
from oracle.operators import MeshOps
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.survey import Survey


def _analytic_setup():
    cs = 25.0
    npad = 7
    hx = [(cs, npad, -1.3), (cs, 21), (cs, npad, 1.3)]
    hz = [(cs, npad, -1.3), (cs, 20)]
    mesh = TensorMesh([hx, hx, hz], origin="CCN")
    x = mesh.cell_centers_x[(mesh.cell_centers_x > -100) & (mesh.cell_centers_x < 100)]
    y = mesh.cell_centers_y[(mesh.cell_centers_y > -100) & (mesh.cell_centers_y < 100)]
    A = np.r_[-200.0, 0.0, 0.0]
    B = np.r_[200.0, 0.0, 0.0]
    M = TensorMesh._ndgrid(x - 25.0, y, np.r_[0.0])
    N = TensorMesh._ndgrid(x + 25.0, y, np.r_[0.0])
    ana = analytic.pole_dipole(A, M, N, 1e-2, earth_type="halfspace") - analytic.pole_dipole(
        B, M, N, 1e-2, earth_type="halfspace")
    rx = receivers.Dipole(M, N)
    src = sources.Dipole([rx], A, B)
    return mesh, Survey([src]), ana


@pytest.mark.slow
def test_analytic_halfspace_robin():
    """tests/em/static/test_DC_analytic.py:69-81: rms relative error < 5 %."""
    mesh, survey, ana = _analytic_setup()
    o = OracleDC3DNodal(mesh, survey, sigma=np.full(mesh.n_cells, 1e-2), bc_type="Robin")
    d = o.dpred()
    err = np.sqrt((((d - ana) / ana) ** 2).sum() / survey.nD)
    assert err < 0.05, err


def _small_problem(seed=0, rho=False):
    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 8), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 6), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 5)]], origin="CCN")
    xs = np.arange(-30.0, 31.0, 10.0)
    srcs = []
    for i in range(3):
        M = np.c_[xs[3:6], np.zeros(3), np.zeros(3)]
        N = np.c_[xs[4:7], np.zeros(3), np.zeros(3)]
        srcs.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[xs[i], 0, 0], np.r_[xs[i] - 10, 0, 0]))
    srcs.append(sources.Pole([receivers.Pole(np.c_[xs[:4], np.full(4, 10.0), np.zeros(4)])], np.r_[20.0, 10.0, 0.0]))
    survey = Survey(srcs)
    rng = np.random.default_rng(seed)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    return mesh, survey, m


def test_adjoint_identity():
    """tests/em/static/test_DC_jvecjtvecadj.py:264-274: |w.Jv - v.Jtw| < 1e-8."""
    mesh, survey, m = _small_problem()
    o = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    o.set_model(m)
    f = o.fields()
    rng = np.random.default_rng(42)
    v = rng.uniform(size=mesh.n_cells)
    w = rng.uniform(size=survey.nD)
    wJv = w @ o.Jvec(m, v, f=f)
    vJtw = v @ o.Jtvec(m, w, f=f)
    assert abs(wJv - vJtw) < 1e-8 * max(1.0, abs(wJv)), (wJv, vJtw)


def test_taylor_derivative_order():
    """discretize.tests.check_derivative recipe: second-order Taylor decay."""
    mesh, survey, m = _small_problem(seed=1)
    o = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    o.set_model(m)
    f = o.fields()
    d0 = o.dpred(f=f)
    rng = np.random.default_rng(562)
    dm = rng.standard_normal(mesh.n_cells) * 0.1
    Jdm = o.Jvec(m, dm, f=f)
    e1, e2 = [], []
    hs = [1e-1, 1e-2, 1e-3]
    for h in hs:
        o.set_model(m + h * dm)
        dh = o.dpred()
        e1.append(np.linalg.norm(dh - d0))
        e2.append(np.linalg.norm(dh - d0 - h * Jdm))
    order1 = np.log10(e1[0] / e1[-1]) / 2
    order2 = np.log10(e2[0] / e2[-1]) / 2
    assert order1 > 0.9 and order2 > 1.8, (order1, order2)


def test_custom_surface_faces_equal_default():
    """tests/em/static/test_DC_Boundaries.py:35-50: explicit top faces == default."""
    mesh = TensorMesh([8, 9, 10])
    ops = MeshOps(mesh.h, mesh.origin)
    bf = ops.boundary_faces()
    top = bf["centers"][:, -1] == bf["centers"][:, -1].max()
    src = sources.Pole([], np.r_[0.5, 0.5, 1.0])
    sigma = np.full(mesh.n_cells, 0.1)
    o1 = OracleDC3DNodal(mesh, Survey([src]), sigma=sigma)
    o2 = OracleDC3DNodal(mesh, Survey([src]), sigma=sigma, surface_faces=top)
    np.testing.assert_equal(o1.fields(), o2.fields())


def test_source_chunks_equal_full():
    """tests/meta/test_meta_sim.py:12-100: chunked sources reproduce the full simulation."""
    mesh = TensorMesh([16, 16, 16], origin="CCN")
    rx_locs = np.mgrid[-0.25:0.25:5j, -0.25:0.25:5j, 0:1:1j].reshape(3, -1).T
    src_locs = np.mgrid[-0.5:0.5:10j, 0:1:1j, 0:1:1j].reshape(3, -1).T
    src_list = [sources.Pole([receivers.Pole(rx_locs)], loc) for loc in src_locs]
    m = np.arange(mesh.n_cells) / mesh.n_cells + 0.1
    full = OracleDC3DNodal(mesh, Survey(src_list), sigma_map=maps.IdentityMap(mesh))
    full.set_model(m)
    ff = full.fields()
    d_full = full.dpred(f=ff)
    rng = np.random.default_rng(0)
    u = rng.random(mesh.n_cells)
    v = rng.random(d_full.size)
    jv_full = full.Jvec(m, u, f=ff)
    jtv_full = full.Jtvec(m, v, f=ff)
    d_parts, jv_parts, jtv_sum, start = [], [], 0, 0
    for i in range(0, len(src_list), 3):
        sub = OracleDC3DNodal(mesh, Survey(src_list[i:i + 3]), sigma_map=maps.IdentityMap(mesh))
        sub.set_model(m)
        fs = sub.fields()
        d = sub.dpred(f=fs)
        d_parts.append(d)
        jv_parts.append(sub.Jvec(m, u, f=fs))
        jtv_sum = jtv_sum + sub.Jtvec(m, v[start:start + d.size], f=fs)
        start += d.size
    np.testing.assert_allclose(np.hstack(d_parts), d_full)
    np.testing.assert_allclose(np.hstack(jv_parts), jv_full)
    np.testing.assert_allclose(jtv_sum, jtv_full, rtol=1e-7, atol=1e-12 * np.abs(jtv_full).max())


def test_jtj_diag_matches_full_J():
    mesh, survey, m = _small_problem(seed=3)
    o = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    o.set_model(m)
    f = o.fields()
    J = o.getJ(m, f=f)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(mesh.n_cells)
    np.testing.assert_allclose(J @ v, o.Jvec(m, v, f=f), rtol=1e-8, atol=1e-14)
    diag = o.getJtJdiag(m, f=f)
    np.testing.assert_allclose(diag, (J * J).sum(axis=0), rtol=1e-12)


def test_operator_hand_checked_2x1x1():
    """A on a 2x1x1-cell mesh written out by hand (Neumann part)."""
    mesh = TensorMesh([[1.0, 2.0], [1.0], [1.0]])
    o = OracleDC3DNodal(mesh, Survey([sources.Pole([], np.r_[0.0, 0.0, 0.0])]), sigma=np.array([1.0, 3.0]),
                        bc_type="Neumann")
    G = o.G
    Me = o.E @ np.array([1.0, 3.0])
    # x-edges of cell 0 carry sigma*V/4 = 1*1/4; of cell 1: 3*2/4
    np.testing.assert_allclose(Me[:8], [0.25, 1.5] * 4)
    A = (G.T @ np.diag(Me) @ G)
    # coupling between nodes 0 and 1 along x: -Me/hx^2
    assert np.isclose(A[0, 1], -0.25)
    assert np.isclose(A[1, 2], -1.5 / 4.0)
    np.testing.assert_allclose(np.asarray(A.sum(axis=1)).ravel(), 0.0, atol=1e-14)


def test_oracle_reproduces_golden_fixture():
    """tests/golden/block_model_oracle.npz (made by tests/golden/make_golden.py) still holds."""
    import os

    from simpeg_gb300.workloads import block_model_survey

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "block_model_oracle.npz"))
    mesh, sigma, survey, blocks = block_model_survey(seed=0)
    np.testing.assert_array_equal(np.log(sigma), g["m"])
    np.testing.assert_array_equal(np.array(blocks), g["blocks"])
    o = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    o.set_model(g["m"])
    f = o.fields()
    np.testing.assert_allclose(o.dpred(f=f), g["dpred"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(o.Jvec(g["m"], g["v"], f=f), g["jvec"], rtol=1e-9, atol=1e-12 * np.abs(g["jvec"]).max())
    np.testing.assert_allclose(o.Jtvec(g["m"], g["w"], f=f), g["jtvec"], rtol=1e-9,
                               atol=1e-12 * np.abs(g["jtvec"]).max())


def _ip_forward_setup():
    """tests/em/static/test_IP_fwd.py:12-46: dipole source, dipole receivers over a
    conductive-chargeable sphere (eta = 0.1) in a 0.01 S/m half-space."""
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
    return mesh, Survey([src]), sigma_inf, eta


def test_ip_oracle_is_the_linearised_dc_response():
    """tests/em/static/test_IP_fwd.py:48-74: IP data vs DC(sigma0) - DC(sigma_inf),
    sigma0 = sigma_inf (1 - eta); mean squared relative error < 0.05."""
    from oracle.ip3d import OracleIP3DNodal

    mesh, survey, sigma_inf, eta = _ip_forward_setup()
    d0 = OracleDC3DNodal(mesh, survey, sigma=sigma_inf * (1.0 - eta)).dpred()
    dinf = OracleDC3DNodal(mesh, survey, sigma=sigma_inf).dpred()
    ip = OracleIP3DNodal(mesh, survey, sigma_inf, eta_map=maps.IdentityMap(mesh))
    d = ip.dpred(eta)
    full = d0 - dinf
    err = np.linalg.norm((d - full) / full) ** 2 / full.size
    assert err < 0.05, err


def test_ip_oracle_adjoint_and_chargeability_scale():
    """tests/em/static/test_IP_jvecjtvecadj.py:146-156 (adjoint, |w.Jv - v.Jtw| < 1e-8),
    and apparent-chargeability data = IP voltage / DC voltage (simulation.py:44-61)."""
    from oracle.ip3d import OracleIP3DNodal

    mesh, survey, _ = _small_problem(seed=3)
    sigma = np.exp(_small_problem(seed=3)[2])
    ip = OracleIP3DNodal(mesh, survey, sigma, eta_map=maps.IdentityMap(mesh))
    rng = np.random.default_rng(30)
    m0 = np.full(mesh.n_cells, 0.1)
    v = rng.uniform(size=mesh.n_cells)
    w = rng.uniform(size=survey.nD)
    assert abs(w @ ip.Jvec(m0, v) - v @ ip.Jtvec(m0, w)) < 1e-8
    d_volt = ip.dpred(m0)
    dc = OracleDC3DNodal(mesh, survey, sigma=sigma).dpred()
    for src in survey.source_list:
        for rx in src.receiver_list:
            rx.data_type = "apparent_chargeability"
    ip2 = OracleIP3DNodal(mesh, survey, sigma, eta_map=maps.IdentityMap(mesh))
    np.testing.assert_allclose(ip2.dpred(m0), d_volt / dc, rtol=1e-12)
    # linear in eta: the prediction is J eta exactly
    np.testing.assert_allclose(ip2.dpred(2.0 * m0), 2.0 * ip2.dpred(m0), rtol=1e-12)


def test_derived_fields_of_a_uniform_gradient():
    """Fields3DNodal e, j, charge, charge_density (resistivity/fields.py:214-253) for
    phi = -x on a non-uniform mesh: e = 1 on x-edges and 0 on the others, j = the
    edge-averaged conductivity on x-edges, no charge at interior nodes (the field is
    divergence-free there); charge only on the x = min / max faces, equal and opposite."""
    mesh = TensorMesh([[(10.0, 2, -1.3), (10.0, 4), (10.0, 2, 1.3)], [(10.0, 5)], [(8.0, 4)]], origin="CCN")
    sigma = np.random.default_rng(0).uniform(0.01, 0.1, mesh.n_cells)
    src = sources.Pole([], np.r_[0.0, 0.0, 0.0])
    o = OracleDC3DNodal(mesh, Survey([src]), sigma=sigma)
    phi = -o.ops.nodes[:, 0]
    e, j, q, rho = o.derived_fields(phi, 8.854187817e-12)
    nx, ny, nz = mesh.shape_cells
    nEx = nx * (ny + 1) * (nz + 1)
    np.testing.assert_allclose(e[:nEx], 1.0, rtol=1e-12)
    np.testing.assert_allclose(e[nEx:], 0.0, atol=1e-12)
    E = o.E
    np.testing.assert_allclose(j[:nEx], (E @ sigma)[:nEx] / (E @ np.ones(mesh.n_cells))[:nEx], rtol=1e-12)
    q3 = q.reshape((nz + 1, ny + 1, nx + 1))
    scale = np.abs(q).max()
    assert scale > 0
    np.testing.assert_allclose(q3[:, :, 1:-1], 0.0, atol=1e-12 * scale)
    np.testing.assert_allclose(q3[:, :, 0].sum(), -q3[:, :, -1].sum(), rtol=1e-12)
    rho3 = rho.reshape((nz, ny, nx))
    assert np.all(np.abs(rho3[:, :, 1:-1]) <= 1e-12 * np.abs(rho).max())


def _multipole_fullspace():
    """tests/em/static/test_DC_FieldsMultipoleFullspace.py:185-282: a three-electrode source
    (+1, +1, -2 A) in a 0.01 S/m whole space on a padded mesh; the analytic electric field is
    the sum of the point-source fields I (x - x_k) / (4 pi sigma |x - x_k|^3) (the reference
    writes it as two finite electric dipoles, the same field), compared on the edges outside
    a 4 m box around the source."""
    cs = 0.5
    h = [(cs, 11, -1.5), (cs, 15), (cs, 11, 1.5)]
    mesh = TensorMesh([h, h, h], origin="CCC")
    sigma = np.full(mesh.n_cells, 1e-2)
    locs = np.array([[2.25, 0.0, 0.0], [1.25, 0.0, 0.0], [-0.25, 0.0, 0.0]])
    currents = np.array([1.0, 1.0, -2.0])
    src = sources.Multipole([], location=locs, current=currents)
    grids = [TensorMesh._ndgrid(mesh.cell_centers_x, mesh.nodes_y, mesh.nodes_z),
             TensorMesh._ndgrid(mesh.nodes_x, mesh.cell_centers_y, mesh.nodes_z),
             TensorMesh._ndgrid(mesh.nodes_x, mesh.nodes_y, mesh.cell_centers_z)]
    e_ana = []
    for axis, g in enumerate(grids):
        r = g[:, None, :] - locs[None, :, :]
        dist = np.linalg.norm(r, axis=-1)
        e_ana.append((currents[None, :] * r[..., axis] / (4 * np.pi * 1e-2 * dist ** 3)).sum(axis=1))
    e_ana = np.concatenate(e_ana)
    pts = np.vstack(grids)
    inside = lambda a: np.all((pts >= -a) & (pts <= a), axis=1)
    roi = inside(75.0) & ~inside(4.0)
    return mesh, sigma, Survey([src]), e_ana, roi


@pytest.mark.slow
def test_multipole_fullspace_derived_fields():
    """The derived fields e and j = sigma e of the oracle within 10 % of the analytic
    whole-space field (the reference's tolerance), charge and density finite."""
    from scipy.constants import epsilon_0

    mesh, sigma, survey, e_ana, roi = _multipole_fullspace()
    o = OracleDC3DNodal(mesh, survey, sigma=sigma)
    phi = o.fields()[:, 0]
    e, j, q, rho = o.derived_fields(phi, epsilon_0)
    err_e = np.linalg.norm(e[roi] - e_ana[roi]) / np.linalg.norm(e_ana[roi])
    err_j = np.linalg.norm(j[roi] - 1e-2 * e_ana[roi]) / np.linalg.norm(1e-2 * e_ana[roi])
    assert err_e < 0.1 and err_j < 0.1, (err_e, err_j)
    assert np.all(np.isfinite(q)) and np.all(np.isfinite(rho))
