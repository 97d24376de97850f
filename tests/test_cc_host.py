"""Cell-centred formulation on the CPU: the oracle against the reference's analytic recipes
(``tests/em/static/test_DC_analytic.py:83-240``, rms relative error < 5 %), and the host
tables of the GPU simulation (electrodes, boundary weights) against the oracle, bit-exact for
the integer work."""

import numpy as np
import pytest

from oracle import analytic
from oracle.cc3d import OracleDC3DCellCentered
from oracle.operators import MeshOps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.boundary import cc_boundary_weights, cell_centre_grid
from simpeg_gb300.resistivity.electrodes import SurveyTables, cc_interp_weights, closest_cells
from simpeg_gb300.resistivity.survey import Survey


def _ndgrid(x, y, z):
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    return np.c_[X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")]


def _analytic_case(fac, hz_extra, origin, lim, pole, earth):
    cs = 25.0
    hx = [(cs, 7, -fac), (cs, 21), (cs, 7, fac)]
    mesh = TensorMesh([hx, hx, [(cs, 7, -fac), (cs, 20)] + hz_extra], origin=origin)
    x = mesh.cell_centers_x[(mesh.cell_centers_x > -lim) & (mesh.cell_centers_x < lim)]
    y = mesh.cell_centers_y[(mesh.cell_centers_y > -lim) & (mesh.cell_centers_y < lim)]
    A, B = np.r_[-200.0, 0, 0], np.r_[200.0, 0, 0]
    if pole:
        M = _ndgrid(x, y, np.r_[0.0])
        ana = analytic.pole_pole(A, M, 1e-2, earth_type=earth)
        sv = Survey([sources.Pole([receivers.Pole(M)], A)])
    else:
        M, N = _ndgrid(x - 25.0, y, np.r_[0.0]), _ndgrid(x + 25.0, y, np.r_[0.0])
        ana = analytic.dipole_dipole(A, B, M, N, 1e-2, earth_type=earth)
        sv = Survey([sources.Dipole([receivers.Dipole(M, N)], A, B)])
    return mesh, sv, ana


ANALYTIC = {
    # bc: (padding factor, extra z padding, origin, receiver half-extent, pole-pole, earth)
    "Mixed": (1.3, [], "CCN", 100.0, False, "halfspace"),
    "Neumann": (1.3, [], "CCN", 100.0, False, "halfspace"),
    "Dirichlet": (1.3, [(25.0, 7, 1.3)], "CCC", 155.0, False, "wholespace"),
    "Mixed_pole": (1.5, [], "CCN", 155.0, True, "halfspace"),
}


@pytest.mark.parametrize("case", sorted(ANALYTIC))
def test_cc_oracle_analytic(case):
    mesh, sv, ana = _analytic_case(*ANALYTIC[case])
    bc = case.split("_")[0]
    o = OracleDC3DCellCentered(mesh, sv, sigma=np.full(mesh.n_cells, 1e-2), bc_type=bc)
    d = o.dpred()
    err = np.sqrt((((d - ana) / ana) ** 2).sum() / sv.nD)
    assert err < 0.05, err


def _mesh():
    return TensorMesh([[(10.0, 2, -1.3), (10.0, 5)], [(10.0, 4)], [(10.0, 2, -1.3), (10.0, 3)]], origin="CCN")


def test_cc_electrode_tables_match_oracle():
    mesh = _mesh()
    ops = MeshOps(mesh.h, mesh.origin)
    rng = np.random.default_rng(1)
    lo = np.array([mesh.nodes_x[0], mesh.nodes_y[0], mesh.nodes_z[0]])
    hi = np.array([mesh.nodes_x[-1], mesh.nodes_y[-1], mesh.nodes_z[-1]])
    pts = np.vstack([lo + rng.uniform(size=(20, 3)) * (hi - lo), mesh.cell_centers[[0, 7, 30]],
                     np.c_[mesh.cell_centers_x[:3], np.zeros(3), np.zeros(3)], hi[None, :], lo[None, :]])
    np.testing.assert_array_equal(closest_cells(mesh, pts), ops.closest_cell(pts))
    idx, w = cc_interp_weights(mesh, pts)
    import scipy.sparse as sp

    P = sp.csr_matrix((w.ravel(), (np.repeat(np.arange(len(pts)), 8), idx.ravel())), shape=(len(pts), mesh.n_cells))
    P.sum_duplicates()
    Q = ops.interpolation_matrix_cc(pts)
    Q.sum_duplicates()
    assert (P != Q).nnz == 0
    with pytest.raises(ValueError):
        cc_interp_weights(mesh, np.array([[1e4, 0.0, 0.0]]))
    # source term: q[closest cell] = current; a dipole with both electrodes in one cell keeps the last
    src = [sources.Dipole([], np.r_[-3.0, 1.0, -2.0], np.r_[12.0, -3.0, -4.0]),
           sources.Dipole([], np.r_[1.0, 1.0, -1.0], np.r_[2.0, 2.0, -2.0]),
           sources.Pole([], np.r_[0.0, 0.0, 0.0])]
    t = SurveyTables(mesh, src, mesh.n_cells, grid="CC")
    q = np.zeros(mesh.n_cells * 3)
    q[t.q_idx] = t.q_val
    o = OracleDC3DCellCentered(mesh, Survey(src), sigma=np.ones(mesh.n_cells))
    np.testing.assert_array_equal(q.reshape(3, -1).T, o.getRHS())


@pytest.mark.parametrize("bc", ["Robin", "Dirichlet"])
def test_cc_boundary_weights_match_oracle(bc):
    """bw_f / rho_c (the packed boundary weights) equals the boundary part of the oracle's
    Div MfRhoI Grad: A minus the interior-face operator, which is diagonal."""
    import scipy.sparse as sp

    mesh = _mesh()
    rng = np.random.default_rng(4)
    rho = 10 ** rng.uniform(1, 2, mesh.n_cells)
    o = OracleDC3DCellCentered(mesh, Survey([]), rho=rho, bc_type=bc)
    A = o.getA()
    keep = np.ones(o.D.shape[1])
    keep[MeshOps(mesh.h, mesh.origin).boundary_face_index()] = 0.0
    Dint = o.D @ sp.diags(keep)
    A0 = (Dint @ o.MfRhoI() @ Dint.T).tocsr()
    extra = np.asarray((A - A0).diagonal())
    assert abs((A - A0) - sp.diags(extra)).max() < 1e-13 * abs(A).max()
    bw = cc_boundary_weights(mesh, bc)
    nx, ny, nz = mesh.shape_cells
    got = np.zeros(mesh.n_cells)
    off = 0
    for side, n in enumerate([ny * nz, ny * nz, nx * nz, nx * nz, nx * ny, nx * ny]):
        w = bw[off:off + n]
        off += n
        a, b = np.meshgrid(*(np.arange(v) for v in ([ny, nz] if side < 2 else [nx, nz] if side < 4 else [nx, ny])),
                           indexing="ij")
        a, b = a.ravel(order="F"), b.ravel(order="F")
        end = [0, nx - 1, 0, ny - 1, 0, nz - 1][side]
        if side < 2:
            c = end + nx * (a + ny * b)
        elif side < 4:
            c = a + nx * (end + ny * b)
        else:
            c = a + nx * (b + ny * end)
        np.add.at(got, c, w / rho[c])
    np.testing.assert_allclose(got, extra, rtol=1e-12, atol=1e-13 * np.abs(A.diagonal()).max())


def test_cell_centre_grid():
    mesh = _mesh()
    g = cell_centre_grid(mesh)
    np.testing.assert_allclose(g.nodes_x, mesh.cell_centers_x)
    np.testing.assert_allclose(g.nodes_z, mesh.cell_centers_z)
    assert g.n_nodes == mesh.n_cells
