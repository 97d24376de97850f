"""Host-side logic of the product (no GPU): geometry, electrode tables,
boundary weights, miniaturisation and the C-ABI library surface."""

import ctypes
import re
from pathlib import Path

import numpy as np
import scipy.sparse as sp
import pytest

from oracle.dc3d import OracleDC3DNodal
from oracle.operators import MeshOps
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh, unpack_widths
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.boundary import robin_face_weights
from simpeg_gb300.resistivity.electrodes import SurveyTables, interpolation_matrix
from simpeg_gb300.resistivity.survey import Survey, geometric_factor
from simpeg_gb300.resistivity.utils import mini_pole_pole
from simpeg_gb300.workloads import block_model_survey

ROOT = Path(__file__).resolve().parents[1]


def test_unpack_widths_padding():
    w = unpack_widths([(25.0, 3, -1.3), (25.0, 2), (25.0, 2, 1.3)])
    np.testing.assert_allclose(w, [25 * 1.3**3, 25 * 1.3**2, 25 * 1.3, 25, 25, 25 * 1.3, 25 * 1.3**2])
    m = TensorMesh([[(10.0, 4)], [(10.0, 2)], [(5.0, 2)]], origin="CCN")
    np.testing.assert_allclose(m.origin, [-20.0, -10.0, -10.0])
    assert m.n_nodes == 5 * 3 * 3
    np.testing.assert_allclose(m.nodes[1], [-10.0, -10.0, -10.0])


def _mesh():
    return TensorMesh([[(5.0, 2, -1.3), (5.0, 6), (5.0, 2, 1.3)], [(5.0, 7)], [(5.0, 2, -1.3), (5.0, 4)]], origin="CCN")


@pytest.mark.parametrize("pts", [
    np.array([[0.0, 0.0, 0.0]]),                      # on a node
    np.array([[1.3, -2.2, -3.7], [2.5, 2.5, -2.5]]),  # inside cells, on a midpoint
    None,                                              # last node on each axis
])
def test_interpolation_bit_exact_vs_oracle(pts):
    mesh = _mesh()
    if pts is None:
        pts = np.array([[mesh.nodes_x[-1], mesh.nodes_y[-1], mesh.nodes_z[-1]],
                        [mesh.nodes_x[0], mesh.nodes_y[0], mesh.nodes_z[0]]])
    P = interpolation_matrix(mesh, pts)
    Q = MeshOps(mesh.h, mesh.origin).interpolation_matrix(pts)
    P.sum_duplicates()
    Q.sum_duplicates()
    assert (P != Q).nnz == 0  # identical indices and identical weights


def test_points_outside_mesh_raise():
    mesh = _mesh()
    with pytest.raises(ValueError):
        interpolation_matrix(mesh, np.array([[1e4, 0.0, 0.0]]))


def test_robin_weights_match_oracle_AvgBC():
    mesh = _mesh()
    rng = np.random.default_rng(0)
    sigma = 10 ** rng.uniform(-3, -1, mesh.n_cells)
    o = OracleDC3DNodal(mesh, Survey([sources.Pole([], np.r_[0.0, 0.0, 0.0])]), sigma=sigma)
    ref = o.AvgBC @ sigma
    bw = robin_face_weights(mesh)
    # rebuild the Robin diagonal from the packed per-side weights
    nx, ny, nz = mesh.shape_cells
    Nx, Ny = nx + 1, ny + 1
    s3 = sigma.reshape(nx, ny, nz, order="F")
    out = np.zeros(mesh.n_nodes)
    off = 0

    def add(face_w, cell_sig, nodes4):
        for n in nodes4:
            np.add.at(out, n, face_w * cell_sig)

    sides = []
    for side, i in ((0, 0), (1, nx)):
        J, K = np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")
        J, K = J.ravel(order="F"), K.ravel(order="F")
        w = bw[off:off + J.size]; off += J.size
        cs = s3[0 if side == 0 else nx - 1, J, K]
        nodes4 = [i + Nx * (J + Ny * K), i + Nx * (J + 1 + Ny * K), i + Nx * (J + Ny * (K + 1)), i + Nx * (J + 1 + Ny * (K + 1))]
        sides.append((w, cs, nodes4))
    for side, j in ((0, 0), (1, ny)):
        I, K = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
        I, K = I.ravel(order="F"), K.ravel(order="F")
        w = bw[off:off + I.size]; off += I.size
        cs = s3[I, 0 if side == 0 else ny - 1, K]
        nodes4 = [I + Nx * (j + Ny * K), I + 1 + Nx * (j + Ny * K), I + Nx * (j + Ny * (K + 1)), I + 1 + Nx * (j + Ny * (K + 1))]
        sides.append((w, cs, nodes4))
    for side, k in ((0, 0), (1, nz)):
        I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        I, J = I.ravel(order="F"), J.ravel(order="F")
        w = bw[off:off + I.size]; off += I.size
        cs = s3[I, J, 0 if side == 0 else nz - 1]
        nodes4 = [I + Nx * (J + Ny * k), I + 1 + Nx * (J + Ny * k), I + Nx * (J + 1 + Ny * k), I + 1 + Nx * (J + 1 + Ny * k)]
        sides.append((w, cs, nodes4))
    assert off == bw.size
    for w, cs, nodes4 in sides:
        add(w, cs, nodes4)
    np.testing.assert_allclose(out, ref, rtol=1e-13, atol=1e-16)
    # top faces carry no Robin weight
    assert np.all(bw[-nx * ny:] == 0.0)


def test_survey_tables_match_oracle_projection():
    mesh, sigma, survey, _ = block_model_survey(seed=0)
    t = SurveyTables(mesh, survey.source_list, mesh.n_nodes)
    o = OracleDC3DNodal(mesh, survey, sigma=sigma)
    # source term
    q = np.zeros(mesh.n_nodes * survey.nSrc)
    q[t.q_idx] = t.q_val
    np.testing.assert_array_equal(q.reshape(survey.nSrc, -1).T, o.getRHS())
    # receiver projection: each datum row restricted to its source block
    row = 0
    for s, P, fac in o._projections():
        blk = t.P[row:row + P.shape[0], s * mesh.n_nodes:(s + 1) * mesh.n_nodes]
        assert (blk != P).nnz == 0
        row += P.shape[0]
    assert t.nD == survey.nD == 300
    # the transpose table is the exact transpose
    PT = np.zeros((t.P.shape[1], t.nD))
    for r, o_idx in enumerate(t.PT_out):
        for e in range(t.PT_ptr[r], t.PT_ptr[r + 1]):
            PT[o_idx, t.PT_idx[e]] += t.PT_w[e]
    np.testing.assert_array_equal(PT, t.P.T.toarray())


def test_survey_slices_and_geometric_factor():
    a, b = np.r_[-10.0, 0, 0], np.r_[10.0, 0, 0]
    M = np.array([[30.0, 0, 0], [40.0, 0, 0]])
    N = np.array([[40.0, 0, 0], [50.0, 0, 0]])
    rx = receivers.Dipole(M, N, data_type="apparent_resistivity")
    rx2 = receivers.Pole(M)
    s1 = sources.Dipole([rx], a, b)
    s2 = sources.Pole([rx2], a)
    sv = Survey([s1, s2])
    sl = sv.get_all_slices()
    assert sl[s1, rx] == slice(0, 2) and sl[s2, rx2] == slice(2, 4) and sv.nD == 4
    g = geometric_factor(sv)
    am, bm, an, bn = 40.0, 20.0, 50.0, 30.0
    assert np.isclose(g[0], (1 / am - 1 / bm - 1 / an + 1 / bn) / (2 * np.pi))
    assert np.isclose(g[2], (1 / 40.0) / (2 * np.pi))
    sv.set_geometric_factor()
    np.testing.assert_allclose(rx.geometric_factor[s1], g[:2])


def test_mini_pole_pole_reassembles_dipole_data():
    mesh, sigma, survey, _ = block_model_survey(seed=0)
    dipoles, invs, mini = mini_pole_pole(survey)
    o = OracleDC3DNodal(mesh, survey, sigma=sigma)
    d_full = o.dpred()
    om = OracleDC3DNodal(mesh, mini, sigma=sigma)
    dm = om.dpred()
    out = dm[invs[0]]
    out[dipoles[0]] -= dm[invs[1]]
    out[dipoles[1]] -= dm[invs[2]]
    out[dipoles[0] & dipoles[1]] += dm[invs[3]]
    np.testing.assert_allclose(out, d_full, rtol=1e-9, atol=1e-12 * np.abs(d_full).max())
    assert mini.nSrc < 4 * survey.nD


def test_maps_derivatives():
    m = np.array([0.1, -0.3, 2.0])
    e = maps.ExpMap(nP=3)
    np.testing.assert_allclose(e * m, np.exp(m))
    np.testing.assert_allclose(e.deriv(m).diagonal(), np.exp(m))
    c = maps.ComboMap([maps.ReciprocalMap(), maps.ExpMap(nP=3)])
    np.testing.assert_allclose(c * m, np.exp(-m))
    np.testing.assert_allclose(c.diag_deriv(m), -np.exp(-m))


def test_library_exports_every_declared_symbol():
    """The C ABI in include/dcgpu.h is exported by libdcgpu.so (no compute call)."""
    from simpeg_gb300 import _lib

    header = (ROOT / "include" / "dcgpu.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|void|long long|const char \*)\s*(dc_\w+)\s*\(", header, re.M))
    assert declared, "no declarations parsed"
    L = _lib.lib()
    for name in sorted(declared):
        assert hasattr(L, name), name
        assert ctypes.cast(getattr(L, name), ctypes.c_void_p).value
    assert declared == set(_lib.declared_symbols())


def test_receiver_transpose_tables_equal_csr_transpose():
    """PT (the adjoint scatter) built from sorted entries equals the CSR
    transpose restricted to its nonzero rows."""
    from simpeg_gb300.resistivity.electrodes import SurveyTables
    from simpeg_gb300.workloads import block_model_survey

    mesh, sigma, survey, _ = block_model_survey(seed=3)
    t = SurveyTables(mesh, survey.source_list, mesh.n_nodes)
    PT = t.P.T.tocsr()
    PT.sum_duplicates()
    nz = np.flatnonzero(np.diff(PT.indptr))
    sub = PT[nz]
    np.testing.assert_array_equal(t.PT_out, nz)
    np.testing.assert_array_equal(t.PT_ptr, sub.indptr)
    np.testing.assert_array_equal(t.PT_idx, sub.indices)
    np.testing.assert_array_equal(t.PT_w, sub.data)


def test_device_map_transforms_match_host():
    """The elementwise device transforms of the maps equal their host transforms."""
    import torch

    from simpeg_gb300 import maps

    rng = np.random.default_rng(0)
    m = rng.uniform(0.1, 3.0, 50)
    for mp in (maps.IdentityMap(nP=50), maps.ExpMap(nP=50), maps.ReciprocalMap(nP=50),
               maps.ExpMap(nP=50) * maps.ReciprocalMap(nP=50)):
        np.testing.assert_allclose(mp.transform_dev(torch.from_numpy(m)).numpy(), mp * m, rtol=1e-15)


def test_double_float_bit_routines(tmp_path):
    """The bit-level double-float split, widening and sum (csrc/dc_dfbits.h), compiled for
    the host: truncation split exact to 2^-48, widening equal to the fp32 -> fp64
    conversion, the pair sum equal to the fp64 addition bit for bit, out-of-range
    values rejected (they take the fp64 instructions)."""
    import shutil
    import subprocess

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "dfbits_check"
    subprocess.run([cxx, "-O2", "-std=c++17", str(ROOT / "tests" / "dfbits_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_survey_source_locations_and_multipole():
    """Survey.source_locations (survey.py:150-166): A and B rows per source in order, NaN B
    for poles; Multipole sources keep all electrodes as A (sources.py:107-132)."""
    from simpeg_gb300.resistivity import receivers, sources
    from simpeg_gb300.resistivity.survey import Survey

    rx = receivers.Pole(np.zeros((1, 3)))
    sv = Survey([sources.Pole([rx], np.r_[1.0, 0, 0]), sources.Dipole([rx], np.r_[0.0, 0, 0], np.r_[2.0, 0, 0])])
    a, b = sv.source_locations
    np.testing.assert_array_equal(a, [[1.0, 0, 0], [0.0, 0, 0]])
    assert np.isnan(b[0]).all()
    np.testing.assert_array_equal(b[1], [2.0, 0, 0])
    with pytest.raises(AttributeError):
        sv.survey_type
    mp = sources.Multipole([rx], location=[[0.0, 0, 0], [1.0, 0, 0], [2.0, 0, 0]], current=[1.0, 1.0, -2.0])
    assert mp.location_a.shape == (3, 3) and np.isnan(mp.location_b).all()
    np.testing.assert_array_equal(mp.electrode_currents(), [1.0, 1.0, -2.0])
    with pytest.raises(ValueError):
        sources.Multipole([rx], location=[[0.0, 0, 0], [1.0, 0, 0]], current=[1.0, 1.0, -2.0])


def _mixed_survey(mesh):
    """Pole, dipole and multipole sources; pole and dipole receivers, volt and apparent
    resistivity; some electrodes exactly on nodes (interpolation weights of 0 and 1)."""
    from simpeg_gb300.resistivity import receivers, sources
    from simpeg_gb300.resistivity.survey import Survey

    xs = np.arange(-40.0, 41.0, 10.0)
    srcs = []
    M = np.c_[xs[4:7], np.zeros(3), np.zeros(3)]
    N = np.c_[xs[5:8], np.zeros(3), np.zeros(3)]
    srcs.append(sources.Dipole([receivers.Dipole(M, N), receivers.Pole(M, data_type="apparent_resistivity")],
                               np.r_[-40.0, 0, 0], np.r_[-30.0, 0, 0]))
    srcs.append(sources.Pole([receivers.Dipole(M + np.r_[3.3, 0, 0], N + np.r_[3.3, 0, 0], data_type="apparent_resistivity")],
                             np.r_[-25.0, 2.5, 0.0]))
    srcs.append(sources.Multipole([receivers.Pole(np.c_[xs[:3], np.full(3, 7.5), np.zeros(3)])],
                                  location=[[-10.0, 0, 0], [0.0, 5.0, 0], [10.0, -5.0, 0]], current=[1.0, 1.0, -2.0]))
    sv = Survey(srcs)
    sv.set_geometric_factor()
    return sv


def test_survey_tables_mixed_survey_match_oracle():
    """The survey tables (one interpolation per electrode kind) reproduce the oracle's
    source term and per-receiver projections, apparent-resistivity scaling included."""
    from simpeg_gb300.mesh import TensorMesh

    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 10), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 6), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 5)]], origin="CCN")
    survey = _mixed_survey(mesh)
    t = SurveyTables(mesh, survey.source_list, mesh.n_nodes)
    o = OracleDC3DNodal(mesh, survey, sigma=np.full(mesh.n_cells, 0.01))
    q = np.zeros(mesh.n_nodes * survey.nSrc)
    q[t.q_idx] = t.q_val
    np.testing.assert_allclose(q.reshape(survey.nSrc, -1).T, o.getRHS(), rtol=1e-15, atol=1e-15)
    row = 0
    for s, P, fac in o._projections():
        blk = t.P[row:row + P.shape[0], s * mesh.n_nodes:(s + 1) * mesh.n_nodes].toarray()
        ref = P.toarray() * (fac[:, None] if fac is not None else 1.0)
        np.testing.assert_allclose(blk, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())
        np.testing.assert_array_equal(t.owner[row:row + P.shape[0]], s)
        row += P.shape[0]
    assert row == t.nD == survey.nD


def test_electrode_tables_mixed_survey():
    """Per-datum electrode indices and weights of the reciprocity JtJ diagonal, checked
    against a per-datum restatement: electrode k of datum d is uniq[idx]; currents of the
    source's A (B) electrode; receiver weights +-1/geometric factor for apparent resistivity."""
    from simpeg_gb300.mesh import TensorMesh
    from simpeg_gb300.resistivity.simulation import Simulation3DNodal

    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 10), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 6), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 5)]], origin="CCN")
    survey = _mixed_survey(mesh)
    survey_2 = type(survey)([s for s in survey.source_list if np.atleast_2d(s.location).shape[0] <= 2])

    class Host:
        pass

    h = Host()
    h.survey = survey
    assert Simulation3DNodal._electrode_tables(h) is None  # a three-electrode source: no reciprocity tables
    h.survey = survey_2
    uniq, t = Simulation3DNodal._electrode_tables(h)
    d = 0
    for src in survey_2.source_list:
        L = np.atleast_2d(src.location)
        cur = src.electrode_currents()
        for rx in src.receiver_list:
            fac = np.ones(rx.nD)
            if rx.data_type == "apparent_resistivity":
                fac = 1.0 / np.asarray(rx.geometric_factor[src])
            dip = isinstance(rx.locations, (list, tuple))
            Ms = np.atleast_2d(rx.locations[0] if dip else rx.locations)
            for i in range(rx.nD):
                np.testing.assert_array_equal(uniq[t["sa"][d]], L[0])
                assert t["ia"][d] == cur[0]
                if L.shape[0] == 2:
                    np.testing.assert_array_equal(uniq[t["sb"][d]], L[1])
                    assert t["ib"][d] == cur[1]
                else:
                    assert t["sb"][d] == -1 and t["ib"][d] == 0.0
                np.testing.assert_array_equal(uniq[t["rm"][d]], Ms[i])
                assert t["wm"][d] == fac[i]
                if dip:
                    np.testing.assert_array_equal(uniq[t["rn"][d]], np.atleast_2d(rx.locations[1])[i])
                    assert t["wn"][d] == -fac[i]
                else:
                    assert t["rn"][d] == -1 and t["wn"][d] == 0.0
                d += 1
    assert d == t["sa"].size
    assert len(np.unique(uniq, axis=0)) == len(uniq)


def test_wenner_source_list():
    """WennerSrcList (resistivity/utils.py:13-74): the 7-electrode, a = 10 array has the
    spacing-1 quadruples (j, j+1, j+2, j+3), j = 0..3, then the spacing-2 one (0, 2, 4, 6)."""
    from simpeg_gb300.resistivity.utils import WennerSrcList

    srcs = WennerSrcList(7, 10.0)
    x = 10.0 * np.arange(7) - 30.0
    quads = [(0, 1, 2, 3), (1, 2, 3, 4), (2, 3, 4, 5), (3, 4, 5, 6), (0, 2, 4, 6)]
    assert len(srcs) == len(quads)
    for src, (a, m, n, b) in zip(srcs, quads):
        np.testing.assert_array_equal(src.location, [[x[a], 0, 0], [x[b], 0, 0]])
        (rx,) = src.receiver_list
        np.testing.assert_array_equal(rx.locations[0], [[x[m], 0, 0]])
        np.testing.assert_array_equal(rx.locations[1], [[x[n], 0, 0]])
    assert len(WennerSrcList(5, 2.5)) == 2


def test_receiver_getP_eval_evalDeriv():
    """Receiver projections on the host (receivers.py:156-244,379-498): getP equals the
    oracle's interp(M) - interp(N); eval = P phi (/ geometric factor for apparent
    resistivity); evalDeriv is P (scaled) and its transpose, consistent with eval."""
    from oracle.dc3d import _rx_projection
    from oracle.operators import MeshOps
    from simpeg_gb300.mesh import TensorMesh

    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 10), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 6), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 5)]], origin="CCN")
    survey = _mixed_survey(mesh)
    ops = MeshOps(mesh.h, mesh.origin)
    rng = np.random.default_rng(4)
    phi = {id(s): rng.standard_normal(mesh.n_nodes) for s in survey.source_list}

    class F:
        def __getitem__(self, key):
            return phi[id(key[0])]

    for src in survey.source_list:
        for rx in src.receiver_list:
            P = rx.getP(mesh)
            assert (P != _rx_projection(ops, rx)).nnz == 0
            fac = 1.0 / rx.geometric_factor[src] if rx.data_type == "apparent_resistivity" else 1.0
            np.testing.assert_allclose(rx.eval(src, mesh, F()), fac * (P @ phi[id(src)]), rtol=1e-14)
            v = rng.standard_normal(mesh.n_nodes)
            w = rng.standard_normal(rx.nD)
            np.testing.assert_allclose(rx.evalDeriv(src, mesh, F(), v=v), fac * (P @ v), rtol=1e-14)
            np.testing.assert_allclose(w @ rx.evalDeriv(src, mesh, F(), v=v),
                                       v @ rx.evalDeriv(src, mesh, F(), v=w, adjoint=True), rtol=1e-12)
            np.testing.assert_allclose(rx.evalDeriv(src, mesh, F()) @ v, fac * (P @ v), rtol=1e-14)
            assert rx.getP(mesh, transpose=True).shape == (mesh.n_nodes, rx.nD)
    with pytest.raises(NotImplementedError):
        survey.source_list[0].receiver_list[0].getP(mesh, "CC")


def test_source_eval_matches_oracle_rhs():
    """BaseSrc.eval (sources.py:64-88, nodal formulation) equals the oracle's source term
    column for pole, dipole and multipole sources; evalDeriv is zero."""
    from simpeg_gb300.mesh import TensorMesh

    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 10), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 6), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 5)]], origin="CCN")
    survey = _mixed_survey(mesh)
    rhs = OracleDC3DNodal(mesh, survey, sigma=np.full(mesh.n_cells, 0.01)).getRHS()

    class Sim:
        pass

    sim = Sim()
    sim.mesh = mesh
    sim._formulation = "EB"
    for i, src in enumerate(survey.source_list):
        np.testing.assert_allclose(src.eval(sim), rhs[:, i], rtol=1e-15, atol=1e-15)
        assert src.evalDeriv(sim) == 0.0
    sim._formulation = "HJ"
    with pytest.raises(NotImplementedError):
        survey.source_list[0].eval(sim)


def test_l2_data_misfit_forms_and_host_products():
    """L2DataMisfit (data_misfit.py:238-343) built the reference's way, (data, simulation)
    with W = 1 / standard deviation, or from dobs and W; phi_d, deriv and deriv2 against
    dense algebra with a linear stand-in simulation on host tensors."""
    import torch

    from simpeg_gb300.data import Data
    from simpeg_gb300.inversion import L2DataMisfit

    rng = np.random.default_rng(8)
    nD, nP = 12, 7
    J = rng.standard_normal((nD, nP))
    c = rng.standard_normal(nD)

    class Fields:
        pass

    class LinearSim:
        device = torch.device("cpu")

        def _fields_for(self, m, f):
            out = Fields()
            out.phi_dev = torch.as_tensor(J @ np.asarray(m) + c)
            return out

        def _gather(self, phi):
            return phi

        def jvec_dev(self, v, f=None):
            return torch.as_tensor(J) @ v

        def jtvec_dev(self, w, f=None):
            return torch.as_tensor(J.T) @ w

    class Srv:
        nD = 12

    sim = LinearSim()
    dobs = rng.standard_normal(nD)
    data = Data(Srv(), dobs=dobs, relative_error=0.05, noise_floor=1e-3)
    std = np.sqrt((0.05 * np.abs(dobs)) ** 2 + 1e-6)
    m = rng.standard_normal(nP)
    v = rng.standard_normal(nP)
    for dm in (L2DataMisfit(data, sim), L2DataMisfit(data=data, simulation=sim), L2DataMisfit(sim, dobs, W=1 / std)):
        w = 1 / std
        r = J @ m + c - dobs
        np.testing.assert_allclose(dm(m), np.sum((w * r) ** 2), rtol=1e-12)
        np.testing.assert_allclose(dm.deriv(m), 2 * J.T @ (w * w * r), rtol=1e-12)
        np.testing.assert_allclose(dm.deriv2(m, v), 2 * J.T @ (w * w * (J @ v)), rtol=1e-12)
        assert dm.nD == nD
    with pytest.raises(ValueError):
        L2DataMisfit(Data(Srv(), dobs=dobs), sim)  # no uncertainties: no W
    np.testing.assert_allclose(L2DataMisfit(sim, dobs).W, np.ones(nD))


def test_weighted_least_squares_construction():
    """WeightedLeastSquares: alphas from length scales (alpha_j = (length_scale_j * smallest
    cell width)^2, regularization/base.py), reference model on the simulation's device, and
    the reference's second positional argument (active cells) accepted only when every cell
    is active."""
    import torch

    from simpeg_gb300.inversion import WeightedLeastSquares
    from simpeg_gb300.mesh import TensorMesh

    mesh = TensorMesh([[(5.0, 4)], [(10.0, 3)], [(2.5, 2)]])

    class Sim:
        engine = None
        device = torch.device("cpu")
        nC = 24

    reg = WeightedLeastSquares(mesh, Sim(), length_scale_x=2.0, alpha_y=3.0, reference_model=np.arange(24.0))
    assert reg.base_length == 2.5
    assert reg.alpha_x == (2.0 * 2.5) ** 2 and reg.alpha_y == 3.0 and reg.alpha_z == 2.5 ** 2
    np.testing.assert_array_equal(reg.mref.numpy(), np.arange(24.0))
    with pytest.raises(ValueError):
        WeightedLeastSquares(mesh, Sim(), alpha_x=1.0, length_scale_x=1.0)
    mask = np.ones(24, bool)
    mask[3] = False
    with pytest.raises(NotImplementedError):
        WeightedLeastSquares(mesh, mask)


def test_inject_active_cells_and_general_combo_derivative():
    """InjectActiveCells (out[active] = m, out[~active] = value) and the chain rule of
    ComboMap through it (sparse, not diagonal); diagonal chains keep diag_deriv and agree
    with the general derivative."""
    import scipy.sparse as sp_

    from simpeg_gb300.maps import ComboMap, ExpMap, IdentityMap, InjectActiveCells
    from simpeg_gb300.mesh import TensorMesh

    mesh = TensorMesh([3, 2, 2])
    act = np.array([True, False, True, True, False, True, True, True, False, True, True, True])
    inj = InjectActiveCells(mesh, act, value_inactive=1e-8)
    assert inj.nP == act.sum() and inj.shape == (12, act.sum()) and not inj.is_diagonal
    rng = np.random.default_rng(2)
    m = rng.standard_normal(inj.nP)
    out = inj * m
    np.testing.assert_array_equal(out[act], m)
    np.testing.assert_array_equal(out[~act], 1e-8)
    np.testing.assert_array_equal(inj.inverse(out), m)
    combo = ComboMap([ExpMap(), inj])
    assert not combo.is_diagonal
    with pytest.raises(NotImplementedError):
        combo.diag_deriv(m)
    D = combo.deriv(m)
    assert sp_.issparse(D) and D.shape == (12, inj.nP)
    v = rng.standard_normal(inj.nP)
    h = 1e-6
    fd = (combo * (m + h * v) - combo * (m - h * v)) / (2 * h)
    np.testing.assert_allclose(D @ v, fd, rtol=1e-6, atol=1e-12)
    diag_chain = ComboMap([ExpMap(), IdentityMap()])
    x = rng.standard_normal(12)
    assert diag_chain.is_diagonal
    np.testing.assert_allclose(diag_chain.deriv(x).diagonal(), diag_chain.diag_deriv(x))
    np.testing.assert_array_equal(InjectActiveCells(mesh, np.flatnonzero(act)).active_cells, act)
    import torch

    np.testing.assert_array_equal(inj.transform_dev(torch.as_tensor(m)).numpy(), out)


def test_simulation_sigma_derivative_selection():
    """The simulation's d sigma / d m: a diagonal array for diagonal maps (the device path),
    a sparse (nC, nP) matrix through InjectActiveCells (applied on the host); the IP
    simulation's -sigma * d eta / dm likewise."""
    import scipy.sparse as sp_

    from simpeg_gb300.induced_polarization.simulation import Simulation3DNodal as IPNodal
    from simpeg_gb300.maps import ComboMap, ExpMap, IdentityMap, InjectActiveCells
    from simpeg_gb300.mesh import TensorMesh
    from simpeg_gb300.resistivity.simulation import Simulation3DNodal

    mesh = TensorMesh([3, 2, 2])
    act = np.arange(12) % 3 != 1
    m_act = np.linspace(-1.0, 1.0, act.sum())

    class Stub:
        @property
        def model(self):
            return self._model

    s = Stub()
    s.sigmaMap = ExpMap(mesh)
    s._model = np.linspace(-1.0, 1.0, 12)
    d = Simulation3DNodal._conductivity_deriv(s)
    assert isinstance(d, np.ndarray)
    np.testing.assert_allclose(d, np.exp(s._model))
    s.sigmaMap = ComboMap([ExpMap(), InjectActiveCells(mesh, act, value_inactive=-3.0)])
    s._model = m_act
    D = Simulation3DNodal._conductivity_deriv(s)
    assert sp_.issparse(D) and D.shape == (12, act.sum())
    np.testing.assert_allclose(D.toarray()[act], np.diag(np.exp(m_act)))

    ip = Stub()
    ip.sigma = np.full(12, 0.01)
    ip.nC = 12
    ip.etaMap = IdentityMap()
    ip._model = np.full(12, 0.1)
    np.testing.assert_allclose(IPNodal._sigma_deriv(ip), -0.01 * np.ones(12))
    ip.etaMap = InjectActiveCells(mesh, act)
    ip._model = np.full(act.sum(), 0.1)
    D = IPNodal._sigma_deriv(ip)
    assert sp_.issparse(D) and D.shape == (12, act.sum())


def test_gpu_solver_unpins_neumann_rows():
    """The Solver plug-in's host transform of a pinned-row matrix (the reference's Neumann getA,
    row 0 = e0): the unpinned matrix is symmetric, and solving it with the pinned column moved to
    the right-hand side gives the pinned matrix's solution (checked with SuperLU on the CPU)."""
    import scipy.sparse.linalg as spla

    from oracle.dc3d import OracleDC3DNodal
    from simpeg_gb300.mesh import TensorMesh
    from simpeg_gb300.resistivity.survey import Survey
    from simpeg_gb300.solver import GPUSolver

    mesh = TensorMesh([[(10.0, 6)], [(10.0, 5)], [(10.0, 4)]], origin="CCN")
    rng = np.random.default_rng(2)
    orc = OracleDC3DNodal(mesh, Survey([]), sigma=10 ** rng.uniform(-2.5, -1.5, mesh.n_cells), bc_type="Neumann")
    A = orc.getA().tocsr()
    A2, pin = GPUSolver._unpin(A)
    assert pin is not None and list(pin[0]) == [0]
    assert abs(A2 - A2.T).max() == 0
    b = rng.standard_normal(A.shape[0])
    rows, diag, C_ = pin
    xp = b[rows] / diag
    x = spla.spsolve(A2.tocsc(), b - C_ @ xp)
    x0 = spla.spsolve(A.tocsc(), b)
    np.testing.assert_allclose(x, x0, rtol=1e-10, atol=1e-12 * np.abs(x0).max())
    # a symmetric matrix passes through unchanged
    S = (A2 + sp.eye(A2.shape[0])).tocsr()
    assert GPUSolver._unpin(S)[1] is None


def test_solver_argument_warns():
    """Simulation3DNodal solves on its own engine: a solver class passed to it is reported as unused."""
    import warnings

    from simpeg_gb300.mesh import TensorMesh
    from simpeg_gb300.resistivity import Simulation3DNodal

    mesh = TensorMesh([[(10.0, 4)], [(10.0, 4)], [(10.0, 4)]], origin="CCN")

    class SolverLU:
        pass

    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        try:
            Simulation3DNodal(mesh, solver=SolverLU)
        except Exception:
            pass  # no CUDA here: the engine may fail to build after the warning
    assert any("SolverLU" in str(w.message) and "not used" in str(w.message) for w in rec)


def test_electrode_tables_numbered_by_first_appearance():
    """The reciprocity tables of getJtJdiag: every datum's A, B, M, N indices point at its electrode
    positions, and electrodes are numbered in order of first appearance over the data, so that along a
    survey line consecutive data use consecutive electrode numbers (distinct shared-memory banks in the
    dc_jtj_diag kernel)."""
    from types import SimpleNamespace

    from simpeg_gb300.resistivity.simulation import Simulation3DNodal

    n_lines, n_st, n_rx = 3, 12, 4
    src_list = []
    for yv in (0.0, 10.0, 20.0):
        for i in range(n_st - n_rx - 2):
            js = i + 1 + np.arange(1, n_rx + 1)
            M = np.c_[5.0 * js, np.full(n_rx, yv), np.zeros(n_rx)]
            N = np.c_[5.0 * (js + 1), np.full(n_rx, yv), np.zeros(n_rx)]
            src_list.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[5.0 * i, yv, 0.0],
                                           np.r_[5.0 * (i + 1), yv, 0.0]))
    survey = Survey(src_list)
    uniq, t = Simulation3DNodal._electrode_tables(SimpleNamespace(survey=survey))
    d = 0
    for src in survey.source_list:
        A, B = np.atleast_2d(src.location)
        for rx in src.receiver_list:
            for r in range(rx.nD):
                np.testing.assert_array_equal(uniq[t["sa"][d]], A)
                np.testing.assert_array_equal(uniq[t["sb"][d]], B)
                np.testing.assert_array_equal(uniq[t["rm"][d]], rx.locations[0][r])
                np.testing.assert_array_equal(uniq[t["rn"][d]], rx.locations[1][r])
                d += 1
    assert d == t["sa"].size
    # every electrode appears once in uniq; along one source's receivers M numbers are consecutive
    assert np.unique(uniq, axis=0).shape[0] == uniq.shape[0]
    assert np.all(np.diff(t["rm"][:n_rx]) == 1)
