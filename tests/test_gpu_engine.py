"""GPU parity of the engine's operators and solves against the CPU oracle."""

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import receivers, sources
from simpeg_gb300.resistivity.boundary import robin_face_weights
from simpeg_gb300.resistivity.survey import Survey

pytestmark = pytest.mark.gpu


def _mesh(kind):
    if kind == "uniform":
        return TensorMesh([[(10.0, 12)], [(10.0, 10)], [(10.0, 8)]], origin="CCN")
    if kind == "padded":
        return TensorMesh([[(5.0, 4, -1.3), (5.0, 10), (5.0, 4, 1.3)], [(5.0, 3, -1.3), (5.0, 9), (5.0, 3, 1.3)],
                           [(5.0, 4, -1.3), (5.0, 7)]], origin="CCN")
    if kind == "odd":
        return TensorMesh([[(7.0, 13)], [(5.0, 11)], [(6.0, 9)]], origin="CCN")
    raise KeyError(kind)


def _sigma(mesh, seed=0):
    rng = np.random.default_rng(seed)
    return 10 ** rng.uniform(-3, -1, mesh.n_cells)


def _oracle(mesh, sigma):
    src = sources.Pole([], np.r_[0.0, 0.0, 0.0])
    return OracleDC3DNodal(mesh, Survey([src]), sigma=sigma)


@pytest.mark.parametrize("kind", ["uniform", "padded", "odd"])
def test_apply_matches_assembled_A(cuda, kind):
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh(kind)
    sigma = _sigma(mesh)
    orc = _oracle(mesh, sigma)
    A = orc.getA()
    eng = DCEngine(mesh.h, robin_face_weights(mesh))
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    rng = np.random.default_rng(1)
    X = rng.standard_normal((3, mesh.n_nodes))
    Y = eng.apply(torch.from_numpy(X).to(cuda)).cpu().numpy()
    Y0 = (A @ X.T).T
    # fp64 stencil vs scipy CSR product: rounding-level agreement
    np.testing.assert_allclose(Y, Y0, rtol=1e-12, atol=1e-12 * np.abs(Y0).max())


@pytest.mark.parametrize("kind", ["uniform", "padded", "odd"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("k", [1, 5, 32, 40])
def test_solve_matches_direct(cuda, kind, mode, k):
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh(kind)
    sigma = _sigma(mesh, seed=k)
    A = _oracle(mesh, sigma).getA().tocsc()
    lu = spla.splu(A)
    eng = DCEngine(mesh.h, robin_face_weights(mesh), coarse_max=64)
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    rng = np.random.default_rng(2)
    B = rng.standard_normal((k, mesh.n_nodes))
    X, info = eng.solve(torch.from_numpy(B).to(cuda), mode=mode, rtol=1e-11)
    X = X.cpu().numpy()
    X0 = lu.solve(B.T).T
    assert info.max_rel_res <= 1e-11
    err = np.linalg.norm(X - X0, axis=1) / np.linalg.norm(X0, axis=1)
    assert err.max() < 1e-8, (err.max(), info)


def _coarse_shapes(h, merge, coarse_max):
    """Cell counts per level under the rule of dc_set_coarsening, restated on the host."""
    hs = [np.asarray(w, dtype=np.float64) for w in h]
    shapes = []
    while True:
        shapes.append(tuple(w.size for w in hs))
        N = int(np.prod([w.size + 1 for w in hs]))
        cz = [w.size >= 4 for w in hs]
        if N <= coarse_max or not any(cz):
            return shapes

        def starts(w, c, wmax):
            n = w.size
            if not c:
                return list(range(n + 1))
            if wmax <= 0:
                fi = list(range(0, n + 1, 2))
                return fi if fi[-1] == n else fi + [n]
            pairs = sorted((i for i in range(n - 1) if w[i] + w[i + 1] <= wmax), key=lambda i: w[i] + w[i + 1])
            used, first = np.zeros(n, bool), np.zeros(n, bool)
            for i in pairs:
                if not used[i] and not used[i + 1]:
                    used[i] = used[i + 1] = first[i] = True
            fi, i = [], 0
            while i < n:
                fi.append(i)
                i += 2 if first[i] else 1
            return fi + [n]

        wmax = 0.0
        if merge > 0:
            wmax = merge * 2.0 * min(w.min() for w in hs) * (1 + 1e-9)
            if np.prod([len(starts(w, c, wmax)) for w, c in zip(hs, cz)]) * 10 > N * 9:
                wmax = 0.0
        new = []
        for w, c in zip(hs, cz):
            fi = starts(w, c, wmax)
            new.append(np.array([w[fi[I]:fi[I + 1]].sum() for I in range(len(fi) - 1)]))
        hs = new


@pytest.mark.parametrize("kind", ["uniform", "padded", "odd", "anisotropic"])
@pytest.mark.parametrize("merge", [0.0, 1.0, 1.5])
def test_coarsening_hierarchy_follows_rule(cuda, kind, merge):
    """Level shapes of full (merge 0) and selective coarsening equal the
    documented rule; on a uniform mesh both are the same hierarchy."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh(kind) if kind != "anisotropic" else \
        TensorMesh([[(20.0, 12)], [(10.0, 16)], [(5.0, 24)]], origin="CCN")
    eng = DCEngine(mesh.h, robin_face_weights(mesh), coarse_max=64, coarsening=merge)
    eng.set_model(torch.from_numpy(_sigma(mesh)).to(cuda))
    got = [cells for cells, _ in eng.levels()]
    assert got == _coarse_shapes(mesh.h, merge, 64), (kind, merge, got)
    if kind == "uniform":
        assert got == _coarse_shapes(mesh.h, 0.0, 64)


def test_selective_coarsening_same_solution_fewer_iterations(cuda):
    """On a padded mesh (1.3x stretched padding) selective coarsening reaches
    the same fp64 residual and solution in fewer PCG iterations."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = TensorMesh([[(5.0, 8, -1.3), (5.0, 32), (5.0, 8, 1.3)], [(5.0, 8, -1.3), (5.0, 32), (5.0, 8, 1.3)],
                       [(5.0, 8, -1.3), (5.0, 24)]], origin="CCN")
    sigma = _sigma(mesh, seed=5)
    rng = np.random.default_rng(6)
    B = torch.from_numpy(rng.standard_normal((16, mesh.n_nodes))).to(cuda)
    out = {}
    for merge in (0.0, 1.0):
        eng = DCEngine(mesh.h, robin_face_weights(mesh), coarsening=merge)
        eng.set_model(torch.from_numpy(sigma).to(cuda))
        X, info = eng.solve(B, mode="mixed", rtol=1e-10)
        assert info.status == 0 and info.max_rel_res <= 1e-10
        out[merge] = (X.cpu().numpy(), info.iterations)
    (X0, it0), (X1, it1) = out[0.0], out[1.0]
    assert np.linalg.norm(X1 - X0) / np.linalg.norm(X0) < 1e-8
    assert it1 < it0, (it0, it1)


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("k", [3, 32, 40])
def test_mixed_solve_every_multigrid_storage(cuda, storage, k):
    """The multigrid storage type changes the preconditioner only: every
    choice reaches the requested fp64 residual and the direct solution."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh("padded")
    sigma = _sigma(mesh, seed=7)
    A = _oracle(mesh, sigma).getA().tocsc()
    eng = DCEngine(mesh.h, robin_face_weights(mesh), coarse_max=64, mg_storage=storage)
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    rng = np.random.default_rng(3)
    B = rng.standard_normal((k, mesh.n_nodes)) * 10.0 ** rng.uniform(-6, 3, (k, 1))  # RHS norms over 9 decades
    X, info = eng.solve(torch.from_numpy(B).to(cuda), mode="mixed", rtol=1e-11)
    X0 = spla.splu(A).solve(B.T).T
    assert info.status == 0 and info.max_rel_res <= 1e-11
    err = np.linalg.norm(X.cpu().numpy() - X0, axis=1) / np.linalg.norm(X0, axis=1)
    assert err.max() < 1e-8, (storage, err.max(), info)


@pytest.mark.parametrize("nu,kind", [(1, 1), (2, 1), (3, 1), (4, 1), (2, 4), (3, 4)])
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_smoother_degrees_and_kinds_reach_the_direct_solution(cuda, nu, kind, mode):
    """Every smoother degree and kind gives a V-cycle that PCG converges with: degree 1 (the first step
    alone), 2 (its second step forms x_1 from r on the coarse levels), 3-4 (the third step forms its
    previous iterate from r too), fourth-kind polynomials; fp64 runs the unfolded steps."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh("padded")
    sigma = _sigma(mesh, seed=13)
    A = _oracle(mesh, sigma).getA().tocsc()
    eng = DCEngine(mesh.h, robin_face_weights(mesh), nu_pre=nu, nu_post=nu, coarse_max=64, smoother=kind)
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    rng = np.random.default_rng(17)
    B = rng.standard_normal((40, mesh.n_nodes))
    X, info = eng.solve(torch.from_numpy(B).to(cuda), mode=mode, rtol=1e-11)
    X0 = spla.splu(A).solve(B.T).T
    assert info.status == 0 and info.max_rel_res <= 1e-11
    assert info.n_levels > 2  # coarse levels with smoothing
    err = np.linalg.norm(X.cpu().numpy() - X0, axis=1) / np.linalg.norm(X0, axis=1)
    assert err.max() < 1e-8, (nu, kind, mode, err.max(), info)


@pytest.mark.parametrize("k", [32, 40, 16])
def test_staged_smoothing_matches_direct_loads(cuda, k):
    """The shared-memory staged finest-level smoothing (bulk asynchronous
    copies) computes the same Chebyshev steps as the direct-load kernel."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = TensorMesh([[(5.0, 4, -1.3), (5.0, 24), (5.0, 4, 1.3)], [(5.0, 3, -1.3), (5.0, 21), (5.0, 3, 1.3)],
                       [(5.0, 4, -1.3), (5.0, 13)]], origin="CCN")
    sigma = _sigma(mesh, seed=11)
    rng = np.random.default_rng(5)
    B = torch.from_numpy(rng.standard_normal((k, mesh.n_nodes))).to(cuda)
    out = {}
    for staged in (True, False):
        eng = DCEngine(mesh.h, robin_face_weights(mesh), coarse_max=64)
        eng.set_staging(staged)
        eng.set_model(torch.from_numpy(sigma).to(cuda))
        X, info = eng.solve(B, mode="mixed", rtol=1e-11)
        assert info.status == 0 and info.max_rel_res <= 1e-11
        out[staged] = (X.cpu().numpy(), info.iterations)
    (xs, its), (xd, itd) = out[True], out[False]
    assert abs(its - itd) <= 1
    np.testing.assert_allclose(xs, xd, rtol=0, atol=1e-9 * np.abs(xd).max())


def test_fp16_multigrid_overflow_falls_back_to_fp32(cuda):
    """1e-8 S/m air cells overflow fp16 multigrid vectors; the solve retries
    with fp32 storage and still reaches the tolerance and the direct solution."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = TensorMesh([[(5.0, 4, -1.3), (5.0, 16), (5.0, 4, 1.3)], [(5.0, 4, -1.3), (5.0, 16), (5.0, 4, 1.3)],
                       [(5.0, 4, -1.3), (5.0, 10), (5.0, 4, 1.3)]], origin="CCN")
    nx, ny, nz = mesh.shape_cells
    s = np.full((nx, ny, nz), 1e-2)
    s[:, :, -4:] = 1e-8
    s[8:14, 8:14, 3:7] = 10.0
    sigma = s.ravel(order="F")
    A = _oracle(mesh, sigma).getA().tocsc()
    rng = np.random.default_rng(4)
    B = np.zeros((12, mesh.n_nodes))
    B[np.arange(12), rng.integers(0, mesh.n_nodes, 12)] = 1.0
    eng = DCEngine(mesh.h, robin_face_weights(mesh), coarse_max=64, mg_storage="fp16")
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    X, info = eng.solve(torch.from_numpy(B).to(cuda), mode="mixed", rtol=1e-10)
    assert info.status == 0 and info.max_rel_res <= 1e-10
    X0 = spla.splu(A).solve(B.T).T
    err = np.linalg.norm(X.cpu().numpy() - X0, axis=1) / np.linalg.norm(X0, axis=1)
    assert err.max() < 1e-7, err.max()


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_fixed_iteration_solve_equals_adaptive(cuda, mode):
    """With at least the adaptive solve's sweeps and iterations, the
    fixed-iteration (graph-recordable) solve returns the same bits: converged
    RHS are frozen, so the extra iterations change nothing."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh("padded")
    sigma = _sigma(mesh, seed=9)
    eng = DCEngine(mesh.h, robin_face_weights(mesh), coarse_max=64)
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    rng = np.random.default_rng(6)
    B = torch.from_numpy(rng.standard_normal((20, mesh.n_nodes))).to(cuda)
    X, info = eng.solve(B, mode=mode, rtol=1e-10)
    Xf, ws = eng.solve_fixed(B, n_inner=info.iterations + 5, n_outer=info.outer + 1, mode=mode, rtol=1e-10)
    mr, na = eng.check_fixed(ws, 20, mode)
    assert na == 0 and mr <= 1e-10
    torch.testing.assert_close(Xf, X, rtol=0, atol=0)


@pytest.mark.parametrize("coarse", ["rediscretised", "galerkin", "series"])
@pytest.mark.parametrize("kind", ["uniform", "padded", "odd"])
def test_coarse_operator_modes_match_direct(cuda, coarse, kind):
    """The coarse multigrid operators change the preconditioner only: with each of the three
    (rediscretised, collapsed Galerkin, series from the finer level) a mixed solve of a model with
    four decades of conductivity contrast reaches the direct solution, for the Robin and the
    Neumann operator."""
    import torch

    from simpeg_gb300.engine import DCEngine

    mesh = _mesh(kind)
    rng = np.random.default_rng(11)
    sigma = 10 ** rng.uniform(-4, 0, mesh.n_cells)
    A = _oracle(mesh, sigma).getA().tocsc()
    lu = spla.splu(A)
    B = rng.standard_normal((6, mesh.n_nodes))
    X0 = lu.solve(B.T).T
    eng = DCEngine(mesh.h, robin_face_weights(mesh))
    eng.set_coarse_operator(coarse)
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    X, info = eng.solve(torch.from_numpy(B).to(cuda), mode="mixed", rtol=1e-11)
    assert info.status == 0 and info.max_rel_res <= 1e-11
    err = np.linalg.norm(X.cpu().numpy() - X0, axis=1) / np.linalg.norm(X0, axis=1)
    assert err.max() < 1e-8, (coarse, err.max(), info)
    # Neumann (the reference pins row 0, simulation.py:535-540) through the simulation, against the oracle
    from simpeg_gb300 import maps
    from simpeg_gb300.resistivity import Simulation3DNodal

    survey = Survey([sources.Pole([receivers.Pole(np.c_[[10.0, 20.0], [0.0, 5.0], [0.0, 0.0]])], np.r_[0.0, 0.0, 0.0])])
    m = np.log(sigma)
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh), bc_type="Neumann")
    orc.set_model(m)
    f = orc.fields()
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), bc_type="Neumann", precision="mixed",
                            rtol=1e-11)
    sim.engine.set_coarse_operator(coarse)
    phi = np.ravel(sim.fields(m)[:, "phi"])
    f = np.ravel(f)
    assert np.linalg.norm(phi - f) / np.linalg.norm(f) < 1e-7, coarse
