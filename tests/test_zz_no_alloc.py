"""GPU test of the allocation-free adjoint entry point ``dc_dadm_adj_noalloc``.

Callers that cannot allocate device memory when they need the adjoint model
derivative (a host framework that has reserved the GPU's memory for its own
pool, or a caller that must not take cudaMalloc's implicit synchronisation)
use this entry point instead of ``dc_dadm_adj``.  It is called here through
the C ABI with caller-owned inputs and outputs, twice in a row, and each
result is compared with the handle-based ``dc_dadm_adj`` on the same inputs.
The file sorts last so that a run stopping at the first failure has already
run every other test.
"""

import ctypes as C

import numpy as np
import pytest

from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity.boundary import robin_face_weights

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _call_noalloc(lib, mesh, h_dev, bf_dev, U, Lam, dsig, scale, stream):
    import torch

    nx, ny, nz = mesh.shape_cells
    g = torch.full((mesh.n_cells,), np.nan, dtype=torch.float64, device=U.device)
    rc = lib.dc_dadm_adj_noalloc(nx, ny, nz, C.c_void_p(h_dev.data_ptr()), C.c_void_p(bf_dev.data_ptr()),
                                 C.c_void_p(U.data_ptr()), C.c_void_p(Lam.data_ptr()), U.shape[0],
                                 C.c_void_p(dsig.data_ptr()), float(scale), C.c_void_p(g.data_ptr()), stream)
    assert rc == 0, lib.dc_last_error().decode()
    return g


def test_noalloc_adjoint_matches_handle_path_twice(cuda):
    import torch

    from simpeg_gb300._lib import lib
    from simpeg_gb300.engine import DCEngine

    L = lib()
    mesh = TensorMesh([[(5.0, 3, -1.3), (5.0, 10), (5.0, 3, 1.3)], [(5.0, 2, -1.3), (5.0, 9), (5.0, 2, 1.3)],
                       [(5.0, 3, -1.3), (5.0, 8)]], origin="CCN")
    rng = np.random.default_rng(17)
    sigma = 10 ** rng.uniform(-3, -1, mesh.n_cells)
    bface = robin_face_weights(mesh)
    eng = DCEngine(mesh.h, bface)
    eng.set_model(torch.from_numpy(sigma).to(cuda))
    h_dev = torch.from_numpy(np.concatenate(mesh.h)).to(cuda)
    bf_dev = torch.from_numpy(bface).to(cuda)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, k in enumerate((7, 3)):
        U = torch.from_numpy(rng.standard_normal((k, mesh.n_nodes))).to(cuda)
        Lam = torch.from_numpy(rng.standard_normal((k, mesh.n_nodes))).to(cuda)
        dsig = torch.from_numpy(sigma * rng.uniform(0.5, 1.5, mesh.n_cells)).to(cuda)
        g_ref = eng.dadm_adj(U, Lam, dsig, scale=-1.0)
        g_new = _call_noalloc(L, mesh, h_dev, bf_dev, U, Lam, dsig, -1.0, stream)
        torch.cuda.synchronize()
        ref = g_ref.cpu().numpy()
        new = g_new.cpu().numpy()
        assert np.all(np.isfinite(new)), f"call {call}: non-finite output"
        err = np.linalg.norm(new - ref) / np.linalg.norm(ref)
        assert err <= TOL, f"call {call}: relative difference {err:.3e}"


def test_noalloc_rejects_oversized_mesh(cuda):
    import torch

    from simpeg_gb300._lib import lib

    L = lib()
    n = 120  # (121)^3 nodes > DC_NOALLOC_MAX_NODES
    dummy = torch.zeros(8, dtype=torch.float64, device=cuda)
    p = C.c_void_p(dummy.data_ptr())
    rc = L.dc_dadm_adj_noalloc(n, n, n, p, p, p, p, 1, p, 1.0, p, C.c_void_p(0))
    assert rc == 1
    assert b"no-allocation scratch" in L.dc_last_error()
