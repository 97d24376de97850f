"""Independent problems of uneven size in one CUDA-graph launch whose solver
loops run on the device: every problem's solution is bit-identical to its own
host-driven adaptive solve (same arithmetic, same stopping rule), its data
matches the simulation's dpred, a second launch reproduces the first, and the
autotuner's choice solves."""

import numpy as np
import pytest

from simpeg_gb300 import maps
from simpeg_gb300.resistivity import Simulation3DNodal
from simpeg_gb300.workloads import batched_problems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_batch_matches_individual_solves(cuda, precision):
    import torch

    from simpeg_gb300.batch import BatchedForward

    probs = batched_problems(seed=7, n=6, lo=(12, 12, 8), hi=(28, 24, 16), src_range=(3, 40), n_rx=5)
    bf = BatchedForward(probs, precision=precision, rtol=1e-10)
    d1 = bf.run()
    assert bf.resolved == []
    conv = bf.convergence()
    assert all(na == 0 and mr <= 1e-10 and it > 0 for mr, na, it, _ in conv), conv
    X1 = [p.X.clone() for p in bf.problems]
    for p in bf.problems:  # stale workspace contents (all-ones bytes: NaN doubles) must not matter
        p.ws.fill_(255)
    bf.launch()
    d2 = bf.data()
    for p, x1, (mr, na, it, sw) in zip(bf.problems, X1, conv):
        xs, info = p.engine.solve(p.Q, mode=precision, rtol=1e-10)
        torch.testing.assert_close(x1, xs, rtol=0, atol=0)
        assert info.iterations == it and info.outer == sw
    for (mesh, sigma, survey), a, b in zip(probs, d1, d2):
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.IdentityMap(mesh), rtol=1e-10)
        ref = sim.dpred(sigma)
        assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < 1e-8
        np.testing.assert_array_equal(a, b)
    bf.close()


def test_autotuner_choice_solves(cuda):
    import torch

    from simpeg_gb300.autotune import tune_engine
    from simpeg_gb300.engine import DCEngine
    from simpeg_gb300.resistivity.boundary import robin_face_weights

    mesh, sigma, survey = batched_problems(seed=8, n=1, lo=(24, 24, 12), hi=(24, 24, 12), src_range=(20, 20))[0]
    eng = DCEngine(mesh.h, robin_face_weights(mesh))
    choice = tune_engine(eng, 20, "mixed", rtol=1e-9, sigma=torch.from_numpy(sigma).cuda(),
                         cands=[(0, 2, 30.0), (8, 3, 60.0), (32, 3, 60.0)])
    assert choice["kb"] in (0, 8, 32) and choice["nu"] in (2, 3)
    B = torch.zeros(20, eng.nN, dtype=torch.float64, device="cuda")
    B[torch.arange(20), torch.arange(20) * 7] = 1.0
    X, info = eng.solve(B, rtol=1e-9)
    assert info.status == 0 and info.max_rel_res <= 1e-9
