"""Source-sharded simulation over two ranks (gloo, CPU): dpred/Jvec gathered
and Jtvec/getJtJdiag all-reduced equal the single-process results
(tests/meta/test_meta_sim.py recipe).  The per-rank simulation here is the
CPU oracle, or (GPU test) the GPU Simulation3DNodal; on a multi-GPU machine each rank
runs it on its own GPU and the collectives go over NCCL with device tensors."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case():
    from simpeg_gb300.mesh import TensorMesh
    from simpeg_gb300.resistivity import receivers, sources
    from simpeg_gb300.resistivity.survey import Survey

    mesh = TensorMesh([[(10.0, 2, -1.3), (10.0, 8), (10.0, 2, 1.3)], [(10.0, 8)], [(10.0, 2, -1.3), (10.0, 5)]],
                      origin="CCN")
    xs = np.arange(-30.0, 31.0, 10.0)
    srcs = []
    for i in range(5):
        M = np.c_[xs[(i + 2) % 5:(i + 2) % 5 + 2], np.zeros(2), np.zeros(2)]
        N = M + np.r_[10.0, 0.0, 0.0]
        srcs.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[xs[i], 0, 0], np.r_[xs[i] - 10.0, 0, 0]))
    rng = np.random.default_rng(0)
    m = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    return mesh, Survey(srcs), m


def _worker(rank, world, port, q, gpu=False):
    import scipy.sparse as sp
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle.dc3d import OracleDC3DNodal
        from simpeg_gb300 import maps
        from simpeg_gb300.parallel import ShardedSimulation

        mesh, survey, m = _case()
        if gpu:  # the GPU simulation as each rank's child (both ranks share cuda:0 here)
            from simpeg_gb300.resistivity import Simulation3DNodal

            factory = lambda sv: Simulation3DNodal(mesh, survey=sv, sigmaMap=maps.ExpMap(mesh), rtol=1e-12,
                                                   precision="fp64")
        else:
            factory = lambda sv: OracleDC3DNodal(mesh, sv, sigma_map=maps.ExpMap(mesh))
        sharded = ShardedSimulation(survey, factory)
        full = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
        rng = np.random.default_rng(3)
        v = rng.standard_normal(mesh.n_cells)
        w = rng.standard_normal(survey.nD)
        W = sp.diags(rng.uniform(0.5, 2.0, survey.nD))
        res = {
            "dpred": (sharded.dpred(m), full.dpred(m)),
            "jvec": (sharded.Jvec(m, v), full.Jvec(m, v)),
            "jtvec": (sharded.Jtvec(m, w), full.Jtvec(m, w)),
            "jtj": (sharded.getJtJdiag(m, W=W), full.getJtJdiag(m, W=W)),
        }
        errs = {k: float(np.linalg.norm(a - b) / np.linalg.norm(b)) for k, (a, b) in res.items()}
        q.put((rank, errs, len(sharded.my_sources)))
    finally:
        dist.destroy_process_group()


def _run_two_ranks(gpu):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q, gpu)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(n for _, _, n in out) == [2, 3]
    for rank, errs, _ in out:
        for k, e in errs.items():
            # GPU children: solves to 1e-12, getJtJdiag with fp32 cell arithmetic (1e-6 of the oracle)
            assert e < ((1e-6 if k == "jtj" else 1e-8) if gpu else 1e-9), (rank, k, e)


def test_sharded_simulation_two_ranks():
    _run_two_ranks(gpu=False)


@pytest.mark.gpu
def test_sharded_simulation_two_ranks_gpu_children():
    """The same collectives with GPU simulations as the ranks' children (gloo between the two
    processes; no kernel of one rank waits on the other)."""
    _run_two_ranks(gpu=True)
