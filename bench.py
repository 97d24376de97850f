"""Benchmark: source-solves/s and Jtvec/s of the 1M-cell nodal DC workload.

Workload (seeded, synthetic): TensorMesh 128x128x64 cells (1,081,665 nodes),
5 m core cells, 8 padding cells at x1.3 on each horizontal side and at the
bottom, log10 sigma a Gaussian random field (mean -2, std 0.5, correlation
10 cells), 256 pole sources on a 16x16 surface grid, 40 dipole receivers each
(10,240 data).  Every solve runs to a relative residual of 1e-9.

One step = one forward pass of all 256 sources (multi-RHS solve + receiver
gather).  ``value`` is device-resident throughput (inputs in HBM) of the
mixed-precision path (fp32 multigrid-PCG inner solves + fp64 refinement);
``e2e`` is the same through the public API ``Simulation3DNodal.dpred(m)`` with
the model on the host and the data copied back every step.  The fp64 plain
PCG and Jtvec throughputs, relative errors against an fp64 solve at 1e-13,
the fine-level stencil roofline and the CPU baseline ride along in the line.

``--impl reference`` times the reference's CPU path restated in ``oracle/``
(scipy assembly of A = G^T Me G + Robin diagonal, then a SciPy solve) on the
host cores: SuperLU (the reference's default solver) does not fit in memory at
this size, so each step solves one source with SciPy CG + Jacobi (the
reference's iterative-solver plug-in path) to the same 1e-9 tolerance.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "source-solves/s + Jtvec/s, 1M-cell DC3D: mixed vs FP64 plain on GB300 @<=1e-6 err"
RTOL = 1e-9


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-side", type=int, default=16, help="sources per side of the surface grid")
    ap.add_argument("--sources", type=int, default=0, help="use only the first N sources (profiling runs)")
    ap.add_argument("--workload", default="forward", choices=["forward", "differentiation", "gauss_newton", "batched"],
                    help="forward: the headline 1M-cell line; differentiation: the 96x96x48 gradient checks")
    ap.add_argument("--fd-directions", type=int, default=32)
    ap.add_argument("--profile-solve", action="store_true",
                    help="set up the forward workload, run one mixed solve and exit (for ncu captures; no timing)")
    return ap.parse_args()


def _dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist

    dist.init_process_group("nccl")
    return dist.get_rank(), dist.get_world_size(), dist


def _workload(n_side, n_sources=0):
    from simpeg_gb300 import workloads
    from simpeg_gb300.resistivity.survey import Survey

    mesh, sigma, survey = workloads.scale_forward(seed=1, n_side=n_side)
    if n_sources:
        survey = Survey(survey.source_list[:n_sources])
    return mesh, sigma, survey


def _config(mesh, survey):
    return {
        "workload": "dc3d_nodal_forward_1M",
        "mesh_cells": list(mesh.shape_cells),
        "nodes": int(mesh.n_nodes),
        "sources": int(survey.nSrc),
        "data": int(survey.nD),
        "rtol": RTOL,
        "l2": "inputs larger than L2 (fields 2.2 GB fp64)",
        "parallelism": "replicas",
    }


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _cpu_baseline(mesh, sigma, survey):
    """The oracle (CPU restatement of the reference path) on one source, SciPy CG + Jacobi to 1e-9."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    from oracle.dc3d import OracleDC3DNodal
    from simpeg_gb300.resistivity.survey import Survey

    t0 = time.perf_counter()
    o = OracleDC3DNodal(mesh, Survey(survey.source_list[:1]), sigma=sigma, solver="cg", cg_rtol=RTOL)
    A = o.getA()
    q = o.getRHS()[:, 0]
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    x, info = spla.cg(A, q, rtol=RTOL, atol=0.0, M=sp.diags(1.0 / A.diagonal()), maxiter=20000)
    t_solve = time.perf_counter() - t0
    d = o.dpred(f=x[:, None])
    return {
        "value": 1.0 / t_solve,
        "unit": "source-solves/s",
        "cores": 1,
        "kind": "port",
        "sample": (f"1 of {survey.nSrc} sources: oracle assembly ({t_setup:.1f} s, excluded) + SciPy CG/Jacobi "
                   f"to rtol {RTOL:g} ({t_solve:.1f} s, info={info}); SuperLU does not fit at this size"),
        "_x": x, "_d": d,
    }


def _cpu_worker(mesh, sigma, survey, i, barrier, out):
    """One source of the CPU path in its own process: assembly, then (after every
    worker has assembled) SciPy CG + Jacobi to rtol."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    from oracle.dc3d import OracleDC3DNodal
    from simpeg_gb300.resistivity.survey import Survey

    o = OracleDC3DNodal(mesh, Survey([survey.source_list[i]]), sigma=sigma, solver="cg", cg_rtol=RTOL)
    A = o.getA()
    q = o.getRHS()[:, 0]
    M = sp.diags(1.0 / A.diagonal())
    barrier.wait(timeout=1800)
    t0 = time.perf_counter()
    _, info = spla.cg(A, q, rtol=RTOL, atol=0.0, M=M, maxiter=20000)
    out.put((i, time.perf_counter() - t0, int(info)))


def _cpu_parallel(mesh, sigma, survey, n_proc):
    """The CPU path on all host cores: n_proc sources solved at once, one process each
    (spawned, single-threaded BLAS); throughput = sources / wall time of the solves."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    n_proc = max(1, min(n_proc, survey.nSrc))
    barrier, out = ctx.Barrier(n_proc + 1), ctx.Queue()
    env_old = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")}
    os.environ.update(OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    procs = [ctx.Process(target=_cpu_worker, args=(mesh, sigma, survey, i, barrier, out)) for i in range(n_proc)]
    for pr in procs:
        pr.start()
    for k, v in env_old.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v
    try:
        barrier.wait(timeout=1800)  # every worker assembled (a dead worker breaks the barrier)
        t0 = time.perf_counter()
        res = [out.get(timeout=3600) for _ in range(n_proc)]
        wall = time.perf_counter() - t0
    finally:
        for pr in procs:
            pr.join(timeout=60)
            if pr.is_alive():
                pr.terminate()
    infos = sorted(set(r[2] for r in res))
    return {
        "value": n_proc / wall, "unit": "source-solves/s", "cores": n_proc, "kind": "port",
        "sample": (f"{n_proc} of {survey.nSrc} sources solved concurrently, one process per core: oracle assembly "
                   f"(excluded) + SciPy CG/Jacobi to rtol {RTOL:g}; wall {wall:.1f} s, info {infos}; "
                   "SuperLU does not fit at this size"),
    }


def run_reference(args):
    rank, world, dist = _dist_init(args.gpus)
    if rank != 0:
        return
    mesh, sigma, survey = _workload(args.n_side, args.sources)
    vals = []
    for _ in range(args.warmup):
        pass  # the CPU path has no warm-up state worth priming beyond the first assembly
    last = None
    n_proc = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    for _ in range(args.steps):
        last = _cpu_parallel(mesh, sigma, survey, n_proc)
        vals.append(last["value"])
    v = statistics.median(vals)
    cb = {k: last[k] for k in ("unit", "cores", "kind", "sample")}
    cb["value"] = v
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "source-solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": _config(mesh, survey), "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "source-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _traffic_per_unit():
    """DRAM bytes per (node x RHS) of the fine-level Chebyshev step (fp16 multigrid storage) from the
    committed ncu summary."""
    p = ROOT / "profiles" / "cheb_step_fp16_dc3d.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_node_rhs:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def run_gb300(args):
    import numpy as np
    import torch

    rank, world, dist = _dist_init(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from simpeg_gb300 import maps
    from simpeg_gb300.engine import csr_spmv, kernel_launches, padded_rhs
    from simpeg_gb300.resistivity import Simulation3DNodal

    mesh, sigma, survey = _workload(args.n_side, args.sources)
    m = np.log(sigma)
    K = survey.nSrc
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=RTOL)
    sim.model = m
    sim._ensure_model()
    eng = sim.engine
    t, tq = sim._get_tables()
    Q = sim.getRHS()
    d_out = torch.empty(t.nD, dtype=torch.float64, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def fwd(mode):
        U, info = eng.solve(Q, mode=mode, rtol=RTOL)
        csr_spmv(tq["P_ptr"], tq["P_idx"], tq["P_w"], U.view(-1), d_out)
        return U, info

    rng = np.random.default_rng(5)
    v_host = rng.standard_normal(t.nD)
    v_dev = torch.from_numpy(v_host).to(dev)

    def jtvec(mode, U):
        PTv = torch.zeros(K, mesh.n_nodes, dtype=torch.float64, device=dev)
        csr_spmv(tq["PT_ptr"], tq["PT_idx"], tq["PT_w"], v_dev, PTv.view(-1), out_idx=tq["PT_out"])
        Lam, _ = eng.solve(PTv, mode=mode, rtol=RTOL)
        return eng.dadm_adj(U, Lam, None, scale=-1.0)

    def timed(fn, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record()
        out = None
        for _ in range(steps):
            out = fn()
        e1.record()
        barrier()
        ms = e0.elapsed_time(e1)
        if dist is not None:
            tt = torch.tensor([ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            ms = float(tt.item())
        return ms, out

    # ---- warm-up (also allocates the solver workspaces)
    for _ in range(args.warmup):
        U, info = fwd("mixed")
    jtvec("mixed", U)
    torch.cuda.synchronize()

    # ---- headline: mixed forward, device resident
    n0 = kernel_launches()
    eng.stencil_timing(True)
    with Clocks(local) as clk:
        ms_mixed, (U_mixed, info_mixed) = timed(lambda: fwd("mixed"), args.steps)
    st_ms, st_n, st_bytes = eng.stencil_timing(False)
    launches = kernel_launches() - n0
    clocks = clk.summary()
    d_mixed = d_out.cpu().numpy()

    # ---- Jtvec (mixed), fp64 forward and Jtvec
    ms_jt_mixed, g_mixed = timed(lambda: jtvec("mixed", U_mixed), args.steps)
    g_mixed = g_mixed.cpu().numpy()
    fwd("fp64")
    ms_fp64, (U64, info64) = timed(lambda: fwd("fp64"), args.steps)
    ms_jt_fp64, _ = timed(lambda: jtvec("fp64", U64), args.steps)

    # ---- accuracy against an fp64 solve at 1e-13 (the oracle at this size).  1e-13 is at the
    # rounding floor of the fp64 residual on this mesh: a solve that stops within 5e-13 is accepted.
    U_ref, info_ref = eng.solve(Q, mode="fp64", rtol=1e-13, raise_on_fail=False)
    csr_spmv(tq["P_ptr"], tq["P_idx"], tq["P_w"], U_ref.view(-1), d_out)
    d_ref = d_out.cpu().numpy()
    PTv = torch.zeros(K, mesh.n_nodes, dtype=torch.float64, device=dev)
    csr_spmv(tq["PT_ptr"], tq["PT_idx"], tq["PT_w"], v_dev, PTv.view(-1), out_idx=tq["PT_out"])
    Lam_ref, info_lam = eng.solve(PTv, mode="fp64", rtol=1e-13, raise_on_fail=False)
    oracle_res = max(info_ref.max_rel_res, info_lam.max_rel_res)
    if not oracle_res <= 5e-13:
        raise RuntimeError(f"fp64 oracle solve stopped at relative residual {oracle_res:.2e}")
    g_ref = eng.dadm_adj(U_ref, Lam_ref, None, scale=-1.0).cpu().numpy()
    del Lam_ref, PTv
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    err = {"dpred": rel(d_mixed, d_ref), "jtvec_sigma": rel(g_mixed, g_ref)}

    # ---- end to end through the public API: host model in, host data out
    m2 = m + 1e-3 * rng.standard_normal(m.size)
    models = [m, m2]
    sim.dpred(m2)
    e2e_steps = args.steps
    barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        dd = sim.dpred(models[i % 2])
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        tt = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    h2d = int(mesh.n_cells * 8)
    d2h = int(t.nD * 8)

    value = world * K * args.steps / (ms_mixed / 1e3)
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = (st_bytes / st_n) / (st_ms / st_n * 1e-3) / 1e9 if st_n else None
    tpu = _traffic_per_unit()
    traffic = tpu * mesh.n_nodes * padded_rhs(K) if tpu is not None else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "source-solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 inner / f64 refinement",
        "data": "synthetic (seeded Gaussian random field, 16x16 pole grid)",
        "config": _config(mesh, survey),
        "jtvec_per_s": world * args.steps / (ms_jt_mixed / 1e3),
        "fp64_plain": {
            "source_solves_per_s": world * K * args.steps / (ms_fp64 / 1e3),
            "jtvec_per_s": world * args.steps / (ms_jt_fp64 / 1e3),
            "iterations": info64.iterations,
        },
        "speedup_vs_fp64": {"forward": ms_fp64 / ms_mixed, "jtvec": ms_jt_fp64 / ms_jt_mixed},
        "mixed_solve": {"inner_iterations": info_mixed.iterations, "outer": info_mixed.outer,
                        "max_rel_res": info_mixed.max_rel_res, "levels": info_mixed.n_levels},
        "rel_err_vs_fp64_1e-13": err,
        "oracle_max_rel_res": oracle_res,
        "e2e": {"value": world * K * e2e_steps / e2e_s, "unit": "source-solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "Simulation3DNodal.dpred(m): host model -> H2D -> exp map on device -> set_model -> solve -> gather -> D2H"},
        "roofline": {
            "kernel": "k_cheb_step<float,__half,*,32> (fine-level Chebyshev stencil step, fp16 multigrid storage)",
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": traffic,
            "launches_timed": st_n,
            "alg_bytes_per_launch": (st_bytes / st_n) if st_n else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if pk.exists() else "fallback",
        },
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = _cpu_baseline(mesh, sigma, survey)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def run_differentiation(args):
    """96x96x48 cells, m = ln sigma (ExpMap), 128 dipole sources x 30 receivers.

    Gradient of the L2 data misfit by the autograd backward (adjoint solve +
    dA/dsigma kernel), checked against central finite differences (step 1e-4)
    on random unit directions, and against an fp64 Jtvec at rtol 5e-13 (the
    oracle at this size); run in fp64 and in mixed precision with forward
    recomputation.  Prints one JSON line.
    """
    import numpy as np
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.autograd import dpred
    from simpeg_gb300.resistivity import Simulation3DNodal

    torch.cuda.set_device(0)
    mesh, m, survey = workloads.differentiation(seed=2)
    rng = np.random.default_rng(11)
    # fp64 reference at 5e-13 (a 1e-13 target sits at the fp64 residual's rounding floor on this mesh)
    ref = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=5e-13)
    d_true = ref.dpred(m)
    dobs = torch.from_numpy(d_true * (1 + 0.03 * rng.standard_normal(d_true.size)))
    m0 = m + 0.1 * rng.standard_normal(m.size)
    r0 = ref.dpred(m0) - dobs.numpy()
    g_ref = ref.Jtvec(m0, r0)
    out = {"metric": "misfit gradient: autograd vs central FD and fp64 Jtvec", "workload": "dc3d_differentiation",
           "config": {"mesh_cells": list(mesh.shape_cells), "nodes": int(mesh.n_nodes), "sources": survey.nSrc,
                      "data": survey.nD, "fd_step": 1e-4, "directions": args.fd_directions}}
    dirs = [v / np.linalg.norm(v) for v in rng.standard_normal((args.fd_directions, m.size))]
    for label, precision, recompute in (("fp64", "fp64", False), ("mixed_recompute", "mixed", True)):
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=1e-11)

        def phi(mm):
            r = dpred(sim, mm, recompute=recompute) - dobs
            return 0.5 * (r * r).sum()

        mt = torch.tensor(m0, requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f = phi(mt)
        f.backward()
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        g = mt.grad.numpy()
        errs = []
        for v in dirs:
            with torch.no_grad():
                fp = phi(torch.from_numpy(m0 + 1e-4 * v)).item()
                fm = phi(torch.from_numpy(m0 - 1e-4 * v)).item()
            fd = (fp - fm) / 2e-4
            errs.append(abs(fd - g @ v) / max(abs(fd), 1e-300))
        out[label] = {"grad_seconds": t_grad, "fd_max_rel_err": float(max(errs)),
                      "fd_median_rel_err": float(np.median(errs)),
                      "rel_err_vs_fp64_jtvec": float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref))}
    print(json.dumps(out), flush=True)


def run_gauss_newton(args):
    """160x160x80 cells (~2.05 M), 512 dipole sources x 48 receivers, m = ln sigma.

    One inexact Gauss-Newton step at the starting model: fields, data misfit
    gradient plus smallness + smoothness regularisation, exact getJtJdiag
    (electrode reciprocity) for the Jacobi preconditioner, and 10 CG iterations
    on 2 J^T W^2 J + 2 beta R, each one batched Jvec and one batched Jtvec.
    Run in mixed precision and in plain fp64 on the same GPU; prints times and
    the relative differences of g, diag(J^T J) and the search direction.
    """
    import numpy as np
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.inversion import L2DataMisfit, WeightedLeastSquares, inexact_gauss_newton_direction
    from simpeg_gb300.resistivity import Simulation3DNodal

    torch.cuda.set_device(0)
    mesh, m_true, m0, survey = workloads.gauss_newton(seed=4)
    truth = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=1e-10)
    rng = np.random.default_rng(9)
    d = truth.dpred(m_true)
    dobs = d * (1 + 0.02 * rng.standard_normal(d.size))
    W = 1.0 / (0.02 * np.abs(dobs) + 1e-5 * np.abs(dobs).max())
    del truth
    torch.cuda.empty_cache()
    beta = 10.0
    # untimed warm-up: one step of a 16x16x8-core problem per precision, so that first-call costs of
    # the process (module loading of every kernel the step uses, torch's and this library's) are
    # paid before either timed step, not by whichever precision runs first
    wmesh, _, wm0, wsurvey = workloads.gauss_newton(seed=4, n_lines=2, src_per_line=4, n_rx=4, ncore_xy=16,
                                                     ncore_z=8)
    for precision in ("mixed", "fp64"):
        wsim = Simulation3DNodal(wmesh, survey=wsurvey, sigmaMap=maps.ExpMap(wmesh), precision=precision,
                                 rtol=RTOL)
        inexact_gauss_newton_direction(L2DataMisfit(wsim, np.zeros(wsurvey.nD)), WeightedLeastSquares(wmesh, wsim),
                                       beta, wm0, cg_maxiter=2)
        del wsim
    torch.cuda.synchronize()
    out = {"metric": "Gauss-Newton step (getJtJdiag + gradient + 10 CG iterations): mixed vs fp64",
           "workload": "dc3d_gauss_newton",
           "config": {"mesh_cells": list(mesh.shape_cells), "nodes": int(mesh.n_nodes), "sources": survey.nSrc,
                      "data": survey.nD, "beta": beta, "cg_iterations": 10, "rtol": RTOL}}
    res = {}
    for precision in ("mixed", "fp64"):
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=RTOL)
        dmis = L2DataMisfit(sim, dobs, W=W)
        reg = WeightedLeastSquares(mesh, sim)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p, info = inexact_gauss_newton_direction(dmis, reg, beta, m0, cg_maxiter=10)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        res[precision] = (p.cpu().numpy(), info["g"].cpu().numpy(), info["jtj_diag"].cpu().numpy())
        out[precision] = {"seconds": dt, "cg_rel_res": info["cg_rel_res"][-1],
                          "phases_seconds": {k: round(v, 3) for k, v in info["seconds"].items()}}
        del sim, dmis, reg, p, info
        torch.cuda.empty_cache()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out["speedup_vs_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    out["rel_err_mixed_vs_fp64"] = {"direction": rel(res["mixed"][0], res["fp64"][0]),
                                    "gradient": rel(res["mixed"][1], res["fp64"][1]),
                                    "jtj_diag": rel(res["mixed"][2], res["fp64"][2])}
    print(json.dumps(out), flush=True)


def run_batched(args):
    """64 independent problems, cell counts log-uniform from 32x32x16 to 96x96x64,
    16-128 pole sources x 20 dipole receivers each, own block + random-field
    conductivity.  After the autotuner picks RHS-block width and smoother per
    problem, all 64 adaptive solves are recorded into one CUDA graph whose
    solver loops run on the device; the timed step is one launch of that graph
    (inputs resident).  Compared with solving the same problems one after the
    other with the host-driven adaptive solver (identical results)."""
    import numpy as np
    import torch

    from simpeg_gb300 import workloads
    from simpeg_gb300.batch import BatchedForward

    torch.cuda.set_device(0)
    probs = workloads.batched_problems(seed=5, n=64)
    nsrc = sum(sv.nSrc for _, _, sv in probs)
    t0 = time.perf_counter()
    bf = BatchedForward(probs, precision="mixed", rtol=RTOL, tune=True)
    t_setup = time.perf_counter() - t0
    for _ in range(args.warmup):
        bf.launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        bf.launch()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    conv = bf.convergence()
    # the same problems one by one, adaptive solver, same engines and workspaces
    torch.cuda.synchronize()
    e0.record()
    for p in bf.problems:
        p.engine.solve(p.Q, mode="mixed", rtol=RTOL, ws=p.ws)
    e1.record()
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1)
    tunes = [getattr(p, "tuning", None) for p in bf.problems]
    out = {"metric": "batched uneven problems: source-solves/s, one CUDA-graph launch vs sequential",
           "workload": "dc3d_batched_64", "value": nsrc / (ms / 1e3), "unit": "source-solves/s",
           "ms_per_launch": ms, "steps": args.steps,
           "sequential": {"ms": ms_seq, "source_solves_per_s": nsrc / (ms_seq / 1e3)},
           "speedup_vs_sequential": ms_seq / ms,
           "converged": all(c[1] == 0 for c in conv), "max_rel_res": max(c[0] for c in conv),
           "inner_iterations": [min(c[2] for c in conv), max(c[2] for c in conv)],
           "setup_seconds": t_setup,
           "config": {"problems": len(probs), "sources": nsrc,
                      "nodes_range": [min(p[0].n_nodes for p in probs), max(p[0].n_nodes for p in probs)],
                      "rtol": RTOL},
           "autotune": {"kb": sorted({t["kb"] for t in tunes if t}), "nu": sorted({t["nu"] for t in tunes if t})}}
    print(json.dumps(out), flush=True)


def run_profile_solve(args):
    """One mixed-precision solve of the forward workload (the first --sources
    sources), nothing else: a short program for ncu to capture."""
    import numpy as np
    import torch

    from simpeg_gb300 import maps
    from simpeg_gb300.resistivity import Simulation3DNodal

    torch.cuda.set_device(0)
    mesh, sigma, survey = _workload(args.n_side, args.sources)
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=RTOL)
    sim.model = np.log(sigma)
    sim._ensure_model()
    _, info = sim.engine.solve(sim.getRHS(), mode="mixed", rtol=RTOL)
    torch.cuda.synchronize()
    print(json.dumps({"profile_solve": str(info), "sources": survey.nSrc}), flush=True)


def main():
    args = _args()
    if args.profile_solve:
        return run_profile_solve(args)
    if args.workload == "batched" and args.impl != "reference":
        return run_batched(args)
    if args.workload == "gauss_newton" and args.impl != "reference":
        return run_gauss_newton(args)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "differentiation":
        run_differentiation(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
