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

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "source-solves/s + Jtvec/s, 1M-cell DC3D: mixed vs FP64 plain on GB300 @<=1e-6 err"
RTOL = 1e-9

# SciPy SuperLU (what the reference's default SolverLU runs) on nodal 7-point matrices, measured
# on one core (Xeon 2.7 GHz): nodes -> (factor s, nnz(L+U), solve s per right-hand side).
SUPERLU_PROBES = {18513: (1.25, 12.2e6, 6.3e-3), 60025: (21.2, 85.3e6, 40.7e-3), 139425: (136.9, 321e6, 154e-3)}


def _superlu_extrapolated(n_nodes=1081665, n_rhs=256):
    """Power laws through the two largest probes, taken to n_nodes (not run: the fill does not fit)."""
    (n1, a), (n2, b) = sorted(SUPERLU_PROBES.items())[1:]
    r = n_nodes / n2
    ex = [float(np.log(b[i] / a[i]) / np.log(n2 / n1)) for i in range(3)]
    fac, nnz, sol = (b[i] * r ** ex[i] for i in range(3))
    return {"nodes": n_nodes, "factor_s": fac, "nnz_LU": nnz, "memory_GB": nnz * 12 / 1e9, "solve_s_per_rhs": sol,
            f"source_solves_per_s_{n_rhs}": n_rhs / (fac + n_rhs * sol),
            "exponents": {"factor": ex[0], "fill": ex[1], "solve": ex[2]},
            "basis": "SciPy SuperLU probes at 60k and 139k nodes (one core), power laws extrapolated; not run"}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle", action="store_true", help="skip the oracle spot checks at full size")
    ap.add_argument("--n-side", type=int, default=16, help="sources per side of the surface grid")
    ap.add_argument("--sources", type=int, default=0, help="use only the first N sources (profiling runs)")
    ap.add_argument("--workload", default="forward",
                    choices=["forward", "block", "differentiation", "gauss_newton", "batched", "cc", "serving"],
                    help="forward: the headline 1M-cell line; differentiation: the 96x96x48 gradient checks")
    ap.add_argument("--fd-directions", type=int, default=32)
    ap.add_argument("--profile-solve", action="store_true",
                    help="set up the forward workload, run one mixed solve and exit (for ncu captures; no timing)")
    ap.add_argument("--sens-full-survey", action="store_true",
                    help="with --profile-sens: the full Gauss-Newton survey on a 64x64x32-cell mesh")
    ap.add_argument("--profile-sens", action="store_true",
                    help="a reduced Gauss-Newton workload (96x96x48 cells, --sources dipoles): one getJtJdiag and one "
                         "Jtvec, nothing else (for ncu captures of the sensitivity kernels; no timing)")
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


ORACLE_RTOL = 1e-12


def _oracle_spot_worker(mesh, m, src, v_s, rtol):
    """One source of the oracle (the CPU restatement of the reference path, fp64 SciPy CG + Jacobi
    to ``rtol``): the source's data and ``J^T v_s`` with respect to m = ln sigma.  Runs in a spawned
    process (never the product path)."""
    from oracle.dc3d import OracleDC3DNodal
    from simpeg_gb300 import maps
    from simpeg_gb300.resistivity.survey import Survey

    t0 = time.perf_counter()
    o = OracleDC3DNodal(mesh, Survey([src]), sigma_map=maps.ExpMap(mesh), solver="cg", cg_rtol=rtol)
    o.set_model(m)
    f = o.fields()
    d = o.dpred(f=f)
    g = o.Jtvec(m, v_s, f=f) if v_s is not None else None
    return d, g, time.perf_counter() - t0


def _oracle_spot_worker_cc(mesh, m, src, v_s, rtol):
    """One source of the cell-centred oracle (``oracle/cc3d.py``: Robin ``Div MfRhoI Grad``, fp64 SciPy
    CG + Jacobi to ``rtol``): the source's data and ``J^T v_s`` with respect to m = ln sigma.  Runs in a
    spawned process (never the product path)."""
    from oracle.cc3d import OracleDC3DCellCentered
    from simpeg_gb300 import maps
    from simpeg_gb300.resistivity.survey import Survey

    t0 = time.perf_counter()
    o = OracleDC3DCellCentered(mesh, Survey([src]), sigma_map=maps.ExpMap(mesh), solver="cg", cg_rtol=rtol)
    o.set_model(m)
    f = o.fields()
    d = o.dpred(f=f)
    g = o.Jtvec(m, v_s, f=f) if v_s is not None else None
    return d, g, time.perf_counter() - t0


class OracleSpots:
    """Independent at-scale parity: a few sources of the workload solved by the oracle on the host
    (spawned processes, one per source, overlapping the GPU work), compared with the GPU path."""

    def __init__(self, mesh, m, survey, idx, v, rtol=ORACLE_RTOL, worker=_oracle_spot_worker):
        import multiprocessing as mp

        self.idx = list(idx)
        self.rtol = rtol
        ctx = mp.get_context("spawn")
        env_old = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")}
        os.environ.update(OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
        self.pool = ctx.Pool(len(self.idx))
        for k, val in env_old.items():
            if val is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = val
        sl = survey.get_all_slices() if hasattr(survey, "get_all_slices") else None
        self.slices = []
        self.jobs = []
        for i in self.idx:
            src = survey.source_list[i]
            rx = src.receiver_list[0]
            s_ = sl[src, rx] if sl is not None else None
            self.slices.append(s_)
            vs = None if v is None else np.ascontiguousarray(v[s_])
            self.jobs.append(self.pool.apply_async(worker, (mesh, m, src, vs, rtol)))

    def compare(self, d_gpu, jtvec_gpu_fn, timeout=1800):
        """d_gpu: the GPU data of the whole survey; jtvec_gpu_fn(i, v_s): the GPU J^T v_s of source i
        alone.  Returns the worst relative errors over the sources."""
        rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
        ed, eg, secs = [], [], []
        try:
            for i, s_, job in zip(self.idx, self.slices, self.jobs):
                d, g, t = job.get(timeout=timeout)
                secs.append(t)
                ed.append(rel(d_gpu[s_], d))
                if g is not None:
                    eg.append(rel(jtvec_gpu_fn(i, s_), g))
        finally:
            self.pool.close()
            self.pool.terminate()
        out = {"sources": self.idx, "dpred": max(ed)}
        if eg:
            out["jtvec_m"] = max(eg)
        out["oracle"] = (f"CPU restatement of the reference path (oracle/), fp64 SciPy CG + Jacobi to rtol "
                         f"{self.rtol:g}, one process per source")
        out["oracle_seconds_per_source"] = secs
        return out


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


# Algorithmic bytes per (node x RHS lane) of each kind of fine-level Chebyshev step with fp16 lanes:
# momentum kinds read r, x_k, x_{k-1} and write x_{k+1}; the others read r, x_k and write x_{k+1}.
STEP_LANE_BYTES = {"plain": 6.0, "zero_start": 6.0, "momentum": 8.0, "momentum_rz": 8.0}


def _traffic_by_kind():
    """DRAM bytes per (node x RHS) of each kind of fine-level Chebyshev step (fp16 multigrid storage),
    from the committed ncu summary (lines ``dram_bytes_per_node_rhs[<kind>]: <value>``)."""
    import re

    p = ROOT / "profiles" / "cheb_step_fp16_dc3d.md"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            mt = re.match(r"\s*dram_bytes_per_node_rhs\[(\w+)\]:\s*([0-9.eE+-]+)", line)
            if mt:
                out[mt.group(1)] = float(mt.group(2))
    return out


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
    rng = np.random.default_rng(5)
    v_host = rng.standard_normal(survey.nD)
    # independent parity at full size: the first and last source solved by the oracle on the host,
    # in spawned processes that overlap the GPU work below
    spots = None
    if rank == 0 and not args.no_oracle:
        spots = OracleSpots(mesh, m, survey, sorted({0, K - 1}), v_host)
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
    kinds = eng.stencil_timing_kinds()
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
    roof = _stencil_roofline(st_ms, st_n, st_bytes, kinds)
    # DRAM traffic per launch: the ncu bytes of each kind of step, weighted by this run's launch mix
    tbk = _traffic_by_kind()
    if roof is not None and kinds and all(k in tbk for k in kinds):
        units = mesh.n_nodes * padded_rhs(K)
        roof["traffic"] = sum(c * tbk[k] * units for k, (c, _, _) in kinds.items()) / st_n
        roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per kind of step "
                                  "(profiles/cheb_step_fp16_dc3d.md), weighted by the launches timed here")
        for k, v in roof["by_kind"].items():
            v["traffic_per_launch"] = tbk[k] * units
    elif roof is not None:
        roof["traffic_source"] = "no ncu figure for every kind of step timed: not reported"
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
        "roofline": roof,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if spots is not None:
        from simpeg_gb300.resistivity.survey import Survey

        def jt_one(i, s_):
            one = Simulation3DNodal(mesh, survey=Survey([survey.source_list[i]]), sigmaMap=maps.ExpMap(mesh),
                                    precision="mixed", rtol=RTOL)
            return one.Jtvec(m, v_host[s_])

        line["rel_err_vs_oracle_cg"] = spots.compare(d_mixed, jt_one)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = _cpu_baseline(mesh, sigma, survey)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        line["cpu_baseline"]["solver"] = ("SciPy CG + Jacobi (an iterative plug-in): the reference's default "
                                          "direct solver (SuperLU) does not fit at this size")
        line["superlu_extrapolated"] = _superlu_extrapolated(mesh.n_nodes, K)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _peak_hbm():
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        return json.loads(pk.read_text()).get("hbm_gbs", 6800.0), "MEASURED_PEAKS.json hbm_gbs (measured)"
    return 6800.0, "fallback"


def _stencil_roofline(ms, n, alg_bytes, kinds=None, what="fine-level Chebyshev steps", scaled_traffic=False):
    """Roofline of the fine-level Chebyshev steps timed with CUDA events inside a timed region."""
    if not n:
        return None
    peak, src = _peak_hbm()
    ach = alg_bytes / (ms * 1e-3) / 1e9
    out = {"kernel": f"k_cheb_step<float,__half,*,*> ({what}, fp16 multigrid storage)", "bound": "hbm",
           "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
           "launches_timed": n, "alg_bytes_per_launch": alg_bytes / n, "peak_source": src}
    if kinds:
        out["by_kind"] = {k: {"launches": c, "us_per_launch": t / c * 1e3, "achieved": b / (t * 1e-3) / 1e9,
                              "frac": b / (t * 1e-3) / 1e9 / peak} for k, (c, t, b) in kinds.items()}
        if scaled_traffic:
            # DRAM bytes over algorithmic bytes of each kind in the profiled 1M-node, 256-RHS solve (fp16 lanes:
            # STEP_LANE_BYTES per node-RHS plus 20 B per node), applied to this run's algorithmic bytes of that kind
            tbk = _traffic_by_kind()
            if all(k in tbk for k in kinds):
                alg_nr = {k: (STEP_LANE_BYTES[k] * 256 + 20.0) / 256 for k in kinds}
                out["traffic"] = sum(b * tbk[k] / alg_nr[k] for k, (_, _, b) in kinds.items()) / n
                out["traffic_source"] = ("ncu DRAM bytes / algorithmic bytes of each kind of step in the profiled "
                                         "1M-node 256-RHS solve (profiles/cheb_step_fp16_dc3d.md), times this run's "
                                         "algorithmic bytes of that kind")
    return out


def run_differentiation(args):
    """96x96x48 cells, m = ln sigma (ExpMap), 128 dipole sources x 30 receivers.

    Gradient of the L2 data misfit by the autograd backward (adjoint solve +
    dA/dsigma kernel), checked against central finite differences (step 1e-4)
    on random unit directions, against an fp64 Jtvec at rtol 5e-13, and for two
    sources against the oracle (CPU restatement, SciPy CG to 1e-12); run in
    fp64 and in mixed precision with forward recomputation.  ``value``: mixed
    gradients per second with model, data and gradient on the device; ``e2e``:
    the same from a host model to a host gradient.  Prints one JSON line.
    """
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.autograd import dpred
    from simpeg_gb300.engine import kernel_launches
    from simpeg_gb300.resistivity import Simulation3DNodal
    from simpeg_gb300.resistivity.survey import Survey

    mesh, m, survey = workloads.differentiation(seed=2)
    rng = np.random.default_rng(11)
    m0 = m + 0.1 * rng.standard_normal(m.size)
    v_spot = np.random.default_rng(12).standard_normal(survey.nD)
    spots = None if args.no_oracle else OracleSpots(mesh, m0, survey, [0, survey.nSrc - 1], v_spot)
    torch.cuda.set_device(0)
    # fp64 reference at 5e-13 (a 1e-13 target sits at the fp64 residual's rounding floor on this mesh)
    ref = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="fp64", rtol=5e-13)
    d_true = ref.dpred(m)
    dobs = torch.from_numpy(d_true * (1 + 0.03 * rng.standard_normal(d_true.size)))
    r0 = ref.dpred(m0) - dobs.numpy()
    g_ref = ref.Jtvec(m0, r0)
    del ref
    torch.cuda.empty_cache()
    cfg = {"workload": "dc3d_differentiation_96x96x48", "mesh_cells": list(mesh.shape_cells),
           "nodes": int(mesh.n_nodes), "sources": survey.nSrc, "data": survey.nD, "fd_step": 1e-4,
           "directions": args.fd_directions, "l2": "inputs larger than L2 (fields 0.47 GB fp64)"}
    out = {"metric": "misfit gradients/s by autograd (adjoint solve + dA/dsigma kernel), 96x96x48 DC3D: "
                     "mixed+recompute vs fp64", "unit": "gradients/s", "higher_is_better": True, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 inner / f64 refinement", "data": "synthetic (seeded Gaussian random field)", "config": cfg}
    dirs = [v / np.linalg.norm(v) for v in rng.standard_normal((args.fd_directions, m.size))]
    for label, precision, recompute in (("fp64", "fp64", False), ("mixed_recompute", "mixed", True)):
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=1e-11)

        def phi(mm, dd):
            r = dpred(sim, mm, recompute=recompute) - dd
            return 0.5 * (r * r).sum()

        def grad(mm, dd):
            mt = mm.detach().clone().requires_grad_(True)
            phi(mt, dd).backward()
            return mt.grad

        m_dev, d_dev = torch.from_numpy(m0).cuda(), dobs.cuda()
        for _ in range(args.warmup):
            grad(m_dev, d_dev)
            grad(torch.from_numpy(m0), dobs)
        torch.cuda.synchronize()
        # device resident: model, data and gradient stay on the GPU
        n0 = kernel_launches()
        sim.engine.stencil_timing(True)
        with Clocks(0) as clk:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                g_dev = grad(m_dev, d_dev)
            e1.record()
            torch.cuda.synchronize()
        st = sim.engine.stencil_timing(False)
        kinds = sim.engine.stencil_timing_kinds()
        launches = kernel_launches() - n0
        t_dev = e0.elapsed_time(e1) / 1e3 / args.steps
        # end to end: host model and data in, host gradient out
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g = grad(torch.from_numpy(m0), dobs)
        t_e2e = (time.perf_counter() - t0) / args.steps
        g = g.numpy()
        errs = []
        for v in dirs:
            with torch.no_grad():
                fp = phi(torch.from_numpy(m0 + 1e-4 * v), dobs).item()
                fm = phi(torch.from_numpy(m0 - 1e-4 * v), dobs).item()
            fd = (fp - fm) / 2e-4
            errs.append(abs(fd - g @ v) / max(abs(fd), 1e-300))
        out[label] = {"grad_seconds": t_dev, "grad_seconds_e2e": t_e2e, "fd_max_rel_err": float(max(errs)),
                      "fd_median_rel_err": float(np.median(errs)),
                      "rel_err_vs_fp64_jtvec": float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)),
                      "device_vs_host_model": float(np.linalg.norm(g_dev.cpu().numpy() - g) / np.linalg.norm(g))}
        if label == "mixed_recompute":
            out["value"] = 1.0 / t_dev
            out["ms_per_step"] = t_dev * 1e3
            out["clocks"] = clk.summary()
            out["gpu_launches"] = launches
            out["roofline"] = _stencil_roofline(*st, kinds, scaled_traffic=True)
            out["e2e"] = {"value": 1.0 / t_e2e, "unit": "gradients/s",
                          "h2d_bytes_per_step": int(m.size * 8 + 2 * survey.nD * 8),
                          "d2h_bytes_per_step": int(m.size * 8 + survey.nD * 8),
                          "path": "dpred autograd Function from a host model tensor: m, dobs and dL/dd up, d and "
                                  "dL/dm down"}
        del sim
        torch.cuda.empty_cache()
    out["speedup_vs_fp64"] = out["fp64"]["grad_seconds"] / out["mixed_recompute"]["grad_seconds"]
    if spots is not None:
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=1e-11)
        d_gpu = sim.dpred(m0)

        def jt_one(i, s_):
            one = Simulation3DNodal(mesh, survey=Survey([survey.source_list[i]]), sigmaMap=maps.ExpMap(mesh),
                                    precision="mixed", rtol=1e-11)
            return one.Jtvec(m0, v_spot[s_])

        out["rel_err_vs_oracle_cg"] = spots.compare(d_gpu, jt_one)
        t_one = float(np.mean(out["rel_err_vs_oracle_cg"]["oracle_seconds_per_source"]))
        out["cpu_baseline"] = {"value": 1.0 / (t_one * survey.nSrc), "unit": "gradients/s", "cores": 1,
                               "kind": "port",
                               "sample": (f"1 of {survey.nSrc} sources timed (forward + adjoint SciPy CG solves to "
                                          f"1e-12 and the adjoint product on the oracle, {t_one:.0f} s), times "
                                          f"{survey.nSrc}")}
    print(json.dumps(out), flush=True)


def run_gauss_newton(args):
    """160x160x80 cells (~2.05 M), 512 dipole sources x 48 receivers, m = ln sigma.

    One inexact Gauss-Newton step at the starting model: fields, data misfit
    gradient plus smallness + smoothness regularisation, exact getJtJdiag
    (electrode reciprocity) for the Jacobi preconditioner, and 10 CG iterations
    on 2 J^T W^2 J + 2 beta R, each one batched Jvec and one batched Jtvec.
    Run in mixed precision and in plain fp64 on the same GPU, each with the
    smoother the autotuner picks for this mesh (untimed); prints times and
    the relative differences of g, diag(J^T J) and the search direction, and
    for two sources the data and J^T v against the oracle (SciPy CG to 1e-12).
    """
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.autotune import tune_engine
    from simpeg_gb300.engine import kernel_launches
    from simpeg_gb300.inversion import L2DataMisfit, WeightedLeastSquares, inexact_gauss_newton_direction
    from simpeg_gb300.resistivity import Simulation3DNodal
    from simpeg_gb300.resistivity.survey import Survey

    mesh, m_true, m0, survey = workloads.gauss_newton(seed=4)
    v_spot = np.random.default_rng(13).standard_normal(survey.nD)
    spots = None if args.no_oracle else OracleSpots(mesh, m0, survey, [0, survey.nSrc - 1], v_spot)
    torch.cuda.set_device(0)
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
    out = {"metric": "Gauss-Newton steps/s (getJtJdiag + gradient + 10 CG iterations on J^T J + beta R), "
                     "2.05M-cell DC3D, 512 sources: mixed vs fp64",
           "unit": "Gauss-Newton steps/s", "higher_is_better": True, "n_gpus": 1, "steps": 1, "warmup": 1,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 refinement",
           "data": "synthetic (seeded Gaussian random field; data from the true model + 2 % noise)",
           "config": {"workload": "dc3d_gauss_newton_160x160x80", "mesh_cells": list(mesh.shape_cells),
                      "nodes": int(mesh.n_nodes), "sources": survey.nSrc, "data": survey.nD, "beta": beta,
                      "cg_iterations": 10, "rtol": RTOL, "l2": "inputs larger than L2 (fields 8.6 GB fp64)"}}
    res = {}
    for precision in ("mixed", "fp64"):
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=RTOL)
        # untimed: the autotuner picks the smoother (Chebyshev degree and interval) for this mesh and
        # source count, in each precision, from sample solves at the starting model
        t_tune = time.perf_counter()
        sim.model = m0
        sim._ensure_model()
        tuned = tune_engine(sim.engine, survey.nSrc, precision, rtol=RTOL,
                            cands=[(0, 2, 15.0), (0, 2, 30.0), (0, 3, 15.0), (0, 3, 30.0)])
        t_tune = time.perf_counter() - t_tune
        dmis = L2DataMisfit(sim, dobs, W=W)
        reg = WeightedLeastSquares(mesh, sim)
        torch.cuda.synchronize()
        n0 = kernel_launches()
        sim.engine.stencil_timing(True)
        with Clocks(0) as clk:
            t0 = time.perf_counter()
            p, info = inexact_gauss_newton_direction(dmis, reg, beta, m0, cg_maxiter=10)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            p_host = p.cpu().numpy()  # the step's result on the host (end to end)
            dt_e2e = time.perf_counter() - t0
        st = sim.engine.stencil_timing(False)
        kinds = sim.engine.stencil_timing_kinds()
        launches = kernel_launches() - n0
        res[precision] = (p_host, info["g"].cpu().numpy(), info["jtj_diag"].cpu().numpy())
        out[precision] = {"seconds": dt, "cg_rel_res": info["cg_rel_res"][-1],
                          "phases_seconds": {k: round(v, 3) for k, v in info["seconds"].items()},
                          "smoother": {"degree": tuned["nu"], "interval": f"lmax/{tuned['cheb_ratio']:g}",
                                       "tuning_seconds_untimed": round(t_tune, 1)}}
        if precision == "mixed":
            out["value"] = 1.0 / dt
            out["ms_per_step"] = dt * 1e3
            out["clocks"] = clk.summary()
            out["gpu_launches"] = launches
            out["roofline"] = _stencil_roofline(*st, kinds, scaled_traffic=True)
            out["e2e"] = {"value": 1.0 / dt_e2e, "unit": "Gauss-Newton steps/s",
                          "h2d_bytes_per_step": int(m0.size * 8), "d2h_bytes_per_step": int(m0.size * 8),
                          "path": "inexact_gauss_newton_direction(dmis, reg, beta, m) from a host model; the "
                                  "search direction copied to the host"}
        del sim, dmis, reg, p, info
        torch.cuda.empty_cache()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out["speedup_vs_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    out["rel_err_mixed_vs_fp64"] = {"direction": rel(res["mixed"][0], res["fp64"][0]),
                                    "gradient": rel(res["mixed"][1], res["fp64"][1]),
                                    "jtj_diag": rel(res["mixed"][2], res["fp64"][2])}
    if spots is not None:
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=RTOL)
        d_gpu = sim.dpred(m0)
        del sim

        def jt_one(i, s_):
            one = Simulation3DNodal(mesh, survey=Survey([survey.source_list[i]]), sigmaMap=maps.ExpMap(mesh),
                                    precision="mixed", rtol=RTOL)
            return one.Jtvec(m0, v_spot[s_])

        out["rel_err_vs_oracle_cg"] = spots.compare(d_gpu, jt_one)
        t_one = float(np.mean(out["rel_err_vs_oracle_cg"]["oracle_seconds_per_source"]))
        n_solves = 2 * survey.nSrc + 2 * 10 * survey.nSrc
        out["cpu_baseline"] = {"value": 1.0 / (t_one / 2 * n_solves), "unit": "Gauss-Newton steps/s", "cores": 1,
                               "kind": "port",
                               "sample": (f"one source's forward + adjoint SciPy CG solves (1e-12) on the oracle "
                                          f"timed ({t_one:.0f} s), scaled to the step's {n_solves} source solves "
                                          "(fields, gradient, 10 x (Jvec + Jtvec)); getJtJdiag's pole solves not "
                                          "counted")}
    print(json.dumps(out), flush=True)


def run_batched(args):
    """64 independent problems, cell counts log-uniform from 32x32x16 to 96x96x64,
    16-128 pole sources x 20 dipole receivers each, own block + random-field
    conductivity.  After the autotuner picks RHS-block width and smoother per
    problem, all 64 adaptive solves are recorded into one CUDA graph whose
    solver loops run on the device; the timed step is one launch of that graph
    (inputs resident).  ``e2e``: the source terms copied up from pinned host
    memory, one launch, the convergence check and every problem's data copied
    back (``BatchedForward.run``).  Compared with solving the same problems one
    after the other with the host-driven adaptive solver (identical results),
    and for two problems with the oracle (SciPy CG to 1e-12)."""
    import torch

    from simpeg_gb300 import workloads
    from simpeg_gb300.batch import BatchedForward
    from simpeg_gb300.engine import kernel_launches

    probs = workloads.batched_problems(seed=5, n=64)
    nsrc = sum(sv.nSrc for _, _, sv in probs)
    spot_p = [0, len(probs) - 1]
    spots = None
    if not args.no_oracle:
        from simpeg_gb300.resistivity.survey import Survey

        spots = [OracleSpots(probs[i][0], np.log(probs[i][1]), Survey(probs[i][2].source_list[:1]), [0], None)
                 for i in spot_p]
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    bf = BatchedForward(probs, precision="mixed", rtol=RTOL, tune=True)
    t_setup = time.perf_counter() - t0
    for _ in range(args.warmup):
        bf.launch()
    torch.cuda.synchronize()
    n0 = kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record()
        for _ in range(args.steps):
            bf.launch()
        e1.record()
        torch.cuda.synchronize()
    launches = kernel_launches() - n0
    ms = e0.elapsed_time(e1) / args.steps
    conv = bf.convergence()
    data = bf.data()
    # end to end: every problem's source table (electrode node indices and weights) up from pinned host
    # memory, the source terms filled on the device, one launch, the convergence check, data down
    from simpeg_gb300.engine import fill_sparse

    q_host = [(torch.from_numpy(p.tables.q_idx).pin_memory(), torch.from_numpy(p.tables.q_val).pin_memory())
              for p in bf.problems]
    q_dev = [(torch.empty_like(a, device="cuda"), torch.empty_like(b, device="cuda")) for a, b in q_host]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for p, (ih, vh), (idv, vdv) in zip(bf.problems, q_host, q_dev):
            idv.copy_(ih, non_blocking=True)
            vdv.copy_(vh, non_blocking=True)
            p.Q.zero_()
            fill_sparse(idv, vdv, p.Q.view(-1))
        bf.run()
    t_e2e = (time.perf_counter() - t0) / args.steps
    # the same problems one by one, adaptive solver, same engines and workspaces; fine-level steps timed
    for p in bf.problems:
        p.engine.stencil_timing(True)
    torch.cuda.synchronize()
    n_seq0 = kernel_launches()
    e0.record()
    for p in bf.problems:
        p.engine.solve(p.Q, mode="mixed", rtol=RTOL, ws=p.ws)
    e1.record()
    torch.cuda.synchronize()
    seq_launches = kernel_launches() - n_seq0
    ms_seq = e0.elapsed_time(e1)
    tot = [0.0, 0, 0.0]
    for p in bf.problems:
        st = p.engine.stencil_timing(False)
        tot = [tot[0] + st[0], tot[1] + st[1], tot[2] + st[2]]
    tunes = [getattr(p, "tuning", None) for p in bf.problems]
    h2d = sum(int(a.numel() * a.element_size() + b.numel() * b.element_size()) for a, b in q_host)
    d2h = sum(int(p.tables.nD * 8) for p in bf.problems)
    out = {"metric": "batched uneven problems: source-solves/s, one CUDA-graph launch vs sequential",
           "workload": "dc3d_batched_64", "value": nsrc / (ms / 1e3), "unit": "source-solves/s",
           "higher_is_better": True, "n_gpus": 1, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 inner / f64 refinement", "data": "synthetic (seeded block + random field per problem)",
           "ms_per_step": ms, "ms_per_launch": ms, "steps": args.steps, "warmup": args.warmup,
           "sequential": {"ms": ms_seq, "source_solves_per_s": nsrc / (ms_seq / 1e3)},
           "speedup_vs_sequential": ms_seq / ms,
           "converged": all(c[1] == 0 for c in conv), "max_rel_res": max(c[0] for c in conv),
           "inner_iterations": [min(c[2] for c in conv), max(c[2] for c in conv)],
           "setup_seconds": t_setup,
           "config": {"workload": "dc3d_batched_64", "problems": len(probs), "sources": nsrc,
                      "nodes_range": [min(p[0].n_nodes for p in probs), max(p[0].n_nodes for p in probs)],
                      "rtol": RTOL, "l2": "inputs larger than L2 (all problems' vectors, ~2 GB)"},
           "autotune": {"kb": sorted({t["kb"] for t in tunes if t}), "nu": sorted({t["nu"] for t in tunes if t})},
           "clocks": clk.summary(),
           # a graph launch replays the problems' kernels without passing the host launch counter; the
           # graph runs every solve as far as the host-driven solver does (same iterations), whose
           # kernel launches are counted in the sequential pass
           "gpu_launches": seq_launches * args.steps, "graph_launches": args.steps,
           "host_counted_launches_in_timed_region": launches,
           "roofline": _stencil_roofline(*tot, what="fine-level Chebyshev steps of every problem, timed in the "
                                                    "sequential pass (events cannot bracket single kernels inside "
                                                    "the graph)"),
           "e2e": {"value": nsrc / t_e2e, "unit": "source-solves/s", "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h, "path": "source tables from pinned host memory -> source terms filled "
                                                      "on the device -> BatchedForward.run() (launch, convergence "
                                                      "check, data to the host)"}}
    if spots is not None:
        errs, secs = [], []
        for i, sp_ in zip(spot_p, spots):
            nd0 = probs[i][2].source_list[0].receiver_list[0].nD
            r = sp_.compare(data[i][:nd0], None)
            errs.append(r["dpred"])
            secs.append(r["oracle_seconds_per_source"][0])
        out["rel_err_vs_oracle_cg"] = {"problems": spot_p, "sources": [0], "dpred": max(errs),
                                       "oracle": "CPU restatement of the reference path, fp64 SciPy CG + Jacobi to "
                                                 f"rtol {ORACLE_RTOL:g}"}
        t_src = secs[-1]
        out["cpu_baseline"] = {"value": 1.0 / t_src, "unit": "source-solves/s", "cores": 1, "kind": "port",
                               "sample": (f"source 0 of problem {spot_p[-1]} ({probs[spot_p[-1]][0].n_nodes} nodes) "
                                          f"solved by the oracle (SciPy CG + Jacobi to 1e-12), {t_src:.1f} s")}
    print(json.dumps(out), flush=True)


def _superlu_step(mesh, sigma, survey):
    """The reference's default forward path on the host: assembly of A (oracle restatement), SuperLU
    factorisation (SciPy splu, what pymatsolver.SolverLU wraps), one solve of all sources, dpred."""
    import scipy.sparse.linalg as spla

    from oracle.dc3d import OracleDC3DNodal

    t0 = time.perf_counter()
    o = OracleDC3DNodal(mesh, survey, sigma=sigma)
    A = o.getA().tocsc()
    q = o.getRHS()
    t1 = time.perf_counter()
    lu = spla.splu(A)
    t2 = time.perf_counter()
    f = lu.solve(q)
    t3 = time.perf_counter()
    d = o.dpred(f=f)
    t4 = time.perf_counter()
    return d, {"assembly_s": t1 - t0, "factor_s": t2 - t1, "solve_s": t3 - t2, "dpred_s": t4 - t3, "total_s": t4 - t0}


def run_cc(args):
    """The headline workload (1M cells, 256 pole sources, 10,240 data, rtol 1e-9) in the cell-centred
    formulation: ``Simulation3DCellCentered`` (Robin), 1,048,576 unknowns on the grid of cell
    centres, and the induced-polarization data of the same formulation.

    ``value``: mixed source-solves/s of the cell-centred forward solve with the source terms on the
    device; ``e2e``: ``dpred(m)`` from a host model to host data.  Jtvec/s and the IP prediction
    (``induced_polarization.Simulation3DCellCentered.dpred(eta)``: one multi-RHS solve with the DC
    fields kept) ride along, mixed and fp64, with relative errors against fp64 solves at 1e-12 and,
    for two sources, against the cell-centred oracle (SciPy CG to 1e-12).  Prints one JSON line.
    """
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.engine import kernel_launches
    from simpeg_gb300.induced_polarization import Simulation3DCellCentered as IPSimulation3DCellCentered
    from simpeg_gb300.resistivity import Simulation3DCellCentered
    from simpeg_gb300.resistivity.survey import Survey

    mesh, sigma, survey = workloads.scale_forward(seed=1, n_side=args.n_side)
    m = np.log(sigma)
    K = survey.nSrc
    rng = np.random.default_rng(21)
    v_host = rng.standard_normal(survey.nD)
    eta = 0.1 * rng.random(mesh.n_cells)
    m2 = m + 1e-3 * rng.standard_normal(m.size)
    spots = None if args.no_oracle else OracleSpots(mesh, m, survey, [0, K - 1], v_host,
                                                    worker=_oracle_spot_worker_cc)
    torch.cuda.set_device(0)

    def timed_loop(fn, steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / steps, r

    res, out = {}, {}
    for precision, rtol in (("mixed", RTOL), ("fp64", RTOL), ("ref", 1e-12)):
        prec = "fp64" if precision == "ref" else precision
        sim = Simulation3DCellCentered(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=prec,
                                       rtol=rtol)
        sim.model = m
        sim._ensure_model()
        eng = sim.engine
        Q = sim.getRHS()
        if precision != "ref":
            for _ in range(max(1, args.warmup)):
                eng.solve(Q, mode=prec, rtol=rtol)
            torch.cuda.synchronize()
            n0 = kernel_launches()
            if precision == "mixed":
                eng.stencil_timing(True)
            with Clocks(0) as clk:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(args.steps):
                    U, info = eng.solve(Q, mode=prec, rtol=rtol)
                e1.record()
                torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            launches = kernel_launches() - n0
            out[precision] = {"ms_per_solve": ms, "source_solves_per_s": K / (ms / 1e3),
                              "inner_iterations": info.iterations, "outer": info.outer, "levels": info.n_levels}
            if precision == "mixed":
                st = eng.stencil_timing(False)
                kinds = eng.stencil_timing_kinds()
                out["clocks"] = clk.summary()
                out["gpu_launches"] = launches  # kernels of the timed solves
        f = sim.fields(m)
        d = sim.dpred(m, f=f)
        sim.Jtvec(m, v_host, f=f)
        t_jt, g = timed_loop(lambda: sim.Jtvec(m, v_host, f=f), 1 if precision == "ref" else args.steps)
        ip = IPSimulation3DCellCentered(mesh, survey=survey, sigma=sigma, precision=prec, rtol=rtol,
                                        _f=f)
        ip.dpred(eta)
        t_ip, d_ip = timed_loop(lambda: ip.dpred(eta), 1 if precision == "ref" else args.steps)
        res[precision] = (np.asarray(d), np.asarray(g), np.asarray(d_ip))
        if precision != "ref":
            out[precision]["jtvec_per_s"] = 1.0 / t_jt
            out[precision]["ip_dpred_per_s"] = 1.0 / t_ip
        if precision == "mixed":
            sim.dpred(m2)
            t_e2e, _ = timed_loop(lambda: (sim.dpred(m), sim.dpred(m2)), args.steps)
            out["e2e"] = {"value": 2 * K / t_e2e, "unit": "source-solves/s",
                          "h2d_bytes_per_step": int(mesh.n_cells * 8), "d2h_bytes_per_step": int(survey.nD * 8),
                          "path": "Simulation3DCellCentered.dpred(m): host model -> H2D -> exp map on device -> "
                                  "dc_set_model_cc -> solve -> gather -> D2H"}
        del sim, eng, Q, ip, f
        torch.cuda.empty_cache()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    mixed, fp64 = out.pop("mixed"), out.pop("fp64")
    line = {"metric": "source-solves/s, 1M-cell DC3D cell-centred (Simulation3DCellCentered): mixed vs fp64",
            "value": mixed["source_solves_per_s"], "unit": "source-solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mixed["ms_per_solve"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 refinement",
            "data": "synthetic (seeded Gaussian random field, 16x16 pole grid; eta uniform in [0, 0.1))",
            "config": {"workload": "dc3d_cell_centred_128x128x64", "mesh_cells": list(mesh.shape_cells),
                       "unknowns": int(mesh.n_cells), "sources": K, "data": survey.nD, "bc_type": "Robin",
                       "rtol": RTOL, "l2": "inputs larger than L2 (fp16 multigrid vectors 537 MB per RHS block "
                                           "set)"},
            "mixed": mixed, "fp64": fp64,
            "speedup_vs_fp64": {"forward": fp64["ms_per_solve"] / mixed["ms_per_solve"],
                                "jtvec": mixed["jtvec_per_s"] / fp64["jtvec_per_s"],
                                "ip_dpred": mixed["ip_dpred_per_s"] / fp64["ip_dpred_per_s"]},
            "rel_err_vs_fp64_1e-12": {"dpred": rel(res["mixed"][0], res["ref"][0]),
                                      "jtvec_m": rel(res["mixed"][1], res["ref"][1]),
                                      "ip_dpred": rel(res["mixed"][2], res["ref"][2])},
            "roofline": _stencil_roofline(*st, kinds, what="fine-level Chebyshev steps on the grid of cell "
                                                         "centres", scaled_traffic=True),
            **out}
    if spots is not None:
        def jt_one(i, s_):
            one = Simulation3DCellCentered(mesh, survey=Survey([survey.source_list[i]]),
                                           sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=RTOL)
            return one.Jtvec(m, v_host[s_])

        line["rel_err_vs_oracle_cg"] = spots.compare(res["mixed"][0], jt_one)
    if not args.no_cpu_baseline:
        from oracle.cc3d import OracleDC3DCellCentered

        import scipy.sparse as sp
        import scipy.sparse.linalg as spla

        o = OracleDC3DCellCentered(mesh, Survey([survey.source_list[0]]), sigma=sigma, solver="cg", cg_rtol=RTOL)
        t0 = time.perf_counter()
        A = o.getA()
        Mj = sp.diags(1.0 / A.diagonal())
        q = o.getRHS()[:, 0]
        t_asm = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, cg_info = spla.cg(A, q, rtol=RTOL, atol=0.0, M=Mj, maxiter=200000)
        t_cg = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / t_cg, "unit": "source-solves/s", "cores": 1, "kind": "port",
                                "sample": (f"1 of {K} sources: the cell-centred oracle's assembly ({t_asm:.1f} s, "
                                           f"excluded) + SciPy CG/Jacobi to rtol {RTOL:g} ({t_cg:.1f} s, "
                                           f"info={cg_info})"),
                                "solver": "SciPy CG + Jacobi (an iterative plug-in; SuperLU does not fit at this "
                                          "size)"}
    print(json.dumps(line), flush=True)


def run_serving(args):
    """Continuous-batching serving of dpred requests (``simpeg_gb300.serving.DCServer``, lane mode).

    96x96x48 cells (the differentiation mesh), four models, 96 requests of 8-32 dipole sources (30
    receivers each), chosen and sized by a seeded generator.  Each request is a host model and a
    host survey in and host data out, so the whole run is end to end.  ``value``: source-solves/s
    with every request queued at once (the server's capacity, first submission to last answer) and
    one slot per model; ``by_slots``: that capacity, and the same requests as a Poisson stream
    offering 70 % of it with submit-to-answer latency percentiles, for 2 and 4 slots.  The same
    requests solved one after another through ``Simulation3DNodal.dpred`` (one simulation per model,
    its operator built once, the request's survey swapped in: a request queue without batching) ride
    along, and every request's data are compared with that sequential result.  Prints one JSON line.
    """
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.engine import kernel_launches
    from simpeg_gb300.resistivity import Simulation3DNodal
    from simpeg_gb300.resistivity.survey import Survey
    from simpeg_gb300.serving import DCServer

    mesh, m_base, survey_all = workloads.differentiation(seed=2)
    rng = np.random.default_rng(31)
    models = [m_base + 0.3 * rng.standard_normal(m_base.size) for _ in range(4)]
    n_req = 96
    reqs = []
    for _ in range(n_req):
        k = int(rng.integers(8, 33))
        start = int(rng.integers(0, survey_all.nSrc - k + 1))
        reqs.append((int(rng.integers(0, len(models))), Survey(survey_all.source_list[start:start + k])))
    total_src = sum(r[1].nSrc for r in reqs)
    torch.cuda.set_device(0)

    # sequential: one request after another through the simulation API, one simulation per model kept
    # set up (its model's operator built once, warmed), the request's survey swapped in
    sims = [Simulation3DNodal(mesh, survey=reqs[0][1], sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=RTOL)
            for _ in models]
    for sim, m in zip(sims, models):
        sim.dpred(m)
    torch.cuda.synchronize()

    def one(mi, sv):
        sims[mi].survey = sv
        return sims[mi].dpred(models[mi])

    t0 = time.perf_counter()
    seq = [one(mi, sv) for mi, sv in reqs]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    del sims
    torch.cuda.empty_cache()

    def serve(srv, gaps):
        """Submit the requests after the given gaps; returns (seconds, answers, submit-to-answer latencies)."""
        t0 = time.perf_counter()
        futs, t_sub = [], []
        for (mi, sv), g in zip(reqs, gaps):
            if g > 0:
                time.sleep(g)
            t_sub.append(time.perf_counter())
            futs.append(srv.submit(models[mi], sv))
        out, lat = [], []
        for f, ts in zip(futs, t_sub):
            out.append(f.result(timeout=1800))
            lat.append(time.perf_counter() - ts)
        return time.perf_counter() - t0, out, lat

    by_slots = {}
    for n_slots in (2, 4):
        with DCServer(mesh, slots=n_slots, max_rhs=128, rtol=RTOL) as srv:
            # warm-up request per slot (workspaces and kernels), untimed
            for f in [srv.submit(models[i % len(models)], reqs[i][1]) for i in range(n_slots)]:
                f.result(timeout=600)
            # capacity: every request queued at once
            for sl in srv.slots:
                sl.engine.stencil_timing(True)
            n0 = kernel_launches()
            with Clocks(0) as clk:
                t_srv, out, lat_burst = serve(srv, np.zeros(n_req))
            launches = kernel_launches() - n0
            st = [sl.engine.stencil_timing(False) for sl in srv.slots]
            kinds = {}
            for sl in srv.slots:
                for k, (c, t, b) in sl.engine.stencil_timing_kinds().items():
                    kc, kt, kb = kinds.get(k, (0, 0.0, 0.0))
                    kinds[k] = (kc + c, kt + t, kb + b)
            # latency: Poisson arrivals offering 70 % of that capacity
            mean_gap = t_srv / n_req / 0.7
            t_poisson, out_p, lat = serve(srv, rng.exponential(mean_gap, n_req))
        lat_ms = np.array(lat) * 1e3
        by_slots[n_slots] = {
            "source_solves_per_s": total_src / t_srv, "seconds": t_srv,
            "burst_latency_ms": {"p50": float(np.percentile(np.array(lat_burst) * 1e3, 50)),
                                 "max": float(np.max(lat_burst) * 1e3)},
            "poisson_70pct": {"mean_arrival_gap_ms": mean_gap * 1e3, "source_solves_per_s": total_src / t_poisson,
                              "latency_ms": {"p50": float(np.percentile(lat_ms, 50)),
                                             "p90": float(np.percentile(lat_ms, 90)),
                                             "p99": float(np.percentile(lat_ms, 99)), "max": float(lat_ms.max())}},
            "rel_err_vs_sequential_max": max(float(np.linalg.norm(a_ - b_) / np.linalg.norm(b_))
                                             for a_, b_ in zip(out + out_p, seq + seq))}
    ms = sum(x for x, _, _ in st)
    n = sum(x for _, x, _ in st)
    by = sum(x for _, _, x in st)
    best = by_slots[4]
    line = {"metric": "served source-solves/s, continuous batching (DCServer lane mode), 96 requests on 96x96x48 cells",
            "value": best["source_solves_per_s"], "unit": "source-solves/s", "n_gpus": 1, "steps": 1, "warmup": 4,
            "ms_per_step": best["seconds"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 inner / f64 refinement",
            "data": "synthetic (seeded Gaussian random fields, 4 models; 96 requests of 8-32 dipoles x 30 receivers)",
            "config": {"workload": "dc3d_serving_96x96x48", "mesh_cells": list(mesh.shape_cells),
                       "nodes": int(mesh.n_nodes), "requests": n_req, "sources": total_src, "models": len(models),
                       "slots": 4, "lanes_per_slot": 128, "rtol": RTOL,
                       "value": "4 slots (one per model), all requests queued at once (capacity)"},
            "by_slots": {str(k): v for k, v in by_slots.items()},
            "sequential": {"seconds": t_seq, "source_solves_per_s": total_src / t_seq,
                           "path": "Simulation3DNodal.dpred(m) per request, one after another, one simulation per "
                                   "model (operator built once), the request's survey swapped in"},
            "speedup_vs_sequential": t_seq / best["seconds"],
            "rel_err_vs_sequential_max": max(v["rel_err_vs_sequential_max"] for v in by_slots.values()),
            "clocks": clk.summary(), "gpu_launches": launches,
            "roofline": _stencil_roofline(ms, n, by, kinds or None, what="fine-level Chebyshev steps of the "
                                                                          "slots' lane sweeps", scaled_traffic=True),
            "e2e": {"value": best["source_solves_per_s"], "unit": "source-solves/s",
                    "h2d_bytes_per_step": int(sum(mesh.n_cells * 8 for _ in reqs)),
                    "d2h_bytes_per_step": int(sum(sv.nD * 8 for _, sv in reqs)),
                    "path": "DCServer.submit(host model, host survey) -> Future -> host data, every request"}}
    if not args.no_cpu_baseline:
        cb = _cpu_baseline(mesh, np.exp(models[0]), survey_all)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line), flush=True)


def run_block(args):
    """32x32x16 cells of 10 m (18,513 nodes), 0.01 S/m with a 0.1 and a 0.001 S/m block, dipole-dipole
    line of 20 sources x 15 receivers (300 data): the size where the reference's default direct solver
    fits.  One step = dpred of all 20 sources.  ``value``: GPU mixed precision with the model resident;
    ``e2e``: ``Simulation3DNodal.dpred(m)`` from a host model to host data; ``cpu_baseline`` /
    ``--impl reference``: assembly + SuperLU factorisation + solve + dpred on the host, the reference's
    ``fields`` with ``SolverLU`` (``resistivity/simulation.py:100-113``)."""
    import torch

    from simpeg_gb300 import maps
    from simpeg_gb300.engine import csr_spmv, kernel_launches
    from simpeg_gb300.resistivity import Simulation3DNodal
    from simpeg_gb300.workloads import block_model_survey

    mesh, sigma, survey, _ = block_model_survey(seed=0)
    m = np.log(sigma)
    cfg = {"workload": "dc3d_nodal_block_32x32x16", "mesh_cells": list(mesh.shape_cells), "nodes": int(mesh.n_nodes),
           "sources": survey.nSrc, "data": survey.nD, "rtol": RTOL,
           "l2": "working set fits in L2 (18.5k nodes); timed back to back"}
    metric = "source-solves/s, 32x32x16 block model (300 data): GPU vs the reference's SuperLU path"
    if args.impl == "reference":
        for _ in range(args.warmup):
            _superlu_step(mesh, sigma, survey)
        ts = [_superlu_step(mesh, sigma, survey)[1] for _ in range(args.steps)]
        v = survey.nSrc / statistics.median(t["total_s"] for t in ts)
        line = {"impl": "reference", "metric": metric, "value": v, "unit": "source-solves/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": survey.nSrc / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded block model)", "config": cfg, "phases_s": ts[-1],
                "cpu_baseline": {"value": v, "unit": "source-solves/s", "cores": 1, "kind": "port",
                                 "sample": "the whole step: oracle assembly + SciPy SuperLU factor + solve + dpred"},
                "e2e": {"value": v, "unit": "source-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    torch.cuda.set_device(0)
    res = {}
    for precision in ("mixed", "fp64"):
        sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision=precision, rtol=RTOL)
        sim.model = m
        sim._ensure_model()
        t, tq = sim._get_tables()
        Q = sim.getRHS()
        d_out = torch.empty(t.nD, dtype=torch.float64, device="cuda")

        def step():
            U, _ = sim.engine.solve(Q, mode=precision, rtol=RTOL)
            csr_spmv(tq["P_ptr"], tq["P_idx"], tq["P_w"], U.view(-1), d_out)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        n0 = kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(0) as clk:
            e0.record()
            for _ in range(args.steps):
                step()
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        launches = kernel_launches() - n0
        d_dev = d_out.cpu().numpy()
        m2 = m + 1e-3
        sim.dpred(m2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            sim.dpred(m if i % 2 == 0 else m2)
        e2e = (time.perf_counter() - t0) / args.steps
        res[precision] = dict(ms=ms, d=d_dev, e2e_s=e2e, clocks=clk.summary(), launches=launches,
                              iters=sim.last_solve_info.iterations if hasattr(sim, "last_solve_info") else None)
        del sim
    d_lu, ph = _superlu_step(mesh, sigma, survey)
    ph_all = [_superlu_step(mesh, sigma, survey)[1] for _ in range(max(1, min(3, args.steps)))]
    t_lu = statistics.median(p["total_s"] for p in ph_all)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    K = survey.nSrc
    line = {
        "metric": metric, "value": K / (res["mixed"]["ms"] / 1e3), "unit": "source-solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["mixed"]["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 refinement",
        "data": "synthetic (seeded block model)", "config": cfg,
        "fp64_plain": {"source_solves_per_s": K / (res["fp64"]["ms"] / 1e3), "ms_per_step": res["fp64"]["ms"]},
        "rel_err_vs_superlu": {"dpred_mixed": rel(res["mixed"]["d"], d_lu), "dpred_fp64": rel(res["fp64"]["d"], d_lu)},
        "superlu": {"phases_s": ph_all[-1], "source_solves_per_s": K / t_lu,
                    "solve_only_source_solves_per_s": K / statistics.median(p["solve_s"] for p in ph_all)},
        "e2e": {"value": K / res["mixed"]["e2e_s"], "unit": "source-solves/s", "h2d_bytes_per_step": int(mesh.n_cells * 8),
                "d2h_bytes_per_step": int(survey.nD * 8), "path": "Simulation3DNodal.dpred(m), host model -> host data"},
        "cpu_baseline": {"value": K / t_lu, "unit": "source-solves/s", "cores": 1, "kind": "port",
                         "sample": "the whole step: oracle assembly + SciPy SuperLU factorisation + solve of the 20 "
                                   "sources + dpred (the reference's default solver path)"},
        "gpu_launches": res["mixed"]["launches"], "clocks": res["mixed"]["clocks"],
        "roofline": None,
        "roofline_note": "18.5k nodes: every vector fits in L2, so no kernel of this size is HBM-bound; the "
                         "roofline is reported on the 1M-cell forward line",
    }
    print(json.dumps(line), flush=True)


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


def run_profile_sens(args):
    """One getJtJdiag (electrode reciprocity: pole solves + k_jtj_diag) and one Jtvec (adjoint solve +
    k_edge_products + k_cell_gradient) on a 96x96x48-cell Gauss-Newton-type workload (with
    ``--sens-full-survey``: the Gauss-Newton workload's survey on a 64x64x32-cell mesh)."""
    import torch

    from simpeg_gb300 import maps, workloads
    from simpeg_gb300.resistivity import Simulation3DNodal
    from simpeg_gb300.resistivity.survey import Survey

    torch.cuda.set_device(0)
    if args.sens_full_survey:
        # the Gauss-Newton survey (512 dipoles x 48 receivers, 1,312 electrodes) on a 64x64x32-cell mesh
        mesh, m_true, m0, survey = workloads.gauss_newton(seed=4, ncore_xy=48, ncore_z=24)
    else:
        mesh, m_true, m0, survey = workloads.gauss_newton(seed=4, n_lines=8, src_per_line=16, n_rx=24, ncore_xy=80,
                                                         ncore_z=40)
    if args.sources:
        survey = Survey(survey.source_list[:args.sources])
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), precision="mixed", rtol=RTOL)
    diag = sim.getJtJdiag(m_true)
    g = sim.Jtvec(m_true, np.ones(survey.nD))
    torch.cuda.synchronize()
    print(json.dumps({"profile_sens": {"nodes": int(mesh.n_nodes), "sources": survey.nSrc, "data": survey.nD,
                                       "jtj_sum": float(diag.sum()), "g_norm": float(np.linalg.norm(g))}}), flush=True)


def main():
    args = _args()
    if args.profile_solve:
        return run_profile_solve(args)
    if args.profile_sens:
        return run_profile_sens(args)
    if args.workload == "block":
        return run_block(args)
    if args.workload == "batched" and args.impl != "reference":
        return run_batched(args)
    if args.workload == "gauss_newton" and args.impl != "reference":
        return run_gauss_newton(args)
    if args.workload == "cc" and args.impl != "reference":
        return run_cc(args)
    if args.workload == "serving" and args.impl != "reference":
        return run_serving(args)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "differentiation":
        run_differentiation(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
