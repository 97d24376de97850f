"""Host-side pieces of the benchmark's JSON contract (no GPU): the per-kind DRAM traffic read
from the committed ncu summary, the roofline arithmetic of the timed stencil steps, the SuperLU
extrapolation and the workload choices."""

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_by_kind_covers_every_step_kind(bench):
    tbk = bench._traffic_by_kind()
    assert set(tbk) == {"zero_start", "momentum", "plain", "momentum_rz"}
    # fp16 lanes: 4, 6 or 8 algorithmic bytes per node-RHS plus the coefficient re-reads
    for k, v in tbk.items():
        alg = bench.STEP_LANE_BYTES[k]
        assert alg < v < 1.2 * alg


def test_stencil_roofline_arithmetic(bench):
    # two kinds, bytes and milliseconds chosen so the expected figures are exact
    kinds = {"plain": (2, 1.0, 2.0e9), "momentum": (1, 1.0, 3.0e9)}
    ms, n, alg = 2.0, 3, 5.0e9
    r = bench._stencil_roofline(ms, n, alg, kinds, scaled_traffic=True)
    peak = r["peak"]
    assert r["achieved"] == pytest.approx(alg / 2e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    assert r["alg_bytes_per_launch"] == pytest.approx(alg / n)
    assert r["by_kind"]["plain"]["us_per_launch"] == pytest.approx(500.0)
    assert r["by_kind"]["momentum"]["achieved"] == pytest.approx(3.0e9 / 1e-3 / 1e9)
    # scaled traffic: each kind's algorithmic bytes times its measured DRAM/algorithmic ratio
    tbk = bench._traffic_by_kind()
    ratio = {k: tbk[k] / ((bench.STEP_LANE_BYTES[k] * 256 + 20.0) / 256) for k in kinds}
    want = (2.0e9 * ratio["plain"] + 3.0e9 * ratio["momentum"]) / n
    assert r["traffic"] == pytest.approx(want)
    assert bench._stencil_roofline(1.0, 0, 1.0) is None


def test_superlu_extrapolation_passes_through_the_probes(bench):
    probes = sorted(bench.SUPERLU_PROBES.items())
    n_top, (fac, nnz, sol) = probes[-1]
    e = bench._superlu_extrapolated(n_top, 1)
    assert e["factor_s"] == pytest.approx(fac)
    assert e["nnz_LU"] == pytest.approx(nnz)
    assert e["solve_s_per_rhs"] == pytest.approx(sol)
    big = bench._superlu_extrapolated(1081665, 256)
    assert big["factor_s"] > 3600 and big["memory_GB"] > 62  # does not fit the probe host


def test_workload_choices(bench, monkeypatch):
    for w in ("forward", "block", "differentiation", "gauss_newton", "batched", "cc", "serving"):
        monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", w])
        assert bench._args().workload == w
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench._args()
    assert (a.gpus, a.workload, a.impl) == (1, "forward", "gb300") and a.warmup >= 3
