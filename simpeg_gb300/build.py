"""Build the CUDA engine ``libdcgpu.so`` in-tree for sm_103a (GB300).

Compiles each translation unit in ``csrc/`` in parallel with ``nvcc`` and links
them into ``simpeg_gb300/libdcgpu.so``.  No cmake, no torch extension
machinery: the library has a plain C ABI (``include/dcgpu.h``) loaded with
ctypes.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "libdcgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["dc_stencil.cu", "dc_ops_f64.cu", "dc_ops_f32.cu", "dc_ops_f16.cu", "dc_ops_bf16.cu", "dc_sens.cu", "dc_engine.cu",
           "dc_noalloc.cu", "dc_csr.cu", "dc_jtj.cu", "dc_cc.cu", "dc_lanes.cu"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA engine cannot be built")
    return cand


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "dcgpu.h"]
    if OUT.exists() and not force:
        t = OUT.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in deps if p.exists()):
            return OUT
    nvcc = _nvcc()
    bdir = PKG / "_build"
    bdir.mkdir(exist_ok=True)
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]

    def compile_one(src: Path):
        obj = bdir / (src.stem + ".o")
        cmd = [nvcc, *common, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
