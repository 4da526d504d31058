"""Builds ``librsgpu.so`` (the CUDA kernels and the C ABI of include/rsgpu.h) in-tree.

Every translation unit under ``ddg-tools_gb300/csrc`` is compiled in parallel: ``.cu`` files by
``nvcc -gencode arch=compute_103a,code=sm_103a`` (GB300 only), ``.cpp`` host files by the host
compiler with ``-ffp-contract=off`` (the face tree must round like the reference). Objects go
to ``ddg-tools_gb300/_build/``, the library to ``ddg-tools_gb300/rs_gb300/librsgpu.so``.
The measurement aid under ``csrc/probe`` (the device's FP32 FMA throughput) becomes its own
``librsprobe.so`` beside it, outside the product's C ABI. Rebuilds only what changed (by
modification time).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent  # ddg-tools_gb300/
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
INCLUDE = ROOT.parent / "include"
LIB = PKG / "librsgpu.so"
PROBE_SRC = CSRC / "probe" / "fp32_peak.cu"
PROBE_LIB = PKG / "librsprobe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Device code that must round like the reference's FP64 host code, operation for operation:
# no multiply-add contraction.
NO_FMAD = {"ccd.cu"}


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h*")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}"]
    cmds = []
    objs = []
    for src in srcs:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if not _stale(obj, [src, *headers, Path(__file__)]):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                   *(["-fmad=false"] if src.name in NO_FMAD else []),
                   "-c", str(src), "-o", str(obj)]
        else:
            cmd = [os.environ.get("CXX", "g++"), *common, "-fPIC", "-ffp-contract=off",
                   f"-I{cuda / 'include'}", "-c", str(src), "-o", str(obj)]
        cmds.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    if _stale(PROBE_LIB, [PROBE_SRC, Path(__file__)]):
        cmds.append([nvcc, *ARCH, "-O3", "-Xcompiler", "-fPIC", "-shared", str(PROBE_SRC), "-o", str(PROBE_LIB)])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(run, cmds))
    if _stale(LIB, objs):
        link = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        run(link)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv))
