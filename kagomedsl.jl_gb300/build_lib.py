"""Builds libkvmc.so (CUDA, sm_103a) in-tree under kagomedsl.jl_gb300/_build/.

The translation units compile in parallel, then link into one shared
library that exports the C ABI of include/kvmc.h.  Needs only nvcc; no GPU.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libkvmc.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", str(ROOT / "include"), "-I", str(CSRC)]
SOURCES = ["kvmc_kernels.cu", "kvmc_warp.cu", "kvmc_complex.cu", "kvmc_grad.cu", "kvmc_refresh32.cu", "kvmc_refresh_tile.cu", "kvmc_cluster.cu", "kvmc_refresh_oz.cu", "kvmc_api.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = [ROOT / "include" / "kvmc.h", CSRC / "kvmc_internal.h", CSRC / "kvmc_device.cuh", CSRC / "kvmc_refine.cuh", CSRC / "kvmc_tile.cuh"]
    objs, procs = [], []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            lang = [] if s.suffix == ".cu" else ["-x", "cu"]
            cmd = [nvcc(), *ARCH, *COMMON, *lang, "-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{out.decode()}")
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout.decode()}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
