"""Builds lpm_gb300/_lib/liblpm_gb300.so for sm_103a with nvcc.

Translation units compile in parallel; the shared library links the static
CUDA runtime so it loads without a CUDA library path.  Used by
``__graft_entry__.build()`` and by ``python -m lpm_gb300.build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "liblpm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["direct_sum.cu", "stepper.cu", "capi.cu", "noalloc.cu", "oneshot.cu", "ensemble.cu", "farfield.cu",
              "mlp.cu", "ffapi.cu", "mesh_dev.cu", "swe.cu"]
CXX_SOURCES = ["mesh.cpp", "ics.cpp", "tree.cpp", "vtk.cpp", "netcdf.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build lpm_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "lpm_gb300.h"]
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    nv = nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", *inc, "-c", str(s), "-o", str(o)])
    for src in CXX_SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            # no contraction: the same FP64 results on x86-64 and aarch64 hosts,
            # and the on-device mesh generator reproduces the host mesh bitwise
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
                         *inc, "-c", str(s), "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd), flush=True)
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        cmd = [nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
    return LIB


if __name__ == "__main__":
    path = build(verbose=True, force="--force" in sys.argv)
    print(path)
