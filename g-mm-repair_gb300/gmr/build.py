"""Builds libgmr.so (the C-ABI engine) in-tree for sm_103a.

Host C++ sources are compiled with g++, the CUDA engine with nvcc
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into
``gmr/libgmr.so`` with the CUDA runtime linked statically.  Objects go to
``g-mm-repair_gb300/_build``.  A rebuild happens only when a source or header
is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent                      # g-mm-repair_gb300/
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
BUILD = ROOT / "_build"
LIB = PKG_DIR / "libgmr.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["grammar_io.cpp", "generators.cpp", "repair.cpp", "plan.cpp"]
CUDA_SOURCES = ["engine.cu", "learn.cu", "plan_device.cu", "repair_device.cu"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [CSRC / s for s in HOST_SOURCES + CUDA_SOURCES]


def _deps():
    return _sources() + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "gmr.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps() if p.exists())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}"]
    jobs = []
    for s in HOST_SOURCES:
        jobs.append(["g++", *common, "-fPIC", "-Wall", "-pthread", "-c", str(CSRC / s),
                     "-o", str(BUILD / (s + ".o"))])
    for s in CUDA_SOURCES:
        # --split-compile=0: device optimisation in parallel threads (engine.cu
        # instantiates many kernel variants)
        jobs.append([nvcc, *ARCH, "-lineinfo", "--split-compile=0", *common, "-Xcompiler", "-fPIC", "-c",
                     str(CSRC / s), "-o", str(BUILD / (s + ".o"))])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    objs = [str(BUILD / (s + ".o")) for s in HOST_SOURCES + CUDA_SOURCES]
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs, "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
