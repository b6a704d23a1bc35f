"""Builds libatlas_rt.so in-tree: CUDA sources for sm_103a with nvcc, host C++
with g++, compiled in parallel and linked into one shared library next to
this file.  No cmake; a couple of translation units, one -gencode.

Host code is compiled with -ffp-contract=off so that the BVH builder rounds
identically on x86-64 and aarch64 (GCC fuses multiply-adds on aarch64 by
default).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
SRC_ROOT = PKG_DIR.parent                      # atlas-engine_gb300/
CSRC = SRC_ROOT / "csrc"
REPO = SRC_ROOT.parent
INCLUDE = REPO / "include"
BUILD_DIR = SRC_ROOT / "_build"
LIB_NAME = "libatlas_rt.so"
LIB_PATH = PKG_DIR / LIB_NAME

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libatlas_rt.so")
    return cand


def _cuda_lib_dir(nvcc: str) -> str:
    return str(Path(nvcc).resolve().parent.parent / "lib64")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((CSRC / "host").glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, headers


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compiles and links libatlas_rt.so if any source is newer than it."""
    cu, cpp, headers = _sources()
    if (not force and LIB_PATH.exists()
            and all(p.stat().st_mtime <= LIB_PATH.stat().st_mtime for p in cu + cpp + headers)):
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CSRC / 'host'}"]
    jobs = []
    objs = []
    for src in cu:
        obj = BUILD_DIR / (src.stem + ".cu.o")
        cmd = [nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off", *inc, "-c", str(src), "-o", str(obj)]
        if ptxas_verbose:
            cmd.insert(2, "-Xptxas=-v")
        jobs.append(cmd)
        objs.append(obj)
    cxx = shutil.which("g++") or "g++"
    for src in cpp:
        obj = BUILD_DIR / (src.stem + ".cpp.o")
        jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", *inc,
                     f"-I{_cuda_lib_dir(nvcc).replace('lib64', 'include')}",
                     "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose or ptxas_verbose:
        for o in outs:
            if o.strip():
                sys.stderr.write(o)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    _run([nvcc, ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
          "-Xlinker", f"-rpath,{_cuda_lib_dir(nvcc)}", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
