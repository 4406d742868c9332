"""Build the native library ``xped_gb300/_lib/libxgb.so`` in-tree.

CUDA sources are compiled for sm_103a only (one -gencode), host C++ with g++;
translation units are compiled in parallel.  No cmake, no network.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
INCLUDE = PKG.parent / "include"
LIB = OUT / "libxgb.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["kernels.cu", "svd.cu", "gemm_tc.cu", "gemm_oz.cu", "rsvd.cu", "mlp.cu"]
CPP_SOURCES = ["meta.cpp", "tensor.cpp", "capi.cpp", "rsvd.cpp", "mlp.cpp", "checkpoint.cpp", "autotune.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _sources_newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.hpp")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = OUT / (s.stem + ".cu.o")
        objs.append(o)
        if force or _sources_newer(o, [s] + headers):
            jobs.append([NVCC, *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
    for src in CPP_SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _sources_newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I", str(CUDA_HOME / "include"), "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-o", str(tmp), *map(str, objs), "-L", str(CUDA_HOME / "lib64"), "-lcudart",
              "-Wl,-rpath," + str(CUDA_HOME / "lib64")])
        shutil.move(str(tmp), str(LIB))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
