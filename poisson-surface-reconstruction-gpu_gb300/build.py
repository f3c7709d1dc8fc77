"""Builds libpsr.so (the CUDA path and its C ABI) in-tree for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into one shared
library next to this file.  No torch extension machinery: the library is a plain C ABI
(include/psr/psr.h) loaded with ctypes by the Python mirror (psr.py) and usable from C++.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = PKG / "libpsr.so"

CUDA_SOURCES = ["primitives.cu", "octree.cu", "field.cu", "solver.cu", "mesh.cu", "transfer.cu", "engine.cu", "surfel.cu", "noalloc.cu", "normals.cu", "weld.cu"]
CXX_SOURCES = ["tables.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = Path(home) / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _stale(obj, srcs):
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def build(force=False, verbose=False, jobs=None):
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.inc")) + \
        list((ROOT / "include" / "psr").glob("*.h"))
    cmds = []
    objs = []
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(CSRC), "-I", str(ROOT / "include")]
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = OUT / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmds.append([nvcc()] + ARCH + common + ["-c", str(s), "-o", str(o)])
    for src in CXX_SOURCES:
        s = CSRC / src
        o = OUT / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I", str(CSRC),
                         "-I", "/usr/local/cuda/include", "-c", str(s), "-o", str(o)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for msg in ex.map(run, cmds):
            if verbose and msg:
                print(msg)
    if cmds or not LIB.exists():
        link = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart"]
        run(link)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
