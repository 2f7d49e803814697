"""Builds librq.so (the CUDA engine + C ABI) in-tree for sm_103a.

nvcc compiles every .cu translation unit and g++ every .cpp unit in parallel; the objects are linked
into candela_gb300/lib/librq.so with the CUDA runtime linked statically, so the library loads on a
machine without a GPU (context creation then fails with RQ_ECUDA).  Host code is compiled with
-ffp-contract=off: the BVH builder must reproduce the reference's float arithmetic exactly on x86
and on aarch64, where gcc would otherwise fuse multiply-adds.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "librq.so"
EXAMPLE_SRC = PKG / "examples" / "rq_intersector_example.cpp"
EXAMPLE = PKG / "lib" / "rq_intersector_example"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
             "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or Path(c).exists()):
            return c
    return "nvcc"


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    hdr = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, hdr


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    cu, cpp, hdr = _sources()
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(obj, [src, *hdr]):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD / (src.stem + ".cpp.o")
        objs.append(obj)
        if force or _stale(obj, [src, *hdr]):
            jobs.append(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"compilation failed: {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs),
               "-Xlinker", "--no-undefined", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link of librq.so failed")
    # C++ host example over the C ABI (the RayIntersector<T> mirror in include/rq_intersector.hpp)
    if force or _stale(EXAMPLE, [EXAMPLE_SRC, LIB, *INCLUDE.glob("*.h*")]):
        cmd = ["g++", "-O2", "-std=c++17", "-I", str(INCLUDE), str(EXAMPLE_SRC), "-o", str(EXAMPLE),
               "-L", str(LIB.parent), "-lrq", f"-Wl,-rpath,{LIB.parent}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("build of the C++ example failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
