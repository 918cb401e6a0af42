"""Build libgcfg.so (the CUDA library) in-tree with nvcc for sm_103a, and
the command-line tools of cli/ into bin/.

The translation units compile in parallel and link into one shared library
next to this file; no cmake, one -gencode.  The tools (solve_mrf,
segment_dat, multiply_mrf) are host C++ linked against the library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libgcfg.so")
OBJ_DIR = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# extra nvcc flags for experiments (e.g. -DGCFG_SOLVE_MIN_BLOCKS=4)
FLAGS += os.environ.get("GCFG_NVCC_EXTRA", "").split()


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    out = sources()
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out.append(os.path.join(HERE, "..", "include", "gcfg.h"))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        cmd = [NVCC, *ARCH, *FLAGS, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


CLI = os.path.join(HERE, "cli")
BIN = os.path.join(HERE, "bin")
INCLUDE = os.path.join(HERE, "..", "include")
TOOLS = {"solve_mrf": True, "segment_dat": True, "multiply_mrf": False}  # name -> links libgcfg


def build_tools(force: bool = False, verbose: bool = False) -> list:
    """Compile cli/<tool>.cpp into bin/<tool> (after the library)."""
    build(force=False, verbose=verbose)
    os.makedirs(BIN, exist_ok=True)
    hdrs = [os.path.join(CLI, f) for f in os.listdir(CLI) if f.endswith(".hpp")]
    hdrs += [os.path.join(INCLUDE, f) for f in ("gcfg.h", "GraphCut.h", "GraphCut.cu", "DataTerm.h")]

    def one(name):
        src = os.path.join(CLI, name + ".cpp")
        exe = os.path.join(BIN, name)
        deps = [src, *hdrs] + ([LIB] if TOOLS[name] else [])
        if not force and os.path.exists(exe) and all(os.path.getmtime(d) <= os.path.getmtime(exe) for d in deps):
            return exe
        cmd = [NVCC, "-std=c++17", "-O2", "-I", INCLUDE, "-I", CLI, src, "-o", exe]
        if TOOLS[name]:
            cmd += ["-L", HERE, "-lgcfg", "-Xlinker", "-rpath=$ORIGIN/.."]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"tool build failed for {name}:\n{r.stderr}")
        return exe

    with ThreadPoolExecutor(max_workers=len(TOOLS)) as ex:
        return list(ex.map(one, sorted(TOOLS)))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_tools(force="--force" in sys.argv, verbose=True))
