"""The reference's own CUDA path on the GPU (test and benchmark infrastructure).

The reference's kernels (GraphCutKernels.cu) are compiled from the reference
checkout into ``oracle/_ref/gc_ref_kernels.cubin`` by
``oracle/refgpu/build_ref_gpu.sh``; ``oracle/refgpu/ref_gpu.cpp`` restates
the reference's host code (GC_Init / GC_SetGraph / GC_Optimize / GC_End,
GraphCut.cu:187-568) launch for launch over those kernels, with every loop
bounded.  It is the reference's CUDA path timed beside this repository's on
the same GPU; it is never part of the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "refgpu", "ref_gpu.cpp")
LIB_PATH = os.path.join(HERE, "librefgpu.so")
CUBIN = os.path.join(HERE, "_ref", "gc_ref_kernels.cubin")
CUBIN8 = os.path.join(HERE, "_ref", "gc_ref_kernels8.cubin")  # the NEIGHBORHOOD 8 build
CUBIN_DT = os.path.join(HERE, "_ref", "gc_ref_dt_kernels.cubin")  # the data-term kernels

STATUS = {0: "ok", 1: "invalid", 2: "cuda error", 3: "iteration or time cap reached", 4: "kernels not loaded"}


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_longlong), ("global_relabels", C.c_longlong),
                ("gr_launches", C.c_longlong), ("spread_launches", C.c_longlong),
                ("initial_energy", C.c_int), ("final_energy", C.c_int), ("converged", C.c_int),
                ("pad", C.c_int), ("ms_init", C.c_double), ("ms_solve", C.c_double),
                ("ms_loop", C.c_double), ("ms_end", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the host driver (plain C++ against the CUDA runtime, static
    cudart) into oracle/librefgpu.so.  Needs no reference source."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call([os.environ.get("NVCC", "nvcc"), "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
                           "-shared", "-o", tmp, SRC])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def unavailable(neighborhood: int = 4) -> str | None:
    """None when the reference's CUDA path can run here, else why not
    (neighborhood 4 or 8: the solver's kernels; 0: the data-term kernels)."""
    path = CUBIN8 if neighborhood == 8 else CUBIN_DT if neighborhood == 0 else CUBIN
    if not os.path.exists(path):
        return (f"the reference's kernels were not compiled (oracle/_ref/{os.path.basename(path)} is built "
                "from the reference checkout)")
    return None


_lib = None
_loaded = set()


def lib(neighborhood: int = 4):
    global _lib
    why = unavailable(neighborhood)
    if why:
        raise RuntimeError(why)
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.refgpu_load.argtypes = [C.c_char_p]
        L.refgpu_load8.argtypes = [C.c_char_p]
        L.refgpu_solve.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, P, P, P, C.c_longlong, C.c_double,
                                   C.POINTER(Stats)]
        L.refgpu_solve8.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, C.c_longlong, C.c_double,
                                    C.POINTER(Stats)]
        L.refgpu_load_dt.argtypes = [C.c_char_p]
        L.refgpu_kde.argtypes = [C.c_int, C.c_int, P, C.c_int, C.c_int, P, P, P, P, P]
        L.refgpu_draw.argtypes = [C.c_int, C.c_int, P, P, P]
        _lib = L
    if neighborhood not in _loaded:
        rc = (_lib.refgpu_load8(CUBIN8.encode()) if neighborhood == 8 else
              _lib.refgpu_load_dt(CUBIN_DT.encode()) if neighborhood == 0 else _lib.refgpu_load(CUBIN.encode()))
        if rc:
            raise RuntimeError(f"loading the reference's kernels failed: {STATUS.get(rc, rc)}")
        _loaded.add(neighborhood)
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def solve(dp, dn, penalty=0, up=None, down=None, left=None, right=None, max_iters=5_000_000,
          max_seconds=60.0):
    """Runs the reference's GC_Init -> GC_SetGraph -> GC_Optimize -> GC_End on
    host arrays (H, W) int32.  Returns dict(label, energy (the printed final
    energy level), status, converged, stats...)."""
    dp = np.ascontiguousarray(dp, np.int32)
    dn = np.ascontiguousarray(dn, np.int32)
    H, W = dp.shape
    arrs = [None if a is None else np.ascontiguousarray(a, np.int32) for a in (up, down, left, right)]
    label = np.zeros((H, W), np.int32)
    st = Stats()
    rc = lib().refgpu_solve(W, H, _p(dp), _p(dn), int(penalty), *[_p(a) for a in arrs], _p(label),
                            int(max_iters), float(max_seconds), C.byref(st))
    return _result(st, rc, label)


def _result(st, rc, label):
    out = {k: getattr(st, k) for k, _ in Stats._fields_ if k != "pad"}
    out.update(status=STATUS.get(rc, rc), rc=rc, label=label, energy=st.final_energy)
    return out


def solve8(dp, dn, penalty=0, arrays=None, max_iters=5_000_000, max_seconds=60.0):
    """The reference's NEIGHBORHOOD 8 solver: arrays = None (constant penalty)
    or the eight (H, W) int32 arrays up, down, left, right, upleft, upright,
    downleft, downright."""
    dp = np.ascontiguousarray(dp, np.int32)
    dn = np.ascontiguousarray(dn, np.int32)
    H, W = dp.shape
    label = np.zeros((H, W), np.int32)
    st = Stats()
    ptrs = None
    keep = None
    if arrays is not None:
        keep = [np.ascontiguousarray(a, np.int32) for a in arrays]
        assert len(keep) == 8
        ptrs = (C.c_void_p * 8)(*[a.ctypes.data for a in keep])
    rc = lib(8).refgpu_solve8(W, H, _p(dp), _p(dn), int(penalty), ptrs, _p(label), int(max_iters),
                              float(max_seconds), C.byref(st))
    return _result(st, rc, label)


def kde(img, points, sigma=0):
    """The reference's kernel-density data term on the GPU (DataTermKernels.cu
    driven as DataTerm.cpp does: init_data_term, setImage, setSigmaGaussian
    when sigma > 0, selectOnMap per point, getDataTermsMixture).  img: (H, W, 3)
    uint8 with H and W multiples of 16; points: (x, y) pairs whose 5x5 squares
    lie inside the image.  Returns dict(pos, neg (H, W) int32, gauss (101,)
    float32, map (H, W) uint8)."""
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape[:2]
    pts = np.ascontiguousarray(np.asarray(points, np.int32).reshape(-1, 2))
    pos = np.zeros((H, W), np.int32)
    neg = np.zeros((H, W), np.int32)
    gauss = np.zeros(101, np.float32)
    sel = np.zeros((H, W), np.uint8)
    rc = lib(0).refgpu_kde(W, H, _p(img), int(sigma), len(pts), _p(pts), _p(pos), _p(neg), _p(gauss), _p(sel))
    if rc:
        raise RuntimeError(f"refgpu_kde: {STATUS.get(rc, rc)}")
    return dict(pos=pos, neg=neg, gauss=gauss, map=sel)


def draw(sel_map, img):
    """The reference's drawSelection (K_DrawMap) on the GPU: the pixels whose
    map entry is 1 painted (0, 0, 255).  H and W multiples of 16."""
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape[:2]
    m = np.ascontiguousarray(sel_map, np.uint8)
    out = np.empty_like(img)
    rc = lib(0).refgpu_draw(W, H, _p(m), _p(img), _p(out))
    if rc:
        raise RuntimeError(f"refgpu_draw: {STATUS.get(rc, rc)}")
    return out
