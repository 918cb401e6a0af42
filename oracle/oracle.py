"""ctypes binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, to check and time against.  The product library
(libgcfg.so) neither links nor calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.join(os.path.dirname(HERE), "gc-fg_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
import synth  # noqa: E402  (input generator; the oracle only checks)
LIB_PATH = os.path.join(HERE, "liboracle.so")

_CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c11", "-Wall",
           "-Wno-unused-function"]


def build(force: bool = False) -> str:
    """Compile oracle.c into liboracle.so next to it (gcc, no cmake)."""
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *_CFLAGS, "-o", tmp, src, "-lm", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


class Stats(C.Structure):
    _fields_ = [("flow", C.c_int64), ("pushes", C.c_int64), ("relabels", C.c_int64),
                ("global_relabels", C.c_int64), ("augments", C.c_int64)]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        _lib.or_histograms.argtypes = [P, P, C.c_int, P, P]
        _lib.or_tlink_lut.argtypes = [P, P, P, P, P, P]
        _lib.or_tlinks.argtypes = [P, C.c_int, P, P, P, P]
        _lib.or_sigma_sum.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        _lib.or_nlink_weight_raw.argtypes = [C.c_int, C.c_double, C.c_int64, C.c_int64]
        _lib.or_nlink_weight_raw.restype = C.c_double
        _lib.or_nlinks.argtypes = [P, C.c_int, C.c_int, C.c_double, P, P, P, P]
        _lib.or_build.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, P, P, P, P]
        _lib.or_maxflow_pr.argtypes = [C.c_int, C.c_int, P, P, C.POINTER(Stats)]
        _lib.or_maxflow_bk.argtypes = [C.c_int, C.c_int, P, P, C.POINTER(Stats)]
        _lib.or_cuts.argtypes = [C.c_int, C.c_int, P, P, P, P]
        _lib.or_cut_energy.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, P, P, P]
        _lib.or_cut_energy.restype = C.c_int64
        _lib.or_interior_dp.argtypes = [C.c_int, C.c_int, P]
        _lib.or_interior_dp.restype = C.c_int64
        _lib.or_reference_energy.argtypes = [C.c_int, C.c_int, P, P]
        _lib.or_reference_energy.restype = C.c_int32
        _lib.or_solve.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, P, P, C.c_int, P, P,
                                  C.POINTER(C.c_int64), P, C.POINTER(Stats)]
        _lib.or_segment.argtypes = [P, P, C.c_int, C.c_int, C.c_double, C.c_int, P, P, P, P, P, P,
                                    P, P, C.POINTER(C.c_int64)]
        _lib.or_segment_batch.argtypes = [C.c_int, P, P, P, P, P, P, C.c_int, C.c_int, P, P, P]
        _lib.or8_solve.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, P, C.POINTER(C.c_int64), P]
        _lib.or_kde_gauss.argtypes = [C.c_int, P]
        _lib.or_kde_select.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P]
        _lib.or_kde_terms.argtypes = [P, P, C.c_int, P, C.c_int, P, P]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def generate(cfg: int, W: int, H: int, seed: int):
    """Synthetic inputs (delegates to the package's generator)."""
    return synth.generate(cfg, W, H, seed)


def histograms(rgb, scrib):
    hf = np.empty(4096, np.int32)
    hb = np.empty(4096, np.int32)
    lib().or_histograms(_p(np.ascontiguousarray(rgb)), _p(np.ascontiguousarray(scrib)),
                        scrib.size, _p(hf), _p(hb))
    return hf, hb


def tlink_lut(hf, hb):
    raw_dp = np.empty(4096, np.float64)
    raw_dn = np.empty(4096, np.float64)
    dp = np.empty(4096, np.int32)
    dn = np.empty(4096, np.int32)
    lib().or_tlink_lut(_p(hf), _p(hb), _p(raw_dp), _p(raw_dn), _p(dp), _p(dn))
    return raw_dp, raw_dn, dp, dn


def tlinks(rgb, scrib):
    hf, hb = histograms(rgb, scrib)
    _, _, dpl, dnl = tlink_lut(hf, hb)
    n = scrib.size
    dp = np.empty(scrib.shape, np.int32)
    dn = np.empty(scrib.shape, np.int32)
    lib().or_tlinks(_p(np.ascontiguousarray(rgb)), n, _p(dpl), _p(dnl), _p(dp), _p(dn))
    return dp, dn


def sigma_sum(rgb):
    H, W = rgb.shape[:2]
    s = C.c_int64()
    c = C.c_int64()
    lib().or_sigma_sum(_p(np.ascontiguousarray(rgb)), W, H, C.byref(s), C.byref(c))
    return s.value, c.value


def nlink_weight_raw(d2: int, lam: float, s: int, c: int) -> float:
    return lib().or_nlink_weight_raw(int(d2), float(lam), int(s), int(c))


def nlinks(rgb, lam: float):
    H, W = rgb.shape[:2]
    up, down, left, right = (np.empty((H, W), np.int32) for _ in range(4))
    lib().or_nlinks(_p(np.ascontiguousarray(rgb)), W, H, float(lam), _p(up), _p(down), _p(left), _p(right))
    return up, down, left, right


def build_graph(dp, dn, penalty=0, up=None, down=None, left=None, right=None):
    H, W = dp.shape
    caps = np.empty((H, W, 4), np.int32)
    ex = np.empty((H, W), np.int32)
    lib().or_build(W, H, _p(dp), _p(dn), int(penalty), _p(up), _p(down), _p(left), _p(right),
                   _p(caps), _p(ex))
    return caps, ex


def solve(dp, dn, penalty=0, up=None, down=None, left=None, right=None, solver="bk"):
    """Exact max-flow in the reference's conventions.

    Returns dict(flow, smin, smax, excess, stats)."""
    dp = np.ascontiguousarray(dp, np.int32)
    dn = np.ascontiguousarray(dn, np.int32)
    arrs = [None if a is None else np.ascontiguousarray(a, np.int32) for a in (up, down, left, right)]
    H, W = dp.shape
    smin = np.empty((H, W), np.uint8)
    smax = np.empty((H, W), np.uint8)
    ex = np.empty((H, W), np.int32)
    flow = C.c_int64()
    st = Stats()
    rc = lib().or_solve(W, H, _p(dp), _p(dn), int(penalty), *[_p(a) for a in arrs],
                        1 if solver == "bk" else 0, _p(smin), _p(smax), C.byref(flow), _p(ex),
                        C.byref(st))
    if rc:
        raise RuntimeError(f"or_solve failed: {rc}")
    return dict(flow=flow.value, smin=smin, smax=smax, excess=ex,
                stats=dict(pushes=st.pushes, relabels=st.relabels,
                           global_relabels=st.global_relabels, augments=st.augments))


def cut_energy(label, dp, dn, penalty=0, up=None, down=None, left=None, right=None) -> int:
    H, W = dp.shape
    arrs = [None if a is None else np.ascontiguousarray(a, np.int32) for a in (up, down, left, right)]
    return lib().or_cut_energy(W, H, _p(np.ascontiguousarray(dp, np.int32)),
                               _p(np.ascontiguousarray(dn, np.int32)), int(penalty),
                               *[_p(a) for a in arrs], _p(np.ascontiguousarray(label, np.uint8)))


def reference_energy(dp, excess_final) -> int:
    H, W = dp.shape
    return lib().or_reference_energy(W, H, _p(np.ascontiguousarray(dp, np.int32)),
                                     _p(np.ascontiguousarray(excess_final, np.int32)))


def segment(rgb, scrib, lam: float, solver="bk"):
    """Full pipeline on one image: t-links, n-links, exact cut."""
    H, W = scrib.shape
    bufs = [np.empty((H, W), np.int32) for _ in range(6)]
    smin = np.empty((H, W), np.uint8)
    smax = np.empty((H, W), np.uint8)
    flow = C.c_int64()
    rc = lib().or_segment(_p(np.ascontiguousarray(rgb)), _p(np.ascontiguousarray(scrib)), W, H,
                          float(lam), 1 if solver == "bk" else 0, *[_p(b) for b in bufs],
                          _p(smin), _p(smax), C.byref(flow))
    if rc:
        raise RuntimeError(f"or_segment failed: {rc}")
    dp, dn, up, down, left, right = bufs
    return dict(flow=flow.value, smin=smin, smax=smax, dp=dp, dn=dn, up=up, down=down,
                left=left, right=right)


def segment_batch(images, lambdas, nthreads: int, solver="bk"):
    """images: list of (rgb, scrib). Solved one image per host thread."""
    Ws = np.array([s.shape[1] for _, s in images], np.int32)
    Hs = np.array([s.shape[0] for _, s in images], np.int32)
    sizes = Ws.astype(np.int64) * Hs
    offs = np.zeros(len(images), np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    rgb = np.concatenate([r.reshape(-1) for r, _ in images])
    scrib = np.concatenate([s.reshape(-1) for _, s in images])
    lam = np.asarray(lambdas, np.float64)
    total = int(sizes.sum())
    smin = np.empty(total, np.uint8)
    smax = np.empty(total, np.uint8)
    flows = np.empty(len(images), np.int64)
    rc = lib().or_segment_batch(len(images), _p(Ws), _p(Hs), _p(offs), _p(rgb), _p(scrib), _p(lam),
                                1 if solver == "bk" else 0, int(nthreads), _p(smin), _p(smax),
                                _p(flows))
    if rc:
        raise RuntimeError(f"or_segment_batch failed: {rc}")
    return flows, smin, smax, offs


def fnv1a(a) -> int:
    return synth.fnv1a(a)


def kde_gauss(sigma: int):
    """The reference's 101-entry Gaussian table (double evaluation)."""
    g = np.empty(101, np.float32)
    lib().or_kde_gauss(int(sigma), _p(g))
    return g


def kde_select(rgb, x: int, y: int):
    """Colours a selectOnMap(x, y) adds, in the reference's order."""
    H, W = rgb.shape[:2]
    sel = np.empty((25, 3), np.uint8)
    k = lib().or_kde_select(_p(np.ascontiguousarray(rgb)), W, H, int(x), int(y), _p(sel))
    return sel[:k]


def kde_terms(gauss, sel, rgb):
    """(pos, neg) int32 of the reference's kernel-density data term."""
    gauss = np.ascontiguousarray(gauss, np.float32)
    sel = np.ascontiguousarray(sel, np.uint8).reshape(-1, 3)
    rgb = np.ascontiguousarray(rgb, np.uint8)
    n = rgb.size // 3
    pos = np.empty(rgb.shape[:-1], np.int32)
    neg = np.empty(rgb.shape[:-1], np.int32)
    lib().or_kde_terms(_p(gauss), _p(sel), len(sel), _p(rgb), n, _p(pos), _p(neg))
    return pos, neg


def solve8(dp, dn, penalty=0, arrays=None):
    """8-connected solve in the reference's conventions.  arrays: None
    (constant penalty) or 8 (H, W) arrays: left, right, up, down, up-left,
    up-right, down-left, down-right.  Returns dict(flow, smin, smax, excess)."""
    dp = np.ascontiguousarray(dp, np.int32)
    dn = np.ascontiguousarray(dn, np.int32)
    H, W = dp.shape
    keep = None
    ptrs = None
    if arrays is not None:
        keep = [np.ascontiguousarray(a, np.int32) for a in arrays]
        assert len(keep) == 8
        ptrs = (C.c_void_p * 8)(*[a.ctypes.data for a in keep])
    smin = np.empty((H, W), np.uint8)
    smax = np.empty((H, W), np.uint8)
    ex = np.empty((H, W), np.int32)
    flow = C.c_int64()
    rc = lib().or8_solve(W, H, _p(dp), _p(dn), int(penalty), C.cast(ptrs, C.c_void_p) if ptrs is not None else None,
                         _p(smin), _p(smax), C.byref(flow), _p(ex))
    if rc != 0:
        raise RuntimeError(f"or8_solve failed: {rc}")
    return dict(flow=flow.value, smin=smin, smax=smax, excess=ex)
