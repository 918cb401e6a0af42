"""Deterministic synthetic inputs (images + scribbles) for the graph-cut
workloads: ctypes binding of synth/synth.c, built with gcc next to it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "synth", "synth.c")
LIB_PATH = os.path.join(HERE, "synth", "libgcfg_synth.so")


def build(force: bool = False) -> str:
    deps = [SRC, os.path.join(HERE, "synth", "synth.h")]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c11", "-Wall",
                           "-o", tmp, SRC, "-lm", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [("family", C.c_int), ("W", C.c_int), ("H", C.c_int), ("seed", C.c_uint64),
                ("ax", C.c_double), ("ay", C.c_double), ("n_extra", C.c_int),
                ("extra_lo", C.c_double), ("extra_hi", C.c_double), ("n_blobs", C.c_int),
                ("r_lo", C.c_double), ("r_hi", C.c_double), ("sd_fg", C.c_double),
                ("sd_bg", C.c_double), ("stripe_amp", C.c_double), ("stripe_period", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        _lib.gs_gen_defaults.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(Params)]
        _lib.gs_generate.argtypes = [C.POINTER(Params), P, P]
        _lib.gs_generate_batch.argtypes = [C.c_int, P, P, P, P, C.c_int]
        _lib.gs_fnv1a.argtypes = [P, C.c_int64]
        _lib.gs_fnv1a.restype = C.c_uint64
        _lib.gs_det_log.argtypes = [C.c_double]
        _lib.gs_det_log.restype = C.c_double
        _lib.gs_det_cos.argtypes = [C.c_double]
        _lib.gs_det_cos.restype = C.c_double
    return _lib


def params(cfg: int, W: int, H: int, seed: int) -> Params:
    p = Params()
    lib().gs_gen_defaults(cfg, W, H, seed, C.byref(p))
    return p


def generate(cfg: int, W: int, H: int, seed: int):
    """One image of a workload family: (rgb uint8 [H, W, 3], scribbles uint8
    [H, W]: 0 none, 1 foreground, 2 background)."""
    p = params(cfg, W, H, seed)
    rgb = np.empty((H, W, 3), np.uint8)
    scrib = np.empty((H, W), np.uint8)
    rc = lib().gs_generate(C.byref(p), rgb.ctypes.data_as(C.c_void_p), scrib.ctypes.data_as(C.c_void_p))
    if rc:
        raise RuntimeError(f"gs_generate failed: {rc}")
    return rgb, scrib


def generate_packed(specs, nthreads: int | None = None):
    """Many images packed back to back: specs = [(cfg, W, H, seed), ...].
    Returns (rgb uint8 [3*sum], scrib uint8 [sum], offsets int64[n])."""
    n = len(specs)
    arr = (Params * n)()
    sizes = np.array([W * H for (_, W, H, _) in specs], np.int64)
    offs = np.zeros(n, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    for i, (cfg, W, H, seed) in enumerate(specs):
        lib().gs_gen_defaults(cfg, W, H, seed, C.byref(arr[i]))
    total = int(sizes.sum())
    rgb = np.empty(3 * total, np.uint8)
    scrib = np.empty(total, np.uint8)
    rc = lib().gs_generate_batch(n, C.cast(arr, C.c_void_p), offs.ctypes.data_as(C.c_void_p),
                                 rgb.ctypes.data_as(C.c_void_p), scrib.ctypes.data_as(C.c_void_p),
                                 int(nthreads or os.cpu_count() or 1))
    if rc:
        raise RuntimeError(f"gs_generate_batch failed: {rc}")
    return rgb, scrib, offs


def fnv1a(a) -> int:
    a = np.ascontiguousarray(a)
    return lib().gs_fnv1a(a.ctypes.data_as(C.c_void_p), a.nbytes)


def batch_shapes(n: int = 256, seed0: int = 1000, lo: int = 64, hi: int = 1024):
    """Uneven batch: side log-uniform in [lo, hi], aspect uniform in [0.5, 2];
    W = round(s * sqrt(a)), H = round(s / sqrt(a)); image i uses seed seed0 + i
    for its pixels and the shape stream below for its size."""
    st = [seed0 * 7919 + 17]
    out = []
    for i in range(n):
        s = float(np.exp(np.log(lo) + _u(st) * (np.log(hi) - np.log(lo))))
        a = 0.5 + _u(st) * 1.5
        W = max(3, int(round(s * np.sqrt(a))))
        H = max(3, int(round(s / np.sqrt(a))))
        out.append((W, H, seed0 + i))
    return out


def _u(st):
    """splitmix64 uniform in [0,1) on a Python-held state (shape stream)."""
    st[0] = (st[0] + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = st[0]
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    z ^= z >> 31
    return (z >> 11) * (1.0 / 9007199254740992.0)


SERVE_SIZES = ((256, 0.6), (1024, 0.3), (2048, 0.1))


def serve_trace(n_req: int = 1200, rate: float = 500.0, seed: int = 4, edit_frac: float = 0.3,
                pool=(48, 24, 8), edit_size: int = 15, lam: float = 50.0):
    """Request trace of the serving workload.

    Poisson arrivals at `rate` requests/s.  A request is a scribble edit with
    probability `edit_frac` (once an image exists): a `edit_size` square of
    class 1 (foreground) or 2 (background) at a uniform position of a uniformly
    chosen earlier image.  Otherwise it is a new square image whose side is
    256 / 1024 / 2048 with probability 0.6 / 0.3 / 0.1, drawn from the
    1920x1080-family generator (cfg 4).  New images of one side cycle through
    a pool of `pool[c]` distinct generated images (seeds 4000 + 100*c + k), so
    that the inputs stay small; every new request is still its own resident
    session.

    Returns (pool_specs, requests): pool_specs = [(4, side, side, seed)], and
    each request a dict with 't' (arrival, seconds from the start), 'kind'
    ('new' | 'edit'), and for new: 'img' (pool index), 'lam'; for edit: 'target'
    (ordinal of the new request it edits), 'x', 'y', 'size', 'cls'.
    """
    st = [seed * 104729 + 3]
    pool_specs, pool_base = [], []
    for c, (side, _) in enumerate(SERVE_SIZES):
        pool_base.append(len(pool_specs))
        pool_specs += [(4, side, side, 4000 + 100 * c + k) for k in range(pool[c])]
    cum = np.cumsum([p for _, p in SERVE_SIZES])
    t = 0.0
    reqs, news, used = [], [], [0] * len(SERVE_SIZES)
    for _ in range(n_req):
        t += float(-np.log(1.0 - _u(st)) / rate)
        if news and _u(st) < edit_frac:
            k = min(int(_u(st) * len(news)), len(news) - 1)
            side = news[k]
            span = max(1, side - edit_size + 1)
            x = min(int(_u(st) * span), span - 1)
            y = min(int(_u(st) * span), span - 1)
            cls = 1 if _u(st) < 0.5 else 2
            reqs.append(dict(t=t, kind="edit", target=k, x=x, y=y, size=edit_size, cls=cls))
        else:
            c = int(np.searchsorted(cum, _u(st), side="right"))
            c = min(c, len(SERVE_SIZES) - 1)
            img = pool_base[c] + used[c] % pool[c]
            used[c] += 1
            news.append(SERVE_SIZES[c][0])
            reqs.append(dict(t=t, kind="new", img=img, lam=lam))
    return pool_specs, reqs
