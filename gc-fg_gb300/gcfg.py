"""Python mirror of the reference's graph-cut interface over libgcfg.so.

The reference exposes C++ free functions (GraphCut.cu:187-568) and a
DataTerm namespace (DataTerm.h:9-19).  This module binds the C ABI of the
CUDA library (include/gcfg.h) with ctypes and offers the same operations
with the same names and argument meanings (GC_Init, GC_SetDataterms,
GC_SetEdges, GC_SetPenalty, GC_SetGraph, GC_Optimize, GC_End), taking CUDA
device buffers as torch tensors.  There is no CPU path: if libgcfg.so is
missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgcfg.so")

GCFG_OK = 0
GCFG_ERR_INVALID = 1
GCFG_ERR_OOM = 2
GCFG_ERR_CUDA = 3
GCFG_ERR_NOT_CONVERGED = 4
GCFG_ERR_STATE = 5
GCFG_ERR_CAPACITY = 6
GCFG_ERR_TOO_LARGE = 7
GCFG_MAX_CAP = (1 << 28) - 1
GCFG_MAX_CAP8 = (1 << 27) - 1
GCFG_NOALLOC_MAX_TILES = 640

# Every function declared in include/gcfg.h (checked by the CPU test suite).
EXPORTS = [
    "gcfg_init", "gcfg_set_dataterms", "gcfg_set_edges", "gcfg_set_penalty", "gcfg_set_graph",
    "gcfg_optimize", "gcfg_get_cuts", "gcfg_end", "gcfg_set_stream", "gcfg_set_schedule",
    "gcfg_tlinks", "gcfg_nlinks", "gcfg_seg_create", "gcfg_seg_run", "gcfg_seg_run_host",
    "gcfg_seg_set_stream", "gcfg_seg_destroy", "gcfg_strerror", "gcfg_launch_count", "gcfg_selftest_ex2",
    "gcfg_profile_enable", "gcfg_profile_read", "gcfg_batch_create", "gcfg_batch_set_stream",
    "gcfg_batch_set_params", "gcfg_batch_run", "gcfg_batch_run_host", "gcfg_batch_submit_host",
    "gcfg_batch_wait", "gcfg_batch_destroy",
    "gcfg_solve_noalloc", "gcfg_batch_set_graph", "gcfg_batch_graph_info", "gcfg_batch_autotune",
    "gcfg_batch_set_solver", "gcfg_batch_phase_split",
    "gcfg_init8", "gcfg_set_dataterms8", "gcfg_set_edges8", "gcfg_set_penalty8", "gcfg_set_graph8",
    "gcfg_optimize8", "gcfg_get_cuts8", "gcfg_end8", "gcfg_set_stream8", "gcfg_set_schedule8",
]

PROF_KINDS = ["hist", "tlut", "sigma", "wlut", "build", "solve", "extract", "other"]


class GcfgError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {strerror(status)} ({status})")


class Result(C.Structure):
    _fields_ = [("flow", C.c_int64), ("ref_energy", C.c_int32), ("status", C.c_int32),
                ("global_relabels", C.c_int32), ("gr_sweeps", C.c_int32),
                ("push_rounds", C.c_int32), ("cut_sweeps", C.c_int32),
                ("reach_tiles", C.c_int64), ("push_tiles", C.c_int64),
                ("gr_tiles", C.c_int64), ("push_sweeps", C.c_int64),
                ("push_local_relabels", C.c_int64), ("t_global_relabel_ms", C.c_float),
                ("t_count_ms", C.c_float), ("t_push_ms", C.c_float), ("t_reach_ms", C.c_float),
                ("cyc_load", C.c_int64), ("cyc_local_relabel", C.c_int64), ("cyc_sweeps", C.c_int64),
                ("cyc_writeback", C.c_int64), ("cyc_take", C.c_int64), ("ms", C.c_float), ("t_push_tail_ms", C.c_float),
                ("bfs_iters_push", C.c_int64), ("bfs_iters_gr", C.c_int64), ("cyc_global_relabel", C.c_int64),
                ("closure_checks", C.c_int32), ("closure_ends", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("push_rounds_per_gr", C.c_int32), ("max_tile_sweeps", C.c_int32),
                ("sweeps_per_local_relabel", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("ms_default", C.c_float), ("ms_best", C.c_float), ("configs_tried", C.c_int32),
                ("tile_w", C.c_int32), ("tile_h", C.c_int32), ("local_relabel_first", C.c_int32),
                ("push_only", C.c_int32), ("threads_y", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PhaseSplit(C.Structure):
    _fields_ = [("ms_relabel", C.c_float), ("ms_push", C.c_float), ("relabel_tiles", C.c_int64),
                ("active_pixels", C.c_int64), ("push_tiles", C.c_int64), ("push_sweeps", C.c_int64),
                ("push_local_relabels", C.c_int64), ("relabel_rounds", C.c_int32), ("push_phases", C.c_int32),
                ("push_queue", C.c_int32), ("grid_blocks", C.c_int32),
                ("relabel_round0_us", C.c_float), ("relabel_pull_us", C.c_float),
                ("relabel_front_us", C.c_float * 32), ("relabel_front_tiles", C.c_int32 * 32),
                ("relabel_front_work_us", C.c_float * 32), ("relabel_front_maxvisit_kcyc", C.c_float * 32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        n = min(int(self.relabel_rounds), 32)
        d["relabel_front_us"] = [round(float(x), 2) for x in self.relabel_front_us[:n]]
        d["relabel_front_tiles"] = [int(x) for x in self.relabel_front_tiles[:n]]
        d["relabel_front_work_us"] = [round(float(x), 2) for x in self.relabel_front_work_us[:n]]
        d["relabel_front_maxvisit_kcyc"] = [round(float(x), 2) for x in self.relabel_front_maxvisit_kcyc[:n]]
        return d


class ProfEntry(C.Structure):
    _fields_ = [("kind", C.c_int32), ("launches", C.c_int32), ("ms", C.c_double)]


_lib = None


def load(path: str = LIB_PATH):
    """Load libgcfg.so.  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libgcfg.so not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    P = C.c_void_p
    I = C.c_int
    S = C.c_int  # gcfg_status
    sig = {
        "gcfg_init": (S, [I, I, P, P, C.c_int32, P, P, P, P, C.POINTER(P)]),
        "gcfg_set_dataterms": (S, [P, P, P]),
        "gcfg_set_edges": (S, [P, P, P, P, P]),
        "gcfg_set_penalty": (S, [P, C.c_int32]),
        "gcfg_set_graph": (S, [P]),
        "gcfg_optimize": (S, [P, P, C.POINTER(Result)]),
        "gcfg_get_cuts": (S, [P, P, P]),
        "gcfg_end": (S, [P]),
        "gcfg_set_stream": (S, [P, P]),
        "gcfg_set_schedule": (S, [P, I, I]),
        "gcfg_tlinks": (S, [P, P, I, P, P, P, P, P]),
        "gcfg_nlinks": (S, [P, I, I, C.c_double, P, P, P, P, P]),
        "gcfg_seg_create": (S, [I, I, C.POINTER(P)]),
        "gcfg_seg_run": (S, [P, P, P, I, I, C.c_double, P, P, C.POINTER(Result)]),
        "gcfg_seg_run_host": (S, [P, P, P, I, I, C.c_double, P, P, C.POINTER(Result)]),
        "gcfg_seg_set_stream": (S, [P, P]),
        "gcfg_seg_destroy": (S, [P]),
        "gcfg_strerror": (C.c_char_p, [I]),
        "gcfg_launch_count": (C.c_int64, []),
        "gcfg_selftest_ex2": (S, [C.c_int64, P]),
        "gcfg_batch_create": (S, [I, C.c_int64, C.POINTER(P)]),
        "gcfg_batch_set_stream": (S, [P, P]),
        "gcfg_batch_set_params": (S, [P, I, I, I]),
        "gcfg_batch_run": (S, [P, I, P, P, P, P, P, P, P, P, P]),
        "gcfg_batch_run_host": (S, [P, I, P, P, P, P, P, P, P, P, P]),
        "gcfg_batch_submit_host": (S, [P, I, P, P, P, P, P, P, P, P]),
        "gcfg_batch_wait": (S, [P, C.c_int64, P, P]),
        "gcfg_batch_destroy": (S, [P]),
        "gcfg_batch_set_graph": (S, [P, I]),
        "gcfg_batch_graph_info": (S, [P, C.POINTER(I), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]),
        "gcfg_batch_autotune": (S, [P, I, P, P, P, P, P, I, C.POINTER(Tuning)]),
        "gcfg_batch_set_solver": (S, [P, C.POINTER(Tuning)]),
        "gcfg_batch_phase_split": (S, [P, I, P, P, P, P, P, C.POINTER(PhaseSplit)]),
        "gcfg_init8": (S, [I, I, P, P, C.c_int32, P, P, P, P, P, P, P, P, C.POINTER(P)]),
        "gcfg_set_dataterms8": (S, [P, P, P]),
        "gcfg_set_edges8": (S, [P, P, P, P, P, P, P, P, P]),
        "gcfg_set_penalty8": (S, [P, C.c_int32]),
        "gcfg_set_graph8": (S, [P]),
        "gcfg_optimize8": (S, [P, P, C.POINTER(Result)]),
        "gcfg_get_cuts8": (S, [P, P, P]),
        "gcfg_end8": (S, [P]),
        "gcfg_set_stream8": (S, [P, P]),
        "gcfg_set_schedule8": (S, [P, I, I]),
        "gcfg_solve_noalloc": (S, [I, I, P, P, C.c_int32, P, P, P, P, P, C.POINTER(C.c_int64), P]),
        "gcfg_profile_enable": (S, [I]),
        "gcfg_profile_read": (S, [C.POINTER(ProfEntry), I, C.POINTER(I)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def strerror(status: int) -> str:
    try:
        return load().gcfg_strerror(status).decode()
    except Exception:  # library not loadable: still give a message
        return f"status {status}"


def _check(rc: int, what: str):
    if rc != GCFG_OK:
        raise GcfgError(rc, what)


def _ptr(t):
    """Device (or host) address of a torch tensor / numpy array, or None."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return C.c_void_p(t.data_ptr())
    return t.ctypes.data_as(C.c_void_p)


def launch_count() -> int:
    return load().gcfg_launch_count()


def selftest_ex2(samples: int = 1 << 24) -> float:
    """Largest relative error of the device's approximate 2^z on [-64, 0]."""
    v = C.c_float()
    _check(load().gcfg_selftest_ex2(int(samples), C.byref(v)), "gcfg_selftest_ex2")
    return v.value


def profile_enable(on: bool = True):
    _check(load().gcfg_profile_enable(1 if on else 0), "gcfg_profile_enable")


def profile_read() -> dict:
    """Per-kernel-kind {launches, ms} since the last read (syncs the device)."""
    arr = (ProfEntry * len(PROF_KINDS))()
    n = C.c_int()
    _check(load().gcfg_profile_read(arr, len(PROF_KINDS), C.byref(n)), "gcfg_profile_read")
    return {PROF_KINDS[e.kind]: dict(launches=e.launches, ms=e.ms) for e in arr[: n.value]}


def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(getattr(stream, "cuda_stream", stream))


# ---------------------------------------------------------------------------
# Graph API: GC_* names, argument meaning and order as in GraphCut.cu
# ---------------------------------------------------------------------------

class GlobalWrapper:
    """Handle of one residual graph (GraphCut.h:110-128's GlobalWrapper)."""

    def __init__(self, handle, width, height):
        self.handle = handle
        self.width = width
        self.height = height
        # keep caller tensors alive while the graph refers to them
        self._refs = []

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                load().gcfg_end(self.handle)
            except Exception:
                pass
            self.handle = None


def GC_Init(width, height, data_positive=None, data_negative=None, penalty=0, up=None, down=None,
            left=None, right=None) -> GlobalWrapper:
    """GC_Init (GraphCut.cu:187): device int32 [H, W] tensors, caller-owned."""
    h = C.c_void_p()
    rc = load().gcfg_init(int(width), int(height), _ptr(data_positive), _ptr(data_negative),
                          int(penalty), _ptr(up), _ptr(down), _ptr(left), _ptr(right), C.byref(h))
    _check(rc, "GC_Init")
    gw = GlobalWrapper(h, width, height)
    gw._refs = [data_positive, data_negative, up, down, left, right]
    return gw


def GC_SetDataterms(gw, data_positive, data_negative):
    _check(load().gcfg_set_dataterms(gw.handle, _ptr(data_positive), _ptr(data_negative)),
           "GC_SetDataterms")
    gw._refs[:2] = [data_positive, data_negative]


def GC_SetEdges(gw, up, down, left, right):
    _check(load().gcfg_set_edges(gw.handle, _ptr(up), _ptr(down), _ptr(left), _ptr(right)),
           "GC_SetEdges")
    gw._refs[2:] = [up, down, left, right]


def GC_SetPenalty(gw, p):
    _check(load().gcfg_set_penalty(gw.handle, int(p)), "GC_SetPenalty")


def GC_SetGraph(gw):
    _check(load().gcfg_set_graph(gw.handle), "GC_SetGraph")


def GC_SetStream(gw, stream):
    _check(load().gcfg_set_stream(gw.handle, _stream_ptr(stream)), "GC_SetStream")


def GC_SetSchedule(gw, push_rounds_per_gr, max_tile_sweeps):
    _check(load().gcfg_set_schedule(gw.handle, int(push_rounds_per_gr), int(max_tile_sweeps)),
           "GC_SetSchedule")


def GC_Optimize(gw, label=None) -> dict:
    """GC_Optimize (GraphCut.cu:385): label is an optional host int32 numpy
    array [H, W] that receives the reference-style labels.  Returns the
    result record (exact flow value, reference-printed energy, counters)."""
    res = Result()
    rc = load().gcfg_optimize(gw.handle, _ptr(label), C.byref(res))
    _check(rc, "GC_Optimize")
    return res.as_dict()


def GC_GetCuts(gw, smin=None, smax=None):
    """Both canonical cuts into device uint8 [H, W] tensors."""
    _check(load().gcfg_get_cuts(gw.handle, _ptr(smin), _ptr(smax)), "GC_GetCuts")


def GC_End(gw):
    if gw.handle:
        _check(load().gcfg_end(gw.handle), "GC_End")
        gw.handle = None


# ---------------------------------------------------------------------------
# Data term and n-links
# ---------------------------------------------------------------------------

def tlinks(d_rgb, d_scrib, d_dp, d_dn, raw=False, stream=None):
    """Histogram t-links into device int32 tensors.  With raw=True returns the
    per-bin pre-rounding doubles (numpy float64[4096] each)."""
    import numpy as np
    rdp = np.empty(4096, np.float64) if raw else None
    rdn = np.empty(4096, np.float64) if raw else None
    n = d_scrib.numel()
    _check(load().gcfg_tlinks(_ptr(d_rgb), _ptr(d_scrib), int(n), _ptr(d_dp), _ptr(d_dn),
                              _ptr(rdp), _ptr(rdn), _stream_ptr(stream)), "gcfg_tlinks")
    return (rdp, rdn) if raw else None


def nlinks(d_rgb, width, height, lam, d_up, d_down, d_left, d_right, stream=None):
    _check(load().gcfg_nlinks(_ptr(d_rgb), int(width), int(height), float(lam), _ptr(d_up),
                              _ptr(d_down), _ptr(d_left), _ptr(d_right), _stream_ptr(stream)),
           "gcfg_nlinks")


class Segmenter:
    """Reusable one-image pipeline (data term, n-links, exact cut)."""

    def __init__(self, max_w, max_h):
        h = C.c_void_p()
        _check(load().gcfg_seg_create(int(max_w), int(max_h), C.byref(h)), "gcfg_seg_create")
        self.handle = h

    def set_stream(self, stream):
        _check(load().gcfg_seg_set_stream(self.handle, _stream_ptr(stream)), "gcfg_seg_set_stream")

    def run(self, d_rgb, d_scrib, width, height, lam, d_smin=None, d_smax=None) -> dict:
        res = Result()
        _check(load().gcfg_seg_run(self.handle, _ptr(d_rgb), _ptr(d_scrib), int(width), int(height),
                                   float(lam), _ptr(d_smin), _ptr(d_smax), C.byref(res)),
               "gcfg_seg_run")
        return res.as_dict()

    def run_host(self, h_rgb, h_scrib, width, height, lam, h_smin=None, h_smax=None) -> dict:
        res = Result()
        _check(load().gcfg_seg_run_host(self.handle, _ptr(h_rgb), _ptr(h_scrib), int(width),
                                        int(height), float(lam), _ptr(h_smin), _ptr(h_smax),
                                        C.byref(res)), "gcfg_seg_run_host")
        return res.as_dict()

    def close(self):
        if self.handle:
            load().gcfg_seg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver:
    """Many images solved together in one persistent launch (gcfg_batch_*).

    Images are packed back to back, row-major: RGB uint8 (3 bytes/pixel) and
    scribbles uint8 (0 none, 1 fg, 2 bg); outputs are packed the same way."""

    def __init__(self, max_images, max_pixels):
        h = C.c_void_p()
        _check(load().gcfg_batch_create(int(max_images), int(max_pixels), C.byref(h)),
               "gcfg_batch_create")
        self.handle = h
        self._pending = {}  # ticket -> number of images

    def set_stream(self, stream):
        _check(load().gcfg_batch_set_stream(self.handle, _stream_ptr(stream)), "gcfg_batch_set_stream")

    def set_params(self, push_rounds_per_gr, max_tile_sweeps, sweeps_per_local_relabel):
        _check(load().gcfg_batch_set_params(self.handle, int(push_rounds_per_gr), int(max_tile_sweeps),
                                            int(sweeps_per_local_relabel)), "gcfg_batch_set_params")

    def set_graph(self, enable=True):
        """CUDA graph replay of repeated identical batches (gcfg_batch_set_graph)."""
        _check(load().gcfg_batch_set_graph(self.handle, int(bool(enable))), "gcfg_batch_set_graph")

    def graph_info(self) -> dict:
        a = C.c_int()
        c, r, k = C.c_int64(), C.c_int64(), C.c_int64()
        _check(load().gcfg_batch_graph_info(self.handle, C.byref(a), C.byref(c), C.byref(r), C.byref(k)),
               "gcfg_batch_graph_info")
        return {"active": bool(a.value), "captures": c.value, "replays": r.value, "kernels_per_replay": k.value}

    def set_solver(self, push_rounds_per_gr=2, max_tile_sweeps=24, sweeps_per_local_relabel=4,
                   blocks_per_sm=0, local_relabel_first=0, push_only=0, threads_y=0, **_ignored):
        """Solver settings (keys as autotune() returns them); threads_y is the
        solver's block shape 32 x threads_y (4, 8, 16 or 32) over each 32x32 tile,
        0 (the default) by the solve's size: 16 up to 2048 tiles, else 8."""
        t = Tuning(push_rounds_per_gr=int(push_rounds_per_gr), max_tile_sweeps=int(max_tile_sweeps),
                   sweeps_per_local_relabel=int(sweeps_per_local_relabel), blocks_per_sm=int(blocks_per_sm),
                   local_relabel_first=int(local_relabel_first), push_only=int(push_only),
                   threads_y=int(threads_y))
        _check(load().gcfg_batch_set_solver(self.handle, C.byref(t)), "gcfg_batch_set_solver")

    def autotune(self, widths, heights, lambdas, d_rgb, d_scrib, reps=3) -> dict:
        """Pick the solver settings for this batch (gcfg_batch_autotune)."""
        w, h, lam = self._arrays(widths, heights, lambdas)
        t = Tuning()
        _check(load().gcfg_batch_autotune(self.handle, len(w), _ptr(w), _ptr(h), _ptr(lam), _ptr(d_rgb),
                                          _ptr(d_scrib), int(reps), C.byref(t)), "gcfg_batch_autotune")
        return t.as_dict()

    def phase_split(self, widths, heights, lambdas, d_rgb, d_scrib) -> dict:
        """Diagnostic (gcfg_batch_phase_split): the first global relabel and the
        push rounds after it as two separate solver launches, with their device
        times and work counters.  Leaves the solve unfinished."""
        w, h, lam = self._arrays(widths, heights, lambdas)
        out = PhaseSplit()
        _check(load().gcfg_batch_phase_split(self.handle, len(w), _ptr(w), _ptr(h), _ptr(lam), _ptr(d_rgb),
                                             _ptr(d_scrib), C.byref(out)), "gcfg_batch_phase_split")
        return out.as_dict()

    @staticmethod
    def _arrays(widths, heights, lambdas):
        import numpy as np
        w = np.ascontiguousarray(widths, np.int32)
        h = np.ascontiguousarray(heights, np.int32)
        lam = np.ascontiguousarray(lambdas, np.float64)
        return w, h, lam

    def run(self, widths, heights, lambdas, d_rgb, d_scrib, d_smin=None, d_smax=None, results=False):
        """Device-resident batch.  Returns (flows int64[n], results or None)."""
        import numpy as np
        w, h, lam = self._arrays(widths, heights, lambdas)
        n = len(w)
        flows = np.empty(n, np.int64)
        res = (Result * n)() if results else None
        _check(load().gcfg_batch_run(self.handle, n, _ptr(w), _ptr(h), _ptr(lam), _ptr(d_rgb),
                                     _ptr(d_scrib), _ptr(d_smin), _ptr(d_smax), _ptr(flows),
                                     res), "gcfg_batch_run")
        return flows, ([r.as_dict() for r in res] if results else None)

    def run_host(self, widths, heights, lambdas, h_rgb, h_scrib, h_smin=None, h_smax=None,
                 results=False):
        import numpy as np
        w, h, lam = self._arrays(widths, heights, lambdas)
        n = len(w)
        flows = np.empty(n, np.int64)
        res = (Result * n)() if results else None
        _check(load().gcfg_batch_run_host(self.handle, n, _ptr(w), _ptr(h), _ptr(lam), _ptr(h_rgb),
                                          _ptr(h_scrib), _ptr(h_smin), _ptr(h_smax), _ptr(flows),
                                          res), "gcfg_batch_run_host")
        return flows, ([r.as_dict() for r in res] if results else None)

    def submit_host(self, widths, heights, lambdas, h_rgb, h_scrib, h_smin=None, h_smax=None) -> int:
        """Queue a batch from host memory (gcfg_batch_submit_host); returns its
        ticket.  The host arrays must stay alive and unchanged until wait()."""
        w, h, lam = self._arrays(widths, heights, lambdas)
        ticket = C.c_int64(0)
        # the size arrays are read during the call; the pixel buffers later
        _check(load().gcfg_batch_submit_host(self.handle, len(w), _ptr(w), _ptr(h), _ptr(lam), _ptr(h_rgb),
                                             _ptr(h_scrib), _ptr(h_smin), _ptr(h_smax), C.byref(ticket)),
               "gcfg_batch_submit_host")
        self._pending[ticket.value] = len(w)
        return ticket.value

    def wait(self, ticket, results=False):
        """Collect a submitted batch: (flows int64[n], results or None)."""
        import numpy as np
        n = self._pending.pop(ticket, None)
        if n is None:
            raise GcfgError(GCFG_ERR_INVALID, f"gcfg_batch_wait (unknown ticket {ticket})")
        flows = np.empty(n, np.int64)
        res = (Result * n)() if results else None
        _check(load().gcfg_batch_wait(self.handle, ticket, _ptr(flows), res), "gcfg_batch_wait")
        return flows, ([r.as_dict() for r in res] if results else None)

    def close(self):
        if self.handle:
            load().gcfg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Serving
# ---------------------------------------------------------------------------

class ServeConfig(C.Structure):
    _fields_ = [("mem_cap_bytes", C.c_int64), ("lanes", C.c_int32), ("max_batch_images", C.c_int32),
                ("max_batch_tiles", C.c_int64), ("max_sessions", C.c_int32), ("pad", C.c_int32)]


class ServeRequest(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad0", C.c_int32), ("session", C.c_int64), ("w", C.c_int32),
                ("h", C.c_int32), ("lam", C.c_double), ("h_rgb", C.c_void_p), ("h_scrib", C.c_void_p),
                ("edit_x", C.c_int32), ("edit_y", C.c_int32), ("edit_size", C.c_int32),
                ("edit_class", C.c_int32), ("h_smin", C.c_void_p), ("h_smax", C.c_void_p)]


class ServeResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("warm", C.c_int32), ("session", C.c_int64), ("flow", C.c_int64),
                ("batch_images", C.c_int32), ("lane", C.c_int32), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "admitted", "completed", "evicted", "batches",
                                          "bytes_in_use", "sessions", "queued")]


REQ_NEW, REQ_EDIT = 0, 1


def _serve_sigs(lib):
    P = C.c_void_p
    sig = {
        "gcfg_serve_create": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(P)]),
        "gcfg_serve_submit": (C.c_int, [P, C.POINTER(ServeRequest), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)]),
        "gcfg_serve_wait": (C.c_int, [P, C.c_int64, C.POINTER(ServeResult), C.c_int]),
        "gcfg_serve_release": (C.c_int, [P, C.c_int64]),
        "gcfg_serve_get_stats": (C.c_int, [P, C.POINTER(ServeStats)]),
        "gcfg_serve_destroy": (C.c_int, [P]),
        "gcfg_serve_now": (C.c_double, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


EXPORTS += ["gcfg_serve_create", "gcfg_serve_submit", "gcfg_serve_wait", "gcfg_serve_release",
            "gcfg_serve_get_stats", "gcfg_serve_destroy", "gcfg_serve_now"]


class Server:
    """Continuous-batching segmentation server (gcfg_serve_*).

    Host buffers passed to submit_* must stay alive until the request is
    waited for; this object keeps references to them until then."""

    def __init__(self, mem_cap_bytes=60 << 30, lanes=2, max_batch_images=256, max_batch_tiles=1 << 16,
                 max_sessions=4096):
        lib = load()
        if not getattr(lib, "_serve_sigs", False):
            _serve_sigs(lib)
            lib._serve_sigs = True
        cfg = ServeConfig(int(mem_cap_bytes), int(lanes), int(max_batch_images), int(max_batch_tiles),
                          int(max_sessions), 0)
        h = C.c_void_p()
        _check(lib.gcfg_serve_create(C.byref(cfg), C.byref(h)), "gcfg_serve_create")
        self.handle = h
        self._refs = {}

    def _submit(self, req, refs):
        t = C.c_int64()
        sid = C.c_int64()
        _check(load().gcfg_serve_submit(self.handle, C.byref(req), C.byref(t), C.byref(sid)),
               "gcfg_serve_submit")
        self._refs[t.value] = refs
        return t.value, sid.value

    def submit_new(self, rgb, scrib, lam, smin=None, smax=None):
        """Returns (ticket, session).  rgb: uint8 [H, W, 3], scrib: uint8 [H, W]."""
        H, W = scrib.shape
        req = ServeRequest(kind=REQ_NEW, w=W, h=H, lam=float(lam), h_rgb=_ptr(rgb).value,
                           h_scrib=_ptr(scrib).value,
                           h_smin=None if smin is None else _ptr(smin).value,
                           h_smax=None if smax is None else _ptr(smax).value)
        return self._submit(req, (rgb, scrib, smin, smax))

    def submit_edit(self, session, x, y, size, cls, smin=None, smax=None):
        req = ServeRequest(kind=REQ_EDIT, session=int(session), edit_x=int(x), edit_y=int(y),
                           edit_size=int(size), edit_class=int(cls),
                           h_smin=None if smin is None else _ptr(smin).value,
                           h_smax=None if smax is None else _ptr(smax).value)
        return self._submit(req, (smin, smax))

    def wait(self, ticket, timeout_ms=-1) -> dict:
        res = ServeResult()
        load().gcfg_serve_wait(self.handle, int(ticket), C.byref(res), int(timeout_ms))
        self._refs.pop(ticket, None)
        return res.as_dict()

    def release(self, session):
        _check(load().gcfg_serve_release(self.handle, int(session)), "gcfg_serve_release")

    def stats(self) -> dict:
        st = ServeStats()
        _check(load().gcfg_serve_get_stats(self.handle, C.byref(st)), "gcfg_serve_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    @staticmethod
    def now() -> float:
        lib = load()
        if not getattr(lib, "_serve_sigs", False):
            _serve_sigs(lib)
            lib._serve_sigs = True
        return lib.gcfg_serve_now()

    def close(self):
        if self.handle:
            load().gcfg_serve_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# DataTerm (DataTerm.h:9-19): gcfg_dt_* handle and the reference's names
# ---------------------------------------------------------------------------

EXPORTS += ["gcfg_dt_create", "gcfg_dt_destroy", "gcfg_dt_set_stream", "gcfg_dt_set_image",
            "gcfg_dt_set_image_device", "gcfg_dt_set_selection", "gcfg_dt_set_scribbles_device",
            "gcfg_dt_reset", "gcfg_dt_select_on_map", "gcfg_dt_set_sigma", "gcfg_dt_compute",
            "gcfg_dt_pos", "gcfg_dt_neg", "gcfg_dt_image", "gcfg_dt_selection",
            "gcfg_dt_draw_selection", "gcfg_dt_nlinks", "gcfg_dt_set_model", "gcfg_dt_kde_table"]

GCFG_DT_HISTOGRAM = 0
GCFG_DT_KDE = 1


def _dt_lib():
    lib = load()
    if not getattr(lib, "_dt_sigs", False):
        P = C.c_void_p
        sig = {
            "gcfg_dt_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(P)]),
            "gcfg_dt_destroy": (C.c_int, [P]),
            "gcfg_dt_set_stream": (C.c_int, [P, P]),
            "gcfg_dt_set_image": (C.c_int, [P, P]),
            "gcfg_dt_set_image_device": (C.c_int, [P, P]),
            "gcfg_dt_set_selection": (C.c_int, [P, P]),
            "gcfg_dt_set_scribbles_device": (C.c_int, [P, P]),
            "gcfg_dt_reset": (C.c_int, [P]),
            "gcfg_dt_select_on_map": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
            "gcfg_dt_set_sigma": (C.c_int, [P, C.c_int]),
            "gcfg_dt_compute": (C.c_int, [P]),
            "gcfg_dt_pos": (P, [P]),
            "gcfg_dt_neg": (P, [P]),
            "gcfg_dt_image": (P, [P]),
            "gcfg_dt_selection": (P, [P]),
            "gcfg_dt_draw_selection": (C.c_int, [P, P, P]),
            "gcfg_dt_nlinks": (C.c_int, [P, C.c_double, P, P, P, P]),
            "gcfg_dt_set_model": (C.c_int, [P, C.c_int]),
            "gcfg_dt_kde_table": (C.c_int, [P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        lib._dt_sigs = True
    return lib


class DeviceArray:
    """A device array owned by the library, seen through
    __cuda_array_interface__ (torch.as_tensor(a, device="cuda") is a view)."""

    def __init__(self, ptr, n, typestr):
        self.ptr, self.n, self.typestr = int(ptr or 0), int(n), typestr

    def data_ptr(self):
        return self.ptr

    @property
    def __cuda_array_interface__(self):
        return {"shape": (self.n,), "typestr": self.typestr, "data": (self.ptr, False), "version": 2}


class DataTermState:
    """gcfg_dt_* handle: image, selection map and t-link arrays of one image."""

    def __init__(self, width, height):
        lib = _dt_lib()
        h = C.c_void_p()
        _check(lib.gcfg_dt_create(int(width), int(height), C.byref(h)), "gcfg_dt_create")
        self.handle, self.width, self.height = h, int(width), int(height)

    def _lib(self):
        if not self.handle:
            raise GcfgError(GCFG_ERR_STATE, "DataTerm used after free")
        return _dt_lib()

    def set_stream(self, stream):
        _check(self._lib().gcfg_dt_set_stream(self.handle, _stream_ptr(stream)), "gcfg_dt_set_stream")

    def set_image(self, h_img):
        a = np.ascontiguousarray(h_img, dtype=np.uint8)
        assert a.size == 3 * self.width * self.height
        _check(self._lib().gcfg_dt_set_image(self.handle, _ptr(a)), "gcfg_dt_set_image")

    def set_image_device(self, d_img):
        _check(self._lib().gcfg_dt_set_image_device(self.handle, _ptr(d_img)), "gcfg_dt_set_image_device")

    def set_selection(self, h_select):
        a = np.ascontiguousarray(h_select, dtype=np.int32)
        assert a.size == self.width * self.height
        _check(self._lib().gcfg_dt_set_selection(self.handle, _ptr(a)), "gcfg_dt_set_selection")

    def set_scribbles_device(self, d_scrib):
        _check(self._lib().gcfg_dt_set_scribbles_device(self.handle, _ptr(d_scrib)),
               "gcfg_dt_set_scribbles_device")

    def reset(self):
        _check(self._lib().gcfg_dt_reset(self.handle), "gcfg_dt_reset")

    def select_on_map(self, x, y, cls=1):
        _check(self._lib().gcfg_dt_select_on_map(self.handle, int(x), int(y), int(cls)),
               "gcfg_dt_select_on_map")

    def set_sigma(self, sigma):
        _check(self._lib().gcfg_dt_set_sigma(self.handle, int(sigma)), "gcfg_dt_set_sigma")

    def set_model(self, model):
        """'histogram' (default) or 'kde' (the reference's kernel density)."""
        m = {"histogram": GCFG_DT_HISTOGRAM, "kde": GCFG_DT_KDE}.get(model, model)
        _check(self._lib().gcfg_dt_set_model(self.handle, int(m)), "gcfg_dt_set_model")

    def kde_table(self):
        g = np.empty(101, np.float32)
        _check(self._lib().gcfg_dt_kde_table(self.handle, _ptr(g)), "gcfg_dt_kde_table")
        return g

    def compute(self):
        _check(self._lib().gcfg_dt_compute(self.handle), "gcfg_dt_compute")

    def pos(self) -> DeviceArray:
        return DeviceArray(self._lib().gcfg_dt_pos(self.handle), self.width * self.height, "<i4")

    def neg(self) -> DeviceArray:
        return DeviceArray(self._lib().gcfg_dt_neg(self.handle), self.width * self.height, "<i4")

    def image(self) -> DeviceArray:
        return DeviceArray(self._lib().gcfg_dt_image(self.handle), 3 * self.width * self.height, "|u1")

    def selection(self) -> DeviceArray:
        return DeviceArray(self._lib().gcfg_dt_selection(self.handle), self.width * self.height, "|u1")

    def draw_selection(self, h_in, h_out=None):
        a = np.ascontiguousarray(h_in, dtype=np.uint8)
        out = np.empty_like(a) if h_out is None else h_out
        _check(self._lib().gcfg_dt_draw_selection(self.handle, _ptr(a), _ptr(out)), "gcfg_dt_draw_selection")
        return out

    def nlinks(self, lam, d_up, d_down, d_left, d_right):
        _check(self._lib().gcfg_dt_nlinks(self.handle, float(lam), _ptr(d_up), _ptr(d_down), _ptr(d_left),
                                          _ptr(d_right)), "gcfg_dt_nlinks")

    def close(self):
        if self.handle:
            _dt_lib().gcfg_dt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DataTerm:
    """The reference's DataTerm namespace (one process-wide state,
    DataTerm.h:7-39) with its function names."""

    _state = None
    width = 0
    height = 0

    @classmethod
    def _s(cls) -> DataTermState:
        if cls._state is None:
            raise GcfgError(GCFG_ERR_STATE, "DataTerm.init_data_term was not called")
        return cls._state

    @classmethod
    def init_data_term(cls, w, h):
        if cls._state is not None:
            cls._state.close()
        cls._state = DataTermState(w, h)
        cls.width, cls.height = int(w), int(h)

    @classmethod
    def free_data_term(cls):
        cls._s().close()
        cls._state = None

    @classmethod
    def setImage(cls, h_img):
        cls._s().set_image(h_img)

    @classmethod
    def setSelection(cls, h_select):
        cls._s().set_selection(h_select)

    @classmethod
    def reset(cls):
        cls._s().reset()

    @classmethod
    def selectOnMap(cls, x, y, sigma=None):
        cls._s().select_on_map(x, y, 1)

    @classmethod
    def selectBackgroundOnMap(cls, x, y):
        cls._s().select_on_map(x, y, 2)

    @classmethod
    def drawSelection(cls, inp, out=None):
        return cls._s().draw_selection(inp, out)

    @classmethod
    def getDataTermsMixture(cls):
        cls._s().compute()

    @classmethod
    def setSigmaGaussian(cls, sigma):
        cls._s().set_sigma(sigma)

    @classmethod
    def useKernelDensity(cls, on=True):
        """The reference's own colour model instead of the histogram pair."""
        cls._s().set_model("kde" if on else "histogram")

    @classmethod
    def getPos(cls) -> DeviceArray:
        return cls._s().pos()

    @classmethod
    def getNeg(cls) -> DeviceArray:
        return cls._s().neg()


# ---------------------------------------------------------------------------
# 8-neighbourhood graphs (the reference built with NEIGHBORHOOD == 8)
# ---------------------------------------------------------------------------

class GlobalWrapper8:
    """Handle of one 8-connected residual graph."""

    def __init__(self, handle, width, height, keep):
        self.handle, self.width, self.height, self._keep = handle, width, height, keep


def GC_Init8(width, height, data_positive=None, data_negative=None, penalty=0, up=None, down=None, left=None,
             right=None, upleft=None, upright=None, downleft=None, downright=None):
    """GC_Init of the reference built with NEIGHBORHOOD == 8
    (GraphCut.cu:187-194): four straight and four diagonal capacity arrays
    (device int32 W*H, torch tensors) or a constant penalty."""
    arrs = (up, down, left, right, upleft, upright, downleft, downright)
    h = C.c_void_p()
    _check(load().gcfg_init8(int(width), int(height), _ptr(data_positive), _ptr(data_negative), int(penalty),
                             *[_ptr(a) for a in arrs], C.byref(h)), "gcfg_init8")
    return GlobalWrapper8(h, width, height, [data_positive, data_negative, *arrs])


def GC_Optimize8(gw, label=None) -> dict:
    res = Result()
    _check(load().gcfg_optimize8(gw.handle, _ptr(label), C.byref(res)), "gcfg_optimize8")
    return res.as_dict()


def GC_SetSchedule8(gw, rounds_per_gr, blocks_per_sm=0):
    _check(load().gcfg_set_schedule8(gw.handle, int(rounds_per_gr), int(blocks_per_sm)), "gcfg_set_schedule8")


def GC_SetGraph8(gw):
    _check(load().gcfg_set_graph8(gw.handle), "gcfg_set_graph8")


def GC_GetCuts8(gw, smin=None, smax=None):
    _check(load().gcfg_get_cuts8(gw.handle, _ptr(smin), _ptr(smax)), "gcfg_get_cuts8")


def GC_End8(gw):
    if gw.handle:
        load().gcfg_end8(gw.handle)
        gw.handle = None
