"""Host-side checks of the harness that runs the reference's CUDA path (no GPU
needed): the driver library builds from this repository's source alone, loads,
exports its two entry points, refuses to solve before the reference's kernels
are loaded, and reports plainly when they were never compiled."""
import ctypes as C
import os

import numpy as np

import ref_cuda


def test_driver_builds_and_exports():
    path = ref_cuda.build()
    lib = C.CDLL(path)
    assert hasattr(lib, "refgpu_load") and hasattr(lib, "refgpu_solve")


def test_solve_before_load_is_refused():
    lib = C.CDLL(ref_cuda.build())
    P = C.c_void_p
    lib.refgpu_solve.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, P, P, P, C.c_longlong, C.c_double,
                                 C.POINTER(ref_cuda.Stats)]
    dp = np.zeros((4, 4), np.int32)
    label = np.zeros((4, 4), np.int32)
    st = ref_cuda.Stats()
    p = dp.ctypes.data_as(P)
    rc = lib.refgpu_solve(4, 4, p, p, 0, None, None, None, None, label.ctypes.data_as(P), 10, 1.0, C.byref(st))
    assert ref_cuda.STATUS[rc] == "kernels not loaded"


def test_missing_kernels_are_reported(monkeypatch, tmp_path):
    monkeypatch.setattr(ref_cuda, "CUBIN", os.path.join(str(tmp_path), "absent.cubin"))
    why = ref_cuda.unavailable()
    assert why and "not compiled" in why


def test_stats_layout_matches_the_driver():
    # refgpu_stats: 4 x int64, 4 x int32, 4 x double
    assert C.sizeof(ref_cuda.Stats) == 4 * 8 + 4 * 4 + 4 * 8
