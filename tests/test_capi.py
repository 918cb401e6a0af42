"""C ABI checks that need no GPU: the library builds, loads, and exports
every entry point include/gcfg.h declares."""
import os
import re
import subprocess

import pytest

import gcfg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:gcfg_status|const char|int64_t|int32_t|uint8_t|double)\s*\*?\s*(gcfg_\w+)\s*\(", src, re.M)))


def test_header_matches_binding_list():
    assert _declared("gcfg.h") == sorted(gcfg.EXPORTS)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(gcfg.LIB_PATH):
        pytest.skip("libgcfg.so not built")
    out = subprocess.run(["nm", "-D", "--defined-only", gcfg.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (gcfg_\w+)", out))
    missing = [s for s in _declared("gcfg.h") if s not in exported]
    assert not missing, missing


def test_library_loads_without_gpu():
    if not os.path.exists(gcfg.LIB_PATH):
        pytest.skip("libgcfg.so not built")
    lib = gcfg.load()
    assert lib.gcfg_strerror(0) == b"ok"
    assert gcfg.strerror(gcfg.GCFG_ERR_INVALID) == "invalid argument"
    assert isinstance(gcfg.launch_count(), int)


def test_invalid_arguments_rejected_on_host():
    """Argument checks happen before any device work."""
    if not os.path.exists(gcfg.LIB_PATH):
        pytest.skip("libgcfg.so not built")
    lib = gcfg.load()
    import ctypes as C
    h = C.c_void_p()
    assert lib.gcfg_init(0, 10, None, None, 0, None, None, None, None, C.byref(h)) == gcfg.GCFG_ERR_INVALID
    assert lib.gcfg_init(10, 10, None, None, -1, None, None, None, None, C.byref(h)) == gcfg.GCFG_ERR_INVALID
    assert lib.gcfg_set_graph(None) == gcfg.GCFG_ERR_INVALID
    assert lib.gcfg_seg_create(0, 5, C.byref(h)) == gcfg.GCFG_ERR_INVALID
