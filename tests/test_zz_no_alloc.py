"""The allocation-free solve against the regular graph entry points.

gcfg_solve_noalloc is for callers that cannot allocate device memory when
they solve: a host framework that owns all of the GPU's memory and forbids
its plug-ins to call cudaMalloc, a process already at its device-memory
limit, or a latency-bound loop that cannot afford the device-wide
synchronisation cudaMalloc/cudaFree can cause.  Its working memory is a fixed
16 MiB device array inside the library, so it accepts images of at most 640
tiles of 32x32 pixels.  Called through the C ABI, it must return exactly the
labels and the flow value of gcfg_init + gcfg_optimize, call after call (the
array keeps the previous call's contents), and repeated calls must leave the
device's free memory unchanged.

The tests here pass alone in a fresh process as well as after the others; the
file name only makes pytest collect it last, so that a run that stops at its
first failure (pytest -x) has already run every other test if one of these
fails.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import gcfg  # noqa: E402


def _instance(seed, H, W, arrays):
    rng = np.random.default_rng(seed)
    dp = rng.integers(0, 300, (H, W)).astype(np.int32)
    dn = rng.integers(0, 300, (H, W)).astype(np.int32)
    if arrays:
        kw = {k: rng.integers(0, 120, (H, W)).astype(np.int32) for k in ("up", "down", "left", "right")}
        return dp, dn, 0, kw
    return dp, dn, int(rng.integers(1, 150)), {}


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _existing(dp, dn, penalty, kw):
    """Labels and flow from gcfg_init + gcfg_optimize (the regular path)."""
    H, W = dp.shape
    t = [_dev(dp), _dev(dn)] + [_dev(kw[k]) if kw else None for k in ("up", "down", "left", "right")]
    gw = gcfg.GC_Init(W, H, t[0], t[1], penalty, *t[2:])
    label = np.zeros((H, W), np.int32)
    res = gcfg.GC_Optimize(gw, label)
    gcfg.GC_End(gw)
    return label, res["flow"]


def _noalloc(dp, dn, penalty, kw):
    """Labels and flow from gcfg_solve_noalloc through the C ABI."""
    H, W = dp.shape
    t = [_dev(dp), _dev(dn)] + [_dev(kw[k]) if kw else None for k in ("up", "down", "left", "right")]
    label = torch.full((H, W), -7, dtype=torch.int32, device="cuda")  # poisoned: every pixel is written
    flow = C.c_int64(-1)
    ptr = [None if x is None else C.c_void_p(x.data_ptr()) for x in t]
    rc = gcfg.load().gcfg_solve_noalloc(W, H, ptr[0], ptr[1], penalty, *ptr[2:],
                                        C.c_void_p(label.data_ptr()), C.byref(flow), None)
    assert rc == gcfg.GCFG_OK, gcfg.strerror(rc)
    return label.cpu().numpy(), flow.value


def test_noalloc_matches_regular_solve_on_consecutive_calls():
    cases = [_instance(11, 200, 300, arrays=True),      # 70 tiles, per-direction capacities
             _instance(12, 389, 517, arrays=False),     # 221 tiles, constant penalty
             _instance(13, 640, 1024, arrays=True)]     # exactly the 640-tile limit
    for dp, dn, penalty, kw in cases:
        ref_label, ref_flow = _existing(dp, dn, penalty, kw)
        label, flow = _noalloc(dp, dn, penalty, kw)
        assert flow == ref_flow
        assert np.array_equal(label, ref_label)


def test_noalloc_refuses_images_beyond_its_working_memory():
    small = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = C.c_void_p(small.data_ptr())
    lib = gcfg.load()
    # 1025 x 640 needs 33 x 20 = 660 tiles > 640: refused before any GPU work
    rc = lib.gcfg_solve_noalloc(1025, 640, p, p, 5, None, None, None, None, p, None, None)
    assert rc == gcfg.GCFG_ERR_TOO_LARGE
    assert "allocation-free" in gcfg.strerror(rc)


def test_noalloc_repeated_calls_leave_free_device_memory_unchanged():
    dp, dn, penalty, kw = _instance(14, 300, 400, arrays=True)
    H, W = dp.shape
    t = [_dev(dp), _dev(dn)] + [_dev(kw[k]) for k in ("up", "down", "left", "right")]
    label = torch.empty((H, W), dtype=torch.int32, device="cuda")
    ptr = [C.c_void_p(x.data_ptr()) for x in t]
    lab = C.c_void_p(label.data_ptr())
    lib = gcfg.load()
    flows = []

    def call():
        flow = C.c_int64(-1)
        rc = lib.gcfg_solve_noalloc(W, H, ptr[0], ptr[1], penalty, *ptr[2:], lab, C.byref(flow), None)
        assert rc == gcfg.GCFG_OK, gcfg.strerror(rc)
        flows.append(flow.value)

    call()  # the first call may load the library's device code and its array
    torch.cuda.synchronize()
    first = label.cpu().numpy()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert len(set(flows)) == 1
    assert np.array_equal(label.cpu().numpy(), first)
