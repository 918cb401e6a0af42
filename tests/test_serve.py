"""Serving: continuous batching with resident images and warm edits.

Each served result (new image or scribble edit, solved in a mix with other
requests) must equal the solve of the same input alone, bit for bit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import gcfg  # noqa: E402
import oracle as O  # noqa: E402
import synth  # noqa: E402

TILE_BYTES = 25496 + 1024 * 6  # device bytes a resident image uses per 32x32 tile


def _alone(rgb, scrib, lam):
    H, W = scrib.shape
    seg = gcfg.Segmenter(W, H)
    smin = np.zeros((H, W), np.uint8)
    smax = np.zeros((H, W), np.uint8)
    r = seg.run_host(rgb, scrib, W, H, lam, smin, smax)
    seg.close()
    return r["flow"], smin, smax


def test_served_results_equal_alone():
    rng = np.random.default_rng(44)
    server = gcfg.Server(mem_cap_bytes=2 << 30, lanes=2, max_batch_images=64, max_batch_tiles=4096,
                         max_sessions=128)
    pending = []
    sessions = []  # (session, rgb, current scribbles, lam)
    # inputs first, so that the requests arrive faster than they are solved
    shapes = [tuple(int(v) for v in rng.integers(40, 420, 2)) for _ in range(24)]
    inputs = [synth.generate(4, W, H, 700 + i) for i, (W, H) in enumerate(shapes)]
    for i in range(24):
        rgb, scrib = inputs[i]
        H, W = scrib.shape
        lam = float((10.0, 50.0, 200.0)[i % 3])
        smin = np.zeros((H, W), np.uint8)
        smax = np.zeros((H, W), np.uint8)
        t, sid = server.submit_new(rgb, scrib, lam, smin, smax)
        pending.append((t, False, rgb, scrib.copy(), lam, smin, smax))
        sessions.append([sid, rgb, scrib.copy(), lam])
        if i % 2 == 1:
            # a scribble edit of an earlier image, queued before it may be solved
            k = int(rng.integers(0, len(sessions)))
            sid2, rgb2, sc2, lam2 = sessions[k]
            Hh, Ww = sc2.shape
            x, y = int(rng.integers(0, max(1, Ww - 15))), int(rng.integers(0, max(1, Hh - 15)))
            cls = int(rng.integers(1, 3))
            sc2 = sc2.copy()
            sc2[y:y + 15, x:x + 15] = cls
            sessions[k][2] = sc2
            smin2 = np.zeros((Hh, Ww), np.uint8)
            smax2 = np.zeros((Hh, Ww), np.uint8)
            t2, _ = server.submit_edit(sid2, x, y, 15, cls, smin2, smax2)
            pending.append((t2, True, rgb2, sc2.copy(), lam2, smin2, smax2))
    results = [server.wait(t, timeout_ms=120000) for t, *_ in pending]
    assert max(r["batch_images"] for r in results) > 1, "requests were never batched together"
    for (t, warm, rgb, scrib, lam, smin, smax), r in zip(pending, results):
        assert r["status"] == gcfg.GCFG_OK
        assert r["warm"] == int(warm)
        flow, amin, amax = _alone(rgb, scrib, lam)
        assert r["flow"] == flow
        assert np.array_equal(smin, amin) and np.array_equal(smax, amax)
    # and a few against the CPU oracle
    for (t, warm, rgb, scrib, lam, smin, smax), r in list(zip(pending, results))[:6]:
        o = O.segment(rgb, scrib, lam)
        assert r["flow"] == o["flow"] and np.array_equal(smax, o["smax"]) and np.array_equal(smin, o["smin"])
    st = server.stats()
    assert st["completed"] == len(pending) and st["queued"] == 0
    server.close()


def test_admission_cap_eviction_and_refusal():
    cap = 40 * TILE_BYTES  # room for two 128x128 images (16 tiles each)
    server = gcfg.Server(mem_cap_bytes=cap, lanes=2, max_batch_images=8, max_batch_tiles=64, max_sessions=16)
    imgs = [synth.generate(4, 128, 128, 900 + i) for i in range(8)]
    tickets = [server.submit_new(rgb, scrib, 50.0) for rgb, scrib in imgs]
    res = [server.wait(t, timeout_ms=120000) for t, _ in tickets]
    for (rgb, scrib), r in zip(imgs, res):
        assert r["status"] == gcfg.GCFG_OK
        assert r["flow"] == _alone(rgb, scrib, 50.0)[0]
    st = server.stats()
    assert st["evicted"] >= 6 and st["bytes_in_use"] <= cap
    # the first images were evicted: editing them is refused
    with pytest.raises(gcfg.GcfgError) as ei:
        server.submit_edit(tickets[0][1], 5, 5, 15, 1)
    assert ei.value.status == gcfg.GCFG_ERR_STATE
    # an image that could never fit under the cap is refused at submission
    big_rgb, big_scrib = synth.generate(4, 300, 300, 990)
    with pytest.raises(gcfg.GcfgError) as ei:
        server.submit_new(big_rgb, big_scrib, 50.0)
    assert ei.value.status == gcfg.GCFG_ERR_CAPACITY
    server.close()
