"""Asynchronous host entry point (gcfg_batch_submit_host / gcfg_batch_wait):
two batches in flight give the same flows and labels as the synchronous
gcfg_batch_run_host, and the in-flight rules are enforced."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import gcfg  # noqa: E402
import synth  # noqa: E402


def _batch(n, seed0, lo=48, hi=400):
    shapes = [(W, H) for (W, H, _) in synth.batch_shapes(n, seed0, lo=lo, hi=hi)]
    rgb, scrib, _ = synth.generate_packed([(3, W, H, seed0 + i) for i, (W, H) in enumerate(shapes)])
    Ws = np.array([w for w, _ in shapes], np.int32)
    Hs = np.array([h for _, h in shapes], np.int32)
    lams = np.array([(10.0, 50.0, 200.0)[i % 3] for i in range(n)])
    return Ws, Hs, lams, rgb, scrib


def _pinned(a):
    return torch.from_numpy(a).pin_memory().numpy()


def _sync_ref(bs, b):
    Ws, Hs, lams, rgb, scrib = b
    h_min = np.zeros(scrib.size, np.uint8)
    h_max = np.zeros(scrib.size, np.uint8)
    flows, _ = bs.run_host(Ws, Hs, lams, rgb, scrib, h_min, h_max)
    return flows, h_min, h_max


def test_two_in_flight_equal_sync():
    batches = [_batch(24, 5100), _batch(7, 5200), _batch(31, 5300, lo=32, hi=600)]
    bs = gcfg.BatchSolver(32, max(b[4].size for b in batches))
    refs = [_sync_ref(bs, b) for b in batches]
    ins = [(_pinned(b[3]), _pinned(b[4])) for b in batches]
    # six batches, alternating sizes, two in flight at a time
    order = [0, 1, 2, 0, 2, 1]
    outs = [(_pinned(np.full(batches[k][4].size, 9, np.uint8)), _pinned(np.full(batches[k][4].size, 9, np.uint8)))
            for k in order]
    pending = []
    for j, k in enumerate(order):
        Ws, Hs, lams, _, _ = batches[k]
        t = bs.submit_host(Ws, Hs, lams, ins[k][0], ins[k][1], outs[j][0], outs[j][1])
        pending.append((t, j, k))
        if len(pending) == 2:
            t0, j0, k0 = pending.pop(0)
            flows, res = bs.wait(t0, results=True)
            assert np.array_equal(flows, refs[k0][0])
            assert all(r["status"] == 0 for r in res)
            assert np.array_equal(outs[j0][0], refs[k0][1]) and np.array_equal(outs[j0][1], refs[k0][2])
    for t0, j0, k0 in pending:
        flows, _ = bs.wait(t0)
        assert np.array_equal(flows, refs[k0][0])
        assert np.array_equal(outs[j0][0], refs[k0][1]) and np.array_equal(outs[j0][1], refs[k0][2])
    # the synchronous path still works afterwards
    assert np.array_equal(_sync_ref(bs, batches[1])[0], refs[1][0])
    bs.close()


def test_in_flight_rules():
    b1, b2 = _batch(5, 5400), _batch(6, 5500)
    bs = gcfg.BatchSolver(8, max(b1[4].size, b2[4].size))
    r1, r2 = _sync_ref(bs, b1), _sync_ref(bs, b2)
    i1 = (_pinned(b1[3]), _pinned(b1[4]))
    i2 = (_pinned(b2[3]), _pinned(b2[4]))
    o1 = (_pinned(np.zeros(b1[4].size, np.uint8)), _pinned(np.zeros(b1[4].size, np.uint8)))
    o2 = (_pinned(np.zeros(b2[4].size, np.uint8)), _pinned(np.zeros(b2[4].size, np.uint8)))
    t1 = bs.submit_host(*b1[:3], *i1, *o1)
    t2 = bs.submit_host(*b2[:3], *i2, *o2)
    assert t2 != t1
    # a third batch, a synchronous run and a stream change are refused
    with pytest.raises(gcfg.GcfgError) as ei:
        bs.submit_host(*b1[:3], *i1, *o1)
    assert ei.value.status == gcfg.GCFG_ERR_STATE
    with pytest.raises(gcfg.GcfgError) as ei:
        _sync_ref(bs, b1)
    assert ei.value.status == gcfg.GCFG_ERR_STATE
    with pytest.raises(gcfg.GcfgError) as ei:
        bs.set_stream(torch.cuda.current_stream())
    assert ei.value.status == gcfg.GCFG_ERR_STATE
    with pytest.raises(gcfg.GcfgError) as ei:
        bs.wait(t2 + 100)
    assert ei.value.status == gcfg.GCFG_ERR_INVALID
    # collected out of order
    f2, _ = bs.wait(t2)
    f1, _ = bs.wait(t1)
    assert np.array_equal(f1, r1[0]) and np.array_equal(f2, r2[0])
    assert np.array_equal(o1[0], r1[1]) and np.array_equal(o1[1], r1[2])
    assert np.array_equal(o2[0], r2[1]) and np.array_equal(o2[1], r2[2])
    # a collected ticket is gone
    with pytest.raises(gcfg.GcfgError):
        bs.wait(t1)
    # labels are optional
    t = bs.submit_host(*b2[:3], *i2)
    assert np.array_equal(bs.wait(t)[0], r2[0])
    bs.close()


def test_two_in_flight_graph_replay():
    """With CUDA graphs on, each run set replays its own captured graph;
    results equal the blocking call across alternating batch sizes."""
    batches = [_batch(20, 5600), _batch(9, 5700)]
    bs = gcfg.BatchSolver(32, max(b[4].size for b in batches))
    refs = [_sync_ref(bs, b) for b in batches]
    bs.set_graph(True)
    ins = [(_pinned(b[3]), _pinned(b[4])) for b in batches]
    order = [0, 0, 0, 1, 1, 0, 0, 0, 0]
    outs = [(_pinned(np.zeros(batches[k][4].size, np.uint8)), _pinned(np.zeros(batches[k][4].size, np.uint8)))
            for k in order]
    pending = []
    for j, k in enumerate(order):
        Ws, Hs, lams, _, _ = batches[k]
        pending.append((bs.submit_host(Ws, Hs, lams, ins[k][0], ins[k][1], outs[j][0], outs[j][1]), j, k))
        if len(pending) == 2:
            t0, j0, k0 = pending.pop(0)
            assert np.array_equal(bs.wait(t0)[0], refs[k0][0])
            assert np.array_equal(outs[j0][0], refs[k0][1]) and np.array_equal(outs[j0][1], refs[k0][2])
    for t0, j0, k0 in pending:
        assert np.array_equal(bs.wait(t0)[0], refs[k0][0])
        assert np.array_equal(outs[j0][0], refs[k0][1]) and np.array_equal(outs[j0][1], refs[k0][2])
    info = bs.graph_info()
    assert info["active"] and info["replays"] >= len(order) - 4
    bs.close()
