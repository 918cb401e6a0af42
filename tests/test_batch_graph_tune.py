"""Batch API: CUDA graph replay and the autotuner change no result."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import gcfg  # noqa: E402
import synth  # noqa: E402


def _batch(n, seed0):
    shapes = [(W, H) for (W, H, _) in synth.batch_shapes(n, seed0, lo=48, hi=400)]
    rgb, scrib, offs = synth.generate_packed([(3, W, H, seed0 + i) for i, (W, H) in enumerate(shapes)])
    Ws = np.array([w for w, _ in shapes], np.int32)
    Hs = np.array([h for _, h in shapes], np.int32)
    lams = np.array([(10.0, 50.0, 200.0)[i % 3] for i in range(n)])
    return Ws, Hs, lams, rgb, scrib


def _run(bs, Ws, Hs, lams, d_rgb, d_scrib):
    n_px = int(np.sum(Ws.astype(np.int64) * Hs))
    smin = torch.empty(n_px, dtype=torch.uint8, device="cuda")
    smax = torch.empty(n_px, dtype=torch.uint8, device="cuda")
    flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, smax)
    return flows, smin.cpu().numpy(), smax.cpu().numpy()


def test_graph_replay_equals_eager():
    Ws, Hs, lams, rgb, scrib = _batch(40, 3100)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(64, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    bs.set_graph(True)
    n_px = scrib.size
    smin = torch.empty(n_px, dtype=torch.uint8, device="cuda")
    smax = torch.empty(n_px, dtype=torch.uint8, device="cuda")
    l0 = gcfg.launch_count()
    for _ in range(3):
        smin.fill_(7)
        smax.fill_(7)
        flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, smax)
        assert np.array_equal(flows, ref[0])
        assert np.array_equal(smin.cpu().numpy(), ref[1]) and np.array_equal(smax.cpu().numpy(), ref[2])
    info = bs.graph_info()
    assert info["active"], "stream capture of the batch pipeline failed"
    assert info["captures"] == 1 and info["replays"] == 3 and info["kernels_per_replay"] >= 5
    assert gcfg.launch_count() - l0 == 3 * info["kernels_per_replay"]
    # other lambdas: recaptured, and equal to an eager run
    lams2 = lams[::-1].copy()
    flows2, _ = bs.run(Ws, Hs, lams2, d_rgb, d_scrib, smin, smax)
    assert bs.graph_info()["captures"] == 2
    bs.set_graph(False)
    assert np.array_equal(flows2, _run(bs, Ws, Hs, lams2, d_rgb, d_scrib)[0])
    # host entry point through the graph
    bs.set_graph(True)
    h_min = np.zeros(n_px, np.uint8)
    h_max = np.zeros(n_px, np.uint8)
    for _ in range(2):
        fh, _ = bs.run_host(Ws, Hs, lams, rgb, scrib, h_min, h_max)
        assert np.array_equal(fh, ref[0]) and np.array_equal(h_min, ref[1]) and np.array_equal(h_max, ref[2])
    # device and host runs alternating: both graphs stay cached, results unchanged
    bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, smax)
    c0 = bs.graph_info()["captures"]
    for _ in range(3):
        flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, smax)
        fh, _ = bs.run_host(Ws, Hs, lams, rgb, scrib, h_min, h_max)
        assert np.array_equal(flows, ref[0]) and np.array_equal(fh, ref[0])
        assert np.array_equal(smin.cpu().numpy(), ref[1]) and np.array_equal(h_max, ref[2])
    assert bs.graph_info()["captures"] == c0
    # a different batch in between: its layout is uploaded again before a replay
    Ws3, Hs3 = Ws[:10].copy(), Hs[:10].copy()
    n3 = int(np.sum(Ws3.astype(np.int64) * Hs3))
    f3, _ = bs.run(Ws3, Hs3, lams[:10], d_rgb, d_scrib, smin[:n3], smax[:n3])
    flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, smax)
    assert np.array_equal(flows, ref[0]) and np.array_equal(f3, ref[0][:10])
    bs.close()


def test_autotune_keeps_results():
    Ws, Hs, lams, rgb, scrib = _batch(48, 3300)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(64, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    t = bs.autotune(Ws, Hs, lams, d_rgb, d_scrib, reps=2)
    assert t["configs_tried"] >= 10
    assert t["push_rounds_per_gr"] in (2, 4, 8, 16) and t["max_tile_sweeps"] in (16, 32, 64, 128)
    assert t["sweeps_per_local_relabel"] in (2, 4, 8, 16, 32, 64) and 1 <= t["blocks_per_sm"] <= 8
    assert t["local_relabel_first"] in (0, 1) and t["push_only"] in (0, 1)
    assert t["ms_best"] <= t["ms_default"] and (t["tile_w"], t["tile_h"]) == (32, 32)
    got = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    bs.close()


@pytest.mark.parametrize("settings", [
    dict(push_only=1, sweeps_per_local_relabel=4),
    dict(push_only=1, sweeps_per_local_relabel=32, max_tile_sweeps=16),
    dict(push_only=1, local_relabel_first=1, push_rounds_per_gr=2),
    dict(push_only=0, local_relabel_first=1, sweeps_per_local_relabel=2, blocks_per_sm=2),
    dict(push_only=0, push_rounds_per_gr=16, max_tile_sweeps=128, blocks_per_sm=1),
])
def test_solver_settings_do_not_change_results(settings):
    Ws, Hs, lams, rgb, scrib = _batch(32, 3500)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(64, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    bs.set_solver(**settings)
    got = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    bs.close()


def test_phase_split_runs_both_phases_and_changes_no_result():
    """gcfg_batch_phase_split runs the first global relabel and the push rounds
    after it as two launches of the solver; the counters it reports are
    consistent, and the handle's next run still gives the full solve's
    results."""
    Ws, Hs, lams, rgb, scrib = _batch(24, 3300)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(32, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    tiles = int(sum(((int(w) + 31) // 32) * ((int(h) + 31) // 32) for w, h in zip(Ws, Hs)))
    for _ in range(2):
        ps = bs.phase_split(Ws, Hs, lams, d_rgb, d_scrib)
        assert ps["ms_relabel"] > 0 and ps["grid_blocks"] >= 1
        assert ps["relabel_tiles"] >= tiles  # round 0 visits every tile
        assert ps["active_pixels"] > 0 and ps["push_queue"] > 0
        assert ps["ms_push"] > 0 and ps["push_tiles"] >= 1 and ps["push_phases"] >= 1
        assert ps["push_sweeps"] >= ps["push_tiles"]
        # the relabel's timeline: round 0 visits every tile, then one entry
        # per frontier round with its tile count
        n = min(ps["relabel_rounds"], 32)
        assert len(ps["relabel_front_tiles"]) == n and len(ps["relabel_front_us"]) == n
        assert ps["relabel_round0_us"] > 0 and ps["relabel_pull_us"] > 0
        assert all(k > 0 for k in ps["relabel_front_tiles"]) and all(u > 0 for u in ps["relabel_front_us"])
        assert all(0 <= w <= u for w, u in zip(ps["relabel_front_work_us"], ps["relabel_front_us"]))
        if ps["relabel_rounds"] <= 32:
            assert sum(ps["relabel_front_tiles"]) == ps["relabel_tiles"] - tiles
        got = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
        assert np.array_equal(got[0], ref[0])
        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])


@pytest.mark.parametrize("threads_y", [4, 8, 16, 32])
def test_every_solver_block_shape_gives_the_same_results(threads_y):
    """The solver's thread block over a 32x32 tile (32 x threads_y, the
    reference's THREADS_X x THREADS_Y) changes only the running time: flows
    and both cuts equal those of the default 32 x 8 block, also with the
    push-only sweeps and fewer blocks per SM."""
    Ws, Hs, lams, rgb, scrib = _batch(20, 3500)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(32, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    for extra in ({}, {"push_only": 1}, {"blocks_per_sm": 1}, {"max_tile_sweeps": 128, "sweeps_per_local_relabel": 2}):
        bs.set_solver(threads_y=threads_y, **extra)
        got = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
        assert np.array_equal(got[0], ref[0])
        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    ps = bs.phase_split(Ws, Hs, lams, d_rgb, d_scrib)
    assert ps["push_tiles"] >= 1 and ps["grid_blocks"] >= 1
    with pytest.raises(gcfg.GcfgError):
        bs.set_solver(threads_y=5)
    bs.close()


def test_autotuner_reports_the_block_shape():
    Ws, Hs, lams, rgb, scrib = _batch(12, 3600)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(16, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    t = bs.autotune(Ws, Hs, lams, d_rgb, d_scrib, reps=1)
    assert t["threads_y"] in (4, 8, 16, 32) and t["tile_w"] == 32 and t["tile_h"] == 32
    assert t["configs_tried"] >= 10
    got = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    bs.close()


def test_cut_outputs_at_any_alignment():
    """The cut pass writes whole 16-byte windows when S_min and S_max share
    their address modulo 16 (at any offset) and falls back to the tile-major
    pass when they do not; either output may be left out.  Every case gives
    the cuts of the aligned run, and no byte outside the outputs changes."""
    Ws, Hs, lams, rgb, scrib = _batch(16, 3800)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_scrib = torch.from_numpy(scrib).cuda()
    bs = gcfg.BatchSolver(16, scrib.size)
    ref = _run(bs, Ws, Hs, lams, d_rgb, d_scrib)
    n_px = scrib.size
    buf_a = torch.empty(n_px + 64, dtype=torch.uint8, device="cuda")
    buf_b = torch.empty(n_px + 64, dtype=torch.uint8, device="cuda")
    for oa, ob in ((0, 0), (5, 5), (13, 13), (1, 0), (0, 7), (3, 11)):
        buf_a.fill_(7)
        buf_b.fill_(9)
        smin, smax = buf_a[oa:oa + n_px], buf_b[ob:ob + n_px]
        flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, smax)
        assert np.array_equal(flows, ref[0])
        assert np.array_equal(smin.cpu().numpy(), ref[1]), (oa, ob)
        assert np.array_equal(smax.cpu().numpy(), ref[2]), (oa, ob)
        a, b = buf_a.cpu().numpy(), buf_b.cpu().numpy()
        assert (a[:oa] == 7).all() and (a[oa + n_px:] == 7).all()
        assert (b[:ob] == 9).all() and (b[ob + n_px:] == 9).all()
    for oa in (0, 6):
        buf_b.fill_(9)
        smax = buf_b[oa:oa + n_px]
        flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, None, smax)
        assert np.array_equal(flows, ref[0]) and np.array_equal(smax.cpu().numpy(), ref[2])
        buf_a.fill_(7)
        smin = buf_a[oa:oa + n_px]
        flows, _ = bs.run(Ws, Hs, lams, d_rgb, d_scrib, smin, None)
        assert np.array_equal(flows, ref[0]) and np.array_equal(smin.cpu().numpy(), ref[1])
    bs.close()
