"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and
the reference's own outputs.  Integer work is compared bit for bit."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import gcfg  # noqa: E402
import oracle as O  # noqa: E402
from gpu_util import dev, gpu_segment, gpu_solve  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(GOLDEN, "reference_pins.json")))["cases"]
DATA = np.load(os.path.join(GOLDEN, "reference_pins.npz"))


def _case(c):
    name = c["name"]
    dp = DATA[f"{name}__dp"].astype(np.int32)
    dn = DATA[f"{name}__dn"].astype(np.int32)
    kw = {"penalty": c["penalty"]}
    if c["arrays"]:
        for k in ("up", "down", "left", "right"):
            kw[k] = DATA[f"{name}__{k}"].astype(np.int32)
    n = c["W"] * c["H"]
    labels = np.unpackbits(DATA[f"{name}__ref_labels"])[:n].reshape(c["H"], c["W"])
    return dp, dn, kw, labels


@pytest.mark.parametrize("case", META, ids=[c["name"] for c in META])
def test_reference_pins(case):
    """GC_Optimize labels and printed energy equal the reference's own."""
    dp, dn, kw, ref_labels = _case(case)
    label, smin, smax, res = gpu_solve(dp, dn, **kw)
    assert np.array_equal(label, ref_labels.astype(np.int32))
    assert res["ref_energy"] == case["ref_energy"]
    assert res["flow"] == case["oracle_flow"]
    o = O.solve(dp, dn, **kw)
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


@pytest.mark.parametrize("seed", range(8))
def test_random_grids_vs_oracle(seed):
    rng = np.random.default_rng(7000 + seed)
    for _ in range(6):
        H, W = (int(v) for v in rng.integers(3, 150, 2))
        dp = rng.integers(0, 300, (H, W)).astype(np.int32)
        dn = rng.integers(0, 300, (H, W)).astype(np.int32)
        if rng.random() < 0.5:
            kw = {k: rng.integers(0, 120, (H, W)).astype(np.int32) for k in ("up", "down", "left", "right")}
        else:
            kw = {"penalty": int(rng.integers(0, 150))}
        label, smin, smax, res = gpu_solve(dp, dn, **kw)
        o = O.solve(dp, dn, **kw)
        assert res["flow"] == o["flow"]
        assert np.array_equal(smax, o["smax"]) and np.array_equal(smin, o["smin"])
        assert np.array_equal(label, o["smax"].astype(np.int32))


@pytest.mark.parametrize("schedule", [(1, 1), (1, 4), (8, 256), (3, 17)])
def test_schedules_do_not_change_result(schedule):
    rng = np.random.default_rng(11)
    H, W = 97, 131
    dp = rng.integers(0, 300, (H, W)).astype(np.int32)
    dn = rng.integers(0, 300, (H, W)).astype(np.int32)
    label, smin, smax, res = gpu_solve(dp, dn, penalty=60, schedule=schedule)
    o = O.solve(dp, dn, penalty=60)
    assert res["flow"] == o["flow"]
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


def test_long_paths_vs_oracle():
    """Flow that must cross many tiles (worst case for tile-local pushes)."""
    H, W = 40, 600
    dp = np.zeros((H, W), np.int32)
    dn = np.zeros((H, W), np.int32)
    dp[:, 1] = 500
    dn[:, W - 2] = 500
    label, smin, smax, res = gpu_solve(dp, dn, penalty=7)
    o = O.solve(dp, dn, penalty=7)
    assert res["flow"] == o["flow"] == 7 * (H - 2)
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


def test_tlinks_bit_exact():
    rgb, scrib = O.generate(0, 256, 256, 0)
    H, W = scrib.shape
    dp = torch.empty((H, W), dtype=torch.int32, device="cuda")
    dn = torch.empty_like(dp)
    rdp, rdn = gcfg.tlinks(dev(rgb), dev(scrib), dp, dn, raw=True)
    hf, hb = O.histograms(rgb, scrib)
    odp_raw, odn_raw, _, _ = O.tlink_lut(hf, hb)
    # pre-quantisation values: within 1e-6 relative (they agree far closer)
    np.testing.assert_allclose(rdp, odp_raw, rtol=1e-12)
    np.testing.assert_allclose(rdn, odn_raw, rtol=1e-12)
    odp, odn = O.tlinks(rgb, scrib)
    assert np.array_equal(dp.cpu().numpy(), odp) and np.array_equal(dn.cpu().numpy(), odn)


@pytest.mark.parametrize("lam", [10.0, 50.0, 200.0])
def test_nlinks_bit_exact(lam):
    rgb, _ = O.generate(1, 320, 200, 5)
    H, W = rgb.shape[:2]
    outs = [torch.empty((H, W), dtype=torch.int32, device="cuda") for _ in range(4)]
    gcfg.nlinks(dev(rgb), W, H, lam, *outs)
    ref = O.nlinks(rgb, lam)
    for a, b in zip(outs, ref):
        assert np.array_equal(a.cpu().numpy(), b)


def test_segment_cfg0_vs_oracle():
    rgb, scrib = O.generate(0, 256, 256, 0)
    smin, smax, res = gpu_segment(rgb, scrib, 50.0)
    o = O.segment(rgb, scrib, 50.0)
    assert res["flow"] == o["flow"]
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


@pytest.mark.parametrize("seed,lam", [(1, 10.0), (2, 50.0), (3, 200.0)])
def test_segment_cfg1_vs_oracle(seed, lam):
    rgb, scrib = O.generate(1, 1920, 1080, seed)
    smin, smax, res = gpu_segment(rgb, scrib, lam)
    o = O.segment(rgb, scrib, lam)
    assert res["flow"] == o["flow"]
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


def test_segment_cfg2_vs_oracle():
    rgb, scrib = O.generate(2, 4096, 4096, 2)
    smin, smax, res = gpu_segment(rgb, scrib, 100.0)
    o = O.segment(rgb, scrib, 100.0)
    assert res["flow"] == o["flow"]
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


def test_host_entry_point_matches_device_path():
    rgb, scrib = O.generate(3, 300, 200, 1005)
    seg = gcfg.Segmenter(512, 512)
    smin_d, smax_d, res_d = gpu_segment(rgb, scrib, 50.0, seg)
    smin_h = np.zeros(scrib.shape, np.uint8)
    smax_h = np.zeros(scrib.shape, np.uint8)
    res_h = seg.run_host(rgb, scrib, 300, 200, 50.0, smin_h, smax_h)
    assert res_h["flow"] == res_d["flow"]
    assert np.array_equal(smin_h, smin_d) and np.array_equal(smax_h, smax_d)


def test_invalid_capacities_rejected():
    dp = np.full((8, 8), 5, np.int32)
    dn = np.full((8, 8), 3, np.int32)
    dp[3, 3] = -1
    with pytest.raises(gcfg.GcfgError) as ei:
        gpu_solve(dp, dn, penalty=1)
    assert ei.value.status == gcfg.GCFG_ERR_INVALID
    dp[3, 3] = gcfg.GCFG_MAX_CAP + 1
    with pytest.raises(gcfg.GcfgError):
        gpu_solve(dp, dn, penalty=1)


def test_optimize_twice_needs_set_graph():
    """As in the reference the graph is consumed by the solve."""
    dp = np.full((16, 16), 9, np.int32)
    dn = np.full((16, 16), 4, np.int32)
    t = [dev(dp), dev(dn)]
    gw = gcfg.GC_Init(16, 16, t[0], t[1], 3)
    r1 = gcfg.GC_Optimize(gw)
    with pytest.raises(gcfg.GcfgError) as ei:
        gcfg.GC_Optimize(gw)
    assert ei.value.status == gcfg.GCFG_ERR_STATE
    gcfg.GC_SetGraph(gw)
    r2 = gcfg.GC_Optimize(gw)
    assert r1["flow"] == r2["flow"]
    gcfg.GC_End(gw)


def _batch_images(n, seed0, max_side=300):
    """Uneven images from the scaled cfg-0 generator (small, for parity)."""
    rng = np.random.default_rng(seed0)
    imgs = []
    for i in range(n):
        s = float(np.exp(rng.uniform(np.log(20), np.log(max_side))))
        a = float(rng.uniform(0.5, 2.0))
        W = max(3, int(round(s * np.sqrt(a))))
        H = max(3, int(round(s / np.sqrt(a))))
        imgs.append(O.generate(3, W, H, seed0 + i))
    return imgs


@pytest.mark.parametrize("n,seed0", [(1, 500), (7, 600), (40, 700)])
def test_batch_vs_oracle(n, seed0):
    """Many uneven images in one solve: every image bit-identical to its own
    oracle solve."""
    imgs = _batch_images(n, seed0)
    lams = [(10.0, 50.0, 200.0)[i % 3] for i in range(n)]
    Ws = [s.shape[1] for _, s in imgs]
    Hs = [s.shape[0] for _, s in imgs]
    rgb = np.concatenate([r.reshape(-1) for r, _ in imgs])
    scrib = np.concatenate([s.reshape(-1) for _, s in imgs])
    total = scrib.size
    bs = gcfg.BatchSolver(n, total)
    smin = torch.zeros(total, dtype=torch.uint8, device="cuda")
    smax = torch.zeros(total, dtype=torch.uint8, device="cuda")
    flows, res = bs.run(Ws, Hs, lams, dev(rgb), dev(scrib), smin, smax, results=True)
    smin = smin.cpu().numpy()
    smax = smax.cpu().numpy()
    off = 0
    for i, ((r, s), lam) in enumerate(zip(imgs, lams)):
        o = O.segment(r, s, lam)
        k = s.size
        assert flows[i] == o["flow"], i
        assert np.array_equal(smin[off:off + k].reshape(s.shape), o["smin"]), i
        assert np.array_equal(smax[off:off + k].reshape(s.shape), o["smax"]), i
        off += k
    # the host entry point gives the same answer
    hmin = np.zeros(total, np.uint8)
    hmax = np.zeros(total, np.uint8)
    flows_h, _ = bs.run_host(Ws, Hs, lams, rgb, scrib, hmin, hmax)
    assert np.array_equal(flows_h, flows)
    assert np.array_equal(hmin, smin) and np.array_equal(hmax, smax)


def test_termination_check_ends_solve_exactly():
    """After its push rounds a typical batch is finished by the sink-side
    reachability check (no final global relabel); flows and both cuts still
    equal the oracle's, and so do those of a heavier image, which can fail a
    check and go on to another global relabel."""
    imgs = _batch_images(16, 1100)
    Ws = [s.shape[1] for _, s in imgs]
    Hs = [s.shape[0] for _, s in imgs]
    rgb = np.concatenate([r.reshape(-1) for r, _ in imgs])
    scrib = np.concatenate([s.reshape(-1) for _, s in imgs])
    bs = gcfg.BatchSolver(16, scrib.size)
    smin = torch.zeros(scrib.size, dtype=torch.uint8, device="cuda")
    smax = torch.zeros(scrib.size, dtype=torch.uint8, device="cuda")
    flows, res = bs.run(Ws, Hs, [50.0] * 16, dev(rgb), dev(scrib), smin, smax, results=True)
    r0 = res[0] if isinstance(res, list) else res
    assert r0["closure_checks"] >= 1 and r0["closure_ends"] == 1
    smin, smax = smin.cpu().numpy(), smax.cpu().numpy()
    off = 0
    for i, (r, s) in enumerate(imgs):
        o = O.segment(r, s, 50.0)
        k = s.size
        assert flows[i] == o["flow"], i
        assert np.array_equal(smin[off:off + k].reshape(s.shape), o["smin"]), i
        assert np.array_equal(smax[off:off + k].reshape(s.shape), o["smax"]), i
        off += k
    rgb, scrib = O.generate(2, 2048, 2048, 2)
    smin_h, smax_h, res = gpu_segment(rgb, scrib, 100.0)
    o = O.segment(rgb, scrib, 100.0)
    # every global relabel after the first follows a failed check
    assert res["closure_checks"] >= res["global_relabels"] - 1
    assert res["flow"] == o["flow"]
    assert np.array_equal(smin_h, o["smin"]) and np.array_equal(smax_h, o["smax"])


@pytest.mark.parametrize("params", [(1, 1, 1), (1, 8, 2), (2, 64, 16), (8, 256, 64)])
def test_batch_params_do_not_change_result(params):
    imgs = _batch_images(12, 900)
    Ws = [s.shape[1] for _, s in imgs]
    Hs = [s.shape[0] for _, s in imgs]
    rgb = np.concatenate([r.reshape(-1) for r, _ in imgs])
    scrib = np.concatenate([s.reshape(-1) for _, s in imgs])
    bs = gcfg.BatchSolver(12, scrib.size)
    bs.set_params(*params)
    flows, _ = bs.run(Ws, Hs, [50.0] * 12, dev(rgb), dev(scrib))
    for i, (r, s) in enumerate(imgs):
        assert flows[i] == O.segment(r, s, 50.0)["flow"]


@pytest.mark.parametrize("cfg,W,H,seed", [(0, 256, 256, 0), (1, 400, 300, 11), (2, 512, 512, 2), (3, 97, 61, 1003)])
@pytest.mark.parametrize("lam", [0.3, 0.5, 1.0, 7.7, 37.3, 50.0, 200.0, 1000.0, 12345.6])
def test_nlinks_bit_exact_many(cfg, W, H, seed, lam):
    """The n-link table (float fast path, double fallback near .5) equals
    the oracle's double evaluation for every weight."""
    rgb, _ = O.generate(cfg, W, H, seed)
    outs = [torch.empty((H, W), dtype=torch.int32, device="cuda") for _ in range(4)]
    gcfg.nlinks(dev(rgb), W, H, lam, *outs)
    for a, b in zip(outs, O.nlinks(rgb, lam)):
        assert np.array_equal(a.cpu().numpy(), b)


@pytest.mark.parametrize("cfg,W,H,seed", [(0, 256, 256, 0), (1, 640, 360, 4), (2, 700, 500, 9), (3, 40, 120, 1010)])
def test_tlinks_bit_exact_many(cfg, W, H, seed):
    rgb, scrib = O.generate(cfg, W, H, seed)
    dp = torch.empty((H, W), dtype=torch.int32, device="cuda")
    dn = torch.empty_like(dp)
    gcfg.tlinks(dev(rgb), dev(scrib), dp, dn)
    odp, odn = O.tlinks(rgb, scrib)
    assert np.array_equal(dp.cpu().numpy(), odp) and np.array_equal(dn.cpu().numpy(), odn)


def test_batch_degenerate_shapes():
    """Images with no interior pixel (1xN, Nx1, 2x2), a single tile, tiles
    just past a multiple of 32, mixed with a normal image in one batch."""
    shapes = [(1, 1), (1, 7), (7, 1), (2, 2), (2, 50), (50, 2), (3, 3), (33, 1), (32, 32), (33, 33), (65, 31),
              (200, 150)]
    imgs = [O.generate(3, W, H, 1700 + i) for i, (W, H) in enumerate(shapes)]
    lams = [(10.0, 50.0, 200.0)[i % 3] for i in range(len(imgs))]
    Ws = [s.shape[1] for _, s in imgs]
    Hs = [s.shape[0] for _, s in imgs]
    rgb = np.concatenate([r.reshape(-1) for r, _ in imgs])
    scrib = np.concatenate([s.reshape(-1) for _, s in imgs])
    total = scrib.size
    bs = gcfg.BatchSolver(len(imgs), total)
    smin = torch.zeros(total, dtype=torch.uint8, device="cuda")
    smax = torch.zeros(total, dtype=torch.uint8, device="cuda")
    flows, _ = bs.run(Ws, Hs, lams, dev(rgb), dev(scrib), smin, smax)
    smin = smin.cpu().numpy()
    smax = smax.cpu().numpy()
    off = 0
    for i, ((r, s), lam) in enumerate(zip(imgs, lams)):
        o = O.segment(r, s, lam)
        k = s.size
        assert flows[i] == o["flow"], shapes[i]
        assert np.array_equal(smin[off:off + k].reshape(s.shape), o["smin"]), shapes[i]
        assert np.array_equal(smax[off:off + k].reshape(s.shape), o["smax"]), shapes[i]
        off += k
    hmin = np.zeros(total, np.uint8)
    hmax = np.zeros(total, np.uint8)
    flows_h, _ = bs.run_host(Ws, Hs, lams, rgb, scrib, hmin, hmax)
    assert np.array_equal(flows_h, flows) and np.array_equal(hmin, smin) and np.array_equal(hmax, smax)


def test_batch256_full_size_cuts_match_per_image():
    """The full 256-image workload: every image's cuts from the batched solve
    equal the one-image path's, and a sample of flows equals the oracle's."""
    import synth
    shapes = synth.batch_shapes(256, 1000)
    rgb, scrib, offs = synth.generate_packed([(3, W, H, s) for (W, H, s) in shapes])
    Ws = [W for (W, _, _) in shapes]
    Hs = [H for (_, H, _) in shapes]
    total = scrib.size
    d_rgb, d_scrib = dev(rgb), dev(scrib)
    bs = gcfg.BatchSolver(256, total)
    smin = torch.zeros(total, dtype=torch.uint8, device="cuda")
    smax = torch.zeros(total, dtype=torch.uint8, device="cuda")
    flows, _ = bs.run(Ws, Hs, [50.0] * 256, d_rgb, d_scrib, smin, smax)
    seg = gcfg.Segmenter(max(Ws), max(Hs))
    for i, (W, H, _) in enumerate(shapes):
        o, n = int(offs[i]), W * H
        a = torch.zeros(n, dtype=torch.uint8, device="cuda")
        b = torch.zeros(n, dtype=torch.uint8, device="cuda")
        r = seg.run(d_rgb[3 * o:3 * (o + n)], d_scrib[o:o + n], W, H, 50.0, a, b)
        assert r["flow"] == flows[i], i
        assert torch.equal(a, smin[o:o + n]) and torch.equal(b, smax[o:o + n]), i
    for i in range(0, 256, 37):
        W, H, _ = shapes[i]
        o, n = int(offs[i]), W * H
        assert flows[i] == O.segment(rgb[3 * o:3 * (o + n)].reshape(H, W, 3), scrib[o:o + n].reshape(H, W), 50.0)["flow"]


def test_ex2_error_within_nlink_bound():
    """The n-link fast path's margin assumes the device's approximate 2^z is
    within 2^-21 relative error on the exponents it meets ([-64, 0])."""
    err = gcfg.selftest_ex2(1 << 24)
    assert 0.0 <= err <= 2.0 ** -21, err


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("lam", [0.7, 3.0, 50.0, 255.5, 4096.0, 65536.0, 3.0e6])
def test_nlinks_bit_exact_random_colours(seed, lam):
    """Uniform random colours spread the squared distances over the whole
    range 0 .. 3*255^2 (generated images keep them small); every weight of
    the float fast path equals the oracle's double evaluation."""
    rng = np.random.default_rng(77 + seed)
    W, H = 611, 409
    rgb = rng.integers(0, 256, size=(H, W, 3), dtype=np.uint8)
    if seed == 1:  # a few colours only: many equal distances (ties of d2)
        pal = rng.integers(0, 256, size=(5, 3), dtype=np.uint8)
        rgb = pal[rng.integers(0, 5, size=(H, W))]
    outs = [torch.empty((H, W), dtype=torch.int32, device="cuda") for _ in range(4)]
    gcfg.nlinks(dev(rgb), W, H, lam, *outs)
    for a, b in zip(outs, O.nlinks(rgb, lam)):
        assert np.array_equal(a.cpu().numpy(), b)


def _serving_edit(k):
    """Image and scribbles of request k of the serving trace (seed 4): the
    edited session's pool image with every edit up to and including k."""
    import synth
    pool_specs, reqs = synth.serve_trace(1200, 500.0, 4)
    news = [q["img"] for q in reqs if q["kind"] == "new"]
    target = reqs[k]["target"]
    _, side, _, seed = pool_specs[news[target]]
    rgb, scrib = synth.generate(4, side, side, seed)
    scrib = scrib.copy()
    for q in reqs[:k + 1]:
        if q["kind"] == "edit" and q["target"] == target:
            scrib[q["y"]:q["y"] + q["size"], q["x"]:q["x"] + q["size"]] = q["cls"]
    return rgb, scrib


@pytest.mark.parametrize("k", [45, 490])
def test_hard_serving_edits_vs_oracle(k):
    """The two slowest solves of the serving trace (15x15 edits of one 1024^2
    pool image: about ten global relabels and forty push colour phases each)
    are exact under the default settings and under the settings the
    autotuner picks for them (32 x 16 block, push-only sweeps, one block per
    SM)."""
    rgb, scrib = _serving_edit(k)
    o = O.segment(rgb, scrib, 50.0)
    smin, smax, res = gpu_segment(rgb, scrib, 50.0)
    assert res["global_relabels"] >= 5
    assert res["flow"] == o["flow"]
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])
    H, W = scrib.shape
    bs = gcfg.BatchSolver(1, W * H)
    Wa = np.array([W], np.int32)
    d_rgb, d_scrib = dev(rgb.reshape(-1)), dev(scrib.reshape(-1))
    for kw in ({}, {"threads_y": 16, "push_rounds_per_gr": 4, "sweeps_per_local_relabel": 16, "blocks_per_sm": 1,
                    "push_only": 1}):
        bs.set_solver(**kw)
        d_min = torch.empty(W * H, dtype=torch.uint8, device="cuda")
        d_max = torch.empty(W * H, dtype=torch.uint8, device="cuda")
        flows, _ = bs.run(Wa, Wa, np.array([50.0]), d_rgb, d_scrib, d_min, d_max)
        assert flows[0] == o["flow"]
        assert np.array_equal(d_min.cpu().numpy().reshape(H, W), o["smin"])
        assert np.array_equal(d_max.cpu().numpy().reshape(H, W), o["smax"])
    bs.close()
