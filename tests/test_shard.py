"""Multi-rank placement (gc-fg_gb300/shard.py) on CPU: the partition covers
every image once and balances pixels, and two gloo ranks that each solve
their share with the CPU oracle reproduce the single-process flows and agree
on the job's time (max over ranks)."""
import os
import socket

import numpy as np
import pytest

import shard
import synth


def test_lpt_partition_covers_and_balances():
    rng = np.random.default_rng(5)
    for world in (1, 2, 3, 8):
        sizes = rng.integers(1, 10_000, 61)
        parts = shard.lpt_partition(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sum(sizes[i] for i in p)) for p in parts]
        assert max(loads) - min(loads) <= int(sizes.max())
        assert parts == shard.lpt_partition(sizes, world)  # deterministic
    assert shard.lpt_partition([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard.lpt_partition([1], 0)


def test_weak_seeds_are_disjoint():
    ranges = [set(range(shard.weak_seed0(1000, 256, r), shard.weak_seed0(1000, 256, r) + 256)) for r in range(8)]
    for a in range(8):
        for b in range(a + 1, 8):
            assert not ranges[a] & ranges[b]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _images():
    shapes = [(W, H) for (W, H, _) in synth.batch_shapes(10, 500, lo=16, hi=48)]
    return [(W, H, 500 + i) for i, (W, H) in enumerate(shapes)]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    import oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    imgs = _images()
    mine = shard.rank_share([W * H for (W, H, _) in imgs], rank, world)
    flows = {}
    for i in mine:
        W, H, seed = imgs[i]
        rgb, scrib = synth.generate(3, W, H, seed)
        flows[i] = O.segment(rgb, scrib, 50.0)["flow"]
    every = shard.gather(flows)
    t = shard.max_over_ranks(1.0 + rank)
    px = shard.sum_over_ranks(sum(imgs[i][0] * imgs[i][1] for i in mine))
    shard.barrier()
    if rank == 0:
        merged = {}
        for part in every:
            assert not set(part) & set(merged)
            merged.update(part)
        np.save(os.path.join(out_dir, "flows.npy"), np.array([merged[i] for i in range(len(imgs))], np.int64))
        np.save(os.path.join(out_dir, "scalars.npy"), np.array([t, px]))
    dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle as O
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    imgs = _images()
    expect = []
    for W, H, seed in imgs:
        rgb, scrib = synth.generate(3, W, H, seed)
        expect.append(O.segment(rgb, scrib, 50.0)["flow"])
    assert np.array_equal(np.load(tmp_path / "flows.npy"), np.array(expect, np.int64))
    t, px = np.load(tmp_path / "scalars.npy")
    assert t == 2.0 and px == sum(W * H for (W, H, _) in imgs)


# ---- serving dispatcher (RequestRouter) ----

def _serve_trace(n=36, seed=9):
    """A small request trace: new square images of side 24/40/64 and 15x15
    scribble edits of earlier ones (about a third), in arrival order."""
    rng = np.random.default_rng(seed)
    reqs, news = [], []
    for k in range(n):
        if news and rng.random() < 0.35:
            t = int(rng.integers(0, len(news)))
            side = news[t][0]
            reqs.append(dict(kind="edit", target=t, x=int(rng.integers(0, side - 15)),
                             y=int(rng.integers(0, side - 15)), cls=int(rng.integers(1, 3))))
        else:
            side = int(rng.choice([24, 40, 64]))
            news.append((side, 7000 + k))
            reqs.append(dict(kind="new", side=side, seed=7000 + k, session=len(news) - 1))
    return reqs, news


def _route(reqs, news, world, cap):
    router = shard.RequestRouter(world, cap)
    ranks = []
    for q in reqs:
        if q["kind"] == "new":
            ranks.append(router.place_new(q["session"], q["side"], q["side"]))
        else:
            ranks.append(router.place_edit(q["target"]))
    return ranks, router


def _serve_local(reqs, news, mine):
    """Flows of the requests in `mine` (indices into reqs, in order), each
    edit applied to its image's current scribbles and re-solved with the
    oracle (a warm re-solve equals a cold solve of the edited image)."""
    import oracle as O
    scribs, out = {}, {}
    for k in mine:
        q = reqs[k]
        t = q["session"] if q["kind"] == "new" else q["target"]
        side, seed = news[t]
        rgb, scrib = synth.generate(4, side, side, seed)
        if q["kind"] == "new":
            scribs[t] = scrib.copy()
        else:
            scribs[t][q["y"]:q["y"] + 15, q["x"]:q["x"] + 15] = q["cls"]
        out[k] = O.segment(rgb, scribs[t], 50.0)["flow"]
    return out


def test_router_places_by_footprint_and_keeps_edits_with_their_image():
    reqs, news = _serve_trace()
    cap = 40 * shard.SERVE_TILE_BYTES
    ranks, router = _route(reqs, news, 2, cap)
    for k, q in enumerate(reqs):
        if q["kind"] == "edit":
            first = next(j for j, p in enumerate(reqs) if p["kind"] == "new" and p["session"] == q["target"])
            assert ranks[k] == ranks[first]
    # every image fits, so the resident state of the two GPUs differs by at
    # most the largest image plus what edits (which follow their image) added
    # to one side's load when the later images were placed
    edits = sum(shard.image_footprint(news[q["target"]][0], news[q["target"]][0]) for q in reqs if q["kind"] == "edit")
    assert abs(router.resident[0] - router.resident[1]) <= shard.image_footprint(64, 64) + edits
    assert min(router.resident) > 0
    assert sum(router.resident) == sum(shard.image_footprint(s, s) for s, _ in news)
    for sess in range(len(news)):
        for q in reqs:
            if (q["kind"] == "new" and q["session"] == sess) or (q["kind"] == "edit" and q["target"] == sess):
                router.done(sess)
    assert router.inflight == [0, 0]
    for sess in range(len(news)):
        router.release(sess)
    assert router.resident == [0, 0]
    with pytest.raises(KeyError):
        router.place_edit(0)
    with pytest.raises(ValueError):
        shard.RequestRouter(2, 1000).place_new(0, 64, 64)
    # a new image prefers the GPU whose cap still holds it
    r = shard.RequestRouter(2, 3 * shard.image_footprint(64, 64))
    assert r.place_new("a", 64, 64) == 0 and r.place_new("b", 64, 64) == 1
    r.done("a"), r.done("b")
    assert r.place_new("c", 64, 64) == 0
    r.done("c")
    r.resident[0] += 2 * shard.image_footprint(64, 64)  # rank 0 is full
    assert r.place_new("d", 64, 64) == 1


def _router_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    reqs, news = _serve_trace()
    placement = [None]
    if rank == 0:  # the front end routes the trace and tells every rank its share
        placement[0] = _route(reqs, news, world, 40 * shard.SERVE_TILE_BYTES)[0]
    dist.broadcast_object_list(placement, src=0)
    mine = [k for k, r in enumerate(placement[0]) if r == rank]
    every = shard.gather(_serve_local(reqs, news, mine))
    if rank == 0:
        merged = {}
        for part in every:
            assert not set(part) & set(merged)
            merged.update(part)
        np.save(os.path.join(out_dir, "served.npy"), np.array([merged[k] for k in range(len(reqs))], np.int64))
        np.save(os.path.join(out_dir, "ranks.npy"), np.array(placement[0]))
    dist.destroy_process_group()


def test_two_gloo_ranks_serve_a_routed_trace_like_one_process(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_router_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    reqs, news = _serve_trace()
    expect = _serve_local(reqs, news, range(len(reqs)))
    assert np.array_equal(np.load(tmp_path / "served.npy"), np.array([expect[k] for k in range(len(reqs))]))
    ranks = np.load(tmp_path / "ranks.npy")
    assert set(ranks.tolist()) == {0, 1}  # both GPUs served requests
