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
