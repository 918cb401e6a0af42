"""Graphs with the 8-neighbourhood (the reference built with NEIGHBORHOOD 8).

Pins: the reference's own solver with NEIGHBORHOOD switched to 8, run on the
CPU emulator (tests/golden/make_reference_pins8.py).  The 8-connected oracle
reproduces every pin (labels and printed energy); the GPU engine reproduces
the pins and the oracle, through the Python mirror and through a C++ caller
compiled against include/GraphCut.cu with NEIGHBORHOOD 8."""
import json
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import gcfg
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
META = json.load(open(os.path.join(GOLDEN, "reference_pins8.json")))["cases"]
DATA = np.load(os.path.join(GOLDEN, "reference_pins8.npz"))
DIRS = ("left", "right", "up", "down", "upleft", "upright", "downleft", "downright")
REF_ORDER = ("up", "down", "left", "right", "upleft", "upright", "downleft", "downright")


def _case(c):
    name = c["name"]
    dp = DATA[f"{name}__dp"].astype(np.int32)
    dn = DATA[f"{name}__dn"].astype(np.int32)
    arrs = {k: DATA[f"{name}__{k}"].astype(np.int32) for k in DIRS} if c["arrays"] else None
    n = c["W"] * c["H"]
    labels = np.unpackbits(DATA[f"{name}__ref_labels"])[:n].reshape(c["H"], c["W"]).astype(np.int32)
    return dp, dn, arrs, labels


def _cut_energy8(dp, dn, penalty, arrs, s):
    """Energy of a labelling (1 = source side) of the 8-connected graph."""
    H, W = dp.shape
    e = 0
    inside = np.zeros((H, W), bool)
    inside[1:H - 1, 1:W - 1] = True
    e += int(dp[inside & (s == 0)].sum()) + int(dn[inside & (s == 1)].sum())
    off = {"left": (0, -1), "right": (0, 1), "up": (-1, 0), "down": (1, 0), "upleft": (-1, -1), "upright": (-1, 1),
           "downleft": (1, -1), "downright": (1, 1)}
    for k, (dy, dx) in off.items():
        for y in range(1, H - 1):
            for x in range(1, W - 1):
                yy, xx = y + dy, x + dx
                if not (1 <= yy <= H - 2 and 1 <= xx <= W - 2):
                    continue
                if s[y, x] == 1 and s[yy, xx] == 0:
                    e += int(arrs[k][y, x]) if arrs is not None else penalty
    return e


@pytest.mark.parametrize("case", META, ids=[c["name"] for c in META])
def test_oracle8_reproduces_reference(case):
    dp, dn, arrs, labels = _case(case)
    o = O.solve8(dp, dn, penalty=case["penalty"], arrays=None if arrs is None else [arrs[k] for k in DIRS])
    assert case["oracle_agrees"]
    assert np.array_equal(o["smax"].astype(np.int32), labels)
    assert O.reference_energy(dp, o["excess"]) == case["ref_energy"]
    assert o["flow"] == case["oracle_flow"]


def test_oracle8_cut_energy_equals_flow():
    rng = np.random.default_rng(81)
    for _ in range(4):
        H, W = (int(v) for v in rng.integers(4, 14, 2))
        dp = rng.integers(0, 60, (H, W)).astype(np.int32)
        dn = rng.integers(0, 60, (H, W)).astype(np.int32)
        arrs = {k: rng.integers(0, 25, (H, W)).astype(np.int32) for k in DIRS}
        o = O.solve8(dp, dn, arrays=[arrs[k] for k in DIRS])
        assert _cut_energy8(dp, dn, 0, arrs, o["smax"]) == o["flow"]
        assert _cut_energy8(dp, dn, 0, arrs, o["smin"]) == o["flow"]


def test_oracle8_without_diagonals_is_the_4_neighbourhood():
    rng = np.random.default_rng(82)
    H, W = 23, 31
    dp = rng.integers(0, 100, (H, W)).astype(np.int32)
    dn = rng.integers(0, 100, (H, W)).astype(np.int32)
    a = [rng.integers(0, 40, (H, W)).astype(np.int32) for _ in range(4)]
    z = [np.zeros((H, W), np.int32)] * 4
    o8 = O.solve8(dp, dn, arrays=a + z)
    o4 = O.solve(dp, dn, left=a[0], right=a[1], up=a[2], down=a[3])
    assert o8["flow"] == o4["flow"]
    assert np.array_equal(o8["smin"], o4["smin"]) and np.array_equal(o8["smax"], o4["smax"])


def _gpu8(dp, dn, penalty, arrs):
    torch = pytest.importorskip("torch")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.int32)).cuda()  # noqa: E731
    H, W = dp.shape
    kw = {} if arrs is None else {k: dev(arrs[k]) for k in DIRS}
    gw = gcfg.GC_Init8(W, H, dev(dp), dev(dn), penalty, **kw)
    label = np.zeros((H, W), np.int32)
    r = gcfg.GC_Optimize8(gw, label)
    smin = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    smax = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    gcfg.GC_GetCuts8(gw, smin, smax)
    gcfg.GC_End8(gw)
    return label, smin.cpu().numpy(), smax.cpu().numpy(), r


@pytest.mark.gpu
@pytest.mark.parametrize("case", META, ids=[c["name"] for c in META])
def test_gpu8_reference_pins(case):
    dp, dn, arrs, labels = _case(case)
    label, smin, smax, r = _gpu8(dp, dn, case["penalty"], arrs)
    assert np.array_equal(label, labels)
    assert r["ref_energy"] == case["ref_energy"] and r["flow"] == case["oracle_flow"]
    o = O.solve8(dp, dn, penalty=case["penalty"], arrays=None if arrs is None else [arrs[k] for k in DIRS])
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(6))
def test_gpu8_random_vs_oracle(seed):
    rng = np.random.default_rng(8800 + seed)
    for _ in range(4):
        H, W = (int(v) for v in rng.integers(3, 160, 2))
        dp = rng.integers(0, 400, (H, W)).astype(np.int32)
        dn = rng.integers(0, 400, (H, W)).astype(np.int32)
        if rng.random() < 0.5:
            arrs = {k: rng.integers(0, int(rng.integers(1, 200)), (H, W)).astype(np.int32) for k in DIRS}
            pen = 0
        else:
            arrs, pen = None, int(rng.integers(0, 120))
        label, smin, smax, r = _gpu8(dp, dn, pen, arrs)
        o = O.solve8(dp, dn, penalty=pen, arrays=None if arrs is None else [arrs[k] for k in DIRS])
        assert r["flow"] == o["flow"]
        assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])
        assert np.array_equal(label, o["smax"].astype(np.int32))


@pytest.mark.gpu
def test_gpu8_640x480_vs_oracle():
    """The size the reference's slides quote for its 8-neighbourhood."""
    rng = np.random.default_rng(8900)
    H, W = 480, 640
    yy, xx = np.mgrid[0:H, 0:W]
    inside = (xx - 300) ** 2 + (yy - 220) ** 2 < 150 ** 2
    dp = (np.where(inside, 60, 10) + rng.integers(0, 40, (H, W))).astype(np.int32)
    dn = (np.where(inside, 10, 60) + rng.integers(0, 40, (H, W))).astype(np.int32)
    label, smin, smax, r = _gpu8(dp, dn, 25, None)
    o = O.solve8(dp, dn, penalty=25)
    assert r["flow"] == o["flow"] and np.array_equal(smax, o["smax"]) and np.array_equal(smin, o["smin"])


def _serpentine(H, W, period=4, source_first=False):
    """A corridor that winds through the whole image: walls every `period`
    rows with one open pixel, alternately at the right and the left end;
    excess at the far end, sink capacity at the start.  Every residual path
    crosses many 32x32 tiles, so each exact global relabel takes many tile
    rounds, and the heights run to thousands.  source_first: a large excess
    at the start and a small sink capacity at the far end instead, so that
    S_min (the closure of the leftover excess) runs the corridor's length."""
    yy, xx = np.mgrid[0:H, 0:W]
    wall = (yy % period == 0) & (yy > 0)
    gap_x = np.where((yy // period) % 2 == 1, W - 3, 2)
    open_ = ~wall | (xx == gap_x)
    dxs = (-1, 1, 0, 0, -1, 1, -1, 1)
    dys = (0, 0, -1, 1, -1, -1, 1, 1)
    arrs = {}
    for k, dx, dy in zip(DIRS, dxs, dys):
        nb = np.zeros_like(open_)
        nb[max(0, -dy):H - max(0, dy), max(0, -dx):W - max(0, dx)] = \
            open_[max(0, dy):H - max(0, -dy), max(0, dx):W - max(0, -dx)]
        arrs[k] = np.where(open_ & nb, 40, 0).astype(np.int32)
    dp = np.zeros((H, W), np.int32)
    dn = np.zeros((H, W), np.int32)
    if source_first:
        dp[1:3, 1:6] = 500
        dn[H - 3:H - 1, W - 8:W - 1] = 2
    else:
        dn[1:3, 1:6] = 500
        dp[H - 3:H - 1, W - 8:W - 1] = 30
    return dp, dn, arrs


@pytest.mark.gpu
@pytest.mark.parametrize("H,W,source_first", [(130, 150, False), (97, 203, False), (130, 150, True),
                                              (97, 203, True)])
def test_gpu8_serpentine_vs_oracle(H, W, source_first):
    dp, dn, arrs = _serpentine(H, W, source_first=source_first)
    label, smin, smax, r = _gpu8(dp, dn, 0, arrs)
    o = O.solve8(dp, dn, penalty=0, arrays=[arrs[k] for k in DIRS])
    assert o["flow"] > 0
    assert r["flow"] == o["flow"]
    assert np.array_equal(smin, o["smin"]) and np.array_equal(smax, o["smax"])
    assert r["gr_sweeps"] > 3 * r["global_relabels"]  # relabels that took many tile rounds
    if source_first:
        assert smin.sum() > H * W // 2 and r["cut_sweeps"] > 3  # a closure across many tiles


@pytest.mark.gpu
def test_gc_solve8_shim_reproduces_reference_pins(tmp_path):
    lib = gcfg.LIB_PATH
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "gc_solve8")
    libdir = os.path.dirname(lib)
    r = subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "shim",
                        "gc_solve8.cu"), "-o", exe, "-L", libdir, "-lgcfg", f"-Xlinker=-rpath={libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    args, expect = [], []
    for c in META:
        dp, dn, arrs, labels = _case(c)
        ip, op = tmp_path / f"{c['name']}.in", tmp_path / f"{c['name']}.out"
        with open(ip, "wb") as f:
            np.array([c["W"], c["H"], c["penalty"], int(arrs is not None)], "<i4").tofile(f)
            dp.astype("<i4").tofile(f)
            dn.astype("<i4").tofile(f)
            if arrs is not None:
                for k in REF_ORDER:
                    arrs[k].astype("<i4").tofile(f)
        args += [str(ip), str(op)]
        expect.append((c, op, labels))
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    energies = [int(v) for v in re.findall(r"Final energy level: (-?\d+)", r.stdout)]
    for k, (c, op, labels) in enumerate(expect):
        assert np.array_equal(np.fromfile(op, "<i4").reshape(c["H"], c["W"]), labels), c["name"]
        assert energies[k] == c["ref_energy"], c["name"]
