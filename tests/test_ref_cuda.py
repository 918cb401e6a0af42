"""The reference's own CUDA path on the GPU (its kernels compiled from its
sources, driven by oracle/refgpu/ref_gpu.cpp) against the pins made by the
reference on the CPU emulator, and against this repository's solver.

This checks the baseline that bench.py times beside the product: the
reference's kernels on a GB300 must reproduce the reference's own labels and
printed energy (GraphCut.cu:456-457, 507-529)."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import oracle as O  # noqa: E402
import ref_cuda  # noqa: E402
from gpu_util import gpu_solve  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(GOLDEN, "reference_pins.json")))["cases"]
DATA = np.load(os.path.join(GOLDEN, "reference_pins.npz"))


@pytest.fixture(scope="module", autouse=True)
def _need_kernels():
    why = ref_cuda.unavailable()
    if why:
        pytest.skip(why)


def _case(c):
    name = c["name"]
    kw = {"penalty": c["penalty"]}
    if c["arrays"]:
        for k in ("up", "down", "left", "right"):
            kw[k] = DATA[f"{name}__{k}"].astype(np.int32)
    n = c["W"] * c["H"]
    labels = np.unpackbits(DATA[f"{name}__ref_labels"])[:n].reshape(c["H"], c["W"])
    return DATA[f"{name}__dp"].astype(np.int32), DATA[f"{name}__dn"].astype(np.int32), kw, labels


@pytest.mark.parametrize("case", META, ids=[c["name"] for c in META])
def test_reference_cuda_reproduces_pins(case):
    dp, dn, kw, ref_labels = _case(case)
    r = ref_cuda.solve(dp, dn, max_seconds=20.0, **kw)
    assert r["rc"] == 0, r["status"]
    assert r["converged"] == 1
    assert r["energy"] == case["ref_energy"]
    assert np.array_equal(r["label"], ref_labels.astype(np.int32))


@pytest.mark.parametrize("cfg,W,H,seed,lam", [(0, 256, 256, 0, 50.0), (3, 200, 120, 1001, 50.0),
                                              (1, 480, 270, 3, 200.0)])
def test_reference_cuda_matches_product_on_segmentation(cfg, W, H, seed, lam):
    """A segmentation graph: the reference's labels on the GPU equal S_max of
    this repository's solver and its printed energy equals ref_energy."""
    rgb, scrib = O.generate(cfg, W, H, seed)
    dp, dn = O.tlinks(rgb, scrib)
    up, down, left, right = O.nlinks(rgb, lam)
    r = ref_cuda.solve(dp, dn, up=up, down=down, left=left, right=right, max_seconds=30.0)
    assert r["rc"] == 0, r["status"]
    label, smin, smax, res = gpu_solve(dp, dn, up=up, down=down, left=left, right=right)
    assert r["energy"] == res["ref_energy"]
    assert np.array_equal(r["label"], label)
    assert np.array_equal(r["label"].astype(np.uint8), smax)


META8 = json.load(open(os.path.join(GOLDEN, "reference_pins8.json")))["cases"]
DATA8 = np.load(os.path.join(GOLDEN, "reference_pins8.npz"))
REF_ORDER8 = ("up", "down", "left", "right", "upleft", "upright", "downleft", "downright")


@pytest.mark.parametrize("case", META8, ids=[c["name"] for c in META8])
def test_reference_cuda8_reproduces_pins(case):
    """The NEIGHBORHOOD 8 build of the reference's kernels on the GPU gives the
    labels and printed energy the reference gave on the CPU emulator."""
    if ref_cuda.unavailable(8):
        pytest.skip(ref_cuda.unavailable(8))
    name = case["name"]
    dp = DATA8[f"{name}__dp"].astype(np.int32)
    dn = DATA8[f"{name}__dn"].astype(np.int32)
    arrays = [DATA8[f"{name}__{k}"].astype(np.int32) for k in REF_ORDER8] if case["arrays"] else None
    n = case["W"] * case["H"]
    labels = np.unpackbits(DATA8[f"{name}__ref_labels"])[:n].reshape(case["H"], case["W"]).astype(np.int32)
    r = ref_cuda.solve8(dp, dn, penalty=case["penalty"], arrays=arrays, max_seconds=20.0)
    assert r["rc"] == 0, r["status"]
    assert r["energy"] == case["ref_energy"]
    assert np.array_equal(r["label"], labels)
