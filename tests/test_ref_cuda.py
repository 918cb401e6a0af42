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
