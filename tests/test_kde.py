"""The reference's kernel-density data term (DataTerm model GCFG_DT_KDE).

Goldens: the reference's own DataTerm.cpp run on the CPU emulator
(tests/golden/make_kde_fixtures.py).  The oracle restatement reproduces them
bit for bit from their Gaussian table; the GPU reproduces the oracle bit for
bit from its own table, and the two tables agree to 2 ulp (the emulator
evaluates expf with the host library, the GPU with CUDA's)."""
import glob
import os

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "kde", "*.npz")))


def _selected(img, points):
    return np.concatenate([O.kde_select(img, x, y) for x, y in points])


def _ulps(a, b):
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


@pytest.mark.parametrize("case", CASES, ids=[os.path.basename(c) for c in CASES])
def test_oracle_reproduces_reference_kde(case):
    g = np.load(case)
    sel = _selected(g["img"], g["points"])
    pos, neg = O.kde_terms(g["gauss"], sel, g["img"])
    assert np.array_equal(pos, g["pos"]) and np.array_equal(neg, g["neg"])
    assert _ulps(O.kde_gauss(int(g["sigma"])), g["gauss"]).max() <= 2


def test_kde_golden_cases_exist():
    assert len(CASES) >= 2


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[os.path.basename(c) for c in CASES])
def test_gpu_kde_matches_reference(case):
    torch = pytest.importorskip("torch")
    import gcfg
    g = np.load(case)
    img = g["img"]
    H, W = img.shape[:2]
    dt = gcfg.DataTermState(W, H)
    dt.set_model("kde")
    dt.set_sigma(int(g["sigma"]))
    dt.set_image(img)
    for x, y in g["points"]:
        dt.select_on_map(int(x), int(y), 1)
    dt.compute()
    pos = torch.as_tensor(dt.pos(), device="cuda").cpu().numpy().reshape(H, W)
    neg = torch.as_tensor(dt.neg(), device="cuda").cpu().numpy().reshape(H, W)
    table = dt.kde_table()
    assert _ulps(table, g["gauss"]).max() <= 2
    opos, oneg = O.kde_terms(table, _selected(img, g["points"]), img)
    assert np.array_equal(pos, opos) and np.array_equal(neg, oneg)
    if np.array_equal(table, g["gauss"]):
        assert np.array_equal(pos, g["pos"]) and np.array_equal(neg, g["neg"])
    dt.close()


@pytest.mark.gpu
def test_gpu_kde_edges_resets_and_sigma():
    """Clipped squares at the border, repeated points, a sigma change between
    selections, set_selection (map only) and reset (density cleared)."""
    torch = pytest.importorskip("torch")
    import gcfg
    rng = np.random.default_rng(31)
    H, W = 37, 50
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    dt = gcfg.DataTermState(W, H)
    dt.set_image(img)
    dt.set_model("kde")

    def terms():
        dt.compute()
        return (torch.as_tensor(dt.pos(), device="cuda").cpu().numpy().reshape(H, W),
                torch.as_tensor(dt.neg(), device="cuda").cpu().numpy().reshape(H, W))

    steps = [(3, (-2, -3)), (3, (47, 35)), (3, (10, 10)), (3, (10, 10)), (7, (30, 3)), (7, (-10, 5))]
    sel, tables = [], []
    pos = neg = None
    for sigma, (x, y) in steps:
        dt.set_sigma(sigma)
        dt.select_on_map(x, y, 1)
        tables.append((dt.kde_table(), O.kde_select(img, x, y)))
    pos, neg = terms()
    # the density is a float sum in selection order, each term from the table current then
    exp_pos = np.empty((H, W), np.int32)
    exp_neg = np.empty((H, W), np.int32)
    flat = img.reshape(-1, 3)
    for i in range(H * W):
        p = np.float32(0)
        for table, s in tables:
            for c in s:
                d = int(((flat[i].astype(np.int64) - c) ** 2).sum())
                if d < 101 * 101:
                    p = np.float32(p + table[int(np.floor(np.sqrt(d)))])
        exp_pos.flat[i] = int(300000.0 * float(p))
        exp_neg.flat[i] = int(300000.0 * float(np.float32(1.0) - p))
    assert np.array_equal(pos, exp_pos) and np.array_equal(neg, exp_neg)
    # set_selection only sets the map in this model; class-2 squares only mark it
    dt.set_selection(np.full((H, W), 2, np.int32))
    dt.select_on_map(5, 5, 2)
    assert np.array_equal(terms()[0], pos)
    dt.reset()
    p0, n0 = terms()
    assert (p0 == 0).all() and (n0 == 300000).all()
    dt.close()
