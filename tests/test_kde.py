"""The reference's kernel-density data term (DataTerm model GCFG_DT_KDE).

Goldens: the reference's own DataTerm.cpp run on the CPU emulator
(tests/golden/make_kde_fixtures.py).  The oracle restatement reproduces them
bit for bit from their Gaussian table; the GPU reproduces the oracle bit for
bit from its own table, and the two tables agree to 2 ulp (the emulator
evaluates expf with the host library, the GPU with CUDA's).  On the GPU the
reference's own data-term kernels (DataTermKernels.cu, built from its sources
into oracle/_ref/gc_ref_dt_kernels.cubin) run beside libgcfg's: their
Gaussian table, t-links, selection map and drawSelection output must be equal
bit for bit, with no condition."""
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


def _ref_dt():
    import ref_cuda
    why = ref_cuda.unavailable(0)
    if why:
        pytest.skip(why)
    return ref_cuda


def _ours_kde(img, points, sigma):
    import torch
    import gcfg
    H, W = img.shape[:2]
    dt = gcfg.DataTermState(W, H)
    dt.set_model("kde")
    if sigma > 0:
        dt.set_sigma(int(sigma))
    dt.set_image(img)
    for x, y in points:
        dt.select_on_map(int(x), int(y), 1)
    dt.compute()
    out = dict(pos=torch.as_tensor(dt.pos(), device="cuda").cpu().numpy().reshape(H, W),
               neg=torch.as_tensor(dt.neg(), device="cuda").cpu().numpy().reshape(H, W),
               gauss=dt.kde_table(), dt=dt)
    return out


def _kde_cases():
    cases = []
    for path in CASES:
        g = np.load(path)
        cases.append((os.path.basename(path), g["img"], [tuple(p) for p in g["points"]], int(g["sigma"])))
    rng = np.random.default_rng(77)
    for k, (H, W, sigma, npts) in enumerate([(48, 64, 5, 4), (32, 32, 0, 2), (64, 48, 11, 6)]):
        img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
        img[H // 4:H // 2, W // 4:W // 2] = (20, 200, 90)  # a uniform patch: many equal colours
        pts = [(int(rng.integers(0, W - 4)), int(rng.integers(0, H - 4))) for _ in range(npts)]
        cases.append((f"random{k}", img, pts, sigma))
    return cases


@pytest.mark.gpu
@pytest.mark.parametrize("name,img,points,sigma", _kde_cases(), ids=[c[0] for c in _kde_cases()])
def test_gpu_kde_equals_reference_gpu_kernels(name, img, points, sigma):
    """libgcfg's KDE data term against the reference's own kernels on the
    same GPU: Gaussian table, pos and neg bit for bit (sigma 0 = the default
    table of init_data_term)."""
    pytest.importorskip("torch")
    ref = _ref_dt().kde(img, points, sigma)
    ours = _ours_kde(img, points, sigma)
    assert np.array_equal(ours["gauss"], ref["gauss"])
    assert np.array_equal(ours["pos"], ref["pos"])
    assert np.array_equal(ours["neg"], ref["neg"])
    ours["dt"].close()


@pytest.mark.gpu
def test_draw_selection_equals_reference_gpu_kernel():
    """drawSelection against K_DrawMap on the same GPU: after selectOnMap
    (map entries 1) and after setSelection with labels 0/1/2 (only 1 marks)."""
    pytest.importorskip("torch")
    import gcfg
    ref_cuda = _ref_dt()
    rng = np.random.default_rng(5)
    H, W = 48, 64
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    pts = [(3, 4), (40, 30), (58, 42)]
    ref = ref_cuda.kde(img, pts, 0)
    dt = gcfg.DataTermState(W, H)
    dt.set_model("kde")
    dt.set_image(img)
    for x, y in pts:
        dt.select_on_map(x, y, 1)
    other = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    assert np.array_equal(dt.draw_selection(other), ref_cuda.draw(ref["map"], other))
    labels = rng.integers(0, 3, (H, W)).astype(np.int32)
    dt.set_selection(labels)
    assert np.array_equal(dt.draw_selection(other), ref_cuda.draw(labels.astype(np.uint8), other))
    dt.close()
