"""The C++ front ends include/GraphCut.h (+ GraphCut.cu) and include/DataTerm.h:
programs written against the reference's GC_* and DataTerm:: names
(tests/shim/*.cu) compile unchanged, link against libgcfg.so, and on a GPU
reproduce the reference's own labels and printed energies."""
import json
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import gcfg
import oracle as O
import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "shim")
GOLDEN = os.path.join(ROOT, "tests", "golden")
META = json.load(open(os.path.join(GOLDEN, "reference_pins.json")))["cases"]
DATA = np.load(os.path.join(GOLDEN, "reference_pins.npz"))


def _nvcc():
    return shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)


@pytest.fixture(scope="module")
def programs(tmp_path_factory):
    if not os.path.exists(gcfg.LIB_PATH):
        pytest.skip("libgcfg.so not built")
    nvcc = _nvcc()
    if not nvcc:
        pytest.skip("nvcc not found")
    out = tmp_path_factory.mktemp("shim")
    libdir = os.path.dirname(gcfg.LIB_PATH)
    exes = {}
    for prog in ("gc_solve", "dt_segment"):
        exe = str(out / prog)
        cmd = [nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"),
               os.path.join(SHIM, prog + ".cu"), "-o", exe, "-L", libdir, "-lgcfg", f"-Xlinker=-rpath={libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        exes[prog] = exe
    return exes


def test_shim_programs_compile_and_link(programs):
    """The reference-style callers build against the headers and the library."""
    for exe in programs.values():
        assert os.access(exe, os.X_OK)
    out = subprocess.run(["nm", "-D", "--undefined-only", programs["dt_segment"]], capture_output=True,
                         text=True).stdout
    for sym in ("gcfg_dt_create", "gcfg_dt_compute", "gcfg_init", "gcfg_optimize"):
        assert sym in out


def _pin(c):
    name = c["name"]
    n = c["W"] * c["H"]
    arrs = [DATA[f"{name}__{k}"].astype(np.int32).ravel() for k in ("dp", "dn")]
    if c["arrays"]:
        arrs += [DATA[f"{name}__{k}"].astype(np.int32).ravel() for k in ("up", "down", "left", "right")]
    labels = np.unpackbits(DATA[f"{name}__ref_labels"])[:n].astype(np.int32)
    hdr = np.array([c["W"], c["H"], c["penalty"], int(c["arrays"])], np.int32)
    return np.concatenate([hdr] + arrs).astype("<i4"), labels


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["once", "resolve"])
def test_graphcut_shim_reproduces_reference_pins(programs, tmp_path, mode):
    """Every pinned instance through GC_Init/GC_Optimize/GC_End compiled
    against the shim: the reference's labels and printed energy."""
    args, expect = [], []
    for c in META:
        inst, labels = _pin(c)
        ip, op = tmp_path / f"{c['name']}.in", tmp_path / f"{c['name']}.out"
        inst.tofile(ip)
        args += [str(ip), str(op)]
        expect.append((c, op, labels))
    r = subprocess.run([programs["gc_solve"], mode] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    energies = [int(v) for v in re.findall(r"Final energy level: (-?\d+)", r.stdout)]
    per = 2 if mode == "resolve" else 1
    assert len(energies) == per * len(META)
    for k, (c, op, labels) in enumerate(expect):
        got = np.fromfile(op, "<i4")
        assert np.array_equal(got, labels), c["name"]
        assert energies[per * k:per * (k + 1)] == [c["ref_energy"]] * per, c["name"]


def _dt_case(seed, W, H):
    rng = np.random.default_rng(seed)
    rgb, _ = synth.generate(0, W, H, seed)
    sel = np.zeros((H, W), np.int32)
    sel[H // 2 - 3:H // 2 + 3, W // 2 - 3:W // 2 + 3] = 1
    sel[:2, :] = 2
    ops = [(int(rng.integers(0, W)), int(rng.integers(0, H)), int(rng.integers(1, 3))) for _ in range(6)]
    ops += [(W - 2, H - 3, 1), (W - 1, 0, 2)]  # squares clipped at the border
    expect = sel.copy()
    for x, y, cls in ops:
        expect[max(y, 0):min(y + 5, H), max(x, 0):min(x + 5, W)] = cls
    return rgb, sel, ops, expect.astype(np.uint8)


@pytest.mark.gpu
@pytest.mark.parametrize("seed,W,H,penalty", [(1, 64, 48, 20), (2, 97, 61, 50), (3, 200, 130, 5)])
def test_dataterm_shim_matches_oracle(programs, tmp_path, seed, W, H, penalty):
    rgb, sel, ops, scrib = _dt_case(seed, W, H)
    f = tmp_path / "in.bin"
    with open(f, "wb") as fh:
        np.array([W, H, penalty, len(ops)], "<i4").tofile(fh)
        rgb.astype(np.uint8).tofile(fh)
        sel.astype("<i4").tofile(fh)
        np.array(ops, "<i4").ravel().tofile(fh)
    pre = str(tmp_path / "out")
    r = subprocess.run([programs["dt_segment"], str(f), pre], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    dp, dn = O.tlinks(rgb, scrib)
    assert np.array_equal(np.fromfile(pre + ".pos", "<i4").reshape(H, W), dp)
    assert np.array_equal(np.fromfile(pre + ".neg", "<i4").reshape(H, W), dn)
    o = O.solve(dp, dn, penalty=penalty)
    assert np.array_equal(np.fromfile(pre + ".label", "<i4").reshape(H, W), o["smax"].astype(np.int32))
    drawn = rgb.copy()
    drawn[scrib == 1] = (0, 0, 255)  # K_DrawMap: map entries equal to 1 only
    assert np.array_equal(np.fromfile(pre + ".draw", np.uint8).reshape(H, W, 3), drawn)


@pytest.mark.gpu
def test_dataterm_python_mirror():
    """gcfg.DataTerm with the reference's names; t-links equal the oracle's."""
    torch = pytest.importorskip("torch")
    W, H = 80, 56
    rgb, sel, ops, scrib = _dt_case(9, W, H)
    DT = gcfg.DataTerm
    DT.init_data_term(W, H)
    DT.setSigmaGaussian(7)
    DT.setImage(rgb)
    DT.setSelection(sel)
    for x, y, cls in ops:
        (DT.selectOnMap(x, y, 5) if cls == 1 else DT.selectBackgroundOnMap(x, y))
    DT.getDataTermsMixture()
    dp, dn = O.tlinks(rgb, scrib)
    pos = torch.as_tensor(DT.getPos(), device="cuda").cpu().numpy().reshape(H, W)
    neg = torch.as_tensor(DT.getNeg(), device="cuda").cpu().numpy().reshape(H, W)
    assert np.array_equal(pos, dp) and np.array_equal(neg, dn)
    # the t-link arrays go straight into the graph API
    gw = gcfg.GC_Init(W, H, DT.getPos(), DT.getNeg(), 30)
    label = np.zeros((H, W), np.int32)
    gcfg.GC_Optimize(gw, label)
    gcfg.GC_End(gw)
    assert np.array_equal(label, O.solve(dp, dn, penalty=30)["smax"].astype(np.int32))
    # reset clears the selection: no scribbles, both classes uniform
    DT.reset()
    DT.getDataTermsMixture()
    pos = torch.as_tensor(DT.getPos(), device="cuda").cpu().numpy()
    assert np.all(pos == pos[0])
    DT.free_data_term()
    with pytest.raises(gcfg.GcfgError):
        DT.getPos()


def test_dataterm_namespace_requires_init():
    """Like calling the reference's DataTerm functions before init_data_term,
    but an error instead of a null dereference (no GPU needed)."""
    gcfg.DataTerm._state = None
    with pytest.raises(gcfg.GcfgError) as ei:
        gcfg.DataTerm.getPos()
    assert ei.value.status == gcfg.GCFG_ERR_STATE
