"""Two-label MRF files, the solveMRF / Application / multiplyMRF tools.

Golden outputs come from the reference's own programs run on synthetic
inputs (tests/golden/make_mrf_fixtures.py).  CPU tests pin the formats, the
reference's cue-to-graph mapping (through the oracle) and the tiler; GPU
tests run the command-line tools built on this library."""
import hashlib
import json
import os
import re
import subprocess

import numpy as np
import pytest

import mrf
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
G = os.path.join(ROOT, "tests", "golden", "mrf")
GOLD = json.load(open(os.path.join(G, "golden.json")))
BIN = os.path.join(ROOT, "gc-fg_gb300", "bin")


def _tool(name):
    exe = os.path.join(BIN, name)
    if not os.path.exists(exe):
        import build_lib
        try:
            build_lib.build_tools()
        except Exception as e:  # no nvcc / library: nothing to test here
            pytest.skip(f"tools not built: {e}")
    return exe


@pytest.mark.parametrize("name", ["small", "wide"])
def test_python_tiler_matches_reference(name):
    m = mrf.read_mrf(os.path.join(G, f"{name}.mrf"))
    for mult in (1, 3):
        text = mrf.tile_mrf_text(m, mult).encode()
        assert hashlib.sha256(text).hexdigest() == GOLD["tile"][f"{name}_x{mult}"]["sha256"]


@pytest.mark.parametrize("name", ["small", "wide"])
def test_cli_tiler_matches_reference(name):
    exe = _tool("multiply_mrf")
    for mult in (1, 3):
        out = subprocess.run([exe, os.path.join(G, f"{name}.mrf"), str(mult)], capture_output=True, check=True).stdout
        assert hashlib.sha256(out).hexdigest() == GOLD["tile"][f"{name}_x{mult}"]["sha256"]


def test_square_mode_matches_reference():
    exe = _tool("multiply_mrf")
    out = subprocess.run([exe, "--square", os.path.join(G, "square.dat")], capture_output=True, check=True).stdout
    assert len(out) == GOLD["square"]["bytes"]
    assert hashlib.sha256(out).hexdigest() == GOLD["square"]["sha256"]
    W, H, dp, dn = mrf.read_dat(os.path.join(G, "square.dat"))
    assert hashlib.sha256(mrf.square_mrf_text(dp, dn).encode()).hexdigest() == GOLD["square"]["sha256"]


@pytest.mark.parametrize("name", ["small", "wide"])
def test_cue_mapping_reproduces_solvemrf(name):
    """The reference's graph of an MRF file, solved by the oracle, gives the
    reference solveMRF's labelMRF.ppm byte for byte and its printed energy."""
    m = mrf.read_mrf(os.path.join(G, f"{name}.mrf"))
    dp, dn, up, down, left, right = mrf.graph_arrays(m)
    o = O.solve(dp, dn, up=up, down=down, left=left, right=right)
    assert mrf.label_ppm_bytes(o["smax"]) == open(os.path.join(G, f"{name}.labelMRF.ppm"), "rb").read()
    assert O.reference_energy(dp, o["excess"]) == GOLD["solve"][name]["final_energy"]


def test_application_overlay_with_oracle():
    W, H, dp, dn = mrf.read_dat(os.path.join(G, "app.dat"))
    img = mrf.read_ppm_ascii(os.path.join(G, "app.ppm"))
    o = O.solve(dp, dn, penalty=GOLD["application"]["penalty"])
    assert mrf.overlay_ppm_bytes(o["smax"], img) == open(os.path.join(G, "app.label.ppm"), "rb").read()
    assert O.reference_energy(dp, o["excess"]) == GOLD["application"]["final_energy"]


def test_reader_rejects_bad_files(tmp_path):
    bad = tmp_path / "three.mrf"
    bad.write_text("2 2 3 " + "0 " * 20)
    with pytest.raises(ValueError):
        mrf.read_mrf(bad)
    short = tmp_path / "short.mrf"
    short.write_text("4 3 2 " + "1 " * 20)
    with pytest.raises(ValueError):
        mrf.read_mrf(short)
    r = subprocess.run([_tool("multiply_mrf"), str(short), "2"], capture_output=True)
    assert r.returncode == 1 and b"expected an integer" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small", "wide"])
def test_solve_mrf_cli(name, tmp_path):
    out = tmp_path / "labels.ppm"
    r = subprocess.run([_tool("solve_mrf"), os.path.join(G, f"{name}.mrf"), str(out)], capture_output=True,
                       text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == open(os.path.join(G, f"{name}.labelMRF.ppm"), "rb").read()
    assert r.stdout.splitlines()[0] == GOLD["solve"][name]["header"]
    assert int(re.findall(r"Final energy level: (-?\d+)", r.stdout)[-1]) == GOLD["solve"][name]["final_energy"]
    # default output name, like the reference's program
    r = subprocess.run([_tool("solve_mrf"), os.path.join(G, f"{name}.mrf")], capture_output=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0 and (tmp_path / "labelMRF.ppm").read_bytes() == out.read_bytes()


@pytest.mark.gpu
def test_segment_dat_cli(tmp_path):
    out = tmp_path / "label.ppm"
    r = subprocess.run([_tool("segment_dat"), os.path.join(G, "app.dat"), os.path.join(G, "app.ppm"),
                        str(GOLD["application"]["penalty"]), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == open(os.path.join(G, "app.label.ppm"), "rb").read()
    assert int(re.findall(r"Final energy level: (-?\d+)", r.stdout)[-1]) == GOLD["application"]["final_energy"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small", "wide"])
def test_python_graph_api_on_mrf(name):
    torch = pytest.importorskip("torch")
    import gcfg
    m = mrf.read_mrf(os.path.join(G, f"{name}.mrf"))
    arrs = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in mrf.graph_arrays(m)]
    gw = gcfg.GC_Init(m["W"], m["H"], arrs[0], arrs[1], 0, *arrs[2:])
    label = np.zeros((m["H"], m["W"]), np.int32)
    r = gcfg.GC_Optimize(gw, label)
    gcfg.GC_End(gw)
    assert mrf.label_ppm_bytes(label) == open(os.path.join(G, f"{name}.labelMRF.ppm"), "rb").read()
    assert r["ref_energy"] == GOLD["solve"][name]["final_energy"]
