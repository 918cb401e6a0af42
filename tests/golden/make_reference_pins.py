"""Generate tests/golden/reference_pins.npz: outputs of the reference's own
solver on fixed instances.

The reference (bfiss/gc-fg) is CUDA-only and ships no tests or golden
vectors.  Its unmodified GraphCut.cu / GraphCutKernels.cu are compiled for a
CPU thread emulator by oracle/refemu/build_ref.sh and driven through
GC_Init / GC_Optimize / GC_End by oracle/refemu/ref_harness.cpp.  For each
instance this script stores the inputs, the label array the reference
returns (GraphCut.cu:528-529) and the energy it prints
(GraphCut.cu:456-457), so that the oracle can be checked against the
reference without the reference checkout being present.

Run here (needs the reference checkout):  python tests/golden/make_reference_pins.py
"""
from __future__ import annotations

import json
import os
import re
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

REF = os.environ.get("GCFG_REFERENCE_DIR", "/root/reference")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
OUT_NPZ = os.path.join(ROOT, "tests", "golden", "reference_pins.npz")
OUT_JSON = os.path.join(ROOT, "tests", "golden", "reference_pins.json")


def debug_instance():
    """The hand-written 15x4 instance of the reference's Debug.cu."""
    src = open(os.path.join(REF, "Debug.cu")).read()
    vals = {}
    for name in ("data_positive", "data_negative"):
        m = re.search(name + r"\[SIZE\]\s*=\s*\{([^}]*)\}", src)
        vals[name] = [int(v) for v in re.findall(r"-?\d+", m.group(1))]
    m = re.search(r"\n\s*height\s*=\s*(\d+);\s*\n\s*width\s*=\s*(\d+);", src)
    h, w = int(m.group(1)), int(m.group(2))
    pen = int(re.search(r"GC_Init\(width,\s*height,\s*d_data_positive,\s*d_data_negative,\s*(\d+)\)", src).group(1))
    dp = np.array(vals["data_positive"][: w * h], np.int32).reshape(h, w)
    dn = np.array(vals["data_negative"][: w * h], np.int32).reshape(h, w)
    return dict(dp=dp, dn=dn, penalty=pen)


def cases():
    out = []
    d = debug_instance()
    out.append(("debug_15x4", d["dp"], d["dn"], d["penalty"], None))
    rng = np.random.default_rng(2012)
    # Debug.cu-style random t-links 0..299 with the constant penalty 50
    for (h, w) in [(16, 16), (32, 32), (40, 40), (64, 64), (48, 45), (33, 70), (9, 100), (128, 128)]:
        dp = rng.integers(0, 300, (h, w)).astype(np.int32)
        dn = rng.integers(0, 300, (h, w)).astype(np.int32)
        out.append((f"rand_pen50_{h}x{w}", dp, dn, 50, None))
    # per-direction (directed) caps, as GC_Init's up/down/left/right arrays
    for (h, w, cmax) in [(32, 32, 100), (37, 53, 100), (64, 64, 40), (24, 96, 300)]:
        dp = rng.integers(0, 300, (h, w)).astype(np.int32)
        dn = rng.integers(0, 300, (h, w)).astype(np.int32)
        arrs = tuple(rng.integers(0, cmax, (h, w)).astype(np.int32) for _ in range(4))
        out.append((f"rand_arrays_{h}x{w}_c{cmax}", dp, dn, 0, arrs))
    # segmentation instances from the synthetic families (histogram t-links,
    # contrast-sensitive n-links)
    for (cfg, w, h, seed, lam) in [(3, 64, 64, 1000, 50.0), (3, 96, 64, 1001, 50.0),
                                   (3, 80, 112, 1002, 50.0), (1, 128, 96, 7, 10.0),
                                   (1, 128, 96, 7, 200.0), (2, 96, 96, 2, 100.0)]:
        rgb, scrib = O.generate(cfg, w, h, seed)
        dp, dn = O.tlinks(rgb, scrib)
        up, down, left, right = O.nlinks(rgb, lam)
        out.append((f"seg_cfg{cfg}_{w}x{h}_s{seed}_l{int(lam)}", dp, dn, 0, (up, down, left, right)))
    # Application.cu / DataTerm-style scale: (int)(300000 p), penalty 600
    p = rng.random((48, 64))
    out.append(("dataterm_scale_48x64", (300000.0 * p).astype(np.int32),
                (300000.0 * (1 - p)).astype(np.int32), 600, None))
    # edge cases
    out.append(("tiny_3x3", np.array([[0, 0, 0], [0, 7, 0], [0, 0, 0]], np.int32),
                np.array([[0, 0, 0], [0, 3, 0], [0, 0, 0]], np.int32), 5, None))
    out.append(("strip_3x20", rng.integers(0, 50, (3, 20)).astype(np.int32),
                rng.integers(0, 50, (3, 20)).astype(np.int32), 10, None))
    out.append(("strip_20x3", rng.integers(0, 50, (20, 3)).astype(np.int32),
                rng.integers(0, 50, (20, 3)).astype(np.int32), 10, None))
    z = np.zeros((20, 20), np.int32)
    out.append(("zeros_20x20", z, z.copy(), 7, None))
    ties = rng.integers(0, 100, (20, 20)).astype(np.int32)
    out.append(("ties_20x20", ties, ties.copy(), 9, None))
    out.append(("all_source_24x24", rng.integers(1, 100, (24, 24)).astype(np.int32),
                np.zeros((24, 24), np.int32), 1000, None))
    out.append(("all_sink_24x24", np.zeros((24, 24), np.int32),
                rng.integers(1, 100, (24, 24)).astype(np.int32), 1000, None))
    out.append(("pen0_24x24", rng.integers(0, 100, (24, 24)).astype(np.int32),
                rng.integers(0, 100, (24, 24)).astype(np.int32), 0, None))
    # a long path: strong source on the left column, strong sink on the right
    dp = np.zeros((10, 120), np.int32)
    dn = np.zeros((10, 120), np.int32)
    dp[:, 1] = 1000
    dn[:, -2] = 1000
    out.append(("long_path_10x120", dp, dn, 3, None))
    return out


def run_reference(dp, dn, penalty, arrs):
    h, w = dp.shape
    with tempfile.TemporaryDirectory() as td:
        inst = os.path.join(td, "inst.bin")
        lab = os.path.join(td, "lab.bin")
        with open(inst, "wb") as f:
            f.write(struct.pack("<4i", w, h, 1 if arrs is not None else 0, int(penalty)))
            f.write(dp.astype("<i4").tobytes())
            f.write(dn.astype("<i4").tobytes())
            if arrs is not None:
                for a in arrs:
                    f.write(a.astype("<i4").tobytes())
        res = subprocess.run([HARNESS, inst, lab], capture_output=True, text=True, timeout=3600)
        if res.returncode:
            raise RuntimeError(res.stderr)
        labels = np.fromfile(lab, "<i4").reshape(h, w)
    energy = int(re.search(r"Final energy level: (-?\d+)", res.stdout).group(1))
    iters = int(re.search(r"Graph Cut used (\d+) iterations", res.stdout).group(1))
    return labels, energy, iters


def small(a):
    a = np.asarray(a)
    if a.min() >= -32768 and a.max() <= 32767:
        return a.astype(np.int16)
    return a.astype(np.int32)


def main():
    subprocess.check_call([os.path.join(ROOT, "oracle", "refemu", "build_ref.sh")])
    arrays = {}
    summary = []
    for name, dp, dn, pen, arrs in cases():
        labels, energy, iters = run_reference(dp, dn, pen, arrs)
        kw = {} if arrs is None else dict(up=arrs[0], down=arrs[1], left=arrs[2], right=arrs[3])
        r = O.solve(dp, dn, penalty=pen, **kw)
        agree = bool((labels == r["smax"]).all()) and energy == O.reference_energy(dp, r["excess"])
        arrays[f"{name}__dp"] = small(dp)
        arrays[f"{name}__dn"] = small(dn)
        if arrs is not None:
            for k, a in zip(("up", "down", "left", "right"), arrs):
                arrays[f"{name}__{k}"] = small(a)
        arrays[f"{name}__ref_labels"] = np.packbits(labels.astype(np.uint8).reshape(-1))
        summary.append(dict(name=name, W=int(dp.shape[1]), H=int(dp.shape[0]), penalty=int(pen),
                            arrays=arrs is not None, ref_energy=energy, ref_iterations=iters,
                            oracle_flow=int(r["flow"]), oracle_agrees=agree))
        print(f"{name:32s} iters {iters:5d} ref_energy {energy:11d} oracle_flow {r['flow']:11d} agree {agree}",
              flush=True)
    np.savez_compressed(OUT_NPZ, **arrays)
    with open(OUT_JSON, "w") as f:
        json.dump(dict(generator="tests/golden/make_reference_pins.py",
                       reference_build="oracle/refemu/build_ref.sh (reference GraphCut.cu on a CPU thread emulator)",
                       cases=summary), f, indent=1)
    print("wrote", OUT_NPZ, os.path.getsize(OUT_NPZ), "bytes")


if __name__ == "__main__":
    main()
