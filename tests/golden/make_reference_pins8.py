"""Generate tests/golden/reference_pins8.npz: outputs of the reference's own
solver built with NEIGHBORHOOD == 8 on fixed instances.

The reference's GraphCut.cu / GraphCutKernels.cu, with the NEIGHBORHOOD
switch of its GraphCut.h set to 8 on the fly, are compiled for the CPU
thread emulator by oracle/refemu/build_ref.sh and driven through GC_Init
(eight per-direction arrays, or a constant penalty) / GC_Optimize / GC_End by
oracle/refemu/ref_harness8.cpp.  Stores the inputs, the reference's labels
and its printed energy, and whether the 8-connected oracle agrees.

Run here (needs the reference checkout):  python tests/golden/make_reference_pins8.py
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

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness8")
OUT_NPZ = os.path.join(ROOT, "tests", "golden", "reference_pins8.npz")
OUT_JSON = os.path.join(ROOT, "tests", "golden", "reference_pins8.json")
# order of the arrays in the oracle's and the library's 8-direction API
DIRS = ("left", "right", "up", "down", "upleft", "upright", "downleft", "downright")
# order of the reference's GC_Init arguments
REF_ORDER = ("up", "down", "left", "right", "upleft", "upright", "downleft", "downright")


def cases():
    out = []
    rng = np.random.default_rng(2013)
    for (h, w) in [(16, 16), (33, 29), (48, 64), (96, 80), (9, 100)]:
        dp = rng.integers(0, 300, (h, w)).astype(np.int32)
        dn = rng.integers(0, 300, (h, w)).astype(np.int32)
        out.append((f"rand_pen40_{h}x{w}", dp, dn, 40, None))
    for (h, w, cmax) in [(20, 20, 30), (37, 41, 80), (64, 50, 200), (70, 70, 15)]:
        dp = rng.integers(0, 300, (h, w)).astype(np.int32)
        dn = rng.integers(0, 300, (h, w)).astype(np.int32)
        arrs = {k: rng.integers(0, cmax, (h, w)).astype(np.int32) for k in DIRS}
        out.append((f"rand_arrays_{h}x{w}_c{cmax}", dp, dn, 0, arrs))
    # a segmentation-like instance: a disc of source preference, contrast
    # weights from a noisy image (diagonals from the diagonal differences)
    h, w = 56, 72
    yy, xx = np.mgrid[0:h, 0:w]
    inside = (xx - 30) ** 2 + (yy - 28) ** 2 < 18 ** 2
    img = np.where(inside, 200, 60) + rng.normal(0, 25, (h, w))
    dp = (np.where(inside, 40, 5) + rng.integers(0, 20, (h, w))).astype(np.int32)
    dn = (np.where(inside, 5, 40) + rng.integers(0, 20, (h, w))).astype(np.int32)

    def wgt(dy, dx):
        sh = np.roll(np.roll(img, -dy, 0), -dx, 1)
        return np.round(50 * np.exp(-((img - sh) ** 2) / (2 * 625.0))).astype(np.int32)

    arrs = {"left": wgt(0, -1), "right": wgt(0, 1), "up": wgt(-1, 0), "down": wgt(1, 0), "upleft": wgt(-1, -1),
            "upright": wgt(-1, 1), "downleft": wgt(1, -1), "downright": wgt(1, 1)}
    out.append((f"seg_like_{w}x{h}", dp, dn, 0, arrs))
    out.append(("tiny_3x3", np.array([[0, 0, 0], [0, 7, 0], [0, 0, 0]], np.int32),
                np.array([[0, 0, 0], [0, 3, 0], [0, 0, 0]], np.int32), 5, None))
    out.append(("tiny_4x4", rng.integers(0, 50, (4, 4)).astype(np.int32), rng.integers(0, 50, (4, 4)).astype(np.int32),
                9, None))
    out.append(("strip_3x20", rng.integers(0, 50, (3, 20)).astype(np.int32),
                rng.integers(0, 50, (3, 20)).astype(np.int32), 11, None))
    out.append(("strip_20x3", rng.integers(0, 50, (20, 3)).astype(np.int32),
                rng.integers(0, 50, (20, 3)).astype(np.int32), 11, None))
    z = np.zeros((20, 20), np.int32)
    out.append(("zeros_20x20", z, z.copy(), 7, None))
    ties = np.full((20, 20), 13, np.int32)
    out.append(("ties_20x20", ties, ties.copy(), 9, None))
    out.append(("all_source_24x24", rng.integers(1, 100, (24, 24)).astype(np.int32),
                np.zeros((24, 24), np.int32), 20, None))
    out.append(("all_sink_24x24", np.zeros((24, 24), np.int32),
                rng.integers(1, 100, (24, 24)).astype(np.int32), 20, None))
    out.append(("pen0_24x24", rng.integers(0, 100, (24, 24)).astype(np.int32),
                rng.integers(0, 100, (24, 24)).astype(np.int32), 0, None))
    # diagonal-only connectivity: flow must travel along diagonals
    dp = np.zeros((30, 30), np.int32)
    dn = np.zeros((30, 30), np.int32)
    dp[5, 5] = 500
    dn[24, 24] = 500
    arrs = {k: np.zeros((30, 30), np.int32) for k in DIRS}
    arrs["downright"][:] = 7
    arrs["upleft"][:] = 3
    out.append(("diagonal_only_30x30", dp, dn, 0, arrs))
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
                for k in REF_ORDER:
                    f.write(arrs[k].astype("<i4").tobytes())
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
    subprocess.check_call([os.path.join(ROOT, "oracle", "refemu", "build_ref.sh")], stdout=subprocess.DEVNULL)
    arrays = {}
    summary = []
    for name, dp, dn, pen, arrs in cases():
        labels, energy, iters = run_reference(dp, dn, pen, arrs)
        r = O.solve8(dp, dn, penalty=pen, arrays=None if arrs is None else [arrs[k] for k in DIRS])
        agree = bool((labels == r["smax"]).all()) and energy == O.reference_energy(dp, r["excess"])
        arrays[f"{name}__dp"] = small(dp)
        arrays[f"{name}__dn"] = small(dn)
        if arrs is not None:
            for k in DIRS:
                arrays[f"{name}__{k}"] = small(arrs[k])
        arrays[f"{name}__ref_labels"] = np.packbits(labels.astype(np.uint8).reshape(-1))
        summary.append(dict(name=name, W=int(dp.shape[1]), H=int(dp.shape[0]), penalty=int(pen),
                            arrays=arrs is not None, ref_energy=energy, ref_iterations=iters,
                            oracle_flow=int(r["flow"]), oracle_agrees=agree))
        print(f"{name:28s} iters {iters:5d} ref_energy {energy:9d} oracle_flow {r['flow']:9d} agree {agree}",
              flush=True)
    np.savez_compressed(OUT_NPZ, **arrays)
    with open(OUT_JSON, "w") as f:
        json.dump(dict(generator="tests/golden/make_reference_pins8.py",
                       reference_build="oracle/refemu/build_ref.sh (reference GraphCut.cu, NEIGHBORHOOD 8, "
                                       "on a CPU thread emulator)", cases=summary), f, indent=1)
    print("wrote", OUT_NPZ, os.path.getsize(OUT_NPZ), "bytes")


if __name__ == "__main__":
    main()
