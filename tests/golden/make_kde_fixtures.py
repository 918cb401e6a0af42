"""Golden outputs of the reference's kernel-density data term.

Runs the reference's own DataTerm.cpp (with DataTermKernels.cu), built for
the CPU thread emulator by oracle/refemu/build_ref.sh, through
oracle/refemu/dt_harness.cpp: init_data_term, setSigmaGaussian, setImage,
selectOnMap at each listed point (in order), getDataTermsMixture.  Stores the
inputs, the reference's 101-entry Gaussian table and its pos/neg t-links in
tests/golden/kde/<case>.npz.  Image sides are multiples of 16 (the
reference's per-pixel kernels cover whole 16x16 blocks only) and every 5x5
selection square lies inside the image (the reference does not clip).
Slow: each selectOnMap is 25 emulated launches of 256^3 threads (minutes).
Usage: python tests/golden/make_kde_fixtures.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "kde")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "dt_harness")

CASES = {
    # name: (W, H, sigma, seed, points)
    "s5": (32, 16, 5, 21, [(3, 4), (5, 6), (20, 9)]),
    "s9": (16, 32, 9, 22, [(2, 2), (9, 20), (9, 21)]),
}


def main():
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "refemu", "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    os.makedirs(OUT, exist_ok=True)
    for name, (W, H, sigma, seed, pts) in CASES.items():
        rng = np.random.default_rng(seed)
        # two colour clusters plus noise, so that selections overlap in colour
        base = np.where(rng.random((H, W, 1)) < 0.5, [[[200, 60, 60]]], [[[60, 120, 200]]])
        img = np.clip(base + rng.normal(0, 25, (H, W, 3)), 0, 255).astype(np.uint8)
        inp = os.path.join(OUT, f".{name}.in")
        outp = os.path.join(OUT, f".{name}.out")
        with open(inp, "wb") as f:
            np.array([W, H, sigma, len(pts)], "<i4").tofile(f)
            img.tofile(f)
            np.array(pts, "<i4").ravel().tofile(f)
        subprocess.run([HARNESS, inp, outp], check=True)
        raw = open(outp, "rb").read()
        gauss = np.frombuffer(raw[:404], "<f4")
        pos = np.frombuffer(raw[404:404 + 4 * W * H], "<i4").reshape(H, W)
        neg = np.frombuffer(raw[404 + 4 * W * H:], "<i4").reshape(H, W)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), img=img, sigma=sigma, points=np.array(pts, np.int32),
                            gauss=gauss, pos=pos, neg=neg)
        os.remove(inp)
        os.remove(outp)
        print(name, "done", int(pos.min()), int(pos.max()))


if __name__ == "__main__":
    main()
