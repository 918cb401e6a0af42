"""Golden outputs of the reference's MRF applications on synthetic inputs.

Runs, in this container, the reference's own programs built by
oracle/refemu/build_ref.sh for the CPU thread emulator:
  * solveMRF (solveMRF.cu): two-label MRF file -> "Final energy level" line
    and labelMRF.ppm;
  * Application (Application.cu): rihanna.dat + rihanna.ppm -> label.ppm
    (constant penalty 600);
  * multiplyMRF_tile (multiplyMRF.cpp, general tiling mode) and multiplyMRF
    (its fixed 3600x3600 mode) -> MRF text on stdout (stored as sha256).
Inputs are seeded synthetic arrays (the reference's datasets are not in its
checkout).  Writes tests/golden/mrf/: the inputs, the reference's image
outputs and golden.json.  Usage: python tests/golden/make_mrf_fixtures.py
"""
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "gc-fg_gb300")]
import mrf  # noqa: E402

OUT = os.path.join(HERE, "mrf")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def synthetic_mrf(W, H, seed):
    """t-links favouring the source inside a disc, noisy cues."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W]
    inside = (xx - W * 0.45) ** 2 + (yy - H * 0.55) ** 2 < (0.3 * min(W, H)) ** 2
    dp = np.where(inside, 60, 10) + rng.integers(0, 40, (H, W))
    dn = np.where(inside, 10, 60) + rng.integers(0, 40, (H, W))
    hc = rng.integers(0, 45, (H, W - 1))
    vc = rng.integers(0, 45, (H - 1, W))
    gt = inside.astype(np.int64)
    return dp, dn, hc, vc, gt


def run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {r.stderr.decode()[-2000:]}")
    return r.stdout


def main():
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "refemu", "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    os.makedirs(OUT, exist_ok=True)
    work = os.path.join(OUT, ".work")
    shutil.rmtree(work, ignore_errors=True)
    os.makedirs(work)
    golden = {"solve": {}, "tile": {}, "square": {}, "application": {}}
    try:
        for name, (W, H, seed) in {"small": (53, 37, 11), "wide": (131, 97, 12)}.items():
            dp, dn, hc, vc, gt = synthetic_mrf(W, H, seed)
            path = os.path.join(OUT, f"{name}.mrf")
            mrf.write_mrf(path, dp, dn, hc, vc, gt)
            out = run([os.path.join(REF_BIN, "solveMRF"), path], work).decode()
            energy = int(re.findall(r"Final energy level: (-?\d+)", out)[-1])
            shutil.copy(os.path.join(work, "labelMRF.ppm"), os.path.join(OUT, f"{name}.labelMRF.ppm"))
            golden["solve"][name] = {"W": W, "H": H, "final_energy": energy,
                                     "header": out.splitlines()[0]}
            for mult in (1, 3):
                txt = run([os.path.join(REF_BIN, "multiplyMRF_tile"), path, str(mult)], work)
                golden["tile"][f"{name}_x{mult}"] = {"sha256": hashlib.sha256(txt).hexdigest(), "bytes": len(txt)}
        # the fixed 3600x3600 mode reads rihanna.dat (H W, sink then source t-links)
        rng = np.random.default_rng(13)
        sq_dp = rng.integers(0, 90, (3600, 5))
        sq_dn = rng.integers(0, 90, (3600, 5))
        mrf.write_dat(os.path.join(work, "rihanna.dat"), sq_dp, sq_dn)
        shutil.copy(os.path.join(work, "rihanna.dat"), os.path.join(OUT, "square.dat"))
        txt = run([os.path.join(REF_BIN, "multiplyMRF"), os.path.join(OUT, "small.mrf"), "1"], work)
        golden["square"] = {"sha256": hashlib.sha256(txt).hexdigest(), "bytes": len(txt)}
        # the demo application: rihanna.dat + rihanna.ppm -> label.ppm, penalty 600
        W, H = 48, 40
        dp, dn, _, _, _ = synthetic_mrf(W, H, 14)
        dp = dp * 20
        dn = dn * 20
        mrf.write_dat(os.path.join(work, "rihanna.dat"), dp, dn)
        img = np.random.default_rng(15).integers(0, 256, (H, W, 3))
        mrf.write_ppm_ascii(os.path.join(work, "rihanna.ppm"), img)
        out = run([os.path.join(REF_BIN, "Application")], work).decode()
        shutil.copy(os.path.join(work, "rihanna.dat"), os.path.join(OUT, "app.dat"))
        shutil.copy(os.path.join(work, "rihanna.ppm"), os.path.join(OUT, "app.ppm"))
        shutil.copy(os.path.join(work, "label.ppm"), os.path.join(OUT, "app.label.ppm"))
        golden["application"] = {"W": W, "H": H, "penalty": 600,
                                 "final_energy": int(re.findall(r"Final energy level: (-?\d+)", out)[-1])}
    finally:
        shutil.rmtree(work, ignore_errors=True)
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    print(json.dumps(golden, indent=1))


if __name__ == "__main__":
    main()
