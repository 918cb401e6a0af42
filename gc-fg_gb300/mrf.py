"""Two-label MRF files, label images and overlays (the reference's file formats).

Middlebury two-label MRF text file, as the reference's MRF solver reads it
(solveMRF.cu:10-65), all values whitespace-separated integers:

    W H nLabels          nLabels must be 2
    W*H                  ground-truth labels (read and ignored)
    W*H                  data_positive: source t-links, row-major
    W*H                  data_negative: sink t-links
    H*(W-1)              horizontal cues, row by row: weight of (x,y)-(x+1,y)
    (H-1)*W              vertical cues, row by row: weight of (x,y)-(x,y+1)

The reference hands the cues to the solver as up = down = vertical cue of the
pixel and left = right = horizontal cue of the pixel (solveMRF.cu:87-90): the
capacity from (x, y) to the pixel above is the weight of the edge BELOW it, and
to the left the weight of the edge to its RIGHT.  `graph_arrays` reproduces
that mapping so that the same file gives the same graph and labels.

Image files are ASCII PPM (P3), written byte for byte as the reference's
applications write them: a label map white/black (solveMRF.cu:114-127) or an
overlay keeping the input colour where the label is 1 (Application.cu:52-72).
The ".dat" t-link file of the reference's demo application is "H W", then
W*H sink and W*H source t-links (Application.cu:17-24).
"""
from __future__ import annotations

import numpy as np


def read_mrf(path) -> dict:
    """Parse a two-label MRF file.  Returns W, H, n_labels and int64 arrays
    gt (H, W), dp (H, W), dn (H, W), hcue (H, W-1), vcue (H-1, W)."""
    v = np.fromfile(path, dtype=np.int64, sep=" ")
    if v.size < 3:
        raise ValueError(f"{path}: not an MRF file")
    W, H, L = (int(x) for x in v[:3])
    if L != 2:
        raise ValueError(f"{path}: {L} labels (only 2 are supported)")
    n = W * H
    need = 3 + 3 * n + H * (W - 1) + (H - 1) * W
    if W < 1 or H < 1 or v.size < need:
        raise ValueError(f"{path}: truncated ({v.size} of {need} values)")
    o = 3
    gt = v[o:o + n].reshape(H, W); o += n
    dp = v[o:o + n].reshape(H, W); o += n
    dn = v[o:o + n].reshape(H, W); o += n
    hc = v[o:o + H * (W - 1)].reshape(H, W - 1); o += H * (W - 1)
    vc = v[o:o + (H - 1) * W].reshape(H - 1, W)
    return dict(W=W, H=H, n_labels=L, gt=gt, dp=dp, dn=dn, hcue=hc, vcue=vc)


def _ints(a) -> str:
    return " ".join(str(int(x)) for x in np.asarray(a).ravel())


def write_mrf(path, dp, dn, hcue, vcue, gt=None):
    """Write a two-label MRF file (one section per line)."""
    dp = np.asarray(dp)
    H, W = dp.shape
    gt = np.ones((H, W), np.int64) if gt is None else gt
    with open(path, "w") as f:
        f.write(f"{W} {H} 2\n")
        for a in (gt, dp, dn, hcue, vcue):
            f.write(_ints(a) + "\n")


def graph_arrays(m: dict):
    """int32 (H, W) arrays dp, dn, up, down, left, right of the reference's
    MRF solver.  The last row of both cues and the last column of the
    horizontal cue are 0 (they only reach the 1-pixel border, whose edges the
    solver zeroes)."""
    H, W = m["H"], m["W"]
    vfull = np.zeros((H, W), np.int32)
    vfull[:H - 1, :] = m["vcue"]
    hfull = np.zeros((H, W), np.int32)
    hfull[:H - 1, :W - 1] = m["hcue"][:H - 1]
    dp = m["dp"].astype(np.int32)
    dn = m["dn"].astype(np.int32)
    return dp, dn, vfull, vfull.copy(), hfull, hfull.copy()


def tile_mrf_text(m: dict, mult: int) -> str:
    """An MRF `mult` times as wide, the reference's tiler's general mode
    (multiplyMRF.cpp:64-92): ground truth all 1, t-links repeated with period
    W, horizontal cues with period W - 1, vertical cues with period W.  Like
    the reference, whose loader clears the last row of the cues
    (multiplyMRF.cpp:56-59), the last row of horizontal cues is written as 0."""
    W, H = m["W"], m["H"]
    Wm = W * mult
    parts = [f"{Wm} {H} 2 ", "1 " * (Wm * H)]
    cols = np.arange(Wm) % W
    for a in (m["dp"], m["dn"]):
        parts.append("".join(f"{int(x)} " for x in a[:, cols].ravel()))
    hc = m["hcue"].copy()
    hc[H - 1, :] = 0
    parts.append("".join(f"{int(x)} " for x in hc[:, np.arange(Wm - 1) % (W - 1)].ravel()))
    parts.append("".join(f"{int(x)} " for x in m["vcue"][:, cols].ravel()))
    return "".join(parts)


def square_mrf_text(dp, dn, side: int = 3600, penalty: int = 600) -> str:
    """The reference tiler's fixed mode (multiplyMRF.cpp:94-122): a side x side
    MRF whose t-links repeat the given (H, W) arrays along each row and whose
    every cue is `penalty`.  Row i reads row i of the arrays, so H >= side."""
    dp = np.asarray(dp)
    dn = np.asarray(dn)
    H, W = dp.shape
    if H < side:
        raise ValueError(f"the t-link arrays have {H} rows; the {side}x{side} mode needs at least {side}")
    cols = np.arange(side) % W
    parts = [f"{side} {side} 2 ", "1 " * (side * side)]
    for a in (dp, dn):
        parts.append("".join(f"{int(x)} " for x in a[:side, cols].ravel()))
    parts.append(f"{penalty} " * (side * (side - 1)))
    parts.append(f"{penalty} " * ((side - 1) * side))
    return "".join(parts)


def read_dat(path):
    """The demo application's t-link file: (W, H, dp, dn) with dp/dn int32 (H, W)."""
    v = np.fromfile(path, dtype=np.int64, sep=" ")
    H, W = int(v[0]), int(v[1])
    n = W * H
    dn = v[2:2 + n].reshape(H, W).astype(np.int32)
    dp = v[2 + n:2 + 2 * n].reshape(H, W).astype(np.int32)
    return W, H, dp, dn


def write_dat(path, dp, dn):
    dp = np.asarray(dp)
    H, W = dp.shape
    with open(path, "w") as f:
        f.write(f"{H} {W}\n{_ints(dn)}\n{_ints(dp)}\n")


def label_ppm_bytes(label) -> bytes:
    """P3 image of a label map: (255, 255, 255) where label != 0, else black."""
    lab = np.asarray(label)
    H, W = lab.shape
    rows = [f"P3 {W} {H} 255 \n"]
    for y in range(H):
        rows.append("".join("255 255 255 " if v else "0 0 0 " for v in lab[y]) + "\n")
    return "".join(rows).encode()


def read_ppm_ascii(path):
    """A P3 image as uint8 (H, W, 3)."""
    tok = open(path).read().split()
    if tok[0] != "P3":
        raise ValueError(f"{path}: not an ASCII PPM")
    W, H = int(tok[1]), int(tok[2])
    px = np.array(tok[4:4 + 3 * W * H], dtype=np.int64)
    return px.reshape(H, W, 3).astype(np.uint8)


def write_ppm_ascii(path, img):
    img = np.asarray(img)
    H, W, _ = img.shape
    with open(path, "w") as f:
        f.write(f"P3\n{W} {H}\n255\n")
        for y in range(H):
            f.write(_ints(img[y]) + "\n")


def overlay_ppm_bytes(label, img) -> bytes:
    """P3 image keeping img's colour where label != 0, black elsewhere."""
    lab = np.asarray(label)
    H, W = lab.shape
    rows = [f"P3 {W} {H} 255 \n"]
    for y in range(H):
        rows.append("".join(f"{int(c[0])} {int(c[1])} {int(c[2])} " if v else "0 0 0 "
                            for v, c in zip(lab[y], img[y])) + "\n")
    return "".join(rows).encode()
