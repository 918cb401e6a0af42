"""Helpers shared by the GPU tests (device buffers via torch)."""
import numpy as np
import torch

import gcfg
import oracle as O


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_solve(dp, dn, penalty=0, up=None, down=None, left=None, right=None, schedule=None):
    """Solve through the reference-style graph API; returns labels (host),
    smin/smax (host) and the result record."""
    H, W = dp.shape
    t = [None if a is None else dev(a.astype(np.int32)) for a in (dp, dn, up, down, left, right)]
    gw = gcfg.GC_Init(W, H, t[0], t[1], penalty, *t[2:])
    if schedule:
        gcfg.GC_SetSchedule(gw, *schedule)
    label = np.zeros((H, W), np.int32)
    res = gcfg.GC_Optimize(gw, label)
    smin = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    smax = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    gcfg.GC_GetCuts(gw, smin, smax)
    gcfg.GC_End(gw)
    return label, smin.cpu().numpy(), smax.cpu().numpy(), res


def gpu_segment(rgb, scrib, lam, seg=None):
    H, W = scrib.shape
    s = seg or gcfg.Segmenter(W, H)
    smin = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    smax = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    res = s.run(dev(rgb), dev(scrib), W, H, lam, smin, smax)
    return smin.cpu().numpy(), smax.cpu().numpy(), res
