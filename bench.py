"""Benchmark: exact min-cut segmentation throughput on GB300.

Prints ONE JSON line (rank 0).  A step = the full hot path over one batch of
synthetic images: colour-histogram t-links, contrast-sensitive n-links,
graph build, exact max-flow, both canonical cuts.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload plain1080|plain256|plain4096]

value : Mpixel/s with the images already resident in HBM (CUDA events per
        step, L2 flushed before every step).
e2e   : the same metric through the host entry point (gcfg_seg_run_host):
        image + scribbles copied in from pinned host memory and both label
        maps copied back inside the timed region.
roofline: the kernel with the largest device time in a profiled step;
        achieved = algorithmic bytes / its summed CUDA-event time.
cpu_baseline: the oracle's Boykov-Kolmogorov solver (oracle/, the CPU
        checker) on a bounded sample of the same workload, host cores.
--impl reference: the reference has no CPU implementation of this path and
        its CUDA path cannot be built on the GPU host, so this arm times the
        CPU port (oracle BK) with all host threads, one image per thread.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "gc-fg_gb300"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

METRIC = "exact-min-cut Mpixel/s"
UNIT = "Mpixel/s"

# Algorithmic bytes per pixel of each kernel kind (int32 layout):
#   push    : read 4 caps + excess + height (24 B), write 4 caps + excess (20 B)
#   gr_tile : read 4 caps + height (20 B), write height (4 B)
#   build   : read RGB (3 B), write 4 caps + excess (20 B)
#   reach   : read 4 caps + mark (17 B), write mark (1 B)
BYTES_PER_PX = {"push": 44, "gr_tile": 24, "build": 23, "reach": 18, "count": 8, "gr_init": 8,
                "extract": 7, "hist": 4, "sigma": 6, "reach_init": 5}

WORKLOADS = {
    # The plain single-image 1920x1080 configuration: lambda in {10, 50, 200},
    # seeds 1..3 (one image per lambda).
    "plain1080": dict(desc="plain per-image, 1920x1080, lambda {10,50,200}, seeds 1-3",
                      images=[(1, 1920, 1080, 1, 10.0), (1, 1920, 1080, 2, 50.0),
                              (1, 1920, 1080, 3, 200.0)]),
    "plain256": dict(desc="plain per-image, 256x256, lambda 50, seed 0",
                     images=[(0, 256, 256, 0, 50.0)]),
    "plain4096": dict(desc="plain per-image, 4096x4096, 2000 blobs, lambda 100, seed 2",
                      images=[(2, 4096, 4096, 2, 100.0)]),
}


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def make_images(spec):
    import oracle as O
    return [(O.generate(cfg, W, H, seed), lam) for (cfg, W, H, seed, lam) in spec["images"]]


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kind: str, workload: str):
    """DRAM bytes per launch from a committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", f"{kind}_{workload}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def cpu_baseline(images, budget_s=10.0, threads=1):
    """Oracle BK on a bounded sample of the workload (host cores)."""
    import oracle as O
    t0 = time.perf_counter()
    px = 0
    flows = []
    k = 0
    while True:
        (rgb, scrib), lam = images[k % len(images)]
        r = O.segment(rgb, scrib, lam, solver="bk")
        flows.append((k % len(images), r["flow"]))
        px += scrib.size
        k += 1
        if time.perf_counter() - t0 > budget_s or k >= 64:
            break
    dt = time.perf_counter() - t0
    return px / dt / 1e6, k, dt, flows


def run_reference_arm(args, spec, rank, world):
    """--impl reference: CPU port of the path on all host threads."""
    if rank != 0:
        return 0
    import oracle as O
    images = make_images(spec)
    nthreads = os.cpu_count() or 1
    lams = [lam for _, lam in images]
    imgs = [im for im, _ in images]
    per_step = []
    total_px = sum(s.size for _, s in imgs)
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        # one image per thread; the step's images are replicated so that every
        # host thread has work (bounded sample of the same workload)
        reps = max(1, nthreads // len(imgs))
        flows, _, _, _ = O.segment_batch(imgs * reps, lams * reps, nthreads)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            per_step.append((dt, total_px * reps))
    secs = sum(d for d, _ in per_step)
    px = sum(p for _, p in per_step)
    value = px / secs / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / len(per_step) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded in-repo generator)",
            "config": {"workload": args.workload, "desc": spec["desc"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{len(imgs)} image(s) x {max(1, nthreads // len(imgs))} replicas per step, "
                                       "oracle Boykov-Kolmogorov, one image per host thread; the reference "
                                       "has no CPU solver and its CUDA path is not buildable on the GPU host"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain1080", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_info()
    spec = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference_arm(args, spec, rank, world)

    import torch
    import __graft_entry__ as ge
    ge.build()
    import gcfg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    images = make_images(spec)
    maxW = max(s.shape[1] for (_, s), _ in images)
    maxH = max(s.shape[0] for (_, s), _ in images)
    seg = gcfg.Segmenter(maxW, maxH)
    stream = torch.cuda.current_stream()
    seg.set_stream(stream)
    dev = []
    for (rgb, scrib), lam in images:
        H, W = scrib.shape
        dev.append(dict(rgb=torch.from_numpy(rgb).cuda(), scrib=torch.from_numpy(scrib).cuda(),
                        smin=torch.empty((H, W), dtype=torch.uint8, device="cuda"),
                        smax=torch.empty((H, W), dtype=torch.uint8, device="cuda"),
                        W=W, H=H, lam=lam,
                        h_rgb=torch.from_numpy(rgb).pin_memory(), h_scrib=torch.from_numpy(scrib).pin_memory(),
                        h_smin=torch.empty((H, W), dtype=torch.uint8).pin_memory(),
                        h_smax=torch.empty((H, W), dtype=torch.uint8).pin_memory()))
    px_per_step = sum(d["W"] * d["H"] for d in dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def step_device():
        res = []
        for d in dev:
            res.append(seg.run(d["rgb"], d["scrib"], d["W"], d["H"], d["lam"], d["smin"], d["smax"]))
        return res

    def step_host():
        res = []
        for d in dev:
            res.append(seg.run_host(d["h_rgb"].numpy(), d["h_scrib"].numpy(), d["W"], d["H"], d["lam"],
                                    d["h_smin"].numpy(), d["h_smax"].numpy()))
        return res

    for _ in range(args.warmup):
        step_device()
        step_host()

    # ---- timed region: device-resident inputs ----
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    l0 = gcfg.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    results = []
    for i in range(args.steps):
        flush.fill_(i & 0xFF)  # L2 flush (256 MB > 129 MB L2), outside the step's events
        ev[i][0].record(stream)
        results.append(step_device())
        ev[i][1].record(stream)
    barrier()
    launches = gcfg.launch_count() - l0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)

    # ---- e2e through the host entry point ----
    barrier()
    e2e_ms = []
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        torch.cuda.synchronize()
        t = time.perf_counter()
        step_host()
        e2e_ms.append((time.perf_counter() - t) * 1e3)
    barrier()
    e2e_total = sum(e2e_ms)

    def max_over_ranks(v):
        if dist is None:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    total_ms = max_over_ranks(total_ms)
    e2e_total = max_over_ranks(e2e_total)
    value = world * px_per_step * args.steps / (total_ms / 1e3) / 1e6
    e2e_value = world * px_per_step * args.steps / (e2e_total / 1e3) / 1e6

    # ---- roofline: one profiled step ----
    gcfg.profile_enable(True)
    gcfg.profile_read()
    flush.fill_(7)
    prof_res = step_device()
    prof = gcfg.profile_read()
    gcfg.profile_enable(False)
    dom = max(prof, key=lambda k: prof[k]["ms"])
    peak, peak_kind = load_peaks()
    if dom == "push":
        units_px = sum(r["push_tiles"] for r in prof_res) * 1024
    elif dom == "gr_tile":
        units_px = sum(r["gr_tiles"] for r in prof_res) * 1024
    elif dom in ("build", "extract", "hist", "sigma"):
        units_px = px_per_step
    else:
        units_px = sum(((d["W"] + 31) // 32) * ((d["H"] + 31) // 32) * 1024 for d in dev)
    launches_dom = max(prof[dom]["launches"], 1)
    alg_bytes = BYTES_PER_PX.get(dom, 24) * units_px
    achieved = alg_bytes / (prof[dom]["ms"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "traffic": ncu_traffic(dom, args.workload),
                "alg_bytes_per_launch": alg_bytes / launches_dom,
                "avg_launch_us": prof[dom]["ms"] / launches_dom * 1e3,
                "share_of_step": prof[dom]["ms"] / sum(v["ms"] for v in prof.values()),
                "kernels_ms": {k: round(v["ms"], 4) for k, v in prof.items() if v["launches"]}}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded in-repo generator; no dataset)",
            "config": {"workload": args.workload, "desc": spec["desc"], "images_per_step": len(dev),
                       "pixels_per_step": px_per_step, "l2": "flushed (256 MB write) before every step",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 4 * px_per_step,
                    "d2h_bytes_per_step": 2 * px_per_step, "ms_per_step": e2e_total / args.steps},
            "roofline": roofline, "clocks": clk, "gpu_launches": launches,
            "solver": {k: results[-1][0][k] for k in ("global_relabels", "gr_sweeps", "push_rounds",
                                                       "cut_sweeps")}}
    if rank == 0:
        cpu_v, n_img, secs, flows = cpu_baseline(images, budget_s=args.cpu_budget)
        ok = all(results[-1][i]["flow"] == f for i, f in flows)
        line["cpu_baseline"] = {"value": cpu_v, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"{n_img} image(s) of the workload in {secs:.1f} s, oracle "
                                          "Boykov-Kolmogorov, 1 thread"}
        line["parity"] = {"flows_equal_oracle": ok, "images_checked": len(set(i for i, _ in flows))}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
