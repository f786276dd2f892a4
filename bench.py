"""Throughput of the cone-beam Siddon projection + voxel-driven backprojection pair.

Workload (one step): forward projection A x and backprojection A^T y of the
512^3 volume over 200x200x150 mm, 360 views over 360 deg, 768x512 detector
(0.8 mm at SDD 1200, SID 600 -> 0.4 mm at the centre), float32, synthetic
random-ellipsoid phantom (seed 2).  Metric: GRay/s = rays / (t_FP + t_BP),
rays = 360 * 768 * 512.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs under torchrun, one rank per GPU: the scan's views are split over
the ranks, each rank projects its views and backprojects them into a partial
volume, and one NCCL all-reduce sums the volumes (strong scaling of one scan;
ctgb.shard).  --replicas runs the whole scan on every rank instead (weak).
The reference arm times the reference algorithm's CPU restatement (the FP64
oracle, OpenMP over all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "ct-research_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "Gray/s proj+backproj (%HBM roofline); SIRT-TV time-to-residual learned vs plain"
UNIT = "GRay/s"
WORKLOAD = "cone_512: 512^3 float32 volume (200x200x150 mm), 360 views / 360 deg, 768x512 detector, " \
           "SID 600 / SDD 1200; one step = Siddon FP + voxel-driven BP"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic():
    """DRAM bytes per launch of the bench's kernels from the committed ncu summary
    (profiles/traffic.json): kernel -> {"bytes_per_launch", "source"}."""
    p = ROOT / "profiles" / "traffic.json"
    try:
        d = json.loads(p.read_text())
    except Exception:
        return {}
    return {k: v for k, v in d.items() if isinstance(v, dict)}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def cpu_sample(geom, vol_np, seconds_target=12.0, max_views=32):
    """Time the oracle's FP + BP on a subset of views (all host threads)."""
    from oracle.oracle import Oracle
    o = Oracle(nthreads=os.cpu_count() or 1)
    g1 = geom.subset_views([7])
    t0 = time.perf_counter()
    p = o.cone_fp(vol_np, g1.beta, g1.P, g1.xi, g1.size, g1.D)
    o.cone_bp(p, g1.beta, g1.P, g1.xi, g1.size, g1.D, g1.vol_shape)
    t1 = time.perf_counter() - t0
    nv = int(max(1, min(max_views, seconds_target / max(t1, 1e-3))))
    idx = np.linspace(0, len(geom.beta) - 1, nv).astype(int)
    gs = geom.subset_views(idx)
    t0 = time.perf_counter()
    p = o.cone_fp(vol_np, gs.beta, gs.P, gs.xi, gs.size, gs.D)
    o.cone_bp(p, gs.beta, gs.P, gs.xi, gs.size, gs.D, gs.vol_shape)
    dt = time.perf_counter() - t0
    rays = gs.n_rays
    return {"value": rays / dt / 1e9, "unit": UNIT, "cores": o.nthreads, "kind": "port",
            "sample": f"FP64 oracle FP+BP of {nv} of the 360 views (all 768x512 rays of each view, full "
                      f"512^3 volume), {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return
    import torch  # noqa: F401  (phantom generation)
    from ctgb import geometry, phantom
    geom = geometry.config_cone_512()
    vol = phantom.ellipsoids_3d(geom.nt, geom.ns, geom.nz, phantom.ellipsoid_params(12, seed=2)).numpy()
    from oracle.oracle import Oracle
    o = Oracle(nthreads=os.cpu_count() or 1)
    # one step = FP + BP of a fixed subset of views (bounded sample of the workload)
    nv = 2
    idx = np.linspace(0, len(geom.beta) - 1, nv).astype(int)
    gs = geom.subset_views(idx)

    def step():
        p = o.cone_fp(vol, gs.beta, gs.P, gs.xi, gs.size, gs.D)
        o.cone_bp(p, gs.beta, gs.P, gs.xi, gs.size, gs.D, gs.vol_shape)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    v = gs.n_rays / dt / 1e9
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": f"{nv} of 360 views per step"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": o.nthreads, "kind": "port",
                             "sample": f"FP64 oracle (reference algorithm restated in C, OpenMP) FP+BP of {nv} "
                                       f"of the 360 views per step; the reference's own code is MATLAB + CUDA "
                                       f"MEX and cannot run on this host"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            # the metric's second half compares a learned start with plain SIRT-TV on the same GPU;
            # the reference has no learned start, and its SIRT-TV is a MATLAB loop
            "sirt_tv_learned_vs_plain": {"unavailable": "the reference has no learned warm start; its SIRT-TV "
                                                        "is a MATLAB script over the MEX operators"}}
    print(json.dumps(line), flush=True)


def pair_parity(plan, geom, vol, proj, views=(44, 200)):
    """rel-L2 of the timed FP and BP against the FP64 oracle on two views of the
    workload, computed after the timed region: the FP on the phantom, the BP on
    the FP's own output of those views (the oracle BP takes the same input)."""
    import torch
    from oracle.oracle import Oracle
    o = Oracle(nthreads=os.cpu_count() or 1)
    idx = [v for v in views if v < len(geom.beta)] or [0]
    gs = geom.subset_views(idx)
    fp = proj[idx].cpu().numpy()
    t0 = time.perf_counter()
    ref_fp = o.cone_fp(vol.cpu().numpy(), gs.beta, gs.P, gs.xi, gs.size, gs.D)
    from ctgb.device import ConePlan
    bp = ConePlan(gs).bp(proj[idx].contiguous()).cpu().numpy()
    ref_bp = o.cone_bp(fp, gs.beta, gs.P, gs.xi, gs.size, gs.D, gs.vol_shape)
    torch.cuda.synchronize()

    def rel(a, b):
        return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))

    return {"fp_rel_l2_vs_oracle": rel(fp, ref_fp), "bp_rel_l2_vs_oracle": rel(bp, ref_bp),
            "views": idx, "tolerance": 1e-5, "oracle": "FP64 C restatement of the reference kernels",
            "seconds": time.perf_counter() - t0}


def small_geometry():
    """Profiling case of the same kernels: 256^3, 90 views, 384x256 detector
    (volume 64 MiB, sinogram 35 MB: inputs above L2 together, one launch ~ms)."""
    from ctgb import geometry
    g = geometry.config_cone_512()
    return geometry.cone_from_physical((256, 256, 256), (200.0, 200.0, 150.0), 90, 384, 256, 1.6, 600.0, 1200.0,
                                       name="cone_256_profile")


def run_ours(args):
    import torch
    rank, world, local = _dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    import ctgb
    from ctgb import geometry, phantom, _lib
    from ctgb.device import ConePlan
    ctgb.load()
    geom = geometry.config_cone_512() if args.size == "full" else small_geometry()
    if args.views:
        # profiling case: every k-th view of the scan (same volume, detector and per-view footprint),
        # or its first N views (--contiguous)
        idx = np.arange(args.views) if args.contiguous else \
            np.linspace(0, len(geom.beta) - 1, args.views).round().astype(int)
        geom = geom.subset_views(idx)
    vol = phantom.ellipsoids_3d(geom.nt, geom.ns, geom.nz, phantom.ellipsoid_params(12, seed=2), device=dev)
    scan = geom
    sharded = world > 1 and not args.replicas
    if sharded:
        # one scan split by views over the ranks: FP of this rank's views, BP into a
        # partial volume, one NCCL all-reduce of the volume (ctgb.shard)
        from ctgb.shard import local_geometry
        geom = local_geometry(scan, rank, world)
    plan = ConePlan(geom)
    if args.bp_chunk:
        plan.set_bp_chunk(args.bp_chunk)
    proj = plan.new_sino(dev)
    back = plan.new_volume(dev)
    stream = torch.cuda.current_stream()
    from ctgb.shard import ShardedPair

    class _Timed:
        """The plan's fp / bp with CUDA events on the launching stream around them."""
        ev = None

        def fp(self, v, out):
            if self.ev:
                self.ev[0].record(stream)
            plan.fp(v, out)
            if self.ev:
                self.ev[1].record(stream)
            return out

        def bp(self, y, out):
            plan.bp(y, out)
            if self.ev:
                self.ev[2].record(stream)
            return out

    timed = _Timed()
    pair = ShardedPair(timed)

    def step(ev=None):
        timed.ev = ev
        pair.step(vol, proj, back)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index or 0) as clk:
        start.record(stream)
        for k in range(args.steps):
            step(evs[k])
        stop.record(stream)
        torch.cuda.synchronize()
    t_total = start.elapsed_time(stop) / 1e3
    t_fp = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps / 1e3
    t_bp = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps / 1e3
    if dist:
        t = torch.tensor([t_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_total = float(t.item())
    t_step = t_total / args.steps
    job_rays = scan.n_rays if sharded else world * scan.n_rays
    value = job_rays / t_step / 1e9

    # e2e through the C ABI with host (pinned) buffers: copies inside the timed region
    import ctypes as C
    h_vol = torch.empty(geom.vol_shape, dtype=torch.float32, pin_memory=True)
    h_vol.copy_(vol.cpu())
    h_proj = torch.empty(geom.sino_shape, dtype=torch.float32, pin_memory=True)
    h_back = torch.empty(geom.vol_shape, dtype=torch.float32, pin_memory=True)
    lib = _lib.lib()
    res = np.array([geom.size[0] / geom.nt, geom.size[1] / geom.ns, geom.size[2] / geom.nz])
    size = np.array(geom.size)
    vp = lambda a: C.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else C.c_void_p(a.data_ptr())

    d_red = torch.empty(geom.vol_shape, dtype=torch.float32, device=dev) if sharded else None

    call_ms = {"fp": [], "bp": []}

    def e2e_step():
        t0 = time.perf_counter()
        _lib.check(lib.ct_ProjectionCone_3D(vp(h_vol), vp(h_proj), vp(geom.beta), vp(geom.P), vp(geom.xi),
                                            geom.nt, geom.ns, geom.nz, size[0] / 2, size[1] / 2, size[2] / 2,
                                            len(geom.beta), len(geom.P), len(geom.xi), geom.D, vp(res)),
                   "ct_ProjectionCone_3D")
        t1 = time.perf_counter()
        _lib.check(lib.ct_BackPro(vp(h_back), vp(h_proj), vp(geom.xi), vp(geom.P), vp(geom.beta), geom.D,
                                  len(geom.beta), len(geom.P), len(geom.xi), vp(size), geom.nt, geom.ns, geom.nz),
                   "ct_BackPro")
        call_ms["fp"].append((t1 - t0) * 1e3)
        call_ms["bp"].append((time.perf_counter() - t1) * 1e3)
        if sharded:
            # the partial volumes of the ranks' views summed into every rank's host volume
            d_red.copy_(h_back, non_blocking=True)
            dist.all_reduce(d_red)
            h_back.copy_(d_red)

    if args.no_e2e:
        t_e2e = float("nan")
    else:
        e2e_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        t_e2e = (time.perf_counter() - t0) / args.steps
    if dist:
        t = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = {"value": job_rays / t_e2e / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": int(h_vol.numel() * 4 + h_proj.numel() * 4 + (h_back.numel() * 4 if sharded else 0)),
           "d2h_bytes_per_step": int(h_proj.numel() * 4 + h_back.numel() * 4 * (2 if sharded else 1)),
           "ms_per_step": t_e2e * 1e3,
           "ms_per_call_median": {k: float(np.median(v[1:])) if len(v) > 1 else None for k, v in call_ms.items()},
           "ms_per_call": {k: [round(x, 2) for x in v[1:]] for k, v in call_ms.items()}}

    if rank != 0:
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    segs = plan.count_segments()
    R, V, B = geom.n_rays, geom.n_voxels, len(geom.beta)
    fp_bytes = 4 * segs + 4 * R
    bp_bytes = 16 * V * B + 8 * V
    peak, peak_kind = _peaks()
    traffic = _traffic()
    kern = {
        "cone_fp_kernel": {"ms": t_fp * 1e3, "algorithmic_bytes": fp_bytes,
                           "achieved_gbs": fp_bytes / t_fp / 1e9, "segments": segs},
        "cone_bp_kernel+pack_quads": {"ms": t_bp * 1e3, "algorithmic_bytes": bp_bytes,
                                      "achieved_gbs": bp_bytes / t_bp / 1e9},
    }
    dom = "cone_fp_kernel" if t_fp >= t_bp else "cone_bp_kernel+pack_quads"
    ach = kern[dom]["achieved_gbs"]
    full_case = args.size == "full" and not args.views
    tr = traffic.get(dom.split("+")[0]) if full_case else None
    roofline = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": tr.get("bytes_per_launch") if isinstance(tr, dict) else tr,
                "traffic_source": ("stored ncu capture of this kernel on this workload, not measured by this run: "
                                   + tr.get("source", "profiles/traffic.json")) if isinstance(tr, dict) else None,
                "kernel": dom, "peak_source": peak_kind,
                "pair_frac": (fp_bytes + bp_bytes) / (t_fp + t_bp) / 1e9 / peak}
    parity = None if args.no_parity else pair_parity(plan, geom, vol, proj)
    cpu = cpu_sample(geom, vol.cpu().numpy()) if (world == 1 and not args.no_cpu) else None
    warm = None
    if world == 1 and full_case and not args.no_warmstart:
        # the metric's second half, measured after the timed region (1 GPU only)
        torch.cuda.empty_cache()
        w = measure_warmstart(500)
        best = w["arms"].get(w["best_arm"] or "", {})
        warm = {"plain_seconds": w["plain_seconds"], "learned_seconds": w["value"], "speedup": w["speedup"],
                "unit": "s", "target_relative_residual": w["target_relative_residual"],
                "plain_iterations": w["plain_iterations"], "learned_iterations": best.get("iterations"),
                "learned_rel_l2_vs_reference": best.get("rel_l2_vs_reference"), "best_arm": w["best_arm"],
                "network_ms": best.get("network_ms_device"), "plain_reaches_1e-3": w["plain_reaches_1e-3"],
                "network_roofline": w["roofline"],
                "workload": "512^3, 90 views, noise-free seed-7 phantom; target = the 500-iteration plain "
                            "SIRT-TV residual; times from the FDK volume, network included"}
    if not full_case:
        line_workload = f"{geom.name}, {len(geom.beta)} views: profiling case (not the benchmark workload)"
    else:
        line_workload = WORKLOAD
    clocks = clk.summary()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "strong" if sharded else "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": line_workload,
                       "parallelism": (f"views split over {world} ranks, NCCL all-reduce of the volume" if sharded
                                       else f"replicas x{world}"),
                       "l2": "inputs larger than L2 (512 MiB volume, 566 MB sinogram, 2.3 GB packed quads)",
                       "phantom": "12 random ellipsoids, seed 2"},
            "roofline": roofline, "kernels": kern, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "parity": parity,
            # per step: transpose_ts, cone_fp, cone_fixup, then pack_quads + cone_bp per view chunk
            "gpu_launches": plan.launches_per_pair() * args.steps, "sirt_tv_learned_vs_plain": warm}
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_batched2d(args):
    """64 uneven 2D fan slices (N 128..512, views 90..720, bins 256..1024, seed 4),
    100 SIRT iterations per slice as one CUDA-graph launch with autotuned blocks."""
    import torch
    import ctgb
    from ctgb import geometry, phantom
    from ctgb.batch import FanBatch, BatchedSirt, autotune
    ctgb.load()
    geoms = geometry.config_batched_fan(64, seed=4)
    batch = FanBatch(geoms)
    imgs = [phantom.ellipses_2d(g.nt, g.ns, phantom.ellipse_params(10, seed=100 + k), device="cuda")
            for k, g in enumerate(geoms)]
    b = batch.fp(batch.pack_images(imgs))
    tune = autotune(batch, b)
    sirt = BatchedSirt(batch, b)
    iters = 100
    x = batch.fbp(b).clamp_(0.0, 1.0)
    g, norms = sirt.capture(x, iters)
    x0 = x.clone()
    times = []
    for _ in range(args.warmup + args.steps):
        x.copy_(x0)
        norms.zero_()
        e0, e1 = _events()
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = min(times[args.warmup:])
    hist = BatchedSirt.history(norms)
    rays = batch.n_rays
    # What a persistent kernel could save: the graph's time per iteration against the
    # two operators of an iteration timed one at a time (each alone on an idle GPU).
    xs = x0.clone()
    nrm = torch.zeros(len(geoms), 2, dtype=torch.float64, device="cuda")
    part = {"fp_residual": [], "bp_update": []}
    for _ in range(5):
        for name, fn in (("fp_residual", lambda: batch.fp_residual(xs, sirt.b, sirt.rowsum, sirt.eps, sirt.e, nrm)),
                         ("bp_update", lambda: batch.bp_update(sirt.e, sirt.colsum, xs, sirt.lam, sirt.eps, sirt.lo,
                                                                sirt.hi))):
            torch.cuda.synchronize()
            e0, e1 = _events()
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            part[name].append(e0.elapsed_time(e1))
    alone = {k: float(np.median(v)) for k, v in part.items()}
    per_it = t * 1e3 / iters
    line = {"metric": "batched 2D fan SIRT: GRay/s of FP+BP iterations", "value": rays * iters / t / 1e9,
            "unit": "GRay/s", "ms_per_launch": t * 1e3, "iterations": iters, "slices": len(geoms),
            "rays_per_iteration": rays, "pixels": batch.n_img, "blocks": tune["blocks"],
            "grazing_rays_per_projection": batch.grazing_rays(),
            "graph_vs_kernels": {"ms_per_iteration_in_graph": per_it, "ms_operators_alone": alone,
                                 "gap_fraction": (per_it - sum(alone.values())) / per_it},
            "residual_first_last_median": [float(np.median(hist[0])), float(np.median(hist[-1]))],
            "config": {"workload": "64 slices N~U{128..512}, views~U{90..720}, bins~U{256..1024}, seed 4; "
                                   "FBPfan start, lam 2, x in [0,1]; one graph launch = 100 iterations"}}
    print(json.dumps(line), flush=True)


def run_sirt_tv(args):
    """SIRT3D + TV on the 512^3 / 360-view / 768x512 workload: Poisson noise at 1e5
    photons/ray (seed 3), FDK start, lam 1, x >= 0, 20 TV sub-steps of 1e-3 per
    iteration; time per iteration and the data residual."""
    import torch
    import ctgb
    from ctgb import geometry, phantom
    from ctgb.device import ConePlan, FDK_FILTER_CLEAN, FDK_BP_ZERO
    from ctgb.sirt import Sirt, SirtConfig
    ctgb.load()
    geom = geometry.config_cone_512()
    vol = phantom.ellipsoids_3d(geom.nt, geom.ns, geom.nz, phantom.ellipsoid_params(12, seed=2), device="cuda")
    plan = ConePlan(geom, fdk_filter=FDK_FILTER_CLEAN, fdk_bp=FDK_BP_ZERO)
    clean = plan.fp(vol)
    b, _ = phantom.poisson_noise(clean, 1e5, 4.0, seed=3)
    x0 = plan.fdk(b).clamp_(min=0.0)
    iters = args.iters
    cfg = SirtConfig(iters=iters, lam=1.0, eps=1e-9, tv_iters=20, tv_step=1e-3, use_graph=True, min_rowsum=0.5 * min(geom.size[a] / n for a, n in enumerate((geom.nt, geom.ns, geom.nz))), min_colsum_frac=0.05,
                     check_every=max(1, iters // 10))
    s = Sirt(plan, b, cfg)
    res = s.run(x0.clone())
    r_final = s.data_residual(res.x)
    rel_err = float(torch.linalg.vector_norm(res.x - vol) / torch.linalg.vector_norm(vol))
    line = {"metric": "SIRT3D-TV 512^3 s/iteration", "value": res.seconds / res.iterations, "unit": "s",
            "iterations": res.iterations, "seconds": res.seconds, "final_relative_residual": r_final,
            "residual_history": res.residuals, "rel_l2_vs_phantom": rel_err,
            "fdk_rel_l2_vs_phantom": float(torch.linalg.vector_norm(x0 - vol) / torch.linalg.vector_norm(vol)),
            "config": {"workload": "cone_512, Poisson 1e5, FDK start, 20 TV sub-steps/iter, graph replay"}}
    print(json.dumps(line), flush=True)


def run_warmstart(args):
    seeds = [int(v) for v in args.seeds.split(",")]
    if len(seeds) == 1:
        print(json.dumps(measure_warmstart(args.ref_iters, seeds[0], args.weights, args.target, args.max_iters)),
              flush=True)
        return
    runs = [measure_warmstart(args.ref_iters, sd, args.weights, args.target, args.max_iters) for sd in seeds]
    sp = [r["speedup"] for r in runs if r["speedup"] is not None]
    line = {"metric": "SIRT-TV wall time to the 500-iteration data residual, learned start", "unit": "s",
            "value": float(np.mean([r["value"] for r in runs if r["value"] is not None])), "higher_is_better": False,
            "seeds": seeds, "speedup_mean": float(np.mean(sp)) if sp else None,
            "speedup_min": float(np.min(sp)) if sp else None,
            "per_seed": [{"seed": sd, "plain_seconds": r["plain_seconds"], "learned_seconds": r["value"],
                          "speedup": r["speedup"], "target_relative_residual": r["target_relative_residual"],
                          "best_arm": r["best_arm"],
                          "learned_iterations": r["arms"][r["best_arm"]]["iterations"] if r["best_arm"] else None,
                          "rel_l2_vs_reference": r["arms"][r["best_arm"]]["rel_l2_vs_reference"]
                          if r["best_arm"] else None,
                          "arms": r["arms"]} for sd, r in zip(seeds, runs)],
            "config": runs[0]["config"]}
    print(json.dumps(line), flush=True)


def measure_warmstart(ref_iters: int = 500, seed: int = 7, weights: str | None = None, target: float | None = None,
                      max_iters: int = 4000) -> dict:
    """Learned warm start vs plain SIRT-TV on the sparse-view 512^3 scan (90 views
    over 360 deg, the cone_512 detector and distances), noise-free data of a
    12-ellipsoid phantom (seed 7 unless given; training used seeds 1000-2999).
    Reference: --ref-iters iterations of SIRT-TV (ASD step, lam 1, 20 TV
    sub-steps) from the FDK start; its final relative data residual is the
    target.  Each learned start (network at 512^3, and at the 128^3 training
    voxel size with the correction upsampled) runs the same loop until it reaches
    that residual.  Times start when the FDK volume exists (both arms pay FDK)
    and include the network's inference.

    With `target` (e.g. 1e-3, the benchmark spec's relative residual), both starts
    instead run until that residual or max_iters iterations; plain SIRT-TV from
    FDK is timed to it in its own run, and rel-L2 is still taken against the
    ref_iters-iteration reference (and against the plain run at the target)."""
    import torch
    import ctgb
    from ctgb import unet, warmstart as ws
    from ctgb.device import ConePlan
    from ctgb.sirt import AsdConfig, AsdLoop
    ctgb.load()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    n, views, iters = 512, 90, ref_iters
    plan = ConePlan(ws.scan(n, views))
    vol = ws.phantom_volume(n, seed)
    b = plan.fp(vol)
    fdk = plan.fdk(b)
    wpath = Path(weights).resolve() if weights else ws.WEIGHTS
    net = ws.load(wpath)
    loop = AsdLoop(plan, AsdConfig(iters=iters))
    ref = loop.run(b, fdk, check_every=1)
    if target is None:
        tol, run_iters, plain_run = ref.residuals[-1][1], iters, ref
    else:
        tol, run_iters = float(target), int(max_iters)
        plain_run = loop.run(b, fdk, iters=run_iters, tol=tol, check_every=1)
    plain = ws.time_to_residual(plain_run, tol)
    plain_1e3 = ws.time_to_residual(plain_run, 1e-3)

    def err(a, c):
        return float(torch.linalg.vector_norm(a - c) / torch.linalg.vector_norm(c))

    arms = {}
    for mode, train_n in (("net_512", None), ("net_128_upsampled", 128)):
        ws.warm_start(net, fdk, train_n)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        x0 = ws.warm_start(net, fdk, train_n)
        e1.record()
        torch.cuda.synchronize()
        t_net = time.perf_counter() - t0
        run = loop.run(b, x0, iters=run_iters, tol=tol, check_every=1)
        hit = ws.time_to_residual(run, tol)
        arms[mode] = {"network_seconds": t_net, "network_ms_device": e0.elapsed_time(e1),
                      "start_rel_l2_vs_reference": err(x0, ref.x),
                      "start_residual": run.residuals[0][1],
                      "iterations": None if hit is None else hit[0],
                      "seconds": None if hit is None else t_net + hit[1],
                      "final_residual": run.residuals[-1][1],
                      "rel_l2_vs_reference": err(run.x, ref.x),
                      "rel_l2_vs_plain_at_target": err(run.x, plain_run.x)}
    ok = {k: v for k, v in arms.items() if v["seconds"] is not None}
    best = min(ok, key=lambda k: ok[k]["seconds"]) if ok else None
    flops = unet.flops_per_voxel() * n ** 3
    t_full = arms["net_512"]["network_ms_device"] / 1e3
    curve = {int(k): float(r) for k, r in plain_run.residuals if k in (1, 50, 100, 200, 300, 500, 1000, 1500, 2000,
                                                                        2500, 3000, 3500, 4000, 5000, 6000)}
    curve[int(plain_run.residuals[-1][0])] = float(plain_run.residuals[-1][1])
    line = {"metric": ("SIRT-TV wall time to the 500-iteration data residual, learned start" if target is None
                       else f"SIRT-TV wall time to relative data residual {target:g}, learned start"),
            "unit": "s",
            "value": None if best is None else arms[best]["seconds"], "higher_is_better": False,
            "best_arm": best, "plain_seconds": None if plain is None else plain[1],
            "plain_iterations": None if plain is None else plain[0],
            "speedup": None if (best is None or plain is None) else plain[1] / arms[best]["seconds"],
            "target_relative_residual": tol, "arms": arms,
            "plain_reaches_1e-3": None if plain_1e3 is None else {"iterations": plain_1e3[0], "seconds": plain_1e3[1]},
            "plain_residual_curve": curve, "plain_iterations_run": int(plain_run.iterations),
            "fdk_rel_l2_vs_reference": err(fdk, ref.x), "reference_rel_l2_vs_phantom": err(ref.x, vol),
            "seconds_per_iteration": ref.seconds / ref.iterations,
            "roofline": {"bound": "tensor", "kernel": "U-Net forward at 512^3 (all convolutions + pooling)",
                         "achieved": flops / t_full / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": flops / t_full / 1e12 / bf16_peak, "peak_source": "measured bf16 burst"},
            "dtype": "bf16 network / f32 SIRT-TV", "data": "synthetic (seeded ellipsoid phantoms, noise-free)",
            "config": {"workload": "cone_512 geometry with 90 views; U-Net trained on 128^3 pairs of the same scan "
                                   "(90-view FDK -> 500-iteration SIRT-TV)",
                       "weights": str(wpath.relative_to(ROOT)) if wpath.is_relative_to(ROOT) else str(wpath)}}
    return line


def run_unet(args):
    """The warm-start U-Net's tensor-core convolutions: each layer shape of the
    network at 512^3 (forward), the whole forward pass at 512^3, and one training
    step (forward + backward + Adam) at 128^3; CUDA events after a warm-up call."""
    import torch
    import ctgb
    from ctgb import unet
    ctgb.load()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    n = 512 if args.size == "full" else 128      # small: the same kernels on 128^3 (profiling case)
    layers = []
    g = torch.Generator(device="cuda").manual_seed(0)
    for cin, cout, lvl in [(32, 32, 1), (64, 32, 1), (32, 64, 2), (64, 64, 2), (128, 64, 2), (64, 128, 4),
                           (128, 128, 4), (256, 128, 4), (128, 256, 8), (256, 256, 8)]:
        m = n // lvl
        x = torch.randn((1, m, m, m, cin), device="cuda", generator=g).to(torch.bfloat16)
        w = (0.05 * torch.randn((cout, 27, cin), device="cuda", generator=g)).to(torch.bfloat16)
        ms = timed(lambda: unet.conv3d(x, w, relu=True), max(2, args.steps))
        fl = 2.0 * m ** 3 * cin * cout * 27
        layers.append({"in": cin, "out": cout, "size": m, "ms": ms, "tflops": fl / ms / 1e9})
        del x, w
    torch.cuda.empty_cache()
    net = unet.UNet3D(seed=0)
    x = torch.rand((1, n, n, n), device="cuda", generator=g)
    fwd_ms = timed(lambda: net.forward(x), 2)
    del x
    torch.cuda.empty_cache()
    xs = torch.rand((1, 128, 128, 128), device="cuda", generator=g)

    def train_step():
        out = net.forward(xs, keep=True)
        net.adam_step(net.backward(2.0 * (out - xs) / out.numel()), lr=1e-6)

    step_ms = timed(train_step, max(3, args.steps))
    status = unet.status()
    best = max(layers, key=lambda r: r["tflops"])
    fl_net = unet.flops_per_voxel() * n ** 3
    line = {"metric": f"U-Net forward at {n}^3", "value": fwd_ms, "unit": "ms", "higher_is_better": False,
            "network_tflops": fl_net / fwd_ms / 1e9, "train_step_128_ms": step_ms, "layers": layers,
            "roofline": {"bound": "tensor", "kernel": f"conv_fwd_kernel<{best['out']}> {best['in']}->{best['out']} "
                                                      f"at {best['size']}^3",
                         "achieved": best["tflops"], "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": best["tflops"] / bf16_peak, "peak_source": "measured bf16 burst"},
            "wait_flags": status, "dtype": "bf16 (FP32 accumulate)", "data": "synthetic",
            "config": {"workload": "warm-start U-Net (4 levels, 32 base channels, 3x3x3), batch 1"}}
    print(json.dumps(line), flush=True)


def run_sirt_step(args):
    """The parts of one SIRT-TV iteration of the warm-start comparison (512^3, 90
    views, ASD step), each timed with CUDA events after 3 warm-up iterations:
    FP + residual, BP + update, and the 20 TV sub-steps."""
    import torch
    import ctgb
    from ctgb import device as dev, warmstart as ws
    from ctgb.device import ConePlan
    from ctgb.sirt import AsdConfig, AsdLoop
    ctgb.load()
    plan = ConePlan(ws.scan(512, 90))
    vol = ws.phantom_volume(512, 7)
    b = plan.fp(vol)
    loop = AsdLoop(plan, AsdConfig(iters=3))
    loop.run(b, plan.fdk(b), iters=3)
    s, x = loop.s, loop.x
    parts = {"fp_residual": [], "bp_update": [], "tv_20_substeps": []}
    for _ in range(max(1, args.steps)):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        loop.prev.copy_(x)
        s.norms.zero_()
        ev[0].record()
        plan.fp_residual(x, loop.b, s.rowsum, 1e-9, out=s.e, norms=s.norms)
        ev[1].record()
        plan.bp_update(s.e, s.colsum, x, lam=1.0, eps=1e-9, lo=0.0, hi=float("inf"))
        ev[2].record()
        dev.tv_flow_asd(x, loop.prev, loop.work, loop.scratch, loop.state, 20, 1e-8, 0.0, 0.95, 0.95)
        ev[3].record()
        torch.cuda.synchronize()
        for k, (a, c) in zip(parts, ((0, 1), (1, 2), (2, 3))):
            parts[k].append(ev[a].elapsed_time(ev[c]))
    med = {k: float(np.median(v)) for k, v in parts.items()}
    line = {"metric": "SIRT-TV iteration parts at 512^3 / 90 views", "unit": "ms", "value": sum(med.values()),
            "higher_is_better": False, "parts_ms": med, "steps": args.steps,
            "config": {"workload": "cone_512 geometry with 90 views, ASD-POCS TV step, 20 sub-steps"}}
    print(json.dumps(line), flush=True)


def run_fdk(args):
    """FDK of the 256^3 / 360-view / 512x384 cone scan (reference launch-order
    filter and sticky backprojection)."""
    import torch
    import ctgb
    from ctgb import geometry, phantom
    from ctgb.device import ConePlan
    ctgb.load()
    geom = geometry.config_cone_fdk()
    vol = phantom.ellipsoids_3d(geom.nt, geom.ns, geom.nz, phantom.ellipsoid_params(12, seed=1), device="cuda")
    plan = ConePlan(geom)
    proj = plan.fp(vol)
    out = plan.new_volume()
    filt = torch.empty_like(proj)
    for _ in range(args.warmup):
        plan.fdk(proj, out)
    ts = []
    for _ in range(args.steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        plan.fdk_filter(proj, filt)
        e[1].record()
        plan.fdk_bp(filt, out)
        e[2].record()
        torch.cuda.synchronize()
        ts.append((e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])))
    tf, tb = np.median([a for a, _ in ts]), np.median([b_ for _, b_ in ts])
    V, B = geom.n_voxels, len(geom.beta)
    line = {"metric": "FDK 256^3 ms", "value": float(tf + tb), "unit": "ms", "filter_ms": float(tf),
            "bp_ms": float(tb), "bp_algorithmic_gbs": (16 * V * B + 8 * V) / (tb / 1e3) / 1e9,
            "rel_l2_vs_phantom": float(torch.linalg.vector_norm(out - vol) / torch.linalg.vector_norm(vol)),
            "config": {"workload": "cone_fdk_256: 256^3 over 128 mm, 360 views, 512x384, SID 600 / SDD 1200"}}
    print(json.dumps(line), flush=True)


def run_fan2d(args):
    """2D fan FP + FBPfan: 256^2, 360 views, 512 bins, source-iso 500 mm."""
    import torch
    import ctgb
    from ctgb import geometry, phantom
    from ctgb.device import FanPlan
    ctgb.load()
    geom = geometry.config_fan2d()
    img = phantom.ellipses_2d(geom.nt, geom.ns, phantom.ellipse_params(10, seed=0), device="cuda")
    plan = FanPlan(geom)
    proj = plan.fp(img)
    rec = plan.fbp(proj)
    for _ in range(args.warmup):
        plan.fp(img, proj)
        plan.fbp(proj, rec)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    for _ in range(args.steps):
        plan.fp(img, proj)
    e[1].record()
    for _ in range(args.steps):
        plan.fbp(proj, rec)
    e[2].record()
    torch.cuda.synchronize()
    tfp, tfbp = e[0].elapsed_time(e[1]) / args.steps, e[1].elapsed_time(e[2]) / args.steps
    line = {"metric": "2D fan FP + FBP ms", "value": tfp + tfbp, "unit": "ms", "fp_ms": tfp, "fbp_ms": tfbp,
            "rays": int(np.prod(geom.sino_shape)),
            "config": {"workload": "fan2d_256: 256^2, 360 views, 512 bins, D 500 mm"}}
    print(json.dumps(line), flush=True)


def run_iterfdk(args):
    """IterativeFDK error slice of IterativeFDK.m's set-up: 128^3 over 60 mm,
    PInt 0.4 (234 bins), D 200, 360 views, 221 depth samples, slice t = 64
    (MATLAB index).  Time per slice, and two views checked against the oracle."""
    import torch
    from scipy.ndimage import gaussian_filter
    import ctgb
    from ctgb import phantom
    from ctgb.device import iterfdk_err
    from ctgb.geometry import iterative_fdk_setup
    ctgb.load()
    shape, size, D, t = (128, 128, 128), (60.0, 60.0, 60.0), 200.0, 63
    beta, U, P, G = iterative_fdk_setup(size, shape, pint=0.4, D=D, n_views=360)
    pic = phantom.ellipsoids_3d(128, 128, 128, phantom.ellipsoid_params(12, seed=6)).numpy()
    pic = gaussian_filter(pic, 0.5).astype(np.float32)          # the script's imgaussfilt3(pic, 0.5) prior
    d_pic = torch.from_numpy(pic).cuda()
    out = torch.empty((len(beta), 128, 128), dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        iterfdk_err(d_pic, beta, U, P, G, size, D, t, out)
    ts = []
    for _ in range(args.steps):
        e0, e1 = _events()
        e0.record()
        iterfdk_err(d_pic, beta, U, P, G, size, D, t, out)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    tsec = float(np.median(ts))
    iters = len(beta) * 128 * 128 * len(U) * len(P)
    line = {"metric": "IterativeFDK error slice ms", "value": tsec * 1e3, "unit": "ms",
            "inner_iterations": iters, "giter_per_s": iters / tsec / 1e9,
            "config": {"workload": "IterativeFDK.m set-up: 128^3 / 60 mm, 360 views, LP 234, LU 221, t = 64"}}
    if not args.no_cpu:
        from oracle.oracle import Oracle
        sel = [0, 1, 137]          # the first two keep the scan interval |beta1 - beta0| of the full scan
        ref = Oracle().iterfdk_err(pic, beta[sel], U, P, G, size, D, t)
        got = out[sel].cpu().numpy()
        line["oracle_check"] = {"views": sel, "rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                                "bit_identical_fraction": float(np.mean(got == ref))}
    print(json.dumps(line), flush=True)


def run_fdkui(args):
    """Curved-detector short-scan FDK of the scanner set-up of ImplementUIData.m:
    936 gammas x 80 rows x 800 views (240 deg) into 512 x 512 x 50 (23 mm),
    D 570, SDD 1060.2; smooth synthetic double projections."""
    import torch
    import ctgb
    from ctgb.device import fdkui_bp, fdkui_filter
    from ctgb.geometry import curved_fdk_case
    ctgb.load()
    c = curved_fdk_case("scanner")
    b = torch.tensor(c["beta"], device="cuda").view(-1, 1, 1)
    x = torch.tensor(c["xi"], device="cuda").view(1, -1, 1)
    g = torch.tensor(c["gama"], device="cuda").view(1, 1, -1)
    R = ((1.0 + 0.3 * torch.cos(b + 0.01 * x)) * (1 - (g / g.abs().max()) ** 2).clamp_(min=0)).contiguous()
    rcov = torch.empty(R.shape, dtype=torch.float32, device="cuda")
    disp = torch.empty((c["z_length"], 512, 512), dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        fdkui_filter(R, c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"], c["ds2d"], rcov)
        fdkui_bp(rcov, c["xi"], c["gama"], c["beta"], c["D"], c["ds2d"], c["size"], c["z_length"], disp)
    ts = []
    for _ in range(args.steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        fdkui_filter(R, c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"], c["ds2d"], rcov)
        e[1].record()
        fdkui_bp(rcov, c["xi"], c["gama"], c["beta"], c["D"], c["ds2d"], c["size"], c["z_length"], disp)
        e[2].record()
        torch.cuda.synchronize()
        ts.append((e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])))
    tf, tb = float(np.median([a for a, _ in ts])), float(np.median([q for _, q in ts]))
    line = {"metric": "curved-detector FDK ms", "value": tf + tb, "unit": "ms", "filter_ms": tf, "bp_ms": tb,
            "filter_macs": 800 * 80 * 936 * 936, "bp_voxel_views": 512 * 512 * 50 * 800,
            "config": {"workload": "ImplementUIData.m set-up: 936 x 80 x 800 (240 deg) -> 512 x 512 x 50, "
                                   "D 570, SDD 1060.2"}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer C-ABI timing")
    ap.add_argument("--no-parity", action="store_true", help="skip the rel-L2 check of the default line")
    ap.add_argument("--replicas", action="store_true",
                    help="N > 1: every rank runs the whole scan (weak scaling) instead of splitting its views")
    ap.add_argument("--bp-chunk", type=int, default=0, help="pair: views per backprojection chunk (tuning)")
    ap.add_argument("--contiguous", action="store_true", help="--views: the scan's first N views, not every k-th")
    ap.add_argument("--views", type=int, default=0,
                    help="pair: use this many of the scan's views (profiling cases; not the benchmark line)")
    ap.add_argument("--no-warmstart", action="store_true",
                    help="skip the learned-vs-plain SIRT-TV measurement of the default line")
    ap.add_argument("--size", choices=["full", "small"], default="full",
                    help="small: the profiling case of the same kernels (pair: 256^3 / 90 views / 384x256; "
                         "unet: 128^3 layers and network)")
    ap.add_argument("--workload", choices=["pair", "batched2d", "sirt_tv", "fdk", "fan2d", "iterfdk", "fdkui",
                                           "warmstart", "unet", "sirt_step"], default="pair",
                    help="pair (default): the FP+BP throughput line; the others report their own metric")
    ap.add_argument("--iters", type=int, default=200, help="SIRT-TV iterations (--workload sirt_tv)")
    ap.add_argument("--ref-iters", type=int, default=500, help="reference SIRT-TV iterations (--workload warmstart)")
    ap.add_argument("--seeds", default="7", help="phantom seeds, comma-separated (--workload warmstart)")
    ap.add_argument("--target", type=float, default=None,
                    help="--workload warmstart: run both starts to this relative residual (e.g. 1e-3) instead of the "
                         "reference's own final residual")
    ap.add_argument("--max-iters", type=int, default=4000, help="iteration cap of the --target runs")
    ap.add_argument("--weights", default=None, help="U-Net weights (.npz) for --workload warmstart; default: the "
                                                     "committed ones")
    args = ap.parse_args()
    if args.warmup < 3:
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "pair":
        run_ours(args)
    else:
        {"batched2d": run_batched2d, "sirt_tv": run_sirt_tv, "fdk": run_fdk, "fan2d": run_fan2d,
         "iterfdk": run_iterfdk, "fdkui": run_fdkui, "warmstart": run_warmstart,
         "unet": run_unet, "sirt_step": run_sirt_step}[args.workload](args)


if __name__ == "__main__":
    main()
