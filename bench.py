"""Benchmark: volume-render Gsamples/s on the AMR perspective workload.

Workload (one "step" = one full render of one view): a 128^3 blob root grid
refined by factor 2 to 3 levels in 16^3 patches, decomposed by the kd-tree
into ~1100 bricks, rendered by VolumeRenderSampler through a perspective lens
at 1024x1024 with an 8-layer ColorTransferFunction, 1 sample per cell.
A sample is one trilinear sample + transfer-function evaluation + update
(= one cell visit at n_samples=1), counted exactly by the kernel.

Arms:
* default (``--impl ours``): ``value`` = samples / device time of the render
  launch with bricks, transfer function, per-pixel rays, kd order and pixel
  rectangles resident in HBM (L2 flushed between steps); ``e2e`` = the same
  render through the drop-in ``VolumeRenderSampler`` call surface from host
  numpy arrays to the host image, copies included.
* ``--impl reference``: yt's own compiled sampler (or, where it was not
  built, the C oracle) on the host cores, over a bounded sample of the same
  view (a reduced-resolution image of the same camera, all bricks).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_SAMPLE = 32   # 8 float32 vertex values gathered per trilinear sample
BYTES_PER_RAY = 64      # float64 RGBA read + written per ray


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--res", type=int, default=1024)
    ap.add_argument("--root", type=int, default=128)
    ap.add_argument("--levels", type=int, default=3)
    ap.add_argument("--cpu-res", type=int, default=0, help="resolution of the CPU-baseline sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.proc = None
        self.index = index
        self.path = Path("/tmp") / f"ytgb_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path.exists():
            return None
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
            except ValueError:
                continue
        self.path.unlink(missing_ok=True)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def build_workload(args):
    from yt_gb300 import workloads

    t = time.time()
    w = workloads.amr_vr(root=args.root, levels=args.levels, res=args.res)
    return w, time.time() - t


def cpu_reference(w, res, threads):
    """Time yt's compiled sampler (or the C oracle) over the view at ``res``."""
    from yt_gb300.camera import Camera

    cam0 = w.views[0].camera
    cam = Camera(cam0.position, cam0.focus, cam0.width, res, lens_type=cam0.lens_type)
    order = w.order(cam)
    p = cam.sampler_params()
    kind = "port"
    try:
        ref_pkg = ROOT / "oracle" / "_ref" / "pkg"
        if not any((ref_pkg / "yt" / "utilities" / "lib").glob("image_samplers*.so")):
            raise ImportError("reference sampler not built")
        sys.path.insert(0, str(ref_pkg))
        from yt.utilities.lib import image_samplers as RIS  # noqa: PLC0415
        from yt.utilities.lib.partitioned_grid import PartitionedGrid  # noqa: PLC0415

        pgs = []
        for k in order:
            data, mask, le, re, dims = w.bricks[k]
            pgs.append(PartitionedGrid(0, data, mask, le, re, np.asarray(dims, dtype=np.int64)))
        s = RIS.VolumeRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"],
                                    p["bounds"], p["image"], p["x_vec"], p["y_vec"], p["width"], "KDTree", w.tf, 1,
                                    lens_type=p["lens_type"], camera_data=p["camera_data"],
                                    zbuffer=np.ones(p["image"].shape[:2]))
        t0 = time.perf_counter()
        for pg in pgs:
            s(pg, num_threads=threads)
        dt = time.perf_counter() - t0
        image = np.array(s.aimage)
        kind = "reference"
        from oracle import cpu as ocpu  # noqa: PLC0415   the visit count comes from the oracle

        so = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"],
                                np.zeros_like(p["image"]), p["x_vec"], p["y_vec"], p["width"],
                                lens_type=p["lens_type"], camera_data=p["camera_data"], tf=w.tf)
        _, counts = so.trace(ocpu.OracleBricks(w.bricks), order, num_threads=threads)
        samples = int(counts.sum())
    except ImportError:
        from oracle import cpu as ocpu  # noqa: PLC0415

        so = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                                p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                                camera_data=p["camera_data"], tf=w.tf)
        ob = ocpu.OracleBricks(w.bricks)
        t0 = time.perf_counter()
        samples = so.render(ob, order, num_threads=threads)
        dt = time.perf_counter() - t0
        image = p["image"]
    return {"samples": samples, "seconds": dt, "kind": kind, "image": image, "camera": cam, "order": order}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w, _ = build_workload(args)
    threads = os.cpu_count() or 1
    res = args.cpu_res or max(64, args.res // 4)
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        info = cpu_reference(w, res, threads)
        if i >= args.warmup:
            vals.append(info["samples"] / info["seconds"] / 1e9)
    v = float(np.mean(vals))
    sample = f"the same camera at {res}x{res} ({info['samples']} samples per step), all {len(w.bricks)} bricks"
    line = {"impl": "reference", "metric": "Gsamples/s", "value": v, "unit": "Gsamples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * info["seconds"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(w, args),
            "cpu_baseline": {"value": v, "unit": "Gsamples/s", "cores": threads, "kind": info["kind"],
                             "sample": sample},
            "e2e": {"value": v, "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(w, args):
    return {"workload": "amr_vr: 128^3 blob root + 3 factor-2 levels (16^3 patches), kd bricks, "
                        "VolumeRenderSampler, perspective lens, 8-layer ColorTransferFunction, 1 sample/cell",
            "resolution": args.res, "bricks": len(w.bricks), "grids": w.info.get("grids"),
            "root": args.root, "levels": args.levels, "l2": "flushed between steps (256 MiB write)"}


def traffic_from_profile():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def run_ours(args):
    import torch

    from yt_gb300 import _lib
    from yt_gb300.render import Renderer, relative_error

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    w, t_build = build_workload(args)
    cam = w.views[0].camera
    r = Renderer(w.bricks, w.tf, device=dev, kdtree=w.kdtree)
    order = r.order(cam)
    view, ppos, pdir = r.view_args(cam)
    px_pos = torch.from_numpy(ppos).to(dev) if ppos is not None else None
    px_dir = torch.from_numpy(pdir).to(dev) if pdir is not None else None
    rects = r.bricks.rects(view, order)
    nx, ny = cam.resolution
    image = torch.zeros((nx, ny, 4), dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2
    stream = torch.cuda.current_stream(dev)
    from yt_gb300.volume import render as vrender

    keep = []

    def step():
        image.zero_()
        vrender(r.bricks, view, order, _lib.VOLUME_RENDER, image, tf=r.packed, counters=r.counters, error=r.error,
                px_pos=px_pos, px_dir=px_dir, stream=stream, rects=rects, keep=keep)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    r.check()
    keep.clear()
    r.counters.zero_()
    times = []
    launches = 0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index)
    with clocks:
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            image.zero_()
            e0.record(stream)
            vrender(r.bricks, view, order, _lib.VOLUME_RENDER, image, tf=r.packed, counters=r.counters,
                    error=r.error, px_pos=px_pos, px_dir=px_dir, stream=stream, rects=rects, keep=keep)
            e1.record(stream)
            launches += 1
            times.append((e0, e1))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if world > 1:
        torch.distributed.barrier()
    r.check()
    keep.clear()
    ms = np.array([a.elapsed_time(b) for a, b in times])
    samples_total = int(r.counters[0].item())
    rays = int(r.counters[2].item()) // max(args.steps, 1)
    samples_step = samples_total // args.steps
    walks_step = int(r.counters[1].item()) // max(args.steps, 1)
    guarded_step = int(r.counters[3].item()) // max(args.steps, 1)
    t_total = float(ms.sum()) / 1e3
    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([t_total], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_total = float(tt.item())
    value = samples_total * world / t_total / 1e9
    hbm, peak_kind = peaks()
    alg_bytes = samples_step * BYTES_PER_SAMPLE + rays * BYTES_PER_RAY
    achieved = alg_bytes / (float(ms.mean()) / 1e3) / 1e9
    prof = traffic_from_profile() or {}
    traffic = prof.get("amr_vr_dram_bytes_per_launch")

    # e2e through the drop-in sampler API: host numpy bricks -> host image
    e2e = None
    if not args.no_e2e:
        from yt_gb300.image_samplers import VolumeRenderSampler
        from yt_gb300.partitioned_grid import PartitionedGrid

        p = cam.sampler_params()
        pgs = [PartitionedGrid(0, *w.bricks[k]) for k in order]
        ets = []
        h2d = d2h = 0
        for i in range(args.warmup + max(3, args.steps // 4)):
            img_h = np.zeros((nx, ny, 4))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s = VolumeRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"],
                                    p["bounds"], img_h, p["x_vec"], p["y_vec"], p["width"], "KDTree", w.tf, 1,
                                    lens_type=p["lens_type"], camera_data=p["camera_data"],
                                    zbuffer=np.ones((nx, ny)))
            for pg in pgs:
                s(pg, num_threads=0)
            out = s.aimage
            t1 = time.perf_counter()
            if i >= args.warmup:
                ets.append(t1 - t0)
        h2d = r.bricks.nbytes + img_h.nbytes + nx * ny * 8 + (ppos.nbytes + pdir.nbytes if ppos is not None else 0)
        d2h = img_h.nbytes
        e2e_v = samples_step / float(np.median(ets)) / 1e9
        e2e = {"value": e2e_v, "unit": "Gsamples/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": 1e3 * float(np.median(ets)), "path": "VolumeRenderSampler(...)(pg) per brick, aimage"}
        del out

    line = {"metric": "Gsamples/s", "value": value, "unit": "Gsamples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(ms.mean()), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 sampling / f64 traversal", "data": "synthetic",
            "config": config_dict(w, args),
            "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99))},
            "samples_per_step": samples_step, "rays_per_step": rays, "brick_walks_per_step": walks_step,
            "out_of_brick_cells_per_step": guarded_step,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic,
                         "peak_source": peak_kind + " hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                         else "fallback 6800 GB/s",
                         "algorithmic_bytes_per_launch": int(alg_bytes),
                         "model": f"{BYTES_PER_SAMPLE} B/sample + {BYTES_PER_RAY} B/ray"},
            "gpu_launches": launches, "e2e": e2e, "clocks": clocks.summary(), "build_seconds": t_build}

    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        res = args.cpu_res or max(64, args.res // 4)
        ref = cpu_reference(w, res, threads)
        img_g = r.render(ref["camera"], kind=_lib.VOLUME_RENDER, order=ref["order"]).cpu().numpy()
        mx, rms = relative_error(img_g, ref["image"], channels=(0, 1, 2))
        line["cpu_baseline"] = {"value": ref["samples"] / ref["seconds"] / 1e9, "unit": "Gsamples/s",
                                "cores": threads, "kind": ref["kind"],
                                "sample": f"the same camera at {res}x{res} ({ref['samples']} samples), all bricks"}
        line["accuracy"] = {"max_rel_err": mx, "rms_rel_err": rms, "vs": f"float64 render at {res}x{res}",
                            "tau": 1e-6}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
