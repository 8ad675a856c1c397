#!/usr/bin/env python
"""Benchmark of the splat pipeline on GB300: forward frames of 1,000,000 Gaussians at 1920x1080.

Workload: the scene-scale forward configuration (1M Gaussians, SH degree 3, seed 1, 64-cluster
mixture in a 20^3 box, camera inside the box, fov 70, 1920x1080, 16x16 tiles), seeded synthetic
data (the reference's scenes are not available). One step = one frame: preprocess, offset scan +
emit, radix sort, tile ranges, raster, replayed from one CUDA graph.

  value  Mpix/s over exactly K frames, scene resident in HBM, image left on the device, timed with
         CUDA events on the context stream (the 236 MB scene is larger than the 129 MB L2).
  e2e    the same metric through the C ABI with host buffers: every step copies the 176-byte view
         block host->device and the rgba8 image device->host (pinned), wall clock.
  roofline, per-pass ms, cpu_baseline (the CPU oracle on the host cores) and clocks ride along.

--impl reference times the reference's own algorithm on the host cores instead: the reference is
WGSL + JavaScript (a WebGPU app) whose GPU path cannot run on this machine, so its CPU restatement
(oracle/) is timed with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "web-gs-renderer_gb300"))

METRIC = "fwd Mpix/s (ms/frame), 1M splats 1920x1080"
WORKLOAD = "scene-scale forward: 1M Gaussians (64-cluster mixture, 20^3 box, seed 1), 1920x1080, fov 70, 16x16 tiles"
PEAKS = ROOT / "MEASURED_PEAKS.json"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--cpu-configs", action="store_true",
                    help="time the CPU oracle on every benchmark configuration (all host cores and one core) "
                         "and print one JSON line; no GPU work")
    ap.add_argument("--launch-check", action="store_true",
                    help="start the ranks and report them (gloo, no GPU work, no metric): a check of the launcher")
    return ap.parse_args()


# ---- clocks ------------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.2)

    def stop(self) -> dict:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        # "under load": samples whose power is in the upper half of the observed range
        if pw:
            thr = min(pw) + 0.5 * (max(pw) - min(pw))
            loaded = [float(r[1]) for r in rows if r[3].replace(".", "").isdigit() and float(r[3]) >= thr
                      and r[1].replace(".", "").isdigit()]
        else:
            loaded = sm
        return {"sm_mhz": statistics.median(loaded or sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


# ---- algorithmic bytes per pass ----------------------------------------------------------------------
def algorithmic_bytes(fi: dict, n: int, pixels: int, passes: int) -> dict:
    npass, vis, s = fi["near_pass"], fi["visible"], fi["sorted_count"]
    tiles = fi["tiles_x"] * fi["tiles_y"]
    return {
        # the tile ranges cleared, the control block's counters and digit histograms reset
        "frame begin": 8 * tiles + 8 * 1024,
        # 12 B position of every Gaussian + the other 224 B of each one in front of the near plane;
        # writes: 4 B count each, 48 B raster record per near-plane survivor, 16 B rect per visible
        "preprocess": 12 * n + 224 * npass + 4 * n + 48 * npass + 16 * vis,
        # counts + rects in, offsets + keys/values out
        "scan+emit": 4 * (n + 1) + 16 * vis + 4 * (n + 1) + 8 * s,
        # each pass reads and writes keys and values (the last one also leaves the tile ranges)
        "sort": passes * 16 * s,
        # the ranges read twice (bin counts, placement), the order written
        "tile order": 2 * 8 * tiles + 4 * tiles,
        # per instance the index and the 48 B record, per tile its range, per pixel 4 B rgba8
        "raster": 52 * s + 8 * tiles + 4 * pixels,
    }


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum, one ncu --set full capture of
# the forward frame of this workload on a GB300) and what bounds each kernel there.
NCU_TRAFFIC_BYTES = {"preprocess": 286.5e6, "raster": 56.6e6}
# issue-slot utilisation of the kernels bound by instruction issue (ncu smsp__issue_active, one
# capture of the kernel at this workload): for them this, not the HBM fraction, is the efficiency measure
NCU_ISSUE_ACTIVE = {"raster": 0.933}
# warp instructions per launch (ncu smsp__inst_executed.sum, the same capture): the numerator of the
# issue-rate roofline of those kernels (four issue slots per SM per cycle)
NCU_WARP_INSTRUCTIONS = {"raster": 275.27e6}
LIMITER = {
    "raster": "instruction issue (ncu: issue slots busy 93.3% at full residency, DRAM 3% of peak; the "
              "48-byte records are re-read from L2, so DRAM traffic is below the algorithmic bytes)",
    "preprocess": "HBM and the pinned arithmetic (ncu: 69% of DRAM peak, 70% of issue slots)",
}


def peaks() -> tuple[float, str]:
    try:
        d = json.loads(PEAKS.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---- CPU side ------------------------------------------------------------------------------------------
def cpu_frame_rate(packed, count, view, target_s: float, row_stride: int = 1, threads: int | None = None) -> dict:
    import oracle
    import webgs

    vb = webgs.view_bytes(view)
    w, h = int(view.texture_size[0]), int(view.texture_size[1])
    threads = threads or os.cpu_count() or 1
    times, frames = [], 0
    t_end = time.perf_counter() + target_s
    while True:
        t0 = time.perf_counter()
        oracle.forward_f32(vb, packed, count, threads=threads, keys=False, timed=True, row_stride=row_stride)
        times.append(time.perf_counter() - t0)
        frames += 1
        if time.perf_counter() >= t_end:
            break
    rows = len(range(0, (h + 15) // 16, row_stride))
    pix = min(h, rows * 16) * w if row_stride > 1 else w * h
    mean = sum(times) / len(times)
    return {"value": pix / mean / 1e6, "ms_per_frame": mean * 1e3, "frames": frames, "threads": threads,
            "pixels_per_frame": pix}


def _cpu_inputs(spec, cam):
    """The scene and the view block from the oracle's own generators (no product library)."""
    import oracle

    packed = oracle.synth_scene(spec.kind, spec.count, spec.seed, spec.clusters, spec.box)
    vb = oracle.camera_view(cam.eye, cam.target, (0.0, 1.0, 0.0), cam.fovy, cam.width, cam.height, cam.z_near,
                            cam.z_far)
    return packed, vb


def cpu_forward(vb: bytes, packed, n: int, threads: int) -> dict:
    """One fp32 frame of the oracle: wall ms and per-pass ms."""
    import oracle

    t0 = time.perf_counter()
    o = oracle.forward_f32(vb, packed, n, threads=threads, keys=False, timed=True)
    ms = (time.perf_counter() - t0) * 1e3
    return {"ms": round(ms, 2), "passes_ms": {k: round(v, 2) for k, v in o["pass_ms"].items()}, "rgb": o["rgb"]}


def cpu_forward_backward(vb: bytes, packed, n: int, target, threads: int) -> dict:
    """One differentiation step on the CPU: the fp32 frame, the FP64 L1 + 0.2 (1 - SSIM) loss and its
    image gradient, and the FP64 adjoint of the whole pipeline (which re-runs the frame in FP64)."""
    import oracle

    f = cpu_forward(vb, packed, n, threads)
    t0 = time.perf_counter()
    _, dl = oracle.loss_l1_ssim(f["rgb"], target, 0.2)
    t_loss = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    oracle.backward_f64(vb, packed, n, dl, threads=threads)
    t_bwd = (time.perf_counter() - t0) * 1e3
    passes = dict(f["passes_ms"])
    passes.update({"loss (FP64)": round(t_loss, 2), "adjoint backward (FP64)": round(t_bwd, 2)})
    return {"ms": round(f["ms"] + t_loss + t_bwd, 2), "passes_ms": passes}


def cpu_configs(threads_list) -> dict:
    """The oracle (oracle/, C++ with OpenMP) on every benchmark configuration, per pass, with each
    thread count of threads_list; the CPU baselines beside the GPU numbers of each configuration."""
    import oracle
    from webgs import workloads as W

    out = {}
    for threads in threads_list:
        row = {}
        packed, vb = _cpu_inputs(W.SMALL_SCENE, W.SMALL_CAMERA)
        f = cpu_forward(vb, packed, W.SMALL_SCENE.count, threads)
        row["small 50k 512x512 fwd"] = {"ms_per_frame": f["ms"], "passes_ms": f["passes_ms"],
                                        "Mpix_s": round(512 * 512 / f["ms"] / 1e3, 3)}
        packed, vb = _cpu_inputs(W.SCENE_1M, W.CAMERA_1080P)
        f = cpu_forward(vb, packed, W.SCENE_1M.count, threads)
        row["scene 1M 1920x1080 fwd"] = {"ms_per_frame": f["ms"], "passes_ms": f["passes_ms"],
                                         "Mpix_s": round(1920 * 1080 / f["ms"] / 1e3, 3)}
        spec, cam = W.SCENE_500K, W.CAMERA_720P
        packed, vb = _cpu_inputs(spec, cam)
        target = oracle.forward_f32(vb, oracle.perturb_scene(packed, spec.count, 99, 0.01, 0.02), spec.count,
                                    threads=threads, keys=False)["rgb"]
        fb = cpu_forward_backward(vb, packed, spec.count, target, threads)
        row["diff 500k 1280x720 fwd+bwd"] = {"ms_per_step": fb["ms"], "passes_ms": fb["passes_ms"],
                                             "Mpix_s": round(1280 * 720 / fb["ms"] / 1e3, 3)}
        # batched forward: the 16 orbit views of the three scenes (one core: the first four views)
        packs = [oracle.synth_scene(sp.kind, sp.count, sp.seed, sp.clusters, sp.box) for sp in W.BATCH_SCENES]
        cams = W.orbit_cameras(16, 2024, 9.0)
        sample = cams if threads > 1 else cams[:4]
        ms, pix = 0.0, 0
        for si, c in sample:
            vbv = oracle.camera_view(c.eye, c.target, (0.0, 1.0, 0.0), c.fovy, c.width, c.height, c.z_near, c.z_far)
            ms += cpu_forward(vbv, packs[si], W.BATCH_SCENES[si].count, threads)["ms"]
            pix += c.width * c.height
        row["batched 16 views fwd"] = {"ms_per_view": round(ms / len(sample), 2), "Mpix_s": round(pix / ms / 1e3, 3),
                                       "views_timed": len(sample)}
        # batched forward+backward: 3M scene, 8 views at 1080p (timed: the first view)
        spec = W.SCENE_3M
        packed = oracle.synth_scene(spec.kind, spec.count, spec.seed, spec.clusters, spec.box)
        c = [c for _, c in W.orbit_cameras(8, 77, 18.0, fixed_resolution=(1920, 1080))][0]
        vbv = oracle.camera_view(c.eye, c.target, (0.0, 1.0, 0.0), c.fovy, c.width, c.height, c.z_near, c.z_far)
        target = oracle.forward_f32(vbv, oracle.perturb_scene(packed, spec.count, 99, 0.01, 0.02), spec.count,
                                    threads=threads, keys=False)["rgb"]
        fb = cpu_forward_backward(vbv, packed, spec.count, target, threads)
        row["batched 3M 8x1080p fwd+bwd"] = {"ms_per_view": fb["ms"], "passes_ms": fb["passes_ms"],
                                             "views_timed": 1}
        out[f"{threads}_threads"] = row
    return out


def run_reference(args, rank: int, world: int) -> None:
    if rank != 0:
        return
    import oracle
    from webgs import workloads as W  # the workload's sizes only: no product code is loaded

    spec, cam = W.SCENE_1M, W.CAMERA_1080P
    # inputs from the oracle's own generators (bit-identical to the product's, tests/test_oracle_inputs.py)
    packed = oracle.synth_scene(spec.kind, spec.count, spec.seed, spec.clusters, spec.box)
    vb = oracle.camera_view(cam.eye, cam.target, (0.0, 1.0, 0.0), cam.fovy, cam.width, cam.height, cam.z_near,
                            cam.z_far)
    threads = os.cpu_count() or 1
    # size the step so W + K steps take about two minutes: the whole frame when that fits, else the
    # global passes plus every m-th tile row of the raster
    t0 = time.perf_counter()
    oracle.forward_f32(vb, packed, spec.count, threads=threads, keys=False)
    t_full = time.perf_counter() - t0
    budget = 120.0
    m = 1
    while (args.warmup + args.steps) * t_full / m > budget and m < 68:
        m *= 2
    for _ in range(args.warmup):
        oracle.forward_f32(vb, packed, spec.count, threads=threads, keys=False, row_stride=m)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.forward_f32(vb, packed, spec.count, threads=threads, keys=False, row_stride=m)
        times.append(time.perf_counter() - t0)
    rows = len(range(0, (cam.height + 15) // 16, m))
    pix = min(cam.height, rows * 16) * cam.width if m > 1 else cam.width * cam.height
    total = sum(times)
    value = pix * args.steps / total / 1e6
    sample = ("whole frame per step" if m == 1 else
              f"per step: all passes over the whole scene, raster of every {m}th tile row ({pix} of "
              f"{cam.width * cam.height} pixels); whole frame {t_full * 1e3:.0f} ms")
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "Mpix/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "l2": "inputs larger than L2"}, "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "Mpix/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "whole_frame_ms": round(t_full * 1e3, 2),
        "note": "the reference is a WebGPU app (WGSL + JavaScript); its GPU path is unavailable on this box, "
                "so its algorithm is timed as the project's CPU restatement (oracle/, C++/OpenMP)",
    }
    print(json.dumps(line), flush=True)


# ---- GPU side ------------------------------------------------------------------------------------------
def run_ours(args, rank: int, world: int, local_rank: int) -> None:
    import ctypes as C

    import numpy as np
    import torch

    import webgs
    from webgs import _abi, workloads as W

    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        if torch.cuda.device_count() <= local_rank:
            raise SystemExit(f"rank {rank}: --gpus {world} needs {world} GPUs, this node has "
                             f"{torch.cuda.device_count()}")
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    spec, cam = W.SCENE_1M, W.CAMERA_1080P
    packed = spec.build()
    view = cam.view()
    w, h = cam.width, cam.height
    pixels = w * h
    lib = webgs.library()

    ctx = webgs.Context(device=local_rank)
    scene = ctx.upload(packed, spec.count)
    rgba = torch.empty(pixels, dtype=torch.int32, device=f"cuda:{local_rank}")
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{local_rank}")

    def frame():
        ctx.forward_device(scene, view, rgba8=rgba.data_ptr())

    sampler = ClockSampler(local_rank)
    sampler.start()
    for _ in range(max(args.warmup, 3)):
        frame()
    ctx.synchronize()
    fi = ctx.frame_info()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        frame()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    dt_ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([dt_ms], device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt_ms = float(t.item())
        dist.barrier()

    # end to end: host view in, host image out, through the C ABI
    host_img = torch.empty(pixels * 4, dtype=torch.uint8, pin_memory=True)
    img = _abi.Image(webgs.GS_MEM_HOST, host_img.data_ptr(), None, None, None)
    for _ in range(3):
        ctx._ck(lib.gs_forward(ctx.handle, scene.handle, C.byref(view), C.byref(img)))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx._ck(lib.gs_forward(ctx.handle, scene.handle, C.byref(view), C.byref(img)))
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    clocks = sampler.stop()

    # per-pass times with CUDA events on the context stream (a profiling context, same workload)
    pctx = webgs.Context(device=local_rank, flags=webgs.GS_FLAG_PROFILE)
    pscene = pctx.upload(packed, spec.count)
    prgba = torch.empty(pixels, dtype=torch.int32, device=f"cuda:{local_rank}")
    for _ in range(3):
        pctx.forward_device(pscene, view, rgba8=prgba.data_ptr())
    acc: dict[str, float] = {}
    prof_steps = max(5, min(args.steps, 50))
    for _ in range(prof_steps):
        pctx.forward_device(pscene, view, rgba8=prgba.data_ptr())
        for k, v in pctx.timings().items():
            acc[k] = acc.get(k, 0.0) + v["ms"]
    pass_ms = {k: v / prof_steps for k, v in acc.items()}
    pscene.close()
    pctx.close()

    # forward + backward: frame, L1 + 0.2 (1 - SSIM) against a perturbed-scene target, gradients of
    # all 59 attributes, everything on the device; timed like the forward
    scene.close()
    ctx.close()
    cpu_legs = not args.no_cpu_baseline and world == 1
    fb_1080 = fwd_bwd(W.SCENE_1M, W.CAMERA_1080P, packed, args.steps, args.warmup, local_rank)
    fb_720 = fwd_bwd(W.SCENE_500K, W.CAMERA_720P, None, args.steps, args.warmup, local_rank, cpu=cpu_legs)
    batched = None if args.no_batched else batched_forward(args.steps, args.warmup, local_rank, cpu=cpu_legs)
    batched_fb = (None if args.no_batched else
                  batched_fwd_bwd(max(3, args.steps // 5), args.warmup, local_rank, cpu=cpu_legs))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    ms = dt_ms / args.steps
    value = world * pixels * args.steps / (dt_ms / 1e3) / 1e6
    e2e = world * pixels * args.steps / e2e_s / 1e6
    passes = fi["sort_passes"]
    bytes_per = algorithmic_bytes(fi, spec.count, pixels, passes)
    kernel_passes = {k: v for k, v in pass_ms.items() if k != "TOTAL"}
    top = max(kernel_passes, key=kernel_passes.get)
    peak, peak_kind = peaks()
    achieved = bytes_per[top] / (kernel_passes[top] * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": NCU_TRAFFIC_BYTES.get(top), "peak_source": peak_kind,
            "algorithmic_bytes": int(bytes_per[top]), "limiter": LIMITER.get(top),
            "issue_active_ncu": NCU_ISSUE_ACTIVE.get(top)}
    # the dominant kernel's own bound: warp instructions per launch over its event time, against four
    # issue slots per SM per cycle at the median SM clock sampled under load
    roof_issue = None
    if top in NCU_WARP_INSTRUCTIONS and clocks.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
        achieved_i = NCU_WARP_INSTRUCTIONS[top] / (kernel_passes[top] * 1e-3) / 1e9
        peak_i = sms * 4 * clocks["sm_mhz"] * 1e6 / 1e9
        roof_issue = {"bound": "instruction issue", "kernel": top, "achieved": round(achieved_i, 1),
                      "peak": round(peak_i, 1), "unit": "G warp-instructions/s", "frac": round(achieved_i / peak_i, 4),
                      "warp_instructions": NCU_WARP_INSTRUCTIONS[top], "sms": sms, "sm_mhz": clocks["sm_mhz"]}
    per_pass = {k: {"ms": round(v, 4), "bytes": int(bytes_per.get(k, 0)),
                    "GBps": round(bytes_per.get(k, 0) / (v * 1e-3) / 1e9, 1) if v > 0 and k in bytes_per else None}
                for k, v in pass_ms.items()}

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        r = cpu_frame_rate(packed, spec.count, view, target_s=10.0)
        r1 = cpu_frame_rate(packed, spec.count, view, target_s=0.0, threads=1)  # one frame on one core
        cpu = {"value": round(r["value"], 4), "unit": "Mpix/s", "cores": r["threads"], "kind": "port",
               "sample": f"{r['frames']} whole frames of the same workload, oracle/ C++ OpenMP, "
                         f"{r['ms_per_frame']:.0f} ms/frame",
               "value_1core": round(r1["value"], 4), "ms_per_frame_1core": round(r1["ms_per_frame"], 1)}

    # frame_begin, preprocess, scan+emit, passes x onesweep, tile bins, tile place, raster
    launches_per_frame = 6 + passes
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas x{world}", "l2": "inputs larger than L2",
                   "instances": fi["instance_count"], "visible": fi["visible"], "sort_passes": passes},
        "e2e": {"value": round(e2e, 3), "unit": "Mpix/s", "ms_per_step": round(e2e_s / args.steps * 1e3, 4),
                "h2d_bytes_per_step": 176, "d2h_bytes_per_step": pixels * 4},
        "roofline": roof, "roofline_issue": roof_issue, "passes": per_pass, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": launches_per_frame * args.steps,
        "fwd_bwd": {"1M_1080p": fb_1080, "500k_720p": fb_720},
        "batched_fwd_16_views": batched, "batched_fwd_bwd_8_views": batched_fb,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def fwd_bwd(spec, cam, packed, steps, warmup, local_rank, cpu: bool = False) -> dict:
    """ms per forward + loss + backward step on the device (CUDA events on the context stream)."""
    import ctypes as C

    import torch

    import webgs
    from webgs import _abi

    lib = webgs.library()
    if packed is None:
        packed = spec.build()
    view = cam.view()
    w, h, n = cam.width, cam.height, spec.count
    dev = f"cuda:{local_rank}"
    ctx = webgs.Context(device=local_rank, flags=webgs.GS_FLAG_DIFFERENTIABLE)
    target = torch.empty(h * w * 3, dtype=torch.float32, device=dev)
    ts = ctx.upload(webgs.perturb_scene(packed, n, 99, 0.01, 0.02), n)
    ctx.forward_device(ts, view, rgb=target.data_ptr())
    ctx.synchronize()
    ts.close()
    sc = ctx.upload(packed, n)
    rgb = torch.empty_like(target)
    dl = torch.empty_like(target)
    grads = torch.empty(59 * n, dtype=torch.float32, device=dev)
    img = _abi.Image(webgs.GS_MEM_DEVICE, None, rgb.data_ptr(), None, None)

    def step():
        ctx._ck(lib.gs_forward(ctx.handle, sc.handle, C.byref(view), C.byref(img)))
        ctx._ck(lib.gs_loss_l1_ssim(ctx.handle, rgb.data_ptr(), target.data_ptr(), w, h, 0.2, None, dl.data_ptr(),
                                    webgs.GS_MEM_DEVICE))
        ctx._ck(lib.gs_backward(ctx.handle, sc.handle, dl.data_ptr(), grads.data_ptr(), webgs.GS_MEM_DEVICE))

    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    for _ in range(max(warmup, 3)):
        step()
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    loss = C.c_double()
    ctx._ck(lib.gs_loss_l1_ssim(ctx.handle, rgb.data_ptr(), target.data_ptr(), w, h, 0.2, C.byref(loss), None,
                                webgs.GS_MEM_DEVICE))
    sc.close()
    ctx.close()

    # per-pass times of the same step from a profiling context (CUDA events between the passes)
    pctx = webgs.Context(device=local_rank, flags=webgs.GS_FLAG_DIFFERENTIABLE | webgs.GS_FLAG_PROFILE)
    psc = pctx.upload(packed, n)
    pimg = _abi.Image(webgs.GS_MEM_DEVICE, None, rgb.data_ptr(), None, None)
    acc: dict[str, float] = {}
    prof_steps = max(3, min(steps, 20))
    for it in range(prof_steps + 1):
        pctx._ck(lib.gs_forward(pctx.handle, psc.handle, C.byref(view), C.byref(pimg)))
        pctx._ck(lib.gs_loss_l1_ssim(pctx.handle, rgb.data_ptr(), target.data_ptr(), w, h, 0.2, None,
                                     dl.data_ptr(), webgs.GS_MEM_DEVICE))
        pctx._ck(lib.gs_backward(pctx.handle, psc.handle, dl.data_ptr(), grads.data_ptr(), webgs.GS_MEM_DEVICE))
        if it:
            for k, v in pctx.timings().items():
                acc[k] = acc.get(k, 0.0) + v["ms"] / prof_steps
    psc.close()
    pctx.close()
    res = {"ms_per_step": round(ms, 4), "Mpix/s": round(w * h / ms / 1e3, 2), "loss": round(loss.value, 6),
           "passes_ms": {k: round(v, 4) for k, v in acc.items()},
           "workload": f"{n} Gaussians {w}x{h}, L1 + 0.2(1-SSIM) vs perturbed-scene target, grads of 59*N floats"}
    if cpu:
        import oracle

        threads = os.cpu_count() or 1
        vb = webgs.view_bytes(view)
        target_cpu = oracle.forward_f32(vb, webgs.perturb_scene(packed, n, 99, 0.01, 0.02), n, threads=threads,
                                        keys=False)["rgb"]
        c = cpu_forward_backward(vb, packed, n, target_cpu, threads)
        res["cpu_baseline"] = {"value": round(w * h / c["ms"] / 1e3, 4), "unit": "Mpix/s", "ms_per_step": c["ms"],
                               "cores": threads, "kind": "port", "passes_ms": c["passes_ms"],
                               "sample": "one step of the same workload: fp32 frame, FP64 loss, FP64 adjoint"}
    return res


def launch_ranks(args) -> int:
    """`bench.py --gpus N` started without a launcher: one process per GPU through
    torch.distributed.run (rendezvous on 127.0.0.1), the same command line in every rank; rank 0
    prints the JSON line. Returns the launcher's exit status."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    env = dict(os.environ)
    # the launcher would pin every rank to one OpenMP thread; the ranks share the host's cores instead
    env.setdefault("OMP_NUM_THREADS", str(max(1, (os.cpu_count() or 1) // args.gpus)))
    return subprocess.call(cmd, env=env)


def launch_check(rank: int, world: int) -> None:
    """Every rank joins a gloo group and reports its rank; rank 0 prints them (no GPU, no metric)."""
    import torch
    import torch.distributed as dist

    if world > 1:
        dist.init_process_group("gloo")
        ranks = [None] * world
        dist.all_gather_object(ranks, {"rank": rank, "local_rank": int(os.environ.get("LOCAL_RANK", "0")),
                                       "pid": os.getpid()})
        dist.barrier()
        dist.destroy_process_group()
    else:
        ranks = [{"rank": 0, "local_rank": 0, "pid": os.getpid()}]
    if rank == 0:
        print(json.dumps({"launch_check": True, "n_gpus": world, "ranks": ranks, "torch": torch.__version__}),
              flush=True)


def main():
    args = parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.launch_check:
        launch_check(rank, world)
    elif args.cpu_configs:
        if rank == 0:
            cores = os.cpu_count() or 1
            print(json.dumps({"cpu_configs": cpu_configs([cores, 1]), "cores": cores, "kind": "port",
                              "note": "the oracle (oracle/, C++/OpenMP): fp32 frames, FP64 loss and FP64 adjoint"}),
                  flush=True)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


def _timed(stream, fn, steps, warmup):
    import torch

    for _ in range(max(warmup, 3)):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def batched_forward(steps, warmup, local_rank, cpu: bool = False) -> dict:
    """3 scenes (100k, 400k, 1.5M; seeds 3-5), 16 cameras on random orbits, resolutions from
    {640x480, 1280x720, 1920x1080}: one batched launch vs 16 plain frames. The autotuner first picks
    tile size, digit width, raster batch depth and sort block on the whole batch."""
    import ctypes as C

    import torch

    import webgs
    from webgs import _abi, workloads as W

    lib = webgs.library()
    dev = f"cuda:{local_rank}"
    packs = [s.build() for s in W.BATCH_SCENES]
    cams = W.orbit_cameras(16, 2024, 9.0)
    views = [c.view() for _, c in cams]
    t0 = time.perf_counter()
    tuned, tuned_ms = webgs.autotune_scenes([(p, s.count) for s, p in zip(W.BATCH_SCENES, packs)], views,
                                            [si for si, _ in cams], iters=2, device=local_rank)
    tune_s = time.perf_counter() - t0
    res = {}
    for label, cfg in (("default", {}), ("autotuned", tuned)):
        ctx = webgs.Context(device=local_rank, **cfg)
        scs = [ctx.upload(p, s.count) for s, p in zip(W.BATCH_SCENES, packs)]
        imgs = [torch.empty(c.width * c.height, dtype=torch.int32, device=dev) for _, c in cams]
        stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
        arr = (_abi.BatchView * len(cams))()
        for k, ((si, c), v) in enumerate(zip(cams, views)):
            arr[k].scene = scs[si].handle
            arr[k].view = v
            arr[k].out = _abi.Image(webgs.GS_MEM_DEVICE, imgs[k].data_ptr(), None, None, None)

        def plain():
            for k, (si, _) in enumerate(cams):
                ctx.forward_device(scs[si], views[k], rgba8=imgs[k].data_ptr())

        def batch():
            ctx._ck(lib.gs_forward_batch(ctx.handle, arr, len(cams)))

        ms_plain = _timed(stream, plain, steps, warmup)
        ms_batch = _timed(stream, batch, steps, warmup)
        pix = sum(c.width * c.height for _, c in cams)
        if label == "default":
            # each view alone (graph-replayed frames): the large views bound what overlap can gain
            per_view = []
            for k, (si, c) in enumerate(cams):
                def one(k=k, si=si):
                    ctx.forward_device(scs[si], views[k], rgba8=imgs[k].data_ptr())
                per_view.append({"scene": W.BATCH_SCENES[si].count, "res": f"{c.width}x{c.height}",
                                 "ms": round(_timed(stream, one, max(5, steps // 2), warmup), 4)})
        res[label] = {"config": cfg or {"tile_size": 16, "digit_bits": 8, "raster_batch": 256, "sort_block": 4096},
                      "plain_ms_per_view": round(ms_plain / len(cams), 4),
                      "batched_ms_per_view": round(ms_batch / len(cams), 4),
                      "plain_Mpix_s": round(pix / ms_plain / 1e3, 1), "batched_Mpix_s": round(pix / ms_batch / 1e3, 1),
                      "batched_over_plain": round(ms_plain / ms_batch, 3)}
        if label == "default":
            big = sum(v["ms"] for v in per_view if v["scene"] == max(s.count for s in W.BATCH_SCENES))
            res[label]["per_view_plain"] = per_view
            res[label]["largest_scene_views_ms"] = round(big, 4)
            res[label]["overlap_bound_batched_over_plain"] = round(sum(v["ms"] for v in per_view) / big, 3)
            # per-pass times of the same 16 frames (profiling context, events between the passes): the
            # raster, issue-bound at full residency on the large views, is the part a batch cannot share
            pctx = webgs.Context(device=local_rank, flags=webgs.GS_FLAG_PROFILE)
            pscs = [pctx.upload(p, s.count) for s, p in zip(W.BATCH_SCENES, packs)]
            acc = {}
            for rep in range(3):
                for k, (si, _) in enumerate(cams):
                    pctx.forward_device(pscs[si], views[k], rgba8=imgs[k].data_ptr())
                    if rep == 2:
                        for name, v in pctx.timings().items():
                            acc[name] = acc.get(name, 0.0) + v["ms"]
            for sc_ in pscs:
                sc_.close()
            pctx.close()
            res[label]["passes_ms_sum_16_views"] = {k: round(v, 4) for k, v in acc.items()}
            res[label]["raster_share_plain"] = round(acc.get("raster", 0.0) / max(acc.get("TOTAL", 1e-9), 1e-9), 3)
            # end to end: every view's rgba8 image lands in pinned host memory; plain = one synchronous
            # gs_forward per view (one Renderer.execute() per view), batched = one gs_forward_batch
            hosts = [torch.empty(c.width * c.height * 4, dtype=torch.uint8, pin_memory=True) for _, c in cams]
            harr = (_abi.BatchView * len(cams))()
            for k, ((si, c), v) in enumerate(zip(cams, views)):
                harr[k].scene = scs[si].handle
                harr[k].view = v
                harr[k].out = _abi.Image(webgs.GS_MEM_HOST, hosts[k].data_ptr(), None, None, None)

            def plain_e2e():
                for k, (si, _) in enumerate(cams):
                    img = _abi.Image(webgs.GS_MEM_HOST, hosts[k].data_ptr(), None, None, None)
                    ctx._ck(lib.gs_forward(ctx.handle, scs[si].handle, C.byref(views[k]), C.byref(img)))

            def batch_e2e():
                ctx._ck(lib.gs_forward_batch(ctx.handle, harr, len(cams)))

            for fn in (plain_e2e, batch_e2e):
                fn(); fn()
            t0 = time.perf_counter()
            for _ in range(steps):
                plain_e2e()
            t_plain = (time.perf_counter() - t0) / steps
            t0 = time.perf_counter()
            for _ in range(steps):
                batch_e2e()
            t_batch = (time.perf_counter() - t0) / steps
            res[label]["e2e"] = {"plain_ms_per_view": round(t_plain * 1e3 / len(cams), 4),
                                 "batched_ms_per_view": round(t_batch * 1e3 / len(cams), 4),
                                 "batched_over_plain": round(t_plain / t_batch, 3),
                                 "d2h_bytes_per_batch": 4 * pix}
        for s in scs:
            s.close()
        ctx.close()
    res["autotune"] = {"best": tuned, "best_ms_per_batch": round(tuned_ms, 4), "sweep_s": round(tune_s, 1)}
    if cpu:
        threads = os.cpu_count() or 1
        ms = sum(cpu_forward(webgs.view_bytes(v), packs[si], W.BATCH_SCENES[si].count, threads)["ms"]
                 for (si, _), v in zip(cams, views))
        pix = sum(c.width * c.height for _, c in cams)
        res["cpu_baseline"] = {"value": round(pix / ms / 1e3, 4), "unit": "Mpix/s",
                               "ms_per_view": round(ms / len(cams), 2), "cores": threads, "kind": "port",
                               "sample": "every one of the 16 views once, one after another (fp32 frames)"}
    return res


def batched_fwd_bwd(steps, warmup, local_rank, cpu: bool = False) -> dict:
    """One 3M-Gaussian scene (seed 6, 128 clusters, 40^3 box), 8 cameras at 1920x1080: one batched
    forward + 8 losses + one batched backward (gradients of the 8 views summed) vs 8 sequential
    forward + loss + backward calls."""
    import ctypes as C

    import torch

    import webgs
    from webgs import _abi, workloads as W

    lib = webgs.library()
    dev = f"cuda:{local_rank}"
    spec = W.SCENE_3M
    packed = spec.build()
    n = spec.count
    cams = [c for _, c in W.orbit_cameras(8, 77, 18.0, fixed_resolution=(1920, 1080))]
    views = [c.view() for c in cams]
    w, h = 1920, 1080
    ctx = webgs.Context(device=local_rank, flags=webgs.GS_FLAG_DIFFERENTIABLE)
    ts = ctx.upload(webgs.perturb_scene(packed, n, 99, 0.01, 0.02), n)
    targets = [torch.empty(w * h * 3, dtype=torch.float32, device=dev) for _ in views]
    for v, t in zip(views, targets):
        ctx.forward_device(ts, v, rgb=t.data_ptr())
    ctx.synchronize()
    ts.close()
    sc = ctx.upload(packed, n)
    rgbs = [torch.empty(w * h * 3, dtype=torch.float32, device=dev) for _ in views]
    dls = [torch.empty_like(r) for r in rgbs]
    grads = torch.empty(59 * n, dtype=torch.float32, device=dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    arr = (_abi.BatchView * len(views))()
    for k, v in enumerate(views):
        arr[k].scene = sc.handle
        arr[k].view = v
        arr[k].out = _abi.Image(webgs.GS_MEM_DEVICE, None, rgbs[k].data_ptr(), None, None)
    dl_ptrs = (C.c_void_p * len(views))(*[d.data_ptr() for d in dls])

    def loss(k):
        ctx._ck(lib.gs_loss_l1_ssim(ctx.handle, rgbs[k].data_ptr(), targets[k].data_ptr(), w, h, 0.2, None,
                                    dls[k].data_ptr(), webgs.GS_MEM_DEVICE))

    def sequential():
        for k, v in enumerate(views):
            img = _abi.Image(webgs.GS_MEM_DEVICE, None, rgbs[k].data_ptr(), None, None)
            ctx._ck(lib.gs_forward(ctx.handle, sc.handle, C.byref(v), C.byref(img)))
            loss(k)
            ctx._ck(lib.gs_backward(ctx.handle, sc.handle, dls[k].data_ptr(), grads.data_ptr(), webgs.GS_MEM_DEVICE))

    def batched():
        ctx._ck(lib.gs_forward_batch(ctx.handle, arr, len(views)))
        for k in range(len(views)):
            loss(k)
        ctx._ck(lib.gs_backward_batch(ctx.handle, sc.handle, dl_ptrs, len(views), grads.data_ptr(),
                                      webgs.GS_MEM_DEVICE))

    ms_seq = _timed(stream, sequential, steps, warmup)
    ms_bat = _timed(stream, batched, steps, warmup)
    sc.close()
    ctx.close()
    # per-pass times of the eight sequential steps (a profiling context, events between the passes): the
    # rasters and raster backwards, issue-bound and per view, are what a batch cannot share or overlap
    pctx = webgs.Context(device=local_rank, flags=webgs.GS_FLAG_DIFFERENTIABLE | webgs.GS_FLAG_PROFILE)
    psc = pctx.upload(packed, n)
    acc: dict[str, float] = {}
    for rep in range(2):
        for k, v in enumerate(views):
            img = _abi.Image(webgs.GS_MEM_DEVICE, None, rgbs[k].data_ptr(), None, None)
            pctx._ck(lib.gs_forward(pctx.handle, psc.handle, C.byref(v), C.byref(img)))
            pctx._ck(lib.gs_loss_l1_ssim(pctx.handle, rgbs[k].data_ptr(), targets[k].data_ptr(), w, h, 0.2, None,
                                         dls[k].data_ptr(), webgs.GS_MEM_DEVICE))
            pctx._ck(lib.gs_backward(pctx.handle, psc.handle, dls[k].data_ptr(), grads.data_ptr(),
                                     webgs.GS_MEM_DEVICE))
            if rep == 1:
                for name, t in pctx.timings().items():
                    acc[name] = acc.get(name, 0.0) + t["ms"]
    psc.close()
    pctx.close()
    unshared = acc.get("raster", 0.0) + acc.get("raster backward", 0.0)
    res = {"workload": "3M Gaussians (128 clusters, 40^3 box, seed 6), 8 x 1920x1080, L1 + 0.2(1-SSIM)",
           "sequential_ms_per_view": round(ms_seq / len(views), 4), "batched_ms_per_view": round(ms_bat / len(views), 4),
           "batched_over_sequential": round(ms_seq / ms_bat, 3),
           "passes_ms_sum_8_views": {k: round(v, 4) for k, v in acc.items()},
           "raster_and_raster_backward_ms_8_views": round(unshared, 4),
           "overlap_bound_batched_over_sequential": round(ms_seq / unshared, 3) if unshared > 0 else None}
    if cpu:
        import oracle

        threads = os.cpu_count() or 1
        vb = webgs.view_bytes(views[0])
        target_cpu = oracle.forward_f32(vb, webgs.perturb_scene(packed, n, 99, 0.01, 0.02), n, threads=threads,
                                        keys=False)["rgb"]
        c = cpu_forward_backward(vb, packed, n, target_cpu, threads)
        res["cpu_baseline"] = {"value": round(w * h / c["ms"] / 1e3, 4), "unit": "Mpix/s", "ms_per_view": c["ms"],
                               "cores": threads, "kind": "port", "passes_ms": c["passes_ms"],
                               "sample": "view 0 of the 8: fp32 frame, FP64 loss, FP64 adjoint"}
    return res


if __name__ == "__main__":
    main()
