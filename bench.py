"""Benchmark of the resize path on GB300 (one JSON line on rank 0).

Default workload (the headline case): one plane 1920x1080 u16 holding 10-bit
values, Lanczos a=3, to 3840x2160, horizontal pass then vertical, bit-exact
against zimg's C path; a step is a batch of 64 such frames. The same line
carries `tc_vs_plain`: the wide-filter FP32 workload (8 planes 7680x4320 ->
480x270, Lanczos a=4, ~128 taps per output) timed in the same process on
the tensor-core passes and on the plain FP32 CUDA-core passes, with the
max-abs error of each against the FP64 oracle beside zimg's C path's.
Other workloads (--workload):
  fhd_uhd_u16     the default
  bicubic_f32     3 planes 4:4:4 1920x1080 f32 -> 1280x720, bicubic b=0 c=0.5
  wide_f32        8 planes 7680x4320 f32 Lanczos-4 16x down -> 480x270
  yuv420_batch    64 YUV 4:2:0 u16 frames of mixed sizes, Spline36 -> 1920x1080
  extreme_f32     32 images 64x64 -> 6400x6400 and 6400x6400 -> 64x64 f32 Lanczos-3, plus 32 interlaced
                  1920x1080 frames as fields -> 1280x720
  depth_f32_u8    depth conversion around resize (zimg's DepthConversion): 16 frames of 3 planes
                  3840x2160 f32 -> u8 8-bit limited range, ordered dither
  unresize_f32    zimg's UnresizeConversion (inverse bilinear): 8 frames of 3 planes 1920x1080 f32
                  -> 1280x720

Synthetic content follows each configuration: u16 planes are 16x16 blocks of
uniform 10-bit noise or smooth sinusoids; the bicubic planes uniform [0,1]
plus 32 step rectangles; the wide and extreme planes band-limited noise.

A step is one pass of the resize path over one batch of synthetic frames that
are already resident in HBM (inputs larger than L2 across the batch). `value`
is output Mpixel/s (output samples summed over planes, as zimg's ns/sample,
resizeapp.cpp:119-123). `e2e` is the same metric with each step's input copied
from pinned host memory and its output copied back inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 1024 * 1024


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------ workloads --

def _job(sw, sh, dw, dh, ptype, depth, kind, a=math.nan, b=math.nan, shift_w=0.0, shift_h=0.0, engine="auto"):
    return dict(sw=sw, sh=sh, dw=dw, dh=dh, ptype=ptype, depth=depth, kind=kind, a=a, b=b, shift_w=shift_w,
                shift_h=shift_h, engine=engine)


def workload(name: str, frames: int | None, seed: int):
    """List of jobs for one step (one batch), plus config metadata."""
    rng = np.random.default_rng(seed)
    if name == "bicubic_f32":
        n = frames or 128
        jobs = [dict(_job(1920, 1080, 1280, 720, "float", 32, "bicubic", 0.0, 0.5), content="edges")
                for _ in range(3 * n)]
        cfg = {"workload": "bicubic_f32: 3 planes 4:4:4 1920x1080 f32 -> 1280x720, bicubic b=0 c=0.5",
               "frames_per_step": n, "planes_per_step": 3 * n}
    elif name == "fhd_uhd_u16":
        n = frames or 64
        jobs = [_job(1920, 1080, 3840, 2160, "word", 10, "lanczos", 3) for _ in range(n)]
        cfg = {"workload": "fhd_uhd_u16: 1 plane 1920x1080 u16 10-bit -> 3840x2160, Lanczos a=3, H then V",
               "frames_per_step": n, "planes_per_step": n}
    elif name == "wide_f32":
        n = frames or 8
        jobs = [_job(7680, 4320, 480, 270, "float", 32, "lanczos", 4) for _ in range(n)]
        cfg = {"workload": "wide_f32: 8 planes 7680x4320 f32 -> 480x270, Lanczos a=4 (128 taps)",
               "frames_per_step": 1, "planes_per_step": n}
    elif name == "yuv420_batch":
        n = frames or 64
        sizes = [(720, 480), (1280, 720), (1920, 1080), (3840, 2160)]
        jobs = []
        for _ in range(n):
            sw, sh = sizes[int(rng.integers(0, 4))]
            jobs.append(_job(sw, sh, 1920, 1080, "word", 10, "spline36", shift_w=0.0))
            # chroma 4:2:0 with MPEG-2 (left) siting on both sides: shift = 0.25 - 0.25 / scale
            shw = 0.25 - 0.25 / (960 / (sw // 2))
            for _c in range(2):
                jobs.append(_job(sw // 2, sh // 2, 960, 540, "word", 10, "spline36", shift_w=shw))
        cfg = {"workload": "yuv420_batch: 64 YUV 4:2:0 u16 10-bit frames, sizes drawn from 720x480..3840x2160, "
                           "Spline36 -> 1920x1080 (+2x960x540), MPEG-2 siting",
               "frames_per_step": n, "planes_per_step": 3 * n}
    elif name == "extreme_f32":
        n = frames or 32
        jobs = [_job(64, 64, 6400, 6400, "float", 32, "lanczos", 3) for _ in range(n)]
        jobs += [_job(6400, 6400, 64, 64, "float", 32, "lanczos", 3) for _ in range(n)]
        for _ in range(n):
            jobs.append(_job(1920, 540, 1280, 360, "float", 32, "lanczos", 3, shift_h=-0.125))
            jobs.append(_job(1920, 540, 1280, 360, "float", 32, "lanczos", 3, shift_h=0.125))
        cfg = {"workload": "extreme_f32: 32x(64^2->6400^2) + 32x(6400^2->64^2) + 32 interlaced 1080 frames "
                           "as fields -> 720, Lanczos a=3", "frames_per_step": n, "planes_per_step": len(jobs)}
    else:
        raise SystemExit(f"unknown workload {name}")
    return jobs, cfg


# ------------------------------------------------------------------ replicas --
# Planes and frames are independent: N ranks are N replicas, each with its own
# seeded batch; no data moves between ranks. Only the timing is reduced.

def rank_workload(name: str, frames: int | None, rank: int):
    """This rank's batch: the workload drawn with a per-rank seed."""
    return workload(name, frames, seed=0x5EED0000 + rank)


def _reduce(x: float, op) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x: float) -> float:
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.MAX)


def sum_over_ranks(x: float) -> float:
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.SUM)


def job_bytes(j):
    bpe = 2 if j["ptype"] == "word" else 4
    return (j["sw"] * j["sh"] + j["dw"] * j["dh"]) * bpe


def u16_blocks(rng, h, w, depth):
    """16x16 blocks, each (p = 0.5) uniform noise over the depth's range or a
    smooth sinusoid round(m/2 + m/2 sin(2 pi (x/lx + y/ly) + phase)), lx, ly
    drawn from [64, 512]."""
    maxv = (1 << depth) - 1
    yy, xx = np.mgrid[0:h, 0:w]
    lx, ly, ph = rng.uniform(64, 512), rng.uniform(64, 512), rng.uniform(0, 2 * np.pi)
    wave = np.round(maxv / 2 + maxv / 2 * np.sin(2 * np.pi * (xx / lx + yy / ly) + ph)).astype(np.uint16)
    noise = rng.integers(0, maxv + 1, size=(h, w), dtype=np.uint16)
    pick = rng.random(((h + 15) // 16, (w + 15) // 16)) < 0.5
    mask = np.kron(pick, np.ones((16, 16), bool))[:h, :w]
    return np.where(mask, noise, wave).astype(np.uint16)


def step_edges(rng, h, w, n=32):
    """Uniform [0, 1) plus n axis-aligned rectangles of +-U[0.2, 0.5], not clamped."""
    x = rng.random((h, w), dtype=np.float32)
    for _ in range(n):
        x0, y0 = rng.integers(0, w), rng.integers(0, h)
        x[y0:y0 + rng.integers(8, 300), x0:x0 + rng.integers(8, 300)] += rng.choice([-1, 1]) * rng.uniform(0.2, 0.5)
    return x


def band_limited(rng, h, w, cutoff=0.25):
    """White noise low-passed to <= cutoff cycles per sample, rescaled to [0, 1]."""
    f = np.fft.rfft2(rng.standard_normal((h, w)).astype(np.float32))
    f[np.abs(np.fft.fftfreq(h)) > cutoff, :] = 0
    f[:, np.fft.rfftfreq(w) > cutoff] = 0
    y = np.fft.irfft2(f, s=(h, w))
    return ((y - y.min()) / (y.max() - y.min())).astype(np.float32)


def fill(rng, j):
    """A synthetic plane with the content the job's configuration names."""
    h, w = j["sh"], j["sw"]
    if j["ptype"] == "word":
        return u16_blocks(rng, h, w, j["depth"])
    if j.get("content") == "edges":
        return step_edges(rng, h, w)
    return band_limited(rng, h, w)


# ------------------------------------------------------------------- clocks --

class ClockSampler:
    """nvidia-smi clock / throttle samples while the GPU is busy."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float):
        rows = [r for t, r in self.rows if t0 - 0.15 <= t <= t1 + 0.15] or [r for _, r in self.rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": num(rows[0][1]),
                "reasons": sorted(reasons), "samples": len(rows)}


# ------------------------------------------------------------------- our arm --

def run_ours(args):
    import torch
    import torch.distributed as dist
    import zimg_gb300 as zg
    from zimg_gb300 import build as zbuild

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    zbuild.build()
    zg.load()

    jobs, cfg = rank_workload(args.workload, args.frames, rank)
    if args.engine:
        for j in jobs:
            j["engine"] = args.engine
        cfg["engine"] = args.engine
    rng = np.random.default_rng(1234 + rank)
    # Distinct source planes per job (the batch is the working set), generated on the device from a few seeded
    # host planes so set-up stays quick.
    host_proto = {}
    srcs, dsts, convs = [], [], []
    for j in jobs:
        key = (j["sw"], j["sh"], j["ptype"])
        if key not in host_proto:
            host_proto[key] = [fill(rng, j) for _ in range(2)]
        proto = host_proto[key][len(srcs) % 2]
        t = torch.from_numpy(proto.view(np.int16) if proto.dtype == np.uint16 else proto).cuda()
        srcs.append(t.clone())
        tdt = torch.int16 if j["ptype"] == "word" else torch.float32
        dsts.append(torch.empty((j["dh"], j["dw"]), dtype=tdt, device="cuda"))
        convs.append(zg.ResizeConversion(j["sw"], j["sh"], j["ptype"]).set_depth(j["depth"])
                     .set_filter(j["kind"], j["a"], j["b"]).set_dst_width(j["dw"]).set_dst_height(j["dh"])
                     .set_shift_w(j["shift_w"]).set_shift_h(j["shift_h"]).set_engine(j["engine"]))
    batch = zg.Batch(convs)
    batch.set_io(srcs, dsts)
    if not args.engine and not args.no_autotune:
        # plan choice per job kind by timing on the bound planes (set-up, not timed)
        cfg["autotune_jobs_changed"] = batch.autotune()
    tmp = torch.empty(max(batch.tmp_size, 1), dtype=torch.uint8, device="cuda")
    launches_per_step = batch.launch_count
    stream = torch.cuda.current_stream()

    out_px = sum(j["dw"] * j["dh"] for j in jobs)
    alg_bytes = sum(job_bytes(j) for j in jobs)
    in_bytes = sum(j["sw"] * j["sh"] * (2 if j["ptype"] == "word" else 4) for j in jobs)
    out_bytes = alg_bytes - in_bytes

    step = (lambda: batch.process_graph(tmp)) if args.graph else (lambda: batch.process(tmp))
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    # spin up the clocks before the timed region
    for _ in range(max(args.warmup, 3)):
        step()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t1 = time.time()
    sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1))
    ms_step = ms / args.steps
    # whole-job throughput: every rank's output samples over the slowest rank's time
    value = sum_over_ranks(out_px) * args.steps / (ms / 1e3) / 1e6

    # ---- end to end through the public API with host buffers ----
    e2e = None
    if not args.no_e2e:
        n_e2e = min(len(jobs), args.e2e_planes)
        hsrc = [srcs[i].cpu().pin_memory() for i in range(n_e2e)]
        hdst = [torch.empty(dsts[i].shape, dtype=dsts[i].dtype).pin_memory() for i in range(n_e2e)]
        # the public host-buffer API: chunked, copies overlapping the launches
        pipe = zg.HostPipeline(convs[:n_e2e], chunks=args.e2e_chunks,
                               autotune=not args.engine and not args.no_autotune)
        for _ in range(3):
            pipe.run(hsrc, hdst)
        torch.cuda.synchronize()
        k = max(3, args.steps // 4)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(k):
            pipe.run(hsrc, hdst)
        a1.record(stream)
        a1.synchronize()
        e_ms = a0.elapsed_time(a1) / k
        e_px = sum(jobs[i]["dw"] * jobs[i]["dh"] for i in range(n_e2e))
        h2d = sum(jobs[i]["sw"] * jobs[i]["sh"] * (2 if jobs[i]["ptype"] == "word" else 4) for i in range(n_e2e))
        d2h = sum(jobs[i]["dw"] * jobs[i]["dh"] * (2 if jobs[i]["ptype"] == "word" else 4) for i in range(n_e2e))
        e_ms = max_over_ranks(e_ms)
        e2e = {"value": round(sum_over_ranks(e_px) / (e_ms / 1e3) / 1e6, 3), "unit": "Mpixel/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "planes_per_step": n_e2e}

    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": read_traffic(args.workload), "algorithmic_bytes_per_step": alg_bytes,
                "kernel_launches_per_step": launches_per_step}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(jobs, seconds=args.cpu_seconds)
    tcp = None
    if rank == 0 and args.workload == "fhd_uhd_u16" and not args.no_tc_vs_plain:
        tcp = tc_vs_plain(max(3, args.steps // 2), args.warmup, peak)

    if rank == 0:
        line = {"metric": "out Mpixel/s on 1 GB300 + % HBM roofline", "value": round(value, 3), "unit": "Mpixel/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 5),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u16" if jobs[0]["ptype"] == "word" else "f32", "data": "synthetic (seeded)",
                "config": dict(cfg, l2="inputs larger than L2 (batch working set %.2f GB)" % (alg_bytes / 1e9),
                               parallelism=f"replicas x{world}", graph=bool(args.graph)),
                "impl": "ours", "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "clocks": sampler.summary(t0, t1), "gpu_launches": launches_per_step * args.steps}
        if tcp is not None:
            line["tc_vs_plain"] = tcp
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def tc_vs_plain(steps, warmup, peak):
    """The wide-filter FP32 workload (8 planes 7680x4320 -> 480x270, Lanczos
    a=4) on the tensor-core passes and on the plain FP32 CUDA-core passes, on
    the same resident planes (band-limited noise), each timed with CUDA events
    over `steps` batches; plus the max-abs error of each against the FP64
    oracle on one plane, beside zimg's C path's."""
    import torch
    import zimg_gb300 as zg
    from oracle.oracle import Oracle, build
    jobs, _ = workload("wide_f32", None, seed=0x5EED0003)
    rng = np.random.default_rng(0x5EED0003)
    protos = [fill(rng, jobs[0]) for _ in range(2)]
    srcs = [torch.from_numpy(protos[i % 2]).cuda() for i in range(len(jobs))]
    out_px = sum(j["dw"] * j["dh"] for j in jobs)
    alg_bytes = sum(job_bytes(j) for j in jobs)
    res, first = {}, {}
    stream = torch.cuda.current_stream()
    for engine in ("tensor", "cuda"):
        convs = [zg.ResizeConversion(j["sw"], j["sh"], "float").set_filter(j["kind"], j["a"], j["b"])
                 .set_dst_width(j["dw"]).set_dst_height(j["dh"]).set_engine(engine) for j in jobs]
        dsts = [torch.empty((j["dh"], j["dw"]), dtype=torch.float32, device="cuda") for j in jobs]
        batch = zg.Batch(convs)
        batch.set_io(srcs, dsts)
        tmp = torch.empty(max(batch.tmp_size, 1), dtype=torch.uint8, device="cuda")
        for _ in range(warmup):
            batch.process(tmp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            batch.process(tmp)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        res[engine] = {"value": round(out_px / (ms / 1e3) / 1e6, 3), "ms_per_step": round(ms, 5),
                       "hbm_frac": round(alg_bytes / (ms / 1e3) / 1e9 / peak, 4),
                       "plan": convs[0].create().info["engine"]}
        first[engine] = dsts[0].cpu().numpy().astype(np.float64)
        del batch, dsts, tmp
    build()
    o = Oracle()
    j = jobs[0]
    f64 = o.resize_plane(protos[0], j["dw"], j["dh"], j["kind"], j["a"], mode="f64", nthreads=os.cpu_count() or 1)
    c = o.resize_plane(protos[0], j["dw"], j["dh"], j["kind"], j["a"], mode="c", nthreads=os.cpu_count() or 1)
    err = {k: float(np.max(np.abs(v - f64))) for k, v in first.items()}
    err["c_path"] = float(np.max(np.abs(c.astype(np.float64) - f64)))
    return {"workload": "wide_f32: 8 planes 7680x4320 f32 -> 480x270, Lanczos a=4 (~128 taps), band-limited noise",
            "unit": "Mpixel/s", "tensor": res["tensor"], "plain": res["cuda"],
            "ratio": round(res["tensor"]["value"] / res["cuda"]["value"], 3),
            "max_abs_err_vs_fp64": {"tensor": err["tensor"], "plain": err["cuda"], "zimg_c_path": err["c_path"]},
            "tensor_pipe_active": read_profile_value("wide_f32", "tensor_pipe_active_pct")}


def read_profile_value(workload_name, key):
    """A figure from the committed ncu summary of the workload, if present."""
    p = os.path.join(ROOT, "profiles", f"traffic_{workload_name}.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":", 1)[1])
    return None


def read_traffic(workload_name):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", f"traffic_{workload_name}.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_step:"):
            return int(float(line.split(":", 1)[1]))
    return None


# ---------------------------------------------------------------- CPU side --

class CpuSample:
    """zimg's C path (the oracle's restatement of it, resize_impl.cpp:44-114)
    on every host thread, as zimg runs frames: each conversion planned once
    (filter contexts built), then frame-parallel workers, one per host
    thread, each resizing whole planes one after another, as zimg's test
    application threads frames (graphapp.cpp:355-425). The planes cycle
    through the workload's first few jobs, with the content the configuration
    names. The in-line `cpu_baseline` and the reference arm (`--impl
    reference`) both time this routine, so their rates agree."""

    def __init__(self, jobs, n_jobs=6, seed=99):
        from oracle.oracle import Oracle, build
        build()
        self.o = Oracle()
        self.cores = os.cpu_count() or 1
        rng = np.random.default_rng(seed)
        self.sample = []
        plans = {}
        for j in jobs[: min(len(jobs), n_jobs)]:
            x = fill(rng, j)
            key = tuple(sorted((k, str(v)) for k, v in j.items()))
            if key not in plans:
                plans[key] = self.o.plan(j["sw"], j["sh"], j["dw"], j["dh"], j["kind"], j["a"], j["b"], x.dtype,
                                         j["depth"], j["shift_w"], j["shift_h"])
            self.sample.append((j, x, plans[key]))

    def run(self, planes=None, seconds=None):
        """Every thread resizes planes until `planes` planes are done in all, or
        for about `seconds`; output Mpixel/s, planes, elapsed seconds."""
        import threading
        lock = threading.Lock()
        state = {"next": 0, "px": 0}
        t0 = time.perf_counter()

        def worker():
            outs = {}
            while True:
                with lock:
                    i = state["next"]
                    if (planes is not None and i >= planes) or (planes is None and time.perf_counter() - t0 >= seconds):
                        return
                    state["next"] = i + 1
                j, x, plan = self.sample[i % len(self.sample)]
                out = outs.get(id(plan))
                if out is None:
                    out = outs[id(plan)] = (np.empty(plan.out_shape, x.dtype), np.empty(max(plan.tmp_size, 1), np.uint8))
                plan.run(x, out[0], out[1])
                with lock:
                    state["px"] += j["dw"] * j["dh"]

        ths = [threading.Thread(target=worker) for _ in range(self.cores)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        dt = time.perf_counter() - t0
        return state["px"] / dt / 1e6, state["next"], dt

    def describe(self, n, dt):
        shapes = sorted({f"{j['sw']}x{j['sh']}->{j['dw']}x{j['dh']}" for j, _, _ in self.sample})
        return (f"{n} planes ({', '.join(shapes)}) in {dt:.2f} s, zimg C-path restatement (oracle/zimg_oracle.c), "
                f"conversions planned once, {self.cores} frame-parallel threads")


def cpu_baseline(jobs, seconds=10.0):
    """The in-line CPU baseline: a bounded sample (about `seconds`) of the workload."""
    cs = CpuSample(jobs)
    cs.run(planes=cs.cores)  # warm
    v, n, dt = cs.run(seconds=seconds)
    return {"value": round(v, 3), "unit": "Mpixel/s", "cores": cs.cores, "kind": "port", "sample": cs.describe(n, dt)}


# ------------------------------------------------------- depth conversion --
# zimg's DepthConversion, the filter the graph puts around resize: a 4K
# output stage, 3 planes 3840x2160 f32 (luma + 2 chroma) -> 8-bit limited
# range with ordered dither. Algorithmic bytes: 4 read + 1 written per sample.

def depth_workload(frames: int | None):
    n = frames or 16
    planes = [dict(w=3840, h=2160, plane=p, chroma=p > 0) for _ in range(n) for p in range(3)]
    cfg = {"workload": "depth_f32_u8: 3 planes 3840x2160 f32 -> u8 8-bit limited range, ordered dither "
                       "(zimg DepthConversion)", "frames_per_step": n, "planes_per_step": 3 * n}
    return planes, cfg


def depth_source(rng, pl):
    x = rng.random((pl["h"], pl["w"]), dtype=np.float32)
    return (x - 0.5).astype(np.float32) if pl["chroma"] else x


def run_depth(args):
    import torch
    import zimg_gb300 as zg
    from zimg_gb300 import build as zbuild

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    zbuild.build()
    zg.load()
    planes, cfg = depth_workload(args.frames)
    rng = np.random.default_rng(4321 + rank)
    proto = [depth_source(rng, dict(planes[p], chroma=p > 0)) for p in range(3)]
    convs, srcs, dsts = [], [], []
    for pl in planes:
        convs.append(zg.DepthConversion(pl["w"], pl["h"]).set_pixel_in("float", 32, False, pl["chroma"])
                     .set_pixel_out("byte", 8, False, pl["chroma"]).set_dither_type("ordered")
                     .set_plane(pl["plane"]).create())
        srcs.append(torch.from_numpy(proto[pl["plane"]]).cuda())
        dsts.append(torch.empty((pl["h"], pl["w"]), dtype=torch.uint8, device="cuda"))
    stream = torch.cuda.Stream()
    # planes are independent: four streams forked from and joined to the timed
    # one, so that one launch's last wave overlaps the next plane's first
    nside = 4
    side = [torch.cuda.Stream() for _ in range(nside)]
    torch.cuda.synchronize()

    def step():
        cur = torch.cuda.current_stream()
        for sd in side:
            sd.wait_stream(cur)
        for k, (c, s, d) in enumerate(zip(convs, srcs, dsts)):
            c.process(s, d, stream=side[k % nside])
        for sd in side:
            cur.wait_stream(sd)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        step()
    torch.cuda.synchronize()
    out_px = sum(pl["w"] * pl["h"] for pl in planes)
    alg_bytes = out_px * 5

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    # replay() launches on the current stream: make that the timed one
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            graph.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.time()
        e0.record(stream)
        for _ in range(args.steps):
            graph.replay()
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        t1 = time.time()
    sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1))
    ms_step = ms / args.steps
    value = sum_over_ranks(out_px) * args.steps / (ms / 1e3) / 1e6

    e2e = None
    if not args.no_e2e:
        # the public API with host buffers: pinned planes in, the launch, planes out; each
        # plane on one of the side streams, so that uploads and downloads overlap
        n_e2e = min(len(planes), 12)
        hsrc = [srcs[i].cpu().pin_memory() for i in range(n_e2e)]
        hdst = [torch.empty(dsts[i].shape, dtype=torch.uint8).pin_memory() for i in range(n_e2e)]

        def e2e_step():
            for sd in side:
                sd.wait_stream(stream)
            for i in range(n_e2e):
                sd = side[i % nside]
                with torch.cuda.stream(sd):
                    srcs[i].copy_(hsrc[i], non_blocking=True)
                    convs[i].process(srcs[i], dsts[i], stream=sd)
                    hdst[i].copy_(dsts[i], non_blocking=True)
            for sd in side:
                stream.wait_stream(sd)
        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        k = max(3, args.steps // 4)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(k):
            e2e_step()
        a1.record(stream)
        a1.synchronize()
        e_ms = max_over_ranks(a0.elapsed_time(a1) / k)
        e_px = sum(planes[i]["w"] * planes[i]["h"] for i in range(n_e2e))
        e2e = {"value": round(sum_over_ranks(e_px) / (e_ms / 1e3) / 1e6, 3), "unit": "Mpixel/s",
               "h2d_bytes_per_step": e_px * 4, "d2h_bytes_per_step": e_px, "planes_per_step": n_e2e}

    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": read_traffic(args.workload), "algorithmic_bytes_per_step": alg_bytes,
                "kernel_launches_per_step": len(planes)}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = depth_cpu_baseline(planes, seconds=args.cpu_seconds)
    if rank == 0:
        line = {"metric": "out Mpixel/s on 1 GB300 + % HBM roofline", "value": round(value, 3), "unit": "Mpixel/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 5),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded)",
                "config": dict(cfg, l2="inputs larger than L2 (step working set %.2f GB)" % (alg_bytes / 1e9),
                               parallelism=f"replicas x{world}", graph=True),
                "impl": "ours", "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "clocks": sampler.summary(t0, t1), "gpu_launches": len(planes) * args.steps}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------- unresize --
# zimg's UnresizeConversion (inverse bilinear, FP32): 8 frames of 3 planes
# 1920x1080 -> 1280x720. Algorithmic bytes: the planes read and written once.

def unresize_workload(frames: int | None):
    n = frames or 8
    planes = [dict(w=1920, h=1080, ow=1280, oh=720) for _ in range(3 * n)]
    cfg = {"workload": "unresize_f32: 3 planes 1920x1080 f32 -> 1280x720, inverse bilinear "
                       "(zimg UnresizeConversion)", "frames_per_step": n, "planes_per_step": 3 * n}
    return planes, cfg


def run_unresize(args):
    import torch
    import zimg_gb300 as zg
    from zimg_gb300 import build as zbuild
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    zbuild.build()
    zg.load()
    planes, cfg = unresize_workload(args.frames)
    rng = np.random.default_rng(777 + rank)
    protos = [rng.random((1080, 1920), dtype=np.float32) for _ in range(2)]
    u = zg.UnresizeConversion(1920, 1080).set_orig_width(1280).set_orig_height(720).create()
    srcs = [torch.from_numpy(protos[i % 2]).cuda() for i in range(len(planes))]
    dsts = [torch.empty((720, 1280), dtype=torch.float32, device="cuda") for _ in planes]
    # the planes are independent: each plane is a chain of four launches whose
    # substitutions occupy a few dozen SMs, so eight streams (each with its own
    # scratch), forked from and joined to the timed one, run planes side by side
    nside = 8
    side = [torch.cuda.Stream() for _ in range(nside)]
    tmps = [torch.empty(max(u.tmp_size, 1), dtype=torch.uint8, device="cuda") for _ in side]
    stream = torch.cuda.Stream()

    def step():
        cur = torch.cuda.current_stream()
        for sd in side:
            sd.wait_stream(cur)
        for k, (s_, d_) in enumerate(zip(srcs, dsts)):
            u.process(s_, d_, tmps[k % nside], stream=side[k % nside])
        for sd in side:
            cur.wait_stream(sd)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        step()
    torch.cuda.synchronize()
    out_px = sum(pl["ow"] * pl["oh"] for pl in planes)
    alg_bytes = sum((pl["w"] * pl["h"] + pl["ow"] * pl["oh"]) * 4 for pl in planes)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            graph.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.time()
        e0.record(stream)
        for _ in range(args.steps):
            graph.replay()
        e1.record(stream)
        e1.synchronize()
        t1 = time.time()
    sampler.stop()
    ms_step = max_over_ranks(e0.elapsed_time(e1)) / args.steps
    value = sum_over_ranks(out_px) / (ms_step / 1e3) / 1e6
    e2e = None
    if not args.no_e2e:
        n_e2e = min(len(planes), 6)
        hsrc = [srcs[i].cpu().pin_memory() for i in range(n_e2e)]
        hdst = [torch.empty((720, 1280), dtype=torch.float32).pin_memory() for _ in range(n_e2e)]

        def e2e_step():
            # each plane's upload, conversion and download on its own stream
            cur = stream
            for sd in side:
                sd.wait_stream(cur)
            for i in range(n_e2e):
                sd = side[i % nside]
                with torch.cuda.stream(sd):
                    srcs[i].copy_(hsrc[i], non_blocking=True)
                    u.process(srcs[i], dsts[i], tmps[i % nside], stream=sd)
                    hdst[i].copy_(dsts[i], non_blocking=True)
            for sd in side:
                cur.wait_stream(sd)
        e2e_step()
        torch.cuda.synchronize()
        k = max(3, args.steps // 4)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(k):
            e2e_step()
        a1.record(stream)
        a1.synchronize()
        e_ms = max_over_ranks(a0.elapsed_time(a1) / k)
        e2e = {"value": round(sum_over_ranks(1280 * 720 * n_e2e) / (e_ms / 1e3) / 1e6, 3), "unit": "Mpixel/s",
               "h2d_bytes_per_step": 1920 * 1080 * 4 * n_e2e, "d2h_bytes_per_step": 1280 * 720 * 4 * n_e2e,
               "planes_per_step": n_e2e}
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle.oracle import Oracle, build
        build()
        o = Oracle()
        x = protos[0]
        n, t_0 = 0, time.perf_counter()
        while time.perf_counter() - t_0 < args.cpu_seconds:
            o.unresize_plane(x, 1280, 720)
            n += 1
        dt = time.perf_counter() - t_0
        cpu = {"value": round(n * 1280 * 720 / dt / 1e6, 3), "unit": "Mpixel/s", "cores": 1, "kind": "port",
               "sample": f"{n} planes 1920x1080 -> 1280x720 in {dt:.1f} s, zimg C-path restatement, one thread"}
    if rank == 0:
        line = {"metric": "out Mpixel/s on 1 GB300 + % HBM roofline", "value": round(value, 3), "unit": "Mpixel/s",
                "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(ms_step, 5), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded)",
                "config": dict(cfg, l2="inputs larger than L2 (step working set %.2f GB)" % (alg_bytes / 1e9),
                               parallelism="replicas x1", graph=True),
                "impl": "ours", "e2e": e2e,
                "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                             "traffic": read_traffic(args.workload), "algorithmic_bytes_per_step": alg_bytes,
                             "kernel_launches_per_step": 2 * len(planes)},
                "cpu_baseline": cpu, "clocks": sampler.summary(t0, t1), "gpu_launches": 2 * len(planes) * args.steps}
        print(json.dumps(line), flush=True)


def depth_cpu_baseline(planes, seconds=10.0):
    """The oracle's restatement of zimg's C path (one thread), on a bounded sample."""
    from oracle.oracle import Oracle, PixelFormat, build
    build()
    o = Oracle()
    rng = np.random.default_rng(98)
    xs = [depth_source(rng, dict(planes[p], chroma=p > 0)) for p in range(3)]
    px, n, t0 = 0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        p = n % 3
        o.depth_convert(xs[p], PixelFormat("float", None, False, p > 0), PixelFormat("byte", 8, False, p > 0),
                        "ordered", p)
        px += xs[p].size
        n += 1
    dt = time.perf_counter() - t0
    return {"value": round(px / dt / 1e6, 3), "unit": "Mpixel/s", "cores": 1, "kind": "port",
            "sample": f"{n} planes 3840x2160 in {dt:.1f} s, zimg C-path restatement (oracle/zimg_oracle.c), "
                      f"one thread"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload.startswith("unresize_"):
        from oracle.oracle import Oracle, build
        build()
        o = Oracle()
        planes, cfg = unresize_workload(args.frames)
        x = np.random.default_rng(99).random((1080, 1920), dtype=np.float32)
        for _ in range(args.warmup):
            o.unresize_plane(x, 1280, 720)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            o.unresize_plane(x, 1280, 720)
        dt = time.perf_counter() - t0
        v = round(1280 * 720 * args.steps / dt / 1e6, 3)
        line = {"metric": "out Mpixel/s on 1 GB300 + % HBM roofline", "value": v, "unit": "Mpixel/s",
                "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": cfg,
                "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "Mpixel/s", "cores": 1, "kind": "port",
                                 "sample": "one plane 1920x1080 -> 1280x720 per step, zimg C-path restatement"},
                "e2e": {"value": v, "unit": "Mpixel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.workload.startswith("depth_"):
        planes, cfg = depth_workload(args.frames)
        cpu = depth_cpu_baseline(planes, seconds=max(1.0, 0.5 * args.steps))
        line = {"metric": "out Mpixel/s on 1 GB300 + % HBM roofline", "value": cpu["value"], "unit": "Mpixel/s",
                "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded)", "config": cfg, "impl": "reference", "cpu_baseline": cpu,
                "e2e": {"value": cpu["value"], "unit": "Mpixel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    jobs, cfg = workload(args.workload, args.frames, seed=0x5EED0000)
    cs = CpuSample(jobs)
    cs.run(planes=args.warmup * cs.cores)
    # a step: one plane of the workload per host thread, the threads in parallel
    value, n, dt = cs.run(planes=args.steps * cs.cores)
    line = {"metric": "out Mpixel/s on 1 GB300 + % HBM roofline", "value": round(value, 3), "unit": "Mpixel/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt / n * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16" if jobs[0]["ptype"] == "word" else "f32",
            "data": "synthetic (seeded)", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": "Mpixel/s", "cores": cs.cores, "kind": "port",
                             "sample": "one plane per host thread per step: " + cs.describe(n, dt)},
            "e2e": {"value": round(value, 3), "unit": "Mpixel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="fhd_uhd_u16")
    ap.add_argument("--frames", type=int, default=None)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--graph", action="store_true", default=None,
                    help="replay the batch from a CUDA graph (the default for yuv420_batch)")
    ap.add_argument("--no-graph", dest="graph", action="store_false")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--e2e-planes", type=int, default=48)
    ap.add_argument("--e2e-chunks", type=int, default=8, help="sub-batches of the host pipeline")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-tc-vs-plain", action="store_true",
                    help="skip the wide-filter tensor-core vs plain FP32 comparison of the default line")
    ap.add_argument("--engine", default=None, choices=["auto", "cuda", "tensor"],
                    help="override every job's engine (cuda = the plain CUDA-core kernels)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.graph is None:
        args.graph = args.workload == "yuv420_batch"
    if args.impl == "reference":
        run_reference(args)
    elif args.workload.startswith("depth_"):
        run_depth(args)
    elif args.workload.startswith("unresize_"):
        run_unresize(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
