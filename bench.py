#!/usr/bin/env python
"""UHD DIC throughput benchmark (frames/s and subsets/s).

Headline workload (one step = one target frame through the whole per-frame
path): 3840x2160 synthetic speckle reference and a 60-frame sequence deformed
by the plane-strain Kirsch field of a circular hole (radius 300 px at the
centre, masked out of the ROI), scaled to a 2 px peak and ramped linearly
over the 60 frames; affine IC-GN with subset 31, step 8, B-spline
interpolation, 3-level GPU pyramid, integer ZNCC seed search on the first
frame, temporal seeding with velocity prediction afterwards, UOD replace.
The warm-up and timed frames are the last W + K frames of the ramp, so the
last timed frame is at the 2 px peak.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` is measured with inputs resident in HBM (device frames through the
resident C-ABI entry, CUDA events on the launching stream); `e2e` runs the
public register_stream API on host NumPy frames (host->device upload and
device->host readback inside the timed region).  With N > 1 (torchrun) every
rank runs an independent replica on its own GPU and frame sequence.  At
N = 1 the line also carries the two other headline measurements: quadratic
pairs with the reference rebuilt every pair, and learned versus ZNCC-seeded
IC-GN on large-motion frames (`--no-extras` leaves them out).
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (ROOT / "live-dic_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "UHD frames/s & subsets/s; learned- vs ZNCC-seeded IC-GN at equal RMSE"
UNIT = "frames/s"


def parse_args() -> argparse.Namespace:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60, help="timed frames (the frames/s unit is a stream of at least 50)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--width", type=int, default=3840)
    ap.add_argument("--height", type=int, default=2160)
    ap.add_argument("--subset", type=int, default=31)
    ap.add_argument("--stride", type=int, default=8)
    ap.add_argument("--levels", type=int, default=3)
    ap.add_argument("--frames", type=int, default=60, help="length of the load ramp")
    ap.add_argument("--hole", type=float, default=300.0)
    ap.add_argument("--peak", type=float, default=2.0)
    ap.add_argument("--search-radius", type=int, default=4,
                    help="ZNCC integer search radius at the coarsest level (first frame, unseeded windows)")
    ap.add_argument("--lanes", type=int, default=16)
    ap.add_argument("--persistent", action="store_true")
    ap.add_argument("--solver-mode", choices=("exact", "fast", "staged", "staged-wide"), default="exact",
                    help="IC-GN pixel loop: the reference's order, the sliding-window sampler, or the reference's "
                         "order on TMA-staged shared-memory tiles (compact or wide)")
    ap.add_argument("--autotune", action="store_true", help="pick lanes/persistence/pixel loop with the autotuner")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-frames", type=int, default=4, help="timed frames of the CPU pipeline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline workload only (no quadratic-pairs and learned-seeding measurements)")
    ap.add_argument("--workload", choices=("uhd-plate", "batch", "learned", "quadratic-pairs"), default="uhd-plate",
                    help="uhd-plate: the headline UHD sequence; batch: 16 uneven pairs in one batched step; "
                         "learned: learned-seed vs Fourier + pyramid + ZNCC seeding on large-motion UHD frames; "
                         "quadratic-pairs: UHD quadratic pairs with the reference rebuilt every pair")
    ap.add_argument("--train-images", type=int, default=400, help="learned workload: training images")
    ap.add_argument("--train-size", type=int, default=640, help="learned workload: training image side (px)")
    ap.add_argument("--train-steps", type=int, default=8000, help="learned workload: Adam steps (batch 512)")
    ap.add_argument("--lattice", type=int, default=16, help="learned workload: network on every n-th subset")
    ap.add_argument("--plain-radius", type=int, default=17,
                    help="learned workload: ZNCC search radius of the plain path at the coarsest level, centred on "
                         "the global translation (covers the strain residual at the frame corners)")
    ap.add_argument("--learned-steps", type=int, default=20, help="timed frames of the learned-seeding comparison")
    ap.add_argument("--pair-steps", type=int, default=10, help="timed pairs of the quadratic-pairs measurement")
    ap.add_argument("--pairs", type=int, default=16, help="batch workload: number of image pairs")
    return ap.parse_args()


def dist_env() -> tuple[int, int, int]:
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def slowest_ms(local_ms: float, world: int, dist, device) -> float:
    """Maximum of a per-rank duration over all ranks (the job's clock)."""
    if dist is None or world <= 1:
        return local_ms
    import torch

    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(*, steps: int, local_ms: float, world: int, dist, device) -> float:
    """Whole-job frames/s: every replica processed `steps` frames; the job
    took as long as its slowest rank."""
    return world * steps / (slowest_ms(local_ms, world, dist, device) / 1e3)


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int) -> None:
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self) -> None:
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc) -> None:
        if self.proc is not None:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}

    def line(self) -> dict:
        s = self.summary()
        return {"sm_mhz": s["sm_mhz"], "sm_max_mhz": s["sm_max_mhz"], "reasons": s["reasons"]}


def make_workload(args, rank: int, device: str):
    from live_dic_gb300 import synthetic

    seed = 1000 + 17 * rank
    ref, sp = synthetic.reference_image(args.width, args.height, seed=seed, device=device)
    field = synthetic.KirschField(args.width, args.height, args.hole, peak=args.peak)
    mask = synthetic.hole_mask(args.width, args.height, args.hole)
    return ref, sp, field, mask, seed


def ramp_loads(args, count: int) -> list[float]:
    """Load factors of the last `count` frames of the ramp (frame k of a ramp
    of n frames has load k / n; the ramp is lengthened to `count` frames if
    it is shorter)."""
    total = max(args.frames, count)
    return [(total - count + k + 1) / total for k in range(count)]


def render_frames(args, sp, field, seed: int, count: int, device: str):
    import torch

    from live_dic_gb300 import synthetic

    return [torch.from_numpy(synthetic.deformed_image(sp, field.torch_field(load), noise_seed=seed + 100 + k,
                                                      device=device))
            for k, load in enumerate(ramp_loads(args, count))]


def pipeline_oracle(args, levels, rois, temporal, refs):
    """The CPU pipeline of one headline frame: the C oracle's prefilter,
    seeded IC-GN, UOD, pyramid reductions, coarse-to-fine transfers, ZNCC
    search, temporal projection with velocity prediction and history merges
    (oracle/pyramid_oracle.py), with the pyramid's default per-level
    schedule (full_pyramid_backend.py:51-62 of the reference)."""
    from live_dic_gb300.full_pyramid_backend import (_DEFAULT_ITERATION_SCHEDULES, _DEFAULT_TOLERANCES,
                                                     _FOUR_LEVEL_TOLERANCES)
    from oracle.pyramid_oracle import PyramidOracle

    tolerances = (_FOUR_LEVEL_TOLERANCES if args.levels == 4 else _DEFAULT_TOLERANCES)[-args.levels:]
    return PyramidOracle(levels, subset_size=args.subset, subset_stride=args.stride,
                         iterations=_DEFAULT_ITERATION_SCHEDULES[args.levels], tolerances=tolerances,
                         lanes=args.lanes, temporal=True, velocity=True, rois=rois, temporal_links=temporal,
                         search_radius=args.search_radius, reference_levels=refs)


def cpu_pipeline_time(oracle, frames: list[np.ndarray], warmup: int, steps: int) -> float:
    """Seconds per frame of the CPU pipeline over `steps` consecutive frames
    after `warmup` untimed ones (the first frame runs the ZNCC search)."""
    for k in range(warmup):
        oracle.register(frames[k])
    t0 = time.perf_counter()
    for k in range(warmup, warmup + steps):
        oracle.register(frames[k])
    return (time.perf_counter() - t0) / steps


def cpu_sample_text(args, steps: int, arrays: str) -> str:
    cores = os.cpu_count()
    return (f"whole frames through the oracle C port of the per-frame path with {cores} OpenMP threads: "
            f"{args.levels}-level pyramid (integer reductions, FIR prefilters, seeded IC-GN, UOD replace, "
            f"coarse-to-fine transfers), ZNCC search on the first frame, temporal projection with velocity "
            f"prediction and history merges, ROI hole; {steps} consecutive timed frames of the sequence after "
            f"its first; {arrays}; the reference's own GPU path (WGSL via wgpu) cannot run here: no graphics "
            "stack or software renderer on this box")


def run_reference_arm(args) -> None:
    """The reference arm: the path's CPU implementation (the oracle port of
    the reference's per-frame WGSL path, with the float64 restatement of
    its _reference_arrays for the reference preparation) on the host cores,
    on the headline workload, frames through the whole pipeline."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import torch

    from oracle import oracle as oracle_c
    from oracle.pyramid_oracle import float64_levels, roi_tables

    oracle_c.build()
    device = "cuda" if torch.cuda.is_available() else "cpu"
    ref, sp, field, mask, seed = make_workload(args, 0, device)
    count = args.warmup + args.steps
    frames = [f.numpy() for f in render_frames(args, sp, field, seed, count, device)]
    plans, rois, temporal = roi_tables(mask, subset_size=args.subset, subset_stride=args.stride, levels=args.levels)
    t0 = time.perf_counter()
    levels, refs = float64_levels(ref, subset_size=args.subset, subset_stride=args.stride, levels=args.levels,
                                  plans=plans)
    prep_s = time.perf_counter() - t0
    oracle = pipeline_oracle(args, levels, rois, temporal, refs)
    per_frame = cpu_pipeline_time(oracle, frames, args.warmup, args.steps)
    value = 1.0 / per_frame
    cores = os.cpu_count()
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * per_frame,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args),
        "reference_preparation_s": prep_s,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": cpu_sample_text(args, args.steps, "float64 reference preparation of every level")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args) -> dict:
    loads = ramp_loads(args, args.warmup + args.steps)
    return {
        "workload": f"{args.width}x{args.height} plate-with-hole (Kirsch, ROI hole r={args.hole:g} px, peak "
                    f"{args.peak:g} px ramped over {max(args.frames, args.warmup + args.steps)} frames; warm-up and "
                    f"timed frames are its last {args.warmup + args.steps}, loads {loads[0]:.3f}-{loads[-1]:.3f}), "
                    f"affine IC-GN S{args.subset}/s{args.stride}, bspline, {args.levels}-level GPU pyramid, ZNCC "
                    f"search (radius {args.search_radius}) on the first frame, temporal+velocity seeding, UOD "
                    "replace",
        "width": args.width,
        "height": args.height,
        "subset_size": args.subset,
        "subset_stride": args.stride,
        "pyramid_levels": args.levels,
        "seed_search_radius": args.search_radius,
        "lanes_per_subset": args.lanes,
        "persistent": bool(args.persistent),
        "solver_mode": args.solver_mode,
        "parallelism": "replicas",
        "l2": "no flush: per-step working set (finest reference plane 133 MB + coefficient planes + states) exceeds "
              "the 129 MB L2",
    }


def run_batch_workload(args) -> None:
    """16 image pairs of uneven size ({640x480, 1280x720, 1920x1080,
    3840x2160}), subset ({15, 21, 31, 41}, step S/3) and shape function
    (affine with a rectangle ROI holding 0-3 holes of radius 40-200 px, or
    quadratic), random smooth affine-plus-sinusoid fields of 0.5-3 px peak,
    registered as one batched step; compared with one launch per pair."""
    import ctypes

    import torch

    from live_dic_gb300 import ICGNBatch, _native, synthetic

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    pairs = synthetic.uneven_workload(3000 + 17 * rank, count=args.pairs, device=device)
    batch = ICGNBatch(device=local, solver_workgroup_size=args.lanes)
    for job in pairs:
        batch.add(job["reference"], motion_model=job["motion_model"], subset_size=job["subset_size"],
                  subset_stride=job["subset_stride"], roi_mask=job["roi_mask"])
    frames = [torch.from_numpy(j["target"]).to(device) for j in pairs]
    if args.autotune:
        batch.autotune([j["target"] for j in pairs])
    for k, f in enumerate(frames):
        batch.load_device(k, f.data_ptr(), f.stride(0))
    torch.cuda.synchronize()
    stream = torch.cuda.Stream(device=device)
    selected = sum(int(j.roi.selected.sum()) if j.roi is not None else j.subsets for j in batch.jobs)

    def timed(mode: str) -> float:
        batch.set_variant(batch.variant[0], mode, batch.variant[2] if mode != "per-job" else 0)
        for _ in range(args.warmup):
            batch.run_device(stream.cuda_stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            batch.run_device(stream.cuda_stream)
        end.record(stream)
        torch.cuda.synchronize()
        return start.elapsed_time(end)

    best = batch.variant
    seq_ms = timed("per-job")
    class_ms = timed("persistent")
    batch.set_variant(*best)
    with ClockSampler(local) as clocks:
        ms = timed("single")
    batch.set_variant(best[0], "single", best[2])
    solver_ms = statistics.median(batch.run_device(stream.cuda_stream, profile=True) for _ in range(5))
    flops = 0.0
    for k, job in enumerate(batch.jobs):
        state = batch.export_state(k)
        n = 12 if job.motion_model == "quadratic" else 6
        iters = float(state[..., n + 1].sum())
        per_px = 120.0 if job.motion_model == "quadratic" else 90.0
        update = 900.0 if job.motion_model == "quadratic" else 150.0
        flops += (per_px * job.subset_size ** 2 + update) * iters
    ms_max = slowest_ms(ms, world, dist, device)
    value = world * args.steps * selected / (ms_max / 1e3)
    host = [j["target"] for j in pairs]
    for _ in range(2):
        batch.register(host)
    t0 = time.perf_counter()
    for _ in range(max(3, args.steps // 4)):
        results = batch.register(host)
    e2e_s = (time.perf_counter() - t0) / max(3, args.steps // 4)
    if rank != 0:
        batch.close()
        if dist:
            dist.destroy_process_group()
        return
    lib = _native.load()
    peak = ctypes.c_double()
    _native.check(lib.gbdic_fp32_peak_probe(local, ctypes.byref(peak)), b"FP32 probe failed")
    achieved = flops / (solver_ms / 1e3) / 1e12
    accepted = sum(int((r.status >= 1).sum()) for r in results)
    summary = clocks.summary()
    line = {
        "metric": "batched uneven workload subsets/s (one persistent launch over every job vs one launch per pair)",
        "value": value,
        "unit": "subsets/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": f"{args.pairs} pairs: " + ", ".join(
                f"{j.width}x{j.height} {j.motion_model} S{j.subset_size}/s{j.subset_stride}" for j in batch.jobs),
            "subsets_per_step": selected,
            "variant": batch.variant_name,
            "l2": "no flush: the step's coefficient planes, reference planes and states exceed the 129 MB L2",
        },
        "sequential_per_pair_subsets_per_s": world * args.steps * selected / (slowest_ms(seq_ms, world, dist, device) / 1e3),
        "speedup_vs_per_pair": seq_ms / ms if ms > 0 else None,
        "per_class_launches_subsets_per_s": world * args.steps * selected
        / (slowest_ms(class_ms, world, dist, device) / 1e3),
        "accepted_fraction": accepted / max(1, selected),
        "tuning_ms": batch.tuning_ms or None,
        "clocks": {"sm_mhz": summary["sm_mhz"], "sm_max_mhz": summary["sm_max_mhz"], "reasons": summary["reasons"]},
        "gpu_launches": (2 * len(batch.jobs) + 1) * args.steps,
        "roofline": {"bound": "fp32", "kernel": "icgn_batch_any_kernel (every job, shape function per job)",
                     "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s", "frac": achieved / peak.value,
                     "solver_ms": solver_ms, "flops_per_step": flops, "traffic": None},
        "e2e": {"value": selected / e2e_s, "unit": "subsets/s",
                "h2d_bytes_per_step": int(sum(j.width * j.height for j in batch.jobs)),
                "d2h_bytes_per_step": int(sum(j.subsets * (64 if j.motion_model == "quadratic" else 32)
                                              for j in batch.jobs)),
                "api": "ICGNBatch.register (host NumPy frames)"},
    }
    print(json.dumps(line), flush=True)
    batch.close()
    if dist:
        dist.destroy_process_group()




def sinusoid_parameters(cx, cy) -> np.ndarray:
    """u = 2 sin(2 pi x / 400) cos(2 pi y / 600), v = 1.5 cos(2 pi x / 500):
    the 12 quadratic parameters [u, ux, uy, v, vx, vy, uxx, uxy, uyy, vxx,
    vxy, vyy] at (cx, cy)."""
    kx, ky, kv = 2 * math.pi / 400.0, 2 * math.pi / 600.0, 2 * math.pi / 500.0
    sx, cxx, sy, cyy = np.sin(kx * cx), np.cos(kx * cx), np.sin(ky * cy), np.cos(ky * cy)
    sv, cv = np.sin(kv * cx), np.cos(kv * cx)
    zero = np.zeros_like(cx)
    return np.stack([2 * sx * cyy, 2 * kx * cxx * cyy, -2 * ky * sx * sy, 1.5 * cv, -1.5 * kv * sv, zero,
                     -2 * kx * kx * sx * cyy, -2 * kx * ky * cxx * sy, -2 * ky * ky * sx * cyy, -1.5 * kv * kv * cv,
                     zero, zero], -1)


def measure_quadratic(args, local: int, world: int, dist, *, steps: int, warmup: int, cpu_reference: bool) -> dict:
    """UHD pairs, quadratic IC-GN S41/s10 with the reference rebuilt for every
    pair (GPU reference preparation: B-spline, gradients, 12x12 Hessians,
    FP64 Cholesky inverses), sinusoid field; pairs/s with both images
    resident (set_reference_device + register_device per pair, host clock
    around synchronised steps because preparation waits on the device), and
    end to end through set_reference + register on host images."""
    import ctypes

    import torch

    from live_dic_gb300 import ICGNWGPU, _native, synthetic

    device = f"cuda:{local}"
    rank = dist_env()[0]
    S, st = 41, 10
    distinct = 4
    field = synthetic.sinusoid_field()
    refs, tgts = [], []
    for k in range(distinct):
        ref, sp = synthetic.reference_image(args.width, args.height, seed=5000 + 31 * k + 7 * rank, device=device)
        refs.append(ref)
        tgts.append(synthetic.deformed_image(sp, field, noise_seed=6000 + 31 * k + 7 * rank, device=device))
    dev_refs = [torch.from_numpy(r).to(device) for r in refs]
    dev_tgts = [torch.from_numpy(t).to(device) for t in tgts]
    engine = ICGNWGPU(subset_size=S, subset_stride=st, motion_model="quadratic", solver_workgroup_size=args.lanes,
                      device=local)
    gw = 1 + (args.width - S) // st
    gh = 1 + (args.height - S) // st
    state = torch.zeros(gw * gh * 16, dtype=torch.float32, device=device)

    def step(k: int) -> float:
        prep = engine.set_reference_device(dev_refs[k % distinct].data_ptr(), args.width, args.height)
        engine.register_device(dev_tgts[k % distinct].data_ptr(), state.data_ptr())
        return prep

    for k in range(warmup):
        step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    engine.set_profiling(True)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prep_ms = [step(k) for k in range(steps)]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
    profile = engine.read_profile()
    engine.set_profiling(False)
    ms_max = slowest_ms((t1 - t0) * 1e3, world, dist, device)
    value = world * steps / (ms_max / 1e3)
    final = state.view(gh, gw, 16).cpu().numpy()
    cx, cy = synthetic.subset_centres(args.width, args.height, S, st)
    truth = sinusoid_parameters(np.asarray(cx, np.float64), np.asarray(cy, np.float64))
    ok = final[..., 12] >= 1.0
    error = final[..., :12].astype(np.float64) - truth
    rmse = float(np.sqrt(np.mean(np.sum(error[..., (0, 3)][ok] ** 2, axis=1)))) if ok.any() else None
    curvature_rmse = float(np.sqrt(np.mean(error[..., 6:][ok] ** 2))) if ok.any() else None
    for k in range(2):
        engine.set_reference(refs[k % distinct])
        engine.register(tgts[k % distinct])
    e2e_steps = max(3, steps // 2)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        engine.set_reference(refs[k % distinct])
        engine.register(tgts[k % distinct])
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    engine.close()
    lib = _native.load()
    peak = ctypes.c_double()
    _native.check(lib.gbdic_fp32_peak_probe(local, ctypes.byref(peak)), b"FP32 probe failed")
    iters = float(profile["iterations"])
    flops = 120.0 * S * S * iters + 900.0 * iters
    achieved = flops / (profile["solver_ms"] / 1e3) / 1e12 if profile["solver_ms"] > 0 else None
    out = {
        "metric": "UHD quadratic pairs/s with the reference rebuilt every pair",
        "value": value,
        "unit": "pairs/s",
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": ms_max / steps,
        "workload": f"{args.width}x{args.height} speckle pairs ({distinct} distinct, cycled), quadratic IC-GN "
                    f"S{S}/s{st}, bspline, sinusoid field (2 px / 1.5 px), GPU reference preparation every pair",
        "subsets_per_pair": gw * gh,
        "reference_prep_ms_median": float(statistics.median(prep_ms)),
        "displacement_rmse_px": rmse,
        "curvature_rmse": curvature_rmse,
        "accepted_fraction": float(ok.mean()),
        "accuracy_pair": "the last timed pair, against the FP64 sinusoid field",
        "clocks": clocks.line(),
        "gpu_launches": profile["launches"],
        "roofline": {"bound": "fp32", "kernel": f"icgn_kernel<quadratic,bspline,{args.lanes} lanes>",
                     "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": None if achieved is None else achieved / peak.value,
                     "solver_ms_per_pair": profile["solver_ms"] / max(1, steps)},
        "e2e": {"value": 1.0 / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": 2 * args.width * args.height,
                "d2h_bytes_per_step": gw * gh * 16 * 4, "api": "ICGNWGPU.set_reference + register (host NumPy images)"},
    }
    if cpu_reference:
        # The reference prepares a quadratic reference on the CPU in float64
        # (wgpu_backend.py:589-823); its restatement, timed on one UHD image.
        from oracle import reference_prep as rp

        t0 = time.perf_counter()
        rp.reference_arrays(refs[0], motion_model="quadratic", subset_size=S, subset_stride=st)
        out["cpu_reference_preparation"] = {
            "seconds_per_pair": time.perf_counter() - t0, "kind": "port", "cores": 1,
            "sample": "float64 NumPy restatement of _reference_arrays (12x12 Hessians, np.linalg.inv) on one "
                      f"{args.width}x{args.height} reference, S{S}/s{st}: the reference's own CPU preparation path"}
    return out


def measure_learned(args, local: int, *, steps: int, warmup: int) -> dict:
    """UHD frames under rigid translations of 15-30 px plus strain and shear
    within +-2 % about the centre, subset 31 / step 8.  Plain method (the
    reference's large-motion path, with the integer search this project
    adds): the global translation by the same GPU phase correlation the
    learned method uses (a 256-pixel window at the centre of the
    half-resolution frame; the reference's own 1024-pixel window fails its
    acceptance rule under this strain) seeds the coarsest level of a 3-level
    pyramid (Fourier initialization), an integer ZNCC search centred on it
    absorbs the strain residual, IC-GN at every level.  Learned method: the
    seed network (trained here on engine-generated pairs) on a lattice of
    subsets after the same phase correlation, IC-GN at the lattice nodes,
    every subset seeded from the node warps and solved at full resolution
    with the plain path's finest-level settings, failed or low-ZNCC subsets
    reseeded by the ZNCC search and solved again."""
    import torch

    from live_dic_gb300 import ICGNWGPU, ICGNWGPUFullPyramid, learned, synthetic

    device = f"cuda:{local}"
    rank = dist_env()[0]
    t0 = time.perf_counter()
    data = learned.training_pairs(args.train_images, size=args.train_size, seed=11 + rank, device=local)
    gen_s = time.perf_counter() - t0
    net = learned.SeedNet(batch=512, device=local, seed=rank)
    t0 = time.perf_counter()
    losses = learned.train(net, data, steps=args.train_steps, lr=2e-3, log_every=max(1, args.train_steps // 10))
    train_s = time.perf_counter() - t0

    W, H, S, st = args.width, args.height, args.subset, args.stride
    rng = np.random.default_rng(77 + rank)
    ref, sp = synthetic.reference_image(W, H, seed=4242 + rank, device=device)
    c = (0.5 * (W - 1), 0.5 * (H - 1))
    count = warmup + steps
    warps, frames = [], []
    for k in range(count):
        ang, r = rng.uniform(0, 2 * math.pi), rng.uniform(15.0, 30.0)
        t = (r * math.cos(ang), r * math.sin(ang))
        e = rng.uniform(-0.02, 0.02, 3)
        warps.append((t, e))

        def field(X, Y, t=t, e=e):
            return (t[0] + e[0] * (X - c[0]) + e[2] * (Y - c[1]), t[1] + e[2] * (X - c[0]) + e[1] * (Y - c[1]))

        frames.append(torch.from_numpy(synthetic.deformed_image(sp, field, noise_seed=5000 + k, device=device)).to(device))
    cx, cy = synthetic.subset_centres(W, H, S, st)

    def truth_of(k):
        (t, e) = warps[k]
        return np.stack([t[0] + e[0] * (cx - c[0]) + e[2] * (cy - c[1]), t[1] + e[2] * (cx - c[0]) + e[1] * (cy - c[1])], -1)

    def score(state, k, gh, gw):
        s = state.view(gh, gw, 8).cpu().numpy()
        ok = s[..., 6] >= 1
        tr = truth_of(k)
        inside = ((cx - S // 2 + tr[..., 0] >= 4) & (cx + S // 2 + tr[..., 0] <= W - 5) &
                  (cy - S // 2 + tr[..., 1] >= 4) & (cy + S // 2 + tr[..., 1] <= H - 5))
        err = np.linalg.norm(s[..., [0, 3]][ok & inside] - tr[ok & inside], axis=-1)
        good = err <= 0.5
        return (float((ok & inside).sum() / inside.sum()), float(np.sqrt(np.mean(err[good] ** 2))),
                float(1.0 - good.mean()) if err.size else 0.0)

    def run(step_fn, gh, gw, after=None):
        for k in range(warmup):
            step_fn(k)
        torch.cuda.synchronize()
        times, acc = [], []
        for k in range(warmup, count):
            t1 = time.perf_counter()
            state = step_fn(k)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t1)
            acc.append(score(state, k, gh, gw))
            if after is not None:
                after(k)
        return times, acc

    with ClockSampler(local) as clocks:
        plain = ICGNWGPUFullPyramid(pyramid_levels=3, subset_size=S, subset_stride=st, initialization="fourier",
                                    seed_search_radius=args.plain_radius, device=local)
        info = plain.set_reference(ref)
        gw, gh = info.grid
        pstate = torch.zeros(gw * gh * 8, device=device)
        pstream = torch.cuda.Stream(device=device)
        shifter = learned.HalfResolutionShift(W, H, device=local)
        shifter.set_reference_frame(torch.from_numpy(ref).to(device))

        def plain_step(k):
            shift = shifter.shift_of(frames[k], pstream)
            with torch.cuda.stream(pstream):
                plain.register_device(frames[k].data_ptr(), pstate.data_ptr(), stream=pstream.cuda_stream,
                                      translation=shift)
            pstream.synchronize()
            return pstate

        plain_times, plain_acc = run(plain_step, gh, gw)
        fine_iterations, fine_tolerance = plain.iterations_per_level[-1], plain.tolerance_per_level[-1]
        plain.close()
        shifter.close()
        engine = ICGNWGPU(subset_size=S, subset_stride=st, device=local, solver_workgroup_size=args.lanes)
        engine.set_reference(ref, iterations=fine_iterations, tolerance=fine_tolerance)
        seeder = learned.LearnedSeeder(engine, net, step=args.lattice)
        seeder.set_reference_image(ref)
        reseeded = []

        def learned_step(k):
            seeder.register_device(frames[k], counts=False)
            return seeder.state

        def learned_count(k):
            reseeded.append(int(seeder.reseed_count.item()))

        learned_times, learned_acc = run(learned_step, engine.grid_height, engine.grid_width, learned_count)
        # stage breakdown (CUDA events, the direct sequence) over the timed frames
        stage_runs = [seeder.stage_times(frames[k]) for k in range(warmup, warmup + min(steps, 5))]
        stages = {name: float(np.median([r[name] for r in stage_runs])) for name in stage_runs[0]}
        engine.close()
    lt, pt = float(np.mean(learned_times)), float(np.mean(plain_times))
    return {
        "metric": "learned- vs ZNCC-seeded IC-GN frames/s at equal RMSE (UHD, 15-30 px translation + 2 % strain)",
        "value": 1.0 / lt,
        "unit": "frames/s",
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": 1e3 * lt,
        "workload": f"{W}x{H}, S{S}/s{st}, rigid translation 15-30 px + strain and shear within 2 % about the "
                    f"frame centre; learned: network on every {args.lattice}-th subset (GPU phase-correlation "
                    "global shift, 2 passes with an affine consensus), IC-GN at the lattice nodes, interpolated "
                    f"seeds for every subset, IC-GN ({fine_iterations} iterations, tolerance {fine_tolerance:g}, "
                    "as the plain path's finest level), ZNCC reseeding of failures; plain: the same GPU phase "
                    "correlation as global translation (Fourier initialization), 3-level pyramid, ZNCC search "
                    f"radius {args.plain_radius} centred on it at the coarsest level",
        "plain_frames_per_s": 1.0 / pt,
        "speedup_vs_plain": pt / lt,
        "learned_accepted": float(np.mean([a for a, _, _ in learned_acc])),
        "plain_accepted": float(np.mean([a for a, _, _ in plain_acc])),
        "learned_rmse_px": float(np.mean([r for _, r, _ in learned_acc])),
        "plain_rmse_px": float(np.mean([r for _, r, _ in plain_acc])),
        "learned_outliers": float(np.mean([o for _, _, o in learned_acc])),
        "plain_outliers": float(np.mean([o for _, _, o in plain_acc])),
        "accuracy_note": "per timed frame against the FP64 field: accepted = status >= 1 among windows whose "
                         "displaced footprint stays in the frame; rmse over accepted windows within 0.5 px of the "
                         "field, outliers = the accepted rest",
        "reseeded_per_frame": float(np.mean(reseeded)) if reseeded else None,
        "timing": "host clock around each synchronised frame (both methods include their host-side steps)",
        "learned_stage_ms": stages,
        "learned_stage_note": "median CUDA-event time per stage of the direct (not graph-replayed) sequence over "
                              "up to 5 timed frames",
        "train_pairs": int(data.size), "train_images": args.train_images, "train_image_size": args.train_size,
        "train_steps": args.train_steps, "train_batch": 512, "pair_generation_s": gen_s, "training_s": train_s,
        "loss_first_last": [losses[0], losses[-1]],
        "clocks": clocks.line(),
    }


def run_quadratic_workload(args) -> None:
    import torch

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    out = measure_quadratic(args, local, world, dist, steps=args.steps, warmup=args.warmup,
                            cpu_reference=rank == 0 and world == 1 and not args.no_cpu_baseline)
    if rank == 0:
        line = {"metric": out.pop("metric"), "value": out.pop("value"), "unit": out.pop("unit"), "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": out.pop("ms_per_step"),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": out.pop("workload"), "subsets_per_pair": out.pop("subsets_per_pair"),
                           "lanes_per_subset": args.lanes,
                           "l2": "no flush: the reference plane (133 MB), metadata + inverses (55 MB) and "
                                 "coefficient plane exceed the 129 MB L2"},
                **out}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_learned_workload(args) -> None:
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    out = measure_learned(args, local, steps=args.steps, warmup=args.warmup)
    if rank == 0:
        line = {"metric": out.pop("metric"), "value": out.pop("value"), "unit": out.pop("unit"), "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": out.pop("ms_per_step"),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 solver, bf16 network (fp32 accumulate)", "data": "synthetic",
                "config": {"workload": out.pop("workload")}, **out}
        print(json.dumps(line), flush=True)


def main() -> None:
    args = parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.workload == "batch":
        run_batch_workload(args)
        return
    if args.workload == "learned":
        run_learned_workload(args)
        return
    if args.workload == "quadratic-pairs":
        run_quadratic_workload(args)
        return
    import torch

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"

    from live_dic_gb300 import ICGNWGPUFullPyramid, _native

    count = args.warmup + args.steps
    ref, sp, field, mask, seed = make_workload(args, rank, device)
    frames = render_frames(args, sp, field, seed, count, device)
    loads = ramp_loads(args, count)
    dev_frames = torch.stack(frames).to(device).contiguous()
    engine = ICGNWGPUFullPyramid(
        pyramid_levels=args.levels, subset_size=args.subset, subset_stride=args.stride,
        initialization="temporal", temporal_prediction="velocity", seed_search_radius=args.search_radius,
        solver_workgroup_size=args.lanes, device=local, pipeline_slots=2, persistent=args.persistent,
        autotune=args.autotune, solver_mode=args.solver_mode,
    )
    info = engine.set_reference(ref, roi_mask=mask)
    args.lanes, args.persistent, args.solver_mode = engine.solver_workgroup_size, engine._persistent, engine.solver_mode
    gw, gh = info.grid
    state = torch.zeros(gw * gh * 8, dtype=torch.float32, device=device)
    stream = torch.cuda.Stream(device=device)

    # ---------------- resident throughput (value): each frame's sequence replayed as its CUDA graph
    def warm_up():
        with torch.cuda.stream(stream):
            for k in range(args.warmup):
                engine.register_device(dev_frames[k].data_ptr(), state.data_ptr(), stream=stream.cuda_stream)
        torch.cuda.synchronize()

    def timed_frames():
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            for k in range(args.warmup, count):
                engine.register_device(dev_frames[k].data_ptr(), state.data_ptr(), stream=stream.cuda_stream)
            end.record(stream)
        torch.cuda.synchronize()
        return start.elapsed_time(end)

    warm_up()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clocks:
        ms = timed_frames()
    if dist:
        dist.barrier()
    final_state = state.view(gh, gw, 8).cpu().numpy()
    # ---------------- the same sequence again (temporal history reset, so the same work) with
    # CUDA events around every solver launch (launches issued directly): solver time and share
    engine.reset_temporal_state()
    warm_up()
    engine.set_profiling(True)
    ms_profiled = timed_frames()
    profile = engine.read_profile()
    engine.set_profiling(False)
    ms_max = slowest_ms(ms, world, dist, device)
    value = job_throughput(steps=args.steps, local_ms=ms, world=world, dist=dist, device=device)

    # ---------------- accuracy of the last timed frame (the ramp's peak) against the FP64 field
    from live_dic_gb300 import synthetic

    cx, cy = synthetic.subset_centres(args.width, args.height, args.subset, args.stride)
    truth = field.truth(cx, cy, load=loads[-1])
    ok = final_state[..., 6] >= 1.0
    err = final_state[..., [0, 3]][ok] - truth[ok]
    rmse = float(np.sqrt(np.mean(np.sum(err * err, axis=1)))) if ok.any() else None
    selected = int(info.roi.selected.sum()) if info.roi is not None else gw * gh
    peak_px = float(np.hypot(truth[..., 0], truth[..., 1])[info.roi.selected].max()) if info.roi is not None else None

    # ---------------- end to end through the public API (host frames)
    e2e = None
    if not args.no_e2e:
        host_frames = [f.numpy() for f in frames]
        engine.reset_temporal_state()
        for k in range(args.warmup):
            engine.register(host_frames[k])
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        results = list(engine.register_stream(host_frames[args.warmup: count], pipeline_depth=2))
        t1 = time.perf_counter()
        e2e_s = slowest_ms((t1 - t0) * 1e3, world, dist, device) / 1e3
        age = [r.timing["resultAgeWallMs"] for r in results]
        e2e = {
            "value": world * args.steps / e2e_s,
            "unit": UNIT,
            "h2d_bytes_per_step": args.width * args.height,
            "d2h_bytes_per_step": gw * gh * 8 * 4 + 16,
            "api": "ICGNWGPUFullPyramid.register_stream(pipeline_depth=2), host NumPy uint8 frames",
            "result_age_ms_p50": float(np.percentile(age, 50)),
            "result_age_ms_p95": float(np.percentile(age, 95)),
        }

    if rank != 0:
        engine.close()
        if dist:
            dist.destroy_process_group()
        return

    # ---------------- roofline of the dominant kernel (IC-GN solver, FP32 pipe)
    lib = _native.load()
    import ctypes

    peak = ctypes.c_double()
    _native.check(lib.gbdic_fp32_peak_probe(local, ctypes.byref(peak)), b"FP32 probe failed")
    S = args.subset
    flops = (90.0 * S * S + 150.0) * profile["iterations"]
    solver_s = profile["solver_ms"] / 1e3
    achieved = flops / solver_s / 1e12 if solver_s > 0 else None
    launches = max(1, profile["timed_launches"])
    traffic = None
    traffic_file = ROOT / "profiles" / "traffic_per_launch.json"
    if traffic_file.exists():
        traffic = json.loads(traffic_file.read_text()).get("icgn_solver_dram_bytes_per_launch")
    roofline = {
        "bound": "fp32",
        "kernel": {"exact": "icgn_kernel", "fast": "icgn_fast_kernel", "staged": "icgn_staged_kernel",
                   "staged-wide": "icgn_staged_kernel"}[args.solver_mode]
        + f"<affine,bspline,{args.lanes} lanes> (all pyramid levels)",
        "achieved": achieved,
        "peak": peak.value,
        "unit": "TFLOP/s",
        "frac": achieved / peak.value if achieved else None,
        "peak_source": "measured in this run by gbdic_fp32_peak_probe (FMA chains on every SM); "
                       "MEASURED_PEAKS.json has no FP32 figure",
        "traffic": traffic,
        "traffic_source": "profiles/traffic_per_launch.json (one ncu capture of the finest level, scaled by units "
                          "processed to the average launch)",
        "flops_per_launch": flops / launches,
        "avg_launch_ms": profile["solver_ms"] / launches,
        "solver_share_of_step": profile["solver_ms"] / ms_profiled if ms_profiled > 0 else None,
        "profiled_pass_frames_per_s": args.steps / (ms_profiled / 1e3) if ms_profiled > 0 else None,
        "profile_note": "solver time, iterations and share from a second pass over the same frames (temporal "
                        "history reset first, so the same work) with CUDA events around every solver launch; "
                        "value comes from the first pass, each frame replayed as its CUDA graph",
        "iterations_per_subset_frame": profile["iterations"] / (args.steps * selected),
    }

    cpu_baseline = None
    if world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as oracle_c
        from oracle.pyramid_oracle import LevelArrays, roi_tables

        oracle_c.build()
        plans, rois, temporal = roi_tables(mask, subset_size=args.subset, subset_stride=args.stride,
                                           levels=args.levels)
        levels, refs = [], [ref]
        for level in range(args.levels):
            lw, lh = engine.level_grid(level)
            w, h = args.width >> level, args.height >> level
            levels.append(LevelArrays(
                w, h, lw, lh,
                engine.export_level(level, _native.EXPORT_PLANE, np.float32, (h * w * 4,)),
                engine.export_level(level, _native.EXPORT_METADATA, np.float32, (lw * lh * 16,)),
                engine.export_level(level, _native.EXPORT_INVERSE, np.float32, (lw * lh * 36,))))
            if level:
                refs.append(oracle_c.reduce(refs[-1]))
        oracle = pipeline_oracle(args, levels, rois, temporal, refs)
        cpu_steps = max(1, min(args.cpu_frames, count - 1))
        per_frame = cpu_pipeline_time(oracle, [f.numpy() for f in frames], 1, cpu_steps)
        cpu_baseline = {
            "value": 1.0 / per_frame,
            "unit": UNIT,
            "cores": os.cpu_count(),
            "kind": "port",
            "sample": cpu_sample_text(args, cpu_steps, "the reference arrays this run prepared on the GPU"),
        }
    engine.close()

    extras = {}
    if world == 1 and not args.no_extras:
        extras["quadratic_pairs"] = measure_quadratic(args, local, world, dist, steps=args.pair_steps, warmup=3,
                                                      cpu_reference=not args.no_cpu_baseline)
        extras["learned_seeding"] = measure_learned(args, local, steps=args.learned_steps, warmup=3)

    kernels_per_frame = 5 * args.levels + 3
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args),
        "solver_variant": engine.solver,
        "solver_tuning_ms": engine.solver_tuning_ms or None,
        "subsets_per_s": value * selected,
        "subsets_per_frame": selected,
        "displacement_rmse_px": rmse,
        "accuracy_frame": {"load": loads[-1], "peak_displacement_px": peak_px,
                           "note": "the last timed frame, at the ramp's 2 px peak"},
        "accepted_fraction": float(ok.sum() / max(1, selected)),
        "clocks": clocks.line(),
        "gpu_launches": kernels_per_frame * args.steps,
        "roofline": roofline,
        "cpu_baseline": cpu_baseline,
        "e2e": e2e,
        **extras,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
