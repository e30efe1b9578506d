"""Benchmark of the moment-image hot path on one GB300.

Headline workload (the target configuration, in the precision form): a 1024^3 float32 mixing-layer grid (256
seeded Fourier modes, 5 % seeded noise, built on the device), a 2048 x 2048 perspective view, 0.5-voxel steps, 64
trigonometric moments, compaction, prediction coding with the default warp and 10-bit codes (table [16, 10 x 63]).
A step is one full pass over the image with the volume resident in HBM, in the flow of the reference's
--generate / --reconstruct (main.cpp:278-391):
    generate_grid_kernel -> scan / compaction -> prediction encode + coding parameters -> quantize and pack the
    codes -> unpack and dequantize -> Lagrange multipliers from the prediction-coded moments -> re-march
The arithmetic is the precision form: Kahan-compensated FP32 moment sums and the MESE preparation's FP64 steps in
float-float arithmetic.  The metric is million rays (pixels) per second of that pass.

The JSON line also carries:
  plain_fp32 / precision_form_fp64   the same pass in the reference's plain FP32 arithmetic / with native FP64 MESE;
  stages        every stage of the step for each form (ms, its own Mrays/s, compulsory bytes against the HBM peak);
  e2e           the same pass through the drop-in host API (mraygb_generate, mraygb_quantize_prediction_coding,
                mraygb_dequantize_prediction_coding, mraygb_reconstruct) on pinned host buffers: the volume goes up
                every step (the reference uploads it in every generate_device call) and every intermediate image
                crosses the host boundary as the reference's API passes it -- every copy inside the timed region;
  roofline      the dominant kernel (generate) against the measured HBM copy bandwidth (compulsory bytes), with its
                FP32 rate against the measured FP32 FMA roof beside it (the binding roof of this method);
  cpu_baseline  the reference's own CPU code (its sources compiled with its Release flags) on a row sample of the
                same workload, OpenMP on all host cores;
  mixing512     the 512^3 / 1024^2 / m = 64 workload (no prediction coding) in the three forms;
  errors_vs_fp64  max / RMS errors of moments, transmittance and RGBA against the FP64 oracle of the same method on
                sampled pixels of both workloads;
and the differentiation form, SPH particles, uncertainty rendering, single scattering and the file format.

--impl reference times the reference's own CPU code (or, where its sources are not staged, the oracle's
restatement) on bounded row samples of the headline workload.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mrays/s moment gen+MESE recon (fwd, fwd+adjoint) vs plain FP32 at ≤1e-4 err"
UNIT = "Mrays/s"

# the workload of the sections that are not the headline: 512^3 mixing layer (64 modes), 1024^2, m = 64
SECTION_SIZE, SECTION_IMAGE, SECTION_M = 512, 1024, 64


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=1024, help="volume edge (voxels)")
    ap.add_argument("--image", type=int, default=2048, help="image edge (pixels)")
    ap.add_argument("--moments", type=int, default=64)
    ap.add_argument("--modes", type=int, default=256, help="Fourier modes of the mixing layer")
    ap.add_argument("--bits", type=int, default=10, help="code bits of moments 1..m-1")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the sections beside the headline (512^3 workload, differentiation form, SPH, ...)")
    ap.add_argument("--sph-particles", type=int, default=16_000_000)
    ap.add_argument("--worker", default="cuda", choices=["cuda", "shim"], help=argparse.SUPPRESS)
    ap.add_argument("--section", default="all",
                    choices=["all", "headline", "mixing512", "diff", "sph", "uncertainty", "scattering", "file",
                             "errors", "refcuda", "refcuda-worker"],
                    help="run only that part and print its JSON (headline: the headline's timed forms only, for "
                         "profiling)")
    return ap.parse_args()


class Headline:
    """The headline workload: view, parameters, quantization table; the volume is built on the device."""

    def __init__(self, args):
        from mray_gb300 import workloads as W

        self.n, self.modes = args.size, args.modes
        self.width = self.height = args.image
        self.num_moments = args.moments
        self.gen, self.rec, self.camera, self.tf1d, self.tf_step = W.mixing_layer_setup(self.n, self.width,
                                                                                        self.height,
                                                                                        prediction_coding=True)
        self.gen.quantization_bits = args.bits
        self.domain_min, self.domain_max = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
        self.table = np.array([16] + [args.bits] * (self.num_moments - 1), dtype=np.uint8)[:self.num_moments]
        self.name = (f"mixing_layer{self.n}^3_{self.width}x{self.height}_m{self.num_moments}_persp_prediction_coded_"
                     f"{args.bits}bit")
        self.volume = None  # host copy, when one is needed

    def volume_device(self):
        from mray_gb300 import workloads as W

        return W.mixing_layer_device(self.n, modes=self.modes, seed=21)

    def config(self):
        return {"workload": self.name,
                "volume": f"{self.n}^3 float32 mixing layer ({self.modes} seeded Fourier modes, 5% seeded noise)",
                "image": f"{self.width}x{self.height} perspective", "num_moments": self.num_moments,
                "step": "0.5 voxel", "codes": f"prediction coded, default warp, table [16, {self.table[-1]} x "
                                              f"{self.num_moments - 1}]"}


def section_workload():
    from mray_gb300 import workloads as W

    return W.mixing_layer_workload(n=SECTION_SIZE, width=SECTION_IMAGE, height=SECTION_IMAGE, num_moments=SECTION_M,
                                   modes=64, seed=21,
                                   name=f"mixing_layer{SECTION_SIZE}^3_{SECTION_IMAGE}x{SECTION_IMAGE}_m{SECTION_M}_persp")


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(values, dist=None, device="cpu"):
    """Max over ranks of a list of floats (the timing of the slowest replica); identity without a process group."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def samples_per_ray(wl) -> np.ndarray:
    """Samples of each ray (first, regular steps while t + step < t_far, last at t_far), counted from the per-ray
    box intersection with the reference's float formulas."""
    W, H = wl.width, wl.height
    cam = wl.camera
    x = np.arange(W, dtype=np.float32)[None, :]
    y = np.arange(H, dtype=np.float32)[:, None]
    nx = (x / np.float32(W)) * np.float32(2) - np.float32(1)
    ny = (y / np.float32(H)) * np.float32(2) - np.float32(1)
    nx, ny = np.broadcast_arrays(nx, ny)
    m = np.array([[cam.transform[i][j] for j in range(4)] for i in range(4)], dtype=np.float32)
    if cam.orthographic:
        o = [np.float32(cam.position[i]) + nx * np.float32(cam.right[i]) + ny * np.float32(cam.up[i])
             for i in range(3)]
        d = [np.full_like(nx, np.float32(cam.dir[i])) for i in range(3)]
    else:
        xs = nx * np.float32(cam.aspect) * np.float32(cam.scale)
        ys = ny * np.float32(cam.scale)
        v = [m[i, 0] * xs + m[i, 1] * ys + m[i, 2] * np.float32(-1) for i in range(3)]
        inv = np.float32(1) / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
        o = [np.full_like(nx, np.float32(cam.position[i])) for i in range(3)]
        d = [v[i] * inv for i in range(3)]
    with np.errstate(divide="ignore", invalid="ignore"):
        tmin, tmax = [], []
        for i in range(3):
            inv = np.float32(1) / d[i]
            tb = inv * (np.float32(wl.domain_min[i]) - o[i])
            tt = inv * (np.float32(wl.domain_max[i]) - o[i])
            tmin.append(np.minimum(tt, tb))
            tmax.append(np.maximum(tt, tb))
        tn = np.maximum(np.maximum(tmin[0], tmin[1]), tmin[2])
        tf = np.minimum(np.minimum(tmax[0], tmax[1]), tmax[2])
    tn = np.maximum(tn, np.float32(cam.znear))
    hit = (tf > tn) & (tf > 0)
    s = np.where(hit, np.ceil((tf - tn) / np.float32(wl.gen.step_size)) + 1, 0)
    return s.astype(np.int64)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}

# ------------------------------------------------------------------------------------------------------------
# The reference's CPU path on row samples (the CPU baseline and the reference arm)
# ------------------------------------------------------------------------------------------------------------

def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    return O


class CpuReference:
    """The reference's CPU path over row samples of the headline workload: generate (per-pixel moments and
    counts) -> compaction -> prediction encode -> quantize / dequantize with the table -> Lagrange multipliers ->
    re-march.  The reference's own code (its sources compiled with its Release flags, oracle/Makefile refrel) where
    its sources are staged; otherwise the oracle's FP32 restatement of it."""

    def __init__(self, hl):
        self.O = _oracle()
        self.hl = hl
        self.row = self.O.preintegrate(hl.tf1d, hl.tf_step)
        self.threads = os.cpu_count() or 1
        try:
            self.pipe = self.O.RefPipeline(hl.volume, hl.domain_min, hl.domain_max)
            self.kind = "reference"
        except OSError:
            self.pipe = None
            self.kind = "port"

    def describe(self):
        if self.kind == "reference":
            return ("the reference's own CPU code (its sources, -O3 -DNDEBUG -fopenmp -D_GLIBCXX_PARALLEL): "
                    "generate_ray + compute_num_moments, compact, prediction_encode, quantize / dequantize, "
                    f"prepare_moments + reconstruct_ray, OpenMP {self.threads} threads over the sampled pixels")
        return (f"the oracle's FP32 restatement of the reference's CPU path (oracle/mray_oracle.c), OpenMP "
                f"{self.threads} threads")

    def run(self, row0, row_step):
        """The sampled rows y = row0 (mod row_step); returns (rays, seconds)."""
        hl, O = self.hl, self.O
        W, H, m = hl.width, hl.height, hl.num_moments
        t0 = time.perf_counter()
        if self.pipe is not None:
            rays = self.pipe.rows(hl.camera, hl.gen, hl.rec, W, H, m, row0, row_step, hl.table, self.row)
        else:
            rows = (row0, H, row_step)
            mo, b, c = O.generate_moments(hl.camera, hl.gen, hl.volume, hl.domain_min, hl.domain_max, W, H, m, "f32",
                                          nthreads=self.threads, rows=rows)
            idx, data = O.compact(c, mo)
            enc, cp = O.prediction_encode(W, H, m, idx, data, hl.gen.coding_warp, hl.gen.bias, nthreads=self.threads)
            packed = O.quantize_prediction_coding(W, H, m, idx, enc, hl.table)
            deq = O.dequantize_prediction_coding(W, H, m, idx, hl.table, packed, enc.size)
            pm = O.prepare_moments(W, H, m, idx, deq, True, hl.gen.coding_warp, cp, hl.rec.bias, "f32",
                                   nthreads=self.threads, rows=rows)
            O.reconstruct(hl.camera, hl.rec, W, H, m, hl.domain_min, hl.domain_max, idx, pm, b, self.row, "f32",
                          nthreads=self.threads, rows=rows)
            rays = len(range(row0, H, row_step)) * W
        return rays, time.perf_counter() - t0

    def rows_for(self, seconds):
        """Rows per sample for about `seconds` of work: calibrated on one and on four rows (a call also has a cost
        that does not grow with the rows, e.g. the reference's allocation of the whole moment image)."""
        H = self.hl.height
        _, t1 = self.run(H // 2, H)
        _, t4 = self.run(H // 8, H // 4)
        per_row = max((t4 - t1) / 3.0, t1 / 8.0, 1e-6)
        fixed = max(0.0, t1 - per_row)
        return int(max(1, min(H, round((seconds - fixed) / per_row))))

    def close(self):
        if self.pipe is not None:
            self.pipe.close()


def cpu_baseline(hl, target_s):
    ref = CpuReference(hl)
    try:
        nrows = ref.rows_for(target_s)
        step = max(1, hl.height // nrows)
        rays, dt = ref.run(0, step)
    finally:
        ref.close()
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": ref.threads, "kind": ref.kind,
            "sample": f"rows y = 0 mod {step} of the {hl.width}x{hl.height} image ({rays} rays, {dt:.1f} s): "
                      f"{ref.describe()}"}


def host_volume(hl):
    """The headline volume in host memory (built on the device, copied back)."""
    import torch

    vol = hl.volume_device()
    host = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True)
    host.copy_(vol)
    del vol
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return host


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return
    import torch

    torch.cuda.set_device(local)
    hl = Headline(args)
    hl.volume = host_volume(hl).numpy()
    ref = CpuReference(hl)
    # each step a bounded sample of the image (about two seconds of host work), rows rotating between steps
    nrows = ref.rows_for(2.0)
    row_step = max(1, hl.height // nrows)
    for i in range(args.warmup):
        ref.run(i % row_step, row_step)
    times, rays_total = [], 0
    for i in range(args.steps):
        rays, dt = ref.run((args.warmup + i) % row_step, row_step)
        times.append(dt)
        rays_total += rays
    ref.close()
    total = sum(times)
    value = rays_total / total / 1e6
    sample = (f"every {row_step}th row per step ({hl.width * len(range(0, hl.height, row_step))} rays), rows rotating; "
              f"{ref.describe()}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {**hl.config(), "sample_per_step": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ref.threads, "kind": ref.kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------------------
# GPU path: the headline
# ------------------------------------------------------------------------------------------------------------

def read_profile_traffic(name):
    """DRAM bytes per launch of a kernel from a committed ncu summary (its 'traffic_bytes_per_launch:' line)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].strip().split()[0])
    except OSError:
        pass
    return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class HeadlinePass:
    """The headline's device buffers and its step on one context (volume resident)."""

    def __init__(self, ctx, stream, hl):
        import torch

        self.ctx, self.stream, self.hl = ctx, stream, hl
        W, H, m = hl.width, hl.height, hl.num_moments
        P = W * H
        self.P = P
        dev = dict(device="cuda")
        self.d_mo = torch.empty(P * m, dtype=torch.float32, **dev)
        self.d_b = torch.empty(2 * P, dtype=torch.int16, **dev)
        self.d_c = torch.empty(P, dtype=torch.int32, **dev)
        self.d_idx = torch.empty(P + 1, dtype=torch.int32, **dev)
        self.d_cm = torch.empty(P * m, dtype=torch.float32, **dev)
        self.d_cp = torch.empty(2 * m, dtype=torch.int16, **dev)
        self.d_codes = torch.empty(P * (int(hl.table.astype(np.int64).sum()) + 7) // 8 + 64, dtype=torch.uint8, **dev)
        self.d_pm = torch.empty(P * m, dtype=torch.float32, **dev)
        self.d_rgba = torch.empty(P * 4, dtype=torch.float32, **dev)
        self.sizes = {}

    def step(self, ev=None):
        """generate -> compaction -> encode -> quantize -> dequantize -> prepare -> reconstruct; events (if given)
        at the stage boundaries: 0 start, 1 after generate, 2 after compaction, 3 after the coding stages, 4 after
        prepare, 5 end."""
        ctx, hl, s = self.ctx, self.hl, self.stream
        W, H, m = hl.width, hl.height, hl.num_moments
        rec = (lambda i: ev[i].record(s)) if ev is not None else (lambda i: None)
        rec(0)
        ctx.stage_generate_moments(hl.camera, hl.gen, W, H, m, self.d_mo, self.d_b, self.d_c)
        rec(1)
        total = ctx.stage_compact(W, H, m, self.d_c, self.d_mo, self.d_idx, self.d_cm)
        rec(2)
        ctx.stage_prediction_encode(W, H, m, self.d_idx, self.d_cm, total, hl.gen.coding_warp, hl.gen.bias, self.d_cp)
        nbytes = ctx.stage_quantize_prediction_coding(W, H, m, self.d_idx, self.d_cm, hl.table, self.d_codes)
        ctx.stage_dequantize_prediction_coding(W, H, m, self.d_idx, hl.table, self.d_codes, nbytes, self.d_cm)
        rec(3)
        ctx.stage_prepare_moments(W, H, m, self.d_idx, self.d_cm, self.d_pm, prediction_code=1,
                                  coding_warp=hl.gen.coding_warp, coding_params=self.d_cp, bias=hl.rec.bias)
        rec(4)
        ctx.stage_reconstruct(hl.camera, hl.rec, W, H, m, hl.domain_min, hl.domain_max, self.d_idx, self.d_pm,
                              self.d_b, self.d_rgba)
        rec(5)
        self.sizes = {"moments": total, "code_bytes": nbytes}


STAGES = ("generate", "compaction", "coding", "prepare", "reconstruct")


def timed_forms(args, ctx, stream, hp, dist, forms, sampler_form, device_index):
    """Warm-up, then exactly `steps` timed steps per form (events on the launching stream around each step, L2
    flushed by a 256 MiB write between steps outside the events).  Returns per form: total ms, per-stage mean ms,
    launches in the timed region, wall seconds; and the clocks sampled during the form `sampler_form`."""
    import torch

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    res, clocks = {}, None
    for name, prec, steps in forms:
        ctx.precision = prec
        for _ in range(args.warmup):
            hp.step()
        ctx.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(steps)]
        sampler = None
        if name == sampler_form:
            sampler = ClockSampler(device_index)
            sampler.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = ctx.kernel_launches
        t0 = time.perf_counter()
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
            hp.step(evs[i])
        ctx.synchronize()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if sampler is not None:
            clocks = sampler.stop()
        step_ms = [e[0].elapsed_time(e[5]) for e in evs]
        stage = {k: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in evs) for i, k in enumerate(STAGES)}
        res[name] = {"total_ms": sum(step_ms), "steps": steps, "stage_ms": stage,
                     "launches": ctx.kernel_launches - launches0, "wall_s": wall}
    del flush
    return res, clocks


def run_ours(args):
    import torch

    import mray_gb300 as M

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    hl = Headline(args)
    W, H, m = hl.width, hl.height, hl.num_moments
    P = W * H
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    vol = hl.volume_device()
    torch.cuda.synchronize()
    ctx.upload_grid(vol, hl.domain_min, hl.domain_max)
    if args.section != "headline" and (not args.no_e2e or (rank == 0 and not (args.no_cpu_baseline and
                                                                             args.no_extras))):
        hl.volume = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True)
        hl.volume.copy_(vol)
    del vol
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    tf = M.preintegrate(hl.tf1d, hl.tf_step)
    ctx.upload_tf(tf.table)
    fp32_roof = max(ctx.measure_fp32_rate() for _ in range(3))
    hp = HeadlinePass(ctx, stream, hl)

    forms = [("plain_fp32", M.PRECISION_FP32, args.steps),
             ("precision_form_fp64", M.PRECISION_COMPENSATED_FP64_MESE, max(1, min(args.steps, 3))),
             ("precision_form", M.PRECISION_COMPENSATED_FF_MESE, args.steps)]
    res, clocks = timed_forms(args, ctx, stream, hp, dist, forms, "precision_form", local)
    maxed = reduce_max([res[f]["total_ms"] / res[f]["steps"] for f, _, _ in forms], dist, "cuda")
    per_step = dict(zip([f for f, _, _ in forms], maxed))
    head = res["precision_form"]
    value = world * P / (per_step["precision_form"] * 1e-3) / 1e6

    # roofline of the dominant kernel (generate, Kahan instance): compulsory bytes and method FLOPs per launch
    gen_ms = head["stage_ms"]["generate"]
    spr = samples_per_ray(hl)
    total_samples = int(spr.sum())
    gen_bytes = hl.n ** 3 * 4 + P * (m * 4 + 4 + 4)
    gen_flops = total_samples * (4 * (m - 1) + 24)
    peaks = measured_peaks()
    hbm_peak, peak_src = peaks.get("hbm_gbs"), "measured (MEASURED_PEAKS.json hbm_gbs)"
    if hbm_peak is None:
        hbm_peak, peak_src = 6800.0, "fallback"
    achieved = gen_bytes / (gen_ms * 1e-3) / 1e9
    fp32_achieved = gen_flops / (gen_ms * 1e-3) / 1e12
    roofline = {"bound": "hbm", "kernel": "generate_grid_kernel<16,true>", "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak, "peak_source": peak_src,
                "traffic": read_profile_traffic(f"generate_grid_kernel_mixing{hl.n}_{W}sq_m{m}.md"),
                "algorithmic_bytes_per_launch": gen_bytes, "kernel_ms": gen_ms,
                "fp32": {"achieved_tflops": fp32_achieved, "peak_tflops": fp32_roof, "frac": fp32_achieved / fp32_roof,
                         "flops_per_launch": gen_flops, "samples_per_launch": total_samples,
                         "peak_source": "measured: FMA-chain kernel on every SM (mraygb_measure_fp32_rate), best of 3",
                         "note": "method FLOPs 4(m-1)+24 per sample (FMA = 2); FP32 issue is the binding roof of "
                                 "this method (no step is a dense contraction; compulsory bytes are ~0.5 B/FLOP)"}}

    nd, nbytes = int(hp.sizes["moments"]), int(hp.sizes["code_bytes"])
    stage_bytes = {"generate": gen_bytes, "compaction": P * m * 4 + nd * 4 + 8 * P,
                   "coding": 3 * nd * 4 + 2 * nbytes + 8 * P, "prepare": 2 * nd * 4 + 4 * P,
                   "reconstruct": nd * 4 + 24 * P}
    stages = {name: {k: {"ms": v, "Mrays_s": P / (v * 1e-3) / 1e6,
                         "hbm_frac": stage_bytes[k] / (v * 1e-3) / 1e9 / hbm_peak,
                         "algorithmic_bytes": stage_bytes[k]} for k, v in res[name]["stage_ms"].items()}
              for name, _, _ in forms}

    if args.section == "headline":
        if rank == 0:
            print(json.dumps({"headline": {"value": value, "stages": stages, "roofline": roofline}}), flush=True)
        ctx.close()
        return

    e2e = None if args.no_e2e else run_e2e(args, ctx, hl, dist)
    cpu = None
    extras = {}
    if rank == 0:
        hl_vol = hl.volume
        hl.volume = hl_vol.numpy() if hl_vol is not None else None
        if not args.no_cpu_baseline and hl.volume is not None:
            cpu = cpu_baseline(hl, args.cpu_seconds)
        if not args.no_extras:
            extras["large_extras"] = run_large_extras(args, ctx, stream, hp)
            extras["errors_vs_fp64"] = precision_errors(args, local, hl)
    hp = None
    ctx.close()
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_extras:
        extras["reference_cuda"] = run_reference_cuda(args)
        extras["mixing512"] = run_mixing512(args, local)
        extras["differentiation_form"] = run_diff(args, local)
        extras["sph"] = run_sph(args, local)
        extras["uncertainty"] = run_uncertainty(args, local)
        extras["single_scattering"] = run_scattering(args, local)
        extras["file_format"] = run_file_format(args, local)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": per_step["precision_form"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+ff", "data": "synthetic",
                "config": {**hl.config(),
                           "precision": "Kahan-compensated FP32 moment sums; MESE preparation with its FP64 steps "
                                        "(exponential moments / decode recursion, Levinson) in float-float "
                                        "arithmetic (~48 significant bits), FP32 correlation tail",
                           "step_stages": "generate, compaction, prediction encode + quantize + dequantize, "
                                          "Lagrange multipliers, re-march",
                           "l2": f"inputs larger than L2 (volume {hl.n ** 3 * 4 / 2 ** 30:.0f} GiB) and a 256 MiB "
                                 "buffer written between timed steps",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "plain_fp32": {"value": world * P / (per_step["plain_fp32"] * 1e-3) / 1e6, "unit": UNIT,
                               "ms_per_step": per_step["plain_fp32"]},
                "precision_form_fp64": {"value": world * P / (per_step["precision_form_fp64"] * 1e-3) / 1e6,
                                        "unit": UNIT, "ms_per_step": per_step["precision_form_fp64"],
                                        "steps": res["precision_form_fp64"]["steps"],
                                        "note": "the same pass with the MESE preparation in native FP64"},
                "precision_over_plain": per_step["plain_fp32"] / per_step["precision_form"],
                "e2e": e2e, "gpu_launches": head["launches"], "roofline": roofline, "stages": stages,
                "cpu_baseline": cpu, "clocks": clocks, "wall_s_timed": head["wall_s"], **extras}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_e2e(args, ctx, hl, dist):
    """The drop-in host API on pinned host buffers: every copy inside the timed region."""
    import torch

    import mray_gb300 as M

    W, H, m = hl.width, hl.height, hl.num_moments
    P = W * H
    ctx.precision = M.PRECISION_COMPENSATED_FF_MESE
    vol_np = hl.volume.numpy() if hasattr(hl.volume, "numpy") else hl.volume
    # the step's input in pinned host memory, as the reference's pinned-host uploads would hold it
    vol_pinned = torch.empty(vol_np.shape, dtype=torch.float32).pin_memory().numpy()
    vol_pinned[...] = vol_np
    grid = M.RegularGrid(vol_pinned, hl.domain_min, hl.domain_max)
    mi = M.MomentImageHost(W, H, m, True, True)
    data_full = torch.empty(P * m, dtype=torch.float32).pin_memory().numpy()
    mi.index = torch.empty(P + 1, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    mi.bounds = torch.empty(2 * P, dtype=torch.int16).pin_memory().numpy().view(np.uint16).reshape(P, 2)
    img = M.ColorImageHost(W, H)
    img.rgba_float = torch.empty(P * 4, dtype=torch.float32).pin_memory().numpy().reshape(H, W, 4)
    img.rgba = torch.empty(P * 4, dtype=torch.uint8).pin_memory().numpy().reshape(H, W, 4)
    tf = M.preintegrate(hl.tf1d, hl.tf_step)
    codes = torch.empty(P * m * 2 + 8, dtype=torch.uint8).pin_memory().numpy()  # 16 bits per value at most
    sizes = {}

    def one():
        mi.data = data_full
        M.generate(hl.camera, grid, mi, hl.gen, context=ctx)
        qs = M.quantize_prediction_coding(mi, hl.table, context=ctx, out=codes)
        M.dequantize_prediction_coding(mi, hl.table, qs, context=ctx)
        M.reconstruct(hl.camera, mi, tf, img, hl.rec, context=ctx)
        sizes["moments"], sizes["codes"] = mi.data.size, qs.size

    for _ in range(max(3, args.warmup)):
        one()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    (dt,) = reduce_max([dt], dist, "cuda")

    # where the time of a step goes: three more steps (after the timed ones) with a clock around each call, the
    # volume upload apart from the generate call (each call returns with its copies done)
    phases = {"upload_grid": [], "generate": [], "quantize": [], "dequantize": [], "reconstruct": []}
    for _ in range(3):
        t = time.perf_counter()
        mi.data = data_full
        ctx.upload_grid(grid.data, grid.domain_min, grid.domain_max)
        t, t_prev = time.perf_counter(), t
        phases["upload_grid"].append(t - t_prev)
        ctx.generate(hl.camera, hl.gen, W, H, m, out=mi)
        t, t_prev = time.perf_counter(), t
        phases["generate"].append(t - t_prev)
        qs = M.quantize_prediction_coding(mi, hl.table, context=ctx, out=codes)
        t, t_prev = time.perf_counter(), t
        phases["quantize"].append(t - t_prev)
        M.dequantize_prediction_coding(mi, hl.table, qs, context=ctx)
        t, t_prev = time.perf_counter(), t
        phases["dequantize"].append(t - t_prev)
        M.reconstruct(hl.camera, mi, tf, img, hl.rec, context=ctx)
        t, t_prev = time.perf_counter(), t
        phases["reconstruct"].append(t - t_prev)
    world = dist.get_world_size() if dist else 1
    nd, nq = 4 * sizes["moments"], sizes["codes"]
    idx_b, cp_b = 4 * (P + 1), 4 * (m - 1)
    # generate: volume up; data, index, bounds, coding parameters down.  quantize: index, data up; codes down.
    # dequantize: index, codes up; data down.  reconstruct: index, data, bounds, coding parameters, TF row up; RGBA
    # (float and u8) down.
    h2d = hl.n ** 3 * 4 + (idx_b + nd) + (idx_b + nq) + (idx_b + nd + 4 * P + cp_b + 256 * 16)
    d2h = (nd + idx_b + 4 * P + cp_b) + nq + nd + (16 * P + 4 * P)
    return {"value": world * P * args.steps / dt / 1e6, "unit": UNIT, "ms_per_step": 1e3 * dt / args.steps,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": args.steps,
            "phases_ms": {k: [round(1e3 * x, 2) for x in v] for k, v in phases.items()},
            "path": "mraygb_upload_grid + mraygb_generate, mraygb_quantize_prediction_coding, "
                    "mraygb_dequantize_prediction_coding, mraygb_upload_tf + mraygb_reconstruct on pinned host "
                    "buffers (the drop-in seams of generate_device / reconstruct_device and the reference's "
                    "quantizer), precision form"}


def run_large_extras(args, ctx, stream, hp):
    """On the headline workload: the data-dependent quantization table of the generate flow, and the
    differentiation form's forward and forward + transfer-function adjoint (no compaction) with their ratio."""
    import torch

    import mray_gb300 as M

    hl = hp.hl
    W, H, m = hl.width, hl.height, hl.num_moments
    P = W * H
    steps = max(1, min(args.steps, 3))
    ctx.precision = M.PRECISION_FP32
    out = {"workload": hl.name}
    out["quantization_table"] = quantization_table_timing(args, ctx, hl.camera, hl.gen, W, H, m, hp.d_mo, hp.d_b,
                                                          hp.d_c, hp.d_idx, hp.d_cm, hp.d_cp, steps)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        ev = _events(steps)
        for e in ev:
            e[0].record(stream)
            fn()
            e[1].record(stream)
        ctx.synchronize()
        return statistics.mean(e[0].elapsed_time(e[1]) for e in ev)

    gen = M.GenerationParameters(**{f: getattr(hl.gen, f) for f, _ in hl.gen._fields_})
    gen.compact_image, gen.prediction_coding = 0, 0
    b4 = torch.empty(P * 4, device="cuda")
    rgba = torch.empty((H, W, 4), device="cuda")
    tab = torch.from_numpy(M.preintegrate(hl.tf1d, hl.tf_step).table).cuda()
    gtab = torch.zeros((256, 4), device="cuda")

    def fwd():
        ctx.diff_forward(hl.camera, gen, hl.rec, W, H, m, tab, hp.d_mo, b4, hp.d_pm, rgba)

    def fwd_bwd():
        fwd()
        with torch.cuda.stream(stream):
            g = 2.0 * rgba
            gtab.zero_()
        ctx.diff_backward(hl.camera, gen, hl.rec, W, H, m, tab, hp.d_mo, b4, hp.d_pm, rgba, g, gtab, None)

    f_ms = timed(fwd)
    fb_ms = timed(fwd_bwd)
    out["diff_fwd"] = {"value": P / (f_ms * 1e-3) / 1e6, "unit": UNIT, "ms": f_ms}
    out["diff_fwd_tf_adjoint"] = {"value": P / (fb_ms * 1e-3) / 1e6, "unit": UNIT, "ms": fb_ms}
    out["diff_fwd_tf_adjoint_over_fwd"] = fb_ms / f_ms
    return out


def refcuda_worker(args, local):
    """One build of the reference's harness (`cuda`: its own CUDA path; `shim`: the drop-in shim over libmraygb.so)
    timing the reference's generate() + reconstruct() calls on the headline workload without quantization."""
    import ctypes as C

    import torch

    from mray_gb300.types import Camera, GenerationParameters, ReconstructionParameters

    O = _oracle()  # puts oracle/ on the path
    from stage_reference import reference_src

    src = reference_src()
    if src is None:
        return {"unavailable": "the reference's sources are not staged (baseline/_ref/src)"}
    target = {"cuda": "refcuda", "shim": "shim"}[args.worker]
    jobs = str(min(16, os.cpu_count() or 1))
    r = subprocess.run(["make", "-s", "-j", jobs, "-C", os.path.join(ROOT, "oracle"), target, f"REF={src}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        return {"unavailable": f"make {target} failed: {r.stderr[-300:]}"}
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", f"libmrayref_{args.worker}.so"))
    if args.worker == "cuda":
        L.ref_init_device(0)  # main.cpp:566
    L.ref_grid_create.restype = C.c_void_p
    L.ref_grid_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.ref_time_flow.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(GenerationParameters),
                                C.POINTER(ReconstructionParameters), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    hl = Headline(args)
    vol = host_volume(hl).numpy()
    dmn = np.asarray(hl.domain_min, np.float32)
    dmx = np.asarray(hl.domain_max, np.float32)
    grid = L.ref_grid_create(vol.ctypes.data, hl.n, hl.n, hl.n, dmn.ctypes.data, dmx.ctypes.data)
    del vol
    row = O.preintegrate(hl.tf1d, hl.tf_step)
    steps = max(1, min(args.steps, 3))
    ms = np.zeros(2 * steps, np.float64)
    rgba8 = np.zeros((hl.height, hl.width, 4), np.uint8)
    size = C.c_uint64()
    L.ref_time_flow(grid, C.byref(hl.camera), C.byref(hl.gen), C.byref(hl.rec), hl.width, hl.height, hl.num_moments,
                    row.ctypes.data, 1, steps, ms.ctypes.data, rgba8.ctypes.data, C.byref(size))
    gen_ms, rec_ms = float(ms[0::2].mean()), float(ms[1::2].mean())
    return {"generate_ms": gen_ms, "reconstruct_ms": rec_ms, "steps": steps, "moment_floats": int(size.value),
            "Mrays_s": hl.width * hl.height / ((gen_ms + rec_ms) * 1e-3) / 1e6, "rgba8_mean": float(rgba8.mean())}


def run_reference_cuda(args):
    """The reference's own CUDA path, compiled from its sources for sm_103a, against ours on the same GPU: the
    reference's generate() and reconstruct() (moment_raymarcher.cpp:168-183, 329-337) on the headline workload
    (prediction coded, no quantization step), timed with a wall clock around each call, through the same harness
    entry point linked once with the reference's moment_raymarcher.cu and once with the drop-in shim over
    libmraygb.so (plain FP32 form).  Both calls include what the reference's calls do: the volume upload, the image
    copies each way and the device work.  Each build runs in a process of its own."""
    out = {"workload": Headline(args).name + " (generate -> reconstruct, no quantization)",
           "timing": "wall clock around each generate() / reconstruct() call, mean of the timed calls after one "
                     "warm-up; the volume goes up in every generate() as the reference's generate_device does",
           "reference_build": "the reference's .cu files with cmake/cuda.cmake:8's flags (fast math) for sm_103a, "
                              "-std=c++17 (CUDA 13's Thrust needs it)"}
    for which in ("cuda", "shim"):
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--section", "refcuda-worker", "--worker", which,
               "--steps", str(args.steps), "--size", str(args.size), "--image", str(args.image), "--moments",
               str(args.moments), "--modes", str(args.modes), "--bits", str(args.bits)]
        env = dict(os.environ)
        if which == "shim":
            env["MRAYGB_SHIM_TIMING"] = "1"
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, env=env)
            res = json.loads(r.stdout.strip().splitlines()[-1])["refcuda-worker"] if r.returncode == 0 else \
                {"unavailable": f"exit {r.returncode}: {r.stderr[-400:]}"}
            if which == "shim" and r.returncode == 0:
                # mean of each phase the shim reports, over the calls after the warm-up
                phases = {}
                for ln in r.stderr.splitlines():
                    if ln.startswith("mraygb shim "):
                        head, ms = ln[len("mraygb shim "):].rsplit(" ", 2)[0], float(ln.rsplit(" ", 2)[1])
                        phases.setdefault(head, []).append(ms)
                res["shim_phases_ms"] = {k: statistics.mean(v[1:] if len(v) > 1 else v) for k, v in phases.items()}
        except (subprocess.TimeoutExpired, ValueError, IndexError, KeyError) as e:
            res = {"unavailable": f"{type(e).__name__}: {str(e)[-300:]}"}
        out["reference_cuda" if which == "cuda" else "ours_through_shim"] = res
    ref, ours = out.get("reference_cuda", {}), out.get("ours_through_shim", {})
    if "Mrays_s" in ref and "Mrays_s" in ours:
        out["ours_over_reference"] = ours["Mrays_s"] / ref["Mrays_s"]
        out["generate_speedup"] = ref["generate_ms"] / ours["generate_ms"]
        out["reconstruct_speedup"] = ref["reconstruct_ms"] / ours["reconstruct_ms"]
    return out


def run_mixing512(args, local):
    """The 512^3 mixing layer (64 modes), 1024^2 perspective view, m = 64, compaction without prediction coding:
    generate -> compaction -> Lagrange multipliers -> re-march in the three arithmetic forms."""
    import torch

    import mray_gb300 as M

    wl = section_workload()
    W, H, m = wl.width, wl.height, wl.num_moments
    P = W * H
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_grid(torch.from_numpy(wl.volume).cuda(), wl.domain_min, wl.domain_max)
    ctx.upload_tf(M.preintegrate(wl.tf1d, wl.tf_step).table)
    d_mo = torch.empty(P * m, device="cuda")
    d_b = torch.empty(2 * P, dtype=torch.int16, device="cuda")
    d_c = torch.empty(P, dtype=torch.int32, device="cuda")
    d_idx = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    d_cm = torch.empty(P * m, device="cuda")
    d_pm = torch.empty(P * m, device="cuda")
    d_rgba = torch.empty(P * 4, device="cuda")

    def step(ev=None):
        rec = (lambda i: ev[i].record(stream)) if ev is not None else (lambda i: None)
        rec(0)
        ctx.stage_generate_moments(wl.camera, wl.gen, W, H, m, d_mo, d_b, d_c)
        rec(1)
        ctx.stage_compact(W, H, m, d_c, d_mo, d_idx, d_cm)
        rec(2)
        ctx.stage_prepare_moments(W, H, m, d_idx, d_cm, d_pm, bias=wl.rec.bias)
        rec(3)
        ctx.stage_reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_rgba)
        rec(4)

    out = {"workload": wl.name + " (compaction, no prediction coding)"}
    for name, prec in (("plain_fp32", M.PRECISION_FP32), ("precision_form_fp64", M.PRECISION_COMPENSATED_FP64_MESE),
                       ("precision_form", M.PRECISION_COMPENSATED_FF_MESE)):
        ctx.precision = prec
        for _ in range(args.warmup):
            step()
        ctx.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]
        for e in evs:
            step(e)
        ctx.synchronize()
        ms = statistics.mean(e[0].elapsed_time(e[4]) for e in evs)
        st = {k: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in evs)
              for i, k in enumerate(("generate", "compaction", "prepare", "reconstruct"))}
        out[name] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms, "stage_ms": st}
    out["precision_over_plain"] = out["plain_fp32"]["ms"] / out["precision_form"]["ms"]
    ctx.close()
    return out


def precision_errors(args, local, hl=None):
    """Max and RMS errors of the moments, the transmittance and the RGBA of the three arithmetic forms against the FP64
    oracle of the same method (the same sample positions; the path without quantization), on 2048 sampled pixels (16
    rows x 128 columns) of each workload: the 512^3 / 1024^2 one and the headline's 1024^3 / 2048^2 one.  Pixels whose
    u16 density bounds differ from the FP64 ones are left out (the bounds are truncated, so a last-bit difference of a
    sampled extreme can move them one step)."""
    import torch

    import mray_gb300 as M

    O = _oracle()
    cases = [("mixing512", section_workload())]
    if hl is not None and hl.volume is not None:
        cases.append(("headline", hl))
    out = {"sample": "rows y = 0 mod H/16, columns x = 0 mod W/128 (2048 pixels per workload); FP64 oracle of the "
                     "same method (oracle/mray_oracle.c, double, exact constants), uncompressed path (generate -> "
                     "compaction -> multipliers -> re-march)",
           "moment_error": "max_j |m_j - m_j(FP64)| / max(|m_0(FP64)|, 1e-3) per pixel",
           "rgba_error": "max over channels |c - c(FP64)| per pixel"}
    for key, wl in cases:
        Wd, H, m = wl.width, wl.height, wl.num_moments
        P = Wd * H
        gen = M.GenerationParameters(**{f: getattr(wl.gen, f) for f, _ in wl.gen._fields_})
        gen.prediction_coding = 0
        rows, cols = (0, H, H // 16), (0, Wd, Wd // 128)
        vol = wl.volume.numpy() if hasattr(wl.volume, "numpy") else wl.volume
        mo64, b64, c64 = O.generate_moments(wl.camera, gen, vol, wl.domain_min, wl.domain_max, Wd, H, m, "f64",
                                            rows=rows, cols=cols)
        idx64, _ = O.compact(c64, mo64.astype(np.float32))
        cnt = c64.reshape(-1)
        data64 = mo64.reshape(-1, m)[cnt > 0].reshape(-1)
        pm64 = O.prepare_moments(Wd, H, m, idx64, data64, False, 1, None, wl.rec.bias, "f64", rows=rows)
        tf = O.preintegrate(wl.tf1d, wl.tf_step)
        rgba64 = O.reconstruct(wl.camera, wl.rec, Wd, H, m, wl.domain_min, wl.domain_max, idx64, pm64, b64, tf, "f64",
                               rows=rows)
        ctx = M.Context(local)
        ctx.set_stream(torch.cuda.current_stream())
        ctx.upload_grid(torch.from_numpy(np.ascontiguousarray(vol)).cuda(), wl.domain_min, wl.domain_max)
        ctx.upload_tf(tf)
        sel = np.zeros((H, Wd), bool)
        sel[rows[0]:rows[1]:rows[2], cols[0]:cols[1]:cols[2]] = True
        res = {"workload": wl.name}
        d_mo = torch.zeros(P * m, device="cuda")
        d_b = torch.zeros(2 * P, dtype=torch.int16, device="cuda")
        d_c = torch.zeros(P, dtype=torch.int32, device="cuda")
        d_idx = torch.zeros(P + 1, dtype=torch.int32, device="cuda")
        d_cm = torch.zeros(P * m, device="cuda")
        d_pm = torch.zeros(P * m, device="cuda")
        d_rgba = torch.zeros(P * 4, device="cuda")
        for name, prec in (("plain_fp32", M.PRECISION_FP32), ("precision_form_fp64", M.PRECISION_COMPENSATED_FP64_MESE),
                           ("precision_form", M.PRECISION_COMPENSATED_FF_MESE)):
            ctx.precision = prec
            ctx.stage_generate_moments(wl.camera, gen, Wd, H, m, d_mo, d_b, d_c)
            ctx.stage_compact(Wd, H, m, d_c, d_mo, d_idx, d_cm)
            ctx.stage_prepare_moments(Wd, H, m, d_idx, d_cm, d_pm, bias=wl.rec.bias)
            ctx.stage_reconstruct(wl.camera, wl.rec, Wd, H, m, wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_rgba)
            ctx.synchronize()
            mo = d_mo.cpu().numpy().reshape(H, Wd, m)[sel].astype(np.float64)
            b = d_b.cpu().numpy().view(np.uint16).reshape(H, Wd, 2)[sel]
            rgba = d_rgba.cpu().numpy().reshape(H, Wd, 4)[sel].astype(np.float64)
            ok = (c64[sel] > 0) & np.all(b == b64[sel], axis=-1)
            ref_m, ref_rgba = mo64[sel], rgba64[sel]
            me = (np.abs(mo - ref_m).max(axis=-1) / np.maximum(np.abs(ref_m[..., 0]), 1e-3))[ok]
            te = np.abs(rgba[..., 3] - ref_rgba[..., 3])[ok]
            re = np.abs(rgba - ref_rgba).max(axis=-1)[ok]
            res[name] = {"pixels": int(ok.sum()),
                         "moments": {"max": float(me.max()), "rms": float(np.sqrt((me ** 2).mean()))},
                         "transmittance": {"max": float(te.max()), "rms": float(np.sqrt((te ** 2).mean()))},
                         "rgba": {"max": float(re.max()), "rms": float(np.sqrt((re ** 2).mean())),
                                  "frac_above_1e-4": float((re > 1e-4).mean()),
                                  "frac_above_1e-3": float((re > 1e-3).mean())}}
        ctx.close()
        del d_mo, d_cm, d_pm
        torch.cuda.empty_cache()
        out[key] = res
    return out


# ------------------------------------------------------------------------------------------------------------
# sections beside the headline
# ------------------------------------------------------------------------------------------------------------

def _events(n):
    import torch

    return [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(n)]


def run_diff(args, local):
    """The differentiation form on its configuration (256^3 Marschner-Lobb, 512^2 orthographic, 31 moments, L2 loss
    against a target rendered with the perturbed transfer function): forward, and forward + adjoint to the
    transfer-function row and all voxel densities."""
    import torch

    import mray_gb300 as M
    from mray_gb300 import workloads as W

    wl, target_tf = W.diff_workload(n=256, width=512, height=512, num_moments=31)
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P = Wd * H
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    vol = torch.from_numpy(wl.volume).cuda()
    ctx.upload_grid(vol, wl.domain_min, wl.domain_max)
    tab = torch.from_numpy(M.preintegrate(wl.tf1d, wl.tf_step).table).cuda()
    ttab = torch.from_numpy(M.preintegrate(target_tf, wl.tf_step).table).cuda()
    mo = torch.empty(P * m, device="cuda")
    b4 = torch.empty(P * 4, device="cuda")
    pm = torch.empty(P * m, device="cuda")
    rgba = torch.empty((H, Wd, 4), device="cuda")
    target = torch.empty((H, Wd, 4), device="cuda")
    gtab = torch.zeros((256, 4), device="cuda")
    gvol = torch.zeros_like(vol)
    torch.cuda.synchronize()
    ctx.diff_forward(wl.camera, wl.gen, wl.rec, Wd, H, m, ttab, mo, b4, pm, target)

    def fwd():
        ctx.diff_forward(wl.camera, wl.gen, wl.rec, Wd, H, m, tab, mo, b4, pm, rgba)

    def fwd_bwd():
        fwd()
        with torch.cuda.stream(stream):
            g = 2.0 * (rgba - target)
            gtab.zero_()
            gvol.zero_()
        ctx.diff_backward(wl.camera, wl.gen, wl.rec, Wd, H, m, tab, mo, b4, pm, rgba, g, gtab, gvol)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        ev = _events(args.steps)
        l0 = ctx.kernel_launches
        for e in ev:
            e[0].record(stream)
            fn()
            e[1].record(stream)
        ctx.synchronize()
        return statistics.mean(e[0].elapsed_time(e[1]) for e in ev), (ctx.kernel_launches - l0) // args.steps

    f_ms, f_l = timed(fwd)
    fb_ms, fb_l = timed(fwd_bwd)
    loss = float(((rgba - target) ** 2).sum())
    # the same with the transfer-function row linear in the front density (the reference's GPU sampling)
    ctx.diff_tf_sampling = M.DIFF_TF_LINEAR
    ctx.diff_forward(wl.camera, wl.gen, wl.rec, Wd, H, m, ttab, mo, b4, pm, target)
    lf_ms, _ = timed(fwd)
    lfb_ms, _ = timed(fwd_bwd)
    ctx.diff_tf_sampling = M.DIFF_TF_BSPLINE
    ctx.close()
    return {"workload": f"{wl.name}_ortho (256^3 Marschner-Lobb, 512x512, m=31, no compaction, ert 1)",
            "fwd": {"value": P / (f_ms * 1e-3) / 1e6, "unit": UNIT, "ms": f_ms, "gpu_launches_per_step": f_l},
            "fwd_adjoint": {"value": P / (fb_ms * 1e-3) / 1e6, "unit": UNIT, "ms": fb_ms,
                            "gpu_launches_per_step": fb_l,
                            "gradients": "transfer-function row (256 x RGBA) and all 256^3 voxel densities"},
            "fwd_adjoint_over_fwd": fb_ms / f_ms, "loss": loss,
            "linear_tf_row": {"fwd_ms": lf_ms, "fwd_adjoint_ms": lfb_ms, "fwd_adjoint_over_fwd": lfb_ms / lf_ms,
                              "note": "the transfer-function row linear in the front density (mraygb_set_diff_tf_"
                                      "sampling), target re-rendered with it"},
            "note": "forward = generate (no compaction) + FP32 Lagrange multipliers + re-march (exact atan, "
                    "B-spline transfer function); adjoint = re-march adjoint + preparation adjoint + generation "
                    "adjoint; the L2 residual and the gradient zeroing (torch) are inside the timed region"}


def run_sph(args, local):
    """SPH particles (16M: 70 % uniform, 30 % in 200 Gaussian clusters, LogNormal values, one smoothing length
    h = 1/256 so that the grid has 256^3 cells), 1024^2 perspective view, 64 moments: the device grid build, the
    forward pass in both arithmetic forms, and the differentiation form with its transfer-function adjoint."""
    import torch

    import mray_gb300 as M
    from mray_gb300 import workloads as W

    n = args.sph_particles
    wl = W.sph_cluster_workload(n=n, width=SECTION_IMAGE, height=SECTION_IMAGE, num_moments=SECTION_M, seed=31)
    x, y, z, v, h = wl.x, wl.y, wl.z, wl.v, wl.h
    dmin, dmax = wl.domain_min, wl.domain_max
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P = Wd * H
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    xs = [torch.from_numpy(a).cuda() for a in (x, y, z, v)]
    torch.cuda.synchronize()
    up = []
    for _ in range(3):
        e = _events(1)[0]
        e[0].record(stream)
        ctx.upload_particles(*xs, h, dmin, dmax)
        e[1].record(stream)
        ctx.synchronize()
        up.append(e[0].elapsed_time(e[1]))
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    ctx.upload_tf(tf.table)
    d_mo = torch.empty(P * m, device="cuda")
    d_b = torch.empty(2 * P, dtype=torch.int16, device="cuda")
    d_c = torch.empty(P, dtype=torch.int32, device="cuda")
    d_idx = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    d_cm = torch.empty(P * m, device="cuda")
    d_pm = torch.empty(P * m, device="cuda")
    d_rgba = torch.empty(P * 4, device="cuda")

    def fwd():
        ctx.stage_generate_moments(wl.camera, wl.gen, Wd, H, m, d_mo, d_b, d_c)
        ctx.stage_compact(Wd, H, m, d_c, d_mo, d_idx, d_cm)
        ctx.stage_prepare_moments(Wd, H, m, d_idx, d_cm, d_pm, bias=wl.rec.bias)
        ctx.stage_reconstruct(wl.camera, wl.rec, Wd, H, m, dmin, dmax, d_idx, d_pm, d_b, d_rgba)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        ev = _events(args.steps)
        for e in ev:
            e[0].record(stream)
            fn()
            e[1].record(stream)
        ctx.synchronize()
        return statistics.mean(e[0].elapsed_time(e[1]) for e in ev)

    out = {"workload": f"sph{n}_h1/256_{Wd}x{H}_m{m}_persp",
           "particles": f"{n} particles, 70 % uniform + 30 % in 200 Gaussian clusters (sigma 0.01-0.05), "
                        "values LogNormal(0, 0.5), one smoothing length h = 1/256 (256^3 cells), cubic spline",
           "grid_build_ms": min(up)}
    for name, prec in (("fwd_fp32", M.PRECISION_FP32), ("fwd_precision_form", M.PRECISION_COMPENSATED_FF_MESE)):
        ctx.precision = prec
        ms = timed(fwd)
        out[name] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    ctx.precision = M.PRECISION_FP32
    # differentiation form: forward + transfer-function adjoint
    wl.gen.compact_image = 0
    b4 = torch.empty(P * 4, device="cuda")
    rgba = torch.empty((H, Wd, 4), device="cuda")
    tab = torch.from_numpy(tf.table).cuda()
    gtab = torch.zeros((256, 4), device="cuda")

    def fwd_bwd():
        ctx.diff_forward(wl.camera, wl.gen, wl.rec, Wd, H, m, tab, d_mo, b4, d_pm, rgba)
        with torch.cuda.stream(stream):
            g = 2.0 * rgba
            gtab.zero_()
        ctx.diff_backward(wl.camera, wl.gen, wl.rec, Wd, H, m, tab, d_mo, b4, d_pm, rgba, g, gtab, None)

    ms = timed(fwd_bwd)
    out["diff_fwd_tf_adjoint"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}

    # the configuration's own text: a smoothing length per particle (0.005-0.02) with the Wendland C2 kernel, a
    # variant the reference does not have (parity unpinned: checked against the oracle's restatement)
    wv = W.sph_wendland_workload(n=n, width=Wd, height=H, num_moments=m, seed=31)
    hs = torch.from_numpy(wv.h).cuda()
    e = _events(1)[0]
    e[0].record(stream)
    ctx.upload_particles_h(*xs[:4], hs, dmin, dmax)
    e[1].record(stream)
    ctx.synchronize()
    build_ms = e[0].elapsed_time(e[1])
    wl.gen.compact_image = 1
    saved = (wl.gen.step_size, wl.rec.step_size, args.steps, args.warmup)
    wl.gen.step_size, wl.rec.step_size = wv.gen.step_size, wv.rec.step_size
    args.steps, args.warmup = 1, 1
    ms = timed(fwd)
    wl.gen.step_size, wl.rec.step_size, args.steps, args.warmup = saved
    out["wendland_variant"] = {
        "workload": wv.name, "grid_build_ms": build_ms,
        "particles": f"{n} particles as above, smoothing length per particle uniform in [0.005, 0.02], Wendland C2 "
                     "kernel, grid cell size = the largest smoothing length, step 2^-9",
        "parity": "unpinned: the reference has no per-particle smoothing length; checked against the oracle's "
                  "restatement (tests/test_gpu_particles.py, tests/test_oracle_wendland.py)",
        "fwd_fp32": {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}}
    ctx.close()
    return out


def quantization_table_timing(args, ctx, cam, gen, Wd, H, m, d_mo, d_b, d_c, d_idx, d_cm, d_cp, steps):
    """The data-dependent quantization table of the generate flow (create_quantization_table on the 64 x 64
    sample_moment_image, main.cpp:318-327) for the prediction-coded image: the stage call's wall time (launches,
    the read-back of the means and the search), and the oracle's sequential search on the same sample on the
    host cores (the reference's CPU path; its OpenMP loops over the sample's pixels)."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    ctx.stage_generate_moments(cam, gen, Wd, H, m, d_mo, d_b, d_c)
    total = ctx.stage_compact(Wd, H, m, d_c, d_mo, d_idx, d_cm)
    ctx.stage_prediction_encode(Wd, H, m, d_idx, d_cm, total, 0, gen.bias, d_cp)
    ctx.synchronize()
    launches0 = ctx.kernel_launches
    times = []
    for i in range(args.warmup + steps):
        t0 = time.perf_counter()
        table = ctx.stage_create_quantization_table(Wd, H, m, d_idx, d_cm, 0, d_cp, 10, sampling=64)
        if i >= args.warmup:
            times.append((time.perf_counter() - t0) * 1e3)
    launches = (ctx.kernel_launches - launches0) // (args.warmup + steps)
    # the sample on the host for the oracle: offsets of the sampled pixels, their moments gathered on the device
    s = 64
    index = d_idx.cpu().numpy().view(np.uint32)
    src = (np.arange(s)[:, None] * (H // s) * Wd + np.arange(s)[None, :] * (Wd // s)).reshape(-1)
    off, cnt = index[src].astype(np.int64), (index[src + 1] - index[src]).astype(np.int64)
    s_index = np.zeros(s * s + 1, np.uint32)
    s_index[1:] = np.cumsum(cnt)
    gather = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)]) if cnt.sum() else np.zeros(0, np.int64)
    s_data = d_cm[torch.from_numpy(gather).cuda()].cpu().numpy() if gather.size else np.zeros(0, np.float32)
    cp = d_cp.cpu().numpy().view(np.uint16)[:2 * (m - 1)]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref_table, _, evals = O.create_quantization_table(s, s, m, s_index, s_data, 0, cp, 10, nthreads=threads)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    return {"sample": f"{s}x{s} of {Wd}x{H}", "start_bits": 10, "ms": statistics.mean(times),
            "gpu_launches": int(launches), "table_bits_per_pixel": int(table.astype(np.int64).sum()),
            "table_equals_oracle": bool(table.tolist() == ref_table.tolist()),
            "cpu_oracle": {"ms": cpu_ms, "threads": threads, "evaluations": evals,
                           "kind": "port (sequential search of measure_coding_error.cpp:374-438)"}}


def run_uncertainty(args, local):
    """Error bounds and uncertainty rendering on the default workload (512^3 mixing layer, 1024^2, m = 64): the
    moment image is generated, compacted and prepared once; then per launch the error-bound kernel for each measure
    (reconstruct_error at the re-march step), the uncertainty table build and the two renderers.  The oracle's
    RMSE error bounds on every 8th row, on the host cores, beside them."""
    import torch

    import mray_gb300 as M
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    wl = section_workload()
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P = Wd * H
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_grid(torch.from_numpy(wl.volume).cuda(), wl.domain_min, wl.domain_max)
    mo = torch.empty(P * m, device="cuda")
    b = torch.empty(2 * P, dtype=torch.int16, device="cuda")
    c = torch.empty(P, dtype=torch.int32, device="cuda")
    idx = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    cm = torch.empty(P * m, device="cuda")
    pm = torch.empty(P * m, device="cuda")
    eb = torch.empty(P, dtype=torch.int16, device="cuda")
    rgba = torch.empty(P * 4, device="cuda")
    ctx.stage_generate_moments(wl.camera, wl.gen, Wd, H, m, mo, b, c)
    ctx.stage_compact(Wd, H, m, c, mo, idx, cm)
    ctx.stage_prepare_moments(Wd, H, m, idx, cm, pm, bias=wl.rec.bias)
    steps = max(1, min(args.steps, 5))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        ev = _events(steps)
        for e in ev:
            e[0].record(stream)
            fn()
            e[1].record(stream)
        ctx.synchronize()
        return statistics.mean(e[0].elapsed_time(e[1]) for e in ev)

    out = {"workload": f"mixing_layer{SECTION_SIZE}^3_{Wd}x{H}_m{m}_persp", "step": "the re-march step"}
    for name, et in (("error_bounds_max", M.MAX_ERROR), ("error_bounds_rmse", M.RMSE),
                     ("error_bounds_p90", M.ERROR_PERCENTILE)):
        ep = M.ErrorReconstructionParameters(error_type=et, step_size=wl.rec.step_size, bias=wl.rec.bias)
        ms = timed(lambda: ctx.stage_reconstruct_error(wl.camera, ep, Wd, H, m, idx, pm, b, eb))
        out[name] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    utf = M.read_from_disk_uncertainty(wl.tf1d, wl.tf_step, M.RMSE)
    t0 = time.perf_counter()
    ctx.upload_uncertainty_tf(utf)
    out["uncertainty_table_ms"] = (time.perf_counter() - t0) * 1e3
    ctx.upload_tf(M.preintegrate(wl.tf1d, wl.tf_step).table)
    for name, mode in (("interpolation", 0), ("convolution", 1)):
        up = M.UncertaintyReconstructionParameters(rec=wl.rec, error_type=M.RMSE)
        ms = timed(lambda: ctx.stage_reconstruct_uncertainty(wl.camera, up, mode, Wd, H, m, wl.domain_min,
                                                             wl.domain_max, idx, pm, b, eb, rgba))
        out[f"uncertainty_{name}"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    ms = timed(lambda: ctx.stage_reconstruct(wl.camera, wl.rec, Wd, H, m, wl.domain_min, wl.domain_max, idx, pm, b,
                                             rgba))
    out["plain_reconstruct"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    # the reference direct volume rendering of the same volume (the ground truth of the moment path), at the
    # generation step
    rp = M.ReferenceParameters(step_size=wl.gen.step_size, medium_emission=wl.rec.medium_emission,
                               early_ray_termination=wl.rec.early_ray_termination, data_min=wl.gen.data_min,
                               data_max=wl.gen.data_max)
    ms = timed(lambda: ctx.stage_generate_reference(wl.camera, rp, Wd, H, rgba))
    out["reference_dvr"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    # the oracle (the reference's CPU method) on every 64th row of the same image
    index = idx.cpu().numpy().view(np.uint32)
    data = cm[:int(index[-1])].cpu().numpy()
    bounds = b.cpu().numpy().view(np.uint16)
    ep = M.ErrorReconstructionParameters(error_type=M.RMSE, step_size=wl.rec.step_size, bias=wl.rec.bias)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    O.reconstruct_error(wl.camera, ep, wl.volume, wl.domain_min, wl.domain_max, Wd, H, m, index, data, False, 0, None,
                        bounds, "f32", nthreads=threads, rows=(0, H, 8))
    cpu_s = time.perf_counter() - t0
    rays = Wd * len(range(0, H, 8))
    out["cpu_oracle_rmse"] = {"value": rays / cpu_s / 1e6, "unit": UNIT, "threads": threads,
                              "sample": f"rows y = 0 mod 8 ({rays} rays, {cpu_s:.1f} s)", "kind": "port"}
    ctx.close()
    return out


def run_scattering(args, local):
    """Single scattering from the transmittance cache on the default workload (512^3 mixing layer, 1024^2 eye image,
    m = 64), with the reference's single-scattering settings (eval/turbine/turbine_single_scattering.json): a 512^2
    light image with 50 moments (compact, bounds, prediction coded, error threshold 0.01) along an oblique light, a
    256 x 128 x 128 cache, emission 0.6, scattering 0.35, intensity 0.28.  Per launch: the cache build (its march
    over the light image, the decode and the copy into the sampled array), the re-march with and without
    in-scattering and the reference renderer sampling the cache.  The oracle's cache loop (one thread, as the
    reference's result is defined) on every 32nd row of the light image beside them."""
    import torch

    import mray_gb300 as M
    from mray_gb300 import workloads as W
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    wl = section_workload()
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P = Wd * H
    lw = lh = max(64, SECTION_IMAGE // 2)
    lm = min(50, m)
    LP = lw * lh
    light = W.light_camera((0.3, -1.0, 0.2), center=(0.5, 0.5, 0.5), half_extent=0.9, distance=2.0)
    ssp = M.SingleScatteringParameters(enable=1, use_cache=1, cache_size_x=256, cache_size_y=128, cache_size_z=128,
                                       step_size_factor=4.0, direction_x=light.dir[0], direction_y=light.dir[1],
                                       direction_z=light.dir[2], intensity_r=0.28, intensity_g=0.28,
                                       intensity_b=0.28)
    rp = M.ReconstructionParameters(step_size=wl.rec.step_size, bias=wl.rec.bias, medium_emission=0.6,
                                    medium_scattering=0.35, early_ray_termination=wl.rec.early_ray_termination,
                                    ss=ssp)
    lgen = M.GenerationParameters(step_size=wl.gen.step_size, error_threshold=0.01, bias=wl.gen.bias, compact_image=1,
                                  prediction_coding=1, transform_to_bounds=1, transform_bound_eps=0.005)
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_grid(torch.from_numpy(wl.volume).cuda(), wl.domain_min, wl.domain_max)
    ctx.upload_tf(M.preintegrate(wl.tf1d, wl.tf_step).table)
    # the light image through the host API (generation, compaction, prediction coding), then prepared on the device
    lmi = ctx.generate(light, lgen, lw, lh, lm)
    l_idx = torch.from_numpy(lmi.index.view(np.int32)).cuda()
    l_data = torch.from_numpy(lmi.data).cuda()
    l_b = torch.from_numpy(lmi.bounds.reshape(-1).view(np.int16)).cuda()
    l_cp = torch.from_numpy(lmi.coding_params.view(np.int16)).cuda()
    l_pm = torch.empty_like(l_data)
    ctx.stage_prepare_moments(lw, lh, lm, l_idx, l_data, l_pm, prediction_code=True, coding_warp=0, coding_params=l_cp,
                              bias=rp.bias)
    # the eye image
    mo = torch.empty(P * m, device="cuda")
    b = torch.empty(2 * P, dtype=torch.int16, device="cuda")
    c = torch.empty(P, dtype=torch.int32, device="cuda")
    idx = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    cm = torch.empty(P * m, device="cuda")
    pm = torch.empty(P * m, device="cuda")
    rgba = torch.empty(P * 4, device="cuda")
    ctx.stage_generate_moments(wl.camera, wl.gen, Wd, H, m, mo, b, c)
    ctx.stage_compact(Wd, H, m, c, mo, idx, cm)
    ctx.stage_prepare_moments(Wd, H, m, idx, cm, pm, bias=wl.rec.bias)
    steps = max(1, min(args.steps, 5))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        ev = _events(steps)
        for e in ev:
            e[0].record(stream)
            fn()
            e[1].record(stream)
        ctx.synchronize()
        return statistics.mean(e[0].elapsed_time(e[1]) for e in ev)

    out = {"workload": f"mixing_layer{SECTION_SIZE}^3_{Wd}x{H}_m{m}_persp; light {lw}x{lh} m{lm} ortho; cache 256x128x128",
           "step": "the re-march step"}
    d_cache = torch.empty(128 * 128 * 256, device="cuda")
    ms = timed(lambda: ctx.stage_reconstruct_single_scattering_cache(light, rp, lw, lh, lm, wl.domain_min,
                                                                     wl.domain_max, l_idx, l_pm, l_b, d_cache))
    out["cache_build"] = {"value": LP / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms,
                          "written_voxels": float((d_cache > 0).float().mean().item())}
    ms = timed(lambda: ctx.stage_reconstruct(wl.camera, rp, Wd, H, m, wl.domain_min, wl.domain_max, idx, pm, b, rgba))
    out["reconstruct_single_scattering"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    rp.ss.enable = 0
    ms = timed(lambda: ctx.stage_reconstruct(wl.camera, rp, Wd, H, m, wl.domain_min, wl.domain_max, idx, pm, b, rgba))
    out["reconstruct_plain"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    rp.ss.enable = 1
    ms = timed(lambda: ctx.stage_generate_reference_reconstructed_ss(wl.camera, rp, Wd, H, rgba))
    out["reference_reconstructed_ss"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    # the oracle's cache loop on every 32nd row of the light image (the others left empty)
    index = lmi.index.astype(np.int64)
    keep = np.repeat(np.arange(lh) % 32 == 0, lw)
    counts = np.diff(index) * keep
    sample_index = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    lpm = l_pm.cpu().numpy()
    sample_pm = np.concatenate([lpm[index[p]:index[p + 1]] for p in np.nonzero(keep)[0]]) if keep.any() else lpm[:0]
    bounds = lmi.bounds.reshape(-1)
    row = M.preintegrate(wl.tf1d, wl.tf_step).table
    t0 = time.perf_counter()
    O.ss_cache(light, rp, lw, lh, lm, wl.domain_min, wl.domain_max, sample_index, sample_pm, bounds, row)
    cpu_s = time.perf_counter() - t0
    rays = int(keep.sum())
    out["cpu_oracle_cache"] = {"value": rays / cpu_s / 1e6, "unit": UNIT, "threads": 1,
                               "sample": f"light rows y = 0 mod 32 ({rays} rays, {cpu_s:.1f} s)", "kind": "port"}
    ctx.close()
    return out


def run_file_format(args, local):
    """The moment-image file format on the default workload's image (1024^2, m = 64, compact, prediction coded):
    write_moment_image / load_moment_image in memory with LZ4-compressed sections, the payload as packed 10-bit codes
    (table [16, 10, ...]) and as the entropy coder's streams.  Quantization runs on the GPU, LZ4 and the arithmetic
    coder on the host (the streams in parallel over the host threads)."""
    import torch

    import mray_gb300 as M

    wl = section_workload()
    Wd, H, m = wl.width, wl.height, wl.num_moments
    ctx = M.Context(local)
    ctx.set_stream(torch.cuda.current_stream())
    ctx.upload_grid(torch.from_numpy(wl.volume).cuda(), wl.domain_min, wl.domain_max)
    gen = wl.gen
    gen.prediction_coding = 1
    mi = ctx.generate(wl.camera, gen, Wd, H, m)
    mi.domain_min, mi.domain_max = wl.domain_min, wl.domain_max
    table = np.array([16] + [10] * (m - 1), np.uint8)
    raw_mb = mi.data.size * 4 / 1e6
    out = {"workload": f"mixing_layer{SECTION_SIZE}^3_{Wd}x{H}_m{m}_persp prediction coded",
           "moments_MB": raw_mb, "host_threads": os.cpu_count()}
    reps = max(1, min(args.steps, 3))
    for name, entropy in (("packed_10bit_lz4", False), ("entropy_coded_lz4", True)):
        blob = ctx.encode_moment_image(mi, True, 10, entropy, table)
        t0 = time.perf_counter()
        for _ in range(reps):
            blob = ctx.encode_moment_image(mi, True, 10, entropy, table)
        enc = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            back, _ = ctx.decode_moment_image(blob)
        dec = (time.perf_counter() - t0) / reps
        out[name] = {"file_MB": len(blob) / 1e6, "write_ms": enc * 1e3, "read_ms": dec * 1e3,
                     "write_moments_GB_s": raw_mb / 1e3 / enc, "read_moments_GB_s": raw_mb / 1e3 / dec}
    ctx.close()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.section in ("all", "headline"):
        run_ours(args)
    else:
        import torch

        _, _, local = dist_info()
        torch.cuda.set_device(local)
        if args.section == "errors":
            print(json.dumps({"errors_vs_fp64": precision_errors(args, local)}), flush=True)
            return
        if args.section == "refcuda":
            print(json.dumps({"refcuda": run_reference_cuda(args)}), flush=True)
            return
        if args.section == "refcuda-worker":
            print(json.dumps({"refcuda-worker": refcuda_worker(args, local)}), flush=True)
            return
        fn = {"mixing512": run_mixing512, "diff": run_diff, "sph": run_sph, "uncertainty": run_uncertainty,
              "scattering": run_scattering, "file": run_file_format}[args.section]
        print(json.dumps({args.section: fn(args, local)}), flush=True)


if __name__ == "__main__":
    main()
