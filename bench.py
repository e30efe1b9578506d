"""Benchmark of the moment-image hot path: generate (moments + compaction) -> MESE preparation -> reconstruct.

Default workload (the precision form): a 512^3 float32 mixing-layer grid (64 seeded Fourier modes, 5 % seeded
noise), a 1024 x 1024 perspective view, 0.5-voxel steps, 64 trigonometric moments, Kahan-compensated FP32 moment
sums and the MESE preparation's FP64 steps in float-float arithmetic.  A step is one full pass over the image
with the volume resident in HBM:
    generate_grid_kernel -> scan / compaction -> prepare_ff_kernel -> reconstruct_kernel
and the metric is million rays (pixels) per second of that pass.

The JSON line also carries:
  e2e           the same pass through the drop-in host API (mraygb_generate / mraygb_reconstruct): the volume is
                uploaded from pinned host memory, the moment image comes back to the host and goes back up, the
                RGBA comes back -- every copy inside the timed region;
  plain_fp32    the same pass in the reference's plain FP32 arithmetic;
  roofline      the dominant kernel (generate) against the measured HBM copy bandwidth (compulsory bytes), with
                its FP32 issue rate beside it (the binding roof of this method);
  cpu_baseline  the reference's CPU method (the oracle's FP32 restatement, OpenMP on all host cores) timed on a
                row-strided sample of the same workload.

--impl reference runs only the CPU reference method on bounded samples of the workload.
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512, help="volume edge (voxels)")
    ap.add_argument("--image", type=int, default=1024, help="image edge (pixels)")
    ap.add_argument("--moments", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the differentiation-form, SPH and FP64-error sections")
    ap.add_argument("--sph-particles", type=int, default=16_000_000)
    ap.add_argument("--section", default="all",
                    choices=["all", "diff", "sph", "large", "uncertainty", "scattering", "file"],
                    help="diff / sph: run only that section and print its JSON (for profiling)")
    return ap.parse_args()


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


def workload(args):
    from mray_gb300 import workloads as W

    return W.mixing_layer_workload(n=args.size, width=args.image, height=args.image, num_moments=args.moments,
                                   modes=64, seed=21,
                                   name=f"mixing_layer{args.size}^3_{args.image}x{args.image}_m{args.moments}_persp")


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
# CPU reference method (the oracle's FP32 restatement of the reference's CPU path)
# ------------------------------------------------------------------------------------------------------------

def cpu_reference_sample(wl, row_step: int, row_offset: int = 0, nthreads: int = 0):
    """generate (per-pixel moments + counts) + prepare + reconstruct on rows y = row_offset (mod row_step), with
    the reference's CPU arithmetic.  Returns (rays, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    W, H, m = wl.width, wl.height, wl.num_moments
    rows = (row_offset, H, row_step)
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    t0 = time.perf_counter()
    mo, b, c = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, W, H, m, "f32",
                                  nthreads=nthreads, rows=rows)
    idx, data = O.compact(c, mo)
    pm = O.prepare_moments(W, H, m, idx, data, bias=wl.rec.bias, precision="f32", nthreads=nthreads, rows=rows)
    O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx, pm, b, tf, "f32",
                  nthreads=nthreads, rows=rows)
    dt = time.perf_counter() - t0
    rays = len(range(row_offset, H, row_step)) * W
    return rays, dt


def cpu_baseline(wl, target_s: float):
    ncores = os.cpu_count() or 1
    # calibrate on a sparse sample, then size the sample to the target time
    probe_step = max(1, wl.height // 8)
    rays, dt = cpu_reference_sample(wl, probe_step, 1)
    rate = rays / max(dt, 1e-9)
    want_rays = rate * target_s
    step = int(max(1, min(wl.height, round(wl.width * wl.height / max(want_rays, 1.0)))))
    rays, dt = cpu_reference_sample(wl, step, 0)
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"rows y = 0 mod {step} of the {wl.width}x{wl.height} image ({rays} rays, {dt:.1f} s): "
                      f"per-pixel generate + prepare + reconstruct in the reference's FP32 arithmetic "
                      f"(oracle/mray_oracle.c, OpenMP {ncores} threads)"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    wl = workload(args)
    ncores = os.cpu_count() or 1
    # each step: a bounded row sample (every 16th row at the default size: 64 rows, enough for every host core),
    # rows rotating between steps
    step_rows = max(1, wl.height // 64)
    for i in range(args.warmup):
        cpu_reference_sample(wl, step_rows, i % step_rows)
    times, rays_total = [], 0
    for i in range(args.steps):
        rays, dt = cpu_reference_sample(wl, step_rows, (args.warmup + i) % step_rows)
        times.append(dt)
        rays_total += rays
    total = sum(times)
    value = rays_total / total / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl.name, "volume": f"{args.size}^3 float32 mixing layer", "image":
                       f"{wl.width}x{wl.height}", "num_moments": wl.num_moments, "step": "0.5 voxel",
                       "sample_per_step": f"every {step_rows}th row ({wl.width * len(range(0, wl.height, step_rows))} rays)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": f"every {step_rows}th row per step, rows rotating; the reference's CPU "
                                       f"method in its FP32 arithmetic (oracle/mray_oracle.c), OpenMP {ncores} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------------------
# GPU path
# ------------------------------------------------------------------------------------------------------------

def read_profile_traffic():
    """DRAM bytes per launch of generate_grid_kernel at the default workload, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "generate_grid_kernel_mixing512_1024sq_m64.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].strip().split()[0])
    except OSError:
        pass
    return None


def run_ours(args):
    import torch

    import mray_gb300 as M

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    wl = workload(args)
    W, H, m = wl.width, wl.height, wl.num_moments
    P = W * H
    ctx = M.Context(local, precision=M.PRECISION_COMPENSATED_FP64_MESE)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    vol = torch.from_numpy(wl.volume).cuda()
    ctx.upload_grid(vol, wl.domain_min, wl.domain_max)
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    ctx.upload_tf(tf.table)
    torch.cuda.synchronize()

    d_mo = torch.empty(P * m, dtype=torch.float32, device="cuda")
    d_b = torch.empty(2 * P, dtype=torch.int16, device="cuda")
    d_c = torch.empty(P, dtype=torch.int32, device="cuda")
    d_idx = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    d_cm = torch.empty(P * m, dtype=torch.float32, device="cuda")
    d_pm = torch.empty(P * m, dtype=torch.float32, device="cuda")
    d_rgba = torch.empty(P * 4, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MiB > 129 MB L2

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        ctx.stage_generate_moments(wl.camera, wl.gen, W, H, m, d_mo, d_b, d_c)
        if ev is not None:
            ev[1].record(stream)
        ctx.stage_compact(W, H, m, d_c, d_mo, d_idx, d_cm)
        if ev is not None:
            ev[3].record(stream)
        ctx.stage_prepare_moments(W, H, m, d_idx, d_cm, d_pm, bias=wl.rec.bias)
        if ev is not None:
            ev[4].record(stream)
        ctx.stage_reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_rgba)
        if ev is not None:
            ev[2].record(stream)

    stage_ms = {}

    def timed_loop(precision):
        ctx.precision = precision
        for _ in range(args.warmup):
            step()
        ctx.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = ctx.kernel_launches
        t0 = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))  # evict the previous step's lines from L2 (outside the timed events)
            step(evs[i])
        ctx.synchronize()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        launches = ctx.kernel_launches - launches0
        step_ms = [e[0].elapsed_time(e[2]) for e in evs]
        gen_ms = [e[0].elapsed_time(e[1]) for e in evs]
        stage_ms[precision] = {
            "generate": statistics.mean(gen_ms),
            "compaction": statistics.mean(e[1].elapsed_time(e[3]) for e in evs),
            "prepare": statistics.mean(e[3].elapsed_time(e[4]) for e in evs),
            "reconstruct": statistics.mean(e[4].elapsed_time(e[2]) for e in evs)}
        return sum(step_ms), statistics.mean(gen_ms), launches, wall

    # the plain FP32 form and the FP64 precision form first (reported beside the headline), then the headline
    # precision form (float-float MESE preparation) under the clock sampler
    plain_ms, _, _, _ = timed_loop(M.PRECISION_FP32)
    fp64_ms, _, _, _ = timed_loop(M.PRECISION_COMPENSATED_FP64_MESE)
    sampler = ClockSampler(local)
    sampler.start()
    total_ms, gen_ms, launches, wall = timed_loop(M.PRECISION_COMPENSATED_FF_MESE)
    clocks = sampler.stop()

    t_max, plain_max, fp64_max = reduce_max([total_ms, plain_ms, fp64_ms], dist, "cuda")
    value = world * P * args.steps / (t_max * 1e-3) / 1e6
    plain_value = world * P * args.steps / (plain_max * 1e-3) / 1e6
    fp64_value = world * P * args.steps / (fp64_max * 1e-3) / 1e6

    # roofline of the dominant kernel (generate): compulsory bytes and method FLOPs per launch
    spr = samples_per_ray(wl)
    total_samples = int(spr.sum())
    vol_bytes = wl.volume.size * 4
    gen_bytes = vol_bytes + P * (m * 4 + 4 + 4)
    gen_flops = total_samples * (4 * (m - 1) + 24)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if hbm_peak is None:
        hbm_peak, peak_src = 6800.0, "fallback"
    achieved = gen_bytes / (gen_ms * 1e-3) / 1e9
    fp32_peak = 152 * 128 * 2 * (clocks.get("sm_max_mhz") or 2070.0) * 1e6 / 1e12
    fp32_achieved = gen_flops / (gen_ms * 1e-3) / 1e12
    traffic = read_profile_traffic()
    roofline = {"bound": "hbm", "kernel": "generate_grid_kernel<16,true>", "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak, "peak_source": peak_src, "traffic": traffic,
                "algorithmic_bytes_per_launch": gen_bytes, "kernel_ms": gen_ms,
                "fp32": {"achieved_tflops": fp32_achieved, "peak_tflops": fp32_peak,
                         "frac": fp32_achieved / fp32_peak, "flops_per_launch": gen_flops,
                         "samples_per_launch": total_samples,
                         "note": "method FLOPs 4(m-1)+24 per sample (FMA = 2) against the nominal FP32 issue rate "
                                 "152 SMs x 128 lanes x 2 at the max SM clock; the binding roof of this method"}}

    # every stage of the step: its own Mrays/s and its compulsory bytes against the measured HBM peak (the kernels
    # are issue bound on FP32 arithmetic, so these fractions are small by the method's nature)
    nd = int(d_idx[-1].item())
    stage_bytes = {"generate": gen_bytes, "compaction": P * m * 4 + nd * 4 + 8 * P,
                   "prepare": 2 * nd * 4 + 4 * P, "reconstruct": nd * 4 + 24 * P}
    stages = {}
    for name, prec in (("plain_fp32", M.PRECISION_FP32), ("precision_form_fp64", M.PRECISION_COMPENSATED_FP64_MESE),
                       ("precision_form", M.PRECISION_COMPENSATED_FF_MESE)):
        stages[name] = {k: {"ms": v, "Mrays_s": P / (v * 1e-3) / 1e6,
                            "hbm_frac": stage_bytes[k] / (v * 1e-3) / 1e9 / hbm_peak,
                            "algorithmic_bytes": stage_bytes[k]} for k, v in stage_ms[prec].items()}

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, ctx, wl, dist)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, args.cpu_seconds)

    extras = {}
    if rank == 0 and not args.no_extras:
        extras["differentiation_form"] = run_diff(args, local)
        extras["sph"] = run_sph(args, local)
        extras["large"] = run_large(args, local)
        extras["uncertainty"] = run_uncertainty(args, local)
        extras["single_scattering"] = run_scattering(args, local)
        extras["file_format"] = run_file_format(args, local)
        extras["errors_vs_fp64"] = precision_errors(args, local)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": {"workload": wl.name, "volume": f"{args.size}^3 float32 mixing layer (64 modes, 5% noise)",
                           "image": f"{W}x{H} perspective", "num_moments": m, "step": "0.5 voxel",
                           "precision": "Kahan-compensated FP32 moment sums; MESE preparation with its FP64 steps "
                                        "(exponential moments, Levinson) in float-float arithmetic, FP32 tail",
                           "l2": "256 MiB buffer written between timed steps (volume 512 MiB > L2)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "plain_fp32": {"value": plain_value, "unit": UNIT, "ms_per_step": plain_max / args.steps},
                "precision_form_fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": fp64_max / args.steps,
                                        "note": "the same pass with the MESE preparation in native FP64"},
                "precision_over_plain": value / plain_value,
                "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "stages": stages, "cpu_baseline": cpu,
                "clocks": clocks,
                "wall_s_timed": wall, **extras}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_e2e(args, ctx, wl, dist):
    """The drop-in host API with pinned host buffers; every copy is inside the timed region."""
    import torch

    import mray_gb300 as M

    W, H, m = wl.width, wl.height, wl.num_moments
    P = W * H
    vol_h = torch.from_numpy(wl.volume).pin_memory()
    vol_np = vol_h.numpy()
    mi = M.MomentImageHost(W, H, m, True, True)
    mi.data = torch.empty(P * m, dtype=torch.float32).pin_memory().numpy()
    mi.index = torch.empty(P + 1, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    mi.bounds = torch.empty(2 * P, dtype=torch.int16).pin_memory().numpy().view(np.uint16).reshape(P, 2)
    img = M.ColorImageHost(W, H)
    img.rgba_float = torch.empty(P * 4, dtype=torch.float32).pin_memory().numpy().reshape(H, W, 4)
    img.rgba = torch.empty(P * 4, dtype=torch.uint8).pin_memory().numpy().reshape(H, W, 4)
    grid = M.RegularGrid(vol_np, wl.domain_min, wl.domain_max)
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    data_full = mi.data

    def one():
        mi.data = data_full
        M.generate(wl.camera, grid, mi, wl.gen, context=ctx)
        M.reconstruct(wl.camera, mi, tf, img, wl.rec, context=ctx)

    for _ in range(max(1, args.warmup)):
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
    world = dist.get_world_size() if dist else 1
    moments_bytes = mi.data.size * 4
    h2d = wl.volume.size * 4 + 256 * 16 + moments_bytes + (P + 1) * 4 + 4 * P
    d2h = moments_bytes + (P + 1) * 4 + 4 * P + P * 16 + P * 4 + 4
    return {"value": world * P * args.steps / dt / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
            "path": "mraygb_upload_grid + mraygb_generate + mraygb_upload_tf + mraygb_reconstruct on pinned host "
                    "buffers (the drop-in seam of generate_device / reconstruct_device)"}


# ------------------------------------------------------------------------------------------------------------
# further sections of the JSON line: the differentiation form, SPH particles, errors against the FP64 oracle
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
    ctx.close()
    return {"workload": f"{wl.name}_ortho (256^3 Marschner-Lobb, 512x512, m=31, no compaction, ert 1)",
            "fwd": {"value": P / (f_ms * 1e-3) / 1e6, "unit": UNIT, "ms": f_ms, "gpu_launches_per_step": f_l},
            "fwd_adjoint": {"value": P / (fb_ms * 1e-3) / 1e6, "unit": UNIT, "ms": fb_ms,
                            "gpu_launches_per_step": fb_l,
                            "gradients": "transfer-function row (256 x RGBA) and all 256^3 voxel densities"},
            "fwd_adjoint_over_fwd": fb_ms / f_ms, "loss": loss,
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
    h = 1.0 / 256
    x, y, z, v = W.sph_particles(n, seed=31)
    wl = W.sph_workload(n=64, h=h, width=args.image, height=args.image, num_moments=args.moments, seed=31)
    rng = np.random.default_rng(38)
    smp = v[rng.integers(0, n, size=100000)]
    wl.gen.data_min, wl.gen.data_max = float(np.percentile(smp, 1)), float(np.percentile(smp, 99))
    dmin = (float(x.min()), float(y.min()), float(z.min()))
    dmax = (float(x.max()), float(y.max()), float(z.max()))
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
    ctx.close()
    return out


def run_large(args, local):
    """The large configuration (both forms): a 1024^3 float32 mixing layer (256 modes, built on the device), a
    2048^2 perspective view, 64 moments, prediction coding with the default warp and 10-bit codes (table [16, 10 x
    63]).  A step: generate -> compaction -> prediction encode + coding parameters -> quantize and pack the codes
    -> unpack and dequantize -> Lagrange multipliers from the prediction-coded moments -> reconstruct; in the plain
    FP32 form and in the float-float precision form.  Then the differentiation form (no compaction) with its
    transfer-function adjoint."""
    import torch

    import mray_gb300 as M
    from mray_gb300 import workloads as W

    n, Wd, H, m = 1024, 2048, 2048, 64
    P = Wd * H
    gen, rec, cam, tf1d, tf_step = W.mixing_layer_setup(n, Wd, H, prediction_coding=True)
    dmin, dmax = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    ctx = M.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    vol = W.mixing_layer_device(n, modes=256, seed=21)
    torch.cuda.synchronize()
    ctx.upload_grid(vol, dmin, dmax)
    del vol
    tf = M.preintegrate(tf1d, tf_step)
    ctx.upload_tf(tf.table)
    table = M.default_quantization_table(m, 10)
    d_mo = torch.empty(P * m, device="cuda")
    d_b = torch.empty(2 * P, dtype=torch.int16, device="cuda")
    d_c = torch.empty(P, dtype=torch.int32, device="cuda")
    d_idx = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    d_cm = torch.empty(P * m, device="cuda")
    d_cp = torch.empty(2 * m, dtype=torch.int16, device="cuda")
    d_codes = torch.empty(P * (16 + 10 * (m - 1)) // 8 + 64, dtype=torch.uint8, device="cuda")
    d_pm = torch.empty(P * m, device="cuda")
    d_rgba = torch.empty(P * 4, device="cuda")
    sizes = {}

    def fwd():
        ctx.stage_generate_moments(cam, gen, Wd, H, m, d_mo, d_b, d_c)
        total = ctx.stage_compact(Wd, H, m, d_c, d_mo, d_idx, d_cm)
        ctx.stage_prediction_encode(Wd, H, m, d_idx, d_cm, total, 0, gen.bias, d_cp)
        nbytes = ctx.stage_quantize_prediction_coding(Wd, H, m, d_idx, d_cm, table, d_codes)
        ctx.stage_dequantize_prediction_coding(Wd, H, m, d_idx, table, d_codes, nbytes, d_cm)
        ctx.stage_prepare_moments(Wd, H, m, d_idx, d_cm, d_pm, prediction_code=1, coding_warp=0, coding_params=d_cp,
                                  bias=rec.bias)
        ctx.stage_reconstruct(cam, rec, Wd, H, m, dmin, dmax, d_idx, d_pm, d_b, d_rgba)
        sizes["moments"], sizes["code_bytes"] = total, nbytes

    def timed(fn, steps):
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

    steps = max(1, min(args.steps, 3))
    out = {"workload": f"mixing_layer{n}^3_{Wd}x{H}_m{m}_persp_prediction_coded_10bit",
           "volume": "1024^3 float32 mixing layer, 256 modes, 5 % noise (built on the device with torch)"}
    for name, prec in (("fwd_fp32", M.PRECISION_FP32), ("fwd_precision_form", M.PRECISION_COMPENSATED_FF_MESE)):
        ctx.precision = prec
        ms = timed(fwd, steps)
        out[name] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
    out["compact_moments"], out["code_bytes"] = int(sizes["moments"]), int(sizes["code_bytes"])
    ctx.precision = M.PRECISION_FP32
    out["quantization_table"] = quantization_table_timing(args, ctx, cam, gen, Wd, H, m, d_mo, d_b, d_c, d_idx,
                                                          d_cm, d_cp, steps)
    del d_cm, d_codes
    # the differentiation form with the transfer-function adjoint
    gen.compact_image, gen.prediction_coding = 0, 0
    b4 = torch.empty(P * 4, device="cuda")
    rgba = torch.empty((H, Wd, 4), device="cuda")
    tab = torch.from_numpy(tf.table).cuda()
    gtab = torch.zeros((256, 4), device="cuda")

    def fwd_bwd():
        ctx.diff_forward(cam, gen, rec, Wd, H, m, tab, d_mo, b4, d_pm, rgba)
        with torch.cuda.stream(stream):
            g = 2.0 * rgba
            gtab.zero_()
        ctx.diff_backward(cam, gen, rec, Wd, H, m, tab, d_mo, b4, d_pm, rgba, g, gtab, None)

    ms = timed(fwd_bwd, steps)
    out["diff_fwd_tf_adjoint"] = {"value": P / (ms * 1e-3) / 1e6, "unit": UNIT, "ms": ms}
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

    wl = workload(args)
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

    out = {"workload": f"mixing_layer{args.size}^3_{Wd}x{H}_m{m}_persp", "step": "the re-march step"}
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

    wl = workload(args)
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P = Wd * H
    lw = lh = max(64, args.image // 2)
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

    out = {"workload": f"mixing_layer{args.size}^3_{Wd}x{H}_m{m}_persp; light {lw}x{lh} m{lm} ortho; cache 256x128x128",
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

    wl = workload(args)
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
    out = {"workload": f"mixing_layer{args.size}^3_{Wd}x{H}_m{m}_persp prediction coded",
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


def precision_errors(args, local):
    """Max and RMS errors of the moments, the transmittance and the RGBA of both arithmetic forms against the FP64
    oracle of the same method, on every 8th row of a 128 x 128 image of the default workload (its volume and
    view); pixels whose u16 density bounds differ from the FP64 ones are left out (the bounds are truncated, so
    a last-bit difference of a sampled extreme can move them one step)."""
    import torch

    import mray_gb300 as M
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    a = argparse.Namespace(**vars(args))
    a.image = 128
    wl = workload(a)
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P = Wd * H
    rows = (0, H, 8)
    mo64, b64, c64 = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, Wd, H, m, "f64",
                                        rows=rows)
    idx64, _ = O.compact(c64, mo64.astype(np.float32))
    cnt = c64.reshape(-1)
    data64 = np.concatenate([mo64.reshape(-1, m)[p, :cnt[p]] for p in range(P)]) if cnt.sum() else np.zeros(0)
    pm64 = O.prepare_moments(Wd, H, m, idx64, data64, False, 1, None, wl.rec.bias, "f64", rows=rows)
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    rgba64 = O.reconstruct(wl.camera, wl.rec, Wd, H, m, wl.domain_min, wl.domain_max, idx64, pm64, b64, tf, "f64",
                           rows=rows)
    ctx = M.Context(local)
    ctx.set_stream(torch.cuda.current_stream())
    ctx.upload_grid(torch.from_numpy(wl.volume).cuda(), wl.domain_min, wl.domain_max)
    ctx.upload_tf(tf)
    sel = np.zeros((H, Wd), bool)
    sel[0:H:8] = True
    out = {"sample": f"rows y = 0 mod 8 of a {Wd}x{H} image of the default volume and view; FP64 oracle of the "
                     "same method (oracle/mray_oracle.c, double, exact constants)",
           "moment_error": "max_j |m_j - m_j(FP64)| / max(|m_0(FP64)|, 1e-3) per pixel",
           "rgba_error": "max over channels |c - c(FP64)| per pixel"}
    for name, prec in (("fp32", M.PRECISION_FP32), ("precision_form_fp64", M.PRECISION_COMPENSATED_FP64_MESE),
                       ("precision_form", M.PRECISION_COMPENSATED_FF_MESE)):
        ctx.precision = prec
        d_mo = torch.zeros(P * m, device="cuda")
        d_b = torch.zeros(2 * P, dtype=torch.int16, device="cuda")
        d_c = torch.zeros(P, dtype=torch.int32, device="cuda")
        d_idx = torch.zeros(P + 1, dtype=torch.int32, device="cuda")
        d_cm = torch.zeros(P * m, device="cuda")
        d_pm = torch.zeros(P * m, device="cuda")
        d_rgba = torch.zeros(P * 4, device="cuda")
        ctx.stage_generate_moments(wl.camera, wl.gen, Wd, H, m, d_mo, d_b, d_c)
        ctx.stage_compact(Wd, H, m, d_c, d_mo, d_idx, d_cm)
        ctx.stage_prepare_moments(Wd, H, m, d_idx, d_cm, d_pm, bias=wl.rec.bias)
        ctx.stage_reconstruct(wl.camera, wl.rec, Wd, H, m, wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_rgba)
        ctx.synchronize()
        mo = d_mo.cpu().numpy().reshape(H, Wd, m).astype(np.float64)
        b = d_b.cpu().numpy().view(np.uint16).reshape(H, Wd, 2)
        rgba = d_rgba.cpu().numpy().reshape(H, Wd, 4).astype(np.float64)
        ok = sel & (c64 > 0) & np.all(b == b64, axis=-1)
        me = (np.abs(mo - mo64).max(axis=-1) / np.maximum(np.abs(mo64[..., 0]), 1e-3))[ok]
        te = np.abs(rgba[..., 3] - rgba64[..., 3])[ok]
        re = np.abs(rgba - rgba64).max(axis=-1)[ok]
        out[name] = {"pixels": int(ok.sum()),
                     "moments": {"max": float(me.max()), "rms": float(np.sqrt((me ** 2).mean()))},
                     "transmittance": {"max": float(te.max()), "rms": float(np.sqrt((te ** 2).mean()))},
                     "rgba": {"max": float(re.max()), "rms": float(np.sqrt((re ** 2).mean())),
                              "frac_above_1e-4": float((re > 1e-4).mean()), "frac_above_1e-3": float((re > 1e-3).mean())}}
    ctx.close()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.section != "all":
        import torch

        _, _, local = dist_info()
        torch.cuda.set_device(local)
        fn = {"diff": run_diff, "sph": run_sph, "large": run_large, "uncertainty": run_uncertainty,
              "scattering": run_scattering, "file": run_file_format}[args.section]
        print(json.dumps({args.section: fn(args, local)}), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
