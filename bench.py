"""Benchmark of the plain GPU absorption tracer.

Default workload (`--workload beamline`): the beamline sample -- 512x512x400
int8 label volume (the synthetic recipe scaled x5: crystal ellipsoid 100/70/50
voxels, liquor shell, loop, bubbles), crystal voxels sampled at stride 4 on
each axis (~23k voxels) and 20,000 reflections (omega ~ U[0, 2pi), 2theta ~
U[5, 120] deg), two rays per (voxel, reflection).  One step = one pass of the
path over all reflections.  Other workloads:

  small    96^3 volume, every crystal voxel (~11.7k), 300 reflections
  batch    12 independent samples (volumes 128^3 .. 640x640x480, 2k-60k
           reflections each) in one persistent launch, autotuned and replayed
           from a CUDA graph
  highabs  1024x1024x800 volume, every crystal voxel (~11.7M), mu x5; timed on
           a reflection subset (--refl, default 2,000) of the 50,000

    python bench.py [--workload W] [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` is reflections/s of the whole job with
every input resident in device memory (kernel time, CUDA events on the
launching stream, L2 flushed between steps); `e2e` is the same metric through
the reference-facing C ABI (ray_tracing_overall) from pinned host buffers,
host set-up and both copies included.  `--impl reference` times the
reference's CPU implementation of the path on the host cores instead.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "reflections/s (plain FP64-step tracer, A_h per reflection)"
WORKLOADS = {
    "beamline": "beamline 512x512x400 int8 volume, stride-4 crystal voxels, 20000 reflections",
    "small": "96^3 int8 volume, all crystal voxels, 300 reflections",
    "batch": "12 samples 128^3..640x640x480, 2k-60k reflections each, one persistent launch (CUDA graph)",
    "highabs": "1024x1024x800 int8 volume, all crystal voxels, mu x5, reflection subset of 50000",
    "surrogate": "beamline sample; 4-member MLP ensemble trained on 100000 traced reflections (20000 Adam "
                 "steps, batch 4096); inference on 1000000 fresh reflections, 2% random audit + spread>1e-3 "
                 "re-traced by the plain kernel",
    "highabs_surrogate": "1024x1024x800 high-absorption sample, all crystal voxels; ensemble trained as for "
                         "the beamline sample; 50000 reflections with the 2% audit + spread fallback",
    "gridding": "beamline sample; absorption map 360 x 180 directions x 22917 voxels built on the GPU, then "
                "nearest-grid-point interpolation of 20000 reflections",
    "bisection": "1024x1024x800 high-absorption sample, all crystal voxels; iterative-bisection paths "
                 "(ib_test) on a reflection subset, beside the plain march",
}
DEFAULT_REFL = {"beamline": 20000, "small": 300, "batch": 0, "highabs": 2000, "surrogate": 1000000,
                "highabs_surrogate": 50000, "gridding": 20000, "bisection": 256}
SURROGATE_METRIC = "reflections/s (surrogate with audit: ensemble A_h, 2% random + high-spread re-traced)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="beamline", choices=sorted(WORKLOADS))
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--refl", type=int, default=None, help="reflections (single-sample workloads)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="N>1: the job is N x the workload's reflections (weak) or the workload itself (strong), "
                         "split over the ranks by anacor_public_gb300.shard")
    ap.add_argument("--no-cold-e2e", action="store_true", help="skip the e2e leg from a fresh process")
    ap.add_argument("--e2e-cold-child", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--batch-only", type=int, default=None,
                    help="batch: only sample K of the 12 (the same sample as in the full batch)")
    ap.add_argument("--stride-tune", action="store_true",
                    help="batch: choose each sample's voxel stride from {2, 4, 8} by its A_h deviation from "
                         "stride 1 on 64 reflections (tracer.choose_stride, tolerance 1e-3; under torchrun "
                         "each rank chooses on its own slice)")
    ap.add_argument("--config", default=None,
                    help="variant,tile,order for a single-sample plan instead of the autotuner (e.g. 8,1024,1)")
    ap.add_argument("--train-refl", type=int, default=100000, help="surrogate: traced training reflections")
    ap.add_argument("--train-steps", type=int, default=20000, help="surrogate: Adam steps")
    ap.add_argument("--train-batch", type=int, default=4096)
    ap.add_argument("--train-voxel-budget", type=int, default=1_500_000,
                    help="surrogate: the training labels are traced on the smallest crystal-voxel stride "
                         "(1, 2, 3, ...) that keeps at most this many voxels")
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--fourier-scale", default="auto",
                    help="surrogate Fourier feature scale, or 'auto' (chosen on held-out training rows)")
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--audit", type=float, default=0.02)
    ap.add_argument("--spread", type=float, default=1e-3)
    a = ap.parse_args()
    if a.refl is None:
        a.refl = DEFAULT_REFL[a.workload]
    return a


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def make_samples(args, rank: int = 0):
    from anacor_public_gb300 import synth
    w = args.workload
    if w == "beamline":
        ss = [synth.beamline_sample(n_refl=args.refl)]
    elif w == "small":
        ss = [synth.small_sample(n_refl=args.refl)]
    elif w == "highabs":
        ss = [synth.high_absorption_sample(n_refl=args.refl)]
    elif w == "surrogate":
        ss = [synth.beamline_sample()]
    elif w == "highabs_surrogate":
        ss = [synth.high_absorption_sample(n_refl=256)]
    elif w == "gridding":
        ss = [synth.beamline_sample(n_refl=args.refl)]
    elif w == "bisection":
        ss = [synth.high_absorption_sample(n_refl=args.refl)]
    else:
        ss = synth.batch_samples(n_samples=12, only=args.batch_only)
    if rank > 0:
        # weak scaling: every rank traces its own reflections through the same samples
        rng = np.random.default_rng(1000 + rank)
        out = []
        for s in ss:
            om, s1 = synth.reflections(s.n_refl, rng)
            t = s.subset()
            t.omega, t.s1 = om, s1
            out.append(t)
        ss = out
    return ss


def job_samples(args, rank: int, world: int):
    """The multi-rank job and this rank's share of it: (samples, job reflection
    counts).  With one rank the job is the workload itself.  With N ranks it
    is N x the workload's reflections (--scaling weak: the same samples, the
    reflections drawn once for the whole job) or the workload itself
    (--scaling strong); each rank takes its contiguous slice of every sample's
    reflections with shard.reflection_slice, the reference's --low/--up split
    (AnACor/main_lite.py:179-185)."""
    from anacor_public_gb300 import shard, synth
    ss = make_samples(args, 0)
    if world == 1:
        return ss, [s.n_refl for s in ss]
    out, job_n = [], []
    for k, s in enumerate(ss):
        t = s
        if args.scaling == "weak":
            om, s1 = synth.reflections(s.n_refl * world, np.random.default_rng(5000 + k), xray=s.xray)
            t = s.subset()
            t.omega, t.s1 = om, s1
        job_n.append(t.n_refl)
        out.append(t.subset(refl=shard.reflection_slice(t.n_refl, rank, world)))
    return out, job_n


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- helpers

def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(workload: str, key: str = "traffic_bytes_per_launch"):
    """A figure of the committed ncu summary of the absorption kernel (`key: value`
    line; DRAM bytes per launch by default), if any."""
    p = os.path.join(ROOT, "profiles", f"absorption_kernel_{workload}.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.strip().startswith(key + ":"):
            try:
                return float(ln.split(":", 1)[1])
            except ValueError:
                return None
    return None


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                             timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_runner(threads: int):
    """The reference algorithm on the host cores: the reference library where it
    was compiled from its sources, else the oracle port."""
    from oracle import oracle as orc
    if os.path.exists(orc.REF_SO):
        try:
            ref = orc.Reference()
            return (lambda sub: ref.overall(sub, num_workers=threads)), "reference"
        except OSError:
            pass
    orc.build_oracle()
    o = orc.Oracle()
    return (lambda sub: o.overall(sub, threads=threads)), "port"


def cpu_rate(s, seconds: float, runner, min_refl: int = 1):
    """Reflections/s of the CPU path on the first reflections of s, in chunks
    until `seconds` have elapsed."""
    chunk = max(os.cpu_count() or 1, 16) if len(s.coords) < 200000 else max(1, os.cpu_count() or 1)
    done, t0 = 0, time.perf_counter()
    while done < s.n_refl and (time.perf_counter() - t0 < seconds or done < min_refl):
        sub = s.subset(refl=slice(done, min(s.n_refl, done + chunk)))
        runner(sub)
        done += sub.n_refl
    return done / (time.perf_counter() - t0), done


def cpu_baseline(samples, seconds: float):
    threads = os.cpu_count() or 1
    runner, kind = cpu_runner(threads)
    if len(samples) == 1:
        s = samples[0]
        rate, n = cpu_rate(s, seconds, runner)
        return {"value": rate, "unit": "reflections/s", "cores": threads, "cpu_model": cpu_model(), "kind": kind,
                "sample": f"first {n} reflections of the workload x {len(s.coords)} voxels (2 rays each)"}
    # a batch: time a slice of every sample and add up the per-sample times
    per = max(0.5, seconds / len(samples))
    total_refl, total_sec, parts = 0, 0.0, []
    for s in samples:
        rate, n = cpu_rate(s, per, runner)
        total_refl += s.n_refl
        total_sec += s.n_refl / rate
        parts.append(n)
    return {"value": total_refl / total_sec, "unit": "reflections/s", "cores": threads, "cpu_model": cpu_model(), "kind": kind,
            "sample": f"per sample the first {min(parts)}..{max(parts)} reflections, extrapolated to all "
                      f"{total_refl} reflections of the {len(samples)} samples"}


# ----------------------------------------------------------- reference arm

def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    samples = make_samples(args)
    threads = os.cpu_count() or 1
    runner, kind = cpu_runner(threads)
    per_step = max(1.0, args.cpu_seconds / 2)
    for _ in range(args.warmup):
        cpu_rate(samples[0].subset(refl=slice(0, 4)), 0.2, runner)
    vals, counts = [], []
    t_all = time.perf_counter()
    for k in range(args.steps):
        total_refl, total_sec = 0, 0.0
        for s in samples:
            off = (k * 97) % max(1, s.n_refl - 8)
            rate, n = cpu_rate(s.subset(refl=slice(off, s.n_refl)), per_step / len(samples), runner)
            total_refl += s.n_refl
            total_sec += s.n_refl / rate
            counts.append(n)
        vals.append(total_refl / total_sec)
    wall = time.perf_counter() - t_all
    v = statistics.median(vals)
    n_vox = sum(len(s.coords) for s in samples)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "reflections/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "n_voxels": n_vox,
                   "n_reflections": sum(s.n_refl for s in samples),
                   "step": f"bounded sample: ~{per_step:.0f} s of reflections per step"},
        "voxel_rays_per_s": v * 2 * n_vox / len(samples),
        "cpu_baseline": {"value": v, "unit": "reflections/s", "cores": threads, "cpu_model": cpu_model(), "kind": kind,
                         "sample": f"{int(statistics.median(counts))} reflections per sample per step"},
        "e2e": {"value": v, "unit": "reflections/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ ours

def run_ours(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from anacor_public_gb300 import _lib, build, shard, tracer
    build.build()
    L = _lib.load()
    samples, job_n = job_samples(args, rank, world)
    stride_report = None
    if args.workload == "batch" and args.stride_tune:
        from anacor_public_gb300 import synth
        stride_report = []
        for s in samples:
            r = tracer.choose_stride(s.label, s.voxel, s.mu, s.s1, s.omega, s.xray, s.omega_axis, s.F,
                                     strides=(2, 4, 8), tol=1e-3)
            s.coords = synth.crystal_coords(s.label, r["stride"])
            c = r["candidates"].get(r["stride"], {})
            stride_report.append({"stride": r["stride"], "voxels": len(s.coords),
                                  "median_dev": c.get("median_dev"), "max_dev": c.get("max_dev")})
    n_refl = sum(s.n_refl for s in samples)
    n_vox = sum(len(s.coords) for s in samples)
    plans = [tracer.Plan.from_sample(s) for s in samples]
    total_steps = sum(p.count_steps() for p in plans)
    # a dedicated stream: the legacy default stream has handle 0, which the
    # library reads as "use the plan's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    batch = None
    if len(plans) > 1:
        batch = tracer.Batch(plans)
        if args.config:
            batch.configure(int(args.config.split(",")[0]))
        elif not args.no_autotune:
            batch.autotune()
        batch.capture(sh)
        run = lambda: batch.replay(sh)  # noqa: E731
        info = batch.info()
        grid, kernels = info["grid"], info["kernels"]
        tuned = {"variant": info["variant"], "kernels_per_run": info["kernels"],
                 "plan_variants": [p.config()["variant"] for p in plans], "tiles": [p.config()["tile"] for p in plans],
                 "order": [p.config()["order"] for p in plans], "cuda_graph": True,
                 "strides": stride_report}
    else:
        if args.config:
            plans[0].configure(*(int(x) for x in args.config.split(",")))
        elif not args.no_autotune:
            plans[0].autotune()
        tuned = plans[0].config()
        grid, kernels = plans[0].launch_info()
        run = lambda: plans[0].run(sh)  # noqa: E731
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    ref_result = [p.result(sh) for p in plans]

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    evs = []
    for _ in range(args.steps):
        flush.zero_()                      # L2 flush, outside the timed events
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = [a.elapsed_time(b) for a, b in evs]
    clk = clocks.stop()
    ms_step = sum(ms) / len(ms)
    if world > 1:
        t = torch.tensor([ms_step], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
    if batch is not None:
        batch.wait(sh)
    for p, r0 in zip(plans, ref_result):
        assert np.array_equal(p.result(sh), r0), "results changed between runs"
    value = sum(job_n) / (ms_step / 1e3)
    job_checksum = None
    if world > 1:
        # every rank's slice back to rank 0 (host gather, off the data path)
        g = torch.distributed.new_group(backend="gloo")
        full = [shard.gather_results(r0, n, rank, world, g) for r0, n in zip(ref_result, job_n)]
        if rank == 0:
            job_checksum = float(sum(np.sum(f) for f in full))
            assert all(np.isfinite(f).all() for f in full), "missing reflections in the gathered job"

    # e2e through the reference-facing C ABI, host buffers pinned
    e2e = None
    if not args.no_e2e:
        e2e = e2e_dropin(L, samples, args.steps, torch)
        if world > 1:
            t = torch.tensor([e2e["seconds"]], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e["value"] = sum(job_n) / float(t.item())
        e2e.pop("seconds", None)
        if world == 1 and not args.no_cold_e2e:
            e2e["cold_process"] = e2e_cold(args)

    if rank == 0:
        peak, src = measured_peak_gbs()
        alg_bytes = total_steps * 1 + sum(s.n_refl * len(s.coords) for s in samples) * 12
        achieved = alg_bytes / (ms_step / 1e3) / 1e9
        traffic = profiled_traffic(args.workload)
        lts = profiled_traffic(args.workload, "lts_bytes_per_launch")
        lts_pct = profiled_traffic(args.workload, "lts_throughput_pct")
        cpu = None if args.no_cpu_baseline else cpu_baseline(samples, args.cpu_seconds)
        line = {
            "metric": METRIC, "value": value, "unit": "reflections/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": args.scaling,
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "arith": "u8 labels, int32/32.32 fixed-point march (FP64 where a step is near a rounding boundary), "
                     "FP32 lengths and exp, FP64 reflection set-up and partial sums",
            "config": {"workload": WORKLOADS[args.workload], "n_samples": len(samples), "n_voxels": n_vox,
                       "n_reflections": sum(job_n), "reflections_per_rank": n_refl,
                       "sharding": ("shard.reflection_slice over the job's reflections, results gathered to "
                                    "rank 0" if world > 1 else None), "job_checksum": job_checksum,
                       "volume": [list(s.label.shape) for s in samples][:3],
                       "l2": "flushed between steps (256 MiB write)", "grid": grid, "block": 256,
                       "tuned": tuned},
            "voxel_rays_per_s": 2.0 * sum(n * len(s.coords) for s, n in zip(samples, job_n)) / (ms_step / 1e3),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": src, "traffic": traffic,
                         "alg_bytes_per_launch": alg_bytes, "label_steps_per_launch": total_steps,
                         # the level the label gathers are served from (ncu summary in profiles/)
                         "l2": {"traffic": lts, "achieved_gbs": (lts / (ms_step / 1e3) / 1e9) if lts else None,
                                "lts_throughput_pct": lts_pct}},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": args.steps * kernels,
        }
        print(json.dumps(line), flush=True)
    if batch is not None:
        batch.close()
    for p in plans:
        p.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def e2e_dropin(L, samples, steps, torch):
    """ray_tracing_overall (the reference's entry point) from pinned host
    memory, one call per sample, as AnACor's worker makes it."""
    import ctypes as ct
    from anacor_public_gb300.worker import python_2_c_3d
    prepared = []
    h2d = 0
    for s in samples:
        vol = torch.empty(s.label.shape, dtype=torch.int8).pin_memory().numpy()
        vol[...] = s.label
        coords = torch.from_numpy(s.coords).pin_memory().numpy()
        s1 = torch.from_numpy(s.s1).pin_memory().numpy()
        om = torch.from_numpy(s.omega).pin_memory().numpy()
        tab, keep = python_2_c_3d(vol)
        prepared.append((s, vol, coords, s1, om, tab, keep))
        h2d += s.label.nbytes + s.coords.nbytes + s.n_refl * 864
    times = []
    checksum = 0.0
    for k in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s, vol, coords, s1, om, tab, keep in prepared:
            n = s.n_refl
            res = L.ray_tracing_overall(0, n, coords, len(coords), s1, om, s.xray, s.omega_axis, s.F, n, s.voxel,
                                        s.mu, tab, s.shape, 0, 0, os.cpu_count() or 1, 1)
            if not res:
                raise RuntimeError(L.anacor_last_error())
            out = np.ctypeslib.as_array(res, shape=(n,)).copy()
            L.free(ct.cast(res, ct.c_void_p))
            checksum += float(out.sum()) if k == 0 else 0.0
        torch.cuda.synchronize()
        if k > 0:
            times.append(time.perf_counter() - t0)
    sec = sum(times) / len(times)
    n_refl = sum(s.n_refl for s in samples)
    return {"value": n_refl / sec, "unit": "reflections/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(n_refl * 8 + 4 * len(samples)),
            "path": "ray_tracing_overall (C ABI, int8*** table), one call per sample", "seconds": sec,
            "checksum": checksum}


def e2e_cold(args):
    """ray_tracing_overall from a fresh process (empty tuning cache: the
    library's default configuration rule, as a new AnACor worker process sees
    it): the first call (CUDA context, module load, device tables) and the
    steady calls after it."""
    cmd = [sys.executable, os.path.abspath(__file__), "--e2e-cold-child", "--workload", args.workload,
           "--steps", str(args.steps)]
    if args.refl is not None:
        cmd += ["--refl", str(args.refl)]
    try:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=900)
        for ln in r.stdout.splitlines()[::-1]:
            if ln.startswith("{"):
                return json.loads(ln)
        return {"error": (r.stderr or r.stdout)[-300:]}
    except Exception as ex:   # the leg is informative; its failure does not void the line
        return {"error": str(ex)[:300]}


def e2e_cold_child(args):
    import ctypes as ct
    t_start = time.perf_counter()
    from anacor_public_gb300 import _lib
    from anacor_public_gb300.worker import python_2_c_3d
    samples = make_samples(args)
    L = _lib.load()
    prepared = [(s, python_2_c_3d(np.ascontiguousarray(s.label))) for s in samples]
    times = []
    for k in range(args.steps + 1):
        t0 = time.perf_counter()
        for s, (tab, keep) in prepared:
            n = s.n_refl
            res = L.ray_tracing_overall(0, n, s.coords, len(s.coords), s.s1, s.omega, s.xray, s.omega_axis, s.F, n,
                                        s.voxel, s.mu, tab, s.shape, 0, 0, os.cpu_count() or 1, 1)
            if not res:
                raise RuntimeError(L.anacor_last_error())
            L.free(ct.cast(res, ct.c_void_p))
        times.append(time.perf_counter() - t0)
    n_refl = sum(s.n_refl for s in samples)
    steady = times[1:] or times
    print(json.dumps({"first_call_s": times[0], "value": n_refl / (sum(steady) / len(steady)),
                      "unit": "reflections/s", "process_start_to_first_result_s": time.perf_counter() - t_start
                      - sum(times[1:]), "calls": len(times)}), flush=True)


def _quantiles(e):
    e = np.asarray(e, dtype=np.float64)
    if e.size == 0:
        return None
    return {"n": int(e.size), "median": float(np.median(e)), "p90": float(np.quantile(e, 0.9)),
            "p99": float(np.quantile(e, 0.99)), "max": float(e.max())}


def run_surrogate(args):
    """Surrogate with audit on one sample: trace a training set with the plain
    kernel, train the ensemble, then time inference over fresh reflections with
    the audit rows and the high-spread rows re-traced."""
    import ctypes as ct
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from anacor_public_gb300 import _lib, build, surrogate, synth, tracer
    build.build()
    L = _lib.load()
    s = make_samples(args, rank)[0]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    plan = tracer.Plan(s.label, s.coords, s.voxel, s.mu)
    plan.set_reflections(s.s1, s.omega, s.xray, s.omega_axis, s.F)
    if not args.no_autotune:
        plan.autotune()
    tuned = plan.config()

    # training labels: the plain kernel on the smallest voxel stride within the
    # budget (every voxel on the beamline sample; the audit below measures the
    # error against the full voxel list either way)
    t_setup0 = time.perf_counter()
    stride = 1
    while len(s.coords) / stride ** 3 > args.train_voxel_budget:
        stride += 1
    if stride > 1:
        sub = s.coords[np.all(s.coords % stride == 0, axis=1)]
        plan_t = tracer.Plan(s.label, sub, s.voxel, s.mu)
        plan_t.set_reflections(s.s1[:64], s.omega[:64], s.xray, s.omega_axis, s.F)
        if not args.no_autotune:
            plan_t.autotune()
    else:
        plan_t = plan
    rng = np.random.default_rng(17 + rank)
    om_t, s1_t = synth.reflections(args.train_refl, rng, xray=s.xray)
    plan_t.set_reflections(s1_t, om_t, s.xray, s.omega_axis, s.F)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plan_t.run(sh)
    e1.record(stream)
    ah_t = plan_t.result(sh)
    trace_ms = e0.elapsed_time(e1)
    train_label_err = None
    if stride > 1:
        # what the stride costs: the first 256 training labels against every voxel
        plan.set_reflections(s1_t[:256], om_t[:256], s.xray, s.omega_axis, s.F)
        plan.run(sh)
        train_label_err = _quantiles(surrogate.relative_error(ah_t[:256], plan.result(sh)))
        n_train_vox = len(sub)
        plan_t.close()
    else:
        n_train_vox = len(s.coords)
    t_setup_trace = time.perf_counter() - t_setup0
    # the plain kernel at full resolution on fresh reflections: the reference
    # point of the speed-ups (the whole inference set where that is quick)
    n_plain = args.refl if len(s.coords) * args.refl <= 2e10 else max(2000, min(args.refl, 20000))
    om_p, s1_p = synth.reflections(n_plain, np.random.default_rng(3000 + rank), xray=s.xray)
    plan.set_reflections(s1_p, om_p, s.xray, s.omega_axis, s.F)
    plan.run(sh)
    plain_ms = statistics.median(_events_ms(torch, stream, lambda: plan.run(sh), 3))
    plain_rate = n_plain / (plain_ms / 1e3)
    x7_t = surrogate.inputs(om_t, s1_t, s.xray, s.omega_axis, s.F)
    t0 = time.perf_counter()
    if args.fourier_scale == "auto":
        fscale, fscores = surrogate.select_fourier_scale(x7_t, np.log(ah_t), members=args.members, seed=1 + rank,
                                                         lr_max=args.lr, spread_threshold=args.spread)
    else:
        fscale, fscores = float(args.fourier_scale), {}
    select_s = time.perf_counter() - t0
    model = surrogate.Surrogate(members=args.members, seed=1 + rank, fourier_scale=fscale)
    model.set_data(x7_t, np.log(ah_t))
    t0 = time.perf_counter()
    loss = model.train(args.train_steps, batch=args.train_batch, lr_max=args.lr, lr_min=args.lr * 1e-2,
                       total_steps=args.train_steps)
    train_s = time.perf_counter() - t0

    # fresh reflections, resident on the device
    n = args.refl
    om_i, s1_i = synth.reflections(n, np.random.default_rng(1000 + rank), xray=s.xray)
    d_om = torch.from_numpy(om_i).to("cuda")
    d_s1 = torch.from_numpy(s1_i).to("cuda")
    d_x7 = torch.empty((n, 7), dtype=torch.float32, device="cuda")
    d_mean = torch.empty(n, dtype=torch.float32, device="cuda")
    d_spread = torch.empty(n, dtype=torch.float32, device="cuda")
    d_flags = torch.empty(n, dtype=torch.uint8, device="cuda")
    d_out = torch.empty(n, dtype=torch.float64, device="cuda")
    geo = (np.ascontiguousarray(s.xray, dtype=np.float64), np.ascontiguousarray(s.omega_axis, dtype=np.float64),
           np.ascontiguousarray(s.F, dtype=np.float64).reshape(-1))
    record = {}

    def step(k, host=None):
        if host is not None:   # e2e: this step's inputs arrive from pinned host memory
            d_om.copy_(host[0], non_blocking=True)
            d_s1.copy_(host[1], non_blocking=True)
        _lib.check(L.anacor_surrogate_inputs_device(ct.c_void_p(d_om.data_ptr()), ct.c_void_p(d_s1.data_ptr()), n,
                                                    *geo, ct.c_void_p(d_x7.data_ptr()), ct.c_void_p(sh)), L)
        model.predict_device(d_x7.data_ptr(), n, d_mean.data_ptr(), d_spread.data_ptr(), sh)
        surrogate.audit_flags(d_spread.data_ptr(), n, 100 + k, args.audit, args.spread, d_flags.data_ptr(), sh)
        d_out.copy_(d_mean)
        flags = d_flags.cpu().numpy()            # synchronises the stream
        idx = np.nonzero(flags)[0]
        if idx.size:
            plan.set_reflections(s1_i[idx], om_i[idx], s.xray, s.omega_axis, s.F)
            plan.run(sh)
            traced = torch.from_numpy(plan.result(sh)).to("cuda", non_blocking=True)
            d_out.index_copy_(0, torch.from_numpy(idx).to("cuda", non_blocking=True), traced)
        else:
            traced = None
        record.update(flags=flags, idx=idx, traced=traced)
        if host is not None:
            host[2].copy_(d_out, non_blocking=True)
        return idx.size

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    # accuracy of this pass (the audit rows: surrogate vs traced)
    err_sur, err_out, fallback, n_traced = [], [], [], []

    def account():
        fl, idx = record["flags"], record["idx"]
        tr = record["traced"].cpu().numpy() if record["traced"] is not None else np.zeros(0)
        mean = d_mean.cpu().numpy().astype(np.float64)
        aud = (fl[idx] & 1) != 0
        e = np.abs(mean[idx[aud]] - tr[aud]) / np.abs(tr[aud])
        err_sur.append(e)
        err_out.append(np.where((fl[idx[aud]] & 2) != 0, 0.0, e))   # fallback rows leave the output exact
        fallback.append(float(np.mean((fl & 2) != 0)))
        n_traced.append(int(idx.size))

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms = []
    for k in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(args.warmup + k)
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
        account()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_step = sum(ms) / len(ms)
    if world > 1:
        t = torch.tensor([ms_step], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
    value = n * world / (ms_step / 1e3)
    # amortised: one batch of n reflections served from scratch -- training
    # labels traced, Fourier scale chosen, ensemble trained, then the audited
    # inference -- against the plain kernel on all n
    setup_s = t_setup_trace + select_s + train_s
    amortised = n / (setup_s + ms_step / 1e3)

    # the network alone: inputs + ensemble inference over the n rows
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.zero_()
    a.record(stream)
    model.predict_device(d_x7.data_ptr(), n, d_mean.data_ptr(), d_spread.data_ptr(), sh)
    b.record(stream)
    b.synchronize()
    infer_ms = a.elapsed_time(b)
    flops_row = 2 * (64 * 256 + 3 * 256 * 256 + 256) * args.members
    tflops = flops_row * n / (infer_ms / 1e3) / 1e12

    e2e = None
    if not args.no_e2e:
        h_om = torch.from_numpy(om_i).pin_memory()
        h_s1 = torch.from_numpy(s1_i).pin_memory()
        h_out = torch.empty(n, dtype=torch.float64).pin_memory()
        tt = []
        for k in range(args.steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step(500 + k, host=(h_om, h_s1, h_out))
            stream.synchronize()
            if k:
                tt.append(time.perf_counter() - t0)
        e2e = {"value": n / (sum(tt) / len(tt)), "unit": "reflections/s",
               "h2d_bytes_per_step": int(n * 32), "d2h_bytes_per_step": int(n * 9),
               "path": "surrogate.audited pipeline from pinned host omega / s1 to host A_h"}
        if world > 1:
            t = torch.tensor([sum(tt) / len(tt)], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e["value"] = n * world / float(t.item())

    if rank == 0:
        peak_tf = None
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            with open(pk) as f:
                peak_tf = float(json.load(f).get("bf16_tflops", 0)) or None
        cpu = None if args.no_cpu_baseline else cpu_baseline([s], args.cpu_seconds)
        es, eo = np.concatenate(err_sur), np.concatenate(err_out)
        line = {
            "metric": SURROGATE_METRIC, "value": value, "unit": "reflections/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "n_voxels": len(s.coords), "n_reflections": n,
                       "volume": list(s.label.shape), "members": args.members, "train_refl": args.train_refl,
                       "train_steps": args.train_steps, "train_batch": args.train_batch,
                       "audit_fraction": args.audit, "spread_threshold": args.spread,
                       "l2": "flushed between steps (256 MiB write)", "tuned": tuned},
            "plain_refl_per_s": plain_rate,
            "plain_sample": f"{n_plain} fresh reflections x {len(s.coords)} voxels (every voxel)",
            "speedup_vs_plain": value / plain_rate,
            "amortised": {"value": amortised, "unit": "reflections/s", "vs_plain": amortised / plain_rate,
                          "served": n, "setup_s": setup_s,
                          "what": "n reflections from scratch: training labels traced + Fourier-scale "
                                  "selection + training + one audited inference pass"},
            "surrogate": {"train_s": train_s, "train_trace_s": trace_ms / 1e3, "fourier_scale": fscale,
                          "train_voxel_stride": stride, "train_voxels": n_train_vox,
                          "train_setup_s": t_setup_trace, "train_label_rel_err": train_label_err,
                          "scale_selection_s": select_s,
                          "scale_scores": {str(k): {"fallback": v[0], "median_err": v[1]} for k, v in fscores.items()},
                          "final_loss": float(np.mean(loss[-100:])), "first_loss": float(np.mean(loss[:10])),
                          "fallback_fraction": float(np.mean(fallback)), "traced_per_step": int(np.mean(n_traced)),
                          "surrogate_rel_err": _quantiles(es), "output_rel_err": _quantiles(eo),
                          "inference_ms": infer_ms, "inference_tflops": tflops},
            "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak_tf, "unit": "TFLOP/s",
                         "frac": (tflops / peak_tf) if peak_tf else None, "traffic": None,
                         "kernel": "ensemble inference (tcgen05 GEMMs + fused bias/GELU epilogues)"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            # per step: inputs, per 262144-row chunk features + 4 GEMMs + head + ensemble,
            # audit flags, the absorption launch(es) of the traced rows
            "gpu_launches": args.steps * (2 + 7 * (-(-n // 262144)) + plan.launch_info()[1]),
        }
        print(json.dumps(line), flush=True)
    model.close()
    plan.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def _events_ms(torch, stream, fn, reps: int, flush=None):
    ms = []
    for _ in range(reps):
        if flush is not None:
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    return ms


def run_modes(args):
    """The gridding and bisection rows: their own throughput on the device,
    beside the plain march on the same sample, and their error against it."""
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    from anacor_public_gb300 import build, gridding, tracer
    build.build()
    s = make_samples(args, rank)[0]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    plan = tracer.Plan.from_sample(s)
    if not args.no_autotune:
        plan.autotune()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    n, n_vox = s.n_refl, len(s.coords)
    e2e = None
    # the plain march on the same reflections (reference point and error baseline)
    for _ in range(args.warmup):
        plan.run(sh)
    plain_ms = statistics.median(_events_ms(torch, stream, lambda: plan.run(sh), args.steps, flush))
    plain = plan.result(sh)
    extra = {}
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if args.workload == "gridding":
        g = gridding.GriddingMap(plan, 360, 180)
        t0 = time.perf_counter()
        g.build()
        build_s = time.perf_counter() - t0
        d_out = torch.empty(n, dtype=torch.float64, device="cuda")
        g.prepare(s.s1, s.omega, s.xray, s.omega_axis, s.F)
        run = lambda: g.run(d_out.data_ptr(), sh)  # noqa: E731
        for _ in range(args.warmup):
            run()
        ms = _events_ms(torch, stream, run, args.steps, flush)
        approx = d_out.cpu().numpy()
        # end to end: host reflections in, host A_h out (host lookups, copies, kernel)
        tt = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g.interpolate(s.s1, s.omega, s.xray, s.omega_axis, s.F)
            tt.append(time.perf_counter() - t0)
        e2e = {"value": n / statistics.median(tt), "unit": "reflections/s", "h2d_bytes_per_step": int(n * 128),
               "d2h_bytes_per_step": int(n * 8), "path": "anacor_gridding_interpolate from host arrays"}
        map_rays = g.n_dirs * n_vox
        extra = {"map_build_s": build_s, "map_directions": g.n_dirs, "map_rays_per_s": map_rays / build_s,
                 "map_bytes": int(g.n_dirs * g.device_map()[1] * 4)}
        alg_bytes = n * n_vox * 2 * 4
        g.close()
        kernels = 1
    else:
        run = lambda: plan.run_bisection(4, sh)  # noqa: E731
        for _ in range(args.warmup):
            run()
        ms = _events_ms(torch, stream, run, args.steps, flush)
        approx = plan.result(sh)
        alg_bytes = None
        kernels = 1
    clk = clocks.stop()
    ms_step = statistics.median(ms)
    value = n / (ms_step / 1e3)
    err = np.abs(approx - plain) / plain
    if rank == 0:
        peak, src = measured_peak_gbs()
        achieved = alg_bytes / (ms_step / 1e3) / 1e9 if alg_bytes else None
        line = {
            "metric": f"reflections/s ({args.workload} mode, A_h per reflection)", "value": value,
            "unit": "reflections/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "n_voxels": n_vox, "n_reflections": n,
                       "volume": list(s.label.shape), "l2": "flushed between steps (256 MiB write)"},
            "plain_refl_per_s": n / (plain_ms / 1e3), "speedup_vs_plain": plain_ms / ms_step,
            "rel_err_vs_plain": _quantiles(err),
            **extra,
            "roofline": ({"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                          "peak_source": src, "traffic": None,
                          "alg_bytes_per_launch": alg_bytes, "kernel": "gridding_interp_kernel"}
                         if achieved else None),
            "cpu_baseline": None,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": args.steps * kernels,
        }
        print(json.dumps(line), flush=True)
    plan.close()


def main():
    args = parse()
    if args.e2e_cold_child:
        e2e_cold_child(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload in ("surrogate", "highabs_surrogate"):
        run_surrogate(args)
    elif args.workload in ("gridding", "bisection"):
        run_modes(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
