"""Benchmark of the plain GPU absorption tracer.

Workload: the beamline sample -- 512x512x400 int8 label volume (the synthetic
recipe scaled x5: crystal ellipsoid 100/70/50 voxels, liquor shell, loop,
bubbles), crystal voxels sampled at stride 4 on each axis (~23k voxels) and
20,000 reflections (omega ~ U[0, 2pi), 2theta ~ U[5, 120] deg), two rays per
(voxel, reflection).  One step = one pass of the path over all reflections.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

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

WORKLOAD = "beamline 512x512x400 int8 volume, stride-4 crystal voxels, 20000 reflections"
METRIC = "reflections/s (plain FP64-step tracer, A_h per reflection)"
N_REFL = 20000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--refl", type=int, default=N_REFL)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


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


def profiled_traffic_per_reflection():
    """DRAM bytes per reflection of the absorption kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "absorption_kernel_beamline.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.strip().startswith("traffic_bytes_per_reflection:"):
            try:
                return float(ln.split(":", 1)[1])
            except ValueError:
                return None
    return None


def cpu_baseline_sample(s, seconds: float):
    """Reference algorithm (the oracle port, or the reference library where it
    was compiled from its sources) on the host cores: reflections in chunks
    until `seconds` have elapsed.  Returns (refl/s, reflections timed, kind, threads)."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    kind = "port"
    runner = None
    if os.path.exists(orc.REF_SO):
        try:
            ref = orc.Reference()
            runner = lambda sub: ref.overall(sub, num_workers=threads)  # noqa: E731
            kind = "reference"
        except OSError:
            runner = None
    if runner is None:
        orc.build_oracle()
        o = orc.Oracle()
        runner = lambda sub: o.overall(sub, threads=threads)  # noqa: E731
    chunk = max(threads, 16)
    done, t0 = 0, time.perf_counter()
    while done < s.n_refl and time.perf_counter() - t0 < seconds:
        sub = s.subset(refl=slice(done, min(s.n_refl, done + chunk)))
        runner(sub)
        done += sub.n_refl
    dt = time.perf_counter() - t0
    return done / dt, done, kind, threads


# ----------------------------------------------------------- reference arm

def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from anacor_public_gb300 import synth
    s = synth.beamline_sample(n_refl=args.refl)
    per_step = max(1.0, args.cpu_seconds / 2)
    for _ in range(args.warmup):
        cpu_baseline_sample(s.subset(refl=slice(0, 32)), 0.5)
    vals, counts = [], []
    kind = threads = None
    t_all = time.perf_counter()
    for k in range(args.steps):
        off = (k * 97) % max(1, s.n_refl - 64)
        rate, n, kind, threads = cpu_baseline_sample(s.subset(refl=slice(off, s.n_refl)), per_step)
        vals.append(rate)
        counts.append(n)
    wall = time.perf_counter() - t_all
    v = statistics.median(vals)
    n_vox = len(s.coords)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "reflections/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_voxels": n_vox, "n_reflections": s.n_refl,
                   "step": f"bounded sample: ~{per_step:.0f} s of reflections per step"},
        "voxel_rays_per_s": v * 2 * n_vox,
        "cpu_baseline": {"value": v, "unit": "reflections/s", "cores": threads, "kind": kind,
                         "sample": f"{int(statistics.median(counts))} reflections x {n_vox} voxels per step"},
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
    from anacor_public_gb300 import build, synth, tracer
    from anacor_public_gb300 import _lib
    build.build()
    L = _lib.load()
    # weak scaling: every rank traces its own 20k reflections through the same sample
    s = synth.beamline_sample(n_refl=args.refl)
    if world > 1:
        rng = np.random.default_rng(1000 + rank)
        om, s1 = synth.reflections(args.refl, rng)
        s = s.subset()
        s.omega, s.s1 = om, s1
    n_vox = len(s.coords)
    plan = tracer.Plan.from_sample(s)
    total_steps = plan.count_steps()
    grid, kernels = plan.launch_info()
    # a dedicated stream: the legacy default stream has handle 0, which the
    # library reads as "use the plan's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    assert sh != 0
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        plan.run(sh)
    torch.cuda.synchronize()
    ref_result = plan.result(sh)

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
        plan.run(sh)
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
    got = plan.result(sh)
    assert np.array_equal(got, ref_result), "results changed between runs"
    value = s.n_refl * world / (ms_step / 1e3)

    # e2e through the reference-facing C ABI, host buffers pinned
    e2e = None
    if not args.no_e2e:
        e2e = e2e_dropin(L, s, args.steps, torch)
        if world > 1:
            t = torch.tensor([e2e["seconds"]], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e["value"] = s.n_refl * world / float(t.item())
        e2e.pop("seconds", None)

    if rank == 0:
        peak, src = measured_peak_gbs()
        alg_bytes = total_steps * 1 + s.n_refl * n_vox * 12
        achieved = alg_bytes / (ms_step / 1e3) / 1e9
        tpr = profiled_traffic_per_reflection()
        cpu = None
        if not args.no_cpu_baseline:
            rate, n, kind, threads = cpu_baseline_sample(s, args.cpu_seconds)
            cpu = {"value": rate, "unit": "reflections/s", "cores": threads, "kind": kind,
                   "sample": f"first {n} reflections of the workload x {n_vox} voxels (all voxels, 2 rays each)"}
        line = {
            "metric": METRIC, "value": value, "unit": "reflections/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_voxels": n_vox, "n_reflections": s.n_refl,
                       "volume": list(s.label.shape), "l2": "flushed between steps (256 MiB write)",
                       "grid": grid, "block": 256},
            "voxel_rays_per_s": value * 2 * n_vox,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": src,
                         "traffic": (tpr * s.n_refl) if tpr else None,
                         "alg_bytes_per_launch": alg_bytes, "label_steps_per_launch": total_steps},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": args.steps * kernels,
        }
        print(json.dumps(line), flush=True)
    plan.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def e2e_dropin(L, s, steps, torch):
    """ray_tracing_overall (the reference's entry point) from pinned host memory."""
    import ctypes as ct
    from anacor_public_gb300.worker import python_2_c_3d
    vol_t = torch.empty(s.label.shape, dtype=torch.int8).pin_memory()
    vol = vol_t.numpy()
    vol[...] = s.label
    coords = torch.from_numpy(s.coords).pin_memory().numpy()
    s1 = torch.from_numpy(s.s1).pin_memory().numpy()
    om = torch.from_numpy(s.omega).pin_memory().numpy()
    tab, keep = python_2_c_3d(vol)
    n = s.n_refl
    times = []
    for k in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = L.ray_tracing_overall(0, n, coords, len(coords), s1, om, s.xray, s.omega_axis, s.F, n, s.voxel,
                                    s.mu, tab, s.shape, 0, 0, os.cpu_count() or 1, 1)
        if not res:
            raise RuntimeError(L.anacor_last_error())
        out = np.ctypeslib.as_array(res, shape=(n,)).copy()
        L.free(ct.cast(res, ct.c_void_p))
        torch.cuda.synchronize()
        if k > 0:
            times.append(time.perf_counter() - t0)
    sec = sum(times) / len(times)
    del keep
    h2d = s.label.nbytes + s.coords.nbytes + n * 864
    return {"value": n / sec, "unit": "reflections/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(n * 8 + 4), "path": "ray_tracing_overall (C ABI, int8*** table)",
            "seconds": sec, "checksum": float(out.sum())}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
