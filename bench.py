"""Benchmark of the GB300 OSEM hot path; prints ONE JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sc3] [--no-cpu-baseline] [--no-e2e]

Workload "sc3" (default): the SC channel of the JSCCSD joint configuration — dense
system matrix of 20 views x 4,096 pixels = 81,920 bins x 36,000 voxels (100 x 360
polar grid), 8 OSEM subsets. One step = one OSEM iteration (8 subset updates:
forward projection, ratio, back projection, EM update). Metric: subset-iterations/s
(higher is better), headline with the matrix stored in BF16 (FP32 accumulation),
the plain FP32-stored run reported beside it. Inputs are synthetic (seeded) and the
matrix (5.9 GB BF16 / 11.8 GB FP32) is far larger than L2, so no L2 flush is needed
between timed iterations.

Multi-GPU: the path is run as independent replicas (one per rank, no collective on
the data path); `value` sums the replicas' subset-iterations over the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np
import torch

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

FALLBACK_HBM_GBS = 6800.0


# ----------------------------------------------------------------------------- utilities
def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": FALLBACK_HBM_GBS, "source": "fallback"}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
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
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ----------------------------------------------------------------------------- workload
class Sc3Workload:
    """SC channel of config 3 (flat form: all 20 views are rows of one matrix)."""

    name = "jsccsd-config3-sc-channel"

    def __init__(self, device, n_r=100, n_theta=360, radius=100.0, det_radius=120.0, n_phi=128, n_axial=32,
                 axial_pitch=2.0, views=20, subsets=8, counts=1e7, seed=None):
        if views != 20 or subsets != 8:
            self.name = f"sc-channel-{views}views-{subsets}subsets"
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop
        from jscc_recon_spect_cylinder_gb300 import synthetic

        self.dev = device
        self.subsets = subsets
        seed = synthetic.SEED if seed is None else seed
        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
        grid = synthetic.polar_grid(n_r, n_theta, radius, device=device)
        self.V = grid.n_vox
        pitch = 2.0 * math.pi * det_radius / n_phi
        blocks = []
        for v in range(views):
            pos = synthetic.cylinder_pixels(det_radius, n_phi, n_axial, axial_pitch, phi0=2 * math.pi * v / views,
                                            device=device)
            blocks.append(synthetic.sc_system_matrix(grid.coor, pos, pitch * axial_pitch, radius, generator=gen))
        A = torch.cat(blocks, dim=0)
        del blocks
        self.B = A.size(0)
        x_true = synthetic.hot_rod_phantom(grid.coor.cpu(), radius).to(device)
        self.proj = synthetic.poisson_projection(A, x_true, counts, generator=gen)
        self.s_map = A.sum(dim=0, keepdim=True).transpose(0, 1).contiguous()
        gcpu = torch.Generator().manual_seed(seed)
        perm = torch.randperm(self.B, generator=gcpu)
        self.subset_ids = [ids.to(device) for ids in rop.split_tensor_even(perm, subsets, dim=0)]
        self.A_f32 = [A[ids].contiguous() for ids in self.subset_ids]
        del A
        self.A_bf16 = [a.to(torch.bfloat16) for a in self.A_f32]
        self.y = [self.proj[ids].contiguous() for ids in self.subset_ids]
        self.rot = torch.arange(1, self.V + 1, dtype=torch.int64, device=device).unsqueeze(1)
        self.inv = self.rot.clone()
        self.rows_per_subset = [a.size(0) for a in self.A_f32]
        torch.cuda.synchronize(device)

    def matrices(self, dtype):
        return self.A_bf16 if dtype == "bf16" else self.A_f32

    def step(self, img, dtype):
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

        A = self.matrices(dtype)
        return rop.osem_bin_mode([[a] for a in A], [[y] for y in self.y], [self.rot], [self.inv], img, self.s_map, 1)

    def units_per_step(self):
        return self.subsets

    def kernel_bytes(self, dtype):
        """Algorithmic bytes per launch of the streaming kernels, averaged over subsets."""
        b = 2 if dtype == "bf16" else 4
        rows = float(np.mean(self.rows_per_subset))
        mat = rows * self.V * b
        return {
            "sc_forward_split": mat + self.V * 4,   # A once + image
            "sc_back_partial": mat + rows * 4,      # A once + ratio
        }

    def bytes_per_step(self, dtype):
        kb = self.kernel_bytes(dtype)
        return self.subsets * (kb["sc_forward_split"] + kb["sc_back_partial"])


def make_workload(name, dev):
    if name == "sc3":
        return Sc3Workload(dev)
    if name == "sc3-small":  # profiling case: 2 views (8,192 x 36,000), one subset; > L2
        return Sc3Workload(dev, views=2, subsets=1)
    raise ValueError(name)


# ----------------------------------------------------------------------------- timing
def timed_steps(work, dtype, steps, warmup, world):
    img = torch.ones((work.V, 1), device=work.dev)
    for _ in range(warmup):
        img = work.step(img, dtype)
    torch.cuda.synchronize(work.dev)
    if world > 1:
        torch.distributed.barrier()
    stream = torch.cuda.current_stream(work.dev)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    from jscc_recon_spect_cylinder_gb300 import _lib

    n0 = _lib.launch_count()
    t0.record(stream)
    for _ in range(steps):
        img = work.step(img, dtype)
    t1.record(stream)
    torch.cuda.synchronize(work.dev)
    launches = _lib.launch_count() - n0
    if world > 1:
        torch.distributed.barrier()
    ms = t0.elapsed_time(t1)
    if world > 1:
        t = torch.tensor([ms], device=work.dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, launches, img


def kernel_times(work, dtype, steps):
    """Per-kernel CUDA-event durations on the launch stream (separate instrumented pass)."""
    from jscc_recon_spect_cylinder_gb300 import _lib

    img = torch.ones((work.V, 1), device=work.dev)
    img = work.step(img, dtype)
    torch.cuda.synchronize(work.dev)
    _lib.kernel_timing_collect()
    _lib.kernel_timing_enable(True)
    for _ in range(steps):
        img = work.step(img, dtype)
    torch.cuda.synchronize(work.dev)
    _lib.kernel_timing_enable(False)
    return _lib.kernel_timing_collect()


def fp64_errors(work, iters, images):
    """Relative L2 and max-voxel error of each image against an FP64 reconstruction of
    the same problem (torch float64 on the GPU, same subsets, same order)."""
    x = torch.ones((work.V, 1), dtype=torch.float64, device=work.dev)
    s = work.s_map.double()
    for _ in range(iters):
        for A, y in zip(work.A_f32, work.y):
            A64 = A.double()
            w = A64.t() @ (y.double() / (A64 @ x))
            x = x * w / s
            del A64
    out = {}
    for k, img in images.items():
        d = (img.double() - x)
        out[k] = {"rel_l2": float(d.norm() / x.norm()), "max_voxel_rel": float(d.abs().max() / x.abs().max())}
    return out


def run_e2e(work, dtype, iters):
    """One reconstruction job through the reference-facing API with host inputs:
    pinned host subset matrices, projections and sensitivity are copied to the GPU
    inside the timed region, `iters` OSEM iterations run, and the image is read back."""
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    host_A = [a.cpu().pin_memory() for a in work.matrices(dtype)]
    host_y = [y.cpu().pin_memory() for y in work.y]
    host_s = work.s_map.cpu().pin_memory()
    host_img = torch.ones((work.V, 1)).pin_memory()
    out = torch.empty((work.V, 1)).pin_memory()
    h2d = sum(a.numel() * a.element_size() for a in host_A) + sum(y.numel() * 4 for y in host_y) + \
        host_s.numel() * 4 + host_img.numel() * 4
    d2h = out.numel() * 4
    torch.cuda.synchronize(work.dev)
    t0 = time.perf_counter()
    A = [[a.to(work.dev, non_blocking=True)] for a in host_A]
    y = [[v.to(work.dev, non_blocking=True)] for v in host_y]
    s = host_s.to(work.dev, non_blocking=True)
    img = host_img.to(work.dev, non_blocking=True)
    rot = torch.arange(1, work.V + 1, dtype=torch.int64).unsqueeze(1).to(work.dev, non_blocking=True)
    for _ in range(iters):
        img = rop.osem_bin_mode(A, y, [rot], [rot], img, s, 1)
    out.copy_(img, non_blocking=True)
    torch.cuda.synchronize(work.dev)
    sec = time.perf_counter() - t0
    return {"value": iters * work.subsets / sec, "unit": "subset-iters/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "step": f"one job: stage inputs + {iters} iterations + read image",
            "seconds": sec}


def cpu_port_rate(work, budget_s=10.0, threads=None):
    """Oracle (numpy port of recon_osem_plane.get_weight_single + EM update) on the
    host cores: subset updates of the same workload until ~budget_s of CPU work."""
    from oracle import osem_sc

    A = work.A_f32[0].cpu().numpy()
    y = work.y[0].cpu().numpy()
    s = work.s_map.cpu().numpy()
    x = np.ones((work.V, 1), dtype=np.float32)
    osem_sc.get_weight_single(A[:64], y[:64], x, dtype=np.float32)
    n, t0 = 0, time.perf_counter()
    while True:
        w = osem_sc.get_weight_single(A, y, x, dtype=np.float32)
        x = (x * w / s).astype(np.float32)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 200:
            break
    return {"value": n / el, "unit": "subset-iters/s", "cores": threads or os.cpu_count(), "kind": "port",
            "sample": f"{n} subset updates of subset 0 ({A.shape[0]} x {A.shape[1]} float32, numpy BLAS)",
            "seconds": el}


# ----------------------------------------------------------------------------- arms
def reference_arm(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    dev = torch.device("cuda", local) if torch.cuda.is_available() else torch.device("cpu")
    work = make_workload(args.workload, dev)
    rates = []
    for i in range(args.warmup + args.steps):
        r = cpu_port_rate(work, budget_s=max(2.0, 20.0 / max(1, args.steps)))
        if i >= args.warmup:
            rates.append(r["value"])
    value = float(np.median(rates))
    line = {
        "impl": "reference", "metric": "OSEM subset-iters/s (SC channel of config 3)", "value": value,
        "unit": "subset-iters/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * work.subsets / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": work.name, "bins": work.B, "voxels": work.V, "subsets": work.subsets},
        "cpu_baseline": {"value": value, "unit": "subset-iters/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "per step: subset updates of subset 0 (numpy float32 BLAS), ~20 s total"},
        "e2e": {"value": value, "unit": "subset-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def ours_arm(args):
    world, rank, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from jscc_recon_spect_cylinder_gb300 import _lib

    _lib.load()
    work = make_workload(args.workload, dev)
    sampler = ClockSampler(local)
    sampler.start()
    ms_bf16, launches, img_bf16 = timed_steps(work, "bf16", args.steps, args.warmup, world)
    clocks = sampler.stop()
    ms_f32, _, img_f32 = timed_steps(work, "f32", args.steps, args.warmup, world)
    units = world * args.steps * work.units_per_step()
    value = units / (ms_bf16 / 1e3)
    value_f32 = units / (ms_f32 / 1e3)

    line = None
    if rank == 0:
        peaks = measured_peaks()
        kt = kernel_times(work, "bf16", max(3, args.steps))
        kbytes = work.kernel_bytes("bf16")
        kernels = {}
        for name, (n, tot) in kt.items():
            avg = tot / n
            entry = {"launches": n, "avg_ms": avg}
            if name in kbytes:
                entry["algorithmic_bytes"] = kbytes[name]
                entry["achieved_gbs"] = kbytes[name] / (avg / 1e3) / 1e9
            kernels[name] = entry
        top = max((k for k in kernels if "achieved_gbs" in kernels[k]), key=lambda k: kernels[k]["avg_ms"] *
                  kernels[k]["launches"])
        traffic = None
        tf = REPO / "profiles" / "traffic_sc3.json"
        if tf.exists():
            traffic = json.loads(tf.read_text()).get(top)
        achieved = kernels[top]["achieved_gbs"]
        roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                    "peak_source": peaks["source"]}
        errors = fp64_errors(work, args.steps + args.warmup, {"bf16": img_bf16, "f32": img_f32}) \
            if not args.no_errors else None
        e2e = run_e2e(work, "bf16", 30) if not args.no_e2e else None
        cpu = cpu_port_rate(work) if (world == 1 and not args.no_cpu_baseline) else None
        errors_iters = args.steps + args.warmup
        line = {
            "metric": "OSEM subset-iters/s: BF16-stored vs plain FP32 (SC channel of config 3), 1xGB300",
            "value": value, "unit": "subset-iters/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_bf16 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic",
            "config": {"workload": work.name, "bins": work.B, "voxels": work.V, "subsets": work.subsets,
                       "matrix_bytes_bf16": work.B * work.V * 2, "l2": "inputs larger than L2 (no flush)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "fp32": {"value": value_f32, "ms_per_step": ms_f32 / args.steps},
            "speedup_bf16_vs_fp32": value / value_f32,
            "errors_vs_fp64": errors,
            "errors_after_iterations": errors_iters,
            "gpu_launches": launches,
            "clocks": clocks,
            "roofline": roofline,
            "kernels": kernels,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["sc3", "sc3-small"], default="sc3")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-errors", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours_arm(args)


if __name__ == "__main__":
    main()
