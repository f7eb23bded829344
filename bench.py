"""Benchmark of the GB300 OSEM hot path; prints ONE JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload jsccsd3|jsccsd-small|sc3|sc3-small|sparse-launch|cone2|map5|batch4]
                    [--no-cpu-baseline] [--no-e2e]

Workload "jsccsd3" (default): JSCCSD joint OSEM at the joint configuration's size —
SC channel 20 views x 4,096 pixels = 81,920 bins x 36,000 voxels (100 x 360 polar grid,
dense matrix 11.8 GB FP32 / 5.9 GB BF16) plus ~1M forward-simulated 662 keV Compton
events built into sparse rows on a 4x theta-coarsened 9,000-voxel grid and materialised
to the fine grid on the fly, alpha = 0.5, 8 subsets. One step = one OSEM iteration
(8 subset updates). Metric: subset-iterations/s (higher is better); headline with the
system matrix and the sparse rows stored in BF16 (FP32 accumulation), the plain FP32
storage run beside it, plus Compton event-voxel pairs/s. Inputs are synthetic (seeded)
and far larger than L2, so no L2 flush is needed between timed iterations. After the main
measurement the line also carries `batched_config4`: the 64-instance batched SC path of
config 4 timed in a region of its own (subset-iterations/s summed over the instances and its
ratio to the plain FP32 single-instance path run 64 times).

Workload "sc3": the SC channel alone; "sc3-small": an 8,192-row SC case for profiling;
"sparse-launch": one grouped sparse Compton weight launch (profiling case); "cone2": the
fused strict cone weight of the list-mode configuration (200k events, event-voxel pairs/s);
"map5": one Adam step of the differentiable MAP objective (SC + 2M Compton events + RDP
prior, MAP steps/s); "batch4": one OSEM iteration of 64 SC instances through the batched
tensor-core GEMM path (subset-iterations/s summed over the instances).

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


# ----------------------------------------------------------------------------- workloads
class Sc3Workload:
    """SC channel of the joint configuration alone (flat form: all 20 views are rows of one
    matrix), subsets copied contiguously as the reference stages them."""

    def __init__(self, device, views=20, subsets=8, counts=1e7, seed=None):
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop
        from jscc_recon_spect_cylinder_gb300 import synthetic

        self.name = "jsccsd-config3-sc-channel" if (views, subsets) == (20, 8) else \
            f"sc-channel-{views}views-{subsets}subsets"
        self.metric = "OSEM subset-iters/s: BF16-stored vs plain FP32 (SC channel of config 3), 1xGB300"
        self.traffic_file = "traffic_sc3.json"
        self.dev = device
        self.subsets = subsets
        seed = synthetic.SEED if seed is None else seed
        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
        grid = synthetic.polar_grid(100, 360, 100.0, device=device)
        self.V = grid.n_vox
        pitch = 2.0 * math.pi * 120.0 / 128
        A = torch.cat([synthetic.sc_system_matrix(grid.coor, synthetic.cylinder_pixels(
            120.0, 128, 32, 2.0, phi0=2 * math.pi * v / views, device=device), pitch * 2.0, 100.0, generator=gen)
            for v in range(views)], dim=0)
        self.B = A.size(0)
        x_true = synthetic.hot_rod_phantom(grid.coor.cpu(), 100.0).to(device)
        self.proj = synthetic.poisson_projection(A, x_true, counts, generator=gen)
        self.s_map = A.sum(dim=0, keepdim=True).transpose(0, 1).contiguous()
        gcpu = torch.Generator().manual_seed(seed)
        ids = [i.to(device) for i in rop.split_tensor_even(torch.randperm(self.B, generator=gcpu), subsets, dim=0)]
        self.A_f32 = [A[i].contiguous() for i in ids]
        del A
        self.A_bf16 = [a.to(torch.bfloat16) for a in self.A_f32]
        self.y = [self.proj[i].contiguous() for i in ids]
        self.rot = torch.arange(1, self.V + 1, dtype=torch.int64, device=device).unsqueeze(1)
        torch.cuda.synchronize(device)

    def matrices(self, dtype):
        return self.A_bf16 if dtype == "bf16" else self.A_f32

    def step(self, img, dtype):
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

        return rop.osem_bin_mode([[a] for a in self.matrices(dtype)], [[y] for y in self.y], [self.rot], [self.rot],
                                 img, self.s_map, 1)

    def units_per_step(self):
        return self.subsets

    def kernel_bytes(self, dtype):
        b = 2 if dtype == "bf16" else 4
        rows = self.B / self.subsets
        return {"sc_forward_split": rows * self.V * b + self.V * 4, "sc_back_partial": rows * self.V * b + rows * 4,
                "sc_fused": rows * self.V * b + self.V * 4 + rows * 4}

    def config(self):
        return {"workload": self.name, "bins": self.B, "voxels": self.V, "subsets": self.subsets,
                "matrix_bytes_bf16": self.B * self.V * 2, "l2": "inputs larger than L2 (no flush)"}

    def fp64_reference(self, iters):
        x = torch.ones((self.V, 1), dtype=torch.float64, device=self.dev)
        s = self.s_map.double()
        for _ in range(iters):
            for A, y in zip(self.A_f32, self.y):
                A64 = A.double()
                x = x * (A64.t() @ (y.double() / (A64 @ x))) / s
                del A64
        return x

    def extra(self, ms_per_step):
        return {}

    def e2e(self, iters):
        """One job through recon_osem_plane.osem_bin_mode with host inputs: pinned host
        subset matrices (BF16), projections and sensitivity copied in, `iters` iterations,
        image read back."""
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

        host_A = [a.cpu().pin_memory() for a in self.A_bf16]
        host_y = [y.cpu().pin_memory() for y in self.y]
        host_s = self.s_map.cpu().pin_memory()
        out = torch.empty((self.V, 1)).pin_memory()
        h2d = sum(a.numel() * a.element_size() for a in host_A) + sum(y.numel() * 4 for y in host_y) + \
            host_s.numel() * 4 + self.V * 4
        torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        A = [[a.to(self.dev, non_blocking=True)] for a in host_A]
        y = [[v.to(self.dev, non_blocking=True)] for v in host_y]
        s = host_s.to(self.dev, non_blocking=True)
        img = torch.ones((self.V, 1)).pin_memory().to(self.dev, non_blocking=True)
        rot = torch.arange(1, self.V + 1, dtype=torch.int64).unsqueeze(1).to(self.dev, non_blocking=True)
        for _ in range(iters):
            img = rop.osem_bin_mode(A, y, [rot], [rot], img, s, 1)
        out.copy_(img, non_blocking=True)
        torch.cuda.synchronize(self.dev)
        sec = time.perf_counter() - t0
        return {"value": iters * self.subsets / sec, "unit": "subset-iters/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(self.V * 4),
                "step": f"one job: stage inputs + {iters} iterations + read image", "seconds": sec}

    def cpu_rate(self, budget_s=10.0):
        """Oracle port (numpy float32 BLAS, all host cores): subset updates of subset 0."""
        from oracle import osem_sc

        A = self.A_f32[0].cpu().numpy()
        y = self.y[0].cpu().numpy()
        s = self.s_map.cpu().numpy()
        x = np.ones((self.V, 1), dtype=np.float32)
        n, t0 = 0, time.perf_counter()
        while True:
            x = (x * osem_sc.get_weight_single(A, y, x, dtype=np.float32) / s).astype(np.float32)
            n += 1
            el = time.perf_counter() - t0
            if el >= budget_s or n >= 200:
                break
        return {"value": n / el, "unit": "subset-iters/s", "cores": os.cpu_count(), "kind": "port",
                "sample": f"{n} subset updates of subset 0 ({A.shape[0]} x {A.shape[1]} float32, numpy BLAS)",
                "seconds": el}


FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
FP32_PEAK_SOURCE = ("nominal: 152 SMs x 128 FP32 lanes x 2 FLOP per FMA x 2.07 GHz (no measured FP32 figure on "
                    "this pool)")


def cone_flop_per_pair():
    """FP32 FLOPs per fully evaluated event-voxel pair of the strict fused cone passes, from
    ncu's FP32 instruction counters on the config-2 forward and back launches
    (profiles/cone_flops_jsccd2.json: FADD, FMUL = 1, FFMA, FADD2, FMUL2 = 2, FFMA2 = 4 per
    thread instruction, over the launch's event-voxel pairs; the special-function unit's
    instructions, compares and selects are not counted), averaged over the two directions;
    the formula's hand count (Cone2Bench.K_CONE) when no capture is committed."""
    f = REPO / "profiles" / "cone_flops_jsccd2.json"
    if f.exists():
        d = json.loads(f.read_text())
        vals = [d[k]["flop_per_pair"] for k in ("cone_forward_pair", "cone_back_pair") if k in d]
        if vals:
            return float(np.mean(vals)), "ncu FP32 instruction counters (profiles/cone_flops_jsccd2.json)"
    return float(Cone2Bench.K_CONE), "hand count of the strict formula"


def cone_roofline(pairs_per_s, over=None):
    fpp, src = cone_flop_per_pair()
    achieved = pairs_per_s * fpp / 1e12
    out = {"bound": "fp32", "achieved": achieved, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
           "frac": achieved / FP32_PEAK_TFLOPS, "peak_source": FP32_PEAK_SOURCE, "flop_per_pair": fpp,
           "flop_source": src}
    if over:
        out["over"] = over
    return out


class Cone2Bench:
    """Config 2 (JSCCD list mode, FP32): the fused strict cone weight w = T^T (1 / T x) with
    T recomputed on the fly from 64-byte event records. 100 x 360 polar grid (36,000 voxels);
    scatter cylinder r = 120 mm and absorber r = 150 mm, 32 x 128 pixels each (8,192 detector
    pixels); 200,000 two-interaction events at 511 keV forward-simulated from the hot-rod
    phantom, energies blurred with the reference's convention (8 % FWHM at 662 keV scaled by
    sqrt(0.662 / E)), selected by the strict builder's filters and row statistics. One step =
    one weight pass (forward and back over every kept event and every voxel: all pairs are
    evaluated, as the reference does; the 9-sigma cos-beta window is timed beside it)."""

    K_CONE = 100  # FP32 operations per fully evaluated event-voxel pair (strict formula, see flops())

    def __init__(self, dev, n_events=200000, seed=None):
        from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
        from jscc_recon_spect_cylinder_gb300 import synthetic

        seed = synthetic.SEED if seed is None else seed
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        grid = synthetic.polar_grid(100, 360, 100.0, device=dev)
        pitch = 2.0 * math.pi * 120.0 / 128
        scat = synthetic.cylinder_pixels(120.0, 128, 32, 2.0, 0.0, dev)
        absb = synthetic.cylinder_pixels(150.0, 128, 32, 2.0, 0.0, dev)
        self.A = synthetic.sc_system_matrix(grid.coor, scat, pitch * 2.0, 100.0, generator=gen)
        det = torch.cat((scat, absb), dim=0).to(torch.float32)
        x_true = synthetic.hot_rod_phantom(grid.coor.cpu(), 100.0).to(dev)
        e0 = 0.511
        lst = synthetic.compton_list(grid.coor, x_true, scat, 150.0, 128, 32, 2.0, e0, int(n_events * 2.3) + 64, gen,
                                     cp1_offset=0, cp2_offset=scat.size(0))[:n_events]
        res = 0.08 * (0.662 / e0) ** 0.5
        noise = torch.randn((lst.size(0), 2), generator=gen, device=dev)
        for k, col in ((0, 1), (1, 3)):
            e = lst[:, col]
            lst[:, col] = e + (e * res / 2.355 * (e0 / e) ** 0.5) * noise[:, k]
        thr_max = 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001
        self.coor = grid.coor.to(torch.float32)
        self.ev = pls.get_compton_event_params(self.A, det, self.coor, lst, 1.0, 1.0, e0, res, thr_max, 0.05,
                                               e0 - 0.06, window_sigmas=9.0)
        self.n_list = lst.size(0)
        self.V = grid.n_vox
        self.dev = dev
        self.subsets = 1
        self.name = "jsccd-config2"
        self.metric = "event-voxel pairs/s: fused strict cone weight (T recomputed on the fly), config 2, 1xGB300"
        self.unit = "event-voxel pairs/s"
        self.dtypes = ("f32",)
        self.traffic_file = "traffic_cone2.json"
        self.w = torch.zeros((self.V, 1), device=dev)
        torch.cuda.synchronize(dev)

    def step(self, img, dtype, use_window=False):
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

        self.w.zero_()
        rop.get_weight_compton_fused(self.ev, self.coor, self.A, img, out=self.w, use_window=use_window)
        return img

    def units_per_step(self):
        return 2 * len(self.ev) * self.V  # forward and back pairs

    def kernel_bytes(self, dtype):
        return {}

    def flops(self):
        """K_CONE per pair: v = x_j - r1 (3), |v|^2 (5), v . u12 (5), cos beta (2), window
        test (2), acos (~12 incl. the SFU), beta - theta (1), sigma_pos^2 Jacobian of beta in
        r1 and r2 with per-axis variances (~45), sigma^2 and the Gaussian exponent (~6), exp
        (~4), Klein-Nishina - sin^2 beta (3), x efficiency (1), forward or back FMA (2); ~90,
        rounded to 100. Pairs outside the window stop after the test (~20)."""
        return self.K_CONE

    def stored_t(self, img):
        """The same weight from a stored dense T (FP32 [E, V], materialised once by the cone
        kernel): build time, the streamed weight's time (T read twice: forward and back),
        its HBM rate against the measured peak, and its agreement with the fused weight."""
        from jscc_recon_spect_cylinder_gb300 import ops
        from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

        ev, dev = self.ev, self.dev
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        _, T = ops.compton_cone_rows(ev.records, ev.row_id, self.coor, model=ev.model, eff=self.A, want_tc=False)
        t1.record()
        torch.cuda.synchronize(dev)
        build_ms = t0.elapsed_time(t1)
        w = rop.get_weight_compton(T, img)
        torch.cuda.synchronize(dev)
        n = 3
        t0.record()
        for _ in range(n):
            w = rop.get_weight_compton(T, img)
        t1.record()
        torch.cuda.synchronize(dev)
        ms = t0.elapsed_time(t1) / n
        self.step(img, "f32")
        rel = float((w - self.w).norm() / self.w.norm())
        nbytes = 2 * T.numel() * 4
        del T, w
        torch.cuda.empty_cache()
        gbs = nbytes / (ms / 1e3) / 1e9
        hbm = measured_peaks()["hbm_gbs"]
        return {"t_bytes": nbytes // 2, "build_ms": build_ms, "weight_ms": ms,
                "pairs_per_s": self.units_per_step() / (ms / 1e3), "hbm_gbs": gbs, "hbm_frac": gbs / hbm,
                "rel_l2_vs_fused": rel}

    def config(self):
        return {"workload": self.name, "voxels": self.V, "events_listed": self.n_list, "events_kept": len(self.ev),
                "detector_pixels": 8192, "e0_mev": 0.511, "window": "none (every pair)", "model": "strict",
                "l2": "records 13 MB, sysmat rows 590 MB; compute-bound"}

    def extra(self, ms_per_step):
        """The FP32 roofline of the timed pass (every pair evaluated, so the flop count is
        exact), the same pass with the 9-sigma cos-beta window, and the stored-T arm."""
        img = torch.ones((self.V, 1), device=self.dev)
        for _ in range(2):
            self.step(img, "f32", use_window=True)
        torch.cuda.synchronize(self.dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        n = 3
        for _ in range(n):
            self.step(img, "f32", use_window=True)
        t1.record()
        torch.cuda.synchronize(self.dev)
        ms_w = t0.elapsed_time(t1) / n
        pairs = self.units_per_step() / (ms_per_step / 1e3)
        stored = self.stored_t(img)
        return {"window_9sigma": {"pairs_per_s": self.units_per_step() / (ms_w / 1e3), "ms_per_step": ms_w},
                "stored_t": stored, "fp32_roofline": cone_roofline(pairs)}


class Map5Bench:
    """Config 5 (differentiable MAP): one Adam step of Phi(z) = -L(e^z) + beta R(e^z) on a
    log-parameterised 100 x 360 image. SC channel: 20 views x 4,096 pixels = 81,920 bins x
    36,000 voxels, FP32, flat (11.8 GB), Poisson data at 1e7 counts from the hot-rod phantom.
    Compton channel: 2,000,000 two-interaction events at 662 keV (scatter cylinder of view 0,
    absorber r = 150 mm), energies blurred as in config 2, strict model, T recomputed in the
    forward and in the adjoint pass (every event-voxel pair evaluated). Prior: relative difference,
    beta = 0.01, gamma = 2, ring +-1 angle and nearest angle in adjacent rings. A step = SC forward + adjoint, Compton forward +
    adjoint, prior value + gradient, the exp / log-chain and the Adam update."""

    K_CONE = Cone2Bench.K_CONE

    def __init__(self, dev, n_events=2_000_000, views=20, seed=None):
        from jscc_recon_spect_cylinder_gb300 import ops, prior
        from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
        from jscc_recon_spect_cylinder_gb300 import synthetic

        seed = synthetic.SEED if seed is None else seed
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        grid = synthetic.polar_grid(100, 360, 100.0, device=dev)
        pitch = 2.0 * math.pi * 120.0 / 128
        scat_views = [synthetic.cylinder_pixels(120.0, 128, 32, 2.0, 2 * math.pi * v / views, dev) for v in range(views)]
        A = torch.cat([synthetic.sc_system_matrix(grid.coor, p, pitch * 2.0, 100.0, generator=gen)
                       for p in scat_views], dim=0)
        x_true = synthetic.hot_rod_phantom(grid.coor.cpu(), 100.0).to(dev)
        self.y = synthetic.poisson_projection(A, x_true, 1e7, generator=gen)
        self.A = A
        scat = scat_views[0]
        absb = synthetic.cylinder_pixels(150.0, 128, 32, 2.0, 0.0, dev)
        det = torch.cat((scat, absb), dim=0).to(torch.float32)
        e0 = 0.662
        lst = synthetic.compton_list(grid.coor, x_true, scat, 150.0, 128, 32, 2.0, e0, int(n_events * 2.3) + 64, gen,
                                     cp1_offset=0, cp2_offset=scat.size(0))[:n_events]
        res = 0.08 * (0.662 / e0) ** 0.5
        noise = torch.randn((lst.size(0), 2), generator=gen, device=dev)
        for k, col in ((0, 1), (1, 3)):
            e = lst[:, col]
            lst[:, col] = e + (e * res / 2.355 * (e0 / e) ** 0.5) * noise[:, k]
        thr_max = 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001
        self.coor = grid.coor.to(torch.float32)
        self.eff = A[:scat.size(0)]  # efficiency rows of the scatter pixels (view 0 of the SC matrix)
        self.ev = pls.get_compton_event_params(self.eff, det, self.coor, lst, 1.0, 1.0, e0, res, thr_max, 0.05,
                                               e0 - 0.06, window_sigmas=9.0)
        self.n_list = lst.size(0)
        del lst, noise
        self.V = grid.n_vox
        self.s_c = ops.compton_backproject(self.ev.records, self.ev.row_id, self.coor,
                                           torch.ones(len(self.ev), device=dev), model=self.ev.model, eff=self.eff)
        self.table = prior.polar_neighbours(grid.coor.cpu()).to(dev)
        self.beta, self.gamma, self.lr = 0.01, 2.0, 0.05
        self.z = torch.zeros((self.V, 1), device=dev, requires_grad=True)
        self.opt = torch.optim.Adam([self.z], lr=self.lr)
        self.dev = dev
        self.subsets = 1
        self.name = "map-config5"
        self.metric = "MAP steps/s: SC + Compton log-likelihood + RDP prior, forward + adjoint + Adam, config 5, 1xGB300"
        self.unit = "MAP steps/s"
        self.dtypes = ("f32",)
        self.traffic_file = "traffic_map5.json"
        torch.cuda.synchronize(dev)

    def objective(self, z):
        from jscc_recon_spect_cylinder_gb300 import autograd as ag

        x = torch.exp(z)
        return (-ag.poisson_log_likelihood(x, sc=(self.A, self.y, None, None),
                                           compton=(self.ev, self.coor, self.eff, self.s_c))
                + ag.rdp_prior(x, self.table, beta=self.beta, gamma=self.gamma))

    def step(self, img, dtype):
        self.opt.zero_grad(set_to_none=False)
        self.objective(self.z).backward()
        self.opt.step()
        return img

    def units_per_step(self):
        return 1

    def kernel_bytes(self, dtype):
        return {}

    def config(self):
        return {"workload": self.name, "voxels": self.V, "sc_bins": self.A.size(0), "sc_dtype": "f32",
                "events_listed": self.n_list, "events_kept": len(self.ev), "e0_mev": 0.662, "window": "none",
                "beta": self.beta, "gamma": self.gamma, "optimizer": f"Adam lr {self.lr} (log-intensity)",
                "l2": "SC matrix 11.8 GB > L2 (streamed twice per step); records 90 MB"}

    def extra(self, ms_per_step):
        """The FP32 roofline of the step's cone passes (forward + adjoint over every pair),
        timed on their own."""
        from jscc_recon_spect_cylinder_gb300 import ops

        x = torch.ones((self.V, 1), device=self.dev)
        g = torch.ones(len(self.ev), device=self.dev)

        def cone_pass():
            f = ops.compton_project(self.ev.records, self.ev.row_id, self.coor, x, model=self.ev.model, eff=self.eff,
                                    use_window=False)
            ops.compton_backproject(self.ev.records, self.ev.row_id, self.coor, g, model=self.ev.model, eff=self.eff,
                                    use_window=False)
            return f

        cone_pass()
        torch.cuda.synchronize(self.dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        cone_pass()
        t1.record()
        torch.cuda.synchronize(self.dev)
        ms = t0.elapsed_time(t1)
        pairs = 2 * len(self.ev) * self.V
        return {"cone_pass": {"pairs_per_s": pairs / (ms / 1e3), "ms": ms},
                "fp32_roofline": cone_roofline(pairs / (ms / 1e3))}


class Batch4Bench:
    """Config 4 (batched): 64 independent SC reconstructions sharing the joint configuration's
    SC geometry (20 views x 4,096 pixels = 81,920 bins x 36,000 voxels, flat), Poisson
    realisations of the hot-rod phantom at contrasts 2-8 with totals log-uniform in 1e5-1e7
    counts, 8 subsets. One step = one OSEM iteration of every instance (8 subset updates x 64
    instances) through the batched tensor-core path (BF16 matrix and its transpose, images and
    ratios as BF16 hi / lo pairs, FP32 accumulation in tensor memory), replayed as one captured
    CUDA graph. Metric: subset-iterations/s summed over the instances."""

    CAPTURE = True

    def __init__(self, dev, n_inst=64, views=20, subsets=8, seed=None):
        from jscc_recon_spect_cylinder_gb300 import batched, synthetic
        from jscc_recon_spect_cylinder_gb300.recon_osem_plane import split_tensor_even

        seed = synthetic.SEED if seed is None else seed
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        grid = synthetic.polar_grid(100, 360, 100.0, device=dev)
        pitch = 2.0 * math.pi * 120.0 / 128
        A = torch.cat([synthetic.sc_system_matrix(grid.coor, synthetic.cylinder_pixels(
            120.0, 128, 32, 2.0, phi0=2 * math.pi * v / views, device=dev), pitch * 2.0, 100.0, generator=gen)
            for v in range(views)], dim=0)
        self.B, self.V = A.shape
        gc = torch.Generator().manual_seed(seed)
        counts = 10 ** (5 + 2 * torch.rand(n_inst, generator=gc, dtype=torch.float64))
        contrasts = 2 + 6 * torch.rand(n_inst, generator=gc, dtype=torch.float64)
        coor = grid.coor.cpu()
        X_true = torch.stack([synthetic.hot_rod_phantom(coor, 100.0, contrast=float(c)).reshape(-1)
                              for c in contrasts]).to(dev)
        mean = X_true @ A.T
        mean = mean * (counts.to(dev).float() / mean.sum(1))[:, None]
        self.Y = torch.poisson(mean, generator=gen)
        del mean
        self.ids = split_tensor_even(torch.randperm(self.B, generator=gc), subsets)
        self.s = A.sum(0)
        self.A32 = A
        self.n_inst, self.subsets, self.dev = n_inst, subsets, dev
        self.bat = self._make_batch(A, grid, X_true, counts, gen, gc)
        self.bat.set_projections(self.Y)
        self.bat.set_images(torch.ones((n_inst, self.V)))
        self.splits = self.bat.autotune()
        if self.CAPTURE:
            self.bat.capture()
        self.bat.set_images(torch.ones((n_inst, self.V)))
        self.name = "batched-config4" if (views, subsets) == (20, 8) else f"batched-{views}views-{subsets}subsets"
        self.metric = ("OSEM subset-iters/s summed over 64 instances: batched BF16 tensor-core GEMM path, "
                       "config 4, 1xGB300")
        self.unit = "subset-iters/s"
        self.dtypes = ("bf16",)
        self.traffic_file = "traffic_batch4.json"
        torch.cuda.synchronize(dev)

    def _make_batch(self, A, grid, X_true, counts, gen, gc):
        from jscc_recon_spect_cylinder_gb300 import batched

        return batched.BatchedScOsem(A, self.ids, self.s, self.n_inst, device=self.dev)

    def step(self, img, dtype):
        self.bat.iterate(1)
        return img

    def step_eager(self, img, dtype):
        """The same iteration launched kernel by kernel (for per-kernel timing)."""
        g, self.bat.graph = self.bat.graph, None
        try:
            self.bat.iterate(1)
        finally:
            self.bat.graph = g
        return img

    def units_per_step(self):
        return self.n_inst * self.subsets

    def _launch_bytes(self):
        """Algorithmic bytes of one forward and one back GEMM launch of a subset (matrix block
        once, BF16 instance operand, FP32 result once)."""
        nbp = max(b[2] for b in self.bat.blocks)
        nr, V = self.bat.nr, self.V
        fwd = nbp * V * 2 + nr * V * 2 + nbp * nr * 4
        back = V * nbp * 2 + nr * nbp * 2 + V * nr * 4
        return fwd, back, 2 * nbp * V * nr

    def kernel_bytes(self, dtype):
        fwd, back, _ = self._launch_bytes()
        return {"bf16_gemm_nt": (fwd + back) / 2}

    def config(self):
        return {"workload": self.name, "instances": self.n_inst, "bins": self.B, "voxels": self.V,
                "subsets": self.subsets, "counts": "log-uniform 1e5-1e7 per instance", "k_splits": {
                    f"{k[0]}{k[1]}": v for k, v in self.splits.items()}, "graph": True,
                "l2": "BF16 matrix 5.9 GB and its transpose, both > L2 (no flush)"}

    def _sequential_fp32(self, iters=2):
        """The plain FP32 single-instance path (jscc_sc_weight on the FP32 matrix with
        row-index subsets + EM update) for one instance: subset-iterations/s."""
        from jscc_recon_spect_cylinder_gb300 import ops

        y = self.Y[0].reshape(-1, 1).contiguous()
        x = torch.ones((self.V, 1), device=self.dev)
        s = self.s.reshape(-1, 1)
        ids = [i.to(self.dev) for i in self.ids]

        def one():
            nonlocal x
            for r in ids:
                w = ops.sc_weight(self.A32, y, x, row_idx=r)
                x = x * w / s

        one()
        torch.cuda.synchronize(self.dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(iters):
            one()
        t1.record()
        torch.cuda.synchronize(self.dev)
        return self.subsets / (t0.elapsed_time(t1) / iters / 1e3)

    def _errors(self, iters=5):
        """Per-instance relative L2 / max-voxel error after `iters` iterations from x = 1,
        against the float64 OSEM on the FP32 matrix (float64 GEMMs on the GPU)."""
        self.bat.set_images(torch.ones((self.n_inst, self.V)))
        X = self.bat.iterate(iters).double().clone()
        self.bat.set_images(torch.ones((self.n_inst, self.V)))
        X64 = torch.ones((self.n_inst, self.V), dtype=torch.float64, device=self.dev)
        Y = self.Y.double()
        s = self.s.double()
        for _ in range(iters):
            for r in self.ids:
                r = r.to(self.dev)
                As = self.A32[r].double()
                W = (Y[:, r] / (X64 @ As.T)) @ As
                X64 = X64 * W / s
                del As, W
        rel = ((X - X64).norm(dim=1) / X64.norm(dim=1)).cpu()
        mx = ((X - X64).abs().max(dim=1).values / X64.abs().max(dim=1).values).cpu()
        return {"iterations": iters, "rel_l2_median": float(rel.median()), "rel_l2_max": float(rel.max()),
                "max_voxel_rel_max": float(mx.max())}

    def extra(self, ms_per_step):
        fwd, back, flops = self._launch_bytes()
        seq = self._sequential_fp32()
        value = self.units_per_step() / (ms_per_step / 1e3)
        tens = None
        kt = kernel_times(self, "bf16", 2)
        if "bf16_gemm_nt" in kt:
            n, tot = kt["bf16_gemm_nt"]
            tf = flops / (tot / n / 1e3) / 1e12
            pk = json.loads((REPO / "MEASURED_PEAKS.json").read_text()) if (REPO / "MEASURED_PEAKS.json").exists() else {}
            peak = float(pk.get("bf16_tflops", 1900.0))
            tens = {"achieved_tflops": tf, "peak_tflops": peak, "frac": tf / peak,
                    "peak_source": "measured" if "bf16_tflops" in pk else "fallback",
                    "flops_per_launch": flops, "note": "two BF16 rows (hi, lo) per instance"}
        return {"sequential_fp32_single_instance": {"subset_iters_per_s": seq, "x64_instances_subset_iters_per_s": seq,
                                                    "batched_speedup_vs_64_sequential": value / seq},
                "tensor_pipe": tens, "errors_vs_fp64": self._errors()}

    def e2e(self, iters):
        """One job through the public batched API with host inputs: the 64 instances'
        projections and initial images copied from pinned host memory, `iters` iterations
        (the captured graph), the images read back. The matrix is the resident geometry."""
        y_h = self.Y.cpu().pin_memory()
        x_h = torch.ones((self.n_inst, self.V)).pin_memory()
        out_h = torch.empty((self.n_inst, self.V)).pin_memory()
        for _ in range(2):
            self.bat.set_projections(y_h.to(self.dev, non_blocking=True))
            self.bat.set_images(x_h.to(self.dev, non_blocking=True))
            self.bat.iterate(iters)
            out_h.copy_(self.bat.X, non_blocking=True)
        torch.cuda.synchronize(self.dev)
        t = time.perf_counter()
        self.bat.set_projections(y_h.to(self.dev, non_blocking=True))
        self.bat.set_images(x_h.to(self.dev, non_blocking=True))
        self.bat.iterate(iters)
        out_h.copy_(self.bat.X, non_blocking=True)
        torch.cuda.synchronize(self.dev)
        sec = time.perf_counter() - t
        self.bat.set_images(torch.ones((self.n_inst, self.V)))
        return {"value": iters * self.units_per_step() / sec, "unit": "subset-iters/s",
                "h2d_bytes_per_step": (y_h.numel() + x_h.numel()) * 4 // iters,
                "d2h_bytes_per_step": out_h.numel() * 4 // iters,
                "step": f"one job: stage projections + images, {iters} iterations, read images", "seconds": sec}


class Batch4JointBench(Batch4Bench):
    """Config 4, joint form: the 64 instances of Batch4Bench each with a Compton channel of
    their own at 511 keV (events log-uniform in 50k-2M listed per instance, forward-simulated
    from the instance's phantom on the view-0 scatter cylinder and a 150 mm absorber, energies
    blurred as in config 2), alpha = 0.5, 8 subsets. One step = one joint OSEM iteration of
    every instance: SC weights from the batched tensor-core GEMMs, the Compton weights of all
    64 instances from one batched fused-cone launch per direction over the subset's events
    (device segment tables), the safe joint EM update with per-instance sensitivities (the
    Compton sensitivity rescaled as build_sparse_sensi_d does); the iteration is replayed as
    one captured CUDA graph."""

    CAPTURE = True

    def __init__(self, dev, n_inst=64, views=20, subsets=8, seed=None, ev_range=(5e4, 2e6)):
        self.ev_range = ev_range
        super().__init__(dev, n_inst=n_inst, views=views, subsets=subsets, seed=seed)
        self.name = "batched-joint-config4"
        self.metric = ("joint OSEM subset-iters/s summed over 64 instances: batched SC tensor-core GEMMs + "
                       "batched fused Compton cone, config 4, 1xGB300")

    def _make_batch(self, A, grid, X_true, counts, gen, gc):
        from jscc_recon_spect_cylinder_gb300 import batched, ops, synthetic
        from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls

        e0 = 0.511
        scat = synthetic.cylinder_pixels(120.0, 128, 32, 2.0, 0.0, self.dev)
        absb = synthetic.cylinder_pixels(150.0, 128, 32, 2.0, 0.0, self.dev)
        det = torch.cat((scat, absb), dim=0).to(torch.float32)
        res = 0.08 * (0.662 / e0) ** 0.5
        thr_max = 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001
        lo, hi = math.log10(self.ev_range[0]), math.log10(self.ev_range[1])
        n_ev = (10 ** (lo + (hi - lo) * torch.rand(self.n_inst, generator=gc, dtype=torch.float64))).long()
        coor = grid.coor.to(torch.float32)
        events, S = [], []
        self.n_listed = int(n_ev.sum())
        for n in range(self.n_inst):
            lst = synthetic.compton_list(grid.coor, X_true[n].reshape(-1, 1), scat, 150.0, 128, 32, 2.0, e0,
                                         int(n_ev[n] * 2.3) + 64, gen, cp1_offset=0, cp2_offset=scat.size(0))
            lst = lst[:int(n_ev[n])]
            noise = torch.randn((lst.size(0), 2), generator=gen, device=self.dev)
            for k, col in ((0, 1), (1, 3)):
                e = lst[:, col]
                lst[:, col] = e + (e * res / 2.355 * (e0 / e) ** 0.5) * noise[:, k]
            ev = pls.get_compton_event_params(A[:scat.size(0)], det, coor, lst, 1.0, 1.0, e0, res, thr_max, 0.05,
                                              e0 - 0.06, window_sigmas=0.0)
            d = ops.compton_backproject(ev.records, ev.row_id, coor, torch.ones(len(ev), device=self.dev),
                                        model=ev.model, eff=A).reshape(-1)
            d = d * self.s.sum() / d.sum() * (len(ev) / max(float(self.Y[n].sum()), 1.0)) if d.sum() > 0 else self.s
            S.append(0.5 * self.s + 1.5 * d)
            events.append(ev.split(self.subsets))
            del lst, noise
        self.n_kept = sum(sum(len(b) for b in ev_n) for ev_n in events)
        self.events, self.S_joint, self.coor, self.n_ev_listed = events, torch.stack(S), coor, n_ev
        return batched.BatchedJointOsem(A, self.ids, self.S_joint, events, coor, alpha=0.5, device=self.dev)

    def config(self):
        c = super().config()
        c.update({"workload": self.name, "compton_events_listed": self.n_listed, "compton_events_kept": self.n_kept,
                  "compton_events_per_instance": "log-uniform 5e4-2e6 listed", "alpha": 0.5,
                  "sc_kev": 140, "compton_kev": 511, "graph": True})
        return c

    def _joint_step_fp(self, n, x, dtype=torch.float32):
        """One joint iteration of instance n alone on the FP32 matrix (the original bin order):
        float32 through the library (jscc_sc_weight + jscc_compton_weight + safe EM), or, for
        float64 images, the library's FP64 projector halves (the reference definitions with every
        sum in double) and float64 SC products."""
        from jscc_recon_spect_cylinder_gb300 import ops

        y = self.Y[n].reshape(-1, 1)
        s = self.S_joint[n].reshape(-1, 1)
        for k in range(self.subsets):
            ids = self.ids[k].to(self.dev)
            ev = self.events[n][k]
            if dtype == torch.float32:
                w = torch.zeros_like(x)
                ops.sc_weight(self.A32, y, x, floor=1e-12, scale=0.5, out=w, row_idx=ids)
                if len(ev):
                    ops.compton_weight(ev.records, ev.row_id, self.coor, x, model=ev.model, eff=self.A32, scale=1.5,
                                       out=w)
                x = ops.em_update(x, w, s, safe=True)
            else:
                As = self.A32[ids].double()
                w = 0.5 * (As.T @ (y[ids].double() / torch.clamp(As @ x, min=1e-12)))
                if len(ev):
                    f = ops.compton_project(ev.records, ev.row_id, self.coor, x, model=ev.model, eff=self.A32)
                    w = w + 1.5 * ops.compton_backproject(ev.records, ev.row_id, self.coor,
                                                          1.0 / f.reshape(-1), model=ev.model,
                                                          eff=self.A32).reshape(-1, 1)
                w = torch.nan_to_num(w, nan=0.0, posinf=0.0, neginf=0.0)
                sd = s.double()
                valid = sd > 1e-12
                x = torch.where(valid, x * torch.clamp(w, min=0.0) / torch.where(valid, sd, torch.ones_like(sd)),
                                torch.zeros_like(x))
        return x

    def _sequential_fp32(self, iters=1):
        """The plain FP32 single-instance joint path run for the 64 instances one after the
        other: subset-iterations/s summed over the instances."""
        xs = [torch.ones((self.V, 1), device=self.dev) for _ in range(self.n_inst)]
        self._joint_step_fp(0, xs[0])  # warm-up (workspaces, cached event orders)
        torch.cuda.synchronize(self.dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(iters):
            for n in range(self.n_inst):
                xs[n] = self._joint_step_fp(n, xs[n])
        t1.record()
        torch.cuda.synchronize(self.dev)
        return self.n_inst * self.subsets / (t0.elapsed_time(t1) / iters / 1e3)

    def _errors(self, iters=2, max_listed=4e5, n_pick=4):
        """Per-instance relative L2 / max-voxel error of the batched BF16 path after `iters`
        iterations from x = 1 against a float64 joint OSEM on the FP32 matrix, for `n_pick`
        instances spread over the event counts up to `max_listed` listed events (the float64
        cone evaluation costs seconds per 100k events)."""
        order = [int(i) for i in torch.argsort(self.n_ev_listed) if self.n_ev_listed[i] <= max_listed]
        pick = sorted({order[int(round(q * (len(order) - 1)))] for q in np.linspace(0, 1, n_pick)}) if order else []
        self.bat.set_images(torch.ones((self.n_inst, self.V)))
        X = self.bat.iterate(iters).double().clone()
        self.bat.set_images(torch.ones((self.n_inst, self.V)))
        rel, mx = [], []
        for n in pick:
            x64 = torch.ones((self.V, 1), dtype=torch.float64, device=self.dev)
            for _ in range(iters):
                x64 = self._joint_step_fp(n, x64, torch.float64)
            x64 = x64.reshape(-1)
            rel.append(float((X[n] - x64).norm() / x64.norm()))
            mx.append(float((X[n] - x64).abs().max() / x64.abs().max()))
        return {"iterations": iters, "instances": pick, "listed_events": [int(self.n_ev_listed[n]) for n in pick],
                "rel_l2": rel, "max_voxel_rel": mx,
                "rel_l2_median": float(np.median(rel)) if rel else None, "rel_l2_max": max(rel) if rel else None,
                "reference": "float64 joint OSEM per instance on the FP32 matrix (float64 SC products, the "
                             "library's FP64 cone projector halves)"}

    def kernel_bytes(self, dtype):
        return {}  # the step is the cone passes' (FP32): the roofline below, not an HBM one

    def extra(self, ms_per_step):
        """Cone pairs per second over the whole step (the cone kernels take nearly all of it),
        the FP32 roofline at Cone2Bench's operations per pair, the plain FP32 single-instance
        joint path run for the 64 instances in turn, and per-instance errors against float64."""
        pairs = 2 * self.n_kept * self.V  # forward + back cone pairs per iteration
        rate = pairs / (ms_per_step / 1e3)
        value = self.units_per_step() / (ms_per_step / 1e3)
        seq = self._sequential_fp32()
        return {"compton_pairs_per_s": rate, "fp32_roofline": cone_roofline(rate, over="the whole step"),
                "sequential_fp32_joint_64_instances": {"subset_iters_per_s": seq,
                                                       "batched_speedup_vs_64_sequential": value / seq},
                "errors_vs_fp64": self._errors()}

    def e2e(self, iters):
        """Batch4Bench's job (projections and initial images staged from pinned host memory,
        the captured iterations, images read back) with at most two iterations: one joint
        iteration of the 64 instances takes seconds."""
        return super().e2e(min(iters, 2))


class SparseLaunchBench:
    """Profiling case: one grouped sparse Compton weight launch with a config-3 subset's sizes
    (99,850 BF16 coarse rows of 9,000 voxels, 12,239 groups, 100 x 360 fine grid, theta-stride-4
    ring stencil, materialise semantics) on a random 16,384-row BF16 sysmat, so that a full
    ncu capture holds ~3 GB on the device. One step = one weight call (the image is not
    updated); the fp32 pass repeats the same BF16 launch."""

    def __init__(self, dev, n_det=16384, n_events=99850, n_groups=12239, seed=1):
        from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
        from jscc_recon_spect_cylinder_gb300 import synthetic

        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        grid = synthetic.polar_grid(100, 360, 100.0)
        self.projector = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1)
        self.tables = cso.tables(self.projector, dev)
        self.V, self.Vc = grid.n_vox, self.projector.coarse_pixel_num
        self.A = torch.rand((n_det, self.V), generator=g, device=dev).to(torch.bfloat16)
        used = torch.randperm(n_det, generator=g, device=dev)[:n_groups].to(torch.int32)
        ids = used[torch.randint(0, n_groups, (n_events,), generator=g, device=dev)]
        self.ids = ids[torch.argsort(ids)].contiguous()
        self.tc = torch.rand((n_events, self.Vc), generator=g, device=dev).to(torch.bfloat16)
        self.n_events, self.n_groups = n_events, int(torch.unique(self.ids).numel())
        self.name = "sparse-launch"
        self.metric = "grouped sparse weight launches/s (one config-3 subset, synthetic rows), 1xGB300"
        self.traffic_file = "traffic_jsccsd3.json"
        self.dev = dev
        self.subsets = 1
        self.w = torch.zeros((self.V, 1), device=dev)
        torch.cuda.synchronize(dev)

    def step(self, img, dtype):
        from jscc_recon_spect_cylinder_gb300 import ops

        self.w.zero_()
        ops.sparse_weight_split(self.ids, self.tc, self.A, self.tables, img, grouped=False, out=self.w)
        return img

    def units_per_step(self):
        return 1

    def kernel_bytes(self, dtype):
        adjoint = self.n_groups * (self.V * 2 + self.Vc * 4)
        coef = self.n_events * (self.Vc * 2 + 4) + self.n_groups * 2 * self.Vc * 4
        scatter = self.n_groups * (self.V * 2 + self.Vc * 4) + 16 * self.V * 4
        fused = self.n_events * (self.Vc * 2 + 4) + self.n_groups * self.V * 2 + 38 * self.V * 4
        return {"sparse_group_adjoint": adjoint, "sparse_group_coef": coef, "sparse_group_scatter": scatter,
                "sparse_group_fused": fused}

    def config(self):
        return {"workload": self.name, "events": self.n_events, "groups": self.n_groups, "voxels": self.V,
                "coarse_voxels": self.Vc, "sysmat_rows": self.A.size(0), "storage": "bf16",
                "l2": "inputs larger than L2 (no flush)"}

    def extra(self, ms_per_step):
        return {}


JOINT_METRIC = ("OSEM subset-iters/s: BF16-stored vs plain FP32 joint JSCCSD (SC + sparse Compton, config 3), "
                "1xGB300")


def joint_config(name, bins, voxels, coarse, listed, kept, subsets, groups, alpha, views):
    """The `config` of the joint workload, the same dict on both arms."""
    return {"workload": name, "sc_bins": bins, "voxels": voxels, "coarse_voxels": coarse,
            "compton_events_listed": listed, "compton_events_kept": kept, "subsets": subsets,
            "groups_per_subset": groups, "alpha": alpha, "views": views,
            "l2": "inputs larger than L2 (no flush)", "parallelism": "single"}


class JointBench:
    """workloads.JointWorkload behind the bench interface."""

    storage = "bf16 system matrix + bf16 sparse rows (int32 ids split out); fp32 arm: fp32 matrix + fp32 sparse rows (the same split layout and kernels)"

    def __init__(self, dev, small=False, radial_stride=1):
        from jscc_recon_spect_cylinder_gb300 import workloads

        kw = dict(views=2, n_events=60000, subsets=2) if small else {}
        self.w = workloads.JointWorkload(dev, radial_stride=radial_stride, **kw)
        self.name = "jsccsd-config3" if not small else "jsccsd-small"
        if radial_stride > 1:
            self.name += f"-radial{radial_stride}"
        self.metric = JOINT_METRIC
        self.traffic_file = "traffic_jsccsd3.json"
        self.dev = dev
        self.small = small
        self.V = self.w.V
        self.subsets = self.w.subsets

    def step(self, img, dtype):
        return self.w.step(img, dtype)

    def units_per_step(self):
        return self.w.subsets

    def kernel_bytes(self, dtype):
        kb = self.w.sc_kernel_bytes(dtype)
        kb.update(self.w.sparse_kernel_bytes(dtype))
        return kb

    def config(self):
        w = self.w
        return joint_config(self.name, w.B, w.V, w.Vc, w.n_list, w.n_events, w.subsets, round(w.group_count(), 1),
                            w.alpha, w.views)

    def fp64_reference(self, iters):
        return self.w.fp64_reference(iters)

    def extra(self, ms_per_step):
        pairs = self.w.pair_count_per_step()
        out = {"compton_event_voxel_pairs_per_s": pairs / (ms_per_step / 1e3)}
        if not self.small:
            out["plain_fp32_gpu_reference"] = self.plain_fp32_gpu_reference()
            ref = out["plain_fp32_gpu_reference"]
            if "value" in ref:
                out["speedup_vs_plain_fp32_gpu"] = self.units_per_step() / (ms_per_step / 1e3) / ref["value"]
            out["batched_config4"] = batched_summary(self.dev)
        return out

    def plain_fp32_gpu_reference(self):
        """The reference's own PyTorch FP32 joint subset update on this GPU (oracle.
        reference_timing.run_gpu_plain_fp32: the same workload's float32 inputs)."""
        from oracle import reference_timing as rt

        torch.cuda.empty_cache()
        res = rt.run_gpu_plain_fp32(self.w)
        torch.cuda.empty_cache()
        return res

    def e2e(self, iters):
        """One job with host inputs: pinned host copies of the BF16 system matrix (also the
        efficiency table), projections, the BF16 sparse rows + ids, subset ids and the
        joint sensitivity go to the GPU inside the timed region, `iters` iterations run
        through the same kernels, and the image is read back. The device buffers the inputs
        land in are allocated once before the job (a service keeps them resident); the
        matrix, projections and sensitivity are copied first, each subset's sparse rows on a
        second stream, and the first iteration's update of subset k waits for subset k's
        rows only. One untimed job into the same buffers comes first (a service's pinned
        staging buffers are reused across jobs; the first DMA out of freshly pinned host
        memory is not representative), then the median of three timed jobs. Every job copies
        all inputs again, and the copies bump the device buffers' versions, so the group
        plans and event sums cached on them are rebuilt inside each timed job."""
        from jscc_recon_spect_cylinder_gb300 import ops

        w = self.w
        hA = w.A["bf16"].cpu().pin_memory()
        hy = w.proj.cpu().pin_memory()
        hs = w.s_joint.cpu().pin_memory()
        hids = [i.cpu().pin_memory() for i in w.ids]
        htc = [t.cpu().pin_memory() for t in w.tc_bf16]
        hsub = [i.cpu().pin_memory() for i in w.subset_ids]
        hx0 = torch.ones((w.V, 1)).pin_memory()
        out = torch.empty((w.V, 1)).pin_memory()
        h2d = hA.numel() * 2 + hy.numel() * 4 + hs.numel() * 4 + sum(i.numel() * 4 for i in hids) + \
            sum(t.numel() * 2 for t in htc) + sum(i.numel() * 8 for i in hsub) + w.V * 4
        A = torch.empty_like(w.A["bf16"])
        y = torch.empty_like(w.proj)
        s = torch.empty_like(w.s_joint)
        ids = [torch.empty_like(i) for i in w.ids]
        tc = [torch.empty_like(t) for t in w.tc_bf16]
        sub = [torch.empty_like(i) for i in w.subset_ids]
        x0 = torch.empty((w.V, 1), device=self.dev)
        side = torch.cuda.Stream(self.dev)
        landed = [torch.cuda.Event() for _ in range(w.subsets)]
        main = torch.cuda.current_stream(self.dev)

        def job():
            torch.cuda.synchronize(self.dev)
            t0 = time.perf_counter()
            for d, h in ((A, hA), (y, hy), (s, hs), (x0, hx0)):
                d.copy_(h, non_blocking=True)
            for d, h in zip(sub, hsub):
                d.copy_(h, non_blocking=True)
            side.wait_stream(main)
            with torch.cuda.stream(side):
                for k in range(w.subsets):
                    ids[k].copy_(hids[k], non_blocking=True)
                    tc[k].copy_(htc[k], non_blocking=True)
                    landed[k].record(side)
            img = x0
            for it in range(iters):
                for k in range(w.subsets):
                    if it == 0:
                        main.wait_event(landed[k])
                    wt = torch.zeros_like(img)
                    ops.sc_weight(A, y, img, floor=1e-12, scale=w.alpha, out=wt, row_idx=sub[k])
                    ops.sparse_weight_split(ids[k], tc[k], A, w.tables, img, grouped=False, scale=2 - w.alpha,
                                            out=wt)
                    img = ops.em_update(img, wt, s, safe=True)
            out.copy_(img, non_blocking=True)
            torch.cuda.synchronize(self.dev)
            return time.perf_counter() - t0

        job()  # untimed: first use of the pinned staging buffers
        secs = [job() for _ in range(3)]
        sec = sorted(secs)[1]
        for t in ids + tc:
            t.record_stream(side)
        return {"value": iters * w.subsets / sec, "unit": "subset-iters/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(w.V * 4),
                "step": (f"one job: stage inputs into resident device buffers (sparse rows on a second stream, "
                         f"overlapping the first iteration) + {iters} iterations + read image (the sparse T rows "
                         "are built beforehand by the GPU T builder, outside the timed job); median of 3 jobs "
                         "after one untimed job into the same buffers"), "seconds": sec,
                "seconds_per_job": secs}

    def cpu_rate(self, steps=2, warmup=1):
        """The reference's own functions on the host cores (oracle.reference_timing): whole-
        subset SC half, sampled Compton half; a bounded run of a few steps."""
        from oracle import reference_timing as rt

        r = rt.run_host(steps, warmup)
        return {"value": r["value"], "unit": r["unit"], "cores": r["cores"], "cpu_model": r["cpu_model"],
                "kind": r["kind"], "sample": r["sample"], "seconds_per_subset_update": r["seconds_per_subset_update"],
                "parts_s": r["parts_s"]}


def batched_summary(dev, steps=5):
    """The batched form of the SC channel (config 4: 64 instances sharing the joint
    configuration's 81,920 x 36,000 SC matrix, one captured graph per OSEM iteration) in a
    timed region of its own, after the main measurement: subset-iterations/s summed over the
    instances, the plain FP32 single-instance path run 64 times for comparison, and the
    tensor-core GEMM's HBM fraction."""
    b = Batch4Bench(dev)
    ms, launches, _ = timed_steps(b, "bf16", steps, 3, 1)
    value = b.units_per_step() * steps / (ms / 1e3)
    seq = b._sequential_fp32()
    kt = kernel_times(b, "bf16", 2)
    frac = None
    if "bf16_gemm_nt" in kt:
        n, tot = kt["bf16_gemm_nt"]
        frac = b.kernel_bytes("bf16")["bf16_gemm_nt"] / (tot / n / 1e3) / 1e9 / measured_peaks()["hbm_gbs"]
    res = {"value": value, "unit": "subset-iters/s summed over 64 instances", "ms_per_iteration": ms / steps,
           "steps": steps, "gpu_launches": launches, "plain_fp32_single_instance_subset_iters_per_s": seq,
           "speedup_vs_64_sequential_plain_fp32": value / seq, "gemm_hbm_frac_of_measured": frac,
           "workload": "bench.py --workload batch4"}
    del b
    torch.cuda.empty_cache()
    return res


SUMMARY_KEYS = {
    "cone2": ("window_9sigma", "stored_t", "fp32_roofline"),
    "map5": ("cone_pass", "fp32_roofline"),
    "batch4-joint": ("compton_pairs_per_s", "fp32_roofline", "sequential_fp32_joint_64_instances", "errors_vs_fp64"),
}


def workload_summary(name, dev, steps=3, warmup=3):
    """Another configuration's workload measured in a timed region of its own (CUDA events on
    the launch stream around `steps` steps after `warmup` untimed ones), with the figures of its
    own bench line that explain it; the workload is freed afterwards."""
    t0 = time.perf_counter()
    work = make_workload(name, dev)
    setup_s = time.perf_counter() - t0
    dt = getattr(work, "dtypes", ("bf16",))[0]
    ms, launches, _ = timed_steps(work, dt, steps, warmup, 1)
    out = {"workload": f"bench.py --workload {name}", "metric": work.metric,
           "value": work.units_per_step() * steps / (ms / 1e3), "unit": getattr(work, "unit", "subset-iters/s"),
           "ms_per_step": ms / steps, "steps": steps, "warmup": warmup, "gpu_launches": launches,
           "config": work.config(), "setup_s": setup_s}
    extra = work.extra(ms / steps)
    out.update({k: extra[k] for k in SUMMARY_KEYS.get(name, ()) if k in extra})
    del work, extra
    torch.cuda.empty_cache()
    return out


def make_workload(name, dev):
    if name == "jsccsd3":
        return JointBench(dev)
    if name == "jsccsd-small":
        return JointBench(dev, small=True)
    if name == "jsccsd3-radial":  # the Compton T on the radially coarsened 25 x 90 grid (an extension)
        return JointBench(dev, radial_stride=4)
    if name == "sparse-launch":
        return SparseLaunchBench(dev)
    if name == "cone2":
        return Cone2Bench(dev)
    if name == "map5":
        return Map5Bench(dev)
    if name == "batch4":
        return Batch4Bench(dev)
    if name == "batch4-joint":
        return Batch4JointBench(dev)
    if name == "batch4-small":  # profiling case: 4 views (16,384 x 36,000), one subset, 64 instances; > L2
        return Batch4Bench(dev, views=4, subsets=1)
    if name == "sc3":
        return Sc3Workload(dev)
    if name == "sc3-small":  # profiling case: 2 views (8,192 x 36,000), one subset; > L2
        return Sc3Workload(dev, views=2, subsets=1)
    raise ValueError(name)


# ----------------------------------------------------------------------------- timing
def max_over_ranks(ms, world, device):
    """The slowest rank's time (every rank gets it): the whole-job time of a replicated run."""
    if world <= 1:
        return ms
    t = torch.tensor([float(ms)], device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


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
    ms = max_over_ranks(t0.elapsed_time(t1), world, work.dev)
    return ms, launches, img


def kernel_times(work, dtype, steps):
    """Per-kernel CUDA-event durations on the launch stream (separate instrumented pass)."""
    from jscc_recon_spect_cylinder_gb300 import _lib

    step = getattr(work, "step_eager", work.step)  # a captured graph records no per-kernel events
    img = torch.ones((work.V, 1), device=work.dev)
    img = step(img, dtype)
    torch.cuda.synchronize(work.dev)
    _lib.kernel_timing_collect()
    _lib.kernel_timing_enable(True)
    for _ in range(steps):
        img = step(img, dtype)
    torch.cuda.synchronize(work.dev)
    _lib.kernel_timing_enable(False)
    return _lib.kernel_timing_collect()


def image_errors(ref64, images):
    out = {}
    for k, img in images.items():
        d = img.double() - ref64
        out[k] = {"rel_l2": float(d.norm() / ref64.norm()), "max_voxel_rel": float(d.abs().max() / ref64.abs().max())}
    return out


# ----------------------------------------------------------------------------- arms
def reference_arm(args):
    """The reference's own CPU implementation of the joint subset update on this machine's
    host cores (oracle.reference_timing: the staged reference modules, else the oracle's
    numpy port). No kernel of this repository runs and its library is not loaded: the inputs
    are built on the host. Each step is one bounded sample of the workload (the SC half on a
    whole subset, the Compton half on a fixed sample of whole groups); `value` is the
    resulting subset-update rate and `ms_per_step` the wall time a step actually took."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    if args.workload != "jsccsd3":
        print(json.dumps({"impl": "reference", "unavailable": f"no reference arm for workload {args.workload}"}))
        return
    from oracle import reference_timing as rt

    c = rt.CONFIG3
    r = rt.run_host(args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": JOINT_METRIC, "value": r["value"], "unit": r["unit"], "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": joint_config("jsccsd-config3", c["views"] * c["n_phi"] * c["n_axial"], c["n_r"] * c["n_theta"],
                               c["n_r"] * c["n_theta"] // c["theta_stride"], c["events_listed"], c["events_kept"],
                               c["subsets"], c["groups_per_subset"], c["alpha"], c["views"]),
        "cpu_baseline": {"value": r["value"], "unit": r["unit"], "cores": r["cores"], "cpu_model": r["cpu_model"],
                         "kind": r["kind"], "sample": r["sample"]},
        "seconds_per_subset_update": r["seconds_per_subset_update"], "parts_s": r["parts_s"],
        "setup_s": r["setup_s"],
        "e2e": {"value": r["value"], "unit": r["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    dtypes = getattr(work, "dtypes", ("bf16", "f32"))  # primary arm first
    unit = getattr(work, "unit", "subset-iters/s")
    sampler = ClockSampler(local)
    sampler.start()
    ms_main, launches, _ = timed_steps(work, dtypes[0], args.steps, args.warmup, world)
    clocks = sampler.stop()
    units = world * args.steps * work.units_per_step()
    value = units / (ms_main / 1e3)
    second = None
    if len(dtypes) > 1:
        ms_2, _, _ = timed_steps(work, dtypes[1], args.steps, args.warmup, world)
        second = {"value": units / (ms_2 / 1e3), "ms_per_step": ms_2 / args.steps}

    line = None
    if rank == 0:
        peaks = measured_peaks()
        kt = kernel_times(work, dtypes[0], max(3, min(args.steps, 10)))
        kbytes = work.kernel_bytes(dtypes[0])
        kernels = {}
        total_ms = sum(tot for _, tot in kt.values())
        for name, (n, tot) in kt.items():
            avg = tot / n
            entry = {"launches": n, "avg_ms": avg, "share": tot / total_ms if total_ms else None}
            if name in kbytes:
                entry["algorithmic_bytes"] = kbytes[name]
                entry["achieved_gbs"] = kbytes[name] / (avg / 1e3) / 1e9
            kernels[name] = entry
        roofline = None
        with_bytes = [k for k in kernels if "achieved_gbs" in kernels[k]]
        if with_bytes:
            top = max(with_bytes, key=lambda k: kernels[k]["avg_ms"] * kernels[k]["launches"])
            traffic = None
            tf = REPO / "profiles" / work.traffic_file
            if tf.exists():
                traffic = json.loads(tf.read_text()).get(top)
            achieved = kernels[top]["achieved_gbs"]
            roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                        "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "peak_source": peaks["source"]}
        errors = None
        err_iters = args.error_iters
        if not args.no_errors and hasattr(work, "fp64_reference"):
            imgs = {}
            for dt in dtypes:
                x = torch.ones((work.V, 1), device=dev)
                for _ in range(err_iters):
                    x = work.step(x, dt)
                imgs[dt] = x
            errors = image_errors(work.fp64_reference(err_iters), imgs)
        e2e = work.e2e(30) if not args.no_e2e and hasattr(work, "e2e") else None
        cpu = work.cpu_rate() if (world == 1 and not args.no_cpu_baseline and hasattr(work, "cpu_rate")) else None
        cfg = work.config()
        cfg["parallelism"] = "replicas" if world > 1 else "single"
        line = {
            "metric": work.metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_main / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtypes[0], "data": "synthetic", "config": cfg,
        }
        if hasattr(work, "storage"):
            line["storage"] = work.storage
        if second is not None:
            line[dtypes[1] if dtypes[1] != "f32" else "fp32"] = second
            line["speedup_bf16_vs_fp32"] = value / second["value"]
        line.update({"errors_vs_fp64": errors, "errors_after_iterations": err_iters, "gpu_launches": launches,
                     "clocks": clocks, "roofline": roofline, "kernels": kernels, "e2e": e2e, "cpu_baseline": cpu})
        extra = {} if args.no_extra else work.extra(ms_main / args.steps)
        if roofline is None and "fp32_roofline" in extra:
            top = max(kernels, key=lambda k: kernels[k]["avg_ms"] * kernels[k]["launches"]) if kernels else None
            line["roofline"] = dict(extra.pop("fp32_roofline"), kernel=top, traffic=None)
        line.update(extra)
        if args.workload == "jsccsd3" and not args.no_extra and not args.no_other_workloads:
            # the other configurations, each in a timed region of its own after the main
            # measurement (the joint workload is freed first)
            del work
            torch.cuda.empty_cache()
            line["other_workloads"] = {name.replace("-", "_"): workload_summary(name, dev)
                                       for name in ("cone2", "map5", "batch4-joint")}
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["jsccsd3", "jsccsd-small", "jsccsd3-radial", "sc3", "sc3-small", "sparse-launch", "cone2", "map5", "batch4",
                             "batch4-small", "batch4-joint"],
                    default="jsccsd3")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-errors", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the workload's extra figures (e.g. cone2's stored-T arm): small profiling runs")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="jsccsd3: skip the summaries of the cone2 / map5 / batch4-joint workloads")
    ap.add_argument("--error-iters", type=int, default=10,
                    help="iterations (from a uniform image) at which BF16 / FP32 images are compared with FP64")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours_arm(args)


if __name__ == "__main__":
    main()
