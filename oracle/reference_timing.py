"""Timing of the reference's own implementation of the joint JSCCSD OSEM subset update --
MEASUREMENT INFRASTRUCTURE for bench.py only (its reference arm, its cpu_baseline and its
plain-FP32-GPU comparison point). Nothing in the product imports this module.

The reference is pure Python / PyTorch. Its functions for this path are timed as they are,
imported from the copies that oracle/stage_ref.py staged, unmodified, into oracle/_ref/:

* SC half: get_weight_single (recon_osem_local_sparse_jsccsd_only.py:8-10, forward clamped
  at 1e-12) on one subset's 10,240 x 36,000 float32 rows;
* Compton half: both of the reference's sparse weights,
    grouped      get_weight_compton_sparse (recon_osem_plane_sparse.py:22-57): per distinct
                 first-hit row, two dense coarse<->fine products over the projector's
                 [36,000 x 9,000] expand matrix and two small products over the group's rows;
    materialise  get_weight_compton_sparse (recon_osem_local_sparse_jsccsd_only.py:13-19):
                 every event row upsampled to the fine grid through the same dense matrix,
                 multiplied by its efficiency row, normalised, then T^T (1 / T x);
* the update safe_em_update (recon_osem_local_sparse_jsccsd_only.py:22-28).

Host cores (reference arm, cpu_baseline). One subset update of the config-3 workload on the
host takes minutes (12,305 groups x two 1.3 GB dense products, or 99,850 events x 6.5e8 FLOP),
so each step runs the SC half on a whole subset and each Compton form on a fixed sample of
whole groups (SAMPLE_GROUPS groups of EVENTS_PER_GROUP events, the subset's mean group size).
The subset-update time is the SC half plus the faster Compton form scaled to the subset (the
grouped form by groups, the materialise form by events: their costs are linear in those) plus
the update; every step's wall time is what `ms_per_step` reports. The inputs are built on the
host from the seeded generators (no GPU kernel of this repository runs): the subset's SC rows
from the SC matrix formula, efficiency rows the same way, the projector by the reference's own
build_compton_sparse_projector, coarse event rows seeded random (the reference's cost does not
depend on their values).

GPU (comparison point: the reference's PyTorch FP32 path on the same GB300). The parts of the
reference's osem_joint_mode_local_sparse (recon_osem_local_sparse_jsccsd_only.py:58-100) run
on the device on the float32 inputs the bench built: the SC half on a whole subset, the
Compton half in both of the reference's forms on samples of the same subset scaled to it, as
on the host; the faster form is the comparison point.

When oracle/_ref/ holds no staged copies, the same steps run through the oracle's numpy
restatement of the same functions (cpu kind "port").
"""
from __future__ import annotations

import math
import os
import platform
import subprocess
import time

import numpy as np
import torch

# The config-3 joint workload (workloads.JointWorkload, seed 20260331): 20 views x 4,096 SC
# pixels = 81,920 bins on a 100 x 360 polar grid (36,000 voxels), 1,000,000 listed Compton
# events of which 798,802 survive the sparse T builder, 8 subsets of 99,850 events in
# 12,305.4 groups (distinct first-hit rows) on average, theta-stride-4 coarse grid (9,000).
CONFIG3 = dict(n_r=100, n_theta=360, radius=100.0, views=20, n_phi=128, n_axial=32, axial_pitch=2.0, scat_r=120.0,
               subsets=8, alpha=0.5, theta_stride=4, events_kept=798_802, events_listed=1_000_000,
               groups_per_subset=12_305.4, sc_counts=1e7)
SAMPLE_GROUPS = 32
EVENTS_PER_GROUP = 8


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.processor() or platform.machine()


def reference_modules():
    """The staged reference modules, or None (the numpy port is used then)."""
    from oracle import stage_ref

    return stage_ref.load() if stage_ref.available() else None


class HostSample:
    """Host inputs of one config-3 subset update: the subset's SC rows, projections and a
    sample of whole event groups with their efficiency rows."""

    def __init__(self, seed=20260331, sample_groups=SAMPLE_GROUPS, events_per_group=EVENTS_PER_GROUP):
        from jscc_recon_spect_cylinder_gb300 import synthetic

        c = CONFIG3
        gen = torch.Generator().manual_seed(seed)
        grid = synthetic.polar_grid(c["n_r"], c["n_theta"], c["radius"])
        self.V = grid.n_vox
        npix = c["n_phi"] * c["n_axial"]
        B = c["views"] * npix
        pitch = 2.0 * math.pi * c["scat_r"] / c["n_phi"]
        area = pitch * c["axial_pitch"]
        views = [synthetic.cylinder_pixels(c["scat_r"], c["n_phi"], c["n_axial"], c["axial_pitch"],
                                           2 * math.pi * v / c["views"]) for v in range(c["views"])]
        pix = torch.cat(views, dim=0)  # bin b = view * 4,096 + pixel
        perm = torch.randperm(B, generator=gen)
        ids = perm[: B // c["subsets"]]  # one subset of the split (split_tensor_even: equal parts here)
        self.A = synthetic.sc_system_matrix(grid.coor, pix[ids], area, c["radius"], generator=gen)
        x_true = synthetic.hot_rod_phantom(grid.coor, c["radius"])
        self.y = synthetic.poisson_projection(self.A, x_true, c["sc_counts"] / c["subsets"], generator=gen)
        self.x = torch.ones((self.V, 1))
        self.s = torch.rand((self.V, 1), generator=gen) + 0.5
        self.coor = grid.coor
        G, n = sample_groups, events_per_group
        self.groups, self.events = G, G * n
        eff_bins = torch.randperm(B, generator=gen)[:G]
        self.eff = synthetic.sc_system_matrix(grid.coor, pix[eff_bins], area, c["radius"], generator=gen)
        self.cp1 = torch.arange(1, G + 1).repeat_interleave(n)  # 1-based rows of self.eff
        self.vc = (c["n_theta"] // c["theta_stride"]) * c["n_r"]
        tc = torch.rand((G * n, self.vc), generator=gen) ** 3
        self.tc = tc / tc.sum(dim=1, keepdim=True)
        self.rows = torch.cat((self.cp1.to(torch.float32).unsqueeze(1), self.tc), dim=1)
        self.events_per_subset = c["events_kept"] / c["subsets"]
        self.groups_per_subset = c["groups_per_subset"]


class HostTimer:
    """Times the reference's functions (or the numpy port) on a HostSample."""

    def __init__(self, sample: HostSample, threads=None):
        self.smp = sample
        torch.set_num_threads(threads or os.cpu_count() or 1)
        self.cores = torch.get_num_threads()
        self.ref = reference_modules()
        self.kind = "reference" if self.ref is not None else "port"
        s = sample
        if self.ref is not None:
            cso = self.ref["compton_sparse_ops"]
            self.projector = cso.build_compton_sparse_projector(s.coor, theta_stride=CONFIG3["theta_stride"],
                                                                z_stride=1, rotate_num=1)
        else:
            from oracle import sparse as osp

            self.projector = osp.build_projector(s.coor.numpy(), theta_stride=CONFIG3["theta_stride"], z_stride=1,
                                                 rotate_num=1)
            self.np = dict(A=s.A.numpy(), y=s.y.numpy(), x=s.x.numpy(), rows=s.rows.numpy(), eff=s.eff.numpy(),
                           s=s.s.numpy())

    # one timed call of each part, seconds
    def sc_half(self):
        t0 = time.perf_counter()
        if self.ref is not None:
            w = self.ref["recon_osem_local_sparse_jsccsd_only"].get_weight_single(self.smp.A, self.smp.y, self.smp.x)
        else:
            from oracle import osem_sc

            w = osem_sc.get_weight_single(self.np["A"], self.np["y"], self.np["x"], floor=1e-12, dtype=np.float32)
        return time.perf_counter() - t0, w

    def compton_grouped(self):
        t0 = time.perf_counter()
        if self.ref is not None:
            w = self.ref["recon_osem_plane_sparse"].get_weight_compton_sparse(self.smp.rows, self.smp.eff, self.smp.x,
                                                                              self.projector)
        else:
            from oracle import sparse as osp

            w = osp.weight_grouped(self.np["rows"], self.np["eff"], self.np["x"], self.projector, dtype=np.float32)
        return time.perf_counter() - t0, w

    def compton_materialise(self):
        t0 = time.perf_counter()
        if self.ref is not None:
            w = self.ref["recon_osem_local_sparse_jsccsd_only"].get_weight_compton_sparse(
                self.smp.rows, self.smp.eff, self.smp.x, self.projector)
        else:
            from oracle import sparse as osp

            w = osp.weight_materialize(self.np["rows"], self.np["eff"], self.np["x"], self.projector,
                                       dtype=np.float32)
        return time.perf_counter() - t0, w

    def em_update(self, w):
        t0 = time.perf_counter()
        if self.ref is not None:
            self.ref["recon_osem_local_sparse_jsccsd_only"].safe_em_update(self.smp.x, torch.as_tensor(w), self.smp.s)
        else:
            from oracle import osem_sc

            osem_sc.safe_em_update(self.np["x"], np.asarray(w), self.np["s"])
        return time.perf_counter() - t0

    def step(self):
        """One step: SC half on the whole subset, both Compton forms on the sample, the
        update. Returns (wall seconds, estimated seconds of one whole subset update, parts)."""
        t0 = time.perf_counter()
        t_sc, w = self.sc_half()
        t_g, _ = self.compton_grouped()
        t_m, _ = self.compton_materialise()
        t_em = self.em_update(w)
        wall = time.perf_counter() - t0
        s = self.smp
        est_g = t_g * s.groups_per_subset / s.groups
        est_m = t_m * s.events_per_subset / s.events
        return wall, t_sc + min(est_g, est_m) + t_em, dict(sc=t_sc, grouped_sample=t_g, materialise_sample=t_m,
                                                            em=t_em, grouped_subset=est_g, materialise_subset=est_m)

    def describe(self, n_steps):
        s = self.smp
        who = "the reference's own functions (staged copies)" if self.ref is not None else "the oracle's numpy port"
        return (f"{n_steps} steps of {who}: SC half get_weight_single on one whole subset ({s.A.size(0)} x {s.V} "
                f"float32); Compton half on a sample of {s.groups} whole groups x {s.events // s.groups} events, "
                f"grouped form scaled by groups ({s.groups_per_subset:.1f} per subset) and materialise form by "
                f"events ({s.events_per_subset:.0f} per subset), the faster taken; safe_em_update")


def run_host(steps, warmup, threads=None):
    """Warm-up then timed steps on the host. Returns a dict for the bench line."""
    t_setup = time.perf_counter()
    timer = HostTimer(HostSample(), threads)
    setup_s = time.perf_counter() - t_setup
    for _ in range(warmup):
        timer.step()
    walls, ests, parts = [], [], []
    for _ in range(steps):
        wall, est, p = timer.step()
        walls.append(wall)
        ests.append(est)
        parts.append(p)
    est = float(np.median(ests))
    med = {k: float(np.median([p[k] for p in parts])) for k in parts[0]}
    return {"value": 1.0 / est, "unit": "subset-iters/s", "seconds_per_subset_update": est,
            "ms_per_step": 1e3 * float(np.mean(walls)), "cores": timer.cores, "cpu_model": cpu_model(),
            "kind": timer.kind, "sample": timer.describe(steps), "parts_s": med, "setup_s": setup_s}


# ------------------------------------------------------------------ the reference's PyTorch path on the GPU
def run_gpu_plain_fp32(work, subset=0, block_events=8192, sample_blocks=2, group_sample=1000):
    """The reference's own float32 torch path for one subset update of the bench workload on
    the GPU (its inputs: the float32 SC matrix, packed float32 event rows, joint sensitivity):
    the SC half (get_weight_single of recon_osem_local_sparse_jsccsd_only.py:8-10) on the whole
    subset, each Compton form on a sample scaled to the subset (the materialise form,
    osem_joint_mode_local_sparse's get_weight_compton_sparse, on `sample_blocks` blocks of
    `block_events` events, by events; the grouped form of recon_osem_plane_sparse.py:22-57 on
    the first `group_sample` groups, by groups), and safe_em_update. Each part is timed after
    one untimed call; the faster Compton form is the comparison point."""
    ref = reference_modules()
    if ref is None:
        return {"unavailable": "the reference's modules are not staged in oracle/_ref (oracle/stage_ref.py)"}
    ljs, rsp, cso = ref["recon_osem_local_sparse_jsccsd_only"], ref["recon_osem_plane_sparse"], ref["compton_sparse_ops"]
    dev = work.dev
    proj = cso.build_compton_sparse_projector(work.grid.coor.cpu(), theta_stride=4, z_stride=1, rotate_num=1).to(dev)
    A = work.A["f32"]
    ids = work.subset_ids[subset]
    rows = work.rows_f32[subset]
    x0 = torch.ones((work.V, 1), device=dev)

    def timed(fn, reps=2):
        out = None
        for _ in range(reps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize(dev)
            dt = time.perf_counter() - t0
        return dt, out

    with torch.no_grad():
        A_s, y_s = A[ids], work.proj[ids]
        t_sc, w = timed(lambda: ljs.get_weight_single(A_s, y_s, x0))
        del A_s, y_s
        n_mat = min(rows.size(0), block_events * sample_blocks)
        t_mat, _ = timed(lambda: [ljs.get_weight_compton_sparse(b, A, x0, proj)
                                  for b in torch.split(rows[:n_mat], block_events, dim=0)])
        cp1 = torch.round(rows[:, 0]).to(torch.int64)
        _, counts = torch.unique_consecutive(cp1, return_counts=True)  # rows are sorted by first-hit row
        g_total = int(counts.numel())
        g_sample = min(group_sample, g_total)
        n_grp = int(counts[:g_sample].sum())
        t_grp, _ = timed(lambda: rsp.get_weight_compton_sparse(rows[:n_grp], A, x0, proj))
        t_em, _ = timed(lambda: ljs.safe_em_update(x0, w, work.s_joint))
    n_ev = rows.size(0)
    mat = t_mat * n_ev / n_mat
    grp = t_grp * g_total / g_sample
    sec = t_sc + min(mat, grp) + t_em
    return {"value": 1.0 / sec, "unit": "subset-iters/s", "seconds_per_subset_update": sec,
            "parts_s": {"sc_half": t_sc, "em": t_em, "materialise_subset": mat, "grouped_subset": grp},
            "sample": (f"SC half on the whole subset ({ids.numel()} bins); materialise form on {n_mat} of the "
                       f"subset's {n_ev} events in blocks of {block_events}, scaled by events; grouped form on "
                       f"{g_sample} of its {g_total} groups ({n_grp} events), scaled by groups"),
            "path": ("the reference's float32 torch code on the GPU (cuBLAS GEMV for SC; Compton: the faster of "
                     "its two sparse forms, both through the dense [36,000 x 9,000] coarse-to-fine matrix)")}
