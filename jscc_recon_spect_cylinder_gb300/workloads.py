"""Benchmark workloads built on the GPU from the seeded synthetic generators.

JointWorkload is the JSCCSD joint configuration: an SC channel of `views` x 4,096 pixels
(32 axial x 128 azimuthal on a 120 mm cylinder) against a 100 x 360 polar grid, stored in
the flat form (all views are rows of one matrix, identity rotation tables), and a sparse
Compton channel: two-interaction events (scatter cylinder r = 120 mm, absorber cylinder
r = 150 mm, same pixelation), forward-simulated from the hot-rod phantom, built into packed
coarse rows by the sparse T builder on a theta-stride-4 grid (100 x 90 = 9,000 coarse
voxels). One OSEM step updates every subset once with
    w = alpha * w_SC + (2 - alpha) * w_Compton,  x <- safe_em_update(x, w, alpha s + (2 - alpha) d)
as osem_joint_mode_local_sparse (recon_osem_local_sparse_jsccsd_only.py:58-100) does, with the
SC forward projection floored at 1e-12 and the Compton weight in the materialise form.
"""
from __future__ import annotations

import math

import torch

from . import compton_sparse_ops as cso
from . import ops, synthetic
from .process_list_plane_sparse import build_sparse_rows_from_smeared
from .recon_osem_plane import split_tensor_even

N_PHI, N_AXIAL, AXIAL_PITCH = 128, 32, 2.0


def _upsample_sparse(tables, device):
    """The fine <- coarse upsample U = Z (x) L of a projector's separable pair (the z map
    and the layer map, CSR on the host) as a float64 torch sparse matrix [V_f, V_c]:
    U[zf * n_lf + lf, zc * n_lc + lc] = Z[zf, zc] * L[lf, lc]."""
    def coo(csr):
        ptr, idx, w = (t.cpu() for t in csr)
        rows = torch.repeat_interleave(torch.arange(ptr.numel() - 1), (ptr[1:] - ptr[:-1]).long())
        return rows, idx.long(), w.double()

    zr, zc, zw = coo(tables.up[0])
    lr, lc, lw = coo(tables.up[1])
    rows = (zr[:, None] * tables.n_lf + lr[None, :]).reshape(-1)
    cols = (zc[:, None] * tables.n_lc + lc[None, :]).reshape(-1)
    vals = (zw[:, None] * lw[None, :]).reshape(-1)
    U = torch.sparse_coo_tensor(torch.stack((rows, cols)), vals,
                                (tables.n_zf * tables.n_lf, tables.n_zc * tables.n_lc))
    return U.coalesce().to(device)


SCAT_R, ABS_R = 120.0, 150.0


class JointWorkload:
    def __init__(self, device, views=20, n_events=1_000_000, subsets=8, alpha=0.5, theta_stride=4, e0=0.662,
                 res_662=0.08, delta_r=1.0, n_r=100, n_theta=360, radius=100.0, sc_counts=1e7, seed=synthetic.SEED,
                 with_fp32=True, sort_events=True, radial_stride=1):
        self.dev = device
        self.subsets = subsets
        self.alpha = alpha
        self.views = views
        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
        grid = synthetic.polar_grid(n_r, n_theta, radius, device=device)
        self.grid = grid
        self.V = grid.n_vox
        pitch = 2.0 * math.pi * SCAT_R / N_PHI
        npix = N_PHI * N_AXIAL
        # ---------------- SC channel (flat: all views are rows)
        scat_views = [synthetic.cylinder_pixels(SCAT_R, N_PHI, N_AXIAL, AXIAL_PITCH, 2 * math.pi * v / views, device)
                      for v in range(views)]
        A = torch.cat([synthetic.sc_system_matrix(grid.coor, p, pitch * AXIAL_PITCH, radius, generator=gen)
                       for p in scat_views], dim=0)
        self.B = A.size(0)
        x_true = synthetic.hot_rod_phantom(grid.coor.cpu(), radius).to(device)
        self.phantom = x_true
        self.proj = synthetic.poisson_projection(A, x_true, sc_counts, generator=gen)
        gcpu = torch.Generator().manual_seed(seed)
        self.subset_ids = [ids.to(device) for ids in
                           split_tensor_even(torch.randperm(self.B, generator=gcpu), subsets, dim=0)]
        # SC subsets are addressed by bin ids into the full matrix (no per-subset copies;
        # the same rows in the same order as the copied subsets)
        self.A = {"f32": A}
        self.A["bf16"] = A.to(torch.bfloat16)
        s_sc = ops.sc_sensitivity(A)  # column sums (views are rows of the flat matrix)
        # ---------------- Compton channel
        abs_views = [synthetic.cylinder_pixels(ABS_R, N_PHI, N_AXIAL, AXIAL_PITCH, 2 * math.pi * v / views, device)
                     for v in range(views)]
        self.detector = torch.cat(scat_views + abs_views, dim=0).to(torch.float32)
        per_view = int(math.ceil(n_events / views))
        lists = []
        for v in range(views):
            got, need = [], per_view
            while need > 0:
                L = synthetic.compton_list(grid.coor, x_true, scat_views[v], ABS_R, N_PHI, N_AXIAL, AXIAL_PITCH, e0,
                                           int(need * 2.3) + 64, gen, cp1_offset=v * npix,
                                           cp2_offset=views * npix + v * npix, abs_phi0=2 * math.pi * v / views)
                got.append(L[:need])
                need -= got[-1].size(0)
            lists.append(torch.cat(got))
        lst = torch.cat(lists)[:n_events]
        self.n_list = lst.size(0)
        res = res_662 * (0.662 / e0) ** 0.5
        noise = torch.randn((lst.size(0), 2), generator=gen, device=device)
        for k, col in ((0, 1), (1, 3)):
            e = lst[:, col]
            lst[:, col] = e + (e * res / 2.355 * (e0 / e) ** 0.5) * noise[:, k]
        if radial_stride > 1:  # the radially coarsened extension (e.g. 25 x 90 for strides 4 x 4)
            self.projector = cso.build_compton_sparse_projector_radial(grid.coor.cpu(), radial_stride, theta_stride)
        else:
            self.projector = cso.build_compton_sparse_projector(grid.coor.cpu(), theta_stride=theta_stride, z_stride=1,
                                                                rotate_num=1)
        self.tables = cso.tables(self.projector, device)
        thr_max = 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001
        rows = build_sparse_rows_from_smeared(A, self.detector, self.projector, lst, delta_r, delta_r, e0, res,
                                              thr_max, 0.05, e0 - 0.06)
        self.n_events = rows.size(0)
        self.Vc = self.projector.coarse_pixel_num
        parts = split_tensor_even(rows, subsets, dim=0)
        if sort_events:
            # events of a subset ordered by first-hit row: the efficiency row (a sysmat row)
            # is then reused from L2 by consecutive events; the weight is a sum over the
            # subset's events, so the order only changes float32 rounding
            parts = [p[torch.argsort(p[:, 0], stable=True)] for p in parts]
        # packed float32 rows (the reference's layout: the float64 reference and the oracle
        # read them) and split storage for the product path, float32 and BF16 coarse rows
        # behind the same int32 row ids
        self.rows_f32 = [p.contiguous() for p in parts] if with_fp32 else None
        split = [ops.split_sparse_rows(p, torch.bfloat16) for p in parts]
        self.ids = [s[0] for s in split]
        self.tc_bf16 = [s[1] for s in split]
        self.tc_f32 = [ops.split_sparse_rows(p, torch.float32)[1] for p in parts] if with_fp32 else None
        del rows, parts
        # ---------------- sensitivities: s (SC column sums), d (Compton, build_sparse_sensi_d
        # rescaling: sum(d) = sum(s) * E_C / E_S), joint s_j = alpha s + (2 - alpha) d
        d = torch.zeros((self.V, 1), dtype=torch.float32, device=device)
        for k in range(subsets):
            if self.rows_f32 is not None:
                ops.sparse_sensitivity(A, self.tables, rows=self.rows_f32[k], out=d)
            else:
                ops.sparse_sensitivity(A, self.tables, row_id=self.ids[k], t_coarse=self.tc_bf16[k], out=d)
        if d.sum() > 0:
            d = d * s_sc.sum() / d.sum() * (self.n_events / max(float(self.proj.sum()), 1.0))
        else:
            d = s_sc.clone()
        self.s_sc, self.s_d = s_sc, d
        self.s_joint = (alpha * s_sc + (2 - alpha) * d).contiguous()
        if not with_fp32:
            del self.A["f32"]
        torch.cuda.synchronize(device)

    # -------------------------------------------------------------------------------- step
    def subset_update(self, img, s, dtype="bf16"):
        """One subset update: w = alpha w_SC + (2 - alpha) w_Compton, safe EM update."""
        A_eff = self.A[dtype]
        w = torch.zeros_like(img)
        ops.sc_weight(A_eff, self.proj, img, floor=1e-12, scale=self.alpha, out=w, row_idx=self.subset_ids[s])
        tc = self.tc_bf16[s] if dtype == "bf16" else self.tc_f32[s]
        ops.sparse_weight_split(self.ids[s], tc, A_eff, self.tables, img, grouped=False, scale=2 - self.alpha, out=w)
        return ops.em_update(img, w, self.s_joint, safe=True)

    def step(self, img, dtype="bf16"):
        """One OSEM iteration (every subset updated once)."""
        for s in range(self.subsets):
            img = self.subset_update(img, s, dtype)
        return img

    def fp64_reference(self, iters):
        """The same iterations in float64 with torch on the GPU (dense float64 matrix
        products; the upsample as a float64 sparse matrix), from the float32-stored inputs."""
        U = _upsample_sparse(self.tables, self.dev)
        x = torch.ones((self.V, 1), dtype=torch.float64, device=self.dev)
        A = self.A["f32"]
        s = self.s_joint.double()
        for _ in range(iters):
            for k in range(self.subsets):
                ids = self.subset_ids[k]
                w = torch.zeros_like(x)
                for a in range(0, ids.numel(), 4096):
                    Ab = A[ids[a:a + 4096]].double()
                    f = torch.clamp(Ab @ x, min=1e-12)
                    w += self.alpha * (Ab.t() @ (self.proj[ids[a:a + 4096]].double() / f))
                rows = self.rows_f32[k]
                for a in range(0, rows.size(0), 4096):
                    r = rows[a:a + 4096]
                    cp1 = torch.clamp(torch.round(r[:, 0]).long() - 1, 0, A.size(0) - 1)
                    t = torch.sparse.mm(U, r[:, 1:].double().t()).t() * A[cp1].double()
                    t = torch.nan_to_num(t, nan=0.0, posinf=0.0, neginf=0.0)
                    rs = t.sum(dim=1, keepdim=True)
                    ok = torch.isfinite(rs[:, 0]) & (rs[:, 0] > 0)
                    tn = t[ok] / rs[ok]
                    wc = tn.t() @ (1.0 / torch.clamp(tn @ x, min=1e-12))
                    w += (2 - self.alpha) * torch.nan_to_num(wc, nan=0.0, posinf=0.0, neginf=0.0)
                w = torch.nan_to_num(w, nan=0.0, posinf=0.0, neginf=0.0)
                valid = s > 1e-12
                x = torch.where(valid, x * torch.clamp(w, min=0.0) / torch.where(valid, s, torch.ones_like(s)),
                                torch.zeros_like(x))
        return x

    def units_per_step(self):
        return self.subsets

    def pair_count_per_step(self):
        """Event x fine-voxel pairs evaluated per step (forward + back of every event)."""
        return 2 * self.n_events * self.V

    def sc_kernel_bytes(self, dtype):
        """Algorithmic bytes of one subset's SC launches: the two-pass forward (rows + image)
        and back (rows + ratios), or the fused single-read kernel (rows once + image +
        projections)."""
        b = 2 if dtype == "bf16" else 4
        rows = self.B / self.subsets
        return {"sc_forward_split": rows * self.V * b + self.V * 4, "sc_back_partial": rows * self.V * b + rows * 4,
                "sc_fused": rows * self.V * b + self.V * 4 + rows * 4}

    def sparse_kernel_bytes(self, dtype):
        """Algorithmic bytes of one launch of the grouped sparse kernels (one subset, the
        subset's mean event and group counts): sparse_group_adjoint reads one sysmat row per
        group (distinct first-hit row) and writes its float32 adjoint b_g [V_c];
        sparse_group_coef reads every coarse row and its event sum once and b_g per group, and
        writes q (float32 [groups, V_c]); sparse_group_scatter reads one sysmat row and one q
        row per group and writes one float32 partial image per group chunk (16 chunks)."""
        b = 2 if dtype == "bf16" else 4
        ev = self.n_events / self.subsets
        groups = float(sum(torch.unique(i).numel() for i in self.ids)) / self.subsets
        adjoint = groups * (self.V * b + self.Vc * 4)
        coef = ev * (self.Vc * b + 4) + groups * 2 * self.Vc * 4
        scatter = groups * (self.V * b + self.Vc * 4) + 16 * self.V * 4
        # the fused cluster kernel: every coarse row and its event sum once, one sysmat row per
        # group, one float32 partial image per cluster (at most 38 clusters of four CTAs)
        fused = ev * (self.Vc * b + 4) + groups * self.V * b + 38 * self.V * 4
        return {"sparse_group_adjoint": adjoint, "sparse_group_coef": coef, "sparse_group_scatter": scatter,
                "sparse_group_fused": fused}

    def group_count(self):
        """Mean number of groups (distinct first-hit rows) per subset."""
        return float(sum(torch.unique(i).numel() for i in self.ids)) / self.subsets
