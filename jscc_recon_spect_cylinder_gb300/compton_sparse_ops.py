"""Drop-in for the reference module ``compton_sparse_ops`` (sparse Compton projector).

The projector is built on the host exactly as compton_sparse_ops.py:212-290 defines it
(ring/z layout inference, per-ring periodic theta reduce/expand, linear z reduce/expand,
stride compatibility with the rotation count, coarse coordinates) and keeps the same
dataclass fields, dense matrices included, so code that reads them still works. The
operators (:293-400) do not multiply by those dense matrices: they run the sparse maps of
``libjscc_gb300.so`` with CSR tables derived once per device from the same matrices.
Operators need CUDA tensors (no CPU fallback); error messages match the reference's.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from . import ops

RADIUS_TOL_MM = 1e-4
Z_TOL_MM = 1e-4


@dataclass
class ComptonSparseProjector:
    """Same fields as compton_sparse_ops.py:11-26."""

    theta_stride: int
    z_stride: int
    ring_strides: tuple
    fine_layer_num: int
    fine_z_num: int
    coarse_layer_num: int
    coarse_z_num: int
    fine_pixel_num: int
    coarse_pixel_num: int
    layer_reduce: torch.Tensor
    z_reduce: torch.Tensor
    layer_expand: torch.Tensor
    z_expand: torch.Tensor
    coor_coarse: torch.Tensor

    def to(self, device):
        """Copy with every tensor on ``device`` (compton_sparse_ops.py:28-44)."""
        out = ComptonSparseProjector(
            self.theta_stride, self.z_stride, self.ring_strides, self.fine_layer_num, self.fine_z_num,
            self.coarse_layer_num, self.coarse_z_num, self.fine_pixel_num, self.coarse_pixel_num,
            self.layer_reduce.to(device), self.z_reduce.to(device), self.layer_expand.to(device),
            self.z_expand.to(device), self.coor_coarse.to(device))
        cache = getattr(self, "_jscc_tables", None)
        if cache:
            out._jscc_tables = dict(cache)  # tables are keyed by device; share them
        return out


def tables(projector: ComptonSparseProjector, device) -> ops.SparseTables:
    """CSR / two-tap tables of ``projector`` on ``device`` (built once, then cached)."""
    device = torch.device(device)
    if device.type == "cuda" and device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    cache = getattr(projector, "_jscc_tables", None)
    if cache is None:
        cache = {}
        projector._jscc_tables = cache
    t = cache.get(device)
    if t is None:
        t = ops.SparseTables(projector.layer_reduce, projector.z_reduce, projector.layer_expand, projector.z_expand,
                             device)
        cache[device] = t
    return t


# ----------------------------------------------------------------------------- construction (host)
def _collect_unique_consecutive(values, tol):
    """Runs of consecutive values within ``tol`` (compton_sparse_ops.py:47-56)."""
    v = values.tolist()
    uniq, counts = [v[0]], [1]
    for a in v[1:]:
        if abs(a - uniq[-1]) <= tol:
            counts[-1] += 1
        else:
            uniq.append(a)
            counts.append(1)
    return torch.tensor(uniq, dtype=values.dtype), counts


def _infer_polar_layout(coor_full):
    """z planes (equal-sized runs of z) and rings (runs of equal radius) of a ring-major
    polar grid (compton_sparse_ops.py:59-92)."""
    if coor_full.ndim != 2 or coor_full.size(1) != 3:
        raise ValueError("coor_full must have shape [pixel_num, 3].")
    if coor_full.size(0) == 0:
        raise ValueError("coor_full is empty.")
    coor = coor_full.detach().cpu()
    z_values, z_counts = _collect_unique_consecutive(coor[:, 2], Z_TOL_MM)
    if len(set(z_counts)) != 1:
        raise ValueError("coor_full does not contain a consistent z-plane layout.")
    fine_layer_num = z_counts[0]
    radii = torch.sqrt(torch.sum(coor[:fine_layer_num, :2] ** 2, dim=1))
    rl = radii.tolist()
    lengths, ring_radii = [], []
    s = 0
    while s < fine_layer_num:
        e = s + 1
        while e < fine_layer_num and abs(rl[e] - rl[s]) <= RADIUS_TOL_MM:
            e += 1
        lengths.append(e - s)
        ring_radii.append(torch.mean(radii[s:e]))
        s = e
    return {"z_values": z_values, "fine_z_num": len(z_counts), "fine_layer_num": fine_layer_num,
            "ring_lengths": lengths, "ring_radii": torch.stack(ring_radii)}


def _check_divisible(n, stride):
    if n % stride != 0:
        raise ValueError(f"fine_num={n} is not divisible by stride={stride}.")


def _build_periodic_reduce_matrix(fine_num, stride, dtype):
    """Point sampling every ``stride`` fine angles (compton_sparse_ops.py:95-106)."""
    _check_divisible(fine_num, stride)
    nc = fine_num // stride
    m = torch.zeros((nc, fine_num), dtype=dtype)
    m[torch.arange(nc), torch.arange(nc) * stride] = 1.0
    return m


def _build_linear_reduce_matrix(fine_num, stride, dtype):
    """Linear interpolation at coarse centres (c + 1/2) stride - 1/2 (:109-129)."""
    _check_divisible(fine_num, stride)
    nc = fine_num // stride
    m = torch.zeros((nc, fine_num), dtype=dtype)
    centres = (torch.arange(nc, dtype=dtype) + 0.5) * stride - 0.5
    for c in range(nc):
        pos = centres[c].item()
        left = max(0, min(fine_num - 1, math.floor(pos)))
        right = min(fine_num - 1, left + 1)
        if right == left:
            m[c, left] = 1.0
        else:
            m[c, left] += 1.0 - (pos - left)
            m[c, right] += pos - left
    return m


def _build_periodic_expand_matrix(fine_num, stride, dtype):
    """Two-tap periodic linear interpolation from coarse samples (:132-154)."""
    _check_divisible(fine_num, stride)
    nc = fine_num // stride
    m = torch.zeros((fine_num, nc), dtype=dtype)
    for f in range(fine_num):
        left = (f // stride) % nc
        right = (left + 1) % nc
        frac = (f - left * stride) / max(stride, 1e-12)
        m[f, left] += 1.0 - frac
        m[f, right] += frac
    return m


def _build_linear_expand_matrix(fine_num, stride, dtype):
    """Two-tap linear interpolation between coarse centres, clamped at the ends (:157-185)."""
    _check_divisible(fine_num, stride)
    nc = fine_num // stride
    m = torch.zeros((fine_num, nc), dtype=dtype)
    centres = (torch.arange(nc, dtype=dtype) + 0.5) * stride - 0.5
    ins_all = torch.searchsorted(centres, torch.arange(fine_num, dtype=dtype)).tolist()
    for f, ins in enumerate(ins_all):
        if ins <= 0:
            m[f, 0] = 1.0
        elif ins >= nc:
            m[f, nc - 1] = 1.0
        else:
            lp, rp = centres[ins - 1].item(), centres[ins].item()
            wr = (float(f) - lp) / max(rp - lp, 1e-12)
            m[f, ins - 1] += 1.0 - wr
            m[f, ins] += wr
    return m


def _choose_compatible_ring_stride(ring_length, rotate_num, target_stride):
    """Largest stride <= target dividing the ring length and, when the ring turns by an
    integer number of samples per view, that per-view step too (:188-209)."""
    if target_stride <= 1:
        return 1
    step = ring_length // rotate_num if (rotate_num and rotate_num > 0 and ring_length % rotate_num == 0) else None
    for cand in range(target_stride, 0, -1):
        if ring_length % cand == 0 and (step is None or step % cand == 0):
            return cand
    return 1


def build_compton_sparse_projector(coor_full, theta_stride=2, z_stride=2, rotate_num=None, dtype=torch.float32):
    """compton_sparse_ops.py:212-290 (built on the host)."""
    if theta_stride <= 0 or z_stride <= 0:
        raise ValueError("theta_stride and z_stride must be positive.")
    layout = _infer_polar_layout(coor_full)
    z_values = layout["z_values"].to(dtype=dtype)
    nz, nl = layout["fine_z_num"], layout["fine_layer_num"]
    if nz % z_stride != 0:
        raise ValueError(f"fine_z_num={nz} is not divisible by z_stride={z_stride}.")
    red, exp, parts, strides = [], [], [], []
    for L, radius in zip(layout["ring_lengths"], layout["ring_radii"].to(dtype=dtype)):
        st = _choose_compatible_ring_stride(L, rotate_num, theta_stride) if rotate_num is not None else theta_stride
        red.append(_build_periodic_reduce_matrix(L, st, dtype))
        exp.append(_build_periodic_expand_matrix(L, st, dtype))
        strides.append(st)
        nc = L // st
        ang = torch.arange(nc, dtype=dtype) * st * (2.0 * math.pi / L)
        parts.append(torch.stack((radius * torch.cos(ang), radius * torch.sin(ang)), dim=1))
    layer_reduce = torch.block_diag(*red)
    layer_expand = torch.block_diag(*exp)
    coarse_layer = torch.cat(parts, dim=0)
    z_reduce = _build_linear_reduce_matrix(nz, z_stride, dtype)
    z_expand = _build_linear_expand_matrix(nz, z_stride, dtype)
    coarse_z = torch.matmul(z_reduce, z_values.unsqueeze(1)).squeeze(1)
    coor_coarse = torch.cat([torch.cat((coarse_layer, torch.full((coarse_layer.size(0), 1), z.item(), dtype=dtype)),
                                       dim=1) for z in coarse_z], dim=0)
    ncl, ncz = coarse_layer.size(0), coarse_z.numel()
    return ComptonSparseProjector(theta_stride, z_stride, tuple(strides), nl, nz, ncl, ncz, nl * nz, ncl * ncz,
                                  layer_reduce, z_reduce, layer_expand, z_expand, coor_coarse)


@dataclass
class RadialComptonSparseProjector(ComptonSparseProjector):
    """A projector that also coarsens the rings of each z plane (an extension: the
    reference's builder coarsens theta and z only). The separable pair keeps the reference's
    fields with the (z plane, ring) index in the z slot and one ring's theta in the layer
    slot, so every operator of this module and every kernel take it unchanged:
    fine_layer_num is the ring length, fine_z_num the planes x rings (coarse likewise)."""

    radial_stride: int = 1
    ring_num: int = 0

    def to(self, device):
        base = ComptonSparseProjector.to(self, device)
        out = RadialComptonSparseProjector(**{f: getattr(base, f) for f in base.__dataclass_fields__},
                                           radial_stride=self.radial_stride, ring_num=self.ring_num)
        if getattr(base, "_jscc_tables", None):
            out._jscc_tables = base._jscc_tables
        return out


def build_compton_sparse_projector_radial(coor_full, radial_stride=4, theta_stride=4, dtype=torch.float32):
    """Radially and angularly coarsened projector of a polar grid whose rings all have one
    length L (e.g. 100 x 360 -> 25 x 90 with strides 4 and 4): each z plane's rings are
    coarsened by `radial_stride` with the reference's linear reduce / expand along the ring
    index (its z convention: samples at (c + 1/2) s - 1/2, two-tap interpolation between
    them, clamped at the ends), each ring's theta by `theta_stride` with its periodic maps.
    The coarse coordinates: radius = the linear reduce of the ring radii, angle
    th_c * s_theta * 2 pi / L, the plane's z. With radial_stride 1 the upsample and the
    coarse coordinates equal build_compton_sparse_projector(..., theta_stride, z_stride=1)'s."""
    if radial_stride <= 0 or theta_stride <= 0:
        raise ValueError("radial_stride and theta_stride must be positive.")
    layout = _infer_polar_layout(coor_full)
    lengths = layout["ring_lengths"]
    L = lengths[0]
    if any(n != L for n in lengths):
        raise ValueError("radial coarsening needs rings of one length.")
    n_rings, nz = len(lengths), layout["fine_z_num"]
    if n_rings % radial_stride != 0:
        raise ValueError(f"ring count {n_rings} is not divisible by radial_stride={radial_stride}.")
    ring_reduce = _build_linear_reduce_matrix(n_rings, radial_stride, dtype)
    ring_expand = _build_linear_expand_matrix(n_rings, radial_stride, dtype)
    planes = torch.eye(nz, dtype=dtype)
    z_reduce = torch.kron(planes, ring_reduce)
    z_expand = torch.kron(planes, ring_expand)
    layer_reduce = _build_periodic_reduce_matrix(L, theta_stride, dtype)
    layer_expand = _build_periodic_expand_matrix(L, theta_stride, dtype)
    n_thc = L // theta_stride
    radii = torch.matmul(ring_reduce.double(), layout["ring_radii"].double()).to(dtype)
    ang = torch.arange(n_thc, dtype=dtype) * theta_stride * (2.0 * math.pi / L)
    plane = torch.cat([torch.stack((r * torch.cos(ang), r * torch.sin(ang)), dim=1) for r in radii], dim=0)
    z_values = layout["z_values"].to(dtype=dtype)
    coor_coarse = torch.cat([torch.cat((plane, torch.full((plane.size(0), 1), z.item(), dtype=dtype)), dim=1)
                             for z in z_values], dim=0)
    n_rc = n_rings // radial_stride
    return RadialComptonSparseProjector(theta_stride, 1, (theta_stride,) * n_rings, L, nz * n_rings, n_thc, nz * n_rc,
                                        nz * n_rings * L, nz * n_rc * n_thc, layer_reduce, z_reduce, layer_expand,
                                        z_expand, coor_coarse, radial_stride=radial_stride, ring_num=n_rings)


# ----------------------------------------------------------------------------- operators (GPU)
def _tables_for(t, projector):
    return tables(projector, t.device)


def reduce_fine_image_to_coarse(img_fine, projector):
    """compton_sparse_ops.py:293-302."""
    if img_fine.ndim != 2 or img_fine.size(1) != 1:
        raise ValueError("img_fine must have shape [fine_pixel_num, 1].")
    if img_fine.size(0) != projector.fine_pixel_num:
        raise ValueError("img_fine size does not match projector.fine_pixel_num.")
    tb = _tables_for(img_fine, projector)
    out = ops.sparse_map(img_fine.reshape(1, -1), tb.red, projector.coarse_z_num, projector.fine_z_num,
                         projector.coarse_layer_num, projector.fine_layer_num)
    return out.reshape(-1, 1)


def upsample_coarse_weight_to_fine(weight_coarse, projector):
    """compton_sparse_ops.py:305-314."""
    if weight_coarse.ndim != 2 or weight_coarse.size(1) != 1:
        raise ValueError("weight_coarse must have shape [coarse_pixel_num, 1].")
    if weight_coarse.size(0) != projector.coarse_pixel_num:
        raise ValueError("weight_coarse size does not match projector.coarse_pixel_num.")
    tb = _tables_for(weight_coarse, projector)
    out = ops.sparse_map(weight_coarse.reshape(1, -1), tb.red_t, projector.fine_z_num, projector.coarse_z_num,
                         projector.fine_layer_num, projector.coarse_layer_num)
    return out.reshape(-1, 1)


def reduce_fine_rows_to_coarse(rows_fine, projector, row_idx=None):
    """compton_sparse_ops.py:317-328. ``row_idx`` (extension) gathers the input rows
    without copying them (the sparse builder reduces sysmat[cp1 - 1])."""
    if rows_fine.ndim != 2:
        raise ValueError("rows_fine must have shape [num_rows, fine_pixel_num].")
    if rows_fine.size(1) != projector.fine_pixel_num:
        raise ValueError("rows_fine size does not match projector.fine_pixel_num.")
    tb = _tables_for(rows_fine, projector)
    return ops.sparse_map(rows_fine, tb.red, projector.coarse_z_num, projector.fine_z_num,
                          projector.coarse_layer_num, projector.fine_layer_num, row_idx=row_idx)


def upsample_coarse_rows_to_fine(rows_coarse, projector):
    """compton_sparse_ops.py:331-342."""
    if rows_coarse.ndim != 2:
        raise ValueError("rows_coarse must have shape [num_rows, coarse_pixel_num].")
    if rows_coarse.size(1) != projector.coarse_pixel_num:
        raise ValueError("rows_coarse size does not match projector.coarse_pixel_num.")
    tb = _tables_for(rows_coarse, projector)
    return ops.sparse_map(rows_coarse, tb.up, projector.fine_z_num, projector.coarse_z_num,
                          projector.fine_layer_num, projector.coarse_layer_num)


def project_fine_rows_to_coarse_adjoint(rows_fine, projector):
    """compton_sparse_ops.py:345-356 (exact adjoint of upsample_coarse_rows_to_fine)."""
    if rows_fine.ndim != 2:
        raise ValueError("rows_fine must have shape [num_rows, fine_pixel_num].")
    if rows_fine.size(1) != projector.fine_pixel_num:
        raise ValueError("rows_fine size does not match projector.fine_pixel_num.")
    tb = _tables_for(rows_fine, projector)
    return ops.sparse_map(rows_fine, tb.adj, projector.coarse_z_num, projector.fine_z_num,
                          projector.coarse_layer_num, projector.fine_layer_num)


def pack_sparse_event_rows(cpnum1, t_compton):
    """compton_sparse_ops.py:359-368: column 0 holds cp1 as float."""
    if cpnum1.ndim != 1:
        raise ValueError("cpnum1 must have shape [num_events].")
    if t_compton.ndim != 2:
        raise ValueError("t_compton must have shape [num_events, coarse_pixel_num].")
    if cpnum1.size(0) != t_compton.size(0):
        raise ValueError("cpnum1 and t_compton must have the same number of rows.")
    if t_compton.dtype != torch.float32:
        return torch.cat((cpnum1.to(dtype=t_compton.dtype).unsqueeze(1), t_compton), dim=1)
    return ops.sparse_pack(cpnum1, t_compton)


def unpack_sparse_event_rows(event_rows):
    """compton_sparse_ops.py:371-377: (round(column 0) as int64, view of the rest)."""
    if event_rows.ndim != 2 or event_rows.size(1) < 2:
        raise ValueError("event_rows must have shape [num_events, 1 + coarse_pixel_num].")
    return ops.sparse_unpack_ids(event_rows), event_rows[:, 1:]


def materialize_sparse_event_rows_to_fine(event_rows, sysmat, projector):
    """compton_sparse_ops.py:380-400 -> (t_norm of the valid rows, valid mask)."""
    if event_rows.ndim != 2 or event_rows.size(1) != projector.coarse_pixel_num + 1:
        raise ValueError("event_rows size does not match sparse projector.")
    if sysmat.ndim != 2 or sysmat.size(1) != projector.fine_pixel_num:
        raise ValueError("sysmat size does not match sparse projector.")
    if event_rows.device != sysmat.device:
        raise ValueError("event_rows and sysmat must be on the same device.")
    if projector.coor_coarse.device != event_rows.device:
        raise ValueError("projector must be on the same device as event_rows.")
    fine, rsum = ops.sparse_materialize(event_rows, sysmat, _tables_for(event_rows, projector))
    valid = torch.isfinite(rsum) & (rsum > 0)
    return fine[valid] / rsum[valid].unsqueeze(1), valid
