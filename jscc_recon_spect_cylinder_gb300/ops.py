"""Tensor-level wrappers over the C-ABI kernels (CUDA tensors in, CUDA tensors out).

These are the building blocks the reference-mirroring modules call. Shapes follow
the reference: images are ``[V, 1]`` float32, rotation tables ``[V, R]`` int64
1-based, system matrices ``[B, V]`` row-major (float32 or bfloat16).
"""
from __future__ import annotations

import torch

from . import _lib


def _dtype_code(t: torch.Tensor) -> int:
    if t.dtype == torch.float32:
        return _lib.DTYPE_F32
    if t.dtype == torch.bfloat16:
        return _lib.DTYPE_BF16
    raise ValueError(f"unsupported system-matrix dtype {t.dtype} (float32 or bfloat16)")


def _rows_contig(t: torch.Tensor) -> torch.Tensor:
    """Row-major with unit column stride (a leading dimension is allowed)."""
    if t.dim() == 2 and t.stride(1) == 1 and t.stride(0) >= t.size(1):
        return t
    return t.contiguous()


def _f32_contig(t: torch.Tensor) -> torch.Tensor:
    if t.dtype != torch.float32:
        t = t.float()
    return t.contiguous()


def _is_identity(t: torch.Tensor, rot_start: int, n_rot: int) -> bool:
    """True when columns rot_start..rot_start+n_rot-1 of a 1-based table are all the
    identity. Checked once per (table object, version, column range); the first
    check synchronises the device, so call once before capturing a CUDA graph."""
    per_table = getattr(t, "_jscc_identity", None)
    if per_table is None:
        per_table = {}
        t._jscc_identity = per_table  # lives and dies with the table object
    key = (t._version, rot_start, n_rot)
    hit = per_table.get(key)
    if hit is None:
        ar = torch.arange(1, t.size(0) + 1, device=t.device, dtype=t.dtype).unsqueeze(1)
        hit = bool((t[:, rot_start:rot_start + n_rot] == ar).all().item())
        per_table[key] = hit
    return hit


def _index_table(t: torch.Tensor | None, n_vox: int, name: str) -> torch.Tensor | None:
    if t is None:
        return None
    if t.dim() != 2 or t.size(0) != n_vox:
        raise ValueError(f"{name} must be [voxels, rotations] with {n_vox} rows")
    if t.dtype != torch.int64:
        t = t.to(torch.int64)
    if t.stride(1) != 1:
        t = t.contiguous()
    return t


def sc_weight(
    sysmat: torch.Tensor,
    proj: torch.Tensor,
    img: torch.Tensor,
    rotmat: torch.Tensor | None = None,
    rotmat_inv: torch.Tensor | None = None,
    rot_start: int = 0,
    n_rot: int | None = None,
    floor: float | None = None,
    scale: float = 1.0,
    out: torch.Tensor | None = None,
    row_idx: torch.Tensor | None = None,
    proj_col: int | None = None,
) -> torch.Tensor:
    """``out += scale * sum_r rotinv_r( A^T (proj[:, r] / A rot_r(img)) )``.

    ``row_idx`` (int64, 0-based, on the device) restricts A and proj to those rows
    without copying them; ids must be in range. ``proj_col`` overrides the first
    projection column used (default ``rot_start``), e.g. 0 for a single shared
    column of ones in the dense-T Compton weight.

    Rotations ``r = rot_start .. rot_start + n_rot - 1`` use column ``r`` of
    ``proj``, ``rotmat`` and ``rotmat_inv`` (no copies are made). With ``rotmat``
    None there is one identity rotation and ``proj`` may be ``[B]`` or ``[B, k]``
    (column ``rot_start`` is used). ``floor`` applies ``clamp_min(floor)`` to the
    forward projection (recon_osem_local_cntstat.py:7).
    """
    dev = _lib.require_cuda(sysmat, proj, img, rotmat, rotmat_inv, out, what="sc_weight")
    if sysmat.dim() != 2:
        raise ValueError("sysmat must be 2-D [bins, voxels]")
    A = _rows_contig(sysmat)
    n_rows, n_vox = A.shape
    if proj.dim() == 1:
        proj = proj.unsqueeze(1)
    p = proj if (proj.dtype == torch.float32 and (proj.stride(1) == 1 or proj.size(1) == 1)) else _f32_contig(proj)
    if p.size(0) != n_rows:
        raise ValueError(f"proj has {p.size(0)} rows, sysmat has {n_rows}")
    if row_idx is not None:
        _lib.require_cuda(row_idx, sysmat, what="sc_weight")
        row_idx = row_idx.to(torch.int64).contiguous()
        n_bins = row_idx.numel()
    else:
        n_bins = n_rows
    rotmat = _index_table(rotmat, n_vox, "rotmat")
    rotmat_inv = _index_table(rotmat_inv, n_vox, "rotmat_inv")
    if (rotmat is None) != (rotmat_inv is None):
        raise ValueError("rotmat and rotmat_inv must be given together")
    if rotmat is None:
        n_rot = 1
    else:
        if rotmat.shape != rotmat_inv.shape:
            raise ValueError("rotmat_inv must match rotmat's shape")
        if n_rot is None:
            n_rot = rotmat.size(1) - rot_start
        if rot_start < 0 or n_rot < 1 or rot_start + n_rot > rotmat.size(1):
            raise ValueError(f"rotation range [{rot_start}, {rot_start + (n_rot or 0)}) out of range")
    col0 = rot_start if proj_col is None else proj_col
    if col0 < 0 or col0 + n_rot > p.size(1):
        raise ValueError("proj has fewer columns than the requested rotations")
    x = img.reshape(-1)
    if x.dtype != torch.float32 or not x.is_contiguous():
        x = _f32_contig(x)
    if x.numel() != n_vox:
        raise ValueError(f"img has {x.numel()} voxels, sysmat has {n_vox}")
    if out is None:
        out = torch.zeros((n_vox, 1), dtype=torch.float32, device=dev)
    if out.dtype != torch.float32 or not out.is_contiguous() or out.numel() != n_vox:
        raise ValueError("out must be a contiguous float32 tensor with one entry per voxel")
    lib = _lib.load()
    nbytes = lib.jscc_sc_weight_workspace_bytes(n_bins, n_vox, n_rot)
    ws = _lib.workspace.get(dev, nbytes)
    p_ptr = p.data_ptr() + col0 * p.element_size() * p.stride(1)
    rm_ptr = None if rotmat is None else rotmat.data_ptr() + rot_start * 8
    ri_ptr = None if rotmat_inv is None else rotmat_inv.data_ptr() + rot_start * 8
    if rotmat is not None and rotmat.stride(0) != rotmat_inv.stride(0):
        rotmat_inv = rotmat_inv.contiguous()
        rotmat = rotmat.contiguous()
        rm_ptr = rotmat.data_ptr() + rot_start * 8
        ri_ptr = rotmat_inv.data_ptr() + rot_start * 8
    if rotmat is not None and _is_identity(rotmat, rot_start, n_rot) and _is_identity(rotmat_inv, rot_start, n_rot):
        rm_ptr = ri_ptr = None  # identity views: no gather / scatter passes
    ld_rot = 0 if rotmat is None else rotmat.stride(0)
    rc = lib.jscc_sc_weight(
        A.data_ptr(), _dtype_code(A), A.stride(0), _lib.ptr(row_idx), n_bins, n_vox,
        p_ptr, p.stride(0), n_rot, x.data_ptr(), rm_ptr, ri_ptr, ld_rot,
        1 if floor is not None else 0, float(floor) if floor is not None else 0.0, float(scale),
        out.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle(dev),
    )
    _lib.check(rc, "jscc_sc_weight")
    return out


def em_update(
    img: torch.Tensor,
    weight: torch.Tensor,
    s_map: torch.Tensor,
    safe: bool,
    coef: float | None = None,
    weight_b: torch.Tensor | None = None,
    coef_b: float = 0.0,
    eps: float = 1e-12,
    out: torch.Tensor | None = None,
) -> torch.Tensor:
    """EM update ``img * w / s`` (``safe=False``) or ``safe_em_update`` (``safe=True``)
    with ``w = coef * weight + coef_b * weight_b`` (``coef`` None: unscaled)."""
    dev = _lib.require_cuda(img, weight, s_map, weight_b, out, what="em_update")
    n = img.numel()
    for name, t in (("weight", weight), ("s_map", s_map), ("weight_b", weight_b)):
        if t is not None and t.numel() != n:
            raise ValueError(f"{name} has {t.numel()} entries, img has {n}")
    x = _f32_contig(img)
    w = _f32_contig(weight)
    s = _f32_contig(s_map)
    wb = _f32_contig(weight_b) if weight_b is not None else None
    if out is None:
        out = torch.empty_like(x)
    rc = _lib.load().jscc_em_update(
        out.data_ptr(), x.data_ptr(), w.data_ptr(), 0 if coef is None else 1,
        0.0 if coef is None else float(coef), _lib.ptr(wb), float(coef_b), s.data_ptr(), n,
        _lib.EM_SAFE if safe else _lib.EM_PLAIN, float(eps), _lib.stream_handle(dev),
    )
    _lib.check(rc, "jscc_em_update")
    return out.view_as(img) if out.shape != img.shape else out
