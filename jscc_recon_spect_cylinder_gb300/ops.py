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


def _rot_tables(rot, n_vox, n_rot, name):
    t = _index_table(rot, n_vox, name)
    if t is None:
        return None, 1, 0
    n = t.size(1) if n_rot is None else n_rot
    if n < 1 or n > t.size(1):
        raise ValueError(f"n_rot={n} out of range")
    return t, n, t.stride(0)


def sc_project(sysmat, img, rotmat=None, n_rot=None, row_idx=None):
    """Forward SC projection ``f[b, r] = A[b] . rot_r(img)`` -> ``[n_bins, n_rot]``
    (jscc_sc_project; a float64 image selects jscc_sc_project_f64 and a float64 result)."""
    dev = _lib.require_cuda(sysmat, img, rotmat, row_idx, what="sc_project")
    A = _rows_contig(sysmat)
    n_rows, n_vox = A.shape
    if row_idx is not None:
        row_idx = row_idx.to(torch.int64).contiguous()
    n_bins = n_rows if row_idx is None else row_idx.numel()
    rm, n_rot, ld_rot = _rot_tables(rotmat, n_vox, n_rot, "rotmat")
    if img.dtype == torch.float64:
        x = img.reshape(-1).contiguous()
        if x.numel() != n_vox:
            raise ValueError(f"img has {x.numel()} voxels, sysmat has {n_vox}")
        out = torch.empty((n_bins, n_rot), dtype=torch.float64, device=dev)
        rc = _lib.load().jscc_sc_project_f64(A.data_ptr(), _dtype_code(A), A.stride(0), _lib.ptr(row_idx), n_bins,
                                             n_vox, n_rot, x.data_ptr(), _lib.ptr(rm), ld_rot, out.data_ptr(),
                                             out.stride(0), _lib.stream_handle(dev))
        _lib.check(rc, "jscc_sc_project_f64")
        return out
    x = _f32_contig(img.reshape(-1))
    if x.numel() != n_vox:
        raise ValueError(f"img has {x.numel()} voxels, sysmat has {n_vox}")
    out = torch.empty((n_bins, n_rot), dtype=torch.float32, device=dev)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_sc_weight_workspace_bytes(n_bins, n_vox, n_rot))
    rc = lib.jscc_sc_project(A.data_ptr(), _dtype_code(A), A.stride(0), _lib.ptr(row_idx), n_bins, n_vox, n_rot,
                             x.data_ptr(), _lib.ptr(rm), ld_rot, out.data_ptr(), out.stride(0), ws.data_ptr(),
                             ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sc_project")
    return out


def sc_backproject(sysmat, g, rotmat_inv=None, n_rot=None, row_idx=None, scale=1.0, out=None):
    """Adjoint of sc_project: ``out += scale * sum_r rotinv_r(A^T g[:, r])`` (jscc_sc_backproject;
    a float64 ``g`` selects jscc_sc_backproject_f64 and a float64 result)."""
    dev = _lib.require_cuda(sysmat, g, rotmat_inv, row_idx, out, what="sc_backproject")
    A = _rows_contig(sysmat)
    n_rows, n_vox = A.shape
    if row_idx is not None:
        row_idx = row_idx.to(torch.int64).contiguous()
    n_bins = n_rows if row_idx is None else row_idx.numel()
    ri, n_rot, ld_rot = _rot_tables(rotmat_inv, n_vox, n_rot, "rotmat_inv")
    if g.dtype == torch.float64:
        gg = g.reshape(n_bins, -1).contiguous()
        if gg.size(1) < n_rot:
            raise ValueError(f"g has {gg.size(1)} columns, {n_rot} rotations requested")
        if out is None:
            out = torch.zeros((n_vox, 1), dtype=torch.float64, device=dev)
        lib = _lib.load()
        ws = _lib.workspace.get(dev, lib.jscc_sc_f64_workspace_bytes(n_vox, n_rot))
        rc = lib.jscc_sc_backproject_f64(A.data_ptr(), _dtype_code(A), A.stride(0), _lib.ptr(row_idx), n_bins, n_vox,
                                         n_rot, gg.data_ptr(), gg.stride(0), _lib.ptr(ri), ld_rot, float(scale),
                                         out.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
        _lib.check(rc, "jscc_sc_backproject_f64")
        return out
    gg = _f32_contig(g.reshape(n_bins, -1))
    if gg.size(1) < n_rot:
        raise ValueError(f"g has {gg.size(1)} columns, {n_rot} rotations requested")
    if out is None:
        out = torch.zeros((n_vox, 1), dtype=torch.float32, device=dev)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_sc_weight_workspace_bytes(n_bins, n_vox, n_rot))
    rc = lib.jscc_sc_backproject(A.data_ptr(), _dtype_code(A), A.stride(0), _lib.ptr(row_idx), n_bins, n_vox, n_rot,
                                 gg.data_ptr(), gg.stride(0), _lib.ptr(ri), ld_rot, float(scale), out.data_ptr(),
                                 ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sc_backproject")
    return out


def compton_project(records, row_id, coor, img, model=_lib.CONE_STRICT, eff=None, use_window=False, rotmat=None,
                    rot_col=0):
    """Forward list-mode projection ``f[i] = sum_j t_ij rot(img)_j`` with T recomputed
    (jscc_compton_project) -> ``[E]``; a float64 image selects jscc_compton_project_f64 (strict
    model, no rotation) and a float64 result."""
    dev = _lib.require_cuda(records, row_id, coor, img, eff, rotmat, what="compton_project")
    c = _f32_contig(coor)
    V = c.size(0)
    if img.dtype == torch.float64:
        if rotmat is not None:
            raise ValueError("compton_project: the float64 evaluation takes no rotation table")
        x = img.reshape(-1).contiguous()
        e, edt, ld = _eff_args(eff)
        n = records.size(0)
        f = torch.empty(n, dtype=torch.float64, device=dev)
        rc = _lib.load().jscc_compton_project_f64(records.data_ptr(), row_id.data_ptr(), n, c.data_ptr(), V, int(model),
                                                  _lib.ptr(e), edt, ld, x.data_ptr(), f.data_ptr(),
                                                  _lib.stream_handle(dev))
        _lib.check(rc, "jscc_compton_project_f64")
        return f
    x = _f32_contig(img.reshape(-1))
    rm = _index_table(rotmat, V, "rotmat")
    e, edt, ld = _eff_args(eff)
    n = records.size(0)
    perm = None
    if e is not None and n > 1:
        # events visited sorted by efficiency row (shared rows in L1/L2, as in compton_weight);
        # f is returned in the caller's event order
        records, row_id, perm = _row_sorted_events(records, row_id)
    f = torch.empty(n, dtype=torch.float32, device=dev)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_compton_weight_workspace_bytes(n, V))
    rc = lib.jscc_compton_project(records.data_ptr(), row_id.data_ptr(), n, c.data_ptr(), V, int(model),
                                  1 if use_window else 0, _lib.ptr(e), edt, ld, x.data_ptr(),
                                  None if rm is None else rm.data_ptr() + rot_col * 8, 0 if rm is None else rm.stride(0),
                                  f.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_compton_project")
    if perm is not None:
        f = torch.empty_like(f).index_copy_(0, perm, f)
    return f


def compton_backproject(records, row_id, coor, g, model=_lib.CONE_STRICT, eff=None, use_window=False, rotmat_inv=None,
                        rot_col=0, scale=1.0, out=None):
    """Adjoint of compton_project: ``out += scale * rotinv(T^T g)`` (jscc_compton_backproject; a
    float64 ``g`` selects jscc_compton_backproject_f64 and a float64 result)."""
    dev = _lib.require_cuda(records, row_id, coor, g, eff, rotmat_inv, out, what="compton_backproject")
    c = _f32_contig(coor)
    V = c.size(0)
    if g.dtype == torch.float64:
        if rotmat_inv is not None:
            raise ValueError("compton_backproject: the float64 evaluation takes no rotation table")
        e, edt, ld = _eff_args(eff)
        n = records.size(0)
        gg = g.reshape(-1).contiguous()
        if gg.numel() != n:
            raise ValueError(f"g has {gg.numel()} entries for {n} events")
        if out is None:
            out = torch.zeros((V, 1), dtype=torch.float64, device=dev)
        rc = _lib.load().jscc_compton_backproject_f64(records.data_ptr(), row_id.data_ptr(), n, c.data_ptr(), V,
                                                      int(model), _lib.ptr(e), edt, ld, gg.data_ptr(), float(scale),
                                                      out.data_ptr(), _lib.stream_handle(dev))
        _lib.check(rc, "jscc_compton_backproject_f64")
        return out
    ri = _index_table(rotmat_inv, V, "rotmat_inv")
    e, edt, ld = _eff_args(eff)
    n = records.size(0)
    gg = _f32_contig(g.reshape(-1))
    if gg.numel() != n:
        raise ValueError(f"g has {gg.numel()} entries for {n} events")
    if e is not None and n > 1:
        # the adjoint is a sum over events: visit them sorted by efficiency row
        records, row_id, perm = _row_sorted_events(records, row_id)
        gg = gg.index_select(0, perm)
    if out is None:
        out = torch.zeros((V, 1), dtype=torch.float32, device=dev)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_compton_weight_workspace_bytes(n, V))
    rc = lib.jscc_compton_backproject(records.data_ptr(), row_id.data_ptr(), n, c.data_ptr(), V, int(model),
                                      1 if use_window else 0, _lib.ptr(e), edt, ld, gg.data_ptr(),
                                      None if ri is None else ri.data_ptr() + rot_col * 8,
                                      0 if ri is None else ri.stride(0), float(scale), out.data_ptr(), ws.data_ptr(),
                                      ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_compton_backproject")
    return out


def bf16_gemm_nt(P, R, out=None, k_splits=1):
    """``out[m, n] = sum_k P[m, k] R[n, k]`` on the tensor cores (jscc_bf16_gemm_nt): P [M, K]
    and R [nr, K] BF16 with unit stride along K (row strides multiples of 8), nr <= 256;
    FP32 result [M, nr]."""
    dev = _lib.require_cuda(P, R, out, what="bf16_gemm_nt")
    if P.dtype != torch.bfloat16 or R.dtype != torch.bfloat16:
        raise ValueError("bf16_gemm_nt: P and R must be bfloat16")
    if P.dim() != 2 or R.dim() != 2 or P.size(1) != R.size(1):
        raise ValueError(f"bf16_gemm_nt: P {tuple(P.shape)} and R {tuple(R.shape)} do not share K")
    if P.stride(1) != 1 or R.stride(1) != 1:
        raise ValueError("bf16_gemm_nt: P and R need unit stride along K")
    M, K = P.shape
    nr = R.size(0)
    if out is None:
        out = torch.empty((M, nr), dtype=torch.float32, device=dev)
    if out.dtype != torch.float32 or out.stride(1) != 1 or out.size(0) != M or out.size(1) < nr:
        raise ValueError("bf16_gemm_nt: out must be float32 [M, >= nr] with unit column stride")
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_bf16_gemm_workspace_bytes(M, nr, K, int(k_splits)))
    rc = lib.jscc_bf16_gemm_nt(P.data_ptr(), P.stride(0), R.data_ptr(), R.stride(0), M, nr, K, int(k_splits),
                               out.data_ptr(), out.stride(0), ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_bf16_gemm_nt")
    return out


def rdp_prior(img, nbr, weight, gamma=2.0, beta=1.0, eps=1e-9, want_value=True, want_grad=True, grad_out=None,
              accumulate=False):
    """Relative-difference prior ``beta R(img)`` and its gradient (jscc_rdp_prior) over a
    neighbour-major table ``nbr`` [K, V] int32 / ``weight`` [K, V] float32. Returns
    ``(value, grad)``: value a float64 0-d device tensor (or None), grad [V, 1] float32
    (``grad_out`` += when ``accumulate``) or None."""
    dev = _lib.require_cuda(img, nbr, weight, grad_out, what="rdp_prior")
    f64 = img.dtype == torch.float64
    x = img.reshape(-1).contiguous() if f64 else _f32_contig(img.reshape(-1))
    rdt = torch.float64 if f64 else torch.float32
    V = x.numel()
    if nbr.dim() != 2 or nbr.size(1) != V or weight.shape != nbr.shape:
        raise ValueError(f"neighbour table {tuple(nbr.shape)} / {tuple(weight.shape)} does not match {V} voxels")
    nb = nbr.to(torch.int32).contiguous()
    wt = _f32_contig(weight)
    value = torch.zeros((), dtype=torch.float64, device=dev) if want_value else None
    grad = None
    if want_grad:
        grad = grad_out if grad_out is not None else torch.empty((V, 1), dtype=rdt, device=dev)
        if grad.numel() != V or grad.dtype != rdt or not grad.is_contiguous():
            raise ValueError(f"grad_out must be a contiguous {rdt} tensor of V elements")
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_rdp_prior_workspace_bytes(V)) if want_value else None
    rc = (lib.jscc_rdp_prior_f64 if f64 else lib.jscc_rdp_prior)(
        x.data_ptr(), nb.data_ptr(), wt.data_ptr(), V, nb.size(0), float(gamma), float(eps), float(beta),
        _lib.ptr(value), _lib.ptr(grad), 1 if (accumulate and grad_out is not None) else 0, _lib.ptr(ws),
        0 if ws is None else ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_rdp_prior")
    return value, grad


def sc_sensitivity(sysmat: torch.Tensor, rotmat_inv: torch.Tensor | None = None, n_rot: int | None = None,
                   out: torch.Tensor | None = None, row_idx: torch.Tensor | None = None) -> torch.Tensor:
    """``out += (sum_r colsum(A)[rotmat_inv[:, r] - 1]) / n_rot`` over the first ``n_rot``
    columns of ``rotmat_inv`` (identity when None): the SC sensitivity of
    main_local_cntstat.py:140-146 / main_plane_sparse.py:440-444, on the device."""
    dev = _lib.require_cuda(sysmat, rotmat_inv, out, row_idx, what="sc_sensitivity")
    if sysmat.dim() != 2:
        raise ValueError("sysmat must be 2-D [bins, voxels]")
    A = _rows_contig(sysmat)
    n_rows, n_vox = A.shape
    if row_idx is not None:
        row_idx = row_idx.to(torch.int64).contiguous()
    n_bins = n_rows if row_idx is None else row_idx.numel()
    ri = _index_table(rotmat_inv, n_vox, "rotmat_inv")
    if ri is None:
        n_rot = 1
    elif n_rot is None:
        n_rot = ri.size(1)
    if n_rot < 1 or (ri is not None and n_rot > ri.size(1)):
        raise ValueError(f"n_rot={n_rot} out of range")
    if out is None:
        out = torch.zeros((n_vox, 1), dtype=torch.float32, device=dev)
    if out.dtype != torch.float32 or not out.is_contiguous() or out.numel() != n_vox:
        raise ValueError("out must be a contiguous float32 tensor with one entry per voxel")
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_sc_weight_workspace_bytes(n_bins, n_vox, 1))
    rc = lib.jscc_sc_sensitivity(A.data_ptr(), _dtype_code(A), A.stride(0), _lib.ptr(row_idx), n_bins, n_vox,
                                 n_rot, _lib.ptr(ri), 0 if ri is None else ri.stride(0), out.data_ptr(),
                                 ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sc_sensitivity")
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


# ============================================================================ Compton cone
def _eff_args(eff: torch.Tensor | None):
    if eff is None:
        return None, _lib.DTYPE_F32, 0
    e = _rows_contig(eff)
    return e, _dtype_code(e), e.stride(0)


def compton_event_prep(list_smeared, detector_pos, sig1_sq, sig2_sq, e0, ene_resolution, thr_max, thr_min, thr_sum,
                       model=_lib.CONE_STRICT, theta_fp64=True, window_sigmas=0.0, delta_r1=0.0, delta_r2=0.0):
    """Event selection + 16-float records (jscc_compton_event_prep). Returns
    ``(keep [E] bool, records [E, 16], row_id [E] int32)`` for all list rows."""
    dev = _lib.require_cuda(list_smeared, detector_pos, sig1_sq, sig2_sq, what="compton_event_prep")
    L = _f32_contig(list_smeared)
    if L.dim() != 2 or L.size(1) < 4:
        raise ValueError("list must be [events, 4] (cp1, e1, cp2, e2)")
    det = _f32_contig(detector_pos)
    s1 = _f32_contig(sig1_sq) if sig1_sq is not None else None
    s2 = _f32_contig(sig2_sq) if sig2_sq is not None else None
    n = L.size(0)
    keep = torch.empty(n, dtype=torch.uint8, device=dev)
    rec = torch.empty((n, _lib.CONE_RECORD_FLOATS), dtype=torch.float32, device=dev)
    rid = torch.empty(n, dtype=torch.int32, device=dev)
    rc = _lib.load().jscc_compton_event_prep(
        L.data_ptr(), L.stride(0), n, det.data_ptr(), _lib.ptr(s1), _lib.ptr(s2), det.size(0), float(e0),
        float(ene_resolution), float(thr_max), float(thr_min), float(thr_sum), int(model), 1 if theta_fp64 else 0,
        float(window_sigmas), float(delta_r1), float(delta_r2), keep.data_ptr(), rec.data_ptr(), rid.data_ptr(),
        _lib.stream_handle(dev))
    _lib.check(rc, "jscc_compton_event_prep")
    return keep.bool(), rec, rid


MAX_ROWS_PER_LAUNCH = 65535


def compton_cone_rows(records, row_id, coor, model=_lib.CONE_STRICT, eff=None, want_tc=True, want_t=True):
    """Materialised cone rows: ``(t_compton, t)`` with ``t = t_compton * eff[row_id]``."""
    dev = _lib.require_cuda(records, row_id, coor, eff, what="compton_cone_rows")
    c = _f32_contig(coor)
    V = c.size(0)
    n = records.size(0)
    tc = torch.empty((n, V), dtype=torch.float32, device=dev) if want_tc else None
    t = torch.empty((n, V), dtype=torch.float32, device=dev) if want_t else None
    e, edt, ld = _eff_args(eff)
    lib = _lib.load()
    for a in range(0, n, MAX_ROWS_PER_LAUNCH):
        b = min(n, a + MAX_ROWS_PER_LAUNCH)
        rc = lib.jscc_compton_cone_rows(
            records[a:b].data_ptr(), row_id[a:b].data_ptr(), b - a, c.data_ptr(), V, int(model), _lib.ptr(e), edt, ld,
            None if tc is None else tc[a:b].data_ptr(), None if t is None else t[a:b].data_ptr(),
            _lib.stream_handle(dev))
        _lib.check(rc, "jscc_compton_cone_rows")
    return tc, t


def compton_row_stats(records, row_id, coor, model=_lib.CONE_STRICT, eff=None, use_window=False):
    """Per-event ``(sum t, sum t^2, any-NaN)`` of ``t = cone * eff`` without storing rows."""
    dev = _lib.require_cuda(records, row_id, coor, eff, what="compton_row_stats")
    c = _f32_contig(coor)
    n = records.size(0)
    s1 = torch.empty(n, dtype=torch.float32, device=dev)
    s2 = torch.empty(n, dtype=torch.float32, device=dev)
    nan = torch.empty(n, dtype=torch.int32, device=dev)
    e, edt, ld = _eff_args(eff)
    rc = _lib.load().jscc_compton_row_stats(
        records.data_ptr(), row_id.data_ptr(), n, c.data_ptr(), c.size(0), int(model), 1 if use_window else 0,
        _lib.ptr(e), edt, ld, s1.data_ptr(), s2.data_ptr(), nan.data_ptr(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_compton_row_stats")
    return s1, s2, nan.bool()


def _row_sorted_events(records, row_id):
    """(records, row_id, perm): the events stably sorted by row id (``records[perm]``),
    cached on the records tensor (rebuilt when either tensor is modified in place)."""
    key = (id(row_id), records._version, row_id._version)
    cache = getattr(records, "_jscc_row_sorted", None)
    if cache is not None and cache[0] == key:
        return cache[1], cache[2], cache[3]
    perm = torch.argsort(row_id.to(torch.int64), stable=True)
    rec_s = records.index_select(0, perm).contiguous()
    rid_s = row_id.index_select(0, perm).contiguous()
    records._jscc_row_sorted = (key, rec_s, rid_s, perm)
    return rec_s, rid_s, perm


def compton_weight(records, row_id, coor, img, model=_lib.CONE_STRICT, eff=None, use_window=False, rotmat=None,
                   rotmat_inv=None, rot_col=0, scale=1.0, out=None):
    """``out += scale * rotinv( T^T (1 / T rot(img)) )`` with T recomputed on the fly."""
    dev = _lib.require_cuda(records, row_id, coor, img, eff, rotmat, rotmat_inv, out, what="compton_weight")
    c = _f32_contig(coor)
    V = c.size(0)
    x = _f32_contig(img.reshape(-1))
    if x.numel() != V:
        raise ValueError(f"img has {x.numel()} voxels, coor has {V}")
    if out is None:
        out = torch.zeros((V, 1), dtype=torch.float32, device=dev)
    rotmat = _index_table(rotmat, V, "rotmat")
    rotmat_inv = _index_table(rotmat_inv, V, "rotmat_inv")
    rm = ri = None
    ld_rot = 0
    if rotmat is not None:
        if not (_is_identity(rotmat, rot_col, 1) and _is_identity(rotmat_inv, rot_col, 1)):
            rm = rotmat.data_ptr() + rot_col * 8
            ri = rotmat_inv.data_ptr() + rot_col * 8
            ld_rot = rotmat.stride(0)
    e, edt, ld = _eff_args(eff)
    n = records.size(0)
    if e is not None and n > 1:
        # the weight is a sum over events: visiting them sorted by efficiency row lets the
        # events a CTA handles share those rows in L1/L2 (only float32 rounding changes)
        records, row_id, _ = _row_sorted_events(records, row_id)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_compton_weight_workspace_bytes(n, V))
    rc = lib.jscc_compton_weight(
        records.data_ptr(), row_id.data_ptr(), n, c.data_ptr(), V, int(model), 1 if use_window else 0, _lib.ptr(e),
        edt, ld, x.data_ptr(), rm, ri, ld_rot, float(scale), out.data_ptr(), ws.data_ptr(), ws.numel(),
        _lib.stream_handle(dev))
    _lib.check(rc, "jscc_compton_weight")
    return out


class ComptonBatch:
    """Several instances' Compton event blocks as one batch for jscc_compton_weight_batched
    (strict model, every pair). ``blocks`` holds one ``(records, row_id)`` pair per instance
    (records [E_b, 16] float32, row_id [E_b] int32 efficiency rows). Each instance's events are
    visited sorted by efficiency row (a stable sort: as compton_weight does, only float32
    rounding changes) and padded to a multiple of 16 with copies of its first event that carry
    no weight; the back projection splits each instance's events into chunks of about
    ``ev_per_chunk`` (default: the batch's events over 256, at least 64). The tables are
    built once; ``weight`` can then be captured in a CUDA graph."""

    def __init__(self, blocks, n_vox, device, ev_per_chunk=None):
        dev = torch.device(device)
        recs, rids, insts, binst, ranges, ichunk = [], [], [], [], [0], [0]
        counts = [int(r.size(0)) for r, _ in blocks]
        total = sum(-(-n // 16) * 16 for n in counts)
        if ev_per_chunk is None:
            ev_per_chunk = max(64, -(-total // 256))
        off = 0
        for b, (rec, rid) in enumerate(blocks):
            n = counts[b]
            if n == 0:
                ichunk.append(ichunk[-1])
                continue
            rec = rec.to(dev, torch.float32).reshape(n, _lib.CONE_RECORD_FLOATS)
            rid = rid.to(dev, torch.int32).reshape(n)
            order = torch.argsort(rid.to(torch.int64), stable=True)
            rec, rid = rec[order], rid[order]
            pad = -(-n // 16) * 16 - n
            if pad:
                rec = torch.cat((rec, rec[:1].expand(pad, -1)))
                rid = torch.cat((rid, rid[:1].expand(pad)))
            npad = n + pad
            recs.append(rec)
            rids.append(rid)
            ev_inst = torch.full((npad,), b, dtype=torch.int32, device=dev)
            ev_inst[n:] = -1
            insts.append(ev_inst)
            binst.append(torch.full((npad // 16,), b, dtype=torch.int32, device=dev))
            k = max(1, -(-npad // ev_per_chunk))
            edges = [off + (npad * i) // k for i in range(1, k + 1)]
            ranges.extend(edges)
            ichunk.append(ichunk[-1] + k)
            off += npad
        self.n_inst = len(blocks)
        self.V = int(n_vox)
        self.dev = dev
        self.n_ev = off
        self.counts = counts
        empty_f = torch.zeros((0, _lib.CONE_RECORD_FLOATS), dtype=torch.float32, device=dev)
        empty_i = torch.zeros(0, dtype=torch.int32, device=dev)
        self.records = torch.cat(recs).contiguous() if recs else empty_f
        self.row_id = torch.cat(rids).contiguous() if rids else empty_i
        self.event_inst = torch.cat(insts).contiguous() if insts else empty_i
        self.block_inst = torch.cat(binst).contiguous() if binst else empty_i
        self.chunk_range = torch.tensor(ranges, dtype=torch.int64, device=dev)
        self.inst_chunk = torch.tensor(ichunk, dtype=torch.int32, device=dev)
        self.n_chunks = len(ranges) - 1

    def weight(self, X, eff, coor, scale=1.0, out=None):
        """``out[b] += scale * T_b^T (1 / T_b X[b])`` for every instance b; X [n_inst, V]."""
        dev = _lib.require_cuda(X, eff, coor, out, what="ComptonBatch.weight")
        c = _f32_contig(coor)
        if c.size(0) != self.V:
            raise ValueError(f"coor has {c.size(0)} voxels, the batch was built for {self.V}")
        if X.dim() != 2 or X.shape != (self.n_inst, self.V) or X.dtype != torch.float32 or X.stride(1) != 1:
            raise ValueError(f"X must be a float32 [{self.n_inst}, {self.V}] tensor with unit column stride")
        if out is None:
            out = torch.zeros((self.n_inst, self.V), dtype=torch.float32, device=dev)
        if out.shape != (self.n_inst, self.V) or out.dtype != torch.float32 or out.stride(1) != 1:
            raise ValueError(f"out must be a float32 [{self.n_inst}, {self.V}] tensor with unit column stride")
        e, edt, ld = _eff_args(eff)
        lib = _lib.load()
        ws = _lib.workspace.get(dev, lib.jscc_compton_batch_workspace_bytes(self.n_ev, self.n_chunks, self.V))
        rc = lib.jscc_compton_weight_batched(
            self.records.data_ptr(), self.row_id.data_ptr(), self.n_ev, self.event_inst.data_ptr(),
            self.block_inst.data_ptr(), self.chunk_range.data_ptr(), self.inst_chunk.data_ptr(), self.n_chunks,
            self.n_inst, c.data_ptr(), self.V, _lib.ptr(e), edt, ld, X.data_ptr(), X.stride(0), float(scale),
            out.data_ptr(), out.stride(0), ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
        _lib.check(rc, "jscc_compton_weight_batched")
        return out


# ============================================================================ sparse rows
def _padded_rows(m):
    """Non-zeros of each row of m as padded [rows, width] (index, weight); padding weight 0."""
    nz = m != 0
    counts = nz.sum(dim=1)
    width = max(int(counts.max()), 1)
    rows, cols = torch.nonzero(nz, as_tuple=True)
    first = torch.zeros(m.size(0), dtype=torch.int64)
    first[1:] = torch.cumsum(counts, 0)[:-1]
    slot = torch.arange(rows.numel()) - first[rows]
    idx = torch.zeros((m.size(0), width), dtype=torch.int64)
    w = torch.zeros((m.size(0), width), dtype=torch.float32)
    idx[rows, slot] = cols
    w[rows, slot] = m[rows, cols]
    return idx, w


def _fixed_width_adjoint(z_expand, layer_expand, device):
    """Adjoint of the upsample as taps of fixed width K per coarse voxel c = zc * n_lc + lc:
    fine index zf * n_lf + lf and weight z_expand[zf, zc] * layer_expand[lf, lc]; returned
    [K, V_c] (tap-major, so a warp reading one tap of consecutive c is coalesced)."""
    ze = z_expand.detach().to("cpu", torch.float32)
    le = layer_expand.detach().to("cpu", torch.float32)
    zi, zw = _padded_rows(ze.t())
    li, lw = _padded_rows(le.t())
    n_lf = le.size(0)
    idx = zi[:, None, :, None] * n_lf + li[None, :, None, :]
    w = zw[:, None, :, None] * lw[None, :, None, :]
    idx = idx.reshape(ze.size(1) * le.size(1), -1)
    w = w.reshape(ze.size(1) * le.size(1), -1)
    return (idx.t().contiguous().to(torch.int32).to(device), w.t().contiguous().to(device), int(idx.size(1)))


def _ring_stencil(z_expand, layer_expand):
    """(ring_len, 4) when the upsample's adjoint is a stride-4 ring stencil: z the identity
    and, within each fine plane, rings of ring_len theta voxels where coarse voxel
    lc = r * (ring_len / 4) + th has exactly the taps r * ring_len + (4 th + d) mod ring_len,
    d = -3..3, with the weights 1 - |d| / 4 (linear theta interpolation with stride 4, as the
    polar projector builds it, compton_sparse_ops.py:132-154); else (0, 0)."""
    ze = z_expand.detach().to("cpu", torch.float32)
    le = layer_expand.detach().to("cpu", torch.float32)
    if ze.size(0) != ze.size(1) or not torch.equal(ze, torch.eye(ze.size(0))):
        return 0, 0
    n_lf, n_lc = le.shape
    if n_lc == 0 or n_lf != 4 * n_lc:
        return 0, 0
    li, lw = _padded_rows(le.t())
    if li.size(1) != 7 or not bool((lw != 0).all()):
        return 0, 0
    ring_len = int(li[0].max()) + 1
    if ring_len < 8 or ring_len % 4 or n_lf % ring_len:
        return 0, 0
    n_thc = ring_len // 4
    lc = torch.arange(n_lc)
    r, th = lc // n_thc, lc % n_thc
    d = torch.arange(-3, 4)
    expect = r[:, None] * ring_len + (4 * th[:, None] + d[None, :]) % ring_len
    if not torch.equal(torch.sort(expect, dim=1).values, torch.sort(li, dim=1).values):
        return 0, 0
    # the polar projector's linear interpolation weights, 1 - |d| / 4 on tap d
    pos = (li - r[:, None] * ring_len - 4 * th[:, None]) % ring_len
    dd = torch.where(pos > ring_len // 2, pos - ring_len, pos)
    if not torch.equal(lw, 1.0 - 0.25 * dd.abs().to(lw.dtype)):
        return 0, 0
    return ring_len, 4


class SparseTables:
    """Device tables of a ComptonSparseProjector: CSR forms of the four separable maps and
    the two-tap upsample arrays of the fused kernels, built from the projector's own
    dense matrices (so the weights are the reference's float32 values)."""

    def __init__(self, layer_reduce, z_reduce, layer_expand, z_expand, device):
        def csr(m):
            m = m.detach().to("cpu", torch.float32)
            nz = m != 0
            counts = nz.sum(dim=1)
            ptr = torch.zeros(m.size(0) + 1, dtype=torch.int32)
            ptr[1:] = torch.cumsum(counts, 0).to(torch.int32)
            rows, cols = torch.nonzero(nz, as_tuple=True)
            return (ptr.to(device), cols.to(torch.int32).to(device), m[rows, cols].contiguous().to(device))

        def two_taps(m):
            # rows of an expand matrix have one or two non-zeros; a single tap is
            # duplicated with weight 0 so the kernels always read two valid indices
            m = m.detach().to("cpu", torch.float32)
            n = m.size(0)
            nz = m != 0
            counts = nz.sum(dim=1)
            if int(counts.max()) > 2 or int(counts.min()) < 1:
                raise ValueError("expand matrix rows must have one or two taps")
            rows, cols = torch.nonzero(nz, as_tuple=True)
            first = torch.zeros(n, dtype=torch.int64)
            first[1:] = torch.cumsum(counts, 0)[:-1]
            idx = torch.empty((n, 2), dtype=torch.int32)
            w = torch.zeros((n, 2), dtype=torch.float32)
            idx[:, 0] = cols[first].to(torch.int32)
            w[:, 0] = m[rows[first], cols[first]]
            two = counts == 2
            sec = first[two] + 1
            idx[:, 1] = idx[:, 0]
            idx[two, 1] = cols[sec].to(torch.int32)
            w[two, 1] = m[rows[sec], cols[sec]]
            return idx.to(device), w.to(device)

        self.n_lf, self.n_lc = layer_expand.shape
        self.n_zf, self.n_zc = z_expand.shape
        self.up = (csr(z_expand), csr(layer_expand))                 # coarse -> fine rows
        self.adj = (csr(z_expand.t()), csr(layer_expand.t()))        # fine -> coarse (adjoint)
        self.red = (csr(z_reduce), csr(layer_reduce))                # fine -> coarse (sample)
        self.red_t = (csr(z_reduce.t()), csr(layer_reduce.t()))      # coarse -> fine (weight image)
        self.z_taps, self.z_tw = two_taps(z_expand)
        self.l_taps, self.l_tw = two_taps(layer_expand)
        self.adj_idx, self.adj_w, self.adj_width = _fixed_width_adjoint(z_expand, layer_expand, device)
        self.ring_len, self.ring_stride = _ring_stencil(z_expand, layer_expand)


def sparse_map(rows_in, maps, n_zo, n_zi, n_lo, n_li, row_idx=None):
    """Apply one separable map (``maps = (Z csr, L csr)``) to every row of ``rows_in``
    (optionally gathered by ``row_idx``). Returns float32 ``[rows, n_zo * n_lo]``."""
    dev = _lib.require_cuda(rows_in, row_idx, what="sparse_map")
    src = rows_in if rows_in.dim() == 2 else rows_in.reshape(1, -1)
    src = _rows_contig(src)
    if src.dtype not in (torch.float32, torch.bfloat16):
        src = src.float()
    n = row_idx.numel() if row_idx is not None else src.size(0)
    if src.size(1) < n_zi * n_li:
        raise ValueError("input rows are shorter than the map's input size")
    rid = row_idx.to(torch.int32).contiguous() if row_idx is not None else None
    out = torch.empty((n, n_zo * n_lo), dtype=torch.float32, device=dev)
    (zp, zi, zw), (lp, li, lw) = maps
    lib = _lib.load()
    for a in range(0, n, MAX_ROWS_PER_LAUNCH):
        b = min(n, a + MAX_ROWS_PER_LAUNCH)
        in_ptr = src.data_ptr() if rid is not None else src[a:b].data_ptr()
        rc = lib.jscc_sparse_map(
            in_ptr, _dtype_code(src), src.stride(0), None if rid is None else rid[a:b].data_ptr(), b - a,
            out[a:b].data_ptr(), out.stride(0), zp.data_ptr(), zi.data_ptr(), zw.data_ptr(), n_zo, n_zi,
            lp.data_ptr(), li.data_ptr(), lw.data_ptr(), n_lo, n_li, _lib.stream_handle(dev))
        _lib.check(rc, "jscc_sparse_map")
    return out


def sparse_pack(cp1, t_compton):
    dev = _lib.require_cuda(cp1, t_compton, what="sparse_pack")
    tc = _f32_contig(t_compton)
    ids = cp1.to(torch.int64).contiguous()
    n, vc = tc.shape
    rows = torch.empty((n, vc + 1), dtype=torch.float32, device=dev)
    lib = _lib.load()
    for a in range(0, n, MAX_ROWS_PER_LAUNCH):
        b = min(n, a + MAX_ROWS_PER_LAUNCH)
        rc = lib.jscc_sparse_pack(ids[a:b].data_ptr(), tc[a:b].data_ptr(), tc.stride(0), b - a, vc,
                                  rows[a:b].data_ptr(), rows.stride(0), _lib.stream_handle(dev))
        _lib.check(rc, "jscc_sparse_pack")
    return rows


def sparse_unpack_ids(rows):
    dev = _lib.require_cuda(rows, what="sparse_unpack_ids")
    r = _rows_contig(rows) if rows.dtype == torch.float32 else _f32_contig(rows)
    out = torch.empty(r.size(0), dtype=torch.int64, device=dev)
    rc = _lib.load().jscc_sparse_unpack_ids(r.data_ptr(), r.stride(0), r.size(0), out.data_ptr(),
                                            _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sparse_unpack_ids")
    return out


def sparse_materialize(rows, sysmat, tables: SparseTables):
    """``(fine [E, V_f], row_sum [E])`` of materialize_sparse_event_rows_to_fine (before the
    validity selection and the division by the row sum)."""
    dev = _lib.require_cuda(rows, sysmat, what="sparse_materialize")
    r = _rows_contig(rows) if rows.dtype == torch.float32 else _f32_contig(rows)
    A = _rows_contig(sysmat)
    n = r.size(0)
    vf = tables.n_zf * tables.n_lf
    fine = torch.empty((n, vf), dtype=torch.float32, device=dev)
    rsum = torch.empty(n, dtype=torch.float32, device=dev)
    rc = _lib.load().jscc_sparse_materialize(
        r.data_ptr(), r.stride(0), n, A.data_ptr(), _dtype_code(A), A.stride(0), A.size(0), tables.z_taps.data_ptr(),
        tables.z_tw.data_ptr(), tables.n_zf, tables.l_taps.data_ptr(), tables.l_tw.data_ptr(), tables.n_lf,
        tables.n_lc, fine.data_ptr(), fine.stride(0), rsum.data_ptr(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sparse_materialize")
    return fine, rsum


def sparse_weight(rows, sysmat, tables: SparseTables, img, grouped=False, rotmat=None, rotmat_inv=None, rot_col=0,
                  scale=1.0, out=None, method="auto"):
    """Fused sparse list-mode weight (MATERIALIZE or GROUPED semantics), accumulated into
    ``out``. method "auto" uses the grouped coarse-space kernel when the grids fit in
    shared memory, "event" the per-event fine-space kernels."""
    if method != "event" and grouped_fits(tables):
        return sparse_weight_grouped(sysmat, tables, img, rows=rows, grouped=grouped, rotmat=rotmat,
                                     rotmat_inv=rotmat_inv, rot_col=rot_col, scale=scale, out=out)
    dev = _lib.require_cuda(rows, sysmat, img, rotmat, rotmat_inv, out, what="sparse_weight")
    r = _rows_contig(rows) if rows.dtype == torch.float32 else _f32_contig(rows)
    A = _rows_contig(sysmat)
    vf = tables.n_zf * tables.n_lf
    x = _f32_contig(img.reshape(-1))
    if x.numel() != vf:
        raise ValueError(f"img has {x.numel()} voxels, the projector has {vf}")
    if out is None:
        out = torch.zeros((vf, 1), dtype=torch.float32, device=dev)
    rotmat = _index_table(rotmat, vf, "rotmat")
    rotmat_inv = _index_table(rotmat_inv, vf, "rotmat_inv")
    rm = ri = None
    ld_rot = 0
    if rotmat is not None:
        if not (_is_identity(rotmat, rot_col, 1) and _is_identity(rotmat_inv, rot_col, 1)):
            rm = rotmat.data_ptr() + rot_col * 8
            ri = rotmat_inv.data_ptr() + rot_col * 8
            ld_rot = rotmat.stride(0)
    n = r.size(0)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_sparse_weight_workspace_bytes(n, vf))
    rc = lib.jscc_sparse_weight(
        r.data_ptr(), r.stride(0), n, A.data_ptr(), _dtype_code(A), A.stride(0), A.size(0), tables.z_taps.data_ptr(),
        tables.z_tw.data_ptr(), tables.n_zf, tables.l_taps.data_ptr(), tables.l_tw.data_ptr(), tables.n_lf,
        tables.n_lc, _lib.SPARSE_GROUPED if grouped else _lib.SPARSE_MATERIALIZE, x.data_ptr(), rm, ri, ld_rot,
        float(scale), out.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sparse_weight")
    return out


def split_sparse_rows(rows, dtype=torch.bfloat16):
    """Packed rows [E, 1 + V_c] -> (row_id int32 0-based, coarse rows [E, V_c] of ``dtype``).
    The coarse rows are a view of a buffer whose leading dimension is a whole number of
    16-byte units (zero padding past V_c), so the bulk-copy kernels move whole rows for any
    coarse grid."""
    ids = (sparse_unpack_ids(rows) - 1).to(torch.int32)
    vc = rows.size(1) - 1
    per16 = 16 // torch.empty((), dtype=dtype).element_size()
    ld = (vc + per16 - 1) // per16 * per16
    if ld == vc:
        return ids, rows[:, 1:].to(dtype).contiguous()
    buf = torch.zeros((rows.size(0), ld), dtype=dtype, device=rows.device)
    buf[:, :vc] = rows[:, 1:]
    return ids, buf[:, :vc]


def sparse_weight_split(row_id, t_coarse, sysmat, tables: SparseTables, img, grouped=False, rotmat=None,
                        rotmat_inv=None, rot_col=0, scale=1.0, out=None, method="auto"):
    """sparse_weight over split storage (int32 row ids + float32/bf16 coarse rows)."""
    if method != "event" and grouped_fits(tables):
        return sparse_weight_grouped(sysmat, tables, img, row_id=row_id, t_coarse=t_coarse, grouped=grouped,
                                     rotmat=rotmat, rotmat_inv=rotmat_inv, rot_col=rot_col, scale=scale, out=out)
    dev = _lib.require_cuda(row_id, t_coarse, sysmat, img, rotmat, rotmat_inv, out, what="sparse_weight_split")
    tc = _rows_contig(t_coarse)
    A = _rows_contig(sysmat)
    vf = tables.n_zf * tables.n_lf
    x = _f32_contig(img.reshape(-1))
    if x.numel() != vf:
        raise ValueError(f"img has {x.numel()} voxels, the projector has {vf}")
    if tc.size(1) < tables.n_lc * tables.n_zc:
        raise ValueError("coarse rows are shorter than the projector's coarse grid")
    if out is None:
        out = torch.zeros((vf, 1), dtype=torch.float32, device=dev)
    rotmat = _index_table(rotmat, vf, "rotmat")
    rotmat_inv = _index_table(rotmat_inv, vf, "rotmat_inv")
    rm = ri = None
    ld_rot = 0
    if rotmat is not None and not (_is_identity(rotmat, rot_col, 1) and _is_identity(rotmat_inv, rot_col, 1)):
        rm = rotmat.data_ptr() + rot_col * 8
        ri = rotmat_inv.data_ptr() + rot_col * 8
        ld_rot = rotmat.stride(0)
    ids = row_id.to(torch.int32).contiguous()
    n = ids.numel()
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_sparse_weight_workspace_bytes(n, vf))
    rc = lib.jscc_sparse_weight_split(
        ids.data_ptr(), tc.data_ptr(), _dtype_code(tc), tc.stride(0), n, A.data_ptr(), _dtype_code(A), A.stride(0),
        A.size(0), tables.z_taps.data_ptr(), tables.z_tw.data_ptr(), tables.n_zf, tables.l_taps.data_ptr(),
        tables.l_tw.data_ptr(), tables.n_lf, tables.n_lc, _lib.SPARSE_GROUPED if grouped else _lib.SPARSE_MATERIALIZE,
        x.data_ptr(), rm, ri, ld_rot, float(scale), out.data_ptr(), ws.data_ptr(), ws.numel(),
        _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sparse_weight_split")
    return out


# ============================================================================ grouped sparse weight
class GroupPlan:
    """Grouping of a block of sparse events by first-hit row for jscc_sparse_weight_grouped:
    event order sorted (stably) by row, group offsets into that order and group rows."""

    def __init__(self, row_ids: torch.Tensor):
        ids = row_ids.to(torch.int64)
        order = torch.argsort(ids, stable=True)
        rows, counts = torch.unique_consecutive(ids[order], return_counts=True)
        offsets = torch.zeros(rows.numel() + 1, dtype=torch.int64, device=ids.device)
        offsets[1:] = torch.cumsum(counts, 0)
        self.order = order.to(torch.int32).contiguous()
        self.offsets = offsets.to(torch.int32).contiguous()
        self.rows = rows.to(torch.int32).contiguous()
        self.n_groups = int(rows.numel())
        self.sums = {}  # per sysmat key: S of the materialise form, by position in `order`


def _group_plan(key_tensor, row_ids_fn):
    """GroupPlan cached on ``key_tensor`` (rebuilt when the tensor is modified in place)."""
    cache = getattr(key_tensor, "_jscc_group_plan", None)
    if cache is not None and cache[0] == key_tensor._version:
        return cache[1]
    plan = GroupPlan(row_ids_fn())
    key_tensor._jscc_group_plan = (key_tensor._version, plan)
    return plan


def sparse_sensitivity(sysmat, tables: SparseTables, rows=None, row_id=None, t_coarse=None, out=None):
    """``out += sum_i t_norm,i``: the sum over events of the normalised fine rows of
    materialize_sparse_event_rows_to_fine (compton_sparse_ops.py:380-400), i.e. the Compton
    sensitivity of main_local_sparse_jsccsd_only.py:95-108. It is the materialise-form
    weight at x = 1: there f_i = S_i, so every valid event gets c_i = 1 / S_i."""
    vf = tables.n_zf * tables.n_lf
    ones = torch.ones((vf, 1), dtype=torch.float32, device=sysmat.device)
    if rows is not None:
        return sparse_weight(rows, sysmat, tables, ones, grouped=False, out=out)
    return sparse_weight_split(row_id, t_coarse, sysmat, tables, ones, grouped=False, out=out)


def plan_groups(row_id: torch.Tensor, n_det: int) -> GroupPlan:
    """Build (and cache on ``row_id``) the first-hit-row grouping that the grouped sparse
    weight uses for split storage, so that a caller staging data can do it ahead of the first
    weight call. ``n_det`` is the sysmat's row count (ids are clamped to it, as the weight
    call does). ``row_id`` must already be a contiguous int32 tensor for the cache to be
    found again by the weight call."""
    _lib.require_cuda(row_id, what="plan_groups")
    if row_id.dtype != torch.int32 or not row_id.is_contiguous():
        raise ValueError("plan_groups: row_id must be a contiguous int32 tensor")
    return _group_plan(row_id, lambda: torch.clamp(row_id.long(), 0, n_det - 1))


def grouped_fits(tables: SparseTables) -> bool:
    """The grouped kernels keep one coarse row per CTA in shared memory."""
    return ((tables.n_zc * tables.n_lc + 3) // 4 * 4) * 4 <= 227 * 1024


def _sms(dev):
    return torch.cuda.get_device_properties(dev).multi_processor_count


def sparse_weight_grouped(sysmat, tables: SparseTables, img, rows=None, row_id=None, t_coarse=None, grouped=False,
                          rotmat=None, rotmat_inv=None, rot_col=0, scale=1.0, out=None):
    """Grouped coarse-space sparse weight over packed ``rows`` or split (``row_id``,
    ``t_coarse``) storage; accumulated into ``out``. Same result as sparse_weight."""
    dev = _lib.require_cuda(sysmat, img, rows, row_id, t_coarse, rotmat, rotmat_inv, out,
                            what="sparse_weight_grouped")
    A = _rows_contig(sysmat)
    vf = tables.n_zf * tables.n_lf
    vc = tables.n_zc * tables.n_lc
    x = _f32_contig(img.reshape(-1))
    if x.numel() != vf:
        raise ValueError(f"img has {x.numel()} voxels, the projector has {vf}")
    if out is None:
        out = torch.zeros((vf, 1), dtype=torch.float32, device=dev)
    if rows is not None:
        r = _rows_contig(rows) if rows.dtype == torch.float32 else _f32_contig(rows)
        n = r.size(0)
        if r.size(1) != vc + 1:
            raise ValueError(f"packed rows must have 1 + {vc} columns (got {r.size(1)})")
        if n == 0:
            return out
        plan = _group_plan(r, lambda: torch.clamp(sparse_unpack_ids(r) - 1, 0, A.size(0) - 1))
        packed, ids_p, tc_p, tc_dt, ld = r.data_ptr(), None, None, _lib.DTYPE_F32, r.stride(0)
    else:
        tc = _rows_contig(t_coarse)
        ids = row_id.to(torch.int32).contiguous()
        n = ids.numel()
        if tc.size(1) < vc or tc.size(0) != n:
            raise ValueError(f"coarse rows must be [{n}, >= {vc}] (got {tuple(tc.shape)})")
        if n == 0:
            return out
        plan = _group_plan(ids, lambda: torch.clamp(ids.long(), 0, A.size(0) - 1))
        packed, ids_p, tc_p, tc_dt, ld = None, ids.data_ptr(), tc.data_ptr(), _dtype_code(tc), tc.stride(0)
    rotmat = _index_table(rotmat, vf, "rotmat")
    rotmat_inv = _index_table(rotmat_inv, vf, "rotmat_inv")
    rm = ri = None
    ld_rot = 0
    if rotmat is not None and not (_is_identity(rotmat, rot_col, 1) and _is_identity(rotmat_inv, rot_col, 1)):
        rm = rotmat.data_ptr() + rot_col * 8
        ri = rotmat_inv.data_ptr() + rot_col * 8
        ld_rot = rotmat.stride(0)
    lib = _lib.load()
    ws = _lib.workspace.get(dev, lib.jscc_sparse_grouped_workspace_bytes(n, vf, vc, plan.n_groups,
                                                                         tables.adj_width))
    # S_i = t_i . adj(A_g) depends on the rows and the sysmat only: kept on the plan per sysmat
    skey = (A.data_ptr(), A._version, A.dtype, tuple(A.shape), _lib.timeout_epoch)
    sums = plan.sums.get(skey)
    have = sums is not None
    if not have:
        sums = torch.empty(n, dtype=torch.float32, device=dev)
    rc = lib.jscc_sparse_weight_grouped(
        ids_p, tc_p, tc_dt, ld, packed, n, plan.order.data_ptr(), plan.offsets.data_ptr(), plan.rows.data_ptr(),
        plan.n_groups, sums.data_ptr(), 1 if have else 0, A.data_ptr(), _dtype_code(A), A.stride(0), A.size(0),
        tables.z_taps.data_ptr(), tables.z_tw.data_ptr(), tables.n_zf, tables.l_taps.data_ptr(),
        tables.l_tw.data_ptr(), tables.n_lf, tables.n_lc, tables.n_zc, tables.adj_idx.data_ptr(),
        tables.adj_w.data_ptr(), tables.adj_width, tables.ring_len, tables.ring_stride,
        _lib.SPARSE_GROUPED if grouped else _lib.SPARSE_MATERIALIZE,
        x.data_ptr(), rm, ri, ld_rot, float(scale), out.data_ptr(), ws.data_ptr(), ws.numel(),
        _lib.stream_handle(dev))
    _lib.check(rc, "jscc_sparse_weight_grouped")
    if not have and not grouped:
        if len(plan.sums) > 4:
            plan.sums.clear()
        plan.sums[skey] = sums
    return out
