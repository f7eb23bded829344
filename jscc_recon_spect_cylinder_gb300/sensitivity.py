"""Sensitivity builders of the reference's entry scripts, on the GPU path.

The reference keeps these in its main scripts: build_sparse_sensi_d
(main_plane_sparse.py:214-231), build_sparse_sensi_d_local
(main_local_sparse_jsccsd_only.py:95-108) and compute_sensitivity_local
(main_local_cntstat.py:140-146, the same formula as the s_map_s loop of
main_plane_sparse.py:440-444). Same names, arguments and returned CPU tensors; the sums run
in the library's kernels (jscc_sparse_weight_grouped at x = 1 for d, jscc_sc_sensitivity for s)
instead of materialising [block, V] fine rows.
"""
from __future__ import annotations

import torch

from . import compton_sparse_ops as cso
from . import ops


def _device(device):
    device = torch.device(device)
    if device.type != "cuda":
        raise RuntimeError(f"the GB300 path runs on CUDA devices only (got {device})")
    return torch.device("cuda", 0) if device.index is None else device


def _sum_d(t_all_energy, sysmat, sparse_projector, device, out):
    tables = cso.tables(sparse_projector, device)
    sysmat_device = sysmat.to(device, non_blocking=True)
    for t_rotate in t_all_energy:
        if t_rotate.numel() == 0:
            continue
        ops.sparse_sensitivity(sysmat_device, tables, rows=t_rotate.to(device, non_blocking=True), out=out)


def build_sparse_sensi_d_local(t_local_all, sysmat_full_all, sparse_projector_all, pixel_num, device, block_size=1024):
    """main_local_sparse_jsccsd_only.py:95-108: d = sum over every event block of the
    normalised fine rows (block_size only bounded the reference's temporaries)."""
    device = _device(device)
    d = torch.zeros((pixel_num, 1), dtype=torch.float32, device=device)
    for t_energy, sysmat_full, sparse_projector in zip(t_local_all, sysmat_full_all, sparse_projector_all):
        _sum_d(t_energy, sysmat_full, sparse_projector, device, d)
    return d.cpu()


def build_sparse_sensi_d(t_all, sysmat_all, sparse_projector_all, s_map_s, single_event_count_total,
                         compton_event_count_total, block_size=1024):
    """main_plane_sparse.py:214-231: d as above on cuda:0, then scaled to
    sum(s_map_s) * E_C / max(E_S, 1) when sum(d) > 0."""
    device = torch.device("cuda", 0)
    d = torch.zeros((s_map_s.numel(), 1), dtype=torch.float32, device=device)
    for t_energy, sysmat, sparse_projector in zip(t_all, sysmat_all, sparse_projector_all):
        _sum_d(t_energy, sysmat, sparse_projector, device, d)
    sensi_d = d.cpu().reshape(s_map_s.shape)
    if torch.sum(sensi_d) > 0:
        sensi_d = sensi_d * torch.sum(s_map_s) / torch.sum(sensi_d)
        sensi_d = sensi_d * compton_event_count_total / max(single_event_count_total, 1)
    return sensi_d


def compute_sensitivity_local(sysmat, rotmat_inv, rotate_num):
    """main_local_cntstat.py:140-146: s = (1/R) sum_r colsum(sysmat)[rotmat_inv[:, r] - 1],
    [V, 1] on the CPU. A CPU sysmat is copied to cuda:0 for the sum."""
    device = sysmat.device if sysmat.is_cuda else torch.device("cuda", 0)
    A = sysmat.to(device)
    ri = rotmat_inv.to(device)
    return ops.sc_sensitivity(A, ri, rotate_num).cpu()
