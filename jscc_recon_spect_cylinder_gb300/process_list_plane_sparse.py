"""Drop-in for the reference module ``process_list_plane_sparse`` (coarse sparse T builder).

get_compton_backproj_list_single_sparse (process_list_plane_sparse.py:25-123): energies are
smeared (not in place) with torch.randn drawn on ``device``, events are selected as in the
strict builder, the strict cone is evaluated on the projector's COARSE coordinates, the
efficiency row is the fine sysmat row reduced to the coarse grid, rows with NaN or a zero
sum are dropped, the effective-support filter (>= 50) is applied to the normalised product,
and the surviving (cp1, normalised t_compton) rows are packed and returned on the CPU.
Selection, cone rows, the reduction of the sysmat rows and the packing run in kernels.
"""
from __future__ import annotations

import torch

from . import _compton, _lib, ops
from .compton_sparse_ops import pack_sparse_event_rows, reduce_fine_rows_to_coarse
from .process_list_plane_strict import ROW_BATCH


def _filter_unstable_event_kernels_sparse(t, t_compton, t_single):
    """Normalise the three row sets and keep effective support >= 50 (:15-22)."""
    t_norm = t / t.sum(dim=1, keepdim=True)
    tc_norm = t_compton / t_compton.sum(dim=1, keepdim=True)
    ts_norm = t_single / t_single.sum(dim=1, keepdim=True)
    stable = _compton.stable_rows(t_norm)
    return t_norm[stable], tc_norm[stable], ts_norm[stable], stable


def build_sparse_rows_from_smeared(sysmat, detector, sparse_projector, list_smeared, delta_r1, delta_r2, e0,
                                   ene_resolution, ene_threshold_max, ene_threshold_min, ene_threshold_sum):
    """Device event rows [E', 1 + V_c] from an already-smeared device list."""
    dev = list_smeared.device
    vc = sparse_projector.coarse_pixel_num
    idx, rec, rid = _compton.select_events(list_smeared, detector, delta_r1, delta_r2, e0, ene_resolution,
                                           ene_threshold_max, ene_threshold_min, ene_threshold_sum,
                                           model=_lib.CONE_STRICT, theta_fp64=False)
    empty = torch.empty((0, vc + 1), dtype=torch.float32, device=dev)
    if idx.numel() == 0:
        return empty
    sys_d = sysmat.to(dev)
    coor_c = sparse_projector.coor_coarse.to(dev, torch.float32)
    out = []
    for a in range(0, idx.numel(), ROW_BATCH):
        b = min(idx.numel(), a + ROW_BATCH)
        tc, _ = ops.compton_cone_rows(rec[a:b], rid[a:b], coor_c, model=_lib.CONE_STRICT, want_t=False)
        ts = reduce_fine_rows_to_coarse(sys_d, sparse_projector, row_idx=rid[a:b])
        t = tc * ts
        ok = _compton.finite_rows(t)
        cp1 = (rid[a:b].long() + 1)[ok]
        t, tc, ts = t[ok], tc[ok], ts[ok]
        if t.size(0) == 0:
            continue
        _, tc_n, _, stable = _filter_unstable_event_kernels_sparse(t, tc, ts)
        out.append(pack_sparse_event_rows(cp1[stable], tc_n))
    return torch.cat(out, dim=0) if out else empty


def get_compton_backproj_list_single_sparse(sysmat, detector, sparse_projector, list_origin, delta_r1, delta_r2, e0,
                                            ene_resolution, ene_threshold_max, ene_threshold_min, ene_threshold_sum,
                                            device, model_compton_generator=None):
    """Sparse builder -> (event_rows on the CPU, None, None) (process_list_plane_sparse.py:25-123)."""
    if model_compton_generator is not None:
        raise NotImplementedError("model_compton_generator is not supported in sparse Compton mode.")
    dev = _compton.require_cuda_device(device)
    L = list_origin.to(dev)
    e1 = L[:, 1]
    e2 = L[:, 3]
    sigma_1 = _compton.smear_sigma(e1, e0, ene_resolution)
    sigma_2 = _compton.smear_sigma(e2, e0, ene_resolution)
    e1 = e1 + sigma_1 * torch.randn(e1.shape[0], device=dev)
    e2 = e2 + sigma_2 * torch.randn(e2.shape[0], device=dev)
    smeared = torch.stack((L[:, 0], e1, L[:, 2], e2), dim=1)
    rows = build_sparse_rows_from_smeared(sysmat, detector, sparse_projector, smeared, delta_r1, delta_r2, e0,
                                          ene_resolution, ene_threshold_max, ene_threshold_min, ene_threshold_sum)
    return rows.cpu(), None, None


def get_compton_backproj_list_mp_sparse(rank, world_size, sysmat, detector, sparse_projector, list_origin_chunk,
                                        delta_r1, delta_r2, e0, ene_resolution, ene_threshold_max, ene_threshold_min,
                                        ene_threshold_sum, result_dict, num_workers, start_time, flag_save_t,
                                        model_compton_generator=None):
    """Per-GPU worker (process_list_plane_sparse.py:126-181)."""
    del world_size, start_time, flag_save_t
    with torch.no_grad():
        torch.cuda.set_device(rank)
        dev = torch.device(f"cuda:{rank}")
        sysmat, detector = sysmat.to(dev), detector.to(dev)
        proj = sparse_projector.to(dev)
        parts = []
        for sub in torch.chunk(list_origin_chunk, num_workers, dim=0):
            if sub.numel() == 0:
                continue
            rows, _, _ = get_compton_backproj_list_single_sparse(
                sysmat, detector, proj, sub.to(dev), delta_r1, delta_r2, e0, ene_resolution, ene_threshold_max,
                ene_threshold_min, ene_threshold_sum, dev, model_compton_generator=model_compton_generator)
            if rows.numel() > 0:
                parts.append(rows)
        result_dict[rank] = torch.cat(parts, dim=0) if parts else torch.empty(
            (0, sparse_projector.coarse_pixel_num + 1), dtype=torch.float32)
