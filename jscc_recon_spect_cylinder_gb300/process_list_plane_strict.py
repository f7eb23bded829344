"""Drop-in for the reference module ``process_list_plane_strict`` (strict dense T builder).

get_compton_backproj_list_single keeps the reference's contract (process_list_plane_strict.py
:151-253): the list is energy-smeared IN PLACE with the same torch.randn draws (the reference
draws them on the CPU and moves them to ``device``), events are selected, the T row of every
surviving event is evaluated, rows with NaN or a zero sum are dropped, rows are normalised,
rows with effective support < 50 are dropped, and (t, t_compton, t_single) come back as CPU
tensors. Event selection and the cone rows run in the jscc_compton_* kernels; the FP32
Compton angle is used here so the rows follow the reference's float32 evaluation.

get_compton_event_params is the fused-path entry (no counterpart in this module of the
reference; its precedent is the lazy recompute of
distributed/python/recon_osem_dist_sparse_jsccsd_only_lazy.py:46-87): it returns compact
per-event records instead of T, for recon_osem_plane.get_weight_compton_fused.
"""
from __future__ import annotations

import time

import torch

from . import _compton, _lib, ops
from ._compton import ELECTRON_REST_MEV, FRONT_LAYER_CRYSTAL_MM, MIN_EVENT_EFFECTIVE_SUPPORT, REAR_LAYER_CRYSTAL_MM

__all__ = [
    "ELECTRON_REST_MEV", "FRONT_LAYER_CRYSTAL_MM", "REAR_LAYER_CRYSTAL_MM", "MIN_EVENT_EFFECTIVE_SUPPORT",
    "get_coor_plane", "get_compton_backproj_list_single", "get_compton_backproj_list_mp",
    "get_compton_backproj_list_dist", "get_compton_event_params", "ComptonEvents",
]

# rows per cone-row launch batch (keeps the [E, V] temporaries bounded)
ROW_BATCH = 32768


def get_coor_plane(pixel_num_x, pixel_num_y, pixel_l_x, pixel_l_y, fov_z):
    """Cartesian pixel centres of a plane (process_list_plane_strict.py:11-21)."""
    hx = (pixel_num_x / 2 - 0.5) * pixel_l_x
    hy = (pixel_num_y / 2 - 0.5) * pixel_l_y
    xs = torch.linspace(-hx, hx, pixel_num_x)
    ys = torch.linspace(-hy, hy, pixel_num_y)
    out = torch.empty((pixel_num_x, pixel_num_y, 3))
    out[:, :, 0] = xs.reshape(1, -1)
    out[:, :, 1] = ys.reshape(-1, 1)
    out[:, :, 2] = fov_z
    return out.reshape(-1, 3)


def _compton_theta_from_e1(e1, e0, ee):
    """Compton angle with the reference's clamp (process_list_plane_strict.py:24-27)."""
    cos_theta = 1 - ((ee * e1) / ((e0 - e1) * e0))
    return torch.acos(torch.clamp(cos_theta, -1.0 + 1e-7, 1.0 - 1e-7))


def _filter_kinematically_valid_events(cpnum1, cpnum2, e1, e2, e0, ee):
    """Events whose Compton cosine is inside (-1 + 1e-6, 1 - 1e-6) (:30-36)."""
    c = 1 - ((ee * e1) / ((e0 - e1) * e0))
    valid = (c > -1.0 + 1e-6) & (c < 1.0 - 1e-6)
    return cpnum1[valid], cpnum2[valid], e1[valid], e2[valid]


def _build_detector_pos_sigma_sq(detector, extra_sigma):
    """Per-detector position variance (:59-96)."""
    return _compton.detector_pos_sigma_sq(detector, extra_sigma)


def _smear_in_place(list_origin, e0, ene_resolution, device):
    e1 = list_origin[:, 1]
    e2 = list_origin[:, 3]
    sigma_1 = _compton.smear_sigma(e1, e0, ene_resolution)
    sigma_2 = _compton.smear_sigma(e2, e0, ene_resolution)
    e1 += sigma_1 * torch.randn(e1.shape[0]).to(device)
    e2 += sigma_2 * torch.randn(e2.shape[0]).to(device)


def build_rows_from_smeared(sysmat, detector, coor, list_smeared, delta_r1, delta_r2, e0, ene_resolution,
                            ene_threshold_max, ene_threshold_min, ene_threshold_sum, model=_lib.CONE_STRICT,
                            model_compton_generator=None, stability=True):
    """Selection + cone rows + row filters on an already-smeared device list.
    Returns device tensors (t_norm, t_compton_norm, t_single_norm, kept list indices)."""
    idx, rec, rid = _compton.select_events(list_smeared, detector, delta_r1, delta_r2, e0, ene_resolution,
                                           ene_threshold_max, ene_threshold_min, ene_threshold_sum, model=model,
                                           theta_fp64=False)
    V = coor.size(0)
    dev = list_smeared.device
    if idx.numel() == 0:
        z = torch.empty((0, V), dtype=torch.float32, device=dev)
        return z, z.clone(), z.clone(), idx
    sys_c = sysmat.to(dev)
    coor_c = coor.to(dev, torch.float32)
    t_parts, tc_parts, ts_parts, id_parts = [], [], [], []
    for a in range(0, idx.numel(), ROW_BATCH):
        b = min(idx.numel(), a + ROW_BATCH)
        if model_compton_generator is None:
            tc, t = ops.compton_cone_rows(rec[a:b], rid[a:b], coor_c, model=model, eff=sys_c)
        else:
            tc, _ = ops.compton_cone_rows(rec[a:b], rid[a:b], coor_c, model=model, want_t=False)
            n = int(tc.shape[1] ** 0.5)
            tc = model_compton_generator((tc / tc.max(dim=1, keepdim=True)[0]).view(-1, 1, n, n)).view(-1, n * n)
            t = tc * sys_c.index_select(0, rid[a:b].long())
        ts = sys_c.index_select(0, rid[a:b].long())
        ok = _compton.finite_rows(t)
        t, tc, ts, ids = t[ok], tc[ok], ts[ok], idx[a:b][ok]
        t = t / t.sum(dim=1, keepdim=True)
        tc = tc / tc.sum(dim=1, keepdim=True)
        ts = ts / ts.sum(dim=1, keepdim=True)
        if stability:
            st = _compton.stable_rows(t)
            t, tc, ts, ids = t[st], tc[st], ts[st], ids[st]
        t_parts.append(t)
        tc_parts.append(tc)
        ts_parts.append(ts)
        id_parts.append(ids)
    return torch.cat(t_parts), torch.cat(tc_parts), torch.cat(ts_parts), torch.cat(id_parts)


def get_compton_backproj_list_single(sysmat, detector, coor, list_origin, delta_r1, delta_r2, e0, ene_resolution,
                                     ene_threshold_max, ene_threshold_min, ene_threshold_sum, device,
                                     model_compton_generator=None):
    """Strict T builder (process_list_plane_strict.py:151-253) -> CPU (t, t_compton, t_single)."""
    dev = _compton.require_cuda_device(device)
    if list_origin.device != dev:
        raise RuntimeError(f"list_origin must be on {dev} (the reference moves chunks there before calling)")
    _smear_in_place(list_origin, e0, ene_resolution, dev)
    t, tc, ts, _ = build_rows_from_smeared(sysmat, detector, coor, list_origin, delta_r1, delta_r2, e0,
                                           ene_resolution, ene_threshold_max, ene_threshold_min, ene_threshold_sum,
                                           model=_lib.CONE_STRICT, model_compton_generator=model_compton_generator)
    return t.cpu(), tc.cpu(), ts.cpu()


def get_compton_backproj_list_mp(rank, world_size, sysmat, detector, coor_plane, list_origin_chunk, delta_r1,
                                 delta_r2, e0, ene_resolution, ene_threshold_max, ene_threshold_min,
                                 ene_threshold_sum, result_dict, num_workers, start_time, flag_save_t,
                                 model_compton_generator=None):
    """Per-GPU worker (process_list_plane_strict.py:256-320): builds T for its chunk in
    ``num_workers`` sub-chunks on cuda:rank and stores it in ``result_dict``."""
    with torch.no_grad():
        torch.cuda.set_device(rank)
        dev = torch.device(f"cuda:{rank}")
        sysmat, detector, coor_plane = sysmat.to(dev), detector.to(dev), coor_plane.to(dev)
        if model_compton_generator is not None:
            model_compton_generator = model_compton_generator.to(dev)
        parts = ([], [], [])
        for sub in torch.chunk(list_origin_chunk, num_workers, dim=0):
            out = get_compton_backproj_list_single(sysmat, detector, coor_plane, sub.to(dev), delta_r1, delta_r2, e0,
                                                   ene_resolution, ene_threshold_max, ene_threshold_min,
                                                   ene_threshold_sum, dev,
                                                   model_compton_generator if flag_save_t == 0 else None)
            for p, o in zip(parts, out):
                p.append(o)
            print(f"Rank {rank}: processed sub-chunk, time used: {time.time() - start_time:.2f}s")
        result_dict[rank] = torch.cat(parts[0], dim=0)
        if flag_save_t != 0:
            result_dict[world_size + rank] = torch.cat(parts[1], dim=0)
            result_dict[2 * world_size + rank] = torch.cat(parts[2], dim=0)
        print(f"Rank {rank} completed processing and stored result")


def get_compton_backproj_list_dist(local_rank, world_size, sysmat, detector, coor_plane, list_origin_chunk, delta_r1,
                                   delta_r2, e0, ene_resolution, ene_threshold_max, ene_threshold_min,
                                   ene_threshold_sum, result_dict, num_workers, start_time, flag_save_t):
    """torchrun variant (process_list_plane_strict.py:323-383): returns the CPU rows."""
    del world_size, result_dict
    torch.cuda.set_device(local_rank)
    dev = torch.device(f"cuda:{local_rank}")
    sysmat, detector, coor_plane = sysmat.to(dev), detector.to(dev), coor_plane.to(dev)
    parts = ([], [], [])
    for sub in torch.chunk(list_origin_chunk, num_workers, dim=0):
        out = get_compton_backproj_list_single(sysmat, detector, coor_plane, sub.to(dev), delta_r1, delta_r2, e0,
                                               ene_resolution, ene_threshold_max, ene_threshold_min,
                                               ene_threshold_sum, dev)
        for p, o in zip(parts, out):
            p.append(o)
        print(f"Rank {local_rank}: processed sub-chunk, time used: {time.time() - start_time:.2f}s")
    if flag_save_t == 0:
        return torch.cat(parts[0], dim=0)
    return tuple(torch.cat(p, dim=0) for p in parts)


class ComptonEvents:
    """Compact per-event state of the fused path (64-byte records + efficiency row ids),
    plus the FP32 list indices of the kept events. ``model`` is the cone model."""

    def __init__(self, records, row_id, list_index, model):
        self.records = records
        self.row_id = row_id
        self.list_index = list_index
        self.model = model

    def __len__(self):
        return int(self.records.size(0))

    def split(self, parts):
        """Floor-balanced contiguous split (the reference's split_tensor_even over T rows)."""
        n = len(self)
        b = [n * k // parts for k in range(parts + 1)]
        return [ComptonEvents(self.records[b[k]:b[k + 1]], self.row_id[b[k]:b[k + 1]],
                              self.list_index[b[k]:b[k + 1]], self.model) for k in range(parts)]

    def to(self, device):
        return ComptonEvents(self.records.to(device), self.row_id.to(device), self.list_index.to(device), self.model)


def get_compton_event_params(sysmat, detector, coor, list_smeared, delta_r1, delta_r2, e0, ene_resolution,
                             ene_threshold_max, ene_threshold_min, ene_threshold_sum, model=_lib.CONE_STRICT,
                             theta_fp64=True, window_sigmas=9.0, stability=True):
    """Fused-path builder: the same event selection and row filters as the strict (or
    legacy) builder, but returning compact records (ComptonEvents) instead of T. Row
    statistics come from one on-the-fly pass (jscc_compton_row_stats); the list must
    already be smeared (see _smear_in_place for the reference's draws)."""
    dev = list_smeared.device
    idx, rec, rid = _compton.select_events(list_smeared, detector, delta_r1, delta_r2, e0, ene_resolution,
                                           ene_threshold_max, ene_threshold_min, ene_threshold_sum, model=model,
                                           theta_fp64=theta_fp64, window_sigmas=window_sigmas)
    if idx.numel() == 0:
        return ComptonEvents(rec, rid, idx, model)
    s1, s2, nan = ops.compton_row_stats(rec, rid, coor.to(dev, torch.float32), model=model, eff=sysmat.to(dev),
                                        use_window=window_sigmas > 0)
    ok = (~nan) & (s1 != 0)
    if stability and model != _lib.CONE_LEGACY:
        ok &= (s1 * s1 / s2) >= MIN_EVENT_EFFECTIVE_SUPPORT
    keep = torch.nonzero(ok).flatten()
    return ComptonEvents(rec.index_select(0, keep).contiguous(), rid.index_select(0, keep).contiguous(),
                         idx.index_select(0, keep), model)
