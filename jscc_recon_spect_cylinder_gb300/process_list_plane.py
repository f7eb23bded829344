"""Drop-in for the reference module ``process_list_plane`` (legacy dense T builder).

process_list_plane.py:17-107: in-place energy smearing with the reference's torch.randn
draws, thresholds without the kinematic filter, the different-layer filter, the legacy
cone (first/second-derivative sigma_E, atan sigma_pos, unclamped angles), NaN/zero-row
filter and row normalisation, no effective-support filter. Selection and cone rows run in
the jscc_compton_* kernels (model JSCC_CONE_LEGACY).
"""
from __future__ import annotations

import time

import torch

from . import _compton, _lib
from .process_list_plane_strict import build_rows_from_smeared, get_coor_plane  # noqa: F401  (same helper)


def get_compton_backproj_list_single(sysmat, detector, coor, list_origin, delta_r1, delta_r2, e0, ene_resolution,
                                     ene_threshold_max, ene_threshold_min, ene_threshold_sum, device,
                                     model_compton_generator=None):
    """Legacy T builder -> CPU (t, t_compton, t_single) (process_list_plane.py:17-107)."""
    dev = _compton.require_cuda_device(device)
    if list_origin.device != dev:
        raise RuntimeError(f"list_origin must be on {dev} (the reference moves chunks there before calling)")
    e1 = list_origin[:, 1]
    e2 = list_origin[:, 3]
    sigma_1 = _compton.smear_sigma(e1, e0, ene_resolution)
    sigma_2 = _compton.smear_sigma(e2, e0, ene_resolution)
    e1 += sigma_1 * torch.randn(e1.shape[0]).to(dev)
    e2 += sigma_2 * torch.randn(e2.shape[0]).to(dev)
    t, tc, ts, _ = build_rows_from_smeared(sysmat, detector, coor, list_origin, delta_r1, delta_r2, e0,
                                           ene_resolution, ene_threshold_max, ene_threshold_min, ene_threshold_sum,
                                           model=_lib.CONE_LEGACY, model_compton_generator=model_compton_generator,
                                           stability=False)
    return t.cpu(), tc.cpu(), ts.cpu()


def get_compton_backproj_list_mp(rank, world_size, sysmat, detector, coor_plane, list_origin_chunk, delta_r1,
                                 delta_r2, e0, ene_resolution, ene_threshold_max, ene_threshold_min,
                                 ene_threshold_sum, result_dict, num_workers, start_time, flag_save_t,
                                 model_compton_generator=None):
    """Per-GPU worker (process_list_plane.py:110-174)."""
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
