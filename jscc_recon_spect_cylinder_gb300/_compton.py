"""Shared host logic of the Compton T builders: energy smearing with the reference's
random draws, detector position variances, and event selection through the
jscc_compton_event_prep kernel."""
from __future__ import annotations

import torch

from . import _lib, ops

ELECTRON_REST_MEV = 0.511
FRONT_LAYER_CRYSTAL_MM = (3.0, 3.0, 3.0)
REAR_LAYER_CRYSTAL_MM = (2.0, 6.0, 2.0)
MIN_EVENT_EFFECTIVE_SUPPORT = 50.0


def require_cuda_device(device):
    dev = torch.device(device)
    if dev.type != "cuda":
        raise RuntimeError("the GB300 T builders run on CUDA devices only; there is no CPU fallback")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def smear_sigma(e, e0, ene_resolution):
    """Energy sigma e * res / 2.355 * (e0 / e) ** 0.5 as the reference forms it
    (process_list_plane_strict.py:158-159), evaluated by the same torch ops."""
    return e * ene_resolution / 2.355 * (e0 / e) ** 0.5


def uniform_sigma_sq_from_size(size_mm):
    """Variance of a uniform distribution over a crystal of ``size_mm`` (:55-56)."""
    return (size_mm ** 2) / 12.0


def detector_pos_sigma_sq(detector, extra_sigma):
    """Per-detector position variance (x, y, z) (process_list_plane_strict.py:59-96):
    crystal variances for a 4-layer planar detector (front layers 3 x 3 x 3 mm, rear
    layer 2 x 6 x 2 mm) plus extra_sigma^2, else an isotropic extra_sigma^2."""
    pos = detector[:, :3]
    yabs = torch.abs(pos[:, 1])
    layers = torch.sort(torch.unique(yabs))[0]
    if layers.numel() != 4:
        return torch.full((pos.size(0), 3), max(extra_sigma, 0.0) ** 2, dtype=pos.dtype, device=pos.device)
    out = torch.zeros((pos.size(0), 3), dtype=pos.dtype, device=pos.device)
    front = torch.tensor([uniform_sigma_sq_from_size(s) for s in FRONT_LAYER_CRYSTAL_MM], dtype=pos.dtype,
                         device=pos.device)
    rear = torch.tensor([uniform_sigma_sq_from_size(s) for s in REAR_LAYER_CRYSTAL_MM], dtype=pos.dtype,
                        device=pos.device)
    for k in range(4):
        out[yabs == layers[k], :] = front if k < 3 else rear
    if extra_sigma > 0:
        out = out + extra_sigma ** 2
    return out


def select_events(list_smeared, detector, delta_r1, delta_r2, e0, ene_resolution, thr_max, thr_min, thr_sum,
                  model=_lib.CONE_STRICT, theta_fp64=True, window_sigmas=0.0):
    """Run the selection kernel on a smeared list and compact the survivors.
    Returns ``(kept list indices int64, records [E', 16], row_id int32 [E'])``."""
    det = detector[:, :3].to(torch.float32).contiguous()
    if model != _lib.CONE_LEGACY:  # strict and simple records carry the strict fields
        s1 = detector_pos_sigma_sq(det, delta_r1).to(torch.float32).contiguous()
        s2 = detector_pos_sigma_sq(det, delta_r2).to(torch.float32).contiguous()
    else:
        s1 = s2 = None
    keep, rec, rid = ops.compton_event_prep(list_smeared, det, s1, s2, e0, ene_resolution, thr_max, thr_min,
                                            thr_sum, model=model, theta_fp64=theta_fp64,
                                            window_sigmas=window_sigmas, delta_r1=delta_r1, delta_r2=delta_r2)
    idx = torch.nonzero(keep).flatten()
    return idx, rec.index_select(0, idx).contiguous(), rid.index_select(0, idx).contiguous()


def finite_rows(t):
    """Rows without NaN and with a non-zero sum (process_list_plane_strict.py:241-246)."""
    return (torch.isnan(t).sum(dim=1) + (t.sum(dim=1) == 0)) == 0


def stable_rows(t_norm):
    """Effective support 1 / sum(t_norm^2) >= 50 (process_list_plane_strict.py:137-148)."""
    return (1.0 / torch.sum(t_norm ** 2, dim=1)) >= MIN_EVENT_EFFECTIVE_SUPPORT
