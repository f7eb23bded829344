"""Oracle: Compton cone T-row builders (TEST INFRASTRUCTURE ONLY — see oracle/__init__.py).

Numpy restatement of process_list_plane_strict.py (strict builder, :24-253) and
process_list_plane.py:17-107 (legacy builder). Energy smearing is NOT done here: the
functions take the already-smeared list (cp1, e1, cp2, e2) so that the random draws
of the reference (torch.randn) can be replayed exactly by the caller.

dtype=np.float32 follows the reference's float32 arithmetic (element-wise ops in the
reference's order); dtype=np.float64 is the high-precision oracle.
"""
from __future__ import annotations

import numpy as np

ELECTRON_REST_MEV = 0.511               # process_list_plane_strict.py:7
FRONT_LAYER_CRYSTAL_MM = (3.0, 3.0, 3.0)  # :5
REAR_LAYER_CRYSTAL_MM = (2.0, 6.0, 2.0)   # :6
MIN_EVENT_EFFECTIVE_SUPPORT = 50.0      # :8


def _c(x, dtype):
    return dtype(x)


def smear_energies(e, noise, e0, ene_resolution, dtype=np.float32):
    """process_list_plane_strict.py:158-161: e + (e * res / 2.355 * (e0 / e) ** 0.5) * noise.
    `e0 / e` is formed as reciprocal(e) * e0, as torch evaluates a scalar divided by a
    tensor. torch's CPU `** 0.5` is not always the correctly rounded square root, so this
    agrees with the reference to 1 ulp, not bit for bit; tests that need the reference's
    exact smeared list take it from the golden fixtures."""
    e = np.asarray(e, dtype=dtype)
    sigma = e * dtype(ene_resolution) / dtype(2.355) * np.sqrt((dtype(1) / e) * dtype(e0))
    return e + sigma * np.asarray(noise, dtype=dtype)


def compton_cos(e1, e0, dtype):
    """process_list_plane_strict.py:24-25 / :31."""
    e1 = np.asarray(e1, dtype=dtype)
    return dtype(1) - ((dtype(ELECTRON_REST_MEV) * e1) / ((dtype(e0) - e1) * dtype(e0)))


def compton_theta(e1, e0, dtype):
    """process_list_plane_strict.py:24-27."""
    c = np.clip(compton_cos(e1, e0, dtype), dtype(-1.0 + 1e-7), dtype(1.0 - 1e-7))
    return np.arccos(c)


def event_filter(list_smeared, detector_pos, e0, thr_max, thr_min, thr_sum, kinematic=True):
    """Thresholds (:164-175), kinematic filter (:30-36) and different-layer filter (:189).
    Returns the indices (into the list) of the surviving events, in list order.
    Always float32, as the reference (these decisions must match bit for bit)."""
    f32 = np.float32
    L = np.asarray(list_smeared, dtype=f32)
    cp1 = L[:, 0].astype(np.int32)
    cp2 = L[:, 2].astype(np.int32)
    e1, e2 = L[:, 1], L[:, 3]
    keep = (e1 < f32(thr_max)) & (e1 > f32(thr_min)) & (e2 > f32(thr_min)) & ((e1 + e2) > f32(thr_sum))
    if kinematic:
        c = compton_cos(e1, e0, f32)
        keep &= (c > f32(-1.0 + 1e-6)) & (c < f32(1.0 - 1e-6))
    det = np.asarray(detector_pos, dtype=f32)
    y1 = det[cp1 - 1, 1]
    y2 = det[cp2 - 1, 1]
    keep &= np.abs(y1 - y2) > f32(0.1)
    return np.nonzero(keep)[0]


def pos_sigma_sq(detector_pos, extra_sigma, dtype=np.float64):
    """process_list_plane_strict.py:55-96: per-detector position variance (x, y, z)."""
    det = np.asarray(detector_pos, dtype=dtype)
    yabs = np.abs(det[:, 1])
    layers = np.unique(yabs)
    if layers.size != 4:
        return np.full((det.shape[0], 3), max(extra_sigma, 0.0) ** 2, dtype=dtype)
    out = np.zeros((det.shape[0], 3), dtype=dtype)
    front = np.array([s * s / 12.0 for s in FRONT_LAYER_CRYSTAL_MM], dtype=dtype)
    rear = np.array([s * s / 12.0 for s in REAR_LAYER_CRYSTAL_MM], dtype=dtype)
    for k in range(4):
        out[yabs == layers[k], :] = front if k < 3 else rear
    if extra_sigma > 0:
        out = out + dtype(extra_sigma ** 2)
    return out


def cone_rows_strict(pos1, pos2, e1, s1sq, s2sq, coor, e0, ene_resolution, dtype=np.float64):
    """Strict cone kernel t_compton[i, j] (process_list_plane_strict.py:201-228):
    exp(-(beta-theta)^2 / (2 sigma^2)) * (KN - sin^2 beta), sigma^2 = sigma_pos^2 + sigma_E^2."""
    d = dtype
    pos1 = np.asarray(pos1, dtype=d)
    pos2 = np.asarray(pos2, dtype=d)
    e1 = np.asarray(e1, dtype=d)
    coor = np.asarray(coor, dtype=d)
    v01 = pos1[:, None, :] - coor[None, :, :]
    v12 = (pos2 - pos1)[:, None, :]
    d01 = np.sqrt((v01 * v01).sum(-1))
    d12 = np.sqrt((v12 * v12).sum(-1))
    theta = compton_theta(e1, e0, d)
    kn = d(e0) / (d(e0) - e1) + (d(e0) - e1) / d(e0)
    bcos = (v01 * v12).sum(-1) / np.maximum(d01 * d12, d(1e-7))
    beta = np.arccos(np.clip(bcos, d(-1.0 + 1e-7), d(1.0 - 1e-7)))
    # sigma_E (:39-52)
    sig_e = e1 * d(ene_resolution) / d(2.355) * np.sqrt(d(e0) / e1)
    lo = np.clip(e1 - sig_e, d(1e-7), d(e0) - d(1e-7))
    hi = np.clip(e1 + sig_e, d(1e-7), d(e0) - d(1e-7))
    s_minus = np.maximum(theta - compton_theta(lo, e0, d), d(1e-7))
    s_plus = np.maximum(compton_theta(hi, e0, d) - theta, d(1e-7))
    delta = beta - theta[:, None]
    sig_ene = np.where(delta >= 0, s_plus[:, None], s_minus[:, None])
    # sigma_pos (:99-134), first-hit source leg excluded
    u01 = v01 / np.maximum(d01, d(1e-7))[..., None]
    u12 = v12 / np.maximum(d12, d(1e-7))[..., None]
    cb = (u01 * u12).sum(-1, keepdims=True)
    sb = np.sqrt(np.maximum(d(1) - cb * cb, d(1e-12)))
    jac = (u01 - cb * u12) / np.maximum(d12, d(1e-7))[..., None]
    g1 = jac / sb
    g2 = -jac / sb
    s1 = np.asarray(s1sq, dtype=d)[:, None, :]
    s2 = np.asarray(s2sq, dtype=d)[:, None, :]
    sp2 = (g1 * g1 * s1).sum(-1) + (g2 * g2 * s2).sum(-1)
    sig_pos = np.sqrt(np.maximum(sp2, d(1e-12)))
    sig = np.sqrt(np.maximum(sig_pos ** 2 + sig_ene ** 2, d(1e-12)))
    return np.exp(-(delta ** 2) / (d(2) * sig ** 2)) * (kn[:, None] - np.sin(beta) ** 2)


def cone_rows_simple(pos1, pos2, e1, coor, e0, ene_resolution, dtype=np.float64):
    """Simple cone kernel: exp(-(beta - theta)^2 / (2 sigma_E^2)) / d01^2, with theta and the
    two-sided sigma_E of the strict model (process_list_plane_strict.py:24-27, :39-52) and
    neither sigma_pos nor the Klein-Nishina factor (the simplified list-mode kernel)."""
    d = dtype
    pos1 = np.asarray(pos1, dtype=d)
    pos2 = np.asarray(pos2, dtype=d)
    e1 = np.asarray(e1, dtype=d)
    coor = np.asarray(coor, dtype=d)
    v01 = pos1[:, None, :] - coor[None, :, :]
    v12 = (pos2 - pos1)[:, None, :]
    d01sq = (v01 * v01).sum(-1)
    d01 = np.sqrt(d01sq)
    d12 = np.sqrt((v12 * v12).sum(-1))
    theta = compton_theta(e1, e0, d)
    bcos = (v01 * v12).sum(-1) / np.maximum(d01 * d12, d(1e-7))
    beta = np.arccos(np.clip(bcos, d(-1.0 + 1e-7), d(1.0 - 1e-7)))
    sig_e = e1 * d(ene_resolution) / d(2.355) * np.sqrt(d(e0) / e1)
    lo = np.clip(e1 - sig_e, d(1e-7), d(e0) - d(1e-7))
    hi = np.clip(e1 + sig_e, d(1e-7), d(e0) - d(1e-7))
    s_minus = np.maximum(theta - compton_theta(lo, e0, d), d(1e-7))
    s_plus = np.maximum(compton_theta(hi, e0, d) - theta, d(1e-7))
    delta = beta - theta[:, None]
    sig = np.where(delta >= 0, s_plus[:, None], s_minus[:, None])
    return np.exp(-(delta ** 2) / (d(2) * sig ** 2)) / np.maximum(d01sq, d(1e-14))


def cone_rows_legacy(pos1, pos2, e1, coor, e0, ene_resolution, delta_r1, delta_r2, dtype=np.float64):
    """Legacy cone kernel (process_list_plane.py:56-83): derivative-based sigma_E, atan sigma_pos,
    no clamps."""
    d = dtype
    pos1 = np.asarray(pos1, dtype=d)
    pos2 = np.asarray(pos2, dtype=d)
    e1 = np.asarray(e1, dtype=d)
    coor = np.asarray(coor, dtype=d)
    ee = d(ELECTRON_REST_MEV)
    v01 = pos1[:, None, :] - coor[None, :, :]
    v12 = (pos2 - pos1)[:, None, :]
    d01 = np.sqrt((v01 * v01).sum(-1))
    d12 = np.sqrt((v12 * v12).sum(-1))
    with np.errstate(invalid="ignore", divide="ignore"):
        theta = np.arccos(d(1) - ((ee * e1) / ((d(e0) - e1) * d(e0))))
        er = e1 * d(ene_resolution) / d(2.355) * np.sqrt(d(e0) / e1)
        dth = (d(1) / np.abs(np.sin(theta))) * ee / (d(e0) - e1) ** 2
        d2th = ee / (np.sin(theta) * (d(e0) - e1) ** 3) * (d(2) - np.cos(theta) / np.sin(theta) ** 2 * ee /
                                                          (d(e0) - e1))
        kn = d(e0) / (d(e0) - e1) + (d(e0) - e1) / d(e0)
        beta = np.arccos((v01 * v12).sum(-1) / (d01 * d12))
        delta = beta - theta[:, None]
        s_plus = np.abs(dth * er + d(0.5) * d2th * er ** 2)[:, None]
        s_minus = np.abs(dth * er - d(0.5) * d2th * er ** 2)[:, None]
        sig_ene = np.where(delta >= 0, s_plus, s_minus)
        p = d01 / d12
        q = d(delta_r1) / d(delta_r2)
        sig_pos = np.arctan(d(delta_r1) / d01) * np.sqrt(d(1) + p ** 2 * (d(1) + q ** 2) + d(2) * p *
                                                          np.cos(theta)[:, None])
        sig = np.sqrt(sig_pos ** 2 + sig_ene ** 2)
        return np.exp(-(delta ** 2) / (d(2) * sig ** 2)) * (kn[:, None] - np.sin(beta) ** 2)


def finish_rows(t_compton, eff, stability=True):
    """NaN/zero-row filter (:241-246), row normalisation and the effective-support filter
    (:137-148). Returns (t_norm, t_compton_norm, t_single_norm, kept_index)."""
    t = t_compton * eff
    bad = np.isnan(t).any(axis=1) | (t.sum(axis=1) == 0)
    keep = np.nonzero(~bad)[0]
    t, tc, ts = t[keep], t_compton[keep], eff[keep]
    with np.errstate(invalid="ignore", divide="ignore"):
        tn = t / t.sum(axis=1, keepdims=True)
        tcn = tc / tc.sum(axis=1, keepdims=True)
        tsn = ts / ts.sum(axis=1, keepdims=True)
    if stability:
        support = 1.0 / np.sum(tn ** 2, axis=1)
        stable = support >= MIN_EVENT_EFFECTIVE_SUPPORT
        return tn[stable], tcn[stable], tsn[stable], keep[stable]
    return tn, tcn, tsn, keep


def strict_builder(sysmat, detector_pos, coor, list_smeared, delta_r1, delta_r2, e0, ene_resolution, thr_max,
                   thr_min, thr_sum, dtype=np.float64):
    """get_compton_backproj_list_single (strict, :151-253) on a pre-smeared list."""
    L = np.asarray(list_smeared, dtype=np.float32)
    idx = event_filter(L, detector_pos, e0, thr_max, thr_min, thr_sum)
    cp1 = L[idx, 0].astype(np.int64)
    cp2 = L[idx, 2].astype(np.int64)
    det = np.asarray(detector_pos)
    s1 = pos_sigma_sq(det, delta_r1, dtype)[cp1 - 1]
    s2 = pos_sigma_sq(det, delta_r2, dtype)[cp2 - 1]
    tc = cone_rows_strict(det[cp1 - 1], det[cp2 - 1], L[idx, 1], s1, s2, coor, e0, ene_resolution, dtype)
    eff = np.asarray(sysmat, dtype=dtype)[cp1 - 1]
    tn, tcn, tsn, keep = finish_rows(tc, eff, stability=True)
    return tn, tcn, tsn, idx[keep]


def legacy_builder(sysmat, detector_pos, coor, list_smeared, delta_r1, delta_r2, e0, ene_resolution, thr_max,
                   thr_min, thr_sum, dtype=np.float64):
    """get_compton_backproj_list_single (legacy, process_list_plane.py:17-107): no kinematic
    or stability filter."""
    L = np.asarray(list_smeared, dtype=np.float32)
    idx = event_filter(L, detector_pos, e0, thr_max, thr_min, thr_sum, kinematic=False)
    cp1 = L[idx, 0].astype(np.int64)
    cp2 = L[idx, 2].astype(np.int64)
    det = np.asarray(detector_pos)
    tc = cone_rows_legacy(det[cp1 - 1], det[cp2 - 1], L[idx, 1], coor, e0, ene_resolution, delta_r1, delta_r2,
                          dtype)
    eff = np.asarray(sysmat, dtype=dtype)[cp1 - 1]
    tn, tcn, tsn, keep = finish_rows(tc, eff, stability=False)
    return tn, tcn, tsn, idx[keep]
