"""Oracle: SC and dense-T OSEM (TEST INFRASTRUCTURE ONLY — see oracle/__init__.py).

Restates recon_osem_plane.py:8-125, recon_osem_local_cntstat.py:6-45 and
recon_osem_plane_sparse.py:60-66 in numpy. Loops keep the reference's order
(subset -> rotation -> energy) so float32 mode rounds like the reference's CPU run.
"""
from __future__ import annotations

import numpy as np


def split_even_bounds(n: int, parts: int) -> list[tuple[int, int]]:
    """recon_osem_plane.py:8-18 (split_tensor_even): floor-balanced bounds."""
    if parts <= 0:
        raise ValueError("parts must be positive")
    return [(n * k // parts, n * (k + 1) // parts) for k in range(parts)]


def chunk_bounds(n: int, parts: int) -> list[tuple[int, int]]:
    """torch.chunk semantics (recon_osem_local_cntstat.py:14): ceil-sized chunks,
    possibly fewer than `parts`."""
    if n == 0:
        return [(0, 0)]
    size = -(-n // parts)
    return [(s, min(s + size, n)) for s in range(0, n, size)]


def get_weight_single(A, y, x, floor=None, dtype=np.float64):
    """recon_osem_plane.py:28-30; with floor: recon_osem_local_cntstat.py:6-8."""
    A = np.asarray(A, dtype=dtype)
    f = A @ np.asarray(x, dtype=dtype)
    if floor is not None:
        f = np.maximum(f, dtype(floor))
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.asarray(y, dtype=dtype) / f
    return A.T @ q


def get_weight_compton(t, x, dtype=np.float64):
    """recon_osem_plane.py:33-42: T^T (1 / (T x))."""
    t = np.asarray(t, dtype=dtype)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = dtype(1.0) / (t @ np.asarray(x, dtype=dtype))
    return t.T @ q


def _rot(x, table, r):
    return x[np.asarray(table)[:, r] - 1]


def osem_bin_mode(sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, img, s_map, rotate_num,
                  floor=None, dtype=np.float64):
    """recon_osem_plane.py:45-61 (floor=None) / recon_osem_local_cntstat.py:28-45 (floor=1e-12)."""
    img = np.asarray(img, dtype=dtype).reshape(-1, 1)
    s = np.asarray(s_map, dtype=dtype).reshape(-1, 1)
    for sysmat_list, proj_list in zip(sysmat_list_all, proj_list_all):
        weight = np.zeros_like(img)
        for i in range(rotate_num):
            for A, y, rm, ri in zip(sysmat_list, proj_list, rotmat_all, rotmat_inv_all):
                if np.asarray(A).shape[0] == 0:
                    continue
                w = get_weight_single(A, np.asarray(y, dtype=dtype)[:, i:i + 1], _rot(img, rm, i), floor, dtype)
                weight = weight + _rot(w, ri, i)
        with np.errstate(divide="ignore", invalid="ignore"):
            img = img * weight / s
    return img


def osem_list_mode(t_list_all, rotmat_all, rotmat_inv_all, img, s_map, rotate_num, dtype=np.float64):
    """recon_osem_plane.py:63-80."""
    img = np.asarray(img, dtype=dtype).reshape(-1, 1)
    s = np.asarray(s_map, dtype=dtype).reshape(-1, 1)
    for t_list in t_list_all:
        weight = np.zeros_like(img)
        for i in range(rotate_num):
            for t in t_list[i]:
                for t_tmp, rm, ri in zip(t, rotmat_all, rotmat_inv_all):
                    if np.asarray(t_tmp).size == 0:
                        continue
                    w = get_weight_compton(t_tmp, _rot(img, rm, i), dtype)
                    weight = weight + _rot(w, ri, i)
        with np.errstate(divide="ignore", invalid="ignore"):
            img = img * weight / s
    return img


def osem_joint_mode(sysmat_list_all, proj_list_all, t_list_all, rotmat_all, rotmat_inv_all, img, s_map, alpha,
                    rotate_num, dtype=np.float64):
    """recon_osem_plane.py:100-125."""
    img = np.asarray(img, dtype=dtype).reshape(-1, 1)
    s = np.asarray(s_map, dtype=dtype).reshape(-1, 1)
    for sysmat_list, proj_list, t_list in zip(sysmat_list_all, proj_list_all, t_list_all):
        w_c = np.zeros_like(img)
        w_s = np.zeros_like(img)
        for i in range(rotate_num):
            for A, y, rm, ri in zip(sysmat_list, proj_list, rotmat_all, rotmat_inv_all):
                w = get_weight_single(A, np.asarray(y, dtype=dtype)[:, i:i + 1], _rot(img, rm, i), None, dtype)
                w_s = w_s + _rot(w, ri, i)
            for t in t_list[i]:
                for t_tmp, rm, ri in zip(t, rotmat_all, rotmat_inv_all):
                    if np.asarray(t_tmp).size == 0:
                        continue
                    w = get_weight_compton(t_tmp, _rot(img, rm, i), dtype)
                    w_c = w_c + _rot(w, ri, i)
        weight = dtype(2 - alpha) * w_c + dtype(alpha) * w_s
        with np.errstate(divide="ignore", invalid="ignore"):
            img = img * weight / s
    return img


def safe_em_update(img, weight, s_map, eps=1e-12, dtype=np.float64):
    """recon_osem_plane_sparse.py:60-66."""
    img = np.asarray(img, dtype=dtype)
    w = np.nan_to_num(np.asarray(weight, dtype=dtype), nan=0.0, posinf=0.0, neginf=0.0)
    s = np.nan_to_num(np.asarray(s_map, dtype=dtype), nan=0.0, posinf=0.0, neginf=0.0)
    valid = s > dtype(eps)
    out = np.zeros_like(img)
    out[valid] = img[valid] * np.maximum(w[valid], 0.0) / s[valid]
    return out


def sc_sensitivity(A, rotinv, rotate_num, dtype=np.float64):
    """main_local_cntstat.py:140-146 (compute_sensitivity_local; the same formula as
    main_plane_sparse.py:440-444): s = (1/R) sum_r colsum(A)[rotinv[:, r] - 1]."""
    A = np.asarray(A, dtype=dtype)
    col = A.sum(axis=0)
    s = np.zeros(A.shape[1], dtype=dtype)
    for r in range(rotate_num):
        s = s + col[np.asarray(rotinv)[:, r].astype(np.int64) - 1]
    return (s / rotate_num)[:, None]
