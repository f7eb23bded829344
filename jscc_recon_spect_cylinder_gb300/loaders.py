"""On-disk formats of the reference, loaded straight into the GPU path's layouts.

* SysMat_polar: raw float32, voxel-major ``[V, B]`` (the reference transposes it on the host:
  main_plane_sparse.py:307-308, ``fromfile(...).reshape(V, -1).T.copy() * intensity``). Here
  the file is read into pinned host memory in column blocks, each block is copied to the GPU
  and transposed / scaled / cast there, so the host never materialises the transposed copy and
  the matrix can land directly in BF16.
* Sensi_s / Sensi_d: raw float32 ``[V, 1]`` (main_plane_sparse.py:310-316).
* CntStat CSV ``[R x B]`` → projections ``[B, R]`` (main_plane_sparse.py:328-329).
* List CSVs ``(cp1, e1, cp2, e2)`` (sparse_main_utils.py:123-127).
* Factor CSVs: detector table, polar coordinates, rotation tables (main_plane_sparse.py:296-299).

Image outputs (raw float32 ``Image_*`` files) are written by ``recon_osem_plane.save_img`` and
the other mirrored savers.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch


def load_sysmat_polar(path, pixel_num, device="cuda", intensity=1.0, dtype=torch.float32, block_bins=4096):
    """The SC system matrix of ``path`` as ``[B, V]`` row-major on ``device`` in ``dtype``
    (float32 or bfloat16), scaled by ``intensity``: the reference's
    ``torch.from_numpy(np.fromfile(path, np.float32).reshape(V, -1).T.copy()) * intensity``.
    On a CUDA device the transpose, scale and cast run on the GPU block by block (``block_bins``
    bins at a time); on the CPU the reference's own expression is evaluated."""
    path = Path(path)
    n = path.stat().st_size // 4
    if n % pixel_num:
        raise ValueError(f"{path}: {n} floats is not a multiple of pixel_num={pixel_num}")
    n_bins = n // pixel_num
    raw = np.memmap(path, dtype=np.float32, mode="r", shape=(pixel_num, n_bins))
    device = torch.device(device)
    if device.type != "cuda":
        out = torch.from_numpy(np.ascontiguousarray(raw.T)) * intensity
        return out.to(dtype)
    out = torch.empty((n_bins, pixel_num), dtype=dtype, device=device)
    host = torch.empty((pixel_num, min(block_bins, n_bins)), dtype=torch.float32).pin_memory()
    stream = torch.cuda.current_stream(device)
    for b0 in range(0, n_bins, block_bins):
        nb = min(block_bins, n_bins - b0)
        h = host[:, :nb]
        stream.synchronize()  # the previous block's copy out of the pinned buffer is done
        h.copy_(torch.from_numpy(np.ascontiguousarray(raw[:, b0:b0 + nb])))
        blk = h.to(device, non_blocking=True)
        out[b0:b0 + nb] = (blk.t() * intensity).to(dtype)
    torch.cuda.synchronize(device)
    return out


def load_sensitivity(path, pixel_num, intensity=1.0):
    """Sensi_s / Sensi_d: ``np.fromfile(path, np.float32).reshape(V, 1) * intensity``."""
    return torch.from_numpy(np.fromfile(path, dtype=np.float32).reshape(pixel_num, 1).copy()) * intensity


def load_cntstat(path, rotate_num):
    """CntStat CSV ``[R x B]`` → projections ``[B, R]`` float32 (main_plane_sparse.py:328-329)."""
    proj_np = np.genfromtxt(path, delimiter=",", dtype=np.float32)
    return torch.from_numpy(proj_np.reshape(rotate_num, -1).T.copy())


def load_list_csv(list_file_path):
    """List CSV → ``[E, 4]`` float32 (cp1, e1, cp2, e2); one event per line, a single-line file
    gives one row (sparse_main_utils.py:123-127)."""
    list_np = np.genfromtxt(list_file_path, delimiter=",", dtype=np.float32)
    if list_np.ndim == 1:
        list_np = np.expand_dims(list_np, axis=0)
    return torch.from_numpy(list_np[:, 0:4])


def load_factors(factor_dir, detector_file_path):
    """Detector positions ``[n_det, 3]`` (columns 1-3 of the detector CSV), polar coordinates
    ``[V, 3]`` and the 1-based int64 rotation tables ``[V, R]`` of a factor directory
    (main_plane_sparse.py:296-299)."""
    factor_dir = Path(factor_dir)
    detector = torch.from_numpy(np.genfromtxt(detector_file_path, delimiter=",", dtype=np.float32)[:, 1:4])
    coor_polar = torch.from_numpy(np.genfromtxt(factor_dir / "coor_polar_full.csv", delimiter=",", dtype=np.float32))
    rotmat = torch.from_numpy(np.genfromtxt(factor_dir / "RotMat_full.csv", delimiter=",", dtype=np.int64))
    rotmat_inv = torch.from_numpy(np.genfromtxt(factor_dir / "RotMatInv_full.csv", delimiter=",", dtype=np.int64))
    return detector, coor_polar, rotmat, rotmat_inv
