"""Oracle: sparse Compton projector and sparse-row weights (TEST INFRASTRUCTURE ONLY).

Numpy restatement of compton_sparse_ops.py (:47-400), the sparse builder
process_list_plane_sparse.py:25-123, the grouped weight recon_osem_plane_sparse.py:22-57
and the materialise weight recon_osem_local_sparse_jsccsd_only.py:13-19. The projector
matrices are built as dense arrays exactly as the reference defines them (so tests can
compare them entry by entry); the operators use them as the reference does (matrix
products), which is slow but unambiguous.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import compton as oc

RADIUS_TOL_MM = 1e-4  # compton_sparse_ops.py:7
Z_TOL_MM = 1e-4       # :8


@dataclass
class Projector:
    theta_stride: int
    z_stride: int
    ring_strides: tuple
    fine_layer_num: int
    fine_z_num: int
    coarse_layer_num: int
    coarse_z_num: int
    fine_pixel_num: int
    coarse_pixel_num: int
    layer_reduce: np.ndarray
    z_reduce: np.ndarray
    layer_expand: np.ndarray
    z_expand: np.ndarray
    coor_coarse: np.ndarray


def _unique_consecutive(values, tol):
    """compton_sparse_ops.py:47-56."""
    uniq, counts = [values[0]], [1]
    for v in values[1:]:
        if abs(v - uniq[-1]) <= tol:
            counts[-1] += 1
        else:
            uniq.append(v)
            counts.append(1)
    return np.array(uniq), counts


def infer_polar_layout(coor_full):
    """compton_sparse_ops.py:59-92."""
    c = np.asarray(coor_full, dtype=np.float32)
    if c.ndim != 2 or c.shape[1] != 3:
        raise ValueError("coor_full must have shape [pixel_num, 3].")
    if c.shape[0] == 0:
        raise ValueError("coor_full is empty.")
    z_vals, z_counts = _unique_consecutive(c[:, 2], Z_TOL_MM)
    if len(set(z_counts)) != 1:
        raise ValueError("coor_full does not contain a consistent z-plane layout.")
    n_layer = z_counts[0]
    radii = np.sqrt(np.sum(c[:n_layer, :2].astype(np.float32) ** 2, axis=1, dtype=np.float32))
    lengths, ring_r = [], []
    s = 0
    while s < n_layer:
        e = s + 1
        while e < n_layer and abs(radii[e] - radii[s]) <= RADIUS_TOL_MM:
            e += 1
        lengths.append(e - s)
        ring_r.append(float(np.mean(radii[s:e], dtype=np.float32)))
        s = e
    return z_vals, len(z_counts), n_layer, lengths, ring_r


def periodic_reduce(n, stride):
    """compton_sparse_ops.py:95-106."""
    if n % stride:
        raise ValueError(f"fine_num={n} is not divisible by stride={stride}.")
    m = np.zeros((n // stride, n), dtype=np.float32)
    for c in range(n // stride):
        m[c, c * stride] = 1.0
    return m


def linear_reduce(n, stride):
    """compton_sparse_ops.py:109-129."""
    if n % stride:
        raise ValueError(f"fine_num={n} is not divisible by stride={stride}.")
    nc = n // stride
    m = np.zeros((nc, n), dtype=np.float32)
    pos_all = (np.arange(nc, dtype=np.float32) + np.float32(0.5)) * np.float32(stride) - np.float32(0.5)
    for c in range(nc):
        pos = float(pos_all[c])
        left = max(0, min(n - 1, math.floor(pos)))
        right = min(n - 1, left + 1)
        if right == left:
            m[c, left] = 1.0
            continue
        wr = pos - left
        m[c, left] += np.float32(1.0 - wr)
        m[c, right] += np.float32(wr)
    return m


def periodic_expand(n, stride):
    """compton_sparse_ops.py:132-154 (2-tap periodic linear interpolation)."""
    if n % stride:
        raise ValueError(f"fine_num={n} is not divisible by stride={stride}.")
    nc = n // stride
    m = np.zeros((n, nc), dtype=np.float32)
    for f in range(n):
        left = (f // stride) % nc
        right = (left + 1) % nc
        lpos = left * stride
        rpos = lpos + stride
        wr = (f - lpos) / max(rpos - lpos, 1e-12)
        m[f, left] += np.float32(1.0 - wr)
        m[f, right] += np.float32(wr)
    return m


def linear_expand(n, stride):
    """compton_sparse_ops.py:157-185."""
    if n % stride:
        raise ValueError(f"fine_num={n} is not divisible by stride={stride}.")
    nc = n // stride
    m = np.zeros((n, nc), dtype=np.float32)
    cpos = (np.arange(nc, dtype=np.float32) + np.float32(0.5)) * np.float32(stride) - np.float32(0.5)
    for f in range(n):
        ins = int(np.searchsorted(cpos, np.float32(f), side="left"))
        if ins <= 0:
            m[f, 0] = 1.0
            continue
        if ins >= nc:
            m[f, nc - 1] = 1.0
            continue
        lp, rp = float(cpos[ins - 1]), float(cpos[ins])
        wr = (float(f) - lp) / max(rp - lp, 1e-12)
        m[f, ins - 1] += np.float32(1.0 - wr)
        m[f, ins] += np.float32(wr)
    return m


def choose_ring_stride(ring_length, rotate_num, target):
    """compton_sparse_ops.py:188-209."""
    if target <= 1:
        return 1
    if rotate_num > 0 and ring_length % rotate_num == 0:
        step = ring_length // rotate_num
        for c in range(target, 0, -1):
            if ring_length % c == 0 and step % c == 0:
                return c
        return 1
    for c in range(target, 0, -1):
        if ring_length % c == 0:
            return c
    return 1


def _block_diag(blocks):
    rows = sum(b.shape[0] for b in blocks)
    cols = sum(b.shape[1] for b in blocks)
    out = np.zeros((rows, cols), dtype=np.float32)
    r = c = 0
    for b in blocks:
        out[r:r + b.shape[0], c:c + b.shape[1]] = b
        r += b.shape[0]
        c += b.shape[1]
    return out


def build_projector(coor_full, theta_stride=2, z_stride=2, rotate_num=None):
    """build_compton_sparse_projector (compton_sparse_ops.py:212-290)."""
    if theta_stride <= 0 or z_stride <= 0:
        raise ValueError("theta_stride and z_stride must be positive.")
    z_vals, nz, nl, lengths, ring_r = infer_polar_layout(coor_full)
    if nz % z_stride:
        raise ValueError(f"fine_z_num={nz} is not divisible by z_stride={z_stride}.")
    red, exp, parts, strides = [], [], [], []
    for L, R in zip(lengths, ring_r):
        st = choose_ring_stride(L, rotate_num, theta_stride) if rotate_num is not None else theta_stride
        red.append(periodic_reduce(L, st))
        exp.append(periodic_expand(L, st))
        strides.append(st)
        nc = L // st
        th = (np.arange(nc, dtype=np.float32) * np.float32(st)) * np.float32(2.0 * math.pi / L)
        parts.append(np.stack((np.float32(R) * np.cos(th), np.float32(R) * np.sin(th)), axis=1))
    lr, le = _block_diag(red), _block_diag(exp)
    layer = np.concatenate(parts, axis=0).astype(np.float32)
    zr, ze = linear_reduce(nz, z_stride), linear_expand(nz, z_stride)
    zc = (zr.astype(np.float64) @ z_vals.astype(np.float64)).astype(np.float32)
    coor = np.concatenate([np.concatenate((layer, np.full((layer.shape[0], 1), z, np.float32)), axis=1)
                           for z in zc], axis=0)
    return Projector(theta_stride, z_stride, tuple(strides), nl, nz, layer.shape[0], zc.size, nl * nz,
                     layer.shape[0] * zc.size, lr, zr, le, ze, coor)


def build_radial_projector(coor_full, radial_stride=4, theta_stride=4):
    """Radially coarsened projector (an extension: the reference's builder coarsens theta and
    z only, compton_sparse_ops.py:212-290). Every ring of the grid has the same length L; the
    rings of each z plane are coarsened by `radial_stride` with the reference's linear
    reduce / expand along the ring index (its z convention, :109-129 / :157-185: samples at
    the centres (c + 1/2) s - 1/2, two-tap interpolation between centres, clamped at the
    ends) and each ring's theta by `theta_stride` with its periodic maps (:95-106 /
    :132-154). Stored as the reference's separable pair with the (z plane, ring) index in the
    z slot and theta in the layer slot: the fine index z * n_rings * L + r * L + th is the
    reference's ring-major layout. Coarse coordinates: radius = the linear reduce of the ring
    radii, angle th_c * s_theta * 2 pi / L, the plane's z."""
    if radial_stride <= 0 or theta_stride <= 0:
        raise ValueError("radial_stride and theta_stride must be positive.")
    z_vals, nz, nl, lengths, ring_r = infer_polar_layout(coor_full)
    L = lengths[0]
    if any(n != L for n in lengths):
        raise ValueError("radial coarsening needs rings of one length.")
    nr = len(lengths)
    if nr % radial_stride:
        raise ValueError(f"ring count {nr} is not divisible by radial_stride={radial_stride}.")
    th_r, th_e = periodic_reduce(L, theta_stride), periodic_expand(L, theta_stride)
    r_r, r_e = linear_reduce(nr, radial_stride), linear_expand(nr, radial_stride)
    eye = np.eye(nz, dtype=np.float32)
    zr, ze = np.kron(eye, r_r).astype(np.float32), np.kron(eye, r_e).astype(np.float32)
    nrc, nthc = nr // radial_stride, L // theta_stride
    rad = (r_r.astype(np.float64) @ np.asarray(ring_r, dtype=np.float64)).astype(np.float32)
    th = (np.arange(nthc, dtype=np.float32) * np.float32(theta_stride)) * np.float32(2.0 * math.pi / L)
    plane = np.concatenate([np.stack((R * np.cos(th), R * np.sin(th)), axis=1) for R in rad], axis=0)
    coor = np.concatenate([np.concatenate((plane, np.full((plane.shape[0], 1), z, np.float32)), axis=1)
                           for z in z_vals.astype(np.float32)], axis=0).astype(np.float32)
    return Projector(theta_stride, 1, (theta_stride,) * nr, L, nz * nr, nthc, nz * nrc, nz * nr * L,
                     nz * nrc * nthc, th_r, zr, th_e, ze, coor)


def _rows3(rows, nz, nl):
    return np.asarray(rows).reshape(rows.shape[0], nz, nl)


def upsample_rows(rows_c, p, dtype=np.float64):
    """upsample_coarse_rows_to_fine (:331-342)."""
    r = _rows3(np.asarray(rows_c, dtype=dtype), p.coarse_z_num, p.coarse_layer_num)
    tmp = r @ p.layer_expand.T.astype(dtype)
    out = np.einsum("ezl,fz->efl", tmp, p.z_expand.astype(dtype))
    return out.reshape(out.shape[0], p.fine_pixel_num)


def adjoint_rows(rows_f, p, dtype=np.float64):
    """project_fine_rows_to_coarse_adjoint (:345-356)."""
    r = _rows3(np.asarray(rows_f, dtype=dtype), p.fine_z_num, p.fine_layer_num)
    tmp = r @ p.layer_expand.astype(dtype)
    out = np.einsum("ezl,zc->ecl", tmp, p.z_expand.astype(dtype))
    return out.reshape(out.shape[0], p.coarse_pixel_num)


def reduce_rows(rows_f, p, dtype=np.float64):
    """reduce_fine_rows_to_coarse (:317-328)."""
    r = _rows3(np.asarray(rows_f, dtype=dtype), p.fine_z_num, p.fine_layer_num)
    tmp = r @ p.layer_reduce.T.astype(dtype)
    out = np.einsum("ezl,cz->ecl", tmp, p.z_reduce.astype(dtype))
    return out.reshape(out.shape[0], p.coarse_pixel_num)


def reduce_image(img_f, p, dtype=np.float64):
    """reduce_fine_image_to_coarse (:293-302)."""
    x = np.asarray(img_f, dtype=dtype).reshape(p.fine_z_num, p.fine_layer_num)
    return (p.z_reduce.astype(dtype) @ (x @ p.layer_reduce.T.astype(dtype))).reshape(-1, 1)


def upsample_weight_image(w_c, p, dtype=np.float64):
    """upsample_coarse_weight_to_fine (:305-314)."""
    w = np.asarray(w_c, dtype=dtype).reshape(p.coarse_z_num, p.coarse_layer_num)
    return ((p.z_reduce.T.astype(dtype) @ w) @ p.layer_reduce.astype(dtype)).reshape(-1, 1)


def pack_rows(cp1, t_c):
    """pack_sparse_event_rows (:359-368)."""
    t_c = np.asarray(t_c)
    return np.concatenate((np.asarray(cp1).astype(t_c.dtype)[:, None], t_c), axis=1)


def unpack_rows(rows):
    """unpack_sparse_event_rows (:371-377)."""
    rows = np.asarray(rows)
    return np.round(rows[:, 0]).astype(np.int64), rows[:, 1:]


def materialize(rows, sysmat, p, dtype=np.float64):
    """materialize_sparse_event_rows_to_fine (:380-400) -> (t_norm[valid], valid)."""
    cp1, t_c = unpack_rows(rows)
    cp1 = np.clip(cp1 - 1, 0, sysmat.shape[0] - 1)
    t = np.nan_to_num(upsample_rows(t_c, p, dtype) * np.asarray(sysmat, dtype=dtype)[cp1], nan=0.0, posinf=0.0,
                      neginf=0.0)
    s = t.sum(axis=1, keepdims=True)
    valid = np.isfinite(s[:, 0]) & (s[:, 0] > 0)
    return t[valid] / s[valid], valid


def weight_materialize(rows, sysmat, x, p, dtype=np.float64):
    """get_weight_compton_sparse, materialise form (recon_osem_local_sparse_jsccsd_only.py:13-19)."""
    t, _ = materialize(rows, sysmat, p, dtype)
    x = np.asarray(x, dtype=dtype).reshape(-1, 1)
    if t.shape[0] == 0:
        return np.zeros_like(x)
    with np.errstate(divide="ignore"):
        w = t.T @ (dtype(1.0) / np.maximum(t @ x, dtype(1e-12)))
    return np.nan_to_num(w, nan=0.0, posinf=0.0, neginf=0.0)


def weight_grouped(rows, sysmat, x, p, dtype=np.float64):
    """get_weight_compton_sparse, grouped form (recon_osem_plane_sparse.py:22-57)."""
    x = np.asarray(x, dtype=dtype).reshape(-1, 1)
    if np.asarray(rows).shape[0] == 0:
        return np.zeros_like(x)
    cp1, t_c = unpack_rows(rows)
    cp1 = np.clip(cp1 - 1, 0, sysmat.shape[0] - 1)
    t_c = np.asarray(t_c, dtype=dtype)
    A = np.asarray(sysmat, dtype=dtype)
    w = np.zeros_like(x)
    for g in np.unique(cp1):
        m = cp1 == g
        s_row = A[g][None, :]
        back = adjoint_rows(x.T * s_row, p, dtype).T
        with np.errstate(divide="ignore"):
            wc = t_c[m].T @ (dtype(1.0) / np.maximum(t_c[m] @ back, dtype(1e-12)))
        w = w + s_row.T * upsample_rows(wc.T, p, dtype).T
    return np.nan_to_num(w, nan=0.0, posinf=0.0, neginf=0.0)


def sparse_builder(sysmat, detector_pos, p, list_smeared, delta_r1, delta_r2, e0, ene_resolution, thr_max,
                   thr_min, thr_sum, dtype=np.float64):
    """get_compton_backproj_list_single_sparse (process_list_plane_sparse.py:25-123) on a
    pre-smeared list -> (event_rows [E', 1 + Vc], surviving list indices)."""
    L = np.asarray(list_smeared, dtype=np.float32)
    idx = oc.event_filter(L, detector_pos, e0, thr_max, thr_min, thr_sum)
    if idx.size == 0:
        return np.zeros((0, p.coarse_pixel_num + 1), np.float32), idx
    cp1 = L[idx, 0].astype(np.int64)
    cp2 = L[idx, 2].astype(np.int64)
    det = np.asarray(detector_pos)
    s1 = oc.pos_sigma_sq(det, delta_r1, dtype)[cp1 - 1]
    s2 = oc.pos_sigma_sq(det, delta_r2, dtype)[cp2 - 1]
    tc = oc.cone_rows_strict(det[cp1 - 1], det[cp2 - 1], L[idx, 1], s1, s2, p.coor_coarse, e0, ene_resolution,
                             dtype)
    ts = reduce_rows(np.asarray(sysmat, dtype=dtype)[cp1 - 1], p, dtype)
    t = tc * ts
    bad = np.isnan(t).any(axis=1) | (t.sum(axis=1) == 0)
    keep = np.nonzero(~bad)[0]
    if keep.size == 0:
        return np.zeros((0, p.coarse_pixel_num + 1), np.float32), keep
    t, tc = t[keep], tc[keep]
    tn = t / t.sum(axis=1, keepdims=True)
    tcn = tc / tc.sum(axis=1, keepdims=True)
    stable = (1.0 / np.sum(tn ** 2, axis=1)) >= oc.MIN_EVENT_EFFECTIVE_SUPPORT
    rows = pack_rows(cp1[keep][stable], tcn[stable].astype(np.float32))
    return rows, idx[keep][stable]


# ----------------------------------------------------------------------------- sparse restatement
def upsample_matrix_csr(p):
    """The upsample operator as one scipy CSR matrix U [V_f, V_c] = kron(z_expand, layer_expand),
    the same linear map as upsample_rows (validated against it in tests), for CPU runs where
    the reference's dense products are prohibitive."""
    import scipy.sparse as sp

    return sp.kron(sp.csr_matrix(p.z_expand.astype(np.float64)), sp.csr_matrix(p.layer_expand.astype(np.float64)),
                   format="csr")


def weight_materialize_csr(rows, sysmat, x, U, dtype=np.float64):
    """weight_materialize with the upsample applied as a sparse matrix product."""
    x = np.asarray(x, dtype=dtype).reshape(-1, 1)
    rows = np.asarray(rows)
    if rows.shape[0] == 0:
        return np.zeros_like(x)
    cp1 = np.clip(np.round(rows[:, 0]).astype(np.int64) - 1, 0, sysmat.shape[0] - 1)
    up = np.asarray((U @ np.asarray(rows[:, 1:], dtype=dtype).T).T, dtype=dtype)
    t = np.nan_to_num(up * np.asarray(sysmat[cp1], dtype=dtype), nan=0.0, posinf=0.0, neginf=0.0)
    s = t.sum(axis=1, keepdims=True)
    valid = np.isfinite(s[:, 0]) & (s[:, 0] > 0)
    t = t[valid] / s[valid]
    with np.errstate(divide="ignore"):
        w = t.T @ (dtype(1.0) / np.maximum(t @ x, dtype(1e-12)))
    return np.nan_to_num(w, nan=0.0, posinf=0.0, neginf=0.0)


def sensitivity_d(rows, sysmat, p, dtype=np.float64):
    """main_local_sparse_jsccsd_only.py:95-108 (build_sparse_sensi_d_local) and the summing
    half of main_plane_sparse.py:214-226 (build_sparse_sensi_d): the sum over events of the
    normalised fine rows of materialize_sparse_event_rows_to_fine."""
    t, _ = materialize(rows, sysmat, p, dtype)
    return t.sum(axis=0)[:, None] if t.size else np.zeros((p.fine_pixel_num, 1), dtype=dtype)


def sensitivity_d_rescale(d, s_map_s, single_event_count_total, compton_event_count_total):
    """main_plane_sparse.py:228-230: d scaled to sum(s) * E_C / max(E_S, 1) when sum(d) > 0."""
    d = np.asarray(d, dtype=np.float64)
    if d.sum() > 0:
        d = d * np.sum(s_map_s) / d.sum()
        d = d * compton_event_count_total / max(single_event_count_total, 1)
    return d
