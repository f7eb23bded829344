"""Drop-in for the reference module ``recon_osem_plane_sparse`` (sparse-Compton OSEM).

get_weight_compton_sparse keeps the grouped form's semantics (recon_osem_plane_sparse.py:22-57:
first-hit ids clamped to the sysmat rows, denominators clamped at 1e-12, nan_to_num of the
block's weight) but runs as one fused kernel pass over the packed coarse rows: the
per-group adjoint / upsample matrix products of the reference become two-tap gathers and
the Python loop over unique first-hit detectors disappears. safe_em_update and the loops
keep the reference's order and nesting.
"""
from __future__ import annotations

import os
import time

import torch
import torch.multiprocessing as mp

from . import compton_sparse_ops as cso
from . import ops
from .recon_osem_plane import collect_worker_weights, join_workers
from .recon_osem_plane import (  # noqa: F401  (re-exported, as the reference does)
    get_gpu_memory_usage,
    get_t_budget_bytes_per_gpu,
    get_weight_single,
    osem_bin_mode,
    save_img,
    split_tensor_even,
)


def get_weight_compton_sparse(event_block, sysmat_full, img_fine, sparse_projector):
    """Compton weight of one packed sparse block (recon_osem_plane_sparse.py:22-57)."""
    dev = img_fine.device
    if event_block.size(0) == 0:
        return torch.zeros_like(img_fine)
    rows = event_block if event_block.device == dev else event_block.to(dev, non_blocking=True)
    sysmat = sysmat_full if sysmat_full.device == dev else sysmat_full.to(dev, non_blocking=True)
    return ops.sparse_weight(rows, sysmat, cso.tables(sparse_projector, dev), img_fine, grouped=True)


def safe_em_update(img, weight, s_map, eps=1e-12):
    """NaN-safe EM update (recon_osem_plane_sparse.py:60-66)."""
    return ops.em_update(img, weight, s_map, safe=True, eps=eps)


def _accumulate_compton_sparse(weight, t_list, sysmat_all, projector_all, rotmat_all, rotmat_inv_all, img, rotate_num,
                               scale=1.0, grouped=True):
    dev = img.device
    for r in range(rotate_num):
        for t in t_list[r]:
            for t_tmp, sysmat_full, rotmat, rotmat_inv, proj in zip(t, sysmat_all, rotmat_all, rotmat_inv_all,
                                                                    projector_all):
                if t_tmp.numel() == 0:
                    continue
                rows = t_tmp if t_tmp.device == dev else t_tmp.to(dev, non_blocking=True)
                sysmat = sysmat_full if sysmat_full.device == dev else sysmat_full.to(dev, non_blocking=True)
                ops.sparse_weight(rows, sysmat, cso.tables(proj, dev), img, grouped=grouped, rotmat=rotmat,
                                  rotmat_inv=rotmat_inv, rot_col=r, scale=scale, out=weight)


def _apply_denoiser(img, model_denoiser):
    n = int(img.shape[0] ** 0.5)
    return torch.clamp(model_denoiser(img.view(1, 1, n, n)).view(n * n, 1), min=0)


def osem_list_mode_sparse(t_list_all, sysmat_all, sparse_projector_all, rotmat_all, rotmat_inv_all, img, s_map,
                          rotate_num, model_denoiser=None):
    """Sparse list-mode OSEM (recon_osem_plane_sparse.py:69-88)."""
    for t_list in t_list_all:
        weight = torch.zeros_like(img)
        _accumulate_compton_sparse(weight, t_list, sysmat_all, sparse_projector_all, rotmat_all, rotmat_inv_all, img,
                                   rotate_num)
        img = safe_em_update(img, weight, s_map)
        if model_denoiser is not None:
            img = _apply_denoiser(img, model_denoiser)
    return img


def osem_joint_mode_sparse(sysmat_list_all, proj_list_all, t_list_all, sysmat_all, sparse_projector_all, rotmat_all,
                           rotmat_inv_all, img, s_map, alpha, rotate_num, model_denoiser=None):
    """Joint SC + sparse Compton OSEM (recon_osem_plane_sparse.py:91-118)."""
    for sysmat_list, proj_list, t_list in zip(sysmat_list_all, proj_list_all, t_list_all):
        w_c = torch.zeros_like(img)
        w_s = torch.zeros_like(img)
        for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_list, proj_list, rotmat_all, rotmat_inv_all):
            ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, rot_start=0, n_rot=rotate_num, out=w_s)
        _accumulate_compton_sparse(w_c, t_list, sysmat_all, sparse_projector_all, rotmat_all, rotmat_inv_all, img,
                                   rotate_num)
        img = ops.em_update(img, w_c, s_map, safe=True, coef=2 - alpha, weight_b=w_s, coef_b=alpha)
        if model_denoiser is not None:
            img = _apply_denoiser(img, model_denoiser)
    return img


def osem_list_mode_mp_sparse(t_list_all, sysmat_all, sparse_projector_all, rotmat_all, rotmat_inv_all, iter_num,
                             rank, img_queue, weight_queue, rotate_num, model_denoiser=None):
    """Queue worker of the multi-process sparse list mode (recon_osem_plane_sparse.py:121-141)."""
    del model_denoiser
    with torch.no_grad():
        dev = torch.device(f"cuda:{rank}")
        sysmat_all = [s.to(dev, non_blocking=True) for s in sysmat_all]
        projector_all = [p.to(dev) for p in sparse_projector_all]
        rot_dev = [r.to(dev) for r in rotmat_all]
        inv_dev = [r.to(dev) for r in rotmat_inv_all]
        for _ in range(iter_num):
            for t_list in t_list_all:
                img = img_queue.get().to(dev)
                weight = torch.zeros_like(img)
                _accumulate_compton_sparse(weight, t_list, sysmat_all, projector_all, rot_dev, inv_dev, img,
                                           rotate_num)
                weight_queue.put(weight.to("cuda:0"))


def run_recon_osem_sparse(sysmat_all, rotmat_all, rotmat_inv_all, proj_all, proj_d_all, t_all, sparse_projector_all,
                          iter_arg, s_map_arg, alpha, save_path, num_gpus, model_denoiser=None):
    """SC -> SC-D -> JSCC-D -> JSCC-SD with sparse Compton rows (recon_osem_plane_sparse.py:144-348)."""
    from .recon_osem_plane import _stage_t_blocks

    os.makedirs(save_path, exist_ok=True)
    dev = torch.device("cuda:0")
    pixel_num = sysmat_all[0].size(1)
    rotate_num = rotmat_all[0].size(1)
    S = iter_arg.osem_subset_num
    step = iter_arg.save_iter_step

    def ones_img():
        return torch.ones([pixel_num, 1], dtype=torch.float32).to(dev, non_blocking=True)

    img_sc, img_scd, img_jsccd, img_jsccsd = ones_img(), ones_img(), ones_img(), ones_img()
    img_sc_iter = torch.ones([round(iter_arg.sc / step), pixel_num], dtype=torch.float32)
    img_scd_iter = torch.ones([round(iter_arg.jsccd / step), pixel_num], dtype=torch.float32)
    img_jsccd_iter = torch.ones([round(iter_arg.jsccd / step), pixel_num], dtype=torch.float32)
    img_jsccsd_iter = torch.ones([round(iter_arg.jsccsd / step), pixel_num], dtype=torch.float32)

    bins = torch.arange(0, proj_all[0].size(dim=0))
    bins = bins[torch.randperm(proj_all[0].size(dim=0))]
    bin_subsets = split_tensor_even(bins, S, dim=0)
    t_list_all = _stage_t_blocks(t_all, rotate_num, iter_arg, num_gpus)
    sysmat_list_all = [[None] * iter_arg.ene_num for _ in range(S)]
    proj_list_all = [[None] * iter_arg.ene_num for _ in range(S)]
    proj_d_list_all = [[None] * iter_arg.ene_num for _ in range(S)]
    for e, (sysmat, proj, proj_d) in enumerate(zip(sysmat_all, proj_all, proj_d_all)):
        rotmat_all[e] = rotmat_all[e].to(dev, non_blocking=True)
        rotmat_inv_all[e] = rotmat_inv_all[e].to(dev, non_blocking=True)
        for s, ids in enumerate(bin_subsets):
            sysmat_list_all[s][e] = sysmat[ids, :].to(dev, non_blocking=True)
            proj_list_all[s][e] = proj[ids, :].to(dev, non_blocking=True)
            proj_d_list_all[s][e] = proj_d[ids, :].to(dev, non_blocking=True)
    if num_gpus == 1:
        sysmat_all = [s.to(dev, non_blocking=True) for s in sysmat_all]
    del t_all
    s_map_arg.s = s_map_arg.s.to(dev, non_blocking=True)
    s_map_arg.d = s_map_arg.d.to(dev, non_blocking=True)
    s_map_arg.j = alpha * s_map_arg.s + (2 - alpha) * s_map_arg.d
    if model_denoiser is not None:
        model_denoiser.to(dev)
    get_gpu_memory_usage(num_gpus)
    t0 = time.time()

    def run_phase(name, n_iter, fn, img, snaps):
        print(f"{name} OSEM starts")
        k = 0
        for it in range(n_iter):
            img = fn(img)
            if (it + 1) % step == 0:
                snaps[k, :] = torch.squeeze(img).cpu()
                k += 1
                print(f"{name} iteration {it + 1} ends, time used: {time.time() - t0:.3f} s")
        return img

    img_sc = run_phase("SC", iter_arg.sc, lambda x: osem_bin_mode(
        sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, x, s_map_arg.s, rotate_num, model_denoiser),
        img_sc, img_sc_iter)
    img_scd = run_phase("SC-D", iter_arg.jsccd, lambda x: osem_bin_mode(
        sysmat_list_all, proj_d_list_all, rotmat_all, rotmat_inv_all, x, s_map_arg.s, rotate_num, model_denoiser),
        img_scd, img_scd_iter)
    if num_gpus == 1:
        proj_gpu = [p.to(dev) for p in sparse_projector_all]
        img_jsccd = run_phase("JSCC-D sparse", iter_arg.jsccd, lambda x: osem_list_mode_sparse(
            t_list_all, sysmat_all, proj_gpu, rotmat_all, rotmat_inv_all, x, s_map_arg.d, rotate_num,
            model_denoiser), img_jsccd, img_jsccd_iter)
        img_jsccsd = run_phase("JSCC-SD sparse", iter_arg.jsccsd, lambda x: osem_joint_mode_sparse(
            sysmat_list_all, proj_list_all, t_list_all, sysmat_all, proj_gpu, rotmat_all, rotmat_inv_all, x,
            s_map_arg.j, alpha, rotate_num, model_denoiser), img_jsccsd, img_jsccsd_iter)
    else:
        img_queue, weight_queue = mp.Queue(), mp.Queue()

        def mp_phase(n_iter, img, snaps, joint):
            procs = [mp.Process(target=osem_list_mode_mp_sparse, args=(
                t_list_all[g], sysmat_all, sparse_projector_all, rotmat_all, rotmat_inv_all, n_iter, g, img_queue,
                weight_queue, rotate_num, model_denoiser)) for g in range(num_gpus)]
            for p in procs:
                p.start()
            k = 0
            for it in range(n_iter):
                for s in range(S):
                    for _ in range(num_gpus):
                        img_queue.put(img)
                    w_c = torch.zeros_like(img)
                    for w in collect_worker_weights(weight_queue, procs, num_gpus, "sparse list-mode OSEM"):
                        w_c = w_c + w
                    if joint:
                        w_s = torch.zeros_like(img)
                        for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_list_all[s], proj_list_all[s], rotmat_all,
                                                                    rotmat_inv_all):
                            ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, n_rot=rotate_num, out=w_s)
                        img = ops.em_update(img, w_c, s_map_arg.j, safe=True, coef=2 - alpha, weight_b=w_s,
                                            coef_b=alpha)
                    else:
                        img = safe_em_update(img, w_c, s_map_arg.d)
                if (it + 1) % step == 0:
                    snaps[k, :] = torch.squeeze(img).cpu()
                    k += 1
            join_workers(procs, "sparse list-mode OSEM")
            return img

        img_jsccd = mp_phase(iter_arg.jsccd, img_jsccd, img_jsccd_iter, joint=False)
        img_jsccsd = mp_phase(iter_arg.jsccsd, img_jsccsd, img_jsccsd_iter, joint=True)
    save_img(img_sc, img_scd, img_jsccd, img_jsccsd, img_sc_iter, img_scd_iter, img_jsccd_iter, img_jsccsd_iter,
             iter_arg, save_path)
