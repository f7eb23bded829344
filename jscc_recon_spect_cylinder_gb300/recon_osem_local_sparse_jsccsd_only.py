"""Drop-in for the reference module ``recon_osem_local_sparse_jsccsd_only``.

Local joint SC + sparse-Compton OSEM (recon_osem_local_sparse_jsccsd_only.py): bin subsets
re-drawn every iteration with a seeded generator on the device, the clamped SC weight
scaled by alpha, the Compton weight in the materialise form (rows upsampled to the fine
grid, multiplied by the first-hit sysmat row, NaN -> 0, invalid rows dropped, rows
normalised, denominators clamped at 1e-12) scaled by (2 - alpha), and safe_em_update.
The Compton weight is one fused kernel pass per block: no fine row is stored.
"""
from __future__ import annotations

import time

import torch

from . import compton_sparse_ops as cso
from . import ops
from .recon_osem_local_cntstat import FORWARD_FLOOR, random_bin_subset_ids


def get_weight_single(sysmat, proj, img_rotate):
    """``A^T (y / clamp_min(A x, 1e-12))`` (recon_osem_local_sparse_jsccsd_only.py:8-10)."""
    return ops.sc_weight(sysmat, proj, img_rotate, floor=FORWARD_FLOOR)


def get_weight_compton_sparse(event_block, sysmat_full, img_rotate, sparse_projector):
    """Materialise-form Compton weight of one block (:13-19)."""
    if event_block.size(0) == 0:
        return torch.zeros_like(img_rotate)
    dev = img_rotate.device
    rows = event_block if event_block.device == dev else event_block.to(dev, non_blocking=True)
    return ops.sparse_weight(rows, sysmat_full, cso.tables(sparse_projector, dev), img_rotate, grouped=False)


def safe_em_update(img, weight, s_map, eps=1e-12):
    """NaN-safe EM update (:22-28)."""
    return ops.em_update(img, weight, s_map, safe=True, eps=eps)


def summarize_image_tensor(img):
    """One-line image statistics (:31-37)."""
    c = img.detach().float().cpu()
    return (f"min={c.min().item():.6e} max={c.max().item():.6e} mean={c.mean().item():.6e} "
            f"sum={c.sum().item():.6e} zero={int((c == 0).sum().item())}/{c.numel()}")


def build_random_bin_subsets(sysmat_all_device, proj_all_device, subset_num, generator):
    """Materialised random bin subsets (:40-55); the permutation is drawn on the
    projections' device when it is a GPU, else on the CPU, as the reference."""
    dev = proj_all_device[0].device if proj_all_device[0].is_cuda else "cpu"
    chunks = random_bin_subset_ids(proj_all_device[0].size(0), subset_num, generator, dev)
    sysmat_list_all = [[None] * len(sysmat_all_device) for _ in range(subset_num)]
    proj_list_all = [[None] * len(proj_all_device) for _ in range(subset_num)]
    for e in range(len(sysmat_all_device)):
        for s in range(min(subset_num, len(chunks))):
            sysmat_list_all[s][e] = sysmat_all_device[e][chunks[s], :]
            proj_list_all[s][e] = proj_all_device[e][chunks[s], :]
    return sysmat_list_all, proj_list_all


def _compton_block_weight(weight, t_l, sysmat_full_all, projector_all, rotmat_all, rotmat_inv_all, img, rotate_num,
                          alpha, device):
    for r in range(rotate_num):
        for t_rotate in t_l[r]:
            for t_block, sysmat_full, rotmat, rotmat_inv, proj in zip(t_rotate, sysmat_full_all, rotmat_all,
                                                                      rotmat_inv_all, projector_all):
                if t_block.numel() == 0:
                    continue
                if t_block.device != device:
                    t_block = t_block.to(device, non_blocking=True)
                ops.sparse_weight(t_block, sysmat_full, cso.tables(proj, device), img, grouped=False, rotmat=rotmat,
                                  rotmat_inv=rotmat_inv, rot_col=r, scale=2 - alpha, out=weight)


def osem_joint_mode_local_sparse(sysmat_l_all, proj_l_all, t_l_all, sysmat_full_all, sparse_projector_all, rotmat_all,
                                 rotmat_inv_all, img, s_map, alpha, rotate_num, device):
    """One joint pass over the subsets (:58-100): alpha * w_s + (2 - alpha) * w_c."""
    for sysmat_l, proj_l, t_l in zip(sysmat_l_all, proj_l_all, t_l_all):
        weight = torch.zeros_like(img)
        for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_l, proj_l, rotmat_all, rotmat_inv_all):
            if sysmat is None or sysmat.size(0) == 0:
                continue
            ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, n_rot=rotate_num, floor=FORWARD_FLOOR, scale=alpha,
                          out=weight)
        _compton_block_weight(weight, t_l, sysmat_full_all, sparse_projector_all, rotmat_all, rotmat_inv_all, img,
                              rotate_num, alpha, device)
        img = safe_em_update(img, weight, s_map)
    return img


def osem_joint_mode_local_sparse_indexed(sysmat_all, proj_all, subset_ids, t_l_all, sysmat_full_all,
                                         sparse_projector_all, rotmat_all, rotmat_inv_all, img, s_map, alpha,
                                         rotate_num, device):
    """osem_joint_mode_local_sparse with subsets given as bin-id chunks (no copies of A)."""
    for ids, t_l in zip(subset_ids, t_l_all):
        weight = torch.zeros_like(img)
        if ids.numel() > 0:
            for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_all, proj_all, rotmat_all, rotmat_inv_all):
                ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, n_rot=rotate_num, floor=FORWARD_FLOOR,
                              scale=alpha, out=weight, row_idx=ids)
        _compton_block_weight(weight, t_l, sysmat_full_all, sparse_projector_all, rotmat_all, rotmat_inv_all, img,
                              rotate_num, alpha, device)
        img = safe_em_update(img, weight, s_map)
    return img


def save_img_local_sparse_jsccsd_only(img_jsccsd, img_jsccsd_iter, iter_arg, save_path):
    """Raw float32 outputs (:103-108)."""
    img_jsccsd.detach().cpu().numpy().astype("float32").tofile(save_path + "Image_JSCCSD")
    img_jsccsd_iter.detach().cpu().numpy().astype("float32").tofile(
        save_path + "Image_JSCCSD_Iter_%d_%d" % (iter_arg.jsccsd, iter_arg.jsccsd / iter_arg.save_iter_step))
    print("Images saved to local disk.")


def stage_t_local(t_local_all, iter_arg, rotate_num, coarse_pixel_num, device):
    """t_local_all[energy][rotation] -> [subset][rotation][divide][energy] with torch.chunk
    at both levels (:141-161)."""
    empty = torch.zeros((0, coarse_pixel_num + 1), dtype=torch.float32, device=device)
    t_list_all = [[[[empty for _ in range(iter_arg.ene_num)] for _ in range(iter_arg.t_divide_num)]
                   for _ in range(rotate_num)] for _ in range(iter_arg.osem_subset_num)]
    for e in range(iter_arg.ene_num):
        for r in range(rotate_num):
            for s, t_sub in enumerate(torch.chunk(t_local_all[e][r], iter_arg.osem_subset_num, dim=0)):
                for d, t_div in enumerate(torch.chunk(t_sub, iter_arg.t_divide_num, dim=0)):
                    t_list_all[s][r][d][e] = t_div.to(device, non_blocking=True)
    return t_list_all


def run_recon_osem_local_sparse_jsccsd_only(sysmat_all, sysmat_full_all, rotmat_all, rotmat_inv_all, proj_all,
                                            t_local_all, sparse_projector_all, iter_arg, s_map_arg, alpha, save_path,
                                            device):
    """Local JSCCSD-only reconstruction (:111-202); ``device`` must be CUDA."""
    if device.type != "cuda":
        raise RuntimeError("the GB300 path runs on CUDA devices only; there is no CPU fallback")
    pixel_num = s_map_arg.j.size(0)
    rotate_num = rotmat_all[0].size(1)
    img = torch.ones([pixel_num, 1], dtype=torch.float32, device=device)
    img_iter = torch.ones([round(iter_arg.jsccsd / iter_arg.save_iter_step), pixel_num], dtype=torch.float32)
    generator = torch.Generator(device=device)
    generator.manual_seed(int(getattr(iter_arg, "seed", 20260331)))
    sys_d = [s.to(device, non_blocking=True) for s in sysmat_all]
    sys_full_d = [s.to(device, non_blocking=True) for s in sysmat_full_all]
    proj_d = [p.to(device, non_blocking=True) for p in proj_all]
    rot_d = [r.to(device, non_blocking=True) for r in rotmat_all]
    inv_d = [r.to(device, non_blocking=True) for r in rotmat_inv_all]
    projectors = [p.to(device) for p in sparse_projector_all]
    s_map = s_map_arg.j.to(device, non_blocking=True)
    t_list_all = stage_t_local(t_local_all, iter_arg, rotate_num, projectors[0].coarse_pixel_num, device)
    print("Starting local sparse JSCCSD-only reconstruction")
    t0 = time.time()
    k = 0
    for it in range(iter_arg.jsccsd):
        ids = random_bin_subset_ids(proj_d[0].size(0), iter_arg.osem_subset_num, generator, device)
        ids = ids + [ids[0][:0]] * (iter_arg.osem_subset_num - len(ids))
        img = osem_joint_mode_local_sparse_indexed(sys_d, proj_d, ids, t_list_all, sys_full_d, projectors, rot_d,
                                                   inv_d, img, s_map, alpha, rotate_num, device)
        if (it + 1) % iter_arg.save_iter_step == 0:
            img_iter[k, :] = img.squeeze().detach().cpu()
            k += 1
            print(f"[JSCCSD-Sparse-Only] Iter: {it + 1}/{iter_arg.jsccsd} | Time: {time.time() - t0:.2f}s | "
                  f"{summarize_image_tensor(img)}")
    print(f"Local sparse JSCCSD-only reconstruction time: {time.time() - t0:.2f}s")
    save_img_local_sparse_jsccsd_only(img, img_iter, iter_arg, save_path)
