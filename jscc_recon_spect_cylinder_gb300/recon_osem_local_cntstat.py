"""Drop-in for the reference module ``recon_osem_local_cntstat`` (device-parameterised SC OSEM).

Mirrors recon_osem_local_cntstat.py: a new seeded ``torch.randperm`` of the bins every
iteration, ``torch.chunk`` (ceil-sized) subsets, clamped forward projection
``clamp_min(1e-12)`` and the plain ``img * w / s`` update. The runner passes the
subset's bin ids straight to the kernel (``row_idx``) instead of copying the subset
rows of A every iteration; the summation order over rows is the same as with the
copied subset, so results are bit-identical to the copying form.
"""
from __future__ import annotations

import time

import torch

from . import ops

FORWARD_FLOOR = 1e-12


def get_weight_single(sysmat, proj, img_rotate):
    """``A^T (y / clamp_min(A x, 1e-12))`` (recon_osem_local_cntstat.py:6-8)."""
    return ops.sc_weight(sysmat, proj, img_rotate, floor=FORWARD_FLOOR)


def random_bin_subset_ids(local_bin_num, subset_num, generator, device):
    """The bin permutation and ceil-sized chunks of recon_osem_local_cntstat.py:12-14."""
    perm = torch.randperm(local_bin_num, generator=generator, device=device)
    return list(torch.chunk(perm, subset_num, dim=0))


def build_random_bin_subsets(sysmat_all_device, proj_all_device, subset_num, generator):
    """Materialised random bin subsets (recon_osem_local_cntstat.py:11-25)."""
    chunks = random_bin_subset_ids(proj_all_device[0].size(0), subset_num, generator,
                                   proj_all_device[0].device)
    sysmat_list_all = [[None] * len(sysmat_all_device) for _ in range(subset_num)]
    proj_list_all = [[None] * len(proj_all_device) for _ in range(subset_num)]
    for e in range(len(sysmat_all_device)):
        for s in range(subset_num):
            sysmat_list_all[s][e] = sysmat_all_device[e][chunks[s], :]
            proj_list_all[s][e] = proj_all_device[e][chunks[s], :]
    return sysmat_list_all, proj_list_all


def osem_bin_mode_local(sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, img, s_map):
    """One SC OSEM pass over materialised subsets (recon_osem_local_cntstat.py:28-45)."""
    rotate_num = rotmat_all[0].size(1)
    for sysmat_list, proj_list in zip(sysmat_list_all, proj_list_all):
        weight = torch.zeros_like(img)
        for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_list, proj_list, rotmat_all, rotmat_inv_all):
            if sysmat.size(0) == 0:
                continue
            ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, n_rot=rotate_num, floor=FORWARD_FLOOR,
                          out=weight)
        img = ops.em_update(img, weight, s_map, safe=False)
    return img


def osem_bin_mode_local_indexed(sysmat_all_device, proj_all_device, subset_ids, rotmat_all, rotmat_inv_all,
                                img, s_map):
    """osem_bin_mode_local over subsets given as bin-id chunks (no copies of A)."""
    rotate_num = rotmat_all[0].size(1)
    for ids in subset_ids:
        weight = torch.zeros_like(img)
        if ids.numel() > 0:
            for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_all_device, proj_all_device, rotmat_all,
                                                        rotmat_inv_all):
                ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, n_rot=rotate_num, floor=FORWARD_FLOOR,
                              out=weight, row_idx=ids)
        img = ops.em_update(img, weight, s_map, safe=False)
    return img


def save_img_local_cntstat(img_sc, img_sc_iter, iter_arg, save_path):
    """Raw float32 outputs (recon_osem_local_cntstat.py:48-53)."""
    img_sc.detach().cpu().numpy().astype("float32").tofile(save_path + "Image_SC")
    img_sc_iter.detach().cpu().numpy().astype("float32").tofile(
        save_path + "Image_SC_Iter_%d_%d" % (iter_arg.sc, iter_arg.sc / iter_arg.save_iter_step))
    print("Images saved to local disk.")


def run_recon_osem_local_cntstat(sysmat_all, rotmat_all, rotmat_inv_all, proj_all, iter_arg, s_map_arg, save_path,
                                 device):
    """SC-only reconstruction (recon_osem_local_cntstat.py:56-100); ``device`` must be CUDA."""
    if device.type != "cuda":
        raise RuntimeError("the GB300 path runs on CUDA devices only; there is no CPU fallback")
    pixel_num = s_map_arg.s.size(0)
    img_sc = torch.ones([pixel_num, 1], dtype=torch.float32, device=device)
    img_sc_iter = torch.ones([round(iter_arg.sc / iter_arg.save_iter_step), pixel_num], dtype=torch.float32)
    generator = torch.Generator(device=device)
    generator.manual_seed(int(getattr(iter_arg, "seed", 20260331)))

    sysmat_dev = [s.to(device, non_blocking=True) for s in sysmat_all]
    proj_dev = [p.to(device, non_blocking=True) for p in proj_all]
    rot_dev = [r.to(device, non_blocking=True) for r in rotmat_all]
    inv_dev = [r.to(device, non_blocking=True) for r in rotmat_inv_all]
    s_map = s_map_arg.s.to(device, non_blocking=True)

    print("Starting local single-photon reconstruction")
    t0 = time.time()
    k = 0
    for it in range(iter_arg.sc):
        ids = random_bin_subset_ids(proj_dev[0].size(0), iter_arg.osem_subset_num, generator, device)
        img_sc = osem_bin_mode_local_indexed(sysmat_dev, proj_dev, ids, rot_dev, inv_dev, img_sc, s_map)
        if (it + 1) % iter_arg.save_iter_step == 0:
            img_sc_iter[k, :] = img_sc.squeeze().detach().cpu()
            k += 1
            print(f"[SC] Iter: {it + 1}/{iter_arg.sc} | Time: {time.time() - t0:.2f}s")
    save_img_local_cntstat(img_sc, img_sc_iter, iter_arg, save_path)
