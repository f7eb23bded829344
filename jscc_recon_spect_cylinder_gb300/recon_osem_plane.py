"""Drop-in for the reference module ``recon_osem_plane`` (dense SC + dense-T Compton OSEM).

Same public names, positional signatures, list nesting and return values as
recon_osem_plane.py; every projection runs in the sm_103a kernels of
``libjscc_gb300.so`` (ops.sc_weight / ops.em_update). Nested inputs keep the
reference layout:

* ``sysmat_list_all[subset][energy]``: subset rows of the SC matrix ``[B_s, V]``
* ``proj_list_all[subset][energy]``: ``[B_s, R]`` counts, column r = rotation r
* ``t_list_all[subset][rotation][divide][energy]``: dense Compton T blocks ``[E_blk, V]``
* ``rotmat_all[energy]`` / ``rotmat_inv_all[energy]``: ``[V, R]`` int64, 1-based

Accumulation order differs from the reference only where several energies are
interleaved with rotations (the kernels sum all rotations of one energy per call);
the result agrees to float32 rounding.
"""
from __future__ import annotations

import os
import time

import torch
import torch.multiprocessing as mp

from . import ops

__all__ = [
    "split_tensor_even",
    "get_t_budget_bytes_per_gpu",
    "get_weight_single",
    "get_weight_compton",
    "osem_bin_mode",
    "osem_list_mode",
    "osem_list_mode_mp",
    "osem_joint_mode",
    "save_img",
    "get_gpu_memory_usage",
    "run_recon_osem",
]


def split_tensor_even(tensor, parts, dim=0):
    """Floor-balanced contiguous split (recon_osem_plane.py:8-18): part k spans
    ``[n*k//parts, n*(k+1)//parts)``; parts may be empty."""
    if parts <= 0:
        raise ValueError("parts must be positive")
    n = tensor.size(dim)
    bounds = [n * k // parts for k in range(parts + 1)]
    return [tensor.narrow(dim, bounds[k], bounds[k + 1] - bounds[k]) for k in range(parts)]


def get_t_budget_bytes_per_gpu(num_gpus, usage_ratio=0.8):
    """Per-GPU byte budget for resident T blocks (recon_osem_plane.py:21-26)."""
    return [
        max(1, int(torch.cuda.get_device_properties(g).total_memory * usage_ratio))
        for g in range(num_gpus)
    ]


def _ones_col(n: int, device: torch.device) -> torch.Tensor:
    key = (device.index, n)
    t = _ONES.get(key)
    if t is None:
        t = torch.ones((n, 1), dtype=torch.float32, device=device)
        _ONES[key] = t
    return t


_ONES: dict = {}


def get_weight_single(sysmat_list_tmp, proj_list_tmp, img_tmp):
    """``A^T (y / (A x))`` for one subset block (recon_osem_plane.py:28-30)."""
    return ops.sc_weight(sysmat_list_tmp, proj_list_tmp, img_tmp)


def get_weight_compton(t_block, img):
    """``T^T (1 / (T x))`` for one dense Compton block (recon_osem_plane.py:33-42).

    A block held in (pinned) host memory is copied to the image's device first,
    as the reference does.
    """
    t_dev = t_block if t_block.device == img.device else t_block.to(img.device, non_blocking=True)
    return ops.sc_weight(t_dev, _ones_col(t_dev.size(0), img.device), img)


def _accumulate_sc(weight, sysmat_list, proj_list, rotmat_all, rotmat_inv_all, img, rotate_num,
                   floor=None, scale=1.0):
    for sysmat, proj, rotmat, rotmat_inv in zip(sysmat_list, proj_list, rotmat_all, rotmat_inv_all):
        if sysmat.numel() == 0:
            continue
        ops.sc_weight(sysmat, proj, img, rotmat, rotmat_inv, rot_start=0, n_rot=rotate_num,
                      floor=floor, scale=scale, out=weight)


def _accumulate_compton_dense(weight, t_list, rotmat_all, rotmat_inv_all, img, rotate_num):
    for i in range(rotate_num):
        for t in t_list[i]:
            for t_tmp, rotmat, rotmat_inv in zip(t, rotmat_all, rotmat_inv_all):
                if t_tmp.numel() == 0:
                    continue
                t_dev = t_tmp if t_tmp.device == img.device else t_tmp.to(img.device, non_blocking=True)
                ops.sc_weight(t_dev, _ones_col(t_dev.size(0), img.device), img, rotmat, rotmat_inv,
                              rot_start=i, n_rot=1, out=weight, proj_col=0)


def _apply_denoiser(img, model_denoiser):
    n = int(img.shape[0] ** 0.5)
    img = model_denoiser(img.view(1, 1, n, n)).view(n * n, 1)
    return torch.clamp(img, min=0)


def osem_bin_mode(sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, img, s_map, rotate_num,
                  model_denoiser=None):
    """SC OSEM over all subsets (recon_osem_plane.py:45-61): per subset
    ``img <- img * w / s`` with ``w`` summed over rotations and energies."""
    for sysmat_list, proj_list in zip(sysmat_list_all, proj_list_all):
        weight = torch.zeros_like(img)
        _accumulate_sc(weight, sysmat_list, proj_list, rotmat_all, rotmat_inv_all, img, rotate_num)
        img = ops.em_update(img, weight, s_map, safe=False)
        if model_denoiser is not None:
            img = _apply_denoiser(img, model_denoiser)
    return img


def osem_list_mode(t_list_all, rotmat_all, rotmat_inv_all, img, s_map, rotate_num, model_denoiser=None):
    """Dense-T list-mode OSEM (recon_osem_plane.py:63-80)."""
    for t_list in t_list_all:
        weight_compton = torch.zeros_like(img)
        _accumulate_compton_dense(weight_compton, t_list, rotmat_all, rotmat_inv_all, img, rotate_num)
        img = ops.em_update(img, weight_compton, s_map, safe=False)
        if model_denoiser is not None:
            img = _apply_denoiser(img, model_denoiser)
    return img


def osem_list_mode_mp(t_list_all, rotmat_all, rotmat_inv_all, iter_num, rank, img_queue, weight_queue,
                      rotate_num, model_denoiser=None):
    """Queue worker of the multi-process list mode (recon_osem_plane.py:82-98).

    For every subset it takes the current image from ``img_queue``, computes the
    Compton weight of its T blocks on ``cuda:rank`` and puts it (on cuda:0) into
    ``weight_queue``.
    """
    del model_denoiser
    with torch.no_grad():
        dev = torch.device(f"cuda:{rank}")
        for _ in range(iter_num):
            for t_list in t_list_all:
                img = img_queue.get().to(dev)
                weight = torch.zeros_like(img)
                rot_dev = [r.to(dev) for r in rotmat_all]
                inv_dev = [r.to(dev) for r in rotmat_inv_all]
                _accumulate_compton_dense(weight, t_list, rot_dev, inv_dev, img, rotate_num)
                weight_queue.put(weight.to("cuda:0"))


def osem_joint_mode(sysmat_list_all, proj_list_all, t_list_all, rotmat_all, rotmat_inv_all, img, s_map,
                    alpha, rotate_num, model_denoiser=None):
    """Joint SC + Compton OSEM (recon_osem_plane.py:100-125):
    ``w = (2 - alpha) w_c + alpha w_s``, ``img <- img * w / s``."""
    for sysmat_list, proj_list, t_list in zip(sysmat_list_all, proj_list_all, t_list_all):
        weight_compton = torch.zeros_like(img)
        weight_single = torch.zeros_like(img)
        _accumulate_sc(weight_single, sysmat_list, proj_list, rotmat_all, rotmat_inv_all, img, rotate_num)
        _accumulate_compton_dense(weight_compton, t_list, rotmat_all, rotmat_inv_all, img, rotate_num)
        img = ops.em_update(img, weight_compton, s_map, safe=False, coef=2 - alpha,
                            weight_b=weight_single, coef_b=alpha)
        if model_denoiser is not None:
            img = _apply_denoiser(img, model_denoiser)
    return img


def _write_f32(path, tensor):
    with open(path, "wb") as fh:
        tensor.detach().cpu().numpy().astype("float32").tofile(fh)


def save_img(img_sc, img_scd, img_jsccd, img_jsccsd, img_sc_iter, img_scd_iter, img_jsccd_iter,
             img_jsccsd_iter, iter_arg, save_path):
    """Raw float32 image files in the reference's names (recon_osem_plane.py:128-147)."""
    _write_f32(save_path + "Image_SC", img_sc)
    _write_f32(save_path + "Image_SCD", img_scd)
    _write_f32(save_path + "Image_JSCCD", img_jsccd)
    _write_f32(save_path + "Image_JSCCSD", img_jsccsd)
    step = iter_arg.save_iter_step
    _write_f32(save_path + "Image_SC_Iter_%d_%d" % (iter_arg.sc, iter_arg.sc / step), img_sc_iter)
    _write_f32(save_path + "Image_SCD_Iter_%d_%d" % (iter_arg.jsccd, iter_arg.jsccd / step), img_scd_iter)
    _write_f32(save_path + "Image_JSCCD_Iter_%d_%d" % (iter_arg.jsccd, iter_arg.jsccd / step), img_jsccd_iter)
    _write_f32(save_path + "Image_JSCCSD_Iter_%d_%d" % (iter_arg.jsccsd, iter_arg.jsccsd / step),
               img_jsccsd_iter)


def get_gpu_memory_usage(num_gpus):
    """Print allocated/reserved GiB per GPU (recon_osem_plane.py:150-158)."""
    for i in range(num_gpus):
        print(f"cuda:{i}")
        print(f"allocated_GB:{round(torch.cuda.memory_allocated(i) / 1024 ** 3, 2)}")
        print(f"reserved_GB:{round(torch.cuda.memory_reserved(i) / 1024 ** 3, 2)}")


def _stage_t_blocks(t_all, rotate_num, iter_arg, num_gpus):
    """Split T per rotation into subsets and divides (split_tensor_even at each
    level) and place blocks on the GPU until 80% of its memory is used, the rest in
    pinned host memory (recon_osem_plane.py:195-238)."""
    S, D, E = iter_arg.osem_subset_num, iter_arg.t_divide_num, iter_arg.ene_num

    def empty_tree():
        return [[[[[] for _ in range(E)] for _ in range(D)] for _ in range(rotate_num)] for _ in range(S)]

    trees = [empty_tree() for _ in range(num_gpus)]
    budget = get_t_budget_bytes_per_gpu(num_gpus)
    used = [0] * num_gpus
    for e, t in enumerate(t_all):
        for i in range(rotate_num):
            per_gpu = [t[i]] if num_gpus == 1 else split_tensor_even(t[i], num_gpus, dim=0)
            for g, t_gpu in enumerate(per_gpu):
                for j, t_sub in enumerate(split_tensor_even(t_gpu, S, dim=0)):
                    for k, chunk in enumerate(split_tensor_even(t_sub, D, dim=0)):
                        nbytes = chunk.nelement() * chunk.element_size()
                        if used[g] + nbytes < budget[g]:
                            trees[g][j][i][k][e] = chunk.to(f"cuda:{g}", non_blocking=True)
                            used[g] += nbytes
                        else:
                            trees[g][j][i][k][e] = chunk.pin_memory()
    print("T staged; share of the per-GPU T budget used (%):",
          [round(100 * used[g] / budget[g], 2) for g in range(num_gpus)])
    return trees[0] if num_gpus == 1 else trees


def run_recon_osem(sysmat_all, rotmat_all, rotmat_inv_all, proj_all, proj_d_all, t_all, iter_arg, s_map_arg,
                   alpha, save_path, num_gpus, model_denoiser=None):
    """Full SC -> SC-D -> JSCC-D -> JSCC-SD reconstruction (recon_osem_plane.py:161-403).

    One global ``torch.randperm`` of the bins, split floor-balanced into subsets,
    fixes the bin subsets for the whole run (recon_osem_plane.py:190-193); images
    are snapshotted every ``save_iter_step`` iterations and written by save_img.
    """
    os.makedirs(save_path, exist_ok=True)
    dev = torch.device("cuda:0")
    pixel_num = sysmat_all[0].size(1)
    rotate_num = rotmat_all[0].size(1)
    S = iter_arg.osem_subset_num

    def ones_img():
        return torch.ones([pixel_num, 1], dtype=torch.float32).to(dev, non_blocking=True)

    img_sc, img_scd, img_jsccd, img_jsccsd = ones_img(), ones_img(), ones_img(), ones_img()
    step = iter_arg.save_iter_step
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
    del sysmat_all, t_all

    s_map_arg.s = s_map_arg.s.to(dev, non_blocking=True)
    s_map_arg.d = s_map_arg.d.to(dev, non_blocking=True)
    s_map_arg.j = alpha * s_map_arg.s + (2 - alpha) * s_map_arg.d
    if model_denoiser is not None:
        model_denoiser.to(dev)

    get_gpu_memory_usage(num_gpus)
    t0 = time.time()

    def run_phase(name, n_iter, step_fn, img, snapshots):
        print(f"{name} OSEM starts")
        k = 0
        for it in range(n_iter):
            img = step_fn(img)
            if (it + 1) % step == 0:
                snapshots[k, :] = torch.squeeze(img).cpu()
                k += 1
                print(f"{name} iteration {it + 1} ends, time used: {time.time() - t0:.3f} s")
        print(f"{name} OSEM ends, time used: {time.time() - t0:.3f} s")
        return img

    img_sc = run_phase("SC", iter_arg.sc, lambda x: osem_bin_mode(
        sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, x, s_map_arg.s, rotate_num,
        model_denoiser), img_sc, img_sc_iter)
    img_scd = run_phase("SC-D", iter_arg.jsccd, lambda x: osem_bin_mode(
        sysmat_list_all, proj_d_list_all, rotmat_all, rotmat_inv_all, x, s_map_arg.s, rotate_num,
        model_denoiser), img_scd, img_scd_iter)

    if num_gpus == 1:
        img_jsccd = run_phase("JSCC-D", iter_arg.jsccd, lambda x: osem_list_mode(
            t_list_all, rotmat_all, rotmat_inv_all, x, s_map_arg.d, rotate_num, model_denoiser),
            img_jsccd, img_jsccd_iter)
        img_jsccsd = run_phase("JSCC-SD", iter_arg.jsccsd, lambda x: osem_joint_mode(
            sysmat_list_all, proj_list_all, t_list_all, rotmat_all, rotmat_inv_all, x, s_map_arg.j, alpha,
            rotate_num, model_denoiser), img_jsccsd, img_jsccsd_iter)
    else:
        img_jsccd, img_jsccsd = _run_multi_gpu_compton(
            t_list_all, sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, img_jsccd, img_jsccsd,
            s_map_arg, alpha, iter_arg, num_gpus, rotate_num, img_jsccd_iter, img_jsccsd_iter, model_denoiser)

    save_img(img_sc, img_scd, img_jsccd, img_jsccsd, img_sc_iter, img_scd_iter, img_jsccd_iter,
             img_jsccsd_iter, iter_arg, save_path)


WORKER_POLL_S = 1.0  # how often a wait for worker results checks that the workers are alive


def collect_worker_weights(weight_queue, procs, count, what):
    """``count`` weight images from ``weight_queue``, in arrival order. Instead of blocking
    forever on a worker that died (the reference's ``weight_queue.get()``), the wait checks
    the workers every WORKER_POLL_S seconds: a worker that exited with a non-zero code, or
    exited while results are still owed, stops every worker and raises RuntimeError, as the
    reference's entry points do for their T-builder workers (main_plane_sparse.py:194-203)."""
    import queue as _queue

    out = []
    while len(out) < count:
        try:
            out.append(weight_queue.get(timeout=WORKER_POLL_S))
            continue
        except _queue.Empty:
            pass
        dead = [(g, p.exitcode) for g, p in enumerate(procs) if p.exitcode is not None and p.exitcode != 0]
        if not dead and all(p.exitcode is not None for p in procs):
            dead = [(g, p.exitcode) for g, p in enumerate(procs)]
        if dead:
            stop_workers(procs)
            g, code = dead[0]
            raise RuntimeError(f"{what} worker {g} exited with code {code} while {count - len(out)} of {count} "
                               "weight images were still owed")
    return out


def stop_workers(procs, timeout=5.0):
    """Terminate and reap every worker that is still running."""
    for p in procs:
        if p.is_alive():
            p.terminate()
    for p in procs:
        p.join(timeout)


def join_workers(procs, what):
    """Join the workers and raise if any exited with a non-zero code."""
    for g, p in enumerate(procs):
        p.join()
        if p.exitcode != 0:
            stop_workers(procs)
            raise RuntimeError(f"{what} worker {g} exited with code {p.exitcode}")


def _run_multi_gpu_compton(t_list_all, sysmat_list_all, proj_list_all, rotmat_all, rotmat_inv_all, img_jsccd,
                           img_jsccsd, s_map_arg, alpha, iter_arg, num_gpus, rotate_num, img_jsccd_iter,
                           img_jsccsd_iter, model_denoiser):
    """Queue ping-pong of recon_osem_plane.py:320-400: one worker process per GPU
    returns its Compton weight per subset; cuda:0 sums them and updates."""
    img_queue, weight_queue = mp.Queue(), mp.Queue()
    step = iter_arg.save_iter_step

    def phase(n_iter, img, snapshots, joint):
        procs = [mp.Process(target=osem_list_mode_mp, args=(
            t_list_all[g], rotmat_all, rotmat_inv_all, n_iter, g, img_queue, weight_queue, rotate_num,
            model_denoiser)) for g in range(num_gpus)]
        for p in procs:
            p.start()
        k = 0
        for it in range(n_iter):
            for s in range(iter_arg.osem_subset_num):
                for _ in range(num_gpus):
                    img_queue.put(img)
                w_c = torch.zeros_like(img)
                for w in collect_worker_weights(weight_queue, procs, num_gpus, "list-mode OSEM"):
                    w_c = w_c + w
                if joint:
                    w_s = torch.zeros_like(img)
                    _accumulate_sc(w_s, sysmat_list_all[s], proj_list_all[s], rotmat_all, rotmat_inv_all,
                                   img, rotate_num)
                    img = ops.em_update(img, w_c, s_map_arg.j, safe=False, coef=2 - alpha, weight_b=w_s,
                                        coef_b=alpha)
                else:
                    img = ops.em_update(img, w_c, s_map_arg.d, safe=False)
            if (it + 1) % step == 0:
                snapshots[k, :] = torch.squeeze(img).cpu()
                k += 1
        join_workers(procs, "list-mode OSEM")
        return img

    img_jsccd = phase(iter_arg.jsccd, img_jsccd, img_jsccd_iter, joint=False)
    if getattr(iter_arg, "mode", 0) == 0:
        img_jsccsd = phase(iter_arg.jsccsd, img_jsccsd, img_jsccsd_iter, joint=True)
    return img_jsccd, img_jsccsd


# ============================================================================ fused dense Compton path
# T recomputed on the fly from compact event records (process_list_plane_strict.
# get_compton_event_params) instead of stored dense blocks; same weight as
# get_weight_compton over the builder's rows (the list-mode weight is invariant to the
# builder's row normalisation).

def get_weight_compton_fused(events, coor, sysmat, img, rotmat=None, rotmat_inv=None, rot_col=0, scale=1.0, out=None,
                             use_window=False):
    """``T^T (1 / (T x))`` for a block of ComptonEvents; accumulated into ``out``. Every
    event-voxel pair is evaluated, as the reference's stored rows hold them; ``use_window``
    skips pairs outside each record's cos(beta) window (t < exp(-K^2 / 2)), which pays only
    when the windows exclude most of the grid."""
    if len(events) == 0:
        return torch.zeros_like(img) if out is None else out
    return ops.compton_weight(events.records, events.row_id, coor, img, model=events.model, eff=sysmat,
                              use_window=use_window, rotmat=rotmat, rotmat_inv=rotmat_inv, rot_col=rot_col,
                              scale=scale, out=out)


def _accumulate_compton_fused(weight, ev_list, coor_all, sysmat_all, rotmat_all, rotmat_inv_all, img, rotate_num,
                              use_window):
    for i in range(rotate_num):
        for ev in ev_list[i]:
            for ev_tmp, coor, sysmat, rotmat, rotmat_inv in zip(ev, coor_all, sysmat_all, rotmat_all, rotmat_inv_all):
                if ev_tmp is None or len(ev_tmp) == 0:
                    continue
                get_weight_compton_fused(ev_tmp, coor, sysmat, img, rotmat, rotmat_inv, rot_col=i, out=weight,
                                         use_window=use_window)


def osem_list_mode_fused(ev_list_all, coor_all, sysmat_all, rotmat_all, rotmat_inv_all, img, s_map, rotate_num,
                         use_window=False):
    """osem_list_mode (recon_osem_plane.py:63-80) with T recomputed on the fly;
    ``ev_list_all[subset][rotation][divide][energy]`` holds ComptonEvents blocks."""
    for ev_list in ev_list_all:
        weight = torch.zeros_like(img)
        _accumulate_compton_fused(weight, ev_list, coor_all, sysmat_all, rotmat_all, rotmat_inv_all, img, rotate_num,
                                  use_window)
        img = ops.em_update(img, weight, s_map, safe=False)
    return img


def osem_joint_mode_fused(sysmat_list_all, proj_list_all, ev_list_all, coor_all, sysmat_all, rotmat_all,
                          rotmat_inv_all, img, s_map, alpha, rotate_num, use_window=False):
    """osem_joint_mode (recon_osem_plane.py:100-125) with the Compton half on the fly."""
    for sysmat_list, proj_list, ev_list in zip(sysmat_list_all, proj_list_all, ev_list_all):
        w_c = torch.zeros_like(img)
        w_s = torch.zeros_like(img)
        _accumulate_sc(w_s, sysmat_list, proj_list, rotmat_all, rotmat_inv_all, img, rotate_num)
        _accumulate_compton_fused(w_c, ev_list, coor_all, sysmat_all, rotmat_all, rotmat_inv_all, img, rotate_num,
                                  use_window)
        img = ops.em_update(img, w_c, s_map, safe=False, coef=2 - alpha, weight_b=w_s, coef_b=alpha)
    return img
