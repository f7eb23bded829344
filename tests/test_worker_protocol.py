"""Multi-GPU list-mode phase of the runners (recon_osem_plane.py:320-400 and
recon_osem_plane_sparse.py:286-348 in the reference): one worker process per GPU takes the
image from img_queue and returns its Compton weight on weight_queue, once per subset. The
reference blocks on weight_queue.get() forever when a worker dies; here the wait checks the
workers and raises, as the reference's entry points do for their T-builder workers
(main_plane_sparse.py:194-203). Fake workers on the CPU: no GPU is involved."""
from __future__ import annotations

import os
import time
from types import SimpleNamespace

import pytest
import torch
import torch.multiprocessing as mp

V = 16


def _worker_dies(t_list_all, rotmat_all, rotmat_inv_all, iter_num, rank, img_queue, weight_queue, rotate_num,
                 model_denoiser=None):
    """Rank 1 fails at once (as a worker whose CUDA context broke would); rank 0 keeps
    waiting for an image that its peer's failure means it would never get to finish."""
    if rank == 1:
        os._exit(3)
    time.sleep(120)


def _worker_returns_early(t_list_all, rotmat_all, rotmat_inv_all, iter_num, rank, img_queue, weight_queue,
                          rotate_num, model_denoiser=None):
    """Every rank exits cleanly without producing any weight."""
    return


def _worker_ok(n, weight_queue, release):
    for _ in range(n):
        weight_queue.put(torch.ones((V, 1)))
    release.wait(60)  # a tensor's shared memory is handed over while its producer is alive


def _call_dense_phase(rop, num_gpus):
    iter_arg = SimpleNamespace(jsccd=2, jsccsd=2, osem_subset_num=2, save_iter_step=1, mode=0)
    s_map = SimpleNamespace(s=torch.ones((V, 1)), d=torch.ones((V, 1)), j=torch.ones((V, 1)))
    img = torch.ones((V, 1))
    snaps = torch.ones((2, V))
    t_lists = [[[[[torch.zeros((0, V))]]] for _ in range(2)] for _ in range(num_gpus)]
    rot = [torch.arange(1, V + 1).unsqueeze(1)]
    return rop._run_multi_gpu_compton(t_lists, [[None]] * 2, [[None]] * 2, rot, rot, img.clone(), img.clone(),
                                      s_map, 0.5, iter_arg, num_gpus, 1, snaps, snaps.clone(), None)


@pytest.mark.parametrize("fake", [_worker_dies, _worker_returns_early])
def test_dead_worker_raises_instead_of_blocking(monkeypatch, fake):
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    monkeypatch.setattr(rop, "osem_list_mode_mp", fake)
    monkeypatch.setattr(rop, "WORKER_POLL_S", 0.2)
    t0 = time.time()
    with pytest.raises(RuntimeError, match="list-mode OSEM worker"):
        _call_dense_phase(rop, 2)
    assert time.time() - t0 < 30  # detected within a few polls; the sleeping peer was stopped


def test_sparse_phase_dead_worker_raises(monkeypatch):
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane_sparse as rsp

    monkeypatch.setattr(rop, "WORKER_POLL_S", 0.2)
    q = mp.Queue()
    procs = [mp.Process(target=os._exit, args=(5,)), mp.Process(target=time.sleep, args=(120,))]
    for p in procs:
        p.start()
    with pytest.raises(RuntimeError, match="exited with code 5"):
        rsp.collect_worker_weights(q, procs, 2, "sparse list-mode OSEM")
    assert all(not p.is_alive() for p in procs)


def test_collect_worker_weights_happy_path():
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    q = mp.Queue()
    release = mp.Event()
    procs = [mp.Process(target=_worker_ok, args=(2, q, release)) for _ in range(2)]
    for p in procs:
        p.start()
    got = rop.collect_worker_weights(q, procs, 4, "list-mode OSEM")
    release.set()
    rop.join_workers(procs, "list-mode OSEM")
    assert len(got) == 4 and all(torch.equal(w, torch.ones((V, 1))) for w in got)


def test_join_workers_reports_failure():
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    procs = [mp.Process(target=os._exit, args=(0,)), mp.Process(target=os._exit, args=(7,))]
    for p in procs:
        p.start()
    with pytest.raises(RuntimeError, match="worker 1 exited with code 7"):
        rop.join_workers(procs, "list-mode OSEM")
