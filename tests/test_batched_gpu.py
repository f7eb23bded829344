"""Batched (multi-instance) SC path on the tensor cores: the tcgen05 BF16 GEMM against an
FP64 product of the same BF16 operands (every product of two BF16 values is exact in FP32,
so only the FP32 accumulation order differs: 1e-5 relative)."""
from __future__ import annotations

import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,nr,K,splits", [(300, 128, 200, 1), (128, 64, 64, 1), (257, 100, 1032, 3), (40, 20, 8, 1),
                                           (1000, 256, 4096, 4), (129, 32, 0, 1)])
def test_bf16_gemm_matches_fp64(cuda, M, nr, K, splits):
    from jscc_recon_spect_cylinder_gb300 import _lib, ops

    g = torch.Generator().manual_seed(M + nr + K)
    P = (torch.rand((M, K), generator=g) - 0.3).to(torch.bfloat16)
    R = (torch.rand((nr, K), generator=g) * 2 - 0.5).to(torch.bfloat16)
    out = ops.bf16_gemm_nt(P.to(cuda), R.to(cuda), k_splits=splits)
    torch.cuda.synchronize()
    assert _lib.take_gemm_timeout_count() == 0
    ref = P.double() @ R.double().T
    if K == 0:
        assert torch.count_nonzero(out.cpu()) == 0
    else:
        assert rel_l2(out.cpu(), ref) < 1e-5


def test_bf16_gemm_strided_operands(cuda):
    """Row strides larger than K (a column slice of a wider matrix, as the back projection
    reads A^T restricted to a subset's bins)."""
    from jscc_recon_spect_cylinder_gb300 import ops

    g = torch.Generator().manual_seed(3)
    big = (torch.rand((200, 512), generator=g)).to(torch.bfloat16).to(cuda)
    P = big[:, 64:64 + 256]
    R = (torch.rand((48, 256), generator=g)).to(torch.bfloat16).to(cuda)
    out = ops.bf16_gemm_nt(P, R)
    ref = P.double().cpu() @ R.double().cpu().T
    assert rel_l2(out.cpu(), ref) < 1e-5


def _fp64_osem(A, y, x0, s, subsets, iters):
    """osem_bin_mode (one identity view) per instance in float64 (recon_osem_plane.py:45-61)."""
    X = x0.double().clone()
    for _ in range(iters):
        for ids in subsets:
            As = A[ids]
            F = X @ As.T                      # [N, bins_s]
            W = (y[:, ids] / F) @ As          # [N, V]
            X = X * W / s
    return X


@pytest.mark.parametrize("graph", [False, True])
def test_batched_osem_matches_fp64(cuda, graph):
    """Five instances (different count levels of one geometry), three subsets of 85-86 bins
    (padded to multiples of 8), three iterations: every instance within 1e-4 relative L2 of
    the float64 OSEM on the same BF16 matrix (the instance vectors carry ~16 bits)."""
    from jscc_recon_spect_cylinder_gb300 import _lib, batched, synthetic
    from jscc_recon_spect_cylinder_gb300.recon_osem_plane import split_tensor_even

    prob = synthetic.sc_problem(n_r=8, n_theta=24, n_phi=64, views=4, flat=True, total_counts=1e5)
    A = prob.sysmat.to(torch.bfloat16)
    B, V = A.shape
    g = torch.Generator().manual_seed(5)
    mean = A.float() @ prob.phantom.reshape(-1)
    y = torch.stack([torch.poisson(mean * (c / mean.sum()), generator=g) for c in (1e4, 3e4, 1e5, 3e5, 1e6)])
    subsets = split_tensor_even(torch.randperm(B, generator=g), 3)
    s = A.double().sum(0)
    x0 = torch.ones((5, V))
    b = batched.BatchedScOsem(A, subsets, s.float(), 5, device=cuda)
    b.set_projections(y)
    b.set_images(x0)
    b.autotune()
    if graph:
        b.capture()
    X = b.iterate(3).cpu()
    torch.cuda.synchronize()
    assert _lib.take_gemm_timeout_count() == 0
    ref = _fp64_osem(A.double(), y.double(), x0, s, subsets, 3)
    for n in range(5):
        assert rel_l2(X[n], ref[n]) < 1e-4, n


def _cone_events(cuda, A, coor, n_ev, seed):
    import numpy as np

    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import synthetic

    scat = synthetic.cylinder_pixels(120.0, 32, 4, 3.0)
    absb = synthetic.cylinder_pixels(150.0, 32, 4, 3.0)
    det = torch.cat((scat, absb)).float().to(cuda)
    e0 = 0.511
    args = (0.8, 0.8, e0, 0.1 * (0.662 / e0) ** 0.5, 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001, 0.05, e0 - 0.06)
    rng = np.random.default_rng(seed)
    L = np.stack((rng.integers(1, 129, n_ev), rng.uniform(0.08, 0.3, n_ev), rng.integers(129, 257, n_ev),
                  np.zeros(n_ev)), axis=1).astype(np.float32)
    L[:, 3] = e0 - L[:, 1]
    return pls.get_compton_event_params(A.float(), det, coor, torch.from_numpy(L).to(cuda), *args, window_sigmas=0.0)


@pytest.mark.parametrize("ev_per_chunk", [None, 64])
def test_compton_batch_matches_per_instance_weights(cuda, ev_per_chunk):
    """ops.ComptonBatch (jscc_compton_weight_batched: one forward and one back launch for all
    instances, device segment tables) against jscc_compton_weight run instance by instance,
    with uneven instances: none, one event, counts that are not multiples of 16, several back
    chunks per instance; BF16 and FP32 efficiency rows; 1e-5, repeated calls bit-identical."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, synthetic

    prob = synthetic.sc_problem(n_r=8, n_theta=24, n_phi=64, views=4, flat=True, total_counts=1e5)
    coor = prob.grid.coor.to(cuda)
    V = coor.size(0)
    evs = [(torch.zeros((0, 16), device=cuda), torch.zeros(0, dtype=torch.int32, device=cuda))]
    for n in (1, 37, 700, 2000):
        e = _cone_events(cuda, prob.sysmat.to(cuda), coor, n, 7 + n)
        evs.append((e.records, e.row_id))
    g = torch.Generator().manual_seed(3)
    X = (torch.rand((len(evs), V), generator=g) + 0.2).to(cuda)
    _lib.take_bad_detector_count()
    for A in (prob.sysmat.to(cuda), prob.sysmat.to(torch.bfloat16).to(cuda)):
        cb = ops.ComptonBatch(evs, V, cuda, ev_per_chunk=ev_per_chunk)
        assert cb.n_ev % 16 == 0 and cb.n_chunks >= len([r for r, _ in evs if r.size(0)])
        W = cb.weight(X, A, coor, scale=1.5)
        W2 = cb.weight(X, A, coor, scale=1.5)
        torch.cuda.synchronize()
        assert torch.equal(W, W2)
        for b, (rec, rid) in enumerate(evs):
            if rec.size(0) == 0:
                assert torch.count_nonzero(W[b]) == 0
                continue
            ref = ops.compton_weight(rec, rid, coor, X[b], eff=A, scale=1.5)
            assert rel_l2(W[b].cpu(), ref.cpu()) < 1e-5, b
    assert _lib.take_bad_detector_count() == 0


@pytest.mark.parametrize("graph", [False, True])
def test_batched_joint_matches_single_instance_loops(cuda, graph):
    """BatchedJointOsem (SC weights from the tensor-core GEMMs, the Compton weights of all
    instances from one batched cone launch per direction, safe EM with per-instance joint
    sensitivities; eager and captured in one CUDA graph) against the single-instance joint loop
    of each instance (jscc_sc_weight with the 1e-12 floor + jscc_compton_weight + safe EM) on
    the same BF16 matrix: 1e-4."""
    import numpy as np

    from jscc_recon_spect_cylinder_gb300 import batched, ops, synthetic
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300.recon_osem_plane import split_tensor_even

    prob = synthetic.sc_problem(n_r=8, n_theta=24, n_phi=64, views=4, flat=True, total_counts=1e5)
    A16 = prob.sysmat.to(torch.bfloat16).to(cuda)
    B, V = A16.shape
    coor = prob.grid.coor.to(cuda)
    scat = synthetic.cylinder_pixels(120.0, 32, 4, 3.0)
    absb = synthetic.cylinder_pixels(150.0, 32, 4, 3.0)
    det = torch.cat((scat, absb)).float().to(cuda)  # 256 detectors: scatter rows index A's 256 rows
    e0, S, alpha, n_inst = 0.511, 2, 0.5, 3
    args = (0.8, 0.8, e0, 0.1 * (0.662 / e0) ** 0.5, 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001, 0.05, e0 - 0.06)
    g = torch.Generator().manual_seed(31)
    subsets = split_tensor_even(torch.randperm(B, generator=g), S)
    mean = A16.float().cpu() @ prob.phantom.reshape(-1)
    Y = torch.stack([torch.poisson(mean * (c / mean.sum()), generator=g) for c in (3e4, 1e5, 3e5)])
    s_sc = A16.double().sum(0).float()
    events, S_joint = [], []
    for n in range(n_inst):
        rng = np.random.default_rng(100 + n)
        m = 400 * (n + 1)
        L = np.stack((rng.integers(1, 129, m), rng.uniform(0.08, 0.3, m), rng.integers(129, 257, m),
                      np.zeros(m)), axis=1).astype(np.float32)
        L[:, 3] = e0 - L[:, 1]
        ev = pls.get_compton_event_params(A16.float(), det, coor, torch.from_numpy(L).to(cuda), *args,
                                          window_sigmas=0.0)
        d = ops.compton_backproject(ev.records, ev.row_id, coor, torch.ones(len(ev), device=cuda), model=ev.model,
                                    eff=A16).reshape(-1)
        S_joint.append(alpha * s_sc.to(cuda) + (2 - alpha) * d)
        events.append(ev.split(S))
    S_joint = torch.stack(S_joint)
    bj = batched.BatchedJointOsem(A16, subsets, S_joint, events, coor, alpha=alpha, device=cuda)
    assert bj.cbatch is not None  # strict events: the batched cone launches
    bj.set_projections(Y)
    bj.set_images(torch.ones((n_inst, V)))
    if graph:
        bj.capture()
        bj.set_images(torch.ones((n_inst, V)))
    X = bj.iterate(2).cpu()
    for n in range(n_inst):
        x = torch.ones((V, 1), device=cuda)
        y = Y[n].reshape(-1, 1).to(cuda)
        for _ in range(2):
            for k in range(S):
                w = torch.zeros((V, 1), device=cuda)
                ops.sc_weight(A16, y, x, floor=1e-12, scale=alpha, out=w, row_idx=subsets[k].to(cuda))
                ev = events[n][k]
                ops.compton_weight(ev.records, ev.row_id, coor, x, model=ev.model, eff=A16, scale=2 - alpha, out=w)
                x = ops.em_update(x, w, S_joint[n].reshape(-1, 1), safe=True)
        assert rel_l2(X[n], x.cpu().reshape(-1)) < 1e-4, n
