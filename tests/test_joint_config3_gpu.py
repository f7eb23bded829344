"""One joint subset update at the joint configuration's grid sizes (100 x 360 fine voxels,
theta-stride-4 coarse grid of 9,000 voxels, 4,096-pixel SC views) with a reduced event count,
against the oracle's float64 restatement of osem_joint_mode_local_sparse
(recon_osem_local_sparse_jsccsd_only.py:58-100): w = alpha get_weight_single (forward floored
at 1e-12) + (2 - alpha) get_weight_compton_sparse (materialise form), then safe_em_update.

* float32 storage: the product's image within 1e-5 relative L2 of the oracle's on the same
  float32 inputs;
* BF16 storage (SC matrix and coarse rows): within 1e-5 of the oracle on the same
  BF16-rounded inputs (the kernels' own arithmetic), and within the 1e-3 BF16 storage tolerance of the
  oracle on the float32 inputs (the storage error itself)."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _oracle_update(A_s, y_s, eff, rows, U, x, s, alpha):
    from oracle import osem_sc
    from oracle import sparse as osp

    w = alpha * osem_sc.get_weight_single(A_s, y_s, x, floor=1e-12)
    w = w + (2 - alpha) * osp.weight_materialize_csr(rows, eff, x, U)
    return osem_sc.safe_em_update(x, w, s)


def test_joint_subset_update_at_config3_sizes(cuda):
    from jscc_recon_spect_cylinder_gb300 import workloads

    w = workloads.JointWorkload(cuda, views=2, n_events=30000, subsets=8)
    assert (w.V, w.Vc) == (36000, 9000)
    s = 0
    ids = w.subset_ids[s]
    rows = w.rows_f32[s]
    assert rows.size(0) > 1000
    ptr, idx, val = (t.cpu().numpy() for t in w.tables.up[1])
    U = sp.csr_matrix((val.astype(np.float64), idx, ptr), shape=(w.tables.n_lf, w.tables.n_lc))
    x0 = np.ones((w.V, 1))
    s_np = w.s_joint.cpu().numpy()
    y_s = w.proj[ids].cpu().numpy()
    rows_np = rows.cpu().numpy()
    cp1 = np.clip(np.round(rows_np[:, 0]).astype(np.int64) - 1, 0, w.B - 1)
    # efficiency rows of the subset's events only (remapped), so the oracle does not copy A
    uniq, inv = np.unique(cp1, return_inverse=True)
    rows_local = rows_np.copy()
    rows_local[:, 0] = inv + 1

    def inputs(dtype):
        A = w.A[dtype]
        A_s = A[ids].float().cpu().numpy()
        eff = A[torch.from_numpy(uniq).to(cuda)].float().cpu().numpy()
        r = rows_local.copy()
        if dtype == "bf16":
            r[:, 1:] = torch.from_numpy(r[:, 1:]).to(torch.bfloat16).float().numpy()
        return A_s, eff, r

    A_s, eff, r32 = inputs("f32")
    ref32 = _oracle_update(A_s, y_s, eff, r32, U, x0, s_np, w.alpha)
    got32 = w.subset_update(torch.ones((w.V, 1), device=cuda), s, "f32").cpu().numpy()
    assert rel_l2(got32, ref32) < 1e-5

    A_s, eff, r16 = inputs("bf16")
    ref16 = _oracle_update(A_s, y_s, eff, r16, U, x0, s_np, w.alpha)
    got16 = w.subset_update(torch.ones((w.V, 1), device=cuda), s, "bf16").cpu().numpy()
    assert rel_l2(got16, ref16) < 1e-5
    assert rel_l2(got16, ref32) < 1e-3
