"""The fused single-read SC weight (sc_fused_kernel: forward projection, ratio and back-
projection in one read of the rows, column halves on a cluster of two CTAs) against the
float64 oracle of get_weight_single (recon_osem_plane.py:28-30, with the floor of
recon_osem_local_cntstat.py:6-8) and against the two-pass kernels on the same inputs (a
workspace without room for the fused partial images selects them), BF16 and float32 rows,
row subsets, fewer rows than clusters, a voxel count that is not a multiple of the vector
width (the two-pass kernels run), bit-identical repeats, and the give-up path of its
bounded waits."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _problem(cuda, n_det, V, dtype, seed):
    g = torch.Generator().manual_seed(seed)
    A = (torch.rand((n_det, V), generator=g) ** 2 + 0.01).to(dtype)
    y = torch.poisson(torch.rand((n_det, 1), generator=g) * 50 + 1, generator=g)
    x = torch.rand((V, 1), generator=g) + 0.3
    return A.to(cuda), y.to(cuda), x.to(cuda), A.float().numpy(), y.numpy(), x.numpy()


def _c_weight(A, y, x, row_idx, floor, scale, shrink):
    """jscc_sc_weight through the C-ABI with the recommended workspace less `shrink` bytes."""
    from jscc_recon_spect_cylinder_gb300 import _lib

    lib = _lib.load()
    n_bins = row_idx.numel() if row_idx is not None else A.size(0)
    V = A.size(1)
    nbytes = int(lib.jscc_sc_weight_workspace_bytes(n_bins, V, 1)) - shrink
    ws = torch.empty(nbytes, dtype=torch.uint8, device=A.device)
    w = torch.zeros((V, 1), device=A.device)
    code = _lib.DTYPE_BF16 if A.dtype == torch.bfloat16 else _lib.DTYPE_F32
    rc = lib.jscc_sc_weight(A.data_ptr(), code, A.stride(0), None if row_idx is None else row_idx.data_ptr(), n_bins,
                            V, y.data_ptr(), y.stride(0), 1, x.data_ptr(), None, None, 1,
                            1 if floor is not None else 0, ctypes.c_float(floor or 0.0), ctypes.c_float(scale),
                            w.data_ptr(), ws.data_ptr(), nbytes, _lib.stream_handle(A.device))
    _lib.check(rc, "jscc_sc_weight")
    return w


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float32])
@pytest.mark.parametrize("V,n_det,subset,floor", [
    (36000, 2000, 700, 1e-12),    # the joint configuration's image, a row subset
    (36000, 2000, 608, None),     # eight rows per cluster: BF16 batches of three, three, two
    (4800, 1500, None, None),     # config-1 image, every row, no floor
    (4800, 150, None, 1e-12),     # two rows per cluster: one two-row batch each
    (4800, 7, None, 1e-12),       # fewer rows than clusters
    (4804, 300, 150, None),       # not a multiple of the vector width: two-pass kernels
])
def test_fused_matches_oracle_and_two_pass(cuda, dtype, V, n_det, subset, floor):
    from oracle import osem_sc

    A, y, x, An, yn, xn = _problem(cuda, n_det, V, dtype, seed=V + n_det)
    ridx = None
    rows = np.arange(n_det)
    if subset is not None:
        perm = torch.randperm(n_det, generator=torch.Generator().manual_seed(3))[:subset]
        ridx = perm.to(torch.int64).to(cuda)
        rows = perm.numpy()
    want = osem_sc.get_weight_single(An[rows], yn[rows], xn, floor=floor) * 0.5
    fused = _c_weight(A, y, x, ridx, floor, 0.5, shrink=0)
    again = _c_weight(A, y, x, ridx, floor, 0.5, shrink=0)
    two_pass = _c_weight(A, y, x, ridx, floor, 0.5, shrink=4096)
    torch.cuda.synchronize()
    assert torch.equal(fused, again), "repeated fused calls must be bit-identical"
    assert rel_l2(fused.cpu().numpy(), want) < TOL
    assert rel_l2(two_pass.cpu().numpy(), want) < TOL
    assert rel_l2(fused.cpu(), two_pass.cpu()) < TOL


def test_fused_waits_give_up_and_recover(cuda):
    from jscc_recon_spect_cylinder_gb300 import _lib

    A, y, x, *_ = _problem(cuda, 3000, 36000, torch.bfloat16, seed=17)
    _lib.take_wait_timeout_count()
    good = _c_weight(A, y, x, None, 1e-12, 1.0, shrink=0)
    torch.cuda.synchronize()
    assert _lib.take_wait_timeout_count() == 0
    try:
        _lib.set_wait_limit(0)
        _c_weight(A, y, x, None, 1e-12, 1.0, shrink=0)
        torch.cuda.synchronize()  # every cluster returned: nothing hangs
        with pytest.raises(RuntimeError, match="gave up"):
            _lib.check_wait_timeouts()
    finally:
        _lib.set_wait_limit(None)
    again = _c_weight(A, y, x, None, 1e-12, 1.0, shrink=0)
    torch.cuda.synchronize()
    _lib.check_wait_timeouts()
    assert torch.equal(again, good)
