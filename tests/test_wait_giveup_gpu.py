"""Failure detection of the bounded device waits, exercised without any fault: with the poll
bound set to 0 (jscc_set_wait_limit) every pipeline wait of the bulk sparse kernels and of
the tensor-core GEMM gives up at once, while every copy and MMA that was issued still
completes normally. The kernels must return (each CTA that gave up first waits, with a bound
of its own, for what it has in flight), the give-ups must be counted, the host check must
raise RuntimeError, and with the default bound restored the next call must match the
reference computation again."""
from __future__ import annotations

import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL_W = 1e-5


def _sparse_problem(cuda):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid = synthetic.polar_grid(16, 96, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1)
    tb = cso.tables(p, cuda)
    g = torch.Generator().manual_seed(11)
    n_det, n = 400, 3000
    A = (torch.rand((n_det, grid.n_vox), generator=g) + 0.05).to(cuda).to(torch.bfloat16)
    tc = (torch.rand((n, p.coarse_pixel_num), generator=g) ** 3).to(cuda).to(torch.bfloat16)
    ids = torch.randint(0, n_det, (n,), generator=g, dtype=torch.int32).to(cuda)
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.2).to(cuda)
    return A, tb, tc, ids, x


def test_sparse_bulk_waits_give_up_and_recover(cuda):
    from jscc_recon_spect_cylinder_gb300 import _lib, ops

    A, tb, tc, ids, x = _sparse_problem(cuda)
    _lib.take_wait_timeout_count()
    ref = ops.sparse_weight_split(ids, tc, A, tb, x, method="event")
    good = ops.sparse_weight_split(ids, tc, A, tb, x)  # bulk pipeline, default bound
    torch.cuda.synchronize()
    assert _lib.take_wait_timeout_count() == 0
    assert rel_l2(good.cpu(), ref.cpu()) < TOL_W
    try:
        _lib.set_wait_limit(0)
        ops.sparse_weight_split(ids, tc, A, tb, x)
        torch.cuda.synchronize()  # the launches returned: nothing hangs
        assert _lib.take_wait_timeout_count() > 0
        ops.sparse_weight_split(ids, tc, A, tb, x)
        torch.cuda.synchronize()
        with pytest.raises(RuntimeError, match="gave up"):
            _lib.check_wait_timeouts()
    finally:
        _lib.set_wait_limit(None)
    again = ops.sparse_weight_split(ids, tc, A, tb, x)
    torch.cuda.synchronize()
    _lib.check_wait_timeouts()  # no give-up with the default bound
    assert torch.equal(again, good)


def test_gemm_waits_give_up_and_recover(cuda):
    from jscc_recon_spect_cylinder_gb300 import _lib, ops

    g = torch.Generator().manual_seed(5)
    P = (torch.rand((1000, 4096), generator=g) - 0.3).to(torch.bfloat16)
    R = (torch.rand((128, 4096), generator=g) * 2 - 0.5).to(torch.bfloat16)
    Pd, Rd = P.to(cuda), R.to(cuda)
    ref = P.double() @ R.double().T
    _lib.take_gemm_timeout_count()
    try:
        _lib.set_wait_limit(0)
        for splits in (1, 4):
            ops.bf16_gemm_nt(Pd, Rd, k_splits=splits)
            torch.cuda.synchronize()  # every CTA returned and freed its tensor memory
            assert _lib.take_gemm_timeout_count() > 0
        ops.bf16_gemm_nt(Pd, Rd)
        torch.cuda.synchronize()
        with pytest.raises(RuntimeError, match="tensor-core GEMM"):
            _lib.check_wait_timeouts()
    finally:
        _lib.set_wait_limit(None)
    for splits in (1, 4):
        out = ops.bf16_gemm_nt(Pd, Rd, k_splits=splits)
        torch.cuda.synchronize()
        _lib.check_wait_timeouts()
        assert rel_l2(out.cpu(), ref) < 1e-5
