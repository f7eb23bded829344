"""The fused cluster form of the grouped sparse Compton weight (one kernel on clusters of four
CTAs that split the polar rings; each event row and group sysmat row read once, the per-group
coarse sums kept on chip) against the two-kernel pipeline and the per-event kernel, for both
semantics (materialise, recon_osem_local_sparse_jsccsd_only.py:13-19, and grouped,
recon_osem_plane_sparse.py:22-57): 1e-5 relative L2, repeated calls bit-identical, no device
wait giving up. Cases: the joint configuration's grid (100 x 360 fine, 9,000 coarse), fewer
groups than clusters, a group larger than the kernel's row slots, ring counts that do not
divide by four, rotated views; and the give-up path of its bounded waits."""
from __future__ import annotations

import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL_W = 1e-5


@pytest.fixture
def fused(cuda):
    """The fused cluster kernel switched on for the test (it is opt-in), off again after."""
    from jscc_recon_spect_cylinder_gb300 import _lib

    _lib.set_fused_cluster(True)
    yield
    _lib.set_fused_cluster(False)


def _problem(cuda, n_r, n_theta, n_det, n_events, seed, big_group=0):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid = synthetic.polar_grid(n_r, n_theta, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1)
    tb = cso.tables(p, cuda)
    assert tb.ring_stride == 4  # the stride-4 ring stencil with linear weights
    g = torch.Generator().manual_seed(seed)
    A = (torch.rand((n_det, grid.n_vox), generator=g) + 0.05).to(torch.bfloat16).to(cuda)
    tc = (torch.rand((n_events, p.coarse_pixel_num), generator=g) ** 3).to(torch.bfloat16).to(cuda)
    ids = torch.randint(0, n_det, (n_events,), generator=g, dtype=torch.int32)
    if big_group:
        ids[:big_group] = 0  # one group with big_group events
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.2).to(cuda)
    return A, tb, tc, ids.to(cuda), x, grid


@pytest.mark.parametrize("n_r,n_theta,n_det,n_events,big", [
    (100, 360, 2000, 6000, 0),    # the joint configuration's grids
    (16, 96, 3, 500, 0),          # fewer groups than clusters
    (16, 96, 300, 2000, 77),      # one group of 77 events (> the 16 row slots)
    (13, 64, 200, 1500, 0),       # 13 rings: slices of 3 and 4 rings, coarse windows past the slices
])
def test_fused_cluster_matches_two_kernel_and_event(cuda, fused, n_r, n_theta, n_det, n_events, big):
    from jscc_recon_spect_cylinder_gb300 import _lib, ops

    A, tb, tc, ids, x, _ = _problem(cuda, n_r, n_theta, n_det, n_events, n_r + n_det, big)
    _lib.take_wait_timeout_count()
    for grouped in (False, True):
        ref = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped, method="event")
        try:
            _lib.set_fused_cluster(False)
            two = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped)
        finally:
            _lib.set_fused_cluster(True)
        fused = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped)
        again = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped)
        torch.cuda.synchronize()
        assert rel_l2(fused.cpu(), ref.cpu()) < TOL_W, grouped
        assert rel_l2(fused.cpu(), two.cpu()) < TOL_W, grouped
        assert torch.equal(fused, again)
    _lib.check_wait_timeouts()


def test_fused_cluster_rotated_views(cuda, fused):
    """Rotation tables (gather the image through rotmat, scatter the weight through
    rotmat_inv) around the fused kernel, as the joint loops call it per view."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, synthetic

    A, tb, tc, ids, x, grid = _problem(cuda, 16, 96, 300, 2000, 5)
    rot, inv = synthetic.cyclic_rotation_tables(16, 96, 4)
    rot, inv = rot.to(cuda), inv.to(cuda)
    for col in range(4):
        ref = ops.sparse_weight_split(ids, tc, A, tb, x, rotmat=rot, rotmat_inv=inv, rot_col=col, method="event")
        fused = ops.sparse_weight_split(ids, tc, A, tb, x, rotmat=rot, rotmat_inv=inv, rot_col=col)
        torch.cuda.synchronize()
        assert rel_l2(fused.cpu(), ref.cpu()) < TOL_W, col
    _lib.check_wait_timeouts()


def test_fused_cluster_waits_give_up_and_recover(cuda, fused):
    """With the poll bound at 0 every wait of the fused kernel gives up at once (the bulk
    copies still complete; the peers give up on their exchanges): the launch returns, the
    give-up is counted and reported, and with the default bound the result is exact again."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops

    A, tb, tc, ids, x, _ = _problem(cuda, 100, 360, 2000, 6000, 9)
    good = ops.sparse_weight_split(ids, tc, A, tb, x)
    torch.cuda.synchronize()
    _lib.check_wait_timeouts()
    try:
        _lib.set_wait_limit(0)
        ops.sparse_weight_split(ids, tc, A, tb, x)
        torch.cuda.synchronize()
        with pytest.raises(RuntimeError, match="gave up"):
            _lib.check_wait_timeouts()
    finally:
        _lib.set_wait_limit(None)
    again = ops.sparse_weight_split(ids, tc, A, tb, x)
    torch.cuda.synchronize()
    _lib.check_wait_timeouts()
    assert torch.equal(again, good)
