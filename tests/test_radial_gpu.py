"""The radially coarsened projector through the GPU path (the same operators, T builder and
weight kernels as the reference's projector; an extension with no reference behaviour, so
the oracle is its numpy restatement, oracle.sparse.build_radial_projector, itself pinned in
tests/test_radial_projector.py): on the golden sparse problem's grid (4 planes of 6 rings x
24 theta) coarsened by 2 radially and 4 in theta, the sparse T builder's rows, the four
separable operators and both weight semantics against the FP64 oracle; on a 16-ring x
96-theta grid coarsened 4 x 4, the bulk split-row path (BF16 and float32 rows) against the
oracle and against the per-event kernel; and the bulk kernels on coarse grids that are not
16-byte multiples (padded rows, shifted q segments)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import sparse as osp

pytestmark = pytest.mark.gpu

TOL_ROW = 1e-4
TOL_W = 1e-5


def test_radial_builder_operators_and_weights(cuda, golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_sparse as psp
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_sparse_jsccsd_only as loc
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane_sparse as rsp

    g = golden("sparse_ops")
    o = osp.build_radial_projector(g["s_coor"], 2, 4)
    p = cso.build_compton_sparse_projector_radial(torch.from_numpy(g["s_coor"]), 2, 4).to(cuda)
    assert p.coarse_pixel_num == 4 * 3 * 6
    A = torch.from_numpy(g["s_sysmat"]).to(cuda)
    a = [float(v) for v in g["s_args"]]
    rows = psp.build_sparse_rows_from_smeared(A, torch.from_numpy(g["s_det"]).to(cuda), p,
                                              torch.from_numpy(g["s_smeared"]).to(cuda), *a)
    ref, _ = osp.sparse_builder(g["s_sysmat"], g["s_det"], o, g["s_smeared"], *a, dtype=np.float64)
    assert rows.shape == ref.shape and rows.shape[0] > 0
    np.testing.assert_array_equal(rows[:, 0].cpu().numpy(), ref[:, 0])
    got = rows[:, 1:].cpu().double().numpy()
    assert np.abs(got - ref[:, 1:]).max() <= TOL_ROW * max(np.abs(ref[:, 1:]).max(), 1e-30)
    # operators
    rc = torch.from_numpy(ref[:, 1:].astype(np.float32)).to(cuda)
    rf = torch.rand((5, p.fine_pixel_num), generator=torch.Generator().manual_seed(2)).to(cuda)
    assert rel_l2(cso.upsample_coarse_rows_to_fine(rc, p).cpu(), osp.upsample_rows(ref[:, 1:], o)) < 1e-6
    assert rel_l2(cso.project_fine_rows_to_coarse_adjoint(rf, p).cpu(), osp.adjoint_rows(rf.cpu().numpy(), o)) < 1e-6
    assert rel_l2(cso.reduce_fine_rows_to_coarse(rf, p).cpu(), osp.reduce_rows(rf.cpu().numpy(), o)) < 1e-6
    # both weight semantics
    R = torch.from_numpy(ref.astype(np.float32)).to(cuda)
    x = torch.from_numpy(g["s_x"]).to(cuda)
    want_g = osp.weight_grouped(ref, g["s_sysmat"], g["s_x"], o)
    want_m = osp.weight_materialize(ref, g["s_sysmat"], g["s_x"], o)
    assert rel_l2(rsp.get_weight_compton_sparse(R, A, x, p).cpu(), want_g) < TOL_W
    assert rel_l2(loc.get_weight_compton_sparse(R, A, x, p).cpu(), want_m) < TOL_W


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float32])
def test_radial_bulk_split_rows(cuda, dtype):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid = synthetic.polar_grid(16, 96, 30.0)
    p = cso.build_compton_sparse_projector_radial(grid.coor, 4, 4)
    o = osp.build_radial_projector(grid.coor.numpy(), 4, 4)
    tb = cso.tables(p, cuda)
    gen = torch.Generator().manual_seed(23)
    n_det, n = 300, 2500
    A = (torch.rand((n_det, grid.n_vox), generator=gen) + 0.05).to(dtype)
    tc = (torch.rand((n, p.coarse_pixel_num), generator=gen) ** 3).to(dtype)
    ids = torch.randint(0, n_det, (n,), generator=gen, dtype=torch.int32)
    x = torch.rand((grid.n_vox, 1), generator=gen) + 0.2
    rows = np.concatenate(((ids.numpy() + 1).astype(np.float64)[:, None], tc.double().numpy()), axis=1)
    want = osp.weight_materialize_csr(rows, A.double().numpy(), x.numpy(), osp.upsample_matrix_csr(o))
    Ad, tcd, idd, xd = A.to(cuda), tc.to(cuda), ids.to(cuda), x.to(cuda)
    bulk = ops.sparse_weight_split(idd, tcd, Ad, tb, xd)
    event = ops.sparse_weight_split(idd, tcd, Ad, tb, xd, method="event")
    torch.cuda.synchronize()
    assert rel_l2(bulk.cpu(), want) < TOL_W
    assert rel_l2(event.cpu(), want) < TOL_W
    assert rel_l2(bulk.cpu(), event.cpu()) < TOL_W


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float32])
def test_bulk_paths_on_unaligned_coarse_grids(cuda, dtype):
    """Six planes of 3 rings x 360 theta coarsened 4 in theta and 2 in z: 810 coarse voxels
    (coarse rows that are not a whole number of 16-byte units: padded split storage, masked
    row tails in the coefficient kernel) and 270 coarse voxels per plane (q segments that start
    off a 16-byte boundary: copied from the boundary below in the bulk scatter, two z taps).
    The bulk kernels match the per-event kernel, both semantics, and no wait gives up."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, synthetic
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    plane = synthetic.polar_grid(3, 360, 30.0).coor
    coor = torch.cat([torch.cat((plane[:, :2], torch.full((plane.size(0), 1), 2.0 * k)), dim=1) for k in range(6)])
    p = cso.build_compton_sparse_projector(coor, 4, 2, rotate_num=1)
    tb = cso.tables(p, cuda)
    vc, n_lc = p.coarse_pixel_num, p.coarse_layer_num
    assert vc % 4 != 0 and n_lc % 4 != 0 and p.fine_layer_num >= 1024
    g = torch.Generator().manual_seed(31)
    n_det, n = 250, 2200
    V = p.fine_pixel_num
    A = (torch.rand((n_det, V), generator=g) + 0.05).to(dtype).to(cuda)
    cp1 = torch.randint(1, n_det + 1, (n,), generator=g)
    rows = torch.cat((cp1.float().unsqueeze(1), torch.rand((n, vc), generator=g) ** 3), dim=1).to(cuda)
    ids, tcd = ops.split_sparse_rows(rows, dtype)
    assert tcd.stride(0) * tcd.element_size() % 16 == 0 and tcd.stride(0) > vc  # padded
    x = (torch.rand((V, 1), generator=g) + 0.2).to(cuda)
    _lib.take_wait_timeout_count()
    for grouped in (False, True):
        a = ops.sparse_weight_split(ids, tcd, A, tb, x, grouped=grouped, method="event")
        b = ops.sparse_weight_split(ids, tcd, A, tb, x, grouped=grouped)
        torch.cuda.synchronize()
        assert rel_l2(b.cpu(), a.cpu()) < TOL_W
    assert _lib.take_wait_timeout_count() == 0
