"""Host-side logic of the drop-in modules (CPU only): projector construction, subset
splits, detector variances, tap tables, synthetic geometry and argument errors."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2  # noqa: F401
from oracle import compton as oc


def test_projector_mirror_matches_reference_r10(golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    g = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["r10_coor_full"]), theta_stride=2, z_stride=2,
                                           rotate_num=10)
    assert p.ring_strides == tuple(g["r10_ring_strides"])
    assert [p.fine_layer_num, p.fine_z_num, p.coarse_layer_num, p.coarse_z_num] == list(g["r10_dims"])
    for name in ("layer_reduce", "layer_expand", "z_reduce", "z_expand"):
        shape = tuple(g[f"r10_{name}_shape"])
        dense = np.zeros(shape, np.float32)
        i = g[f"r10_{name}_idx"]
        dense[i[0], i[1]] = g[f"r10_{name}_val"]
        np.testing.assert_array_equal(getattr(p, name).numpy(), dense)
    np.testing.assert_array_equal(p.coor_coarse.numpy(), g["r10_coor_coarse"])


def test_projector_mirror_stride_reduction(golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    g = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["s_coor"]), theta_stride=4, z_stride=2, rotate_num=4)
    assert p.ring_strides == tuple(g["s_ring_strides"])
    for name in ("layer_expand", "z_expand", "layer_reduce", "z_reduce"):
        np.testing.assert_array_equal(getattr(p, name).numpy(), g[f"s_{name}"])
    np.testing.assert_array_equal(p.coor_coarse.numpy(), g["s_coor_coarse"])


@pytest.mark.parametrize("L,R,target,expect", [(360, 20, 4, 3), (360, 1, 4, 4), (10, 10, 2, 1), (80, 10, 2, 2),
                                               (25, 7, 4, 1), (36, None, 4, 4), (12, 5, 5, 4)])
def test_ring_stride_choice(L, R, target, expect):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from oracle import sparse as osp

    got = cso._choose_compatible_ring_stride(L, R, target)
    assert got == expect == (osp.choose_ring_stride(L, R, target) if R is not None else expect)


def test_projector_errors_match_reference_messages():
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    with pytest.raises(ValueError, match="coor_full must have shape"):
        cso.build_compton_sparse_projector(torch.zeros((4, 2)))
    with pytest.raises(ValueError, match="coor_full is empty"):
        cso.build_compton_sparse_projector(torch.zeros((0, 3)))
    with pytest.raises(ValueError, match="theta_stride and z_stride must be positive"):
        cso.build_compton_sparse_projector(torch.zeros((4, 3)), theta_stride=0)
    bad_z = torch.tensor([[1.0, 0, 0], [0, 1.0, 0], [1.0, 0, 1.0]])
    with pytest.raises(ValueError, match="consistent z-plane"):
        cso.build_compton_sparse_projector(bad_z)
    from jscc_recon_spect_cylinder_gb300 import synthetic

    p = cso.build_compton_sparse_projector(synthetic.polar_grid(3, 12, 10.0).coor, 2, 1)
    with pytest.raises(ValueError, match="img_fine must have shape"):
        cso.reduce_fine_image_to_coarse(torch.zeros(5), p)
    with pytest.raises(ValueError, match="rows_coarse size does not match"):
        cso.upsample_coarse_rows_to_fine(torch.zeros((2, p.coarse_pixel_num + 1)), p)
    with pytest.raises(ValueError, match="event_rows size does not match"):
        cso.materialize_sparse_event_rows_to_fine(torch.zeros((2, 3)), torch.zeros((4, p.fine_pixel_num)), p)
    with pytest.raises(ValueError, match="cpnum1 and t_compton"):
        cso.pack_sparse_event_rows(torch.zeros(3), torch.zeros((2, 4)))
    with pytest.raises(ValueError, match="event_rows must have shape"):
        cso.unpack_sparse_event_rows(torch.zeros((2, 1)))


def test_tap_tables_reconstruct_dense_matrices(golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops

    g = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["s_coor"]), theta_stride=4, z_stride=2, rotate_num=4)
    tb = ops.SparseTables(p.layer_reduce, p.z_reduce, p.layer_expand, p.z_expand, torch.device("cpu"))

    def dense(csr, shape):
        ptr, idx, w = csr
        m = torch.zeros(shape)
        for r in range(shape[0]):
            for k in range(int(ptr[r]), int(ptr[r + 1])):
                m[r, int(idx[k])] += w[k]
        return m

    assert torch.equal(dense(tb.up[1], p.layer_expand.shape), p.layer_expand)
    assert torch.equal(dense(tb.up[0], p.z_expand.shape), p.z_expand)
    assert torch.equal(dense(tb.adj[1], p.layer_expand.t().shape), p.layer_expand.t())
    assert torch.equal(dense(tb.red[1], p.layer_reduce.shape), p.layer_reduce)
    # two-tap arrays reproduce the expand rows
    le = torch.zeros_like(p.layer_expand)
    for r in range(le.size(0)):
        for k in range(2):
            le[r, tb.l_taps[r, k]] += tb.l_tw[r, k]
    assert torch.equal(le, p.layer_expand)


def test_split_tensor_even_mirror(golden):
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    g = golden("sc_osem")
    for (n, k), sizes in zip(g["split_cases"], g["split_sizes"]):
        got = [int(t.numel()) for t in rop.split_tensor_even(torch.arange(int(n)), int(k))]
        assert got == [int(s) for s in sizes[:k]]
    with pytest.raises(ValueError, match="parts must be positive"):
        rop.split_tensor_even(torch.arange(3), 0)


def test_detector_variances_match_oracle(golden):
    from jscc_recon_spect_cylinder_gb300 import _compton

    g = golden("compton_builders")
    for tag, extra in (("planar", 0.0), ("planar", 0.7), ("cyl", 0.5), ("cyl", 0.0)):
        det = torch.from_numpy(g[f"{tag}_det"])
        got = _compton.detector_pos_sigma_sq(det, extra).numpy()
        np.testing.assert_allclose(got, oc.pos_sigma_sq(g[f"{tag}_det"], extra), rtol=1e-6)


def test_synthetic_rotation_tables_are_inverse():
    from jscc_recon_spect_cylinder_gb300 import synthetic

    rot, inv = synthetic.cyclic_rotation_tables(5, 24, 6)
    for r in range(6):
        assert torch.equal(rot[inv[:, r] - 1, r], torch.arange(1, 121))
        assert torch.equal(torch.sort(rot[:, r])[0], torch.arange(1, 121))


def test_shipped_rotation_tables_are_mutually_inverse(golden):
    """The shipped Factors/511keV_RotateNum10 RotMat_full / RotMatInv_full (23,200 x 10,
    1-based) are inverse permutations of each other, column by column."""
    g = golden("sparse_ops")
    rot, inv = g["r10_rotmat"].astype(np.int64), g["r10_rotmat_inv"].astype(np.int64)
    assert rot.shape == inv.shape == (23200, 10)
    ar = np.arange(1, 23201)
    for r in range(10):
        np.testing.assert_array_equal(rot[inv[:, r] - 1, r], ar)
        np.testing.assert_array_equal(inv[rot[:, r] - 1, r], ar)


def test_install_registers_reference_names():
    import sys

    import jscc_recon_spect_cylinder_gb300 as gb

    saved = {m: sys.modules.get(m) for m in gb._MIRRORED}
    try:
        gb.install()
        import recon_osem_plane  # noqa: F401

        assert sys.modules["recon_osem_plane"].__name__ == "jscc_recon_spect_cylinder_gb300.recon_osem_plane"
        from compton_sparse_ops import build_compton_sparse_projector  # noqa: F401
    finally:
        for m, v in saved.items():
            if v is None:
                sys.modules.pop(m, None)
            else:
                sys.modules[m] = v


def test_product_path_refuses_cpu_tensors():
    from jscc_recon_spect_cylinder_gb300 import batched, ops

    with pytest.raises(RuntimeError, match="no CPU fallback"):
        ops.sc_weight(torch.ones((2, 3)), torch.ones((2, 1)), torch.ones((3, 1)))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        ops.sc_project(torch.ones((2, 8)), torch.ones((8, 1), dtype=torch.float64))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        ops.bf16_gemm_nt(torch.ones((4, 8), dtype=torch.bfloat16), torch.ones((2, 8), dtype=torch.bfloat16))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        ops.rdp_prior(torch.ones(4), torch.zeros((1, 4), dtype=torch.int32), torch.ones((1, 4)))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        batched.BatchedScOsem(torch.ones((8, 8)), [torch.arange(8)], torch.ones(8), 2, device="cpu")


def test_fixed_width_adjoint_equals_dense_adjoint(golden):
    """The [K, V_c] adjoint tap table (grouped sparse kernel) reproduces the transpose of
    the reference's upsample matrices, multi-plane grid with stride reduction included."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops

    g = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["s_coor"]), theta_stride=4, z_stride=2, rotate_num=4)
    tb = ops.SparseTables(p.layer_reduce, p.z_reduce, p.layer_expand, p.z_expand, torch.device("cpu"))
    x = torch.rand(p.fine_pixel_num, dtype=torch.float64)
    U = torch.kron(p.z_expand.double(), p.layer_expand.double())  # [V_f, V_c]
    dense = U.t() @ x
    fw = (tb.adj_w.double() * x[tb.adj_idx.long()]).sum(0)
    assert torch.allclose(fw, dense, rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("n_r,n_theta,stride,z_stride,expect", [
    (100, 360, 4, 1, (360, 4)), (12, 72, 4, 1, (72, 4)), (12, 72, 2, 1, (0, 0)), (12, 72, 8, 1, (0, 0))])
def test_ring_stencil_detection(n_r, n_theta, stride, z_stride, expect):
    """The stride-4 ring-stencil claim passed to the grouped kernel holds exactly for the
    polar projector's stride-4 theta interpolation and for nothing else; a re-ordered
    table (rings not in voxel order) is refused."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops, synthetic

    grid = synthetic.polar_grid(n_r, n_theta, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, stride, z_stride, rotate_num=1)
    assert ops._ring_stencil(p.z_expand, p.layer_expand) == expect
    if expect != (0, 0):
        # the claimed taps are exactly the table's
        ring_len = expect[0]
        le = p.layer_expand
        lc = torch.arange(le.size(1))
        th, r = lc % (ring_len // 4), lc // (ring_len // 4)
        for d in range(-3, 4):
            j = r * ring_len + (4 * th + d) % ring_len
            assert bool((le[j, lc] != 0).all())
        perm = torch.randperm(le.size(1), generator=torch.Generator().manual_seed(0))
        assert ops._ring_stencil(p.z_expand, le[:, perm]) == (0, 0)
